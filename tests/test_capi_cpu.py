"""The C-ABI library on the CPU: it loads, exports every function include/wcfe.h
declares, and its host-side integer bookkeeping matches the reference's mesh
structures and the oracle.  No kernel runs here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from oracle import oracle_py as O
from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import Params, default_params


def header_functions():
    src = open(os.path.join(ROOT, "include", "wcfe.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(wcfe_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    names = header_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python mirror binds each of them with a signature
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


_C_KIND = {"int32_t": "i32", "int": "i32", "uint32_t": "u32", "int64_t": "i64", "uint64_t": "u64", "double": "f64",
           "float": "f32", "uint16_t": "u16", "size_t": "u64", "uint8_t": "u8", "void": "void"}
_PY_KIND = {C.c_int32: "i32", C.c_int: "i32", C.c_uint32: "u32", C.c_int64: "i64", C.c_uint64: "u64",
            C.c_longlong: "i64", C.c_ulonglong: "u64", C.c_double: "f64", C.c_float: "f32", C.c_uint16: "u16",
            C.c_size_t: "u64", C.c_uint8: "u8", None: "void"}


def _c_kind(decl):
    decl = re.sub(r"\bconst\b", "", decl).strip()
    if "*" in decl or "[" in decl:
        return "ptr"
    words = decl.split()
    return _C_KIND.get(words[0] if len(words) else "", "?" + decl)


def _py_kind(ct):
    if ct in (C.c_void_p, C.c_char_p) or (isinstance(ct, type) and issubclass(ct, C._Pointer)):
        return "ptr"
    return _PY_KIND.get(ct, "?" + str(ct))


def test_bindings_match_the_header_prototypes():
    """Each ctypes signature in capi.py has the prototype's parameter count, and per
    parameter and for the result the same kind (pointer, or the scalar's width and type)."""
    src = open(os.path.join(ROOT, "include", "wcfe.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#[^\n]*", "", src)
    protos = re.findall(r"([A-Za-z_][A-Za-z0-9_ \t\*]*?)\s*\b(wcfe_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src)
    assert len(protos) >= 60
    bad = []
    for ret, name, args in protos:
        args = args.strip()
        want = [] if args in ("", "void") else [_c_kind(a) for a in args.split(",")]
        rt, at = capi.SIGNATURES[name]
        got = [_py_kind(a) for a in at]
        ret_c = "ptr" if "*" in ret else _C_KIND.get(ret.split()[-1], "?" + ret)
        if want != got or ret_c != _py_kind(rt):
            bad.append((name, ret_c, want, _py_kind(rt), got))
    assert not bad, bad


@pytest.mark.parametrize("lang,std", [("c", "c99"), ("c++", "c++11")])
def test_header_is_plain_c(tmp_path, lang, std):
    """include/wcfe.h compiles on its own as strict C99 and C++11 (the ABI a cgo, JNI or
    ctypes binding includes), warnings as errors."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / "use_header.c"
    src.write_text('#include "wcfe.h"\nint main(void) { wcfe_params p; (void)p; return WCFE_OK; }\n')
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    r = subprocess.run([cc, "-x", lang, f"-std={std}", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", inc, "-c",
                        str(src), "-o", str(tmp_path / "use_header.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_engine_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is visible")
    h = C.c_void_p()
    rc = capi.load().wcfe_engine_create(0, 0, 0, C.byref(h))
    assert rc == 9  # WCFE_ERR_NODEVICE


def test_params_layout_and_defaults():
    for v, name in ((0, "kMD"), (1, "k1"), (2, "k31")):
        a = Params()
        capi.load().wcfe_params_default(C.byref(a), v)
        b = default_params(name)
        assert bytes(a) == bytes(b)
        c = Params()
        O.lib().wo_params_default(C.byref(c), v)
        assert bytes(a) == bytes(c)


def test_philox_and_ap_stream_match_oracle():
    L = capi.load()
    c = (C.c_uint32 * 4)(0, 0, 0, 0)
    k = (C.c_uint32 * 2)(0, 0)
    o = (C.c_uint32 * 4)()
    L.wcfe_philox4x32_10(c, k, o)
    assert tuple(o) == (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)
    # the other published Philox4x32-10 known-answer vectors (Salmon et al., SC'11; Random123)
    for ctr, key, want in [((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
                           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
                            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]:
        L.wcfe_philox4x32_10((C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), o)
        assert tuple(o) == want
    rng = np.random.default_rng(3)
    for _ in range(200):
        s, st, call, kk = (int(rng.integers(0, 2**32)), int(rng.integers(0, 2**32)), int(rng.integers(0, 2**40)),
                           int(rng.integers(0, 2**20)))
        assert L.wcfe_ap_draw(s, st, call, kk) == O.lib().wo_ap_draw(s, st, call, kk)


def _j1j2_from_candidates(x, rank, cptr, cand, v):
    """Evaluate the engine's candidate list with the reference's sign rule (UL:1517-1525)."""
    r = rank[v]
    j1 = j2 = -1
    for nj, ni in cand[cptr[r]:cptr[r + 1]]:
        d1 = x[v] - x[nj]
        d2 = x[ni] - x[v]
        ncz = d1[0] * d2[1] - d1[1] * d2[0]
        if ncz > 0:
            j1 = nj
        else:
            j2 = nj
    return j1, j2


@pytest.mark.parametrize("n", [60, 500, 3000])
def test_boundary_candidates_reproduce_reference_scan(n):
    x, tri = synth.disk_mesh(n, seed=n)
    t = capi.debug_topology(tri, len(x))
    m = O.OMesh(tri, len(x))
    j1o, j2o, cto = O.bnd_table(m, x)
    bnd = m.bnd
    assert t["nb"] == int(bnd.sum())
    assert np.array_equal(t["rank"] >= 0, bnd.astype(bool))
    for v in np.nonzero(bnd)[0]:
        j1, j2 = _j1j2_from_candidates(x, t["rank"], t["cptr"], t["cand"], v)
        assert (j1, j2) == (j1o[v], j2o[v])
        assert t["cptr"][t["rank"][v] + 1] - t["cptr"][t["rank"][v]] == cto[v]


@pytest.mark.parametrize("n", [400, 3000])
def test_boundary_candidates_on_an_annulus(n):
    """Two boundary loops (an inner hole): the candidates reproduce the reference's
    neighbour scan (UL:1500-1531) on both loops."""
    x, tri = synth.annulus_mesh(n, 0.35, seed=n + 1)
    t = capi.debug_topology(tri, len(x))
    m = O.OMesh(tri, len(x))
    j1o, j2o, cto = O.bnd_table(m, x)
    bnd = m.bnd
    r = np.hypot(x[:, 0] - x[:, 0].mean(), x[:, 1] - x[:, 1].mean())
    assert bnd[r < 0.5 * r.max()].any() and bnd[r > 0.9 * r.max()].any()   # both loops
    assert t["nb"] == int(bnd.sum())
    assert np.array_equal(t["rank"] >= 0, bnd.astype(bool))
    for v in np.nonzero(bnd)[0]:
        j1, j2 = _j1j2_from_candidates(x, t["rank"], t["cptr"], t["cand"], v)
        assert (j1, j2) == (j1o[v], j2o[v])
        assert t["cptr"][t["rank"][v] + 1] - t["cptr"][t["rank"][v]] == cto[v]


def test_one_ring_limit_and_tiny_meshes():
    """A vertex whose one-ring fills a patch exactly is accepted, one element more is
    refused with a message; one- and two-triangle meshes are one patch."""
    def fan(d):
        return np.array([[0, 1 + i, 1 + (i + 1) % d] for i in range(d)], np.int32), d + 1
    tri, n = fan(512)
    t = capi.debug_topology(tri, n, emax=512)
    assert t["np"] >= 1 and int(t["patch"][:, 3].max()) <= 512
    tri, n = fan(513)
    with pytest.raises(capi.WcfeError, match="one-ring"):
        capi.debug_topology(tri, n, emax=512)
    for tri, n in ((np.array([[0, 1, 2]], np.int32), 3), (np.array([[0, 1, 2], [0, 2, 3]], np.int32), 4)):
        t = capi.debug_topology(tri, n, emax=512)
        assert t["np"] == 1 and t["patch"][0].tolist() == [0, n, 0, len(tri)]
        assert t["nb"] == n and sorted(t["rank"].tolist()) == list(range(n))


def test_topology_matches_reference_mesh_structures(golden):
    g = golden
    n = len(g["x0"])
    t = capi.debug_topology(g["tri"], n, vt_ptr=g["vt_ptr"], vt_idx=g["vt_idx"], bnd=g["bnd"])
    t2 = capi.debug_topology(g["tri"], n)   # map and flags derived by the engine itself
    for k in ("rank", "cptr", "cand", "patch", "elems", "codes"):
        assert np.array_equal(t[k], t2[k]), k


@pytest.mark.parametrize("emax", [24, 96, 320, 1024])
def test_patches_cover_each_one_ring(emax):
    x, tri = synth.disk_mesh(2000, seed=4)
    n = len(x)
    vt_ptr, vt_idx = synth.vertex_triangle_map(n, tri)
    t = capi.debug_topology(tri, n, emax=emax)
    P = t["patch"]
    assert P[0, 0] == 0 and P[-1, 0] + P[-1, 1] == n and (P[1:, 0] == P[:-1, 0] + P[:-1, 1]).all()
    assert (P[:, 3] <= emax).all()
    for p in range(t["np"]):
        v0, nvp, e0, ne = P[p]
        elems = t["elems"][e0:e0 + ne]
        assert len(set(elems.tolist())) == ne
        for v in range(v0, v0 + nvp):
            for k in range(vt_ptr[v], vt_ptr[v + 1]):
                code = int(t["codes"][k])
                slot, corner = code >> 2, code & 3
                assert elems[slot] == vt_idx[k]
                assert tri[vt_idx[k], corner] == v


def test_topology_rejects_bad_meshes():
    L = capi.load()
    tri = np.array([[0, 1, 5]], np.int32)
    with pytest.raises(capi.WcfeError):
        capi.debug_topology(tri, 3)
    with pytest.raises(capi.WcfeError):   # a vertex with no triangle
        capi.debug_topology(np.array([[0, 1, 2]], np.int32), 4)
    assert L is not None


@pytest.mark.parametrize("emax", [24, 96, 512])
def test_patch_staging_description(emax):
    """Halo lists, patch-local corners and code ranges of the mixed form's staged patches."""
    x, tri = synth.disk_mesh(1500, seed=6)
    n = len(x)
    vt_ptr, vt_idx = synth.vertex_triangle_map(n, tri)
    t = capi.debug_topology(tri, n, emax=emax)
    s = capi.debug_patch_staging(tri, n, emax=emax)
    assert s["np"] == t["np"]
    mx = np.zeros(4, np.int64)
    for p in range(t["np"]):
        v0, nvp, e0, ne = t["patch"][p]
        h0, nh, c0, nc = s["xinfo"][p]
        assert e0 % 2 == 0
        assert c0 == vt_ptr[v0] and nc == vt_ptr[v0 + nvp] - vt_ptr[v0]
        halo = s["halo"][h0:h0 + nh]
        assert (np.diff(halo) > 0).all()
        assert ((halo < v0) | (halo >= v0 + nvp)).all()
        corners = tri[t["elems"][e0:e0 + ne]]
        want = np.unique(corners[(corners < v0) | (corners >= v0 + nvp)])
        assert np.array_equal(halo, want)
        loc = s["loc"][e0:e0 + ne].astype(np.int64)
        assert (loc[:, 3] == 0).all()
        local = np.where(loc[:, :3] < nvp, v0 + loc[:, :3], halo[np.clip(loc[:, :3] - nvp, 0, max(nh - 1, 0))])
        assert np.array_equal(local, corners)
        mx = np.maximum(mx, [ne, nvp, nh, nc])
    assert list(mx) == [s["max_ne"], s["max_nvp"], s["max_nh"], s["max_nc"]]
