"""Python mirror of the C ABI (include/wcfe.h) over ctypes.

This is host-side plumbing for tests, the benchmark and Python callers; the
compute path is the sm_103a library ``libwcfe.so`` built in-tree by
``wholecellfe_gb300/build.py``.  There is no CPU fallback: if the library is
missing or no CUDA device is visible, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .params import Params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwcfe.so")

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)
PREC_FP64, PREC_MIXED = 0, 1

class NewtonStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("max_refine_iters", C.c_int32), ("unconverged", C.c_int32),
                ("floor_exits", C.c_int32), ("max_rel_residual", C.c_double), ("max_refine_rel_residual", C.c_double),
                ("lu_ms", C.c_double), ("lu_gflop", C.c_double), ("solve_ms", C.c_double)]


class Request(C.Structure):
    _fields_ = [("n_vert", C.c_int32), ("n_tri", C.c_int32), ("tri", _i), ("x", _d), ("params", C.POINTER(Params)),
                ("n_steps", C.c_int32), ("sub_tri", _i), ("sub_X", _d), ("sub_n_vert", C.c_int32),
                ("sub_n_tri", C.c_int32)]


# exported symbols and their signatures (checked against include/wcfe.h by the tests)
SIGNATURES = {
    "wcfe_params_default": (None, [C.POINTER(Params), C.c_int32]),
    "wcfe_last_error": (C.c_char_p, []),
    "wcfe_ap_draw": (C.c_uint32, [C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32]),
    "wcfe_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "wcfe_engine_create": (C.c_int, [C.c_int32, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "wcfe_engine_destroy": (C.c_int, [C.c_void_p]),
    "wcfe_engine_precision": (C.c_int, [C.c_void_p]),
    "wcfe_engine_free_bytes": (C.c_uint64, [C.c_void_p]),
    "wcfe_cell_bytes": (C.c_uint64, [C.c_int32, C.c_int32]),
    "wcfe_engine_sync": (C.c_int, [C.c_void_p]),
    "wcfe_cell_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _i, _i, _i, _u8, C.POINTER(Params),
                                   C.POINTER(C.c_int32)]),
    "wcfe_cell_destroy": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_cell_set_params": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(Params)]),
    "wcfe_cell_set_topology": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _i, _i, _i, _u8]),
    "wcfe_cell_set_substrate": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _i, _d, _d]),
    "wcfe_cell_set_state": (C.c_int, [C.c_void_p, C.c_int32, _d, _d, _d, _d, _d, _d, _d]),
    "wcfe_cell_get_state": (C.c_int, [C.c_void_p, C.c_int32, _d, _d, _d, _d, _d, _d, _d]),
    "wcfe_cell_set_clock": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_uint64]),
    "wcfe_cell_set_step_budget": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "wcfe_cell_get_step_budget": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "wcfe_cell_get_clock": (C.c_int, [C.c_void_p, C.c_int32, _d, C.POINTER(C.c_uint64)]),
    "wcfe_cell_status": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_uint32)]),
    "wcfe_cell_sizes": (C.c_int, [C.c_void_p, C.c_int32, _i, _i, _i, _i]),
    "wcfe_cell_predict": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, _d, _d]),
    "wcfe_cell_update_fa": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, _d, _d, _d, _d]),
    "wcfe_cell_update_forces": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double]),
    "wcfe_cell_eval_residual": (C.c_int, [C.c_void_p, C.c_int32, _d, _d, C.c_double, _d, C.c_double, _d, _d, _d,
                                          _d, _d]),
    "wcfe_cell_eval_forces": (C.c_int, [C.c_void_p, C.c_int32, _d, C.c_double, _d, _d, _d, _d, _d]),
    "wcfe_engine_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    "wcfe_engine_step_cells": (C.c_int, [C.c_void_p, _i, C.c_int32, C.c_int32, C.c_double]),
    "wcfe_engine_set_graphs": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_engine_set_shape": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "wcfe_engine_get_shape": (C.c_int, [C.c_void_p, _i, _i]),
    "wcfe_engine_autotune": (C.c_int, [C.c_void_p, C.c_double, C.c_int32]),
    "wcfe_engine_last_timing": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "wcfe_engine_set_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_engine_launches": (C.c_uint64, [C.c_void_p]),
    "wcfe_engine_stream": (C.c_void_p, [C.c_void_p]),
    "wcfe_debug_pipe_rates": (C.c_int, [_d, _d, _d]),
    "wcfe_engine_step_times": (C.c_int64, [C.c_void_p, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float)]),
    "wcfe_engine_total_vertices": (C.c_int64, [C.c_void_p]),
    "wcfe_engine_predict": (C.c_int, [C.c_void_p, C.c_double, _d]),
    "wcfe_engine_update": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _d]),
    "wcfe_engine_set_exchange_groups": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_debug_lu_schedule": (C.c_int, [C.c_int32, C.c_int32, _i, C.c_int32, _i]),
    "wcfe_cell_set_integrins": (C.c_int, [C.c_void_p, C.c_int32, _d]),
    "wcfe_server_create": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_void_p)]),
    "wcfe_server_destroy": (C.c_int, [C.c_void_p]),
    "wcfe_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "wcfe_server_iterate": (C.c_int, [C.c_void_p, _i, _i]),
    "wcfe_server_result": (C.c_int, [C.c_void_p, C.c_int64, _d, _d]),
    "wcfe_server_step_times": (C.c_int64, [C.c_void_p, _d, C.c_int64]),
    "wcfe_server_set_iteration_ms": (C.c_int, [C.c_void_p, C.c_double]),
    "wcfe_server_cell_steps": (C.c_uint64, [C.c_void_p]),
    "wcfe_engine_set_patch_kernel": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_engine_set_vertex_kernel": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_engine_get_kernels": (C.c_int, [C.c_void_p, _i, _i]),
    "wcfe_engine_set_fused": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_engine_get_fused": (C.c_int, [C.c_void_p]),
    "wcfe_engine_set_element_precision": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_engine_get_element_precision": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "wcfe_cell_set_element_mu": (C.c_int, [C.c_void_p, C.c_int32, _d]),
    "wcfe_cell_couple_substrate": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double]),
    "wcfe_engine_step_implicit": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_int32, C.c_void_p]),
    "wcfe_cell_newton_tangent": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, _d, C.POINTER(C.c_float), _d]),
    "wcfe_debug_lu_solve": (C.c_int, [C.c_int32, C.POINTER(C.c_float), _d, C.POINTER(C.c_float)]),
    "wcfe_debug_trsv_withheld": (C.c_int, [C.c_int32, C.POINTER(C.c_float), _d, C.POINTER(C.c_float), C.c_int32,
                                           C.c_int64]),
    "wcfe_debug_lu_solve_with": (C.c_int, [C.c_int32, C.POINTER(C.c_float), _d, C.POINTER(C.c_float), C.c_int32,
                                           C.c_int32]),
    "wcfe_engine_set_lu": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "wcfe_engine_set_lu_reuse": (C.c_int, [C.c_void_p, C.c_int32]),
    "wcfe_cell_remesh": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _i, C.c_int32, _i, C.c_int32, _i, _i, _i, _u8,
                                   _d]),
    "wcfe_frames_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "wcfe_frames_write": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_char_p]),
    "wcfe_frames_flush": (C.c_int, [C.c_void_p]),
    "wcfe_frames_destroy": (C.c_int, [C.c_void_p]),
    "wcfe_vtk_format": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _i, _d, _d, _d, _d, _d, C.c_double, C.c_double,
                                  C.c_int32, C.c_double, C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]),
    "wcfe_area_tot_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "wcfe_debug_topology": (C.c_int, [C.c_int32, C.c_int32, _i, _i, _i, _u8, C.c_int32, _i, _i, _i, _i, C.c_int32, _i,
                                      _i, C.c_int32, _i, C.c_int32, C.POINTER(C.c_uint16)]),
    "wcfe_debug_patch_staging": (C.c_int, [C.c_int32, C.c_int32, _i, C.c_int32, _i, _i, C.c_int32, _i, C.c_int32,
                                           C.POINTER(C.c_uint16), C.c_int32, _i]),
}


def debug_topology(tri, n_vert, emax=320, vt_ptr=None, vt_idx=None, bnd=None):
    """The engine's host preprocessing (boundary candidates, patches, slot codes); no device needed."""
    tri = i32(tri)
    nt = len(tri)
    nb = C.c_int32()
    npatch = C.c_int32()
    rank = np.zeros(n_vert, np.int32)
    cptr = np.zeros(n_vert + 1, np.int32)
    cand = np.zeros(2 * 12 * n_vert + 16, np.int32)
    patch = np.zeros(4 * n_vert + 16, np.int32)
    elems = np.zeros(6 * nt + 16, np.int32)
    codes = np.zeros(3 * nt, np.uint16)
    check(load().wcfe_debug_topology(n_vert, nt, ip(tri), ip(None if vt_ptr is None else i32(vt_ptr)),
                                     ip(None if vt_idx is None else i32(vt_idx)),
                                     None if bnd is None else np.ascontiguousarray(bnd, np.uint8).ctypes.data_as(_u8),
                                     emax, C.byref(nb), ip(rank), ip(cptr), ip(cand), len(cand), C.byref(npatch),
                                     ip(patch), len(patch), ip(elems), len(elems),
                                     codes.ctypes.data_as(C.POINTER(C.c_uint16))), "wcfe_debug_topology")
    nbv, npv = nb.value, npatch.value
    cptr = cptr[:nbv + 1]
    patch = patch[:4 * npv].reshape(npv, 4)
    n_el = int(patch[-1, 2] + patch[-1, 3] + (patch[-1, 3] & 1)) if npv else 0
    return dict(nb=nbv, rank=rank, cptr=cptr, cand=cand[:2 * cptr[-1]].reshape(-1, 2), np=npv, patch=patch,
                elems=elems[:n_el], codes=codes)


def debug_patch_staging(tri, n_vert, emax=320):
    """Staging description of each patch (halo lists, patch-local corners, code ranges)."""
    tri = i32(tri)
    nt = len(tri)
    npatch = C.c_int32()
    xinfo = np.zeros(4 * n_vert + 16, np.int32)
    halo = np.zeros(8 * n_vert + 64, np.int32)
    loc = np.zeros(4 * (6 * nt + 16), np.uint16)
    mx = np.zeros(4, np.int32)
    check(load().wcfe_debug_patch_staging(n_vert, nt, ip(tri), emax, C.byref(npatch), ip(xinfo), len(xinfo), ip(halo),
                                          len(halo), loc.ctypes.data_as(C.POINTER(C.c_uint16)), len(loc), ip(mx)),
          "wcfe_debug_patch_staging")
    npv = npatch.value
    xinfo = xinfo[:4 * npv].reshape(npv, 4)
    return dict(np=npv, xinfo=xinfo, halo=halo, loc=loc.reshape(-1, 4),
                max_ne=int(mx[0]), max_nvp=int(mx[1]), max_nh=int(mx[2]), max_nc=int(mx[3]))


def pipe_rates():
    """Measured TF32 tensor, FP64 and FP32 FMA rates of the current device (TFLOP/s)."""
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    check(load().wcfe_debug_pipe_rates(C.byref(a), C.byref(b), C.byref(c)), "wcfe_debug_pipe_rates")
    return {"tf32_tflops": a.value, "fp64_tflops": b.value, "fp32_tflops": c.value}


def debug_lu_schedule(m: int, block: int = 512):
    """The tensor-core LU's schedule (host logic): an int32 array [nops][14] of
    (type, k0, nreg, ka, kb, K, rlo0, rhi0, clo0, chi0, rlo1, rhi1, clo1, chi1)."""
    n = C.c_int32()
    check(load().wcfe_debug_lu_schedule(m, block, None, 0, C.byref(n)), "wcfe_debug_lu_schedule")
    ops = np.zeros((n.value, 14), np.int32)
    check(load().wcfe_debug_lu_schedule(m, block, ip(ops), ops.size, C.byref(n)), "wcfe_debug_lu_schedule")
    return ops


def debug_lu_solve(A, b, block: int | None = None, kind: int = 0):
    """The implicit step's dense LU (TF32 trailing updates) and one unrefined solve.
    block None: the default LU; else the outer block width (a multiple of 64 up to 512) and
    kind (0 tcgen05, 1 mma.sync with block 64) of wcfe_engine_set_lu."""
    A = np.ascontiguousarray(A, np.float32)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(len(b), np.float32)
    fp = C.POINTER(C.c_float)
    if block is None:
        check(load().wcfe_debug_lu_solve(len(b), A.ctypes.data_as(fp), dp(b), x.ctypes.data_as(fp)),
              "wcfe_debug_lu_solve")
    else:
        check(load().wcfe_debug_lu_solve_with(len(b), A.ctypes.data_as(fp), dp(b), x.ctypes.data_as(fp), block, kind),
              "wcfe_debug_lu_solve_with")
    return x


def debug_trsv_withheld(A, b, withhold: int, wait_clocks: int):
    """The triangular sweep with block `withhold`'s solution never published (its
    dependents' waits run out after wait_clocks SM clocks); returns (status, message)."""
    A = np.ascontiguousarray(A, np.float32)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(len(b), np.float32)
    fp = C.POINTER(C.c_float)
    rc = load().wcfe_debug_trsv_withheld(len(b), A.ctypes.data_as(fp), dp(b), x.ctypes.data_as(fp), withhold,
                                         wait_clocks)
    return rc, (load().wcfe_last_error().decode() if rc else "")


def vtk_format(fmt: int, x, tri, cA=None, cC=None, fau=None, ea=None, time: float = 0.0, kint: float = -1.0,
               law: int = 0, k_fa: float = 0.0) -> bytes:
    """The text of a VTK frame (cellBP/iomesh.cpp:690-1047 formats) from host arrays."""
    x = f64(x)
    tri = i32(tri)
    n = len(x)
    args = [dp(None if a is None else f64(a)) for a in (cA, cC, fau, ea)]
    ln = C.c_int64()
    check(load().wcfe_vtk_format(fmt, n, len(tri), ip(tri), dp(x), *args, time, kint, law, k_fa, None, 0,
                                 C.byref(ln)), "wcfe_vtk_format")
    buf = C.create_string_buffer(ln.value)
    check(load().wcfe_vtk_format(fmt, n, len(tri), ip(tri), dp(x), *args, time, kint, law, k_fa, buf, ln.value,
                                 C.byref(ln)), "wcfe_vtk_format")
    return buf.raw[:ln.value]


class WcfeError(RuntimeError):
    pass


_lib = None


def load(path: str = LIB_PATH):
    """Load libwcfe.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise WcfeError(f"{path} is missing: build it with wholecellfe_gb300/build.py (no CPU fallback exists)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def check(rc: int, what: str = ""):
    if rc != 0:
        msg = load().wcfe_last_error().decode()
        raise WcfeError(f"{what} failed with status {rc}: {msg}")


def dp(a):
    return None if a is None else a.ctypes.data_as(_d)


def ip(a):
    return None if a is None else a.ctypes.data_as(_i)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Engine:
    """One device, one stream, many cells (wcfe_engine)."""

    def __init__(self, precision: int = PREC_FP64, device: int = 0, budget_bytes: int = 0):
        L = load()
        h = C.c_void_p()
        check(L.wcfe_engine_create(device, precision, budget_bytes, C.byref(h)), "wcfe_engine_create")
        self.h = h
        self.precision = precision
        self.cells: dict[int, "Cell"] = {}

    def close(self):
        if self.h:
            load().wcfe_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_cell(self, x, tri, params: Params, vt_ptr=None, vt_idx=None, bnd=None, state=None, t=0.0, ap_calls=0,
                 substrate=None) -> "Cell":
        tri = i32(tri)
        n = len(x)
        cid = C.c_int32()
        check(load().wcfe_cell_create(self.h, n, len(tri), ip(tri), ip(None if vt_ptr is None else i32(vt_ptr)),
                                      ip(None if vt_idx is None else i32(vt_idx)),
                                      None if bnd is None else np.ascontiguousarray(bnd, np.uint8).ctypes.data_as(_u8),
                                      C.byref(params), C.byref(cid)), "wcfe_cell_create")
        c = Cell(self, cid.value, n, len(tri))
        if state is None:
            c.set_state(x=x)
        else:
            c.set_state(*state)
        c.set_clock(t, ap_calls)
        if substrate is not None:
            c.set_substrate(*substrate)
        self.cells[c.id] = c
        return c

    def step(self, nsteps: int, dt: float):
        check(load().wcfe_engine_step(self.h, nsteps, dt), "wcfe_engine_step")

    def step_implicit(self, nsteps: int, dt: float, rtol: float = 1e-10, max_newton: int = 8):
        """Backward-Euler steps (FP64 engines); returns the Newton statistics."""
        st = NewtonStats()
        check(load().wcfe_engine_step_implicit(self.h, nsteps, dt, rtol, max_newton, C.byref(st)),
              "wcfe_engine_step_implicit")
        return {k: getattr(st, k) for k, _ in NewtonStats._fields_}

    def step_cells(self, cells, nsteps: int, dt: float):
        ids = i32([c.id for c in cells])
        check(load().wcfe_engine_step_cells(self.h, ip(ids), len(ids), nsteps, dt), "wcfe_engine_step_cells")

    def sync(self):
        check(load().wcfe_engine_sync(self.h), "wcfe_engine_sync")

    def set_graphs(self, on: bool):
        check(load().wcfe_engine_set_graphs(self.h, int(on)), "wcfe_engine_set_graphs")

    def set_timing(self, on: bool):
        check(load().wcfe_engine_set_timing(self.h, int(on)), "wcfe_engine_set_timing")

    def last_timing(self):
        a, b = C.c_float(), C.c_float()
        check(load().wcfe_engine_last_timing(self.h, C.byref(a), C.byref(b)), "wcfe_engine_last_timing")
        return a.value, b.value

    def step_times(self):
        """(per-step device ms list, span ms) of the last timed step() call."""
        n = load().wcfe_engine_step_times(self.h, None, 0, None)
        buf = (C.c_float * max(n, 1))()
        span = C.c_float()
        load().wcfe_engine_step_times(self.h, buf, n, C.byref(span))
        return list(buf)[:n], span.value

    def set_shape(self, threads: int, emax: int):
        check(load().wcfe_engine_set_shape(self.h, threads, emax), "wcfe_engine_set_shape")

    def set_lu(self, block: int = 512, kind: int = 0):
        """The implicit step's LU: outer block width (64 to 512 in steps of 64); kind 0 tcgen05,
        1 mma.sync (block 64)."""
        check(load().wcfe_engine_set_lu(self.h, block, kind), "wcfe_engine_set_lu")

    def set_lu_reuse(self, reuse: bool):
        """Implicit step: True (default) factor once per step, False every Newton iteration."""
        check(load().wcfe_engine_set_lu_reuse(self.h, int(reuse)), "wcfe_engine_set_lu_reuse")

    def set_patch_kernel(self, kind: int):
        """Mixed engines: 0 staged patch kernel where it fits, 1 plain (default)."""
        check(load().wcfe_engine_set_patch_kernel(self.h, kind), "wcfe_engine_set_patch_kernel")

    def set_vertex_kernel(self, kind: int):
        check(load().wcfe_engine_set_vertex_kernel(self.h, kind), "wcfe_engine_set_vertex_kernel")

    def set_fused(self, enable: bool):
        """Mixed engines: fold each next vertex phase into the patch phase in runs of steps."""
        check(load().wcfe_engine_set_fused(self.h, 1 if enable else 0), "wcfe_engine_set_fused")

    def fused(self) -> bool:
        """True where a run of steps of this engine is fused."""
        return load().wcfe_engine_get_fused(self.h) == 1

    def set_element_precision(self, mode: int):
        """Mixed engines: 0 the FP32 element, 1 the float-float element."""
        check(load().wcfe_engine_set_element_precision(self.h, int(mode)), "wcfe_engine_set_element_precision")

    def element_precision(self) -> int:
        m = C.c_int32(-1)
        check(load().wcfe_engine_get_element_precision(self.h, C.byref(m)), "wcfe_engine_get_element_precision")
        return int(m.value)

    def kernels(self):
        """(patch kernel kind, vertex kernel kind) in use."""
        a, b = C.c_int32(), C.c_int32()
        check(load().wcfe_engine_get_kernels(self.h, C.byref(a), C.byref(b)), "wcfe_engine_get_kernels")
        return a.value, b.value

    def shape(self):
        a, b = C.c_int32(), C.c_int32()
        check(load().wcfe_engine_get_shape(self.h, C.byref(a), C.byref(b)), "wcfe_engine_get_shape")
        return a.value, b.value

    def autotune(self, dt: float, reps: int = 3):
        check(load().wcfe_engine_autotune(self.h, dt, reps), "wcfe_engine_autotune")

    def launches(self) -> int:
        return int(load().wcfe_engine_launches(self.h))

    def stream_ptr(self) -> int:
        """The engine's main cudaStream_t as an integer (torch.cuda.ExternalStream)."""
        return int(load().wcfe_engine_stream(self.h) or 0)

    def total_vertices(self) -> int:
        return int(load().wcfe_engine_total_vertices(self.h))

    def predict_all(self, dt: float, x_pred: np.ndarray):
        check(load().wcfe_engine_predict(self.h, dt, dp(x_pred)), "wcfe_engine_predict")

    def update_all(self, dt: float, dt_real: float, x_new: np.ndarray):
        check(load().wcfe_engine_update(self.h, dt, dt_real, dp(x_new)), "wcfe_engine_update")

    def set_exchange_groups(self, groups: int):
        """Exchange path: cells stepped in `groups` (1-8) overlapped groups."""
        check(load().wcfe_engine_set_exchange_groups(self.h, groups), "wcfe_engine_set_exchange_groups")

    def free_bytes(self) -> int:
        return int(load().wcfe_engine_free_bytes(self.h))

    def engine_precision(self) -> int:
        return int(load().wcfe_engine_precision(self.h))


class Frames:
    """Asynchronous VTK frame writer of an engine (wcfe_frames_*)."""

    def __init__(self, eng: Engine, slots: int = 4, threads: int = 1):
        self.h = C.c_void_p()
        check(load().wcfe_frames_create(eng.h, slots, threads, C.byref(self.h)), "wcfe_frames_create")

    def write(self, cell: "Cell", fmt: int, path: str, time: float = float("nan"), kint: float = -1.0):
        check(load().wcfe_frames_write(self.h, cell.id, fmt, time, kint, str(path).encode()), "wcfe_frames_write")

    def flush(self):
        check(load().wcfe_frames_flush(self.h), "wcfe_frames_flush")

    def close(self):
        if self.h:
            load().wcfe_frames_destroy(self.h)
            self.h = C.c_void_p()


class Cell:
    def __init__(self, eng: Engine, cid: int, n: int, nt: int):
        self.eng, self.id, self.n, self.nt = eng, cid, n, nt

    def destroy(self):
        check(load().wcfe_cell_destroy(self.eng.h, self.id), "wcfe_cell_destroy")
        self.eng.cells.pop(self.id, None)

    def set_state(self, x=None, V=None, A=None, ea=None, cA=None, cC=None, fau=None):
        arrs = [None if a is None else f64(a) for a in (x, V, A, ea, cA, cC, fau)]
        check(load().wcfe_cell_set_state(self.eng.h, self.id, *[dp(a) for a in arrs]), "wcfe_cell_set_state")

    def get_state(self):
        n = self.n
        out = [np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 6)), np.zeros(n), np.zeros(n),
               np.zeros((n, 3))]
        check(load().wcfe_cell_get_state(self.eng.h, self.id, *[dp(a) for a in out]), "wcfe_cell_get_state")
        return tuple(out)

    def set_params(self, p: Params):
        check(load().wcfe_cell_set_params(self.eng.h, self.id, C.byref(p)), "wcfe_cell_set_params")

    def couple_substrate(self, sub, margin: float = 0.05):
        """Couple this cell to a deformable substrate cell of the same engine (None: uncouple)."""
        check(load().wcfe_cell_couple_substrate(self.eng.h, self.id, -1 if sub is None else sub.id, margin),
              "wcfe_cell_couple_substrate")

    def set_topology(self, tri, n_vert=None, vt_ptr=None, vt_idx=None, bnd=None):
        """Replace the connectivity (the state, clock and integrins must be set again)."""
        tri = i32(tri)
        n = self.n if n_vert is None else int(n_vert)
        check(load().wcfe_cell_set_topology(self.eng.h, self.id, n, len(tri), ip(tri),
                                            ip(None if vt_ptr is None else i32(vt_ptr)),
                                            ip(None if vt_idx is None else i32(vt_idx)),
                                            None if bnd is None else np.ascontiguousarray(bnd, np.uint8).ctypes.data_as(_u8)),
              "wcfe_cell_set_topology")
        self.n, self.nt = n, len(tri)

    def remesh(self, split_ab, keep, tri, x_new, vt_ptr=None, vt_idx=None, bnd=None):
        """Rebuild after El Topo's remeshing with the state carried on the device: split_ab
        [n_split][2] (VERTEX_ADD events in order), keep [nv_new] (the defrag map)."""
        sab = i32(np.zeros((0, 2)) if split_ab is None else split_ab).reshape(-1)
        keep = i32(keep)
        tri = i32(tri)
        x_new = f64(x_new)
        check(load().wcfe_cell_remesh(self.eng.h, self.id, len(sab) // 2, ip(sab) if len(sab) else None, len(keep),
                                      ip(keep), len(tri), ip(tri), ip(None if vt_ptr is None else i32(vt_ptr)),
                                      ip(None if vt_idx is None else i32(vt_idx)),
                                      None if bnd is None else np.ascontiguousarray(bnd, np.uint8).ctypes.data_as(_u8),
                                      dp(x_new)), "wcfe_cell_remesh")
        self.n, self.nt = len(keep), len(tri)

    def set_element_mu(self, mu):
        """Per-element shear modulus [n_tri] (None: the cell's params.mu everywhere)."""
        check(load().wcfe_cell_set_element_mu(self.eng.h, self.id, None if mu is None else dp(f64(mu))),
              "wcfe_cell_set_element_mu")

    def set_integrins(self, rho):
        check(load().wcfe_cell_set_integrins(self.eng.h, self.id, dp(None if rho is None else f64(rho))),
              "wcfe_cell_set_integrins")

    def set_clock(self, t: float, ap_calls: int):
        check(load().wcfe_cell_set_clock(self.eng.h, self.id, t, ap_calls), "wcfe_cell_set_clock")

    def set_step_budget(self, steps: int):
        check(load().wcfe_cell_set_step_budget(self.eng.h, self.id, steps), "wcfe_cell_set_step_budget")

    def step_budget(self) -> int:
        b = C.c_int32()
        check(load().wcfe_cell_get_step_budget(self.eng.h, self.id, C.byref(b)), "wcfe_cell_get_step_budget")
        return b.value

    def clock(self):
        t = C.c_double()
        k = C.c_uint64()
        check(load().wcfe_cell_get_clock(self.eng.h, self.id, C.byref(t), C.byref(k)), "wcfe_cell_get_clock")
        return t.value, k.value

    def status(self) -> int:
        s = C.c_uint32()
        check(load().wcfe_cell_status(self.eng.h, self.id, C.byref(s)), "wcfe_cell_status")
        return s.value

    def sizes(self):
        v = [C.c_int32() for _ in range(4)]
        check(load().wcfe_cell_sizes(self.eng.h, self.id, *[C.byref(a) for a in v]), "wcfe_cell_sizes")
        return tuple(a.value for a in v)

    def set_substrate(self, Xs, tri_s, xs=None):
        tri_s = i32(tri_s)
        Xs = f64(Xs)
        check(load().wcfe_cell_set_substrate(self.eng.h, self.id, len(Xs), len(tri_s), ip(tri_s), dp(Xs),
                                             dp(None if xs is None else f64(xs))), "wcfe_cell_set_substrate")

    # drop-in pieces
    def predict(self, dt: float):
        xp = np.zeros((self.n, 3))
        vh = np.zeros((self.n, 3))
        check(load().wcfe_cell_predict(self.eng.h, self.id, dt, dp(xp), dp(vh)), "wcfe_cell_predict")
        return vh, xp

    def update_fa(self, dt_real: float, x_new, X=None, Xs=None, xs=None):
        check(load().wcfe_cell_update_fa(self.eng.h, self.id, dt_real, dp(None if X is None else f64(X)),
                                         dp(f64(x_new)), dp(None if Xs is None else f64(Xs)),
                                         dp(None if xs is None else f64(xs))), "wcfe_cell_update_fa")

    def update_forces(self, dt: float, dt_real: float, t_tot: float):
        check(load().wcfe_cell_update_forces(self.eng.h, self.id, dt, dt_real, t_tot), "wcfe_cell_update_forces")

    def eval_residual(self, X, x_new, dt_real, centroid, t_tot):
        n = self.n
        out = [np.zeros((n, 3)), np.zeros((n, 6)), np.zeros(n), np.zeros(n), np.zeros(n)]
        cen = f64(centroid)
        check(load().wcfe_cell_eval_residual(self.eng.h, self.id, dp(f64(X)), dp(f64(x_new)), dt_real, dp(cen), t_tot,
                                             *[dp(a) for a in out]), "wcfe_cell_eval_residual")
        return tuple(out)

    def newton_tangent(self, x, dt):
        """Dense implicit-step tangent (2n x 2n, FP32) at positions x, and the mass diagonal."""
        n = self.n
        J = np.zeros((2 * n, 2 * n), np.float32)
        d = np.zeros(n)
        check(load().wcfe_cell_newton_tangent(self.eng.h, self.id, dt, dp(f64(x)),
                                              J.ctypes.data_as(C.POINTER(C.c_float)), dp(d)), "wcfe_cell_newton_tangent")
        return J, d

    def eval_forces(self, x, dt_real):
        n = self.n
        out = [np.zeros((n, 3)) for _ in range(4)] + [np.zeros(4)]
        check(load().wcfe_cell_eval_forces(self.eng.h, self.id, dp(f64(x)), dt_real, *[dp(a) for a in out]),
              "wcfe_cell_eval_forces")
        return tuple(out)
