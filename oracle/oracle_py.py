"""ctypes bindings of the oracle (wcfe_oracle.c) and of the reference built from
its sources (oracle/_ref/libwcfe_ref_<variant>.so).  TEST INFRASTRUCTURE ONLY:
tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it as the
checker; the product package never imports it."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from wholecellfe_gb300.params import Params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc, -ffp-contract=off so x86 and Arm agree)."""
    src = os.path.join(HERE, "wcfe_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB, src, "-lm",
                               "-lpthread"])
    return LIB


class Mesh(C.Structure):
    _fields_ = [("nv", C.c_int32), ("nt", C.c_int32), ("tri", _i), ("vt_ptr", _i), ("vt_idx", _i), ("bnd", _u8),
                ("mu_e", _d)]


class Cell(C.Structure):
    _fields_ = [("mesh", Mesh), ("x", _d), ("V", _d), ("A", _d), ("ea", _d), ("cA", _d), ("cC", _d), ("fau", _d),
                ("rho_w", _d), ("p", Params), ("t", C.c_double), ("ap_call", C.c_uint64),
                ("sub", C.POINTER(Mesh)), ("Xs", _d)]


class ForceDump(C.Structure):
    _fields_ = [("Res", _d), ("F_FA", _d), ("F_AP", _d), ("F_bend", _d), ("F_area", _d), ("area4", _d)]


def dp(a):
    return None if a is None else a.ctypes.data_as(_d)


def ip(a):
    return None if a is None else a.ctypes.data_as(_i)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.wo_ap_draw.restype = C.c_uint32
        _lib.wo_ap_draw.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32]
        _lib.wo_locate.restype = C.c_int32
        assert _lib.wo_sizeof_params() == C.sizeof(Params), "wcfe_params layout mismatch"
        assert _lib.wo_sizeof_cell() == C.sizeof(Cell), "wo_cell layout mismatch"
    return _lib


class OMesh:
    """Mesh arrays kept alive together with the ctypes struct that points into them."""

    def __init__(self, tri, n_vert, vt_ptr=None, vt_idx=None, bnd=None, mu_e=None):
        """mu_e: optional per-element shear modulus (an extension: the reference has one per material)."""
        from wholecellfe_gb300 import synth
        self.tri = np.ascontiguousarray(tri, dtype=np.int32)
        self.nv = int(n_vert)
        if vt_ptr is None:
            vt_ptr, vt_idx = synth.vertex_triangle_map(self.nv, self.tri)
        if bnd is None:
            bnd = synth.boundary_flags(self.nv, self.tri)
        self.vt_ptr = np.ascontiguousarray(vt_ptr, dtype=np.int32)
        self.vt_idx = np.ascontiguousarray(vt_idx, dtype=np.int32)
        self.bnd = np.ascontiguousarray(bnd, dtype=np.uint8)
        self.mu_e = None if mu_e is None else f64(mu_e).copy()
        self.s = Mesh(self.nv, len(self.tri), ip(self.tri), ip(self.vt_ptr), ip(self.vt_idx),
                      self.bnd.ctypes.data_as(_u8), dp(self.mu_e))


# ---- thin wrappers ----------------------------------------------------------
def predict(x, V, A, dt):
    n = len(x)
    Vh = np.zeros((n, 3)); xp = np.zeros((n, 3))
    lib().wo_predict(n, dp(f64(x)), dp(f64(V)), dp(f64(A)), C.c_double(dt), dp(Vh), dp(xp))
    return Vh, xp


def area_tot(m: OMesh, x):
    out = np.zeros(4)
    lib().wo_area_tot(C.byref(m.s), dp(f64(x)), dp(out))
    return out


def calc_res(m: OMesh, X, x, ea, cA, cC, dt_real, mat, p: Params, centroid, time):
    n = m.nv
    Res = np.zeros((n, 3)); Rea = np.zeros((n, 6)); MM = np.zeros(n); RA = np.zeros(n); RC = np.zeros(n)
    cen = None if centroid is None else f64(centroid)
    lib().wo_calc_res(C.byref(m.s), dp(f64(X)), dp(f64(x)), dp(f64(ea)), dp(None if cA is None else f64(cA)),
                      dp(None if cC is None else f64(cC)), C.c_double(dt_real), C.c_int(mat), C.byref(p), dp(cen),
                      C.c_double(time), dp(Res), dp(Rea), dp(MM), dp(RA), dp(RC))
    return Res, Rea, MM, RA, RC


def force_fa(m: OMesh, x, cC, fau, p: Params, rho_w=None):
    F = np.zeros((m.nv, 3))
    lib().wo_force_fa(C.byref(m.s), dp(f64(x)), dp(f64(cC)), dp(f64(fau)), C.byref(p),
                      dp(None if rho_w is None else f64(rho_w)), dp(F))
    return F


def force_ap(m: OMesh, x, dt_real, p: Params, call):
    F = np.zeros((m.nv, 3))
    lib().wo_force_ap(C.byref(m.s), dp(f64(x)), C.c_double(dt_real), C.byref(p), C.c_uint64(call), dp(F))
    return F


def force_bending(m: OMesh, x, p: Params):
    F = np.zeros((m.nv, 3))
    lib().wo_force_bending(C.byref(m.s), dp(f64(x)), C.byref(p), dp(F))
    return F


def force_area(m: OMesh, x, tot, p: Params):
    F = np.zeros((m.nv, 3))
    lib().wo_force_area(C.byref(m.s), dp(f64(x)), C.c_double(tot), C.byref(p), dp(F))
    return F


def bnd_table(m: OMesh, x):
    j1 = np.zeros(m.nv, np.int32); j2 = np.zeros(m.nv, np.int32); ct = np.zeros(m.nv, np.int32)
    lib().wo_bnd_table(C.byref(m.s), dp(f64(x)), ip(j1), ip(j2), ip(ct))
    return j1, j2, ct


def update_fa(cA, cC, fau, dt_real, X, x, p: Params, sub: OMesh | None = None, Xs=None, xs=None):
    cA = f64(cA).copy(); cC = f64(cC).copy(); fau = f64(fau).copy()
    loc = np.zeros(len(cC), np.int32)
    subp = C.byref(sub.s) if sub is not None else None
    lib().wo_update_fa(len(cC), dp(cA), dp(cC), dp(fau), C.c_double(dt_real), dp(f64(X)), dp(f64(x)), subp,
                       dp(None if Xs is None else f64(Xs)), dp(None if xs is None else f64(xs)), C.byref(p), ip(loc))
    return cA, cC, fau, loc


def update_forces(m: OMesh, X, x, V, Vh, A, ea, cA, cC, fau, dt, dt_real, t_tot, p: Params, call, rho_w=None):
    V = f64(V).copy(); A = f64(A).copy(); ea = f64(ea).copy()
    n = m.nv
    outs = {k: np.zeros((n, 3)) for k in ("Res", "F_FA", "F_AP", "F_bend", "F_area")}
    outs["area4"] = np.zeros(4)
    dump = ForceDump(*(dp(outs[k]) for k in ("Res", "F_FA", "F_AP", "F_bend", "F_area", "area4")))
    lib().wo_update_forces(C.byref(m.s), dp(f64(X)), dp(f64(x)), dp(V), dp(f64(Vh)), dp(A), dp(ea), dp(f64(cA)),
                           dp(f64(cC)), dp(f64(fau)), C.c_double(dt), C.c_double(dt_real), C.c_double(t_tot),
                           C.byref(p), dp(None if rho_w is None else f64(rho_w)), C.c_uint64(call), C.byref(dump))
    return V, A, ea, outs


def update_forces_subs(ms: OMesh, Xs, xs, Vs, Vhs, As, eas, dt, dt_real, t_tot, fau, cC, xcell, mc: OMesh,
                       p: Params, rho_w=None):
    """Substrate overload of updateForces_Explicit (UL:429-504): returns updated (Vs, As, eas)."""
    Vs = f64(Vs).copy(); As = f64(As).copy(); eas = f64(eas).copy()
    lib().wo_update_forces_subs(C.byref(ms.s), dp(f64(Xs)), dp(f64(xs)), dp(Vs), dp(f64(Vhs)), dp(As), dp(eas),
                                C.c_double(dt), C.c_double(dt_real), C.c_double(t_tot), dp(f64(fau)), dp(f64(cC)),
                                dp(f64(xcell)), C.byref(mc.s), C.byref(p), dp(None if rho_w is None else f64(rho_w)),
                                None, None)
    return Vs, As, eas


def force_fa_subs(ms: OMesh, Xs, xs, cC, xcell, fau, mc: OMesh, p: Params, rho_w=None):
    F = np.zeros((ms.nv, 3))
    lib().wo_force_fa_subs(C.byref(ms.s), dp(f64(Xs)), dp(f64(xs)), dp(f64(cC)), dp(f64(xcell)), dp(f64(fau)),
                           C.byref(mc.s), C.byref(p), dp(None if rho_w is None else f64(rho_w)), dp(F))
    return F


class OCell:
    """A cell advanced by the oracle's full synthetic step (wo_cell_steps)."""

    def __init__(self, m: OMesh, state, p: Params, t=0.0, ap_call=0, sub: OMesh | None = None, Xs=None,
                 rho_w=None):
        self.m = m
        self.x, self.V, self.A, self.ea, self.cA, self.cC, self.fau = (f64(a).copy() for a in state)
        self.rho_w = None if rho_w is None else f64(rho_w).copy()
        self.sub = sub
        self.Xs = None if Xs is None else f64(Xs).copy()
        self.s = Cell(m.s, dp(self.x), dp(self.V), dp(self.A), dp(self.ea), dp(self.cA), dp(self.cC), dp(self.fau),
                      dp(self.rho_w), p, t, ap_call, C.pointer(sub.s) if sub is not None else None, dp(self.Xs))

    def steps(self, n, dt):
        lib().wo_cell_steps(C.byref(self.s), C.c_int32(n), C.c_double(dt))

    @property
    def t(self):
        return self.s.t

    @property
    def ap_call(self):
        return self.s.ap_call

    def state(self):
        return (self.x.copy(), self.V.copy(), self.A.copy(), self.ea.copy(), self.cA.copy(), self.cC.copy(),
                self.fau.copy())


def cells_steps_mt(cells: list[OCell], nsteps: int, dt: float, nthreads: int):
    arr = (Cell * len(cells))(*[c.s for c in cells])
    lib().wo_cells_steps_mt(arr, len(cells), nsteps, C.c_double(dt), nthreads)
    for i, c in enumerate(cells):
        c.s = arr[i]


# ---- the reference built from its sources (present only where oracle/build_ref.sh ran) ---------------
def ref_available(variant: str = "kMD") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libwcfe_ref_{variant}.so"))


class Ref:
    """The reference's own functions (oracle/_ref/libwcfe_ref_<variant>.so)."""

    def __init__(self, variant: str = "kMD"):
        self.variant = variant
        self.lib = C.CDLL(os.path.join(REF_DIR, f"libwcfe_ref_{variant}.so"))
        self.lib.ref_mesh_new.restype = C.c_void_p
        self.lib.ref_mesh_new.argtypes = [C.c_int32, C.c_int32, _i]
        self.lib.ref_mesh_free.argtypes = [C.c_void_p]
        self.lib.ref_mesh_map.restype = C.c_int32
        self.lib.ref_mesh_map.argtypes = [C.c_void_p, _i, _i, _u8]
        for name in ("ref_area_tot", "ref_calc_res", "ref_force_fa", "ref_force_ap", "ref_force_bending",
                     "ref_force_area", "ref_update_fa", "ref_update_forces", "ref_update_forces_subs",
                     "ref_force_fa_subs", "ref_steps", "ref_predict"):
            getattr(self.lib, name).restype = None

    def write_vtk(self, h, fmt, x, cA, cC, fau, ea, time, kint, path):
        """The reference's VTK frame writer `fmt` (cellBP/iomesh.cpp:690-1047) into `path`."""
        f = self.lib.ref_write_vtk
        f.restype = None
        f.argtypes = [C.c_void_p, C.c_int32, C.c_int32] + [C.POINTER(C.c_double)] * 5 + [C.c_double, C.c_double,
                                                                                        C.c_char_p]
        f(h, fmt, len(x), dp(f64(x)), dp(f64(cA)), dp(f64(cC)), dp(f64(fau)), dp(f64(ea)), time, kint,
          str(path).encode())

    def mesh(self, tri, n_vert):
        tri = np.ascontiguousarray(tri, dtype=np.int32)
        h = self.lib.ref_mesh_new(n_vert, len(tri), ip(tri))
        return C.c_void_p(h)

    def mesh_map(self, h, n_vert, n_tri):
        ptr = np.zeros(n_vert + 1, np.int32); idx = np.zeros(3 * n_tri, np.int32); b = np.zeros(n_vert, np.uint8)
        k = self.lib.ref_mesh_map(h, ip(ptr), ip(idx), b.ctypes.data_as(_u8))
        return ptr, idx[:k], b

    def predict(self, x, V, A, dt):
        n = len(x)
        Vh = np.zeros((n, 3)); xp = np.zeros((n, 3))
        self.lib.ref_predict(n, dp(f64(x)), dp(f64(V).copy()), dp(f64(A)), C.c_double(dt), dp(Vh), dp(xp))
        return Vh, xp

    def area_tot(self, h, x):
        out = np.zeros(4)
        self.lib.ref_area_tot(h, len(x), dp(f64(x)), dp(out))
        return out

    def calc_res(self, h, X, x, ea, cA, cC, dt_real, mat, centroid, time):
        n = len(X)
        Res = np.zeros((n, 3)); Rea = np.zeros((n, 6)); MM = np.zeros(n); RA = np.zeros(n); RC = np.zeros(n)
        cen = f64(centroid if centroid is not None else np.zeros(3))
        self.lib.ref_calc_res(h, n, dp(f64(X)), dp(f64(x)), dp(f64(ea)), dp(None if cA is None else f64(cA)),
                              dp(None if cC is None else f64(cC)), C.c_double(dt_real), C.c_int32(mat), dp(cen),
                              C.c_double(time), dp(Res), dp(Rea), dp(MM), dp(RA), dp(RC))
        return Res, Rea, MM, RA, RC

    def force_fa(self, h, X, x, cC, fau, kint):
        F = np.zeros((len(x), 3))
        self.lib.ref_force_fa(h, len(x), dp(f64(X)), dp(f64(x)), dp(f64(cC)), dp(f64(fau)), C.c_double(kint), dp(F))
        return F

    def force_ap(self, h, X, x, cA, dt_real, seed, stream, call):
        F = np.zeros((len(x), 3))
        self.lib.ref_force_ap(h, len(x), dp(f64(X)), dp(f64(x)), dp(f64(cA)), C.c_double(dt_real),
                              C.c_uint32(seed), C.c_uint32(stream), C.c_uint64(call), dp(F))
        return F

    def force_bending(self, h, X, x):
        F = np.zeros((len(x), 3))
        self.lib.ref_force_bending(h, len(x), dp(f64(X)), dp(f64(x)), dp(F))
        return F

    def force_area(self, h, X, x, tot):
        F = np.zeros((len(x), 3))
        self.lib.ref_force_area(h, len(x), dp(f64(X)), dp(f64(x)), C.c_double(tot), dp(F))
        return F

    def update_fa(self, hc, cA, cC, fau, dt_real, X, x, hs, Xs, xs, kint):
        cA = f64(cA).copy(); cC = f64(cC).copy(); fau = f64(fau).copy()
        self.lib.ref_update_fa(hc, len(cC), dp(cA), dp(cC), dp(fau), C.c_double(dt_real), dp(f64(X)), dp(f64(x)),
                               hs, len(Xs), dp(f64(Xs)), dp(f64(xs)), C.c_double(kint))
        return cA, cC, fau

    def update_forces(self, h, X, x, V, Vh, A, ea, cA, cC, fau, dt, dt_real, t_tot, seed, stream, call):
        V = f64(V).copy(); A = f64(A).copy(); ea = f64(ea).copy()
        self.lib.ref_update_forces(h, len(x), dp(f64(X)), dp(f64(x)), dp(V), dp(f64(Vh)), dp(A), dp(ea),
                                   dp(f64(cA).copy()), dp(f64(cC).copy()), dp(f64(fau).copy()), C.c_double(dt),
                                   C.c_double(dt_real), C.c_double(t_tot), C.c_uint32(seed), C.c_uint32(stream),
                                   C.c_uint64(call))
        return V, A, ea

    def force_fa_subs(self, hs, Xs, xs, cC, hc, xcell, fau, kint):
        F = np.zeros((len(Xs), 3))
        self.lib.ref_force_fa_subs(hs, len(Xs), dp(f64(Xs)), dp(f64(xs)), dp(f64(cC)), hc, len(xcell),
                                   dp(f64(xcell)), dp(f64(fau)), C.c_double(kint), dp(F))
        return F

    def update_forces_subs(self, hs, Xs, xs, Vs, Vhs, As, eas, dt, dt_real, t_tot, fau, cC, hc, xcell):
        Vs = f64(Vs).copy(); As = f64(As).copy(); eas = f64(eas).copy()
        self.lib.ref_update_forces_subs(hs, len(Xs), dp(f64(Xs)), dp(f64(xs)), dp(Vs), dp(f64(Vhs)), dp(As), dp(eas),
                                        C.c_double(dt), C.c_double(dt_real), C.c_double(t_tot), dp(f64(fau).copy()),
                                        dp(f64(cC)), hc, len(xcell), dp(f64(xcell)))
        return Vs, As, eas

    def steps(self, hc, state, hs, Xs, kint, dt, nsteps, t, seed, stream, call):
        x, V, A, ea, cA, cC, fau = (f64(a).copy() for a in state)
        tt = C.c_double(t); cc = C.c_uint64(call)
        self.lib.ref_steps(hc, len(x), dp(x), dp(V), dp(A), dp(ea), dp(cA), dp(cC), dp(fau), hs, len(Xs),
                           dp(f64(Xs)), C.c_double(kint), C.c_double(dt), C.c_int32(nsteps), C.byref(tt), C.c_uint32(seed),
                           C.c_uint32(stream), C.byref(cc))
        return (x, V, A, ea, cA, cC, fau), tt.value, cc.value
