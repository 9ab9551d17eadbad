"""Generate the golden fixtures from the reference itself.

Runs the reference's own functions, compiled from its sources by
oracle/build_ref.sh into oracle/_ref/, on seeded synthetic inputs and on the
reference's own shipped meshes.  It stores their inputs and outputs as
tests/golden/golden_<variant>.npz and tests/golden/shipped_<variant>.npz.  The reference
ships no tests, expected outputs or golden vectors, so these fixtures are the
parity anchor.  The oracle must reproduce them (tests/test_oracle_golden.py)
on any machine, including ones without the reference sources.

usage: python tests/golden/make_golden.py     (needs oracle/_ref; run oracle/build_ref.sh first)
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402
from wholecellfe_gb300 import synth  # noqa: E402
from wholecellfe_gb300.params import default_params, kint_for  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
DT = 5e-5
T_TOT = 0.7           # inside the active-stress ramp (t < 2 s)
AP_DT = 0.03          # large enough that the actin push fires on some vertices
AP_CALL = 7


def make(variant: str) -> dict:
    R = O.Ref(variant)
    p = default_params(variant)
    x0, tri = synth.disk_mesh(300, seed=3)
    n = len(x0)
    hc = R.mesh(tri, n)
    vt_ptr, vt_idx, bnd = R.mesh_map(hc, n, len(tri))
    Xs, tri_s = synth.square_substrate(50.0, 24)
    hs = R.mesh(tri_s, len(Xs))
    rng = np.random.default_rng(11)
    xs_def = Xs + rng.normal(0, 0.01, Xs.shape) * np.array([1.0, 1.0, 0.0])
    x, V, A, ea, cA, cC, fau = synth.initial_state(x0, perturb=1.0, seed=5)
    kin = 31000.0 if variant == "kMD" else p.k_lin   # the value updateForces_Explicit hard-sets (UL:559-560)
    g: dict = dict(x0=x0, tri=tri, vt_ptr=vt_ptr, vt_idx=vt_idx, bnd=bnd, Xs=Xs, tri_s=tri_s, xs_def=xs_def,
                   x=x, V=V, A=A, ea=ea, cA=cA, cC=cC, fau=fau, dt=DT, t_tot=T_TOT, ap_dt=AP_DT, ap_call=AP_CALL,
                   seed=p.seed, stream=p.stream)
    Vh, xn = R.predict(x, V, A, DT)
    g.update(pred_Vh=Vh, pred_x=xn)
    area4 = R.area_tot(hc, xn)
    g.update(area4=area4)
    Res, Rea, MM, RA, RC = R.calc_res(hc, x, xn, ea, cA, cC, DT, 1, area4[1:], T_TOT)
    g.update(res_Res=Res, res_Rea=Rea, res_MM=MM, res_RA=RA, res_RC=RC)
    Res, Rea, MM, _, _ = R.calc_res(hs, Xs, xs_def, np.zeros((len(Xs), 6)), None, None, DT, 2, None, T_TOT)
    g.update(sres_Res=Res, sres_Rea=Rea, sres_MM=MM)
    g.update(f_fa=R.force_fa(hc, x, xn, cC, fau, kin))
    g.update(f_ap=R.force_ap(hc, x, xn, cA, AP_DT, p.seed, p.stream, AP_CALL))
    g.update(f_bend=R.force_bending(hc, x, xn))
    g.update(f_area=R.force_area(hc, x, xn, area4[0]))
    cA2, cC2, fau2 = R.update_fa(hc, cA, cC, fau, DT, x, xn, hs, Xs, xs_def, kint_for(variant))
    g.update(ufa_cA=cA2, ufa_cC=cC2, ufa_fau=fau2)
    V2, A2, ea2 = R.update_forces(hc, x, xn, V, Vh, A, ea, cA2, cC2, fau2, DT, DT, T_TOT, p.seed, p.stream, AP_CALL)
    g.update(uf_V=V2, uf_A=A2, uf_ea=ea2)
    # dt_real <= dt/2 branch of the velocity update (UL:622-628)
    V3, A3, ea3 = R.update_forces(hc, x, xn, V, Vh, A, ea, cA2, cC2, fau2, DT, 0.4 * DT, T_TOT, p.seed, p.stream,
                                  AP_CALL)
    g.update(uf2_V=V3, uf2_A=A3, uf2_ea=ea3)
    g.update(fsub=R.force_fa_subs(hs, Xs, xs_def, cC2, hc, xn, fau2, kin))
    Vs, As, eas = R.update_forces_subs(hs, Xs, xs_def, np.zeros_like(Xs), np.zeros_like(Xs), np.zeros_like(Xs),
                                       np.zeros((len(Xs), 6)), DT, DT, T_TOT, fau2, cC2, hc, xn)
    g.update(ufs_V=Vs, ufs_A=As, ufs_ea=eas)
    # trajectories: 40 steps from the reference start state, 40 from the perturbed one
    st0 = synth.initial_state(x0)
    s, t, c = R.steps(hc, st0, hs, Xs, kint_for(variant), DT, 40, 0.0, p.seed, p.stream, 0)
    for k, a in zip(("x", "V", "A", "ea", "cA", "cC", "fau"), s):
        g["traj0_" + k] = a
    g.update(traj0_t=t, traj0_call=c)
    s, t, c = R.steps(hc, (x, V, A, ea, cA, cC, fau), hs, Xs, kint_for(variant), DT, 40, T_TOT, p.seed, p.stream,
                      AP_CALL)
    for k, a in zip(("x", "V", "A", "ea", "cA", "cC", "fau"), s):
        g["traj1_" + k] = a
    g.update(traj1_t=t, traj1_call=c)
    return g


# VTK frames: the reference's writers on one seeded state, bond vectors spanning every
# segment of the MD table (cellBP/iomesh.cpp:927-949)
VTK_FRAMES = [("kMD", 0, -1.0), ("kMD", 1, -1.0), ("kMD", 2, -1.0), ("kMD", 2, 1000.0), ("k1", 2, -1.0),
              ("k31", 2, -1.0)]
VTK_TIME = 0.35


def vtk_state():
    x0, tri = synth.disk_mesh(60, seed=3)
    x, V, A, ea, cA, cC, fau = synth.initial_state(x0, perturb=1.0, seed=9)
    x = x + np.array([0.0, 0.0, 1e-3]) * np.sin(np.arange(len(x)))[:, None]
    ext = np.array([0.0, 0.001, 0.003, 0.005, 0.008, 0.013, 0.02, 0.03])
    for i, d in enumerate(ext):   # bond vectors of these lengths, one per MD segment and beyond
        fau[i] = d * np.array([0.6, 0.8, 0.0])
    ea[:, 2] = 0.002 * np.cos(np.arange(len(x)))
    return dict(x=x, tri=tri, cA=cA, cC=cC, fau=fau, ea=ea, time=VTK_TIME)


def vtk_name(variant, fmt, kint):
    return f"{variant}_f{fmt}" + ("_kint%g" % kint if kint >= 0 else "") + ".vtk"


# The reference's own meshes (cellBP/scripts, read as read_ecomsol reads them,
# cellBP/iomesh.cpp:491-565): three COMSOL-edited disks of 20 um diameter and the 100 um
# square substrate, used as the rigid substrate of every run below.
SHIPPED = ("disk_20um_diam_edited", "disk_20um_diam_N1025", "disk_20um_diam_N2944")
SHIPPED_SUBSTRATE = "sq_subs_100um"
SHIPPED_MOVING_STEPS = 20     # from a seeded moving, pre-strained state (all variants)
SHIPPED_REST_STEPS = 200      # from the reference start state (k1, k31; kMD from rest is noise-driven)
SHIPPED_SEED = 21
FINAL = ("x", "V", "ea", "cC", "fau")   # the end-state arrays stored


def read_comsol(path):
    """Vertices and triangles of a COMSOL text mesh as read_ecomsol reads it: the count on
    the line after the line holding "Nodes", that many coordinate lines (x y, z forced to 0);
    the count after "Elements", that many lines of three 0-based vertex indices."""
    lines = open(path).read().splitlines()
    x, tri = None, None
    for i, line in enumerate(lines):
        if "Nodes" in line:
            n = int(lines[i + 1].split()[0])
            x = np.zeros((n, 3))
            for k in range(n):
                f = lines[i + 2 + k].split()
                x[k, 0], x[k, 1] = float(f[0]), float(f[1])
        elif "Elements" in line:
            n = int(lines[i + 1].split()[0])
            tri = np.array([[int(v) for v in lines[i + 2 + k].split()[:3]] for k in range(n)], dtype=np.int32)
    return x, tri


def make_shipped(variant: str, ref_root: str) -> dict:
    """Trajectories of the reference's own step loop on its shipped meshes: for each mesh,
    SHIPPED_MOVING_STEPS steps from a seeded moving state and (k1, k31) SHIPPED_REST_STEPS
    steps from rest, over the shipped substrate held rigid."""
    R = O.Ref(variant)
    p = default_params(variant)
    d = os.path.join(ref_root, "wholeCellFE_kMD", "cellBP", "scripts")
    Xs, tri_s = read_comsol(os.path.join(d, SHIPPED_SUBSTRATE + ".txt"))
    hs = R.mesh(tri_s, len(Xs))
    g: dict = dict(Xs=Xs, tri_s=tri_s, dt=DT, seed=p.seed, stream=p.stream)
    keep = ("x", "V", "A", "ea", "cA", "cC", "fau")
    for m, name in enumerate(SHIPPED):
        x0, tri = read_comsol(os.path.join(d, name + ".txt"))
        hc = R.mesh(tri, len(x0))
        g[f"m{m}_x0"], g[f"m{m}_tri"] = x0, tri
        st = synth.initial_state(x0, perturb=1.0, seed=SHIPPED_SEED + m)
        for k, a in zip(keep, st):
            g[f"m{m}_mov0_{k}"] = a
        s, t, c = R.steps(hc, st, hs, Xs, kint_for(variant), DT, SHIPPED_MOVING_STEPS, T_TOT, p.seed, p.stream, AP_CALL)
        for k, a in zip(keep, s):
            if k in FINAL:
                g[f"m{m}_mov_{k}"] = a
        g[f"m{m}_mov_t"], g[f"m{m}_mov_call"] = t, c
        if variant != "kMD":
            s, t, c = R.steps(hc, synth.initial_state(x0), hs, Xs, kint_for(variant), DT, SHIPPED_REST_STEPS, 0.0,
                              p.seed, p.stream, 0)
            for k, a in zip(keep, s):
                if k in FINAL:
                    g[f"m{m}_rest_{k}"] = a
            g[f"m{m}_rest_t"], g[f"m{m}_rest_call"] = t, c
    return g


def main():
    ref_root = os.environ.get("WCFE_REF", "/root/reference")
    for variant in ("kMD", "k1", "k31"):
        if not O.ref_available(variant):
            sys.exit("oracle/_ref not built: run oracle/build_ref.sh first")
        g = make_shipped(variant, ref_root)
        path = os.path.join(HERE, f"shipped_{variant}.npz")
        np.savez_compressed(path, **g)
        print("wrote", path, os.path.getsize(path), "bytes")
    for variant in ("kMD", "k1", "k31"):
        if not O.ref_available(variant):
            sys.exit("oracle/_ref not built: run oracle/build_ref.sh first")
        g = make(variant)
        path = os.path.join(HERE, f"golden_{variant}.npz")
        np.savez_compressed(path, **g)
        print("wrote", path, os.path.getsize(path), "bytes")
    st = vtk_state()
    os.makedirs(os.path.join(HERE, "vtk"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "vtk", "state.npz"), **st)
    for variant, fmt, kint in VTK_FRAMES:
        R = O.Ref(variant)
        h = R.mesh(st["tri"], len(st["x"]))
        path = os.path.join(HERE, "vtk", vtk_name(variant, fmt, kint))
        R.write_vtk(h, fmt, st["x"], st["cA"], st["cC"], st["fau"], st["ea"], VTK_TIME, kint, path)
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
