"""Seeded synthetic cells: disk membranes, substrates and initial state.

The reference reads its meshes from edited-COMSOL text files
(cellBP/iomesh.cpp:491-565 read_ecomsol); the workloads here are generated
instead, with the shapes the benchmark configurations name:

* ``disk_mesh`` — a triangulated disk (default radius 10 um).  Vertices sit on
  concentric rings of spacing h = R/K with round(2*pi*k) points on ring k, so
  the triangles are close to equilateral; neighbouring rings are stitched by a
  merge walk in angle, and interior vertices get a seeded jitter of +-2% of h.
  Triangles are counter-clockwise (z-up normal), like the reference meshes.
  Vertices are renumbered along a Morton (Z-order) curve so that consecutive
  vertex ranges are compact patches of the membrane.
* ``square_substrate`` — a structured square substrate mesh.
* ``initial_state`` — the reference's start state (all zero, c_A = 100,
  cellBP/main.cpp:674-677) or a seeded perturbed state for parity tests.
"""
from __future__ import annotations

import math

import numpy as np


def _ring_counts(K: int) -> list[int]:
    return [1] + [max(6, int(round(2.0 * math.pi * k))) for k in range(1, K + 1)]


def rings_for(n_target: int) -> int:
    """Ring count K whose disk has about n_target vertices."""
    K = max(2, int(round(math.sqrt(max(n_target, 8) / math.pi))))
    while K > 2 and sum(_ring_counts(K)) > n_target * 1.02:
        K -= 1
    while sum(_ring_counts(K + 1)) <= n_target:
        K += 1
    return K


def _morton_order(xy: np.ndarray) -> np.ndarray:
    lo = xy.min(axis=0)
    span = max(float((xy.max(axis=0) - lo).max()), 1e-30)
    q = np.floor((xy - lo) / span * 65535.0).astype(np.uint64)
    code = np.zeros(len(xy), dtype=np.uint64)
    for b in range(16):
        code |= ((q[:, 0] >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b)
        code |= ((q[:, 1] >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b + 1)
    return np.argsort(code, kind="stable")


def disk_mesh(n_target: int, radius: float = 10.0, jitter: float = 0.02, seed: int = 1,
              reorder: bool = True):
    """Return (x[n,3] float64, tri[t,3] int32) for a disk of about n_target vertices."""
    K = rings_for(n_target)
    counts = _ring_counts(K)
    h = radius / K
    rng = np.random.default_rng(seed)
    pts = [np.zeros((1, 2))]
    angles = [np.zeros(1)]
    for k in range(1, K + 1):
        n = counts[k]
        phase = (0.5 * (k % 2)) * 2.0 * math.pi / n
        th = phase + 2.0 * math.pi * np.arange(n) / n
        angles.append(th)
        pts.append(np.stack([k * h * np.cos(th), k * h * np.sin(th)], axis=1))
    start = np.cumsum([0] + counts)
    tris = []
    # center fan
    n1 = counts[1]
    for j in range(n1):
        tris.append((0, start[1] + j, start[1] + (j + 1) % n1))
    # zipper between ring k-1 and ring k
    for k in range(2, K + 1):
        na, nb = counts[k - 1], counts[k]
        ta = np.concatenate([angles[k - 1], angles[k - 1][:1] + 2 * math.pi])
        tb = np.concatenate([angles[k], angles[k][:1] + 2 * math.pi])
        i = j = 0
        while i < na or j < nb:
            a0, b0 = start[k - 1] + i % na, start[k] + j % nb
            if j >= nb or (i < na and ta[i + 1] < tb[j + 1]):
                tris.append((a0, b0, start[k - 1] + (i + 1) % na))
                i += 1
            else:
                tris.append((a0, b0, start[k] + (j + 1) % nb))
                j += 1
    xy = np.concatenate(pts, axis=0)
    n = len(xy)
    interior = np.ones(n, dtype=bool)
    interior[start[K]:] = False
    jit = rng.uniform(-jitter * h, jitter * h, size=(n, 2))
    xy = xy + jit * interior[:, None]
    tri = np.asarray(tris, dtype=np.int64)
    if reorder:
        order = _morton_order(xy)
        inv = np.empty(n, dtype=np.int64)
        inv[order] = np.arange(n)
        xy = xy[order]
        tri = inv[tri]
        tri = tri[np.argsort(tri.min(axis=1), kind="stable")]
    x = np.zeros((n, 3))
    x[:, :2] = xy
    return x, tri.astype(np.int32)


def annulus_mesh(n_target: int, hole: float = 0.35, radius: float = 10.0, seed: int = 1):
    """A disk mesh with the triangles whose centroid lies within hole * radius of the
    centre removed, unused vertices dropped (vertex order kept): a mesh with two
    boundary loops.  Returns (x[n,3] float64, tri[t,3] int32)."""
    x, tri = disk_mesh(n_target, radius=radius, seed=seed)
    c = x[tri].mean(axis=1)
    tri = tri[np.hypot(c[:, 0], c[:, 1]) > hole * radius]
    used = np.unique(tri)
    remap = -np.ones(len(x), np.int64)
    remap[used] = np.arange(len(used))
    return np.ascontiguousarray(x[used]), np.ascontiguousarray(remap[tri].astype(np.int32))


def square_substrate(half: float = 50.0, cells: int = 24):
    """Structured square mesh [-half, half]^2 with alternating diagonals (CCW)."""
    m = cells + 1
    g = np.linspace(-half, half, m)
    X, Y = np.meshgrid(g, g, indexing="xy")
    x = np.zeros((m * m, 3))
    x[:, 0] = X.ravel()
    x[:, 1] = Y.ravel()
    tris = []
    for r in range(cells):
        for c in range(cells):
            v00 = r * m + c
            v01 = v00 + 1
            v10 = v00 + m
            v11 = v10 + 1
            if (r + c) % 2 == 0:
                tris += [(v00, v01, v11), (v00, v11, v10)]
            else:
                tris += [(v00, v01, v10), (v01, v11, v10)]
    return x, np.asarray(tris, dtype=np.int32)


def vertex_triangle_map(n: int, tri: np.ndarray):
    """CSR vertex -> triangle map in ascending triangle order (what add_triangle builds)."""
    tri = np.asarray(tri)
    flat = tri.ravel()
    order = np.argsort(flat, kind="stable")
    counts = np.bincount(flat, minlength=n)
    ptr = np.zeros(n + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(counts)
    idx = (order // 3).astype(np.int32)
    return ptr, idx


def boundary_flags(n: int, tri: np.ndarray) -> np.ndarray:
    """1 for vertices on an edge with an odd triangle count."""
    tri = np.asarray(tri, dtype=np.int64)
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]], axis=0)
    e.sort(axis=1)
    key = e[:, 0] * n + e[:, 1]
    uniq, cnt = np.unique(key, return_counts=True)
    odd = uniq[cnt % 2 == 1]
    b = np.zeros(n, dtype=np.uint8)
    b[odd // n] = 1
    b[odd % n] = 1
    return b


def initial_state(x: np.ndarray, perturb: float = 0.0, seed: int = 0):
    """State arrays (x, V, A, ea, cA, cC, fau).  perturb > 0 gives a seeded non-trivial state."""
    n = len(x)
    rng = np.random.default_rng(seed)
    V = np.zeros((n, 3))
    A = np.zeros((n, 3))
    ea = np.zeros((n, 6))
    cA = np.full(n, 100.0)
    cC = np.zeros(n)
    fau = np.zeros((n, 3))
    x = np.array(x, dtype=np.float64, copy=True)
    if perturb > 0:
        V[:, :2] = rng.normal(0, 0.05 * perturb, size=(n, 2))
        A[:, :2] = rng.normal(0, 1.0 * perturb, size=(n, 2))
        ea[:, [0, 1, 3]] = rng.normal(0, 0.01 * perturb, size=(n, 3))
        cC[:] = rng.uniform(0.0, 0.5, size=n)
        fau[:, :2] = rng.normal(0, 0.004 * perturb, size=(n, 2))
    return x, V, A, ea, cA, cC, fau


def protruding_cell(n_target: int = 2100, integrins: int = 600, dt: float = 5e-5, seed: int = 1,
                    E: float = 1000.0, nu: float = 0.45, thickness: float = 0.1):
    """The single-cell workload with a protruding edge: a disk of radius 10 um with about
    n_target vertices (seeded +-2 % jitter; 2,044 vertices and 3,929 triangles by default), membrane modulus E (Pa) and Poisson ratio nu
    mapped to the shear modulus mu = E / (2 (1 + nu)) (the small-strain map of the
    reference's incompressible neo-Hookean membrane, UL:861-865), thickness in um, linear
    integrin springs of 1 pN/nm with a 20 nm rest length on `integrins` vertices (the ones
    nearest to as many seeded anchor points uniform over the disk, distinct), and every
    boundary vertex driven radially outward by 10 nm per step of dt.  Returns
    (x0, tri, params, rho) with rho the per-vertex integrin density."""
    from .params import LAW_LINEAR, default_params
    x0, tri = disk_mesh(n_target, seed=seed)
    p = default_params("k1")
    p.mu = E / (2.0 * (1.0 + nu))
    p.thick = thickness
    p.force_law, p.k_lin, p.rest_len = LAW_LINEAR, 1000.0, 0.02
    p.protrude_v = 0.010 / dt
    p.protrude_cx = p.protrude_cy = 0.0
    rng = np.random.default_rng([seed, 600])
    r = 10.0 * np.sqrt(rng.uniform(0.0, 1.0, 4 * integrins))
    a = rng.uniform(0.0, 2.0 * np.pi, 4 * integrins)
    anchors = np.c_[r * np.cos(a), r * np.sin(a)]
    rho = np.zeros(len(x0))
    taken = 0
    for q in anchors:   # nearest free vertex of each anchor, until `integrins` vertices carry one
        d = np.sum((x0[:, :2] - q) ** 2, axis=1)
        d[rho > 0] = np.inf
        rho[int(np.argmin(d))] = p.rho_i_max
        taken += 1
        if taken == integrins:
            break
    return x0, tri, p, rho
