"""Benchmark: cell-steps/s of the batched mixed-precision form against the plain
one-cell FP64 form on one GB300 (the metric of the wholeCellFE mechanics step).

Workload (N = 1): 256 uneven cells, vertex counts log-uniform in [500, 20000]
(seeded disk meshes), integrins on 0.4 x N vertices, stiffness model per cell
drawn from {linear 1 pN/nm, linear 31 pN/nm, polynomial k0 = 31 pN/nm x0 = 5 nm},
flat rigid substrate, dt = 5e-5 s, from rest.  One "step" advances every cell by
one explicit step (A1-A9), so a step is 256 cell-steps.

Reported on one JSON line: the headline value (batched mixed form: FP32 element
assembly and forces, float-float state and accumulation; device-timed, inputs
resident, the steps replayed from captured CUDA graphs; the same steps launched
eagerly with per-step events give the p50/p99 step latency), e2e (the same loop through the batched drop-in exchange with
pinned host buffers: per step the predicted positions go to the host and the
integrated positions come back), the plain FP64 one-cell form (about 2000 vertices),
the relative displacement error of the mixed form against the FP64 form, per-step
p50/p99 latency, the roofline of the dominant kernel, GPU clocks sampled during the
timed region, and the CPU baseline.

--impl reference: the reference's CPU path on the host cores (the oracle port of
cellBP/UL_growth_explicit.cpp, all threads), same workload, bounded sample.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s batched+mixed vs plain FP64 on 1 GB300 at <=1e-6 rel err; p50/p99"
ELEMENT_FLOPS = 2360   # FP64 flops of the reference's cell element (oracle/flop_count.cpp)
DT = 5e-5
N_CELLS = 256


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- workload
def workload_specs(seed: int, ncells: int):
    """Per-cell draws of the workload (vertex target, stiffness model); cheap, so every
    rank draws the whole population and builds only its own shard."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(ncells):
        n = int(round(math.exp(rng.uniform(math.log(500), math.log(20000)))))
        specs.append(dict(index=i, n=n, model=int(rng.integers(0, 3))))
    return specs


def build_cell(seed: int, spec):
    from wholecellfe_gb300 import synth
    from wholecellfe_gb300.params import default_params
    i, model = spec["index"], spec["model"]
    x0, tri = synth.disk_mesh(spec["n"], seed=seed * 100003 + i)
    if model == 0:
        p = default_params("k1")
    elif model == 1:
        p = default_params("k31")
    else:
        p = default_params("k31")
        p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
    p.seed, p.stream = seed & 0xffffffff, i
    nv = len(x0)
    rho = np.zeros(nv)
    pick = np.random.default_rng([seed, i]).choice(nv, size=max(1, int(round(0.4 * nv))), replace=False)
    rho[pick] = p.rho_i_max
    return dict(x0=x0, tri=tri, p=p, rho=rho, model=model)


def make_workload(seed: int, ncells: int = N_CELLS, shard=None):
    """The cells of the workload (all of them, or the indices in `shard`)."""
    specs = workload_specs(seed, ncells)
    idx = range(ncells) if shard is None else shard
    return [build_cell(seed, specs[i]) for i in idx]


def load_cells(eng, cells):
    from wholecellfe_gb300 import synth
    hs = []
    for c in cells:
        h = eng.add_cell(c["x0"], c["tri"], c["p"], state=synth.initial_state(c["x0"]))
        h.set_integrins(c["rho"])
        hs.append(h)
    return hs


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([s.strip() for s in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ----------------------------------------------------------------------------- CPU baseline
def cpu_baseline(cells, steps: int, budget_s: float = 15.0):
    """The oracle (C port of the reference's step) on the host cores, all threads, on a
    bounded sample of the workload's cells; returns cell-steps/s and what was run."""
    from oracle import oracle_py as O
    from wholecellfe_gb300 import synth
    nthreads = os.cpu_count() or 1
    # probe one mid-size cell for one step to size the sample
    probe = min(cells, key=lambda c: abs(len(c["x0"]) - 5000))
    m = O.OMesh(probe["tri"], len(probe["x0"]))
    oc = O.OCell(m, synth.initial_state(probe["x0"]), probe["p"], rho_w=probe["rho"])
    t0 = time.perf_counter()
    oc.steps(1, DT)
    per_vertex_step = (time.perf_counter() - t0) / len(probe["x0"])
    mean_nv = float(np.mean([len(c["x0"]) for c in cells]))
    ncs = max(nthreads, min(len(cells), 64))
    nsteps = max(1, int(budget_s * nthreads / (per_vertex_step * mean_nv * ncs)))
    nsteps = min(nsteps, steps)
    sample = cells[:ncs]
    ocs = []
    meshes = []
    for c in sample:
        mm = O.OMesh(c["tri"], len(c["x0"]))
        meshes.append(mm)
        ocs.append(O.OCell(mm, synth.initial_state(c["x0"]), c["p"], rho_w=c["rho"]))
    t0 = time.perf_counter()
    O.cells_steps_mt(ocs, nsteps, DT, nthreads)
    dt = time.perf_counter() - t0
    return {"value": len(sample) * nsteps / dt, "unit": "cell-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{len(sample)} of the workload's cells (mean {np.mean([len(c['x0']) for c in sample]):.0f} "
                      f"vertices) x {nsteps} steps, oracle/wcfe_oracle.c on {nthreads} host threads, {dt:.1f} s"}


def _ref_worker(job):
    """One process of the reference-build baseline: the reference's own step loop
    (oracle/_ref, cellBP/UL_growth_explicit.cpp compiled from its sources) on its cells."""
    from oracle import oracle_py as O
    from wholecellfe_gb300 import synth
    from wholecellfe_gb300.params import kint_for
    cells, nsteps = job
    Xs = np.array([[-60.0, -60.0, 0.0], [60.0, -60.0, 0.0], [60.0, 60.0, 0.0], [-60.0, 60.0, 0.0]])
    tri_s = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int32)   # a rigid plane under the cells
    t0 = time.perf_counter()
    done = 0
    for c in cells:
        variant = "k1" if c["model"] == 0 else "k31"
        R = O.Ref(variant)
        hc, hs = R.mesh(c["tri"], len(c["x0"])), R.mesh(tri_s, len(Xs))
        R.steps(hc, synth.initial_state(c["x0"]), hs, Xs, kint_for(variant), DT, nsteps, 0.0, c["p"].seed,
                c["p"].stream, 0)
        done += nsteps
    return done, time.perf_counter() - t0


def ref_build_baseline(cells, steps: int, budget_s: float = 15.0, procs: int | None = None):
    """The reference's own CPU path (oracle/_ref, built from the reference's sources) on a
    bounded sample of the workload's linear-law cells (the reference has no polynomial
    law), one process per core (its rand() stand-in is process-global).  None where
    oracle/_ref is absent (it is built only where the reference sources are)."""
    import multiprocessing as mp
    from oracle import oracle_py as O
    if not (O.ref_available("k1") and O.ref_available("k31")):
        return None
    procs = procs or (os.cpu_count() or 1)
    lin = [c for c in cells if c["model"] in (0, 1)]
    probe = min(lin, key=lambda c: abs(len(c["x0"]) - 5000))
    done, sec = _ref_worker(([probe], 1))
    per_vertex_step = sec / len(probe["x0"])
    sample = lin[:max(procs, min(len(lin), 32))]
    mean_nv = float(np.mean([len(c["x0"]) for c in sample]))
    nsteps = max(1, min(steps, int(budget_s * procs / (per_vertex_step * mean_nv * len(sample)))))
    jobs = [(sample[i::procs], nsteps) for i in range(procs) if sample[i::procs]]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        res = pool.map(_ref_worker, jobs)
    wall = time.perf_counter() - t0
    return {"value": round(sum(r[0] for r in res) / wall, 1), "unit": "cell-steps/s", "cores": len(jobs),
            "kind": "reference",
            "sample": f"{len(sample)} linear-law cells of the workload (mean {mean_nv:.0f} vertices) x {nsteps} steps, "
                      f"the reference's UL_growth_explicit.cpp built from its sources (oracle/_ref), {len(jobs)} "
                      f"processes, {wall:.1f} s wall"}


# ----------------------------------------------------------------------------- measurements
def kernel_bytes_patch_mixed(nv_total: int, nt_total: int) -> float:
    """Algorithmic DRAM bytes of one mixed patch-phase launch (float-float state).
    Per owned vertex it reads the FP32 element record (48 B), the high half of the
    bond vector (16), c_C (4, its high word), the integrin density (8), V (32), the
    FP32 acceleration (16), the strain xx yy zz xy (32), the one-ring offset and
    boundary rank (8) and 2 B of slot code per incidence (3 per triangle); it writes
    A (16), V (32) and the strain (32).  Per element it reads the triangle (16) and
    its patch entry (4)."""
    per_v = 48 + 16 + 4 + 8 + 32 + 16 + 32 + 8 + 16 + 32 + 32
    per_t = 16 + 4 + 3 * 2
    return per_v * nv_total + per_t * nt_total


def kernel_bytes_vertex_mixed(nv_total: int) -> float:
    """Algorithmic DRAM bytes of one mixed vertex-phase launch: per vertex it reads the
    triple-float position (32 B), V (32), the FP32 acceleration (16), the bond vector
    (32), c_C and c_A (8 each), the strain's high words (16) and the boundary rank (4);
    it writes the predicted position (32), the bond vector (32), c_C (8) and the FP32
    element record (48)."""
    return (32 + 32 + 16 + 32 + 8 + 8 + 16 + 4 + 32 + 32 + 8 + 48) * nv_total


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    f, c = math.floor(k), math.ceil(k)
    return xs[f] if f == c else xs[f] + (xs[c] - xs[f]) * (k - f)


def timed_steps(eng, steps, dt, ranks_barrier=None):
    """Device-timed steps on the engine's own stream: the engine records CUDA events
    before each phase of every step (no host synchronisation inside the timed region);
    total = first event to last event, plus per-step and per-phase durations."""
    import torch
    eng.set_timing(True)
    eng.sync()
    torch.cuda.synchronize()
    if ranks_barrier:
        ranks_barrier()
    t_host0 = time.perf_counter()
    eng.step(steps, dt)          # returns after the last event completed
    eng.sync()
    wall = time.perf_counter() - t_host0
    torch.cuda.synchronize()
    per_step, span = eng.step_times()
    ms_v, ms_p = eng.last_timing()
    eng.set_timing(False)
    return dict(total_ms=span, wall_s=wall, per_step=per_step, ms_v=ms_v, ms_p=ms_p)


def timed_graph_steps(eng, steps, dt, ranks_barrier=None):
    """The same loop replayed from captured CUDA graphs (eight steps per graph), timed by
    CUDA events recorded on the engine's own stream."""
    import torch
    eng.set_graphs(True)
    eng.step(8, dt)   # capture and first replay
    eng.sync()
    st = torch.cuda.ExternalStream(eng.stream_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if ranks_barrier:
        ranks_barrier()
    l0 = eng.launches()
    e0.record(st)
    eng.step(steps, dt)
    e1.record(st)
    e1.synchronize()
    launches = eng.launches() - l0
    eng.set_graphs(False)
    return {"total_ms": e0.elapsed_time(e1), "launches": launches}


def run_ours(args):
    import torch
    from wholecellfe_gb300 import capi
    from wholecellfe_gb300.params import default_params
    from wholecellfe_gb300 import synth

    from wholecellfe_gb300.replicas import max_over_ranks, partition_cells, rank_env

    env = rank_env()
    world, rank, local = env.world, env.rank, env.local
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if world > 1 else 0
    torch.cuda.init()

    def barrier():
        if dist:
            dist.barrier()

    # weak scaling: a population of cells x world cells, sharded by vertex count, no data-path collective
    specs = workload_specs(1000, args.cells * world)
    shards = partition_cells([s["n"] for s in specs], world)
    cells = [build_cell(1000, specs[i]) for i in shards[rank]]
    nv_total = sum(len(c["x0"]) for c in cells)
    nt_total = sum(len(c["tri"]) for c in cells)
    log(f"[bench] rank {rank}: {len(cells)} cells, {nv_total} vertices, {nt_total} triangles")

    # ---- batched mixed form (headline) ----
    eng = capi.Engine(capi.PREC_MIXED, device=device)
    load_cells(eng, cells)
    eng.autotune(DT, 3)
    thr, emax = eng.shape()
    kinds = eng.kernels()
    # clocks over the whole measurement window (warm-up, the eager and graph-captured timed
    # steps and the e2e steps): a timed region of a few ms is shorter than nvidia-smi's period
    clocks = ClockSampler()
    clocks.start()
    for _ in range(args.warmup):
        eng.step(1, DT)
    eng.sync()
    launches0 = eng.launches()
    res = timed_steps(eng, args.steps, DT, barrier)
    launches = eng.launches() - launches0
    graph = timed_graph_steps(eng, args.steps, DT, barrier)
    graph_s = max_over_ranks(graph["total_ms"] / 1e3, dist, f"cuda:{local}")
    eager_s = max_over_ranks(res["total_ms"] / 1e3, dist, f"cuda:{local}")
    eager_value = len(specs) * args.steps / eager_s
    # the headline: the batched form as it runs in production, its steps replayed from captured
    # CUDA graphs (the same K steps, CUDA events on the engine stream around them)
    t_s = graph_s
    value = len(specs) * args.steps / t_s
    p50 = percentile(res["per_step"], 0.5)
    p99 = percentile(res["per_step"], 0.99)
    avg_v = res["ms_v"] / args.steps
    avg_p = res["ms_p"] / args.steps
    log(f"[bench] mixed: {t_s * 1e3 / args.steps:.3f} ms/step from graphs, {value:.3e} cell-steps/s; eager "
        f"{eager_s * 1e3 / args.steps:.3f} ms/step (vertex {avg_v:.3f}, patch {avg_p:.3f})")

    # ---- e2e through the batched drop-in exchange, pinned host buffers ----
    ntot = eng.total_vertices()
    host = torch.empty((ntot, 3), dtype=torch.float64, pin_memory=True)
    xbuf = host.numpy()
    # the exchange groups (streams whose predict and copies overlap the others' updates):
    # fewer, larger groups keep the kernels' waves full, more hide more of the copies;
    # the count is chosen by timing a few exchange steps of each (public API:
    # wcfe_engine_set_exchange_groups), then the timed loop runs with it
    group_ms = {}
    for groups in (1, 2, 4, 8):
        eng.set_exchange_groups(groups)
        for _ in range(2):
            eng.predict_all(DT, xbuf)
            eng.update_all(DT, DT, xbuf)
        eng.sync()
        t0 = time.perf_counter()
        for _ in range(4):
            eng.predict_all(DT, xbuf)
            eng.update_all(DT, DT, xbuf)
        eng.sync()
        group_ms[groups] = (time.perf_counter() - t0) / 4 * 1e3
    best_groups = min(group_ms, key=group_ms.get)
    eng.set_exchange_groups(best_groups)
    for _ in range(2):
        eng.predict_all(DT, xbuf)
        eng.update_all(DT, DT, xbuf)
    eng.sync()
    barrier()
    e_launch0 = eng.launches()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.predict_all(DT, xbuf)          # device step part 1 + D2H of the predicted positions
        eng.update_all(DT, DT, xbuf)       # H2D of the integrated positions + device step part 2
    eng.sync()
    e2e_s = time.perf_counter() - t0
    e2e_launches = eng.launches() - e_launch0
    e2e_s = max_over_ranks(e2e_s, dist, f"cuda:{local}")
    e2e = {"value": len(specs) * args.steps / e2e_s, "unit": "cell-steps/s",
           "h2d_bytes_per_step": int(ntot * 24), "d2h_bytes_per_step": int(ntot * 24),
           "api": "wcfe_engine_predict + wcfe_engine_update (include/wcfe.h), pinned host buffers",
           "exchange_groups": best_groups,
           "ms_per_step_by_groups": {str(k): round(v, 4) for k, v in group_ms.items()},
           "gpu_launches": int(e2e_launches)}
    log(f"[bench] e2e: {e2e['value']:.3e} cell-steps/s")
    # the timed regions last a few ms, shorter than nvidia-smi's 50 ms period: the same steps
    # continue (untimed) for 0.6 s so that the clock record holds samples under this load
    t_clk = time.perf_counter() + 0.6
    while time.perf_counter() < t_clk:
        eng.step(50, DT)
        eng.sync()
    clocks_info = clocks.stop()
    clocks_info["window"] = ("warm-up, eager and graph-captured timed steps, e2e steps, then 0.6 s more of the "
                             "same steps (untimed)")
    eng.close()

    out = None
    if rank == 0:
        # ---- error of the mixed form against the FP64 form (same workload), at the
        # workload's own 300-step horizon and at 20 steps beside the FP64 form's own noise ----
        accuracy = mixed_error(cells, device)
        max_err = accuracy["gate"]["max_rel_displacement_error"]
        err_steps = accuracy["gate"]["steps"]
        log(f"[bench] mixed vs FP64: {json.dumps(accuracy)}")

        # ---- the pipe rates of this GPU (roofline denominators the peak file does not hold) ----
        rates = capi.pipe_rates()
        log(f"[bench] pipe rates: {rates}")

        # ---- plain one-cell FP64 form: the single-cell workload with a protruding edge (2,044
        # vertices, E 1 kPa / nu 0.45, 0.1 um thick, 600 integrins 1 pN/nm rest 20 nm, 10 nm/step) ----
        x0, tri, p, rho = synth.protruding_cell(dt=DT)
        ep = capi.Engine(capi.PREC_FP64, device=device)
        hp = ep.add_cell(x0, tri, p, state=synth.initial_state(x0))
        hp.set_integrins(rho)
        ep.autotune(DT, 5)
        plain_shape = ep.shape()
        for _ in range(args.warmup):
            ep.step(1, DT)
        plain_steps = 200
        pr = timed_steps(ep, plain_steps, DT)
        ep.close()
        plain_value = plain_steps / (pr["total_ms"] / 1e3)
        # its FP64 work: the reference's element, 2,360 flops (oracle/flop_count.cpp), per triangle and step
        plain_flops = ELEMENT_FLOPS * len(tri)
        plain_achieved = plain_flops / (pr["total_ms"] / plain_steps * 1e-3) / 1e12
        plain_roofline = {"bound": "fp64", "achieved": round(plain_achieved, 5), "peak": round(rates["fp64_tflops"], 4),
                          "unit": "TFLOP/s", "frac": round(plain_achieved / rates["fp64_tflops"], 4),
                          "peak_source": "measured FP64 FMA rate of this GPU (wcfe_debug_pipe_rates)",
                          "note": "2,360 FP64 flops per element x 3,929 elements per step over the step's device "
                                  "time; one 2,044-vertex cell is a few dozen CTAs per phase, less than one wave of the "
                                  "152 SMs, so the form is latency-bound"}
        plain_wall = plain_steps / pr["wall_s"]
        log(f"[bench] plain FP64 one cell: {pr['total_ms'] / plain_steps * 1e3:.1f} us/step device, "
            f"{plain_value:.3e} cell-steps/s device, {plain_wall:.3e} wall")

        # ---- roofline of the dominant kernel ----
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except OSError:
            pass
        hbm = peaks.get("hbm_gbs", 6800.0)
        kbytes = kernel_bytes_patch_mixed(nv_total, nt_total)
        achieved = kbytes / (avg_p * 1e-3) / 1e9
        traffic = None
        prof = os.path.join(ROOT, "profiles", "k_patch_phase_mixed.md")
        if os.path.exists(prof):
            for line in open(prof):
                if line.startswith("dram_bytes_per_vertex:"):
                    traffic = float(line.split(":")[1]) * nv_total
        vbytes = kernel_bytes_vertex_mixed(nv_total)
        step_ms = t_s * 1e3 / args.steps
        roofline = {"bound": "hbm", "kernel": "k_patch_phase_mixed", "achieved": round(achieved, 1),
                    "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                    "traffic": traffic, "algorithmic_bytes_per_launch": int(kbytes),
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s",
                    "avg_launch_ms": round(avg_p, 4), "vertex_phase_avg_launch_ms": round(avg_v, 4),
                    "vertex_phase": {"algorithmic_bytes_per_launch": int(vbytes),
                                     "achieved": round(vbytes / (avg_v * 1e-3) / 1e9, 1),
                                     "frac": round(vbytes / (avg_v * 1e-3) / 1e9 / hbm, 4)},
                    "step": {"algorithmic_bytes": int(kbytes + vbytes), "ms": round(step_ms, 4),
                             "achieved": round((kbytes + vbytes) / (step_ms * 1e-3) / 1e9, 1),
                             "frac": round((kbytes + vbytes) / (step_ms * 1e-3) / 1e9 / hbm, 4),
                             "note": "both phases' algorithmic bytes over the graph-replayed step time"}}

        config2 = run_config2()
        log(f"[bench] config 2: {config2}")
        newton = run_newton(args.newton_cells, tf32_peak=rates["tf32_tflops"]) if args.newton_cells > 0 else None
        if newton:
            log(f"[bench] newton: {newton}")
        serving = None
        if args.serve_seconds > 0:
            serving = {"poisson": run_serving(args.serve_seconds),
                       "saturated": run_serving(saturate=args.serve_saturate, budget_gb=4.0, seed=8)}
            serving["capacity_vs_plain_fp64"] = round(serving["saturated"]["cell_steps_per_s"] / plain_value, 2)
            log(f"[bench] serving: {serving}")
        cpu = None
        if not args.no_cpu:
            port = cpu_baseline(cells, args.steps)
            ref = ref_build_baseline(cells, args.steps)
            cpu = ref if ref else port
            if ref:
                cpu["port"] = port
            else:
                cpu["reference_build"] = ("unavailable here: the reference's sources are not on this machine and "
                                          "oracle/_ref holds no build for it; the oracle port is timed instead")
        out = {
            "metric": METRIC, "value": round(value, 1), "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_s * 1e3 / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (assembly, forces) + float-float (state, accumulation)",
            "data": "synthetic: seeded disk meshes, random-init state from rest",
            "config": {**workload_config(cells),
                       "l2": f"state {nv_total * 600 / 1e9:.2f} GB resident > 129 MB L2 (inputs larger than L2)",
                       "patch_threads": thr, "patch_elems": emax, "patch_kernel": kinds[0],
                       "vertex_kernel": kinds[1], "autotuned": True,
                       "parallelism": f"cell shards x{world} (population {len(specs)} cells, LPT by vertex count, "
                                      "no data-path collective)"},
            "p50_ms_per_step": round(p50, 4), "p99_ms_per_step": round(p99, 4),
            "timing": "value: the K steps replayed from captured CUDA graphs (8 steps each), CUDA events on the "
                      "engine stream around them; p50/p99: the same K steps launched eagerly with events around "
                      "every step (`eager`)",
            "eager": {"value": round(eager_value, 1), "unit": "cell-steps/s",
                      "ms_per_step": round(eager_s * 1e3 / args.steps, 4),
                      "vertex_phase_ms": round(avg_v, 4), "patch_phase_ms": round(avg_p, 4),
                      "gpu_launches": int(launches)},
            "plain_fp64": {"value": round(plain_value, 1), "unit": "cell-steps/s", "cell_vertices": len(x0),
                           "workload": "one cell of 2,044 vertices / 3,929 triangles, E 1 kPa, nu 0.45, 0.1 um, 600 "
                                       "integrins (1 pN/nm, rest 20 nm), boundary protruding 10 nm/step, 200 steps",
                           "shape": list(plain_shape),
                           "roofline": plain_roofline,
                           "p50_ms_per_step": round(percentile(pr["per_step"], 0.5), 4),
                           "p99_ms_per_step": round(percentile(pr["per_step"], 0.99), 4),
                           "wall_cell_steps_per_s": round(plain_wall, 1)},
            "ratio_vs_plain_fp64": round(value / world / plain_value, 2),
            "mixed_vs_fp64_rel_displacement_error": max_err, "error_steps": err_steps,
            "accuracy": accuracy,
            "element_assemblies_per_s": round(value / len(cells) * nt_total / world, 1),
            "e2e": e2e, "gpu_launches": int(graph["launches"]), "roofline": roofline, "cpu_baseline": cpu, "serving": serving,
            "newton": newton, "config2": config2,
            "clocks": clocks_info, "pipe_rates": rates,
        }
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if out:
        print(json.dumps(out), flush=True)


SHIFT = (0.5, -0.25, 0.0)   # a rigid in-plane translation: the physics is unchanged, the rounding is not


def mixed_error(cells, device=0, horizons=(20, 300), gate_steps=300, tol=1e-6):
    """Relative displacement error of the mixed form against the FP64 form on the same
    cells: per cell max|x_mixed - x_fp64| / max|x_fp64 - x0|, the max over cells.

    The gate (<= tol) is taken at the workload's own horizon (gate_steps, 300 steps for
    the 256-cell workload), whatever --steps is.  At shorter horizons from rest the
    slowest cells have moved only ~1e-9 um while binary64 positions near 10 um round at
    ~1e-15 um per step, so the FP64 form's own rounding noise is itself ~1e-6 of the
    displacement there.  That noise is measured by stepping the FP64 form once more on
    the rigidly translated cells (x0 + SHIFT: the same physics, other roundings):
    fp64_noise = max|(x_fp64' - SHIFT) - x_fp64| / max|x_fp64 - x0|.  A cell is within
    the FP64 form's noise when its mixed error <= max(tol, 2 fp64_noise)."""
    from wholecellfe_gb300 import capi, synth
    shift = np.asarray(SHIFT)
    hz = sorted(set(horizons) | {gate_steps})
    runs = {}
    for name, prec, sh in (("mixed", capi.PREC_MIXED, 0.0), ("fp64", capi.PREC_FP64, 0.0),
                           ("fp64_shift", capi.PREC_FP64, 1.0)):
        e = capi.Engine(prec, device=device)
        hs = []
        for c in cells:
            x0 = c["x0"] + sh * shift
            h = e.add_cell(x0, c["tri"], c["p"], state=synth.initial_state(x0))
            h.set_integrins(c["rho"])
            hs.append(h)
        done, out = 0, {}
        for n in hz:
            e.step(n - done, DT)
            e.sync()
            done = n
            out[n] = [h.get_state()[0] - sh * shift for h in hs]
        runs[name] = out
        e.close()
    res = {}
    for n in hz:
        em, en, um, within = [], [], [], 0
        for i, c in enumerate(cells):
            xd = runs["fp64"][n][i]
            u = float(np.max(np.abs(xd - c["x0"])))
            a = float(np.max(np.abs(runs["mixed"][n][i] - xd)))
            b = float(np.max(np.abs(runs["fp64_shift"][n][i] - xd)))
            um.append(u)
            em.append(a / u if u > 0 else (0.0 if a == 0 else math.inf))
            en.append(b / u if u > 0 else (0.0 if b == 0 else math.inf))
            within += em[-1] <= max(tol, 2.0 * en[-1])
        res[n] = {"steps": n, "max_rel_displacement_error": max(em), "median_rel_displacement_error": float(np.median(em)),
                  "fp64_noise_max": max(en), "fp64_noise_median": float(np.median(en)),
                  "min_displacement_um": min(um), "cells_within_fp64_noise": f"{within}/{len(cells)}"}
    gate = dict(res[gate_steps])
    gate["tol"] = tol
    gate["pass"] = gate["max_rel_displacement_error"] <= tol
    return {"gate": gate, "horizons": [res[n] for n in hz if n != gate_steps],
            "definition": "per cell max|x_mixed - x_fp64| / max|x_fp64 - x0|, max over cells; fp64_noise: the FP64 "
                          f"form on the cells translated by {list(SHIFT)} um against the untranslated run"}


def run_serving(seconds: float = 10.0, rate: float = 200.0, budget_gb: float = 16.0, seed: int = 7,
                saturate: int = 0):
    """Config 5, bounded: Poisson arrivals (rate per second) of cell simulations with 1k-50k
    vertices (log-uniform), 50-2000 steps (uniform) and a random stiffness model, admitted by
    an HBM budget into one mixed-precision engine (wcfe_server_*).  Arrivals stop after
    `seconds`; the loop then drains.  saturate > 0 instead submits that many requests at
    once (the offered load far above capacity, the budget binding), so that the measured
    rate is the serving form's capacity.  Meshes come from a pool of 24 seeded disks."""
    import ctypes as C
    from wholecellfe_gb300 import capi, synth
    from wholecellfe_gb300.params import default_params
    L = capi.load()
    rng = np.random.default_rng(seed)
    pool = []
    for i in range(24):
        n = int(round(math.exp(rng.uniform(math.log(1000), math.log(50000)))))
        x0, tri = synth.disk_mesh(n, seed=9000 + i)
        pool.append((np.ascontiguousarray(x0), np.ascontiguousarray(tri, np.int32)))
    params = []
    for law in range(3):
        p = default_params("k31" if law else "k1")
        if law == 2:
            p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
        params.append(p)
    eng = capi.Engine(capi.PREC_MIXED, budget_bytes=int(budget_gb * 2**30))
    srv = C.c_void_p()
    capi.check(L.wcfe_server_create(eng.h, DT, C.byref(srv)), "wcfe_server_create")
    ids, steps_of, nv_of = [], [], []

    def submit():
        x0, tri = pool[int(rng.integers(0, len(pool)))]
        p = params[int(rng.integers(0, 3))]
        steps = int(rng.integers(50, 2001))
        rq = capi.Request(len(x0), len(tri), capi.ip(tri), capi.dp(x0), C.pointer(p), steps, None, None, 0, 0)
        rid = C.c_int64()
        capi.check(L.wcfe_server_submit(srv, C.byref(rq), C.byref(rid)), "wcfe_server_submit")
        ids.append(rid.value)
        steps_of.append(steps)
        nv_of.append(len(x0))

    t0 = time.perf_counter()
    if saturate:
        for _ in range(saturate):
            submit()
    next_arrival = rng.exponential(1.0 / rate)
    na, nq = C.c_int32(), C.c_int32()
    active_hist = []
    while True:
        now = time.perf_counter() - t0
        while not saturate and next_arrival <= now and next_arrival < seconds:
            submit()
            next_arrival += rng.exponential(1.0 / rate)
        capi.check(L.wcfe_server_iterate(srv, C.byref(na), C.byref(nq)), "wcfe_server_iterate")
        active_hist.append(na.value)
        if (saturate or now >= seconds) and na.value == 0 and nq.value == 0:
            break
        if now > (0 if saturate else seconds) + 300:   # drain bound
            break
        if na.value == 0 and not saturate:
            time.sleep(0.0005)
    wall = time.perf_counter() - t0
    n = L.wcfe_server_step_times(srv, None, 0)
    buf = (C.c_double * max(n, 1))()
    L.wcfe_server_step_times(srv, buf, n)
    it_ms = [b * 1e3 for b in list(buf)[:n]]
    lat = []
    done_steps = 0
    for rid, st in zip(ids, steps_of):
        t = C.c_double()
        if L.wcfe_server_result(srv, rid, None, C.byref(t)) == 0:
            lat.append(t.value)
            done_steps += st
    L.wcfe_server_destroy(srv)
    used_peak = max(active_hist) if active_hist else 0
    eng.close()
    out = {"requests": len(ids), "completed": len(lat),
           "vertices_per_request": "log-uniform [1000, 50000] (pool of 24 meshes)", "steps_per_request": "uniform [50, 2000]",
           "hbm_budget_gb": budget_gb, "wall_s": round(wall, 2),
           "cell_steps_per_s": round(done_steps / wall, 1),
           "p50_step_ms": round(percentile(it_ms, 0.5), 4) if it_ms else None,
           "p99_step_ms": round(percentile(it_ms, 0.99), 4) if it_ms else None,
           "p50_request_s": round(percentile(lat, 0.5), 3) if lat else None,
           "p99_request_s": round(percentile(lat, 0.99), 3) if lat else None,
           "max_resident_cells": used_peak}
    if saturate:
        out["arrivals"] = f"{saturate} requests submitted at once (offered load above capacity)"
    else:
        out.update({"arrival_rate_per_s": rate, "arrival_seconds": seconds,
                    "offered_cell_steps_per_s": round(sum(steps_of) / max(seconds, 1e-9), 1)})
    return out


def run_config2(steps: int = 500, seed: int = 2):
    """Config 2: one 20,000-vertex cell, 8,000 integrins with k(x) = k0 (1 + (x/x0)^2), k0 = 31 pN/nm,
    x0 = 5 nm, shear modulus log-normal per element (median mu, sigma 0.3), 500 steps, in the FP64
    form and in the mixed form with the FP32 element and with the float-float element; device
    time per step of each and each mixed run's relative displacement error against the FP64
    form."""
    import torch
    from wholecellfe_gb300 import capi, synth
    from wholecellfe_gb300.params import default_params
    rng = np.random.default_rng(seed)
    x0, tri = synth.disk_mesh(20000, seed=seed)
    p = default_params("k31")
    p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
    rho = np.zeros(len(x0))
    rho[rng.choice(len(x0), size=8000, replace=False)] = p.rho_i_max
    mu = p.mu * np.exp(0.3 * rng.standard_normal(len(tri)))
    out = {}
    for name, prec, ff in (("fp64", capi.PREC_FP64, 0), ("mixed", capi.PREC_MIXED, 0),
                           ("mixed_ff", capi.PREC_MIXED, 1)):
        eng = capi.Engine(prec)
        if ff:
            eng.set_element_precision(1)
        h = eng.add_cell(x0, tri, p, state=synth.initial_state(x0))
        h.set_integrins(rho)
        h.set_element_mu(mu)
        eng.autotune(DT, 3)
        r = timed_steps(eng, steps, DT)
        out[name] = (h.get_state()[0], r["total_ms"] / steps, h.status())
        eng.close()
    u = out["fp64"][0] - x0
    err = float(np.max(np.abs(out["mixed"][0] - out["fp64"][0])) / np.max(np.abs(u)))
    err_ff = float(np.max(np.abs(out["mixed_ff"][0] - out["fp64"][0])) / np.max(np.abs(u)))
    return {"vertices": len(x0), "triangles": len(tri), "integrins": 8000, "steps": steps,
            "fp64_ms_per_step": round(out["fp64"][1], 4), "mixed_ms_per_step": round(out["mixed"][1], 4),
            "mixed_vs_fp64_rel_displacement_error": err, "within_1e-6": bool(err <= 1e-6),
            "mixed_ff_element": {"ms_per_step": round(out["mixed_ff"][1], 4),
                                 "rel_displacement_error": err_ff, "within_1e-6": bool(err_ff <= 1e-6),
                                 "note": "the mixed form with the float-float element "
                                         "(wcfe_engine_set_element_precision 1)"},
            "status": [out["fp64"][2], out["mixed"][2], out["mixed_ff"][2]]}


def lu_roofline(tflops, outer_block=512, tf32_peak=None):
    """The LU's rate against the TF32 tensor rate measured on this GPU by
    wcfe_debug_pipe_rates (tcgen05 MMAs of the LU's shape from resident operands); without
    it, half the measured bf16 GEMM rate."""
    if tf32_peak and tf32_peak > 0:
        peak, src = tf32_peak, "measured TF32 tcgen05 rate of this GPU (wcfe_debug_pipe_rates, M 128 N 256)"
    else:
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except (OSError, ValueError):
            peaks = {}
        bf16 = peaks.get("bf16_tflops_sustained")
        src = "MEASURED_PEAKS.json bf16_tflops_sustained / 2"
        if bf16 is None:
            bf16, src = 1700.0, "fallback 1700 TFLOP/s bf16 sustained / 2"
        peak = bf16 / 2.0
    return {"bound": "tensor", "achieved": tflops, "peak": round(peak, 1), "unit": "TFLOP/s",
            "frac": round(tflops / peak, 4) if tflops else None, "peak_source": src,
            "note": "TF32 flops 2/3 (2N)^3 per factorisation over the LU's device time; "
                    f"a trailing update moves 8 B of the matrix per 2 K flops (K = {outer_block})"}


def cpu_lu_baseline(sizes, budget_s: float = 12.0):
    """FP64 LU (LAPACK dgetrf through scipy.linalg.lu_factor, all host threads) of the
    workload's 2N x 2N matrices, cell by cell until the time budget is spent: the CPU
    counterpart of the implicit step's factorisation.  Diagonally dominant random matrices
    of the cells' sizes (dgetrf's time does not depend on the values)."""
    try:
        import scipy.linalg as sla
    except ImportError as ex:
        return {"unavailable": f"scipy: {ex}"}
    rng = np.random.default_rng(5)
    done, secs, flops = 0, 0.0, 0.0
    for n in sizes:
        m = 2 * int(n)
        A = rng.standard_normal((m, m)) + m * np.eye(m)
        A = np.asfortranarray(A)
        t0 = time.perf_counter()
        sla.lu_factor(A, overwrite_a=True, check_finite=False)
        secs += time.perf_counter() - t0
        flops += 2.0 / 3.0 * m ** 3
        done += 1
        if secs > budget_s:
            break
    return {"kind": "scipy.linalg.lu_factor (LAPACK dgetrf, FP64, partial pivoting)", "cores": os.cpu_count(),
            "sample": f"the first {done} of the workload's {len(sizes)} matrices (2N = {2 * min(sizes[:done])}"
                      f"-{2 * max(sizes[:done])})",
            "lu_per_s": round(done / secs, 3), "tflop_per_s": round(flops / secs / 1e12, 4)}


def run_newton(ncells: int = 64, steps: int = 2, seed: int = 4, lu=(1024, 0), tf32_peak=None):
    """Config 4, bounded: implicit (Newton) steps of `ncells` cells with 1000-4000 vertices
    (uniform), dense 2N x 2N tangents, LU with TF32 tensor-core trailing updates, FP64
    residual and refinement to 1e-10.  Reports cell-steps/s, Newton iterations, the
    residuals reached and the LU's FLOP rate over the timed steps."""
    import torch
    from wholecellfe_gb300 import capi, synth
    from wholecellfe_gb300.params import default_params
    rng = np.random.default_rng(seed)
    eng = capi.Engine(capi.PREC_FP64)
    eng.set_lu(*lu)
    sizes = []
    for i in range(ncells):
        n = int(rng.integers(1000, 4001))
        x0, tri = synth.disk_mesh(n, seed=7000 + i)
        p = default_params(["k1", "k31", "k31"][i % 3])
        if i % 3 == 2:
            p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
        p.stream = i
        eng.add_cell(x0, tri, p, state=synth.initial_state(x0))
        sizes.append(len(x0))
    eng.step_implicit(1, DT, rtol=1e-10, max_newton=8)   # warm-up (and first allocations)
    eng.sync()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = eng.step_implicit(steps, DT, rtol=1e-10, max_newton=8)
    eng.sync()
    wall = time.perf_counter() - t0
    eng.close()
    iters = st["newton_iters"]   # Newton updates over the timed steps (all cells in lockstep)
    return {"cells": ncells, "vertices": "uniform [1000, 4000]", "steps": steps,
            "lu": {"outer_block": lu[0], "updates": ["tcgen05", "mma.sync"][lu[1]]},
            "cell_steps_per_s": round(ncells * steps / wall, 2), "ms_per_step": round(wall / steps * 1e3, 2),
            "newton_iters_per_step": iters / steps, "max_refine_passes": st["max_refine_iters"],
            "max_rel_residual": st["max_rel_residual"], "max_refine_rel_residual": st["max_refine_rel_residual"],
            "unconverged_cell_steps": st["unconverged"], "rounding_floor_exits": st["floor_exits"],
            "lu_ms_per_step": round(st["lu_ms"] / steps, 2),
            "lu_tflop_per_s": round(st["lu_gflop"] / st["lu_ms"], 2) if st["lu_ms"] > 0 else None,
            "lu_share_of_step": round(st["lu_ms"] / (wall * 1e3), 3),
            "lu_roofline": lu_roofline(st["lu_gflop"] / st["lu_ms"] if st["lu_ms"] > 0 else None, lu[0], tf32_peak),
            "solve_ms_per_step": round(st["solve_ms"] / steps, 2),
            "cpu_lu_baseline": cpu_lu_baseline(sizes),
            "timing": "host wall clock around wcfe_engine_step_implicit (it synchronises per Newton iteration); "
                      "LU: CUDA events around each factorisation, TF32 flops 2/3 (2N)^3 per factored cell"}


def run_phase(args):
    """One timed loop only, for profiling: the batched mixed or FP64 form on the workload
    (--cells of them), or the plain one-cell FP64 form."""
    import torch
    from wholecellfe_gb300 import capi, synth
    from wholecellfe_gb300.params import default_params
    torch.cuda.init()
    if args.phase == "config2":
        print(json.dumps(run_config2(max(1, min(args.steps, 500)))))
        return
    if args.phase == "serve":
        pois = run_serving(args.serve_seconds) if args.serve_seconds > 0 else None
        sat = run_serving(saturate=args.serve_saturate, budget_gb=4.0, seed=8) if args.serve_saturate > 0 else None
        print(json.dumps({"poisson": pois, "saturated": sat}))
        return
    if args.phase == "newton":
        lu = tuple(int(v) for v in args.lu.split(","))
        print(json.dumps(run_newton(args.cells if args.cells != N_CELLS else 64, max(1, min(args.steps, 5)), lu=lu)))
        return
    if args.phase == "plain":
        x0, tri, p, rho = synth.protruding_cell(dt=DT)
        eng = capi.Engine(capi.PREC_FP64)
        eng.add_cell(x0, tri, p, state=synth.initial_state(x0)).set_integrins(rho)
        ncells = 1
    else:
        cells = make_workload(seed=1000, ncells=args.cells)
        eng = capi.Engine(capi.PREC_MIXED if args.phase == "mixed" else capi.PREC_FP64)
        if args.phase == "mixed":
            eng.set_patch_kernel(args.patch_kernel)
            eng.set_vertex_kernel(args.vertex_kernel)
            eng.set_fused(bool(args.fused))
            eng.set_element_precision(args.element_ff)
        if args.shape:
            t, e_ = (int(x) for x in args.shape.split(","))
            eng.set_shape(t, e_)
        load_cells(eng, cells)
        ncells = len(cells)
    for _ in range(args.warmup):
        eng.step(1, DT)
    r = timed_steps(eng, args.steps, DT)
    thr, emax = eng.shape()
    print(json.dumps({"phase": args.phase, "cells": ncells, "ms_per_step": r["total_ms"] / args.steps,
                      "vertex_ms": r["ms_v"] / args.steps, "patch_ms": r["ms_p"] / args.steps,
                      "cell_steps_per_s": ncells * args.steps / (r["total_ms"] / 1e3), "shape": [thr, emax],
                      "patch_kernel": args.patch_kernel, "vertex_kernel": args.vertex_kernel,
                      "fused": eng.fused(), "element_ff": args.element_ff}))
    eng.close()


def workload_config(cells):
    """The workload keys of `config`, shared by both arms (the same seeded population)."""
    return {"workload": f"{len(cells)} uneven cells per GPU, vertices log-uniform [500, 20000], "
                        "integrins 0.4 x vertices, stiffness {linear 1, linear 31, poly 31 pN/nm x0 5 nm}, "
                        "flat rigid substrate, dt 5e-5 s, explicit step A1-A9",
            "cells": len(cells), "vertices": int(sum(len(c["x0"]) for c in cells)),
            "triangles": int(sum(len(c["tri"]) for c in cells))}


def run_reference(args):
    """The reference's CPU implementation of the step (the oracle port; the reference's own
    sources are not on this machine) on all host cores, bounded sample of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle_py as O
    from wholecellfe_gb300 import synth
    cells = make_workload(seed=1000, ncells=args.cells)
    nthreads = os.cpu_count() or 1
    if O.ref_available("k1") and O.ref_available("k31"):
        return run_reference_build(args, cells, nthreads)
    # one timed "step" = every sampled cell advanced by a few explicit steps, sized to finish in minutes
    sample = cells[:max(nthreads, 32)]
    ocs = [O.OCell(O.OMesh(c["tri"], len(c["x0"])), synth.initial_state(c["x0"]), c["p"], rho_w=c["rho"])
           for c in sample]
    per = 2
    for _ in range(min(args.warmup, 1)):
        O.cells_steps_mt(ocs, 1, DT, nthreads)
    times = []
    steps = min(args.steps, 10)
    for _ in range(steps):
        t0 = time.perf_counter()
        O.cells_steps_mt(ocs, per, DT, nthreads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = len(sample) * per * steps / tot
    cpu = {"value": round(value, 1), "unit": "cell-steps/s", "cores": nthreads, "kind": "port",
           "sample": f"{len(sample)} of the {len(cells)} workload cells x {per} explicit steps per timed step, "
                     f"{steps} timed steps, oracle/wcfe_oracle.c (C port of cellBP/UL_growth_explicit.cpp)"}
    out = {"metric": METRIC, "value": round(value, 1), "unit": "cell-steps/s", "n_gpus": 0, "steps": steps,
           "warmup": args.warmup, "ms_per_step": round(tot / steps * 1e3, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
           "config": {**workload_config(cells), "cells_sampled": len(sample)},
           "impl": "reference", "cpu_baseline": cpu,
           "e2e": {"value": round(value, 1), "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "p50_ms_per_step": round(percentile(times, 0.5) * 1e3, 3),
           "p99_ms_per_step": round(percentile(times, 0.99) * 1e3, 3)}
    print(json.dumps(out), flush=True)


def run_reference_build(args, cells, nprocs):
    """--impl reference where the reference was built from its sources (oracle/_ref): its own
    step loop, one process per host core, on the workload's linear-law cells."""
    import multiprocessing as mp
    lin = [c for c in cells if c["model"] in (0, 1)]
    sample = lin[:max(nprocs, 32)]
    per = 2
    jobs = [(sample[i::nprocs], per) for i in range(nprocs) if sample[i::nprocs]]
    times = []
    steps = min(args.steps, 10)
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        for _ in range(min(args.warmup, 1)):
            pool.map(_ref_worker, jobs)
        for _ in range(steps):
            t0 = time.perf_counter()
            pool.map(_ref_worker, jobs)
            times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = len(sample) * per * steps / tot
    cpu = {"value": round(value, 1), "unit": "cell-steps/s", "cores": len(jobs), "kind": "reference",
           "sample": f"{len(sample)} linear-law cells of the {len(cells)} workload cells x {per} explicit steps per "
                     f"timed step, {steps} timed steps, the reference's UL_growth_explicit.cpp built from its sources "
                     f"(oracle/_ref), {len(jobs)} processes"}
    out = {"metric": METRIC, "value": round(value, 1), "unit": "cell-steps/s", "n_gpus": 0, "steps": steps,
           "warmup": args.warmup, "ms_per_step": round(tot / steps * 1e3, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
           "config": {**workload_config(cells), "cells_sampled": len(sample)},
           "impl": "reference", "cpu_baseline": cpu,
           "e2e": {"value": round(value, 1), "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "p50_ms_per_step": round(percentile(times, 0.5) * 1e3, 3),
           "p99_ms_per_step": round(percentile(times, 0.99) * 1e3, 3)}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=N_CELLS)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="length of the Poisson arrival window of the serving measurement (0: skip)")
    ap.add_argument("--serve-saturate", type=int, default=1000,
                    help="requests submitted at once for the serving capacity measurement")
    ap.add_argument("--phase", default="all", choices=["all", "mixed", "fp64", "plain", "newton", "config2", "serve"],
                    help="profiling aid: run only one timed loop (default shape, no autotune) and print its timing")
    ap.add_argument("--lu", default="1024,0", help="--phase newton: LU outer block and kind (0 tcgen05, 1 mma.sync)")
    ap.add_argument("--newton-cells", type=int, default=512,
                    help="cells of the bounded implicit-step (Newton, dense LU) measurement (0: skip)")
    ap.add_argument("--shape", default="", help="with --phase: patch threads,elements (default: the engine's)")
    ap.add_argument("--patch-kernel", type=int, default=1, choices=[0, 1, 2, 3, 4],
                    help="with --phase mixed: 0 staged patch kernel, 1 plain (default), 2-4 plain with registers "
                         "capped for 6-8 CTAs per SM")
    ap.add_argument("--vertex-kernel", type=int, default=0, choices=[0, 1, 2, 3],
                    help="with --phase mixed: vertex kernel for 5, 4, 6 or 8 blocks per SM")
    ap.add_argument("--element-ff", type=int, default=0, choices=[0, 1],
                    help="--phase mixed: 1 = the float-float element (wcfe_engine_set_element_precision)")
    ap.add_argument("--fused", type=int, default=0, choices=[0, 1],
                    help="with --phase mixed: fold each next vertex phase into the patch phase (default 0)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    from oracle import oracle_py
    oracle_py.build()
    if args.impl == "reference":
        run_reference(args)
    elif args.phase != "all":
        run_phase(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
