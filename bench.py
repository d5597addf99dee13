"""Benchmark of the ECSPRT per-timestep hot path on GB300.

Workload (N=1): 128^3 periodic grid, dx = 1 (normalised), 64 ions per cell
(134,217,728 ions), initial density 1 + 0.05 sin(2 pi x / Lx), Maxwellian ions
(per-component thermal speed 1) drifting at 1.0 along x, B along z with ion
gyrofrequency 0.1, ion-neutral collision frequency 0.02 (Maxwellian neutrals
at the ion temperature), kappa_e ~ 2, dt = 0.1, variable-coefficient
potential solve to 1e-8 relative residual.  Mixed path: FP32 cell-sorted
particles (sorted every 2 steps), FP32 multigrid-FGMRES inside FP64
iterative refinement.  Synthetic seeded data (no dataset exists for this
benchmark).

A step is one pass of src/pic.c:244-258: push + collide + move/BC + deposit
+ RHS + operator set-up + solve.  value = ions x steps / device time of the
timed steps (ion records resident in HBM, 8.6 GB >> L2, so no flush is needed).
e2e = the same metric through the host-buffer C-ABI call ecs_step_host
(particles copied in and out of pinned host memory every step, plus the
moments and potential out).

"serving" reports the request loop (include/ecs_serve.h) on its two
workloads: stand-alone solves (Poisson arrivals at 200/s, grids uniform over
{32,48,64,96,128}^3, lognormal x Fourier-mode densities, 40 GB HBM budget,
latency p50/p99 from submit to result, plus the saturated solve rate of a
burst), and an ensemble of 48 small simulations ({32,48,64}^3, 16 ions/cell,
500 steps each, per-step p50/p99).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os

# The request loop overlaps up to SERVE_INFLIGHT solves on separate streams;
# the device runs that many streams at once only with as many hardware work
# queues (CUDA reads this before its first use in the process).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {
    "name": "128^3 periodic, 64 ions/cell, drift 1.0, nu 0.02, density 1+0.05 sin(2 pi x/Lx)",
    "n": 128, "ppc": 64, "dt": 0.1, "drift": 1.0, "nu": 0.02, "seed": 20261205,
}
SORT_EVERY = 2          # cell sort cadence of the mixed path
# Through host buffers every step moves every ion across the link both ways,
# and the pass is hidden behind those copies.  The step after a sort gathers
# the ions from the old order, so some of its tile ranges wait for upload
# chunks far ahead (ions that crossed a periodic face) and it runs a little
# longer than the others.  The host-buffer run sorts every 4 steps (the
# results do not depend on the cadence) and is timed over eight cycles (32
# steps, about 1.4 s) after two cycles of warm-up, long enough that one
# transient slow-down of the host link (about 100 ms, seen in some runs) does
# not dominate the figure; each cycle's rate is reported beside the whole
# run's.
E2E_SORT_EVERY = 4
E2E_CYCLES = 8
# Algorithmic bytes per particle-step (the roofline's numerator): the ion's
# state read and written once, mixed: int32 cell + 3 FP32 offsets + 3 FP32
# velocities = 28 B each way; FP64: 6 FP64 each way.  The grid fields and the
# counting sort are not counted.
ALGO_BYTES_MIXED = 56
ALGO_BYTES_FP64 = 96
# What the mixed pass moves by design per particle-step: one 32-byte record
# (the 28-byte state padded to a DRAM sector) read + written, and 4 bytes of
# the index sort (the permutation read by the pass after a sort, or the cell
# key written by the counting pass before one; with a sort every 2 steps
# each pass moves one of the two).
RECORD_BYTES_MIXED = 68
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per ion of a
# k_tiles32 step launch, measured by ncu on the 64^3 x 64 ppc case of this
# workload: 66.3 B for a pass that counts cells for the next sort, 70.4 B for
# the pass after a sort (records read through the permutation); the steps
# alternate, so a launch moves their mean x N (the traffic grows with the ion
# count).
TRAFFIC_BYTES_PER_ION = 68.3


def mg_levels(nx, ny, nz):
    """Cells of the multigrid levels: full coarsening while every axis stays
    even and at least 8 (the solver's rule)."""
    out = []
    while True:
        out.append(nx * ny * nz)
        flat = nz == 1
        even = nx % 2 == 0 and ny % 2 == 0 and (flat or nz % 2 == 0)
        if not even or min(nx, ny, nx if flat else nz) < 8 or len(out) >= 12:
            return out
        nx, ny = nx // 2, ny // 2
        if not flat:
            nz //= 2


# Algorithmic bytes of the field phase (RHS, operator set-up, solve), by the
# rule 12 B a cell for an FP32 operator or smoother application and 24 B for
# an FP64 one (read the iterate and the density, write the result), 4 B (FP32)
# or 8 B (FP64) a cell for every other vector read or written; each level at
# its own cell count.
B_OP32, B_OP64, B_V32, B_V64 = 12, 24, 4, 8


def field_phase_bytes(levels, iterations, refinements):
    """Bytes of one field phase of the mixed path with `iterations` FGMRES
    steps in `refinements` FP64 refinement sweeps (the steps taken as evenly
    spread over the sweeps' cycles)."""
    n0 = levels[0]
    rhs = 4 * B_V64 * n0 + B_V64 * n0 + 2 * B_V64 * n0  # moments in, b out; mean removal (read, write)
    setup = (B_V64 + B_V32) * n0  # FP64 density -> FP32
    for i, n in enumerate(levels):
        if i:
            setup += B_V32 * (levels[i - 1] + n)  # full-weighting restriction of the density
        setup += B_V32 * n * (1 + 2 + 2 + 6)  # z-line rows (density in, 2 out), factors (2 in, 6 out)
    vcycle = 0
    for i, n in enumerate(levels[:-1]):
        vcycle += 2 * B_OP32 * n + 2 * B_OP32 * n  # pre- and post-smoothing, residual, post-smoothing RHS
        vcycle += B_V32 * (3 * n + 2 * levels[i + 1])  # restriction (read r, write b), prolongation (x in, t rw)
    vcycle += B_V32 * levels[-1] * (levels[-1] + 2)  # coarsest: explicit inverse times b
    k = iterations / max(refinements, 1)
    steps = 0.0
    j = 0.0
    while j < k:  # Arnoldi step j: V-cycle, mean, operator, two Gram-Schmidt passes
        frac = min(1.0, k - j)
        steps += frac * (vcycle + B_V32 * n0 + B_OP32 * n0 + 2 * B_V32 * n0 + (3 * j + 9) * B_V32 * n0)
        j += 1.0
    cycle = B_V32 * n0 * 5 + B_V32 * n0 * (k + 1)  # ||b||, start vectors; x = Z y
    sweep = (B_OP64 + 2 * B_V64) * n0 + B_V64 * n0 + (B_V64 + B_V32) * n0 + (B_V32 + 2 * B_V64) * n0 + \
        3 * B_V64 * n0  # FP64 residual, norm, scale to FP32, phi += e, mean projection
    return rhs + setup + refinements * (cycle + sweep) + refinements * steps


def options(w):
    n = w["n"]
    return (f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x {w['drift']} "
            f"-nui {w['nu']} -nue 8.79e9 -Te 11604.5 -E0 0 -Np -{w['ppc']} -dt {w['dt']}")


def make_particles(w, count=None):
    """Seeded synthetic ions: x by rejection on 1 + 0.05 sin(2 pi x/L),
    y, z uniform, Maxwellian velocities plus the drift along x."""
    n = w["n"]
    N = count or n ** 3 * w["ppc"]
    rng = np.random.default_rng(w["seed"])
    L = float(n)
    pos = np.empty((N, 3))
    got = 0
    while got < N:
        m = int((N - got) * 1.06) + 1024
        x = rng.uniform(0.0, L, m)
        keep = x[rng.uniform(0.0, 1.05, m) < 1.0 + 0.05 * np.sin(2 * np.pi * x / L)]
        take = min(keep.size, N - got)
        pos[got:got + take, 0] = keep[:take]
        got += take
    pos[:, 1] = rng.uniform(0.0, L, N)
    pos[:, 2] = rng.uniform(0.0, L, N)
    vel = rng.standard_normal((N, 3))
    vel[:, 0] += w["drift"]
    return pos, vel


def measured_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms, each
    sample stamped with the host clock; summary() keeps the samples taken
    inside the window set by mark() (the timed region)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_first(self, timeout=10.0):
        """Block until the first sample arrives (nvidia-smi start-up)."""
        t_end = time.perf_counter() + timeout
        while self.proc and not self.lines and time.perf_counter() < t_end:
            time.sleep(0.01)

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0, t1 = getattr(self, "window", (float("-inf"), float("inf")))
        inside = [ln for t, ln in self.lines if t0 <= t <= t1]
        if not inside and self.lines:  # region shorter than a sample period: nearest sample
            inside = [min(self.lines, key=lambda x: abs(x[0] - 0.5 * (t0 + t1)))[1]]
        for ln in inside:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(w, pos, vel, phi, seconds_target=20.0):
    """The oracle port of the reference's particle phase (push, collide,
    move + BC, deposit in FP64), timed on the host cores on a bounded sample
    of the same workload; the potential solve is timed separately
    (cpu_solve_baseline)."""
    from oracle import oracle as orc
    import ecsprt_gb300 as E

    orc.build()
    p = E.params_from_options(options(w))
    O = orc.Oracle(p)
    threads = orc.num_threads()
    S = min(pos.shape[0], 1 << 21)
    sp, sv = pos[:S].copy(), vel[:S].copy()
    dt = w["dt"]
    t0 = time.perf_counter()
    steps = 0
    while True:
        sv = O.push(sp, sv, phi, dt)
        sv, _, _ = O.collide(sv, dt)
        sp, sv = O.move(sp, sv, dt)
        O.collect_mt(sp, sv)
        steps += 1
        el = time.perf_counter() - t0
        if el > seconds_target or steps >= 50:
            break
    rate = S * steps / el
    return {"value": rate, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{S} ions of the workload x {steps} steps of push+collide+move+deposit (FP64, "
                      f"{threads} OpenMP threads for push, move and deposit (the deposit split into one z slab "
                      f"a thread, as the reference's ranks split the domain); collide serial as in the "
                      f"reference); the potential solve is timed separately (solve)"}


def cpu_solve_baseline(w, moments):
    """The FP64 potential solve on the host cores, to the workload's 1e-8
    relative residual: the oracle's RHS and variable-coefficient operator
    (OpenMP) in restarted GMRES right-preconditioned by the FFT inverse of
    the mean-density operator (numpy; a stand-in for the reference's PETSc
    GMRES + hypre BoomerAMG, neither of which exists here).  Timed on the
    workload's own moments (the system the GPU solved) and on one density of
    each stand-alone solve size ({32,48,64,96,128}^3, lognormal x Fourier
    modes, flux = density)."""
    from oracle import oracle as orc
    import ecsprt_gb300 as E
    from ecsprt_gb300 import workloads as W

    orc.build()

    def one(p, m):
        O = orc.Oracle(p)
        t0 = time.perf_counter()
        b = O.rhs(m)
        _, its, rel = O.solve_fft(m[..., 0], b, rtol=1e-8)
        return time.perf_counter() - t0, its, rel

    t, its, rel = one(E.params_from_options(options(w)), moments)
    sizes = {}
    rng = np.random.default_rng(20261206)
    for n in W.SOLVE_SIZES:
        dens = W.solve_density(n, rng)
        m = np.zeros(dens.shape + (4,))
        m[..., 0] = dens
        m[..., 1:] = dens[..., None]
        tn, itn, _ = one(E.params_from_options(W.solver_options(n)), m)
        sizes[str(n)] = {"ms": 1e3 * tn, "iterations": itn}
    mix = len(sizes) / sum(v["ms"] * 1e-3 for v in sizes.values())
    return {"kind": "port", "cores": orc.num_threads(),
            "method": "oracle RHS + FP64 GMRES(40), FFT-preconditioned by the mean-density operator, to 1e-8",
            "workload_solve_ms": 1e3 * t, "workload_iterations": its, "workload_relres": rel,
            "solves_per_s": 1.0 / t, "by_size": sizes, "mixed_sizes_solves_per_s": mix}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"  # gloo: host tensors
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def workload_config(w, world):
    n = w["n"]
    return {"workload": w["name"], "grid": [n] * 3, "ions": n ** 3 * w["ppc"], "ppc": w["ppc"], "dt": w["dt"],
            "precision": "mixed (FP32 particles + FP32 MG-FGMRES inside FP64 refinement)",
            "solve_rtol": 1e-8, "sort_every": SORT_EVERY,
            "l2": "inputs larger than L2 (8.6 GB of ion records per step)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def run_reference(args, world, rank):
    """The reference's CPU path (the oracle port) for a whole step of the
    workload on a bounded sample: a 32^3 box at the workload's 64 ions per
    cell (2,097,152 ions) with the same physics, each step push + collide +
    move/BC + deposit + RHS + the FP64 potential solve to 1e-8
    (cpu_solve_baseline's method), the potential carried from step to step."""
    if rank != 0:
        return
    from oracle import oracle as orc
    import ecsprt_gb300 as E

    orc.build()
    w = dict(WORKLOAD, n=32, name=WORKLOAD["name"].replace("128^3", "32^3"))
    pos, vel = make_particles(w)
    S = pos.shape[0]
    p = E.params_from_options(options(w))
    O = orc.Oracle(p)
    dt = w["dt"]
    m = O.collect_mt(pos, vel)
    phi, _, _ = O.solve_fft(m[..., 0], O.rhs(m), rtol=1e-8)

    def step():
        nonlocal pos, vel, phi
        vel = O.push(pos, vel, phi, dt)
        vel, _, _ = O.collide(vel, dt)
        pos, vel = O.move(pos, vel, dt)
        mm = O.collect_mt(pos, vel)
        phi, _, rel = O.solve_fft(mm[..., 0], O.rhs(mm), rtol=1e-8)
        assert rel <= 1e-8

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    value = S * args.steps / el
    threads = orc.num_threads()
    c = {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
         "sample": f"a 32^3 box of the workload at 64 ions/cell ({S} ions), {args.steps} whole steps: push, "
                   f"collide (serial, as the reference), move/BC, deposit ({threads} OpenMP threads), RHS and "
                   f"the FP64 potential solve to 1e-8 (oracle operator, FFT-preconditioned GMRES), the "
                   f"potential carried between steps"}
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(workload_config(WORKLOAD, 1), sample="32^3 x 64 ions/cell", sample_ions=S,
                       precision="FP64 (the reference's CPU path, restated by the oracle)"),
        "cpu_baseline": c,
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


SERVE_BUDGET = 40 << 30
SERVE_INFLIGHT = 16


def _size_percentiles(res, sizes):
    by = {}
    for r in res:
        by.setdefault(sizes[r["id"]], []).append(r["latency"])
    return {str(n): {"count": len(v), "p50_ms": 1e3 * float(np.percentile(v, 50)),
                     "p99_ms": 1e3 * float(np.percentile(v, 99))} for n, v in sorted(by.items())}


def run_serve_solves(E, W, nreq, rate=200.0, seed=20261206):
    """Open-loop stand-alone solve load, then a saturated burst."""
    rng = np.random.default_rng(seed)
    params = {n: E.params_from_options(W.solver_options(n)) for n in W.SOLVE_SIZES}
    pool = 4  # seeded densities per grid size, cycled (each request does the full work)
    dens = {}
    for n in W.SOLVE_SIZES:
        dens[n] = []
        for _ in range(pool):
            d = E.pinned_empty((n,) * 3)
            d[:] = W.solve_density(n, rng)
            dens[n].append(d)
    free = {n: [] for n in W.SOLVE_SIZES}

    def out_buf(n):
        return free[n].pop() if free[n] else E.pinned_empty((n,) * 3)

    t_arr, sz = W.solve_requests(nreq, rate, seed + 1)
    with E.Server(hbm_budget_bytes=SERVE_BUDGET, max_inflight=SERVE_INFLIGHT) as srv:
        held = {}

        def collect(rs, sizes_of):
            for r in rs:
                n, o = held.pop(r["id"])
                free[n].append(o)
                sizes_of[r["id"]] = n
            return rs

        warm_sizes = {}
        for n in W.SOLVE_SIZES:  # one request per size builds the slots' graphs
            o = out_buf(n)
            rid = srv.submit_solve(params[n], dens[n][0], o)
            held[rid] = (n, o)
        collect(srv.wait_all(120), warm_sizes)
        srv.reset_stats()
        sizes_of = {}
        res = []
        t0 = time.perf_counter()
        for q in range(nreq):
            n = int(sz[q])
            while True:
                wait = t_arr[q] - (time.perf_counter() - t0)
                if wait <= 0:
                    break
                res += collect(srv.poll(256, 0), sizes_of)
                time.sleep(min(wait, 2e-4))
            o = out_buf(n)
            rid = srv.submit_solve(params[n], dens[n][q % pool], o)
            held[rid] = (n, o)
        res += collect(srv.wait_all(600), sizes_of)
        wall = time.perf_counter() - t0
        st = srv.stats()
        bad = [r for r in res if r["status"] != 0]
        open_loop = {
            "requests": nreq, "arrival_rate_per_s": rate, "wall_s": wall, "solves_per_s": len(res) / wall,
            "p50_ms": 1e3 * st["solve_p50"], "p99_ms": 1e3 * st["solve_p99"],
            "p99_over_p50": st["solve_p99"] / st["solve_p50"] if st["solve_p50"] > 0 else None,
            "mean_ms": 1e3 * st["solve_mean"], "max_ms": 1e3 * st["solve_max"],
            "max_relres": max(r["relres"] for r in res), "failed": len(bad),
            "mean_iterations": float(np.mean([r["iterations"] for r in res])),
            "by_size": _size_percentiles(res, sizes_of),
            "peak_inflight": st["peak_inflight"], "peak_device_bytes": st["peak_device_bytes"],
            "slot_hits": st["slot_hits"], "slots_created": st["slots_created"],
            "busy_fraction": st["busy_seconds"] / wall, "gpu_launches": st["gpu_launches"],
        }
        # saturated: a burst of requests all queued at once
        srv.reset_stats()
        nb = min(2000, nreq)
        sizes_b = {}
        t0 = time.perf_counter()
        for q in range(nb):
            n = int(sz[q])
            o = out_buf(n)
            rid = srv.submit_solve(params[n], dens[n][q % pool], o)
            held[rid] = (n, o)
        rb = collect(srv.wait_all(600), sizes_b)
        wall_b = time.perf_counter() - t0
        stb = srv.stats()
        saturated = {"requests": nb, "wall_s": wall_b, "solves_per_s": nb / wall_b,
                     "failed": sum(r["status"] != 0 for r in rb), "peak_inflight": stb["peak_inflight"],
                     "gpu_launches": stb["gpu_launches"]}
    return {"workload": "stand-alone solves: grids uniform over {32,48,64,96,128}^3, density lognormal(0,0.1) x "
                        "(1 + 12 Fourier modes of amplitude 0.05), FP32 MG-FGMRES + FP64 refinement to 1e-8",
            "data": f"synthetic, {pool} seeded densities per size cycled",
            "hbm_budget_bytes": SERVE_BUDGET, "max_inflight": SERVE_INFLIGHT,
            "open_loop": open_loop, "saturated": saturated}


def run_serve_sims(E, W, ninst, nsteps, seed=20261207):
    """Ensemble of small simulations stepped concurrently."""
    inst = W.sim_instances(ninst, seed)
    rng = np.random.default_rng(seed + 1)
    ppc = 16
    reqs = []
    for n, drift, nu in inst:
        p = E.params_from_options(W.sim_options(n, ppc, drift, nu))
        pos, vel = W.uniform_ions(n, ppc, drift, rng)
        reqs.append((p, pos, vel, np.zeros(nsteps)))
    ions = sum(r[1].shape[0] for r in reqs)
    with E.Server(hbm_budget_bytes=SERVE_BUDGET, max_inflight=SERVE_INFLIGHT) as srv:
        t0 = time.perf_counter()
        for q, (p, pos, vel, secs) in enumerate(reqs):
            srv.submit_sim(p, pos, vel, nsteps, 0.1, seed=1000 + q, step_seconds=secs)
        res = srv.wait_all(1800)
        wall = time.perf_counter() - t0
        st = srv.stats()
    steps = np.concatenate([r[3] for r in reqs])
    return {"workload": f"{ninst} simulations, grids uniform over {{32,48,64}}^3, {ppc} ions/cell, drift U[0.2,1.5], "
                        f"collision frequency log-U[0.005,0.1], {nsteps} steps each, mixed precision",
            "data": "synthetic, seeded", "instances": ninst, "steps_each": nsteps, "ions": ions,
            "wall_s": wall, "particle_steps_per_s": ions * nsteps / wall,
            "step_p50_ms": 1e3 * float(np.percentile(steps, 50)), "step_p99_ms": 1e3 * float(np.percentile(steps, 99)),
            "failed": sum(r["status"] != 0 for r in res), "peak_inflight": st["peak_inflight"],
            "peak_device_bytes": st["peak_device_bytes"], "gpu_launches": st["gpu_launches"],
            "hbm_budget_bytes": SERVE_BUDGET, "max_inflight": SERVE_INFLIGHT}


def _timed_steps(ctx, stream, n_ions, steps, warmup, dt, rtol=1e-8):
    import torch

    for _ in range(warmup):
        ctx.step(dt, rtol, 400)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    st = [ctx.step(dt, rtol, 400) for _ in range(steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    el = e0.elapsed_time(e1) * 1e-3
    return {"value": n_ions * steps / el, "unit": "particle-steps/s", "ms_per_step": 1e3 * el / steps,
            "steps": steps, "warmup": warmup,
            "particle_ms": 1e3 * float(np.mean([s.particle_seconds for s in st])),
            "field_ms": 1e3 * float(np.mean([s.solve.seconds for s in st])),
            "iterations": [s.solve.iterations for s in st], "max_relres": max(s.solve.relres for s in st),
            "collisions_per_step": float(np.mean([s.collisions for s in st]))}


def run_c1(E, stream, args):
    """32^3 periodic, 16 ions/cell (524,288), drift 0.5, nu 0.05, dt 0.1, the
    reference's Sobol positions and Maxwellian velocities (generated on the
    device), solve to 1e-8: the plain FP64 path and the mixed path."""
    n = 32
    p = E.params_from_options(f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 "
                              f"-vi0x 0.5 -nui 0.05 -nue 8.79e9 -Te 11604.5 -E0 0")
    N = 16 * n ** 3
    out = {"workload": "32^3 periodic, 16 ions/cell (524,288 ions), drift 0.5, nu 0.05, Sobol positions, dt 0.1"}
    for name, prec in (("fp64", E.ECS_PREC_FP64), ("mixed", E.ECS_PREC_MIXED)):
        with E.Context(p, prec, np_capacity=N, stream=stream.cuda_stream) as ctx:
            ctx.init_particles(E.ECS_INIT_SOBOL, N, seed=20261203)
            ctx.collect()
            ctx.compute_potential(rtol=1e-8, max_it=400)
            out[name] = _timed_steps(ctx, stream, N, max(args.steps, 20), max(args.warmup, 3), 0.1)
    return out


def run_c3(E, stream, args):
    """256 x 256 x 128, periodic x/y, reflecting z, 32 ions/cell
    (268,435,456 ions), density 1 + 8 Fourier modes of amplitude 0.02,
    drift 0.5, nu 0.02, mixed precision, cell sort every 4 steps, solve to
    1e-8."""
    from ecsprt_gb300 import workloads as W

    p = E.params_from_options("-Nx 256 -Ny 256 -Nz 128 -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 0.5 "
                              "-nui 0.02 -nue 8.79e9 -Te 11604.5 -E0 0 -zBC inject-reflect")
    N = 256 * 256 * 128 * 32
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=N, stream=stream.cuda_stream) as ctx:
        ctx.set_sort_every(4)
        ctx.init_particles(E.ECS_INIT_MODES, N, seed=W.C3_SEED, modes=W.c3_modes())
        ctx.collect()
        ctx.compute_potential(rtol=1e-8, max_it=400)
        r = _timed_steps(ctx, stream, N, max(args.steps, 8), max(args.warmup, 3), 0.1)
    r["workload"] = ("256x256x128, periodic x/y, reflecting z, 32 ions/cell (268,435,456 ions), density 1 + 8 "
                     "Fourier modes (0.02), drift 0.5, nu 0.02, sort every 4, mixed")
    return r


def run_ours(args, world, rank, local):
    import torch

    import ecsprt_gb300 as E

    w = WORKLOAD
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    p = E.params_from_options(options(w))
    pos, vel = make_particles(w)
    N = pos.shape[0]
    dt = w["dt"]
    rtol = 1e-8

    # ---------------- device-resident mixed path -----------------------
    ctx = E.Context(p, E.ECS_PREC_MIXED, np_capacity=N, stream=stream.cuda_stream)
    ctx.set_sort_every(SORT_EVERY)
    if args.no_solver_graphs:
        ctx.set_solver_graphs(False)
    ctx.upload_particles(pos, vel)
    ctx.collect()
    ctx.compute_potential(rtol=rtol, max_it=400)
    for _ in range(args.warmup):
        ctx.step(dt, rtol, 400)
    stats = []
    launches0 = ctx.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        clk.wait_first()
        barrier(world)
        torch.cuda.synchronize()
        t_host0 = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            stats.append(ctx.step(dt, rtol, 400))
        e1.record(stream)
        torch.cuda.synchronize()
        clk.mark(t_host0, time.perf_counter())
    launches = ctx.launches - launches0
    el = e0.elapsed_time(e1) * 1e-3
    el_max = max_over_ranks(el, world)
    value = N * args.steps * world / el_max
    part_s = np.array([s.particle_seconds for s in stats])
    solve_s = np.array([s.solve.seconds for s in stats])
    sort_s = np.array([s.sort_seconds for s in stats if s.sorted])
    relres = max(s.solve.relres for s in stats)
    its = [s.solve.iterations for s in stats]
    collisions = float(np.mean([s.collisions for s in stats]))
    peak, peak_kind = measured_peaks()
    achieved = ALGO_BYTES_MIXED * N / part_s.mean() / 1e9
    phi_now = ctx.phi
    mom_now = ctx.moments if not args.skip_cpu else None
    lv = mg_levels(p.Nx, p.Ny, p.Nz)
    fbytes = np.array([field_phase_bytes(lv, s.solve.iterations, s.solve.refinements) for s in stats])
    solve_gbs = float((fbytes / solve_s).mean()) / 1e9

    # ---------------- end to end through host buffers ------------------
    e2e = None
    e2e_steps = 0 if args.no_e2e else E2E_SORT_EVERY * E2E_CYCLES
    if e2e_steps:
        ctx.set_sort_every(E2E_SORT_EVERY)
        hpos = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
        hvel = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
        hmom = torch.empty((p.Nz, p.Ny, p.Nx, 4), dtype=torch.float64, pin_memory=True).numpy()
        hphi = torch.empty((p.Nz, p.Ny, p.Nx), dtype=torch.float64, pin_memory=True).numpy()
        hpos[:] = pos
        hvel[:] = vel
        # warm-up: two sort cycles (the first call uploads; later ones pipeline)
        for _ in range(max(2 * E2E_SORT_EVERY, args.warmup)):
            ctx.step_host(hpos, hvel, dt, rtol, 400, hmom, hphi)
        barrier(world)
        t0 = time.perf_counter()
        marks = [t0]
        for q in range(e2e_steps):
            ctx.step_host(hpos, hvel, dt, rtol, 400, hmom, hphi)
            if (q + 1) % E2E_SORT_EVERY == 0:
                marks.append(time.perf_counter())
        e2e_el = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": N * e2e_steps * world / e2e_el, "unit": "particle-steps/s",
               "h2d_bytes_per_step": 48 * N, "d2h_bytes_per_step": 48 * N + 40 * p.Nx * p.Ny * p.Nz,
               "steps": e2e_steps, "warmup": max(2 * E2E_SORT_EVERY, args.warmup), "api": "ecs_step_host",
               "sort_every": E2E_SORT_EVERY,
               "link_gbs": (96 * N + 40 * p.Nx * p.Ny * p.Nz) * e2e_steps / e2e_el / 1e9,
               # each sort cycle on its own (host wall clock, this rank): the
               # value above is the whole run
               "cycle_values": [N * E2E_SORT_EVERY / (b - a) for a, b in zip(marks, marks[1:])]}
        del hpos, hvel
    ctx.close()

    # ---------------- plain FP64 GPU path, same workload ---------------
    plain = None
    if not args.skip_fp64:
        ctx64 = E.Context(p, E.ECS_PREC_FP64, np_capacity=N, stream=stream.cuda_stream)
        ctx64.upload_particles(pos, vel)
        ctx64.collect()
        ctx64.compute_potential(rtol=rtol, max_it=400)
        ctx64.step(dt, rtol, 400)
        k64 = max(1, args.steps)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        st64 = [ctx64.step(dt, rtol, 400) for _ in range(k64)]
        f1.record(stream)
        torch.cuda.synchronize()
        el64 = max_over_ranks(f0.elapsed_time(f1) * 1e-3, world)
        plain = {"value": N * k64 * world / el64, "ms_per_step": 1e3 * el64 / k64, "steps": k64,
                 "particle_ms": 1e3 * float(np.mean([s.particle_seconds for s in st64])),
                 "solve_ms": 1e3 * float(np.mean([s.solve.seconds for s in st64]))}
        ctx64.close()

    configs = None if args.skip_configs else {"c1": run_c1(E, stream, args), "c3": run_c3(E, stream, args)}

    serving = None
    if not args.skip_serve:
        from ecsprt_gb300 import workloads as W

        serving = {"solves": run_serve_solves(E, W, args.serve_requests),
                   "ensemble": run_serve_sims(E, W, 48, args.serve_steps)}
    if rank != 0:
        return
    cpu = cpu_baseline(w, pos, vel, phi_now) if not args.skip_cpu else None
    if cpu is not None:
        cpu["solve"] = cpu_solve_baseline(w, mom_now)
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": workload_config(w, world),
        "roofline": {"bound": "hbm", "kernel": "k_tiles32 (fused push+collide+move+deposit, ions by tile)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": TRAFFIC_BYTES_PER_ION * N,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one step launch "
                                       "on the 64^3 case, per ion, times the ions here",
                     "algorithmic_bytes_per_launch": ALGO_BYTES_MIXED * N,
                     "design_bytes_per_launch": RECORD_BYTES_MIXED * N},
        "roofline_solve": {"bound": "hbm", "phase": "field phase: RHS + operator set-up + solve (one graph)",
                           "achieved": solve_gbs, "peak": peak, "unit": "GB/s", "frac": solve_gbs / peak,
                           "peak_kind": peak_kind, "bytes_per_phase": float(fbytes.mean()),
                           "bytes_rule": "12 B a cell an FP32 operator or smoother application, 24 B FP64, "
                                         "4 / 8 B a cell every other FP32 / FP64 vector read or written, each "
                                         "multigrid level at its own size (bench.field_phase_bytes)",
                           "solves_per_s": float(1.0 / solve_s.mean())},
        "solve_latency_ms": {"p50": 1e3 * float(np.percentile(solve_s, 50)),
                             "p99": 1e3 * float(np.percentile(solve_s, 99)),
                             "iterations": its, "max_relres": relres},
        "phase_ms": {"particles": 1e3 * float(part_s.mean()), "solve": 1e3 * float(solve_s.mean()),
                     "sort": 1e3 * float(sort_s.mean()) if sort_s.size else 0.0},
        "collisions_per_step": collisions,
        "plain_fp64": plain,
        "configs": configs,
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "serving": serving,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--skip-serve", action="store_true", help="leave out the request-loop measurements")
    ap.add_argument("--skip-configs", action="store_true",
                    help="leave out the 32^3 FP64 and 256x256x128 reflecting-z workload lines")
    ap.add_argument("--serve-requests", type=int, default=10000, help="stand-alone solve requests (Poisson, 200/s)")
    ap.add_argument("--serve-steps", type=int, default=500, help="steps of each of the 48 served simulations")
    ap.add_argument("--grid", type=int, default=None, help="profiling only: smaller cube edge")
    ap.add_argument("--ppc", type=int, default=None, help="profiling only: ions per cell")
    ap.add_argument("--no-solver-graphs", action="store_true",
                    help="profiling only: launch the field phase (RHS, set-up, refinement sweeps, FGMRES steps) "
                         "kernel by kernel from the host instead of as one CUDA graph (same kernels; ncu then "
                         "lists each one)")
    args = ap.parse_args()
    if args.grid:
        WORKLOAD["n"] = args.grid
        WORKLOAD["name"] = WORKLOAD["name"].replace("128^3", f"{args.grid}^3")
    if args.ppc:
        WORKLOAD["ppc"] = args.ppc
        WORKLOAD["name"] = WORKLOAD["name"].replace("64 ions/cell", f"{args.ppc} ions/cell")
    world, rank, local = dist_setup() if args.impl == "ours" else (
        int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        from ecsprt_gb300 import build

        build.build()
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
