"""Benchmark: served steady SUPG transport solves at relative residual 1e-10.

Workload (one step): 256 independent steady SUPG/CAU convection-diffusion
requests, structured N x N node meshes with N uniform in [33, 513] (seed 4),
velocity angle uniform in [0, 360), conductivity log-uniform in
[1e-8, 1e-2], submitted to the request server (continuous batching, meshes
resident in HBM).  Each request is assembled on the device (SUPG + CAU at
u = 0), Diag-preconditioned and solved to true relative residual 1e-10 with
FP32 GMRES(30) cycles inside FP64 iterative refinement; requests join and
leave the running batch between restart cycles.  The plain method for
comparison is the reference's FP64 GMRES(30) run one request at a time on
the same GPU.

Output: one JSON line (rank 0).  `value` is served solves/s with every
request submitted at t = 0, latency p50/p99 = done - submit;
`served_poisson` repeats the pass with Poisson arrivals at 80% of that rate;
`e2e` is the same metric through the host-buffer C ABI: every step serves
each request from host buffers (fg_server_submit_host: element blocks and
right-hand side copied in, the solution copied out before the request is
polled); `e2e.synchronous_batch` is the same through the synchronous calls.
`--impl reference` times the reference's CPU implementation of the path (the
oracle port where the reference's own build is absent) on the host cores,
on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s + p50/p99 latency @1e-10 resid: served mixed vs plain FP64 GMRES"
WORKLOAD = ("served steady SUPG/CAU transport: 256 requests, NxN nodes N~U[33,513] (seed 4), "
            "angle~U[0,360), k~logU[1e-8,1e-2]; device assembly + Diag + GMRES(30), FP32 inner + FP64 "
            "refinement to true rel. residual 1e-10, continuous batching")
KMAX, TOL = 30, 1e-10
BASIS = "fp32"          # storage of the Krylov basis in the mixed-precision solves (--basis)


def served_precision(fg):
    """Precision of the mixed solves: FP32 arithmetic, basis in FP32 or FP16."""
    return fg.FG_PREC_MIXED16 if BASIS == "fp16" else fg.FG_PREC_MIXED
# DRAM bytes / algorithmic bytes of one batched FP32 matvec, measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum of the two k_ebe_mv3p
# launches of one matvec of `bench.py --matvec-only --count 32 --steps 1`,
# cold): 481.6 MB for 418.19 MB algorithmic; the difference is the patches'
# index blobs (16-bit x-segment positions, dof lists and incidence lists,
# ~16.5 B per element where the algorithmic count charges 12 B of equation
# numbers) and the x segments' 8-entry alignment.  The traffic scales with
# the instances (each patch reads its own blocks and blob once).
MATVEC_TRAFFIC_RATIO = 481.61 / 418.19


# ------------------------------------------------------------------ CPU legs
# The CPU arm solves the same instances with the reference's method
# (Build_K_F_SUPG + CAU, Diag_precond_EBE_setup, FP64 pgmres GMRES(30), tol
# 1e-10) built with the reference's own compiler flags (-Ofast
# -march=native), one instance per host core, every core busy: the
# reference's own functions where oracle.build() compiled them
# (oracle/Makefile `ref_fast`, only where the reference's sources are),
# else the oracle's restatement of them (`fast`).  The timed
# region of a solve is what the reference's Process_Time covers for one
# linear solve: assembly, preconditioner set-up and GMRES; the mesh and its
# connectivity (Preprocess) are made before it, as the GPU arm's meshes are
# resident before its timed region.
CPU_KINDS = {
    "reference": "the reference's own Process iteration (Build_K_F_SUPG.c + F_assembly.c, scaling, "
                 "Diag_precond_EBE_setup.c, pgmres.c) compiled from its sources with -Ofast -march=native, one "
                 "rank",
    "port": "oracle restatement of the reference's Build_K_F_SUPG + Diag + FP64 GMRES(30), built -Ofast "
            "-march=native"}


def cpu_kind():
    """("reference" | "port") for the timed CPU arm: the reference's -Ofast
    build where oracle.build() made it, else the restatement (call before the
    CPU pool starts)."""
    import oracle as O
    O.build(ref=False, fast=True)
    return "reference" if O.ref_fast_available() else "port"


def _cpu_init(kind="port"):
    sys.path.insert(0, ROOT)
    import oracle as O
    O.use_fast_build()
    if kind == "reference":
        O.use_ref_fast()


def _cpu_solve(args):
    """One instance on the host: (idx, t_start, t_end, GMRES iterations, elements)."""
    idx, count, seed = args
    import oracle as O
    from parallel_fem_codes_gb300 import meshgen as G
    p = G.batch_transport_problem(idx, count, seed)
    m = p.mesh
    if O.using_ref_fast():
        # the reference's own Process iteration, timed inside its build after
        # its (untimed) Fill_LM and local reordering
        sec, it = O.ref_timed_solve(p, kmax=KMAX, lmax=100000, tol=TOL)
        t1 = time.perf_counter()
        return idx, t1 - sec, t1, it, m.nel
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    t0 = time.perf_counter()
    A, F = O.build_k_f_supg(p)
    X, it, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=KMAX, lmax=100000, tol=TOL)
    return idx, t0, time.perf_counter(), it, m.nel


def _c1_cpu(_):
    """Steady transport 129 x 129 (velocity angle 30, k = 1e-6): the
    reference's method on one host core (assembly + Diag + FP64 GMRES(30)),
    timed; returns (seconds, iterations, solution)."""
    import oracle as O
    from parallel_fem_codes_gb300 import meshgen as G
    p = G.transport_problem(129, angle_deg=30.0, k=1e-6)
    m = p.mesh
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    t0 = time.perf_counter()
    A, F = O.build_k_f_supg(p)
    X, it, *_ = O.ebe_diag_solve(lm, A, m.neq, F, perm, inv, kmax=KMAX, lmax=100000, tol=TOL)
    return time.perf_counter() - t0, int(it), X[:m.neq].copy()


def _euler_cpu(args):
    """Euler OBLIQUO n x n: `steps` steps of Predictor_Old (2 corrections,
    GMRES(25), BlockDiag, FP64) by the oracle on one host core; returns
    (seconds, stats, final state)."""
    n, steps = args
    import oracle as O
    from parallel_fem_codes_gb300 import meshgen as G
    p = G.obliquo_problem(n)
    to = O.TimeOpts(0, 2, 1e-3, 0, steps * p.dt, 1e-6, 0)
    t0 = time.perf_counter()
    u, a, st = O.euler_predictor(p, to, tol=1e-10, kmax=25)
    return time.perf_counter() - t0, st, u


def cpu_sample_groups(nel, size, groups):
    """A sample of `size` instances stratified by element count (the middle
    instance of each of `size` equal strata of the instances sorted by
    size), cut into `groups` consecutive groups of similar sizes (one group
    per timed step, so the cores of a step finish together)."""
    order = sorted(range(len(nel)), key=lambda i: (nel[i], i))
    size = max(1, min(size, len(nel)))
    pick = [order[int((j + 0.5) * len(nel) / size)] for j in range(size)]
    groups = max(1, min(groups, size))
    return [pick[g * size // groups:(g + 1) * size // groups] for g in range(groups)]


def run_cpu_steps(pool, count, seed, groups):
    """Run each group as one step (its instances concurrently, one per core).
    Returns (solves, summed step walls, per-step walls, per-solve seconds,
    iterations)."""
    walls, lat, its = [], [], []
    for grp in groups:
        res = pool.map(_cpu_solve, [(i, count, seed) for i in reversed(grp)], chunksize=1)   # largest first
        walls.append(max(r[2] for r in res) - min(r[1] for r in res))
        lat += [r[2] - r[1] for r in res]
        its += [r[3] for r in res]
    return sum(len(g) for g in groups), sum(walls), walls, lat, its


def cpu_leg(pool, cores, count, seed, steps, kind="port"):
    """CPU throughput on a sample of min(count, cores x steps) instances
    stratified by size, `steps` steps of up to one instance per core.  The
    value is the packed throughput cores x solves / (summed solve seconds):
    the rate of every core solving back to back, each solve timed while the
    other cores solve too (the whole batch on the host would approach it;
    the tail of a step, where cores idle, is not charged)."""
    nel, _ = _sizes(count, seed)
    groups = cpu_sample_groups(nel, cores * steps, steps)
    n, wall, walls, lat, its = run_cpu_steps(pool, count, seed, groups)
    picked = [i for g in groups for i in g]
    mean_s = float(np.mean([nel[i] for i in picked]))
    sample = (f"{n} of {count} instances, stratified by element count (sample mean {mean_s:.0f} elements vs "
              f"workload mean {np.mean(nel):.0f}, ratio {mean_s / np.mean(nel):.3f}), {len(groups)} step(s) of "
              f"up to {cores} concurrent solves, one instance per core; value = cores x solves / summed solve "
              f"seconds; {CPU_KINDS[kind]}, tol 1e-10; timed per solve: assembly + set-up + GMRES")
    return {"value": cores * n / sum(lat), "solves": n, "wall_s": wall, "step_walls_s": walls, "lat": lat,
            "iterations_mean": float(np.mean(its)), "sample": sample, "sample_mean_ratio": mean_s / np.mean(nel)}


def _sizes(count, seed):
    from parallel_fem_codes_gb300 import meshgen as G
    return G.batch_transport_sizes(count, seed)


def workload_config(count, seed):
    """The `config` of both arms' JSON lines (identical by construction)."""
    nel, neq = _sizes(count, seed)
    return {"workload": WORKLOAD, "instances": count, "seed": seed, "elements": int(sum(nel)),
            "dofs": int(sum(neq)), "kmax": KMAX, "tol": TOL,
            "l2": "inputs larger than L2 (per-step working set >1 GB)"}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self, dev=0):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except OSError:
            return None
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == str(dev)]
        if not rows:
            return None
        sm = [float(r[1].split()[0]) for r in rows if r[1].split()[0].replace(".", "").isdigit()]
        mx = [float(r[2].split()[0]) for r in rows if r[2].split()[0].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ helpers
def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def pct(v, q):
    return float(np.percentile(np.asarray(v, dtype=np.float64), q)) if len(v) else None


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        return rank, ws, dist
    return 0, 1, None


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ reference arm
def run_reference(args, rank, ws, dist):
    """The reference's CPU method on every host core: W warm-up steps (the
    smallest instances, one per core), then K timed steps, each a group of
    one instance per core from a sample of K x cores instances stratified by
    size (the whole workload when K x cores >= instances)."""
    if rank != 0:
        return 0
    kind = cpu_kind()
    cores = os.cpu_count() or 1
    nel, _ = _sizes(args.count, args.seed)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_cpu_init, initargs=(kind,)) as pool:
        small = sorted(range(args.count), key=lambda i: (nel[i], i))[:cores]
        for _ in range(args.warmup):
            run_cpu_steps(pool, args.count, args.seed, [small])
        leg = cpu_leg(pool, cores, args.count, args.seed, args.steps, kind)
    value = leg["value"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * leg["wall_s"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(args.count, args.seed),
            "latency_ms": {"p50": 1e3 * pct(leg["lat"], 50), "p99": 1e3 * pct(leg["lat"], 99),
                           "note": "per solve, with every core solving"},
            "iterations_mean": leg["iterations_mean"], "wall_s": leg["wall_s"],
            "wall_solves_per_s": leg["solves"] / leg["wall_s"],
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": kind,
                             "sample": leg["sample"]},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ our arm
# ------------------------------------------------------------------ other drivers
def euler_leg(fg, G, n=513, steps=20, corrections=2, kmax=25, cpu_job=None):
    """Euler OBLIQUO on n x n nodes (Mach 2, dimensionless, dt = 0.5 min h /
    (|v| + c)), `steps` time steps of Predictor_Old with `corrections`
    corrections each (StopMulticorrection = ITERATION), GMRES(kmax) with the
    reference's 4x4 BlockDiag, FP64 and mixed precision; plus the 12x12 EBE
    matvec roofline on the same system."""
    p = G.obliquo_problem(n)
    t0 = time.perf_counter()
    s = fg.euler_system(p)
    setup_s = time.perf_counter() - t0
    s.euler_predictor(p, fg.time_opts(0, 1, 1e-3, 0, p.dt, 1e-6, max_steps=1), kmax=kmax)     # warm-up
    out = {"workload": f"Euler OBLIQUO {n}x{n} nodes, {p.mesh.nel} elements, {p.mesh.neq} dofs, "
                       f"{steps} steps x {corrections} corrections, GMRES({kmax}), BlockDiag, tol 1e-10",
           "setup_s": setup_s}
    us = {}
    for name, prec in (("fp64", fg.FG_PREC_FP64), ("mixed", fg.FG_PREC_MIXED)):
        to = fg.time_opts(0, corrections, 1e-3, 0, steps * p.dt, 1e-6, max_steps=steps)
        t0 = time.perf_counter()
        u, a, st = s.euler_predictor(p, to, kmax=kmax, tol=1e-10, precision=prec)
        wall = time.perf_counter() - t0
        us[name] = u
        out[name] = {"seconds": wall, "steps": st["steps"], "corrections": st["corrections"],
                     "gmres_iterations": st["gmres_iterations"], "steps_per_s": st["steps"] / wall,
                     "ms_per_correction": 1e3 * wall / st["corrections"],
                     "last_true_rel_residual": st["true_rel_residual"]}
    out["mixed_rel_diff_vs_fp64"] = float(np.linalg.norm(us["mixed"] - us["fp64"]) / np.linalg.norm(us["fp64"]))
    if cpu_job is not None:
        # the reference method on one host core, one step (a bounded sample),
        # and the GPU's one-step FP64 state against it
        secs, sto, uo = cpu_job.get()
        u1, _, st1 = s.euler_predictor(p, fg.time_opts(0, corrections, 1e-3, 0, p.dt, 1e-6, max_steps=1),
                                       kmax=kmax, tol=1e-10)
        out["cpu_reference_method_1step"] = {
            "seconds": secs, "ms_per_correction": 1e3 * secs / max(1, sto["corrections"]),
            "gmres_iterations": sto["gmres_iterations"], "cores": 1, "kind": "port, -Ofast -march=native",
            "gpu_fp64_rel_diff": float(np.linalg.norm(u1 - uo) / np.linalg.norm(uo)),
            "gpu_gmres_iterations": st1["gmres_iterations"]}
    out["matvec"] = _matvec_roofline(fg, s)
    # the reference's second configuration of this problem: CSR operator on the
    # RCM numbering with ILU(0) (MatrixVectorProductScheme "CSR", "ILU0")
    t0 = time.perf_counter()
    sc = fg.euler_system(p, reorder=True)
    sc.set_operator(fg.FG_OP_CSR)
    ilu = {"setup_s": time.perf_counter() - t0}
    sc.euler_predictor(p, fg.time_opts(0, 1, 1e-3, 0, p.dt, 1e-6, max_steps=1, precond=fg.FG_PRECOND_ILU0,
                                       setup_flags=0), kmax=kmax)                                  # warm-up
    isteps = min(steps, 3)            # the ILU(0) substitutions are latency-bound: fewer steps
    ilu["steps_timed"] = isteps
    u_bd, _, _ = s.euler_predictor(p, fg.time_opts(0, corrections, 1e-3, 0, isteps * p.dt, 1e-6, max_steps=isteps),
                                   kmax=kmax, tol=1e-10)
    for name, prec in (("fp64", fg.FG_PREC_FP64), ("mixed", fg.FG_PREC_MIXED)):
        to = fg.time_opts(0, corrections, 1e-3, 0, isteps * p.dt, 1e-6, max_steps=isteps, precond=fg.FG_PRECOND_ILU0,
                          setup_flags=0)
        t0 = time.perf_counter()
        u, a, st = sc.euler_predictor(p, to, kmax=kmax, tol=1e-10, precision=prec)
        wall = time.perf_counter() - t0
        ilu[name] = {"seconds": wall, "steps": st["steps"], "corrections": st["corrections"],
                     "gmres_iterations": st["gmres_iterations"], "steps_per_s": st["steps"] / wall,
                     "ms_per_correction": 1e3 * wall / st["corrections"],
                     "last_true_rel_residual": st["true_rel_residual"],
                     "rel_diff_vs_blockdiag_fp64": float(np.linalg.norm(u - u_bd) / np.linalg.norm(u_bd))}
    out["csr_ilu0_rcm"] = ilu
    # block-Jacobi ILU(0) over P row blocks of the RCM numbering: what P MPI
    # ranks of the reference factorise (each its own rows); substitutions a
    # warp per block.  Every step of the configuration.
    u_bd, _, _ = s.euler_predictor(p, fg.time_opts(0, corrections, 1e-3, 0, steps * p.dt, 1e-6, max_steps=steps),
                                   kmax=kmax, tol=1e-10)
    for nblk in (1024, 4096):
        blk = {"blocks": nblk, "steps_timed": steps}
        sc.set_ilu_blocks(nblk)
        sc.euler_predictor(p, fg.time_opts(0, 1, 1e-3, 0, p.dt, 1e-6, max_steps=1, precond=fg.FG_PRECOND_ILU0,
                                           setup_flags=0), kmax=kmax)                              # warm-up
        for name, prec in (("fp64", fg.FG_PREC_FP64), ("mixed", fg.FG_PREC_MIXED)):
            to = fg.time_opts(0, corrections, 1e-3, 0, steps * p.dt, 1e-6, max_steps=steps,
                              precond=fg.FG_PRECOND_ILU0, setup_flags=0)
            t0 = time.perf_counter()
            u, a, st = sc.euler_predictor(p, to, kmax=kmax, tol=1e-10, precision=prec)
            wall = time.perf_counter() - t0
            blk[name] = {"seconds": wall, "steps": st["steps"], "corrections": st["corrections"],
                         "gmres_iterations": st["gmres_iterations"], "steps_per_s": st["steps"] / wall,
                         "ms_per_correction": 1e3 * wall / st["corrections"],
                         "last_true_rel_residual": st["true_rel_residual"],
                         "rel_diff_vs_blockdiag_fp64": float(np.linalg.norm(u - u_bd) / np.linalg.norm(u_bd))}
        blk["ms_per_correction_vs_blockdiag"] = {
            k: blk[k]["ms_per_correction"] / out[k]["ms_per_correction"] for k in ("fp64", "mixed")}
        out[f"csr_block{nblk}_ilu0_rcm"] = blk
    return out


def c1_leg(fg, G, cpu_job=None, reps=5):
    """Steady transport 129 x 129 nodes (velocity angle 30, k = 1e-6, SUPG +
    CAU at u = 0, Diag, GMRES(30), tol 1e-10): latency of the plain FP64
    solve and of the mixed solve on the GPU (device assembly + set-up +
    solve, CUDA events), the whole CAU Process loop, and beside them the
    reference method on one host core with the GPU solutions' error
    against its FP64 solution."""
    p = G.transport_problem(129, angle_deg=30.0, k=1e-6)
    s = fg.transport_system(p)
    import torch
    stream = torch.cuda.ExternalStream(s.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"workload": f"steady transport 129x129 nodes, {p.mesh.nel} elements, {p.mesh.neq} dofs, angle 30, "
                       f"k 1e-6, SUPG+CAU, Diag, GMRES(30), tol 1e-10"}
    xs = {}
    for name, prec in (("fp64", fg.FG_PREC_FP64), ("mixed", fg.FG_PREC_MIXED)):
        lat = []
        for _ in range(reps + 1):
            e0.record(stream)
            s.transport_prepare(p)
            r = fg.solve_resident([s], kmax=KMAX, lmax=100000, tol=TOL, precision=prec)[0]
            e1.record(stream)
            e1.synchronize()
            lat.append(e0.elapsed_time(e1))
        xs[name] = s.solution()
        out[name] = {"ms_median": float(np.median(lat[1:])), "solves_per_s": 1e3 / float(np.median(lat[1:])),
                     "iterations": r["iterations"], "true_rel_residual": r["true_rel_residual"]}
    t0 = time.perf_counter()
    U, st = s.transport_process(p, KMAX, 1000, TOL, 1e-3)
    out["process"] = {"seconds": time.perf_counter() - t0, "nonlinear_iterations": st["nonlinear_iterations"],
                      "gmres_iterations": st["gmres_iterations"]}
    if cpu_job is not None:
        secs, it, X = cpu_job.get()
        out["cpu_reference_method"] = {"seconds": secs, "iterations": it, "cores": 1,
                                       "kind": "port, -Ofast -march=native"}
        for name in xs:
            out[name]["rel_err_vs_cpu_fp64"] = float(np.linalg.norm(xs[name][:len(X)] - X) / np.linalg.norm(X))
        out["speedup_fp64_vs_cpu_core"] = secs / (out["fp64"]["ms_median"] / 1e3)
    return out


def ns_leg(fg, G, n=1025, reynolds=1000.0, kmax=50, cycles=20):
    """Navier-Stokes CAVITY on n x n nodes (interior jittered by 0.2 h, seed 3),
    Re = 1000: one Picard step (device assembly, BlockDiagDOF3, GMRES(kmax)),
    the linear solve capped at `cycles` restart cycles (at this size and
    Reynolds number BlockDiagDOF3-GMRES needs far more to reach 1e-10), FP64
    and mixed; reported as Arnoldi iterations per second, plus the 9x9 EBE
    matvec roofline."""
    p = G.cavity_problem(n, reynolds=reynolds, jitter=0.2)
    t0 = time.perf_counter()
    s = fg.ns_system(p)
    setup_s = time.perf_counter() - t0
    s.ns_process(p, kmax=kmax, lmax=1, max_nonlinear=1)                                       # warm-up
    out = {"workload": f"NS CAVITY {n}x{n} nodes (jitter 0.2h), Re={reynolds:g}, {p.mesh.nel} elements, "
                       f"{p.mesh.neq} dofs; one Picard step, GMRES({kmax}) capped at {cycles} cycles, BlockDiagDOF3",
           "setup_s": setup_s}
    us = {}
    for name, prec in (("fp64", fg.FG_PREC_FP64), ("mixed", fg.FG_PREC_MIXED)):
        t0 = time.perf_counter()
        u, st = s.ns_process(p, kmax=kmax, lmax=cycles, tol=1e-10, max_nonlinear=1, precision=prec)
        us[name] = u
        wall = time.perf_counter() - t0
        out[name] = {"seconds": wall, "gmres_iterations": st["gmres_iterations"],
                     "iterations_per_s": st["gmres_iterations"] / wall,
                     "dof_iterations_per_s": p.mesh.neq * st["gmres_iterations"] / wall,
                     "true_rel_residual": st["true_rel_residual"]}
    out["mixed_rel_diff_vs_fp64"] = float(np.linalg.norm(us["mixed"] - us["fp64"]) / np.linalg.norm(us["fp64"]))
    out["note"] = ("restarted GMRES(50) with the 3x3 block-diagonal preconditioner stagnates on this problem: "
                   "the true residual stays near 7e-3 after 78 400 iterations (1 600 cycles) at 1025x1025, "
                   "near 1e-3 after 400 cycles at 257x257, so the leg times a fixed number of cycles")
    out["matvec"] = _matvec_roofline(fg, s)
    return out


def c5_leg(fg, G, count=96, rates=(10, 30, 100, 300, 1000, 2000), seed=5):
    """Mixed serving: Poisson arrivals at each rate of `count` requests, 70%
    steady SUPG/CAU transport and 30% 10-step Euler OBLIQUO loops
    (Predictor_Old, 2 corrections per step), elements log-uniform in
    [1e3, 2e6] (angle, conductivity as the batched transport workload), all
    mixed precision to 1e-10; transport requests are batched continuously,
    Euler loops run beside them.  Reports per rate the throughput (requests
    / makespan) and p50/p99 latency (done - submit) per kind."""
    rng = np.random.Generator(np.random.PCG64(seed))
    kinds = rng.random(count) < 0.3
    elems = np.exp(rng.uniform(np.log(1e3), np.log(2e6), size=count))
    sides = np.maximum(9, (1 + np.sqrt(elems / 2)).astype(int))
    angles = rng.uniform(0.0, 360.0, size=count)
    kappa = np.exp(rng.uniform(np.log(1e-8), np.log(1e-2), size=count))
    reqs = []
    t0 = time.perf_counter()
    for i in range(count):
        if kinds[i]:
            pr = G.obliquo_problem(int(sides[i]))
            to = fg.time_opts(0, 2, 1e-3, 0, 10 * pr.dt, 1e-6, max_steps=10)
            reqs.append(("euler", fg.euler_system(pr), pr, to))
        else:
            pr = G.transport_problem(int(sides[i]), angle_deg=float(angles[i]), k=float(kappa[i]))
            reqs.append(("transport", fg.transport_system(pr), pr, None))
    setup_s = time.perf_counter() - t0

    def one(rate):
        sv = fg.Server(kmax=KMAX, lmax=10000, tol=TOL, precision=served_precision(fg))
        gaps = rng.exponential(1.0 / rate, size=count) if rate else np.zeros(count)
        arrive = np.cumsum(gaps) - gaps[0]
        t_start = sv.now()
        for i, (kind, sy, pr, to) in enumerate(reqs):
            delay = arrive[i] - (sv.now() - t_start)
            if delay > 0:
                time.sleep(delay)
            if kind == "euler":
                sv.submit_euler(sy, pr, to, i)
            else:
                sv.submit(sy, pr, i)
        sv.wait(count, timeout=900)
        res = sv.poll(count + 16)
        sv.close()
        t_end = max(r["t_done"] for r in res)
        out = {"rate_req_per_s": rate, "requests_per_s": count / (t_end - t_start),
               "converged_all": all(r["true_rel_residual"] <= TOL for r in res)}
        for kind in ("transport", "euler"):
            lat = [r["t_done"] - r["t_submit"] for r in res if reqs[r["tag"]][0] == kind]
            if lat:
                out[kind] = {"n": len(lat), "p50_ms": 1e3 * pct(lat, 50), "p99_ms": 1e3 * pct(lat, 99)}
        return out

    one(0)                                                                   # warm-up, all at once
    out = {"workload": f"{count} requests: 70% steady transport, 30% 10-step Euler OBLIQUO (2 corrections/step), "
                       f"elements logU[1e3, 2e6] (seed {seed}), mixed precision to 1e-10; Poisson arrivals",
           "transport_requests": int((~kinds).sum()), "euler_requests": int(kinds.sum()),
           "elements_total": int(sum(2 * (int(n) - 1) ** 2 for n in sides)), "setup_s": setup_s,
           "rates": [one(r) for r in rates]}
    return out


def _matvec_roofline(fg, s):
    peak, kind = peaks()
    r = {}
    for prec in (64, 32):
        ms, b = fg.bench_matvec([s], precision=prec, reps=20)
        gbs = b / (ms * 1e-3) / 1e9
        r[f"fp{prec}"] = {"ms": ms, "bytes": b, "GB_per_s": gbs, "frac": gbs / peak}
    r["peak"], r["peak_source"] = peak, kind
    return r


def run_kernel_tour(args):
    """Each kernel family once at a moderate size (the workload of the
    per-kernel ncu table): transport 8 x 257^2 (assembly, Diag, two restart
    cycles mixed and FP64), Euler 257^2 (one step FP64 and mixed,
    BlockDiag), NS cavity 257^2 (one GMRES(50) cycle FP64 and mixed,
    BlockDiagDOF3), Euler 129^2 on the RCM CSR operator with ILU(0),
    block-Jacobi ILU(0) over 64 blocks and SPIKE.  Cycle limits stop the
    solves early on purpose; those statuses are printed, not raised."""
    from parallel_fem_codes_gb300 import femgpu as fg, meshgen as G
    fg.lib(build_if_missing=False)

    def run(f, *a, **k):
        try:
            f(*a, **k)
        except fg.FemGpuError as e:
            print("note:", e)

    probs = [G.transport_problem(257, angle_deg=20.0 * i, k=1e-5) for i in range(8)]
    sy = [fg.transport_system(p) for p in probs]
    for prec in (fg.FG_PREC_MIXED, fg.FG_PREC_FP64):
        for s, p in zip(sy, probs):
            s.transport_prepare(p)
        run(fg.solve_resident, sy, kmax=30, lmax=2, tol=1e-10, precision=prec)
    pe = G.obliquo_problem(257)
    se = fg.euler_system(pe)
    for prec in (fg.FG_PREC_FP64, fg.FG_PREC_MIXED):
        run(se.euler_predictor, pe, fg.time_opts(0, 1, 1e-3, 0, pe.dt, 1e-6, max_steps=1), kmax=25, lmax=2, tol=1e-10,
            precision=prec)
    pn = G.cavity_problem(257, reynolds=1000.0, jitter=0.2)
    sn = fg.ns_system(pn)
    for prec in (fg.FG_PREC_FP64, fg.FG_PREC_MIXED):
        run(sn.ns_process, pn, kmax=50, lmax=1, tol=1e-10, max_nonlinear=1, precision=prec)
    pc = G.obliquo_problem(129)
    sc = fg.euler_system(pc, reorder=True)
    sc.set_operator(fg.FG_OP_CSR)
    to = fg.time_opts(0, 1, 1e-3, 0, pc.dt, 1e-6, max_steps=1, precond=fg.FG_PRECOND_ILU0, setup_flags=0)
    run(sc.euler_predictor, pc, to, kmax=25, lmax=2, tol=1e-10)
    sc.set_ilu_blocks(64)
    run(sc.euler_predictor, pc, to, kmax=25, lmax=2, tol=1e-10)
    sc.set_spike(16, 16)
    to2 = fg.time_opts(0, 1, 1e-3, 0, pc.dt, 1e-6, max_steps=1, precond=fg.FG_PRECOND_SPIKE, setup_flags=0)
    run(sc.euler_predictor, pc, to2, kmax=25, lmax=2, tol=1e-10)
    print("kernel tour done", flush=True)
    return 0


def run_probe(args):
    """Small single-kernel workloads for profiling (one JSON line each):
    matvec:euler|ns:N:32|64   the S x S EBE matvec of Euler OBLIQUO / NS cavity N x N
                              (assembled blocks), 2 warm-up + 2 timed matvecs;
    ilu:N:P:steps             Euler OBLIQUO N x N, BlockDiag and block-Jacobi ILU(0)
                              over P row blocks of the RCM CSR operator, FP64 and
                              mixed, ms per correction;
    ilusetup:N:P              the ILU(0) set-up (CSR values, factorisation, F <- M^-1 F)
                              and one application through the host API."""
    from parallel_fem_codes_gb300 import femgpu as fg, meshgen as G
    fg.lib(build_if_missing=False)
    kind, *rest = args.probe.split(":")
    if kind == "matvec":
        mesh, n, prec = rest[0], int(rest[1]), int(rest[2])
        if mesh == "euler":
            p = G.obliquo_problem(n)
            s = fg.euler_system(p)
            s.euler_assemble(p)
        else:
            p = G.cavity_problem(n, reynolds=1000.0, jitter=0.2)
            s = fg.ns_system(p)
            s.ns_assemble(p)
        ms, b = fg.bench_matvec([s], precision=prec, reps=2)
        peak, kindp = peaks()
        print(json.dumps({"probe": args.probe, "ms": ms, "algorithmic_bytes": b, "GB_per_s": b / ms / 1e6,
                          "frac": b / ms / 1e6 / peak, "peak_source": kindp, "patch_colours": s.info()["ncolours"]}),
              flush=True)
    elif kind == "ilu":
        n, nb, steps = int(rest[0]), int(rest[1]), int(rest[2])
        p = G.obliquo_problem(n)
        s = fg.euler_system(p)
        s.euler_predictor(p, fg.time_opts(0, 1, 1e-3, 0, p.dt, 1e-6, max_steps=1), kmax=25)
        out = {"probe": args.probe}
        t0 = time.perf_counter()
        u_bd, _, st = s.euler_predictor(p, fg.time_opts(0, 2, 1e-3, 0, steps * p.dt, 1e-6, max_steps=steps), kmax=25,
                                        tol=1e-10)
        out["blockdiag_ms_per_correction"] = 1e3 * (time.perf_counter() - t0) / st["corrections"]
        sc = fg.euler_system(p, reorder=True)
        sc.set_operator(fg.FG_OP_CSR)
        sc.set_ilu_blocks(nb)
        sc.euler_predictor(p, fg.time_opts(0, 1, 1e-3, 0, p.dt, 1e-6, max_steps=1, precond=fg.FG_PRECOND_ILU0,
                                           setup_flags=0), kmax=25)
        for name, prec in (("fp64", fg.FG_PREC_FP64), ("mixed", fg.FG_PREC_MIXED)):
            to = fg.time_opts(0, 2, 1e-3, 0, steps * p.dt, 1e-6, max_steps=steps, precond=fg.FG_PRECOND_ILU0,
                              setup_flags=0)
            t0 = time.perf_counter()
            u, _, st = sc.euler_predictor(p, to, kmax=25, tol=1e-10, precision=prec)
            out[name] = {"ms_per_correction": 1e3 * (time.perf_counter() - t0) / st["corrections"],
                         "gmres_iterations": st["gmres_iterations"], "true_rel_residual": st["true_rel_residual"],
                         "rel_diff_vs_blockdiag": float(np.linalg.norm(u - u_bd) / np.linalg.norm(u_bd))}
        print(json.dumps(out), flush=True)
    elif kind == "ilusetup":
        n, nb = int(rest[0]), int(rest[1])
        p = G.obliquo_problem(n)
        sc = fg.euler_system(p, reorder=True)
        sc.set_operator(fg.FG_OP_CSR)
        sc.set_ilu_blocks(nb)
        R = sc.euler_assemble(p)
        sc.precond_setup(fg.FG_PRECOND_ILU0, 0, R.copy())
        t0 = time.perf_counter()
        sc.precond_setup(fg.FG_PRECOND_ILU0, 0, R.copy())
        t1 = time.perf_counter()
        sc.precond_apply(R.copy())
        t2 = time.perf_counter()
        print(json.dumps({"probe": args.probe, "setup_ms": 1e3 * (t1 - t0), "apply_ms_host_api": 1e3 * (t2 - t1)}),
              flush=True)
    else:
        raise SystemExit(f"unknown probe {args.probe}")
    return 0


def run_matvec_only(args):
    from parallel_fem_codes_gb300 import femgpu as fg, meshgen as G
    fg.lib(build_if_missing=False)
    probs = G.batch_transport_problems(args.count, args.seed)
    systems = [fg.transport_system(p) for p in probs]
    for s, p in zip(systems, probs):
        s.transport_assemble(p)
    ms, b = fg.bench_matvec(systems, precision=32, reps=max(1, args.steps))   # after 2 warm-up matvecs
    print(json.dumps({"matvec_only": True, "instances": args.count, "elements": sum(p.mesh.nel for p in probs),
                      "ms": ms, "algorithmic_bytes": b, "GB_per_s": b / ms / 1e6,
                      "matvecs": 2 + max(1, args.steps)}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--cpu-budget", type=int, default=400_000, help="elements in the CPU sample")
    ap.add_argument("--plain-count", type=int, default=0, help="instances in the plain FP64 leg (0 = all)")
    ap.add_argument("--basis", choices=["fp32", "fp16"], default="fp32",
                    help="storage of the Krylov basis in the mixed-precision solves (FP32 arithmetic either way)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-legs", action="store_true", help="skip the Euler and Navier-Stokes legs")
    ap.add_argument("--euler-n", type=int, default=513, help="nodes per side of the Euler leg")
    ap.add_argument("--ns-n", type=int, default=1025, help="nodes per side of the Navier-Stokes leg (odd)")
    ap.add_argument("--c5-count", type=int, default=96, help="requests per rate of the mixed serving leg")
    ap.add_argument("--kernel-tour", action="store_true",
                    help="run every kernel family once at a moderate size (the per-kernel ncu table's workload)")
    ap.add_argument("--probe", default="", help="a single-kernel workload for profiling (see run_probe)")
    ap.add_argument("--matvec-only", action="store_true",
                    help="only the batched FP32 EBE matvec of --count instances (2 warm-up + --steps "
                         "matvecs); the small case the ncu traffic capture runs")
    args = ap.parse_args()
    global BASIS
    BASIS = args.basis
    rank, ws, dist = dist_setup()
    if args.impl == "reference":
        return run_reference(args, rank, ws, dist)

    if args.probe:
        return run_probe(args)
    if args.matvec_only:
        return run_matvec_only(args)
    if args.kernel_tour:
        return run_kernel_tour(args)

    # spawn the CPU pool before the first GPU call
    cores = os.cpu_count() or 1
    pool = None
    cpu_k = "port"
    if rank == 0 and not args.no_cpu:
        cpu_k = cpu_kind()
        pool = mp.get_context("spawn").Pool(cores, initializer=_cpu_init, initargs=(cpu_k,))

    import torch
    from parallel_fem_codes_gb300 import femgpu as fg, meshgen as G

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    fg.lib(build_if_missing=False)
    probs = G.batch_transport_problems(args.count, args.seed + 1000 * rank)
    t0 = time.perf_counter()
    systems = [fg.transport_system(p) for p in probs]
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(systems[0].stream)

    def served_pass(arrivals=None):
        """Serve every instance once through the request server (continuous
        batching); arrivals: submit times in seconds (None = all at once).
        Returns (makespan_s, list of per-request results)."""
        sv = fg.Server(kmax=KMAX, lmax=10000, tol=TOL, precision=served_precision(fg))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        t_start = sv.now()
        for i, (s, p) in enumerate(zip(systems, probs)):
            if arrivals is not None:
                delay = arrivals[i] - (sv.now() - t_start)
                if delay > 0:
                    time.sleep(delay)
            sv.submit(s, p, i)
        sv.wait(len(systems), timeout=600)
        res = sv.poll(len(systems) + 16)
        torch.cuda.synchronize()
        e1.record()
        e1.synchronize()
        sv.close()
        return e0.elapsed_time(e1) / 1e3, res

    # autotuner (set-up, untimed): launch shapes of the full batch, mixed and FP64
    for s, p in zip(systems, probs):
        s.transport_prepare(p)
    tuned = {"mixed": fg.autotune(systems, kmax=KMAX, lmax=10000, tol=TOL, precision=served_precision(fg)),
             "fp64": fg.autotune(systems, kmax=KMAX, lmax=100000, tol=TOL, precision=fg.FG_PREC_FP64)}

    for _ in range(args.warmup):
        served_pass()
    barrier(dist)
    torch.cuda.synchronize()
    clk = ClockSampler(os.path.join(tempfile.gettempdir(), f"pfc_bench_clocks_{os.getpid()}_rank{rank}.csv"))
    l0 = fg.launch_count()
    launches_before_timed = l0
    times, lat = [], []
    with clk:
        for _ in range(args.steps):
            mk, res = served_pass()
            times.append(mk)
            lat += [r["t_done"] - r["t_submit"] for r in res]
    torch.cuda.synchronize()
    barrier(dist)
    launches = (fg.launch_count() - l0) / args.steps
    step_s = reduce_max(dist, sum(times) / len(times))
    value = ws * args.count / step_s
    conv = all(r["converged"] == 1 for r in res)
    worst_res = max(r["true_rel_residual"] for r in res)
    iters = [r["iterations"] for r in res]
    clocks = clk.summary(dev)
    xs_mixed = [s.solution() for s in systems[: min(8, len(systems))]]

    # Poisson arrivals at 80% of the saturated throughput
    rate = 0.8 * value / ws
    rng = np.random.Generator(np.random.PCG64(5 + rank))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=args.count))
    mk_p, res_p = served_pass(arrivals)
    lat_p = [r["t_done"] - r["t_submit"] for r in res_p]
    poisson = {"rate_req_per_s": rate, "solves_per_s": args.count / mk_p, "p50_ms": 1e3 * pct(lat_p, 50),
               "p99_ms": 1e3 * pct(lat_p, 99), "seed": 5}

    # the same instances as one synchronous batch (all finish together)
    def batch_step():
        for s, p in zip(systems, probs):
            s.transport_prepare(p)
        return fg.solve_resident(systems, kmax=KMAX, lmax=10000, tol=TOL, precision=served_precision(fg))

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    batch_step()
    e1.record(stream)
    e1.synchronize()
    sync_batch = {"solves_per_s": args.count / (e0.elapsed_time(e1) / 1e3)}

    # the plain method (FP64 GMRES(30)) over all instances as one batch: the
    # batching gain without the precision gain
    torch.cuda.synchronize()
    e0.record(stream)
    for s, p in zip(systems, probs):
        s.transport_prepare(p)
    r64b = fg.solve_resident(systems, kmax=KMAX, lmax=100000, tol=TOL, precision=fg.FG_PREC_FP64)
    e1.record(stream)
    e1.synchronize()
    plain_batched = {"solves_per_s": args.count / (e0.elapsed_time(e1) / 1e3),
                     "iterations_mean": float(np.mean([r["iterations"] for r in r64b])),
                     "converged_all": all(r["converged"] == 1 for r in r64b)}

    # plain FP64 GMRES, one instance at a time (latency distribution)
    nplain = args.count if args.plain_count <= 0 else min(args.plain_count, args.count)
    plain_lat, plain_iters, plain_err = [], [], []
    for i in range(nplain):
        s, p = systems[i], probs[i]
        s.transport_prepare(p)
        e0.record(stream)
        r = fg.solve_resident([s], kmax=KMAX, lmax=100000, tol=TOL, precision=fg.FG_PREC_FP64)
        e1.record(stream)
        e1.synchronize()
        plain_lat.append(e0.elapsed_time(e1) / 1e3)
        plain_iters.append(r[0]["iterations"])
        if i < len(xs_mixed):
            x64 = s.solution()
            plain_err.append(float(np.linalg.norm(xs_mixed[i] - x64) / max(np.linalg.norm(x64), 1e-300)))
    plain_value = nplain / sum(plain_lat)

    # roofline: the batched FP32 EBE matvec alone
    ms_mv, bytes_mv = fg.bench_matvec(systems, precision=32, reps=20)
    peak, peak_kind = peaks()
    achieved = bytes_mv / (ms_mv * 1e-3) / 1e9

    # e2e through the host-buffer C ABI: blocks + F in, X out, every step
    e2e = None
    if not args.no_e2e:
        # inputs in pinned host memory (page-locked: the copies are DMA at
        # full link speed and overlap nothing else of the step)
        keep = []

        def pinned(a):
            t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
            keep.append(t)
            out = t.numpy()
            out[...] = a
            return out

        As, Fs, Xs = [], [], []
        for s, p in zip(systems, probs):
            Fs.append(pinned(s.transport_assemble(p)))
            As.append(pinned(s.get_blocks()))
            Xs.append(pinned(np.zeros(s.n + 1)))
        h2d = sum(a.nbytes for a in As) + sum(f.nbytes for f in Fs)
        d2h = sum(x.nbytes for x in Xs)

        def e2e_step():
            """One served pass of host-buffer requests (fg_server_submit_host):
            each request copies its blocks and F in, is admitted into the
            running batch, and its X is copied out before it is polled."""
            sv = fg.Server(kmax=KMAX, lmax=10000, tol=TOL, precision=served_precision(fg))
            for i, (s, A, F, X) in enumerate(zip(systems, As, Fs, Xs)):
                sv.submit_host(s, A, F, X, i)
            sv.wait(len(systems), timeout=600)
            out = sv.poll(len(systems) + 16)
            sv.close()
            return out

        def e2e_sync_step():
            Bs = []
            for s, A, F in zip(systems, As, Fs):
                s.set_blocks(A)
                Bs.append(s.precond_setup(fg.FG_PRECOND_DIAG, 0, F))
            return fg.solve_batch(systems, Bs, Fs, kmax=KMAX, lmax=10000, tol=TOL, precision=served_precision(fg))

        def timed(fn):
            fn()
            et = []
            for _ in range(max(1, args.steps)):
                torch.cuda.synchronize()
                e0.record(stream)
                out = fn()
                e1.record(stream)
                e1.synchronize()
                et.append(e0.elapsed_time(e1) / 1e3)
            return reduce_max(dist, sum(et) / len(et)), out

        e2e_s, res_h = timed(e2e_step)
        sync_s, _ = timed(e2e_sync_step)
        e2e = {"value": ws * args.count / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "path": "fg_server_submit_host",
               "converged_all": all(r["converged"] == 1 for r in res_h),
               "worst_true_rel_residual": max(r["true_rel_residual"] for r in res_h),
               "synchronous_batch": {"value": ws * args.count / sync_s, "unit": "solves/s",
                                     "path": "fg_set_blocks + fg_precond_setup + fg_solve_batch"}}

    legs = None
    if not args.no_legs and rank == 0:
        jc1 = pool.apply_async(_c1_cpu, (0,)) if pool is not None else None
        jeu = pool.apply_async(_euler_cpu, ((args.euler_n, 1),)) if pool is not None else None
        legs = {"c1_transport": c1_leg(fg, G, jc1),
                "euler_obliquo": euler_leg(fg, G, n=args.euler_n, cpu_job=jeu), "ns_cavity": ns_leg(fg, G, n=args.ns_n),
                "served_mixed_c5": c5_leg(fg, G, count=args.c5_count)}

    cpu = None
    if pool is not None:
        leg = cpu_leg(pool, cores, args.count, args.seed, 2, cpu_k)
        pool.close()
        cpu = {"value": leg["value"], "unit": "solves/s", "cores": cores, "kind": cpu_k, "sample": leg["sample"],
               "p50_ms": 1e3 * pct(leg["lat"], 50), "p99_ms": 1e3 * pct(leg["lat"], 99)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 inner (f16 basis) / f64 refinement" if BASIS == "fp16" else "f32 inner / f64 refinement", "data": "synthetic",
            "config": workload_config(args.count, args.seed),
            "latency_ms": {"p50": 1e3 * pct(lat, 50), "p99": 1e3 * pct(lat, 99),
                           "note": "served, all requests submitted at t=0; latency = done - submit"},
            "served_poisson": poisson, "sync_batch": sync_batch,
            "plain_fp64": {"solves_per_s": plain_value, "instances": nplain, "p50_ms": 1e3 * pct(plain_lat, 50),
                           "p99_ms": 1e3 * pct(plain_lat, 99), "iterations_mean": float(np.mean(plain_iters))},
            "plain_fp64_batched": plain_batched,
            "speedup_vs_plain_fp64": value / plain_value,
            "speedup_vs_plain_fp64_batched": value / plain_batched["solves_per_s"],
            "mixed": {"converged_all": conv, "worst_true_rel_residual": worst_res,
                      "iterations_mean": float(np.mean(iters)),
                      "rel_err_vs_fp64_max": max(plain_err) if plain_err else None},
            "clocks": clocks, "gpu_launches": launches, "launches_before_timed": launches_before_timed, "e2e": e2e,
            "roofline": {"bound": "hbm", "kernel": "k_ebe_mv3p<float,float> (all patch colours, batched)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind, "traffic": MATVEC_TRAFFIC_RATIO * bytes_mv,
                         "traffic_source": "ncu dram__bytes_read+write per matvec of a 32-instance capture "
                                           "(bench.py --matvec-only --count 32), scaled by algorithmic bytes",
                         "ms_per_matvec": ms_mv,
                         "bytes_per_matvec": bytes_mv},
            "cpu_baseline": cpu, "setup_s": setup_s, "legs": legs, "autotune": tuned,
        }
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
