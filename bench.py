#!/usr/bin/env python
"""Throughput of the 2D unstructured Euler residual-and-update path on GB300.

Workload (one "step" = one SSP-RK3 pseudo-time iteration over the whole mesh, including
the per-iteration residual norms, forces and controller): NACA 0012, 512x128 O-grid split
into 131,072 triangles with a seeded diagonal, interior nodes jittered by up to 10% of the
local spacing, cells and faces permuted by the seed; M=0.8, alpha=1.25 deg, HLLC + MUSCL
with the venkat limiter, characteristic far field, local time stepping at CFL 0.8.
Synthetic data generated on the host from a fixed seed.

Metric: Mcell-iter/s = cells x iterations / device seconds, FP32-bulk (headline) and FP64
plain; |dCL| between them after a common number of iterations.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Multi-GPU (torchrun): every rank runs an independent replica (a single case does not
shard); value is the sum over ranks of cells x K divided by the slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "aero-cfd-solver_gb300" / "python"))

import numpy as np  # noqa: E402

METRIC = "Mcell-iter/s FP64 plain vs FP32 batched, |dCL|<1e-4; adjoint/primal time"
WORKLOAD = dict(n_circ=512, n_radial=128, cell_type=3, permute=True, jitter=0.1, seed=2,
                wall_spacing=0.005, farfield_radius=20.0)
CASE = dict(mach=0.8, aoa_deg=1.25, flux=1, limiter=1, precond_farfield_bc=1, cfl_start=0.2, cfl_max=0.8,
            cfl_ramp_iters=120, startup_first_order_iters=25, iterations=5000, min_iterations=5000,
            residual_reduction_target=0.0)
STARTUP = 25  # first-order start-up iterations run untimed before warm-up
E2E_REPEATS = 3  # timed end-to-end runs of K iterations (median reported)

# DRAM traffic of the face pass (dram__bytes_read.sum + dram__bytes_write.sum per launch) comes
# from an ncu capture recorded in profiles/dram_traffic.txt together with a hash of the kernel
# sources it was captured from; a capture of other sources is not reported (traffic null).
TRAFFIC_FILE = REPO / "profiles" / "dram_traffic.txt"
KERNEL_SOURCES = ("aero_face_kernels.cuh", "aero_numerics.cuh", "aero_kernels.cuh")


def kernel_source_hash() -> str:
    import hashlib

    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        h.update((REPO / "aero-cfd-solver_gb300" / "csrc" / name).read_bytes())
    return h.hexdigest()[:16]


def measured_traffic(kernel: str, precision: str, cells: int):
    """(bytes per launch, note) from the recorded capture of the current sources, else (None, why)."""
    if not TRAFFIC_FILE.exists():
        return None, "no capture recorded"
    want = kernel_source_hash()
    stale = False
    for line in TRAFFIC_FILE.read_text().splitlines():
        parts = line.split()
        if len(parts) < 5 or line.startswith("#"):
            continue
        k, prec, n, sha, nbytes = parts[:5]
        if k == kernel and prec == precision and int(n) == cells:
            if sha == want:
                return int(nbytes), f"ncu capture of sources {sha}"
            stale = True
    return None, ("recorded capture is of other kernel sources" if stale else "no capture of this workload")


def algorithmic_bytes(kernel: str, n: int, slots: int, precision: str, faces: int = 0) -> float:
    """Compulsory bytes of one launch: every array element the kernel reads or writes,
    once (neighbour re-reads excluded). s = bulk real size; `slots` per cell."""
    s = 4 if precision == "fp32" else 8
    slot_geo = 4 + 2 * s  # link, face vector
    if kernel == "face":
        # face pass: W and gradients of every cell once; per face its two cell ids, normal,
        # length and MUSCL offsets, and the F*A (4 reals) and wave-speed term it writes
        return n * (4 * s + 8 * s) + faces * (8 + 3 * s + 4 * s + 5 * s)
    if kernel == "gradient":  # W, slot geometry, 1/vol, gradients
        return n * (4 * s + slots * slot_geo + s + 8 * s)
    if kernel == "update":
        # average over the three RK stages: R, SR, U_n (double), stage state / increment
        # (4 reals) read from stage 1 on and written before the last stage, U_n written and the
        # wall flags read in the last stage, W written every stage
        per = [4 * s + s + 32 + 4 * s + 4 * s,
               4 * s + s + 32 + 4 * s + 4 * s + 4 * s,
               4 * s + s + 32 + 4 * s + 32 + 1 + 4 * s]
        return n * sum(per) / 3.0
    raise KeyError(kernel)


def workload_config(args, cells: int, faces: int, world: int) -> dict:
    """`config` of both arms' lines, identical in both: the workload, how the GPU arm's timed
    iterations treat L2, and the replication over ranks. Measured figures go elsewhere."""
    if args.mesh:
        name = f"NACA0012 {args.mesh[0]}x{args.mesh[1]} O-grid (small profiling case)"
    else:
        name = ("NACA0012 512x128 O-grid, 131072 triangles, jitter 10%, permuted; M=0.8, alpha=1.25, "
                "HLLC+MUSCL venkat, RK3 local dt, CFL 0.8")
    return {"workload": name, "cells": cells, "faces": faces,
            "l2": "flushed before every timed iteration (256 MiB write)" if not args.no_flush else "not flushed",
            "parallelism": f"replicas x{world}"}


def measured_peak():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples every 200 ms over a window in which the GPU runs the timed workload.

    The timed steps of the workload last a few milliseconds, less than one sampling period, so
    the caller keeps the GPU on the same iterations (untimed, L2 flushed as in the timed run)
    for LOAD_BEFORE_S before and LOAD_AFTER_S after them: every sample then sees the workload's
    own load and clocks."""

    LOAD_BEFORE_S = 0.8
    LOAD_AFTER_S = 0.4

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return None
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "window": f"{self.LOAD_BEFORE_S:g} s of untimed iterations of the workload, the timed steps, "
                          f"{self.LOAD_AFTER_S:g} s of untimed iterations"}


def keep_busy(solver, seconds: float) -> None:
    """Untimed iterations of the solver (graphs, L2 flushed before each, as in the timed run)
    for about `seconds` of wall time."""
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        solver.time_iterations(200, use_graph=True, flush_l2=True)


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        td.init_process_group(backend=backend)
        dist = td
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_mesh(args):
    import aero_gb300

    w = dict(WORKLOAD)
    if args.mesh:
        w["n_circ"], w["n_radial"] = args.mesh
    return aero_gb300.ogrid_synthetic(**w)


# ------------------------------------------------------------------------------------------
# CPU arms (the oracle port of the reference, bit-identical to it in float mode)
# ------------------------------------------------------------------------------------------
def _cpu_worker(mesh_kw, case_kw, warmup, steps, barrier_, out_q):
    """One single-thread oracle replica (spawned process): builds the workload mesh with the
    oracle's own generator, so that no process of the reference arm loads the product."""
    sys.path.insert(0, str(REPO))
    from oracle import oracle_py as op

    mesh = op.ogrid_synthetic(**mesh_kw)
    sol = op.OracleSolver(op.MODE_FLOAT, mesh, op.make_case(**case_kw))
    sol.run(warmup)
    if barrier_ is not None:
        barrier_.wait()
    t0 = time.perf_counter()
    sol.run(steps)
    out_q.put(time.perf_counter() - t0)


def _cpu_sweep_worker(tasks, warmup, steps, barrier_, out_q):
    """One single-thread oracle process of the sweep's CPU baseline (spawned): its share of the
    96 cases, each built with the oracle's own generator, `warmup` untimed and `steps` timed
    second-order iterations from the free stream. Returns (cell-iterations, seconds)."""
    sys.path.insert(0, str(REPO))
    from oracle import oracle_py as op

    meshes = {}
    sols = []
    for (nc, nr, seed), case_kw in tasks:
        if (nc, nr, seed) not in meshes:
            meshes[(nc, nr, seed)] = op.ogrid_synthetic(nc, nr, cell_type=3, permute=True, jitter=0.1, seed=seed,
                                                        wall_spacing=0.005, farfield_radius=20.0)
        sol = op.OracleSolver(op.MODE_FLOAT, meshes[(nc, nr, seed)], op.make_case(**case_kw))
        sol.run(warmup)
        sols.append((sol, 2 * nc * nr))
    if barrier_ is not None:
        barrier_.wait()
    t0 = time.perf_counter()
    work = 0
    for sol, cells in sols:
        sol.run(steps)
        work += cells * steps
    out_q.put((work, time.perf_counter() - t0))


def c4_cpu_sweep(rank: int, warmup: int = 1, steps: int = 2) -> dict:
    """CPU baseline of the batched sweep: the same 96 cases (sizes, alpha, Mach) in the oracle's
    float mode, bit-identical to the reference CPU path, one single-thread process per host core
    with the cases dealt round-robin; a bounded sample of each case's iterations."""
    import multiprocessing as mp

    from oracle import oracle_py as op

    op.build()
    pick, alphas, machs = c4_draw(rank)
    tasks = []
    for k in range(C4_CASES):
        kw = dict(CASE)
        kw.update(mach=float(machs[k]), aoa_deg=float(alphas[k]), startup_first_order_iters=0)
        nc, nr = C4_SIZES[pick[k]]
        tasks.append(((nc, nr, 100 + int(pick[k])), kw))
    procs_n = max(1, min(os.cpu_count() or 1, C4_CASES))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    bar = ctx.Barrier(procs_n)
    procs = [ctx.Process(target=_cpu_sweep_worker, args=(tasks[i::procs_n], warmup, steps, bar, q))
             for i in range(procs_n)]
    for p in procs:
        p.start()
    res = [q.get() for _ in procs]
    for p in procs:
        p.join()
    work = sum(w for w, _ in res)
    wall = max(t for _, t in res)
    return {"value": work / wall / 1e6, "unit": "Mcell-iter/s", "cores": procs_n, "kind": "port",
            "sample": f"the 96 cases' second-order iterations from the free stream ({warmup} untimed, {steps} "
                      f"timed per case) in the oracle's float mode, bit-identical to the reference CPU path; "
                      f"{procs_n} single-thread processes, cases dealt round-robin; value = all cell-iterations "
                      f"/ the slowest process's time"}


def cpu_sample(mesh, target_s=12.0, max_iters=40, warmup=3):
    """Single-core oracle port on a bounded sample of the workload, the same iterations as each
    replica of the reference arm runs: second-order iterations from the free stream, `warmup`
    of them untimed, then as many as fit in about target_s seconds of CPU work."""
    from oracle import oracle_py as op

    op.build()
    kw = dict(CASE, startup_first_order_iters=0)
    sol = op.OracleSolver(op.MODE_FLOAT, mesh, op.make_case(**kw))
    sol.run(warmup)
    t0 = time.perf_counter()
    sol.run(1)
    one = time.perf_counter() - t0
    n = int(max(1, min(max_iters, target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    sol.run(n)
    dt = time.perf_counter() - t0
    return {"value": mesh.num_cells * n / dt / 1e6, "unit": "Mcell-iter/s", "cores": 1, "kind": "port",
            "sample": f"{n} second-order iterations (after {warmup + 1} untimed) from the free stream of the "
                      f"oracle's float mode (bit-identical to the reference CPU path) on the "
                      f"{mesh.num_cells}-cell workload mesh, 1 thread"}


def run_reference_arm(args):
    """The reference's CPU implementation of the path (the oracle's float mode, bit-identical
    to the compiled reference) on every host core: one single-thread replica per core, each
    running the workload case from its first-order start-up state. Nothing from the product
    package is imported or loaded in any process of this arm."""
    world, rank, local, dist = dist_setup(args)
    if rank != 0:
        return
    import multiprocessing as mp

    from oracle import oracle_py as op

    op.build()
    mesh_kw = dict(WORKLOAD)
    if args.mesh:
        mesh_kw["n_circ"], mesh_kw["n_radial"] = args.mesh
    n = 2 * mesh_kw["n_circ"] * mesh_kw["n_radial"]
    faces = mesh_kw["n_circ"] * (3 * mesh_kw["n_radial"] + 1)
    procs_n = args.cpu_procs if args.cpu_procs > 0 else max(1, os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    bar = ctx.Barrier(procs_n)
    kw = dict(CASE, startup_first_order_iters=0)
    procs = [ctx.Process(target=_cpu_worker, args=(mesh_kw, kw, args.warmup, args.steps, bar, q))
             for _ in range(procs_n)]
    t0 = time.perf_counter()
    for p in procs:
        p.start()
    times = [q.get() for _ in procs]
    for p in procs:
        p.join()
    wall = max(times)
    value = procs_n * n * args.steps / wall / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mcell-iter/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, n, faces, world),
        "cpu_baseline": {"value": value, "unit": "Mcell-iter/s", "cores": procs_n, "kind": "port",
                         "sample": f"{args.steps} second-order iterations per process after {args.warmup} "
                                   f"warm-up, {procs_n} independent single-thread replicas (one per host core) "
                                   f"of the oracle's float mode, which reproduces the reference CPU path bit for "
                                   f"bit (pinned by the oracle tests against the compiled reference); the "
                                   f"GPU host carries no reference sources, so the reference binary itself "
                                   f"is not built there"},
        "e2e": {"value": value, "unit": "Mcell-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "elapsed_s": time.perf_counter() - t0,
    }
    print(json.dumps(line))


# ------------------------------------------------------------------------------------------
# Batched sweep (the AoA/Mach sweep configuration): 96 cases in one batched context
# ------------------------------------------------------------------------------------------
C4_SIZES = [(64, 16), (128, 32), (256, 64), (512, 128)]
C4_CASES = 96


def c4_draw(rank: int):
    """The sweep's cases on one rank (ranks shard the sweep, each with its own seeded draw):
    mesh size index, alpha (deg) and Mach per case."""
    rng = np.random.default_rng(4 + rank)
    pick = rng.integers(0, len(C4_SIZES), C4_CASES)
    alphas = rng.uniform(-4.0, 8.0, C4_CASES)
    machs = rng.uniform(0.3, 0.85, C4_CASES)
    return pick, alphas, machs


def c4_cases(aero_gb300, capi, rank, precision):
    """The sweep's meshes and cases on one rank (C4_CASES of them)."""
    base = {sz: aero_gb300.ogrid_synthetic(sz[0], sz[1], cell_type=3, permute=True, jitter=0.1, seed=100 + i,
                                           wall_spacing=0.005, farfield_radius=20.0)
            for i, sz in enumerate(C4_SIZES)}
    pick, alphas, machs = c4_draw(rank)
    meshes = [base[C4_SIZES[i]] for i in pick]
    cases = []
    for k in range(C4_CASES):
        kw = dict(CASE)
        kw.update(mach=float(machs[k]), aoa_deg=float(alphas[k]))
        c = capi.make_case(**kw, precision=precision)
        c.density_l2_target = 1e-8
        cases.append(c)
    return meshes, cases


def c4_sweep(args, aero_gb300, capi, rank):
    """96 FP32 cases, mesh sizes drawn from the four O-grids, alpha ~ U[-4, 8] deg, M ~
    U[0.3, 0.85], HLLC + MUSCL venkat, per-case CFL ramp to 0.8 and a density-residual stop
    mask at 1e-8 relative; seeded synthetic inputs. Block size, cell ordering and cells per
    thread come from the autotuner (aero_autotune on the largest mesh of the draw with the
    first case's flow). Returns device ms of `steps` iterations (L2 flushed before each), the
    batch's cell count, its launches per iteration, the tuned (ordering, block size, cells
    per thread), the in-graph kernel profile and the context's info."""
    meshes, cases = c4_cases(aero_gb300, capi, rank, capi.PRECISION_FP32)
    largest = max(range(C4_CASES), key=lambda k: meshes[k].num_cells)
    tuned, _ = aero_gb300.autotune(meshes[largest], cases[0], iters=10)
    for c in cases:
        c.block_size = tuned.block_size
        c.ordering = tuned.ordering
        c.cells_per_thread = tuned.cells_per_thread
    with aero_gb300.Batch(meshes, cases) as b:
        cells = b.info()["cells"]
        b.run(STARTUP)
        b.time_iterations(args.warmup, use_graph=True, flush_l2=True)
        ms = b.time_iterations(args.steps, use_graph=True, flush_l2=not args.no_flush)
        info = b.info()
        prof, _ = b.profile_graph(max(3, min(args.steps, 10)), flush_l2=not args.no_flush)
    tuned_t = (int(tuned.ordering), int(tuned.block_size), int(tuned.cells_per_thread))
    return ms, int(cells), int(info["launches_per_iteration"]), tuned_t, prof, info


def kernel_fractions(prof: dict, info: dict, precision: str, peak: float) -> dict:
    """Per kernel class (gradient, face pass, update): algorithmic bytes per launch, the mean
    in-graph launch time, the achieved GB/s and its fraction of the measured HBM peak."""
    n, f, d = int(info["cells"]), int(info["faces"]), int(info["slots_per_cell"])
    out = {}
    for name, kernel in (("gradient", "gradient"), ("face_pass", "face"), ("update", "update")):
        t_ms, cnt = prof[name]
        if not cnt:
            continue
        nbytes = algorithmic_bytes(kernel, n, d, precision, f)
        avg = t_ms / cnt
        gbs = nbytes / (avg / 1e3) / 1e9
        out[name] = {"algorithmic_bytes_per_launch": nbytes, "avg_launch_us": avg * 1e3, "achieved_gbs": gbs,
                     "frac": gbs / peak}
    return out


def batch_roofline(ms_per_step: float, prof: dict, info: dict, peak: float) -> dict:
    """HBM fractions of the batched sweep: its packed working set (4.8 M cells) is far larger
    than L2. The face pass's algorithmic bytes per launch over its in-graph launch time, and
    the algorithmic bytes of a whole iteration (3 gradient passes, 3 face passes, 3 updates)
    over the timed iteration."""
    n, f, d = int(info["cells"]), int(info["faces"]), int(info["slots_per_cell"])
    face = algorithmic_bytes("face", n, d, "fp32", f)
    step = 3 * (algorithmic_bytes("gradient", n, d, "fp32") + face + algorithmic_bytes("update", n, d, "fp32"))
    f_ms, f_n = prof["face_pass"]
    face_ms = f_ms / max(f_n, 1)
    return {"face_pass": {"achieved": face / (face_ms / 1e3) / 1e9, "frac": face / (face_ms / 1e3) / 1e9 / peak,
                          "algorithmic_bytes_per_launch": face, "avg_launch_ms": face_ms},
            "iteration": {"achieved": step / (ms_per_step / 1e3) / 1e9, "frac": step / (ms_per_step / 1e3) / 1e9 / peak,
                          "algorithmic_bytes": step},
            "peak": peak, "unit": "GB/s"}


def c3_low_mach(args, aero_gb300, capi, peak):
    """Low-Mach precision case on the 1024x256 triangulated O-grid (524,288 cells, jittered,
    permuted): preconditioning, low-Mach fix and all-speed flux fix on, characteristic far
    field, HLLC + minmod, alpha=3. At M=0.05: throughput of FP32 and FP64 (L2 flushed before
    each timed iteration) and the face pass's roofline at this size (its working set no longer
    fits in L2). At M=0.05 and M=0.01: |dCL|, |dCD|, max |dCp| at the wall between FP32 and
    FP64 after 400 iterations from free stream. FP32 forms the preconditioned energy row in
    double-float arithmetic below Mach 0.1 (the default); the same figures with the row in
    float, and with the whole preconditioner in IEEE double, are reported beside them."""
    mesh = aero_gb300.ogrid_synthetic(1024, 256, cell_type=3, permute=True, jitter=0.1, seed=3)
    wall = mesh.wall_faces
    mach = 0.05
    res = {}
    legs = (("fp32", capi.PRECISION_FP32, 0), ("fp32_float_precond", capi.PRECISION_FP32, -1),
            ("fp32_fp64_precond", capi.PRECISION_FP32, 1), ("fp64", capi.PRECISION_FP64, 0))
    for prec, code, pfp in legs:
        case = c3_case(capi, code)
        case.precond_fp64 = pfp
        with aero_gb300.Solver(mesh, case) as s:
            info = s.info()
            _, rec = s.run(400)
            p = s.get_primitive()[3]  # the wall pressures after the same 400 iterations as CL, CD
            s.time_iterations(args.warmup, use_graph=True, flush_l2=True)
            ms = s.time_iterations(args.steps, use_graph=True, flush_l2=not args.no_flush)
            prof, graph_ms = s.profile_graph(max(3, min(args.steps, 10)), flush_l2=not args.no_flush)
        f_ms, f_n = prof["face_pass"]
        avg = f_ms / max(f_n, 1)
        nbytes = algorithmic_bytes("face", mesh.num_cells, info["slots_per_cell"], prec[:4], int(info["faces"]))
        res[prec] = dict(mcell=mesh.num_cells * args.steps / (ms / 1e3) / 1e6, cl=float(rec["cl"][-1]),
                         cd=float(rec["cd"][-1]), pw=p[mesh.owner[wall]], face_ms=avg, face_gbs=nbytes / (avg / 1e3) / 1e9,
                         kernels=kernel_times(prof), fractions=kernel_fractions(prof, info, prec[:4], peak))
    q = 0.5 * 1.4 * 101325.0 * mach * mach
    m01 = {}
    for prec, code, pfp in legs:
        case = c3_case(capi, code, 0.01)
        case.precond_fp64 = pfp
        with aero_gb300.Solver(mesh, case) as s:
            _, rec = s.run(400)
            m01[prec] = (float(rec["cl"][-1]), float(rec["cd"][-1]), s.get_primitive()[3][mesh.owner[wall]],
                         float(rec["residual_ratio"][-1]))
    q01 = 0.5 * 1.4 * 101325.0 * 0.01 * 0.01
    mach01 = {"abs_dcl_400": abs(m01["fp32"][0] - m01["fp64"][0]), "abs_dcd_400": abs(m01["fp32"][1] - m01["fp64"][1]),
              "max_abs_dcp_wall_400": float(np.max(np.abs(m01["fp32"][2] - m01["fp64"][2])) / q01),
              "residual_ratio_fp64_400": m01["fp64"][3],
              "float_precond": {"abs_dcl_400": abs(m01["fp32_float_precond"][0] - m01["fp64"][0]),
                                "abs_dcd_400": abs(m01["fp32_float_precond"][1] - m01["fp64"][1])},
              "fp64_precond": {"abs_dcl_400": abs(m01["fp32_fp64_precond"][0] - m01["fp64"][0]),
                               "abs_dcd_400": abs(m01["fp32_fp64_precond"][1] - m01["fp64"][1])},
              "note": "a comparison of two unconverged transients, not a gate result: neither precision "
                      "converges on this case, and float pressure resolves p ~ 1/(gamma M^2) only to ~4e-4 "
                      "of the free-stream dynamic pressure's scale"}
    return {"cells": mesh.num_cells, "mach": mach, "fp32_mcell_iter_s": res["fp32"]["mcell"],
            "accuracy_note": "the 400-iteration figures compare two transients: the case converges in neither "
                             "precision (run to 5,000 iterations, both residual ratios grow to ~10 and the "
                             "precisions separate after ~1,000 iterations)",
            "mach_0.01": mach01,
            "fp64_mcell_iter_s": res["fp64"]["mcell"], "fp32_over_fp64": res["fp32"]["mcell"] / res["fp64"]["mcell"],
            "abs_dcl_400": abs(res["fp32"]["cl"] - res["fp64"]["cl"]),
            "abs_dcd_400": abs(res["fp32"]["cd"] - res["fp64"]["cd"]),
            "max_abs_dcp_wall_400": float(np.max(np.abs(res["fp32"]["pw"] - res["fp64"]["pw"])) / q),
            "precond_energy_row": "double-float below Mach 0.1 (default)",
            **{leg: {"mcell_iter_s": res[leg]["mcell"],
                     "abs_dcl_400": abs(res[leg]["cl"] - res["fp64"]["cl"]),
                     "abs_dcd_400": abs(res[leg]["cd"] - res["fp64"]["cd"]),
                     "max_abs_dcp_wall_400": float(np.max(np.abs(res[leg]["pw"] - res["fp64"]["pw"])) / q),
                     "face_pass_frac": res[leg]["face_gbs"] / peak,
                     "in_graph_kernel_us_per_launch": res[leg]["kernels"]}
               for leg in ("fp32_float_precond", "fp32_fp64_precond")},
            "roofline_face_pass_fp32": {"achieved": res["fp32"]["face_gbs"], "peak": peak, "unit": "GB/s",
                                        "frac": res["fp32"]["face_gbs"] / peak, "avg_launch_ms": res["fp32"]["face_ms"]},
            "roofline_face_pass_fp64": {"achieved": res["fp64"]["face_gbs"], "frac": res["fp64"]["face_gbs"] / peak,
                                        "avg_launch_ms": res["fp64"]["face_ms"]},
            "in_graph_kernel_us_per_launch_fp32": res["fp32"]["kernels"],
            "hbm_fraction_per_kernel_fp32": res["fp32"]["fractions"]}


def c3_case(capi, precision, mach=0.05):
    return capi.make_case(mach=mach, aoa_deg=3.0, flux=capi.FLUX_HLLC, limiter=capi.LIMITER_MINMOD, precond_on=1,
                          low_mach_fix=1, all_speed_flux_fix=1, precond_farfield_bc=1, iterations=100000,
                          min_iterations=100000, cfl_start=0.2, cfl_max=0.8, cfl_ramp_iters=120,
                          startup_first_order_iters=25, precision=precision)


def profile_run(args):
    """One of the measured cases with direct (non-graph) launches, for kernel profilers: 30
    iterations (25 first-order start-up, 5 second-order), then 5 timed second-order iterations.
    workload: the 512x128 single-case workload (FP32); workload_fp64: the same in FP64; c3: the
    1024x256 low-Mach case (FP32)."""
    import aero_gb300
    from aero_gb300 import capi

    aero_gb300.load()
    if args.profile_run == "c3":
        mesh = aero_gb300.ogrid_synthetic(1024, 256, cell_type=3, permute=True, jitter=0.1, seed=3)
        case = c3_case(capi, capi.PRECISION_FP32)
    else:
        mesh = make_mesh(args)
        prec = capi.PRECISION_FP64 if args.profile_run == "workload_fp64" else capi.PRECISION_FP32
        case = capi.make_case(**CASE, precision=prec)
    with aero_gb300.Solver(mesh, case) as s:
        s.time_iterations(30, use_graph=False, flush_l2=False)
        ms = s.time_iterations(5, use_graph=False, flush_l2=True)
    print(json.dumps({"profile_run": {"case": args.profile_run, "cells": mesh.num_cells, "ms_5_iters": ms,
                                      "mcell_iter_s": mesh.num_cells * 5 / ms / 1e3}}))


def c5_adjoint(args, aero_gb300, capi):
    """Adjoint gradient case: triangulated 512x128 O-grid, M=0.75, alpha=2, HLLC, 16 Hicks-Henne
    bumps (8 upper, 8 lower, peaks ~U[0.05, 0.95], width exponent 3, amplitudes ~N(0, 1e-3 c),
    seeded) with inverse-distance-weighted volume deformation; J = CD. The scheme is first
    order throughout: with the reference's second-order limiters the primal stalls at a
    density-residual ratio near 1e-3 and has no steady state to differentiate.
    Primal: FP64 pseudo-time iterations to a density-residual ratio of 1e-8 (and an FP32
    primal to 1e-6 whose state seeds an FP64 adjoint). Adjoint: linearisation, the same RK3
    smoother to a residual reduction of 1e-8, dJ/dalpha and the 16 shape products. Wall-clock
    seconds of each, the primal's host loop included. --c5-fd adds central differences (step
    1e-6 in alpha [deg] and in two amplitudes) of converged primal solutions (ratio 1e-13) on
    the 128x32 grid of the same family, against the adjoint there."""
    from aero_gb300.adjoint import ShapeProblem

    rng = np.random.default_rng(5)
    peaks = rng.uniform(0.05, 0.95, 16)
    upper = np.array([1] * 8 + [0] * 8)
    amps = rng.normal(0.0, 1e-3, 16)
    kw = dict(CASE)
    kw.update(mach=0.75, aoa_deg=2.0, startup_first_order_iters=10 ** 9)
    case = capi.make_case(**kw, precision=capi.PRECISION_FP64)

    def problem(mesh, rho, adj_tol, prec=capi.PRECISION_FP64):
        return ShapeProblem(mesh, case, peaks=peaks, upper=upper, width=3.0, max_iters=400000, rho_target=rho,
                            chunk=20000, adjoint_max_iters=800000, adjoint_tol=adj_tol, adjoint_method="smoother",
                            primal_precision=prec)

    mesh = aero_gb300.ogrid_synthetic(512, 128, cell_type=3, permute=True, jitter=0.1, seed=55)
    prob = problem(mesh, 1e-8, 1e-8)
    base = prob.solve(amps, 2.0)
    da, dal = prob.gradient(base, 1.0, 0.0)
    out = {"cells": mesh.num_cells, "primal_fp64_s": base.seconds, "primal_iters": base.iterations,
           "primal_rho_ratio": base.rho_ratio, "cd": base.cd, "cl": base.cl,
           "adjoint_s": prob.last_adjoint_seconds, "adjoint_iters": prob.last_adjoint_iterations,
           "adjoint_residual_ratio": prob.last_adjoint_ratio,
           "adjoint_over_primal": prob.last_adjoint_seconds / base.seconds,
           "dcd_dalpha_per_deg": dal, "dcd_damp": [float(x) for x in da]}
    base.solver.close()
    prob32 = problem(mesh, 1e-6, 1e-8, capi.PRECISION_FP32)
    b32 = prob32.solve(amps, 2.0)
    da32, dal32 = prob32.gradient(b32, 1.0, 0.0)
    out.update({"primal_fp32_s": b32.seconds, "primal_fp32_iters": b32.iterations,
                "primal_fp32_rho_ratio": b32.rho_ratio, "adjoint_after_fp32_s": prob32.last_adjoint_seconds,
                "fp32_primal_gradient_rel_diff": float(np.linalg.norm(np.append(da32, dal32) - np.append(da, dal)) /
                                                       np.linalg.norm(np.append(da, dal)))})
    b32.solver.close()
    if args.c5_fd:
        small = aero_gb300.ogrid_synthetic(128, 32, cell_type=3, permute=True, jitter=0.1, seed=55)
        pf = problem(small, 1e-13, 1e-12)
        b = pf.solve(amps, 2.0)
        sda, sdal = pf.gradient(b, 1.0, 0.0)
        fd = {"cells": small.num_cells, "primal_rho_ratio": b.rho_ratio, "adjoint_residual_ratio": pf.last_adjoint_ratio}
        b.solver.close()
        h = 1e-6
        for name, e, al in [("alpha", np.zeros(16), h)] + [(f"a{k}", np.eye(16)[k] * h, 0.0) for k in (0, 8)]:
            p, m = pf.solve(amps + e, 2.0 + al), pf.solve(amps - e, 2.0 - al)
            fdv = (p.cd - m.cd) / (2 * h)
            adj = sdal if name == "alpha" else float(sda[int(name[1:])])
            fd[name] = {"adjoint": adj, "central_fd": fdv, "rel_err": abs(adj - fdv) / abs(fdv)}
            p.solver.close()
            m.solver.close()
        out["fd_check_128x32_step_1e-6"] = fd
    return out


# ------------------------------------------------------------------------------------------
# Checks against the FP64 oracle, run in spawned processes on host cores while the GPU legs run
# ------------------------------------------------------------------------------------------
C1_MESH = dict(n_circ=128, n_radial=32, cell_type=4, permute=False, jitter=0.0, seed=1, wall_spacing=0.005,
               farfield_radius=20.0)
C1_CASE = dict(mach=0.5, aoa_deg=2.0, flux=0, limiter=0, cfl_start=0.8, cfl_max=0.8, startup_first_order_iters=10 ** 9,
               iterations=2000, min_iterations=2000, residual_reduction_target=0.0)
C1_ITERS = 2000
C2_ORACLE_ITERS = 100  # 25 first-order start-up iterations and 75 second-order ones


def _oracle_history(tag, mesh_kw, case_kw, iters, out_q):
    """The FP64 oracle's run of a case (spawned process): its CL / CD / CM / residual history
    and wall seconds on one host core."""
    sys.path.insert(0, str(REPO))
    from oracle import oracle_py as op

    mesh = op.ogrid_synthetic(**mesh_kw)
    sol = op.OracleSolver(op.MODE_DOUBLE, mesh, op.make_case(**case_kw))
    t0 = time.perf_counter()
    _, rec = sol.run(iters)
    dt = time.perf_counter() - t0
    out_q.put((tag, {k: rec[k].tolist() for k in ("cl", "cd", "cm", "residual_l2")}, dt, mesh.num_cells))


def start_oracle_checks(enabled: bool):
    """Spawned before the first GPU call: the C1 case (plain FP64 quads, 2,000 iterations) and
    the first 100 iterations of the workload case, both in the FP64 oracle."""
    if not enabled:
        return None
    import multiprocessing as mp

    from oracle import oracle_py as op

    op.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    jobs = [("c1", C1_MESH, dict(C1_CASE), C1_ITERS),
            ("c2", dict(WORKLOAD), dict(CASE), C2_ORACLE_ITERS)]
    procs = [ctx.Process(target=_oracle_history, args=(tag, m, c, n, q)) for tag, m, c, n in jobs]
    for p in procs:
        p.start()
    return q, procs


def collect_oracle_checks(handle) -> dict:
    if handle is None:
        return {}
    q, procs = handle
    out = {}
    for _ in procs:
        tag, hist, dt, cells = q.get(timeout=1800)
        out[tag] = (hist, dt, cells)
    for p in procs:
        p.join()
    return out


def history_diff(rec, hist, n) -> dict:
    return {f"max_abs_d{k}": float(np.max(np.abs(np.asarray(rec[k][:n]) - np.asarray(hist[k][:n]))))
            for k in ("cl", "cd", "cm")}


# ------------------------------------------------------------------------------------------
# GPU legs
# ------------------------------------------------------------------------------------------
def c1_quad(aero_gb300, capi):
    """Plain-FP64 configuration: NACA 0012 on a 128x32 quad O-grid (4,096 cells, cosine
    clustering at the leading and trailing edges, first wall spacing 0.005 c, geometric growth
    to a far field at 20 c), M=0.5, alpha=2 deg, first-order Rusanov, local time stepping at
    CFL 0.8, 2,000 iterations: the records of the run and its device time (graphs, no flush:
    the 1 MB working set lives in L2)."""
    mesh = aero_gb300.ogrid_synthetic(**C1_MESH)
    case = capi.make_case(**C1_CASE, precision=capi.PRECISION_FP64)
    with aero_gb300.Solver(mesh, case) as s:
        t0 = time.perf_counter()
        _, rec = s.run(C1_ITERS)
        wall = time.perf_counter() - t0
    with aero_gb300.Solver(mesh, case) as s:
        ms = s.time_iterations(C1_ITERS, use_graph=True, flush_l2=False)
    return {"cells": mesh.num_cells, "faces": mesh.num_faces, "iterations": C1_ITERS,
            "gpu_fp64_mcell_iter_s": mesh.num_cells * C1_ITERS / (ms / 1e3) / 1e6,
            "gpu_run_with_records_s": wall, "cl": float(rec["cl"][-1]), "cd": float(rec["cd"][-1]),
            "residual_ratio": float(rec["residual_ratio"][-1])}, rec


def wall_cp(mesh, s, case):
    """Cp at the wall faces' owner cells from the primitive state (p - p_inf) / q_inf."""
    p = s.get_primitive()[3][mesh.owner[mesh.wall_faces]]
    q = 0.5 * case.gamma * case.p_inf * case.mach * case.mach
    return (p - case.p_inf) / q


def c2_gate(mesh, aero_gb300, capi):
    """The workload case run for its configured 5,000 iterations from free stream in FP32 and
    FP64: |dCL|, |dCD| and the largest wall |dCp| between them at the end."""
    out = {}
    for prec, code in (("fp32", capi.PRECISION_FP32), ("fp64", capi.PRECISION_FP64)):
        case = capi.make_case(**CASE, precision=code)
        with aero_gb300.Solver(mesh, case) as s:
            t0 = time.perf_counter()
            _, rec = s.run(CASE["iterations"])
            wall = time.perf_counter() - t0
            out[prec] = (rec, wall_cp(mesh, s, case), wall)
    r32, r64 = out["fp32"][0], out["fp64"][0]
    return {"iterations": int(len(r64)), "abs_dcl": abs(float(r32["cl"][-1] - r64["cl"][-1])),
            "abs_dcd": abs(float(r32["cd"][-1] - r64["cd"][-1])),
            "max_abs_dcp_wall": float(np.max(np.abs(out["fp32"][1] - out["fp64"][1]))),
            "cl_fp64": float(r64["cl"][-1]), "cd_fp64": float(r64["cd"][-1]),
            "residual_ratio_fp64": float(r64["residual_ratio"][-1]),
            "residual_ratio_fp32": float(r32["residual_ratio"][-1]),
            "run_s_fp32": out["fp32"][2], "run_s_fp64": out["fp64"][2]}, r64


def c4_accuracy(args, aero_gb300, capi, rank, n_check=8, iters=1000):
    """FP32 batch against FP64 single runs: the sweep's 96 cases run as one FP32 batch for
    `iters` iterations from free stream, and the first n_check of them again, one FP64 context
    each; |dCL| and |dCD| at the end of each case's run (a case stops early at its mask)."""
    meshes, cases = c4_cases(aero_gb300, capi, rank, capi.PRECISION_FP32)
    with aero_gb300.Batch(meshes, cases) as b:
        _, recs = b.run(iters)
    per = []
    for k in range(n_check):
        c64 = capi.make_case(**dict(capi.case_to_dict(cases[k]), precision=capi.PRECISION_FP64))
        with aero_gb300.Solver(meshes[k], c64) as s:
            _, r = s.run(iters)
        per.append({"cells": meshes[k].num_cells, "mach": round(float(cases[k].mach), 4),
                    "alpha": round(float(cases[k].aoa_deg), 4), "iterations_fp32": int(len(recs[k])),
                    "iterations_fp64": int(len(r)), "abs_dcl": abs(float(recs[k]["cl"][-1] - r["cl"][-1])),
                    "abs_dcd": abs(float(recs[k]["cd"][-1] - r["cd"][-1]))})
    return {"iterations": iters, "cases_checked": n_check, "max_abs_dcl": max(p["abs_dcl"] for p in per),
            "max_abs_dcd": max(p["abs_dcd"] for p in per), "per_case": per}


def c5_bounded(aero_gb300, capi):
    """The adjoint configuration's family at a bounded size: 128x32 triangulated O-grid (8,192
    cells), M=0.75, alpha=2, HLLC first order, 16 seeded Hicks-Henne bumps, J = CD. FP64 primal
    to a density-residual ratio of 1e-8, adjoint by the same RK3 smoother to 1e-8, and the
    gradient again from an FP32 primal (ratio 1e-6) whose state seeds the FP64 adjoint."""
    from aero_gb300.adjoint import ShapeProblem

    rng = np.random.default_rng(5)
    peaks = rng.uniform(0.05, 0.95, 16)
    upper = np.array([1] * 8 + [0] * 8)
    amps = rng.normal(0.0, 1e-3, 16)
    kw = dict(CASE)
    kw.update(mach=0.75, aoa_deg=2.0, startup_first_order_iters=10 ** 9)
    case = capi.make_case(**kw, precision=capi.PRECISION_FP64)
    mesh = aero_gb300.ogrid_synthetic(128, 32, cell_type=3, permute=True, jitter=0.1, seed=55)

    def problem(rho, prec):
        return ShapeProblem(mesh, case, peaks=peaks, upper=upper, width=3.0, max_iters=200000, rho_target=rho,
                            chunk=20000, adjoint_max_iters=400000, adjoint_tol=1e-8, adjoint_method="smoother",
                            primal_precision=prec)

    prob = problem(1e-8, capi.PRECISION_FP64)
    base = prob.solve(amps, 2.0)
    da, dal = prob.gradient(base, 1.0, 0.0)
    base.solver.close()
    out = {"cells": mesh.num_cells, "bumps": 16, "scheme": "HLLC first order", "primal_fp64_s": base.seconds,
           "primal_iters": base.iterations, "primal_rho_ratio": base.rho_ratio, "cd": base.cd, "cl": base.cl,
           "adjoint_s": prob.last_adjoint_seconds, "adjoint_iters": prob.last_adjoint_iterations,
           "adjoint_residual_ratio": prob.last_adjoint_ratio,
           "adjoint_over_primal": prob.last_adjoint_seconds / base.seconds,
           "dcd_dalpha_per_deg": dal, "dcd_damp_norm": float(np.linalg.norm(da))}
    p32 = problem(1e-6, capi.PRECISION_FP32)
    b32 = p32.solve(amps, 2.0)
    da32, dal32 = p32.gradient(b32, 1.0, 0.0)
    b32.solver.close()
    ref = np.append(da, dal)
    out.update({"primal_fp32_s": b32.seconds, "primal_fp32_iters": b32.iterations,
                "fp32_primal_gradient_rel_diff": float(np.linalg.norm(np.append(da32, dal32) - ref) /
                                                       np.linalg.norm(ref))})
    return out


def kernel_times(prof: dict) -> dict:
    return {k: (v[0] / v[1] * 1e3 if v[1] else 0.0) for k, v in prof.items()}


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def run_gpu_arm(args):
    world, rank, local, dist = dist_setup(args)
    checks = start_oracle_checks(rank == 0 and world == 1 and not args.no_cpu and not args.mesh)
    import aero_gb300
    from aero_gb300 import capi

    aero_gb300.load()
    aero_gb300.select_device(local)
    mesh = make_mesh(args)
    n = mesh.num_cells
    precisions = ["fp32", "fp64"] if args.precision == "both" else [args.precision]
    results = {}
    peak, peak_kind = measured_peak()
    nprof = max(3, min(args.steps, 10))
    for prec in precisions:
        pcode = capi.PRECISION_FP32 if prec == "fp32" else capi.PRECISION_FP64
        case = capi.make_case(**CASE, precision=pcode)
        with aero_gb300.Solver(mesh, case) as s:
            info = s.info()
            s.run(STARTUP)
            s.time_iterations(args.warmup, use_graph=True, flush_l2=True)
            barrier(dist)
            sampler = ClockSampler(local) if prec == "fp32" and not args.no_clocks else None
            if sampler:
                sampler.__enter__()
                u_start = s.get_state()
                keep_busy(s, ClockSampler.LOAD_BEFORE_S)
                s.set_state(u_start)  # the timed steps start from the warmed-up flow, as without the load
            ms = s.time_iterations(args.steps, use_graph=True, flush_l2=not args.no_flush)
            if sampler:
                keep_busy(s, ClockSampler.LOAD_AFTER_S)
                sampler.__exit__(None, None, None)
            barrier(dist)
            ms_max = reduce_max(dist, ms)
            warm_ms = s.time_iterations(args.steps, use_graph=True, flush_l2=False)
            graph_prof, graph_ms = s.profile_graph(nprof, flush_l2=not args.no_flush)
            prof = s.profile_kernels(nprof, flush_l2=not args.no_flush)
            state = s.get_state() if prec == "fp32" else None
            finite = bool(np.all(np.isfinite(s.get_state())))
        value = world * n * args.steps / (ms_max / 1e3) / 1e6
        f_ms, f_n = graph_prof["face_pass"]
        avg_face = f_ms / max(f_n, 1)
        bytes_face = algorithmic_bytes("face", n, info["slots_per_cell"], prec, int(info["faces"]))
        main_ms = sum(v[0] for k, v in graph_prof.items() if k != "control")
        in_graph = {"us_per_launch": kernel_times(graph_prof),
                    "hbm_fraction_per_kernel": kernel_fractions(graph_prof, info, prec, peak),
                    "launches_per_iteration": {k: v[1] / nprof for k, v in graph_prof.items()},
                    "us_per_iteration": {k: v[0] / nprof * 1e3 for k, v in graph_prof.items()},
                    "kernels_on_main_stream_us_per_iteration": main_ms / nprof * 1e3,
                    "iteration_us_while_traced": graph_ms / nprof * 1e3,
                    "untraced_step_us": ms_max / args.steps * 1e3,
                    "launch_gaps_us_per_iteration": ms_max / args.steps * 1e3 - main_ms / nprof * 1e3,
                    "note": "kernel start/end recorded by CUPTI inside the timed iteration graphs (L2 flushed "
                            "before each iteration as in the timed run); the main-stream kernels run one after "
                            "another, the controller on a side stream beside the next iteration's first "
                            "kernels; the untraced step time minus the main-stream kernels is the launch gaps"}
        results[prec] = dict(value=value, ms=ms_max, warm_ms=warm_ms, info=info, state=state, finite=finite,
                             achieved=bytes_face / (avg_face / 1e3) / 1e9, avg_face_ms=avg_face, bytes_face=bytes_face,
                             share=f_ms / main_ms if main_ms else None, in_graph=in_graph,
                             isolated=kernel_times(prof), clocks=sampler.summary() if sampler else None)
    head = results[precisions[0]]

    # end to end through the C ABI with host buffers: upload the state, run K iterations
    # with every iteration's record copied to the host, download the state
    e2e = None
    if head["state"] is not None or precisions[0] == "fp64":
        pcode = capi.PRECISION_FP32 if precisions[0] == "fp32" else capi.PRECISION_FP64
        with aero_gb300.Solver(mesh, capi.make_case(**CASE, precision=pcode)) as s:
            u0 = s.get_state() if head["state"] is None else head["state"]
            # untimed warm-up through the same calls: the start-up iterations and W
            # second-order iterations (this instantiates the iteration graphs)
            s.run(STARTUP + args.warmup)
            u1 = np.empty_like(u0)  # the caller's result buffer, reused across calls
            s.set_state(u0)
            s.get_state(out=u1)
            # three timed runs of K iterations from the same state; the median is reported
            dts = []
            for _ in range(E2E_REPEATS):
                barrier(dist)
                t0 = time.perf_counter()
                s.set_state(u0)
                _, rec = s.run(args.steps)
                s.get_state(out=u1)
                dts.append(time.perf_counter() - t0)
            barrier(dist)
        dt = reduce_max(dist, statistics.median(dts))
        rec_bytes = len(rec) * rec.dtype.itemsize
        e2e = {"value": world * n * args.steps / dt / 1e6, "unit": "Mcell-iter/s",
               "h2d_bytes_per_step": int(u0.nbytes / args.steps),
               "d2h_bytes_per_step": int((rec_bytes + u1.nbytes) / args.steps),
               "runs": E2E_REPEATS, "statistic": "median of the runs' wall times",
               "run_values": [world * n * args.steps / x / 1e6 for x in dts]}

    c4 = None
    if not args.no_c4 and "fp32" in precisions:
        barrier(dist)
        c4_ms, c4_cells, c4_launch, c4_tuned, c4_prof, c4_info = c4_sweep(args, aero_gb300, capi, rank)
        c4_ms = reduce_max(dist, c4_ms)
        c4 = {"cases_per_gpu": C4_CASES, "cells_per_gpu": c4_cells, "steps": args.steps,
              "ms_per_step": c4_ms / args.steps,
              "fp32_batched_mcell_iter_s": world * c4_cells * args.steps / (c4_ms / 1e3) / 1e6,
              "launches_per_step": c4_launch,
              "in_graph_kernel_us_per_launch": kernel_times(c4_prof),
              "hbm_fraction_per_kernel": kernel_fractions(c4_prof, c4_info, "fp32", peak),
              "roofline": batch_roofline(c4_ms / args.steps, c4_prof, c4_info, peak),
              "autotuned": {"ordering": {1: "morton", 2: "rcm"}.get(c4_tuned[0], c4_tuned[0]),
                            "block_size": c4_tuned[1], "cells_per_thread": c4_tuned[2]},
              "inputs": "96 seeded cases per GPU: sizes from {64x16,128x32,256x64,512x128} triangulated "
                        "O-grids, alpha~U[-4,8], M~U[0.3,0.85], HLLC+MUSCL venkat, CFL ramp to 0.8, "
                        "density-residual stop mask 1e-8; one batched context, L2 flushed per step"}
        if rank == 0 and not args.mesh:
            c4["fp32_batch_vs_fp64_single"] = c4_accuracy(args, aero_gb300, capi, rank)
        if rank == 0 and world == 1 and not args.no_cpu and not args.mesh:
            c4["cpu_baseline"] = c4_cpu_sweep(rank)

    gate = c1 = c3 = c5 = None
    gate_rec64 = c1_rec = None
    if rank == 0 and not args.mesh:
        if "fp32" in precisions and "fp64" in precisions:
            gate, gate_rec64 = c2_gate(mesh, aero_gb300, capi)
        c1, c1_rec = c1_quad(aero_gb300, capi)
        if not args.no_c3:
            c3 = c3_low_mach(args, aero_gb300, capi, peak)
        if not args.no_c5:
            c5 = c5_adjoint(args, aero_gb300, capi) if args.c5 or args.c5_fd else c5_bounded(aero_gb300, capi)

    oracle = collect_oracle_checks(checks)
    if "c1" in oracle and c1 is not None:
        hist, dt, cells = oracle["c1"]
        c1.update(history_diff(c1_rec, hist, C1_ITERS))
        c1.update({"cpu_oracle_fp64_mcell_iter_s": cells * C1_ITERS / dt / 1e6, "cpu_oracle_cores": 1,
                   "cpu_oracle_s": dt})
    if "c2" in oracle and gate is not None:
        hist, dt, cells = oracle["c2"]
        gate["fp64_gpu_vs_fp64_cpu_oracle"] = dict(iterations=C2_ORACLE_ITERS,
                                                   **history_diff(gate_rec64, hist, C2_ORACLE_ITERS),
                                                   cpu_oracle_fp64_mcell_iter_s=cells * C2_ORACLE_ITERS / dt / 1e6)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu and head["state"] is not None:
        cpu = cpu_sample(mesh)

    if rank != 0:
        return
    r32 = results.get("fp32")
    r64 = results.get("fp64")
    traffic, traffic_note = measured_traffic("face_pass", precisions[0], n)
    config = workload_config(args, n, int(head["info"]["faces"]), world)
    measurements = {
        "precision_headline": precisions[0],
        "timing": "CUDA events on the library stream, CUDA graph per iteration",
        "fp32_mcell_iter_s": r32["value"] if r32 else None,
        "fp64_mcell_iter_s": r64["value"] if r64 else None,
        "fp32_over_fp64": (r32["value"] / r64["value"]) if (r32 and r64) else None,
        "fp32_l2_warm_mcell_iter_s": world * n * args.steps / (r32["warm_ms"] / 1e3) / 1e6 if r32 else None,
        "fp64_l2_warm_mcell_iter_s": world * n * args.steps / (r64["warm_ms"] / 1e3) / 1e6 if r64 else None,
        "in_graph_kernels": {p: results[p]["in_graph"] for p in precisions},
        "isolated_kernel_us_per_launch": {p: results[p]["isolated"] for p in precisions},
        "c2_gate": gate,
        "c1": c1,
        "c4_batched_sweep": c4,
        "c3_low_mach": c3,
        "c5_adjoint": c5,
        "state_finite": head["finite"],
    }
    line = {
        "metric": METRIC, "value": head["value"], "unit": "Mcell-iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if precisions[0] == "fp32" else "f64", "data": "synthetic",
        "config": config,
        "roofline": {"bound": "hbm", "kernel": "k_face_flux (MUSCL reconstruction + HLLC flux, one thread per face)",
                     "achieved": head["achieved"], "peak": peak, "unit": "GB/s", "frac": head["achieved"] / peak,
                     "peak_kind": peak_kind, "traffic": traffic, "traffic_source": traffic_note,
                     "algorithmic_bytes_per_launch": head["bytes_face"], "avg_launch_ms": head["avg_face_ms"],
                     "launch_time": "kernel duration inside the timed iteration graphs (CUPTI)",
                     "time_share": head["share"]},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(head["info"]["launches_per_iteration"]) * args.steps,
        "clocks": head["clocks"],
        "measurements": measurements,
    }
    if r64 and precisions[0] == "fp32":
        line["roofline_fp64"] = {"achieved": r64["achieved"], "frac": r64["achieved"] / peak,
                                 "avg_launch_ms": r64["avg_face_ms"]}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--precision", choices=["fp32", "fp64", "both"], default="both")
    ap.add_argument("--mesh", type=int, nargs=2, default=None, help="n_circ n_radial of a smaller mesh")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-flush", action="store_true")
    ap.add_argument("--no-clocks", action="store_true")
    ap.add_argument("--no-c4", action="store_true", help="skip the 96-case batched sweep measurement")
    ap.add_argument("--cpu-procs", type=int, default=0, help="processes of the reference arm (0: all cores)")
    ap.add_argument("--no-c3", action="store_true", help="skip the 524k-cell low-Mach measurement")
    ap.add_argument("--profile-run", choices=["workload", "workload_fp64", "c3"], default=None,
                    help="only run one case with direct launches (for kernel profilers)")
    ap.add_argument("--no-c5", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--c5", action="store_true",
                    help="the adjoint leg on the configured 512x128 grid instead of the bounded 128x32 one")
    ap.add_argument("--c5-fd", action="store_true", help="--c5 plus central differences for alpha and two bumps")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.profile_run:
        profile_run(args)
    elif args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
