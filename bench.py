#!/usr/bin/env python
"""Benchmark: body-steps/s of the GPU rigid-body step on a 262,144-box pile.

Workload (both arms): 64x64 columns of 64 unit boxes (8-vertex hulls, half extent 0.5, mass 1)
resting on a static plane -- the settled form of the 64^3 lattice pile (x/z spacing 1.1,
jitter +-0.05, seed 0) -- PGS solver, 10 iterations, dt 1/60, gravity -9.8.  One step =
stepSimulation: AABBs, grid broadphase, narrowphase, colouring, PGS solve, integration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload pile|batched|stress]

The line also carries `configurations` (rank 0, one GPU, pile workload): the other benchmark
configurations at full size, device-timed in the same run -- collision at scale (131,072 mixed
bodies), batched scenes (4,096 scenes) and the million-body pour (1,048,576 bodies, 600 steps).

And `to_residual` (rank 0, one GPU, pile workload): every PGS solve run to a
1e-4 contact residual, once per warm-start mode (plain = cold start, learned, persistent,
persistent + learned), with the mean sweeps, solve ms and step ms per step of each, on two
workloads: the falling 64^3 lattice (spacing 1.1, jitter 0.05) and 512 held-out batched piles.  --workload batched times 4,096
independent scenes (counts log-uniform in [8, 256]) stepped together through per-scene offset
tables instead of the pile.

--impl reference times the reference's CPU algorithm for the same step (the composed CPU step:
b3TransformAabb2, exact pair set, b3ContactConvexConvexSAT / computeContactPlaneConvex,
b3PgsJacobiSolver, integrateSingleTransform) through the plain-C oracle restatement (pinned
bit-for-bit to the reference's own code by tests/test_oracle_golden.py), with every host thread
the oracle can use.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "body-steps/s at 256k bodies"
WORKLOAD = ("box pile 64x64x64 = 262,144 unit boxes resting in 64x64 columns on a static plane "
            "(settled form of the spacing-1.1 jitter-0.05 lattice, seed 0), PGS 10 iterations, dt 1/60")
WORKLOAD_BATCHED = ("{n} independent scenes (body counts log-uniform in [8, 256], seed 0; {bodies} bodies), each a "
                    "jittered box/sphere pile (spacing 1.1, base 0.6, jitter 0.01) on its own plane, all at the "
                    "origin, stepped together through per-scene offset tables, PGS 10 iterations, dt 1/60")
WORKLOAD_STRESS = ("{bodies} bodies: 1,048,576 mixed convex bodies (50% boxes, 25% spheres, 25% Gaussian hulls, "
                   "random orientations, zero velocity) poured from heights U[0, 512] into a 128x64x128 container of "
                   "5 static planes; PGS to a 1e-4 residual with a 16-sweep cap, persistent + learned warm start with "
                   "the cold fallback, graph-captured step; timed steps {first}..{last} of the 600-step pour")
PILES_WORKLOAD = ("512 batched box/sphere piles (counts log-uniform in [8, 256], {bodies} bodies, seed 1007, not a "
                  "training seed) falling onto a shared plane, steps 20..79, every PGS solve run to a {tol:g} contact "
                  "residual (at most {cap} sweeps)")
RESIDUAL_WORKLOAD = ("box pile lattice 64x64x64 = 262,144 unit boxes (spacing 1.1, jitter 0.05, seed 0) falling onto "
                     "a static plane from rest, steps 0..{last}, every PGS solve run to a {tol:g} contact residual "
                     "(at most {cap} sweeps)")


def solver_mode_code(args):
    """Oracle solver mode: 0 PGS (contact rows then friction rows), 1 Jacobi, 2 PGS with rows
    interleaved per contact point (B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_CONSTRAINTS)."""
    if args.solver != "pgs":
        return 1
    return 2 if args.row_order == "interleaved" else 0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None, help="timed steps (default 30; stress: 597)")
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--nx", type=int, default=64)
    p.add_argument("--cpu-steps", type=int, default=3)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--solver", choices=["pgs", "jacobi"], default="pgs")
    p.add_argument("--iterations", type=int, default=10)
    p.add_argument("--row-order", choices=["interleaved", "separate"], default="interleaved",
                   help="PGS row order: per contact point (reference B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_"
                        "CONSTRAINTS mode) or all contact rows then all friction rows (reference default)")
    p.add_argument("--workload", choices=["pile", "batched", "stress"], default="pile",
                   help="pile: the 262,144-box pile; batched: independent scenes stepped together; stress: "
                        "1,048,576 mixed bodies poured into a 5-plane container")
    p.add_argument("--settle", type=int, default=None,
                   help="untimed steps before the warm-up (default: 120 for batched, so the piles have landed; 0 otherwise)")
    p.add_argument("--scenes", type=int, default=4096, help="number of scenes of the batched workload")
    p.add_argument("--residual-steps", type=int, default=60,
                   help="steps of the falling 64^3 lattice solved to the residual, per warm-start mode (0 = skip)")
    p.add_argument("--residual-cap", type=int, default=4000)
    p.add_argument("--residual-tol", type=float, default=1e-4)
    p.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    p.add_argument("--no-configurations", action="store_true",
                   help="skip the other configurations (collision at scale, batched scenes, million-body pour)")
    p.add_argument("--no-pour", action="store_true", help="skip the million-body pour among the other configurations")
    a = p.parse_args()
    if a.steps is None:
        a.steps = 597 if a.workload == "stress" else 30
    if a.settle is None:
        a.settle = 120 if a.workload == "batched" else 0
    if a.workload == "stress":
        a.iterations = 16
    return a


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def dist_init(world):
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
        return dist
    return None


def dist_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def solve_kernels(tuning) -> str:
    """The solve stage's kernels for the PGS work split that ran (the autotuner's choice, else the
    library's rule for AUTO: grid-wide colours)."""
    split = (tuning or {}).get("pgs_partitions", -1)
    if split in (-1, 0, 2):  # AUTO rule / B3G_PGS_PARTITIONS_NONE
        return ("solve stage: k_manifold_prep + k_colour (colouring) + k_setup_rows (rows in colour order) "
                "+ k_pgs_sweeps (persistent, a grid barrier per colour)")
    return "solve stage: k_setup_rows + k_solve_pgs (persistent, block partitions)"


def solver_traffic():
    """DRAM bytes per manifold of the solve stage's kernels from a committed ncu capture (ncu cannot
    run inside this measurement): the file names the command, workload and launch shapes of the
    capture, which the roofline object repeats beside the scaled figure."""
    p = ROOT / "profiles" / "solver_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


def scene_seed(args, rank: int) -> int:
    """Seed of a rank's scene set: under torchrun the batched workload gives every rank its own
    scenes (seed = rank: independent scenes, no exchange between ranks, per-GPU work fixed); the
    single-scene workloads run the same scene on every rank (replicas)."""
    return rank if args.workload == "batched" else 0


def make_scene(args, rank: int = 0):
    from bullet3_gb300 import scenes
    if args.workload == "batched":
        return scenes.batched_piles(args.scenes, seed=scene_seed(args, rank), separate=True)
    if args.workload == "stress":
        return scenes.stress_container(1048576, seed=0)
    return scenes.box_stack(args.nx, 64, args.nx, seed=0)


def workload_name(args, scene):
    if args.workload == "batched":
        return WORKLOAD_BATCHED.format(n=args.scenes, bodies=scene.num_bodies) + f", steps {args.settle + args.warmup}.."
    if args.workload == "stress":
        return WORKLOAD_STRESS.format(bodies=scene.num_bodies, first=args.warmup, last=args.warmup + args.steps - 1)
    return WORKLOAD


# ------------------------------------------------------------------------------ CPU arm
CPU_KIND = ("the oracle's composed step (the reference CPU algorithms, pinned bit for bit to the compiled "
            "reference; exact pair set from a uniform-grid search, which is the set the reference's dynamic-BVH "
            "broadphase gives after its tight AABB test) with OpenMP over bodies and pairs, {threads} threads; "
            "the PGS sweep is sequential, as in the reference; the reference's own CPU pipeline is single-threaded")


def bench_config(args, scene, world: int = 1) -> dict:
    """The configuration both arms report (identical keys and values for the same workload)."""
    return {"workload": workload_name(args, scene), "bodies": int(scene.num_bodies), "solver": args.solver,
            "iterations": args.iterations, "row_order": args.row_order,
            "parallelism": (f"{world} ranks, own scene set each (seed = rank)"
                            if world > 1 and args.workload == "batched"
                            else f"replicas x{world}" if world > 1 else "single GPU"),
            "l2": "inputs larger than L2 (constraint rows and pair buffers exceed 129 MB)"}


def cpu_tables(scene):
    """The scene's shape, body and inertia tables, registered by the oracle's restatement of the
    reference's registration (oracle/b3hull.c): the CPU legs load nothing of the product."""
    from oracle import oracle as O
    return O.register_scene(scene)


def cpu_run(scene, tables, steps, iterations, mode):
    """Times `steps` composed oracle steps on the scene; returns (seconds, threads, bodies)."""
    from oracle import oracle as O
    t = tables
    shapes = O.Shapes.from_tables(t)
    threads = O.max_threads()
    b, I = t["bodies"], t["inertias"]
    first = getattr(scene, "scene_first", None)
    if first is not None:
        # independent scenes: the reference steps one pipeline per scene; the scenes are spread over
        # the host threads, each stepped by the single-threaded oracle
        from concurrent.futures import ThreadPoolExecutor
        O.set_threads(1)
        n = len(b)
        ranges = [(int(a), int(first[k + 1]) if k + 1 < len(first) else n) for k, a in enumerate(first)]
        parts = [(b[a:e].copy(), I[a:e].copy()) for a, e in ranges]

        def one(k):
            bb, II = parts[k]
            for _ in range(steps):
                bb, _, _, _ = O.step(bb, II, shapes, mode=mode, iterations=iterations, cell=1.7320508, use_grid=True)
            return k

        t0 = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, range(len(parts))))
        return time.perf_counter() - t0, threads, scene.num_bodies
    O.set_threads(threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        b, nc, npairs, npts = O.step(b, I, shapes, mode=mode, iterations=iterations, cell=1.7320508, use_grid=True)
    return time.perf_counter() - t0, threads, scene.num_bodies


def reference_arm(args):
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    scene = make_scene(args)
    mode = solver_mode_code(args)
    tables = cpu_tables(scene)
    # warm-up steps are run (untimed) from the same initial state; each timed step is one full
    # composed CPU step of the whole 262,144-body scene
    # (the million-body pour is sampled: at most 3 timed CPU steps, as its CPU baseline is)
    steps = args.steps if args.workload != "stress" else min(args.steps, 3)
    cpu_run(scene, tables, args.warmup, args.iterations, mode) if args.warmup else None
    secs, threads, n = cpu_run(scene, tables, steps, args.iterations, mode)
    value = n * steps / secs
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args, scene, world),
            "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{steps} composed CPU steps of the full {n}-body scene: "
                                       + CPU_KIND.format(threads=threads)},
            "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------ learned vs plain
def _residual_modes(sc, args, device, net, steps, first):
    """Mean sweeps / solve ms / step ms per step over steps [first, steps) for each warm-start mode,
    every mode stepped from the same initial state."""
    import numpy as np

    from bullet3_gb300 import capi, scenes
    from bullet3_gb300.pipeline import b3Config
    modes = {"plain": capi.WARM_COLD, "learned": capi.WARM_LEARNED, "persistent": capi.WARM_PERSISTENT,
             "persistent_learned": capi.WARM_PERSISTENT_LEARNED}
    out = {}
    for name, code in modes.items():
        cfg = b3Config(solver_mode=capi.SOLVER_PGS, solver_iterations=args.residual_cap,
                       residual_tol=args.residual_tol, pgs_interleave=True, warm_start=code, use_cuda_graph=True)
        np_, bp, pl = scenes.load_scene(sc, cfg, device=device)
        if code in (capi.WARM_LEARNED, capi.WARM_PERSISTENT_LEARNED):
            pl.setWarmStartModel(net)
        pl.setProfiling(True)
        sweeps, solve_ms, step_ms, dropped, capped = [], [], [], 0, 0
        for step in range(steps):
            pl.stepSimulation(1.0 / 60.0)
            pl.synchronize()
            st = pl.stats()
            t = pl.stageTimes()
            if step >= first:
                sweeps.append(st.iterations)
                solve_ms.append(float(t[4]))
                step_ms.append(float(np.sum(t)))
                dropped += bool(st.status & capi.FLAG_WARM_DISCARDED)
                capped += st.iterations >= args.residual_cap
            pl.status(clear=True)
        pl.setProfiling(False)
        out[name] = {"sweeps_per_step": float(np.mean(sweeps)), "solve_ms_per_step": float(np.mean(solve_ms)),
                     "step_ms": float(np.mean(step_ms)), "steps_at_cap": int(capped), "fallback_steps": int(dropped),
                     "manifolds_last_step": int(st.num_contacts)}
        del np_, bp, pl
    base = out["plain"]
    for name in ("learned", "persistent", "persistent_learned"):
        out[name]["sweeps_vs_plain"] = out[name]["sweeps_per_step"] / max(base["sweeps_per_step"], 1e-9)
        out[name]["solve_ms_vs_plain"] = out[name]["solve_ms_per_step"] / max(base["solve_ms_per_step"], 1e-9)
    return out


def to_residual(args, device):
    """Sweeps and solve time per step when every solve runs to the residual target, per warm-start
    mode: plain (cold start, the reference's solver), learned (the network predicts every point),
    persistent (points matched to the previous step's manifolds start from their converged
    impulses) and persistent + learned (the network predicts the new points).  Two workloads: the
    falling 64^3 lattice, and held-out batched piles like the ones the network was trained on
    (seeds it never saw).  A warm start whose first sweep is worse than a cold start is dropped and
    counted in `fallback_steps`."""
    from bullet3_gb300 import scenes
    from bullet3_gb300.warmstart import DEFAULT_WEIGHTS, WarmStartMLP
    net = WarmStartMLP.load(DEFAULT_WEIGHTS)
    lattice = scenes.box_pile(args.nx, 64, args.nx, jitter=0.05, seed=0)
    piles = scenes.batched_piles(512, seed=1007)
    return {"tol": args.residual_tol, "cap": args.residual_cap,
            "residual": "||lambda_k - lambda_k-1||_2 / ||lambda_k||_2 over all contact and friction rows, per sweep",
            "lattice": {"workload": RESIDUAL_WORKLOAD.format(last=args.residual_steps - 1, tol=args.residual_tol,
                                                             cap=args.residual_cap),
                        "modes": _residual_modes(lattice, args, device, net, args.residual_steps, 0)},
            "held_out_piles": {"workload": PILES_WORKLOAD.format(bodies=piles.num_bodies, tol=args.residual_tol,
                                                                 cap=args.residual_cap),
                               "modes": _residual_modes(piles, args, device, net, 80, 20)}}


# ------------------------------------------------------------------------------ other configurations
def _stage_fracs(acc, N, st, peak):
    C_, I_, P_ = st.num_contacts, max(1, st.iterations), st.num_pairs
    stage_bytes = {"aabb": 56 * N, "pairs": 112 * N + 8 * P_, "contacts": 64 * P_ + 88 * C_,
                   "solve": C_ * (416 + 16 + 24) + 352 * C_ * I_, "integrate": 116 * N}
    stage_ms = {"aabb": acc[0], "pairs": acc[1], "contacts": acc[2], "solve": acc[4], "integrate": acc[6]}
    return {k: {"ms": float(v), "frac_of_hbm": (stage_bytes[k] / (v / 1000.0) / 1e9 / peak) if v > 0 else None}
            for k, v in stage_ms.items()}


def _time_config(sc, cfg, device, settle, steps, warm_model=None, profile_steps=2):
    """Device-timed steps of one configuration: body-steps/s, ms/step, per-stage times after."""
    import ctypes as C

    import numpy as np

    from bullet3_gb300 import capi, scenes
    dt = 1.0 / 60.0
    t_load = time.perf_counter()
    np_, bp, pl = scenes.load_scene(sc, cfg, device=device)
    t_load = time.perf_counter() - t_load
    if warm_model is not None:
        pl.setWarmStartModel(warm_model)
    for _ in range(settle):
        pl.stepSimulation(dt)
    pl.synchronize()
    tuning = pl.autotune(dt, repeats=2)
    h = np_.world.handle
    pl.status(clear=True)
    capi.call("b3g_record_event", h, C.c_int(2))
    for _ in range(steps):
        pl.stepSimulation(dt)
    capi.call("b3g_record_event", h, C.c_int(3))
    ms = C.c_float()
    capi.call("b3g_event_elapsed", h, C.c_int(2), C.c_int(3), C.byref(ms))
    pl.synchronize()
    status = pl.status()
    pl.setProfiling(True)
    acc = np.zeros(7)
    for _ in range(profile_steps):
        pl.stepSimulation(dt)
        acc += pl.stageTimes()
    pl.setProfiling(False)
    st = pl.stats()
    peak, _ = measured_peaks()
    N = sc.num_bodies
    out = {"bodies": int(N), "steps_timed": steps, "first_timed_step": settle,
           "value": N * steps / (ms.value / 1000.0), "unit": "body-steps/s", "ms_per_step": ms.value / steps,
           "pairs": st.num_pairs, "manifolds": st.num_contacts, "colors": st.num_colors,
           "stages_after": _stage_fracs(acc / profile_steps, N, st, peak), "device_status": int(status),
           "registration_s": t_load, "broadphase": "lbvh" if tuning and tuning.get("broadphase") == 1 else "grid"}
    del np_, bp, pl
    return out


def other_configurations(args, device):
    """The benchmark's other configurations at full size, device-timed in the same run (graph-captured
    steps, launch shapes autotuned after the settle): collision at scale (131,072 mixed bodies,
    steps 3..63 of 64), batched scenes (4,096 scenes, 30 steps after 120 settle steps), the 64^3
    lattice while it falls and settles (steps 60..119, PGS 10 iterations) and the million-body pour
    (steps 3..599 of 600, PGS to 1e-4 with a 16-sweep cap, persistent + learned warm start)."""
    from bullet3_gb300 import capi, scenes
    from bullet3_gb300.pipeline import b3Config
    out = {}
    sc = scenes.mixed_scene(131072, extent=64.0, seed=0)
    cfg = b3Config(solver_mode=capi.SOLVER_PGS, solver_iterations=10, use_cuda_graph=True, pgs_interleave=True,
                   broadphase=capi.BROADPHASE_AUTO)
    out["collision_at_scale"] = dict(
        workload="131,072 bodies (50% boxes, 25% spheres, 25% Gaussian hulls) uniform in a 64^3 box, random "
                 "orientations, N(0,1) velocities, grid cell 2x the largest AABB extent, PGS 10 iterations",
        **_time_config(sc, cfg, device, settle=3, steps=61))
    sc = scenes.batched_piles(args.scenes, seed=0, separate=True)
    cfg = b3Config(solver_mode=capi.SOLVER_PGS, solver_iterations=10, use_cuda_graph=True, pgs_interleave=True,
                   broadphase=capi.BROADPHASE_AUTO)
    out["batched_scenes"] = dict(workload=WORKLOAD_BATCHED.format(n=args.scenes, bodies=sc.num_bodies),
                                 **_time_config(sc, cfg, device, settle=120, steps=30))
    # the pile while it falls and topples (the learned-warm-start configuration's lattice, at the
    # headline's fixed 10 iterations): every box in contact with its neighbours, several manifolds
    # a body, far more colours than the settled columns
    sc = scenes.box_pile(args.nx, 64, args.nx, jitter=0.05, seed=0)
    cfg = b3Config(solver_mode=capi.SOLVER_PGS, solver_iterations=10, use_cuda_graph=True, pgs_interleave=True,
                   broadphase=capi.BROADPHASE_AUTO)
    out["falling_lattice"] = dict(
        workload=f"box pile lattice {args.nx}x64x{args.nx} = {sc.num_bodies - 1:,} unit boxes (spacing 1.1, jitter "
                 "0.05, seed 0) falling onto a static plane from rest, PGS 10 iterations; timed steps 60..119, "
                 "while the lattice lands and its columns settle",
        **_time_config(sc, cfg, device, settle=60, steps=60))
    if not args.no_pour:
        from bullet3_gb300.warmstart import DEFAULT_WEIGHTS, WarmStartMLP
        sc = scenes.stress_container(1048576, seed=0)
        cfg = b3Config(solver_mode=capi.SOLVER_PGS, solver_iterations=16, residual_tol=1e-4, use_cuda_graph=True,
                       pgs_interleave=True, warm_start=capi.WARM_PERSISTENT_LEARNED, broadphase=capi.BROADPHASE_AUTO)
        net = WarmStartMLP.load(DEFAULT_WEIGHTS, device=device)
        out["million_body_pour"] = dict(
            workload=WORKLOAD_STRESS.format(bodies=sc.num_bodies, first=3, last=599),
            **_time_config(sc, cfg, device, settle=3, steps=597, warm_model=net))
    return out


# ------------------------------------------------------------------------------ GPU arm
def gpu_arm(args):
    import ctypes as C

    import numpy as np

    import __graft_entry__ as ge
    rank, world, local = dist_info()
    dist = dist_init(world)
    if rank == 0 or not (ROOT / "bullet3_gb300" / "libb3gpu.so").exists():
        ge.build()
    dist_barrier(dist)
    from bullet3_gb300 import capi, scenes
    from bullet3_gb300.pipeline import b3Config
    capi.load()
    scene = make_scene(args, rank)
    mode = capi.SOLVER_PGS if args.solver == "pgs" else capi.SOLVER_JACOBI
    # broadphase AUTO: the autotuner (below) times the grid and the LBVH and keeps the faster
    cfg = b3Config(solver_mode=mode, solver_iterations=args.iterations, use_cuda_graph=True,
                   pgs_interleave=args.solver == "pgs" and args.row_order == "interleaved",
                   broadphase=capi.BROADPHASE_AUTO)
    stress = args.workload == "stress"
    if stress:
        cfg.residual_tol = 1e-4
        cfg.warm_start = capi.WARM_PERSISTENT_LEARNED
    np_, bp, pl = scenes.load_scene(scene, cfg, device=local)
    if stress:
        from bullet3_gb300.warmstart import DEFAULT_WEIGHTS, WarmStartMLP
        net = WarmStartMLP.load(DEFAULT_WEIGHTS, device=local)
        pl.setWarmStartModel(net)
    h = np_.world.handle
    N = scene.num_bodies
    dt = 1.0 / 60.0
    for _ in range(args.settle):
        pl.stepSimulation(dt)
    for _ in range(max(3, args.warmup)):
        pl.stepSimulation(dt)
    pl.synchronize()
    # launch shapes chosen by the autotuner on this state (it leaves the state unchanged)
    tuning = pl.autotune(dt, repeats=3) if not args.no_autotune else None
    # the state after the warm-up steps is the timed workload (the e2e leg starts from it too)
    state0 = np_.readbackAllBodiesToCpu()
    # ---- timed region: device events on the library's stream
    clocks = ClockSampler(local)
    clocks.start()
    # keep the GPU stepping while the clock sampler starts (its samples then cover load only),
    # then put the warm-up state back
    # (the pour is timed as one long run from its warm-up state: no pre-roll there)
    t_roll = time.perf_counter()
    while not stress and time.perf_counter() - t_roll < 1.0:
        for _ in range(10):
            pl.stepSimulation(dt)
        pl.synchronize()
    np_.writeBodiesToGpu(state0)
    pl.synchronize()
    dist_barrier(dist)
    pl.synchronize()
    pl.status(clear=True)  # the device status word accumulates over the timed steps
    l0 = pl.launchCount()
    capi.call("b3g_record_event", h, C.c_int(0))
    for _ in range(args.steps):
        pl.stepSimulation(dt)
    capi.call("b3g_record_event", h, C.c_int(1))
    ms = C.c_float()
    capi.call("b3g_event_elapsed", h, C.c_int(0), C.c_int(1), C.byref(ms))
    pl.synchronize()
    launches = pl.launchCount() - l0
    clk = clocks.stop()
    dist_barrier(dist)
    t_rank = ms.value / 1000.0
    t_max = dist_max(dist, t_rank)
    value = world * N * args.steps / t_max
    status = pl.status()

    # ---- per-stage times (profiled steps after the timed region, events around each stage)
    pl.setProfiling(True)
    acc = np.zeros(7)
    P = 3
    for _ in range(P):
        pl.stepSimulation(dt)
        acc += pl.stageTimes()
    pl.setProfiling(False)
    acc /= P
    st = pl.stats()
    C_ = st.num_contacts
    I_ = max(1, st.iterations)
    P_ = st.num_pairs
    # algorithmic bytes (fp32/int32 widths, each field once): solve stage = constraint setup
    # 416 B + colouring 16 B + applied impulses 24 B per manifold, 352 B per manifold-iteration
    solve_bytes = C_ * (416 + 16 + 24) + 352 * C_ * I_
    stage_bytes = {"aabb": 56 * N, "pairs": 112 * N + 8 * P_, "contacts": 64 * P_ + 88 * C_,
                   "solve": solve_bytes, "integrate": 116 * N}
    stage_ms = {"aabb": acc[0], "pairs": acc[1], "contacts": acc[2], "solve": acc[4], "integrate": acc[6]}
    peak, peak_kind = measured_peaks()
    solve_s = stage_ms["solve"] / 1000.0
    achieved = solve_bytes / solve_s / 1e9 if solve_s > 0 else 0.0
    traffic = solver_traffic()
    roofline = {"bound": "hbm", "kernel": solve_kernels(tuning),
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind, "algorithmic_bytes": solve_bytes,
                "traffic": (traffic["bytes_per_manifold"] * C_ if traffic and "bytes_per_manifold" in traffic
                            else None),
                "traffic_source": ((f"not measured in this run: ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                    f"{', '.join(traffic.get('kernels', []))} per manifold from profiles/"
                                    f"solver_traffic.json ({traffic.get('workload', '')}; "
                                    f"{traffic.get('launch', 'launch shapes as captured')}), times this run's "
                                    f"{C_} manifolds") if traffic else None)}
    stages = {k: {"ms": float(v), "algorithmic_GBps": stage_bytes[k] / (v / 1000.0) / 1e9 if v > 0 else None,
                  "frac_of_hbm": (stage_bytes[k] / (v / 1000.0) / 1e9 / peak) if v > 0 else None}
              for k, v in stage_ms.items()}

    # ---- end to end through the C ABI with host buffers (pinned): upload state, step, download
    e2e = None
    try:
        import torch
        nbytes = N * capi.BODY.itemsize
        pin_in = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        pin_out = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        host_in = pin_in.numpy().view(capi.BODY)
        host_out = pin_out.numpy().view(capi.BODY)
        host_in[:] = state0
        pl.synchronize()
        dist_barrier(dist)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            capi.call("b3g_write_bodies", h, capi.ptr(host_in), C.c_int(N))
            capi.call("b3g_step", h, C.c_float(dt))
            capi.call("b3g_read_bodies", h, capi.ptr(host_out), C.c_int(N))
            host_in, host_out = host_out, host_in  # this step's result is the next step's input
        t_e2e = dist_max(dist, time.perf_counter() - t0)
        e2e = {"value": world * N * args.steps / t_e2e, "unit": "body-steps/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes}
    except Exception as ex:  # pinned memory needs torch; report why instead of guessing
        e2e = {"value": None, "unit": "body-steps/s", "error": str(ex)}

    # ---- CPU baseline: the oracle's composed step on the same scene, bounded sample
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        secs, threads, n = cpu_run(scene, cpu_tables(scene), args.cpu_steps, args.iterations, solver_mode_code(args))
        what = (f"every one of the {args.scenes} scenes" if args.workload == "batched" else "the same scene")
        cpu = {"value": n * args.cpu_steps / secs, "unit": "body-steps/s", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_steps} composed CPU steps of {what} ({n} bodies) from its initial state: "
                         + CPU_KIND.format(threads=threads)}

    # ---- learned vs plain: sweeps and ms per step to the residual target (rank 0, one GPU)
    residual = None
    configurations = None
    if rank == 0 and world == 1 and args.workload == "pile":
        del np_, bp, pl
        if args.residual_steps > 0:
            residual = to_residual(args, local)
        if not args.no_configurations:
            configurations = other_configurations(args, local)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": 1000 * t_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": bench_config(args, scene, world),
                "workload_stats": {"pairs": P_, "manifolds": C_, "contact_points": st.num_points,
                                   "colors": st.num_colors, "tuning": tuning},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "stages": stages, "device_status": int(status), "to_residual": residual,
                "configurations": configurations}
        print(json.dumps(line), flush=True)
    dist_barrier(dist)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
