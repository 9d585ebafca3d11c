"""Step a synthetic workload for a fixed number of steps and print one line of statistics.

Meant for running the pipeline under an external profiler (ncu) or by hand: nothing but the
scene upload, the warm-up steps and the measured steps touch the GPU.

    python -m bullet3_gb300.stepper [--workload pile|lattice|batched|mixed|stress|chains|compound|terrain] [--settle S]
                                    [--steps K] [--warmup W] [--solver pgs|jacobi] [--iterations I]
                                    [--autotune] [--broadphase grid|lbvh] [--stage-times] [--profile-range]

--profile-range brackets the K measured steps with b3g_profiler_range, for a profiler started
with profiling off (ncu --profile-from-start off --clock-control none); --settle steps first, untimed.

  pile     262,144 unit boxes resting in 64x64 columns on a plane (the settled 64^3 lattice)
  lattice  the 64^3 lattice (spacing 1.1, jitter 0.05) falling onto the plane from rest
  batched  4,096 independent box/sphere piles, each on its own plane, through per-scene offsets
  mixed    131,072 boxes, spheres and Gaussian hulls in a 64^3 box, random orientations, N(0,1) velocities
  stress   1,048,576 bodies of the same mix poured into a 5-plane container from heights U[0, 512]
  chains   8,192 chains of 32 spheres (262,144 bodies and ball joints, every 8th joint fixed)
           hanging from one static box in a 3 m grid, swinging
  compound 131,072 bodies (2,048 x nx) on a plane: compounds of convex hulls (an L of two boxes, a
           dumbbell of two hulls and a box) among single boxes and hulls, dropped as a lattice from rest
  terrain  32,768 bodies (512 x nx) of the same four kinds dropped as a lattice onto a static
           256 x 256-quad height-field mesh (131,072 triangles)
"""
from __future__ import annotations

import argparse
import json
import time

from . import capi, scenes
from .pipeline import b3Config


def make(workload: str, n: int = 64):
    if workload == "pile":
        return scenes.box_stack(n, 64, n, seed=0)
    if workload == "lattice":
        return scenes.box_pile(n, 64, n, jitter=0.05, seed=0)
    if workload == "batched":
        return scenes.batched_piles(4096, seed=0, separate=True)
    if workload == "mixed":
        return scenes.mixed_scene(131072, extent=64.0, seed=0)
    if workload == "stress":
        return scenes.stress_container(1048576, seed=0)
    if workload == "chains":
        return scenes.hanging_chains(8192, 32, seed=0, fixed_every=8, anchor_index=-1, random_orn=False,
                                     per_row=91)
    if workload == "compound":
        return scenes.compound_scene(2048 * n, seed=0, lattice=True)
    if workload == "terrain":
        return scenes.terrain_scene(512 * n, grid=256, seed=0, drop=True)
    raise ValueError(workload)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--workload", choices=["pile", "lattice", "batched", "mixed", "stress", "chains", "compound", "terrain"],
                   default="pile")
    p.add_argument("--settle", type=int, default=0)
    p.add_argument("--profile-range", action="store_true")
    p.add_argument("--nx", type=int, default=64)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--solver", choices=["pgs", "jacobi"], default="pgs")
    p.add_argument("--iterations", type=int, default=10)
    p.add_argument("--autotune", action="store_true")
    p.add_argument("--no-graph", action="store_true")
    p.add_argument("--broadphase", choices=["grid", "lbvh", "auto"], default="grid")
    p.add_argument("--pgs-flow", type=int, default=0, help="PGS grid-wide sweeps: 0 default (grid barrier per colour), 1 dataflow, 2 grid barrier")
    p.add_argument("--pgs-tail", type=int, default=0, help="trailing-colour size solved in one block (0: library default)")
    p.add_argument("--rays", type=int, default=0,
                   help="after the steps, time castRays of this many random downward rays over the bodies")
    p.add_argument("--stage-times", action="store_true",
                   help="also run the measured steps once more with per-stage events and print their means")
    a = p.parse_args(argv)
    sc = make(a.workload, a.nx)
    cfg = b3Config(solver_mode=capi.SOLVER_PGS if a.solver == "pgs" else capi.SOLVER_JACOBI,
                   solver_iterations=a.iterations, pgs_interleave=a.solver == "pgs",
                   use_cuda_graph=not a.no_graph,
                   broadphase={"grid": capi.BROADPHASE_GRID, "lbvh": capi.BROADPHASE_LBVH,
                               "auto": capi.BROADPHASE_AUTO}[a.broadphase],
                   pgs_flow=a.pgs_flow, pgs_tail_manifolds=a.pgs_tail)
    if a.workload == "terrain":
        cfg.m_maxTriConvexPairCapacity = 64 * sc.num_bodies  # about 30 triangle-convex pairs a body at rest
    np_, bp, pl = scenes.load_scene(sc, cfg)
    dt = 1.0 / 60.0
    for _ in range(a.settle):
        pl.stepSimulation(dt)
    for _ in range(a.warmup):
        pl.stepSimulation(dt)
    pl.synchronize()
    tuning = pl.autotune(dt) if a.autotune else None
    if a.profile_range:
        capi.call("b3g_profiler_range", capi.C.c_int(1))
    t0 = time.perf_counter()
    for _ in range(a.steps):
        pl.stepSimulation(dt)
    pl.synchronize()
    secs = time.perf_counter() - t0
    if a.profile_range:
        capi.call("b3g_profiler_range", capi.C.c_int(0))
    stage_ms = None
    if a.stage_times:
        import numpy as np
        pl.setProfiling(True)
        acc = np.zeros(7)
        for _ in range(a.steps):
            pl.stepSimulation(dt)
            pl.synchronize()
            acc += pl.stageTimes()
        pl.setProfiling(False)
        names = ["aabbs", "pairs", "contacts", "joints", "solver", None, "integrate"]
        stage_ms = {k: round(float(v) / max(a.steps, 1), 4) for k, v in zip(names, acc) if k}
    rays_out = None
    if a.rays > 0:
        import numpy as np
        b = np_.readbackAllBodiesToCpu()
        dyn = b[b["invMass"] != 0]["pos"][:, :3]
        lo, hi = dyn.min(0), dyn.max(0)
        rng = np.random.Generator(np.random.PCG64(0))
        rays = np.zeros(a.rays, capi.RAY)
        xz = rng.uniform(lo[[0, 2]], hi[[0, 2]], (a.rays, 2)).astype(np.float32)
        rays["from"][:, 0], rays["from"][:, 2], rays["from"][:, 1] = xz[:, 0], xz[:, 1], hi[1] + 5.0
        rays["to"][:, 0], rays["to"][:, 2], rays["to"][:, 1] = xz[:, 0], xz[:, 1], lo[1] - 1.0
        h = np_.world.handle
        for _ in range(3):
            hits = pl.castRays(rays)
        reps = 5
        t0 = time.perf_counter()
        capi.call("b3g_record_event", h, capi.C.c_int(0))
        for _ in range(reps):
            hits = pl.castRays(rays)
        capi.call("b3g_record_event", h, capi.C.c_int(1))
        wall = (time.perf_counter() - t0) / reps
        ms = capi.C.c_float()
        capi.call("b3g_event_elapsed", h, capi.C.c_int(0), capi.C.c_int(1), capi.C.byref(ms))
        rays_out = {"rays": a.rays, "hit_fraction": float((hits["hitFraction"] < 1.0).mean()),
                    "device_ms_per_cast": ms.value / reps, "host_ms_per_cast": 1000 * wall,
                    "rays_per_s": a.rays / wall}
        # the same cast on rays and hits already on the device (no host copies)
        import torch
        d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
        hits0 = np.zeros(a.rays, capi.RAYHIT)
        hits0["hitBody"] = -1
        hits0["hitResult2"] = -1
        d_hits = torch.from_numpy(hits0.view(np.uint8)).cuda()
        torch.cuda.synchronize()
        for _ in range(3):
            pl.castRaysDevice(d_rays.data_ptr(), d_hits.data_ptr(), a.rays)
        capi.call("b3g_record_event", h, capi.C.c_int(0))
        for _ in range(reps):
            pl.castRaysDevice(d_rays.data_ptr(), d_hits.data_ptr(), a.rays)
        capi.call("b3g_record_event", h, capi.C.c_int(1))
        capi.call("b3g_event_elapsed", h, capi.C.c_int(0), capi.C.c_int(1), capi.C.byref(ms))
        rays_out["device_resident_ms_per_cast"] = ms.value / reps
        rays_out["device_resident_rays_per_s"] = a.rays / (ms.value / reps / 1000.0)
    st = pl.stats()
    print(json.dumps({"workload": a.workload, "broadphase": a.broadphase, "rays": rays_out, "bodies": sc.num_bodies, "steps": a.steps,
                      "joints": pl.getNumConstraints(), "stage_ms": stage_ms,
                      "host_ms_per_step": 1000 * secs / max(a.steps, 1), "pairs": st.num_pairs,
                      "manifolds": st.num_contacts, "points": st.num_points, "colors": st.num_colors,
                      "child_pairs": st.num_child_pairs, "concave_pairs": st.num_concave_pairs,
                      "status": int(pl.status()), "tuning": tuning}))
    return 0 if pl.status() == 0 else 1


if __name__ == "__main__":
    raise SystemExit(main())
