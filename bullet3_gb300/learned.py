"""Training and evaluation of the learned warm start.

Data: the plain solver's own converged impulses.  Seeded batches of box/sphere piles (the
batched-scene shapes: counts log-uniform in [8, 256], jittered lattices on a plane) are stepped
with a cold PGS solve run to a 1e-4 residual while the step records, per active contact point,
its 12 features, its converged impulses and whether it persisted from the previous step
(B3G_WARM_RECORD).  Training: Adam on the GPU through the library's tensor-core forward and
backward kernels.  Evaluation: the same scene stepped with the plain solver and with each warm
start, every solve run to the same residual; the per-step sweep counts and solve times are
compared.

    python -m bullet3_gb300.learned train --out weights.npz
    python -m bullet3_gb300.learned evaluate --weights weights.npz
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import capi, scenes
from .pipeline import b3Config
from .warmstart import DEFAULT_WEIGHTS, WarmStartMLP

DT = 1.0 / 60.0


def collect(n_scenes=200, steps=120, every=2, seed=0, tol=1e-4, cap=1000, new_only=False):
    """Features, targets and persistence flags logged from cold solves run to `tol`."""
    sc = scenes.batched_piles(n_scenes, seed=seed)
    cfg = b3Config(solver_mode=capi.SOLVER_PGS, solver_iterations=cap, residual_tol=tol, pgs_interleave=True,
                   warm_start=capi.WARM_RECORD, use_cuda_graph=True)
    np_, bp, pl = scenes.load_scene(sc, cfg)
    xs, ts, ns = [], [], []
    for step in range(steps):
        pl.stepSimulation(DT)
        if step % every == 0:
            pl.synchronize()
            f, t, new = pl.readWarmSamples(with_new=True)
            if new_only:
                f, t = f[new], t[new]
            xs.append(f)
            ts.append(t)
            ns.append(new if not new_only else new[new])
    return np.concatenate(xs), np.concatenate(ts), np.concatenate(ns)


def train(x, t, epochs=8, batch=4096, lr=1e-3, seed=0, log=print):
    m = WarmStartMLP(seed=seed)
    m.fit_normalization(x, t)
    rng = np.random.Generator(np.random.PCG64(seed))
    n = len(x) // batch * batch
    history = []
    for e in range(epochs):
        perm = rng.permutation(len(x))[:n]
        m.set_training_data(x[perm], t[perm])
        rate = lr * (0.5 ** (e // 3))
        loss = m.train(steps=n // batch, batch=batch, lr=rate)
        history.append(loss)
        log(f"epoch {e}: mean batch loss {loss:.4f} (lr {rate:g})")
    return m, history


def evaluation_scene(kind="piles", size=512, seed=1):
    """piles: `size` batched piles (held-out seed); lattice: size^3 boxes, spacing 1.1, jitter 0.05."""
    if kind == "piles":
        return scenes.batched_piles(size, seed=1000 + seed)
    return scenes.box_pile(size, size, size, jitter=0.05, seed=seed)


def evaluate(weights=None, kind="piles", size=512, steps=120, first=30, tol=1e-4, cap=1000, seed=1,
             modes=("cold", "learned", "persistent", "persistent_learned")):
    """Sweeps and solve ms per step to `tol` (at most `cap` sweeps), each mode stepped from the
    same initial state; averages over steps [first, steps)."""
    sc = evaluation_scene(kind, size, seed)
    code = {"cold": capi.WARM_COLD, "learned": capi.WARM_LEARNED, "persistent": capi.WARM_PERSISTENT,
            "persistent_learned": capi.WARM_PERSISTENT_LEARNED}
    net = WarmStartMLP.load(weights) if weights is not None else None
    out = {}
    for mode in modes:
        cfg = b3Config(solver_mode=capi.SOLVER_PGS, solver_iterations=cap, residual_tol=tol, pgs_interleave=True,
                       warm_start=code[mode], use_cuda_graph=True)
        np_, bp, pl = scenes.load_scene(sc, cfg)
        if net is not None and mode in ("learned", "persistent_learned"):
            pl.setWarmStartModel(net)
        iters, ms, contacts, resid, dropped = [], [], [], [], 0
        pl.setProfiling(True)
        for step in range(steps):
            pl.stepSimulation(DT)
            pl.synchronize()
            st = pl.stats()
            if step >= first:
                iters.append(st.iterations)
                ms.append(float(pl.stageTimes()[4]))
                contacts.append(st.num_contacts)
                resid.append(st.residual)
                dropped += bool(st.status & capi.FLAG_WARM_DISCARDED)
            pl.status(clear=True)
        pl.setProfiling(False)
        out[mode] = {"iterations": float(np.mean(iters)), "solve_ms": float(np.mean(ms)),
                     "manifolds": float(np.mean(contacts)), "dropped_steps": int(dropped),
                     "converged": float(np.mean(np.array(iters) < cap)), "residual": float(np.mean(resid)),
                     "iterations_per_step": [int(i) for i in iters]}
        del np_, bp, pl
    return out


def main(argv=None):
    p = argparse.ArgumentParser()
    sub = p.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default=str(DEFAULT_WEIGHTS))
    t.add_argument("--scenes", type=int, default=200)
    t.add_argument("--steps", type=int, default=120)
    t.add_argument("--epochs", type=int, default=8)
    t.add_argument("--new-only", action="store_true")
    ev = sub.add_parser("evaluate")
    ev.add_argument("--weights", default=str(DEFAULT_WEIGHTS))
    ev.add_argument("--kind", choices=["piles", "lattice"], default="piles")
    ev.add_argument("--size", type=int, default=512)
    ev.add_argument("--steps", type=int, default=120)
    ev.add_argument("--cap", type=int, default=1000)
    a = p.parse_args(argv)
    if a.cmd == "train":
        t0 = time.perf_counter()
        x, y, new = collect(a.scenes, a.steps, new_only=a.new_only)
        t1 = time.perf_counter()
        print(f"{len(x)} samples ({new.mean():.2%} new) from {a.scenes} scenes x {a.steps} steps in {t1 - t0:.1f} s")
        m, hist = train(x, y, epochs=a.epochs)
        print(f"trained in {time.perf_counter() - t1:.1f} s")
        m.save(a.out, samples=len(x), loss_history=np.array(hist))
    else:
        print(json.dumps(evaluate(a.weights, a.kind, a.size, a.steps, cap=a.cap)))


if __name__ == "__main__":
    main()
