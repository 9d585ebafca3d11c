"""The learned warm start inside the step: features, the network's predictions as initial
impulses, their application before the first sweep and the cold-start fallback.

Bars: features within 1e-5 relative of a float32 restatement from the same state; warm-started
PGS velocities bit-exact against the oracle sweeping the GPU's order from the same initial
impulses; a warm start worse than a cold start is dropped and the result equals the cold solve
bit for bit, with the dropped sweep counted.
"""
import numpy as np
import pytest

from gpu_helpers import load, run_stages
from bullet3_gb300 import capi, scenes
from oracle import mlp_oracle as MO
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _network(bias_out=(0.0, 0.0, 0.0), seed=4, scale=1.0):
    from bullet3_gb300.warmstart import WarmStartMLP
    m = WarmStartMLP(seed=seed)
    p = MO.init_params(seed) * scale
    p[-3:] = bias_out
    m.params = p
    n = MO.identity_norm()
    n[24:27] = (0.5, 0.0, 0.0)  # target mean: a positive contact impulse
    n[27:30] = (2.0, 10.0, 10.0)
    m.normalization = n
    return m


def _features_cpu(b, c, dt=1 / 60, g=(0.0, -9.8, 0.0), threshold=0.02):
    f32 = np.float32
    rows = []
    for m in range(len(c)):
        A, B = abs(int(c["bodyA"][m])), abs(int(c["bodyB"][m]))
        imA, imB = b["invMass"][A], b["invMass"][B]
        npts = min(int(c["normal"][m, 3]), 4)
        if imA == 0 and imB == 0:
            continue
        n = c["normal"][m, :3].astype(f32)
        n = n * f32(f32(1.0) / np.sqrt(f32(n @ n)))
        for j in range(npts):
            dist = c["worldPosB"][m, j, 3]
            if not dist <= threshold:
                continue
            p2 = c["worldPosB"][m, j, :3]
            p1 = p2 + n * dist
            r1 = p1 - b["pos"][A, :3]
            r2 = p2 - b["pos"][B, :3]
            v1 = b["linVel"][A, :3] + np.cross(b["angVel"][A, :3], r1)
            v2 = b["linVel"][B, :3] + np.cross(b["angVel"][B, :3], r2)
            v = (v1 - v2).astype(f32)
            vt = v - n * f32(n @ v)
            rows.append(np.concatenate([v, n, [dist, imA, imB, npts, np.sqrt(vt @ vt), dt * (np.dot(g, n))]]))
    return np.array(rows, np.float32)


def test_features_match_restatement():
    sc = scenes.mixed_scene(2048, extent=14.0, seed=8, plane=True)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=300000, warm_start=2)
    b = np_.readbackAllBodiesToCpu()
    run_stages(np_, bp, pl)
    f, t = pl.readWarmSamples()
    ref = _features_cpu(b, np_.getContactsCPU())
    assert len(f) == len(ref) > 1000
    np.testing.assert_allclose(f, ref, rtol=1e-5, atol=2e-6)
    # targets are the converged impulses of the same points
    imp = pl.readImpulses()
    assert np.isfinite(t).all() and (t[:, 0] >= 0).all()
    assert np.isclose(t[:, 0].sum(), imp[:, 0::3].sum(), rtol=1e-5)


@pytest.mark.parametrize("interleave", [False, True])
@pytest.mark.parametrize("parts", [capi.PGS_PARTITIONS_AUTO, capi.PGS_PARTITIONS_STREAMED])
def test_warm_started_solve_bitexact(interleave, parts):
    sc = scenes.box_stack(12, 10, 12, seed=6)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, warm_start=1,
                               pgs_interleave=interleave, pgs_partitions=parts)
    net = _network()
    pl.setWarmStartModel(net)
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    gc = np_.getContactsCPU()
    warm = pl.readWarmStart()
    assert (warm[:, 0::3] > 0).any()  # the network produced non-trivial initial impulses
    order = pl.readSolveOrder()
    ob, oimp, it, res, disc = O.solve_ordered_ex(b, I, gc, order, warm=warm, iterations=10, interleave=interleave)
    gb = np_.readbackAllBodiesToCpu()
    st = pl.stats()
    assert bool(st.status & capi.FLAG_WARM_DISCARDED) == disc
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    assert np.array_equal(pl.readImpulses(), oimp)
    assert st.iterations == it


def test_bad_warm_start_is_dropped():
    # one layer of boxes on the plane: absurd initial contact impulses launch every box, so the
    # first sweep clamps them back to ~0 (residual >> 1).  (In tall stacks a uniform impulse
    # cancels between neighbours and would not be detected as worse -- nor is it.)
    sc = scenes.box_stack(4, 1, 4, seed=2)
    outs = []
    for warm in (0, 1):
        np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, warm_start=warm,
                                   pgs_interleave=True)
        if warm:
            pl.setWarmStartModel(_network(bias_out=(50.0, 0.0, 0.0)))  # absurd impulses
        run_stages(np_, bp, pl)
        st = pl.stats()
        outs.append((np_.readbackAllBodiesToCpu(), st))
    (cold, st0), (warmb, st1) = outs
    assert st1.status & capi.FLAG_WARM_DISCARDED and not st0.status & capi.FLAG_WARM_DISCARDED
    assert st1.iterations == st0.iterations + 1
    assert np.array_equal(cold["linVel"], warmb["linVel"]) and np.array_equal(cold["angVel"], warmb["angVel"])


def test_graph_step_with_network():
    # the network's launches are part of the captured step; graph and staged steps agree
    res = []
    for graph in (True, False):
        sc = scenes.box_pile(5, 5, 5, seed=3)
        np_, bp, pl, shapes = load(sc, use_cuda_graph=graph, warm_start=1, pgs_interleave=True)
        pl.setWarmStartModel(_network())
        for _ in range(30):
            pl.stepSimulation(1 / 60)
        pl.synchronize()
        res.append(np_.readbackAllBodiesToCpu())
        assert pl.status() & ~capi.FLAG_WARM_DISCARDED == 0
    assert np.array_equal(res[0].view(np.uint8), res[1].view(np.uint8))


def test_persistent_contacts_start_from_previous_impulses():
    # a settled stack: after one cold step nearly every point persists; its initial impulses are
    # the previous solve's converged impulses and the solve reaches the tolerance in fewer sweeps
    sc = scenes.box_stack(6, 3, 6, seed=1)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=1000, residual_tol=1e-4,
                               warm_start=capi.WARM_PERSISTENT_LEARNED, pgs_interleave=True)
    pl.stepSimulation(1 / 60)  # one full step (cold: nothing to persist from)
    pl.synchronize()
    it_cold = pl.stats().iterations
    imp1 = pl.readImpulses()
    _, _, new0 = pl.readWarmSamples(with_new=True)
    assert new0.all()
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)  # the next step's stages from the integrated state
    _, _, new1 = pl.readWarmSamples(with_new=True)
    assert new1.mean() < 0.05
    warm = pl.readWarmStart()
    gc = np_.getContactsCPU()
    assert len(warm) == len(imp1)
    # persisting points of an unchanged manifold list carry the previous impulses
    same = np.isclose(warm, imp1, rtol=0, atol=0).mean()
    assert same > 0.9
    st = pl.stats()
    assert st.iterations < it_cold
    # and the warm-started solve is the oracle's, bit for bit, over the same number of sweeps (the
    # stopping test compares a float32-accumulated residual with the tolerance, so the sweep count
    # is taken from the GPU)
    order = pl.readSolveOrder()
    ob, _, it, res, disc = O.solve_ordered_ex(b, I, gc, order, warm=warm, iterations=st.iterations,
                                              interleave=True)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    assert it == st.iterations and not disc and res <= 1.5e-4


def test_trained_network_cuts_sweeps_on_held_out_piles():
    # the committed network (trained on the GPU by bullet3_gb300.learned from the plain solver's
    # converged impulses) against the cold start on piles it never saw, every solve run to 1e-4:
    # alone it saves at least 15% of the sweeps (measured 28%); predicting the new points beside
    # the persisting ones' carried impulses it reaches the target of at least 30% fewer sweeps than
    # the cold start (measured 53%) and fewer than persistence alone (measured 6%); no step falls
    # back to a cold start
    from bullet3_gb300 import learned
    from bullet3_gb300.warmstart import DEFAULT_WEIGHTS
    r = learned.evaluate(DEFAULT_WEIGHTS, kind="piles", size=128, steps=60, first=20, cap=1000, seed=7)
    for mode in r.values():
        assert mode["converged"] == 1.0 and mode["dropped_steps"] == 0, r
    cold = r["cold"]["iterations"]
    assert r["learned"]["iterations"] < 0.85 * cold, r
    assert r["persistent_learned"]["iterations"] <= 0.70 * cold, r
    assert r["persistent_learned"]["iterations"] < r["persistent"]["iterations"], r
