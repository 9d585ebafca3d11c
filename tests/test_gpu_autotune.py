"""The autotuner (b3g_autotune): every candidate is timed from the same saved state, the state is
left unchanged, the chosen shapes come from the candidate lists, and results stay exact under the
tuned shapes (pair sets, manifolds and Jacobi velocities bit-exact against the oracle)."""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, run_stages, valid_points_equal
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_autotune_keeps_state_and_picks_candidates():
    sc = scenes.box_pile(12, 6, 12, seed=4)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, pgs_interleave=True,
                               use_cuda_graph=True)
    for _ in range(20):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    before = np_.readbackAllBodiesToCpu()
    t = pl.autotune(1 / 60, repeats=2)
    after = np_.readbackAllBodiesToCpu()
    assert np.array_equal(before.view(np.uint8), after.view(np.uint8))
    assert t["sort_blocks_per_sm"] in (2, 4, 8)
    assert t["pairs_blocks_per_sm"] in (2, 4, 8, 16) and t["narrow_blocks_per_sm"] in (2, 4, 8, 16)
    assert t["pgs_partitions"] in (capi.PGS_PARTITIONS_NONE, capi.PGS_PARTITIONS_SHARED,
                                   capi.PGS_PARTITIONS_GLOBAL_DELTAS, capi.PGS_PARTITIONS_STREAMED)
    assert t["candidates_timed"] == 3 + 4 + 4 + 4 and t["solve_ms"] > 0
    assert pl.tuning() == t
    for _ in range(5):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() == 0


def test_results_exact_under_tuned_shapes():
    sc = scenes.mixed_scene(3000, extent=18.0, seed=8, plane=True)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000, solver_mode=capi.SOLVER_JACOBI, solver_iterations=8,
                               autotune=True)
    pl.stepSimulation(1 / 60)  # the first step tunes, then steps
    pl.synchronize()
    assert pl.tuning()["candidates_timed"] > 0
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    oa = O.aabbs(b, shapes)
    gp = bp.getOverlappingPairsCPU()
    assert np.array_equal(pairs_xy(gp), pairs_xy(O.pairs_bruteforce(oa)))
    oc, _ = O.contacts(b, shapes, gp)
    gc = np_.getContactsCPU()
    assert valid_points_equal(gc, oc)
    ob, _, _, _ = O.solve(b, I, oc, mode=1, iterations=8)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
