"""Sweep and prune over large finite static AABBs: per scene, the static boxes sorted along one
axis each step; every dynamic body scans the window of mins that can reach it.  Bar: the pair
set bit-exact against the oracle's brute-force set (and per scene with independent scenes),
including the unsorted fallback for scenes with more static proxies than one block sorts."""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, run_stages
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _check(sc, np_, bp, pl, shapes, per_scene=False):
    b = np_.readbackAllBodiesToCpu()
    run_stages(np_, bp, pl, solve=False)
    ga = bp.getAllAabbsCPU()
    assert np.array_equal(ga.view(np.uint8), O.aabbs(b, shapes).view(np.uint8))
    gp = pairs_xy(bp.getOverlappingPairsCPU())
    op = O.pairs_scenes(ga, sc.scene_first) if per_scene else O.pairs_bruteforce(ga)
    assert len(op) > 0
    assert np.array_equal(gp, pairs_xy(op))
    return gp


@pytest.mark.parametrize("n_static", [1500, 5000])
def test_sap_pair_set_bitexact(n_static):
    # 5000 static proxies in one scene exceed the per-scene sort and take the unsorted scan
    sc = scenes.static_field(n_static, 6000, extent=90.0, seed=n_static)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000, solver_mode=capi.SOLVER_PGS, use_cuda_graph=True)
    gp = _check(sc, np_, bp, pl, shapes)
    static = sc.mass == 0
    assert static[gp[:, 0]].any() or static[gp[:, 1]].any()  # static-dynamic pairs found
    assert pl.stats().num_large == int(static.sum())
    for _ in range(10):  # the pile moves among the statics; the window follows
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() == 0
    _check(sc, np_, bp, pl, shapes)


def test_sap_with_independent_scenes():
    sc = scenes.static_field(1200, 3000, extent=40.0, seed=3, scenes=6)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000)
    _check(sc, np_, bp, pl, shapes, per_scene=True)
