"""Batched independent scenes (b3g_set_scene_offsets): many scenes of uneven size, all at the
origin and each with its own plane, stepped together in one world.

Bars: AABBs and the pair set bit-exact against the oracle's per-scene pair sets (the reference
runs one broadphase per scene); with the Jacobi solver every scene's bodies after a run of
graph-captured steps are bit-identical to the same scene stepped as a world of its own; with PGS
no contact crosses scenes, batches are legal and the piles rest on their planes.
"""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, run_stages
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_scene_pairs_bitexact():
    sc = scenes.batched_piles(64, seed=5, separate=True)
    np_, bp, pl, shapes = load(sc)
    b = np_.readbackAllBodiesToCpu()
    run_stages(np_, bp, pl, solve=False)
    oa = O.aabbs(b, shapes)
    assert np.array_equal(bp.getAllAabbsCPU().view(np.uint8), oa.view(np.uint8))
    gp = pairs_xy(bp.getOverlappingPairsCPU())
    op = pairs_xy(O.pairs_scenes(oa, sc.scene_first))
    assert len(op) > 0
    assert np.array_equal(gp, op)
    # the scenes overlap in space: one world without the offset table pairs across scenes
    allp = pairs_xy(O.pairs_bruteforce(oa))
    assert len(allp) > 2 * len(op)


def _bodies_by_scene(bodies, first):
    n = len(bodies)
    return [bodies[a:(first[s + 1] if s + 1 < len(first) else n)] for s, a in enumerate(first)]


def test_scene_worlds_match_standalone_jacobi():
    sc = scenes.batched_piles(12, seed=9, separate=True)
    steps = 15
    np_, bp, pl, _ = load(sc, solver_mode=capi.SOLVER_JACOBI, solver_iterations=10, use_cuda_graph=True)
    for _ in range(steps):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() == 0
    batched = _bodies_by_scene(np_.readbackAllBodiesToCpu(), sc.scene_first)
    for s in range(len(sc.scene_first)):
        one = scenes.scene_part(sc, s)
        n1, b1, p1, _ = load(one, solver_mode=capi.SOLVER_JACOBI, solver_iterations=10, use_cuda_graph=True)
        for _ in range(steps):
            p1.stepSimulation(1 / 60)
        p1.synchronize()
        alone = n1.readbackAllBodiesToCpu()
        assert np.array_equal(batched[s].view(np.uint8), alone.view(np.uint8)), f"scene {s}"


def test_scene_pgs_contacts_stay_within_scenes():
    sc = scenes.batched_piles(256, seed=11, separate=True)
    np_, bp, pl, _ = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, pgs_interleave=True,
                          use_cuda_graph=True)
    for _ in range(90):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() == 0
    run_stages(np_, bp, pl)
    gc = np_.getContactsCPU()
    assert len(gc) > 0
    a, b = np.abs(gc["bodyA"]), np.abs(gc["bodyB"])
    assert np.array_equal(sc.scene_of[a], sc.scene_of[b])
    bodies = np_.readbackAllBodiesToCpu()
    assert O.check_batches(gc, pl.readBatches(), bodies) == 0
    dyn = bodies["invMass"] > 0
    # every pile has landed on its own plane and rests there (boxes and spheres of half size 0.5)
    assert bodies["pos"][dyn, 1].min() > 0.4


def test_empty_scenes_in_the_offset_table():
    # empty scenes (repeated offsets, at the start, middle and end) change nothing
    sc = scenes.batched_piles(8, seed=21, separate=True)
    runs = []
    for first in (sc.scene_first, np.array([0, 0] + sc.scene_first[1:4].tolist() + [sc.scene_first[4]] * 3
                                           + sc.scene_first[5:].tolist() + [sc.num_bodies], np.int32)):
        sc.scene_first = first
        np_, bp, pl, _ = load(sc, solver_mode=capi.SOLVER_JACOBI, solver_iterations=10, use_cuda_graph=True)
        for _ in range(20):
            pl.stepSimulation(1 / 60)
        pl.synchronize()
        assert pl.status() == 0
        runs.append((pairs_xy(bp.getOverlappingPairsCPU()), np_.readbackAllBodiesToCpu()))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1].view(np.uint8), runs[1][1].view(np.uint8))
