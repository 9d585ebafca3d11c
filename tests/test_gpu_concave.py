"""Concave triangle meshes on the GPU through the C ABI, against the oracle on the same inputs
(the oracle's concave path is pinned byte for byte to the reference's BVH traversal and concave
kernels' host twins by the golden fixture concave.npz).

Bars: the triangle-convex pair count equal to the oracle's; manifolds bit-exact on their valid
points in the GPU's order (the pairs', the compound child pairs', then one per touching triangle
(and child) in (pair, triangle, child) order); Jacobi velocities bit-exact; PGS velocities
bit-exact against the oracle sweeping the GPU's colour order; bodies dropped on the mesh come to
rest on it.
"""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, run_stages, valid_points_equal
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

INFO = capi.FLAG_WARM_DISCARDED  # informational, not an error


def _expected(b, shapes, pairs):
    aabbs = O.aabbs(b, shapes)
    oc, _ = O.contacts(b, shapes, pairs)
    cc, _ = O.compound_contacts(b, shapes, O.compound_pairs(b, shapes, pairs))
    tp = O.concave_pairs(b, shapes, aabbs, pairs)
    mc, _ = O.concave_contacts(b, shapes, aabbs, tp)
    return np.concatenate([oc, cc, mc]), len(tp), len(mc)


def _check_manifolds(gc, exp):
    assert valid_points_equal(gc, exp)
    assert np.array_equal(gc["childA"], exp["childA"]) and np.array_equal(gc["childB"], exp["childB"])


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("broadphase", [capi.BROADPHASE_GRID, capi.BROADPHASE_LBVH])
def test_concave_stages_bitexact(seed, broadphase):
    sc = scenes.terrain_scene(2048, seed=seed)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000, solver_mode=capi.SOLVER_JACOBI,
                               broadphase=broadphase)
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    ga = bp.getAllAabbsCPU()
    assert np.array_equal(ga.view(np.uint8), O.aabbs(b, shapes).view(np.uint8))
    op = O.pairs_bruteforce(ga)
    assert np.array_equal(pairs_xy(bp.getOverlappingPairsCPU()), pairs_xy(op))
    exp, ntri, nmesh = _expected(b, shapes, op)
    assert ntri > 30000 and nmesh > 3000
    assert pl.stats().num_concave_pairs == ntri
    gc = np_.getContactsCPU()
    _check_manifolds(gc, exp)
    ob, oimp, _, _ = O.solve(b, I, exp, mode=1, iterations=10)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    assert np.array_equal(pl.readImpulses(), oimp)
    assert pl.status() & ~INFO == 0


@pytest.mark.parametrize("interleave", [False, True])
def test_concave_pgs_colour_order_bitexact(interleave):
    sc = scenes.terrain_scene(2048, seed=2)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000, solver_mode=capi.SOLVER_PGS, solver_iterations=10,
                               pgs_interleave=interleave)
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    gc = np_.getContactsCPU()
    exp, _, _ = _expected(b, shapes, bp.getOverlappingPairsCPU())
    _check_manifolds(gc, exp)
    col = pl.readBatches()
    assert (col >= 0).all() and O.check_batches(gc, col, b) == 0
    order = pl.readSolveOrder()
    assert np.array_equal(np.sort(order), np.arange(len(gc)))
    ob, _ = O.solve_ordered(b, I, gc, order, iterations=10, interleave=interleave)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    assert pl.status() & ~INFO == 0


def test_bodies_dropped_on_a_mesh_come_to_rest_on_it():
    # a lattice of boxes, hulls and compounds dropped on the height field, 480 graph-captured steps
    # with the default solver; then they lie on the terrain, most at rest, and every stage from
    # the GPU's own state is bit-exact again
    sc = scenes.terrain_scene(1536, seed=3, drop=True)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000, use_cuda_graph=True)
    for _ in range(480):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() & ~INFO == 0
    b = np_.readbackAllBodiesToCpu()
    assert np.isfinite(b["pos"]).all() and np.isfinite(b["quat"]).all()
    verts = sc.shapes[0]["verts"]
    # nearly all stay on the mesh (a few roll off its edge and fall: there is nothing below it), and
    # at most a few over it went through (the reference's concave path, like this one, has no
    # continuous detection: a thin body landing at 20 m/s can pass a triangle between two steps;
    # measured: 1 of 1,536 on this seed)
    inside = (b["pos"][1:, 0] > 0) & (b["pos"][1:, 0] < 64) & (b["pos"][1:, 2] > 0) & (b["pos"][1:, 2] < 64)
    assert inside.mean() > 0.9
    assert (b["pos"][1:, 1][inside] < verts[:, 1].min() - 0.5).sum() <= 3
    speed = np.linalg.norm(b["linVel"][1:, :3], axis=1)
    assert np.percentile(speed[inside], 75) < 0.3, np.percentile(speed, [50, 75, 90, 100])
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    exp, ntri, nmesh = _expected(b, shapes, bp.getOverlappingPairsCPU())
    assert nmesh > 500
    gc = np_.getContactsCPU()
    _check_manifolds(gc, exp)
    order = pl.readSolveOrder()
    ob, _ = O.solve_ordered(b, I, gc, order, iterations=10, interleave=False)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])


def test_concave_capacity_overflow_is_flagged():
    # more triangle-convex pairs than m_maxTriConvexPairCapacity: the overflow flag is raised, the
    # first pairs' manifolds are kept, and the step goes on
    sc = scenes.terrain_scene(2048, seed=0)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000, m_maxTriConvexPairCapacity=8192,
                               solver_mode=capi.SOLVER_JACOBI)
    b = np_.readbackAllBodiesToCpu()
    run_stages(np_, bp, pl)
    assert pl.status() & capi.FLAG_CONTACT_OVERFLOW
    pairs = bp.getOverlappingPairsCPU()
    aabbs = O.aabbs(b, shapes)
    tp = O.concave_pairs(b, shapes, aabbs, pairs)
    assert len(tp) > 8192 and pl.stats().num_concave_pairs == 8192
    oc, _ = O.contacts(b, shapes, pairs)
    cc, _ = O.compound_contacts(b, shapes, O.compound_pairs(b, shapes, pairs))
    mc, _ = O.concave_contacts(b, shapes, aabbs, tp[:8192])
    _check_manifolds(np_.getContactsCPU(), np.concatenate([oc, cc, mc]))
