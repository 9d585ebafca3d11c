"""The collision-at-scale and million-body configurations at full size, checked against the oracle.

  collision at scale   131,072 mixed bodies (50% boxes, 25% spheres, 25% Gaussian hulls) in a
                       64^3 box, random orientations, N(0,1) velocities, PGS 10 iterations: all
                       64 steps; every step the world AABBs and the pair set bit for bit against
                       the oracle, and the manifolds of 20,000 sampled pairs bit for bit on their
                       valid points against the oracle's contacts from the same input state
  million-body pour    1,048,576 bodies of the same mix poured into a 5-plane container: after 590
                       steps of the pour (the dense end), one step checked the same way (AABBs,
                       pair set, 60,000 sampled pairs' manifolds)

The oracle's contacts follow the reference's b3ContactConvexConvexSAT / computeContactPlaneConvex
/ computeContactSphereConvex bit for bit (tests/test_oracle_golden.py); its pair set is the exact
set the reference's dynamic-BVH broadphase yields after its tight AABB test.
"""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, valid_points_equal
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair_key(x, y):
    # (a manifold stores a static body's index negated; pairs store it as is)
    x, y = np.abs(x).astype(np.int64), np.abs(y).astype(np.int64)
    return np.minimum(x, y) << 32 | np.maximum(x, y)


def _check_step(np_, bp, pl, shapes, cell, b, rng, sample=20000):
    """AABBs and pairs of the last step bit-exact; manifolds of sampled pairs bit-exact."""
    ga = bp.getAllAabbsCPU()
    assert np.array_equal(ga.view(np.uint8), O.aabbs(b, shapes).view(np.uint8))
    gp = bp.getOverlappingPairsCPU()
    op = O.pairs_grid(ga, cell, cap=max(1024, 2 * len(gp)))
    assert np.array_equal(pairs_xy(gp), pairs_xy(op))
    pick = np.sort(rng.choice(len(gp), size=min(sample, len(gp)), replace=False))
    ref, _ = O.contacts(b, shapes, gp[pick])
    gc = np_.getContactsCPU()
    gk = _pair_key(gc["bodyA"], gc["bodyB"])
    order = np.argsort(gk)
    rk = _pair_key(ref["bodyA"], ref["bodyB"])
    at = np.searchsorted(gk[order], rk)
    assert (at < len(gk)).all() and np.array_equal(gk[order][at], rk)
    mine = gc[order][at]
    assert valid_points_equal(mine, ref)
    # the sampled pairs without an oracle manifold have no GPU manifold either
    sk = _pair_key(gp["x"][pick], gp["y"][pick])
    with_manifold = np.isin(sk, gk)
    assert with_manifold.sum() == len(ref)
    return len(gp), len(gc), len(ref)


def test_collision_at_scale_64_steps():
    sc = scenes.mixed_scene(131072, extent=64.0, seed=0)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, use_cuda_graph=True)
    rng = np.random.Generator(np.random.PCG64(11))
    checked = 0
    for step in range(64):
        b = np_.readbackAllBodiesToCpu()
        pl.stepSimulation(1 / 60)
        pl.synchronize()
        npairs, nman, nref = _check_step(np_, bp, pl, shapes, sc.cell, b, rng)
        assert npairs > 100000 and nref > 500, step
        checked += nref
    assert pl.status() == 0
    assert checked > 64 * 500


def test_million_body_pour_dense_step():
    sc = scenes.stress_container(1048576, seed=0)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=16, residual_tol=1e-4,
                               use_cuda_graph=True, warm_start=capi.WARM_PERSISTENT)
    for _ in range(590):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    # (a persistent warm start that did worse than a cold start was dropped: informational)
    assert pl.status() & ~capi.FLAG_WARM_DISCARDED == 0
    b = np_.readbackAllBodiesToCpu()
    pl.stepSimulation(1 / 60)
    pl.synchronize()
    rng = np.random.Generator(np.random.PCG64(12))
    # (one pair in eight has a manifold at the dense end: 60,000 sampled pairs give ~7,500)
    npairs, nman, nref = _check_step(np_, bp, pl, shapes, sc.cell, b, rng, sample=60000)
    # the dense end of the pour: most bodies rest on others
    assert npairs > 2_000_000 and nman > 1_000_000 and nref > 5000
    assert pl.status() & ~capi.FLAG_WARM_DISCARDED == 0
