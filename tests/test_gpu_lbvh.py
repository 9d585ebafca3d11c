"""The linear-BVH broadphase (b3GpuParallelLinearBvhBroadphase) against the grid broadphase and the
oracle's brute force.

Bar: integer output, bit-exact.  The LBVH's canonical pair list equals the brute-force pair set
(and the grid's) on mixed shapes, on bodies whose sizes span two orders of magnitude, on
independent scenes sharing one region of space, and on the degenerate sizes (one or two dynamic
bodies); and since every later stage consumes only that list, whole stepped trajectories with
either broadphase are bit-identical."""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, run_stages
from bullet3_gb300 import capi, scenes
from bullet3_gb300.pipeline import b3Config, b3GpuParallelLinearBvhBroadphase
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pairs(np_, bp, pl, mode):
    pl.setBroadphase(mode)
    pl.setupGpuAabbsFull()
    bp.calculateOverlappingPairs()
    pl.synchronize()
    return pairs_xy(bp.getOverlappingPairsCPU()), bp.getAllAabbsCPU()


def _both(sc, **cfg):
    np_, bp, pl, shapes = load(sc, **cfg)
    grid, aabbs = _pairs(np_, bp, pl, capi.BROADPHASE_GRID)
    lbvh, aabbs2 = _pairs(np_, bp, pl, capi.BROADPHASE_LBVH)
    assert np.array_equal(aabbs.view(np.uint8), aabbs2.view(np.uint8))
    assert pl.status() == 0
    return grid, lbvh, aabbs


def _spheres(n, seed, rmin=0.05, rmax=5.0, extent=60.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    radii = np.exp(np.linspace(np.log(rmin), np.log(rmax), 48)).astype(np.float32)
    sc = scenes.Scene(name="sizes")
    sc.shapes = [{"type": "sphere", "radius": float(r)} for r in radii]
    sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    sc.body_shape = np.concatenate([rng.integers(0, 48, n), [48]]).astype(np.int32)
    sc.mass = np.concatenate([np.ones(n), [0.0]]).astype(np.float32)
    sc.pos = np.concatenate([rng.uniform(0, extent, (n, 3)), [[0, 0, 0]]]).astype(np.float32)
    sc.orn = np.tile(np.array([0, 0, 0, 1], np.float32), (n + 1, 1))
    return sc


@pytest.mark.parametrize("seed", [0, 1])
def test_mixed_shapes_pairs_equal_grid_and_bruteforce(seed):
    sc = scenes.mixed_scene(4096, extent=24.0, seed=seed, plane=True)
    grid, lbvh, aabbs = _both(sc, m_maxBroadphasePairs=400000)
    assert len(lbvh) > 4096
    assert np.array_equal(lbvh, grid)
    assert np.array_equal(lbvh, pairs_xy(O.pairs_bruteforce(aabbs)))


def test_sizes_over_two_decades_pairs_equal_bruteforce():
    sc = _spheres(6000, seed=3)
    grid, lbvh, aabbs = _both(sc, m_maxBroadphasePairs=2000000)
    assert np.array_equal(lbvh, pairs_xy(O.pairs_bruteforce(aabbs)))
    assert np.array_equal(lbvh, grid)


def test_scenes_sharing_space_pairs_equal_grid():
    sc = scenes.batched_piles(64, seed=5, separate=True)  # all scenes at the origin
    grid, lbvh, aabbs = _both(sc)
    assert len(lbvh) > 0 and np.array_equal(lbvh, grid)
    scene_of = sc.scene_of
    assert (scene_of[lbvh[:, 0]] == scene_of[lbvh[:, 1]]).all()


@pytest.mark.parametrize("n_dyn", [1, 2, 3])
def test_few_dynamic_bodies(n_dyn):
    sc = _spheres(n_dyn, seed=7, rmin=2.0, rmax=3.0, extent=2.0)
    grid, lbvh, aabbs = _both(sc)
    assert np.array_equal(lbvh, grid)
    assert np.array_equal(lbvh, pairs_xy(O.pairs_bruteforce(aabbs)))


def test_trajectories_bit_identical_with_either_broadphase():
    res = []
    for mode in (capi.BROADPHASE_GRID, capi.BROADPHASE_LBVH):
        sc = scenes.box_pile(8, 8, 8, seed=2)
        np_, bp, pl, shapes = load(sc, use_cuda_graph=True, broadphase=mode)
        for _ in range(60):
            pl.stepSimulation(1 / 60)
        pl.synchronize()
        assert pl.status() == 0 and pl.stats().num_pairs > 0
        res.append(np_.readbackAllBodiesToCpu())
    assert np.array_equal(res[0].view(np.uint8), res[1].view(np.uint8))


def test_broadphase_class_switches_the_world():
    sc = scenes.mixed_scene(1024, extent=12.0, seed=9, plane=True)
    cfg = b3Config(use_cuda_graph=False)
    np_, bp, pl = scenes.load_scene(sc, cfg)
    b = b3GpuParallelLinearBvhBroadphase()
    b._attach(np_)
    run_stages(np_, bp, pl)
    got = pairs_xy(bp.getOverlappingPairsCPU())
    assert np.array_equal(got, pairs_xy(O.pairs_bruteforce(bp.getAllAabbsCPU())))


def test_autotune_picks_a_broadphase_and_keeps_the_pairs():
    sc = scenes.mixed_scene(16384, extent=36.0, seed=11, plane=True)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=1000000, broadphase=capi.BROADPHASE_AUTO)
    grid, _ = _pairs(np_, bp, pl, capi.BROADPHASE_AUTO)  # AUTO before tuning: the grid
    pl.setBroadphase(capi.BROADPHASE_AUTO)
    t = pl.autotune(1 / 60, repeats=2)
    assert t["broadphase"] in (capi.BROADPHASE_GRID, capi.BROADPHASE_LBVH)
    pl.setupGpuAabbsFull()
    bp.calculateOverlappingPairs()
    pl.synchronize()
    assert np.array_equal(pairs_xy(bp.getOverlappingPairsCPU()), grid)
    assert pl.status() == 0


def test_lbvh_equals_grid_at_scale_every_step():
    # the 131,072-body collision-at-scale mix: pair lists identical at every step while it moves
    sc = scenes.mixed_scene(131072, extent=64.0, seed=0)
    np_, bp, pl, shapes = load(sc, use_cuda_graph=False)
    for step in range(4):
        grid, _ = _pairs(np_, bp, pl, capi.BROADPHASE_GRID)
        lbvh, _ = _pairs(np_, bp, pl, capi.BROADPHASE_LBVH)
        assert len(grid) > 100000 and np.array_equal(lbvh, grid), step
        pl.stepSimulation(1 / 60)
    assert pl.status() == 0


def test_million_body_pour_grid_and_lbvh_agree():
    # the 1,048,576-body pour (five static planes, mixed shapes, heights U[0, 512]): after 240 steps
    # of the pour the two pair searches, built independently, give the same pair list on 3 steps
    sc = scenes.stress_container(1048576, seed=0)
    np_, bp, pl, shapes = load(sc, use_cuda_graph=True)
    for _ in range(240):
        pl.stepSimulation(1 / 60)
    for step in range(3):
        grid, _ = _pairs(np_, bp, pl, capi.BROADPHASE_GRID)
        lbvh, _ = _pairs(np_, bp, pl, capi.BROADPHASE_LBVH)
        assert len(grid) > 100000 and np.array_equal(lbvh, grid), step
        pl.setBroadphase(capi.BROADPHASE_GRID)
        pl.stepSimulation(1 / 60)
    assert pl.status() == 0
