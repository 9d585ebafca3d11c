"""GPU parity through the C ABI, stage by stage, against the reference's golden vectors and the
CPU oracle on the same inputs.

Bars (stated per test): pair sets bit-exact; manifolds bit-exact on their valid points (the kernels
follow the reference's operation order and are compiled without FMA contraction); Jacobi
velocities bit-exact; PGS velocities bit-exact against the oracle solving the same manifolds in the
GPU's colour order, and batches legal; integrated poses within 1e-6 relative (sinf/cosf).
"""
import numpy as np
import pytest

from conftest import load_golden
from gpu_helpers import load, pairs_xy, run_stages, scene_from_golden, valid_points_equal
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _write_golden_state(np_, d):
    b = np_.readbackAllBodiesToCpu()
    assert len(b) == len(d["bodies"])
    b["linVel"], b["angVel"] = d["bodies"]["linVel"], d["bodies"]["angVel"]
    np_.writeBodiesToGpu(b)
    return b


@pytest.mark.parametrize("name", ["pile", "mixed"])
def test_golden_stages_match_reference(name):
    d = load_golden(name)
    np_, bp, pl, shapes = load(scene_from_golden(d))
    b = _write_golden_state(np_, d)
    run_stages(np_, bp, pl, solve=False)
    # AABBs: bit-exact with the reference's b3TransformAabb2
    ga = bp.getAllAabbsCPU()
    assert np.array_equal(ga.view(np.uint8), d["aabbs"].view(np.uint8))
    # pairs: bit-exact with the reference's filtered dynamic-BVH pair set
    assert np.array_equal(pairs_xy(bp.getOverlappingPairsCPU()), d["pairs"])
    # manifolds: bit-exact with the reference's CPU contact code where it has some
    gc = np_.getContactsCPU()
    oc, pr = O.contacts(b, shapes, bp.getOverlappingPairsCPU())
    assert valid_points_equal(gc, oc)
    has = np.where(pr["z"] >= 0)[0]
    keep = [i for i, p in enumerate(has) if p in set(d["contact_pair"].tolist())]
    assert valid_points_equal(gc[keep], d["contacts"])


@pytest.mark.parametrize("name", ["pile", "mixed"])
@pytest.mark.parametrize("iters", [1, 10])
def test_golden_jacobi_bitexact(name, iters):
    d = load_golden(name)
    np_, bp, pl, shapes = load(scene_from_golden(d), solver_mode=capi.SOLVER_JACOBI, solver_iterations=iters)
    b = _write_golden_state(np_, d)
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    oc, _ = O.contacts(b, shapes, bp.getOverlappingPairsCPU())
    ob, oimp, it, res = O.solve(b, I, oc, mode=1, iterations=iters)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    gimp = pl.readImpulses()
    assert np.array_equal(gimp, oimp)


@pytest.mark.parametrize("name", ["pile", "mixed"])
@pytest.mark.parametrize("interleave", [False, True])
def test_golden_pgs_colour_order_bitexact(name, interleave):
    d = load_golden(name)
    np_, bp, pl, shapes = load(scene_from_golden(d), solver_mode=capi.SOLVER_PGS, solver_iterations=10,
                               pgs_interleave=interleave)
    b = _write_golden_state(np_, d)
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    gc = np_.getContactsCPU()
    col = pl.readBatches()
    assert (col >= 0).all()
    # batch legality (integer, exact): no dynamic body twice in a colour
    assert O.check_batches(gc, col, b) == 0
    # the GPU's processing order (block partitions, then cross-partition colours) is a permutation
    # whose sequential Gauss-Seidel sweep the oracle reproduces bit for bit
    order = pl.readSolveOrder()
    assert np.array_equal(np.sort(order), np.arange(len(col)))
    ob, _ = O.solve_ordered(b, I, gc, order, iterations=10, interleave=interleave)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    st = pl.stats()
    assert st.num_colors == col.max() + 1 and st.status == 0


def test_integrate_matches_oracle():
    d = load_golden("pile")
    np_, bp, pl, shapes = load(scene_from_golden(d))
    b = _write_golden_state(np_, d)
    pl.integrate(1 / 60)
    pl.synchronize()
    gb = np_.readbackAllBodiesToCpu()
    ob = O.integrate(b)
    np.testing.assert_allclose(gb["pos"], ob["pos"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(gb["quat"], ob["quat"], rtol=1e-6, atol=1e-7)
    assert np.array_equal(gb["linVel"], ob["linVel"])


@pytest.mark.parametrize("seed", [0, 1])
def test_mixed_scene_stages_bitexact(seed):
    # the C1 shape mix (boxes, Gaussian hulls, spheres, random orientations, N(0,1) velocities), 4k bodies
    sc = scenes.mixed_scene(4096, extent=24.0, seed=seed, plane=True)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000, solver_mode=capi.SOLVER_JACOBI)
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    ga = bp.getAllAabbsCPU()
    assert np.array_equal(ga.view(np.uint8), O.aabbs(b, shapes).view(np.uint8))
    gp = bp.getOverlappingPairsCPU()
    op = O.pairs_grid(ga, sc.cell)
    assert np.array_equal(pairs_xy(gp), pairs_xy(op))
    assert np.array_equal(pairs_xy(op), pairs_xy(O.pairs_bruteforce(ga)))
    gc = np_.getContactsCPU()
    oc, _ = O.contacts(b, shapes, op)
    assert valid_points_equal(gc, oc)
    ob, _, _, _ = O.solve(b, I, oc, mode=1, iterations=10)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    assert pl.status() == 0


def test_box_pile_trajectory_jacobi():
    # 1,000-box lattice on a plane, 120 steps: every stage bit-exact per step (from the GPU's own
    # state), and after 120 graph-captured steps the poses stay within 1e-3 of an oracle trajectory
    sc = scenes.box_pile(10, 10, 10, seed=0)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_JACOBI, solver_iterations=10)
    I = np_.readInertiasToCpu()
    dt = 1 / 60
    ob = np_.readbackAllBodiesToCpu()
    for step in range(120):
        gb = np_.readbackAllBodiesToCpu()
        run_stages(np_, bp, pl, dt)
        op = O.pairs_bruteforce(O.aabbs(gb, shapes))
        assert np.array_equal(pairs_xy(bp.getOverlappingPairsCPU()), pairs_xy(op)), step
        oc, _ = O.contacts(gb, shapes, op)
        assert valid_points_equal(np_.getContactsCPU(), oc), step
        sb, _, _, _ = O.solve(gb, I, oc, mode=1, iterations=10)
        after = np_.readbackAllBodiesToCpu()
        assert np.array_equal(after["linVel"], sb["linVel"]), step
        pl.integrate(dt)
        ob, _, _, _ = O.step(ob, I, shapes, dt=dt, mode=1, iterations=10, use_grid=False)
    pl.synchronize()
    gb = np_.readbackAllBodiesToCpu()
    assert np.abs(gb["pos"] - ob["pos"]).max() < 1e-3
    assert gb["pos"][1:, 1].min() > 0.4  # resting on the plane, no tunnelling


@pytest.mark.parametrize("interleave", [False, True])
def test_pgs_residual_and_penetration_bounds(interleave):
    # order-sensitive PGS: colour-order GPU solve vs the reference's sequential order (same row
    # interleaving mode) on the same manifolds -- same contact residual class and penetration bounds
    sc = scenes.box_stack(8, 16, 8, seed=1)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, pgs_interleave=interleave)
    I = np_.readInertiasToCpu()
    dt = 1 / 60
    mode = 2 if interleave else 0
    ob = np_.readbackAllBodiesToCpu()
    for _ in range(30):
        pl.stepSimulation(dt)
        ob, _, _, _ = O.step(ob, I, shapes, dt=dt, mode=mode, iterations=10, use_grid=False)
    pl.synchronize()
    b = np_.readbackAllBodiesToCpu()

    def deepest(bodies):
        c, _ = O.contacts(bodies, shapes, O.pairs_bruteforce(O.aabbs(bodies, shapes)))
        return c["worldPosB"][..., 3][np.arange(4)[None, :] < c["normal"][:, 3:4].astype(int)].min()

    # Gauss-Seidel in colour order propagates support fewer levels per sweep than the reference's
    # bottom-up sequential order on tall stacks; the stated bound: the deepest penetration after 30
    # steps is at most 2.25 times the sequential order's (measured: 38.4 mm vs 19.1 mm on 16-high
    # stacks with colours carried from step to step)
    assert deepest(b) >= 2.25 * deepest(ob)
    run_stages(np_, bp, pl, dt)
    gc = np_.getContactsCPU()
    gpu_res = pl.stats().residual
    _, _, _, seq_res = O.solve(b, I, gc, mode=mode, iterations=10)
    assert gpu_res < max(2.0 * seq_res, 0.05)
    assert pl.status() == 0


def test_determinism():
    out = []
    for _ in range(2):
        sc = scenes.mixed_scene(2048, extent=16.0, seed=5, plane=True)
        np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=300000)
        for _ in range(10):
            pl.stepSimulation(1 / 60)
        pl.synchronize()
        out.append(np_.readbackAllBodiesToCpu())
    assert np.array_equal(out[0].view(np.uint8), out[1].view(np.uint8))


def test_graph_step_equals_staged_step():
    res = []
    for graph in (True, False):
        sc = scenes.box_pile(6, 6, 6, seed=3)
        np_, bp, pl, shapes = load(sc, use_cuda_graph=graph)
        for _ in range(40):
            pl.stepSimulation(1 / 60)
        pl.synchronize()
        res.append(np_.readbackAllBodiesToCpu())
    assert np.array_equal(res[0].view(np.uint8), res[1].view(np.uint8))


@pytest.mark.parametrize("parts", [capi.PGS_PARTITIONS_AUTO, capi.PGS_PARTITIONS_SHARED,
                                   capi.PGS_PARTITIONS_STREAMED, capi.PGS_PARTITIONS_GLOBAL_DELTAS,
                                   capi.PGS_PARTITIONS_NONE])
@pytest.mark.parametrize("scene", ["stack", "mixed"])
@pytest.mark.parametrize("interleave", [False, True])
def test_pgs_partitioned_solve_bitexact(parts, scene, interleave):
    # every PGS work split (block-owned body ranges with shared- or global-memory deltas, or
    # grid-wide colours only) is a legal Gauss-Seidel order: the oracle sweeping the GPU's
    # reported order over the GPU's own manifolds reproduces the velocities bit for bit
    if scene == "stack":
        sc = scenes.box_stack(16, 16, 16, seed=2)
        np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, pgs_partitions=parts,
                                   pgs_interleave=interleave)
    else:
        sc = scenes.mixed_scene(4096, extent=20.0, seed=3, plane=True)
        np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000, solver_mode=capi.SOLVER_PGS,
                                   solver_iterations=10, pgs_partitions=parts, pgs_interleave=interleave)
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    gc = np_.getContactsCPU()
    assert len(gc) > 1000
    col = pl.readBatches()
    assert (col >= 0).all() and O.check_batches(gc, col, b) == 0
    order = pl.readSolveOrder()
    assert np.array_equal(np.sort(order), np.arange(len(gc)))
    ob, _ = O.solve_ordered(b, I, gc, order, iterations=10, interleave=interleave)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    st = pl.stats()
    assert st.status == 0 and st.num_colors == col.max() + 1


def test_collision_at_scale_pair_sets_every_step():
    # the collision-at-scale shapes at full size: 131,072 bodies in a 64^3 box (boxes, spheres,
    # Gaussian hulls, random orientations, N(0,1) velocities), grid cell 2x the largest AABB
    # extent, PGS 10 iterations; the pair set of every step is checked bit for bit against the
    # oracle's grid pair search over the same AABBs, and the AABBs against the oracle's from the
    # step's input bodies
    sc = scenes.mixed_scene(131072, extent=64.0, seed=0)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, use_cuda_graph=True)
    for step in range(4):
        b = np_.readbackAllBodiesToCpu()
        pl.stepSimulation(1 / 60)
        pl.synchronize()
        ga = bp.getAllAabbsCPU()
        assert np.array_equal(ga.view(np.uint8), O.aabbs(b, shapes).view(np.uint8)), step
        gp = pairs_xy(bp.getOverlappingPairsCPU())
        assert len(gp) > 100000
        assert np.array_equal(gp, pairs_xy(O.pairs_grid(ga, sc.cell))), step
    assert pl.status() == 0


@pytest.mark.parametrize("flow", [1, 2])
@pytest.mark.parametrize("interleave", [False, True])
def test_pgs_carried_colours_bitexact(interleave, flow):
    # grid-wide PGS colours the manifolds before the row setup and carries each body pair's colour
    # over from the last solve (from scratch again every 8 solves and after a host write of the
    # bodies); after many steps, and after bodies switched between static and dynamic, the
    # batches stay legal and the solve equals the oracle sweeping the GPU's reported order bit for
    # bit
    # (flow 1: the dataflow sweeps with per-body update counters; 2: a grid barrier per colour)
    sc = scenes.box_stack(12, 16, 12, seed=4)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, solver_iterations=10, use_cuda_graph=True,
                               pgs_partitions=capi.PGS_PARTITIONS_NONE, pgs_interleave=interleave, pgs_flow=flow)
    for _ in range(12):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    first_colours = pl.stats().num_colors
    b = np_.readbackAllBodiesToCpu()
    flip = np.arange(1, len(b), 7)
    saved = b["invMass"][flip].copy()
    b["invMass"][flip] = 0.0
    np_.writeBodiesToGpu(b)
    for _ in range(3):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    b = np_.readbackAllBodiesToCpu()
    b["invMass"][flip] = saved
    np_.writeBodiesToGpu(b)
    for _ in range(3):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    gc = np_.getContactsCPU()
    assert len(gc) > 2000
    col = pl.readBatches()
    assert (col >= 0).all() and O.check_batches(gc, col, b) == 0
    order = pl.readSolveOrder()
    assert np.array_equal(np.sort(order), np.arange(len(gc)))
    assert (np.diff(col[order]) >= 0).all()  # records in colour order
    ob, _ = O.solve_ordered(b, I, gc, order, iterations=10, interleave=interleave)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    st = pl.stats()
    assert st.status == 0 and st.num_colors == col.max() + 1 and st.num_colors <= first_colours + 4


@pytest.mark.parametrize("tail", [1, 32, 1024, 1 << 30])
def test_pgs_trailing_colours_in_one_block_bitexact(tail):
    # the trailing small colours run in one block (one grid barrier for all of them); any split
    # point gives the same Gauss-Seidel order, so the velocities equal the oracle's either way
    sc = scenes.mixed_scene(4096, extent=20.0, seed=3, plane=True)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000, solver_mode=capi.SOLVER_PGS, solver_iterations=10,
                               pgs_partitions=capi.PGS_PARTITIONS_NONE, pgs_tail_manifolds=tail, pgs_flow=2)
    for _ in range(3):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    gc = np_.getContactsCPU()
    order = pl.readSolveOrder()
    ob, _ = O.solve_ordered(b, I, gc, order, iterations=10, interleave=False)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    assert pl.status() == 0
