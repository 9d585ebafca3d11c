"""GPU joints (point to point and fixed) against the CPU restatement of the reference's joint
solver (b3GpuPgsConstraintSolver::solveJoints + kernels/jointSolver.cl).

Bar: bit-exact.  From the same bodies, inertias and joints, one joint stage on the GPU gives the
oracle's velocities and enabled flags bit for bit, and the GPU's batches equal the oracle's
restatement of sortConstraintByBatch3, step after step (the GPU integrates in between), through
joint creation, removal, breaking, and both the one-block and the grid-wide kernel shapes.
Whole-step trajectories (integration uses sinf/cosf, which differ from the host's in the last
bit) are checked with a tolerance and physical invariants."""
import numpy as np
import pytest

from gpu_helpers import load
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _stage_step(np_, pl):
    """One GPU joint stage compared with the oracle's; returns the GPU joints after it."""
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    j = pl.copyConstraintsToHost()
    pl.solveJoints()
    pl.synchronize()
    order, off = pl.readJointOrder()
    oorder, ooff = O.joint_batches(j, b)
    assert np.array_equal(order, oorder) and np.array_equal(off, ooff)
    ob, oj = O.solve_joints(b, I, j, oorder, ooff)
    gb = np_.readbackAllBodiesToCpu()
    gj = pl.copyConstraintsToHost()
    assert np.array_equal(gb["linVel"], ob["linVel"])
    assert np.array_equal(gb["angVel"], ob["angVel"])
    assert np.array_equal(gb["pos"], b["pos"]) and np.array_equal(gb["quat"], b["quat"])
    assert np.array_equal(gj["flags"], oj["flags"])
    return gj


def _run_stages(np_, pl, steps):
    for _ in range(steps):
        gj = _stage_step(np_, pl)
        pl.integrate(1 / 60)
    return gj


@pytest.mark.parametrize("anchor", [0, -1])
def test_chain_stage_bitexact(anchor):
    # anchor 0: static body 0 counts as dynamic in the batching (one batch per chain top);
    # anchor -1: a static anchor at a higher index, shared freely within a batch
    sc = scenes.hanging_chains(8, 12, seed=1, anchor_index=anchor)
    np_, bp, pl, shapes = load(sc)
    _run_stages(np_, pl, 40)
    order, off = pl.readJointOrder()
    # anchor 0: the 8 chain tops need 8 batches (6 of them single joints); else a chain's 2 colours
    assert len(off) - 1 == (8 if anchor == 0 else 2)
    assert pl.status() == 0


def test_fixed_joint_stage_bitexact():
    sc = scenes.welded_pairs(64, seed=2, twist=0.4)
    np_, bp, pl, shapes = load(sc)
    b0 = np_.readbackAllBodiesToCpu()
    _run_stages(np_, pl, 30)
    # the fixed rows act: the pairs' relative orientations move toward their targets
    b = np_.readbackAllBodiesToCpu()
    assert not np.array_equal(b["angVel"], b0["angVel"])


def test_mixed_chain_stage_bitexact_through_create_and_remove():
    sc = scenes.hanging_chains(6, 10, seed=4, fixed_every=3)
    np_, bp, pl, shapes = load(sc)
    _run_stages(np_, pl, 10)
    uids = list(pl.copyConstraintsToHost()["uid"])
    pl.removeConstraintByUid(uids[5])  # cuts a chain: its lower part falls
    pl.removeConstraintByUid(uids[0])
    u = pl.createPoint2PointConstraint(12, 25, (0.5, 0, 0), (-0.5, 0, 0), 1e30)  # links two chains
    assert u == len(uids)
    _run_stages(np_, pl, 10)
    j = pl.copyConstraintsToHost()
    assert len(j) == len(uids) - 1 and uids[5] not in list(j["uid"]) and u in list(j["uid"])


def test_breaking_thresholds_bitexact():
    sc = scenes.hanging_chains(8, 12, seed=5, threshold=0.9, swing=3.0)
    np_, bp, pl, shapes = load(sc)
    gj = _run_stages(np_, pl, 20)
    broken = gj["flags"] == 0
    assert broken.any() and not broken.all()
    # broken joints stay broken and their rows are no longer solved
    gj2 = _run_stages(np_, pl, 5)
    assert (gj2["flags"][broken] == 0).all()


def test_many_joints_grid_kernel_bitexact():
    # 24k joints, batches of 12k: the grid-wide kernel shape (cooperative launch, grid barrier)
    sc = scenes.hanging_chains(600, 40, seed=6, anchor_index=-1, fixed_every=7)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000)
    _run_stages(np_, pl, 3)
    order, off = pl.readJointOrder()
    assert np.diff(off).max() > 256
    assert pl.status() == 0


def test_graph_step_with_joints_equals_staged_step():
    res = []
    for graph in (True, False):
        sc = scenes.hanging_chains(6, 10, seed=7, fixed_every=4, ground=True)
        np_, bp, pl, shapes = load(sc, use_cuda_graph=graph)
        for s in range(60):
            if graph:
                pl.stepSimulation(1 / 60)
            else:
                pl.setupGpuAabbsFull()
                bp.calculateOverlappingPairs()
                np_.computeContacts()
                pl.solveJoints()
                pl.solveContacts(1 / 60)
                pl.integrate(1 / 60)
        pl.synchronize()
        res.append(np_.readbackAllBodiesToCpu())
    assert np.array_equal(res[0].view(np.uint8), res[1].view(np.uint8))


def _pivot_error(b, joints):
    def rot(q, v):
        u = q[:, :3]
        w = q[:, 3:4]
        t = 2.0 * np.cross(u, v)
        return v + w * t + np.cross(u, t)
    a = b["pos"][joints["rbA"], :3] + rot(b["quat"][joints["rbA"]], joints["pivotInA"][:, :3])
    c = b["pos"][joints["rbB"], :3] + rot(b["quat"][joints["rbB"]], joints["pivotInB"][:, :3])
    return np.linalg.norm(a - c, axis=1)


def test_trajectory_matches_oracle_and_chains_hold():
    # unrotated links: the fixed joints hold the identity relative orientation (with random
    # targets the reference's fixed rows, which drive wA - wB, let welded links fold and collide)
    sc = scenes.hanging_chains(8, 12, seed=8, fixed_every=5, random_orn=False)
    np_, bp, pl, shapes = load(sc, use_cuda_graph=True)
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    j = pl.copyConstraintsToHost()
    ob = b.copy()
    for s in range(120):
        pl.stepSimulation(1 / 60)
        ob, j = O.solve_joints(ob, I, j)
        ob = O.integrate(ob)
        if s % 30 == 29:
            assert pl.stats().num_contacts == 0  # joints and integration only: the oracle loop's step
    pl.synchronize()
    gb = np_.readbackAllBodiesToCpu()
    np.testing.assert_allclose(gb["pos"], ob["pos"], atol=1e-4)
    np.testing.assert_allclose(gb["linVel"], ob["linVel"], atol=1e-3)
    # 4 iterations at erp 0.2 leave the chains soft: pivots stay within 0.15 of each other
    err = _pivot_error(gb, pl.copyConstraintsToHost())
    assert err.max() < 0.15, err.max()
    # the chains swung and still hang below the anchor
    assert (gb["pos"][sc.mass > 0, 1] < b["pos"][0, 1]).all()


def test_edge_joints_static_pair_and_zero_threshold():
    # a joint between two static bodies (rows with no mass: jacDiagABInv 0, inert) and a joint whose
    # breaking threshold is 0 (|impulse| >= 0 holds at once: it breaks in its first stage)
    sc = scenes.hanging_chains(2, 3, seed=9, ground=True)
    np_, bp, pl, shapes = load(sc)
    anchor, ground = 0, sc.num_bodies - 1
    u_static = pl.createPoint2PointConstraint(anchor, ground, (0, 0, 0), (0, 5, 0), 1e30)
    u_zero = pl.createFixedConstraint(1, 4, (0, 0, 0), (0, 0, 0), (0, 0, 0, 1), 0.0)
    gj = _run_stages(np_, pl, 3)
    flags = dict(zip(gj["uid"], gj["flags"]))
    assert flags[u_zero] == 0 and flags[u_static] == 1
    b = np_.readbackAllBodiesToCpu()
    assert np.array_equal(b["linVel"][[anchor, ground]], np.zeros((2, 4), np.float32))


def test_joint_stage_matches_reference_constraint_classes():
    # 120 independent joints (ball and fixed; static or dynamic first body) against the reference's
    # own b3Point2PointConstraint / b3FixedConstraint rows solved by b3PgsJacobiSolver, each joint
    # alone (golden vectors); and bit for bit against the oracle
    from conftest import load_golden
    from gpu_helpers import scene_from_golden
    from test_oracle_golden import _joints_close
    g = load_golden("joints")
    np_, bp, pl, shapes = load(scene_from_golden(g))
    np_.writeBodiesToGpu(g["bodies"])
    for j in g["joints"]:
        if j["type"] == capi.JOINT_POINT2POINT:
            pl.createPoint2PointConstraint(int(j["rbA"]), int(j["rbB"]), j["pivotInA"], j["pivotInB"], 1e30)
        else:
            pl.createFixedConstraint(int(j["rbA"]), int(j["rbB"]), j["pivotInA"], j["pivotInB"], j["relTargetAB"],
                                     1e30)
    gj = _stage_step(np_, pl)
    _joints_close(np_.readbackAllBodiesToCpu(), g["solved"])
    assert (gj["flags"] == 1).all()
