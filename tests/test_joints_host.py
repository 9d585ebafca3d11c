"""CPU checks of the joint path: the host joint registry behind the C ABI (create / remove by uid
/ read back, before any upload; b3GpuRigidBodyPipeline.cpp:159-219), the oracle's acos against
its error bound, and the oracle's batching (sortConstraintByBatch3) against its invariants."""
import ctypes as C

import numpy as np
import pytest

from bullet3_gb300 import capi, scenes
from bullet3_gb300.pipeline import b3Config, b3GpuNarrowPhase, b3GpuRigidBodyPipeline
from oracle import oracle as O


def _world(n=6):
    np_ = b3GpuNarrowPhase(b3Config())
    pl = b3GpuRigidBodyPipeline(np_)
    box = np_.registerConvexHullShape(scenes.box_vertices(0.5, 0.5, 0.5))
    for k in range(n):
        pl.registerPhysicsInstance(0.0 if k == 0 else 1.0, (2.0 * k, 1, 0), (0, 0, 0, 1), box)
    return np_, pl


def test_registry_create_remove_read():
    np_, pl = _world()
    u0 = pl.createPoint2PointConstraint(0, 1, (1, 0, 0), (-1, 0, 0), 5.0)
    u1 = pl.createFixedConstraint(1, 2, (1, 0, 0), (-1, 0, 0), (0, 0, 0, 1), 1e30)
    u2 = pl.createPoint2PointConstraint(2, 3, (1, 0, 0), (-1, 0, 0), 1e30)
    assert (u0, u1, u2) == (0, 1, 2) and pl.getNumConstraints() == 3
    j = pl.copyConstraintsToHost()
    assert list(j["type"]) == [capi.JOINT_POINT2POINT, capi.JOINT_FIXED, capi.JOINT_POINT2POINT]
    assert (j["flags"] == capi.CONSTRAINT_FLAG_ENABLED).all() and list(j["uid"]) == [0, 1, 2]
    assert j["breakingImpulseThreshold"][0] == 5.0 and np.array_equal(j["relTargetAB"][1], [0, 0, 0, 1])
    assert np.array_equal(j["pivotInA"][0], [1, 0, 0, 0]) and np.array_equal(j["pivotInB"][2], [-1, 0, 0, 0])
    # removal swaps the last joint into the hole (b3GpuRigidBodyPipeline::removeConstraintByUid)
    pl.removeConstraintByUid(u0)
    j = pl.copyConstraintsToHost()
    assert list(j["uid"]) == [2, 1]
    assert pl.createPoint2PointConstraint(4, 5, (0, 0, 0), (0, 0, 0), 1.0) == 3  # uids never repeat
    with pytest.raises(capi.B3GError) as e:
        pl.removeConstraintByUid(77)
    assert e.value.status == 2


def test_registry_rejects_bad_bodies():
    np_, pl = _world(3)
    for a, b in ((0, 3), (-1, 1), (1, 1)):
        with pytest.raises(capi.B3GError):
            pl.createPoint2PointConstraint(a, b, (0, 0, 0), (0, 0, 0), 1.0)
    assert pl.getNumConstraints() == 0
    with pytest.raises(capi.B3GError):
        capi.call("b3g_create_fixed_constraint", np_.world.handle, C.c_int(0), C.c_int(1), (C.c_float * 3)(),
                  (C.c_float * 3)(), None, C.c_float(1.0), None)


def test_joint_acos_error_bound():
    x = np.concatenate([np.linspace(-1, 1, 40001), 1 - np.logspace(-7, -1, 200), -1 + np.logspace(-7, -1, 200)])
    x = x.astype(np.float32)
    got = O.joint_acos(x).astype(np.float64)
    exact = np.arccos(x.astype(np.float64))
    ulp = np.spacing(exact.astype(np.float32)).astype(np.float64)
    err = np.abs(got - exact) / ulp
    assert err.max() <= 1.5, (err.max(), x[err.argmax()])
    assert O.joint_acos([1.0])[0] == 0.0


def test_oracle_batches_are_legal_and_greedy():
    sc = scenes.hanging_chains(6, 10, seed=3, fixed_every=3)
    b = np.zeros(sc.num_bodies, O.BODY)
    b["invMass"] = np.where(sc.mass > 0, 1.0 / np.maximum(sc.mass, 1e-30), 0.0)
    j = np.zeros(len(sc.joints), O.JOINT)
    j["rbA"] = [x["a"] for x in sc.joints]
    j["rbB"] = [x["b"] for x in sc.joints]
    order, off = O.joint_batches(j, b)
    assert sorted(order) == list(range(len(j)))
    for k in range(len(off) - 1):
        seen = set()
        for c in order[off[k]:off[k + 1]]:
            for body in (j["rbA"][c], j["rbB"][c]):
                # body 0 counts as dynamic even though it is static (staticIdx = -1 in the GPU solver)
                if b["invMass"][body] != 0 or body == 0:
                    assert body not in seen
                    seen.add(body)
    # every chain hangs from static body 0, so no two anchor joints share a batch
    first_links = [c for c in range(len(j)) if j["rbA"][c] == 0]
    batch_of = np.empty(len(j), int)
    for k in range(len(off) - 1):
        batch_of[order[off[k]:off[k + 1]]] = k
    assert len(set(batch_of[first_links])) == len(first_links)
    # with the anchor at a higher index, static anchor joints share batches freely
    sc2 = scenes.hanging_chains(6, 10, seed=3, anchor_index=-1)
    b2 = np.zeros(sc2.num_bodies, O.BODY)
    b2["invMass"] = np.where(sc2.mass > 0, 1.0, 0.0)
    j2 = np.zeros(len(sc2.joints), O.JOINT)
    j2["rbA"] = [x["a"] for x in sc2.joints]
    j2["rbB"] = [x["b"] for x in sc2.joints]
    _, off2 = O.joint_batches(j2, b2)
    assert len(off2) - 1 == 2  # a chain is 2-colourable


def _two_bodies(inv_mass_b, vel_b, pos_b=(0.0, 0.0, 0.0)):
    b = np.zeros(2, O.BODY)
    b["quat"][:, 3] = 1.0
    b["pos"][1, :3] = pos_b
    b["invMass"] = [0.0, inv_mass_b]
    b["linVel"][1, :3] = vel_b
    I = np.zeros(2, O.INERTIA)
    for r in range(3):
        I["invInertiaWorld"][1, r, r] = inv_mass_b  # a unit-inertia-like body
    return b, I


def _joint(kind, threshold=1e30, pivot_a=(0, 0, 0), pivot_b=(0, 0, 0)):
    j = np.zeros(1, O.JOINT)
    j["type"] = kind
    j["rbA"], j["rbB"] = 0, 1
    j["pivotInA"][0, :3] = pivot_a
    j["pivotInB"][0, :3] = pivot_b
    j["relTargetAB"][0] = (0, 0, 0, 1)
    j["breakingImpulseThreshold"] = threshold
    j["flags"] = 1
    return j


@pytest.mark.parametrize("inv_mass", [1.0, 0.5, 0.25])
@pytest.mark.parametrize("kind", [capi.JOINT_POINT2POINT, capi.JOINT_FIXED])
def test_oracle_joint_cancels_the_velocity_of_a_hanging_body(inv_mass, kind):
    # pivots coincide at the body's centre: no positional error, so the stage drives the velocity
    # along every row to zero (power-of-two masses keep every product exact)
    b, I = _two_bodies(inv_mass, (0.0, -9.8 / 60, 0.0))
    nb, nj = O.solve_joints(b, I, _joint(kind))
    assert np.array_equal(nb["linVel"][1, :3], np.zeros(3, np.float32))
    assert np.array_equal(nb["linVel"][0], b["linVel"][0])  # the static anchor is untouched
    assert nj["flags"][0] == 1


def test_oracle_joint_breaks_above_its_threshold():
    # the impulse that stops the body is m |v| = 0.163 > 0.1: the joint breaks in its first stage,
    # and a disabled joint is not solved any more
    b, I = _two_bodies(1.0, (0.0, -9.8 / 60, 0.0))
    nb, nj = O.solve_joints(b, I, _joint(capi.JOINT_POINT2POINT, threshold=0.1))
    assert nj["flags"][0] == 0
    # its rows were clamped at the threshold: the velocity change is exactly the threshold impulse
    assert np.isclose(nb["linVel"][1, 1] - b["linVel"][1, 1], 0.1, rtol=1e-6)
    nb2, nj2 = O.solve_joints(nb, I, nj)
    assert np.array_equal(nb2["linVel"], nb["linVel"]) and nj2["flags"][0] == 0


def test_oracle_joint_pulls_a_displaced_pivot_back():
    # body B's pivot sits 0.1 below the anchor's: the rows ask for a velocity of erp/dt x error
    b, I = _two_bodies(1.0, (0.0, 0.0, 0.0), pos_b=(0.0, -0.1, 0.0))
    nb, _ = O.solve_joints(b, I, _joint(capi.JOINT_POINT2POINT))
    assert np.isclose(nb["linVel"][1, 1], 0.2 * 60 * 0.1, rtol=1e-5)
    assert np.allclose(nb["linVel"][1, [0, 2]], 0.0)
