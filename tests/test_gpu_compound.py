"""Compounds of convex hulls on the GPU through the C ABI, against the oracle on the same inputs
(the oracle's compound path is pinned bit for bit to the reference's compound kernels by the
golden fixture compound.npz).

Bars: pair sets bit-exact; manifolds bit-exact on their valid points, in the GPU's order (the
pairs' own manifolds, then one per touching child pair in (pair, child of A, child of B) order,
with the child indices the reference stores); Jacobi velocities bit-exact; PGS velocities bit-exact
against the oracle sweeping the GPU's colour order; a settling pile keeps its bodies above the
plane (penetration below 0.1).
"""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, run_stages, valid_points_equal
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

INFO = capi.FLAG_WARM_DISCARDED  # informational, not an error


def _expected(b, shapes, pairs):
    oc, _ = O.contacts(b, shapes, pairs)
    cp = O.compound_pairs(b, shapes, pairs)
    cc, _ = O.compound_contacts(b, shapes, cp)
    return np.concatenate([oc, cc]), len(oc), cp


def _rotate(q, v):
    # rotate the rows of v by the unit quaternion q (x, y, z, w)
    u, w = q[:3].astype(np.float64), float(q[3])
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def _qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by + ay * bw + az * bx - ax * bz,
                     aw * bz + az * bw + ax * by - ay * bx, aw * bw - ax * bx - ay * by - az * bz])


def _lowest_points(b, shapes):
    """The lowest vertex (world y) of every body's hulls: its own, or its children's at their poses."""
    cols, hulls, verts = shapes.collidables, shapes.hulls, shapes.verts
    children = np.ascontiguousarray(shapes.children).view(O.CHILD)
    out = np.full(len(b), np.inf)

    def hull_low(col, pos, q):
        h = hulls[cols[col]["shapeIndex"]]
        v = verts[h["vertexOffset"]:h["vertexOffset"] + h["numVertices"], :3].astype(np.float64)
        return float((_rotate(q, v) + pos)[:, 1].min())

    for i, body in enumerate(b):
        c = cols[body["collidableIdx"]]
        pos, q = body["pos"][:3].astype(np.float64), body["quat"].astype(np.float64)
        if c["shapeType"] == capi.SHAPE_CONVEX_HULL:
            out[i] = hull_low(body["collidableIdx"], pos, q)
        elif c["shapeType"] == capi.SHAPE_COMPOUND:
            for k in range(c["numChildShapes"]):
                ch = children[c["shapeIndex"] + k]
                cpos = pos + _rotate(q, ch["pos"][None, :3].astype(np.float64))[0]
                out[i] = min(out[i], hull_low(ch["shapeIndex"], cpos, _qmul(q, ch["orn"])))
    return out


def _check_manifolds(gc, exp):
    assert valid_points_equal(gc, exp)
    assert np.array_equal(gc["childA"], exp["childA"]) and np.array_equal(gc["childB"], exp["childB"])


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("broadphase", [capi.BROADPHASE_GRID, capi.BROADPHASE_LBVH])
def test_compound_stages_bitexact(seed, broadphase):
    sc = scenes.compound_scene(2048, seed=seed)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000, solver_mode=capi.SOLVER_JACOBI,
                               broadphase=broadphase)
    b = np_.readbackAllBodiesToCpu()
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    ga = bp.getAllAabbsCPU()
    assert np.array_equal(ga.view(np.uint8), O.aabbs(b, shapes).view(np.uint8))
    op = O.pairs_bruteforce(ga)
    assert np.array_equal(pairs_xy(bp.getOverlappingPairsCPU()), pairs_xy(op))
    exp, nplain, cp = _expected(b, shapes, op)
    assert len(cp) > 20000 and len(exp) - nplain > 2000  # child manifolds dominate
    gc = np_.getContactsCPU()
    _check_manifolds(gc, exp)
    ob, oimp, _, _ = O.solve(b, I, exp, mode=1, iterations=10)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])
    assert np.array_equal(pl.readImpulses(), oimp)
    assert pl.status() & ~INFO == 0


@pytest.mark.parametrize("interleave", [False, True])
def test_compound_pgs_colour_order_bitexact(interleave):
    sc = scenes.compound_scene(2048, seed=2)
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


def test_compound_pile_settles_and_stays_bitexact():
    # a lattice of compounds, boxes and hulls dropped on the plane, 480 graph-captured steps with
    # the default solver (carried colours, recolouring every 8 solves); then every stage from the
    # GPU's own state is bit-exact again
    sc = scenes.compound_scene(2048, seed=3, lattice=True)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000, use_cuda_graph=True)
    for _ in range(480):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() & ~INFO == 0
    b = np_.readbackAllBodiesToCpu()
    assert np.isfinite(b["pos"]).all() and np.isfinite(b["quat"]).all()
    # no body sank through the plane: every hull's lowest vertex, the compounds' children's too,
    # stays above -0.1
    assert _lowest_points(b[1:], shapes).min() > -0.1
    # and most of the pile came to rest (a resting body carries the step's gravity, 9.8 / 60 m/s;
    # a fall from the top row lands at 15 m/s; an exploding pile throws bodies faster still), save
    # the bodies rolling off it
    speed = np.linalg.norm(b["linVel"][1:, :3], axis=1)
    assert np.percentile(speed, 90) < 0.35 and speed.max() < 3.0, np.percentile(speed, [50, 90, 99, 100])
    I = np_.readInertiasToCpu()
    run_stages(np_, bp, pl)
    exp, nplain, _ = _expected(b, shapes, bp.getOverlappingPairsCPU())
    gc = np_.getContactsCPU()
    assert len(exp) - nplain > 1000
    _check_manifolds(gc, exp)
    order = pl.readSolveOrder()
    ob, _ = O.solve_ordered(b, I, gc, order, iterations=10, interleave=False)
    gb = np_.readbackAllBodiesToCpu()
    assert np.array_equal(gb["linVel"], ob["linVel"]) and np.array_equal(gb["angVel"], ob["angVel"])


def test_compound_capacity_overflow_is_flagged():
    # more child pairs than max_compound_child_pairs: the overflow flag is raised, the manifolds
    # kept are the first child pairs', and the step goes on
    sc = scenes.compound_scene(2048, seed=0)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000, m_compoundPairCapacity=4096,
                               solver_mode=capi.SOLVER_JACOBI)
    b = np_.readbackAllBodiesToCpu()
    run_stages(np_, bp, pl)
    assert pl.status() & capi.FLAG_CONTACT_OVERFLOW
    exp, nplain, cp = _expected(b, shapes, bp.getOverlappingPairsCPU())
    assert len(cp) > 4096
    cc, _ = O.compound_contacts(b, shapes, cp[:4096])
    gc = np_.getContactsCPU()
    _check_manifolds(gc, np.concatenate([exp[:nplain], cc]))
