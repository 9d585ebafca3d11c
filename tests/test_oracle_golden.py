"""The CPU oracle against golden vectors produced by the reference's own CPU code.

Pins oracle/b3oracle.c (the checker every GPU parity test uses) to the reference:
b3TransformAabb2, the dynamic-BVH pair set filtered by the tight test, b3ContactConvexConvexSAT,
computeContactPlaneConvex, computeContactSphereConvex, b3PgsJacobiSolver (PGS and Jacobi) and
integrateSingleTransform, plus a 30-step composed trajectory; the registration path
(b3ConvexHullComputer + b3ConvexUtility hull tables, registerPhysicsInstance body and inertia
records) that the CPU legs use to build their scenes; and the compound path
(processCompoundPairsKernel + clipCompoundsHullHullKernel host twins, computeContactPlaneCompound).
"""
import numpy as np
import pytest

from conftest import load_golden, shapes_from
from oracle import oracle as O


def _pairs_xy(p):
    return np.stack([p["x"], p["y"]], 1)


@pytest.mark.parametrize("name", ["pile", "mixed"])
def test_aabbs_bitexact(name):
    d = load_golden(name)
    sh = shapes_from(d)
    a = O.aabbs(d["bodies"], sh)
    assert np.array_equal(a.view(np.uint8), d["aabbs"].view(np.uint8))


@pytest.mark.parametrize("name", ["pile", "mixed"])
def test_pairs_bitexact(name):
    d = load_golden(name)
    bf = O.pairs_bruteforce(d["aabbs"])
    assert np.array_equal(_pairs_xy(bf), d["pairs"])
    cell = float(np.max(d["aabbs"]["max"][d["aabbs"]["maxw"] == 1] - d["aabbs"]["min"][d["aabbs"]["maxw"] == 1]))
    gr = O.pairs_grid(d["aabbs"], cell)
    assert np.array_equal(_pairs_xy(gr), d["pairs"])


def test_touching_aabbs_known_answer():
    # test/b3DynamicBvhBroadphase/main.cpp:40-69: [0,1]^3 and [1,2]^3 touch -> exactly one pair
    d = load_golden("kat_aabb")
    assert d["pairs"].tolist() == [[0, 1]]
    assert _pairs_xy(O.pairs_bruteforce(d["aabbs"])).tolist() == [[0, 1]]
    assert _pairs_xy(O.pairs_grid(d["aabbs"], 1.0)).tolist() == [[0, 1]]


@pytest.mark.parametrize("name", ["pile", "mixed"])
def test_contacts_match_reference(name):
    d = load_golden(name)
    sh = shapes_from(d)
    pairs = np.zeros(len(d["pairs"]), O.PAIR)
    pairs["x"], pairs["y"] = d["pairs"][:, 0], d["pairs"][:, 1]
    c, pr = O.contacts(d["bodies"], sh, pairs)
    has = np.where(pr["z"] >= 0)[0]
    # the reference has no CPU sphere-sphere / plane-sphere code: compare the other pairs
    types = sh.collidables["shapeType"][d["bodies"]["collidableIdx"]]
    ta, tb = types[d["pairs"][:, 0]], types[d["pairs"][:, 1]]
    covered = ~(((ta == 7) & (tb == 7)) | ((ta == 4) & (tb == 7)) | ((ta == 7) & (tb == 4)))
    mine = [i for i, p in enumerate(has) if covered[p]]
    assert np.array_equal(has[mine], d["contact_pair"])
    ref = d["contacts"]
    got = c[mine]
    assert len(got) == len(ref) > 0
    np.testing.assert_array_equal(got["normal"][:, 3], ref["normal"][:, 3])  # point counts
    npts = ref["normal"][:, 3].astype(int)
    valid = np.arange(4)[None, :] < npts[:, None]
    # stated tolerance: 1e-5 relative on points, depths and normals
    np.testing.assert_allclose(got["worldPosB"][valid], ref["worldPosB"][valid], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(got["normal"], ref["normal"], rtol=1e-5, atol=1e-6)
    assert np.array_equal(got["bodyA"], ref["bodyA"]) and np.array_equal(got["bodyB"], ref["bodyB"])
    assert np.array_equal(got["frictionCmp"], ref["frictionCmp"])
    # on this machine the restatement reproduces the reference bit-for-bit
    assert np.array_equal(got["worldPosB"][valid], ref["worldPosB"][valid])
    assert np.array_equal(got["normal"], ref["normal"])


@pytest.mark.parametrize("name", ["pile", "mixed"])
@pytest.mark.parametrize("mode,key", [(0, "pgs"), (1, "jacobi"), (2, "pgsi")])
@pytest.mark.parametrize("iters", [1, 10])
def test_solver_matches_reference(name, mode, key, iters):
    d = load_golden(name)
    b, imp, it, res = O.solve(d["bodies"], d["inertias"], d["contacts"], mode=mode, iterations=iters)
    ref = d[f"{key}_bodies_{iters}"]
    np.testing.assert_allclose(b["linVel"], ref["linVel"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(b["angVel"], ref["angVel"], rtol=1e-5, atol=1e-6)
    assert it == iters


@pytest.mark.parametrize("name", ["pile", "mixed"])
def test_integrate_matches_reference(name):
    d = load_golden(name)
    b = O.integrate(d["jacobi_bodies_10"])
    ref = d["integrated"]
    np.testing.assert_allclose(b["pos"], ref["pos"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(b["quat"], ref["quat"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(b["linVel"], ref["linVel"], rtol=1e-6, atol=1e-6)


def test_composed_trajectory_matches_reference():
    d = load_golden("trajectory")
    sh = shapes_from(d)
    traj = d["traj"]
    b = traj[0].copy()
    worst = 0.0
    for s in range(1, len(traj)):
        b, nc, npairs, npts = O.step(b, d["inertias"], sh, mode=1, iterations=10, use_grid=False)
        worst = max(worst, float(np.abs(b["pos"] - traj[s]["pos"]).max()))
    # stated tolerance for poses after 30 steps: 1e-4 absolute (transcendentals in the integrator)
    assert worst < 1e-4, worst


def _hull_fixtures():
    for name in ("hulls", "registration"):
        g = load_golden(name)
        for i in range(int(g["count"])):
            yield g[f"in_{i}"], (g[f"v_{i}"], g[f"p_{i}"], g[f"fc_{i}"], g[f"ix_{i}"], g[f"e_{i}"])


def test_hull_tables_bitexact():
    """Vertices, face planes, face polygons (same faces, same order, same start vertex) and unique
    edges of 170 point clouds equal the reference's bit for bit, welded faces included."""
    n = 0
    for pts, ref in _hull_fixtures():
        mine = O.hull(pts)
        for a, b in zip(mine[:5], ref):
            assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))
        c = np.zeros(3, np.float32)
        for p in ref[0]:
            c = (c + p).astype(np.float32)
        assert np.array_equal(mine[5], (c * np.float32(1.0 / np.float32(len(ref[0])))).astype(np.float32))
        n += 1
    assert n == 170


def test_body_registration_bitexact():
    g = load_golden("registration")
    reg = O.Registry()
    for i in range(len(g["bodies"])):
        reg.laabbs.append(np.zeros(1, O.AABB)[0])
        reg.laabbs[-1]["min"], reg.laabbs[-1]["max"] = g["body_local_min"][i], g["body_local_max"][i]
        reg.body(float(g["body_mass"][i]), g["body_pos"][i], g["body_orn"][i], len(reg.laabbs) - 1)
    t = reg.tables()
    t["bodies"]["collidableIdx"] = 3  # the fixture registers every body with collidable 3
    assert t["bodies"].tobytes() == g["bodies"].tobytes()
    assert t["inertias"].tobytes() == g["inertias"].tobytes()


def _ray_close(mine, ref, rays):
    """Hits of the ray kernels against the reference's host twin b3GpuRaycast::castRaysHost: the
    same rays hit the same bodies (the same faces: equal normals within 1 ulp); the twin moves each
    ray into the body's frame with b3Transform::inverse, the kernels with quaternion rotations, so
    fractions agree within 4e-6 and hit points within 4e-6 of the ray length."""
    hit = ref["hitBody"] >= 0
    assert np.array_equal(mine["hitBody"], ref["hitBody"])
    assert np.abs(mine["hitFraction"][hit] - ref["hitFraction"][hit]).max() <= 4e-6
    assert np.abs(mine["hitNormal"][hit] - ref["hitNormal"][hit]).max() <= 2.5e-7
    length = np.linalg.norm(rays["to"][:, :3] - rays["from"][:, :3], axis=1)[hit]
    assert (np.abs(mine["hitPoint"][hit, :3] - ref["hitPoint"][hit, :3]).max(1) <= 4e-6 * length + 1e-6).all()
    return hit


def test_rays_match_reference_host_twin():
    g = load_golden("rays")
    o = O.cast_rays(g["bodies"], shapes_from(g), g["rays"])
    hit = _ray_close(o, g["hits"], g["rays"])
    assert hit.sum() > 1000


def _joints_close(mine, ref):
    """One joint stage against the reference's CPU constraint classes solved by b3PgsJacobiSolver:
    the velocities agree within 1e-5 of max(|v|, 1) (the CPU rows round a few operations
    differently from the joint kernels the oracle and the GPU follow; measured 3.1e-6)."""
    for f in ("linVel", "angVel"):
        d = np.abs(mine[f][:, :3] - ref[f][:, :3])
        assert (d <= 1e-5 * np.maximum(np.abs(ref[f][:, :3]), 1.0)).all(), (f, d.max())


def test_joints_match_reference_constraint_classes():
    g = load_golden("joints")
    ob, oj = O.solve_joints(g["bodies"], g["inertias"], g["joints"])
    _joints_close(ob, g["solved"])
    assert (oj["flags"] == 1).all()


def _manifold_equal(a, b):
    n = int(b["normal"][3])
    return (np.array_equal(a["normal"], b["normal"]) and np.array_equal(a["worldPosB"][:n], b["worldPosB"][:n])
            and a["bodyA"] == b["bodyA"] and a["bodyB"] == b["bodyB"] and a["frictionCmp"] == b["frictionCmp"])


def test_compound_contacts_match_reference_kernels():
    # compound children against hulls and other compounds: the reference's own kernel host twins
    # (processCompoundPairsKernel's three separating-axis passes, clipCompoundsHullHullKernel's clip
    # and reduction) give these manifolds; the oracle reproduces them bit for bit, child indices too
    d = load_golden("compound")
    sh = shapes_from(d)
    b = d["bodies"]
    cp = O.compound_pairs(b, sh, d["pairs"])
    assert np.array_equal(cp.view(np.int32), d["child_pairs"].view(np.int32))
    mine, idx = O.compound_contacts(b, sh, cp)
    by_child = {int(i): m for m, i in zip(mine, idx)}
    ref = d["hull_contacts"]
    assert len(ref) > 1000
    for r, i in zip(ref, d["hull_child_index"]):
        m = by_child[int(i)]
        assert _manifold_equal(m, r) and m["childA"] == r["childA"] and m["childB"] == r["childB"], int(i)
    # and no other hull child pair has one
    def hull_side(body, child):
        return child >= 0 or sh.collidables[b[body]["collidableIdx"]]["shapeType"] == 3
    hull_mine = {int(i) for i in idx if hull_side(cp[i]["x"], cp[i]["z"]) and hull_side(cp[i]["y"], cp[i]["w"])}
    assert hull_mine == set(int(i) for i in d["hull_child_index"])


def test_plane_compound_contacts_match_reference():
    # computeContactPlaneCompound: one manifold per child below the plane, in child order
    d = load_golden("compound")
    sh = shapes_from(d)
    b = d["bodies"]
    cp = O.compound_pairs(b, sh, d["pairs"])
    mine, idx = O.compound_contacts(b, sh, cp)
    ref, owner = d["plane_contacts"], d["plane_owner"]
    assert len(ref) > 50
    for k, (x, y) in enumerate(d["plane_pairs"]):
        r = ref[owner == k]
        m = [c for c, i in zip(mine, idx) if cp[i]["x"] == x and cp[i]["y"] == y]
        assert len(m) == len(r)
        for mc, rc in zip(m, r):
            assert _manifold_equal(mc, rc)


def test_concave_pairs_match_reference_traversal():
    # registerConcaveMesh's BVH (b3OptimizedBvh with quantized AABBs) walked by the reference's
    # b3BvhTraversal gives these triangle-convex pairs (sorted); the oracle's quantized leaf test
    # over every triangle finds exactly the same set, in (pair, triangle, child) order
    d = load_golden("concave")
    sh = shapes_from(d)
    cp = O.concave_pairs(d["bodies"], sh, d["aabbs"], d["pairs"])
    assert len(cp) > 5000
    assert np.array_equal(cp.view(np.int32), d["tri_pairs"].view(np.int32))


def test_concave_contacts_match_reference_kernels():
    # b3FindConcaveSeparatingAxisKernel, clipFacesAndFindContactsKernel and
    # b3NewContactReductionKernel (the reference's host twins) give these manifolds, one per
    # touching triangle (and child); the oracle's records equal them byte for byte
    d = load_golden("concave")
    sh = shapes_from(d)
    mine, idx = O.concave_contacts(d["bodies"], sh, d["aabbs"], d["tri_pairs"])
    assert len(mine) > 500
    assert np.array_equal(idx, d["contact_pair"])
    assert np.array_equal(mine.view(np.uint8), d["contacts"].view(np.uint8))
    assert (mine["childA"] == -1).all() and (mine["childB"] == -1).all()
