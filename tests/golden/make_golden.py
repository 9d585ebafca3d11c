"""Generates the golden vectors in tests/golden/ from the REFERENCE's own CPU code.

Needs oracle/_ref/libb3ref.so, which oracle/build_ref.sh compiles in place from the reference
sources (only possible where those sources exist).  The committed .npz files are what the
test-suite uses everywhere else.

Fixtures:
  hulls.npz       box + Gaussian point sets -> b3ConvexUtility hull tables
  pile.npz        4x4x4 interpenetrating unit boxes on a plane (reference hull tables):
                  b3TransformAabb2 AABBs, dynamic-BVH pairs (tight-test filtered), contacts
                  (b3ContactConvexConvexSAT / computeContactPlaneConvex), b3PgsJacobiSolver PGS and
                  Jacobi velocities, integrateSingleTransform poses
  mixed.npz       boxes, Gaussian hulls and spheres overlapping on a plane: same stages; the
                  reference has no CPU code for sphere-sphere and plane-sphere, so those pairs carry
                  no reference manifold
  trajectory.npz  3x3x3 pile, 30 composed reference steps with the Jacobi solver (poses per step)
  kat_aabb.npz    the touching-AABB known answer of test/b3DynamicBvhBroadphase/main.cpp:40-69
  registration.npz  registerConvexHullShape tables of 140 point clouds (Gaussian clouds of the
                  collision-at-scale mix, boxes, rotated boxes, cylinders, lattice points, sphere
                  clouds, clouds with repeated points) and registerPhysicsInstance body / inertia
                  records of 400 bodies (the reference's b3TransformAabb and b3Matrix3x3)

  rays.npz        b3GpuRaycast::castRaysHost hits of 3,000 rays over a plane and 240 rotated boxes and
                  Gaussian hulls (no spheres: the host twin's sphere case falls through into its
                  hull case, b3GpuRaycast.cpp:196-207, which the ray kernels do not do)

  joints.npz      120 independent joints (ball and fixed, one or both bodies dynamic, random pivots,
                  poses and velocities), each solved alone by the reference's b3PgsJacobiSolver over
                  b3Point2PointConstraint / b3FixedConstraint rows (4 iterations, dt 1/60)

  compound.npz    compounds of boxes and Gaussian hulls among boxes and hulls over a plane: the
                  child pairs of every pair with a compound (the oracle's expansion), the manifolds
                  of the reference's processCompoundPairsKernel + clipCompoundsHullHullKernel host
                  twins for the hull child pairs, and computeContactPlaneCompound's for each
                  (plane, compound) pair

  python tests/golden/make_golden.py [registration|rays|joints|compound]   (no argument: every fixture)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def box_vertices(h):
    s = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], np.float32)
    return s * np.asarray(h, np.float32)


class TableBuilder:
    """Shape tables in the device layout, built from REFERENCE hull tables."""

    def __init__(self):
        self.cols, self.laabbs, self.hulls, self.faces = [], [], [], []
        self.indices, self.verts, self.edges = [], [], []

    def plane(self, n, c):
        f = np.zeros(1, O.FACE)[0]
        f["plane"] = [n[0], n[1], n[2], c]
        self.faces.append(f)
        col = np.zeros(1, O.COLLIDABLE)[0]
        col["radius"], col["shapeType"], col["shapeIndex"] = c, 4, len(self.faces) - 1
        a = np.zeros(1, O.AABB)[0]
        a["min"], a["max"] = -1e30, 1e30
        self.cols.append(col)
        self.laabbs.append(a)
        return len(self.cols) - 1

    def sphere(self, r):
        col = np.zeros(1, O.COLLIDABLE)[0]
        col["radius"], col["shapeType"], col["shapeIndex"] = r, 7, 0
        a = np.zeros(1, O.AABB)[0]
        a["min"], a["max"] = -r, r
        self.cols.append(col)
        self.laabbs.append(a)
        return len(self.cols) - 1

    def hull(self, points):
        v, pl, fc, ix, e = O.ref_hull(points)
        h = np.zeros(1, O.HULL)[0]
        c = np.zeros(3, np.float32)
        for p in v:  # vertex mean, float32, as b3GpuNarrowPhase::registerConvexHullShape
            c = (c + p).astype(np.float32)
        c = (c * np.float32(1.0 / np.float32(len(v)))).astype(np.float32)
        h["localCenter"][:3] = c
        h["uniqueEdgesOffset"], h["numUniqueEdges"] = len(self.edges), len(e)
        for x in e:
            self.edges.append([x[0], x[1], x[2], 0.0])
        h["faceOffset"], h["numFaces"] = len(self.faces), len(fc)
        off = 0
        for k in range(len(fc)):
            f = np.zeros(1, O.FACE)[0]
            f["plane"] = pl[k]
            f["indexOffset"], f["numIndices"] = len(self.indices), fc[k]
            self.indices.extend(ix[off:off + fc[k]].tolist())
            off += fc[k]
            self.faces.append(f)
        h["vertexOffset"], h["numVertices"] = len(self.verts), len(v)
        for p in v:
            self.verts.append([p[0], p[1], p[2], 0.0])
        self.hulls.append(h)
        col = np.zeros(1, O.COLLIDABLE)[0]
        col["shapeType"], col["shapeIndex"] = 3, len(self.hulls) - 1
        a = np.zeros(1, O.AABB)[0]
        a["min"], a["max"] = v.min(0), v.max(0)
        self.cols.append(col)
        self.laabbs.append(a)
        return len(self.cols) - 1

    def shapes(self) -> O.Shapes:
        def arr(x, dt):
            return np.array(x, dt) if len(x) else np.zeros(1, dt)
        return O.Shapes(arr(self.cols, O.COLLIDABLE), arr(self.laabbs, O.AABB), arr(self.hulls, O.HULL),
                        arr(self.faces, O.FACE), np.array(self.indices or [0], np.int32),
                        np.array(self.verts or [[0, 0, 0, 0]], np.float32),
                        np.array(self.edges or [[0, 0, 0, 0]], np.float32))


def quat_mat(q):
    x, y, z, w = [np.float32(t) for t in q]
    d = x * x + y * y + z * z + w * w
    s = np.float32(2.0) / d
    xs, ys, zs = x * s, y * s, z * s
    wx, wy, wz = w * xs, w * ys, w * zs
    xx, xy, xz = x * xs, x * ys, x * zs
    yy, yz, zz = y * ys, y * zs, z * zs
    one = np.float32(1.0)
    return np.array([[one - (yy + zz), xy - wz, xz + wy], [xy + wz, one - (xx + zz), yz - wx],
                     [xz - wy, yz + wx, one - (xx + yy)]], np.float32)


def make_bodies(shapes: O.Shapes, body_shape, mass, pos, orn):
    """registerPhysicsInstance + registerRigidBody: AABB with margin 0.01, AABB-box inertia with
    the full extent used as half extent, world inverse inertia R diag(1/I) R^T."""
    n = len(mass)
    b = np.zeros(n, O.BODY)
    I = np.zeros(n, O.INERTIA)
    for i in range(n):
        b[i]["pos"][:3] = pos[i]
        b[i]["quat"] = orn[i]
        b[i]["collidableIdx"] = body_shape[i]
        b[i]["invMass"] = np.float32(1.0) / np.float32(mass[i]) if mass[i] else 0.0
        b[i]["friction"] = 1.0
        if mass[i]:
            la = shapes.local_aabbs[body_shape[i]]
            R = quat_mat(orn[i])
            he = (np.float32(0.5) * (la["max"] - la["min"]) + np.float32(0.01)).astype(np.float32)
            ext = np.abs(R) @ he
            full = (2 * ext).astype(np.float32)
            lx, ly, lz = [np.float32(2) * f for f in full]
            m12 = np.float32(mass[i]) / np.float32(12.0)
            li = np.array([m12 * (ly * ly + lz * lz), m12 * (lx * lx + lz * lz), m12 * (lx * lx + ly * ly)], np.float32)
            inv = (np.float32(1) / li).astype(np.float32)
            I[i]["initInvInertia"][0, 0], I[i]["initInvInertia"][1, 1], I[i]["initInvInertia"][2, 2] = inv
            W = (R * inv[None, :]) @ R.T
            I[i]["invInertiaWorld"][:, :3] = W
    return b, I


def stage_fixture(name, tb: TableBuilder, body_shape, mass, pos, orn, linvel=None, angvel=None):
    shapes = tb.shapes()
    bodies, inertias = make_bodies(shapes, body_shape, mass, pos, orn)
    if linvel is not None:
        bodies["linVel"][:, :3] = linvel
    if angvel is not None:
        bodies["angVel"][:, :3] = angvel
    aabbs = O.ref_aabbs(bodies, shapes)
    pairs = O.ref_pairs_dbvt(aabbs)
    contacts, pidx = O.ref_contacts(bodies, shapes, pairs)
    out = dict(bodies=bodies, inertias=inertias, aabbs=aabbs, pairs=pairs, contacts=contacts, contact_pair=pidx)
    for it in (1, 10):
        out[f"pgs_bodies_{it}"] = O.ref_solve(bodies, inertias, contacts, use_pgs=True, iterations=it)
        out[f"jacobi_bodies_{it}"] = O.ref_solve(bodies, inertias, contacts, use_pgs=False, iterations=it)
        # PGS with B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_CONSTRAINTS
        out[f"pgsi_bodies_{it}"] = O.ref_solve(bodies, inertias, contacts, use_pgs=2, iterations=it)
    out["integrated"] = O.ref_integrate(out["jacobi_bodies_10"])
    for k in ("collidables", "local_aabbs", "hulls", "faces", "indices", "verts", "edges"):
        out["shape_" + k] = getattr(shapes, k)
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(name, len(bodies), "bodies", len(pairs), "pairs", len(contacts), "manifolds")


def main():
    if O.load_reference() is None:
        raise SystemExit("oracle/_ref/libb3ref.so is missing: run oracle/build_ref.sh first")
    rng = np.random.Generator(np.random.PCG64(2024))
    # hulls
    inputs = [box_vertices([0.5, 0.5, 0.5])] + [box_vertices(rng.uniform(0.2, 0.6, 3)) for _ in range(5)]
    inputs += [(rng.standard_normal((int(rng.integers(12, 33)), 3)) * 0.4).astype(np.float32) for _ in range(24)]
    hd = {}
    for i, p in enumerate(inputs):
        v, pl, fc, ix, e = O.ref_hull(p)
        hd[f"in_{i}"], hd[f"v_{i}"], hd[f"p_{i}"], hd[f"fc_{i}"], hd[f"ix_{i}"], hd[f"e_{i}"] = p, v, pl, fc, ix, e
    hd["count"] = np.array(len(inputs))
    np.savez_compressed(OUT / "hulls.npz", **hd)

    # pile: interpenetrating boxes on a plane
    tb = TableBuilder()
    plane = tb.plane((0.0, 1.0, 0.0), 0.0)
    box = tb.hull(box_vertices([0.5, 0.5, 0.5]))
    g = np.stack(np.meshgrid(np.arange(4), np.arange(4), np.arange(4), indexing="ij"), -1).reshape(-1, 3)
    pos = (g * np.array([1.0, 0.98, 1.0]) + [-1.5, 0.47, -1.5] + rng.uniform(-0.02, 0.02, g.shape)).astype(np.float32)
    ang = rng.uniform(-0.03, 0.03, (len(g), 3))
    orn = np.concatenate([np.sin(ang / 2) * [1, 1, 1], np.ones((len(g), 1))], 1)
    orn = (orn / np.linalg.norm(orn, axis=1, keepdims=True)).astype(np.float32)
    body_shape = [plane] + [box] * len(g)
    mass = [0.0] + [1.0] * len(g)
    pos = np.vstack([np.zeros((1, 3), np.float32), pos])
    orn = np.vstack([np.array([[0, 0, 0, 1]], np.float32), orn])
    lin = np.vstack([np.zeros((1, 3)), rng.normal(0, 0.3, (len(g), 3))]).astype(np.float32)
    stage_fixture("pile", tb, body_shape, mass, pos, orn, linvel=lin)

    # mixed shapes
    tb = TableBuilder()
    plane = tb.plane((0.0, 1.0, 0.0), 0.0)
    n = 300
    body_shape, mass = [plane], [0.0]
    for i in range(n):
        k = i % 4
        if k in (0, 1):
            body_shape.append(tb.hull(box_vertices(rng.uniform(0.2, 0.6, 3))))
        elif k == 2:
            body_shape.append(tb.sphere(float(rng.uniform(0.2, 0.5))))
        else:
            body_shape.append(tb.hull((rng.standard_normal((int(rng.integers(12, 33)), 3)) * 0.4).astype(np.float32)))
        mass.append(1.0)
    pos = np.vstack([np.zeros((1, 3)), rng.uniform([-3, 0.1, -3], [3, 4, 3], (n, 3))]).astype(np.float32)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    orn = np.vstack([np.array([[0, 0, 0, 1]]), q]).astype(np.float32)
    lin = np.vstack([np.zeros((1, 3)), rng.normal(0, 1.0, (n, 3))]).astype(np.float32)
    stage_fixture("mixed", tb, body_shape, mass, pos, orn, linvel=lin)

    # trajectory: composed reference step (AABB, dbvt pairs, contacts, Jacobi solve, integrate)
    tb = TableBuilder()
    plane = tb.plane((0.0, 1.0, 0.0), 0.0)
    box = tb.hull(box_vertices([0.5, 0.5, 0.5]))
    g = np.stack(np.meshgrid(np.arange(3), np.arange(3), np.arange(3), indexing="ij"), -1).reshape(-1, 3)
    p = (g * 1.1 + [-1.1, 0.6, -1.1] + rng.uniform(-0.01, 0.01, g.shape)).astype(np.float32)
    shapes = tb.shapes()
    bodies, inertias = make_bodies(shapes, [plane] + [box] * len(g), [0.0] + [1.0] * len(g),
                                   np.vstack([np.zeros((1, 3)), p]).astype(np.float32),
                                   np.tile(np.array([0, 0, 0, 1], np.float32), (len(g) + 1, 1)))
    traj = [bodies.copy()]
    for step in range(30):
        aabbs = O.ref_aabbs(bodies, shapes)
        pairs = O.ref_pairs_dbvt(aabbs)
        contacts, _ = O.ref_contacts(bodies, shapes, pairs)
        bodies = O.ref_solve(bodies, inertias, contacts, use_pgs=False, iterations=10)
        bodies = O.ref_integrate(bodies)
        traj.append(bodies.copy())
    out = dict(traj=np.stack(traj), inertias=inertias)
    for k in ("collidables", "local_aabbs", "hulls", "faces", "indices", "verts", "edges"):
        out["shape_" + k] = getattr(shapes, k)
    np.savez_compressed(OUT / "trajectory.npz", **out)
    print("trajectory", len(traj) - 1, "steps")

    # touching AABBs [0,1]^3 and [1,2]^3 give exactly one pair (inclusive overlap)
    a = np.zeros(2, O.AABB)
    a[0]["min"], a[0]["max"], a[0]["minw"], a[0]["maxw"] = 0, 1, 0, 1
    a[1]["min"], a[1]["max"], a[1]["minw"], a[1]["maxw"] = 1, 2, 1, 1
    np.savez_compressed(OUT / "kat_aabb.npz", aabbs=a, pairs=O.ref_pairs_dbvt(a))
    print("kat pairs", O.ref_pairs_dbvt(a).tolist())


def registration_fixture():
    """registration.npz: hull tables and body records from the reference's registration code."""
    rng = np.random.Generator(np.random.PCG64(77))

    def rot(q):
        x, y, z, w = q
        return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                         [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                         [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])

    clouds = []
    for _ in range(50):
        clouds.append((rng.standard_normal((int(rng.integers(12, 33)), 3)) * 0.4).astype(np.float32))
    for _ in range(20):
        clouds.append(box_vertices(rng.uniform(0.2, 0.6, 3)))
    for _ in range(20):
        q = rng.standard_normal(4)
        clouds.append((box_vertices(rng.uniform(0.2, 0.6, 3)) @ rot(q / np.linalg.norm(q)).T).astype(np.float32))
    for _ in range(15):
        k = int(rng.integers(6, 24))
        a = np.linspace(0, 2 * np.pi, k, endpoint=False)
        ring = np.stack([np.cos(a), np.zeros(k), np.sin(a)], 1)
        clouds.append((np.concatenate([ring + [0, -0.5, 0], ring + [0, 0.5, 0]]) * rng.uniform(0.2, 1.0)).astype(np.float32))
    for _ in range(10):
        g = np.stack(np.meshgrid(*[np.arange(int(rng.integers(2, 4)))] * 3, indexing="ij"), -1).reshape(-1, 3)
        clouds.append((g * rng.uniform(0.1, 1.0)).astype(np.float32))
    for _ in range(15):
        p = rng.standard_normal((int(rng.integers(20, 120)), 3))
        clouds.append((p / np.linalg.norm(p, axis=1, keepdims=True)).astype(np.float32))
    for _ in range(10):
        p = (rng.standard_normal((int(rng.integers(12, 33)), 3)) * 0.4).astype(np.float32)
        clouds.append(np.concatenate([p, p[:int(rng.integers(1, 6))]]))
    out = {"count": np.array(len(clouds))}
    for i, p in enumerate(clouds):
        v, pl, fc, ix, e = O.ref_hull(p)
        out[f"in_{i}"], out[f"v_{i}"], out[f"p_{i}"], out[f"fc_{i}"], out[f"ix_{i}"], out[f"e_{i}"] = p, v, pl, fc, ix, e
    n = 400
    mass = np.where(rng.uniform(size=n) < 0.1, 0.0, rng.uniform(0.1, 5.0, n)).astype(np.float32)
    pos = rng.uniform(-100, 100, (n, 3)).astype(np.float32)
    q = rng.standard_normal((n, 4))
    q = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    lo = -rng.uniform(0.1, 1.0, (n, 3)).astype(np.float32)
    hi = rng.uniform(0.1, 1.0, (n, 3)).astype(np.float32)
    bodies = np.zeros(n, O.BODY)
    inertias = np.zeros(n, O.INERTIA)
    for i in range(n):
        bodies[i], inertias[i] = O.ref_register_body(float(mass[i]), pos[i], q[i], 3, lo[i], hi[i])
    out.update(body_mass=mass, body_pos=pos, body_orn=q, body_local_min=lo, body_local_max=hi, bodies=bodies,
               inertias=inertias)
    np.savez_compressed(OUT / "registration.npz", **out)
    print("registration", len(clouds), "hulls", n, "bodies")


def rays_fixture():
    """rays.npz: the reference's host ray cast over rotated boxes and Gaussian hulls on a plane."""
    rng = np.random.Generator(np.random.PCG64(91))
    tb = TableBuilder()
    plane = tb.plane((0.0, 1.0, 0.0), 0.0)
    body_shape, mass = [plane], [0.0]
    n = 240
    for i in range(n):
        if i % 3 == 2:
            body_shape.append(tb.hull((rng.standard_normal((int(rng.integers(12, 33)), 3)) * 0.4).astype(np.float32)))
        else:
            body_shape.append(tb.hull(box_vertices(rng.uniform(0.2, 0.8, 3))))
        mass.append(1.0)
    pos = np.vstack([np.zeros((1, 3)), rng.uniform([-10, 0.5, -10], [10, 6, 10], (n, 3))]).astype(np.float32)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    orn = np.vstack([np.array([[0, 0, 0, 1]]), q]).astype(np.float32)
    shapes = tb.shapes()
    bodies, inertias = make_bodies(shapes, body_shape, mass, pos, orn)
    nr = 3000
    rays = np.zeros(nr, O.RAY)
    f = rng.uniform([-11, 0, -11], [11, 7, 11], (nr, 3)).astype(np.float32)
    t = f.copy()
    down = np.arange(nr) < nr // 2
    f[down, 1] = 12.0
    t[down, 1] = -1.0
    d = rng.standard_normal(((~down).sum(), 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t[~down] = (f[~down] + d * rng.uniform(2.0, 25.0, ((~down).sum(), 1))).astype(np.float32)
    rays["from"][:, :3] = f
    rays["to"][:, :3] = t
    hits = O.ref_cast_rays(bodies, shapes, rays)
    out = dict(bodies=bodies, rays=rays, hits=hits)
    for k in ("collidables", "local_aabbs", "hulls", "faces", "indices", "verts", "edges"):
        out["shape_" + k] = getattr(shapes, k)
    np.savez_compressed(OUT / "rays.npz", **out)
    print("rays", nr, "rays", int((hits["hitBody"] >= 0).sum()), "hits")


def joints_fixture():
    """joints.npz: single joints solved by the reference's CPU constraint classes."""
    rng = np.random.Generator(np.random.PCG64(123))

    def quat(scale=None):
        if scale is None:
            x = rng.standard_normal(4)
            return (x / np.linalg.norm(x)).astype(np.float32)
        a = rng.uniform(-scale, scale, 3)
        t = np.linalg.norm(a)
        return np.concatenate([np.sin(t / 2) * a / t, [np.cos(t / 2)]]).astype(np.float32)

    reg = O.Registry()
    box = reg.convex_hull(box_vertices([0.5, 0.4, 0.3]))
    n = 120
    joints = np.zeros(n, O.JOINT)
    for k in range(n):
        static_a = k % 4 == 0
        reg.body(0.0 if static_a else float(rng.uniform(0.5, 3.0)), rng.uniform(-1, 1, 3), quat(), box)
        reg.body(float(rng.uniform(0.5, 3.0)), rng.uniform(-1, 1, 3), quat(), box)
        j = joints[k]
        j["type"] = 3 if k % 2 == 0 else 4
        j["rbA"], j["rbB"] = 2 * k, 2 * k + 1
        j["breakingImpulseThreshold"] = 1e30
        j["flags"] = 1
        j["uid"] = k
        j["pivotInA"][:3] = rng.uniform(-0.6, 0.6, 3)
        j["pivotInB"][:3] = rng.uniform(-0.6, 0.6, 3)
        j["relTargetAB"] = [0, 0, 0, 1] if k % 6 != 3 else quat(0.3)
    t = reg.tables()
    bodies, inertias = t["bodies"], t["inertias"]
    dyn = bodies["invMass"] != 0
    bodies["linVel"][:, :3] = rng.standard_normal((len(bodies), 3)) * dyn[:, None]
    bodies["angVel"][:, :3] = rng.standard_normal((len(bodies), 3)) * dyn[:, None]
    out = bodies.copy()
    for k in range(n):  # each joint alone: its two bodies and nothing else
        sub = bodies[2 * k:2 * k + 2].copy()
        jj = joints[k:k + 1].copy()
        jj["rbA"], jj["rbB"] = 0, 1
        out[2 * k:2 * k + 2] = O.ref_solve_joints(sub, inertias[2 * k:2 * k + 2], jj)
    shapes = t
    res = dict(bodies=bodies, inertias=inertias, joints=joints, solved=out)
    for k in ("collidables", "local_aabbs", "hulls", "faces", "indices", "verts", "edges"):
        res["shape_" + k] = shapes[k]
    np.savez_compressed(OUT / "joints.npz", **res)
    print("joints", n)


def compound_fixture():
    """compound.npz: the reference's compound kernels on a dense mix of compounds, boxes and hulls."""
    rng = np.random.Generator(np.random.PCG64(77))

    def quat():
        x = rng.standard_normal(4)
        return (x / np.linalg.norm(x)).astype(np.float32)

    reg = O.Registry()
    plane = reg.plane((0.0, 1.0, 0.0), 0.0)
    bx = reg.convex_hull(box_vertices([0.5, 0.25, 0.25]))
    by = reg.convex_hull(box_vertices([0.25, 0.5, 0.25]))
    gauss = reg.convex_hull((rng.standard_normal((20, 3)) * 0.3).astype(np.float32))
    ell = reg.compound([(bx, (0.25, 0.0, 0.0), (0, 0, 0, 1)), (by, (0.0, 0.5, 0.0), (0, 0, 0, 1))])
    dumb = reg.compound([(gauss, (-0.6, 0.0, 0.0), quat()), (bx, (0.0, 0.0, 0.0), (0, 0, 0, 1)),
                         (gauss, (0.6, 0.0, 0.0), quat())])
    cols = [ell, dumb, bx, gauss]
    reg.body(0.0, (0, 0, 0), (0, 0, 0, 1), plane)
    for i in range(300):
        p = rng.uniform(-3, 3, 3)
        p[1] = rng.uniform(0.0, 1.5)
        reg.body(1.0, p, quat(), cols[i % 4])
    t = reg.tables()
    shapes = O.Shapes.from_tables(t)
    bodies = t["bodies"]
    pairs = O.pairs_bruteforce(O.aabbs(bodies, shapes))
    cp = O.compound_pairs(bodies, shapes, pairs)

    def side(body, child):
        return 3 if child >= 0 else int(shapes.collidables[bodies[body]["collidableIdx"]]["shapeType"])
    hh = np.array([side(p["x"], p["z"]) == 3 and side(p["y"], p["w"]) == 3 for p in cp])
    sel = np.where(hh)[0]
    ref, ridx = O.ref_compound_hull_contacts(bodies, shapes, cp[hh])
    plane_pairs, plane_contacts, plane_owner = [], [], []
    for p in pairs:
        x, y = int(p["x"]), int(p["y"])
        tx = int(shapes.collidables[bodies[x]["collidableIdx"]]["shapeType"])
        ty = int(shapes.collidables[bodies[y]["collidableIdx"]]["shapeType"])
        if tx == 4 and ty == 6:
            c = O.ref_plane_compound_contacts(bodies, shapes, x, y)
            plane_contacts.append(c)
            plane_owner.extend([len(plane_pairs)] * len(c))
            plane_pairs.append((x, y))
    out = dict(bodies=bodies, pairs=pairs, child_pairs=cp, hull_contacts=ref, hull_child_index=sel[ridx],
               plane_pairs=np.array(plane_pairs, np.int32).reshape(-1, 2),
               plane_contacts=np.concatenate(plane_contacts) if plane_contacts else np.zeros(0, O.CONTACT),
               plane_owner=np.array(plane_owner, np.int32))
    for k in ("collidables", "local_aabbs", "hulls", "faces", "indices", "verts", "edges", "children"):
        out["shape_" + k] = t[k]
    np.savez_compressed(OUT / "compound.npz", **out)
    print("compound", len(cp), "child pairs,", len(ref), "hull manifolds,", len(out["plane_contacts"]), "plane manifolds")


def concave_fixture():
    """concave.npz: the reference's concave-mesh path on a height-field mesh (scenes.terrain_mesh,
    24 x 24 quads) under 300 boxes, Gaussian hulls and compounds touching it: the BVH of
    registerConcaveMesh (b3OptimizedBvh) with b3BvhTraversal gives the triangle-convex pairs, the
    host twins b3FindConcaveSeparatingAxisKernel / clipFacesAndFindContactsKernel /
    b3NewContactReductionKernel give the manifolds."""
    from bullet3_gb300 import scenes
    sc = scenes.terrain_scene(300, grid=24, seed=21, spheres=False)
    t = O.register_scene(sc)
    shapes = O.Shapes.from_tables(t)
    bodies = t["bodies"]
    aabbs = O.aabbs(bodies, shapes)
    pairs = O.pairs_bruteforce(aabbs)
    rp = O.ref_concave_pairs(bodies, shapes, aabbs, pairs, sc.shapes[0]["verts"], sc.shapes[0]["indices"])
    rp = rp[np.lexsort((rp["w"], rp["z"], rp["y"], rp["x"]))]
    ref, ridx = O.ref_concave_contacts(bodies, shapes, aabbs, rp)
    out = dict(bodies=bodies, pairs=pairs, aabbs=aabbs, tri_pairs=rp, contacts=ref, contact_pair=ridx,
               mesh_verts=sc.shapes[0]["verts"], mesh_indices=sc.shapes[0]["indices"])
    for k in ("collidables", "local_aabbs", "hulls", "faces", "indices", "verts", "edges", "children"):
        out["shape_" + k] = t[k]
    np.savez_compressed(OUT / "concave.npz", **out)
    print("concave", len(rp), "triangle-convex pairs,", len(ref), "manifolds")


if __name__ == "__main__":
    if O.load_reference() is None:
        raise SystemExit("oracle/_ref/libb3ref.so is missing: run oracle/build_ref.sh first")
    if len(sys.argv) > 1 and sys.argv[1] == "registration":
        registration_fixture()
    elif len(sys.argv) > 1 and sys.argv[1] == "rays":
        rays_fixture()
    elif len(sys.argv) > 1 and sys.argv[1] == "joints":
        joints_fixture()
    elif len(sys.argv) > 1 and sys.argv[1] == "compound":
        compound_fixture()
    elif len(sys.argv) > 1 and sys.argv[1] == "concave":
        concave_fixture()
    else:
        main()
        registration_fixture()
        rays_fixture()
        joints_fixture()
        compound_fixture()
        concave_fixture()
        joints_fixture()
