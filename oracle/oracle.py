"""ctypes wrappers of the CPU oracle (oracle/liboracle.so) and of the compiled reference
(oracle/_ref/libb3ref.so).  TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and
the bench's CPU-baseline leg; never by the product package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

BODY = np.dtype([("pos", "<f4", 4), ("quat", "<f4", 4), ("linVel", "<f4", 4), ("angVel", "<f4", 4),
                 ("collidableIdx", "<i4"), ("invMass", "<f4"), ("restitution", "<f4"), ("friction", "<f4")])
INERTIA = np.dtype([("invInertiaWorld", "<f4", (3, 4)), ("initInvInertia", "<f4", (3, 4))])
COLLIDABLE = np.dtype([("numChildShapes", "<i4"), ("radius", "<f4"), ("shapeType", "<i4"), ("shapeIndex", "<i4")])
HULL = np.dtype([("localCenter", "<f4", 4), ("extents", "<f4", 4), ("mC", "<f4", 4), ("mE", "<f4", 4),
                 ("radius", "<f4"), ("faceOffset", "<i4"), ("numFaces", "<i4"), ("numVertices", "<i4"),
                 ("vertexOffset", "<i4"), ("uniqueEdgesOffset", "<i4"), ("numUniqueEdges", "<i4"), ("unused", "<i4")])
FACE = np.dtype([("plane", "<f4", 4), ("indexOffset", "<i4"), ("numIndices", "<i4"), ("pad", "<i4", 2)])
AABB = np.dtype([("min", "<f4", 3), ("minw", "<i4"), ("max", "<f4", 3), ("maxw", "<i4")])
CONTACT = np.dtype([("worldPosB", "<f4", (4, 4)), ("normal", "<f4", 4), ("restitutionCmp", "<u2"),
                    ("frictionCmp", "<u2"), ("batchIdx", "<i4"), ("bodyA", "<i4"), ("bodyB", "<i4"),
                    ("childA", "<i4"), ("childB", "<i4"), ("unused", "<i4", 2)])
PAIR = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("w", "<i4")])
CHILD = np.dtype([("pos", "<f4", 4), ("orn", "<f4", 4), ("shapeIndex", "<i4"), ("numChildShapes", "<i4"),
                  ("collidableShapeIndex", "<i4"), ("shapeType", "<i4")])


class OShapes(C.Structure):
    _fields_ = [("cols", C.c_void_p), ("local_aabbs", C.c_void_p), ("hulls", C.c_void_p), ("faces", C.c_void_p),
                ("indices", C.c_void_p), ("verts", C.c_void_p), ("edges", C.c_void_p), ("num_collidables", C.c_int),
                ("children", C.c_void_p)]


class OStepParams(C.Structure):
    _fields_ = [("dt", C.c_float), ("damping", C.c_float), ("gravity", C.c_float * 3), ("erp", C.c_float),
                ("threshold", C.c_float), ("cell", C.c_float), ("residual_tol", C.c_float), ("mode", C.c_int),
                ("iterations", C.c_int), ("use_grid", C.c_int), ("friction_cmp", C.c_ushort)]


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


_ORACLE = None
_REF = None


def load_oracle():
    global _ORACLE
    if _ORACLE is None:
        p = HERE / "liboracle.so"
        if not p.exists():
            from oracle import build as _b
            _b.build_oracle()
        _ORACLE = C.CDLL(str(p))
        _ORACLE.oracle_solve.restype = C.c_int
    return _ORACLE


def load_reference():
    """The reference's own CPU code (only where its sources were available to build it)."""
    global _REF
    if _REF is None:
        p = HERE / "_ref" / "libb3ref.so"
        if not p.exists():
            return None
        _REF = C.CDLL(str(p))
    return _REF


class Shapes:
    """Shape tables as numpy arrays (same layout the GPU library uses)."""

    def __init__(self, collidables, local_aabbs, hulls, faces, indices, verts, edges, children=None):
        self.children = np.ascontiguousarray(children if children is not None and len(children) else
                                             np.zeros(1, CHILD), CHILD)
        self.collidables = np.ascontiguousarray(collidables, COLLIDABLE)
        self.local_aabbs = np.ascontiguousarray(local_aabbs, AABB)
        self.hulls = np.ascontiguousarray(hulls, HULL)
        self.faces = np.ascontiguousarray(faces, FACE)
        self.indices = np.ascontiguousarray(indices, np.int32)
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 4)
        self.edges = np.ascontiguousarray(edges, np.float32).reshape(-1, 4)

    @classmethod
    def from_tables(cls, t: dict):
        return cls(t["collidables"], t["local_aabbs"], t["hulls"], t["faces"], t["indices"], t["verts"], t["edges"],
                   t.get("children"))

    def c(self) -> OShapes:
        s = OShapes()
        s.cols = self.collidables.ctypes.data
        s.local_aabbs = self.local_aabbs.ctypes.data
        s.hulls = self.hulls.ctypes.data
        s.faces = self.faces.ctypes.data
        s.indices = self.indices.ctypes.data
        s.verts = self.verts.ctypes.data
        s.edges = self.edges.ctypes.data
        s.num_collidables = len(self.collidables)
        s.children = self.children.ctypes.data
        return s


def set_threads(n: int):
    load_oracle().oracle_set_threads(C.c_int(n))


def max_threads() -> int:
    return int(load_oracle().oracle_num_threads())


def aabbs(bodies, shapes: Shapes):
    b = np.ascontiguousarray(bodies, BODY)
    out = np.zeros(len(b), AABB)
    sc = shapes.c()
    load_oracle().oracle_aabbs(_p(b), C.c_int(len(b)), C.byref(sc), _p(out))
    return out


def pairs_bruteforce(aabbs_, cap=None):
    a = np.ascontiguousarray(aabbs_, AABB)
    cap = cap or max(1024, 64 * len(a))
    out = np.zeros(cap, PAIR)
    n = load_oracle().oracle_pairs_bruteforce(_p(a), C.c_int(len(a)), _p(out), C.c_int(cap))
    return out[:min(n, cap)].copy()


def pairs_scenes(aabbs_, scene_first):
    """Pair set of independent scenes: the reference runs one broadphase per scene (one
    b3GpuGridBroadphase per b3GpuRigidBodyPipeline, b3GpuGridBroadphase.cpp:117-259, whose exact
    set is calculateOverlappingPairsHost :260-294); here each scene's bodies are paired by the brute
    force test on their own and the indices shifted back by the scene's first body, concatenated
    in (a, b) order."""
    n = len(aabbs_)
    first = [int(x) for x in scene_first]
    out = []
    for s, a in enumerate(first):
        b = first[s + 1] if s + 1 < len(first) else n
        if b - a < 2:
            continue
        p = pairs_bruteforce(aabbs_[a:b])
        p["x"] += a
        p["y"] += a
        out.append(p)
    return np.concatenate(out) if out else np.zeros(0, PAIR)


def pairs_grid(aabbs_, cell, cap=None):
    a = np.ascontiguousarray(aabbs_, AABB)
    cap = cap or max(1024, 64 * len(a))
    out = np.zeros(cap, PAIR)
    n = load_oracle().oracle_pairs_grid(_p(a), C.c_int(len(a)), C.c_float(cell), _p(out), C.c_int(cap))
    return out[:min(n, cap)].copy()


def compound_pairs(bodies, shapes: Shapes, pairs):
    """Child pairs (x, y, child of x or -1, child of y or -1) of the pairs with a compound, in
    (pair, child of x, child of y) order."""
    b = np.ascontiguousarray(bodies, BODY)
    pr = np.ascontiguousarray(pairs, PAIR)
    sc = shapes.c()
    lib = load_oracle()
    n = lib.oracle_compound_pairs(_p(b), C.byref(sc), _p(pr), C.c_int(len(pr)), None, C.c_int(0))
    out = np.zeros(max(1, n), PAIR)
    lib.oracle_compound_pairs(_p(b), C.byref(sc), _p(pr), C.c_int(len(pr)), _p(out), C.c_int(len(out)))
    return out[:n].copy()


def compound_contacts(bodies, shapes: Shapes, child_pairs):
    """(manifolds, child-pair index of each) of the given child pairs."""
    b = np.ascontiguousarray(bodies, BODY)
    cp = np.ascontiguousarray(child_pairs, PAIR)
    out = np.zeros(max(1, len(cp)), CONTACT)
    idx = np.zeros(max(1, len(cp)), np.int32)
    sc = shapes.c()
    n = load_oracle().oracle_compound_contacts(_p(b), C.byref(sc), _p(cp), C.c_int(len(cp)), _p(out), _p(idx),
                                               C.c_int(len(out)))
    return out[:n].copy(), idx[:n].copy()


def concave_pairs(bodies, shapes: Shapes, aabbs_, pairs):
    """Triangle-convex pairs (mesh body, other body, triangle, child shape or 0) of the pairs whose
    first body is a concave mesh, in (pair, triangle, child) order."""
    b = np.ascontiguousarray(bodies, BODY)
    a = np.ascontiguousarray(aabbs_, AABB)
    pr = np.ascontiguousarray(pairs, PAIR)
    sc = shapes.c()
    lib = load_oracle()
    n = lib.oracle_concave_pairs(_p(b), C.byref(sc), _p(a), _p(pr), C.c_int(len(pr)), None, C.c_int(0))
    out = np.zeros(max(1, n), PAIR)
    lib.oracle_concave_pairs(_p(b), C.byref(sc), _p(a), _p(pr), C.c_int(len(pr)), _p(out), C.c_int(len(out)))
    return out[:n].copy()


def concave_contacts(bodies, shapes: Shapes, aabbs_, tri_pairs):
    """(manifolds, triangle-convex pair index of each) of the given triangle-convex pairs."""
    b = np.ascontiguousarray(bodies, BODY)
    a = np.ascontiguousarray(aabbs_, AABB)
    tp = np.ascontiguousarray(tri_pairs, PAIR)
    out = np.zeros(max(1, len(tp)), CONTACT)
    idx = np.zeros(max(1, len(tp)), np.int32)
    sc = shapes.c()
    n = load_oracle().oracle_concave_contacts(_p(b), C.byref(sc), _p(a), _p(tp), C.c_int(len(tp)), _p(out), _p(idx),
                                              C.c_int(len(out)))
    return out[:n].copy(), idx[:n].copy()


def contacts(bodies, shapes: Shapes, pairs, friction_cmp=45874):
    b = np.ascontiguousarray(bodies, BODY)
    pr = np.array(pairs, PAIR, copy=True)
    out = np.zeros(max(1, len(pr)), CONTACT)
    sc = shapes.c()
    n = load_oracle().oracle_contacts(_p(b), C.byref(sc), _p(pr), C.c_int(len(pr)), _p(out), C.c_int(len(out)),
                                      C.c_ushort(friction_cmp))
    return out[:n].copy(), pr


def solve(bodies, inertias, contacts_, mode=0, iterations=10, dt=1 / 60, erp=0.2, threshold=0.02, residual_tol=0.0):
    """Returns (new bodies, impulses (nc,12), iterations run, residual)."""
    b = np.array(bodies, BODY, copy=True)
    I = np.ascontiguousarray(inertias, INERTIA)
    c = np.ascontiguousarray(contacts_, CONTACT)
    imp = np.zeros((max(1, len(c)), 12), np.float32)
    res = C.c_float(0)
    it = load_oracle().oracle_solve(_p(b), _p(I), C.c_int(len(b)), _p(c), C.c_int(len(c)), C.c_int(mode),
                                    C.c_int(iterations), C.c_float(dt), C.c_float(erp), C.c_float(threshold),
                                    C.c_float(residual_tol), _p(imp), C.byref(res))
    return b, imp[:len(c)], it, res.value


def solve_ordered(bodies, inertias, contacts_, order, iterations=10, dt=1 / 60, erp=0.2, threshold=0.02,
                  interleave=False):
    b = np.array(bodies, BODY, copy=True)
    I = np.ascontiguousarray(inertias, INERTIA)
    c = np.ascontiguousarray(contacts_, CONTACT)
    o = np.ascontiguousarray(order, np.int32)
    imp = np.zeros((max(1, len(c)), 12), np.float32)
    load_oracle().oracle_solve_ordered(_p(b), _p(I), C.c_int(len(b)), _p(c), C.c_int(len(c)), _p(o),
                                       C.c_int(1 if interleave else 0), C.c_int(iterations), C.c_float(dt),
                                       C.c_float(erp), C.c_float(threshold), _p(imp))
    return b, imp[:len(c)]


def solve_ordered_ex(bodies, inertias, contacts_, order, warm=None, iterations=10, residual_tol=0.0, dt=1 / 60,
                     erp=0.2, threshold=0.02, interleave=False):
    """PGS in a given manifold order with an optional warm start (12 floats per manifold, the
    layout of the impulses) and residual tolerance.  Returns (bodies, impulses, iterations run,
    final residual, warm start discarded)."""
    b = np.array(bodies, BODY, copy=True)
    I = np.ascontiguousarray(inertias, INERTIA)
    c = np.ascontiguousarray(contacts_, CONTACT)
    o = np.ascontiguousarray(order, np.int32)
    imp = np.zeros((max(1, len(c)), 12), np.float32)
    w = None if warm is None else np.ascontiguousarray(warm, np.float32).reshape(-1, 12)
    res = C.c_float(0)
    disc = C.c_int(0)
    it = load_oracle().oracle_solve_ordered_ex(_p(b), _p(I), C.c_int(len(b)), _p(c), C.c_int(len(c)), _p(o),
                                               C.c_int(1 if interleave else 0), _p(w) if w is not None else None,
                                               C.c_int(iterations), C.c_float(dt), C.c_float(erp),
                                               C.c_float(threshold), C.c_float(residual_tol), _p(imp), C.byref(res),
                                               C.byref(disc))
    return b, imp[:len(c)], it, res.value, bool(disc.value)


def integrate(bodies, dt=1 / 60, damping=0.99, gravity=(0.0, -9.8, 0.0)):
    b = np.array(bodies, BODY, copy=True)
    g = (C.c_float * 3)(*gravity)
    load_oracle().oracle_integrate(_p(b), C.c_int(len(b)), C.c_float(dt), C.c_float(damping), g)
    return b


JOINT = np.dtype([("type", "<i4"), ("rbA", "<i4"), ("rbB", "<i4"), ("breakingImpulseThreshold", "<f4"),
                  ("pivotInA", "<f4", 4), ("pivotInB", "<f4", 4), ("relTargetAB", "<f4", 4), ("flags", "<i4"),
                  ("uid", "<i4"), ("pad", "<i4", 2)])


def joint_batches(joints, bodies):
    """The joint solver's greedy batching: (order, batch offsets)."""
    j = np.ascontiguousarray(joints, JOINT)
    b = np.ascontiguousarray(bodies, BODY)
    order = np.zeros(max(1, len(j)), np.int32)
    off = np.zeros(len(j) + 2, np.int32)
    nb = load_oracle().oracle_joint_batches(_p(j), C.c_int(len(j)), _p(b), C.c_int(len(b)), _p(order), _p(off))
    return order[:len(j)], off[:nb + 1]


def solve_joints(bodies, inertias, joints, order=None, batch_off=None):
    """One joint stage: returns (new bodies, new joints).  Batches from joint_batches unless given."""
    b = np.array(bodies, BODY, copy=True)
    I = np.ascontiguousarray(inertias, INERTIA)
    j = np.array(joints, JOINT, copy=True)
    if order is None:
        order, batch_off = joint_batches(j, b)
    o = np.ascontiguousarray(order, np.int32)
    off = np.ascontiguousarray(batch_off, np.int32)
    load_oracle().oracle_solve_joints(_p(b), _p(I), C.c_int(len(b)), _p(j), C.c_int(len(j)), _p(o), _p(off),
                                      C.c_int(len(off) - 1))
    return b, j


def joint_acos(x):
    f = load_oracle().oracle_joint_acos
    f.restype = C.c_float
    f.argtypes = [C.c_float]
    return np.array([f(float(v)) for v in np.asarray(x, np.float32).ravel()], np.float32)


RAY = np.dtype([("from", "<f4", 4), ("to", "<f4", 4)])
RAYHIT = np.dtype([("hitFraction", "<f4"), ("hitBody", "<i4"), ("hitResult1", "<i4"), ("hitResult2", "<i4"),
                   ("hitPoint", "<f4", 4), ("hitNormal", "<f4", 4)])


def cast_rays(bodies, shapes: Shapes, rays, hits=None, body_scene=None):
    """Ray casts as the reference's ray kernels compute them (see oracle_cast_rays)."""
    b = np.ascontiguousarray(bodies, BODY)
    r = np.ascontiguousarray(rays, RAY)
    h = np.zeros(len(r), RAYHIT) if hits is None else np.array(hits, RAYHIT, copy=True)
    if hits is None:
        h["hitResult2"] = -1
        h["hitBody"] = -1
    sc = shapes.c()
    bs = None if body_scene is None else np.ascontiguousarray(body_scene, np.int32)
    load_oracle().oracle_cast_rays(_p(b), C.c_int(len(b)), C.byref(sc), _p(r), _p(h), C.c_int(len(r)),
                                   _p(bs) if bs is not None else None)
    return h


def check_batches(contacts_, colors, bodies) -> int:
    c = np.ascontiguousarray(contacts_, CONTACT)
    col = np.ascontiguousarray(colors, np.int32)
    b = np.ascontiguousarray(bodies, BODY)
    return int(load_oracle().oracle_check_batches(_p(c), C.c_int(len(c)), _p(col), _p(b), C.c_int(len(b))))


def step(bodies, inertias, shapes: Shapes, dt=1 / 60, mode=0, iterations=10, cell=0.0, use_grid=True,
         gravity=(0.0, -9.8, 0.0), damping=0.99, residual_tol=0.0):
    """One composed CPU step in place on a copy; returns (bodies, manifolds, pairs, points)."""
    b = np.array(bodies, BODY, copy=True)
    I = np.ascontiguousarray(inertias, INERTIA)
    p = OStepParams()
    p.dt, p.damping, p.erp, p.threshold, p.cell, p.residual_tol = dt, damping, 0.2, 0.02, cell, residual_tol
    for i in range(3):
        p.gravity[i] = gravity[i]
    p.mode, p.iterations, p.use_grid, p.friction_cmp = mode, iterations, int(use_grid), 45874
    npairs = C.c_int()
    npts = C.c_int()
    sc = shapes.c()
    nc = load_oracle().oracle_step(_p(b), _p(I), C.c_int(len(b)), C.byref(sc), C.byref(p), C.byref(npairs),
                                   C.byref(npts))
    return b, nc, npairs.value, npts.value


# ------------------------------------------------------------------ reference (compiled in place)
def ref_hull(points):
    lib = load_reference()
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    cap = max(64, 8 * len(pts))
    v = np.zeros((cap, 3), np.float32)
    pl = np.zeros((cap, 4), np.float32)
    fc = np.zeros(cap, np.int32)
    ix = np.zeros(8 * cap, np.int32)
    e = np.zeros((cap, 3), np.float32)
    counts = np.array([cap, cap, 8 * cap, cap], np.int32)
    r = lib.ref_hull(_p(pts), C.c_int(len(pts)), _p(v), _p(pl), _p(fc), _p(ix), _p(e), _p(counts))
    assert r == 0
    nv, nf, ni, ne = (int(x) for x in counts)
    return v[:nv].copy(), pl[:nf].copy(), fc[:nf].copy(), ix[:ni].copy(), e[:ne].copy()


def ref_aabbs(bodies, shapes: Shapes):
    lib = load_reference()
    b = np.ascontiguousarray(bodies, BODY)
    out = np.zeros(len(b), AABB)
    lib.ref_aabbs(_p(b), C.c_int(len(b)), _p(shapes.collidables), _p(shapes.local_aabbs), _p(out))
    return out


def ref_pairs_dbvt(aabbs_):
    lib = load_reference()
    a = np.ascontiguousarray(aabbs_, AABB)
    cap = max(1024, 64 * len(a))
    out = np.zeros((cap, 2), np.int32)
    n = lib.ref_pairs_dbvt(_p(a), C.c_int(len(a)), _p(out), C.c_int(cap))
    return out[:n].copy()


def ref_contacts(bodies, shapes: Shapes, pairs_xy):
    lib = load_reference()
    b = np.ascontiguousarray(bodies, BODY)
    pr = np.ascontiguousarray(pairs_xy, np.int32).reshape(-1, 2)
    out = np.zeros(max(1, len(pr)), CONTACT)
    pidx = np.zeros(max(1, len(pr)), np.int32)
    n = lib.ref_contacts(_p(b), C.c_int(len(b)), _p(shapes.collidables), C.c_int(len(shapes.collidables)),
                         _p(shapes.hulls), C.c_int(len(shapes.hulls)), _p(shapes.faces), C.c_int(len(shapes.faces)),
                         _p(shapes.indices), C.c_int(len(shapes.indices)), _p(shapes.verts),
                         C.c_int(len(shapes.verts)), _p(shapes.edges), C.c_int(len(shapes.edges)), _p(pr),
                         C.c_int(len(pr)), _p(out), _p(pidx), C.c_int(len(out)))
    return out[:n].copy(), pidx[:n].copy()


def ref_compound_hull_contacts(bodies, shapes: Shapes, child_pairs):
    """The reference's processCompoundPairsKernel + clipCompoundsHullHullKernel host twins on the
    given child pairs (both sides convex hulls): (manifolds, child-pair index of each)."""
    lib = load_reference()
    b = np.ascontiguousarray(bodies, BODY)
    cp = np.ascontiguousarray(child_pairs, PAIR)
    out = np.zeros(max(1, len(cp)), CONTACT)
    idx = np.zeros(max(1, len(cp)), np.int32)
    n = lib.ref_compound_hull_contacts(_p(b), _p(shapes.collidables), _p(shapes.hulls), _p(shapes.faces),
                                       C.c_int(len(shapes.faces)), _p(shapes.indices), C.c_int(len(shapes.indices)),
                                       _p(shapes.verts), C.c_int(len(shapes.verts)), _p(shapes.edges),
                                       C.c_int(len(shapes.edges)), _p(shapes.children), _p(cp), C.c_int(len(cp)),
                                       _p(out), _p(idx), C.c_int(len(out)))
    return out[:n].copy(), idx[:n].copy()


def ref_plane_compound_contacts(bodies, shapes: Shapes, plane_body, compound_body):
    """The reference's computeContactPlaneCompound for one (plane, compound) body pair."""
    lib = load_reference()
    b = np.ascontiguousarray(bodies, BODY)
    out = np.zeros(64, CONTACT)
    n = lib.ref_plane_compound_contacts(_p(b), _p(shapes.collidables), _p(shapes.hulls), _p(shapes.faces),
                                        _p(shapes.indices), _p(shapes.verts), _p(shapes.children),
                                        C.c_int(int(plane_body)), C.c_int(int(compound_body)), _p(out),
                                        C.c_int(len(out)))
    return out[:n].copy()


def ref_concave_pairs(bodies, shapes: Shapes, aabbs_, pairs, mesh_verts, mesh_indices):
    """The reference's registerConcaveMesh BVH (b3OptimizedBvh over the given unscaled mesh, with the
    mesh collidable's local AABB) and b3BvhTraversal for every pair; the triangle-convex pairs in
    the traversal's order."""
    lib = load_reference()
    b = np.ascontiguousarray(bodies, BODY)
    a = np.ascontiguousarray(aabbs_, AABB)
    pr = np.ascontiguousarray(pairs, PAIR)
    v = np.ascontiguousarray(mesh_verts, np.float32).reshape(-1, 3)
    ix = np.ascontiguousarray(mesh_indices, np.int32).reshape(-1)
    mesh_col = [i for i, c in enumerate(shapes.collidables) if c["shapeType"] == 5]
    if len(mesh_col) != 1:
        raise ValueError("one concave mesh expected")
    la = shapes.local_aabbs[mesh_col[0]]
    mn = np.ascontiguousarray(la["min"], np.float32)
    mx = np.ascontiguousarray(la["max"], np.float32)
    cap = 64 * max(1, len(pr)) * 8
    out = np.zeros(cap, PAIR)
    n = lib.ref_concave_pairs(_p(v), C.c_int(len(v)), _p(ix), C.c_int(len(ix) // 3), _p(mn), _p(mx), _p(b),
                              _p(shapes.collidables), _p(a), C.c_int(len(b)), _p(pr), C.c_int(len(pr)), _p(out),
                              C.c_int(cap))
    return out[:min(n, cap)].copy()


def ref_concave_contacts(bodies, shapes: Shapes, aabbs_, tri_pairs):
    """The reference's b3FindConcaveSeparatingAxisKernel, clipFacesAndFindContactsKernel and
    b3NewContactReductionKernel (host twins) on the given triangle-convex pairs, in order:
    (manifolds, pair index of each)."""
    lib = load_reference()
    b = np.ascontiguousarray(bodies, BODY)
    a = np.ascontiguousarray(aabbs_, AABB)
    tp = np.ascontiguousarray(tri_pairs, PAIR)
    out = np.zeros(max(1, len(tp)), CONTACT)
    idx = np.zeros(max(1, len(tp)), np.int32)
    n = lib.ref_concave_contacts(_p(b), _p(shapes.collidables), _p(shapes.hulls), _p(shapes.faces),
                                 _p(shapes.indices), _p(shapes.verts), _p(shapes.edges), _p(shapes.children), _p(a),
                                 C.c_int(len(b)), _p(tp), C.c_int(len(tp)), _p(out), _p(idx), C.c_int(len(out)))
    return out[:n].copy(), idx[:n].copy()


def ref_solve(bodies, inertias, contacts_, use_pgs=True, iterations=10, dt=1 / 60):
    lib = load_reference()
    b = np.array(bodies, BODY, copy=True)
    I = np.array(inertias, INERTIA, copy=True)
    c = np.ascontiguousarray(contacts_, CONTACT)
    lib.ref_solve(_p(b), _p(I), C.c_int(len(b)), _p(c), C.c_int(len(c)), C.c_int(int(use_pgs)), C.c_int(iterations),
                  C.c_float(dt))
    return b


def ref_integrate(bodies, dt=1 / 60, damping=0.99, gravity=(0.0, -9.8, 0.0)):
    lib = load_reference()
    b = np.array(bodies, BODY, copy=True)
    g = (C.c_float * 3)(*gravity)
    lib.ref_integrate(_p(b), C.c_int(len(b)), C.c_float(dt), C.c_float(damping), g)
    return b


def ref_cast_rays(bodies, shapes: Shapes, rays, hits=None):
    """The reference's b3GpuRaycast::castRaysHost on the given bodies and shape tables."""
    lib = load_reference()
    b = np.ascontiguousarray(bodies, BODY)
    r = np.ascontiguousarray(rays, RAY)
    h = np.zeros(len(r), RAYHIT) if hits is None else np.array(hits, RAYHIT, copy=True)
    if hits is None:
        h["hitFraction"] = 1.0
        h["hitBody"] = -1
        h["hitResult2"] = -1
    lib.ref_cast_rays(_p(r), C.c_int(len(r)), _p(h), _p(b), C.c_int(len(b)), _p(shapes.collidables),
                      C.c_int(len(shapes.collidables)), _p(shapes.hulls), C.c_int(len(shapes.hulls)),
                      _p(shapes.faces), C.c_int(len(shapes.faces)))
    return h


def ref_solve_joints(bodies, inertias, joints, iterations=4, dt=1 / 60):
    """The reference's CPU joint path: b3Point2PointConstraint / b3FixedConstraint rows solved by
    b3PgsJacobiSolver (PGS, joints only), one solveGroup call; returns the bodies."""
    lib = load_reference()
    b = np.array(bodies, BODY, copy=True)
    I = np.ascontiguousarray(inertias, INERTIA)
    j = np.ascontiguousarray(joints, JOINT)
    t = np.ascontiguousarray(j["type"], np.int32)
    ab = np.ascontiguousarray(np.stack([j["rbA"], j["rbB"]], 1), np.int32)
    prm = np.ascontiguousarray(np.concatenate([j["pivotInA"][:, :3], j["pivotInB"][:, :3], j["relTargetAB"]], 1),
                               np.float32)
    lib.ref_solve_joints(_p(b), _p(I), C.c_int(len(b)), _p(t), _p(ab), _p(prm), C.c_int(len(t)),
                         C.c_int(iterations), C.c_float(dt))
    return b


def ref_register_body(mass, pos, orn, collidable, local_min, local_max):
    """The reference's body and inertia records for one registerPhysicsInstance call."""
    lib = load_reference()
    b = np.zeros(1, BODY)
    inr = np.zeros(1, INERTIA)
    p = np.ascontiguousarray(pos, np.float32)[:3]
    q = np.ascontiguousarray(orn, np.float32)[:4]
    lo = np.ascontiguousarray(local_min, np.float32)[:3]
    hi = np.ascontiguousarray(local_max, np.float32)[:3]
    lib.ref_register_body(C.c_float(mass), _p(p), _p(q), C.c_int(collidable), _p(lo), _p(hi), _p(b), _p(inr))
    return b[0], inr[0]


# ------------------------------------------------------------------ registration (oracle/b3hull.c)
def hull(points, scaling=(1.0, 1.0, 1.0)):
    """Hull tables of registerConvexHullShape: (vertices (n,3), planes (f,4), face_counts (f,),
    indices, unique edges (e,3), local centre (3,))."""
    lib = load_oracle()
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    # registerConvexHullShape scales every input vertex first (b3GpuNarrowPhase.cpp:302-307)
    pts = (pts * np.asarray(scaling, np.float32)).astype(np.float32)
    cap = max(64, 8 * len(pts))
    v = np.zeros((cap, 3), np.float32)
    pl = np.zeros((cap, 4), np.float32)
    fc = np.zeros(cap, np.int32)
    ix = np.zeros(8 * cap, np.int32)
    e = np.zeros((cap, 3), np.float32)
    c = np.zeros(3, np.float32)
    counts = np.array([cap, cap, 8 * cap, cap], np.int32)
    r = lib.oracle_hull(_p(pts), C.c_int(len(pts)), _p(v), _p(pl), _p(fc), _p(ix), _p(e), _p(c), _p(counts))
    if r != 0:
        raise RuntimeError(f"oracle_hull failed ({r})")
    nv, nf, ni, ne = (int(x) for x in counts)
    return v[:nv].copy(), pl[:nf].copy(), fc[:nf].copy(), ix[:ni].copy(), e[:ne].copy(), c


class Registry:
    """Shape and body tables in the device layout, registered the way b3GpuNarrowPhase and
    b3GpuRigidBodyPipeline register them (hull tables from oracle_hull, bodies and inertias from
    oracle_register_body).  Used by the CPU legs to build their scene without the product."""

    def __init__(self):
        self.cols, self.laabbs, self.hull_recs, self.faces = [], [], [], []
        self.indices, self.verts, self.edges = [], [], []
        self.bodies, self.inertias = [], []
        self.children = []
        self.num_meshes = 0

    def concave_mesh(self, vertices, indices, scaling=(1.0, 1.0, 1.0)):
        """registerConcaveMesh + registerConcaveMeshShape (b3GpuNarrowPhase.cpp:521-667): the scaled
        vertices, one face per triangle (plane = normalised (v1 - v0) x (v2 - v0), w = -n.v0, float32
        throughout), the local AABB over the scaled vertices; the collidable's numChildShapes is the
        mesh's BVH index."""
        f32 = np.float32
        v = (np.asarray(vertices, f32).reshape(-1, 3) * np.asarray(scaling, f32)).astype(f32)
        tri = np.asarray(indices, np.int32).reshape(-1, 3)
        h = np.zeros(1, HULL)[0]
        h["uniqueEdgesOffset"], h["numUniqueEdges"] = len(self.edges), 0
        h["faceOffset"], h["numFaces"] = len(self.faces), len(tri)
        for t in tri:
            a, b, c = v[t[0]], v[t[1]], v[t[2]]
            e1, e2 = b - a, c - a
            n = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                          e1[0] * e2[1] - e1[1] * e2[0]], f32)
            inv = f32(1.0) / np.sqrt(f32(n[0] * n[0] + n[1] * n[1]) + f32(n[2] * n[2]))
            n = (n * inv).astype(f32)
            f = np.zeros(1, FACE)[0]
            f["plane"] = [n[0], n[1], n[2], -(f32(f32(n[0] * a[0] + n[1] * a[1]) + f32(n[2] * a[2])))]
            f["indexOffset"], f["numIndices"] = len(self.indices), 3
            self.indices.extend(int(x) for x in t)
            self.faces.append(f)
        h["vertexOffset"], h["numVertices"] = len(self.verts), len(v)
        self.verts.extend(np.concatenate([v, np.zeros((len(v), 1), f32)], 1))
        self.hull_recs.append(h)
        col = np.zeros(1, COLLIDABLE)[0]
        col["shapeType"], col["shapeIndex"], col["numChildShapes"] = 5, len(self.hull_recs) - 1, self.num_meshes
        self.num_meshes += 1
        a = np.zeros(1, AABB)[0]
        a["min"], a["max"] = v.min(0), v.max(0)
        self.cols.append(col)
        self.laabbs.append(a)
        return len(self.cols) - 1

    def plane(self, normal, constant):
        f = np.zeros(1, FACE)[0]
        f["plane"] = [normal[0], normal[1], normal[2], constant]
        self.faces.append(f)
        col = np.zeros(1, COLLIDABLE)[0]
        col["radius"], col["shapeType"], col["shapeIndex"] = constant, 4, len(self.faces) - 1
        a = np.zeros(1, AABB)[0]
        a["min"], a["max"] = -1e30, 1e30
        self.cols.append(col)
        self.laabbs.append(a)
        return len(self.cols) - 1

    def sphere(self, radius):
        col = np.zeros(1, COLLIDABLE)[0]
        col["radius"], col["shapeType"], col["shapeIndex"] = radius, 7, 0
        a = np.zeros(1, AABB)[0]
        a["min"], a["max"] = -np.float32(radius), np.float32(radius)
        self.cols.append(col)
        self.laabbs.append(a)
        return len(self.cols) - 1

    def convex_hull(self, points, scaling=(1.0, 1.0, 1.0)):
        v, pl, fc, ix, e, c = hull(points, scaling)
        h = np.zeros(1, HULL)[0]
        h["localCenter"][:3] = c
        h["uniqueEdgesOffset"], h["numUniqueEdges"] = len(self.edges), len(e)
        self.edges.extend(np.concatenate([e, np.zeros((len(e), 1), np.float32)], 1))
        h["faceOffset"], h["numFaces"] = len(self.faces), len(fc)
        off = 0
        for k in range(len(fc)):
            f = np.zeros(1, FACE)[0]
            f["plane"] = pl[k]
            f["indexOffset"], f["numIndices"] = len(self.indices), fc[k]
            self.indices.extend(ix[off:off + fc[k]].tolist())
            off += fc[k]
            self.faces.append(f)
        h["vertexOffset"], h["numVertices"] = len(self.verts), len(v)
        self.verts.extend(np.concatenate([v, np.zeros((len(v), 1), np.float32)], 1))
        self.hull_recs.append(h)
        col = np.zeros(1, COLLIDABLE)[0]
        col["shapeType"], col["shapeIndex"] = 3, len(self.hull_recs) - 1
        a = np.zeros(1, AABB)[0]
        a["min"], a["max"] = v.min(0), v.max(0)  # b3Vector3::setMin / setMax over the hull vertices
        self.cols.append(col)
        self.laabbs.append(a)
        return len(self.cols) - 1

    def compound(self, children):
        """registerCompoundShape (b3GpuNarrowPhase.cpp:370-433): children = [(hull collidable, pos,
        orn), ...]; the compound's local AABB is the union of the children's, moved into its frame."""
        recs = np.zeros(len(children), CHILD)
        for i, (c, pos, orn) in enumerate(children):
            if self.cols[c]["shapeType"] != 3:
                raise ValueError("compound children must be convex hulls")
            recs[i]["pos"][:3] = np.asarray(pos, np.float32)[:3]
            recs[i]["orn"] = np.asarray(orn, np.float32)[:4]
            recs[i]["shapeIndex"] = c
            recs[i]["shapeType"] = 3
        local = np.array([self.laabbs[int(c)] for c, _, _ in children], AABB)
        out = np.zeros(1, AABB)
        load_oracle().oracle_compound_local_aabb(_p(local), _p(recs), C.c_int(len(recs)), _p(out))
        col = np.zeros(1, COLLIDABLE)[0]
        col["shapeType"], col["shapeIndex"], col["numChildShapes"] = 6, len(self.children), len(recs)
        self.children.extend(recs)
        self.cols.append(col)
        self.laabbs.append(out[0])
        return len(self.cols) - 1

    def body(self, mass, pos, orn, collidable):
        lib = load_oracle()
        b = np.zeros(1, BODY)
        inr = np.zeros(1, INERTIA)
        la = self.laabbs[collidable]
        lo = np.ascontiguousarray(la["min"], np.float32)
        hi = np.ascontiguousarray(la["max"], np.float32)
        p = np.ascontiguousarray(pos, np.float32)[:3]
        q = np.ascontiguousarray(orn, np.float32)[:4]
        lib.oracle_register_body(C.c_float(mass), _p(p), _p(q), C.c_int(collidable), _p(lo), _p(hi), _p(b), _p(inr))
        self.bodies.append(b[0])
        self.inertias.append(inr[0])
        return len(self.bodies) - 1

    def tables(self) -> dict:
        def arr(x, dt):
            return np.array(x, dt) if len(x) else np.zeros(1, dt)
        return {"collidables": arr(self.cols, COLLIDABLE), "local_aabbs": arr(self.laabbs, AABB),
                "hulls": arr(self.hull_recs, HULL), "faces": arr(self.faces, FACE),
                "indices": np.array(self.indices or [0], np.int32),
                "verts": np.array(self.verts, np.float32).reshape(-1, 4) if self.verts else np.zeros((1, 4), np.float32),
                "edges": np.array(self.edges, np.float32).reshape(-1, 4) if self.edges else np.zeros((1, 4), np.float32),
                "bodies": np.array(self.bodies, BODY), "inertias": np.array(self.inertias, INERTIA),
                "children": arr(self.children, CHILD)}


def register_scene(scene) -> dict:
    """Tables of a synthetic scene (shapes: dicts of type hull / sphere / plane; per body its shape,
    mass, position, orientation and optional velocities), registered in scene order.  Same
    dictionary keys as the product's registered tables."""
    reg = Registry()
    col = []
    for s in scene.shapes:
        if s["type"] == "hull":
            col.append(reg.convex_hull(s["verts"]))
        elif s["type"] == "sphere":
            col.append(reg.sphere(s["radius"]))
        elif s["type"] == "plane":
            col.append(reg.plane(s["normal"], s["constant"]))
        elif s["type"] == "compound":
            # children: (index of an earlier shape of the scene, position, orientation)
            col.append(reg.compound([(col[i], p, q) for i, p, q in s["children"]]))
        elif s["type"] == "mesh":
            col.append(reg.concave_mesh(s["verts"], s["indices"], s.get("scaling", (1.0, 1.0, 1.0))))
        else:
            raise ValueError(s["type"])
    for i in range(len(scene.mass)):
        reg.body(float(scene.mass[i]), scene.pos[i], scene.orn[i], col[scene.body_shape[i]])
    t = reg.tables()
    if getattr(scene, "linvel", None) is not None:
        t["bodies"]["linVel"][:, :3] = scene.linvel
    if getattr(scene, "angvel", None) is not None:
        t["bodies"]["angVel"][:, :3] = scene.angvel
    return t
