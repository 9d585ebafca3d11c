"""ctypes binding of the C ABI (include/b3g_capi.h) plus numpy dtypes of the shared layouts.

The layouts are byte-compatible with the reference's structs (b3RigidBodyData, b3InertiaData,
b3Collidable, b3ConvexPolyhedronData, b3GpuFace, b3Aabb, b3Contact4Data).  Loading fails loudly
when libb3gpu.so is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

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
# b3GpuChildShape: a compound's child (its convex hull collidable at a pose in the compound's frame)
CHILD = np.dtype([("childPosition", "<f4", 4), ("childOrientation", "<f4", 4), ("shapeIndex", "<i4"),
                  ("numChildShapes", "<i4"), ("collidableShapeIndex", "<i4"), ("shapeType", "<i4")])
# a concave mesh's quantized triangle BVH (b3gBvhInfo / b3gBvhNode)
BVHINFO = np.dtype([("aabbMin", "<f4", 4), ("aabbMax", "<f4", 4), ("quantization", "<f4", 4), ("numNodes", "<i4"),
                    ("nodeOffset", "<i4"), ("numTriangles", "<i4"), ("pad", "<i4")])
BVHNODE = np.dtype([("qmin", "<u2", 3), ("qmax", "<u2", 3), ("escapeOrTriangle", "<i4")])
RAY = np.dtype([("from", "<f4", 4), ("to", "<f4", 4)])
RAYHIT = np.dtype([("hitFraction", "<f4"), ("hitBody", "<i4"), ("hitResult1", "<i4"), ("hitResult2", "<i4"),
                   ("hitPoint", "<f4", 4), ("hitNormal", "<f4", 4)])
JOINT = np.dtype([("type", "<i4"), ("rbA", "<i4"), ("rbB", "<i4"), ("breakingImpulseThreshold", "<f4"),
                  ("pivotInA", "<f4", 4), ("pivotInB", "<f4", 4), ("relTargetAB", "<f4", 4), ("flags", "<i4"),
                  ("uid", "<i4"), ("pad", "<i4", 2)])
for _dt, _sz in ((BODY, 80), (INERTIA, 96), (COLLIDABLE, 16), (HULL, 96), (FACE, 32), (AABB, 32), (CONTACT, 112),
                 (PAIR, 16), (RAY, 32), (RAYHIT, 48), (JOINT, 80), (BVHINFO, 64), (BVHNODE, 16)):
    assert _dt.itemsize == _sz, (_dt, _sz)

SHAPE_CONVEX_HULL, SHAPE_PLANE, SHAPE_CONCAVE_TRIMESH, SHAPE_COMPOUND, SHAPE_SPHERE = 3, 4, 5, 6, 7
SOLVER_PGS, SOLVER_JACOBI = 0, 1
JOINT_POINT2POINT, JOINT_FIXED = 3, 4
BROADPHASE_GRID, BROADPHASE_LBVH, BROADPHASE_AUTO = 0, 1, 2
CONSTRAINT_FLAG_ENABLED = 1
PGS_PARTITIONS_AUTO, PGS_PARTITIONS_GLOBAL_DELTAS, PGS_PARTITIONS_NONE, PGS_PARTITIONS_SHARED = 0, 1, 2, 3
PGS_PARTITIONS_STREAMED = 4
WARM_COLD, WARM_LEARNED, WARM_RECORD, WARM_PERSISTENT, WARM_PERSISTENT_LEARNED = 0, 1, 2, 3, 4

FLAG_PAIR_OVERFLOW = 0x1
FLAG_CONTACT_OVERFLOW = 0x2
FLAG_BATCH_OVERFLOW = 0x4
FLAG_BARRIER_TIMEOUT = 0x8
FLAG_NAN = 0x10
FLAG_CLIP_OVERFLOW = 0x20
FLAG_MLP_TIMEOUT = 0x40
FLAG_WARM_DISCARDED = 0x80

STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "INVALID_INDEX", 3: "CAPACITY", 4: "CUDA", 5: "NOT_UPLOADED",
                6: "UNSUPPORTED", 7: "BARRIER_TIMEOUT", 8: "DEGENERATE"}


class b3gConfig(C.Structure):
    _fields_ = [("max_bodies", C.c_int), ("max_shapes", C.c_int), ("max_pairs", C.c_int),
                ("max_contacts", C.c_int), ("grid_cell_size", C.c_float), ("grid_dim", C.c_int),
                ("gravity", C.c_float * 3), ("angular_damping", C.c_float), ("solver_mode", C.c_int),
                ("solver_iterations", C.c_int), ("erp", C.c_float), ("contact_threshold", C.c_float),
                ("contact_friction", C.c_float), ("residual_tol", C.c_float), ("update_world_inertia", C.c_int),
                ("use_cuda_graph", C.c_int), ("warm_start", C.c_int), ("barrier_spin_limit", C.c_int),
                ("solver_blocks_per_sm", C.c_int), ("pgs_partitions", C.c_int), ("pgs_interleave", C.c_int),
                ("warm_start_max_points", C.c_int), ("autotune", C.c_int), ("broadphase", C.c_int),
                ("pgs_tail_manifolds", C.c_int), ("pgs_flow", C.c_int),
                ("max_compound_child_pairs", C.c_int), ("max_concave_pairs", C.c_int), ("warm_start_factor", C.c_float)]


class b3gTuning(C.Structure):
    _fields_ = [("pgs_partitions", C.c_int), ("pairs_blocks_per_sm", C.c_int), ("narrow_blocks_per_sm", C.c_int),
                ("sort_blocks_per_sm", C.c_int), ("pairs_ms", C.c_float), ("contacts_ms", C.c_float),
                ("solve_ms", C.c_float), ("candidates_timed", C.c_int), ("broadphase", C.c_int)]


class b3gStepStats(C.Structure):
    _fields_ = [("num_pairs", C.c_int), ("num_contacts", C.c_int), ("num_points", C.c_int),
                ("num_colors", C.c_int), ("iterations", C.c_int), ("residual", C.c_float),
                ("status", C.c_uint), ("num_large", C.c_int), ("num_child_pairs", C.c_int),
                ("num_concave_pairs", C.c_int)]


class B3GError(RuntimeError):
    def __init__(self, status: int, fn: str, msg: str):
        self.status = status
        super().__init__(f"{fn} -> {STATUS_NAMES.get(status, status)}: {msg}")


_LIB = None

# every symbol declared in include/b3g_capi.h (checked by the CPU test-suite)
EXPORTS = [
    "b3g_config_default", "b3g_create", "b3g_destroy", "b3g_last_error", "b3g_version", "b3g_register_sphere",
    "b3g_register_plane", "b3g_register_hull", "b3g_register_hull_tables", "b3g_register_body",
    "b3g_write_all_to_gpu", "b3g_set_gravity", "b3g_set_solver", "b3g_set_scene_offsets", "b3g_set_broadphase", "b3g_autotune", "b3g_get_tuning", "b3g_profiler_range", "b3g_cast_rays", "b3g_cast_rays_device", "b3g_create_point2point_constraint", "b3g_create_fixed_constraint",
    "b3g_remove_constraint", "b3g_get_num_constraints", "b3g_read_constraints", "b3g_read_joint_order",
    "b3g_solve_joints", "b3g_step", "b3g_setup_aabbs",
    "b3g_calculate_overlapping_pairs", "b3g_compute_contacts", "b3g_solve_contacts", "b3g_integrate",
    "b3g_synchronize", "b3g_get_stats", "b3g_status", "b3g_get_num_bodies", "b3g_get_body_buffer",
    "b3g_get_inertia_buffer", "b3g_get_aabb_buffer", "b3g_get_pair_buffer", "b3g_get_contact_buffer",
    "b3g_get_stream", "b3g_read_bodies", "b3g_write_bodies", "b3g_read_inertias", "b3g_read_aabbs",
    "b3g_write_aabbs", "b3g_read_pairs", "b3g_read_contacts", "b3g_write_contacts", "b3g_read_batches", "b3g_read_solve_order",
    "b3g_register_compound", "b3g_read_child_shapes", "b3g_register_concave_mesh", "b3g_read_mesh_bvh",
    "b3g_read_impulses", "b3g_get_num_collidables", "b3g_read_registered_bodies", "b3g_read_shape_tables",
    "b3g_set_profiling",
    "b3g_get_stage_times", "b3g_get_launch_count", "b3g_record_event", "b3g_event_elapsed", "b3g_hull_compute",
    "b3g_grid_pairs_noalloc", "b3g_mlp_create", "b3g_mlp_destroy", "b3g_mlp_set_params", "b3g_mlp_get_params",
    "b3g_mlp_set_normalization", "b3g_mlp_get_normalization", "b3g_mlp_predict", "b3g_mlp_set_training_data",
    "b3g_mlp_train", "b3g_mlp_gradients", "b3g_set_warm_start_model", "b3g_read_warm_samples",
    "b3g_read_warm_start", "b3g_radix_sort32", "b3g_radix_sort32_keys", "b3g_prefix_scan32", "b3g_bound_search",
    "b3g_fill32", "b3g_reset", "b3g_compute_contacts_for_pairs", "b3g_buffer_alloc", "b3g_buffer_free",
    "b3g_buffer_copy"]


def lib_path() -> Path:
    return Path(__file__).resolve().parent / "libb3gpu.so"


def load(build_if_missing: bool = False):
    """Load libb3gpu.so (raises if it is absent; no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not p.exists():
        if build_if_missing:
            from . import _build
            _build.build_library()
        else:
            raise RuntimeError(f"{p} is missing: build it with bullet3_gb300._build.build_library() "
                               "(the GPU step has no CPU fallback)")
    lib = C.CDLL(str(p))
    lib.b3g_last_error.restype = C.c_char_p
    lib.b3g_version.restype = C.c_char_p
    for name in EXPORTS:
        f = getattr(lib, name)
        if name not in ("b3g_last_error", "b3g_version"):
            f.restype = C.c_int
    _LIB = lib
    return lib


def check(status: int, fn: str):
    if status != 0:
        raise B3GError(status, fn, _LIB.b3g_last_error().decode() if _LIB else "")


def call(name: str, *args):
    lib = load()
    st = getattr(lib, name)(*args)
    check(st, name)
    return st


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def default_config(**overrides) -> b3gConfig:
    cfg = b3gConfig()
    call("b3g_config_default", C.byref(cfg))
    for k, v in overrides.items():
        if k == "gravity":
            for i in range(3):
                cfg.gravity[i] = v[i]
        else:
            setattr(cfg, k, v)
    return cfg


def hull_compute(points: np.ndarray, scaling=(1.0, 1.0, 1.0)):
    """Host-only convex hull topology (no GPU needed): vertices, planes, face counts, indices, edges, centre."""
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    n = len(pts)
    cap = max(64, 4 * n)
    v = np.zeros((cap, 3), np.float32)
    pl = np.zeros((2 * cap, 4), np.float32)
    fc = np.zeros(2 * cap, np.int32)
    idx = np.zeros(12 * cap, np.int32)
    e = np.zeros((6 * cap, 3), np.float32)
    c = np.zeros(3, np.float32)
    counts = np.array([cap, 2 * cap, 12 * cap, 6 * cap, 0, 0], np.int32)
    sc = (C.c_float * 3)(*scaling)
    call("b3g_hull_compute", fptr(pts), C.c_int(12), C.c_int(n), sc, fptr(v), fptr(pl), iptr(fc), iptr(idx), fptr(e),
         fptr(c), iptr(counts))
    nv, nf, ni, ne = (int(x) for x in counts[:4])
    return v[:nv].copy(), pl[:nf].copy(), fc[:nf].copy(), idx[:ni].copy(), e[:ne].copy(), c
