"""Host-side mirror of the reference's GPU rigid-body API.

Same class names, method names, argument meaning and error behaviour as the reference's
b3GpuNarrowPhase (src/Bullet3OpenCL/RigidBody/b3GpuNarrowPhase.h:9-99), b3GpuBroadphaseInterface /
b3GpuGridBroadphase (src/Bullet3OpenCL/BroadphaseCollision/b3GpuBroadphaseInterface.h:12-40) and
b3GpuRigidBodyPipeline (src/Bullet3OpenCL/RigidBody/b3GpuRigidBodyPipeline.h:25-67), implemented
on the C ABI of libb3gpu.so.  Indices that the reference reports as -1 + b3Error are reported the
same way here (the error text goes to `b3Error` below); CUDA failures raise.

One native "world" backs the three objects, as the reference's three objects share one OpenCL
context and queue: the narrowphase owns it, the broadphase and pipeline attach to it.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import capi
from .capi import AABB, BODY, CONTACT, PAIR, INERTIA, call, fptr, iptr, ptr


def b3Error(msg: str):
    """The reference's b3Error sink (Bullet3Common/b3Logging.h:50-68): message to stderr."""
    sys.stderr.write("b3Error: " + msg.rstrip() + "\n")


class b3Config:
    """b3Config (src/Bullet3Collision/.../b3Config.h:4-37) plus the constants the reference hard-codes."""

    def __init__(self, **kw):
        self.m_maxConvexBodies = 128 * 1024
        self.m_maxConvexShapes = 8 * 1024
        self.m_maxBroadphasePairs = 0
        self.m_maxContactCapacity = 0
        self.m_compoundPairCapacity = 0  # child pairs of compounds per step (0 = m_maxBroadphasePairs)
        self.m_maxTriConvexPairCapacity = 0  # triangle-convex pairs of meshes per step (0 = m_maxBroadphasePairs)
        self.grid_cell_size = 0.0
        self.grid_dim = 128
        self.solver_mode = capi.SOLVER_PGS
        self.solver_iterations = 10
        self.residual_tol = 0.0
        self.use_cuda_graph = True
        self.contact_friction = 0.7
        self.update_world_inertia = False
        self.gravity = (0.0, -9.8, 0.0)
        self.solver_blocks_per_sm = 0
        self.pgs_partitions = capi.PGS_PARTITIONS_AUTO
        self.pgs_interleave = False
        self.warm_start = 0
        self.warm_start_max_points = 0
        self.warm_start_factor = 0.0  # persisting impulses scaled by this (0 = 1; the reference uses 0.85)
        self.autotune = False
        self.broadphase = capi.BROADPHASE_GRID
        self.pgs_tail_manifolds = 0
        self.pgs_flow = 0
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)

    def to_c(self) -> capi.b3gConfig:
        return capi.default_config(max_bodies=self.m_maxConvexBodies, max_shapes=self.m_maxConvexShapes,
                                   max_pairs=self.m_maxBroadphasePairs, max_contacts=self.m_maxContactCapacity,
                                   grid_cell_size=self.grid_cell_size, grid_dim=self.grid_dim,
                                   solver_mode=self.solver_mode, solver_iterations=self.solver_iterations,
                                   residual_tol=self.residual_tol, use_cuda_graph=int(self.use_cuda_graph),
                                   contact_friction=self.contact_friction,
                                   update_world_inertia=int(self.update_world_inertia), gravity=self.gravity,
                                   solver_blocks_per_sm=self.solver_blocks_per_sm,
                                   pgs_partitions=self.pgs_partitions,
                                   pgs_interleave=int(self.pgs_interleave), warm_start=int(self.warm_start),
                                   warm_start_max_points=int(self.warm_start_max_points),
                                   warm_start_factor=float(self.warm_start_factor),
                                   autotune=int(self.autotune), broadphase=int(self.broadphase),
                                   pgs_tail_manifolds=int(self.pgs_tail_manifolds), pgs_flow=int(self.pgs_flow),
                                   max_compound_child_pairs=int(self.m_compoundPairCapacity),
                                   max_concave_pairs=int(self.m_maxTriConvexPairCapacity))


class _World:
    def __init__(self, config: b3Config, device: int = 0):
        capi.load()
        self.handle = C.c_void_p()
        self.config = config
        call("b3g_create", C.byref(config.to_c()), C.c_int(device), C.byref(self.handle))
        self.uploaded = False

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and capi._LIB is not None:
            capi._LIB.b3g_destroy(h)
            self.handle = None

    def num_bodies(self) -> int:
        n = C.c_int()
        call("b3g_get_num_bodies", self.handle, C.byref(n))
        return n.value


class b3GpuNarrowPhase:
    """b3GpuNarrowPhase: shape and body registry plus contact generation."""

    def __init__(self, config: b3Config | None = None, device: int = 0):
        self.m_config = config or b3Config()
        self._w = _World(self.m_config, device)
        self.m_static0Index = -1

    @property
    def world(self):
        return self._w

    # -- shapes -------------------------------------------------------------------------
    def _reg(self, fn, *args) -> int:
        out = C.c_int(-1)
        st = getattr(capi.load(), fn)(self._w.handle, *args, C.byref(out))
        if st in (2, 3, 8):  # invalid index / capacity / degenerate -> -1 + b3Error, as the reference
            b3Error(capi._LIB.b3g_last_error().decode())
            return -1
        capi.check(st, fn)
        return out.value

    def registerSphereShape(self, radius: float) -> int:
        return self._reg("b3g_register_sphere", C.c_float(radius))

    def registerPlaneShape(self, planeNormal, planeConstant: float) -> int:
        n = (C.c_float * 3)(*[float(x) for x in planeNormal[:3]])
        return self._reg("b3g_register_plane", n, C.c_float(planeConstant))

    def registerConvexHullShape(self, vertices, strideInBytes: int | None = None, numVertices: int | None = None,
                                scaling=(1.0, 1.0, 1.0)) -> int:
        v = np.ascontiguousarray(vertices, dtype=np.float32)
        if strideInBytes is None:
            v = v.reshape(-1, 3)
            strideInBytes = 12
            numVertices = len(v)
        sc = (C.c_float * 3)(*[float(x) for x in scaling])
        return self._reg("b3g_register_hull", fptr(v), C.c_int(strideInBytes), C.c_int(numVertices), sc)

    def registerConvexHullShapeTables(self, vertices, planes, face_counts, indices, unique_edges) -> int:
        """registerConvexHullShape(b3ConvexUtility*): precomputed hull tables."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        p = np.ascontiguousarray(planes, np.float32).reshape(-1, 4)
        fc = np.ascontiguousarray(face_counts, np.int32)
        ix = np.ascontiguousarray(indices, np.int32)
        e = np.ascontiguousarray(unique_edges, np.float32).reshape(-1, 3)
        return self._reg("b3g_register_hull_tables", fptr(v), C.c_int(len(v)), fptr(p), iptr(fc), C.c_int(len(fc)),
                         iptr(ix), fptr(e), C.c_int(len(e)))

    def registerCompoundShape(self, childShapes) -> int:
        """registerCompoundShape(b3AlignedObjectArray<b3GpuChildShape>*): childShapes is a
        capi.CHILD array, or a list of (hull collidable, position, orientation)."""
        if isinstance(childShapes, np.ndarray) and childShapes.dtype == capi.CHILD:
            ch = np.ascontiguousarray(childShapes)
        else:
            ch = np.zeros(len(childShapes), capi.CHILD)
            for i, (c, pos, orn) in enumerate(childShapes):
                ch[i]["childPosition"][:3] = np.asarray(pos, np.float32)[:3]
                ch[i]["childOrientation"] = np.asarray(orn, np.float32)[:4]
                ch[i]["shapeIndex"] = int(c)
                ch[i]["shapeType"] = 3
        return self._reg("b3g_register_compound", capi.ptr(ch), C.c_int(len(ch)))

    def registerConcaveMesh(self, vertices, indices, scaling=(1.0, 1.0, 1.0)) -> int:
        """registerConcaveMesh(b3AlignedObjectArray<b3Vector3>*, b3AlignedObjectArray<int>*, const float*):
        vertices (n, 3), indices (3 per triangle); -1 + b3Error on invalid input."""
        if vertices is None or indices is None:
            b3Error("registerConcaveMesh: no vertices or indices")
            return -1
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        ix = np.ascontiguousarray(indices, np.int32).reshape(-1)
        if len(ix) % 3:
            b3Error("registerConcaveMesh: the index count is not a multiple of 3")
            return -1
        sc = (C.c_float * 3)(*[float(x) for x in scaling])
        st = capi.load().b3g_register_concave_mesh(self._w.handle, fptr(v), C.c_int(12), C.c_int(len(v)), iptr(ix),
                                                   C.c_int(len(ix) // 3), sc, C.byref(out := C.c_int(-1)))
        if st != 0:
            b3Error(capi._LIB.b3g_last_error().decode())
            return -1
        return out.value

    # -- bodies -------------------------------------------------------------------------
    def getNumRigidBodies(self) -> int:
        return self._w.num_bodies()

    def getNumCollidablesGpu(self) -> int:
        n = C.c_int()
        call("b3g_get_num_collidables", self._w.handle, C.byref(n))
        return n.value

    def writeAllBodiesToGpu(self):
        call("b3g_write_all_to_gpu", self._w.handle)
        self._w.uploaded = True

    def readbackAllBodiesToCpu(self) -> np.ndarray:
        n = self.getNumRigidBodies()
        out = np.zeros(n, BODY)
        call("b3g_read_bodies", self._w.handle, ptr(out), C.c_int(n))
        return out

    def writeBodiesToGpu(self, bodies: np.ndarray):
        b = np.ascontiguousarray(bodies, BODY)
        call("b3g_write_bodies", self._w.handle, ptr(b), C.c_int(len(b)))

    def readInertiasToCpu(self) -> np.ndarray:
        n = self.getNumRigidBodies()
        out = np.zeros(n, INERTIA)
        call("b3g_read_inertias", self._w.handle, ptr(out), C.c_int(n))
        return out

    def getObjectTransformFromCpu(self, bodyIndex: int):
        b = self.readbackAllBodiesToCpu()[bodyIndex]
        return b["pos"][:3].copy(), b["quat"].copy()

    def computeContacts(self):
        """computeContacts (b3GpuNarrowPhase.cpp:751-809) on the current overlapping pairs."""
        call("b3g_compute_contacts", self._w.handle)

    def getNumContactsGpu(self) -> int:
        n = C.c_int()
        call("b3g_read_contacts", self._w.handle, None, C.c_int(0), C.byref(n))
        return n.value

    def getContactsCPU(self) -> np.ndarray:
        n = C.c_int()
        call("b3g_read_contacts", self._w.handle, None, C.c_int(0), C.byref(n))
        out = np.zeros(n.value, CONTACT)
        if n.value:
            call("b3g_read_contacts", self._w.handle, ptr(out), C.c_int(n.value), C.byref(n))
        return out

    def getContactsGpu(self) -> int:
        p = C.c_void_p()
        n = C.c_int()
        call("b3g_get_contact_buffer", self._w.handle, C.byref(p), C.byref(n))
        return p.value or 0

    def setContactsFromCpu(self, contacts: np.ndarray):
        c = np.ascontiguousarray(contacts, CONTACT)
        call("b3g_write_contacts", self._w.handle, ptr(c), C.c_int(len(c)))

    def getBodiesGpu(self) -> int:
        p = C.c_void_p()
        call("b3g_get_body_buffer", self._w.handle, C.byref(p))
        return p.value or 0

    def getBodyInertiasGpu(self) -> int:
        p = C.c_void_p()
        call("b3g_get_inertia_buffer", self._w.handle, C.byref(p))
        return p.value or 0

    def getStatic0Index(self) -> int:
        return self.m_static0Index


class b3GpuBroadphaseInterface:
    """b3GpuBroadphaseInterface (pure interface)."""

    def createProxy(self, aabbMin, aabbMax, userPtr, collisionFilterGroup, collisionFilterMask):
        raise NotImplementedError

    def createLargeProxy(self, aabbMin, aabbMax, userPtr, collisionFilterGroup, collisionFilterMask):
        raise NotImplementedError

    def calculateOverlappingPairs(self, maxPairs: int):
        raise NotImplementedError

    def calculateOverlappingPairsHost(self, maxPairs: int):
        raise NotImplementedError


class b3GpuGridBroadphase(b3GpuBroadphaseInterface):
    """Uniform-grid broadphase (b3GpuGridBroadphase.cpp); large (static) proxies via the large-AABB path."""

    CreateFunc = None

    def __init__(self, narrowphase: b3GpuNarrowPhase | None = None):
        self._np = narrowphase
        self.m_smallAabbsMappingCPU = []
        self.m_largeAabbsMappingCPU = []

    def _attach(self, narrowphase: b3GpuNarrowPhase):
        self._np = narrowphase

    @property
    def _h(self):
        if self._np is None:
            raise RuntimeError("broadphase not attached to a narrowphase/pipeline")
        return self._np.world.handle

    def createProxy(self, aabbMin, aabbMax, userPtr, collisionFilterGroup=1, collisionFilterMask=1):
        self.m_smallAabbsMappingCPU.append(userPtr)

    def createLargeProxy(self, aabbMin, aabbMax, userPtr, collisionFilterGroup=1, collisionFilterMask=1):
        self.m_largeAabbsMappingCPU.append(userPtr)

    def calculateOverlappingPairs(self, maxPairs: int = 0):
        call("b3g_calculate_overlapping_pairs", self._h)

    def calculateOverlappingPairsHost(self, maxPairs: int = 0):
        raise NotImplementedError("there is no CPU broadphase in this library (the GPU path has no fallback)")

    def writeAabbsToGpu(self):
        pass  # AABBs are derived on the device from the body buffer every step

    def getNumOverlap(self) -> int:
        n = C.c_int()
        call("b3g_read_pairs", self._h, None, C.c_int(0), C.byref(n))
        return n.value

    def getOverlappingPairsCPU(self) -> np.ndarray:
        n = self.getNumOverlap()
        out = np.zeros(n, PAIR)
        if n:
            m = C.c_int()
            call("b3g_read_pairs", self._h, ptr(out), C.c_int(n), C.byref(m))
        return out

    def getOverlappingPairBuffer(self) -> int:
        p = C.c_void_p()
        n = C.c_int()
        call("b3g_get_pair_buffer", self._h, C.byref(p), C.byref(n))
        return p.value or 0

    def getAabbBufferWS(self) -> int:
        p = C.c_void_p()
        call("b3g_get_aabb_buffer", self._h, C.byref(p))
        return p.value or 0

    def getAllAabbsCPU(self) -> np.ndarray:
        n = self._np.getNumRigidBodies()
        out = np.zeros(n, AABB)
        call("b3g_read_aabbs", self._h, ptr(out), C.c_int(n))
        return out

    def setAllAabbsCPU(self, aabbs: np.ndarray):
        a = np.ascontiguousarray(aabbs, AABB)
        call("b3g_write_aabbs", self._h, ptr(a), C.c_int(len(a)))


class b3GpuParallelLinearBvhBroadphase(b3GpuGridBroadphase):
    """Linear-BVH broadphase (b3GpuParallelLinearBvhBroadphase.cpp): Morton-ordered binary radix
    tree over the dynamic bodies, complete for any AABB sizes; the same canonical pair list as the
    grid.  Attaching it to a pipeline switches the world's pair search to the LBVH."""

    def _attach(self, narrowphase: b3GpuNarrowPhase):
        self._np = narrowphase
        call("b3g_set_broadphase", self._h, C.c_int(capi.BROADPHASE_LBVH))


class b3GpuRigidBodyPipeline:
    """b3GpuRigidBodyPipeline: registration and the per-frame step."""

    def __init__(self, narrowphase: b3GpuNarrowPhase, broadphase: b3GpuBroadphaseInterface | None = None,
                 broadphaseDbvt=None, config: b3Config | None = None):
        self.m_narrowphase = narrowphase
        self.m_broadphase = broadphase or b3GpuGridBroadphase()
        if isinstance(self.m_broadphase, b3GpuGridBroadphase):
            self.m_broadphase._attach(narrowphase)
        self.m_config = config or narrowphase.m_config

    @property
    def _h(self):
        return self.m_narrowphase.world.handle

    def registerPhysicsInstance(self, mass: float, position, orientation, collidableIndex: int, userIndex: int = -1,
                                writeInstanceToGpu: bool = False) -> int:
        pos = (C.c_float * 3)(*[float(x) for x in position[:3]])
        orn = (C.c_float * 4)(*[float(x) for x in orientation[:4]])
        out = C.c_int(-1)
        st = capi.load().b3g_register_body(self._h, C.c_float(mass), pos, orn, C.c_int(collidableIndex),
                                           C.c_int(userIndex), C.byref(out))
        if st in (2, 3):
            b3Error(capi._LIB.b3g_last_error().decode())
            return -1
        capi.check(st, "b3g_register_body")
        idx = out.value
        if mass:
            self.m_broadphase.createProxy(None, None, idx)
        else:
            self.m_broadphase.createLargeProxy(None, None, idx)
            if self.m_narrowphase.m_static0Index < 0 and idx == 0:
                self.m_narrowphase.m_static0Index = 0
        return idx

    def autotune(self, deltaTime: float = 1.0 / 60.0, repeats: int = 3) -> dict:
        """Times candidate launch shapes on the current state and keeps the fastest (b3g_autotune;
        no reference counterpart).  The simulation state is left unchanged."""
        t = capi.b3gTuning()
        call("b3g_autotune", self._h, C.c_float(deltaTime), C.c_int(repeats), C.byref(t))
        return {f: getattr(t, f) for f, _ in capi.b3gTuning._fields_}

    def tuning(self) -> dict:
        t = capi.b3gTuning()
        call("b3g_get_tuning", self._h, C.byref(t))
        return {f: getattr(t, f) for f, _ in capi.b3gTuning._fields_}

    def setBroadphase(self, mode: int):
        """capi.BROADPHASE_GRID or capi.BROADPHASE_LBVH for the pair search (b3g_set_broadphase)."""
        call("b3g_set_broadphase", self._h, C.c_int(mode))

    def setSceneOffsets(self, firstBody):
        """Independent scenes stepped together (no reference counterpart: the reference runs one
        pipeline per scene).  Scene s owns bodies [firstBody[s], firstBody[s+1]), its static bodies
        included; no pair is formed across scenes.  Call before writeAllInstancesToGpu."""
        off = np.ascontiguousarray(np.asarray(firstBody, np.int32))
        call("b3g_set_scene_offsets", self._h, iptr(off) if len(off) else None, C.c_int(len(off)))

    def writeAllInstancesToGpu(self):
        self.m_narrowphase.writeAllBodiesToGpu()

    # joints (b3GpuRigidBodyPipeline.cpp:159-219); solved every step right before the contacts
    def createPoint2PointConstraint(self, bodyA: int, bodyB: int, pivotInA, pivotInB,
                                    breakingThreshold: float) -> int:
        """Ball joint: pivotInA (in A's frame) and pivotInB (in B's frame) are held together.  Returns
        the joint's uid.  Breaks for good once a row's impulse reaches breakingThreshold."""
        uid = C.c_int()
        pa = (C.c_float * 3)(*[float(x) for x in pivotInA[:3]])
        pb = (C.c_float * 3)(*[float(x) for x in pivotInB[:3]])
        call("b3g_create_point2point_constraint", self._h, C.c_int(bodyA), C.c_int(bodyB), pa, pb,
             C.c_float(breakingThreshold), C.byref(uid))
        return uid.value

    def createFixedConstraint(self, bodyA: int, bodyB: int, pivotInA, pivotInB, relTargetAB,
                              breakingThreshold: float) -> int:
        """Point to point plus the relative orientation ornA * ornB^-1 held at relTargetAB (x, y, z, w)."""
        uid = C.c_int()
        pa = (C.c_float * 3)(*[float(x) for x in pivotInA[:3]])
        pb = (C.c_float * 3)(*[float(x) for x in pivotInB[:3]])
        rel = (C.c_float * 4)(*[float(x) for x in relTargetAB[:4]])
        call("b3g_create_fixed_constraint", self._h, C.c_int(bodyA), C.c_int(bodyB), pa, pb, rel,
             C.c_float(breakingThreshold), C.byref(uid))
        return uid.value

    def removeConstraintByUid(self, uid: int):
        call("b3g_remove_constraint", self._h, C.c_int(uid))

    def getNumConstraints(self) -> int:
        n = C.c_int()
        call("b3g_get_num_constraints", self._h, C.byref(n))
        return n.value

    def copyConstraintsToHost(self) -> np.ndarray:
        """The joints (b3GpuGenericConstraint layout) with the enabled flags as the device left them."""
        n = self.getNumConstraints()
        out = np.zeros(n, capi.JOINT)
        if n:
            got = C.c_int()
            call("b3g_read_constraints", self._h, C.c_void_p(out.ctypes.data), C.c_int(n), C.byref(got))
        return out

    def readJointOrder(self):
        """(joint indices batch by batch, batch offsets) of the last joint solve."""
        n = self.getNumConstraints()
        order = np.zeros(max(1, n), np.int32)
        off = np.zeros(n + 2, np.int32)
        nb = C.c_int()
        call("b3g_read_joint_order", self._h, iptr(order), C.c_int(n), iptr(off), C.c_int(n + 2), C.byref(nb))
        return order[:n], off[:nb.value + 1]

    def solveJoints(self):
        """The joint stage alone (b3GpuPgsConstraintSolver::solveJoints)."""
        call("b3g_solve_joints", self._h)

    def setGravity(self, grav):
        g = (C.c_float * 3)(*[float(x) for x in grav[:3]])
        call("b3g_set_gravity", self._h, g)

    def setSolver(self, mode: int, iterations: int, residual_tol: float = 0.0):
        call("b3g_set_solver", self._h, C.c_int(mode), C.c_int(iterations), C.c_float(residual_tol))

    def stepSimulation(self, deltaTime: float):
        call("b3g_step", self._h, C.c_float(deltaTime))

    def setupGpuAabbsFull(self):
        call("b3g_setup_aabbs", self._h)

    def solveContacts(self, deltaTime: float):
        call("b3g_solve_contacts", self._h, C.c_float(deltaTime))

    def integrate(self, timeStep: float):
        call("b3g_integrate", self._h, C.c_float(timeStep))

    def synchronize(self):
        call("b3g_synchronize", self._h)

    def getNumBodies(self) -> int:
        return self.m_narrowphase.getNumRigidBodies()

    def getBodyBuffer(self) -> int:
        return self.m_narrowphase.getBodiesGpu()

    def stats(self) -> capi.b3gStepStats:
        s = capi.b3gStepStats()
        call("b3g_get_stats", self._h, C.byref(s))
        return s

    def status(self, clear: bool = False) -> int:
        f = C.c_uint()
        call("b3g_status", self._h, C.byref(f), C.c_int(1 if clear else 0))
        return f.value

    def readBatches(self) -> np.ndarray:
        n = C.c_int()
        call("b3g_read_batches", self._h, None, C.c_int(0), C.byref(n))
        out = np.zeros(n.value, np.int32)
        if n.value:
            call("b3g_read_batches", self._h, iptr(out), C.c_int(n.value), C.byref(n))
        return out

    def readSolveOrder(self) -> np.ndarray:
        """Manifold order whose sequential PGS sweep reproduces the GPU's last solve bit for bit."""
        n = C.c_int()
        call("b3g_read_solve_order", self._h, None, C.c_int(0), C.byref(n))
        out = np.zeros(n.value, np.int32)
        if n.value:
            call("b3g_read_solve_order", self._h, iptr(out), C.c_int(n.value), C.byref(n))
        return out

    def setWarmStartModel(self, model):
        """Attach a bullet3_gb300.warmstart.WarmStartMLP (None detaches); used when warm_start=1."""
        self._warm_model = model  # keep it alive while attached
        call("b3g_set_warm_start_model", self._h, model.handle if model is not None else None)

    def readWarmSamples(self, with_new: bool = False):
        """(features n x 12, converged impulses n x 3[, is_new n]) of the last solve's active points."""
        n = C.c_int()
        call("b3g_read_warm_samples", self._h, None, None, None, C.c_int(0), C.byref(n))
        f = np.zeros((n.value, 12), np.float32)
        t = np.zeros((n.value, 3), np.float32)
        new = np.zeros(n.value, np.int32)
        if n.value:
            call("b3g_read_warm_samples", self._h, fptr(f), fptr(t), iptr(new), C.c_int(n.value), C.byref(n))
        return (f, t, new.astype(bool)) if with_new else (f, t)

    def readWarmStart(self) -> np.ndarray:
        """Initial impulses of the last solve, 12 per manifold in the readImpulses layout."""
        n = C.c_int()
        call("b3g_read_warm_start", self._h, None, C.c_int(0), C.byref(n))
        out = np.zeros((n.value, 12), np.float32)
        if n.value:
            call("b3g_read_warm_start", self._h, fptr(out), C.c_int(n.value), C.byref(n))
        return out

    def readImpulses(self) -> np.ndarray:
        n = C.c_int()
        call("b3g_read_impulses", self._h, None, C.c_int(0), C.byref(n))
        out = np.zeros((n.value, 12), np.float32)
        if n.value:
            call("b3g_read_impulses", self._h, fptr(out), C.c_int(n.value), C.byref(n))
        return out

    def setProfiling(self, on: bool):
        call("b3g_set_profiling", self._h, C.c_int(1 if on else 0))

    def stageTimes(self) -> np.ndarray:
        out = np.zeros(7, np.float32)
        call("b3g_get_stage_times", self._h, fptr(out))
        return out

    def launchCount(self) -> int:
        n = C.c_longlong()
        call("b3g_get_launch_count", self._h, C.byref(n))
        return n.value

    def castRaysDevice(self, deviceRays: int, deviceHits: int, numRays: int):
        """castRays on device buffers (b3g_cast_rays_device): capi.RAY and capi.RAYHIT arrays already
        on the world's device, given by address; enqueued, not synchronised."""
        call("b3g_cast_rays_device", self._h, C.c_void_p(deviceRays), C.c_void_p(deviceHits), C.c_int(numRays))

    def castRays(self, rays, hitResults=None) -> np.ndarray:
        """b3GpuRigidBodyPipeline::castRays: rays as a capi.RAY array (from, to; from[3] = scene in a
        world of several scenes) or a sequence of (from, to) points; hitResults (capi.RAYHIT, optional)
        carries each ray's body to ignore in hitResult2.  Returns the hits: hitFraction 1 = no hit."""
        if not isinstance(rays, np.ndarray) or rays.dtype != capi.RAY:
            r = np.zeros(len(rays), capi.RAY)
            for i, (f, t) in enumerate(rays):
                r["from"][i, :3] = f[:3]
                r["to"][i, :3] = t[:3]
            rays = r
        rays = np.ascontiguousarray(rays, capi.RAY)
        if hitResults is None:
            hits = np.zeros(len(rays), capi.RAYHIT)
            hits["hitBody"] = -1
            hits["hitResult2"] = -1
        else:
            hits = np.array(hitResults, capi.RAYHIT, copy=True)
        call("b3g_cast_rays", self._h, ptr(rays), ptr(hits), C.c_int(len(rays)))
        return hits
