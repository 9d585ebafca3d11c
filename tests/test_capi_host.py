"""CPU-only checks of the boundary: the library loads without a GPU, exports every entry point
include/b3g_capi.h declares, and the host-side registry (shapes, bodies, hull builder, error
codes) behaves like the reference's registration API."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, load_golden
from bullet3_gb300 import capi, scenes
from bullet3_gb300.pipeline import b3Config, b3GpuNarrowPhase, b3GpuRigidBodyPipeline


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    decl = set()
    for hdr in Path(ROOT, "include").glob("*.h"):
        decl |= set(re.findall(r"\b(b3g_[a-z0-9_]+)\s*\(", hdr.read_text()))
    assert decl, "no declarations found"
    missing = [s for s in sorted(decl) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(capi.EXPORTS) <= decl


def test_layouts_match_reference_sizes():
    sizes = {capi.BODY: 80, capi.INERTIA: 96, capi.COLLIDABLE: 16, capi.HULL: 96, capi.FACE: 32, capi.AABB: 32,
             capi.CONTACT: 112, capi.RAY: 32, capi.RAYHIT: 48, capi.JOINT: 80}
    for dt, n in sizes.items():
        assert dt.itemsize == n


def test_registration_errors_match_reference_conventions():
    np_ = b3GpuNarrowPhase(b3Config(m_maxConvexShapes=2, m_maxConvexBodies=2))
    pl = b3GpuRigidBodyPipeline(np_)
    s = np_.registerSphereShape(0.5)
    assert s == 0
    assert np_.registerPlaneShape((0, 1, 0), 0.0) == 1
    assert np_.registerSphereShape(0.2) == -1  # capacity: -1 + b3Error (allocateCollidable)
    assert pl.registerPhysicsInstance(1.0, (0, 0, 0), (0, 0, 0, 1), 7) == -1  # invalid collidable index
    assert pl.registerPhysicsInstance(1.0, (0, 0, 0), (0, 0, 0, 1), s) == 0
    assert pl.registerPhysicsInstance(0.0, (0, 0, 0), (0, 0, 0, 1), 1) == 1
    assert pl.registerPhysicsInstance(1.0, (0, 0, 0), (0, 0, 0, 1), s) == -1  # body capacity
    assert np_.registerCompoundShape([]) == -1 and np_.registerConcaveMesh(None, None) == -1
    with pytest.raises(capi.B3GError):
        capi.call("b3g_step", C.c_void_p(None), C.c_float(1 / 60))
    with pytest.raises(capi.B3GError) as e:
        capi.call("b3g_step", np_.world.handle, C.c_float(1 / 60))
    assert e.value.status == 5  # not uploaded
    assert np_.registerConvexHullShape(np.zeros((3, 3), np.float32)) == -1  # degenerate hull


def test_compound_registration_matches_the_oracle_registry():
    # registerCompoundShape: the collidable (type 6, first child, child count), the children with
    # their poses, and the local AABB as the union of the children's moved into the compound's frame
    # (b3GpuNarrowPhase.cpp:370-433), bit-exact with the oracle's registry
    from bullet3_gb300 import scenes
    from oracle import oracle as O
    sc = scenes.compound_scene(64, seed=5)
    np_, bp, pl = scenes.load_scene(sc, b3Config(use_cuda_graph=False), upload=False)
    t = scenes.registered_tables(np_)
    ref = O.register_scene(sc)
    for k in ("collidables", "local_aabbs", "children"):
        assert np.array_equal(t[k].view(np.uint8), ref[k].view(np.uint8)), k
    assert (t["collidables"]["shapeType"] == capi.SHAPE_COMPOUND).sum() == 2
    # a child that is not a convex hull is refused (-1 + b3Error), the table left unchanged
    assert np_.registerCompoundShape([(0, (0, 0, 0), (0, 0, 0, 1))]) == -1  # collidable 0 is the plane
    assert np_.getNumCollidablesGpu() == len(t["collidables"])


def test_concave_mesh_registration_and_bvh():
    # registerConcaveMesh: the collidable (type 5, BVH index), one face per triangle with the
    # reference's plane (normalised (v1 - v0) x (v2 - v0), w = -n.v0), the scaled vertices and the
    # local AABB, bit-exact with the oracle's registry; the BVH holds every triangle once as a leaf,
    # in index order depth first, inside the mesh's quantization bounds, and a walk of it finds the
    # oracle's triangle-convex pairs (the reference's traversal on the same leaf boxes)
    from bullet3_gb300 import scenes
    from oracle import oracle as O
    sc = scenes.terrain_scene(200, grid=16, seed=4)
    np_, bp, pl = scenes.load_scene(sc, b3Config(use_cuda_graph=False), upload=False)
    t = scenes.registered_tables(np_)
    ref = O.register_scene(sc)
    for k in ("collidables", "local_aabbs", "hulls", "faces", "indices", "verts"):
        assert np.array_equal(t[k].view(np.uint8), ref[k].view(np.uint8)), k
    ni, nn = C.c_int(), C.c_int()
    capi.call("b3g_read_mesh_bvh", np_.world.handle, None, C.c_int(0), None, C.c_int(0), C.byref(ni), C.byref(nn))
    infos = np.zeros(ni.value, capi.BVHINFO)
    nodes = np.zeros(nn.value, capi.BVHNODE)
    capi.call("b3g_read_mesh_bvh", np_.world.handle, capi.ptr(infos), C.c_int(ni.value), capi.ptr(nodes),
              C.c_int(nn.value), C.byref(ni), C.byref(nn))
    assert ni.value == 1 and infos[0]["numTriangles"] == 2 * 16 * 16 and infos[0]["numNodes"] == 2 * 512 - 1
    la = t["local_aabbs"][0]
    f32 = np.float32
    assert np.array_equal(infos[0]["aabbMin"][:3], (la["min"] - f32(1)).astype(f32))
    assert np.array_equal(infos[0]["quantization"][:3],
                          (f32(65533) / (infos[0]["aabbMax"][:3] - infos[0]["aabbMin"][:3])).astype(f32))
    leaves = nodes["escapeOrTriangle"][nodes["escapeOrTriangle"] >= 0]
    assert np.array_equal(leaves, np.arange(512))

    def walk(qmin, qmax):
        out, cur = [], 0
        while cur < len(nodes):
            n = nodes[cur]
            ov = not ((qmin > n["qmax"]).any() or (qmax < n["qmin"]).any())
            e = int(n["escapeOrTriangle"])
            if ov and e >= 0:
                out.append(e)
            cur += 1 if (ov or e >= 0) else -e
        return out

    b = ref["bodies"]
    sh = O.Shapes.from_tables(ref)
    aabbs = O.aabbs(b, sh)
    pairs = O.pairs_bruteforce(aabbs)
    want = O.concave_pairs(b, sh, aabbs, pairs)
    info = infos[0]

    def quant(p, is_max):
        c = np.minimum(np.maximum(p.astype(f32), info["aabbMin"][:3]), info["aabbMax"][:3])
        v = ((c - info["aabbMin"][:3]) * info["quantization"][:3]).astype(f32)
        return ((v + f32(1)).astype(np.uint16) | 1) if is_max else (v.astype(np.uint16) & 0xfffe)

    got = []
    for p in pairs:
        x, y = int(p["x"]), int(p["y"])
        if x != 0 or b[y]["invMass"] == 0:
            continue
        col = t["collidables"][b[y]["collidableIdx"]]
        nch = int(col["numChildShapes"]) if col["shapeType"] == capi.SHAPE_COMPOUND else 1
        for tri in walk(quant(aabbs[y]["min"], False), quant(aabbs[y]["max"], True)):
            for c in range(nch):
                got.append((x, y, tri, int(col["shapeIndex"]) + c if col["shapeType"] == capi.SHAPE_COMPOUND else 0))
    assert len(want) > 500
    assert np.array_equal(np.array(got, np.int32).reshape(-1, 4), want.view(np.int32).reshape(-1, 4))
    # invalid input: -1 + b3Error, as the reference's registration reports it
    assert np_.registerConcaveMesh(np.zeros((3, 3), np.float32), [0, 1, 5]) == -1
    assert np_.registerConcaveMesh(None, None) == -1


def test_config_validation():
    h = C.c_void_p()
    for bad in (dict(pgs_partitions=5), dict(pgs_partitions=-1), dict(solver_blocks_per_sm=-2), dict(grid_dim=100),
                dict(pgs_interleave=2), dict(broadphase=3)):
        cfg = capi.default_config(**bad)
        with pytest.raises(capi.B3GError) as e:
            capi.call("b3g_create", C.byref(cfg), C.c_int(0), C.byref(h))
        assert e.value.status == 1  # invalid argument
    for ok in (capi.PGS_PARTITIONS_AUTO, capi.PGS_PARTITIONS_GLOBAL_DELTAS, capi.PGS_PARTITIONS_NONE,
               capi.PGS_PARTITIONS_SHARED, capi.PGS_PARTITIONS_STREAMED):
        cfg = capi.default_config(pgs_partitions=ok, solver_blocks_per_sm=1)
        capi.call("b3g_create", C.byref(cfg), C.c_int(0), C.byref(h))
        capi.call("b3g_destroy", h)


def test_registered_body_matches_reference_registration():
    # registerPhysicsInstance: margin-0.01 AABB, AABB-box inertia using the full extent as the
    # "half extent" (b3GpuNarrowPhase.cpp:876-901), friction 1, restitution 0
    np_ = b3GpuNarrowPhase(b3Config())
    pl = b3GpuRigidBodyPipeline(np_)
    box = np_.registerConvexHullShape(scenes.box_vertices(0.5, 0.5, 0.5))
    pl.registerPhysicsInstance(2.0, (1, 2, 3), (0, 0, 0, 1), box)
    t = scenes.registered_tables(np_)
    b, I = t["bodies"][0], t["inertias"][0]
    assert b["invMass"] == np.float32(0.5) and b["friction"] == 1.0 and b["restitution"] == 0.0
    l = 2 * (1.0 + 0.02)
    expect = 1.0 / ((2.0 / 12.0) * (l * l + l * l))
    np.testing.assert_allclose(np.diag(I["initInvInertia"][:, :3]), [expect] * 3, rtol=1e-6)
    np.testing.assert_allclose(I["invInertiaWorld"][:, :3], np.diag([expect] * 3), rtol=1e-6, atol=1e-9)


def test_hull_builder_bitexact_against_reference():
    """registerConvexHullShape's tables from the product's hull builder equal the reference's bit
    for bit (same vertex order, faces in the same order with the same planes and start vertices,
    same unique edges) on 170 point clouds: Gaussian clouds, boxes, rotated boxes, cylinders,
    lattice points, sphere clouds and clouds with repeated points."""
    n = 0
    for name in ("hulls", "registration"):
        g = load_golden(name)
        for i in range(int(g["count"])):
            mine = capi.hull_compute(g[f"in_{i}"])
            ref = (g[f"v_{i}"], g[f"p_{i}"], g[f"fc_{i}"], g[f"ix_{i}"], g[f"e_{i}"])
            for a, b in zip(mine[:5], ref):
                assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), (name, i)
            n += 1
    assert n == 170
    # boxes: 6 quads, 3 unique edges
    g = load_golden("hulls")
    for i in range(6):
        mine = capi.hull_compute(g[f"in_{i}"])
        assert len(mine[2]) == 6 and (mine[2] == 4).all() and len(mine[4]) == 3


def test_body_registration_bitexact_against_reference():
    """registerPhysicsInstance through the C ABI writes the reference's body and inertia records bit
    for bit (margin-0.01 world AABB, full-extent AABB-box inertia, frozen world inverse inertia)."""
    g = load_golden("registration")
    n = len(g["bodies"])
    np_ = b3GpuNarrowPhase(b3Config(m_maxConvexBodies=n, m_maxConvexShapes=n))
    pl = b3GpuRigidBodyPipeline(np_)
    for i in range(n):
        lo, hi = g["body_local_min"][i], g["body_local_max"][i]
        corners = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])],
                           np.float32)
        # a hull registered from its tables: its local AABB is exactly [lo, hi]
        col = np_.registerConvexHullShapeTables(corners, np.array([[0, 1, 0, 0]], np.float32), [3], [0, 1, 2],
                                                np.zeros((0, 3), np.float32))
        assert pl.registerPhysicsInstance(float(g["body_mass"][i]), g["body_pos"][i], g["body_orn"][i], col, i) == i
    t = scenes.registered_tables(np_)
    t["bodies"]["collidableIdx"] = 3
    assert t["bodies"].tobytes() == g["bodies"].tobytes()
    assert t["inertias"].tobytes() == g["inertias"].tobytes()


def test_scene_offsets_validation():
    np_ = b3GpuNarrowPhase(b3Config())
    pl = b3GpuRigidBodyPipeline(np_)
    plane = np_.registerPlaneShape((0, 1, 0), 0.0)
    box = np_.registerConvexHullShape(scenes.box_vertices(0.5, 0.5, 0.5))
    for k in range(6):
        pl.registerPhysicsInstance(0.0 if k % 3 == 0 else 1.0, (0, 1 + k, 0), (0, 0, 0, 1), plane if k % 3 == 0 else box)
    for bad in ([1, 3], [0, 4, 2]):  # must start at body 0 and never decrease
        with pytest.raises(capi.B3GError) as e:
            pl.setSceneOffsets(bad)
        assert e.value.status == 1
    pl.setSceneOffsets([0, 3, 3])  # an empty scene is allowed
    pl.setSceneOffsets([0, 3])
    pl.setSceneOffsets([])  # back to one scene


def test_cpp_dropin_header_compiles(tmp_path):
    # the C++ classes of include/b3g_compat.h compile on their own against the public headers, with
    # the reference's constructor and method signatures
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "use.cpp"
    src.write_text('#include "b3g_compat.h"\n'
                   "int main() {\n"
                   "  cl_context ctx = b3gCreateContext(0); cl_device_id dev = b3gGetDevice(ctx);\n"
                   "  cl_command_queue q = b3gCreateCommandQueue(ctx, dev);\n"
                   "  b3Config c; b3GpuNarrowPhase np(ctx, dev, q, c); b3GpuGridBroadphase bp(ctx, dev, q);\n"
                   "  b3DynamicBvhBroadphase dbvt(c.m_maxConvexBodies);\n"
                   "  b3GpuRigidBodyPipeline rbp(ctx, dev, q, &np, &bp, &dbvt, c);\n"
                   "  int first[2] = {0, 1}; rbp.setSceneOffsets(first, 2);\n"
                   "  b3GpuBroadphaseInterface::CreateFunc* f = b3GpuSapBroadphase::CreateFuncBarrier; delete f(ctx, dev, q);\n"
                   "  f = b3GpuParallelLinearBvhBroadphase::CreateFunc; delete f(ctx, dev, q);\n"
                   "  f = b3GpuGridBroadphase::CreateFunc; delete f(ctx, dev, q);\n"
                   "  b3GpuParallelLinearBvhBroadphase lbvh(ctx, dev, q);\n"
                   "  float p[3], o[4]; np.getObjectTransformFromCpu(p, o, 0); np.setObjectTransformCpu(p, o, 0);\n"
                   "  np.registerPlaneShape(b3MakeVector3(0, 1, 0), 0.f);\n"
                   "  b3ConvexUtility u; b3AlignedObjectArray<b3Vector3> v; v.push_back(b3MakeVector3(0, 0, 0));\n"
                   "  u.initializePolyhedralFeatures(&v[0], v.size()); np.registerConvexHullShape(&u);\n"
                   "  rbp.registerConvexPolyhedron(&u);\n"
                   "  b3AlignedObjectArray<b3GpuChildShape> kids; b3GpuChildShape ch;\n"
                   "  ch.m_childPosition = b3MakeVector3(0.5f, 0, 0); ch.m_childOrientation = b3Quaternion(0, 0, 0, 1);\n"
                   "  ch.m_shapeIndex = 1; ch.m_numChildShapes = 0; ch.m_collidableShapeIndex = 0; ch.m_shapeType = 3;\n"
                   "  kids.push_back(ch); np.registerCompoundShape(&kids);\n"
                   "  b3AlignedObjectArray<int> tri; tri.push_back(0); tri.push_back(0); tri.push_back(0);\n"
                   "  float one[3] = {1.f, 1.f, 1.f}; np.registerConcaveMesh(&v, &tri, one);\n"
                   "  bp.calculateOverlappingPairsHost(0); bp.getAllAabbsCPU(); rbp.copyConstraintsToHost();\n"
                   "  b3OpenCLArray<b3Int4>& pairs = bp.getOverlappingPairsGPU();\n"
                   "  np.computeContacts(pairs.getBufferCL(), (int)pairs.size(), bp.getAabbBufferWS(), 0);\n"
                   "  b3AlignedObjectArray<b3RayInfo> rays; b3AlignedObjectArray<b3RayHit> hits; rbp.castRays(rays, hits);\n"
                   "  float pa[3] = {0, 0, 0}, rel[4] = {0, 0, 0, 1};\n"
                   "  int id = rbp.createPoint2PointConstraint(0, 1, pa, pa, 1e30f);\n"
                   "  id += rbp.createFixedConstraint(0, 1, pa, pa, rel, 1e30f); rbp.removeConstraintByUid(id);\n"
                   "  rbp.reset(); np.reset(); const b3Contact4* cc = np.getContactsCPU(); (void)cc;\n"
                   "  b3Quaternion orn(0, 0, 0, 1); rbp.registerPhysicsInstance(1.f, b3MakeVector3(0, 1, 0), orn, 0, 0, false);\n"
                   "  rbp.stepSimulation(1.f / 60.f); b3gRelease(q); b3gRelease(dev); b3gRelease(ctx);\n"
                   "  return rbp.getNumBodies();\n"
                   "}\n")
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", str(Path(ROOT, "include")), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


# The physics parts of the reference's own GPU rigid-body demos, read from the reference's sources
# when they are on this machine (they are not part of this repository): the pipeline construction
# of GpuRigidBodyDemo::initPhysics, the scene setup of GpuConvexScene::createDynamicsObjects2 and
# the step of GpuRigidBodyDemo::stepSimulation.
DEMO_SNIPPETS = [
    ("examples/OpenCL/rigidbody/GpuRigidBodyDemo.cpp", "m_data->m_config.m_maxConvexBodies = b3Max(",
     "bp->writeAabbsToGpu();"),
    ("examples/OpenCL/rigidbody/GpuConvexScene.cpp",
     "int shapeId = m_guiHelper->getRenderInterface()->registerShape(&vertices[0], numVertices, indices, "
     "numIndices, B3_GL_TRIANGLES, textureIndex);", "return index;"),
    ("examples/OpenCL/rigidbody/GpuRigidBodyDemo.cpp", "m_data->m_rigidBodyPipeline->stepSimulation(1. / 60.f);",
     "m_data->m_rigidBodyPipeline->stepSimulation(1. / 60.f);"),
]

DEMO_HARNESS = r"""
#include <cstdio>
#include "b3g_compat.h"
// stand-ins for the demo framework's renderer, its state and its globals
#define B3_GL_TRIANGLES 1
#define b3Assert(x) ((void)0)
struct RenderInterface {
    int registerShape(const float*, int, const int*, int, int, int) { return 0; }
    int registerGraphicsInstance(int, const float*, const float*, const float*, const float*) { return 0; }
};
struct GuiHelper {
    RenderInterface r;
    RenderInterface* getRenderInterface() { return &r; }
};
struct ClData {
    cl_context m_clContext;
    cl_device_id m_clDevice;
    cl_command_queue m_clQueue;
};
struct DemoData {
    b3Config m_config;
    b3GpuNarrowPhase* m_np = nullptr;
    b3GpuBroadphaseInterface* m_bp = nullptr;
    b3DynamicBvhBroadphase* m_broadphaseDbvt = nullptr;
    b3GpuRigidBodyPipeline* m_rigidBodyPipeline = nullptr;
};
static bool gUseInstancedCollisionShapes = true;
static bool useUniformGrid = true;
static int gGpuArraySizeX = 4, gGpuArraySizeY = 4, gGpuArraySizeZ = 4;
static b3Vector4 colors[4] = {b3MakeVector4(1, 0, 0, 1), b3MakeVector4(0, 1, 0, 1), b3MakeVector4(0, 0, 1, 1),
                              b3MakeVector4(0, 1, 1, 1)};
struct Demo {
    GuiHelper guiHelper;
    GuiHelper* m_guiHelper = &guiHelper;
    ClData clData;
    ClData* m_clData = &clData;
    DemoData data;
    DemoData* m_data = &data;
    void setupScene() {}
    void initPhysics() {
@@INIT@@
    }
    int createDynamicsObjects2(const float* vertices, int numVertices, const int* indices, int numIndices,
                               int strideInBytes, int textureIndex) {
@@SCENE@@
    }
    void stepSimulation() {
@@STEP@@
    }
};
int main(int argc, char**) {
    Demo d;
    d.clData.m_clContext = b3gCreateContext(0);
    d.clData.m_clDevice = b3gGetDevice(d.clData.m_clContext);
    d.clData.m_clQueue = b3gCreateCommandQueue(d.clData.m_clContext, d.clData.m_clDevice);
    const float cube[8 * 9] = {
        -1, -1, -1, 1, 0, 0, 0, 0, 0,  1, -1, -1, 1, 0, 0, 0, 0, 0,  -1, 1, -1, 1, 0, 0, 0, 0, 0,
        1, 1, -1, 1, 0, 0, 0, 0, 0,    -1, -1, 1, 1, 0, 0, 0, 0, 0,  1, -1, 1, 1, 0, 0, 0, 0, 0,
        -1, 1, 1, 1, 0, 0, 0, 0, 0,    1, 1, 1, 1, 0, 0, 0, 0, 0};
    const int idx[3] = {0, 1, 2};
    if (argc > 1) {  // with a GPU: construct, set up, upload and step
        d.initPhysics();
        int n = d.createDynamicsObjects2(cube, 8, idx, 3, 9 * sizeof(float), 0);
        d.m_data->m_rigidBodyPipeline->writeAllInstancesToGpu();
        for (int i = 0; i < 10; i++) d.stepSimulation();
        std::printf("bodies %d\n", n);
    }
    return 0;
}
"""


def _demo_source():
    from oracle import build as oracle_build
    root = oracle_build.reference_root()
    if root is None:
        return None
    parts = []
    for rel, first, last in DEMO_SNIPPETS:
        lines = Path(root, rel).read_text().splitlines()
        i = next(k for k, l in enumerate(lines) if first in l)
        j = next(k for k in range(i, len(lines)) if last in lines[k])
        parts.append("\n".join(lines[i:j + 1]))
    return (DEMO_HARNESS.replace("@@INIT@@", parts[0]).replace("@@SCENE@@", parts[1])
            .replace("@@STEP@@", parts[2]))


def test_reference_demo_physics_code_builds_against_the_dropin(tmp_path):
    """The reference demos' own pipeline construction, scene setup (hull registration through
    b3ConvexUtility, registerPhysicsInstance with b3Vector3 / b3Quaternion) and step compile and
    link, unmodified, against include/b3g_compat.h and libb3gpu.so; only the renderer and the
    OpenCL context creation are stand-ins.  Skipped where the reference's sources are absent."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = _demo_source()
    if src is None:
        pytest.skip("the reference's sources are not on this machine")
    f = tmp_path / "demo.cpp"
    f.write_text(src)
    lib_dir = Path(ROOT, "bullet3_gb300")
    exe = tmp_path / "demo"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(Path(ROOT, "include")), str(f), "-o", str(exe),
                        "-L", str(lib_dir), "-lb3gpu", f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr


def test_broadphase_switch_validation_before_upload():
    np_ = b3GpuNarrowPhase(b3Config())
    pl = b3GpuRigidBodyPipeline(np_)
    for mode in (capi.BROADPHASE_GRID, capi.BROADPHASE_LBVH, capi.BROADPHASE_AUTO):
        pl.setBroadphase(mode)  # before the upload: recorded in the config, no device work
    for bad in (-1, 3):
        with pytest.raises(capi.B3GError) as e:
            pl.setBroadphase(bad)
        assert e.value.status == 1
    with pytest.raises(capi.B3GError):
        capi.call("b3g_cast_rays_device", np_.world.handle, C.c_void_p(None), C.c_void_p(None), C.c_int(4))
