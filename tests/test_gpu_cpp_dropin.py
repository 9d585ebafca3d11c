"""The C++ drop-in: a program written against the reference's classes and signatures (OpenCL-style
handles, b3ConvexUtility, b3Vector3, b3OpenCLArray; include/b3g_compat.h) is compiled with g++,
linked against libb3gpu.so, and steps a box pile on the GPU through the C ABI.  Bar: it builds,
runs without a b3Error, the boxes come to rest on the plane, the broadphase/narrowphase getters
report the pairs and contacts of the settled pile, computeContacts on caller-supplied pairs gives
the manifolds of exactly those pairs, a ray hits the top box, a ball joint lifts and holds a box
until it is removed, and after reset() the world takes a new scene."""
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include "b3g_compat.h"

int main() {
    // in place of b3OpenCLUtils::createContextFromType / getDevice / clCreateCommandQueue
    cl_context ctx = b3gCreateContext(0);
    cl_device_id dev = b3gGetDevice(ctx, 0);
    cl_command_queue queue = b3gCreateCommandQueue(ctx, dev);
    b3Config config;
    config.m_maxConvexBodies = 1000;
    config.m_maxConvexShapes = config.m_maxConvexBodies;
    config.m_maxBroadphasePairs = 16 * config.m_maxConvexBodies;
    config.m_maxContactCapacity = config.m_maxBroadphasePairs;
    b3GpuNarrowPhase* np = new b3GpuNarrowPhase(ctx, dev, queue, config);
    b3GpuBroadphaseInterface* bp = new b3GpuGridBroadphase(ctx, dev, queue);
    b3DynamicBvhBroadphase* dbvt = new b3DynamicBvhBroadphase(config.m_maxConvexBodies);
    b3GpuRigidBodyPipeline* rbp = new b3GpuRigidBodyPipeline(ctx, dev, queue, np, bp, dbvt, config);
    // hull tables through b3ConvexUtility, as the reference's demos register them
    b3AlignedObjectArray<b3Vector3> verts;
    for (int i = 0; i < 8; i++)
        verts.push_back(b3MakeVector3((i & 4) ? 0.5f : -0.5f, (i & 2) ? 0.5f : -0.5f, (i & 1) ? 0.5f : -0.5f));
    b3ConvexUtility* util = new b3ConvexUtility();
    util->initializePolyhedralFeatures(&verts[0], verts.size(), true);
    const int boxShape = np->registerConvexHullShape(util);
    const int boxShape2 = rbp->registerConvexPolyhedron(util);
    delete util;
    const int ground = np->registerPlaneShape(b3MakeVector3(0, 1, 0), 0.f);
    if (boxShape < 0 || boxShape2 < 0 || ground < 0) return 2;
    b3Quaternion orn(0, 0, 0, 1);
    rbp->registerPhysicsInstance(0.f, b3MakeVector3(0, 0, 0), orn, ground, 0, false);
    for (int x = 0; x < 4; x++)
        for (int y = 0; y < 4; y++)
            for (int z = 0; z < 4; z++) {
                b3Vector3 pos = b3MakeVector3(1.1f * x, 0.6f + 1.1f * y, 1.1f * z);
                if (rbp->registerPhysicsInstance(1.f, pos, orn, (x + y + z) % 2 ? boxShape : boxShape2, 1, false) < 0)
                    return 3;
            }
    rbp->writeAllInstancesToGpu();
    np->writeAllBodiesToGpu();
    bp->writeAabbsToGpu();
    for (int frame = 0; frame < 150; frame++) rbp->stepSimulation(1.f / 60.f);
    // the body buffer through b3OpenCLArray, as the demos read it back
    b3OpenCLArray<b3RigidBodyData> gpuBodies(ctx, queue);
    gpuBodies.setFromOpenCLBuffer(rbp->getBodyBuffer(), rbp->getNumBodies());
    b3AlignedObjectArray<b3RigidBodyData> bodies;
    gpuBodies.copyToHost(bodies);
    float ymin = 1e30f, vmax = 0.f;
    for (int i = 1; i < bodies.size(); i++) {
        ymin = std::fmin(ymin, bodies[i].m_pos.getY());
        vmax = std::fmax(vmax, std::fabs(bodies[i].m_linVel.getY()));
    }
    // the stage calls on the settled state: 16 columns of 4 boxes -> 16 plane + 48 box-box manifolds
    rbp->setupGpuAabbsFull();
    bp->calculateOverlappingPairs(config.m_maxBroadphasePairs);
    np->computeContacts(bp->getOverlappingPairBuffer(), bp->getNumOverlap(), bp->getAabbBufferWS(),
                        rbp->getNumBodies());
    const int pairs = bp->getNumOverlap(), contacts = np->getNumContactsGpu();
    std::printf("bodies %d ymin %.4f vmax %.4f pairs %d contacts %d\n", rbp->getNumBodies(), ymin, vmax, pairs,
                contacts);
    bool ok = rbp->getNumBodies() == 65 && ymin > 0.4f && vmax < 0.5f && pairs >= 64 && contacts == 64 &&
              np->getBodiesGpu() != nullptr && bp->getOverlappingPairBuffer() != nullptr;
    // computeContacts on pairs the caller passes: the overlapping pairs copied into a b3OpenCLArray
    // of its own, every second one dropped -> the manifolds of the kept pairs only
    b3AlignedObjectArray<b3Int4> hostPairs;
    bp->getOverlappingPairsGPU().copyToHost(hostPairs);
    b3AlignedObjectArray<b3Int4> half;
    for (int i = 0; i < hostPairs.size(); i += 2) half.push_back(hostPairs[i]);
    b3OpenCLArray<b3Int4> myPairs(ctx, queue);
    myPairs.copyFromHost(half);
    np->computeContacts(myPairs.getBufferCL(), half.size(), bp->getAabbBufferWS(), rbp->getNumBodies());
    const int halfContacts = np->getNumContactsGpu();
    const b3Contact4* hc = np->getContactsCPU();
    int inHalf = 0;
    for (int c = 0; c < halfContacts; c++)
        for (int i = 0; i < half.size(); i++)
            if ((std::abs(hc[c].bodyA) == half[i].x && std::abs(hc[c].bodyB) == half[i].y) ||
                (std::abs(hc[c].bodyA) == half[i].y && std::abs(hc[c].bodyB) == half[i].x)) {
                inHalf++;
                break;
            }
    std::printf("caller pairs %d -> contacts %d (all from those pairs: %d)\n", half.size(), halfContacts, inHalf);
    ok = ok && halfContacts > 0 && halfContacts < contacts && inHalf == halfContacts;
    // host copies: read the pose of the top box of one column (body 13), kick it upwards, write, step
    ok = ok && np->getStatic0Index() == 0 && bp->getAllAabbsCPU().size() == 65;
    ok = ok && (int)bp->getSmallAabbIndicesGPU().size() == 64 && (int)bp->getLargeAabbIndicesGPU().size() == 1;
    bp->calculateOverlappingPairsHost(config.m_maxBroadphasePairs);
    ok = ok && bp->getNumOverlap() == pairs;
    np->readbackAllBodiesToCpu();
    float p0[3] = {0, 0, 0}, q0[4] = {0, 0, 0, 1};
    ok = ok && np->getObjectTransformFromCpu(p0, q0, 13);
    float up5[3] = {0.f, 5.f, 0.f}, zero[3] = {0.f, 0.f, 0.f};
    np->setObjectVelocityCpu(up5, zero, 13);
    np->writeAllBodiesToGpu();
    rbp->stepSimulation(1.f / 60.f);
    np->readbackAllBodiesToCpu();
    float p1[3] = {0, 0, 0}, q1[4] = {0, 0, 0, 1};
    ok = ok && np->getObjectTransformFromCpu(p1, q1, 13) && p1[1] > p0[1] + 0.05f;
    // a ray straight down onto column (0, 0) hits its top box, the one just kicked
    b3AlignedObjectArray<b3RayInfo> rays;
    b3AlignedObjectArray<b3RayHit> hits;
    b3RayInfo ray;
    ray.m_from = b3MakeVector3(0.f, 20.f, 0.f);
    ray.m_to = b3MakeVector3(0.f, -1.f, 0.f);
    rays.push_back(ray);
    b3RayHit hit;
    hit.m_hitFraction = 1.f;
    hit.m_hitBody = -1;
    hit.m_hitResult2 = -1;
    hits.push_back(hit);
    rbp->castRays(rays, hits);
    ok = ok && hits[0].m_hitFraction < 1.f && hits[0].m_hitBody == 13;
    // a ball joint from the static plane (body 0) at (0, 10, 0) to the centre of box 13 lifts it
    // there and holds it; removing the joint lets it fall
    const float pivotA[3] = {0.f, 10.f, 0.f}, pivotB[3] = {0.f, 0.f, 0.f};
    const int uid = rbp->createPoint2PointConstraint(0, 13, pivotA, pivotB, 1e30f);
    for (int frame = 0; frame < 120; frame++) rbp->stepSimulation(1.f / 60.f);
    rbp->copyConstraintsToHost();
    np->readbackAllBodiesToCpu();
    float p2[3] = {0, 0, 0}, q2[4] = {0, 0, 0, 1};
    ok = ok && uid >= 0 && np->getObjectTransformFromCpu(p2, q2, 13);
    const float hang = std::sqrt(p2[0] * p2[0] + (p2[1] - 10.f) * (p2[1] - 10.f) + p2[2] * p2[2]);
    ok = ok && hang < 0.1f && rbp->getConstraintsCPU().size() == 1 && rbp->getConstraintsCPU()[0].flags == 1;
    rbp->removeConstraintByUid(uid);
    for (int frame = 0; frame < 20; frame++) rbp->stepSimulation(1.f / 60.f);
    np->readbackAllBodiesToCpu();
    float p3[3] = {0, 0, 0}, q3[4] = {0, 0, 0, 1};
    ok = ok && np->getObjectTransformFromCpu(p3, q3, 13) && p3[1] < p2[1] - 0.5f;
    std::printf("joint holds box at %.4f %.4f %.4f (off %.4f); released -> y %.4f\n", p2[0], p2[1], p2[2], hang,
                p3[1]);
    // reset(): the pipeline drops its joints, the narrowphase every shape and body; the world then
    // takes a fresh scene
    rbp->createPoint2PointConstraint(0, 13, pivotA, pivotB, 1e30f);
    rbp->reset();
    rbp->copyConstraintsToHost();
    ok = ok && rbp->getConstraintsCPU().size() == 0;
    np->reset();
    ok = ok && rbp->getNumBodies() == 0 && np->getNumCollidablesGpu() == 0;
    const int sphere = np->registerSphereShape(0.5f);
    const int plane2 = np->registerPlaneShape(b3MakeVector3(0, 1, 0), 0.f);
    rbp->registerPhysicsInstance(0.f, b3MakeVector3(0, 0, 0), orn, plane2, 0, false);
    rbp->registerPhysicsInstance(1.f, b3MakeVector3(0, 3, 0), orn, sphere, 1, false);
    rbp->writeAllInstancesToGpu();
    for (int frame = 0; frame < 120; frame++) rbp->stepSimulation(1.f / 60.f);
    np->readbackAllBodiesToCpu();
    float p4[3] = {0, 0, 0}, q4[4] = {0, 0, 0, 1};
    ok = ok && rbp->getNumBodies() == 2 && np->getObjectTransformFromCpu(p4, q4, 1) && std::fabs(p4[1] - 0.5f) < 0.05f;
    std::printf("after reset: sphere rests at y %.4f\n", p4[1]);
    b3GpuBroadphaseInterface::CreateFunc* create = b3GpuSapBroadphase::CreateFuncLocalMemory;
    b3GpuBroadphaseInterface* other = create(ctx, dev, queue);
    ok = ok && other != nullptr;
    delete other;
    std::printf("kicked box %.4f -> %.4f\n", p0[1], p1[1]);
    delete rbp;
    delete dbvt;
    delete bp;
    delete np;
    b3gRelease(queue);
    b3gRelease(dev);
    b3gRelease(ctx);
    return ok ? 0 : 1;
}
'''


def test_cpp_program_steps_a_pile_through_the_dropin(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    lib_dir = Path(ROOT, "bullet3_gb300")
    src = tmp_path / "dropin.cpp"
    exe = tmp_path / "dropin"
    src.write_text(PROGRAM)
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(Path(ROOT, "include")), str(src), "-o", str(exe),
                        "-L", str(lib_dir), "-lb3gpu", f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "b3Error" not in r.stderr, r.stderr
    assert r.stdout.startswith("bodies 65"), r.stdout
