"""The C++ drop-in: a program written against the reference's class names (include/b3g_compat.h)
is compiled with g++, linked against libb3gpu.so, and steps a box pile on the GPU through the C
ABI.  Bar: it builds, runs without a b3Error, the boxes come to rest on the plane, the
broadphase/narrowphase getters report the pairs and contacts of the settled pile, a ray hits the
top box, and a ball joint lifts and holds a box until it is removed."""
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include <vector>
#include "b3g_compat.h"
using namespace b3g_compat;

int main() {
    b3Config config;
    config.m_maxConvexBodies = 1000;
    b3GpuNarrowPhase* np = new b3GpuNarrowPhase(0, config);        // was (ctx, device, queue, config)
    b3GpuGridBroadphase* bp = new b3GpuGridBroadphase();
    b3GpuRigidBodyPipeline* rbp = new b3GpuRigidBodyPipeline(np, bp, nullptr, config);
    float box[8 * 3];
    for (int i = 0; i < 8; i++) {
        box[3 * i + 0] = (i & 4) ? 0.5f : -0.5f;
        box[3 * i + 1] = (i & 2) ? 0.5f : -0.5f;
        box[3 * i + 2] = (i & 1) ? 0.5f : -0.5f;
    }
    const float scaling[3] = {1, 1, 1}, up[3] = {0, 1, 0}, orn[4] = {0, 0, 0, 1};
    const int boxShape = np->registerConvexHullShape(box, 3 * sizeof(float), 8, scaling);
    const int ground = np->registerPlaneShape(up, 0.f);
    if (boxShape < 0 || ground < 0) return 2;
    const float origin[3] = {0, 0, 0};
    rbp->registerPhysicsInstance(0.f, origin, orn, ground, 0, false);
    for (int x = 0; x < 4; x++)
        for (int y = 0; y < 4; y++)
            for (int z = 0; z < 4; z++) {
                const float pos[3] = {1.1f * x, 0.6f + 1.1f * y, 1.1f * z};
                if (rbp->registerPhysicsInstance(1.f, pos, orn, boxShape, 1, false) < 0) return 3;
            }
    rbp->writeAllInstancesToGpu();
    for (int frame = 0; frame < 150; frame++) rbp->stepSimulation(1.f / 60.f);
    std::vector<b3gBody> bodies;
    np->readbackAllBodiesToCpu(bodies);
    float ymin = 1e30f, vmax = 0.f;
    for (size_t i = 1; i < bodies.size(); i++) {
        ymin = std::fmin(ymin, bodies[i].pos.y);
        vmax = std::fmax(vmax, std::fabs(bodies[i].linVel.y));
    }
    // the drop-in stage calls on the settled state: 16 columns of 4 boxes -> 16 plane + 48 box-box manifolds
    rbp->setupGpuAabbsFull();
    bp->calculateOverlappingPairs(0);
    np->computeContacts();
    const int pairs = bp->getNumOverlap(), contacts = np->getNumContactsGpu();
    std::printf("bodies %d ymin %.4f vmax %.4f pairs %d contacts %d\n", rbp->getNumBodies(), ymin, vmax, pairs,
                contacts);
    bool ok = rbp->getNumBodies() == 65 && ymin > 0.4f && vmax < 0.5f && pairs >= 64 && contacts == 64 &&
              np->getBodiesGpu() != nullptr && bp->getOverlappingPairBuffer() != nullptr;
    // host copies: read the pose of the top box of one column (body 13), kick it upwards, write, step
    ok = ok && np->getStatic0Index() == 0 && (int)bp->getAllAabbsCPU().size() == 65;
    bp->calculateOverlappingPairsHost(0);
    ok = ok && bp->getNumOverlap() == pairs;
    np->readbackAllBodiesToCpu();
    float p0[3], q0[4];
    ok = ok && np->getObjectTransformFromCpu(p0, q0, 13);
    const float up5[3] = {0.f, 5.f, 0.f}, zero[3] = {0.f, 0.f, 0.f};
    np->setObjectVelocityCpu(up5, zero, 13);
    np->writeAllBodiesToGpu();
    rbp->stepSimulation(1.f / 60.f);
    np->readbackAllBodiesToCpu();
    float p1[3], q1[4];
    ok = ok && np->getObjectTransformFromCpu(p1, q1, 13) && p1[1] > p0[1] + 0.05f;
    // a ray straight down onto column (0, 0) hits its top box, the one just kicked
    std::vector<b3gRayInfo> rays(1);
    std::vector<b3gRayHit> hits(1);
    rays[0].from = b3gFloat4{0.f, 20.f, 0.f, 0.f};
    rays[0].to = b3gFloat4{0.f, -1.f, 0.f, 0.f};
    hits[0].hitResult2 = -1;
    rbp->castRays(rays, hits);
    ok = ok && hits[0].hitFraction < 1.f && hits[0].hitBody == 13;
    // a ball joint from the static plane (body 0) at (0, 10, 0) to the centre of box 13 lifts it
    // there and holds it; removing the joint lets it fall
    const float pivotA[3] = {0.f, 10.f, 0.f}, pivotB[3] = {0.f, 0.f, 0.f};
    const int uid = rbp->createPoint2PointConstraint(0, 13, pivotA, pivotB, 1e30f);
    for (int frame = 0; frame < 120; frame++) rbp->stepSimulation(1.f / 60.f);
    rbp->copyConstraintsToHost();
    np->readbackAllBodiesToCpu();
    float p2[3], q2[4];
    ok = ok && uid >= 0 && np->getObjectTransformFromCpu(p2, q2, 13);
    const float hang = std::sqrt(p2[0] * p2[0] + (p2[1] - 10.f) * (p2[1] - 10.f) + p2[2] * p2[2]);
    ok = ok && hang < 0.1f && rbp->getConstraintsCPU().size() == 1 && rbp->getConstraintsCPU()[0].flags == 1;
    rbp->removeConstraintByUid(uid);
    for (int frame = 0; frame < 20; frame++) rbp->stepSimulation(1.f / 60.f);
    np->readbackAllBodiesToCpu();
    float p3[3], q3[4];
    ok = ok && np->getObjectTransformFromCpu(p3, q3, 13) && p3[1] < p2[1] - 0.5f;
    std::printf("joint holds box at %.4f %.4f %.4f (off %.4f); released -> y %.4f\n", p2[0], p2[1], p2[2], hang,
                p3[1]);
    b3GpuBroadphaseInterface::CreateFunc* create = b3GpuSapBroadphase::CreateFunc;
    b3GpuBroadphaseInterface* other = create(0);
    ok = ok && other != nullptr;
    delete other;
    std::printf("kicked box %.4f -> %.4f\n", p0[1], p1[1]);
    delete rbp;
    delete bp;
    delete np;
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
