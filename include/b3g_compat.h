/*
 * b3g_compat.h -- header-only C++ drop-in for the reference's GPU rigid-body API, implemented on
 * the C ABI of libb3gpu.so (include/b3g_capi.h).
 *
 * Class names, method names, argument meaning and error behaviour follow
 *   b3GpuNarrowPhase         src/Bullet3OpenCL/RigidBody/b3GpuNarrowPhase.h:9-99
 *   b3GpuBroadphaseInterface src/Bullet3OpenCL/BroadphaseCollision/b3GpuBroadphaseInterface.h:12-40
 *   b3GpuGridBroadphase      src/Bullet3OpenCL/BroadphaseCollision/b3GpuGridBroadphase.h
 *   b3GpuRigidBodyPipeline   src/Bullet3OpenCL/RigidBody/b3GpuRigidBodyPipeline.h:25-67
 *   b3Config                 src/Bullet3OpenCL/RigidBody/b3Config.h:4-37
 * The OpenCL handles of the reference constructors (cl_context, cl_device_id, cl_command_queue)
 * become a CUDA device ordinal; cl_mem results become device pointers (void*).  Indices the
 * reference reports as -1 + b3Error are reported the same way (message on stderr); CUDA failures
 * are reported through b3g_last_error().  Like the reference, the pipeline does not own the
 * narrowphase or broadphase objects.
 */
#ifndef B3G_COMPAT_H
#define B3G_COMPAT_H

#include <cstdio>
#include <vector>

#include "b3g_capi.h"
#include "b3g_types.h"

namespace b3g_compat {

inline void b3Error(const char* what) { std::fprintf(stderr, "b3Error: %s: %s\n", what, b3g_last_error()); }
inline void b3Warning(const char* what) { std::fprintf(stderr, "b3Warning: %s\n", what); }

struct b3Config {
    int m_maxConvexBodies = 128 * 1024;
    int m_maxConvexShapes = 8 * 1024;
    int m_maxBroadphasePairs = 0;
    int m_maxContactCapacity = 0;
    b3gConfig toC() const {
        b3gConfig c;
        b3g_config_default(&c);
        c.max_bodies = m_maxConvexBodies;
        c.max_shapes = m_maxConvexShapes;
        c.max_pairs = m_maxBroadphasePairs;
        c.max_contacts = m_maxContactCapacity;
        return c;
    }
};

class b3GpuNarrowPhase {
public:
    b3GpuNarrowPhase(int cudaDevice, const b3Config& config) : m_config(config) {
        b3gConfig c = config.toC();
        if (b3g_create(&c, cudaDevice, &m_world) != B3G_OK) {
            b3Error("b3GpuNarrowPhase");
            m_world = nullptr;
        }
    }
    virtual ~b3GpuNarrowPhase() {
        if (m_world) b3g_destroy(m_world);
    }
    int registerSphereShape(float radius) { return reg(b3g_register_sphere(m_world, radius, &m_out), "registerSphereShape"); }
    int registerPlaneShape(const float planeNormal[3], float planeConstant) {
        return reg(b3g_register_plane(m_world, planeNormal, planeConstant, &m_out), "registerPlaneShape");
    }
    int registerConvexHullShape(const float* vertices, int strideInBytes, int numVertices, const float* scaling) {
        return reg(b3g_register_hull(m_world, vertices, strideInBytes, numVertices, scaling, &m_out),
                   "registerConvexHullShape");
    }
    int registerCompoundShape(void*) {
        std::fprintf(stderr, "b3Error: registerCompoundShape: compound shapes are not supported\n");
        return -1;
    }
    int registerConcaveMesh(void*, void*, const float*) {
        std::fprintf(stderr, "b3Error: registerConcaveMesh: concave meshes are not supported\n");
        return -1;
    }
    /* b3GpuNarrowPhase::registerRigidBody (b3GpuNarrowPhase.cpp:816-908).  The AABB arguments are
       recomputed from the shape (the reference stores them for the proxy it creates). */
    int registerRigidBody(int collidableIndex, float mass, const float* position, const float* orientation,
                          const float* /*aabbMin*/, const float* /*aabbMax*/, bool /*writeToGpu*/) {
        return registerBody(mass, position, orientation, collidableIndex, -1);
    }
    int registerBody(float mass, const float* position, const float* orientation, int collidableIndex, int user) {
        int out = -1;
        if (b3g_register_body(m_world, mass, position, orientation, collidableIndex, user, &out) != B3G_OK) {
            b3Error("registerRigidBody");
            return -1;
        }
        if (mass == 0.f && m_static0 < 0) m_static0 = out;  // first static body (m_static0Index)
        return out;
    }
    /* The first call uploads every registry (b3g_write_all_to_gpu); later calls write the host
       copy of the bodies (after setObjectTransformCpu / setObjectVelocityCpu), as the reference's
       writeAllBodiesToGpu copies m_bodyBufferCPU (b3GpuNarrowPhase.cpp:915-944). */
    void writeAllBodiesToGpu() {
        if (!m_uploaded) {
            if (b3g_write_all_to_gpu(m_world) != B3G_OK) {
                b3Error("writeAllBodiesToGpu");
                return;
            }
            m_uploaded = true;
            return;
        }
        if (!m_bodiesCPU.empty() &&
            b3g_write_bodies(m_world, m_bodiesCPU.data(), (int)m_bodiesCPU.size()) != B3G_OK)
            b3Error("writeAllBodiesToGpu");
    }
    void readbackAllBodiesToCpu() { readbackAllBodiesToCpu(m_bodiesCPU); }
    /* host copy of a body's pose (b3GpuNarrowPhase::getObjectTransformFromCpu): valid after
       readbackAllBodiesToCpu() */
    bool getObjectTransformFromCpu(float* position, float* orientation, int bodyIndex) const {
        if (bodyIndex < 0 || bodyIndex >= (int)m_bodiesCPU.size()) {
            b3Warning("getObjectTransformFromCpu out of range.");
            return false;
        }
        const b3gBody& b = m_bodiesCPU[bodyIndex];
        position[0] = b.pos.x; position[1] = b.pos.y; position[2] = b.pos.z;
        orientation[0] = b.quat.x; orientation[1] = b.quat.y; orientation[2] = b.quat.z; orientation[3] = b.quat.w;
        return true;
    }
    void setObjectTransformCpu(const float* position, const float* orientation, int bodyIndex) {
        if (bodyIndex < 0 || bodyIndex >= (int)m_bodiesCPU.size()) {
            b3Warning("setObjectTransformCpu out of range.");  // b3GpuNarrowPhase.cpp:979
            return;
        }
        b3gBody& b = m_bodiesCPU[bodyIndex];
        b.pos.x = position[0]; b.pos.y = position[1]; b.pos.z = position[2];
        b.quat.x = orientation[0]; b.quat.y = orientation[1]; b.quat.z = orientation[2]; b.quat.w = orientation[3];
    }
    void setObjectVelocityCpu(const float* linVel, const float* angVel, int bodyIndex) {
        if (bodyIndex < 0 || bodyIndex >= (int)m_bodiesCPU.size()) {
            b3Warning("setObjectVelocityCpu out of range.");  // b3GpuNarrowPhase.cpp:991
            return;
        }
        b3gBody& b = m_bodiesCPU[bodyIndex];
        b.linVel.x = linVel[0]; b.linVel.y = linVel[1]; b.linVel.z = linVel[2];
        b.angVel.x = angVel[0]; b.angVel.y = angVel[1]; b.angVel.z = angVel[2];
    }
    int getNumBodiesGpu() const { return getNumRigidBodies(); }
    int getNumCollidablesGpu() const {
        int n = 0;
        b3g_get_num_collidables(m_world, &n);
        return n;
    }
    int getStatic0Index() const { return m_static0; }
    void getContactsCPU(std::vector<b3gContact4>& out) {
        int n = getNumContactsGpu();
        out.resize(n);
        if (n > 0 && b3g_read_contacts(m_world, out.data(), n, &n) != B3G_OK) b3Error("getContactsCPU");
        out.resize(n);
    }
    int getNumRigidBodies() const {
        int n = 0;
        b3g_get_num_bodies(m_world, &n);
        return n;
    }
    void readbackAllBodiesToCpu(std::vector<b3gBody>& out) {
        out.resize(getNumRigidBodies());
        if (b3g_read_bodies(m_world, out.data(), (int)out.size()) != B3G_OK) b3Error("readbackAllBodiesToCpu");
    }
    void computeContacts() {
        if (b3g_compute_contacts(m_world) != B3G_OK) b3Error("computeContacts");
    }
    /* computeContacts(pairs, numPairs, aabbs, numObjects) (b3GpuNarrowPhase.h:53): the world's own
       pair and AABB buffers are the ones the broadphase filled */
    void computeContacts(void* /*pairs*/, int /*numPairs*/, void* /*aabbsWorldSpace*/, int /*numObjects*/) {
        computeContacts();
    }
    void* getBodiesGpu() {
        void* p = nullptr;
        b3g_get_body_buffer(m_world, &p);
        return p;
    }
    void* getBodyInertiasGpu() {
        void* p = nullptr;
        b3g_get_inertia_buffer(m_world, &p);
        return p;
    }
    void* getContactsGpu() {
        void* p = nullptr;
        int n = 0;
        b3g_get_contact_buffer(m_world, &p, &n);
        return p;
    }
    int getNumContactsGpu() {
        void* p = nullptr;
        int n = 0;
        b3g_get_contact_buffer(m_world, &p, &n);
        return n;
    }
    b3g_handle world() const { return m_world; }

private:
    int reg(b3gStatus st, const char* what) {
        if (st == B3G_OK) return m_out;
        b3Error(what);
        return -1;
    }
    b3Config m_config;
    b3g_handle m_world = nullptr;
    int m_out = -1;
    int m_static0 = -1;
    bool m_uploaded = false;
    std::vector<b3gBody> m_bodiesCPU;
};

class b3GpuBroadphaseInterface {
public:
    /* b3GpuBroadphaseInterface::CreateFunc (b3GpuBroadphaseInterface.h:14): the OpenCL handles
       become a CUDA device ordinal */
    typedef b3GpuBroadphaseInterface*(CreateFunc)(int cudaDevice);
    virtual ~b3GpuBroadphaseInterface() {}
    virtual void calculateOverlappingPairs(int maxPairs) = 0;
    virtual int getNumOverlap() = 0;
    virtual void* getOverlappingPairBuffer() = 0;
    virtual void* getAabbBufferWS() = 0;
};

class b3GpuGridBroadphase : public b3GpuBroadphaseInterface {
public:
    explicit b3GpuGridBroadphase(b3GpuNarrowPhase* np = nullptr) : m_np(np) {}
    static b3GpuBroadphaseInterface* CreateFunc(int /*cudaDevice*/) { return new b3GpuGridBroadphase(); }
    virtual void attach(b3GpuNarrowPhase* np) { m_np = np; }
    /* Proxies: registerPhysicsInstance / registerRigidBody create them (dynamic bodies small,
       static bodies large), as the reference pipeline does (b3GpuRigidBodyPipeline.cpp:650-657) */
    void createProxy(const float*, const float*, int, int, int) {}
    void createLargeProxy(const float*, const float*, int, int, int) {}
    void calculateOverlappingPairs(int) override {
        if (b3g_calculate_overlapping_pairs(m_np->world()) != B3G_OK) b3Error("calculateOverlappingPairs");
    }
    /* calculateOverlappingPairsHost (b3GpuGridBroadphase.cpp:260-294) computes the exact pair set;
       the device search gives the same set */
    void calculateOverlappingPairsHost(int maxPairs) { calculateOverlappingPairs(maxPairs); }
    /* host copies of the world AABBs (getAllAabbsCPU) and their upload (writeAabbsToGpu) */
    std::vector<b3gAabb>& getAllAabbsCPU() {
        m_aabbsCPU.resize(m_np->getNumRigidBodies());
        if (!m_aabbsCPU.empty() && b3g_read_aabbs(m_np->world(), m_aabbsCPU.data(), (int)m_aabbsCPU.size()) != B3G_OK)
            b3Error("getAllAabbsCPU");
        return m_aabbsCPU;
    }
    void writeAabbsToGpu() {
        if (!m_aabbsCPU.empty() &&
            b3g_write_aabbs(m_np->world(), m_aabbsCPU.data(), (int)m_aabbsCPU.size()) != B3G_OK)
            b3Error("writeAabbsToGpu");
    }
    void* getAllAabbsGPU() { return getAabbBufferWS(); }
    void* getOverlappingPairsGPU() { return getOverlappingPairBuffer(); }
    int getNumOverlap() override {
        void* p = nullptr;
        int n = 0;
        b3g_get_pair_buffer(m_np->world(), &p, &n);
        return n;
    }
    void* getOverlappingPairBuffer() override {
        void* p = nullptr;
        int n = 0;
        b3g_get_pair_buffer(m_np->world(), &p, &n);
        return p;
    }
    void* getAabbBufferWS() override {
        void* p = nullptr;
        b3g_get_aabb_buffer(m_np->world(), &p);
        return p;
    }

private:
    b3GpuNarrowPhase* m_np;
    std::vector<b3gAabb> m_aabbsCPU;
};

/* b3GpuSapBroadphase (b3GpuSapBroadphase.cpp): the same exact pair set; here the grid search
   with the 1-axis sweep and prune for large static proxies serves both names. */
class b3GpuSapBroadphase : public b3GpuGridBroadphase {
public:
    explicit b3GpuSapBroadphase(b3GpuNarrowPhase* np = nullptr) : b3GpuGridBroadphase(np) {}
    static b3GpuBroadphaseInterface* CreateFunc(int /*cudaDevice*/) { return new b3GpuSapBroadphase(); }
};

/* b3GpuParallelLinearBvhBroadphase (Bullet3OpenCL/BroadphaseCollision/b3GpuParallelLinearBvhBroadphase.h):
   the linear-BVH pair search, complete for any AABB sizes; same pair list as the grid.  Attaching it
   to a pipeline switches the world's pair search to it. */
class b3GpuParallelLinearBvhBroadphase : public b3GpuGridBroadphase {
public:
    explicit b3GpuParallelLinearBvhBroadphase(b3GpuNarrowPhase* np = nullptr) : b3GpuGridBroadphase(np) {
        if (np) attach(np);
    }
    static b3GpuBroadphaseInterface* CreateFunc(int /*cudaDevice*/) { return new b3GpuParallelLinearBvhBroadphase(); }
    void attach(b3GpuNarrowPhase* np) override {
        b3GpuGridBroadphase::attach(np);
        if (np && b3g_set_broadphase(np->world(), B3G_BROADPHASE_LBVH) != B3G_OK) b3Error("b3GpuParallelLinearBvhBroadphase");
    }
};

class b3GpuRigidBodyPipeline {
public:
    b3GpuRigidBodyPipeline(b3GpuNarrowPhase* narrowphase, b3GpuGridBroadphase* broadphase, void* /*dbvt*/,
                           const b3Config& config)
        : m_np(narrowphase), m_bp(broadphase), m_config(config) {
        if (m_bp) m_bp->attach(narrowphase);
    }
    int registerPhysicsInstance(float mass, const float* position, const float* orientation, int collidableIndex,
                                int userData, bool /*writeInstanceToGpu*/) {
        return m_np->registerBody(mass, position, orientation, collidableIndex, userData);
    }
    void writeAllInstancesToGpu() { m_np->writeAllBodiesToGpu(); }
    /* independent scenes stepped together (no reference counterpart: the reference runs one
       pipeline per scene); call before writeAllInstancesToGpu */
    bool setSceneOffsets(const int* firstBody, int numScenes) {
        if (b3g_set_scene_offsets(m_np->world(), firstBody, numScenes) != B3G_OK) {
            b3Error("setSceneOffsets");
            return false;
        }
        return true;
    }
    void setGravity(const float* grav) { b3g_set_gravity(m_np->world(), grav); }
    void stepSimulation(float deltaTime) {
        if (b3g_step(m_np->world(), deltaTime) != B3G_OK) b3Error("stepSimulation");
    }
    void setupGpuAabbsFull() { b3g_setup_aabbs(m_np->world()); }
    void integrate(float timeStep) { b3g_integrate(m_np->world(), timeStep); }
    int getNumBodies() const { return m_np->getNumRigidBodies(); }
    void* getBodyBuffer() { return m_np->getBodiesGpu(); }
    void reset() { b3Error("reset: re-create the pipeline (registries are fixed once uploaded)"); }
    /* joints (b3GpuRigidBodyPipeline.h:52-58): solved every step right before the contacts.  The
       host copy (b3gJoint == b3GpuGenericConstraint) carries the enabled flags as the device's break
       check left them after copyConstraintsToHost(). */
    void copyConstraintsToHost() {
        int n = 0;
        b3g_get_num_constraints(m_np->world(), &n);
        m_constraints.resize((size_t)n);
        if (n > 0 && b3g_read_constraints(m_np->world(), m_constraints.data(), n, &n) != B3G_OK)
            b3Error("copyConstraintsToHost");
    }
    const std::vector<b3gJoint>& getConstraintsCPU() const { return m_constraints; }
    void removeConstraintByUid(int uid) {
        if (b3g_remove_constraint(m_np->world(), uid) != B3G_OK) b3Error("removeConstraintByUid");
    }
    int createPoint2PointConstraint(int bodyA, int bodyB, const float* pivotInA, const float* pivotInB,
                                    float breakingThreshold) {
        int uid = -1;
        if (b3g_create_point2point_constraint(m_np->world(), bodyA, bodyB, pivotInA, pivotInB, breakingThreshold,
                                              &uid) != B3G_OK) {
            b3Error("createPoint2PointConstraint");
            return -1;
        }
        return uid;
    }
    int createFixedConstraint(int bodyA, int bodyB, const float* pivotInA, const float* pivotInB,
                              const float* relTargetAB, float breakingThreshold) {
        int uid = -1;
        if (b3g_create_fixed_constraint(m_np->world(), bodyA, bodyB, pivotInA, pivotInB, relTargetAB,
                                        breakingThreshold, &uid) != B3G_OK) {
            b3Error("createFixedConstraint");
            return -1;
        }
        return uid;
    }
    /* castRays(rays, hitResults) (b3GpuRigidBodyPipeline.h:63): arrays of b3RayInfo / b3RayHit (or
       b3gRayInfo / b3gRayHit, the same layouts) of equal size; hitResults[i].m_hitResult2 names a
       body the ray ignores */
    template <class Rays, class Hits>
    void castRays(const Rays& rays, Hits& hitResults) {
        const int n = (int)rays.size();
        if ((int)hitResults.size() != n) {
            b3Warning("castRays: hitResults must have one entry per ray");
            return;
        }
        if (n > 0 && b3g_cast_rays(m_np->world(), &rays[0], &hitResults[0], n) != B3G_OK) b3Error("castRays");
    }

private:
    b3GpuNarrowPhase* m_np;
    b3GpuGridBroadphase* m_bp;
    b3Config m_config;
    std::vector<b3gJoint> m_constraints;
};

}  // namespace b3g_compat

#endif
