/*
 * b3g_compat.h -- header-only C++ drop-in for the reference's GPU rigid-body API, implemented on
 * the C ABI of libb3gpu.so (include/b3g_capi.h).  No CUDA or OpenCL header is needed to build
 * against it: link with -lb3gpu.
 *
 * Class names, constructors, method signatures, argument meaning and error behaviour follow
 *   b3GpuNarrowPhase          src/Bullet3OpenCL/RigidBody/b3GpuNarrowPhase.h:9-99
 *   b3GpuBroadphaseInterface  src/Bullet3OpenCL/BroadphaseCollision/b3GpuBroadphaseInterface.h:12-40
 *   b3GpuGridBroadphase       src/Bullet3OpenCL/BroadphaseCollision/b3GpuGridBroadphase.h
 *   b3GpuSapBroadphase        src/Bullet3OpenCL/BroadphaseCollision/b3GpuSapBroadphase.h:85-117
 *   b3GpuParallelLinearBvhBroadphase
 *                             src/Bullet3OpenCL/BroadphaseCollision/b3GpuParallelLinearBvhBroadphase.h
 *   b3GpuRigidBodyPipeline    src/Bullet3OpenCL/RigidBody/b3GpuRigidBodyPipeline.h:25-67
 *   b3OpenCLArray<T>          src/Bullet3OpenCL/ParallelPrimitives/b3OpenCLArray.h:39-300
 * and the value types of include/b3g_compat_types.h (b3Vector3, b3AlignedObjectArray,
 * b3ConvexUtility, b3Config, ...).
 *
 * The OpenCL handles keep their names: cl_context, cl_device_id and cl_command_queue are opaque
 * handles naming a CUDA device, made by b3gCreateContext / b3gGetDevice / b3gCreateCommandQueue
 * (in place of b3OpenCLUtils::createContextFromType, getDevice and clCreateCommandQueue), and
 * cl_mem is a device pointer.  So a program written against the reference compiles after its
 * includes and its context creation change.  Indices the reference reports as -1 + b3Error are
 * reported the same way (message on stderr); CUDA failures through b3g_last_error().  Like the
 * reference, the pipeline owns neither the narrowphase nor the broadphase.
 */
#ifndef B3G_COMPAT_H
#define B3G_COMPAT_H

#include <cstdio>
#include <cstring>
#include <vector>

#include "b3g_capi.h"
#include "b3g_compat_types.h"
#include "b3g_types.h"

/* ---------------------------------------------------------------- device and buffer handles */
#ifndef __OPENCL_CL_H
struct _cl_context {
    int cudaDevice;
};
struct _cl_device_id {
    int cudaDevice;
};
struct _cl_command_queue {
    int cudaDevice;
};
typedef struct _cl_context* cl_context;
typedef struct _cl_device_id* cl_device_id;
typedef struct _cl_command_queue* cl_command_queue;
typedef void* cl_mem;
#endif

/* b3OpenCLUtils::createContextFromType / getDevice and clCreateCommandQueue, for CUDA devices;
 * release with b3gRelease. */
inline cl_context b3gCreateContext(int cudaDevice = 0) { return new _cl_context{cudaDevice}; }
inline cl_device_id b3gGetDevice(cl_context ctx, int /*deviceIndex*/ = 0) {
    return new _cl_device_id{ctx ? ctx->cudaDevice : 0};
}
inline cl_command_queue b3gCreateCommandQueue(cl_context ctx, cl_device_id device) {
    return new _cl_command_queue{device ? device->cudaDevice : ctx ? ctx->cudaDevice : 0};
}
inline void b3gRelease(cl_context p) { delete p; }
inline void b3gRelease(cl_device_id p) { delete p; }
inline void b3gRelease(cl_command_queue p) { delete p; }
inline int b3gDeviceOf(cl_context ctx, cl_device_id dev, cl_command_queue q) {
    return dev ? dev->cudaDevice : q ? q->cudaDevice : ctx ? ctx->cudaDevice : 0;
}

inline void b3Error(const char* what) { std::fprintf(stderr, "b3Error: %s: %s\n", what, b3g_last_error()); }
inline void b3Warning(const char* what) { std::fprintf(stderr, "b3Warning: %s\n", what); }

/* ---------------------------------------------------------------- b3OpenCLArray */
/* A device array of T on one CUDA device: owned (grown by reserve / resize / push_back, copying
 * the old contents) or a view of a buffer it does not own (setFromOpenCLBuffer).  Copies are
 * synchronous, as the reference's are with waitForCompletion = true. */
template <typename T>
class b3OpenCLArray {
public:
    b3OpenCLArray(cl_context ctx, cl_command_queue queue, size_t initialCapacity = 0, bool allowGrowingCapacity = true)
        : m_device(b3gDeviceOf(ctx, nullptr, queue)), m_allowGrowingCapacity(true) {
        if (initialCapacity) reserve(initialCapacity);
        m_allowGrowingCapacity = allowGrowingCapacity;
    }
    virtual ~b3OpenCLArray() { deallocate(); }
    b3OpenCLArray(const b3OpenCLArray&) = delete;
    b3OpenCLArray& operator=(const b3OpenCLArray&) = delete;

    void setFromOpenCLBuffer(cl_mem buffer, size_t sizeInElements) {
        deallocate();
        m_ownsMemory = false;
        m_allowGrowingCapacity = false;
        m_buf = static_cast<T*>(buffer);
        m_size = m_capacity = sizeInElements;
    }
    cl_mem getBufferCL() const { return m_buf; }
    bool push_back(const T& v, bool /*waitForCompletion*/ = true) {
        const size_t n = m_size;
        if (!resize(n + 1)) return false;
        copyFromHostPointer(&v, 1, n);
        return true;
    }
    T forcedAt(size_t n) const {
        T v;
        b3g_buffer_copy(m_device, &v, m_buf + n, sizeof(T), B3G_COPY_D2H);
        return v;
    }
    T at(size_t n) const {
        if (n >= m_size) {
            b3Warning("b3OpenCLArray::at out of range");
            return T();
        }
        return forcedAt(n);
    }
    bool resize(size_t newsize, bool copyOldContents = true) {
        if (newsize > m_capacity && !reserve(newsize, copyOldContents)) return false;
        m_size = newsize;
        return true;
    }
    size_t size() const { return m_size; }
    size_t capacity() const { return m_capacity; }
    bool reserve(size_t count, bool copyOldContents = true) {
        if (count <= m_capacity) return true;
        if (!m_allowGrowingCapacity) {
            b3Warning("b3OpenCLArray: exceeding the preallocated capacity that may not grow");
            return false;
        }
        void* p = nullptr;
        if (b3g_buffer_alloc(m_device, sizeof(T) * count, &p) != B3G_OK) {
            b3Error("b3OpenCLArray::reserve");
            return false;
        }
        if (copyOldContents && m_size)
            b3g_buffer_copy(m_device, p, m_buf, sizeof(T) * m_size, B3G_COPY_D2D);
        deallocate();
        m_buf = static_cast<T*>(p);
        m_ownsMemory = true;
        m_capacity = count;
        return true;
    }
    void copyToCL(cl_mem destination, size_t numElements, size_t firstElem = 0, size_t dstOffsetInElems = 0) const {
        if (numElements == 0) return;
        if (firstElem + numElements > m_size) {
            b3Warning("b3OpenCLArray::copyToCL out of range");
            return;
        }
        b3g_buffer_copy(m_device, static_cast<T*>(destination) + dstOffsetInElems, m_buf + firstElem,
                        sizeof(T) * numElements, B3G_COPY_D2D);
    }
    void copyFromHost(const b3AlignedObjectArray<T>& src, bool waitForCompletion = true) {
        const size_t n = (size_t)src.size();
        resize(n);
        if (n) copyFromHostPointer(&src[0], n, 0, waitForCompletion);
    }
    void copyFromHostPointer(const T* src, size_t numElems, size_t destFirstElem = 0, bool /*wait*/ = true) {
        if (numElems == 0) return;
        if (destFirstElem + numElems > m_capacity) {
            b3Warning("b3OpenCLArray::copyFromHostPointer out of range");
            return;
        }
        b3g_buffer_copy(m_device, m_buf + destFirstElem, src, sizeof(T) * numElems, B3G_COPY_H2D);
    }
    void copyToHost(b3AlignedObjectArray<T>& dst, bool waitForCompletion = true) const {
        dst.resize((int)m_size);
        if (m_size) copyToHostPointer(&dst[0], m_size, 0, waitForCompletion);
    }
    void copyToHostPointer(T* dst, size_t numElem, size_t srcFirstElem = 0, bool /*wait*/ = true) const {
        if (numElem == 0) return;
        if (srcFirstElem + numElem > m_capacity) {
            b3Warning("b3OpenCLArray::copyToHostPointer out of range");
            return;
        }
        b3g_buffer_copy(m_device, dst, m_buf + srcFirstElem, sizeof(T) * numElem, B3G_COPY_D2H);
    }
    void copyFromOpenCLArray(const b3OpenCLArray& src) {
        const size_t n = src.size();
        resize(n);
        if (n) src.copyToCL(m_buf, n);
    }

private:
    void deallocate() {
        if (m_buf && m_ownsMemory) b3g_buffer_free(m_device, m_buf);
        m_buf = nullptr;
        m_size = m_capacity = 0;
    }
    T* m_buf = nullptr;
    size_t m_size = 0, m_capacity = 0;
    int m_device;
    bool m_ownsMemory = true;
    bool m_allowGrowingCapacity;
};

/* ---------------------------------------------------------------- b3GpuNarrowPhase */
inline b3gConfig b3gConfigFrom(const b3Config& c) {
    b3gConfig out;
    b3g_config_default(&out);
    out.max_bodies = c.m_maxConvexBodies;
    out.max_shapes = c.m_maxConvexShapes;
    out.max_pairs = c.m_maxBroadphasePairs;
    out.max_contacts = c.m_maxContactCapacity;
    out.max_compound_child_pairs = c.m_compoundPairCapacity;
    out.max_concave_pairs = c.m_maxTriConvexPairCapacity;
    return out;
}

class b3GpuNarrowPhase {
public:
    b3GpuNarrowPhase(cl_context ctx, cl_device_id dev, cl_command_queue q, const b3Config& config)
        : m_device(b3gDeviceOf(ctx, dev, q)), m_config(config) {
        b3gConfig c = b3gConfigFrom(config);
        if (b3g_create(&c, m_device, &m_world) != B3G_OK) {
            b3Error("b3GpuNarrowPhase");
            m_world = nullptr;
        }
    }
    virtual ~b3GpuNarrowPhase() {
        if (m_world) b3g_destroy(m_world);
    }

    int registerSphereShape(float radius) { return reg(b3g_register_sphere(m_world, radius, &m_out), "registerSphereShape"); }
    int registerPlaneShape(const b3Vector3& planeNormal, float planeConstant) {
        const float n[3] = {planeNormal.getX(), planeNormal.getY(), planeNormal.getZ()};
        return reg(b3g_register_plane(m_world, n, planeConstant, &m_out), "registerPlaneShape");
    }
    /* registerCompoundShape (b3GpuNarrowPhase.cpp:370-433): children are convex hull collidables at
       poses in the compound's frame; the compound's local AABB is the union of theirs */
    int registerCompoundShape(b3AlignedObjectArray<b3GpuChildShape>* childShapes) {
        if (!childShapes || childShapes->size() == 0) {
            std::fprintf(stderr, "b3Error: registerCompoundShape: no child shapes\n");
            return -1;
        }
        return reg(b3g_register_compound(m_world, reinterpret_cast<const b3gChildShape*>(&childShapes->at(0)),
                                         childShapes->size(), &m_out),
                   "registerCompoundShape");
    }
    /* registerConcaveMesh (b3GpuNarrowPhase.cpp:521-613): a static triangle mesh (3 indices per
       triangle) with a quantized triangle BVH; meant to stay at the identity pose, as in the reference */
    int registerConcaveMesh(b3AlignedObjectArray<b3Vector3>* vertices, b3AlignedObjectArray<int>* indices,
                            const float* scaling) {
        if (!vertices || !indices || vertices->size() == 0 || indices->size() < 3) {
            std::fprintf(stderr, "b3Error: registerConcaveMesh: no vertices or triangles\n");
            return -1;
        }
        const float one[3] = {1.f, 1.f, 1.f};
        return reg(b3g_register_concave_mesh(m_world, vertices->at(0).m_floats, (int)sizeof(b3Vector3), vertices->size(),
                                             &indices->at(0), indices->size() / 3, scaling ? scaling : one, &m_out),
                   "registerConcaveMesh");
    }
    /* registerConvexHullShape(b3ConvexUtility*) (b3GpuNarrowPhase.cpp:322-368): the utility's tables
       as they are, with the vertex mean as local centre */
    int registerConvexHullShape(b3ConvexUtility* utilPtr) {
        if (!utilPtr || utilPtr->m_vertices.size() == 0 || utilPtr->m_faces.size() == 0) {
            std::fprintf(stderr, "b3Error: registerConvexHullShape: empty convex utility\n");
            return -1;
        }
        std::vector<float> v, planes, edges;
        std::vector<int> counts, indices;
        for (int i = 0; i < utilPtr->m_vertices.size(); i++)
            for (int k = 0; k < 3; k++) v.push_back(utilPtr->m_vertices[i][k]);
        for (int f = 0; f < utilPtr->m_faces.size(); f++) {
            const b3MyFace& face = utilPtr->m_faces[f];
            for (int k = 0; k < 4; k++) planes.push_back(face.m_plane[k]);
            counts.push_back(face.m_indices.size());
            for (int k = 0; k < face.m_indices.size(); k++) indices.push_back(face.m_indices[k]);
        }
        for (int i = 0; i < utilPtr->m_uniqueEdges.size(); i++)
            for (int k = 0; k < 3; k++) edges.push_back(utilPtr->m_uniqueEdges[i][k]);
        return reg(b3g_register_hull_tables(m_world, v.data(), utilPtr->m_vertices.size(), planes.data(), counts.data(),
                                            (int)counts.size(), indices.data(), edges.empty() ? nullptr : edges.data(),
                                            utilPtr->m_uniqueEdges.size(), &m_out),
                   "registerConvexHullShape");
    }
    int registerConvexHullShape(const float* vertices, int strideInBytes, int numVertices, const float* scaling) {
        return reg(b3g_register_hull(m_world, vertices, strideInBytes, numVertices, scaling, &m_out),
                   "registerConvexHullShape");
    }
    /* registerRigidBody (b3GpuNarrowPhase.cpp:816-908).  The AABB arguments are recomputed from the
       shape, as registerPhysicsInstance computes them (margin 0.01). */
    int registerRigidBody(int collidableIndex, float mass, const float* position, const float* orientation,
                          const float* /*aabbMin*/, const float* /*aabbMax*/, bool /*writeToGpu*/) {
        return registerBody(mass, position, orientation, collidableIndex, -1);
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
        if (m_bodiesCPU.size() && b3g_write_bodies(m_world, &m_bodiesCPU[0], m_bodiesCPU.size()) != B3G_OK)
            b3Error("writeAllBodiesToGpu");
    }
    /* b3GpuNarrowPhase::reset (b3GpuNarrowPhase.cpp:946-962): every shape and body is dropped */
    void reset() {
        if (b3g_reset(m_world, B3G_RESET_SHAPES_AND_BODIES) != B3G_OK) b3Error("reset");
        m_static0 = -1;
        m_uploaded = false;
        m_bodiesCPU.clear();
    }
    void readbackAllBodiesToCpu() {
        m_bodiesCPU.resize(getNumRigidBodies());
        if (m_bodiesCPU.size() && b3g_read_bodies(m_world, &m_bodiesCPU[0], m_bodiesCPU.size()) != B3G_OK)
            b3Error("readbackAllBodiesToCpu");
    }
    /* pose from the host copy (valid after readbackAllBodiesToCpu) */
    bool getObjectTransformFromCpu(float* position, float* orientation, int bodyIndex) const {
        if (bodyIndex < 0 || bodyIndex >= m_bodiesCPU.size()) {
            b3Warning("getObjectTransformFromCpu out of range.");
            return false;
        }
        const b3RigidBodyData& b = m_bodiesCPU[bodyIndex];
        for (int k = 0; k < 3; k++) position[k] = b.m_pos[k];
        for (int k = 0; k < 4; k++) orientation[k] = b.m_quat[k];
        return true;
    }
    void setObjectTransformCpu(float* position, float* orientation, int bodyIndex) {
        if (bodyIndex < 0 || bodyIndex >= m_bodiesCPU.size()) {
            b3Warning("setObjectTransformCpu out of range.");  // b3GpuNarrowPhase.cpp:979
            return;
        }
        b3RigidBodyData& b = m_bodiesCPU[bodyIndex];
        for (int k = 0; k < 3; k++) b.m_pos[k] = position[k];
        for (int k = 0; k < 4; k++) b.m_quat[k] = orientation[k];
    }
    void setObjectVelocityCpu(float* linVel, float* angVel, int bodyIndex) {
        if (bodyIndex < 0 || bodyIndex >= m_bodiesCPU.size()) {
            b3Warning("setObjectVelocityCpu out of range.");  // b3GpuNarrowPhase.cpp:991
            return;
        }
        b3RigidBodyData& b = m_bodiesCPU[bodyIndex];
        for (int k = 0; k < 3; k++) {
            b.m_linVel[k] = linVel[k];
            b.m_angVel[k] = angVel[k];
        }
    }
    /* setObjectTransform (b3GpuNarrowPhase.cpp:999-1016): one body's pose written to the device */
    void setObjectTransform(const float* position, const float* orientation, int bodyIndex) {
        readbackAllBodiesToCpu();
        if (bodyIndex < 0 || bodyIndex >= m_bodiesCPU.size()) {
            b3Warning("setObjectTransform out of range.");  // b3GpuNarrowPhase.cpp:1011
            return;
        }
        setObjectTransformCpu(const_cast<float*>(position), const_cast<float*>(orientation), bodyIndex);
        writeAllBodiesToGpu();
    }
    /* computeContacts(pairs, numPairs, aabbsWorldSpace, numObjects) (b3GpuNarrowPhase.cpp:751-809):
       the manifolds of the given pairs (b3Int4 device buffer); the AABBs are not needed for
       convex shapes */
    virtual void computeContacts(cl_mem broadphasePairs, int numBroadphasePairs, cl_mem /*aabbsWorldSpace*/,
                                 int /*numObjects*/) {
        void* own = nullptr;
        int n = 0;
        b3g_get_pair_buffer(m_world, &own, &n);
        const b3gStatus st = (broadphasePairs == own && numBroadphasePairs == n)
                                 ? b3g_compute_contacts(m_world)
                                 : b3g_compute_contacts_for_pairs(m_world, broadphasePairs, numBroadphasePairs);
        if (st != B3G_OK) b3Error("computeContacts");
    }
    cl_mem getBodiesGpu() {
        void* p = nullptr;
        b3g_get_body_buffer(m_world, &p);
        return p;
    }
    /* host copy of the bodies (valid after readbackAllBodiesToCpu) */
    const b3RigidBodyData* getBodiesCpu() const { return m_bodiesCPU.size() ? &m_bodiesCPU[0] : nullptr; }
    int getNumBodiesGpu() const { return getNumRigidBodies(); }
    cl_mem getBodyInertiasGpu() {
        void* p = nullptr;
        b3g_get_inertia_buffer(m_world, &p);
        return p;
    }
    int getNumBodyInertiasGpu() const { return getNumRigidBodies(); }
    int getNumCollidablesGpu() const {
        int n = 0;
        b3g_get_num_collidables(m_world, &n);
        return n;
    }
    /* host copy of the collidables and their local AABBs (read on each call) */
    const b3Collidable* getCollidablesCpu() const {
        readShapeTables();
        return m_collidables.size() ? &m_collidables[0] : nullptr;
    }
    const b3Collidable& getCollidableCpu(int collidableIndex) const {
        readShapeTables();
        return m_collidables[collidableIndex];
    }
    const b3SapAabb* getLocalSpaceAabbsCpu() const {
        readShapeTables();
        return m_localAabbs.size() ? &m_localAabbs[0] : nullptr;
    }
    const b3SapAabb& getLocalSpaceAabb(int collidableIndex) const {
        readShapeTables();
        return m_localAabbs[collidableIndex];
    }
    /* host copy of the last computeContacts' manifolds (read on each call) */
    const b3Contact4* getContactsCPU() const {
        int n = getNumContactsGpu();
        m_contactsCPU.resize(n);
        if (n > 0 && b3g_read_contacts(m_world, &m_contactsCPU[0], n, &n) != B3G_OK) b3Error("getContactsCPU");
        return n ? &m_contactsCPU[0] : nullptr;
    }
    cl_mem getContactsGpu() {
        void* p = nullptr;
        int n = 0;
        b3g_get_contact_buffer(m_world, &p, &n);
        return p;
    }
    int getNumContactsGpu() const {
        void* p = nullptr;
        int n = 0;
        b3g_get_contact_buffer(m_world, &p, &n);
        return n;
    }
    int getNumRigidBodies() const {
        int n = 0;
        b3g_get_num_bodies(m_world, &n);
        return n;
    }
    int getStatic0Index() const { return m_static0; }

    /* not in the reference: the world behind the classes, for the other classes of this header */
    b3g_handle world() const { return m_world; }
    int cudaDevice() const { return m_device; }
    int registerBody(float mass, const float* position, const float* orientation, int collidableIndex, int user) {
        int out = -1;
        if (b3g_register_body(m_world, mass, position, orientation, collidableIndex, user, &out) != B3G_OK) {
            b3Error("registerRigidBody");
            return -1;
        }
        if (mass == 0.f && m_static0 < 0) m_static0 = out;  // first static body (m_static0Index)
        return out;
    }

private:
    int reg(b3gStatus st, const char* what) {
        if (st == B3G_OK) return m_out;
        b3Error(what);
        return -1;
    }
    void readShapeTables() const {
        int counts[6] = {0, 0, 0, 0, 0, 0};
        b3g_read_shape_tables(m_world, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, counts);
        m_collidables.resize(counts[0]);
        m_localAabbs.resize(counts[0]);
        if (counts[0] == 0) return;
        const int caps[6] = {counts[0], 0, 0, 0, 0, 0};
        b3g_read_shape_tables(m_world, &m_collidables[0], nullptr, nullptr, nullptr, nullptr, nullptr, &m_localAabbs[0],
                              const_cast<int*>(caps));
    }
    int m_device;
    b3Config m_config;
    b3g_handle m_world = nullptr;
    int m_out = -1;
    int m_static0 = -1;
    bool m_uploaded = false;
    b3AlignedObjectArray<b3RigidBodyData> m_bodiesCPU;
    mutable b3AlignedObjectArray<b3Contact4> m_contactsCPU;
    mutable b3AlignedObjectArray<b3Collidable> m_collidables;
    mutable b3AlignedObjectArray<b3SapAabb> m_localAabbs;
};

/* ---------------------------------------------------------------- broadphases */
class b3GpuBroadphaseInterface {
public:
    typedef b3GpuBroadphaseInterface*(CreateFunc)(cl_context ctx, cl_device_id device, cl_command_queue q);
    virtual ~b3GpuBroadphaseInterface() {}
    virtual void createProxy(const b3Vector3& aabbMin, const b3Vector3& aabbMax, int userPtr, int collisionFilterGroup,
                             int collisionFilterMask) = 0;
    virtual void createLargeProxy(const b3Vector3& aabbMin, const b3Vector3& aabbMax, int userPtr,
                                  int collisionFilterGroup, int collisionFilterMask) = 0;
    virtual void calculateOverlappingPairs(int maxPairs) = 0;
    virtual void calculateOverlappingPairsHost(int maxPairs) = 0;
    virtual void writeAabbsToGpu() = 0;
    virtual cl_mem getAabbBufferWS() = 0;
    virtual int getNumOverlap() = 0;
    virtual cl_mem getOverlappingPairBuffer() = 0;
    virtual b3OpenCLArray<b3SapAabb>& getAllAabbsGPU() = 0;
    virtual b3AlignedObjectArray<b3SapAabb>& getAllAabbsCPU() = 0;
    virtual b3OpenCLArray<b3Int4>& getOverlappingPairsGPU() = 0;
    virtual b3OpenCLArray<int>& getSmallAabbIndicesGPU() = 0;
    virtual b3OpenCLArray<int>& getLargeAabbIndicesGPU() = 0;
    /* not in the reference: the pipeline's constructor binds the broadphase to the narrowphase's
       world (the reference's broadphase owns its AABB buffers; here the world does) */
    virtual void attach(b3GpuNarrowPhase* np) = 0;
};

/* The grid pair search of the world (b3GpuGridBroadphase); its pair set is the exact one. */
class b3GpuGridBroadphase : public b3GpuBroadphaseInterface {
public:
    b3GpuGridBroadphase(cl_context ctx, cl_device_id device, cl_command_queue q)
        : m_aabbsGPU(ctx, q), m_pairsGPU(ctx, q), m_small(ctx, q), m_large(ctx, q) {
        (void)device;
    }
    static b3GpuBroadphaseInterface* CreateFunc(cl_context ctx, cl_device_id device, cl_command_queue q) {
        return new b3GpuGridBroadphase(ctx, device, q);
    }
    void attach(b3GpuNarrowPhase* np) override { m_np = np; }
    /* proxies: registerPhysicsInstance creates them (dynamic bodies small, static bodies large), as
       the reference pipeline does (b3GpuRigidBodyPipeline.cpp:650-657) */
    void createProxy(const b3Vector3&, const b3Vector3&, int, int, int) override {}
    void createLargeProxy(const b3Vector3&, const b3Vector3&, int, int, int) override {}
    void calculateOverlappingPairs(int /*maxPairs*/) override {
        if (!bound("calculateOverlappingPairs")) return;
        if (b3g_calculate_overlapping_pairs(m_np->world()) != B3G_OK) b3Error("calculateOverlappingPairs");
    }
    /* calculateOverlappingPairsHost (b3GpuGridBroadphase.cpp:260-294) computes the exact pair set;
       the device search gives the same set */
    void calculateOverlappingPairsHost(int maxPairs) override { calculateOverlappingPairs(maxPairs); }
    void writeAabbsToGpu() override {
        if (!bound("writeAabbsToGpu") || m_aabbsCPU.size() == 0) return;
        if (b3g_write_aabbs(m_np->world(), &m_aabbsCPU[0], m_aabbsCPU.size()) != B3G_OK) b3Error("writeAabbsToGpu");
    }
    cl_mem getAabbBufferWS() override {
        void* p = nullptr;
        if (bound("getAabbBufferWS")) b3g_get_aabb_buffer(m_np->world(), &p);
        return p;
    }
    int getNumOverlap() override {
        void* p = nullptr;
        int n = 0;
        if (bound("getNumOverlap")) b3g_get_pair_buffer(m_np->world(), &p, &n);
        return n;
    }
    cl_mem getOverlappingPairBuffer() override {
        void* p = nullptr;
        int n = 0;
        if (bound("getOverlappingPairBuffer")) b3g_get_pair_buffer(m_np->world(), &p, &n);
        return p;
    }
    /* the world AABBs: a device view, and a host copy read on each call */
    b3OpenCLArray<b3SapAabb>& getAllAabbsGPU() override {
        m_aabbsGPU.setFromOpenCLBuffer(getAabbBufferWS(), m_np ? m_np->getNumRigidBodies() : 0);
        return m_aabbsGPU;
    }
    b3AlignedObjectArray<b3SapAabb>& getAllAabbsCPU() override {
        m_aabbsCPU.resize(m_np ? m_np->getNumRigidBodies() : 0);
        if (m_aabbsCPU.size() && b3g_read_aabbs(m_np->world(), &m_aabbsCPU[0], m_aabbsCPU.size()) != B3G_OK)
            b3Error("getAllAabbsCPU");
        return m_aabbsCPU;
    }
    b3OpenCLArray<b3Int4>& getOverlappingPairsGPU() override {
        m_pairsGPU.setFromOpenCLBuffer(getOverlappingPairBuffer(), getNumOverlap());
        return m_pairsGPU;
    }
    /* dynamic (small) and static (large) proxies: the bodies with inverse mass != 0 and == 0 */
    b3OpenCLArray<int>& getSmallAabbIndicesGPU() override {
        proxyLists();
        return m_small;
    }
    b3OpenCLArray<int>& getLargeAabbIndicesGPU() override {
        proxyLists();
        return m_large;
    }

protected:
    bool bound(const char* what) const {
        if (m_np) return true;
        std::fprintf(stderr, "b3Error: %s: the broadphase is not attached to a pipeline\n", what);
        return false;
    }
    void proxyLists() {
        b3AlignedObjectArray<b3SapAabb>& a = getAllAabbsCPU();
        b3AlignedObjectArray<int> small, large;
        for (int i = 0; i < a.size(); i++) (a[i].m_signedMaxIndices[3] ? small : large).push_back(i);
        m_small.copyFromHost(small);
        m_large.copyFromHost(large);
    }
    b3GpuNarrowPhase* m_np = nullptr;
    b3AlignedObjectArray<b3SapAabb> m_aabbsCPU;
    b3OpenCLArray<b3SapAabb> m_aabbsGPU;
    b3OpenCLArray<b3Int4> m_pairsGPU;
    b3OpenCLArray<int> m_small, m_large;
};

/* b3GpuSapBroadphase (b3GpuSapBroadphase.h:85-117): the same exact pair set; the world's grid search
   with its 1-axis sweep and prune for large static proxies serves every kernel type. */
class b3GpuSapBroadphase : public b3GpuGridBroadphase {
public:
    enum b3GpuSapKernelType {
        B3_GPU_SAP_KERNEL_BRUTE_FORCE_CPU = 1,
        B3_GPU_SAP_KERNEL_BRUTE_FORCE_GPU,
        B3_GPU_SAP_KERNEL_ORIGINAL,
        B3_GPU_SAP_KERNEL_BARRIER,
        B3_GPU_SAP_KERNEL_LOCAL_SHARED_MEMORY
    };
    b3GpuSapBroadphase(cl_context ctx, cl_device_id device, cl_command_queue q,
                       b3GpuSapKernelType kernelType = B3_GPU_SAP_KERNEL_LOCAL_SHARED_MEMORY)
        : b3GpuGridBroadphase(ctx, device, q), m_kernelType(kernelType) {}
    static b3GpuBroadphaseInterface* CreateFuncBruteForceCpu(cl_context c, cl_device_id d, cl_command_queue q) {
        return new b3GpuSapBroadphase(c, d, q, B3_GPU_SAP_KERNEL_BRUTE_FORCE_CPU);
    }
    static b3GpuBroadphaseInterface* CreateFuncBruteForceGpu(cl_context c, cl_device_id d, cl_command_queue q) {
        return new b3GpuSapBroadphase(c, d, q, B3_GPU_SAP_KERNEL_BRUTE_FORCE_GPU);
    }
    static b3GpuBroadphaseInterface* CreateFuncOriginal(cl_context c, cl_device_id d, cl_command_queue q) {
        return new b3GpuSapBroadphase(c, d, q, B3_GPU_SAP_KERNEL_ORIGINAL);
    }
    static b3GpuBroadphaseInterface* CreateFuncBarrier(cl_context c, cl_device_id d, cl_command_queue q) {
        return new b3GpuSapBroadphase(c, d, q, B3_GPU_SAP_KERNEL_BARRIER);
    }
    static b3GpuBroadphaseInterface* CreateFuncLocalMemory(cl_context c, cl_device_id d, cl_command_queue q) {
        return new b3GpuSapBroadphase(c, d, q, B3_GPU_SAP_KERNEL_LOCAL_SHARED_MEMORY);
    }
    b3GpuSapKernelType kernelType() const { return m_kernelType; }

private:
    b3GpuSapKernelType m_kernelType;
};

/* b3GpuParallelLinearBvhBroadphase: the linear-BVH pair search, complete for any AABB sizes; same
   pair list as the grid.  Attaching it to a pipeline switches the world's pair search to it. */
class b3GpuParallelLinearBvhBroadphase : public b3GpuGridBroadphase {
public:
    b3GpuParallelLinearBvhBroadphase(cl_context ctx, cl_device_id device, cl_command_queue q)
        : b3GpuGridBroadphase(ctx, device, q) {}
    static b3GpuBroadphaseInterface* CreateFunc(cl_context ctx, cl_device_id device, cl_command_queue q) {
        return new b3GpuParallelLinearBvhBroadphase(ctx, device, q);
    }
    void attach(b3GpuNarrowPhase* np) override {
        b3GpuGridBroadphase::attach(np);
        if (np && b3g_set_broadphase(np->world(), B3G_BROADPHASE_LBVH) != B3G_OK)
            b3Error("b3GpuParallelLinearBvhBroadphase");
    }
};

/* ---------------------------------------------------------------- b3GpuRigidBodyPipeline */
class b3GpuRigidBodyPipeline {
public:
    b3GpuRigidBodyPipeline(cl_context /*ctx*/, cl_device_id /*device*/, cl_command_queue /*q*/,
                           b3GpuNarrowPhase* narrowphase, b3GpuBroadphaseInterface* broadphaseSap,
                           b3DynamicBvhBroadphase* /*broadphaseDbvt*/, const b3Config& config)
        : m_np(narrowphase), m_bp(broadphaseSap), m_config(config) {
        if (m_bp) m_bp->attach(narrowphase);
    }
    virtual ~b3GpuRigidBodyPipeline() {}
    void stepSimulation(float deltaTime) {
        if (b3g_step(m_np->world(), deltaTime) != B3G_OK) b3Error("stepSimulation");
    }
    void integrate(float timeStep) { b3g_integrate(m_np->world(), timeStep); }
    void setupGpuAabbsFull() { b3g_setup_aabbs(m_np->world()); }
    /* registerConvexPolyhedron (b3GpuRigidBodyPipeline.cpp:591-595): the narrowphase's
       registerConvexHullShape(b3ConvexUtility*) */
    int registerConvexPolyhedron(b3ConvexUtility* convex) { return m_np->registerConvexHullShape(convex); }
    int registerPhysicsInstance(float mass, const float* position, const float* orientation, int collidableIndex,
                                int userData, bool /*writeInstanceToGpu*/) {
        return m_np->registerBody(mass, position, orientation, collidableIndex, userData);
    }
    void writeAllInstancesToGpu() { m_np->writeAllBodiesToGpu(); }
    /* copyConstraintsToHost: the host copy (b3gJoint == b3GpuGenericConstraint) carries the enabled
       flags as the device's break check left them */
    void copyConstraintsToHost() {
        int n = 0;
        b3g_get_num_constraints(m_np->world(), &n);
        m_constraints.resize((size_t)n);
        if (n > 0 && b3g_read_constraints(m_np->world(), m_constraints.data(), n, &n) != B3G_OK)
            b3Error("copyConstraintsToHost");
    }
    void setGravity(const float* grav) { b3g_set_gravity(m_np->world(), grav); }
    /* b3GpuRigidBodyPipeline::reset (b3GpuRigidBodyPipeline.cpp:141-147): every joint is dropped */
    void reset() {
        if (b3g_reset(m_np->world(), B3G_RESET_CONSTRAINTS) != B3G_OK) b3Error("reset");
        m_constraints.clear();
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
    void removeConstraintByUid(int uid) {
        if (b3g_remove_constraint(m_np->world(), uid) != B3G_OK) b3Error("removeConstraintByUid");
    }
    /* addConstraint / removeConstraint take the CPU solver's b3TypedConstraint, which this GPU step
       does not solve (the reference's GPU step ignores them too) */
    void addConstraint(class b3TypedConstraint*) { b3Warning("addConstraint: b3TypedConstraint is not solved on the GPU"); }
    void removeConstraint(class b3TypedConstraint*) {}
    /* castRays (b3GpuRigidBodyPipeline.h:63): one hit per ray; hitResults[i].m_hitResult2 names a
       body the ray ignores */
    void castRays(const b3AlignedObjectArray<b3RayInfo>& rays, b3AlignedObjectArray<b3RayHit>& hitResults) {
        const int n = rays.size();
        if (hitResults.size() != n) {
            b3Warning("castRays: hitResults must have one entry per ray");
            return;
        }
        if (n > 0 && b3g_cast_rays(m_np->world(), &rays[0], &hitResults[0], n) != B3G_OK) b3Error("castRays");
    }
    cl_mem getBodyBuffer() { return m_np->getBodiesGpu(); }
    int getNumBodies() const { return m_np->getNumRigidBodies(); }

    /* not in the reference: host copy of the joints after copyConstraintsToHost, and independent
       scenes stepped together (the reference runs one pipeline per scene; call before
       writeAllInstancesToGpu) */
    const std::vector<b3gJoint>& getConstraintsCPU() const { return m_constraints; }
    bool setSceneOffsets(const int* firstBody, int numScenes) {
        if (b3g_set_scene_offsets(m_np->world(), firstBody, numScenes) != B3G_OK) {
            b3Error("setSceneOffsets");
            return false;
        }
        return true;
    }

private:
    b3GpuNarrowPhase* m_np;
    b3GpuBroadphaseInterface* m_bp;
    b3Config m_config;
    std::vector<b3gJoint> m_constraints;
};

#endif
