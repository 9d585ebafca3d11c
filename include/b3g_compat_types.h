/*
 * b3g_compat_types.h -- host-side value types of the reference's API for the C++ drop-in
 * (include/b3g_compat.h), written for this library with the reference's names, members and byte
 * layouts, so that code written against Bullet3's GPU pipeline compiles without the reference's
 * Bullet3Common / Bullet3Collision headers:
 *
 *   b3Scalar, b3Vector3, b3Vector4, b3MakeVector3/4  Bullet3Common/b3Vector3.h (16-byte x, y, z, w)
 *   b3Quaternion                                     Bullet3Common/b3Quaternion.h (x, y, z, w)
 *   b3AlignedObjectArray<T>                          Bullet3Common/b3AlignedObjectArray.h
 *   b3Int4                                           Bullet3Common/shared/b3Int4.h
 *   b3SapAabb                                        Bullet3OpenCL/BroadphaseCollision/b3SapAabb.h
 *   b3RigidBodyData, b3InertiaData, b3Collidable,
 *   b3Contact4                                       Bullet3Collision/NarrowPhaseCollision/shared/ (same names)
 *   b3RayInfo, b3RayHit                              Bullet3Collision/NarrowPhaseCollision/b3RaycastInfo.h
 *   b3MyFace, b3ConvexUtility                        Bullet3Collision/NarrowPhaseCollision/b3ConvexUtility.h
 *                                                    (initializePolyhedralFeatures runs this library's
 *                                                    hull builder, which gives the reference's tables
 *                                                    bit for bit)
 *   b3Config                                         Bullet3Collision/NarrowPhaseCollision/b3Config.h
 *   b3Min, b3Max                                     Bullet3Common/b3MinMax.h
 *   b3DynamicBvhBroadphase (constructor only)        Bullet3Collision/BroadPhaseCollision/b3DynamicBvhBroadphase.h
 *
 * Each block is skipped when the reference's own header was included first (same include-guard
 * macro), so a program may mix them; the layouts are the same either way.
 */
#ifndef B3G_COMPAT_TYPES_H
#define B3G_COMPAT_TYPES_H

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <vector>

#include "b3g_capi.h"
#include "b3g_types.h"

#ifndef B3_SCALAR_H
typedef float b3Scalar;
#endif

#ifndef B3_VECTOR3_H
#define B3_VECTOR3_H
struct alignas(16) b3Vector3 {
    b3Scalar m_floats[4];
    b3Vector3() {}
    b3Scalar getX() const { return m_floats[0]; }
    b3Scalar getY() const { return m_floats[1]; }
    b3Scalar getZ() const { return m_floats[2]; }
    b3Scalar getW() const { return m_floats[3]; }
    void setValue(b3Scalar x, b3Scalar y, b3Scalar z) {
        m_floats[0] = x;
        m_floats[1] = y;
        m_floats[2] = z;
        m_floats[3] = 0.f;
    }
    void setZero() { setValue(0.f, 0.f, 0.f); }
    operator b3Scalar*() { return m_floats; }
    operator const b3Scalar*() const { return m_floats; }
    b3Vector3& operator+=(const b3Vector3& v) {
        for (int k = 0; k < 3; k++) m_floats[k] += v.m_floats[k];
        return *this;
    }
    b3Vector3& operator-=(const b3Vector3& v) {
        for (int k = 0; k < 3; k++) m_floats[k] -= v.m_floats[k];
        return *this;
    }
    b3Vector3& operator*=(b3Scalar s) {
        for (int k = 0; k < 3; k++) m_floats[k] *= s;
        return *this;
    }
    b3Vector3& operator/=(b3Scalar s) { return *this *= (1.f / s); }
    b3Scalar dot(const b3Vector3& v) const {
        return m_floats[0] * v.m_floats[0] + m_floats[1] * v.m_floats[1] + m_floats[2] * v.m_floats[2];
    }
    b3Scalar length2() const { return dot(*this); }
    b3Scalar length() const { return std::sqrt(length2()); }
    b3Vector3& normalize() { return *this /= length(); }
    b3Vector3 cross(const b3Vector3& v) const {
        b3Vector3 r;
        r.setValue(m_floats[1] * v.m_floats[2] - m_floats[2] * v.m_floats[1],
                   m_floats[2] * v.m_floats[0] - m_floats[0] * v.m_floats[2],
                   m_floats[0] * v.m_floats[1] - m_floats[1] * v.m_floats[0]);
        return r;
    }
    void setMin(const b3Vector3& o) {
        for (int k = 0; k < 3; k++) m_floats[k] = std::min(m_floats[k], o.m_floats[k]);
    }
    void setMax(const b3Vector3& o) {
        for (int k = 0; k < 3; k++) m_floats[k] = std::max(m_floats[k], o.m_floats[k]);
    }
};
typedef b3Vector3 b3Vector4;
inline b3Vector3 b3MakeVector3(b3Scalar x, b3Scalar y, b3Scalar z, b3Scalar w = 0.f) {
    b3Vector3 v;
    v.m_floats[0] = x;
    v.m_floats[1] = y;
    v.m_floats[2] = z;
    v.m_floats[3] = w;
    return v;
}
inline b3Vector3 b3MakeVector4(b3Scalar x, b3Scalar y, b3Scalar z, b3Scalar w) { return b3MakeVector3(x, y, z, w); }
inline b3Vector3 operator+(b3Vector3 a, const b3Vector3& b) { return a += b; }
inline b3Vector3 operator-(b3Vector3 a, const b3Vector3& b) { return a -= b; }
inline b3Vector3 operator*(b3Vector3 a, b3Scalar s) { return a *= s; }
inline b3Vector3 operator*(b3Scalar s, b3Vector3 a) { return a *= s; }
inline b3Vector3 operator-(const b3Vector3& a) { return b3MakeVector3(-a.m_floats[0], -a.m_floats[1], -a.m_floats[2]); }
#endif

#ifndef B3_SIMD__QUATERNION_H_
#define B3_SIMD__QUATERNION_H_
struct alignas(16) b3Quaternion {
    b3Scalar m_floats[4];
    b3Quaternion() {}
    b3Quaternion(b3Scalar x, b3Scalar y, b3Scalar z, b3Scalar w) { setValue(x, y, z, w); }
    void setValue(b3Scalar x, b3Scalar y, b3Scalar z, b3Scalar w) {
        m_floats[0] = x;
        m_floats[1] = y;
        m_floats[2] = z;
        m_floats[3] = w;
    }
    b3Scalar getX() const { return m_floats[0]; }
    b3Scalar getY() const { return m_floats[1]; }
    b3Scalar getZ() const { return m_floats[2]; }
    b3Scalar getW() const { return m_floats[3]; }
    operator b3Scalar*() { return m_floats; }
    operator const b3Scalar*() const { return m_floats; }
};
#endif

#ifndef B3_OBJECT_ARRAY__
#define B3_OBJECT_ARRAY__
/* The reference's growable array: contiguous storage, size/capacity, push_back/expand, and its
 * remove (the first match swapped with the last element, then popped). */
template <typename T>
class b3AlignedObjectArray {
public:
    int size() const { return (int)m_data.size(); }
    int capacity() const { return (int)m_data.capacity(); }
    void reserve(int n) { m_data.reserve((size_t)n); }
    void resize(int n, const T& fill = T()) { m_data.resize((size_t)n, fill); }
    void clear() { m_data.clear(); }
    void push_back(const T& v) { m_data.push_back(v); }
    void pop_back() { m_data.pop_back(); }
    T& expand(const T& v = T()) {
        m_data.push_back(v);
        return m_data.back();
    }
    T& operator[](int i) { return m_data[(size_t)i]; }
    const T& operator[](int i) const { return m_data[(size_t)i]; }
    T& at(int i) { return m_data.at((size_t)i); }
    const T& at(int i) const { return m_data.at((size_t)i); }
    int findLinearSearch(const T& key) const {
        for (int i = 0; i < size(); i++)
            if (m_data[(size_t)i] == key) return i;
        return size();
    }
    void swap(int i, int j) { std::swap(m_data[(size_t)i], m_data[(size_t)j]); }
    void remove(const T& key) {
        const int i = findLinearSearch(key);
        if (i < size()) {
            swap(i, size() - 1);
            pop_back();
        }
    }
    template <typename L>
    void quickSort(const L& less) {
        std::sort(m_data.begin(), m_data.end(), less);
    }

private:
    std::vector<T> m_data;
};
#endif

#ifndef B3_INT4_H
#define B3_INT4_H
typedef b3gPair b3Int4;
#endif

#ifndef B3_SAP_AABB_H
#define B3_SAP_AABB_H
/* 32 B: min xyz + (body index in the w slot), max xyz + (signed w slot), as b3SapAabb */
struct b3SapAabb {
    union {
        float m_min[4];
        int m_minIndices[4];
    };
    union {
        float m_max[4];
        int m_signedMaxIndices[4];
    };
};
#endif

#ifndef B3_RIGIDBODY_DATA_H
#define B3_RIGIDBODY_DATA_H
struct b3RigidBodyData {  // 80 B, the layout of b3gBody
    b3Vector3 m_pos;
    b3Quaternion m_quat;
    b3Vector3 m_linVel;
    b3Vector3 m_angVel;
    int m_collidableIdx;
    float m_invMass;
    float m_restituitionCoeff;
    float m_frictionCoeff;
};
struct b3InertiaData {  // 96 B: two 3x4 row matrices, the layout of b3gInertia
    float m_invInertiaWorld[3][4];
    float m_initInvInertia[3][4];
};
#endif

#ifndef B3_COLLIDABLE_H
#define B3_COLLIDABLE_H
typedef b3gCollidable b3Collidable;
#endif

#ifndef B3_CONTACT4_H
#define B3_CONTACT4_H
typedef b3gContact4 b3Contact4;
#endif

/* b3GpuChildShape (Bullet3Collision/NarrowPhaseCollision/shared/b3Collidable.h:41-58): a child of a
 * compound, the layout of b3gChildShape (48 B) */
struct alignas(16) b3GpuChildShape {
    b3Vector3 m_childPosition;
    b3Quaternion m_childOrientation;
    union {
        int m_shapeIndex;  // the child's collidable (a convex hull)
        int m_capsuleAxis;
    };
    union {
        float m_radius;
        int m_numChildShapes;
    };
    union {
        float m_height;
        int m_collidableShapeIndex;
    };
    int m_shapeType;
};
static_assert(sizeof(b3GpuChildShape) == sizeof(b3gChildShape), "b3GpuChildShape layout");

#ifndef B3_GEN_MINMAX_H
#define B3_GEN_MINMAX_H
template <class T>
inline const T& b3Min(const T& a, const T& b) {
    return a < b ? a : b;
}
template <class T>
inline const T& b3Max(const T& a, const T& b) {
    return a > b ? a : b;
}
#endif

#ifndef B3_DBVT_BROADPHASE_H
#define B3_DBVT_BROADPHASE_H
/* The reference pipeline's CPU broadphase slot (b3DynamicBvhBroadphase): the GPU step here does not
 * use it, so the stand-in only has the constructor the demos call. */
struct b3DynamicBvhBroadphase {
    explicit b3DynamicBvhBroadphase(int /*proxyCapacity*/) {}
};
#endif

#ifndef B3_RAYCAST_INFO_H
#define B3_RAYCAST_INFO_H
struct b3RayInfo {  // the layout of b3gRayInfo
    b3Vector3 m_from;
    b3Vector3 m_to;
};
struct b3RayHit {  // the layout of b3gRayHit
    b3Scalar m_hitFraction;
    int m_hitBody;
    int m_hitResult1;
    int m_hitResult2;
    b3Vector3 m_hitPoint;
    b3Vector3 m_hitNormal;
};
#endif

#ifndef B3_CONFIG_H
#define B3_CONFIG_H
/* capacities with the reference's defaults (b3Config.h:22-36) */
struct b3Config {
    int m_maxConvexBodies;
    int m_maxConvexShapes;
    int m_maxBroadphasePairs;
    int m_maxContactCapacity;
    int m_compoundPairCapacity;
    int m_maxVerticesPerFace;
    int m_maxFacesPerShape;
    int m_maxConvexVertices;
    int m_maxConvexIndices;
    int m_maxConvexUniqueEdges;
    int m_maxCompoundChildShapes;
    int m_maxTriConvexPairCapacity;
    b3Config()
        : m_maxConvexBodies(128 * 1024),
          m_maxVerticesPerFace(64),
          m_maxFacesPerShape(12),
          m_maxConvexVertices(8192),
          m_maxConvexIndices(81920),
          m_maxConvexUniqueEdges(8192),
          m_maxCompoundChildShapes(8192),
          m_maxTriConvexPairCapacity(256 * 1024) {
        m_maxConvexShapes = m_maxConvexBodies;
        m_maxBroadphasePairs = 16 * m_maxConvexBodies;
        m_maxContactCapacity = m_maxBroadphasePairs;
        m_compoundPairCapacity = 1024 * 1024;
    }
};
#endif

#ifndef _BT_CONVEX_UTILITY_H
#define _BT_CONVEX_UTILITY_H
struct b3MyFace {
    b3AlignedObjectArray<int> m_indices;
    b3Scalar m_plane[4];
};
/* Hull topology of a point cloud (b3ConvexUtility::initializePolyhedralFeatures): vertices, merged
 * faces with their planes, unique edge directions.  Built by this library's hull builder
 * (b3g_hull_compute), whose tables equal the reference's bit for bit.  m_localCenter is the
 * vertex mean, as registerConvexHullShape sets it; m_extents, mC, mE and m_radius are zero (the
 * reference leaves them unset). */
class b3ConvexUtility {
public:
    b3Vector3 m_localCenter;
    b3Vector3 m_extents;
    b3Vector3 mC;
    b3Vector3 mE;
    b3Scalar m_radius = 0.f;
    b3AlignedObjectArray<b3Vector3> m_vertices;
    b3AlignedObjectArray<b3MyFace> m_faces;
    b3AlignedObjectArray<b3Vector3> m_uniqueEdges;

    b3ConvexUtility() {
        m_localCenter.setZero();
        m_extents.setZero();
        mC.setZero();
        mE.setZero();
    }
    virtual ~b3ConvexUtility() {}
    bool initializePolyhedralFeatures(const b3Vector3* orgVertices, int numVertices, bool /*mergeCoplanarTriangles*/ = true) {
        m_vertices.clear();
        m_faces.clear();
        m_uniqueEdges.clear();
        if (numVertices <= 0) return true;
        const int cap = 8 * numVertices + 64;
        std::vector<float> v(3 * (size_t)cap), planes(4 * (size_t)cap), edges(3 * (size_t)cap), centre(3);
        std::vector<int> counts((size_t)cap), indices(8 * (size_t)cap);
        int sizes[6] = {cap, cap, 8 * cap, cap, 0, 0};
        const float one[3] = {1.f, 1.f, 1.f};
        if (b3g_hull_compute(&orgVertices[0].m_floats[0], (int)sizeof(b3Vector3), numVertices, one, v.data(),
                             planes.data(), counts.data(), indices.data(), edges.data(), centre.data(), sizes) != B3G_OK) {
            std::fprintf(stderr, "b3Error: initializePolyhedralFeatures: %s\n", b3g_last_error());
            return false;
        }
        for (int i = 0; i < sizes[0]; i++) m_vertices.push_back(b3MakeVector3(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
        int off = 0;
        for (int f = 0; f < sizes[1]; f++) {
            b3MyFace& face = m_faces.expand();
            for (int k = 0; k < 4; k++) face.m_plane[k] = planes[4 * (size_t)f + k];
            for (int k = 0; k < counts[(size_t)f]; k++) face.m_indices.push_back(indices[(size_t)off + k]);
            off += counts[(size_t)f];
        }
        for (int i = 0; i < sizes[3]; i++) m_uniqueEdges.push_back(b3MakeVector3(edges[3 * i], edges[3 * i + 1], edges[3 * i + 2]));
        m_localCenter = b3MakeVector3(centre[0], centre[1], centre[2]);
        return true;
    }
};
#endif

#endif
