/*
 * Device/host data layouts of the GPU rigid-body step.
 *
 * Every struct here is byte-compatible with the reference's shared layout so
 * that buffers returned by the drop-in API (getBodyBuffer, getContactsGpu, ...)
 * can be handed to code written against the reference:
 *   b3gBody        == b3RigidBodyData      (Bullet3Collision/NarrowPhaseCollision/shared/b3RigidBodyData.h:10)   80 B
 *   b3gInertia     == b3InertiaData        (same file :25)                                                      96 B
 *   b3gCollidable  == b3Collidable         (Bullet3Collision/NarrowPhaseCollision/shared/b3Collidable.h:22)     16 B
 *   b3gHull        == b3ConvexPolyhedronData (.../shared/b3ConvexPolyhedronData.h:20)                          96 B
 *   b3gFace        == b3GpuFace            (same file :9)                                                        32 B
 *   b3gAabb        == b3Aabb / b3SapAabb   (Bullet3Collision/BroadPhaseCollision/shared/b3Aabb.h:10)            32 B
 *   b3gContact4    == b3Contact4Data       (.../shared/b3Contact4Data.h:8)                                     112 B
 *   b3gPair        == b3Int4 overlapping pair (x=bodyA, y=bodyB, z=contact index or -1, w=-1)                  16 B
 *   b3gRayInfo     == b3RayInfo            (Bullet3Collision/NarrowPhaseCollision/b3RaycastInfo.h:7)          32 B
 *   b3gRayHit      == b3RayHit             (same file :14)                                                    48 B
 *   b3gJoint       == b3GpuGenericConstraint (Bullet3OpenCL/RigidBody/b3GpuGenericConstraint.h:77)            80 B
 * Shape type codes follow b3ShapeTypes (b3Collidable.h:8).
 */
#ifndef B3G_TYPES_H
#define B3G_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

#define B3G_SHAPE_CONVEX_HULL 3
#define B3G_SHAPE_PLANE 4
#define B3G_SHAPE_CONCAVE_TRIMESH 5  /* SHAPE_CONCAVE_TRIMESH */
#define B3G_SHAPE_COMPOUND 6   /* SHAPE_COMPOUND_OF_CONVEX_HULLS */
#define B3G_SHAPE_SPHERE 7

typedef struct b3gFloat4 { float x, y, z, w; } b3gFloat4;

typedef struct b3gBody {
    b3gFloat4 pos;
    b3gFloat4 quat;      /* x,y,z,w */
    b3gFloat4 linVel;
    b3gFloat4 angVel;
    int collidableIdx;
    float invMass;
    float restitution;
    float friction;
} b3gBody;

typedef struct b3gMat3 { b3gFloat4 row[3]; } b3gMat3;

typedef struct b3gInertia {
    b3gMat3 invInertiaWorld;
    b3gMat3 initInvInertia;
} b3gInertia;

typedef struct b3gCollidable {
    int numChildShapes;  /* unused for the supported shapes */
    float radius;        /* sphere radius; plane constant for planes */
    int shapeType;
    int shapeIndex;      /* hull index for hulls, face index for planes, 0 for spheres */
} b3gCollidable;

typedef struct b3gHull {
    b3gFloat4 localCenter;
    b3gFloat4 extents;
    b3gFloat4 mC;
    b3gFloat4 mE;
    float radius;
    int faceOffset;
    int numFaces;
    int numVertices;
    int vertexOffset;
    int uniqueEdgesOffset;
    int numUniqueEdges;
    int unused;
} b3gHull;

typedef struct b3gFace {
    b3gFloat4 plane;  /* outward normal xyz, w = plane constant (n.x + w = 0 on the face) */
    int indexOffset;
    int numIndices;
    int pad0, pad1;
} b3gFace;

typedef struct b3gAabb {
    float minv[3];
    int minw;   /* body index */
    float maxv[3];
    int maxw;   /* 1 = dynamic, 0 = static */
} b3gAabb;

typedef struct b3gContact4 {
    b3gFloat4 worldPosB[4];      /* w = signed distance (negative = penetration) */
    b3gFloat4 worldNormalOnB;    /* w = number of points */
    unsigned short restitutionCmp;
    unsigned short frictionCmp;
    int batchIdx;
    int bodyA;                   /* negative when static (reference sign convention) */
    int bodyB;
    int childIndexA;
    int childIndexB;
    int unused1;
    int unused2;
} b3gContact4;

/* b3GpuChildShape (Bullet3Collision/NarrowPhaseCollision/shared/b3Collidable.h:41-62), 48 B: a
 * compound's child, a convex hull collidable at a pose in the compound's frame */
typedef struct b3gChildShape {
    b3gFloat4 childPosition;
    b3gFloat4 childOrientation;  /* x,y,z,w */
    int shapeIndex;              /* the child's collidable (a convex hull) */
    int numChildShapes;          /* unused for children */
    int collidableShapeIndex;    /* unused for children */
    int shapeType;               /* B3G_SHAPE_CONVEX_HULL */
} b3gChildShape;

typedef struct b3gPair { int x, y, z, w; } b3gPair;

/* A concave mesh's triangle BVH (the quantized form of b3QuantizedBvh / b3BvhInfo,
 * Bullet3OpenCL/NarrowphaseCollision/b3BvhInfo.h:6-15): the mesh's local AABB widened by 1 on every
 * side, 65533 / its extent per axis, and the mesh's nodes (depth-first, nodeOffset..+numNodes). */
typedef struct b3gBvhInfo {
    b3gFloat4 aabbMin;
    b3gFloat4 aabbMax;
    b3gFloat4 quantization;
    int numNodes;
    int nodeOffset;
    int numTriangles;
    int pad;
} b3gBvhInfo;

/* b3QuantizedBvhNodeData (shared/b3QuantizedBvhNodeData.h:14-22), 16 B: quantized AABB; a leaf
 * holds its triangle index (>= 0), an internal node minus the size of its subtree in nodes. */
typedef struct b3gBvhNode {
    unsigned short quantizedAabbMin[3];
    unsigned short quantizedAabbMax[3];
    int escapeIndexOrTriangleIndex;
} b3gBvhNode;

typedef struct b3gJoint {
    int type;            /* 3 point to point, 4 fixed (b3GpuGenericConstraintType) */
    int rbA, rbB;
    float breakingImpulseThreshold;
    b3gFloat4 pivotInA;
    b3gFloat4 pivotInB;
    b3gFloat4 relTargetAB;  /* fixed: target relative orientation (quaternion x, y, z, w) */
    int flags;           /* 1 = enabled; 0 once broken */
    int uid;
    int padding[2];
} b3gJoint;

typedef struct b3gRayInfo {
    b3gFloat4 from;  /* w: the ray's scene in a world of several scenes (b3g_set_scene_offsets) */
    b3gFloat4 to;
} b3gRayInfo;

typedef struct b3gRayHit {
    float hitFraction;  /* 1 when nothing is hit */
    int hitBody;
    int hitResult1;
    int hitResult2;     /* input: a body the ray ignores (-1: none) */
    b3gFloat4 hitPoint;
    b3gFloat4 hitNormal;
} b3gRayHit;

#ifdef __cplusplus
}
#endif

#endif
