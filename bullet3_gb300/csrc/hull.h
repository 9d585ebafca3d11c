// Host-side convex hull builder used by registerConvexHullShape.
#ifndef B3G_HULL_H
#define B3G_HULL_H

#include <vector>

namespace b3g {

struct HullTables {
    std::vector<float> vertices;   // xyz per hull vertex
    std::vector<float> planes;     // xyzw per face (outward normal, constant)
    std::vector<int> face_counts;  // indices per face
    std::vector<int> indices;      // flat face vertex indices (counter-clockwise seen from outside)
    std::vector<float> edges;      // xyz per unique edge direction
    float center[3] = {0, 0, 0};   // vertex mean
};

// Returns 0 on success, 1 when the input is degenerate (fewer than 4 affinely independent points).
int build_hull(const float* verts, int stride_bytes, int num_verts, const float scaling[3], HullTables& out);

}  // namespace b3g

#endif
