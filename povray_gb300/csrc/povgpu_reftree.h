// povgpu_reftree.h -- the reference's bounding tree for the traversal.
//
// POV-Ray bounds a scene with Build_Bounding_Slabs / Build_BBox_Tree
// (source/core/bounding/boundingbox.cpp:262-430, sort_and_split :834-928):
// a bottom-up tree over the finite top-level objects' float boxes whose
// nodes hold at most BUNCHING_FACTOR (4) entries, and each mesh2 its own
// tree of the same kind over its triangles (Build_Mesh_BBox_Tree,
// source/core/shape/mesh.cpp:1376-1450).  This module restates that build
// and flattens the result into the traversal's four-wide nodes, each mesh's
// tree grafted under the mesh's leaf, so the device can trace the same tree
// the reference traces (the library's default is its own binned-SAH tree).
#ifndef POVGPU_REFTREE_H
#define POVGPU_REFTREE_H

#include <cstdint>
#include <vector>

#include "povgpu_internal.h"

namespace povgpu {

// BoundingBox as the reference stores it: lower-left corner and size, float.
struct RefBox {
    float ll[3];
    float sz[3];
};

// A finite top-level object: its box (the shape's Compute_BBox) and either
// its primitive references (first, count into RefTreeInput::refs) or, for a
// mesh2, the index of its triangle list.
struct RefObject {
    RefBox   box;
    uint32_t first = 0, count = 0;
    int32_t  mesh = -1;
};

// A mesh2 triangle: its box (min/max of its three vertices) and its
// primitive reference.
struct RefTriangle {
    RefBox   box;
    uint32_t ref;
};

struct RefTreeInput {
    std::vector<RefObject> objects;   // in scene order (Build_Bounding_Slabs keeps it)
    int32_t infinite = 0;             // infinite top-level objects (planes; the traversal tests them first)
    std::vector<uint32_t> refs;
    std::vector<std::vector<RefTriangle>> meshes;
    bool empty() const { return objects.empty(); }
};

struct RefTreeOutput {
    std::vector<Bvh4Node> nodes;   // four-wide nodes, each after its subtrees (root: `root`)
    std::vector<uint32_t> refs;    // leaf primitive references
    int32_t root = BVH_EMPTY;
    int     depth = 0;             // levels of four-wide nodes
    int     top_nodes = 0;         // composite nodes of the reference's top tree: none below
                                   // Bounding_Threshold (3 objects), one more for the infinite
                                   // objects' node
    int     mesh_nodes = 0;        // composite nodes of the mesh trees
};

// Builds the reference's trees over `in` and flattens them (host only).
void build_reference_tree(const RefTreeInput& in, RefTreeOutput& out);

}  // namespace povgpu

#endif
