// povgpu_reftree.cpp -- see povgpu_reftree.h.
#include "povgpu_reftree.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace povgpu {
namespace {

constexpr int BUNCHING_FACTOR = 4;         // boundingbox.cpp:68
constexpr double BOUND_HUGE = 2.0e10;      // configcore.h

// BBOX_TREE (boundingbox.h:98-104): a composite node lists its entries, a
// leaf stands for one item (an object, or a triangle of a mesh tree).
struct Node {
    RefBox box;
    int32_t entries;   // 0 = leaf
    int32_t first;     // composite: into kids; leaf: the item
};

struct Tree {
    std::vector<Node> nodes;
    std::vector<int32_t> kids;
    int32_t root = -1;
};

// compboxes<Axis> (boundingbox.cpp): the key 2 * lowerLeft + size, in float
thread_local const Tree* g_tree = nullptr;
thread_local int g_axis = 0;

int compboxes(const void* a, const void* b)
{
    const RefBox& ba = g_tree->nodes[*static_cast<const int32_t*>(a)].box;
    const RefBox& bb = g_tree->nodes[*static_cast<const int32_t*>(b)].box;
    const float am = (float)(2.0 * ba.ll[g_axis] + ba.sz[g_axis]);
    const float bm = (float)(2.0 * bb.ll[g_axis] + bb.sz[g_axis]);
    if (am < bm)
        return -1;
    return am == bm ? 0 : 1;
}

// find_axis: the axis of the largest extent of the boxes, in float
int find_axis(const Tree& t, const std::vector<int32_t>& fin, ptrdiff_t first, ptrdiff_t last)
{
    float mins[3] = {(float)BOUND_HUGE, (float)BOUND_HUGE, (float)BOUND_HUGE};
    float maxs[3] = {(float)-BOUND_HUGE, (float)-BOUND_HUGE, (float)-BOUND_HUGE};
    for (ptrdiff_t i = first; i < last; i++) {
        const RefBox& b = t.nodes[fin[i]].box;
        for (int k = 0; k < 3; k++) {
            mins[k] = std::min(mins[k], b.ll[k]);
            maxs[k] = std::max(maxs[k], b.ll[k] + b.sz[k]);
        }
    }
    int which = 0;
    float d = (float)-BOUND_HUGE;
    for (int k = 0; k < 3; k++) {
        const float e = maxs[k] - mins[k];
        if (e > d) {
            d = e;
            which = k;
        }
    }
    return which;
}

// Make_BBox_from_min_max (boundingbox.h:125)
RefBox from_min_max(const double* mn, const double* mx)
{
    RefBox b;
    for (int k = 0; k < 3; k++) {
        b.ll[k] = (float)mn[k];
        b.sz[k] = (float)(mx[k] - mn[k]);
    }
    return b;
}

// calc_bbox: the union of the boxes, in double over their float corners
RefBox calc_bbox(const Tree& t, const int32_t* ids, ptrdiff_t first, ptrdiff_t last)
{
    double mn[3] = {BOUND_HUGE, BOUND_HUGE, BOUND_HUGE}, mx[3] = {-BOUND_HUGE, -BOUND_HUGE, -BOUND_HUGE};
    for (ptrdiff_t i = first; i < last; i++) {
        const RefBox& b = t.nodes[ids[i]].box;
        for (int k = 0; k < 3; k++) {
            const double lo = b.ll[k], hi = lo + b.sz[k];
            mn[k] = std::min(mn[k], lo);
            mx[k] = std::max(mx[k], hi);
        }
    }
    return from_min_max(mn, mx);
}

// build_area_table: surface areas of the running unions from a towards b
void build_area_table(const Tree& t, const std::vector<int32_t>& fin, ptrdiff_t a, ptrdiff_t b, float* areas)
{
    const ptrdiff_t imin = a < b ? a : b, dir = a < b ? 1 : -1;
    float bmin[3] = {(float)BOUND_HUGE, (float)BOUND_HUGE, (float)BOUND_HUGE};
    float bmax[3] = {(float)-BOUND_HUGE, (float)-BOUND_HUGE, (float)-BOUND_HUGE};
    for (ptrdiff_t i = a; i != b + dir; i += dir) {
        const RefBox& bb = t.nodes[fin[i]].box;
        for (int k = 0; k < 3; k++) {
            const float lo = bb.ll[k], hi = lo + bb.sz[k];
            bmin[k] = std::min(bmin[k], lo);
            bmax[k] = std::max(bmax[k], hi);
        }
        const float len[3] = {bmax[0] - bmin[0], bmax[1] - bmin[1], bmax[2] - bmin[2]};
        areas[i - imin] = len[0] * (len[1] + len[2]) + len[1] * len[2];
    }
}

struct Builder {
    Tree& t;
    std::vector<int32_t> fin;    // the finite list: leaves, then the nodes each pass adds
    std::vector<float> area;

    explicit Builder(Tree& tree) : t(tree) {}

    // sort_and_split: true when the range was split (another pass follows)
    bool sort_and_split(ptrdiff_t first, ptrdiff_t last)
    {
        const ptrdiff_t size = last - first;
        ptrdiff_t best_loc = -1;
        if (size <= 0)
            return false;
        if (size > BUNCHING_FACTOR) {
            g_tree = &t;
            g_axis = find_axis(t, fin, first, last);
            std::qsort(fin.data() + first, (size_t)size, sizeof(int32_t), compboxes);
            if (area.size() < (size_t)(2 * size))
                area.resize((size_t)(2 * size));
            float* left = area.data();
            float* right = left + size;
            build_area_table(t, fin, first, last - 1, left);
            build_area_table(t, fin, last - 1, first, right);
            float best = right[0] * (float)(size - 3);
            for (ptrdiff_t i = 1; i < size; i++) {
                const float v = (float)i * left[i - 1] + (float)(size - i) * right[i];
                if (v < best) {
                    best = v;
                    best_loc = i + first;
                }
            }
        }
        if (best_loc < 0) {
            Node cd;
            cd.entries = (int32_t)size;
            cd.first = (int32_t)t.kids.size();
            for (ptrdiff_t i = 0; i < size; i++)
                t.kids.push_back(fin[first + i]);
            cd.box = calc_bbox(t, fin.data(), first, last);
            const int32_t id = (int32_t)t.nodes.size();
            t.nodes.push_back(cd);
            t.root = id;
            fin.push_back(id);
            return false;
        }
        sort_and_split(first, best_loc);
        sort_and_split(best_loc, last);
        return true;
    }

    // Build_BBox_Tree over finite leaves (no infinite objects here: the
    // traversal tests planes before the tree)
    void build(const std::vector<int32_t>& leaves)
    {
        t.root = -1;
        if (leaves.empty())
            return;
        fin = leaves;
        ptrdiff_t low = 0, high = (ptrdiff_t)fin.size();
        while (sort_and_split(low, high)) {
            low = high;
            high = (ptrdiff_t)fin.size();
        }
    }
};

int count_composites(const Tree& t)
{
    int n = 0;
    for (const Node& nd : t.nodes)
        n += nd.entries > 0;
    return n;
}

struct Flatten {
    const RefTreeInput& in;
    RefTreeOutput& out;
    std::vector<Tree> mesh_trees;
    int max_depth = 0;

    Flatten(const RefTreeInput& i, RefTreeOutput& o) : in(i), out(o) {}

    // a child box for the traversal: the reference's float box, widened by
    // one float step on every side (its corners are rounded to float)
    static void child_box(const RefBox& b, float lo[3], float hi[3])
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::nextafter(b.ll[k], -INFINITY);
            hi[k] = std::nextafter((float)((double)b.ll[k] + (double)b.sz[k]), INFINITY);
        }
    }

    int32_t leaf_refs(const uint32_t* refs, uint32_t count, const RefBox& box, int depth)
    {
        if (count == 0)
            return BVH_EMPTY;
        if (count <= 8) {
            const uint32_t first = (uint32_t)out.refs.size();
            out.refs.insert(out.refs.end(), refs, refs + count);
            return (int32_t)~((first << 3) | (count - 1));
        }
        // more primitives than a leaf holds (a union's children): chunks of
        // eight under nodes of four, each with the object's box
        std::vector<std::pair<int32_t, RefBox>> ch;
        for (uint32_t c = 0; c < count; c += 8)
            ch.push_back({leaf_refs(refs + c, std::min<uint32_t>(8, count - c), box, depth + 1), box});
        return emit_children(ch, depth);
    }

    // one four-wide node (or a small subtree, above four entries) over the
    // given (link, box) children
    int32_t emit_children(std::vector<std::pair<int32_t, RefBox>> ch, int depth)
    {
        while (ch.size() > 4) {   // group by four under nodes of their union
            std::vector<std::pair<int32_t, RefBox>> up;
            for (size_t c = 0; c < ch.size(); c += 4) {
                const size_t e = std::min(ch.size(), c + 4);
                std::vector<std::pair<int32_t, RefBox>> g(ch.begin() + c, ch.begin() + e);
                double mn[3] = {BOUND_HUGE, BOUND_HUGE, BOUND_HUGE}, mx[3] = {-BOUND_HUGE, -BOUND_HUGE, -BOUND_HUGE};
                for (auto& x : g)
                    for (int k = 0; k < 3; k++) {
                        mn[k] = std::min(mn[k], (double)x.second.ll[k]);
                        mx[k] = std::max(mx[k], (double)x.second.ll[k] + x.second.sz[k]);
                    }
                RefBox u = from_min_max(mn, mx);
                for (int k = 0; k < 3; k++)   // round the union's size up to hold every child
                    u.sz[k] = std::nextafter(u.sz[k], INFINITY);
                up.push_back({emit_node(g, depth + 1), u});
            }
            ch.swap(up);
        }
        return emit_node(ch, depth);
    }

    int32_t emit_node(const std::vector<std::pair<int32_t, RefBox>>& ch, int depth)
    {
        max_depth = std::max(max_depth, depth + 1);
        const int32_t me = (int32_t)out.nodes.size();
        out.nodes.push_back(Bvh4Node{});
        float v[6][4];
        int32_t links[4];
        for (int k = 0; k < 4; k++) {
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            links[k] = BVH_EMPTY;
            if (k < (int)ch.size() && ch[k].first != BVH_EMPTY) {
                child_box(ch[k].second, lo, hi);
                links[k] = ch[k].first;
            }
            for (int a = 0; a < 3; a++) {
                v[2 * a][k] = lo[a];
                v[2 * a + 1][k] = hi[a];
            }
        }
        Bvh4Node& o = out.nodes[me];
        o.lox = make_float4(v[0][0], v[0][1], v[0][2], v[0][3]);
        o.hix = make_float4(v[1][0], v[1][1], v[1][2], v[1][3]);
        o.loy = make_float4(v[2][0], v[2][1], v[2][2], v[2][3]);
        o.hiy = make_float4(v[3][0], v[3][1], v[3][2], v[3][3]);
        o.loz = make_float4(v[4][0], v[4][1], v[4][2], v[4][3]);
        o.hiz = make_float4(v[5][0], v[5][1], v[5][2], v[5][3]);
        o.link = make_int4(links[0], links[1], links[2], links[3]);
        o.pad = make_int4(0, 0, 0, 0);
        return me;
    }

    // the link standing for tree node n of the top tree (mesh < 0) or of
    // mesh tree `mesh`
    int32_t emit(const Tree& t, int32_t n, int mesh, int depth)
    {
        const Node& nd = t.nodes[n];
        if (nd.entries == 0) {
            if (mesh >= 0)
                return leaf_refs(&in.meshes[mesh][nd.first].ref, 1, nd.box, depth);
            const RefObject& ob = in.objects[nd.first];
            if (ob.mesh >= 0) {
                const Tree& mt = mesh_trees[ob.mesh];
                return mt.root >= 0 ? emit(mt, mt.root, ob.mesh, depth) : BVH_EMPTY;
            }
            return leaf_refs(in.refs.data() + ob.first, ob.count, nd.box, depth);
        }
        // the children first (post-order: a node follows its subtrees)
        std::vector<std::pair<int32_t, RefBox>> ch;
        for (int32_t k = 0; k < nd.entries; k++) {
            const int32_t c = t.kids[nd.first + k];
            ch.push_back({emit(t, c, mesh, depth + 1), t.nodes[c].box});
        }
        // more than four entries (sort_and_split found no split) become a
        // small subtree of nodes of four
        return emit_children(ch, depth);
    }
};

}  // namespace

void build_reference_tree(const RefTreeInput& in, RefTreeOutput& out)
{
    out = RefTreeOutput{};
    Flatten F(in, out);
    // each mesh's own tree over its triangles (Build_Mesh_BBox_Tree)
    F.mesh_trees.resize(in.meshes.size());
    for (size_t m = 0; m < in.meshes.size(); m++) {
        Tree& mt = F.mesh_trees[m];
        std::vector<int32_t> leaves;
        for (size_t i = 0; i < in.meshes[m].size(); i++) {
            Node n;
            n.box = in.meshes[m][i].box;
            n.entries = 0;
            n.first = (int32_t)i;
            leaves.push_back((int32_t)mt.nodes.size());
            mt.nodes.push_back(n);
        }
        Builder(mt).build(leaves);
        out.mesh_nodes += count_composites(mt);
    }
    // the top tree over the finite objects (Build_Bounding_Slabs)
    Tree top;
    std::vector<int32_t> leaves;
    for (size_t i = 0; i < in.objects.size(); i++) {
        Node n;
        n.box = in.objects[i].box;
        n.entries = 0;
        n.first = (int32_t)i;
        leaves.push_back((int32_t)top.nodes.size());
        top.nodes.push_back(n);
    }
    Builder(top).build(leaves);
    // BoundingTask: no slabs below Bounding_Threshold 3 objects
    // (boundingtask.cpp:170); the infinite objects get a node of their own
    // under the root (Build_BBox_Tree, boundingbox.cpp:300-320)
    const bool slabs = (int)in.objects.size() + in.infinite >= 3;
    out.top_nodes = slabs ? count_composites(top) + (in.infinite > 0 ? 1 : 0) : 0;
    if (top.root < 0) {
        out.root = BVH_EMPTY;
        return;
    }
    if (top.nodes[top.root].entries == 0) {   // one object: a root node above its leaf
        std::vector<std::pair<int32_t, RefBox>> ch{{F.emit(top, top.root, -1, 1), top.nodes[top.root].box}};
        out.root = F.emit_node(ch, 0);
    } else {
        out.root = F.emit(top, top.root, -1, 0);
    }
    out.depth = F.max_depth;
}

}  // namespace povgpu
