// povgpu_host.cpp -- C ABI of libpovgpu (include/povgpu.h): scene
// validation, reference-identical mesh2 triangle setup, BVH construction,
// device upload and the per-batch kernel sequence.
//
// The scene arrives as the reference's parser leaves it (SceneData walked by
// the caller).  Shapes the GPU path does not implement are rejected here with
// POV_GPU_E_UNSUPPORTED: there is no CPU fallback.
#include "povgpu.h"
#include "povgpu_internal.h"
#include "povgpu_reftree.h"
#include "povgpu_kernels.h"
#include "povgpu_radiosity.h"
#include "povgpu_nic.h"
#include "povgpu_noise_table.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

using namespace povgpu;

namespace {

constexpr double EPSILON = 1.0e-10;   // source/core/configcore.h:153
constexpr int TRACE_BLOCK = 128;

// ------------------------------------------------------------ device mem --
struct DevBuf {
    void*  p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n)
    {
        if (n <= bytes)
            return cudaSuccess;
        if (p)
            cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t want = std::max<size_t>(n, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess)
            bytes = want;
        return e;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

template <class T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v)
{
    cudaError_t e = b.ensure(sizeof(T) * std::max<size_t>(v.size(), 1));
    if (e != cudaSuccess || v.empty())
        return e;
    return cudaMemcpy(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
}

// ------------------------------------------------------------------ BVH --
struct AABB {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const AABB& b)
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    void grow(const float* p)
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    float area() const
    {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx < 0 || dy < 0 || dz < 0)
            return 0.f;
        return 2.f * (dx * dy + dy * dz + dz * dx);
    }
};

struct BuildItem {
    AABB     box;
    float    c[3];
    uint32_t ref;
    float    cost;   // relative cost of its intersection test (a triangle's is 1)
};

// Relative test costs per primitive kind for the SAH: a torus runs the FP32
// pre-cull and, when it passes, the FP64 quartic; a CSG finds every child's
// roots and tests each against the siblings; boxes take three slabs.
inline float prim_cost(uint32_t kind)
{
    switch (kind) {
    case PK_TORUS: return 8.0f;
    case PK_CSG: return 6.0f;
    case PK_BOX: return 1.5f;
    default: return 1.0f;
    }
}

// Binned-SAH binary BVH emitted as two-wide 64-byte nodes in depth-first
// order, each primitive weighted by its test cost.  Leaves hold at most
// LEAF_MAX_PRIMS prim references.
class BvhBuilder {
public:
    std::vector<BuildItem> items;
    std::vector<BvhNode>   nodes;
    std::vector<uint32_t>  refs;
    int max_depth = 0;

    int build_root()
    {
        nodes.clear();
        refs.clear();
        max_depth = 0;
        if (items.empty())
            return 0x7fffffff;   // traversal sentinel: nothing to visit
        AABB lb;
        return build(0, (int)items.size(), 1, lb);   // an inner node or a leaf link
    }

private:
    static void put(float4& f, float a, float b, float c, float d) { f = make_float4(a, b, c, d); }

    void write_node(int ni, const AABB& b0, int l0, const AABB& b1, int l1)
    {
        BvhNode& n = nodes[ni];
        put(n.a, b0.lo[0], b0.hi[0], b0.lo[1], b0.hi[1]);
        put(n.b, b1.lo[0], b1.hi[0], b1.lo[1], b1.hi[1]);
        put(n.c, b0.lo[2], b0.hi[2], b1.lo[2], b1.hi[2]);
        n.d = make_float4(__builtin_bit_cast(float, l0), __builtin_bit_cast(float, l1), 0.f, 0.f);
    }

    int make_leaf(int begin, int end, AABB& bounds)
    {
        bounds = AABB();
        uint32_t first = (uint32_t)refs.size();
        for (int i = begin; i < end; i++) {
            bounds.grow(items[i].box);
            refs.push_back(items[i].ref);
        }
        uint32_t code = (first << 3) | (uint32_t)(end - begin - 1);
        return (int)~code;
    }

    int build(int begin, int end, int depth, AABB& bounds)
    {
        max_depth = std::max(max_depth, depth);
        int n = end - begin;
        AABB cb;
        float cost_all = 0.0f;
        for (int i = begin; i < end; i++) {
            cb.grow(items[i].c);
            cost_all += items[i].cost;
        }
        if (n == 1 || (n <= 2 && cost_all <= 2.0f))   // two cheap primitives: a leaf
            return make_leaf(begin, end, bounds);
        int axis = 0;
        float ext[3] = {cb.hi[0] - cb.lo[0], cb.hi[1] - cb.lo[1], cb.hi[2] - cb.lo[2]};
        int mid = -1;
        if (ext[0] <= 0.f && ext[1] <= 0.f && ext[2] <= 0.f) {
            if (n <= LEAF_MAX_PRIMS)
                return make_leaf(begin, end, bounds);
            mid = begin + n / 2;
        } else if (depth >= 48) {
            // depth guard: object-median split keeps the stack bounded
            axis = ext[1] > ext[axis] ? 1 : axis;
            axis = ext[2] > ext[axis] ? 2 : axis;
            mid = begin + n / 2;
            std::nth_element(items.begin() + begin, items.begin() + mid, items.begin() + end,
                             [axis](const BuildItem& a, const BuildItem& b) { return a.c[axis] < b.c[axis]; });
        } else {
            constexpr int NB = 32;
            float best_cost = INFINITY;
            int best_axis = -1, best_bin = -1;
            AABB total;
            for (int i = begin; i < end; i++)
                total.grow(items[i].box);
            for (int ax = 0; ax < 3; ax++) {
                if (ext[ax] <= 0.f)
                    continue;
                AABB bb[NB];
                int cnt[NB] = {0};
                float bcost[NB] = {0.0f};
                float scale = NB / ext[ax];
                for (int i = begin; i < end; i++) {
                    int b = std::min(NB - 1, (int)((items[i].c[ax] - cb.lo[ax]) * scale));
                    cnt[b]++;
                    bcost[b] += items[i].cost;
                    bb[b].grow(items[i].box);
                }
                float rarea[NB], rcost[NB];
                int rcnt[NB];
                AABB acc;
                int c = 0;
                float w = 0.0f;
                for (int b = NB - 1; b > 0; b--) {
                    acc.grow(bb[b]);
                    c += cnt[b];
                    w += bcost[b];
                    rarea[b] = acc.area();
                    rcnt[b] = c;
                    rcost[b] = w;
                }
                acc = AABB();
                c = 0;
                w = 0.0f;
                for (int b = 0; b < NB - 1; b++) {
                    acc.grow(bb[b]);
                    c += cnt[b];
                    w += bcost[b];
                    if (c == 0 || rcnt[b + 1] == 0)
                        continue;
                    float cost = acc.area() * w + rarea[b + 1] * rcost[b + 1];
                    if (cost < best_cost) {
                        best_cost = cost;
                        best_axis = ax;
                        best_bin = b;
                    }
                }
            }
            float leaf_cost = total.area() * cost_all;
            float trav = total.area() * 1.0f;
            if (best_axis < 0 || (n <= 4 && best_cost + trav >= leaf_cost)) {
                if (n <= LEAF_MAX_PRIMS)
                    return make_leaf(begin, end, bounds);
                mid = begin + n / 2;
                axis = ext[1] > ext[axis] ? 1 : axis;
                axis = ext[2] > ext[axis] ? 2 : axis;
                std::nth_element(items.begin() + begin, items.begin() + mid, items.begin() + end,
                                 [axis](const BuildItem& a, const BuildItem& b) { return a.c[axis] < b.c[axis]; });
            } else {
                float scale = NB / ext[best_axis];
                float lo = cb.lo[best_axis];
                auto it = std::partition(items.begin() + begin, items.begin() + end, [&](const BuildItem& x) {
                    int b = std::min(NB - 1, (int)((x.c[best_axis] - lo) * scale));
                    return b <= best_bin;
                });
                mid = (int)(it - items.begin());
                if (mid == begin || mid == end)
                    mid = begin + n / 2;
            }
        }
        int ni = (int)nodes.size();
        nodes.push_back(BvhNode{});
        AABB b0, b1;
        int l0 = build(begin, mid, depth + 1, b0);
        int l1 = build(mid, end, depth + 1, b1);
        write_node(ni, b0, l0, b1, l1);
        bounds = b0;
        bounds.grow(b1);
        return ni;
    }
};

// Collapses the binary tree into four-wide nodes: starting from a node's two
// children, the inner child with the largest box surface area is replaced
// by its own two children until four are held or only leaves remain.
struct Bvh4Collapse {
    const std::vector<BvhNode>& in;
    std::vector<Bvh4Node> out;
    int max_depth = 0;

    explicit Bvh4Collapse(const std::vector<BvhNode>& n) : in(n) {}

    struct Child {
        float lo[3], hi[3];
        int link;
    };

    static float area(const Child& c)
    {
        float d[3] = {c.hi[0] - c.lo[0], c.hi[1] - c.lo[1], c.hi[2] - c.lo[2]};
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }

    void children_of(int ni, Child& a, Child& b) const
    {
        const BvhNode& n = in[ni];
        a = {{n.a.x, n.a.z, n.c.x}, {n.a.y, n.a.w, n.c.y}, __builtin_bit_cast(int, n.d.x)};
        b = {{n.b.x, n.b.z, n.c.z}, {n.b.y, n.b.w, n.c.w}, __builtin_bit_cast(int, n.d.y)};
    }

    // returns the index of the four-wide node for binary inner node ni
    int collapse(int ni, int depth)
    {
        max_depth = std::max(max_depth, depth);
        Child ch[4];
        int n = 2;
        children_of(ni, ch[0], ch[1]);
        while (n < 4) {
            int best = -1;
            float ba = -1.0f;
            for (int k = 0; k < n; k++)
                if (ch[k].link >= 0 && area(ch[k]) > ba) {
                    ba = area(ch[k]);
                    best = k;
                }
            if (best < 0)
                break;
            Child a, b;
            children_of(ch[best].link, a, b);
            ch[best] = a;
            ch[n++] = b;
        }
        const int me = (int)out.size();
        out.push_back(Bvh4Node{});
        int links[4];
        for (int k = 0; k < 4; k++)
            links[k] = k < n ? (ch[k].link >= 0 ? collapse(ch[k].link, depth + 1) : ch[k].link) : BVH_EMPTY;
        Bvh4Node& o = out[me];
        float v[6][4];
        for (int k = 0; k < 4; k++)
            for (int a = 0; a < 3; a++) {
                v[2 * a][k] = k < n ? ch[k].lo[a] : INFINITY;
                v[2 * a + 1][k] = k < n ? ch[k].hi[a] : -INFINITY;
            }
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
};

// ------------------------------------------------- mesh2 triangle setup --
static int max3_coordinate(double x, double y, double z)
{
    if (x > y)
        return x > z ? 0 : 2;
    return y > z ? 1 : 2;
}

struct V3d {
    double x, y, z;
};
static V3d vsub(V3d a, V3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static V3d vcross(V3d a, V3d b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static double vlen(V3d a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// Object -> world point with a TRANSFORM's forward matrix (row-vector form).
static V3d mtrans_point(const double* m, V3d v)
{
    return {v.x * m[0] + v.y * m[4] + v.z * m[8] + m[12], v.x * m[1] + v.y * m[5] + v.z * m[9] + m[13],
            v.x * m[2] + v.y * m[6] + v.z * m[10] + m[14]};
}

static void grow_outward(AABB& b, double x, double y, double z)
{
    const float p[3] = {(float)x, (float)y, (float)z};
    for (int k = 0; k < 3; k++) {
        b.lo[k] = std::min(b.lo[k], std::nextafter(p[k], -INFINITY));
        b.hi[k] = std::max(b.hi[k], std::nextafter(p[k], INFINITY));
    }
}

}  // namespace

// ---------------------------------------------------------------- scene --
namespace {

// Deferred torus tests a wavefront's list holds: four per shadow ray
// (64 Mi at most); beyond it the traversal solves them in line.
inline size_t tcand_cap(size_t maxq, int nl)
{
    return std::min<size_t>((size_t)4 * maxq * (size_t)std::max(nl, 1), (size_t)64 << 20);
}

// Counter slots of a wavefront (PathBufs::counters).
enum {
    C_QA = 0,     // count of queue A
    C_QB = 1,     // count of queue B
    C_SQ = 2,     // shadow queue
    C_W0 = 3,     // work counter, closest-hit
    C_W1 = 4,     // work counter, any-hit
    C_NS = 5,     // AA: samples of this round
    C_NC = 6,     // AA: active cells
    C_NN = 7,     // AA: next cells
    C_AQ = 8,     // area-light shadow items
    C_RQ = 9,     // radiosity queries
    C_MC = 10,    // rays crossing a media container's interior
    C_ML = 11,    // media samples listed for the next round
    C_MW = 12,    // work counter of the media sample rounds
    C_TC = 13,    // deferred torus tests of the current traversal launch
    C_TO = 14,    // rays handed to the second traversal launch (torus-free variant)
    C_TW = 15,    // work counter of that launch
    C_NUM = 16
};

// One wavefront of ray queues and per-path state: the camera's, or the
// sample rays of one radiosity bounce depth.  Counters live in `counters`
// (C_* slots).
struct PathBufs {
    DevBuf qA, qB, pathA, pathB, hits, paths, slot_contrib, sq, sq_slot, blocked, skipA, skipB, sskip;
    DevBuf aq, aq_slot, aq_skip;   // area-light shadow items
    DevBuf rq, rq_amb;             // radiosity queries of the hits, and their answers
    DevBuf quality, first_t;       // sample rays: quality of each, depth of its first hit
    DevBuf stateA, stateB, smedium; // media containers: per-ray level and medium, shadow-ray medium
    DevBuf mlist, mte, mod;         // media containers: listed rays, per-interval sums
    DevBuf mcbuf, mrounds;          // media containers: sample slots of a chunk, round lists
    DevBuf bin_keys, bin_hist, bin_order;   // textured scenes: the shade queue binned by material
    DevBuf rinA, rinB, srin;        // transparent scenes: per-ray and shadow-ray interior lists
    DevBuf thrA, thrB;              // transparent surfaces that reflect: per-ray throughput
    DevBuf tcand, tkey;             // scenes with tori: deferred torus tests, per-ray nearest roots
    DevBuf tovf;                    // torus-free traversal: rays for the second launch
    DevBuf counters;

    // media_ni: interval slots per ray segment (0: the scene has no media
    // containers); transparent: rays carry their level and interior list
    cudaError_t ensure(size_t maxq, int nl, int nal, bool rad, bool sample_rays, int media_ni = 0,
                       bool binned = false, bool transparent = false, bool tori = false, bool torus_free = false)
    {
        maxq = std::max<size_t>(maxq, 1);
        nl = std::max(nl, 1);
        cudaError_t e;
#define PB_ENSURE(buf, bytes) if ((e = (buf).ensure(bytes)) != cudaSuccess) return e
        PB_ENSURE(counters, sizeof(int) * C_NUM);
        PB_ENSURE(qA, sizeof(QRay) * maxq);
        PB_ENSURE(qB, sizeof(QRay) * maxq);
        PB_ENSURE(pathA, sizeof(int) * maxq);
        PB_ENSURE(pathB, sizeof(int) * maxq);
        PB_ENSURE(hits, sizeof(QHit) * maxq);
        PB_ENSURE(paths, sizeof(PathState) * maxq);
        PB_ENSURE(slot_contrib, sizeof(float4) * maxq * nl);
        PB_ENSURE(sq, sizeof(QRay) * maxq * nl);
        PB_ENSURE(sq_slot, sizeof(int) * maxq * nl);
        PB_ENSURE(blocked, (maxq * nl + 3) & ~(size_t)3);   // whole words (k_torus_solve's atomicOr)
        PB_ENSURE(skipA, sizeof(uint2) * maxq);
        PB_ENSURE(skipB, sizeof(uint2) * maxq);
        PB_ENSURE(sskip, sizeof(uint2) * maxq * nl);
        if (nal > 0) {
            PB_ENSURE(aq, sizeof(QRay) * maxq * nal);
            PB_ENSURE(aq_slot, sizeof(int) * maxq * nal);
            PB_ENSURE(aq_skip, sizeof(uint2) * maxq * nal);
        }
        if (rad) {
            PB_ENSURE(rq, sizeof(RadQuery) * maxq);
            PB_ENSURE(rq_amb, sizeof(float4) * maxq);
        }
        if (sample_rays) {
            PB_ENSURE(quality, sizeof(float) * maxq);
            PB_ENSURE(first_t, sizeof(float) * maxq);
        }
        if (binned) {
            PB_ENSURE(bin_keys, maxq);
            PB_ENSURE(bin_hist, sizeof(int) * 2 * SHADE_BINS);
            PB_ENSURE(bin_order, sizeof(int) * maxq);
        }
        if (media_ni > 0) {
            PB_ENSURE(stateA, sizeof(int) * maxq);
            PB_ENSURE(stateB, sizeof(int) * maxq);
            PB_ENSURE(smedium, sizeof(int) * maxq * nl);
            PB_ENSURE(mlist, sizeof(int) * maxq);
            PB_ENSURE(mte, sizeof(float4) * maxq * media_ni);
            PB_ENSURE(mod, sizeof(float4) * maxq * media_ni);
        }
        if (tori) {
            PB_ENSURE(tcand, sizeof(uint2) * tcand_cap(maxq, nl));
            PB_ENSURE(tkey, sizeof(unsigned long long) * maxq);
        }
        if (torus_free)
            PB_ENSURE(tovf, sizeof(int) * maxq * nl);
        if (transparent) {
            PB_ENSURE(stateA, sizeof(int) * maxq);
            PB_ENSURE(stateB, sizeof(int) * maxq);
            PB_ENSURE(rinA, sizeof(uint64_t) * maxq);
            PB_ENSURE(rinB, sizeof(uint64_t) * maxq);
            PB_ENSURE(srin, sizeof(uint64_t) * maxq * nl);
        }
#undef PB_ENSURE
        return cudaSuccess;
    }
    void release()
    {
        DevBuf* all[] = {&qA, &qB, &pathA, &pathB, &hits, &paths, &slot_contrib, &sq, &sq_slot, &blocked, &skipA,
                         &skipB, &sskip, &aq, &aq_slot, &aq_skip, &rq, &rq_amb, &quality, &first_t, &stateA,
                         &stateB, &smedium, &mlist, &mte, &mod, &mcbuf, &mrounds, &bin_keys, &bin_hist,
                         &bin_order, &rinA, &rinB, &srin, &thrA, &thrB, &tcand, &tkey, &tovf, &counters};
        for (DevBuf* b : all)
            b->release();
    }

    // Transparent surfaces that reflect (a ray may queue two): the per-pass
    // scratch for `n` current rays, which holds nothing between passes --
    // the hits, light slots, shadow rays, shade bins, torus lists.
    cudaError_t ensure_work(size_t n, int nl, bool binned, bool tori, bool torus_free)
    {
        n = std::max<size_t>(n, 1);
        nl = std::max(nl, 1);
        cudaError_t e;
#define PB_ENSURE(buf, bytes) if ((e = (buf).ensure(bytes)) != cudaSuccess) return e
        PB_ENSURE(hits, sizeof(QHit) * n);
        PB_ENSURE(slot_contrib, sizeof(float4) * n * nl);
        PB_ENSURE(sq, sizeof(QRay) * n * nl);
        PB_ENSURE(sq_slot, sizeof(int) * n * nl);
        PB_ENSURE(blocked, (n * nl + 3) & ~(size_t)3);
        PB_ENSURE(sskip, sizeof(uint2) * n * nl);
        PB_ENSURE(srin, sizeof(uint64_t) * n * nl);
        if (binned) {
            PB_ENSURE(bin_keys, n);
            PB_ENSURE(bin_order, sizeof(int) * n);
        }
        if (tori) {
            PB_ENSURE(tcand, sizeof(uint2) * tcand_cap(n, nl));
            PB_ENSURE(tkey, sizeof(unsigned long long) * n);
        }
        if (torus_free)
            PB_ENSURE(tovf, sizeof(int) * n * nl);
        return cudaSuccess;
    }
    // One side's queue arrays (A or B) for `n` rays; called only while
    // that side is empty (the next queue, before the pass fills it).
    cudaError_t ensure_side(int side, size_t n)
    {
        n = std::max<size_t>(n, 1);
        cudaError_t e;
        PB_ENSURE(side ? qB : qA, sizeof(QRay) * n);
        PB_ENSURE(side ? pathB : pathA, sizeof(int) * n);
        PB_ENSURE(side ? skipB : skipA, sizeof(uint2) * n);
        PB_ENSURE(side ? stateB : stateA, sizeof(int) * n);
        PB_ENSURE(side ? rinB : rinA, sizeof(uint64_t) * n);
        PB_ENSURE(side ? thrB : thrA, sizeof(float4) * n);
#undef PB_ENSURE
        return cudaSuccess;
    }
};

// Buffers of one radiosity bounce depth: the open / waiting / seed query
// lists of the rounds, each query's partial cache sums and answer, the
// round's cell claims, and the wavefront of the depth's sample rays.
struct RadLevel {
    DevBuf open, next, seeds, partial, claims, counts;
    PathBufs rays;
    cudaError_t ensure(size_t nq)
    {
        nq = std::max<size_t>(nq, 1);
        cudaError_t e;
        if ((e = open.ensure(sizeof(int) * nq)) != cudaSuccess) return e;
        if ((e = next.ensure(sizeof(int) * nq)) != cudaSuccess) return e;
        if ((e = seeds.ensure(sizeof(int) * nq)) != cudaSuccess) return e;
        if ((e = partial.ensure(sizeof(float4) * nq)) != cudaSuccess) return e;
        size_t slots = 64;
        while (slots < 2 * nq)
            slots *= 2;
        if ((e = claims.ensure(sizeof(unsigned long long) * slots)) != cudaSuccess) return e;
        return counts.ensure(sizeof(int) * 4);
    }
    uint32_t claim_mask() const
    {
        size_t slots = claims.bytes / sizeof(unsigned long long);
        size_t p = 64;
        while (p * 2 <= slots)
            p *= 2;
        return (uint32_t)(p - 1);
    }
    void release()
    {
        open.release(); next.release(); seeds.release(); partial.release(); claims.release(); counts.release();
        rays.release();
    }
};

constexpr size_t GATHER_CHUNK_RAYS = 1u << 20;   // sample rays in flight per depth
constexpr int RAD_ROUNDS = 8;                    // query rounds before every open query gathers

}  // namespace

// Radiosity state of a scene: settings, the device sample cache, and the
// running position of each bounce depth's direction sequence.
struct RadiosityState {
    bool            enabled = false;
    PovGpuRadiosity set{};
    DevBuf          blocks, quick, bslot, members, count, keys, seg_off, seg_cnt, seg_cur, range, occupancy, rstats;
    bool            seg_dirty = false;   // blocks added since the node segments were rebuilt
    int             cap_blocks = 0;
    uint32_t        key_mask = 0;
    bool            dirs_uploaded = false;
    int             dir_base[RAD_LEVELS] = {0, 0, 0, 0};
    bool            final_trace = true;
    double          error_bound = 0.0;
    uint64_t        rays_shot = 0;
    std::vector<double> jitter;
    std::vector<RadBlock> loaded;   // samples of a loaded cache file, in every frame's cache from its start
    RadLevel        level[RAD_LEVELS];
    // neural irradiance cache: configuration, parameters (FP32 master, BF16
    // copy, Adam moments, gradient), training batches, and whether the last
    // training passed its held-out gate
    PovGpuNeuralCache nic_cfg{};
    bool            nic_ok = false;
    double          nic_val_error = 0.0;
    float3          nic_lo{}, nic_scale{};
    bool            nic_init = false;   // shared network: weights, moments and bounds in place
    int             nic_step = 0;       // Adam steps taken by the shared network
    DevBuf          nic_params, nic_wb, nic_m, nic_v, nic_grad, nic_loss, nic_idx, nic_pred, nic_err;
    void release()
    {
        DevBuf* all[] = {&blocks, &quick, &bslot, &members, &count, &keys, &seg_off, &seg_cnt, &seg_cur, &range,
                         &occupancy, &rstats, &nic_params, &nic_wb, &nic_m,
                         &nic_v, &nic_grad, &nic_loss, &nic_idx, &nic_pred, &nic_err};
        for (DevBuf* b : all)
            b->release();
        for (auto& l : level)
            l.release();
    }
};


struct PovGpuScene {
    std::mutex  lock;
    int         device = 0;
    cudaStream_t stream = nullptr;
    DeviceScene S{};
    int         stack_depth = 32;
    int         num_sms = 148;
    // persistent scene data
    DevBuf nodes, refs, tri_v0, tri_e1, tri_e2, tri_global, tri_shade, tri_normal, tri_local, normals;
    DevBuf spheres, spheres64, boxes64, sphere_obj, sphere_flags, planes, plane_obj, boxes, tori, tori32, csgs, csg_children, objects,
        materials, lights, medias, patterns, tnormals, noise_hash, noise_rtab, noise_perm, noise_grad, noise_waves,
        noise_prand;
    DevBuf encode_buf;     // staging of pov_gpu_encode_u8 for host outputs
    DevBuf cam_tab;        // per-call column / row offsets of the camera rays
    PovGpuLaunchConfig lc{8, 128, 0, 16, 0, {0, 0, 0}};   // launch shapes (pov_gpu_set_launch_config)
    // the device work of a plain frame (no radiosity, media or AA) as a
    // captured CUDA graph, replayed while the frame's shape stays the same
    struct GraphKey {
        int n, nblocks, width, height;
        const void* out;
        const void* bufs[16];
        PovGpuLaunchConfig lc;
        DeviceScene S;
    };
    GraphKey graph_key{}, graph_last{};
    bool graph_last_valid = false;
    cudaGraphExec_t graph_exec = nullptr;
    uint32_t graph_launches = 0;   // kernels in the graph
    bool   textured = false;   // some material has a pattern pigment or a normal: bin the shade queue
    bool   transparent = false;   // some surface filters or transmits: rays carry interior lists
    bool   branching = false;     // some such surface also reflects: a hit may queue two rays
    bool   top_tori = false;      // tori outside CSG: traversal defers their FP64 tests
    bool   csg_torus = false;     // a CSG has a torus child: no torus-free traversal variant
    // bounding trees: the library's binned-SAH tree (nodes, refs) and, on
    // request, the reference's (ref_nodes, ref_refs, built from ref_input)
    int32_t sah_root = BVH_EMPTY;
    int     sah_stack_depth = 8, sah_depth = 0, sah_nodes = 0;
    int     tree_mode = 0;        // 0 SAH, 1 the reference's tree
    bool    ref_built = false;
    RefTreeInput  ref_input;
    RefTreeOutput ref_output;
    DevBuf ref_nodes, ref_refs;
    DevBuf obj_interior, interiors;   // per object its interior id; per interior its float4 pair
    int    media_ni = 0;   // interval slots per media segment (0: no media containers)
    int    media_smax = 0;  // sample slots per interval (ends + sample-tree nodes)
    int    media_sub = 0;   // largest sub-interval count
    int    media_levels = 0;   // largest AA_Level
    int    media_stamp = 0;    // marks the slots a chunk's samples fill
    std::vector<int32_t> h_containers;   // the media containers' object ids
    std::vector<PovGpuObject> h_objects; // the scene's objects (the camera-inside tests of set_camera)
    // host copies of the id maps (prim -> flattened object id)
    std::vector<int32_t> h_sphere_obj, h_plane_obj, h_box_obj, h_torus_obj, h_tri_global, h_tri_local, h_tri_obj;
    std::vector<DevCsg> h_csgs;
    std::vector<DevCsgChild> h_csg_children;
    // per-batch work buffers (grown on demand, reused); qA, hits, rays_in
    // and t64 serve pov_gpu_trace_rays
    DevBuf blocks, block_off, corner_off, qA, hits, out, counters, stats, err, rays_in, t64;
    // the camera wavefront
    PathBufs top;
    // radiosity cache and buffers
    RadiosityState rad;
    // adaptive antialiasing buffers
    DevBuf corners, aa_grid, aa_mask, aa_subdiv, aa_xy, cellsA, cellsB, spos, sslot;
    DevBuf pos_count;   // explicit sample positions in spos (radiosity pretrace)
    int     num_lights = 0;
    int     max_trace_level = 1;
    // streams and profiling
    cudaStream_t user_stream = nullptr;
    int          profiling = 0;
    PovGpuTimings timings{};
    std::vector<cudaEvent_t> events;   // pool, created on first profiled call
    DevBuf       wcount;

    cudaStream_t active() const { return user_stream ? user_stream : stream; }
    // host wait limit of a call (pov_gpu_set_timeout; 0 = wait as long as
    // the work takes), the current call's deadline, and whether work of a
    // call that gave up is still on the stream
    double       timeout_s = 0.0;
    std::chrono::steady_clock::time_point deadline{};
    bool         pending = false;
    cudaEvent_t  wait_event = nullptr;
    // pinned host words the host reads device counts and statistics into:
    // a copy into pageable memory would block the host until the device is
    // done, without the wait limit
    unsigned char* pinned = nullptr;
    static constexpr size_t PIN_BYTES = 4096, PIN_ERR = 256, PIN_STATS = 512, PIN_WORK = 1536;
    int* pin_int(int k) { return reinterpret_cast<int*>(pinned) + k; }

    void release_all()
    {
        for (cudaEvent_t e : events)
            cudaEventDestroy(e);
        events.clear();
        if (wait_event)
            cudaEventDestroy(wait_event);
        wait_event = nullptr;
        if (pinned)
            cudaFreeHost(pinned);
        pinned = nullptr;
        if (graph_exec)
            cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
        DevBuf* all[] = {&nodes, &refs, &tri_v0, &tri_e1, &tri_e2, &tri_global, &tri_shade, &tri_normal, &tri_local,
                         &normals, &spheres, &spheres64, &boxes64, &sphere_obj, &sphere_flags, &planes, &plane_obj, &boxes, &tori, &tori32, &csgs,
                         &csg_children, &objects, &materials, &lights, &blocks, &block_off, &corner_off, &qA,
                         &hits, &out, &counters, &stats, &err, &rays_in, &t64, &corners, &aa_grid, &aa_mask,
                         &aa_subdiv, &aa_xy, &cellsA, &cellsB, &spos, &sslot, &wcount, &pos_count, &medias,
                         &encode_buf, &cam_tab, &patterns, &tnormals, &noise_hash, &noise_rtab, &noise_perm, &noise_grad,
                         &noise_waves, &noise_prand, &obj_interior, &interiors, &ref_nodes, &ref_refs};
        for (DevBuf* b : all)
            b->release();
        top.release();
        rad.release();
        if (stream)
            cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

namespace {

#define CK(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess)                                                         \
            return e_ == cudaErrorMemoryAllocation ? POV_GPU_E_NOMEM : POV_GPU_E_CUDA; \
    } while (0)

// The host's wait for the work queued on the scene's stream.  Without a
// limit: cudaStreamSynchronize.  With one (pov_gpu_set_timeout): an event
// recorded behind the work is polled until it completes or the call's
// deadline passes; then the scene is marked pending (its work still runs
// and still owns the scene's buffers and the call's output) and the call
// returns POV_GPU_E_TIMEOUT.
int host_wait(PovGpuScene* sc, cudaStream_t st)
{
    if (sc->timeout_s <= 0.0) {
        CK(cudaStreamSynchronize(st));
        sc->pending = false;
        return POV_GPU_OK;
    }
    if (!sc->wait_event)
        CK(cudaEventCreateWithFlags(&sc->wait_event, cudaEventDisableTiming));
    CK(cudaEventRecord(sc->wait_event, st));
    for (;;) {
        cudaError_t q = cudaEventQuery(sc->wait_event);
        if (q == cudaSuccess) {
            sc->pending = false;
            return POV_GPU_OK;
        }
        if (q != cudaErrorNotReady)
            CK(q);
        if (std::chrono::steady_clock::now() >= sc->deadline) {
            sc->pending = true;
            return POV_GPU_E_TIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

#define HW(st)                                      \
    do {                                            \
        if (int hw_ = host_wait(sc, (st)))          \
            return hw_;                             \
    } while (0)

// Start of a call that queues work: its deadline, and the wait for work a
// call before it left on the stream when it gave up.
int begin_call(PovGpuScene* sc)
{
    sc->deadline = std::chrono::steady_clock::now() +
                   std::chrono::microseconds((long long)(sc->timeout_s * 1e6));
    if (sc->pending)
        return host_wait(sc, sc->active());
    return POV_GPU_OK;
}

constexpr int TRANSPARENT_PASSES_PER_LEVEL = 64;   // surfaces a ray crosses straight on at one trace level
constexpr int MAX_AA_DEPTH = 4;   // (2^4+1)^2 = 289 grid points, 21 subdividable cells per pixel

bool is_csg(int t) { return t == POV_OBJ_UNION || t == POV_OBJ_INTERSECTION || t == POV_OBJ_MERGE; }

// Media container: a hollow object holding media (validated to be a
// top-level box whose surface only transmits).
bool is_container(const PovGpuObject& o) { return o.media > 0 && (o.flags & POV_FLAG_HOLLOW); }

// Media containers as the GPU path restates them: hollow top-level boxes
// without transform whose surface only transmits (pigment transmit 1, no
// finish terms), each holding one constant isotropic media sampled by
// method 3 without jitter (Min_Samples = Max_Samples), the camera outside,
// point lights only; no other surface transmits.  Marks the materials the
// containers use in `cmat`.
bool host_inside(const PovGpuSceneDesc* d, int i, const double* P);

int validate_media(const PovGpuSceneDesc* d, std::vector<char>& cmat, int32_t* bad)
{
    cmat.assign((size_t)d->num_materials, 0);
    int containers = 0;
    for (int i = 0; i < d->num_objects; i++) {
        const PovGpuObject& o = d->objects[i];
        if (o.media < 0 || o.media > d->num_medias || (o.media > 0 && !d->medias))
            return POV_GPU_E_INVALID;
        const PovGpuMaterial* m =
            (o.material >= 0 && o.material < d->num_materials) ? &d->materials[o.material] : nullptr;
        if (o.media == 0)
            continue;   // a transparent surface outside containers: validate_transparency
        if (bad) *bad = i;
        const PovGpuMedia* md = o.media > 0 ? &d->medias[o.media - 1] : nullptr;
        if (!md || (o.type != POV_OBJ_BOX && o.type != POV_OBJ_SPHERE) || (o.flags & POV_FLAG_INVERTED) ||
            !(o.flags & POV_FLAG_HOLLOW) || o.parent >= 0 || !m ||
            m->pigment[3] != 0.0f || m->pigment[4] != 1.0f || m->diffuse != 0.0f || m->phong != 0.0f ||
            m->specular != 0.0f || m->emission[0] != 0.0f || m->emission[1] != 0.0f || m->emission[2] != 0.0f ||
            m->ambient[0] != 0.0f || m->ambient[1] != 0.0f || m->ambient[2] != 0.0f ||
            m->reflection_max[0] != 0.0f || m->reflection_max[1] != 0.0f || m->reflection_max[2] != 0.0f ||
            md->method != 3 || md->jitter != 0.0f || md->scattering_type < 1 || md->scattering_type > 5 ||
            md->min_samples != md->max_samples ||
            md->min_samples < 1 || md->aa_level < 1 || md->aa_level > MEDIA_MAX_AA_LEVEL || md->intervals < 1 ||
            md->intervals > MEDIA_MAX_INTERVALS || containers >= MAX_CONTAINERS)
            return POV_GPU_E_UNSUPPORTED;
        if (host_inside(d, i, d->camera.location))
            return POV_GPU_E_UNSUPPORTED;   // camera rays would start inside the media
        cmat[o.material] = 1;
        containers++;
    }
    if (bad) *bad = -1;
    if (containers > 0 && d->max_trace_level > 255)
        return POV_GPU_E_UNSUPPORTED;   // a ray's level is held in 8 bits of its state
    for (int i = 0; containers > 0 && i < d->num_lights; i++) {
        const PovGpuLight& L = d->lights[i];
        if (L.kind != POV_LIGHT_POINT || L.light_type > POV_LIGHT_TYPE_POINT || L.parallel || L.fade_power > 0.0)
            return POV_GPU_E_UNSUPPORTED;   // media samples test plain point-light shadows only
    }
    return POV_GPU_OK;
}

// Object::Inside in FP64 for the camera test below (sphere.cpp:333-382,
// box.cpp:535-598, plane.cpp:213-258, torus.cpp:364-385, csg.cpp:405-484);
// a mesh is solid only with an inside_vector, which the GPU path does not
// take, so it contains no point.
bool host_inside(const PovGpuSceneDesc* d, int i, const double* P)
{
    const PovGpuObject& o = d->objects[i];
    const bool inv = (o.flags & POV_FLAG_INVERTED) != 0;
    switch (o.type) {
    case POV_OBJ_SPHERE: {
        double dd = 0.0;
        for (int k = 0; k < 3; k++)
            dd += (o.p[k] - P[k]) * (o.p[k] - P[k]);
        return inv ? dd > o.p[3] * o.p[3] : dd < o.p[3] * o.p[3];
    }
    case POV_OBJ_BOX: {
        bool in = true;
        for (int k = 0; k < 3; k++)
            in = in && P[k] >= std::min(o.p[k], o.p[3 + k]) && P[k] <= std::max(o.p[k], o.p[3 + k]);
        return inv ? !in : in;
    }
    case POV_OBJ_PLANE:
        return (P[0] * o.p[0] + P[1] * o.p[1] + P[2] * o.p[2] + o.p[3]) < EPSILON;
    case POV_OBJ_TORUS: {
        const double* m = o.trans + 16;
        double q[3];
        for (int k = 0; k < 3; k++)
            q[k] = P[0] * m[k] + P[1] * m[4 + k] + P[2] * m[8 + k] + m[12 + k];
        const double r = std::sqrt(q[0] * q[0] + q[2] * q[2]);
        const bool in = q[1] * q[1] + (r - o.p[0]) * (r - o.p[0]) <= o.p[1] * o.p[1];
        return inv ? !in : in;
    }
    case POV_OBJ_UNION:
    case POV_OBJ_MERGE:
        for (int c = 0; c < o.num_children; c++)
            if (host_inside(d, o.first_child + c, P))
                return true;
        return false;
    case POV_OBJ_INTERSECTION:
        for (int c = 0; c < o.num_children; c++)
            if (!host_inside(d, o.first_child + c, P))
                return false;
        return true;
    default:
        return false;
    }
}

// Transparent surfaces (a plain pigment that filters or transmits, outside
// media containers) as the GPU path restates them: every hit continues into
// at most one ray, so a transparent material reflects nothing (its
// transmitted or refracted ray is the one; total internal reflection takes
// its place); interiors without dispersion or caustics; no media
// containers, radiosity or area lights beside them; the camera inside no
// object (its rays start with an empty interior list); a ray inside at most
// RIN_MAX interiors (checked on the device).  Sets *transparent.
bool material_transparent(const PovGpuSceneDesc* d, const PovGpuMaterial& m);

int validate_transparency(const PovGpuSceneDesc* d, const std::vector<char>& cmat, bool* transparent,
                          int32_t* bad)
{
    *transparent = false;
    for (int i = 0; i < d->num_materials; i++) {
        const PovGpuMaterial& m = d->materials[i];
        if (cmat[i] || !material_transparent(d, m))
            continue;
        *transparent = true;
    }
    if (d->num_interiors < 0 || (d->num_interiors > 0 && !d->interiors))
        return POV_GPU_E_INVALID;
    if (d->object_interior)
        for (int i = 0; i < d->num_objects; i++)
            if (d->object_interior[i] < 0 || d->object_interior[i] > d->num_interiors)
                return POV_GPU_E_INVALID;
    if (!*transparent)
        return POV_GPU_OK;
    for (char c : cmat)
        if (c)
            return POV_GPU_E_UNSUPPORTED;
    if (d->radiosity.enabled || d->max_trace_level > 255)
        return POV_GPU_E_UNSUPPORTED;
    for (int i = 0; i < d->num_lights; i++)
        if (d->lights[i].kind != POV_LIGHT_POINT)
            return POV_GPU_E_UNSUPPORTED;
    for (int i = 0; i < d->num_interiors; i++)
        if (d->interiors[i].dispersion != 1.0 || d->interiors[i].caustics != 0.0 || !(d->interiors[i].ior > 0.0))
            return POV_GPU_E_UNSUPPORTED;
    for (int i = 0; i < d->num_objects; i++)
        if (d->objects[i].parent < 0 && host_inside(d, i, d->camera.location)) {
            if (bad) *bad = i;
            return POV_GPU_E_UNSUPPORTED;
        }
    return POV_GPU_OK;
}

int validate(const PovGpuSceneDesc* d, int32_t* bad)
{
    if (!d || d->abi_version != POV_GPU_ABI_VERSION || d->num_objects < 0 || d->num_materials < 1 ||
        d->num_lights < 0 || d->num_meshes < 0 || (d->num_objects > 0 && !d->objects) || !d->materials ||
        (d->num_lights > 0 && !d->lights) || (d->num_meshes > 0 && !d->meshes))
        return POV_GPU_E_INVALID;
    if (d->camera.type != 0)
        return POV_GPU_E_UNSUPPORTED;
    if (d->radiosity.enabled) {
        // radiosity{} as the GPU path restates it: default normal/media off,
        // bounce depths within the buffer levels, sensible counts
        const PovGpuRadiosity& r = d->radiosity;
        if (r.count < 1 || r.nearest_count < 1 || r.recursion_limit < 1 || r.error_bound <= 0.0 ||
            r.pretrace_start <= 0.0 || r.pretrace_end <= 0.0 || r.pretrace_end > r.pretrace_start)
            return POV_GPU_E_INVALID;
        if (r.recursion_limit > RAD_LEVELS || r.normal || r.media)
            return POV_GPU_E_UNSUPPORTED;
    }
    for (int i = 0; i < d->num_lights; i++) {
        const PovGpuLight& L = d->lights[i];
        if ((L.kind != POV_LIGHT_POINT && L.kind != POV_LIGHT_AREA) || L.light_type < 0 ||
            L.light_type > POV_LIGHT_TYPE_CYLINDER)
            return POV_GPU_E_INVALID;
        // a beam (spot, cylinder, parallel) needs its direction; area lights
        // take no parallel beams
        const double dx = L.points_at[0] - L.center[0], dy = L.points_at[1] - L.center[1],
                     dz = L.points_at[2] - L.center[2];
        const bool beam = L.light_type == POV_LIGHT_TYPE_SPOT || L.light_type == POV_LIGHT_TYPE_CYLINDER || L.parallel;
        if (beam && !(std::sqrt(dx * dx + dy * dy + dz * dz) > 1.0e-10))
            return POV_GPU_E_UNSUPPORTED;
        if (L.kind == POV_LIGHT_AREA && (L.parallel || L.light_type == POV_LIGHT_TYPE_CYLINDER))
            return POV_GPU_E_UNSUPPORTED;
        // area lights: the grid fits the per-point visibility masks; jitter
        // draws on the reference's random stream and is not restated
        if (L.kind == POV_LIGHT_AREA &&
            (L.area_size1 < 1 || L.area_size2 < 1 || L.area_size1 * L.area_size2 > AREA_MAX_POINTS ||
             L.jitter || (L.circular && (L.area_size1 < 2 || L.area_size2 < 2))))
            return POV_GPU_E_UNSUPPORTED;
    }
    std::vector<char> cmat;
    {
        int rc = validate_media(d, cmat, bad);
        if (rc != POV_GPU_OK)
            return rc;
        bool transparent = false;
        rc = validate_transparency(d, cmat, &transparent, bad);
        if (rc != POV_GPU_OK)
            return rc;
    }
    // patterns: the nine pigment patterns and the three normal-only ones,
    // 0..16 ascending colour map entries, noise generators 1..3, the six
    // waves, 1..32 octaves; a pigment reads one of the nine with 1..16
    // entries (checker: 2), a normal any but checker (whose normal form is a
    // normal map), with a positive delta
    if (d->num_patterns < 0 || (d->num_patterns > 0 && !d->patterns))
        return POV_GPU_E_INVALID;
    for (int i = 0; i < d->num_patterns; i++) {
        const PovGpuPattern& pt = d->patterns[i];
        if (pt.type < POV_PATTERN_CHECKER || pt.type > POV_PATTERN_QUILTED || pt.num_entries < 0 ||
            (pt.type == POV_PATTERN_CRACKLE && !(pt.crackle_metric > 0.0)) ||
            pt.num_entries > POV_PATTERN_MAX_ENTRIES || pt.noise_generator < 1 || pt.noise_generator > 3 ||
            pt.wave_type < POV_WAVE_RAMP || pt.wave_type > POV_WAVE_POLY || pt.octaves < 1 || pt.octaves > 32 ||
            (pt.type == POV_PATTERN_CHECKER && pt.num_entries != 2) ||
            (pt.type == POV_PATTERN_SQUARE && pt.num_entries != 4) ||
            ((pt.type == POV_PATTERN_TRIANGULAR || pt.type == POV_PATTERN_CUBIC) && pt.num_entries != 6) ||
            (pt.type == POV_PATTERN_HEXAGON && pt.num_entries != 3) ||
            (pt.type == POV_PATTERN_BRICK && (pt.num_entries != 2 || !(pt.brick_size[0] > 0.0) ||
                                              !(pt.brick_size[1] > 0.0) || !(pt.brick_size[2] > 0.0))))
            return POV_GPU_E_UNSUPPORTED;
        for (int k = 1; k < pt.num_entries; k++)
            if (pt.values[k] < pt.values[k - 1])
                return POV_GPU_E_INVALID;
    }
    if (d->num_normals < 0 || (d->num_normals > 0 && !d->normals))
        return POV_GPU_E_INVALID;
    for (int i = 0; i < d->num_normals; i++) {
        const PovGpuNormal& nm = d->normals[i];
        if (nm.pattern < 1 || nm.pattern > d->num_patterns)
            return POV_GPU_E_INVALID;
        const int nt = d->patterns[nm.pattern - 1].type;
        // the discrete patterns' normal forms are normal maps (not built)
        const bool discrete = nt == POV_PATTERN_CHECKER || (nt >= POV_PATTERN_SQUARE && nt <= POV_PATTERN_BRICK) ||
                              nt == POV_PATTERN_QUILTED;   // quilted's normal is its own function
        if (discrete || !(nm.delta > 0.0f) || !std::isfinite(nm.amount))
            return POV_GPU_E_UNSUPPORTED;
    }
    for (int i = 0; i < d->num_materials; i++) {
        const PovGpuMaterial& m = d->materials[i];
        if (m.pattern < 0 || m.pattern > d->num_patterns || m.normal < 0 || m.normal > d->num_normals)
            return POV_GPU_E_INVALID;
        if (m.pattern > 0) {
            const PovGpuPattern& pt = d->patterns[m.pattern - 1];
            if (pt.type == POV_PATTERN_BUMPS || pt.num_entries < 1 ||
                (pt.type == POV_PATTERN_CHECKER && pt.num_entries != 2))
                return POV_GPU_E_UNSUPPORTED;
        }
    }
    for (int i = 0; i < d->num_materials; i++) {
        const PovGpuMaterial& m = d->materials[i];
        // the classic finish terms; fresnel reflection and conserve_energy
        // on transparent surfaces only, whose interiors the device holds
        // (transparency: validate_transparency)
        const bool see = material_transparent(d, m);
        if (m.fresnel != 0.0f || m.reflect_exp != 1.0f ||
            m.irid != 0.0f || m.crand != 0.0f || (m.diffuse_back != 0.0f && d->radiosity.enabled) ||
            ((m.reflection_fresnel || m.conserve_energy) && !see))
            return POV_GPU_E_UNSUPPORTED;
    }
    const int n = d->num_objects;
    for (int i = 0; i < n; i++) {
        const PovGpuObject& o = d->objects[i];
        if (bad) *bad = i;
        if (o.type < POV_OBJ_SPHERE || o.type > POV_OBJ_MERGE || o.parent >= n || o.parent >= i)
            return POV_GPU_E_INVALID;
        if (o.material >= d->num_materials || (o.material < 0 && o.parent < 0))
            return POV_GPU_E_INVALID;
        if (o.type == POV_OBJ_MESH && (o.mesh < 0 || o.mesh >= d->num_meshes))
            return POV_GPU_E_INVALID;
        // transforms: the torus always has one; sphere (ellipsoid), box, mesh
        // and plane transforms are not on the GPU path
        if (o.type == POV_OBJ_TORUS ? !(o.flags & POV_FLAG_HAS_TRANS) : (o.flags & POV_FLAG_HAS_TRANS) != 0)
            return POV_GPU_E_UNSUPPORTED;
        // no_shadow, no_reflection and no_image (the ray-kind object tests of
        // FindIntersection's preconditions, trace.cpp:1943-1950) are not on
        // the GPU path: refused rather than rendered as if absent
        if (o.flags & (POV_FLAG_NO_SHADOW | POV_FLAG_NO_REFLECTION | POV_FLAG_NO_IMAGE))
            return POV_GPU_E_UNSUPPORTED;
        if (is_csg(o.type)) {
            if (o.parent >= 0)
                return POV_GPU_E_UNSUPPORTED;   // nested CSG
            if (o.num_children < 1 || o.first_child != i + 1 || o.first_child + o.num_children > n)
                return POV_GPU_E_INVALID;
            for (int c = 0; c < o.num_children; c++) {
                const PovGpuObject& ch = d->objects[o.first_child + c];
                if (ch.parent != i)
                    return POV_GPU_E_INVALID;
                // leaf children: spheres, boxes and tori (no planes, meshes or nested CSG)
                if (ch.type != POV_OBJ_SPHERE && ch.type != POV_OBJ_BOX && ch.type != POV_OBJ_TORUS) {
                    if (bad) *bad = o.first_child + c;
                    return POV_GPU_E_UNSUPPORTED;
                }
            }
        } else if (o.parent >= 0 && !is_csg(d->objects[o.parent].type)) {
            return POV_GPU_E_INVALID;
        }
    }
    if (bad) *bad = -1;
    for (int i = 0; i < d->num_meshes; i++) {
        const PovGpuMesh& m = d->meshes[i];
        if (m.num_triangles < 0 || m.num_vertices < 0 || (m.num_triangles > 0 && (!m.face_indices || !m.vertices)))
            return POV_GPU_E_INVALID;
        for (int t = 0; t < 3 * m.num_triangles; t++) {
            if (m.face_indices[t] < 0 || m.face_indices[t] >= m.num_vertices)
                return POV_GPU_E_INVALID;
            if (m.normal_indices && (m.normal_indices[t] < 0 || m.normal_indices[t] >= m.num_normals))
                return POV_GPU_E_INVALID;
        }
    }
    return POV_GPU_OK;
}

// A material that can filter or transmit: its plain pigment does, or (with
// a pattern) an entry of the colour map does (Post_Pigment's HAS_FILTER).
bool material_transparent(const PovGpuSceneDesc* d, const PovGpuMaterial& m)
{
    if (m.pattern > 0 && m.pattern <= d->num_patterns && d->patterns) {
        const PovGpuPattern& pt = d->patterns[m.pattern - 1];
        for (int k = 0; k < pt.num_entries && k < POV_PATTERN_MAX_ENTRIES; k++)
            if (pt.filters[k] != 0.0f || pt.transmits[k] != 0.0f)
                return true;
        return false;
    }
    return m.pigment[3] != 0.0f || m.pigment[4] != 0.0f;
}

DevMaterial make_material(const PovGpuMaterial& m, const float* ambient_light, bool radiosity, int language_version)
{
    DevMaterial d{};
    d.pigment = make_float4(m.pigment[0], m.pigment[1], m.pigment[2], m.pigment[3]);
    // emission, plus ambient * ambient_light unless radiosity replaces the
    // ambient term (trace.cpp:982-987)
    const float a = radiosity ? 0.0f : 1.0f;
    d.emission = make_float4(m.emission[0] + a * m.ambient[0] * ambient_light[0],
                             m.emission[1] + a * m.ambient[1] * ambient_light[1],
                             m.emission[2] + a * m.ambient[2] * ambient_light[2], 0.f);
    float wmax = std::max(m.reflection_max[0], std::max(m.reflection_max[1], m.reflection_max[2]));
    float wmin = std::max(m.reflection_min[0], std::max(m.reflection_min[1], m.reflection_min[2]));
    d.reflect = make_float4(m.reflection_max[0], m.reflection_max[1], m.reflection_max[2], m.reflection_falloff);
    d.reflect_min = make_float4(m.reflection_min[0], m.reflection_min[1], m.reflection_min[2], std::max(wmax, wmin));
    d.diffuse = m.diffuse * m.brilliance_adjust;
    d.diffuse_back = m.diffuse_back * m.brilliance_adjust;
    d.metallic = m.metallic;
    d.reflect_metallic = m.reflect_metallic;
    d.brilliance = m.brilliance;
    d.phong = m.phong;
    d.phong_size = m.phong_size;
    d.specular = m.specular;
    d.roughness = m.roughness;
    bool anyr = false;
    for (int k = 0; k < 3; k++)
        anyr = anyr || m.reflection_max[k] != 0.f || m.reflection_min[k] != 0.f;
    d.reflect_flags = (anyr ? REFL_ANY : 0) | (m.reflection_fresnel ? REFL_FRESNEL : 0) |
                      (m.conserve_energy ? REFL_CONSERVE : 0);
    d.diffuse_raw = m.diffuse;
    d.pattern = m.pattern;
    d.normal = m.normal;
    d.transmit = m.pigment[4];
    d.see_through = (m.pigment[3] != 0.0f || m.pigment[4] != 0.0f) ? SEE_PLAIN : 0;
    // TransColour::Opacity (LegacyOpacity before 3.7), in the colour's float
    d.opacity = 1.0f;
    if (d.see_through)
        d.opacity = language_version < 370
                        ? (float)(1.0 - (m.pigment[3] * std::max(m.pigment[0], std::max(m.pigment[1], m.pigment[2])) +
                                         m.pigment[4]))
                        : (float)(1.0 - (double)m.pigment[3] - (double)m.pigment[4]);
    return d;
}

// Scene arrays under construction (host side).
struct Builder {
    BvhBuilder bvh;
    std::vector<float4> spheres, planes, tri_v0, tri_e1, tri_e2, tri_normal, normals;
    std::vector<double> spheres64, boxes64;
    std::vector<int32_t> sphere_obj, sphere_flags, plane_obj, tri_global, tri_local, box_obj, torus_obj;
    std::vector<int4> tri_shade;
    std::vector<DevBox> boxes;
    std::vector<DevTorus> tori;
    std::vector<DevCsg> csgs;
    std::vector<DevCsgChild> csg_children;
    // every primitive pushed, with the top-level object it belongs to (the
    // input of the reference's bounding tree)
    int32_t cur_obj = -1;
    std::vector<std::pair<int32_t, uint32_t>> pushed;

    int add_sphere(const PovGpuObject& o, int id, AABB* box)
    {
        int idx = (int)spheres.size();
        spheres.push_back(make_float4((float)o.p[0], (float)o.p[1], (float)o.p[2], (float)o.p[3]));
        spheres64.insert(spheres64.end(), {o.p[0], o.p[1], o.p[2], o.p[3]});
        sphere_obj.push_back(id);
        // bit 0 inverted; bit 1 (SPHERE_CONTAINER) the surface of a media container
        sphere_flags.push_back((o.flags & POV_FLAG_INVERTED ? 1 : 0) | (is_container(o) ? SPHERE_CONTAINER : 0));
        if (box)
            for (int k = 0; k < 3; k++) {
                box->lo[k] = std::min(box->lo[k], std::nextafter((float)(o.p[k] - o.p[3]), -INFINITY));
                box->hi[k] = std::max(box->hi[k], std::nextafter((float)(o.p[k] + o.p[3]), INFINITY));
            }
        return idx;
    }
    int add_box(const PovGpuObject& o, int id, AABB* box)
    {
        int idx = (int)boxes.size();
        DevBox b;
        b.lo = make_float4((float)o.p[0], (float)o.p[1], (float)o.p[2], __builtin_bit_cast(float, id));
        const int32_t bflags = (o.flags & POV_FLAG_INVERTED ? 1 : 0) | (is_container(o) ? BOX_CONTAINER : 0);
        b.hi = make_float4((float)o.p[3], (float)o.p[4], (float)o.p[5], __builtin_bit_cast(float, bflags));
        boxes.push_back(b);
        boxes64.insert(boxes64.end(), {o.p[0], o.p[1], o.p[2], o.p[3], o.p[4], o.p[5]});
        box_obj.push_back(id);
        if (box) {
            grow_outward(*box, o.p[0], o.p[1], o.p[2]);
            grow_outward(*box, o.p[3], o.p[4], o.p[5]);
        }
        return idx;
    }
    int add_torus(const PovGpuObject& o, int id, AABB* box)
    {
        int idx = (int)tori.size();
        DevTorus t{};
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 3; c++)
                t.inv[r * 3 + c] = o.trans[16 + r * 4 + c];
        t.R = o.p[0];
        t.r = o.p[1];
        t.object = id;
        t.flags = o.flags & POV_FLAG_INVERTED ? 1 : 0;
        tori.push_back(t);
        torus_obj.push_back(id);
        if (box) {
            // Torus::Compute_BBox + Recompute_BBox: the local box's corners, transformed
            double r1 = o.p[1], r2 = o.p[0] + o.p[1];
            for (int i = 0; i < 8; i++) {
                V3d c = {(i & 1) ? r2 : -r2, (i & 2) ? r1 : -r1, (i & 4) ? r2 : -r2};
                V3d w = mtrans_point(o.trans, c);
                double pad = 1e-6 * (std::fabs(w.x) + std::fabs(w.y) + std::fabs(w.z) + 1.0);
                grow_outward(*box, w.x - pad, w.y - pad, w.z - pad);
                grow_outward(*box, w.x + pad, w.y + pad, w.z + pad);
            }
        }
        return idx;
    }
    void push_prim(uint32_t kind, uint32_t idx, const AABB& box)
    {
        BuildItem it;
        it.box = box;
        for (int k = 0; k < 3; k++)
            it.c[k] = 0.5f * (box.lo[k] + box.hi[k]);
        it.ref = (kind << PRIM_KIND_SHIFT) | idx;
        it.cost = prim_cost(kind);
        bvh.items.push_back(it);
        pushed.push_back({cur_obj, it.ref});
    }
};

// Compute_BBox of a top-level object as the reference stores it (float
// lower-left and size): Sphere (sphere.cpp:646-658), Box (box.cpp:947-957),
// Torus with Recompute_BBox of its local box (torus.cpp:849-859,
// boundingbox.cpp:168), Mesh over its vertices (mesh.cpp:790-808), CSG as
// the union of its children or, for an intersection, the overlap of the
// children that are not inverted (csg.cpp).
RefBox ref_object_box(const PovGpuSceneDesc* d, int i)
{
    const PovGpuObject& o = d->objects[i];
    const double H = 2.0e10;   // BOUND_HUGE
    double mn[3] = {H, H, H}, mx[3] = {-H, -H, -H};
    RefBox b{};
    auto from = [&](const double* lo, const double* hi) {
        for (int k = 0; k < 3; k++) {
            b.ll[k] = (float)lo[k];
            b.sz[k] = (float)(hi[k] - lo[k]);
        }
    };
    switch (o.type) {
    case POV_OBJ_SPHERE:
        for (int k = 0; k < 3; k++) {
            b.ll[k] = (float)(o.p[k] - o.p[3]);
            b.sz[k] = (float)(2.0 * o.p[3]);
        }
        return b;
    case POV_OBJ_BOX:
        from(o.p, o.p + 3);
        return b;
    case POV_OBJ_TORUS: {
        const double r1 = o.p[1], r2 = o.p[0] + o.p[1];
        const float ll[3] = {(float)-r2, (float)-r1, (float)-r2};
        const float sz[3] = {(float)(2.0 * r2), (float)(2.0 * r1), (float)(2.0 * r2)};
        for (int c = 1; c <= 8; c++) {
            V3d p = {ll[0] + ((c & 1) ? (double)sz[0] : 0.0), ll[1] + ((c & 2) ? (double)sz[1] : 0.0),
                     ll[2] + ((c & 4) ? (double)sz[2] : 0.0)};
            V3d w = mtrans_point(o.trans, p);
            const double v[3] = {w.x, w.y, w.z};
            for (int k = 0; k < 3; k++) {
                mn[k] = std::min(mn[k], v[k]);
                mx[k] = std::max(mx[k], v[k]);
            }
        }
        from(mn, mx);
        return b;
    }
    case POV_OBJ_MESH: {
        const PovGpuMesh& m = d->meshes[o.mesh];
        for (int t = 0; t < 3 * m.num_triangles; t++) {
            const float* v = m.vertices + 3 * m.face_indices[t];
            for (int k = 0; k < 3; k++) {
                mn[k] = std::min(mn[k], (double)v[k]);
                mx[k] = std::max(mx[k], (double)v[k]);
            }
        }
        from(mn, mx);
        return b;
    }
    case POV_OBJ_UNION:
    case POV_OBJ_MERGE:
    case POV_OBJ_INTERSECTION: {
        const bool isect = o.type == POV_OBJ_INTERSECTION;
        if (isect)
            for (int k = 0; k < 3; k++) {
                mn[k] = -H;
                mx[k] = H;
            }
        for (int c = 0; c < o.num_children; c++) {
            const PovGpuObject& ch = d->objects[o.first_child + c];
            if (isect && (ch.flags & POV_FLAG_INVERTED))
                continue;
            const RefBox cb = ref_object_box(d, o.first_child + c);
            for (int k = 0; k < 3; k++) {
                const double lo = cb.ll[k], hi = (double)cb.ll[k] + cb.sz[k];
                mn[k] = isect ? std::max(mn[k], lo) : std::min(mn[k], lo);
                mx[k] = isect ? std::min(mx[k], hi) : std::max(mx[k], hi);
            }
        }
        from(mn, mx);
        return b;
    }
    default:
        return b;
    }
}

void add_mesh(Builder& B, const PovGpuSceneDesc* d, const PovGpuObject& o, int id, int nb)
{
    const PovGpuMesh& m = d->meshes[o.mesh];
    for (int t = 0; t < m.num_triangles; t++) {
        const int32_t* f = m.face_indices + 3 * t;
        int p1 = f[0], p2 = f[1], p3 = f[2];
        int n1 = 0, n2 = 0, n3 = 0;
        bool smooth = false;
        // without normal_indices the parser reuses the face indices when
        // there is one normal per vertex (parser.cpp:4488-4502)
        const int32_t* ni = m.normal_indices ? m.normal_indices
                            : (m.num_normals == m.num_vertices ? m.face_indices : nullptr);
        if (ni && m.num_normals > 0 && m.normals) {
            n1 = ni[3 * t];
            n2 = ni[3 * t + 1];
            n3 = ni[3 * t + 2];
            const float4 a = B.normals[nb + n1], b = B.normals[nb + n2], c = B.normals[nb + n3];
            double d1x = (double)a.x - b.x, d1y = (double)a.y - b.y, d1z = (double)a.z - b.z;
            double d2x = (double)a.x - c.x, d2y = (double)a.y - c.y, d2z = (double)a.z - c.z;
            double l1 = d1x * d1x + d1y * d1y + d1z * d1z, l2 = d2x * d2x + d2y * d2y + d2z * d2z;
            smooth = (std::fabs(l1) > EPSILON) || (std::fabs(l2) > EPSILON);   // parser.cpp:4545
        }
        auto V = [&](int k) {
            return V3d{(double)m.vertices[3 * k], (double)m.vertices[3 * k + 1], (double)m.vertices[3 * k + 2]};
        };
        V3d P1 = V(p1), P2 = V(p2), P3 = V(p3);
        // Compute_Mesh_Triangle (source/core/shape/mesh.cpp:838-982)
        V3d N = vcross(vsub(P3, P1), vsub(P2, P1));
        double len = vlen(N);
        float4 gn = make_float4(0.f, 0.f, 0.f, __builtin_bit_cast(float, id));
        float plane_dist = 0.f;
        if (len != 0.0) {
            N = {N.x / len, N.y / len, N.z / len};
            plane_dist = (float)(-(N.x * P1.x + N.y * P1.y + N.z * P1.z));   // Triangle->Distance
            gn.x = (float)N.x;
            gn.y = (float)N.y;
            gn.z = (float)N.z;
            int axis = max3_coordinate(std::fabs(N.x), std::fabs(N.y), std::fabs(N.z));
            bool swap;
            if (axis == 0)
                swap = (P2.y - P3.y) * (P2.z - P1.z) < (P2.z - P3.z) * (P2.y - P1.y);
            else if (axis == 1)
                swap = (P2.x - P3.x) * (P2.z - P1.z) < (P2.z - P3.z) * (P2.x - P1.x);
            else
                swap = (P2.x - P3.x) * (P2.y - P1.y) < (P2.y - P3.y) * (P2.x - P1.x);
            if (swap) {
                std::swap(p1, p2);
                std::swap(P1, P2);
                if (smooth)
                    std::swap(n1, n2);
            }
        }
        int g = (int)B.tri_v0.size();
        float v0[3] = {(float)P1.x, (float)P1.y, (float)P1.z};
        float v1[3] = {(float)P2.x, (float)P2.y, (float)P2.z};
        float v2[3] = {(float)P3.x, (float)P3.y, (float)P3.z};
        B.tri_v0.push_back(make_float4(v0[0], v0[1], v0[2], plane_dist));
        B.tri_e1.push_back(make_float4(v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2], 0.f));
        B.tri_e2.push_back(make_float4(v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2], 0.f));
        B.tri_normal.push_back(gn);
        B.tri_shade.push_back(make_int4(nb + n1, nb + n2, nb + n3, smooth ? 1 : 0));
        B.tri_local.push_back(t);
        AABB box;
        box.grow(v0);
        box.grow(v1);
        box.grow(v2);
        B.push_prim(PK_TRIANGLE, (uint32_t)g, box);
    }
}

// The noise tables the renderer builds at start-up (InitTextureTable,
// noise.cpp:231-256; RTable with its odd entries halved, noise.cpp:181-182;
// InitSolidNoise, noise.cpp:306-347), from the reference's linear
// congruential sequence kept in a 32-bit int.
struct NoiseTables {
    std::vector<uint16_t> hash = std::vector<uint16_t>(1, 0);
    std::vector<float> rtab = std::vector<float>(1, 0.f);
    std::vector<int32_t> perm = std::vector<int32_t>(1, 0);
    std::vector<float4> grad = std::vector<float4>(1, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float4> waves = std::vector<float4>(1, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float> prand = std::vector<float>(1, 0.f);

    static int32_t next(int32_t x) { return (int32_t)(uint32_t)((int64_t)x * 1812433253LL + 12345LL); }

    // The pattern random table the cells pattern reads (gPatternRands,
    // pattern.cpp:91: RandomDoubleSequence(0, 1, 32768), i.e. boost's
    // mt19937 at its default seed 5489 through uniform_real, x / 2^32,
    // randomsequence.cpp:138-149): the Mersenne Twister of Matsumoto and
    // Nishimura (1998).  Hash3d indices stay below 4096 and crackle reads
    // two past its index: 4100 entries.
    void build_prand()
    {
        uint32_t mt[624];
        mt[0] = 5489u;
        for (int i = 1; i < 624; i++)
            mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
        prand.assign(4100, 0.f);
        int idx = 624;
        for (int n = 0; n < 4100; n++) {
            if (idx >= 624) {
                for (int i = 0; i < 624; i++) {
                    const uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
                    mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
                }
                idx = 0;
            }
            uint32_t y = mt[idx++];
            y ^= y >> 11;
            y ^= (y << 7) & 0x9d2c5680u;
            y ^= (y << 15) & 0xefc60000u;
            y ^= y >> 18;
            prand[n] = (float)((double)y / 4294967296.0);
        }
    }

    void build()
    {
        build_prand();
        hash.assign(8192, 0);
        int32_t r = 0;
        for (int i = 0; i < 4096; i++)
            hash[i] = (uint16_t)i;
        for (int i = 4095; i >= 0; i--) {
            r = next(r);
            int j = ((int)(r >> 16) & 0x7FFF) % 4096;
            std::swap(hash[i], hash[j]);
        }
        for (int i = 0; i < 4096; i++)
            hash[4096 + i] = hash[i];
        rtab.assign(2 * POV_NOISE_RTABLE_SIZE, 0.f);
        for (int i = 0; i < POV_NOISE_RTABLE_SIZE; i++) {
            rtab[2 * i] = (float)kPovNoiseRTable[i];
            rtab[2 * i + 1] = (float)(kPovNoiseRTable[i] * 0.5);
        }
        const int E = 2048;
        perm.assign(2 * (E + 1), 0);
        grad.assign(2 * (E + 1), make_float4(0.f, 0.f, 0.f, 0.f));
        r = 1;
        for (int i = 0; i < E; i++) {
            double v[3], q;
            do {
                for (int k = 0; k < 3; k++) {
                    r = next(r);
                    v[k] = (double)((((int)(r >> 16) & 0x7FFF) % (E << 1)) - E) / (double)E;
                }
                q = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            } while (q > 1.0 || q < 1.0e-5);
            q = std::sqrt(q);
            grad[i] = make_float4((float)(v[0] / q), (float)(v[1] / q), (float)(v[2] / q), 0.f);
        }
        for (int i = 0; i < E; i++)
            perm[i] = i;
        for (int i = E; i > 0; i -= 2) {
            int k = perm[i];
            r = next(r);
            int j = ((int)(r >> 16) & 0x7FFF) % E;
            perm[i] = perm[j];
            perm[j] = k;
        }
        for (int i = 0; i < E + 2; i++) {
            perm[E + i] = perm[i];
            grad[E + i] = grad[i];
        }
        // the scene's wave sources and frequencies (Initialize_Waves,
        // noise.cpp:189-205; SceneData::numberOfWaves = 10): source i is the
        // normalised DNoise at (i, 0, 0), in double as the reference has it
        waves.assign(POV_NUM_WAVES, make_float4(0.f, 0.f, 0.f, 0.f));
        r = -560851967;
        for (int i = 0; i < POV_NUM_WAVES; i++) {
            double d[3];
            dnoise((double)i, 0.0, 0.0, d);
            const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (l != 0.0)
                for (double& c : d)
                    c /= l;
            r = next(r);
            const double f = (double)((int)(r >> 16) & 0x7FFF) * 0.000030518509476 + 0.01;
            waves[i] = make_float4((float)d[0], (float)d[1], (float)d[2], (float)f);
        }
    }

    // DNoise (PortableDNoise, portablenoise.cpp:261-360) in double over the
    // hash table and RTable: the eight lattice corners in the reference's
    // order, three components each.
    void dnoise(double x, double y, double z, double out[3]) const
    {
        const double p[3] = {x, y, z};
        int ii[3];
        double f[3], g[3], sc[3], tc[3];
        for (int a = 0; a < 3; a++) {
            const int tmp = p[a] >= 0 ? (int)p[a] : (int)(p[a] - (1 - 1.0e-10));
            ii[a] = (tmp + 10000) & 0xFFF;
            f[a] = p[a] - tmp;
            g[a] = f[a] - 1;
            sc[a] = f[a] * f[a] * (3.0 - 2.0 * f[a]);
            tc[a] = 1 - sc[a];
        }
        auto h2 = [&](int a, int b) { return (int)hash[(int)hash[a] ^ b]; };
        auto rt = [&](int m) { return (m & 1) ? kPovNoiseRTable[m >> 1] * 0.5 : kPovNoiseRTable[m >> 1]; };
        const int h00 = h2(ii[0], ii[1]), h10 = h2(ii[0] + 1, ii[1]), h01 = h2(ii[0], ii[1] + 1),
                  h11 = h2(ii[0] + 1, ii[1] + 1);
        const double txty = tc[0] * tc[1], sxty = sc[0] * tc[1], txsy = tc[0] * sc[1], sxsy = sc[0] * sc[1];
        const int hc[8] = {h00, h10, h11, h01, h01, h11, h10, h00};
        const double sw[8] = {txty * tc[2], sxty * tc[2], sxsy * tc[2], txsy * tc[2],
                              txsy * sc[2], sxsy * sc[2], sxty * sc[2], txty * sc[2]};
        for (int k = 0; k < 8; k++) {
            const int zc = k >> 2;
            const int xo = (k == 1 || k == 2 || k == 5 || k == 6), yo = (k == 2 || k == 3 || k == 4 || k == 5);
            int m = (hash[hc[k] ^ (ii[2] + zc)] & 0xFF) * 2;
            const double xx = xo ? g[0] : f[0], yy = yo ? g[1] : f[1], zz = zc ? g[2] : f[2];
            for (int c = 0; c < 3; c++, m += 8) {
                const double v = sw[k] * (rt(m + 1) + rt(m + 2) * xx + rt(m + 4) * yy + rt(m + 6) * zz);
                out[c] = k == 0 ? v : out[c] + v;
            }
        }
    }
};

int rad_reset(PovGpuScene* sc);

// Switches the traversal between the library's binned-SAH tree (0) and the
// reference's bounding tree (1), built and uploaded on first use.
int apply_tree(PovGpuScene* sc, int mode)
{
    DeviceScene& S = sc->S;
    if (mode == 1) {
        if (!sc->ref_built) {
            build_reference_tree(sc->ref_input, sc->ref_output);
            std::vector<Bvh4Node> nodes = sc->ref_output.nodes;
            std::vector<uint32_t> refs = sc->ref_output.refs;
            if (nodes.empty())
                nodes.push_back(Bvh4Node{});
            if (refs.empty())
                refs.push_back(0u);
            CK(upload(sc->ref_nodes, nodes));
            CK(upload(sc->ref_refs, refs));
            sc->ref_built = true;
        }
        const int sd = std::max(8, 3 * sc->ref_output.depth + 2);
        if (sd > 160)
            return POV_GPU_E_UNSUPPORTED;
        S.nodes = sc->ref_nodes.as<Bvh4Node>();
        S.prim_refs = sc->ref_refs.as<uint32_t>();
        S.root = sc->ref_output.root;
        sc->stack_depth = sd;
    } else {
        S.nodes = sc->nodes.as<Bvh4Node>();
        S.prim_refs = sc->refs.as<uint32_t>();
        S.root = sc->sah_root;
        sc->stack_depth = sc->sah_stack_depth;
    }
    sc->tree_mode = mode;
    return POV_GPU_OK;
}

int build_scene(PovGpuScene* sc, const PovGpuSceneDesc* d)
{
    Builder B;
    std::vector<ObjectShade> objects((size_t)std::max(d->num_objects, 1));
    std::vector<int> mesh_normal_base((size_t)std::max(d->num_meshes, 1), 0);

    // mesh normals: Parse_Mesh2 normalises every normal_vectors entry
    // (source/parser/parser.cpp:4143-4152)
    for (int mi = 0; mi < d->num_meshes; mi++) {
        const PovGpuMesh& m = d->meshes[mi];
        mesh_normal_base[mi] = (int)B.normals.size();
        for (int i = 0; i < m.num_normals && m.normals; i++) {
            double x = m.normals[3 * i], y = m.normals[3 * i + 1], z = m.normals[3 * i + 2];
            if (std::fabs(x) < EPSILON && std::fabs(y) < EPSILON && std::fabs(z) < EPSILON)
                x = 1.0;
            double l = std::sqrt(x * x + y * y + z * z);
            B.normals.push_back(make_float4((float)(x / l), (float)(y / l), (float)(z / l), 0.f));
        }
    }

    for (int i = 0; i < d->num_objects; i++) {
        const PovGpuObject& o = d->objects[i];
        // texture: own, else inherited from the enclosing CSG (Post_Process)
        int mat = o.material;
        for (int p = o.parent; mat < 0 && p >= 0; p = d->objects[p].parent)
            mat = d->objects[p].material;
        objects[i].material = mat < 0 ? 0 : mat;
        objects[i].flags = (o.flags & POV_FLAG_INVERTED ? 1 : 0) | (o.flags & POV_FLAG_DOUBLE_ILLUM ? 16 : 0);
        objects[i].type = o.type;
        objects[i].mesh = o.mesh;
    }
    // interiors (Post_Process, parser.cpp:9225-9267): the description's,
    // plus a default one (the atmosphere's ior) for every top-level object
    // given none; a CSG child without one shares its parent's.  Each
    // object's id goes with whether its top-level object is opaque
    // (OPAQUE_FLAG, parser.cpp:9296-9297: a leaf whose plain pigment neither
    // filters nor transmits; a CSG whose children all are).
    const double atm_ior = d->atmosphere_ior > 0.0 ? d->atmosphere_ior : 1.0;
    sc->transparent = false;
    sc->branching = false;
    for (int i = 0; i < d->num_objects; i++) {
        const PovGpuMaterial& m = d->materials[objects[i].material];
        if (d->objects[i].type < POV_OBJ_UNION && !is_container(d->objects[i]) && material_transparent(d, m)) {
            sc->transparent = true;
            for (int k = 0; k < 3; k++)
                sc->branching = sc->branching || m.reflection_max[k] != 0.0f || m.reflection_min[k] != 0.0f;
        }
    }
    std::vector<float4> interiors;
    std::vector<int32_t> obj_interior((size_t)std::max(d->num_objects, 1), 0);
    {
        auto pair_of = [](const PovGpuInterior& I, std::vector<float4>& out) {
            out.push_back(make_float4((float)I.ior, (float)I.fade_distance, (float)I.fade_power, I.old_refract));
            out.push_back(make_float4(I.fade_colour[0], I.fade_colour[1], I.fade_colour[2], 0.f));
        };
        for (int k = 0; k < d->num_interiors; k++)
            pair_of(d->interiors[k], interiors);
        int nints = d->num_interiors;
        for (int i = 0; i < d->num_objects; i++) {
            const int given = d->object_interior ? d->object_interior[i] : 0;
            const int parent = d->objects[i].parent;
            if (given > 0) {
                obj_interior[i] = given - 1;
            } else if (parent >= 0) {
                obj_interior[i] = obj_interior[parent];
            } else {
                PovGpuInterior def{};
                def.ior = atm_ior;
                def.dispersion = 1.0;
                def.old_refract = 1.0f;
                pair_of(def, interiors);
                obj_interior[i] = nints++;
            }
        }
        // ids: only the interiors of transparent surfaces ever enter an
        // interior list; they are numbered 0.. (8-bit ids in the lists),
        // every other object gets id 0, which is never looked up
        std::vector<int> remap((size_t)std::max(nints, 1), -1);
        int nused = 0;
        for (int i = 0; i < d->num_objects; i++) {
            const PovGpuMaterial& m = d->materials[objects[i].material];
            if (d->objects[i].type < POV_OBJ_UNION && !is_container(d->objects[i]) && material_transparent(d, m) &&
                remap[obj_interior[i]] < 0)
                remap[obj_interior[i]] = nused++;
        }
        if (nused > 256)
            return POV_GPU_E_UNSUPPORTED;   // interior lists hold 8-bit ids
        std::vector<float4> used(2 * (size_t)std::max(nused, 1), make_float4(1.f, 0.f, 0.f, 1.f));
        for (int k = 0; k < nints; k++)
            if (remap[k] >= 0) {
                used[2 * (size_t)remap[k]] = interiors[2 * (size_t)k];
                used[2 * (size_t)remap[k] + 1] = interiors[2 * (size_t)k + 1];
            }
        interiors.swap(used);
        for (int i = 0; i < d->num_objects; i++)
            obj_interior[i] = std::max(remap[obj_interior[i]], 0);
        // opacity, children before parents
        std::vector<char> opaque((size_t)std::max(d->num_objects, 1), 1);
        for (int i = d->num_objects - 1; i >= 0; i--) {
            const PovGpuObject& o = d->objects[i];
            if (o.type < POV_OBJ_UNION) {
                opaque[i] = !material_transparent(d, d->materials[objects[i].material]);
            }
            if (o.parent >= 0 && !opaque[i])
                opaque[o.parent] = 0;
        }
        for (int i = 0; i < d->num_objects; i++) {
            int top = i;
            while (d->objects[top].parent >= 0)
                top = d->objects[top].parent;
            obj_interior[i] = (obj_interior[i] & 0xffff) | (opaque[top] ? (1 << 16) : 0);
        }
    }
    // media containers, numbered in object order
    std::vector<int> container_obj;
    for (int i = 0; i < d->num_objects; i++)
        if (is_container(d->objects[i])) {
            objects[i].flags |= OBJ_CONTAINER | ((int)container_obj.size() << 16);
            container_obj.push_back(i);
        }
    for (int i = 0; i < d->num_objects; i++) {
        const PovGpuObject& o = d->objects[i];
        if (o.parent >= 0)
            continue;   // CSG children are added with their parent
        B.cur_obj = i;
        AABB box;
        switch (o.type) {
        case POV_OBJ_SPHERE: B.push_prim(PK_SPHERE, B.add_sphere(o, i, &box), box); break;
        case POV_OBJ_BOX: B.push_prim(PK_BOX, B.add_box(o, i, &box), box); break;
        case POV_OBJ_TORUS: B.push_prim(PK_TORUS, B.add_torus(o, i, &box), box); break;
        case POV_OBJ_PLANE:
            B.planes.push_back(make_float4((float)o.p[0], (float)o.p[1], (float)o.p[2], (float)o.p[3]));
            B.plane_obj.push_back(i);
            break;
        case POV_OBJ_MESH: add_mesh(B, d, o, i, mesh_normal_base[o.mesh]); break;
        case POV_OBJ_UNION:
            // CSGUnion::All_Intersections pushes every child hit: the closest
            // hit is the same as with the children as separate objects
            for (int c = 0; c < o.num_children; c++) {
                int ci = o.first_child + c;
                const PovGpuObject& ch = d->objects[ci];
                AABB cb;
                if (ch.type == POV_OBJ_SPHERE) B.push_prim(PK_SPHERE, B.add_sphere(ch, ci, &cb), cb);
                else if (ch.type == POV_OBJ_BOX) B.push_prim(PK_BOX, B.add_box(ch, ci, &cb), cb);
                else B.push_prim(PK_TORUS, B.add_torus(ch, ci, &cb), cb);
            }
            break;
        default: {   // CSG intersection (difference) / merge as one primitive
            DevCsg g;
            g.type = o.type;
            g.first = (int)B.csg_children.size();
            g.count = o.num_children;
            g.object = i;
            AABB uni, inter;
            for (int k = 0; k < 3; k++) {
                inter.lo[k] = -INFINITY;
                inter.hi[k] = INFINITY;
            }
            bool any_plain = false;
            for (int c = 0; c < o.num_children; c++) {
                int ci = o.first_child + c;
                const PovGpuObject& ch = d->objects[ci];
                AABB cb;
                DevCsgChild cc;
                cc.flags = ch.flags & POV_FLAG_INVERTED ? 1 : 0;
                cc.object = ci;
                if (ch.type == POV_OBJ_SPHERE) { cc.kind = PK_SPHERE; cc.index = B.add_sphere(ch, ci, &cb); }
                else if (ch.type == POV_OBJ_BOX) { cc.kind = PK_BOX; cc.index = B.add_box(ch, ci, &cb); }
                else { cc.kind = PK_TORUS; cc.index = B.add_torus(ch, ci, &cb); }
                B.csg_children.push_back(cc);
                uni.grow(cb);
                if (!cc.flags) {   // CSG::Compute_BBox: overlap of the non-inverted children
                    any_plain = true;
                    for (int k = 0; k < 3; k++) {
                        inter.lo[k] = std::max(inter.lo[k], cb.lo[k]);
                        inter.hi[k] = std::min(inter.hi[k], cb.hi[k]);
                    }
                }
            }
            AABB gb = (o.type == POV_OBJ_INTERSECTION && any_plain) ? inter : uni;
            if (gb.lo[0] > gb.hi[0] || gb.lo[1] > gb.hi[1] || gb.lo[2] > gb.hi[2])
                gb = uni;   // empty overlap: keep a valid (never hit) box
            int idx = (int)B.csgs.size();
            B.csgs.push_back(g);
            B.push_prim(PK_CSG, (uint32_t)idx, gb);
            break;
        }
        }
    }
    if (B.tri_v0.size() >= (size_t)PRIM_INDEX_MASK || B.bvh.items.size() >= (1u << 28))
        return POV_GPU_E_UNSUPPORTED;

    int root2 = B.bvh.build_root();
    // four-wide nodes for the traversal; a node pushes at most three
    // children, so the stack holds 3 per level of the collapsed tree
    Bvh4Collapse wide(B.bvh.nodes);
    int root = root2 >= 0 && root2 != BVH_EMPTY ? wide.collapse(root2, 1) : root2;
    if (wide.out.empty())
        wide.out.push_back(Bvh4Node{});
    sc->stack_depth = std::max(8, 3 * wide.max_depth + 2);
    if (sc->stack_depth > 160)
        return POV_GPU_E_UNSUPPORTED;
    sc->sah_root = root;
    sc->sah_stack_depth = sc->stack_depth;
    sc->sah_depth = wide.max_depth;
    sc->sah_nodes = (int)wide.out.size();

    // reorder triangle records into leaf order (prim refs then index the
    // leaf-order slot directly, so a leaf's triangles are contiguous)
    std::vector<float4> lv0, le1, le2;
    std::vector<int32_t> tri_global;
    sc->top_tori = false;
    for (uint32_t r : B.bvh.refs)
        sc->top_tori = sc->top_tori || (r >> PRIM_KIND_SHIFT) == PK_TORUS;
    sc->csg_torus = false;
    for (const DevCsgChild& c : B.csg_children)
        sc->csg_torus = sc->csg_torus || c.kind == PK_TORUS;
    lv0.reserve(B.tri_v0.size());
    le1.reserve(B.tri_v0.size());
    le2.reserve(B.tri_v0.size());
    for (uint32_t& r : B.bvh.refs) {
        if ((r >> PRIM_KIND_SHIFT) == PK_TRIANGLE) {
            uint32_t g = r & PRIM_INDEX_MASK;
            uint32_t slot = (uint32_t)lv0.size();
            lv0.push_back(B.tri_v0[g]);
            le1.push_back(B.tri_e1[g]);
            le2.push_back(B.tri_e2[g]);
            tri_global.push_back((int32_t)g);
            r = (PK_TRIANGLE << PRIM_KIND_SHIFT) | slot;
        }
    }

    // the input of the reference's bounding tree (built when a launch
    // configuration asks for it): the finite top-level objects in scene
    // order with their Compute_BBox boxes and primitives, each mesh2's
    // triangles with their boxes (min/max of the vertices)
    {
        std::vector<uint32_t> tri_slot(B.tri_v0.size(), 0);
        for (size_t sl = 0; sl < tri_global.size(); sl++)
            tri_slot[(size_t)tri_global[sl]] = (uint32_t)sl;
        RefTreeInput& R = sc->ref_input;
        R = RefTreeInput{};
        std::vector<int> obj_slot((size_t)std::max(d->num_objects, 1), -1);
        for (int i = 0; i < d->num_objects; i++) {
            const PovGpuObject& o = d->objects[i];
            if (o.parent < 0 && o.type == POV_OBJ_PLANE)
                R.infinite++;
            if (o.parent >= 0 || o.type == POV_OBJ_PLANE)
                continue;
            RefObject ro;
            ro.box = ref_object_box(d, i);
            if (o.type == POV_OBJ_MESH) {
                ro.mesh = (int32_t)R.meshes.size();
                R.meshes.emplace_back();
            }
            obj_slot[i] = (int)R.objects.size();
            R.objects.push_back(ro);
        }
        // the pushes come in object order: gather each object's primitives
        for (size_t k = 0; k < B.pushed.size();) {
            const int32_t obj = B.pushed[k].first;
            size_t e = k;
            while (e < B.pushed.size() && B.pushed[e].first == obj)
                e++;
            if (obj >= 0 && obj_slot[obj] >= 0) {
                RefObject& ro = R.objects[obj_slot[obj]];
                if (ro.mesh >= 0) {
                    const PovGpuMesh& m = d->meshes[d->objects[obj].mesh];
                    for (size_t j = k; j < e; j++) {
                        const uint32_t g = B.pushed[j].second & PRIM_INDEX_MASK;
                        const int t = B.tri_local[g];   // the triangle's place in the mesh
                        double mn[3] = {2.0e10, 2.0e10, 2.0e10}, mx[3] = {-2.0e10, -2.0e10, -2.0e10};
                        for (int c = 0; c < 3; c++) {
                            const float* v = m.vertices + 3 * m.face_indices[3 * t + c];
                            for (int a = 0; a < 3; a++) {
                                mn[a] = std::min(mn[a], (double)v[a]);
                                mx[a] = std::max(mx[a], (double)v[a]);
                            }
                        }
                        RefTriangle rt;
                        for (int a = 0; a < 3; a++) {
                            rt.box.ll[a] = (float)mn[a];
                            rt.box.sz[a] = (float)(mx[a] - mn[a]);
                        }
                        rt.ref = (PK_TRIANGLE << PRIM_KIND_SHIFT) | tri_slot[g];
                        R.meshes[ro.mesh].push_back(rt);
                    }
                } else {
                    ro.first = (uint32_t)R.refs.size();
                    ro.count = (uint32_t)(e - k);
                    for (size_t j = k; j < e; j++)
                        R.refs.push_back(B.pushed[j].second);
                }
            }
            k = e;
        }
        sc->ref_built = false;
        sc->tree_mode = 0;
    }

    std::vector<DevMaterial> mats((size_t)d->num_materials);
    for (int i = 0; i < d->num_materials; i++) {
        mats[i] = make_material(d->materials[i], d->ambient_light,
                                d->radiosity.enabled && d->language_version >= 370, d->language_version);
        if (d->materials[i].pattern > 0 && material_transparent(d, d->materials[i]))
            mats[i].see_through = SEE_PATTERN | (d->language_version < 370 ? SEE_LEGACY : 0);
    }
    std::vector<DevLight> lights((size_t)std::max(d->num_lights, 1));
    int num_area = 0;
    for (int i = 0; i < d->num_lights; i++) {
        const PovGpuLight& L = d->lights[i];
        lights[i].center = make_float4((float)L.center[0], (float)L.center[1], (float)L.center[2], (float)L.kind);
        lights[i].colour = make_float4(L.colour[0], L.colour[1], L.colour[2], 0.f);
        double len1 = std::sqrt(L.axis1[0] * L.axis1[0] + L.axis1[1] * L.axis1[1] + L.axis1[2] * L.axis1[2]);
        lights[i].axis1 = make_float4((float)L.axis1[0], (float)L.axis1[1], (float)L.axis1[2], (float)len1);
        lights[i].axis2 = make_float4((float)L.axis2[0], (float)L.axis2[1], (float)L.axis2[2], 0.f);
        lights[i].area = make_int4(L.area_size1, L.area_size2, L.adaptive_level,
                                   (L.circular ? 1 : 0) | (L.orient ? 2 : 0));
        // Direction (Parse_Light_Source, parser.cpp:3521-3528)
        double dv[3] = {L.points_at[0] - L.center[0], L.points_at[1] - L.center[1], L.points_at[2] - L.center[2]};
        double dl = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        if (dl > 1.0e-10)
            for (double& x : dv)
                x /= dl;
        const int type = L.light_type == 0 ? LIGHT_POINT : L.light_type;
        lights[i].dir = make_float4((float)dv[0], (float)dv[1], (float)dv[2], (float)type);
        const bool parallel = L.parallel || type == LIGHT_CYLINDER;
        lights[i].beam = make_float4((float)L.radius, (float)L.falloff, (float)L.tightness, parallel ? 1.f : 0.f);
        lights[i].fade = make_float4((float)L.fade_distance, (float)L.fade_power, 0.f, 0.f);
        if (L.kind == POV_LIGHT_AREA)
            num_area++;
    }

    CK(upload(sc->nodes, wide.out));
    CK(upload(sc->refs, B.bvh.refs));
    CK(upload(sc->tri_v0, lv0));
    CK(upload(sc->tri_e1, le1));
    CK(upload(sc->tri_e2, le2));
    CK(upload(sc->tri_global, tri_global));
    CK(upload(sc->tri_shade, B.tri_shade));
    CK(upload(sc->tri_normal, B.tri_normal));
    CK(upload(sc->tri_local, B.tri_local));
    CK(upload(sc->normals, B.normals));
    CK(upload(sc->spheres, B.spheres));
    CK(upload(sc->spheres64, B.spheres64));
    CK(upload(sc->boxes64, B.boxes64));
    CK(upload(sc->sphere_obj, B.sphere_obj));
    CK(upload(sc->sphere_flags, B.sphere_flags));
    CK(upload(sc->planes, B.planes));
    CK(upload(sc->plane_obj, B.plane_obj));
    CK(upload(sc->boxes, B.boxes));
    CK(upload(sc->tori, B.tori));
    {
        // FP32 copy of each torus's local frame for the pre-cull: the rows
        // giving local x, y and z (p' = p * M of the inverse), then R, r
        std::vector<float4> t32(std::max<size_t>(B.tori.size(), 1) * 4);
        for (size_t i = 0; i < B.tori.size(); i++) {
            const double* m = B.tori[i].inv;
            for (int c = 0; c < 3; c++)
                t32[4 * i + c] = make_float4((float)m[c], (float)m[3 + c], (float)m[6 + c], (float)m[9 + c]);
            t32[4 * i + 3] = make_float4((float)B.tori[i].R, (float)B.tori[i].r, 0.f, 0.f);
        }
        CK(upload(sc->tori32, t32));
    }
    CK(upload(sc->csgs, B.csgs));
    CK(upload(sc->csg_children, B.csg_children));
    // one DevMedia per container: its media and its box primitive
    std::vector<DevMedia> medias(std::max<size_t>(container_obj.size(), 1));
    int media_ni = 0;
    for (size_t c = 0; c < container_obj.size(); c++) {
        const PovGpuObject& o = d->objects[container_obj[c]];
        const PovGpuMedia& md = d->medias[o.media - 1];
        // the container's primitive: a box or a sphere
        const bool sphere = o.type == POV_OBJ_SPHERE;
        int box = -1;
        const std::vector<int32_t>& owners = sphere ? B.sphere_obj : B.box_obj;
        for (size_t b = 0; b < owners.size(); b++)
            if (owners[b] == container_obj[c])
                box = (int)b;
        if (box < 0)
            return POV_GPU_E_INVALID;
        sc->h_containers.push_back(container_obj[c]);
        DevMedia& m = medias[c];
        m.emission = make_float4(md.emission[0], md.emission[1], md.emission[2], md.aa_threshold);
        bool scat = md.scattering[0] != 0.0f || md.scattering[1] != 0.0f || md.scattering[2] != 0.0f;
        m.scattering = make_float4(md.scattering[0], md.scattering[1], md.scattering[2], scat ? 1.0f : 0.0f);
        m.extinction = make_float4(md.extinction[0], md.extinction[1], md.extinction[2], 0.0f);
        m.n = make_int4(md.intervals, std::max((md.min_samples + 1) / 2, 1), md.aa_level, box);
        m.phase = make_float4((float)md.scattering_type, md.eccentricity, sphere ? 1.0f : 0.0f, 0.0f);
        media_ni = std::max(media_ni, md.intervals + 1);   // + the padding interval
        const int sub = m.n.y, T = (1 << md.aa_level) - 1;
        sc->media_smax = std::max(sc->media_smax, sub + 1 + sub * T);
        sc->media_sub = std::max(sc->media_sub, sub);
        sc->media_levels = std::max(sc->media_levels, md.aa_level);
    }

    // pattern pigments and the noise tables they read
    std::vector<DevPattern> pats(std::max(d->num_patterns, 1));
    for (int i = 0; i < d->num_patterns; i++) {
        const PovGpuPattern& pt = d->patterns[i];
        DevPattern& q = pats[i];
        for (int c = 0; c < 3; c++)
            q.col[c] = make_float4((float)pt.inverse[0 * 4 + c], (float)pt.inverse[1 * 4 + c],
                                   (float)pt.inverse[2 * 4 + c], (float)pt.inverse[3 * 4 + c]);
        q.gradient = make_float4((float)pt.gradient[0], (float)pt.gradient[1], (float)pt.gradient[2],
                                 (float)pt.agate_turb);
        q.turb = make_float4((float)pt.turbulence[0], (float)pt.turbulence[1], (float)pt.turbulence[2],
                             (float)pt.omega);
        q.wave = make_float4((float)pt.frequency, (float)pt.phase, (float)pt.exponent, (float)pt.lambda);
        q.kind = make_int4(pt.type, pt.noise_generator, pt.num_entries, pt.wave_type);
        q.kind2 = make_int4(pt.octaves, pt.has_turbulence, pt.arms, 0);
        q.brick = make_float4((float)pt.brick_size[0], (float)pt.brick_size[1], (float)pt.brick_size[2],
                              (float)pt.mortar);
        q.crackle = make_float4((float)pt.crackle_form[0], (float)pt.crackle_form[1], (float)pt.crackle_form[2],
                                (float)pt.crackle_metric);
        q.crackle2 = make_float4((float)pt.crackle_offset, (float)pt.control0, (float)pt.control1,
                                 pt.crackle_solid ? 1.f : 0.f);
        for (int k = 0; k < POV_PATTERN_MAX_ENTRIES; k++) {
            q.values[k] = pt.values[k];
            q.colours[k] = make_float4(pt.colours[k][0], pt.colours[k][1], pt.colours[k][2], pt.filters[k]);
            q.transmits[k] = pt.transmits[k];
        }
    }
    // normal perturbations: the forward TRANSFORM's 3x3 rows
    // (MInvTransNormal with the matrix, matrix.cpp:495-508)
    std::vector<DevNormal> nrms(std::max(d->num_normals, 1));
    for (int i = 0; i < d->num_normals; i++) {
        const PovGpuNormal& nm = d->normals[i];
        DevNormal& q = nrms[i];
        for (int r = 0; r < 3; r++)
            q.fwd[r] = make_float4((float)nm.matrix[r * 4 + 0], (float)nm.matrix[r * 4 + 1],
                                   (float)nm.matrix[r * 4 + 2], 0.f);
        // the slope's factor as the reference forms it in double
        // (normal.cpp:887-889)
        const double slope = (double)nm.amount * -5.0 * (0.02 / (double)nm.delta);
        q.params = make_float4(nm.amount, nm.delta, (float)slope, 0.f);
        q.kind = make_int4(nm.pattern - 1, nm.dont_scale_bumps ? 1 : 0, 0, 0);
    }
    NoiseTables nt;
    if (d->num_patterns > 0)
        nt.build();
    sc->textured = false;
    for (int i = 0; i < d->num_materials; i++)
        sc->textured = sc->textured || d->materials[i].pattern > 0 || d->materials[i].normal > 0;

    CK(upload(sc->objects, objects));
    CK(upload(sc->materials, mats));
    CK(upload(sc->obj_interior, obj_interior));
    CK(upload(sc->interiors, interiors));
    CK(upload(sc->lights, lights));
    CK(upload(sc->medias, medias));
    CK(upload(sc->patterns, pats));
    CK(upload(sc->tnormals, nrms));
    CK(upload(sc->noise_hash, nt.hash));
    CK(upload(sc->noise_rtab, nt.rtab));
    CK(upload(sc->noise_perm, nt.perm));
    CK(upload(sc->noise_grad, nt.grad));
    CK(upload(sc->noise_waves, nt.waves));
    CK(upload(sc->noise_prand, nt.prand));

    sc->h_sphere_obj = B.sphere_obj;
    sc->h_plane_obj = B.plane_obj;
    sc->h_box_obj = B.box_obj;
    sc->h_torus_obj = B.torus_obj;
    sc->h_tri_global = tri_global;
    sc->h_tri_local = B.tri_local;
    sc->h_tri_obj.resize(B.tri_normal.size());
    for (size_t k = 0; k < B.tri_normal.size(); k++)
        sc->h_tri_obj[k] = __builtin_bit_cast(int32_t, B.tri_normal[k].w);
    sc->h_csgs = B.csgs;
    sc->h_objects.assign(d->objects, d->objects + d->num_objects);
    sc->h_csg_children = B.csg_children;

    DeviceScene& S = sc->S;
    S.nodes = sc->nodes.as<Bvh4Node>();
    S.prim_refs = sc->refs.as<uint32_t>();
    S.root = root;
    S.tri_v0 = sc->tri_v0.as<float4>();
    S.tri_e1 = sc->tri_e1.as<float4>();
    S.tri_e2 = sc->tri_e2.as<float4>();
    S.tri_global = sc->tri_global.as<int32_t>();
    S.tri_shade = sc->tri_shade.as<int4>();
    S.tri_normal = sc->tri_normal.as<float4>();
    S.tri_local = sc->tri_local.as<int32_t>();
    S.normals = sc->normals.as<float4>();
    S.spheres = sc->spheres.as<float4>();
    S.sphere_obj = sc->sphere_obj.as<int32_t>();
    S.sphere_flags = sc->sphere_flags.as<int32_t>();
    S.planes = sc->planes.as<float4>();
    S.plane_obj = sc->plane_obj.as<int32_t>();
    S.num_planes = (int)B.planes.size();
    S.boxes = sc->boxes.as<DevBox>();
    S.tori = sc->tori.as<DevTorus>();
    S.tori32 = sc->tori32.as<float4>();
    S.csgs = sc->csgs.as<DevCsg>();
    S.csg_children = sc->csg_children.as<DevCsgChild>();
    S.has_full_prims = (!B.tori.empty() || !B.csgs.empty()) ? 1 : 0;
    S.spheres64 = sc->spheres64.as<double>();
    S.boxes64 = sc->boxes64.as<double>();
    S.objects = sc->objects.as<ObjectShade>();
    S.materials = sc->materials.as<DevMaterial>();
    S.obj_interior = sc->obj_interior.as<int32_t>();
    S.interiors = sc->interiors.as<float4>();
    S.atm_ior = (float)atm_ior;
    S.transparent = sc->transparent ? 1 : 0;
    S.lights = sc->lights.as<DevLight>();
    S.num_lights = d->num_lights;
    S.num_area_lights = num_area;
    S.medias = sc->medias.as<DevMedia>();
    S.patterns = sc->patterns.as<DevPattern>();
    S.tnormals = sc->tnormals.as<DevNormal>();
    S.noise.hash = sc->noise_hash.as<uint16_t>();
    S.noise.rtab = sc->noise_rtab.as<float>();
    S.noise.perm = sc->noise_perm.as<int32_t>();
    S.noise.grad = sc->noise_grad.as<float4>();
    S.noise.waves = sc->noise_waves.as<float4>();
    S.noise.prand = sc->noise_prand.as<float>();
    S.num_containers = (int)container_obj.size();
    sc->media_ni = container_obj.empty() ? 0 : media_ni;
    S.max_trace_level = d->max_trace_level;
    S.adc_bailout = d->adc_bailout;
    S.background = make_float4(d->background[0], d->background[1], d->background[2], d->background[3]);
    for (int k = 0; k < 3; k++) {
        S.cam_loc[k] = d->camera.location[k];
        S.cam_dir[k] = d->camera.direction[k];
        S.cam_right[k] = d->camera.right[k];
        S.cam_up[k] = d->camera.up[k];
    }
    set_camera_ff(S);
    sc->num_lights = d->num_lights;
    sc->max_trace_level = d->max_trace_level;
    if (d->radiosity.enabled) {
        // the sample cache and the direction pool: Halton(2,3) cosine-weighted
        // (GetSubRandomCosWeightedDirectionGenerator(0, 1600) picks that
        // generator, randomsequence.cpp:1019-1037; HaltonGenerator and
        // HaltonCosWeightedDirectionGenerator, randomsequence.cpp:730-747,
        // 907-915)
        RadiosityState& R = sc->rad;
        R.enabled = true;
        R.set = d->radiosity;
        R.cap_blocks = 1 << 21;
        size_t slots = 1u << 22;
        R.key_mask = (uint32_t)(slots - 1);
        CK(R.blocks.ensure(sizeof(RadBlock) * (size_t)R.cap_blocks));
        CK(R.quick.ensure(sizeof(float4) * (size_t)R.cap_blocks));
        CK(R.bslot.ensure(sizeof(int32_t) * (size_t)R.cap_blocks));
        CK(R.members.ensure(sizeof(int32_t) * (size_t)R.cap_blocks));
        CK(R.count.ensure(sizeof(int32_t) * 2));   // block count, rebuild allocation cursor
        CK(R.keys.ensure(sizeof(unsigned long long) * slots));
        CK(R.seg_off.ensure(sizeof(int32_t) * slots));
        CK(R.seg_cnt.ensure(sizeof(int32_t) * slots));
        CK(R.seg_cur.ensure(sizeof(int32_t) * slots));
        CK(R.range.ensure(sizeof(int32_t) * 2 * RAD_LEVELS));
        CK(R.occupancy.ensure(1u << 21));   // 2^24 occupancy bits
        CK(R.rstats.ensure(sizeof(unsigned long long) * RST_COUNT));
        std::vector<float> dirs(3 * (size_t)RAD_DIRECTIONS);
        for (int i = 0; i < RAD_DIRECTIONS; i++) {
            double hb[2];
            const unsigned base[2] = {2, 3};
            for (int k = 0; k < 2; k++) {
                size_t idx = (size_t)i + 1;
                double h = 0.0, q = 1.0 / base[k];
                while (idx > 0) {
                    h += (double)(idx % base[k]) * q;
                    idx /= base[k];
                    q /= base[k];
                }
                hb[k] = h;
            }
            double r = std::sqrt(hb[0]), th = hb[1] * (2 * 3.14159265358979323846);
            double x = r * std::cos(th), z = r * std::sin(th);
            dirs[3 * i + 0] = (float)x;
            dirs[3 * i + 1] = (float)std::sqrt(1 - x * x - z * z);
            dirs[3 * i + 2] = (float)z;
        }
        CK(rad_upload_directions(dirs.data()));
        int rc = rad_reset(sc);
        if (rc != POV_GPU_OK)
            return rc;
    }
    return POV_GPU_OK;
}


static_assert(PovGpuScene::PIN_STATS + sizeof(unsigned long long) * ST_COUNT <= PovGpuScene::PIN_WORK &&
                  PovGpuScene::PIN_WORK + 8 * sizeof(unsigned long long) <= PovGpuScene::PIN_BYTES,
              "pinned readback regions overlap");

int check_device_error(PovGpuScene* sc, PovGpuStats* stats, unsigned long long* host_stats)
{
    cudaStream_t st = sc->active();
    uint32_t* perr = reinterpret_cast<uint32_t*>(sc->pinned + PovGpuScene::PIN_ERR);
    unsigned long long* pst = reinterpret_cast<unsigned long long*>(sc->pinned + PovGpuScene::PIN_STATS);
    CK(cudaMemcpyAsync(perr, sc->err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(pst, sc->stats.p, sizeof(unsigned long long) * ST_COUNT, cudaMemcpyDeviceToHost, st));
    HW(st);
    const uint32_t errw = *perr;
    std::memcpy(host_stats, pst, sizeof(unsigned long long) * ST_COUNT);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->number_of_rays = host_stats[ST_RAYS];
        stats->shadow_ray_tests = host_stats[ST_SHADOW_TESTS];
        stats->shadow_rays_succeeded = host_stats[ST_SHADOW_SUCCEEDED];
        stats->reflected_rays = host_stats[ST_REFLECTED];
        stats->transmitted_rays = host_stats[ST_TRANSMITTED];
        stats->media_samples = host_stats[ST_MEDIA_SAMPLES];
        stats->refracted_rays = host_stats[ST_REFRACTED];
        stats->internal_reflected_rays = host_stats[ST_INTERNAL_REFLECTED];
        stats->device_error = errw;
    }
    return errw ? POV_GPU_E_DEVICE : POV_GPU_OK;
}

// Records per-stage CUDA events on the launch stream (profiling bit 0) and
// counts launches; stage durations are summed after the final sync.
class StageClock {
public:
    StageClock(PovGpuScene* sc, cudaStream_t st) : sc_(sc), st_(st)
    {
        std::memset(&sc_->timings, 0, sizeof(sc_->timings));
        timing_ = (sc_->profiling & POV_GPU_PROFILE_TIMES) != 0;
    }
    cudaError_t begin(int stage)
    {
        cur_ = stage;
        if (!timing_)
            return cudaSuccess;
        cudaError_t e = next_event(a_);
        if (e == cudaSuccess)
            e = cudaEventRecord(a_, st_);
        return e;
    }
    cudaError_t end(int launches = 1)
    {
        sc_->timings.stage_launches[cur_] += launches;
        sc_->timings.kernel_launches += launches;
        if (!timing_)
            return cudaSuccess;
        cudaEvent_t b;
        cudaError_t e = next_event(b);
        if (e == cudaSuccess)
            e = cudaEventRecord(b, st_);
        marks_.push_back({cur_, a_, b});
        return e;
    }
    void collect()
    {
        for (auto& m : marks_) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess)
                sc_->timings.stage_ms[m.stage] += ms;
        }
    }

private:
    struct Mark {
        int stage;
        cudaEvent_t a, b;
    };
    cudaError_t next_event(cudaEvent_t& ev)
    {
        if (used_ >= sc_->events.size()) {
            cudaEvent_t e;
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess)
                return r;
            sc_->events.push_back(e);
        }
        ev = sc_->events[used_++];
        return cudaSuccess;
    }
    PovGpuScene* sc_;
    cudaStream_t st_;
    bool timing_ = false;
    int cur_ = 0;
    size_t used_ = 0;
    cudaEvent_t a_ = nullptr;
    std::vector<Mark> marks_;
};


int rad_resolve(PovGpuScene* sc, StageClock& clk, int d, const RadQuery* queries, int n, float4* out);

// RadiosityRecursionSettings of bounce depth d (radiosity.cpp:177-294) and
// the current task's error bound.
RadParams rad_params(const PovGpuScene* sc, int d)
{
    const RadiosityState& R = sc->rad;
    const PovGpuRadiosity& rs = R.set;
    RadParams p{};
    p.depth = d;
    p.final_trace = R.final_trace ? 1 : 0;
    p.always_sample = rs.always_sample;
    p.reuse_count = d == 0 ? rs.nearest_count : (d == 1 ? std::min(2, rs.nearest_count) : 1);
    int n = (int)(rs.count * std::pow(0.5, (double)d));
    p.rays_per_sample = std::min(std::max(5, n), RAD_DIRECTIONS);
    p.error_bound = (float)R.error_bound;
    p.error_bound_factor = (float)std::pow(2.0, (double)d);
    p.min_reuse_factor = (float)(rs.minimum_reuse * std::pow(2.0, (double)d));
    p.max_reuse_factor = (float)(rs.maximum_reuse * std::pow(2.0, (double)d));
    p.address_factor = (float)(rs.error_bound * std::pow(2.0, (double)d) / (d == 0 ? 1.0 : 8.0));
    p.gather_weight = (float)std::max(rs.adc_bailout + EPSILON, std::pow(0.5 * rs.brightness, (double)d + 1));
    p.gray = (float)rs.gray_threshold;
    p.brightness = (float)rs.brightness;
    p.adc = (float)rs.adc_bailout;
    return p;
}

RadCacheView cache_view(PovGpuScene* sc)
{
    RadiosityState& R = sc->rad;
    RadCacheView c{};
    c.blocks = R.blocks.as<RadBlock>();
    c.quick = R.quick.as<float4>();
    c.bslot = R.bslot.as<int32_t>();
    c.count = R.count.as<int32_t>();
    c.cap = R.cap_blocks;
    c.keys = R.keys.as<unsigned long long>();
    c.seg_off = R.seg_off.as<int32_t>();
    c.seg_cnt = R.seg_cnt.as<int32_t>();
    c.seg_cur = R.seg_cur.as<int32_t>();
    c.members = R.members.as<int32_t>();
    c.seg_total = R.count.as<int32_t>() + 1;
    c.mask = R.key_mask;
    c.size_range = R.range.as<int32_t>();
    c.occupancy = R.occupancy.as<uint32_t>();
    c.occ_mask = (uint32_t)(R.occupancy.bytes * 8 - 1);
    return c;
}

// Empties the sample cache and restarts the direction sequences (a new
// frame: the reference keeps one cache per view).
int rad_reset(PovGpuScene* sc)
{
    RadiosityState& R = sc->rad;
    cudaStream_t st = sc->active();
    CK(cudaMemsetAsync(R.count.p, 0, sizeof(int32_t), st));
    CK(cudaMemsetAsync(R.keys.p, 0, R.keys.bytes, st));
    R.seg_dirty = false;   // no blocks, no node keys
    int32_t range[2 * RAD_LEVELS];
    for (int d = 0; d < RAD_LEVELS; d++) {
        range[2 * d] = 1 << 30;
        range[2 * d + 1] = -1;
    }
    CK(cudaMemcpy(R.range.p, range, sizeof(range), cudaMemcpyHostToDevice));
    CK(cudaMemsetAsync(R.occupancy.p, 0, R.occupancy.bytes, st));
    for (int& b : R.dir_base)
        b = 0;
    // a loaded cache file's samples start every frame's cache, as the
    // reference's RadiosityCache loads its file when it is built
    const int nl = (int)std::min<size_t>(R.loaded.size(), (size_t)R.cap_blocks);
    if (nl > 0) {
        CK(cudaMemcpyAsync(R.blocks.p, R.loaded.data(), sizeof(RadBlock) * (size_t)nl, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(R.count.p, &nl, sizeof(int32_t), cudaMemcpyHostToDevice, st));
        float af[RAD_LEVELS];
        for (int d = 0; d < RAD_LEVELS; d++)
            af[d] = rad_params(sc, d).address_factor;
        CK(launch_rad_file(cache_view(sc), af, 0, nl, sc->err.as<uint32_t>(), st));
        R.seg_dirty = true;
        CK(cudaStreamSynchronize(st));   // the host vectors above must outlive the copies
    }
    return POV_GPU_OK;
}

// Media of the current queue's rays inside containers (MediaFunction::
// ComputeMedia per segment): lists them, samples them in chunks whose sample
// slots fit the scratch (rounds of the adaptive recursion), and folds each
// segment's emission and transmittance into its path before shading.
int run_media(PovGpuScene* sc, PathBufs& B, const QRay* q, const int* state, const int* path, const int* qcount,
              size_t maxq, int grid, int* launches)
{
    cudaStream_t st = sc->active();
    int* cnt = B.counters.as<int>();
    const DeviceScene& S = sc->S;
    const int NI = sc->media_ni, SMAX = sc->media_smax;
    CK(cudaMemsetAsync(cnt + C_MC, 0, sizeof(int), st));
    CK(launch_media_list(state, B.hits.as<QHit>(), qcount, (int)maxq, B.mlist.as<int>(), cnt + C_MC, grid, st));
    CK(cudaMemcpyAsync(sc->pin_int(0), cnt + C_MC, sizeof(int), cudaMemcpyDeviceToHost, st));
    HW(st);
    const int nm = std::min<int>(*sc->pin_int(0), (int)maxq);
    *launches = 1;
    if (nm == 0)
        return POV_GPU_OK;
    // chunk: sample slots within ~1 GiB; a round lists at most every node
    // of the deepest tree level
    const size_t per_seg = (size_t)NI * SMAX;
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nm, ((size_t)1 << 30) / (per_seg * 16)));
    const size_t list_cap = (size_t)chunk * NI * sc->media_sub * ((size_t)1 << (sc->media_levels - 1));
    CK(B.mcbuf.ensure(sizeof(float4) * (size_t)chunk * per_seg));
    CK(B.mrounds.ensure(sizeof(int) * list_cap));
    for (int first = 0; first < nm; first += chunk) {
        const int nseg = std::min(chunk, nm - first);
        if (++sc->media_stamp == 0)
            ++sc->media_stamp;
        CK(launch_media_chunk(S, q, state, B.hits.as<QHit>(), B.mlist.as<int>(), first, nseg, NI, SMAX,
                              sc->media_sub, sc->media_levels, B.mcbuf.as<float4>(), B.mrounds.as<int>(),
                              B.mrounds.as<int>(), cnt + C_ML, (int)list_cap, sc->media_stamp, B.mte.as<float4>(),
                              B.mod.as<float4>(), sc->stack_depth, grid, sc->err.as<uint32_t>(),
                              sc->stats.as<unsigned long long>(), st));
        *launches += 2 + 2 * (sc->media_levels - 1);
    }
    CK(launch_media_combine(S, state, path, B.hits.as<QHit>(), B.mlist.as<int>(), cnt + C_MC, (int)maxq, NI,
                            B.mte.as<float4>(), B.mod.as<float4>(), B.paths.as<PathState>(), grid, st));
    *launches += 1;
    return POV_GPU_OK;
}

// Traces one wavefront through trace levels level0 .. max_level-1: the rays
// in B.qA (count in the C_QA counter, path index in B.pathA, origin surface
// in B.skipA) and the reflection rays they spawn.  With radiosity on and
// `hit_depth` below the recursion limit, every level's hits query the
// radiosity cache at that bounce depth (RadiosityFunction::ComputeAmbient)
// and the answers are added to their paths before the next level.
// `sample_rays`: the wavefront holds radiosity sample rays, shaded the way
// the radiosity Trace shades them.
int run_levels(PovGpuScene* sc, StageClock& clk, PathBufs& B, size_t maxq, int level0, int max_level, int hit_depth,
               bool sample_rays)
{
    const int nl = std::max(sc->num_lights, 1);
    const int nal = sample_rays ? 0 : sc->S.num_area_lights;
    const bool rad = sc->rad.enabled && hit_depth < sc->rad.set.recursion_limit;
    const bool media = sc->media_ni > 0;
    const bool transparent = sc->transparent;
    const bool staged = media || transparent;   // rays carry their own level
    // scenes with tori or CSG: torus tests deferred out of the traversal,
    // and where no CSG holds a torus the traversal's torus-free variant
    const bool torus_free = sc->S.has_full_prims && !sc->csg_torus;
    CK(B.ensure(maxq, nl, nal, rad, sample_rays, sc->media_ni, sc->textured, transparent, sc->top_tori,
                torus_free));
    // transparent surfaces that also reflect: a ray may queue two rays, so
    // the queue sides and the per-pass scratch grow with the ray count
    // (the host reads each pass's count); rays carry their throughput
    const bool branching = transparent && sc->branching;
    size_t cap_work = maxq;                  // current rays the per-pass scratch holds
    size_t cap_side[2] = {maxq, maxq};       // rays each queue side (A, B) holds
    if (branching) {
        CK(B.ensure_side(0, maxq));
        CK(B.ensure_side(1, maxq));
    }
    TorusDefer tdc{}, tds{};   // closest-hit and any-hit launches
    const bool defer = sc->top_tori || torus_free;
    auto bind_work = [&]() {
        if (defer) {
            tdc.count = tds.count = B.counters.as<int>() + C_TC;
            tdc.ovf_count = tds.ovf_count = B.counters.as<int>() + C_TO;
            tdc.ovf_work = tds.ovf_work = B.counters.as<int>() + C_TW;
        }
        if (sc->top_tori) {
            tdc.cand = tds.cand = B.tcand.as<uint2>();
            tdc.cap = tds.cap = (int)tcand_cap(cap_work, nl);
            tdc.key = B.tkey.as<unsigned long long>();
        }
        if (torus_free) {
            tdc.ovf = tds.ovf = B.tovf.as<int>();
            tdc.ovf_cap = (int)cap_work;
            tds.ovf_cap = (int)(cap_work * nl);
        }
    };
    bind_work();
    cudaStream_t st = sc->active();
    int* cnt = B.counters.as<int>();
    unsigned long long* dstats = sc->stats.as<unsigned long long>();
    uint32_t* derr = sc->err.as<uint32_t>();
    unsigned long long* wc = (sc->profiling & POV_GPU_PROFILE_WORK) ? sc->wcount.as<unsigned long long>() : nullptr;
    const DeviceScene& S = sc->S;
    const int grid_trace = sc->num_sms * sc->lc.trace_blocks_per_sm;
    const int grid_shade = std::max(1, std::min(sc->num_sms * sc->lc.shade_blocks_per_sm, (int)((maxq + 127) / 128)));
    const int tblock = sc->lc.trace_block, tocc = sc->lc.trace_occupancy;
    const size_t max_area = maxq * (size_t)nal;
    // the queue sides: the current pass reads side `side`, fills the other
    int side = 0;
    QRay *qcur, *qnext;
    int *pcur, *pnext, *ccur, *cnext, *scur, *snext;
    uint2 *kcur, *knext;
    uint64_t *rcur, *rnext;
    float4 *tcur, *tnext;
    ShadeRad sr{};
    sr.rq = rad ? B.rq.as<RadQuery>() : nullptr;
    sr.rq_count = cnt + C_RQ;
    sr.rq_cap = (int)maxq;
    sr.adc = sample_rays ? (float)sc->rad.set.adc_bailout : S.adc_bailout;
    sr.gather = sample_rays ? 1 : 0;
    // media containers: rays carry their own level and medium; a ray that
    // crosses a container wall goes on at its level in the next pass, so
    // the passes run until the queue is empty (each pass raises a ray's
    // level or takes it across a wall: at most 1 + 2 * containers passes a
    // level)
    // Transparent surfaces likewise: a ray continued through a surface
    // with equal iors on both sides stays at its level; each pass takes
    // every ray across one surface, and a pass limit ends a frame whose
    // rays still cross surfaces after it with an error (no ray is dropped
    // silently).
    auto bind = [&]() {
        DevBuf* q[2] = {&B.qA, &B.qB};
        DevBuf* pa[2] = {&B.pathA, &B.pathB};
        DevBuf* sk[2] = {&B.skipA, &B.skipB};
        DevBuf* stt[2] = {&B.stateA, &B.stateB};
        DevBuf* ri[2] = {&B.rinA, &B.rinB};
        DevBuf* th[2] = {&B.thrA, &B.thrB};
        const int o = side ^ 1;
        qcur = q[side]->as<QRay>();
        qnext = q[o]->as<QRay>();
        pcur = pa[side]->as<int>();
        pnext = pa[o]->as<int>();
        ccur = cnt + (side ? C_QB : C_QA);
        cnext = cnt + (side ? C_QA : C_QB);
        kcur = sk[side]->as<uint2>();
        knext = sk[o]->as<uint2>();
        scur = staged ? stt[side]->as<int>() : nullptr;
        snext = staged ? stt[o]->as<int>() : nullptr;
        rcur = transparent ? ri[side]->as<uint64_t>() : nullptr;
        rnext = transparent ? ri[o]->as<uint64_t>() : nullptr;
        tcur = branching ? th[side]->as<float4>() : nullptr;
        tnext = branching ? th[o]->as<float4>() : nullptr;
    };
    bind();
    const int max_pass = media         ? (max_level - level0) * (1 + 2 * S.num_containers)
                         : transparent ? (max_level - level0) * TRANSPARENT_PASSES_PER_LEVEL
                                       : max_level - level0;
    if (staged)
        CK(launch_fill_int(scur, ccur, (int)maxq, ray_state(level0, -1), grid_shade, st));
    if (transparent)   // camera and sample rays start inside no interior
        CK(cudaMemsetAsync(rcur, 0, sizeof(uint64_t) * maxq, st));
    for (int pass = 0;; pass++) {
        const int level = level0 + pass;   // the level of every ray without media or transparency
        if (staged && pass > 0) {
            CK(cudaMemcpyAsync(sc->pin_int(1), ccur, sizeof(int), cudaMemcpyDeviceToHost, st));
            HW(st);
            if (*sc->pin_int(1) == 0)
                break;
            if (pass >= max_pass && transparent)
                return POV_GPU_E_CAPACITY;
        }
        if (pass >= max_pass)
            break;
        if (branching) {   // room for this pass's rays and up to two children each
            const size_t ncur = pass == 0 ? maxq : std::min((size_t)*sc->pin_int(1), cap_side[side]);
            if (ncur > cap_work) {
                CK(B.ensure_work(ncur, nl, sc->textured, sc->top_tori, torus_free));
                cap_work = ncur;
                bind_work();
            }
            const size_t need = std::max(2 * ncur, maxq);
            if (need > cap_side[side ^ 1]) {
                CK(B.ensure_side(side ^ 1, need));
                cap_side[side ^ 1] = need;
                bind();
            }
        }
        const int capq = (int)std::min(cap_work, cap_side[side]);   // the current queue's clamp
        CK(cudaMemsetAsync(cnext, 0, sizeof(int), st));
        CK(cudaMemsetAsync(cnt + C_SQ, 0, sizeof(int) * 3, st));   // SQ, W0, W1
        CK(cudaMemsetAsync(cnt + C_AQ, 0, sizeof(int) * 2, st));   // AQ, RQ
        CK(clk.begin(POV_GPU_STAGE_TRACE_CLOSEST));
        CK(launch_trace(S, false, qcur, ccur, cnt + C_W0, B.hits.as<QHit>(), nullptr, sc->stack_depth, grid_trace,
                        derr, dstats, wc, capq, kcur, st, tblock, tocc, defer ? &tdc : nullptr));
        CK(clk.end());
        if (sample_rays && pass == 0)
            CK(launch_first_hit(B.hits.as<QHit>(), ccur, (int)maxq, B.first_t.as<float>(), grid_shade, st));
        if (media && !sample_rays) {   // the radiosity Trace runs with media off
            CK(clk.begin(POV_GPU_STAGE_MEDIA));
            int nlaunch = 0;
            int rc = run_media(sc, B, qcur, scur, pcur, ccur, maxq, grid_trace, &nlaunch);
            if (rc != POV_GPU_OK)
                return rc;
            CK(clk.end(nlaunch));
        }
        CK(clk.begin(POV_GPU_STAGE_SHADE));
        ShadeMedia sm{scur, snext, media ? B.smedium.as<int>() : nullptr, rcur, rnext,
                      transparent ? B.srin.as<uint64_t>() : nullptr, pass > 0 ? tcur : nullptr, tnext,
                      branching ? 1 : 0, branching ? (int)cap_side[side ^ 1] : 0};
        const int* order = nullptr;
        if (sc->textured) {   // one material per warp in k_shade
            CK(launch_shade_bins(S, B.hits.as<QHit>(), ccur, capq, B.bin_keys.as<uint8_t>(),
                                 B.bin_hist.as<int>(), B.bin_order.as<int>(), grid_shade, st));
            order = B.bin_order.as<int>();
        }
        CK(launch_shade(S, level, max_level, qcur, pcur, B.hits.as<QHit>(), ccur, B.paths.as<PathState>(),
                        B.slot_contrib.as<float4>(), B.sq.as<QRay>(), B.sq_slot.as<int>(), cnt + C_SQ,
                        B.sskip.as<uint2>(), qnext, pnext, knext, cnext, capq, (int)((size_t)capq * nl),
                        B.aq.as<QRay>(), B.aq_slot.as<int>(), B.aq_skip.as<uint2>(), cnt + C_AQ, (int)max_area, sr,
                        sm, order, grid_shade, derr, dstats, st));
        CK(clk.end(sc->textured ? 4 : 1));
        if (nal > 0) {
            CK(clk.begin(POV_GPU_STAGE_AREA_SHADOW));
            CK(launch_area_shadow(S, B.aq.as<QRay>(), B.aq_slot.as<int>(), B.aq_skip.as<uint2>(), cnt + C_AQ,
                                  (int)max_area, B.slot_contrib.as<float4>(), sc->stack_depth, grid_shade, derr,
                                  dstats, st));
            CK(clk.end());
        }
        if (sc->num_lights > 0) {
            CK(clk.begin(POV_GPU_STAGE_TRACE_SHADOW));
            if (media)
                CK(launch_shadow_through(S, B.sq.as<QRay>(), B.sq_slot.as<int>(), B.sskip.as<uint2>(),
                                         B.smedium.as<int>(), cnt + C_SQ, (int)(maxq * nl), cnt + C_W1,
                                         B.blocked.as<uint8_t>(),
                                         B.slot_contrib.as<float4>(), !sample_rays, sc->stack_depth, grid_trace,
                                         derr, dstats, st));
            else if (transparent)
                CK(launch_shadow_filter(S, B.sq.as<QRay>(), B.sq_slot.as<int>(), B.sskip.as<uint2>(),
                                        B.srin.as<uint64_t>(), cnt + C_SQ, (int)((size_t)capq * nl), cnt + C_W1,
                                        B.blocked.as<uint8_t>(), B.slot_contrib.as<float4>(), sc->stack_depth,
                                        grid_trace, derr, dstats, st));
            else
                CK(launch_trace(S, true, B.sq.as<QRay>(), cnt + C_SQ, cnt + C_W1, nullptr, B.blocked.as<uint8_t>(),
                                sc->stack_depth, grid_trace, derr, dstats, wc ? wc + 4 : nullptr,
                                (int)((size_t)capq * nl), B.sskip.as<uint2>(), st, tblock, tocc,
                                defer ? &tds : nullptr));
            CK(clk.end());
            CK(clk.begin(POV_GPU_STAGE_RESOLVE));
            CK(launch_resolve(pcur, ccur, sc->num_lights, B.sq_slot.as<int>(), B.blocked.as<uint8_t>(), cnt + C_SQ,
                              B.slot_contrib.as<float4>(), B.paths.as<PathState>(), grid_shade, capq,
                              (int)((size_t)capq * nl), st, branching));
            CK(clk.end(2));
        }
        if (rad) {
            CK(cudaMemcpyAsync(sc->pin_int(2), cnt + C_RQ, sizeof(int), cudaMemcpyDeviceToHost, st));
            HW(st);
            const int nq = std::min(*sc->pin_int(2), (int)maxq);
            if (nq > 0) {
                int rc = rad_resolve(sc, clk, hit_depth, B.rq.as<RadQuery>(), nq, B.rq_amb.as<float4>());
                if (rc != POV_GPU_OK)
                    return rc;
                CK(clk.begin(POV_GPU_STAGE_RADIOSITY));
                CK(launch_rad_apply(B.rq.as<RadQuery>(), cnt + C_RQ, (int)maxq, B.rq_amb.as<float4>(),
                                    B.paths.as<PathState>(), sample_rays ? B.quality.as<float>() : nullptr,
                                    grid_shade, st));
                CK(clk.end());
            }
        }
        side ^= 1;
        bind();
    }
    return POV_GPU_OK;
}

// New samples for `ns` queries of bounce depth d (RadiosityFunction::
// GatherLight, radiosity.cpp:509-756): count sample rays each, traced as
// one wavefront by the radiosity Trace starting at the depth's trace level
// (radiosity.cpp:544-549), then reduced per seed into the new block and the
// seed's ambient answer.
int rad_gather(PovGpuScene* sc, StageClock& clk, int d, const RadQuery* queries, const int* seeds, int ns,
               const float4* partial, float4* out)
{
    RadiosityState& R = sc->rad;
    const RadParams P = rad_params(sc, d);
    PathBufs& B = R.level[d].rays;
    const int count = P.rays_per_sample;
    const size_t nr = (size_t)ns * count;
    const bool nested = d + 1 < R.set.recursion_limit;
    CK(B.ensure(nr, std::max(sc->num_lights, 1), 0, nested, true));
    cudaStream_t st = sc->active();
    int* cnt = B.counters.as<int>();
    const int grid = std::max(1, std::min(sc->num_sms * 16, (int)((nr + 255) / 256)));
    CK(cudaMemsetAsync(cnt, 0, sizeof(int) * C_NUM, st));
    const int base = R.dir_base[d];
    CK(clk.begin(POV_GPU_STAGE_RADIOSITY));
    CK(launch_gather_rays(queries, seeds, ns, count, base, P.gather_weight, B.qA.as<QRay>(), B.pathA.as<int>(),
                          B.skipA.as<uint2>(), B.paths.as<PathState>(), B.quality.as<float>(), cnt + C_QA,
                          sc->stats.as<unsigned long long>(), grid, st));
    CK(clk.end());
    R.dir_base[d] = (int)(((long long)base + (long long)nr) % RAD_DIRECTIONS);
    R.rays_shot += nr;
    const int tl = (int)(1.5 * (d + 1));
    const int maxl = std::max(sc->max_trace_level, tl + 1);
    int rc = run_levels(sc, clk, B, nr, tl, maxl, d + 1, true);
    if (rc != POV_GPU_OK)
        return rc;
    CK(clk.begin(POV_GPU_STAGE_RADIOSITY));
    CK(launch_gather_reduce(sc->S, cache_view(sc), P, queries, seeds, ns, base, B.first_t.as<float>(),
                            B.paths.as<PathState>(), B.quality.as<float>(), partial, out,
                            R.rstats.as<unsigned long long>(), sc->err.as<uint32_t>(),
                            std::max(1, std::min(sc->num_sms * 16, (ns * 32 + 127) / 128)), st));
    CK(clk.end());
    R.seg_dirty = true;   // the new blocks join their nodes at the next query round
    return POV_GPU_OK;
}

// Answers n radiosity queries of bounce depth d into out[] (ambient colour,
// quality): rounds of cache queries and gathers, see povgpu_radiosity.cu.
int rad_resolve(PovGpuScene* sc, StageClock& clk, int d, const RadQuery* queries, int n, float4* out)
{
    RadiosityState& R = sc->rad;
    if (d >= RAD_LEVELS)
        return POV_GPU_E_UNSUPPORTED;
    RadLevel& L = R.level[d];
    CK(L.ensure((size_t)n));
    const RadParams P = rad_params(sc, d);
    const RadCacheView C = cache_view(sc);
    cudaStream_t st = sc->active();
    int* cn = L.counts.as<int>();
    int* lists[2] = {L.open.as<int>(), L.next.as<int>()};
    const int* open = nullptr;
    int n_open = n;
    const int grid = std::max(1, std::min(sc->num_sms * 16, (n + 127) / 128));
    const int per_chunk = std::max(1, (int)(GATHER_CHUNK_RAYS / (size_t)P.rays_per_sample));
    // final trace with a trained neural cache: one round; what no cached
    // sample covers is answered by the network instead of a new gather
    const bool use_nic = R.nic_ok && d == 0 && R.final_trace;
    const int last_round = use_nic ? 0 : RAD_ROUNDS - 1;
    for (int round = 0; round <= last_round && n_open > 0; round++) {
        int* nxt = lists[round & 1];
        CK(cudaMemsetAsync(cn, 0, sizeof(int) * 2, st));
        CK(cudaMemsetAsync(L.claims.p, 0, L.claims.bytes, st));
        CK(clk.begin(POV_GPU_STAGE_RADIOSITY));
        if (R.seg_dirty) {   // file the blocks added since the last rebuild
            CK(launch_seg_rebuild(C, sc->num_sms * 4, st));
            R.seg_dirty = false;
        }
        // one warp per open query
        const int qgrid = std::max(1, std::min(sc->num_sms * 16, (int)(((long)n_open * 32 + 127) / 128)));
        CK(launch_rad_query(sc->S, C, P, queries, open, n_open, n, round, last_round, out,
                            L.partial.as<float4>(), L.claims.as<unsigned long long>(), L.claim_mask(),
                            L.seeds.as<int>(), cn, nxt, cn + 1, R.rstats.as<unsigned long long>(),
                            sc->err.as<uint32_t>(), qgrid, st));
        CK(clk.end());
        CK(cudaMemcpyAsync(sc->pin_int(3), cn, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
        HW(st);
        const int ns = std::min(*sc->pin_int(3), n), nn = std::min(*sc->pin_int(4), n);
        if (use_nic) {
            if (ns > 0) {
                CK(R.nic_pred.ensure(sizeof(float4) * (size_t)ns));
                nic::NicIO io{};
                io.pos = reinterpret_cast<const float4*>(queries);
                io.nrm = reinterpret_cast<const float4*>(queries) + 1;
                io.stride = (int)(sizeof(RadQuery) / sizeof(float4));
                io.idx = L.seeds.as<int>();
                io.n = ns;
                io.out = R.nic_pred.as<float4>();
                io.lo = R.nic_lo;
                io.scale = R.nic_scale;
                CK(clk.begin(POV_GPU_STAGE_RADIOSITY));
                CK(nic::launch_forward(io, R.nic_wb.as<unsigned char>(), R.nic_params.as<float>(),
                                       sc->err.as<uint32_t>(), sc->num_sms * 2, st));
                CK(launch_rad_nic_answer(P, L.seeds.as<int>(), ns, R.nic_pred.as<float4>(), out,
                                         R.rstats.as<unsigned long long>(), grid, st));
                CK(clk.end(2));
            }
            break;
        }
        for (int c0 = 0; c0 < ns; c0 += per_chunk) {
            int rc = rad_gather(sc, clk, d, queries, L.seeds.as<int>() + c0, std::min(per_chunk, ns - c0),
                                L.partial.as<float4>(), out);
            if (rc != POV_GPU_OK)
                return rc;
        }
        open = nxt;
        n_open = nn;
    }
    return POV_GPU_OK;
}

// Traces `n` image samples through every trace level and writes their RGBT
// to out[slot[i]] (slot == nullptr: out[i]).  Samples come from the block
// list (mode 0 centres, mode 1 corners) or from `pos` (mode 2, count in the
// device word `npos`).  Counters accumulate into sc->stats.
int run_samples(PovGpuScene* sc, StageClock& clk, int mode, int nblocks, const int* block_off, const double2* pos,
                const int* npos, int n, int width, int height, const int* slot, float4* out)
{
    PathBufs& B = sc->top;
    const size_t maxq = (size_t)std::max(n, 1);
    CK(B.ensure(maxq, std::max(sc->num_lights, 1), sc->S.num_area_lights, sc->rad.enabled, false));
    cudaStream_t st = sc->active();
    int* cnt = B.counters.as<int>();
    CK(cudaMemsetAsync(cnt, 0, sizeof(int) * C_NUM, st));
    if (mode != 2)
        CK(sc->cam_tab.ensure(sizeof(float2) * ((size_t)width + (size_t)height + 2)));
    CK(clk.begin(POV_GPU_STAGE_CAMERA));
    CK(launch_camera(sc->S, mode, sc->blocks.as<int4>(), block_off, nblocks, pos, npos, n, width, height,
                     B.qA.as<QRay>(), B.pathA.as<int>(), B.paths.as<PathState>(), cnt + C_QA,
                     sc->stats.as<unsigned long long>(), B.skipA.as<uint2>(), sc->cam_tab.as<float2>(), st));
    CK(clk.end(mode != 2 ? 2 : 1));
    int rc = run_levels(sc, clk, B, maxq, 0, sc->max_trace_level, 0, false);
    if (rc != POV_GPU_OK)
        return rc;
    // finalize reads the sample count from the block offsets / position count
    CK(clk.begin(POV_GPU_STAGE_FINALIZE));
    CK(launch_finalize(B.paths.as<PathState>(), mode == 2 ? npos : block_off + nblocks, (int)maxq, slot, out, st));
    CK(clk.end());
    return POV_GPU_OK;
}

// Radiosity counters of the call into the public statistics.
int rad_collect(PovGpuScene* sc, PovGpuStats* stats)
{
    if (!sc->rad.enabled || !stats)
        return POV_GPU_OK;
    unsigned long long h[RST_COUNT] = {0};
    CK(cudaMemcpy(h, sc->rad.rstats.p, sizeof(h), cudaMemcpyDeviceToHost));
    stats->radiosity_reuse = h[RST_REUSED];
    stats->radiosity_gathers_d0 = h[RST_GATHERS0];
    stats->radiosity_gathers_d1 = h[RST_GATHERS1];
    stats->radiosity_gathers = h[RST_GATHERS0] + h[RST_GATHERS1];
    stats->radiosity_rays = sc->rad.rays_shot;
    stats->nic_answers = h[RST_NIC];
    stats->nic_val_error_ppm = sc->rad.nic_cfg.enabled ? (uint64_t)(sc->rad.nic_val_error * 1e6) : 0;
    return POV_GPU_OK;
}

// Trains the neural cache on the depth-0 samples of the cache (every eighth
// held out) and decides the gate.  Runs at the end of the pretrace.
int nic_train(PovGpuScene* sc)
{
    RadiosityState& R = sc->rad;
    const PovGpuNeuralCache& cfg = R.nic_cfg;
    R.nic_ok = false;
    R.nic_val_error = 0.0;
    cudaStream_t st = sc->active();
    int nb = 0;
    CK(cudaMemcpyAsync(&nb, R.count.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    HW(st);
    nb = std::min(nb, R.cap_blocks);
    if (nb <= 0)
        return POV_GPU_OK;
    std::vector<RadBlock> hb((size_t)nb);
    CK(cudaMemcpy(hb.data(), R.blocks.p, sizeof(RadBlock) * (size_t)nb, cudaMemcpyDeviceToHost));
    std::vector<int> train, val;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < nb; i++) {
        const RadBlock& b = hb[i];
        int depth;
        std::memcpy(&depth, &b.ill.w, sizeof(int));
        if (depth != 0)
            continue;
        (((train.size() + val.size()) % 8) == 7 ? val : train).push_back(i);
        const float p[3] = {b.p.x, b.p.y, b.p.z};
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    if (train.size() < 256 || val.empty())
        return POV_GPU_OK;
    // a shared network keeps its weights, Adam moments and input bounds
    // from the pretraces before (other views of the same scene)
    const bool resume = cfg.shared && R.nic_init;
    if (!resume) {
        float sc3[3];
        for (int k = 0; k < 3; k++) {
            float ext = std::max(hi[k] - lo[k], 1e-6f);
            lo[k] -= 0.01f * ext;
            sc3[k] = 2.0f / (1.02f * ext);
        }
        R.nic_lo = make_float3(lo[0], lo[1], lo[2]);
        R.nic_scale = make_float3(sc3[0], sc3[1], sc3[2]);
        R.nic_step = 0;
    }
    // parameters: He-uniform initialisation, zero biases, padded rows zero
    const size_t NP = (size_t)nic::NPARAM;
    CK(R.nic_params.ensure(sizeof(float) * NP));
    CK(R.nic_wb.ensure(nic::WIMG_BYTES));
    CK(R.nic_m.ensure(sizeof(float) * NP));
    CK(R.nic_v.ensure(sizeof(float) * NP));
    // batch 0: one 128-sample tile per SM, every SM busy in each step
    const int steps = std::max(cfg.steps, 1),
              batch = cfg.batch > 0 ? std::max(cfg.batch, nic::TILE) : nic::TILE * sc->num_sms;
    const int slices = nic::train_slices(batch, sc->num_sms);
    CK(R.nic_grad.ensure(sizeof(float) * NP * (size_t)slices));
    CK(R.nic_loss.ensure(sizeof(float) * (size_t)slices));
    CK(R.nic_err.ensure(sizeof(uint32_t)));
    std::mt19937 rng(cfg.seed + (uint32_t)R.nic_step);
    std::vector<float> hp(NP, 0.0f);
    auto init = [&](int off, int rows, int cols, int live_rows) {
        std::uniform_real_distribution<float> u(-std::sqrt(6.0f / cols), std::sqrt(6.0f / cols));
        for (int r = 0; r < live_rows; r++)
            for (int c = 0; c < cols; c++)
                hp[(size_t)off + (size_t)r * cols + c] = (cols == nic::K1 && c >= nic::FEAT) ? 0.0f : u(rng);
        (void)rows;
    };
    init(nic::P_W1, nic::HID, nic::K1, nic::HID);
    init(nic::P_W2, nic::HID, nic::HID, nic::HID);
    init(nic::P_W3, nic::HID, nic::HID, nic::HID);
    init(nic::P_W4, nic::HID, nic::HID, nic::HID);
    init(nic::P_W5, nic::NO, nic::HID, nic::NOUT);
    if (!resume) {
        CK(cudaMemcpyAsync(R.nic_params.p, hp.data(), sizeof(float) * NP, cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(R.nic_m.p, 0, sizeof(float) * NP, st));
        CK(cudaMemsetAsync(R.nic_v.p, 0, sizeof(float) * NP, st));
        CK(nic::launch_to_bf16(R.nic_params.as<float>(), R.nic_wb.as<unsigned char>(), st));
        R.nic_init = true;
    }
    CK(cudaMemsetAsync(R.nic_err.p, 0, sizeof(uint32_t), st));
    // every step's batch, drawn up front
    std::vector<int> idx((size_t)steps * batch + val.size());
    std::uniform_int_distribution<int> pick(0, (int)train.size() - 1);
    for (size_t i = 0; i < (size_t)steps * batch; i++)
        idx[i] = train[(size_t)pick(rng)];
    std::copy(val.begin(), val.end(), idx.begin() + (size_t)steps * batch);
    CK(R.nic_idx.ensure(sizeof(int) * idx.size()));
    CK(cudaMemcpyAsync(R.nic_idx.p, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, st));
    nic::NicIO io{};
    io.pos = reinterpret_cast<const float4*>(R.blocks.p);
    io.nrm = io.pos + 1;
    io.target = io.pos + 3;
    io.stride = (int)(sizeof(RadBlock) / sizeof(float4));
    io.lo = R.nic_lo;
    io.scale = R.nic_scale;
    StageClock clk(sc, st);
    CK(clk.begin(POV_GPU_STAGE_RADIOSITY));
    for (int s = 0; s < steps; s++) {
        io.idx = R.nic_idx.as<int>() + (size_t)s * batch;
        io.n = batch;
        CK(nic::launch_train(io, R.nic_wb.as<unsigned char>(), R.nic_params.as<float>(), R.nic_grad.as<float>(),
                             R.nic_loss.as<float>(), 1.0f / (float)batch, R.nic_err.as<uint32_t>(), sc->num_sms,
                             st));
        CK(nic::launch_adam(R.nic_params.as<float>(), R.nic_m.as<float>(), R.nic_v.as<float>(),
                            R.nic_grad.as<float>(), slices, R.nic_wb.as<unsigned char>(), cfg.learning_rate,
                            R.nic_step + s + 1, st));
    }
    R.nic_step += steps;
    CK(clk.end(2 * steps));
    // held-out relative RMSE
    const int nv = (int)val.size();
    CK(R.nic_pred.ensure(sizeof(float4) * (size_t)nv));
    io.idx = R.nic_idx.as<int>() + (size_t)steps * batch;
    io.n = nv;
    io.out = R.nic_pred.as<float4>();
    CK(nic::launch_forward(io, R.nic_wb.as<unsigned char>(), R.nic_params.as<float>(), R.nic_err.as<uint32_t>(),
                           sc->num_sms * 2, st));
    std::vector<float4> pred((size_t)nv);
    uint32_t nerr = 0;
    CK(cudaMemcpyAsync(pred.data(), R.nic_pred.p, sizeof(float4) * (size_t)nv, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&nerr, R.nic_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    HW(st);
    double se = 0.0, sy = 0.0;
    for (int i = 0; i < nv; i++) {
        const RadBlock& b = hb[(size_t)val[i]];
        const float y[3] = {b.ill.x, b.ill.y, b.ill.z}, p[3] = {pred[i].x, pred[i].y, pred[i].z};
        for (int k = 0; k < 3; k++) {
            se += (double)(p[k] - y[k]) * (p[k] - y[k]);
            sy += (double)y[k];
        }
    }
    double mean = sy / (3.0 * nv);
    R.nic_val_error = mean > 0 ? std::sqrt(se / (3.0 * nv)) / mean : 1.0;
    R.nic_ok = nerr == 0 && R.nic_val_error <= cfg.gate;
    return nerr ? POV_GPU_E_DEVICE : POV_GPU_OK;
}

int rad_begin_call(PovGpuScene* sc, bool final_trace)
{
    RadiosityState& R = sc->rad;
    if (!R.enabled)
        return POV_GPU_OK;
    R.final_trace = final_trace;
    R.error_bound = R.set.error_bound * (final_trace ? 1.0 : R.set.low_error_factor);
    R.rays_shot = 0;
    CK(cudaMemsetAsync(R.rstats.p, 0, sizeof(unsigned long long) * RST_COUNT, sc->active()));
    return POV_GPU_OK;
}

// The device work of a plain frame, run through a CUDA graph: the first
// call of a frame shape runs it directly (which sizes every buffer), the
// second captures it into a graph and launches that, later calls of the
// same shape (same pixel count, blocks, image size, output buffer, work
// buffers, launch shapes and scene/camera state) launch the graph alone --
// one launch instead of ~17.  The kernels read their queue counts from
// device memory, so the captured sequence is the frame for any block list
// of that shape; the block list itself is copied before the graph runs.
int trace_plain_graph(PovGpuScene* sc, StageClock& clk, int num_blocks, int n, int width, int height, float4* dout)
{
    cudaStream_t st = sc->active();
    PovGpuScene::GraphKey key;
    std::memset(&key, 0, sizeof(key));
    key.n = n;
    key.nblocks = num_blocks;
    key.width = width;
    key.height = height;
    key.out = dout;
    const DevBuf* bufs[] = {&sc->top.qA, &sc->top.qB, &sc->top.pathA, &sc->top.pathB, &sc->top.hits,
                            &sc->top.paths, &sc->top.slot_contrib, &sc->top.sq, &sc->top.sq_slot, &sc->top.blocked,
                            &sc->top.sskip, &sc->top.aq, &sc->top.bin_order, &sc->cam_tab, &sc->blocks,
                            &sc->block_off};
    static_assert(sizeof(bufs) / sizeof(bufs[0]) == sizeof(key.bufs) / sizeof(key.bufs[0]), "graph key buffers");
    for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++)
        key.bufs[i] = bufs[i]->p;
    std::memcpy(&key.lc, &sc->lc, sizeof(key.lc));
    std::memcpy(&key.S, &sc->S, sizeof(key.S));   // bytes, padding included, for the comparison
    auto same = [](const PovGpuScene::GraphKey& a, const PovGpuScene::GraphKey& b) {
        return std::memcmp(&a, &b, sizeof(a)) == 0;
    };
    auto body = [&]() -> int {
        CK(cudaMemsetAsync(sc->counters.p, 0, sizeof(int) * C_NUM, st));
        CK(cudaMemsetAsync(sc->stats.p, 0, sizeof(unsigned long long) * ST_COUNT, st));
        CK(cudaMemsetAsync(sc->err.p, 0, sizeof(uint32_t) * 4, st));
        return run_samples(sc, clk, 0, num_blocks, sc->block_off.as<int>(), nullptr, nullptr, n, width, height,
                           nullptr, dout);
    };
    if (sc->graph_exec && same(key, sc->graph_key)) {
        CK(cudaGraphLaunch(sc->graph_exec, st));
        sc->timings.kernel_launches += sc->graph_launches;
        return POV_GPU_OK;
    }
    if (!(sc->graph_last_valid && same(key, sc->graph_last))) {
        // first call of this shape: run directly; it sizes the buffers
        int rc = body();
        // the buffers may have grown: the key is taken after the run
        for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++)
            key.bufs[i] = bufs[i]->p;
        sc->graph_last = key;
        sc->graph_last_valid = rc == POV_GPU_OK;
        return rc;
    }
    // second call of the shape: capture, then launch
    const uint32_t launches0 = sc->timings.kernel_launches;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = body();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc != POV_GPU_OK || e != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        cudaGetLastError();
        sc->graph_last_valid = false;
        return rc != POV_GPU_OK ? rc : POV_GPU_E_CUDA;
    }
    if (sc->graph_exec)
        cudaGraphExecDestroy(sc->graph_exec);
    sc->graph_exec = nullptr;
    e = cudaGraphInstantiate(&sc->graph_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        sc->graph_exec = nullptr;
        return POV_GPU_E_CUDA;
    }
    sc->graph_key = key;
    sc->graph_launches = sc->timings.kernel_launches - launches0;
    CK(cudaGraphLaunch(sc->graph_exec, st));
    return POV_GPU_OK;
}

}  // namespace

extern "C" {

int pov_gpu_abi_version(void) { return POV_GPU_ABI_VERSION; }

const char* pov_gpu_error_string(int status)
{
    switch (status) {
    case POV_GPU_OK: return "ok";
    case POV_GPU_E_INVALID: return "invalid argument or scene description";
    case POV_GPU_E_UNSUPPORTED: return "object, texture or light not supported by the GPU trace path";
    case POV_GPU_E_CUDA: return "CUDA runtime error";
    case POV_GPU_E_TIMEOUT: return "host wait limit reached (pov_gpu_set_timeout); device work still queued";
    case POV_GPU_E_NOMEM: return "device memory allocation failed";
    case POV_GPU_E_DEVICE: return "kernel reported an error in its device error word";
    case POV_GPU_E_NODEVICE: return "no CUDA device";
    case POV_GPU_E_CAPACITY: return "request exceeds the fixed scratch capacity (POV_GPU_STATIC_MAX_RAYS rays)";
    default: return "unknown status";
    }
}

int pov_gpu_scene_create(const PovGpuSceneDesc* desc, PovGpuScene** out, int32_t* bad_index)
{
    if (bad_index)
        *bad_index = -1;
    if (!out)
        return POV_GPU_E_INVALID;
    *out = nullptr;
    int st = validate(desc, bad_index);
    if (st != POV_GPU_OK)
        return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
        return POV_GPU_E_NODEVICE;
    PovGpuScene* sc = new (std::nothrow) PovGpuScene();
    if (!sc)
        return POV_GPU_E_NOMEM;
    cudaGetDevice(&sc->device);
    cudaDeviceGetAttribute(&sc->num_sms, cudaDevAttrMultiProcessorCount, sc->device);
    if (cudaStreamCreateWithFlags(&sc->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete sc;
        return POV_GPU_E_CUDA;
    }
    if (cudaHostAlloc(reinterpret_cast<void**>(&sc->pinned), PovGpuScene::PIN_BYTES, cudaHostAllocDefault) !=
        cudaSuccess) {
        sc->release_all();
        delete sc;
        return POV_GPU_E_NOMEM;
    }
    std::memset(sc->pinned, 0, PovGpuScene::PIN_BYTES);
    st = build_scene(sc, desc);
    if (st == POV_GPU_OK) {
        if (sc->counters.ensure(sizeof(int) * C_NUM) != cudaSuccess ||
            sc->stats.ensure(sizeof(unsigned long long) * ST_COUNT) != cudaSuccess ||
            sc->err.ensure(sizeof(uint32_t) * 4) != cudaSuccess)
            st = POV_GPU_E_NOMEM;
    }
    if (st != POV_GPU_OK) {
        sc->release_all();
        delete sc;
        return st;
    }
    *out = sc;
    return POV_GPU_OK;
}

void pov_gpu_scene_destroy(PovGpuScene* scene)
{
    if (!scene)
        return;
    cudaStreamSynchronize(scene->active());
    scene->release_all();
    delete scene;
}

// Cache files: the reference's .rca text format, one "C" line per sample
// (ot_write_block, source/core/support/octree.cpp:1345-1370: 1-based bounce
// depth, point, packed normal, illuminance, harmonic mean and nearest
// distance, packed direction to the nearest surface); read back as
// RadiosityCache::Load reads it (radiosity.cpp:909-1010: packed vectors
// unpacked and normalised, quality 1).
namespace {

unsigned pack_unit(float v) { return (unsigned)((v + 1.0) * 0.5 * 254.0 + 0.499999); }

double unpack_unit(unsigned u) { return ((double)u * (1.0 / 254.0)) * 2.0 - 1.0; }

void unpack_dir(const char* s, double out[3])
{
    unsigned t[3] = {0, 0, 0};
    std::sscanf(s, "%02x%02x%02x", &t[0], &t[1], &t[2]);
    double len = 0.0;
    for (int k = 0; k < 3; k++) {
        out[k] = unpack_unit(t[k]);
        len += out[k] * out[k];
    }
    len = std::sqrt(len);
    for (int k = 0; k < 3; k++)
        out[k] = len > 0.0 ? out[k] / len : 0.0;
}

}  // namespace

int pov_gpu_cache_save(PovGpuScene* sc, const char* path)
{
    if (!sc || !path)
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    RadiosityState& R = sc->rad;
    if (!R.enabled)
        return POV_GPU_E_INVALID;
    CK(cudaSetDevice(sc->device));
    if (int bc = begin_call(sc))
        return bc;
    cudaStream_t st = sc->active();
    int nb = 0;
    CK(cudaMemcpyAsync(&nb, R.count.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    HW(st);
    nb = std::min(nb, R.cap_blocks);
    std::vector<RadBlock> hb((size_t)std::max(nb, 0));
    if (nb > 0) {
        CK(cudaMemcpyAsync(hb.data(), R.blocks.p, sizeof(RadBlock) * (size_t)nb, cudaMemcpyDeviceToHost, st));
        HW(st);
    }
    std::FILE* f = std::fopen(path, "w");
    if (!f)
        return POV_GPU_E_INVALID;
    for (const RadBlock& b : hb) {
        int depth;
        std::memcpy(&depth, &b.ill.w, sizeof(int));
        std::fprintf(f, "C%d\t%g\t%g\t%g\t%02x%02x%02x\t%.4f\t%.4f\t%.4f\t%g\t%g\t%02x%02x%02x\n", depth + 1,
                     (double)b.p.x, (double)b.p.y, (double)b.p.z, pack_unit(b.n.x), pack_unit(b.n.y), pack_unit(b.n.z),
                     (double)b.ill.x, (double)b.ill.y, (double)b.ill.z, (double)b.p.w, (double)b.n.w,
                     pack_unit(b.tn.x), pack_unit(b.tn.y), pack_unit(b.tn.z));
    }
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok ? POV_GPU_OK : POV_GPU_E_INVALID;
}

int pov_gpu_cache_load(PovGpuScene* sc, const char* path, int32_t* loaded)
{
    if (loaded)
        *loaded = 0;
    if (!sc)
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    RadiosityState& R = sc->rad;
    if (!R.enabled)
        return POV_GPU_E_INVALID;
    std::vector<RadBlock> blocks;
    if (path) {
        std::FILE* f = std::fopen(path, "r");
        if (!f)
            return POV_GPU_E_INVALID;
        char line[256];
        while (std::fgets(line, sizeof(line), f)) {
            if (line[0] != 'C')
                continue;   // B and P lines carry nothing the cache uses; others are skipped
            int depth = 0;
            double p[3], hmd = 0.0, nearest = 0.0;
            float ill[3];
            char ns[32], tns[32];
            if (std::sscanf(line, "C%d %lf %lf %lf %31s %f %f %f %lf %lf %31s", &depth, &p[0], &p[1], &p[2], ns,
                            &ill[0], &ill[1], &ill[2], &hmd, &nearest, tns) != 11)
                continue;
            depth -= 1;   // the file counts bounce depths from 1
            if (depth < 0 || depth >= RAD_LEVELS)
                continue;
            double n[3], tn[3];
            unpack_dir(ns, n);
            unpack_dir(tns, tn);
            RadBlock b;
            b.p = make_float4((float)p[0], (float)p[1], (float)p[2], (float)hmd);
            b.n = make_float4((float)n[0], (float)n[1], (float)n[2], (float)nearest);
            b.tn = make_float4((float)tn[0], (float)tn[1], (float)tn[2], 1.0f);
            int32_t dbits = depth;
            float dw;
            std::memcpy(&dw, &dbits, sizeof(float));
            b.ill = make_float4(ill[0], ill[1], ill[2], dw);
            blocks.push_back(b);
        }
        std::fclose(f);
        if ((int)blocks.size() > R.cap_blocks)
            return POV_GPU_E_CAPACITY;
    }
    CK(cudaSetDevice(sc->device));
    if (int bc = begin_call(sc))
        return bc;
    R.loaded.swap(blocks);
    if (int rc = rad_reset(sc))
        return rc;
    if (loaded)
        *loaded = (int32_t)R.loaded.size();
    return POV_GPU_OK;
}

int pov_gpu_set_launch_config(PovGpuScene* sc, const PovGpuLaunchConfig* cfg)
{
    if (!sc || !cfg)
        return POV_GPU_E_INVALID;
    PovGpuLaunchConfig c = *cfg;
    if (c.trace_blocks_per_sm == 0)
        c.trace_blocks_per_sm = 8;
    if (c.trace_block == 0)
        c.trace_block = 128;
    if (c.shade_blocks_per_sm == 0)
        c.shade_blocks_per_sm = 16;
    if (c.trace_blocks_per_sm < 1 || c.trace_blocks_per_sm > 32 || (c.trace_block != 64 && c.trace_block != 128) ||
        (c.trace_occupancy != 0 && c.trace_occupancy != 1) || c.shade_blocks_per_sm < 1 ||
        c.shade_blocks_per_sm > 64 || (c.bounding_tree != 0 && c.bounding_tree != 1))
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    if (c.bounding_tree != sc->tree_mode) {
        CK(cudaSetDevice(sc->device));
        CK(cudaStreamSynchronize(sc->active()));   // no traversal may run on the old tree
        const int rc = apply_tree(sc, c.bounding_tree);
        if (rc != POV_GPU_OK)
            return rc;
    }
    sc->lc = c;
    return POV_GPU_OK;
}

int pov_gpu_get_tree_info(PovGpuScene* sc, PovGpuTreeInfo* info)
{
    if (!sc || !info)
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    std::memset(info, 0, sizeof(*info));
    info->bounding_tree = sc->tree_mode;
    if (sc->tree_mode == 1) {
        info->nodes = (int32_t)sc->ref_output.nodes.size();
        info->depth = sc->ref_output.depth;
    } else {
        info->nodes = sc->sah_nodes;
        info->depth = sc->sah_depth;
    }
    info->ref_top_nodes = sc->ref_built ? sc->ref_output.top_nodes : -1;
    info->ref_mesh_nodes = sc->ref_built ? sc->ref_output.mesh_nodes : -1;
    return POV_GPU_OK;
}

int pov_gpu_set_timeout(PovGpuScene* sc, double seconds)
{
    if (!sc || !(seconds >= 0.0) || !std::isfinite(seconds))
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    sc->timeout_s = seconds;
    return POV_GPU_OK;
}

int pov_gpu_scene_set_stream(PovGpuScene* sc, void* cuda_stream)
{
    if (!sc)
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    sc->user_stream = reinterpret_cast<cudaStream_t>(cuda_stream);
    return POV_GPU_OK;
}

int pov_gpu_set_camera(PovGpuScene* sc, const PovGpuCamera* cam, const double* look_at, const double* sky)
{
    if (!sc || !cam)
        return POV_GPU_E_INVALID;
    if (cam->type != 0)
        return POV_GPU_E_UNSUPPORTED;
    double loc[3], dir[3], right[3], up[3];
    for (int k = 0; k < 3; k++) {
        loc[k] = cam->location[k];
        dir[k] = cam->direction[k];
        right[k] = cam->right[k];
        up[k] = cam->up[k];
    }
    auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    auto cross = [](const double* a, const double* b, double* o) {
        double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
        o[0] = x;
        o[1] = y;
        o[2] = z;
    };
    if (look_at) {
        // View::StartRender applies look_at to the view camera
        // (source/backend/scene/view.cpp:922-975): lengths and handedness
        // kept, direction towards look_at, right from sky x direction
        // (unchanged when degenerate), up = direction x right
        const double sk[3] = {sky ? sky[0] : 0.0, sky ? sky[1] : 1.0, sky ? sky[2] : 0.0};
        const double dlen = std::sqrt(dot(dir, dir)), ulen = std::sqrt(dot(up, up)), rlen = std::sqrt(dot(right, right));
        double t[3];
        cross(up, dir, t);
        const double hand = dot(t, right);
        for (int k = 0; k < 3; k++)
            dir[k] = look_at[k] - loc[k];
        if (dot(dir, dir) < EPSILON)
            return POV_GPU_E_INVALID;   // location and look_at must differ
        double l = std::sqrt(dot(dir, dir));
        for (double& v : dir)
            v /= l;
        double r[3];
        cross(sk, dir, r);
        if (!(std::fabs(r[0]) < EPSILON && std::fabs(r[1]) < EPSILON && std::fabs(r[2]) < EPSILON))
            for (int k = 0; k < 3; k++)
                right[k] = r[k];
        l = std::sqrt(dot(right, right));
        for (double& v : right)
            v /= l;
        cross(dir, right, up);
        for (int k = 0; k < 3; k++) {
            dir[k] *= dlen;
            right[k] *= hand > 0.0 ? rlen : -rlen;
            up[k] *= ulen;
        }
    }
    std::lock_guard<std::mutex> g(sc->lock);
    if (int bc = begin_call(sc))
        return bc;
    // camera rays start outside every media container
    if (!sc->h_containers.empty()) {
        PovGpuSceneDesc dd{};
        dd.num_objects = (int32_t)sc->h_objects.size();
        dd.objects = sc->h_objects.data();
        for (int32_t c : sc->h_containers)
            if (host_inside(&dd, c, loc))
                return POV_GPU_E_UNSUPPORTED;
    }
    for (int k = 0; k < 3; k++) {
        sc->S.cam_loc[k] = loc[k];
        sc->S.cam_dir[k] = dir[k];
        sc->S.cam_right[k] = right[k];
        sc->S.cam_up[k] = up[k];
    }
    set_camera_ff(sc->S);
    return POV_GPU_OK;
}

int pov_gpu_encode_u8(PovGpuScene* sc, const float* rgbt, int64_t npix, int32_t curve, uint8_t* out)
{
    if (!sc || npix < 0 || (npix > 0 && (!rgbt || !out)) ||
        (curve != POV_GPU_CURVE_SRGB && curve != POV_GPU_CURVE_BT709))
        return POV_GPU_E_INVALID;
    if (npix == 0)
        return POV_GPU_OK;
    std::lock_guard<std::mutex> g(sc->lock);
    CK(cudaSetDevice(sc->device));
    if (int bc = begin_call(sc))
        return bc;
    cudaPointerAttributes in{}, oa{};
    CK(cudaPointerGetAttributes(&in, rgbt));
    if (in.type != cudaMemoryTypeDevice && in.type != cudaMemoryTypeManaged)
        return POV_GPU_E_INVALID;   // the pixels must already be on the device
    // midpoints of neighbouring decoded levels, in FP32 as IntEncode forms them
    auto decode = [curve](float x) {
        if (curve == POV_GPU_CURVE_BT709)   // colourspace.cpp:211-222
            return x < 0.081f ? x / 4.5f : std::pow((x + 0.099f) / 1.099f, 1.0f / 0.45f);
        return x < 0.04045f ? x / 12.92f : std::pow((x + 0.055f) / 1.055f, 2.4f);   // sRGB, :181-191
    };
    float thr[255];
    for (int v = 0; v < 255; v++)
        thr[v] = 0.5f * decode((float)v / 255.0f) + 0.5f * decode((float)(v + 1) / 255.0f);
    cudaStream_t st = sc->active();
    const bool direct = cudaPointerGetAttributes(&oa, out) == cudaSuccess &&
                        (oa.type == cudaMemoryTypeDevice || oa.type == cudaMemoryTypeManaged);
    cudaGetLastError();   // an unregistered host pointer may leave an error behind
    uint8_t* dst = out;
    if (!direct) {
        CK(sc->encode_buf.ensure((size_t)npix * 3));
        dst = sc->encode_buf.as<uint8_t>();
    }
    const int grid = sc->num_sms * 8;
    CK(launch_encode_u8(reinterpret_cast<const float4*>(rgbt), (long long)npix, curve, thr, dst, grid, st));
    if (!direct)
        CK(cudaMemcpyAsync(out, dst, (size_t)npix * 3, cudaMemcpyDeviceToHost, st));
    HW(st);
    return POV_GPU_OK;
}

int pov_gpu_set_profiling(PovGpuScene* sc, int flags)
{
    if (!sc || (flags & ~(POV_GPU_PROFILE_TIMES | POV_GPU_PROFILE_WORK)))
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    sc->profiling = flags;
    if ((flags & POV_GPU_PROFILE_WORK) && sc->wcount.ensure(sizeof(unsigned long long) * 8) != cudaSuccess)
        return POV_GPU_E_NOMEM;
    return POV_GPU_OK;
}

int pov_gpu_get_timings(PovGpuScene* sc, PovGpuTimings* out)
{
    if (!sc || !out)
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    *out = sc->timings;
    return POV_GPU_OK;
}

int pov_gpu_trace_blocks(PovGpuScene* sc, const PovGpuBlock* blocks, int32_t num_blocks,
                         const PovGpuRenderParams* params, float* out_rgbt, PovGpuStats* stats)
{
    if (!sc || !params || num_blocks < 0 || (num_blocks > 0 && (!blocks || !out_rgbt)))
        return POV_GPU_E_INVALID;
    const bool aa = params->antialias != 0;
    if (aa && (params->sampling_method != 2 || params->jitter || params->aa_depth < 1 ||
               params->aa_depth > MAX_AA_DEPTH))
        return POV_GPU_E_UNSUPPORTED;
    if (params->width <= 0 || params->height <= 0)
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    cudaSetDevice(sc->device);
    if (int bc = begin_call(sc))
        return bc;
    if (num_blocks == 0) {
        if (stats)
            std::memset(stats, 0, sizeof(*stats));
        return POV_GPU_OK;
    }
    std::vector<int4> hb((size_t)num_blocks);
    std::vector<int> off((size_t)num_blocks + 1, 0), coff((size_t)num_blocks + 1, 0);
    long long npix = 0, ncorner = 0;
    for (int i = 0; i < num_blocks; i++) {
        const PovGpuBlock& b = blocks[i];
        if (b.left < 0 || b.top < 0 || b.right < b.left || b.bottom < b.top || b.right >= params->width ||
            b.bottom >= params->height)
            return POV_GPU_E_INVALID;
        hb[i] = make_int4(b.left, b.top, b.right, b.bottom);
        off[i] = (int)npix;
        coff[i] = (int)ncorner;
        npix += (long long)(b.right - b.left + 1) * (b.bottom - b.top + 1);
        ncorner += (long long)(b.right - b.left + 2) * (b.bottom - b.top + 2);
    }
    off[num_blocks] = (int)npix;
    coff[num_blocks] = (int)ncorner;
    if (ncorner > (1ll << 27))
        return POV_GPU_E_INVALID;
    const int n = (int)npix;

    cudaPointerAttributes pa{};
    bool out_on_device = cudaPointerGetAttributes(&pa, out_rgbt) == cudaSuccess &&
                         (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    float4* dout = reinterpret_cast<float4*>(out_rgbt);
    if (!out_on_device) {
        CK(sc->out.ensure(sizeof(float4) * n));
        dout = sc->out.as<float4>();
    }
    CK(sc->blocks.ensure(sizeof(int4) * num_blocks));
    CK(sc->block_off.ensure(sizeof(int) * (num_blocks + 1)));
    CK(sc->corner_off.ensure(sizeof(int) * (num_blocks + 1)));

    cudaStream_t st = sc->active();
    int* cnt = sc->counters.as<int>();
    unsigned long long* wc = (sc->profiling & POV_GPU_PROFILE_WORK) ? sc->wcount.as<unsigned long long>() : nullptr;
    StageClock clk(sc, st);
    CK(cudaMemcpyAsync(sc->blocks.p, hb.data(), sizeof(int4) * num_blocks, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(sc->block_off.p, off.data(), sizeof(int) * (num_blocks + 1), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(sc->counters.p, 0, sizeof(int) * C_NUM, st));
    CK(cudaMemsetAsync(sc->stats.p, 0, sizeof(unsigned long long) * ST_COUNT, st));
    CK(cudaMemsetAsync(sc->err.p, 0, sizeof(uint32_t) * 4, st));
    if (wc)
        CK(cudaMemsetAsync(wc, 0, sizeof(unsigned long long) * 8, st));
    if (int rr = rad_begin_call(sc, true))
        return rr;

    uint64_t n_pixels = (uint64_t)n, n_samples = 0;
    // plain frames (no radiosity, media containers or AA: no host reads
    // between the launches) replay a captured graph of their device work
    const bool graphable = !aa && !sc->rad.enabled && sc->media_ni == 0 && !sc->transparent && sc->profiling == 0;
    if (graphable) {
        int rc = trace_plain_graph(sc, clk, num_blocks, n, params->width, params->height, dout);
        if (rc != POV_GPU_OK)
            return rc;
    } else if (!aa) {
        int rc = run_samples(sc, clk, 0, num_blocks, sc->block_off.as<int>(), nullptr, nullptr, n, params->width,
                             params->height, nullptr, dout);
        if (rc != POV_GPU_OK)
            return rc;
    } else {
        // TraceTask::AdaptiveSupersamplingM2 (tracetask.cpp:604-657): the
        // block corners first, then rounds of SubdivideOnePixel
        const int depth = params->aa_depth;
        const int sub = 1 << depth;
        const int G = sub + 1;
        const int MW = (G * G + 31) / 32;
        CK(cudaMemcpyAsync(sc->corner_off.p, coff.data(), sizeof(int) * (num_blocks + 1), cudaMemcpyHostToDevice, st));
        CK(sc->corners.ensure(sizeof(float4) * ncorner));
        CK(sc->aa_grid.ensure(sizeof(float4) * (size_t)n * G * G));
        CK(sc->aa_mask.ensure(sizeof(uint32_t) * (size_t)n * MW));
        CK(sc->aa_subdiv.ensure(sizeof(uint32_t) * (size_t)n));
        CK(sc->aa_xy.ensure(sizeof(int2) * (size_t)n));
        // active cells per round are bounded by 4^round * pixels; both
        // ping-pong lists are sized for the last round up front (growing a
        // list later would drop the cells it holds)
        size_t max_cells = (size_t)n;
        for (int r = 0; r < depth - 1; r++)
            max_cells *= 4;
        CK(sc->cellsA.ensure(sizeof(int4) * std::max(max_cells, (size_t)n)));
        CK(sc->cellsB.ensure(sizeof(int4) * std::max(max_cells, (size_t)n)));
        int rc = run_samples(sc, clk, 1, num_blocks, sc->corner_off.as<int>(), nullptr, nullptr, (int)ncorner,
                             params->width, params->height, nullptr, sc->corners.as<float4>());
        if (rc != POV_GPU_OK)
            return rc;
        CK(launch_aa_init(sc->blocks.as<int4>(), sc->block_off.as<int>(), sc->corner_off.as<int>(), num_blocks, n,
                          sc->corners.as<float4>(), G, MW, sc->aa_grid.as<float4>(), sc->aa_mask.as<uint32_t>(),
                          sc->aa_subdiv.as<uint32_t>(), sc->aa_xy.as<int2>(), sc->cellsA.as<int4>(), cnt + C_NC,
                          depth - 1, st));
        sc->timings.kernel_launches++;
        n_pixels = (uint64_t)ncorner;
        int ncells = n;
        int4* ccur = sc->cellsA.as<int4>();
        for (int round = 0; round < depth - 1 && ncells > 0; round++) {
            const int scap = 5 * ncells, ncap = 4 * ncells;
            CK(sc->spos.ensure(sizeof(double2) * (size_t)scap));
            CK(sc->sslot.ensure(sizeof(int) * (size_t)scap));
            int4* cnext = (ccur == sc->cellsA.as<int4>()) ? sc->cellsB.as<int4>() : sc->cellsA.as<int4>();
            CK(cudaMemsetAsync(cnt + C_NS, 0, sizeof(int), st));
            CK(cudaMemsetAsync(cnt + C_NN, 0, sizeof(int), st));
            int gb = std::max(1, std::min(sc->num_sms * 16, (ncells + 127) / 128));
            CK(launch_aa_classify(ccur, cnt + C_NC, ncells, G, MW, sc->aa_grid.as<float4>(),
                                  sc->aa_mask.as<uint32_t>(), sc->aa_subdiv.as<uint32_t>(), sc->aa_xy.as<int2>(),
                                  (double)params->aa_threshold, (double)sub, sc->spos.as<double2>(),
                                  sc->sslot.as<int>(), cnt + C_NS, scap, cnext, cnt + C_NN, ncap,
                                  sc->err.as<uint32_t>(), gb, st));
            sc->timings.kernel_launches++;
            CK(cudaMemcpyAsync(sc->pin_int(5), cnt + C_NS, sizeof(int), cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(sc->pin_int(6), cnt + C_NN, sizeof(int), cudaMemcpyDeviceToHost, st));
            HW(st);
            const int hc[2] = {*sc->pin_int(5), *sc->pin_int(6)};
            const int nsamp = std::min(hc[0], scap);
            if (nsamp > 0) {
                rc = run_samples(sc, clk, 2, 0, nullptr, sc->spos.as<double2>(), cnt + C_NS, nsamp, params->width,
                                 params->height, sc->sslot.as<int>(), sc->aa_grid.as<float4>());
                if (rc != POV_GPU_OK)
                    return rc;
            }
            n_samples += (uint64_t)nsamp;
            ncells = std::min(hc[1], ncap);
            CK(cudaMemcpyAsync(cnt + C_NC, &ncells, sizeof(int), cudaMemcpyHostToDevice, st));
            ccur = cnext;
        }
        CK(launch_aa_resolve(sc->aa_grid.as<float4>(), sc->aa_subdiv.as<uint32_t>(), n, G, depth, dout, st));
        sc->timings.kernel_launches++;
    }
    if (!out_on_device)
        CK(cudaMemcpyAsync(out_rgbt, dout, sizeof(float4) * n, cudaMemcpyDeviceToHost, st));
    unsigned long long* pwork = reinterpret_cast<unsigned long long*>(sc->pinned + PovGpuScene::PIN_WORK);
    if (wc)
        CK(cudaMemcpyAsync(pwork, wc, sizeof(unsigned long long) * 8, cudaMemcpyDeviceToHost, st));
    unsigned long long hs[ST_COUNT];
    int rc = check_device_error(sc, stats, hs);
    if (rc == POV_GPU_E_TIMEOUT)
        return rc;
    unsigned long long hw[8];
    std::memcpy(hw, pwork, sizeof(hw));
    if (stats) {
        stats->number_of_pixels = n_pixels;
        stats->number_of_samples = n_samples;
        if (int rr = rad_collect(sc, stats))
            return rr;
    }
    clk.collect();
    if (wc) {
        for (int k = 0; k < 2; k++) {
            sc->timings.node_visits[k] = hw[4 * k + 0];
            sc->timings.prim_tests[k] = hw[4 * k + 1];
            sc->timings.tri_tests[k] = hw[4 * k + 2];
            sc->timings.rays_traced[k] = hw[4 * k + 3];
        }
    }
    return rc;
}

int pov_gpu_set_pretrace_jitter(PovGpuScene* sc, const double* table, int32_t n)
{
    if (!sc || n < 0 || (n > 0 && !table))
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    sc->rad.jitter.assign(table, table + n);
    return POV_GPU_OK;
}

int pov_gpu_radiosity_pretrace(PovGpuScene* sc, const PovGpuBlock* blocks, int32_t num_blocks,
                               const PovGpuRenderParams* params, PovGpuStats* stats)
{
    if (!sc || !params || num_blocks < 0 || (num_blocks > 0 && !blocks) || params->width <= 0 ||
        params->height <= 0)
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    if (!sc->rad.enabled)
        return POV_GPU_E_INVALID;
    cudaSetDevice(sc->device);
    if (int bc = begin_call(sc))
        return bc;
    RadiosityState& R = sc->rad;
    const PovGpuRadiosity& rs = R.set;
    // pass sizes (View::StartRender, view.cpp:1060-1080)
    const double maxwh = (double)std::max(params->width, params->height);
    double start = maxwh * rs.pretrace_start, end = maxwh * rs.pretrace_end;
    if (end < 1.0)
        end = 1.0;
    int steps = (int)std::floor(std::log(start / end) / std::log(2.0) + (1.0 - EPSILON)) + 1;
    if (steps > 253) {
        steps = 253;
        start = end * std::pow(2.0, (double)steps);
    }
    // sample positions of every pass (RadiosityTask::Run,
    // radiositytask.cpp:123-207): a grid of the pass's spacing over each
    // block, jittered by the task's table when the caller supplied it
    std::vector<std::vector<double2>> passes((size_t)steps);
    for (int pass = 0; pass < steps; pass++) {
        const double size = std::max(start * (double)std::pow(0.5f, (float)pass), end);
        const double jit = std::min(1.0, size / 2.0), offset = (size - 1.0) / 2.0;
        const unsigned step_id = 1u + (unsigned)pass;   // kOctreePassFirst + pass
        for (int b = 0; b < num_blocks; b++) {
            const PovGpuBlock& B = blocks[b];
            if (B.left < 0 || B.top < 0 || B.right < B.left || B.bottom < B.top || B.right >= params->width ||
                B.bottom >= params->height)
                return POV_GPU_E_INVALID;
            const double sx = std::ceil((B.left - 0.5) / size) * size, sy = std::ceil((B.top - 0.5) / size) * size;
            const double ex = B.left + (double)(B.right - B.left + 1), ey = B.top + (double)(B.bottom - B.top + 1);
            size_t ji = R.jitter.empty() ? 0 : (size_t)(step_id * 17u + B.serial * 13u) % R.jitter.size();
            uint32_t hseed = step_id * 0x9E3779B1u ^ B.serial * 0x85EBCA77u;
            for (double y = sy; y < ey; y += size) {
                if (y < B.top)
                    continue;
                for (double x = sx; x < ex; x += size) {
                    if (x < B.left)
                        continue;
                    double jx, jy;
                    if (!R.jitter.empty()) {
                        // the reference build evaluates the y argument's
                        // jitter first (radiositytask.cpp:197)
                        ji = (ji + 1) % R.jitter.size();
                        jy = R.jitter[ji];
                        ji = (ji + 1) % R.jitter.size();
                        jx = R.jitter[ji];
                    } else {
                        hseed = hseed * 1664525u + 1013904223u;
                        jy = (double)(hseed >> 8) / 8388608.0 - 1.0;
                        hseed = hseed * 1664525u + 1013904223u;
                        jx = (double)(hseed >> 8) / 8388608.0 - 1.0;
                    }
                    passes[pass].push_back(make_double2(x + offset + jit * jx, y + offset + jit * jy));
                }
            }
        }
    }
    cudaStream_t st = sc->active();
    StageClock clk(sc, st);
    CK(cudaMemsetAsync(sc->stats.p, 0, sizeof(unsigned long long) * ST_COUNT, st));
    CK(cudaMemsetAsync(sc->err.p, 0, sizeof(uint32_t) * 4, st));
    if (int rr = rad_reset(sc))
        return rr;
    if (int rr = rad_begin_call(sc, false))
        return rr;
    uint64_t npix = 0;
    for (int pass = 0; pass < steps; pass++) {
        const std::vector<double2>& pos = passes[pass];
        const int n = (int)pos.size();
        if (n == 0)
            continue;
        npix += (uint64_t)n;
        CK(sc->spos.ensure(sizeof(double2) * (size_t)n));
        CK(sc->pos_count.ensure(sizeof(int)));
        CK(sc->out.ensure(sizeof(float4) * (size_t)n));
        CK(cudaMemcpyAsync(sc->spos.p, pos.data(), sizeof(double2) * (size_t)n, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(sc->pos_count.p, &n, sizeof(int), cudaMemcpyHostToDevice, st));
        int rc = run_samples(sc, clk, 2, 0, nullptr, sc->spos.as<double2>(), sc->pos_count.as<int>(), n,
                             params->width, params->height, nullptr, sc->out.as<float4>());
        HW(st);   // `n` and `pos` must outlive the copies
        if (rc != POV_GPU_OK)
            return rc;
    }
    clk.collect();
    PovGpuTimings keep = sc->timings;
    R.nic_ok = false;
    if (R.nic_cfg.enabled) {
        if (int rr = nic_train(sc))
            return rr;
        for (int k = 0; k < POV_GPU_STAGES; k++) {   // this call's stages plus the training's
            keep.stage_ms[k] += sc->timings.stage_ms[k];
            keep.stage_launches[k] += sc->timings.stage_launches[k];
        }
        keep.kernel_launches += sc->timings.kernel_launches;
    }
    unsigned long long hs[ST_COUNT];
    int rc = check_device_error(sc, stats, hs);
    if (rc == POV_GPU_E_TIMEOUT)
        return rc;
    if (stats) {
        stats->number_of_pixels = npix;
        if (int rr = rad_collect(sc, stats))
            return rr;
    }
    sc->timings = keep;
    return rc;
}

static_assert(POV_GPU_NIC_PARAMS == nic::NPARAM, "public and internal parameter counts differ");

int pov_gpu_set_neural_cache(PovGpuScene* sc, const PovGpuNeuralCache* cfg)
{
    if (!sc || !cfg || (cfg->enabled && (cfg->steps < 1 || cfg->batch < 0 || cfg->learning_rate <= 0.0f)))
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    if (!sc->rad.enabled)
        return POV_GPU_E_INVALID;
    sc->rad.nic_cfg = *cfg;
    sc->rad.nic_ok = false;
    sc->rad.nic_init = false;   // a new configuration starts a new network
    return POV_GPU_OK;
}

int pov_gpu_nic_eval(const float* params, const float* bounds, const float* points, const float* normals,
                     const float* targets, int32_t n, float* out, float* grad, float* loss)
{
    if (!params || !bounds || n < 0 || (n > 0 && (!points || !normals)) || (targets && (!grad || !loss)))
        return POV_GPU_E_INVALID;
    if (n == 0)
        return POV_GPU_OK;
    const size_t NP = (size_t)nic::NPARAM;
    DevBuf dp, dwb, dpos, dnrm, dtg, dout, dgrad, dloss, derr;
    struct Free {
        DevBuf* b[9];
        ~Free() { for (DevBuf* x : b) x->release(); }
    } fr{{&dp, &dwb, &dpos, &dnrm, &dtg, &dout, &dgrad, &dloss, &derr}};
    CK(dp.ensure(sizeof(float) * NP));
    CK(dwb.ensure(nic::WIMG_BYTES));
    CK(dpos.ensure(sizeof(float4) * (size_t)n));
    CK(dnrm.ensure(sizeof(float4) * (size_t)n));
    CK(dout.ensure(sizeof(float4) * (size_t)n));
    CK(derr.ensure(sizeof(uint32_t)));
    std::vector<float4> hp((size_t)n), hn((size_t)n), ht((size_t)n);
    for (int i = 0; i < n; i++) {
        hp[i] = make_float4(points[3 * i], points[3 * i + 1], points[3 * i + 2], 0.f);
        hn[i] = make_float4(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2], 0.f);
        if (targets)
            ht[i] = make_float4(targets[3 * i], targets[3 * i + 1], targets[3 * i + 2], 0.f);
    }
    CK(cudaMemcpy(dp.p, params, sizeof(float) * NP, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dpos.p, hp.data(), sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dnrm.p, hn.data(), sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice));
    CK(cudaMemset(derr.p, 0, sizeof(uint32_t)));
    CK(nic::launch_to_bf16(dp.as<float>(), dwb.as<unsigned char>(), 0));
    nic::NicIO io{};
    io.pos = dpos.as<float4>();
    io.nrm = dnrm.as<float4>();
    io.stride = 1;
    io.n = n;
    io.out = dout.as<float4>();
    for (int k = 0; k < 3; k++) {
        float ext = std::max(bounds[3 + k] - bounds[k], 1e-6f);
        (&io.lo.x)[k] = bounds[k];
        (&io.scale.x)[k] = 2.0f / ext;
    }
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (out) {
        CK(nic::launch_forward(io, dwb.as<unsigned char>(), dp.as<float>(), derr.as<uint32_t>(), sms * 2, 0));
        std::vector<float4> ho((size_t)n);
        CK(cudaMemcpy(ho.data(), dout.p, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; i++) {
            out[3 * i] = ho[i].x;
            out[3 * i + 1] = ho[i].y;
            out[3 * i + 2] = ho[i].z;
        }
    }
    if (targets) {
        const int slices = nic::train_slices(n, sms);
        CK(dtg.ensure(sizeof(float4) * (size_t)n));
        CK(dgrad.ensure(sizeof(float) * NP * (size_t)(slices + 1)));
        CK(dloss.ensure(sizeof(float) * (size_t)(slices + 1)));
        CK(cudaMemcpy(dtg.p, ht.data(), sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice));
        io.target = dtg.as<float4>();
        float* gsum = dgrad.as<float>() + NP * (size_t)slices;   // the summed gradient after the slices
        float* lsum = dloss.as<float>() + slices;
        CK(nic::launch_train(io, dwb.as<unsigned char>(), dp.as<float>(), dgrad.as<float>(), dloss.as<float>(),
                             1.0f / (float)n, derr.as<uint32_t>(), sms, 0));
        CK(nic::launch_reduce(dgrad.as<float>(), dloss.as<float>(), slices, gsum, lsum, 0));
        CK(cudaMemcpy(grad, gsum, sizeof(float) * NP, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(loss, lsum, sizeof(float), cudaMemcpyDeviceToHost));
    }
    uint32_t e = 0;
    CK(cudaMemcpy(&e, derr.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return e ? POV_GPU_E_DEVICE : POV_GPU_OK;
}

int pov_gpu_trace_rays(PovGpuScene* sc, const double* origins, const double* directions, int32_t num_rays,
                       PovGpuHit* hits)
{
    if (!sc || num_rays < 0 || (num_rays > 0 && (!origins || !directions || !hits)))
        return POV_GPU_E_INVALID;
    std::lock_guard<std::mutex> g(sc->lock);
    cudaSetDevice(sc->device);
    if (int bc = begin_call(sc))
        return bc;
    if (num_rays == 0)
        return POV_GPU_OK;
    cudaStream_t st = sc->active();
    const size_t n = (size_t)num_rays;
    CK(sc->rays_in.ensure(sizeof(double) * 6 * n));
    CK(sc->qA.ensure(sizeof(QRay) * n));
    CK(sc->hits.ensure(sizeof(QHit) * n));
    CK(sc->t64.ensure(sizeof(double) * n));
    double* dorg = sc->rays_in.as<double>();
    double* ddir = dorg + 3 * n;
    CK(cudaMemcpyAsync(dorg, origins, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ddir, directions, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    int* cnt = sc->counters.as<int>();
    CK(cudaMemsetAsync(sc->counters.p, 0, sizeof(int) * C_NUM, st));
    CK(cudaMemsetAsync(sc->err.p, 0, sizeof(uint32_t) * 4, st));
    CK(cudaMemsetAsync(sc->stats.p, 0, sizeof(unsigned long long) * ST_COUNT, st));
    CK(launch_load_rays(dorg, ddir, num_rays, sc->qA.as<QRay>(), cnt + C_QA, st));
    CK(launch_trace(sc->S, false, sc->qA.as<QRay>(), cnt + C_QA, cnt + C_W0, sc->hits.as<QHit>(), nullptr,
                    sc->stack_depth, sc->num_sms * 8, sc->err.as<uint32_t>(), sc->stats.as<unsigned long long>(),
                    nullptr, num_rays, nullptr, st));
    CK(launch_refine(sc->S, dorg, ddir, sc->hits.as<QHit>(), sc->t64.as<double>(), num_rays, st));
    std::vector<QHit> hh(n);
    std::vector<double> t64(n);
    CK(cudaMemcpyAsync(hh.data(), sc->hits.p, sizeof(QHit) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(t64.data(), sc->t64.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    unsigned long long hs[ST_COUNT];
    int rc = check_device_error(sc, nullptr, hs);
    if (rc == POV_GPU_E_TIMEOUT)
        return rc;
    // map prim references to flattened object ids / mesh triangle indices
    for (size_t i = 0; i < n; i++) {
        const QHit& h = hh[i];
        hits[i].object = -1;
        hits[i].triangle = -1;
        hits[i].t = 0.0;
        if (h.prim == 0xffffffffu)
            continue;
        uint32_t kind = h.prim >> PRIM_KIND_SHIFT, idx = h.prim & PRIM_INDEX_MASK;
        hits[i].t = t64[i];
        if (kind == PK_SPHERE) {
            hits[i].object = sc->h_sphere_obj[idx];
        } else if (kind == PK_PLANE) {
            hits[i].object = sc->h_plane_obj[idx];
        } else if (kind == PK_BOX) {
            hits[i].object = sc->h_box_obj[idx];
        } else if (kind == PK_TORUS) {
            hits[i].object = sc->h_torus_obj[idx];
        } else if (kind == PK_CSG) {
            uint32_t aux = __builtin_bit_cast(uint32_t, h.u);
            const DevCsg& cg = sc->h_csgs[idx];
            hits[i].object = sc->h_csg_children[cg.first + (aux & 0xffffu)].object;
        } else if (kind == PK_TRIANGLE) {
            int gidx = sc->h_tri_global[idx];
            hits[i].object = sc->h_tri_obj[gidx];
            hits[i].triangle = sc->h_tri_local[gidx];
        }
    }
    return rc;
}


// The same query as pov_gpu_trace_rays with every buffer in the library's
// fixed device scratch (static_ray_scratch) instead of the scene's growable
// buffers, and the hit mapping done by a kernel instead of host vectors:
// nothing is allocated.  Its callers are integrations whose device memory
// belongs to another allocator (cudaMalloc would fail although memory is
// cached there) and render threads that must not stall frames in flight on
// the device-wide synchronisation of cudaFree.
int pov_gpu_trace_rays_static(PovGpuScene* sc, const double* origins, const double* directions, int32_t num_rays,
                              PovGpuHit* hits)
{
    static_assert(sizeof(PovGpuHit) == 16, "scratch sizes PovGpuHit as 16 bytes");
    static_assert(POV_GPU_STATIC_MAX_RAYS == STATIC_MAX_RAYS, "public and internal capacity differ");
    static_assert(sizeof(int) * C_NUM <= STATIC_OFF_ERR && STATIC_OFF_ERR + 16 <= STATIC_OFF_STATS &&
                      STATIC_OFF_STATS + sizeof(unsigned long long) * ST_COUNT <= STATIC_HEADER_BYTES,
                  "scratch header regions overlap");
    if (!sc || num_rays < 0 || (num_rays > 0 && (!origins || !directions || !hits)))
        return POV_GPU_E_INVALID;
    if (num_rays > POV_GPU_STATIC_MAX_RAYS)
        return POV_GPU_E_CAPACITY;
    std::lock_guard<std::mutex> g(sc->lock);
    CK(cudaSetDevice(sc->device));
    if (int bc = begin_call(sc))
        return bc;
    unsigned char* base = nullptr;
    CK(static_ray_scratch(sc->device, &base));   // one-time set-up per device
    if (num_rays == 0)
        return POV_GPU_OK;
    cudaStream_t st = sc->active();
    const size_t n = (size_t)num_rays;
    int* cnt = reinterpret_cast<int*>(base + STATIC_OFF_COUNTERS);
    uint32_t* err = reinterpret_cast<uint32_t*>(base + STATIC_OFF_ERR);
    unsigned long long* stats = reinterpret_cast<unsigned long long*>(base + STATIC_OFF_STATS);
    double* dorg = reinterpret_cast<double*>(base + STATIC_OFF_ORG);
    double* ddir = reinterpret_cast<double*>(base + STATIC_OFF_DIR);
    QRay* rays = reinterpret_cast<QRay*>(base + STATIC_OFF_RAYS);
    QHit* qh = reinterpret_cast<QHit*>(base + STATIC_OFF_HITS);
    double* t64 = reinterpret_cast<double*>(base + STATIC_OFF_T64);
    PovGpuHit* out = reinterpret_cast<PovGpuHit*>(base + STATIC_OFF_OUT);
    // counters, error word and statistics start at zero
    CK(cudaMemsetAsync(base, 0, STATIC_HEADER_BYTES, st));
    CK(cudaMemcpyAsync(dorg, origins, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ddir, directions, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    CK(launch_load_rays(dorg, ddir, num_rays, rays, cnt + C_QA, st));
    CK(launch_trace(sc->S, false, rays, cnt + C_QA, cnt + C_W0, qh, nullptr, sc->stack_depth, sc->num_sms * 8, err,
                    stats, nullptr, num_rays, nullptr, st));
    CK(launch_refine(sc->S, dorg, ddir, qh, t64, num_rays, st));
    CK(launch_hits_abi(sc->S, qh, t64, num_rays, out, st));
    uint32_t errw = 0;
    CK(cudaMemcpyAsync(hits, out, sizeof(PovGpuHit) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&errw, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    HW(st);
    return errw ? POV_GPU_E_DEVICE : POV_GPU_OK;
}

}  // extern "C"
