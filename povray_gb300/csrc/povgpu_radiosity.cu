// povgpu_radiosity.cu -- radiosity on the GPU: the sample cache query
// (RadiosityCache::FindReusableBlock / AverageNearBlock), the gather of new
// samples (RadiosityFunction::GatherLight) and their insertion
// (RadiosityCache::AddBlock), source/core/lighting/radiosity.cpp.
//
// The reference answers queries one at a time, each one either reusing the
// cache or gathering a new sample that later queries see.  Here a batch of
// queries runs in rounds: every round queries the cache for all open
// queries; those the cache satisfies resolve, and of the rest one per
// spatial cell (cells shrinking round by round from the largest reuse
// radius to the smallest) gathers a new sample; the others wait for the
// next round and see the new samples.  The last round gathers for all that
// remain.
//
// The cache keeps the reference's octree addressing: a sample is filed at
// the node ot_index_sphere picks (source/core/support/octree.cpp:1035-1190)
// and a query sees exactly the samples of nodes whose half-size-extended
// box holds the query point (what ot_dist_traverse visits, octree.cpp:
// 800-855).  Nodes live in an open-addressing hash keyed by a 64-bit mix of
// (size, x, y, z); each node holds a lock-free list of its blocks.
#include "povgpu_internal.h"
#include "povgpu_kernels.h"
#include "povgpu_radiosity.h"

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

namespace povgpu {

namespace {

constexpr double OT_BIAS = 10000000.;            // octree.h:81
constexpr float RAD_EPSILON = 0.001f;            // radiosity.cpp:110
constexpr float AVG_NEAR_EPSILON = 0.000001f;    // radiosity.cpp:109
constexpr float IN_FRONT_LIMIT = -0.05f;         // radiosity.cpp:100
constexpr float WEIGHT_ERROR_BOUND_OFFSET = 0.25f;   // radiosity.cpp:111
constexpr int MAX_PROBES = 1 << 20;

__constant__ float3 c_dirs[RAD_DIRECTIONS];      // Halton(2,3) cosine-weighted directions

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 mul(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 normalized(float3 v) { return mul(v, rsqrtf(dot(v, v))); }

__device__ __forceinline__ float to_eye(const DeviceScene& S, float3 p)
{
    double dx = S.cam_loc[0] - p.x, dy = S.cam_loc[1] - p.y, dz = S.cam_loc[2] - p.z;
    return (float)sqrt(dx * dx + dy * dy + dz * dz);
}

// The same distance in FP32, for the rounds' claim cells (a GPU schedule,
// not a reference decision).
__device__ __forceinline__ float to_eye_f(const DeviceScene& S, float3 p)
{
    float dx = (float)S.cam_loc[0] - p.x, dy = (float)S.cam_loc[1] - p.y, dz = (float)S.cam_loc[2] - p.z;
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

// Pow2Floor / BiasedIntLog2 / BiasedIntPow2 (octree.cpp:169-250).
__device__ __forceinline__ float pow2_floor(float a) { return __uint_as_float(__float_as_uint(a) & 0xFF800000u); }
__device__ __forceinline__ int biased_log2(float a) { return (int)((__float_as_uint(a) & 0x7F800000u) >> 23); }
__device__ __forceinline__ double biased_pow2(int e) { return (double)__uint_as_float(((uint32_t)e & 0xFFu) << 23); }

// ot_point_in_node (octree.cpp:985-997).
__device__ __forceinline__ bool in_node(double px, double py, double pz, int size, int x, int y, int z)
{
    double s = biased_pow2(size);
    return fabs(px + OT_BIAS - ((double)x + 0.5) * s) < s && fabs(py + OT_BIAS - ((double)y + 0.5) * s) < s &&
           fabs(pz + OT_BIAS - ((double)z + 0.5) * s) < s;
}

__device__ __forceinline__ unsigned long long node_key(int size, int x, int y, int z)
{
    unsigned long long h = (unsigned long long)(uint32_t)size * 0x9E3779B97F4A7C15ull;
    h ^= (unsigned long long)(uint32_t)x * 0xC2B2AE3D27D4EB4Full;
    h = (h ^ (h >> 29)) * 0xBF58476D1CE4E5B9ull;
    h ^= (unsigned long long)(uint32_t)y * 0x94D049BB133111EBull;
    h = (h ^ (h >> 32)) * 0x9E3779B97F4A7C15ull;
    h ^= (unsigned long long)(uint32_t)z * 0xD6E8FEB86659FD93ull;
    h ^= h >> 31;
    return h ? h : 1ull;
}

// Slot of the node, -1 when the node holds nothing.
__device__ __forceinline__ int node_lookup(const RadCacheView& C, unsigned long long key)
{
    uint32_t slot = (uint32_t)key & C.mask;
    for (int n = 0; n < MAX_PROBES; n++) {
        unsigned long long k = C.keys[slot];
        if (k == key)
            return (int)slot;
        if (k == 0ull)
            return -1;
        slot = (slot + 1) & C.mask;
    }
    return -1;
}

// Slot of the node, created when absent; -1 when the table is full.
__device__ __forceinline__ int node_insert(const RadCacheView& C, unsigned long long key)
{
    uint32_t slot = (uint32_t)key & C.mask;
    for (int n = 0; n < MAX_PROBES && n <= (int)C.mask; n++) {
        unsigned long long k = atomicCAS(&C.keys[slot], 0ull, key);
        if (k == 0ull || k == key)
            return (int)slot;
        slot = (slot + 1) & C.mask;
    }
    return -1;
}

// ot_index_sphere / ot_index_box with SAFE_METHOD and ot_parent
// (octree.cpp:1035-1238): the node a sample of this address radius is
// filed at.
__device__ void ot_index_sphere(float3 c, double radius, int& size, int& x, int& y, int& z)
{
    double lo[3] = {c.x - radius, c.y - radius, c.z - radius};
    double hi[3] = {c.x + radius, c.y + radius, c.z + radius};
    double desired = fmax(fmax(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    double bsized = pow2_floor((float)desired);
    if (bsized == 0.0)
        bsized = 1.0;
    double maxord = fmax(fmax(fabs(lo[0]), fabs(lo[1])), fabs(lo[2])) + OT_BIAS;
    for (int k = 0; k < 64 && maxord / bsized > 1000000000.0; k++)
        bsized *= 2.0;
    x = (int)floor(((lo[0] + hi[0]) / 2 + OT_BIAS) / bsized);
    y = (int)floor(((lo[1] + hi[1]) / 2 + OT_BIAS) / bsized);
    z = (int)floor(((lo[2] + hi[2]) / 2 + OT_BIAS) / bsized);
    size = biased_log2((float)bsized);
    for (int k = 0; k < 64 && !(in_node(lo[0], lo[1], lo[2], size, x, y, z) && in_node(hi[0], hi[1], hi[2], size, x, y, z));
         k++) {
        size += 1;
        x = x >= 0 ? x >> 1 : (x + 1) / 2;
        y = y >= 0 ? y >> 1 : (y + 1) / 2;
        z = z >= 0 ? z >> 1 : (z + 1) / 2;
    }
}

// RadiosityCache::AverageNearBlock (radiosity.cpp:1551-1770): pseudo-sigmoid
// weight for final-trace depth-0 queries, linear otherwise; no gradient.
// The weight of one block is formed in FP32; the sums of weights and of
// weighted illuminances accumulate in FP64, as the reference's WT_AVG sums
// them in DBL (radiosity.cpp:122, 1755-1757).
__device__ __forceinline__ void average_near(const RadBlock& b, float3 P, float3 N, float eb, bool final_trace,
                                             double& W, double3& WI)
{
    float3 bp = xyz(b.p);
    float3 delta = sub(P, bp);
    float sq = dot(delta, delta);
    float quick = b.p.w * eb;
    if (!(sq < quick * quick))
        return;
    float dist = sqrtf(sq);
    float ri = b.p.w;
    bool far = dist > AVG_NEAR_EPSILON;
    float3 du = f3(0.f, 0.f, 0.f);
    if (far) {
        du = mul(delta, 1.0f / dist);
        float c = dot(xyz(b.tn), du);
        if (c > 0.0f)
            ri = c * b.n.w + (1.0f - c) * ri;
    }
    if (!(dist < ri * eb))
        return;
    float3 bn = xyz(b.n);
    float e = dist / ri + 2.0f * sqrtf(fabsf(1.0f - dot(N, bn)));
    if (!(e < eb))
        return;
    float in_front = 1.0f;
    if (far) {
        float3 half = add(N, bn);
        in_front = dot(du, half) * rsqrtf(dot(half, half));
    }
    if (!(in_front > IN_FRONT_LIMIT))
        return;
    int bdepth = __float_as_int(b.ill.w);
    float w;
    if (!final_trace || bdepth > 0) {
        w = 1.0f - e / eb;
    } else {
        w = e / eb;
        w = w < 0.5f ? 1.0f - (w * 2.0f) * (w * 2.0f) / 2.0f : ((1.0f - w) * 2.0f) * ((1.0f - w) * 2.0f) / 2.0f;
    }
    if (in_front <= 0.0f)
        w *= 1.0f - in_front / IN_FRONT_LIMIT;
    if (w > RAD_EPSILON) {
        const double wq = (double)w * (double)b.tn.w;
        WI.x = fma((double)b.ill.x, wq, WI.x);
        WI.y = fma((double)b.ill.y, wq, WI.y);
        WI.z = fma((double)b.ill.z, wq, WI.z);
        W += wq;
    }
}

// RadiosityCache::FindReusableBlock (radiosity.cpp:1458-1512).
__device__ __forceinline__ uint32_t occ_bit(const RadCacheView& C, unsigned long long key)
{
    return (uint32_t)(key >> 29) & C.occ_mask;
}

// RadiosityCache::FindReusableBlock (radiosity.cpp:1458-1512), one warp per
// query.  Nodes are keyed per bounce depth (ot_dist_traverse passes only
// blocks of the query's depth to AverageNearBlock, octree.cpp:843), so lists
// hold one depth; the occupancy bits skip the probe of nodes that hold
// nothing.  The candidate nodes -- per node size in use, the cells of the
// 2x2x2 neighbourhood whose half-size-extended interval holds the point
// (ot_point_in_node) -- are dealt to the lanes, each lane walks its nodes'
// block lists, and the warp sums the weights (every lane gets the sums).
__device__ void find_reusable_warp(const RadCacheView& C, int smin, int smax, float3 P, float3 N, float eb,
                                   int depth, bool final_trace, int lane, double& W, double3& WI)
{
    W = 0.0;
    WI = make_double3(0.0, 0.0, 0.0);
    const float pf[3] = {P.x, P.y, P.z};
    const int ncand = (smax - smin + 1) * 8;
    for (int cand = lane; cand < ncand; cand += 32) {
        const int size = smin + (cand >> 3), k = cand & 7;
        const int d3[3] = {k & 1, (k >> 1) & 1, k >> 2};
        int cell[3];
        bool in = true;
        const int e = size - 127;   // node edge 2^e
        if (e >= -7 && e <= 7) {
            // OT_BIAS = 10^7 = 2^7 * 78125 is a whole number of such nodes,
            // so the node grid is the unbiased one shifted by 10^7 / 2^e
            // nodes: the same cells and the same inside test in FP32
            const float sf = __int_as_float((e + 127) << 23), invf = __int_as_float((127 - e) << 23);
            const int shift = e >= 0 ? (10000000 >> e) : (10000000 << -e);
            for (int a = 0; a < 3; a++) {
                const float bu = floorf(pf[a] * invf - 1.5f);
                cell[a] = (int)bu + shift + 1 + d3[a];
                in = in && fabsf(pf[a] - (bu + 1.5f + (float)d3[a]) * sf) < sf;
            }
        } else {
            const double s = biased_pow2(size), inv = 1.0 / s;   // powers of two: exact
            const double c[3] = {(double)P.x + OT_BIAS, (double)P.y + OT_BIAS, (double)P.z + OT_BIAS};
            for (int a = 0; a < 3; a++) {
                const int b = (int)floor(c[a] * inv - 1.5);
                cell[a] = b + 1 + d3[a];
                in = in && fabs(c[a] - ((double)b + 1.5 + d3[a]) * s) < s;
            }
        }
        if (!in)
            continue;
        const unsigned long long key = node_key(size + 256 * depth, cell[0], cell[1], cell[2]);
        const uint32_t bit = occ_bit(C, key);
        if (!((C.occupancy[bit >> 5] >> (bit & 31)) & 1u))
            continue;
        const int slot = node_lookup(C, key);
        if (slot < 0)
            continue;
        const int off = C.seg_off[slot], cnt = min(C.seg_cnt[slot], C.cap);
        for (int j = 0; j < cnt; j++) {
            // the quick test (AverageNearBlock's first check) on the 16-byte
            // record; the whole block only for the blocks that pass it
            const int bi = C.members[off + j];
            const float4 qk = C.quick[bi];
            const float3 dl = sub(P, xyz(qk));
            const float qr = qk.w * eb;
            if (dot(dl, dl) < qr * qr) {
                RadBlock blk = C.blocks[bi];
                if (__float_as_int(blk.ill.w) == depth)
                    average_near(blk, P, N, eb, final_trace, W, WI);
            }
        }
    }
    // FP64 warp sum of the four values as a reduce-scatter: across lane
    // halves each lane keeps two of the values, across quarters one, then
    // eight lanes sum that one -- 6 FP64 adds per lane instead of the 20 of
    // a butterfly on all four (FP64 is a narrow pipe on this part).  The
    // order of the adds is fixed, so the sums are reproducible.
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    const double s0 = h16 ? W : WI.y, s1 = h16 ? WI.x : WI.z;
    const double a0 = (h16 ? WI.y : W) + __shfl_xor_sync(0xffffffffu, s0, 16);
    const double a1 = (h16 ? WI.z : WI.x) + __shfl_xor_sync(0xffffffffu, s1, 16);
    double b = (h8 ? a1 : a0) + __shfl_xor_sync(0xffffffffu, h8 ? a0 : a1, 8);
    b += __shfl_xor_sync(0xffffffffu, b, 4);
    b += __shfl_xor_sync(0xffffffffu, b, 2);
    b += __shfl_xor_sync(0xffffffffu, b, 1);
    // lanes 0-7 hold W, 8-15 WI.x, 16-23 WI.y, 24-31 WI.z
    W = __shfl_sync(0xffffffffu, b, 0);
    WI.x = __shfl_sync(0xffffffffu, b, 8);
    WI.y = __shfl_sync(0xffffffffu, b, 16);
    WI.z = __shfl_sync(0xffffffffu, b, 24);
}

__device__ __forceinline__ float4 finish_ambient(float3 a, float quality, const RadParams& R)
{
    // ComputeAmbient's grey threshold and brightness (radiosity.cpp:457-461)
    float grey = 0.297f * a.x + 0.589f * a.y + 0.114f * a.z;
    a = f3((a.x * (1.0f - R.gray) + R.gray * grey) * R.brightness, (a.y * (1.0f - R.gray) + R.gray * grey) * R.brightness,
           (a.z * (1.0f - R.gray) + R.gray * grey) * R.brightness);
    return make_float4(a.x, a.y, a.z, quality);
}

// Node segments rebuilt from every block's slot (a counting sort by node):
// reset the touched slots, count, give each node its segment, file the blocks.
__global__ void k_seg_reset(RadCacheView C)
{
    const int n = min(*C.count, C.cap);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        const int s = C.bslot[b];
        if (s < 0)
            continue;
        C.seg_cnt[s] = 0;
        C.seg_cur[s] = 0;
    }
}
__global__ void k_seg_count(RadCacheView C)
{
    const int n = min(*C.count, C.cap);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x)
        if (C.bslot[b] >= 0)
            atomicAdd(&C.seg_cnt[C.bslot[b]], 1);
}
__global__ void k_seg_alloc(RadCacheView C)
{
    const int n = min(*C.count, C.cap);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        const int s = C.bslot[b];
        if (s >= 0 && atomicCAS(&C.seg_cur[s], 0, -1) == 0)   // the node's first block allocates
            C.seg_off[s] = atomicAdd(C.seg_total, C.seg_cnt[s]);
    }
}
__global__ void k_seg_fill(RadCacheView C)
{
    const int n = min(*C.count, C.cap);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        const int s = C.bslot[b];
        if (s < 0)
            continue;
        // after the allocation seg_cur holds -1 and counts down: -1 - old is
        // the block's place in its node's segment
        const int old = atomicSub(&C.seg_cur[s], 1);
        C.members[C.seg_off[s] + (-1 - old)] = b;
    }
}

// One thread per open query: the cache lookup of ComputeAmbient
// (radiosity.cpp:385-413).  Reusable -> the ambient colour and quality go to
// out[q]; else the query's partial sums are kept and it either claims its
// cell for this round (a seed: gathers now) or waits for the next round.
__global__ void k_rad_query(DeviceScene S, RadCacheView C, RadParams R, const RadQuery* __restrict__ queries,
                            const int* __restrict__ open, int n_open, int cap, int round,
                            int last_round, float4* __restrict__ out, float4* __restrict__ partial,
                            unsigned long long* __restrict__ claims, uint32_t claim_mask, int* __restrict__ seeds,
                            int* __restrict__ n_seeds, int* __restrict__ next, int* __restrict__ n_next,
                            unsigned long long* __restrict__ rstats, uint32_t* err)
{
    const int n = min(n_open, cap);
    const int smin = C.size_range[2 * R.depth], smax = C.size_range[2 * R.depth + 1];
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long reused = 0;   // this warp's reused queries (lane 0), one atomic at the end
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {   // one warp per query
        int qi = open ? open[i] : i;
        RadQuery q = queries[qi];
        float3 P = xyz(q.p), N = xyz(q.n);
        float eb = R.error_bound;
        if (q.p.w < WEIGHT_ERROR_BOUND_OFFSET)
            eb += WEIGHT_ERROR_BOUND_OFFSET - q.p.w;
        eb *= R.error_bound_factor;
        double W = 0.0;
        double3 WI = make_double3(0.0, 0.0, 0.0);
        if (smax >= smin)
            find_reusable_warp(C, smin, smax, P, N, eb, R.depth, R.final_trace != 0, lane, W, WI);
        if (lane != 0)
            continue;
        bool reuse = W * 4.0 >= (double)R.reuse_count || (R.final_trace && !R.always_sample && W > 0.0);
        if (reuse) {
            // the weighted mean formed from the FP64 sums, then kept in
            // single precision like the reference's ambient colour
            const double inv = 1.0 / W;
            float3 a = f3((float)(WI.x * inv), (float)(WI.y * inv), (float)(WI.z * inv));
            out[qi] = finish_ambient(a, (float)fmin(4.0 * W / (double)R.reuse_count, 1.0), R);
            reused++;
            continue;
        }
        partial[qi] = make_float4((float)WI.x, (float)WI.y, (float)WI.z, (float)W);
        bool seed = round >= last_round;
        if (!seed) {
            // cell of this round: the largest reuse radius halved per round,
            // not below the smallest (GatherLight's reuse distance clamps)
            float te = to_eye_f(S, P);
            float h = fmaxf(te * R.max_reuse_factor * eb * exp2f(-(float)round), te * R.min_reuse_factor * eb);
            int lvl = (int)ceilf(log2f(fmaxf(h, 1e-6f)));
            float cs = exp2f((float)lvl);
            int cx = (int)floorf(P.x / cs), cy = (int)floorf(P.y / cs), cz = (int)floorf(P.z / cs);
            unsigned long long key = node_key(lvl + 1024 * round, cx, cy, cz);
            uint32_t slot = (uint32_t)key & claim_mask;
            for (int k = 0; k <= (int)claim_mask; k++) {
                unsigned long long old = atomicCAS(&claims[slot], 0ull, key);
                if (old == 0ull) { seed = true; break; }
                if (old == key) break;
                slot = (slot + 1) & claim_mask;
            }
        }
        if (seed) {
            int s = atomicAdd(n_seeds, 1);
            if (s < cap) seeds[s] = qi; else atomicOr(err, DE_QUEUE_OVERFLOW);
        } else {
            int s = atomicAdd(n_next, 1);
            if (s < cap) next[s] = qi; else atomicOr(err, DE_QUEUE_OVERFLOW);
        }
    }
    if (reused)
        atomicAdd(&rstats[RST_REUSED], reused);
}

// Direction k of seed s: entry (base + s*count + k) of the direction pool,
// turned into the frame of the seed's normal (SampleDirectionGenerator::
// InitSequence / GetDirection, radiosity.cpp:815-888).
__device__ __forceinline__ float3 sample_direction(float3 fy, int base, int s, int count, int k)
{
    float3 off = fabsf(fy.z) > 0.9f ? f3(0.f, 1.f, 0.f) : f3(0.f, 0.f, 1.f);
    float3 fx = normalized(cross(fy, off));
    float3 fz = normalized(cross(fx, fy));
    float3 rv = c_dirs[(int)(((long long)base + (long long)s * count + k) % RAD_DIRECTIONS)];
    rv.y = fabsf(rv.y);
    if (fy.y > 1.0f - RAD_EPSILON)
        return rv;
    if (fy.y < -1.0f + RAD_EPSILON)
        return mul(rv, -1.0f);
    return add(add(mul(fx, rv.x), mul(fy, rv.y)), mul(fz, rv.z));
}

// One thread per sample ray of the seeds: the first queue of the sample
// rays' wavefront (path i = ray i, quality 1, weight of the depth).
__global__ void k_gather_rays(const RadQuery* __restrict__ queries, const int* __restrict__ seeds, int ns, int count,
                              int base, float weight, QRay* __restrict__ rays, int* __restrict__ q_path,
                              uint2* __restrict__ skips, PathState* __restrict__ paths, float* __restrict__ quality,
                              int* __restrict__ q_count, unsigned long long* __restrict__ stats)
{
    const long total = (long)ns * count;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *q_count = (int)total;
        atomicAdd(&stats[ST_RAYS], (unsigned long long)total);   // each is a TraceRay call
    }
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        int s = (int)(i / count), k = (int)(i % count);
        RadQuery q = queries[seeds[s]];
        float3 d = sample_direction(xyz(q.n), base, s, count, k);
        QRay r;
        r.org = make_float4(q.p.x, q.p.y, q.p.z, 1.0e-4f);   // MIN_ISECT_DEPTH
        r.dir = make_float4(d.x, d.y, d.z, CUDART_INF_F);
        rays[i] = r;
        q_path[i] = (int)i;
        skips[i] = make_uint2(q.prim, q.aux);
        PathState ps;
        ps.colour = make_float4(0.f, 0.f, 0.f, 0.f);
        ps.throughput = make_float4(1.f, 1.f, 1.f, weight);
        paths[i] = ps;
        quality[i] = 1.0f;
    }
}

// Depth of each sample ray's first hit (infinite for a miss), kept for the
// reduction while the wavefront moves on to reflection levels.
__global__ void k_first_hit(const QHit* __restrict__ hits, const int* __restrict__ q_count, int cap,
                            float* __restrict__ first_t)
{
    const int n = min(*q_count, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        QHit h = hits[i];
        first_t[i] = h.prim == 0xffffffffu ? CUDART_INF_F : h.t;
    }
}

// Ambient answers of nested queries (the sample rays' hits) into their rays:
// colour += ambient * factor; the ray's sample quality is the nested
// query's (ComputeAmbient's ticket.radiosityQuality, radiosity.cpp:454).
__global__ void k_rad_apply(const RadQuery* __restrict__ queries, const int* __restrict__ n_queries, int cap,
                            const float4* __restrict__ amb, PathState* __restrict__ paths,
                            float* __restrict__ quality)
{
    const int n = min(*n_queries, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        RadQuery q = queries[i];
        float4 a = amb[i];
        float4 c = paths[q.path].colour;
        paths[q.path].colour = make_float4(c.x + a.x * q.factor.x, c.y + a.y * q.factor.y, c.z + a.z * q.factor.z, c.w);
        if (quality)
            quality[q.path] = fminf(quality[q.path], a.w);
    }
}

// One warp per seed: the sums of GatherLight (radiosity.cpp:583-681) over
// the seed's sample rays, the new block (AddBlock, radiosity.cpp:1194-1233)
// and the seed's ambient colour (ComputeAmbient, radiosity.cpp:428-461).
__global__ void k_gather_reduce(DeviceScene S, RadCacheView C, RadParams R, const RadQuery* __restrict__ queries,
                                const int* __restrict__ seeds, int ns, int base, const float* __restrict__ first_t,
                                const PathState* __restrict__ paths, const float* __restrict__ quality,
                                const float4* __restrict__ partial, float4* __restrict__ out,
                                unsigned long long* __restrict__ rstats, uint32_t* err)
{
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int count = R.rays_per_sample;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < ns; s += warps) {
        float3 sum = f3(0.f, 0.f, 0.f);
        float qsum = 0.f, inv = 0.f, best = CUDART_INF_F;
        int best_k = -1;
        for (int k = lane; k < count; k += 32) {
            long i = (long)s * count + k;
            float q = quality[i];
            float3 c = xyz(paths[i].colour);
            sum = add(sum, mul(c, q));
            qsum += q;
            float t = first_t[i];
            inv += 1.0f / t;
            if (t < best || (t == best && k < best_k)) { best = t; best_k = k; }
        }
        for (int off = 16; off > 0; off >>= 1) {
            sum.x += __shfl_down_sync(0xffffffffu, sum.x, off);
            sum.y += __shfl_down_sync(0xffffffffu, sum.y, off);
            sum.z += __shfl_down_sync(0xffffffffu, sum.z, off);
            qsum += __shfl_down_sync(0xffffffffu, qsum, off);
            inv += __shfl_down_sync(0xffffffffu, inv, off);
            float ob = __shfl_down_sync(0xffffffffu, best, off);
            int ok = __shfl_down_sync(0xffffffffu, best_k, off);
            if (ok >= 0 && (ob < best || (ob == best && (best_k < 0 || ok < best_k)))) { best = ob; best_k = ok; }
        }
        if (lane != 0)
            continue;
        int qi = seeds[s];
        RadQuery q = queries[qi];
        float3 P = xyz(q.p);
        float3 ill = qsum == 0.f ? sum : mul(sum, 1.0f / qsum);
        float quality_s = qsum / (float)count;
        float te = to_eye(S, P);
        float min_d = te * R.min_reuse_factor, max_d = te * R.max_reuse_factor;
        float mean = (float)count / inv;
        if (best > max_d * 0.0001f) {
            mean = fminf(fmaxf(mean, min_d), max_d);
            int b = atomicAdd(C.count, 1);
            if (b < C.cap) {
                float3 tn = best_k >= 0 ? sample_direction(xyz(q.n), base, s, count, best_k) : f3(0.f, 0.f, 0.f);
                RadBlock blk;
                blk.p = make_float4(P.x, P.y, P.z, mean);
                blk.n = make_float4(q.n.x, q.n.y, q.n.z, best);
                blk.tn = make_float4(tn.x, tn.y, tn.z, quality_s);
                blk.ill = make_float4(ill.x, ill.y, ill.z, __int_as_float(R.depth));
                C.blocks[b] = blk;
                C.quick[b] = blk.p;
                int size, x, y, z;
                ot_index_sphere(P, (double)mean * R.address_factor, size, x, y, z);
                unsigned long long key = node_key(size + 256 * R.depth, x, y, z);
                int slot = node_insert(C, key);
                if (slot >= 0) {
                    C.bslot[b] = slot;   // filed into the node's segment by the next rebuild
                    uint32_t bit = occ_bit(C, key);
                    atomicOr(&C.occupancy[bit >> 5], 1u << (bit & 31));
                    atomicMin(&C.size_range[2 * R.depth], size);
                    atomicMax(&C.size_range[2 * R.depth + 1], size);
                } else {
                    C.bslot[b] = -1;
                    atomicOr(err, DE_CACHE_FULL);
                }
            } else {
                atomicOr(err, DE_CACHE_FULL);
            }
        }
        float4 pw = partial[qi];
        float W = pw.w;
        // (reused mean * reuse + gathered * quality) / (reuse + quality);
        // the reused mean times its weight is the weighted sum kept in partial
        float3 a = W > 0.f ? mul(add(xyz(pw), mul(ill, quality_s)), 1.0f / (W + quality_s)) : ill;
        out[qi] = finish_ambient(a, fminf(4.0f * (W + quality_s) / (float)R.reuse_count, 1.0f), R);
        atomicAdd(&rstats[RST_GATHERS0 + min(R.depth, 1)], 1ull);
    }
}

// Blocks written by the host (a loaded cache file, RadiosityCache::Load,
// radiosity.cpp:909-1010, which AddBlock's every line) filed as
// k_gather_reduce files a new sample: the quick-test record, the node
// ot_index_sphere picks for the harmonic mean distance times the depth's
// address factor, the node's occupancy bit and the depth's node-size range.
struct AddressFactors {
    float f[RAD_LEVELS];
};

__global__ void k_rad_file(RadCacheView C, AddressFactors af, int first, int n, uint32_t* err)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int b = first + i;
        if (b >= C.cap)
            break;
        const RadBlock blk = C.blocks[b];
        const int depth = __float_as_int(blk.ill.w);
        C.quick[b] = blk.p;
        C.bslot[b] = -1;
        if (depth < 0 || depth >= RAD_LEVELS)
            continue;
        int size, x, y, z;
        ot_index_sphere(xyz(blk.p), (double)blk.p.w * af.f[depth], size, x, y, z);
        const unsigned long long key = node_key(size + 256 * depth, x, y, z);
        const int slot = node_insert(C, key);
        if (slot < 0) {
            atomicOr(err, DE_CACHE_FULL);
            continue;
        }
        C.bslot[b] = slot;
        const uint32_t bit = occ_bit(C, key);
        atomicOr(&C.occupancy[bit >> 5], 1u << (bit & 31));
        atomicMin(&C.size_range[2 * depth], size);
        atomicMax(&C.size_range[2 * depth + 1], size);
    }
}

__global__ void k_rad_nic_answer(RadParams R, const int* __restrict__ seeds, int ns, const float4* __restrict__ pred,
                                 float4* __restrict__ out, unsigned long long* __restrict__ rstats)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        float4 p = pred[i];
        out[seeds[i]] = finish_ambient(f3(fmaxf(p.x, 0.f), fmaxf(p.y, 0.f), fmaxf(p.z, 0.f)), 1.0f, R);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(&rstats[RST_NIC], (unsigned long long)ns);
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace

cudaError_t rad_upload_directions(const float* xyz3)
{
    return cudaMemcpyToSymbol(c_dirs, xyz3, sizeof(float3) * RAD_DIRECTIONS);
}

cudaError_t launch_seg_rebuild(const RadCacheView& C, int grid, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(C.seg_total, 0, sizeof(int32_t), st);
    if (e != cudaSuccess)
        return e;
    k_seg_reset<<<grid, 256, 0, st>>>(C);
    k_seg_count<<<grid, 256, 0, st>>>(C);
    k_seg_alloc<<<grid, 256, 0, st>>>(C);
    k_seg_fill<<<grid, 256, 0, st>>>(C);
    return cudaGetLastError();
}

cudaError_t launch_rad_query(const DeviceScene& S, const RadCacheView& C, const RadParams& R, const RadQuery* queries,
                             const int* open, int n_open, int cap, int round, int last_round, float4* out,
                             float4* partial, unsigned long long* claims, uint32_t claim_mask, int* seeds,
                             int* n_seeds, int* next, int* n_next, unsigned long long* rstats, uint32_t* err,
                             int grid, cudaStream_t st)
{
    k_rad_query<<<grid, 128, 0, st>>>(S, C, R, queries, open, n_open, cap, round, last_round, out, partial, claims,
                                      claim_mask, seeds, n_seeds, next, n_next, rstats, err);
    return cudaGetLastError();
}

cudaError_t launch_gather_rays(const RadQuery* queries, const int* seeds, int ns, int count, int base, float weight,
                               QRay* rays, int* q_path, uint2* skips, PathState* paths, float* quality, int* q_count,
                               unsigned long long* stats, int grid, cudaStream_t st)
{
    k_gather_rays<<<grid, 256, 0, st>>>(queries, seeds, ns, count, base, weight, rays, q_path, skips, paths, quality,
                                        q_count, stats);
    return cudaGetLastError();
}

cudaError_t launch_first_hit(const QHit* hits, const int* q_count, int cap, float* first_t, int grid, cudaStream_t st)
{
    k_first_hit<<<grid, 128, 0, st>>>(hits, q_count, cap, first_t);
    return cudaGetLastError();
}

cudaError_t launch_rad_apply(const RadQuery* queries, const int* n_queries, int cap, const float4* amb,
                             PathState* paths, float* quality, int grid, cudaStream_t st)
{
    k_rad_apply<<<grid, 256, 0, st>>>(queries, n_queries, cap, amb, paths, quality);
    return cudaGetLastError();
}

cudaError_t launch_rad_file(const RadCacheView& C, const float* address_factor, int first, int n, uint32_t* err,
                            cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    AddressFactors af;
    for (int d = 0; d < RAD_LEVELS; d++)
        af.f[d] = address_factor[d];
    k_rad_file<<<cdiv(n, 256), 256, 0, st>>>(C, af, first, n, err);
    return cudaGetLastError();
}

cudaError_t launch_rad_nic_answer(const RadParams& R, const int* seeds, int ns, const float4* pred, float4* out,
                                  unsigned long long* rstats, int grid, cudaStream_t st)
{
    k_rad_nic_answer<<<grid, 256, 0, st>>>(R, seeds, ns, pred, out, rstats);
    return cudaGetLastError();
}

cudaError_t launch_gather_reduce(const DeviceScene& S, const RadCacheView& C, const RadParams& R,
                                 const RadQuery* queries, const int* seeds, int ns, int base, const float* first_t,
                                 const PathState* paths, const float* quality, const float4* partial, float4* out,
                                 unsigned long long* rstats, uint32_t* err, int grid, cudaStream_t st)
{
    k_gather_reduce<<<grid, 128, 0, st>>>(S, C, R, queries, seeds, ns, base, first_t, paths, quality, partial, out,
                                          rstats, err);
    return cudaGetLastError();
}

}  // namespace povgpu
