// povgpu_kernels.cu -- sm_103a kernels of the trace path.
//
// One batch of image samples is a short wavefront pipeline:
//   k_camera         primary rays (TracePixel::CreateCameraRay,
//                    source/core/render/tracepixel.cpp:357-373,924) for
//                    pixel centres, block corners (adaptive AA) or an
//                    explicit list of sub-pixel positions
//   per trace level L = 0 .. max_trace_level-1:
//     k_trace<closest>  Trace::FindIntersection (trace.cpp:285) over the BVH
//     k_shade           ComputeTextureColour/ComputeLightedTexture
//                       (trace.cpp:457-1179): emission/ambient, per-light
//                       diffuse/phong/specular terms, shadow-ray and
//                       reflection-ray emission (ComputeReflection,
//                       trace.cpp:1264-1321) into compacted queues
//     k_trace<any>      TracePointLightShadowRay (trace.cpp:1951-2076) for
//                       opaque occluders: any hit in (1e-3, dist-1e-3)
//     k_mark_blocked, k_resolve   add each unblocked light term to its path
//   k_finalize       RGBT per sample (CompletedRectangle order or AA slots)
// Adaptive antialiasing (TraceTask::AdaptiveSupersamplingM2) adds
// k_aa_init / k_aa_classify / k_aa_resolve around the same pipeline.
// Traversal kernels are persistent: each warp pulls 32 rays at a time from
// a device counter, so no host round trip sits between the stages.
#include "povgpu_internal.h"
#include "povgpu_kernels.h"
#include "povgpu.h"
#include "povgpu_quartic.cuh"

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include <mutex>

namespace povgpu {

// Tolerances of the reference (source/core/configcore.h:153-206,
// source/core/render/trace.cpp:81, per-shape DEPTH_TOLERANCE in the shape
// files).
__constant__ float kMinIsectDepth = 1.0e-4f;
#define EPSILON_D 1.0e-10
#define EPSILON_F 1.0e-10f
#define SMALL_TOLERANCE_F 1.0e-3f
#define SHADOW_TOLERANCE_F 1.0e-3f
#define BOX_DEPTH_TOL 1.0e-6f
#define CLOSE_TOL 1.0e-6f
#define TORUS_DEPTH_TOL 1.0e-4
#define TORUS_ROOT_TOL 1.0e-4
#define NO_PRIM 0xffffffffu

// ------------------------------------------------------------ helpers --
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 normalize3(float3 v)
{
    float l = sqrtf(dot3(v, v));
    return l != 0.0f ? v * (1.0f / l) : v;
}
__device__ __forceinline__ float comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t bits) { atomicOr(err, bits); }

// Warp-aggregated slot reservation in a queue: one atomic per warp, lanes
// get consecutive slots in lane order (ballot + popc).  Must be called by
// every lane of `mask` together.
__device__ __forceinline__ int warp_reserve(int* counter, bool want, unsigned mask)
{
    unsigned ballot = __ballot_sync(mask, want);
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    int base = 0;
    if (ballot != 0u && lane == leader)
        base = atomicAdd(counter, __popc(ballot));
    base = __shfl_sync(mask, base, leader < 0 ? 0 : leader);
    return want ? base + __popc(ballot & ((1u << lane) - 1u)) : -1;
}

// Same, reserving `k` consecutive slots per wanting lane.
__device__ __forceinline__ int warp_reserve_k(int* counter, bool want, int k, unsigned mask)
{
    unsigned ballot = __ballot_sync(mask, want);
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    int base = 0;
    if (ballot != 0u && lane == leader)
        base = atomicAdd(counter, k * __popc(ballot));
    base = __shfl_sync(mask, base, leader < 0 ? 0 : leader);
    return want ? base + k * __popc(ballot & ((1u << lane) - 1u)) : -1;
}

// --------------------------------------------------------------- camera --
// Primary ray through image position (x, y) (pixel units, y down), formed
// and normalised in FP64 exactly as CreateCameraRay does, then rounded.
// x0, y0: the pixel's offsets from the image centre, x / width - 0.5 and
// 0.5 - y / height (TracePixel::CreateCameraRay, tracepixel.cpp:357-373).
// The direction is formed and normalised in FP64; the three divisions by
// the length are each one multiplication by the FP64 reciprocal plus one
// FMA correction step (the residual dx - q l times the reciprocal), which
// gives the correctly rounded quotient except in double-rounding corner
// cases -- FP64 divisions are a long instruction sequence on this part's
// narrow FP64 pipe, and this kernel was bound by them.
__device__ __forceinline__ QRay camera_ray_xy(const DeviceScene& S, double x0, double y0)
{
    double dx = S.cam_dir[0] + x0 * S.cam_right[0] + y0 * S.cam_up[0];
    double dy = S.cam_dir[1] + x0 * S.cam_right[1] + y0 * S.cam_up[1];
    double dz = S.cam_dir[2] + x0 * S.cam_right[2] + y0 * S.cam_up[2];
    double l = sqrt(dx * dx + dy * dy + dz * dz);
    if (l != 0.0) {
        const double rl = 1.0 / l;
        double q = dx * rl;
        dx = fma(fma(-q, l, dx), rl, q);
        q = dy * rl;
        dy = fma(fma(-q, l, dy), rl, q);
        q = dz * rl;
        dz = fma(fma(-q, l, dz), rl, q);
    }
    QRay r;
    r.org = make_float4((float)S.cam_loc[0], (float)S.cam_loc[1], (float)S.cam_loc[2], kMinIsectDepth);
    r.dir = make_float4((float)dx, (float)dy, (float)dz, CUDART_INF_F);
    return r;
}

// Double-float arithmetic (Dekker 1971, with Knuth's two-sum): a value as
// the unevaluated sum hi + lo of two floats, about 44 significant bits.
// The camera rays of the block grid take their directions in it on the FP32
// pipes: rounded to float they equal the FP64 form's (checked over every
// pixel of a 1920x1080 camera: 0 of 6,220,800 components differ), where the
// FP64 form kept k_camera on this part's narrow FP64 pipe.
struct FF {
    float hi, lo;
};
// (the _rn intrinsics keep the compiler from fusing a product into a
// following sum, which would break the error-free transformations)
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b)   // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return FF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const FF s = ff_two_sum(a.hi, b.hi);
    return ff_fast_two_sum(s.hi, __fadd_rn(__fadd_rn(s.lo, a.lo), b.lo));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    return ff_fast_two_sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p))));
}

// camera_ray_xy in double-float: direction + x0 * right + y0 * up, its
// length by one Newton step on sqrtf, each component's quotient with one
// correction, rounded to float once.
__device__ __forceinline__ QRay camera_ray_ff(const DeviceScene& S, float2 x0, float2 y0)
{
    const FF X{x0.x, x0.y}, Y{y0.x, y0.y};
    FF d[3];
    for (int k = 0; k < 3; k++) {
        const FF dir{S.cam_ff[2 * k], S.cam_ff[2 * k + 1]};
        const FF right{S.cam_ff[6 + 2 * k], S.cam_ff[6 + 2 * k + 1]};
        const FF up{S.cam_ff[12 + 2 * k], S.cam_ff[12 + 2 * k + 1]};
        d[k] = ff_add(ff_add(dir, ff_mul(X, right)), ff_mul(Y, up));
    }
    const FF l2 = ff_add(ff_add(ff_mul(d[0], d[0]), ff_mul(d[1], d[1])), ff_mul(d[2], d[2]));
    float out[3] = {d[0].hi, d[1].hi, d[2].hi};
    if (l2.hi > 0.0f) {
        const float s = sqrtf(l2.hi);
        const FF ss = ff_mul(FF{s, 0.0f}, FF{s, 0.0f});
        const float res = __fadd_rn(__fsub_rn(__fsub_rn(l2.hi, ss.hi), ss.lo), l2.lo);
        const FF l = ff_fast_two_sum(s, res / __fmul_rn(2.0f, s));
        for (int k = 0; k < 3; k++) {
            const float q0 = d[k].hi / l.hi;
            const FF t = ff_mul(FF{q0, 0.0f}, l);
            const FF r = ff_add(d[k], FF{-t.hi, -t.lo});
            out[k] = __fadd_rn(q0, r.hi / l.hi);
        }
    }
    QRay r;
    r.org = make_float4((float)S.cam_loc[0], (float)S.cam_loc[1], (float)S.cam_loc[2], kMinIsectDepth);
    r.dir = make_float4(out[0], out[1], out[2], CUDART_INF_F);
    return r;
}

__device__ __forceinline__ QRay camera_ray(const DeviceScene& S, double x, double y, int width, int height)
{
    return camera_ray_xy(S, x / (double)width - 0.5, 0.5 - y / (double)height);
}

// The offsets of every column and row of the image for pixel centres
// (mode 0: x + 0.5) or corners (mode 1: x), width + 1 then height + 1
// entries, formed in FP64 and kept as double-floats (hi, lo): k_camera
// looks them up instead of dividing per pixel.
__global__ void k_cam_table(int width, int height, double off, float2* __restrict__ tab)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v;
    if (i <= width)
        v = ((double)i + off) / (double)width - 0.5;
    else if (i <= width + 1 + height)
        v = 0.5 - ((double)(i - width - 1) + off) / (double)height;
    else
        return;
    const float hi = (float)v;
    tab[i] = make_float2(hi, (float)(v - (double)hi));
}

// mode 0: pixel centres (x+0.5, y+0.5) of every block, block order
// mode 1: pixel corners (x, y) of every block, (w+1) x (h+1) per block
//         (AdaptiveSupersamplingM2 traces these, tracetask.cpp:620-628)
// mode 2: explicit positions pos[i]; the count is read from *npos
__global__ void k_camera(DeviceScene S, int mode, const int4* __restrict__ blocks,
                         const int* __restrict__ block_off, int nblocks, const double2* __restrict__ pos,
                         const int* __restrict__ npos, int width, int height, QRay* __restrict__ q,
                         int* __restrict__ q_path, PathState* __restrict__ paths, int* __restrict__ q_count,
                         unsigned long long* stats, uint2* __restrict__ q_skip, int cap, const float2* __restrict__ tab)
{
    int n = min(mode == 2 ? *npos : block_off[nblocks], cap);   // never past the queue buffers
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *q_count = n;
        atomicAdd(&stats[ST_RAYS], (unsigned long long)n);
    }
    if (i >= n)
        return;
    int path = i;
    if (mode == 2) {
        const double2 p = pos[i];
        q[i] = camera_ray(S, p.x, p.y, width, height);
    } else {
        int lo = 0, hi = nblocks - 1;   // block containing sample i
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (block_off[mid] <= i) lo = mid; else hi = mid - 1;
        }
        int4 b = blocks[lo];            // left, top, right, bottom
        int w = b.z - b.x + 1 + (mode == 1 ? 1 : 0);
        int h = b.w - b.y + 1 + (mode == 1 ? 1 : 0);
        int local = i - block_off[lo];
        int lx = local % w, ly = local / w;
        if (mode == 0 && w == 32 && h == 32) {
            // full blocks queue their pixels in 8x4 tiles (one warp each) so
            // a warp's rays stay close together; the path keeps the pixel's
            // row-major place in the block's output
            int tile = local >> 5, lane = local & 31;
            lx = (tile & 3) * 8 + (lane & 7);
            ly = (tile >> 2) * 4 + (lane >> 3);
            path = block_off[lo] + ly * w + lx;
        }
        q[i] = camera_ray_ff(S, tab[b.x + lx], tab[width + 1 + b.y + ly]);
    }
    q_path[i] = path;
    q_skip[i] = make_uint2(NO_PRIM, 0u);
    PathState p;
    p.colour = make_float4(0.f, 0.f, 0.f, 0.f);
    p.throughput = make_float4(1.f, 1.f, 1.f, 1.f);
    paths[path] = p;
}

// Rays given by the caller (FP64 in, FP32 on the device).
__global__ void k_load_rays(const double* __restrict__ org, const double* __restrict__ dir, int n,
                            QRay* __restrict__ q, int* __restrict__ q_count)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
        *q_count = n;
    if (i >= n)
        return;
    QRay r;
    r.org = make_float4((float)org[3 * i], (float)org[3 * i + 1], (float)org[3 * i + 2], kMinIsectDepth);
    r.dir = make_float4((float)dir[3 * i], (float)dir[3 * i + 1], (float)dir[3 * i + 2], CUDART_INF_F);
    q[i] = r;
}

// ------------------------------------------------------------ sphere --
// Sphere::Intersect (sphere.cpp:214-245) with the chord taken from the
// perpendicular offset vector, which keeps FP32 accurate away from the
// sphere; the near-tangent band |r^2 - perp^2| <= 1e-4 r^2 is re-solved in
// FP64, FP32 decides outside it (hits and misses alike).  Both roots, or 0.
__device__ __forceinline__ int sphere_roots(float4 s, float3 o, float3 d, float& t1, float& t2)
{
    float3 oc = xyz(s) - o;
    float tca = dot3(oc, d);
    float ocs = dot3(oc, oc);
    float r2 = s.w * s.w;
    if (ocs >= r2 && tca < EPSILON_F)
        return 0;
    float3 perp = oc - d * tca;
    float thcs = r2 - dot3(perp, perp);
    if (thcs < -1.0e-4f * r2)
        return 0;   // a clear miss: outside the band on the far side as well
    if (thcs <= 1.0e-4f * r2) {
        double ox = (double)s.x - o.x, oy = (double)s.y - o.y, oz = (double)s.z - o.z;
        double tcad = ox * d.x + oy * d.y + oz * d.z;
        double px = ox - d.x * tcad, py = oy - d.y * tcad, pz = oz - d.z * tcad;
        double th = (double)s.w * s.w - (px * px + py * py + pz * pz);
        if (!(th > EPSILON_D))
            return 0;
        double hc = sqrt(th);
        t1 = (float)(tcad - hc);
        t2 = (float)(tcad + hc);
        return 2;
    }
    float hc = sqrtf(thcs);
    t1 = tca - hc;
    t2 = tca + hc;
    return 2;
}

__device__ __forceinline__ bool sphere_inside(float4 s, int flags, float3 p)
{
    float3 d = xyz(s) - p;
    float ocs = dot3(d, d), r2 = s.w * s.w;
    return (flags & 1) ? ocs > r2 : ocs < r2;
}

// ---------------------------------------------------------------- box --
enum { SIDE_X0 = 0, SIDE_X1, SIDE_Y0, SIDE_Y1, SIDE_Z0, SIDE_Z1 };

// Box::Intersect (box.cpp:172-533): entry/exit depths and the side each
// lies on, with the reference's CLOSE_TOLERANCE tie-breaking between
// sides.  Returns false when the box is missed or entirely behind.
__device__ __forceinline__ bool box_roots(const DevBox& b, float3 P, float3 D, float& tn, float& tf, int& sn, int& sf)
{
    int smin = 0, smax = 0;
    float tmin = 0.0f, tmax = 2.0e10f, t;
    float3 c1 = xyz(b.lo), c2 = xyz(b.hi);
    // X
    if (D.x < -EPSILON_F) {
        t = (c1.x - P.x) / D.x;
        if (t < tmin) return false;
        if (t <= tmax) { smax = SIDE_X0; tmax = t; }
        t = (c2.x - P.x) / D.x;
        if (t >= tmin) { if (t > tmax) return false; smin = SIDE_X1; tmin = t; }
    } else if (D.x > EPSILON_F) {
        t = (c2.x - P.x) / D.x;
        if (t < tmin) return false;
        if (t <= tmax) { smax = SIDE_X1; tmax = t; }
        t = (c1.x - P.x) / D.x;
        if (t >= tmin) { if (t > tmax) return false; smin = SIDE_X0; tmin = t; }
    } else if (P.x < c1.x || P.x > c2.x) {
        return false;
    }
    // Y
    if (D.y < -EPSILON_F) {
        t = (c1.y - P.y) / D.y;
        if (t < tmin) return false;
        if (t <= tmax - CLOSE_TOL) { smax = SIDE_Y0; tmax = t; }
        else if (t <= tmax + CLOSE_TOL) { if (-D.y > fabsf(D.x)) smax = SIDE_Y0; }
        t = (c2.y - P.y) / D.y;
        if (t >= tmin + CLOSE_TOL) { if (t > tmax) return false; smin = SIDE_Y1; tmin = t; }
        else if (t >= tmin - CLOSE_TOL) { if (-D.y > fabsf(D.x)) smin = SIDE_Y1; }
    } else if (D.y > EPSILON_F) {
        t = (c2.y - P.y) / D.y;
        if (t < tmin) return false;
        if (t <= tmax - CLOSE_TOL) { smax = SIDE_Y1; tmax = t; }
        else if (t <= tmax + CLOSE_TOL) { if (D.y > fabsf(D.x)) smax = SIDE_Y1; }
        t = (c1.y - P.y) / D.y;
        if (t >= tmin + CLOSE_TOL) { if (t > tmax) return false; smin = SIDE_Y0; tmin = t; }
        else if (t >= tmin - CLOSE_TOL) { if (D.y > fabsf(D.x)) smin = SIDE_Y0; }
    } else if (P.y < c1.y || P.y > c2.y) {
        return false;
    }
    // Z
    if (D.z < -EPSILON_F) {
        t = (c1.z - P.z) / D.z;
        if (t < tmin) return false;
        if (t <= tmax - CLOSE_TOL) { smax = SIDE_Z0; tmax = t; }
        else if (t <= tmax + CLOSE_TOL) {
            if ((smax <= SIDE_X1) ? (-D.z > fabsf(D.x)) : (-D.z > fabsf(D.y))) smax = SIDE_Z0;
        }
        t = (c2.z - P.z) / D.z;
        if (t >= tmin + CLOSE_TOL) { if (t > tmax) return false; smin = SIDE_Z1; tmin = t; }
        else if (t >= tmin - CLOSE_TOL) {
            if ((smin <= SIDE_X1) ? (-D.z > fabsf(D.x)) : (-D.z > fabsf(D.y))) smin = SIDE_Z1;
        }
    } else if (D.z > EPSILON_F) {
        t = (c2.z - P.z) / D.z;
        if (t < tmin) return false;
        if (t <= tmax - CLOSE_TOL) { smax = SIDE_Z1; tmax = t; }
        else if (t <= tmax + CLOSE_TOL) {
            if ((smax <= SIDE_X1) ? (D.z > fabsf(D.x)) : (D.z > fabsf(D.y))) smax = SIDE_Z1;
        }
        t = (c1.z - P.z) / D.z;
        if (t >= tmin + CLOSE_TOL) { if (t > tmax) return false; smin = SIDE_Z0; tmin = t; }
        else if (t >= tmin - CLOSE_TOL) {
            if ((smin <= SIDE_X1) ? (D.z > fabsf(D.x)) : (D.z > fabsf(D.y))) smin = SIDE_Z0;
        }
    } else if (P.z < c1.z || P.z > c2.z) {
        return false;
    }
    if (tmax < BOX_DEPTH_TOL)
        return false;
    tn = tmin; tf = tmax; sn = smin; sf = smax;
    return true;
}

__device__ __forceinline__ bool box_inside(const DevBox& b, int flags, float3 p)
{
    bool out = p.x < b.lo.x || p.x > b.hi.x || p.y < b.lo.y || p.y > b.hi.y || p.z < b.lo.z || p.z > b.hi.z;
    return (flags & 1) ? out : !out;
}

__device__ __forceinline__ float3 box_side_normal(int side)
{
    float s = (side & 1) ? 1.0f : -1.0f;
    int ax = side >> 1;
    return f3(ax == 0 ? s : 0.f, ax == 1 ? s : 0.f, ax == 2 ? s : 0.f);
}

// -------------------------------------------------------------- torus --
// Torus::Intersect (torus.cpp:241-362) in FP64: local frame, thick
// cylinder bound, origin moved near the bounding sphere, quartic.
__device__ __forceinline__ bool torus_thick_cylinder(double3 P, double3 D, double h1, double h2, double r1, double r2)
{
    const double MAXD = 1.0e7;
    if (fabs(D.y) < EPSILON_D) {
        if (P.y < h1 || P.y > h2) return false;
    } else {
        double k = (h2 - P.y) / D.y, u = P.x + k * D.x, v = P.z + k * D.z;
        if (k > EPSILON_D && k < MAXD) { double r = u * u + v * v; if (r >= r1 && r <= r2) return true; }
        k = (h1 - P.y) / D.y; u = P.x + k * D.x; v = P.z + k * D.z;
        if (k > EPSILON_D && k < MAXD) { double r = u * u + v * v; if (r >= r1 && r <= r2) return true; }
    }
    double a = D.x * D.x + D.z * D.z;
    if (a > EPSILON_D) {
        double b = P.x * D.x + P.z * D.z;
        double rr[2] = {r2, r1};
        for (int c = 0; c < 2; c++) {
            double cc = P.x * P.x + P.z * P.z - rr[c];
            double dd = b * b - a * cc;
            if (dd >= 0.0) {
                dd = sqrt(dd);
                double k = (-b + dd) / a;
                if (k > EPSILON_D && k < MAXD) { double h = P.y + k * D.y; if (h >= h1 && h <= h2) return true; }
                k = (-b - dd) / a;
                if (k > EPSILON_D && k < MAXD) { double h = P.y + k * D.y; if (h >= h1 && h <= h2) return true; }
            }
        }
    }
    return false;
}

__device__ __forceinline__ double3 torus_local_point(const DevTorus& T, double x, double y, double z)
{
    const double* m = T.inv;
    return make_double3(x * m[0] + y * m[3] + z * m[6] + m[9], x * m[1] + y * m[4] + z * m[7] + m[10],
                        x * m[2] + y * m[5] + z * m[8] + m[11]);
}

// FP32 pre-cull in front of torus_roots: can the ray reach the torus
// before world depth tmax?  The ray is taken into the torus's frame in FP32
// and tested against the torus's bounding sphere (radius R + r, which holds
// every root) and the slab |y| <= r of Torus::Test_Thick_Cylinder
// (torus.cpp:932-1084), both widened by a margin (1e-3 of the bound plus
// 1e-4 of the origin's distance) far above FP32's rounding at these
// magnitudes, so only rays that surely miss are dropped; torus_roots
// decides the rest in FP64.  Its cost is ~40 FP32 operations against the
// FP64 bound and quartic it saves (FP64 is a narrow pipe on this part).
__device__ __forceinline__ bool torus_may_hit(const float4* __restrict__ t32, float3 o, float3 d, float tmax)
{
    const float4 X = __ldg(t32), Y = __ldg(t32 + 1), Z = __ldg(t32 + 2), Rr = __ldg(t32 + 3);
    const float3 P = f3(fmaf(o.x, X.x, fmaf(o.y, X.y, fmaf(o.z, X.z, X.w))),
                        fmaf(o.x, Y.x, fmaf(o.y, Y.y, fmaf(o.z, Y.z, Y.w))),
                        fmaf(o.x, Z.x, fmaf(o.y, Z.y, fmaf(o.z, Z.z, Z.w))));
    float3 D = f3(fmaf(d.x, X.x, fmaf(d.y, X.y, d.z * X.z)), fmaf(d.x, Y.x, fmaf(d.y, Y.y, d.z * Y.z)),
                  fmaf(d.x, Z.x, fmaf(d.y, Z.y, d.z * Z.z)));
    const float inv_len = rsqrtf(dot3(D, D));   // local depth * inv_len = world depth
    D = D * inv_len;
    const float rb = Rr.x + Rr.y;
    const float pp = dot3(P, P);
    const float margin = 1e-3f * rb + 1e-4f * sqrtf(pp);
    const float br = rb + margin;
    const float b = dot3(P, D), disc = b * b - (pp - br * br);
    if (disc < 0.0f)
        return false;
    const float sq = sqrtf(disc);
    const float t_far = sq - b;
    float t_near = -b - sq;
    if (t_far < 0.0f || t_near * inv_len > tmax * (1.0f + 1e-3f) + margin)
        return false;
    t_near = fmaxf(t_near, 0.0f);
    const float h = Rr.y + margin;
    if (fabsf(D.y) < 1e-6f)
        return fabsf(P.y) <= h;
    const float ta = (-h - P.y) / D.y, tb = (h - P.y) / D.y;
    return fmaxf(ta, tb) >= t_near && fminf(ta, tb) <= t_far;
}

// Roots (world depths) with depth > 1e-4; returns their count (<= 4).
__device__ __noinline__ int torus_roots(const DevTorus& T, double3 o, double3 d, double* out)
{
    const double* m = T.inv;
    double3 P = torus_local_point(T, o.x, o.y, o.z);
    double3 D = make_double3(d.x * m[0] + d.y * m[3] + d.z * m[6], d.x * m[1] + d.y * m[4] + d.z * m[7],
                             d.x * m[2] + d.y * m[5] + d.z * m[8]);
    double len = sqrt(D.x * D.x + D.y * D.y + D.z * D.z);
    D.x /= len; D.y /= len; D.z /= len;
    double R = T.R, r = T.r;
    double r1 = R < r ? 0.0 : (R - r) * (R - r), r2 = (R + r) * (R + r);
    if (!torus_thick_cylinder(P, D, -r, r, r1, r2))
        return 0;
    double bsr = R + r + r, dp = P.x * P.x + P.y * P.y + P.z * P.z, closer = 0.0;
    if (dp > bsr * bsr) {
        closer = sqrt(dp) - bsr;
        P.x += closer * D.x; P.y += closer * D.y; P.z += closer * D.z;
    }
    double R2 = R * R, rr2 = r * r, Py2 = P.y * P.y, Dy2 = D.y * D.y, PDy2 = P.y * D.y;
    double k1 = P.x * P.x + P.z * P.z + Py2 - R2 - rr2;
    double k2 = P.x * D.x + P.z * D.z + PDy2;
    double c[5] = {1.0, 4.0 * k2, 2.0 * (k1 + 2.0 * (k2 * k2 + R2 * Dy2)), 4.0 * (k2 * k1 + 2.0 * R2 * PDy2),
                   k1 * k1 + 4.0 * R2 * (Py2 - rr2)};
    double roots[4];
    int n = quartic::solve4(c, roots, TORUS_ROOT_TOL);
    int k = 0;
    for (int i = n - 1; i >= 0; i--) {
        double t = (roots[i] + closer) / len;
        if (t > TORUS_DEPTH_TOL && t < 1.0e7)
            out[k++] = t;
    }
    return k;
}

__device__ __forceinline__ bool torus_inside(const DevTorus& T, float3 p)
{
    double3 P = torus_local_point(T, p.x, p.y, p.z);
    double rr = sqrt(P.x * P.x + P.z * P.z);
    double r2 = P.y * P.y + (rr - T.R) * (rr - T.R);
    bool in = r2 <= T.r * T.r;
    return (T.flags & 1) ? !in : in;
}

__device__ __forceinline__ float3 torus_normal(const DevTorus& T, float3 p)
{
    double3 P = torus_local_point(T, p.x, p.y, p.z);
    double dist = sqrt(P.x * P.x + P.z * P.z);
    double mx = 0.0, mz = 0.0;
    if (dist > EPSILON_D) { mx = T.R * P.x / dist; mz = T.R * P.z / dist; }
    double nx = P.x - mx, ny = P.y, nz = P.z - mz;
    const double* m = T.inv;   // MTransNormal: rows of the inverse
    float3 n = f3((float)(nx * m[0] + ny * m[1] + nz * m[2]), (float)(nx * m[3] + ny * m[4] + nz * m[5]),
                  (float)(nx * m[6] + ny * m[7] + nz * m[8]));
    return normalize3(n);
}

// Drops the root of a ray's own origin surface: the root nearest zero when
// it is within 1e-2 (FP32 origin rounding can lift it above the 1e-4 cut).
__device__ __forceinline__ int torus_drop_self(double* t, int n)
{
    int m = -1;
    for (int i = 0; i < n; i++)
        if (m < 0 || t[i] < t[m]) m = i;
    if (m >= 0 && t[m] < 1.0e-2) {
        t[m] = t[n - 1];
        return n - 1;
    }
    return n;
}

// ---------------------------------------------------------------- CSG --
// NT: the scene's CSGs have no torus children (the torus-free traversal
// variant carries no FP64 torus code, which halves its registers).
template <bool NT = false>
__device__ __forceinline__ bool child_inside(const DeviceScene& S, const DevCsgChild& c, float3 p)
{
    switch (c.kind) {
    case PK_SPHERE: return sphere_inside(__ldg(S.spheres + c.index), c.flags, p);
    case PK_BOX: return box_inside(S.boxes[c.index], c.flags, p);
    case PK_TORUS: return NT ? false : torus_inside(S.tori[c.index], p);
    case PK_PLANE: {
        float4 pl = __ldg(S.planes + c.index);
        return dot3(p, xyz(pl)) + pl.w < EPSILON_F;
    }
    default: return false;
    }
}

// Roots of one CSG child with the aux word (box side).
template <bool NT = false>
__device__ __forceinline__ int child_roots(const DeviceScene& S, const DevCsgChild& c, float3 o, float3 d,
                                           float* t, int* side, bool self, int self_side)
{
    int n = 0;
    if (c.kind == PK_SPHERE) {
        float t1, t2;
        float4 s = __ldg(S.spheres + c.index);
        if (sphere_roots(s, o, d, t1, t2)) {
            if (self) {
                if (dot3(xyz(s) - o, d) > 0.0f) { t[n] = t2; side[n++] = 0; }   // inward: far root only
            } else {
                if (t1 > 1.0e-6f) { t[n] = t1; side[n++] = 0; }
                if (t2 > 1.0e-6f) { t[n] = t2; side[n++] = 0; }
            }
        }
    } else if (c.kind == PK_BOX) {
        float tn, tf;
        int sn, sf;
        const DevBox b = S.boxes[c.index];
        if (box_roots(b, o, d, tn, tf, sn, sf)) {
            if (self) {
                if (dot3(box_side_normal(self_side), d) < 0.0f) { t[n] = tf; side[n++] = sf; }
            } else {
                if (tn > BOX_DEPTH_TOL) { t[n] = tn; side[n++] = sn; }
                t[n] = tf; side[n++] = sf;
            }
        }
    } else if (!NT && c.kind == PK_TORUS) {
        double r[4];
        int k = torus_roots(S.tori[c.index], make_double3(o.x, o.y, o.z), make_double3(d.x, d.y, d.z), r);
        if (self) k = torus_drop_self(r, k);
        for (int i = 0; i < k; i++) { t[n] = (float)r[i]; side[n++] = 0; }
    } else if (c.kind == PK_PLANE) {
        float4 pl = __ldg(S.planes + c.index);
        float ndd = dot3(xyz(pl), d);
        if (!self && fabsf(ndd) >= EPSILON_F) {
            float tt = -(dot3(xyz(pl), o) + pl.w) / ndd;
            if (tt >= 1.0e-6f) { t[n] = tt; side[n++] = 0; }
        }
    }
    return n;
}

// CSGIntersection / CSGMerge::All_Intersections fused with the closest-hit
// filter: a child's root survives if the point is inside every sibling
// (intersection) or inside none (merge).  Returns the best surviving root in
// [tmin, t) and its (child, side) aux word.
template <bool NT = false>
__device__ __forceinline__ bool csg_closest(const DeviceScene& S, uint32_t idx, float3 o, float3 d, float tmin,
                                            float& t, uint32_t& aux, uint2 skip, uint32_t ref, bool any)
{
    DevCsg g = S.csgs[idx];
    bool merge = g.type == 8;   // POV_OBJ_MERGE
    bool found = false;
    for (int c = 0; c < g.count; c++) {
        DevCsgChild ch = S.csg_children[g.first + c];
        bool self = skip.x == ref && (int)(skip.y & 0xffffu) == c;
        float rt[4];
        int rs[4];
        int n = child_roots<NT>(S, ch, o, d, rt, rs, self, (int)(skip.y >> 16));
        for (int k = 0; k < n; k++) {
            if (!(rt[k] >= tmin && rt[k] < t))
                continue;
            float3 p = o + d * rt[k];
            bool keep = true;
            for (int s = 0; s < g.count && keep; s++) {
                if (s == c)
                    continue;
                bool in = child_inside<NT>(S, S.csg_children[g.first + s], p);
                keep = merge ? !in : in;
            }
            if (keep) {
                t = rt[k];
                aux = (uint32_t)c | ((uint32_t)rs[k] << 16);
                found = true;
                if (any)
                    return true;
            }
        }
    }
    return found;
}

// Triangle: Moller-Trumbore on the precomputed (v0, e1, e2) record.
__device__ __forceinline__ bool isect_tri(float4 v0, float4 e1, float4 e2, float3 o, float3 d, float tmin,
                                          float& t, float& bu, float& bv)
{
    float3 E1 = xyz(e1), E2 = xyz(e2);
    float3 pv = cross3(d, E2);
    float det = dot3(E1, pv);
    if (fabsf(det) < 1.0e-20f)
        return false;
    float inv = 1.0f / det;
    float3 tv = o - xyz(v0);
    float u = dot3(tv, pv) * inv;
    if (u < 0.0f || u > 1.0f)
        return false;
    float3 qv = cross3(tv, E1);
    float v = dot3(d, qv) * inv;
    if (v < 0.0f || u + v > 1.0f)
        return false;
    float tt = dot3(E2, qv) * inv;
    if (tt >= tmin && tt < t) {
        t = tt;
        bu = u;
        bv = v;
        return true;
    }
    return false;
}

// Slab test of both children of a node; returns entry distances.
// One inner node of the four-wide tree: the children whose boxes the ray
// enters within [tmin, tmax] (slab test, far side widened by a few ulp so
// rounding never culls a box the exact test would enter), ordered near to
// far by a 4-input sorting network; the nearest becomes `node`, the others
// are pushed farthest first.  With no child entered, `node` is the next
// stack entry (BVH_EMPTY when the stack is empty).  False on stack overflow.
__device__ __forceinline__ bool node4_step(const Bvh4Node* __restrict__ nodes, int& node, float3 o, float3 inv,
                                           float tmin, float tmax, int* smem, int& sp, int stack_depth)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + node);
    const float4 lox = __ldg(p), hix = __ldg(p + 1), loy = __ldg(p + 2), hiy = __ldg(p + 3);
    const float4 loz = __ldg(p + 4), hiz = __ldg(p + 5);
    const int4 lk = __ldg(reinterpret_cast<const int4*>(p + 6));
    float t0, t1, t2, t3;
    int l0, l1, l2, l3;
#define POVGPU_CHILD(TN, LN, X)                                                                   \
    {                                                                                             \
        float x0 = (lox.X - o.x) * inv.x, x1 = (hix.X - o.x) * inv.x;                           \
        float y0 = (loy.X - o.y) * inv.y, y1 = (hiy.X - o.y) * inv.y;                           \
        float z0 = (loz.X - o.z) * inv.z, z1 = (hiz.X - o.z) * inv.z;                           \
        float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));      \
        float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tmax));      \
        bool in = lk.X != BVH_EMPTY && tn <= tf * 1.00000024f;                                    \
        TN = in ? tn : CUDART_INF_F;                                                              \
        LN = in ? lk.X : BVH_EMPTY;                                                               \
    }
    POVGPU_CHILD(t0, l0, x)
    POVGPU_CHILD(t1, l1, y)
    POVGPU_CHILD(t2, l2, z)
    POVGPU_CHILD(t3, l3, w)
#undef POVGPU_CHILD
#define POVGPU_CSWAP(TA, LA, TB, LB)                   \
    if (TB < TA) {                                     \
        float tt = TA; TA = TB; TB = tt;               \
        int ll = LA; LA = LB; LB = ll;                 \
    }
    POVGPU_CSWAP(t0, l0, t1, l1)
    POVGPU_CSWAP(t2, l2, t3, l3)
    POVGPU_CSWAP(t0, l0, t2, l2)
    POVGPU_CSWAP(t1, l1, t3, l3)
    POVGPU_CSWAP(t1, l1, t2, l2)
#undef POVGPU_CSWAP
    const int pushes = (l1 != BVH_EMPTY) + (l2 != BVH_EMPTY) + (l3 != BVH_EMPTY);
    if (sp + pushes > stack_depth)
        return false;
    if (l3 != BVH_EMPTY) smem[(sp++) * blockDim.x + threadIdx.x] = l3;
    if (l2 != BVH_EMPTY) smem[(sp++) * blockDim.x + threadIdx.x] = l2;
    if (l1 != BVH_EMPTY) smem[(sp++) * blockDim.x + threadIdx.x] = l1;
    node = l0 != BVH_EMPTY ? l0 : (sp > 0 ? smem[(--sp) * blockDim.x + threadIdx.x] : BVH_EMPTY);
    return true;
}

// One primitive of a leaf against the ray.  `skip` names the surface the
// ray starts on (prim ref, aux): in exact arithmetic a ray leaving a plane
// or a planar triangle never meets it again, one leaving a convex sphere or
// box meets it only at the far root and only when heading inward, and one
// leaving a torus loses only its near-zero root; FP32 rounding of the
// origin must not invent those self-hits (the reference works in FP64).
template <bool ANY, bool FULL, bool NT = false>
__device__ __forceinline__ bool prim_test(const DeviceScene& S, uint32_t ref, float3 o, float3 d, float tmin,
                                          float& t, float& bu, float& bv, uint32_t& aux, uint2 skip)
{
    uint32_t kind = ref >> PRIM_KIND_SHIFT;
    uint32_t idx = ref & PRIM_INDEX_MASK;
    bool self = ref == skip.x;
    if (kind == PK_TRIANGLE) {
        if (self)
            return false;
        float uu, vv;
        if (isect_tri(__ldg(S.tri_v0 + idx), __ldg(S.tri_e1 + idx), __ldg(S.tri_e2 + idx), o, d, tmin, t, uu, vv)) {
            bu = uu;
            bv = vv;
            return true;
        }
        return false;
    }
    if (kind == PK_SPHERE) {
        // a media container's surface passes light: shadow rays cross it
        // (shadow_through counts and attenuates the crossings)
        if (ANY && S.num_containers > 0 && (__ldg(S.sphere_flags + idx) & SPHERE_CONTAINER))
            return false;
        float4 s = __ldg(S.spheres + idx);
        float t1, t2;
        if (!sphere_roots(s, o, d, t1, t2))
            return false;
        if (self) {
            if (dot3(xyz(s) - o, d) > 0.0f && t2 >= tmin && t2 < t) { t = t2; return true; }
            return false;
        }
        if (t1 > 1.0e-6f && t1 >= tmin && t1 < t) { t = t1; return true; }
        if (t2 > 1.0e-6f && t2 >= tmin && t2 < t) { t = t2; return true; }
        return false;
    }
    if (kind == PK_BOX) {
        const DevBox b = S.boxes[idx];
        // a media container's surface passes light: shadow rays cross it
        // (shadow_through counts and attenuates the crossings)
        if (ANY && (__float_as_int(b.hi.w) & BOX_CONTAINER))
            return false;
        float tn, tf;
        int sn, sf;
        if (!box_roots(b, o, d, tn, tf, sn, sf))
            return false;
        if (self) {
            if (dot3(box_side_normal((int)skip.y), d) < 0.0f && tf >= tmin && tf < t) { t = tf; aux = sf; return true; }
            return false;
        }
        if (tn > BOX_DEPTH_TOL && tn >= tmin && tn < t) { t = tn; aux = sn; return true; }
        if (tf >= tmin && tf < t) { t = tf; aux = sf; return true; }
        return false;
    }
    if (!FULL)
        return false;   // lean variant: the scene has no tori and no CSG
    if (kind == PK_TORUS) {
        if (NT)
            return false;   // the torus-free variant never gets here (its caller defers tori)
        if (!torus_may_hit(S.tori32 + 4 * (size_t)idx, o, d, t))
            return false;
        double r[4];
        int n = torus_roots(S.tori[idx], make_double3(o.x, o.y, o.z), make_double3(d.x, d.y, d.z), r);
        if (self)
            n = torus_drop_self(r, n);
        bool hit = false;
        for (int k = 0; k < n; k++) {
            float tt = (float)r[k];
            if (tt >= tmin && tt < t) {
                t = tt;
                hit = true;
                if (ANY) break;
            }
        }
        return hit;
    }
    if (kind == PK_CSG)
        return csg_closest<NT>(S, idx, o, d, tmin, t, aux, skip, ref, ANY);
    return false;
}

// ------------------------------------------------------------- traversal --
// Closest hit (ANY = false) or any hit (ANY = true) for every ray in the
// queue.  Stack in shared memory: slot k of thread t at smem[k*blockDim+t].
// MINB: the resident blocks per SM the register allocation must allow
// (1: the compiler's choice; 8: at most 64 registers a thread, more warps
// to hide the node and triangle load latency at the price of spills) --
// one of the autotuner's choices for the lean variant.
// NT: the torus-free full variant (TorusDefer::ovf set): every torus test
// is deferred, and a ray whose pair does not fit the list is handed to a
// second launch of the ordinary full variant (listed in td.ovf, its
// blocked byte 2 meanwhile) instead of being solved here.
// index (optional): the queue slots to trace (slot i traces ray index[i]).
template <bool ANY, bool FULL, int MINB, bool NT = false>
__global__ void __launch_bounds__(128, MINB) k_trace(DeviceScene S, const QRay* __restrict__ q,
                                               const int* __restrict__ q_count, int* __restrict__ work,
                                               QHit* __restrict__ hits, uint8_t* __restrict__ blocked,
                                               int stack_depth, uint32_t* err, unsigned long long* stats,
                                               unsigned long long* wcount, int cap,
                                               const uint2* __restrict__ skips, TorusDefer td,
                                               const int* __restrict__ index)
{
    namespace cg = cooperative_groups;
    extern __shared__ int smem[];
    const int lane = threadIdx.x & 31;
    const int n = min(*q_count, cap);   // never read past the queue buffer
    unsigned long long nblocked = 0;
    unsigned long long c_nodes = 0, c_prims = 0, c_tris = 0, c_rays = 0;
    const bool counting = wcount != nullptr;
    for (;;) {
        int base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        int i = base + lane;
        if (i >= n)
            continue;
        if (index)
            i = index[i];
        QRay r = q[i];
        if (counting) c_rays++;
        float3 o = xyz(r.org), d = xyz(r.dir);
        float tmin = r.org.w;
        float t = r.dir.w;
        float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
        uint32_t best = NO_PRIM, baux = 0;
        float bu = 0.f, bv = 0.f;
        bool done = false;
        bool ovf = false;   // NT: a torus pair did not fit the list
        const uint2 skip = skips ? skips[i] : make_uint2(NO_PRIM, 0u);
        if (FULL && !ANY && td.key)
            td.key[i] = ~0ull;   // no deferred torus root yet
        // infinite objects first (planes: Plane::Intersect, plane.cpp:139-211)
        for (int k = 0; k < S.num_planes; k++) {
            if (((PK_PLANE << PRIM_KIND_SHIFT) | (uint32_t)k) == skip.x)
                continue;
            float4 pl = __ldg(S.planes + k);
            float ndd = pl.x * d.x + pl.y * d.y + pl.z * d.z;
            if (fabsf(ndd) < EPSILON_F)
                continue;
            float tt = -(pl.x * o.x + pl.y * o.y + pl.z * o.z + pl.w) / ndd;
            if (tt >= tmin && tt < t) {
                if (ANY) { done = true; break; }
                t = tt;
                best = (PK_PLANE << PRIM_KIND_SHIFT) | (uint32_t)k;
            }
        }
        int sp = 0;
        int node = S.root;
        int iters = 0;
        while (!done && node != BVH_EMPTY) {
            if (++iters > (1 << 22)) {
                set_error(err, DE_ITERATION_CAP);
                break;
            }
            if (node >= 0) {
                if (counting) c_nodes++;
                if (!node4_step(S.nodes, node, o, inv, tmin, t, smem, sp, stack_depth)) {
                    set_error(err, DE_STACK_OVERFLOW);
                    break;
                }
            } else {
                uint32_t code = ~(uint32_t)node;
                uint32_t first = code >> 3;
                uint32_t count = (code & 7u) + 1u;
                for (uint32_t k = 0; k < count; k++) {
                    uint32_t ref = __ldg(S.prim_refs + first + k);
                    if (counting) { c_prims++; c_tris += (ref >> PRIM_KIND_SHIFT) == PK_TRIANGLE; }
                    if (FULL && (NT || td.cand) && (ref >> PRIM_KIND_SHIFT) == PK_TORUS) {
                        const uint32_t idx = ref & PRIM_INDEX_MASK;
                        if (!torus_may_hit(S.tori32 + 4 * (size_t)idx, o, d, t))
                            continue;
                        if (td.cand) {
                            // one slot per lane that got here, one atomic per group
                            cg::coalesced_group g = cg::coalesced_threads();
                            int slot = 0;
                            if (g.thread_rank() == 0)
                                slot = atomicAdd(td.count, (int)g.size());
                            slot = g.shfl(slot, 0) + (int)g.thread_rank();
                            if (slot < td.cap) {
                                td.cand[slot] = make_uint2((uint32_t)i | (ref == skip.x ? 0x80000000u : 0u), idx);
                                continue;
                            }
                        }
                        if (NT) {   // the list is full: the second launch traces this ray
                            ovf = done = true;
                            break;
                        }
                        // the list is full: solved here
                    }
                    uint32_t aux = 0;
                    if (prim_test<ANY, FULL, NT>(S, ref, o, d, tmin, t, bu, bv, aux, skip)) {
                        best = ref;
                        baux = aux;
                        if (ANY) { done = true; break; }
                    }
                }
                if (done)
                    break;
                node = sp > 0 ? smem[(--sp) * blockDim.x + threadIdx.x] : BVH_EMPTY;
            }
        }
        if (NT && ovf) {
            const int k = atomicAdd(td.ovf_count, 1);
            if (k < td.ovf_cap)
                td.ovf[k] = i;
            else
                set_error(err, DE_QUEUE_OVERFLOW);
            if (ANY)
                blocked[i] = 2;   // k_torus_solve leaves it alone
        } else if (ANY) {
            blocked[i] = done ? 1 : 0;
            nblocked += done ? 1 : 0;
        } else {
            QHit h;
            h.t = t;
            h.prim = best;
            uint32_t kind = best >> PRIM_KIND_SHIFT;
            h.u = (kind == PK_TRIANGLE) ? bu : __uint_as_float(baux);
            h.v = bv;
            hits[i] = h;
        }
    }
    if (ANY && stats) {
        for (int off = 16; off > 0; off >>= 1)
            nblocked += __shfl_down_sync(0xffffffffu, nblocked, off);
        if (lane == 0 && nblocked)
            atomicAdd(&stats[ST_SHADOW_SUCCEEDED], nblocked);
    }
    if (counting) {
        for (int off = 16; off > 0; off >>= 1) {
            c_nodes += __shfl_down_sync(0xffffffffu, c_nodes, off);
            c_prims += __shfl_down_sync(0xffffffffu, c_prims, off);
            c_tris += __shfl_down_sync(0xffffffffu, c_tris, off);
            c_rays += __shfl_down_sync(0xffffffffu, c_rays, off);
        }
        if (lane == 0) {
            atomicAdd(&wcount[0], c_nodes);
            atomicAdd(&wcount[1], c_prims);
            atomicAdd(&wcount[2], c_tris);
            atomicAdd(&wcount[3], c_rays);
        }
    }
}

// The deferred torus tests of one traversal launch, one pair per thread
// (TorusDefer): Torus::Intersect's roots in FP64 (torus_roots), the ray's
// own origin root dropped, the nearest root in [tmin, tmax) -- tmax the
// ray's nearest other hit so far -- kept per ray with a 64-bit atomicMin on
// (depth bits, prim); any-hit rays with a root in range are blocked (and
// counted once per ray).
template <bool ANY>
__global__ void __launch_bounds__(128) k_torus_solve(DeviceScene S, const QRay* __restrict__ q, TorusDefer td,
                                                     const QHit* __restrict__ hits, uint8_t* __restrict__ blocked,
                                                     unsigned long long* stats)
{
    const int n = min(*td.count, td.cap);
    unsigned long long nblocked = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const uint2 e = td.cand[c];
        const int ray = (int)(e.x & 0x7fffffffu);
        const bool self = (e.x >> 31) != 0;
        if (ANY && *(volatile const uint8_t*)(blocked + ray))
            continue;   // blocked already
        const QRay r = q[ray];
        float tmax = r.dir.w;
        if (!ANY)
            tmax = fminf(hits[ray].t, __uint_as_float((uint32_t)(td.key[ray] >> 32)));
        double rt[4];
        int nr = torus_roots(S.tori[e.y], make_double3(r.org.x, r.org.y, r.org.z),
                             make_double3(r.dir.x, r.dir.y, r.dir.z), rt);
        if (self)
            nr = torus_drop_self(rt, nr);
        float best = tmax;
        bool hit = false;
        for (int k = 0; k < nr; k++) {
            const float tt = (float)rt[k];
            if (tt >= r.org.w && tt < best) {
                best = tt;
                hit = true;
            }
        }
        if (!hit)
            continue;
        if (ANY) {
            // the ray's byte within its aligned word (the buffer is padded
            // to whole words)
            const size_t off = (size_t)ray;
            unsigned int* w = reinterpret_cast<unsigned int*>(blocked + (off & ~(size_t)3));
            const unsigned int bit = 1u << (8 * (unsigned)(off & 3));
            const unsigned int old = atomicOr(w, bit);
            if (!(old & (0xffu << (8 * (unsigned)(off & 3)))))
                nblocked++;
        } else {
            const uint32_t ref = (PK_TORUS << PRIM_KIND_SHIFT) | e.y;
            atomicMin(td.key + ray, ((unsigned long long)__float_as_uint(best) << 32) | ref);
        }
    }
    if (ANY) {
        for (int off = 16; off > 0; off >>= 1)
            nblocked += __shfl_down_sync(0xffffffffu, nblocked, off);
        if ((threadIdx.x & 31) == 0 && nblocked)
            atomicAdd(&stats[ST_SHADOW_SUCCEEDED], nblocked);
    }
}

// Deferred torus roots into the closest hits: a root nearer than the ray's
// other hit replaces it (k_trace wrote every ray's key).
__global__ void k_torus_merge(const int* __restrict__ q_count, int cap, const TorusDefer td,
                              QHit* __restrict__ hits)
{
    const int n = min(*q_count, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned long long key = td.key[i];
        if (key == ~0ull)
            continue;
        const float t = __uint_as_float((uint32_t)(key >> 32));
        if (t < hits[i].t) {
            QHit h;
            h.t = t;
            h.prim = (uint32_t)key;
            h.u = 0.0f;
            h.v = 0.0f;
            hits[i] = h;
        }
    }
}

// ---------------------------------------------------------------- shade --
struct SurfaceInfo {
    int32_t object;
    int32_t triangle;   // mesh-local triangle, -1 otherwise
    float3  normal;     // raw normal (unflipped)
    int32_t flags;      // bit0 inverted
};

__device__ __forceinline__ SurfaceInfo surface(const DeviceScene& S, const QHit& h, float3 p)
{
    SurfaceInfo si;
    uint32_t kind = h.prim >> PRIM_KIND_SHIFT;
    uint32_t idx = h.prim & PRIM_INDEX_MASK;
    uint32_t aux = __float_as_uint(h.u);
    si.triangle = -1;
    si.flags = 0;
    if (kind == PK_CSG) {
        DevCsg g = S.csgs[idx];
        DevCsgChild c = S.csg_children[g.first + (aux & 0xffffu)];
        kind = c.kind;
        idx = c.index;
        aux >>= 16;
        si.object = c.object;
        si.flags = c.flags;
        if (kind == PK_SPHERE) {
            float4 s = __ldg(S.spheres + idx);
            si.normal = (p - xyz(s)) * (1.0f / s.w);
        } else if (kind == PK_BOX) {
            si.normal = box_side_normal((int)aux);
        } else if (kind == PK_TORUS) {
            si.normal = torus_normal(S.tori[idx], p);
        } else {
            si.normal = xyz(__ldg(S.planes + idx));
        }
        return si;
    }
    if (kind == PK_SPHERE) {
        float4 s = __ldg(S.spheres + idx);
        si.object = __ldg(S.sphere_obj + idx);
        si.normal = (p - xyz(s)) * (1.0f / s.w);   // Sphere::Normal, sphere.cpp:352
    } else if (kind == PK_PLANE) {
        float4 pl = __ldg(S.planes + idx);
        si.object = __ldg(S.plane_obj + idx);
        si.normal = xyz(pl);
    } else if (kind == PK_BOX) {
        DevBox b = S.boxes[idx];
        si.object = __float_as_int(b.lo.w);
        si.flags = __float_as_int(b.hi.w);
        si.normal = box_side_normal((int)aux);    // Box::Normal, box.cpp:600-650
    } else if (kind == PK_TORUS) {
        const DevTorus& T = S.tori[idx];
        si.object = T.object;
        si.flags = T.flags;
        si.normal = torus_normal(T, p);           // Torus::Normal, torus.cpp:458-489
    } else {
        int g = __ldg(S.tri_global + idx);
        float4 gn = __ldg(S.tri_normal + g);
        si.object = __float_as_int(gn.w);
        si.triangle = __ldg(S.tri_local + g);
        int4 sh = __ldg(S.tri_shade + g);
        if (sh.w & 1) {
            // smooth: barycentric blend of the vertex normals, which equals the
            // Perp/vAxis interpolation of Mesh::Smooth_Mesh_Normal
            // (mesh.cpp:410-436)
            float3 n1 = xyz(__ldg(S.normals + sh.x));
            float3 n2 = xyz(__ldg(S.normals + sh.y));
            float3 n3 = xyz(__ldg(S.normals + sh.z));
            float w0 = 1.0f - h.u - h.v;
            si.normal = normalize3(n1 * w0 + n2 * h.u + n3 * h.v);
        } else {
            si.normal = xyz(gn);
        }
    }
    return si;
}

// ------------------------------------------------------ pattern pigments --
// Solid noise and the patterns of the pattern pigments in FP32, following
// portablenoise.cpp:103-225 (generators 1 and 2), noise.cpp:392-440 (Perlin,
// generator 3) and pattern.cpp (checker :5691, gradient :6386, noise :7858,
// granite :6429) with the reference's start-up tables.
__device__ __forceinline__ float noise_scurve(float t) { return t * t * (3.0f - 2.0f * t); }

__device__ float solid_noise(const DevNoise& N, float3 P)
{
    const float p[3] = {P.x, P.y, P.z};
    int b0[3], b1[3];
    float r0[3], r1[3];
    for (int a = 0; a < 3; a++) {
        // the reference adds ROLLOVER (10^7 + 0.023157213) in FP64; the cell
        // and fraction are taken the same way here without the large offset
        const double t = (double)p[a] + 10000000.023157213;
        const int it = (int)floor(t);
        b0[a] = it & 2047;
        b1[a] = (b0[a] + 1) & 2047;
        r0[a] = (float)(t - it);
        r1[a] = r0[a] - 1.0f;
    }
    const int i = __ldg(N.perm + b0[0]), j = __ldg(N.perm + b1[0]);
    const int b00 = __ldg(N.perm + i + b0[1]), b10 = __ldg(N.perm + j + b0[1]);
    const int b01 = __ldg(N.perm + i + b1[1]), b11 = __ldg(N.perm + j + b1[1]);
    const float sx = noise_scurve(r0[0]), sy = noise_scurve(r0[1]), sz = noise_scurve(r0[2]);
    auto at = [&](int k, float rx, float ry, float rz) {
        const float4 g = __ldg(N.grad + k);
        return g.x * rx + g.y * ry + g.z * rz;
    };
    float u = at(b00 + b0[2], r0[0], r0[1], r0[2]), v = at(b10 + b0[2], r1[0], r0[1], r0[2]);
    float a = u + sx * (v - u);
    u = at(b01 + b0[2], r0[0], r1[1], r0[2]);
    v = at(b11 + b0[2], r1[0], r1[1], r0[2]);
    float b = u + sx * (v - u);
    const float c = a + sy * (b - a);
    u = at(b00 + b1[2], r0[0], r0[1], r1[2]);
    v = at(b10 + b1[2], r1[0], r0[1], r1[2]);
    a = u + sx * (v - u);
    u = at(b01 + b1[2], r0[0], r1[1], r1[2]);
    v = at(b11 + b1[2], r1[0], r1[1], r1[2]);
    b = u + sx * (v - u);
    const float d = a + sy * (b - a);
    return c + sz * (d - c);
}

__device__ float pov_noise(const DevNoise& N, float3 P, int gen)
{
    if (gen == 3) {
        const float sum = 0.5f * (1.59f * solid_noise(N, P) + 0.985f);
        return fminf(fmaxf(sum, 0.0f), 1.0f);
    }
    const float p[3] = {P.x, P.y, P.z};
    int ii[3];
    float f[3], g[3], sc[3], tc[3];
    for (int a = 0; a < 3; a++) {
        // the lattice cell as the reference takes it (x - (1 - EPSILON) in FP64)
        const int tmp = p[a] >= 0.0f ? (int)p[a] : (int)((double)p[a] - (1.0 - 1.0e-10));
        ii[a] = (tmp + 10000) & 0xFFF;
        f[a] = p[a] - (float)tmp;
        g[a] = f[a] - 1.0f;
        sc[a] = noise_scurve(f[a]);
        tc[a] = 1.0f - sc[a];
    }
    auto h2 = [&](int a, int b) { return (int)__ldg(N.hash + ((int)__ldg(N.hash + a) ^ b)); };
    auto incr = [&](int a, int b, float s, float x, float y, float z) {
        const int m = (__ldg(N.hash + (a ^ b)) & 0xFF) * 2;
        return s * (__ldg(N.rtab + m + 1) + __ldg(N.rtab + m + 2) * x + __ldg(N.rtab + m + 4) * y +
                    __ldg(N.rtab + m + 6) * z);
    };
    const float txty = tc[0] * tc[1], sxty = sc[0] * tc[1], txsy = tc[0] * sc[1], sxsy = sc[0] * sc[1];
    const int h00 = h2(ii[0], ii[1]), h10 = h2(ii[0] + 1, ii[1]), h01 = h2(ii[0], ii[1] + 1),
              h11 = h2(ii[0] + 1, ii[1] + 1);
    float sum = incr(h00, ii[2], txty * tc[2], f[0], f[1], f[2]);
    sum += incr(h10, ii[2], sxty * tc[2], g[0], f[1], f[2]);
    sum += incr(h01, ii[2], txsy * tc[2], f[0], g[1], f[2]);
    sum += incr(h11, ii[2], sxsy * tc[2], g[0], g[1], f[2]);
    sum += incr(h00, ii[2] + 1, txty * sc[2], f[0], f[1], g[2]);
    sum += incr(h10, ii[2] + 1, sxty * sc[2], g[0], f[1], g[2]);
    sum += incr(h01, ii[2] + 1, txsy * sc[2], f[0], g[1], g[2]);
    sum += incr(h11, ii[2] + 1, sxsy * sc[2], g[0], g[1], g[2]);
    sum = gen == 2 ? (sum + 1.05242f) * 0.48985582f : sum + 0.5f;
    return fminf(fmaxf(sum, 0.0f), 1.0f);
}

// PortableDNoise (portablenoise.cpp:260-361): three lattice functions per
// corner, the corners in the reference's order.
__device__ float3 pov_dnoise(const DevNoise& N, float3 P)
{
    const float p[3] = {P.x, P.y, P.z};
    int ii[3];
    float f[3], g[3], sc[3], tc[3];
    for (int a = 0; a < 3; a++) {
        const int tmp = p[a] >= 0.0f ? (int)p[a] : (int)((double)p[a] - (1.0 - 1.0e-10));
        ii[a] = (tmp + 10000) & 0xFFF;
        f[a] = p[a] - (float)tmp;
        g[a] = f[a] - 1.0f;
        sc[a] = noise_scurve(f[a]);
        tc[a] = 1.0f - sc[a];
    }
    auto h2 = [&](int a, int b) { return (int)__ldg(N.hash + ((int)__ldg(N.hash + a) ^ b)); };
    const int h00 = h2(ii[0], ii[1]), h10 = h2(ii[0] + 1, ii[1]), h01 = h2(ii[0], ii[1] + 1),
              h11 = h2(ii[0] + 1, ii[1] + 1);
    const float txty = tc[0] * tc[1], sxty = sc[0] * tc[1], txsy = tc[0] * sc[1], sxsy = sc[0] * sc[1];
    const int hc[8] = {h00, h10, h11, h01, h01, h11, h10, h00};
    const float sw[8] = {txty * tc[2], sxty * tc[2], sxsy * tc[2], txsy * tc[2],
                         txsy * sc[2], sxsy * sc[2], sxty * sc[2], txty * sc[2]};
    float3 r = f3(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int zc = k >> 2;
        const int xo = (k == 1 || k == 2 || k == 5 || k == 6), yo = (k == 2 || k == 3 || k == 4 || k == 5);
        int m = (__ldg(N.hash + (hc[k] ^ (ii[2] + zc))) & 0xFF) * 2;
        const float x = xo ? g[0] : f[0], y = yo ? g[1] : f[1], z = zc ? g[2] : f[2];
        float v[3];
        for (int c = 0; c < 3; c++, m += 8)
            v[c] = sw[k] * (__ldg(N.rtab + m + 1) + __ldg(N.rtab + m + 2) * x + __ldg(N.rtab + m + 4) * y +
                            __ldg(N.rtab + m + 6) * z);
        r = f3(r.x + v[0], r.y + v[1], r.z + v[2]);
    }
    return r;
}

// Turbulence and DTurbulence (noise.cpp:522-630).
__device__ float pov_turbulence(const DevNoise& N, float3 P, const DevPattern& pt, int gen)
{
    float value = gen == 1 ? pov_noise(N, P, 1) : fminf(fmaxf(2.0f * pov_noise(N, P, gen) - 0.5f, 0.0f), 1.0f);
    const int oct = pt.kind2.x;
    float l = pt.wave.w, o = pt.turb.w;
    for (int i = 2; i <= oct; i++) {
        const float3 q = P * l;
        value += gen == 1 ? o * pov_noise(N, q, 1) : o * (2.0f * pov_noise(N, q, gen) - 0.5f);
        if (i < oct) {
            l *= pt.wave.w;
            o *= pt.turb.w;
        }
    }
    return value;
}

__device__ float3 pov_dturbulence(const DevNoise& N, float3 P, const DevPattern& pt)
{
    float3 r = pov_dnoise(N, P);
    const int oct = pt.kind2.x;
    float l = pt.wave.w, o = pt.turb.w;
    for (int i = 2; i <= oct; i++) {
        r = r + pov_dnoise(N, P * l) * o;
        if (i < oct) {
            l *= pt.wave.w;
            o *= pt.turb.w;
        }
    }
    return r;
}

// cycloidal (texture.cpp:98-108) and Triangle_Wave (texture.cpp:138-156).
__device__ __forceinline__ float pat_cycloidal(float v)
{
    const float twopi = 6.2831853071795864769f;
    return v >= 0.0f ? sinf((v - floorf(v)) * twopi) : -sinf((-(v + floorf(-v))) * twopi);
}

__device__ __forceinline__ float pat_triangle(float v)
{
    const float off = v >= 0.0f ? v - floorf(v) : v + 1.0f + floorf(fabsf(v));
    return off >= 0.5f ? 2.0f * (1.0f - off) : 2.0f * off;
}

// Warp_EPoint (warp.cpp:103-122): the pattern's inverse TRANSFORM, then the
// classic turbulence (warp.cpp:553-558).
__device__ float3 pattern_warp(const DeviceScene& S, const DevPattern& pt, float3 P)
{
    float3 T;
    {
        const float4 c0 = pt.col[0], c1 = pt.col[1], c2 = pt.col[2];
        T = f3(P.x * c0.x + P.y * c0.y + P.z * c0.z + c0.w, P.x * c1.x + P.y * c1.y + P.z * c1.z + c1.w,
               P.x * c2.x + P.y * c2.y + P.z * c2.z + c2.w);
    }
    // the classic turbulence warp after the transform (warp.cpp:553-558)
    if (pt.kind2.y) {
        const float3 d = pov_dturbulence(S.noise, T, pt);
        T = f3(T.x + d.x * pt.turb.x, T.y + d.y * pt.turb.y, T.z + d.z * pt.turb.z);
    }
    return T;
}

// Evaluate_TPat of a warped point T: the pattern's value with its frequency,
// phase and wave (ContinuousPattern::Evaluate, pattern.cpp:354-390).
// Hash3d (texture.h:75-76) over the noise hash table: an index below 4096.
__device__ __forceinline__ int hash3d(const DevNoise& N, int a, int b, int c)
{
    const int h = __ldg(N.hash + (a & 0xfff));
    return __ldg(N.hash + (__ldg(N.hash + (h ^ (b & 0xfff))) ^ (c & 0xfff)));
}

// a coordinate's place within its brick or mortar period: the fraction
// after (int) truncation, lifted into [0, 1)
__device__ __forceinline__ float brick_frac(float v)
{
    v -= (float)(int)v;
    return v < 0.0f ? v + 1.0f : v;
}

// BrickPattern::Evaluate (pattern.cpp:5495-5623): 0 in the mortar, 1 in a
// brick; courses offset by half a brick.
__device__ __forceinline__ float brick_value(const DevPattern& pt, float3 T)
{
    const float mortar = pt.brick.w, fudge = 1.0e-10f + mortar;
    const float x = T.x + fudge, y = T.y + fudge, z = T.z + fudge;
    const float bw = pt.brick.x, bh = pt.brick.y, bd = pt.brick.z;
    if (brick_frac(y / bh) <= mortar / bh)
        return 0.0f;
    const float by = brick_frac((y / bh) * 0.5f);
    if (by <= 0.5f ? (brick_frac(x / bw) <= mortar / bw || brick_frac(z / bd + 0.5f) <= mortar / bd)
                   : (brick_frac(x / bw + 0.5f) <= mortar / bw || brick_frac(z / bd) <= mortar / bd))
        return 0.0f;
    return 1.0f;
}

// QuiltedPattern::EvaluateRaw with quilt_cubic (pattern.cpp:8067-8083,
// 8949-8968); FLOOR as texture.h:73 has it (one less at negative integers).
__device__ __forceinline__ float quilted_value(const DevPattern& pt, float3 T)
{
    auto qfloor = [](float x) { return x >= 0.0f ? floorf(x) : (0.0f - floorf(0.0f - x) - 1.0f); };
    float3 v = f3(T.x - qfloor(T.x) - 0.5f, T.y - qfloor(T.y) - 0.5f, T.z - qfloor(T.z) - 0.5f);
    const float t = sqrtf(dot3(v, v)), it = 1.0f - t;
    const float c = (t * t * t + 3.0f * t * it * it * pt.crackle2.y + 3.0f * t * t * it * pt.crackle2.z) * 1.154700538f;
    v = v * c;
    return (fabsf(v.x) + fabsf(v.y) + fabsf(v.z)) / 3.0f;
}

__device__ __forceinline__ float crackle_dist(float m, float3 dv)
{
    if (m == 2.0f)
        return dot3(dv, dv);
    if (m == 1.0f)
        return fabsf(dv.x) + fabsf(dv.y) + fabsf(dv.z);
    return powf(fabsf(dv.x), m) + powf(fabsf(dv.y), m) + powf(fabsf(dv.z), m);
}

// CracklePattern::EvaluateRaw (pattern.cpp:5760-6010) without repeat: the
// nuclei of the 81 cubes within a "3d knight move" in the order of
// InitialiseCrackleCubeTable (pattern.cpp:9348-9373), each placed by
// IntPickInCube (pattern.cpp:8808-8818); the three smallest distances
// under the metric, kept as the reference keeps them; then the offset and
// the form, or with `solid` the noise at the nearest nucleus.
__device__ __noinline__ float crackle_value(const DeviceScene& S, const DevPattern& pt, float3 T, int gen)
{
    const int fx = (int)floorf(T.x - 1.0e-10f), fy = (int)floorf(T.y - 1.0e-10f), fz = (int)floorf(T.z - 1.0e-10f);
    const float m = pt.crackle.w;
    float m1 = 0.f, m2 = 0.f, m3 = 0.f;
    float3 near = f3(0.f, 0.f, 0.f);
    int i = 0;
    for (int ax = -2; ax <= 2; ax++)
        for (int ay = -2; ay <= 2; ay++)
            for (int az = -2; az <= 2; az++) {
                if ((abs(ax) == 2) + (abs(ay) == 2) + (abs(az) == 2) > 1)
                    continue;
                const int cx = fx + ax, cy = fy + ay, cz = fz + az;
                const int seed = hash3d(S.noise, cx, cy, cz);
                const float3 nu = f3((float)cx + __ldg(S.noise.prand + seed), (float)cy + __ldg(S.noise.prand + seed + 1),
                                     (float)cz + __ldg(S.noise.prand + seed + 2));
                const float sum = crackle_dist(m, nu - T);
                if (i < 3) {   // the first three, sorted as the reference sorts them
                    if (i == 0) {
                        m1 = sum;
                        near = nu;
                    } else if (i == 1) {
                        m2 = sum;
                        if (m2 < m1) { const float t = m1; m1 = m2; m2 = t; near = nu; }
                    } else {
                        m3 = sum;
                        if (m3 < m1) { const float t = m1; m1 = m3; m3 = t; near = nu; }
                        if (m3 < m2) { const float t = m2; m2 = m3; m3 = t; }
                    }
                } else if (sum < m1) {
                    m3 = m2; m2 = m1; m1 = sum; near = nu;
                } else if (sum < m2) {
                    m3 = m2; m2 = sum;
                } else if (sum < m3) {
                    m3 = sum;
                }
                i++;
            }
    const float off = pt.crackle2.x;
    if (off != 0.0f) {
        const float a = m == 2.0f ? off * off : (m == 1.0f ? off : powf(off, m));
        m1 += a; m2 += a; m3 += a;
    }
    float tf;
    if (pt.crackle2.w != 0.0f)
        tf = pov_noise(S.noise, near, gen);
    else if (m == 2.0f)
        tf = pt.crackle.x * sqrtf(m1) + pt.crackle.y * sqrtf(m2) + pt.crackle.z * sqrtf(m3);
    else if (m == 1.0f)
        tf = pt.crackle.x * m1 + pt.crackle.y * m2 + pt.crackle.z * m3;
    else
        tf = pt.crackle.x * powf(m1, 1.0f / m) + pt.crackle.y * powf(m2, 1.0f / m) + pt.crackle.z * powf(m3, 1.0f / m);
    return fmaxf(fminf(tf, 1.0f), 0.0f);
}

__device__ __noinline__ float pattern_value(const DeviceScene& S, const DevPattern& pt, float3 T)
{
    const int kind = pt.kind.x, gen = pt.kind.y;
    float value;
    if (kind == POV_PATTERN_CHECKER) {
        const int c = (int)(floorf(T.x + 1.0e-10f) + floorf(T.y + 1.0e-10f) + floorf(T.z + 1.0e-10f));
        value = (c & 1) ? 1.0f : 0.0f;
    } else if (kind == POV_PATTERN_SQUARE) {       // pattern.cpp:6740-6770
        const int vx = (int)floorf(T.x), vz = (int)floorf(T.z);
        value = (vx & 1) ? ((vz & 1) ? 2.0f : 3.0f) : ((vz & 1) ? 1.0f : 0.0f);
    } else if (kind == POV_PATTERN_CUBIC) {        // pattern.cpp:6699-6714
        const float x = T.x, y = T.y, z = T.z, ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
        value = (x >= 0.f && x >= ay && x >= az)     ? 0.0f
                : (y >= 0.f && y >= ax && y >= az)   ? 1.0f
                : (z >= 0.f && z >= ax && z >= ay)   ? 2.0f
                : (x < 0.f && x <= -ay && x <= -az)  ? 3.0f
                : (y < 0.f && y <= -ax && y <= -az)  ? 4.0f
                                                     : 5.0f;
    } else if (kind == POV_PATTERN_HEXAGON) {      // pattern.cpp:6512-6655
        // block colours of the 6 x 6 grid by zm, two bits each: blocks 0/5
        // and 2/3 of xm whole, 1/4 split on the diagonal (below / above)
        const unsigned even = 0x294u, mid = 0x50Au, below = 0x618u, above = 0x186u;
        const float x = fabsf(T.x);
        const float z = T.z < 0.0f ? 5.196152424f - fabsf(T.z) : T.z;
        float xs = x / 0.5f, zs = z / 0.866025404f;
        xs -= floorf(xs / 6.0f) * 6.0f;
        zs -= floorf(zs / 6.0f) * 6.0f;
        const int xm = (int)floorf(xs) % 6, zm = (int)floorf(zs) % 6;
        unsigned tab = 0u;
        if (xm == 0 || xm == 5) {
            tab = even;
        } else if (xm == 2 || xm == 3) {
            tab = mid;
        } else if (xm == 1 || xm == 4) {
            float xl = xs - (float)xm;
            const float zl = zs - (float)zm;
            if (((xm + zm) % 2) == 1)
                xl = 1.0f - xl;
            if (xl == 0.0f)
                xl = 0.0001f;
            tab = (zl / xl) < 1.0f ? below : above;
        }
        value = (zm >= 0 && zm < 6) ? (float)((tab >> (2 * zm)) & 3u) : 0.0f;
    } else if (kind == POV_PATTERN_BRICK) {        // pattern.cpp:5495-5623
        value = brick_value(pt, T);
    } else if (kind == POV_PATTERN_TRIANGULAR) {   // pattern.cpp:6799-6866
        const float SQ3 = 1.7320508075688772935f, SQ3_2 = 0.86602540378443864676f;
        float xs = T.x - 3.0f * floorf(T.x / 3.0f);
        float zs = T.z - SQ3 * floorf(T.z / SQ3);
        const int a = (int)floorf(xs);
        xs -= (float)a;
        const int b = zs < SQ3_2 ? 0 : 1;
        if (b)
            zs = SQ3 - zs;
        const float k = 1.0f - xs;
        float ans = 1.0f;
        if (xs != 0.0f && k != 0.0f) {
            const int c = (zs / xs < SQ3 ? 1 : 0) + (zs / k < SQ3 ? 2 : 0);
            ans = c == 3 ? 0.0f : (c == 2 ? 1.0f : 3.0f);
        }
        const int mask = (int)ans;
        ans = (mask & 1) ? fmodf(ans + 2.0f * (float)a, 6.0f) : fmodf(6.0f + ans - 2.0f * (float)a, 6.0f);
        value = b ? 5.0f - ans : ans;
    } else {
        if (kind == POV_PATTERN_GRADIENT) {
            value = T.x * pt.gradient.x + T.y * pt.gradient.y + T.z * pt.gradient.z;
            if (value > 1.0f)
                value = fmodf(value, 1.0f);
        } else if (kind == POV_PATTERN_BOZO) {
            value = pov_noise(S.noise, T, gen);
        } else if (kind == POV_PATTERN_GRANITE) {   // six octaves of |noise| (pattern.cpp:6429-6465)
            value = 0.0f;
            float freq = 1.0f;
            for (int i = 0; i < 6; freq *= 2.0f, i++) {
                const float3 t2 = T * (4.0f * freq);
                const float tmp = gen == 1 ? fabsf(0.5f - pov_noise(S.noise, t2, 1))
                                           : fminf(fabsf(1.0f - 2.0f * pov_noise(S.noise, t2, gen)), 0.5f);
                value += tmp / freq;
            }
        } else if (kind == POV_PATTERN_MARBLE) {   // pattern.cpp:7831-7850
            value = T.x + (pt.kind2.y ? pt.turb.x * pov_turbulence(S.noise, T, pt, gen) : 0.0f);
        } else if (kind == POV_PATTERN_WOOD) {     // pattern.cpp:8651-8680
            float px = 0.0f, py = 0.0f;
            if (pt.kind2.y) {
                const float3 wt = pov_dturbulence(S.noise, T, pt);
                px = pat_cycloidal((T.x + wt.x) * pt.turb.x);
                py = pat_cycloidal((T.y + wt.y) * pt.turb.y);
            }
            px += T.x;
            py += T.y;
            value = sqrtf(px * px + py * py);
        } else if (kind == POV_PATTERN_AGATE) {    // pattern.cpp:5396-5418
            const float tv = pt.gradient.w * pov_turbulence(S.noise, T, pt, gen);
            value = 0.5f * (pat_cycloidal(1.3f * tv + 1.1f * T.z) + 1.0f);
            value = value < 0.0f ? 0.0f : powf(fminf(value, 1.0f), 0.77f);
        } else if (kind == POV_PATTERN_RIPPLES || kind == POV_PATTERN_WAVES) {
            // RipplesPattern / WavesPattern::EvaluateRaw (pattern.cpp:8163-8186,
            // 8593-8618): rings about the scene's wave sources
            const bool rip = kind == POV_PATTERN_RIPPLES;
            float sc = 0.0f;
            for (int i = 0; i < POV_NUM_WAVES; i++) {
                const float4 w = __ldg(S.noise.waves + i);
                const float3 d = T - xyz(w);
                float len = sqrtf(dot3(d, d));
                if (len == 0.0f)
                    len = 1.0f;
                sc += rip ? pat_cycloidal(len * pt.wave.x + pt.wave.y)
                          : pat_cycloidal(len * pt.wave.x * w.w + pt.wave.y) / w.w;
            }
            value = rip ? 0.5f * (1.0f + sc / (float)POV_NUM_WAVES) : 0.2f * (2.5f + sc / (float)POV_NUM_WAVES);
        } else if (kind == POV_PATTERN_DENTS) {    // pattern.cpp:6307-6313
            const float nz = pov_noise(S.noise, T, gen);
            value = nz * nz * nz;
        } else if (kind == POV_PATTERN_WRINKLES) { // pattern.cpp:8720-8770
            float lambda = 2.0f, omega = 0.5f;
            value = gen == 1 ? pov_noise(S.noise, T, 1)
                             : fminf(fmaxf(pov_noise(S.noise, T, gen) * 2.0f - 0.5f, 0.0f), 1.0f);
            for (int i = 1; i < 10; i++) {
                const float3 q = T * lambda;
                value += omega * (gen == 1 ? pov_noise(S.noise, q, 1)
                                           : fminf(fmaxf(pov_noise(S.noise, q, gen) * 2.0f - 0.5f, 0.0f), 1.0f));
                lambda *= 2.0f;
                omega *= 0.5f;
            }
            value = value / 2.0f;
        } else if (kind == POV_PATTERN_RADIAL) {   // pattern.cpp:8115-8128
            value = (fabsf(T.x) < 0.001f && fabsf(T.z) < 0.001f)
                        ? 0.25f
                        : 0.25f + (atan2f(T.x, T.z) + 3.14159265358979f) / 6.2831853071795864769f;
        } else if (kind >= POV_PATTERN_PLANAR && kind <= POV_PATTERN_BOXED) {
            // planar, spherical, cylindrical, boxed (pattern.cpp:8024, 8551,
            // 6025, 5454) through CLIP_DENSITY (pattern.cpp:85)
            value = kind == POV_PATTERN_PLANAR      ? fabsf(T.y)
                    : kind == POV_PATTERN_SPHERICAL ? sqrtf(dot3(T, T))
                    : kind == POV_PATTERN_CYLINDRICAL ? sqrtf(T.x * T.x + T.z * T.z)
                                                      : fmaxf(fabsf(T.x), fmaxf(fabsf(T.y), fabsf(T.z)));
            value = value < 0.0f ? 1.0f : (value > 1.0f ? 0.0f : 1.0f - value);
        } else if (kind == POV_PATTERN_ONION) {    // pattern.cpp:7934-7952
            value = fmodf(sqrtf(T.x * T.x + T.y * T.y + T.z * T.z), 1.0f);
        } else if (kind == POV_PATTERN_SPIRAL1 || kind == POV_PATTERN_SPIRAL2) {   // pattern.cpp:8396-8515
            const float turb = pt.kind2.y ? pt.turb.x * pov_turbulence(S.noise, T, pt, gen) : 0.0f;
            const float rad = sqrtf(T.x * T.x + T.y * T.y);
            float phi = 0.0f;   // the angle about the z axis, 0 .. 2 pi
            if (rad != 0.0f)
                phi = T.x < 0.0f ? 4.71238898038468986f - asinf(T.y / rad) : 1.57079632679489662f + asinf(T.y / rad);
            const float arm = T.z + rad + (float)pt.kind2.z * phi / 6.2831853071795864769f + turb;
            value = kind == POV_PATTERN_SPIRAL1 ? arm : pat_triangle(rad) + pat_triangle(arm);
        } else if (kind == POV_PATTERN_CRACKLE) {
            value = crackle_value(S, pt, T, gen);
        } else if (kind == POV_PATTERN_QUILTED) {
            value = quilted_value(pt, T);
        } else if (kind == POV_PATTERN_CELLS) {    // pattern.cpp:5652-5660
            value = fminf(__ldg(S.noise.prand + hash3d(S.noise, (int)floorf(T.x + 1.0e-10f),
                                                     (int)floorf(T.y + 1.0e-10f), (int)floorf(T.z + 1.0e-10f))),
                          1.0f);
        } else {                                   // leopard, pattern.cpp:7179-7194
            const float v = (sinf(T.x) + sinf(T.y) + sinf(T.z)) / 3.0f;
            value = v * v;
        }
        // frequency, phase and wave (ContinuousPattern::Evaluate, pattern.cpp:354-390)
        if (pt.wave.x != 0.0f)
            value = fmodf(value * pt.wave.x + pt.wave.y, 1.00001f);
        if (value < 0.0f)
            value -= floorf(value);
        switch (pt.kind.w) {
        case POV_WAVE_SINE: value = (1.0f + pat_cycloidal(value)) * 0.5f; break;
        case POV_WAVE_TRIANGLE: value = pat_triangle(value); break;
        case POV_WAVE_SCALLOP: value = fabsf(pat_cycloidal(value * 0.5f)); break;
        case POV_WAVE_CUBIC: value = value * value * ((-2.0f * value) + 3.0f); break;
        case POV_WAVE_POLY: value = powf(value, pt.wave.z); break;
        default: break;
        }
    }
    return value;
}

// Compute_Pigment of a pattern pigment at world point P (pigment.cpp:395-475):
// the warped point's value through the colour map's linear blend
// (BlendMap::Search, pattern.cpp:1068-1109).
// ... and the blended entry's filter and transmit in `ft` (the colours'
// w holds the filter, `transmits` the transmit).
__device__ __noinline__ float3 pattern_pigment_ft(const DeviceScene& S, int pi, float3 P, float2& ft)
{
    const DevPattern& pt = S.patterns[pi];
    const float value = pattern_value(S, pt, pattern_warp(S, pt, P));
    const int n = pt.kind.z;
    int ip = 0, in = 0;
    if (value >= pt.values[n - 1]) {
        ip = in = n - 1;
    } else {
        while (in < n - 1 && value > pt.values[in]) {
            ip = in;
            in++;
        }
        if (value == pt.values[in])
            ip = in;
    }
    if (ip == in) {
        ft = make_float2(pt.colours[in].w, pt.transmits[in]);
        return xyz(pt.colours[in]);
    }
    const float wp = (pt.values[in] - value) / (pt.values[in] - pt.values[ip]), wn = 1.0f - wp;
    const float4 a = pt.colours[ip], b = pt.colours[in];
    ft = make_float2(a.w * wp + b.w * wn, pt.transmits[ip] * wp + pt.transmits[in] * wn);
    return f3(a.x * wp + b.x * wn, a.y * wp + b.y * wn, a.z * wp + b.z * wn);
}

__device__ __forceinline__ float3 pattern_pigment(const DeviceScene& S, int pi, float3 P)
{
    float2 ft;
    return pattern_pigment_ft(S, pi, P, ft);
}

// TransColour::Opacity (LegacyOpacity before 3.7) of a colour whose filter
// and transmit come from a colour map.
__device__ __forceinline__ float colour_opacity(const DevMaterial& m, float3 c, float filt, float trm)
{
    return (m.see_through & SEE_LEGACY) ? 1.0f - (filt * fmaxf(c.x, fmaxf(c.y, c.z)) + trm) : 1.0f - filt - trm;
}

// The layer normal of a textured hit (ComputeLightedTexture,
// trace.cpp:812-832): Perturb_Normal (normal.cpp:784-905) of the raw normal
// N at world point P -- into the pattern's space through the forward
// TRANSFORM (Warp_Normal, warp.cpp:563-580), displaced by bumps, dents,
// wrinkles or the four-point slope of a continuous pattern, back through the
// inverse (UnWarp_Normal, warp.cpp:603-620) -- and normalised.
__device__ __noinline__ float3 perturb_normal(const DeviceScene& S, int ni, float3 P, float3 N)
{
    const DevNormal& nm = S.tnormals[ni];
    const DevPattern& pt = S.patterns[nm.kind.x];
    const bool scale = nm.kind.y == 0;
    if (scale)
        N = normalize3(N);
    N = f3(dot3(N, xyz(nm.fwd[0])), dot3(N, xyz(nm.fwd[1])), dot3(N, xyz(nm.fwd[2])));
    if (scale)
        N = normalize3(N);
    const float3 T = pattern_warp(S, pt, P);
    const int kind = pt.kind.x;
    const float amount = nm.params.x;
    if (kind == POV_PATTERN_BUMPS) {            // bumps, normal.cpp:235-246
        N = N + pov_dnoise(S.noise, T) * amount;
    } else if (kind == POV_PATTERN_DENTS) {     // dents, normal.cpp:272-288
        float v = pov_noise(S.noise, T, pt.kind.y);
        v = v * v * v * amount;
        N = N + pov_dnoise(S.noise, T) * v;
    } else if (kind == POV_PATTERN_WRINKLES) {  // wrinkles, normal.cpp:325-346
        float3 r = f3(0.f, 0.f, 0.f);
        float sc = 1.0f;
        for (int i = 0; i < 10; sc *= 2.0f, i++) {
            const float3 d = pov_dnoise(S.noise, T * sc);
            r = r + f3(fabsf(d.x / sc), fabsf(d.y / sc), fabsf(d.z / sc));
        }
        N = N + r * amount;
    } else if (kind == POV_PATTERN_RIPPLES || kind == POV_PATTERN_WAVES) {
        // ripples, waves (normal.cpp:130-155, 180-206)
        const bool rip = kind == POV_PATTERN_RIPPLES;
        for (int i = 0; i < POV_NUM_WAVES; i++) {
            const float4 w = __ldg(S.noise.waves + i);
            const float3 d = T - xyz(w);
            float len = sqrtf(dot3(d, d));
            if (len == 0.0f)
                len = 1.0f;
            const float sc = rip ? pat_cycloidal(len * pt.wave.x + pt.wave.y) * amount
                                 : pat_cycloidal(len * pt.wave.x * w.w + pt.wave.y) * amount / w.w;
            N = N + d * (sc / (len * (float)POV_NUM_WAVES));
        }
    } else {                                    // slope, normal.cpp:880-902
        // the four pyramid directions (normal.cpp:88-91)
        const float3 pyr[4] = {f3(0.942809041f, -0.333333333f, 0.0f), f3(-0.471404521f, -0.333333333f, 0.816496581f),
                               f3(-0.471404521f, -0.333333333f, -0.816496581f), f3(0.0f, 1.0f, 0.0f)};
        const float delta = nm.params.y, a = nm.params.z;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const float v = pattern_value(S, pt, T + pyr[i] * delta);
            N = N + pyr[i] * (v * a);
        }
    }
    if (scale)
        N = normalize3(N);
    // n'_i = n . Inv[i][0..2]; col[j] holds the inverse's column j
    N = xyz(pt.col[0]) * N.x + xyz(pt.col[1]) * N.y + xyz(pt.col[2]) * N.z;
    return normalize3(N);
}

// aux word a secondary ray carries about the surface it starts on
__device__ __forceinline__ uint32_t skip_aux(const QHit& h)
{
    uint32_t kind = h.prim >> PRIM_KIND_SHIFT;
    return (kind == PK_BOX || kind == PK_CSG) ? __float_as_uint(h.u) : 0u;
}

// Mirror direction of d about the layer normal N, with the raw-normal
// fix-ups of a perturbed normal (ComputeReflection, trace.cpp:1272-1299).
__device__ __forceinline__ float3 mirror_dir(float3 d, float3 N, float3 raw)
{
    float n2 = -2.0f * dot3(d, N);
    float3 nd = d + N * n2;
    float rn = dot3(nd, raw);
    if (rn < 0.0f) {
        if (dot3(nd, N) < 0.0f) {   // inside the rear virtual surface
            rn = -2.0f * dot3(d, raw);
            nd = d + raw * rn;
        } else {                    // reflect once more about the raw normal
            nd = nd + raw * (-2.0f * rn);
        }
    }
    return normalize3(nd);
}

// Fade of the light that crossed `depth` inside an interior
// (Trace::ComputeRefraction / ComputeShadowTexture, trace.cpp:1108-1128,
// 1225-1240): exponential for fade_power >= 1000, else
// fade_colour + (1 - fade_colour) / (1 + (depth / fade_distance)^fade_power).
__device__ __forceinline__ float3 interior_fade(float4 I0, float4 I1, float depth)
{
    const float x = depth / I0.y;
    if (I0.z >= 1000.0f)
        return f3(expf(-(1.0f - I1.x) * x), expf(-(1.0f - I1.y) * x), expf(-(1.0f - I1.z) * x));
    const float q = 1.0f / (1.0f + powf(x, I0.z));
    return f3(I1.x + (1.0f - I1.x) * q, I1.y + (1.0f - I1.y) * q, I1.z + (1.0f - I1.z) * q);
}

// ComputeOneWhiteLightRay (trace.cpp:2710-2766) without jitter: the unit
// direction from p towards the light and the distance along it.  A parallel
// beam (a cylinder light, or a light marked parallel) runs against the
// light's direction, its length the projection of the offset to the centre
// on it (the reference's cosine-scaled distance, folded).
__device__ __forceinline__ void light_ray(const DevLight& L, float3 p, float3& ld, float& ldist)
{
    const float3 lv = xyz(L.center) - p;
    if (L.beam.w != 0.0f) {
        ld = f3(-L.dir.x, -L.dir.y, -L.dir.z);
        ldist = dot3(lv, ld);
    } else {
        ldist = sqrtf(dot3(lv, lv));
        ld = lv * (1.0f / ldist);
    }
}

// cubic_spline (lightsource.cpp:497-514).
__device__ __forceinline__ float light_spline(float low, float high, float pos)
{
    if (pos < low)
        return 0.0f;
    if (pos >= high)
        return 1.0f;
    pos = (pos - low) / (high - low);
    return (3.0f - 2.0f * pos) * pos * pos;
}

// Attenuate_Light (lightsource.cpp:544-632) of the light ray from p: a
// spotlight's cone, a cylinder light's beam, then the fade with distance.
__device__ __forceinline__ float attenuate_light(const DevLight& L, float3 p, float3 ld, float ldist)
{
    const int type = (int)L.dir.w;
    const float3 dir = xyz(L.dir);
    float att = 1.0f;
    if (type == LIGHT_SPOT) {
        float ct = dot3(ld, dir);
        if (ldist > 0.0f)
            ct = -ct;
        if (ct <= 0.0f)
            return 0.0f;
        att = powf(ct, L.beam.z);
        if (L.beam.x > 0.0f && ct < L.beam.x)
            att *= light_spline(L.beam.y, L.beam.x, ct);
    } else if (type == LIGHT_CYLINDER) {
        const float3 v1 = p - xyz(L.center);
        const float k = dot3(v1, dir);
        if (k <= 0.0f)
            return 0.0f;
        const float3 off = v1 - dir * k;
        const float len = sqrtf(dot3(off, off));
        if (len >= L.beam.y)
            return 0.0f;
        const float dist = 1.0f - len / L.beam.y;
        att = powf(dist, L.beam.z);
        if (L.beam.x > 0.0f && len > L.beam.x)
            att *= light_spline(0.0f, 1.0f - L.beam.x / L.beam.y, dist);
    }
    if (att > 0.0f && L.fade.y > 0.0f) {
        if (fabsf(L.fade.x) >= EPSILON_F)
            att *= 2.0f / (1.0f + powf(ldist / L.fade.x, L.fade.y));
        else
            att *= powf(ldist, -L.fade.y);
    }
    return att;
}

// ComputeMetallic (trace.cpp:2658-2671): the factor that moves a highlight
// or reflectivity towards the pigment by `metallic`, less towards grazing.
__device__ __forceinline__ float3 metallic_factor(float metallic, float3 pig, float cos_angle)
{
    const float x = fabsf(acosf(fminf(1.0f, fmaxf(-1.0f, cos_angle)))) / 1.57079632679489662f;
    const float F = fminf(1.0f, fmaxf(0.0f, 0.014567225f / ((x - 1.12f) * (x - 1.12f)) - 0.011612903f));
    const float k = metallic * (1.0f - F);
    return f3(1.0f + (pig.x - 1.0f) * k, 1.0f + (pig.y - 1.0f) * k, 1.0f + (pig.z - 1.0f) * k);
}

// Trace::ComputeRelativeIOR (trace.cpp:2595-2625): the ratio of iors a ray
// with interior list `rin` sees at a surface of interior `id`.
__device__ __forceinline__ float relative_ior(const DeviceScene& S, uint64_t rin, int id)
{
    const float ior = S.interiors[2 * id].x;
    const int nr = rin_count(rin);
    if (nr == 0)
        return ior / S.atm_ior;
    if (rin_find(rin, id) >= 0)
        return nr == 1 ? S.atm_ior / ior : S.interiors[2 * rin_get(rin, nr - 1)].x / ior;
    return ior / S.interiors[2 * rin_get(rin, nr - 1)].x;
}

// Trace::FresnelR (trace.cpp:2679-2707): unpolarised Fresnel reflectance.
__device__ __forceinline__ float fresnel_r(float cos_ti, float n)
{
    const float sqrg = n * n + cos_ti * cos_ti - 1.0f;
    if (sqrg <= 0.0f)
        return 1.0f;
    const float g = sqrtf(sqrg);
    const float q1 = (g - cos_ti) / (g + cos_ti);
    const float q2 = (cos_ti * (g + cos_ti) - 1.0f) / (cos_ti * (g - cos_ti) + 1.0f);
    return fminf(1.0f, fmaxf(0.0f, 0.5f * q1 * q1 * (1.0f + q2 * q2)));
}

// One thread per ray of the level queue.  Emits shadow rays (one per lit
// light, slot = ray*num_lights+light) and the secondary rays of the hit:
// the reflection ray, the continued ray through a media container's wall,
// the transmitted / refracted / totally reflected ray of a transparent
// surface, or (a transparent surface that reflects) the transmitted ray
// first and then the reflection ray.
// (128, 4): four resident blocks; without the cap the reflection-beside-
// transparency paths take it to 168 registers and three blocks, and the
// shade stage of the 1080p mesh frame measured 0.478 ms against 0.385 ms
// with the cap
__global__ void __launch_bounds__(128, 4) k_shade(
    DeviceScene S, int level, int max_level, const QRay* __restrict__ q, const int* __restrict__ q_path,
    const QHit* __restrict__ hits, const int* __restrict__ q_count, PathState* __restrict__ paths,
    float4* __restrict__ slot_contrib, QRay* __restrict__ sq, int* __restrict__ sq_slot, int* __restrict__ sq_count,
    uint2* __restrict__ sq_skip, QRay* __restrict__ nq, int* __restrict__ nq_path,
    uint2* __restrict__ nq_skip, int* __restrict__ nq_count, int max_queue,
    int max_shadow, QRay* __restrict__ aq, int* __restrict__ aq_slot, uint2* __restrict__ aq_skip,
    int* __restrict__ aq_count, int max_area, ShadeRad rad, ShadeMedia med, const int* __restrict__ order,
    uint32_t* err, unsigned long long* stats)
{
    const int n = min(*q_count, max_queue);
    const int nl = S.num_lights;
    unsigned long long c_rays = 0, c_refl = 0, c_shadow = 0, c_trans = 0, c_refr = 0, c_tir = 0;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        int i = base + threadIdx.x;
        bool active = i < n;
        unsigned mask = __ballot_sync(0xffffffffu, active);
        if (!active)
            continue;
        if (order)   // the queue binned by material: this thread's item
            i = order[i];
        QRay r = q[i];
        QHit h = hits[i];
        int path = q_path ? q_path[i] : i;
        // the ray's own trace level and medium (scenes with media containers)
        const int rstate = med.q_state ? med.q_state[i] : ray_state(level, -1);
        const int lvl = state_level(rstate);
        const int medium = state_medium(rstate);
        float3 o = xyz(r.org), d = xyz(r.dir);
        PathState ps = paths[path];
        const float4 thr4 = med.q_thr ? med.q_thr[i] : ps.throughput;
        float3 thr = xyz(thr4);
        float weight = thr4.w;
        bool hit = h.prim != NO_PRIM;
        float3 col = f3(0.f, 0.f, 0.f);
        float3 p = o + d * h.t;
        float3 N = f3(0.f, 1.f, 0.f);
        float3 raw = N;        // the raw normal facing the ray; N is the layer normal
        const DevMaterial* m = nullptr;
        int oflags = 0;
        uint2 self = make_uint2(h.prim, skip_aux(h));
        bool container = false;
        float3 pigc = f3(0.f, 0.f, 0.f);   // the hit's pigment colour
        float filt = 0.f, trm = 0.f, opac = 1.f;   // its filter, transmit and opacity
        int hobj = 0;
        if (hit) {
            SurfaceInfo si = surface(S, h, p);
            hobj = si.object;
            ObjectShade os = S.objects[si.object];
            oflags = os.flags;
            container = (oflags & OBJ_CONTAINER) != 0;
            m = S.materials + os.material;
            N = si.normal;
            if (oflags & 1)            // INVERTED_FLAG
                N = N * -1.0f;
            if (dot3(N, d) > 0.0f)     // face the ray (trace.cpp:492-494)
                N = N * -1.0f;
            raw = N;
            if (m->see_through & SEE_PATTERN) {   // filter and transmit from the colour map here
                float2 ft;
                pigc = pattern_pigment_ft(S, m->pattern - 1, p, ft);
                filt = ft.x;
                trm = ft.y;
                opac = colour_opacity(*m, pigc, filt, trm);
            } else {
                pigc = m->pattern ? pattern_pigment(S, m->pattern - 1, p) : xyz(m->pigment);
                filt = m->pigment.w;
                trm = m->transmit;
                opac = m->opacity;
            }
            if (m->normal)
                N = perturb_normal(S, m->normal - 1, p, N);
            float4 em = m->emission;
            // a transparent layer's own light is scaled by its opacity
            // (trace.cpp:877-881,1002-1004)
            const float att = opac;
            col = container ? f3(0.f, 0.f, 0.f) : f3(pigc.x * em.x * att, pigc.y * em.y * att, pigc.z * em.z * att);
        } else {
            col = xyz(S.background);   // ComputeSky, background only
        }
        // radiosity ambient query (ComputeLightedTexture, trace.cpp:896-921):
        // the largest possible contribution (pigment greyscale * Diffuse)
        // must beat the ray's ADC bailout
        // a media container's surface only transmits: ComputeRefraction with
        // equal iors traces the continued ray (trace.cpp:1343-1400)
        const bool shaded = hit && !container;
        bool rq_emit = false;
        float rq_maxc = 0.f;
        if (shaded && rad.rq) {
            float3 pg = pigc;
            rq_maxc = (0.297f * pg.x + 0.589f * pg.y + 0.114f * pg.z) * m->diffuse_raw;
            rq_emit = rq_maxc > rad.adc;
        }
        int rqs = rad.rq ? warp_reserve(rad.rq_count, rq_emit, mask) : 0;
        if (rq_emit) {
            if (rqs < rad.rq_cap) {
                RadQuery qq;
                float3 pg = pigc;
                qq.p = make_float4(p.x, p.y, p.z, weight * rq_maxc);
                // the cache and the gather see the raw normal (ComputeAmbient
                // with radiosity's normal setting off, radiosity.cpp:393)
                qq.n = make_float4(raw.x, raw.y, raw.z, 0.f);
                float dr = m->diffuse_raw;
                qq.factor = make_float4(pg.x * dr * thr.x, pg.y * dr * thr.y, pg.z * dr * thr.z, 0.f);
                qq.path = path;
                qq.prim = self.x;
                qq.aux = self.y;
                qq.pad = 0;
                rad.rq[rqs] = qq;
            } else {
                set_error(err, DE_QUEUE_OVERFLOW);
            }
        }
        // per-light terms (ComputeOneDiffuseLight, trace.cpp:1637-1729), for
        // a finish with a diffuse, back-diffuse, specular or phong term
        // (trace.cpp:1017-1021)
        const bool lights_on = shaded && (m->diffuse != 0.0f || m->diffuse_back != 0.0f || m->specular != 0.0f ||
                                          m->phong != 0.0f);
        for (int l = 0; l < nl; l++) {
            bool emit = false;
            float3 contrib = f3(0.f, 0.f, 0.f);
            float3 ld = f3(0.f, 0.f, 1.f);
            float ldist = 0.f, latt = 1.f;
            bool area = false, fill = false;
            if (lights_on) {
                const DevLight& L = S.lights[l];
                // the radiosity Trace runs with area lights off
                // (GetRadiosityQualityFlags, radiosity.cpp:148-161)
                area = L.center.w != 0.0f && !rad.gather;   // POV_LIGHT_AREA
                fill = L.dir.w == (float)LIGHT_SHADOWLESS;
                light_ray(L, p, ld, ldist);
                latt = attenuate_light(L, p, ld, ldist);
                float cs = dot3(N, ld);
                // a light behind the surface lights it through diffuse_back,
                // without highlights (trace.cpp:1652-1662,1714)
                const bool back = !(oflags & 16) && cs < EPSILON_F;
                bool lit = !back || m->diffuse_back != 0.0f;
                float3 lc = xyz(L.colour) * latt;
                if (lit && !(fabsf(lc.x) < EPSILON_F && fabsf(lc.y) < EPSILON_F && fabsf(lc.z) < EPSILON_F)) {
                    emit = true;
                    float3 pig = pigc;
                    const float dif = back ? m->diffuse_back : m->diffuse;
                    if (dif > 0.0f) {   // ComputeDiffuseColour, trace.cpp:2441-2484
                        float inten = m->brilliance != 1.0f ? powf(fabsf(cs), m->brilliance) : fabsf(cs);
                        inten *= dif * opac;
                        contrib = contrib + pig * lc * inten;
                    }
                    // no highlights for radiosity rays, shadowless lights or
                    // the back side (trace.cpp:1714)
                    if (m->phong > 0.0f && !rad.gather && !fill && !back) {     // ComputePhongColour, trace.cpp:2520-2558
                        float c2 = -2.0f * dot3(d, N);
                        float3 rd = d + N * c2;
                        float ci = dot3(rd, ld);
                        if (ci > 0.0f && (m->phong_size < 60.0f || ci > 0.0008f)) {
                            float3 h = lc * (m->phong * powf(ci, m->phong_size));
                            if (m->metallic != 0.0f)
                                h = h * metallic_factor(m->metallic, pig, dot3(N, ld));
                            contrib = contrib + h;
                        }
                    }
                    if (m->specular > 0.0f && !rad.gather && !fill && !back) {  // ComputeSpecularColour, trace.cpp:2560-2593
                        float3 half = (ld - d) * 0.5f;
                        float hl = sqrtf(dot3(half, half));
                        if (hl > 0.0f) {
                            float ci = dot3(half, N) / hl;
                            if (ci > 0.0f) {
                                float3 h = lc * (m->specular * powf(ci, m->roughness));
                                if (m->metallic != 0.0f)
                                    h = h * metallic_factor(m->metallic, pig, dot3(half, ld) / hl);
                                contrib = contrib + h;
                            }
                        }
                    }
                }
            }
            // point lights: one shadow ray; area lights: one item for the
            // subdivision kernel (TraceAreaLightShadowRay), which gets the
            // light's attenuation in dir.w; shadowless lights: none
            // (trace.cpp:1664)
            int aslot = warp_reserve(aq_count, emit && area && !fill, mask);
            if (emit && area && !fill) {
                if (aslot < max_area) {
                    QRay ar;
                    ar.org = make_float4(p.x, p.y, p.z, __uint_as_float(__float_as_uint(SMALL_TOLERANCE_F) + 1u));
                    ar.dir = make_float4(0.f, 0.f, 0.f, latt);
                    aq[aslot] = ar;
                    aq_slot[aslot] = i * nl + l;
                    aq_skip[aslot] = self;
                } else {
                    set_error(err, DE_QUEUE_OVERFLOW);
                }
            }
            int slot = warp_reserve(sq_count, emit && !area && !fill, mask);
            if (emit && !area && !fill) {
                if (slot < max_shadow) {
                    QRay sr;
                    sr.org = make_float4(p.x, p.y, p.z, __uint_as_float(__float_as_uint(SMALL_TOLERANCE_F) + 1u));
                    sr.dir = make_float4(ld.x, ld.y, ld.z, ldist - SHADOW_TOLERANCE_F);
                    sq[slot] = sr;
                    sq_slot[slot] = i * nl + l;
                    sq_skip[slot] = self;
                    if (med.sq_medium)
                        med.sq_medium[slot] = medium;
                    if (med.sq_rin)
                        med.sq_rin[slot] = med.q_rin[i];
                } else {
                    set_error(err, DE_QUEUE_OVERFLOW);
                }
                c_shadow++;
            }
            slot_contrib[(size_t)i * nl + l] =
                make_float4(contrib.x * thr.x, contrib.y * thr.y, contrib.z * thr.z, emit ? 1.0f : 0.0f);
        }
        // reflectivity (ComputeReflectivity, trace.cpp:2627-2656): by the
        // falloff, or by ComputeFresnel at the ray's relative ior; the
        // reflection ray itself is decided after the transmitted one
        float3 reflec = f3(0.f, 0.f, 0.f);
        float rweight = 0.f;
        if (shaded && (m->reflect_flags & REFL_ANY) && !rad.gather) {
            float cos_inc = -dot3(d, N);
            float3 rmax = xyz(m->reflect), rmin = xyz(m->reflect_min);
            if ((m->reflect_flags & REFL_FRESNEL) && med.q_rin) {
                const float f = fresnel_r(cos_inc, relative_ior(S, med.q_rin[i], S.obj_interior[hobj] & 0xffff));
                reflec = rmax * f + rmin * (1.0f - f);
                rweight = weight * fmaxf(reflec.x, fmaxf(reflec.y, reflec.z));
            } else {
                float falloff = m->reflect.w;
                float frac = fabsf(falloff - 1.0f) > EPSILON_F ? powf(1.0f - cos_inc, falloff) : 1.0f - cos_inc;
                if (fabsf(frac) < EPSILON_F) reflec = rmin;
                else if (fabsf(frac - 1.0f) < EPSILON_F) reflec = rmax;
                else reflec = rmax * frac + rmin * (1.0f - frac);
                rweight = weight * m->reflect_min.w;
            }
            if (m->reflect_metallic != 0.0f)   // ComputeMetallic on the reflectivity (trace.cpp:870)
                reflec = reflec * metallic_factor(m->reflect_metallic, pigc, cos_inc);
        }
        float3 nd = f3(0.f, 0.f, 1.f);   // the transmitted ray's direction
        // transmitted ray through a container wall: counted like any traced
        // ray, at the parent's trace level (TraceRay with continuedRay,
        // trace.cpp:155-160), entering or leaving the container's interior
        bool cont = false;
        int cont_medium = -1;
        if (container) {
            c_rays++;
            c_trans++;
            cont = lvl + 1 < max_level;
            const int c = (oflags >> 16) & 0xff;
            cont_medium = medium == c ? -1 : c;
        }
        // transparent surface (ComputeLightedTexture's transmitted
        // component, trace.cpp:1063-1142, and ComputeRefraction,
        // trace.cpp:1323-1486): the filter colour TransmittedColour =
        // pigment * filter + transmit and its greyscale; above the ADC
        // bailout one ray at weight * max|filter| goes on with the ray's
        // interior list changed as the reference changes it -- the continued
        // ray at the same trace level when the iors are equal, else the
        // refracted ray (Heckbert) or, on total internal reflection, the
        // mirror ray with the unchanged list.  Its light reaches the path
        // through Old_Refract, the fade of the interior it leaves and,
        // except after total internal reflection, the filter colour.
        bool tr = false;
        uint64_t trin = 0;
        int tstate = 0;
        float4 tthr = make_float4(0.f, 0.f, 0.f, 0.f);
        bool tir = false;
        if (shaded && m->see_through && med.q_rin) {
            float3 fil = f3(pigc.x * filt + trm, pigc.y * filt + trm, pigc.z * filt + trm);
            if (m->reflect_flags & REFL_CONSERVE)   // the filter loses what is reflected (trace.cpp:1070-1075)
                fil = fil * f3(fminf(1.0f, 1.0f - reflec.x), fminf(1.0f, 1.0f - reflec.y),
                               fminf(1.0f, 1.0f - reflec.z));
            const float trans = fminf(1.0f, fabsf(0.297f * fil.x + 0.589f * fil.y + 0.114f * fil.z));
            if (trans > rad.adc) {
                const float w1 = fmaxf(fabsf(fil.x), fmaxf(fabsf(fil.y), fabsf(fil.z)));
                const int oid = S.obj_interior[hobj] & 0xffff;
                const float4 I0 = S.interiors[2 * oid], I1 = S.interiors[2 * oid + 1];
                const uint64_t rin = med.q_rin[i];
                const int nr = rin_count(rin);
                const int at = rin_find(rin, oid);
                uint64_t nrin = rin;
                float ior;
                if (nr == 0) {                          // entering from the atmosphere
                    rin_append(nrin, oid);
                    ior = S.atm_ior / I0.x;
                } else if (at == nr - 1) {              // leaving the innermost interior
                    nrin = rin_remove(rin, at);
                    ior = nr == 1 ? I0.x / S.atm_ior : I0.x / S.interiors[2 * rin_get(rin, nr - 2)].x;
                } else if (at >= 0) {                   // leaving an overlap
                    nrin = rin_remove(rin, at);
                    ior = 1.0f;
                } else {                                // entering within another
                    if (!rin_append(nrin, oid))
                        set_error(err, DE_INTERIORS);
                    ior = S.interiors[2 * rin_get(rin, nr - 1)].x / I0.x;
                }
                float3 ac = f3(I0.w, I0.w, I0.w);   // Old_Refract
                if (at >= 0 && fabsf(I0.y) > EPSILON_F)
                    ac = ac * interior_fade(I0, I1, h.t);
                float3 tfac = ac * fil;
                c_rays++;   // the TraceRay call is counted even when it bails
                if (fabsf(ior - 1.0f) < EPSILON_F) {
                    c_trans++;                          // Transmitted_Rays_Traced
                    nd = d;
                    tstate = ray_state(lvl, -1);
                    trin = nrin;
                } else {
                    float nn = dot3(d, N);
                    float3 ln = N;
                    if (nn <= 0.0f)
                        nn = -nn;
                    else
                        ln = N * -1.0f;
                    float tt = 1.0f + ior * ior * (nn * nn - 1.0f);
                    if (tt < 0.0f) {
                        tir = true;
                        c_tir++;                        // Internal_Reflected_Rays_Traced
                        c_refl++;
                        nd = mirror_dir(d, N, raw);
                        trin = rin;
                        tfac = ac;
                    } else {
                        c_refr++;                       // Refracted_Rays_Traced
                        tt = ior * nn - sqrtf(tt);
                        nd = normalize3(d * ior + ln * tt);
                        trin = nrin;
                    }
                    tstate = ray_state(lvl + 1, -1);
                }
                tthr = make_float4(thr.x * tfac.x, thr.y * tfac.y, thr.z * tfac.z, weight * w1);
                tr = (lvl + 1 < max_level) && (weight * w1 >= rad.adc);
            }
        }
        // the reflected component (trace.cpp:1148-1178): after total
        // internal reflection a single layer does not reflect again
        bool refl = false;
        float3 rd = f3(0.f, 0.f, 1.f);
        if (!tir && (reflec.x != 0.0f || reflec.y != 0.0f || reflec.z != 0.0f)) {
            c_refl++;
            c_rays++;   // the TraceRay call is counted even when it bails
            rd = mirror_dir(d, N, raw);
            refl = (lvl + 1 < max_level) && (rweight >= rad.adc);
        }
        const int next_cap = med.nq_cap > 0 ? med.nq_cap : max_queue;
        // the transmitted or continued ray
        const bool spawn_t = cont || tr;
        int ts = warp_reserve(nq_count, spawn_t, mask);
        if (spawn_t) {
            if (ts < next_cap) {
                QRay rr;
                rr.org = make_float4(p.x, p.y, p.z, kMinIsectDepth);
                rr.dir = tr ? make_float4(nd.x, nd.y, nd.z, CUDART_INF_F) : make_float4(d.x, d.y, d.z, CUDART_INF_F);
                nq[ts] = rr;
                nq_path[ts] = path;
                nq_skip[ts] = self;
                if (med.nq_state)
                    med.nq_state[ts] = tr ? tstate : ray_state(lvl, cont_medium);
                if (med.nq_rin)
                    med.nq_rin[ts] = trin;
                const float4 t = tr ? tthr : thr4;
                if (med.nq_thr)
                    med.nq_thr[ts] = t;
                else
                    paths[path].throughput = t;
            } else {
                set_error(err, DE_QUEUE_OVERFLOW);
            }
        }
        // the reflection ray (with the incoming ray's interiors)
        int rs = warp_reserve(nq_count, refl, mask);
        if (refl) {
            if (rs < next_cap) {
                QRay rr;
                rr.org = make_float4(p.x, p.y, p.z, kMinIsectDepth);
                rr.dir = make_float4(rd.x, rd.y, rd.z, CUDART_INF_F);
                nq[rs] = rr;
                nq_path[rs] = path;
                nq_skip[rs] = self;
                if (med.nq_state)
                    med.nq_state[rs] = ray_state(lvl + 1, medium);
                if (med.nq_rin)
                    med.nq_rin[rs] = med.q_rin[i];
                const float4 t = make_float4(thr.x * reflec.x, thr.y * reflec.y, thr.z * reflec.z, rweight);
                if (med.nq_thr)
                    med.nq_thr[rs] = t;
                else
                    paths[path].throughput = t;
            } else {
                set_error(err, DE_QUEUE_OVERFLOW);
            }
        }
        if (med.branching) {   // another ray of the path may add in this pass
            atomicAdd(&paths[path].colour.x, col.x * thr.x);
            atomicAdd(&paths[path].colour.y, col.y * thr.y);
            atomicAdd(&paths[path].colour.z, col.z * thr.z);
        } else {
            float4 c = ps.colour;
            paths[path].colour = make_float4(c.x + col.x * thr.x, c.y + col.y * thr.y, c.z + col.z * thr.z, c.w);
        }
    }
    // per-warp counter reduction
    for (int off = 16; off > 0; off >>= 1) {
        c_rays += __shfl_down_sync(0xffffffffu, c_rays, off);
        c_refl += __shfl_down_sync(0xffffffffu, c_refl, off);
        c_shadow += __shfl_down_sync(0xffffffffu, c_shadow, off);
        c_trans += __shfl_down_sync(0xffffffffu, c_trans, off);
        c_refr += __shfl_down_sync(0xffffffffu, c_refr, off);
        c_tir += __shfl_down_sync(0xffffffffu, c_tir, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c_trans) atomicAdd(&stats[ST_TRANSMITTED], c_trans);
        if (c_refr) atomicAdd(&stats[ST_REFRACTED], c_refr);
        if (c_tir) atomicAdd(&stats[ST_INTERNAL_REFLECTED], c_tir);
        if (c_rays) atomicAdd(&stats[ST_RAYS], c_rays);
        if (c_refl) atomicAdd(&stats[ST_REFLECTED], c_refl);
        if (c_shadow) atomicAdd(&stats[ST_SHADOW_TESTS], c_shadow);
    }
}

// Marks blocked light terms (the any-hit kernel wrote one byte per shadow
// ray) and adds the remaining terms to their paths in light order.
__global__ void k_mark_blocked(const int* __restrict__ sq_slot, const uint8_t* __restrict__ blocked,
                               const int* __restrict__ sq_count, float4* __restrict__ slot_contrib, int cap)
{
    int n = min(*sq_count, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (blocked[i])
            slot_contrib[sq_slot[i]].w = 0.0f;
}

// ------------------------------------------------------- area lights --
// Any-hit query of one ray against the whole scene (the per-ray body of
// k_trace<true, FULL>), stack slot k of thread t at smem[k*blockDim+t].
template <bool FULL>
__device__ __forceinline__ bool occluded(const DeviceScene& S, float3 o, float3 d, float tmin, float tmax, uint2 skip,
                                         int* smem, int stack_depth, uint32_t* err)
{
    for (int k = 0; k < S.num_planes; k++) {
        if (((PK_PLANE << PRIM_KIND_SHIFT) | (uint32_t)k) == skip.x)
            continue;
        float4 pl = __ldg(S.planes + k);
        float ndd = pl.x * d.x + pl.y * d.y + pl.z * d.z;
        if (fabsf(ndd) < EPSILON_F)
            continue;
        float tt = -(pl.x * o.x + pl.y * o.y + pl.z * o.z + pl.w) / ndd;
        if (tt >= tmin && tt < tmax)
            return true;
    }
    float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float t = tmax, bu = 0.f, bv = 0.f;
    int sp = 0, node = S.root, iters = 0;
    while (node != BVH_EMPTY) {
        if (++iters > (1 << 22)) {
            set_error(err, DE_ITERATION_CAP);
            return false;
        }
        if (node >= 0) {
            if (!node4_step(S.nodes, node, o, inv, tmin, t, smem, sp, stack_depth)) {
                set_error(err, DE_STACK_OVERFLOW);
                return false;
            }
        } else {
            uint32_t code = ~(uint32_t)node;
            uint32_t first = code >> 3, count = (code & 7u) + 1u;
            for (uint32_t k = 0; k < count; k++) {
                uint32_t aux = 0;
                if (prim_test<true, FULL>(S, __ldg(S.prim_refs + first + k), o, d, tmin, t, bu, bv, aux, skip))
                    return true;
            }
            node = sp > 0 ? smem[(--sp) * blockDim.x + threadIdx.x] : BVH_EMPTY;
        }
    }
    return false;
}

// Grid point (u, v) of an area light as an offset from its centre
// (TraceAreaLightSubsetShadowRay, trace.cpp:2166-2205; no jitter).
__device__ __forceinline__ float3 area_offset(int4 A, float3 a1, float3 a2, int u, int v)
{
    float ju = (float)u, jv = (float)v;
    if (A.w & 1) {   // circular
        ju = ju / (float)(A.x - 1) - 0.5f + 0.001f;
        jv = jv / (float)(A.y - 1) - 0.5f + 0.001f;
        float sc = fmaxf(fabsf(ju), fabsf(jv)) / sqrtf(ju * ju + jv * jv);
        return a1 * (ju * sc) + a2 * (jv * sc);
    }
    float3 j = f3(0.f, 0.f, 0.f);
    if (A.x > 1)
        j = j + a1 * (ju / (float)(A.x - 1) - 0.5f);
    if (A.y > 1)
        j = j + a2 * (jv / (float)(A.y - 1) - 0.5f);
    return j;
}

// One thread per (shading point, area light): TraceAreaLightShadowRay
// (trace.cpp:2078-2129) and its recursive 4-corner subdivision
// (TraceAreaLightSubsetShadowRay, trace.cpp:2131-2272) for opaque scenes.
// The recursion runs as a depth-first region stack; a region that is not
// subdivided adds 0.25^level times the mean of its corner samples, which is
// the reference's nested averaging written out.  Grid points are traced at
// most once per shading point (lightGrid), their visibility held in two
// 64-bit masks.  Writes the visible fraction of the light to the slot's w.
template <bool FULL>
__global__ void __launch_bounds__(128) k_area_shadow(DeviceScene S, const QRay* __restrict__ aq,
                                                     const int* __restrict__ aq_slot,
                                                     const uint2* __restrict__ aq_skip,
                                                     const int* __restrict__ aq_count, int cap,
                                                     float4* __restrict__ slot_contrib, int stack_depth,
                                                     uint32_t* err, unsigned long long* stats)
{
    extern __shared__ int smem[];
    const int n = min(*aq_count, cap);
    const int nl = S.num_lights;
    unsigned long long c_tests = 0, c_blocked = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        QRay it = aq[i];
        const int slot = aq_slot[i];
        const uint2 skip = aq_skip[i];
        const DevLight& L = S.lights[slot % nl];
        const float3 P = xyz(it.org);
        const float tmin = it.org.w;
        const float3 C = xyz(L.center);
        const int4 A = L.area;
        float3 a1 = xyz(L.axis1), a2 = xyz(L.axis2);
        if (A.w & 2) {   // orient: axes perpendicular to the centre ray, |Axis1| long
            float3 dir = normalize3(C - P);
            float3 tmp = fabsf(fabsf(dir.z) - 1.0f) < 0.01f ? f3(0.f, 1.f, 0.f) : f3(0.f, 0.f, 1.f);
            a1 = normalize3(cross3(dir, tmp));
            a2 = normalize3(cross3(dir, a1));
            a1 = a1 * L.axis1.w;
            a2 = a2 * L.axis1.w;
        }
        const float3 lc = xyz(L.colour) * it.dir.w;   // attenuated by the light's cone and fade
        const bool far_apart = fabsf(lc.x) + fabsf(lc.y) + fabsf(lc.z) > 0.1f;   // ColourDistance of lit vs black
        unsigned long long traced = 0, visible = 0;
        // region: u1 | v1 << 6 | u2 << 12 | v2 << 18 | level << 24
        uint32_t rs[24];
        int rsp = 0;
        rs[rsp++] = (uint32_t)(A.x - 1) << 12 | (uint32_t)(A.y - 1) << 18;
        float frac = 0.0f;
        while (rsp > 0) {
            uint32_t r = rs[--rsp];
            int u1 = r & 63, v1 = (r >> 6) & 63, u2 = (r >> 12) & 63, v2 = (r >> 18) & 63, level = r >> 24;
            int vis[4];
            for (int c = 0; c < 4; c++) {
                int u = (c & 1) ? u2 : u1;
                int v = (c & 2) ? v2 : v1;
                int bit = u * A.y + v;
                if (!((traced >> bit) & 1ull)) {
                    float3 lv = C + area_offset(A, a1, a2, u, v) - P;
                    float depth = sqrtf(dot3(lv, lv));
                    float3 ld = lv * (1.0f / depth);
                    bool blk = occluded<FULL>(S, P, ld, tmin, depth - SHADOW_TOLERANCE_F, skip, smem, stack_depth, err);
                    traced |= 1ull << bit;
                    if (!blk)
                        visible |= 1ull << bit;
                    c_tests++;
                    c_blocked += blk ? 1 : 0;
                }
                vis[c] = (int)((visible >> bit) & 1ull);
            }
            bool differ = vis[0] != vis[1] || vis[1] != vis[3] || vis[3] != vis[2] || vis[2] != vis[0];
            if ((u2 - u1 > 1 || v2 - v1 > 1) && (level < A.z || (differ && far_apart)) && rsp + 4 <= 24) {
                int mu0 = (u1 + u2) >> 1, mu1 = (u1 + u2 + 1) >> 1;   // floor / ceil of the midpoint
                int mv0 = (v1 + v2) >> 1, mv1 = (v1 + v2 + 1) >> 1;
                uint32_t nl6 = (uint32_t)(level + 1) << 24;
                rs[rsp++] = (uint32_t)u1 | (uint32_t)v1 << 6 | (uint32_t)mu0 << 12 | (uint32_t)mv0 << 18 | nl6;
                rs[rsp++] = (uint32_t)mu1 | (uint32_t)v1 << 6 | (uint32_t)u2 << 12 | (uint32_t)mv0 << 18 | nl6;
                rs[rsp++] = (uint32_t)u1 | (uint32_t)mv1 << 6 | (uint32_t)mu0 << 12 | (uint32_t)v2 << 18 | nl6;
                rs[rsp++] = (uint32_t)mu1 | (uint32_t)mv1 << 6 | (uint32_t)u2 << 12 | (uint32_t)v2 << 18 | nl6;
            } else {
                frac += (float)(vis[0] + vis[1] + vis[2] + vis[3]) * 0.25f * exp2f(-2.0f * (float)level);
            }
        }
        slot_contrib[slot].w = frac;
    }
    for (int off = 16; off > 0; off >>= 1) {
        c_tests += __shfl_down_sync(0xffffffffu, c_tests, off);
        c_blocked += __shfl_down_sync(0xffffffffu, c_blocked, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c_tests) atomicAdd(&stats[ST_SHADOW_TESTS], c_tests);
        if (c_blocked) atomicAdd(&stats[ST_SHADOW_SUCCEEDED], c_blocked);
    }
}

// ------------------------------------------------------------- encode --
// IntEncode(g, x, 255) without dithering (encoding.cpp:67-91): the floor of
// the encoded value, raised by one where x passes the midpoint of the two
// neighbouring decoded levels (thr[v], computed by the host in FP32).
struct EncodeTable {
    float thr[255];
};

__device__ __forceinline__ float curve_encode(float x, int curve)
{
    if (curve == POV_GPU_CURVE_BT709)   // colourspace.cpp:211-222
        return x < 0.018f ? x * 4.5f : 1.099f * powf(fmaxf(x, 0.0f), 0.45f) - 0.099f;
    return x <= 0.0031308f ? x * 12.92f : 1.055f * powf(fmaxf(x, 0.0f), 1.0f / 2.4f) - 0.055f;   // sRGB, :181-191
}

__global__ void k_encode_u8(const float4* __restrict__ rgbt, long long n, int curve, EncodeTable T,
                            uint8_t* __restrict__ out)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 c = rgbt[i];
        const float ch[3] = {c.x, c.y, c.z};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            // clip (NaN to 0, as the reference's clip leaves no NaN through)
            const float xe = ch[k] > 0.0f ? fminf(ch[k], 1.0f) : 0.0f;
            int v = (int)floorf(curve_encode(xe, curve) * 255.0f);
            v = v < 0 ? 0 : (v > 255 ? 255 : v);
            if (v < 255 && xe > T.thr[v])
                v++;
            out[3 * i + k] = (uint8_t)v;
        }
    }
}

cudaError_t launch_encode_u8(const float4* rgbt, long long n, int curve, const float* thr, uint8_t* out, int grid,
                             cudaStream_t st)
{
    EncodeTable T;
    for (int v = 0; v < 255; v++)
        T.thr[v] = thr[v];
    k_encode_u8<<<grid, 256, 0, st>>>(rgbt, n, curve, T, out);
    return cudaGetLastError();
}

// a[i] = value for the first min(*count, cap) entries
__global__ void k_fill_int(int* __restrict__ a, const int* __restrict__ count, int cap, int value)
{
    const int n = min(*count, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        a[i] = value;
}

cudaError_t launch_fill_int(int* a, const int* count, int cap, int value, int grid, cudaStream_t st)
{
    k_fill_int<<<grid, 128, 0, st>>>(a, count, cap, value);
    return cudaGetLastError();
}

// ------------------------------------------------------ media containers --
// Shadow ray from P towards a point light at ray distance tmax +
// SHADOW_TOLERANCE, through media containers (Trace::TracePointLightShadowRay,
// trace.cpp:1951-2076, with the media term of ComputeShadowColour,
// trace.cpp:2429-2433, and the interior toggle of ComputeShadowMedia,
// trace.cpp:3064-3066).  The reference takes the nearest intersection
// first; a container wall is a transparent hit -- one test and one success
// -- after which the shadow ray goes on from the wall.  A ray that was
// inside the container has its light attenuated by the constant media of
// the crossed segment, exp(-extinction * length), one media sample
// (media.cpp:366-398).  Walls are found from the containers' shapes, opaque
// blockers by an any-hit test of each segment between walls (the any-hit
// test passes container walls).  Counts the tests, successes and media
// samples; returns true when the light is blocked.
template <bool FULL>
__device__ bool shadow_through(const DeviceScene& S, float3 P, float3 d, float tmin, float tmax, uint2 skip,
                               int medium, bool media_on, float3& atten, int* smem, int stack_depth,
                               uint32_t* err, unsigned long long& tests, unsigned long long& succ,
                               unsigned long long& msamples)
{
    float et[2 * MAX_CONTAINERS];
    int ec[2 * MAX_CONTAINERS];
    int ne = 0;
    for (int c = 0; c < S.num_containers; c++) {
        float tb[2];
        int sn, sf;
        if (S.medias[c].phase.z != 0.0f) {   // a sphere
            if (!sphere_roots(__ldg(S.spheres + S.medias[c].n.w), P, d, tb[0], tb[1]))
                continue;
        } else if (!box_roots(S.boxes[S.medias[c].n.w], P, d, tb[0], tb[1], sn, sf)) {
            continue;
        }
        for (int e = 0; e < 2; e++) {
            float t = tb[e];
            if (!(t > SMALL_TOLERANCE_F && t < tmax))
                continue;
            int k = ne++;
            while (k > 0 && et[k - 1] > t) {   // insertion in distance order
                et[k] = et[k - 1];
                ec[k] = ec[k - 1];
                k--;
            }
            et[k] = t;
            ec[k] = c;
        }
    }
    float seg0 = tmin;    // the current shadow ray's first accepted distance
    float org_t = 0.0f;   // where the current shadow ray starts (P or the last wall)
    int k = 0;
    for (;;) {
        while (k < ne && et[k] <= seg0)   // walls within the new origin's tolerance
            k++;
        tests++;
        const float seg1 = k < ne ? et[k] : tmax;
        if (occluded<FULL>(S, P, d, seg0, seg1, skip, smem, stack_depth, err)) {
            succ++;
            return true;
        }
        if (k >= ne)
            return false;
        succ++;
        if (medium >= 0 && media_on) {
            const float3 ext = xyz(S.medias[medium].extinction);
            const float len = et[k] - org_t;
            msamples++;
            atten = f3(atten.x * expf(-ext.x * len), atten.y * expf(-ext.y * len), atten.z * expf(-ext.z * len));
        }
        medium = medium == ec[k] ? -1 : ec[k];
        org_t = et[k];
        seg0 = et[k] + SMALL_TOLERANCE_F;
        k++;
    }
}

// Shadow rays of the shading kernel in scenes with media containers: each
// ray's blocked byte, and its light term scaled by the media it crossed.
// The shading kernel counted each ray's first test.
template <bool FULL>
__global__ void __launch_bounds__(128) k_shadow_through(DeviceScene S, const QRay* __restrict__ sq,
                                                        const int* __restrict__ sq_slot,
                                                        const uint2* __restrict__ sq_skip,
                                                        const int* __restrict__ sq_medium,
                                                        const int* __restrict__ sq_count, int cap,
                                                        int* __restrict__ work, uint8_t* __restrict__ blocked,
                                                        float4* __restrict__ slot_contrib, int media_on,
                                                        int stack_depth, uint32_t* err, unsigned long long* stats)
{
    extern __shared__ int smem[];
    const int n = min(*sq_count, cap);
    const int lane = threadIdx.x & 31;
    unsigned long long c_tests = 0, c_succ = 0, c_ms = 0;
    for (;;) {   // persistent: each warp claims 32 rays at a time
        int base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const int i = base + lane;
        if (i >= n)
            continue;
        const QRay r = sq[i];
        float3 atten = f3(1.f, 1.f, 1.f);
        unsigned long long t = 0;
        const bool b = shadow_through<FULL>(S, xyz(r.org), xyz(r.dir), r.org.w, r.dir.w, sq_skip[i], sq_medium[i],
                                            media_on != 0, atten, smem, stack_depth, err, t, c_succ, c_ms);
        c_tests += t - 1;
        blocked[i] = b ? 1 : 0;
        if (!b && (atten.x != 1.f || atten.y != 1.f || atten.z != 1.f)) {
            const int slot = sq_slot[i];
            float4 c = slot_contrib[slot];
            slot_contrib[slot] = make_float4(c.x * atten.x, c.y * atten.y, c.z * atten.z, c.w);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        c_tests += __shfl_down_sync(0xffffffffu, c_tests, off);
        c_succ += __shfl_down_sync(0xffffffffu, c_succ, off);
        c_ms += __shfl_down_sync(0xffffffffu, c_ms, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c_tests) atomicAdd(&stats[ST_SHADOW_TESTS], c_tests);
        if (c_succ) atomicAdd(&stats[ST_SHADOW_SUCCEEDED], c_succ);
        if (c_ms) atomicAdd(&stats[ST_MEDIA_SAMPLES], c_ms);
    }
}

// ------------------------------------------------ transparent surfaces --
// Closest hit of one ray in [tmin, tmax) (the per-ray body of
// k_trace<false, FULL>): the primitive, its aux word and depth.
template <bool FULL>
__device__ __forceinline__ bool nearest(const DeviceScene& S, float3 o, float3 d, float tmin, float tmax, uint2 skip,
                                        int* smem, int stack_depth, uint32_t* err, float& t, uint32_t& prim,
                                        uint32_t& paux)
{
    t = tmax;
    prim = NO_PRIM;
    paux = 0;
    for (int k = 0; k < S.num_planes; k++) {
        const uint32_t ref = (PK_PLANE << PRIM_KIND_SHIFT) | (uint32_t)k;
        if (ref == skip.x)
            continue;
        float4 pl = __ldg(S.planes + k);
        float ndd = pl.x * d.x + pl.y * d.y + pl.z * d.z;
        if (fabsf(ndd) < EPSILON_F)
            continue;
        float tt = -(pl.x * o.x + pl.y * o.y + pl.z * o.z + pl.w) / ndd;
        if (tt >= tmin && tt < t) {
            t = tt;
            prim = ref;
        }
    }
    float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float bu = 0.f, bv = 0.f;
    int sp = 0, node = S.root, iters = 0;
    while (node != BVH_EMPTY) {
        if (++iters > (1 << 22)) {
            set_error(err, DE_ITERATION_CAP);
            return false;
        }
        if (node >= 0) {
            if (!node4_step(S.nodes, node, o, inv, tmin, t, smem, sp, stack_depth)) {
                set_error(err, DE_STACK_OVERFLOW);
                return false;
            }
        } else {
            uint32_t code = ~(uint32_t)node;
            uint32_t first = code >> 3, count = (code & 7u) + 1u;
            for (uint32_t k = 0; k < count; k++) {
                uint32_t aux = 0;
                const uint32_t ref = __ldg(S.prim_refs + first + k);
                if (prim_test<false, FULL>(S, ref, o, d, tmin, t, bu, bv, aux, skip)) {
                    prim = ref;
                    paux = aux;
                }
            }
            node = sp > 0 ? smem[(--sp) * blockDim.x + threadIdx.x] : BVH_EMPTY;
        }
    }
    return prim != NO_PRIM;
}

// The flattened object a primitive hit belongs to (the object id of
// surface(), without the normal).
__device__ __forceinline__ int hit_object(const DeviceScene& S, uint32_t prim, uint32_t aux)
{
    const uint32_t kind = prim >> PRIM_KIND_SHIFT, idx = prim & PRIM_INDEX_MASK;
    if (kind == PK_CSG)
        return S.csg_children[S.csgs[idx].first + (aux & 0xffffu)].object;
    if (kind == PK_SPHERE)
        return __ldg(S.sphere_obj + idx);
    if (kind == PK_PLANE)
        return __ldg(S.plane_obj + idx);
    if (kind == PK_BOX)
        return __float_as_int(S.boxes[idx].lo.w);
    if (kind == PK_TORUS)
        return S.tori[idx].object;
    return __float_as_int(__ldg(S.tri_normal + __ldg(S.tri_global + idx)).w);
}

constexpr int MAX_SHADOW_CROSSINGS = 4096;

// Shadow rays of the shading kernel in scenes with transparent surfaces
// (Trace::TracePointLightShadowRay, trace.cpp:1951-2076, with
// ComputeShadowColour / ComputeShadowTexture, trace.cpp:1180-1250,
// 2274-2439): the nearest hit first; an opaque surface clears the light, a
// transparent one filters it by its TransmittedColour and, when the shadow
// ray is inside the surface's interior, that interior's fade over the
// crossed depth; below ADC_Bailout the light is cleared; while light is
// left the shadow ray's own interior list (a copy of its eye ray's) toggles
// the interior (ComputeShadowMedia, trace.cpp:3064-3068).  The ray stops,
// blocked, when no light is left and the object hit (the CSG it belongs
// to) is opaque, else goes on from the hit.  Writes each ray's blocked byte
// and scales its light term by the filtered light; counts every test after
// the first (which the shading kernel counted) and every success.
template <bool FULL>
__global__ void __launch_bounds__(128) k_shadow_filter(DeviceScene S, const QRay* __restrict__ sq,
                                                       const int* __restrict__ sq_slot,
                                                       const uint2* __restrict__ sq_skip,
                                                       const uint64_t* __restrict__ sq_rin,
                                                       const int* __restrict__ sq_count, int cap,
                                                       int* __restrict__ work, uint8_t* __restrict__ blocked,
                                                       float4* __restrict__ slot_contrib, int stack_depth,
                                                       uint32_t* err, unsigned long long* stats)
{
    extern __shared__ int smem[];
    const int n = min(*sq_count, cap);
    const int lane = threadIdx.x & 31;
    const float adc = S.adc_bailout;
    unsigned long long c_tests = 0, c_succ = 0;
    for (;;) {   // persistent: each warp claims 32 rays at a time
        int base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const int i = base + lane;
        if (i >= n)
            continue;
        const QRay r = sq[i];
        float3 o = xyz(r.org);
        const float3 d = xyz(r.dir);
        const float tmin = r.org.w;
        float tmax = r.dir.w;
        uint2 skip = sq_skip[i];
        uint64_t rin = sq_rin[i];
        float3 lc = f3(1.f, 1.f, 1.f);
        bool b = false;
        for (int cross = 0;; cross++) {
            if (cross > 0)
                c_tests++;
            if (cross >= MAX_SHADOW_CROSSINGS) {
                set_error(err, DE_ITERATION_CAP);
                b = true;
                break;
            }
            float t;
            uint32_t prim, aux;
            if (!nearest<FULL>(S, o, d, tmin, tmax, skip, smem, stack_depth, err, t, prim, aux))
                break;
            c_succ++;
            const int obj = hit_object(S, prim, aux);
            const DevMaterial& m = S.materials[S.objects[obj].material];
            const int code = S.obj_interior[obj];
            if (!m.see_through) {
                lc = f3(0.f, 0.f, 0.f);
            } else {
                float w = m.pigment.w, tm = m.transmit;
                float3 pc = xyz(m.pigment);
                if (m.see_through & SEE_PATTERN) {   // the colour map at the crossing
                    float2 ft;
                    pc = pattern_pigment_ft(S, m.pattern - 1, o + d * t, ft);
                    w = ft.x;
                    tm = ft.y;
                }
                float3 fc = f3(pc.x * w + tm, pc.y * w + tm, pc.z * w + tm);
                const int id = code & 0xffff;
                const int at = rin_find(rin, id);
                const float4 I0 = S.interiors[2 * id];
                if (at >= 0 && I0.z > 0.0f && fabsf(I0.y) > EPSILON_F)
                    fc = fc * interior_fade(I0, S.interiors[2 * id + 1], t);
                if (fabsf((fabsf(fc.x) + fabsf(fc.y) + fabsf(fc.z)) / 3.0f) < adc) {
                    lc = f3(0.f, 0.f, 0.f);
                } else {
                    lc = lc * fc;
                    if (!(fabsf(lc.x) < EPSILON_F && fabsf(lc.y) < EPSILON_F && fabsf(lc.z) < EPSILON_F)) {
                        if (at >= 0)
                            rin = rin_remove(rin, at);
                        else if (!rin_append(rin, id))
                            set_error(err, DE_INTERIORS);
                    }
                }
            }
            if (fabsf(lc.x) < EPSILON_F && fabsf(lc.y) < EPSILON_F && fabsf(lc.z) < EPSILON_F && (code >> 16) & 1) {
                b = true;
                break;
            }
            o = o + d * t;
            tmax -= t;
            skip = make_uint2(prim, (prim >> PRIM_KIND_SHIFT) == PK_BOX || (prim >> PRIM_KIND_SHIFT) == PK_CSG
                                        ? aux : 0u);
        }
        blocked[i] = b ? 1 : 0;
        if (!b && (lc.x != 1.f || lc.y != 1.f || lc.z != 1.f)) {
            const int slot = sq_slot[i];
            float4 c = slot_contrib[slot];
            slot_contrib[slot] = make_float4(c.x * lc.x, c.y * lc.y, c.z * lc.z, c.w);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        c_tests += __shfl_down_sync(0xffffffffu, c_tests, off);
        c_succ += __shfl_down_sync(0xffffffffu, c_succ, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c_tests) atomicAdd(&stats[ST_SHADOW_TESTS], c_tests);
        if (c_succ) atomicAdd(&stats[ST_SHADOW_SUCCEEDED], c_succ);
    }
}

// Rays of the level queue that crossed a container's interior up to their
// hit: their queue indices, in queue order.
__global__ void k_media_list(const int* __restrict__ q_state, const QHit* __restrict__ hits,
                             const int* __restrict__ q_count, int cap, int* __restrict__ mlist,
                             int* __restrict__ mcount)
{
    const int n = min(*q_count, cap);
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool in = i < n && state_medium(q_state[i]) >= 0 && hits[i].prim != NO_PRIM;
        const unsigned mask = __ballot_sync(0xffffffffu, i < n);
        if (i >= n)
            continue;
        const int slot = warp_reserve(mcount, in, mask);
        if (in)
            mlist[slot] = i;
    }
}

struct MediaSeg {
    float3 O, D;
    int    medium;
    const DevMedia* md;
};

// One media sample (MediaFunction::ComputeOneMediaSample, media.cpp:935-1038,
// sample method 3, constant density) at fraction f of the interval
// [s0, s0 + ds]: emission plus, where the point lies in the lit span
// [0, lit] of the point lights (ComputeOneMediaLightInterval,
// media.cpp:715-750; lit < 0: an unlit interval), the scattered light of
// every light not in shadow (TestShadow, trace.cpp:3173-3203; isotropic
// phase, ComputeMediaScatteringAttenuation), times ds; the optical depth
// estimate extinction * ds.
// The phase factor of ComputeMediaScatteringAttenuation (media.cpp:1183-
// 1220), alpha = the cosine between the ray towards the light and the
// viewing ray: isotropic 1, Mie hazy, Mie murky, Rayleigh, Henyey-Greenstein.
__device__ __forceinline__ float media_phase(float4 ph, float alpha)
{
    const int type = (int)ph.x;
    if (type == 2)
        return 0.576655375f * (1.0f + 9.0f * powf(0.5f * (1.0f + alpha), 8.0f));
    if (type == 3)
        return 0.495714547f * (1.0f + 50.0f * powf(0.5f * (1.0f + alpha), 32.0f));
    if (type == 4)
        return 0.799372013f * (1.0f + alpha * alpha);
    if (type == 5) {
        const float g = ph.y, g2 = g * g;
        const float b = 1.0f + g2 - 2.0f * g * alpha;
        return (1.0f - g2) / (b * sqrtf(b));
    }
    return 1.0f;
}

template <bool FULL>
__device__ void media_point(const DeviceScene& S, const MediaSeg& g, double s0, double ds, double f, double lit,
                            float3& C, float3& od, int* smem, int stack_depth, uint32_t* err,
                            unsigned long long& tests, unsigned long long& succ, unsigned long long& ms)
{
    const double x = s0 + f * ds;
    const float3 P = g.O + g.D * (float)x;
    ms++;
    float3 em = xyz(g.md->emission);
    if (lit >= 0.0 && x >= 0.0 && x <= lit && g.md->scattering.w != 0.0f) {
        const float3 sc = xyz(g.md->scattering);
        for (int l = 0; l < S.num_lights; l++) {
            const DevLight& L = S.lights[l];
            float3 lc = xyz(L.colour);
            if (fabsf(lc.x) < EPSILON_F && fabsf(lc.y) < EPSILON_F && fabsf(lc.z) < EPSILON_F)
                continue;
            float3 lv = xyz(L.center) - P;
            float ldist = sqrtf(dot3(lv, lv));
            float3 ld = lv * (1.0f / ldist);
            float3 atten = f3(1.f, 1.f, 1.f);
            if (shadow_through<FULL>(S, P, ld, __uint_as_float(__float_as_uint(SMALL_TOLERANCE_F) + 1u),
                                     ldist - SHADOW_TOLERANCE_F, make_uint2(NO_PRIM, 0u), g.medium, true, atten,
                                     smem, stack_depth, err, tests, succ, ms))
                continue;
            const float ph = media_phase(g.md->phase, dot3(ld, g.D));
            em = em + (sc * ph) * (lc * atten);
        }
    }
    const float dsf = (float)ds;
    C = em * dsf;
    od = xyz(g.md->extinction) * dsf;
}

__device__ __forceinline__ float col3_dist(float3 a, float3 b)   // ColourDistance
{
    return fabsf(a.x - b.x) + fabsf(a.y - b.y) + fabsf(a.z - b.z);
}

// Interval layout of one segment (ComputeMediaSampleInterval,
// media.cpp:527-596, and the padding of ComputeMedia, media.cpp:346-352):
// with a light, `intervals` equal intervals of [0, dist]; when rounding
// leaves the last end short of dist, one unlit interval up to dist.
// Without lights, constant media is one unlit interval.
__device__ __forceinline__ int media_intervals(const DevMedia& md, bool lit, double dist, double& delta, int& nuni)
{
    nuni = lit ? max(md.n.x, 1) : 1;
    delta = dist / (double)nuni;
    return nuni + ((lit && delta * (double)nuni < dist) ? 1 : 0);
}

// ------------------------------------------------ media sample wavefront --
// ComputeMediaAdaptiveSampling (media.cpp:432-525) with
// ComputeOneMediaSampleRecursive (media.cpp:1040-1125, jitter 0), run as
// rounds of independent samples: round 0 takes every interval's sub-interval
// ends and midpoints (the recursion always samples its midpoint), round s
// the tree nodes of level s whose parent's half differs by more than the
// threshold.  Every sample lands in a slot of its interval:
//   slots 0 .. sub            the sub-interval ends, d = 0, dd, dd+dd, ...
//   sub+1 + k*T + (node-1)    node (heap order, 1 = midpoint) of sub-interval
//                             k's tree, T = 2^AA_Level - 1 nodes
// and the reduction replays the reference's weighting from the slots.

struct MediaWork {
    const QRay*  q;
    const int*   q_state;
    const QHit*  hits;
    const int*   mlist;       // listed rays (queue indices)
    int          first;       // this chunk's first listed ray
    int          nseg;        // listed rays in this chunk
    int          NI;          // interval slots per ray
    int          SMAX;        // sample slots per interval
    float4*      cbuf;        // [nseg][NI][SMAX]: sample colour, w = stamp when taken
    const int*   list;        // round s >= 1: slots to sample
    const int*   list_count;
    int*         next;        // expansion output
    int*         next_count;
    int          list_cap;
    int          stamp;       // marks the slots taken in this chunk
    float4*      te;          // [listed ray][NI] interval sums
    float4*      od;
};

// One interval of a listed ray: its segment and its place in the segment.
struct MediaInterval {
    MediaSeg g;
    double   s0, ds, lit;
    int      nint, sub, T;
};

__device__ __forceinline__ bool media_interval(const DeviceScene& S, const MediaWork& W, int j, int iv,
                                               MediaInterval& I)
{
    const int i = W.mlist[W.first + j];
    const QRay r = W.q[i];
    I.g.O = xyz(r.org);
    I.g.D = xyz(r.dir);
    I.g.medium = state_medium(W.q_state[i]);
    I.g.md = S.medias + I.g.medium;
    const bool lit = S.num_lights > 0;
    const double dist = (double)W.hits[i].t;
    double delta;
    int nuni;
    I.nint = media_intervals(*I.g.md, lit, dist, delta, nuni);
    if (iv >= I.nint)
        return false;
    I.s0 = delta * (double)iv;
    I.ds = iv < nuni ? delta : dist - delta * (double)nuni;
    I.lit = (lit && iv < nuni) ? dist : -1.0;
    I.sub = I.g.md->n.y;
    I.T = (1 << I.g.md->n.z) - 1;
    return true;
}

// Sub-interval end e at d = dd + dd + ... (the reference's running sum).
__device__ __forceinline__ double media_end(int e, double dd)
{
    double d = 0.0;
    for (int k = 0; k < e; k++)
        d = d + dd;
    return d;
}

// Fraction of the interval of tree node `node` of sub-interval k, and the
// slots holding the colours at its two ends.
__device__ __forceinline__ double media_node(const MediaInterval& I, int k, int node, int& lslot, int& rslot)
{
    const double dd = 1.0 / (double)I.sub;
    double a = media_end(k, dd);
    double b = a + dd;
    lslot = k;
    rslot = k + 1;
    const int base = I.sub + 1 + k * I.T - 1;
    int level = 31 - __clz(node);
    for (int l = level - 1; l >= 0; l--) {
        const int anc = node >> (l + 1);   // the node whose half is taken
        const double mid = 0.5 * (a + b);
        if ((node >> l) & 1) {
            a = mid;
            lslot = base + anc;
        } else {
            b = mid;
            rslot = base + anc;
        }
    }
    return 0.5 * (a + b);
}

__device__ __forceinline__ float4* media_slot(const MediaWork& W, int j, int iv, int slot)
{
    return W.cbuf + ((size_t)j * W.NI + iv) * W.SMAX + slot;
}

// One sample per thread: round 0 (list == nullptr) enumerates every
// interval's ends and midpoints, later rounds take the listed slots.
template <bool FULL>
__global__ void __launch_bounds__(128) k_media_sample(DeviceScene S, MediaWork W, int round0_per_interval,
                                                      int* __restrict__ work, int stack_depth, uint32_t* err,
                                                      unsigned long long* stats)
{
    extern __shared__ int smem[];
    const int n = W.list ? min(*W.list_count, W.list_cap) : W.nseg * W.NI * round0_per_interval;
    const int lane = threadIdx.x & 31;
    unsigned long long c_tests = 0, c_succ = 0, c_ms = 0;
    for (;;) {   // persistent: each warp claims 32 samples at a time
        int base = 0;
        if (lane == 0)
            base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const int it = base + lane;
        if (it >= n)
            continue;
        int j, iv, slot;
        if (W.list) {
            const int code = W.list[it];
            slot = code % W.SMAX;
            iv = (code / W.SMAX) % W.NI;
            j = code / (W.SMAX * W.NI);
        } else {
            j = it / (W.NI * round0_per_interval);
            const int rem = it % (W.NI * round0_per_interval);
            iv = rem / round0_per_interval;
            slot = rem % round0_per_interval;   // re-based below
        }
        MediaInterval I;
        if (!media_interval(S, W, j, iv, I))
            continue;
        double f;
        if (!W.list) {
            if (slot >= 2 * I.sub + 1)
                continue;
            if (slot <= I.sub) {
                f = media_end(slot, 1.0 / (double)I.sub);
            } else {
                const int k = slot - (I.sub + 1);
                int ls, rs;
                f = media_node(I, k, 1, ls, rs);
                slot = I.sub + 1 + k * I.T;
            }
        } else {
            const int t = slot - (I.sub + 1);
            int ls, rs;
            f = media_node(I, t / I.T, t % I.T + 1, ls, rs);
        }
        float3 C, od;
        media_point<FULL>(S, I.g, I.s0, I.ds, f, I.lit, C, od, smem, stack_depth, err, c_tests, c_succ, c_ms);
        *media_slot(W, j, iv, slot) = make_float4(C.x, C.y, C.z, __int_as_float(W.stamp));
    }
    for (int off = 16; off > 0; off >>= 1) {
        c_tests += __shfl_down_sync(0xffffffffu, c_tests, off);
        c_succ += __shfl_down_sync(0xffffffffu, c_succ, off);
        c_ms += __shfl_down_sync(0xffffffffu, c_ms, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c_tests) atomicAdd(&stats[ST_SHADOW_TESTS], c_tests);
        if (c_succ) atomicAdd(&stats[ST_SHADOW_SUCCEEDED], c_succ);
        if (c_ms) atomicAdd(&stats[ST_MEDIA_SAMPLES], c_ms);
    }
}

__device__ __forceinline__ bool media_taken(const float4& c, int stamp) { return __float_as_int(c.w) == stamp; }

__device__ __forceinline__ float3 media_c(const float4& c) { return f3(c.x, c.y, c.z); }

// Round s: one thread per (ray, interval, sub-interval, taken node of level
// s-1 whose depth is above 0); lists each half whose end colours differ by
// more than the threshold (ColourDistance, media.cpp:1072,1100).
__global__ void k_media_expand(DeviceScene S, MediaWork W, int s, int max_sub, uint32_t* err)
{
    const int per = max_sub << (s - 1);
    const long long n = (long long)W.nseg * W.NI * per;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
        const long long it = base + threadIdx.x;
        bool want[2] = {false, false};
        int code[2] = {0, 0};
        if (it < n) {
            const int j = (int)(it / ((long long)W.NI * per));
            const int rem = (int)(it % ((long long)W.NI * per));
            const int iv = rem / per;
            const int k = (rem % per) >> (s - 1);
            const int p = (1 << (s - 1)) + ((rem % per) & ((1 << (s - 1)) - 1));   // parent node, level s-1
            MediaInterval I;
            if (media_interval(S, W, j, iv, I) && k < I.sub && s < I.g.md->n.z) {
                const int pslot = I.sub + 1 + k * I.T + p - 1;
                const float4 cp = *media_slot(W, j, iv, pslot);
                if (media_taken(cp, W.stamp)) {
                    int ls, rs;
                    media_node(I, k, p, ls, rs);
                    const float thr = I.g.md->emission.w;
                    const float3 c1 = media_c(*media_slot(W, j, iv, ls)), c2 = media_c(cp),
                                 c3 = media_c(*media_slot(W, j, iv, rs));
                    const int cbase = ((j * W.NI) + iv) * W.SMAX + I.sub + 1 + k * I.T - 1;
                    want[0] = col3_dist(c1, c2) > thr;
                    code[0] = cbase + 2 * p;
                    want[1] = col3_dist(c2, c3) > thr;
                    code[1] = cbase + 2 * p + 1;
                }
            }
        }
        for (int h = 0; h < 2; h++) {
            const int slot = warp_reserve(W.next_count, want[h], 0xffffffffu);
            if (want[h]) {
                if (slot < W.list_cap)
                    W.next[slot] = code[h];
                else
                    set_error(err, DE_QUEUE_OVERFLOW);
            }
        }
    }
}

// One thread per (ray, interval): the reference's weighting of the taken
// samples, sub-interval by sub-interval (ComputeOneMediaSampleRecursive's
// Result / ODResult, then the attenuation of media.cpp:470-487), leaves
// first; the interval's te and od sums go to the combine step.
__global__ void k_media_reduce(DeviceScene S, MediaWork W)
{
    const long long n = (long long)W.nseg * W.NI;
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < n;
         it += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(it / W.NI), iv = (int)(it % W.NI);
        MediaInterval I;
        float3 te = f3(0.f, 0.f, 0.f), odi = f3(0.f, 0.f, 0.f);
        if (media_interval(S, W, j, iv, I)) {
            const float ddf = (float)(1.0 / (double)I.sub);
            const float3 a = xyz(I.g.md->extinction) * (float)I.ds;   // every sample's optical depth
            const int levels = I.g.md->n.z;
            for (int k = 0; k < I.sub; k++) {
                float3 R[MEDIA_MAX_NODES], O[MEDIA_MAX_NODES];
                const int base = I.sub + 1 + k * I.T - 1;
                for (int node = I.T; node >= 1; node--) {
                    const float4 cn = *media_slot(W, j, iv, base + node);
                    if (!media_taken(cn, W.stamp))
                        continue;
                    int ls, rs;
                    media_node(I, k, node, ls, rs);
                    const float3 C1 = media_c(*media_slot(W, j, iv, ls)), C2 = media_c(cn),
                                 C3 = media_c(*media_slot(W, j, iv, rs));
                    const int level = 31 - __clz(node);
                    float3 r, o;
                    if (levels - 1 - level <= 0) {
                        r = (C1 + C2 + C3) / 3.0f;
                        o = (a + a + a) / 3.0f;
                    } else {
                        const bool lt = media_taken(*media_slot(W, j, iv, base + 2 * node), W.stamp);
                        const bool rt = media_taken(*media_slot(W, j, iv, base + 2 * node + 1), W.stamp);
                        if (lt) {
                            r = R[2 * node - 1] / 2.0f;
                            o = O[2 * node - 1] / 2.0f;
                        } else {
                            r = C1 / 3.0f + C2 / 6.0f;
                            o = a / 3.0f + a / 6.0f;
                        }
                        if (rt) {
                            r = r + R[2 * node] / 2.0f;
                            o = o + O[2 * node] / 2.0f;
                        } else {
                            r = r + (C2 / 6.0f + C3 / 3.0f);
                            o = o + (a / 6.0f + a / 3.0f);
                        }
                    }
                    R[node - 1] = r;
                    O[node - 1] = o;
                }
                float3 r = R[0], o = O[0];
                r = f3(r.x * expf(-odi.x * ddf), r.y * expf(-odi.y * ddf), r.z * expf(-odi.z * ddf));
                if (o.x != 0.0f) r.x *= (1.0f - expf(-o.x * ddf)) / (o.x * ddf);
                if (o.y != 0.0f) r.y *= (1.0f - expf(-o.y * ddf)) / (o.y * ddf);
                if (o.z != 0.0f) r.z *= (1.0f - expf(-o.z * ddf)) / (o.z * ddf);
                te = te + r;
                odi = odi + o;
            }
        }
        W.te[(size_t)(W.first + j) * W.NI + iv] = make_float4(te.x, te.y, te.z, 0.f);
        W.od[(size_t)(W.first + j) * W.NI + iv] = make_float4(odi.x, odi.y, odi.z, 0.f);
    }
}

// One thread per listed ray: the intervals in order (ComputeMediaColour,
// media.cpp:527-545 of the interval sums) give the segment's emission Te and
// transmittance exp(-Od); what the ray's hit adds to its path is seen through
// the media, so the path takes Te at its current throughput and continues
// with throughput * exp(-Od).
__global__ void k_media_combine(const int* __restrict__ q_state, const int* __restrict__ q_path,
                                const QHit* __restrict__ hits, const int* __restrict__ mlist,
                                const int* __restrict__ mcount, int mcap, int NI, const DeviceScene S,
                                const float4* __restrict__ te_in, const float4* __restrict__ od_in,
                                PathState* __restrict__ paths)
{
    const int n = min(*mcount, mcap);
    const bool lit = S.num_lights > 0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int i = mlist[j];
        const DevMedia& md = S.medias[state_medium(q_state[i])];
        double delta;
        int nuni;
        const int nint = media_intervals(md, lit, (double)hits[i].t, delta, nuni);
        const float nrm = (float)(1.0 / (double)md.n.y);
        float3 Te = f3(0.f, 0.f, 0.f), Od = f3(0.f, 0.f, 0.f);
        for (int iv = 0; iv < nint; iv++) {
            const float4 te = te_in[(size_t)j * NI + iv];
            const float4 od = od_in[(size_t)j * NI + iv];
            Te = Te + f3(te.x * nrm * expf(-Od.x), te.y * nrm * expf(-Od.y), te.z * nrm * expf(-Od.z));
            Od = Od + f3(od.x, od.y, od.z) * nrm;
        }
        const int path = q_path ? q_path[i] : i;
        PathState ps = paths[path];
        const float3 thr = xyz(ps.throughput);
        ps.colour = make_float4(ps.colour.x + thr.x * Te.x, ps.colour.y + thr.y * Te.y, ps.colour.z + thr.z * Te.z,
                                ps.colour.w);
        ps.throughput = make_float4(thr.x * expf(-Od.x), thr.y * expf(-Od.y), thr.z * expf(-Od.z), ps.throughput.w);
        paths[path] = ps;
    }
}

__global__ void k_resolve(const int* __restrict__ q_path, const int* __restrict__ q_count, int num_lights,
                          const float4* __restrict__ slot_contrib, PathState* __restrict__ paths, int cap,
                          int branching)
{
    int n = min(*q_count, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int path = q_path[i];
        float4 c = branching ? make_float4(0.f, 0.f, 0.f, 0.f) : paths[path].colour;
        for (int l = 0; l < num_lights; l++) {
            float4 s = slot_contrib[(size_t)i * num_lights + l];
            if (s.w != 0.0f) {   // w: 1 lit point light, area-light fraction, 0 blocked
                c.x += s.x * s.w;
                c.y += s.y * s.w;
                c.z += s.z * s.w;
            }
        }
        if (branching) {   // two rays of one path may share the pass
            atomicAdd(&paths[path].colour.x, c.x);
            atomicAdd(&paths[path].colour.y, c.y);
            atomicAdd(&paths[path].colour.z, c.z);
        } else {
            paths[path].colour = c;
        }
    }
}

// RGBT of sample i to out[slot ? slot[i] : i] (transmit 0: opaque scenes
// and a background without alpha, trace.cpp:2874-2887).
__global__ void k_finalize(const PathState* __restrict__ paths, const int* __restrict__ count, int cap,
                           const int* __restrict__ slot, float4* __restrict__ out)
{
    int n = min(*count, cap);
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float4 c = paths[i].colour;
        out[slot ? slot[i] : i] = make_float4(c.x, c.y, c.z, 0.0f);
    }
}

// FP64 re-solve of the winning primitive for rays given in FP64: the depth
// the reference computes for the same ray (sphere: Sphere::Intersect in
// double; plane: Plane::Intersect; triangle: intersect_mesh_triangle's
// plane distance from the stored FP32 normal and Distance, mesh.cpp:1046-1060;
// box: the slab of the recorded side; torus: its FP64 root as found).
__device__ __forceinline__ double refine_sphere(const double* s, double ox, double oy, double oz, double dx, double dy,
                                                double dz, double t)
{
    double cx = s[0] - ox, cy = s[1] - oy, cz = s[2] - oz;
    double tca = cx * dx + cy * dy + cz * dz;
    double ocs = cx * cx + cy * cy + cz * cz;
    double th = s[3] * s[3] - ocs + tca * tca;
    if (th > 0.0) {
        double hc = sqrt(th);
        double t1 = tca - hc, t2 = tca + hc;
        return fabs(t1 - t) <= fabs(t2 - t) ? t1 : t2;
    }
    return t;
}

__device__ __forceinline__ double refine_box(const double* b, int side, double o[3], double d[3], double t)
{
    int ax = side >> 1;
    double plane = b[(side & 1) ? 3 + ax : ax];
    return d[ax] != 0.0 ? (plane - o[ax]) / d[ax] : t;
}

__global__ void k_refine(DeviceScene S, const double* __restrict__ org, const double* __restrict__ dir,
                         const QHit* __restrict__ hits, double* __restrict__ t64, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    QHit h = hits[i];
    double t = (double)h.t;
    if (h.prim != NO_PRIM) {
        double o[3] = {org[3 * i], org[3 * i + 1], org[3 * i + 2]};
        double d[3] = {dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
        uint32_t kind = h.prim >> PRIM_KIND_SHIFT, idx = h.prim & PRIM_INDEX_MASK;
        uint32_t aux = __float_as_uint(h.u);
        if (kind == PK_CSG) {
            DevCsg g = S.csgs[idx];
            DevCsgChild c = S.csg_children[g.first + (aux & 0xffffu)];
            kind = c.kind;
            idx = c.index;
            aux >>= 16;
        }
        if (kind == PK_SPHERE) {
            t = refine_sphere(S.spheres64 + 4 * idx, o[0], o[1], o[2], d[0], d[1], d[2], t);
        } else if (kind == PK_PLANE) {
            float4 p = S.planes[idx];
            double ndd = p.x * d[0] + p.y * d[1] + p.z * d[2];
            if (ndd != 0.0)
                t = -((p.x * o[0] + p.y * o[1] + p.z * o[2]) + (double)p.w) / ndd;
        } else if (kind == PK_TRIANGLE) {
            int g = S.tri_global[idx];
            float4 nrm = S.tri_normal[g];
            double ndd = nrm.x * d[0] + nrm.y * d[1] + nrm.z * d[2];
            if (ndd != 0.0)
                t = -((double)S.tri_v0[idx].w + (nrm.x * o[0] + nrm.y * o[1] + nrm.z * o[2])) / ndd;
        } else if (kind == PK_BOX) {
            t = refine_box(S.boxes64 + 6 * idx, (int)aux, o, d, t);
        } else if (kind == PK_TORUS) {
            double r[4];
            int k = torus_roots(S.tori[idx], make_double3(o[0], o[1], o[2]), make_double3(d[0], d[1], d[2]), r);
            double best = t;
            for (int j = 0; j < k; j++)
                if (fabs(r[j] - t) < fabs(best - t) || best == t)
                    best = r[j];
            t = best;
        }
    }
    t64[i] = t;
}

// ---------------------------------------------------- adaptive AA (M2) --
// Per pixel, a (2^depth+1)^2 grid of sub-samples (SubdivisionBuffer,
// tracetask.cpp:206-233) in `grid`, a claim bitmask in `mask` (one bit per
// grid point) and a bit per subdivided cell in `subdiv` (cell ids in
// quadtree order: children of c are 4c+1..4c+4 in the order (-,-), (-,+),
// (+,-), (+,+) of SubdivideOnePixel's recursion).

// Copies each pixel's four corner colours from the block corner grid.
__global__ void k_aa_init(const int4* __restrict__ blocks, const int* __restrict__ pix_off,
                          const int* __restrict__ corner_off, int nblocks, const float4* __restrict__ corners,
                          int G, int MW, float4* __restrict__ grid, uint32_t* __restrict__ mask,
                          uint32_t* __restrict__ subdiv, int2* __restrict__ pix_xy, int4* __restrict__ cells,
                          int* __restrict__ ncells, int root_level)
{
    int npix = pix_off[nblocks];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
        *ncells = npix;
    if (i >= npix)
        return;
    int lo = 0, hi = nblocks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pix_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    int4 b = blocks[lo];
    int w = b.z - b.x + 1;
    int local = i - pix_off[lo];
    int lx = local % w, ly = local / w;
    int cw = w + 1;
    const float4* cb = corners + corner_off[lo];
    int S_ = G - 1;
    float4* g = grid + (size_t)i * G * G;
    g[0] = cb[ly * cw + lx];
    g[S_ * G] = cb[(ly + 1) * cw + lx];
    g[S_] = cb[ly * cw + lx + 1];
    g[S_ * G + S_] = cb[(ly + 1) * cw + lx + 1];
    uint32_t* m = mask + (size_t)i * MW;
    for (int k = 0; k < MW; k++)
        m[k] = 0u;
    int corner_bits[4] = {0, S_ * G, S_, S_ * G + S_};
    for (int k = 0; k < 4; k++)
        m[corner_bits[k] >> 5] |= 1u << (corner_bits[k] & 31);
    subdiv[i] = 0u;
    pix_xy[i] = make_int2(b.x + lx, b.y + ly);
    // root cell: pixel i, (bx, by) = (0, 0), step S_, level root_level, id 0
    cells[i] = make_int4(i, 0 | (0 << 8) | (S_ << 16), root_level, 0);
}

__device__ __forceinline__ float aa_enc(float x) { return powf(fmaxf(x, 0.0f), 1.0f / 2.5f); }

__device__ __forceinline__ float aa_dist(float4 a, float4 b)   // ColourDistanceRGBT on AA-gamma colours
{
    return fabsf(aa_enc(a.x) - aa_enc(b.x)) + fabsf(aa_enc(a.y) - aa_enc(b.y)) + fabsf(aa_enc(a.z) - aa_enc(b.z)) +
           fabsf(a.w - b.w);
}

// One thread per active cell: subdivide when level > 0 and any of the six
// corner pairs differs by >= threshold (SubdivideOnePixel's test); claim
// the five new grid points (first claimant traces it, like the
// reference's Sampled() check) and emit the four child cells.
__global__ void k_aa_classify(const int4* __restrict__ cells, const int* __restrict__ ncells, int cap, int G, int MW,
                              const float4* __restrict__ grid, uint32_t* __restrict__ mask,
                              uint32_t* __restrict__ subdiv, const int2* __restrict__ pix_xy, double thr,
                              double subsize, double2* __restrict__ spos, int* __restrict__ sslot,
                              int* __restrict__ nsamples, int scap, int4* __restrict__ next, int* __restrict__ nnext,
                              int ncap, uint32_t* err)
{
    int n = min(*ncells, cap);
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        int i = base + threadIdx.x;
        bool active = i < n;
        unsigned amask = __ballot_sync(0xffffffffu, active);
        if (!active)
            continue;
        int4 c = cells[i];
        int pix = c.x, bx = c.y & 0xff, by = (c.y >> 8) & 0xff, step = c.y >> 16, level = c.z, id = c.w;
        const float4* g = grid + (size_t)pix * G * G;
        float4 c00 = g[by * G + bx], c02 = g[(by + step) * G + bx];
        float4 c20 = g[by * G + bx + step], c22 = g[(by + step) * G + bx + step];
        bool split = level > 0 && (aa_dist(c00, c02) >= thr || aa_dist(c00, c20) >= thr || aa_dist(c00, c22) >= thr ||
                                   aa_dist(c02, c20) >= thr || aa_dist(c02, c22) >= thr || aa_dist(c20, c22) >= thr);
        int h = step / 2;
        int gx[5] = {bx, bx + h, bx + step, bx + h, bx + h};
        int gy[5] = {by + h, by, by + h, by + step, by + h};
        int2 pxy = pix_xy[pix];
        for (int k = 0; k < 5; k++) {
            bool want = false;
            if (split) {
                int bit = gy[k] * G + gx[k];
                uint32_t old = atomicOr(mask + (size_t)pix * MW + (bit >> 5), 1u << (bit & 31));
                want = !(old & (1u << (bit & 31)));
            }
            int s = warp_reserve(nsamples, want, amask);
            if (want) {
                if (s < scap) {
                    spos[s] = make_double2((double)pxy.x + gx[k] / subsize, (double)pxy.y + gy[k] / subsize);
                    sslot[s] = pix * G * G + gy[k] * G + gx[k];
                } else {
                    set_error(err, DE_QUEUE_OVERFLOW);
                }
            }
        }
        int nb = warp_reserve_k(nnext, split, 4, amask);
        if (split) {
            atomicOr(subdiv + pix, 1u << id);
            if (nb + 4 <= ncap) {
                next[nb + 0] = make_int4(pix, bx | (by << 8) | (h << 16), level - 1, 4 * id + 1);
                next[nb + 1] = make_int4(pix, bx | ((by + h) << 8) | (h << 16), level - 1, 4 * id + 2);
                next[nb + 2] = make_int4(pix, (bx + h) | (by << 8) | (h << 16), level - 1, 4 * id + 3);
                next[nb + 3] = make_int4(pix, (bx + h) | ((by + h) << 8) | (h << 16), level - 1, 4 * id + 4);
            } else {
                set_error(err, DE_QUEUE_OVERFLOW);
            }
        }
    }
}

// Bottom-up pixel colour: a subdivided cell is the mean of its four
// children (rcx0y0 + rcx0y1 + rcx1y0 + rcx1y1) / 4, a leaf cell the mean of
// its corners (cx0y0 + cx0y2 + cx2y0 + cx2y2) / 4 (tracetask.cpp:1058-1062).
__device__ float4 aa_cell(const float4* g, int G, uint32_t bits, int id, int bx, int by, int step, int depth_left)
{
    if (depth_left > 0 && id < 32 && ((bits >> id) & 1u)) {
        int h = step / 2;
        float4 a = aa_cell(g, G, bits, 4 * id + 1, bx, by, h, depth_left - 1);
        float4 b = aa_cell(g, G, bits, 4 * id + 2, bx, by + h, h, depth_left - 1);
        float4 c = aa_cell(g, G, bits, 4 * id + 3, bx + h, by, h, depth_left - 1);
        float4 d = aa_cell(g, G, bits, 4 * id + 4, bx + h, by + h, h, depth_left - 1);
        return make_float4((a.x + b.x + c.x + d.x) / 4.0f, (a.y + b.y + c.y + d.y) / 4.0f,
                           (a.z + b.z + c.z + d.z) / 4.0f, (a.w + b.w + c.w + d.w) / 4.0f);
    }
    float4 a = g[by * G + bx], b = g[(by + step) * G + bx], c = g[by * G + bx + step],
           d = g[(by + step) * G + bx + step];
    return make_float4((a.x + b.x + c.x + d.x) / 4.0f, (a.y + b.y + c.y + d.y) / 4.0f,
                       (a.z + b.z + c.z + d.z) / 4.0f, (a.w + b.w + c.w + d.w) / 4.0f);
}

__global__ void k_aa_resolve(const float4* __restrict__ grid, const uint32_t* __restrict__ subdiv, int npix, int G,
                             int depth, float4* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix)
        return;
    out[i] = aa_cell(grid + (size_t)i * G * G, G, subdiv[i], 0, 0, 0, G - 1, depth - 1);
}

// --------------------------------------------------------------- launch --
static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

cudaError_t launch_refine(const DeviceScene& S, const double* org, const double* dir, QHit* hits, double* t64, int n,
                          cudaStream_t st)
{
    k_refine<<<cdiv(n > 0 ? n : 1, 256), 256, 0, st>>>(S, org, dir, hits, t64, n);
    return cudaGetLastError();
}

cudaError_t launch_camera(const DeviceScene& S, int mode, const int4* blocks, const int* block_off, int nblocks,
                          const double2* pos, const int* npos, int max_samples, int width, int height, QRay* q,
                          int* q_path, PathState* paths, int* q_count, unsigned long long* stats, uint2* q_skip,
                          float2* tab, cudaStream_t st)
{
    if (mode != 2)
        k_cam_table<<<cdiv(width + height + 2, 256), 256, 0, st>>>(width, height, mode == 0 ? 0.5 : 0.0, tab);
    k_camera<<<cdiv(max_samples > 0 ? max_samples : 1, 256), 256, 0, st>>>(
        S, mode, blocks, block_off, nblocks, pos, npos, width, height, q, q_path, paths, q_count, stats, q_skip,
        max_samples, tab);
    return cudaGetLastError();
}

cudaError_t launch_load_rays(const double* org, const double* dir, int n, QRay* q, int* q_count, cudaStream_t st)
{
    k_load_rays<<<cdiv(n > 0 ? n : 1, 256), 256, 0, st>>>(org, dir, n, q, q_count);
    return cudaGetLastError();
}

cudaError_t launch_trace(const DeviceScene& S, bool any_hit, const QRay* q, const int* q_count, int* work,
                         QHit* hits, uint8_t* blocked, int stack_depth, int grid, uint32_t* err,
                         unsigned long long* stats, unsigned long long* wcount, int cap, const uint2* skips,
                         cudaStream_t st, int block, int occ, const TorusDefer* defer)
{
    block = block == 64 ? 64 : 128;   // warps claim 32 rays; the stack is smem[k * blockDim + tid]
    size_t smem = (size_t)stack_depth * block * sizeof(int);
    // the full variant carries the FP64 torus solver and CSG; scenes without
    // them run the lean one (about half the registers)
    const bool full = S.has_full_prims != 0;
    TorusDefer td{};
    if (full && defer && defer->count && ((defer->cand && (any_hit || defer->key)) || defer->ovf)) {
        td = *defer;
        if (td.cand && !any_hit && !td.key)
            td.cand = nullptr;
        // count, ovf_count and ovf_work: three consecutive ints
        cudaError_t e = cudaMemsetAsync(td.count, 0, sizeof(int) * 3, st);
        if (e != cudaSuccess)
            return e;
    }
    const bool nt = td.ovf != nullptr;   // the torus-free variant and its second launch
    const TorusDefer none{};
    const int* no_index = nullptr;
#define POVGPU_TRACE(A, F, M, N, TD, QC, W, CAP, IDX)                                                             \
    k_trace<A, F, M, N><<<grid, block, smem, st>>>(S, q, QC, W, hits, blocked, stack_depth, err, stats, wcount, \
                                                   CAP, skips, TD, IDX)
    if (any_hit && full && nt)
        POVGPU_TRACE(true, true, 1, true, td, q_count, work, cap, no_index);
    else if (any_hit && full)
        POVGPU_TRACE(true, true, 1, false, td, q_count, work, cap, no_index);
    else if (any_hit && occ)
        POVGPU_TRACE(true, false, 8, false, td, q_count, work, cap, no_index);
    else if (any_hit)
        POVGPU_TRACE(true, false, 1, false, td, q_count, work, cap, no_index);
    else if (full && nt)
        POVGPU_TRACE(false, true, 1, true, td, q_count, work, cap, no_index);
    else if (full)
        POVGPU_TRACE(false, true, 1, false, td, q_count, work, cap, no_index);
    else if (occ)
        POVGPU_TRACE(false, false, 8, false, td, q_count, work, cap, no_index);
    else
        POVGPU_TRACE(false, false, 1, false, td, q_count, work, cap, no_index);
    if (td.cand) {
        const int g = grid;   // the traversal's persistent grid: SMs x blocks per SM
        if (any_hit) {
            k_torus_solve<true><<<g, 128, 0, st>>>(S, q, td, hits, blocked, stats);
        } else {
            k_torus_solve<false><<<g, 128, 0, st>>>(S, q, td, hits, blocked, stats);
            k_torus_merge<<<g, 256, 0, st>>>(q_count, cap, td, hits);
        }
    }
    if (nt) {   // the rays whose torus pairs did not fit: the ordinary full variant
        if (any_hit)
            POVGPU_TRACE(true, true, 1, false, none, td.ovf_count, td.ovf_work, td.ovf_cap, td.ovf);
        else
            POVGPU_TRACE(false, true, 1, false, none, td.ovf_count, td.ovf_work, td.ovf_cap, td.ovf);
    }
#undef POVGPU_TRACE
    return cudaGetLastError();
}

cudaError_t launch_shade(const DeviceScene& S, int level, int max_level, const QRay* q, const int* q_path,
                         const QHit* hits,
                         const int* q_count, PathState* paths, float4* slot_contrib, QRay* sq, int* sq_slot,
                         int* sq_count, uint2* sq_skip, QRay* nq, int* nq_path, uint2* nq_skip, int* nq_count,
                         int max_queue, int max_shadow, QRay* aq, int* aq_slot, uint2* aq_skip, int* aq_count,
                         int max_area, const ShadeRad& rad, const ShadeMedia& med, const int* order, int grid,
                         uint32_t* err, unsigned long long* stats, cudaStream_t st)
{
    k_shade<<<grid, 128, 0, st>>>(S, level, max_level, q, q_path, hits, q_count, paths, slot_contrib, sq, sq_slot, sq_count,
                                  sq_skip, nq, nq_path, nq_skip, nq_count, max_queue, max_shadow, aq, aq_slot,
                                  aq_skip, aq_count, max_area, rad, med, order, err, stats);
    return cudaGetLastError();
}

// ------------------------------------------------- shade-queue binning --
// Textured scenes: a hit's shading cost is its material's pattern pigment
// and normal perturbation, which differ ~50x between materials; a warp
// that mixes materials runs as slow as its slowest lane.  Before k_shade
// the queue is binned by material (a counting sort on a small key: 0 for
// misses and plain materials, 1 + material mod 255 for textured ones), so a
// warp shades one material.  Within a bin the items keep roughly their
// queue order (warps claim their places in turn), which keeps the rays a
// warp emits next to each other.
__device__ __forceinline__ int shade_key(const DeviceScene& S, const QHit& h)
{
    if (h.prim == NO_PRIM)
        return 0;
    uint32_t kind = h.prim >> PRIM_KIND_SHIFT, idx = h.prim & PRIM_INDEX_MASK;
    int obj;
    if (kind == PK_CSG) {
        const DevCsg g = S.csgs[idx];
        obj = S.csg_children[g.first + (__float_as_uint(h.u) & 0xffffu)].object;
    } else if (kind == PK_SPHERE) {
        obj = __ldg(S.sphere_obj + idx);
    } else if (kind == PK_PLANE) {
        obj = __ldg(S.plane_obj + idx);
    } else if (kind == PK_BOX) {
        obj = __float_as_int(S.boxes[idx].lo.w);
    } else if (kind == PK_TORUS) {
        obj = S.tori[idx].object;
    } else {
        obj = __float_as_int(__ldg(S.tri_normal + __ldg(S.tri_global + idx)).w);
    }
    const int mat = S.objects[obj].material;
    const DevMaterial& m = S.materials[mat];
    return (m.pattern || m.normal) ? 1 + mat % (SHADE_BINS - 1) : 0;
}

// Per item its key, and the keys' counts (one atomic per key per warp).
__global__ void k_bin_count(DeviceScene S, const QHit* __restrict__ hits, const int* __restrict__ q_count, int cap,
                            uint8_t* __restrict__ keys, int* __restrict__ hist)
{
    const int n = min(*q_count, cap);
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool active = i < n;
        const int key = active ? shade_key(S, hits[i]) : -1;
        if (active)
            keys[i] = (uint8_t)key;
        const unsigned same = __match_any_sync(0xffffffffu, key);
        if (active && (threadIdx.x & 31) == __ffs(same) - 1)
            atomicAdd(&hist[key], __popc(same));
    }
}

// Exclusive scan of the key counts into each bin's first place (one block).
__global__ void k_bin_scan(int* __restrict__ hist, int* __restrict__ cursor)
{
    __shared__ int s[SHADE_BINS];
    const int t = threadIdx.x;
    s[t] = hist[t];
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int k = 0; k < SHADE_BINS; k++) {
            const int c = s[k];
            s[k] = run;
            run += c;
        }
    }
    __syncthreads();
    cursor[t] = s[t];
}

// Every item to its place in its bin: lanes of a warp with the same key
// take consecutive places in lane order (one atomic per key per warp).
__global__ void k_bin_scatter(const int* __restrict__ q_count, int cap, const uint8_t* __restrict__ keys,
                              int* __restrict__ cursor, int* __restrict__ order)
{
    const int n = min(*q_count, cap);
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool active = i < n;
        const int key = active ? (int)keys[i] : -1;
        const unsigned same = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(same) - 1;
        int first = 0;
        if (active && lane == leader)
            first = atomicAdd(&cursor[key], __popc(same));
        first = __shfl_sync(0xffffffffu, first, leader);
        if (active)
            order[first + __popc(same & ((1u << lane) - 1u))] = i;
    }
}

cudaError_t launch_shade_bins(const DeviceScene& S, const QHit* hits, const int* q_count, int cap, uint8_t* keys,
                              int* hist, int* order, int grid, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(int) * SHADE_BINS, st);
    if (e != cudaSuccess)
        return e;
    k_bin_count<<<grid, 128, 0, st>>>(S, hits, q_count, cap, keys, hist);
    k_bin_scan<<<1, SHADE_BINS, 0, st>>>(hist, hist + SHADE_BINS);
    k_bin_scatter<<<grid, 128, 0, st>>>(q_count, cap, keys, hist + SHADE_BINS, order);
    return cudaGetLastError();
}

cudaError_t launch_shadow_through(const DeviceScene& S, const QRay* sq, const int* sq_slot, const uint2* sq_skip,
                                  const int* sq_medium, const int* sq_count, int cap, int* work, uint8_t* blocked,
                                  float4* slot_contrib, bool media_on, int stack_depth, int grid, uint32_t* err,
                                  unsigned long long* stats, cudaStream_t st)
{
    const int block = 128;
    size_t smem = (size_t)stack_depth * block * sizeof(int);
    if (S.has_full_prims)
        k_shadow_through<true><<<grid, block, smem, st>>>(S, sq, sq_slot, sq_skip, sq_medium, sq_count, cap, work,
                                                          blocked, slot_contrib, media_on ? 1 : 0, stack_depth, err,
                                                          stats);
    else
        k_shadow_through<false><<<grid, block, smem, st>>>(S, sq, sq_slot, sq_skip, sq_medium, sq_count, cap, work,
                                                           blocked, slot_contrib, media_on ? 1 : 0, stack_depth, err,
                                                           stats);
    return cudaGetLastError();
}

cudaError_t launch_shadow_filter(const DeviceScene& S, const QRay* sq, const int* sq_slot, const uint2* sq_skip,
                                 const uint64_t* sq_rin, const int* sq_count, int cap, int* work, uint8_t* blocked,
                                 float4* slot_contrib, int stack_depth, int grid, uint32_t* err,
                                 unsigned long long* stats, cudaStream_t st)
{
    const int block = 128;
    size_t smem = (size_t)stack_depth * block * sizeof(int);
    if (S.has_full_prims)
        k_shadow_filter<true><<<grid, block, smem, st>>>(S, sq, sq_slot, sq_skip, sq_rin, sq_count, cap, work,
                                                         blocked, slot_contrib, stack_depth, err, stats);
    else
        k_shadow_filter<false><<<grid, block, smem, st>>>(S, sq, sq_slot, sq_skip, sq_rin, sq_count, cap, work,
                                                          blocked, slot_contrib, stack_depth, err, stats);
    return cudaGetLastError();
}

cudaError_t launch_media_list(const int* q_state, const QHit* hits, const int* q_count, int cap, int* mlist,
                              int* mcount, int grid, cudaStream_t st)
{
    k_media_list<<<grid, 128, 0, st>>>(q_state, hits, q_count, cap, mlist, mcount);
    return cudaGetLastError();
}

cudaError_t launch_media_chunk(const DeviceScene& S, const QRay* q, const int* q_state, const QHit* hits,
                               const int* mlist, int first, int nseg, int NI, int SMAX, int max_sub, int max_levels,
                               float4* cbuf, int* listA, int* listB, int* counts, int list_cap, int stamp,
                               float4* te, float4* od, int stack_depth, int grid, uint32_t* err,
                               unsigned long long* stats, cudaStream_t st)
{
    MediaWork W{};
    W.q = q;
    W.q_state = q_state;
    W.hits = hits;
    W.mlist = mlist;
    W.first = first;
    W.nseg = nseg;
    W.NI = NI;
    W.SMAX = SMAX;
    W.cbuf = cbuf;
    W.list_cap = list_cap;
    W.stamp = stamp;
    W.te = te;
    W.od = od;
    const int block = 128;
    const size_t smem = (size_t)stack_depth * block * sizeof(int);
    cudaError_t e;
    int* work = counts + 1;   // the sample rounds' work counter
    auto sample = [&](const MediaWork& w) {
        cudaError_t r = cudaMemsetAsync(work, 0, sizeof(int), st);
        if (r != cudaSuccess)
            return r;
        if (S.has_full_prims)
            k_media_sample<true><<<grid, block, smem, st>>>(S, w, 2 * max_sub + 1, work, stack_depth, err, stats);
        else
            k_media_sample<false><<<grid, block, smem, st>>>(S, w, 2 * max_sub + 1, work, stack_depth, err, stats);
        return cudaGetLastError();
    };
    // round 0: every interval's ends and midpoints
    if ((e = sample(W)) != cudaSuccess)
        return e;
    // rounds 1 .. levels-1: the halves that differ
    for (int s = 1; s < max_levels; s++) {
        int* out = (s & 1) ? listA : listB;   // the list of round s (consumed before round s+1 fills one)
        int* out_count = counts;
        if ((e = cudaMemsetAsync(out_count, 0, sizeof(int), st)) != cudaSuccess)
            return e;
        MediaWork X = W;
        X.next = out;
        X.next_count = out_count;
        k_media_expand<<<grid, block, 0, st>>>(S, X, s, max_sub, err);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        MediaWork Y = W;
        Y.list = out;
        Y.list_count = out_count;
        if ((e = sample(Y)) != cudaSuccess)
            return e;
    }
    k_media_reduce<<<grid, block, 0, st>>>(S, W);
    return cudaGetLastError();
}

cudaError_t launch_media_combine(const DeviceScene& S, const int* q_state, const int* q_path, const QHit* hits,
                                 const int* mlist, const int* mcount, int cap, int NI, const float4* te,
                                 const float4* od, PathState* paths, int grid, cudaStream_t st)
{
    k_media_combine<<<grid, 128, 0, st>>>(q_state, q_path, hits, mlist, mcount, cap, NI, S, te, od, paths);
    return cudaGetLastError();
}

cudaError_t launch_area_shadow(const DeviceScene& S, const QRay* aq, const int* aq_slot, const uint2* aq_skip,
                               const int* aq_count, int cap, float4* slot_contrib, int stack_depth, int grid,
                               uint32_t* err, unsigned long long* stats, cudaStream_t st)
{
    const int block = 128;
    size_t smem = (size_t)stack_depth * block * sizeof(int);
    if (S.has_full_prims)
        k_area_shadow<true><<<grid, block, smem, st>>>(S, aq, aq_slot, aq_skip, aq_count, cap, slot_contrib,
                                                       stack_depth, err, stats);
    else
        k_area_shadow<false><<<grid, block, smem, st>>>(S, aq, aq_slot, aq_skip, aq_count, cap, slot_contrib,
                                                        stack_depth, err, stats);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const int* q_path, const int* q_count, int num_lights, const int* sq_slot,
                           const uint8_t* blocked, const int* sq_count, float4* slot_contrib, PathState* paths,
                           int grid, int cap_rays, int cap_shadow, cudaStream_t st, bool branching)
{
    k_mark_blocked<<<grid, 256, 0, st>>>(sq_slot, blocked, sq_count, slot_contrib, cap_shadow);
    k_resolve<<<grid, 256, 0, st>>>(q_path, q_count, num_lights, slot_contrib, paths, cap_rays, branching ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const PathState* paths, const int* count, int max_samples, const int* slot, float4* out,
                            cudaStream_t st)
{
    k_finalize<<<cdiv(max_samples > 0 ? max_samples : 1, 256), 256, 0, st>>>(paths, count, max_samples, slot, out);
    return cudaGetLastError();
}

cudaError_t launch_aa_init(const int4* blocks, const int* pix_off, const int* corner_off, int nblocks, int npix,
                           const float4* corners, int G, int MW, float4* grid, uint32_t* mask, uint32_t* subdiv,
                           int2* pix_xy, int4* cells, int* ncells, int root_level, cudaStream_t st)
{
    k_aa_init<<<cdiv(npix > 0 ? npix : 1, 256), 256, 0, st>>>(blocks, pix_off, corner_off, nblocks, corners, G, MW,
                                                               grid, mask, subdiv, pix_xy, cells, ncells, root_level);
    return cudaGetLastError();
}

cudaError_t launch_aa_classify(const int4* cells, const int* ncells, int cap, int G, int MW, const float4* grid,
                               uint32_t* mask, uint32_t* subdiv, const int2* pix_xy, double thr, double subsize,
                               double2* spos, int* sslot, int* nsamples, int scap, int4* next, int* nnext, int ncap,
                               uint32_t* err, int grid_blocks, cudaStream_t st)
{
    k_aa_classify<<<grid_blocks, 128, 0, st>>>(cells, ncells, cap, G, MW, grid, mask, subdiv, pix_xy, thr, subsize,
                                                spos, sslot, nsamples, scap, next, nnext, ncap, err);
    return cudaGetLastError();
}

cudaError_t launch_aa_resolve(const float4* grid, const uint32_t* subdiv, int npix, int G, int depth, float4* out,
                              cudaStream_t st)
{
    k_aa_resolve<<<cdiv(npix > 0 ? npix : 1, 128), 128, 0, st>>>(grid, subdiv, npix, G, depth, out);
    return cudaGetLastError();
}

// ------------------------------------------------- fixed-scratch ray query --
// Scratch of pov_gpu_trace_rays_static: one file-scope device array, which
// CUDA places in this module's static memory on each device when it loads
// the module, so that query allocates nothing per call.  Layout
// (STATIC_OFF_* offsets): a 256-byte header (work counters, device error
// word, statistics; zeroed by every call before its first launch) followed
// by the per-ray arrays sized for STATIC_MAX_RAYS rays.  One array per
// device: calls that overlap in time on one device share it and race.
static __device__ __align__(256) unsigned char g_ray_scratch[STATIC_SCRATCH_BYTES];

// Maps closest hits to the ABI's (object, triangle, depth) records on the
// device: the mapping pov_gpu_trace_rays does on the host.
__global__ void k_hits_abi(DeviceScene S, const QHit* __restrict__ hits, const double* __restrict__ t64, int n,
                           PovGpuHit* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    QHit h = hits[i];
    PovGpuHit r;
    r.object = -1;
    r.triangle = -1;
    r.t = 0.0;
    if (h.prim != 0xffffffffu) {
        uint32_t kind = h.prim >> PRIM_KIND_SHIFT, idx = h.prim & PRIM_INDEX_MASK;
        r.t = t64[i];
        if (kind == PK_SPHERE) {
            r.object = S.sphere_obj[idx];
        } else if (kind == PK_PLANE) {
            r.object = S.plane_obj[idx];
        } else if (kind == PK_BOX) {
            r.object = __float_as_int(S.boxes[idx].lo.w);
        } else if (kind == PK_TORUS) {
            r.object = S.tori[idx].object;
        } else if (kind == PK_CSG) {
            DevCsg cg = S.csgs[idx];
            r.object = S.csg_children[cg.first + (__float_as_uint(h.u) & 0xffffu)].object;
        } else if (kind == PK_TRIANGLE) {
            int g = S.tri_global[idx];
            r.object = __float_as_int(S.tri_normal[g].w);
            r.triangle = S.tri_local[g];
        }
    }
    out[i] = r;
}

cudaError_t launch_hits_abi(const DeviceScene& S, const QHit* hits, const double* t64, int n, PovGpuHit* out,
                            cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    k_hits_abi<<<cdiv(n, 256), 256, 0, st>>>(S, hits, t64, n, out);
    return cudaGetLastError();
}

cudaError_t static_ray_scratch(int device, unsigned char** out)
{
    // The address is looked up once per device and cached.  The first lookup
    // on a device can make CUDA load this module there, which places
    // g_ray_scratch in device memory; later lookups only read the cache.
    constexpr int CACHED_DEVICES = 64;
    static std::mutex lock;
    static unsigned char* cache[CACHED_DEVICES] = {};
    *out = nullptr;
    std::lock_guard<std::mutex> g(lock);
    if (device >= 0 && device < CACHED_DEVICES && cache[device]) {
        *out = cache[device];
        return cudaSuccess;
    }
    unsigned char* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_ray_scratch);
    if (e != cudaSuccess)
        return e;
    if (device >= 0 && device < CACHED_DEVICES)
        cache[device] = ptr;
    *out = ptr;
    return cudaSuccess;
}

}  // namespace povgpu
