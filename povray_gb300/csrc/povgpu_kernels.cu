// povgpu_kernels.cu -- sm_103a kernels of the trace path.
//
// One frame (a batch of render blocks) is a short wavefront pipeline:
//   k_camera         primary rays of every pixel (TracePixel::CreateCameraRay,
//                    source/core/render/tracepixel.cpp:357-373,924)
//   per trace level L = 0 .. max_trace_level-1:
//     k_trace<closest>  Trace::FindIntersection (trace.cpp:285) over the BVH
//     k_shade           ComputeTextureColour/ComputeLightedTexture
//                       (trace.cpp:457-1179): emission/ambient, per-light
//                       diffuse/phong/specular terms, shadow-ray and
//                       reflection-ray emission (ComputeReflection,
//                       trace.cpp:1264-1321) into compacted queues
//     k_trace<any>      TracePointLightShadowRay (trace.cpp:1951-2076) for
//                       opaque occluders: any hit in (1e-3, dist-1e-3)
//     k_resolve         adds each unblocked light term to its path
//   k_finalize       RGBT per pixel in block order (CompletedRectangle).
// Traversal kernels are persistent: each warp pulls 32 rays at a time from
// a device counter, so no host round trip sits between the stages and the
// whole sequence can be captured into one CUDA graph.
#include "povgpu_internal.h"
#include "povgpu_kernels.h"

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

namespace povgpu {

// Tolerances of the reference (source/core/configcore.h:153-206,
// source/core/render/trace.cpp:81).
__constant__ float kMinIsectDepth = 1.0e-4f;
#define EPSILON_D 1.0e-10
#define EPSILON_F 1.0e-10f
#define SMALL_TOLERANCE_F 1.0e-3f
#define SHADOW_TOLERANCE_F 1.0e-3f
#define MAX_DISTANCE_F 1.0e7f

// ------------------------------------------------------------ helpers --
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
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

// --------------------------------------------------------------- camera --
// Primary ray of pixel centre (x+0.5, y+0.5); direction formed and
// normalised in FP64 exactly as CreateCameraRay does, then rounded.
__global__ void k_camera(DeviceScene S, const int4* __restrict__ blocks, const int* __restrict__ block_off,
                         int nblocks, int width, int height, QRay* __restrict__ q, int* __restrict__ q_path,
                         PathState* __restrict__ paths, int* __restrict__ q_count, unsigned long long* stats,
                         uint32_t* __restrict__ q_skip)
{
    int npix = block_off[nblocks];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *q_count = npix;
        atomicAdd(&stats[ST_RAYS], (unsigned long long)npix);
    }
    if (i >= npix)
        return;
    // block containing pixel i (binary search over the prefix offsets)
    int lo = 0, hi = nblocks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (block_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    int4 b = blocks[lo];   // left, top, right, bottom
    int w = b.z - b.x + 1;
    int local = i - block_off[lo];
    int x = b.x + local % w;
    int y = b.y + local / w;
    double x0 = ((double)x + 0.5) / (double)width - 0.5;
    double y0 = 0.5 - ((double)y + 0.5) / (double)height;
    double dx = S.cam_dir[0] + x0 * S.cam_right[0] + y0 * S.cam_up[0];
    double dy = S.cam_dir[1] + x0 * S.cam_right[1] + y0 * S.cam_up[1];
    double dz = S.cam_dir[2] + x0 * S.cam_right[2] + y0 * S.cam_up[2];
    double l = sqrt(dx * dx + dy * dy + dz * dz);
    if (l != 0.0) { dx /= l; dy /= l; dz /= l; }
    QRay r;
    r.org = make_float4((float)S.cam_loc[0], (float)S.cam_loc[1], (float)S.cam_loc[2], kMinIsectDepth);
    r.dir = make_float4((float)dx, (float)dy, (float)dz, CUDART_INF_F);
    q[i] = r;
    q_path[i] = i;
    q_skip[i] = 0xffffffffu;
    PathState p;
    p.colour = make_float4(0.f, 0.f, 0.f, 0.f);
    p.throughput = make_float4(1.f, 1.f, 1.f, 1.f);
    paths[i] = p;
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

// ------------------------------------------------------------ intersect --
// Sphere (Sphere::Intersect, sphere.cpp:214-245) with the chord computed
// from the perpendicular offset vector, which keeps FP32 accurate far from
// the sphere; near-tangent rays (the reference's grazing band) are re-solved
// in FP64.  Returns the nearest root in (tmin, tmax), or tmax.
__device__ __forceinline__ bool isect_sphere(float4 s, float3 o, float3 d, float tmin, float& t)
{
    float3 oc = xyz(s) - o;
    float tca = dot3(oc, d);
    float ocs = dot3(oc, oc);
    float r2 = s.w * s.w;
    if (ocs >= r2 && tca < EPSILON_F)
        return false;
    float3 perp = oc - d * tca;
    float thcs = r2 - dot3(perp, perp);
    if (thcs <= 1.0e-4f * r2) {
        // grazing band: FP64 re-solve (the reference works in double)
        double ox = (double)s.x - o.x, oy = (double)s.y - o.y, oz = (double)s.z - o.z;
        double tcad = ox * d.x + oy * d.y + oz * d.z;
        double px = ox - d.x * tcad, py = oy - d.y * tcad, pz = oz - d.z * tcad;
        double th = (double)s.w * s.w - (px * px + py * py + pz * pz);
        if (!(th > EPSILON_D))
            return false;
        double hc = sqrt(th);
        double t1 = tcad - hc, t2 = tcad + hc;
        if (t1 > 1.0e-6 && (float)t1 >= tmin && (float)t1 < t) { t = (float)t1; return true; }
        if (t2 > 1.0e-6 && (float)t2 >= tmin && (float)t2 < t) { t = (float)t2; return true; }
        return false;
    }
    float hc = sqrtf(thcs);
    float t1 = tca - hc, t2 = tca + hc;
    if (t1 >= tmin && t1 < t) { t = t1; return true; }
    if (t2 >= tmin && t2 < t) { t = t2; return true; }
    return false;
}

// A ray starting on the sphere's own surface: only the far root, and only
// when the ray heads into the sphere (tca > 0).
__device__ __forceinline__ bool isect_sphere_far(float4 s, float3 o, float3 d, float tmin, float& t)
{
    float3 oc = xyz(s) - o;
    float tca = dot3(oc, d);
    if (tca <= 0.0f)
        return false;
    float3 perp = oc - d * tca;
    float thcs = s.w * s.w - dot3(perp, perp);
    if (!(thcs > 0.0f))
        return false;
    float t2 = tca + sqrtf(thcs);
    if (t2 >= tmin && t2 < t) {
        t = t2;
        return true;
    }
    return false;
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
__device__ __forceinline__ void node_test(const BvhNode* __restrict__ nodes, int ni, float3 o, float3 inv,
                                          float tmin, float tmax, bool& h0, bool& h1, float& t0, float& t1,
                                          int& l0, int& l1)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + ni);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    float ax0 = (a.x - o.x) * inv.x, ax1 = (a.y - o.x) * inv.x;
    float ay0 = (a.z - o.y) * inv.y, ay1 = (a.w - o.y) * inv.y;
    float az0 = (c.x - o.z) * inv.z, az1 = (c.y - o.z) * inv.z;
    float bx0 = (b.x - o.x) * inv.x, bx1 = (b.y - o.x) * inv.x;
    float by0 = (b.z - o.y) * inv.y, by1 = (b.w - o.y) * inv.y;
    float bz0 = (c.z - o.z) * inv.z, bz1 = (c.w - o.z) * inv.z;
    float an = fmaxf(fmaxf(fminf(ax0, ax1), fminf(ay0, ay1)), fmaxf(fminf(az0, az1), tmin));
    float af = fminf(fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1)), fminf(fmaxf(az0, az1), tmax));
    float bn = fmaxf(fmaxf(fminf(bx0, bx1), fminf(by0, by1)), fmaxf(fminf(bz0, bz1), tmin));
    float bf = fminf(fminf(fmaxf(bx0, bx1), fmaxf(by0, by1)), fminf(fmaxf(bz0, bz1), tmax));
    // conservative: widen the far side by 3 ulp-ish so rounding never culls
    // a box the exact test would enter
    h0 = an <= af * 1.00000024f;
    h1 = bn <= bf * 1.00000024f;
    t0 = an;
    t1 = bn;
    l0 = __float_as_int(d.x);
    l1 = __float_as_int(d.y);
}

// ------------------------------------------------------------- traversal --
// Closest hit (ANY = false) or any hit (ANY = true) for every ray in the
// queue.  Stack in shared memory: slot k of thread t at smem[k*blockDim+t].
template <bool ANY>
__global__ void __launch_bounds__(128) k_trace(DeviceScene S, const QRay* __restrict__ q,
                                               const int* __restrict__ q_count, int* __restrict__ work,
                                               QHit* __restrict__ hits, uint8_t* __restrict__ blocked,
                                               int stack_depth, uint32_t* err, unsigned long long* stats,
                                               unsigned long long* wcount, int cap,
                                               const uint32_t* __restrict__ skips)
{
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
        QRay r = q[i];
        if (counting) c_rays++;
        float3 o = xyz(r.org), d = xyz(r.dir);
        float tmin = r.org.w;
        float t = r.dir.w;
        float3 inv = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
        uint32_t best = 0xffffffffu;
        float bu = 0.f, bv = 0.f;
        bool done = false;
        // The surface a secondary ray starts on: in exact arithmetic a ray
        // leaving a plane or a planar triangle never meets it again, and one
        // leaving a sphere meets it only at the far root; FP32 rounding of the
        // origin must not invent those self-hits (the reference works in FP64).
        const uint32_t skip = skips ? skips[i] : 0xffffffffu;
        // infinite objects first (planes: Plane::Intersect, plane.cpp:139-211)
        for (int k = 0; k < S.num_planes; k++) {
            if (((PK_PLANE << PRIM_KIND_SHIFT) | (uint32_t)k) == skip)
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
        while (!done && node != 0x7fffffff) {
            if (++iters > (1 << 22)) {
                set_error(err, DE_ITERATION_CAP);
                break;
            }
            if (node >= 0) {
                bool h0, h1;
                float t0, t1;
                int l0, l1;
                node_test(S.nodes, node, o, inv, tmin, t, h0, h1, t0, t1, l0, l1);
                if (counting) c_nodes++;
                if (h0 && h1) {
                    int nearl = l0, farl = l1;
                    if (t1 < t0) { nearl = l1; farl = l0; }
                    if (sp >= stack_depth) {
                        set_error(err, DE_STACK_OVERFLOW);
                        break;
                    }
                    smem[sp * blockDim.x + threadIdx.x] = farl;
                    sp++;
                    node = nearl;
                } else if (h0) {
                    node = l0;
                } else if (h1) {
                    node = l1;
                } else {
                    node = sp > 0 ? smem[(--sp) * blockDim.x + threadIdx.x] : 0x7fffffff;
                }
            } else {
                uint32_t code = ~(uint32_t)node;
                uint32_t first = code >> 3;
                uint32_t count = (code & 7u) + 1u;
                for (uint32_t k = 0; k < count; k++) {
                    uint32_t ref = __ldg(S.prim_refs + first + k);
                    uint32_t kind = ref >> PRIM_KIND_SHIFT;
                    uint32_t idx = ref & PRIM_INDEX_MASK;
                    bool hit = false;
                    if (counting) { c_prims++; c_tris += kind == PK_TRIANGLE; }
                    if (ref == skip) {
                        if (kind == PK_SPHERE)
                            hit = isect_sphere_far(__ldg(S.spheres + idx), o, d, tmin, t);
                    } else if (kind == PK_TRIANGLE) {
                        float uu, vv;
                        hit = isect_tri(__ldg(S.tri_v0 + idx), __ldg(S.tri_e1 + idx), __ldg(S.tri_e2 + idx), o,
                                        d, tmin, t, uu, vv);
                        if (hit) { bu = uu; bv = vv; }
                    } else if (kind == PK_SPHERE) {
                        hit = isect_sphere(__ldg(S.spheres + idx), o, d, tmin, t);
                    }
                    if (hit) {
                        best = ref;
                        if (ANY) { done = true; break; }
                    }
                }
                if (done)
                    break;
                node = sp > 0 ? smem[(--sp) * blockDim.x + threadIdx.x] : 0x7fffffff;
            }
        }
        if (ANY) {
            blocked[i] = done ? 1 : 0;
            nblocked += done ? 1 : 0;
        } else {
            QHit h;
            h.t = t;
            h.prim = best;
            h.u = bu;
            h.v = bv;
            hits[i] = h;
        }
    }
    if (ANY && stats) {
        // one atomic per warp
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

// ---------------------------------------------------------------- shade --
struct SurfaceInfo {
    int32_t object;
    int32_t triangle;   // mesh-local triangle, -1 otherwise
    float3  normal;     // raw normal (unflipped)
};

__device__ __forceinline__ SurfaceInfo surface(const DeviceScene& S, const QHit& h, float3 p)
{
    SurfaceInfo si;
    uint32_t kind = h.prim >> PRIM_KIND_SHIFT;
    uint32_t idx = h.prim & PRIM_INDEX_MASK;
    si.triangle = -1;
    if (kind == PK_SPHERE) {
        float4 s = __ldg(S.spheres + idx);
        si.object = __ldg(S.sphere_obj + idx);
        si.normal = (p - xyz(s)) * (1.0f / s.w);   // Sphere::Normal, sphere.cpp:352
    } else if (kind == PK_PLANE) {
        float4 pl = __ldg(S.planes + idx);
        si.object = __ldg(S.plane_obj + idx);
        si.normal = xyz(pl);
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

// One thread per ray of the level queue.  Emits shadow rays (one per lit
// light, slot = ray*num_lights+light) and the reflection ray.
__global__ void __launch_bounds__(128) k_shade(
    DeviceScene S, int level, const QRay* __restrict__ q, const int* __restrict__ q_path,
    const QHit* __restrict__ hits, const int* __restrict__ q_count, PathState* __restrict__ paths,
    float4* __restrict__ slot_contrib, QRay* __restrict__ sq, int* __restrict__ sq_slot, int* __restrict__ sq_count,
    uint32_t* __restrict__ sq_skip, QRay* __restrict__ nq, int* __restrict__ nq_path,
    uint32_t* __restrict__ nq_skip, int* __restrict__ nq_count, int max_queue,
    int max_shadow, uint32_t* err, unsigned long long* stats)
{
    const int n = min(*q_count, max_queue);
    const int nl = S.num_lights;
    unsigned long long c_rays = 0, c_refl = 0, c_shadow = 0;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        int i = base + threadIdx.x;
        bool active = i < n;
        unsigned mask = __ballot_sync(0xffffffffu, active);
        if (!active)
            continue;
        QRay r = q[i];
        QHit h = hits[i];
        int path = q_path[i];
        float3 o = xyz(r.org), d = xyz(r.dir);
        PathState ps = paths[path];
        float3 thr = xyz(ps.throughput);
        float weight = ps.throughput.w;
        bool hit = h.prim != 0xffffffffu;
        float3 col = f3(0.f, 0.f, 0.f);
        float3 p = o + d * h.t;
        float3 N = f3(0.f, 1.f, 0.f);
        const DevMaterial* m = nullptr;
        int oflags = 0;
        if (hit) {
            SurfaceInfo si = surface(S, h, p);
            ObjectShade os = S.objects[si.object];
            oflags = os.flags;
            m = S.materials + os.material;
            N = si.normal;
            if (oflags & 1)            // INVERTED_FLAG
                N = N * -1.0f;
            if (dot3(N, d) > 0.0f)     // face the ray (trace.cpp:492-494)
                N = N * -1.0f;
            float4 pig = m->pigment;
            float4 em = m->emission;
            col = f3(pig.x * em.x, pig.y * em.y, pig.z * em.z);
        } else {
            col = xyz(S.background);   // ComputeSky, background only
        }
        // per-light terms (ComputeOneDiffuseLight, trace.cpp:1637-1729)
        for (int l = 0; l < nl; l++) {
            bool emit = false;
            float3 contrib = f3(0.f, 0.f, 0.f);
            float3 ld = f3(0.f, 0.f, 1.f);
            float ldist = 0.f;
            if (hit) {
                DevLight L = S.lights[l];
                float3 lv = xyz(L.center) - p;
                ldist = sqrtf(dot3(lv, lv));
                ld = lv * (1.0f / ldist);
                float cs = dot3(N, ld);
                bool lit = (oflags & 16) || cs >= EPSILON_F;
                float3 lc = xyz(L.colour);
                if (lit && !(fabsf(lc.x) < EPSILON_F && fabsf(lc.y) < EPSILON_F && fabsf(lc.z) < EPSILON_F)) {
                    emit = true;
                    float3 pig = xyz(m->pigment);
                    if (m->diffuse > 0.0f) {   // ComputeDiffuseColour, trace.cpp:2441-2484
                        float inten = m->brilliance != 1.0f ? powf(fabsf(cs), m->brilliance) : fabsf(cs);
                        inten *= m->diffuse;
                        contrib = contrib + pig * lc * inten;
                    }
                    if (m->phong > 0.0f) {     // ComputePhongColour, trace.cpp:2520-2558
                        float c2 = -2.0f * dot3(d, N);
                        float3 rd = d + N * c2;
                        float ci = dot3(rd, ld);
                        if (ci > 0.0f && (m->phong_size < 60.0f || ci > 0.0008f))
                            contrib = contrib + lc * (m->phong * powf(ci, m->phong_size));
                    }
                    if (m->specular > 0.0f) {  // ComputeSpecularColour, trace.cpp:2560-2593
                        float3 half = (ld - d) * 0.5f;
                        float hl = sqrtf(dot3(half, half));
                        if (hl > 0.0f) {
                            float ci = dot3(half, N) / hl;
                            if (ci > 0.0f)
                                contrib = contrib + lc * (m->specular * powf(ci, m->roughness));
                        }
                    }
                }
            }
            int slot = warp_reserve(sq_count, emit, mask);
            if (emit) {
                if (slot < max_shadow) {
                    QRay sr;
                    sr.org = make_float4(p.x, p.y, p.z, __uint_as_float(__float_as_uint(SMALL_TOLERANCE_F) + 1u));
                    sr.dir = make_float4(ld.x, ld.y, ld.z, ldist - SHADOW_TOLERANCE_F);
                    sq[slot] = sr;
                    sq_slot[slot] = i * nl + l;
                    sq_skip[slot] = h.prim;
                } else {
                    set_error(err, DE_QUEUE_OVERFLOW);
                }
                c_shadow++;
            }
            slot_contrib[(size_t)i * nl + l] =
                make_float4(contrib.x * thr.x, contrib.y * thr.y, contrib.z * thr.z, emit ? 1.0f : 0.0f);
        }
        // reflection (ComputeReflectivity, trace.cpp:2627-2656, non-fresnel)
        bool refl = false;
        float3 reflec = f3(0.f, 0.f, 0.f);
        float rweight = 0.f;
        float3 nd = f3(0.f, 0.f, 1.f);
        if (hit && m->has_reflection) {
            float cos_inc = -dot3(d, N);
            float falloff = m->reflect.w;
            float frac = fabsf(falloff - 1.0f) > EPSILON_F ? powf(1.0f - cos_inc, falloff) : 1.0f - cos_inc;
            float3 rmax = xyz(m->reflect), rmin = xyz(m->reflect_min);
            if (fabsf(frac) < EPSILON_F) reflec = rmin;
            else if (fabsf(frac - 1.0f) < EPSILON_F) reflec = rmax;
            else reflec = rmax * frac + rmin * (1.0f - frac);
            rweight = weight * m->reflect_min.w;
            if (reflec.x != 0.0f || reflec.y != 0.0f || reflec.z != 0.0f) {
                c_refl++;
                c_rays++;   // the TraceRay call is counted even when it bails
                // mirror direction; with an unperturbed normal the raw-normal
                // fix-ups of ComputeReflection never trigger
                float n2 = -2.0f * dot3(d, N);
                nd = normalize3(d + N * n2);
                refl = (level + 1 < S.max_trace_level) && (rweight >= S.adc_bailout);
            }
        }
        int rs = warp_reserve(nq_count, refl, mask);
        if (refl) {
            if (rs < max_queue) {
                QRay rr;
                rr.org = make_float4(p.x, p.y, p.z, kMinIsectDepth);
                rr.dir = make_float4(nd.x, nd.y, nd.z, CUDART_INF_F);
                nq[rs] = rr;
                nq_path[rs] = path;
                nq_skip[rs] = h.prim;
                paths[path].throughput = make_float4(thr.x * reflec.x, thr.y * reflec.y, thr.z * reflec.z, rweight);
            } else {
                set_error(err, DE_QUEUE_OVERFLOW);
            }
        }
        float4 c = ps.colour;
        paths[path].colour = make_float4(c.x + col.x * thr.x, c.y + col.y * thr.y, c.z + col.z * thr.z, c.w);
    }
    // per-warp counter reduction
    for (int off = 16; off > 0; off >>= 1) {
        c_rays += __shfl_down_sync(0xffffffffu, c_rays, off);
        c_refl += __shfl_down_sync(0xffffffffu, c_refl, off);
        c_shadow += __shfl_down_sync(0xffffffffu, c_shadow, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c_rays) atomicAdd(&stats[ST_RAYS], c_rays);
        if (c_refl) atomicAdd(&stats[ST_REFLECTED], c_refl);
        if (c_shadow) atomicAdd(&stats[ST_SHADOW_TESTS], c_shadow);
    }
}

// Marks blocked light terms (the any-hit kernel wrote one byte per shadow
// ray) and adds the remaining terms to their paths in light order.
__global__ void k_mark_blocked(const int* __restrict__ sq_slot, const uint8_t* __restrict__ blocked,
                               const int* __restrict__ sq_count, float4* __restrict__ slot_contrib)
{
    int n = *sq_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (blocked[i])
            slot_contrib[sq_slot[i]].w = 0.0f;
}

__global__ void k_resolve(const int* __restrict__ q_path, const int* __restrict__ q_count, int num_lights,
                          const float4* __restrict__ slot_contrib, PathState* __restrict__ paths)
{
    int n = *q_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int path = q_path[i];
        float4 c = paths[path].colour;
        for (int l = 0; l < num_lights; l++) {
            float4 s = slot_contrib[(size_t)i * num_lights + l];
            if (s.w != 0.0f) {
                c.x += s.x;
                c.y += s.y;
                c.z += s.z;
            }
        }
        paths[path].colour = c;
    }
}

__global__ void k_finalize(const PathState* __restrict__ paths, int npix, float4* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npix) {
        float4 c = paths[i].colour;
        out[i] = make_float4(c.x, c.y, c.z, 0.0f);
    }
}

__global__ void k_zero(int* p, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        p[i] = 0;
}

// FP64 re-solve of the winning primitive for rays given in FP64: the depth
// the reference computes for the same ray (sphere: Sphere::Intersect in
// double; plane: Plane::Intersect; triangle: intersect_mesh_triangle's
// plane distance from the stored FP32 normal and Distance, mesh.cpp:1046-1060).
__global__ void k_refine(DeviceScene S, const double* __restrict__ org, const double* __restrict__ dir,
                         const QHit* __restrict__ hits, double* __restrict__ t64, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    QHit h = hits[i];
    double t = (double)h.t;
    if (h.prim != 0xffffffffu) {
        double ox = org[3 * i], oy = org[3 * i + 1], oz = org[3 * i + 2];
        double dx = dir[3 * i], dy = dir[3 * i + 1], dz = dir[3 * i + 2];
        uint32_t kind = h.prim >> PRIM_KIND_SHIFT, idx = h.prim & PRIM_INDEX_MASK;
        if (kind == PK_SPHERE) {
            float4 s = S.spheres[idx];
            double cx = (double)s.x - ox, cy = (double)s.y - oy, cz = (double)s.z - oz;
            double tca = cx * dx + cy * dy + cz * dz;
            double ocs = cx * cx + cy * cy + cz * cz;
            double th = (double)s.w * (double)s.w - ocs + tca * tca;
            if (th > 0.0) {
                double hc = sqrt(th);
                double t1 = tca - hc, t2 = tca + hc;
                t = (t1 >= 1.0e-4) ? t1 : t2;
            }
        } else if (kind == PK_PLANE) {
            float4 p = S.planes[idx];
            double ndd = p.x * dx + p.y * dy + p.z * dz;
            if (ndd != 0.0)
                t = -((p.x * ox + p.y * oy + p.z * oz) + (double)p.w) / ndd;
        } else if (kind == PK_TRIANGLE) {
            int g = S.tri_global[idx];
            float4 nrm = S.tri_normal[g];
            double ndd = nrm.x * dx + nrm.y * dy + nrm.z * dz;
            if (ndd != 0.0)
                t = -((double)S.tri_v0[idx].w + (nrm.x * ox + nrm.y * oy + nrm.z * oz)) / ndd;
        }
    }
    t64[i] = t;
}

// --------------------------------------------------------------- launch --
static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

cudaError_t launch_refine(const DeviceScene& S, const double* org, const double* dir, QHit* hits, double* t64, int n,
                          cudaStream_t st)
{
    k_refine<<<cdiv(n > 0 ? n : 1, 256), 256, 0, st>>>(S, org, dir, hits, t64, n);
    return cudaGetLastError();
}

cudaError_t launch_camera(const DeviceScene& S, const int4* blocks, const int* block_off, int nblocks, int npix,
                          int width, int height, QRay* q, int* q_path, PathState* paths, int* q_count,
                          unsigned long long* stats, uint32_t* q_skip, cudaStream_t st)
{
    k_camera<<<cdiv(npix > 0 ? npix : 1, 256), 256, 0, st>>>(S, blocks, block_off, nblocks, width, height, q,
                                                             q_path, paths, q_count, stats, q_skip);
    return cudaGetLastError();
}

cudaError_t launch_load_rays(const double* org, const double* dir, int n, QRay* q, int* q_count, cudaStream_t st)
{
    k_load_rays<<<cdiv(n > 0 ? n : 1, 256), 256, 0, st>>>(org, dir, n, q, q_count);
    return cudaGetLastError();
}

cudaError_t launch_trace(const DeviceScene& S, bool any_hit, const QRay* q, const int* q_count, int* work,
                         QHit* hits, uint8_t* blocked, int stack_depth, int grid, uint32_t* err,
                         unsigned long long* stats, unsigned long long* wcount, int cap, const uint32_t* skips,
                         cudaStream_t st)
{
    const int block = 128;
    size_t smem = (size_t)stack_depth * block * sizeof(int);
    if (any_hit)
        k_trace<true><<<grid, block, smem, st>>>(S, q, q_count, work, hits, blocked, stack_depth, err, stats,
                                                 wcount, cap, skips);
    else
        k_trace<false><<<grid, block, smem, st>>>(S, q, q_count, work, hits, blocked, stack_depth, err, stats,
                                                  wcount, cap, skips);
    return cudaGetLastError();
}

cudaError_t launch_shade(const DeviceScene& S, int level, const QRay* q, const int* q_path, const QHit* hits,
                         const int* q_count, PathState* paths, float4* slot_contrib, QRay* sq, int* sq_slot,
                         int* sq_count, uint32_t* sq_skip, QRay* nq, int* nq_path, uint32_t* nq_skip, int* nq_count,
                         int max_queue, int max_shadow, int grid, uint32_t* err, unsigned long long* stats,
                         cudaStream_t st)
{
    k_shade<<<grid, 128, 0, st>>>(S, level, q, q_path, hits, q_count, paths, slot_contrib, sq, sq_slot, sq_count,
                                  sq_skip, nq, nq_path, nq_skip, nq_count, max_queue, max_shadow, err, stats);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const int* q_path, const int* q_count, int num_lights, const int* sq_slot,
                           const uint8_t* blocked, const int* sq_count, float4* slot_contrib, PathState* paths,
                           int grid, cudaStream_t st)
{
    k_mark_blocked<<<grid, 256, 0, st>>>(sq_slot, blocked, sq_count, slot_contrib);
    k_resolve<<<grid, 256, 0, st>>>(q_path, q_count, num_lights, slot_contrib, paths);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const PathState* paths, int npix, float4* out, cudaStream_t st)
{
    k_finalize<<<cdiv(npix > 0 ? npix : 1, 256), 256, 0, st>>>(paths, npix, out);
    return cudaGetLastError();
}

cudaError_t launch_zero(int* p, int n, cudaStream_t st)
{
    k_zero<<<cdiv(n, 256), 256, 0, st>>>(p, n);
    return cudaGetLastError();
}

}  // namespace povgpu
