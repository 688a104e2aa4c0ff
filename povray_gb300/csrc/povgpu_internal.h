// povgpu_internal.h -- device data layout shared by the host builder
// (povgpu_host.cpp) and the kernels (povgpu_kernels.cu).
//
// HBM layout (all arrays structure-of-arrays, 16-byte aligned):
//   nodes      BvhNode[num_nodes]      64 B: two child AABBs + two links
//   prim_refs  uint32[num_prim_refs]   leaf order; type in bits 28..31
//   tri_v0/e1/e2 float4[num_tris]      48 B per triangle, leaf order
//   tri_id     int32[num_tris]         leaf order -> (mesh-local) index
//   spheres    float4[num_spheres]     centre.xyz, radius
//   ...        per-primitive shading records, see DeviceScene
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace povgpu {

// Primitive kinds stored in the top 4 bits of a prim reference.
enum PrimKind : uint32_t {
    PK_SPHERE = 0u,
    PK_TRIANGLE = 1u,
    PK_BOX = 2u,
    PK_TORUS = 3u,
    PK_CSG = 4u,
    PK_PLANE = 5u,
};
constexpr uint32_t PRIM_KIND_SHIFT = 28;
constexpr uint32_t PRIM_INDEX_MASK = (1u << PRIM_KIND_SHIFT) - 1u;

// Two-wide BVH node (both children's boxes in one 64-byte record, loaded as
// four float4):  a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//                b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//                c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//                d = (link0, link1, -, -) as int bits
// link >= 0: inner node index.  link < 0: leaf, ~link = (first << 3) | (count-1)
// over prim_refs.
struct __align__(16) BvhNode {
    float4 a, b, c, d;
};
constexpr int LEAF_MAX_PRIMS = 8;

// Four-wide BVH node (128 B, the binary tree collapsed: each node takes the
// children and grandchildren with the largest surface area): child c's box
// in component c of the six slab vectors, child links as in BvhNode; an
// empty child has an inverted box and link BVH_EMPTY.
struct __align__(16) Bvh4Node {
    float4 lox, hix, loy, hiy, loz, hiz;
    int4   link;
    int4   pad;
};
constexpr int BVH_EMPTY = 0x7fffffff;   // no node: the traversal's stop value

// Shading record of one scene object (flattened object id).
struct __align__(16) ObjectShade {
    int32_t material;
    int32_t flags;
    int32_t type;
    int32_t mesh;       // mesh index or -1
};

// Material as the shading kernel reads it (float, pre-derived terms).
// DevMaterial::reflect_flags: a reflection at all, its reflectivity by
// ComputeFresnel at the ray's relative ior (transparent surfaces), and
// conserve_energy (the transmitted light loses what is reflected).
constexpr int REFL_ANY = 1, REFL_FRESNEL = 2, REFL_CONSERVE = 4;

struct __align__(16) DevMaterial {
    float4 pigment;         // rgb, filter
    float4 emission;        // emission + ambient * ambient_light, rgb
    float4 reflect;         // reflection_max rgb, falloff
    float4 reflect_min;     // reflection_min rgb, max(WeightMax(max), WeightMax(min))
    float diffuse;          // diffuse * brilliance_adjust
    float brilliance;
    float phong;
    float phong_size;
    float specular;
    float roughness;        // already inverted
    int32_t reflect_flags;  // REFL_ANY | REFL_FRESNEL | REFL_CONSERVE
    float   diffuse_raw;    // Finish->Diffuse, the radiosity ambient's factor (trace.cpp:898)
    int32_t pattern;        // pigment pattern + 1 (0: the plain pigment above)
    int32_t normal;         // normal perturbation + 1 (0: the raw normal)
    // transparency: the plain pigment's transmit, its opacity (the factor of
    // the layer's own light, TransColour::Opacity), whether it filters or
    // transmits at all
    float   transmit;
    float   opacity;
    int32_t see_through;    // SEE_PLAIN | SEE_PATTERN | SEE_LEGACY (0: opaque)
    float   diffuse_back;   // diffuse_back * brilliance_adjust: light from behind the surface
    float   metallic;       // highlights tinted by the pigment (ComputeMetallic)
    float   reflect_metallic;   // the reflectivity tinted likewise
};
// DevMaterial::see_through: the plain pigment filters or transmits; the
// pattern's colour map has an entry that does (filter, transmit and
// opacity taken per hit); LegacyOpacity (scenes before 3.7)
constexpr int SEE_PLAIN = 1, SEE_PATTERN = 2, SEE_LEGACY = 4;

// Pattern pigment (Compute_Pigment with a colour map): the inverse TRANSFORM
// as three columns (q_i = p . col_i + col_i.w), the gradient vector, the
// colour map.
struct __align__(16) DevPattern {
    float4 col[3];
    float4 gradient;        // xyz (normalised), agate_turb
    float4 turb;            // classic turbulence vector xyz, omega
    float4 wave;            // frequency, phase, exponent, lambda
    int4   kind;            // type, noise generator, entries, wave type
    int4   kind2;           // octaves, has turbulence, spiral arms, -
    float4 brick;           // brick_size xyz, mortar
    float4 crackle;         // crackle form xyz, metric
    float4 crackle2;        // crackle offset, quilted control0, control1, crackle solid (0 / 1)
    float  values[16];
    float4 colours[16];     // rgb, filter
    float  transmits[16];
};

// Normal perturbation (Perturb_Normal): the pattern's forward TRANSFORM as
// three rows of its 3x3 part (a normal enters the pattern's space as
// n'_i = n . fwd_i), the amount, the slope's delta, the pattern (0-based)
// and the no_bump_scale flag.
struct __align__(16) DevNormal {
    float4 fwd[3];
    float4 params;          // amount, delta, -5 * amount * (0.02 / delta), -
    int4   kind;            // pattern, dont_scale_bumps, -, -
};

// The scene's number of wave sources (SceneData::numberOfWaves).
#define POV_NUM_WAVES 10

// Noise tables in device memory (the reference's start-up tables).
struct DevNoise {
    const uint16_t* hash;   // 8192 (InitTextureTable)
    const float*    rtab;   // 534 (RTable, odd entries halved)
    const int32_t*  perm;   // 2 * (2048 + 1) (InitSolidNoise)
    const float4*   grad;   // 2 * (2048 + 1)
    const float4*   waves;  // POV_NUM_WAVES wave sources xyz, frequency w (Initialize_Waves)
    const float*    prand;  // 4100 entries of the pattern random table (gPatternRands)
};

struct __align__(16) DevLight {
    float4 center;          // xyz, kind
    float4 colour;          // rgb, -
    float4 axis1;           // area light: Axis1 xyz, |Axis1|
    float4 axis2;           // area light: Axis2 xyz, -
    int4   area;            // Area_Size1, Area_Size2, Adaptive_Level, bit0 Circular | bit1 Orient
    float4 dir;             // Direction (unit, points_at - center) xyz, w = Light_Type (LIGHT_*)
    float4 beam;            // Radius, Falloff, Coeff (tightness), Parallel (0 / 1)
    float4 fade;            // Fade_Distance, Fade_Power, -, -
};
constexpr int LIGHT_POINT = 1, LIGHT_SPOT = 2, LIGHT_SHADOWLESS = 3, LIGHT_CYLINDER = 4;
constexpr int AREA_MAX_POINTS = 64;   // area-light grid points the GPU path holds per shading point

struct __align__(16) DevMesh {
    int32_t tri_base;        // offset of this mesh's triangles in the global tables
    int32_t num_tris;
    int32_t object;          // flattened object id of the mesh
    int32_t normal_base;     // offset into the global normal table
};

// Axis-aligned box (Box without a transform): corners, object id and flags.
struct __align__(16) DevBox {
    float4 lo;      // xyz, w = object id (int bits)
    float4 hi;      // xyz, w = flags (int bits, bit0 inverted, bit1 BOX_CONTAINER)
};

// Torus in its own frame: the inverse TRANSFORM rows 0..3, columns 0..2
// (p_local = p . M^-1), radii, object id, flags.  FP64: the quartic is
// solved in double (source/core/shape/torus.cpp:241-362).
struct __align__(16) DevTorus {
    double inv[12];
    double R, r;
    int32_t object;
    int32_t flags;
    int32_t pad[2];
};

// CSG intersection / merge evaluated as one primitive over its leaf
// children (source/core/shape/csg.cpp:219-403).  Unions are flattened into
// their children at build time.
struct __align__(16) DevCsg {
    int32_t type;       // POV_OBJ_INTERSECTION or POV_OBJ_MERGE
    int32_t first;      // into csg_children
    int32_t count;
    int32_t object;
};
struct __align__(16) DevCsgChild {
    int32_t kind;       // PK_SPHERE, PK_BOX, PK_TORUS or PK_PLANE
    int32_t index;      // into the per-kind arrays
    int32_t flags;      // bit0 inverted
    int32_t object;
};

// One media container: a hollow axis-aligned box (its box primitive carries
// BOX_CONTAINER) holding one constant isotropic media sampled by method 3
// (MediaFunction::ComputeMedia, source/core/material/media.cpp:287-364).
struct __align__(16) DevMedia {
    float4 emission;     // rgb, AA_Threshold
    float4 scattering;   // rgb, 1 when any channel scatters
    float4 extinction;   // rgb (absorption + scattering), -
    int4   n;            // Intervals, sub-intervals (Min_Samples+1)/2, AA_Level, container primitive
    float4 phase;        // scattering type (1 isotropic .. 5 Henyey-Greenstein), eccentricity,
                         // container kind (0 box: n.w a box, 1 sphere: n.w a sphere), -
};
constexpr int BOX_CONTAINER = 2;         // DevBox flag: surface of a media container
constexpr int SPHERE_CONTAINER = 2;      // sphere_flags bit: surface of a media container
constexpr int OBJ_CONTAINER = 1 << 30;   // ObjectShade flag; container index in bits 16..23
constexpr int MAX_CONTAINERS = 8;
constexpr int MEDIA_MAX_INTERVALS = 32;  // Intervals the GPU path holds per ray segment
constexpr int MEDIA_MAX_AA_LEVEL = 4;
constexpr int MEDIA_MAX_NODES = (1 << MEDIA_MAX_AA_LEVEL) - 1;   // sample tree nodes per sub-interval

// Per-ray state of a wavefront queue in scenes with media containers: the
// ray's trace level (bits 0..7) and the container it travels in, plus one
// (bits 8..15; 0 = none).  Transmitted rays keep their parent's level.
__host__ __device__ __forceinline__ int ray_state(int level, int medium) { return level | ((medium + 1) << 8); }
__host__ __device__ __forceinline__ int state_level(int s) { return s & 0xff; }
__host__ __device__ __forceinline__ int state_medium(int s) { return ((s >> 8) & 0xff) - 1; }

struct DeviceScene {
    const Bvh4Node* nodes;
    const uint32_t* prim_refs;
    int32_t         root;           // BVH_EMPTY = no finite primitives
    // triangles (leaf order)
    const float4*   tri_v0;
    const float4*   tri_e1;
    const float4*   tri_e2;
    const int32_t*  tri_global;     // leaf-order slot -> global triangle index
    // triangle shading (global triangle order)
    const int4*     tri_shade;      // n1, n2, n3 (global normal index), flags (bit0 smooth)
    const float4*   tri_normal;     // geometric normal xyz, mesh object id (int bits)
    const int32_t*  tri_local;      // global triangle -> triangle index within its mesh
    const float4*   normals;        // smooth normals (normalised like the parser)
    // spheres
    const float4*   spheres;        // centre, radius
    const int32_t*  sphere_obj;     // object id
    // planes (infinite, tested by every ray)
    const float4*   planes;         // normal xyz, Distance
    const int32_t*  plane_obj;
    int32_t         num_planes;
    // boxes, tori, CSG
    const DevBox*      boxes;
    const DevTorus*    tori;
    const float4*      tori32;      // per torus 4 float4: local x, y, z rows of the inverse (FP32), (R, r, 0, 0)
    const DevCsg*      csgs;
    const DevCsgChild* csg_children;
    const int32_t*     sphere_flags;   // bit0 inverted (spheres inside CSG)
    int32_t            has_full_prims; // tori or CSG present: full traversal variant
    // transparency: per object its interior id (bits 0-15) and whether the
    // top-level object it belongs to is opaque (bit 16: the OPAQUE_FLAG of
    // the CSG a child belongs to); per interior (ior, fade_distance,
    // fade_power, old_refract) and (fade colour rgb, 0); the atmosphere's ior
    const int32_t*     obj_interior;
    const float4*      interiors;
    float              atm_ior;
    int32_t            transparent;
    // FP64 geometry as the parser stores it, read only by the parity
    // re-solve (k_refine): centre+radius per sphere, 6 corners per box
    const double*      spheres64;
    const double*      boxes64;
    // objects, materials, lights
    const ObjectShade* objects;
    const DevMaterial* materials;
    const DevLight*    lights;
    int32_t         num_lights;
    int32_t         num_area_lights;
    // media containers
    const DevMedia* medias;         // one per container
    int32_t         num_containers;
    // pattern pigments
    const DevPattern* patterns;
    const DevNormal*  tnormals;       // normal perturbations (TNORMAL)
    DevNoise          noise;
    int32_t         max_trace_level;
    float           adc_bailout;
    float4          background;
    // camera
    double          cam_loc[3], cam_dir[3], cam_right[3], cam_up[3];
    // the same direction, right and up vectors as double-floats (each
    // component hi + lo, two floats, set by set_camera_ff)
    float           cam_ff[18];
};

// DeviceScene::cam_ff from the FP64 camera vectors.
inline void set_camera_ff(DeviceScene& S)
{
    const double* v[3] = {S.cam_dir, S.cam_right, S.cam_up};
    for (int a = 0; a < 3; a++)
        for (int k = 0; k < 3; k++) {
            const float hi = (float)v[a][k];
            S.cam_ff[6 * a + 2 * k] = hi;
            S.cam_ff[6 * a + 2 * k + 1] = (float)(v[a][k] - (double)hi);
        }
}

// One ray of a wavefront queue (32 B) + its path slot.
struct __align__(16) QRay {
    float4 org;     // xyz, tmin
    float4 dir;     // xyz, tmax
};

// Closest-hit record (16 B).
struct __align__(16) QHit {
    float    t;
    uint32_t prim;   // prim reference (kind|index), 0xffffffff = miss
    float    u, v;   // triangle barycentrics
};

// Deferred torus tests of one traversal launch.  The traversal kernel
// appends each (ray, torus) pair that passes the FP32 pre-cull to `cand`
// (ray index | bit 31 when the torus is the ray's own origin surface, torus
// index) instead of running the FP64 quartic in the one lane that met it;
// k_torus_solve then solves the pairs one per thread, so a warp's FP64
// instructions run with all 32 lanes instead of the few that reached a
// torus together.  Closest hits keep the nearest root per ray in `key`
// (depth bits << 32 | prim reference, atomicMin), merged into the hits
// afterwards; any-hit rays set their blocked byte.  Pairs beyond `cap` are
// solved in line, as without deferral -- or, with `ovf` set (scenes whose
// CSGs have no torus children), the traversal runs its torus-free variant
// and lists such rays in `ovf` for a second launch of the ordinary one.
// count, ovf_count and ovf_work are three consecutive ints, zeroed per launch.
struct TorusDefer {
    uint2*              cand;
    int*                count;
    int                 cap;
    unsigned long long* key;   // per ray (closest hits)
    int*                ovf;       // rays to trace again with the full variant
    int*                ovf_count;
    int*                ovf_work;  // the second launch's work counter
    int                 ovf_cap;
};

// Per-path state (one path per image sample).
struct __align__(16) PathState {
    float4 colour;      // accumulated rgb, transm
    float4 throughput;  // rgb, weight
};

// ------------------------------------------------------------ radiosity --
// One radiosity ambient query (RadiosityFunction::ComputeAmbient): a hit
// point, its ray-facing normal, the query weight, the factor the ambient
// colour is added with (pigment * Diffuse * path throughput), the path or
// gather ray it adds to, and the surface a gather from it starts on.
struct __align__(16) RadQuery {
    float4   p;         // xyz, weight (ray weight * largest possible contribution)
    float4   n;         // xyz, -
    float4   factor;    // rgb, -
    int32_t  path;
    uint32_t prim, aux;
    int32_t  pad;
};

// One cached radiosity sample (ot_block_struct, octree.h:86-104).
struct __align__(16) RadBlock {
    float4 p;           // Point, Harmonic_Mean_Distance
    float4 n;           // S_Normal, Nearest_Distance
    float4 tn;          // To_Nearest_Surface, Quality
    float4 ill;         // Illuminance, Bounce_Depth (int bits)
};

// The sample cache in device memory: blocks, and the octree nodes as an
// open-addressing hash (64-bit node key -> slot).  Each node's blocks sit
// contiguously in `members` (segment seg_off/seg_cnt of the node's slot),
// rebuilt from every block's slot after blocks are added, so a lookup reads
// a node's blocks with independent loads instead of chasing a list.
struct RadCacheView {
    RadBlock*           blocks;
    float4*             quick;      // per block: point, harmonic mean distance (the quick reuse test)
    int32_t*            bslot;      // per block: the hash slot of its node
    int32_t*            count;      // blocks in use (device word)
    int32_t             cap;
    unsigned long long* keys;       // 0 = empty slot
    int32_t*            seg_off;    // per slot: first entry of the node's blocks in members
    int32_t*            seg_cnt;    // per slot: number of the node's blocks
    int32_t*            seg_cur;    // per slot: rebuild cursor / allocation flag
    int32_t*            members;    // block indices grouped by node
    int32_t*            seg_total;  // rebuild: entries allocated (device word)
    uint32_t            mask;       // slots - 1
    int32_t*            size_range; // per bounce depth d: [2d] smallest, [2d+1] largest node size in use
    uint32_t*           occupancy;  // one bit per hashed node key: set once the node holds a block
    uint32_t            occ_mask;   // bits - 1
};

// Settings of one bounce depth for the query and gather kernels
// (RadiosityRecursionSettings, radiosity.cpp:177-294, plus the task's state).
struct RadParams {
    int32_t depth;
    int32_t final_trace;        // final trace (1) or pretrace (0)
    int32_t always_sample;
    int32_t reuse_count;
    int32_t rays_per_sample;
    float   error_bound;        // errorBound, times low_error_factor in pretrace
    float   error_bound_factor;
    float   min_reuse_factor, max_reuse_factor, address_factor;
    float   gather_weight;      // weight of this depth's sample rays
    float   gray, brightness;
    float   adc;                // radiosity adc_bailout
};

// What the shading kernel does for radiosity: emit an ambient query per
// hit (rq non-null) when the hit's largest possible contribution beats
// `adc`; `gather` marks radiosity sample rays, shaded by the radiosity
// Trace (no highlights, area lights as point lights, no reflection rays).
struct ShadeRad {
    RadQuery* rq;
    int32_t*  rq_count;
    int32_t   rq_cap;
    float     adc;
    int32_t   gather;
};

// What the level loop does for media containers (all null without them):
// per-ray state of the current and next queue, and the medium each shadow
// ray starts in.
struct ShadeMedia {
    const int32_t* q_state;
    int32_t*       nq_state;
    int32_t*       sq_medium;
    // transparent scenes: each queued ray's interior list (rin_*), handed
    // to its shadow rays and to the transmitted or refracted ray
    const uint64_t* q_rin;
    uint64_t*       nq_rin;
    uint64_t*       sq_rin;
    // transparent surfaces that also reflect: a hit may queue two rays, so
    // each ray carries its own throughput (rgb, weight; q_thr NULL: the
    // path's, for the camera rays) and paths take their colour by atomic
    // adds; nq_cap is the next queue's capacity (0: the current one's)
    const float4* q_thr;
    float4*       nq_thr;
    int32_t       branching;
    int32_t       nq_cap;
};

// A ray's interior list (Ray::GetInteriors): the ids of the interiors it
// travels inside, innermost last, as bytes 1..7 of a 64-bit word whose
// byte 0 holds the count.
constexpr int RIN_MAX = 7;
__host__ __device__ __forceinline__ int rin_count(uint64_t r) { return (int)(r & 0xffu); }
__host__ __device__ __forceinline__ int rin_get(uint64_t r, int k) { return (int)((r >> (8 * (k + 1))) & 0xffu); }
__host__ __device__ __forceinline__ uint64_t rin_set(uint64_t r, int k, int id)
{
    const int sh = 8 * (k + 1);
    return (r & ~(0xffull << sh)) | ((uint64_t)(id & 0xff) << sh);
}
__host__ __device__ __forceinline__ int rin_find(uint64_t r, int id)
{
    for (int k = 0; k < rin_count(r); k++)
        if (rin_get(r, k) == id)
            return k;
    return -1;
}
__host__ __device__ __forceinline__ uint64_t rin_remove(uint64_t r, int k)
{
    const int n = rin_count(r);
    for (int j = k; j + 1 < n; j++)
        r = rin_set(r, j, rin_get(r, j + 1));
    r = rin_set(r, n - 1, 0);
    return (r & ~0xffull) | (uint64_t)(n - 1);
}
// false when the list is full (the caller flags the device error)
__host__ __device__ __forceinline__ bool rin_append(uint64_t& r, int id)
{
    const int n = rin_count(r);
    if (n >= RIN_MAX)
        return false;
    r = (rin_set(r, n, id) & ~0xffull) | (uint64_t)(n + 1);
    return true;
}

// Device error word bits.
enum DevError : uint32_t {
    DE_STACK_OVERFLOW = 1u,
    DE_ITERATION_CAP  = 2u,
    DE_QUEUE_OVERFLOW = 4u,
    DE_CACHE_FULL     = 8u,
    DE_INTERIORS      = 16u,   // a ray inside more than RIN_MAX interiors
};

// Counters (device, uint64).
enum StatIdx {
    ST_RAYS = 0,
    ST_SHADOW_TESTS = 1,
    ST_SHADOW_SUCCEEDED = 2,
    ST_REFLECTED = 3,
    ST_SAMPLES = 4,
    ST_TRANSMITTED = 5,
    ST_MEDIA_SAMPLES = 6,
    ST_REFRACTED = 7,
    ST_INTERNAL_REFLECTED = 8,
    ST_COUNT = 10,
};

}  // namespace povgpu
