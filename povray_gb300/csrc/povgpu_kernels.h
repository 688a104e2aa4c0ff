// povgpu_kernels.h -- host-callable launchers of the kernels in
// povgpu_kernels.cu (all asynchronous on the given stream).
#pragma once
#include "povgpu.h"
#include "povgpu_internal.h"

namespace povgpu {

// mode 0: pixel centres per block, 1: block corners, 2: explicit positions
cudaError_t launch_camera(const DeviceScene& S, int mode, const int4* blocks, const int* block_off, int nblocks,
                          const double2* pos, const int* npos, int max_samples, int width, int height, QRay* q,
                          int* q_path, PathState* paths, int* q_count, unsigned long long* stats, uint2* q_skip,
                          float2* tab /* width + height + 2 double-floats (modes 0, 1) */,
                          cudaStream_t st);
cudaError_t launch_load_rays(const double* org, const double* dir, int n, QRay* q, int* q_count, cudaStream_t st);
cudaError_t launch_trace(const DeviceScene& S, bool any_hit, const QRay* q, const int* q_count, int* work,
                         QHit* hits, uint8_t* blocked, int stack_depth, int grid, uint32_t* err,
                         unsigned long long* stats, unsigned long long* wcount, int cap, const uint2* skips,
                         cudaStream_t st, int block = 128, int occ = 0, const TorusDefer* defer = nullptr);
cudaError_t launch_shade(const DeviceScene& S, int level, int max_level, const QRay* q, const int* q_path,
                         const QHit* hits,
                         const int* q_count, PathState* paths, float4* slot_contrib, QRay* sq, int* sq_slot,
                         int* sq_count, uint2* sq_skip, QRay* nq, int* nq_path, uint2* nq_skip, int* nq_count,
                         int max_queue, int max_shadow, QRay* aq, int* aq_slot, uint2* aq_skip, int* aq_count,
                         int max_area, const ShadeRad& rad, const ShadeMedia& med, const int* order, int grid, uint32_t* err,
                         unsigned long long* stats, cudaStream_t st);
// Bins the shade queue by material (SHADE_BINS keys): keys[cap] bytes,
// hist[2 * SHADE_BINS] ints (counts, then cursors), order[cap] receives the
// binned item order for k_shade.
constexpr int SHADE_BINS = 256;
cudaError_t launch_shade_bins(const DeviceScene& S, const QHit* hits, const int* q_count, int cap, uint8_t* keys,
                              int* hist, int* order, int grid, cudaStream_t st);
cudaError_t launch_fill_int(int* a, const int* count, int cap, int value, int grid, cudaStream_t st);
// 8-bit RGB of n RGBT pixels; thr[v] (v < 255) = the midpoint of decoded levels v and v+1
cudaError_t launch_encode_u8(const float4* rgbt, long long n, int curve, const float* thr, uint8_t* out, int grid,
                             cudaStream_t st);
// Shadow rays through media containers (scenes with containers: replaces
// the any-hit trace of the shadow queue).
cudaError_t launch_shadow_through(const DeviceScene& S, const QRay* sq, const int* sq_slot, const uint2* sq_skip,
                                  const int* sq_medium, const int* sq_count, int cap, int* work, uint8_t* blocked,
                                  float4* slot_contrib, bool media_on, int stack_depth, int grid, uint32_t* err,
                                  unsigned long long* stats, cudaStream_t st);
// Shadow rays through transparent surfaces: each ray's blocked byte and
// its light term scaled by the filters it crossed (sq_rin: each shadow
// ray's interior list, from its eye ray).
cudaError_t launch_shadow_filter(const DeviceScene& S, const QRay* sq, const int* sq_slot, const uint2* sq_skip,
                                 const uint64_t* sq_rin, const int* sq_count, int cap, int* work, uint8_t* blocked,
                                 float4* slot_contrib, int stack_depth, int grid, uint32_t* err,
                                 unsigned long long* stats, cudaStream_t st);
// Media of the queue's rays inside containers, applied to their paths
// before shading: list the rays (mcount zeroed by the caller); per chunk of
// listed rays, the sample rounds into cbuf and the per-interval sums (counts:
// the round list's count, then the rounds' work counter); then
// combine every listed ray's intervals into its path.
cudaError_t launch_media_list(const int* q_state, const QHit* hits, const int* q_count, int cap, int* mlist,
                              int* mcount, int grid, cudaStream_t st);
cudaError_t launch_media_chunk(const DeviceScene& S, const QRay* q, const int* q_state, const QHit* hits,
                               const int* mlist, int first, int nseg, int NI, int SMAX, int max_sub, int max_levels,
                               float4* cbuf, int* listA, int* listB, int* counts, int list_cap, int stamp,
                               float4* te, float4* od, int stack_depth, int grid, uint32_t* err,
                               unsigned long long* stats, cudaStream_t st);
cudaError_t launch_media_combine(const DeviceScene& S, const int* q_state, const int* q_path, const QHit* hits,
                                 const int* mlist, const int* mcount, int cap, int NI, const float4* te,
                                 const float4* od, PathState* paths, int grid, cudaStream_t st);
cudaError_t launch_area_shadow(const DeviceScene& S, const QRay* aq, const int* aq_slot, const uint2* aq_skip,
                               const int* aq_count, int cap, float4* slot_contrib, int stack_depth, int grid,
                               uint32_t* err, unsigned long long* stats, cudaStream_t st);
cudaError_t launch_resolve(const int* q_path, const int* q_count, int num_lights, const int* sq_slot,
                           const uint8_t* blocked, const int* sq_count, float4* slot_contrib, PathState* paths,
                           int grid, int cap_rays, int cap_shadow, cudaStream_t st, bool branching = false);
cudaError_t launch_finalize(const PathState* paths, const int* count, int max_samples, const int* slot, float4* out,
                            cudaStream_t st);
cudaError_t launch_refine(const DeviceScene& S, const double* org, const double* dir, QHit* hits, double* t64, int n,
                          cudaStream_t st);
cudaError_t launch_aa_init(const int4* blocks, const int* pix_off, const int* corner_off, int nblocks, int npix,
                           const float4* corners, int G, int MW, float4* grid, uint32_t* mask, uint32_t* subdiv,
                           int2* pix_xy, int4* cells, int* ncells, int root_level, cudaStream_t st);
cudaError_t launch_aa_classify(const int4* cells, const int* ncells, int cap, int G, int MW, const float4* grid,
                               uint32_t* mask, uint32_t* subdiv, const int2* pix_xy, double thr, double subsize,
                               double2* spos, int* sslot, int* nsamples, int scap, int4* next, int* nnext, int ncap,
                               uint32_t* err, int grid_blocks, cudaStream_t st);
cudaError_t launch_aa_resolve(const float4* grid, const uint32_t* subdiv, int npix, int G, int depth, float4* out,
                              cudaStream_t st);

// Fixed scratch of pov_gpu_trace_rays_static (a file-scope device array in
// povgpu_kernels.cu).  Header: work counters at 0, error word at 64,
// statistics at 128 -- all must be zero before the first launch of a call.
// Per-ray regions follow, each sized for STATIC_MAX_RAYS rays.
constexpr int STATIC_MAX_RAYS = 65536;
constexpr size_t STATIC_OFF_COUNTERS = 0;
constexpr size_t STATIC_OFF_ERR = 64;
constexpr size_t STATIC_OFF_STATS = 128;
constexpr size_t STATIC_HEADER_BYTES = 256;
constexpr size_t STATIC_OFF_ORG = STATIC_HEADER_BYTES;                               // double[3 * max]
constexpr size_t STATIC_OFF_DIR = STATIC_OFF_ORG + sizeof(double) * 3 * STATIC_MAX_RAYS;  // double[3 * max]
constexpr size_t STATIC_OFF_RAYS = STATIC_OFF_DIR + sizeof(double) * 3 * STATIC_MAX_RAYS; // QRay[max]
constexpr size_t STATIC_OFF_HITS = STATIC_OFF_RAYS + sizeof(QRay) * STATIC_MAX_RAYS;      // QHit[max]
constexpr size_t STATIC_OFF_T64 = STATIC_OFF_HITS + sizeof(QHit) * STATIC_MAX_RAYS;       // double[max]
constexpr size_t STATIC_OFF_OUT = STATIC_OFF_T64 + sizeof(double) * STATIC_MAX_RAYS;      // PovGpuHit[max]
constexpr size_t STATIC_SCRATCH_BYTES = STATIC_OFF_OUT + 16 * (size_t)STATIC_MAX_RAYS;     // 7.5 MiB + 256 B

// Device address of that scratch on the current device (looked up once per
// device, then cached).  Call with `device` current.
cudaError_t static_ray_scratch(int device, unsigned char** out);
cudaError_t launch_hits_abi(const DeviceScene& S, const QHit* hits, const double* t64, int n, PovGpuHit* out,
                            cudaStream_t st);

}  // namespace povgpu
