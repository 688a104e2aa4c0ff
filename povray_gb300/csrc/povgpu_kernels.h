// povgpu_kernels.h -- host-callable launchers of the kernels in
// povgpu_kernels.cu (all asynchronous on the given stream).
#pragma once
#include "povgpu_internal.h"

namespace povgpu {

cudaError_t launch_camera(const DeviceScene& S, const int4* blocks, const int* block_off, int nblocks, int npix,
                          int width, int height, QRay* q, int* q_path, PathState* paths, int* q_count,
                          unsigned long long* stats, uint32_t* q_skip, cudaStream_t st);
cudaError_t launch_load_rays(const double* org, const double* dir, int n, QRay* q, int* q_count, cudaStream_t st);
cudaError_t launch_trace(const DeviceScene& S, bool any_hit, const QRay* q, const int* q_count, int* work,
                         QHit* hits, uint8_t* blocked, int stack_depth, int grid, uint32_t* err,
                         unsigned long long* stats, unsigned long long* wcount, int cap, const uint32_t* skips,
                         cudaStream_t st);
cudaError_t launch_shade(const DeviceScene& S, int level, const QRay* q, const int* q_path, const QHit* hits,
                         const int* q_count, PathState* paths, float4* slot_contrib, QRay* sq, int* sq_slot,
                         int* sq_count, uint32_t* sq_skip, QRay* nq, int* nq_path, uint32_t* nq_skip, int* nq_count,
                         int max_queue, int max_shadow, int grid, uint32_t* err, unsigned long long* stats,
                         cudaStream_t st);
cudaError_t launch_resolve(const int* q_path, const int* q_count, int num_lights, const int* sq_slot,
                           const uint8_t* blocked, const int* sq_count, float4* slot_contrib, PathState* paths,
                           int grid, cudaStream_t st);
cudaError_t launch_finalize(const PathState* paths, int npix, float4* out, cudaStream_t st);
cudaError_t launch_zero(int* p, int n, cudaStream_t st);
cudaError_t launch_refine(const DeviceScene& S, const double* org, const double* dir, QHit* hits, double* t64, int n,
                          cudaStream_t st);

}  // namespace povgpu
