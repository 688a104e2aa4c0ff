// povgpu_radiosity.h -- launchers of the radiosity kernels
// (povgpu_radiosity.cu), all asynchronous on the given stream.
#pragma once
#include "povgpu_internal.h"

namespace povgpu {

constexpr int RAD_DIRECTIONS = 1600;   // RADIOSITY_MAX_SAMPLE_DIRECTIONS (radiosity.h:78)
constexpr int RAD_LEVELS = 4;          // bounce depths with their own buffers and cache nodes

// Radiosity counters (device, uint64).
enum RadStatIdx {
    RST_REUSED = 0,     // queries answered from the cache
    RST_GATHERS0 = 1,   // samples gathered at bounce depth 0
    RST_GATHERS1 = 2,   // ... at depth 1 and deeper
    RST_NIC = 3,        // queries the neural cache answered
    RST_COUNT = 4,
};

// The Halton(2,3) cosine-weighted direction pool, 3 floats per direction.
cudaError_t rad_upload_directions(const float* xyz3);

// Rebuilds the node segments from every block's slot (after blocks were added).
cudaError_t launch_seg_rebuild(const RadCacheView& C, int grid, cudaStream_t st);
cudaError_t launch_rad_query(const DeviceScene& S, const RadCacheView& C, const RadParams& R, const RadQuery* queries,
                             const int* open, int n_open, int cap, int round, int last_round, float4* out,
                             float4* partial, unsigned long long* claims, uint32_t claim_mask, int* seeds,
                             int* n_seeds, int* next, int* n_next, unsigned long long* rstats, uint32_t* err,
                             int grid, cudaStream_t st);
cudaError_t launch_gather_rays(const RadQuery* queries, const int* seeds, int ns, int count, int base, float weight,
                               QRay* rays, int* q_path, uint2* skips, PathState* paths, float* quality, int* q_count,
                               unsigned long long* stats, int grid, cudaStream_t st);
cudaError_t launch_first_hit(const QHit* hits, const int* q_count, int cap, float* first_t, int grid, cudaStream_t st);
cudaError_t launch_rad_apply(const RadQuery* queries, const int* n_queries, int cap, const float4* amb,
                             PathState* paths, float* quality, int grid, cudaStream_t st);
// Files blocks [first, first + n) of the cache, written there by the host
// (a loaded cache file), into their octree nodes; address_factor[d] is
// bounce depth d's (RadParams::address_factor).
cudaError_t launch_rad_file(const RadCacheView& C, const float* address_factor, int first, int n, uint32_t* err,
                            cudaStream_t st);
// Answers of the neural cache (pred[i] for query seeds[i]) into out[].
cudaError_t launch_rad_nic_answer(const RadParams& R, const int* seeds, int ns, const float4* pred, float4* out,
                                  unsigned long long* rstats, int grid, cudaStream_t st);
cudaError_t launch_gather_reduce(const DeviceScene& S, const RadCacheView& C, const RadParams& R,
                                 const RadQuery* queries, const int* seeds, int ns, int base, const float* first_t,
                                 const PathState* paths, const float* quality, const float4* partial, float4* out,
                                 unsigned long long* rstats, uint32_t* err, int grid, cudaStream_t st);

}  // namespace povgpu
