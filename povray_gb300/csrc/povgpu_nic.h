// povgpu_nic.h -- the neural irradiance cache's kernels (povgpu_nic.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace povgpu {
namespace nic {

constexpr int FEAT = 102;   // 6 coordinates + sin/cos of 8 frequencies each
constexpr int K1 = 112;     // input width padded to the MMA's K step
constexpr int HID = 64;     // hidden width (four hidden layers)
constexpr int NOUT = 3;     // RGB
constexpr int NO = 16;      // output width padded to the MMA's N step
constexpr int TILE = 128;   // samples per CTA tile (MMA M)

// FP32 parameter vector: W1 [64x112], b1, W2 [64x64], b2, W3, b3, W4, b4,
// W5 [16x64] (rows 3..15 zero), b5 [16] (3..15 zero); weights row-major
// [out][in].
constexpr int P_W1 = 0, P_B1 = P_W1 + HID * K1, P_W2 = P_B1 + HID, P_B2 = P_W2 + HID * HID, P_W3 = P_B2 + HID,
              P_B3 = P_W3 + HID * HID, P_W4 = P_B3 + HID, P_B4 = P_W4 + HID * HID, P_W5 = P_B4 + HID,
              P_B5 = P_W5 + NO * HID, NPARAM = P_B5 + NO;
static_assert(P_B2 - P_B1 == P_B3 - P_B2 && P_B3 - P_B2 == P_B4 - P_B3, "uniform hidden-layer stride");

// Samples: sample i is element idx[i] (or i) of pos / nrm / target, each
// `stride` float4s apart; the point is scaled by (p - lo) * scale - 1.
struct NicIO {
    const float4* pos;
    const float4* nrm;
    const float4* target;   // training: illuminance
    int           stride;
    const int*    idx;
    int           n;
    float4*       out;      // inference: prediction of sample i at out[i]
    float3        lo, scale;
};

// The BF16 weights as the kernels' shared-memory tiles want them (the
// "weight image", written by the Adam step): the forward tiles W1..W5 then
// the transposed tiles W2^T..W5^T of the backward pass, each K-major in
// 8x16-byte core matrices, so a CTA fetches them with one bulk copy each.
constexpr uint32_t WIMG_FWD = (HID * K1 + 3 * HID * HID + NO * HID) * 2;
constexpr uint32_t WIMG_BWD = (3 * HID * HID + NO * HID) * 2;
constexpr uint32_t WIMG_BYTES = WIMG_FWD + WIMG_BWD;

size_t smem_bytes(bool train);
cudaError_t launch_forward(const NicIO& io, const unsigned char* wimg, const float* params, uint32_t* err, int grid,
                           cudaStream_t st);
// Gradient of (1/batch) * sum (p - y)^2 / (p^2 + 0.01) over io's samples:
// CTA b writes its part to grad[b * NPARAM ...] and loss[b], for the
// train_slices(io.n, grid) CTAs the launch uses (the buffers hold that many
// slices).  Nothing is accumulated across launches.
int train_slices(int n, int grid);
cudaError_t launch_train(const NicIO& io, const unsigned char* wimg, const float* params, float* grad, float* loss,
                         float inv_batch, uint32_t* err, int grid, cudaStream_t st);
// Adam step on the gradient summed (in slice order) from `slices` slices.
cudaError_t launch_adam(float* params, float* m, float* v, const float* grad, int slices, unsigned char* wimg,
                        float lr, int step, cudaStream_t st);
// The slices' sum into grad[NPARAM] and *loss.
cudaError_t launch_reduce(const float* grad_slices, const float* loss_slices, int slices, float* grad, float* loss,
                          cudaStream_t st);
cudaError_t launch_to_bf16(const float* params, unsigned char* wimg, cudaStream_t st);

}  // namespace nic
}  // namespace povgpu
