// povgpu_nic.cu -- neural irradiance cache: a small MLP that predicts the
// radiosity illuminance at (point, normal), trained online on the samples the
// radiosity pretrace gathered.  No reference counterpart.
//
// Model: 102 input features (the point scaled to [-1,1] in the training
// samples' bounding box, the normal, and sin/cos(2^k pi x / 8) of those six
// coordinates for k = 0..7), zero-padded to 112; four hidden layers of 64
// with ReLU; 3 outputs (padded to 16).  Weights BF16, accumulation FP32.
//
// Every GEMM runs on the 5th-generation tensor cores: one CTA of 128 threads
// takes a tile of 128 samples (thread t = sample t = TMEM lane t); the layer
// input is a BF16 K-major tile in shared memory, the weights another, one
// elected thread issues tcgen05.mma (M=128, N=64 or 16, K=16 per
// instruction) into a TMEM accumulator and commits to an mbarrier; the
// epilogue reads its lane with tcgen05.ld, adds the bias, applies ReLU and
// writes the next layer's input tile.  Training adds the backward pass on
// the same units: dH = dZ * W (A = dZ tile, B = W^T tile) and
// dW = dZ^T * H (A = dZ^T tile, M = 128 padded output rows, K = the 128
// samples, B = H^T tile), the transposed tiles written by the threads.
// Each CTA keeps its own gradient slice in global memory (the sum over its
// tiles, in tile order); the Adam step sums the slices in CTA order, so a
// training step gives the same parameters on every run.
#include "povgpu_internal.h"
#include "povgpu_nic.h"
#include "povgpu_umma.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace povgpu {
namespace nic {

namespace {

// shared-memory map (bytes); every tile offset is a multiple of 128
constexpr uint32_t SZ_W1 = HID * K1 * 2, SZ_WH = HID * HID * 2, SZ_W5 = NO * HID * 2;
constexpr uint32_t OFF_W1 = 0, OFF_W2 = OFF_W1 + SZ_W1, OFF_W3 = OFF_W2 + SZ_WH, OFF_W4 = OFF_W3 + SZ_WH,
                   OFF_W5 = OFF_W4 + SZ_WH, END_W = OFF_W5 + SZ_W5;
// backward: transposed weights in the same region ([in][out], K-major over out)
constexpr uint32_t OFF_W2T = 0, OFF_W3T = OFF_W2T + SZ_WH, OFF_W4T = OFF_W3T + SZ_WH, OFF_W5T = OFF_W4T + SZ_WH;
constexpr uint32_t OFF_A0 = END_W, SZ_A0 = TILE * K1 * 2, OFF_A1 = OFF_A0 + SZ_A0, SZ_A1 = TILE * HID * 2;
constexpr uint32_t END_P_FWD = OFF_A1 + SZ_A1;
// backward: dZ^T (128 padded output rows x 128 samples) and dZ (128 samples x out) in the same region
constexpr uint32_t OFF_DZT = OFF_A0, SZ_DZT = TILE * TILE * 2, OFF_DZ = OFF_DZT + SZ_DZT;
constexpr uint32_t END_P_TRAIN = OFF_DZ + TILE * HID * 2;
// training: transposed activations (features x 128 samples, K-major over samples)
constexpr uint32_t OFF_X0T = END_P_TRAIN, OFF_H1T = OFF_X0T + K1 * TILE * 2, OFF_H2T = OFF_H1T + HID * TILE * 2,
                   OFF_H3T = OFF_H2T + HID * TILE * 2, OFF_H4T = OFF_H3T + HID * TILE * 2,
                   END_T = OFF_H4T + HID * TILE * 2;

template <bool TRAIN> struct Map {
    static constexpr uint32_t BIAS = TRAIN ? END_T : END_P_FWD;          // 4*64 + 16 floats
    static constexpr uint32_t BGRAD = BIAS + (4 * HID + NO) * 4;          // 4 warps x 64 floats
    static constexpr uint32_t LOSS = BGRAD + 4 * HID * 4;                 // 8 floats (1 + 4 warps used)
    static constexpr uint32_t MBAR = LOSS + 32;                           // 8-byte aligned
    static constexpr uint32_t CBAR = MBAR + 8;                            // bulk-copy barrier
    static constexpr uint32_t TSLOT = CBAR + 8;
    static constexpr uint32_t BYTES = TSLOT + 8;
    static constexpr uint32_t TMEM_COLS = TRAIN ? 256 : 64;
};
static_assert(Map<true>::BYTES <= 227 * 1024, "training tile exceeds shared memory");
static_assert(END_W == WIMG_FWD && OFF_W5T + NO * HID * 2 == WIMG_BWD, "weight image and tile map differ");
static_assert(WIMG_FWD % 16 == 0 && WIMG_BWD % 16 == 0, "bulk copies move multiples of 16 bytes");
static_assert(END_W >= OFF_W5T + NO * HID * 2, "transposed weights overflow the weight region");

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v)
{
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}
__device__ __forceinline__ float ld_bf16(const unsigned char* base, uint32_t off)
{
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(base + off));
}

// Byte offset of weight (r, k) of layer l (rows x cols, row-major [out][in])
// in the weight image: its forward tile, and for l >= 1 its transposed tile.
__device__ __forceinline__ uint32_t wimg_fwd(int l, int r, int k)
{
    const uint32_t base[5] = {OFF_W1, OFF_W2, OFF_W3, OFF_W4, OFF_W5};
    return base[l] + umma::kmajor_offset(r, k, l == 0 ? K1 : HID);
}
__device__ __forceinline__ uint32_t wimg_bwd(int l, int r, int k)
{
    const uint32_t base[5] = {0, OFF_W2T, OFF_W3T, OFF_W4T, OFF_W5T};
    return WIMG_FWD + base[l] + umma::kmajor_offset(k, r, l == 4 ? NO : HID);
}

// Layer, row and column of weight parameter i; false for a bias.
__device__ __forceinline__ bool weight_of(int i, int& l, int& r, int& k)
{
    const int wb[5] = {P_W1, P_W2, P_W3, P_W4, P_W5}, we[5] = {P_B1, P_B2, P_B3, P_B4, P_B5};
    for (l = 0; l < 5; l++)
        if (i >= wb[l] && i < we[l]) {
            const int cols = l == 0 ? K1 : HID;
            r = (i - wb[l]) / cols;
            k = (i - wb[l]) % cols;
            return true;
        }
    return false;
}

__device__ __forceinline__ void wimg_store(unsigned char* img, int i, float p)
{
    int l, r, k;
    if (!weight_of(i, l, r, k))
        return;
    const __nv_bfloat16 b = __float2bfloat16_rn(p);
    *reinterpret_cast<__nv_bfloat16*>(img + wimg_fwd(l, r, k)) = b;
    if (l > 0)
        *reinterpret_cast<__nv_bfloat16*>(img + wimg_bwd(l, r, k)) = b;
}

// One bulk copy global -> shared (cp.async.bulk, completion counted on the
// mbarrier in bytes), issued by thread 0; every thread waits.  Addresses and
// size are multiples of 16.  False when the wait gave up.
__device__ __forceinline__ bool bulk_load(unsigned char* sm, uint32_t dst_off, const unsigned char* src,
                                          uint32_t bytes, uint64_t* cbar, uint32_t& phase)
{
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma::smem_u32(cbar)),
                     "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                umma::smem_u32(sm + dst_off)),
            "l"(src), "r"(bytes), "r"(umma::smem_u32(cbar))
            : "memory");
    }
    const bool ok = umma::mbar_wait(cbar, phase);
    phase ^= 1u;
    return ok;
}

// Eight BF16 values as one 16-byte row of a core matrix.
__device__ __forceinline__ void st_bf16x8(unsigned char* base, uint32_t off, const float* v)
{
    uint4 u;
    __nv_bfloat162 h0 = __floats2bfloat162_rn(v[0], v[1]), h1 = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 h2 = __floats2bfloat162_rn(v[4], v[5]), h3 = __floats2bfloat162_rn(v[6], v[7]);
    u.x = *reinterpret_cast<uint32_t*>(&h0);
    u.y = *reinterpret_cast<uint32_t*>(&h1);
    u.z = *reinterpret_cast<uint32_t*>(&h2);
    u.w = *reinterpret_cast<uint32_t*>(&h3);
    *reinterpret_cast<uint4*>(base + off) = u;
}

// Feature f of the encoding (f < FEAT; FEAT..K1-1 are zero padding).
__device__ __forceinline__ float feature(const float* c6, int f)
{
    if (f < 6)
        return c6[f];
    if (f >= FEAT)
        return 0.0f;
    int j = f - 6, c = j >> 4, k = (j >> 1) & 7;
    float s, co;
    sincospif(c6[c] * (float)(1 << k) * 0.125f, &s, &co);   // frequencies pi/8 .. 16 pi
    return (j & 1) ? co : s;
}

// One layer: D[tmem] = A_tile (128 x K) * W_tile (N x K)^T, thread 0 issues,
// everyone waits.  Returns false when the wait gave up.
__device__ __forceinline__ bool layer_mma(uint32_t d_tmem, uint32_t a_saddr, uint32_t b_saddr, int K, int N,
                                          uint64_t* mbar, uint32_t& phase)
{
    if (threadIdx.x == 0) {
        for (int kk = 0; kk < K / 16; kk++)
            umma::mma_bf16(d_tmem, umma::tile_desc(a_saddr, K, kk), umma::tile_desc(b_saddr, K, kk),
                           umma::idesc_bf16(TILE, N), kk > 0);
        umma::commit(mbar);
    }
    bool ok = umma::mbar_wait(mbar, phase);
    phase ^= 1u;
    umma::fence_after_sync();
    return ok;
}

__device__ __forceinline__ void sync_for_mma()
{
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
}

// Hidden-layer epilogue: this thread's row + bias, ReLU, BF16 into the next
// input tile (row t, K = 64) and, training, into the transposed tile.
// Returns the ReLU mask of this thread's row (bit c: the BF16 activation of
// column c is positive), the backward pass's gate.
template <bool TRAIN>
__device__ __forceinline__ uint64_t hidden_epilogue(uint32_t taddr, const float* bias, unsigned char* sm,
                                                    uint32_t next_off, uint32_t ht_off)
{
    const int t = threadIdx.x;
    uint64_t mask = 0;
#pragma unroll
    for (int c = 0; c < HID; c += 16) {
        float v[16];
        umma::tmem_ld16(taddr + c, v);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            v[j] = fmaxf(v[j] + bias[c + j], 0.0f);
            if (TRAIN) {
                st_bf16(sm, ht_off + umma::kmajor_offset(c + j, t, TILE), v[j]);
                if (__bfloat162float(__float2bfloat16_rn(v[j])) > 0.0f)
                    mask |= 1ull << (c + j);
            }
        }
        st_bf16x8(sm, next_off + umma::kmajor_offset(t, c, HID), v);
        st_bf16x8(sm, next_off + umma::kmajor_offset(t, c + 8, HID), v + 8);
    }
    return mask;
}

template <bool TRAIN>
__global__ void __launch_bounds__(128, 1) k_nic(NicIO io, const unsigned char* __restrict__ wimg,
                                               const float* __restrict__ params, float* __restrict__ grad,
                                               float* __restrict__ loss, float inv_batch, uint32_t* err)
{
    extern __shared__ __align__(128) unsigned char sm[];
    using MP = Map<TRAIN>;
    const int t = threadIdx.x, warp = t >> 5;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + MP::MBAR);
    uint64_t* cbar = reinterpret_cast<uint64_t*>(sm + MP::CBAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + MP::TSLOT);
    float* sbias = reinterpret_cast<float*>(sm + MP::BIAS);
    float* sbgrad = reinterpret_cast<float*>(sm + MP::BGRAD);
    float* sloss = reinterpret_cast<float*>(sm + MP::LOSS);
    if (warp == 0)
        umma::tmem_alloc(tslot, MP::TMEM_COLS);
    if (t == 0) {
        umma::mbar_init(mbar, 1);
        umma::mbar_init(cbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
        for (int w = 0; w < 5; w++)
            sloss[w] = 0.0f;
    }
    for (int i = t; i < 4 * HID + NO; i += blockDim.x)
        sbias[i] = params[i < 4 * HID ? P_B1 + (i / HID) * (P_B2 - P_B1) + (i % HID) : P_B5 + (i - 4 * HID)];

    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = *tslot;
    const uint32_t lane = (uint32_t)(warp * 32) << 16;
    const uint32_t s0 = umma::smem_u32(sm);
    uint32_t phase = 0, cphase = 0;
    bool ok = true;
    // this CTA's gradient slice: its first tile stores, later tiles add
    float* const gslice = TRAIN ? grad + (size_t)blockIdx.x * NPARAM : nullptr;
    for (int tile = blockIdx.x; tile * TILE < io.n; tile += gridDim.x) {
        const bool first = tile == (int)blockIdx.x;
        ok &= bulk_load(sm, OFF_W1, wimg, WIMG_FWD, cbar, cphase);   // the forward tiles
        const int i = tile * TILE + t;
        const bool valid = i < io.n;
        const int si = valid ? (io.idx ? io.idx[i] : i) : 0;
        float c6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (valid) {
            float4 p = io.pos[(long)si * io.stride], nv = io.nrm[(long)si * io.stride];
            c6[0] = fminf(fmaxf((p.x - io.lo.x) * io.scale.x - 1.0f, -1.0f), 1.0f);
            c6[1] = fminf(fmaxf((p.y - io.lo.y) * io.scale.y - 1.0f, -1.0f), 1.0f);
            c6[2] = fminf(fmaxf((p.z - io.lo.z) * io.scale.z - 1.0f, -1.0f), 1.0f);
            c6[3] = nv.x;
            c6[4] = nv.y;
            c6[5] = nv.z;
        }
        for (int f0 = 0; f0 < K1; f0 += 8) {
            float v8[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                v8[j] = valid ? feature(c6, f0 + j) : 0.0f;
                if (TRAIN)
                    st_bf16(sm, OFF_X0T + umma::kmajor_offset(f0 + j, t, TILE), v8[j]);
            }
            st_bf16x8(sm, OFF_A0 + umma::kmajor_offset(t, f0, K1), v8);
        }
        sync_for_mma();
        // forward: A0(112) -> A1 -> A0 -> A1 -> A0 -> out
        ok &= layer_mma(tm, s0 + OFF_A0, s0 + OFF_W1, K1, HID, mbar, phase);
        uint64_t relu[4];
        relu[0] = hidden_epilogue<TRAIN>(tm + lane, sbias + 0 * HID, sm, OFF_A1, OFF_H1T);
        sync_for_mma();
        ok &= layer_mma(tm, s0 + OFF_A1, s0 + OFF_W2, HID, HID, mbar, phase);
        relu[1] = hidden_epilogue<TRAIN>(tm + lane, sbias + 1 * HID, sm, OFF_A0, OFF_H2T);
        sync_for_mma();
        ok &= layer_mma(tm, s0 + OFF_A0, s0 + OFF_W3, HID, HID, mbar, phase);
        relu[2] = hidden_epilogue<TRAIN>(tm + lane, sbias + 2 * HID, sm, OFF_A1, OFF_H3T);
        sync_for_mma();
        ok &= layer_mma(tm, s0 + OFF_A1, s0 + OFF_W4, HID, HID, mbar, phase);
        relu[3] = hidden_epilogue<TRAIN>(tm + lane, sbias + 3 * HID, sm, OFF_A0, OFF_H4T);
        sync_for_mma();
        ok &= layer_mma(tm, s0 + OFF_A0, s0 + OFF_W5, HID, NO, mbar, phase);
        float y[16];
        umma::tmem_ld16(tm + lane, y);
#pragma unroll
        for (int c = 0; c < NO; c++)
            y[c] += sbias[4 * HID + c];
        if (!TRAIN) {
            if (valid)
                io.out[i] = make_float4(y[0], y[1], y[2], 0.0f);
            umma::fence_before_sync();
            __syncthreads();
            umma::fence_after_sync();
            continue;
        }
        // ---------------------------------------------------------- backward
        // loss (p - y)^2 / (p^2 + 0.01), p the prediction held constant in
        // the denominator; dL/dp = 2 (p - y) / (p^2 + 0.01)
        float dz[HID];
        float lsum = 0.0f;
        float4 tg = valid ? io.target[(long)si * io.stride] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float tgc[3] = {tg.x, tg.y, tg.z};
#pragma unroll
        for (int c = 0; c < NO; c++) {
            float g = 0.0f;
            if (valid && c < NOUT) {
                float den = y[c] * y[c] + 0.01f;
                float d = y[c] - tgc[c];
                lsum += d * d / den * inv_batch;
                g = 2.0f * d / den * inv_batch;
            }
            dz[c] = g;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
            lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
        if ((t & 31) == 0)
            sloss[1 + warp] += lsum;   // one partial per warp, summed at the end
        // the weight region now holds the transposed weights; rows 16..63
        // of dZ^T are cleared for the 16-output layer
        ok &= bulk_load(sm, OFF_W2T, wimg + WIMG_FWD, WIMG_BWD, cbar, cphase);
        // the forward pass reused the dZ^T region: its padded rows are
        // cleared again (rows 16..127 for the 16-output layer; 64..127 stay)
        for (int r = NO; r < TILE; r++)
            st_bf16(sm, OFF_DZT + umma::kmajor_offset(r, t, TILE), 0.0f);
        const uint32_t ht_off[5] = {OFF_X0T, OFF_H1T, OFF_H2T, OFF_H3T, OFF_H4T};
        const uint32_t wt_off[5] = {0, OFF_W2T, OFF_W3T, OFF_W4T, OFF_W5T};
        const int wofs[5] = {P_W1, P_W2, P_W3, P_W4, P_W5};
        const int bofs[5] = {P_B1, P_B2, P_B3, P_B4, P_B5};
        for (int l = 4; l >= 0; l--) {
            const int nout = l == 4 ? NO : HID;
            const int nin = l == 0 ? K1 : HID;
            for (int o = 0; o < nout; o += 8) {
                float d8[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    d8[j] = dz[o + j];
                    st_bf16(sm, OFF_DZT + umma::kmajor_offset(o + j, t, TILE), d8[j]);
                    // bias gradient: the warp's sum of this column, one
                    // shared partial per warp (no shared-memory atomics)
                    float w = d8[j];
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1)
                        w += __shfl_xor_sync(0xffffffffu, w, off);
                    if ((t & 31) == 0)
                        sbgrad[warp * HID + o + j] = w;
                }
                st_bf16x8(sm, OFF_DZ + umma::kmajor_offset(t, o, nout), d8);
            }
            sync_for_mma();
            if (t == 0) {
                for (int kk = 0; kk < TILE / 16; kk++)   // dW = dZ^T * H
                    umma::mma_bf16(tm + 128, umma::tile_desc(s0 + OFF_DZT, TILE, kk),
                                   umma::tile_desc(s0 + ht_off[l], TILE, kk), umma::idesc_bf16(TILE, nin), kk > 0);
                if (l > 0)
                    for (int kk = 0; kk < nout / 16; kk++)   // dH = dZ * W
                        umma::mma_bf16(tm, umma::tile_desc(s0 + OFF_DZ, nout, kk),
                                       umma::tile_desc(s0 + wt_off[l], nout, kk), umma::idesc_bf16(TILE, HID),
                                       kk > 0);
                umma::commit(mbar);
            }
            ok &= umma::mbar_wait(mbar, phase);
            phase ^= 1u;
            umma::fence_after_sync();
            for (int c = 0; c < nin; c += 16) {   // lane t = output row t of dW
                float v[16];
                umma::tmem_ld16(tm + lane + 128 + c, v);
                if (t < nout) {
                    float* g = gslice + wofs[l] + t * nin + c;
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        g[j] = first ? v[j] : g[j] + v[j];
                }
            }
            if (l > 0) {
                const uint64_t m = relu[l - 1];   // the input of layer l is hidden layer l's output
#pragma unroll
                for (int c = 0; c < HID; c += 16) {
                    float v[16];
                    umma::tmem_ld16(tm + lane + c, v);
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        dz[c + j] = ((m >> (c + j)) & 1ull) ? v[j] : 0.0f;
                }
            }
            umma::fence_before_sync();
            __syncthreads();
            umma::fence_after_sync();
            if (t < nout) {
                const float b = sbgrad[t] + sbgrad[HID + t] + sbgrad[2 * HID + t] + sbgrad[3 * HID + t];
                gslice[bofs[l] + t] = first ? b : gslice[bofs[l] + t] + b;
            }
            __syncthreads();
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 0)
        umma::tmem_dealloc(tm, MP::TMEM_COLS);
    if (TRAIN && t == 0)
        loss[blockIdx.x] = sloss[1] + sloss[2] + sloss[3] + sloss[4];
    if (!ok && t == 0)
        atomicOr(err, DE_ITERATION_CAP);
}

// Sum of parameter i's gradient over the CTA slices in a fixed order: eight
// running sums over slices b = j (mod 8), then those eight in order.  The
// eight independent loads per round keep the slice reads in flight.
__device__ __forceinline__ float slice_sum(const float* __restrict__ parts, int nparts, int i)
{
    float g[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int b = 0;
    for (; b + 8 <= nparts; b += 8) {
#pragma unroll
        for (int j = 0; j < 8; j++)
            g[j] += __ldcg(parts + (size_t)(b + j) * NPARAM + i);
    }
    for (int j = 0; b + j < nparts; j++)
        g[j] += __ldcg(parts + (size_t)(b + j) * NPARAM + i);
    return ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + (g[6] + g[7]));
}

// Adam on the FP32 master parameters, the gradient summed from the CTA
// slices; refreshes the BF16 copy.  Parameters of the padded output rows
// stay zero.
__global__ void k_nic_adam(float* __restrict__ params, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ parts, int nparts, unsigned char* __restrict__ wimg, float lr,
                           float b1, float b2, float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x) {
        bool pad = (i >= P_W5 && i < P_B5 && (i - P_W5) / HID >= NOUT) || (i >= P_B5 && i - P_B5 >= NOUT);
        float g = pad ? 0.0f : slice_sum(parts, nparts, i);
        float mi = b1 * m[i] + (1.0f - b1) * g;
        float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        float p = pad ? 0.0f : params[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        params[i] = p;
        wimg_store(wimg, i, p);
    }
}

// The gradient and loss of a training launch summed from its CTA slices.
__global__ void k_nic_reduce(const float* __restrict__ parts, const float* __restrict__ loss_parts, int nparts,
                             float* __restrict__ grad, float* __restrict__ loss)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x)
        grad[i] = slice_sum(parts, nparts, i);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float l = 0.0f;
        for (int b = 0; b < nparts; b++)
            l += loss_parts[b];
        *loss = l;
    }
}

__global__ void k_nic_to_bf16(const float* __restrict__ params, unsigned char* __restrict__ wimg)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x)
        wimg_store(wimg, i, params[i]);
}

}  // namespace

size_t smem_bytes(bool train) { return train ? Map<true>::BYTES : Map<false>::BYTES; }

cudaError_t launch_forward(const NicIO& io, const unsigned char* wimg, const float* params, uint32_t* err, int grid,
                           cudaStream_t st)
{
    if (io.n <= 0)
        return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_nic<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)Map<false>::BYTES);
        if (e != cudaSuccess)
            return e;
        attr = true;
    }
    int tiles = (io.n + TILE - 1) / TILE;
    k_nic<false><<<grid < tiles ? grid : tiles, TILE, Map<false>::BYTES, st>>>(io, wimg, params, nullptr, nullptr,
                                                                               0.0f, err);
    return cudaGetLastError();
}

int train_slices(int n, int grid)
{
    const int tiles = (n + TILE - 1) / TILE;
    return n <= 0 ? 0 : (grid < tiles ? grid : tiles);
}

cudaError_t launch_train(const NicIO& io, const unsigned char* wimg, const float* params, float* grad, float* loss,
                         float inv_batch, uint32_t* err, int grid, cudaStream_t st)
{
    if (io.n <= 0)
        return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_nic<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)Map<true>::BYTES);
        if (e != cudaSuccess)
            return e;
        attr = true;
    }
    int tiles = (io.n + TILE - 1) / TILE;
    k_nic<true><<<grid < tiles ? grid : tiles, TILE, Map<true>::BYTES, st>>>(io, wimg, params, grad, loss, inv_batch,
                                                                             err);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* params, float* m, float* v, const float* grad, int slices, unsigned char* wimg,
                        float lr, int step, cudaStream_t st)
{
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_nic_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(params, m, v, grad, slices, wimg, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_reduce(const float* grad_slices, const float* loss_slices, int slices, float* grad, float* loss,
                          cudaStream_t st)
{
    k_nic_reduce<<<(NPARAM + 255) / 256, 256, 0, st>>>(grad_slices, loss_slices, slices, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* params, unsigned char* wimg, cudaStream_t st)
{
    k_nic_to_bf16<<<(NPARAM + 255) / 256, 256, 0, st>>>(params, wimg);
    return cudaGetLastError();
}

}  // namespace nic
}  // namespace povgpu
