// k_mlp.cu -- fused BF16 tcgen05 kernels of the learned residual network.
//
// Network: 32 -> 64 -> 64 -> 64 -> 3 (padded to 16), SiLU on the hidden
// layers; BF16 operands in shared memory, FP32 accumulation in TMEM, one
// elected thread issues tcgen05.mma and commits to an mbarrier, and the four
// warps of the CTA run the epilogues on their own TMEM lane quarter (thread t
// owns sample row t of a 128-sample tile).
//
// Shared-memory staging (canonical no-swizzle layout of gs_tc.cuh): a
// tile of R samples x F features is stored at kmajor_offset(s, f, F).  The
// same bytes are the K-major A operand of the forward GEMM (M = samples,
// K = features) and the MN-major operand of the weight-gradient GEMM
// (N = features, K = samples); weights W[n][k] are staged once and serve as
// K-major B in the forward GEMM and MN-major B in the input-gradient GEMM.
//
//   k_mlp_forward : pred = net(feat), persistent over 128-sample tiles.
//   k_mlp_train   : forward, MSE loss, backward and weight / bias gradients
//                   of a mini-batch; pre-activations z1..z3 stay in TMEM,
//                   dW1..dW4 accumulate in TMEM across the CTA's tiles and
//                   are added to the global gradient at the end.
//   k_mlp_adam    : Adam update of the FP32 master weights.
#include "gs_mlp.h"
#include "gs_tc.cuh"

#include <cuda_bf16.h>

#include <atomic>
#include <cmath>
#include <random>
#include <vector>

namespace gs {

namespace {

// ---- shared-memory plan (bytes) -------------------------------------------
constexpr uint32_t SM_W1 = 0;                                   // 64 x 32
constexpr uint32_t SM_W2 = SM_W1 + MLP_H * MLP_IN * 2;          // 64 x 64
constexpr uint32_t SM_W3 = SM_W2 + MLP_H * MLP_H * 2;           // 64 x 64
constexpr uint32_t SM_W4 = SM_W3 + MLP_H * MLP_H * 2;           // 16 x 64
constexpr uint32_t SM_X = SM_W4 + MLP_OUT_PAD * MLP_H * 2;      // 128 x 32
constexpr uint32_t SM_H1 = SM_X + MLP_TILE * MLP_IN * 2;        // 128 x 64
constexpr uint32_t SM_H2 = SM_H1 + MLP_TILE * MLP_H * 2;
constexpr uint32_t SM_H3 = SM_H2 + MLP_TILE * MLP_H * 2;
constexpr uint32_t SM_FWD_END = SM_H3 + MLP_TILE * MLP_H * 2;   // 81920
constexpr int DW = 128;                                         // delta tile width
constexpr uint32_t SM_D0 = SM_FWD_END;                          // 128 x 128
constexpr uint32_t SM_D1 = SM_D0 + MLP_TILE * DW * 2;
constexpr uint32_t SM_TRAIN_END = SM_D1 + MLP_TILE * DW * 2;    // 147456

// TMEM columns
constexpr uint32_t TM_Z1 = 0, TM_Z2 = 64, TM_Z3 = 128, TM_OUT = 192;
constexpr uint32_t TM_DW1 = 256, TM_DW2 = 288, TM_DW3 = 352, TM_DW4 = 416;

// The quotients use the fast reciprocal (__fdividef, about 2 ulp) rather than
// the IEEE division's longer sequence: the activations are rounded to BF16
// (8 significant bits) right after.  For v < -88, 1 + exp(-v) is infinite and
// the quotient is -0, the limit of SiLU.
__device__ __forceinline__ float silu(float v) { return __fdividef(v, 1.0f + __expf(-v)); }
__device__ __forceinline__ float silu_grad(float v)
{
    const float s = __fdividef(1.0f, 1.0f + __expf(-v));
    return s * (1.0f + v * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// 8 consecutive features (f0 % 8 == 0) of row r -> one 16-byte store.
__device__ __forceinline__ void store8(unsigned char *tile, int r, int f0, int F, const float *v)
{
    uint4 q;
    q.x = pack2(v[0], v[1]);
    q.y = pack2(v[2], v[3]);
    q.z = pack2(v[4], v[5]);
    q.w = pack2(v[6], v[7]);
    *reinterpret_cast<uint4 *>(tile + kmajor_offset(r, f0, F)) = q;
}

// Stage W[n][k] (FP32, row-major) K-major as BF16.
__device__ void stage_weights(unsigned char *sm, const float *__restrict__ P)
{
    for (int e = threadIdx.x; e < MLP_H * MLP_IN; e += blockDim.x)
        *reinterpret_cast<__nv_bfloat16 *>(sm + SM_W1 + kmajor_offset(e / MLP_IN, e % MLP_IN, MLP_IN)) =
            __float2bfloat16_rn(P[MLP_OFF_W1 + e]);
    for (int e = threadIdx.x; e < MLP_H * MLP_H; e += blockDim.x) {
        const int n = e / MLP_H, k = e % MLP_H;
        *reinterpret_cast<__nv_bfloat16 *>(sm + SM_W2 + kmajor_offset(n, k, MLP_H)) =
            __float2bfloat16_rn(P[MLP_OFF_W2 + e]);
        *reinterpret_cast<__nv_bfloat16 *>(sm + SM_W3 + kmajor_offset(n, k, MLP_H)) =
            __float2bfloat16_rn(P[MLP_OFF_W3 + e]);
    }
    for (int e = threadIdx.x; e < MLP_OUT_PAD * MLP_H; e += blockDim.x)
        *reinterpret_cast<__nv_bfloat16 *>(sm + SM_W4 + kmajor_offset(e / MLP_H, e % MLP_H, MLP_H)) =
            __float2bfloat16_rn(P[MLP_OFF_W4 + e]);
}

// Features of sample row r (FP32, 32 per sample) -> X tile; rows past n are zero.
__device__ __forceinline__ void stage_features(unsigned char *sm, const float *__restrict__ feat,
                                               long long base, int n, int r)
{
    const long long i = base + r;
    float v[MLP_IN];
    if (i < n) {
        const float4 *src = reinterpret_cast<const float4 *>(feat + i * MLP_IN);
#pragma unroll
        for (int q = 0; q < MLP_IN / 4; ++q) {
            const float4 t = src[q];
            v[4 * q] = t.x;
            v[4 * q + 1] = t.y;
            v[4 * q + 2] = t.z;
            v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < MLP_IN; ++q) v[q] = 0.0f;
    }
#pragma unroll
    for (int f = 0; f < MLP_IN; f += 8) store8(sm + SM_X, r, f, MLP_IN, v + f);
}

// All threads: smem writes visible to the tensor core, TMEM reads done.
__device__ __forceinline__ void tc_sync()
{
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// D (+)= A[128 x K] * B[N x K]^T with K/16 MMAs; A/B start addresses advance
// by astep/bstep bytes per 16-wide K step.
__device__ __forceinline__ void mma_run(uint32_t d, uint32_t a, uint32_t a_lbo, uint32_t a_sbo,
                                        uint32_t astep, uint32_t b, uint32_t b_lbo, uint32_t b_sbo,
                                        uint32_t bstep, int K, uint32_t idesc, bool accumulate)
{
    for (int kk = 0; kk < K / 16; ++kk) {
        const uint64_t ad = smem_desc(a + kk * astep, a_lbo, a_sbo);
        const uint64_t bd = smem_desc(b + kk * bstep, b_lbo, b_sbo);
        umma_bf16(d, ad, bd, idesc, (accumulate || kk > 0) ? 1u : 0u);
    }
}

// Forward GEMM of a layer: D = Tile[128 x kin] * W[nout x kin]^T (both K-major).
__device__ __forceinline__ void mma_forward(uint32_t d, uint32_t tile, uint32_t w, int kin, int nout)
{
    mma_run(d, tile, 128, kin * 16, 256, w, 128, kin * 16, 256, kin,
            idesc_bf16_f32(128, nout, false, false), false);
}

// Input gradient: D[128 x kin] = Delta[128 x nout] (K-major, width DW) * W (MN-major).
__device__ __forceinline__ void mma_input_grad(uint32_t d, uint32_t delta, uint32_t w, int kin,
                                               int nout)
{
    mma_run(d, delta, 128, DW * 16, 256, w, kin * 16, 128, 2 * kin * 16, nout,
            idesc_bf16_f32(128, kin, false, true), false);
}

// Weight gradient: D[128(nout) x kin] += Delta^T * Tile (both MN-major, K = samples).
__device__ __forceinline__ void mma_weight_grad(uint32_t d, uint32_t delta, uint32_t tile, int kin,
                                                bool accumulate)
{
    mma_run(d, delta, DW * 16, 128, 2 * DW * 16, tile, kin * 16, 128, 2 * kin * 16, MLP_TILE,
            idesc_bf16_f32(128, kin, true, true), accumulate);
}

__device__ __forceinline__ bool wait_mma(uint64_t *bar, uint32_t &phase, unsigned *status)
{
    const bool ok = mbar_wait(bar, phase & 1u);
    ++phase;
    if (!ok && (threadIdx.x & 31) == 0) atomicOr(status, ST_WAIT_TIMEOUT);
    return __syncthreads_and(ok);
}

// Hidden-layer epilogue: h = SiLU(z + b) -> BF16 tile (64 wide).
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem_row, uint32_t col, const float *bias,
                                                unsigned char *tile, int r)
{
#pragma unroll
    for (int c0 = 0; c0 < MLP_H; c0 += 16) {
        float v[16];
        tmem_ld16(tmem_row + col + c0, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = silu(v[j] + bias[c0 + j]);
        store8(tile, r, c0, MLP_H, v);
        store8(tile, r, c0 + 8, MLP_H, v + 8);
    }
}

}  // namespace

// Forward-only plan: each hidden layer's MMA has completed (read its input
// tile) before the epilogue writes the next activations, so one hidden tile
// serves all three layers, and one 64-column accumulator all three hidden
// GEMMs: 46 KB of shared memory and 128 TMEM columns per CTA, four CTAs per SM.
constexpr uint32_t SM_FWD_H = SM_H1;
constexpr uint32_t SM_FWD_END1 = SM_FWD_H + MLP_TILE * MLP_H * 2;   // 47104
constexpr uint32_t TM_FWD_Z = 0, TM_FWD_OUT = 64, TM_FWD_COLS = 128;
constexpr int FWD_CTAS_PER_SM = 4;

// Features of sample row r (FP32, 32 per sample) -> registers; rows past n are zero.
__device__ __forceinline__ void load_features(float *v, const float *__restrict__ feat,
                                              long long base, int n, int r)
{
    const long long i = base + r;
    if (i < n) {
        const float4 *src = reinterpret_cast<const float4 *>(feat + i * MLP_IN);
#pragma unroll
        for (int q = 0; q < MLP_IN / 4; ++q) {
            const float4 t = __ldcs(src + q);
            v[4 * q] = t.x;
            v[4 * q + 1] = t.y;
            v[4 * q + 2] = t.z;
            v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < MLP_IN; ++q) v[q] = 0.0f;
    }
}

__global__ void __launch_bounds__(128, FWD_CTAS_PER_SM)
k_mlp_forward(const float *__restrict__ P, const float *__restrict__ feat, int n,
              float *__restrict__ pred, unsigned *__restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t taddr_s;
    __shared__ float bias[3 * MLP_H + MLP_OUT_PAD];
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(&taddr_s, TM_FWD_COLS);
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    stage_weights(sm, P);
    for (int j = tid; j < MLP_H; j += blockDim.x) {
        bias[j] = P[MLP_OFF_B1 + j];
        bias[MLP_H + j] = P[MLP_OFF_B2 + j];
        bias[2 * MLP_H + j] = P[MLP_OFF_B3 + j];
    }
    if (tid < MLP_OUT_PAD) bias[3 * MLP_H + tid] = P[MLP_OFF_B4 + tid];
    tc_sync();
    const uint32_t tmem = taddr_s;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t s0 = smem_u32(sm);
    uint32_t phase = 0;
    bool ok = true;
    const int tiles = (n + MLP_TILE - 1) / MLP_TILE;
    float v[MLP_IN];
    if (blockIdx.x < tiles) load_features(v, feat, (long long)blockIdx.x * MLP_TILE, n, tid);
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const long long base = (long long)t * MLP_TILE;
#pragma unroll
        for (int f = 0; f < MLP_IN; f += 8) store8(sm + SM_X, tid, f, MLP_IN, v + f);
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_FWD_Z, s0 + SM_X, s0 + SM_W1, MLP_IN, MLP_H);
            umma_commit(&bar);
        }
        // the next tile's features are in flight while this tile's layers run
        if (t + (int)gridDim.x < tiles)
            load_features(v, feat, (long long)(t + gridDim.x) * MLP_TILE, n, tid);
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        hidden_epilogue(trow, TM_FWD_Z, bias, sm + SM_FWD_H, tid);
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_FWD_Z, s0 + SM_FWD_H, s0 + SM_W2, MLP_H, MLP_H);
            umma_commit(&bar);
        }
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        hidden_epilogue(trow, TM_FWD_Z, bias + MLP_H, sm + SM_FWD_H, tid);
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_FWD_Z, s0 + SM_FWD_H, s0 + SM_W3, MLP_H, MLP_H);
            umma_commit(&bar);
        }
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        hidden_epilogue(trow, TM_FWD_Z, bias + 2 * MLP_H, sm + SM_FWD_H, tid);
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_FWD_OUT, s0 + SM_FWD_H, s0 + SM_W4, MLP_H, MLP_OUT_PAD);
            umma_commit(&bar);
        }
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        float o[16];
        tmem_ld16(trow + TM_FWD_OUT, o);
        const long long i = base + tid;
        if (i < n) {
            pred[3 * i + 0] = o[0] + bias[3 * MLP_H + 0];
            pred[3 * i + 1] = o[1] + bias[3 * MLP_H + 1];
            pred[3 * i + 2] = o[2] + bias[3 * MLP_H + 2];
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TM_FWD_COLS);
}

// ------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
k_mlp_train(const float *__restrict__ P, const float *__restrict__ feat,
            const float *__restrict__ target, int n, float grad_scale, float *__restrict__ G,
            float *__restrict__ loss, unsigned *__restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t taddr_s;
    __shared__ float bias[3 * MLP_H + MLP_OUT_PAD];
    __shared__ float dbias[3 * MLP_H + MLP_OUT_PAD];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tmem_alloc(&taddr_s, 512);
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    stage_weights(sm, P);
    for (int j = tid; j < MLP_H; j += blockDim.x) {
        bias[j] = P[MLP_OFF_B1 + j];
        bias[MLP_H + j] = P[MLP_OFF_B2 + j];
        bias[2 * MLP_H + j] = P[MLP_OFF_B3 + j];
    }
    if (tid < MLP_OUT_PAD) bias[3 * MLP_H + tid] = P[MLP_OFF_B4 + tid];
    for (int j = tid; j < 3 * MLP_H + MLP_OUT_PAD; j += blockDim.x) dbias[j] = 0.0f;
    // delta tiles start at zero (their padding columns are read but unused)
    for (uint32_t b = tid * 16; b < SM_TRAIN_END - SM_D0; b += blockDim.x * 16)
        *reinterpret_cast<uint4 *>(sm + SM_D0 + b) = make_uint4(0, 0, 0, 0);
    tc_sync();
    const uint32_t tmem = taddr_s;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t s0 = smem_u32(sm);
    uint32_t phase = 0;
    bool ok = true;
    bool first = true;
    float lsum = 0.0f;
    const int tiles = (n + MLP_TILE - 1) / MLP_TILE;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const long long base = (long long)t * MLP_TILE;
        const long long i = base + tid;
        const bool valid = i < n;
        stage_features(sm, feat, base, n, tid);
        // forward, keeping z1..z3 in TMEM
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_Z1, s0 + SM_X, s0 + SM_W1, MLP_IN, MLP_H);
            umma_commit(&bar);
        }
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        hidden_epilogue(trow, TM_Z1, bias, sm + SM_H1, tid);
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_Z2, s0 + SM_H1, s0 + SM_W2, MLP_H, MLP_H);
            umma_commit(&bar);
        }
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        hidden_epilogue(trow, TM_Z2, bias + MLP_H, sm + SM_H2, tid);
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_Z3, s0 + SM_H2, s0 + SM_W3, MLP_H, MLP_H);
            umma_commit(&bar);
        }
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        hidden_epilogue(trow, TM_Z3, bias + 2 * MLP_H, sm + SM_H3, tid);
        tc_sync();
        if (tid == 0) {
            mma_forward(tmem + TM_OUT, s0 + SM_H3, s0 + SM_W4, MLP_H, MLP_OUT_PAD);
            umma_commit(&bar);
        }
        if (!(ok = wait_mma(&bar, phase, status))) break;
        tc_fence_after();
        // output error -> delta4 (tile D0, columns 0..15)
        {
            float o[16];
            tmem_ld16(trow + TM_OUT, o);
            float d[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) d[j] = 0.0f;
            if (valid) {
#pragma unroll
                for (int j = 0; j < MLP_OUT; ++j) {
                    const float e = o[j] + bias[3 * MLP_H + j] - target[3 * i + j];
                    lsum += e * e;
                    d[j] = grad_scale * e;
                }
            }
            store8(sm + SM_D0, tid, 0, DW, d);
            store8(sm + SM_D0, tid, 8, DW, d + 8);
#pragma unroll
            for (int j = 0; j < MLP_OUT; ++j) {
                float s = d[j];
                for (int o2 = 16; o2 > 0; o2 >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o2);
                if (lane == 0) atomicAdd(&dbias[3 * MLP_H + j], s);
            }
        }
        // backward through layers 4, 3, 2 and weight gradients 4, 3, 2, 1
        const uint32_t tile_in[4] = {SM_X, SM_H1, SM_H2, SM_H3};
        const uint32_t wsm[4] = {SM_W1, SM_W2, SM_W3, SM_W4};
        const uint32_t zcol[3] = {TM_Z1, TM_Z2, TM_Z3};
        const uint32_t dwcol[4] = {TM_DW1, TM_DW2, TM_DW3, TM_DW4};
        uint32_t dcur = SM_D0, dnext = SM_D1;
        for (int l = 3; l >= 0; --l) {
            const int kin = l == 0 ? MLP_IN : MLP_H;
            const int nout = l == 3 ? MLP_OUT_PAD : MLP_H;
            tc_sync();
            if (tid == 0) {
                mma_weight_grad(tmem + dwcol[l], s0 + dcur, s0 + tile_in[l], kin, !first);
                if (l > 0) mma_input_grad(tmem + TM_OUT, s0 + dcur, s0 + wsm[l], kin, nout);
                umma_commit(&bar);
            }
            if (!(ok = wait_mma(&bar, phase, status))) break;
            if (l == 0) break;
            tc_fence_after();
            // delta_{l-1} = (delta_l W_l) * SiLU'(z_{l-1} + b_{l-1})
            const float *bl = bias + (l - 1) * MLP_H;
            float *dbl = dbias + (l - 1) * MLP_H;
#pragma unroll
            for (int c0 = 0; c0 < MLP_H; c0 += 16) {
                float g[16], z[16];
                tmem_ld16(trow + TM_OUT + c0, g);
                tmem_ld16(trow + zcol[l - 1] + c0, z);
#pragma unroll
                for (int j = 0; j < 16; ++j) g[j] = valid ? g[j] * silu_grad(z[j] + bl[c0 + j]) : 0.0f;
                store8(sm + dnext, tid, c0, DW, g);
                store8(sm + dnext, tid, c0 + 8, DW, g + 8);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float s = g[j];
                    for (int o2 = 16; o2 > 0; o2 >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o2);
                    if (lane == 0) atomicAdd(&dbl[c0 + j], s);
                }
            }
            const uint32_t tmp = dcur;
            dcur = dnext;
            dnext = tmp;
        }
        first = false;
    }
    // gradients out: row r of dW_l is output unit r
    tc_fence_after();
    if (ok && !first) {
        const int r = tid;
        const uint32_t dwcol[4] = {TM_DW1, TM_DW2, TM_DW3, TM_DW4};
        const int kins[4] = {MLP_IN, MLP_H, MLP_H, MLP_H};
        const int offs[4] = {MLP_OFF_W1, MLP_OFF_W2, MLP_OFF_W3, MLP_OFF_W4};
        const int nouts[4] = {MLP_H, MLP_H, MLP_H, MLP_OUT};
        for (int l = 0; l < 4; ++l) {
            for (int c0 = 0; c0 < kins[l]; c0 += 16) {
                float v[16];
                tmem_ld16(trow + dwcol[l] + c0, v);
                if (r < nouts[l]) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) atomicAdd(&G[offs[l] + r * kins[l] + c0 + j], v[j]);
                }
            }
        }
    }
    __syncthreads();
    if (ok && !first) {
        for (int j = tid; j < MLP_H; j += blockDim.x) {
            atomicAdd(&G[MLP_OFF_B1 + j], dbias[j]);
            atomicAdd(&G[MLP_OFF_B2 + j], dbias[MLP_H + j]);
            atomicAdd(&G[MLP_OFF_B3 + j], dbias[2 * MLP_H + j]);
        }
        if (tid < MLP_OUT) atomicAdd(&G[MLP_OFF_B4 + tid], dbias[3 * MLP_H + tid]);
        for (int o2 = 16; o2 > 0; o2 >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o2);
        if (lane == 0) atomicAdd(&loss[0], lsum);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// Adam on the FP32 master weights (padding rows of the last layer stay 0).
__global__ void k_mlp_adam(float *__restrict__ P, float *__restrict__ G, float *__restrict__ M,
                           float *__restrict__ V, float lr, float b1, float b2, float c1, float c2,
                           float eps)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= MLP_NPARAM) return;
    const bool pad = (p >= MLP_OFF_W4 + MLP_OUT * MLP_H && p < MLP_OFF_B4) ||
                     (p >= MLP_OFF_B4 + MLP_OUT);
    const float g = G[p];
    G[p] = 0.0f;
    if (pad) return;
    const float m = b1 * M[p] + (1.0f - b1) * g;
    const float v = b2 * V[p] + (1.0f - b2) * g * g;
    M[p] = m;
    V[p] = v;
    P[p] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// ------------------------------------------------------------------------
ErrorStatus MlpDevice::setup(unsigned long long seed, cudaStream_t s)
{
    GS_TRY(params.reserve(MLP_NPARAM * sizeof(float)));
    GS_TRY(grads.reserve(MLP_NPARAM * sizeof(float)));
    GS_TRY(adam_m.reserve(MLP_NPARAM * sizeof(float)));
    GS_TRY(adam_v.reserve(MLP_NPARAM * sizeof(float)));
    GS_TRY(loss.reserve(2 * sizeof(float)));
    GS_TRY(status.reserve(sizeof(unsigned)));
    std::vector<float> h(MLP_NPARAM, 0.0f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int nout, int kin, float gain, int nreal) {
        std::uniform_real_distribution<float> u(-1.0f, 1.0f);
        const float a = gain / std::sqrt((float)kin);
        for (int r = 0; r < nout; ++r)
            for (int k = 0; k < kin; ++k) h[off + r * kin + k] = r < nreal ? a * u(rng) : 0.0f;
    };
    fill(MLP_OFF_W1, MLP_H, MLP_IN, 1.7f, MLP_H);
    fill(MLP_OFF_W2, MLP_H, MLP_H, 1.7f, MLP_H);
    fill(MLP_OFF_W3, MLP_H, MLP_H, 1.7f, MLP_H);
    fill(MLP_OFF_W4, MLP_OUT_PAD, MLP_H, 0.1f, MLP_OUT);
    GS_CUDA(cudaMemcpyAsync(params.p, h.data(), MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice, s));
    GS_CUDA(cudaMemsetAsync(grads.p, 0, MLP_NPARAM * sizeof(float), s));
    GS_CUDA(cudaMemsetAsync(adam_m.p, 0, MLP_NPARAM * sizeof(float), s));
    GS_CUDA(cudaMemsetAsync(adam_v.p, 0, MLP_NPARAM * sizeof(float), s));
    GS_CUDA(cudaMemsetAsync(loss.p, 0, 2 * sizeof(float), s));
    GS_CUDA(cudaMemsetAsync(status.p, 0, sizeof(unsigned), s));
    GS_CUDA(cudaStreamSynchronize(s));
    adam_t = 0;
    return ok();
}

ErrorStatus MlpDevice::forward(const float *feat, int n, float *pred, cudaStream_t s)
{
    if (n <= 0) return ok();
    const DeviceInfo *dev = nullptr;
    GS_TRY(device_info(&dev));
    // the attribute belongs to the current device: set on every call
    GS_CUDA(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SM_FWD_END1));
    const int tiles = (n + MLP_TILE - 1) / MLP_TILE;
    const int grid = std::min(tiles, dev->sm_count * FWD_CTAS_PER_SM);
    k_mlp_forward<<<grid, 128, SM_FWD_END1, s>>>(params.as<float>(), feat, n, pred,
                                                status.as<unsigned>());
    GS_CUDA(cudaGetLastError());
    return ok();
}

ErrorStatus MlpDevice::gradients(const float *feat, const float *target, int n, cudaStream_t s)
{
    if (n <= 0) return ok();
    const DeviceInfo *dev = nullptr;
    GS_TRY(device_info(&dev));
    // the attribute belongs to the current device: set on every call
    GS_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SM_TRAIN_END));
    const int tiles = (n + MLP_TILE - 1) / MLP_TILE;
    const int grid = std::min(tiles, dev->sm_count);
    // mean over samples of the squared error summed over the 3 outputs
    const float grad_scale = 2.0f / (float)n;
    k_mlp_train<<<grid, 128, SM_TRAIN_END, s>>>(params.as<float>(), feat, target, n, grad_scale,
                                                grads.as<float>(), loss.as<float>(),
                                                status.as<unsigned>());
    GS_CUDA(cudaGetLastError());
    return ok();
}

ErrorStatus MlpDevice::train_step(const float *feat, const float *target, int n, float lr,
                                  cudaStream_t s)
{
    if (n <= 0) return ok();
    GS_TRY(gradients(feat, target, n, s));
    ++adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)adam_t), c2 = 1.0f - std::pow(b2, (float)adam_t);
    k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(params.as<float>(), grads.as<float>(),
                                                        adam_m.as<float>(), adam_v.as<float>(), lr,
                                                        b1, b2, c1, c2, 1e-8f);
    GS_CUDA(cudaGetLastError());
    return ok();
}

ErrorStatus MlpDevice::read_loss(cudaStream_t s, double *sum_sq)
{
    float h[2] = {0.0f, 0.0f};
    GS_CUDA(cudaMemcpyAsync(h, loss.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaMemsetAsync(loss.p, 0, sizeof(h), s));
    GS_CUDA(cudaStreamSynchronize(s));
    *sum_sq = h[0];
    return ok();
}

ErrorStatus MlpDevice::check(cudaStream_t s)
{
    unsigned h = 0;
    GS_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
    if (h & ST_WAIT_TIMEOUT) return GS_RAISE(GRAV_FAILURE, "MLP kernel: tensor-core wait timed out");
    return ok();
}

}  // namespace gs
