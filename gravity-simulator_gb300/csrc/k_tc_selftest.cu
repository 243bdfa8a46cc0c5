// k_tc_selftest.cu -- one-tile BF16 GEMM through tcgen05, for checking the
// operand layouts the learned-correction kernels use.
//
//   C[M x N] (FP32) = A[M x K] * B[N x K]^T,  M = 128, N in {16..256}, K % 16 == 0
//
// A and B arrive row-major (A[m][k], B[n][k]) in global memory and are
// written to shared memory either K-major or MN-major (canonical
// no-swizzle layouts of gs_tc.cuh); one thread issues K/16 MMAs into TMEM,
// commits them to an mbarrier, and the four warps read D back with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows of C).
#include "gs_internal.h"
#include "gs_tc.cuh"

#include <cuda_bf16.h>

#include <cstdio>

namespace gs {

constexpr int TS_M = 128;
constexpr int TS_MAX_NK = 256;

__global__ void __launch_bounds__(128)
k_tc_gemm_selftest(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B, int N,
                   int K, int a_mn, int b_mn, float *__restrict__ C, unsigned *__restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char ts_smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t taddr_s;
    unsigned char *sa = ts_smem;                                  // 128 x K
    unsigned char *sb = ts_smem + (size_t)TS_M * TS_MAX_NK * 2;   // N x K
    const int tid = threadIdx.x;
    const int warp = tid >> 5;

    if (warp == 0) tmem_alloc(&taddr_s, 256);
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    for (int e = tid; e < TS_M * K; e += blockDim.x) {
        const int r = e / K, k = e % K;
        const uint32_t off = a_mn ? mnmajor_offset(r, k, TS_M) : kmajor_offset(r, k, K);
        *reinterpret_cast<__nv_bfloat16 *>(sa + off) = A[e];
    }
    for (int e = tid; e < N * K; e += blockDim.x) {
        const int r = e / K, k = e % K;
        const uint32_t off = b_mn ? mnmajor_offset(r, k, N) : kmajor_offset(r, k, K);
        *reinterpret_cast<__nv_bfloat16 *>(sb + off) = B[e];
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = taddr_s;
    if (tid == 0) {
        const uint32_t a_lbo = a_mn ? TS_M * 16 : 128, a_sbo = a_mn ? 128 : K * 16;
        const uint32_t b_lbo = b_mn ? N * 16 : 128, b_sbo = b_mn ? 128 : K * 16;
        const uint32_t idesc = idesc_bf16_f32(TS_M, N, a_mn != 0, b_mn != 0);
        for (int kk = 0; kk < K / 16; ++kk) {
            const uint64_t ad = smem_desc(smem_u32(sa) + kk * 2 * a_lbo, a_lbo, a_sbo);
            const uint64_t bd = smem_desc(smem_u32(sb) + kk * 2 * b_lbo, b_lbo, b_sbo);
            umma_bf16(tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        umma_commit(&bar);
    }
    const bool done = mbar_wait(&bar, 0);
    if (!done && (tid & 31) == 0) atomicOr(status, ST_WAIT_TIMEOUT);
    tc_fence_after();
    if (__syncthreads_and(done)) {
        const int row = warp * 32 + (tid & 31);
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            for (int j = 0; j < 16; ++j) C[(size_t)row * N + c0 + j] = v[j];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

}  // namespace gs

// Test entry point (no counterpart in the reference).
extern "C" int gsgpu_tc_gemm_selftest(int N, int K, int a_mn_major, int b_mn_major,
                                      const uint16_t *hA, const uint16_t *hB, float *hC)
{
    using namespace gs;
    if (!hA || !hB || !hC) return GRAV_POINTER_ERROR;
    // N, K <= 128 keeps every operand address inside the 128 KiB of shared
    // memory below for any reading of the descriptor's two byte offsets.
    if (N < 16 || N > 128 || N % 16 != 0 || K < 16 || K > 128 || K % 16 != 0)
        return GRAV_VALUE_ERROR;
    const DeviceInfo *dev = nullptr;
    ErrorStatus st = device_info(&dev);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    DBuf a, b, c, s;
    st = a.reserve((size_t)TS_M * K * 2);
    if (st.return_code == GRAV_SUCCESS) st = b.reserve((size_t)N * K * 2);
    if (st.return_code == GRAV_SUCCESS) st = c.reserve((size_t)TS_M * N * 4);
    if (st.return_code == GRAV_SUCCESS) st = s.reserve(sizeof(unsigned));
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    const size_t smem = (size_t)2 * TS_M * TS_MAX_NK * 2;
    cudaError_t e = cudaMemcpy(a.p, hA, (size_t)TS_M * K * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b.p, hB, (size_t)N * K * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(s.p, 0, sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tc_gemm_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
    if (e == cudaSuccess) {
        k_tc_gemm_selftest<<<1, 128, smem>>>(a.as<__nv_bfloat16>(), b.as<__nv_bfloat16>(), N, K,
                                             a_mn_major, b_mn_major, c.as<float>(),
                                             s.as<unsigned>());
        e = cudaGetLastError();
    }
    unsigned hs = 0;
    if (e == cudaSuccess) e = cudaMemcpy(hC, c.p, (size_t)TS_M * N * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&hs, s.p, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "gsgpu_tc_gemm_selftest: %s\n", cudaGetErrorString(e));
        return GRAV_FAILURE;
    }
    return hs ? GRAV_FAILURE : GRAV_SUCCESS;
}

namespace gs {

// A bounded wait that runs out: thread 0 waits on an mbarrier that no
// thread arrives at, polling %globaltimer; after limit_ns it gives up and
// records ST_WAIT_TIMEOUT, and the kernel ends normally.  This is the exit
// every wait of the library's kernels takes (mbar_wait: 2 s), exercised
// with a short limit.
__global__ void k_wait_timeout_selftest(unsigned long long limit_ns, unsigned *status)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    bool done = mbar_try_wait(&bar, 0);
    const unsigned long long t0 = global_ns();
    while (!done && global_ns() - t0 <= limit_ns) done = mbar_try_wait(&bar, 0);
    if (!done) atomicOr(status, ST_WAIT_TIMEOUT);
}

}  // namespace gs

// Test entry point (no counterpart in the reference): runs the expiring
// wait with a limit of limit_ms (1..2000) and returns the status word.
extern "C" int gsgpu_wait_timeout_selftest(double limit_ms, unsigned *status_out)
{
    using namespace gs;
    if (!status_out) return GRAV_POINTER_ERROR;
    if (!(limit_ms >= 1.0 && limit_ms <= 2000.0)) return GRAV_VALUE_ERROR;
    const DeviceInfo *dev = nullptr;
    ErrorStatus st = device_info(&dev);
    if (st.return_code == GRAV_SUCCESS) {
        DBuf s;
        st = s.reserve(sizeof(unsigned));
        if (st.return_code == GRAV_SUCCESS) {
            cudaError_t e = cudaMemset(s.p, 0, sizeof(unsigned));
            if (e == cudaSuccess) {
                k_wait_timeout_selftest<<<1, 32>>>((unsigned long long)(limit_ms * 1e6),
                                                   s.as<unsigned>());
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMemcpy(status_out, s.p, sizeof(unsigned), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) st = GS_RAISE(GRAV_FAILURE, "wait selftest: %s", cudaGetErrorString(e));
        }
    }
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return GRAV_SUCCESS;
}
