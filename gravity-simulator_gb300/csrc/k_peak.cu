// k_peak.cu -- FP32 / FP64 FMA throughput probes.
//
// The roofline of the direct sum and of the tree walk is the FP32 pipe (and
// of the WHFast Kepler drift the FP64 pipe), whose peaks are not among the
// measured copy-bandwidth and GEMM figures.  These probes measure them on
// the running GPU: every thread runs 8 independent FMA chains, 2 FLOP per
// FMA, on a grid of 8 CTAs of 256 threads per SM.
#include "gs_internal.h"

namespace gs {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chain(T *out, T a0, T b, int iters)
{
    T c[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = a0 + (T)(threadIdx.x + k);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k] = fma(c[k], b, a0);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += c[k];
    if (s == (T)-1.2345) out[blockIdx.x] = s;   // keeps the chains live
}

template <typename T>
static ErrorStatus measure(double *tflops, double *ms_out)
{
    const DeviceInfo *d = nullptr;
    GS_TRY(device_info(&d));
    const int grid = d->sm_count * 8;
    const int iters = sizeof(T) == 4 ? 8192 : 1024;
    DBuf out;
    GS_TRY(out.reserve(sizeof(T) * grid));
    cudaEvent_t e0, e1;
    GS_CUDA(cudaEventCreate(&e0));
    GS_CUDA(cudaEventCreate(&e1));
    k_fma_chain<T><<<grid, 256>>>(out.as<T>(), (T)0.5, (T)0.999, iters);   // warm-up
    GS_CUDA(cudaGetLastError());
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        GS_CUDA(cudaEventRecord(e0));
        k_fma_chain<T><<<grid, 256>>>(out.as<T>(), (T)0.5, (T)0.999, iters);
        GS_CUDA(cudaEventRecord(e1));
        GS_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        GS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flop = 2.0 * 8.0 * (double)iters * 256.0 * grid;
    *tflops = flop / (best * 1e-3) / 1e12;
    if (ms_out) *ms_out = best;
    return ok();
}

}  // namespace gs

extern "C" int gsgpu_measure_fma_peak(int fp64, double *tflops, double *ms)
{
    ErrorStatus st = fp64 ? gs::measure<double>(tflops, ms) : gs::measure<float>(tflops, ms);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}
