// k_massless.cu -- massive/massless direct sum (GRAV_GPU_MASSLESS).
//
// Replaces acceleration_massless (src/acceleration.c:236-367).  Particles
// with m != 0 ("massive") interact pairwise; every massless particle feels
// every massive one; massless particles exert nothing.  FP64 throughout, in
// the reference's operation order with every product and sum rounded alone,
// so the result equals the reference's bit for bit:
//   * k_mass_flags / k_mass_scatter: stable partition of particle indices
//     into the massive and massless lists (array order kept);
//   * k_massive_pairs: one thread per massive particle, the reference's
//     symmetric i<j loop seen from that particle (terms in list order);
//   * k_massless_from_massive: one thread per massless particle, terms in
//     massive-list order, weighted by m[p] with p the massive loop index --
//     the reference reads the mass array at the loop index (:357-359),
//     which equals the massive particle's own mass when massive particles
//     come first in the arrays.
#include "gs_internal.h"
#include "gs_ptx.cuh"

namespace gs {

constexpr int ML_THREADS = 256;
constexpr int ML_TILE = 4096;

__global__ void __launch_bounds__(ML_THREADS)
k_mass_flags(const double *__restrict__ m, int n, unsigned *__restrict__ tile_heavy)
{
    __shared__ unsigned red[ML_THREADS];
    unsigned c = 0;
    const int base = blockIdx.x * ML_TILE;
    for (int k = threadIdx.x; k < ML_TILE; k += ML_THREADS) {
        const int i = base + k;
        if (i < n && m[i] != 0.0) ++c;
    }
    red[threadIdx.x] = c;
    __syncthreads();
    for (int w = ML_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_heavy[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(1024) k_scan_tiles(unsigned *__restrict__ v, int len,
                                                     int *__restrict__ total)
{
    __shared__ unsigned part[1024];
    const int per = (len + 1023) / 1024;
    const int b = threadIdx.x * per;
    const int e = min(len, b + per);
    unsigned s = 0;
    for (int i = b; i < e; ++i) s += v[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const unsigned t = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    unsigned run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (int i = b; i < e; ++i) {
        const unsigned c = v[i];
        v[i] = run;
        run += c;
    }
    if (threadIdx.x == 1023) *total = (int)part[1023];
}

// Stable scatter of indices: massive ones to heavy[], massless to light[].
__global__ void __launch_bounds__(ML_THREADS)
k_mass_scatter(const double *__restrict__ m, int n, const unsigned *__restrict__ tile_off,
               int *__restrict__ heavy, int *__restrict__ light)
{
    constexpr int PER = ML_TILE / ML_THREADS;
    __shared__ unsigned part[ML_THREADS];
    const int base = blockIdx.x * ML_TILE + threadIdx.x * PER;
    unsigned c = 0;
    for (int k = 0; k < PER; ++k) {
        const int i = base + k;
        if (i < n && m[i] != 0.0) ++c;
    }
    part[threadIdx.x] = c;
    __syncthreads();
    for (int off = 1; off < ML_THREADS; off <<= 1) {
        const unsigned t = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    unsigned h = tile_off[blockIdx.x] + (threadIdx.x ? part[threadIdx.x - 1] : 0u);
    for (int k = 0; k < PER; ++k) {
        const int i = base + k;
        if (i >= n) break;
        if (m[i] != 0.0)
            heavy[h++] = i;
        else
            light[i - (int)h] = i;   // massless rank = index - massive before it
    }
}

__device__ __forceinline__ void pair_fp64(double xi0, double xi1, double xi2, double xj0,
                                          double xj1, double xj2, double eps2, double G,
                                          double &t, double &r0, double &r1, double &r2)
{
    r0 = __dsub_rn(xi0, xj0);
    r1 = __dsub_rn(xi1, xj1);
    r2 = __dsub_rn(xi2, xj2);
    const double s = __dadd_rn(
        __dadd_rn(__dadd_rn(__dmul_rn(r0, r0), __dmul_rn(r1, r1)), __dmul_rn(r2, r2)), eps2);
    const double rn = __dsqrt_rn(s);
    t = __ddiv_rn(G, __dmul_rn(__dmul_rn(rn, rn), rn));
}

// Massive particles: terms from all other massive particles in list order
// (src/acceleration.c:299-333 seen from one particle).
__global__ void k_massive_pairs(const double *__restrict__ x, const double *__restrict__ m,
                                const int *__restrict__ heavy, const int *__restrict__ counts,
                                double G, double eps2, double *__restrict__ a)
{
    const int nh = counts[0];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nh; p += gridDim.x * blockDim.x) {
        const int i = heavy[p];
        const double xi0 = x[3 * i], xi1 = x[3 * i + 1], xi2 = x[3 * i + 2];
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int q = 0; q < nh; ++q) {
            if (q == p) continue;
            const int j = heavy[q];
            double t, r0, r1, r2;
            pair_fp64(xi0, xi1, xi2, x[3 * j], x[3 * j + 1], x[3 * j + 2], eps2, G, t, r0, r1, r2);
            const double mj = m[j];
            a0 = __dsub_rn(a0, __dmul_rn(__dmul_rn(t, r0), mj));
            a1 = __dsub_rn(a1, __dmul_rn(__dmul_rn(t, r1), mj));
            a2 = __dsub_rn(a2, __dmul_rn(__dmul_rn(t, r2), mj));
        }
        a[3 * i] = a0;
        a[3 * i + 1] = a1;
        a[3 * i + 2] = a2;
    }
}

// Massless particles (src/acceleration.c:336-361): a_j += (t * R) * m[p].
__global__ void k_massless_from_massive(const double *__restrict__ x, const double *__restrict__ m,
                                        const int *__restrict__ heavy,
                                        const int *__restrict__ light,
                                        const int *__restrict__ counts, int n, double G,
                                        double eps2, double *__restrict__ a)
{
    const int nh = counts[0];
    const int nl = n - nh;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nl; q += gridDim.x * blockDim.x) {
        const int j = light[q];
        const double xj0 = x[3 * j], xj1 = x[3 * j + 1], xj2 = x[3 * j + 2];
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int p = 0; p < nh; ++p) {
            const int i = heavy[p];
            double t, r0, r1, r2;
            pair_fp64(x[3 * i], x[3 * i + 1], x[3 * i + 2], xj0, xj1, xj2, eps2, G, t, r0, r1, r2);
            const double mp = m[p];
            a0 = __dadd_rn(a0, __dmul_rn(__dmul_rn(t, r0), mp));
            a1 = __dadd_rn(a1, __dmul_rn(__dmul_rn(t, r1), mp));
            a2 = __dadd_rn(a2, __dmul_rn(__dmul_rn(t, r2), mp));
        }
        a[3 * j] = a0;
        a[3 * j + 1] = a1;
        a[3 * j + 2] = a2;
    }
}

namespace {

class MasslessEngine final : public Engine {
  public:
    ErrorStatus setup(int n, double G, const AccelerationParam &p) override
    {
        n_ = n;
        G_ = G;
        eps_ = p.softening_length;
        tiles_ = (n + ML_TILE - 1) / ML_TILE;
        GS_TRY(heavy_.reserve((size_t)n * sizeof(int)));
        GS_TRY(light_.reserve((size_t)n * sizeof(int)));
        GS_TRY(tile_.reserve((size_t)(tiles_ + 1) * sizeof(unsigned)));
        GS_TRY(count_.reserve(sizeof(int) * 2));
        const DeviceInfo *d = nullptr;
        GS_TRY(device_info(&d));
        sms_ = d->sm_count;
        return ok();
    }

    ErrorStatus compute(const double *d_x, const double *d_m, double *d_a, cudaStream_t s,
                        ForceTimer *timer) override
    {
        k_mass_flags<<<tiles_, ML_THREADS, 0, s>>>(d_m, n_, tile_.as<unsigned>());
        k_scan_tiles<<<1, 1024, 0, s>>>(tile_.as<unsigned>(), tiles_, count_.as<int>());
        k_mass_scatter<<<tiles_, ML_THREADS, 0, s>>>(d_m, n_, tile_.as<unsigned>(), heavy_.as<int>(),
                                                     light_.as<int>());
        GS_CUDA(cudaGetLastError());
        const double eps2 = eps_ * eps_;
        const int grid = sms_ * 4;
        if (timer) GS_TRY(timer->begin(s));
        k_massive_pairs<<<grid, 128, 0, s>>>(d_x, d_m, heavy_.as<int>(), count_.as<int>(), G_, eps2,
                                             d_a);
        k_massless_from_massive<<<grid, 128, 0, s>>>(d_x, d_m, heavy_.as<int>(), light_.as<int>(),
                                                     count_.as<int>(), n_, G_, eps2, d_a);
        GS_CUDA(cudaGetLastError());
        if (timer) GS_TRY(timer->end(s));
        return ok();
    }

    int kernels_per_eval() const override { return 5; }

  private:
    int n_ = 0, tiles_ = 0, sms_ = 1;
    double G_ = 1.0, eps_ = 0.0;
    DBuf heavy_, light_, tile_, count_;
};

}  // namespace

std::unique_ptr<Engine> make_massless_engine()
{
    return std::unique_ptr<Engine>(new MasslessEngine());
}

}  // namespace gs
