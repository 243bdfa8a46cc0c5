// k_direct.cu -- direct-sum accelerations on sm_103a.
//
// Replaces acceleration_pairwise (src/acceleration.c:177-234).
//
// GRAV_GPU_PAIRWISE (compensated FP32):
//   * positions and masses are packed once per evaluation into a float4
//     array (x, y, z, m) relative to a fixed frame centre, padded to a whole
//     number of 1024-particle tiles with massless far-away particles;
//   * a CTA of 128 threads owns 1024 i-particles (8 per thread, register
//     blocked; two CTAs per SM) and one contiguous j-chunk; j-tiles of 1024
//     particles (16 KiB)
//     stream through a 3-stage shared-memory ring filled by TMA bulk copies
//     (cp.async.bulk + mbarrier complete_tx), read back as broadcast float4;
//   * each pair term is 3 FADD + 3 FFMA + rsqrt + 3 FMUL + 3 FFMA in FP32;
//     each partial sum of 128 pair terms is added into a Kahan-compensated FP32
//     accumulator;
//   * the (i-tile, j-chunk) work units are sized so that their count is a
//     whole number of waves of resident CTAs (152 SMs x occupancy); partial
//     sums go to an FP64 scratch array [split][3][N] that a second kernel
//     reduces in fixed order and scales by G.
//
// GRAV_GPU_PAIRWISE_FP64 (reference order): a warp per ten particles forms
// the pair terms of all other particles, 32 at a time, and sums them in index
// order with every FP64 product, sum, sqrt and quotient rounded separately --
// the same operations as the reference's symmetric loop applies to that
// particle, so the result equals the reference's bit for bit where the
// reference is not FMA-contracted.
#include "gs_internal.h"
#include "gs_ptx.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

namespace gs {

constexpr int DS_THREADS = 128;
constexpr int DS_IPT = 8;
constexpr int DS_ITILE = DS_THREADS * DS_IPT;  // 1024
constexpr int DS_JTILE = 1024;                 // 16 KiB of float4
constexpr int DS_STAGES = 3;
constexpr int DS_SMEM = DS_STAGES * DS_JTILE * 16;
constexpr int DS_KAHAN_CHUNK = 128;            // plain FP32 partials of 128 terms
static_assert(DS_ITILE == DS_JTILE, "i and j tiles share the padding unit");

// Padding particle: massless and far from everything (its pair terms are 0).
constexpr float kPadPos = 1.0e15f;

__global__ void k_pack_float4(const double *__restrict__ x, const double *__restrict__ m,
                              int n, int n_pad, double cx, double cy, double cz,
                              float4 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    float4 p;
    if (i < n) {
        p.x = (float)(x[3 * i + 0] - cx);
        p.y = (float)(x[3 * i + 1] - cy);
        p.z = (float)(x[3 * i + 2] - cz);
        p.w = (float)m[i];
    } else {
        p = make_float4(kPadPos, kPadPos, kPadPos, 0.0f);
    }
    out[i] = p;
}

template <bool SOFT>
__device__ __forceinline__ void pair_term(const float4 q, float xi, float yi, float zi,
                                          float eps2, float &ax, float &ay, float &az)
{
    const float dx = q.x - xi;
    const float dy = q.y - yi;
    const float dz = q.z - zi;
    float r2 = fmaf(dx, dx, eps2);
    r2 = fmaf(dy, dy, r2);
    r2 = fmaf(dz, dz, r2);
    float ri = rsqrt_approx(r2);
    if (!SOFT) ri = (r2 > 0.0f) ? ri : 0.0f;   // self term without softening
    const float mr = q.w * ri;
    const float ri2 = ri * ri;
    const float s = mr * ri2;
    ax = fmaf(dx, s, ax);
    ay = fmaf(dy, s, ay);
    az = fmaf(dz, s, az);
}

// One (i-tile, j-chunk) work unit: the 1024 i-particles start at pi_tile;
// partial sums go to partial[split][3][plane] at rows itile*1024 + ...
// Two i-particles per instruction: Blackwell's paired FP32 operations
// (add / mul / fma on float2, each lane rounded as the scalar operation)
// carry the pair terms of particles (k, k+1) together, halving the FP32
// instructions issued per term; the arithmetic of each particle is exactly
// pair_term's (q.x - x_i is formed as q.x + (-x_i)).
template <bool SOFT>
__device__ __forceinline__ void pair_term2(const float4 q, float2 nxi, float2 nyi, float2 nzi,
                                           float2 eps2, float2 &ax, float2 &ay, float2 &az)
{
    const float2 dx = __fadd2_rn(make_float2(q.x, q.x), nxi);
    const float2 dy = __fadd2_rn(make_float2(q.y, q.y), nyi);
    const float2 dz = __fadd2_rn(make_float2(q.z, q.z), nzi);
    float2 r2 = __ffma2_rn(dx, dx, eps2);
    r2 = __ffma2_rn(dy, dy, r2);
    r2 = __ffma2_rn(dz, dz, r2);
    float2 ri = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
    if (!SOFT) {
        ri.x = (r2.x > 0.0f) ? ri.x : 0.0f;
        ri.y = (r2.y > 0.0f) ? ri.y : 0.0f;
    }
    const float2 mr = __fmul2_rn(make_float2(q.w, q.w), ri);
    const float2 ri2 = __fmul2_rn(ri, ri);
    const float2 sc = __fmul2_rn(mr, ri2);
    ax = __ffma2_rn(dx, sc, ax);
    ay = __ffma2_rn(dy, sc, ay);
    az = __ffma2_rn(dz, sc, az);
}

template <bool SOFT>
__device__ __forceinline__ void direct_sum_unit(const float4 *__restrict__ pi_tile,
                                                const float4 *__restrict__ pj, int plane,
                                                int itile, int split, int jt_per_chunk,
                                                int jt_total, float eps2,
                                                double *__restrict__ partial,
                                                unsigned *__restrict__ status, float4 *sj,
                                                uint64_t *full_bar)
{
    const int jt0 = split * jt_per_chunk;
    const int ntiles = min(jt_total, jt0 + jt_per_chunk) - jt0;

    float xi[DS_IPT], yi[DS_IPT], zi[DS_IPT];
#pragma unroll
    for (int k = 0; k < DS_IPT; ++k) {
        const float4 p = pi_tile[k * DS_THREADS + threadIdx.x];
        xi[k] = p.x;
        yi[k] = p.y;
        zi[k] = p.z;
    }

    if (threadIdx.x == 0) {
        for (int s = 0; s < DS_STAGES; ++s) mbar_init(&full_bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int pre = min(DS_STAGES, ntiles);
        for (int s = 0; s < pre; ++s) {
            mbar_expect_tx(&full_bar[s], DS_JTILE * 16);
            bulk_g2s(sj + s * DS_JTILE, pj + (size_t)(jt0 + s) * DS_JTILE, DS_JTILE * 16,
                     &full_bar[s]);
        }
    }

    float sx[DS_IPT], sy[DS_IPT], sz[DS_IPT], cx[DS_IPT], cy[DS_IPT], cz[DS_IPT];
#pragma unroll
    for (int k = 0; k < DS_IPT; ++k) {
        sx[k] = sy[k] = sz[k] = 0.0f;
        cx[k] = cy[k] = cz[k] = 0.0f;
    }
    static_assert(DS_IPT % 2 == 0, "i-particles are paired");
    float2 nx2[DS_IPT / 2], ny2[DS_IPT / 2], nz2[DS_IPT / 2];
#pragma unroll
    for (int k = 0; k < DS_IPT / 2; ++k) {
        nx2[k] = make_float2(-xi[2 * k], -xi[2 * k + 1]);
        ny2[k] = make_float2(-yi[2 * k], -yi[2 * k + 1]);
        nz2[k] = make_float2(-zi[2 * k], -zi[2 * k + 1]);
    }
    const float2 eps2v = make_float2(eps2, eps2);

    int issued = min(DS_STAGES, ntiles);
    int t = 0;
    for (; t < ntiles; ++t) {
        const int st = t % DS_STAGES;
        const unsigned parity = (unsigned)(t / DS_STAGES) & 1u;
        const bool ready = mbar_wait(&full_bar[st], parity);
        if (!__syncthreads_and(ready)) {
            if (threadIdx.x == 0) atomicOr(status, ST_WAIT_TIMEOUT);
            break;
        }
        const float4 *tile = sj + st * DS_JTILE;
        for (int j0 = 0; j0 < DS_JTILE; j0 += DS_KAHAN_CHUNK) {
            float2 ax[DS_IPT / 2], ay[DS_IPT / 2], az[DS_IPT / 2];
#pragma unroll
            for (int k = 0; k < DS_IPT / 2; ++k)
                ax[k] = ay[k] = az[k] = make_float2(0.0f, 0.0f);
#pragma unroll 8
            for (int j = j0; j < j0 + DS_KAHAN_CHUNK; ++j) {
                const float4 q = tile[j];
#pragma unroll
                for (int k = 0; k < DS_IPT / 2; ++k)
                    pair_term2<SOFT>(q, nx2[k], ny2[k], nz2[k], eps2v, ax[k], ay[k], az[k]);
            }
#pragma unroll
            for (int k = 0; k < DS_IPT / 2; ++k) {
                kahan_add(sx[2 * k], cx[2 * k], ax[k].x);
                kahan_add(sy[2 * k], cy[2 * k], ay[k].x);
                kahan_add(sz[2 * k], cz[2 * k], az[k].x);
                kahan_add(sx[2 * k + 1], cx[2 * k + 1], ax[k].y);
                kahan_add(sy[2 * k + 1], cy[2 * k + 1], ay[k].y);
                kahan_add(sz[2 * k + 1], cz[2 * k + 1], az[k].y);
            }
        }
        __syncthreads();   // every thread is done with stage st
        if (threadIdx.x == 0 && issued < ntiles) {
            mbar_expect_tx(&full_bar[st], DS_JTILE * 16);
            bulk_g2s(sj + st * DS_JTILE, pj + (size_t)(jt0 + issued) * DS_JTILE, DS_JTILE * 16,
                     &full_bar[st]);
            ++issued;
        }
    }
    if (t < ntiles) {
        // Timed out: let copies already issued land before the CTA exits.
        if (threadIdx.x == 0) {
            for (int u = t; u < issued; ++u)
                (void)mbar_wait(&full_bar[u % DS_STAGES], (unsigned)(u / DS_STAGES) & 1u);
        }
        __syncthreads();
        return;
    }

    double *out = partial + (size_t)split * 3 * (size_t)plane;
#pragma unroll
    for (int k = 0; k < DS_IPT; ++k) {
        const size_t i = (size_t)itile * DS_ITILE + k * DS_THREADS + threadIdx.x;
        out[0 * (size_t)plane + i] = (double)sx[k] - (double)cx[k];
        out[1 * (size_t)plane + i] = (double)sy[k] - (double)cy[k];
        out[2 * (size_t)plane + i] = (double)sz[k] - (double)cz[k];
    }
}

template <bool SOFT>
__global__ void __launch_bounds__(DS_THREADS, 2)
k_direct_sum(const float4 *__restrict__ pj, int n_pad, int i_tiles, int jt_per_chunk,
             int jt_total, float eps2, double *__restrict__ partial,
             unsigned *__restrict__ status)
{
    extern __shared__ __align__(128) unsigned char ds_smem[];
    __shared__ __align__(8) uint64_t full_bar[DS_STAGES];
    const int itile = blockIdx.x % i_tiles;
    const int split = blockIdx.x / i_tiles;
    direct_sum_unit<SOFT>(pj + (size_t)itile * DS_ITILE, pj, n_pad, itile, split, jt_per_chunk,
                          jt_total, eps2, partial, status, reinterpret_cast<float4 *>(ds_smem),
                          full_bar);
}

// Direct sum for a separate list of target particles pi [ni_pad] (padded to
// whole 1024-particle tiles) against all sources pj: the sampled rows of the
// learned method's training targets and per-step judge.
template <bool SOFT>
__global__ void __launch_bounds__(DS_THREADS, 2)
k_direct_rows(const float4 *__restrict__ pi, int ni_pad, const float4 *__restrict__ pj,
              int i_tiles, int jt_per_chunk, int jt_total, float eps2,
              double *__restrict__ partial, unsigned *__restrict__ status)
{
    extern __shared__ __align__(128) unsigned char ds_smem[];
    __shared__ __align__(8) uint64_t full_bar[DS_STAGES];
    const int itile = blockIdx.x % i_tiles;
    const int split = blockIdx.x / i_tiles;
    direct_sum_unit<SOFT>(pi + (size_t)itile * DS_ITILE, pj, ni_pad, itile, split, jt_per_chunk,
                          jt_total, eps2, partial, status, reinterpret_cast<float4 *>(ds_smem),
                          full_bar);
}

// a_i = G * sum_s partial[s][.][i], summed in split order.
__global__ void k_reduce_splits(const double *__restrict__ partial, int splits, int n,
                                int n_pad, double G, double *__restrict__ a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t plane = (size_t)n_pad;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int s = 0; s < splits; ++s) {
        const double *p = partial + (size_t)s * 3 * plane;
        s0 += p[i];
        s1 += p[plane + i];
        s2 += p[2 * plane + i];
    }
    a[3 * i + 0] = G * s0;
    a[3 * i + 1] = G * s1;
    a[3 * i + 2] = G * s2;
}

// FP64, reference operation order (see file comment).  One warp per PER
// particles: for 32 consecutive j the lanes form the pair terms of the PER
// particles (each term is independent), then lane 3p + c subtracts the
// component-c terms of particle p from its accumulator one by one in j
// order, which is the order the reference's loop adds them to a_i.  With
// PER = 10, ten particles share each in-order accumulation instruction (30
// of 32 lanes); with PER = 1 there are ten times as many warps, which small
// systems need to fill the GPU.
constexpr int RF_WARPS = 4;
constexpr int RF_PER_WARP_LARGE = 10;
constexpr int RF_LARGE_N = 32768;   // from here on, ten particles per warp

template <int RF_PER_WARP>
__global__ void __launch_bounds__(32 * RF_WARPS)
k_direct_fp64_reference_order(const double *__restrict__ x, const double *__restrict__ m,
                              int n, double G, double eps2, double *__restrict__ a)
{
    __shared__ double terms[RF_WARPS][RF_PER_WARP * 3][32];
    __shared__ double xi_s[RF_WARPS][RF_PER_WARP * 3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i0 = (blockIdx.x * RF_WARPS + w) * RF_PER_WARP;
    if (i0 >= n) return;   // warp-uniform
    const int np = min(RF_PER_WARP, n - i0);
    if (lane < 3 * np) xi_s[w][lane] = x[3 * i0 + lane];
    __syncwarp();
    double acc = 0.0;   // lane 3p + c < 3 np: component c of a_(i0 + p)
    for (int base = 0; base < n; base += 32) {
        const int j = base + lane;
        double xj0 = 0.0, xj1 = 0.0, xj2 = 0.0, mj = 0.0;
        if (j < n) {
            xj0 = x[3 * j + 0];
            xj1 = x[3 * j + 1];
            xj2 = x[3 * j + 2];
            mj = m[j];
        }
        for (int p = 0; p < np; ++p) {
            double t0 = 0.0, t1 = 0.0, t2 = 0.0;
            if (j < n && j != i0 + p) {
                const double r0 = __dsub_rn(xi_s[w][3 * p + 0], xj0);
                const double r1 = __dsub_rn(xi_s[w][3 * p + 1], xj1);
                const double r2 = __dsub_rn(xi_s[w][3 * p + 2], xj2);
                const double s = __dadd_rn(
                    __dadd_rn(__dadd_rn(__dmul_rn(r0, r0), __dmul_rn(r1, r1)), __dmul_rn(r2, r2)),
                    eps2);
                const double rn = __dsqrt_rn(s);
                const double t = __ddiv_rn(G, __dmul_rn(__dmul_rn(rn, rn), rn));
                t0 = __dmul_rn(__dmul_rn(t, r0), mj);
                t1 = __dmul_rn(__dmul_rn(t, r1), mj);
                t2 = __dmul_rn(__dmul_rn(t, r2), mj);
            }
            terms[w][3 * p + 0][lane] = t0;
            terms[w][3 * p + 1][lane] = t1;
            terms[w][3 * p + 2][lane] = t2;
        }
        __syncwarp();
        if (lane < 3 * np) {
            const int cnt = min(32, n - base);
            const int self = i0 + lane / 3 - base;   // this particle's own slot, if in the chunk
            const double *tc = terms[w][lane];
            for (int q = 0; q < cnt; ++q)
                if (q != self) acc = __dsub_rn(acc, tc[q]);
        }
        __syncwarp();
    }
    if (lane < 3 * np) a[3 * i0 + lane] = acc;
}

// ------------------------------------------------------------------------
namespace {

class DirectEngine final : public Engine {
  public:
    explicit DirectEngine(bool fp64) : fp64_(fp64) {}

    ErrorStatus setup(int n, double G, const AccelerationParam &p) override
    {
        n_ = n;
        G_ = G;
        eps_ = p.softening_length;
        if (fp64_) return ok();
        const DeviceInfo *dev = nullptr;
        GS_TRY(device_info(&dev));
        n_pad_ = ((n + DS_JTILE - 1) / DS_JTILE) * DS_JTILE;
        i_tiles_ = n_pad_ / DS_ITILE;
        jt_total_ = n_pad_ / DS_JTILE;
        int per_sm = 0;
        GS_CUDA(cudaFuncSetAttribute(k_direct_sum<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     DS_SMEM));
        GS_CUDA(cudaFuncSetAttribute(k_direct_sum<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     DS_SMEM));
        GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_direct_sum<true>, DS_THREADS,
                                                              DS_SMEM));
        per_sm = std::max(per_sm, 1);
        const long slots = (long)dev->sm_count * per_sm;
        // Choose the j-split count: minimise (waves x tiles per unit) with a
        // small per-unit overhead, so the last wave is (nearly) full.
        int best_s = 1;
        double best_cost = 1e300;
        const int max_s = std::min(jt_total_, 64);
        for (int s = 1; s <= max_s; ++s) {
            const int chunk = (jt_total_ + s - 1) / s;
            const int used = (jt_total_ + chunk - 1) / chunk;   // non-empty splits
            const long units = (long)i_tiles_ * used;
            const long waves = (units + slots - 1) / slots;
            const double cost = (double)waves * (chunk + 0.25);
            if (cost < best_cost - 1e-9) {
                best_cost = cost;
                best_s = used;
                jt_per_chunk_ = chunk;
            }
        }
        splits_ = best_s;
        GS_TRY(pj_.reserve((size_t)n_pad_ * sizeof(float4)));
        GS_TRY(partial_.reserve((size_t)splits_ * 3 * n_pad_ * sizeof(double)));
        GS_TRY(status_.reserve(sizeof(unsigned)));
        GS_CUDA(cudaMemset(status_.p, 0, sizeof(unsigned)));
        return ok();
    }

    void set_frame_centre(double cx, double cy, double cz) override
    {
        c_[0] = cx;
        c_[1] = cy;
        c_[2] = cz;
    }

    ErrorStatus compute(const double *d_x, const double *d_m, double *d_a, cudaStream_t s,
                        ForceTimer *timer) override
    {
        if (fp64_) {
            const bool large = n_ >= RF_LARGE_N;
            const int per_cta = RF_WARPS * (large ? RF_PER_WARP_LARGE : 1);
            const int grid = (n_ + per_cta - 1) / per_cta;
            if (timer) GS_TRY(timer->begin(s));
            auto kernel = large ? k_direct_fp64_reference_order<RF_PER_WARP_LARGE>
                                : k_direct_fp64_reference_order<1>;
            kernel<<<grid, 32 * RF_WARPS, 0, s>>>(d_x, d_m, n_, G_, eps_ * eps_,
                                                                      d_a);
            GS_CUDA(cudaGetLastError());
            if (timer) GS_TRY(timer->end(s));
            return ok();
        }
        k_pack_float4<<<(n_pad_ + 255) / 256, 256, 0, s>>>(d_x, d_m, n_, n_pad_, c_[0], c_[1], c_[2],
                                                           pj_.as<float4>());
        GS_CUDA(cudaGetLastError());
        const float eps2 = (float)(eps_ * eps_);
        const int grid = i_tiles_ * splits_;
        if (timer) GS_TRY(timer->begin(s));
        if (eps2 > 0.0f)
            k_direct_sum<true><<<grid, DS_THREADS, DS_SMEM, s>>>(
                pj_.as<float4>(), n_pad_, i_tiles_, jt_per_chunk_, jt_total_, eps2,
                partial_.as<double>(), status_.as<unsigned>());
        else
            k_direct_sum<false><<<grid, DS_THREADS, DS_SMEM, s>>>(
                pj_.as<float4>(), n_pad_, i_tiles_, jt_per_chunk_, jt_total_, eps2,
                partial_.as<double>(), status_.as<unsigned>());
        GS_CUDA(cudaGetLastError());
        if (timer) GS_TRY(timer->end(s));
        k_reduce_splits<<<(n_ + 255) / 256, 256, 0, s>>>(partial_.as<double>(), splits_, n_, n_pad_,
                                                         G_, d_a);
        GS_CUDA(cudaGetLastError());
        return ok();
    }

    int kernels_per_eval() const override { return fp64_ ? 1 : 3; }

    ErrorStatus check_status(cudaStream_t s) override
    {
        if (fp64_) return ok();
        unsigned h = 0;
        GS_CUDA(cudaMemcpyAsync(&h, status_.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        GS_CUDA(cudaStreamSynchronize(s));
        if (h & ST_WAIT_TIMEOUT)
            return GS_RAISE(GRAV_FAILURE, "direct-sum kernel: shared-memory tile wait timed out");
        return ok();
    }

  private:
    bool fp64_;
    int n_ = 0, n_pad_ = 0, i_tiles_ = 0, jt_total_ = 0, jt_per_chunk_ = 1, splits_ = 1;
    double G_ = 1.0, eps_ = 0.0;
    double c_[3] = {0.0, 0.0, 0.0};
    DBuf pj_, partial_, status_;
};

}  // namespace

std::unique_ptr<Engine> make_direct_engine(bool fp64_reference_order)
{
    return std::unique_ptr<Engine>(new DirectEngine(fp64_reference_order));
}

// ---- direct sum over selected rows ----------------------------------------
// Sources packed relative to frame[0..2] (a device FP64 centre).
__global__ void k_pack_frame(const double *__restrict__ x, const double *__restrict__ m, int n,
                             int n_pad, const double *__restrict__ frame, float4 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    float4 p;
    if (i < n) {
        p.x = (float)(x[3 * i + 0] - frame[0]);
        p.y = (float)(x[3 * i + 1] - frame[1]);
        p.z = (float)(x[3 * i + 2] - frame[2]);
        p.w = (float)m[i];
    } else {
        p = make_float4(kPadPos, kPadPos, kPadPos, 0.0f);
    }
    out[i] = p;
}

__global__ void k_gather_rows(const float4 *__restrict__ pj, const int *__restrict__ rows,
                              int nrows, int nrows_pad, float4 *__restrict__ pi)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows_pad) return;
    pi[r] = r < nrows ? pj[rows[r]] : make_float4(kPadPos, kPadPos, kPadPos, 0.0f);
}

void DirectRows::split_for(int i_tiles, int max_splits, int *splits, int *chunk) const
{
    double best = 1e300;
    *splits = 1;
    *chunk = jt_total_;
    for (int s = 1; s <= std::min(jt_total_, max_splits); ++s) {
        const int c = (jt_total_ + s - 1) / s;
        const int used = (jt_total_ + c - 1) / c;
        const long units = (long)i_tiles * used;
        const double cost = (double)((units + slots_ - 1) / slots_) * (c + 0.25);
        if (cost < best - 1e-9) {
            best = cost;
            *splits = used;
            *chunk = c;
        }
    }
}

ErrorStatus DirectRows::setup(int nj, int max_rows)
{
    const DeviceInfo *dev = nullptr;
    GS_TRY(device_info(&dev));
    nj_ = nj;
    nj_pad_ = ((nj + DS_JTILE - 1) / DS_JTILE) * DS_JTILE;
    ni_pad_ = ((max_rows + DS_ITILE - 1) / DS_ITILE) * DS_ITILE;
    jt_total_ = nj_pad_ / DS_JTILE;
    int per_sm = 0;
    GS_CUDA(cudaFuncSetAttribute(k_direct_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 DS_SMEM));
    GS_CUDA(cudaFuncSetAttribute(k_direct_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 DS_SMEM));
    GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_direct_rows<true>, DS_THREADS,
                                                          DS_SMEM));
    slots_ = (long)dev->sm_count * std::max(per_sm, 1);
    // Partial sums sized for the largest launch and for a launch of a single
    // row tile, which splits the j range most finely.
    int sp = 1, ch = 1;
    split_for(ni_pad_ / DS_ITILE, 128, &sp, &ch);
    partial_rows_ = (size_t)sp * ni_pad_;
    split_for(1, 128, &sp, &ch);
    partial_rows_ = std::max(partial_rows_, (size_t)sp * DS_ITILE);
    GS_TRY(pj_.reserve((size_t)nj_pad_ * sizeof(float4)));
    GS_TRY(pi_.reserve((size_t)ni_pad_ * sizeof(float4)));
    GS_TRY(partial_.reserve(partial_rows_ * 3 * sizeof(double)));
    GS_TRY(status_.reserve(sizeof(unsigned)));
    GS_CUDA(cudaMemset(status_.p, 0, sizeof(unsigned)));
    return ok();
}

ErrorStatus DirectRows::compute(const double *d_x, const double *d_m, const double *d_frame,
                                const int *d_rows, int nrows, double G, double eps, double *d_a_rows,
                                cudaStream_t s, ForceTimer *timer)
{
    if (nrows <= 0) return ok();
    if (((nrows + DS_ITILE - 1) / DS_ITILE) * DS_ITILE > ni_pad_)
        return GS_RAISE(GRAV_VALUE_ERROR, "direct rows: %d rows exceed the prepared %d", nrows, ni_pad_);
    k_pack_frame<<<(nj_pad_ + 255) / 256, 256, 0, s>>>(d_x, d_m, nj_, nj_pad_, d_frame,
                                                       pj_.as<float4>());
    const int nr_pad = ((nrows + DS_ITILE - 1) / DS_ITILE) * DS_ITILE;
    k_gather_rows<<<(nr_pad + 255) / 256, 256, 0, s>>>(pj_.as<float4>(), d_rows, nrows, nr_pad,
                                                       pi_.as<float4>());
    const float eps2 = (float)(eps * eps);
    const int i_tiles = nr_pad / DS_ITILE;
    // the split is chosen for this launch's row count (few rows: many
    // j-chunks, so that the launch still fills every SM)
    int splits = 1, chunk = jt_total_;
    split_for(i_tiles, (int)std::min<size_t>(128, partial_rows_ / nr_pad), &splits, &chunk);
    if (timer) GS_TRY(timer->begin(s));
    if (eps2 > 0.0f)
        k_direct_rows<true><<<i_tiles * splits, DS_THREADS, DS_SMEM, s>>>(
            pi_.as<float4>(), nr_pad, pj_.as<float4>(), i_tiles, chunk, jt_total_, eps2,
            partial_.as<double>(), status_.as<unsigned>());
    else
        k_direct_rows<false><<<i_tiles * splits, DS_THREADS, DS_SMEM, s>>>(
            pi_.as<float4>(), nr_pad, pj_.as<float4>(), i_tiles, chunk, jt_total_, eps2,
            partial_.as<double>(), status_.as<unsigned>());
    if (timer) GS_TRY(timer->end(s));
    k_reduce_splits<<<(nrows + 255) / 256, 256, 0, s>>>(partial_.as<double>(), splits, nrows,
                                                        nr_pad, G, d_a_rows);
    GS_CUDA(cudaGetLastError());
    return ok();
}

ErrorStatus DirectRows::check(cudaStream_t s)
{
    unsigned h = 0;
    GS_CUDA(cudaMemcpyAsync(&h, status_.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
    if (h) {
        GS_CUDA(cudaMemsetAsync(status_.p, 0, sizeof(unsigned), s));
        if (h & ST_WAIT_TIMEOUT)
            return GS_RAISE(GRAV_FAILURE, "direct-sum rows kernel: shared-memory tile wait timed out");
    }
    return ok();
}

// ------------------------------------------------------------------------
// Allocation-free compensated-FP32 direct sum.
//
// For callers that cannot allocate device memory while they run: code that
// records or replays a fixed plan of work and may not call cudaMalloc
// (which can synchronise the device) in the middle of it, embedders whose
// allocator is a pool they own, and real-time loops that must not touch the
// allocator at all.  This entry point computes the same accelerations as
// acceleration() with GRAV_GPU_PAIRWISE, from device arrays the caller
// owns, using the same kernels; its scratch (the packed float4 particles,
// the per-split partial sums, the status word and the frame centre) lives
// in one file-scope device array instead of memory the library allocates.
// That array is part of the library image: every GPU that loads the library
// holds its NOALLOC_BYTES (about 6.5 MiB) until the process exits.
//
// Like acceleration(), it takes positions relative to the centre of their
// bounding box before rounding them to FP32; here that centre is reduced on
// the device (k_noalloc_frame) into the scratch array, so that systems far
// from the origin keep their accuracy.  A bulk-copy wait that runs out in
// k_direct_sum sets the status word, and the reduction then writes NaN into
// every output row instead of partial sums.
constexpr int NOALLOC_MAX_N = 32768;      // largest particle count accepted
constexpr int NOALLOC_MAX_SPLITS = 8;
constexpr size_t NOALLOC_PJ_BYTES = (size_t)NOALLOC_MAX_N * sizeof(float4);
constexpr size_t NOALLOC_PARTIAL_BYTES =
    (size_t)NOALLOC_MAX_SPLITS * 3 * NOALLOC_MAX_N * sizeof(double);
constexpr size_t NOALLOC_BYTES = NOALLOC_PJ_BYTES + NOALLOC_PARTIAL_BYTES + 256;
static_assert(NOALLOC_MAX_N % DS_JTILE == 0, "capacity must be whole tiles");
// The last 256 bytes: the status word at offset 0, the FP64 frame centre at 64.
constexpr size_t NOALLOC_STATUS_OFF = NOALLOC_PJ_BYTES + NOALLOC_PARTIAL_BYTES;
constexpr size_t NOALLOC_FRAME_OFF = NOALLOC_STATUS_OFF + 64;
static_assert(NOALLOC_FRAME_OFF + 3 * sizeof(double) <= NOALLOC_BYTES, "tail holds the frame");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Centre of the bounding box of x [n] (one CTA), formed as acceleration()
// forms it on the host: per axis the exact minimum and maximum, then
// 0.5 (lo + hi).
constexpr int NA_FRAME_THREADS = 1024;
__global__ void __launch_bounds__(NA_FRAME_THREADS)
k_noalloc_frame(const double *__restrict__ x, int n, double *__restrict__ frame)
{
    __shared__ double lo_s[3][NA_FRAME_THREADS / 32], hi_s[3][NA_FRAME_THREADS / 32];
    double lo[3] = {x[0], x[1], x[2]}, hi[3] = {x[0], x[1], x[2]};
    for (int i = threadIdx.x; i < n; i += NA_FRAME_THREADS)
        for (int k = 0; k < 3; ++k) {
            const double q = x[3 * i + k];
            lo[k] = q < lo[k] ? q : lo[k];
            hi[k] = q > hi[k] ? q : hi[k];
        }
    for (int k = 0; k < 3; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            const double l = __shfl_xor_sync(0xffffffffu, lo[k], o);
            const double h = __shfl_xor_sync(0xffffffffu, hi[k], o);
            lo[k] = l < lo[k] ? l : lo[k];
            hi[k] = h > hi[k] ? h : hi[k];
        }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) {
            lo_s[k][w] = lo[k];
            hi_s[k][w] = hi[k];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        double l = lo_s[k][0], h = hi_s[k][0];
        for (int v = 1; v < NA_FRAME_THREADS / 32; ++v) {
            l = lo_s[k][v] < l ? lo_s[k][v] : l;
            h = hi_s[k][v] > h ? hi_s[k][v] : h;
        }
        frame[k] = 0.5 * (l + h);
    }
}

// k_reduce_splits for this entry point: when a tile wait of k_direct_sum
// ran out (status bit ST_WAIT_TIMEOUT), some partial sums were never
// written, and every row gets NaN instead of a wrong finite value.
__global__ void k_noalloc_reduce(const double *__restrict__ partial, int splits, int n, int n_pad,
                                 double G, const unsigned *__restrict__ status,
                                 double *__restrict__ a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (*status & ST_WAIT_TIMEOUT) {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        a[3 * i + 0] = nan;
        a[3 * i + 1] = nan;
        a[3 * i + 2] = nan;
        return;
    }
    const size_t plane = (size_t)n_pad;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int s = 0; s < splits; ++s) {
        const double *p = partial + (size_t)s * 3 * plane;
        s0 += p[i];
        s1 += p[plane + i];
        s2 += p[2 * plane + i];
    }
    a[3 * i + 0] = G * s0;
    a[3 * i + 1] = G * s1;
    a[3 * i + 2] = G * s2;
}

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device.  On a host
// `g_noalloc_scratch` only names a host-side stand-in for the symbol, so
// its address is looked up once per device (with that device current) by
// cudaGetSymbolAddress, which allocates nothing.
cudaError_t noalloc_scratch(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return cudaSuccess;
}

}  // namespace

}  // namespace gs

extern "C" int gsgpu_pairwise_acceleration_noalloc(const double *d_x, const double *d_m,
                                                   int num_particles, double G,
                                                   double softening_length, double *d_a,
                                                   void *stream)
{
    using namespace gs;
    if (!d_x || !d_m || !d_a) {
        std::fprintf(stderr, "gsgpu_pairwise_acceleration_noalloc: NULL array argument\n");
        return GRAV_POINTER_ERROR;
    }
    if (num_particles < 1 || num_particles > NOALLOC_MAX_N) {
        std::fprintf(stderr,
                     "gsgpu_pairwise_acceleration_noalloc: num_particles must be in [1, %d] "
                     "(the fixed scratch capacity). Got: %d\n",
                     NOALLOC_MAX_N, num_particles);
        return GRAV_VALUE_ERROR;
    }
    if (!(softening_length >= 0.0)) {
        std::fprintf(stderr, "gsgpu_pairwise_acceleration_noalloc: Softening length is "
                             "negative. Got: %.3g\n", softening_length);
        return GRAV_VALUE_ERROR;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void *base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    int dev = 0, sms = 0, per_sm = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_direct_sum<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 DS_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_direct_sum<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 DS_SMEM);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_direct_sum<true>, DS_THREADS,
                                                          DS_SMEM);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "gsgpu_pairwise_acceleration_noalloc: %s\n", cudaGetErrorString(e));
        return GRAV_FAILURE;
    }
    unsigned char *scratch = static_cast<unsigned char *>(base);
    float4 *pj = reinterpret_cast<float4 *>(scratch);
    double *partial = reinterpret_cast<double *>(scratch + NOALLOC_PJ_BYTES);
    unsigned *status = reinterpret_cast<unsigned *>(scratch + NOALLOC_STATUS_OFF);
    double *frame = reinterpret_cast<double *>(scratch + NOALLOC_FRAME_OFF);

    // Same work split as the allocating engine, with at most 8 j-chunks.
    const int n_pad = ((num_particles + DS_JTILE - 1) / DS_JTILE) * DS_JTILE;
    const int i_tiles = n_pad / DS_ITILE;
    const int jt_total = n_pad / DS_JTILE;
    const long slots = (long)sms * (per_sm > 0 ? per_sm : 1);
    int splits = 1, jt_per_chunk = jt_total;
    double best = 1e300;
    for (int sp = 1; sp <= std::min(jt_total, NOALLOC_MAX_SPLITS); ++sp) {
        const int chunk = (jt_total + sp - 1) / sp;
        const int used = (jt_total + chunk - 1) / chunk;
        const long units = (long)i_tiles * used;
        const double cost = (double)((units + slots - 1) / slots) * (chunk + 0.25);
        if (cost < best - 1e-9) {
            best = cost;
            splits = used;
            jt_per_chunk = chunk;
        }
    }

    // The status word must start at zero; the frame centre, the packed array
    // and the partial sums are fully rewritten by every call.
    e = cudaMemsetAsync(status, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        k_noalloc_frame<<<1, NA_FRAME_THREADS, 0, s>>>(d_x, num_particles, frame);
        k_pack_frame<<<(n_pad + 255) / 256, 256, 0, s>>>(d_x, d_m, num_particles, n_pad, frame,
                                                         pj);
        const float eps2 = (float)(softening_length * softening_length);
        if (eps2 > 0.0f)
            k_direct_sum<true><<<i_tiles * splits, DS_THREADS, DS_SMEM, s>>>(
                pj, n_pad, i_tiles, jt_per_chunk, jt_total, eps2, partial, status);
        else
            k_direct_sum<false><<<i_tiles * splits, DS_THREADS, DS_SMEM, s>>>(
                pj, n_pad, i_tiles, jt_per_chunk, jt_total, eps2, partial, status);
        k_noalloc_reduce<<<(num_particles + 255) / 256, 256, 0, s>>>(
            partial, splits, num_particles, n_pad, G, status, d_a);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        std::fprintf(stderr, "gsgpu_pairwise_acceleration_noalloc: %s\n", cudaGetErrorString(e));
        return GRAV_FAILURE;
    }
    return GRAV_SUCCESS;
}
