// k_integrate.cu -- FP64 kick / drift / stage updates of grav_sim's
// fixed-step integrators (src/integrator.c), one thread per array element.
//
// Every FP64 operation is an explicitly rounded intrinsic (__dmul_rn,
// __dadd_rn, __dsub_rn) in the order of the reference's C expressions, so
// no product is fused into an FMA: given the same accelerations the state
// after a step equals the reference's bit for bit (the reference compiled
// without FMA contraction).  These kernels are HBM-bound: a compensated
// update reads y, err, d and writes y, err (40 B per element).
#include "gs_internal.h"
#include "gs_ptx.cuh"

namespace gs {

namespace {
constexpr int TPB = 256;
inline int blocks(int len) { return (len + TPB - 1) / TPB; }
}  // namespace

// y, err updated with d * (factor * dt) ... see launch_comp_update.
__global__ void k_comp_update(double *__restrict__ y, double *__restrict__ err,
                              const double *__restrict__ d, double h, int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    double yy = y[k], ee = err[k];
    comp_update(yy, ee, d[k], h);
    y[k] = yy;
    err[k] = ee;
}

// Leapfrog initial half kick: err += (0.5 * a) * dt (src/integrator.c:978).
__global__ void k_comp_update_scaled(double *__restrict__ y, double *__restrict__ err,
                                     const double *__restrict__ d, double coef, double dt,
                                     int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    const double y0 = y[k];
    double e = __dadd_rn(err[k], __dmul_rn(__dmul_rn(coef, d[k]), dt));
    const double yn = __dadd_rn(y0, e);
    e = __dadd_rn(e, __dsub_rn(y0, yn));
    y[k] = yn;
    err[k] = e;
}

void launch_comp_update(double *y, double *err, const double *d, double dt, double factor,
                        int len, cudaStream_t s)
{
    if (len <= 0) return;
    if (factor == 1.0)
        k_comp_update<<<blocks(len), TPB, 0, s>>>(y, err, d, dt, len);
    else
        k_comp_update_scaled<<<blocks(len), TPB, 0, s>>>(y, err, d, factor, dt, len);
}

// src/integrator.c:382-395 (euler): both updates use the state at the start
// of the step.
__global__ void k_euler(double *__restrict__ x, double *__restrict__ v, double *__restrict__ xe,
                        double *__restrict__ ve, const double *__restrict__ a, double dt, int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    const double x0 = x[k], v0 = v[k];
    double ex = __dadd_rn(xe[k], __dmul_rn(v0, dt));
    double ev = __dadd_rn(ve[k], __dmul_rn(a[k], dt));
    const double xn = __dadd_rn(x0, ex);
    const double vn = __dadd_rn(v0, ev);
    ex = __dadd_rn(ex, __dsub_rn(x0, xn));
    ev = __dadd_rn(ev, __dsub_rn(v0, vn));
    x[k] = xn;
    v[k] = vn;
    xe[k] = ex;
    ve[k] = ev;
}

void launch_euler_update(double *x, double *v, double *xe, double *ve, const double *a, double dt,
                         int len, cudaStream_t s)
{
    if (len <= 0) return;
    k_euler<<<blocks(len), TPB, 0, s>>>(x, v, xe, ve, a, dt, len);
}

// v -= (coef * a) * dt, uncompensated (src/integrator.c:1088-1094).
__global__ void k_plain_kick(double *__restrict__ v, const double *__restrict__ a, double coef,
                             double dt, int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    v[k] = __dsub_rn(v[k], __dmul_rn(__dmul_rn(coef, a[k]), dt));
}

void launch_plain_kick(double *v, const double *a, double coef, double dt, int len, cudaStream_t s)
{
    if (len <= 0) return;
    k_plain_kick<<<blocks(len), TPB, 0, s>>>(v, a, coef, dt, len);
}

// src/integrator.c:746-793: x = x0 + (coef * xk) * dt, v likewise.
__global__ void k_rk4_stage(double *__restrict__ x, double *__restrict__ v,
                            const double *__restrict__ x0, const double *__restrict__ v0,
                            const double *__restrict__ xk, const double *__restrict__ vk,
                            double coef, double dt, int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    x[k] = __dadd_rn(x0[k], __dmul_rn(__dmul_rn(coef, xk[k]), dt));
    v[k] = __dadd_rn(v0[k], __dmul_rn(__dmul_rn(coef, vk[k]), dt));
}

void launch_rk4_stage(double *x, double *v, const double *x0, const double *v0, const double *xk,
                      const double *vk, double coef, double dt, int len, cudaStream_t s)
{
    if (len <= 0) return;
    k_rk4_stage<<<blocks(len), TPB, 0, s>>>(x, v, x0, v0, xk, vk, coef, dt, len);
}

// src/integrator.c:806-819: compensated combine of the four stages,
// increment = ((((k1 + 2 k2) + 2 k3) + k4) * dt) / 6.
__device__ __forceinline__ double rk4_incr(double k1, double k2, double k3, double k4, double dt)
{
    const double s = __dadd_rn(__dadd_rn(__dadd_rn(k1, __dmul_rn(2.0, k2)), __dmul_rn(2.0, k3)), k4);
    return __ddiv_rn(__dmul_rn(s, dt), 6.0);
}

struct Rk4Ptrs {
    const double *xk[4];
    const double *vk[4];
};

__global__ void k_rk4_final(double *__restrict__ x, double *__restrict__ v,
                            const double *__restrict__ x0, const double *__restrict__ v0,
                            double *__restrict__ xe, double *__restrict__ ve, Rk4Ptrs p, double dt,
                            int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    double ev = __dadd_rn(ve[k], rk4_incr(p.vk[0][k], p.vk[1][k], p.vk[2][k], p.vk[3][k], dt));
    double ex = __dadd_rn(xe[k], rk4_incr(p.xk[0][k], p.xk[1][k], p.xk[2][k], p.xk[3][k], dt));
    const double vn = __dadd_rn(v0[k], ev);
    const double xn = __dadd_rn(x0[k], ex);
    ev = __dadd_rn(ev, __dsub_rn(v0[k], vn));
    ex = __dadd_rn(ex, __dsub_rn(x0[k], xn));
    v[k] = vn;
    x[k] = xn;
    ve[k] = ev;
    xe[k] = ex;
}

void launch_rk4_final(double *x, double *v, const double *x0, const double *v0, double *xe,
                      double *ve, const double *const *xk, const double *const *vk, double dt,
                      int len, cudaStream_t s)
{
    if (len <= 0) return;
    Rk4Ptrs p;
    for (int i = 0; i < 4; ++i) {
        p.xk[i] = xk[i];
        p.vk[i] = vk[i];
    }
    k_rk4_final<<<blocks(len), TPB, 0, s>>>(x, v, x0, v0, xe, ve, p, dt, len);
}

// ---- embedded Runge-Kutta (src/integrator_rk_embedded.c:721-856) ----------
// Stage and weight coefficients travel as kernel parameters (at most 13
// stages); vk / xk are S arrays of len doubles, stage i at offset i * len.
struct RkEmbCoef {
    double c[13];    // a[s][0..s-1] for the stage kernel; b for the combine
    double dc[13];   // dt * (b - b_hat) for the combine
};

// Stage s: position / velocity at which the next acceleration is taken,
//   tv = sum_{i<s} a[s][i] vk[i],  tx = sum_{i<s} a[s][i] xk[i]  (from +0.0)
//   tv = (v + dt tv) + ve,  tx = (x + dt tx) + xe,  xk[s] = tv.
__global__ void k_rk_emb_stage(const double *__restrict__ x, const double *__restrict__ v,
                               const double *__restrict__ xe, const double *__restrict__ ve,
                               const double *__restrict__ vk, double *__restrict__ xk,
                               double *__restrict__ xs, RkEmbCoef cf, int stage, double dt,
                               int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    double tv = 0.0, tx = 0.0;
    for (int i = 0; i < stage; ++i) {
        tv = __dadd_rn(tv, __dmul_rn(cf.c[i], vk[(size_t)i * len + k]));
        tx = __dadd_rn(tx, __dmul_rn(cf.c[i], xk[(size_t)i * len + k]));
    }
    tv = __dadd_rn(__dadd_rn(v[k], __dmul_rn(dt, tv)), ve[k]);
    tx = __dadd_rn(__dadd_rn(x[k], __dmul_rn(dt, tx)), xe[k]);
    xs[k] = tx;
    xk[(size_t)stage * len + k] = tv;
}

// Weights, error deltas, compensated x1 / v1 and the two squared scaled
// error terms of element k, written at terms[2k] (velocity) and
// terms[2k + 1] (position): the order in which the reference sums them.
__global__ void k_rk_emb_combine(const double *__restrict__ x, const double *__restrict__ v,
                                 const double *__restrict__ xe, const double *__restrict__ ve,
                                 const double *__restrict__ vk, const double *__restrict__ xk,
                                 double *__restrict__ x1, double *__restrict__ v1,
                                 double *__restrict__ txe, double *__restrict__ tve,
                                 double *__restrict__ terms, RkEmbCoef cf, int stages, double dt,
                                 double abs_tol, double rel_tol, int len)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    double tv = 0.0, tx = 0.0, dv = 0.0, dx = 0.0;
    for (int s = 0; s < stages; ++s) {
        const double a = vk[(size_t)s * len + k], b = xk[(size_t)s * len + k];
        tv = __dadd_rn(tv, __dmul_rn(cf.c[s], a));
        tx = __dadd_rn(tx, __dmul_rn(cf.c[s], b));
        dv = __dadd_rn(dv, __dmul_rn(cf.dc[s], a));
        dx = __dadd_rn(dx, __dmul_rn(cf.dc[s], b));
    }
    const double v0 = v[k], x0 = x[k];
    double ev = __dadd_rn(ve[k], __dmul_rn(dt, tv));
    double ex = __dadd_rn(xe[k], __dmul_rn(dt, tx));
    const double vn = __dadd_rn(v0, ev), xn = __dadd_rn(x0, ex);
    ev = __dadd_rn(ev, __dsub_rn(v0, vn));
    ex = __dadd_rn(ex, __dsub_rn(x0, xn));
    v1[k] = vn;
    x1[k] = xn;
    tve[k] = ev;
    txe[k] = ex;
    const double sv = __dadd_rn(abs_tol, __dmul_rn(fmax(fabs(v0), fabs(vn)), rel_tol));
    const double sx = __dadd_rn(abs_tol, __dmul_rn(fmax(fabs(x0), fabs(xn)), rel_tol));
    const double qv = __ddiv_rn(dv, sv), qx = __ddiv_rn(dx, sx);
    terms[2 * (size_t)k] = __dmul_rn(qv, qv);
    terms[2 * (size_t)k + 1] = __dmul_rn(qx, qx);
}

void launch_rk_emb_stage(const double *x, const double *v, const double *xe, const double *ve,
                         const double *vk, double *xk, double *xs, const double *a_row,
                         int stage, double dt, int len, cudaStream_t s)
{
    if (len <= 0) return;
    RkEmbCoef cf{};
    for (int i = 0; i < stage && i < 13; ++i) cf.c[i] = a_row[i];
    k_rk_emb_stage<<<blocks(len), TPB, 0, s>>>(x, v, xe, ve, vk, xk, xs, cf, stage, dt, len);
}

void launch_rk_emb_combine(const double *x, const double *v, const double *xe, const double *ve,
                           const double *vk, const double *xk, double *x1, double *v1,
                           double *txe, double *tve, double *terms, const double *w,
                           const double *dtdw, int stages, double dt, double abs_tol,
                           double rel_tol, int len, cudaStream_t s)
{
    if (len <= 0) return;
    RkEmbCoef cf{};
    for (int i = 0; i < stages && i < 13; ++i) {
        cf.c[i] = w[i];
        cf.dc[i] = dtdw[i];
    }
    k_rk_emb_combine<<<blocks(len), TPB, 0, s>>>(x, v, xe, ve, vk, xk, x1, v1, txe, tve, terms,
                                                 cf, stages, dt, abs_tol, rel_tol, len);
}

// Sum of the embedded Runge-Kutta error terms on the device: each of
// ES_BLOCKS x ES_THREADS threads adds its strided share in index order, each
// block adds its threads' sums in a fixed tree, and one block adds the block
// sums the same way.  The grouping depends on the count alone, so the result
// is the same on every run; it is not the reference's one-by-one order (that
// sum is reproduced on the host), but its rounding error is smaller.
constexpr int ES_BLOCKS = 256, ES_THREADS = 256;

__device__ __forceinline__ double block_tree_sum(double v, double *sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = ES_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    return sh[0];
}

__global__ void __launch_bounds__(ES_THREADS)
k_error_sum_blocks(const double *__restrict__ terms, long long count, double *__restrict__ part)
{
    __shared__ double sh[ES_THREADS];
    double acc = 0.0;
    const long long stride = (long long)ES_BLOCKS * ES_THREADS;
    for (long long i = (long long)blockIdx.x * ES_THREADS + threadIdx.x; i < count; i += stride)
        acc = __dadd_rn(acc, terms[i]);
    const double b = block_tree_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = b;
}

__global__ void __launch_bounds__(ES_THREADS)
k_error_sum_final(const double *__restrict__ part, double *__restrict__ out)
{
    __shared__ double sh[ES_THREADS];
    const double b = block_tree_sum(part[threadIdx.x], sh);
    if (threadIdx.x == 0) out[0] = b;
}

void launch_error_sum(const double *terms, long long count, double *scratch, cudaStream_t s)
{
    static_assert(ES_BLOCKS == ES_THREADS, "the final block adds one partial per thread");
    k_error_sum_blocks<<<ES_BLOCKS, ES_THREADS, 0, s>>>(terms, count, scratch);
    k_error_sum_final<<<1, ES_THREADS, 0, s>>>(scratch, scratch + ES_BLOCKS);
}

}  // namespace gs
