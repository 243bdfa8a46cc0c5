// k_ias15.cu -- element-wise kernels of the IAS15 integrator
// (src/integrator_ias15.c, integrator code 9).
//
// Compiled with --fmad=false: every expression below is the reference's C
// expression in the reference's operation order, and no product is fused
// into an FMA, so given the same accelerations each kernel produces the
// reference's doubles bit for bit.  Divisions are IEEE (the default
// -prec-div=true).  The predictor-corrector loop, the convergence test and
// the step-size control run on the host (host_sim.cpp); the maxima they need
// come from exact max reductions here (the maximum does not depend on order).
#include "gs_internal.h"

#include <algorithm>

namespace gs {

/* Gauss-Radau spacings h_0..h_7 (host: the predictor node is a kernel argument) */
const double kIas15H[8] = {0.0, 0x1.cce7242fd9812p-5, 0x1.7122082358d27p-3, 0x1.6916742f0c9c5p-2, 0x1.18248525f4802p-1, 0x1.77ea65770fa49p-1, 0x1.c548c982467cdp-1, 0x1.f47d94f4d2bb2p-1};
/* c[i][j] (j <= i): b from g */
__constant__ double kRadauC[7][7] = {
    {0x1.0000000000000p+0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.cce7242fd9812p-5, 0x1.0000000000000p+0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.4c4b384151c1ep-7, -0x1.e45bd12f4f32cp-3, 0x1.0000000000000p+0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.d4b3379a1992dp-9, 0x1.7f2161e152586p-4, -0x1.2da22e635a1aep-1, 0x1.0000000000000p+0, 0.0, 0.0, 0.0},
    {0x1.007370e57b89dp-9, -0x1.c08e5e7efcf23p-5, 0x1.a9dcc2e57fbbfp-2, -0x1.22e359c4a74d8p+0, 0x1.0000000000000p+0, 0.0, 0.0},
    {-0x1.7893e98a2a997p-10, 0x1.595cd739ee74fp-5, -0x1.70bdf2d91dd44p-2, 0x1.4009e0866d488p+0, -0x1.ded88c802f1fcp+0, 0x1.0000000000000p+0, 0.0},
    {0x1.4d64672378b3dp-10, -0x1.3d865cb429919p-5, 0x1.71a0161ae20fep-2, -0x1.7785b93619434p+0, 0x1.73fc45dfb9889p+1, -0x1.60be78a0a92f1p+1, 0x1.0000000000000p+0}};
/* r[i][j] = 1 / (h_i - h_j) (j < i): g from the accelerations */
__constant__ double kRadauR[8][8] = {
    {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.1c618574b517bp+4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.6314ac07f6a9ap+2, 0x1.021c2b5e4af6fp+3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.6afdfcc2a4aefp+1, 0x1.afe76c59caa8ap+1, 0x1.73439c0b4562bp+2, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.d3e03b89d73cfp+0, 0x1.04c014a3946fbp+1, 0x1.5cdb4a576d57ap+1, 0x1.48fffc3fdf2e6p+2, 0.0, 0.0, 0.0, 0.0},
    {0x1.5cac8b52e27b1p+0, 0x1.799c3c56b4e9dp+0, 0x1.ce1e8b86f5ae8p+0, 0x1.4f714afea15ccp+1, 0x1.56247c4b878b4p+2, 0.0, 0.0, 0.0},
    {0x1.212921ce4baffp+0, 0x1.34c8b7028f418p+0, 0x1.6b1448c75e4d5p+0, 0x1.e092f6d7c8a42p+0, 0x1.7a82c7145ec17p+1, 0x1.a787c6413556bp+2, 0.0, 0.0},
    {0x1.05e3166485188p+0, 0x1.15e18175af101p+0, 0x1.41177c7d3aff5p+0, 0x1.99ab118ef2216p+0, 0x1.296bab4a3e0d2p+1, 0x1.0709d7d8d5e3cp+2, 0x1.5b12a584540e2p+3, 0.0}};


namespace {
constexpr int TPB = 256;
inline int blocks(int len) { return (len + TPB - 1) / TPB; }
}  // namespace

// Predictor at spacing h (src/integrator_ias15.c:808-919).
__global__ void k_ias_predict(int L, double *__restrict__ x1, double *__restrict__ v1,
                              const double *__restrict__ x0, const double *__restrict__ v0,
                              const double *__restrict__ a0, double h, const double *__restrict__ b,
                              double dt, const double *__restrict__ xe,
                              const double *__restrict__ ve)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    const double *bk = b + k;
    const double dth = dt * h;
    double p = bk[5 * (size_t)L] / 28.0 + h * bk[6 * (size_t)L] / 36.0;
    p = bk[4 * (size_t)L] / 21.0 + h * p;
    p = bk[3 * (size_t)L] / 15.0 + h * p;
    p = bk[2 * (size_t)L] / 10.0 + h * p;
    p = bk[1 * (size_t)L] / 6.0 + h * p;
    p = bk[0] / 3.0 + h * p;
    double xv = x0[k];
    xv += xe[k] + dth * (v0[k] + dth * (a0[k] + h * p) / 2.0);
    x1[k] = xv;
    double q = bk[5 * (size_t)L] / 7.0 + h * bk[6 * (size_t)L] / 8.0;
    q = bk[4 * (size_t)L] / 6.0 + h * q;
    q = bk[3 * (size_t)L] / 5.0 + h * q;
    q = bk[2 * (size_t)L] / 4.0 + h * q;
    q = bk[1 * (size_t)L] / 3.0 + h * q;
    q = bk[0] / 2.0 + h * q;
    double vv = v0[k];
    vv += ve[k] + dth * (a0[k] + h * q);
    v1[k] = vv;
}

// g from the accelerations at spacings 0..i, then b from g
// (src/integrator_ias15.c:1117-1274 and :985-1115).
__global__ void k_ias_update_gb(int L, double *__restrict__ g, double *__restrict__ b,
                                const double *__restrict__ F, int i)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    double *gk = g + k, *bk = b + k;
    const double f0 = F[k];
    for (int m = 1; m <= i && m <= 7; ++m) {
        double t = (F[(size_t)m * L + k] - f0) * kRadauR[m][0];
        for (int j = 1; j < m; ++j) t = (t - gk[(size_t)(j - 1) * L]) * kRadauR[m][j];
        gk[(size_t)(m - 1) * L] = t;
    }
    for (int r = 0; r < i && r < 7; ++r) {
        double t = kRadauC[r][r] * gk[(size_t)r * L];
        for (int j = r + 1; j < 7; ++j) t += kRadauC[j][r] * gk[(size_t)j * L];
        bk[(size_t)r * L] = t;
    }
}

// Largest |value| of two vectors into out[0], out[1] (zeroed by the caller):
// non-negative doubles order like their bit patterns, so an unsigned max
// is exact; NaNs are skipped, as fmax skips them.
__device__ __forceinline__ void max_into(unsigned long long *slot, double v)
{
    v = fabs(v);
    if (v == v) atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}

__global__ void k_ias_absmax2(int L, const double *__restrict__ u, const double *__restrict__ w,
                              unsigned long long *__restrict__ out)
{
    __shared__ unsigned long long s[2];
    if (threadIdx.x < 2) s[threadIdx.x] = 0ull;
    __syncthreads();
    double mu = 0.0, mw = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
        const double a = fabs(u[k]), c = fabs(w[k]);
        if (a == a) mu = fmax(mu, a);
        if (c == c) mw = fmax(mw, c);
    }
    max_into(&s[0], mu);
    max_into(&s[1], mw);
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicMax(&out[0], s[0]);
        atomicMax(&out[1], s[1]);
    }
}

// Predictor-corrector convergence: |b_6 - b0_6| (into d7), then b0 = b.
__global__ void k_ias_delta(int L, const double *__restrict__ b, double *__restrict__ b0,
                            double *__restrict__ d7)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    d7[k] = b[6 * (size_t)L + k] - b0[6 * (size_t)L + k];
    for (int r = 0; r < 7; ++r) b0[(size_t)r * L + k] = b[(size_t)r * L + k];
}

// End of the step with compensated sums (src/integrator_ias15.c:921-983).
__global__ void k_ias_advance(int L, double *__restrict__ x1, double *__restrict__ v1,
                              double *__restrict__ txe, double *__restrict__ tve,
                              const double *__restrict__ x0, const double *__restrict__ v0,
                              const double *__restrict__ a0, const double *__restrict__ b, double dt)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    const double *bk = b + k;
    const size_t S = (size_t)L;
    const double sx = a0[k] + bk[0] / 3.0 + bk[S] / 6.0 + bk[2 * S] / 10.0 + bk[3 * S] / 15.0 +
                      bk[4 * S] / 21.0 + bk[5 * S] / 28.0 + bk[6 * S] / 36.0;
    double ex = txe[k];
    ex += dt * (v0[k] + dt * sx / 2.0);
    const double xn = x0[k] + ex;
    ex += x0[k] - xn;
    x1[k] = xn;
    txe[k] = ex;
    const double sv = a0[k] + bk[0] / 2.0 + bk[S] / 3.0 + bk[2 * S] / 4.0 + bk[3 * S] / 5.0 +
                      bk[4 * S] / 6.0 + bk[5 * S] / 7.0 + bk[6 * S] / 8.0;
    double ev = tve[k];
    ev += dt * sv;
    const double vn = v0[k] + ev;
    ev += v0[k] - vn;
    v1[k] = vn;
    tve[k] = ev;
}

// Prediction of b for the next step (src/integrator_ias15.c:1276-1382).
struct IasQ {
    double q[7];   // q, q^2 .. q^7 (formed on the host as the reference does)
};

__global__ void k_ias_refine(int L, double *__restrict__ b, double *__restrict__ e, IasQ Q,
                             int refine)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    const size_t S = (size_t)L;
    double db[7];
    for (int r = 0; r < 7; ++r) db[r] = refine ? b[r * S + k] - e[r * S + k] : 0.0;
    const double b0 = b[k], b1 = b[S + k], b2 = b[2 * S + k], b3 = b[3 * S + k], b4 = b[4 * S + k],
                 b5 = b[5 * S + k], b6 = b[6 * S + k];
    double en[7];
    en[0] = Q.q[0] * (b6 * 7.0 + b5 * 6.0 + b4 * 5.0 + b3 * 4.0 + b2 * 3.0 + b1 * 2.0 + b0);
    en[1] = Q.q[1] * (b6 * 21.0 + b5 * 15.0 + b4 * 10.0 + b3 * 6.0 + b2 * 3.0 + b1);
    en[2] = Q.q[2] * (b6 * 35.0 + b5 * 20.0 + b4 * 10.0 + b3 * 4.0 + b2);
    en[3] = Q.q[3] * (b6 * 35.0 + b5 * 15.0 + b4 * 5.0 + b3);
    en[4] = Q.q[4] * (b6 * 21.0 + b5 * 6.0 + b4);
    en[5] = Q.q[5] * (b6 * 7.0 + b5);
    en[6] = Q.q[6] * b6;
    for (int r = 0; r < 7; ++r) {
        e[r * S + k] = en[r];
        b[r * S + k] = en[r] + db[r];
    }
}

// out = x + c v and out = u - w (the initial-step estimate, :702-806).
__global__ void k_ias_axpy(int L, double *__restrict__ out, const double *__restrict__ x, double c,
                           const double *__restrict__ v)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < L) out[k] = x[k] + c * v[k];
}

__global__ void k_ias_sub(int L, double *__restrict__ out, const double *__restrict__ u,
                          const double *__restrict__ w)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < L) out[k] = u[k] - w[k];
}

void launch_ias_axpy(int L, double *out, const double *x, double c, const double *v,
                     cudaStream_t s)
{
    k_ias_axpy<<<blocks(L), TPB, 0, s>>>(L, out, x, c, v);
}

void launch_ias_sub(int L, double *out, const double *u, const double *w, cudaStream_t s)
{
    k_ias_sub<<<blocks(L), TPB, 0, s>>>(L, out, u, w);
}

void launch_ias_predict(int L, double *x1, double *v1, const double *x0, const double *v0,
                        const double *a0, double h, const double *b, double dt, const double *xe,
                        const double *ve, cudaStream_t s)
{
    k_ias_predict<<<blocks(L), TPB, 0, s>>>(L, x1, v1, x0, v0, a0, h, b, dt, xe, ve);
}

void launch_ias_update_gb(int L, double *g, double *b, const double *F, int i, cudaStream_t s)
{
    k_ias_update_gb<<<blocks(L), TPB, 0, s>>>(L, g, b, F, i);
}

void launch_ias_absmax2(int L, const double *u, const double *w, unsigned long long *out,
                        cudaStream_t s)
{
    const int grid = std::min(blocks(L), 1024);
    k_ias_absmax2<<<grid, TPB, 0, s>>>(L, u, w, out);
}

void launch_ias_delta(int L, const double *b, double *b0, double *d7, cudaStream_t s)
{
    k_ias_delta<<<blocks(L), TPB, 0, s>>>(L, b, b0, d7);
}

void launch_ias_advance(int L, double *x1, double *v1, double *txe, double *tve, const double *x0,
                        const double *v0, const double *a0, const double *b, double dt,
                        cudaStream_t s)
{
    k_ias_advance<<<blocks(L), TPB, 0, s>>>(L, x1, v1, txe, tve, x0, v0, a0, b, dt);
}

void launch_ias_refine(int L, double *b, double *e, const double q[7], int refine, cudaStream_t s)
{
    IasQ Q;
    for (int r = 0; r < 7; ++r) Q.q[r] = q[r];
    k_ias_refine<<<blocks(L), TPB, 0, s>>>(L, b, e, Q, refine);
}

}  // namespace gs
