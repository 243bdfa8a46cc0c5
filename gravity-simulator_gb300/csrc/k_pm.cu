// k_pm.cu -- particle-mesh gravity (src/acceleration_PM.c:15-391) and the
// cosmological leapfrog (src/integrator_cosmology_leapfrog.c:24-255).
//
// One evaluation on a g^3 periodic mesh:
//   k_pm_deposit   cloud-in-cell mass deposit, one thread per particle,
//                  eight FP64 atomic adds (the reference's OpenMP loop has
//                  unsynchronised += here);
//   k_pm_contrast  delta = rho / (V_cell rho_mean) - 1;
//   cuFFT D2Z      the r2c transform (FFTW's layout: g x g x (g/2+1));
//   k_pm_green     multiply by -1/k^2 (0 at k = 0);
//   cuFFT Z2D      the unnormalised c2r transform;
//   k_pm_gradient  fourth-order central differences of phi * factor into the
//                  acceleration mesh (the reference scales phi in place
//                  first; the product is formed on load here, same bits);
//   k_pm_interp    cloud-in-cell interpolation back to the particles.
// Every kernel computes the reference's quantity in FP64.  The FP64 pipe of
// this GPU runs at 1/64 of the FP32 rate and bounds the particle kernels, so
// they use algebraically equal forms with fewer FP64 operations than the
// reference's expressions: weight products shared between the eight
// corners, fused multiply-adds, the constant divisions of the kicks, the
// drift and the gradient folded into one multiplier each.  These round
// differently from the reference's order by a few ulps, far below the
// differences of the transforms (cuFFT against FFTW) and of the atomic
// deposit order.  The file is compiled with --fmad=false; the fused
// operations are the explicit fma() calls.
//
// Memory: delta / phi g^3 doubles, the spectrum g^2 (g/2+1) complex, the
// acceleration mesh 3 g^3 doubles: 56 g^3 bytes, 940 MB at g = 256.
#include "gs_internal.h"

#include <cufft.h>

#include <cmath>
#include <cstdio>
#include <memory>

namespace gs {
namespace {

constexpr int TPB = 256;
inline unsigned blocks(long long n) { return (unsigned)((n + TPB - 1) / TPB); }

const char *cufft_name(cufftResult r)
{
    switch (r) {
    case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
    case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    default: return "cuFFT error";
    }
}

#define GS_CUFFT(call)                                                                   \
    do {                                                                                 \
        cufftResult r_ = (call);                                                         \
        if (r_ != CUFFT_SUCCESS)                                                         \
            return GS_RAISE(r_ == CUFFT_ALLOC_FAILED ? GRAV_MEMORY_ERROR : GRAV_FAILURE,   \
                            "%s failed: %s", #call, cufft_name(r_));                     \
    } while (0)

// Mesh geometry of one evaluation (src/acceleration_PM.c:35-37).
struct PmGeom {
    double cx, cy, cz;   // box centre
    double half;         // box_length / 2
    double inv_cell;     // 1 / (box_length / g)
    int g;
};

__device__ __forceinline__ int wrap_index(int n, int g)
{
    // the reference indexes n % g; n >= 0 inside the box.  A particle
    // outside it (n < 0) wraps here instead of indexing out of bounds.
    const int r = n % g;
    return r < 0 ? r + g : r;
}

// Cell indices and weights of one particle (src/acceleration_PM.c:44-58).
__device__ __forceinline__ void cic_cell(const double *xi, const PmGeom &G, int idx[2][3],
                                         double w[2][3])
{
    const double c[3] = {G.cx, G.cy, G.cz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double normalized = (xi[d] - c[d] + G.half) * G.inv_cell;
        const int nd = (int)normalized;
        const double weight = normalized - nd;
        w[1][d] = weight;
        w[0][d] = 1.0 - weight;
        idx[0][d] = wrap_index(nd, G.g);
        idx[1][d] = wrap_index(nd + 1, G.g);
    }
}

// Corner order of the reference's eight terms: bit 0 x, bit 1 y, bit 2 z
// (a constant in unrolled loops, so the per-corner arrays stay in registers).
__host__ __device__ constexpr int corner_bits(int c)
{
    return c == 3 ? 4 : (c == 4 ? 3 : c);
}

__global__ void k_pm_deposit(const double *__restrict__ x, const double *__restrict__ m, int n,
                             PmGeom G, double *__restrict__ delta)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int idx[2][3];
    double w[2][3];
    cic_cell(x + 3 * (size_t)i, G, idx, w);
    const long long g = G.g, g2 = g * g;
    const double mi = m[i];
    double mx[2], mxy[2][2];
#pragma unroll
    for (int bx = 0; bx < 2; ++bx) {
        mx[bx] = mi * w[bx][0];
#pragma unroll
        for (int by = 0; by < 2; ++by) mxy[bx][by] = mx[bx] * w[by][1];
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int bx = corner_bits(c) & 1, by = (corner_bits(c) >> 1) & 1,
                  bz = (corner_bits(c) >> 2) & 1;
        const long long cell = idx[bx][0] * g2 + idx[by][1] * g + idx[bz][2];
        atomicAdd(delta + cell, mxy[bx][by] * w[bz][2]);
    }
}

// delta = rho / (V_cell rho_mean) - 1 with inv = 1 / (V_cell rho_mean)
__global__ void k_pm_contrast(double *__restrict__ delta, long long cells, double inv)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cells) return;
    delta[i] = fma(delta[i], inv, -1.0);
}

// src/acceleration_PM.c:321-345
__global__ void k_pm_green(double2 *__restrict__ spec, int g, double two_pi_over_l2)
{
    const int h = g / 2 + 1;
    const long long total = (long long)g * g * h;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int k = (int)(e % h);
    const long long ij = e / h;
    const int j = (int)(ij % g), i = (int)(ij / g);
    const int kx = (i < h) ? i : i - g;
    const int ky = (j < h) ? j : j - g;
    const int kz = k;
    const double k_sq = (double)(kx * kx + ky * ky + kz * kz) * two_pi_over_l2;
    const double kernel = k_sq == 0.0 ? 0.0 : -1.0 / k_sq;
    double2 v = spec[e];
    v.x *= kernel;
    v.y *= kernel;
    spec[e] = v;
}

// src/acceleration_PM.c:212-272: (phi[-2] - 8 phi[-1] + 8 phi[+1] - phi[+2])
// * factor / (12 cell_length), as ((phi[-2] - phi[+2]) + 8 (phi[+1] - phi[-1]))
// * scale with scale = factor / (12 cell_length).
__global__ void k_pm_gradient(const double *__restrict__ phi, int g, double scale,
                              double *__restrict__ acc)
{
    const long long g2 = (long long)g * g, cells = g2 * g;
    const long long index = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= cells) return;
    const int k = (int)(index % g);
    const int j = (int)((index / g) % g);
    const int i = (int)(index / g2);
    const int c[3] = {i, j, k};
    const long long st[3] = {g2, g, 1};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long b = index - c[d] * st[d];
        const double pm2 = phi[b + (long long)((c[d] - 2 + g) % g) * st[d]];
        const double pm1 = phi[b + (long long)((c[d] - 1 + g) % g) * st[d]];
        const double pp1 = phi[b + (long long)((c[d] + 1) % g) * st[d]];
        const double pp2 = phi[b + (long long)((c[d] + 2) % g) * st[d]];
        acc[index * 3 + d] = fma(8.0, pp1 - pm1, pm2 - pp2) * scale;
    }
}

// src/acceleration_PM.c:112-210
__global__ void k_pm_interp(const double *__restrict__ x, int n, PmGeom G,
                            const double *__restrict__ acc, double *__restrict__ a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int idx[2][3];
    double w[2][3];
    cic_cell(x + 3 * (size_t)i, G, idx, w);
    const long long g = G.g, g2 = g * g;
    double wxy[2][2];
#pragma unroll
    for (int bx = 0; bx < 2; ++bx)
#pragma unroll
        for (int by = 0; by < 2; ++by) wxy[bx][by] = w[bx][0] * w[by][1];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int bx = corner_bits(c) & 1, by = (corner_bits(c) >> 1) & 1,
                  bz = (corner_bits(c) >> 2) & 1;
        const long long cell = idx[bx][0] * g2 + idx[by][1] * g + idx[bz][2];
        const double wc = wxy[bx][by] * w[bz][2];
        const double *ac = acc + cell * 3;
        s0 = fma(ac[0], wc, s0);
        s1 = fma(ac[1], wc, s1);
        s2 = fma(ac[2], wc, s2);
    }
    a[3 * (size_t)i + 0] = s0;
    a[3 * (size_t)i + 1] = s1;
    a[3 * (size_t)i + 2] = s2;
}

// ---- cosmological leapfrog (src/integrator_cosmology_leapfrog.c) -----------
// src/system.c:1337-1375 for one coordinate.
__device__ __forceinline__ double periodic(double xv, double c, double bw)
{
    const double p = xv - c;
    if (p < -bw) {
        xv = ((int)(p / bw) % 2 != 0) ? fmod(p, bw) + bw : fmod(p, bw);
        xv += c;
    } else if (p > bw) {
        xv = ((int)(p / bw) % 2 != 0) ? fmod(p, bw) - bw : fmod(p, bw);
        xv += c;
    }
    return xv;
}

__global__ void k_cosmo_wrap(double *__restrict__ x, int len, double cx, double cy, double cz,
                             double bw)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    const int d = k % 3;
    x[k] = periodic(x[k], d == 0 ? cx : (d == 1 ? cy : cz), bw);
}

// momentum = a^2 v (:92-98)
__global__ void k_cosmo_momentum(double *__restrict__ p, const double *__restrict__ v, int len,
                                 double t)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    p[k] = t * t * v[k];
}

// velocity = momentum / a^2 at a snapshot (:200-209)
__global__ void k_cosmo_velocity(double *__restrict__ v, const double *__restrict__ p, int len,
                                 double t)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    v[k] = p[k] / (t * t);
}

// momentum -= (0.5 dt) a / da (:142-149, :176-183); c = 0.5 dt / da
__global__ void k_cosmo_kick(double *__restrict__ p, const double *__restrict__ a, int len,
                             double c)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    p[k] = fma(-c, a[k], p[k]);
}

// x += dt p / (a^2 da) (:152-160), then the periodic wrap (:163); c = dt / (a^2 da)
__global__ void k_cosmo_drift(double *__restrict__ x, const double *__restrict__ p, int len,
                              double c, double cx, double cy, double cz, double bw)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    const int d = k % 3;
    const double xv = fma(c, p[k], x[k]);
    x[k] = periodic(xv, d == 0 ? cx : (d == 1 ? cy : cz), bw);
}

}  // namespace

// One particle-mesh solver per grid size: cuFFT plans and the meshes.
class PmSolver {
  public:
    ~PmSolver()
    {
        if (fwd_) cufftDestroy(fwd_);
        if (inv_) cufftDestroy(inv_);
    }

    ErrorStatus setup(int g)
    {
        if (g == g_) return ok();
        if (fwd_) cufftDestroy(fwd_);
        if (inv_) cufftDestroy(inv_);
        fwd_ = inv_ = 0;
        g_ = 0;
        const long long cells = (long long)g * g * g;
        const long long half = (long long)g * g * (g / 2 + 1);
        GS_TRY(mesh_.reserve((size_t)cells * sizeof(double)));
        GS_TRY(spec_.reserve((size_t)half * sizeof(double2)));
        GS_TRY(acc_.reserve((size_t)cells * 3 * sizeof(double)));
        GS_CUFFT(cufftPlan3d(&fwd_, g, g, g, CUFFT_D2Z));
        GS_CUFFT(cufftPlan3d(&inv_, g, g, g, CUFFT_Z2D));
        g_ = g;
        return ok();
    }

    // src/acceleration_PM.c:274-391 on device arrays.
    ErrorStatus compute(double *d_a, int n, const double *d_x, const double *d_m,
                        const double *box_center, double box_width, double H0, double omega_m,
                        double mean_bkg_density, int g, double scale_factor, cudaStream_t s)
    {
        GS_TRY(setup(g));
        const double box_length = box_width * 2.0;
        const long long cells = (long long)g * g * g;
        PmGeom G;
        G.cx = box_center[0];
        G.cy = box_center[1];
        G.cz = box_center[2];
        G.half = box_length / 2.0;
        const double cell_length = box_length / g;
        G.inv_cell = 1.0 / cell_length;
        G.g = g;
        double *mesh = mesh_.as<double>();
        GS_CUDA(cudaMemsetAsync(mesh, 0, (size_t)cells * sizeof(double), s));
        k_pm_deposit<<<blocks(n), TPB, 0, s>>>(d_x, d_m, n, G, mesh);
        const double cell_volume = cell_length * cell_length * cell_length;
        k_pm_contrast<<<blocks(cells), TPB, 0, s>>>(mesh, cells,
                                                    1.0 / (cell_volume * mean_bkg_density));
        GS_CUDA(cudaGetLastError());
        GS_CUFFT(cufftSetStream(fwd_, s));
        GS_CUFFT(cufftExecD2Z(fwd_, mesh, spec_.as<cufftDoubleComplex>()));
        const double two_pi_over_l2 = 4.0 * M_PI * M_PI / (box_length * box_length);
        const long long half = (long long)g * g * (g / 2 + 1);
        k_pm_green<<<blocks(half), TPB, 0, s>>>(spec_.as<double2>(), g, two_pi_over_l2);
        GS_CUDA(cudaGetLastError());
        GS_CUFFT(cufftSetStream(inv_, s));
        GS_CUFFT(cufftExecZ2D(inv_, spec_.as<cufftDoubleComplex>(), mesh));
        const double factor = ((3.0 / 2.0) * omega_m * H0 * H0) / (scale_factor * (double)cells);
        k_pm_gradient<<<blocks(cells), TPB, 0, s>>>(mesh, g, factor / (12.0 * cell_length),
                                                    acc_.as<double>());
        k_pm_interp<<<blocks(n), TPB, 0, s>>>(d_x, n, G, acc_.as<double>(), d_a);
        GS_CUDA(cudaGetLastError());
        return ok();
    }

  private:
    int g_ = 0;
    cufftHandle fwd_ = 0, inv_ = 0;
    DBuf mesh_, spec_, acc_;
};

namespace {

struct PmCall {
    cudaStream_t stream = nullptr;
    PmSolver solver;
    DBuf x, m, a;
    cudaEvent_t ev[2] = {nullptr, nullptr};   // around the step loop
    double loop_ms = 0.0;
    int64_t loop_steps = 0;
    ~PmCall()
    {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

thread_local std::unique_ptr<PmCall> tl_pm;

ErrorStatus pm_call(PmCall **out)
{
    if (!tl_pm) {
        const DeviceInfo *d = nullptr;
        GS_TRY(device_info(&d));
        std::unique_ptr<PmCall> c(new PmCall());
        GS_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        GS_CUDA(cudaEventCreate(&c->ev[0]));
        GS_CUDA(cudaEventCreate(&c->ev[1]));
        tl_pm = std::move(c);
    }
    *out = tl_pm.get();
    return ok();
}

ErrorStatus pm_check(int n, const double *x, const double *m, const double *box_center,
                     int g)
{
    if (!x || !m || !box_center) return GS_RAISE(GRAV_POINTER_ERROR, "NULL array");
    if (n <= 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles must be positive. Got: %d", n);
    if (g <= 0) return GS_RAISE(GRAV_VALUE_ERROR, "pm_grid_size must be positive. Got: %d", g);
    if ((long long)g * g * g > (1LL << 31))
        return GS_RAISE(GRAV_VALUE_ERROR, "pm_grid_size %d gives more than 2^31 cells", g);
    return ok();
}

}  // namespace

ErrorStatus pm_acceleration_host(double *a, int n, const double *x, const double *m,
                                 const double *box_center, double box_width, double H0,
                                 double omega_m, double mean_bkg_density, int g,
                                 double scale_factor)
{
    if (!a) return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration array is NULL");
    GS_TRY(pm_check(n, x, m, box_center, g));
    PmCall *c = nullptr;
    GS_TRY(pm_call(&c));
    const size_t b3 = (size_t)n * 3 * sizeof(double);
    GS_TRY(c->x.reserve(b3));
    GS_TRY(c->a.reserve(b3));
    GS_TRY(c->m.reserve((size_t)n * sizeof(double)));
    GS_CUDA(cudaMemcpyAsync(c->x.p, x, b3, cudaMemcpyHostToDevice, c->stream));
    GS_CUDA(cudaMemcpyAsync(c->m.p, m, (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                            c->stream));
    GS_TRY(c->solver.compute(c->a.as<double>(), n, c->x.as<double>(), c->m.as<double>(),
                             box_center, box_width, H0, omega_m, mean_bkg_density, g,
                             scale_factor, c->stream));
    GS_CUDA(cudaMemcpyAsync(a, c->a.p, b3, cudaMemcpyDeviceToHost, c->stream));
    GS_CUDA(cudaStreamSynchronize(c->stream));
    return ok();
}

// src/integrator_cosmology_leapfrog.c:24-255.  x is advanced in HBM; the
// host v is written only at snapshots (v = p / a^2), as the reference
// writes it, and is otherwise left as given.
ErrorStatus pm_leapfrog_cosmology(CosmologicalSystem *system, SimulationStatus *status,
                                  OutputParam *op, const bool *is_exit, double dt, double a_begin,
                                  double a_final, int g)
{
    const int n = system->num_particles;
    GS_TRY(pm_check(n, system->x, system->m, system->box_center, g));
    const double H0 = system->h * 100.0;
    const double omega_m = system->omega_m, omega_lambda = system->omega_lambda;
    const double *c = system->box_center;
    const double bw = system->box_width;
    PmCall *pc = nullptr;
    GS_TRY(pm_call(&pc));
    cudaStream_t s = pc->stream;
    const int L = 3 * n;
    const size_t b3 = (size_t)L * sizeof(double);
    DBuf x, v, m, p, a;
    GS_TRY(x.reserve(b3));
    GS_TRY(v.reserve(b3));
    GS_TRY(p.reserve(b3));
    GS_TRY(a.reserve(b3));
    GS_TRY(m.reserve((size_t)n * sizeof(double)));
    GS_CUDA(cudaMemcpyAsync(x.p, system->x, b3, cudaMemcpyHostToDevice, s));
    GS_CUDA(cudaMemcpyAsync(v.p, system->v, b3, cudaMemcpyHostToDevice, s));
    GS_CUDA(cudaMemcpyAsync(m.p, system->m, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));

    double t = a_begin;
    if (status) status->t = t;
    // snapshots (:49-52, :76-88): the initial one of the caller's arrays
    const bool is_output = op && op->method != OUTPUT_METHOD_DISABLED;
    double next_output_time = is_output ? op->output_interval : 0.0;
    if (is_output && op->output_initial) GS_TRY(output_snapshot_cosmology(op, system, t));
    double msum = 0.0;   // vec_sum (src/math_functions.c:13-21), in order
    for (int i = 0; i < n; ++i) msum += system->m[i];
    const double mean_bkg_density = msum / ((bw * 2) * (bw * 2) * (bw * 2));

    k_cosmo_wrap<<<blocks(L), TPB, 0, s>>>(x.as<double>(), L, c[0], c[1], c[2], bw);
    k_cosmo_momentum<<<blocks(L), TPB, 0, s>>>(p.as<double>(), v.as<double>(), L, t);
    GS_CUDA(cudaGetLastError());
    GS_TRY(pc->solver.compute(a.as<double>(), n, x.as<double>(), m.as<double>(), c, bw, H0,
                              omega_m, mean_bkg_density, g, t, s));
    // ceil((a_final - a_begin) / dt) steps; dt = 0 (allowed by the checks)
    // gives no finite count, and no steps are taken
    const double q = (a_final - a_begin) / dt;
    const int64_t total = (std::isfinite(q) && q >= 0.0) ? (int64_t)std::ceil(q) : 0;
    if (status) status->dt = dt;
    int64_t steps = 0;
    GS_CUDA(cudaEventRecord(pc->ev[0], s));
    while (steps < total) {
        if (t + dt > a_final) dt = a_final - t;
        if (status) status->dt = dt;
        double da = compute_da(t, H0, omega_m, omega_lambda);
        k_cosmo_kick<<<blocks(L), TPB, 0, s>>>(p.as<double>(), a.as<double>(), L, 0.5 * dt / da);
        t += 0.5 * dt;
        da = compute_da(t, H0, omega_m, omega_lambda);
        k_cosmo_drift<<<blocks(L), TPB, 0, s>>>(x.as<double>(), p.as<double>(), L,
                                                dt / (t * t * da), c[0], c[1], c[2], bw);
        GS_CUDA(cudaGetLastError());
        GS_TRY(pc->solver.compute(a.as<double>(), n, x.as<double>(), m.as<double>(), c, bw, H0,
                                  omega_m, mean_bkg_density, g, t, s));
        k_cosmo_kick<<<blocks(L), TPB, 0, s>>>(p.as<double>(), a.as<double>(), L, 0.5 * dt / da);
        GS_CUDA(cudaGetLastError());
        ++steps;
        t = a_begin + steps * dt;
        if (status) {
            status->t = t;
            status->num_steps = steps;
        }
        if (is_output && t >= next_output_time) {
            // the host arrays get x and v = p / a^2, then the snapshot (:198-221)
            k_cosmo_velocity<<<blocks(L), TPB, 0, s>>>(v.as<double>(), p.as<double>(), L, t);
            GS_CUDA(cudaGetLastError());
            GS_CUDA(cudaMemcpyAsync(system->x, x.p, b3, cudaMemcpyDeviceToHost, s));
            GS_CUDA(cudaMemcpyAsync(system->v, v.p, b3, cudaMemcpyDeviceToHost, s));
            GS_CUDA(cudaStreamSynchronize(s));
            GS_TRY(output_snapshot_cosmology(op, system, t));
            next_output_time = op->output_count_ * op->output_interval;
        }
        if (is_exit && *is_exit) break;
    }
    GS_CUDA(cudaEventRecord(pc->ev[1], s));
    GS_CUDA(cudaMemcpyAsync(system->x, x.p, b3, cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    GS_CUDA(cudaEventElapsedTime(&ms, pc->ev[0], pc->ev[1]));
    pc->loop_ms = ms;
    pc->loop_steps = steps;
    return ok();
}

ErrorStatus pm_last_timing(double *loop_ms, int64_t *steps)
{
    if (!tl_pm) return GS_RAISE(GRAV_VALUE_ERROR, "no cosmological run on this thread");
    if (loop_ms) *loop_ms = tl_pm->loop_ms;
    if (steps) *steps = tl_pm->loop_steps;
    return ok();
}

}  // namespace gs
