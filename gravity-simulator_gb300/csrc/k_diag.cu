// k_diag.cu -- FP64 energy and momentum diagnostics on the GPU.
//
// Replaces compute_energy_python / compute_linear_momentum_python /
// compute_angular_momentum_python (src/python_interface.c:195-304) and
// compute_energy (src/utils.c:27-59).  sol_state holds, per snapshot and
// particle, (m, x, y, z, vx, vy, vz).  Per particle i a thread forms
// KE_i - sum_{j>i} G m_i m_j / |x_i - x_j| in the reference's expression
// order; the per-particle terms are then summed in index order by a fixed
// two-level tree, so the result is deterministic and agrees with the
// reference's serial sum to round-off (relative 1e-13 at N = 10^4).
// The "momentum" figures keep the reference's definition: sums of vector
// components, m (vx + vy + vz) and m (L_x + L_y + L_z) per particle.
#include "gs_internal.h"
#include "gs_ptx.cuh"

#include <algorithm>
#include <cstdio>
#include <vector>

namespace gs {

constexpr int DG_THREADS = 256;

__device__ __forceinline__ double norm3(double a, double b, double c)
{
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c)));
}

// kind 0: energy, 1: linear momentum, 2: angular momentum.  One block sums
// DG_THREADS consecutive particles of one snapshot into part[snapshot][block].
__global__ void __launch_bounds__(DG_THREADS)
k_diag_terms(const double *__restrict__ st, int n, int blocks_per_snap, double G, int kind,
             double *__restrict__ part)
{
    __shared__ double red[DG_THREADS];
    const int snap = blockIdx.x / blocks_per_snap;
    const int blk = blockIdx.x % blocks_per_snap;
    const int i = blk * DG_THREADS + threadIdx.x;
    const double *S = st + (size_t)snap * n * 7;
    double e = 0.0;
    if (i < n) {
        const double mi = S[7 * i + 0];
        const double xi = S[7 * i + 1], yi = S[7 * i + 2], zi = S[7 * i + 3];
        const double vx = S[7 * i + 4], vy = S[7 * i + 5], vz = S[7 * i + 6];
        if (kind == 0) {
            const double vn = norm3(vx, vy, vz);
            e = __dmul_rn(__dmul_rn(__dmul_rn(0.5, mi), vn), vn);
            for (int j = i + 1; j < n; ++j) {
                const double mj = S[7 * j + 0];
                const double r = norm3(__dsub_rn(xi, S[7 * j + 1]), __dsub_rn(yi, S[7 * j + 2]),
                                       __dsub_rn(zi, S[7 * j + 3]));
                e = __dsub_rn(e, __ddiv_rn(__dmul_rn(__dmul_rn(G, mi), mj), r));
            }
        } else if (kind == 1) {
            e = __dmul_rn(mi, __dadd_rn(__dadd_rn(vx, vy), vz));
        } else {
            const double c0 = __dsub_rn(__dmul_rn(yi, vz), __dmul_rn(zi, vy));
            const double c1 = __dsub_rn(__dmul_rn(zi, vx), __dmul_rn(xi, vz));
            const double c2 = __dsub_rn(__dmul_rn(xi, vy), __dmul_rn(yi, vx));
            e = __dmul_rn(mi, __dadd_rn(__dadd_rn(c0, c1), c2));
        }
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int w = DG_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

static ErrorStatus diag(const double *h_state, int num_snapshots, int n, double G, int kind,
                        double *h_out)
{
    if (!h_state || !h_out) return GS_RAISE(GRAV_POINTER_ERROR, "NULL argument");
    if (num_snapshots <= 0 || n <= 0) return ok();
    const DeviceInfo *d = nullptr;
    GS_TRY(device_info(&d));
    const int bps = (n + DG_THREADS - 1) / DG_THREADS;
    // snapshots in batches bounded to ~256 MiB of state
    const size_t per_snap = (size_t)n * 7 * sizeof(double);
    int batch = (int)std::max<size_t>(1, ((size_t)256 << 20) / per_snap);
    if (batch > num_snapshots) batch = num_snapshots;
    DBuf st, part;
    GS_TRY(st.reserve(per_snap * batch));
    GS_TRY(part.reserve((size_t)batch * bps * sizeof(double)));
    std::vector<double> hp((size_t)batch * bps);
    for (int s0 = 0; s0 < num_snapshots; s0 += batch) {
        const int nb = std::min(batch, num_snapshots - s0);
        GS_CUDA(cudaMemcpy(st.p, h_state + (size_t)s0 * n * 7, per_snap * nb,
                           cudaMemcpyHostToDevice));
        k_diag_terms<<<nb * bps, DG_THREADS>>>(st.as<double>(), n, bps, G, kind,
                                                part.as<double>());
        GS_CUDA(cudaGetLastError());
        GS_CUDA(cudaMemcpy(hp.data(), part.p, (size_t)nb * bps * sizeof(double),
                           cudaMemcpyDeviceToHost));
        for (int s = 0; s < nb; ++s) {
            double acc = 0.0;
            for (int b = 0; b < bps; ++b) acc += hp[(size_t)s * bps + b];
            h_out[s0 + s] = acc;
        }
    }
    return ok();
}

// ---- softened potential energy for large N --------------------------------
// phi_i = sum_{j != i} m_j / sqrt(|x_i - x_j|^2 + eps^2) for one i per
// thread, with the j particles staged through shared memory 256 at a time.
// Coordinates are double-float (hi + lo) relative to the bounding-box
// centre, so each difference keeps about 48 bits; the terms are summed in
// FP32 per 64 and the partial sums Kahan-compensated.
constexpr int EN_THREADS = 256;
constexpr int EN_PARTIAL = 64;

__global__ void __launch_bounds__(EN_THREADS)
k_softened_phi(const float4 *__restrict__ ph, const float4 *__restrict__ pl, int n, float eps2,
               double *__restrict__ phi)
{
    __shared__ float4 sh[EN_THREADS], sl[EN_THREADS];
    const int i = blockIdx.x * EN_THREADS + threadIdx.x;
    const float4 xh = i < n ? ph[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 xl = i < n ? pl[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float s = 0.f, c = 0.f;
    for (int t0 = 0; t0 < n; t0 += EN_THREADS) {
        __syncthreads();
        const int j = t0 + threadIdx.x;
        sh[threadIdx.x] = j < n ? ph[j] : make_float4(0.f, 0.f, 0.f, 0.f);   // m = 0 pads
        sl[threadIdx.x] = j < n ? pl[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        const int cnt = min(EN_THREADS, n - t0);
        for (int k0 = 0; k0 < cnt; k0 += EN_PARTIAL) {
            float part = 0.f;
            const int k1 = min(cnt, k0 + EN_PARTIAL);
#pragma unroll 4
            for (int k = k0; k < k1; ++k) {
                const float4 yh = sh[k], yl = sl[k];
                const float dx = (yh.x - xh.x) + (yl.x - xl.x);
                const float dy = (yh.y - xh.y) + (yl.y - xl.y);
                const float dz = (yh.z - xh.z) + (yl.z - xl.z);
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                const float w = (t0 + k == i) ? 0.f : yh.w;
                part = fmaf(w, rsqrt_approx(r2), part);
            }
            kahan_add(s, c, part);
        }
    }
    if (i < n) phi[i] = (double)s - (double)c;
}

ErrorStatus softened_energy(const double *x, const double *v, const double *m, int n, double G,
                            double eps, double *energy)
{
    double ke = 0.0;
    for (int i = 0; i < n; ++i) {
        const double v2 = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
                          v[3 * i + 2] * v[3 * i + 2];
        ke += 0.5 * m[i] * v2;
    }
    if (n < 2) {
        *energy = ke;
        return ok();
    }
    double lo[3] = {x[0], x[1], x[2]}, hi[3] = {x[0], x[1], x[2]};
    for (int i = 1; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], x[3 * i + k]);
            hi[k] = std::max(hi[k], x[3 * i + k]);
        }
    std::vector<float4> hph(n), hpl(n);
    for (int i = 0; i < n; ++i) {
        float h[3], l[3];
        for (int k = 0; k < 3; ++k) {
            const double d = x[3 * i + k] - 0.5 * (lo[k] + hi[k]);
            h[k] = (float)d;
            l[k] = (float)(d - (double)h[k]);
        }
        hph[i] = make_float4(h[0], h[1], h[2], (float)m[i]);
        hpl[i] = make_float4(l[0], l[1], l[2], 0.f);
    }
    DBuf dph, dpl, dphi;
    GS_TRY(dph.reserve((size_t)n * sizeof(float4)));
    GS_TRY(dpl.reserve((size_t)n * sizeof(float4)));
    GS_TRY(dphi.reserve((size_t)n * sizeof(double)));
    GS_CUDA(cudaMemcpy(dph.p, hph.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice));
    GS_CUDA(cudaMemcpy(dpl.p, hpl.data(), (size_t)n * sizeof(float4), cudaMemcpyHostToDevice));
    k_softened_phi<<<(n + EN_THREADS - 1) / EN_THREADS, EN_THREADS>>>(
        dph.as<float4>(), dpl.as<float4>(), n, (float)(eps * eps), dphi.as<double>());
    GS_CUDA(cudaGetLastError());
    std::vector<double> phi(n);
    GS_CUDA(cudaMemcpy(phi.data(), dphi.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    double pe = 0.0;
    for (int i = 0; i < n; ++i) pe += m[i] * phi[i];
    *energy = ke - 0.5 * G * pe;
    return ok();
}

}  // namespace gs

using namespace gs;

extern "C" {

int gsgpu_softened_energy(const double *x, const double *v, const double *m, int n, double G,
                          double eps, double *energy)
{
    if (!x || !v || !m || !energy) return GRAV_POINTER_ERROR;
    if (n < 0) return GRAV_VALUE_ERROR;
    ErrorStatus st = softened_energy(x, v, m, n, G, eps, energy);
    if (st.return_code != GRAV_SUCCESS) {
        const int rc = st.return_code;
        print_and_free_traceback(&st);
        return rc;
    }
    return GRAV_SUCCESS;
}

void compute_energy_python(double *energy, double G, const double *sol_state,
                           int32_t num_snapshots, int32_t num_particles)
{
    ErrorStatus st = diag(sol_state, num_snapshots, num_particles, G, 0, energy);
    if (st.return_code != GRAV_SUCCESS) print_and_free_traceback(&st);
}

void compute_linear_momentum_python(double *linear_momentum, const double *sol_state,
                                    int32_t num_snapshots, int32_t num_particles)
{
    ErrorStatus st = diag(sol_state, num_snapshots, num_particles, 0.0, 1, linear_momentum);
    if (st.return_code != GRAV_SUCCESS) print_and_free_traceback(&st);
}

void compute_angular_momentum_python(double *angular_momentum, const double *sol_state,
                                     int32_t num_snapshots, int32_t num_particles)
{
    ErrorStatus st = diag(sol_state, num_snapshots, num_particles, 0.0, 2, angular_momentum);
    if (st.return_code != GRAV_SUCCESS) print_and_free_traceback(&st);
}

double compute_energy(const System *system)
{
    if (!system || system->num_particles <= 0 || !system->x || !system->v || !system->m)
        return 0.0;
    const int n = system->num_particles;
    std::vector<double> state((size_t)n * 7);
    for (int i = 0; i < n; ++i) {
        state[7 * i] = system->m[i];
        for (int k = 0; k < 3; ++k) {
            state[7 * i + 1 + k] = system->x[3 * i + k];
            state[7 * i + 4 + k] = system->v[3 * i + k];
        }
    }
    double e = 0.0;
    ErrorStatus st = diag(state.data(), 1, n, system->G, 0, &e);
    if (st.return_code != GRAV_SUCCESS) print_and_free_traceback(&st);
    return e;
}

}  // extern "C"
