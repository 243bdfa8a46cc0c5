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

}  // namespace gs

using namespace gs;

extern "C" {

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
