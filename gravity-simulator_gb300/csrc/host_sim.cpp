// host_sim.cpp -- acceleration(), launch_simulation(), the Python entry point
// and the device-resident simulation object.
//
// The integrator loops follow src/integrator.c (euler :281-454,
// euler_cromer :456-628, rk4 :630-892, leapfrog :894-1121): the same step
// count ceil(tf/dt), the same last-step dt clamp (all but rk4), t = steps*dt,
// one is_exit check per step.  The state (x, v, compensation terms) stays in
// HBM for the whole run; only the initial state goes host->device and the
// final state device->host.  A step's kernels are captured once in a CUDA
// graph and replayed; a clamped last step is launched directly.
#include "gs_internal.h"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

namespace gs {
namespace {

// How embedded Runge-Kutta runs add their error terms: 0 on the host in the
// reference's order (bit-exact step control, the default), 1 on the device
// (gsgpu_set_rk_error_sum).
std::atomic<int> g_rk_error_sum{0};

struct Frame {
    double c[3];
};

// Centre of the bounding box (the FP64 origin of FP32 pair terms).
Frame bbox_centre(int n, const double *x)
{
    double lo[3] = {x[0], x[1], x[2]}, hi[3] = {x[0], x[1], x[2]};
    for (int i = 1; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const double q = x[3 * i + k];
            lo[k] = q < lo[k] ? q : lo[k];
            hi[k] = q > hi[k] ? q : hi[k];
        }
    Frame f;
    for (int k = 0; k < 3; ++k) f.c[k] = 0.5 * (lo[k] + hi[k]);
    return f;
}

// Per-thread state for host-buffer acceleration() calls.
struct CallContext {
    cudaStream_t stream = nullptr;
    DBuf x, m, a;
    std::unique_ptr<Engine> engine;
    int method = -1, n = -1, leaf = 0;
    double G = 0.0, eps = -1.0, theta = -1.0;
    ~CallContext()
    {
        if (stream) cudaStreamDestroy(stream);
    }
};

}  // namespace

thread_local std::unique_ptr<CallContext> tl_call;

namespace {

ErrorStatus call_context(CallContext **out)
{
    if (!tl_call) {
        const DeviceInfo *d = nullptr;
        GS_TRY(device_info(&d));
        std::unique_ptr<CallContext> c(new CallContext());
        GS_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        tl_call = std::move(c);
    }
    *out = tl_call.get();
    return ok();
}

ErrorStatus check_system(const System *s, bool need_v)
{
    if (!s) return GS_RAISE(GRAV_POINTER_ERROR, "System is NULL");
    if (s->num_particles <= 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles must be positive. Got: %d",
                        s->num_particles);
    if (s->num_particles > kMaxParticles)
        return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles exceeds %d. Got: %d", kMaxParticles,
                        s->num_particles);
    if (!s->x) return GS_RAISE(GRAV_POINTER_ERROR, "System array x is NULL");
    if (need_v && !s->v) return GS_RAISE(GRAV_POINTER_ERROR, "System array v is NULL");
    if (!s->m) return GS_RAISE(GRAV_POINTER_ERROR, "System array m is NULL");
    return ok();
}

}  // namespace

// Host-buffer acceleration on the GPU (src/acceleration.c:131-153).
ErrorStatus accel_host(double *a, const System *system, const AccelerationParam *param_in)
{
    if (!a) return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration array is NULL");
    if (!param_in) return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration parameter pointer is NULL");
    GS_TRY(check_system(system, false));
    AccelerationParam p = *param_in;
    GS_TRY(finalize_acceleration_param(&p));
    CallContext *c = nullptr;
    GS_TRY(call_context(&c));
    const int n = system->num_particles;
    const bool same = c->engine && c->method == p.method && c->n == n && c->G == system->G &&
                      c->eps == p.softening_length && c->theta == p.opening_angle &&
                      c->leaf == p.max_num_particles_per_leaf;
    if (!same) {
        c->engine.reset();
        GS_TRY(make_engine(p.method, c->engine));
        GS_TRY(c->engine->setup(n, system->G, p));
        c->method = p.method;
        c->n = n;
        c->G = system->G;
        c->eps = p.softening_length;
        c->theta = p.opening_angle;
        c->leaf = p.max_num_particles_per_leaf;
    }
    const Frame f = bbox_centre(n, system->x);
    c->engine->set_frame_centre(f.c[0], f.c[1], f.c[2]);
    GS_TRY(c->x.reserve((size_t)n * 3 * sizeof(double)));
    GS_TRY(c->m.reserve((size_t)n * sizeof(double)));
    GS_TRY(c->a.reserve((size_t)n * 3 * sizeof(double)));
    GS_CUDA(cudaMemcpyAsync(c->x.p, system->x, (size_t)n * 3 * sizeof(double),
                            cudaMemcpyHostToDevice, c->stream));
    GS_CUDA(cudaMemcpyAsync(c->m.p, system->m, (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                            c->stream));
    GS_TRY(c->engine->compute(c->x.as<double>(), c->m.as<double>(), c->a.as<double>(), c->stream,
                              nullptr));
    GS_CUDA(cudaMemcpyAsync(a, c->a.p, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    GS_CUDA(cudaStreamSynchronize(c->stream));
    GS_TRY(c->engine->check_status(c->stream));
    return ok();
}

}  // namespace gs

// ---------------------------------------------------------------------------
// Device-resident simulation.
// ---------------------------------------------------------------------------
using namespace gs;

struct gsgpu_sim {
    int n = 0;
    double G = 1.0;
    AccelerationParam p{};
    int integrator = INTEGRATOR_LEAPFROG;
    double dt = 0.0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    DBuf x, v, m, a, xe, ve, x0, v0, tmp;
    DBuf rk[8];   // rk4: vk1..vk4, xk1..xk4
    std::unique_ptr<Engine> engine;
    bool primed = false;   // leapfrog: half kick applied
    double last_dt = 0.0;  // dt of the most recent step
    cudaGraphExec_t graph = nullptr;
    double graph_dt = 0.0;
    bool graph_failed = false;
    ForceTimer timer;
    ForceTimer t_morton, t_sort;   // tree builds of Barnes-Hut engines
    int kernels_last = 0;
    // embedded Runge-Kutta (integrators 5-8) and IAS15 (9)
    double tolerance = -1.0, initial_dt = -1.0;
    DBuf e_vk, e_xk, e_x1, e_v1, e_txe, e_tve, e_xs, e_terms, e_esum;
    double *h_terms = nullptr;   // pinned host copy of the 6N error terms
    DBuf i_b0, i_b, i_g, i_e, i_F, i_a1, i_d7, i_max;
    unsigned long long *h_max = nullptr;   // pinned: two maxima

    ~gsgpu_sim()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (h_terms) cudaFreeHost(h_terms);
        if (h_max) cudaFreeHost(h_max);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    // src/integrator_rk_embedded.c:346-520 on host copies of x, v and the
    // GPU accelerations, with the reference's long double intermediates.
    ErrorStatus rk_emb_initial_dt(int power, double *out)
    {
        const size_t L = (size_t)3 * n;
        std::vector<double> hx(L), hv(L), ha(L), ha1(L), sx(L), sv(L), hx1(L), hv1(L);
        GS_TRY(force(a.as<double>()));
        GS_CUDA(cudaMemcpyAsync(hx.data(), x.p, bytes3(), cudaMemcpyDeviceToHost, stream));
        GS_CUDA(cudaMemcpyAsync(hv.data(), v.p, bytes3(), cudaMemcpyDeviceToHost, stream));
        GS_CUDA(cudaMemcpyAsync(ha.data(), a.p, bytes3(), cudaMemcpyDeviceToHost, stream));
        GS_CUDA(cudaStreamSynchronize(stream));
        GS_TRY(engine->check_status(stream));
        const double tol = tolerance;
        for (size_t k = 0; k < L; ++k) {
            sx[k] = tol + tol * std::fabs(hx[k]);
            sv[k] = tol + tol * std::fabs(hv[k]);
        }
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (size_t k = 0; k < L; ++k) {
            s0 += (hx[k] / sx[k]) * (hx[k] / sx[k]);
            s0 += (hv[k] / sv[k]) * (hv[k] / sv[k]);
            s1 += (hv[k] / sx[k]) * (hv[k] / sx[k]);
            s1 += (ha[k] / sv[k]) * (ha[k] / sv[k]);
        }
        const double d0 = std::sqrt(s0 / (n * 6));
        const double d1 = std::sqrt(s1 / (n * 6));
        const double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-4 : d0 / d1;
        for (size_t k = 0; k < L; ++k) {
            hx1[k] = hx[k] + (dt0 / 100.0) * hv[k];
            hv1[k] = hv[k] + (dt0 / 100.0) * ha[k];
        }
        GS_CUDA(cudaMemcpyAsync(e_xs.p, hx1.data(), bytes3(), cudaMemcpyHostToDevice, stream));
        GS_TRY(engine->compute(e_xs.as<double>(), m.as<double>(), tmp.as<double>(), stream,
                               nullptr));
        GS_CUDA(cudaMemcpyAsync(ha1.data(), tmp.p, bytes3(), cudaMemcpyDeviceToHost, stream));
        GS_CUDA(cudaStreamSynchronize(stream));
        GS_TRY(engine->check_status(stream));
        for (size_t k = 0; k < L; ++k) {
            s2 += ((hv1[k] - hv[k]) / sx[k]) * ((hv1[k] - hv[k]) / sx[k]);
            s2 += ((ha1[k] - ha[k]) / sv[k]) * ((ha1[k] - ha[k]) / sv[k]);
        }
        const double d2 = std::sqrt(s2 / (n * 6)) / dt0;
        const double dt1 = std::pow((double)(0.01L / (long double)std::fmax(d1, d2)),
                                    (double)(1.0L / (long double)(1 + power)));
        const double dtv = std::fmin((double)(100.0L * (long double)dt0), dt1);
        *out = dtv * 1e-2;
        if (*out <= 0.0) return GS_RAISE(GRAV_VALUE_ERROR, "Initial dt is negative");
        return ok();
    }

    // Exact maxima of |u| and |w| over 3N elements (one synchronisation).
    ErrorStatus absmax2(const double *u, const double *w, double *mu, double *mw)
    {
        GS_CUDA(cudaMemsetAsync(i_max.p, 0, 2 * sizeof(unsigned long long), stream));
        launch_ias_absmax2(len(), u, w, i_max.as<unsigned long long>(), stream);
        GS_CUDA(cudaGetLastError());
        GS_CUDA(cudaMemcpyAsync(h_max, i_max.p, 2 * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, stream));
        GS_CUDA(cudaStreamSynchronize(stream));
        GS_TRY(engine->check_status(stream));
        std::memcpy(mu, &h_max[0], sizeof(double));
        std::memcpy(mw, &h_max[1], sizeof(double));
        return ok();
    }

    // src/integrator_ias15.c:229-616.  The element-wise predictor, g / b
    // updates, step end and b prediction run on the GPU (k_ias15.cu); the
    // predictor-corrector iterations, the convergence test, the error
    // estimate (glibc pow) and the step-size control run here on exact
    // maxima, so the step sequence is the reference's.
    ErrorStatus ias15_run(double tf, SimulationStatus *status, const bool *is_exit,
                          OutputContext *oc)
    {
        if (!(tolerance > 0.0))
            return GS_RAISE(GRAV_VALUE_ERROR, "tolerance must be positive. Got: %g", tolerance);
        const int L = len();
        const size_t SL = (size_t)L;
        double *b0 = i_b0.as<double>(), *b = i_b.as<double>(), *g = i_g.as<double>(),
               *e = i_e.as<double>(), *F = i_F.as<double>(), *a1 = i_a1.as<double>(),
               *d7 = i_d7.as<double>();
        double *x1 = e_x1.as<double>(), *v1 = e_v1.as<double>(), *txe = e_txe.as<double>(),
               *tve = e_tve.as<double>();
        GS_CUDA(cudaMemsetAsync(b0, 0, 7 * SL * sizeof(double), stream));
        GS_CUDA(cudaMemsetAsync(b, 0, 7 * SL * sizeof(double), stream));
        GS_CUDA(cudaMemsetAsync(g, 0, 7 * SL * sizeof(double), stream));
        GS_CUDA(cudaMemsetAsync(e, 0, 7 * SL * sizeof(double), stream));
        GS_CUDA(cudaMemsetAsync(F, 0, 8 * SL * sizeof(double), stream));
        GS_TRY(force(a.as<double>()));
        double h;
        if (initial_dt > 0.0) {
            h = initial_dt;
        } else {
            // src/integrator_ias15.c:702-806 (power 15)
            double d0 = 0.0, d1 = 0.0, d2 = 0.0, dummy = 0.0;
            GS_TRY(absmax2(x.as<double>(), a.as<double>(), &d0, &d1));
            const double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
            launch_ias_axpy(L, x1, x.as<double>(), dt0, v.as<double>(), stream);
            GS_CUDA(cudaGetLastError());
            GS_TRY(engine->compute(x1, m.as<double>(), a1, stream, nullptr));
            launch_ias_sub(L, d7, a1, a.as<double>(), stream);
            GS_CUDA(cudaGetLastError());
            GS_TRY(absmax2(d7, d7, &d2, &dummy));
            d2 = d2 / dt0;
            double dt1;
            if (std::fmax(d1, d2) <= 1e-15)
                dt1 = std::fmax(1e-6, dt0 * 1e-3);
            else
                dt1 = std::pow((0.01 / std::fmax(d1, d2)), 1.0 / (1.0 + (double)15));
            h = std::fmin(100.0 * dt0, dt1);
            if (h <= 0.0) return GS_RAISE(GRAV_VALUE_ERROR, "Initial dt is less than or equal to zero");
            if (h > tf) h = tf;
        }
        GS_TRY(initial_snapshot(oc, status));
        double t = 0.0;
        int64_t steps = 0;
        bool refine = false;
        if (status) {
            status->t = 0.0;
            status->dt = h;
            status->num_steps = 0;
        }
        while (t < tf) {
            for (int it = 0; it < 12; ++it) {
                for (int i = 0; i < 8; ++i) {
                    launch_ias_predict(L, x1, v1, x.as<double>(), v.as<double>(), a.as<double>(),
                                       kIas15H[i], b, h, xe.as<double>(), ve.as<double>(), stream);
                    GS_CUDA(cudaGetLastError());
                    GS_TRY(engine->compute(x1, m.as<double>(), F + (size_t)i * SL, stream,
                                           timer.enabled ? &timer : nullptr));
                    launch_ias_update_gb(L, g, b, F, i, stream);
                    GS_CUDA(cudaGetLastError());
                }
                launch_ias_delta(L, b, b0, d7, stream);
                GS_CUDA(cudaGetLastError());
                double md = 0.0, mf = 0.0;
                GS_TRY(absmax2(d7, F + 7 * SL, &md, &mf));
                if ((md / mf) < 1e-16) break;
            }
            GS_CUDA(cudaMemcpyAsync(txe, xe.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
            GS_CUDA(cudaMemcpyAsync(tve, ve.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
            launch_ias_advance(L, x1, v1, txe, tve, x.as<double>(), v.as<double>(), a.as<double>(),
                               b, h, stream);
            GS_CUDA(cudaGetLastError());
            GS_TRY(engine->compute(x1, m.as<double>(), a1, stream, nullptr));
            double mb = 0.0, ma = 0.0;
            GS_TRY(absmax2(b + 6 * SL, a1, &mb, &ma));
            const double eb7 = mb / ma;
            double error = std::pow((eb7 / tolerance), 1.0 / 7.0);
            // With every acceleration zero (a single particle, or no mass) the
            // estimate is 0/0; the reference's loop then never advances t and
            // never ends.  Stop with an error instead.
            if (std::isnan(error))
                return GS_RAISE(GRAV_VALUE_ERROR,
                                "IAS15 error estimate is not a number (all accelerations are "
                                "zero); the step size cannot be controlled");
            if (error < 1e-10) error = 1e-10;
            const double dt_new = h / error;
            if (error <= 1.0 || h == tf * 1e-12) {
                ++steps;
                t += h;
                const double q = dt_new / h;
                double qs[7];
                qs[0] = q;
                for (int r = 1; r < 7; ++r) qs[r] = qs[r - 1] * q;
                launch_ias_refine(L, b, e, qs, refine ? 1 : 0, stream);
                GS_CUDA(cudaGetLastError());
                refine = true;
                GS_CUDA(cudaMemcpyAsync(xe.p, txe, bytes3(), cudaMemcpyDeviceToDevice, stream));
                GS_CUDA(cudaMemcpyAsync(ve.p, tve, bytes3(), cudaMemcpyDeviceToDevice, stream));
                GS_CUDA(cudaMemcpyAsync(x.p, x1, bytes3(), cudaMemcpyDeviceToDevice, stream));
                GS_CUDA(cudaMemcpyAsync(v.p, v1, bytes3(), cudaMemcpyDeviceToDevice, stream));
                GS_CUDA(cudaMemcpyAsync(a.p, a1, bytes3(), cudaMemcpyDeviceToDevice, stream));
                if (oc && oc->due(t)) GS_TRY(snapshot(oc, v.as<double>(), t, h));
            }
            if (dt_new > (h / 0.25))
                h /= 0.25;
            else if (dt_new < h * 0.25)
                h *= 0.25;
            else
                h = dt_new;
            if (dt_new < tf * 1e-12) h = tf * 1e-12;
            if (t < tf && t + h > tf) h = tf - t;
            if (status) {
                status->t = t;
                status->dt = h;
                status->num_steps = steps;
            }
            if (is_exit && *is_exit) break;
        }
        GS_CUDA(cudaStreamSynchronize(stream));
        if (oc) GS_TRY(oc->finish());
        return ok();
    }

    // src/integrator_rk_embedded.c:522-987: stages and the weighted combine
    // on the GPU; the RMS error is summed on the host in the reference's
    // element order from the per-element terms, and the step-size control
    // (glibc pow) runs on the host, so accept / reject decisions and dt
    // follow the reference's exactly.
    ErrorStatus rk_emb_run(double tf, SimulationStatus *status, const bool *is_exit,
                           OutputContext *oc)
    {
        const RkTableau *T = rk_tableau(integrator);
        if (!T) return GS_RAISE(GRAV_VALUE_ERROR, "Invalid integrator method");
        if (!(tolerance > 0.0))
            return GS_RAISE(GRAV_VALUE_ERROR, "tolerance must be positive. Got: %g", tolerance);
        const int S = T->stages, L = len();
        const int min_power = T->power < T->power_test ? T->power : T->power_test;
        double dw[13];
        for (int s = 0; s < S; ++s) dw[s] = T->b[s] - T->b_hat[s];
        const double fac = std::pow(0.38, 1.0 / (1.0 + (double)min_power));
        const double fac_max = 6.0, fac_min = 0.33;
        double h;
        if (initial_dt > 0.0) {
            h = initial_dt;
        } else {
            GS_TRY(rk_emb_initial_dt(T->power, &h));
            if (h > tf) h = tf;
        }
        GS_TRY(initial_snapshot(oc, status));
        double t = 0.0;
        int64_t steps = 0;
        if (status) {
            status->t = 0.0;
            status->dt = h;
            status->num_steps = 0;
        }
        double *vk = e_vk.as<double>(), *xk = e_xk.as<double>();
        const bool device_sum = g_rk_error_sum.load(std::memory_order_relaxed) == 1;
        while (t < tf) {
            GS_TRY(force(vk));
            GS_CUDA(cudaMemcpyAsync(xk, v.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
            for (int s = 1; s < S; ++s) {
                launch_rk_emb_stage(x.as<double>(), v.as<double>(), xe.as<double>(),
                                    ve.as<double>(), vk, xk, e_xs.as<double>(), T->a[s], s, h, L,
                                    stream);
                GS_CUDA(cudaGetLastError());
                GS_TRY(engine->compute(e_xs.as<double>(), m.as<double>(), vk + (size_t)s * L,
                                       stream, timer.enabled ? &timer : nullptr));
            }
            double dtdw[13];
            for (int s = 0; s < S; ++s) dtdw[s] = h * dw[s];
            launch_rk_emb_combine(x.as<double>(), v.as<double>(), xe.as<double>(),
                                  ve.as<double>(), vk, xk, e_x1.as<double>(), e_v1.as<double>(),
                                  e_txe.as<double>(), e_tve.as<double>(), e_terms.as<double>(),
                                  T->b, dtdw, S, h, tolerance, tolerance, L, stream);
            GS_CUDA(cudaGetLastError());
            double sum = 0.0;
            if (device_sum) {
                // one double comes back instead of the 6N terms; not the
                // reference's order, so the step control is not bit-exact
                launch_error_sum(e_terms.as<double>(), 2LL * L, e_esum.as<double>(), stream);
                GS_CUDA(cudaGetLastError());
                GS_CUDA(cudaMemcpyAsync(h_terms, e_esum.as<double>() + kErrorSumScratch - 1,
                                        sizeof(double), cudaMemcpyDeviceToHost, stream));
                GS_CUDA(cudaStreamSynchronize(stream));
                GS_TRY(engine->check_status(stream));
                sum = h_terms[0];
            } else {
                GS_CUDA(cudaMemcpyAsync(h_terms, e_terms.p, (size_t)2 * L * sizeof(double),
                                        cudaMemcpyDeviceToHost, stream));
                GS_CUDA(cudaStreamSynchronize(stream));
                GS_TRY(engine->check_status(stream));
                for (int k = 0; k < 2 * L; ++k) sum += h_terms[k];
            }
            double error = std::sqrt(sum / (n * 3 * 2));
            if (error <= 1 || h <= tf * 1e-12) {
                ++steps;
                t += h;
                GS_CUDA(cudaMemcpyAsync(x.p, e_x1.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
                GS_CUDA(cudaMemcpyAsync(v.p, e_v1.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
                GS_CUDA(cudaMemcpyAsync(xe.p, e_txe.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
                GS_CUDA(cudaMemcpyAsync(ve.p, e_tve.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
                if (oc && oc->due(t)) GS_TRY(snapshot(oc, v.as<double>(), t, h));
            }
            if (error < 1e-10) error = 1e-10;
            const double dt_new = h * fac / std::pow(error, 1.0 / (1.0 + (double)min_power));
            if (dt_new > fac_max * h)
                h *= fac_max;
            else if (dt_new < fac_min * h)
                h *= fac_min;
            else
                h = dt_new;
            if (dt_new / tf < 1e-12) h = tf * 1e-12;
            if (t < tf && t + h > tf) h = tf - t;
            if (status) {
                status->t = t;
                status->dt = h;
                status->num_steps = steps;
            }
            if (is_exit && *is_exit) break;
        }
        GS_CUDA(cudaStreamSynchronize(stream));
        if (oc) GS_TRY(oc->finish());
        return ok();
    }

    // The initial snapshot (output_initial): the caller's host state, with
    // the time and dt the status holds on entry, as the reference writes it.
    ErrorStatus initial_snapshot(OutputContext *oc, const SimulationStatus *status)
    {
        if (!oc) return ok();
        oc->begin();
        if (!oc->initial()) return ok();
        const System *sys = oc->system;
        return output_snapshot(oc->op, n, sys->particle_ids, sys->x, sys->v, sys->m, G,
                               status ? status->t : 0.0, status ? status->dt : 0.0);
    }

    // A snapshot of x and the velocity array dv at time t after a step of h
    // (asynchronous: dv must stay unchanged until the next step's kernels).
    ErrorStatus snapshot(OutputContext *oc, const double *dv, double t, double h)
    {
        return oc->take(n, x.as<double>(), dv, nullptr, nullptr, nullptr, stream, t, h);
    }

    size_t bytes3() const { return (size_t)n * 3 * sizeof(double); }
    int len() const { return 3 * n; }

    ErrorStatus force(double *out)
    {
        GS_TRY(engine->compute(x.as<double>(), m.as<double>(), out, stream,
                               timer.enabled ? &timer : nullptr));
        return ok();
    }

    // Leapfrog initial acceleration and half kick (src/integrator.c:962-982).
    ErrorStatus prime()
    {
        if (primed) return ok();
        if (integrator == INTEGRATOR_LEAPFROG) {
            GS_TRY(force(a.as<double>()));
            launch_comp_update(v.as<double>(), ve.as<double>(), a.as<double>(), dt, 0.5, len(),
                               stream);
            GS_CUDA(cudaGetLastError());
        }
        primed = true;
        return ok();
    }

    // Enqueue one step of size h.
    ErrorStatus step(double h)
    {
        const int L = len();
        switch (integrator) {
        case INTEGRATOR_EULER:
            GS_TRY(force(a.as<double>()));
            launch_euler_update(x.as<double>(), v.as<double>(), xe.as<double>(), ve.as<double>(),
                                a.as<double>(), h, L, stream);
            break;
        case INTEGRATOR_EULER_CROMER:
            GS_TRY(force(a.as<double>()));
            launch_comp_update(v.as<double>(), ve.as<double>(), a.as<double>(), h, 1.0, L, stream);
            launch_comp_update(x.as<double>(), xe.as<double>(), v.as<double>(), h, 1.0, L, stream);
            break;
        case INTEGRATOR_RK4: {
            double *vk[4], *xk[4];
            for (int s = 0; s < 4; ++s) {
                vk[s] = rk[s].as<double>();
                xk[s] = rk[4 + s].as<double>();
            }
            GS_CUDA(cudaMemcpyAsync(x0.p, x.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
            GS_CUDA(cudaMemcpyAsync(v0.p, v.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
            const double coef[4] = {0.0, 0.5, 0.5, 1.0};
            for (int s = 0; s < 4; ++s) {
                if (s > 0)
                    launch_rk4_stage(x.as<double>(), v.as<double>(), x0.as<double>(),
                                     v0.as<double>(), xk[s - 1], vk[s - 1], coef[s], h, L, stream);
                GS_TRY(force(vk[s]));
                GS_CUDA(cudaMemcpyAsync(xk[s], v.p, bytes3(), cudaMemcpyDeviceToDevice, stream));
            }
            const double *cx[4] = {xk[0], xk[1], xk[2], xk[3]};
            const double *cv[4] = {vk[0], vk[1], vk[2], vk[3]};
            launch_rk4_final(x.as<double>(), v.as<double>(), x0.as<double>(), v0.as<double>(),
                             xe.as<double>(), ve.as<double>(), cx, cv, h, L, stream);
            GS_CUDA(cudaMemcpyAsync(a.p, vk[3], bytes3(), cudaMemcpyDeviceToDevice, stream));
            break;
        }
        case INTEGRATOR_LEAPFROG:
            launch_comp_update(x.as<double>(), xe.as<double>(), v.as<double>(), h, 1.0, L, stream);
            GS_TRY(force(a.as<double>()));
            launch_comp_update(v.as<double>(), ve.as<double>(), a.as<double>(), h, 1.0, L, stream);
            break;
        default:
            return GS_RAISE(GRAV_NOT_IMPLEMENTED_ERROR, "integrator %d is not built", integrator);
        }
        GS_CUDA(cudaGetLastError());
        last_dt = h;
        return ok();
    }

    int kernels_per_step() const
    {
        const int f = engine->kernels_per_eval();
        switch (integrator) {
        case INTEGRATOR_EULER: return f + 1;
        case INTEGRATOR_EULER_CROMER: return f + 2;
        case INTEGRATOR_RK4: return 4 * f + 4;
        case INTEGRATOR_LEAPFROG: return f + 2;
        default: return f;
        }
    }

    // One step through the CUDA graph when possible.
    ErrorStatus step_graph(double h)
    {
        if (timer.enabled || graph_failed || !engine->capturable()) return step(h);
        if (!graph || graph_dt != h) {
            if (graph) {
                cudaGraphExecDestroy(graph);
                graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            GS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            ErrorStatus st = step(h);
            cudaError_t e = cudaStreamEndCapture(stream, &g);
            if (st.return_code != GRAV_SUCCESS) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (e != cudaSuccess || !g) {
                (void)cudaGetLastError();
                graph_failed = true;
                return step(h);
            }
            e = cudaGraphInstantiate(&graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                graph = nullptr;
                graph_failed = true;
                return step(h);
            }
            graph_dt = h;
        }
        GS_CUDA(cudaGraphLaunch(graph, stream));
        last_dt = h;
        return ok();
    }
};

namespace gs {

ErrorStatus sim_create(gsgpu_sim **out, int n, double G, const AccelerationParam *param,
                       int integrator, double dt, cudaStream_t stream)
{
    if (!out) return GS_RAISE(GRAV_POINTER_ERROR, "output pointer is NULL");
    if (!param) return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration parameter pointer is NULL");
    if (n <= 0) return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles must be positive. Got: %d", n);
    if (n > kMaxParticles)
        return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles exceeds %d. Got: %d", kMaxParticles, n);
    if (!(dt > 0.0)) return GS_RAISE(GRAV_VALUE_ERROR, "dt must be positive. Got: %g", dt);
    const DeviceInfo *d = nullptr;
    GS_TRY(device_info(&d));
    std::unique_ptr<gsgpu_sim> s(new gsgpu_sim());
    s->n = n;
    s->G = G;
    s->p = *param;
    GS_TRY(finalize_acceleration_param(&s->p));
    s->integrator = integrator;
    s->dt = dt;
    if (stream) {
        s->stream = stream;
    } else {
        GS_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    const size_t b3 = s->bytes3();
    GS_TRY(s->x.reserve(b3));
    GS_TRY(s->v.reserve(b3));
    GS_TRY(s->a.reserve(b3));
    GS_TRY(s->xe.reserve(b3));
    GS_TRY(s->ve.reserve(b3));
    GS_TRY(s->tmp.reserve(b3));
    GS_TRY(s->m.reserve((size_t)n * sizeof(double)));
    if (integrator == INTEGRATOR_RK4) {
        GS_TRY(s->x0.reserve(b3));
        GS_TRY(s->v0.reserve(b3));
        for (int k = 0; k < 8; ++k) GS_TRY(s->rk[k].reserve(b3));
    } else if (integrator == INTEGRATOR_IAS15) {
        DBuf *b7[] = {&s->i_b0, &s->i_b, &s->i_g, &s->i_e};
        for (DBuf *b : b7) GS_TRY(b->reserve(7 * b3));
        GS_TRY(s->i_F.reserve(8 * b3));
        DBuf *b1[] = {&s->i_a1, &s->i_d7, &s->e_x1, &s->e_v1, &s->e_txe, &s->e_tve};
        for (DBuf *b : b1) GS_TRY(b->reserve(b3));
        GS_TRY(s->i_max.reserve(2 * sizeof(unsigned long long)));
        GS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&s->h_max), 2 * sizeof(unsigned long long),
                              cudaHostAllocDefault));
    } else if (const RkTableau *T = rk_tableau(integrator)) {
        GS_TRY(s->e_vk.reserve(b3 * T->stages));
        GS_TRY(s->e_xk.reserve(b3 * T->stages));
        DBuf *bufs[] = {&s->e_x1, &s->e_v1, &s->e_txe, &s->e_tve, &s->e_xs};
        for (DBuf *b : bufs) GS_TRY(b->reserve(b3));
        GS_TRY(s->e_terms.reserve(2 * b3));
        GS_TRY(s->e_esum.reserve(kErrorSumScratch * sizeof(double)));
        GS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&s->h_terms), 2 * b3,
                              cudaHostAllocDefault));
    } else if (integrator != INTEGRATOR_EULER && integrator != INTEGRATOR_EULER_CROMER &&
               integrator != INTEGRATOR_LEAPFROG) {
        return GS_RAISE(GRAV_NOT_IMPLEMENTED_ERROR,
                        "integrator %d has no GPU implementation in this library", integrator);
    }
    GS_TRY(make_engine(s->p.method, s->engine));
    GS_TRY(s->engine->setup(n, G, s->p));
    *out = s.release();
    return ok();
}

ErrorStatus sim_upload(gsgpu_sim *s, const double *x, const double *v, const double *m)
{
    if (!s || !x || !v || !m) return GS_RAISE(GRAV_POINTER_ERROR, "NULL argument");
    const Frame f = bbox_centre(s->n, x);
    s->engine->set_frame_centre(f.c[0], f.c[1], f.c[2]);
    GS_CUDA(cudaMemcpyAsync(s->x.p, x, s->bytes3(), cudaMemcpyHostToDevice, s->stream));
    GS_CUDA(cudaMemcpyAsync(s->v.p, v, s->bytes3(), cudaMemcpyHostToDevice, s->stream));
    GS_CUDA(cudaMemcpyAsync(s->m.p, m, (size_t)s->n * sizeof(double), cudaMemcpyHostToDevice,
                            s->stream));
    GS_CUDA(cudaMemsetAsync(s->xe.p, 0, s->bytes3(), s->stream));
    GS_CUDA(cudaMemsetAsync(s->ve.p, 0, s->bytes3(), s->stream));
    GS_CUDA(cudaMemsetAsync(s->a.p, 0, s->bytes3(), s->stream));
    s->primed = false;
    s->last_dt = s->dt;
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return ok();
}

ErrorStatus sim_download(gsgpu_sim *s, double *x, double *v)
{
    if (!s) return GS_RAISE(GRAV_POINTER_ERROR, "NULL simulation");
    if (x)
        GS_CUDA(cudaMemcpyAsync(x, s->x.p, s->bytes3(), cudaMemcpyDeviceToHost, s->stream));
    if (v) {
        if (s->integrator == INTEGRATOR_LEAPFROG && s->primed) {
            // v_1 from v_{1+1/2} without touching the state (src/integrator.c:1088-1094)
            GS_CUDA(cudaMemcpyAsync(s->tmp.p, s->v.p, s->bytes3(), cudaMemcpyDeviceToDevice,
                                    s->stream));
            launch_plain_kick(s->tmp.as<double>(), s->a.as<double>(), 0.5, s->last_dt, s->len(),
                              s->stream);
            GS_CUDA(cudaGetLastError());
            GS_CUDA(cudaMemcpyAsync(v, s->tmp.p, s->bytes3(), cudaMemcpyDeviceToHost, s->stream));
        } else {
            GS_CUDA(cudaMemcpyAsync(v, s->v.p, s->bytes3(), cudaMemcpyDeviceToHost, s->stream));
        }
    }
    GS_CUDA(cudaStreamSynchronize(s->stream));
    GS_TRY(s->engine->check_status(s->stream));
    return ok();
}

// Run the reference's step loop for time tf with an is_exit check per step.
ErrorStatus sim_run_until(gsgpu_sim *s, double tf, SimulationStatus *status, const bool *is_exit,
                          OutputContext *out)
{
    OutputContext *oc = out && out->active() ? out : nullptr;
    if (rk_tableau(s->integrator)) return s->rk_emb_run(tf, status, is_exit, oc);
    if (s->integrator == INTEGRATOR_IAS15) return s->ias15_run(tf, status, is_exit, oc);
    double dt = s->dt;
    const int64_t total = (int64_t)std::ceil(tf / dt);
    GS_TRY(s->initial_snapshot(oc, status));
    GS_TRY(s->prime());
    double t = 0.0;
    int64_t steps = 0;
    if (status) {
        status->t = 0.0;
        status->dt = dt;
        status->num_steps = 0;
    }
    const bool clamp = s->integrator != INTEGRATOR_RK4;
    while (steps < total) {
        if (clamp && t + dt > tf) dt = tf - t;
        if (status) status->dt = dt;
        GS_TRY(s->step_graph(dt));
        ++steps;
        t = (double)steps * dt;
        if (oc && oc->due(t)) {
            // A force that failed on the device (node-capacity overflow, a
            // wait that ran out) is reported before its state reaches a file.
            GS_CUDA(cudaStreamSynchronize(s->stream));
            GS_TRY(s->engine->check_status(s->stream));
            // leapfrog writes v at integer time, v - 0.5 a dt (src/integrator.c:1043-1071)
            const double *dv = s->v.as<double>();
            if (s->integrator == INTEGRATOR_LEAPFROG) {
                GS_CUDA(cudaMemcpyAsync(s->tmp.p, s->v.p, s->bytes3(), cudaMemcpyDeviceToDevice,
                                        s->stream));
                launch_plain_kick(s->tmp.as<double>(), s->a.as<double>(), 0.5, dt, s->len(),
                                  s->stream);
                GS_CUDA(cudaGetLastError());
                dv = s->tmp.as<double>();
            }
            GS_TRY(s->snapshot(oc, dv, t, dt));
        }
        if ((steps & 31) == 0) {
            GS_CUDA(cudaStreamSynchronize(s->stream));
            GS_TRY(s->engine->check_status(s->stream));
        }
        if (is_exit && *is_exit) break;
    }
    if (status) {
        status->t = t;
        status->num_steps = steps;
    }
    GS_CUDA(cudaStreamSynchronize(s->stream));
    GS_TRY(s->engine->check_status(s->stream));
    if (oc) GS_TRY(oc->finish());
    return ok();
}

}  // namespace gs

// ---------------------------------------------------------------------------
extern "C" {

ErrorStatus acceleration(double *a, const System *system,
                         const AccelerationParam *acceleration_param)
{
    return gs::accel_host(a, system, acceleration_param);
}

int gsgpu_sim_create(gsgpu_sim **out, int num_particles, double G,
                     const AccelerationParam *acceleration_param, int integrator, double dt,
                     void *stream)
{
    ErrorStatus st = gs::sim_create(out, num_particles, G, acceleration_param, integrator, dt,
                                    static_cast<cudaStream_t>(stream));
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_sim_upload(gsgpu_sim *sim, const double *x, const double *v, const double *m)
{
    ErrorStatus st = gs::sim_upload(sim, x, v, m);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_sim_run(gsgpu_sim *sim, int64_t num_steps)
{
    if (!sim) return GRAV_POINTER_ERROR;
    ErrorStatus st = sim->prime();
    for (int64_t k = 0; k < num_steps && st.return_code == GRAV_SUCCESS; ++k)
        st = sim->step_graph(sim->dt);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    sim->kernels_last = sim->kernels_per_step();
    return 0;
}

int gsgpu_sim_set_tolerance(gsgpu_sim *sim, double tolerance, double initial_dt)
{
    if (!sim) return GRAV_POINTER_ERROR;
    if (!(tolerance > 0.0)) {
        ErrorStatus st = GS_RAISE(GRAV_VALUE_ERROR, "tolerance must be positive. Got: %g",
                                  tolerance);
        print_and_free_traceback(&st);
        return st.return_code;
    }
    sim->tolerance = tolerance;
    sim->initial_dt = initial_dt;
    return 0;
}

int gsgpu_sim_run_until(gsgpu_sim *sim, double tf)
{
    if (!sim) return GRAV_POINTER_ERROR;
    SimulationStatus ss{};
    ErrorStatus st = gs::sim_run_until(sim, tf, &ss, nullptr, nullptr);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_sim_download(gsgpu_sim *sim, double *x, double *v)
{
    ErrorStatus st = gs::sim_download(sim, x, v);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

const double *gsgpu_sim_device_acceleration(const gsgpu_sim *sim)
{
    return sim ? sim->a.as<double>() : nullptr;
}

int gsgpu_sim_download_acceleration(gsgpu_sim *sim, double *a)
{
    if (!sim || !a) return GRAV_POINTER_ERROR;
    if (cudaMemcpyAsync(a, sim->a.p, sim->bytes3(), cudaMemcpyDeviceToHost, sim->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(sim->stream) != cudaSuccess) {
        ErrorStatus st = GS_RAISE(GRAV_FAILURE, "acceleration download failed: %s",
                                  cudaGetErrorString(cudaGetLastError()));
        print_and_free_traceback(&st);
        return GRAV_FAILURE;
    }
    return 0;
}

int gsgpu_sim_set_force_timing(gsgpu_sim *sim, int enable)
{
    if (!sim) return GRAV_POINTER_ERROR;
    for (gs::ForceTimer *t : {&sim->timer, &sim->t_morton, &sim->t_sort}) {
        t->enabled = enable != 0;
        t->total_ms = 0.0;
        t->launches = 0;
        t->used = 0;
    }
    sim->engine->set_build_timers(enable ? &sim->t_morton : nullptr, enable ? &sim->t_sort : nullptr);
    return 0;
}

int gsgpu_sim_build_timing(const gsgpu_sim *sim, double *morton_ms, double *sort_ms,
                           int64_t *builds)
{
    if (!sim) return GRAV_POINTER_ERROR;
    gsgpu_sim *s = const_cast<gsgpu_sim *>(sim);
    ErrorStatus st = s->t_morton.collect();
    if (st.return_code == GRAV_SUCCESS) st = s->t_sort.collect();
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    if (morton_ms) *morton_ms = s->t_morton.total_ms;
    if (sort_ms) *sort_ms = s->t_sort.total_ms;
    if (builds) *builds = s->t_sort.launches;
    return 0;
}

int gsgpu_sim_force_timing(const gsgpu_sim *sim, double *total_ms, int64_t *launches)
{
    if (!sim) return GRAV_POINTER_ERROR;
    gsgpu_sim *s = const_cast<gsgpu_sim *>(sim);
    ErrorStatus st = s->timer.collect();
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    if (total_ms) *total_ms = s->timer.total_ms;
    if (launches) *launches = s->timer.launches;
    return 0;
}

int gsgpu_sim_kernels_per_step(const gsgpu_sim *sim)
{
    return sim ? sim->kernels_per_step() : 0;
}

int gsgpu_sim_interaction_counts(gsgpu_sim *sim, long long *counts)
{
    if (!sim || !counts) return GRAV_POINTER_ERROR;
    ErrorStatus st = sim->engine->interaction_counts(sim->stream, counts);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_sim_warmup_until_ready(gsgpu_sim *sim, int64_t max_steps, int64_t *steps_taken)
{
    if (!sim) return GRAV_POINTER_ERROR;
    ErrorStatus st = sim->prime();
    int64_t k = 0;
    while (st.return_code == GRAV_SUCCESS && !sim->engine->ready() && k < max_steps) {
        st = sim->step(sim->dt);
        ++k;
    }
    if (st.return_code == GRAV_SUCCESS && cudaStreamSynchronize(sim->stream) != cudaSuccess)
        st = GS_RAISE(GRAV_FAILURE, "stream synchronisation failed");
    if (steps_taken) *steps_taken = k;
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return sim->engine->ready() ? 0 : GRAV_FAILURE;
}

int gsgpu_sim_training_samples(gsgpu_sim *sim, int snapshot, float *features, float *targets,
                               int count)
{
    if (!sim) return -GRAV_POINTER_ERROR;
    cudaStreamSynchronize(sim->stream);
    return sim->engine->dataset(snapshot, features, targets, count);
}

int gsgpu_set_rk_error_sum(int mode)
{
    if (mode != 0 && mode != 1) return GRAV_VALUE_ERROR;
    gs::g_rk_error_sum.store(mode, std::memory_order_relaxed);
    return 0;
}

int gsgpu_sim_set_learned_policy(gsgpu_sim *sim, int policy)
{
    if (!sim) return GRAV_POINTER_ERROR;
    cudaStreamSynchronize(sim->stream);
    if (!sim->engine->set_learned_policy(policy)) return GRAV_VALUE_ERROR;
    if (sim->graph) {   // the captured step holds the previous policy's launches
        cudaGraphExecDestroy(sim->graph);
        sim->graph = nullptr;
    }
    return 0;
}

int gsgpu_sim_report(gsgpu_sim *sim, double *out, int nmax)
{
    if (!sim || !out) return -GRAV_POINTER_ERROR;
    cudaStreamSynchronize(sim->stream);
    return sim->engine->report(out, nmax);
}

int gsgpu_last_interaction_counts(long long *counts)
{
    if (!counts) return GRAV_POINTER_ERROR;
    counts[0] = counts[1] = 0;
    if (!gs::tl_call || !gs::tl_call->engine) return 0;
    ErrorStatus st = gs::tl_call->engine->interaction_counts(gs::tl_call->stream, counts);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

void gsgpu_sim_destroy(gsgpu_sim *sim) { delete sim; }

// src/grav_sim.c:61-138
ErrorStatus launch_simulation(System *system, IntegratorParam *integrator_param,
                              AccelerationParam *acceleration_param, OutputParam *output_param,
                              SimulationStatus *simulation_status, Settings *settings, double tf)
{
    // finalize_system (src/system.c:70-111)
    if (!system) return GS_RAISE(GRAV_POINTER_ERROR, "System is NULL");
    if (system->num_particles <= 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles must be positive. Got: %d",
                        system->num_particles);
    if (!system->particle_ids)
        return GS_RAISE(GRAV_POINTER_ERROR, "System array particle_ids is NULL");
    if (!system->x) return GS_RAISE(GRAV_POINTER_ERROR, "System array x is NULL");
    if (!system->v) return GS_RAISE(GRAV_POINTER_ERROR, "System array v is NULL");
    if (!system->m) return GS_RAISE(GRAV_POINTER_ERROR, "System array m is NULL");
    if (system->G <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Gravitational constant G must be positive. Got: %g",
                        system->G);
    if (!acceleration_param)
        return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration parameter pointer is NULL");
    GS_TRY(finalize_acceleration_param(acceleration_param));
    // finalize_integration_param (src/integrator.c:131-189)
    if (!integrator_param) return GS_RAISE(GRAV_POINTER_ERROR, "integration_param is NULL");
    const int integ = integrator_param->integrator;
    if (integ < INTEGRATOR_EULER || integ > INTEGRATOR_WHFAST)
        return GS_RAISE(GRAV_VALUE_ERROR, "Unknown integrator. Got: %d", integ);
    const bool fixed = integ == INTEGRATOR_EULER || integ == INTEGRATOR_EULER_CROMER ||
                       integ == INTEGRATOR_RK4 || integ == INTEGRATOR_LEAPFROG ||
                       integ == INTEGRATOR_WHFAST;
    if (fixed && integrator_param->dt <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "dt must be positive. Got: %g", integrator_param->dt);
    if (!fixed && integrator_param->tolerance <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "tolerance must be positive. Got: %g",
                        integrator_param->tolerance);
    // finalize_output_param (src/output.c:126-239)
    if (!settings) return GS_RAISE(GRAV_POINTER_ERROR, "settings is NULL");
    GS_TRY(output_prepare(output_param, settings));
    if (tf < 0.0) return GS_RAISE(GRAV_VALUE_ERROR, "tf must be non-negative. Got: %g", tf);
    if (!simulation_status) return GS_RAISE(GRAV_POINTER_ERROR, "simulation_status is NULL");
    OutputContext oc;
    oc.op = output_param;
    oc.system = system;


    if (integ == INTEGRATOR_WHFAST) {
        // src/integrator_whfast.c:200-407 as a one-system ensemble; the
        // arrays are permuted (sort by distance) and compacted (removals) in
        // place, num_particles shrinking like the reference's.
        const int n0 = system->num_particles;
        gsgpu_ensemble *raw = nullptr;
        GS_TRY(gs::ensemble_create(&raw, 1, &n0, system->G, integ, acceleration_param->method,
                                   acceleration_param->softening_length, integrator_param->dt,
                                   integrator_param->whfast_remove_invalid_particles ? 1 : 0,
                                   nullptr));
        std::unique_ptr<gsgpu_ensemble, void (*)(gsgpu_ensemble *)> ens(raw, gs::ensemble_destroy);
        GS_TRY(gs::ensemble_upload(ens.get(), system->particle_ids, system->x, system->v,
                                   system->m));
        if (settings->verbose >= 1) std::fputs("Launching simulation...\n", stdout);
        GS_TRY(gs::ensemble_run_until(ens.get(), tf, simulation_status, settings->is_exit_ptr,
                                      &oc));
        int n1 = n0;
        GS_TRY(gs::ensemble_download(ens.get(), &n1, system->particle_ids, system->x, system->v,
                                     system->m));
        system->num_particles = n1;
        return ok();
    }

    if (settings->verbose >= 2) {   // GRAV_VERBOSITY_NORMAL (src/grav_sim.c:111-121)
        print_compilation_info();
        const DeviceInfo *d = nullptr;
        GS_TRY(device_info(&d));
        std::printf("grav_sim GB300 library: %s (%d SMs), method %d, integrator %d, N = %d\n",
                    d->name, d->sm_count, acceleration_param->method, integ,
                    system->num_particles);
    }
    if (settings->verbose >= 1) std::fputs("Launching simulation...\n", stdout);

    gsgpu_sim *raw = nullptr;
    // adaptive integrators carry no fixed dt: the creation dt is a placeholder
    GS_TRY(gs::sim_create(&raw, system->num_particles, system->G, acceleration_param, integ,
                          fixed ? integrator_param->dt : 1.0, nullptr));
    std::unique_ptr<gsgpu_sim> sim(raw);
    sim->tolerance = integrator_param->tolerance;
    sim->initial_dt = integrator_param->initial_dt;
    if (integ == INTEGRATOR_EULER || integ == INTEGRATOR_EULER_CROMER || integ == INTEGRATOR_RK4 ||
        integ == INTEGRATOR_LEAPFROG) {
        // force evaluations of this run: ceil(tf / dt) steps (the last one
        // clamped), four per RK4 step, one more for leapfrog's initial force
        const double steps = std::ceil(tf / integrator_param->dt);
        if (steps >= 0.0 && steps < 1e15)
            sim->engine->set_evaluation_budget((long long)steps * (integ == INTEGRATOR_RK4 ? 4 : 1) +
                                               (integ == INTEGRATOR_LEAPFROG ? 1 : 0));
    }
    GS_TRY(gs::sim_upload(sim.get(), system->x, system->v, system->m));
    GS_TRY(gs::sim_run_until(sim.get(), tf, simulation_status, settings->is_exit_ptr, &oc));
    GS_TRY(gs::sim_download(sim.get(), system->x, system->v));
    return ok();
}

// src/python_interface.c:94-193
int launch_simulation_python(int32_t *num_particles, int32_t *particle_ids, double *x, double *v,
                             double *m, int32_t **new_particle_ids_ptr, double **new_x_ptr,
                             double **new_v_ptr, double **new_m_ptr, double G, int32_t integrator,
                             double dt, double tolerance, double initial_dt,
                             bool whfast_remove_invalid_particles, int32_t acceleration_method,
                             double opening_angle, double softening_length,
                             int32_t max_num_particles_per_leaf, int32_t output_method,
                             char *output_dir, bool output_initial, double output_interval,
                             int32_t coordinate_output_dtype, int32_t velocity_output_dtype,
                             int32_t mass_output_dtype, int32_t verbose, bool enable_progress_bar,
                             bool *is_exit_ptr, double tf)
{
    System system = get_new_system();
    system.num_particles = num_particles ? *num_particles : 0;
    system.particle_ids = particle_ids;
    system.x = x;
    system.v = v;
    system.m = m;
    system.G = G;

    AccelerationParam ap = get_new_acceleration_param();
    ap.method = acceleration_method;
    ap.opening_angle = opening_angle;
    ap.softening_length = softening_length;
    ap.max_num_particles_per_leaf = max_num_particles_per_leaf;

    IntegratorParam ip = get_new_integrator_param();
    ip.integrator = integrator;
    ip.dt = dt;
    ip.tolerance = tolerance;
    ip.initial_dt = initial_dt;
    ip.whfast_remove_invalid_particles = whfast_remove_invalid_particles;

    OutputParam op = get_new_output_param();
    op.method = output_method;
    op.output_dir = output_dir;
    op.output_interval = output_interval;
    op.output_initial = output_initial;
    op.coordinate_output_dtype = coordinate_output_dtype;
    op.velocity_output_dtype = velocity_output_dtype;
    op.mass_output_dtype = mass_output_dtype;

    SimulationStatus ss;
    ss.t = 0.0;
    ss.dt = dt;
    ss.num_steps = 0;

    Settings settings = get_new_settings();
    settings.verbose = verbose;
    settings.enable_progress_bar = enable_progress_bar;
    if (is_exit_ptr) settings.is_exit_ptr = is_exit_ptr;

    ErrorStatus st = launch_simulation(&system, &ip, &ap, &op, &ss, &settings, tf);
    if (st.return_code != GRAV_SUCCESS) {
        st = gs::traceback(st, "launch_simulation(&system, ...)", __FILE__, __LINE__, __func__);
        print_and_free_traceback(&st);
        return 1;
    }
    if (num_particles) *num_particles = system.num_particles;
    if (new_particle_ids_ptr) *new_particle_ids_ptr = system.particle_ids;
    if (new_x_ptr) *new_x_ptr = system.x;
    if (new_v_ptr) *new_v_ptr = system.v;
    if (new_m_ptr) *new_m_ptr = system.m;
    return 0;
}

}  // extern "C"
