// gs_internal.h -- internal declarations of libgrav_sim_gb300.
//
// Host code is C++ over the CUDA runtime; every public entry point is
// `extern "C"` in include/grav_sim_gb300.h.  Errors travel as grav_sim's
// ErrorStatus (src/error.h:31-36) with a heap traceback string; CUDA errors
// and device status words are mapped onto the GRAV_* codes.
#pragma once

#include "../../include/grav_sim_gb300.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

namespace gs {

// Bits of the device status word written by kernels (never a trap).
enum StatusBits : unsigned {
    ST_WAIT_TIMEOUT = 1u,     // an mbarrier / flag wait ran out of time
    ST_TREE_OVERFLOW = 2u,    // node capacity exceeded (GRAV_MEMORY_ERROR)
    ST_STACK_OVERFLOW = 4u,   // walk stack deeper than the octree limit
    ST_NONFINITE = 8u,        // NaN/Inf seen where the kernel checks
    ST_BAD_KEY = 16u,         // octant digit out of range while building
    ST_NO_PRIMARY = 32u,      // an ensemble system has no particle with id 0
    ST_CAPACITY = 64u,        // an ensemble system outgrew its sort capacity
};

// ---- errors ------------------------------------------------------------
ErrorStatus ok();
ErrorStatus raise_error(int code, const char *file, int line, const char *func,
                        const char *fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 5, 6)))
#endif
    ;
ErrorStatus traceback(ErrorStatus st, const char *call, const char *file,
                      int line, const char *func);
ErrorStatus cuda_error(cudaError_t e, const char *what, const char *file,
                       int line, const char *func);

#define GS_RAISE(code, ...) gs::raise_error((code), __FILE__, __LINE__, __func__, __VA_ARGS__)
#define GS_TRY(call)                                                           \
    do {                                                                       \
        ErrorStatus st_ = (call);                                              \
        if (st_.return_code != GRAV_SUCCESS)                                   \
            return gs::traceback(st_, #call, __FILE__, __LINE__, __func__);   \
    } while (0)
#define GS_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return gs::cuda_error(e_, #call, __FILE__, __LINE__, __func__);   \
    } while (0)

// Largest particle count: 3N components are indexed with int, as in the
// reference's arrays.
constexpr int kMaxParticles = 0x7fffffff / 3;

// ---- device buffers ----------------------------------------------------
// Grow-only device allocation owned by an engine or simulation.
struct DBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf();
    ErrorStatus reserve(size_t b);
    void release();
    template <class T> T *as() const { return static_cast<T *>(p); }
};

struct DeviceInfo {
    int id = 0;
    int sm_count = 0;
    int cc_major = 0;
    int cc_minor = 0;
    char name[256] = {0};
};
// Properties of the current device (queried once per device); fails when
// there is no usable GPU.
constexpr int kMaxDevices = 64;
ErrorStatus device_info(const DeviceInfo **out);

// Records CUDA events around the dominant kernel of each force evaluation.
struct ForceTimer {
    bool enabled = false;
    std::vector<cudaEvent_t> ev;   // pairs (start, stop)
    size_t used = 0;
    double total_ms = 0.0;
    int64_t launches = 0;
    ErrorStatus begin(cudaStream_t s);
    ErrorStatus end(cudaStream_t s);
    ErrorStatus collect();   // after the stream is synchronised
    ~ForceTimer();
};

// ---- force engines -----------------------------------------------------
// One engine per (method, N); it owns its scratch memory.  compute() reads
// FP64 positions and masses on the device and writes FP64 accelerations.
class Engine {
  public:
    virtual ~Engine() {}
    virtual ErrorStatus setup(int n, double G, const AccelerationParam &p) = 0;
    virtual ErrorStatus compute(const double *d_x, const double *d_m, double *d_a,
                                cudaStream_t s, ForceTimer *timer) = 0;
    // kernels launched by one compute()
    virtual int kernels_per_eval() const = 0;
    // true when compute() never synchronises with the host (graph-capturable)
    virtual bool capturable() const { return true; }
    // device status word of the engine (may be null)
    virtual ErrorStatus check_status(cudaStream_t s) { (void)s; return ok(); }
    // FP64 origin subtracted before positions are rounded to FP32
    virtual void set_frame_centre(double cx, double cy, double cz)
    {
        (void)cx; (void)cy; (void)cz;
    }
    // Barnes-Hut engines: CUDA events around the Morton-key kernel and the
    // key sort of each tree build (null: not timed).
    virtual void set_build_timers(ForceTimer *morton, ForceTimer *sort)
    {
        (void)morton;
        (void)sort;
    }
    // false while the engine is still preparing itself (collecting training
    // data): its forces are then the fallback method's
    virtual bool ready() const { return true; }
    // The run will ask for at most evals forces (a one-shot run with a fixed
    // step); an engine whose preparation could not finish within them may
    // skip it.  Not called: no limit.
    virtual void set_evaluation_budget(long long evals) { (void)evals; }
    // Learned engines: 0 follow the held-out rule, 1 always apply the
    // network (the judge still guards each step), 2 never; false elsewhere.
    virtual bool set_learned_policy(int policy)
    {
        (void)policy;
        return false;
    }
    // Engine-specific statistics; returns how many values were written.
    virtual int report(double *out, int nmax) const
    {
        (void)out;
        (void)nmax;
        return 0;
    }
    // Learned engines: training samples of one snapshot (count written).
    virtual int dataset(int snap, float *feat, float *target, int count) const
    {
        (void)snap; (void)feat; (void)target; (void)count;
        return 0;
    }
    // Interactions of the most recent compute(): out[0] cell (monopole)
    // terms, out[1] particle-particle terms.  Synchronises the stream.
    virtual ErrorStatus interaction_counts(cudaStream_t s, long long out[2])
    {
        (void)s;
        out[0] = 0;
        out[1] = 0;
        return ok();
    }
};

// Compensated-FP32 direct sum for a list of target particles against all
// sources (k_direct.cu); positions are taken relative to a device FP64
// centre d_frame[0..2].  a_rows[3r..3r+2] = acceleration of particle rows[r].
class DirectRows {
  public:
    ErrorStatus setup(int nj, int max_rows);
    ErrorStatus compute(const double *d_x, const double *d_m, const double *d_frame,
                        const int *d_rows, int nrows, double G, double eps, double *d_a_rows,
                        cudaStream_t s, ForceTimer *timer = nullptr);
    // Reports (and clears) a shared-memory tile wait that ran out.
    ErrorStatus check(cudaStream_t s);
    static constexpr int kernels() { return 4; }

  private:
    // j-split of a launch over i_tiles row tiles: the whole number of waves
    // of resident CTAs that needs the fewest tiles per CTA, with at most
    // max_splits chunks.
    void split_for(int i_tiles, int max_splits, int *splits, int *chunk) const;
    int nj_ = 0, nj_pad_ = 0, ni_pad_ = 0, jt_total_ = 0;
    long slots_ = 1;
    size_t partial_rows_ = 0;   // capacity of partial_ in (split, row) pairs
    DBuf pj_, pi_, partial_, status_;
};

bool is_gpu_method(int method);
ErrorStatus make_engine(int method, std::unique_ptr<Engine> &out);

std::unique_ptr<Engine> make_direct_engine(bool fp64_reference_order);
std::unique_ptr<Engine> make_massless_engine();
std::unique_ptr<Engine> make_barnes_hut_engine(bool compat, bool quad = false, bool group = false);
std::unique_ptr<Engine> make_learned_engine();

// ---- integrator kernels (k_integrate.cu) -------------------------------
void launch_comp_update(double *y, double *err, const double *d, double dt,
                        double factor, int len, cudaStream_t s);
void launch_euler_update(double *x, double *v, double *xe, double *ve,
                         const double *a, double dt, int len, cudaStream_t s);
void launch_plain_kick(double *v, const double *a, double coef, double dt, int len,
                       cudaStream_t s);
void launch_rk4_stage(double *x, double *v, const double *x0, const double *v0,
                      const double *xk, const double *vk, double coef, double dt,
                      int len, cudaStream_t s);
void launch_rk4_final(double *x, double *v, const double *x0, const double *v0,
                      double *xe, double *ve, const double *const *xk,
                      const double *const *vk, double dt, int len, cudaStream_t s);
void launch_rk_emb_stage(const double *x, const double *v, const double *xe, const double *ve,
                         const double *vk, double *xk, double *xs, const double *a_row,
                         int stage, double dt, int len, cudaStream_t s);
void launch_rk_emb_combine(const double *x, const double *v, const double *xe, const double *ve,
                           const double *vk, const double *xk, double *x1, double *v1,
                           double *txe, double *tve, double *terms, const double *w,
                           const double *dtdw, int stages, double dt, double abs_tol,
                           double rel_tol, int len, cudaStream_t s);
// Sum of count error terms on the device, in a fixed grouping (not the
// reference's order): scratch holds kErrorSumScratch doubles, the sum lands in
// scratch[kErrorSumScratch - 1].
constexpr int kErrorSumScratch = 257;
void launch_error_sum(const double *terms, long long count, double *scratch, cudaStream_t s);

// ---- IAS15 (k_ias15.cu) ------------------------------------------------
extern const double kIas15H[8];   // Gauss-Radau spacings
void launch_ias_predict(int L, double *x1, double *v1, const double *x0, const double *v0,
                        const double *a0, double h, const double *b, double dt, const double *xe,
                        const double *ve, cudaStream_t s);
void launch_ias_update_gb(int L, double *g, double *b, const double *F, int i, cudaStream_t s);
void launch_ias_absmax2(int L, const double *u, const double *w, unsigned long long *out,
                        cudaStream_t s);
void launch_ias_delta(int L, const double *b, double *b0, double *d7, cudaStream_t s);
void launch_ias_advance(int L, double *x1, double *v1, double *txe, double *tve, const double *x0,
                        const double *v0, const double *a0, const double *b, double dt,
                        cudaStream_t s);
void launch_ias_refine(int L, double *b, double *e, const double q[7], int refine, cudaStream_t s);
void launch_ias_axpy(int L, double *out, const double *x, double c, const double *v,
                     cudaStream_t s);
void launch_ias_sub(int L, double *out, const double *u, const double *w, cudaStream_t s);

// ---- embedded Runge-Kutta tableaus (host_rk.cpp) -------------------------
struct RkTableau {
    int stages, power, power_test;
    double a[13][12];   // a[s][i], i < s
    double b[13], b_hat[13];
};
// Integrator codes 5-8; nullptr for any other code.
const RkTableau *rk_tableau(int integrator);

// ---- diagnostics (k_diag.cu) -------------------------------------------
ErrorStatus gpu_energy(const double *h_state7, int num_snapshots, int n, double G,
                       double *h_energy);

// ---- octree (k_octree.cu) ----------------------------------------------
struct OctreeDevice;   // opaque; owned by a Barnes-Hut engine
ErrorStatus octree_to_host(const AccelerationParam &p, const System *system,
                           const double *box_center, double box_width,
                           LinearOctree *out);

// ---- particle mesh and cosmology (k_pm.cu) ------------------------------
ErrorStatus pm_acceleration_host(double *a, int n, const double *x, const double *m,
                                 const double *box_center, double box_width, double H0,
                                 double omega_m, double mean_bkg_density, int pm_grid_size,
                                 double scale_factor);
// op: snapshots as src/integrator_cosmology_leapfrog.c writes them (NULL or
// disabled for none); at each one the host x and v are updated.
ErrorStatus pm_leapfrog_cosmology(CosmologicalSystem *system, SimulationStatus *status,
                                  OutputParam *op, const bool *is_exit, double dt, double a_begin,
                                  double a_final, int pm_grid_size);
// Device time of the step loop of this thread's last cosmological run.
ErrorStatus pm_last_timing(double *loop_ms, int64_t *steps);

// ---- snapshots (host_output.cpp) ----------------------------------------
ErrorStatus output_prepare(OutputParam *op, const Settings *settings);
// Write snapshot number op->output_count_ from host arrays and count it.
ErrorStatus output_snapshot(OutputParam *op, int n, const int *ids, const double *x,
                            const double *v, const double *m, double G, double t, double dt);
// The header values a cosmological snapshot adds (src/output.c:697-900).
struct CosmologyHeader {
    double omega_m, omega_lambda, unit_length, unit_mass, unit_time;
};
ErrorStatus write_snapshot_hdf5(const char *path, int n, const int *ids, const double *x,
                                const double *v, const double *m, double t, bool x_float,
                                bool v_float, bool m_float, const CosmologyHeader *cosmo);
// src/output.c:294-345: a cosmological snapshot of the host arrays (HDF5
// only), numbered and counted like output_snapshot.
ErrorStatus output_snapshot_cosmology(OutputParam *op, const CosmologicalSystem *system,
                                      double t);

class SnapshotWriter;

// Snapshots during a launch_simulation run.  A snapshot taken inside the
// step loop is copied device->host on the run's stream into pinned memory
// and written to its file by a writer thread, so the loop does not wait for
// the file system; the file number is fixed when the snapshot is taken.
struct OutputContext {
    OutputParam *op = nullptr;
    const System *system = nullptr;   // host ids and masses, G
    double next_time = 0.0;           // the reference's next_output_time
    std::unique_ptr<SnapshotWriter> writer;

    OutputContext();
    ~OutputContext();   // waits for the writer
    bool active() const
    {
        return op && (op->method == OUTPUT_METHOD_CSV || op->method == OUTPUT_METHOD_HDF5);
    }
    // Start of a run: the first snapshot after the initial one is due at
    // one output interval (src/integrator.c:300-303).
    void begin() { next_time = op->output_interval; }
    bool initial() const { return op->output_initial; }
    bool due(double t) const { return t >= next_time; }
    // Take a snapshot of n particles at time t after a step of dt: x and v
    // from the device; ids and masses from the device when d_ids / d_m are
    // given (n then counts the slots copied and *d_cnt the particles
    // written), else the host system's.  Moves the next output time to
    // output_count * interval as the reference does after each snapshot.
    ErrorStatus take(int n, const double *d_x, const double *d_v, const int *d_ids,
                     const double *d_m, const int *d_cnt, cudaStream_t s, double t, double dt);
    // Wait until every snapshot taken is on disk; the first write error.
    ErrorStatus finish();
};

}  // namespace gs

// ---- batched ensembles (k_whfast.cu) -----------------------------------
struct gsgpu_ensemble;
namespace gs {
ErrorStatus ensemble_create(gsgpu_ensemble **out, int num_systems, const int *counts, double G,
                            int integrator, int method, double eps, double dt,
                            int remove_invalid, cudaStream_t stream);
ErrorStatus ensemble_upload(gsgpu_ensemble *e, const int *ids, const double *x, const double *v,
                            const double *m);
ErrorStatus ensemble_run_until(gsgpu_ensemble *e, double tf, SimulationStatus *status,
                               const bool *is_exit, OutputContext *out = nullptr);
ErrorStatus ensemble_download(gsgpu_ensemble *e, int *counts, int *ids, double *x, double *v,
                              double *m);
void ensemble_destroy(gsgpu_ensemble *e);
}  // namespace gs
