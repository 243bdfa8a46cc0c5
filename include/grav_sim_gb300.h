/*
 * grav_sim_gb300.h -- C ABI of the GB300-native force-evaluation library.
 *
 * libgrav_sim_gb300.so is a drop-in for grav_sim's libgrav_sim on the
 * force-evaluation hot path.  Struct layouts and entry points below are the
 * ones grav_sim declares (each cites the declaration it replaces); the GPU
 * path is selected through the existing AccelerationParam.method field with
 * the GRAV_GPU_* codes.  The reference's CPU codes (1-3) are rejected with
 * GRAV_VALUE_ERROR: this library has no CPU fallback.
 *
 * All signatures use plain C types and pointers.  Host pointers are host
 * memory; entry points named gsgpu_* take device pointers where stated.
 */
#ifndef GRAV_SIM_GB300_H
#define GRAV_SIM_GB300_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error handling (src/error.h:14-36) ---------------------------- */
#define GRAV_UNKNOWN_ERROR -1
#define GRAV_SUCCESS 0
#define GRAV_FAILURE 1
#define GRAV_VALUE_ERROR 2
#define GRAV_POINTER_ERROR 3
#define GRAV_MEMORY_ERROR 4
#define GRAV_OS_ERROR 5
#define GRAV_NOT_IMPLEMENTED_ERROR 6

typedef struct ErrorStatus {
    int return_code;
    char *traceback;
    int traceback_code_;
} ErrorStatus;

/* src/error.h:105 */
ErrorStatus make_success_error_status(void);
/* src/error.h:195 */
void free_traceback(ErrorStatus *error_status);
/* src/error.h:202 */
void print_and_free_traceback(ErrorStatus *error_status);
/* src/error.h:105-127 (behind WRAP_RAISE_WARNING / WRAP_RAISE_WARNING_FMT) */
void raise_warning(const char *warning_file, const int warning_line, const char *warning_func,
                   const char *warning_msg);
ErrorStatus raise_warning_fmt(const char *warning_file, const int warning_line,
                              const char *warning_func, const char *format, ...);
/* src/error.h:146-172 (behind WRAP_RAISE_ERROR / WRAP_RAISE_ERROR_FMT) */
ErrorStatus raise_error(const char *error_file, const int error_line, const char *error_func,
                        const int error_code, const char *error_msg);
ErrorStatus raise_error_fmt(const char *error_file, const int error_line, const char *error_func,
                            const int error_code, const char *format, ...);
/* src/error.h:186-192 (behind WRAP_TRACEBACK): prepends the caller's frame
 * to the traceback of a failed status; a success passes through. */
ErrorStatus traceback(ErrorStatus error_status, const char *function_call_source_code,
                      const char *error_file, const int error_line, const char *error_func);

/* ---- system / parameters (src/system.h:12-20, src/acceleration.h:16-26,
 *      src/common.h:29-56, src/settings.h:11-16) --------------------- */
typedef struct System {
    int num_particles;
    int *particle_ids;
    double *x;
    double *v;
    double *m;
    double G;
} System;

#define ACCELERATION_METHOD_PAIRWISE 1
#define ACCELERATION_METHOD_MASSLESS 2
#define ACCELERATION_METHOD_BARNES_HUT 3

/* GPU method codes (new; same AccelerationParam.method field). */
#define GRAV_GPU_PAIRWISE 101           /* compensated-FP32 direct sum */
#define GRAV_GPU_MASSLESS 102           /* FP64 massive/massless direct sum */
#define GRAV_GPU_BARNES_HUT 103         /* FP32 walk, true leaf multipoles */
#define GRAV_GPU_BH_LEARNED 104         /* theta-cheap walk + learned residual */
#define GRAV_GPU_BARNES_HUT_QUAD 105    /* FP32 walk, monopole + quadrupole cells */
#define GRAV_GPU_BARNES_HUT_GROUP 106   /* group walk, interaction lists, quadrupoles */
#define GRAV_GPU_BARNES_HUT_GROUP_MONO 107  /* group walk, monopole cells only */
#define GRAV_GPU_PAIRWISE_FP64 111      /* FP64 direct sum, reference order */
#define GRAV_GPU_BARNES_HUT_COMPAT 113  /* FP32 walk, reference tree quirks */

typedef struct AccelerationParam {
    int method;
    double opening_angle;
    double softening_length;
    int max_num_particles_per_leaf;
} AccelerationParam;

typedef struct IntegratorParam {
    int integrator;
    double dt;
    double tolerance;
    double initial_dt;
    bool whfast_remove_invalid_particles;
} IntegratorParam;

#define INTEGRATOR_EULER 1
#define INTEGRATOR_EULER_CROMER 2
#define INTEGRATOR_RK4 3
#define INTEGRATOR_LEAPFROG 4
#define INTEGRATOR_RKF45 5
#define INTEGRATOR_DOPRI 6
#define INTEGRATOR_DVERK 7
#define INTEGRATOR_RKF78 8
#define INTEGRATOR_IAS15 9
#define INTEGRATOR_WHFAST 10

typedef struct OutputParam {
    int method;
    char *output_dir;
    bool output_initial;
    double output_interval;
    int coordinate_output_dtype;
    int velocity_output_dtype;
    int mass_output_dtype;
    int output_count_;
} OutputParam;

#define OUTPUT_METHOD_DISABLED 1
#define OUTPUT_METHOD_CSV 2
#define OUTPUT_METHOD_HDF5 3
/* src/output.h:18-19 */
#define OUTPUT_DTYPE_FLOAT 1
#define OUTPUT_DTYPE_DOUBLE 2

typedef struct SimulationStatus {
    double t;
    double dt;
    int64_t num_steps;
} SimulationStatus;

typedef struct Settings {
    int verbose;
    bool enable_progress_bar;
    bool *is_exit_ptr;
} Settings;

/* src/system.h:28 */
System get_new_system(void);
/* An HDF5 snapshot in the layout of grav_sim's output method 3
 * (src/output.c:483-695): /Header attributes NumFilesPerSnapshot,
 * NumPart_ThisFile, NumPart_Total and Time, /PartType0 datasets ParticleIDs,
 * Masses, Coordinates and Velocities in the given output dtypes
 * (OUTPUT_DTYPE_FLOAT or _DOUBLE).  Written without libhdf5.  Returns a
 * GRAV_* code. */
int gsgpu_write_snapshot_hdf5(const char *path, int num_particles, const int *ids,
                              const double *x, const double *v, const double *m, double t,
                              int coordinate_output_dtype, int velocity_output_dtype,
                              int mass_output_dtype);
/* The values of a dataset (attribute NULL) or of an attribute of the object
 * at the path `object` ("/PartType0/Masses", "/Header") of an HDF5 file, as
 * doubles.  *count receives the number of values; out (capacity values) may
 * be NULL to ask for the count only.  Returns a GRAV_* code. */
int gsgpu_hdf5_read(const char *path, const char *object, const char *attribute, double *out,
                    long long capacity, long long *count);

/* src/system.h:55-58: arrays of num_particles (ids 0..n-1, x, v, m zeroed)
 * allocated with malloc; release with free_system. */
ErrorStatus get_initialized_system(System *system, const int num_particles);
/* src/system.h:125 */
void free_system(System *system);

/* Gadget-2 initial conditions from an HDF5 file, as grav_sim's galaxy-collision
 * example reads them through libhdf5 (examples/galaxy_collision/c/
 * galaxy_collision.c:109-293): particles of PartType1 then PartType2 (Masses,
 * Coordinates, Velocities), ids 0..n-1, and the three unit attributes of
 * /Units.  The file is parsed directly (no libhdf5); the arrays are allocated
 * with malloc and released by free_system.  G is left to the caller. */
ErrorStatus load_gadget2_ic(const char *path, System *system, double *unit_length,
                            double *unit_mass, double *unit_time);
/* src/acceleration.h:33 */
AccelerationParam get_new_acceleration_param(void);
/* src/acceleration.h:40-42 */
ErrorStatus finalize_acceleration_param(AccelerationParam *acceleration_param);
/* src/integrator.h (get_new_integrator_param, integrator.c:119-129) */
IntegratorParam get_new_integrator_param(void);
/* src/output.h (get_new_output_param) */
OutputParam get_new_output_param(void);
/* src/settings.h:23 */
Settings get_new_settings(void);

/* ---- utilities (src/utils.h:19-48, pcg/pcg_basic.h:58) -------------- */
/* PCG32 generator state (the layout of pcg_basic.h's pcg32_random_t). */
typedef struct pcg_state_setseq_64 {
    uint64_t state;
    uint64_t inc;
} pcg32_random_t;
/* src/utils.h:19: CLOCK_MONOTONIC seconds. */
double grav_get_current_time(void);
/* src/utils.h:35: a PCG32 generator seeded from the clock. */
pcg32_random_t init_pcg_rng(void);
/* src/utils.h:44-48: uniform in [min, max) from one 32-bit PCG32 draw. */
double grav_randrange(const double min, const double max, pcg32_random_t *rng);

/* ---- acceleration (src/acceleration.h:53-70) ----------------------- */

/* src/acceleration.h:53-57.  a: host array [3N]; system->x, ->m host.  The
 * GPU method in acceleration_param->method computes a on the GPU. */
ErrorStatus acceleration(double *a, const System *system,
                         const AccelerationParam *acceleration_param);

/* src/acceleration.h:66-70.  GPU Barnes-Hut: GRAV_GPU_BARNES_HUT_COMPAT
 * when acceleration_param->method is the reference's BARNES_HUT code or
 * GRAV_GPU_BARNES_HUT_COMPAT, else GRAV_GPU_BARNES_HUT. */
ErrorStatus acceleration_barnes_hut(double *a, const System *system,
                                    const AccelerationParam *acceleration_param);

/* src/acceleration.h:98-103 (src/acceleration.c:369-506): runs
 * acceleration() num_times_acceleration_param[i] times for each parameter
 * set, timing each call with CLOCK_MONOTONIC, and prints per set the mean
 * and sample standard deviation of the run times and the mean absolute
 * error (three components summed, divided by N) of its first call against
 * the first call of set 0.  Accepts the GPU method codes. */
ErrorStatus benchmark_acceleration(const System *system,
                                   const AccelerationParam *acceleration_params,
                                   const int num_acceleration_params,
                                   const int *num_times_acceleration_param);

/* ---- linear octree (src/linear_octree.h:14-101) -------------------- */
#define MORTON_MAX_LEVEL 21

typedef struct LinearOctree {
    double box_width;
    int num_internal_nodes;
    int64_t *particle_morton_indices_deepest_level;
    int *sorted_indices;
    int *tree_num_particles;
    int *tree_num_internal_children;
    int *tree_first_particle_sorted_idx;
    int *tree_first_internal_children_idx;
    double *tree_mass;
    double *tree_center_of_mass_x;
    double *tree_center_of_mass_y;
    double *tree_center_of_mass_z;
} LinearOctree;

/* src/linear_octree.h:64 */
LinearOctree get_new_linear_octree(void);
/* src/linear_octree.h:75-81.  Built on the GPU (bounding box, Morton keys,
 * radix sort, tree, multipoles) and copied into host arrays that
 * free_linear_octree releases.  Node numbering, keys, order and internal
 * node mass / centre of mass are those of the reference. */
ErrorStatus construct_octree(LinearOctree *octree, const System *system,
                             const AccelerationParam *acceleration_param,
                             const double *box_center, double box_width);
/* src/linear_octree.h:88 */
void free_linear_octree(LinearOctree *octree);
/* src/linear_octree.h:97-101 */
bool linear_octree_check_if_included(int64_t morton_index_i,
                                     int64_t morton_index_j, int level);

/* ---- simulation (src/grav_sim.h:47-55, src/python_interface.c:8-304) */

/* src/grav_sim.h:47-55 */
ErrorStatus launch_simulation(System *system, IntegratorParam *integrator_param,
                              AccelerationParam *acceleration_param,
                              OutputParam *output_param,
                              SimulationStatus *simulation_status,
                              Settings *settings, double tf);

/* ---- particle mesh and cosmology (src/acceleration_PM.c,
 *      src/integrator_cosmology_leapfrog.c, src/cosmology.c) ----------- */

/* src/system.h:22-38 */
typedef struct CosmologicalSystem {
    int num_particles;
    int *particle_ids;
    double *x;
    double *v;
    double *m;
    double h;
    double omega_m;
    double omega_lambda;
    double omega_k;
    double box_center[3];
    double box_width;
    double unit_mass;
    double unit_length;
    double unit_time;
} CosmologicalSystem;

/* src/system.h:78 */
CosmologicalSystem get_new_cosmological_system(void);
/* src/system.h:111 */
ErrorStatus finalize_cosmological_system(CosmologicalSystem *system);
/* src/system.h:287 (host arrays) */
void set_periodic_boundary_conditions(CosmologicalSystem *system);
/* src/cosmology.h:5-15 */
double compute_omega_k(double omega_m, double omega_lambda);
double compute_da(double a, double H0, double omega_m, double omega_lambda);

/* src/acceleration.h:73-85.  Host arrays in and out; the cloud-in-cell
 * deposit and interpolation, the Green's function and the gradient run on the
 * GPU, the 3-D r2c / c2r transforms through cuFFT (FFTW's layout). */
ErrorStatus acceleration_PM(double *a, int num_particles, const double *x, const double *m,
                            const double *box_center, double box_width, double H0,
                            double omega_m, double mean_bkg_density, int pm_grid_size,
                            double scale_factor);

/* src/integrator.h:155-164.  Snapshots are HDF5 (src/output.c:697-900; CSV
 * is refused as the reference refuses it).  x advances in place; v is
 * written only at snapshots, as momentum / a^2. */
ErrorStatus leapfrog_cosmology(CosmologicalSystem *system, OutputParam *output_param,
                               SimulationStatus *simulation_status, Settings *settings, double dt,
                               double a_begin, double a_final, int pm_grid_size);

/* src/grav_sim.h:71-80 */
ErrorStatus launch_cosmological_simulation(CosmologicalSystem *system, OutputParam *output_param,
                                           SimulationStatus *simulation_status,
                                           Settings *settings, double dt, double a_begin,
                                           double a_final, int pm_grid_size);

/* No reference counterpart: device time (CUDA events on the run's stream) of
 * the step loop of the calling thread's last cosmological run, its steps,
 * and this library's kernels per step (cuFFT's own kernels not counted). */
int gsgpu_cosmology_last_timing(double *loop_ms, int64_t *steps, int *kernels_per_step);

/* src/python_interface.c:94-125 */
int launch_simulation_python(
    int32_t *num_particles, int32_t *particle_ids, double *x, double *v,
    double *m, int32_t **new_particle_ids_ptr, double **new_x_ptr,
    double **new_v_ptr, double **new_m_ptr, double G, int32_t integrator,
    double dt, double tolerance, double initial_dt,
    bool whfast_remove_invalid_particles, int32_t acceleration_method,
    double opening_angle, double softening_length,
    int32_t max_num_particles_per_leaf, int32_t output_method,
    char *output_dir, bool output_initial, double output_interval,
    int32_t coordinate_output_dtype, int32_t velocity_output_dtype,
    int32_t mass_output_dtype, int32_t verbose, bool enable_progress_bar,
    bool *is_exit_ptr, double tf);

/* src/python_interface.c:195-201 (FP64 on the GPU) */
void compute_energy_python(double *energy, double G, const double *sol_state,
                           int32_t num_snapshots, int32_t num_particles);
/* Total energy with the softened potential (no counterpart in the reference,
 * whose compute_energy uses the unsoftened one): sum_i m_i |v_i|^2 / 2 -
 * G sum_{i<j} m_i m_j / sqrt(|x_i - x_j|^2 + eps^2) of n host particles.
 * Kinetic part and the final sums in FP64; the potential's pair terms in
 * compensated FP32 on double-float coordinates relative to the bounding-box
 * centre (about 1e-7 relative), for energy drift at sizes where the FP64
 * O(N^2) sum is too slow.  Returns a GRAV_* code. */
int gsgpu_softened_energy(const double *x, const double *v, const double *m, int n, double G,
                          double eps, double *energy);
/* src/python_interface.c:245-250 */
void compute_linear_momentum_python(double *linear_momentum,
                                    const double *sol_state,
                                    int32_t num_snapshots, int32_t num_particles);
/* src/python_interface.c:270-275 */
void compute_angular_momentum_python(double *angular_momentum,
                                     const double *sol_state,
                                     int32_t num_snapshots, int32_t num_particles);
/* src/utils.h (compute_energy, src/utils.c:27) */
double compute_energy(const System *system);

/* src/python_interface.c:8-16 */
/* src/grav_sim.h:92: the build's facts (CUDA runtime, device code, cuFFT,
 * the HDF5 writer), printed to stdout. */
void print_compilation_info(void);
void free_memory_int32(int32_t *ptr);
void free_memory_double(double *ptr);
/* src/python_interface.c:18-26.  Built-in initial conditions are host
 * bookkeeping outside this library's scope: returns GRAV_NOT_IMPLEMENTED_ERROR. */
int32_t load_built_in_system_python(const char *system_name, int *num_particles_ptr,
                                    int32_t **particle_ids_ptr, double **x_ptr,
                                    double **v_ptr, double **m_ptr, double *G_ptr);
/* src/python_interface.c:55-70 */
void keplerian_to_cartesian_python(double *x, double *y, double *z, double *v_x,
                                   double *v_y, double *v_z,
                                   double semi_major_axis, double eccentricity,
                                   double inclination, double argument_of_periapsis,
                                   double longitude_of_ascending_node,
                                   double true_anomaly, double total_mass,
                                   double G);

/* ---- device-resident simulation (no counterpart in the reference) ----
 * The same integrator loops as launch_simulation with the state kept in
 * HBM between calls, for callers that time or steer the GPU loop directly.
 * `stream` is a cudaStream_t (NULL = the library's own stream). */
typedef struct gsgpu_sim gsgpu_sim;

int gsgpu_sim_create(gsgpu_sim **out, int num_particles, double G,
                     const AccelerationParam *acceleration_param,
                     int integrator, double dt, void *stream);
/* Host -> device copy of x [3N], v [3N], m [N]; resets compensation terms. */
int gsgpu_sim_upload(gsgpu_sim *sim, const double *x, const double *v,
                     const double *m);
/* Enqueue num_steps integrator steps (asynchronous on the stream); fixed-step
 * integrators (1-4) only. */
int gsgpu_sim_run(gsgpu_sim *sim, int64_t num_steps);
/* The reference's loop to time tf (src/integrator.c, fixed-step: ceil(tf/dt)
 * steps with the last one clamped; src/integrator_rk_embedded.c:680-930,
 * integrators 5-8, and src/integrator_ias15.c:229-616, integrator 9:
 * adaptive steps from the initial dt to tf).  Synchronous. */
int gsgpu_sim_run_until(gsgpu_sim *sim, double tf);
/* Adaptive integrators (5-9): the tolerance and the initial dt (<= 0: the
 * reference's estimate, src/integrator_rk_embedded.c:346-520 and
 * src/integrator_ias15.c:702-806). */
int gsgpu_sim_set_tolerance(gsgpu_sim *sim, double tolerance, double initial_dt);
/* Device -> host copy of x, v (v synchronised to integer time for leapfrog). */
int gsgpu_sim_download(gsgpu_sim *sim, double *x, double *v);
/* Device pointer of the current acceleration array [3N] (FP64). */
const double *gsgpu_sim_device_acceleration(const gsgpu_sim *sim);
/* Device -> host copy of the most recent accelerations a [3N]. */
int gsgpu_sim_download_acceleration(gsgpu_sim *sim, double *a);
/* Accumulated device time and launch count of the force kernel (CUDA
 * events on the simulation's stream); enable before gsgpu_sim_run. */
int gsgpu_sim_set_force_timing(gsgpu_sim *sim, int enable);
int gsgpu_sim_force_timing(const gsgpu_sim *sim, double *total_ms,
                           int64_t *launches);
/* Number of kernels launched by the most recent gsgpu_sim_run step. */
/* Barnes-Hut methods, while force timing is on: summed milliseconds of the
 * Morton-key kernel and of the particle key sort over the tree builds
 * since it was turned on, and the number of builds. */
int gsgpu_sim_build_timing(const gsgpu_sim *sim, double *morton_ms, double *sort_ms,
                           int64_t *builds);
int gsgpu_sim_kernels_per_step(const gsgpu_sim *sim);
/* Interactions of the most recent force evaluation: counts[0] cell
 * (monopole) terms, counts[1] particle-particle terms (tree methods; both 0
 * for the direct sums, whose count is N(N-1)). */
int gsgpu_sim_interaction_counts(gsgpu_sim *sim, long long *counts);
/* The same for the calling thread's most recent acceleration() call. */
int gsgpu_last_interaction_counts(long long *counts);
/* Advance the simulation until its force engine is ready (the learned
 * method collects its training snapshots during its first steps and then
 * trains); at most max_steps steps.  0 when ready. */
int gsgpu_sim_warmup_until_ready(gsgpu_sim *sim, int64_t max_steps, int64_t *steps_taken);
/* Engine statistics; returns the number of values written (learned method:
 * trained, snapshots, first-epoch loss, last-epoch loss, held-out median
 * residual before and after the network, last judged median error, steps
 * judged, steps that fell back, cheap opening angle, training seconds, Adam
 * steps, network in use: 1 if it cut the held-out median residual by at
 * least 20 % and the corrected held-out median is within the judge's 1e-3
 * bound, else 0 and every step uses the judged fallback walk). */
int gsgpu_sim_report(gsgpu_sim *sim, double *out, int nmax);
/* Learned method (104): 0 follows the rule above (the default), 1 applies the
 * network at every step whatever it gained (the judge still checks each step
 * and falls back to the theta 0.5 walk when the median error exceeds 1e-3),
 * 2 never applies it.  GRAV_VALUE_ERROR for other methods or policies.  The
 * next step is captured afresh. */
int gsgpu_sim_set_learned_policy(gsgpu_sim *sim, int policy);

/* How the embedded Runge-Kutta integrators (5-8; src/integrator_rk_embedded.c
 * :522-987 is the loop this replaces) add the 6N error terms of an attempt,
 * for every run started after the call: 0 (the default) copies the terms to
 * the host and adds them one by one in the reference's order, so the step
 * control -- and the run -- equal the reference's bit for bit; 1 adds them on
 * the device in a fixed grouping and copies one double back (no 6N-double copy
 * and host loop per attempt; the sum's rounding differs from the reference's
 * in the last bits, so accepted steps and step sizes may differ slightly).
 * GRAV_VALUE_ERROR for other modes. */
int gsgpu_set_rk_error_sum(int mode);
/* Learned method: copy up to `count` training samples of one snapshot
 * (features [count][32], targets [count][3]); returns the number copied. */
int gsgpu_sim_training_samples(gsgpu_sim *sim, int snapshot, float *features, float *targets,
                               int count);
void gsgpu_sim_destroy(gsgpu_sim *sim);

/* Batched planetary ensembles: many independent systems of uneven size
 * advanced together, every phase one launch over all systems.  Replaces the
 * reference's per-system WHFast (src/integrator_whfast.c:200-407, integrator
 * 10, with its sort by distance src/system.c:1210-1335 and particle removal
 * src/system.c:444-577) and leapfrog (src/integrator.c:894-1121, integrator
 * 4) driven by the massless (GRAV_GPU_MASSLESS) or pairwise
 * (GRAV_GPU_PAIRWISE / GRAV_GPU_PAIRWISE_FP64: FP64, reference order)
 * accelerations.  Each system evolves bit for bit as the reference evolves
 * it alone.  counts[s] particles per system (1..16384); arrays are the
 * systems concatenated, ids system-local with the primary's id 0.  WHFast
 * removes particles whose Kepler solve fails; downloads then report the new
 * counts and leave the freed slots at each system's end. */
typedef struct gsgpu_ensemble gsgpu_ensemble;

int gsgpu_ensemble_create(gsgpu_ensemble **out, int num_systems, const int *counts,
                          double G, int integrator, int acceleration_method,
                          double softening_length, double dt,
                          int remove_invalid_particles, void *stream);
int gsgpu_ensemble_upload(gsgpu_ensemble *e, const int *ids, const double *x,
                          const double *v, const double *m);
/* Enqueue num_steps steps of the creation dt (asynchronous). */
int gsgpu_ensemble_run(gsgpu_ensemble *e, int64_t num_steps);
/* The reference's loop to time tf: ceil(tf/dt) steps, the last one clamped. */
int gsgpu_ensemble_run_until(gsgpu_ensemble *e, double tf);
/* counts [S], ids [P], x, v [3P], m [P]; any pointer may be NULL. */
int gsgpu_ensemble_download(gsgpu_ensemble *e, int *counts, int *ids, double *x,
                            double *v, double *m);
int gsgpu_ensemble_kernels_per_step(const gsgpu_ensemble *e);
int gsgpu_ensemble_num_particles(const gsgpu_ensemble *e);
/* Thread-block sizes the ensemble's autotuner chose for its per-particle
 * acceleration and drift kernels (timed once after the first half kick;
 * 0 before that). */
int gsgpu_ensemble_tuning(const gsgpu_ensemble *e, int *accel_threads, int *drift_threads);
/* Threads per system the autotuner chose for the sort by distance, one
 * entry per size class of systems present (the class's power-of-two
 * capacity in pow2[k], its threads in threads[k]); returns the number of
 * classes written (at most n). */
int gsgpu_ensemble_sort_tuning(const gsgpu_ensemble *e, int *pow2, int *threads, int n);
/* Self-check (no counterpart in the reference): the Kepler drift's Stumpff
 * series divides by 13 small integer constants through a division-free
 * correctly rounded quotient; this compares it with the division itself
 * (__ddiv_rn) bit for bit on n samples (random bit patterns and quotients
 * next to rounding ties).  *mismatches receives the number that differ. */
int gsgpu_stumpff_division_selftest(long long n, unsigned long long seed, long long *mismatches);
/* Self-check (no counterpart in the reference): the Morton keys divide the
 * centred coordinates by the box width through a division-free correctly
 * rounded quotient; this compares it with __ddiv_rn bit for bit on n samples
 * (random widths and dividends, quotients next to rounding ties).
 * *mismatches receives the number that differ. */
int gsgpu_width_division_selftest(long long n, unsigned long long seed, long long *mismatches);
/* Kernel timing (no counterpart in the reference): while enabled, steps are
 * launched directly instead of from the captured graph, with CUDA events
 * around the Kepler drift and around the interaction accelerations (the
 * pair sums and the per-particle terms; for leapfrog the massless
 * accelerations).  gsgpu_ensemble_kernel_timing returns the summed
 * milliseconds of each and the number of timed steps since timing was
 * enabled. */
int gsgpu_ensemble_set_kernel_timing(gsgpu_ensemble *e, int enable);
int gsgpu_ensemble_kernel_timing(const gsgpu_ensemble *e, double *drift_ms, double *accel_ms,
                                 int64_t *steps);
void gsgpu_ensemble_destroy(gsgpu_ensemble *e);

/* Library / device information: fills name (NUL-terminated, <= len). */
int gsgpu_device_info(char *name, int len, int *sm_count, int *cc_major,
                      int *cc_minor);

/* Allocation-free compensated-FP32 direct sum.  No counterpart in the
 * reference.  For callers that must not allocate device memory while they
 * run -- code that records or replays a fixed plan of GPU work, where a
 * cudaMalloc (which may synchronise the device) would break the plan;
 * embedders whose device memory is a pool they manage; real-time loops that
 * may not touch the allocator.  Computes the accelerations of
 * acceleration() with GRAV_GPU_PAIRWISE (positions taken relative to the
 * centre of their bounding box, which is found on the device) from
 * caller-owned device arrays d_x [3N], d_m [N] into d_a [3N], enqueued on
 * `stream` (a cudaStream_t; NULL = legacy default stream) and not
 * synchronised.  Errors found on the device cannot be returned by a call
 * that does not wait for the GPU: if a shared-memory tile wait of the
 * kernel runs out, every element of d_a is NaN, never partial sums.  It calls no cudaMalloc, cudaFree or allocating library
 * routine: its scratch is a fixed device array in the library image of about
 * 6.5 MiB, which every GPU that loads the library keeps until the process
 * exits, so num_particles is limited to 1..32768 (larger counts return
 * GRAV_VALUE_ERROR).  The first call on each device looks up that array's
 * device address with the device current; make that first call before any
 * stream capture.  All calls share the one array and it keeps the last
 * call's contents: calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.  Returns a GRAV_*
 * code; messages go to stderr. */
int gsgpu_pairwise_acceleration_noalloc(const double *d_x, const double *d_m,
                                        int num_particles, double G,
                                        double softening_length, double *d_a,
                                        void *stream);

/* Tensor-core self-test (no counterpart in the reference): one 128 x N tile
 * C = A * B^T through tcgen05 BF16 MMA with FP32 accumulation in TMEM.
 * hA [128 x K], hB [N x K] are row-major BF16 bit patterns on the host, hC
 * [128 x N] FP32; the operands are staged K-major or MN-major as selected.
 * 16 <= N, K <= 128, multiples of 16. */
int gsgpu_tc_gemm_selftest(int N, int K, int a_mn_major, int b_mn_major,
                           const uint16_t *hA, const uint16_t *hB, float *hC);

/* ---- learned residual network (no counterpart in the reference) ------
 * 32 -> 64 -> 64 -> 64 -> 3 MLP with SiLU, BF16 tcgen05 kernels with FP32
 * accumulation.  Parameters are FP32 (gsgpu_mlp_num_params() floats:
 * W1[64][32] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[16][64] b4[16],
 * last-layer rows 3..15 zero).  Features [n][32] and targets / predictions
 * [n][3] are FP32 host arrays. */
typedef struct gsgpu_mlp gsgpu_mlp;
int gsgpu_mlp_num_params(void);
int gsgpu_mlp_create(gsgpu_mlp **out, unsigned long long seed);
void gsgpu_mlp_destroy(gsgpu_mlp *mlp);
int gsgpu_mlp_get_params(gsgpu_mlp *mlp, float *params);
int gsgpu_mlp_set_params(gsgpu_mlp *mlp, const float *params);
int gsgpu_mlp_forward(gsgpu_mlp *mlp, const float *features, int n, float *pred);
/* Gradient of mean_n sum_k (pred_k - target_k)^2 w.r.t. the parameters (no
 * update); loss_sum receives sum_n sum_k (pred_k - target_k)^2. */
int gsgpu_mlp_gradients(gsgpu_mlp *mlp, const float *features, const float *target, int n,
                        float *grad, double *loss_sum);
/* One Adam step (beta1 0.9, beta2 0.999) with learning rate lr. */
int gsgpu_mlp_train_step(gsgpu_mlp *mlp, const float *features, const float *target, int n,
                         float lr, double *loss_sum);

/* FMA-throughput probe of the running GPU (fp64 = 0: FP32, 1: FP64):
 * TFLOP/s at 2 FLOP per FMA, best of 5 launches.  No counterpart in the
 * reference; it supplies the FP32/FP64 pipe peaks of the rooflines. */
int gsgpu_measure_fma_peak(int fp64, double *tflops, double *ms);

/* No reference counterpart: a kernel whose bounded wait runs out (an
 * mbarrier nobody arrives at, limit_ms in 1..2000) writes the device status
 * word, which is returned in *status_out (ST_WAIT_TIMEOUT = 1).  Shows that
 * an expired wait ends with an error status and leaves the context usable. */
int gsgpu_wait_timeout_selftest(double limit_ms, unsigned *status_out);

/* No reference counterpart: host-side fault injection for tests.  The k-th
 * device allocation from now on fails as an out-of-memory cudaMalloc would
 * (the call returns GRAV_MEMORY_ERROR); k = 0 switches it off. */
void gsgpu_test_fail_allocation(int k);

#ifdef __cplusplus
}
#endif

#endif /* GRAV_SIM_GB300_H */
