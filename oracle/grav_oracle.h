/*
 * grav_oracle.h -- CPU restatement of grav_sim's force-evaluation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * product: tests/, __graft_entry__.smoke() and the cpu_baseline leg of
 * bench.py may load it; the product library never does.
 *
 * Every function restates (in FP64, serial, no FMA contraction) the
 * algorithm of the grav_sim file:line named in its comment.  The
 * restatement is pinned against the reference itself (compiled from its own
 * sources into oracle/_ref/) and against the committed golden vectors in
 * tests/golden/.
 */
#ifndef GRAV_ORACLE_H
#define GRAV_ORACLE_H

#include <stdint.h>

#define ORC_MORTON_MAX_LEVEL 21

/* src/acceleration.c:177-234 (symmetric i<j loop, Plummer softening) */
void orc_pairwise(int n, const double *x, const double *m, double G,
                  double eps, double *a);

/* src/acceleration.c:198-231 restricted to outer rows [i_begin, i_end);
 * returns the number of pair evaluations (for timing bounded samples). */
int64_t orc_pairwise_slice(int n, const double *x, const double *m, double G,
                           double eps, int i_begin, int i_end, double *a);

/* src/acceleration.c:236-367, including the m[i] loop-index mass read at
 * :357-359 (the reference reads the mass of the i-th particle in array order,
 * not of the i-th massive particle). */
int orc_massless(int n, const double *x, const double *m, double G,
                 double eps, double *a);

/* src/linear_octree.c:113-146 */
void orc_bbox(int n, const double *x, double center[3], double *width);

/* src/linear_octree.c:159-202 (normalise, truncate, 21-bit mask, spread) */
void orc_morton(int n, const double *x, const double center[3], double width,
                int64_t *keys);

/* src/linear_octree.c:216-326: stable LSD radix sort of keys with their
 * indices (9-bit digits, ceil(63/9) passes). */
int orc_radix_sort(int n, int64_t *keys, int *idx);

/* Node arrays of the linear octree, in the reference's node numbering
 * (src/linear_octree.h:20-57). */
typedef struct OrcTree {
    double box_width;
    double center[3];
    int num_nodes;
    int capacity;
    int64_t *keys;          /* sorted Morton keys            [n] */
    int *sorted_indices;    /* particle id at sorted slot    [n] */
    int *num_particles;     /* [num_nodes] */
    int *num_children;      /* [num_nodes], 0 for leaves */
    int *first_particle;    /* [num_nodes] */
    int *first_child;       /* [num_nodes], -1 for leaves */
    int *depth;             /* [num_nodes] */
    double *mass;           /* [num_nodes] */
    double *com;            /* [num_nodes*3] */
} OrcTree;

/* src/linear_octree.c:825-962 (construct_octree) with the tree build of
 * :342-823.  compat=1 keeps the reference's zero leaf mass/centre of mass
 * (:567-570, :662-677); compat=0 gives leaves their true mass and centre of
 * mass, summed over their particles in sorted order. */
int orc_build_tree(int n, const double *x, const double *m, int leaf_max,
                   int compat, OrcTree *tree);
void orc_free_tree(OrcTree *tree);

/* src/acceleration_barnes_hut.c:78-248.  compat=1 reproduces the reference's
 * cell-membership test, which indexes the sorted key array by particle id
 * (:120, :145); compat=0 uses each particle's own sorted key.  If counts is
 * not NULL it receives, per particle, the number of accepted cells (counts[2i])
 * and of leaf particle-particle terms (counts[2i+1]); if absum is not NULL it
 * receives the sum of the magnitudes of the particle's terms. */
void orc_bh_walk(int n, const double *x, const double *m, double G,
                 double eps, double theta, const OrcTree *tree, int compat,
                 double *a, int64_t *counts, double *absum);

/* The walk for the sorted positions offset + k * stride, k < count (a strided
 * sample); in the OpenMP build (liboracle_omp.so) the loop over them is
 * parallel as the reference's (src/acceleration_barnes_hut.c:114-117). */
void orc_bh_walk_sample(const double *x, const double *m, double G, double eps,
                        double theta, const OrcTree *tree, int compat, int64_t offset,
                        int64_t stride, int count, double *a);
/* Threads the build uses (1 without OpenMP). */
int orc_num_threads(void);

/* Quadrupole extension (not in grav_sim): traceless node quadrupoles about
 * the centre of mass, q[6*node] = (xx, xy, xz, yy, yz, zz), and the
 * corrected walk with monopole + quadrupole cell terms. */
void orc_quadrupoles(const OrcTree *tree, const double *x, const double *m,
                     double *q);
void orc_bh_walk_quad(int n, const double *x, const double *m, double G,
                      double eps, double theta, const OrcTree *tree,
                      const double *q, double *a, double *absum);

/* Whole Barnes-Hut evaluation: build + walk (src/acceleration_barnes_hut.c:33-76). */
int orc_barnes_hut(int n, const double *x, const double *m, double G,
                   double eps, double theta, int leaf_max, int compat,
                   double *a);

/* Compensated kick/drift of src/integrator.c:1009-1018 and :1030-1039:
 *   err += d*dt; y_new = y + err; err += y - y_new. */
void orc_comp_update(int len, double *y, double *err, const double *d,
                     double dt);

/* Fixed-step integrators of src/integrator.c driven by the FP64 pairwise
 * sum (method 1) or the massless sum (method 2): integrator codes 1 euler,
 * 2 euler-cromer, 3 rk4, 4 leapfrog.  Reproduces total_num_steps =
 * ceil(tf/dt), the last-step dt clamp and t = steps*dt. */
/* Opening angle, particles per leaf and quirk mode of method 3 (Barnes-Hut)
 * in orc_fixed_step_run. */
void orc_set_bh_params(double theta, int leaf_max, int compat);
int orc_fixed_step_run(int integrator, int method, int n, double *x, double *v,
                       const double *m, double G, double eps, double dt,
                       double tf);

/* src/integrator_rk_embedded.c:346-987: RKF45 (5), DOPRI (6), DVERK (7) and
 * RKF78 (8) with the pairwise (method 1) or massless (method 2) sum;
 * abs = rel = tolerance; initial_dt <= 0 selects the reference's initial
 * step estimate.  Reports the accepted steps, final t and the next dt. */
int orc_rk_embedded_run(int integrator, int method, int n, double *x, double *v,
                        const double *m, double G, double eps, double tolerance,
                        double initial_dt, double tf, int64_t *num_steps, double *t_out,
                        double *dt_out);

/* src/integrator_ias15.c:229-616 (IAS15, integrator 9) with the pairwise
 * (method 1) or massless (method 2) sum; initial_dt <= 0 selects the
 * reference's estimate.  Reports the accepted steps, final t and next dt. */
int orc_ias15_run(int method, int n, double *x, double *v, const double *m, double G, double eps,
                  double tolerance, double initial_dt, double tf, int64_t *num_steps,
                  double *t_out, double *dt_out);

/* src/integrator_whfast.c:200-407 for one system: sort by distance, eta,
 * Jacobi transforms, universal-variable Kepler drift, the interaction
 * accelerations (pairwise=0: the massless variant :959-1264, 1: the
 * pairwise variant :839-957) and kicks; a[0] and the uninitialised aux of
 * the reference are taken as zero.  *n shrinks when remove_invalid removes
 * particles whose Kepler solve failed. */
int orc_whfast_run(int *n, int *ids, double *x, double *v, double *m, double G,
                   double eps, double dt, double tf, int remove_invalid, int pairwise);

/* FFTW 3's r2c / c2r 3-D transforms (unnormalised) by direct DFT
 * (pm_dft.c); out of r2c and in of c2r are n0 x n1 x (n2/2+1) complex
 * values, interleaved. */
void orc_dft3_r2c(int n0, int n1, int n2, const double *in, double *out);
void orc_dft3_c2r(int n0, int n1, int n2, const double *in, double *out);

/* src/acceleration_PM.c:15-391: cloud-in-cell deposit, Poisson solve in
 * Fourier space, fourth-order gradient, cloud-in-cell interpolation. */
void orc_acceleration_pm(double *a, int n, const double *x, const double *m,
                         const double *box_center, double box_width, double H0, double omega_m,
                         double mean_bkg_density, int pm_grid_size, double scale_factor);
/* src/cosmology.c:15-26 */
double orc_compute_da(double a, double H0, double omega_m, double omega_lambda);
/* src/system.c:1337-1375 */
void orc_periodic_boundary(int n, double *x, const double *box_center, double box_width);
/* src/integrator_cosmology_leapfrog.c:24-255, output disabled; v_last (may
 * be NULL) gets momentum / a^2 after the last step. */
void orc_leapfrog_cosmology(int n, double *x, const double *v, const double *m, double h,
                            double omega_m, double omega_lambda, const double *box_center,
                            double box_width, double dt, double a_begin, double a_final,
                            int pm_grid_size, int64_t *num_steps, double *t_out, double *v_last);

/* src/utils.c:27-59 (kinetic + unsoftened pairwise potential energy). */
double orc_energy(int n, const double *x, const double *v, const double *m,
                  double G);

/* src/python_interface.c:245-304, component sums as the reference forms them. */
double orc_linear_momentum(int n, const double *v, const double *m);
double orc_angular_momentum(int n, const double *x, const double *v,
                            const double *m);

/* Exact FP64 direct sum in a fixed j order, used as the ground truth for
 * relative-error statistics (not a reference restatement). */
void orc_direct_rows(int n, const double *x, const double *m, double G,
                     double eps, int nrows, const int *rows, double *a_rows);

/* Sum of pair-term magnitudes, A_i = G sum_j m_j |r_ij| / (r_ij^2+eps^2)^1.5:
 * the scale against which the rounding of FP32 pair terms is bounded. */
void orc_abs_sum_rows(int n, const double *x, const double *m, double G,
                      double eps, int nrows, const int *rows, double *out);

/* Independent systems, each run as the reference runs it alone (WHFast with
 * removal, integrator 10, or leapfrog, integrator 4; massless acceleration,
 * no softening); one system per thread in the OpenMP build. */
int orc_ensemble_run(int S, int *counts, const int64_t *off, int *ids, double *x,
                     double *v, double *m, double G, double dt, double tf,
                     int integrator);

#endif
