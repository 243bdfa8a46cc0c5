/*
 * grav_oracle.c -- CPU restatement of grav_sim's force-evaluation hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see grav_oracle.h).  Compiled with
 * -ffp-contract=off: every product and sum is rounded on its own, in the
 * order the reference's C expressions evaluate them.
 */
#include "grav_oracle.h"

#ifdef ORC_OPENMP
#include <omp.h>
#endif

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Direct sums                                                          */
/* ------------------------------------------------------------------ */

/* src/acceleration.c:177-234.  For the pair (i<j) the reference forms
 * R = x_i - x_j, |R| = sqrt(R.R + eps^2), t = G/|R|^3, then
 * a_i -= (t R) m_j and a_j += (t R) m_i. */
void orc_pairwise(int n, const double *x, const double *m, double G,
                  double eps, double *a)
{
    for (int k = 0; k < 3 * n; ++k) a[k] = 0.0;
    const double eps2 = eps * eps;
    for (int i = 0; i < n; ++i) {
        const double mi = m[i];
        for (int j = i + 1; j < n; ++j) {
            double r0 = x[3 * i + 0] - x[3 * j + 0];
            double r1 = x[3 * i + 1] - x[3 * j + 1];
            double r2 = x[3 * i + 2] - x[3 * j + 2];
            double s = r0 * r0 + r1 * r1 + r2 * r2 + eps2;
            double rn = sqrt(s);
            double t = G / (rn * rn * rn);
            double mj = m[j];
            double t0 = t * r0, t1 = t * r1, t2 = t * r2;
            a[3 * i + 0] -= t0 * mj;
            a[3 * i + 1] -= t1 * mj;
            a[3 * i + 2] -= t2 * mj;
            a[3 * j + 0] += t0 * mi;
            a[3 * j + 1] += t1 * mi;
            a[3 * j + 2] += t2 * mi;
        }
    }
}

/* The reference's symmetric loop (src/acceleration.c:198-231) restricted to
 * outer rows [i_begin, i_end): every pair (i, j>i) of those rows is
 * evaluated once and updates both a_i and a_j.  A bounded slice of the
 * reference's own work, used to time it without running all N(N-1)/2 pairs.
 * Returns the number of pair evaluations performed. */
int64_t orc_pairwise_slice(int n, const double *x, const double *m, double G,
                           double eps, int i_begin, int i_end, double *a)
{
    int64_t pairs = 0;
    for (int k = 0; k < 3 * n; ++k) a[k] = 0.0;
    const double eps2 = eps * eps;
    for (int i = i_begin; i < i_end && i < n; ++i) {
        const double mi = m[i];
        for (int j = i + 1; j < n; ++j) {
            double r0 = x[3 * i + 0] - x[3 * j + 0];
            double r1 = x[3 * i + 1] - x[3 * j + 1];
            double r2 = x[3 * i + 2] - x[3 * j + 2];
            double rn = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + eps2);
            double t = G / (rn * rn * rn);
            double mj = m[j];
            double t0 = t * r0, t1 = t * r1, t2 = t * r2;
            a[3 * i + 0] -= t0 * mj;
            a[3 * i + 1] -= t1 * mj;
            a[3 * i + 2] -= t2 * mj;
            a[3 * j + 0] += t0 * mi;
            a[3 * j + 1] += t1 * mi;
            a[3 * j + 2] += t2 * mi;
        }
        pairs += n - 1 - i;
    }
    return pairs;
}

/* src/acceleration.c:236-367.  Massive particles (m != 0) interact
 * symmetrically; each massless particle feels every massive one.  The
 * massless term reads m[i] where i counts massive particles (:357-359). */
int orc_massless(int n, const double *x, const double *m, double G,
                 double eps, double *a)
{
    for (int k = 0; k < 3 * n; ++k) a[k] = 0.0;
    int *heavy = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *light = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!heavy || !light) { free(heavy); free(light); return 4; }
    int nh = 0, nl = 0;
    for (int i = 0; i < n; ++i) {
        if (m[i] != 0.0) heavy[nh++] = i; else light[nl++] = i;
    }
    const double eps2 = eps * eps;
    for (int p = 0; p < nh; ++p) {
        const int i = heavy[p];
        const double mi = m[i];
        for (int q = p + 1; q < nh; ++q) {
            const int j = heavy[q];
            const double mj = m[j];
            double r0 = x[3 * i + 0] - x[3 * j + 0];
            double r1 = x[3 * i + 1] - x[3 * j + 1];
            double r2 = x[3 * i + 2] - x[3 * j + 2];
            double rn = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + eps2);
            double t = G / (rn * rn * rn);
            double t0 = t * r0, t1 = t * r1, t2 = t * r2;
            a[3 * i + 0] -= t0 * mj;
            a[3 * i + 1] -= t1 * mj;
            a[3 * i + 2] -= t2 * mj;
            a[3 * j + 0] += t0 * mi;
            a[3 * j + 1] += t1 * mi;
            a[3 * j + 2] += t2 * mi;
        }
    }
    for (int p = 0; p < nh; ++p) {
        const int i = heavy[p];
        for (int q = 0; q < nl; ++q) {
            const int j = light[q];
            double r0 = x[3 * i + 0] - x[3 * j + 0];
            double r1 = x[3 * i + 1] - x[3 * j + 1];
            double r2 = x[3 * i + 2] - x[3 * j + 2];
            double rn = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + eps2);
            double t = G / (rn * rn * rn);
            a[3 * j + 0] += t * r0 * m[p];
            a[3 * j + 1] += t * r1 * m[p];
            a[3 * j + 2] += t * r2 * m[p];
        }
    }
    free(heavy);
    free(light);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Linear octree                                                        */
/* ------------------------------------------------------------------ */

/* src/linear_octree.c:113-146 */
void orc_bbox(int n, const double *x, double center[3], double *width)
{
    double lo[3] = {x[0], x[1], x[2]};
    double hi[3] = {x[0], x[1], x[2]};
    for (int i = 1; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fmin(lo[k], x[3 * i + k]);
            hi[k] = fmax(hi[k], x[3 * i + k]);
        }
    }
    for (int k = 0; k < 3; ++k) center[k] = (hi[k] + lo[k]) / 2.0;
    double w = fmax(fmax(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    *width = w;
}

/* Interleave the low 21 bits of v with two zero bits between each bit. */
static int64_t spread21(int64_t v)
{
    uint64_t u = (uint64_t)v & 0x1fffffULL;
    uint64_t out = 0;
    for (int b = 0; b < 21; ++b) out |= ((u >> b) & 1ULL) << (3 * b);
    return (int64_t)out;
}

/* src/linear_octree.c:159-202.  The normalised coordinate is converted to
 * an integer by C truncation, so a particle at the box maximum gives 2^21,
 * which the 21-bit mask turns into 0. */
void orc_morton(int n, const double *x, const double center[3], double width,
                int64_t *keys)
{
    for (int i = 0; i < n; ++i) {
        int64_t c[3];
        for (int k = 0; k < 3; ++k) {
            double u = (x[3 * i + k] - center[k]) / width + 0.5;
            c[k] = (int64_t)(u * (double)(1 << 21));
        }
        keys[i] = spread21(c[0]) | (spread21(c[1]) << 1) | (spread21(c[2]) << 2);
    }
}

/* src/linear_octree.c:216-326: stable LSD radix sort, 9-bit digits. */
int orc_radix_sort(int n, int64_t *keys, int *idx)
{
    const int bits = 9, radix = 1 << 9;
    const int passes = (3 * ORC_MORTON_MAX_LEVEL + bits - 1) / bits;
    int64_t *k2 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int *i2 = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *cnt = (int *)malloc(sizeof(int) * radix);
    if (!k2 || !i2 || !cnt) { free(k2); free(i2); free(cnt); return 4; }
    int64_t *src_k = keys, *dst_k = k2;
    int *src_i = idx, *dst_i = i2;
    for (int p = 0; p < passes; ++p) {
        const int shift = p * bits;
        memset(cnt, 0, sizeof(int) * radix);
        for (int j = 0; j < n; ++j) cnt[(src_k[j] >> shift) & (radix - 1)]++;
        int run = 0;
        for (int d = 0; d < radix; ++d) { int c = cnt[d]; cnt[d] = run; run += c; }
        for (int j = 0; j < n; ++j) {
            int d = (int)((src_k[j] >> shift) & (radix - 1));
            int at = cnt[d]++;
            dst_k[at] = src_k[j];
            dst_i[at] = src_i[j];
        }
        int64_t *tk = src_k; src_k = dst_k; dst_k = tk;
        int *ti = src_i; src_i = dst_i; dst_i = ti;
    }
    if (src_k != keys) {
        memcpy(keys, src_k, sizeof(int64_t) * (size_t)n);
        memcpy(idx, src_i, sizeof(int) * (size_t)n);
    }
    free(k2); free(i2); free(cnt);
    return 0;
}

static int tree_reserve(OrcTree *t, int need)
{
    if (need <= t->capacity) return 0;
    int cap = t->capacity > 0 ? t->capacity : 64;
    while (cap < need) cap *= 2;
#define GROW(field, type, per)                                               \
    do {                                                                     \
        type *p_ = (type *)realloc(t->field, sizeof(type) * (size_t)cap * per); \
        if (!p_) return 4;                                                   \
        t->field = p_;                                                       \
    } while (0)
    GROW(num_particles, int, 1);
    GROW(num_children, int, 1);
    GROW(first_particle, int, 1);
    GROW(first_child, int, 1);
    GROW(depth, int, 1);
    GROW(mass, double, 1);
    GROW(com, double, 3);
#undef GROW
    t->capacity = cap;
    return 0;
}

/* Octant digit of a deepest-level key at a given depth (1..21). */
static int octant_at(int64_t key, int depth)
{
    return (int)((key >> (3 * (ORC_MORTON_MAX_LEVEL - depth))) & 7);
}

/* Append the non-empty octants of node `nd` (depth d) as consecutive new
 * nodes, octant order (src/linear_octree.c:342-393 counts, :406-576 append). */
static int expand_node(OrcTree *t, int nd)
{
    const int d = t->depth[nd];
    const int begin = t->first_particle[nd];
    const int end = begin + t->num_particles[nd];
    int j = begin;
    int first = -1, count = 0;
    while (j < end) {
        const int oct = octant_at(t->keys[j], d + 1);
        int k = j;
        while (k < end && octant_at(t->keys[k], d + 1) == oct) ++k;
        if (tree_reserve(t, t->num_nodes + 1)) return 4;
        const int c = t->num_nodes++;
        if (first < 0) first = c;
        ++count;
        t->num_particles[c] = k - j;
        t->first_particle[c] = j;
        t->num_children[c] = 0;
        t->first_child[c] = -1;
        t->depth[c] = d + 1;
        t->mass[c] = 0.0;
        t->com[3 * c + 0] = t->com[3 * c + 1] = t->com[3 * c + 2] = 0.0;
        j = k;
    }
    t->first_child[nd] = first;
    t->num_children[nd] = count;
    return 0;
}

/* src/linear_octree.c:590-823 (tree build) and :825-962 (driver). */
int orc_build_tree(int n, const double *x, const double *m, int leaf_max,
                   int compat, OrcTree *t)
{
    memset(t, 0, sizeof(*t));
    if (n < 1) return 2;
    orc_bbox(n, x, t->center, &t->box_width);
    t->keys = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    t->sorted_indices = (int *)malloc(sizeof(int) * (size_t)n);
    if (!t->keys || !t->sorted_indices) return 4;
    for (int i = 0; i < n; ++i) t->sorted_indices[i] = i;
    orc_morton(n, x, t->center, t->box_width, t->keys);
    if (orc_radix_sort(n, t->keys, t->sorted_indices)) return 4;
    if (tree_reserve(t, n > 64 ? n : 64)) return 4;

    t->num_nodes = 1;
    t->num_particles[0] = n;
    t->first_particle[0] = 0;
    t->num_children[0] = 0;
    t->first_child[0] = -1;
    t->depth[0] = 0;
    t->mass[0] = 0.0;
    t->com[0] = t->com[1] = t->com[2] = 0.0;

    /* Pre-order walk over internal nodes; each internal node is expanded
     * when first reached, so children of a node are numbered contiguously
     * in the order the nodes are expanded.  Sums are carried up on exit. */
    struct Frame { int node; int next; double msum; double s[3]; } st[ORC_MORTON_MAX_LEVEL + 2];
    int top = 0;
    if (expand_node(t, 0)) return 4;
    st[0].node = 0; st[0].next = 0; st[0].msum = 0.0;
    st[0].s[0] = st[0].s[1] = st[0].s[2] = 0.0;
    for (;;) {
        struct Frame *f = &st[top];
        const int nd = f->node;
        if (f->next < t->num_children[nd]) {
            const int c = t->first_child[nd] + f->next;
            const int cnt = t->num_particles[c];
            if (cnt <= leaf_max || t->depth[c] >= ORC_MORTON_MAX_LEVEL) {
                double lm = 0.0, ls[3] = {0.0, 0.0, 0.0};
                for (int q = 0; q < cnt; ++q) {
                    const int pid = t->sorted_indices[t->first_particle[c] + q];
                    const double mp = m[pid];
                    f->msum += mp;
                    for (int k = 0; k < 3; ++k) f->s[k] += mp * x[3 * pid + k];
                    lm += mp;
                    for (int k = 0; k < 3; ++k) ls[k] += mp * x[3 * pid + k];
                }
                if (!compat) {
                    t->mass[c] = lm;
                    for (int k = 0; k < 3; ++k) t->com[3 * c + k] = ls[k] / lm;
                }
                f->next++;
                continue;
            }
            if (expand_node(t, c)) return 4;
            ++top;
            st[top].node = c; st[top].next = 0; st[top].msum = 0.0;
            st[top].s[0] = st[top].s[1] = st[top].s[2] = 0.0;
            continue;
        }
        /* all children of nd done */
        t->mass[nd] = f->msum;
        for (int k = 0; k < 3; ++k) t->com[3 * nd + k] = f->s[k] / f->msum;
        if (top == 0) break;
        struct Frame *p = &st[top - 1];
        p->msum += f->msum;
        for (int k = 0; k < 3; ++k) p->s[k] += f->s[k];
        p->next++;
        --top;
    }
    return 0;
}

void orc_free_tree(OrcTree *t)
{
    free(t->keys); free(t->sorted_indices); free(t->num_particles);
    free(t->num_children); free(t->first_particle); free(t->first_child);
    free(t->depth); free(t->mass); free(t->com);
    memset(t, 0, sizeof(*t));
}

/* src/acceleration_barnes_hut.c:78-248.  Per particle (sorted order), a
 * depth-first scan of the children of each opened node: a cell that does
 * not contain the particle and satisfies (w_c)^2 < theta^2 |R|^2 adds its
 * monopole; otherwise a leaf adds its particles (skipping the particle
 * itself) and an internal node is opened. */
/* One particle (sorted position s) of the walk of src/acceleration_barnes_hut.c:117-247. */
static void bh_walk_particle(int s, const double *x, const double *m, double G,
                             double eps2, double th2, double box_length,
                             const OrcTree *t, int compat, double *a,
                             int64_t *counts, double *absum)
{
    const int id = t->sorted_indices[s];
    const int64_t key_i = compat ? t->keys[id] : t->keys[s];
    const double xi0 = x[3 * id + 0], xi1 = x[3 * id + 1], xi2 = x[3 * id + 2];
    double ax = 0.0, ay = 0.0, az = 0.0, mag = 0.0;
    int64_t n_cell = 0, n_pp = 0;
    struct { int node; int next; } st[ORC_MORTON_MAX_LEVEL + 2];
    int top = 0;
    st[0].node = 0; st[0].next = 0;
    int level = 1;
    for (;;) {
        const int nd = st[top].node;
        if (st[top].next < t->num_children[nd]) {
            const int c = t->first_child[nd] + st[top].next;
            const int first = t->first_particle[c];
            const int64_t key_c = compat ? t->keys[t->sorted_indices[first]]
                                         : t->keys[first];
            const int sh = 3 * (ORC_MORTON_MAX_LEVEL - level);
            const int inside = (key_i >> sh) == (key_c >> sh);
            if (!inside) {
                const double r0 = xi0 - t->com[3 * c + 0];
                const double r1 = xi1 - t->com[3 * c + 1];
                const double r2 = xi2 - t->com[3 * c + 2];
                const double bl = box_length / (double)(2 << level);
                const double ns = r0 * r0 + r1 * r1 + r2 * r2;
                if (bl * bl < th2 * ns) {
                    const double rn = sqrt(ns + eps2);
                    const double tv = G * t->mass[c] / (rn * rn * rn);
                    ax -= tv * r0; ay -= tv * r1; az -= tv * r2;
                    mag += fabs(tv) * sqrt(ns);
                    ++n_cell;
                    st[top].next++;
                    continue;
                }
            }
            if (t->num_children[c] <= 0) {
                const int cnt = t->num_particles[c];
                for (int q = 0; q < cnt; ++q) {
                    const int pj = t->sorted_indices[first + q];
                    if (pj == id) continue;
                    const double r0 = xi0 - x[3 * pj + 0];
                    const double r1 = xi1 - x[3 * pj + 1];
                    const double r2 = xi2 - x[3 * pj + 2];
                    const double rn = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + eps2);
                    const double tv = G * m[pj] / (rn * rn * rn);
                    ax -= tv * r0; ay -= tv * r1; az -= tv * r2;
                    mag += fabs(tv) * sqrt(r0 * r0 + r1 * r1 + r2 * r2);
                    ++n_pp;
                }
                st[top].next++;
                continue;
            }
            ++top;
            st[top].node = c; st[top].next = 0;
            ++level;
            continue;
        }
        if (top == 0) break;
        --top;
        st[top].next++;
        --level;
    }
    a[3 * id + 0] = ax; a[3 * id + 1] = ay; a[3 * id + 2] = az;
    if (counts) { counts[2 * id] = n_cell; counts[2 * id + 1] = n_pp; }
    if (absum) absum[id] = mag;
}

void orc_bh_walk(int n, const double *x, const double *m, double G,
                 double eps, double theta, const OrcTree *t, int compat,
                 double *a, int64_t *counts, double *absum)
{
    for (int s = 0; s < n; ++s)
        bh_walk_particle(s, x, m, G, eps * eps, theta * theta, t->box_width * 2.0, t, compat, a,
                         counts, absum);
}

/* The walk for `count` sorted positions offset + k * stride (a strided
 * sample of the particles), the loop over them parallel as the reference's
 * (`#pragma omp parallel for`, src/acceleration_barnes_hut.c:114-117) when
 * built with ORC_OPENMP. */
void orc_bh_walk_sample(const double *x, const double *m, double G, double eps,
                        double theta, const OrcTree *t, int compat, int64_t offset,
                        int64_t stride, int count, double *a)
{
    const double eps2 = eps * eps, th2 = theta * theta, bl = t->box_width * 2.0;
#ifdef ORC_OPENMP
    #pragma omp parallel for
#endif
    for (int k = 0; k < count; ++k)
        bh_walk_particle((int)(offset + (int64_t)k * stride), x, m, G, eps2, th2, bl, t, compat,
                         a, NULL, NULL);
}

int orc_num_threads(void)
{
#ifdef ORC_OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Traceless quadrupole moment of every node about its centre of mass,
 * Q = sum_p m_p (3 d d^T - |d|^2 I), d = x_p - com, summed directly over the
 * node's particles; stored (xx, xy, xz, yy, yz, zz).  Not part of grav_sim:
 * the checker for the quadrupole extension of the walk. */
void orc_quadrupoles(const OrcTree *t, const double *x, const double *m,
                     double *q)
{
    for (int c = 0; c < t->num_nodes; ++c) {
        double s[6] = {0, 0, 0, 0, 0, 0};
        const double *cm = &t->com[3 * c];
        for (int p = t->first_particle[c]; p < t->first_particle[c] + t->num_particles[c]; ++p) {
            const int id = t->sorted_indices[p];
            const double d0 = x[3 * id] - cm[0], d1 = x[3 * id + 1] - cm[1], d2 = x[3 * id + 2] - cm[2];
            const double r2 = d0 * d0 + d1 * d1 + d2 * d2, mm = m[id];
            s[0] += mm * (3 * d0 * d0 - r2);
            s[1] += mm * 3 * d0 * d1;
            s[2] += mm * 3 * d0 * d2;
            s[3] += mm * (3 * d1 * d1 - r2);
            s[4] += mm * 3 * d1 * d2;
            s[5] += mm * (3 * d2 * d2 - r2);
        }
        for (int k = 0; k < 6; ++k) q[6 * c + k] = s[k];
    }
}

/* The corrected walk (compat = 0 decisions) with monopole + quadrupole terms
 * for accepted cells:  a += G [ -M R / r^3 + Q R / r^5 - 2.5 (R.Q.R) R / r^7 ],
 * R = x_i - com, r^2 = |R|^2 + eps^2.  Leaves add particle terms as usual. */
void orc_bh_walk_quad(int n, const double *x, const double *m, double G,
                      double eps, double theta, const OrcTree *t, const double *q,
                      double *a, double *absum)
{
    const double eps2 = eps * eps;
    const double th2 = theta * theta;
    const double box_length = t->box_width * 2.0;
    for (int s = 0; s < n; ++s) {
        const int id = t->sorted_indices[s];
        const int64_t key_i = t->keys[s];
        double acc[3] = {0.0, 0.0, 0.0}, mag = 0.0;
        struct { int node; int next; } st[ORC_MORTON_MAX_LEVEL + 2];
        int top = 0, level = 1;
        st[0].node = 0; st[0].next = 0;
        for (;;) {
            const int nd = st[top].node;
            if (st[top].next < t->num_children[nd]) {
                const int c = t->first_child[nd] + st[top].next;
                const int first = t->first_particle[c];
                const int sh = 3 * (ORC_MORTON_MAX_LEVEL - level);
                const int inside = (key_i >> sh) == (t->keys[first] >> sh);
                if (!inside) {
                    double R[3];
                    for (int k = 0; k < 3; ++k) R[k] = x[3 * id + k] - t->com[3 * c + k];
                    const double bl = box_length / (double)(2 << level);
                    const double ns = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
                    if (bl * bl < th2 * ns) {
                        const double r2 = ns + eps2, ri = 1.0 / sqrt(r2);
                        const double ri3 = ri * ri * ri, ri5 = ri3 * ri * ri, ri7 = ri5 * ri * ri;
                        const double *Q = &q[6 * c];
                        const double QR[3] = {Q[0] * R[0] + Q[1] * R[1] + Q[2] * R[2],
                                              Q[1] * R[0] + Q[3] * R[1] + Q[4] * R[2],
                                              Q[2] * R[0] + Q[4] * R[1] + Q[5] * R[2]};
                        const double RQR = R[0] * QR[0] + R[1] * QR[1] + R[2] * QR[2];
                        for (int k = 0; k < 3; ++k) {
                            const double tm = -t->mass[c] * ri3 * R[k];
                            const double tq = QR[k] * ri5 - 2.5 * RQR * R[k] * ri7;
                            acc[k] += G * (tm + tq);
                        }
                        mag += G * t->mass[c] * ri3 * sqrt(ns);
                        st[top].next++;
                        continue;
                    }
                }
                if (t->num_children[c] <= 0) {
                    for (int p = first; p < first + t->num_particles[c]; ++p) {
                        const int j = t->sorted_indices[p];
                        if (j == id) continue;
                        double R[3];
                        for (int k = 0; k < 3; ++k) R[k] = x[3 * id + k] - x[3 * j + k];
                        const double q2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
                        const double r2 = q2 + eps2, ri = 1.0 / sqrt(r2);
                        for (int k = 0; k < 3; ++k) acc[k] -= G * m[j] * ri * ri * ri * R[k];
                        mag += G * m[j] * ri * ri * ri * sqrt(q2);
                    }
                    st[top].next++;
                    continue;
                }
                ++top;
                st[top].node = c; st[top].next = 0;
                ++level;
                continue;
            }
            if (top == 0) break;
            --top;
            st[top].next++;
            --level;
        }
        for (int k = 0; k < 3; ++k) a[3 * id + k] = acc[k];
        if (absum) absum[id] = mag;
    }
}

int orc_barnes_hut(int n, const double *x, const double *m, double G,
                   double eps, double theta, int leaf_max, int compat,
                   double *a)
{
    OrcTree t;
    int rc = orc_build_tree(n, x, m, leaf_max, compat, &t);
    if (rc == 0) orc_bh_walk(n, x, m, G, eps, theta, &t, compat, a, NULL, NULL);
    orc_free_tree(&t);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Integrators                                                          */
/* ------------------------------------------------------------------ */

void orc_comp_update(int len, double *y, double *err, const double *d,
                     double dt)
{
    for (int k = 0; k < len; ++k) {
        const double y0 = y[k];
        err[k] += d[k] * dt;
        y[k] = y0 + err[k];
        err[k] += y0 - y[k];
    }
}

/* Barnes-Hut parameters of method 3 (src/acceleration.h:16-26: opening
 * angle, particles per leaf) for orc_fixed_step_run, and whether the tree
 * keeps the reference's quirks Q1/Q2 (compat) or computes true leaf
 * multipoles. */
static double g_bh_theta = 0.5;
static int g_bh_leaf = 1, g_bh_compat = 0;

void orc_set_bh_params(double theta, int leaf_max, int compat)
{
    g_bh_theta = theta;
    g_bh_leaf = leaf_max;
    g_bh_compat = compat;
}

static int accel_of(int method, int n, const double *x, const double *m,
                    double G, double eps, double *a)
{
    if (method == 1) { orc_pairwise(n, x, m, G, eps, a); return 0; }
    if (method == 2) return orc_massless(n, x, m, G, eps, a);
    if (method == 3)
        return orc_barnes_hut(n, x, m, G, eps, g_bh_theta, g_bh_leaf, g_bh_compat, a);
    return 2;
}

/* src/integrator.c:281-454 (euler), :456-628 (euler_cromer),
 * :630-892 (rk4), :894-1121 (leapfrog). */
int orc_fixed_step_run(int integrator, int method, int n, double *x, double *v,
                       const double *m, double G, double eps, double dt,
                       double tf)
{
    const int L = 3 * n;
    double *a = (double *)calloc((size_t)L * 11 + 1, sizeof(double));
    if (!a) return 4;
    double *xe = a + L, *ve = a + 2 * L, *x0 = a + 3 * L, *v0 = a + 4 * L;
    double *k1 = a + 5 * L, *k2 = a + 6 * L, *k3 = a + 7 * L, *k4 = a + 8 * L;
    double *vk = a + 9 * L, *tmp = a + 10 * L;
    (void)tmp;
    int rc = 0;
    const int64_t steps = (int64_t)ceil(tf / dt);
    double t = 0.0;
    double h = dt;
    if (integrator == 4) {
        if ((rc = accel_of(method, n, x, m, G, eps, a))) goto done;
        for (int k = 0; k < L; ++k) {
            const double y0 = v[k];
            ve[k] += 0.5 * a[k] * h;
            v[k] = y0 + ve[k];
            ve[k] += y0 - v[k];
        }
    }
    for (int64_t s = 0; s < steps; ++s) {
        if (integrator != 3 && t + h > tf) h = tf - t;
        if (integrator == 1) {
            memcpy(x0, x, sizeof(double) * L);
            memcpy(v0, v, sizeof(double) * L);
            if ((rc = accel_of(method, n, x, m, G, eps, a))) goto done;
            for (int k = 0; k < L; ++k) {
                xe[k] += v[k] * h;
                ve[k] += a[k] * h;
                x[k] = x0[k] + xe[k];
                v[k] = v0[k] + ve[k];
                xe[k] += x0[k] - x[k];
                ve[k] += v0[k] - v[k];
            }
        } else if (integrator == 2) {
            /* src/integrator.c:557-569: kick v with a(x), then drift x with
             * the new v, both compensated. */
            if ((rc = accel_of(method, n, x, m, G, eps, a))) goto done;
            orc_comp_update(L, v, ve, a, h);
            orc_comp_update(L, x, xe, v, h);
        } else if (integrator == 3) {
            memcpy(x0, x, sizeof(double) * L);
            memcpy(v0, v, sizeof(double) * L);
            if ((rc = accel_of(method, n, x, m, G, eps, k1))) goto done;
            memcpy(vk, v, sizeof(double) * L);                 /* xk1 */
            double *xk1 = vk;
            double *xk2 = (double *)malloc(sizeof(double) * (size_t)L * 3);
            if (!xk2) { rc = 4; goto done; }
            double *xk3 = xk2 + L, *xk4 = xk2 + 2 * L;
            for (int k = 0; k < L; ++k) {
                x[k] = x0[k] + 0.5 * xk1[k] * h;
                v[k] = v0[k] + 0.5 * k1[k] * h;
            }
            if ((rc = accel_of(method, n, x, m, G, eps, k2))) { free(xk2); goto done; }
            memcpy(xk2, v, sizeof(double) * L);
            for (int k = 0; k < L; ++k) {
                x[k] = x0[k] + 0.5 * xk2[k] * h;
                v[k] = v0[k] + 0.5 * k2[k] * h;
            }
            if ((rc = accel_of(method, n, x, m, G, eps, k3))) { free(xk2); goto done; }
            memcpy(xk3, v, sizeof(double) * L);
            for (int k = 0; k < L; ++k) {
                x[k] = x0[k] + xk3[k] * h;
                v[k] = v0[k] + k3[k] * h;
            }
            if ((rc = accel_of(method, n, x, m, G, eps, k4))) { free(xk2); goto done; }
            memcpy(xk4, v, sizeof(double) * L);
            for (int k = 0; k < L; ++k) {
                ve[k] += (k1[k] + 2 * k2[k] + 2 * k3[k] + k4[k]) * h / 6.0;
                xe[k] += (xk1[k] + 2 * xk2[k] + 2 * xk3[k] + xk4[k]) * h / 6.0;
                v[k] = v0[k] + ve[k];
                x[k] = x0[k] + xe[k];
                ve[k] += v0[k] - v[k];
                xe[k] += x0[k] - x[k];
            }
            free(xk2);
        } else if (integrator == 4) {
            orc_comp_update(L, x, xe, v, h);
            if ((rc = accel_of(method, n, x, m, G, eps, a))) goto done;
            orc_comp_update(L, v, ve, a, h);
        } else {
            rc = 2;
            goto done;
        }
        t = (double)(s + 1) * h;
    }
    if (integrator == 4) {
        for (int k = 0; k < L; ++k) v[k] -= 0.5 * a[k] * h;
    }
done:
    free(a);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Embedded Runge-Kutta (src/integrator_rk_embedded.c)                  */
/* ------------------------------------------------------------------ */

/* The published tableaus as exact rationals {p, q}: the stage matrix as its
 * lower triangle, row s (s = 1..S-1) holding a[s][0..s-1], then the weights
 * b[0..S-1] and the comparison weights bt[0..S-1].  Every quotient rounds
 * to the same double whether formed in double or long double. */
typedef struct { int p, q; } OrcQ;
typedef struct { int stages, power, power_test; const OrcQ *a, *b, *bt; } OrcTableau;

static const OrcQ rkf45_a[] = {
    {1, 4},
    {3, 32}, {9, 32},
    {1932, 2197}, {-7200, 2197}, {7296, 2197},
    {439, 216}, {-8, 1}, {3680, 513}, {-845, 4104},
    {-8, 27}, {2, 1}, {-3544, 2565}, {1859, 4104}, {-11, 40}};
static const OrcQ rkf45_b[] = {{25, 216}, {0, 1}, {1408, 2565}, {2197, 4104}, {-1, 5}, {0, 1}};
static const OrcQ rkf45_bt[] = {{16, 135}, {0, 1}, {6656, 12825}, {28561, 56430}, {-9, 50}, {2, 55}};

static const OrcQ dopri_a[] = {
    {1, 5},
    {3, 40}, {9, 40},
    {44, 45}, {-56, 15}, {32, 9},
    {19372, 6561}, {-25360, 2187}, {64448, 6561}, {-212, 729},
    {9017, 3168}, {-355, 33}, {46732, 5247}, {49, 176}, {-5103, 18656},
    {35, 384}, {0, 1}, {500, 1113}, {125, 192}, {-2187, 6784}, {11, 84}};
static const OrcQ dopri_b[] = {{35, 384}, {0, 1}, {500, 1113}, {125, 192}, {-2187, 6784},
                               {11, 84}, {0, 1}};
static const OrcQ dopri_bt[] = {{5179, 57600}, {0, 1}, {7571, 16695}, {393, 640},
                                {-92097, 339200}, {187, 2100}, {1, 40}};

static const OrcQ dverk_a[] = {
    {1, 6},
    {4, 75}, {16, 75},
    {5, 6}, {-8, 3}, {5, 2},
    {-165, 64}, {55, 6}, {-425, 64}, {85, 96},
    {12, 5}, {-8, 1}, {4015, 612}, {-11, 36}, {88, 255},
    {-8263, 15000}, {124, 75}, {-643, 680}, {-81, 250}, {2484, 10625}, {0, 1},
    {3501, 1720}, {-300, 43}, {297275, 52632}, {-319, 2322}, {24068, 84065}, {0, 1},
    {3850, 26703}};
static const OrcQ dverk_b[] = {{3, 40}, {0, 1}, {875, 2244}, {23, 72}, {264, 1955}, {0, 1},
                               {125, 11592}, {43, 616}};
static const OrcQ dverk_bt[] = {{13, 160}, {0, 1}, {2375, 5984}, {5, 16}, {12, 85}, {3, 44},
                                {0, 1}, {0, 1}};

static const OrcQ rkf78_a[] = {
    {2, 27},
    {1, 36}, {1, 12},
    {1, 24}, {0, 1}, {1, 8},
    {5, 12}, {0, 1}, {-25, 16}, {25, 16},
    {1, 20}, {0, 1}, {0, 1}, {1, 4}, {1, 5},
    {-25, 108}, {0, 1}, {0, 1}, {125, 108}, {-65, 27}, {125, 54},
    {31, 300}, {0, 1}, {0, 1}, {0, 1}, {61, 225}, {-2, 9}, {13, 900},
    {2, 1}, {0, 1}, {0, 1}, {-53, 6}, {704, 45}, {-107, 9}, {67, 90}, {3, 1},
    {-91, 108}, {0, 1}, {0, 1}, {23, 108}, {-976, 135}, {311, 54}, {-19, 60}, {17, 6},
    {-1, 12},
    {2383, 4100}, {0, 1}, {0, 1}, {-341, 164}, {4496, 1025}, {-301, 82}, {2133, 4100},
    {45, 82}, {45, 164}, {18, 41},
    {3, 205}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {-6, 41}, {-3, 205}, {-3, 41}, {3, 41},
    {6, 41}, {0, 1},
    {-1777, 4100}, {0, 1}, {0, 1}, {-341, 164}, {4496, 1025}, {-289, 82}, {2193, 4100},
    {51, 82}, {33, 164}, {19, 41}, {0, 1}, {1, 1}};
static const OrcQ rkf78_b[] = {{41, 840}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {34, 105}, {9, 35},
                               {9, 35}, {9, 280}, {9, 280}, {41, 840}, {0, 1}, {0, 1}};
static const OrcQ rkf78_bt[] = {{0, 1}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {34, 105}, {9, 35},
                                {9, 35}, {9, 280}, {9, 280}, {0, 1}, {41, 840}, {41, 840}};

/* integrator codes 5..8 (src/integrator_rk_embedded.c:36-58) */
static const OrcTableau *orc_tableau(int integrator)
{
    static const OrcTableau t[4] = {
        {6, 4, 5, rkf45_a, rkf45_b, rkf45_bt},
        {7, 5, 4, dopri_a, dopri_b, dopri_bt},
        {8, 6, 7, dverk_a, dverk_b, dverk_bt},
        {13, 7, 8, rkf78_a, rkf78_b, rkf78_bt}};
    return (integrator >= 5 && integrator <= 8) ? &t[integrator - 5] : NULL;
}

static double qv(OrcQ r) { return (double)r.p / (double)r.q; }

/* :346-520, including the long double intermediates and the branch whose
 * result is always overwritten (:496-501). */
static int rk_initial_dt(int method, int n, const double *x, const double *v, const double *m,
                         double G, double eps, double rel_tol, double abs_tol, int power,
                         double *dt_out)
{
    const int L = 3 * n;
    double *buf = (double *)malloc(sizeof(double) * (size_t)L * 6);
    if (!buf) return 4;
    double *sx = buf, *sv = buf + L, *x1 = buf + 2 * L, *v1 = buf + 3 * L, *a1 = buf + 4 * L,
           *a = buf + 5 * L;
    int rc = accel_of(method, n, x, m, G, eps, a);
    if (rc) { free(buf); return rc; }
    for (int k = 0; k < L; ++k) {
        sx[k] = abs_tol + rel_tol * fabs(x[k]);
        sv[k] = abs_tol + rel_tol * fabs(v[k]);
    }
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = 0; k < L; ++k) {
        s0 += (x[k] / sx[k]) * (x[k] / sx[k]);
        s0 += (v[k] / sv[k]) * (v[k] / sv[k]);
        s1 += (v[k] / sx[k]) * (v[k] / sx[k]);
        s1 += (a[k] / sv[k]) * (a[k] / sv[k]);
    }
    const double d0 = sqrt(s0 / (n * 6));
    const double d1 = sqrt(s1 / (n * 6));
    const double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-4 : d0 / d1;
    for (int k = 0; k < L; ++k) {
        x1[k] = x[k] + (dt0 / 100.0) * v[k];
        v1[k] = v[k] + (dt0 / 100.0) * a[k];
    }
    rc = accel_of(method, n, x1, m, G, eps, a1);
    if (rc) { free(buf); return rc; }
    for (int k = 0; k < L; ++k) {
        s2 += ((v1[k] - v[k]) / sx[k]) * ((v1[k] - v[k]) / sx[k]);
        s2 += ((a1[k] - a[k]) / sv[k]) * ((a1[k] - a[k]) / sv[k]);
    }
    const double d2 = sqrt(s2 / (n * 6)) / dt0;
    const double dt1 = pow((double)(0.01L / (long double)fmax(d1, d2)),
                           (double)(1.0L / (long double)(1 + power)));
    const double dt = fmin((double)(100.0L * (long double)dt0), dt1);
    free(buf);
    *dt_out = dt * 1e-2;
    return *dt_out > 0.0 ? 0 : 2;
}

int orc_rk_embedded_run(int integrator, int method, int n, double *x, double *v,
                        const double *m, double G, double eps, double tolerance,
                        double initial_dt, double tf, int64_t *num_steps, double *t_out,
                        double *dt_out)
{
    const OrcTableau *T = orc_tableau(integrator);
    if (!T) return 2;
    const int S = T->stages, L = 3 * n;
    const int min_power = T->power < T->power_test ? T->power : T->power_test;
    double a[13][12], w[13], dw[13];
    int off = 0;
    for (int s = 1; s < S; ++s)
        for (int i = 0; i < s; ++i) a[s][i] = qv(T->a[off++]);
    for (int s = 0; s < S; ++s) {
        w[s] = qv(T->b[s]);
        dw[s] = w[s] - qv(T->bt[s]);
    }
    const double abs_tol = tolerance, rel_tol = tolerance;
    const double fac_max = 6.0, fac_min = 0.33;
    const double fac = pow(0.38, 1.0 / (1.0 + (double)min_power));
    double *buf = (double *)calloc((size_t)L * (2 * (size_t)S + 12), sizeof(double));
    if (!buf) return 4;
    double *vk = buf, *xk = buf + (size_t)S * L, *p = buf + 2 * (size_t)S * L;
    double *x1 = p, *v1 = p + L, *tv = p + 2 * L, *tx = p + 3 * L, *dv = p + 4 * L,
           *dx = p + 5 * L, *xe = p + 8 * L, *ve = p + 9 * L, *txe = p + 10 * L,
           *tve = p + 11 * L;
    int rc = 0;
    double dt;
    if (initial_dt > 0.0) {
        dt = initial_dt;
    } else {
        if ((rc = rk_initial_dt(method, n, x, v, m, G, eps, rel_tol, abs_tol, T->power, &dt)))
            goto done;
        if (dt > tf) dt = tf;
    }
    double t = 0.0;
    int64_t steps = 0;
    while (t < tf) {
        /* stages (:721-777) */
        if ((rc = accel_of(method, n, x, m, G, eps, vk))) goto done;
        memcpy(xk, v, sizeof(double) * L);
        for (int s = 1; s < S; ++s) {
            for (int k = 0; k < L; ++k) { tv[k] = 0.0; tx[k] = 0.0; }
            for (int i = 0; i < s; ++i)
                for (int k = 0; k < L; ++k) {
                    tv[k] += a[s][i] * vk[(size_t)i * L + k];
                    tx[k] += a[s][i] * xk[(size_t)i * L + k];
                }
            for (int k = 0; k < L; ++k) {
                tv[k] = v[k] + dt * tv[k] + ve[k];
                tx[k] = x[k] + dt * tx[k] + xe[k];
            }
            if ((rc = accel_of(method, n, tx, m, G, eps, vk + (size_t)s * L))) goto done;
            memcpy(xk + (size_t)s * L, tv, sizeof(double) * L);
        }
        /* weights, error deltas, compensated x1 / v1 (:779-830) */
        for (int k = 0; k < L; ++k) { tv[k] = tx[k] = dv[k] = dx[k] = 0.0; }
        for (int s = 0; s < S; ++s)
            for (int k = 0; k < L; ++k) {
                tv[k] += w[s] * vk[(size_t)s * L + k];
                tx[k] += w[s] * xk[(size_t)s * L + k];
                dv[k] += dt * dw[s] * vk[(size_t)s * L + k];
                dx[k] += dt * dw[s] * xk[(size_t)s * L + k];
            }
        memcpy(txe, xe, sizeof(double) * L);
        memcpy(tve, ve, sizeof(double) * L);
        for (int k = 0; k < L; ++k) {
            tve[k] += dt * tv[k];
            txe[k] += dt * tx[k];
            v1[k] = v[k] + tve[k];
            x1[k] = x[k] + txe[k];
            tve[k] += v[k] - v1[k];
            txe[k] += x[k] - x1[k];
        }
        /* RMS of the scaled error (:832-856) */
        double sum = 0.0;
        for (int k = 0; k < L; ++k) {
            const double sv = abs_tol + fmax(fabs(v[k]), fabs(v1[k])) * rel_tol;
            const double sx = abs_tol + fmax(fabs(x[k]), fabs(x1[k])) * rel_tol;
            double q = dv[k] / sv;
            sum += q * q;
            q = dx[k] / sx;
            sum += q * q;
        }
        double error = sqrt(sum / (n * 3 * 2));
        /* accept (:859-888) and step-size control (:895-923) */
        if (error <= 1 || dt <= tf * 1e-12) {
            ++steps;
            t += dt;
            memcpy(x, x1, sizeof(double) * L);
            memcpy(v, v1, sizeof(double) * L);
            memcpy(xe, txe, sizeof(double) * L);
            memcpy(ve, tve, sizeof(double) * L);
        }
        if (error < 1e-10) error = 1e-10;
        const double dt_new = dt * fac / pow(error, 1.0 / (1.0 + (double)min_power));
        if (dt_new > fac_max * dt) dt *= fac_max;
        else if (dt_new < fac_min * dt) dt *= fac_min;
        else dt = dt_new;
        if (dt_new / tf < 1e-12) dt = tf * 1e-12;
        if (t < tf && t + dt > tf) dt = tf - t;
    }
    if (num_steps) *num_steps = steps;
    if (t_out) *t_out = t;
    if (dt_out) *dt_out = dt;
done:
    free(buf);
    return rc;
}

/* ------------------------------------------------------------------ */
/* IAS15 (src/integrator_ias15.c)                                       */
/* ------------------------------------------------------------------ */

/* The method's constants (Gauss-Radau spacings and the c / r coefficient
 * tables of src/integrator_ias15.c:617-700) as exact doubles; each rounds the
 * same from its decimal form in double or long double. */
/* Gauss-Radau spacings h_0..h_7 */
static const double kRadauH[8] = {0.0, 0x1.cce7242fd9812p-5, 0x1.7122082358d27p-3, 0x1.6916742f0c9c5p-2, 0x1.18248525f4802p-1, 0x1.77ea65770fa49p-1, 0x1.c548c982467cdp-1, 0x1.f47d94f4d2bb2p-1};
/* c[i][j] (j <= i): b from g */
static const double kRadauC[7][7] = {
    {0x1.0000000000000p+0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.cce7242fd9812p-5, 0x1.0000000000000p+0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.4c4b384151c1ep-7, -0x1.e45bd12f4f32cp-3, 0x1.0000000000000p+0, 0.0, 0.0, 0.0, 0.0},
    {-0x1.d4b3379a1992dp-9, 0x1.7f2161e152586p-4, -0x1.2da22e635a1aep-1, 0x1.0000000000000p+0, 0.0, 0.0, 0.0},
    {0x1.007370e57b89dp-9, -0x1.c08e5e7efcf23p-5, 0x1.a9dcc2e57fbbfp-2, -0x1.22e359c4a74d8p+0, 0x1.0000000000000p+0, 0.0, 0.0},
    {-0x1.7893e98a2a997p-10, 0x1.595cd739ee74fp-5, -0x1.70bdf2d91dd44p-2, 0x1.4009e0866d488p+0, -0x1.ded88c802f1fcp+0, 0x1.0000000000000p+0, 0.0},
    {0x1.4d64672378b3dp-10, -0x1.3d865cb429919p-5, 0x1.71a0161ae20fep-2, -0x1.7785b93619434p+0, 0x1.73fc45dfb9889p+1, -0x1.60be78a0a92f1p+1, 0x1.0000000000000p+0}};
/* r[i][j] = 1 / (h_i - h_j) (j < i): g from the accelerations */
static const double kRadauR[8][8] = {
    {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.1c618574b517bp+4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.6314ac07f6a9ap+2, 0x1.021c2b5e4af6fp+3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.6afdfcc2a4aefp+1, 0x1.afe76c59caa8ap+1, 0x1.73439c0b4562bp+2, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0x1.d3e03b89d73cfp+0, 0x1.04c014a3946fbp+1, 0x1.5cdb4a576d57ap+1, 0x1.48fffc3fdf2e6p+2, 0.0, 0.0, 0.0, 0.0},
    {0x1.5cac8b52e27b1p+0, 0x1.799c3c56b4e9dp+0, 0x1.ce1e8b86f5ae8p+0, 0x1.4f714afea15ccp+1, 0x1.56247c4b878b4p+2, 0.0, 0.0, 0.0},
    {0x1.212921ce4baffp+0, 0x1.34c8b7028f418p+0, 0x1.6b1448c75e4d5p+0, 0x1.e092f6d7c8a42p+0, 0x1.7a82c7145ec17p+1, 0x1.a787c6413556bp+2, 0.0, 0.0},
    {0x1.05e3166485188p+0, 0x1.15e18175af101p+0, 0x1.41177c7d3aff5p+0, 0x1.99ab118ef2216p+0, 0x1.296bab4a3e0d2p+1, 0x1.0709d7d8d5e3cp+2, 0x1.5b12a584540e2p+3, 0.0}};


static double absmax(const double *v, int len)
{
    double mx = fabs(v[0]);
    for (int i = 1; i < len; ++i) mx = fmax(mx, fabs(v[i]));
    return mx;
}

/* :808-919, predictor at spacing h */
static void ias_predict(int L, double *x1, double *v1, const double *x0, const double *v0,
                        const double *a0, double h, const double *b, double dt,
                        const double *xe, const double *ve)
{
    for (int k = 0; k < L; ++k) {
        const double *bk = b + k;
        const double dth = dt * h;
        double p = bk[5 * L] / 28.0 + h * bk[6 * L] / 36.0;
        p = bk[4 * L] / 21.0 + h * p;
        p = bk[3 * L] / 15.0 + h * p;
        p = bk[2 * L] / 10.0 + h * p;
        p = bk[1 * L] / 6.0 + h * p;
        p = bk[0] / 3.0 + h * p;
        x1[k] = x0[k];
        x1[k] += xe[k] + dth * (v0[k] + dth * (a0[k] + h * p) / 2.0);
        double q = bk[5 * L] / 7.0 + h * bk[6 * L] / 8.0;
        q = bk[4 * L] / 6.0 + h * q;
        q = bk[3 * L] / 5.0 + h * q;
        q = bk[2 * L] / 4.0 + h * q;
        q = bk[1 * L] / 3.0 + h * q;
        q = bk[0] / 2.0 + h * q;
        v1[k] = v0[k];
        v1[k] += ve[k] + dth * (a0[k] + h * q);
    }
}

/* :921-983, end of the step with compensated sums */
static void ias_advance(int L, double *x1, double *v1, double *txe, double *tve, const double *x0,
                        const double *v0, const double *a0, const double *b, double dt)
{
    for (int k = 0; k < L; ++k) {
        const double *bk = b + k;
        const double sx = a0[k] + bk[0] / 3.0 + bk[1 * L] / 6.0 + bk[2 * L] / 10.0 +
                          bk[3 * L] / 15.0 + bk[4 * L] / 21.0 + bk[5 * L] / 28.0 + bk[6 * L] / 36.0;
        txe[k] += dt * (v0[k] + dt * sx / 2.0);
        x1[k] = x0[k] + txe[k];
        txe[k] += x0[k] - x1[k];
        const double sv = a0[k] + bk[0] / 2.0 + bk[1 * L] / 3.0 + bk[2 * L] / 4.0 + bk[3 * L] / 5.0 +
                          bk[4 * L] / 6.0 + bk[5 * L] / 7.0 + bk[6 * L] / 8.0;
        tve[k] += dt * sv;
        v1[k] = v0[k] + tve[k];
        tve[k] += v0[k] - v1[k];
    }
}

/* :1117-1274 (g from the accelerations F at spacings 0..i) and :985-1115
 * (b from g), element by element */
static void ias_update_gb(int L, double *g, double *b, const double *F, int i)
{
    for (int k = 0; k < L; ++k) {
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
}

/* :1276-1382 */
static void ias_refine(int L, double *b, double *e, double *db, double q, int refine)
{
    const double q2 = q * q, q3 = q2 * q, q4 = q3 * q, q5 = q4 * q, q6 = q5 * q, q7 = q6 * q;
    for (size_t k = 0; k < (size_t)7 * L; ++k) db[k] = refine ? b[k] - e[k] : 0.0;
    for (int k = 0; k < L; ++k) {
        const double b0 = b[k], b1 = b[L + k], b2 = b[2 * L + k], b3 = b[3 * L + k],
                     b4 = b[4 * L + k], b5 = b[5 * L + k], b6 = b[6 * L + k];
        e[k] = q * (b6 * 7.0 + b5 * 6.0 + b4 * 5.0 + b3 * 4.0 + b2 * 3.0 + b1 * 2.0 + b0);
        e[L + k] = q2 * (b6 * 21.0 + b5 * 15.0 + b4 * 10.0 + b3 * 6.0 + b2 * 3.0 + b1);
        e[2 * L + k] = q3 * (b6 * 35.0 + b5 * 20.0 + b4 * 10.0 + b3 * 4.0 + b2);
        e[3 * L + k] = q4 * (b6 * 35.0 + b5 * 15.0 + b4 * 5.0 + b3);
        e[4 * L + k] = q5 * (b6 * 21.0 + b5 * 6.0 + b4);
        e[5 * L + k] = q6 * (b6 * 7.0 + b5);
        e[6 * L + k] = q7 * b6;
    }
    for (size_t k = 0; k < (size_t)7 * L; ++k) b[k] = e[k] + db[k];
}

int orc_ias15_run(int method, int n, double *x, double *v, const double *m, double G, double eps,
                  double tolerance, double initial_dt, double tf, int64_t *num_steps,
                  double *t_out, double *dt_out)
{
    const int L = 3 * n;
    const size_t SL = (size_t)L;
    double *buf = (double *)calloc(SL * (7 * 5 + 8 + 10), sizeof(double));
    if (!buf) return 4;
    double *b0 = buf, *b = b0 + 7 * SL, *g = b + 7 * SL, *e = g + 7 * SL, *db = e + 7 * SL;
    double *F = db + 7 * SL;   /* 8 * L */
    double *a = F + 8 * SL, *x1 = a + SL, *v1 = x1 + SL, *a1 = v1 + SL, *d7 = a1 + SL,
           *xe = d7 + SL, *ve = xe + SL, *txe = ve + SL, *tve = txe + SL;
    double *tmp = tve + SL;
    int rc = accel_of(method, n, x, m, G, eps, a);
    if (rc) goto done;
    double dt;
    if (initial_dt > 0.0) {
        dt = initial_dt;
    } else {
        /* :702-806, power 15 */
        const double d0 = absmax(x, L), d1 = absmax(a, L);
        const double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
        for (int k = 0; k < L; ++k) tmp[k] = x[k] + dt0 * v[k];
        if ((rc = accel_of(method, n, tmp, m, G, eps, a1))) goto done;
        for (int k = 0; k < L; ++k) a1[k] = a1[k] - a[k];
        const double d2 = absmax(a1, L) / dt0;
        double dt1;
        if (fmax(d1, d2) <= 1e-15)
            dt1 = fmax(1e-6, dt0 * 1e-3);
        else
            dt1 = pow((0.01 / fmax(d1, d2)), 1.0 / (1.0 + (double)15));
        dt = fmin(100.0 * dt0, dt1);
        if (dt <= 0.0) { rc = 2; goto done; }
        if (dt > tf) dt = tf;
    }
    {
        double t = 0.0, dt_new;
        int64_t steps = 0;
        int refine = 0;
        while (t < tf) {
            for (int it = 0; it < 12; ++it) {
                for (int i = 0; i < 8; ++i) {
                    ias_predict(L, x1, v1, x, v, a, kRadauH[i], b, dt, xe, ve);
                    if ((rc = accel_of(method, n, x1, m, G, eps, F + (size_t)i * SL))) goto done;
                    ias_update_gb(L, g, b, F, i);
                }
                for (int k = 0; k < L; ++k) d7[k] = b[6 * SL + k] - b0[6 * SL + k];
                memcpy(b0, b, sizeof(double) * 7 * SL);
                if ((absmax(d7, L) / absmax(F + 7 * SL, L)) < 1e-16) break;
            }
            memcpy(txe, xe, sizeof(double) * SL);
            memcpy(tve, ve, sizeof(double) * SL);
            ias_advance(L, x1, v1, txe, tve, x, v, a, b, dt);
            if ((rc = accel_of(method, n, x1, m, G, eps, a1))) goto done;
            const double eb7 = absmax(b + 6 * SL, L) / absmax(a1, L);
            double err = pow((eb7 / tolerance), 1.0 / 7.0);
            if (err < 1e-10) err = 1e-10;
            dt_new = dt / err;
            if (err <= 1.0 || dt == tf * 1e-12) {
                ++steps;
                t += dt;
                ias_refine(L, b, e, db, dt_new / dt, refine);
                refine = 1;
                memcpy(xe, txe, sizeof(double) * SL);
                memcpy(ve, tve, sizeof(double) * SL);
                memcpy(x, x1, sizeof(double) * SL);
                memcpy(v, v1, sizeof(double) * SL);
                memcpy(a, a1, sizeof(double) * SL);
            }
            if (dt_new > (dt / 0.25)) dt /= 0.25;
            else if (dt_new < dt * 0.25) dt *= 0.25;
            else dt = dt_new;
            if (dt_new < tf * 1e-12) dt = tf * 1e-12;
            if (t < tf && t + dt > tf) dt = tf - t;
        }
        if (num_steps) *num_steps = steps;
        if (t_out) *t_out = t;
        if (dt_out) *dt_out = dt;
    }
done:
    free(buf);
    return rc;
}

/* ------------------------------------------------------------------ */
/* WHFast (src/integrator_whfast.c)                                     */
/* ------------------------------------------------------------------ */

static double norm3v(const double *p)
{
    return sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
}

typedef struct { double d; int i; } OrcDist;

static int cmp_dist(const void *a, const void *b)
{
    const OrcDist *p = (const OrcDist *)a, *q = (const OrcDist *)b;
    if (p->d < q->d) return -1;
    if (p->d > q->d) return 1;
    return (p->i > q->i) - (p->i < q->i);   /* ties: array order */
}

/* src/system.c:1210-1335: order particles by |x_i - x_primary| (primary's
 * distance forced to 0), permuting ids, the given vectors and m. */
static int sort_by_distance(int n, int *ids, double *xa, double *va, double *m)
{
    int prim = -1;
    if (0 < n && ids[0] == 0) prim = 0;
    else for (int i = 0; i < n; ++i) if (ids[i] == 0) { prim = i; break; }
    if (prim < 0) return 2;
    OrcDist *h = (OrcDist *)malloc(sizeof(OrcDist) * (size_t)n);
    int *ni = (int *)malloc(sizeof(int) * (size_t)n);
    double *nx = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *nv = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *nm = (double *)malloc(sizeof(double) * (size_t)n);
    if (!h || !ni || !nx || !nv || !nm) { free(h); free(ni); free(nx); free(nv); free(nm); return 4; }
    for (int i = 0; i < n; ++i) {
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = xa[3 * i + k] - xa[3 * prim + k];
        h[i].d = norm3v(d);
        h[i].i = i;
    }
    h[prim].d = 0.0;
    qsort(h, (size_t)n, sizeof(OrcDist), cmp_dist);
    for (int i = 0; i < n; ++i) {
        const int j = h[i].i;
        ni[i] = ids[j];
        for (int k = 0; k < 3; ++k) { nx[3 * i + k] = xa[3 * j + k]; nv[3 * i + k] = va[3 * j + k]; }
        nm[i] = m[j];
    }
    memcpy(ids, ni, sizeof(int) * (size_t)n);
    memcpy(xa, nx, sizeof(double) * 3 * (size_t)n);
    memcpy(va, nv, sizeof(double) * 3 * (size_t)n);
    memcpy(m, nm, sizeof(double) * (size_t)n);
    free(h); free(ni); free(nx); free(nv); free(nm);
    return 0;
}

/* :1266-1279 */
static void wh_eta(int n, const double *m, double *eta)
{
    eta[0] = m[0];
    for (int i = 1; i < n; ++i) eta[i] = eta[i - 1] + m[i];
}

/* :682-724 */
static void wh_cart_to_jac(int n, const double *x, const double *v, const double *m,
                           const double *eta, double *jx, double *jv)
{
    double xc[3], vc[3];
    for (int k = 0; k < 3; ++k) { xc[k] = m[0] * x[k]; vc[k] = m[0] * v[k]; }
    for (int i = 1; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            jx[3 * i + k] = x[3 * i + k] - xc[k] / eta[i - 1];
            jv[3 * i + k] = v[3 * i + k] - vc[k] / eta[i - 1];
            xc[k] = xc[k] * (1.0 + m[i] / eta[i - 1]) + m[i] * jx[3 * i + k];
            vc[k] = vc[k] * (1.0 + m[i] / eta[i - 1]) + m[i] * jv[3 * i + k];
        }
    }
    for (int k = 0; k < 3; ++k) {
        jx[k] = xc[k] / eta[n - 1];
        jv[k] = vc[k] / eta[n - 1];
    }
}

/* :726-772 */
static void wh_jac_to_cart(int n, const double *jx, const double *jv, const double *m,
                           const double *eta, double *x, double *v)
{
    double xc[3], vc[3];
    for (int k = 0; k < 3; ++k) { xc[k] = eta[n - 1] * jx[k]; vc[k] = eta[n - 1] * jv[k]; }
    for (int i = n - 1; i > 0; --i) {
        for (int k = 0; k < 3; ++k) {
            xc[k] = (xc[k] - m[i] * jx[3 * i + k]) / eta[i];
            vc[k] = (vc[k] - m[i] * jv[3 * i + k]) / eta[i];
            x[3 * i + k] = jx[3 * i + k] + xc[k];
            v[3 * i + k] = jv[3 * i + k] + vc[k];
            xc[k] = eta[i - 1] * xc[k];
            vc[k] = eta[i - 1] * vc[k];
        }
    }
    for (int k = 0; k < 3; ++k) { x[k] = xc[k] / m[0]; v[k] = vc[k] / m[0]; }
}

/* :774-815 */
static void stumpff(double z, double *c0, double *c1, double *c2, double *c3)
{
    int q = 0;
    while (fabs(z) > 0.1) { z /= 4.0; ++q; }
    double s3 = (1.0 - z / 20.0 * (1.0 - z / 42.0 * (1.0 - z / 72.0 * (1.0 - z / 110.0
                 * (1.0 - z / 156.0 * (1.0 - z / 210.0)))))) / 6.0;
    double s2 = (1.0 - z / 12.0 * (1.0 - z / 30.0 * (1.0 - z / 56.0 * (1.0 - z / 90.0
                 * (1.0 - z / 132.0 * (1.0 - z / 182.0)))))) / 2.0;
    double s1 = 1.0 - z * s3;
    double s0 = 1.0 - z * s2;
    while (q > 0) {
        s3 = (s2 + s0 * s3) / 4.0;
        s2 = (s1 * s1) / 2.0;
        s1 = s0 * s1;
        s0 = (2.0 * s0 * s0) - 1.0;
        --q;
    }
    *c0 = s0; *c1 = s1; *c2 = s2; *c3 = s3;
}

/* :424-600: universal-variable Kepler drift of Jacobi body i; returns
 * 1 when the particle is to be removed (not converged with error above
 * 1e-5, or non-finite argument), else 0. */
static int wh_drift_one(double *jx, double *jv, double gm, double dt)
{
    const double xx[3] = {jx[0], jx[1], jx[2]};
    const double vv[3] = {jv[0], jv[1], jv[2]};
    const double xn = norm3v(xx);
    const double vn = norm3v(vv);
    const double rv = (xx[0] * vv[0] + xx[1] * vv[1] + xx[2] * vv[2]) / xn;
    const double alpha = 2.0 * gm / xn - (vn * vn);
    double s = dt / xn;
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
    int conv = 0, bad_z = 0;
    for (int it = 0; it < 500; ++it) {
        const double z = alpha * (s * s);
        if (!isfinite(z)) { bad_z = 1; break; }
        stumpff(z, &c0, &c1, &c2, &c3);
        const double F = xn * s * c1 + xn * rv * (s * s) * c2 + gm * (s * s * s) * c3 - dt;
        const double dF = xn * c0 + xn * rv * s * c1 + gm * (s * s) * c2;
        const double ds = -F / dF;
        s += ds;
        if (fabs(ds) < 1e-12) { conv = 1; break; }
    }
    const double r = xn * c0 + xn * rv * s * c1 + gm * (s * s) * c2;
    int remove = 0;
    if (!conv) {
        const double err = (xn * s * c1 + xn * rv * (s * s) * c2 + gm * (s * s * s) * c3 - dt) / r;
        if (err > 1e-5 || bad_z) remove = 1;
    }
    const double f = 1.0 - gm * (s * s) * c2 / xn;
    const double g = dt - gm * (s * s * s) * c3;
    const double df = -gm * s * c1 / (r * xn);
    const double dg = 1.0 - gm * (s * s) * c2 / r;
    for (int k = 0; k < 3; ++k) {
        jx[k] = f * xx[k] + g * vv[k];
        jv[k] = df * xx[k] + dg * vv[k];
    }
    return remove;
}

/* :959-1264 (massless variant, aux taken as zero where the reference
 * reads it uninitialised) and :839-957 (pairwise variant). a[0] is 0. */
static int wh_accel(int n, const double *x, const double *jx, const double *m,
                    const double *eta, double G, double eps, int pairwise, double *a)
{
    const double e3 = eps * eps * eps;
    int *hv = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!hv) return 4;
    int nh = 0;
    for (int i = 0; i < n; ++i)
        if (pairwise || m[i] != 0.0) hv[nh++] = i;
    for (int k = 0; k < 3 * n; ++k) a[k] = 0.0;
    for (int i = 1; i < n; ++i) {
        const int massive = pairwise || m[i] != 0.0;
        double tv[3], aux[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 3; ++k) tv[k] = x[3 * i + k] - x[k];
        const double tn = norm3v(tv);
        const double tc = (tn * tn * tn) + e3;
        const double jn = norm3v(&jx[3 * i]);
        const double jc = (jn * jn * jn) + e3;
        for (int k = 0; k < 3; ++k) {
            const double pre = massive ? G * m[0] * eta[i] / eta[i - 1] : G * m[0];
            a[3 * i + k] = pre * (jx[3 * i + k] / jc - tv[k] / tc);
        }
        /* interior massive bodies j in (0, i) */
        for (int p = 1; p < nh && hv[p] < i; ++p) {
            const int j = hv[p];
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = x[3 * i + k] - x[3 * j + k];
            const double dn = norm3v(d);
            const double dc = (dn * dn * dn) + e3;
            for (int k = 0; k < 3; ++k) aux[k] += G * m[j] * d[k] / dc;
        }
        for (int k = 0; k < 3; ++k)
            a[3 * i + k] -= massive ? aux[k] * eta[i] / eta[i - 1] : aux[k];
        aux[0] = aux[1] = aux[2] = 0.0;
        /* exterior massive bodies */
        for (int p = 1; p < nh; ++p) {
            const int j = hv[p];
            if (j <= i) continue;
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = x[3 * j + k] - x[3 * i + k];
            const double dn = norm3v(d);
            const double dc = (dn * dn * dn) + e3;
            for (int k = 0; k < 3; ++k) aux[k] += G * m[j] * d[k] / dc;
        }
        for (int k = 0; k < 3; ++k) a[3 * i + k] += aux[k];
        aux[0] = aux[1] = aux[2] = 0.0;
        /* pairs (interior j incl. 0, exterior k) */
        for (int p = 0; p < nh && hv[p] < i; ++p) {
            const int j = hv[p];
            for (int q = p + 1; q < nh; ++q) {
                const int kk = hv[q];
                if (kk <= i) continue;
                double d[3];
                for (int k = 0; k < 3; ++k) d[k] = x[3 * kk + k] - x[3 * j + k];
                const double dn = norm3v(d);
                const double dc = (dn * dn * dn) + e3;
                for (int k = 0; k < 3; ++k) aux[k] += G * m[j] * m[kk] * d[k] / dc;
            }
        }
        for (int k = 0; k < 3; ++k) a[3 * i + k] -= aux[k] / eta[i - 1];
    }
    free(hv);
    return 0;
}

static void remove_rows(int n, const int *rm, int nrm, int width, double *arr)
{
    int w = 0, r = 0;
    for (int i = 0; i < n; ++i) {
        if (r < nrm && rm[r] == i) { ++r; continue; }
        for (int k = 0; k < width; ++k) arr[width * w + k] = arr[width * i + k];
        ++w;
    }
}

/* src/integrator_whfast.c:200-407 for one system; *n may shrink when
 * invalid particles are removed (remove_invalid != 0). */
int orc_whfast_run(int *n_io, int *ids, double *x, double *v, double *m, double G, double eps,
                   double dt, double tf, int remove_invalid, int pairwise)
{
    int n = *n_io;
    double *jx = (double *)calloc((size_t)n * 3, sizeof(double));
    double *jv = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *a = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *eta = (double *)malloc(sizeof(double) * (size_t)n);
    int *rm = (int *)malloc(sizeof(int) * (size_t)n);
    int rc = 0;
    if (!jx || !jv || !a || !eta || !rm) { rc = 4; goto out; }
    if ((rc = sort_by_distance(n, ids, x, v, m))) goto out;
    wh_eta(n, m, eta);
    wh_cart_to_jac(n, x, v, m, eta, jx, jv);
    if ((rc = wh_accel(n, x, jx, m, eta, G, eps, pairwise, a))) goto out;
    for (int k = 0; k < 3 * n; ++k) jv[k] += a[k] * (0.5 * dt);
    {
        const int64_t steps = (int64_t)ceil(tf / dt);
        double t = 0.0, h = dt;
        for (int64_t s = 0; s < steps; ++s) {
            if (t + h > tf) h = tf - t;
            if ((rc = sort_by_distance(n, ids, jx, jv, m))) goto out;
            wh_eta(n, m, eta);
            int nrm = 0;
            for (int i = 1; i < n; ++i) {
                const double gm = G * m[0] * eta[i] / eta[i - 1];
                if (wh_drift_one(&jx[3 * i], &jv[3 * i], gm, h) && remove_invalid) rm[nrm++] = i;
            }
            if (nrm > 0) {
                int *idsrc = ids;
                /* compact ids, cartesian x, v, m, then jx, jv (and eta) */
                int w = 0, r = 0;
                for (int i = 0; i < n; ++i) {
                    if (r < nrm && rm[r] == i) { ++r; continue; }
                    idsrc[w++] = idsrc[i];
                }
                remove_rows(n, rm, nrm, 3, x);
                remove_rows(n, rm, nrm, 3, v);
                remove_rows(n, rm, nrm, 1, m);
                remove_rows(n, rm, nrm, 3, jx);
                remove_rows(n, rm, nrm, 3, jv);
                n -= nrm;
                wh_eta(n, m, eta);
            }
            wh_jac_to_cart(n, jx, jv, m, eta, x, v);
            if ((rc = wh_accel(n, x, jx, m, eta, G, eps, pairwise, a))) goto out;
            for (int k = 0; k < 3 * n; ++k) jv[k] += a[k] * h;
            t = (double)(s + 1) * h;
        }
    }
out:
    *n_io = n;
    free(jx); free(jv); free(a); free(eta); free(rm);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Diagnostics                                                          */
/* ------------------------------------------------------------------ */

static double norm3(const double *p)
{
    return sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
}

/* src/utils.c:27-59 */
double orc_energy(int n, const double *x, const double *v, const double *m,
                  double G)
{
    double e = 0.0;
    for (int i = 0; i < n; ++i) {
        const double vn = norm3(&v[3 * i]);
        e += 0.5 * m[i] * vn * vn;
        for (int j = i + 1; j < n; ++j) {
            double r[3];
            for (int k = 0; k < 3; ++k) r[k] = x[3 * i + k] - x[3 * j + k];
            e -= G * m[i] * m[j] / norm3(r);
        }
    }
    return e;
}

/* src/python_interface.c:245-268 */
double orc_linear_momentum(int n, const double *v, const double *m)
{
    double p = 0.0;
    for (int i = 0; i < n; ++i)
        p += m[i] * (v[3 * i] + v[3 * i + 1] + v[3 * i + 2]);
    return p;
}

/* src/python_interface.c:270-304 */
double orc_angular_momentum(int n, const double *x, const double *v,
                            const double *m)
{
    double L = 0.0;
    for (int i = 0; i < n; ++i) {
        const double *r = &x[3 * i], *u = &v[3 * i];
        const double c0 = r[1] * u[2] - r[2] * u[1];
        const double c1 = r[2] * u[0] - r[0] * u[2];
        const double c2 = r[0] * u[1] - r[1] * u[0];
        L += m[i] * (c0 + c1 + c2);
    }
    return L;
}

void orc_abs_sum_rows(int n, const double *x, const double *m, double G,
                      double eps, int nrows, const int *rows, double *out)
{
    const double eps2 = eps * eps;
    for (int r = 0; r < nrows; ++r) {
        const int i = rows[r];
        double s = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            const double d0 = x[3 * j + 0] - x[3 * i + 0];
            const double d1 = x[3 * j + 1] - x[3 * i + 1];
            const double d2 = x[3 * j + 2] - x[3 * i + 2];
            const double q = d0 * d0 + d1 * d1 + d2 * d2;
            const double r2 = q + eps2;
            if (r2 > 0.0) s += m[j] * sqrt(q) / (r2 * sqrt(r2));
        }
        out[r] = G * s;
    }
}

void orc_direct_rows(int n, const double *x, const double *m, double G,
                     double eps, int nrows, const int *rows, double *a_rows)
{
    const double eps2 = eps * eps;
    for (int r = 0; r < nrows; ++r) {
        const int i = rows[r];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            const double d0 = x[3 * j + 0] - x[3 * i + 0];
            const double d1 = x[3 * j + 1] - x[3 * i + 1];
            const double d2 = x[3 * j + 2] - x[3 * i + 2];
            const double r2 = d0 * d0 + d1 * d1 + d2 * d2 + eps2;
            const double inv = 1.0 / (r2 * sqrt(r2));
            ax += m[j] * inv * d0; ay += m[j] * inv * d1; az += m[j] * inv * d2;
        }
        a_rows[3 * r + 0] = G * ax; a_rows[3 * r + 1] = G * ay; a_rows[3 * r + 2] = G * az;
    }
}

/* Independent planetary systems run as the reference runs each alone through
 * launch_simulation_python: WHFast (integrator 10, src/integrator_whfast.c:
 * 200-407, invalid particles removed) or leapfrog (integrator 4,
 * src/integrator.c:894-1121) with the massless acceleration, no softening.
 * System s owns rows [off[s], off[s] + counts[s]); counts[s] receives its
 * final count.  In the OpenMP build one system runs per thread at a time
 * (the fair-share baseline of one system per core).  Returns 0, or the
 * first non-zero code of a system. */
int orc_ensemble_run(int S, int *counts, const int64_t *off, int *ids, double *x,
                     double *v, double *m, double G, double dt, double tf,
                     int integrator)
{
    int rc_all = 0;
#ifdef ORC_OPENMP
    #pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int s = 0; s < S; ++s) {
        const int64_t o = off[s];
        int rc;
        if (integrator == 10)
            rc = orc_whfast_run(&counts[s], ids + o, x + 3 * o, v + 3 * o, m + o, G, 0.0, dt, tf,
                                1, 0);
        else
            rc = orc_fixed_step_run(4, 2, counts[s], x + 3 * o, v + 3 * o, m + o, G, 0.0, dt, tf);
        if (rc) {
#ifdef ORC_OPENMP
            #pragma omp critical
#endif
            if (!rc_all) rc_all = rc;
        }
    }
    return rc_all;
}
