/* pm_oracle.c -- TEST INFRASTRUCTURE ONLY: CPU restatement of grav_sim's
 * particle-mesh force and cosmological leapfrog, used as the checker of the
 * GPU path.  The transforms are oracle/pm_dft.c's direct DFT (FFTW's r2c /
 * c2r semantics); everything else repeats the reference's FP64 operations in
 * the reference's order, so this code and the reference compiled against
 * oracle/fftw_compat agree bit for bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "grav_oracle.h"

static int wrap(int n, int g)
{
    /* the reference indexes n % g; n >= 0 for particles inside the box */
    const int r = n % g;
    return r < 0 ? r + g : r;
}

/* Cell indices and CIC weights of one particle (src/acceleration_PM.c:44-58). */
static void cic_cell(const double *xi, const double *box_center, double box_width,
                     double inv_cell_length, int g, int idx[2][3], double w[2][3])
{
    for (int d = 0; d < 3; d++)
    {
        const double normalized = (xi[d] - box_center[d] + box_width) * inv_cell_length;
        const int nd = (int) normalized;
        const double weight = normalized - nd;
        w[1][d] = weight;
        w[0][d] = 1.0 - weight;
        idx[0][d] = wrap(nd, g);
        idx[1][d] = wrap(nd + 1, g);
    }
}

/* The eight corners in the reference's order (src/acceleration_PM.c:60-99). */
static const int kCorner[8][3] = {
    {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1},
};

void orc_acceleration_pm(double *a, int n, const double *x, const double *m,
                         const double *box_center, double box_width, double H0, double omega_m,
                         double mean_bkg_density, int g, double scale_factor)
{
    const double box_length = box_width * 2.0;
    const long long g2 = (long long) g * g;
    const long long g3 = g2 * g;
    const int h = g / 2 + 1;
    double *delta = calloc((size_t) g3, sizeof(double));
    double *spec = malloc(sizeof(double) * 2 * (size_t) (g2 * h));
    double *phi = malloc(sizeof(double) * (size_t) g3);
    double *acc = malloc(sizeof(double) * 3 * (size_t) g3);

    /* src/acceleration_PM.c:15-110 */
    const double half_length = box_length / 2.0;
    const double cell_length = box_length / g;
    const double inv_cell_length = 1.0 / cell_length;
    for (int i = 0; i < n; i++)
    {
        int idx[2][3];
        double w[2][3];
        cic_cell(x + 3 * i, box_center, half_length, inv_cell_length, g, idx, w);
        for (int c = 0; c < 8; c++)
        {
            const int *k = kCorner[c];
            const long long cell = idx[k[0]][0] * g2 + idx[k[1]][1] * (long long) g + idx[k[2]][2];
            delta[cell] += m[i] * w[k[0]][0] * w[k[1]][1] * w[k[2]][2];
        }
    }
    const double cell_volume = cell_length * cell_length * cell_length;
    for (long long i = 0; i < g3; i++) delta[i] = (delta[i] / (cell_volume * mean_bkg_density)) - 1.0;

    /* src/acceleration_PM.c:311-345 */
    orc_dft3_r2c(g, g, g, delta, spec);
    const double two_pi_over_box_length_squared = 4.0 * M_PI * M_PI / (box_length * box_length);
    for (int i = 0; i < g; i++)
    {
        const int kx = (i < h) ? i : i - g;
        for (int j = 0; j < g; j++)
        {
            const int ky = (j < h) ? j : j - g;
            for (int k = 0; k < h; k++)
            {
                const int kz = k;
                const double k_sq = (kx * kx + ky * ky + kz * kz) * two_pi_over_box_length_squared;
                const double kernel = k_sq == 0.0 ? 0.0 : -1.0 / k_sq;
                const long long index = i * ((long long) g * h) + (long long) j * h + k;
                spec[2 * index] *= kernel;
                spec[2 * index + 1] *= kernel;
            }
        }
    }
    orc_dft3_c2r(g, g, g, spec, phi);
    const double factor = ((3.0 / 2.0) * omega_m * H0 * H0) / (scale_factor * (double) g3);
    for (long long i = 0; i < g3; i++) phi[i] *= factor;

    /* src/acceleration_PM.c:212-272 */
    for (int i = 0; i < g; i++)
    {
        for (int j = 0; j < g; j++)
        {
            for (int k = 0; k < g; k++)
            {
                const long long index = i * g2 + (long long) j * g + k;
                const int c[3] = {i, j, k};
                const long long st[3] = {g2, g, 1};
                for (int d = 0; d < 3; d++)
                {
                    const long long b = index - c[d] * st[d];
                    const double pm2 = phi[b + wrap(c[d] - 2, g) * st[d]];
                    const double pm1 = phi[b + wrap(c[d] - 1, g) * st[d]];
                    const double pp1 = phi[b + wrap(c[d] + 1, g) * st[d]];
                    const double pp2 = phi[b + wrap(c[d] + 2, g) * st[d]];
                    acc[index * 3 + d] = (pm2 - 8.0 * pm1 + 8.0 * pp1 - pp2) / (12.0 * cell_length);
                }
            }
        }
    }

    /* src/acceleration_PM.c:112-210 */
    for (int i = 0; i < n; i++)
    {
        int idx[2][3];
        double w[2][3];
        cic_cell(x + 3 * i, box_center, half_length, inv_cell_length, g, idx, w);
        for (int d = 0; d < 3; d++)
        {
            double s = 0.0;
            for (int c = 0; c < 8; c++)
            {
                const int *k = kCorner[c];
                const long long cell = idx[k[0]][0] * g2 + idx[k[1]][1] * (long long) g + idx[k[2]][2];
                const double t = acc[cell * 3 + d] * w[k[0]][0] * w[k[1]][1] * w[k[2]][2];
                s = (c == 0) ? t : s + t;
            }
            a[3 * i + d] = s;
        }
    }
    free(delta);
    free(spec);
    free(phi);
    free(acc);
}

/* src/cosmology.c:5-26 */
double orc_compute_da(double a, double H0, double omega_m, double omega_lambda)
{
    const double omega_k = 1.0 - omega_m - omega_lambda;
    return H0 * a * sqrt(omega_lambda + omega_m / (a * a * a) + omega_k / (a * a));
}

/* src/system.c:1337-1375 */
void orc_periodic_boundary(int n, double *x, const double *box_center, double box_width)
{
    for (int i = 0; i < n; i++)
    {
        for (int j = 0; j < 3; j++)
        {
            const double p = x[i * 3 + j] - box_center[j];
            if (p < -box_width)
            {
                if ((int) (p / box_width) % 2 != 0)
                    x[i * 3 + j] = fmod(p, box_width) + box_width;
                else
                    x[i * 3 + j] = fmod(p, box_width);
                x[i * 3 + j] += box_center[j];
            }
            else if (p > box_width)
            {
                if ((int) (p / box_width) % 2 != 0)
                    x[i * 3 + j] = fmod(p, box_width) - box_width;
                else
                    x[i * 3 + j] = fmod(p, box_width);
                x[i * 3 + j] += box_center[j];
            }
        }
    }
}

/* src/integrator_cosmology_leapfrog.c:24-255 with output disabled.  x is
 * advanced in place; v is left as given (the reference converts momenta
 * back to velocities only for snapshots).  v_last (3n, may be NULL)
 * receives the velocities a snapshot after the last step would hold,
 * momentum / a^2 (:200-209). */
void orc_leapfrog_cosmology(int n, double *x, const double *v, const double *m, double h,
                            double omega_m, double omega_lambda, const double *box_center,
                            double box_width, double dt, double a_begin, double a_final,
                            int pm_grid_size, int64_t *num_steps, double *t_out, double *v_last)
{
    const double H0 = h * 100.0;
    double t = a_begin;
    double *p = malloc(sizeof(double) * 3 * (size_t) n);
    double *acc = malloc(sizeof(double) * 3 * (size_t) n);
    double msum = 0.0;
    for (int i = 0; i < n; i++) msum += m[i];
    const double mean_bkg_density =
        msum / ((box_width * 2) * (box_width * 2) * (box_width * 2));
    orc_periodic_boundary(n, x, box_center, box_width);
    for (int i = 0; i < 3 * n; i++) p[i] = t * t * v[i];
    orc_acceleration_pm(acc, n, x, m, box_center, box_width, H0, omega_m, mean_bkg_density,
                        pm_grid_size, t);
    const int64_t total = (int64_t) ceil((a_final - a_begin) / dt);
    int64_t steps = 0;
    while (steps < total)
    {
        if (t + dt > a_final) dt = a_final - t;
        double da = orc_compute_da(t, H0, omega_m, omega_lambda);
        for (int i = 0; i < 3 * n; i++) p[i] -= (0.5 * dt) * acc[i] / da;
        t += 0.5 * dt;
        da = orc_compute_da(t, H0, omega_m, omega_lambda);
        for (int i = 0; i < 3 * n; i++) x[i] += dt * p[i] / (t * t * da);
        orc_periodic_boundary(n, x, box_center, box_width);
        orc_acceleration_pm(acc, n, x, m, box_center, box_width, H0, omega_m, mean_bkg_density,
                            pm_grid_size, t);
        for (int i = 0; i < 3 * n; i++) p[i] -= (0.5 * dt) * acc[i] / da;
        steps++;
        t = a_begin + steps * dt;
    }
    if (num_steps) *num_steps = steps;
    if (t_out) *t_out = t;
    if (v_last)
        for (int i = 0; i < 3 * n; i++) v_last[i] = p[i] / (t * t);
    free(p);
    free(acc);
}
