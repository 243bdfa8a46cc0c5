/* pm_dft.c -- TEST INFRASTRUCTURE ONLY: the discrete Fourier transforms the
 * particle-mesh checker needs, written from the definition of the DFT.
 *
 * grav_sim's particle-mesh force (src/acceleration_PM.c:274-391) calls FFTW 3
 * (fftw_plan_dft_r2c_3d / fftw_plan_dft_c2r_3d, any 3.x release), which is
 * not installed here.  FFTW's documented semantics are restated instead:
 *
 *   r2c: Y[k0][k1][k2] = sum_{x0,x1,x2} X[x0][x1][x2] exp(-2 pi i (k.x / n)),
 *        stored for k2 = 0 .. n2/2 (n0 x n1 x (n2/2+1) complex, row-major);
 *   c2r: the unnormalised inverse, X[x] = sum_k Y[k] exp(+2 pi i (k.x / n)),
 *        taking the missing half from Hermitian symmetry
 *        (Y[-k] = conj(Y[k])): complex inverse transforms along dimensions 0
 *        and 1, then along dimension 2 the real line
 *        Re Y[0] + 2 sum_{0<k2<n2/2} Re(Y[k2] e^{i..}) + Re(Y[n2/2] e^{i..}).
 *
 * Each 1-D transform is a direct O(n^2) sum in double precision with
 * twiddles cos / sin (2 pi t / n), t = j k mod n, in a fixed order, so the
 * result is deterministic and identical wherever libm's cos / sin agree.
 * The grids used by the tests are at most 64 cells a side.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "grav_oracle.h"

static void twiddle_table(int n, double *c, double *s)
{
    const double two_pi = 6.283185307179586476925286766559;
    for (int t = 0; t < n; t++)
    {
        c[t] = cos(two_pi * (double) t / (double) n);
        s[t] = sin(two_pi * (double) t / (double) n);
    }
}

/* One complex line of length n (interleaved re, im) in place; sign -1
 * forward, +1 inverse.  c, s: the twiddle table; tmp holds 2n doubles. */
static void dft_line(int n, double *line, int sign, const double *c, const double *s, double *tmp)
{
    for (int k = 0; k < n; k++)
    {
        double re = 0.0;
        double im = 0.0;
        for (int j = 0; j < n; j++)
        {
            const int t = (int) (((long long) j * k) % n);
            const double wr = c[t];
            const double wi = sign * s[t];
            const double xr = line[2 * j];
            const double xi = line[2 * j + 1];
            re += xr * wr - xi * wi;
            im += xr * wi + xi * wr;
        }
        tmp[2 * k] = re;
        tmp[2 * k + 1] = im;
    }
    memcpy(line, tmp, (size_t) 2 * n * sizeof(double));
}

/* Complex transform along dimension `dim` of an array of complex values
 * with extents e[0..2] (row-major). */
static void dft_axis(double *a, const int e[3], int dim, int sign)
{
    const int n = e[dim];
    double *c = malloc(sizeof(double) * n);
    double *s = malloc(sizeof(double) * n);
    double *line = malloc(sizeof(double) * 2 * n);
    double *tmp = malloc(sizeof(double) * 2 * n);
    twiddle_table(n, c, s);
    const long long st[3] = {(long long) e[1] * e[2], e[2], 1};
    int o[2];
    int k = 0;
    for (int d = 0; d < 3; d++)
        if (d != dim) o[k++] = d;
    for (int i = 0; i < e[o[0]]; i++)
    {
        for (int j = 0; j < e[o[1]]; j++)
        {
            const long long base = i * st[o[0]] + j * st[o[1]];
            for (int q = 0; q < n; q++)
            {
                line[2 * q] = a[2 * (base + q * st[dim])];
                line[2 * q + 1] = a[2 * (base + q * st[dim]) + 1];
            }
            dft_line(n, line, sign, c, s, tmp);
            for (int q = 0; q < n; q++)
            {
                a[2 * (base + q * st[dim])] = line[2 * q];
                a[2 * (base + q * st[dim]) + 1] = line[2 * q + 1];
            }
        }
    }
    free(c);
    free(s);
    free(line);
    free(tmp);
}

void orc_dft3_r2c(int n0, int n1, int n2, const double *in, double *out)
{
    const int h = n2 / 2 + 1;
    double *c = malloc(sizeof(double) * n2);
    double *s = malloc(sizeof(double) * n2);
    twiddle_table(n2, c, s);
    /* dimension 2: real line -> half spectrum */
    for (long long r = 0; r < (long long) n0 * n1; r++)
    {
        const double *x = in + r * n2;
        for (int k = 0; k < h; k++)
        {
            double re = 0.0;
            double im = 0.0;
            for (int j = 0; j < n2; j++)
            {
                const int t = (int) (((long long) j * k) % n2);
                re += x[j] * c[t];
                im += x[j] * -s[t];
            }
            out[2 * (r * h + k)] = re;
            out[2 * (r * h + k) + 1] = im;
        }
    }
    free(c);
    free(s);
    const int e[3] = {n0, n1, h};
    dft_axis(out, e, 1, -1);
    dft_axis(out, e, 0, -1);
}

void orc_dft3_c2r(int n0, int n1, int n2, const double *in, double *out)
{
    const int h = n2 / 2 + 1;
    const long long half = (long long) n0 * n1 * h;
    double *y = malloc(sizeof(double) * 2 * half);
    memcpy(y, in, sizeof(double) * 2 * half);
    const int e[3] = {n0, n1, h};
    dft_axis(y, e, 0, +1);
    dft_axis(y, e, 1, +1);
    double *c = malloc(sizeof(double) * n2);
    double *s = malloc(sizeof(double) * n2);
    twiddle_table(n2, c, s);
    for (long long r = 0; r < (long long) n0 * n1; r++)
    {
        const double *Y = y + 2 * r * h;
        for (int z = 0; z < n2; z++)
        {
            double acc = Y[0];
            for (int k = 1; k < h; k++)
            {
                const int t = (int) (((long long) z * k) % n2);
                const double term = Y[2 * k] * c[t] - Y[2 * k + 1] * s[t];
                /* the Nyquist term of an even length appears once */
                acc += (2 * k == n2) ? term : 2.0 * term;
            }
            out[r * n2 + z] = acc;
        }
    }
    free(c);
    free(s);
    free(y);
}
