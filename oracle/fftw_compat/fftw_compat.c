/* fftw_compat.c -- TEST INFRASTRUCTURE ONLY: the FFTW 3 calls of grav_sim's
 * particle-mesh code on top of the oracle's direct DFT (oracle/pm_dft.c).
 * A plan records its sizes and arrays; executing it runs the transform. */
#include <stdlib.h>

#include "fftw3.h"
#include "../grav_oracle.h"

const char fftw_version[] = "oracle direct DFT (FFTW 3 interface)";

struct orc_fftw_plan_s
{
    int kind; /* 0: r2c, 1: c2r */
    int n0, n1, n2;
    void *in;
    void *out;
};

void *fftw_malloc(size_t n) { return malloc(n); }

void fftw_free(void *p) { free(p); }

static fftw_plan make_plan(int kind, int n0, int n1, int n2, void *in, void *out)
{
    fftw_plan p = malloc(sizeof(*p));
    if (!p) return NULL;
    p->kind = kind;
    p->n0 = n0;
    p->n1 = n1;
    p->n2 = n2;
    p->in = in;
    p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out,
                               unsigned flags)
{
    (void) flags;
    return make_plan(0, n0, n1, n2, in, out);
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out,
                               unsigned flags)
{
    (void) flags;
    return make_plan(1, n0, n1, n2, in, out);
}

void fftw_execute(const fftw_plan p)
{
    if (p->kind == 0)
        orc_dft3_r2c(p->n0, p->n1, p->n2, (const double *) p->in, (double *) p->out);
    else
        orc_dft3_c2r(p->n0, p->n1, p->n2, (const double *) p->in, (double *) p->out);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
