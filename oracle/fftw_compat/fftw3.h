/* fftw3.h -- TEST INFRASTRUCTURE ONLY.
 *
 * FFTW 3 is not installed here, so grav_sim's particle-mesh code
 * (src/acceleration_PM.c, and src/grav_sim.c with USE_FFTW3) is compiled
 * against this header instead: FFTW 3's names and signatures for exactly
 * the calls those files make, implemented in fftw_compat.c by the direct DFT
 * of oracle/pm_dft.c (FFTW's documented r2c / c2r semantics, unnormalised).
 * Only the oracle Makefile's `ref` target uses it.
 */
#ifndef ORACLE_FFTW_COMPAT_H
#define ORACLE_FFTW_COMPAT_H

#include <stddef.h>

typedef double fftw_complex[2];
typedef struct orc_fftw_plan_s *fftw_plan;

#define FFTW_ESTIMATE (1U << 6)

extern const char fftw_version[];

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out,
                               unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#endif
