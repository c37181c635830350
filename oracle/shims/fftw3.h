/*
 * fftw3.h -- the FFTW calls cpic's MFT solver makes (src/solver.c:208-509),
 * implemented over the oracle's own FP64 FFT (oracle/orc_fft.h).
 * TEST INFRASTRUCTURE ONLY.  FFTW itself is not available here, so parity
 * with FFTW's rounding is not pinned.
 */
#ifndef ORC_SHIM_FFTW3_H
#define ORC_SHIM_FFTW3_H

#include <stddef.h>

typedef double _Complex fftw_complex;   /* <complex.h> precedes this header */
typedef struct orc_fftw_plan *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_complex *fftw_alloc_complex(size_t n);
double *fftw_alloc_real(size_t n);
void fftw_free(void *p);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);

#endif
