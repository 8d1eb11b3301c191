/*
 * fftw3.h stand-in for building the reference's serial sources as a CPU
 * oracle.  FFTW3 itself is not installed here.  Only the declarations the
 * reference uses are provided; fftw_shim.cpp implements them on top of the
 * oracle's mixed-radix DFT (ora_fft.c).  TEST INFRASTRUCTURE.
 */
#ifndef GA_FFTW3_SHIM_H
#define GA_FFTW3_SHIM_H
#include <stddef.h>
typedef double fftw_complex[2];
typedef struct ga_fftw_plan_s *fftw_plan;
typedef struct { int n, is, os; } fftw_iodim;
typedef int fftw_r2r_kind;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_RODFT00 10
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in,
                             const int *inembed, int istride, int idist, fftw_complex *out,
                             const int *onembed, int ostride, int odist, int sign, unsigned flags);
fftw_plan fftw_plan_many_r2r(int rank, const int *n, int howmany, double *in, const int *inembed,
                             int istride, int idist, double *out, const int *onembed, int ostride,
                             int odist, const fftw_r2r_kind *kind, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#endif
