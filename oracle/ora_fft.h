/*
 * ora_fft.h - CPU mixed-radix complex DFT used by the oracle.
 *
 * TEST INFRASTRUCTURE.  This file belongs to the CPU oracle: only the tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may use it.  It also
 * backs the FFTW stand-in that the reference build links (oracle/ref/), since
 * FFTW3 (the reference's third-party dependency, pinned only by the build
 * script paths: 3.3.6 in source/scompile.sh:9-10, 3.3.8.2 in
 * source/ncompile.sh:11-12) is not installed here.
 *
 * Semantics are those of an unnormalised FFTW complex DFT:
 *   out[m] = sum_n in[n] * exp(sign * 2*pi*i * m*n / N),  sign = -1 forward.
 * Complex numbers are interleaved (re, im) doubles, like fftw_complex.
 */
#ifndef ORA_FFT_H
#define ORA_FFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_fft_plan {
    int     n;          /* transform length                               */
    int     nfac;       /* number of prime factors                        */
    int     fac[64];    /* factors, smallest first                        */
    double *tw;         /* tw[2t], tw[2t+1] = cos, -sin(2*pi*t/n), t<n    */
    double *scratch;    /* 2*n doubles                                    */
} ora_fft_plan;

int  ora_fft_plan_init(ora_fft_plan *p, int n);
void ora_fft_plan_free(ora_fft_plan *p);

/* One 1-D transform.  in/out are complex arrays with element strides istride
 * and ostride (in complex units).  in and out may alias only if both strides
 * are equal. */
void ora_fft_1d(const ora_fft_plan *p, int sign,
                const double *in, long istride, double *out, long ostride);

/* 2-D transform of an ni x nj row-major complex array (j fastest). */
void ora_fft_2d(const ora_fft_plan *pi, const ora_fft_plan *pj, int sign,
                const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
