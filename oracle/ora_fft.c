/*
 * ora_fft.c - CPU mixed-radix complex DFT (oracle test infrastructure).
 *
 * Recursive decimation in time: a length-n transform with smallest prime
 * factor r is split into r interleaved length-n/r transforms, which are then
 * combined with a direct r-point DFT per output group.  Cost is
 * O(n * sum of factors); for the grid sizes of this model (products of 2, 3,
 * 5 and a few larger primes for periodic domains) that is close to a plain
 * radix FFT.  Twiddles come from one table of cos/sin(2*pi*t/n) evaluated
 * directly for every t, so no recurrence error accumulates.
 */
#include "ora_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

int ora_fft_plan_init(ora_fft_plan *p, int n)
{
    memset(p, 0, sizeof(*p));
    if (n < 1) return -1;
    p->n = n;
    int m = n;
    for (int f = 2; m > 1 && p->nfac < 64;) {
        if (m % f == 0) { p->fac[p->nfac++] = f; m /= f; }
        else f = (f == 2) ? 3 : f + 2;
    }
    p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    p->scratch = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!p->tw || !p->scratch) return -1;
    const double two_pi = 6.283185307179586476925286766559;
    for (int t = 0; t < n; t++) {
        double a = two_pi * (double)t / (double)n;
        p->tw[2 * t] = cos(a);
        p->tw[2 * t + 1] = -sin(a);
    }
    return 0;
}

void ora_fft_plan_free(ora_fft_plan *p)
{
    free(p->tw);
    free(p->scratch);
    memset(p, 0, sizeof(*p));
}

/* Transform n points of `in` (stride istride) into contiguous `out`.
 * twstep maps this level's roots of unity onto the full-length table. */
static void fft_rec(const ora_fft_plan *p, int sign, const double *in, long istride,
                    double *out, int n, int fi, long twstep)
{
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    const int r = p->fac[fi];
    const int m = n / r;
    for (int q = 0; q < r; q++)
        fft_rec(p, sign, in + 2 * q * istride, istride * r, out + 2 * (long)q * m, m, fi + 1,
                twstep * r);

    double yre[64], yim[64];
    double *ybig = NULL;
    double *yr = yre, *yi = yim;
    if (r > 64) {
        ybig = (double *)malloc(sizeof(double) * 2 * (size_t)r);
        yr = ybig;
        yi = ybig + r;
    }
    const long N = p->n;
    const double s = (sign < 0) ? 1.0 : -1.0; /* table holds exp(-i...) */
    for (int k = 0; k < m; k++) {
        for (int q = 0; q < r; q++) {
            yr[q] = out[2 * ((long)q * m + k)];
            yi[q] = out[2 * ((long)q * m + k) + 1];
        }
        for (int g = 0; g < r; g++) {
            const long kk = k + (long)g * m; /* output index within this level */
            double are = 0.0, aim = 0.0;
            for (int q = 0; q < r; q++) {
                long t = ((long)q * kk) % n;
                t = (t * twstep) % N;
                const double wr = p->tw[2 * t];
                const double wi = s * p->tw[2 * t + 1];
                are += wr * yr[q] - wi * yi[q];
                aim += wr * yi[q] + wi * yr[q];
            }
            out[2 * kk] = are;
            out[2 * kk + 1] = aim;
        }
    }
    free(ybig);
}

void ora_fft_1d(const ora_fft_plan *p, int sign, const double *in, long istride, double *out,
                long ostride)
{
    double *tmp = p->scratch;
    fft_rec(p, sign, in, istride, tmp, p->n, 0, 1);
    for (int t = 0; t < p->n; t++) {
        out[2 * t * ostride] = tmp[2 * t];
        out[2 * t * ostride + 1] = tmp[2 * t + 1];
    }
}

void ora_fft_2d(const ora_fft_plan *pi, const ora_fft_plan *pj, int sign, const double *in,
                double *out)
{
    const int ni = pi->n, nj = pj->n;
    /* rows: transform along j for every i */
    for (int i = 0; i < ni; i++)
        ora_fft_1d(pj, sign, in + 2 * (long)i * nj, 1, out + 2 * (long)i * nj, 1);
    /* columns: transform along i for every j (in place in out) */
    for (int j = 0; j < nj; j++)
        ora_fft_1d(pi, sign, out + 2 * (long)j, nj, out + 2 * (long)j, nj);
}
