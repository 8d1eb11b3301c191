/*
 * FFTW3 API subset on top of the oracle's DFT (ora_fft.c), so that the
 * reference's own pressure solver (pressure.cpp:724-893) runs unmodified in
 * the CPU oracle build.  Semantics follow FFTW's advanced interface for the
 * layouts the reference plans: rank-2 contiguous batches (pressure.cpp:747,
 * damping.cpp:309) and rank-1 strided batches (laplacian.cpp:79).  The r2r
 * plans of laplacian.cpp are initialisation-only and are not supported.
 * TEST INFRASTRUCTURE.
 */
#include "fftw3.h"
extern "C" {
#include "../../ora_fft.h"
}
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

struct ga_fftw_plan_s {
    int rank, n0, n1, howmany, istride, idist, ostride, odist, sign;
    double *in, *out;
    ora_fft_plan p0, p1;
};

void *fftw_malloc(size_t n) { return calloc(1, n ? n : 1); }
void fftw_free(void *p) { free(p); }

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in, const int *,
                             int istride, int idist, fftw_complex *out, const int *, int ostride,
                             int odist, int sign, unsigned)
{
    if (rank != 1 && rank != 2) { fprintf(stderr, "fftw shim: rank %d\n", rank); abort(); }
    if (rank == 2 && (istride != 1 || ostride != 1)) { fprintf(stderr, "fftw shim: stride\n"); abort(); }
    ga_fftw_plan_s *p = new ga_fftw_plan_s();
    p->rank = rank; p->n0 = n[0]; p->n1 = rank == 2 ? n[1] : 1; p->howmany = howmany;
    p->istride = istride; p->idist = idist; p->ostride = ostride; p->odist = odist; p->sign = sign;
    p->in = (double *)in; p->out = (double *)out;
    ora_fft_plan_init(&p->p0, p->n0);
    if (rank == 2) ora_fft_plan_init(&p->p1, p->n1);
    return p;
}

fftw_plan fftw_plan_many_r2r(int, const int *, int, double *, const int *, int, int, double *,
                             const int *, int, int, const fftw_r2r_kind *, unsigned)
{
    return nullptr; /* only reached by laplacian.cpp initialisers, never by the step */
}

void fftw_execute(const fftw_plan p)
{
    if (!p) { fprintf(stderr, "fftw shim: r2r plans are not supported\n"); abort(); }
    if (p->rank == 2) {
        const long sz = (long)p->n0 * p->n1;
        for (int b = 0; b < p->howmany; b++)
            ora_fft_2d(&p->p0, &p->p1, p->sign, p->in + 2 * (long)b * p->idist,
                       p->out + 2 * (long)b * p->odist);
        (void)sz;
    } else {
        for (int b = 0; b < p->howmany; b++)
            ora_fft_1d(&p->p0, p->sign, p->in + 2 * (long)b * p->idist, p->istride,
                       p->out + 2 * (long)b * p->odist, p->ostride);
    }
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    ora_fft_plan_free(&p->p0);
    if (p->rank == 2) ora_fft_plan_free(&p->p1);
    delete p;
}
