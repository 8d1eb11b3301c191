/*
 * ga_oracle.h - CPU restatement (FP64) of the reference's per-step dynamical
 * core, used as the parity oracle.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it, and only as the checker or the
 * timed CPU baseline.  The GPU library never calls it.
 *
 * Every arithmetic expression keeps the evaluation order of the reference's
 * expression it restates (cited file:line), so that with contraction off
 * (-ffp-contract=off) the results match the reference's serial build bit for
 * bit except in the FFT, whose rounding differs from FFTW's.
 */
#ifndef GA_ORACLE_H
#define GA_ORACLE_H

#include "../include/ga_anelastic.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_state ora_state;

ora_state *ora_create(const ga_config *cfg, const ga_columns *cols);
void       ora_destroy(ora_state *s);
int        ora_set_field(ora_state *s, int field, int slot, const double *src, long n);
int        ora_get_field(ora_state *s, int field, int slot, double *dst, long n);
int        ora_op(ora_state *s, int op, double step);
int        ora_step(ora_state *s, int nsteps);
long long  ora_bigcounter(ora_state *s);
void       ora_set_counters(ora_state *s, long long bigcounter, double mtime);
/* Non-zero once Kessler met E>100, where the reference calls exit(0). */
int        ora_error(ora_state *s);

/* Same column builders as the library's, restated independently. */
int ora_columns_build(int nz, double dz, double height_lowest_level,
                      const double *tb_in, const double *qb_in, ga_column_store *out);
int ora_coriolis_build(int ny, double dy, double corner_lat, double *f_out);

/* Tangent-linear model and adjoint of the dry, non-periodic step
 * (ga_oracle_lin.c).  An ora_lin holds perturbation (or adjoint) copies of the
 * current, P and M buffers of u, v, w, theta and of pi; its slots follow the
 * state's rotation. */
typedef struct ora_lin ora_lin;
ora_lin *ora_lin_create(ora_state *s);
void     ora_lin_destroy(ora_lin *l);
int      ora_lin_set(ora_lin *l, int field, int slot, const double *src, long n);
int      ora_lin_get(ora_lin *l, int field, int slot, double *dst, long n);
/* advance the state and the tangent together */
int      ora_tlm_step(ora_state *s, ora_lin *t, int nsteps);
/* advance the state nsteps (recording), then map the adjoint of the final
 * state held in a to the adjoint of the initial state */
int      ora_adj_run(ora_state *s, ora_lin *a, int nsteps);

#ifdef __cplusplus
}
#endif
#endif
