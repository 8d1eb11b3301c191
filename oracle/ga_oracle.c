/*
 * ga_oracle.c - CPU restatement (FP64) of the reference's per-step dynamical
 * core: s_integrate_rk3 (source/driver_serial.cpp:178-286) and everything it
 * calls on the non-hydrostatic, nonlinear, serial path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: the parity oracle and the CPU
 * baseline.  Built with -ffp-contract=off so no multiply-add is fused.
 *
 * Structure (own design, not the reference's): instead of sweeping YZ slabs of
 * "cell" structs and carrying the west face over from the previous column,
 * every face flux is a pure function of the current fields, evaluated where a
 * tendency needs it.  The arithmetic inside each face and tendency keeps the
 * reference expression's evaluation order, so the values are identical.
 * Index helpers: IX(i,j,k) = (i*NY + j)*NZ + k, the reference's INDEX.
 */
#include "ga_oracle.h"
#include "ora_fft.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* physical constants: include/model.h:248-259 */
static const double Rd = 287.0, cp = 1004, cv = 717, p0 = 100000, grav = 9.8, Lv = 2.5e6;
static const double trigpi = 3.14159265358979324;
static const double pressfc = 100200;
static const double fc = 7.292e-5;
static const double meters_per_degree = 111000;
/* interpolation weights: fluxes.cpp:247-251 */
static const double onetwelfth = 1.0 / 12.0;
static const double seventwelfth = 7.0 / 12.0;
static const double thirtyseven60ths = 37.0 / 60.0;
static const double two15ths = 2.0 / 15.0;
static const double one60ths = 1.0 / 60.0;
static const double minvar = 1.0e-12; /* kessler.cpp:5 */

/* prognostic fields; snow and cloud ice follow the seven of GA_U..GA_QR */
enum { F_U, F_V, F_W, F_TH, F_QV, F_QC, F_QR, F_QS, F_QI, ORA_NF };

struct ora_state {
    ga_config c;
    int NX, NY, NZ;
    long N;
    double dx, dy, dz, dt, dtx, dty, dtz, one_d_dx, one_d_dy, one_d_dz;
    double *zu, *zw, *zsu, *zsw, *mu, *mw, *rhou, *rhow, *one_d_rhou, *one_d_rhow;
    double *tb, *tbv, *tbw, *qb, *pib, *f;
    double *buf[ORA_NF][3];
    double *cur[ORA_NF], *P[ORA_NF], *M[ORA_NF];
    double *pi, *bar[6], *vt, *accrain;
    /* ice microphysics (microphysics_option 2): snow and ice fall speeds,
     * accumulated snow, and the snow intercept N0S, a file-scope variable of
     * rutledge.cpp:90 that each snowy point of a microphysics pass rewrites */
    int ice;
    double *sts, *its, *accsnow, n0s;
    /* pressure solver */
    int ni, nj, nk, ioff;
    double *hcoef;  /* (cos kx + cos ly) - 2, per (p,q) */
    double *acoef, *ccoef, *vcoef;
    double *spec;   /* complex [k][p][q] */
    double *specw;  /* work */
    ora_fft_plan fi, fj;
    /* sponge */
    double *east_coeff, *west_coeff, *north_coeff, *south_coeff;
    int eb, ee, wb, we, nb, ne, sb, se;
    /* rayleigh */
    int raylevel;
    double *ray_u, *ray_w;
    /* PPM remap scratch; qp_edges persists between calls as in the reference */
    double *qp_edges, *qn_edges, *mono;
    double *za, *qa, *qd, *ve;
    /* turbulence (turbulence.cpp): mixing coefficients, the tendencies of
     * the step (u, v, w friction; theta, qv, qc, qr diffusion), Kessler's
     * saturation record, the vertical mixing-length tables */
    double *kmix, *khmix, *ttend[7];
    unsigned char *sat;
    double *l2, *kvmax;
    double kmixh_max, lH, water_temp, es_water;
    /* the linearised driver never calls compute_sign_cells, so the scalar
     * faces read sign arrays as allocation left them: zero (see
     * linear_rk3_step) */
    int stale_signs;
    /* hydrostatic equation set: the lid-pressure Poisson solve (init_fft2d,
     * pressure.cpp:601-645), column-average density (initializer.cpp:1265) */
    double *div2d, *rhoavg, *bco2, *ac2, *cc2, *p2, *q2, *io2d;
    long long bigcounter;
    double mtime;
    int err;
};

#define IX(i, j, k) (((long)(i) * S->NY + (j)) * S->NZ + (k))
#define IX2(i, j) ((long)(i) * S->NY + (j))

static inline double sgn(double x) { return x > 0 ? 1.0 : -1.0; } /* signof, fluxes.cpp:295-311 */

/* INTERP_5TH_EAST of fluxes.cpp:110-122 with the 6-point stencil passed as
 * a(-2) .. a(+3) around the face between a0 and a1. */
static inline double face5(double am2, double am1, double a0, double a1, double a2, double a3,
                           double sign)
{
    double c6 = thirtyseven60ths * (a1 + a0) - two15ths * (a2 + am1) + one60ths * (a3 + am2);
    double u5 = -(a3 - am2) + 5.0 * (a2 - am1) - 10.0 * (a1 - a0);
    return c6 + one60ths * sign * u5;
}

/* INTERP_3RD_TOP of fluxes.cpp:131-136: 4-point stencil a(-1)..a(+2) */
static inline double face3(double am1, double a0, double a1, double a2, double sign)
{
    double c4 = seventwelfth * (a1 + a0) - onetwelfth * (a2 + am1);
    double u3 = (a2 - am1) - 3.0 * (a1 - a0);
    return c4 + onetwelfth * sign * u3;
}

/* stencil fetch helpers along i, j, k */
#define SI(a, i, j, k)                                                                        \
    a[IX((i)-2, j, k)], a[IX((i)-1, j, k)], a[IX(i, j, k)], a[IX((i) + 1, j, k)],           \
        a[IX((i) + 2, j, k)], a[IX((i) + 3, j, k)]
#define SJ(a, i, j, k)                                                                        \
    a[IX(i, (j)-2, k)], a[IX(i, (j)-1, k)], a[IX(i, j, k)], a[IX(i, (j) + 1, k)],           \
        a[IX(i, (j) + 2, k)], a[IX(i, (j) + 3, k)]
#define SK(a, i, j, k) a[IX(i, j, (k)-1)], a[IX(i, j, k)], a[IX(i, j, (k) + 1)], a[IX(i, j, (k) + 2)]

/* the velocity that advects the perturbation at a face: basic state plus
 * perturbation, or in the linearised model (ISLINEAR, fluxes.cpp:328-337,
 * 366-374, 594-624, 642-650, 1204-1357) the basic state alone, for both the
 * upwind sign and the flux */
static inline double adv_vel(const ora_state *S, double basic, double pert)
{
    return S->c.linear_model ? basic : basic + pert;
}

/* ------------------------------------------------------------------------
 * Momentum face fluxes: interpolate_velocity (fluxes.cpp:1384-1592),
 * advecting_velocity (:1109-1164), compute_fluxes (:582-627).
 * ---------------------------------------------------------------------- */
static double u_east(const ora_state *S, int i, int j, int k)
{
    const double *U = S->cur[F_U], *UB = S->bar[0];
    double ua = 0.5 * (U[IX(i + 1, j, k)] + U[IX(i, j, k)]);
    double uba = 0.5 * (UB[IX(i + 1, j, k)] + UB[IX(i, j, k)]);
    const double at = adv_vel(S, uba, ua);
    double ue = face5(SI(U, i, j, k), sgn(at));
    double ube = face5(SI(UB, i, j, k), sgn(ua));
    return ua * ube + at * ue;
}
static double u_north(const ora_state *S, int i, int j, int k)
{
    const double *U = S->cur[F_U], *UB = S->bar[0], *V = S->cur[F_V], *VB = S->bar[1];
    double va = 0.5 * (V[IX(i, j + 1, k)] + V[IX(i - 1, j + 1, k)]);
    double vba = 0.5 * (VB[IX(i, j + 1, k)] + VB[IX(i - 1, j + 1, k)]);
    const double at = adv_vel(S, vba, va);
    double un = face5(SJ(U, i, j, k), sgn(at));
    double ubn = face5(SJ(UB, i, j, k), sgn(va));
    return va * ubn + at * un;
}
static double u_top(const ora_state *S, int i, int j, int k)
{
    if (k == 0) return 0.0; /* compute_fluxes :591 */
    const double *U = S->cur[F_U], *UB = S->bar[0], *W = S->cur[F_W], *WB = S->bar[2];
    double wa = 0.5 * (W[IX(i, j, k + 1)] + W[IX(i - 1, j, k + 1)]);
    double wba = 0.5 * (WB[IX(i, j, k + 1)] + WB[IX(i - 1, j, k + 1)]);
    double ut, ubt;
    if (k == 1 || k == S->NZ - 2) { /* interpolate_velocity_vertical_2nd :1170 */
        ut = 0.5 * (U[IX(i, j, k + 1)] + U[IX(i, j, k)]);
        ubt = 0.5 * (UB[IX(i, j, k + 1)] + UB[IX(i, j, k)]);
    } else {
        ut = face3(SK(U, i, j, k), sgn(adv_vel(S, wba, wa)));
        ubt = face3(SK(UB, i, j, k), sgn(wa));
    }
    return wa * ubt + adv_vel(S, wba, wa) * ut;
}
static double v_east(const ora_state *S, int i, int j, int k)
{
    const double *U = S->cur[F_U], *UB = S->bar[0], *V = S->cur[F_V], *VB = S->bar[1];
    double ua = 0.5 * (U[IX(i + 1, j, k)] + U[IX(i + 1, j - 1, k)]);
    double uba = 0.5 * (UB[IX(i + 1, j, k)] + UB[IX(i + 1, j - 1, k)]);
    const double at = adv_vel(S, uba, ua);
    double ve = face5(SI(V, i, j, k), sgn(at));
    double vbe = face5(SI(VB, i, j, k), sgn(ua));
    return ua * vbe + at * ve;
}
static double v_north(const ora_state *S, int i, int j, int k)
{
    const double *V = S->cur[F_V], *VB = S->bar[1];
    double va = 0.5 * (V[IX(i, j + 1, k)] + V[IX(i, j, k)]);
    double vba = 0.5 * (VB[IX(i, j + 1, k)] + VB[IX(i, j, k)]);
    const double at = adv_vel(S, vba, va);
    double vn = face5(SJ(V, i, j, k), sgn(at));
    double vbn = face5(SJ(VB, i, j, k), sgn(va));
    return va * vbn + at * vn;
}
static double v_top(const ora_state *S, int i, int j, int k)
{
    if (k == 0) return 0.0;
    const double *V = S->cur[F_V], *VB = S->bar[1], *W = S->cur[F_W], *WB = S->bar[2];
    double wa = 0.5 * (W[IX(i, j, k + 1)] + W[IX(i, j - 1, k + 1)]);
    double wba = 0.5 * (WB[IX(i, j, k + 1)] + WB[IX(i, j - 1, k + 1)]);
    double vt, vbt;
    if (k == 1 || k == S->NZ - 2) {
        vt = 0.5 * (V[IX(i, j, k + 1)] + V[IX(i, j, k)]);
        vbt = 0.5 * (VB[IX(i, j, k + 1)] + VB[IX(i, j, k)]);
    } else {
        vt = face3(SK(V, i, j, k), sgn(adv_vel(S, wba, wa)));
        vbt = face3(SK(VB, i, j, k), sgn(wa));
    }
    return wa * vbt + adv_vel(S, wba, wa) * vt;
}

/* advect_uvw_velocity (advection.cpp:304-339) with u_tend_cell (:73-94) and
 * v_tend_cell (:101-122).  The WCELL flux tendency written at :323 is
 * overwritten by the buoyancy loop (:329-337) before anyone reads it, so only
 * the buoyancy update is restated. */
static void op_advect_uvw(ora_state *S, double step)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    const double *U = S->cur[F_U], *V = S->cur[F_V];
    const double *rhow = S->rhow, *one_d_rhou = S->one_d_rhou;
    for (int i = 3; i < NX - 3; i++)
        for (int j = 3; j < NY - 3; j++)
            for (int k = 1; k < NZ - 1; k++) {
                double DTZ = S->dtz * S->mu[k];
                double ov_u = 0.25 * (V[IX(i, j, k)] + V[IX(i, j + 1, k)] + V[IX(i - 1, j, k)] +
                                      V[IX(i - 1, j + 1, k)]);
                double ut = -S->dtx * (u_east(S, i, j, k) - u_east(S, i - 1, j, k)) -
                            S->dty * (u_north(S, i, j, k) - u_north(S, i, j - 1, k)) -
                            DTZ * (rhow[k + 1] * u_top(S, i, j, k) - rhow[k] * u_top(S, i, j, k - 1)) *
                                one_d_rhou[k] +
                            S->dt * S->f[j] * ov_u;
                S->P[F_U][IX(i, j, k)] = S->M[F_U][IX(i, j, k)] + step * ut;

                double ov_v = 0.25 * (U[IX(i, j, k)] + U[IX(i + 1, j, k)] + U[IX(i, j - 1, k)] +
                                      U[IX(i + 1, j - 1, k)]);
                double vt = -S->dtx * (v_east(S, i, j, k) - v_east(S, i - 1, j, k)) -
                            S->dty * (v_north(S, i, j, k) - v_north(S, i, j - 1, k)) -
                            DTZ * (rhow[k + 1] * v_top(S, i, j, k) - rhow[k] * v_top(S, i, j, k - 1)) *
                                one_d_rhou[k] -
                            S->dt * S->f[j] * ov_v;
                S->P[F_V][IX(i, j, k)] = S->M[F_V][IX(i, j, k)] + step * vt;
            }
    if (S->c.hydrostatic) return; /* advect_uv_velocity (advection.cpp:269-293): no w */
    /* buoyancy: advection.cpp:329-337 with buoyancy_dry / buoyancy_warm_micro /
     * buoyancy_cold_micro (:42-58) */
    const double *TH = S->cur[F_TH], *tbv = S->tbv;
    const int moist = S->c.microphysics_option != 0;
    for (int i = 3; i < NX - 3; i++)
        for (int j = 3; j < NY - 3; j++)
            for (int k = 2; k < NZ - 1; k++) {
                double b0, b1;
                if (!moist) {
                    b0 = TH[IX(i, j, k)] / tbv[k];
                    b1 = TH[IX(i, j, k - 1)] / tbv[k - 1];
                } else {
                    const double *QV = S->cur[F_QV], *QC = S->cur[F_QC], *QR = S->cur[F_QR];
                    b0 = TH[IX(i, j, k)] / tbv[k] + 0.61 * QV[IX(i, j, k)] - QC[IX(i, j, k)] -
                         QR[IX(i, j, k)];
                    b1 = TH[IX(i, j, k - 1)] / tbv[k - 1] + 0.61 * QV[IX(i, j, k - 1)] -
                         QC[IX(i, j, k - 1)] - QR[IX(i, j, k - 1)];
                    if (S->ice) {
                        const double *QI = S->cur[F_QI], *QS = S->cur[F_QS];
                        b0 = b0 - QI[IX(i, j, k)] - QS[IX(i, j, k)];
                        b1 = b1 - QI[IX(i, j, k - 1)] - QS[IX(i, j, k - 1)];
                    }
                }
                S->P[F_W][IX(i, j, k)] = S->M[F_W][IX(i, j, k)] + step * S->dt * grav * 0.5 * (b0 + b1);
            }
}

/* ------------------------------------------------------------------------
 * Scalar face fluxes with a basic state: interpolate_scalar(s,sb,...)
 * (fluxes.cpp:797-867), compute_fluxes_scalar (:632-654); the signs are those
 * of compute_sign_cells (:316-341) taken directly from the current winds.
 * Returned: perturbation-flux + basic-state-flux (the sum is commutative, so
 * the order of compute_fluxes_moisture :740-770 gives the same value).
 * ---------------------------------------------------------------------- */
static double s_east(const ora_state *S, const double *s, const double *sb, int i, int j, int k)
{
    const double *U = S->cur[F_U], *UB = S->bar[0];
    double u1 = U[IX(i + 1, j, k)];
    double ut = sb ? adv_vel(S, UB[IX(i + 1, j, k)], u1) : UB[IX(i + 1, j, k)] + u1;
    /* the face east of column 2 comes from compute_west_scalar (fluxes.cpp:
     * 479-501), whose signs are taken from the winds */
    const int z = sb && S->stale_signs && i != 2;
    double se = face5(SI(s, i, j, k), z ? 0.0 : sgn(ut));
    if (!sb) return ut * se;
    double be = face5(SI(sb, i, j, k), z ? 0.0 : sgn(u1));
    return u1 * be + ut * se;
}
static double s_north(const ora_state *S, const double *s, const double *sb, int i, int j, int k)
{
    const double *V = S->cur[F_V], *VB = S->bar[1];
    double v1 = V[IX(i, j + 1, k)];
    double vt = sb ? adv_vel(S, VB[IX(i, j + 1, k)], v1) : VB[IX(i, j + 1, k)] + v1;
    const int z = sb && S->stale_signs;
    double sn = face5(SJ(s, i, j, k), z ? 0.0 : sgn(vt));
    if (!sb) return vt * sn;
    double bn = face5(SJ(sb, i, j, k), z ? 0.0 : sgn(v1));
    return v1 * bn + vt * sn;
}
static double s_top(const ora_state *S, const double *s, const double *sb, int i, int j, int k)
{
    if (k == 0) return 0.0;
    const double *W = S->cur[F_W], *WB = S->bar[2];
    double w1 = W[IX(i, j, k + 1)];
    double wt = sb ? adv_vel(S, WB[IX(i, j, k + 1)], w1) : WB[IX(i, j, k + 1)] + w1;
    double st, bt = 0.0;
    if (k == 1 || k == S->NZ - 2) {
        st = 0.5 * (s[IX(i, j, k + 1)] + s[IX(i, j, k)]);
        if (sb) bt = 0.5 * (sb[IX(i, j, k + 1)] + sb[IX(i, j, k)]);
    } else {
        const int z = sb && S->stale_signs;
        st = face3(SK(s, i, j, k), z ? 0.0 : sgn(wt));
        if (sb) bt = face3(SK(sb, i, j, k), z ? 0.0 : sgn(w1));
    }
    if (!sb) return wt * st;
    return w1 * bt + wt * st;
}
/* a field with a fall speed: interpolate_scalar_with_fallspeed
 * (fluxes.cpp:953-1032) with the qr fluxes of compute_fluxes_moisture
 * (:719-784) or compute_fluxes_scalar_with_fallspeed (:699-716), incl. the
 * bottom outflow */
static double r_top(const ora_state *S, const double *s, const double *VT, int i, int j, int k)
{
    const double *W = S->cur[F_W], *WB = S->bar[2];
    if (k == 0) {
        double s0 = 0.5 * (s[IX(i, j, 0)] + s[IX(i, j, 1)]);
        return -0.5 * (VT[IX(i, j, 1)] + VT[IX(i, j, 0)]) * s0;
    }
    double wb = WB[IX(i, j, k + 1)] + W[IX(i, j, k + 1)];
    double wf = wb - 0.5 * (VT[IX(i, j, k)] + VT[IX(i, j, k + 1)]);
    double st;
    if (k == 1 || k == S->NZ - 2)
        st = 0.5 * (s[IX(i, j, k + 1)] + s[IX(i, j, k)]);
    else
        st = face3(SK(s, i, j, k), sgn(wf));
    return wf * st;
}

/* tendency of a flux-form scalar: theta_tend_cell / qv_tend_cell (advection.cpp
 * :152-168, :197-213) with Z_ADVECT_BASE (:16-18) when base != NULL */
static double s_tend(const ora_state *S, const double *s, const double *sb, const double *base,
                     int i, int j, int k)
{
    const double *rhow = S->rhow, *one_d_rhou = S->one_d_rhou;
    double DTZ = S->dtz * S->mu[k];
    double t = -S->dtx * (s_east(S, s, sb, i, j, k) - s_east(S, s, sb, i - 1, j, k)) -
               S->dty * (s_north(S, s, sb, i, j, k) - s_north(S, s, sb, i, j - 1, k)) -
               DTZ * (rhow[k + 1] * s_top(S, s, sb, i, j, k) - rhow[k] * s_top(S, s, sb, i, j, k - 1)) *
                   one_d_rhou[k];
    if (base) {
        const double *W = S->cur[F_W];
        double zab = 0.50 *
                     (rhow[k + 1] * W[IX(i, j, k + 1)] * (base[k + 1] - base[k]) +
                      rhow[k] * W[IX(i, j, k)] * (base[k] - base[k - 1])) *
                     one_d_rhou[k];
        t = t - DTZ * zab;
    }
    return t;
}

static void op_advect_theta(ora_state *S, double step) /* advection.cpp:349-373 */
{
    for (int i = 3; i < S->NX - 3; i++)
        for (int j = 3; j < S->NY - 3; j++)
            for (int k = 1; k < S->NZ - 1; k++)
                S->P[F_TH][IX(i, j, k)] =
                    S->M[F_TH][IX(i, j, k)] +
                    step * s_tend(S, S->cur[F_TH], S->bar[3], S->tb, i, j, k);
}

/* advect_qv (advection.cpp:577-601): the vapour alone, the linearised
 * model's moisture advection */
static void op_advect_qv(ora_state *S, double step)
{
    for (int i = 3; i < S->NX - 3; i++)
        for (int j = 3; j < S->NY - 3; j++)
            for (int k = 1; k < S->NZ - 1; k++)
                S->P[F_QV][IX(i, j, k)] =
                    S->M[F_QV][IX(i, j, k)] + step * s_tend(S, S->cur[F_QV], S->bar[4], S->qb, i, j, k);
}

/* calculate_rain_fall_speed_kessler (kessler.cpp:222-252) over [il,ih)x[jl,jh) */
static void fall_speed(ora_state *S, const double *qr, int il, int ih, int jl, int jh)
{
    double *vt = S->vt;
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                vt[IX(i, j, k)] = 0.0;
                if (qr[IX(i, j, k)] > minvar) {
                    double qrr = fmax(qr[IX(i, j, k)] * 0.001 * S->rhou[k], 0.0);
                    double vtden = sqrt(S->rhou[1] / S->rhou[k]);
                    vt[IX(i, j, k)] = 36.34 * (pow(qrr, 0.1364)) * vtden;
                }
            }
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++) vt[IX(i, j, 0)] = vt[IX(i, j, 1)];
}

/* ------------------------------------------------------------------------
 * Ice microphysics constants (rutledge.cpp:13-147) and fall speeds
 * (calculate_snow/rain/ice_fall_speed_rutledge, :503-600).
 * ---------------------------------------------------------------------- */
static const double Ls = 2.85e6, Lf = 3.50e5;          /* model.h:256-257 */
static const double rut_tmin = -30 + 273.15, rut_tmax = 0 + 273.15;
static const double rut_minvar = 1.0e-10;             /* minvar_snow/cice/rain/cwat */
static const double N0r = 8e6, ERC = 1, M0 = 1e-12, Rstar = 8.314e3, Mw = 18.016, Ka = 2.43e-2,
                    chi = 2.26e-5, dimax = 500.0e-6, app = 1.139, bexp = 0.11, rhoS = 200, ESC = 1.0,
                    mu_s = 1.718e-5, ap_lin = 3.0e3;
static double rut_rfall(void) { return 2115.0 * pow(0.01, 0.2) * 17.83786; } /* rutledge.cpp:140 */
/* CONVERT_PRESSURE + PBAR (rutledge.cpp:20-24) */
static double rut_pressure(const ora_state *S, long ix, int k)
{
    return (S->c.hydrostatic ? S->pi[ix] : S->pi[ix] / (cp * S->tbv[k])) + S->bar[5][ix];
}
static void rut_rain_fall(ora_state *S, double *vtr, const double *qr, int il, int ih, int jl, int jh)
{
    const double cpRd = cp / Rd, rfall = rut_rfall();
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long ix = IX(i, j, k);
                if (qr[ix] > rut_minvar) {
                    double pd = p0 * pow(rut_pressure(S, ix, k), cpRd);
                    double lambdaR = sqrt(sqrt((trigpi * 1000 * N0r) / (S->rhou[k] * qr[ix])));
                    vtr[ix] = rfall / (6.0 * pow(lambdaR, 0.8)) * pow(p0 / pd, 0.4);
                } else
                    vtr[ix] = 0;
            }
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++) vtr[IX(i, j, 0)] = vtr[IX(i, j, 1)];
}
static void rut_snow_fall(ora_state *S, double *vts, const double *qs, int il, int ih, int jl, int jh)
{
    const double cpRd = cp / Rd;
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long ix = IX(i, j, k);
                if (qs[ix] > rut_minvar) {
                    double pd = p0 * pow(rut_pressure(S, ix, k), cpRd);
                    double lambdaS = pow((trigpi * rhoS * S->n0s) / (S->rhou[k] * qs[ix]), 0.25);
                    vts[ix] = app * 1.15 * pow(lambdaS, -bexp) * pow(p0 / pd, 0.4);
                } else
                    vts[ix] = 0;
            }
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++) vts[IX(i, j, 0)] = vts[IX(i, j, 1)];
}
/* the ice fall speed is written only where its input exceeds the threshold
 * and keeps its value elsewhere */
static void rut_ice_fall(ora_state *S, double *vti, const double *qi, int il, int ih, int jl, int jh)
{
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long ix = IX(i, j, k);
                if (qi[ix] > rut_minvar) {
                    double nc = fmin(fmax(5.38e7 * pow(S->rhou[k] * qi[ix], 0.75), 1.0e3), 1.0e6);
                    double MI = S->rhou[k] * fmax(qi[ix], 0) / nc;
                    double Dl = fmax(fmin(11.9 * sqrt(MI), dimax), 1.0e-25);
                    vti[ix] = 1.49e4 * pow(Dl, 1.31);
                }
            }
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++) vti[IX(i, j, 0)] = vti[IX(i, j, 1)];
}

static void op_advect_micro(ora_state *S, double step) /* advection.cpp:451-498 */
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    /* calculate_eulerian_fall_speed_rain (microphysics.cpp:169-179) */
    if (S->c.rain_fallout == 1) {
        if (S->ice) rut_rain_fall(S, S->vt, S->cur[F_QR], 3, NX - 3, 3, NY - 3);
        else fall_speed(S, S->cur[F_QR], 3, NX - 3, 3, NY - 3);
    }
    const double *rhow = S->rhow, *one_d_rhou = S->one_d_rhou;
    const double *QC = S->cur[F_QC], *QR = S->cur[F_QR];
    for (int i = 3; i < NX - 3; i++)
        for (int j = 3; j < NY - 3; j++)
            for (int k = 1; k < NZ - 1; k++) {
                long ix = IX(i, j, k);
                S->P[F_QV][ix] =
                    S->M[F_QV][ix] + step * s_tend(S, S->cur[F_QV], S->bar[4], S->qb, i, j, k);
                S->P[F_QC][ix] = S->M[F_QC][ix] + step * s_tend(S, QC, NULL, NULL, i, j, k);
                double DTZ = S->dtz * S->mu[k];
                double tr = -S->dtx * (s_east(S, QR, NULL, i, j, k) - s_east(S, QR, NULL, i - 1, j, k)) -
                            S->dty * (s_north(S, QR, NULL, i, j, k) - s_north(S, QR, NULL, i, j - 1, k)) -
                            DTZ * (rhow[k + 1] * r_top(S, QR, S->vt, i, j, k) - rhow[k] * r_top(S, QR, S->vt, i, j, k - 1)) *
                                one_d_rhou[k];
                S->P[F_QR][ix] = S->M[F_QR][ix] + step * tr;
            }
}

/* advect_ice_cell (advection.cpp:508-567): snow, then cloud ice, each with
 * its fall speed; the Eulerian fall speeds first (calculate_eulerian_fall_
 * speed_snow_ice, microphysics.cpp:188-199), whose ice argument is the
 * pressure field (advection.cpp:514) */
static void op_advect_ice(ora_state *S, double step)
{
    if (!S->ice) return;
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    if (S->c.rain_fallout == 1) {
        rut_ice_fall(S, S->its, S->pi, 3, NX - 3, 3, NY - 3);
        rut_snow_fall(S, S->sts, S->cur[F_QS], 3, NX - 3, 3, NY - 3);
    }
    const double *rhow = S->rhow, *one_d_rhou = S->one_d_rhou;
    const int fld[2] = {F_QS, F_QI};
    const double *fall[2] = {S->sts, S->its};
    for (int n = 0; n < 2; n++) {
        const double *q = S->cur[fld[n]];
        for (int i = 3; i < NX - 3; i++)
            for (int j = 3; j < NY - 3; j++)
                for (int k = 1; k < NZ - 1; k++) {
                    const long ix = IX(i, j, k);
                    double DTZ = S->dtz * S->mu[k];
                    double t = -S->dtx * (s_east(S, q, NULL, i, j, k) - s_east(S, q, NULL, i - 1, j, k)) -
                               S->dty * (s_north(S, q, NULL, i, j, k) - s_north(S, q, NULL, i, j - 1, k)) -
                               DTZ * (rhow[k + 1] * r_top(S, q, fall[n], i, j, k) -
                                      rhow[k] * r_top(S, q, fall[n], i, j, k - 1)) *
                                   one_d_rhou[k];
                    S->P[fld[n]][ix] = S->M[fld[n]][ix] + step * t;
                }
    }
}

static void op_zero_moisture(ora_state *S) /* microphysics.cpp:675-700 */
{
    double *qc = S->P[F_QC], *qr = S->P[F_QR], *qv = S->P[F_QV];
    for (long n = 0; n < S->N; n++)
        if (qc[n] < 0) qc[n] = 0;
    for (long n = 0; n < S->N; n++)
        if (qr[n] < 0) qr[n] = 0;
    if (S->ice)
        for (long n = 0; n < S->N; n++) {
            if (S->P[F_QI][n] < 0) S->P[F_QI][n] = 0;
            if (S->P[F_QS][n] < 0) S->P[F_QS][n] = 0;
        }
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                long ix = IX(i, j, k);
                if (qv[ix] + S->bar[4][ix] + S->qb[k] < 0) qv[ix] = -(S->bar[4][ix] + S->qb[k]);
            }
}

/* ------------------------------------------------------------------------
 * Pressure: solve_pressure (pressure.cpp:142-224, serial non-hydrostatic
 * branch :187-208), divergence3d (:1340-1381) / divergence3d_periodic
 * (:1390-1424), poisson_fft3d (:805-893), init_fft3d (:724-797).
 * ---------------------------------------------------------------------- */
static void mirror(ora_state *S, double *s) /* mirror_boundaries, boundaries.cpp:363-379 */
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    for (int k = 1; k < NZ - 1; k++) {
        for (int j = 0; j < NY; j++) {
            s[IX(0, j, k)] = s[IX(1, j, k)];
            s[IX(NX - 1, j, k)] = s[IX(NX - 2, j, k)];
        }
        for (int i = 0; i < NX; i++) {
            s[IX(i, 0, k)] = s[IX(i, 1, k)];
            s[IX(i, NY - 1, k)] = s[IX(i, NY - 2, k)];
        }
    }
}
static void periodic_ew(ora_state *S, double *v) /* boundaries.cpp:562-574 */
{
    const int NX = S->NX;
    for (int k = 0; k < S->NZ; k++)
        for (int j = 0; j < S->NY; j++) {
            v[IX(0, j, k)] = v[IX(NX - 6, j, k)];
            v[IX(1, j, k)] = v[IX(NX - 5, j, k)];
            v[IX(2, j, k)] = v[IX(NX - 4, j, k)];
            v[IX(NX - 3, j, k)] = v[IX(3, j, k)];
            v[IX(NX - 2, j, k)] = v[IX(4, j, k)];
            v[IX(NX - 1, j, k)] = v[IX(5, j, k)];
        }
}

#define SP(p, q, k) (S->spec + 2 * (((long)(k) * S->ni + (p)) * S->nj + (q)))

static void poisson(ora_state *S, double step)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    const int ni = S->ni, nj = S->nj, nk = S->nk;
    const double *UP = S->P[F_U], *VP = S->P[F_V], *WP = S->P[F_W];
    const double *rhou = S->rhou, *rhow = S->rhow;
    /* divergence tendency into the real part; imaginary part zero */
    memset(S->spec, 0, sizeof(double) * 2 * (size_t)ni * nj * nk);
    int il, ih, jl = 1, jh = NY - 1, off;
    if (!S->c.periodic_ew_boundaries) { il = 1; ih = NX - 1; off = 0; }
    else { il = 3; ih = NX - 3; off = 3; }
    for (int i = il; i < ih; i++)
        for (int j = jl; j < jh; j++)
            for (int k = 1; k < NZ - 1; k++) {
                double d = rhou[k] * (UP[IX(i + 1, j, k)] - UP[IX(i, j, k)]) * S->one_d_dx +
                           rhou[k] * (VP[IX(i, j + 1, k)] - VP[IX(i, j, k)]) * S->one_d_dy +
                           (rhow[k + 1] * WP[IX(i, j, k + 1)] - rhow[k] * WP[IX(i, j, k)]) *
                               (S->one_d_dz * S->mu[k]);
                d /= (step * S->dt);
                SP(i - off, j, k)[0] = d;
            }
    for (int k = 1; k < NZ - 1; k++) {
        if (!S->c.periodic_ew_boundaries)
            for (int j = 0; j < NY; j++) {
                SP(0, j, k)[0] = SP(1, j, k)[0];
                SP(NX - 1, j, k)[0] = SP(NX - 2, j, k)[0];
            }
        for (int i = 0; i < ni; i++) {
            SP(i, 0, k)[0] = SP(i, 1, k)[0];
            SP(i, NY - 1, k)[0] = SP(i, NY - 2, k)[0];
        }
    }
    /* the copies to levels 0 and NZ-1 (:1372-1380) feed transforms whose
     * results are never read back, so those two levels are skipped */
    const double size2d = (double)(ni * nj);
    for (int k = 1; k < nk - 1; k++) {
        ora_fft_2d(&S->fi, &S->fj, -1, SP(0, 0, k), S->specw);
        memcpy(SP(0, 0, k), S->specw, sizeof(double) * 2 * (size_t)ni * nj);
    }
    for (int k = 1; k < nk - 1; k++)
        for (int p = 0; p < ni; p++)
            for (int q = 0; q < nj; q++) {
                SP(p, q, k)[0] /= size2d;
                SP(p, q, k)[1] /= size2d;
            }
    /* Thomas algorithm per (p,q) (pressure.cpp:834-871); the diagonal
     * B(p,q,k) of init_fft3d's stretched branch (:778-792) */
    double *F = (double *)malloc(sizeof(double) * nk);
    const double dx2 = S->dx * S->dx;
    for (int p = 0; p < ni; p++)
        for (int q = 0; q < nj; q++) {
            double h = S->hcoef[(long)p * nj + q];
            double z = 1.0 / (rhou[1] * 2.0 * h / dx2 - S->vcoef[1]);
            F[1] = S->ccoef[1] * z;
            SP(p, q, 1)[0] = SP(p, q, 1)[0] * z;
            SP(p, q, 1)[1] = SP(p, q, 1)[1] * z;
            for (int k = 2; k < nk - 1; k++) {
                double b = rhou[k] * 2.0 * h / dx2 - S->vcoef[k];
                z = 1.0 / (b - S->acoef[k] * F[k - 1]);
                F[k] = S->ccoef[k] * z;
                SP(p, q, k)[0] = (SP(p, q, k)[0] - S->acoef[k] * SP(p, q, k - 1)[0]) * z;
                SP(p, q, k)[1] = (SP(p, q, k)[1] - S->acoef[k] * SP(p, q, k - 1)[1]) * z;
            }
            if (p == 0 && q == 0) { /* mean mode gauge (:858-859), T3 */
                SP(0, 0, NZ - 2)[0] = 0;
                SP(0, 0, NZ - 2)[1] = 0;
            }
            for (int k = NZ - 3; k >= 1; k--) {
                SP(p, q, k)[0] -= F[k] * SP(p, q, k + 1)[0];
                SP(p, q, k)[1] -= F[k] * SP(p, q, k + 1)[1];
            }
        }
    free(F);
    for (int k = 1; k < nk - 1; k++) {
        ora_fft_2d(&S->fi, &S->fj, +1, SP(0, 0, k), S->specw);
        memcpy(SP(0, 0, k), S->specw, sizeof(double) * 2 * (size_t)ni * nj);
    }
    double *PI = S->pi;
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < nj; j++) {
            PI[IX(i + off, j, 0)] = SP(i, j, 1)[0];
            for (int k = 1; k < nk - 1; k++) PI[IX(i + off, j, k)] = SP(i, j, k)[0];
            PI[IX(i + off, j, NZ - 1)] = SP(i, j, NZ - 2)[0];
        }
}

static void op_solve_pressure(ora_state *S, double step)
{
    if (!S->c.periodic_ew_boundaries) {
        mirror(S, S->P[F_U]);
        mirror(S, S->P[F_V]);
        mirror(S, S->P[F_W]);
        poisson(S, step);
        mirror(S, S->pi);
    } else {
        periodic_ew(S, S->P[F_U]);
        periodic_ew(S, S->P[F_V]);
        periodic_ew(S, S->P[F_W]);
        poisson(S, step);
        periodic_ew(S, S->pi);
    }
}

static void op_project(ora_state *S, double step) /* solver.cpp:120-135 */
{
    double *UP = S->P[F_U], *VP = S->P[F_V], *WP = S->P[F_W];
    const double *PI = S->pi;
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++) {
            UP[IX(i, j, 1)] -= step * (S->dtx * (PI[IX(i, j, 1)] - PI[IX(i - 1, j, 1)]));
            VP[IX(i, j, 1)] -= step * (S->dty * (PI[IX(i, j, 1)] - PI[IX(i, j - 1, 1)]));
            for (int k = 2; k < S->NZ - 1; k++) {
                UP[IX(i, j, k)] -= step * (S->dtx * (PI[IX(i, j, k)] - PI[IX(i - 1, j, k)]));
                VP[IX(i, j, k)] -= step * (S->dty * (PI[IX(i, j, k)] - PI[IX(i, j - 1, k)]));
                WP[IX(i, j, k)] -= step * ((S->dtz * S->mw[k]) * (PI[IX(i, j, k)] - PI[IX(i, j, k - 1)]));
            }
        }
}

/* ------------------------------------------------------------------------
 * Boundary conditions: boundaries.cpp:119-284, 304-326, 436-498.
 * ---------------------------------------------------------------------- */
static void sponge(ora_state *S, double *v, int ns_only)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    if (!ns_only) {
        for (int i = S->eb; i < S->ee; i++)
            for (int j = 1; j < NY; j++)
                for (int k = 1; k < NZ; k++) v[IX(i, j, k)] -= S->east_coeff[i - S->eb] * v[IX(i, j, k)];
        for (int i = S->wb; i < S->we; i++)
            for (int j = 1; j < NY; j++)
                for (int k = 1; k < NZ; k++) v[IX(i, j, k)] -= S->west_coeff[i - S->wb] * v[IX(i, j, k)];
    }
    for (int i = 1; i < NX; i++)
        for (int j = S->sb; j < S->se; j++)
            for (int k = 1; k < NZ; k++) v[IX(i, j, k)] -= S->south_coeff[j - S->sb] * v[IX(i, j, k)];
    for (int i = 1; i < NX; i++)
        for (int j = S->nb; j < S->ne; j++)
            for (int k = 1; k < NZ; k++) v[IX(i, j, k)] -= S->north_coeff[j - S->nb] * v[IX(i, j, k)];
}
static void upper_lower(ora_state *S, double *v)
{
    for (int i = 1; i < S->NX; i++)
        for (int j = 1; j < S->NY; j++) {
            v[IX(i, j, 0)] = v[IX(i, j, 1)];
            v[IX(i, j, S->NZ - 1)] = v[IX(i, j, S->NZ - 2)];
        }
}
static void upper_lower_zero(ora_state *S, double *v)
{
    for (int i = 1; i < S->NX; i++)
        for (int j = 1; j < S->NY; j++) {
            v[IX(i, j, 0)] = 0;
            v[IX(i, j, 1)] = 0;
            v[IX(i, j, S->NZ - 1)] = 0;
        }
}

/* the array the boundary conditions and damping treat as w: the forecast,
 * or under the hydrostatic equation set the diagnosed current w
 * (boundaries.cpp:152-156, damping.cpp:1168-1172) */
static double *w_bc(ora_state *S) { return S->c.hydrostatic ? S->cur[F_W] : S->P[F_W]; }

static void op_bc(ora_state *S)
{
    const int per = S->c.periodic_ew_boundaries;
    if (!per) {
        sponge(S, S->P[F_U], 0);
        sponge(S, S->P[F_V], 0);
        sponge(S, S->P[F_TH], 0);
        upper_lower(S, S->P[F_U]);
        upper_lower(S, S->P[F_V]);
        upper_lower(S, S->P[F_TH]);
        sponge(S, w_bc(S), 0);
        upper_lower_zero(S, w_bc(S));
    } else {
        sponge(S, S->P[F_U], 1);
        sponge(S, S->P[F_V], 1);
        sponge(S, S->P[F_TH], 1);
        periodic_ew(S, S->P[F_U]);
        periodic_ew(S, S->P[F_V]);
        periodic_ew(S, S->pi);
        periodic_ew(S, S->P[F_TH]);
        upper_lower(S, S->P[F_U]);
        upper_lower(S, S->P[F_V]);
        upper_lower(S, S->P[F_TH]);
        sponge(S, w_bc(S), 1);
        periodic_ew(S, w_bc(S));
        upper_lower_zero(S, w_bc(S));
    }
}

static void op_bc_micro(ora_state *S)
{
    const int per = S->c.periodic_ew_boundaries;
    const int f5[5] = {F_QV, F_QC, F_QR, F_QI, F_QS}, nf = S->ice ? 5 : 3;
    for (int n = 0; n < nf; n++) sponge(S, S->P[f5[n]], per);
    if (per)
        for (int n = 0; n < nf; n++) periodic_ew(S, S->P[f5[n]]);
    for (int n = 0; n < nf; n++) upper_lower(S, S->P[f5[n]]);
}

static void op_rayleigh(ora_state *S) /* damping.cpp:1148-1177 */
{
    for (int k = S->raylevel; k < S->NZ; k++) {
        double cu = S->ray_u[k], cw = S->ray_w[k];
        for (int i = 1; i < S->NX - 1; i++)
            for (int j = 1; j < S->NY - 1; j++) {
                long ix = IX(i, j, k);
                S->P[F_U][ix] -= cu * S->P[F_U][ix];
                S->P[F_V][ix] -= cu * S->P[F_V][ix];
                w_bc(S)[ix] -= cw * w_bc(S)[ix];
                S->P[F_TH][ix] -= cu * S->P[F_TH][ix];
            }
    }
}

/* ------------------------------------------------------------------------
 * Explicit diffusion: apply_explicit_diffusion (damping.cpp:1125-1146) with
 * diffusion_{2nd,4th,6th}_var (:769-940) on the start-of-step fields, over
 * i in [3, NX-3), j in [3, NY-3), k in [1, NZ-1).  Every tendency is formed
 * from the old values before any is added.  The vertical operator of the
 * stretched-grid build weights the column with the finite-difference weights
 * of init_diffusion_weights (:158-270): Fornberg's recurrence (util.cpp:
 * 199-247) on the heights scaled by the local spacing, the order's weights
 * for k in [order/2, NZ-order/2), 4th-order rows at k = 2 and NZ-3 (order 6)
 * and 2nd-order rows at k = 1 and NZ-2 (orders 4 and 6).
 * ---------------------------------------------------------------------- */

/* weights c[i*(m+1)+d] of derivative d at z from the points x[0..n] */
static void fornberg(double z, const double *x, int n, int m, double *c)
{
    double c1 = 1.0, c4 = x[0] - z;
    c[0] = 1.0;
    for (int i = 1; i <= n; i++) {
        const int mn = i < m ? i : m;
        double c2 = 1.0;
        const double c5 = c4;
        c4 = x[i] - z;
        for (int j = 0; j <= i - 1; j++) {
            const double c3 = x[i] - x[j];
            c2 = c2 * c3;
            if (j == i - 1) {
                for (int d = mn; d >= 1; d--)
                    c[i * (m + 1) + d] = c1 * (d * c[(i - 1) * (m + 1) + d - 1] - c5 * c[(i - 1) * (m + 1) + d]) / c2;
                c[i * (m + 1)] = -c1 * c5 * c[(i - 1) * (m + 1)] / c2;
            }
            for (int d = mn; d >= 1; d--)
                c[j * (m + 1) + d] = (c4 * c[j * (m + 1) + d] - d * c[j * (m + 1) + d - 1]) / c3;
            c[j * (m + 1)] = c4 * c[j * (m + 1)] / c3;
        }
        c1 = c2;
    }
}

/* rows of order+1 weights per level: the order's derivative at level k from
 * levels k-lo .. k-lo+n */
static void diffusion_weights(int order, const double *h, int NZ, double *w)
{
    double hs[512], c[64];
    memset(w, 0, sizeof(double) * (size_t)(order + 1) * NZ);
    for (int n = 0; n < NZ; n++) hs[n] = 0.0;
    for (int k = order / 2; k < NZ - order / 2; k++) {
        for (int n = 0; n < NZ; n++) hs[n] = (h[n] - h[k]) / (h[k + 1] - h[k]);
        memset(c, 0, sizeof c);
        fornberg(hs[k], hs - order / 2 + k, order, order, c);
        for (int j = 0; j <= order; j++) w[(order + 1) * k + j] = c[(order + 1) * j + order];
    }
    const int rows[2][2] = {{2, NZ - 3}, {1, NZ - 2}};
    for (int pass = 0; pass < 2; pass++) {
        const int lower = pass == 0 ? 4 : 2;
        if (order <= lower) continue;
        for (int r = 0; r < 2; r++) {
            const int k = rows[pass][r];
            /* the row at k = 2 rescales levels 0 .. NZ-2 only (damping.cpp:200) */
            const int top = (pass == 0 && r == 0) ? NZ - 1 : NZ;
            for (int n = 0; n < top; n++) hs[n] = (h[n] - h[k]) / (h[k + 1] - h[k]);
            memset(c, 0, sizeof c);
            fornberg(hs[k], hs - lower / 2 + k, lower, lower, c);
            for (int j = 0; j <= lower; j++) w[(order + 1) * k + j] = c[(lower + 1) * j + lower];
        }
    }
}

static double d2(const double *v, long c, long s) { return v[c + s] - 2.0 * v[c] + v[c - s]; }
static double d4(const double *v, long c, long s)
{
    return v[c - 2 * s] - 4.0 * v[c - s] + 6.0 * v[c] - 4.0 * v[c + s] + v[c + 2 * s];
}
static double d6(const double *v, long c, long s)
{
    return v[c - 3 * s] - 6.0 * v[c - 2 * s] + 15.0 * v[c - s] - 20.0 * v[c] + 15.0 * v[c + s] - 6.0 * v[c + 2 * s] +
           v[c + 3 * s];
}
/* weighted column sums of the stretched-grid operators (diffuse_k_*, :556-715) */
static double wk2(const double *v, long c, const double *w) { return w[0] * v[c - 1] + w[1] * v[c] + w[2] * v[c + 1]; }
static double wk4(const double *v, long c, const double *w)
{
    return w[0] * v[c - 2] + w[1] * v[c - 1] + w[2] * v[c] + w[3] * v[c + 1] + w[4] * v[c + 2];
}
static double wk6(const double *v, long c, const double *w)
{
    return w[0] * v[c - 3] + w[1] * v[c - 2] + w[2] * v[c - 1] + w[3] * v[c] + w[4] * v[c + 1] + w[5] * v[c + 2] +
           w[6] * v[c + 3];
}

static void op_explicit_diffusion(ora_state *S, double step)
{
    const int order = S->c.diffusion_order, NZ = S->NZ;
    const int nf = S->ice ? ORA_NF : S->c.microphysics_option ? 7 : 4; /* damping.cpp:1016-1021 */
    if (order != 2 && order != 4 && order != 6) return;
    const double kh = S->c.kdiffh, kv = S->c.kdiffv;
    const long sx = (long)S->NY * S->NZ, sy = S->NZ;
    const int ind = order + 1;
    double *w = (double *)calloc((size_t)ind * NZ, sizeof(double));
    diffusion_weights(order, S->zsu, NZ, w);
    double *tend = (double *)calloc((size_t)S->N, sizeof(double));
    for (int f = 0; f < nf; f++) {
        if (f == F_W && S->c.hydrostatic) continue; /* damping.cpp:1052 */
        double *v = S->M[f];
        for (int i = 3; i < S->NX - 3; i++)
            for (int j = 3; j < S->NY - 3; j++)
                for (int k = 1; k < NZ - 1; k++) {
                    const long c = IX(i, j, k);
                    double d;
                    if (order == 2) {
                        d = kh * d2(v, c, sx) + kh * d2(v, c, sy) + kv * wk2(v, c, w + ind * k);
                    } else if (order == 4) {
                        if (k == 1 || k == NZ - 2) /* both ends with row NZ-2 (damping.cpp:820, 861) */
                            d = -kh * d4(v, c, sx) - kh * d4(v, c, sy) + kv * wk2(v, c, w + ind * (NZ - 2));
                        else
                            d = -kh * d4(v, c, sx) - kh * d4(v, c, sy) - kv * wk4(v, c, w + ind * k);
                    } else {
                        double z;
                        if (k == 1 || k == NZ - 2) z = kv * wk2(v, c, w + ind * k);
                        else if (k == 2 || k == NZ - 3) z = -kv * wk4(v, c, w + ind * k);
                        else z = kv * wk6(v, c, w + ind * k);
                        d = kh * d6(v, c, sx) + kh * d6(v, c, sy) + z;
                    }
                    tend[c] = step * d;
                }
        for (int i = 3; i < S->NX - 3; i++)
            for (int j = 3; j < S->NY - 3; j++)
                for (int k = 1; k < NZ - 1; k++) v[IX(i, j, k)] += tend[IX(i, j, k)];
    }
    free(tend);
    free(w);
}

/* ------------------------------------------------------------------------
 * Turbulence (turbulence.cpp): once per step, from the start-of-step fields,
 * the mixing coefficients (get_Kmix / get_Kmix_dry, :563-835) and the
 * tendencies of the turbulent stress (turbulent_diffusion_velocity,
 * :839-1022) and scalar fluxes (turbulent_diffusion_scalars / _theta,
 * :1027-1276); in every RK stage they are added to the forecast fields
 * (apply_*_diffusion, :233-290).  Flat ground (HTOPO = 0) and an all-ocean
 * surface.  The reference's YZ-slab sweep keeps the previous slab's stresses
 * as the "west" ones and carries each level's vertical flux to the next
 * level; both are the stress or flux of the neighbouring point, evaluated
 * here by the same expressions where they are used.
 * ---------------------------------------------------------------------- */
static const double tb_cs = 0.25, tb_one_d_Pr = 3.0, tb_lv_max = 200.0, tb_cmixh_max = 0.05,
                    tb_cmixv_max = 0.15;

static void turb_init(ora_state *S) /* init_kmix, turbulence.cpp:85-151 */
{
    const int NZ = S->NZ;
    S->kmix = (double *)calloc((size_t)S->N, sizeof(double));
    S->khmix = (double *)calloc((size_t)S->N, sizeof(double));
    for (int t = 0; t < 7; t++) S->ttend[t] = (double *)calloc((size_t)S->N, sizeof(double));
    S->sat = (unsigned char *)calloc((size_t)S->N, 1);
    S->l2 = (double *)calloc(NZ, sizeof(double));
    S->kvmax = (double *)calloc(NZ, sizeof(double));
    S->kmixh_max = tb_cmixh_max * S->dx * S->dx / S->dt;
    S->lH = S->dx / 4.0;
    for (int k = 1; k < NZ; k++) {
        const double dz = S->zsu[k] - S->zsu[k - 1];
        S->l2[k] = dz > tb_lv_max ? tb_lv_max * tb_lv_max : dz * dz;
        S->kvmax[k] = tb_cmixv_max * S->l2[k] / S->dt;
    }
    S->water_temp = S->c.water_temp + 273.15;
    S->es_water = 611.2 * exp(17.67 * (S->water_temp - 273.15) / (S->water_temp - 29.65));
}

static void turb_kmix(ora_state *S)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ, moist = S->c.microphysics_option != 0;
    const long sx = (long)NY * NZ, sy = NZ;
    const double *U = S->M[F_U], *V = S->M[F_V], *W = S->M[F_W], *TH = S->M[F_TH];
    const double *UB = S->bar[0], *VB = S->bar[1], *WB = S->bar[2], *THB = S->bar[3], *QB = S->bar[4],
                 *PB = S->bar[5];
    const double odx = S->one_d_dx, ody = S->one_d_dy, cpRd = cp / Rd;
    for (int i = 1; i < NX - 1; i++)
        for (int j = 1; j < NY - 1; j++) {
            S->kmix[IX(i, j, 1)] = 0;
            S->kmix[IX(i, j, NZ - 1)] = 0;
            for (int k = 2; k < NZ - 1; k++) {
                const long c = IX(i, j, k);
                const double odzw = S->one_d_dz * S->mw[k];
                const double D11 = 0.50 *
                                   (U[c + sx] + U[c + sx - 1] - U[c - sx] - U[c - sx - 1] + UB[c + sx] + UB[c + sx - 1] -
                                    UB[c - sx] - UB[c - sx - 1]) *
                                   odx;
                const double D22 = 0.50 *
                                   (V[c + sy] + V[c + sy - 1] - V[c - sy] - V[c - sy - 1] + VB[c + sy] + VB[c + sy - 1] -
                                    VB[c - sy] - VB[c - sy - 1]) *
                                   ody;
                const double D33 = 1.0 * (W[c + 1] - W[c - 1] + WB[c + 1] - WB[c - 1]) * odzw;
                const double D12 =
                    0.5 * ((U[c + sy] + U[c + sy - 1] - U[c - sy] - U[c - sy - 1] + UB[c + sy] + UB[c + sy - 1] -
                            UB[c - sy] - UB[c - sy - 1]) *
                               ody +
                           (V[c + sx] + V[c + sx - 1] - V[c - sx] - V[c - sx - 1] + VB[c + sx] + VB[c + sx - 1] -
                            VB[c - sx] - VB[c - sx - 1]) *
                               odx);
                const double D13 = 0.5 * ((U[c] + U[c + sx] - U[c - 1] - U[c + sx - 1] + UB[c] + UB[c + sx] -
                                           UB[c - 1] - UB[c + sx - 1]) *
                                              odzw +
                                          (W[c + sx] - W[c - sx] + WB[c + sx] - WB[c - sx]) * odx);
                const double D23 = 0.5 * ((V[c] + V[c + sy] - V[c - 1] - V[c + sy - 1] + VB[c] + VB[c + sy] -
                                           VB[c - 1] - VB[c + sy - 1]) *
                                              odzw +
                                          (W[c + sy] - W[c - sy] + WB[c + sy] - WB[c - sy]) * ody);
                const double S2 = D11 * D11 + D22 * D22 + D33 * D33 + D12 * D12 + D13 * D13 + D23 * D23;
                double bruntv;
                if (!moist) {
                    const double hi = (TH[c] + THB[c] + S->tb[k]) * (1 + 0.61 * S->qb[k]);
                    const double lo = (TH[c - 1] + THB[c - 1] + S->tb[k - 1]) * (1 + 0.61 * S->qb[k - 1]);
                    bruntv = 2.0 * grav / (S->tbv[k] + S->tbv[k - 1]) * (hi - lo) * odzw;
                } else {
                    const double *QV = S->M[F_QV], *QC = S->M[F_QC], *QR = S->M[F_QR], *PI = S->pi;
                    if (!S->sat[c] || !S->sat[c - 1]) {
                        const double hi = (TH[c] + THB[c] + S->tb[k]) * (1 + 0.61 * (QV[c] + QB[c] + S->qb[k]));
                        const double lo =
                            (TH[c - 1] + THB[c - 1] + S->tb[k - 1]) * (1 + 0.61 * (QV[c - 1] + QB[c - 1] + S->qb[k - 1]));
                        bruntv = 2.0 * grav / (S->tbv[k] + S->tbv[k - 1]) * (hi - lo) * odzw;
                    } else {
                        double hi = TH[c] + THB[c] + S->tb[k];
                        double lo = TH[c - 1] + THB[c - 1] + S->tb[k - 1];
                        const double tH = hi * (PB[c] + PI[c] / (cp * S->tbv[k]));
                        const double tL = lo * (PB[c - 1] + PI[c - 1] / (cp * S->tbv[k - 1]));
                        const double temp = 0.5 * (tH + tL);
                        const double dQL = QC[c] + QR[c] - QC[c - 1] - QR[c - 1] + QV[c] - QV[c - 1] + QB[c] - QB[c - 1] +
                                           S->qb[k] - S->qb[k - 1];
                        const double qv = 0.5 * (QV[c] + QV[c - 1] + QB[c] + QB[c - 1] + S->qb[k] + S->qb[k - 1]);
                        const double pdH = p0 * pow(PB[c], cpRd) + PI[c] * S->rhou[k];
                        const double pdL = p0 * pow(PB[c - 1], cpRd) + PI[c - 1] * S->rhou[k - 1];
                        const double eH = 611.2 * exp(17.67 * (tH - 273.15) / (tH - 29.65));
                        const double eL = 611.2 * exp(17.67 * (tL - 273.15) / (tL - 29.65));
                        const double qsH = 0.62197 * eH / (pdH - eH);
                        const double qsL = 0.62197 * eL / (pdL - eL);
                        hi = hi * (1 + Lv * qsH / (cp * tH));
                        lo = lo * (1 + Lv * qsL / (cp * tL));
                        const double A = (grav / S->tbw[k]) * (1.0 + Lv * qv / (Rd * temp)) /
                                         (1.0 + 0.622 * Lv * Lv * qv / (cp * Rd * temp * temp));
                        bruntv = (A * (hi - lo) - grav * dQL) * odzw;
                    }
                }
                if (S2 - tb_one_d_Pr * bruntv > 0) {
                    const double cc = S->l2[k] * tb_cs * tb_cs;
                    S->kmix[c] = cc * sqrt(S2 - tb_one_d_Pr * bruntv);
                    S->khmix[c - 1] = 0.5 * (S->kmix[c - 1] / S->l2[k - 1] + S->kmix[c] / S->l2[k]) * S->lH * S->lH;
                    if (S->kmix[c] > S->kvmax[k]) S->kmix[c] = S->kvmax[k];
                    if (S->khmix[c - 1] > S->kmixh_max) S->khmix[c - 1] = S->kmixh_max;
                } else {
                    S->kmix[c] = 0;
                    S->khmix[c - 1] = 0 + 0.5 * S->kmix[c - 1] / S->l2[k - 1] * S->lH * S->lH;
                }
            }
        }
}
/* the deformation-rate components of turbulent_diffusion_velocity
 * (turbulence.cpp:918-932) at a point of the start-of-step fields; the
 * vertical ones are zero at level 0 (the reference never writes them there) */
static double tau11(const ora_state *S, int i, int j, int k)
{
    const double *U = S->M[F_U];
    return 2.0 * (U[IX(i + 1, j, k)] - U[IX(i, j, k)]) * S->one_d_dx;
}
static double tau22(const ora_state *S, int i, int j, int k)
{
    const double *V = S->M[F_V];
    return 2.0 * (V[IX(i, j + 1, k)] - V[IX(i, j, k)]) * S->one_d_dy;
}
static double tau33(const ora_state *S, int i, int j, int k)
{
    const double *W = S->M[F_W];
    if (k == 0) return 0;
    return 2.0 * (W[IX(i, j, k + 1)] - W[IX(i, j, k)]) * (S->one_d_dz * S->mu[k]);
}
static double tau13(const ora_state *S, int i, int j, int k)
{
    const double *U = S->M[F_U], *W = S->M[F_W];
    if (k == 0) return 0;
    return (W[IX(i + 1, j, k + 1)] - W[IX(i, j, k + 1)]) * S->one_d_dx +
           (U[IX(i + 1, j, k + 1)] - U[IX(i + 1, j, k)]) * (S->one_d_dz * S->mw[k + 1]);
}
static double tau23(const ora_state *S, int i, int j, int k)
{
    const double *V = S->M[F_V], *W = S->M[F_W];
    if (k == 0) return 0;
    return (W[IX(i, j + 1, k + 1)] - W[IX(i, j, k + 1)]) * S->one_d_dy +
           (V[IX(i, j + 1, k + 1)] - V[IX(i, j + 1, k)]) * (S->one_d_dz * S->mw[k + 1]);
}
static double tau12(const ora_state *S, int i, int j, int k)
{
    const double *U = S->M[F_U], *V = S->M[F_V];
    return (U[IX(i + 1, j + 1, k)] - U[IX(i + 1, j, k)]) * S->one_d_dy +
           (V[IX(i + 1, j + 1, k)] - V[IX(i, j + 1, k)]) * S->one_d_dx;
}

/* wind speed of the full and of the basic-state wind at the lowest level */
static void surface_wind(const ora_state *S, long c, double *ws, double *wsb)
{
    const double u = S->M[F_U][c], v = S->M[F_V][c], ub = S->bar[0][c], vb = S->bar[1][c];
    *ws = sqrt((u + ub) * (u + ub) + (v + vb) * (v + vb));
    *wsb = sqrt(ub * ub + vb * vb);
}

/* turbulent_diffusion_velocity (turbulence.cpp:839-1022): the ocean drag
 * (:899-905) at the lowest level, the stress divergences above */
static void turb_velocity(ora_state *S)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    const double *KM = S->kmix, *KH = S->khmix, *U = S->M[F_U], *V = S->M[F_V];
    const double *UB = S->bar[0], *VB = S->bar[1];
    double *fu = S->ttend[0], *fv = S->ttend[1], *fw = S->ttend[2];
    const double odx = S->one_d_dx, ody = S->one_d_dy;
#define KMX(a, b, c) KM[IX(a, b, c)]
#define KHX(a, b, c) KH[IX(a, b, c)]
    for (int i = 1; i < NX - 1; i++)
        for (int j = 1; j < NY - 1; j++) {
            double ws, wsb;
            const long c1 = IX(i, j, 1);
            surface_wind(S, c1, &ws, &wsb);
            const double drag = (1.1e-3 + 4.0e-5 * ws);
            double tau_u_zl = drag * (ws * U[c1] + (ws - wsb) * UB[c1]);
            double tau_v_zl = drag * (ws * V[c1] + (ws - wsb) * VB[c1]);
            for (int k = 1; k < NZ - 1; k++) {
                const double odz = S->one_d_dz * S->mu[k], odzw = S->one_d_dz * S->mw[k];
                const double uK11H_h = KHX(i, j, k);
                const double uK11H_l = KHX(i - 1, j, k);
                const double uK12H_h = 0.25 * (KHX(i, j, k) + KHX(i - 1, j, k) + KHX(i - 1, j + 1, k) + KHX(i, j + 1, k));
                const double uK12H_l = 0.25 * (KHX(i, j - 1, k) + KHX(i - 1, j - 1, k) + KHX(i - 1, j, k) + KHX(i, j, k));
                const double uK13V_h = 0.50 * (KMX(i, j, k + 1) + KMX(i - 1, j, k + 1));
                const double vK12H_h = 0.25 * (KHX(i, j - 1, k) + KHX(i, j, k) + KHX(i + 1, j - 1, k) + KHX(i + 1, j, k));
                const double vK12H_l = uK12H_l;
                const double vK22H_h = KHX(i, j, k);
                const double vK22H_l = KHX(i, j - 1, k);
                const double vK23V_h = 0.5 * (KMX(i, j, k + 1) + KMX(i, j - 1, k + 1));
                const double wK13H_h = 0.25 * (KHX(i, j, k) + KHX(i, j, k - 1) + KHX(i + 1, j, k) + KHX(i + 1, j, k - 1));
                const double wK13H_l = 0.25 * (KHX(i, j, k) + KHX(i, j, k - 1) + KHX(i - 1, j, k) + KHX(i - 1, j, k - 1));
                const double wK23H_h = 0.25 * (KHX(i, j, k) + KHX(i, j, k - 1) + KHX(i, j + 1, k) + KHX(i, j + 1, k - 1));
                const double wK23H_l = 0.25 * (KHX(i, j, k) + KHX(i, j, k - 1) + KHX(i, j - 1, k) + KHX(i, j - 1, k - 1));
                const double wK33V_h = 0.50 * (KMX(i, j, k) + KMX(i, j, k + 1));
                const double wK33V_l = 0.50 * (KMX(i, j, k) + KMX(i, j, k - 1));
                const double t13w = tau13(S, i - 1, j, k), t23s = tau23(S, i, j - 1, k);
                const long c = IX(i, j, k);
                fu[c] = (uK11H_h * tau11(S, i, j, k) - uK11H_l * tau11(S, i - 1, j, k)) * odx +
                        (uK12H_h * tau12(S, i - 1, j, k) - uK12H_l * tau12(S, i - 1, j - 1, k)) * ody +
                        (uK13V_h * t13w - tau_u_zl) * odz;
                fv[c] = (vK12H_h * tau12(S, i, j - 1, k) - vK12H_l * tau12(S, i - 1, j - 1, k)) * odx +
                        (vK22H_h * tau22(S, i, j, k) - vK22H_l * tau22(S, i, j - 1, k)) * ody +
                        (vK23V_h * t23s - tau_v_zl) * odz;
                fw[c] = (wK13H_h * tau13(S, i, j, k - 1) - wK13H_l * tau13(S, i - 1, j, k - 1)) * odx +
                        (wK23H_h * tau23(S, i, j, k - 1) - wK23H_l * tau23(S, i, j - 1, k - 1)) * ody +
                        (wK33V_h * tau33(S, i, j, k) - wK33V_l * tau33(S, i, j, k - 1)) * odzw;
                tau_u_zl = uK13V_h * t13w;
                tau_v_zl = vK23V_h * t23s;
            }
        }
#undef KMX
#undef KHX
}

/* the scalar flux divergence of turbulent_diffusion_scalars / _theta
 * (turbulence.cpp:1116-1173): horizontal fluxes with the Prandtl-scaled
 * coefficients averaged to the faces, the vertical flux carried upward from
 * the surface value tau_l */
static double scalar_divergence(const ora_state *S, const double *q, int i, int j, int k, double tau_l,
                                double *tau_h)
{
    const double *KM = S->kmix, *KH = S->khmix, P = tb_one_d_Pr;
    const long c = IX(i, j, k), sx = (long)S->NY * S->NZ, sy = S->NZ;
    const double odx = S->one_d_dx, ody = S->one_d_dy;
    const double th = -P * KM[c + 1] * (q[c + 1] - q[c]) * (S->one_d_dz * S->mw[k + 1]);
    double KHh = 0.5 * (P * KH[c + sy] + P * KH[c]);
    double KLl = 0.5 * (P * KH[c] + P * KH[c - sy]);
    const double t22h = -KHh * (q[c + sy] - q[c]) * ody;
    const double t22l = -KLl * (q[c] - q[c - sy]) * ody;
    KHh = 0.5 * (P * KH[c + sx] + P * KH[c]);
    KLl = 0.5 * (P * KH[c] + P * KH[c - sx]);
    const double t11h = -KHh * (q[c + sx] - q[c]) * odx;
    const double t11l = -KLl * (q[c] - q[c - sx]) * odx;
    *tau_h = th;
    return -((t11h - t11l) * odx + (t22h - t22l) * ody + (th - tau_l) * (S->one_d_dz * S->mu[k]));
}

/* turbulent_diffusion_scalars (moist, turbulence.cpp:1027-1183) and
 * turbulent_diffusion_theta (dry, :1190-1276); the ocean surface fluxes of
 * heat and vapour (:1083-1104) when SURFACE_HEAT_FLUX is set */
static void turb_scalars(ora_state *S)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ, moist = S->c.microphysics_option != 0;
    const double cpRd = cp / Rd;
    const double dp_to_surface = grav * S->zsu[1] / (cp * S->tbv[1]);
    for (int i = 1; i < NX - 1; i++)
        for (int j = 1; j < NY - 1; j++) {
            double tl[4] = {0, 0, 0, 0}; /* theta, qv, qc, qr */
            const long c1 = IX(i, j, 1);
            if (moist && S->c.use_surface_heat_flux) {
                double ws, wsb;
                surface_wind(S, c1, &ws, &wsb);
                const double drag = (1.1e-3 + 4.0e-5 * ws) * 1.0 * 1.0;
                const double PB = S->bar[5][c1], PI = S->pi[c1];
                const double pressure = p0 * pow(PB + dp_to_surface, cpRd) + PI * S->rhou[1];
                const double pisfc = PB + PI / (cp * S->tbv[1]) + dp_to_surface;
                const double qvs = 0.62197 * S->es_water / (pressure - S->es_water);
                const double tsb = (S->bar[3][c1] + S->tb[1]) * pisfc;
                const double tsp = S->M[F_TH][c1] * pisfc;
                tl[1] = drag * ((ws - wsb) * (qvs - S->bar[4][c1] - S->qb[1]) - ws * S->M[F_QV][c1]);
                tl[0] = drag * ((ws - wsb) * (S->water_temp - tsb) - ws * tsp);
            }
            const int nf = moist ? 4 : 1;
            for (int k = 1; k < NZ - 1; k++) {
                const long c = IX(i, j, k);
                for (int n = 0; n < nf; n++) {
                    double th;
                    S->ttend[3 + n][c] = scalar_divergence(S, S->M[F_TH + n], i, j, k, tl[n], &th);
                    tl[n] = th;
                }
            }
        }
}

/* calculate_diff_tend (turbulence.cpp:158-188) over i, j in [1, N-1) */
static void op_turbulence(ora_state *S)
{
    turb_kmix(S);
    turb_velocity(S);
    turb_scalars(S);
}

/* apply_velocity_diffusion (turbulence.cpp:233-256) over i, j in [3, N-3):
 * u and v from level 1, w from level 2 */
static void turb_apply_velocity(ora_state *S, double step)
{
    const double deltaT = step * S->dt;
    for (int i = 3; i < S->NX - 3; i++)
        for (int j = 3; j < S->NY - 3; j++) {
            long c = IX(i, j, 1);
            S->P[F_U][c] += S->ttend[0][c] * deltaT;
            S->P[F_V][c] += S->ttend[1][c] * deltaT;
            for (int k = 2; k < S->NZ - 1; k++) {
                c = IX(i, j, k);
                S->P[F_U][c] += S->ttend[0][c] * deltaT;
                S->P[F_V][c] += S->ttend[1][c] * deltaT;
                S->P[F_W][c] += S->ttend[2][c] * deltaT;
            }
        }
}

/* apply_scalar_diffusion (:263-273) and apply_moisture_diffusion (:278-291)
 * over i, j in [1, N-1) */
static void turb_apply_theta(ora_state *S, double step)
{
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long c = IX(i, j, k);
                S->P[F_TH][c] += S->ttend[3][c] * step * S->dt;
            }
}

static void turb_apply_moisture(ora_state *S, double step)
{
    const double deltaT = step * S->dt;
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long c = IX(i, j, k);
                S->P[F_QV][c] += S->ttend[4][c] * deltaT;
                S->P[F_QC][c] += S->ttend[5][c] * deltaT;
                S->P[F_QR][c] += S->ttend[6][c] * deltaT;
            }
}

/* ------------------------------------------------------------------------
 * Kessler warm rain: run_kessler_microphysics (kessler.cpp:25-213).
 * ---------------------------------------------------------------------- */
static void kessler_points(ora_state *S)
{
    const double cpRd = cp / Rd;
    double *THP = S->P[F_TH], *QVP = S->P[F_QV], *QCP = S->P[F_QC], *QRP = S->P[F_QR];
    const double *THBAR = S->bar[3], *QBAR = S->bar[4], *PBAR = S->bar[5], *PI = S->pi;
    const double dt = S->dt;
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                long ix = IX(i, j, k);
                const double rhou = S->rhou[k];
                double theta = THP[ix] + THBAR[ix] + S->tb[k];
                /* CONVERT_PRESSURE (kessler.cpp:7-11): the hydrostatic set's pi is
                 * already the Exner perturbation */
                double pressure = (S->c.hydrostatic ? PI[ix] : PI[ix] / (cp * S->tbv[k])) + PBAR[ix];
                double vapor = QVP[ix] + QBAR[ix] + S->qb[k];
                double temperature = theta * pressure;
                double pd = p0 * pow(pressure, cpRd);
                double A, B, E, esl, qvsat;
                if (QCP[ix] > 1.0e-3) A = 0.001 * (QCP[ix] - 1.0e-3) * dt;
                else A = 0;
                if (QRP[ix] > minvar) B = rhou * 2.2 * QCP[ix] * pow(QRP[ix], 0.875) * dt;
                else B = 0;
                if (QRP[ix] > minvar) {
                    esl = 611.2 * exp(17.67 * (temperature - 273.15) / (temperature - 29.65));
                    qvsat = 0.62197 * esl / (pd - esl);
                    double cvent = 1.6 + 30.3922 * pow(rhou * QRP[ix], 0.2046);
                    E = (1.0 / rhou) *
                        (((1.0 - vapor / qvsat) * cvent * pow(rhou * QRP[ix], 0.525)) /
                         (2.03e4 + 9.58e6 / (pd * qvsat))) *
                        dt;
                    E = fmin(QRP[ix], E);
                    E = fmax(E, 0.0);
                    if (E > 100) S->err = GA_ERR_KESSLER;
                } else
                    E = 0;
                QVP[ix] += E;
                double total_convert = fmin(A + B, QCP[ix]);
                QCP[ix] -= total_convert;
                QRP[ix] += (total_convert - E);
                double de = (Lv / (cp * pressure)) * E;
                THP[ix] -= de;
                /* saturation adjustment (:119-176) */
                theta = THP[ix] + THBAR[ix] + S->tb[k];
                vapor = QVP[ix] + QBAR[ix] + S->qb[k];
                temperature = theta * pressure;
                esl = 611.2 * exp(17.67 * (temperature - 273.15) / (temperature - 29.65));
                qvsat = 0.62197 * esl / (pd - esl);
                const double f = 17.67 * (273.15 - 29.65) * Lv / cp;
                /* pow(x,2) is folded to x*x by the reference's compiler */
                double tm = temperature - 29.65;
                double phi = pd / (pd - esl) * qvsat * f / (tm * tm);
                double C = 0.0;
                if (vapor > qvsat) {
                    C = (vapor - qvsat) / (1.0 + phi);
                    if (S->sat) S->sat[ix] = 1;
                } else if (vapor < qvsat && QCP[ix] > 0) {
                    C = -fmin(QCP[ix], (qvsat - vapor) / (1.0 + phi));
                    if (S->sat) S->sat[ix] = -C < QCP[ix];
                } else if (S->sat) {
                    S->sat[ix] = vapor == qvsat;  /* kessler.cpp:141-163 */
                }
                QCP[ix] += C;
                QVP[ix] -= C;
                double dc = (Lv / (cp * pressure)) * C;
                THP[ix] += dc;
            }
}

/* PPM semi-Lagrangian fallout: hydrometeor_fallout (microphysics.cpp:210-292),
 * piecewise_parabolic_interp (:516-579), calculate_edge_values (:590-637),
 * integrate_parabolic (:339-350), below_surface_rainfall (:355-370). */
static double integrate_parabolic(const double *zin, const double *qin, int p, double zl, double zh,
                                  const double *qp, const double *qn)
{
    double t0 = (zl - zin[p]) / (zin[p + 1] - zin[p]);
    double t1 = (zh - zin[p]) / (zin[p + 1] - zin[p]);
    double high = (qp[p] + qn[p] - 2.0 * qin[p]) * t1 * t1 * t1 -
                  (qp[p] + 2.0 * qn[p] - 3.0 * qin[p]) * t1 * t1 + qn[p] * t1;
    double low = (qp[p] + qn[p] - 2.0 * qin[p]) * t0 * t0 * t0 -
                 (qp[p] + 2.0 * qn[p] - 3.0 * qin[p]) * t0 * t0 + qn[p] * t0;
    return high - low;
}
static void edge_values(ora_state *S, const double *zin, const double *qin, int n)
{
    double *qp = S->qp_edges, *qn = S->qn_edges, *mono = S->mono;
    for (int k = 1; k < n - 1; k++) {
        double dq = 0.25 * (qin[k + 1] - qin[k - 1]);
        double dmax = fmax(qin[k + 1], fmax(qin[k], qin[k - 1])) - qin[k];
        double dmin = qin[k] - fmin(qin[k + 1], fmin(qin[k], qin[k - 1]));
        mono[k] = sgn(dq) * fmin(fabs(dq), fmin(dmax, dmin));
    }
    mono[0] = mono[1];
    mono[n - 1] = mono[n - 2];
    for (int k = 1; k < n - 1; k++) {
        qn[k] = (qin[k - 1] * (zin[k + 1] - zin[k]) + qin[k] * (zin[k] - zin[k - 1])) /
                    (zin[k + 1] - zin[k - 1]) -
                (mono[k] - mono[k - 1]) / 3.0;
        qp[k - 1] = qn[k];
    }
    /* qp[n-2] is not set above: it keeps the value of the previous call */
    qp[n - 1] = qin[n - 1];
    qp[0] = qin[0];
    qn[n - 1] = qin[n - 1];
    qn[0] = qin[0];
    for (int k = 0; k < n; k++) {
        qn[k] = qin[k] - sgn(mono[k]) * fmin(fabs(2.0 * mono[k]), fabs(qn[k] - qin[k]));
        qp[k] = qin[k] + sgn(mono[k]) * fmin(fabs(2.0 * mono[k]), fabs(qp[k] - qin[k]));
    }
}
static double ppm_remap(ora_state *S, const double *zin, const double *zout, const double *qin,
                        double *qout, int n)
{
    memset(qout, 0, sizeof(double) * n);
    int hn = 1;
    /* the reference accumulates into an uninitialised local here; 0 is used */
    double rainfall = 0.0;
    for (int j = 1; j < n - 2; j++)
        if (zin[j] < 0 && zin[j + 1] < 0) {
            rainfall += qin[j] * (zin[j + 1] - zin[j]);
            hn = j + 1;
        }
    edge_values(S, zin, qin, n);
    const double *qp = S->qp_edges, *qn = S->qn_edges;
    if (zin[hn] < 0)
        rainfall += integrate_parabolic(zin, qin, hn, zin[hn], 0, qp, qn) * -zin[hn] *
                    ((zin[hn + 1] - zin[hn]) / -zin[hn]);
    for (int i = 0; i < n - 1; i++)
        for (int j = 0; j < n - 1; j++) {
            double scale = (zin[j + 1] - zin[j]) / (zout[i + 1] - zout[i]);
            if (zout[i] < zin[j] && zout[i + 1] < zin[j + 1] && zout[i + 1] > zin[j])
                qout[i] = qout[i] + integrate_parabolic(zin, qin, j, zin[j], zout[i + 1], qp, qn) * scale;
            if (zout[i] < zin[j + 1] && zout[i + 1] > zin[j + 1] && zout[i] > zin[j])
                qout[i] = qout[i] + integrate_parabolic(zin, qin, j, zout[i], zin[j + 1], qp, qn) * scale;
            if (zout[i] >= zin[j] && zout[i + 1] <= zin[j + 1])
                qout[i] = qout[i] + integrate_parabolic(zin, qin, j, zout[i], zout[i + 1], qp, qn) * scale;
            if (zout[i] < zin[j] && zout[i + 1] > zin[j + 1])
                qout[i] = qout[i] + integrate_parabolic(zin, qin, j, zin[j], zin[j + 1], qp, qn) * scale;
        }
    return rainfall;
}
static void fallout(ora_state *S, double *var, const double *vel, double *acc)
{
    const int NZ = S->NZ;
    const double *ZW = S->zsw;
    const double DeCFL0 = 0.05, dt = S->dt;
    double *ZA = S->za, *QA = S->qa, *QD = S->qd, *Ve = S->ve;
    for (int k = 0; k < NZ; k++) { ZA[k] = ZW[k]; Ve[k] = 0; QD[k] = 0; QA[k] = 0; }
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++) {
            int has = 0;
            for (int k = 1; k < NZ; k++)
                if (var[IX(i, j, k)] > minvar) { has = 1; break; }
            if (!has) continue;
            for (int k = 1; k < NZ; k++) Ve[k] = 0.5 * (vel[IX(i, j, k)] + vel[IX(i, j, k - 1)]);
            Ve[0] = Ve[1];
            for (int k = NZ - 2; k >= 0; k--) {
                double dzu = ZW[k + 1] - ZW[k];
                double decfl = (Ve[k + 1] - Ve[k]) * dt / dzu;
                if (decfl >= DeCFL0) Ve[k] = Ve[k + 1] - DeCFL0 * dzu / dt;
            }
            for (int k = 0; k < NZ - 1; k++) ZA[k] = ZW[k] - dt * Ve[k];
            for (int k = 0; k < NZ - 1; k++)
                QA[k] = S->rhou[k] * var[IX(i, j, k)] * (ZW[k + 1] - ZW[k]) / (ZA[k + 1] - ZA[k]);
            acc[IX2(i, j)] += ppm_remap(S, ZA, ZW, QA, QD, NZ);
            for (int k = 0; k < NZ; k++) var[IX(i, j, k)] = QD[k] * S->one_d_rhou[k];
        }
}

static void op_kessler(ora_state *S) /* run_microphysics(1,NX-1,1,NY-1) */
{
    if (S->c.microphysics_option != 1) return;
    kessler_points(S);
    if (S->c.rain_fallout == 2) {
        fall_speed(S, S->P[F_QR], 1, S->NX - 1, 1, S->NY - 1);
        fallout(S, S->P[F_QR], S->vt, S->accrain);
        memset(S->vt, 0, sizeof(double) * S->N);
    } else {
        /* precip_rate (microphysics.cpp:143-160) */
        for (int i = 1; i < S->NX - 1; i++)
            for (int j = 1; j < S->NY - 1; j++)
                S->accrain[IX2(i, j)] += S->rhow[1] * 0.5 *
                                         (S->vt[IX(i, j, 0)] + S->vt[IX(i, j, 1)]) * 0.5 *
                                         (S->P[F_QR][IX(i, j, 0)] + S->P[F_QR][IX(i, j, 1)]) * S->dt;
    }
}

/* ------------------------------------------------------------------------
 * Ice microphysics: run_rutledge_microphysics (rutledge.cpp:150-452), the
 * point processes of Rutledge and Hobbs (1983) with the changes of Hong et
 * al. (2004), then saturation_adjustment (:700-820) with get_qvsat (:611-693),
 * zero_moisture, and the rain, ice and snow fallout.
 * ---------------------------------------------------------------------- */
#define RUT_ESL(t) (611.2 * exp(17.67 * ((t) - 273.15) / ((t) - 29.65)))      /* SAT_VAP_WAT */
#define RUT_ESI(t) (611.2 * exp(21.8745584 * ((t) - 273.15) / ((t) - 7.66))) /* SAT_VAP_ICE */
#define RUT_QSAT(e, p) (0.62197 * (e) / ((p) - (e)))                         /* SAT_MIX_RATIO */
#define RUT_ALPHA(x) (1.0 + ((x) - 273.15) / (rut_tmax - rut_tmin))

static void rutledge_points(ora_state *S)
{
    const double cpRd = cp / Rd, dt = S->dt;
    const double a0 = -0.267, a1 = 5.15e3, a2 = -1.0225e6, a3 = 7.55e7; /* rain fall-speed polynomial */
    double *THP = S->P[F_TH], *QVP = S->P[F_QV], *QCP = S->P[F_QC], *QRP = S->P[F_QR];
    double *QIP = S->P[F_QI], *QSP = S->P[F_QS];
    const double *THBAR = S->bar[3], *QBAR = S->bar[4];
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long ix = IX(i, j, k);
                const double rhou = S->rhou[k], odr = S->one_d_rhou[k];
                double theta = THP[ix] + THBAR[ix] + S->tb[k];
                double pressure = rut_pressure(S, ix, k);
                double vapor = QVP[ix] + QBAR[ix] + S->qb[k];
                double temperature = theta * pressure;
                double pd = p0 * pow(pressure, cpRd);
                double esl = RUT_ESL(temperature), esi = RUT_ESI(temperature);
                double qvl_sat = RUT_QSAT(esl, pd), qvi_sat = RUT_QSAT(esi, pd);
                double pcond = 0, lambdaS, lambdaR, var, Ap, Bp, App = 0, Bpp = 0;
                if (QSP[ix] != 0) {
                    S->n0s = fmin(2.0e6 * exp(0.12 * (273.16 - temperature)), 2.0e8);
                    lambdaS = sqrt(sqrt((trigpi * rhoS * S->n0s) / (rhou * QSP[ix])));
                } else
                    lambdaS = 0;
                const double N0S = S->n0s;
                /* rain: autoconversion, accretion, evaporation, freezing */
                double A = 0, B = 0, E = 0, prfrz = 0;
                if (QCP[ix] > 1.0e-3) A = 0.001 * (QCP[ix] - 1.0e-3) * dt;
                if (QRP[ix] > rut_minvar) {
                    lambdaR = pow((trigpi * 1000 * N0r) / (rhou * QRP[ix]), 0.25);
                    B = 0.25 * trigpi * QCP[ix] * ERC * N0r * pow(p0 / pd, 0.4) * 2 / pow(lambdaR, 3) *
                        (a0 + a1 * 3 / lambdaR + a2 * 12 / (lambdaR * lambdaR) +
                         a3 * 60 / (lambdaR * lambdaR * lambdaR)) *
                        dt;
                    Ap = (Lv / (Ka * temperature)) * ((Lv * Mw) / (Rstar * temperature) - 1);
                    Bp = Rstar * temperature / (chi * Mw * esl);
                    var = 0.78 / (lambdaR * lambdaR) +
                          0.31 * sqrt(ap_lin * rhou / mu_s) / (lambdaR * lambdaR * lambdaR) * 2.0 * pow((p0 / pd), 0.2);
                    E = var * 2 * trigpi * N0r * (vapor / qvl_sat - 1.0) / (Ap + Bp) * dt * odr;
                    if (temperature < 273.16) {
                        prfrz = 20 * trigpi * trigpi * 100.0 * N0r * (1000.0 / rhou) *
                                exp(0.66 * (273.16 - temperature) - 1) /
                                (lambdaR * lambdaR * lambdaR * lambdaR * lambdaR * lambdaR * lambdaR);
                        prfrz = fmin(prfrz * odr * dt, QRP[ix]);
                    }
                    if (E > 100) S->err = GA_ERR_KESSLER;
                }
                /* cloud ice: initiation, deposition, autoconversion to snow,
                 * collection by snow, melting */
                double pint = 0, pdepi = 0, pconv = 0, psaci = 0, psmlti = 0;
                if (temperature < 273.16) {
                    double nc0 = 1.0e3 * exp(0.1 * (273.16 - temperature));
                    double nc = fmin(fmax(5.38e7 * pow(rhou * QIP[ix], 0.75), 1.0e3), 1.0e6);
                    if (qvi_sat < vapor) pint = fmin(M0 * nc0 / rhou, vapor - qvi_sat);
                    if (QIP[ix] > rut_minvar || QSP[ix] > rut_minvar) {
                        App = (Lv / (Ka * temperature)) * ((Ls * Mw) / (Rstar * temperature) - 1);
                        Bpp = Rstar * temperature / (chi * Mw * esi);
                        double MI = rhou * QIP[ix] / nc;
                        double Dl = 11.3 * sqrt(MI);
                        pdepi = (4 * Dl * (vapor / qvi_sat - 1) * nc) / (App + Bpp) * odr * dt;
                    }
                    if (QIP[ix] > rut_minvar) {
                        double qimax;
                        if (temperature > 233.16 && pd > 30000) qimax = 8.0e-5 * odr;
                        else qimax = 0.18e-3;
                        if (QIP[ix] > qimax) pconv = QIP[ix] - qimax;
                    }
                    if (QIP[ix] > rut_minvar && lambdaS > 1e-15) {
                        double ESI = exp(0.05 * (temperature - 273.16));
                        psaci = (trigpi * app * QIP[ix] * ESI * N0S) / 4 * pow(p0 / pd, 0.4) * 2.22 /
                                pow(lambdaS, 3.11) * dt;
                    }
                } else
                    psmlti = QIP[ix];
                /* snow: melting, deposition, evaporation of melting snow */
                double psmlt = 0, psdep = 0, pmltev = 0;
                if (QSP[ix] > rut_minvar && lambdaS > 1e-15) {
                    var = 0.65 / (lambdaS * lambdaS) +
                          0.44 * sqrt(app * rhou / mu_s) * pow(p0 / pd, 0.2) * 1.383 / pow(lambdaS, 2.555);
                    if (temperature > 273.16) {
                        psmlt = -(2 * trigpi * N0S / Lf) * Ka * (temperature - 273.16) * var;
                        psmlt = dt * psmlt * odr;
                    }
                    if (temperature < 273.16) {
                        psdep = 4 * (vapor / qvi_sat - 1) * N0S / (App + Bpp) * var;
                        psdep = dt * psdep * odr;
                    }
                    if (temperature >= 273.16) {
                        Ap = (Lv / (Ka * temperature)) * ((Lv * Mw) / (Rstar * temperature) - 1);
                        Bp = Rstar * temperature / (chi * Mw * esl);
                        pmltev = 4 * (vapor / qvl_sat - 1) * N0S / (Ap + Bp) * var;
                        pmltev = dt * pmltev * odr;
                    }
                    if (fabs(psmlt) > 100) S->err = GA_ERR_KESSLER;
                }
                /* cloud water collected by snow, frozen below tmin */
                double psacw_cold = 0, psacw_warm = 0;
                if (QCP[ix] > rut_minvar && lambdaS > 1e-15) {
                    double psacw = (trigpi * app * QCP[ix] * ESC * N0S) / 4 * pow(p0 / pd, 0.4) * 2.22 /
                                   pow(lambdaS, 3.11) * dt;
                    if (temperature < 273.16) psacw_cold = psacw;
                    else psacw_warm = psacw;
                }
                double pcfrz = 0;
                if (temperature < rut_tmin) pcfrz = QCP[ix];
                double pint_p_pdepi = fmin(pint + pdepi, vapor);
                pint_p_pdepi = -fmin(-pint_p_pdepi, QIP[ix]);
                QVP[ix] += -(pcond + E + psdep + pmltev + pint_p_pdepi);
                QCP[ix] += pcond + psmlti - A - B - psacw_warm - psacw_cold - pcfrz;
                QIP[ix] += pint_p_pdepi - psmlti - psaci - pconv + pcfrz;
                QRP[ix] += E + A + B - psmlt + psacw_warm - prfrz;
                QSP[ix] += psdep + pmltev + psaci + psmlt + psacw_cold + pconv + prfrz;
                double diabatic = Lv / (cp * S->pib[k]) * (pcond + E + pmltev) +
                                  Ls / (cp * S->pib[k]) * (pint_p_pdepi + psdep) +
                                  Lf / (cp * S->pib[k]) * (psmlt + psmlti + psacw_cold + pcfrz + prfrz);
                THP[ix] += diabatic;
            }
}

/* get_qvsat (rutledge.cpp:611-693): saturation mixing ratio over water, ice
 * or the temperature-weighted mix, and the latent-heating correction terms;
 * pow(x,2) is folded to x*x by the reference's compiler */
static double rut_qvsat(double T, double pd, double *phi, double *phil, double *phii)
{
    double qvsat;
    if (T > rut_tmax) {
        double esl = RUT_ESL(T);
        qvsat = RUT_QSAT(esl, pd);
        double f = 17.67 * (273.15 - 29.65) * Lv / cp, tm = T - 29.65;
        *phi = *phil = *phii = pd / (pd - esl) * qvsat * f / (tm * tm);
    } else if (T < rut_tmin) {
        double esl = RUT_ESI(T);
        qvsat = RUT_QSAT(esl, pd);
        double f = 21.8745584 * (273.15 - 7.66) * Ls / cp, tm = T - 7.66;
        *phi = *phil = *phii = pd / (pd - esl) * qvsat * f / (tm * tm);
    } else {
        double esl = RUT_ESL(T), esi = RUT_ESI(T);
        double qvl_sat = RUT_QSAT(esl, pd), qvi_sat = RUT_QSAT(esi, pd);
        double fl = 17.67 * (273.15 - 29.65) * Lv / cp, fi = 21.8745584 * (273.15 - 7.66) * Ls / cp;
        double tl = T - 29.65, ti = T - 7.66;
        *phil = pd / (pd - esl) * qvl_sat * fl / (tl * tl);
        *phii = pd / (pd - esi) * qvi_sat * fi / (ti * ti);
        qvsat = RUT_ALPHA(T) * qvl_sat + (1.0 - RUT_ALPHA(T)) * qvi_sat;
        *phi = RUT_ALPHA(T) * *phil + (1.0 - RUT_ALPHA(T)) * *phii;
    }
    return qvsat;
}

static void rut_saturation_adjustment(ora_state *S)
{
    const double cpRd = cp / Rd;
    double *THP = S->P[F_TH], *QVP = S->P[F_QV], *QCP = S->P[F_QC], *QIP = S->P[F_QI];
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long ix = IX(i, j, k);
                double theta = THP[ix] + S->bar[3][ix] + S->tb[k];
                double pressure = rut_pressure(S, ix, k);
                double vapor = QVP[ix] + S->bar[4][ix] + S->qb[k];
                double T = theta * pressure;
                double pd = p0 * pow(pressure, cpRd);
                double phi, phil, phii;
                double qvsat = rut_qvsat(T, pd, &phi, &phil, &phii);
                double Cl = 0, Ci = 0;
                if (vapor > qvsat) {
                    if (T > rut_tmax) Cl = (vapor - qvsat) / (1.0 + phi);
                    else if (T < rut_tmin) Ci = (vapor - qvsat) / (1.0 + phi);
                    else {
                        Cl = RUT_ALPHA(T) * (vapor - qvsat) / (1.0 + phi);
                        Ci = (1.0 - RUT_ALPHA(T)) * (vapor - qvsat) / (1.0 + phi);
                    }
                    if (S->sat) S->sat[ix] = 1;
                } else if (vapor < qvsat && (QCP[ix] + QIP[ix]) > 0) {
                    if (T > rut_tmax) Cl = -fmin(QCP[ix], (qvsat - vapor) / (1.0 + phi));
                    else if (T < rut_tmin) Ci = -fmin(QIP[ix], (qvsat - vapor) / (1.0 + phi));
                    else {
                        Cl = -fmin(QCP[ix], (qvsat - vapor) / (1.0 + phil));
                        if (Cl + QCP[ix] <= 0) Ci = -fmin(QIP[ix], (qvsat - vapor + Cl) / (1.0 + phii));
                    }
                    if (S->sat) S->sat[ix] = -(Ci + Cl) < QCP[ix] + QIP[ix];
                } else if (S->sat) {
                    S->sat[ix] = vapor == qvsat;
                }
                QIP[ix] += Ci;
                QCP[ix] += Cl;
                QVP[ix] -= (Ci + Cl);
                double diabatic = (Lv / (cp * S->pib[k])) * Cl + (Ls / (cp * S->pib[k])) * Ci;
                THP[ix] += diabatic;
            }
}

static void op_rutledge(ora_state *S)
{
    const int NX = S->NX, NY = S->NY;
    rutledge_points(S);
    rut_saturation_adjustment(S);
    op_zero_moisture(S);
    if (S->c.rain_fallout == 2) {
        rut_snow_fall(S, S->sts, S->P[F_QS], 1, NX - 1, 1, NY - 1);
        rut_ice_fall(S, S->its, S->P[F_QI], 1, NX - 1, 1, NY - 1);
        rut_rain_fall(S, S->vt, S->P[F_QR], 1, NX - 1, 1, NY - 1);
        fallout(S, S->P[F_QR], S->vt, S->accrain);
        fallout(S, S->P[F_QI], S->its, S->accsnow);
        fallout(S, S->P[F_QS], S->sts, S->accsnow);
        memset(S->vt, 0, sizeof(double) * S->N);
        memset(S->sts, 0, sizeof(double) * S->N);
        memset(S->its, 0, sizeof(double) * S->N);
    } else {
        /* precip_rate (microphysics.cpp:143-160) of rain, of rain at the snow
         * fall speed, and of ice at the snow fall speed (rutledge.cpp:486-489) */
        for (int i = 1; i < NX - 1; i++)
            for (int j = 1; j < NY - 1; j++) {
                const double r = S->rhow[1];
                const double *qr = S->P[F_QR], *qi = S->P[F_QI];
                S->accrain[IX2(i, j)] += r * 0.5 * (S->vt[IX(i, j, 0)] + S->vt[IX(i, j, 1)]) * 0.5 *
                                         (qr[IX(i, j, 0)] + qr[IX(i, j, 1)]) * S->dt;
                S->accsnow[IX2(i, j)] += r * 0.5 * (S->sts[IX(i, j, 0)] + S->sts[IX(i, j, 1)]) * 0.5 *
                                         (qr[IX(i, j, 0)] + qr[IX(i, j, 1)]) * S->dt;
                S->accsnow[IX2(i, j)] += r * 0.5 * (S->sts[IX(i, j, 0)] + S->sts[IX(i, j, 1)]) * 0.5 *
                                         (qi[IX(i, j, 0)] + qi[IX(i, j, 1)]) * S->dt;
            }
    }
}

/* run_microphysics (microphysics.cpp:97-131) over (1,NX-1,1,NY-1) */
static void op_microphysics(ora_state *S)
{
    if (S->ice) op_rutledge(S);
    else op_kessler(S);
}

/* ------------------------------------------------------------------------
 * Buffer rotation: solver.cpp:229-263, microphysics.cpp:642-669.
 * ---------------------------------------------------------------------- */
static void swap_f(ora_state *S, int f)
{
    double *t = S->cur[f];
    S->cur[f] = S->P[f];
    S->P[f] = t;
}
static void advance_inner(ora_state *S) /* solver.cpp:240-248: w stays put when hydrostatic */
{
    for (int f = 0; f < 4; f++)
        if (f != F_W || !S->c.hydrostatic) swap_f(S, f);
}
static void micro_advance_inner(ora_state *S)
{
    const int nf = S->ice ? ORA_NF : 7;
    for (int f = 4; f < nf; f++) swap_f(S, f);
}
static void advance_outer(ora_state *S)
{
    for (int f = 0; f < 4; f++)
        if (f != F_W || !S->c.hydrostatic) memcpy(S->M[f], S->P[f], sizeof(double) * S->N);
    advance_inner(S);
}
static void micro_advance(ora_state *S)
{
    const int nf = S->ice ? ORA_NF : 7;
    for (int f = 4; f < nf; f++) memcpy(S->M[f], S->P[f], sizeof(double) * S->N);
    micro_advance_inner(S);
}

/* ------------------------------------------------------------------------
 * Hydrostatic equation set (HYDROSTATIC): integrate_hydro (solver.cpp:33-80)
 * with solve_hydrostatic_pressure (pressure.cpp:229-298), poisson_fft2d
 * (:652-715), hydrostatic_pressure (:453-537) and w_velocity_LH
 * (solver.cpp:144-163); non-periodic domains.
 * ---------------------------------------------------------------------- */
static double dzu(const ora_state *S, int k) { return S->zsw[k + 1] - S->zsw[k]; } /* DZU, model.h:205 */
static double dzw(const ora_state *S, int k) { return S->zsu[k] - S->zsu[k - 1]; } /* DZW, model.h:206 */

static void hyd_init(ora_state *S)
{
    const int NX = S->NX, NY = S->NY;
    S->div2d = (double *)calloc((size_t)NX * NY, sizeof(double));
    S->rhoavg = (double *)calloc((size_t)NX * NY, sizeof(double));
    S->bco2 = (double *)calloc((size_t)NX * NY, sizeof(double));
    S->ac2 = (double *)calloc(NY, sizeof(double));
    S->cc2 = (double *)calloc(NY, sizeof(double));
    S->p2 = (double *)calloc(NY + 1, sizeof(double));
    S->q2 = (double *)calloc(NY + 1, sizeof(double));
    S->io2d = (double *)calloc(2 * (size_t)NX * NY, sizeof(double));
    for (long c = 0; c < (long)NX * NY; c++) { /* column_average_density, flat ground */
        double r = 0, zsum = 0;
        for (int k = 1; k < S->NZ - 1; k++) {
            r = r + S->rhou[k] * S->tbv[k] * dzu(S, k);
            zsum += dzu(S, k);
        }
        S->rhoavg[c] = r / zsum;
    }
    const double dx = S->dx, dy = S->dy;
    for (int j = 0; j < NY; j++) S->ac2[j] = S->cc2[j] = 1. / (dy * dy);
    S->ac2[0] = 0;
    S->cc2[NY - 1] = 0;
    for (int i = 0; i < NX; i++) {
        const double kw = i < NX / 2 ? 2 * trigpi * (double)i / NX : 2 * trigpi * (double)(NX - i) / NX;
        for (int j = 0; j < NY; j++) {
            S->bco2[(long)i * NY + j] = 2. * (cos(kw) - 1.) / (dx * dx) - S->cc2[j] - S->ac2[j];
            if (j == 0) S->bco2[(long)i * NY + j] = -S->rhow[2] / (dx * dx);
        }
    }
}

/* poisson_fft2d on div2d: FFT along i, scaled by 1/ni, a tridiagonal solve
 * along j per wavenumber (its last row keeps the transformed value: the back
 * substitution starts at nj-2), inverse FFT, real part */
static void hyd_poisson2d(ora_state *S)
{
    const int ni = S->NX, nj = S->NY;
    double *io = S->io2d;
    for (long c = 0; c < (long)ni * nj; c++) {
        io[2 * c] = S->div2d[c];
        io[2 * c + 1] = 0;
    }
    for (int j = 0; j < nj; j++) ora_fft_1d(&S->fi, -1, io + 2 * j, nj, io + 2 * j, nj);
    for (long c = 0; c < (long)ni * nj; c++) {
        io[2 * c] = io[2 * c] / ni;
        io[2 * c + 1] = io[2 * c + 1] / ni;
    }
    double *P = S->p2, *Q = S->q2;
    for (int i = 0; i < ni; i++)
        for (int part = 0; part < 2; part++) {
            double *o = io + 2 * (long)i * nj + part;
            for (int j = 0; j < nj; j++) {
                const double denom = S->bco2[(long)i * nj + j] + S->ac2[j] * P[j];
                P[j + 1] = -S->cc2[j] / denom;
                Q[j + 1] = (o[2 * j] - S->ac2[j] * Q[j]) / denom;
            }
            for (int j = nj - 2; j >= 0; j--) o[2 * j] = P[j + 1] * o[2 * (j + 1)] + Q[j + 1];
        }
    for (int j = 0; j < nj; j++) ora_fft_1d(&S->fi, +1, io + 2 * j, nj, io + 2 * j, nj);
    for (long c = 0; c < (long)ni * nj; c++) S->div2d[c] = io[2 * c];
}

/* the moisture factor of hydrostatic_pressure (pressure.cpp:457-490): 1 dry;
 * 1 + 0.61 qv - qc - qr with Kessler; less snow and ice with the ice scheme */
static double hyd_moist(const ora_state *S, long a)
{
    if (!S->c.microphysics_option) return 1;
    double m = 1. + 0.61 * S->cur[F_QV][a] - S->cur[F_QC][a] - S->cur[F_QR][a];
    if (S->ice) m = m - S->cur[F_QS][a] - S->cur[F_QI][a];
    return m;
}

static void op_solve_hydrostatic(ora_state *S, double step)
{
    const int NX = S->NX, NY = S->NY, NZ = S->NZ;
    const double *UP = S->P[F_U], *VP = S->P[F_V], *TH = S->cur[F_TH];
    double *PI = S->pi, *D = S->div2d;
    mirror(S, S->P[F_U]);
    mirror(S, S->P[F_V]);
    for (int i = 1; i < NX - 1; i++) /* density-weighted column divergence */
        for (int j = 1; j < NY - 1; j++) {
            const long c = IX2(i, j);
            double zsum = 0;
            D[c] = 0;
            for (int k = 1; k < NZ - 1; k++) {
                D[c] += S->rhou[k] * dzu(S, k) *
                        ((UP[IX(i + 1, j, k)] - UP[IX(i, j, k)]) * S->one_d_dx +
                         (VP[IX(i, j + 1, k)] - VP[IX(i, j, k)]) * S->one_d_dy);
                zsum += dzu(S, k);
            }
            D[c] /= (cp * zsum * step * S->dt);
        }
    for (int j = 0; j < NY; j++) { /* mirror_boundaries_2d (boundaries.cpp:331-345) */
        D[IX2(0, j)] = D[IX2(1, j)];
        D[IX2(NX - 1, j)] = D[IX2(NX - 2, j)];
    }
    for (int i = 0; i < NX; i++) {
        D[IX2(i, 0)] = D[IX2(i, 1)];
        D[IX2(i, NY - 1)] = D[IX2(i, NY - 2)];
    }
    hyd_poisson2d(S);
    const double *tbv = S->tbv;
    for (int i = 1; i < NX - 1; i++) /* hydrostatic_pressure(1,NX-1,1,NY-1) */
        for (int j = 1; j < NY - 1; j++) {
            long a = IX(i, j, NZ - 2);
            PI[IX(i, j, NZ - 1)] = 0;
            const double m0 = hyd_moist(S, a);
            PI[a] = -0.5 * (grav / cp) * ((TH[a] * m0) / (tbv[NZ - 2] * tbv[NZ - 2])) * dzw(S, NZ - 1);
            for (int k = NZ - 3; k > 0; k--) {
                const long u = IX(i, j, k + 1), d = IX(i, j, k);
                const double mu_ = hyd_moist(S, u);
                const double md = hyd_moist(S, d);
                const double tup = (TH[u] * mu_) / (tbv[k + 1] * tbv[k + 1]);
                const double tdn = (TH[d] * md) / (tbv[k] * tbv[k]);
                PI[d] = PI[u] - 0.5 * (grav / cp) * (tup + tdn) * dzw(S, k + 1);
            }
            double zsum = 0;
            PI[IX(i, j, 0)] = 0;
            for (int k = 1; k < NZ - 1; k++) {
                PI[IX(i, j, 0)] += S->rhou[k] * tbv[k] * PI[IX(i, j, k)] * dzu(S, k);
                zsum += dzu(S, k);
            }
            PI[IX(i, j, 0)] /= zsum;
        }
    for (int i = 1; i < NX - 1; i++) /* lid pressure */
        for (int j = 1; j < NY - 1; j++)
            PI[IX(i, j, NZ - 1)] = (D[IX2(i, j)] - PI[IX(i, j, 0)]) / S->rhoavg[IX2(i, j)];
    for (int i = 0; i < NX; i++)
        for (int j = 0; j < NY; j++)
            for (int k = 1; k < NZ - 1; k++) PI[IX(i, j, k)] += PI[IX(i, j, NZ - 1)];
    mirror(S, PI);
}

/* w_velocity_LH (solver.cpp:144-163): w of the current slot from the
 * anelastic continuity equation and the forecast u, v */
static void hyd_w(ora_state *S)
{
    double *W = S->cur[F_W];
    const double *UP = S->P[F_U], *VP = S->P[F_V];
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++) {
            W[IX(i, j, 0)] = 0;
            W[IX(i, j, 1)] = 0;
            W[IX(i, j, S->NZ - 1)] = 0;
            for (int k = 2; k < S->NZ - 1; k++)
                W[IX(i, j, k)] = (S->rhow[k - 1] / S->rhow[k]) * W[IX(i, j, k - 1)] +
                                 (S->rhou[k - 1] / S->rhow[k]) *
                                     (-(UP[IX(i + 1, j, k - 1)] - UP[IX(i, j, k - 1)]) * S->one_d_dx -
                                      (VP[IX(i, j + 1, k - 1)] - VP[IX(i, j, k - 1)]) * S->one_d_dy) *
                                     S->dz / S->mu[k - 1];
        }
}

static void integrate_hydro(ora_state *S, double step) /* solver.cpp:33-80 */
{
    op_advect_uvw(S, step); /* u and v only */
    op_solve_hydrostatic(S, step);
    for (int i = 1; i < S->NX - 1; i++)
        for (int j = 1; j < S->NY - 1; j++)
            for (int k = 1; k < S->NZ - 1; k++) {
                const long c = IX(i, j, k);
                S->P[F_U][c] -= step * (S->dtx * cp * S->tbv[k] * (S->pi[c] - S->pi[IX(i - 1, j, k)]));
                S->P[F_V][c] -= step * (S->dty * cp * S->tbv[k] * (S->pi[c] - S->pi[IX(i, j - 1, k)]));
            }
}

static void integrate_non_hydro(ora_state *S, double step) /* solver.cpp:87-138 */
{
    op_advect_uvw(S, step);
    if (S->c.turbulence_option) turb_apply_velocity(S, step); /* solver.cpp:103 */
    op_solve_pressure(S, step);
    op_project(S, step);
}

static void rk3_step(ora_state *S) /* driver_serial.cpp:178-286 */
{
    static const double steps[3] = {1. / 3., 0.5, 1.0};
    const int micro = S->c.microphysics_option != 0;
    const int turb = S->c.turbulence_option != 0;
    if (S->c.use_explicit_diffusion) op_explicit_diffusion(S, 1.0);
    if (turb) op_turbulence(S);
    for (int s = 0; s < 3; s++) {
        if (S->c.hydrostatic) integrate_hydro(S, steps[s]);
        else integrate_non_hydro(S, steps[s]);
        op_advect_theta(S, steps[s]);
        if (turb) turb_apply_theta(S, steps[s]);
        if (micro) {
            op_advect_micro(S, steps[s]);
            if (S->ice) op_advect_ice(S, steps[s]); /* driver_serial.cpp:229 */
            if (turb) turb_apply_moisture(S, steps[s]);
            op_zero_moisture(S);
        }
        if (S->c.hydrostatic) hyd_w(S); /* driver_serial.cpp:239 */
        op_bc(S);
        if (micro) {
            op_bc_micro(S);
            if (s < 2) micro_advance_inner(S);
        }
        if (s < 2) advance_inner(S);
    }
    if (micro) {
        op_microphysics(S);
        op_bc_micro(S);
        micro_advance(S);
    }
    op_bc(S);
    op_rayleigh(S);
    advance_outer(S);
    S->mtime += S->dt; /* s_run_model :366-369 */
    S->bigcounter++;
}

/* the linearised model's rescaling every 12 hours (driver_serial.cpp:160-
 * 166): find_max2 (util.cpp:818-829) of the forecast slot of v weighted by
 * rho, then rescale_pert2 (util.cpp:920-943) of the current and start-of-
 * step u, v, w and theta (its vapour lines sit under a preprocessor test of a
 * run-time variable and are compiled out) */
static void linear_rescale(ora_state *S)
{
    const double *VP = S->P[F_V];
    double mymax = 0;
    for (int i = 0; i < S->NX; i++)
        for (int j = 0; j < S->NY; j++)
            for (int k = 0; k < S->NZ; k++)
                if (VP[IX(i, j, k)] * S->rhou[k] > fabs(mymax)) mymax = fabs(VP[IX(i, j, k)] * S->rhou[k]);
    const double scale = 5.0;
    for (long x = 0; x < S->N; x++)
        for (int f = F_U; f <= F_TH; f++) {
            S->cur[f][x] = scale * S->cur[f][x] / mymax;
            S->M[f][x] = scale * S->M[f][x] / mymax;
        }
}

static void linear_rk3_step(ora_state *S) /* linear_integrate_rk3, driver_serial.cpp:83-171 */
{
    static const double steps[3] = {1. / 3., 0.5, 1.0};
    const int micro = S->c.microphysics_option != 0;
    /* unlike s_integrate_rk3 (driver_serial.cpp:202) this driver never calls
     * compute_sign_cells (fluxes.cpp:316-341), and interpolate_scalar
     * (fluxes.cpp:797-942) takes the theta and vapour faces' upwind signs from
     * those arrays, which initialize_sign_cells (:273-277) left as allocated:
     * zero, so those faces are the centred ones */
    S->stale_signs = 1;
    for (int s = 0; s < 3; s++) {
        integrate_non_hydro(S, steps[s]);
        op_advect_theta(S, steps[s]);
        if (S->c.use_explicit_diffusion) op_explicit_diffusion(S, steps[s]);
        op_bc(S);
        if (s < 2) advance_inner(S);
        if (micro) { /* after the winds' swap: stages 1 and 2 advect with the new winds */
            op_advect_qv(S, steps[s]);
            op_bc_micro(S);
            if (s < 2) micro_advance_inner(S);
        }
    }
    op_bc(S);
    op_rayleigh(S);
    advance_outer(S);
    if (micro) {
        op_bc_micro(S);
        micro_advance(S);
    }
    S->stale_signs = 0;
    const long period = 12 * 60 * 60 / (int)S->dt;
    if (period > 0 && S->bigcounter % period == 0 && S->bigcounter != 0) linear_rescale(S);
    S->mtime += S->dt;
    S->bigcounter++;
}

/* ------------------------------------------------------------------------
 * Column builders: setup_vertical_height_levels (initializer.cpp:840-849),
 * stretched_grid (:1340-1385), initialize_vertical_basic_state2 (:858-928),
 * setup_coordinates (:1948-1967), initialize_coriolis_parameter (:826-833).
 * ---------------------------------------------------------------------- */
int ora_columns_build(int NZ, double dz, double z0, const double *tb_in, const double *qb_in,
                      ga_column_store *o)
{
    if (NZ < 6 || NZ > 512) return GA_ERR_ARG;
    memset(o, 0, sizeof(*o));
    for (int k = 0; k < NZ; k++) {
        o->zu[k] = ((double)k - 0.5) * dz;
        o->zw[k] = ((double)k - 1) * dz;
    }
    const int lev = 1, nt = NZ - 1;
    const double dzp = dz;
    double c2 = (1 - z0 / (dzp * lev)) / ((nt - 1) * dzp - dzp * lev);
    double c1 = z0 / (dzp * lev) - c2 * dzp * lev;
    for (int i = 0; i <= nt; i++) {
        double fullLev = ((double)i - 1.0) * dzp;
        double halfLev = ((double)i - 0.5) * dzp;
        o->zsw[i] = (c1 + c2 * fullLev) * fullLev;
        o->mw[i] = 1 / (c1 + 2 * c2 * fullLev);
        o->zsu[i] = (c1 + c2 * halfLev) * halfLev;
        o->mu[i] = 1 / (c1 + 2 * c2 * halfLev);
    }
    double *tb = o->tb, *qb = o->qb, *tbw = o->tbw, *tbv = o->tbv, *pib = o->pib;
    double *rhou = o->rhou, *rhow = o->rhow, *zsu = o->zsu;
    for (int k = 0; k < NZ; k++) { tb[k] = tb_in[k]; qb[k] = qb_in[k]; }
    tb[0] = tb[1];
    tb[NZ - 1] = tb[NZ - 2];
    qb[0] = qb[1];
    qb[NZ - 1] = qb[NZ - 2];
    tbw[0] = 0.5 * (tb[0] + tb[1]);
    for (int k = 1; k < NZ; k++) tbw[k] = 0.5 * (tb[k] + tb[k - 1]);
    for (int k = 0; k < NZ; k++) tbv[k] = tb[k] * (1.0 + 0.61 * qb[k]);
    double pisfc = pow((pressfc / p0), (Rd / cp));
    pib[1] = pisfc - grav * (zsu[1] - 0) / (cp * tbv[1]);
    pib[0] = pisfc + grav * (0 - zsu[0]) / (cp * tbv[0]);
    for (int k = 2; k < NZ; k++) pib[k] = pib[k - 1] - grav * (zsu[k] - zsu[k - 1]) / (cp * (0.5 * (tbv[k] + tbv[k - 1])));
    for (int k = 0; k < NZ; k++) rhou[k] = p0 * pow(pib[k], (cv / Rd)) / (Rd * tbv[k]);
    rhow[1] = pressfc / (Rd * tbw[1]);
    for (int k = 1; k < NZ; k++) rhow[k] = 0.5 * (rhou[k] + rhou[k - 1]);
    tbv[0] = tbv[1];
    tbv[NZ - 1] = tbv[NZ - 2];
    tbw[0] = tbw[1];
    tbw[NZ - 1] = tbw[NZ - 2];
    pib[0] = pib[1];
    pib[NZ - 1] = pib[NZ - 2];
    rhow[0] = rhow[1];
    for (int k = 0; k < NZ; k++) {
        o->one_d_rhow[k] = 1. / rhow[k];
        o->one_d_rhou[k] = 1. / rhou[k];
    }
    return GA_OK;
}

int ora_coriolis_build(int NY, double dy, double corner_lat, double *f)
{
    double lat = -89.462997 + corner_lat + dy / meters_per_degree;
    for (int j = 0; j < NY; j++) {
        if (j > 0) lat = lat + dy / meters_per_degree;
        f[j] = 2 * fc * sin(lat * trigpi / 180.);
    }
    return GA_OK;
}

/* ------------------------------------------------------------------------
 * State management
 * ---------------------------------------------------------------------- */
static double cos_profile(double pl, double ph, double frac, double shift) /* util.cpp:740-749 */
{
    if (frac >= 0 && frac <= 1.0) return cos(pl * 2 * trigpi + (ph - pl) * 2 * trigpi * frac) + shift;
    return 0;
}

static double *dup_col(const double *src, int n)
{
    double *d = (double *)calloc((size_t)n, sizeof(double));
    if (src) memcpy(d, src, sizeof(double) * n);
    return d;
}

ora_state *ora_create(const ga_config *cfg, const ga_columns *cols)
{
    if (!cfg || !cols) return NULL;
    if (cfg->nx < 12 || cfg->ny < 12 || cfg->nz < 6 || cfg->nz > 512) return NULL;
    ora_state *S = (ora_state *)calloc(1, sizeof(ora_state));
    S->c = *cfg;
    const int NX = cfg->nx, NY = cfg->ny, NZ = cfg->nz;
    S->NX = NX; S->NY = NY; S->NZ = NZ;
    S->N = (long)NX * NY * NZ;
    S->dx = cfg->dx; S->dy = cfg->dy; S->dz = cfg->dz; S->dt = cfg->dt;
    S->dtx = S->dt / S->dx; S->dty = S->dt / S->dy; S->dtz = S->dt / S->dz;
    S->one_d_dx = 1.0 / S->dx; S->one_d_dy = 1.0 / S->dy; S->one_d_dz = 1.0 / S->dz;
    S->zu = dup_col(cols->zu, NZ); S->zw = dup_col(cols->zw, NZ);
    S->zsu = dup_col(cols->zsu, NZ); S->zsw = dup_col(cols->zsw, NZ);
    S->mu = dup_col(cols->mu, NZ); S->mw = dup_col(cols->mw, NZ);
    S->rhou = dup_col(cols->rhou, NZ); S->rhow = dup_col(cols->rhow, NZ);
    S->one_d_rhou = dup_col(cols->one_d_rhou, NZ); S->one_d_rhow = dup_col(cols->one_d_rhow, NZ);
    S->tb = dup_col(cols->tb, NZ); S->tbv = dup_col(cols->tbv, NZ); S->tbw = dup_col(cols->tbw, NZ);
    S->qb = dup_col(cols->qb, NZ); S->pib = dup_col(cols->pib, NZ);
    S->f = dup_col(cols->f, NY);
    for (int f = 0; f < ORA_NF; f++) {
        for (int s = 0; s < 3; s++) S->buf[f][s] = (double *)calloc((size_t)S->N, sizeof(double));
        S->cur[f] = S->buf[f][0];
        S->P[f] = S->buf[f][1];
        S->M[f] = S->buf[f][2];
    }
    S->pi = (double *)calloc((size_t)S->N, sizeof(double));
    for (int b = 0; b < 6; b++) S->bar[b] = (double *)calloc((size_t)S->N, sizeof(double));
    S->vt = (double *)calloc((size_t)S->N, sizeof(double));
    S->accrain = (double *)calloc((size_t)NX * NY, sizeof(double));
    S->ice = cfg->microphysics_option == 2;
    S->sts = (double *)calloc((size_t)S->N, sizeof(double));
    S->its = (double *)calloc((size_t)S->N, sizeof(double));
    S->accsnow = (double *)calloc((size_t)NX * NY, sizeof(double));
    S->n0s = 8e6; /* rutledge.cpp:90 */
    /* pressure solver set-up: initialize_pressure_solver (pressure.cpp:99-134) */
    S->ni = cfg->periodic_ew_boundaries ? NX - 6 : NX;
    S->nj = NY;
    S->nk = NZ;
    const int ni = S->ni, nj = S->nj, nk = S->nk;
    ora_fft_plan_init(&S->fi, ni);
    ora_fft_plan_init(&S->fj, nj);
    S->spec = (double *)calloc(2 * (size_t)ni * nj * nk, sizeof(double));
    S->specw = (double *)calloc(2 * (size_t)ni * nj, sizeof(double));
    S->hcoef = (double *)calloc((size_t)ni * nj, sizeof(double));
    double *kw = (double *)calloc(ni, sizeof(double)), *lw = (double *)calloc(nj, sizeof(double));
    for (int i = 0; i < ni; i++) kw[i] = (double)i * 2 * trigpi / ((double)ni);
    for (int j = 0; j < nj; j++) lw[j] = (double)j * 2 * trigpi / ((double)nj);
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < nj; j++) S->hcoef[(long)i * nj + j] = cos(kw[i]) + cos(lw[j]) - 2.0;
    free(kw);
    free(lw);
    S->acoef = (double *)calloc(nk, sizeof(double));
    S->ccoef = (double *)calloc(nk, sizeof(double));
    S->vcoef = (double *)calloc(nk, sizeof(double));
    const double dz2 = S->dz * S->dz;
    for (int k = 1; k < nk - 1; k++) {
        S->acoef[k] = S->mu[k] * S->mw[k] * S->rhow[k] / dz2;
        S->ccoef[k] = S->mu[k] * S->mw[k + 1] * S->rhow[k + 1] / dz2;
    }
    S->acoef[1] = 0;
    S->ccoef[nk - 2] = 0;
    S->vcoef[1] = S->mu[1] * S->mw[2] * S->rhow[2] / dz2;
    for (int k = 2; k < nk - 2; k++)
        S->vcoef[k] = S->mu[k] * (S->mw[k + 1] * S->rhow[k + 1] + S->mw[k] * S->rhow[k]) / dz2;
    S->vcoef[nk - 2] = (S->mu[nk - 2] * S->mw[nk - 2] * S->rhow[nk - 2]) / dz2;
    /* init_boundaries(iebuffer,iwbuffer,jnbuffer,jsbuffer,-1) (boundaries.cpp:44-114) */
    int ie = cfg->boundary_width_east, iw = cfg->boundary_width_west;
    int jn = cfg->boundary_width_north, js = cfg->boundary_width_south;
    S->east_coeff = (double *)calloc(ie + 1, sizeof(double));
    S->west_coeff = (double *)calloc(iw + 1, sizeof(double));
    S->north_coeff = (double *)calloc(jn + 1, sizeof(double));
    S->south_coeff = (double *)calloc(js + 1, sizeof(double));
    S->eb = NX - ie; S->ee = NX; S->wb = 0; S->we = iw;
    S->nb = NY - jn; S->ne = NY; S->sb = 0; S->se = js;
    for (int i = 0; i < ie; i++) S->east_coeff[i] = 0.5 * cos_profile(-0.5, 0, (double)(i + 1) / (double)ie, 1);
    for (int i = 0; i < iw; i++) S->west_coeff[i] = 0.5 * cos_profile(0, 0.5, (double)i / (double)iw, 1);
    for (int i = 0; i < jn; i++) S->north_coeff[i] = 0.5 * cos_profile(-0.5, 0, (double)(i + 1) / (double)jn, 1);
    for (int i = 0; i < js; i++) S->south_coeff[i] = 0.5 * cos_profile(0, 0.5, (double)i / (double)js, 1);
    /* Rayleigh coefficients (damping.cpp:1150-1162) */
    S->raylevel = cfg->rayleigh_damping_z;
    S->ray_u = (double *)calloc(NZ, sizeof(double));
    S->ray_w = (double *)calloc(NZ, sizeof(double));
    if (S->raylevel >= 0 && S->raylevel < NZ) {
        double raydmpcoef = 0.05, raydmpz = S->zu[S->raylevel];
        for (int k = S->raylevel; k < NZ; k++) {
            S->ray_u[k] = raydmpcoef * 0.5 * (1.0 - cos(trigpi * (S->zu[k] - raydmpz) / (S->zu[NZ - 1] - raydmpz)));
            S->ray_w[k] = raydmpcoef * 0.5 * (1.0 - cos(trigpi * (S->zw[k] - raydmpz) / (S->zw[NZ - 1] - raydmpz)));
        }
    }
    S->qp_edges = (double *)calloc(NZ, sizeof(double));
    S->qn_edges = (double *)calloc(NZ, sizeof(double));
    S->mono = (double *)calloc(NZ, sizeof(double));
    S->za = (double *)calloc(NZ, sizeof(double));
    S->qa = (double *)calloc(NZ, sizeof(double));
    S->qd = (double *)calloc(NZ, sizeof(double));
    S->ve = (double *)calloc(NZ, sizeof(double));
    if (cfg->turbulence_option) turb_init(S);
    if (cfg->hydrostatic) hyd_init(S);
    return S;
}

void ora_destroy(ora_state *S)
{
    if (!S) return;
    double *cols[] = {S->zu, S->zw, S->zsu, S->zsw, S->mu, S->mw, S->rhou, S->rhow, S->one_d_rhou,
                      S->one_d_rhow, S->tb, S->tbv, S->tbw, S->qb, S->pib, S->f};
    for (unsigned n = 0; n < sizeof(cols) / sizeof(cols[0]); n++) free(cols[n]);
    for (int f = 0; f < ORA_NF; f++)
        for (int s = 0; s < 3; s++) free(S->buf[f][s]);
    free(S->sts); free(S->its); free(S->accsnow);
    free(S->pi);
    for (int b = 0; b < 6; b++) free(S->bar[b]);
    free(S->vt); free(S->accrain);
    ora_fft_plan_free(&S->fi); ora_fft_plan_free(&S->fj);
    free(S->spec); free(S->specw); free(S->hcoef);
    free(S->acoef); free(S->ccoef); free(S->vcoef);
    free(S->east_coeff); free(S->west_coeff); free(S->north_coeff); free(S->south_coeff);
    free(S->ray_u); free(S->ray_w);
    free(S->qp_edges); free(S->qn_edges); free(S->mono);
    free(S->za); free(S->qa); free(S->qd); free(S->ve);
    free(S->kmix); free(S->khmix);
    for (int t = 0; t < 7; t++) free(S->ttend[t]);
    free(S->sat); free(S->l2); free(S->kvmax);
    free(S->div2d); free(S->rhoavg); free(S->bco2); free(S->ac2); free(S->cc2); free(S->p2); free(S->q2);
    free(S->io2d);
    free(S);
}

static double *field_ptr(ora_state *S, int field, int slot, long *n)
{
    *n = S->N;
    if (field >= 0 && field < GA_NPROG) {
        if (slot == GA_SLOT_CUR) return S->cur[field];
        if (slot == GA_SLOT_P) return S->P[field];
        if (slot == GA_SLOT_M) return S->M[field];
        return NULL;
    }
    switch (field) {
    case GA_PI: return S->pi;
    case GA_UBAR: case GA_VBAR: case GA_WBAR: case GA_THBAR: case GA_QBAR: case GA_PBAR:
        return S->bar[field - GA_UBAR];
    case GA_VT: return S->vt;
    case GA_ACCRAIN: *n = (long)S->NX * S->NY; return S->accrain;
    case GA_KMIX: return S->kmix;
    case GA_KHMIX: return S->khmix;
    case GA_UFRIC: case GA_VFRIC: case GA_WFRIC: case GA_THDIFF: case GA_QVDIFF: case GA_QCDIFF: case GA_QRDIFF:
        return S->ttend[field - GA_UFRIC];
    }
    if (!S->ice) return NULL;
    switch (field) {
    case GA_QS: case GA_QI: {
        const int f = field == GA_QS ? F_QS : F_QI;
        if (slot == GA_SLOT_CUR) return S->cur[f];
        if (slot == GA_SLOT_P) return S->P[f];
        if (slot == GA_SLOT_M) return S->M[f];
        return NULL;
    }
    case GA_VTS: return S->sts;
    case GA_VTI: return S->its;
    case GA_ACCSNOW: *n = (long)S->NX * S->NY; return S->accsnow;
    case GA_N0S: *n = 1; return &S->n0s;
    }
    return NULL;
}

int ora_set_field(ora_state *S, int field, int slot, const double *src, long n)
{
    long nn;
    if (field == GA_SATURATED) {
        if (!S->sat || n != S->N) return GA_ERR_ARG;
        for (long x = 0; x < n; x++) S->sat[x] = src[x] != 0;
        return GA_OK;
    }
    double *d = field_ptr(S, field, slot, &nn);
    if (!d || n != nn) return GA_ERR_ARG;
    memcpy(d, src, sizeof(double) * n);
    return GA_OK;
}

int ora_get_field(ora_state *S, int field, int slot, double *dst, long n)
{
    long nn;
    if (field == GA_SATURATED) {
        if (!S->sat || n != S->N) return GA_ERR_ARG;
        for (long x = 0; x < n; x++) dst[x] = S->sat[x];
        return GA_OK;
    }
    double *d = field_ptr(S, field, slot, &nn);
    if (!d || n != nn) return GA_ERR_ARG;
    memcpy(dst, d, sizeof(double) * n);
    return GA_OK;
}

int ora_op(ora_state *S, int op, double step)
{
    switch (op) {
    case GA_OP_SIGN_CELLS: return GA_OK;
    case GA_OP_ADVECT_UVW: op_advect_uvw(S, step); return GA_OK;
    case GA_OP_SOLVE_PRESSURE:
        if (S->c.hydrostatic) op_solve_hydrostatic(S, step);
        else op_solve_pressure(S, step);
        return GA_OK;
    case GA_OP_PROJECT: op_project(S, step); return GA_OK;
    case GA_OP_INTEGRATE_NON_HYDRO:
        if (S->c.hydrostatic) integrate_hydro(S, step);
        else integrate_non_hydro(S, step);
        return GA_OK;
    case GA_OP_ADVECT_THETA: op_advect_theta(S, step); return GA_OK;
    case GA_OP_ADVECT_MICRO:
        if (S->c.linear_model) op_advect_qv(S, step);
        else op_advect_micro(S, step);
        return GA_OK;
    case GA_OP_ZERO_MOISTURE: op_zero_moisture(S); return GA_OK;
    case GA_OP_BC: op_bc(S); return GA_OK;
    case GA_OP_BC_MICRO: op_bc_micro(S); return GA_OK;
    case GA_OP_KESSLER: op_microphysics(S); return S->err;
    case GA_OP_ADVECT_ICE:
        if (!S->ice) return GA_ERR_ARG;
        op_advect_ice(S, step);
        return GA_OK;
    case GA_OP_RAYLEIGH: op_rayleigh(S); return GA_OK;
    case GA_OP_ADVANCE_INNER: advance_inner(S); if (S->c.microphysics_option) micro_advance_inner(S); return GA_OK;
    case GA_OP_ADVANCE_OUTER: advance_outer(S); if (S->c.microphysics_option) micro_advance(S); return GA_OK;
    case GA_OP_EXPLICIT_DIFFUSION: op_explicit_diffusion(S, step); return GA_OK;
    case GA_OP_TURBULENCE:
        if (!S->kmix) return GA_ERR_ARG;
        op_turbulence(S);
        return GA_OK;
    }
    return GA_ERR_ARG;
}

int ora_step(ora_state *S, int nsteps)
{
    for (int n = 0; n < nsteps; n++) {
        if (S->c.linear_model) linear_rk3_step(S);
        else rk3_step(S);
        if (S->err) return S->err;
    }
    return GA_OK;
}

long long ora_bigcounter(ora_state *S) { return S->bigcounter; }
void ora_set_counters(ora_state *S, long long bigcounter, double mtime)
{
    S->bigcounter = bigcounter;
    S->mtime = mtime;
}
int ora_error(ora_state *S) { return S->err; }

/* Tangent-linear model and adjoint of the dry step (test infrastructure). */
#include "ga_oracle_lin.c"
