// ga_kernels.cuh - device code of the anelastic step, templated on the real
// type T (double: parity path, compiled without FMA contraction; float: fast
// path).  Included once per precision by ga_f64.cu / ga_f32.cu.
//
// Layout: every 3-D field is [i][j][k], k fastest, as the reference's
// INDEX(i,j,k) (include/model.h:50).  The spectral buffer of the pressure
// solver is complex [i][q][k] (transform index q along y), so that the
// vertical tridiagonal solve of one wavenumber reads one contiguous column.
//
// Arithmetic in every stencil, tendency, boundary and microphysics expression
// keeps the evaluation order of the reference expression it implements (cited
// file:line); with FP64 and no contraction the results match the reference's
// serial build except where CUDA's pow/exp and the FFT round differently.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ga {

template <typename T> struct V2;
template <> struct V2<double> { typedef double2 t; };
template <> struct V2<float> { typedef float2 t; };

// ---------------------------------------------------------------------------
// parameters passed by value to every kernel
// ---------------------------------------------------------------------------
template <typename T>
struct KParams {
    int nx, ny, nz;
    long n;
    double dt_d;             // time step in double (step constants are formed from it)
    int ni, nj, ioff;        // spectral grid and its first physical column
    int periodic, moist, rf;
    T dtx, dty, dtz, dt, one_d_dx, one_d_dy, one_d_dz;
    // vertical columns [nz] and Coriolis [ny]
    const T *mu, *mw, *rhou, *rhow, *one_d_rhou, *tb, *tbv, *qb, *f, *zsw;
    // Rayleigh coefficients [nz]
    const T *ray_u, *ray_w;
    int raylevel;
    // sponge coefficients and strips (boundaries.cpp:44-114)
    const T *ce, *cw, *cn, *cs;
    int eb, ee, wb, we, nb, ne, sb, se;
    // pressure solver tables (pressure.cpp:759-792)
    const double *hcoef;                        // (cos kx + cos ly) - 2 per (p,q)
    const T *acoef, *ccoef, *vcoef;             // [nz]
    const double *acoef_d, *ccoef_d, *vcoef_d, *rhou_d;  // FP64 islands
    double dx2;
    T rhou1;
    int low_modes;  // |p|,|q| below this solve in FP64 (FP32 contexts)
    // FP32: inverse of the mean mode's gauge-pinned system, nl x nl row-major
    // (rows and columns: levels 1 .. NZ-2), or null
    const double *mean_inv;
    // horizontally uniform basic state: per-level tables (BT_* rows of nz)
    int ubase_adv;  // UBAR, VBAR, WBAR, THBAR, QBAR depend on k only
    int ubase_kes;  // THBAR, QBAR, PBAR depend on k only
    const T *btab;
    // the linearised model (ISLINEAR): perturbation faces advected by the
    // basic-state velocity alone; stale_signs: its driver's theta and vapour
    // faces take upwind signs of zero (the sign arrays it never computes)
    int linear, stale_signs;
    // the hydrostatic equation set: pi is the Exner perturbation itself
    // (CONVERT_PRESSURE, kessler.cpp:7-11), w is diagnosed
    int hydrostatic;
    // ice microphysics (microphysics_option 2): snow and cloud ice, the
    // Rutledge fall speeds stored by their own kernel; rfall is the rain
    // fall-speed constant of rutledge.cpp:140
    int ice;
    T rfall;
    const T *pib;  // Exner function of the base state [nz] (the ice scheme's latent heating)
};

// rows of the basic-state table (each nz long), filled by k_base_tables
enum {
    BT_UB = 0, BT_VB, BT_WB, BT_THB, BT_QB, BT_PB,  // column values
    BT_C6_UB, BT_C6_VB, BT_C6_THB, BT_C6_QB,         // 5th-order face of six equal values
    BT_C4_UB, BT_U3_UB, BT_C4_VB, BT_U3_VB,          // parts of the 3rd-order top face
    BT_C4_THB, BT_U3_THB, BT_C4_QB, BT_U3_QB,
    BT_H2_UB, BT_H2_VB, BT_H2_THB, BT_H2_QB,         // 2nd-order top face
    BT_UA, BT_VA, BT_WA,                             // averaged advecting velocities
    BT_COUNT
};

template <typename T>
struct KFields {
    T *cur[9], *P[9], *M[9];  // u v w th qv qc qr, and snow, ice with the ice scheme
    const T *bar[6];
    T *pi, *vt;
    double *accrain;
    // ice scheme: snow and ice fall speeds, accumulated snow, the snow
    // intercept carried between microphysics passes (one value), each snowy
    // point's intercept of the last pass and the largest snowy point index
    T *sts, *its;
    double *accsnow;
    T *n0s, *n0s_pt;
    int *n0s_idx;
    // optional: per point of the advected cells, which moisture fields
    // zero_moisture clipped (bit 0 qv, 1 qc, 2 qr) -- the branch record of
    // the linearisation
    unsigned char *qmask;
    // optional: Kessler's saturation record for the turbulence scheme
    unsigned char *sat;
};

enum { FU = 0, FV, FW, FTH, FQV, FQC, FQR, FQS, FQI };

// grids are limited to fewer than 2^31 points (checked by the engine)
__host__ __device__ __forceinline__ int gix(int ny, int nz, int i, int j, int k)
{
    return (i * ny + j) * nz + k;
}

template <typename T>
__device__ __forceinline__ T sgn(T x) { return x > T(0) ? T(1) : T(-1); }

// interpolation weights (fluxes.cpp:247-251)
template <typename T> struct W {
    static constexpr T c1_12 = T(1.0 / 12.0);
    static constexpr T c7_12 = T(7.0 / 12.0);
    static constexpr T c37_60 = T(37.0 / 60.0);
    static constexpr T c2_15 = T(2.0 / 15.0);
    static constexpr T c1_60 = T(1.0 / 60.0);
};

// INTERP_5TH_EAST (fluxes.cpp:110-122, 155-180): stencil a(-2)..a(+3)
template <typename T>
__device__ __forceinline__ T face5(T am2, T am1, T a0, T a1, T a2, T a3, T sign)
{
    T c6 = W<T>::c37_60 * (a1 + a0) - W<T>::c2_15 * (a2 + am1) + W<T>::c1_60 * (a3 + am2);
    T u5 = -(a3 - am2) + T(5.0) * (a2 - am1) - T(10.0) * (a1 - a0);
    return c6 + W<T>::c1_60 * sign * u5;
}
// INTERP_3RD_TOP (fluxes.cpp:131-136, 185-199): stencil a(-1)..a(+2)
template <typename T>
__device__ __forceinline__ T face3(T am1, T a0, T a1, T a2, T sign)
{
    T c4 = W<T>::c7_12 * (a1 + a0) - W<T>::c1_12 * (a2 + am1);
    T u3 = (a2 - am1) - T(3.0) * (a1 - a0);
    return c4 + W<T>::c1_12 * sign * u3;
}

template <typename T>
struct Grid {
    const KParams<T> &p;
    __device__ Grid(const KParams<T> &pp) : p(pp) {}
    __device__ __forceinline__ long ix(int i, int j, int k) const { return gix(p.ny, p.nz, i, j, k); }
};

#define LD(a, idx) __ldg((a) + (idx))

// six points along i / j around the face between index 0 and +1
template <typename T>
__device__ __forceinline__ T f5i(const T *a, const KParams<T> &p, int i, int j, int k, T sign)
{
    const int s = p.ny * p.nz, c = gix(p.ny, p.nz, i, j, k);
    return face5<T>(LD(a, c - 2 * s), LD(a, c - s), LD(a, c), LD(a, c + s), LD(a, c + 2 * s),
                    LD(a, c + 3 * s), sign);
}
template <typename T>
__device__ __forceinline__ T f5j(const T *a, const KParams<T> &p, int i, int j, int k, T sign)
{
    const int s = p.nz, c = gix(p.ny, p.nz, i, j, k);
    return face5<T>(LD(a, c - 2 * s), LD(a, c - s), LD(a, c), LD(a, c + s), LD(a, c + 2 * s),
                    LD(a, c + 3 * s), sign);
}
template <typename T>
__device__ __forceinline__ T f3k(const T *a, const KParams<T> &p, int i, int j, int k, T sign)
{
    const long c = gix(p.ny, p.nz, i, j, k);
    return face3<T>(LD(a, c - 1), LD(a, c), LD(a, c + 1), LD(a, c + 2), sign);
}
template <typename T>
__device__ __forceinline__ T f2k(const T *a, const KParams<T> &p, int i, int j, int k)
{
    const long c = gix(p.ny, p.nz, i, j, k);
    return T(0.5) * (LD(a, c + 1) + LD(a, c));
}

// the velocity advecting the perturbation at a face: basic state plus
// perturbation, or the basic state alone in the linearised model (ISLINEAR,
// fluxes.cpp:328-337, 366-374, 594-650, 1204-1357), for both the upwind sign
// and the flux
template <typename T>
__device__ __forceinline__ T adv_vel(const KParams<T> &p, T basic, T pert)
{
    return p.linear ? basic : basic + pert;
}

// ---------------------------------------------------------------------------
// momentum face fluxes: interpolate_velocity (fluxes.cpp:1384-1592),
// advecting_velocity (:1109-1164), compute_fluxes (:582-627)
// ---------------------------------------------------------------------------
template <typename T>
__device__ T u_east(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *U = F.cur[FU], *UB = F.bar[0];
    const long c = gix(p.ny, p.nz, i, j, k), s = (long)p.ny * p.nz;
    T ua = T(0.5) * (LD(U, c + s) + LD(U, c));
    T uba = T(0.5) * (LD(UB, c + s) + LD(UB, c));
    const T at = adv_vel(p, uba, ua);
    T ue = f5i(U, p, i, j, k, sgn(at));
    T ube = f5i(UB, p, i, j, k, sgn(ua));
    return ua * ube + at * ue;
}
template <typename T>
__device__ T u_north(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *U = F.cur[FU], *UB = F.bar[0], *V = F.cur[FV], *VB = F.bar[1];
    const long a = gix(p.ny, p.nz, i, j + 1, k), b = gix(p.ny, p.nz, i - 1, j + 1, k);
    T va = T(0.5) * (LD(V, a) + LD(V, b));
    T vba = T(0.5) * (LD(VB, a) + LD(VB, b));
    const T at = adv_vel(p, vba, va);
    T un = f5j(U, p, i, j, k, sgn(at));
    T ubn = f5j(UB, p, i, j, k, sgn(va));
    return va * ubn + at * un;
}
template <typename T>
__device__ T u_top(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    if (k == 0) return T(0);
    const T *U = F.cur[FU], *UB = F.bar[0], *Wc = F.cur[FW], *WB = F.bar[2];
    const long a = gix(p.ny, p.nz, i, j, k + 1), b = gix(p.ny, p.nz, i - 1, j, k + 1);
    T wa = T(0.5) * (LD(Wc, a) + LD(Wc, b));
    T wba = T(0.5) * (LD(WB, a) + LD(WB, b));
    T ut, ubt;
    if (k == 1 || k == p.nz - 2) {
        ut = f2k(U, p, i, j, k);
        ubt = f2k(UB, p, i, j, k);
    } else {
        ut = f3k(U, p, i, j, k, sgn(adv_vel(p, wba, wa)));
        ubt = f3k(UB, p, i, j, k, sgn(wa));
    }
    return wa * ubt + adv_vel(p, wba, wa) * ut;
}
template <typename T>
__device__ T v_east(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *U = F.cur[FU], *UB = F.bar[0], *V = F.cur[FV], *VB = F.bar[1];
    const long a = gix(p.ny, p.nz, i + 1, j, k), b = gix(p.ny, p.nz, i + 1, j - 1, k);
    T ua = T(0.5) * (LD(U, a) + LD(U, b));
    T uba = T(0.5) * (LD(UB, a) + LD(UB, b));
    const T at = adv_vel(p, uba, ua);
    T ve = f5i(V, p, i, j, k, sgn(at));
    T vbe = f5i(VB, p, i, j, k, sgn(ua));
    return ua * vbe + at * ve;
}
template <typename T>
__device__ T v_north(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *V = F.cur[FV], *VB = F.bar[1];
    const long c = gix(p.ny, p.nz, i, j, k);
    T va = T(0.5) * (LD(V, c + p.nz) + LD(V, c));
    T vba = T(0.5) * (LD(VB, c + p.nz) + LD(VB, c));
    const T at = adv_vel(p, vba, va);
    T vn = f5j(V, p, i, j, k, sgn(at));
    T vbn = f5j(VB, p, i, j, k, sgn(va));
    return va * vbn + at * vn;
}
template <typename T>
__device__ T v_top(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    if (k == 0) return T(0);
    const T *V = F.cur[FV], *VB = F.bar[1], *Wc = F.cur[FW], *WB = F.bar[2];
    const long a = gix(p.ny, p.nz, i, j, k + 1), b = gix(p.ny, p.nz, i, j - 1, k + 1);
    T wa = T(0.5) * (LD(Wc, a) + LD(Wc, b));
    T wba = T(0.5) * (LD(WB, a) + LD(WB, b));
    T vt, vbt;
    if (k == 1 || k == p.nz - 2) {
        vt = f2k(V, p, i, j, k);
        vbt = f2k(VB, p, i, j, k);
    } else {
        vt = f3k(V, p, i, j, k, sgn(adv_vel(p, wba, wa)));
        vbt = f3k(VB, p, i, j, k, sgn(wa));
    }
    return wa * vbt + adv_vel(p, wba, wa) * vt;
}

// ---------------------------------------------------------------------------
// scalar face fluxes: interpolate_scalar (fluxes.cpp:797-942) and
// compute_fluxes_scalar / compute_fluxes_moisture (:632-654, :719-784).
// Signs as compute_sign_cells (:316-341), taken from the current winds.
// ---------------------------------------------------------------------------
template <typename T>
__device__ T s_east(const KParams<T> &p, const KFields<T> &F, const T *s, const T *sb, int i, int j, int k)
{
    const long a = gix(p.ny, p.nz, i + 1, j, k);
    T u1 = LD(F.cur[FU], a);
    T ut = sb ? adv_vel(p, LD(F.bar[0], a), u1) : LD(F.bar[0], a) + u1;
    // the linearised driver's stale signs, except on the face east of column
    // 2, which compute_west_scalar (fluxes.cpp:479-501) forms from the winds
    const bool z = sb && p.stale_signs && i != 2;
    T se = f5i(s, p, i, j, k, z ? T(0) : sgn(ut));
    if (!sb) return ut * se;
    T be = f5i(sb, p, i, j, k, z ? T(0) : sgn(u1));
    return u1 * be + ut * se;
}
template <typename T>
__device__ T s_north(const KParams<T> &p, const KFields<T> &F, const T *s, const T *sb, int i, int j, int k)
{
    const long a = gix(p.ny, p.nz, i, j + 1, k);
    T v1 = LD(F.cur[FV], a);
    T vt = sb ? adv_vel(p, LD(F.bar[1], a), v1) : LD(F.bar[1], a) + v1;
    const bool z = sb && p.stale_signs;
    T sn = f5j(s, p, i, j, k, z ? T(0) : sgn(vt));
    if (!sb) return vt * sn;
    T bn = f5j(sb, p, i, j, k, z ? T(0) : sgn(v1));
    return v1 * bn + vt * sn;
}
template <typename T>
__device__ T s_top(const KParams<T> &p, const KFields<T> &F, const T *s, const T *sb, int i, int j, int k)
{
    if (k == 0) return T(0);
    const long a = gix(p.ny, p.nz, i, j, k + 1);
    T w1 = LD(F.cur[FW], a);
    T wt = sb ? adv_vel(p, LD(F.bar[2], a), w1) : LD(F.bar[2], a) + w1;
    T st, bt = T(0);
    if (k == 1 || k == p.nz - 2) {
        st = f2k(s, p, i, j, k);
        if (sb) bt = f2k(sb, p, i, j, k);
    } else {
        const bool z = sb && p.stale_signs;
        st = f3k(s, p, i, j, k, z ? T(0) : sgn(wt));
        if (sb) bt = f3k(sb, p, i, j, k, z ? T(0) : sgn(w1));
    }
    if (!sb) return wt * st;
    return w1 * bt + wt * st;
}

// rain fall speed of one point: calculate_rain_fall_speed_kessler
// (kessler.cpp:222-252)
template <typename T>
__device__ __forceinline__ T fall_speed_point(const KParams<T> &p, T qr, int k)
{
    if (qr > T(1.0e-12)) {
        T qrr = fmax(qr * T(0.001) * p.rhou[k], T(0.0));
        T vtden = sqrt(p.rhou1 / p.rhou[k]);
        return T(36.34) * (pow(qrr, T(0.1364))) * vtden;
    }
    return T(0);
}

// fall speed seen by the rain flux of an advected column: recomputed from the
// current rain (Eulerian Kessler fallout, advection.cpp:456-457) or the stored
// field (semi-Lagrangian fallout; the ice scheme, whose rain fall speed reads
// the pressure solved in the same stage)
template <typename T>
__device__ __forceinline__ T vt_at(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    if (p.rf == 1 && !p.ice && k < p.nz - 1) {
        int kk = k == 0 ? 1 : k;
        return fall_speed_point(p, LD(F.cur[FQR], gix(p.ny, p.nz, i, j, kk)), kk);
    }
    return F.vt[gix(p.ny, p.nz, i, j, k)];
}

// interpolate_scalar_with_fallspeed + compute_fluxes_moisture, rain
template <typename T>
__device__ T r_top(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *s = F.cur[FQR];
    if (k == 0) {
        T s0 = T(0.5) * (LD(s, gix(p.ny, p.nz, i, j, 0)) + LD(s, gix(p.ny, p.nz, i, j, 1)));
        return T(-0.5) * (vt_at(p, F, i, j, 1) + vt_at(p, F, i, j, 0)) * s0;
    }
    const long a = gix(p.ny, p.nz, i, j, k + 1);
    T wb = LD(F.bar[2], a) + LD(F.cur[FW], a);
    T wf = wb - T(0.5) * (vt_at(p, F, i, j, k) + vt_at(p, F, i, j, k + 1));
    T st;
    if (k == 1 || k == p.nz - 2) st = f2k(s, p, i, j, k);
    else st = f3k(s, p, i, j, k, sgn(wf));
    return wf * st;
}

// tendency of a flux-form scalar: theta_tend_cell / qv_tend_cell
// (advection.cpp:152-168, :197-213), Z_ADVECT_BASE (:16-18)
template <typename T>
__device__ T s_tend(const KParams<T> &p, const KFields<T> &F, const T *s, const T *sb, const T *base,
                    int i, int j, int k)
{
    const T DTZ = p.dtz * p.mu[k];
    T t = -p.dtx * (s_east(p, F, s, sb, i, j, k) - s_east(p, F, s, sb, i - 1, j, k)) -
          p.dty * (s_north(p, F, s, sb, i, j, k) - s_north(p, F, s, sb, i, j - 1, k)) -
          DTZ * (p.rhow[k + 1] * s_top(p, F, s, sb, i, j, k) - p.rhow[k] * s_top(p, F, s, sb, i, j, k - 1)) *
              p.one_d_rhou[k];
    if (base) {
        const T *Wc = F.cur[FW];
        T zab = T(0.50) *
                (p.rhow[k + 1] * LD(Wc, gix(p.ny, p.nz, i, j, k + 1)) * (base[k + 1] - base[k]) +
                 p.rhow[k] * LD(Wc, gix(p.ny, p.nz, i, j, k)) * (base[k] - base[k - 1])) *
                p.one_d_rhou[k];
        t = t - DTZ * zab;
    }
    return t;
}

// ---------------------------------------------------------------------------
// advection kernel: advect_uvw_velocity (+ buoyancy), advect_theta,
// advect_microphysics_cell, optionally zero_moisture on the written points.
// One thread per interior point [3,NX-3) x [3,NY-3) x [1,NZ-1).
// ---------------------------------------------------------------------------
// ADV_MIRROR (four-level kernel, non-periodic): the launch also makes the
// lateral mirror copies of P u, v, w that precede the pressure solve; they read
// and write only points the advection does not write.  ADV_ROWS (four-level
// kernel): east and north faces by sliding rows instead of one per work item
// ADV_QVONLY (with ADV_Q): the vapour alone (advect_qv, advection.cpp:577-601).
// ADV_ICE (four-level kernel, ice scheme): snow and cloud ice too
enum { ADV_UV = 1, ADV_WB = 2, ADV_TH = 4, ADV_Q = 8, ADV_ZERO = 16, ADV_MIRROR = 32, ADV_ROWS = 64,
       ADV_QVONLY = 128, ADV_ICE = 256 };

template <typename T>
__global__ void __launch_bounds__(128) k_advect(KParams<T> p, KFields<T> F, T step, T sdtg, int what)
{
    const int nzi = p.nz - 2, nyi = p.ny - 6, nxi = p.nx - 6;
    const long tot = (long)nxi * nyi * nzi;
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tot) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 3 + (int)((t / nzi) % nyi);
    const int i = 3 + (int)(t / ((long)nzi * nyi));
    const long c = gix(p.ny, p.nz, i, j, k);
    const T DTZ = p.dtz * p.mu[k];
    if (what & ADV_UV) {  // advection.cpp:318-322 with u_tend_cell / v_tend_cell (:73-122)
        const T *U = F.cur[FU], *V = F.cur[FV];
        const long sy = p.nz, sx = (long)p.ny * p.nz;
        T ov_u = T(0.25) * (LD(V, c) + LD(V, c + sy) + LD(V, c - sx) + LD(V, c - sx + sy));
        T ut = -p.dtx * (u_east(p, F, i, j, k) - u_east(p, F, i - 1, j, k)) -
               p.dty * (u_north(p, F, i, j, k) - u_north(p, F, i, j - 1, k)) -
               DTZ * (p.rhow[k + 1] * u_top(p, F, i, j, k) - p.rhow[k] * u_top(p, F, i, j, k - 1)) *
                   p.one_d_rhou[k] +
               p.dt * p.f[j] * ov_u;
        F.P[FU][c] = LD(F.M[FU], c) + step * ut;
        T ov_v = T(0.25) * (LD(U, c) + LD(U, c + sx) + LD(U, c - sy) + LD(U, c + sx - sy));
        T vt = -p.dtx * (v_east(p, F, i, j, k) - v_east(p, F, i - 1, j, k)) -
               p.dty * (v_north(p, F, i, j, k) - v_north(p, F, i, j - 1, k)) -
               DTZ * (p.rhow[k + 1] * v_top(p, F, i, j, k) - p.rhow[k] * v_top(p, F, i, j, k - 1)) *
                   p.one_d_rhou[k] -
               p.dt * p.f[j] * ov_v;
        F.P[FV][c] = LD(F.M[FV], c) + step * vt;
    }
    if ((what & ADV_WB) && k >= 2) {  // buoyancy overwrite, advection.cpp:329-337
        const T *TH = F.cur[FTH];
        T b0, b1;
        if (!p.moist) {
            b0 = LD(TH, c) / p.tbv[k];
            b1 = LD(TH, c - 1) / p.tbv[k - 1];
        } else {
            const T *QV = F.cur[FQV], *QC = F.cur[FQC], *QR = F.cur[FQR];
            b0 = LD(TH, c) / p.tbv[k] + T(0.61) * LD(QV, c) - LD(QC, c) - LD(QR, c);
            b1 = LD(TH, c - 1) / p.tbv[k - 1] + T(0.61) * LD(QV, c - 1) - LD(QC, c - 1) - LD(QR, c - 1);
            if (p.ice) {  // buoyancy_cold_micro (advection.cpp:56-58)
                const T *QI = F.cur[FQI], *QS = F.cur[FQS];
                b0 = b0 - LD(QI, c) - LD(QS, c);
                b1 = b1 - LD(QI, c - 1) - LD(QS, c - 1);
            }
        }
        F.P[FW][c] = LD(F.M[FW], c) + sdtg * (b0 + b1);
    }
    if (what & ADV_TH)  // advection.cpp:366-370
        F.P[FTH][c] = LD(F.M[FTH], c) + step * s_tend(p, F, F.cur[FTH], F.bar[3], p.tb, i, j, k);
    if ((what & ADV_Q) && (what & ADV_QVONLY)) {  // advect_qv, advection.cpp:577-601
        F.P[FQV][c] = LD(F.M[FQV], c) + step * s_tend(p, F, F.cur[FQV], F.bar[4], p.qb, i, j, k);
    } else if (what & ADV_Q) {  // advection.cpp:466-497
        if (p.rf == 1 && !p.ice) {
            const T *QR = F.cur[FQR];
            F.vt[c] = fall_speed_point(p, LD(QR, c), k);
            if (k == 1) F.vt[c - 1] = fall_speed_point(p, LD(QR, c), 1);
        }
        T qv = LD(F.M[FQV], c) + step * s_tend(p, F, F.cur[FQV], F.bar[4], p.qb, i, j, k);
        T qc = LD(F.M[FQC], c) + step * s_tend(p, F, F.cur[FQC], (const T *)nullptr, (const T *)nullptr, i, j, k);
        T tr = -p.dtx * (s_east(p, F, F.cur[FQR], (const T *)nullptr, i, j, k) -
                         s_east(p, F, F.cur[FQR], (const T *)nullptr, i - 1, j, k)) -
               p.dty * (s_north(p, F, F.cur[FQR], (const T *)nullptr, i, j, k) -
                        s_north(p, F, F.cur[FQR], (const T *)nullptr, i, j - 1, k)) -
               DTZ * (p.rhow[k + 1] * r_top(p, F, i, j, k) - p.rhow[k] * r_top(p, F, i, j, k - 1)) *
                   p.one_d_rhou[k];
        T qr = LD(F.M[FQR], c) + step * tr;
        if (what & ADV_ZERO) {  // zero_moisture on this point (microphysics.cpp:675-700)
            unsigned char bits = 0;
            if (qc < 0) { qc = 0; bits |= 2; }
            if (qr < 0) { qr = 0; bits |= 4; }
            T qbar = LD(F.bar[4], c);
            if (qv + qbar + p.qb[k] < 0) { qv = -(qbar + p.qb[k]); bits |= 1; }
            if (F.qmask) F.qmask[c] = bits;
        }
        F.P[FQV][c] = qv;
        F.P[FQC][c] = qc;
        F.P[FQR][c] = qr;
    }
}

// ---------------------------------------------------------------------------
// Horizontally uniform basic state.  With UBAR..QBAR functions of k only, the
// basic-state face values and averaged advecting velocities are per-level
// constants.  For six equal values the upwind part of INTERP_5TH is exactly
// zero and the face equals its centred part for either sign, so a table
// evaluated once with the same device functions reproduces the general
// expressions bit for bit.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_base_tables(KParams<T> p, const T *ub, const T *vb, const T *wb, const T *thb, const T *qb,
                              const T *pb, T *tab)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nz = p.nz;
    if (k >= nz) return;
    // column 0 holds the profile (the host checked that every column equals it)
    const T *src[6] = {ub, vb, wb, thb, qb, pb};
    for (int r = 0; r < 6; r++) tab[r * nz + k] = src[r][k];
    const T *hsrc[4] = {ub, vb, thb, qb};
    for (int r = 0; r < 4; r++) {
        const T a = hsrc[r][k];
        tab[(BT_C6_UB + r) * nz + k] = face5<T>(a, a, a, a, a, a, T(1));
        if (k >= 1 && k <= nz - 3) {
            const T am1 = hsrc[r][k - 1], a0 = a, a1 = hsrc[r][k + 1], a2 = hsrc[r][k + 2];
            tab[(BT_C4_UB + 2 * r) * nz + k] = W<T>::c7_12 * (a1 + a0) - W<T>::c1_12 * (a2 + am1);
            tab[(BT_U3_UB + 2 * r) * nz + k] = (a2 - am1) - T(3.0) * (a1 - a0);
        } else {
            tab[(BT_C4_UB + 2 * r) * nz + k] = T(0);
            tab[(BT_U3_UB + 2 * r) * nz + k] = T(0);
        }
        tab[(BT_H2_UB + r) * nz + k] = k + 1 < nz ? T(0.5) * (hsrc[r][k + 1] + a) : T(0);
    }
    tab[BT_UA * nz + k] = T(0.5) * (ub[k] + ub[k]);
    tab[BT_VA * nz + k] = T(0.5) * (vb[k] + vb[k]);
    tab[BT_WA * nz + k] = k + 1 < nz ? T(0.5) * (wb[k + 1] + wb[k + 1]) : T(0);
}

#define BTAB(row, k) p.btab[(row) * p.nz + (k)]

template <typename T>
__device__ __forceinline__ T face3_tab(const KParams<T> &p, int rc4, int k, T sign)
{
    return BTAB(rc4, k) + W<T>::c1_12 * sign * BTAB(rc4 + 1, k);
}

template <typename T>
__device__ T u_east_ub(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *U = F.cur[FU];
    const int c = gix(p.ny, p.nz, i, j, k), s = p.ny * p.nz;
    T ua = T(0.5) * (LD(U, c + s) + LD(U, c));
    T uba = BTAB(BT_UA, k);
    T ue = f5i(U, p, i, j, k, sgn(uba + ua));
    return ua * BTAB(BT_C6_UB, k) + (uba + ua) * ue;
}
template <typename T>
__device__ T u_north_ub(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *U = F.cur[FU], *V = F.cur[FV];
    const int a = gix(p.ny, p.nz, i, j + 1, k), b = gix(p.ny, p.nz, i - 1, j + 1, k);
    T va = T(0.5) * (LD(V, a) + LD(V, b));
    T vba = BTAB(BT_VA, k);
    T un = f5j(U, p, i, j, k, sgn(vba + va));
    return va * BTAB(BT_C6_UB, k) + (vba + va) * un;
}
template <typename T>
__device__ T u_top_ub(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    if (k == 0) return T(0);
    const T *U = F.cur[FU], *Wc = F.cur[FW];
    const int a = gix(p.ny, p.nz, i, j, k + 1), b = gix(p.ny, p.nz, i - 1, j, k + 1);
    T wa = T(0.5) * (LD(Wc, a) + LD(Wc, b));
    T wba = BTAB(BT_WA, k);
    T ut, ubt;
    if (k == 1 || k == p.nz - 2) {
        ut = f2k(U, p, i, j, k);
        ubt = BTAB(BT_H2_UB, k);
    } else {
        ut = f3k(U, p, i, j, k, sgn(wba + wa));
        ubt = face3_tab(p, BT_C4_UB, k, sgn(wa));
    }
    return wa * ubt + (wba + wa) * ut;
}
template <typename T>
__device__ T v_east_ub(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *U = F.cur[FU], *V = F.cur[FV];
    const int a = gix(p.ny, p.nz, i + 1, j, k), b = gix(p.ny, p.nz, i + 1, j - 1, k);
    T ua = T(0.5) * (LD(U, a) + LD(U, b));
    T uba = BTAB(BT_UA, k);
    T ve = f5i(V, p, i, j, k, sgn(uba + ua));
    return ua * BTAB(BT_C6_VB, k) + (uba + ua) * ve;
}
template <typename T>
__device__ T v_north_ub(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *V = F.cur[FV];
    const int c = gix(p.ny, p.nz, i, j, k);
    T va = T(0.5) * (LD(V, c + p.nz) + LD(V, c));
    T vba = BTAB(BT_VA, k);
    T vn = f5j(V, p, i, j, k, sgn(vba + va));
    return va * BTAB(BT_C6_VB, k) + (vba + va) * vn;
}
template <typename T>
__device__ T v_top_ub(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    if (k == 0) return T(0);
    const T *V = F.cur[FV], *Wc = F.cur[FW];
    const int a = gix(p.ny, p.nz, i, j, k + 1), b = gix(p.ny, p.nz, i, j - 1, k + 1);
    T wa = T(0.5) * (LD(Wc, a) + LD(Wc, b));
    T wba = BTAB(BT_WA, k);
    T vt, vbt;
    if (k == 1 || k == p.nz - 2) {
        vt = f2k(V, p, i, j, k);
        vbt = BTAB(BT_H2_VB, k);
    } else {
        vt = f3k(V, p, i, j, k, sgn(wba + wa));
        vbt = face3_tab(p, BT_C4_VB, k, sgn(wa));
    }
    return wa * vbt + (wba + wa) * vt;
}
// scalar faces; brow = basic-state row offset (0: theta, 1: qv) or -1 (none)
template <typename T>
__device__ T s_east_ub(const KParams<T> &p, const KFields<T> &F, const T *s, int brow, int i, int j, int k)
{
    const int a = gix(p.ny, p.nz, i + 1, j, k);
    T u1 = LD(F.cur[FU], a);
    T ut = BTAB(BT_UB, k) + u1;
    T se = f5i(s, p, i, j, k, sgn(ut));
    if (brow < 0) return ut * se;
    return u1 * BTAB(BT_C6_THB + brow, k) + ut * se;
}
template <typename T>
__device__ T s_north_ub(const KParams<T> &p, const KFields<T> &F, const T *s, int brow, int i, int j, int k)
{
    const int a = gix(p.ny, p.nz, i, j + 1, k);
    T v1 = LD(F.cur[FV], a);
    T vt = BTAB(BT_VB, k) + v1;
    T sn = f5j(s, p, i, j, k, sgn(vt));
    if (brow < 0) return vt * sn;
    return v1 * BTAB(BT_C6_THB + brow, k) + vt * sn;
}
template <typename T>
__device__ T s_top_ub(const KParams<T> &p, const KFields<T> &F, const T *s, int brow, int i, int j, int k)
{
    if (k == 0) return T(0);
    const int a = gix(p.ny, p.nz, i, j, k + 1);
    T w1 = LD(F.cur[FW], a);
    T wt = BTAB(BT_WB, k + 1) + w1;
    T st, bt = T(0);
    if (k == 1 || k == p.nz - 2) {
        st = f2k(s, p, i, j, k);
        if (brow >= 0) bt = BTAB(BT_H2_THB + brow, k);
    } else {
        st = f3k(s, p, i, j, k, sgn(wt));
        if (brow >= 0) bt = face3_tab(p, BT_C4_THB + 2 * brow, k, sgn(w1));
    }
    if (brow < 0) return wt * st;
    return w1 * bt + wt * st;
}
template <typename T>
__device__ T r_top_ub(const KParams<T> &p, const KFields<T> &F, int i, int j, int k)
{
    const T *s = F.cur[FQR];
    if (k == 0) {
        T s0 = T(0.5) * (LD(s, gix(p.ny, p.nz, i, j, 0)) + LD(s, gix(p.ny, p.nz, i, j, 1)));
        return T(-0.5) * (vt_at(p, F, i, j, 1) + vt_at(p, F, i, j, 0)) * s0;
    }
    const int a = gix(p.ny, p.nz, i, j, k + 1);
    T wb = BTAB(BT_WB, k + 1) + LD(F.cur[FW], a);
    T wf = wb - T(0.5) * (vt_at(p, F, i, j, k) + vt_at(p, F, i, j, k + 1));
    T st;
    if (k == 1 || k == p.nz - 2) st = f2k(s, p, i, j, k);
    else st = f3k(s, p, i, j, k, sgn(wf));
    return wf * st;
}

// ---------------------------------------------------------------------------
// Tiled advection: a block owns a TI x TJ tile of interior columns and every
// interior level.  Phase 1 evaluates each east, north and top face flux of the
// tile once (plus the west / south faces of its first row and column) into
// shared memory; phase 2 forms every tendency from those faces.  Arithmetic is
// that of k_advect, so results are identical.
// ---------------------------------------------------------------------------
constexpr int ADV_TI = 4, ADV_TJ = 4, ADV_NF = 6;  // flux fields: u, v, th, qv, qc, qr

template <typename T>
__device__ __forceinline__ void faces_east(const KParams<T> &p, const KFields<T> &F, int what, int i, int j, int k,
                                           T *out)
{
    if (p.ubase_adv) {
        if (what & ADV_UV) {
            out[0] = u_east_ub(p, F, i, j, k);
            out[1] = v_east_ub(p, F, i, j, k);
        }
        if (what & ADV_TH) out[2] = s_east_ub(p, F, F.cur[FTH], 0, i, j, k);
        if (what & ADV_Q) {
            out[3] = s_east_ub(p, F, F.cur[FQV], 1, i, j, k);
            out[4] = s_east_ub(p, F, F.cur[FQC], -1, i, j, k);
            out[5] = s_east_ub(p, F, F.cur[FQR], -1, i, j, k);
        }
        return;
    }
    if (what & ADV_UV) {
        out[0] = u_east(p, F, i, j, k);
        out[1] = v_east(p, F, i, j, k);
    }
    if (what & ADV_TH) out[2] = s_east(p, F, F.cur[FTH], F.bar[3], i, j, k);
    if (what & ADV_Q) {
        out[3] = s_east(p, F, F.cur[FQV], F.bar[4], i, j, k);
        out[4] = s_east(p, F, F.cur[FQC], (const T *)nullptr, i, j, k);
        out[5] = s_east(p, F, F.cur[FQR], (const T *)nullptr, i, j, k);
    }
}
template <typename T>
__device__ __forceinline__ void faces_north(const KParams<T> &p, const KFields<T> &F, int what, int i, int j, int k,
                                            T *out)
{
    if (p.ubase_adv) {
        if (what & ADV_UV) {
            out[0] = u_north_ub(p, F, i, j, k);
            out[1] = v_north_ub(p, F, i, j, k);
        }
        if (what & ADV_TH) out[2] = s_north_ub(p, F, F.cur[FTH], 0, i, j, k);
        if (what & ADV_Q) {
            out[3] = s_north_ub(p, F, F.cur[FQV], 1, i, j, k);
            out[4] = s_north_ub(p, F, F.cur[FQC], -1, i, j, k);
            out[5] = s_north_ub(p, F, F.cur[FQR], -1, i, j, k);
        }
        return;
    }
    if (what & ADV_UV) {
        out[0] = u_north(p, F, i, j, k);
        out[1] = v_north(p, F, i, j, k);
    }
    if (what & ADV_TH) out[2] = s_north(p, F, F.cur[FTH], F.bar[3], i, j, k);
    if (what & ADV_Q) {
        out[3] = s_north(p, F, F.cur[FQV], F.bar[4], i, j, k);
        out[4] = s_north(p, F, F.cur[FQC], (const T *)nullptr, i, j, k);
        out[5] = s_north(p, F, F.cur[FQR], (const T *)nullptr, i, j, k);
    }
}
template <typename T>
__device__ __forceinline__ void faces_top(const KParams<T> &p, const KFields<T> &F, int what, int i, int j, int k,
                                          T *out)
{
    if (p.ubase_adv) {
        if (what & ADV_UV) {
            out[0] = u_top_ub(p, F, i, j, k);
            out[1] = v_top_ub(p, F, i, j, k);
        }
        if (what & ADV_TH) out[2] = s_top_ub(p, F, F.cur[FTH], 0, i, j, k);
        if (what & ADV_Q) {
            out[3] = s_top_ub(p, F, F.cur[FQV], 1, i, j, k);
            out[4] = s_top_ub(p, F, F.cur[FQC], -1, i, j, k);
            out[5] = r_top_ub(p, F, i, j, k);
        }
        return;
    }
    if (what & ADV_UV) {
        out[0] = u_top(p, F, i, j, k);
        out[1] = v_top(p, F, i, j, k);
    }
    if (what & ADV_TH) out[2] = s_top(p, F, F.cur[FTH], F.bar[3], i, j, k);
    if (what & ADV_Q) {
        out[3] = s_top(p, F, F.cur[FQV], F.bar[4], i, j, k);
        out[4] = s_top(p, F, F.cur[FQC], (const T *)nullptr, i, j, k);
        out[5] = r_top(p, F, i, j, k);
    }
}

template <typename T, int TI = ADV_TI, int TJ = ADV_TJ>
__device__ void advect_tile_body(const KParams<T> &p, const KFields<T> &F, int bx, int by, T step, T sdtg, int what)
{
    extern __shared__ unsigned char smem_raw[];
    const int NF = ADV_NF;
    const int nz = p.nz, nzi = nz - 2;
    const int i0 = 3 + bx * TI, j0 = 3 + by * TJ;
    const int ti = min(TI, p.nx - 3 - i0), tj = min(TJ, p.ny - 3 - j0);
    // face stores, each [field][...][level k = 0..nz-1]
    T *E = (T *)smem_raw;                    // [(TI+1)][TJ] columns, east face of column i0-1+a
    T *Nf = E + NF * (TI + 1) * TJ * nz;      // [TI][(TJ+1)] columns, north face of column j0-1+b
    T *Tf = Nf + NF * TI * (TJ + 1) * nz;     // [TI][TJ] columns, top face at level k
    const int sE = (TI + 1) * TJ * nz, sN = TI * (TJ + 1) * nz, sT = TI * TJ * nz;
    T tmp[NF];
    // phase 1a: east faces of columns i0-1 .. i0+ti-1
    for (int w = threadIdx.x; w < (TI + 1) * TJ * nzi; w += blockDim.x) {
        const int kk = w % nzi, c = w / nzi, b = c % TJ, a = c / TJ;
        if (a > ti || b >= tj) continue;
        faces_east(p, F, what, i0 - 1 + a, j0 + b, 1 + kk, tmp);
        const int o = (a * TJ + b) * nz + 1 + kk;
#pragma unroll
        for (int f = 0; f < NF; f++) E[f * sE + o] = tmp[f];
    }
    // phase 1b: north faces of rows j0-1 .. j0+tj-1
    for (int w = threadIdx.x; w < TI * (TJ + 1) * nzi; w += blockDim.x) {
        const int kk = w % nzi, c = w / nzi, b = c % (TJ + 1), a = c / (TJ + 1);
        if (a >= ti || b > tj) continue;
        faces_north(p, F, what, i0 + a, j0 - 1 + b, 1 + kk, tmp);
        const int o = (a * (TJ + 1) + b) * nz + 1 + kk;
#pragma unroll
        for (int f = 0; f < NF; f++) Nf[f * sN + o] = tmp[f];
    }
    // phase 1c: top faces at levels 0 .. nz-2
    for (int w = threadIdx.x; w < TI * TJ * (nz - 1); w += blockDim.x) {
        const int k = w % (nz - 1), c = w / (nz - 1), b = c % TJ, a = c / TJ;
        if (a >= ti || b >= tj) continue;
        faces_top(p, F, what, i0 + a, j0 + b, k, tmp);
        const int o = (a * TJ + b) * nz + k;
#pragma unroll
        for (int f = 0; f < NF; f++) Tf[f * sT + o] = tmp[f];
    }
    __syncthreads();
    // phase 2: tendencies
    for (int w = threadIdx.x; w < TI * TJ * nzi; w += blockDim.x) {
        const int kk = w % nzi, c = w / nzi, b = c % TJ, a = c / TJ;
        if (a >= ti || b >= tj) continue;
        const int i = i0 + a, j = j0 + b, k = 1 + kk;
        const int cix = gix(p.ny, nz, i, j, k);
        const T DTZ = p.dtz * p.mu[k];
        const int oe = ((a + 1) * TJ + b) * nz + k, ow = (a * TJ + b) * nz + k;
        const int on = (a * (TJ + 1) + b + 1) * nz + k, os = (a * (TJ + 1) + b) * nz + k;
        const int ot = (a * TJ + b) * nz + k;
        if (what & ADV_UV) {
            const T *U = F.cur[FU], *V = F.cur[FV];
            const int sy = nz, sx = p.ny * nz;
            T ov_u = T(0.25) * (LD(V, cix) + LD(V, cix + sy) + LD(V, cix - sx) + LD(V, cix - sx + sy));
            T ut = -p.dtx * (E[oe] - E[ow]) - p.dty * (Nf[on] - Nf[os]) -
                   DTZ * (p.rhow[k + 1] * Tf[ot] - p.rhow[k] * Tf[ot - 1]) * p.one_d_rhou[k] +
                   p.dt * p.f[j] * ov_u;
            F.P[FU][cix] = LD(F.M[FU], cix) + step * ut;
            T ov_v = T(0.25) * (LD(U, cix) + LD(U, cix + sx) + LD(U, cix - sy) + LD(U, cix + sx - sy));
            T vt = -p.dtx * (E[sE + oe] - E[sE + ow]) - p.dty * (Nf[sN + on] - Nf[sN + os]) -
                   DTZ * (p.rhow[k + 1] * Tf[sT + ot] - p.rhow[k] * Tf[sT + ot - 1]) * p.one_d_rhou[k] -
                   p.dt * p.f[j] * ov_v;
            F.P[FV][cix] = LD(F.M[FV], cix) + step * vt;
        }
        if ((what & ADV_WB) && k >= 2) {
            const T *TH = F.cur[FTH];
            T b0, b1;
            if (!p.moist) {
                b0 = LD(TH, cix) / p.tbv[k];
                b1 = LD(TH, cix - 1) / p.tbv[k - 1];
            } else {
                const T *QV = F.cur[FQV], *QC = F.cur[FQC], *QR = F.cur[FQR];
                b0 = LD(TH, cix) / p.tbv[k] + T(0.61) * LD(QV, cix) - LD(QC, cix) - LD(QR, cix);
                b1 = LD(TH, cix - 1) / p.tbv[k - 1] + T(0.61) * LD(QV, cix - 1) - LD(QC, cix - 1) - LD(QR, cix - 1);
                if (p.ice) {  // buoyancy_cold_micro (advection.cpp:56-58)
                    const T *QI = F.cur[FQI], *QS = F.cur[FQS];
                    b0 = b0 - LD(QI, cix) - LD(QS, cix);
                    b1 = b1 - LD(QI, cix - 1) - LD(QS, cix - 1);
                }
            }
            F.P[FW][cix] = LD(F.M[FW], cix) + sdtg * (b0 + b1);
        }
        auto tend = [&](int f) {
            return -p.dtx * (E[f * sE + oe] - E[f * sE + ow]) - p.dty * (Nf[f * sN + on] - Nf[f * sN + os]) -
                   DTZ * (p.rhow[k + 1] * Tf[f * sT + ot] - p.rhow[k] * Tf[f * sT + ot - 1]) * p.one_d_rhou[k];
        };
        const T *Wc = F.cur[FW];
        if (what & ADV_TH) {
            T t = tend(2);
            T zab = T(0.50) *
                    (p.rhow[k + 1] * LD(Wc, cix + 1) * (p.tb[k + 1] - p.tb[k]) +
                     p.rhow[k] * LD(Wc, cix) * (p.tb[k] - p.tb[k - 1])) *
                    p.one_d_rhou[k];
            t = t - DTZ * zab;
            F.P[FTH][cix] = LD(F.M[FTH], cix) + step * t;
        }
        if (what & ADV_Q) {
            if (p.rf == 1 && !p.ice && !(what & ADV_QVONLY)) {
                const T *QR = F.cur[FQR];
                F.vt[cix] = fall_speed_point(p, LD(QR, cix), k);
                if (k == 1) F.vt[cix - 1] = fall_speed_point(p, LD(QR, cix), 1);
            }
            T tv = tend(3);
            T zab = T(0.50) *
                    (p.rhow[k + 1] * LD(Wc, cix + 1) * (p.qb[k + 1] - p.qb[k]) +
                     p.rhow[k] * LD(Wc, cix) * (p.qb[k] - p.qb[k - 1])) *
                    p.one_d_rhou[k];
            tv = tv - DTZ * zab;
            T qv = LD(F.M[FQV], cix) + step * tv;
            T qc = LD(F.M[FQC], cix) + step * tend(4);
            T qr = LD(F.M[FQR], cix) + step * tend(5);
            if (what & ADV_ZERO) {
                unsigned char bits = 0;
                if (qc < 0) { qc = 0; bits |= 2; }
                if (qr < 0) { qr = 0; bits |= 4; }
                T qbar = p.ubase_adv ? BTAB(BT_QB, k) : LD(F.bar[4], cix);
                if (qv + qbar + p.qb[k] < 0) { qv = -(qbar + p.qb[k]); bits |= 1; }
                if (F.qmask) F.qmask[cix] = bits;
            }
            F.P[FQV][cix] = qv;
            if (!(what & ADV_QVONLY)) {
                F.P[FQC][cix] = qc;
                F.P[FQR][cix] = qr;
            }
        }
    }
}

template <typename T, int TI = ADV_TI, int TJ = ADV_TJ>
__global__ void __launch_bounds__(256) k_advect_tile(KParams<T> p, KFields<T> F, T step, T sdtg, int what)
{
    advect_tile_body<T, TI, TJ>(p, F, blockIdx.x, blockIdx.y, step, sdtg, what);
}

// shared memory of an advection tile: the face stores of every flux field
__host__ __device__ constexpr size_t advect_tile_smem(int ti, int tj, int nz, size_t tsize)
{
    return (size_t)ADV_NF * ((ti + 1) * tj + ti * (tj + 1) + ti * tj) * nz * tsize;
}

// ---------------------------------------------------------------------------
// lateral copies of UP/VP/WP before the pressure solve:
// mirror_boundaries (boundaries.cpp:363-379) or periodic_uvw_boundaries
// (:546-555).  Writes only edge points, reads only non-edge points.
// ---------------------------------------------------------------------------
template <typename T>
__device__ void mirror_edges_body(const KParams<T> &p, T *a, T *b, T *c, long t)
{
    const int ne = 2 * (p.nx + p.ny - 2);  // edge columns
    const int nzi = p.nz - 2;
    if (t >= (long)ne * nzi) return;
    const int k = 1 + (int)(t % nzi);
    int e = (int)(t / nzi);
    int i, j;
    if (e < p.ny) { i = 0; j = e; }
    else if ((e -= p.ny) < p.ny) { i = p.nx - 1; j = e; }
    else if ((e -= p.ny) < p.nx - 2) { i = 1 + e; j = 0; }
    else { e -= p.nx - 2; i = 1 + e; j = p.ny - 1; }
    const int si = min(max(i, 1), p.nx - 2), sj = min(max(j, 1), p.ny - 2);
    const long d = gix(p.ny, p.nz, i, j, k), s = gix(p.ny, p.nz, si, sj, k);
    a[d] = a[s];
    b[d] = b[s];
    c[d] = c[s];
}
template <typename T>
__global__ void k_mirror_edges(KParams<T> p, T *a, T *b, T *c)
{
    mirror_edges_body(p, a, b, c, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

// periodic_boundaries_east_west (boundaries.cpp:562-574) for up to 4 fields:
// columns 0,1,2 <- NX-6..NX-4 and NX-3..NX-1 <- 3..5, all j and k
template <typename T>
__global__ void k_periodic_copy(KParams<T> p, T *a, T *b, T *c, T *d)
{
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long per = (long)p.ny * p.nz;
    if (t >= 6 * per) return;
    const int col = (int)(t / per);
    const long r = t % per;
    const int dst = col < 3 ? col : p.nx - 6 + col;
    const int src = col < 3 ? p.nx - 6 + col : col;  // col 3..5 -> dst NX-3..NX-1, src 3..5
    const long od = (long)dst * per + r, os = (long)src * per + r;
    if (a) a[od] = a[os];
    if (b) b[od] = b[os];
    if (c) c[od] = c[os];
    if (d) d[od] = d[os];
}

// ---------------------------------------------------------------------------
// shared-memory mixed-radix FFT (Stockham autosort).  Element (point n,
// line l) of a batch of L lines lives at buf[n*L + l].  Twiddle table
// tw[t] = exp(-2 pi i t / N); inverse transforms use its conjugate.
// Unnormalised, like FFTW.
// ---------------------------------------------------------------------------
constexpr int PPM_MAXZ = 128;  // largest NZ the column kernels support

// asynchronous element copy global -> shared (cp.async), zero-filled where
// `ok` is false (src is then a placeholder address and is not read).
// 4- and 8-byte elements go through L1; 16-byte ones (complex FP64) bypass it.
template <typename E>
__device__ __forceinline__ void cp_elem(E *dst, const E *src, bool ok)
{
    static_assert(sizeof(E) == 4 || sizeof(E) == 8 || sizeof(E) == 16, "cp.async copies 4, 8 or 16 bytes");
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = ok ? (int)sizeof(E) : 0;
    if (sizeof(E) == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
    else if (sizeof(E) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
// every copy of this thread complete, then visible to the block
__device__ __forceinline__ void cp_wait_all_sync()
{
    cp_commit();
    cp_wait<0>();
    __syncthreads();
}

struct FftPlan {
    int n, nfac;
    int fac[24];
    int nslog[24];  // log2 of the sub-transform size before each pass, -1 if not a power of two
};

template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b)
{
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename T2>
__device__ __forceinline__ T2 twid(const T2 *tw, int t, bool inv)
{
    T2 w = tw[t];
    if (inv) w.y = -w.y;
    return w;
}

// Batched shared-memory FFT.  L lines; element (point n, line l) lives at
// buf[n*ps + l] with ps >= L (padding keeps a thread that walks one line
// across points off a single bank).  Threads are 2-D: x runs over lines,
// y over the butterflies of a pass, so no index needs a division by L.
template <typename T, typename T2>
__device__ T2 *fft_smem(T2 *a, T2 *b, int L, const FftPlan &P, const T2 *__restrict__ tw, bool inv, int ps)
{
    const int N = P.n;
    int Ns = 1;
    for (int f = 0; f < P.nfac; ++f) {
        const int R = P.fac[f];
        const int nb = N / R;
        const int ts = N / (Ns * R);
        const int nsl = P.nslog[f];
        for (int j = threadIdx.y; j < nb; j += blockDim.y) {
            int k, jb;
            if (nsl >= 0) { k = j & (Ns - 1); jb = j >> nsl; }
            else { k = j % Ns; jb = j / Ns; }
            const int ob = jb * Ns * R + k;
            for (int l = threadIdx.x; l < L; l += blockDim.x) {
                if (R == 2) {
                    T2 v0 = a[j * ps + l];
                    T2 v1 = a[(j + nb) * ps + l];
                    if (k) v1 = cmul(v1, twid(tw, k * ts, inv));
                    T2 s, d;
                    s.x = v0.x + v1.x; s.y = v0.y + v1.y;
                    d.x = v0.x - v1.x; d.y = v0.y - v1.y;
                    b[ob * ps + l] = s;
                    b[(ob + Ns) * ps + l] = d;
                } else if (R == 4) {
                    T2 v0 = a[j * ps + l];
                    T2 v1 = a[(j + nb) * ps + l];
                    T2 v2 = a[(j + 2 * nb) * ps + l];
                    T2 v3 = a[(j + 3 * nb) * ps + l];
                    if (k) {
                        v1 = cmul(v1, twid(tw, k * ts, inv));
                        v2 = cmul(v2, twid(tw, 2 * k * ts, inv));
                        v3 = cmul(v3, twid(tw, 3 * k * ts, inv));
                    }
                    T2 s02, d02, s13, d13, x0, x1, x2, x3;
                    s02.x = v0.x + v2.x; s02.y = v0.y + v2.y;
                    d02.x = v0.x - v2.x; d02.y = v0.y - v2.y;
                    s13.x = v1.x + v3.x; s13.y = v1.y + v3.y;
                    d13.x = v1.x - v3.x; d13.y = v1.y - v3.y;
                    x0.x = s02.x + s13.x; x0.y = s02.y + s13.y;
                    x2.x = s02.x - s13.x; x2.y = s02.y - s13.y;
                    if (!inv) {  // X1 = d02 - i d13, X3 = d02 + i d13
                        x1.x = d02.x + d13.y; x1.y = d02.y - d13.x;
                        x3.x = d02.x - d13.y; x3.y = d02.y + d13.x;
                    } else {
                        x1.x = d02.x - d13.y; x1.y = d02.y + d13.x;
                        x3.x = d02.x + d13.y; x3.y = d02.y - d13.x;
                    }
                    b[ob * ps + l] = x0;
                    b[(ob + Ns) * ps + l] = x1;
                    b[(ob + 2 * Ns) * ps + l] = x2;
                    b[(ob + 3 * Ns) * ps + l] = x3;
                } else {  // generic radix: direct R-point DFT with combined twiddles
                    for (int m = 0; m < R; ++m) {
                        T2 acc;
                        acc.x = T(0);
                        acc.y = T(0);
                        for (int r = 0; r < R; ++r) {
                            const int t = (k * r * ts + ((r * m) % R) * nb) % N;
                            T2 x = a[(j + r * nb) * ps + l];
                            T2 wv = twid(tw, t, inv);
                            acc.x += x.x * wv.x - x.y * wv.y;
                            acc.y += x.x * wv.y + x.y * wv.x;
                        }
                        b[(ob + m * Ns) * ps + l] = acc;
                    }
                }
            }
        }
        __syncthreads();
        T2 *tmp = a;
        a = b;
        b = tmp;
        Ns *= R;
    }
    return a;
}

// divergence tendency of the pressure equation at a physical point
// (divergence3d, pressure.cpp:1340-1381)
template <typename T>
__device__ __forceinline__ T divergence(const KParams<T> &p, const KFields<T> &F, int i, int j, int k, T sdt)
{
    const T *UP = F.P[FU], *VP = F.P[FV], *WP = F.P[FW];
    const long c = gix(p.ny, p.nz, i, j, k);
    T d = p.rhou[k] * (UP[c + (long)p.ny * p.nz] - UP[c]) * p.one_d_dx +
          p.rhou[k] * (VP[c + p.nz] - VP[c]) * p.one_d_dy +
          (p.rhow[k + 1] * WP[c + 1] - p.rhow[k] * WP[c]) * (p.one_d_dz * p.mu[k]);
    d /= sdt;
    return d;
}

// divergence (with the mirror / periodic placement of divergence3d and
// divergence3d_periodic) + forward FFT along y.  Block = (spectral row i,
// tile of KT levels starting at level 1).
template <typename T>
__device__ void div_fft_y_body(const KParams<T> &p, const KFields<T> &F, typename V2<T>::t *spec, const FftPlan &pj,
                               const typename V2<T>::t *tw, T sdt, int KT, int bx, int by)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.nj * KT;
    const int is = bx;
    const int k0 = 1 + by * KT;
    const int kt = min(KT, p.nz - 1 - k0);
    int ii;
    if (!p.periodic) ii = min(max(is, 1), p.nx - 2);
    else ii = is + 3;
    // several rows in flight per thread: the loads of a row do not wait for
    // the previous row's store
#pragma unroll 4
    for (int q = threadIdx.y; q < p.nj; q += blockDim.y)
        for (int l = threadIdx.x; l < KT; l += blockDim.x) {
            T2 v;
            v.y = T(0);
            v.x = T(0);
            if (l < kt) {
                const int jj = min(max(q, 1), p.ny - 2);
                v.x = divergence(p, F, ii, jj, k0 + l, sdt);
            }
            a[q * KT + l] = v;
        }
    __syncthreads();
    T2 *r = fft_smem<T, T2>(a, b, KT, pj, tw, false, KT);
    for (int q = threadIdx.y; q < p.nj; q += blockDim.y)
        for (int l = threadIdx.x; l < kt; l += blockDim.x)
            spec[((long)is * p.nj + q) * p.nz + k0 + l] = r[q * KT + l];
}
template <typename T>
__global__ void k_div_fft_y(KParams<T> p, KFields<T> F, typename V2<T>::t *spec, FftPlan pj,
                            const typename V2<T>::t *tw, T sdt, int KT)
{
    div_fft_y_body(p, F, spec, pj, tw, sdt, KT, blockIdx.y, blockIdx.x);
}

// FFT along x of the spectral buffer for one y-wavenumber q and level tile
// bx.  sign: forward (false) or inverse (true).  Block (KT, any).
template <typename T>
__device__ void fft_x_body(const KParams<T> &p, typename V2<T>::t *spec, const FftPlan &pi,
                           const typename V2<T>::t *tw, int inv, int KT, int q, int bx)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.ni * KT;
    const int k0 = 1 + bx * KT;
    const int kt = min(KT, p.nz - 1 - k0);
    for (int i = threadIdx.y; i < p.ni; i += blockDim.y)
        for (int l = threadIdx.x; l < KT; l += blockDim.x)
            cp_elem(a + i * KT + l, spec + ((long)i * p.nj + q) * p.nz + k0 + min(l, kt - 1), l < kt);
    cp_wait_all_sync();
    T2 *r = fft_smem<T, T2>(a, b, KT, pi, tw, inv != 0, KT);
    for (int i = threadIdx.y; i < p.ni; i += blockDim.y)
        for (int l = threadIdx.x; l < kt; l += blockDim.x)
            spec[((long)i * p.nj + q) * p.nz + k0 + l] = r[i * KT + l];
}
// the level tiles of a wavenumber run next to each other (shared rows)
template <typename T>
__global__ void k_fft_x(KParams<T> p, typename V2<T>::t *spec, FftPlan pi, const typename V2<T>::t *tw,
                        int inv, int KT)
{
    fft_x_body(p, spec, pi, tw, inv, KT, blockIdx.y, blockIdx.x);
}

// normalisation (pressure.cpp:827) + Thomas algorithm per horizontal
// wavenumber (:834-871), with the diagonal of init_fft3d's stretched branch
// (:778-792) formed from the (cos kx + cos ly - 2) table.  One thread per
// column; columns staged through shared memory for coalesced access.
template <typename T, typename A>
__device__ void thomas_column(const KParams<T> &p, typename V2<T>::t *x, A *Fw, long col, double size2d,
                              const A *rhou, const A *ac, const A *cc, const A *vc)
{
    typedef typename V2<T>::t T2;
    const int nz = p.nz;
    const A h = (A)p.hcoef[col];
    const A dx2 = (A)p.dx2;
    A xr[2], z;
    // level 1
    z = A(1.0) / (rhou[1] * A(2.0) * h / dx2 - vc[1]);
    A Fk = cc[1] * z;
    Fw[1] = Fk;
    A pr = (A)x[1].x / (A)size2d, pim = (A)x[1].y / (A)size2d;
    pr = pr * z;
    pim = pim * z;
    x[1].x = (T)pr;
    x[1].y = (T)pim;
    xr[0] = pr;
    xr[1] = pim;
    for (int k = 2; k < nz - 1; k++) {
        A bk = rhou[k] * A(2.0) * h / dx2 - vc[k];
        z = A(1.0) / (bk - ac[k] * Fk);
        Fk = cc[k] * z;
        Fw[k] = Fk;
        A vr = (A)x[k].x / (A)size2d, vi = (A)x[k].y / (A)size2d;
        vr = (vr - ac[k] * xr[0]) * z;
        vi = (vi - ac[k] * xr[1]) * z;
        x[k].x = (T)vr;
        x[k].y = (T)vi;
        xr[0] = vr;
        xr[1] = vi;
    }
    if (col == 0) {  // mean-mode gauge (pressure.cpp:858-859)
        x[nz - 2].x = T(0);
        x[nz - 2].y = T(0);
    }
    A nr = (A)x[nz - 2].x, ni = (A)x[nz - 2].y;
    for (int k = nz - 3; k >= 1; k--) {
        A vr = (A)x[k].x, vi = (A)x[k].y;
        vr -= Fw[k] * nr;
        vi -= Fw[k] * ni;
        x[k].x = (T)vr;
        x[k].y = (T)vi;
        nr = vr;
        ni = vi;
    }
}

// FP32 Thomas solve of one wavenumber: the reference recurrence
// (pressure.cpp:834-871) with the horizontal term of the diagonal hoisted and
// one reciprocal per level instead of three divisions.
__device__ __forceinline__ void thomas_column_fast(float2 *x, float *Fw, int nz, float hb, float inv_size2d,
                                                   const float *rhou, const float *ac, const float *cc,
                                                   const float *vc, bool gauge)
{
    float z = __frcp_rn(rhou[1] * hb - vc[1]);
    float Fk = cc[1] * z;
    Fw[1] = Fk;
    float xr = x[1].x * inv_size2d * z, xi = x[1].y * inv_size2d * z;
    x[1] = make_float2(xr, xi);
    for (int k = 2; k < nz - 1; k++) {
        z = __frcp_rn(rhou[k] * hb - vc[k] - ac[k] * Fk);
        Fk = cc[k] * z;
        Fw[k] = Fk;
        xr = (x[k].x * inv_size2d - ac[k] * xr) * z;
        xi = (x[k].y * inv_size2d - ac[k] * xi) * z;
        x[k] = make_float2(xr, xi);
    }
    if (gauge) { xr = 0.f; xi = 0.f; x[nz - 2] = make_float2(0.f, 0.f); }
    for (int k = nz - 3; k >= 1; k--) {
        xr = x[k].x - Fw[k] * xr;
        xi = x[k].y - Fw[k] * xi;
        x[k] = make_float2(xr, xi);
    }
}

// FP64 solve of one wavenumber by parallel cyclic reduction across a warp
// (rows 1..nl in shared memory, log2(nl) reduction steps, every row at once)
// for the near-singular low wavenumbers of FP32 contexts.  For the mean mode
// (gauge) the last row is replaced by x = 0, which is what the reference's
// pinning after forward elimination (pressure.cpp:858-859) amounts to.
constexpr int PCR_ROWS = PPM_MAXZ;      // rows of one reduction (levels 1..NZ-2, NZ <= PPM_MAXZ)
constexpr int PCR_WK = 10 * PCR_ROWS;    // workspace doubles: 2 buffers x (a, b, c, dr, di)

template <typename T2>
__device__ void pcr_column_f64(T2 *x, int nl, double hcol, double dx2, double size2d, const double *rhou,
                               const double *ac, const double *cc, const double *vc, bool gauge, double *wk)
{
    // wk: PCR_WK doubles, 2 buffers x 5 arrays x PCR_ROWS rows (a, b, c, dr,
    // di).  Blocks may be 2-D, so the lane comes from the linear thread index.
    const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
    constexpr int R = PCR_ROWS;
    double *A0 = wk, *B0 = wk + R, *C0 = wk + 2 * R, *R0 = wk + 3 * R, *I0 = wk + 4 * R;
    double *A1 = wk + 5 * R, *B1 = wk + 6 * R, *C1 = wk + 7 * R, *R1 = wk + 8 * R, *I1 = wk + 9 * R;
    for (int r = lane; r < R; r += 32) {
        if (r < nl) {
            const int k = r + 1;
            double a = ac[k], c = cc[k];
            double b = rhou[k] * 2.0 * hcol / dx2 - vc[k];
            double dr = (double)x[k].x / size2d, di = (double)x[k].y / size2d;
            if (gauge && r == nl - 1) { a = 0.0; b = 1.0; c = 0.0; dr = 0.0; di = 0.0; }
            A0[r] = a; B0[r] = b; C0[r] = c; R0[r] = dr; I0[r] = di;
        }
    }
    __syncwarp();
    for (int s = 1; s < nl; s <<= 1) {
        for (int r = lane; r < nl; r += 32) {
            double a = A0[r], b = B0[r], c = C0[r], dr = R0[r], di = I0[r];
            double na = 0.0, nc = 0.0;
            if (r - s >= 0) {
                const double al = -a / B0[r - s];
                na = al * A0[r - s];
                b += al * C0[r - s];
                dr += al * R0[r - s];
                di += al * I0[r - s];
            }
            if (r + s < nl) {
                const double ga = -c / B0[r + s];
                nc = ga * C0[r + s];
                b += ga * A0[r + s];
                dr += ga * R0[r + s];
                di += ga * I0[r + s];
            }
            A1[r] = na; B1[r] = b; C1[r] = nc; R1[r] = dr; I1[r] = di;
        }
        __syncwarp();
        double *t;
        t = A0; A0 = A1; A1 = t; t = B0; B0 = B1; B1 = t; t = C0; C0 = C1; C1 = t;
        t = R0; R0 = R1; R1 = t; t = I0; I0 = I1; I1 = t;
    }
    for (int r = lane; r < nl; r += 32) {
        T2 v;
        v.x = (decltype(v.x))(R0[r] / B0[r]);
        v.y = (decltype(v.y))(I0[r] / B0[r]);
        x[r + 1] = v;
    }
    __syncwarp();
}

// x[r+1] = sum_j A[r][j] d[j] for the real (d = wk) and imaginary (d = wk + nl)
// parts, A = Minv or (TRANS) its transpose, the last row zero when TRANS.  Four
// lanes share an output (columns j = g, g+4, ...) and add their partial sums by
// shuffles; only the block's full warps take part.
template <bool TRANS, typename T2>
__device__ __forceinline__ void mean_mode_products(T2 *x, int nl, const double *__restrict__ Minv, const double *wk)
{
    constexpr int GL = 4;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    const int nfull = nth & ~31, nout = 2 * nl;
    if (tid >= nfull) return;
    for (int base = 0; base < nout * GL; base += nfull) {
        const int w = base + tid, o = w / GL, g = w % GL;
        double s = 0.0;
        int r = 0, part = 0;
        if (o < nout) {
            r = o % nl;
            part = o / nl;
            const double *d = wk + part * nl;
            for (int j = g; j < nl; j += GL)
                s += (TRANS ? Minv[(size_t)j * nl + r] : Minv[(size_t)r * nl + j]) * d[j];
        }
        s += __shfl_down_sync(0xffffffffu, s, 2, GL);
        s += __shfl_down_sync(0xffffffffu, s, 1, GL);
        if (o < nout && g == 0) {
            if (TRANS && r == nl - 1) s = 0.0;
            if (part == 0) x[r + 1].x = (decltype(x[0].x))s;
            else x[r + 1].y = (decltype(x[0].y))s;
        }
    }
}

// The mean mode (p, q) = (0, 0) of an FP32 context in FP64: x = M'^-1 d with
// the inverse of its gauge-pinned tridiagonal system (top row x = 0, as the
// reduction above sets it) built once on the host; d = the column / size2d,
// zero in the gauge row.  Every thread of the block calls it (it holds two
// block barriers); x[1 .. nl] is the column, wk 2 nl doubles of shared memory.
template <typename T2>
__device__ void mean_mode_solve(T2 *x, int nl, const double *__restrict__ Minv, double size2d, double *wk)
{
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    for (int r = tid; r < nl; r += nth) {
        const bool g = r == nl - 1;
        wk[r] = g ? 0.0 : (double)x[r + 1].x / size2d;
        wk[nl + r] = g ? 0.0 : (double)x[r + 1].y / size2d;
    }
    __syncthreads();
    mean_mode_products<false>(x, nl, Minv, wk);
    __syncthreads();
}

// The adjoint of mean_mode_solve: z = (M'^T)^-1 d = (M'^-1)^T d with d = the
// column / size2d in every row, then z_top = 0 (the transposed gauge).  Block-
// wide as mean_mode_solve.
template <typename T2>
__device__ void mean_mode_solve_T(T2 *x, int nl, const double *__restrict__ Minv, double size2d, double *wk)
{
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    for (int r = tid; r < nl; r += nth) {
        wk[r] = (double)x[r + 1].x / size2d;
        wk[nl + r] = (double)x[r + 1].y / size2d;
    }
    __syncthreads();
    mean_mode_products<true>(x, nl, Minv, wk);
    __syncthreads();
}

// true for the low horizontal wavenumbers solved in FP64 in FP32 contexts
template <typename T>
__device__ __forceinline__ bool low_mode(const KParams<T> &p, long col)
{
    if (p.low_modes <= 0) return false;
    const int pp = (int)(col / p.nj), qq = (int)(col % p.nj);
    return min(pp, p.ni - pp) < p.low_modes && min(qq, p.nj - qq) < p.low_modes;
}

// columns bx*TC .. of the spectral buffer
template <typename T>
__device__ void thomas_body(const KParams<T> &p, typename V2<T>::t *spec, int TC, long bx)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    __shared__ double pcr_wk[PCR_WK];
    const int cs = p.nz | 1;  // odd column stride: no bank conflicts between columns
    T2 *xs = (T2 *)smem_raw;
    T *fs = (T *)(xs + (long)TC * cs);
    const long ncol = (long)p.ni * p.nj;
    const long c0 = bx * TC;
    const int nc = (int)min((long)TC, ncol - c0);
    T2 *g = spec + c0 * p.nz;
    for (int w = threadIdx.x; w < nc * p.nz; w += blockDim.x) cp_elem(xs + (w / p.nz) * cs + w % p.nz, g + w, true);
    cp_wait_all_sync();
    const double size2d = (double)(p.ni * p.nj);
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const long col = c0 + c;
        if (sizeof(T) == 8) {
            double Floc[PPM_MAXZ];
            thomas_column<T, double>(p, xs + (long)c * cs, Floc, col, size2d, p.rhou_d, p.acoef_d, p.ccoef_d,
                                     p.vcoef_d);
        } else if (!low_mode(p, col)) {
            const float hb = 2.0f * (float)p.hcoef[col] / (float)p.dx2;
            thomas_column_fast((float2 *)(xs + (long)c * cs), (float *)(fs + (long)c * cs), p.nz, hb,
                               (float)(1.0 / size2d), (const float *)p.rhou, (const float *)p.acoef,
                               (const float *)p.ccoef, (const float *)p.vcoef, col == 0);
        }
    }
    if (sizeof(T) != 8 && p.low_modes > 0) {
        const int warp = threadIdx.x >> 5;
        if (warp == 0) {  // the low modes of this block, one after the other
            for (int c = 0; c < nc; c++) {
                const long col = c0 + c;
                if (!low_mode(p, col) || (col == 0 && p.mean_inv)) continue;
                pcr_column_f64(xs + (long)c * cs, p.nz - 2, p.hcoef[col], p.dx2, size2d, p.rhou_d, p.acoef_d,
                               p.ccoef_d, p.vcoef_d, col == 0, pcr_wk);
            }
        }
        if (c0 == 0 && p.mean_inv) {  // the mean mode: block-wide, after warp 0's reductions
            __syncthreads();
            mean_mode_solve(xs, p.nz - 2, p.mean_inv, size2d, pcr_wk);
        }
    }
    __syncthreads();
    for (int w = threadIdx.x; w < nc * p.nz; w += blockDim.x) g[w] = xs[(w / p.nz) * cs + w % p.nz];
}
template <typename T>
__global__ void k_thomas(KParams<T> p, typename V2<T>::t *spec, int TC)
{
    thomas_body(p, spec, TC, blockIdx.x);
}

template <typename T>
__device__ void spectral_x_body(const KParams<T> &p, typename V2<T>::t *spec, const FftPlan &pi,
                                const typename V2<T>::t *tw, int ps, int bx)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    __shared__ T c_r[PPM_MAXZ], c_a[PPM_MAXZ], c_c[PPM_MAXZ], c_v[PPM_MAXZ];
    __shared__ double d_r[PPM_MAXZ], d_a[PPM_MAXZ], d_c[PPM_MAXZ], d_v[PPM_MAXZ];
    __shared__ double pcr_wk[PCR_WK];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.ni * ps;
    const int q = bx;
    const int nl = p.nz - 2;  // levels 1..NZ-2 are the lines
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    for (int k = tid; k < p.nz; k += nth) {
        c_r[k] = p.rhou[k]; c_a[k] = p.acoef[k]; c_c[k] = p.ccoef[k]; c_v[k] = p.vcoef[k];
        d_r[k] = p.rhou_d[k]; d_a[k] = p.acoef_d[k]; d_c[k] = p.ccoef_d[k]; d_v[k] = p.vcoef_d[k];
    }
    for (int i = threadIdx.y; i < p.ni; i += blockDim.y)
        for (int l = threadIdx.x; l < nl; l += blockDim.x)
            cp_elem(a + i * ps + l, spec + ((long)i * p.nj + q) * p.nz + 1 + l, true);
    cp_wait_all_sync();
    T2 *r = fft_smem<T, T2>(a, b, nl, pi, tw, false, ps);
    T2 *fr = (r == a) ? b : a;  // free buffer: holds the Thomas coefficients
    const double size2d = (double)(p.ni * p.nj);
    const int aq = min(q, p.nj - q);
    const bool q_low = p.low_modes > 0 && aq < p.low_modes;
    if (sizeof(T) == 8) {  // parity path: the reference's Thomas recurrence in FP64
        for (int pp = tid; pp < p.ni; pp += nth) {
            const long col = (long)pp * p.nj + q;
            double *Fw = (double *)(fr + (long)pp * ps) - 1;
            thomas_column<T, double>(p, r + (long)pp * ps - 1, Fw, col, size2d, d_r, d_a, d_c, d_v);
        }
    } else {
        const float dx2 = (float)p.dx2, inv_s = (float)(1.0 / size2d);
        for (int pp = tid; pp < p.ni; pp += nth) {
            const int ap = min(pp, p.ni - pp);
            if (q_low && ap < p.low_modes) continue;  // FP64 islands below
            const long col = (long)pp * p.nj + q;
            const float hb = 2.0f * (float)p.hcoef[col] / dx2;
            float *Fw = (float *)(fr + (long)pp * ps) - 1;
            thomas_column_fast((float2 *)(r + (long)pp * ps - 1), Fw, p.nz, hb, inv_s, (const float *)c_r,
                               (const float *)c_a, (const float *)c_c, (const float *)c_v, col == 0);
        }
        if (q_low) {  // low (p,q) wavenumbers: FP64 by warp PCR on warp 0
            const int warp = tid >> 5;
            if (warp == 0) {
                int islands[16], nis = 0;
                for (int pp = 0; pp < p.low_modes && nis < 15; pp++) {
                    islands[nis++] = pp;
                    if (pp > 0) islands[nis++] = p.ni - pp;
                }
                for (int w = 0; w < nis; w++) {
                    const int pp = islands[w];
                    const long col = (long)pp * p.nj + q;
                    if (col == 0 && p.mean_inv) continue;
                    pcr_column_f64(r + (long)pp * ps - 1, nl, p.hcoef[col], p.dx2, size2d, d_r, d_a, d_c, d_v,
                                   col == 0, pcr_wk);
                }
            }
            if (q == 0 && p.mean_inv) {  // the mean mode: block-wide, after warp 0's reductions
                __syncthreads();
                mean_mode_solve(r - 1, nl, p.mean_inv, size2d, pcr_wk);
            }
        }
    }
    __syncthreads();
    T2 *o = fft_smem<T, T2>(r, fr, nl, pi, tw, true, ps);
    for (int i = threadIdx.y; i < p.ni; i += blockDim.y)
        for (int l = threadIdx.x; l < nl; l += blockDim.x) spec[((long)i * p.nj + q) * p.nz + 1 + l] = o[i * ps + l];
}
template <typename T>
__global__ void k_spectral_x(KParams<T> p, typename V2<T>::t *spec, FftPlan pi, const typename V2<T>::t *tw,
                             int ps)
{
    spectral_x_body(p, spec, pi, tw, ps, blockIdx.x);
}
// the same with registers sized for blocks of up to 1024 threads
template <typename T>
__global__ void __launch_bounds__(1024) k_spectral_x_1k(KParams<T> p, typename V2<T>::t *spec, FftPlan pi,
                                                        const typename V2<T>::t *tw, int ps)
{
    spectral_x_body(p, spec, pi, tw, ps, blockIdx.x);
}

// inverse FFT along y + PI = real part, with the level copies of
// poisson_fft3d (pressure.cpp:878-892) and the lateral placement of
// mirror_boundaries(PI) or periodic_pressure_boundaries.
template <typename T>
__device__ void ifft_y_pi_body(const KParams<T> &p, const KFields<T> &F, typename V2<T>::t *spec, const FftPlan &pj,
                               const typename V2<T>::t *tw, int KT, int bx, int by)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.nj * KT;
    const int is = bx;
    const int k0 = 1 + by * KT;
    const int kt = min(KT, p.nz - 1 - k0);
    for (int q = threadIdx.y; q < p.nj; q += blockDim.y)
        for (int l = threadIdx.x; l < KT; l += blockDim.x)
            cp_elem(a + q * KT + l, spec + ((long)is * p.nj + q) * p.nz + k0 + min(l, kt - 1), l < kt);
    cp_wait_all_sync();
    T2 *r = fft_smem<T, T2>(a, b, KT, pj, tw, true, KT);
    T *PI = F.pi;
    const int nz = p.nz, ny = p.ny;
    for (int j = threadIdx.y; j < p.nj; j += blockDim.y)
      for (int l = threadIdx.x; l < kt; l += blockDim.x) {
        const int w = j * KT + l;
        const int k = k0 + l;
        if (!p.periodic) {
            const int i = is;
            // levels 1..NZ-2: mirrored in x and y
            const T v = r[min(max(j, 1), ny - 2) * KT + l].x;
            if (i >= 1 && i <= p.nx - 2) {
                PI[gix(ny, nz, i, j, k)] = v;
                if (i == 1) PI[gix(ny, nz, 0, j, k)] = v;
                if (i == p.nx - 2) PI[gix(ny, nz, p.nx - 1, j, k)] = v;
            }
            // levels 0 and NZ-1: raw copies of levels 1 and NZ-2
            const T raw = r[w].x;
            if (k == 1) PI[gix(ny, nz, i, j, 0)] = raw;
            if (k == nz - 2) PI[gix(ny, nz, i, j, nz - 1)] = raw;
        } else {
            const int i = is + 3;
            const T raw = r[w].x;
            int dst[2] = {i, -1};
            if (i >= p.nx - 6 && i <= p.nx - 4) dst[1] = i - (p.nx - 6);
            if (i >= 3 && i <= 5) dst[1] = p.nx - 3 + (i - 3);
            for (int d = 0; d < 2; d++) {
                if (dst[d] < 0) continue;
                PI[gix(ny, nz, dst[d], j, k)] = raw;
                if (k == 1) PI[gix(ny, nz, dst[d], j, 0)] = raw;
                if (k == nz - 2) PI[gix(ny, nz, dst[d], j, nz - 1)] = raw;
            }
        }
    }
}

template <typename T>
__global__ void k_ifft_y_pi(KParams<T> p, KFields<T> F, typename V2<T>::t *spec, FftPlan pj,
                            const typename V2<T>::t *tw, int KT)
{
    ifft_y_pi_body(p, F, spec, pj, tw, KT, blockIdx.y, blockIdx.x);
}

// ---------------------------------------------------------------------------
// column post-processing: a warp per (i,j) column applies, per field and in
// the reference's order, zero_moisture (microphysics.cpp:675-700), the
// pressure-gradient projection (solver.cpp:120-135), the sponge strips
// (boundaries.cpp:436-498), the periodic copy (:562-574), the top/bottom
// conditions (:304-326) and Rayleigh damping (damping.cpp:1148-1177); then
// writes the forecast buffer and optionally the start-of-step buffer.  All
// values of a column are read before any is written, and the k=1 / k=NZ-2
// values the vertical condition needs travel by shuffle, so no thread reads a
// point another thread writes.
// ---------------------------------------------------------------------------
enum { PF_ZERO = 1, PF_PROJECT = 2, PF_SPONGE = 4, PF_VBC = 8, PF_RAYLEIGH = 16, PF_WRITE_M = 32,
       PF_PCOPY = 64 };
enum { COLS_ALL = 0, COLS_TARGETS = 1, COLS_NONTARGETS = 2 };
constexpr int KPL = 4;  // levels per lane: NZ <= 128

template <typename T>
__device__ __forceinline__ T chain_value(const KParams<T> &p, const KFields<T> &F, int f, int flags, int i,
                                         int j, int k, T v, T step)
{
    const long c = gix(p.ny, p.nz, i, j, k);
    if (flags & PF_ZERO) {
        if (f == FQC || f == FQR) {
            if (v < 0) v = 0;
        } else if (f == FQV) {
            if (i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1 && k >= 1 && k < p.nz - 1) {
                T qbar = F.bar[4][c];
                if (v + qbar + p.qb[k] < 0) v = -(qbar + p.qb[k]);
            }
        }
    }
    if ((flags & PF_PROJECT) && f <= FW && i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1 && k >= 1 &&
        k < p.nz - 1) {
        const T *PI = F.pi;
        if (f == FU) v = v - step * (p.dtx * (PI[c] - PI[c - (long)p.ny * p.nz]));
        else if (f == FV) v = v - step * (p.dty * (PI[c] - PI[c - p.nz]));
        else if (k >= 2) v = v - step * ((p.dtz * p.mw[k]) * (PI[c] - PI[c - 1]));
    }
    if ((flags & PF_SPONGE) && k >= 1) {
        if (!p.periodic && j >= 1) {
            if (i >= p.eb && i < p.ee) v = v - p.ce[i - p.eb] * v;
            if (i >= p.wb && i < p.we) v = v - p.cw[i - p.wb] * v;
        }
        if (i >= 1) {
            if (j >= p.sb && j < p.se) v = v - p.cs[j - p.sb] * v;
            if (j >= p.nb && j < p.ne) v = v - p.cn[j - p.nb] * v;
        }
    }
    return v;
}

// One block owns POST_COLS whole columns; one thread per (column, level)
// element, up to POST_R elements per thread.  Chain values at k=1 and k=NZ-2
// are exchanged through shared memory for the top/bottom condition.
constexpr int POST_COLS = 8, POST_R = 4, POST_THREADS = 256;  // POST_COLS * NZ <= POST_R * POST_THREADS

__device__ __forceinline__ void post_column(const int mode, const long c, const int nx, const int ny, int &i, int &j,
                                            bool &ok)
{
    ok = true;
    if (mode == COLS_TARGETS) {
        if (c >= 6L * ny) { ok = false; return; }
        const int col = (int)(c / ny);
        j = (int)(c % ny);
        i = col < 3 ? col : nx - 6 + col;
    } else if (mode == COLS_NONTARGETS) {
        if (c >= (long)(nx - 6) * ny) { ok = false; return; }
        i = 3 + (int)(c / ny);
        j = (int)(c % ny);
    } else {
        if (c >= (long)nx * ny) { ok = false; return; }
        i = (int)(c / ny);
        j = (int)(c % ny);
    }
}

template <typename T>
__device__ void post_body(const KParams<T> &p, const KFields<T> &F, int nfields, int4 fl0, int4 fl1, T step, int cols,
                          long bx)
{
    __shared__ T edge[7][POST_COLS][2];
    const int nz = p.nz, sx = p.ny * p.nz, sy = p.nz;
    const int flv[7] = {fl0.x, fl0.y, fl0.z, fl0.w, fl1.x, fl1.y, fl1.z};
    const long c0 = bx * POST_COLS;
    T vals[7][POST_R];
#pragma unroll
    for (int r = 0; r < POST_R; ++r) {
        const int e = threadIdx.x + r * POST_THREADS;
        const int cl = e / nz, k = e - cl * nz;
        int i = 0, j = 0;
        bool ok = false;
        if (cl < POST_COLS) post_column(cols, c0 + cl, p.nx, p.ny, i, j, ok);
        if (!ok) continue;
        // the chain runs at the source column (the column itself, or the
        // column a periodic target copies)
        const int si = cols == COLS_TARGETS ? (i < 3 ? p.nx - 6 + i : 3 + (i - (p.nx - 3))) : i;
        const int c = gix(p.ny, nz, si, j, k);
        const bool inner = si >= 1 && si < p.nx - 1 && j >= 1 && j < p.ny - 1 && k >= 1 && k < nz - 1;
        // sponge strips of this point, in the reference's order (boundaries.cpp:481-498)
        const bool kin = k >= 1;
        const bool hE = kin && !p.periodic && j >= 1 && si >= p.eb && si < p.ee;
        const bool hW = kin && !p.periodic && j >= 1 && si >= p.wb && si < p.we;
        const bool hS = kin && si >= 1 && j >= p.sb && j < p.se;
        const bool hN = kin && si >= 1 && j >= p.nb && j < p.ne;
        const T cE = hE ? p.ce[si - p.eb] : T(0), cW = hW ? p.cw[si - p.wb] : T(0);
        const T cS = hS ? p.cs[j - p.sb] : T(0), cN = hN ? p.cn[j - p.nb] : T(0);
        T dpx = T(0), dpy = T(0), dpz = T(0);
        if (inner && ((flv[FU] | flv[FV] | flv[FW]) & PF_PROJECT)) {
            const T pc = F.pi[c];
            dpx = pc - F.pi[c - sx];
            dpy = pc - F.pi[c - sy];
            dpz = pc - F.pi[c - 1];
        }
#pragma unroll
        for (int f = 0; f < 7; ++f) {
            const int flags = flv[f];
            if (f >= nfields || !flags) continue;
            T v = F.P[f][c];
            if (flags & PF_ZERO) {  // zero_moisture, microphysics.cpp:675-700
                if (f == FQC || f == FQR) {
                    if (v < 0) v = 0;
                } else if (f == FQV && inner) {
                    const T qbar = F.bar[4][c];
                    if (v + qbar + p.qb[k] < 0) v = -(qbar + p.qb[k]);
                }
            }
            if ((flags & PF_PROJECT) && inner) {  // solver.cpp:123-135
                if (f == FU) v = v - step * (p.dtx * dpx);
                else if (f == FV) v = v - step * (p.dty * dpy);
                else if (f == FW && k >= 2) v = v - step * ((p.dtz * p.mw[k]) * dpz);
            }
            if (flags & PF_SPONGE) {
                if (hE) v = v - cE * v;
                if (hW) v = v - cW * v;
                if (hS) v = v - cS * v;
                if (hN) v = v - cN * v;
            }
            vals[f][r] = v;
            if (k == 1) edge[f][cl][0] = v;
            if (k == nz - 2) edge[f][cl][1] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < POST_R; ++r) {
        const int e = threadIdx.x + r * POST_THREADS;
        const int cl = e / nz, k = e - cl * nz;
        int i = 0, j = 0;
        bool ok = false;
        if (cl < POST_COLS) post_column(cols, c0 + cl, p.nx, p.ny, i, j, ok);
        if (!ok) continue;
        const int c = gix(p.ny, nz, i, j, k);
        const bool vbc = i >= 1 && j >= 1;
        const bool ray = i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1 && k >= p.raylevel;
#pragma unroll
        for (int f = 0; f < 7; ++f) {
            const int flags = flv[f];
            if (f >= nfields || !flags) continue;
            T v = vals[f][r];
            if ((flags & PF_VBC) && vbc) {  // boundaries.cpp:304-326
                if (f == FW) {
                    if (k == 0 || k == 1 || k == nz - 1) v = T(0);
                } else {
                    if (k == 0) v = edge[f][cl][0];
                    if (k == nz - 1) v = edge[f][cl][1];
                }
            }
            if ((flags & PF_RAYLEIGH) && f <= FTH && ray) {  // damping.cpp:1148-1177
                const T cr = (f == FW) ? p.ray_w[k] : p.ray_u[k];
                v = v - cr * v;
            }
            F.P[f][c] = v;
            if (flags & PF_WRITE_M) F.M[f][c] = v;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(POST_THREADS) k_post(KParams<T> p, KFields<T> F, int nfields, int4 fl0, int4 fl1,
                                                       T step, int cols)
{
    post_body(p, F, nfields, fl0, fl1, step, cols, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Kessler warm rain, pointwise (kessler.cpp:25-183).  kessler_point is written
// once for a scalar type S: the real type T (the step) or Dual<T,N> (the
// linearisation, which differentiates exactly this arithmetic with the branch
// decisions of the trajectory).  The k=1 thread of each column then adds the
// Eulerian precipitation (precip_rate, microphysics.cpp:143-160) when
// rain_fallout == 1.
// ---------------------------------------------------------------------------
template <typename T, int N>
struct Dual {
    T v, d[N];
};
template <typename T> __device__ __forceinline__ T val(T x) { return x; }
template <typename T, int N> __device__ __forceinline__ T val(const Dual<T, N> &x) { return x.v; }

#define DUAL_T template <typename T, int N> __device__ __forceinline__ Dual<T, N>
DUAL_T operator+(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a.v + b.v;
    for (int q = 0; q < N; q++) r.d[q] = a.d[q] + b.d[q];
    return r;
}
DUAL_T operator-(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a.v - b.v;
    for (int q = 0; q < N; q++) r.d[q] = a.d[q] - b.d[q];
    return r;
}
DUAL_T operator*(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a.v * b.v;
    for (int q = 0; q < N; q++) r.d[q] = a.d[q] * b.v + a.v * b.d[q];
    return r;
}
DUAL_T operator/(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a.v / b.v;
    for (int q = 0; q < N; q++) r.d[q] = (a.d[q] - r.v * b.d[q]) / b.v;
    return r;
}
DUAL_T operator+(const Dual<T, N> &a, T b)
{
    Dual<T, N> r = a;
    r.v = a.v + b;
    return r;
}
DUAL_T operator+(T a, const Dual<T, N> &b) { return b + a; }
DUAL_T operator-(const Dual<T, N> &a, T b)
{
    Dual<T, N> r = a;
    r.v = a.v - b;
    return r;
}
DUAL_T operator-(T a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a - b.v;
    for (int q = 0; q < N; q++) r.d[q] = -b.d[q];
    return r;
}
DUAL_T operator*(const Dual<T, N> &a, T b)
{
    Dual<T, N> r;
    r.v = a.v * b;
    for (int q = 0; q < N; q++) r.d[q] = a.d[q] * b;
    return r;
}
DUAL_T operator*(T a, const Dual<T, N> &b) { return b * a; }
DUAL_T operator/(const Dual<T, N> &a, T b)
{
    Dual<T, N> r;
    r.v = a.v / b;
    for (int q = 0; q < N; q++) r.d[q] = a.d[q] / b;
    return r;
}
DUAL_T operator/(T a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a / b.v;
    for (int q = 0; q < N; q++) r.d[q] = -r.v * b.d[q] / b.v;
    return r;
}
DUAL_T kpow(const Dual<T, N> &x, T e)  // x > 0 wherever it is used
{
    Dual<T, N> r;
    r.v = pow(x.v, e);
    const T g = e * r.v / x.v;
    for (int q = 0; q < N; q++) r.d[q] = g * x.d[q];
    return r;
}
DUAL_T kexp(const Dual<T, N> &x)
{
    Dual<T, N> r;
    r.v = exp(x.v);
    for (int q = 0; q < N; q++) r.d[q] = r.v * x.d[q];
    return r;
}
DUAL_T kmin(const Dual<T, N> &a, const Dual<T, N> &b) { return b.v < a.v ? b : a; }
DUAL_T kmax(const Dual<T, N> &a, const Dual<T, N> &b) { return b.v > a.v ? b : a; }
DUAL_T kneg(const Dual<T, N> &a)
{
    Dual<T, N> r;
    r.v = -a.v;
    for (int q = 0; q < N; q++) r.d[q] = -a.d[q];
    return r;
}
DUAL_T kconst(T c)
{
    Dual<T, N> r;
    r.v = c;
    for (int q = 0; q < N; q++) r.d[q] = T(0);
    return r;
}
#undef DUAL_T
template <typename T> __device__ __forceinline__ T kpow(T x, T e) { return pow(x, e); }
template <typename T> __device__ __forceinline__ T kexp(T x) { return exp(x); }
template <typename T> __device__ __forceinline__ T kmin(T a, T b) { return fmin(a, b); }
template <typename T> __device__ __forceinline__ T kmax(T a, T b) { return fmax(a, b); }
template <typename T> __device__ __forceinline__ T kneg(T a) { return -a; }

// the column values Kessler reads at a point
template <typename T>
struct KesPoint {
    T thbar, qbar, pbar, tb, qb, tbv, rhou, dt;
    int hyd;  // hydrostatic set: pressure = pi + pbar
};

// run_kessler_microphysics at one point: (thp, qvp, qcp, qrp) updated in
// place from themselves and pi.  Returns true where the reference exits
// (evaporation E > 100, kessler.cpp:83-88).
template <typename S, typename T>
__device__ __forceinline__ bool kessler_point(S &thp, S &qvp, S &qcp, S &qrp, const S &pi, const KesPoint<T> &c,
                                              unsigned char *sat = nullptr)
{
    const T cp = T(1004), p0 = T(100000), Lv = T(2.5e6);
    const T cpRd = T(1004.0 / 287.0);
    const T dt = c.dt, rhou = c.rhou;
    const S zero = thp - thp;  // 0 of the scalar type, derivative 0
    S theta = thp + c.thbar + c.tb;
    S pressure = c.hyd ? pi + c.pbar : pi / (cp * c.tbv) + c.pbar;
    S vapor = qvp + c.qbar + c.qb;
    S temperature = theta * pressure;
    S pd = p0 * kpow(pressure, cpRd);
    S A = zero, B = zero, E = zero, esl, qvsat;
    bool bad = false;
    if (val(qcp) > T(1.0e-3)) A = T(0.001) * (qcp - T(1.0e-3)) * dt;
    if (val(qrp) > T(1.0e-12)) B = rhou * T(2.2) * qcp * kpow(qrp, T(0.875)) * dt;
    if (val(qrp) > T(1.0e-12)) {
        esl = T(611.2) * kexp(T(17.67) * (temperature - T(273.15)) / (temperature - T(29.65)));
        qvsat = T(0.62197) * esl / (pd - esl);
        S cvent = T(1.6) + T(30.3922) * kpow(rhou * qrp, T(0.2046));
        E = (T(1.0) / rhou) *
            (((T(1.0) - vapor / qvsat) * cvent * kpow(rhou * qrp, T(0.525))) / (T(2.03e4) + T(9.58e6) / (pd * qvsat))) *
            dt;
        E = kmin(qrp, E);
        E = kmax(E, zero);
        bad = val(E) > T(100);
    }
    qvp = qvp + E;
    S total_convert = kmin(A + B, qcp);
    qcp = qcp - total_convert;
    qrp = qrp + (total_convert - E);
    S de = (Lv / (cp * pressure)) * E;
    thp = thp - de;
    theta = thp + c.thbar + c.tb;
    vapor = qvp + c.qbar + c.qb;
    temperature = theta * pressure;
    esl = T(611.2) * kexp(T(17.67) * (temperature - T(273.15)) / (temperature - T(29.65)));
    qvsat = T(0.62197) * esl / (pd - esl);
    const T fcoef = T(17.67 * (273.15 - 29.65) * 2.5e6 / 1004.0);
    S tm = temperature - T(29.65);
    S phi = pd / (pd - esl) * qvsat * fcoef / (tm * tm);
    S C = zero;
    // the saturation record of the turbulence scheme (isSaturated,
    // kessler.cpp:137-163): saturated after condensation, after a partial
    // evaporation of the cloud, or at exact saturation
    unsigned char s_rec;
    if (val(vapor) > val(qvsat)) {
        C = (vapor - qvsat) / (T(1.0) + phi);
        s_rec = 1;
    } else if (val(vapor) < val(qvsat) && val(qcp) > 0) {
        C = kneg(kmin(qcp, (qvsat - vapor) / (T(1.0) + phi)));
        s_rec = -val(C) < val(qcp);
    } else {
        s_rec = val(vapor) == val(qvsat);
    }
    if (sat) *sat = s_rec;
    qcp = qcp + C;
    qvp = qvp - C;
    S dc = (Lv / (cp * pressure)) * C;
    thp = thp + dc;
    return bad;
}

template <typename T>
__device__ __forceinline__ KesPoint<T> kes_point(const KParams<T> &p, const KFields<T> &F, int k, long ix)
{
    KesPoint<T> c;
    c.thbar = p.ubase_kes ? BTAB(BT_THB, k) : F.bar[3][ix];
    c.qbar = p.ubase_kes ? BTAB(BT_QB, k) : F.bar[4][ix];
    c.pbar = p.ubase_kes ? BTAB(BT_PB, k) : F.bar[5][ix];
    c.tb = p.tb[k];
    c.qb = p.qb[k];
    c.tbv = p.tbv[k];
    c.rhou = p.rhou[k];
    c.dt = p.dt;
    c.hyd = p.hydrostatic;
    return c;
}

template <typename T>
__device__ void kessler_body(const KParams<T> &p, const KFields<T> &F, int precip, int *err, long t)
{
    const int nzi = p.nz - 2, nyi = p.ny - 2, nxi = p.nx - 2;
    if (t >= (long)nxi * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 1 + (int)((t / nzi) % nyi);
    const int i = 1 + (int)(t / ((long)nzi * nyi));
    const long ix = gix(p.ny, p.nz, i, j, k);
    T *THP = F.P[FTH], *QVP = F.P[FQV], *QCP = F.P[FQC], *QRP = F.P[FQR];
    T thp = THP[ix], qvp = QVP[ix], qcp = QCP[ix], qrp = QRP[ix];
    const T piv = F.pi[ix];
    if (kessler_point(thp, qvp, qcp, qrp, piv, kes_point(p, F, k, ix), F.sat ? F.sat + ix : nullptr))
        atomicExch(err, 1);
    THP[ix] = thp;
    QVP[ix] = qvp;
    QCP[ix] = qcp;
    QRP[ix] = qrp;
    if (precip && k == 1) {
        const T dt = p.dt;
        const long i0 = ix - 1;
        const double inc = (double)(p.rhow[1] * T(0.5) * (F.vt[i0] + F.vt[ix]) * T(0.5) * (QRP[i0] + qrp) * dt);
        F.accrain[(long)i * p.ny + j] += inc;
    }
}
template <typename T>
__global__ void __launch_bounds__(128) k_kessler(KParams<T> p, KFields<T> F, int precip, int *err)
{
    kessler_body(p, F, precip, err, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

// fall speed over [1,NX-1) x [1,NY-1) from the forecast rain (semi-Lagrangian
// fallout path, kessler.cpp:190)
template <typename T>
__global__ void k_fall_speed(KParams<T> p, KFields<T> F)
{
    const int nyi = p.ny - 2, nxi = p.nx - 2;
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nxi * nyi * p.nz) return;
    const int k = (int)(t % p.nz);
    const int j = 1 + (int)((t / p.nz) % nyi);
    const int i = 1 + (int)(t / ((long)p.nz * nyi));
    const long c = gix(p.ny, p.nz, i, j, k);
    if (k >= 1 && k < p.nz - 1) F.vt[c] = fall_speed_point(p, F.P[FQR][c], k);
    else if (k == 0) F.vt[c] = fall_speed_point(p, F.P[FQR][c + 1], 1);
}

// ---------------------------------------------------------------------------
// semi-Lagrangian PPM fallout: hydrometeor_fallout (microphysics.cpp:210-292),
// piecewise_parabolic_interp (:516-579), calculate_edge_values (:590-637),
// integrate_parabolic (:339-350).  One thread per column.  The reference
// keeps its edge buffer qp_edges between columns and steps and never
// rewrites element NZ-2 of it, so that element carries from one rainy column
// to the next in (i,j) order; pass 1 computes each column's inputs to that
// recurrence, pass 2 (one thread) runs it, pass 3 remaps.
// ---------------------------------------------------------------------------
template <typename T>
__device__ bool ppm_column_setup(const KParams<T> &p, const KFields<T> &F, int i, int j, T *ZA, T *QA)
{
    const int nz = p.nz;
    const T *var = F.P[FQR], *vel = F.vt, *ZW = p.zsw;
    bool has = false;
    for (int k = 1; k < nz; k++)
        if (var[gix(p.ny, nz, i, j, k)] > T(1e-12)) { has = true; break; }
    if (!has) return false;
    T Ve[PPM_MAXZ];
    for (int k = 1; k < nz; k++) Ve[k] = T(0.5) * (vel[gix(p.ny, nz, i, j, k)] + vel[gix(p.ny, nz, i, j, k - 1)]);
    Ve[0] = Ve[1];
    const T DeCFL0 = T(0.05), dt = p.dt;
    for (int k = nz - 2; k >= 0; k--) {
        T dzu = ZW[k + 1] - ZW[k];
        T decfl = (Ve[k + 1] - Ve[k]) * dt / dzu;
        if (decfl >= DeCFL0) Ve[k] = Ve[k + 1] - DeCFL0 * dzu / dt;
    }
    for (int k = 0; k < nz - 1; k++) ZA[k] = ZW[k] - dt * Ve[k];
    ZA[nz - 1] = ZW[nz - 1];
    for (int k = 0; k < nz - 1; k++)
        QA[k] = p.rhou[k] * var[gix(p.ny, nz, i, j, k)] * (ZW[k + 1] - ZW[k]) / (ZA[k + 1] - ZA[k]);
    QA[nz - 1] = T(0);
    return true;
}

template <typename T>
__device__ __forceinline__ T ppm_mono(const T *qin, int k)
{
    T dq = T(0.25) * (qin[k + 1] - qin[k - 1]);
    T dmax = fmax(qin[k + 1], fmax(qin[k], qin[k - 1])) - qin[k];
    T dmin = qin[k] - fmin(qin[k + 1], fmin(qin[k], qin[k - 1]));
    return sgn(dq) * fmin(fabs(dq), fmin(dmax, dmin));
}

template <typename T>
__global__ void k_ppm_prepare(KParams<T> p, KFields<T> F, unsigned char *has, T *topq, T *topm)
{
    const int nyi = p.ny - 2, nxi = p.nx - 2;
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nxi * nyi) return;
    const int j = 1 + (int)(t % nyi), i = 1 + (int)(t / nyi);
    T ZA[PPM_MAXZ], QA[PPM_MAXZ];
    bool h = ppm_column_setup(p, F, i, j, ZA, QA);
    has[t] = h;
    if (h) {
        const int n = p.nz;
        topq[t] = QA[n - 2];
        topm[t] = ppm_mono(QA, n - 2);  // mono[n-2] uses qin[n-1], qin[n-2], qin[n-3]
    }
}

// The edge value that the reference carries from one rainy column to the next
// (microphysics.cpp:616-631): a sequential recurrence over the columns in
// index order, c <- a + sgn(m) min(|2m|, |c - a|), so it stays one chain.
// One warp walks it: the lanes load 32 columns at once (the next 32 are
// loaded while the chain runs), and every lane evaluates the same chain from
// shuffled values, so no step of it waits for memory.  Launch with 32 threads.
template <typename T>
__global__ void k_ppm_carry(long ncol, const unsigned char *has, const T *topq, const T *topm, T *carry_in,
                            T *carry)
{
    if (blockIdx.x) return;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    T c = *carry;
    auto load = [&](long base, bool &h, T &a, T &m) {
        const long t = base + lane;
        h = t < ncol && has[t];
        a = h ? topq[t] : T(0);
        m = h ? topm[t] : T(0);
    };
    bool h;
    T a, m;
    load(0, h, a, m);
    for (long base = 0; base < ncol; base += 32) {
        bool hn = false;
        T an = T(0), mn = T(0);
        if (base + 32 < ncol) load(base + 32, hn, an, mn);
        unsigned mask = __ballot_sync(full, h);
        while (mask) {
            const int l = __ffs(mask) - 1;
            mask &= mask - 1;
            const T al = __shfl_sync(full, a, l), ml = __shfl_sync(full, m, l);
            if (lane == l) carry_in[base + l] = c;
            c = al + sgn(ml) * fmin(fabs(T(2.0) * ml), fabs(c - al));
        }
        h = hn;
        a = an;
        m = mn;
    }
    if (lane == 0) *carry = c;
}

template <typename T>
__device__ T integ_parab(const T *zin, const T *qin, int p_, T zl, T zh, const T *qp, const T *qn)
{
    T t0 = (zl - zin[p_]) / (zin[p_ + 1] - zin[p_]);
    T t1 = (zh - zin[p_]) / (zin[p_ + 1] - zin[p_]);
    T high = (qp[p_] + qn[p_] - T(2.0) * qin[p_]) * t1 * t1 * t1 - (qp[p_] + T(2.0) * qn[p_] - T(3.0) * qin[p_]) * t1 * t1 +
             qn[p_] * t1;
    T low = (qp[p_] + qn[p_] - T(2.0) * qin[p_]) * t0 * t0 * t0 - (qp[p_] + T(2.0) * qn[p_] - T(3.0) * qin[p_]) * t0 * t0 +
            qn[p_] * t0;
    return high - low;
}

template <typename T>
__global__ void k_ppm_remap(KParams<T> p, KFields<T> F, const unsigned char *has, const T *carry_in)
{
    const int nyi = p.ny - 2, nxi = p.nx - 2;
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nxi * nyi || !has[t]) return;
    const int j = 1 + (int)(t % nyi), i = 1 + (int)(t / nyi);
    const int n = p.nz;
    T ZA[PPM_MAXZ], QA[PPM_MAXZ], QD[PPM_MAXZ], qp[PPM_MAXZ], qn[PPM_MAXZ], mono[PPM_MAXZ];
    ppm_column_setup(p, F, i, j, ZA, QA);
    const T *zin = ZA, *qin = QA, *zout = p.zsw;
    for (int k = 0; k < n; k++) QD[k] = T(0);
    int hn = 1;
    T rainfall = T(0);
    for (int jj = 1; jj < n - 2; jj++)
        if (zin[jj] < 0 && zin[jj + 1] < 0) {
            rainfall += qin[jj] * (zin[jj + 1] - zin[jj]);
            hn = jj + 1;
        }
    // calculate_edge_values
    for (int k = 1; k < n - 1; k++) mono[k] = ppm_mono(qin, k);
    mono[0] = mono[1];
    mono[n - 1] = mono[n - 2];
    for (int k = 1; k < n - 1; k++) {
        qn[k] = (qin[k - 1] * (zin[k + 1] - zin[k]) + qin[k] * (zin[k] - zin[k - 1])) / (zin[k + 1] - zin[k - 1]) -
                (mono[k] - mono[k - 1]) / T(3.0);
        qp[k - 1] = qn[k];
    }
    qp[n - 2] = carry_in[t];
    qp[n - 1] = qin[n - 1];
    qp[0] = qin[0];
    qn[n - 1] = qin[n - 1];
    qn[0] = qin[0];
    for (int k = 0; k < n; k++) {
        qn[k] = qin[k] - sgn(mono[k]) * fmin(fabs(T(2.0) * mono[k]), fabs(qn[k] - qin[k]));
        qp[k] = qin[k] + sgn(mono[k]) * fmin(fabs(T(2.0) * mono[k]), fabs(qp[k] - qin[k]));
    }
    if (zin[hn] < 0)
        rainfall += integ_parab(zin, qin, hn, zin[hn], T(0), qp, qn) * -zin[hn] * ((zin[hn + 1] - zin[hn]) / -zin[hn]);
    for (int a = 0; a < n - 1; a++)
        for (int b = 0; b < n - 1; b++) {
            T scale = (zin[b + 1] - zin[b]) / (zout[a + 1] - zout[a]);
            if (zout[a] < zin[b] && zout[a + 1] < zin[b + 1] && zout[a + 1] > zin[b])
                QD[a] = QD[a] + integ_parab(zin, qin, b, zin[b], zout[a + 1], qp, qn) * scale;
            if (zout[a] < zin[b + 1] && zout[a + 1] > zin[b + 1] && zout[a] > zin[b])
                QD[a] = QD[a] + integ_parab(zin, qin, b, zout[a], zin[b + 1], qp, qn) * scale;
            if (zout[a] >= zin[b] && zout[a + 1] <= zin[b + 1])
                QD[a] = QD[a] + integ_parab(zin, qin, b, zout[a], zout[a + 1], qp, qn) * scale;
            if (zout[a] < zin[b] && zout[a + 1] > zin[b + 1])
                QD[a] = QD[a] + integ_parab(zin, qin, b, zin[b], zin[b + 1], qp, qn) * scale;
        }
    F.accrain[(long)i * p.ny + j] += (double)rainfall;
    for (int k = 0; k < n; k++) F.P[FQR][gix(p.ny, n, i, j, k)] = QD[k] * p.one_d_rhou[k];
}

template <typename T>
__global__ void k_fill(T *a, long n, T v)
{
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] = v;
}

template <typename T>
__global__ void k_check_finite(const T *a, long n, int *flag)
{
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; t < n; t += (long)gridDim.x * blockDim.x)
        if (!isfinite(a[t])) { atomicExch(flag, 1); return; }
}

// ---------------------------------------------------------------------------
// Explicit diffusion of the start-of-step fields (apply_explicit_diffusion,
// damping.cpp:1125-1146, with diffusion_{2nd,4th,6th}_var, :769-940) over
// i in [3, NX-3), j in [3, NY-3), k in [1, NZ-1).  Every point's diffusion
// is formed from the old values (the reference's temp_var) and written into a
// second buffer (k_diffuse_into).  The vertical operator of the stretched-grid
// build weights the
// column with the finite-difference weights `dw` (order+1 per level, built
// on the host as init_diffusion_weights does, :158-270).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T dif2(const T *v, long c, long s) { return v[c + s] - T(2.0) * v[c] + v[c - s]; }
template <typename T>
__device__ __forceinline__ T dif4(const T *v, long c, long s)
{
    return v[c - 2 * s] - T(4.0) * v[c - s] + T(6.0) * v[c] - T(4.0) * v[c + s] + v[c + 2 * s];
}
template <typename T>
__device__ __forceinline__ T dif6(const T *v, long c, long s)
{
    return v[c - 3 * s] - T(6.0) * v[c - 2 * s] + T(15.0) * v[c - s] - T(20.0) * v[c] + T(15.0) * v[c + s] -
           T(6.0) * v[c + 2 * s] + v[c + 3 * s];
}

// weighted column sums (diffuse_k_2nd/4th/6th with weights, damping.cpp:556-715)
template <typename T>
__device__ __forceinline__ T wk2(const T *v, long c, const T *w) { return w[0] * v[c - 1] + w[1] * v[c] + w[2] * v[c + 1]; }
template <typename T>
__device__ __forceinline__ T wk4(const T *v, long c, const T *w)
{
    return w[0] * v[c - 2] + w[1] * v[c - 1] + w[2] * v[c] + w[3] * v[c + 1] + w[4] * v[c + 2];
}
template <typename T>
__device__ __forceinline__ T wk6(const T *v, long c, const T *w)
{
    return w[0] * v[c - 3] + w[1] * v[c - 2] + w[2] * v[c - 1] + w[3] * v[c] + w[4] * v[c + 1] + w[5] * v[c + 2] +
           w[6] * v[c + 3];
}

// the diffused fields written whole into a second buffer per field (the
// interior points M + step d, every other point copied), which then takes the
// start-of-step slot's place: one pass instead of the tendency buffer and its
// addition (every tendency is still formed from the old values)
template <typename T>
struct DiffOut {
    T *out[9];
};
template <typename T>
__global__ void __launch_bounds__(256) k_diffuse_into(KParams<T> p, KFields<T> F, DiffOut<T> o, int nf, int order,
                                                      T kh, T kv, const T *dw, T step)
{
    const long per = p.n, tot = per * nf;
    const long sx = (long)p.ny * p.nz, sy = p.nz;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long)gridDim.x * blockDim.x) {
        const int f = (int)(t / per);
        const long c = t - f * per;
        T *out = o.out[f];
        if (!out) continue;  // a field left alone (w of the hydrostatic set)
        const T *v = F.M[f];
        const int k = (int)(c % p.nz), j = (int)((c / p.nz) % p.ny), i = (int)(c / sx);
        if (i < 3 || i >= p.nx - 3 || j < 3 || j >= p.ny - 3 || k < 1 || k >= p.nz - 1) {
            out[c] = v[c];
            continue;
        }
        const int ind = order + 1, nz = p.nz;
        T d;
        if (order == 2) {
            d = kh * dif2(v, c, sx) + kh * dif2(v, c, sy) + kv * wk2(v, c, dw + ind * k);
        } else if (order == 4) {
            if (k == 1 || k == nz - 2)  // both ends with row NZ-2, as damping.cpp:820 and :861 do
                d = -kh * dif4(v, c, sx) - kh * dif4(v, c, sy) + kv * wk2(v, c, dw + ind * (nz - 2));
            else
                d = -kh * dif4(v, c, sx) - kh * dif4(v, c, sy) - kv * wk4(v, c, dw + ind * k);
        } else {
            T z;
            if (k == 1 || k == nz - 2) z = kv * wk2(v, c, dw + ind * k);
            else if (k == 2 || k == nz - 3) z = -kv * wk4(v, c, dw + ind * k);
            else z = kv * wk6(v, c, dw + ind * k);
            d = kh * dif6(v, c, sx) + kh * dif6(v, c, sy) + z;
        }
        out[c] = v[c] + step * d;
    }
}

// ---------------------------------------------------------------------------
// FP64 domain budgets of one rotation slot.  Over the physical cells
// i in [1, NX-1), j in [1, NY-1), k in [1, NZ-1), with the weight
// wk[k] = rhou[k] dx dy dz / mu[k] (density times cell volume), in FP64 for
// either precision of the fields:
//   0 theta', 1 qv, 2 qc, 3 qr (rho-weighted integrals; the flux form of
//   the advection conserves them up to boundary fluxes), 5 the perturbation
//   kinetic energy 0.5 rho (u^2 + v^2 + w^2) at cell points, 7 the mass;
//   6 the accumulated surface rain times dx dy (columns i, j of the same
//   range).  4 (total water, 1 + 2 + 3) is formed on the host.
// Each block writes its GA_NB partial sums; k_budget_sum adds the blocks in
// index order, so the result does not depend on the schedule.
// ---------------------------------------------------------------------------
constexpr int GA_NB = 11;  // GA_NBUDGET
constexpr int BUDGET_BLOCKS = 304;

template <typename T>
__global__ void __launch_bounds__(256) k_budget(int nx, int ny, int nz, const T *u, const T *v, const T *w,
                                                const T *th, const T *qv, const T *qc, const T *qr,
                                                const T *qi, const T *qs, const double *accrain,
                                                const double *accsnow, const double *wk, double dxdy, double *part)
{
    double acc[GA_NB];
#pragma unroll
    for (int b = 0; b < GA_NB; b++) acc[b] = 0.0;
    const long n = (long)nx * ny * nz, stride = (long)gridDim.x * blockDim.x;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        const int k = (int)(t % nz);
        const long ij = t / nz;
        const int j = (int)(ij % ny), i = (int)(ij / ny);
        if (i < 1 || i >= nx - 1 || j < 1 || j >= ny - 1 || k < 1 || k >= nz - 1) continue;
        const double wt = wk[k];
        acc[0] += wt * (double)th[t];
        if (qv) {
            acc[1] += wt * (double)qv[t];
            acc[2] += wt * (double)qc[t];
            acc[3] += wt * (double)qr[t];
        }
        if (qi) {  // the ice scheme's cloud ice and snow
            acc[8] += wt * (double)qi[t];
            acc[9] += wt * (double)qs[t];
        }
        const double uu = u[t], vv = v[t], ww = w[t];
        acc[5] += wt * 0.5 * (uu * uu + vv * vv + ww * ww);
        acc[7] += wt;
    }
    if (accrain) {
        for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < (long)nx * ny; t += stride) {
            const int j = (int)(t % ny), i = (int)(t / ny);
            if (i >= 1 && i < nx - 1 && j >= 1 && j < ny - 1) {
                acc[6] += accrain[t] * dxdy;
                if (accsnow) acc[10] += accsnow[t] * dxdy;
            }
        }
    }
    __shared__ double red[8][GA_NB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int b = 0; b < GA_NB; b++) {
        double x = acc[b];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][b] = x;
    }
    __syncthreads();
    if (threadIdx.x < GA_NB) {
        double x = 0.0;
        for (int wi = 0; wi < (int)(blockDim.x >> 5); wi++) x += red[wi][threadIdx.x];
        part[(long)blockIdx.x * GA_NB + threadIdx.x] = x;
    }
}

static __global__ void k_budget_sum(const double *part, int nblocks, double *out)
{
    if (threadIdx.x < GA_NB) {
        double x = 0.0;
        for (int b = 0; b < nblocks; b++) x += part[(long)b * GA_NB + threadIdx.x];
        out[threadIdx.x] = x;
    }
}

template <typename T>
__global__ void k_convert_in(T *dst, const double *src, long n)
{
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (T)src[t];
}
template <typename T>
__global__ void k_convert_out(double *dst, const T *src, long n)
{
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (double)src[t];
}

}  // namespace ga

// ---------------------------------------------------------------------------
// the linearised model's rescaling every 12 hours of model time
// (driver_serial.cpp:160-166): find_max2 (util.cpp:818-829), the largest
// positive rho-weighted value of v in the forecast slot, then rescale_pert2
// (util.cpp:920-943), x <- (5 x) / max for the current and start-of-step u,
// v, w and theta.  The maximum is order-independent, so blocks combine it
// with an atomic maximum on the bit pattern of a non-negative double (whose
// unsigned order is its numeric order); *out must start at 0.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_lin_vmax(const T *v, const T *rhou, int nz, long n, double *out)
{
    double m = 0.0;
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x) {
        const double r = (double)(v[x] * rhou[(int)(x % nz)]);
        if (r > m) m = r;
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ double wm[8];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmax(m, wm[w]);
        atomicMax((unsigned long long *)out, (unsigned long long)__double_as_longlong(m));
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_lin_rescale(T *u, T *v, T *w, T *th, T *um, T *vm, T *wm, T *thm,
                                                     long n, const double *vmax)
{
    const T mx = (T)*vmax, scale = T(5.0);
    for (long x = (long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x) {
        u[x] = scale * u[x] / mx;
        v[x] = scale * v[x] / mx;
        w[x] = scale * w[x] / mx;
        th[x] = scale * th[x] / mx;
        um[x] = scale * um[x] / mx;
        vm[x] = scale * vm[x] / mx;
        wm[x] = scale * wm[x] / mx;
        thm[x] = scale * thm[x] / mx;
    }
}
