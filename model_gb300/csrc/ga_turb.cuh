// ga_turb.cuh - the turbulence scheme (turbulence.cpp): mixing coefficients
// and the tendencies of the turbulent stress and scalar fluxes, computed once
// per step from the start-of-step fields (calculate_diff_tend, :158-188,
// called at driver_serial.cpp:194), and their addition to the forecast fields
// in every RK stage (apply_velocity/scalar/moisture_diffusion, :233-290).
// Flat ground and an all-ocean surface (the land-sea mask the reference sets
// without a file, :370-375).
//
// The reference sweeps the domain one YZ slab at a time, keeping the previous
// slab's stresses as the "west" ones and carrying each level's vertical flux
// to the level above.  Every one of those carried values is the stress or
// flux of a neighbouring point, so here each point evaluates them directly:
// the tendency kernel is pointwise over the grid and reads its stencils
// through L1, one thread per point with the level index fastest.  The FP64
// build keeps the reference's evaluation order (no contraction), so the
// coefficients and tendencies agree with it to the last bit except where
// pow and exp enter (the saturated Brunt-Vaisala frequency, surface fluxes).
#pragma once
#include "ga_kernels.cuh"

namespace ga {

template <typename T>
struct TurbArgs {
    T *kmix, *khmix;           // Kmix (w levels), KHmix
    T *tend[7];                // u, v, w friction; theta, qv, qc, qr diffusion
    const unsigned char *sat;  // Kessler's saturation record (moist)
    const T *l2, *kvmax;       // vert_mixing_length_squared, vert_mix_Kmax [nz]
    const T *tbw;              // basic-state virtual theta on w levels [nz]
    T kmixh_max, lH;           // horizontal bound and mixing length
    T water_temp, es_water, dp_to_surface;  // ocean surface (SURFACE_HEAT_FLUX)
    int surface_flux;
};

// cs, one_d_Pr (turbulence.cpp:51-58)
template <typename T> struct TurbC {
    static constexpr T cs = T(0.25), one_d_Pr = T(3.0), grav = T(9.8), cp = T(1004), Rd = T(287.0),
                       Lv = T(2.5e6), p0 = T(100000);
};

// ---------------------------------------------------------------------------
// mixing coefficients: get_Kmix (moist, turbulence.cpp:563-731) and
// get_Kmix_dry (:737-835).  KMIX(k) before its clamp depends on the fields
// only; KHMIX(k-1) needs the clamped KMIX(k-1) and the unclamped KMIX(k).  A
// block holds whole columns (x: levels, rounded up to a warp multiple; y:
// columns): each thread forms its level's unclamped coefficient into shared
// memory, then the column's pairs give both arrays.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T turb_raw_kmix(const KParams<T> &p, const KFields<T> &F, const TurbArgs<T> &a, int i,
                                           int j, int k, bool *positive)
{
    typedef TurbC<T> C;
    const long sx = (long)p.ny * p.nz, sy = p.nz;
    const long c = gix(p.ny, p.nz, i, j, k);
    const T *U = F.M[FU], *V = F.M[FV], *W = F.M[FW], *TH = F.M[FTH];
    const T *UB = F.bar[0], *VB = F.bar[1], *WB = F.bar[2], *THB = F.bar[3];
    const T odx = p.one_d_dx, ody = p.one_d_dy, odzw = p.one_d_dz * p.mw[k];
    const T D11 = T(0.50) *
                  (U[c + sx] + U[c + sx - 1] - U[c - sx] - U[c - sx - 1] + UB[c + sx] + UB[c + sx - 1] - UB[c - sx] -
                   UB[c - sx - 1]) *
                  odx;
    const T D22 = T(0.50) *
                  (V[c + sy] + V[c + sy - 1] - V[c - sy] - V[c - sy - 1] + VB[c + sy] + VB[c + sy - 1] - VB[c - sy] -
                   VB[c - sy - 1]) *
                  ody;
    const T D33 = T(1.0) * (W[c + 1] - W[c - 1] + WB[c + 1] - WB[c - 1]) * odzw;
    const T D12 = T(0.5) * ((U[c + sy] + U[c + sy - 1] - U[c - sy] - U[c - sy - 1] + UB[c + sy] + UB[c + sy - 1] -
                             UB[c - sy] - UB[c - sy - 1]) *
                                ody +
                            (V[c + sx] + V[c + sx - 1] - V[c - sx] - V[c - sx - 1] + VB[c + sx] + VB[c + sx - 1] -
                             VB[c - sx] - VB[c - sx - 1]) *
                                odx);
    const T D13 = T(0.5) * ((U[c] + U[c + sx] - U[c - 1] - U[c + sx - 1] + UB[c] + UB[c + sx] - UB[c - 1] -
                             UB[c + sx - 1]) *
                                odzw +
                            (W[c + sx] - W[c - sx] + WB[c + sx] - WB[c - sx]) * odx);
    const T D23 = T(0.5) * ((V[c] + V[c + sy] - V[c - 1] - V[c + sy - 1] + VB[c] + VB[c + sy] - VB[c - 1] -
                             VB[c + sy - 1]) *
                                odzw +
                            (W[c + sy] - W[c - sy] + WB[c + sy] - WB[c - sy]) * ody);
    const T S2 = D11 * D11 + D22 * D22 + D33 * D33 + D12 * D12 + D13 * D13 + D23 * D23;
    T bruntv;
    if (!p.moist) {
        const T hi = (TH[c] + THB[c] + p.tb[k]) * (T(1) + T(0.61) * p.qb[k]);
        const T lo = (TH[c - 1] + THB[c - 1] + p.tb[k - 1]) * (T(1) + T(0.61) * p.qb[k - 1]);
        bruntv = T(2.0) * C::grav / (p.tbv[k] + p.tbv[k - 1]) * (hi - lo) * odzw;
    } else {
        const T *QV = F.M[FQV], *QB = F.bar[4];
        if (!a.sat[c] || !a.sat[c - 1]) {
            const T hi = (TH[c] + THB[c] + p.tb[k]) * (T(1) + T(0.61) * (QV[c] + QB[c] + p.qb[k]));
            const T lo = (TH[c - 1] + THB[c - 1] + p.tb[k - 1]) * (T(1) + T(0.61) * (QV[c - 1] + QB[c - 1] + p.qb[k - 1]));
            bruntv = T(2.0) * C::grav / (p.tbv[k] + p.tbv[k - 1]) * (hi - lo) * odzw;
        } else {
            const T *QC = F.M[FQC], *QR = F.M[FQR], *PB = F.bar[5], *PI = F.pi;
            const T cpRd = T(1004.0 / 287.0);
            T hi = TH[c] + THB[c] + p.tb[k];
            T lo = TH[c - 1] + THB[c - 1] + p.tb[k - 1];
            const T tH = hi * (PB[c] + PI[c] / (C::cp * p.tbv[k]));
            const T tL = lo * (PB[c - 1] + PI[c - 1] / (C::cp * p.tbv[k - 1]));
            const T temp = T(0.5) * (tH + tL);
            const T dQL = QC[c] + QR[c] - QC[c - 1] - QR[c - 1] + QV[c] - QV[c - 1] + QB[c] - QB[c - 1] + p.qb[k] -
                          p.qb[k - 1];
            const T qv = T(0.5) * (QV[c] + QV[c - 1] + QB[c] + QB[c - 1] + p.qb[k] + p.qb[k - 1]);
            const T pdH = C::p0 * kpow(PB[c], cpRd) + PI[c] * p.rhou[k];
            const T pdL = C::p0 * kpow(PB[c - 1], cpRd) + PI[c - 1] * p.rhou[k - 1];
            const T eH = T(611.2) * kexp(T(17.67) * (tH - T(273.15)) / (tH - T(29.65)));
            const T eL = T(611.2) * kexp(T(17.67) * (tL - T(273.15)) / (tL - T(29.65)));
            const T qsH = T(0.62197) * eH / (pdH - eH);
            const T qsL = T(0.62197) * eL / (pdL - eL);
            hi = hi * (T(1) + C::Lv * qsH / (C::cp * tH));
            lo = lo * (T(1) + C::Lv * qsL / (C::cp * tL));
            const T A = (C::grav / a.tbw[k]) * (T(1.0) + C::Lv * qv / (C::Rd * temp)) /
                        (T(1.0) + T(0.622) * C::Lv * C::Lv * qv / (C::cp * C::Rd * temp * temp));
            bruntv = (A * (hi - lo) - C::grav * dQL) * odzw;
        }
    }
    const T arg = S2 - C::one_d_Pr * bruntv;
    *positive = arg > T(0);
    return *positive ? a.l2[k] * C::cs * C::cs * sqrt(arg) : T(0);
}

template <typename T>
__global__ void __launch_bounds__(256) k_turb_kmix(KParams<T> p, KFields<T> F, TurbArgs<T> a)
{
    extern __shared__ unsigned char turb_smem[];
    const int kx = blockDim.x;
    T *raw = (T *)turb_smem;  // [columns][kx]
    unsigned char *pos = (unsigned char *)(raw + (size_t)blockDim.y * kx);
    const int k = threadIdx.x, cy = threadIdx.y;
    const int nyi = p.ny - 2;
    const long col = (long)blockIdx.x * blockDim.y + cy;
    const bool colok = col < (long)(p.nx - 2) * nyi;
    const int i = colok ? 1 + (int)(col / nyi) : 1, j = colok ? 1 + (int)(col % nyi) : 1;
    bool ps = false;
    T r = T(0);
    if (colok && k >= 2 && k < p.nz - 1) r = turb_raw_kmix(p, F, a, i, j, k, &ps);
    raw[cy * kx + k] = r;
    pos[cy * kx + k] = ps;
    __syncthreads();
    if (!colok || k < 1 || k >= p.nz) return;
    const long c = gix(p.ny, p.nz, i, j, k);
    if (k == 1 || k == p.nz - 1) {  // zero at the ground and the top (:580-581)
        a.kmix[c] = T(0);
        return;
    }
    T km1 = T(0);  // KMIX(k-1) as the level below left it
    if (k - 1 >= 2 && pos[cy * kx + k - 1]) {
        const T rr = raw[cy * kx + k - 1];
        km1 = rr > a.kvmax[k - 1] ? a.kvmax[k - 1] : rr;
    }
    T kh;
    if (ps) {
        kh = T(0.5) * (km1 / a.l2[k - 1] + r / a.l2[k]) * a.lH * a.lH;
        a.kmix[c] = r > a.kvmax[k] ? a.kvmax[k] : r;
        if (kh > a.kmixh_max) kh = a.kmixh_max;
    } else {
        a.kmix[c] = T(0);
        kh = T(0) + T(0.5) * km1 / a.l2[k - 1] * a.lH * a.lH;
    }
    a.khmix[c - 1] = kh;
}

// ---------------------------------------------------------------------------
// stress and flux divergences: turbulent_diffusion_velocity (:839-1022),
// turbulent_diffusion_scalars (:1027-1183) and _theta (:1190-1276)
// ---------------------------------------------------------------------------
// the deformation rates of the start-of-step velocity (:918-932); the
// vertical ones are zero at level 0, where the reference never sets them
template <typename T>
struct TurbTau {
    const T *U, *V, *W, *mu, *mw;
    long sx, sy;
    T odx, ody, odz;
    __device__ __forceinline__ T t11(long c) const { return T(2.0) * (U[c + sx] - U[c]) * odx; }
    __device__ __forceinline__ T t22(long c) const { return T(2.0) * (V[c + sy] - V[c]) * ody; }
    __device__ __forceinline__ T t33(long c, int k) const
    {
        return k == 0 ? T(0) : T(2.0) * (W[c + 1] - W[c]) * (odz * mu[k]);
    }
    __device__ __forceinline__ T t13(long c, int k) const
    {
        return k == 0 ? T(0) : (W[c + sx + 1] - W[c + 1]) * odx + (U[c + sx + 1] - U[c + sx]) * (odz * mw[k + 1]);
    }
    __device__ __forceinline__ T t23(long c, int k) const
    {
        return k == 0 ? T(0) : (W[c + sy + 1] - W[c + 1]) * ody + (V[c + sy + 1] - V[c + sy]) * (odz * mw[k + 1]);
    }
    __device__ __forceinline__ T t12(long c) const
    {
        return (U[c + sx + sy] - U[c + sx]) * ody + (V[c + sx + sy] - V[c + sy]) * odx;
    }
};

// flux divergence of one scalar (:1116-1173) with the vertical flux tau_l
// into the bottom face
template <typename T>
__device__ __forceinline__ T turb_scalar(const KParams<T> &p, const TurbArgs<T> &a, const T *q, long c, int k,
                                         long sx, long sy, T tau_l)
{
    const T P = TurbC<T>::one_d_Pr;
    const T odx = p.one_d_dx, ody = p.one_d_dy;
    const T *KM = a.kmix, *KH = a.khmix;
    const T th = -P * KM[c + 1] * (q[c + 1] - q[c]) * (p.one_d_dz * p.mw[k + 1]);
    T KHh = T(0.5) * (P * KH[c + sy] + P * KH[c]);
    T KLl = T(0.5) * (P * KH[c] + P * KH[c - sy]);
    const T t22h = -KHh * (q[c + sy] - q[c]) * ody;
    const T t22l = -KLl * (q[c] - q[c - sy]) * ody;
    KHh = T(0.5) * (P * KH[c + sx] + P * KH[c]);
    KLl = T(0.5) * (P * KH[c] + P * KH[c - sx]);
    const T t11h = -KHh * (q[c + sx] - q[c]) * odx;
    const T t11l = -KLl * (q[c] - q[c - sx]) * odx;
    return -((t11h - t11l) * odx + (t22h - t22l) * ody + (th - tau_l) * (p.one_d_dz * p.mu[k]));
}

// the vertical flux through the bottom face of level k > 1: the top flux of
// level k-1
template <typename T>
__device__ __forceinline__ T turb_flux_below(const KParams<T> &p, const TurbArgs<T> &a, const T *q, long c, int k)
{
    return -TurbC<T>::one_d_Pr * a.kmix[c] * (q[c] - q[c - 1]) * (p.one_d_dz * p.mw[k]);
}

template <typename T>
__global__ void __launch_bounds__(256) k_turb_tend(KParams<T> p, KFields<T> F, TurbArgs<T> a)
{
    const int nzi = p.nz - 2, nyi = p.ny - 2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)(p.nx - 2) * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 1 + (int)((t / nzi) % nyi);
    const int i = 1 + (int)(t / ((long)nzi * nyi));
    const long sx = (long)p.ny * p.nz, sy = p.nz;
    const long c = gix(p.ny, p.nz, i, j, k);
    const T *KM = a.kmix, *KH = a.khmix;
    const T odx = p.one_d_dx, ody = p.one_d_dy;
    const T odz = p.one_d_dz * p.mu[k], odzw = p.one_d_dz * p.mw[k];
    TurbTau<T> tau{F.M[FU], F.M[FV], F.M[FW], p.mu, p.mw, sx, sy, odx, ody, p.one_d_dz};
    const long c1 = c - (k - 1);  // level 1 of this column

    // ---- momentum ----
    const T uK11H_h = KH[c];
    const T uK11H_l = KH[c - sx];
    const T uK12H_h = T(0.25) * (KH[c] + KH[c - sx] + KH[c - sx + sy] + KH[c + sy]);
    const T uK12H_l = T(0.25) * (KH[c - sy] + KH[c - sx - sy] + KH[c - sx] + KH[c]);
    const T uK13V_h = T(0.50) * (KM[c + 1] + KM[c - sx + 1]);
    const T vK12H_h = T(0.25) * (KH[c - sy] + KH[c] + KH[c + sx - sy] + KH[c + sx]);
    const T vK12H_l = uK12H_l;
    const T vK22H_h = KH[c];
    const T vK22H_l = KH[c - sy];
    const T vK23V_h = T(0.5) * (KM[c + 1] + KM[c - sy + 1]);
    const T wK13H_h = T(0.25) * (KH[c] + KH[c - 1] + KH[c + sx] + KH[c + sx - 1]);
    const T wK13H_l = T(0.25) * (KH[c] + KH[c - 1] + KH[c - sx] + KH[c - sx - 1]);
    const T wK23H_h = T(0.25) * (KH[c] + KH[c - 1] + KH[c + sy] + KH[c + sy - 1]);
    const T wK23H_l = T(0.25) * (KH[c] + KH[c - 1] + KH[c - sy] + KH[c - sy - 1]);
    const T wK33V_h = T(0.50) * (KM[c] + KM[c + 1]);
    const T wK33V_l = T(0.50) * (KM[c] + KM[c - 1]);
    T tau_u_zl, tau_v_zl;
    if (k == 1) {  // ocean surface stress (:899-905)
        const T u = F.M[FU][c1], v = F.M[FV][c1], ub = F.bar[0][c1], vb = F.bar[1][c1];
        const T ws = sqrt((u + ub) * (u + ub) + (v + vb) * (v + vb));
        const T wsb = sqrt(ub * ub + vb * vb);
        const T drag = (T(1.1e-3) + T(4.0e-5) * ws);
        tau_u_zl = drag * (ws * u + (ws - wsb) * ub);
        tau_v_zl = drag * (ws * v + (ws - wsb) * vb);
    } else {  // the stress the level below passed up (:1000-1001)
        tau_u_zl = (T(0.50) * (KM[c] + KM[c - sx])) * tau.t13(c - sx - 1, k - 1);
        tau_v_zl = (T(0.5) * (KM[c] + KM[c - sy])) * tau.t23(c - sy - 1, k - 1);
    }
    const T t13w = tau.t13(c - sx, k), t23s = tau.t23(c - sy, k);
    a.tend[0][c] = (uK11H_h * tau.t11(c) - uK11H_l * tau.t11(c - sx)) * odx +
                   (uK12H_h * tau.t12(c - sx) - uK12H_l * tau.t12(c - sx - sy)) * ody + (uK13V_h * t13w - tau_u_zl) * odz;
    a.tend[1][c] = (vK12H_h * tau.t12(c - sy) - vK12H_l * tau.t12(c - sx - sy)) * odx +
                   (vK22H_h * tau.t22(c) - vK22H_l * tau.t22(c - sy)) * ody + (vK23V_h * t23s - tau_v_zl) * odz;
    a.tend[2][c] = (wK13H_h * tau.t13(c - 1, k - 1) - wK13H_l * tau.t13(c - sx - 1, k - 1)) * odx +
                   (wK23H_h * tau.t23(c - 1, k - 1) - wK23H_l * tau.t23(c - sy - 1, k - 1)) * ody +
                   (wK33V_h * tau.t33(c, k) - wK33V_l * tau.t33(c - 1, k - 1)) * odzw;

    // ---- scalars ----
    const int nf = p.moist ? 4 : 1;
    T tl[4] = {T(0), T(0), T(0), T(0)};  // theta, qv, qc, qr fluxes into the bottom face
    if (k == 1) {
        if (p.moist && a.surface_flux) {  // ocean heat and vapour fluxes (:1083-1104)
            typedef TurbC<T> C;
            const T u = F.M[FU][c1], v = F.M[FV][c1], ub = F.bar[0][c1], vb = F.bar[1][c1];
            const T ws = sqrt((u + ub) * (u + ub) + (v + vb) * (v + vb));
            const T wsb = sqrt(ub * ub + vb * vb);
            const T drag = (T(1.1e-3) + T(4.0e-5) * ws) * T(1.0) * T(1.0);
            const T PB = F.bar[5][c1], PI = F.pi[c1];
            const T pressure = C::p0 * kpow(PB + a.dp_to_surface, T(1004.0 / 287.0)) + PI * p.rhou[1];
            const T pisfc = PB + PI / (C::cp * p.tbv[1]) + a.dp_to_surface;
            const T qvs = T(0.62197) * a.es_water / (pressure - a.es_water);
            const T tsb = (F.bar[3][c1] + p.tb[1]) * pisfc;
            const T tsp = F.M[FTH][c1] * pisfc;
            tl[1] = drag * ((ws - wsb) * (qvs - F.bar[4][c1] - p.qb[1]) - ws * F.M[FQV][c1]);
            tl[0] = drag * ((ws - wsb) * (a.water_temp - tsb) - ws * tsp);
        }
    } else {
        for (int n = 0; n < nf; n++) tl[n] = turb_flux_below(p, a, F.M[FTH + n], c, k);
    }
    for (int n = 0; n < nf; n++) a.tend[3 + n][c] = turb_scalar(p, a, F.M[FTH + n], c, k, sx, sy, tl[n]);
}

// The same tendencies by tiles: a block owns TI x TJ columns and every
// level.  Phase 1 evaluates each deformation-rate component once on the
// tile's columns and the column row and line west and south of them into
// shared memory; phase 2 forms each point's stress divergence from those (the
// pointwise kernel evaluates every component at each point that uses it,
// about eighteen evaluations per point against six here) and its scalar flux
// divergences as k_turb_tend does.  The arithmetic is k_turb_tend's.
constexpr int TT_TI = 4, TT_TJ = 4;

__host__ __device__ constexpr size_t turb_tile_smem(int nz, size_t tsize)
{
    return 6 * (size_t)(TT_TI + 1) * (TT_TJ + 1) * nz * tsize;
}

template <typename T>
__global__ void __launch_bounds__(256) k_turb_tend_tile(KParams<T> p, KFields<T> F, TurbArgs<T> a)
{
    extern __shared__ unsigned char tt_smem[];
    constexpr int RA = TT_TI + 1, RB = TT_TJ + 1;
    const int nz = p.nz;
    T *S = (T *)tt_smem;  // [6][RA][RB][nz]: t11, t22, t33, t13, t23, t12
    const long rs = (long)RA * RB * nz;
    const int i0 = 1 + blockIdx.x * TT_TI, j0 = 1 + blockIdx.y * TT_TJ;
    const int ti = min(TT_TI, p.nx - 1 - i0), tj = min(TT_TJ, p.ny - 1 - j0);
    const long sx = (long)p.ny * nz, sy = nz;
    const T odx = p.one_d_dx, ody = p.one_d_dy;
    TurbTau<T> tau{F.M[FU], F.M[FV], F.M[FW], p.mu, p.mw, sx, sy, odx, ody, p.one_d_dz};
    for (int w = threadIdx.x; w < RA * RB * (nz - 1); w += blockDim.x) {
        const int k = w % (nz - 1), r = w / (nz - 1), bb = r % RB, aa = r / RB;
        if (aa > ti || bb > tj) continue;
        const long c = gix(p.ny, nz, i0 - 1 + aa, j0 - 1 + bb, k);
        const long o = (long)r * nz + k;
        S[o] = tau.t11(c);
        S[rs + o] = tau.t22(c);
        S[2 * rs + o] = tau.t33(c, k);
        S[3 * rs + o] = tau.t13(c, k);
        S[4 * rs + o] = tau.t23(c, k);
        S[5 * rs + o] = tau.t12(c);
    }
    __syncthreads();
    const T *S11 = S, *S22 = S + rs, *S33 = S + 2 * rs, *S13 = S + 3 * rs, *S23 = S + 4 * rs, *S12 = S + 5 * rs;
    const T *KM = a.kmix, *KH = a.khmix;
    for (int w = threadIdx.x; w < TT_TI * TT_TJ * (nz - 2); w += blockDim.x) {
        const int k = 1 + w % (nz - 2), r = w / (nz - 2), b = r % TT_TJ, aa = r / TT_TJ;
        if (aa >= ti || b >= tj) continue;
        const int i = i0 + aa, j = j0 + b;
        const long c = gix(p.ny, nz, i, j, k);
        const long oc = (long)((aa + 1) * RB + b + 1) * nz, ow = (long)(aa * RB + b + 1) * nz;
        const long os = (long)((aa + 1) * RB + b) * nz, osw = (long)(aa * RB + b) * nz;
        const T odz = p.one_d_dz * p.mu[k], odzw = p.one_d_dz * p.mw[k];
        const long c1 = c - (k - 1);
        const T uK11H_h = KH[c];
        const T uK11H_l = KH[c - sx];
        const T uK12H_h = T(0.25) * (KH[c] + KH[c - sx] + KH[c - sx + sy] + KH[c + sy]);
        const T uK12H_l = T(0.25) * (KH[c - sy] + KH[c - sx - sy] + KH[c - sx] + KH[c]);
        const T uK13V_h = T(0.50) * (KM[c + 1] + KM[c - sx + 1]);
        const T vK12H_h = T(0.25) * (KH[c - sy] + KH[c] + KH[c + sx - sy] + KH[c + sx]);
        const T vK12H_l = uK12H_l;
        const T vK22H_h = KH[c];
        const T vK22H_l = KH[c - sy];
        const T vK23V_h = T(0.5) * (KM[c + 1] + KM[c - sy + 1]);
        const T wK13H_h = T(0.25) * (KH[c] + KH[c - 1] + KH[c + sx] + KH[c + sx - 1]);
        const T wK13H_l = T(0.25) * (KH[c] + KH[c - 1] + KH[c - sx] + KH[c - sx - 1]);
        const T wK23H_h = T(0.25) * (KH[c] + KH[c - 1] + KH[c + sy] + KH[c + sy - 1]);
        const T wK23H_l = T(0.25) * (KH[c] + KH[c - 1] + KH[c - sy] + KH[c - sy - 1]);
        const T wK33V_h = T(0.50) * (KM[c] + KM[c + 1]);
        const T wK33V_l = T(0.50) * (KM[c] + KM[c - 1]);
        T tau_u_zl, tau_v_zl;
        if (k == 1) {  // ocean surface stress (:899-905)
            const T u = F.M[FU][c1], v = F.M[FV][c1], ub = F.bar[0][c1], vb = F.bar[1][c1];
            const T ws = sqrt((u + ub) * (u + ub) + (v + vb) * (v + vb));
            const T wsb = sqrt(ub * ub + vb * vb);
            const T drag = (T(1.1e-3) + T(4.0e-5) * ws);
            tau_u_zl = drag * (ws * u + (ws - wsb) * ub);
            tau_v_zl = drag * (ws * v + (ws - wsb) * vb);
        } else {
            tau_u_zl = (T(0.50) * (KM[c] + KM[c - sx])) * S13[ow + k - 1];
            tau_v_zl = (T(0.5) * (KM[c] + KM[c - sy])) * S23[os + k - 1];
        }
        const T t13w = S13[ow + k], t23s = S23[os + k];
        a.tend[0][c] = (uK11H_h * S11[oc + k] - uK11H_l * S11[ow + k]) * odx +
                       (uK12H_h * S12[ow + k] - uK12H_l * S12[osw + k]) * ody + (uK13V_h * t13w - tau_u_zl) * odz;
        a.tend[1][c] = (vK12H_h * S12[os + k] - vK12H_l * S12[osw + k]) * odx +
                       (vK22H_h * S22[oc + k] - vK22H_l * S22[os + k]) * ody + (vK23V_h * t23s - tau_v_zl) * odz;
        a.tend[2][c] = (wK13H_h * S13[oc + k - 1] - wK13H_l * S13[ow + k - 1]) * odx +
                       (wK23H_h * S23[oc + k - 1] - wK23H_l * S23[os + k - 1]) * ody +
                       (wK33V_h * S33[oc + k] - wK33V_l * S33[oc + k - 1]) * odzw;
        const int nf = p.moist ? 4 : 1;
        T tl[4] = {T(0), T(0), T(0), T(0)};
        if (k == 1) {
            if (p.moist && a.surface_flux) {  // ocean heat and vapour fluxes (:1083-1104)
                typedef TurbC<T> C;
                const T u = F.M[FU][c1], v = F.M[FV][c1], ub = F.bar[0][c1], vb = F.bar[1][c1];
                const T ws = sqrt((u + ub) * (u + ub) + (v + vb) * (v + vb));
                const T wsb = sqrt(ub * ub + vb * vb);
                const T drag = (T(1.1e-3) + T(4.0e-5) * ws) * T(1.0) * T(1.0);
                const T PB = F.bar[5][c1], PI = F.pi[c1];
                const T pressure = C::p0 * kpow(PB + a.dp_to_surface, T(1004.0 / 287.0)) + PI * p.rhou[1];
                const T pisfc = PB + PI / (C::cp * p.tbv[1]) + a.dp_to_surface;
                const T qvs = T(0.62197) * a.es_water / (pressure - a.es_water);
                const T tsb = (F.bar[3][c1] + p.tb[1]) * pisfc;
                const T tsp = F.M[FTH][c1] * pisfc;
                tl[1] = drag * ((ws - wsb) * (qvs - F.bar[4][c1] - p.qb[1]) - ws * F.M[FQV][c1]);
                tl[0] = drag * ((ws - wsb) * (a.water_temp - tsb) - ws * tsp);
            }
        } else {
            for (int n = 0; n < nf; n++) tl[n] = turb_flux_below(p, a, F.M[FTH + n], c, k);
        }
        for (int n = 0; n < nf; n++) a.tend[3 + n][c] = turb_scalar(p, a, F.M[FTH + n], c, k, sx, sy, tl[n]);
    }
}

// ---------------------------------------------------------------------------
// the tendencies added to the forecast fields in an RK stage: velocity
// (apply_velocity_diffusion, :233-256, over [3,N-3): u and v from level 1, w
// from level 2), theta (apply_scalar_diffusion, :263-273) and moisture
// (apply_moisture_diffusion, :278-291) over [1,N-1)
// ---------------------------------------------------------------------------
enum { TA_VEL = 1, TA_TH = 2, TA_Q = 4 };

template <typename T>
__global__ void __launch_bounds__(256) k_turb_apply(KParams<T> p, KFields<T> F, TurbArgs<T> a, int what, T deltaT,
                                                    T step)
{
    const int nzi = p.nz - 2, nyi = p.ny - 2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)(p.nx - 2) * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 1 + (int)((t / nzi) % nyi);
    const int i = 1 + (int)(t / ((long)nzi * nyi));
    const long c = gix(p.ny, p.nz, i, j, k);
    if ((what & TA_VEL) && i >= 3 && i < p.nx - 3 && j >= 3 && j < p.ny - 3) {
        F.P[FU][c] = F.P[FU][c] + a.tend[0][c] * deltaT;
        F.P[FV][c] = F.P[FV][c] + a.tend[1][c] * deltaT;
        if (k >= 2) F.P[FW][c] = F.P[FW][c] + a.tend[2][c] * deltaT;
    }
    if (what & TA_TH) F.P[FTH][c] = F.P[FTH][c] + a.tend[3][c] * step * p.dt;
    if ((what & TA_Q) && p.moist) {
        F.P[FQV][c] = F.P[FQV][c] + a.tend[4][c] * deltaT;
        F.P[FQC][c] = F.P[FQC][c] + a.tend[5][c] * deltaT;
        F.P[FQR][c] = F.P[FQR][c] + a.tend[6][c] * deltaT;
    }
}

}  // namespace ga
