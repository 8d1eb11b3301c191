// Ice microphysics of the reference's microphysics_option 2: the processes of
// Rutledge and Hobbs (1983) with the changes of Hong et al. (2004)
// (run_rutledge_microphysics, rutledge.cpp:150-452), the saturation
// adjustment over water, ice and the mixed phase (saturation_adjustment and
// get_qvsat, :611-820), the fall speeds of rain, snow and cloud ice (:503-600)
// and the advection of snow and ice with them (advect_ice_cell,
// advection.cpp:508-567).
//
// The processes and the adjustment of a point read and write that point only,
// so one thread runs both, then zero_moisture's clipping, and the thread of
// level 1 adds the column's precipitation.  Two couplings between points are
// kept as the reference has them:
//  - the snow intercept N0S is a file-scope variable that every snowy point
//    of a pass rewrites (:197-205) and the snow fall speed reads later
//    (:514); each snowy point records its value and a 32-bit atomic max finds
//    the last snowy point in the reference's (i, j, k) order, whose value a
//    one-thread kernel keeps (deterministic);
//  - the Eulerian ice fall speed is rewritten only where its input exceeds
//    the threshold and keeps its previous value elsewhere (:580-600); the
//    input is the pressure field, which advect_ice_cell passes where the ice
//    field belongs (advection.cpp:514).
#pragma once

#include "ga_kernels.cuh"

namespace ga {

// rutledge.cpp:13-147 and model.h:250-258
struct RutC {
    static constexpr double cp = 1004, Rd = 287.0, p0 = 100000, Lv = 2.5e6, Ls = 2.85e6, Lf = 3.50e5;
    static constexpr double trigpi = 3.14159265358979324;
    static constexpr double tmin = -30 + 273.15, tmax = 0 + 273.15;
    static constexpr double minvar = 1.0e-10;  // minvar_snow, _cice, _rain, _cwat
    static constexpr double N0r = 8e6, ERC = 1, M0 = 1e-12, Rstar = 8.314e3, Mw = 18.016, Ka = 2.43e-2,
                            chi = 2.26e-5, dimax = 500.0e-6, app = 1.139, bexp = 0.11, rhoS = 200, ESC = 1.0,
                            mu_s = 1.718e-5, ap = 3.0e3;
};

// CONVERT_PRESSURE(i,j,k) + PBAR(i,j,k) (rutledge.cpp:18-24)
template <typename T>
__device__ __forceinline__ T ice_pressure(const KParams<T> &p, const KFields<T> &F, long c, int k)
{
    const T pv = F.pi[c];
    return (p.hydrostatic ? pv : pv / (T(RutC::cp) * p.tbv[k])) + F.bar[5][c];
}

// the pressure factor (p0/pd)^0.4 of the rain and snow fall speeds, pd the
// dimensional pressure p0 pressure^(cp/Rd); both speeds evaluate the same
// expression of the same pressure (rutledge.cpp:512-517, 539-545), so one
// evaluation serves both
template <typename T>
__device__ __forceinline__ T rut_p04(T pressure)
{
    const T pd = T(RutC::p0) * pow(pressure, T(RutC::cp / RutC::Rd));
    return pow(T(RutC::p0) / pd, T(0.4));
}
// calculate_rain_fall_speed_rutledge at one point (rutledge.cpp:530-555)
template <typename T>
__device__ __forceinline__ T rut_rain_speed(const KParams<T> &p, T qr, T p04, int k)
{
    if (qr > T(RutC::minvar)) {
        const T lambdaR = sqrt(sqrt((T(RutC::trigpi) * T(1000) * T(RutC::N0r)) / (p.rhou[k] * qr)));
        return p.rfall / (T(6.0) * pow(lambdaR, T(0.8))) * p04;
    }
    return T(0);
}
// calculate_snow_fall_speed_rutledge at one point (:503-520), with the
// intercept the last microphysics pass left
template <typename T>
__device__ __forceinline__ T rut_snow_speed(const KParams<T> &p, T qs, T p04, T n0s, int k)
{
    if (qs > T(RutC::minvar)) {
        const T lambdaS = pow((T(RutC::trigpi) * T(RutC::rhoS) * n0s) / (p.rhou[k] * qs), T(0.25));
        return T(RutC::app) * T(1.15) * pow(lambdaS, -T(RutC::bexp)) * p04;
    }
    return T(0);
}
// calculate_ice_fall_speed_rutledge at one point (:580-600): old where the
// input is at or below the threshold
template <typename T>
__device__ __forceinline__ T rut_ice_speed(const KParams<T> &p, T qi, T old, int k)
{
    if (qi > T(RutC::minvar)) {
        const T rhou = p.rhou[k];
        const T nc = fmin(fmax(T(5.38e7) * pow(rhou * qi, T(0.75)), T(1.0e3)), T(1.0e6));
        const T MI = rhou * fmax(qi, T(0)) / nc;
        const T Dl = fmax(fmin(T(11.9) * sqrt(MI), T(RutC::dimax)), T(1.0e-25));
        return T(1.49e4) * pow(Dl, T(1.31));
    }
    return old;
}

enum { IF_RAIN = 1, IF_SNOW = 2, IF_ICE = 4 };

// The Rutledge fall speeds over columns [i0,i1) x [j0,j1), levels 1..NZ-2,
// with level 0 copied from level 1 (the lower boundary condition of each
// routine).  from_p = 0: from the current rain and snow and, for the ice, the
// pressure (the Eulerian updates of advect_microphysics_cell and
// advect_ice_cell, advection.cpp:456-457, 513-514); from_p = 1: from the
// forecast rain, snow and ice (the semi-Lagrangian fallout, rutledge.cpp:
// 460-464).  One thread per point; the level-1 thread also writes level 0.
template <typename T>
__global__ void k_ice_fall(KParams<T> p, KFields<T> F, int i0, int i1, int j0, int j1, int what, int from_p)
{
    const int nzi = p.nz - 2, nj = j1 - j0;
    const long tot = (long)(i1 - i0) * nj * nzi;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tot) return;
    const int k = 1 + (int)(t % nzi);
    const int j = j0 + (int)((t / nzi) % nj);
    const int i = i0 + (int)(t / ((long)nzi * nj));
    const long c = gix(p.ny, p.nz, i, j, k);
    const T qr = (what & IF_RAIN) ? (from_p ? F.P[FQR] : F.cur[FQR])[c] : T(0);
    const T qs = (what & IF_SNOW) ? (from_p ? F.P[FQS] : F.cur[FQS])[c] : T(0);
    // the pressure factor only where a rain or snow speed needs it
    const T p04 = (qr > T(RutC::minvar) || qs > T(RutC::minvar)) ? rut_p04(ice_pressure(p, F, c, k)) : T(0);
    if (what & IF_RAIN) {
        const T v = rut_rain_speed(p, qr, p04, k);
        F.vt[c] = v;
        if (k == 1) F.vt[c - 1] = v;
    }
    if (what & IF_SNOW) {
        const T v = rut_snow_speed(p, qs, p04, *F.n0s, k);
        F.sts[c] = v;
        if (k == 1) F.sts[c - 1] = v;
    }
    if (what & IF_ICE) {
        const T v = rut_ice_speed(p, from_p ? F.P[FQI][c] : F.pi[c], F.its[c], k);
        F.its[c] = v;
        if (k == 1) F.its[c - 1] = v;
    }
}

// top face of a field with a stored fall speed: interpolate_scalar_with_
// fallspeed (fluxes.cpp:953-1032) with compute_fluxes_scalar_with_fallspeed
// (:699-716), incl. the outflow through the ground at k = 0
template <typename T>
__device__ T fall_top(const KParams<T> &p, const KFields<T> &F, const T *s, const T *fall, int i, int j, int k)
{
    if (k == 0) {
        const long c0 = gix(p.ny, p.nz, i, j, 0);
        T s0 = T(0.5) * (LD(s, c0) + LD(s, c0 + 1));
        return T(-0.5) * (fall[c0 + 1] + fall[c0]) * s0;
    }
    const long a = gix(p.ny, p.nz, i, j, k + 1);
    T wb = LD(F.bar[2], a) + LD(F.cur[FW], a);
    T wf = wb - T(0.5) * (fall[a - 1] + fall[a]);
    T st;
    if (k == 1 || k == p.nz - 2) st = f2k(s, p, i, j, k);
    else st = f3k(s, p, i, j, k, sgn(wf));
    return wf * st;
}

// advect_ice_cell (advection.cpp:508-567): snow and cloud ice at the interior
// points [3,NX-3) x [3,NY-3) x [1,NZ-1), flux form with their fall speeds
template <typename T>
__global__ void __launch_bounds__(128) k_advect_ice(KParams<T> p, KFields<T> F, T step)
{
    const int nzi = p.nz - 2, nyi = p.ny - 6, nxi = p.nx - 6;
    const long tot = (long)nxi * nyi * nzi;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tot) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 3 + (int)((t / nzi) % nyi);
    const int i = 3 + (int)(t / ((long)nzi * nyi));
    const long c = gix(p.ny, p.nz, i, j, k);
    const T DTZ = p.dtz * p.mu[k];
    const int fld[2] = {FQS, FQI};
    const T *fall[2] = {F.sts, F.its};
    for (int n = 0; n < 2; n++) {
        const T *q = F.cur[fld[n]];
        T tend = -p.dtx * (s_east(p, F, q, (const T *)nullptr, i, j, k) -
                           s_east(p, F, q, (const T *)nullptr, i - 1, j, k)) -
                 p.dty * (s_north(p, F, q, (const T *)nullptr, i, j, k) -
                          s_north(p, F, q, (const T *)nullptr, i, j - 1, k)) -
                 DTZ * (p.rhow[k + 1] * fall_top(p, F, q, fall[n], i, j, k) -
                        p.rhow[k] * fall_top(p, F, q, fall[n], i, j, k - 1)) *
                     p.one_d_rhou[k];
        F.P[fld[n]][c] = LD(F.M[fld[n]], c) + step * tend;
    }
}

#define RUT_ESL(t) (T(611.2) * exp(T(17.67) * ((t) - T(273.15)) / ((t) - T(29.65))))      // SAT_VAP_WAT
#define RUT_ESI(t) (T(611.2) * exp(T(21.8745584) * ((t) - T(273.15)) / ((t) - T(7.66))))  // SAT_VAP_ICE
#define RUT_QSAT(e, pr) (T(0.62197) * (e) / ((pr) - (e)))                                // SAT_MIX_RATIO
#define RUT_ALPHA(x) (T(1.0) + ((x) - T(273.15)) / (T(RutC::tmax) - T(RutC::tmin)))

// get_qvsat (rutledge.cpp:611-693); pow(x,2) as x*x, as the reference's
// compiler folds it
template <typename T>
__device__ __forceinline__ T rut_qvsat(T temp, T pd, T &phi, T &phil, T &phii)
{
    const T Lv = T(RutC::Lv), Ls = T(RutC::Ls), cp = T(RutC::cp);
    T qvsat;
    if (temp > T(RutC::tmax)) {
        const T esl = RUT_ESL(temp);
        qvsat = RUT_QSAT(esl, pd);
        const T f = T(17.67) * (T(273.15) - T(29.65)) * Lv / cp, tm = temp - T(29.65);
        phi = phil = phii = pd / (pd - esl) * qvsat * f / (tm * tm);
    } else if (temp < T(RutC::tmin)) {
        const T esl = RUT_ESI(temp);
        qvsat = RUT_QSAT(esl, pd);
        const T f = T(21.8745584) * (T(273.15) - T(7.66)) * Ls / cp, tm = temp - T(7.66);
        phi = phil = phii = pd / (pd - esl) * qvsat * f / (tm * tm);
    } else {
        const T esl = RUT_ESL(temp), esi = RUT_ESI(temp);
        const T qvl_sat = RUT_QSAT(esl, pd), qvi_sat = RUT_QSAT(esi, pd);
        const T fl = T(17.67) * (T(273.15) - T(29.65)) * Lv / cp;
        const T fi = T(21.8745584) * (T(273.15) - T(7.66)) * Ls / cp;
        const T tl = temp - T(29.65), ti = temp - T(7.66);
        phil = pd / (pd - esl) * qvl_sat * fl / (tl * tl);
        phii = pd / (pd - esi) * qvi_sat * fi / (ti * ti);
        qvsat = RUT_ALPHA(temp) * qvl_sat + (T(1.0) - RUT_ALPHA(temp)) * qvi_sat;
        phi = RUT_ALPHA(temp) * phil + (T(1.0) - RUT_ALPHA(temp)) * phii;
    }
    return qvsat;
}

template <typename T>
__device__ __forceinline__ void ice_precip_col(const KParams<T> &p, const KFields<T> &F, int i, int j)
{
    const long c0 = gix(p.ny, p.nz, i, j, 0), c1 = c0 + 1, a = (long)i * p.ny + j;
    const T r = p.rhow[1], dt = p.dt;
    const T *QR = F.P[FQR], *QI = F.P[FQI];
    F.accrain[a] += (double)(r * T(0.5) * (F.vt[c0] + F.vt[c1]) * T(0.5) * (QR[c0] + QR[c1]) * dt);
    F.accsnow[a] += (double)(r * T(0.5) * (F.sts[c0] + F.sts[c1]) * T(0.5) * (QR[c0] + QR[c1]) * dt);
    F.accsnow[a] += (double)(r * T(0.5) * (F.sts[c0] + F.sts[c1]) * T(0.5) * (QI[c0] + QI[c1]) * dt);
}

// The processes (rutledge.cpp:172-436) and the saturation adjustment
// (:716-812) of the point c of the forecast fields, then zero_moisture
// (microphysics.cpp:675-700) of it; over [1,NX-1) x [1,NY-1) x [1,NZ-1).
// The level-1 thread adds the column's Eulerian precipitation (precip_rate of
// rain, of rain at the snow fall speed and of ice at the snow fall speed,
// rutledge.cpp:486-489).  err[0] is set where the reference exits (rain
// evaporation E > 100 or snow melting |psmlt| > 100, :252-258, :370-376).
template <typename T>
__global__ void __launch_bounds__(128) k_rutledge(KParams<T> p, KFields<T> F, int precip, int *err)
{
    const int nzi = p.nz - 2, nyi = p.ny - 2, nxi = p.nx - 2;
    const long tot = (long)nxi * nyi * nzi;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tot) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 1 + (int)((t / nzi) % nyi);
    const int i = 1 + (int)(t / ((long)nzi * nyi));
    const long c = gix(p.ny, p.nz, i, j, k);
    typedef RutC R;
    const T cp = T(R::cp), p0 = T(R::p0), Lv = T(R::Lv), Ls = T(R::Ls), Lf = T(R::Lf);
    const T trigpi = T(R::trigpi), minvar = T(R::minvar), cpRd = T(R::cp / R::Rd);
    const T N0r = T(R::N0r), Ka = T(R::Ka), Mw = T(R::Mw), Rstar = T(R::Rstar), chi = T(R::chi);
    const T app = T(R::app), mu_s = T(R::mu_s), dt = p.dt;
    const T a0 = T(-0.267), a1 = T(5.15e3), a2 = T(-1.0225e6), a3 = T(7.55e7);  // rain fall-speed polynomial
    const T rhou = p.rhou[k], odr = p.one_d_rhou[k];
    T thp = F.P[FTH][c], qvp = F.P[FQV][c], qcp = F.P[FQC][c], qrp = F.P[FQR][c];
    T qip = F.P[FQI][c], qsp = F.P[FQS][c];
    const T thbar = F.bar[3][c], qbar = F.bar[4][c];
    const T pressure = ice_pressure(p, F, c, k);
    const T pd = p0 * pow(pressure, cpRd);
    const T cpp = cp * p.pib[k];
    bool bad = false;
    {
        const T theta = thp + thbar + p.tb[k];
        const T vapor = qvp + qbar + p.qb[k];
        const T temperature = theta * pressure;
        const T esl = RUT_ESL(temperature), esi = RUT_ESI(temperature);
        const T qvl_sat = RUT_QSAT(esl, pd), qvi_sat = RUT_QSAT(esi, pd);
        const T pcond = T(0);
        T lambdaS = T(0), N0S = T(0), var, Ap, Bp, App = T(0), Bpp = T(0);
        if (qsp != T(0)) {
            N0S = fmin(T(2.0e6) * exp(T(0.12) * (T(273.16) - temperature)), T(2.0e8));
            lambdaS = sqrt(sqrt((trigpi * T(R::rhoS) * N0S) / (rhou * qsp)));
            F.n0s_pt[c] = N0S;
            atomicMax(F.n0s_idx, (int)c);
        }
        // rain: autoconversion, accretion, evaporation, freezing
        T A = T(0), B = T(0), E = T(0), prfrz = T(0);
        if (qcp > T(1.0e-3)) A = T(0.001) * (qcp - T(1.0e-3)) * dt;
        if (qrp > minvar) {
            const T lambdaR = pow((trigpi * T(1000) * N0r) / (rhou * qrp), T(0.25));
            B = T(0.25) * trigpi * qcp * T(R::ERC) * N0r * pow(p0 / pd, T(0.4)) * T(2) / pow(lambdaR, T(3)) *
                (a0 + a1 * T(3) / lambdaR + a2 * T(12) / (lambdaR * lambdaR) +
                 a3 * T(60) / (lambdaR * lambdaR * lambdaR)) *
                dt;
            Ap = (Lv / (Ka * temperature)) * ((Lv * Mw) / (Rstar * temperature) - T(1));
            Bp = Rstar * temperature / (chi * Mw * esl);
            var = T(0.78) / (lambdaR * lambdaR) +
                  T(0.31) * sqrt(T(R::ap) * rhou / mu_s) / (lambdaR * lambdaR * lambdaR) * T(2.0) * pow((p0 / pd), T(0.2));
            E = var * T(2) * trigpi * N0r * (vapor / qvl_sat - T(1.0)) / (Ap + Bp) * dt * odr;
            if (temperature < T(273.16)) {
                prfrz = T(20) * trigpi * trigpi * T(100.0) * N0r * (T(1000.0) / rhou) *
                        exp(T(0.66) * (T(273.16) - temperature) - T(1)) /
                        (lambdaR * lambdaR * lambdaR * lambdaR * lambdaR * lambdaR * lambdaR);
                prfrz = fmin(prfrz * odr * dt, qrp);
            }
            if (E > T(100)) bad = true;
        }
        // cloud ice: initiation, deposition, conversion to snow, collection by
        // snow; melting above freezing
        T pint = T(0), pdepi = T(0), pconv = T(0), psaci = T(0), psmlti = T(0);
        if (temperature < T(273.16)) {
            const T nc0 = T(1.0e3) * exp(T(0.1) * (T(273.16) - temperature));
            const T nc = fmin(fmax(T(5.38e7) * pow(rhou * qip, T(0.75)), T(1.0e3)), T(1.0e6));
            if (qvi_sat < vapor) pint = fmin(T(R::M0) * nc0 / rhou, vapor - qvi_sat);
            if (qip > minvar || qsp > minvar) {
                App = (Lv / (Ka * temperature)) * ((Ls * Mw) / (Rstar * temperature) - T(1));
                Bpp = Rstar * temperature / (chi * Mw * esi);
                const T MI = rhou * qip / nc;
                const T Dl = T(11.3) * sqrt(MI);
                pdepi = (T(4) * Dl * (vapor / qvi_sat - T(1)) * nc) / (App + Bpp) * odr * dt;
            }
            if (qip > minvar) {
                const T qimax = (temperature > T(233.16) && pd > T(30000)) ? T(8.0e-5) * odr : T(0.18e-3);
                if (qip > qimax) pconv = qip - qimax;
            }
            if (qip > minvar && lambdaS > T(1e-15)) {
                const T ESI = exp(T(0.05) * (temperature - T(273.16)));
                psaci = (trigpi * app * qip * ESI * N0S) / T(4) * pow(p0 / pd, T(0.4)) * T(2.22) /
                        pow(lambdaS, T(3.11)) * dt;
            }
        } else {
            psmlti = qip;
        }
        // snow: melting, deposition, evaporation of melting snow
        T psmlt = T(0), psdep = T(0), pmltev = T(0);
        if (qsp > minvar && lambdaS > T(1e-15)) {
            var = T(0.65) / (lambdaS * lambdaS) +
                  T(0.44) * sqrt(app * rhou / mu_s) * pow(p0 / pd, T(0.2)) * T(1.383) / pow(lambdaS, T(2.555));
            if (temperature > T(273.16)) {
                psmlt = -(T(2) * trigpi * N0S / Lf) * Ka * (temperature - T(273.16)) * var;
                psmlt = dt * psmlt * odr;
            }
            if (temperature < T(273.16)) {
                psdep = T(4) * (vapor / qvi_sat - T(1)) * N0S / (App + Bpp) * var;
                psdep = dt * psdep * odr;
            }
            if (temperature >= T(273.16)) {
                Ap = (Lv / (Ka * temperature)) * ((Lv * Mw) / (Rstar * temperature) - T(1));
                Bp = Rstar * temperature / (chi * Mw * esl);
                pmltev = T(4) * (vapor / qvl_sat - T(1)) * N0S / (Ap + Bp) * var;
                pmltev = dt * pmltev * odr;
            }
            if (fabs(psmlt) > T(100)) bad = true;
        }
        // cloud water collected by snow; frozen below tmin
        T psacw_cold = T(0), psacw_warm = T(0);
        if (qcp > minvar && lambdaS > T(1e-15)) {
            const T psacw = (trigpi * app * qcp * T(R::ESC) * N0S) / T(4) * pow(p0 / pd, T(0.4)) * T(2.22) /
                            pow(lambdaS, T(3.11)) * dt;
            if (temperature < T(273.16)) psacw_cold = psacw;
            else psacw_warm = psacw;
        }
        T pcfrz = T(0);
        if (temperature < T(R::tmin)) pcfrz = qcp;
        T pint_p_pdepi = fmin(pint + pdepi, vapor);
        pint_p_pdepi = -fmin(-pint_p_pdepi, qip);
        qvp += -(pcond + E + psdep + pmltev + pint_p_pdepi);
        qcp += pcond + psmlti - A - B - psacw_warm - psacw_cold - pcfrz;
        qip += pint_p_pdepi - psmlti - psaci - pconv + pcfrz;
        qrp += E + A + B - psmlt + psacw_warm - prfrz;
        qsp += psdep + pmltev + psaci + psmlt + psacw_cold + pconv + prfrz;
        const T diabatic = Lv / cpp * (pcond + E + pmltev) + Ls / cpp * (pint_p_pdepi + psdep) +
                           Lf / cpp * (psmlt + psmlti + psacw_cold + pcfrz + prfrz);
        thp += diabatic;
    }
    {   // saturation_adjustment (rutledge.cpp:700-820)
        const T theta = thp + thbar + p.tb[k];
        const T vapor = qvp + qbar + p.qb[k];
        const T temp = theta * pressure;
        T phi, phil, phii;
        const T qvsat = rut_qvsat(temp, pd, phi, phil, phii);
        T Cl = T(0), Ci = T(0);
        if (vapor > qvsat) {
            if (temp > T(R::tmax)) Cl = (vapor - qvsat) / (T(1.0) + phi);
            else if (temp < T(R::tmin)) Ci = (vapor - qvsat) / (T(1.0) + phi);
            else {
                Cl = RUT_ALPHA(temp) * (vapor - qvsat) / (T(1.0) + phi);
                Ci = (T(1.0) - RUT_ALPHA(temp)) * (vapor - qvsat) / (T(1.0) + phi);
            }
            if (F.sat) F.sat[c] = 1;
        } else if (vapor < qvsat && (qcp + qip) > T(0)) {
            if (temp > T(R::tmax)) Cl = -fmin(qcp, (qvsat - vapor) / (T(1.0) + phi));
            else if (temp < T(R::tmin)) Ci = -fmin(qip, (qvsat - vapor) / (T(1.0) + phi));
            else {
                Cl = -fmin(qcp, (qvsat - vapor) / (T(1.0) + phil));
                if (Cl + qcp <= T(0)) Ci = -fmin(qip, (qvsat - vapor + Cl) / (T(1.0) + phii));
            }
            if (F.sat) F.sat[c] = -(Ci + Cl) < qcp + qip;
        } else if (F.sat) {
            F.sat[c] = vapor == qvsat;
        }
        qip += Ci;
        qcp += Cl;
        qvp -= (Ci + Cl);
        const T diabatic = (Lv / cpp) * Cl + (Ls / cpp) * Ci;
        thp += diabatic;
    }
    // zero_moisture of this point
    if (qcp < T(0)) qcp = T(0);
    if (qrp < T(0)) qrp = T(0);
    if (qip < T(0)) qip = T(0);
    if (qsp < T(0)) qsp = T(0);
    if (qvp + qbar + p.qb[k] < T(0)) qvp = -(qbar + p.qb[k]);
    F.P[FTH][c] = thp;
    F.P[FQV][c] = qvp;
    F.P[FQC][c] = qcp;
    F.P[FQR][c] = qrp;
    F.P[FQI][c] = qip;
    F.P[FQS][c] = qsp;
    if (bad) atomicExch(err, 1);
    if (precip && k == 1) ice_precip_col(p, F, i, j);
}

// the column's Eulerian precipitation over the last step (precip_rate,
// microphysics.cpp:143-160): rain at the rain fall speed into accRain, rain
// and cloud ice at the snow fall speed into accSnow (rutledge.cpp:486-489)
template <typename T>
__global__ void k_ice_precip(KParams<T> p, KFields<T> F)
{
    const int nyi = p.ny - 2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)(p.nx - 2) * nyi) return;
    ice_precip_col(p, F, 1 + (int)(t / nyi), 1 + (int)(t % nyi));
}

// the intercept that the last snowy point of the pass left (the largest
// point index in the reference's loop order), kept for the snow fall speed;
// the record is reset for the next pass
template <typename T>
__global__ void k_ice_n0s(KFields<T> F)
{
    if (blockIdx.x || threadIdx.x) return;
    const int idx = *F.n0s_idx;
    if (idx >= 0) *F.n0s = F.n0s_pt[idx];
    *F.n0s_idx = -1;
}

#undef RUT_ESL
#undef RUT_ESI
#undef RUT_QSAT
#undef RUT_ALPHA

}  // namespace ga
