// ga_lin_kernels.cuh - device code of the tangent-linear model (TLM) and the
// adjoint of the dry, non-periodic step, templated on the real type T.
// Included after ga_kernels.cuh by ga_f64.cu / ga_f32.cu.
//
// The reference has no linearisation; these kernels differentiate the step
// implemented by ga_kernels.cuh (s_integrate_rk3, driver_serial.cpp:178-286).
//
// Conventions:
//   - upwind signs (signof, fluxes.cpp:295-311) are frozen at the trajectory;
//   - every advective face flux has the form F = a*B + (ab + a)*S
//     (compute_fluxes / compute_fluxes_scalar, fluxes.cpp:582-654), a the
//     advecting perturbation velocity, ab its basic-state part, B the basic
//     state of the advected field interpolated with sign(a), S the advected
//     perturbation interpolated with sign(ab + a).  Its tangent is
//     dF = (B + S)*da + (ab + a)*dS;
//   - the pressure solve, projection, sponges, top/bottom conditions and
//     Rayleigh damping are linear: the TLM runs the forward kernels on the
//     tangent buffers; the adjoint runs the transposes below;
//   - the adjoint is in gather form: every output point sums the
//     contributions that reach it, so no kernel needs atomics.  Where an
//     operator is in place and a point's transpose reads a neighbour that
//     another thread rewrites (the lateral mirror, the top/bottom copies),
//     the kernel reads everything before writing (block-wide phases).
#pragma once
#include "ga_kernels.cuh"

namespace ga {

// cells whose tendency the advection step writes (advection.cpp:304-373):
// i in [3,NX-3), j in [3,NY-3), k in [kmin,NZ-1); kmin 1 (u, v, theta), 2 (w)
template <typename T>
__device__ __forceinline__ bool adv_cell(const KParams<T> &p, int i, int j, int k, int kmin)
{
    return i >= 3 && i < p.nx - 3 && j >= 3 && j < p.ny - 3 && k >= kmin && k < p.nz - 1;
}

// A linearised advective face: the stencil of the advecting velocity
// (field `dir`: u for x faces, v for y, w for z), the stencil of the advected
// field and the two coefficients of its tangent.
template <typename T>
struct LinFace {
    int ia0, ia1;  // advecting stencil (ia1 < 0: one point, weight 1; else two, 0.5 each)
    int x0, xs;    // advected stencil: first point and stride
    int nx;        // 6 (5th order), 4 (3rd order), 2 (2nd order, no sign term)
    T sg;          // sign(ab + a)
    T ga, gs;      // dF = ga*da + gs*dS
};

// The equations of the linearised advection: 0 u, 1 v, 2 theta, 3 qv, 4 qc,
// 5 qr.  FX: advected field; BX: its basic state (-1: none); ZBIT: its
// zero_moisture clipping bit.
template <int EQ>
struct LinEq {
    static constexpr int FX = EQ == 0 ? FU : EQ == 1 ? FV : EQ == 2 ? FTH : EQ == 3 ? FQV : EQ == 4 ? FQC : FQR;
    static constexpr int BX = EQ == 0 ? 0 : EQ == 1 ? 1 : EQ == 2 ? 3 : EQ == 3 ? 4 : -1;
    static constexpr int ZBIT = EQ == 3 ? 1 : EQ == 4 ? 2 : EQ == 5 ? 4 : 0;
};

// fall speed of the rain flux at level m of a column (vt_at): recomputed from
// the rain on levels 1..NZ-2 (level 0 uses level 1), stored above
template <typename T>
__device__ __forceinline__ T lin_vt(const KParams<T> &p, const KFields<T> &R, int c0, int m)
{
    if (m < p.nz - 1) {
        const int mm = m == 0 ? 1 : m;
        return fall_speed_point(p, R.cur[FQR][c0 + mm], mm);
    }
    return R.vt[c0 + m];
}
// d(fall speed)/d(rain) at level m (0 where the fall speed is stored or
// the rain is below the threshold): vt = c * qr^0.1364
template <typename T>
__device__ __forceinline__ T lin_dvt(const KParams<T> &p, const KFields<T> &R, int c0, int m)
{
    if (m < 1 || m > p.nz - 2) return T(0);
    const T qr = R.cur[FQR][c0 + m];
    if (!(qr > T(1.0e-12))) return T(0);
    return T(0.1364) * fall_speed_point(p, qr, m) / qr;
}

// The rain's vertical face (interpolate_scalar_with_fallspeed and the qr
// fluxes of compute_fluxes_moisture): F = wf * st with wf = WBAR + W -
// (VT_k + VT_k+1)/2; at the bottom F = -(VT_1 + VT_1)/2 * (qr_0 + qr_1)/2,
// the outflow.  ga = st, gs = wf; the fall-speed part of d(wf) is carried by
// lin_dvt.
template <typename T>
__device__ __forceinline__ bool lin_face_rain(const KParams<T> &p, const KFields<T> &R, int i, int j, int k,
                                              LinFace<T> &L)
{
    const int nz = p.nz;
    const int c = gix(p.ny, nz, i, j, k), c0 = c - k;
    const T *Q = R.cur[FQR];
    T Sv, wf;
    if (k == 0) {
        const T v1 = lin_vt(p, R, c0, 1);
        Sv = T(0.5) * (Q[c] + Q[c + 1]);
        wf = T(-0.5) * (v1 + v1);
        L.ia0 = -1;
        L.x0 = c; L.nx = 2;
    } else {
        const int a = c + 1;
        const T wb = R.bar[2][a] + R.cur[FW][a];
        wf = wb - T(0.5) * (lin_vt(p, R, c0, k) + lin_vt(p, R, c0, k + 1));
        L.ia0 = a;
        if (k == 1 || k == nz - 2) {
            Sv = T(0.5) * (Q[c + 1] + Q[c]);
            L.x0 = c; L.nx = 2;
        } else {
            Sv = face3(Q[c - 1], Q[c], Q[c + 1], Q[c + 2], sgn(wf));
            L.x0 = c - 1; L.nx = 4;
        }
    }
    L.ia1 = -1;
    L.xs = 1;
    L.sg = sgn(wf);
    L.ga = Sv;
    L.gs = wf;
    return true;
}

// Build the face of equation EQ and direction DIR at (i,j,k) about the
// trajectory R (R.cur = fields at the start of the stage).  Returns false
// where the forward flux is identically zero (bottom faces but the rain's).
template <typename T, int EQ, int DIR>
__device__ __forceinline__ bool lin_face_t(const KParams<T> &p, const KFields<T> &R, int i, int j, int k,
                                           LinFace<T> &L)
{
    if (EQ == 5 && DIR == 2) return lin_face_rain(p, R, i, j, k, L);
    const int ny = p.ny, nz = p.nz;
    if (DIR == 2 && k == 0) return false;
    constexpr int FX = LinEq<EQ>::FX, BX = LinEq<EQ>::BX;
    const T *X = R.cur[FX], *XB = BX >= 0 ? R.bar[BX] : nullptr;
    const T *A = R.cur[DIR], *AB = R.bar[DIR];
    const int c = gix(ny, nz, i, j, k);
    constexpr int one = 1;
    const int sx = ny * nz, sy = nz;
    if (EQ >= 2) {
        L.ia0 = DIR == 0 ? c + sx : DIR == 1 ? c + sy : c + one;
        L.ia1 = -1;
    } else if (EQ == 0) {
        if (DIR == 0) { L.ia0 = c + sx; L.ia1 = c; }
        else if (DIR == 1) { L.ia0 = c + sy; L.ia1 = c - sx + sy; }
        else { L.ia0 = c + 1; L.ia1 = c - sx + 1; }
    } else {
        if (DIR == 0) { L.ia0 = c + sx; L.ia1 = c + sx - sy; }
        else if (DIR == 1) { L.ia0 = c + sy; L.ia1 = c; }
        else { L.ia0 = c + 1; L.ia1 = c - sy + 1; }
    }
    T a, ab;
    if (EQ >= 2) {
        a = A[L.ia0];
        ab = AB[L.ia0];
    } else {
        a = T(0.5) * (A[L.ia0] + A[L.ia1]);
        ab = T(0.5) * (AB[L.ia0] + AB[L.ia1]);
    }
    const T sgs = sgn(ab + a), sgb = sgn(a);
    T Sv, Bv = T(0);
    if (DIR < 2) {
        const int st = DIR == 0 ? sx : sy;
        const int c0 = c - 2 * st;
        L.x0 = c0; L.xs = st; L.nx = 6;
        Sv = face5(X[c0], X[c0 + st], X[c0 + 2 * st], X[c0 + 3 * st], X[c0 + 4 * st], X[c0 + 5 * st], sgs);
        if (BX >= 0)
            Bv = face5(XB[c0], XB[c0 + st], XB[c0 + 2 * st], XB[c0 + 3 * st], XB[c0 + 4 * st], XB[c0 + 5 * st], sgb);
    } else if (k == 1 || k == nz - 2) {
        L.x0 = c; L.xs = 1; L.nx = 2;
        Sv = T(0.5) * (X[c + 1] + X[c]);
        if (BX >= 0) Bv = T(0.5) * (XB[c + 1] + XB[c]);
    } else {
        const int c0 = c - 1;
        L.x0 = c0; L.xs = 1; L.nx = 4;
        Sv = face3(X[c0], X[c0 + 1], X[c0 + 2], X[c0 + 3], sgs);
        if (BX >= 0) Bv = face3(XB[c0], XB[c0 + 1], XB[c0 + 2], XB[c0 + 3], sgb);
    }
    L.sg = sgs;
    L.ga = Bv + Sv;
    L.gs = ab + a;
    return true;
}

template <typename T>
__device__ __forceinline__ bool lin_face(const KParams<T> &p, const KFields<T> &R, int eq, int dir, int i, int j,
                                         int k, LinFace<T> &L)
{
    switch (eq * 3 + dir) {
    case 0: return lin_face_t<T, 0, 0>(p, R, i, j, k, L);
    case 1: return lin_face_t<T, 0, 1>(p, R, i, j, k, L);
    case 2: return lin_face_t<T, 0, 2>(p, R, i, j, k, L);
    case 3: return lin_face_t<T, 1, 0>(p, R, i, j, k, L);
    case 4: return lin_face_t<T, 1, 1>(p, R, i, j, k, L);
    case 5: return lin_face_t<T, 1, 2>(p, R, i, j, k, L);
    case 6: return lin_face_t<T, 2, 0>(p, R, i, j, k, L);
    case 7: return lin_face_t<T, 2, 1>(p, R, i, j, k, L);
    case 8: return lin_face_t<T, 2, 2>(p, R, i, j, k, L);
    case 9: return lin_face_t<T, 3, 0>(p, R, i, j, k, L);
    case 10: return lin_face_t<T, 3, 1>(p, R, i, j, k, L);
    case 11: return lin_face_t<T, 3, 2>(p, R, i, j, k, L);
    case 12: return lin_face_t<T, 4, 0>(p, R, i, j, k, L);
    case 13: return lin_face_t<T, 4, 1>(p, R, i, j, k, L);
    case 14: return lin_face_t<T, 4, 2>(p, R, i, j, k, L);
    case 15: return lin_face_t<T, 5, 0>(p, R, i, j, k, L);
    case 16: return lin_face_t<T, 5, 1>(p, R, i, j, k, L);
    default: return lin_face_t<T, 5, 2>(p, R, i, j, k, L);
    }
}

// tangent of one face flux
template <typename T>
__device__ __forceinline__ T tl_face(const KParams<T> &p, const KFields<T> &R, const KFields<T> &D, int eq, int dir,
                                     int i, int j, int k)
{
    LinFace<T> L;
    if (!lin_face(p, R, eq, dir, i, j, k, L)) return T(0);
    const T *dA = D.cur[dir];
    const int fx = eq == 0 ? FU : eq == 1 ? FV : eq == 2 ? FTH : eq == 3 ? FQV : eq == 4 ? FQC : FQR;
    const T *dX = D.cur[fx];
    T da = L.ia0 < 0 ? T(0) : L.ia1 < 0 ? dA[L.ia0] : T(0.5) * (dA[L.ia0] + dA[L.ia1]);
    if (eq == 5 && dir == 2) {  // the fall speed follows the rain
        const int c0 = gix(p.ny, p.nz, i, j, 0);
        const T *dQ = D.cur[FQR];
        if (k == 0) {
            const T d1 = lin_dvt(p, R, c0, 1) * dQ[c0 + 1];
            da = da - T(0.5) * (d1 + d1);
        } else {
            const T d0 = lin_dvt(p, R, c0, k) * dQ[c0 + k];
            const T d1 = k + 1 < p.nz ? lin_dvt(p, R, c0, k + 1) * dQ[c0 + k + 1] : T(0);
            da = da - T(0.5) * (d0 + d1);
        }
    }
    T ds;
    const int c = L.x0, st = L.xs;
    if (L.nx == 6) ds = face5(dX[c], dX[c + st], dX[c + 2 * st], dX[c + 3 * st], dX[c + 4 * st], dX[c + 5 * st], L.sg);
    else if (L.nx == 4) ds = face3(dX[c], dX[c + 1], dX[c + 2], dX[c + 3], L.sg);
    else ds = T(0.5) * (dX[c + 1] + dX[c]);
    return L.ga * da + L.gs * ds;
}

// tangent of the tendency of equation eq at a cell (u_tend_cell, v_tend_cell,
// theta/qv/qc/qr_tend_cell with Z_ADVECT_BASE: advection.cpp:16-18, 73-122,
// 152-253)
template <typename T>
__device__ T tl_tend(const KParams<T> &p, const KFields<T> &R, const KFields<T> &D, int eq, int i, int j, int k)
{
    const int ny = p.ny, nz = p.nz;
    const T DTZ = p.dtz * p.mu[k];
    T t = -p.dtx * (tl_face(p, R, D, eq, 0, i, j, k) - tl_face(p, R, D, eq, 0, i - 1, j, k)) -
          p.dty * (tl_face(p, R, D, eq, 1, i, j, k) - tl_face(p, R, D, eq, 1, i, j - 1, k)) -
          DTZ * (p.rhow[k + 1] * tl_face(p, R, D, eq, 2, i, j, k) - p.rhow[k] * tl_face(p, R, D, eq, 2, i, j, k - 1)) *
              p.one_d_rhou[k];
    if (eq == 0) {
        const T *dV = D.cur[FV];
        t += p.dt * p.f[j] * T(0.25) *
             (dV[gix(ny, nz, i, j, k)] + dV[gix(ny, nz, i, j + 1, k)] + dV[gix(ny, nz, i - 1, j, k)] +
              dV[gix(ny, nz, i - 1, j + 1, k)]);
    } else if (eq == 1) {
        const T *dU = D.cur[FU];
        t -= p.dt * p.f[j] * T(0.25) *
             (dU[gix(ny, nz, i, j, k)] + dU[gix(ny, nz, i + 1, j, k)] + dU[gix(ny, nz, i, j - 1, k)] +
              dU[gix(ny, nz, i + 1, j - 1, k)]);
    } else if (eq == 2 || eq == 3) {
        const T *dW = D.cur[FW], *base = eq == 2 ? p.tb : p.qb;
        const int c = gix(ny, nz, i, j, k);
        t -= DTZ * T(0.5) *
             (p.rhow[k + 1] * dW[c + 1] * (base[k + 1] - base[k]) + p.rhow[k] * dW[c] * (base[k] - base[k - 1])) *
             p.one_d_rhou[k];
    }
    return t;
}

// TLM of advect_uvw_velocity, advect_theta and (moist) advect_microphysics_
// cell with zero_moisture (advection.cpp:304-498, microphysics.cpp:675-700):
// D.P = D.M + step * d(tendency) on the cells the forward step writes; a
// moisture point the trajectory clipped (R.qmask) has no tangent.
template <typename T>
__global__ void k_tl_advect(KParams<T> p, KFields<T> R, KFields<T> D, T step, T sdtg)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nzi = p.nz - 2, nyi = p.ny - 6, nxi = p.nx - 6;
    if (t >= (long)nxi * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 3 + (int)((t / nzi) % nyi);
    const int i = 3 + (int)(t / ((long)nzi * nyi));
    const int c = gix(p.ny, p.nz, i, j, k);
    D.P[FU][c] = D.M[FU][c] + step * tl_tend(p, R, D, 0, i, j, k);
    D.P[FV][c] = D.M[FV][c] + step * tl_tend(p, R, D, 1, i, j, k);
    D.P[FTH][c] = D.M[FTH][c] + step * tl_tend(p, R, D, 2, i, j, k);
    if (k >= 2) {  // buoyancy_dry / buoyancy_warm_micro (advection.cpp:42-58, 329-337): linear
        T b0 = D.cur[FTH][c] / p.tbv[k], b1 = D.cur[FTH][c - 1] / p.tbv[k - 1];
        if (p.moist) {
            b0 = b0 + T(0.61) * D.cur[FQV][c] - D.cur[FQC][c] - D.cur[FQR][c];
            b1 = b1 + T(0.61) * D.cur[FQV][c - 1] - D.cur[FQC][c - 1] - D.cur[FQR][c - 1];
        }
        D.P[FW][c] = D.M[FW][c] + sdtg * (b0 + b1);
    }
    if (p.moist) {
        const unsigned char bits = R.qmask ? R.qmask[c] : 0;
        D.P[FQV][c] = (bits & 1) ? T(0) : D.M[FQV][c] + step * tl_tend(p, R, D, 3, i, j, k);
        D.P[FQC][c] = (bits & 2) ? T(0) : D.M[FQC][c] + step * tl_tend(p, R, D, 4, i, j, k);
        D.P[FQR][c] = (bits & 4) ? T(0) : D.M[FQR][c] + step * tl_tend(p, R, D, 5, i, j, k);
    }
}

// Jacobian of run_kessler_microphysics at one point: d(theta, qv, qc, qr)/
// d(theta, qv, qc, qr, pi), by kessler_point on dual numbers (the branch
// decisions are the trajectory's)
template <typename T>
__device__ __forceinline__ void kessler_jacobian(const KParams<T> &p, const KFields<T> &R, int k, int ix,
                                                 const T in[5], T J[4][5])
{
    Dual<T, 5> x[5];
    for (int a = 0; a < 5; a++) {
        x[a].v = in[a];
        for (int q = 0; q < 5; q++) x[a].d[q] = a == q ? T(1) : T(0);
    }
    kessler_point(x[0], x[1], x[2], x[3], x[4], kes_point(p, R, k, ix));
    for (int a = 0; a < 4; a++)
        for (int q = 0; q < 5; q++) J[a][q] = x[a].d[q];
}

// TLM of the Kessler step: D.P (theta, qv, qc, qr) <- J * (D.P, D.pi) with J
// at the trajectory R.P, R.pi (before the trajectory's own Kessler step)
template <typename T>
__global__ void __launch_bounds__(128) k_tl_kessler(KParams<T> p, KFields<T> R, KFields<T> D)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nzi = p.nz - 2, nyi = p.ny - 2, nxi = p.nx - 2;
    if (t >= (long)nxi * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 1 + (int)((t / nzi) % nyi);
    const int i = 1 + (int)(t / ((long)nzi * nyi));
    const int ix = gix(p.ny, p.nz, i, j, k);
    const int fl[4] = {FTH, FQV, FQC, FQR};
    T in[5], d[5], J[4][5];
    for (int a = 0; a < 4; a++) {
        in[a] = R.P[fl[a]][ix];
        d[a] = D.P[fl[a]][ix];
    }
    in[4] = R.pi[ix];
    d[4] = D.pi[ix];
    kessler_jacobian(p, R, k, ix, in, J);
    for (int a = 0; a < 4; a++) {
        T v = T(0);
        for (int q = 0; q < 5; q++) v += J[a][q] * d[q];
        D.P[fl[a]][ix] = v;
    }
}

// adjoint of the Kessler step about the recorded inputs kin (theta, qv, qc,
// qr, pi: kin + q*N): A.P <- J^T A.P, pi-bar gets the pi row.  Covers every
// point: off the Kessler points pi-bar is only reset (acc = 0) or kept.
template <typename T>
__global__ void __launch_bounds__(128) k_adj_kessler(KParams<T> p, KFields<T> R, const T *kin, KFields<T> A, int acc)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const int nz = p.nz, ny = p.ny;
    const int k = (int)(t % nz), j = (int)((t / nz) % ny), i = (int)(t / ((long)nz * ny));
    const int ix = (int)t;
    const T pib = acc ? A.pi[ix] : T(0);
    if (i < 1 || i > p.nx - 2 || j < 1 || j > ny - 2 || k < 1 || k > nz - 2) {
        A.pi[ix] = pib;
        return;
    }
    const int fl[4] = {FTH, FQV, FQC, FQR};
    T in[5], ob[4], J[4][5];
    for (int q = 0; q < 5; q++) in[q] = kin[(size_t)q * p.n + ix];
    for (int a = 0; a < 4; a++) ob[a] = A.P[fl[a]][ix];
    kessler_jacobian(p, R, k, ix, in, J);
    for (int q = 0; q < 4; q++) {
        T v = T(0);
        for (int a = 0; a < 4; a++) v += J[a][q] * ob[a];
        A.P[fl[q]][ix] = v;
    }
    T v = T(0);
    for (int a = 0; a < 4; a++) v += J[a][4] * ob[a];
    A.pi[ix] = pib + v;
}

// ---------------------------------------------------------------------------
// adjoint of the advection step, gather form.  A block owns a tile of
// AJ_TI x AJ_TJ x AJ_TK cells (AJ_CPT per thread); for each of the nine face
// families (three equations x three directions, each specialised at compile
// time) it evaluates the adjoint of every face whose stencil reaches the tile
// into shared memory (S' = Fbar*(ab+a), sign*S', a' = Fbar*(B+S)), then every
// cell sums what reaches it.  The same kernel finishes the stage's
// bookkeeping on the cells it owns:
//   - M-bar += P-bar where the forward advection overwrote P (the P-bar there
//     is zeroed when the buffer next receives adjoint contributions: with
//     zero_cur the current-slot values of the advected cells are replaced,
//     not added to, since they are that stale P-bar);
//   - the lateral ring of P-bar u, v, w is zeroed (mirror_boundaries wrote
//     it; k_adj_div has already moved its values to the mirrored points).
// ---------------------------------------------------------------------------
// 8 levels per tile: a row of a tile is a whole 32-byte sector in FP32
constexpr int AJ_TI = 16, AJ_TJ = 8, AJ_TK = 8, AJ_THREADS = 256;
constexpr int AJ_CPT = AJ_TI * AJ_TJ * AJ_TK / AJ_THREADS;
constexpr int AJ_BOX_X = (AJ_TI + 5) * (AJ_TJ + 1) * AJ_TK;
constexpr int AJ_BOX_Y = (AJ_TI + 1) * (AJ_TJ + 5) * AJ_TK;
constexpr int AJ_BOX_Z = (AJ_TI + 1) * (AJ_TJ + 1) * (AJ_TK + 3);
constexpr int AJ_NFACE = AJ_BOX_X > AJ_BOX_Y ? (AJ_BOX_X > AJ_BOX_Z ? AJ_BOX_X : AJ_BOX_Z)
                                             : (AJ_BOX_Y > AJ_BOX_Z ? AJ_BOX_Y : AJ_BOX_Z);  // largest face box
// box of tendency adjoints one equation's faces read: the tile + 3 points in
// x and y, 2 below and 2 above
constexpr int AJ_BI = AJ_TI + 6, AJ_BJ = AJ_TJ + 6, AJ_BK = AJ_TK + 4, AJ_NTB = AJ_BI * AJ_BJ * AJ_BK;

// The two coefficients of every linearised face, once per stage: for each
// cell c and face family (EQ, DIR), coef[GA*N + c] = B + S and
// coef[GS*N + c] = ab + a of the face at c (its sign is the frozen upwind
// sign), zero where the face is not next to an advected cell.  The scalar
// equations (theta, qv, qc, qr) share ab + a on every face but the rain's
// vertical one, so those are stored once per direction (LinSlot).
constexpr int LIN_NCOEF = 18;        // dry: u, v (6 families x 2), scalar ab+a (3), theta B+S (3)
constexpr int LIN_NCOEF_MOIST = 29;  // moist: + qv, qc, qr B+S (9), rain vertical ab+a, d(fall speed)/d(rain)
constexpr int LIN_DVT_SLOT = 28;
template <int EQ, int DIR> struct LinSlot {
    static constexpr int GA = EQ < 2 ? 2 * (3 * EQ + DIR) : 15 + 3 * (EQ - 2) + DIR;
    static constexpr int GS = EQ < 2 ? 2 * (3 * EQ + DIR) + 1 : (EQ == 5 && DIR == 2) ? 27 : 12 + DIR;
    static constexpr bool OWNS_GS = EQ < 3 || (EQ == 5 && DIR == 2);  // the family that writes GS
};

template <typename T, int EQ, int DIR>
__device__ __forceinline__ void lin_coef_face(const KParams<T> &p, const KFields<T> &R, T *coef, int i, int j, int k,
                                              int c)
{
    bool need;
    if (DIR == 0) need = adv_cell(p, i, j, k, 1) || adv_cell(p, i + 1, j, k, 1);
    else if (DIR == 1) need = adv_cell(p, i, j, k, 1) || adv_cell(p, i, j + 1, k, 1);
    else need = adv_cell(p, i, j, k, 1) || (k + 1 < p.nz && adv_cell(p, i, j, k + 1, 1));
    T ga = T(0), gs = T(0);
    LinFace<T> L;
    if (need && lin_face_t<T, EQ, DIR>(p, R, i, j, k, L)) {
        ga = L.ga;
        gs = L.gs;
    }
    coef[(size_t)LinSlot<EQ, DIR>::GA * p.n + c] = ga;
    if (LinSlot<EQ, DIR>::OWNS_GS) coef[(size_t)LinSlot<EQ, DIR>::GS * p.n + c] = gs;
}

// The moist pass also zeroes P-bar of qv, qc, qr at the advected points
// the stage's zero_moisture clipped (qm bits 1, 2, 4): the clipped value does
// not depend on the advection, so its adjoint reaches neither the tendency
// nor the M fold.
template <typename T>
__global__ void k_lin_coef(KParams<T> p, KFields<T> R, T *coef, KFields<T> A, const unsigned char *qm)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const int nz = p.nz, ny = p.ny;
    const int k = (int)(t % nz), j = (int)((t / nz) % ny), i = (int)(t / ((long)nz * ny));
    const int c = (int)t;
    lin_coef_face<T, 0, 0>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 0, 1>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 0, 2>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 1, 0>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 1, 1>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 1, 2>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 2, 0>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 2, 1>(p, R, coef, i, j, k, c);
    lin_coef_face<T, 2, 2>(p, R, coef, i, j, k, c);
    if (p.moist) {
        lin_coef_face<T, 3, 0>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 3, 1>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 3, 2>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 4, 0>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 4, 1>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 4, 2>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 5, 0>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 5, 1>(p, R, coef, i, j, k, c);
        lin_coef_face<T, 5, 2>(p, R, coef, i, j, k, c);
        const bool inner = i >= 3 && i < p.nx - 3 && j >= 3 && j < p.ny - 3;
        coef[(size_t)LIN_DVT_SLOT * p.n + c] = inner ? lin_dvt(p, R, c - k, k) : T(0);
        const unsigned char b = qm[c];
        if (b && adv_cell(p, i, j, k, 1)) {
            if (b & 1) A.P[FQV][c] = T(0);
            if (b & 2) A.P[FQC][c] = T(0);
            if (b & 4) A.P[FQR][c] = T(0);
        }
    }
}

// Shared memory of k_adj_advect.  FP32 double-buffers the coefficient and
// tendency boxes (the next family's copies run under the current one's
// work, 3 blocks per SM); FP64 has one of each (2 blocks per SM) and copies
// the next family's coefficients during the current gather, so it keeps the
// face signs in an array of their own (fs2).
template <typename T>
struct AjCfg {
    static constexpr int CB = sizeof(T) == 4 ? 2 : 1;   // coefficient box buffers (B+S and ab+a each)
    static constexpr int TBB = sizeof(T) == 4 ? 2 : 1;  // tendency box buffers
    static constexpr int NFS = CB == 1 ? 3 : 2;          // face arrays: fs1, fab (+ fs2)
    static constexpr int NZF = AJ_TK + 3;                // z faces of a tile column (level factors)
    static constexpr int FS = 2 * CB * AJ_NFACE, TB = FS + NFS * AJ_NFACE, ZF = TB + TBB * AJ_NTB;
    static constexpr size_t smem = (size_t)(ZF + 2 * NZF) * sizeof(T);
};

// face-box geometry of the family (EQ, DIR): the tile plus the faces whose
// stencil reaches it (3 before and 2 after in x and y, 2 below and 1 above in z)
template <int DIR>
struct AjBox {
    static constexpr int bdi = DIR == 0 ? 3 : 0, bdj = DIR == 1 ? 3 : 0, bdk = DIR == 2 ? 2 : 0;
    static constexpr int bni = DIR == 0 ? AJ_TI + 5 : AJ_TI + 1;
    static constexpr int bnj = DIR == 1 ? AJ_TJ + 5 : AJ_TJ + 1;
    static constexpr int bnk = DIR == 2 ? AJ_TK + 3 : AJ_TK;
    static constexpr int nf = bni * bnj * bnk;
    static constexpr int NPF = (nf + AJ_THREADS - 1) / AJ_THREADS;
    static_assert(nf <= AJ_NFACE, "face box larger than its shared-memory store");
};

// copies of the family's two coefficient boxes (zero off the domain)
template <typename T, int EQ, int DIR>
__device__ __forceinline__ void issue_coef(const KParams<T> &p, const T *__restrict__ coef, int i0, int j0, int k0,
                                           T *cb)
{
    using B = AjBox<DIR>;
    const T *ga_f = coef + (size_t)LinSlot<EQ, DIR>::GA * p.n, *gs_f = coef + (size_t)LinSlot<EQ, DIR>::GS * p.n;
    const int bi0 = i0 - B::bdi, bj0 = j0 - B::bdj, bk0 = k0 - B::bdk;
    // not unrolled: the copies are asynchronous, and an unrolled issue holds
    // every address in registers at once
#pragma unroll 1
    for (int q = 0; q < B::NPF; q++) {
        const int f = threadIdx.x + q * AJ_THREADS;
        if (f < B::nf) {
            const int fi = bi0 + f / (B::bnk * B::bnj), fj = bj0 + (f / B::bnk) % B::bnj, fk = bk0 + f % B::bnk;
            const bool ok = fi >= 0 && fi < p.nx && fj >= 0 && fj < p.ny && fk >= 0 && fk < p.nz;
            const int c = ok ? gix(p.ny, p.nz, fi, fj, fk) : 0;
            cp_elem(cb + f, ga_f + c, ok);
            cp_elem(cb + AJ_NFACE + f, gs_f + c, ok);
        }
    }
}

// copy of equation EQ's P-bar over the tendency box, zero off the advected
// cells: times the stage's step it is the tendency adjoint.  The moisture
// fields hold no P-bar at their clipped points (k_lin_coef zeroes it).
template <typename T, int EQ>
__device__ __forceinline__ void issue_tb(const KParams<T> &p, const KFields<T> &A, int i0, int j0, int k0, T *tb)
{
    const T *P = A.P[LinEq<EQ>::FX];
    constexpr int NQ = (AJ_NTB + AJ_THREADS - 1) / AJ_THREADS;
#pragma unroll 1
    for (int q = 0; q < NQ; q++) {
        const int e = threadIdx.x + q * AJ_THREADS;
        if (e < AJ_NTB) {
            const int i = i0 - 3 + e / (AJ_BK * AJ_BJ), j = j0 - 3 + (e / AJ_BK) % AJ_BJ, k = k0 - 2 + e % AJ_BK;
            const bool ok = adv_cell(p, i, j, k, 1);
            cp_elem(tb + e, P + (ok ? gix(p.ny, p.nz, i, j, k) : 0), ok);
        }
    }
}

// the terms of equation EQ outside the face fluxes, from its tendency box:
// Coriolis of u into v and of v into u (advection.cpp:84-92, 112-120), the
// vertical advection of the basic-state theta (Z_ADVECT_BASE) into w
template <typename T, int EQ>
__device__ __forceinline__ void adj_extra(const KParams<T> &p, const T *tb, T step, int i0, int j0, int k0,
                                          T (&acc)[AJ_CPT][7])
{
    const T fdt = p.dt * T(0.25);
#pragma unroll
    for (int r = 0; r < AJ_CPT; r++) {
        const int e = threadIdx.x + r * AJ_THREADS;
        const int li = e / (AJ_TK * AJ_TJ), lj = (e / AJ_TK) % AJ_TJ, lk = e % AJ_TK;
        const int pj = j0 + lj, pk = k0 + lk;
        auto TB = [&](int di, int dj, int dk) {
            return step * tb[((li + 3 + di) * AJ_BJ + (lj + 3 + dj)) * AJ_BK + lk + 2 + dk];
        };
        if (EQ == 0) {
            const int di[4] = {0, 0, 1, 1}, dj[4] = {0, -1, 0, -1};
#pragma unroll
            for (int n = 0; n < 4; n++) {
                const T tu = TB(di[n], dj[n], 0);
                if (tu != T(0)) acc[r][FV] += (fdt * p.f[pj + dj[n]]) * tu;
            }
        } else if (EQ == 1) {
            const int di[4] = {0, -1, 0, -1}, dj[4] = {0, 0, 1, 1};
#pragma unroll
            for (int n = 0; n < 4; n++) {
                const T tv = TB(di[n], dj[n], 0);
                if (tv != T(0)) acc[r][FU] -= (fdt * p.f[pj + dj[n]]) * tv;
            }
        } else if (EQ == 2 || EQ == 3) {
            const T *base = EQ == 2 ? p.tb : p.qb;
            const T t0 = TB(0, 0, -1), t1 = TB(0, 0, 0);
            if (t0 != T(0))
                acc[r][FW] -= (p.dtz * p.mu[pk - 1]) * T(0.5) * p.rhow[pk] * (base[pk] - base[pk - 1]) *
                              p.one_d_rhou[pk - 1] * t0;
            if (t1 != T(0))
                acc[r][FW] -= (p.dtz * p.mu[pk]) * T(0.5) * p.rhow[pk] * (base[pk] - base[pk - 1]) *
                              p.one_d_rhou[pk] * t1;
        }
    }
}

// One face family (EQ, DIR) of group G: wait for its coefficient box (and,
// for DIR 0, the equation's tendency box), start the copies of the next
// family's, evaluate the adjoint of every face of the box into shared memory
// (S' = Fbar*(ab+a), a' = Fbar*(B+S)), then every cell of the tile gathers
// what reaches it.
template <typename T, int G, int EQ, int DIR>
__device__ __forceinline__ void adj_family(const KParams<T> &p, const T *__restrict__ coef, const KFields<T> &A,
                                           T step, int i0, int j0, int k0, T *sm, T (&acc)[AJ_CPT][7])
{
    using C = AjCfg<T>;
    using B = AjBox<DIR>;
    constexpr int EQ0 = 3 * G, n = 3 * (EQ - EQ0) + DIR;
    constexpr bool HAS_NEXT = n < 8, NEXT_EQ = DIR == 2 && EQ < EQ0 + 2;
    constexpr int NEQ = DIR == 2 ? EQ + 1 : EQ, NDIR = (DIR + 1) % 3;
    constexpr int XF = LinEq<EQ>::FX;
    constexpr bool RAIN_Z = EQ == 5 && DIR == 2;
    const T *cga = sm + (n % C::CB) * 2 * AJ_NFACE, *cgs = cga + AJ_NFACE;
    T *fs1 = sm + C::FS, *fab = fs1 + AJ_NFACE, *fs2 = fab + AJ_NFACE;
    const T *tb = sm + C::TB + ((EQ - EQ0) % C::TBB) * AJ_NTB;
    const T *zf0 = sm + C::ZF, *zf1 = zf0 + C::NZF;
    const int nz = p.nz, t = threadIdx.x;
    if (C::CB == 2) {
        if (HAS_NEXT) issue_coef<T, NEQ, NDIR>(p, coef, i0, j0, k0, sm + ((n + 1) % 2) * 2 * AJ_NFACE);
        if (C::TBB == 2 && DIR == 0 && EQ < EQ0 + 2)
            issue_tb<T, (EQ < EQ0 + 2 ? EQ + 1 : EQ)>(p, A, i0, j0, k0, sm + C::TB + ((EQ + 1 - EQ0) % 2) * AJ_NTB);
        cp_commit();
        cp_wait<1>();
    } else {
        cp_wait<0>();
    }
    // the rain's fall-speed derivative at the tile's cells
    T dvr[AJ_CPT];
    if (RAIN_Z) {
#pragma unroll
        for (int r = 0; r < AJ_CPT; r++) {
            const int e = t + r * AJ_THREADS;
            const int pi = i0 + e / (AJ_TK * AJ_TJ), pj = j0 + (e / AJ_TK) % AJ_TJ, pk = k0 + e % AJ_TK;
            dvr[r] = (pi < p.nx && pj < p.ny && pk >= 1 && pk <= nz - 2)
                         ? coef[(size_t)LIN_DVT_SLOT * p.n + gix(p.ny, nz, pi, pj, pk)]
                         : T(0);
        }
    }
    __syncthreads();
    if (DIR == 0) adj_extra<T, EQ>(p, tb, step, i0, j0, k0, acc);
    // offset of a face's own cell in the tendency box, and of its +1 neighbour
    constexpr int tstep = DIR == 0 ? AJ_BJ * AJ_BK : DIR == 1 ? AJ_BK : 1;
#pragma unroll
    for (int q = 0; q < B::NPF; q++) {
        const int f = t + q * AJ_THREADS;
        if (f >= B::nf) break;
        const int li = f / (B::bnk * B::bnj), lj = (f / B::bnk) % B::bnj, lk = f % B::bnk;
        const T ga = cga[f], gs = cgs[f];
        const int tb0 = ((li + 3 - B::bdi) * AJ_BJ + (lj + 3 - B::bdj)) * AJ_BK + (lk + 2 - B::bdk);
        const T t0 = step * tb[tb0], t1 = step * tb[tb0 + tstep];
        T fb;
        if (DIR == 0) fb = p.dtx * (t1 - t0);
        else if (DIR == 1) fb = p.dty * (t1 - t0);
        else fb = zf1[lk] * t1 - zf0[lk] * t0;
        const T s1 = fb * gs;
        fs1[f] = s1;
        if (C::CB == 1) fs2[f] = gs > T(0) ? s1 : -s1;
        fab[f] = fb * ga;
    }
    __syncthreads();
    if (C::CB == 1) {
        // the face phase has read the coefficient and tendency boxes
        if (HAS_NEXT) issue_coef<T, NEQ, NDIR>(p, coef, i0, j0, k0, sm);
        if (NEXT_EQ) issue_tb<T, (NEXT_EQ ? EQ + 1 : EQ)>(p, A, i0, j0, k0, sm + C::TB);
        cp_commit();
    }
    const T C5[6] = {W<T>::c1_60, -W<T>::c2_15, W<T>::c37_60, W<T>::c37_60, -W<T>::c2_15, W<T>::c1_60};
    const T U5[6] = {W<T>::c1_60, T(-5) * W<T>::c1_60, T(10) * W<T>::c1_60, T(-10) * W<T>::c1_60,
                     T(5) * W<T>::c1_60, -W<T>::c1_60};
    const T C3[4] = {-W<T>::c1_12, W<T>::c7_12, W<T>::c7_12, -W<T>::c1_12};
    const T U3[4] = {-W<T>::c1_12, T(3) * W<T>::c1_12, T(-3) * W<T>::c1_12, W<T>::c1_12};
    // the upwind part of a face: sign(ab+a) * S'
    auto sgn = [&](int w, T s) { return C::CB == 1 ? fs2[w] : (cgs[w] > T(0) ? s : -s); };
#pragma unroll
    for (int r = 0; r < AJ_CPT; r++) {
        const int e = t + r * AJ_THREADS;
        const int li = e / (AJ_TK * AJ_TJ), lj = (e / AJ_TK) % AJ_TJ, lk = e % AJ_TK;
        // face-box coordinates of the cell
        const int bi = li + B::bdi, bj = lj + B::bdj, bk = lk + B::bdk;
        auto at = [&](int di, int dj, int dk) { return ((bi + di) * B::bnj + (bj + dj)) * B::bnk + (bk + dk); };
        T gx = T(0), ga;
        if (DIR == 0) {
#pragma unroll
            for (int m = 0; m < 6; m++) {
                const int w = at(2 - m, 0, 0);
                const T s = fs1[w];
                gx += C5[m] * s + U5[m] * sgn(w, s);
            }
            if (EQ == 0) ga = T(0.5) * (fab[at(-1, 0, 0)] + fab[at(0, 0, 0)]);
            else if (EQ == 1) ga = T(0.5) * (fab[at(-1, 0, 0)] + fab[at(-1, 1, 0)]);
            else ga = fab[at(-1, 0, 0)];
        } else if (DIR == 1) {
#pragma unroll
            for (int m = 0; m < 6; m++) {
                const int w = at(0, 2 - m, 0);
                const T s = fs1[w];
                gx += C5[m] * s + U5[m] * sgn(w, s);
            }
            if (EQ == 0) ga = T(0.5) * (fab[at(0, -1, 0)] + fab[at(1, -1, 0)]);
            else if (EQ == 1) ga = T(0.5) * (fab[at(0, -1, 0)] + fab[at(0, 0, 0)]);
            else ga = fab[at(0, -1, 0)];
        } else {
            const int pk = k0 + lk;
#pragma unroll
            for (int d = -2; d <= 1; d++) {
                const int fk = pk + d;
                if (fk < (RAIN_Z ? 0 : 1) || fk > nz - 2) continue;
                const int w = at(0, 0, d);
                const T s = fs1[w];
                if (fk <= 1 || fk == nz - 2) {  // 2nd order (and the rain's bottom outflow)
                    if (d == 0 || d == -1) gx += T(0.5) * s;
                } else {
                    const int m = 1 - d;  // position of the cell in the face's stencil fk-1..fk+2
                    gx += C3[m] * s + U3[m] * sgn(w, s);
                }
            }
            if (EQ == 0) ga = T(0.5) * (fab[at(0, 0, -1)] + fab[at(1, 0, -1)]);
            else if (EQ == 1) ga = T(0.5) * (fab[at(0, 0, -1)] + fab[at(0, 1, -1)]);
            else if (RAIN_Z) {
                // the bottom outflow does not depend on w; the fall speed of
                // levels 1..NZ-2 follows their rain (face 0 holds level 1 twice)
                ga = pk >= 2 ? fab[at(0, 0, -1)] : T(0);
                if (pk >= 1 && pk <= nz - 2) {
                    const T below = fab[at(0, 0, -1)] * (pk == 1 ? T(2) : T(1));
                    gx -= T(0.5) * dvr[r] * (fab[at(0, 0, 0)] + below);
                }
            } else ga = fab[at(0, 0, -1)];
        }
        acc[r][XF] += gx;
        acc[r][DIR] += ga;
    }
    __syncthreads();
}

template <typename T, int G, int EQ>
__device__ __forceinline__ void adj_equation(const KParams<T> &p, const T *__restrict__ coef, const KFields<T> &A,
                                             T step, int i0, int j0, int k0, T *sm, T (&acc)[AJ_CPT][7])
{
    adj_family<T, G, EQ, 0>(p, coef, A, step, i0, j0, k0, sm, acc);
    adj_family<T, G, EQ, 1>(p, coef, A, step, i0, j0, k0, sm, acc);
    adj_family<T, G, EQ, 2>(p, coef, A, step, i0, j0, k0, sm, acc);
}

// The adjoint advection runs as two launches over the same tiles: group 0
// the momentum and theta equations (gathering into u, v, w, theta), group 1
// the moisture equations (into u, v, w, qv, qc, qr), so that each keeps only
// its own accumulators live.  Group 0 runs first: it replaces the stale
// current-slot values (zero_cur) of u, v, w, theta and zeroes the mirror ring;
// group 1 adds into u, v, w and replaces qv, qc, qr.
template <typename T, int G>
__global__ void __launch_bounds__(AJ_THREADS, sizeof(T) == 4 ? 3 : 2)
    k_adj_advect(KParams<T> p, const T *__restrict__ coef, KFields<T> A, T step, T sdtg, int zero_cur)
{
    using C = AjCfg<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = (T *)smem_raw;
    const int ny = p.ny, nz = p.nz;
    // the level tiles of a column run next to each other: their rows share
    // DRAM lines, read once while all of them are resident
    const int i0 = blockIdx.y * AJ_TI, j0 = blockIdx.z * AJ_TJ, k0 = blockIdx.x * AJ_TK;
    constexpr int EQ0 = 3 * G;
    issue_tb<T, EQ0>(p, A, i0, j0, k0, sm + C::TB);
    issue_coef<T, EQ0, 0>(p, coef, i0, j0, k0, sm);
    cp_commit();
    // level factors of the z faces fk = k0-2 .. k0+TK: d(flux)/d(tendency)
    // below and above the face
    if (threadIdx.x < C::NZF) {
        const int fk = k0 - 2 + threadIdx.x;
        T z0 = T(0), z1 = T(0);
        if (fk >= 0 && fk <= nz - 2) {
            z0 = (p.dtz * p.mu[fk]) * p.rhow[fk + 1] * p.one_d_rhou[fk];
            z1 = (p.dtz * p.mu[fk + 1]) * p.rhow[fk + 1] * p.one_d_rhou[fk + 1];
        }
        sm[C::ZF + threadIdx.x] = z0;
        sm[C::ZF + C::NZF + threadIdx.x] = z1;
    }
    T acc[AJ_CPT][7];
#pragma unroll
    for (int r = 0; r < AJ_CPT; r++)
#pragma unroll
        for (int f = 0; f < 7; f++) acc[r][f] = T(0);
    adj_equation<T, G, EQ0>(p, coef, A, step, i0, j0, k0, sm, acc);
    adj_equation<T, G, EQ0 + 1>(p, coef, A, step, i0, j0, k0, sm, acc);
    adj_equation<T, G, EQ0 + 2>(p, coef, A, step, i0, j0, k0, sm, acc);
    // the fields this group gathers into
    constexpr int NG = G == 0 ? 4 : 6;
    constexpr int GF[2][6] = {{FU, FV, FW, FTH, -1, -1}, {FU, FV, FW, FQV, FQC, FQR}};
#pragma unroll
    for (int r = 0; r < AJ_CPT; r++) {
        const int e = threadIdx.x + r * AJ_THREADS;
        const int pi = i0 + e / (AJ_TK * AJ_TJ), pj = j0 + (e / AJ_TK) % AJ_TJ, pk = k0 + e % AJ_TK;
        if (pi >= p.nx || pj >= ny || pk >= nz) continue;
        T *a = acc[r];
        const int c = gix(ny, nz, pi, pj, pk);
        // buoyancy of w into theta (group 0) and the moisture loading (group 1)
        {
            T bw = T(0);
            if (adv_cell(p, pi, pj, pk, 2)) bw += A.P[FW][c];
            if (adv_cell(p, pi, pj, pk + 1, 2)) bw += A.P[FW][c + 1];
            if (bw != T(0)) {
                if (G == 0) {
                    a[FTH] += sdtg / p.tbv[pk] * bw;
                } else {
                    a[FQV] += sdtg * T(0.61) * bw;
                    a[FQC] -= sdtg * bw;
                    a[FQR] -= sdtg * bw;
                }
            }
        }
#pragma unroll
        for (int g = 0; g < NG; g++) {
            const int f = GF[G][g];
            const bool cell = adv_cell(p, pi, pj, pk, f == FW ? 2 : 1);
            const bool mine = G == 0 || f >= FQV;  // fields this group folds and replaces
            // (a clipped moisture point holds no P-bar: the fold adds zero)
            if (mine && cell) A.M[f][c] += A.P[f][c];
            if (mine && zero_cur && cell) A.cur[f][c] = a[f];
            else if (a[f] != T(0)) A.cur[f][c] += a[f];
        }
        if (G == 0 && pk >= 1 && pk <= nz - 2 && (pi == 0 || pi == p.nx - 1 || pj == 0 || pj == ny - 1)) {
            A.P[FU][c] = T(0);
            A.P[FV][c] = T(0);
            A.P[FW][c] = T(0);
        }
    }
}

// after the last stage of an adjoint run: the forward advection overwrote P
// on its cells, so their P-bar is zero
template <typename T>
__global__ void k_adj_zero_cells(KParams<T> p, KFields<T> A)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nzi = p.nz - 2, nyi = p.ny - 6, nxi = p.nx - 6;
    if (t >= (long)nxi * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 3 + (int)((t / nzi) % nyi);
    const int i = 3 + (int)(t / ((long)nzi * nyi));
    const int c = gix(p.ny, p.nz, i, j, k);
    const int nf = p.moist ? 7 : 4;
    for (int f = 0; f < nf; f++) {
        if (f == FW && k < 2) continue;
        A.P[f][c] = T(0);
    }
}

// ---------------------------------------------------------------------------
// transposes of the column post-processing (k_post): the M <- P copy of
// advance_outer, Rayleigh damping, the top/bottom conditions and the sponge
// strips, in reverse order, for u, v, w, theta.  Blocks own whole columns.
// ---------------------------------------------------------------------------
// AP_SPONGE2: the sponge twice (the step-final post and the last stage's post
// act on the same buffer back to back; the second top/bottom transpose is
// then the identity, so only the sponge repeats)
enum { AP_OUTER = 1, AP_RAYLEIGH = 2, AP_VBC = 4, AP_SPONGE = 8, AP_SPONGE2 = 16 };

template <typename T>
__device__ __forceinline__ T adj_post_pre(const KParams<T> &p, const KFields<T> &A, int f, int i, int j, int k,
                                          int flags)
{
    const int c = gix(p.ny, p.nz, i, j, k);
    T v = A.P[f][c];
    if (flags & AP_OUTER) v = v + A.M[f][c];
    if ((flags & AP_RAYLEIGH) && f <= FTH && i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1 && k >= p.raylevel) {
        const T cr = (f == FW) ? p.ray_w[k] : p.ray_u[k];
        v = v - cr * v;
    }
    return v;
}

template <typename T>
__global__ void __launch_bounds__(POST_THREADS) k_adj_post(KParams<T> p, KFields<T> A, int flags)
{
    const int nz = p.nz, nf = p.moist ? 7 : 4;
    const long c0 = (long)blockIdx.x * POST_COLS;
    T vals[7][POST_R];
#pragma unroll
    for (int r = 0; r < POST_R; ++r) {
        const int e = threadIdx.x + r * POST_THREADS;
        const int cl = e / nz, k = e - cl * nz;
        const long col = c0 + cl;
        if (cl >= POST_COLS || col >= (long)p.nx * p.ny) continue;
        const int i = (int)(col / p.ny), j = (int)(col % p.ny);
        const bool vbc = (flags & AP_VBC) && i >= 1 && j >= 1;
        const bool kin = k >= 1;
        const bool hE = kin && j >= 1 && i >= p.eb && i < p.ee;
        const bool hW = kin && j >= 1 && i >= p.wb && i < p.we;
        const bool hS = kin && i >= 1 && j >= p.sb && j < p.se;
        const bool hN = kin && i >= 1 && j >= p.nb && j < p.ne;
#pragma unroll
        for (int f = 0; f < 7; ++f) {
            if (f >= nf) break;
            T v = adj_post_pre(p, A, f, i, j, k, flags);
            if (vbc) {  // transposed boundaries.cpp:304-326
                if (f == FW) {
                    if (k == 0 || k == 1 || k == nz - 1) v = T(0);
                } else {
                    if (k == 0 || k == nz - 1) v = T(0);
                    else if (k == 1) v = v + adj_post_pre(p, A, f, i, j, 0, flags);
                    else if (k == nz - 2) v = v + adj_post_pre(p, A, f, i, j, nz - 1, flags);
                }
            }
            for (int rep = (flags & AP_SPONGE2) ? 2 : (flags & AP_SPONGE) ? 1 : 0; rep > 0; rep--) {
                if (hN) v = v - p.cn[j - p.nb] * v;
                if (hS) v = v - p.cs[j - p.sb] * v;
                if (hW) v = v - p.cw[i - p.wb] * v;
                if (hE) v = v - p.ce[i - p.eb] * v;
            }
            vals[f][r] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < POST_R; ++r) {
        const int e = threadIdx.x + r * POST_THREADS;
        const int cl = e / nz, k = e - cl * nz;
        const long col = c0 + cl;
        if (cl >= POST_COLS || col >= (long)p.nx * p.ny) continue;
        const int c = (int)col * nz + k;
#pragma unroll
        for (int f = 0; f < 7; ++f) {
            if (f >= nf) break;
            A.P[f][c] = vals[f][r];
            if (flags & AP_OUTER) A.M[f][c] = T(0);
        }
    }
}

// transpose of advance_outer's M <- P copy, every point: P-bar += M-bar,
// M-bar = 0
template <typename T>
__global__ void k_adj_fold_m(KParams<T> p, KFields<T> A)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const int nf = p.moist ? 7 : 4;
    for (int f = 0; f < nf; f++) {
        A.P[f][t] += A.M[f][t];
        A.M[f][t] = T(0);
    }
}

// The transposed column chain without the M fold: Rayleigh damping, the
// top/bottom copies, the sponge strips (once, or twice with AP_SPONGE2), in
// that order, for every linearised field.  One thread per (field, column)
// visits only the levels these operators change: every level of a
// sponge-strip column, otherwise levels 0, 1, NZ-2, NZ-1 and (Rayleigh) the
// damped levels.
template <typename T>
__global__ void k_adj_cols(KParams<T> p, KFields<T> A, int flags)
{
    // one thread per (field, column)
    const int nf = p.moist ? 7 : 4;
    const long ncols = (long)p.nx * p.ny;
    const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ncols * nf) return;
    const long col = tid % ncols;
    const int fsel = (int)(tid / ncols);
    const int nz = p.nz;
    const int i = (int)(col / p.ny), j = (int)(col % p.ny);
    const bool hE = j >= 1 && i >= p.eb && i < p.ee, hW = j >= 1 && i >= p.wb && i < p.we;
    const bool hS = i >= 1 && j >= p.sb && j < p.se, hN = i >= 1 && j >= p.nb && j < p.ne;
    const int reps = (flags & AP_SPONGE2) ? 2 : (flags & AP_SPONGE) ? 1 : 0;
    const bool strip = reps > 0 && (hE || hW || hS || hN);
    const bool vbc = (flags & AP_VBC) && i >= 1 && j >= 1;
    const bool rcol = (flags & AP_RAYLEIGH) && i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1;
    const long c0 = col * nz;
    for (int f = fsel; f <= fsel; f++) {
        T *P = A.P[f];
        const bool ray = rcol && f <= FTH;
        auto pre = [&](int k) {
            T v = P[c0 + k];
            if (ray && k >= p.raylevel) {
                const T cr = (f == FW) ? p.ray_w[k] : p.ray_u[k];
                v = v - cr * v;
            }
            return v;
        };
        const T vb = vbc ? pre(0) : T(0), vt = vbc ? pre(nz - 1) : T(0);
        // levels to visit: all (strip), else 0, 1 and from the first damped or
        // top-copy level up
        const int kup = strip ? 2 : min(nz - 2, ray ? max(p.raylevel, 2) : nz - 2);
        for (int k = 0; k < nz; k++) {
            if (!strip && k >= 2 && k < kup) k = kup;
            T v = pre(k);
            if (vbc) {
                if (f == FW) {
                    if (k == 0 || k == 1 || k == nz - 1) v = T(0);
                } else {
                    if (k == 0 || k == nz - 1) v = T(0);
                    else if (k == 1) v = v + vb;
                    else if (k == nz - 2) v = v + vt;
                }
            }
            if (strip && k >= 1)
                for (int rp = 0; rp < reps; rp++) {
                    if (hN) v = v - p.cn[j - p.nb] * v;
                    if (hS) v = v - p.cs[j - p.sb] * v;
                    if (hW) v = v - p.cw[i - p.wb] * v;
                    if (hE) v = v - p.ce[i - p.eb] * v;
                }
            P[c0 + k] = v;
        }
    }
}

// transposed projection (solver.cpp:120-135): pi-bar from P-bar of u, v, w.
// acc = 0 overwrites pi-bar (it is zero after every transposed solve).
template <typename T>
__global__ void k_adj_project(KParams<T> p, KFields<T> A, T step, int acc)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const int nz = p.nz, ny = p.ny, nx = p.nx;
    const int k = (int)(t % nz), j = (int)((t / nz) % ny), i = (int)(t / ((long)nz * ny));
    auto inner = [&](int a, int b, int c) { return a >= 1 && a <= nx - 2 && b >= 1 && b <= ny - 2 && c >= 1 && c <= nz - 2; };
    const int c = (int)t, sx = ny * nz, sy = nz;
    T v = acc ? A.pi[c] : T(0);
    if (inner(i, j, k)) {
        v -= step * p.dtx * A.P[FU][c];
        v -= step * p.dty * A.P[FV][c];
        if (k >= 2) v -= step * (p.dtz * p.mw[k]) * A.P[FW][c];
    }
    if (inner(i + 1, j, k)) v += step * p.dtx * A.P[FU][c + sx];
    if (inner(i, j + 1, k)) v += step * p.dty * A.P[FV][c + sy];
    if (inner(i, j, k + 1) && k + 1 >= 2) v += step * (p.dtz * p.mw[k + 1]) * A.P[FW][c + 1];
    A.pi[c] = v;
}

// Transposed placement of the pressure (the level copies of
// poisson_fft3d, pressure.cpp:878-892, and mirror_boundaries of PI) + forward
// FFT along y of the real result.  Block = (spectral row i, level tile).
template <typename T>
__global__ void k_adj_fft_y_in(KParams<T> p, const T *pib, typename V2<T>::t *spec, FftPlan pj,
                               const typename V2<T>::t *tw, int KT)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.nj * KT;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int i = blockIdx.y;
    const int k0 = 1 + blockIdx.x * KT;
    const int kt = min(KT, nz - 1 - k0);
    const bool ii = i >= 1 && i <= nx - 2;
    // several rows in flight per thread: the loads of a row do not wait for
    // the previous row's store
#pragma unroll 4
    for (int q = threadIdx.y; q < p.nj; q += blockDim.y)
        for (int l = threadIdx.x; l < KT; l += blockDim.x) {
            T2 v;
            v.x = T(0);
            v.y = T(0);
            if (l < kt) {
                const int k = k0 + l, j = q;
                T s = T(0);
                if (ii && j >= 1 && j <= ny - 2) {
                    s = pib[gix(ny, nz, i, j, k)];
                    if (i == 1) s += pib[gix(ny, nz, 0, j, k)];
                    if (i == nx - 2) s += pib[gix(ny, nz, nx - 1, j, k)];
                    if (j == 1 || j == ny - 2) {
                        const int jr = j == 1 ? 0 : ny - 1;
                        s += pib[gix(ny, nz, i, jr, k)];
                        if (i == 1) s += pib[gix(ny, nz, 0, jr, k)];
                        if (i == nx - 2) s += pib[gix(ny, nz, nx - 1, jr, k)];
                    }
                }
                if (k == 1) s += pib[gix(ny, nz, i, j, 0)];
                if (k == nz - 2) s += pib[gix(ny, nz, i, j, nz - 1)];
                v.x = s;
            }
            a[q * KT + l] = v;
        }
    __syncthreads();
    T2 *r = fft_smem<T, T2>(a, b, KT, pj, tw, false, KT);
    for (int q = threadIdx.y; q < p.nj; q += blockDim.y)
        for (int l = threadIdx.x; l < kt; l += blockDim.x) spec[((long)i * p.nj + q) * nz + k0 + l] = r[q * KT + l];
}

// inverse FFT along y and real part: the adjoint of the divergence field
// (with its lateral copies still folded in), real [i][j][k]
template <typename T>
__global__ void k_adj_ifft_y_out(KParams<T> p, const typename V2<T>::t *spec, T *dbar, FftPlan pj,
                                 const typename V2<T>::t *tw, int KT)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.nj * KT;
    const int nz = p.nz;
    const int i = blockIdx.y;
    const int k0 = 1 + blockIdx.x * KT;
    const int kt = min(KT, nz - 1 - k0);
    for (int q = threadIdx.y; q < p.nj; q += blockDim.y)
        for (int l = threadIdx.x; l < KT; l += blockDim.x)
            cp_elem(a + q * KT + l, spec + ((long)i * p.nj + q) * nz + k0 + min(l, kt - 1), l < kt);
    cp_wait_all_sync();
    T2 *r = fft_smem<T, T2>(a, b, KT, pj, tw, true, KT);
    for (int j = threadIdx.y; j < p.nj; j += blockDim.y)
        for (int l = threadIdx.x; l < kt; l += blockDim.x) dbar[gix(p.ny, nz, i, j, k0 + l)] = r[j * KT + l].x;
}

// Transposed Thomas solve of one wavenumber: M^T z = y / (ni nj), with M the
// tridiagonal matrix of pressure.cpp:834-871 (rows 1..K, K = NZ-2).  For the
// mean mode the forward pins x_K = 0 after elimination, which solves M' x = d'
// with row K replaced by x_K = 0 and d'_K = 0; its transpose solves
// M'^T z = y and then zeroes z_K.
template <typename T2, typename A>
__device__ void thomas_T_column(T2 *x, A *Fw, int nz, A hb, A inv_s, const A *rhou, const A *ac, const A *cc,
                                const A *vc, bool gauge)
{
    const int K = nz - 2;
    auto diag = [&](int k) { return (gauge && k == K) ? A(1) : rhou[k] * hb - vc[k]; };
    auto sup = [&](int k) { return (k >= K || (gauge && k == K - 1)) ? A(0) : ac[k + 1]; };
    A den = diag(1);
    A w = sup(1) / den;
    Fw[1] = w;
    A gr = (A)x[1].x * inv_s / den, gi = (A)x[1].y * inv_s / den;
    x[1].x = (decltype(x[1].x))gr;
    x[1].y = (decltype(x[1].y))gi;
    for (int k = 2; k <= K; k++) {
        const A sb = cc[k - 1];
        den = diag(k) - sb * w;
        w = sup(k) / den;
        Fw[k] = w;
        gr = ((A)x[k].x * inv_s - sb * gr) / den;
        gi = ((A)x[k].y * inv_s - sb * gi) / den;
        x[k].x = (decltype(x[k].x))gr;
        x[k].y = (decltype(x[k].y))gi;
    }
    for (int k = K - 1; k >= 1; k--) {
        gr = (A)x[k].x - Fw[k] * gr;
        gi = (A)x[k].y - Fw[k] * gi;
        x[k].x = (decltype(x[k].x))gr;
        x[k].y = (decltype(x[k].y))gi;
    }
    if (gauge) {
        x[K].x = 0;
        x[K].y = 0;
    }
}

// FP32 transposed solve of one wavenumber (not the mean mode): the recurrence
// of thomas_T_column with one reciprocal per level
__device__ __forceinline__ void thomas_T_column_fast(float2 *x, float *Fw, int nz, float hb, float inv_s,
                                                     const float *rhou, const float *ac, const float *cc,
                                                     const float *vc)
{
    const int K = nz - 2;
    float rb = __frcp_rn(rhou[1] * hb - vc[1]);
    float w = (1 < K) ? ac[2] * rb : 0.f;
    Fw[1] = w;
    float gr = x[1].x * inv_s * rb, gi = x[1].y * inv_s * rb;
    x[1] = make_float2(gr, gi);
    for (int k = 2; k <= K; k++) {
        const float sb = cc[k - 1];
        rb = __frcp_rn(rhou[k] * hb - vc[k] - sb * w);
        w = (k < K) ? ac[k + 1] * rb : 0.f;
        Fw[k] = w;
        gr = (x[k].x * inv_s - sb * gr) * rb;
        gi = (x[k].y * inv_s - sb * gi) * rb;
        x[k] = make_float2(gr, gi);
    }
    for (int k = K - 1; k >= 1; k--) {
        gr = x[k].x - Fw[k] * gr;
        gi = x[k].y - Fw[k] * gi;
        x[k] = make_float2(gr, gi);
    }
}

// FP64 solve of the transposed mean-mode system M'^T z = y / (ni nj) by
// parallel cyclic reduction across a warp (rows 1..nl), then z_K = 0 (see
// thomas_T_column).  wk as for pcr_column_f64.
template <typename T2>
__device__ void pcr_column_T_f64(T2 *x, int nl, double hcol, double dx2, double size2d, const double *rhou,
                                 const double *ac, const double *cc, const double *vc, double *wk)
{
    const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
    constexpr int R = PCR_ROWS;
    double *A0 = wk, *B0 = wk + R, *C0 = wk + 2 * R, *R0 = wk + 3 * R, *I0 = wk + 4 * R;
    double *A1 = wk + 5 * R, *B1 = wk + 6 * R, *C1 = wk + 7 * R, *R1 = wk + 8 * R, *I1 = wk + 9 * R;
    const int K = nl;
    for (int r = lane; r < R; r += 32) {
        if (r < nl) {
            const int k = r + 1;
            const double a = k >= 2 ? cc[k - 1] : 0.0;
            const double b = k == K ? 1.0 : rhou[k] * 2.0 * hcol / dx2 - vc[k];
            const double c = k < K - 1 ? ac[k + 1] : 0.0;
            A0[r] = a; B0[r] = b; C0[r] = c;
            R0[r] = (double)x[k].x / size2d;
            I0[r] = (double)x[k].y / size2d;
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
        v.x = (decltype(v.x))(r == nl - 1 ? 0.0 : R0[r] / B0[r]);
        v.y = (decltype(v.y))(r == nl - 1 ? 0.0 : I0[r] / B0[r]);
        x[r + 1] = v;
    }
    __syncwarp();
}

// transposed spectral step of one y-wavenumber q: forward FFT along x,
// transposed tridiagonal solves, inverse FFT along x (the adjoint of
// k_spectral_x has the same transform directions)
template <typename T>
__global__ void k_spectral_x_adj(KParams<T> p, typename V2<T>::t *spec, FftPlan pi, const typename V2<T>::t *tw,
                                 int ps)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    __shared__ T c_r[PPM_MAXZ], c_a[PPM_MAXZ], c_c[PPM_MAXZ], c_v[PPM_MAXZ];
    __shared__ double d_r[PPM_MAXZ], d_a[PPM_MAXZ], d_c[PPM_MAXZ], d_v[PPM_MAXZ];
    __shared__ double pcr_wk[PCR_WK];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.ni * ps;
    const int q = blockIdx.x;
    const int nl = p.nz - 2;
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
    T2 *fr = (r == a) ? b : a;
    const double size2d = (double)(p.ni * p.nj);
    if (sizeof(T) == 8) {
        for (int pp = tid; pp < p.ni; pp += nth) {
            const long col = (long)pp * p.nj + q;
            double *Fw = (double *)(fr + (long)pp * ps) - 1;
            thomas_T_column<T2, double>(r + (long)pp * ps - 1, Fw, p.nz, 2.0 * p.hcoef[col] / p.dx2, 1.0 / size2d, d_r,
                                        d_a, d_c, d_v, col == 0);
        }
    } else {
        const float dx2 = (float)p.dx2, inv_s = (float)(1.0 / size2d);
        for (int pp = tid; pp < p.ni; pp += nth) {
            const long col = (long)pp * p.nj + q;
            if (col == 0) continue;  // mean mode: FP64 below
            const float hb = 2.0f * (float)p.hcoef[col] / dx2;
            float *Fw = (float *)(fr + (long)pp * ps) - 1;
            thomas_T_column_fast((float2 *)(r + (long)pp * ps - 1), Fw, p.nz, hb, inv_s, (const float *)c_r,
                                 (const float *)c_a, (const float *)c_c, (const float *)c_v);
        }
        if (q == 0 && p.mean_inv) mean_mode_solve_T(r - 1, nl, p.mean_inv, size2d, pcr_wk);  // block-wide
        else if (q == 0 && tid < 32)
            pcr_column_T_f64(r - 1, nl, p.hcoef[0], p.dx2, size2d, d_r, d_a, d_c, d_v, pcr_wk);
    }
    __syncthreads();
    T2 *o = fft_smem<T, T2>(r, fr, nl, pi, tw, true, ps);
    for (int i = threadIdx.y; i < p.ni; i += blockDim.y)
        for (int l = threadIdx.x; l < nl; l += blockDim.x) spec[((long)i * p.nj + q) * p.nz + 1 + l] = o[i * ps + l];
}

// transposed solves of every wavenumber, TC columns per block staged through
// shared memory (one thread per column).  FP32 contexts solve the mean mode
// in FP64.
template <typename T>
__global__ void k_thomas_adj(KParams<T> p, typename V2<T>::t *spec, int TC)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    const int cs = p.nz | 1;
    T2 *xs = (T2 *)smem_raw;
    T *fs = (T *)(xs + (long)TC * cs);
    const long ncol = (long)p.ni * p.nj;
    const long c0 = (long)blockIdx.x * TC;
    const int nc = (int)min((long)TC, ncol - c0);
    T2 *g = spec + c0 * p.nz;
    for (int w = threadIdx.x; w < nc * p.nz; w += blockDim.x) cp_elem(xs + (w / p.nz) * cs + w % p.nz, g + w, true);
    cp_wait_all_sync();
    const double inv_s = 1.0 / (double)(p.ni * p.nj);
    const bool mean_block = sizeof(T) != 8 && c0 == 0 && p.mean_inv;  // the mean mode, block-wide below
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const long col = c0 + c;
        if (col == 0 && mean_block) continue;
        if (sizeof(T) == 8 || col == 0) {
            double Floc[PPM_MAXZ];
            thomas_T_column<T2, double>(xs + (long)c * cs, Floc, p.nz, 2.0 * p.hcoef[col] / p.dx2, inv_s, p.rhou_d,
                                        p.acoef_d, p.ccoef_d, p.vcoef_d, col == 0);
        } else {
            thomas_T_column<T2, T>(xs + (long)c * cs, fs + (long)c * cs, p.nz, (T)(2.0 * p.hcoef[col] / p.dx2),
                                   (T)inv_s, p.rhou, p.acoef, p.ccoef, p.vcoef, false);
        }
    }
    if (mean_block) {
        __shared__ double mwk[2 * PPM_MAXZ];
        mean_mode_solve_T(xs, p.nz - 2, p.mean_inv, (double)(p.ni * p.nj), mwk);
    }
    __syncthreads();
    for (int w = threadIdx.x; w < nc * p.nz; w += blockDim.x) g[w] = xs[(w / p.nz) * cs + w % p.nz];
}

// transposed divergence (divergence3d, pressure.cpp:1340-1381) with its
// lateral copies, then the transposed mirror_boundaries (boundaries.cpp:
// 363-379) of P u, v, w that preceded it: a point of the lateral ring (levels
// 1..NZ-2) passes its value to the interior point it copied, so every
// interior point gathers the ring points that mirror it.  Ring points are
// left as they are here and zeroed by k_adj_advect, which never reads them.
template <typename T>
__device__ __forceinline__ T adj_dint(const KParams<T> &p, const T *db, int a, int b, int c)
{
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    if (a < 1 || a > nx - 2 || b < 1 || b > ny - 2 || c < 1 || c > nz - 2) return T(0);
    T v = db[gix(ny, nz, a, b, c)];
    if (a == 1) v += db[gix(ny, nz, 0, b, c)];
    if (a == nx - 2) v += db[gix(ny, nz, nx - 1, b, c)];
    if (b == 1 || b == ny - 2) {
        const int br = b == 1 ? 0 : ny - 1;
        v += db[gix(ny, nz, a, br, c)];
        if (a == 1) v += db[gix(ny, nz, 0, br, c)];
        if (a == nx - 2) v += db[gix(ny, nz, nx - 1, br, c)];
    }
    return v;
}

// P-bar of u, v, w at (i,j,k) plus the transposed divergence there
template <typename T>
__device__ __forceinline__ void adj_div_point(const KParams<T> &p, const KFields<T> &A, const T *db, T sdt, int i,
                                              int j, int k, T &u, T &v, T &w)
{
    const int c = gix(p.ny, p.nz, i, j, k);
    const T d0 = adj_dint(p, db, i, j, k), dxm = adj_dint(p, db, i - 1, j, k);
    const T dym = adj_dint(p, db, i, j - 1, k), dzm = adj_dint(p, db, i, j, k - 1);
    u = A.P[FU][c];
    v = A.P[FV][c];
    w = A.P[FW][c];
    if (dxm != T(0) || d0 != T(0)) u += p.rhou[k] * p.one_d_dx * (dxm - d0) / sdt;
    if (dym != T(0) || d0 != T(0)) v += p.rhou[k] * p.one_d_dy * (dym - d0) / sdt;
    if (dzm != T(0) || d0 != T(0)) {
        T s = T(0);
        if (dzm != T(0)) s += p.mu[k - 1] * dzm;
        if (d0 != T(0)) s -= p.mu[k] * d0;
        w += p.rhow[k] * p.one_d_dz * s / sdt;
    }
}

template <typename T>
__global__ void k_adj_div(KParams<T> p, KFields<T> A, const T *db, T sdt)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const int nz = p.nz, ny = p.ny, nx = p.nx;
    const int k = (int)(t % nz), j = (int)((t / nz) % ny), i = (int)(t / ((long)nz * ny));
    const bool lev = k >= 1 && k <= nz - 2;
    if (lev && (i == 0 || i == nx - 1 || j == 0 || j == ny - 1)) return;
    T u, v, w;
    adj_div_point(p, A, db, sdt, i, j, k, u, v, w);
    if (lev) {
        const int is[2] = {i, i == 1 ? 0 : i == nx - 2 ? nx - 1 : -1};
        const int js[2] = {j, j == 1 ? 0 : j == ny - 2 ? ny - 1 : -1};
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 2; b++) {
                if ((a == 0 && b == 0) || is[a] < 0 || js[b] < 0) continue;
                T ru, rv, rw;
                adj_div_point(p, A, db, sdt, is[a], js[b], k, ru, rv, rw);
                u += ru;
                v += rv;
                w += rw;
            }
    }
    const int c = (int)t;
    A.P[FU][c] = u;
    A.P[FV][c] = v;
    A.P[FW][c] = w;
}

// a += b over n elements (tangent and adjoint bookkeeping)
template <typename T>
__global__ void k_axpy1(T *a, const T *b, long n)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] += b[t];
}

}  // namespace ga
