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

// Build the face of equation eq (0 u, 1 v, 2 theta) and direction dir at
// (i,j,k) about the trajectory R (R.cur = fields at the start of the stage).
// Returns false where the forward flux is identically zero (bottom faces).
template <typename T>
__device__ __forceinline__ bool lin_face(const KParams<T> &p, const KFields<T> &R, int eq, int dir, int i, int j,
                                         int k, LinFace<T> &L)
{
    const int ny = p.ny, nz = p.nz;
    if (dir == 2 && k == 0) return false;
    const int fx = eq == 0 ? FU : eq == 1 ? FV : FTH;
    const T *X = R.cur[fx], *XB = R.bar[eq == 2 ? 3 : eq];
    const T *A = R.cur[dir], *AB = R.bar[dir];
    if (eq == 2) {
        L.ia0 = dir == 0 ? gix(ny, nz, i + 1, j, k) : dir == 1 ? gix(ny, nz, i, j + 1, k) : gix(ny, nz, i, j, k + 1);
        L.ia1 = -1;
    } else if (eq == 0) {
        if (dir == 0) { L.ia0 = gix(ny, nz, i + 1, j, k); L.ia1 = gix(ny, nz, i, j, k); }
        else if (dir == 1) { L.ia0 = gix(ny, nz, i, j + 1, k); L.ia1 = gix(ny, nz, i - 1, j + 1, k); }
        else { L.ia0 = gix(ny, nz, i, j, k + 1); L.ia1 = gix(ny, nz, i - 1, j, k + 1); }
    } else {
        if (dir == 0) { L.ia0 = gix(ny, nz, i + 1, j, k); L.ia1 = gix(ny, nz, i + 1, j - 1, k); }
        else if (dir == 1) { L.ia0 = gix(ny, nz, i, j + 1, k); L.ia1 = gix(ny, nz, i, j, k); }
        else { L.ia0 = gix(ny, nz, i, j, k + 1); L.ia1 = gix(ny, nz, i, j - 1, k + 1); }
    }
    T a, ab;
    if (L.ia1 < 0) {
        a = A[L.ia0];
        ab = AB[L.ia0];
    } else {
        a = T(0.5) * (A[L.ia0] + A[L.ia1]);
        ab = T(0.5) * (AB[L.ia0] + AB[L.ia1]);
    }
    const T sgs = sgn(ab + a), sgb = sgn(a);
    T Sv, Bv;
    if (dir < 2) {
        const int st = dir == 0 ? ny * nz : nz;
        const int c = gix(ny, nz, i, j, k) - 2 * st;
        L.x0 = c; L.xs = st; L.nx = 6;
        Sv = face5(X[c], X[c + st], X[c + 2 * st], X[c + 3 * st], X[c + 4 * st], X[c + 5 * st], sgs);
        Bv = face5(XB[c], XB[c + st], XB[c + 2 * st], XB[c + 3 * st], XB[c + 4 * st], XB[c + 5 * st], sgb);
    } else if (k == 1 || k == nz - 2) {
        const int c = gix(ny, nz, i, j, k);
        L.x0 = c; L.xs = 1; L.nx = 2;
        Sv = T(0.5) * (X[c + 1] + X[c]);
        Bv = T(0.5) * (XB[c + 1] + XB[c]);
    } else {
        const int c = gix(ny, nz, i, j, k) - 1;
        L.x0 = c; L.xs = 1; L.nx = 4;
        Sv = face3(X[c], X[c + 1], X[c + 2], X[c + 3], sgs);
        Bv = face3(XB[c], XB[c + 1], XB[c + 2], XB[c + 3], sgb);
    }
    L.sg = sgs;
    L.ga = Bv + Sv;
    L.gs = ab + a;
    return true;
}

// tangent of one face flux
template <typename T>
__device__ __forceinline__ T tl_face(const KParams<T> &p, const KFields<T> &R, const KFields<T> &D, int eq, int dir,
                                     int i, int j, int k)
{
    LinFace<T> L;
    if (!lin_face(p, R, eq, dir, i, j, k, L)) return T(0);
    const T *dA = D.cur[dir];
    const T *dX = D.cur[eq == 0 ? FU : eq == 1 ? FV : FTH];
    const T da = L.ia1 < 0 ? dA[L.ia0] : T(0.5) * (dA[L.ia0] + dA[L.ia1]);
    T ds;
    const int c = L.x0, st = L.xs;
    if (L.nx == 6) ds = face5(dX[c], dX[c + st], dX[c + 2 * st], dX[c + 3 * st], dX[c + 4 * st], dX[c + 5 * st], L.sg);
    else if (L.nx == 4) ds = face3(dX[c], dX[c + 1], dX[c + 2], dX[c + 3], L.sg);
    else ds = T(0.5) * (dX[c + 1] + dX[c]);
    return L.ga * da + L.gs * ds;
}

// tangent of the tendency of equation eq at a cell (u_tend_cell, v_tend_cell,
// theta_tend_cell with Z_ADVECT_BASE: advection.cpp:16-18, 73-122, 152-168)
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
    } else {
        const T *dW = D.cur[FW];
        const int c = gix(ny, nz, i, j, k);
        t -= DTZ * T(0.5) *
             (p.rhow[k + 1] * dW[c + 1] * (p.tb[k + 1] - p.tb[k]) + p.rhow[k] * dW[c] * (p.tb[k] - p.tb[k - 1])) *
             p.one_d_rhou[k];
    }
    return t;
}

// TLM of advect_uvw_velocity + advect_theta (advection.cpp:304-373): D.P =
// D.M + step * d(tendency) on the cells the forward step writes.
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
    if (k >= 2) {  // buoyancy_dry (advection.cpp:42-52, 329-337): linear in theta
        const T b0 = D.cur[FTH][c] / p.tbv[k], b1 = D.cur[FTH][c - 1] / p.tbv[k - 1];
        D.P[FW][c] = D.M[FW][c] + sdtg * (b0 + b1);
    }
}

// ---------------------------------------------------------------------------
// adjoint of the advection step, gather form.  A block owns a tile of
// AJ_TI x AJ_TJ x AJ_TK cells; for each of the nine face families (three
// equations x three directions) it evaluates the adjoint of every face whose
// stencil reaches the tile into shared memory (S' = Fbar*(ab+a), sign*S',
// a' = Fbar*(B+S)), then every cell sums what reaches it.
// ---------------------------------------------------------------------------
constexpr int AJ_TI = 8, AJ_TJ = 8, AJ_TK = 4, AJ_THREADS = AJ_TI * AJ_TJ * AJ_TK;
constexpr int AJ_NFACE = (AJ_TI + 1) * (AJ_TJ + 1) * (AJ_TK + 3);  // largest face box (z faces)

// adjoint of the tendency of equation eq at a cell (zero outside the cells
// the forward step writes)
template <typename T>
__device__ __forceinline__ T adj_tbar(const KParams<T> &p, const KFields<T> &A, int eq, int i, int j, int k, T step)
{
    if (!adv_cell(p, i, j, k, 1)) return T(0);
    return step * A.P[eq == 0 ? FU : eq == 1 ? FV : FTH][gix(p.ny, p.nz, i, j, k)];
}

// adjoint of the face flux (eq, dir) at (i,j,k): the transposed difference
// operator of the tendency
template <typename T>
__device__ __forceinline__ T adj_fbar(const KParams<T> &p, const KFields<T> &A, int eq, int dir, int i, int j, int k,
                                      T step)
{
    if (dir == 0) return p.dtx * (adj_tbar(p, A, eq, i + 1, j, k, step) - adj_tbar(p, A, eq, i, j, k, step));
    if (dir == 1) return p.dty * (adj_tbar(p, A, eq, i, j + 1, k, step) - adj_tbar(p, A, eq, i, j, k, step));
    if (k < 1) return T(0);
    T fb = T(0);
    const T t0 = adj_tbar(p, A, eq, i, j, k, step);
    if (t0 != T(0)) fb -= (p.dtz * p.mu[k]) * p.rhow[k + 1] * p.one_d_rhou[k] * t0;
    const T t1 = adj_tbar(p, A, eq, i, j, k + 1, step);
    if (t1 != T(0)) fb += (p.dtz * p.mu[k + 1]) * p.rhow[k + 1] * p.one_d_rhou[k + 1] * t1;
    return fb;
}

template <typename T>
__global__ void __launch_bounds__(AJ_THREADS) k_adj_advect(KParams<T> p, KFields<T> R, KFields<T> A, T step, T sdtg)
{
    __shared__ T fs1[AJ_NFACE], fs2[AJ_NFACE], fab[AJ_NFACE];
    const int ny = p.ny, nz = p.nz;
    const int i0 = blockIdx.x * AJ_TI, j0 = blockIdx.y * AJ_TJ, k0 = blockIdx.z * AJ_TK;
    const int t = threadIdx.x;
    const int lk = t % AJ_TK, lj = (t / AJ_TK) % AJ_TJ, li = t / (AJ_TK * AJ_TJ);
    const int pi = i0 + li, pj = j0 + lj, pk = k0 + lk;
    const bool own = pi < p.nx && pj < ny && pk < nz;
    // face-stencil weights: w(sign) = C + sign * U
    const T C5[6] = {W<T>::c1_60, -W<T>::c2_15, W<T>::c37_60, W<T>::c37_60, -W<T>::c2_15, W<T>::c1_60};
    const T U5[6] = {W<T>::c1_60, T(-5) * W<T>::c1_60, T(10) * W<T>::c1_60, T(-10) * W<T>::c1_60,
                     T(5) * W<T>::c1_60, -W<T>::c1_60};
    const T C3[4] = {-W<T>::c1_12, W<T>::c7_12, W<T>::c7_12, -W<T>::c1_12};
    const T U3[4] = {-W<T>::c1_12, T(3) * W<T>::c1_12, T(-3) * W<T>::c1_12, W<T>::c1_12};
    T acc[4] = {T(0), T(0), T(0), T(0)};  // u, v, w, theta
    for (int eq = 0; eq < 3; eq++) {
        const int xf = eq == 0 ? FU : eq == 1 ? FV : FTH;
        for (int dir = 0; dir < 3; dir++) {
            int bi0, bj0, bk0, bni, bnj, bnk;
            if (dir == 0) { bi0 = i0 - 3; bni = AJ_TI + 5; bj0 = j0; bnj = AJ_TJ + 1; bk0 = k0; bnk = AJ_TK; }
            else if (dir == 1) { bi0 = i0; bni = AJ_TI + 1; bj0 = j0 - 3; bnj = AJ_TJ + 5; bk0 = k0; bnk = AJ_TK; }
            else { bi0 = i0; bni = AJ_TI + 1; bj0 = j0; bnj = AJ_TJ + 1; bk0 = k0 - 2; bnk = AJ_TK + 3; }
            const int nf = bni * bnj * bnk;
            for (int f = t; f < nf; f += AJ_THREADS) {
                const int fk = bk0 + f % bnk, fj = bj0 + (f / bnk) % bnj, fi = bi0 + f / (bnk * bnj);
                T s1 = T(0), s2 = T(0), sa = T(0);
                const T fb = adj_fbar(p, A, eq, dir, fi, fj, fk, step);
                LinFace<T> L;
                if (fb != T(0) && lin_face(p, R, eq, dir, fi, fj, fk, L)) {
                    s1 = fb * L.gs;
                    s2 = L.nx == 2 ? T(0) : L.sg * s1;
                    sa = fb * L.ga;
                }
                fs1[f] = s1;
                fs2[f] = s2;
                fab[f] = sa;
            }
            __syncthreads();
            if (own) {
                auto at = [&](int fi, int fj, int fk) { return ((fi - bi0) * bnj + (fj - bj0)) * bnk + (fk - bk0); };
                T gx = T(0), ga = T(0);
                if (dir == 0) {
#pragma unroll
                    for (int m = 0; m < 6; m++) {
                        const int w = at(pi + 2 - m, pj, pk);
                        gx += C5[m] * fs1[w] + U5[m] * fs2[w];
                    }
                    if (eq == 0) ga = T(0.5) * (fab[at(pi - 1, pj, pk)] + fab[at(pi, pj, pk)]);
                    else if (eq == 1) ga = T(0.5) * (fab[at(pi - 1, pj, pk)] + fab[at(pi - 1, pj + 1, pk)]);
                    else ga = fab[at(pi - 1, pj, pk)];
                } else if (dir == 1) {
#pragma unroll
                    for (int m = 0; m < 6; m++) {
                        const int w = at(pi, pj + 2 - m, pk);
                        gx += C5[m] * fs1[w] + U5[m] * fs2[w];
                    }
                    if (eq == 0) ga = T(0.5) * (fab[at(pi, pj - 1, pk)] + fab[at(pi + 1, pj - 1, pk)]);
                    else if (eq == 1) ga = T(0.5) * (fab[at(pi, pj - 1, pk)] + fab[at(pi, pj, pk)]);
                    else ga = fab[at(pi, pj - 1, pk)];
                } else {
                    for (int fk = pk - 2; fk <= pk + 1; fk++) {
                        if (fk < 1 || fk > nz - 2) continue;
                        const int w = at(pi, pj, fk);
                        if (fk == 1 || fk == nz - 2) {
                            if (pk == fk || pk == fk + 1) gx += T(0.5) * fs1[w];
                        } else {
                            const int m = pk - (fk - 1);
                            gx += C3[m] * fs1[w] + U3[m] * fs2[w];
                        }
                    }
                    if (eq == 0) ga = T(0.5) * (fab[at(pi, pj, pk - 1)] + fab[at(pi + 1, pj, pk - 1)]);
                    else if (eq == 1) ga = T(0.5) * (fab[at(pi, pj, pk - 1)] + fab[at(pi, pj + 1, pk - 1)]);
                    else ga = fab[at(pi, pj, pk - 1)];
                }
                acc[xf] += gx;
                acc[dir] += ga;
            }
            __syncthreads();
        }
    }
    if (!own) return;
    // Coriolis terms of u and v (advection.cpp:84-92, 112-120)
    {
        const T fdt = p.dt * T(0.25);
        const int ci[4] = {pi, pi, pi + 1, pi + 1}, cj[4] = {pj, pj - 1, pj, pj - 1};
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const T tu = adj_tbar(p, A, 0, ci[n], cj[n], pk, step);
            if (tu != T(0)) acc[FV] += (fdt * p.f[cj[n]]) * tu;
        }
        const int di[4] = {pi, pi - 1, pi, pi - 1}, dj[4] = {pj, pj, pj + 1, pj + 1};
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const T tv = adj_tbar(p, A, 1, di[n], dj[n], pk, step);
            if (tv != T(0)) acc[FU] -= (fdt * p.f[dj[n]]) * tv;
        }
    }
    // vertical advection of the basic-state theta (Z_ADVECT_BASE) into w
    {
        const T t0 = adj_tbar(p, A, 2, pi, pj, pk - 1, step);
        const T t1 = adj_tbar(p, A, 2, pi, pj, pk, step);
        if (t0 != T(0))
            acc[FW] -= (p.dtz * p.mu[pk - 1]) * T(0.5) * p.rhow[pk] * (p.tb[pk] - p.tb[pk - 1]) * p.one_d_rhou[pk - 1] * t0;
        if (t1 != T(0))
            acc[FW] -= (p.dtz * p.mu[pk]) * T(0.5) * p.rhow[pk] * (p.tb[pk] - p.tb[pk - 1]) * p.one_d_rhou[pk] * t1;
    }
    // buoyancy of w into theta
    {
        const int c = gix(ny, nz, pi, pj, pk);
        T bw = T(0);
        if (adv_cell(p, pi, pj, pk, 2)) bw += A.P[FW][c];
        if (adv_cell(p, pi, pj, pk + 1, 2)) bw += A.P[FW][c + 1];
        if (bw != T(0)) acc[FTH] += sdtg / p.tbv[pk] * bw;
    }
    const int c = gix(ny, nz, pi, pj, pk);
#pragma unroll
    for (int f = 0; f < 4; f++)
        if (acc[f] != T(0)) A.cur[f][c] += acc[f];
}

// the forward advection overwrote P on its cells: M-bar += P-bar, P-bar = 0 there
template <typename T>
__global__ void k_adj_fold(KParams<T> p, KFields<T> A)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nzi = p.nz - 2, nyi = p.ny - 6, nxi = p.nx - 6;
    if (t >= (long)nxi * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 3 + (int)((t / nzi) % nyi);
    const int i = 3 + (int)(t / ((long)nzi * nyi));
    const int c = gix(p.ny, p.nz, i, j, k);
#pragma unroll
    for (int f = 0; f < 4; f++) {
        if (f == FW && k < 2) continue;
        A.M[f][c] += A.P[f][c];
        A.P[f][c] = T(0);
    }
}

// ---------------------------------------------------------------------------
// transposes of the column post-processing (k_post): the M <- P copy of
// advance_outer, Rayleigh damping, the top/bottom conditions and the sponge
// strips, in reverse order, for u, v, w, theta.  Blocks own whole columns.
// ---------------------------------------------------------------------------
enum { AP_OUTER = 1, AP_RAYLEIGH = 2, AP_VBC = 4, AP_SPONGE = 8 };

template <typename T>
__device__ __forceinline__ T adj_post_pre(const KParams<T> &p, const KFields<T> &A, int f, int i, int j, int k,
                                          int flags)
{
    const int c = gix(p.ny, p.nz, i, j, k);
    T v = A.P[f][c];
    if (flags & AP_OUTER) v = v + A.M[f][c];
    if ((flags & AP_RAYLEIGH) && i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1 && k >= p.raylevel) {
        const T cr = (f == FW) ? p.ray_w[k] : p.ray_u[k];
        v = v - cr * v;
    }
    return v;
}

template <typename T>
__global__ void __launch_bounds__(POST_THREADS) k_adj_post(KParams<T> p, KFields<T> A, int flags)
{
    const int nz = p.nz;
    const long c0 = (long)blockIdx.x * POST_COLS;
    T vals[4][POST_R];
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
        for (int f = 0; f < 4; ++f) {
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
            if (flags & AP_SPONGE) {
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
        for (int f = 0; f < 4; ++f) {
            A.P[f][c] = vals[f][r];
            if (flags & AP_OUTER) A.M[f][c] = T(0);
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
    const int i = blockIdx.x;
    const int k0 = 1 + blockIdx.y * KT;
    const int kt = min(KT, nz - 1 - k0);
    const bool ii = i >= 1 && i <= nx - 2;
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
    const int i = blockIdx.x;
    const int k0 = 1 + blockIdx.y * KT;
    const int kt = min(KT, nz - 1 - k0);
    for (int q = threadIdx.y; q < p.nj; q += blockDim.y)
        for (int l = threadIdx.x; l < KT; l += blockDim.x) {
            T2 v;
            v.x = T(0);
            v.y = T(0);
            if (l < kt) v = spec[((long)i * p.nj + q) * nz + k0 + l];
            a[q * KT + l] = v;
        }
    __syncthreads();
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
    for (int w = threadIdx.x; w < nc * p.nz; w += blockDim.x) xs[(w / p.nz) * cs + w % p.nz] = g[w];
    __syncthreads();
    const double inv_s = 1.0 / (double)(p.ni * p.nj);
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const long col = c0 + c;
        if (sizeof(T) == 8 || col == 0) {
            double Floc[PPM_MAXZ];
            thomas_T_column<T2, double>(xs + (long)c * cs, Floc, p.nz, 2.0 * p.hcoef[col] / p.dx2, inv_s, p.rhou_d,
                                        p.acoef_d, p.ccoef_d, p.vcoef_d, col == 0);
        } else {
            thomas_T_column<T2, T>(xs + (long)c * cs, fs + (long)c * cs, p.nz, (T)(2.0 * p.hcoef[col] / p.dx2),
                                   (T)inv_s, p.rhou, p.acoef, p.ccoef, p.vcoef, false);
        }
    }
    __syncthreads();
    for (int w = threadIdx.x; w < nc * p.nz; w += blockDim.x) g[w] = xs[(w / p.nz) * cs + w % p.nz];
}

// transposed divergence (divergence3d, pressure.cpp:1340-1381) with its
// lateral copies: adds to P-bar of u, v, w at every point
template <typename T>
__global__ void k_adj_div(KParams<T> p, KFields<T> A, const T *db, T sdt)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const int nz = p.nz, ny = p.ny, nx = p.nx;
    const int k = (int)(t % nz), j = (int)((t / nz) % ny), i = (int)(t / ((long)nz * ny));
    auto dint = [&](int a, int b, int c) -> T {
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
    };
    const T d0 = dint(i, j, k), dxm = dint(i - 1, j, k), dym = dint(i, j - 1, k), dzm = dint(i, j, k - 1);
    const int c = (int)t;
    if (dxm != T(0) || d0 != T(0)) A.P[FU][c] += p.rhou[k] * p.one_d_dx * (dxm - d0) / sdt;
    if (dym != T(0) || d0 != T(0)) A.P[FV][c] += p.rhou[k] * p.one_d_dy * (dym - d0) / sdt;
    if (dzm != T(0) || d0 != T(0)) {
        T v = T(0);
        if (dzm != T(0)) v += p.mu[k - 1] * dzm;
        if (d0 != T(0)) v -= p.mu[k] * d0;
        A.P[FW][c] += p.rhow[k] * p.one_d_dz * v / sdt;
    }
}

// transposed mirror_boundaries (boundaries.cpp:363-379) of up to three
// fields, in place: block = one level; the j copies were applied last, so
// their transpose runs first
template <typename T>
__global__ void k_adj_mirror(KParams<T> p, T *a0, T *a1, T *a2)
{
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int k = 1 + blockIdx.x;
    T *fl[3] = {a0, a1, a2};
    for (int n = 0; n < 3; n++) {
        T *a = fl[n];
        if (!a) continue;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) {
            a[gix(ny, nz, i, 1, k)] += a[gix(ny, nz, i, 0, k)];
            a[gix(ny, nz, i, 0, k)] = T(0);
            a[gix(ny, nz, i, ny - 2, k)] += a[gix(ny, nz, i, ny - 1, k)];
            a[gix(ny, nz, i, ny - 1, k)] = T(0);
        }
        __syncthreads();
        for (int j = threadIdx.x; j < ny; j += blockDim.x) {
            a[gix(ny, nz, 1, j, k)] += a[gix(ny, nz, 0, j, k)];
            a[gix(ny, nz, 0, j, k)] = T(0);
            a[gix(ny, nz, nx - 2, j, k)] += a[gix(ny, nz, nx - 1, j, k)];
            a[gix(ny, nz, nx - 1, j, k)] = T(0);
        }
        __syncthreads();
    }
}

// a += b over n elements (tangent and adjoint bookkeeping)
template <typename T>
__global__ void k_axpy1(T *a, const T *b, long n)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] += b[t];
}

}  // namespace ga
