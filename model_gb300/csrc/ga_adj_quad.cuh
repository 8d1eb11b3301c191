// ---------------------------------------------------------------------------
// FP32 adjoint advection with four levels per thread: k_adj_advect's gather
// form on the same 16 x 8 x 8 tiles and the same cp.async pipeline, with one
// cell quad (a column, four consecutive levels) per thread and the face
// boxes laid out so that every shared-memory access of a quad is one 16-byte
// (or two 8-byte) operation.  Per level the arithmetic is k_adj_advect's,
// expression for expression.  NZ % 4 == 0.
//
// Row layouts (k fastest):
//   - x and y face boxes: levels k0 .. k0+7 (8 slots, copied as 16-byte quads);
//   - z face box and tendency box: levels k0-2 .. k0+9 (12 slots, copied as
//     8-byte level pairs; a pair that straddles a non-advected level of the
//     tendency box is copied as two 4-byte halves so that the zero fill stays
//     exact).
// ---------------------------------------------------------------------------
#pragma once
#include "ga_lin_kernels.cuh"
#include "ga_quad.cuh"

namespace ga {

constexpr int QJ_ZR = AJ_TK + 4;  // slots of a z-box / tendency-box row: levels k0-2 .. k0+TK+1
constexpr int QJ_BX = (AJ_TI + 5) * (AJ_TJ + 1) * AJ_TK;
constexpr int QJ_BY = (AJ_TI + 1) * (AJ_TJ + 5) * AJ_TK;
constexpr int QJ_BZ = (AJ_TI + 1) * (AJ_TJ + 1) * QJ_ZR;
constexpr int QJ_NFACE = QJ_BX > QJ_BY ? (QJ_BX > QJ_BZ ? QJ_BX : QJ_BZ) : (QJ_BY > QJ_BZ ? QJ_BY : QJ_BZ);
constexpr int QJ_NTB = AJ_BI * AJ_BJ * QJ_ZR;
static_assert(QJ_NFACE % 4 == 0 && QJ_NTB % 4 == 0, "16-byte aligned shared arrays");
static_assert(AJ_TI * AJ_TJ * (AJ_TK / 4) == AJ_THREADS, "one cell quad per thread");
static_assert(AJ_BK == QJ_ZR, "tendency rows hold levels k0-2 .. k0+TK+1");
// shared memory: coefficient boxes x2 (B+S, ab+a), fs1, fab, tendency boxes
// x2, level factors of the z faces
constexpr int QJ_CB = 0, QJ_FS = 4 * QJ_NFACE, QJ_FAB = 5 * QJ_NFACE, QJ_TB = 6 * QJ_NFACE,
              QJ_ZF = 6 * QJ_NFACE + 2 * QJ_NTB;
// then the basic-state term factors of the tile's levels (theta, qv; below
// and above the cell) and the Coriolis parameter of rows j0-1 .. j0+TJ
constexpr int QJ_BF = QJ_ZF + 2 * QJ_ZR, QJ_FC = QJ_BF + 4 * AJ_TK;
constexpr size_t QJ_SMEM = (size_t)(QJ_FC + AJ_TJ + 2) * sizeof(float);

template <int DIR>
struct QBox {
    static constexpr int bdi = DIR == 0 ? 3 : 0, bdj = DIR == 1 ? 3 : 0;
    static constexpr int bni = DIR == 0 ? AJ_TI + 5 : AJ_TI + 1;
    static constexpr int bnj = DIR == 1 ? AJ_TJ + 5 : AJ_TJ + 1;
    static constexpr int R = DIR == 2 ? QJ_ZR : AJ_TK;  // slots per row
    static constexpr int NCH = R / 4;                   // face quads per row
    static constexpr int rows = bni * bnj;
    static_assert(rows * R <= QJ_NFACE, "face box larger than its store");
};

__device__ __forceinline__ void cp16(float *dst, const float *src, bool ok)
{
    cp_elem(reinterpret_cast<float4 *>(dst), reinterpret_cast<const float4 *>(src), ok);
}
__device__ __forceinline__ void cp8(float *dst, const float *src, bool ok)
{
    cp_elem(reinterpret_cast<float2 *>(dst), reinterpret_cast<const float2 *>(src), ok);
}
__device__ __forceinline__ Q4 lds2x2(const float *a)  // 8-byte aligned quad
{
    const float2 x = *reinterpret_cast<const float2 *>(a), y = *reinterpret_cast<const float2 *>(a + 2);
    return Q4{{x.x, x.y, y.x, y.y}};
}

// the family's two coefficient boxes (zero off the domain)
template <int EQ, int DIR>
__device__ __forceinline__ void qj_issue_coef(const KParams<float> &p, const float *__restrict__ coef, int i0,
                                              int j0, int k0, float *cb)
{
    using B = QBox<DIR>;
    const float *ga_f = coef + (size_t)LinSlot<EQ, DIR>::GA * p.n, *gs_f = coef + (size_t)LinSlot<EQ, DIR>::GS * p.n;
    constexpr int NCP = DIR == 2 ? QJ_ZR / 2 : AJ_TK / 4;  // copies per row: level pairs (z) or quads
#pragma unroll 1
    for (int it = threadIdx.x; it < B::rows * NCP; it += AJ_THREADS) {
        const int r = it / NCP, ch = it % NCP;
        const int fi = i0 - B::bdi + r / B::bnj, fj = j0 - B::bdj + r % B::bnj;
        const bool row_ok = fi >= 0 && fi < p.nx && fj >= 0 && fj < p.ny;
        if (DIR == 2) {
            const int k = k0 - 2 + 2 * ch;
            const bool ok = row_ok && k >= 0 && k < p.nz;
            const int c = ok ? gix(p.ny, p.nz, fi, fj, k) : 0;
            cp8(cb + r * QJ_ZR + 2 * ch, ga_f + c, ok);
            cp8(cb + QJ_NFACE + r * QJ_ZR + 2 * ch, gs_f + c, ok);
        } else {
            const int k = k0 + 4 * ch;
            const bool ok = row_ok && k < p.nz;
            const int c = ok ? gix(p.ny, p.nz, fi, fj, k) : 0;
            cp16(cb + r * AJ_TK + 4 * ch, ga_f + c, ok);
            cp16(cb + QJ_NFACE + r * AJ_TK + 4 * ch, gs_f + c, ok);
        }
    }
}

// equation EQ's P-bar over the tendency box, zero off the advected cells
template <int EQ>
__device__ __forceinline__ void qj_issue_tb(const KParams<float> &p, const KFields<float> &A, int i0, int j0,
                                            int k0, float *tb)
{
    const float *P = A.P[LinEq<EQ>::FX];
    constexpr int NCP = QJ_ZR / 2;
#pragma unroll 1
    for (int it = threadIdx.x; it < AJ_BI * AJ_BJ * NCP; it += AJ_THREADS) {
        const int r = it / NCP, m = it % NCP;
        const int i = i0 - 3 + r / AJ_BJ, j = j0 - 3 + r % AJ_BJ, ka = k0 - 2 + 2 * m;
        const bool oka = adv_cell(p, i, j, ka, 1), okb = adv_cell(p, i, j, ka + 1, 1);
        float *dst = tb + r * QJ_ZR + 2 * m;
        if (oka == okb) {
            cp8(dst, P + (oka ? gix(p.ny, p.nz, i, j, ka) : 0), oka);
        } else {
            cp_elem(dst, P + (oka ? gix(p.ny, p.nz, i, j, ka) : 0), oka);
            cp_elem(dst + 1, P + (okb ? gix(p.ny, p.nz, i, j, ka + 1) : 0), okb);
        }
    }
}

// Coriolis of u into v and of v into u, the basic-state theta / qv term into
// w, for the thread's cell quad (adj_extra)
template <int EQ>
__device__ __forceinline__ void qj_extra(const KParams<float> &p, const float *tb, const float *sm, float step,
                                         int j0, int k0, int li, int lj, int lq, float (&acc)[4][7])
{
    auto row = [&](int di, int dj) { return tb + ((li + 3 + di) * AJ_BJ + (lj + 3 + dj)) * QJ_ZR; };
    if (EQ == 0 || EQ == 1) {
        const int di[4] = {0, 0, 1, 1}, dj[4] = {0, -1, 0, -1};
        const int ei[4] = {0, -1, 0, -1}, ej[4] = {0, 0, 1, 1};
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const int a = EQ == 0 ? di[n] : ei[n], b = EQ == 0 ? dj[n] : ej[n];
            const Q4 t = lds2x2(row(a, b) + 4 * lq + 2);
            const float fc = sm[QJ_FC + lj + 1 + b];  // fdt * f of row j0+lj+b
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float tv = step * t.v[e];
                if (tv != 0.f) {
                    if (EQ == 0) acc[e][FV] += fc * tv;
                    else acc[e][FU] -= fc * tv;
                }
            }
        }
    } else if (EQ == 2 || EQ == 3) {
        const float *bf = sm + QJ_BF + (EQ - 2) * 2 * AJ_TK;  // [below | above] x tile levels
        const float *rw = row(0, 0) + 4 * lq;
        const Q4 lo = lds4(rw), hi = lds4(rw + 4);
        const float w8[8] = {lo.v[0], lo.v[1], lo.v[2], lo.v[3], hi.v[0], hi.v[1], hi.v[2], hi.v[3]};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int lk = 4 * lq + e;
            const float t0 = step * w8[e + 1], t1 = step * w8[e + 2];
            if (t0 != 0.f) acc[e][FW] -= bf[lk] * t0;
            if (t1 != 0.f) acc[e][FW] -= bf[AJ_TK + lk] * t1;
        }
    }
}

template <int G, int EQ, int DIR>
__device__ __forceinline__ void qj_family(const KParams<float> &p, const float *__restrict__ coef,
                                          const KFields<float> &A, float step, int i0, int j0, int k0, float *sm,
                                          float (&acc)[4][7])
{
    using B = QBox<DIR>;
    constexpr int EQ0 = 3 * G, n = 3 * (EQ - EQ0) + DIR;
    constexpr bool HAS_NEXT = n < 8;
    constexpr int NEQ = DIR == 2 ? EQ + 1 : EQ, NDIR = (DIR + 1) % 3;
    constexpr int XF = LinEq<EQ>::FX;
    constexpr bool RAIN_Z = EQ == 5 && DIR == 2;
    const float *cga = sm + QJ_CB + (n % 2) * 2 * QJ_NFACE, *cgs = cga + QJ_NFACE;
    float *fs1 = sm + QJ_FS, *fab = sm + QJ_FAB;
    const float *tb = sm + QJ_TB + ((EQ - EQ0) % 2) * QJ_NTB;
    const float *zf0 = sm + QJ_ZF, *zf1 = zf0 + QJ_ZR;
    const int nz = p.nz, t = threadIdx.x;
    const int li = t >> 4, lj = (t >> 1) & 7, lq = t & 1;
    if (HAS_NEXT) qj_issue_coef<NEQ, NDIR>(p, coef, i0, j0, k0, sm + QJ_CB + ((n + 1) % 2) * 2 * QJ_NFACE);
    if (DIR == 0 && EQ < EQ0 + 2)
        qj_issue_tb<(EQ < EQ0 + 2 ? EQ + 1 : EQ)>(p, A, i0, j0, k0, sm + QJ_TB + ((EQ + 1 - EQ0) % 2) * QJ_NTB);
    cp_commit();
    cp_wait<1>();
    // the rain's fall-speed derivative at the thread's cells
    Q4 dvr{{0.f, 0.f, 0.f, 0.f}};
    if (RAIN_Z) {
        const int pi = i0 + li, pj = j0 + lj, pk0 = k0 + 4 * lq;
        if (pi < p.nx && pj < p.ny && pk0 < nz) dvr = ldg4(coef + (size_t)LIN_DVT_SLOT * p.n, gix(p.ny, nz, pi, pj, pk0));
    }
    __syncthreads();
    if (DIR == 0) qj_extra<EQ>(p, tb, sm, step, j0, k0, li, lj, lq, acc);
    // faces of the box, one face quad per item
#pragma unroll
    for (int q = 0; q < (B::rows * B::NCH + AJ_THREADS - 1) / AJ_THREADS; q++) {
        const int it = t + q * AJ_THREADS;
        if (it >= B::rows * B::NCH) break;
        const int r = it / B::NCH, ch = it % B::NCH;
        const int fi_l = r / B::bnj, fj_l = r % B::bnj;
        const int f = r * B::R + 4 * ch;
        const Q4 ga = lds4(cga + f), gs = lds4(cgs + f);
        Q4 t0, t1;
        if (DIR < 2) {
            const int r0 = (fi_l + 3 - B::bdi) * AJ_BJ + (fj_l + 3 - B::bdj);
            const int r1 = DIR == 0 ? r0 + AJ_BJ : r0 + 1;
            t0 = lds2x2(tb + r0 * QJ_ZR + 4 * ch + 2);
            t1 = lds2x2(tb + r1 * QJ_ZR + 4 * ch + 2);
        } else {
            const float *a = tb + ((fi_l + 3) * AJ_BJ + (fj_l + 3)) * QJ_ZR + 4 * ch;
            t0 = lds4(a);
            const float nx = ch < B::NCH - 1 ? a[4] : 0.f;  // the last slot is a padding face
            t1 = Q4{{t0.v[1], t0.v[2], t0.v[3], nx}};
        }
        Q4 s1, ab;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float a0 = step * t0.v[e], a1 = step * t1.v[e];
            float fb;
            if (DIR == 0) fb = p.dtx * (a1 - a0);
            else if (DIR == 1) fb = p.dty * (a1 - a0);
            else fb = zf1[4 * ch + e] * a1 - zf0[4 * ch + e] * a0;
            s1.v[e] = fb * gs.v[e];
            ab.v[e] = fb * ga.v[e];
        }
        sts4(fs1 + f, s1);
        sts4(fab + f, ab);
    }
    __syncthreads();
    const float C5[6] = {W<float>::c1_60, -W<float>::c2_15, W<float>::c37_60, W<float>::c37_60, -W<float>::c2_15,
                         W<float>::c1_60};
    const float U5[6] = {W<float>::c1_60, -5.f * W<float>::c1_60, 10.f * W<float>::c1_60, -10.f * W<float>::c1_60,
                         5.f * W<float>::c1_60, -W<float>::c1_60};
    const float C3[4] = {-W<float>::c1_12, W<float>::c7_12, W<float>::c7_12, -W<float>::c1_12};
    const float U3[4] = {-W<float>::c1_12, 3.f * W<float>::c1_12, -3.f * W<float>::c1_12, W<float>::c1_12};
    float gx[4] = {0.f, 0.f, 0.f, 0.f}, gav[4];
    if (DIR < 2) {
        const int bi = li + B::bdi, bj = lj + B::bdj;
        auto at = [&](int di, int dj) { return ((bi + di) * B::bnj + (bj + dj)) * AJ_TK + 4 * lq; };
#pragma unroll
        for (int m = 0; m < 6; m++) {
            const int w = DIR == 0 ? at(2 - m, 0) : at(0, 2 - m);
            const Q4 s = lds4(fs1 + w), g = lds4(cgs + w);
#pragma unroll
            for (int e = 0; e < 4; e++) gx[e] += C5[m] * s.v[e] + U5[m] * (g.v[e] > 0.f ? s.v[e] : -s.v[e]);
        }
        if (EQ == 0) {
            const Q4 a = lds4(fab + (DIR == 0 ? at(-1, 0) : at(0, -1))), b = lds4(fab + (DIR == 0 ? at(0, 0) : at(1, -1)));
#pragma unroll
            for (int e = 0; e < 4; e++) gav[e] = 0.5f * (a.v[e] + b.v[e]);
        } else if (EQ == 1) {
            const Q4 a = lds4(fab + (DIR == 0 ? at(-1, 0) : at(0, -1))), b = lds4(fab + (DIR == 0 ? at(-1, 1) : at(0, 0)));
#pragma unroll
            for (int e = 0; e < 4; e++) gav[e] = 0.5f * (a.v[e] + b.v[e]);
        } else {
            const Q4 a = lds4(fab + (DIR == 0 ? at(-1, 0) : at(0, -1)));
#pragma unroll
            for (int e = 0; e < 4; e++) gav[e] = a.v[e];
        }
    } else {
        // the z faces of the row at slots 4lq .. 4lq+7 (levels k0-2+4lq ..)
        const int rw = (li * B::bnj + lj) * QJ_ZR + 4 * lq;
        auto win = [&](const float *a, float (&o)[8]) {
            const Q4 x = lds4(a), y = lds4(a + 4);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                o[e] = x.v[e];
                o[4 + e] = y.v[e];
            }
        };
        float s8[8], g8[8], f8[8], h8[8];
        win(fs1 + rw, s8);
        win(cgs + rw, g8);
        win(fab + rw, f8);
        if (EQ == 0) win(fab + rw + B::bnj * QJ_ZR, h8);  // row i+1
        else if (EQ == 1) win(fab + rw + QJ_ZR, h8);     // row j+1
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int pk = k0 + 4 * lq + e;
#pragma unroll
            for (int d = -2; d <= 1; d++) {
                const int fk = pk + d;
                if (fk < (RAIN_Z ? 0 : 1) || fk > nz - 2) continue;
                const float s = s8[e + d + 2];
                if (fk <= 1 || fk == nz - 2) {  // 2nd order (and the rain's bottom outflow)
                    if (d == 0 || d == -1) gx[e] += 0.5f * s;
                } else {
                    const int m = 1 - d;
                    gx[e] += C3[m] * s + U3[m] * (g8[e + d + 2] > 0.f ? s : -s);
                }
            }
            if (EQ == 0 || EQ == 1) gav[e] = 0.5f * (f8[e + 1] + h8[e + 1]);
            else if (RAIN_Z) {
                gav[e] = pk >= 2 ? f8[e + 1] : 0.f;
                if (pk >= 1 && pk <= nz - 2) {
                    const float below = f8[e + 1] * (pk == 1 ? 2.f : 1.f);
                    gx[e] -= 0.5f * dvr.v[e] * (f8[e + 2] + below);
                }
            } else gav[e] = f8[e + 1];
        }
    }
#pragma unroll
    for (int e = 0; e < 4; e++) {
        acc[e][XF] += gx[e];
        acc[e][DIR] += gav[e];
    }
    __syncthreads();
}

template <int G, int EQ>
__device__ __forceinline__ void qj_equation(const KParams<float> &p, const float *__restrict__ coef,
                                            const KFields<float> &A, float step, int i0, int j0, int k0, float *sm,
                                            float (&acc)[4][7])
{
    qj_family<G, EQ, 0>(p, coef, A, step, i0, j0, k0, sm, acc);
    qj_family<G, EQ, 1>(p, coef, A, step, i0, j0, k0, sm, acc);
    qj_family<G, EQ, 2>(p, coef, A, step, i0, j0, k0, sm, acc);
}

// Group 0 (u, v, theta) and group 1 (qv, qc, qr), as k_adj_advect.
template <typename T, int G>
__global__ void __launch_bounds__(AJ_THREADS, 3)
    k_adj_advect_quad(KParams<T> p, const T *__restrict__ coef, KFields<T> A, T step, T sdtg, int zero_cur)
{
    static_assert(sizeof(T) == 4, "four-level kernels are FP32");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = (float *)smem_raw;
    const int ny = p.ny, nz = p.nz;
    const int i0 = blockIdx.y * AJ_TI, j0 = blockIdx.z * AJ_TJ, k0 = blockIdx.x * AJ_TK;
    constexpr int EQ0 = 3 * G;
    qj_issue_tb<EQ0>(p, A, i0, j0, k0, sm + QJ_TB);
    qj_issue_coef<EQ0, 0>(p, coef, i0, j0, k0, sm + QJ_CB);
    cp_commit();
    // level factors of the z faces fk = k0-2 .. k0+TK+1
    if (threadIdx.x < QJ_ZR) {
        const int fk = k0 - 2 + threadIdx.x;
        float z0 = 0.f, z1 = 0.f;
        if (fk >= 0 && fk <= nz - 2) {
            z0 = (p.dtz * p.mu[fk]) * p.rhow[fk + 1] * p.one_d_rhou[fk];
            z1 = (p.dtz * p.mu[fk + 1]) * p.rhow[fk + 1] * p.one_d_rhou[fk + 1];
        }
        sm[QJ_ZF + threadIdx.x] = z0;
        sm[QJ_ZF + QJ_ZR + threadIdx.x] = z1;
    }
    // the basic-state term of theta (G 0) or qv (G 1) into w: for the cell
    // at level pk, the factor of the tendency adjoint below and above it
    // (adj_extra's products, in its order, without the tendency)
    if (threadIdx.x >= 32 && threadIdx.x < 32 + 2 * AJ_TK) {
        const int h = (threadIdx.x - 32) / AJ_TK, lk = (threadIdx.x - 32) % AJ_TK, pk = k0 + lk;
        const float *base = G == 0 ? p.tb : p.qb;
        float v = 0.f;
        if (pk >= 1 && pk < nz && (G == 0 || p.moist)) {
            const int kk = h == 0 ? pk - 1 : pk;
            v = (p.dtz * p.mu[kk]) * 0.5f * p.rhow[pk] * (base[pk] - base[pk - 1]) * p.one_d_rhou[kk];
        }
        sm[QJ_BF + (G == 0 ? 0 : 2 * AJ_TK) + h * AJ_TK + lk] = v;
    }
    // fdt * f of rows j0-1 .. j0+TJ (Coriolis)
    if (threadIdx.x >= 64 && threadIdx.x < 64 + AJ_TJ + 2) {
        const int jj = j0 - 1 + (threadIdx.x - 64);
        sm[QJ_FC + threadIdx.x - 64] = jj >= 0 && jj < ny ? p.dt * 0.25f * p.f[jj] : 0.f;
    }
    float acc[4][7];
#pragma unroll
    for (int e = 0; e < 4; e++)
#pragma unroll
        for (int f = 0; f < 7; f++) acc[e][f] = 0.f;
    qj_equation<G, EQ0>(p, coef, A, step, i0, j0, k0, sm, acc);
    qj_equation<G, EQ0 + 1>(p, coef, A, step, i0, j0, k0, sm, acc);
    qj_equation<G, EQ0 + 2>(p, coef, A, step, i0, j0, k0, sm, acc);
    // epilogue on the thread's cell quad
    const int t = threadIdx.x, li = t >> 4, lj = (t >> 1) & 7, lq = t & 1;
    const int pi = i0 + li, pj = j0 + lj, pk0 = k0 + 4 * lq;
    if (pi >= p.nx || pj >= ny || pk0 >= nz) return;
    const int c = gix(ny, nz, pi, pj, pk0);
    constexpr int GF[2][6] = {{FU, FV, FW, FTH, -1, -1}, {FU, FV, FW, FQV, FQC, FQR}};
    // the fold and the gathered sums of field g from its loaded quads
    auto finish = [&](int g, Q4 cur, const Q4 &m0, const Q4 &pv) {
        const int f = GF[G][g];
        const bool mine = G == 0 || f >= FQV;  // fields this group folds and replaces
        if (mine) {
            Q4 m = m0;
            bool any = false;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                if (adv_cell(p, pi, pj, pk0 + e, f == FW ? 2 : 1)) {
                    m.v[e] += pv.v[e];
                    any = true;
                }
            }
            if (any) stg4(A.M[f] + c, m);
        }
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const bool cell = adv_cell(p, pi, pj, pk0 + e, f == FW ? 2 : 1);
            if (mine && zero_cur && cell) cur.v[e] = acc[e][f];
            else if (acc[e][f] != 0.f) cur.v[e] += acc[e][f];
        }
        stg4(A.cur[f] + c, cur);
    };
    // buoyancy of w into theta (group 0) and the moisture loading (group 1)
    auto buoyancy = [&](const Q4 &w4) {
        const float w5 = pk0 + 4 < nz ? A.P[FW][c + 4] : 0.f;
        const float wv[5] = {w4.v[0], w4.v[1], w4.v[2], w4.v[3], w5};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int pk = pk0 + e;
            float bw = 0.f;
            if (adv_cell(p, pi, pj, pk, 2)) bw += wv[e];
            if (adv_cell(p, pi, pj, pk + 1, 2)) bw += wv[e + 1];
            if (bw != 0.f) {
                if (G == 0) {
                    acc[e][FTH] += sdtg / p.tbv[pk] * bw;
                } else {
                    acc[e][FQV] += sdtg * 0.61f * bw;
                    acc[e][FQC] -= sdtg * bw;
                    acc[e][FQR] -= sdtg * bw;
                }
            }
        }
    };
    // every load of a batch of fields before its first store (a store would
    // otherwise order the later loads after it): group 0 in one batch, group 1
    // as u, v, w (sums only) and then qv, qc, qr
    if (G == 0) {
        Q4 cu[4], mm[4], pp[4];
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const int f = GF[G][g];
            cu[g] = ldg4(A.cur[f], c);
            mm[g] = ldg4(A.M[f], c);
            pp[g] = ldg4(A.P[f], c);
        }
        buoyancy(pp[2]);
#pragma unroll
        for (int g = 0; g < 4; g++) finish(g, cu[g], mm[g], pp[g]);
    } else {
        const Q4 z4{{0.f, 0.f, 0.f, 0.f}};
        {
            Q4 cu[3];
#pragma unroll
            for (int g = 0; g < 3; g++) cu[g] = ldg4(A.cur[GF[G][g]], c);
            buoyancy(ldg4(A.P[FW], c));
#pragma unroll
            for (int g = 0; g < 3; g++) finish(g, cu[g], z4, z4);
        }
        {
            Q4 cu[3], mm[3], pp[3];
#pragma unroll
            for (int g = 0; g < 3; g++) {
                const int f = GF[G][3 + g];
                cu[g] = ldg4(A.cur[f], c);
                mm[g] = ldg4(A.M[f], c);
                pp[g] = ldg4(A.P[f], c);
            }
#pragma unroll
            for (int g = 0; g < 3; g++) finish(3 + g, cu[g], mm[g], pp[g]);
        }
    }
    if (G == 0 && (pi == 0 || pi == p.nx - 1 || pj == 0 || pj == ny - 1)) {
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int pk = pk0 + e;
            if (pk >= 1 && pk <= nz - 2) {
                A.P[FU][c + e] = 0.f;
                A.P[FV][c + e] = 0.f;
                A.P[FW][c + e] = 0.f;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// k_lin_coef_quad: k_lin_coef for a cell quad per thread (FP32, NZ % 4 == 0,
// basic state a function of height).  The basic state's column values come
// from the basic-state table in shared memory; every face is lin_face_t's
// expression on the same values, so the coefficients are k_lin_coef's.
// ---------------------------------------------------------------------------
constexpr int LQ_THREADS = 256;

template <int EQ, int DIR>
__device__ __forceinline__ void lq_family(const KParams<float> &p, const KFields<float> &R, const float *tab,
                                          float *coef, int i, int j, int k0, int c)
{
    const int nz = p.nz, sx = p.ny * nz, sy = nz;
    constexpr int FX = LinEq<EQ>::FX, BX = LinEq<EQ>::BX;
    bool need[4], any = false;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int k = k0 + e;
        if (DIR == 0) need[e] = adv_cell(p, i, j, k, 1) || adv_cell(p, i + 1, j, k, 1);
        else if (DIR == 1) need[e] = adv_cell(p, i, j, k, 1) || adv_cell(p, i, j + 1, k, 1);
        else need[e] = adv_cell(p, i, j, k, 1) || (k + 1 < nz && adv_cell(p, i, j, k + 1, 1));
        any = any || need[e];
    }
    Q4 ga{{0.f, 0.f, 0.f, 0.f}}, gs{{0.f, 0.f, 0.f, 0.f}};
    if (any) {
        const float *X = R.cur[FX];
        if (EQ == 5 && DIR == 2) {
            // the rain's vertical face (lin_face_rain)
            const Win q = ldwin(X, c, k0, nz), w = ldwin(R.cur[FW], c, k0, nz);
            const int c0 = c - k0;
            float vt[5];
#pragma unroll
            for (int e = 0; e < 5; e++) {
                const int m = k0 + e;
                float v = 0.f;
                if (m < nz - 1) {
                    const int mm = m == 0 ? 1 : m;
                    v = fall_speed_point(p, q.at(mm - k0), mm);
                } else if (m < nz) {
                    v = R.vt[c0 + m];
                }
                vt[e] = v;
            }
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = k0 + e;
                if (!need[e]) continue;
                float Sv, wf;
                if (k == 0) {
                    const float v1 = vt[1 - k0];
                    Sv = 0.5f * (q.at(0) + q.at(1));
                    wf = -0.5f * (v1 + v1);
                } else {
                    const float wb = tab[2 * nz + k + 1] + w.at(e + 1);
                    wf = wb - 0.5f * (vt[e] + vt[e + 1]);
                    if (k == 1 || k == nz - 2) Sv = 0.5f * (q.at(e + 1) + q.at(e));
                    else Sv = face3<float>(q.at(e - 1), q.at(e), q.at(e + 1), q.at(e + 2), sgn(wf));
                }
                ga.v[e] = Sv;
                gs.v[e] = wf;
            }
        } else if (DIR < 2) {
            const int st = DIR == 0 ? sx : sy;
            Q4 x[6];
#pragma unroll
            for (int m = 0; m < 6; m++) x[m] = ldg4(X, c + (m - 2) * st);
            const float *A = R.cur[DIR];
            Q4 a0, a1;
            if (EQ >= 2) a0 = ldg4(A, c + st);
            else if (EQ == 0) {
                a0 = ldg4(A, DIR == 0 ? c + sx : c + sy);
                a1 = ldg4(A, DIR == 0 ? c : c - sx + sy);
            } else {
                a0 = ldg4(A, DIR == 0 ? c + sx : c + sy);
                a1 = ldg4(A, DIR == 0 ? c + sx - sy : c);
            }
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = k0 + e;
                if (!need[e]) continue;
                const float abv = tab[DIR * nz + k];
                float a, ab;
                if (EQ >= 2) {
                    a = a0.v[e];
                    ab = abv;
                } else {
                    a = 0.5f * (a0.v[e] + a1.v[e]);
                    ab = 0.5f * (abv + abv);
                }
                const float sgs = sgn(ab + a), sgb = sgn(a);
                const float Sv = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e], sgs);
                float Bv = 0.f;
                if (BX >= 0) {
                    const float b = tab[BX * nz + k];
                    Bv = face5<float>(b, b, b, b, b, b, sgb);
                }
                ga.v[e] = Bv + Sv;
                gs.v[e] = ab + a;
            }
        } else {
            const Win x = ldwin(X, c, k0, nz);
            const float *A = R.cur[FW];
            const Win w0 = ldwin(A, c, k0, nz);
            Win w1 = w0;
            if (EQ == 0) w1 = ldwin(A, c - sx, k0, nz);
            else if (EQ == 1) w1 = ldwin(A, c - sy, k0, nz);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = k0 + e;
                if (!need[e] || k == 0) continue;
                const float abv = tab[2 * nz + k + 1];
                float a, ab;
                if (EQ >= 2) {
                    a = w0.at(e + 1);
                    ab = abv;
                } else {
                    a = 0.5f * (w0.at(e + 1) + w1.at(e + 1));
                    ab = 0.5f * (abv + abv);
                }
                const float sgs = sgn(ab + a), sgb = sgn(a);
                float Sv, Bv = 0.f;
                if (k == 1 || k == nz - 2) {
                    Sv = 0.5f * (x.at(e + 1) + x.at(e));
                    if (BX >= 0) Bv = 0.5f * (tab[BX * nz + k + 1] + tab[BX * nz + k]);
                } else {
                    Sv = face3<float>(x.at(e - 1), x.at(e), x.at(e + 1), x.at(e + 2), sgs);
                    if (BX >= 0)
                        Bv = face3<float>(tab[BX * nz + k - 1], tab[BX * nz + k], tab[BX * nz + k + 1],
                                          tab[BX * nz + k + 2], sgb);
                }
                ga.v[e] = Bv + Sv;
                gs.v[e] = ab + a;
            }
        }
    }
    stg4(coef + (size_t)LinSlot<EQ, DIR>::GA * p.n + c, ga);
    if (LinSlot<EQ, DIR>::OWNS_GS) stg4(coef + (size_t)LinSlot<EQ, DIR>::GS * p.n + c, gs);
}

template <typename T>
__global__ void __launch_bounds__(LQ_THREADS)
    k_lin_coef_quad(KParams<T> p, KFields<T> R, T *coef, KFields<T> A, const unsigned char *qm)
{
    static_assert(sizeof(T) == 4, "four-level kernels are FP32");
    __shared__ float tab[5 * PPM_MAXZ];  // column values of UBAR, VBAR, WBAR, THBAR, QBAR
    const int nz = p.nz, NQ = nz >> 2;
    for (int e = threadIdx.x; e < 5 * nz; e += LQ_THREADS) tab[e] = p.btab[e];
    __syncthreads();
    const long w = (long)blockIdx.x * LQ_THREADS + threadIdx.x;
    if (w >= (long)p.nx * p.ny * NQ) return;
    const int q = (int)(w % NQ), col = (int)(w / NQ);
    const int j = col % p.ny, i = col / p.ny, k0 = 4 * q;
    const int c = gix(p.ny, nz, i, j, k0);
    lq_family<0, 0>(p, R, tab, coef, i, j, k0, c);
    lq_family<0, 1>(p, R, tab, coef, i, j, k0, c);
    lq_family<0, 2>(p, R, tab, coef, i, j, k0, c);
    lq_family<1, 0>(p, R, tab, coef, i, j, k0, c);
    lq_family<1, 1>(p, R, tab, coef, i, j, k0, c);
    lq_family<1, 2>(p, R, tab, coef, i, j, k0, c);
    lq_family<2, 0>(p, R, tab, coef, i, j, k0, c);
    lq_family<2, 1>(p, R, tab, coef, i, j, k0, c);
    lq_family<2, 2>(p, R, tab, coef, i, j, k0, c);
    if (p.moist) {
        lq_family<3, 0>(p, R, tab, coef, i, j, k0, c);
        lq_family<3, 1>(p, R, tab, coef, i, j, k0, c);
        lq_family<3, 2>(p, R, tab, coef, i, j, k0, c);
        lq_family<4, 0>(p, R, tab, coef, i, j, k0, c);
        lq_family<4, 1>(p, R, tab, coef, i, j, k0, c);
        lq_family<4, 2>(p, R, tab, coef, i, j, k0, c);
        lq_family<5, 0>(p, R, tab, coef, i, j, k0, c);
        lq_family<5, 1>(p, R, tab, coef, i, j, k0, c);
        lq_family<5, 2>(p, R, tab, coef, i, j, k0, c);
        // d(fall speed)/d(rain) (lin_dvt) and the clipped points' P-bar
        const bool inner = i >= 3 && i < p.nx - 3 && j >= 3 && j < p.ny - 3;
        const Q4 qr = ldg4(R.cur[FQR], c);
        Q4 dv{{0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int m = k0 + e;
            if (inner && m >= 1 && m <= nz - 2 && qr.v[e] > 1.0e-12f)
                dv.v[e] = 0.1364f * fall_speed_point(p, qr.v[e], m) / qr.v[e];
        }
        stg4(coef + (size_t)LIN_DVT_SLOT * p.n + c, dv);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const unsigned char b = qm[c + e];
            if (b && adv_cell(p, i, j, k0 + e, 1)) {
                if (b & 1) A.P[FQV][c + e] = 0.f;
                if (b & 2) A.P[FQC][c + e] = 0.f;
                if (b & 4) A.P[FQR][c + e] = 0.f;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// k_adj_div_quad: k_adj_div for a cell quad per thread (FP32, NZ % 4 == 0).
// Columns at least three points inside the lateral boundary involve no mirror
// copy: their four adj_dint terms are plain reads of db, done as 16-byte
// rows.  Other columns run adj_div_point level by level.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256, 4) k_adj_div_quad(KParams<T> p, KFields<T> A, const T *db, T sdt)
{
    static_assert(sizeof(T) == 4, "four-level kernels are FP32");
    const int nz = p.nz, ny = p.ny, nx = p.nx, NQ = nz >> 2;
    const long w = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= (long)nx * ny * NQ) return;
    const int q = (int)(w % NQ), col = (int)(w / NQ);
    const int j = col % ny, i = col / ny, k0 = 4 * q;
    const int c = gix(ny, nz, i, j, k0), sx = ny * nz, sy = nz;
    if (i >= 3 && i <= nx - 3 && j >= 3 && j <= ny - 3) {
        const Win d = ldwin(db, c, k0, nz);
        const Q4 dx = ldg4(db, c - sx), dy = ldg4(db, c - sy);
        Q4 u = ldg4(A.P[FU], c), v = ldg4(A.P[FV], c), wv = ldg4(A.P[FW], c);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            const bool lv = k >= 1 && k <= nz - 2, lvm = k - 1 >= 1 && k - 1 <= nz - 2;
            const float d0 = lv ? d.at(e) : 0.f, dxm = lv ? dx.v[e] : 0.f, dym = lv ? dy.v[e] : 0.f;
            const float dzm = lvm ? d.at(e - 1) : 0.f;
            if (dxm != 0.f || d0 != 0.f) u.v[e] += p.rhou[k] * p.one_d_dx * (dxm - d0) / sdt;
            if (dym != 0.f || d0 != 0.f) v.v[e] += p.rhou[k] * p.one_d_dy * (dym - d0) / sdt;
            if (dzm != 0.f || d0 != 0.f) {
                float s = 0.f;
                if (dzm != 0.f) s += p.mu[k - 1] * dzm;
                if (d0 != 0.f) s -= p.mu[k] * d0;
                wv.v[e] += p.rhow[k] * p.one_d_dz * s / sdt;
            }
        }
        stg4(A.P[FU] + c, u);
        stg4(A.P[FV] + c, v);
        stg4(A.P[FW] + c, wv);
        return;
    }
    for (int e = 0; e < 4; e++) {
        const int k = k0 + e;
        const bool lev = k >= 1 && k <= nz - 2;
        if (lev && (i == 0 || i == nx - 1 || j == 0 || j == ny - 1)) continue;
        float u, v, wz;
        adj_div_point(p, A, db, sdt, i, j, k, u, v, wz);
        if (lev) {
            const int is[2] = {i, i == 1 ? 0 : i == nx - 2 ? nx - 1 : -1};
            const int js[2] = {j, j == 1 ? 0 : j == ny - 2 ? ny - 1 : -1};
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int b = 0; b < 2; b++) {
                    if ((a == 0 && b == 0) || is[a] < 0 || js[b] < 0) continue;
                    float ru, rv, rw;
                    adj_div_point(p, A, db, sdt, is[a], js[b], k, ru, rv, rw);
                    u += ru;
                    v += rv;
                    wz += rw;
                }
        }
        A.P[FU][c + e] = u;
        A.P[FV][c + e] = v;
        A.P[FW][c + e] = wz;
    }
}

// ---------------------------------------------------------------------------
// k_adj_project_quad: k_adj_project for a cell quad per thread (FP32,
// NZ % 4 == 0): pi-bar from the projection's transposed gradient.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_adj_project_quad(KParams<T> p, KFields<T> A, T step, int acc)
{
    static_assert(sizeof(T) == 4, "four-level kernels are FP32");
    const int nz = p.nz, ny = p.ny, nx = p.nx, NQ = nz >> 2;
    const long w = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= (long)nx * ny * NQ) return;
    const int q = (int)(w % NQ), col = (int)(w / NQ);
    const int j = col % ny, i = col / ny, k0 = 4 * q;
    const int c = gix(ny, nz, i, j, k0), sx = ny * nz, sy = nz;
    const bool cin = i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2;        // column (i, j) inner
    const bool cxp = i + 1 >= 1 && i + 1 <= nx - 2 && j >= 1 && j <= ny - 2;  // column (i+1, j)
    const bool cyp = i >= 1 && i <= nx - 2 && j + 1 >= 1 && j + 1 <= ny - 2;  // column (i, j+1)
    const Q4 z{{0.f, 0.f, 0.f, 0.f}};
    Q4 v = acc ? ldg4(A.pi, c) : z;
    const Q4 pu = cin ? ldg4(A.P[FU], c) : z, pv = cin ? ldg4(A.P[FV], c) : z;
    const Win pw = cin ? ldwin(A.P[FW], c, k0, nz) : Win{};
    const Q4 pux = cxp ? ldg4(A.P[FU], c + sx) : z, pvy = cyp ? ldg4(A.P[FV], c + sy) : z;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int k = k0 + e;
        const bool lv = k >= 1 && k <= nz - 2, lvp = k + 1 >= 1 && k + 1 <= nz - 2;
        float x = v.v[e];
        if (cin && lv) {
            x -= step * p.dtx * pu.v[e];
            x -= step * p.dty * pv.v[e];
            if (k >= 2) x -= step * (p.dtz * p.mw[k]) * pw.at(e);
        }
        if (cxp && lv) x += step * p.dtx * pux.v[e];
        if (cyp && lv) x += step * p.dty * pvy.v[e];
        if (cin && lvp && k + 1 >= 2) x += step * (p.dtz * p.mw[k + 1]) * pw.at(e + 1);
        v.v[e] = x;
    }
    stg4(A.pi + c, v);
}

// ---------------------------------------------------------------------------
// k_adj_cols_quad: k_adj_cols (one (field, column) per thread, FP32,
// NZ % 4 == 0) on 16-byte level quads: a sponge-strip column goes through
// every quad, any other through quad 0 and the quads from its first damped
// or top-copy level up.  The transposed top and bottom copies couple levels
// 0 and 1, and NZ-2 and NZ-1, each pair inside one quad; on the levels of a
// visited quad that k_adj_cols would not visit the chain leaves the value
// as it is.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_adj_cols_quad(KParams<T> p, KFields<T> A, int flags)
{
    static_assert(sizeof(T) == 4, "four-level kernels are FP32");
    const int nf = p.moist ? 7 : 4, nz = p.nz, NQ = nz >> 2;
    const long ncols = (long)p.nx * p.ny;
    const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ncols * nf) return;
    const long col = tid % ncols;
    const int f = (int)(tid / ncols);
    const int i = (int)(col / p.ny), j = (int)(col % p.ny);
    const bool hE = j >= 1 && i >= p.eb && i < p.ee, hW = j >= 1 && i >= p.wb && i < p.we;
    const bool hS = i >= 1 && j >= p.sb && j < p.se, hN = i >= 1 && j >= p.nb && j < p.ne;
    const int reps = (flags & AP_SPONGE2) ? 2 : (flags & AP_SPONGE) ? 1 : 0;
    const bool strip = reps > 0 && (hE || hW || hS || hN);
    const bool vbc = (flags & AP_VBC) && i >= 1 && j >= 1;
    const bool rcol = (flags & AP_RAYLEIGH) && i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1;
    const bool ray = rcol && f <= FTH;
    if (!strip && !vbc && !ray) return;  // nothing changes in this column
    const int kup = strip ? 2 : min(nz - 2, ray ? max(p.raylevel, 2) : nz - 2);
    float *P = A.P[f] + col * nz;
    auto quad = [&](int k0) {
        const Q4 in = ldg4(P, k0);
        float pre[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            float v = in.v[e];
            if (ray && k >= p.raylevel) {
                const float cr = (f == FW) ? p.ray_w[k] : p.ray_u[k];
                v = v - cr * v;
            }
            pre[e] = v;
        }
        Q4 out;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            float v = pre[e];
            if (vbc) {
                if (f == FW) {
                    if (k == 0 || k == 1 || k == nz - 1) v = 0.f;
                } else {
                    if (k == 0 || k == nz - 1) v = 0.f;
                    else if (k == 1) v = v + pre[0];       // + pre(0): level 0 is in this quad
                    else if (k == nz - 2) v = v + pre[3];  // + pre(NZ-1): level NZ-1 is in this quad
                }
            }
            if (strip && k >= 1)
                for (int rp = 0; rp < reps; rp++) {
                    if (hN) v = v - p.cn[j - p.nb] * v;
                    if (hS) v = v - p.cs[j - p.sb] * v;
                    if (hW) v = v - p.cw[i - p.wb] * v;
                    if (hE) v = v - p.ce[i - p.eb] * v;
                }
            out.v[e] = v;
        }
        stg4(P + k0, out);
    };
    quad(0);
    for (int q = strip ? 1 : max(1, kup >> 2); q < NQ; q++) quad(4 * q);
}

}  // namespace ga
