// ---------------------------------------------------------------------------
// FP32 kernels with four levels per thread: a work item is one column and one
// aligned quad of levels k0..k0+3, read and written as 16-byte rows.  NZ is a
// multiple of 4.
//
// k_advect_quad: advection (advection.cpp:304-497 with the face fluxes of
// fluxes.cpp) for a horizontally uniform basic state.
//
// A block owns TI x TJ interior columns at every level, as k_advect_tile
// does, but a work item is one column and one aligned quad of levels
// k0..k0+3: each stencil row is one 16-byte load, and the index arithmetic is
// paid once per four levels.  The six flux fields go in three passes of two
// (u and v; theta and qv; qc and qr), so only two fields' face columns are in
// shared memory at a time.  Per level the arithmetic is that of the
// k_advect_tile face and tendency functions, expression for expression.
// Levels outside a face's or a cell's range are computed on padding values
// and never stored.
// ---------------------------------------------------------------------------
#pragma once
#include "ga_kernels.cuh"
#include "ga_tma.cuh"

#include <cooperative_groups.h>

namespace ga {

constexpr int AQ_THREADS = 256;
constexpr int AQ_LV = 7;  // staged level arrays: mu, rhow, one_d_rhou, tb, qb, tbv, rhou

template <int TI, int TJ>
struct AQGeom {
    static constexpr int CE = (TI + 1) * TJ;  // east-face columns: i0-1 .. i0+TI-1
    static constexpr int CN = TI * (TJ + 1);  // north-face columns: j0-1 .. j0+TJ-1
    static constexpr int CT = TI * TJ;        // top faces, and the cells
    static constexpr int CF = CE + CN + CT;   // face columns of one field
};

// two field slots of face columns, the basic-state table, the level arrays
__host__ __device__ constexpr size_t advect_quad_smem(int ti, int tj, int nz)
{
    return (2 * (size_t)((ti + 1) * tj + ti * (tj + 1) + ti * tj) * nz + (size_t)BT_COUNT * nz +
            (size_t)AQ_LV * nz) *
           sizeof(float);
}

struct Q4 {
    float v[4];
};
__device__ __forceinline__ Q4 ldg4(const float *a, int idx)
{
    const float4 t = __ldg(reinterpret_cast<const float4 *>(a + idx));
    return Q4{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ Q4 lds4(const float *a)
{
    const float4 t = *reinterpret_cast<const float4 *>(a);
    return Q4{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ void sts4(float *a, const Q4 &q)
{
    *reinterpret_cast<float4 *>(a) = make_float4(q.v[0], q.v[1], q.v[2], q.v[3]);
}
__device__ __forceinline__ void stg4(float *a, const Q4 &q)
{
    *reinterpret_cast<float4 *>(a) = make_float4(q.v[0], q.v[1], q.v[2], q.v[3]);
}
// a column window of 12 levels k0-4 .. k0+7 (zero outside the column)
struct Win {
    float v[12];
    __device__ __forceinline__ float at(int d) const { return v[4 + d]; }  // level k0 + d
};
__device__ __forceinline__ Win ldwin(const float *a, int c, int k0, int nz)
{
    Win w;
    const Q4 lo = k0 >= 4 ? ldg4(a, c - 4) : Q4{{0.f, 0.f, 0.f, 0.f}};
    const Q4 mi = ldg4(a, c);
    const Q4 hi = k0 + 4 < nz ? ldg4(a, c + 4) : Q4{{0.f, 0.f, 0.f, 0.f}};
#pragma unroll
    for (int e = 0; e < 4; e++) {
        w.v[e] = lo.v[e];
        w.v[4 + e] = mi.v[e];
        w.v[8 + e] = hi.v[e];
    }
    return w;
}

// field kinds of the passes: 0 u, 1 v, 2 theta, 3 qv, 4 qc, 5 qr, and with
// the ice scheme 6 snow, 7 cloud ice (5-7 fall with their fall speeds)
__host__ __device__ constexpr int aq_field(int fk)
{
    return fk == 0 ? FU : fk == 1 ? FV : fk == 2 ? FTH : fk == 3 ? FQV : fk == 4 ? FQC : fk == 5 ? FQR
           : fk == 6 ? FQS : FQI;
}
// basic-state row of a scalar (brow of s_*_ub): 0 theta, 1 qv, -1 none
__host__ __device__ constexpr int aq_brow(int fk) { return fk == 2 ? 0 : fk == 3 ? 1 : -1; }

// Where the current fields are read from.  at(i, j, k0) is the index of a
// column quad; ld4 / win read the quad or the 12-level window of field f at
// column offset (di, dj) from it.
//
// GSrc: the fields in global memory, through the read-only path.
struct GSrc {
    const KFields<float> &F;
    int ny, nz, sx, sy;
    __device__ __forceinline__ GSrc(const KFields<float> &F_, int ny_, int nz_)
        : F(F_), ny(ny_), nz(nz_), sx(ny_ * nz_), sy(nz_) {}
    __device__ __forceinline__ int at(int i, int j, int k0) const { return gix(ny, nz, i, j, k0); }
    __device__ __forceinline__ Q4 ld4(int f, int c, int di, int dj) const
    {
        return ldg4(F.cur[f], c + di * sx + dj * sy);
    }
    __device__ __forceinline__ Win win(int f, int c, int di, int dj, int k0) const
    {
        return ldwin(F.cur[f], c + di * sx + dj * sy, k0, nz);
    }
    // stored fall speed (array a) at level k0 + e of column (i, j)
    __device__ __forceinline__ float vt(const float *a, int i, int j, int k0, int c, int e) const { return a[c + e]; }
};

// SSrc: halo boxes of the fields in shared memory, [i][j][k] with BJ x BK
// floats per i, the box of field f at base + f * fs, origin (oi, oj, ok) in
// global coordinates.  Points outside the field hold zeros, as the windows of
// GSrc do.
template <int BJ, int BK>
struct SSrc {
    const KFields<float> &F;
    const float *base;
    int fs, oi, oj, ok, ny, nz;
    __device__ __forceinline__ int at(int i, int j, int k0) const { return ((i - oi) * BJ + (j - oj)) * BK + k0 - ok; }
    __device__ __forceinline__ Q4 ld4(int f, int c, int di, int dj) const
    {
        return lds4(base + f * fs + c + (di * BJ + dj) * BK);
    }
    __device__ __forceinline__ Win win(int f, int c, int di, int dj, int k0) const
    {
        const float *a = base + f * fs + c + (di * BJ + dj) * BK;
        // the top faces of the quad below a slab (only its last level is
        // used) would read levels below the box: zeros, as below the column
        const Q4 lo = k0 - 4 >= ok ? lds4(a - 4) : Q4{{0.f, 0.f, 0.f, 0.f}};
        const Q4 mi = lds4(a), hi = lds4(a + 4);
        Win w;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            w.v[e] = lo.v[e];
            w.v[4 + e] = mi.v[e];
            w.v[8 + e] = hi.v[e];
        }
        return w;
    }
    __device__ __forceinline__ float vt(const float *a, int i, int j, int k0, int c, int e) const
    {
        return a[gix(ny, nz, i, j, k0) + e];
    }
};

// east face (between i and i+1) at levels k0..k0+3: u_east_ub, v_east_ub, s_east_ub
template <int FK, class S>
__device__ __forceinline__ Q4 aq_east(const KParams<float> &p, const S &src, const float *tab, int i, int j, int k0)
{
    const int nz = p.nz;
    const int c = src.at(i, j, k0);
    constexpr int XF = aq_field(FK);
    Q4 x[6];
#pragma unroll
    for (int m = 0; m < 6; m++) x[m] = src.ld4(XF, c, m - 2, 0);
    Q4 r;
    if (FK == 0) {
        const Q4 up = src.ld4(FU, c, 1, 0), u0 = src.ld4(FU, c, 0, 0), uba = lds4(tab + BT_UA * nz + k0),
                 c6 = lds4(tab + BT_C6_UB * nz + k0);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float ua = 0.5f * (up.v[e] + u0.v[e]);
            const float ue = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                          sgn(uba.v[e] + ua));
            r.v[e] = ua * c6.v[e] + (uba.v[e] + ua) * ue;
        }
    } else if (FK == 1) {
        const Q4 ua_ = src.ld4(FU, c, 1, 0), ub_ = src.ld4(FU, c, 1, -1), uba = lds4(tab + BT_UA * nz + k0),
                 c6 = lds4(tab + BT_C6_VB * nz + k0);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float ua = 0.5f * (ua_.v[e] + ub_.v[e]);
            const float ve = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                          sgn(uba.v[e] + ua));
            r.v[e] = ua * c6.v[e] + (uba.v[e] + ua) * ve;
        }
    } else {
        constexpr int BR = aq_brow(FK);
        const Q4 u1 = src.ld4(FU, c, 1, 0), ub = lds4(tab + BT_UB * nz + k0);
        const Q4 c6 = BR >= 0 ? lds4(tab + (BT_C6_THB + BR) * nz + k0) : Q4{{0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float ut = ub.v[e] + u1.v[e];
            const float se = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                          sgn(ut));
            if (BR < 0) r.v[e] = ut * se;
            else r.v[e] = u1.v[e] * c6.v[e] + ut * se;
        }
    }
    return r;
}

// north face (between j and j+1): u_north_ub, v_north_ub, s_north_ub
template <int FK, class S>
__device__ __forceinline__ Q4 aq_north(const KParams<float> &p, const S &src, const float *tab, int i, int j, int k0)
{
    const int nz = p.nz;
    const int c = src.at(i, j, k0);
    constexpr int XF = aq_field(FK);
    Q4 x[6];
#pragma unroll
    for (int m = 0; m < 6; m++) x[m] = src.ld4(XF, c, 0, m - 2);
    Q4 r;
    if (FK == 0) {
        const Q4 va_ = src.ld4(FV, c, 0, 1), vb_ = src.ld4(FV, c, -1, 1), vba = lds4(tab + BT_VA * nz + k0),
                 c6 = lds4(tab + BT_C6_UB * nz + k0);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float va = 0.5f * (va_.v[e] + vb_.v[e]);
            const float un = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                          sgn(vba.v[e] + va));
            r.v[e] = va * c6.v[e] + (vba.v[e] + va) * un;
        }
    } else if (FK == 1) {
        const Q4 vp = src.ld4(FV, c, 0, 1), v0 = src.ld4(FV, c, 0, 0), vba = lds4(tab + BT_VA * nz + k0),
                 c6 = lds4(tab + BT_C6_VB * nz + k0);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float va = 0.5f * (vp.v[e] + v0.v[e]);
            const float vn = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                          sgn(vba.v[e] + va));
            r.v[e] = va * c6.v[e] + (vba.v[e] + va) * vn;
        }
    } else {
        constexpr int BR = aq_brow(FK);
        const Q4 v1 = src.ld4(FV, c, 0, 1), vb = lds4(tab + BT_VB * nz + k0);
        const Q4 c6 = BR >= 0 ? lds4(tab + (BT_C6_THB + BR) * nz + k0) : Q4{{0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float vt = vb.v[e] + v1.v[e];
            const float sn = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                          sgn(vt));
            if (BR < 0) r.v[e] = vt * sn;
            else r.v[e] = v1.v[e] * c6.v[e] + vt * sn;
        }
    }
    return r;
}

// face columns per row segment of the row form
constexpr int AQ_SEG = 3;

// east faces (between i and i+1) of row j at levels k0..k0+3 for face
// columns a = a0 .. min(a0+AQ_SEG, ti+1)-1, i = i0-1+a (u_east_ub, v_east_ub,
// s_east_ub), into E + a * TJ * nz.  The six-point stencil slides along i, so
// a segment loads each x column once; the table rows depend on k0 alone.
template <int TI, int TJ, int FK>
__device__ __forceinline__ void aq_east_row(const KParams<float> &p, const KFields<float> &F, const float *tab,
                                            float *E, int i0, int j, int k0, int ti, int a0)
{
    const int nz = p.nz, sx = p.ny * nz, sy = nz;
    const int c = gix(p.ny, nz, i0 - 1 + a0, j, k0);
    const float *X = F.cur[aq_field(FK)], *U = F.cur[FU];
    constexpr int BR = aq_brow(FK);
    const Q4 z4{{0.f, 0.f, 0.f, 0.f}};
    const Q4 ubar = lds4(tab + (FK <= 1 ? BT_UA : BT_UB) * nz + k0);
    const Q4 c6 = FK == 0 ? lds4(tab + BT_C6_UB * nz + k0)
                  : FK == 1 ? lds4(tab + BT_C6_VB * nz + k0)
                  : BR >= 0 ? lds4(tab + (BT_C6_THB + BR) * nz + k0)
                            : z4;
    Q4 x[6];
#pragma unroll
    for (int m = 0; m < 5; m++) x[m] = ldg4(X, c + (m - 2) * sx);
    Q4 u0 = FK == 0 ? ldg4(U, c) : z4;
#pragma unroll
    for (int s = 0; s < AQ_SEG; s++) {
        const int a = a0 + s;
        if (a > ti) break;
        const int ca = c + s * sx;
        x[5] = ldg4(X, ca + 3 * sx);
        Q4 r;
        if (FK == 0) {
            const Q4 up = ldg4(U, ca + sx);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float ua = 0.5f * (up.v[e] + u0.v[e]);
                const float ue = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                              sgn(ubar.v[e] + ua));
                r.v[e] = ua * c6.v[e] + (ubar.v[e] + ua) * ue;
            }
            u0 = up;
        } else if (FK == 1) {
            const Q4 ua_ = ldg4(U, ca + sx), ub_ = ldg4(U, ca + sx - sy);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float ua = 0.5f * (ua_.v[e] + ub_.v[e]);
                const float ve = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                              sgn(ubar.v[e] + ua));
                r.v[e] = ua * c6.v[e] + (ubar.v[e] + ua) * ve;
            }
        } else {
            const Q4 u1 = ldg4(U, ca + sx);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float ut = ubar.v[e] + u1.v[e];
                const float se = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                              sgn(ut));
                if (BR < 0) r.v[e] = ut * se;
                else r.v[e] = u1.v[e] * c6.v[e] + ut * se;
            }
        }
        sts4(E + a * TJ * nz, r);
#pragma unroll
        for (int m = 0; m < 5; m++) x[m] = x[m + 1];
    }
}

// north faces (between j and j+1) of row i for face columns
// b = b0 .. min(b0+AQ_SEG, tj+1)-1, j = j0-1+b (u_north_ub, v_north_ub,
// s_north_ub), into N + b * nz
template <int TI, int TJ, int FK>
__device__ __forceinline__ void aq_north_row(const KParams<float> &p, const KFields<float> &F, const float *tab,
                                             float *N, int i, int j0, int k0, int tj, int b0)
{
    const int nz = p.nz, sx = p.ny * nz, sy = nz;
    const int c = gix(p.ny, nz, i, j0 - 1 + b0, k0);
    const float *X = F.cur[aq_field(FK)], *V = F.cur[FV];
    constexpr int BR = aq_brow(FK);
    const Q4 z4{{0.f, 0.f, 0.f, 0.f}};
    const Q4 vbar = lds4(tab + (FK <= 1 ? BT_VA : BT_VB) * nz + k0);
    const Q4 c6 = FK == 0 ? lds4(tab + BT_C6_UB * nz + k0)
                  : FK == 1 ? lds4(tab + BT_C6_VB * nz + k0)
                  : BR >= 0 ? lds4(tab + (BT_C6_THB + BR) * nz + k0)
                            : z4;
    Q4 x[6];
#pragma unroll
    for (int m = 0; m < 5; m++) x[m] = ldg4(X, c + (m - 2) * sy);
    Q4 v0 = FK == 1 ? ldg4(V, c) : z4;
#pragma unroll
    for (int s = 0; s < AQ_SEG; s++) {
        const int b = b0 + s;
        if (b > tj) break;
        const int cb = c + s * sy;
        x[5] = ldg4(X, cb + 3 * sy);
        Q4 r;
        if (FK == 0) {
            const Q4 va_ = ldg4(V, cb + sy), vb_ = ldg4(V, cb - sx + sy);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float va = 0.5f * (va_.v[e] + vb_.v[e]);
                const float un = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                              sgn(vbar.v[e] + va));
                r.v[e] = va * c6.v[e] + (vbar.v[e] + va) * un;
            }
        } else if (FK == 1) {
            const Q4 vp = ldg4(V, cb + sy);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float va = 0.5f * (vp.v[e] + v0.v[e]);
                const float vn = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                              sgn(vbar.v[e] + va));
                r.v[e] = va * c6.v[e] + (vbar.v[e] + va) * vn;
            }
            v0 = vp;
        } else {
            const Q4 v1 = ldg4(V, cb + sy);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float vt = vbar.v[e] + v1.v[e];
                const float sn = face5<float>(x[0].v[e], x[1].v[e], x[2].v[e], x[3].v[e], x[4].v[e], x[5].v[e],
                                              sgn(vt));
                if (BR < 0) r.v[e] = vt * sn;
                else r.v[e] = v1.v[e] * c6.v[e] + vt * sn;
            }
        }
        sts4(N + b * nz, r);
#pragma unroll
        for (int m = 0; m < 5; m++) x[m] = x[m + 1];
    }
}

// top face (between k and k+1) at k = k0..k0+3: u_top_ub, v_top_ub,
// s_top_ub, r_top_ub; level NZ-1 is not a face of an advected cell (0)
template <int FK, class S>
__device__ __forceinline__ Q4 aq_top(const KParams<float> &p, const S &src, const float *tab, int i, int j, int k0)
{
    const int nz = p.nz;
    const int c = src.at(i, j, k0);
    const Win x = src.win(aq_field(FK), c, 0, 0, k0);
    const Win w = src.win(FW, c, 0, 0, k0);
    Q4 r;
    if (FK == 0 || FK == 1) {
        // the second w of the averaged advecting velocity: column i-1 (u) or j-1 (v)
        const Win w2 = src.win(FW, c, FK == 0 ? -1 : 0, FK == 0 ? 0 : -1, k0);
        constexpr int C4 = FK == 0 ? BT_C4_UB : BT_C4_VB, H2 = FK == 0 ? BT_H2_UB : BT_H2_VB;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            float f = 0.f;
            if (k >= 1 && k <= nz - 2) {
                const float wa = 0.5f * (w.at(e + 1) + w2.at(e + 1));
                const float wba = tab[BT_WA * nz + k];
                float xt, xbt;
                if (k == 1 || k == nz - 2) {
                    xt = 0.5f * (x.at(e + 1) + x.at(e));
                    xbt = tab[H2 * nz + k];
                } else {
                    xt = face3<float>(x.at(e - 1), x.at(e), x.at(e + 1), x.at(e + 2), sgn(wba + wa));
                    xbt = tab[C4 * nz + k] + W<float>::c1_12 * sgn(wa) * tab[(C4 + 1) * nz + k];
                }
                f = wa * xbt + (wba + wa) * xt;
            }
            r.v[e] = f;
        }
    } else if (FK < 5) {
        constexpr int BR = aq_brow(FK);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            float f = 0.f;
            if (k >= 1 && k <= nz - 2) {
                const float w1 = w.at(e + 1);
                const float wt = tab[BT_WB * nz + k + 1] + w1;
                float st, bt = 0.f;
                if (k == 1 || k == nz - 2) {
                    st = 0.5f * (x.at(e + 1) + x.at(e));
                    if (BR >= 0) bt = tab[(BT_H2_THB + BR) * nz + k];
                } else {
                    st = face3<float>(x.at(e - 1), x.at(e), x.at(e + 1), x.at(e + 2), sgn(wt));
                    if (BR >= 0)
                        bt = tab[(BT_C4_THB + 2 * BR) * nz + k] +
                             W<float>::c1_12 * sgn(w1) * tab[(BT_C4_THB + 2 * BR + 1) * nz + k];
                }
                if (BR < 0) f = wt * st;
                else f = w1 * bt + wt * st;
            }
            r.v[e] = f;
        }
    } else {
        // rain, snow, ice: the fall speed at levels k0..k0+4 (vt_at; the
        // ice scheme's speeds are stored by their own kernel)
        const float *fa = FK == 5 ? src.F.vt : FK == 6 ? src.F.sts : src.F.its;
        float vt[5];
#pragma unroll
        for (int e = 0; e < 5; e++) {
            const int k = k0 + e;
            float v = 0.f;
            if (k < nz) {
                if (FK == 5 && p.rf == 1 && !p.ice && k < nz - 1) {
                    const int kk = k == 0 ? 1 : k;
                    v = fall_speed_point(p, x.at(kk - k0), kk);
                } else {
                    v = src.vt(fa, i, j, k0, c, e);
                }
            }
            vt[e] = v;
        }
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            float f = 0.f;
            if (k == 0) {
                const float s0 = 0.5f * (x.at(0) + x.at(1));
                f = -0.5f * (vt[1] + vt[0]) * s0;
            } else if (k <= nz - 2) {
                const float wb = tab[BT_WB * nz + k + 1] + w.at(e + 1);
                const float wf = wb - 0.5f * (vt[e] + vt[e + 1]);
                float st;
                if (k == 1 || k == nz - 2) st = 0.5f * (x.at(e + 1) + x.at(e));
                else st = face3<float>(x.at(e - 1), x.at(e), x.at(e + 1), x.at(e + 2), sgn(wf));
                f = wf * st;
            }
            r.v[e] = f;
        }
    }
    return r;
}

// the face columns of field FK into slot `sl` (E, N and T of the tile).
// Level slab: cells ks..ke-1; the slot holds levels kb..ke-1 of every face
// column at stride SK, where kb = ks, or ks - 4 when the slab starts above
// the bottom (the divergence of level ks needs the top face of level ks - 1).
// rows (global source, whole columns only): east and north faces by row
// segments of up to AQ_SEG face columns whose stencil slides (fewer loads and
// less index arithmetic, but a segment's loads one after another); otherwise
// one work item per face column and quad.  In the row form one loop covers
// three kinds of work item, each padded to whole warps: east segments
// (segment, b, quad), north segments (segment, a, quad) and top faces
// (column, quad).  Both forms evaluate the same expressions.
template <int TI, int TJ, int FK, class S>
__device__ __forceinline__ void aq_faces(const KParams<float> &p, const KFields<float> &F, const S &src,
                                         const float *tab, float *sl, int i0, int j0, int ti, int tj, bool rows,
                                         int ks, int ke, int kb, int SK)
{
    using G = AQGeom<TI, TJ>;
    float *E = sl, *N = sl + G::CE * SK, *T = N + G::CN * SK;
    const int NQ = (ke - ks) >> 2, NQT = (ke - kb) >> 2;
    if (rows) {  // GSrc, ks = kb = 0, ke = SK = nz
        const int nz = p.nz;
        constexpr int SE = (TI + AQ_SEG) / AQ_SEG, SN = (TJ + AQ_SEG) / AQ_SEG;  // segments of TI+1, TJ+1
        const int nE = (SE * TJ * NQ + 31) & ~31, nN = (SN * TI * NQ + 31) & ~31, nall = nE + nN + G::CT * NQ;
        for (int w = threadIdx.x; w < nall; w += AQ_THREADS) {
            if (w < nE) {
                const int q = w % NQ, r = w / NQ, b = r % TJ, a0 = (r / TJ) * AQ_SEG;
                if (b < tj && a0 <= ti)
                    aq_east_row<TI, TJ, FK>(p, F, tab, E + b * nz + 4 * q, i0, j0 + b, 4 * q, ti, a0);
            } else if (w < nE + nN) {
                const int v = w - nE, q = v % NQ, r = v / NQ, a = r % TI, b0 = (r / TI) * AQ_SEG;
                if (a < ti && b0 <= tj)
                    aq_north_row<TI, TJ, FK>(p, F, tab, N + a * (TJ + 1) * nz + 4 * q, i0 + a, j0, 4 * q, tj, b0);
            } else {
                const int v = w - nE - nN, q = v % NQ, col = v / NQ, b = col % TJ, a = col / TJ;
                if (a < ti && b < tj) sts4(T + col * nz + 4 * q, aq_top<FK>(p, src, tab, i0 + a, j0 + b, 4 * q));
            }
        }
        return;
    }
    for (int w = threadIdx.x; w < G::CE * NQ; w += AQ_THREADS) {
        const int q = w % NQ, col = w / NQ, b = col % TJ, a = col / TJ;
        if (a > ti || b >= tj) continue;
        const int k0 = ks + 4 * q;
        sts4(E + col * SK + k0 - kb, aq_east<FK>(p, src, tab, i0 - 1 + a, j0 + b, k0));
    }
    for (int w = threadIdx.x; w < G::CN * NQ; w += AQ_THREADS) {
        const int q = w % NQ, col = w / NQ, b = col % (TJ + 1), a = col / (TJ + 1);
        if (a >= ti || b > tj) continue;
        const int k0 = ks + 4 * q;
        sts4(N + col * SK + k0 - kb, aq_north<FK>(p, src, tab, i0 + a, j0 - 1 + b, k0));
    }
    for (int w = threadIdx.x; w < G::CT * NQT; w += AQ_THREADS) {
        const int q = w % NQT, col = w / NQT, b = col % TJ, a = col / TJ;
        if (a >= ti || b >= tj) continue;
        const int k0 = kb + 4 * q;
        sts4(T + col * SK + k0 - kb, aq_top<FK>(p, src, tab, i0 + a, j0 + b, k0));
    }
}

// flux divergence of the slot at the cell quad (tend of k_advect_tile)
template <int TI, int TJ>
__device__ __forceinline__ Q4 aq_div(const KParams<float> &p, const float *sl, const float *lv, int a, int b, int k0,
                                     int kb, int SK)
{
    using G = AQGeom<TI, TJ>;
    const int nz = p.nz;
    const float *E = sl, *N = sl + G::CE * SK, *T = N + G::CN * SK;
    const float *s_mu = lv, *s_rhow = lv + nz, *s_odr = lv + 2 * nz;
    const int kk = k0 - kb;
    const int oe = ((a + 1) * TJ + b) * SK + kk, ow = (a * TJ + b) * SK + kk;
    const int on = (a * (TJ + 1) + b + 1) * SK + kk, os = (a * (TJ + 1) + b) * SK + kk;
    const int ot = (a * TJ + b) * SK + kk;
    const Q4 ee = lds4(E + oe), ew = lds4(E + ow), nn = lds4(N + on), ns = lds4(N + os), tt = lds4(T + ot);
    const float tb0 = k0 > 0 ? T[ot - 1] : 0.f;
    Q4 r;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int k = k0 + e;
        const float tlo = e == 0 ? tb0 : tt.v[e - 1];
        const float DTZ = p.dtz * s_mu[k];
        const int kp1 = min(k + 1, nz - 1);  // level NZ-1 is padding
        r.v[e] = -p.dtx * (ee.v[e] - ew.v[e]) - p.dty * (nn.v[e] - ns.v[e]) -
                 DTZ * (s_rhow[kp1] * tt.v[e] - s_rhow[k] * tlo) * s_odr[k];
    }
    return r;
}

// store the levels of a quad that are cells of the field (kmin .. NZ-2)
__device__ __forceinline__ void aq_store(float *dst, int c, int k0, int nz, int kmin, const Q4 &q)
{
    if (k0 >= kmin && k0 + 3 <= nz - 2) {
        stg4(dst + c, q);
    } else {
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            if (k >= kmin && k <= nz - 2) dst[c + e] = q.v[e];
        }
    }
}

// the level arrays and the basic-state table of a block, into shared memory
__device__ __forceinline__ void aq_stage_tables(const KParams<float> &p, float *tab, float *lv)
{
    const int nz = p.nz;
    for (int e = threadIdx.x; e < BT_COUNT * nz; e += AQ_THREADS) tab[e] = p.btab[e];
    for (int k = threadIdx.x; k < nz; k += AQ_THREADS) {
        lv[k] = p.mu[k];
        lv[nz + k] = p.rhow[k];
        lv[2 * nz + k] = p.one_d_rhou[k];
        lv[3 * nz + k] = p.tb[k];
        lv[4 * nz + k] = p.moist ? p.qb[k] : 0.f;
        lv[5 * nz + k] = p.tbv[k];
        lv[6 * nz + k] = p.rhou[k];
    }
}

// the three passes over cells (i0..i0+ti-1, j0..j0+tj-1) and levels
// ks..ke-1 with the current fields read from `src`; face slots s0, s1 with
// levels kb..ke-1 at stride SK (see aq_faces); tables staged and synchronised
template <int TI, int TJ, class S>
__device__ __forceinline__ void advect_quad_cells(const KParams<float> &p, const KFields<float> &F, const S &src,
                                                  float *s0, float *s1, const float *tab, const float *lv, int i0,
                                                  int j0, int ti, int tj, int ks, int ke, int kb, int SK, float step,
                                                  float sdtg, int what)
{
    using G = AQGeom<TI, TJ>;
    const int nz = p.nz, NQ = (ke - ks) >> 2, sx = p.ny * nz, sy = nz;
    const float *s_mu = lv, *s_rhow = lv + nz, *s_odr = lv + 2 * nz, *s_tb = lv + 3 * nz, *s_qb = lv + 4 * nz,
                *s_tbv = lv + 5 * nz;
    const bool rows = (what & ADV_ROWS) != 0;
    (void)sx;
    (void)sy;

    // ---- pass 1: u, v (and the buoyancy of w)
    if (what & (ADV_UV | ADV_WB)) {
        if (what & ADV_UV) {
            aq_faces<TI, TJ, 0>(p, F, src, tab, s0, i0, j0, ti, tj, rows, ks, ke, kb, SK);
            aq_faces<TI, TJ, 1>(p, F, src, tab, s1, i0, j0, ti, tj, rows, ks, ke, kb, SK);
        }
        __syncthreads();
        for (int w = threadIdx.x; w < G::CT * NQ; w += AQ_THREADS) {
            const int q = w % NQ, col = w / NQ, b = col % TJ, a = col / TJ;
            if (a >= ti || b >= tj) continue;
            const int i = i0 + a, j = j0 + b, k0 = ks + 4 * q;
            const int c = gix(p.ny, nz, i, j, k0), cs = src.at(i, j, k0);
            // every load of the quad's u, v and w results before any store
            // (a store to P would otherwise order the later loads after it)
            Q4 ru, rv;
            if (what & ADV_UV) {
                const float fj = p.f[j];
                const Q4 v0 = src.ld4(FV, cs, 0, 0), v1 = src.ld4(FV, cs, 0, 1), v2 = src.ld4(FV, cs, -1, 0),
                         v3 = src.ld4(FV, cs, -1, 1);
                const Q4 u0 = src.ld4(FU, cs, 0, 0), u1 = src.ld4(FU, cs, 1, 0), u2 = src.ld4(FU, cs, 0, -1),
                         u3 = src.ld4(FU, cs, 1, -1);
                const Q4 mu = ldg4(F.M[FU], c), mv = ldg4(F.M[FV], c);
                const Q4 du = aq_div<TI, TJ>(p, s0, lv, a, b, k0, kb, SK), dv = aq_div<TI, TJ>(p, s1, lv, a, b, k0, kb, SK);
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float ov_u = 0.25f * (v0.v[e] + v1.v[e] + v2.v[e] + v3.v[e]);
                    const float ut = du.v[e] + p.dt * fj * ov_u;
                    ru.v[e] = mu.v[e] + step * ut;
                    const float ov_v = 0.25f * (u0.v[e] + u1.v[e] + u2.v[e] + u3.v[e]);
                    const float vt = dv.v[e] - p.dt * fj * ov_v;
                    rv.v[e] = mv.v[e] + step * vt;
                }
            }
            Q4 rw;
            if (what & ADV_WB) {
                // buoyancy at levels k0-1 .. k0+3 (b1 of level k is b0 of level k-1)
                const Win th = src.win(FTH, cs, 0, 0, k0);
                Win qv, qc, qr;
                if (p.moist) {
                    qv = src.win(FQV, cs, 0, 0, k0);
                    qc = src.win(FQC, cs, 0, 0, k0);
                    qr = src.win(FQR, cs, 0, 0, k0);
                }
                float bb[5];
#pragma unroll
                for (int e = 0; e < 5; e++) {
                    const int k = k0 + e - 1;
                    const int kc = max(k, 0);
                    if (!p.moist) bb[e] = th.at(e - 1) / s_tbv[kc];
                    else bb[e] = th.at(e - 1) / s_tbv[kc] + 0.61f * qv.at(e - 1) - qc.at(e - 1) - qr.at(e - 1);
                }
                if (p.ice) {  // buoyancy_cold_micro (advection.cpp:56-58): less ice, then snow
                    const Win qi = src.win(FQI, cs, 0, 0, k0);
#pragma unroll
                    for (int e = 0; e < 5; e++) bb[e] = bb[e] - qi.at(e - 1);
                    const Win qs = src.win(FQS, cs, 0, 0, k0);
#pragma unroll
                    for (int e = 0; e < 5; e++) bb[e] = bb[e] - qs.at(e - 1);
                }
                const Q4 m = ldg4(F.M[FW], c);
#pragma unroll
                for (int e = 0; e < 4; e++) rw.v[e] = m.v[e] + sdtg * (bb[e + 1] + bb[e]);
            }
            if (what & ADV_UV) {
                aq_store(F.P[FU], c, k0, nz, 1, ru);
                aq_store(F.P[FV], c, k0, nz, 1, rv);
            }
            if (what & ADV_WB) aq_store(F.P[FW], c, k0, nz, 2, rw);
        }
        __syncthreads();
    }

    // ---- pass 2: theta, qv (qv's clipping bit)
    const bool th_on = (what & ADV_TH) != 0, q_on = (what & ADV_Q) != 0;
    if (th_on || q_on) {
        if (th_on) aq_faces<TI, TJ, 2>(p, F, src, tab, s0, i0, j0, ti, tj, rows, ks, ke, kb, SK);
        if (q_on) aq_faces<TI, TJ, 3>(p, F, src, tab, s1, i0, j0, ti, tj, rows, ks, ke, kb, SK);
        __syncthreads();
        for (int w = threadIdx.x; w < G::CT * NQ; w += AQ_THREADS) {
            const int q = w % NQ, col = w / NQ, b = col % TJ, a = col / TJ;
            if (a >= ti || b >= tj) continue;
            const int i = i0 + a, j = j0 + b, k0 = ks + 4 * q;
            const int c = gix(p.ny, nz, i, j, k0), cs = src.at(i, j, k0);
            const Win wc = src.win(FW, cs, 0, 0, k0);
            // both fields' start-of-step values before either store
            const Q4 z4{{0.f, 0.f, 0.f, 0.f}};
            const Q4 mq[2] = {th_on ? ldg4(F.M[FTH], c) : z4, q_on ? ldg4(F.M[FQV], c) : z4};
            Q4 rq[2];
            unsigned bits = 0;
#pragma unroll
            for (int fi = 0; fi < 2; fi++) {
                if (fi == 0 ? !th_on : !q_on) continue;
                const float *base = fi == 0 ? s_tb : s_qb;
                const Q4 d = aq_div<TI, TJ>(p, fi == 0 ? s0 : s1, lv, a, b, k0, kb, SK);
                const Q4 m = mq[fi];
                Q4 r;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int k = k0 + e;
                    const int kl = max(k - 1, 0), kh = min(k + 1, nz - 1);
                    const float DTZ = p.dtz * s_mu[k];
                    const float zab = 0.50f *
                                      (s_rhow[kh] * wc.at(e + 1) * (base[kh] - base[k]) +
                                       s_rhow[k] * wc.at(e) * (base[k] - base[kl])) *
                                      s_odr[k];
                    const float t = d.v[e] - DTZ * zab;
                    float v = m.v[e] + step * t;
                    if (fi == 1 && (what & ADV_ZERO)) {
                        const float qbar = tab[BT_QB * nz + k];
                        if (v + qbar + s_qb[k] < 0) {
                            v = -(qbar + s_qb[k]);
                            bits |= 1u << (8 * e);
                        }
                    }
                    r.v[e] = v;
                }
                rq[fi] = r;
            }
            if (th_on) aq_store(F.P[FTH], c, k0, nz, 1, rq[0]);
            if (q_on) aq_store(F.P[FQV], c, k0, nz, 1, rq[1]);
            if (q_on && (what & ADV_ZERO) && F.qmask) {
                unsigned char *qm = F.qmask + c;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int k = k0 + e;
                    if (k >= 1 && k <= nz - 2) qm[e] = (unsigned char)((bits >> (8 * e)) & 1u);
                }
            }
        }
        __syncthreads();
    }

    // ---- pass 3: qc, qr (clipping bits 2 and 4, the rain's fall speed)
    if (q_on) {
        aq_faces<TI, TJ, 4>(p, F, src, tab, s0, i0, j0, ti, tj, rows, ks, ke, kb, SK);
        aq_faces<TI, TJ, 5>(p, F, src, tab, s1, i0, j0, ti, tj, rows, ks, ke, kb, SK);
        __syncthreads();
        for (int w = threadIdx.x; w < G::CT * NQ; w += AQ_THREADS) {
            const int q = w % NQ, col = w / NQ, b = col % TJ, a = col / TJ;
            if (a >= ti || b >= tj) continue;
            const int i = i0 + a, j = j0 + b, k0 = ks + 4 * q;
            const int c = gix(p.ny, nz, i, j, k0), cs = src.at(i, j, k0);
            const Q4 dc = aq_div<TI, TJ>(p, s0, lv, a, b, k0, kb, SK);
            const Q4 dr = aq_div<TI, TJ>(p, s1, lv, a, b, k0, kb, SK);
            const Q4 mc = ldg4(F.M[FQC], c), mr = ldg4(F.M[FQR], c);
            Q4 rc, rr;
            unsigned char bits[4] = {0, 0, 0, 0};
#pragma unroll
            for (int e = 0; e < 4; e++) {
                float qc = mc.v[e] + step * dc.v[e];
                float qr = mr.v[e] + step * dr.v[e];
                if (what & ADV_ZERO) {
                    if (qc < 0) { qc = 0; bits[e] |= 2; }
                    if (qr < 0) { qr = 0; bits[e] |= 4; }
                }
                rc.v[e] = qc;
                rr.v[e] = qr;
            }
            aq_store(F.P[FQC], c, k0, nz, 1, rc);
            aq_store(F.P[FQR], c, k0, nz, 1, rr);
            if ((what & ADV_ZERO) && F.qmask) {
                unsigned char *qm = F.qmask + c;
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int k = k0 + e;
                    if (k >= 1 && k <= nz - 2) qm[e] |= bits[e];
                }
            }
            if (p.rf == 1 && !p.ice) {
                // fall speed of the advected cells; level 0 repeats level 1
                const Q4 qrc = src.ld4(FQR, cs, 0, 0);
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int k = k0 + e;
                    if (k >= 1 && k <= nz - 2) F.vt[c + e] = fall_speed_point(p, qrc.v[e], k);
                    if (k == 1) F.vt[c + e - 1] = fall_speed_point(p, qrc.v[e], 1);
                }
            }
        }
    }

    // ---- pass 4 (ice scheme): snow and cloud ice with their fall speeds
    // (advect_ice_cell, advection.cpp:508-567), clipped with the moisture
    if (what & ADV_ICE) {
        __syncthreads();
        aq_faces<TI, TJ, 6>(p, F, src, tab, s0, i0, j0, ti, tj, rows, ks, ke, kb, SK);
        aq_faces<TI, TJ, 7>(p, F, src, tab, s1, i0, j0, ti, tj, rows, ks, ke, kb, SK);
        __syncthreads();
        for (int w = threadIdx.x; w < G::CT * NQ; w += AQ_THREADS) {
            const int q = w % NQ, col = w / NQ, b = col % TJ, a = col / TJ;
            if (a >= ti || b >= tj) continue;
            const int i = i0 + a, j = j0 + b, k0 = ks + 4 * q;
            const int c = gix(p.ny, nz, i, j, k0);
            const Q4 ds = aq_div<TI, TJ>(p, s0, lv, a, b, k0, kb, SK);
            const Q4 di = aq_div<TI, TJ>(p, s1, lv, a, b, k0, kb, SK);
            const Q4 ms = ldg4(F.M[FQS], c), mi = ldg4(F.M[FQI], c);
            Q4 rs, ri;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                float qs = ms.v[e] + step * ds.v[e];
                float qi = mi.v[e] + step * di.v[e];
                if (what & ADV_ZERO) {
                    if (qs < 0) qs = 0;
                    if (qi < 0) qi = 0;
                }
                rs.v[e] = qs;
                ri.v[e] = qi;
            }
            aq_store(F.P[FQS], c, k0, nz, 1, rs);
            aq_store(F.P[FQI], c, k0, nz, 1, ri);
        }
    }
}


// one TI x TJ tile (bx, by), every level, the fields read from global memory;
// the batched ensemble kernel calls it per member
template <int TI, int TJ>
__device__ __forceinline__ void advect_quad_body(const KParams<float> &p, const KFields<float> &F, int bx, int by,
                                                 float step, float sdtg, int what)
{
    using G = AQGeom<TI, TJ>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nz = p.nz;
    float *s0 = (float *)smem_raw, *s1 = s0 + G::CF * nz;
    float *tab = s1 + G::CF * nz;
    float *lv = tab + BT_COUNT * nz;
    aq_stage_tables(p, tab, lv);
    const int i0 = 3 + bx * TI, j0 = 3 + by * TJ;
    const int ti = min(TI, p.nx - 3 - i0), tj = min(TJ, p.ny - 3 - j0);
    __syncthreads();
    const GSrc src(F, p.ny, nz);
    advect_quad_cells<TI, TJ>(p, F, src, s0, s1, tab, lv, i0, j0, ti, tj, 0, nz, 0, nz, step, sdtg, what);
}

// MB: blocks per SM the registers are sized for (3: 80 registers, 4: 64)
template <int TI, int TJ, int MB>
__global__ void __launch_bounds__(AQ_THREADS, MB)
    k_advect_quad(KParams<float> p, KFields<float> F, float step, float sdtg, int what)
{
    if (what & ADV_MIRROR) {  // mirror copies (edge points from non-advected ones), grid-stride
        const long nt = (long)gridDim.x * gridDim.y * AQ_THREADS;
        const long ntot = 2L * (p.nx + p.ny - 2) * (p.nz - 2);
        for (long t = ((long)blockIdx.y * gridDim.x + blockIdx.x) * AQ_THREADS + threadIdx.x; t < ntot; t += nt)
            mirror_edges_body(p, F.P[FU], F.P[FV], F.P[FW], t);
    }
    advect_quad_body<TI, TJ>(p, F, blockIdx.x, blockIdx.y, step, sdtg, what);
}

// ---------------------------------------------------------------------------
// k_advect_tma: the same passes with every current field staged into shared
// memory by the tensor memory accelerator.  A block owns TI x TJ columns and a
// slab of KZ levels (ks .. ks+KZ-1, the last slab cut at NZ).  One elected
// thread issues a 3-D tiled copy per field of the box i0-3 .. i0+TI+2,
// j0-3 .. j0+TJ+2, ks-4 .. ks+KZ+3 (the widest stencil of a face, and the
// 12-level windows of the top faces; points outside the field arrive as
// zeros), all completing on one mbarrier; the face and cell arithmetic then
// reads shared memory only, expression for expression the arithmetic of
// k_advect_quad, so the results are bit-identical.  The start-of-step fields
// (read once per point) and the stores stay in global memory.  A slab above
// the bottom also evaluates the top faces of the quad below it (the
// divergence of level ks needs the face at ks-1).
// ---------------------------------------------------------------------------
template <int TI, int TJ, int KZ>
struct AQTma {
    static constexpr int BI = TI + 6, BJ = TJ + 6, BK = KZ + 8;
    static constexpr int BOX = BI * BJ * BK;          // floats per field box
    static constexpr int BOXP = (BOX + 31) & ~31;     // boxes 128-byte aligned
    static constexpr int SK = KZ + 4;                 // face-slot levels per column
};

// boxes of nf fields, two face slots, the basic-state table, the level
// arrays, the barrier
__host__ __device__ constexpr size_t advect_tma_smem(int ti, int tj, int kz, int nz, int nf)
{
    return ((size_t)nf * ((((ti + 6) * (tj + 6) * (kz + 8)) + 31) & ~31) +
            2 * (size_t)((ti + 1) * tj + ti * (tj + 1) + ti * tj) * (kz + 4) + (size_t)BT_COUNT * nz +
            (size_t)AQ_LV * nz) *
               sizeof(float) +
           16;
}

template <int TI, int TJ, int KZ, int MB>
__global__ void __launch_bounds__(AQ_THREADS, MB)
    k_advect_tma(const __grid_constant__ TmaMaps maps, KParams<float> p, KFields<float> F, float step, float sdtg,
                 int what, int *err)
{
    using A = AQTma<TI, TJ, KZ>;
    using G = AQGeom<TI, TJ>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int nz = p.nz, nf = p.moist ? 7 : 4;
    float *boxes = (float *)smem_raw;
    float *s0 = boxes + nf * A::BOXP, *s1 = s0 + G::CF * A::SK;
    float *tab = s1 + G::CF * A::SK;
    float *lv = tab + BT_COUNT * nz;
    uint64_t *bar = (uint64_t *)(lv + AQ_LV * nz);
    if (what & ADV_MIRROR) {  // mirror copies (edge points from non-advected ones), grid-stride
        const long nt = (long)gridDim.x * gridDim.y * gridDim.z * AQ_THREADS;
        const long ntot = 2L * (p.nx + p.ny - 2) * (p.nz - 2);
        const long b = ((long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        for (long t = b * AQ_THREADS + threadIdx.x; t < ntot; t += nt) mirror_edges_body(p, F.P[FU], F.P[FV], F.P[FW], t);
    }
    const int i0 = 3 + blockIdx.x * TI, j0 = 3 + blockIdx.y * TJ, ks = blockIdx.z * KZ;
    const int ti = min(TI, p.nx - 3 - i0), tj = min(TJ, p.ny - 3 - j0);
    const int ke = min(ks + KZ, nz), kb = ks > 0 ? ks - 4 : 0;
    if (smem_addr(boxes) & 127u) {  // the copies need 128-byte aligned destinations
        if (threadIdx.x == 0) atomicOr(err, kErrStaging);
        return;
    }
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, (uint32_t)(nf * A::BOX * sizeof(float)));
        for (int f = 0; f < nf; f++) tma_load_3d(boxes + f * A::BOXP, &maps.m[f], ks - 4, j0 - 3, i0 - 3, bar);
    }
    aq_stage_tables(p, tab, lv);
    // bounded wait; every thread leaves together if the copies did not land
    const bool landed = __syncthreads_and(mbar_wait_bounded(bar, 0) ? 1 : 0);
    if (!landed) {
        if (threadIdx.x == 0) atomicOr(err, kErrStaging);
        mbar_wait_bounded(bar, 0);  // the copies still in flight, bounded again
        return;
    }
    const SSrc<A::BJ, A::BK> src{F, boxes, A::BOXP, i0 - 3, j0 - 3, ks - 4, p.ny, nz};
    advect_quad_cells<TI, TJ>(p, F, src, s0, s1, tab, lv, i0, j0, ti, tj, ks, ke, kb, A::SK, step, sdtg,
                              what & ~ADV_ROWS);
}

// ---------------------------------------------------------------------------
// k_post_quad: the column post-processing of k_post, expression for
// expression.  A column's bottom and top conditions copy level 1 to 0 and
// NZ-2 to NZ-1, both inside one quad, so every thread reads and writes only
// its own points and the fields go one after another without a barrier.
// ---------------------------------------------------------------------------
constexpr int PQ_THREADS = 256;

// item w: column w / (NZ/4) of the enumeration `cols`, level quad w % (NZ/4).
// KES: the step's last pass with Kessler (run_kessler_microphysics,
// kessler.cpp:25-213) and the Eulerian precipitation (precip_rate,
// microphysics.cpp:143-160) applied to the loaded forecast values ahead of the
// chain, as the reference applies them before its last boundary conditions;
// err receives Kessler's E > 100 flag.  A periodic target pass evaluates the
// source column's Kessler again (the same inputs, the same values) and leaves
// the rain total to the source's own pass.
template <typename T, bool KES = false>
__device__ __forceinline__ void post_quad_body(const KParams<T> &p, const KFields<T> &F, int4 fl0, int4 fl1, T step,
                                               int cols, long w, int *err = nullptr)
{
    static_assert(sizeof(T) == 4, "four-level kernels are FP32");
    const int nz = p.nz, NQ = nz >> 2, sx = p.ny * nz, sy = nz;
    const int q = (int)(w % NQ), k0 = 4 * q;
    int i = 0, j = 0;
    bool ok = false;
    post_column(cols, w / NQ, p.nx, p.ny, i, j, ok);
    if (!ok) return;
    const int flv[7] = {fl0.x, fl0.y, fl0.z, fl0.w, fl1.x, fl1.y, fl1.z};
    // the chain runs at the source column (the column itself, or the column a
    // periodic target copies)
    const int si = cols == COLS_TARGETS ? (i < 3 ? p.nx - 6 + i : 3 + (i - (p.nx - 3))) : i;
    const int cs = gix(p.ny, nz, si, j, k0), c = gix(p.ny, nz, i, j, k0);
    const bool col_in = si >= 1 && si < p.nx - 1 && j >= 1 && j < p.ny - 1;
    const bool vbc = i >= 1 && j >= 1;
    const bool ray_col = i >= 1 && i < p.nx - 1 && j >= 1 && j < p.ny - 1;
    // sponge strips of the column (boundaries.cpp:481-498); every level k >= 1
    const bool hE = !p.periodic && j >= 1 && si >= p.eb && si < p.ee;
    const bool hW = !p.periodic && j >= 1 && si >= p.wb && si < p.we;
    const bool hS = si >= 1 && j >= p.sb && j < p.se;
    const bool hN = si >= 1 && j >= p.nb && j < p.ne;
    const float cE = hE ? p.ce[si - p.eb] : 0.f, cW = hW ? p.cw[si - p.wb] : 0.f;
    const float cS = hS ? p.cs[j - p.sb] : 0.f, cN = hN ? p.cn[j - p.nb] : 0.f;
    float dpx[4] = {0.f, 0.f, 0.f, 0.f}, dpy[4] = {0.f, 0.f, 0.f, 0.f}, dpz[4] = {0.f, 0.f, 0.f, 0.f};
    if (col_in && ((flv[FU] | flv[FV] | flv[FW]) & PF_PROJECT)) {
        const Win pc = ldwin(F.pi, cs, k0, nz);
        const Q4 px = ldg4(F.pi, cs - sx), py = ldg4(F.pi, cs - sy);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            dpx[e] = pc.at(e) - px.v[e];
            dpy[e] = pc.at(e) - py.v[e];
            dpz[e] = pc.at(e) - pc.at(e - 1);
        }
    }
    // every field's quad is loaded before any is written (a store to one
    // field's buffer would otherwise order the next field's load after it)
    Q4 inq[7];
#pragma unroll
    for (int f = 0; f < 7; ++f) inq[f] = flv[f] ? ldg4(F.P[f], cs) : Q4{{0.f, 0.f, 0.f, 0.f}};
    if constexpr (KES) {
        if (col_in) {
            const float qr0 = inq[FQR].v[0];  // level 0 before the chain (precip_rate reads it)
            const Q4 pq = ldg4(F.pi, cs);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = k0 + e;
                if (k < 1 || k >= nz - 1) continue;
                float th = inq[FTH].v[e], qv = inq[FQV].v[e], qc = inq[FQC].v[e], qr = inq[FQR].v[e];
                if (kessler_point(th, qv, qc, qr, pq.v[e], kes_point(p, F, k, (long)cs + e),
                                  F.sat ? F.sat + cs + e : nullptr))
                    atomicExch(err, 1);
                inq[FTH].v[e] = th;
                inq[FQV].v[e] = qv;
                inq[FQC].v[e] = qc;
                inq[FQR].v[e] = qr;
            }
            if (q == 0 && cols != COLS_TARGETS) {
                const double inc = (double)(p.rhow[1] * 0.5f * (F.vt[cs] + F.vt[cs + 1]) * 0.5f *
                                            (qr0 + inq[FQR].v[1]) * p.dt);
                F.accrain[(long)si * p.ny + j] += inc;
            }
        }
    }
    Q4 qb4{{0.f, 0.f, 0.f, 0.f}};
    if ((flv[FQV] & PF_ZERO) && col_in) qb4 = ldg4(F.bar[4], cs);
#pragma unroll
    for (int f = 0; f < 7; ++f) {
        const int flags = flv[f];
        if (!flags) continue;
        const Q4 in = inq[f];
        float ch[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            const bool inner = col_in && k >= 1 && k < nz - 1;
            float v = in.v[e];
            if (flags & PF_ZERO) {  // zero_moisture, microphysics.cpp:675-700
                if (f == FQC || f == FQR) {
                    if (v < 0) v = 0;
                } else if (f == FQV && inner) {
                    const float qbar = qb4.v[e];
                    if (v + qbar + p.qb[k] < 0) v = -(qbar + p.qb[k]);
                }
            }
            if ((flags & PF_PROJECT) && inner) {  // solver.cpp:123-135
                if (f == FU) v = v - step * (p.dtx * dpx[e]);
                else if (f == FV) v = v - step * (p.dty * dpy[e]);
                else if (f == FW && k >= 2) v = v - step * ((p.dtz * p.mw[k]) * dpz[e]);
            }
            if ((flags & PF_SPONGE) && k >= 1) {
                if (hE) v = v - cE * v;
                if (hW) v = v - cW * v;
                if (hS) v = v - cS * v;
                if (hN) v = v - cN * v;
            }
            ch[e] = v;
        }
        Q4 out;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int k = k0 + e;
            float v = ch[e];
            if ((flags & PF_VBC) && vbc) {  // boundaries.cpp:304-326
                if (f == FW) {
                    if (k == 0 || k == 1 || k == nz - 1) v = 0.f;
                } else {
                    if (k == 0) v = ch[1];
                    if (k == nz - 1) v = ch[2];
                }
            }
            if ((flags & PF_RAYLEIGH) && f <= FTH && ray_col && k >= p.raylevel) {  // damping.cpp:1148-1177
                const float cr = (f == FW) ? p.ray_w[k] : p.ray_u[k];
                v = v - cr * v;
            }
            out.v[e] = v;
        }
        stg4(F.P[f] + c, out);
        if (flags & PF_WRITE_M) stg4(F.M[f] + c, out);
    }
}

template <typename T, bool KES = false>
__global__ void __launch_bounds__(PQ_THREADS)
    k_post_quad(KParams<T> p, KFields<T> F, int4 fl0, int4 fl1, T step, int cols, int *err)
{
    post_quad_body<T, KES>(p, F, fl0, fl1, step, cols, (long)blockIdx.x * PQ_THREADS + threadIdx.x, err);
}

// ---------------------------------------------------------------------------
// k_spectral_x_pair: the fused x transform + Thomas + inverse x transform of
// k_spectral_x for one y-wavenumber, split over a cluster of two CTAs (FP32).
// CTA r transforms levels l0 .. l1-1 of every x line (half the lines), then
// solves the tridiagonal columns of x-wavenumbers p0 .. p1-1 (half the
// columns): it gathers the other half of those columns' levels from its
// peer's shared memory, solves them in a local buffer and writes the peer's
// half back; after a second cluster barrier each CTA runs the inverse
// transform of its own lines.  Per column the arithmetic is k_spectral_x's.
// ---------------------------------------------------------------------------
struct SxPair {
    int ps;  // point stride of a CTA's half lines (1 mod 16 complex values)
    int xs;  // column stride of the gathered columns (odd)
};
__host__ inline SxPair sx_pair_layout(int nz)
{
    const int nl = nz - 2, nlr = (nl + 1) / 2;
    const int ps = nlr + ((1 - nlr % 16) % 16 + 16) % 16;
    return SxPair{ps, nl | 1};
}
__host__ inline size_t sx_pair_smem(int ni, int nz)
{
    const SxPair L = sx_pair_layout(nz);
    return (2 * (size_t)ni * L.ps + (size_t)((ni + 1) / 2) * L.xs) * sizeof(float2);
}

template <typename T>
__global__ void __cluster_dims__(2, 1, 1) k_spectral_x_pair(KParams<T> p, typename V2<T>::t *spec, FftPlan pi,
                                                           const typename V2<T>::t *tw, SxPair lay)
{
    static_assert(sizeof(T) == 4, "the paired x kernel is FP32");
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float c_r[PPM_MAXZ], c_a[PPM_MAXZ], c_c[PPM_MAXZ], c_v[PPM_MAXZ];
    __shared__ double d_r[PPM_MAXZ], d_a[PPM_MAXZ], d_c[PPM_MAXZ], d_v[PPM_MAXZ];
    __shared__ double pcr_wk[PCR_WK];
    const int rank = (int)cluster.block_rank(), q = blockIdx.x / 2;
    const int nl = p.nz - 2, ni = p.ni, ps = lay.ps, xs = lay.xs;
    const int l0 = rank * ((nl + 1) / 2), l1 = rank ? nl : (nl + 1) / 2, nlr = l1 - l0;
    const int ol0 = rank ? 0 : (nl + 1) / 2;  // the peer's first level
    const int p0 = rank * ((ni + 1) / 2), p1 = rank ? ni : (ni + 1) / 2, np = p1 - p0;
    float2 *a = (float2 *)smem_raw, *b = a + (long)ni * ps, *X = b + (long)ni * ps;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    for (int k = tid; k < p.nz; k += nth) {
        c_r[k] = p.rhou[k]; c_a[k] = p.acoef[k]; c_c[k] = p.ccoef[k]; c_v[k] = p.vcoef[k];
        d_r[k] = p.rhou_d[k]; d_a[k] = p.acoef_d[k]; d_c[k] = p.ccoef_d[k]; d_v[k] = p.vcoef_d[k];
    }
    // this CTA's levels of every x line
    for (int i = threadIdx.y; i < ni; i += blockDim.y)
        for (int l = threadIdx.x; l < nlr; l += blockDim.x)
            cp_elem(a + i * ps + l, spec + ((long)i * p.nj + q) * p.nz + 1 + l0 + l, true);
    cp_wait_all_sync();
    float2 *r = fft_smem<float, float2>(a, b, nlr, pi, tw, false, ps);
    float2 *fr = (r == a) ? b : a;  // free: the Thomas coefficients
    cluster.sync();  // both halves transformed (both CTAs end in the same buffer)
    float2 *pr = cluster.map_shared_rank(r, rank ^ 1);
    // gather the columns p0 .. p1-1: own levels locally, the peer's from its shared memory
    for (int w = tid; w < np * nl; w += nth) {
        const int pc = w / nl, l = w % nl, pp = p0 + pc;
        const bool own = l >= l0 && l < l1;
        X[pc * xs + l] = own ? r[pp * ps + (l - l0)] : pr[pp * ps + (l - ol0)];
    }
    __syncthreads();
    const double size2d = (double)(ni * p.nj);
    const int aq = min(q, p.nj - q);
    const bool q_low = p.low_modes > 0 && aq < p.low_modes;
    {
        const float dx2 = (float)p.dx2, inv_s = (float)(1.0 / size2d);
        for (int pc = tid; pc < np; pc += nth) {
            const int pp = p0 + pc, ap = min(pp, ni - pp);
            if (q_low && ap < p.low_modes) continue;  // FP64 islands below
            const long col = (long)pp * p.nj + q;
            const float hb = 2.0f * (float)p.hcoef[col] / dx2;
            float *Fw = (float *)fr + (long)pc * xs - 1;  // nl floats per column
            thomas_column_fast(X + (long)pc * xs - 1, Fw, p.nz, hb, inv_s, c_r, c_a, c_c, c_v, col == 0);
        }
        if (q_low && (tid >> 5) == 0) {  // low (p, q) wavenumbers of this CTA: FP64 by warp PCR
            for (int pc = 0; pc < np; pc++) {
                const int pp = p0 + pc, ap = min(pp, ni - pp);
                if (ap >= p.low_modes) continue;
                const long col = (long)pp * p.nj + q;
                if (col == 0 && p.mean_inv) continue;
                pcr_column_f64(X + (long)pc * xs - 1, nl, p.hcoef[col], p.dx2, size2d, d_r, d_a, d_c, d_v,
                               col == 0, pcr_wk);
            }
        }
        if (q_low && q == 0 && p0 == 0 && p.mean_inv) {  // the mean mode: block-wide
            __syncthreads();
            mean_mode_solve(X - 1, nl, p.mean_inv, size2d, pcr_wk);
        }
    }
    __syncthreads();
    // the solved columns back to both CTAs' lines
    for (int w = tid; w < np * nl; w += nth) {
        const int pc = w / nl, l = w % nl, pp = p0 + pc;
        if (l >= l0 && l < l1) r[pp * ps + (l - l0)] = X[pc * xs + l];
        else pr[pp * ps + (l - ol0)] = X[pc * xs + l];
    }
    cluster.sync();  // every column written back
    float2 *o = fft_smem<float, float2>(r, fr, nlr, pi, tw, true, ps);
    for (int i = threadIdx.y; i < ni; i += blockDim.y)
        for (int l = threadIdx.x; l < nlr; l += blockDim.x) spec[((long)i * p.nj + q) * p.nz + 1 + l0 + l] = o[i * ps + l];
}

}  // namespace ga
