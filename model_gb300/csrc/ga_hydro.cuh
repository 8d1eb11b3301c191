// ga_hydro.cuh - the hydrostatic equation set (HYDROSTATIC): integrate_hydro
// (solver.cpp:33-80) advects u and v, solves for pressure with
// solve_hydrostatic_pressure (pressure.cpp:229-298) and applies the
// pressure-gradient force with the factor cp * tbv; w is diagnosed from the
// anelastic continuity equation after each stage (w_velocity_LH,
// solver.cpp:144-163) and lives in the current slot only.
//
// The pressure is a lid pressure plus the hydrostatic integral of the
// buoyancy.  The lid pressure solves a 2-D Poisson problem for the
// density-weighted column divergence (poisson_fft2d, pressure.cpp:652-715):
// a transform along x, scaled by 1/nx, one tridiagonal solve along y per
// x-wavenumber (whose back substitution leaves the last row at its
// transformed value), and the inverse transform.  The transforms reuse the
// shared-memory Stockham FFT of the 3-D solve (fft_smem), batched over a tile
// of y-lines; the tridiagonal solves run in FP64.  Non-periodic domains.
#pragma once
#include "ga_kernels.cuh"

namespace ga {

template <typename T>
struct HydArgs {
    const T *dzu, *dzw;    // DZU(k) = zsw[k+1]-zsw[k], DZW(k) = zsu[k]-zsu[k-1] (model.h:205-206)
    const double *bco;     // BCOEF(i, j) of init_fft2d (pressure.cpp:634-641), [nx][ny]
    const double *ac, *cc; // acoef, ccoef [ny]
    double *pw;            // tridiagonal work, [nx][ny+1] (P; real and imaginary Q follow)
    T *div;                // div_avg, [nx][ny]
    typename V2<T>::t *spec2;  // transformed div_avg, [nx][ny]
    T rhoavg;              // column-average density (column_average_density, initializer.cpp:1265-1282)
    T dz;
};

// density-weighted column divergence of the forecast u, v (pressure.cpp:248-261)
template <typename T>
__global__ void __launch_bounds__(256) k_hyd_divavg(KParams<T> p, KFields<T> F, HydArgs<T> h, T step)
{
    const int nyi = p.ny - 2;
    const long col = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (long)(p.nx - 2) * nyi) return;
    const int i = 1 + (int)(col / nyi), j = 1 + (int)(col % nyi);
    const T *UP = F.P[FU], *VP = F.P[FV];
    const long sx = (long)p.ny * p.nz, sy = p.nz;
    T d = T(0), zsum = T(0);
    for (int k = 1; k < p.nz - 1; k++) {
        const long c = gix(p.ny, p.nz, i, j, k);
        d += p.rhou[k] * h.dzu[k] * ((UP[c + sx] - UP[c]) * p.one_d_dx + (VP[c + sy] - VP[c]) * p.one_d_dy);
        zsum += h.dzu[k];
    }
    d /= (T(1004) * zsum * step * p.dt);
    h.div[(long)i * p.ny + j] = d;
}

// mirror_boundaries_2d (boundaries.cpp:331-345): the edges take their
// clamped interior neighbour (the corners the diagonal one, as the two
// passes of the reference leave them)
template <typename T>
__global__ void k_hyd_mirror2d(KParams<T> p, T *s)
{
    const int ne = 2 * (p.nx + p.ny - 2);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne) return;
    int i, j, e = t;
    if (e < p.ny) { i = 0; j = e; }
    else if ((e -= p.ny) < p.ny) { i = p.nx - 1; j = e; }
    else if ((e -= p.ny) < p.nx - 2) { i = 1 + e; j = 0; }
    else { e -= p.nx - 2; i = 1 + e; j = p.ny - 1; }
    const int si = min(max(i, 1), p.nx - 2), sj = min(max(j, 1), p.ny - 2);
    s[(long)i * p.ny + j] = s[(long)si * p.ny + sj];
}

// transform along x of L y-lines (block (L, any)): forward from div_avg with
// the 1/nx scaling, or inverse into div_avg (real part)
template <typename T>
__global__ void k_hyd_fft(KParams<T> p, HydArgs<T> h, FftPlan P, const typename V2<T>::t *tw, int inv, int L)
{
    typedef typename V2<T>::t T2;
    extern __shared__ unsigned char smem_raw[];
    T2 *a = (T2 *)smem_raw;
    T2 *b = a + (long)p.nx * L;
    const int j0 = blockIdx.x * L;
    const int lt = min(L, p.ny - j0);
    for (int i = threadIdx.y; i < p.nx; i += blockDim.y)
        for (int l = threadIdx.x; l < L; l += blockDim.x) {
            T2 v;
            if (l < lt) {
                if (inv) {
                    v = h.spec2[(long)i * p.ny + j0 + l];
                } else {
                    v.x = h.div[(long)i * p.ny + j0 + l];
                    v.y = T(0);
                }
            } else {
                v.x = T(0);
                v.y = T(0);
            }
            a[i * L + l] = v;
        }
    __syncthreads();
    T2 *r = fft_smem<T, T2>(a, b, L, P, tw, inv != 0, L);
    const T n = (T)p.nx;
    for (int i = threadIdx.y; i < p.nx; i += blockDim.y)
        for (int l = threadIdx.x; l < lt; l += blockDim.x) {
            const T2 v = r[i * L + l];
            if (inv) {
                h.div[(long)i * p.ny + j0 + l] = v.x;
            } else {
                T2 o;
                o.x = v.x / n;
                o.y = v.y / n;
                h.spec2[(long)i * p.ny + j0 + l] = o;
            }
        }
}

// the tridiagonal solve along y of one x-wavenumber (pressure.cpp:675-700),
// real and imaginary parts with the same P; in FP64
template <typename T>
__global__ void k_hyd_thomas(KParams<T> p, HydArgs<T> h)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nx) return;
    typedef typename V2<T>::t T2;
    const int nj = p.ny;
    double *P = h.pw + (long)i * 3 * (nj + 1), *Qr = P + (nj + 1), *Qi = Qr + (nj + 1);
    T2 *x = h.spec2 + (long)i * nj;
    const double *B = h.bco + (long)i * nj;
    P[0] = 0.0;
    Qr[0] = 0.0;
    Qi[0] = 0.0;
    for (int j = 0; j < nj; j++) {
        const double denom = B[j] + h.ac[j] * P[j];
        P[j + 1] = -h.cc[j] / denom;
        Qr[j + 1] = ((double)x[j].x - h.ac[j] * Qr[j]) / denom;
        Qi[j + 1] = ((double)x[j].y - h.ac[j] * Qi[j]) / denom;
    }
    double xr = (double)x[nj - 1].x, xi = (double)x[nj - 1].y;
    for (int j = nj - 2; j >= 0; j--) {
        xr = P[j + 1] * xr + Qr[j + 1];
        xi = P[j + 1] * xi + Qi[j + 1];
        x[j].x = (T)xr;
        x[j].y = (T)xi;
    }
}

// hydrostatic_pressure (pressure.cpp:453-537) from the current theta (and
// moisture), its density-weighted column average into level 0, the lid
// pressure (:285-286) into level NZ-1, and the total (:293-296); one thread
// per interior column
template <typename T>
__global__ void __launch_bounds__(128) k_hyd_pi(KParams<T> p, KFields<T> F, HydArgs<T> h)
{
    const int nyi = p.ny - 2, nz = p.nz;
    const long col = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (long)(p.nx - 2) * nyi) return;
    const int i = 1 + (int)(col / nyi), j = 1 + (int)(col % nyi);
    const long c0 = gix(p.ny, nz, i, j, 0);
    const T *TH = F.cur[FTH], *QV = F.cur[FQV], *QC = F.cur[FQC], *QR = F.cur[FQR];
    T *PI = F.pi;
    const T gcp = T(9.8 / 1004.0);
    auto fac = [&](int k) {
        return p.moist ? (T(1.) + T(0.61) * QV[c0 + k] - QC[c0 + k] - QR[c0 + k]) : T(1);
    };
    PI[c0 + nz - 1] = T(0);
    T up = -T(0.5) * gcp * ((TH[c0 + nz - 2] * fac(nz - 2)) / (p.tbv[nz - 2] * p.tbv[nz - 2])) * h.dzw[nz - 1];
    PI[c0 + nz - 2] = up;
    for (int k = nz - 3; k > 0; k--) {
        const T tup = (TH[c0 + k + 1] * fac(k + 1)) / (p.tbv[k + 1] * p.tbv[k + 1]);
        const T tdn = (TH[c0 + k] * fac(k)) / (p.tbv[k] * p.tbv[k]);
        up = up - T(0.5) * gcp * (tup + tdn) * h.dzw[k + 1];
        PI[c0 + k] = up;
    }
    T avg = T(0), zsum = T(0);
    for (int k = 1; k < nz - 1; k++) {
        avg += p.rhou[k] * p.tbv[k] * PI[c0 + k] * h.dzu[k];
        zsum += h.dzu[k];
    }
    avg /= zsum;
    PI[c0] = avg;
    const T lid = (h.div[(long)i * p.ny + j] - avg) / h.rhoavg;
    PI[c0 + nz - 1] = lid;
    for (int k = 1; k < nz - 1; k++) PI[c0 + k] += lid;
}

// the pressure-gradient force of integrate_hydro (solver.cpp:70-79) over
// [1,N-1) x [1,N-1) x [1,NZ-1)
template <typename T>
__global__ void __launch_bounds__(256) k_hyd_project(KParams<T> p, KFields<T> F, T step)
{
    const int nzi = p.nz - 2, nyi = p.ny - 2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)(p.nx - 2) * nyi * nzi) return;
    const int k = 1 + (int)(t % nzi);
    const int j = 1 + (int)((t / nzi) % nyi);
    const int i = 1 + (int)(t / ((long)nzi * nyi));
    const long c = gix(p.ny, p.nz, i, j, k), sx = (long)p.ny * p.nz, sy = p.nz;
    const T *PI = F.pi;
    F.P[FU][c] = F.P[FU][c] - step * (p.dtx * T(1004) * p.tbv[k] * (PI[c] - PI[c - sx]));
    F.P[FV][c] = F.P[FV][c] - step * (p.dty * T(1004) * p.tbv[k] * (PI[c] - PI[c - sy]));
}

// w_velocity_LH (solver.cpp:144-163) into the current w, one thread per
// interior column
template <typename T>
__global__ void __launch_bounds__(128) k_hyd_w(KParams<T> p, KFields<T> F, HydArgs<T> h)
{
    const int nyi = p.ny - 2, nz = p.nz;
    const long col = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (long)(p.nx - 2) * nyi) return;
    const int i = 1 + (int)(col / nyi), j = 1 + (int)(col % nyi);
    const long c0 = gix(p.ny, nz, i, j, 0), sx = (long)p.ny * nz, sy = nz;
    const T *UP = F.P[FU], *VP = F.P[FV];
    T *W = F.cur[FW];
    W[c0] = T(0);
    W[c0 + 1] = T(0);
    W[c0 + nz - 1] = T(0);
    T w = T(0);
    for (int k = 2; k < nz - 1; k++) {
        const long c = c0 + k - 1;
        w = (p.rhow[k - 1] / p.rhow[k]) * w +
            (p.rhou[k - 1] / p.rhow[k]) * (-(UP[c + sx] - UP[c]) * p.one_d_dx - (VP[c + sy] - VP[c]) * p.one_d_dy) *
                h.dz / p.mu[k - 1];
        W[c0 + k] = w;
    }
}

}  // namespace ga
