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
// of y-lines; the tridiagonal solves run in the context's precision with
// elimination factors formed once on the host in FP64.  Non-periodic domains.
#pragma once
#include "ga_kernels.cuh"

namespace ga {

template <typename T>
struct HydArgs {
    const T *dzu, *dzw;    // DZU(k) = zsw[k+1]-zsw[k], DZW(k) = zsu[k]-zsu[k-1] (model.h:205-206)
    // the tridiagonal system of init_fft2d (pressure.cpp:621-641) does not
    // change during a run: its elimination factors P[j+1] = -ccoef[j]/denom
    // and 1/denom, denom = BCOEF(i,j) + acoef[j] P[j], are formed once on the
    // host (the reference's expressions, FP64, stored in the context's
    // precision: FP64 is scarce on this GPU, and the FP32 solve keeps the
    // FP32 step's accuracy), [ny+1][nx] and [ny][nx] (x-wavenumber fastest:
    // a warp of wavenumbers reads one row at a time)
    const T *pf, *rden;
    const T *ac;           // acoef [ny]
    T *pw;                 // work of the back substitution, [2][ny+1][nx] (real and imaginary Q)
    T *div;                // div_avg, [nx][ny]
    typename V2<T>::t *spec2;  // transformed div_avg, [ny][nx]
    T rhoavg;              // column-average density (column_average_density, initializer.cpp:1265-1282)
    T dz;
};

// The column kernels below hold HC columns per block with their levels in
// shared memory: the pointwise parts of each recurrence are formed by all
// threads with loads coalesced along k, then one thread per column runs the
// recurrence in the reference's order from shared memory.
constexpr int HC = 16, HC_THREADS = 128;

template <typename T>
__host__ __device__ constexpr size_t hyd_col_smem(int nz)
{
    return 2 * (size_t)HC * nz * sizeof(T);
}

// density-weighted column divergence of the forecast u, v (pressure.cpp:248-261)
template <typename T>
__global__ void __launch_bounds__(HC_THREADS) k_hyd_divavg(KParams<T> p, KFields<T> F, HydArgs<T> h, T step)
{
    extern __shared__ unsigned char hyd_smem[];
    T *term = (T *)hyd_smem;  // [HC][nz]
    const int nyi = p.ny - 2, nz = p.nz;
    const long ncol = (long)(p.nx - 2) * nyi, col0 = (long)blockIdx.x * HC;
    const T *UP = F.P[FU], *VP = F.P[FV];
    const long sx = (long)p.ny * nz, sy = nz;
    for (int w = threadIdx.x; w < HC * nz; w += blockDim.x) {
        const int cl = w / nz, k = w % nz;
        const long col = col0 + cl;
        if (col >= ncol || k < 1 || k >= nz - 1) continue;
        const int i = 1 + (int)(col / nyi), j = 1 + (int)(col % nyi);
        const long c = gix(p.ny, nz, i, j, k);
        term[cl * nz + k] =
            p.rhou[k] * h.dzu[k] * ((UP[c + sx] - UP[c]) * p.one_d_dx + (VP[c + sy] - VP[c]) * p.one_d_dy);
    }
    __syncthreads();
    const long col = col0 + threadIdx.x;
    if (threadIdx.x >= HC || col >= ncol) return;
    const int i = 1 + (int)(col / nyi), j = 1 + (int)(col % nyi);
    T d = T(0), zsum = T(0);
    for (int k = 1; k < nz - 1; k++) {
        d += term[threadIdx.x * nz + k];
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
                    v = h.spec2[(long)(j0 + l) * p.nx + i];
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
                h.spec2[(long)(j0 + l) * p.nx + i] = o;
            }
        }
}

// the tridiagonal solve along y of one x-wavenumber (pressure.cpp:675-700),
// real and imaginary parts, with the precomputed factors: each step
// of the recurrence is a multiply-subtract and a multiply by 1/denom (the
// reference divides by denom; the two differ by an ulp, well inside the
// transform's own rounding)
template <typename T>
__global__ void k_hyd_thomas(KParams<T> p, HydArgs<T> h)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nx) return;
    typedef typename V2<T>::t T2;
    const int nj = p.ny, nx = p.nx;
    // rows are [j][i]: each step of the recurrence is one coalesced row for
    // the warp; distinct arrays, so the loads of later rows may be issued
    // before the stores of earlier ones
    T *__restrict__ Qr = h.pw + i;
    T *__restrict__ Qi = h.pw + (long)(nj + 1) * nx + i;
    const T *__restrict__ P = h.pf + i;
    const T *__restrict__ R = h.rden + i;
    const T *__restrict__ ac = h.ac;
    T2 *__restrict__ x = h.spec2 + i;
    // each chunk's rows are loaded before its steps run, so a chunk waits on
    // memory once rather than once per step
    constexpr int CH = 16;
    T qr = T(0), qi = T(0);
    for (int j0 = 0; j0 < nj; j0 += CH) {
        T2 v[CH];
        T r[CH], av[CH];
#pragma unroll
        for (int t = 0; t < CH; t++) {
            const int j = min(j0 + t, nj - 1);
            v[t] = x[(long)j * nx];
            r[t] = R[(long)j * nx];
            av[t] = ac[j];
        }
#pragma unroll
        for (int t = 0; t < CH; t++) {
            const int j = j0 + t;
            if (j < nj) {
                qr = (v[t].x - av[t] * qr) * r[t];
                qi = (v[t].y - av[t] * qi) * r[t];
                Qr[(long)(j + 1) * nx] = qr;
                Qi[(long)(j + 1) * nx] = qi;
            }
        }
    }
    T xr = x[(long)(nj - 1) * nx].x, xi = x[(long)(nj - 1) * nx].y;
    for (int j1 = nj - 2; j1 >= 0; j1 -= CH) {
        T pj[CH], qrj[CH], qij[CH];
#pragma unroll
        for (int t = 0; t < CH; t++) {
            const int j = max(j1 - t, 0);
            pj[t] = P[(long)(j + 1) * nx];
            qrj[t] = Qr[(long)(j + 1) * nx];
            qij[t] = Qi[(long)(j + 1) * nx];
        }
#pragma unroll
        for (int t = 0; t < CH; t++) {
            const int j = j1 - t;
            if (j >= 0) {
                xr = pj[t] * xr + qrj[t];
                xi = pj[t] * xi + qij[t];
                x[(long)j * nx].x = xr;
                x[(long)j * nx].y = xi;
            }
        }
    }
}

// hydrostatic_pressure (pressure.cpp:453-537) from the current theta (and
// moisture), its density-weighted column average into level 0, the lid
// pressure (:285-286) into level NZ-1, and the total (:293-296)
template <typename T>
__global__ void __launch_bounds__(HC_THREADS) k_hyd_pi(KParams<T> p, KFields<T> F, HydArgs<T> h)
{
    extern __shared__ unsigned char hyd_smem[];
    const int nyi = p.ny - 2, nz = p.nz;
    T *g = (T *)hyd_smem;   // [HC][nz]: theta (times the water loading) / tbv^2
    T *ps = g + HC * nz;    // [HC][nz]: the integral, then the total
    const long ncol = (long)(p.nx - 2) * nyi, col0 = (long)blockIdx.x * HC;
    const T *TH = F.cur[FTH], *QV = F.cur[FQV], *QC = F.cur[FQC], *QR = F.cur[FQR];
    T *PI = F.pi;
    for (int w = threadIdx.x; w < HC * nz; w += blockDim.x) {
        const int cl = w / nz, k = w % nz;
        const long col = col0 + cl;
        if (col >= ncol || k < 1 || k >= nz - 1) continue;
        const long c = gix(p.ny, nz, 1 + (int)(col / nyi), 1 + (int)(col % nyi), k);
        T fac = p.moist ? (T(1.) + T(0.61) * QV[c] - QC[c] - QR[c]) : T(1);
        if (p.ice) fac = fac - F.cur[FQS][c] - F.cur[FQI][c];  // pressure.cpp:459-475
        g[cl * nz + k] = (TH[c] * fac) / (p.tbv[k] * p.tbv[k]);
    }
    __syncthreads();
    const T gcp = T(9.8 / 1004.0);
    const int cl = threadIdx.x;
    const long col = col0 + cl;
    if (cl < HC && col < ncol) {
        const int i = 1 + (int)(col / nyi), j = 1 + (int)(col % nyi);
        const T *gc = g + cl * nz;
        T *pc = ps + cl * nz;
        T up = -T(0.5) * gcp * gc[nz - 2] * h.dzw[nz - 1];
        pc[nz - 2] = up;
        for (int k = nz - 3; k > 0; k--) {
            up = up - T(0.5) * gcp * (gc[k + 1] + gc[k]) * h.dzw[k + 1];
            pc[k] = up;
        }
        T avg = T(0), zsum = T(0);
        for (int k = 1; k < nz - 1; k++) {
            avg += p.rhou[k] * p.tbv[k] * pc[k] * h.dzu[k];
            zsum += h.dzu[k];
        }
        avg /= zsum;
        pc[0] = avg;
        pc[nz - 1] = (h.div[(long)i * p.ny + j] - avg) / h.rhoavg;
    }
    __syncthreads();
    for (int w = threadIdx.x; w < HC * nz; w += blockDim.x) {
        const int c2 = w / nz, k = w % nz;
        const long cc = col0 + c2;
        if (cc >= ncol) continue;
        const long c = gix(p.ny, nz, 1 + (int)(cc / nyi), 1 + (int)(cc % nyi), k);
        const T *pc = ps + c2 * nz;
        PI[c] = (k == 0 || k == nz - 1) ? pc[k] : pc[k] + pc[nz - 1];
    }
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

// w_velocity_LH (solver.cpp:144-163) into the current w
template <typename T>
__global__ void __launch_bounds__(HC_THREADS) k_hyd_w(KParams<T> p, KFields<T> F, HydArgs<T> h)
{
    extern __shared__ unsigned char hyd_smem[];
    const int nyi = p.ny - 2, nz = p.nz;
    T *dv = (T *)hyd_smem;  // [HC][nz]: the horizontal convergence of level k
    T *ws = dv + HC * nz;   // [HC][nz]: w
    const long ncol = (long)(p.nx - 2) * nyi, col0 = (long)blockIdx.x * HC;
    const T *UP = F.P[FU], *VP = F.P[FV];
    const long sx = (long)p.ny * nz, sy = nz;
    for (int w = threadIdx.x; w < HC * nz; w += blockDim.x) {
        const int cl = w / nz, k = w % nz;
        const long col = col0 + cl;
        if (col >= ncol || k < 1 || k >= nz - 2) continue;
        const long c = gix(p.ny, nz, 1 + (int)(col / nyi), 1 + (int)(col % nyi), k);
        dv[cl * nz + k] = -(UP[c + sx] - UP[c]) * p.one_d_dx - (VP[c + sy] - VP[c]) * p.one_d_dy;
    }
    __syncthreads();
    const int cl = threadIdx.x;
    if (cl < HC && col0 + cl < ncol) {
        T *wc = ws + cl * nz;
        const T *dc = dv + cl * nz;
        wc[0] = T(0);
        wc[1] = T(0);
        wc[nz - 1] = T(0);
        T w = T(0);
        for (int k = 2; k < nz - 1; k++) {
            w = (p.rhow[k - 1] / p.rhow[k]) * w + (p.rhou[k - 1] / p.rhow[k]) * dc[k - 1] * h.dz / p.mu[k - 1];
            wc[k] = w;
        }
    }
    __syncthreads();
    T *W = F.cur[FW];
    for (int w = threadIdx.x; w < HC * nz; w += blockDim.x) {
        const int c2 = w / nz, k = w % nz;
        const long cc = col0 + c2;
        if (cc >= ncol) continue;
        W[gix(p.ny, nz, 1 + (int)(cc / nyi), 1 + (int)(cc % nyi), k)] = ws[c2 * nz + k];
    }
}

}  // namespace ga
