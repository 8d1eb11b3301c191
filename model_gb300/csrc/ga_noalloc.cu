// ga_noalloc.cu - pressure solve on caller-owned device arrays, without any
// device allocation.
//
// Some callers cannot allocate device memory at all: a host model that hands
// out every byte of GPU memory from its own pool, or a plugin loaded into a
// process whose allocator forbids foreign cudaMalloc calls.  For them,
// ga_solve_pressure_noalloc runs the FP64 anelastic pressure solve (the same
// kernels as the context path) with every intermediate in one fixed
// file-scope device array instead of context buffers.
//
// The array is GA_NOALLOC_SCRATCH_BYTES (32 MiB) and is reserved on every GPU
// that loads this library, for as long as the library stays loaded.  Every
// call shares it and it keeps the previous call's contents; nothing in it has
// to start at zero (each call writes every element it later reads).  Calls
// that overlap on the GPU (different streams, or different host threads
// without ordering) race on it.
//
// The caller's column arrays travel by value inside a kernel argument
// (NoallocColumns, 4 KiB), so a call reads no host memory after it returns
// and queues no host-to-device copy.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "ga_engine.h"
#include "ga_kernels.cuh"

namespace ga {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GA_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64] = {};  // device address of the scratch array, per device

static inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// The NZ-length columns the solve reads, passed by value (NZ <= 128).
struct NoallocColumns {
    double mu[128], mw[128], rhou[128], rhow[128];
};

// Twiddles, the (cos kx + cos ly - 2) table and the tridiagonal coefficients,
// computed on the device into the scratch tables, and the columns written from
// the kernel argument into the scratch (no host buffers needed).
__global__ void k_noalloc_tables(int ni, int nj, int nz, double dz, double2 *tw_i, double2 *tw_j,
                                 double *hcoef, const NoallocColumns cols, double *mu, double *mw,
                                 double *rhou, double *rhow, double *ac, double *cc, double *vc)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long nh = (long)ni * nj;
    if (t < nh) {
        const int p = (int)(t / nj), q = (int)(t % nj);
        hcoef[t] = cospi(2.0 * p / ni) + cospi(2.0 * q / nj) - 2.0;
    }
    if (t < ni) {
        double s, c;
        sincospi(2.0 * (double)t / (double)ni, &s, &c);
        tw_i[t] = make_double2(c, -s);
    }
    if (t < nj) {
        double s, c;
        sincospi(2.0 * (double)t / (double)nj, &s, &c);
        tw_j[t] = make_double2(c, -s);
    }
    if (t < nz) {  // init_fft3d, pressure.cpp:776-792 (stretched branch)
        const int k = (int)t;
        mu[k] = cols.mu[k];
        mw[k] = cols.mw[k];
        rhou[k] = cols.rhou[k];
        rhow[k] = cols.rhow[k];
        const double dz2 = dz * dz;
        double a = 0, c = 0, v = 0;
        if (k >= 1 && k < nz - 1) {
            a = cols.mu[k] * cols.mw[k] * cols.rhow[k] / dz2;
            c = cols.mu[k] * cols.mw[k + 1] * cols.rhow[k + 1] / dz2;
        }
        if (k == 1) a = 0;
        if (k == nz - 2) c = 0;
        if (k == 1) v = cols.mu[1] * cols.mw[2] * cols.rhow[2] / dz2;
        else if (k >= 2 && k < nz - 2)
            v = cols.mu[k] * (cols.mw[k + 1] * cols.rhow[k + 1] + cols.mw[k] * cols.rhow[k]) / dz2;
        else if (k == nz - 2) v = (cols.mu[nz - 2] * cols.mw[nz - 2] * cols.rhow[nz - 2]) / dz2;
        ac[k] = a;
        cc[k] = c;
        vc[k] = v;
    }
}

static FftPlan plan_for(int n)
{
    FftPlan P;
    std::memset(&P, 0, sizeof(P));
    P.n = n;
    int m = n;
    while (m % 4 == 0 && P.nfac < 23) { P.fac[P.nfac++] = 4; m /= 4; }
    for (int f = 2; m > 1 && P.nfac < 24;) {
        if (m % f == 0) { P.fac[P.nfac++] = f; m /= f; }
        else f = (f == 2) ? 3 : f + 2;
    }
    int ns = 1;
    for (int f = 0; f < P.nfac; f++) {
        P.nslog[f] = (ns & (ns - 1)) == 0 ? __builtin_ctz(ns) : -1;
        ns *= P.fac[f];
    }
    return P;
}

size_t noalloc_bytes_needed(const ga_config *c)
{
    const size_t ni = c->periodic_ew_boundaries ? c->nx - 6 : c->nx, nj = c->ny, nz = c->nz;
    return align256(16 * ni * nj * nz) + align256(16 * ni) + align256(16 * nj) + align256(8 * ni * nj) +
           7 * align256(8 * nz);
}

// Launch shapes of one call, fixed before anything is queued.
struct NoallocPlan {
    int ni, nj, KTy, KTx, nkt_y, nkt_x, ps, fused;
    size_t smem_y, smem_x, smem_spec, smem_th;
};

static const size_t kNoallocSmemOptin = 200 * 1024;
static const int kNoallocThomasCols = 64;

static NoallocPlan noalloc_plan(const ga_config *c)
{
    NoallocPlan P;
    const int NZ = c->nz;
    P.ni = c->periodic_ew_boundaries ? c->nx - 6 : c->nx;
    P.nj = c->ny;
    auto pow2_tile = [&](int n) {
        const long budget = 32 * 1024;
        long want = std::max(1L, budget / (long)(2 * n * sizeof(double2)));
        int kt = 1;
        while ((kt << 1) <= want && (kt << 1) <= 2 * (NZ - 2)) kt <<= 1;
        while (kt > 1 && (kt >> 1) >= NZ - 2) kt >>= 1;
        return kt;
    };
    P.KTy = pow2_tile(P.nj);
    P.KTx = pow2_tile(P.ni);
    P.smem_y = 2 * (size_t)P.nj * P.KTy * sizeof(double2);
    P.smem_x = 2 * (size_t)P.ni * P.KTx * sizeof(double2);
    P.nkt_y = (NZ - 2 + P.KTy - 1) / P.KTy;
    P.nkt_x = (NZ - 2 + P.KTx - 1) / P.KTx;
    const int nl = NZ - 2, m = 8;
    P.ps = nl + ((1 - nl % m) % m + m) % m;
    P.smem_spec = 2 * (size_t)P.ni * P.ps * sizeof(double2);
    P.fused = P.smem_spec <= kNoallocSmemOptin;
    P.smem_th = (size_t)kNoallocThomasCols * (NZ | 1) * (sizeof(double2) + sizeof(double));
    return P;
}

int noalloc_check(const ga_config *c, std::string *why)
{
    const size_t need = noalloc_bytes_needed(c);
    if (need > GA_NOALLOC_SCRATCH_BYTES) {
        *why = "grid needs " + std::to_string(need) + " bytes of scratch, more than the fixed " +
               std::to_string((size_t)GA_NOALLOC_SCRATCH_BYTES) + " bytes";
        return GA_ERR_ARG;
    }
    const NoallocPlan P = noalloc_plan(c);
    const size_t worst = std::max(P.smem_y, P.fused ? P.smem_spec : std::max(P.smem_x, P.smem_th));
    if (worst > kNoallocSmemOptin) {
        *why = "grid needs " + std::to_string(worst) + " bytes of shared memory per block, more than the " +
               std::to_string(kNoallocSmemOptin) + " bytes the transform kernels are set up for (NX or NY too long)";
        return GA_ERR_ARG;
    }
    return GA_OK;
}

// Set-up, once per device, with that device current: the device address of
// the scratch array and the shared-memory limits of the kernels this file
// launches.  The device is marked ready only when every step succeeded.
static int noalloc_setup(int dev, unsigned char **base)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            set_error(std::string("ga_solve_pressure_noalloc: cudaGetSymbolAddress failed: ") +
                      cudaGetErrorString(e));
            return GA_ERR_CUDA;
        }
        const int optin = (int)kNoallocSmemOptin;
        struct { const void *fn; const char *name; } kernels[] = {
            {(const void *)k_div_fft_y<double>, "k_div_fft_y"},
            {(const void *)k_ifft_y_pi<double>, "k_ifft_y_pi"},
            {(const void *)k_spectral_x<double>, "k_spectral_x"},
            {(const void *)k_fft_x<double>, "k_fft_x"},
            {(const void *)k_thomas<double>, "k_thomas"},
        };
        for (auto &k : kernels) {
            e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            if (e != cudaSuccess) {
                set_error(std::string("ga_solve_pressure_noalloc: setting the shared-memory limit of ") + k.name +
                          " failed: " + cudaGetErrorString(e));
                return GA_ERR_CUDA;
            }
        }
        g_noalloc_ptr[dev] = ptr;
    }
    *base = (unsigned char *)g_noalloc_ptr[dev];
    return GA_OK;
}

int solve_pressure_noalloc(const ga_config *c, const ga_columns *cols, double *up, double *vp, double *wp,
                           double *pi, double step, cudaStream_t stream)
{
    std::string why;
    if (noalloc_check(c, &why) != GA_OK) {
        set_error("ga_solve_pressure_noalloc: " + why);
        return GA_ERR_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        set_error("ga_solve_pressure_noalloc: no current CUDA device");
        return GA_ERR_CUDA;
    }
    unsigned char *base = nullptr;
    const int rc = noalloc_setup(dev, &base);
    if (rc != GA_OK) return rc;

    const int NX = c->nx, NY = c->ny, NZ = c->nz;
    const int periodic = c->periodic_ew_boundaries;
    const NoallocPlan P = noalloc_plan(c);
    const int ni = P.ni, nj = P.nj;
    typedef double2 T2;
    // carve the scratch array (the layout noalloc_bytes_needed counts)
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += align256(bytes);
        return p;
    };
    T2 *spec = (T2 *)take(16 * (size_t)ni * nj * NZ);
    T2 *tw_i = (T2 *)take(16 * (size_t)ni);
    T2 *tw_j = (T2 *)take(16 * (size_t)nj);
    double *hcoef = (double *)take(8 * (size_t)ni * nj);
    double *mu = (double *)take(8 * NZ), *mw = (double *)take(8 * NZ), *rhou = (double *)take(8 * NZ);
    double *rhow = (double *)take(8 * NZ), *ac = (double *)take(8 * NZ), *cc = (double *)take(8 * NZ);
    double *vc = (double *)take(8 * NZ);
    // columns by value: read from the caller's host arrays here, during the call
    NoallocColumns hc;
    std::memset(&hc, 0, sizeof(hc));
    std::memcpy(hc.mu, cols->mu, 8 * (size_t)NZ);
    std::memcpy(hc.mw, cols->mw, 8 * (size_t)NZ);
    std::memcpy(hc.rhou, cols->rhou, 8 * (size_t)NZ);
    std::memcpy(hc.rhow, cols->rhow, 8 * (size_t)NZ);
    {
        const long nt = std::max((long)ni * nj, (long)std::max(std::max(ni, nj), NZ));
        k_noalloc_tables<<<(int)((nt + 255) / 256), 256, 0, stream>>>(ni, nj, NZ, c->dz, tw_i, tw_j, hcoef, hc, mu,
                                                                       mw, rhou, rhow, ac, cc, vc);
    }
    KParams<double> kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.nx = NX; kp.ny = NY; kp.nz = NZ; kp.n = (long)NX * NY * NZ;
    kp.ni = ni; kp.nj = nj; kp.ioff = periodic ? 3 : 0; kp.periodic = periodic;
    kp.dt = c->dt;
    kp.one_d_dx = 1.0 / c->dx; kp.one_d_dy = 1.0 / c->dy; kp.one_d_dz = 1.0 / c->dz;
    kp.mu = mu; kp.mw = mw; kp.rhou = rhou; kp.rhow = rhow;
    kp.hcoef = hcoef;
    kp.acoef = ac; kp.ccoef = cc; kp.vcoef = vc;
    kp.acoef_d = ac; kp.ccoef_d = cc; kp.vcoef_d = vc; kp.rhou_d = rhou;
    kp.dx2 = c->dx * c->dx;
    kp.low_modes = 0;
    KFields<double> F;
    std::memset(&F, 0, sizeof(F));
    F.P[FU] = up; F.P[FV] = vp; F.P[FW] = wp; F.pi = pi;
    // lateral copies before the solve (mirror or periodic), as solve_pressure
    if (!periodic) {
        const long tot = 2L * (NX + NY - 2) * (NZ - 2);
        k_mirror_edges<double><<<(int)((tot + 255) / 256), 256, 0, stream>>>(kp, up, vp, wp);
    } else {
        const long tot = 6L * NY * NZ;
        k_periodic_copy<double><<<(int)((tot + 255) / 256), 256, 0, stream>>>(kp, up, vp, wp, (double *)nullptr);
    }
    // divergence + FFT along y
    const FftPlan pj = plan_for(nj), pi_plan = plan_for(ni);
    const dim3 by_y(P.KTy, std::max(1, 256 / P.KTy)), by_x(P.KTx, std::max(1, 256 / P.KTx));
    k_div_fft_y<double><<<dim3(P.nkt_y, ni), by_y, P.smem_y, stream>>>(kp, F, spec, pj, tw_j, step * c->dt, P.KTy);
    // FFT along x + Thomas + inverse FFT along x
    const int nl = NZ - 2;
    if (P.fused) {
        const int bx = std::min(nl, 64);
        k_spectral_x<double><<<nj, dim3(bx, std::max(1, 256 / bx)), P.smem_spec, stream>>>(kp, spec, pi_plan, tw_i,
                                                                                         P.ps);
    } else {
        const int TC = kNoallocThomasCols;
        k_fft_x<double><<<dim3(P.nkt_x, nj), by_x, P.smem_x, stream>>>(kp, spec, pi_plan, tw_i, 0, P.KTx);
        const long ncol = (long)ni * nj;
        k_thomas<double><<<(int)((ncol + TC - 1) / TC), TC, P.smem_th, stream>>>(kp, spec, TC);
        k_fft_x<double><<<dim3(P.nkt_x, nj), by_x, P.smem_x, stream>>>(kp, spec, pi_plan, tw_i, 1, P.KTx);
    }
    // inverse FFT along y + PI with the level copies and lateral placement
    k_ifft_y_pi<double><<<dim3(P.nkt_y, ni), by_y, P.smem_y, stream>>>(kp, F, spec, pj, tw_j, P.KTy);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("ga_solve_pressure_noalloc: launch failed: ") + cudaGetErrorString(e));
        return GA_ERR_CUDA;
    }
    return GA_OK;
}

}  // namespace ga
