// ga_engine.cuh - host side of one precision: device buffers, the buffer
// rotation of the reference (solver.cpp:229-263, microphysics.cpp:642-669),
// the per-operator launch sequences and the fused RK3 step.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <tuple>
#include <string>
#include <vector>

#include "ga_engine.h"
#include "ga_kernels.cuh"
#include "ga_quad.cuh"
#include "ga_turb.cuh"
#include "ga_hydro.cuh"
#include "ga_ice.cuh"

#include <cudaTypedefs.h>

namespace ga {

static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

// Factor plan of the shared-memory FFT of length n.  order (autotuned):
// 0 radix 4 first, then 2, then odd primes; 1 the radix 2 first; 2 radix 2
// only; 3 odd primes first.  Returns nfac = 0 for an order that gives no new
// plan for this n.
static inline FftPlan make_fft_plan(int n, int order = 0)
{
    FftPlan P;
    std::memset(&P, 0, sizeof(P));
    P.n = n;
    int m = n, c4 = 0, c2 = 0, odd[24], no = 0;
    while (m % 4 == 0) { c4++; m /= 4; }
    if (m % 2 == 0) { c2 = 1; m /= 2; }
    for (int f = 3; m > 1 && no < 24;) {
        if (m % f == 0) { odd[no++] = f; m /= f; }
        else f += 2;
    }
    if (order == 1 && c2 == 0) return P;   // same as order 0
    if (order == 2) {
        if (c4 == 0) return P;
        c2 += 2 * c4;
        c4 = 0;
    }
    if (order == 3 && (no == 0 || (c4 == 0 && c2 == 0))) return P;
    auto push = [&](int f) { if (P.nfac < 24) P.fac[P.nfac++] = f; };
    if (order == 3)
        for (int t = 0; t < no; t++) push(odd[t]);
    if (order == 1)
        for (int t = 0; t < c2; t++) push(2);
    for (int t = 0; t < c4; t++) push(4);
    if (order != 1)
        for (int t = 0; t < c2; t++) push(2);
    if (order != 3)
        for (int t = 0; t < no; t++) push(odd[t]);
    int ns = 1;
    for (int f = 0; f < P.nfac; f++) {
        P.nslog[f] = (ns & (ns - 1)) == 0 ? __builtin_ctz(ns) : -1;
        ns *= P.fac[f];
    }
    return P;
}

template <typename T>
struct Lin;

template <typename T>
class Engine : public EngineBase {
    typedef typename V2<T>::t T2;

  public:
    ga_config cfg;
    int NX, NY, NZ;
    long N;
    int nprog;  // 4 dry, 7 with Kessler, 9 with the ice scheme (snow FQS, ice FQI)
    T *buf[9][3] = {};
    int ci[9], pi_[9], mi[9];  // rotation: which buffer is current / forecast / start-of-step
    T *pi = nullptr, *bar[6] = {}, *vt = nullptr;
    double *accrain = nullptr;
    // ice scheme (ga_ice.cuh): snow and ice fall speeds, accumulated snow, the
    // snow intercept (one value) and its per-point record of the last pass
    T *sts = nullptr, *its = nullptr, *n0s = nullptr, *n0s_pt = nullptr;
    double *accsnow = nullptr;
    int *n0s_idx = nullptr;
    T2 *spec = nullptr;
    T2 *tw_i = nullptr, *tw_j = nullptr;
    FftPlan plan_i, plan_j;
    std::vector<void *> allocs;
    KParams<T> kp;
    int *d_err = nullptr;
    unsigned char *ppm_has = nullptr;
    T *ppm_topq = nullptr, *ppm_topm = nullptr, *ppm_cin = nullptr, *ppm_carry = nullptr;
    double *staging = nullptr;
    int KTy = 1, KTx = 1, lgKTy = 0, lgKTx = 0, TC = 64;
    int psx = 0;  // point stride of the fused spectral-x kernel (0: unfused path)
    int sx_threads = 256;  // threads of a fused spectral-x block (autotuned)
    // FP32: the fused x kernel as clusters of two CTAs per y-wavenumber
    // (autotuned; GA_SPECTRAL_X=pair makes it the default)
    bool sx_pair = false;
    size_t smem_sxp = 0;
    size_t smem_y = 0, smem_x = 0, smem_th = 0, smem_sx = 0, smem_adv = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool bar_uniform[6] = {false, false, false, false, false, false};
    bool btab_dirty = true;
    T *btab = nullptr;
    long long graph_launches[2] = {0, 0};
    bool use_graphs = true;
    int status = GA_OK;
    std::unique_ptr<LinBase> lin;  // tangent-linear / adjoint buffers, on first use
    int adv_ti = ADV_TI, adv_tj = ADV_TJ;  // advection tile (autotuned)
    // the four-level advection kernel (FP32, uniform basic state, NZ % 4 == 0)
    // and its tile; GA_ADVECT=tile or =quad restricts both the default and the
    // autotuner to one kernel
    int adv_quad = 1, adv_qi = 4, adv_qj = 8, adv_force = 0;
    int adv_qb = 3;  // blocks per SM the four-level kernel's registers are sized for (3 or 4)
    int adv_rows = 0;  // four-level kernel: east and north faces by sliding rows (ADV_ROWS)
    // the four-level kernel with the current fields staged into shared memory
    // by the tensor memory accelerator (k_advect_tma), and its candidate
    int adv_tma = 0, adv_tmc = 0;
    double *budget_w = nullptr, *budget_part = nullptr;  // FP64 budget weights and partial sums
    T *diff_tend = nullptr;  // explicit diffusion: a second buffer for every prognostic field
    T *diff_buf[9] = {};     // (the one each field's diffused start-of-step values go to)
    const T *diff_w = nullptr;  // and the vertical finite-difference weights, order+1 per level
    // turbulence: coefficients, tendencies, tables (ga_turb.cuh); turb.kmix
    // is null when the scheme is off.  turb_sat is Kessler's saturation record.
    TurbArgs<T> turb{};
    unsigned char *turb_sat = nullptr;
    double *lin_vmax = nullptr;  // the linearised model's rescaling maximum
    HydArgs<T> hyd{};            // the hydrostatic equation set (hyd.div null when off)
    // a second stream for the theta and moisture advection, which needs
    // nothing of the stage's pressure solve and runs beside it (forked from
    // and joined back into `stream`; captured into the same graph).  On when
    // the x solve (one block per y-wavenumber) leaves SMs idle; GA_OVERLAP=0
    // or =1 overrides
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool overlap = true;
    // the adjoint's recorded steps copy each stage's start fields to the tape
    // on the second stream, beside the stage that only reads them
    bool overlap_rec = true;
    std::function<void()> mid_solve;  // queued by poisson() after its first launch
    // launches inside run on the second stream (the launch helpers use `stream`)
    struct OnSide {
        Engine *e;
        explicit OnSide(Engine *x) : e(x) { std::swap(e->stream, e->stream2); }
        ~OnSide() { std::swap(e->stream, e->stream2); }
    };
    struct OnSideIf {
        Engine *e;
        bool on;
        OnSideIf(Engine *x, bool o) : e(x), on(o)
        {
            if (on) std::swap(e->stream, e->stream2);
        }
        ~OnSideIf()
        {
            if (on) std::swap(e->stream, e->stream2);
        }
    };
    void fork()
    {
        cudaEventRecord(ev_fork, stream);
        cudaStreamWaitEvent(stream2, ev_fork, 0);
    }
    void join()
    {
        cudaEventRecord(ev_join, stream2);
        cudaStreamWaitEvent(stream, ev_join, 0);
    }
    int hyd_L = 1;               // y-lines per block of its x transforms

    // Fornberg's recurrence for finite-difference weights: c[i*(m+1)+d] is the
    // weight of point x[i] in derivative d at z (util.cpp:199-247)
    static void fornberg(double z, const double *x, int n, int m, double *c)
    {
        double c1 = 1.0, c4 = x[0] - z;
        c[0] = 1.0;
        for (int i = 1; i <= n; i++) {
            const int mn = std::min(i, m);
            double c2 = 1.0;
            const double c5 = c4;
            c4 = x[i] - z;
            for (int j = 0; j <= i - 1; j++) {
                const double c3 = x[i] - x[j];
                c2 = c2 * c3;
                if (j == i - 1) {
                    for (int d = mn; d >= 1; d--)
                        c[i * (m + 1) + d] =
                            c1 * (d * c[(i - 1) * (m + 1) + d - 1] - c5 * c[(i - 1) * (m + 1) + d]) / c2;
                    c[i * (m + 1)] = -c1 * c5 * c[(i - 1) * (m + 1)] / c2;
                }
                for (int d = mn; d >= 1; d--)
                    c[j * (m + 1) + d] = (c4 * c[j * (m + 1) + d] - d * c[j * (m + 1) + d - 1]) / c3;
                c[j * (m + 1)] = c4 * c[j * (m + 1)] / c3;
            }
            c1 = c2;
        }
    }
    // the weights of init_diffusion_weights (damping.cpp:158-270) on heights h:
    // the order's derivative at k in [order/2, NZ-order/2) from levels
    // k-order/2 .. k+order/2 of the heights scaled by the local spacing; 4th-
    // order rows at k = 2 and NZ-3 (order 6), 2nd-order rows at k = 1 and NZ-2
    // (orders 4 and 6)
    static std::vector<double> diffusion_weights(int order, const double *h, int nz)
    {
        std::vector<double> w((size_t)(order + 1) * nz, 0.0), hs(nz, 0.0), c(64);
        for (int k = order / 2; k < nz - order / 2; k++) {
            for (int n = 0; n < nz; n++) hs[n] = (h[n] - h[k]) / (h[k + 1] - h[k]);
            std::fill(c.begin(), c.end(), 0.0);
            fornberg(hs[k], hs.data() - order / 2 + k, order, order, c.data());
            for (int j = 0; j <= order; j++) w[(size_t)(order + 1) * k + j] = c[(order + 1) * j + order];
        }
        const int rows[2][2] = {{2, nz - 3}, {1, nz - 2}};
        for (int pass = 0; pass < 2; pass++) {
            const int lower = pass == 0 ? 4 : 2;
            if (order <= lower) continue;
            for (int r = 0; r < 2; r++) {
                const int k = rows[pass][r];
                const int top = (pass == 0 && r == 0) ? nz - 1 : nz;  // damping.cpp:200 rescales to NZ-2
                for (int n = 0; n < top; n++) hs[n] = (h[n] - h[k]) / (h[k + 1] - h[k]);
                std::fill(c.begin(), c.end(), 0.0);
                fornberg(hs[k], hs.data() - lower / 2 + k, lower, lower, c.data());
                for (int j = 0; j <= lower; j++) w[(size_t)(order + 1) * k + j] = c[(lower + 1) * j + lower];
            }
        }
        return w;
    }
    std::map<std::tuple<const void *, int, int, int>, CUtensorMap> tma_maps;  // per buffer and box
    // the four-level post-processing kernel (FP32, NZ % 4 == 0); GA_POST=column
    // keeps the per-level one
    bool post_quad = true;
    // the step's last four-level pass also runs Kessler (rain_fallout 1);
    // GA_KESSLER=separate keeps the separate kernel
    bool kes_fused = true, post_kes = false;
    unsigned char *qmask = nullptr;         // clipping record of the next advection (linearisation)
    int plan_order_i = 0, plan_order_j = 0;

    Lin<T> *linear();
    int lin_supported() const;
    int lin_set_field(int field, int slot, const double *host, size_t n) override;
    int lin_get_field(int field, int slot, double *host, size_t n) override;
    int tlm_step(int nsteps) override;
    int adjoint(int nsteps, int checkpoint_every) override;

    template <typename X>
    X *dalloc(size_t n)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, n * sizeof(X) ? n * sizeof(X) : 1) != cudaSuccess) {
            status = GA_ERR_NOMEM;
            return nullptr;
        }
        cudaMemset(p, 0, n * sizeof(X));
        allocs.push_back(p);
        return (X *)p;
    }
    template <typename X>
    X *upload(const std::vector<X> &h)
    {
        X *d = dalloc<X>(h.size());
        if (d) cudaMemcpy(d, h.data(), h.size() * sizeof(X), cudaMemcpyHostToDevice);
        return d;
    }
    template <typename X>
    const T *col_T(const X *src, int n)
    {
        std::vector<T> h(n);
        for (int k = 0; k < n; k++) h[k] = (T)src[k];
        return upload(h);
    }

    Engine(const ga_config *c, const ga_columns *cols) : cfg(*c)
    {
        NX = c->nx; NY = c->ny; NZ = c->nz;
        N = (long)NX * NY * NZ;
        if (N >= (1L << 31)) { status = GA_ERR_CONFIG; return; }
        device = c->device;
        if (cudaSetDevice(device) != cudaSuccess) { status = GA_ERR_CUDA; return; }
        if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) { status = GA_ERR_CUDA; return; }
        // the second stream at the lowest priority: the solve's blocks, on the
        // step's critical path, are dispatched first as SMs free up
        int prio_lo = 0, prio_hi = 0;
        cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
        if (cudaStreamCreateWithPriority(&stream2, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming) != cudaSuccess) {
            status = GA_ERR_CUDA;
            return;
        }
        {
            int nsm = 0;
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
            overlap = c->ny <= nsm;  // kp.nj = NY blocks in the x solve
            if (const char *ev = std::getenv("GA_OVERLAP")) overlap_rec = overlap = std::strcmp(ev, "0") != 0;
        }
        const bool moist = c->microphysics_option >= 1;
        const bool ice = c->microphysics_option == 2;
        nprog = ice ? 9 : moist ? 7 : 4;
        for (int f = 0; f < 9; f++) {
            const int nb = f < nprog ? 3 : 0;
            for (int s = 0; s < nb; s++) buf[f][s] = dalloc<T>(N);
            ci[f] = 0; pi_[f] = 1; mi[f] = 2;
        }
        pi = dalloc<T>(N);
        for (int b = 0; b < 6; b++) bar[b] = dalloc<T>(N);
        vt = dalloc<T>(N);
        accrain = dalloc<double>((size_t)NX * NY);
        d_err = dalloc<int>(2);  // [0] Kessler, [1] staging (kErrStaging)
        const int periodic = c->periodic_ew_boundaries;
        const int ni = periodic ? NX - 6 : NX, nj = NY;
        spec = dalloc<T2>((size_t)ni * nj * NZ);
        btab = dalloc<T>((size_t)BT_COUNT * NZ);

        // ---- scalars (initialize_globals, initializer.cpp:168-179) ----
        const double dx = c->dx, dy = c->dy, dz = c->dz, dt = c->dt;
        std::memset(&kp, 0, sizeof(kp));
        kp.nx = NX; kp.ny = NY; kp.nz = NZ; kp.n = N;
        kp.ni = ni; kp.nj = nj; kp.ioff = periodic ? 3 : 0;
        kp.periodic = periodic; kp.moist = moist; kp.rf = c->rain_fallout;
        kp.dtx = (T)(dt / dx); kp.dty = (T)(dt / dy); kp.dtz = (T)(dt / dz); kp.dt = (T)dt;
        kp.one_d_dx = (T)(1.0 / dx); kp.one_d_dy = (T)(1.0 / dy); kp.one_d_dz = (T)(1.0 / dz);
        kp.mu = col_T(cols->mu, NZ); kp.mw = col_T(cols->mw, NZ);
        kp.rhou = col_T(cols->rhou, NZ); kp.rhow = col_T(cols->rhow, NZ);
        kp.one_d_rhou = col_T(cols->one_d_rhou, NZ);
        kp.tb = col_T(cols->tb, NZ); kp.tbv = col_T(cols->tbv, NZ); kp.qb = col_T(cols->qb, NZ);
        kp.f = col_T(cols->f, NY); kp.zsw = col_T(cols->zsw, NZ);
        kp.rhou1 = (T)cols->rhou[1];
        if (ice) {  // the ice scheme's state (initializer.cpp:457-466, rutledge.cpp:90)
            kp.ice = 1;
            kp.rfall = (T)(2115.0 * std::pow(0.01, 0.2) * 17.83786);  // rutledge.cpp:140
            kp.pib = col_T(cols->pib, NZ);
            sts = dalloc<T>(N);
            its = dalloc<T>(N);
            accsnow = dalloc<double>((size_t)NX * NY);
            n0s = upload(std::vector<T>(1, (T)8e6));
            n0s_pt = dalloc<T>(N);
            n0s_idx = dalloc<int>(1);
            if (n0s_idx) cudaMemset(n0s_idx, 0xff, sizeof(int));  // -1: no snowy point recorded
        }

        // ---- Rayleigh coefficients (damping.cpp:1150-1162) ----
        const double trigpi = 3.14159265358979324;
        std::vector<double> ru(NZ, 0.0), rw(NZ, 0.0);
        kp.raylevel = c->rayleigh_damping_z;
        if (kp.raylevel >= 0 && kp.raylevel < NZ) {
            double raydmpcoef = 0.05, raydmpz = cols->zu[kp.raylevel];
            for (int k = kp.raylevel; k < NZ; k++) {
                ru[k] = raydmpcoef * 0.5 * (1.0 - cos(trigpi * (cols->zu[k] - raydmpz) / (cols->zu[NZ - 1] - raydmpz)));
                rw[k] = raydmpcoef * 0.5 * (1.0 - cos(trigpi * (cols->zw[k] - raydmpz) / (cols->zw[NZ - 1] - raydmpz)));
            }
        } else {
            kp.raylevel = NZ;
        }
        kp.ray_u = col_T(ru.data(), NZ); kp.ray_w = col_T(rw.data(), NZ);

        // ---- sponge (init_boundaries, boundaries.cpp:44-114; cos_profile util.cpp:740) ----
        auto cos_profile = [&](double pl, double ph, double frac, double shift) {
            if (frac >= 0 && frac <= 1.0) return cos(pl * 2 * trigpi + (ph - pl) * 2 * trigpi * frac) + shift;
            return 0.0;
        };
        const int ie = c->boundary_width_east, iw = c->boundary_width_west;
        const int jn = c->boundary_width_north, js = c->boundary_width_south;
        std::vector<double> ce(ie + 1), cw(iw + 1), cn(jn + 1), cs(js + 1);
        for (int i = 0; i < ie; i++) ce[i] = 0.5 * cos_profile(-0.5, 0, (double)(i + 1) / (double)ie, 1);
        for (int i = 0; i < iw; i++) cw[i] = 0.5 * cos_profile(0, 0.5, (double)i / (double)iw, 1);
        for (int i = 0; i < jn; i++) cn[i] = 0.5 * cos_profile(-0.5, 0, (double)(i + 1) / (double)jn, 1);
        for (int i = 0; i < js; i++) cs[i] = 0.5 * cos_profile(0, 0.5, (double)i / (double)js, 1);
        kp.ce = col_T(ce.data(), ie + 1); kp.cw = col_T(cw.data(), iw + 1);
        kp.cn = col_T(cn.data(), jn + 1); kp.cs = col_T(cs.data(), js + 1);
        kp.eb = NX - ie; kp.ee = NX; kp.wb = 0; kp.we = iw;
        kp.nb = NY - jn; kp.ne = NY; kp.sb = 0; kp.se = js;

        // ---- pressure solver tables (init_fft3d, pressure.cpp:724-797) ----
        std::vector<double> hcoef((size_t)ni * nj), kw(ni), lw(nj);
        for (int i = 0; i < ni; i++) kw[i] = (double)i * 2 * trigpi / ((double)ni);
        for (int j = 0; j < nj; j++) lw[j] = (double)j * 2 * trigpi / ((double)nj);
        for (int i = 0; i < ni; i++)
            for (int j = 0; j < nj; j++) hcoef[(size_t)i * nj + j] = cos(kw[i]) + cos(lw[j]) - 2.0;
        kp.hcoef = upload(hcoef);
        std::vector<double> ac(NZ, 0.0), cc(NZ, 0.0), vc(NZ, 0.0);
        const double dz2 = dz * dz;
        const double *mu = cols->mu, *mw = cols->mw, *rhow = cols->rhow;
        for (int k = 1; k < NZ - 1; k++) {
            ac[k] = mu[k] * mw[k] * rhow[k] / dz2;
            cc[k] = mu[k] * mw[k + 1] * rhow[k + 1] / dz2;
        }
        ac[1] = 0;
        cc[NZ - 2] = 0;
        vc[1] = mu[1] * mw[2] * rhow[2] / dz2;
        for (int k = 2; k < NZ - 2; k++) vc[k] = mu[k] * (mw[k + 1] * rhow[k + 1] + mw[k] * rhow[k]) / dz2;
        vc[NZ - 2] = (mu[NZ - 2] * mw[NZ - 2] * rhow[NZ - 2]) / dz2;
        kp.acoef = col_T(ac.data(), NZ); kp.ccoef = col_T(cc.data(), NZ); kp.vcoef = col_T(vc.data(), NZ);
        kp.acoef_d = upload(ac); kp.ccoef_d = upload(cc); kp.vcoef_d = upload(vc);
        kp.rhou_d = upload(std::vector<double>(cols->rhou, cols->rhou + NZ));
        {  // budget weights: density times cell volume, rhou[k] dx dy dz / mu[k]
            std::vector<double> wk(NZ);
            for (int k = 0; k < NZ; k++) wk[k] = cols->rhou[k] * dx * c->dy * c->dz / cols->mu[k];
            budget_w = upload(wk);
            budget_part = dalloc<double>((size_t)BUDGET_BLOCKS * GA_NB + GA_NB);
        }
        if (c->hydrostatic) {  // init_fft2d (pressure.cpp:601-645), column_average_density
            kp.hydrostatic = 1;
            std::vector<double> du(NZ, 0.0), dw(NZ, 0.0);
            for (int k = 0; k + 1 < NZ; k++) du[k] = cols->zsw[k + 1] - cols->zsw[k];
            for (int k = 1; k < NZ; k++) dw[k] = cols->zsu[k] - cols->zsu[k - 1];
            hyd.dzu = col_T(du.data(), NZ);
            hyd.dzw = col_T(dw.data(), NZ);
            double r = 0, zsum = 0;
            for (int k = 1; k < NZ - 1; k++) {
                r = r + cols->rhou[k] * cols->tbv[k] * du[k];
                zsum += du[k];
            }
            hyd.rhoavg = (T)(r / zsum);
            hyd.dz = (T)dz;
            std::vector<double> ac(NY, 1. / (dy * dy)), cc(NY, 1. / (dy * dy));
            std::vector<double> pf((size_t)NX * (NY + 1), 0.0), rden((size_t)NX * NY);
            ac[0] = 0;
            cc[NY - 1] = 0;
            for (int i = 0; i < NX; i++) {  // layouts [j][i]
                const double kw = i < NX / 2 ? 2 * trigpi * (double)i / NX : 2 * trigpi * (double)(NX - i) / NX;
                double Pj = 0.0;
                for (int j = 0; j < NY; j++) {
                    const double b = j == 0 ? -cols->rhow[2] / (dx * dx)
                                            : 2. * (cos(kw) - 1.) / (dx * dx) - cc[j] - ac[j];
                    const double denom = b + ac[j] * Pj;
                    Pj = -cc[j] / denom;
                    pf[(size_t)(j + 1) * NX + i] = Pj;
                    rden[(size_t)j * NX + i] = 1.0 / denom;
                }
            }
            hyd.pf = col_T(pf.data(), (int)pf.size());
            hyd.rden = col_T(rden.data(), (int)rden.size());
            hyd.ac = col_T(ac.data(), NY);
            hyd.pw = dalloc<T>((size_t)NX * 2 * (NY + 1));
            hyd.div = dalloc<T>((size_t)NX * NY);
            hyd.spec2 = dalloc<T2>((size_t)NX * NY);
            hyd_L = (int)std::max<size_t>(1, std::min<size_t>(8, 49152 / (2 * (size_t)NX * sizeof(T2))));
        }
        if (c->linear_model) {  // linear_integrate_rk3: eager steps (a rescaling may fall on any step)
            kp.linear = 1;
            use_graphs = false;
            lin_vmax = dalloc<double>(1);
        }
        if (c->turbulence_option) {  // init_kmix (turbulence.cpp:85-151)
            cudaFuncSetAttribute(k_turb_tend_tile<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            turb.kmix = dalloc<T>(N);
            turb.khmix = dalloc<T>(N);
            const int nt = std::min(nprog, 7);  // no tendencies of snow or ice (turbulence.cpp:233-290)
            T *tt = dalloc<T>((size_t)nt * N);
            for (int f = 0; f < 7; f++) turb.tend[f] = f < nt ? tt + (size_t)f * N : nullptr;
            if (moist) turb_sat = dalloc<unsigned char>(N);
            turb.sat = turb_sat;
            std::vector<double> l2(NZ, 0.0), kv(NZ, 0.0);
            for (int k = 1; k < NZ; k++) {
                const double dzk = cols->zsu[k] - cols->zsu[k - 1];
                l2[k] = dzk > 200.0 ? 200.0 * 200.0 : dzk * dzk;  // lv_max = 200 m
                kv[k] = 0.15 * l2[k] / dt;                         // cmixv_max = 0.15
            }
            turb.l2 = col_T(l2.data(), NZ);
            turb.kvmax = col_T(kv.data(), NZ);
            turb.tbw = col_T(cols->tbw, NZ);
            turb.kmixh_max = (T)(0.05 * dx * dx / dt);  // cmixh_max = 0.05
            turb.lH = (T)(dx / 4.0);
            const double wt = c->water_temp + 273.15;
            turb.water_temp = (T)wt;
            turb.es_water = (T)(611.2 * exp(17.67 * (wt - 273.15) / (wt - 29.65)));
            turb.dp_to_surface = (T)(9.8 * cols->zsu[1] / (1004.0 * cols->tbv[1]));
            turb.surface_flux = c->use_surface_heat_flux && moist;
        }
        if (c->use_explicit_diffusion) {
            diff_tend = dalloc<T>((size_t)nprog * N);
            for (int f = 0; f < nprog; f++) diff_buf[f] = diff_tend + (size_t)f * N;
            const std::vector<double> w = diffusion_weights(c->diffusion_order, cols->zsu, NZ);
            diff_w = col_T(w.data(), (int)w.size());
        }
        kp.dx2 = dx * dx;
        kp.low_modes = sizeof(T) == 8 ? 0 : 1;  // FP32: the mean mode (0,0) solves in FP64
        if (const char *ev = std::getenv("GA_LOW_MODES"))  // FP32: |p|, |q| below this solve in FP64
            if (sizeof(T) == 4) kp.low_modes = std::max(0, std::atoi(ev));
        kp.mean_inv = nullptr;
        if (sizeof(T) == 4 && kp.low_modes > 0) {
            // the mean mode's system, rows = levels 1..NZ-2 as the FP64 reduction
            // builds them (top row replaced by x = 0), inverted column by
            // column with the Thomas algorithm in extended precision
            const int nl = NZ - 2;
            std::vector<long double> a(nl), b(nl), c(nl), f(nl), y(nl);
            for (int r = 0; r < nl; r++) {
                const int k = r + 1;
                a[r] = ac[k];
                b[r] = cols->rhou[k] * 2.0 * hcoef[0] / kp.dx2 - vc[k];
                c[r] = cc[k];
            }
            a[nl - 1] = 0; b[nl - 1] = 1; c[nl - 1] = 0;
            std::vector<double> inv((size_t)nl * nl);
            for (int jc = 0; jc < nl; jc++) {
                long double den = b[0];
                f[0] = c[0] / den;
                y[0] = (jc == 0 ? 1.0L : 0.0L) / den;
                for (int r = 1; r < nl; r++) {
                    den = b[r] - a[r] * f[r - 1];
                    f[r] = c[r] / den;
                    y[r] = ((r == jc ? 1.0L : 0.0L) - a[r] * y[r - 1]) / den;
                }
                for (int r = nl - 2; r >= 0; r--) y[r] -= f[r] * y[r + 1];
                for (int r = 0; r < nl; r++) inv[(size_t)r * nl + jc] = (double)y[r];
            }
            kp.mean_inv = upload(inv);
        }

        // ---- FFT plans and twiddles ----
        plan_i = make_fft_plan(ni);
        plan_j = make_fft_plan(nj);
        auto twiddles = [&](int n) {
            std::vector<T2> h(n);
            for (int t = 0; t < n; t++) {
                const double a = 6.283185307179586476925286766559 * (double)t / (double)n;
                h[t].x = (T)cos(a);
                h[t].y = (T)(-sin(a));
            }
            return upload(h);
        };
        tw_i = twiddles(ni);
        tw_j = twiddles(nj);
        // power-of-two level tiles for the y and x transforms (~32 KiB per buffer)
        auto pow2_tile = [&](int n, int *lg) {
            const long budget = 32 * 1024;
            long want = std::max(1L, budget / (long)(2 * n * sizeof(T2)));
            int kt = 1, l = 0;
            while ((kt << 1) <= want && (kt << 1) <= 2 * (NZ - 2)) { kt <<= 1; l++; }
            while (kt > 1 && (kt >> 1) >= NZ - 2) { kt >>= 1; l--; }
            *lg = l;
            return kt;
        };
        KTy = pow2_tile(nj, &lgKTy);
        KTx = pow2_tile(ni, &lgKTx);
        smem_y = 2 * (size_t)nj * KTy * sizeof(T2);
        smem_x = 2 * (size_t)ni * KTx * sizeof(T2);
        smem_th = (size_t)TC * (NZ | 1) * (sizeof(T2) + sizeof(T));
        const int optin = 200 * 1024;
        {   // fused x transform + Thomas when all levels of a wavenumber fit.  The
            // point stride is padded to 1 mod (banks per element) so the Thomas
            // threads, one per x-wavenumber, hit distinct banks.
            const int nl = NZ - 2;
            const int m = 32 / (int)(sizeof(T2) / 4);
            const int ps = nl + ((1 - nl % m) % m + m) % m;
            if (2 * (size_t)ni * ps * sizeof(T2) <= (size_t)optin) psx = ps;
            else if (2 * (size_t)ni * (nl | 1) * sizeof(T2) <= (size_t)optin) psx = nl | 1;
            smem_sx = 2 * (size_t)ni * psx * sizeof(T2);
        }
        cudaFuncSetAttribute(k_spectral_x<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_spectral_x_1k<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        smem_adv = advect_tile_smem(adv_ti, adv_tj, NZ, sizeof(T));
        cudaFuncSetAttribute(k_advect_tile<T, 4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_tile<T, 2, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_tile<T, 4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_tile<T, 4, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_tile<T, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (const char *ev = std::getenv("GA_ADVECT")) {
            if (!std::strcmp(ev, "tile")) adv_force = 1;
            else if (!std::strcmp(ev, "quad")) adv_force = 2;
            else if (!std::strcmp(ev, "tma")) adv_force = 3;
        }
        if (const char *ev = std::getenv("GA_ADVECT_TMA")) {  // default staged candidate 0..3
            const int c = std::atoi(ev);
            if (c >= 0 && c < 4) adv_tmc = c;
        }
        adv_tma = adv_force == 3;
        adv_quad = adv_force != 1;
        if (const char *ev = std::getenv("GA_ADVECT_BLOCKS")) adv_qb = std::atoi(ev) == 4 ? 4 : 3;
        if (const char *ev = std::getenv("GA_ADVECT_TILE")) {  // default four-level tile, "TIxTJ"
            int a = 0, b = 0;
            if (std::sscanf(ev, "%dx%d", &a, &b) == 2)
                for (auto &tl : kQuadTiles)
                    if (tl[0] == a && tl[1] == b) { adv_qi = a; adv_qj = b; }
        }
        if (const char *ev = std::getenv("GA_ADVECT_FACES")) adv_rows = !std::strcmp(ev, "rows");
        if (const char *ev = std::getenv("GA_SPECTRAL_X"))  // fused x block of 1024 threads by default
            if (!std::strcmp(ev, "1024")) sx_threads = 1024;
        if (const char *ev = std::getenv("GA_POST")) post_quad = std::strcmp(ev, "column") != 0;
        post_quad = post_quad && sizeof(T) == 4 && NZ % 4 == 0;
        if (const char *ev = std::getenv("GA_KESSLER")) kes_fused = std::strcmp(ev, "separate") != 0;
        if constexpr (sizeof(T) == 4) {
            smem_sxp = sx_pair_smem(kp.ni, NZ);
            cudaFuncSetAttribute(k_spectral_x_pair<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            const char *ev = std::getenv("GA_SPECTRAL_X");
            sx_pair = ev && !std::strcmp(ev, "pair") && pair_ok();
        }
        if constexpr (sizeof(T) == 4) {
            for (auto &tl : kQuadTiles) quad_attr(tl[0], tl[1], optin);
            tma_attr(optin);
        }
        cudaFuncSetAttribute(k_div_fft_y<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_ifft_y_pi<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_fft_x<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_thomas<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);

        if (moist && c->rain_fallout == 2) {
            const long ncol = (long)(NX - 2) * (NY - 2);
            ppm_has = dalloc<unsigned char>(ncol);
            ppm_topq = dalloc<T>(ncol);
            ppm_topm = dalloc<T>(ncol);
            ppm_cin = dalloc<T>(ncol);
            ppm_carry = dalloc<T>(1);
        }
        if (cudaDeviceSynchronize() != cudaSuccess && status == GA_OK) status = GA_ERR_CUDA;
    }

    ~Engine() override
    {
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        for (auto &g : graph)
            if (g) cudaGraphExecDestroy(g);
        for (void *p : allocs) cudaFree(p);
        if (staging) cudaFree(staging);
        if (stream2) cudaStreamSynchronize(stream2);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (stream2) cudaStreamDestroy(stream2);
        if (stream) cudaStreamDestroy(stream);
    }

    KFields<T> fields() const
    {
        KFields<T> F;
        std::memset(&F, 0, sizeof(F));
        for (int f = 0; f < 9; f++) {
            F.cur[f] = buf[f][ci[f]];
            F.P[f] = buf[f][pi_[f]];
            F.M[f] = buf[f][mi[f]];
        }
        for (int b = 0; b < 6; b++) F.bar[b] = bar[b];
        F.pi = pi;
        F.vt = vt;
        F.accrain = accrain;
        F.sts = sts;
        F.its = its;
        F.accsnow = accsnow;
        F.n0s = n0s;
        F.n0s_pt = n0s_pt;
        F.n0s_idx = n0s_idx;
        F.qmask = qmask;
        F.sat = turb_sat;
        if (hyd.div) F.P[FW] = F.M[FW] = F.cur[FW];  // w lives in the current slot (boundaries.cpp:152-156)
        return F;
    }

    T *host_field(int field, int slot, long *n)
    {
        *n = N;
        if (field >= 0 && field < GA_NPROG) {
            if (field >= nprog) return nullptr;
            if (slot == GA_SLOT_CUR) return buf[field][ci[field]];
            if (slot == GA_SLOT_P) return buf[field][pi_[field]];
            if (slot == GA_SLOT_M) return buf[field][mi[field]];
            return nullptr;
        }
        switch (field) {
        case GA_PI: return pi;
        case GA_UBAR: case GA_VBAR: case GA_WBAR: case GA_THBAR: case GA_QBAR: case GA_PBAR:
            return bar[field - GA_UBAR];
        case GA_VT: return vt;
        case GA_KMIX: return turb.kmix;
        case GA_KHMIX: return turb.kmix ? turb.khmix : nullptr;
        case GA_UFRIC: case GA_VFRIC: case GA_WFRIC: case GA_THDIFF: case GA_QVDIFF: case GA_QCDIFF: case GA_QRDIFF:
            return turb.kmix ? turb.tend[field - GA_UFRIC] : nullptr;
        case GA_QS: case GA_QI: {
            if (!kp.ice) return nullptr;
            const int f = field == GA_QS ? FQS : FQI;
            if (slot == GA_SLOT_CUR) return buf[f][ci[f]];
            if (slot == GA_SLOT_P) return buf[f][pi_[f]];
            if (slot == GA_SLOT_M) return buf[f][mi[f]];
            return nullptr;
        }
        case GA_VTS: return sts;
        case GA_VTI: return its;
        case GA_N0S: *n = 1; return n0s;
        }
        return nullptr;
    }

    void *field_ptr(int field, int slot) override
    {
        if (field == GA_ACCRAIN) return accrain;
        if (field == GA_ACCSNOW) return accsnow;
        long n;
        return host_field(field, slot, &n);
    }

    int ensure_staging()
    {
        if (!staging && cudaMalloc(&staging, N * sizeof(double)) != cudaSuccess) return GA_ERR_NOMEM;
        return GA_OK;
    }

    // the saturation record as 0 / 1 values
    int sat_field(double *get, const double *set, size_t n)
    {
        if (!turb_sat || n != (size_t)N) return GA_ERR_ARG;
        std::vector<unsigned char> h(N);
        if (set) {
            for (long x = 0; x < N; x++) h[x] = set[x] != 0;
            cudaMemcpyAsync(turb_sat, h.data(), N, cudaMemcpyHostToDevice, stream);
            return sync_status();
        }
        cudaMemcpyAsync(h.data(), turb_sat, N, cudaMemcpyDeviceToHost, stream);
        const int rc = sync_status();
        for (long x = 0; x < N; x++) get[x] = h[x];
        return rc;
    }

    int set_field(int field, int slot, const double *host, size_t n) override
    {
        if (!host) return GA_ERR_ARG;
        cudaSetDevice(device);
        if (field == GA_SATURATED) return sat_field(nullptr, host, n);
        if (field == GA_ACCRAIN || (field == GA_ACCSNOW && accsnow)) {
            if (n != (size_t)NX * NY) return GA_ERR_ARG;
            cudaMemcpyAsync(field == GA_ACCRAIN ? accrain : accsnow, host, n * sizeof(double),
                            cudaMemcpyHostToDevice, stream);
            return sync_status();
        }
        if (field == GA_N0S && n0s) {
            if (n != 1) return GA_ERR_ARG;
            const T v = (T)host[0];
            cudaMemcpyAsync(n0s, &v, sizeof(T), cudaMemcpyHostToDevice, stream);
            return sync_status();
        }
        long nn;
        T *d = host_field(field, slot, &nn);
        if (!d || (long)n != nn) return GA_ERR_ARG;
        if (field >= GA_UBAR && field <= GA_PBAR) {
            // a basic state that depends on k only takes the tabulated path
            bool uni = true;
            for (long c = 1; c < (long)NX * NY && uni; c++)
                uni = std::memcmp(host + c * NZ, host, NZ * sizeof(double)) == 0;
            bar_uniform[field - GA_UBAR] = uni;
            btab_dirty = true;
            drop_graphs();
        }
        if (sizeof(T) == sizeof(double)) {
            cudaMemcpyAsync(d, host, n * sizeof(double), cudaMemcpyHostToDevice, stream);
        } else {
            if (ensure_staging() != GA_OK) return GA_ERR_NOMEM;
            cudaMemcpyAsync(staging, host, n * sizeof(double), cudaMemcpyHostToDevice, stream);
            k_convert_in<T><<<cdiv(n, 256), 256, 0, stream>>>(d, staging, (long)n);
            launches++;
        }
        return sync_status();
    }

    int get_field(int field, int slot, double *host, size_t n) override
    {
        if (!host) return GA_ERR_ARG;
        cudaSetDevice(device);
        if (field == GA_SATURATED) return sat_field(host, nullptr, n);
        if (field == GA_ACCRAIN || (field == GA_ACCSNOW && accsnow)) {
            if (n != (size_t)NX * NY) return GA_ERR_ARG;
            cudaMemcpyAsync(host, field == GA_ACCRAIN ? accrain : accsnow, n * sizeof(double),
                            cudaMemcpyDeviceToHost, stream);
            return sync_status();
        }
        if (field == GA_N0S && n0s) {
            if (n != 1) return GA_ERR_ARG;
            T v = T(0);
            cudaMemcpyAsync(&v, n0s, sizeof(T), cudaMemcpyDeviceToHost, stream);
            const int rc = sync_status();
            host[0] = (double)v;
            return rc;
        }
        long nn;
        T *d = host_field(field, slot, &nn);
        if (!d || (long)n != nn) return GA_ERR_ARG;
        if (sizeof(T) == sizeof(double)) {
            cudaMemcpyAsync(host, d, n * sizeof(double), cudaMemcpyDeviceToHost, stream);
        } else {
            if (ensure_staging() != GA_OK) return GA_ERR_NOMEM;
            k_convert_out<T><<<cdiv(n, 256), 256, 0, stream>>>(staging, d, (long)n);
            launches++;
            cudaMemcpyAsync(host, staging, n * sizeof(double), cudaMemcpyDeviceToHost, stream);
        }
        return sync_status();
    }

    int sync_status()
    {
        cudaError_t e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) {
            set_error(std::string("CUDA: ") + cudaGetErrorString(e));
            return GA_ERR_CUDA;
        }
        return staging_status();
    }

    int launch_status()
    {
        if (status != GA_OK) return status;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(std::string("CUDA launch: ") + cudaGetErrorString(e));
            return GA_ERR_CUDA;
        }
        return GA_OK;
    }

    void drop_graphs()
    {
        for (auto &g : graph)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
        if (lin) lin->drop_graphs();
    }

    // per-level basic-state tables (k_base_tables) when the basic state is
    // horizontally uniform; rebuilt after any basic-state field changes
    void refresh_base()
    {
        if (!btab_dirty) return;
        btab_dirty = false;
        const bool adv = bar_uniform[0] && bar_uniform[1] && bar_uniform[2] && bar_uniform[3] && bar_uniform[4];
        const bool kes = bar_uniform[3] && bar_uniform[4] && bar_uniform[5];
        if (adv || kes) {
            k_base_tables<T><<<cdiv(NZ, 128), 128, 0, stream>>>(kp, bar[0], bar[1], bar[2], bar[3], bar[4], bar[5],
                                                               btab);
            launches++;
        }
        kp.btab = btab;
        kp.ubase_adv = adv && !cfg.linear_model;  // the tables hold the full-velocity faces only
        kp.ubase_kes = kes;
    }

    // ------------------------------------------------------------------ ops
    // the advection tiles the autotuner chooses from
    static constexpr int kAdvTiles[5][2] = {{4, 4}, {2, 4}, {4, 2}, {4, 8}, {8, 4}};
    template <int TI, int TJ>
    void launch_advect_tile(T step, T sdtg, int what)
    {
        dim3 grid(cdiv(NX - 6, TI), cdiv(NY - 6, TJ));
        k_advect_tile<T, TI, TJ><<<grid, 256, smem_adv, stream>>>(kp, fields(), step, sdtg, what);
    }

    // the four-level kernel's tiles the autotuner chooses from
    static constexpr int kQuadTiles[5][2] = {{4, 4}, {4, 8}, {8, 4}, {2, 8}, {8, 8}};
    template <int TI, int TJ>
    void launch_advect_quad(T step, T sdtg, int what)
    {
        if constexpr (sizeof(T) == 4) {
            dim3 grid(cdiv(NX - 6, TI), cdiv(NY - 6, TJ));
            const size_t sm = advect_quad_smem(TI, TJ, NZ);
            if (adv_qb == 4) k_advect_quad<TI, TJ, 4><<<grid, AQ_THREADS, sm, stream>>>(kp, fields(), step, sdtg, what);
            else k_advect_quad<TI, TJ, 3><<<grid, AQ_THREADS, sm, stream>>>(kp, fields(), step, sdtg, what);
        }
    }
    template <int TI, int TJ>
    static void quad_attr_t(int optin)
    {
        cudaFuncSetAttribute(k_advect_quad<TI, TJ, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_quad<TI, TJ, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    }
    static void quad_attr(int ti, int tj, int optin)
    {
        if (ti == 4 && tj == 4) quad_attr_t<4, 4>(optin);
        else if (ti == 4 && tj == 8) quad_attr_t<4, 8>(optin);
        else if (ti == 8 && tj == 4) quad_attr_t<8, 4>(optin);
        else if (ti == 2 && tj == 8) quad_attr_t<2, 8>(optin);
        else if (ti == 8 && tj == 8) quad_attr_t<8, 8>(optin);
    }
    // the staged kernel's candidates: tile, level slab and the blocks per SM
    // its registers are sized for (its shared memory admits as many, moist,
    // for NZ up to 64)
    struct TmaCand {
        int ti, tj, kz, mb;
    };
    static constexpr TmaCand kTmaCands[4] = {{4, 4, 8, 4}, {4, 8, 8, 2}, {8, 8, 8, 2}, {4, 4, 16, 2}};

    // cuTensorMapEncodeTiled from the driver, looked up once per process
    static PFN_cuTensorMapEncodeTiled_v12000 tma_encoder()
    {
        static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
        static bool looked = false;
        if (!looked) {
            looked = true;
            void *ptr = nullptr;
            cudaDriverEntryPointQueryResult q;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                    cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
                fn = (PFN_cuTensorMapEncodeTiled_v12000)ptr;
        }
        return fn;
    }
    // the tensor map of one [NX][NY][NZ] FP32 buffer with a box of bk x bj x bi
    // points (k, j, i), cached per buffer and box
    bool tma_map(const T *ptr, int bi, int bj, int bk, CUtensorMap *out)
    {
        const auto key = std::make_tuple((const void *)ptr, bi, bj, bk);
        auto it = tma_maps.find(key);
        if (it != tma_maps.end()) {
            *out = it->second;
            return true;
        }
        PFN_cuTensorMapEncodeTiled_v12000 enc = tma_encoder();
        if (!enc) return false;
        CUtensorMap m;
        const cuuint64_t dims[3] = {(cuuint64_t)NZ, (cuuint64_t)NY, (cuuint64_t)NX};
        const cuuint64_t strides[2] = {(cuuint64_t)NZ * sizeof(T), (cuuint64_t)NY * NZ * sizeof(T)};
        const cuuint32_t box[3] = {(cuuint32_t)bk, (cuuint32_t)bj, (cuuint32_t)bi};
        const cuuint32_t estr[3] = {1, 1, 1};
        const CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)ptr, dims, strides, box, estr,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
        tma_maps[key] = m;
        *out = m;
        return true;
    }
    template <int TI, int TJ, int KZ, int MB>
    void launch_advect_tma(T step, T sdtg, int what)
    {
        if constexpr (sizeof(T) == 4) {
            using A = AQTma<TI, TJ, KZ>;
            const int nf = kp.moist ? 7 : 4;
            KFields<T> F = fields();
            TmaMaps maps;
            std::memset(&maps, 0, sizeof(maps));
            for (int f = 0; f < nf; f++)
                if (!tma_map(F.cur[f], A::BI, A::BJ, A::BK, &maps.m[f])) {
                    status = GA_ERR_CUDA;
                    set_error("advection: cuTensorMapEncodeTiled failed");
                    return;
                }
            dim3 grid(cdiv(NX - 6, TI), cdiv(NY - 6, TJ), cdiv(NZ, KZ));
            const size_t sm = advect_tma_smem(TI, TJ, KZ, NZ, nf);
            k_advect_tma<TI, TJ, KZ, MB><<<grid, AQ_THREADS, sm, stream>>>(maps, kp, F, step, sdtg, what, d_err + 1);
        }
    }
    void launch_advect_tma_cand(int c, T step, T sdtg, int what)
    {
        switch (c) {
        case 0: launch_advect_tma<4, 4, 8, 4>(step, sdtg, what); break;
        case 1: launch_advect_tma<4, 8, 8, 2>(step, sdtg, what); break;
        case 2: launch_advect_tma<8, 8, 8, 2>(step, sdtg, what); break;
        default: launch_advect_tma<4, 4, 16, 2>(step, sdtg, what); break;
        }
    }
    static void tma_attr(int optin)
    {
        cudaFuncSetAttribute(k_advect_tma<4, 4, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_tma<4, 8, 8, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_tma<8, 8, 8, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_advect_tma<4, 4, 16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    }
    // the staged kernel applies where the four-level one does, with the
    // driver's tensor-map encoder and the candidate's shared memory
    bool tma_ok(int c) const
    {
        // the staged boxes hold the seven fields of the Kessler step, not snow and ice
        if (!(sizeof(T) == 4 && kp.ubase_adv && NZ % 4 == 0 && c >= 0 && c < 4 && !kp.ice && tma_encoder()))
            return false;
        const TmaCand &t = kTmaCands[c];
        return advect_tma_smem(t.ti, t.tj, t.kz, NZ, kp.moist ? 7 : 4) <= 200 * 1024;
    }
    // the staging bit of the device error word (a bounded wait ran out)
    int staging_status()
    {
        int e = 0;
        cudaMemcpy(&e, d_err + 1, sizeof(int), cudaMemcpyDeviceToHost);
        if (e & kErrStaging) {
            set_error("advection: a shared-memory staging copy did not complete within its bound");
            return GA_ERR_CUDA;
        }
        return GA_OK;
    }

    // the paired x kernel applies: FP32, the fused path, its shared memory
    bool pair_ok() const { return sizeof(T) == 4 && psx > 0 && smem_sxp <= 200 * 1024; }
    // the four-level kernel applies: FP32, basic state a function of height,
    // whole quads of levels, face columns within the shared-memory limit
    bool quad_ok(int ti, int tj) const
    {
        return sizeof(T) == 4 && kp.ubase_adv && NZ % 4 == 0 && advect_quad_smem(ti, tj, NZ) <= 200 * 1024;
    }

    // apply_explicit_diffusion (damping.cpp:1125-1146) on the start-of-step slot
    void diffuse(double step)
    {
        const int order = cfg.diffusion_order;
        if (!diff_tend || !diff_w || (order != 2 && order != 4 && order != 6)) return;
        ProfScope ps(this, PC_DIFFUSION, 1);
        const long tot = N * nprog;
        const int nb = (int)std::min((tot + 255) / 256, 152L * 16);
        KFields<T> F = fields();
        DiffOut<T> o;
        for (int f = 0; f < 9; f++) o.out[f] = (f < nprog && !(f == FW && hyd.div)) ? diff_buf[f] : nullptr;
        k_diffuse_into<T><<<nb, 256, 0, stream>>>(kp, F, o, nprog, order, (T)cfg.kdiffh, (T)cfg.kdiffv, diff_w,
                                                  (T)step);
        // the diffused copy becomes the start-of-step slot; two steps swap
        // back, so a captured two-step graph leaves the pointers as it found them
        for (int f = 0; f < nprog; f++)
            if (o.out[f]) std::swap(buf[f][mi[f]], diff_buf[f]);
        launches += 1;
    }

    // solve_pressure of the hydrostatic set (pressure.cpp:142-170, 229-298)
    void hyd_solve(double step)
    {
        KFields<T> F = fields();
        ProfScope ps(this, PC_THOMAS, 8);
        const long e3 = 2L * (NX + NY - 2) * (NZ - 2);
        k_mirror_edges<T><<<cdiv(e3, 256), 256, 0, stream>>>(kp, F.P[FU], F.P[FV], F.P[FV]);
        const long ncol = (long)(NX - 2) * (NY - 2);
        const size_t hs = hyd_col_smem<T>(NZ);
        k_hyd_divavg<T><<<cdiv(ncol, HC), HC_THREADS, hs, stream>>>(kp, F, hyd, (T)step);
        k_hyd_mirror2d<T><<<cdiv(2L * (NX + NY - 2), 256), 256, 0, stream>>>(kp, hyd.div);
        const size_t sm = 2 * (size_t)NX * hyd_L * sizeof(T2);
        const dim3 fb(hyd_L, std::max(1, 256 / hyd_L));
        k_hyd_fft<T><<<cdiv(NY, hyd_L), fb, sm, stream>>>(kp, hyd, plan_i, tw_i, 0, hyd_L);
        k_hyd_thomas<T><<<cdiv(NX, 64), 64, 0, stream>>>(kp, hyd);
        k_hyd_fft<T><<<cdiv(NY, hyd_L), fb, sm, stream>>>(kp, hyd, plan_i, tw_i, 1, hyd_L);
        k_hyd_pi<T><<<cdiv(ncol, HC), HC_THREADS, hs, stream>>>(kp, F, hyd);
        k_mirror_edges<T><<<cdiv(e3, 256), 256, 0, stream>>>(kp, pi, pi, pi);
        launches += 8;
    }
    void hyd_project(double step)
    {
        const long tot = (long)(NX - 2) * (NY - 2) * (NZ - 2);
        k_hyd_project<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, fields(), (T)step);
        launches++;
    }
    void hyd_w()
    {
        const long ncol = (long)(NX - 2) * (NY - 2);
        k_hyd_w<T><<<cdiv(ncol, HC), HC_THREADS, hyd_col_smem<T>(NZ), stream>>>(kp, fields(), hyd);
        launches++;
    }

    // calculate_diff_tend (turbulence.cpp:158-188) from the start-of-step slot
    void turbulence()
    {
        if (!turb.kmix) return;
        ProfScope ps(this, PC_TURBULENCE, 2);
        KFields<T> F = fields();
        const int kx = (NZ + 31) / 32 * 32, cy = std::max(1, 256 / kx);
        const long ncol = (long)(NX - 2) * (NY - 2);
        const size_t sm = (size_t)cy * kx * (sizeof(T) + 1);
        k_turb_kmix<T><<<cdiv(ncol, cy), dim3(kx, cy), sm, stream>>>(kp, F, turb);
        const size_t st = turb_tile_smem(NZ, sizeof(T));
        if (st <= 200 * 1024) {
            const dim3 g(cdiv(NX - 2, TT_TI), cdiv(NY - 2, TT_TJ));
            k_turb_tend_tile<T><<<g, 256, st, stream>>>(kp, F, turb);
        } else {
            const long tot = (long)(NX - 2) * (NY - 2) * (NZ - 2);
            k_turb_tend<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, F, turb);
        }
        launches += 2;
    }
    // the tendencies' share of an RK stage (apply_*_diffusion, :233-290)
    void turb_apply(int what, double step)
    {
        if (!turb.kmix) return;
        ProfScope ps(this, PC_TURBULENCE, 1);
        const long tot = (long)(NX - 2) * (NY - 2) * (NZ - 2);
        k_turb_apply<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, fields(), turb, what, (T)(step * cfg.dt), (T)step);
        launches++;
    }

    void advect(double step, int what)
    {
        const double sdtg = step * cfg.dt * 9.8 * 0.5;  // step*dt*grav*0.5, advection.cpp:330
        ProfScope ps(this, PC_ADVECT, 1);
        if (adv_quad && adv_tma && tma_ok(adv_tmc)) {
            launch_advect_tma_cand(adv_tmc, (T)step, (T)sdtg, what);
        } else if (adv_quad && quad_ok(adv_qi, adv_qj)) {
            const T st = (T)step, sg = (T)sdtg;
            const int wq = what | (adv_rows ? ADV_ROWS : 0);
            if (adv_qi == 4 && adv_qj == 4) launch_advect_quad<4, 4>(st, sg, wq);
            else if (adv_qi == 8 && adv_qj == 4) launch_advect_quad<8, 4>(st, sg, wq);
            else if (adv_qi == 2) launch_advect_quad<2, 8>(st, sg, wq);
            else if (adv_qi == 8) launch_advect_quad<8, 8>(st, sg, wq);
            else launch_advect_quad<4, 8>(st, sg, wq);
        } else if (smem_adv <= 200 * 1024) {
            const T st = (T)step, sg = (T)sdtg;
            if (adv_ti == 2) launch_advect_tile<2, 4>(st, sg, what);
            else if (adv_tj == 2) launch_advect_tile<4, 2>(st, sg, what);
            else if (adv_tj == 8) launch_advect_tile<4, 8>(st, sg, what);
            else if (adv_ti == 8) launch_advect_tile<8, 4>(st, sg, what);
            else launch_advect_tile<4, 4>(st, sg, what);
        } else {  // face tiles of very tall columns do not fit: per-point form
            const long tot = (long)(NX - 6) * (NY - 6) * (NZ - 2);
            k_advect<T><<<cdiv(tot, 128), 128, 0, stream>>>(kp, fields(), (T)step, (T)sdtg, what);
        }
        launches++;
    }

    void edges_uvw()
    {
        KFields<T> F = fields();
        ProfScope ps(this, PC_EDGES, 1);
        if (!kp.periodic) {
            const long tot = 2L * (NX + NY - 2) * (NZ - 2);
            k_mirror_edges<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, F.P[FU], F.P[FV], F.P[FW]);
        } else {
            const long tot = 6L * NY * NZ;
            k_periodic_copy<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, F.P[FU], F.P[FV], F.P[FW], (T *)nullptr);
        }
        launches++;
    }

    void poisson(double step)
    {
        KFields<T> F = fields();
        const T sdt = (T)(step * cfg.dt);
        const int nkt_y = cdiv(NZ - 2, KTy), nkt_x = cdiv(NZ - 2, KTx);
        const dim3 by_y(KTy, std::max(1, 256 / KTy)), by_x(KTx, std::max(1, 256 / KTx));
        {
            ProfScope ps(this, PC_DIV_FFT_Y, 1);
            k_div_fft_y<T><<<dim3(nkt_y, kp.ni), by_y, smem_y, stream>>>(kp, F, spec, plan_j, tw_j, sdt, KTy);
        }
        if (mid_solve) {  // work queued beside the rest of the solve (the x solve leaves SMs idle)
            auto fn = std::move(mid_solve);
            mid_solve = nullptr;
            fn();
        }
        if (psx > 0) {
            ProfScope ps(this, PC_THOMAS, 1);
            const int nl = NZ - 2, bx = std::min(nl, 64);
            bool pair = false;
            if constexpr (sizeof(T) == 4) pair = sx_pair && pair_ok();
            if (pair) {
                if constexpr (sizeof(T) == 4) {
                    const int bh = std::min((nl + 1) / 2, 32);
                    k_spectral_x_pair<T><<<2 * kp.nj, dim3(bh, std::max(1, sx_threads / bh)), smem_sxp, stream>>>(
                        kp, spec, plan_i, tw_i, sx_pair_layout(NZ));
                }
            } else if (sx_threads > 512) {
                k_spectral_x_1k<T><<<kp.nj, dim3(bx, sx_threads / bx), smem_sx, stream>>>(kp, spec, plan_i, tw_i, psx);
            } else {
                k_spectral_x<T><<<kp.nj, dim3(bx, std::max(1, sx_threads / bx)), smem_sx, stream>>>(kp, spec, plan_i,
                                                                                                   tw_i, psx);
            }
            launches += 1;
        } else {
            {
                ProfScope ps(this, PC_FFT_X, 1);
                k_fft_x<T><<<dim3(nkt_x, kp.nj), by_x, smem_x, stream>>>(kp, spec, plan_i, tw_i, 0, KTx);
            }
            const long ncol = (long)kp.ni * kp.nj;
            {
                ProfScope ps(this, PC_THOMAS, 1);
                k_thomas<T><<<cdiv(ncol, TC), 256, smem_th, stream>>>(kp, spec, TC);  // 256 threads stage, TC solve
            }
            {
                ProfScope ps(this, PC_FFT_X, 1);
                k_fft_x<T><<<dim3(nkt_x, kp.nj), by_x, smem_x, stream>>>(kp, spec, plan_i, tw_i, 1, KTx);
            }
            launches += 3;
        }
        {
            ProfScope ps(this, PC_IFFT_Y_PI, 1);
            k_ifft_y_pi<T><<<dim3(nkt_y, kp.ni), by_y, smem_y, stream>>>(kp, F, spec, plan_j, tw_j, KTy);
        }
        launches += 2;
    }

    void solve_pressure(double step)
    {
        edges_uvw();
        poisson(step);
    }

    // per-field flags for k_post (nfields up to 9: snow and ice last); pcopy
    // selects the periodic two-pass form.  Snow and ice take a second pass of
    // the same kernel, in the slots of cloud water and rain, whose clipping,
    // sponge and top/bottom conditions they share (microphysics.cpp:675-700,
    // boundaries.cpp:200-284).
    void post(const int *flags, int nfields, double step, bool pcopy)
    {
        int fl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int f = 0; f < nfields && f < 7; f++) fl[f] = f < nprog ? flags[f] : 0;
        post_pass(fields(), fl, step, pcopy);
        if (nprog == 9 && nfields == 9 && (flags[FQS] | flags[FQI])) {
            KFields<T> F = fields();
            F.cur[FQC] = F.cur[FQS]; F.P[FQC] = F.P[FQS]; F.M[FQC] = F.M[FQS];
            F.cur[FQR] = F.cur[FQI]; F.P[FQR] = F.P[FQI]; F.M[FQR] = F.M[FQI];
            int fi[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            fi[FQC] = flags[FQS] & (PF_ZERO | PF_SPONGE | PF_VBC | PF_WRITE_M);
            fi[FQR] = flags[FQI] & (PF_ZERO | PF_SPONGE | PF_VBC | PF_WRITE_M);
            const bool kes = post_kes;
            post_kes = false;
            post_pass(F, fi, step, pcopy);
            post_kes = kes;
        }
    }

    void post_pass(const KFields<T> &F, const int *fl, double step, bool pcopy)
    {
        if (!(fl[0] | fl[1] | fl[2] | fl[3] | fl[4] | fl[5] | fl[6])) return;
        int4 a = make_int4(fl[0], fl[1], fl[2], fl[3]), b = make_int4(fl[4], fl[5], fl[6], fl[7]);
        ProfScope ps(this, PC_POST, (pcopy && kp.periodic) ? 2 : 1);
        if constexpr (sizeof(T) == 4) {
            if (post_quad) {
                const long nq = NZ / 4;
                auto go = [&](long ncols, int mode) {
                    if (post_kes)
                        k_post_quad<T, true><<<cdiv(ncols * nq, PQ_THREADS), PQ_THREADS, 0, stream>>>(
                            kp, F, a, b, (T)step, mode, d_err);
                    else
                        k_post_quad<T><<<cdiv(ncols * nq, PQ_THREADS), PQ_THREADS, 0, stream>>>(kp, F, a, b, (T)step,
                                                                                            mode, d_err);
                    launches++;
                };
                if (pcopy && kp.periodic) {
                    go(6L * NY, COLS_TARGETS);
                    go((long)(NX - 6) * NY, COLS_NONTARGETS);
                } else {
                    go((long)NX * NY, COLS_ALL);
                }
                return;
            }
        }
        if (pcopy && kp.periodic) {
            k_post<T><<<cdiv(6L * NY, POST_COLS), POST_THREADS, 0, stream>>>(kp, F, 7, a, b, (T)step, COLS_TARGETS);
            k_post<T><<<cdiv((long)(NX - 6) * NY, POST_COLS), POST_THREADS, 0, stream>>>(kp, F, 7, a, b, (T)step,
                                                                                      COLS_NONTARGETS);
            launches += 2;
        } else {
            k_post<T><<<cdiv((long)NX * NY, POST_COLS), POST_THREADS, 0, stream>>>(kp, F, 7, a, b, (T)step, COLS_ALL);
            launches++;
        }
    }

    void kessler()
    {
        if (!kp.moist) return;
        KFields<T> F = fields();
        const long tot = (long)(NX - 2) * (NY - 2) * (NZ - 2);
        {
        ProfScope ps(this, PC_KESSLER, 1);
        k_kessler<T><<<cdiv(tot, 128), 128, 0, stream>>>(kp, F, kp.rf != 2, d_err);
        launches++;
        }
        if (kp.rf == 2) {
            ProfScope ps(this, PC_PPM, 5);
            const long tv = (long)(NX - 2) * (NY - 2) * NZ;
            k_fall_speed<T><<<cdiv(tv, 256), 256, 0, stream>>>(kp, F);
            const long ncol = (long)(NX - 2) * (NY - 2);
            k_ppm_prepare<T><<<cdiv(ncol, 64), 64, 0, stream>>>(kp, F, ppm_has, ppm_topq, ppm_topm);
            k_ppm_carry<T><<<1, 32, 0, stream>>>(ncol, ppm_has, ppm_topq, ppm_topm, ppm_cin, ppm_carry);
            k_ppm_remap<T><<<cdiv(ncol, 64), 64, 0, stream>>>(kp, F, ppm_has, ppm_cin);
            k_fill<T><<<cdiv(N, 256), 256, 0, stream>>>(vt, N, T(0));
            launches += 5;
        }
    }

    // Rutledge fall speeds of the Eulerian advection (advect_microphysics_cell's
    // rain, advect_ice_cell's snow and ice) over the advected columns
    void ice_fall_euler(int what)
    {
        KFields<T> F = fields();
        const long tot = (long)(NX - 6) * (NY - 6) * (NZ - 2);
        k_ice_fall<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, F, 3, NX - 3, 3, NY - 3, what, 0);
        launches++;
    }

    void advect_ice(double step)  // advect_ice_cell (advection.cpp:508-567)
    {
        KFields<T> F = fields();
        ProfScope ps(this, PC_ADVECT, 1);
        const long tot = (long)(NX - 6) * (NY - 6) * (NZ - 2);
        k_advect_ice<T><<<cdiv(tot, 128), 128, 0, stream>>>(kp, F, (T)step);
        launches++;
    }

    // semi-Lagrangian PPM fallout of one hydrometeor (hydrometeor_fallout,
    // microphysics.cpp:210-292) with its fall speed into its accumulator; the
    // edge value the reference carries between columns runs on through the
    // calls in their order
    void ppm_fallout(KFields<T> F, T *var, T *fall, double *acc)
    {
        F.P[FQR] = var;
        F.vt = fall;
        F.accrain = acc;
        const long ncol = (long)(NX - 2) * (NY - 2);
        k_ppm_prepare<T><<<cdiv(ncol, 64), 64, 0, stream>>>(kp, F, ppm_has, ppm_topq, ppm_topm);
        k_ppm_carry<T><<<1, 32, 0, stream>>>(ncol, ppm_has, ppm_topq, ppm_topm, ppm_cin, ppm_carry);
        k_ppm_remap<T><<<cdiv(ncol, 64), 64, 0, stream>>>(kp, F, ppm_has, ppm_cin);
        launches += 3;
    }

    // run_rutledge_microphysics (rutledge.cpp:150-501).  exact: zero_moisture
    // of the points outside the interior and the precipitation as passes of
    // their own, for a forecast state that no stage has clipped (the single
    // operator); in the step every such point is already clipped and the
    // level-1 threads add the precipitation
    void rutledge(bool exact)
    {
        KFields<T> F = fields();
        const long tot = (long)(NX - 2) * (NY - 2) * (NZ - 2);
        const bool rf1 = kp.rf != 2;
        {
            ProfScope ps(this, PC_KESSLER, 2);
            k_rutledge<T><<<cdiv(tot, 128), 128, 0, stream>>>(kp, F, rf1 && !exact, d_err);
            k_ice_n0s<T><<<1, 32, 0, stream>>>(F);
            launches += 2;
        }
        if (exact) {
            int fz[9] = {};
            fz[FQV] = fz[FQC] = fz[FQR] = fz[FQS] = fz[FQI] = PF_ZERO;
            post(fz, 9, 1.0, false);
            if (rf1) {
                const long ncol = (long)(NX - 2) * (NY - 2);
                k_ice_precip<T><<<cdiv(ncol, 128), 128, 0, stream>>>(kp, F);
                launches++;
            }
        }
        if (!rf1) {
            ProfScope ps(this, PC_PPM, 13);
            k_ice_fall<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, F, 1, NX - 1, 1, NY - 1,
                                                              IF_RAIN | IF_SNOW | IF_ICE, 1);
            ppm_fallout(F, F.P[FQR], vt, accrain);
            ppm_fallout(F, F.P[FQI], its, accsnow);
            ppm_fallout(F, F.P[FQS], sts, accsnow);
            k_fill<T><<<cdiv(N, 256), 256, 0, stream>>>(vt, N, T(0));
            k_fill<T><<<cdiv(N, 256), 256, 0, stream>>>(sts, N, T(0));
            k_fill<T><<<cdiv(N, 256), 256, 0, stream>>>(its, N, T(0));
            launches += 4;
        }
    }

    void microphysics(bool exact)  // run_microphysics (microphysics.cpp:97-131)
    {
        if (kp.ice) rutledge(exact);
        else kessler();
    }

    void swap_micro()  // microphysics_advance_inner (microphysics.cpp:642-653)
    {
        for (int f = 4; f < nprog; f++) std::swap(ci[f], pi_[f]);
    }

    void swap_inner(bool micro)
    {
        for (int f = 0; f < 4; f++)
            if (f != FW || !hyd.div) std::swap(ci[f], pi_[f]);  // solver.cpp:240-248
        if (micro)
            for (int f = 4; f < nprog; f++) std::swap(ci[f], pi_[f]);
    }

    void copy_m_from_p(int f0, int f1)
    {
        ProfScope ps(this, PC_COPY, 0);
        for (int f = f0; f < f1 && f < nprog; f++)
            if (f != FW || !hyd.div)
                cudaMemcpyAsync(buf[f][mi[f]], buf[f][pi_[f]], N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
    }

    int op(int o, double step) override
    {
        cudaSetDevice(device);
        refresh_base();
        const bool moist = kp.moist;
        int fl[9] = {};
        switch (o) {
        case GA_OP_SIGN_CELLS: break;
        case GA_OP_ADVECT_UVW: advect(step, hyd.div ? ADV_UV : ADV_UV | ADV_WB); break;  // advect_uv_velocity
        case GA_OP_SOLVE_PRESSURE:
            if (hyd.div) hyd_solve(step);
            else solve_pressure(step);
            break;
        case GA_OP_PROJECT:
            if (hyd.div) {
                hyd_project(step);
                break;
            }
            fl[FU] = fl[FV] = fl[FW] = PF_PROJECT;
            post(fl, 9, step, false);
            break;
        case GA_OP_INTEGRATE_NON_HYDRO:
            if (hyd.div) {  // integrate_hydro (solver.cpp:33-80)
                advect(step, ADV_UV);
                hyd_solve(step);
                hyd_project(step);
                break;
            }
            advect(step, ADV_UV | ADV_WB);
            turb_apply(TA_VEL, step);  // solver.cpp:103
            solve_pressure(step);
            fl[FU] = fl[FV] = fl[FW] = PF_PROJECT;
            post(fl, 9, step, false);
            break;
        case GA_OP_ADVECT_THETA: advect(step, ADV_TH); break;
        case GA_OP_ADVECT_MICRO:
            if (!moist) break;
            if (kp.ice && kp.rf == 1) ice_fall_euler(IF_RAIN);  // advection.cpp:456-457
            advect(step, cfg.linear_model ? (ADV_Q | ADV_QVONLY) : ADV_Q);  // advect_qv when linear
            break;
        case GA_OP_ADVECT_ICE:
            if (!kp.ice) return GA_ERR_ARG;
            if (kp.rf == 1) ice_fall_euler(IF_SNOW | IF_ICE);  // advection.cpp:513-514
            advect_ice(step);
            break;
        case GA_OP_ZERO_MOISTURE:
            if (moist) {
                fl[FQV] = fl[FQC] = fl[FQR] = fl[FQS] = fl[FQI] = PF_ZERO;
                post(fl, 9, step, false);
            }
            break;
        case GA_OP_BC:
            fl[FU] = fl[FV] = fl[FW] = fl[FTH] = PF_SPONGE | PF_VBC;
            if (kp.periodic) periodic_pi();
            post(fl, 9, step, true);
            break;
        case GA_OP_BC_MICRO:
            if (moist) {
                fl[FQV] = fl[FQC] = fl[FQR] = fl[FQS] = fl[FQI] = PF_SPONGE | PF_VBC;
                post(fl, 9, step, true);
            }
            break;
        case GA_OP_KESSLER: microphysics(true); break;
        case GA_OP_EXPLICIT_DIFFUSION: diffuse(step); break;
        case GA_OP_TURBULENCE:
            if (!turb.kmix) return GA_ERR_ARG;
            turbulence();
            break;
        case GA_OP_RAYLEIGH:
            fl[FU] = fl[FV] = fl[FW] = fl[FTH] = PF_RAYLEIGH;
            post(fl, 9, step, false);
            break;
        case GA_OP_ADVANCE_INNER: swap_inner(true); break;
        case GA_OP_ADVANCE_OUTER:
            copy_m_from_p(0, 9);
            swap_inner(true);
            break;
        default: return GA_ERR_ARG;
        }
        // a captured two-step graph pairs the rotation parity with the
        // diffusion buffers' parity; a single operator may break the pairing
        if (diff_tend) drop_graphs();
        int rc = launch_status();
        if (rc) return rc;
        rc = sync_status();
        if (rc) return rc;
        return kessler_status();
    }

    void periodic_pi()
    {
        const long tot = 6L * NY * NZ;
        k_periodic_copy<T><<<cdiv(tot, 256), 256, 0, stream>>>(kp, pi, (T *)nullptr, (T *)nullptr, (T *)nullptr);
        launches++;
    }

    int kessler_status()
    {
        if (!kp.moist) return GA_OK;
        int e = 0;
        cudaMemcpy(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (e) {
            set_error(kp.ice ? "ice microphysics: rain evaporation E>100 or snow melting |psmlt|>100 (the reference "
                               "exits here, rutledge.cpp:252-258, 370-376)"
                             : "Kessler evaporation E>100 (the reference exits here, kessler.cpp:83-88)");
            return GA_ERR_KESSLER;
        }
        return GA_OK;
    }

    // one RK3 step: s_integrate_rk3 (driver_serial.cpp:178-286), fused.
    // rec (optional), the trajectory of the adjoint: the stage-start
    // prognostic fields go to rec + (nprog*stage + field)*N and, when moist,
    // the inputs of Kessler (P of theta, qv, qc, qr, then pi) to
    // rec + (3*nprog + q)*N, with each stage's clipping record in
    // mrec + stage*N.
    void rk3_step(T *rec = nullptr, unsigned char *mrec = nullptr)
    {
        static const double steps[3] = {1. / 3., 0.5, 1.0};
        const bool moist = kp.moist;
        if (cfg.use_explicit_diffusion) diffuse(1.0);  // driver_serial.cpp:188, before the RK stages
        const bool turbulent = turb.kmix != nullptr;
        if (turbulent) turbulence();  // driver_serial.cpp:194
        for (int s = 0; s < 3; s++) {
            const double st = steps[s];
            // the stage-start fields to the tape: the stage reads them and
            // writes only the forecast slots, so the copies may run beside it
            // until the stage's end (the next stage writes these buffers)
            const bool rec_side = rec && overlap_rec && !prof && !hyd.div && !kp.ice;
            if (rec) {
                if (rec_side) fork();
                OnSideIf os(this, rec_side);
                for (int f = 0; f < nprog; f++)
                    cudaMemcpyAsync(rec + (size_t)(nprog * s + f) * N, buf[f][ci[f]], N * sizeof(T),
                                    cudaMemcpyDeviceToDevice, stream);
            }
            qmask = mrec ? mrec + (size_t)s * N : nullptr;
            if (hyd.div) {  // the hydrostatic set: driver_serial.cpp:208-239 with integrate_hydro
                // theta and moisture beside the lid-pressure solve; joined
                // before w_velocity_LH rewrites the current w they read
                // with the ice scheme the moisture follows the solve (the
                // Rutledge fall speeds read the solved Exner perturbation)
                const bool ice = kp.ice;
                const int scal = ADV_TH | (moist && !ice ? (ADV_Q | ADV_ZERO) : 0);
                const bool side = overlap && !prof;
                advect(st, ADV_UV | (side ? 0 : scal));
                if (side) {  // with their column pass
                    fork();
                    OnSide os(this);
                    advect(st, scal);
                    int fs[9] = {};
                    fs[FTH] = PF_SPONGE | PF_VBC;
                    if (moist && !ice) fs[FQV] = fs[FQC] = fs[FQR] = PF_ZERO | PF_SPONGE | PF_VBC;
                    post(fs, 9, st, true);
                }
                hyd_solve(st);
                hyd_project(st);
                if (ice) {
                    const bool quad = adv_quad && quad_ok(adv_qi, adv_qj) && !(adv_tma && tma_ok(adv_tmc));
                    if (kp.rf == 1) ice_fall_euler(IF_RAIN | IF_SNOW | IF_ICE);
                    if (quad) {
                        advect(st, ADV_Q | ADV_ICE | ADV_ZERO);
                    } else {
                        advect(st, ADV_Q | ADV_ZERO);
                        advect_ice(st);
                    }
                }
                if (side) join();
                hyd_w();
                int fh[9] = {};
                fh[FU] = fh[FV] = fh[FW] = PF_SPONGE | PF_VBC;  // w: the current slot
                if (!side) fh[FTH] = PF_SPONGE | PF_VBC;
                if (!side || ice) fh[FQV] = fh[FQC] = fh[FQR] = PF_ZERO | PF_SPONGE | PF_VBC;
                if (ice) fh[FQS] = fh[FQI] = PF_ZERO | PF_SPONGE | PF_VBC;
                post(fh, 9, st, true);
                qmask = nullptr;
                if (s < 2) swap_inner(true);
                continue;
            }
            if (kp.ice) {  // driver_serial.cpp:198-247 with advect_ice_cell
                // the Rutledge fall speeds read the pressure of this stage's
                // solve, so the moisture advection follows it; the four-level
                // kernel (FP32) advects snow and ice in the same launch
                const bool quad = adv_quad && quad_ok(adv_qi, adv_qj) && !(adv_tma && tma_ok(adv_tmc));
                const bool fuse = !kp.periodic && quad;
                const bool side = overlap && !prof;  // theta beside the solve
                advect(st, ADV_UV | ADV_WB | (side ? 0 : ADV_TH) | (fuse ? ADV_MIRROR : 0));
                if (turbulent) turb_apply(side ? TA_VEL : TA_VEL | TA_TH, st);
                if (side)
                    mid_solve = [this, st, turbulent] {
                        fork();
                        OnSide os(this);
                        advect(st, ADV_TH);
                        if (turbulent) turb_apply(TA_TH, st);
                        int fs[9] = {};
                        fs[FTH] = PF_SPONGE | PF_VBC;
                        post(fs, 9, st, true);
                    };
                if (fuse) poisson(st);
                else solve_pressure(st);
                if (kp.rf == 1) ice_fall_euler(IF_RAIN | IF_SNOW | IF_ICE);
                const int zero = turbulent ? 0 : ADV_ZERO;
                if (quad) {
                    advect(st, ADV_Q | ADV_ICE | zero);
                } else {
                    advect(st, ADV_Q | zero);
                    advect_ice(st);
                }
                if (turbulent) turb_apply(TA_Q, st);
                int fl[9] = {};
                fl[FU] = fl[FV] = fl[FW] = PF_PROJECT | PF_SPONGE | PF_VBC;
                if (!side) fl[FTH] = PF_SPONGE | PF_VBC;
                fl[FQV] = fl[FQC] = fl[FQR] = fl[FQS] = fl[FQI] = PF_ZERO | PF_SPONGE | PF_VBC;
                post(fl, 9, st, true);
                if (side) join();
                if (s < 2) swap_inner(true);
                continue;
            }
            // the four-level advection launch also makes the mirror copies of
            // the pressure solve (they touch no point the advection writes)
            const bool fuse_mirror = !kp.periodic && adv_quad && quad_ok(adv_qi, adv_qj);
            // with turbulence the stage's tendencies come after the advection
            // and before zero_moisture (driver_serial.cpp:205-230), which the
            // post-processing pass then applies; they touch no point that the
            // mirror copies read
            const int zero = turbulent ? 0 : ADV_ZERO;
            const int scal = ADV_TH | (moist ? (ADV_Q | zero) : 0);
            if (overlap && !prof) {
                // theta and moisture beside the pressure solve: they read the
                // current and start-of-step fields, which the solve leaves alone
                advect(st, ADV_UV | ADV_WB | (fuse_mirror ? ADV_MIRROR : 0));
                if (turbulent) turb_apply(TA_VEL, st);
                unsigned char *qm = qmask;
                // their column pass (sponge, top/bottom, clipping) follows on
                // the same stream; the main stream's pass projects u, v, w
                mid_solve = [this, st, scal, turbulent, qm, moist] {
                    fork();
                    OnSide os(this);
                    qmask = qm;
                    advect(st, scal);
                    qmask = nullptr;
                    if (turbulent) turb_apply(TA_TH | TA_Q, st);
                    int fs[9] = {};
                    fs[FTH] = PF_SPONGE | PF_VBC;
                    if (moist) fs[FQV] = fs[FQC] = fs[FQR] = PF_ZERO | PF_SPONGE | PF_VBC;
                    post(fs, 9, st, true);
                };
                qmask = nullptr;
                if (fuse_mirror) poisson(st);
                else solve_pressure(st);
                int fl[9] = {};
                fl[FU] = fl[FV] = fl[FW] = PF_PROJECT | PF_SPONGE | PF_VBC;
                post(fl, 9, st, true);
                join();
            } else {
                advect(st, ADV_UV | ADV_WB | scal | (fuse_mirror ? ADV_MIRROR : 0));
                if (turbulent) turb_apply(TA_VEL | TA_TH | TA_Q, st);
                qmask = nullptr;
                if (fuse_mirror) poisson(st);
                else solve_pressure(st);
                int fl[9] = {};
                fl[FU] = fl[FV] = fl[FW] = PF_PROJECT | PF_SPONGE | PF_VBC;
                fl[FTH] = PF_SPONGE | PF_VBC;
                fl[FQV] = fl[FQC] = fl[FQR] = PF_ZERO | PF_SPONGE | PF_VBC;
                post(fl, 9, st, true);
                if (rec_side) join();
            }
            if (s < 2) swap_inner(true);
        }
        if (moist && rec) {
            const int kin[4] = {FTH, FQV, FQC, FQR};
            for (int q = 0; q < 4; q++)
                cudaMemcpyAsync(rec + (size_t)(3 * nprog + q) * N, buf[kin[q]][pi_[kin[q]]], N * sizeof(T),
                                cudaMemcpyDeviceToDevice, stream);
            cudaMemcpyAsync(rec + (size_t)(3 * nprog + 4) * N, pi, N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        }
        // FP32, Eulerian rain, non-periodic: Kessler runs inside the last
        // column pass (a periodic domain's copied columns take their own
        // rain totals, so it keeps the separate kernel)
        const bool fuse_kes = moist && !kp.ice && kes_fused && post_quad && kp.rf == 1 && !kp.periodic;
        if (moist && !fuse_kes) microphysics(false);
        int fl[9] = {};
        fl[FU] = fl[FV] = fl[FW] = fl[FTH] = PF_SPONGE | PF_VBC | PF_RAYLEIGH | PF_WRITE_M;
        fl[FQV] = fl[FQC] = fl[FQR] = fl[FQS] = fl[FQI] = PF_SPONGE | PF_VBC | PF_WRITE_M;
        post_kes = fuse_kes;
        post(fl, 9, 1.0, true);
        post_kes = false;
        swap_inner(true);
        mtime += cfg.dt;
        bigcounter++;
    }

    // one step of the linearised model: linear_integrate_rk3
    // (driver_serial.cpp:83-171).  Within a stage the vapour is advected after
    // the winds' rotation, so stages 1 and 2 advect it with the new winds;
    // explicit diffusion acts on the start-of-step fields in every stage; no
    // microphysics; the perturbation is rescaled every 12 hours.
    void linear_step()
    {
        static const double steps[3] = {1. / 3., 0.5, 1.0};
        const bool moist = kp.moist;
        kp.stale_signs = 1;
        for (int s = 0; s < 3; s++) {
            const double st = steps[s];
            const bool side = overlap && !prof;  // theta beside the pressure solve
            advect(st, ADV_UV | ADV_WB | (side ? 0 : ADV_TH));
            if (side)
                mid_solve = [this, st] {
                    fork();
                    OnSide os(this);
                    advect(st, ADV_TH);
                };
            solve_pressure(st);
            if (side) join();
            int fl[9] = {};
            fl[FU] = fl[FV] = fl[FW] = PF_PROJECT | PF_SPONGE | PF_VBC;
            fl[FTH] = PF_SPONGE | PF_VBC;
            post(fl, 9, st, true);
            if (cfg.use_explicit_diffusion) diffuse(st);  // the start-of-step slot, driver_serial.cpp:102
            if (s < 2) swap_inner(false);
            if (moist) {
                advect(st, ADV_Q | ADV_QVONLY);
                int fq[9] = {};
                fq[FQV] = fq[FQC] = fq[FQR] = PF_SPONGE | PF_VBC;
                post(fq, 9, st, true);
                if (s < 2) swap_micro();
            }
        }
        int fl[9] = {};
        fl[FU] = fl[FV] = fl[FW] = fl[FTH] = PF_SPONGE | PF_VBC | PF_RAYLEIGH | PF_WRITE_M;
        fl[FQV] = fl[FQC] = fl[FQR] = PF_SPONGE | PF_VBC | PF_WRITE_M;
        post(fl, 9, 1.0, true);
        swap_inner(true);
        kp.stale_signs = 0;
        const long period = 12 * 60 * 60 / (int)cfg.dt;
        if (period > 0 && bigcounter % period == 0 && bigcounter != 0) {
            cudaMemsetAsync(lin_vmax, 0, sizeof(double), stream);
            k_lin_vmax<T><<<152 * 4, 256, 0, stream>>>(buf[FV][pi_[FV]], kp.rhou, NZ, N, lin_vmax);
            k_lin_rescale<T><<<152 * 4, 256, 0, stream>>>(buf[FU][ci[FU]], buf[FV][ci[FV]], buf[FW][ci[FW]],
                                                          buf[FTH][ci[FTH]], buf[FU][mi[FU]], buf[FV][mi[FV]],
                                                          buf[FW][mi[FW]], buf[FTH][mi[FTH]], N, lin_vmax);
            launches += 2;
        }
        mtime += cfg.dt;
        bigcounter++;
    }

    // ---------------------------------------------------------------- tuning
    // Times the candidates of each tunable kernel group on this context's own
    // data and keeps the fastest: the advection tile, the level tile of the y
    // transforms, the factor order of both FFTs and (unfused x path) the level
    // tile of the x transforms.  The groups write P, the fall speed, the
    // spectral buffer and pi; P, the fall speed and pi are restored afterwards.
    int tune() override
    {
        cudaSetDevice(device);
        refresh_base();
        const int nsnap = nprog + 2;
        T *snap = nullptr;
        if (cudaMalloc(&snap, (size_t)nsnap * N * sizeof(T)) != cudaSuccess) return GA_ERR_NOMEM;
        for (int f = 0; f < nprog; f++)
            cudaMemcpyAsync(snap + (size_t)f * N, buf[f][pi_[f]], N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        cudaMemcpyAsync(snap + (size_t)nprog * N, pi, N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        cudaMemcpyAsync(snap + (size_t)(nprog + 1) * N, vt, N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        cudaEvent_t ea, eb;
        cudaEventCreate(&ea);
        cudaEventCreate(&eb);
        const long long l0 = launches;
        // L2 is written over before each candidate's timed launches: a grid
        // whose state fits in L2 is otherwise timed hot, which favours tiles
        // with more halo re-reads than a step that starts from DRAM can afford
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device);
        const size_t flush_bytes = 2 * (size_t)std::max(l2, 0);
        void *flush = nullptr;
        if (flush_bytes && cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
            flush = nullptr;
            cudaGetLastError();
        }
        auto timeit = [&](auto fn) {
            fn();  // warm-up
            if (flush) cudaMemsetAsync(flush, 0, flush_bytes, stream);
            cudaEventRecord(ea, stream);
            for (int r = 0; r < 3; r++) fn();
            cudaEventRecord(eb, stream);
            cudaEventSynchronize(eb);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ea, eb);
            return cudaGetLastError() == cudaSuccess ? ms / 3.f : 1e30f;
        };
        const int what = ADV_UV | ADV_WB | ADV_TH | (kp.moist ? (ADV_Q | ADV_ZERO) : 0);
        std::string info;
        char line[160];
        // advection tile
        {
            float best = 1e30f;
            int bi = adv_ti, bj = adv_tj, bq = 0, qi = adv_qi, qj = adv_qj, qb = adv_qb, br = adv_rows;
            int bt = 0, tc = adv_tmc;
            adv_tma = 0;
            if ((adv_force != 2 && adv_force != 3) || !quad_ok(adv_qi, adv_qj)) {
                adv_quad = 0;
                for (auto &tl : kAdvTiles) {
                    const size_t sm = advect_tile_smem(tl[0], tl[1], NZ, sizeof(T));
                    if (sm > 200 * 1024) continue;
                    adv_ti = tl[0]; adv_tj = tl[1]; smem_adv = sm;
                    const float t = timeit([&] { advect(1. / 3., what); });
                    if (t < best) { best = t; bi = tl[0]; bj = tl[1]; }
                }
            }
            if (adv_force == 0 || adv_force == 2) {
                adv_quad = 1;
                for (auto &tl : kQuadTiles) {
                    if (!quad_ok(tl[0], tl[1])) continue;
                    for (int mb = 3; mb <= 4; mb++)
                        for (int rows = 0; rows <= 1; rows++) {
                            adv_qi = tl[0]; adv_qj = tl[1]; adv_qb = mb; adv_rows = rows;
                            const float t = timeit([&] { advect(1. / 3., what); });
                            if (t < best) { best = t; bq = 1; qi = tl[0]; qj = tl[1]; qb = mb; br = rows; bt = 0; }
                        }
                }
            }
            if (adv_force == 0 || adv_force == 3) {
                adv_quad = 1;
                adv_tma = 1;
                for (int c = 0; c < 4; c++) {
                    if (!tma_ok(c)) continue;
                    adv_tmc = c;
                    const float t = timeit([&] { advect(1. / 3., what); });
                    if (t < best) { best = t; bq = 1; bt = 1; tc = c; }
                }
                adv_tma = 0;
            }
            adv_ti = bi; adv_tj = bj; adv_quad = bq; adv_qi = qi; adv_qj = qj; adv_qb = qb; adv_rows = br;
            adv_tma = bt; adv_tmc = tc;
            smem_adv = advect_tile_smem(bi, bj, NZ, sizeof(T));
            if (bt) {
                const TmaCand &t = kTmaCands[tc];
                std::snprintf(line, sizeof line,
                              "advect tile %dx%d, %d-level slabs staged by TMA, %d blocks/SM (%.4f ms); ", t.ti, t.tj,
                              t.kz, t.mb, best);
            } else if (bq)
                std::snprintf(line, sizeof line, "advect tile %dx%d, four levels per thread, %d blocks/SM%s (%.4f ms); ",
                              qi, qj, qb, br ? ", face rows" : "", best);
            else std::snprintf(line, sizeof line, "advect tile %dx%d (%.4f ms); ", bi, bj, best);
            info += line;
        }
        // y transforms: level tile, then factor order
        auto set_kty = [&](int kt) {
            KTy = kt;
            lgKTy = 0;
            while ((1 << lgKTy) < kt) lgKTy++;
            smem_y = 2 * (size_t)kp.nj * KTy * sizeof(T2);
        };
        {
            float best = 1e30f;
            int bk = KTy;
            for (int kt = 1; kt <= 64 && kt <= 2 * (NZ - 2); kt <<= 1) {
                if (2 * (size_t)kp.nj * kt * sizeof(T2) > 200 * 1024) break;
                set_kty(kt);
                const float t = timeit([&] { solve_pressure(1. / 3.); });
                if (t < best) { best = t; bk = kt; }
            }
            set_kty(bk);
            float bestp = best;
            int bo = 0;
            for (int order = 1; order < 4; order++) {
                FftPlan cand = make_fft_plan(kp.nj, order);
                if (!cand.nfac) continue;
                const FftPlan keep = plan_j;
                plan_j = cand;
                const float t = timeit([&] { solve_pressure(1. / 3.); });
                if (t < bestp) { bestp = t; bo = order; }
                plan_j = keep;
            }
            plan_order_j = bo;
            plan_j = make_fft_plan(kp.nj, bo);
            std::snprintf(line, sizeof line, "y level tile %d, y FFT order %d; ", bk, bo);
            info += line;
            // x transforms: factor order (and the level tile of the unfused path)
            float bx = bestp;
            int bxo = 0;
            for (int order = 1; order < 4; order++) {
                FftPlan cand = make_fft_plan(kp.ni, order);
                if (!cand.nfac) continue;
                const FftPlan keep = plan_i;
                plan_i = cand;
                const float t = timeit([&] { solve_pressure(1. / 3.); });
                if (t < bx) { bx = t; bxo = order; }
                plan_i = keep;
            }
            plan_order_i = bxo;
            plan_i = make_fft_plan(kp.ni, bxo);
            // the fused x kernel's block size, and (FP32) its paired-CTA form
            if (psx > 0) {
                const int keep = sx_threads;
                int bt = keep;
                bool bp = false;
                sx_pair = false;
                for (int nt : {512, 1024}) {
                    sx_threads = nt;
                    const float t = timeit([&] { solve_pressure(1. / 3.); });
                    if (t < bx) { bx = t; bt = nt; }
                }
                float t;
                if (pair_ok()) {
                    sx_pair = true;
                    for (int nt : {256, 512}) {
                        sx_threads = nt;
                        t = timeit([&] { solve_pressure(1. / 3.); });
                        if (t < bx) { bx = t; bt = nt; bp = true; }
                    }
                }
                sx_threads = bt;
                sx_pair = bp;
            }
            // the unfused path (x FFT, Thomas, inverse x FFT) and its level
            // tile, against the fused kernel where that fits
            {
                const int keep_psx = psx, keep_kt = KTx;
                psx = 0;
                int bkx = -1;
                for (int kt = 1; kt <= 64 && kt <= 2 * (NZ - 2); kt <<= 1) {
                    if (2 * (size_t)kp.ni * kt * sizeof(T2) > 200 * 1024) break;
                    KTx = kt;
                    smem_x = 2 * (size_t)kp.ni * KTx * sizeof(T2);
                    const float t = timeit([&] { solve_pressure(1. / 3.); });
                    if (t < bx || (keep_psx == 0 && bkx < 0)) { bx = std::min(bx, t); bkx = kt; }
                }
                if (bkx > 0) {
                    KTx = bkx;
                } else {
                    psx = keep_psx;
                    KTx = keep_kt;
                }
                lgKTx = 0;
                while ((1 << lgKTx) < KTx) lgKTx++;
                smem_x = 2 * (size_t)kp.ni * KTx * sizeof(T2);
                if (psx == 0) std::snprintf(line, sizeof line, "x level tile %d, ", KTx);
                else std::snprintf(line, sizeof line, "x fused%s, %d threads, ", sx_pair ? " (CTA pairs)" : "",
                                   sx_threads);
                info += line;
            }
            std::snprintf(line, sizeof line, "x FFT order %d (pressure solve %.4f ms)", bxo, bx);
            info += line;
        }
        for (int f = 0; f < nprog; f++)
            cudaMemcpyAsync(buf[f][pi_[f]], snap + (size_t)f * N, N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        cudaMemcpyAsync(pi, snap + (size_t)nprog * N, N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        cudaMemcpyAsync(vt, snap + (size_t)(nprog + 1) * N, N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        const int rc = sync_status();
        cudaEventDestroy(ea);
        cudaEventDestroy(eb);
        if (flush) cudaFree(flush);
        cudaFree(snap);
        launches = l0;
        drop_graphs();
        tuning = info;
        return rc;
    }

    // CUDA graph of two steps: the rotation of the three buffers has period
    // two steps, so one graph per starting parity replays any even count.
    int capture_pair(int parity)
    {
        const long long bc = bigcounter, l0 = launches;
        const double mt = mtime;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GA_ERR_CUDA;
        rk3_step();
        rk3_step();
        if (cudaStreamEndCapture(stream, &g) != cudaSuccess) return GA_ERR_CUDA;
        cudaError_t e = cudaGraphInstantiate(&graph[parity], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return GA_ERR_CUDA;
        graph_launches[parity] = launches - l0;
        launches = l0;
        bigcounter = bc;
        mtime = mt;
        return GA_OK;
    }

    int step(int nsteps) override
    {
        cudaSetDevice(device);
        refresh_base();
        int n = 0;
        if (use_graphs && !prof) {
            while (nsteps - n >= 2) {
                const int parity = ci[0] == 0 ? 0 : 1;
                if (!graph[parity]) {
                    int rc = capture_pair(parity);
                    if (rc) {
                        cudaGetLastError();
                        use_graphs = false;
                        break;
                    }
                }
                if (cudaGraphLaunch(graph[parity], stream) != cudaSuccess) return launch_status();
                launches += graph_launches[parity];
                bigcounter += 2;
                mtime += 2 * cfg.dt;
                n += 2;
            }
        }
        for (; n < nsteps; n++) {
            if (cfg.linear_model) linear_step();
            else rk3_step();
            int rc = launch_status();
            if (rc) return rc;
        }
        return launch_status();
    }

    int budget(int slot, double *out) override
    {
        if (slot < 0 || slot > 2) return GA_ERR_ARG;
        cudaSetDevice(device);
        auto sl = [&](int f) -> const T * {
            if (f >= nprog) return nullptr;
            return buf[f][slot == GA_SLOT_CUR ? ci[f] : slot == GA_SLOT_P ? pi_[f] : mi[f]];
        };
        k_budget<T><<<BUDGET_BLOCKS, 256, 0, stream>>>(NX, NY, NZ, sl(FU), sl(FV), sl(FW), sl(FTH), sl(FQV), sl(FQC),
                                                       sl(FQR), sl(FQI), sl(FQS), kp.moist ? accrain : nullptr,
                                                       accsnow, budget_w, cfg.dx * cfg.dy, budget_part);
        k_budget_sum<<<1, 32, 0, stream>>>(budget_part, BUDGET_BLOCKS, budget_part + (size_t)BUDGET_BLOCKS * GA_NB);
        launches += 2;
        int rc = launch_status();
        if (rc) return rc;
        double h[GA_NB];
        cudaMemcpyAsync(h, budget_part + (size_t)BUDGET_BLOCKS * GA_NB, sizeof h, cudaMemcpyDeviceToHost, stream);
        rc = sync_status();
        if (rc) return rc;
        h[4] = h[1] + h[2] + h[3] + h[8] + h[9];  // total water (ice and snow 0 without the ice scheme)
        for (int b = 0; b < GA_NB; b++) out[b] = h[b];
        return GA_OK;
    }

    int check_finite() override
    {
        cudaSetDevice(device);
        cudaMemsetAsync(d_err + 0, 0, 0, stream);
        int *flag = nullptr;
        if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) return GA_ERR_NOMEM;
        cudaMemsetAsync(flag, 0, sizeof(int), stream);
        for (int f = 0; f < nprog; f++)
            for (int s = 0; s < 3; s++) {
                k_check_finite<T><<<1024, 256, 0, stream>>>(buf[f][s], N, flag);
                launches++;
            }
        int h = 0;
        cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, stream);
        int rc = sync_status();
        cudaFree(flag);
        if (rc) return rc;
        return h ? GA_ERR_NONFINITE : GA_OK;
    }
};

template <typename T>
EngineBase *make_engine(const ga_config *cfg, const ga_columns *cols, int *rc)
{
    Engine<T> *e = new Engine<T>(cfg, cols);
    if (e->status != GA_OK) {
        *rc = e->status;
        delete e;
        return nullptr;
    }
    *rc = GA_OK;
    return e;
}

}  // namespace ga

// tangent-linear model and adjoint: members of Engine<T> declared above
#include "ga_lin.cuh"
