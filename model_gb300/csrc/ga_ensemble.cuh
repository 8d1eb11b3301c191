// ga_ensemble.cuh - ensembles of independent domains of uneven sizes, advanced
// together: one launch per kernel phase covers every member.
//
// The reference runs ensemble members as separate serial models, one MPI task
// each (run_ensemble, ensemble.cpp:45-144).  Here the members' parameters and
// field pointers live in a packed device table; each batched kernel walks a
// flattened list of virtual blocks (grid-stride, so the grid is sized to the
// machine, not to the work), maps a virtual block to (member, local block) by
// binary search over per-member block prefixes, and calls the same device
// body as the single-domain kernel.  Every member therefore computes exactly
// what it computes alone.  The buffer rotation of all members moves in lock
// step and takes only two states, so two field tables cover it, and the two-
// step cycle is captured in a CUDA graph.
#pragma once
#include <algorithm>
#include <vector>

#include "ga_engine.cuh"

namespace ga {

// per-member data of the pressure solve that is not in KParams
template <typename T>
struct MemberAux {
    typename V2<T>::t *spec, *tw_i, *tw_j;
    FftPlan plan_i, plan_j;
    int KTy, psx;
};

enum { EK_ADV = 0, EK_MIRROR, EK_DIVY, EK_SX, EK_IFFTY, EK_POST, EK_KES, EK_FX, EK_TH, EK_COUNT };

__device__ __forceinline__ int find_member(const long *pre, int nmem, long vb)
{
    int lo = 0, hi = nmem;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(pre + mid) <= vb) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <typename T, int TI, int TJ>
__global__ void __launch_bounds__(256) kb_advect(const KParams<T> *P, const KFields<T> *F, const long *pre, int nmem,
                                                 double step, int what)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        const KParams<T> &p = P[m];
        const long lb = vb - pre[m];
        const int gx = (p.nx - 6 + TI - 1) / TI;
        const double sdtg = step * p.dt_d * 9.8 * 0.5;  // step*dt*grav*0.5, advection.cpp:330
        advect_tile_body<T, TI, TJ>(p, F[m], (int)(lb % gx), (int)(lb / gx), (T)step, (T)sdtg, what);
        __syncthreads();
    }
}

// FP32 members with whole level quads: the four-level advection and post
template <typename T, int TI, int TJ, int MB>
__global__ void __launch_bounds__(AQ_THREADS, MB) kb_advect_quad(const KParams<T> *__restrict__ P,
                                                               const KFields<T> *__restrict__ F,
                                                               const long *__restrict__ pre, int nmem, double step,
                                                               int what)
{
    static_assert(sizeof(T) == 4, "four-level kernels are FP32");
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        const KParams<T> &p = P[m];
        const long lb = vb - pre[m];
        const int gx = (p.nx - 6 + TI - 1) / TI;
        const double sdtg = step * p.dt_d * 9.8 * 0.5;  // step*dt*grav*0.5, advection.cpp:330
        // the row form spills in this kernel at either register budget;
        // masking ADV_ROWS lets the compiler drop it
        advect_quad_body<TI, TJ>(p, F[m], (int)(lb % gx), (int)(lb / gx), (T)step, (T)sdtg, what & ~ADV_ROWS);
        __syncthreads();
    }
}
template <typename T>
__global__ void __launch_bounds__(PQ_THREADS) kb_post_quad(const KParams<T> *P, const KFields<T> *F, const long *pre,
                                                           int nmem, int4 fl0, int4 fl1, double step)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        post_quad_body(P[m], F[m], fl0, fl1, (T)step, COLS_ALL, (vb - pre[m]) * PQ_THREADS + threadIdx.x);
    }
}

template <typename T>
__global__ void kb_mirror(const KParams<T> *P, const KFields<T> *F, const long *pre, int nmem)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        const long t = (vb - pre[m]) * blockDim.x + threadIdx.x;
        mirror_edges_body(P[m], F[m].P[FU], F[m].P[FV], F[m].P[FW], t);
    }
}

template <typename T>
__global__ void kb_div_fft_y(const KParams<T> *P, const KFields<T> *F, const MemberAux<T> *A, const long *pre,
                             int nmem, double step)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        const KParams<T> &p = P[m];
        const MemberAux<T> &a = A[m];
        const long lb = vb - pre[m];
        const long nkt = (p.nz - 2 + a.KTy - 1) / a.KTy;  // level tiles of a plane run next to each other
        div_fft_y_body(p, F[m], a.spec, a.plan_j, a.tw_j, (T)(step * p.dt_d), a.KTy, (int)(lb / nkt),
                       (int)(lb % nkt));
        __syncthreads();
    }
}

template <typename T>
__global__ void kb_spectral_x(const KParams<T> *P, const MemberAux<T> *A, const long *pre, int nmem)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        const MemberAux<T> &a = A[m];
        spectral_x_body(P[m], a.spec, a.plan_i, a.tw_i, a.psx, (int)(vb - pre[m]));
        __syncthreads();
    }
}

// the unfused x solve: x FFT per (y-wavenumber, level tile KT shared by every
// member), then Thomas per TC columns, then the inverse x FFT
template <typename T>
__global__ void kb_fft_x(const KParams<T> *P, const MemberAux<T> *A, const long *pre, int nmem, int inv, int KT)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        const KParams<T> &p = P[m];
        const MemberAux<T> &a = A[m];
        const long lb = vb - pre[m];
        const long nkt = (p.nz - 2 + KT - 1) / KT;  // level tiles of a wavenumber run next to each other
        fft_x_body(p, a.spec, a.plan_i, a.tw_i, inv, KT, (int)(lb / nkt), (int)(lb % nkt));
        __syncthreads();
    }
}
template <typename T>
__global__ void kb_thomas(const KParams<T> *P, const MemberAux<T> *A, const long *pre, int nmem, int TC)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        thomas_body(P[m], A[m].spec, TC, vb - pre[m]);
        __syncthreads();
    }
}

template <typename T>
__global__ void kb_ifft_y_pi(const KParams<T> *P, const KFields<T> *F, const MemberAux<T> *A, const long *pre,
                             int nmem)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        const KParams<T> &p = P[m];
        const MemberAux<T> &a = A[m];
        const long lb = vb - pre[m];
        const long nkt = (p.nz - 2 + a.KTy - 1) / a.KTy;
        ifft_y_pi_body(p, F[m], a.spec, a.plan_j, a.tw_j, a.KTy, (int)(lb / nkt), (int)(lb % nkt));
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(POST_THREADS) kb_post(const KParams<T> *P, const KFields<T> *F, const long *pre,
                                                        int nmem, int4 fl0, int4 fl1, double step)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        post_body(P[m], F[m], 7, fl0, fl1, (T)step, COLS_ALL, vb - pre[m]);
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(128) kb_kessler(const KParams<T> *P, const KFields<T> *F, const long *pre, int nmem,
                                                  int *err)
{
    const long total = pre[nmem];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int m = find_member(pre, nmem, vb);
        kessler_body(P[m], F[m], 1, err, (vb - pre[m]) * blockDim.x + threadIdx.x);
    }
}

template <typename T>
class Ensemble : public EnsembleBase {
    typedef typename V2<T>::t T2;

  public:
    std::vector<Engine<T> *> mem;
    int nmem = 0;
    cudaStream_t stream = nullptr;
    KParams<T> *d_p = nullptr;
    KFields<T> *d_f[2] = {nullptr, nullptr};
    MemberAux<T> *d_aux = nullptr;
    long *d_pre[EK_COUNT] = {};
    long total[EK_COUNT] = {};
    size_t smem[EK_COUNT] = {};
    int grid[EK_COUNT] = {};
    int rot = 0;  // which field table is current
    int *d_err = nullptr;
    bool tables_dirty = true;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_launches[2] = {0, 0};
    bool moist = false;
    int dev = 0;
    int adv_ti = ADV_TI, adv_tj = ADV_TJ;  // advection tile of every member (autotuned)
    // FP32 members with whole level quads run the four-level post, and the
    // four-level advection (tile adv_qi x adv_qj) while every basic state is
    // a function of height and adv_quad is set (autotuned)
    bool quad = false, adv_quad = true;
    int adv_qi = 4, adv_qj = 8, adv_qb = 3;  // quad tile, blocks per SM of its register budget
    int sx_threads = 256;  // threads of a fused spectral-x block (autotuned)
    // the x solve: fused kernel (0) or x FFT, Thomas, inverse x FFT (1), the
    // level tile of the x FFTs and the columns of a Thomas block (autotuned)
    int sx_unfused = 0, KTx = 8, TC = 64;
    bool fused_ok = true;  // every member fits the fused x kernel
    int nsm = 0;
    bool adv_quad_now = false;  // the choice build_prefixes made (prefixes and launches agree)
    bool quad_applies() const
    {
        if (!quad || !adv_quad) return false;
        for (auto *e : mem)
            if (!e->quad_ok(adv_qi, adv_qj)) return false;
        return true;
    }
    bool use_adv_quad() const { return adv_quad_now; }

    Ensemble(const ga_config *cfgs, const ga_columns *cols, int n, int *rc)
    {
        *rc = GA_OK;
        nmem = n;
        dev = cfgs[0].device;
        cudaSetDevice(dev);
        cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        moist = cfgs[0].microphysics_option == 1;
        for (int m = 0; m < n; m++) {
            Engine<T> *e = new Engine<T>(&cfgs[m], &cols[m]);
            if (e->status != GA_OK) {
                *rc = e->status;
                delete e;
                return;
            }
            if (e->smem_adv > 200 * 1024) {
                *rc = GA_ERR_UNSUPPORTED;
                set_error("ensemble: member too large for the batched kernels");
                delete e;
                return;
            }
            fused_ok = fused_ok && e->psx > 0;  // every level of a wavenumber fits shared memory
            mem.push_back(e);
        }
        cudaMalloc(&d_p, sizeof(KParams<T>) * n);
        cudaMalloc(&d_f[0], sizeof(KFields<T>) * n);
        cudaMalloc(&d_f[1], sizeof(KFields<T>) * n);
        cudaMalloc(&d_aux, sizeof(MemberAux<T>) * n);
        cudaMalloc(&d_err, sizeof(int));
        cudaMemset(d_err, 0, sizeof(int));
        const int optin = 200 * 1024;
        cudaFuncSetAttribute(kb_advect<T, 4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_advect<T, 2, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_advect<T, 4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_advect<T, 4, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_advect<T, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_div_fft_y<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_spectral_x<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_ifft_y_pi<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_fft_x<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(kb_thomas<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (const char *ev = std::getenv("GA_SPECTRAL_X")) sx_unfused = !std::strcmp(ev, "unfused");
        if (!fused_ok) sx_unfused = 1;
        while (KTx > 1 && !ktx_fits(KTx)) KTx >>= 1;
        if constexpr (sizeof(T) == 4) {
            quad = true;
            for (auto *e : mem) quad = quad && e->NZ % 4 == 0;
            cudaFuncSetAttribute(kb_advect_quad<T, 4, 4, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 4, 4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 4, 8, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 4, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 8, 4, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 8, 4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 2, 8, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 2, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 8, 8, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(kb_advect_quad<T, 8, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        }
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        build_prefixes();
        if (cudaDeviceSynchronize() != cudaSuccess) *rc = GA_ERR_CUDA;
    }

    ~Ensemble() override
    {
        cudaSetDevice(dev);
        if (stream) cudaStreamSynchronize(stream);
        for (auto &g : graph)
            if (g) cudaGraphExecDestroy(g);
        for (auto *e : mem) delete e;
        cudaFree(d_p);
        cudaFree(d_f[0]);
        cudaFree(d_f[1]);
        cudaFree(d_aux);
        cudaFree(d_err);
        for (auto *p : d_pre) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }

    // the batched four-level advection of tile TI x TJ in the chosen register budget
    template <int TI, int TJ>
    const void *quad_fn() const
    {
        if (adv_qb == 4) return (const void *)kb_advect_quad<T, TI, TJ, 4>;
        return (const void *)kb_advect_quad<T, TI, TJ, 3>;
    }
    template <int TI, int TJ>
    void launch_quad(dim3 g, size_t sm, const long *pr, const KFields<T> *F, double st, int what)
    {
        if (adv_qb == 4) kb_advect_quad<T, TI, TJ, 4><<<g, AQ_THREADS, sm, stream>>>(d_p, F, pr, nmem, st, what);
        else kb_advect_quad<T, TI, TJ, 3><<<g, AQ_THREADS, sm, stream>>>(d_p, F, pr, nmem, st, what);
    }
    const void *advect_fn() const
    {
        if constexpr (sizeof(T) == 4) {
            if (use_adv_quad()) {
                if (adv_qi == 4 && adv_qj == 4) return quad_fn<4, 4>();
                if (adv_qi == 8 && adv_qj == 4) return quad_fn<8, 4>();
                if (adv_qi == 2) return quad_fn<2, 8>();
                if (adv_qi == 8) return quad_fn<8, 8>();
                return quad_fn<4, 8>();
            }
        }
        if (adv_ti == 2) return (const void *)kb_advect<T, 2, 4>;
        if (adv_tj == 2) return (const void *)kb_advect<T, 4, 2>;
        if (adv_tj == 8) return (const void *)kb_advect<T, 4, 8>;
        if (adv_ti == 8) return (const void *)kb_advect<T, 8, 4>;
        return (const void *)kb_advect<T, 4, 4>;
    }
    void launch_advect(const KFields<T> *F, double st, int what)
    {
        const dim3 g(grid[EK_ADV]);
        const size_t sm = smem[EK_ADV];
        const long *pr = d_pre[EK_ADV];
        if constexpr (sizeof(T) == 4) {
            if (use_adv_quad()) {
                if (adv_qi == 4 && adv_qj == 4) launch_quad<4, 4>(g, sm, pr, F, st, what);
                else if (adv_qi == 8 && adv_qj == 4) launch_quad<8, 4>(g, sm, pr, F, st, what);
                else if (adv_qi == 2) launch_quad<2, 8>(g, sm, pr, F, st, what);
                else if (adv_qi == 8) launch_quad<8, 8>(g, sm, pr, F, st, what);
                else launch_quad<4, 8>(g, sm, pr, F, st, what);
                return;
            }
        }
        if (adv_ti == 2) kb_advect<T, 2, 4><<<g, 256, sm, stream>>>(d_p, F, pr, nmem, st, what);
        else if (adv_tj == 2) kb_advect<T, 4, 2><<<g, 256, sm, stream>>>(d_p, F, pr, nmem, st, what);
        else if (adv_tj == 8) kb_advect<T, 4, 8><<<g, 256, sm, stream>>>(d_p, F, pr, nmem, st, what);
        else if (adv_ti == 8) kb_advect<T, 8, 4><<<g, 256, sm, stream>>>(d_p, F, pr, nmem, st, what);
        else kb_advect<T, 4, 4><<<g, 256, sm, stream>>>(d_p, F, pr, nmem, st, what);
    }

    void launch_post(const KFields<T> *F, int4 a, int4 b, double st)
    {
        if constexpr (sizeof(T) == 4) {
            if (quad) {
                kb_post_quad<T><<<grid[EK_POST], PQ_THREADS, 0, stream>>>(d_p, F, d_pre[EK_POST], nmem, a, b, st);
                return;
            }
        }
        kb_post<T><<<grid[EK_POST], POST_THREADS, 0, stream>>>(d_p, F, d_pre[EK_POST], nmem, a, b, st);
    }
    void launch_sx()
    {
        if (sx_unfused) {
            const dim3 bx(KTx, std::max(1, 256 / KTx));
            kb_fft_x<T><<<grid[EK_FX], bx, smem[EK_FX], stream>>>(d_p, d_aux, d_pre[EK_FX], nmem, 0, KTx);
            kb_thomas<T><<<grid[EK_TH], 256, smem[EK_TH], stream>>>(d_p, d_aux, d_pre[EK_TH], nmem, TC);
            kb_fft_x<T><<<grid[EK_FX], bx, smem[EK_FX], stream>>>(d_p, d_aux, d_pre[EK_FX], nmem, 1, KTx);
            return;
        }
        kb_spectral_x<T><<<grid[EK_SX], dim3(64, sx_threads / 64), smem[EK_SX], stream>>>(d_p, d_aux, d_pre[EK_SX],
                                                                                          nmem);
    }
    int sx_launches() const { return sx_unfused ? 3 : 1; }
    // an x level tile every member's x FFT can hold in shared memory
    bool ktx_fits(int kt) const
    {
        for (auto *e : mem)
            if (kt > 2 * (e->NZ - 2) || 2 * (size_t)e->kp.ni * kt * sizeof(typename V2<T>::t) > 200 * 1024)
                return false;
        return true;
    }

    // virtual-block prefixes per kernel phase (for the current advection tile
    // and level tiles) and the persistent grid of each phase: as many blocks
    // as stay resident
    void build_prefixes()
    {
        const int n = nmem;
        adv_quad_now = quad_applies();
        for (int k = 0; k < EK_COUNT; k++) {
            std::vector<long> pre(n + 1, 0);
            size_t sm = 0;
            for (int m = 0; m < n; m++) {
                Engine<T> &e = *mem[m];
                long c = 0;
                switch (k) {
                case EK_ADV:
                    if (use_adv_quad()) {
                        c = (long)cdiv(e.NX - 6, adv_qi) * cdiv(e.NY - 6, adv_qj);
                        sm = std::max(sm, advect_quad_smem(adv_qi, adv_qj, e.NZ));
                    } else {
                        c = (long)cdiv(e.NX - 6, adv_ti) * cdiv(e.NY - 6, adv_tj);
                        sm = std::max(sm, advect_tile_smem(adv_ti, adv_tj, e.NZ, sizeof(T)));
                    }
                    break;
                case EK_MIRROR: c = cdiv(2L * (e.NX + e.NY - 2) * (e.NZ - 2), 256); break;
                case EK_DIVY:
                case EK_IFFTY:
                    c = (long)e.kp.ni * cdiv(e.NZ - 2, e.KTy);
                    sm = std::max(sm, e.smem_y);
                    break;
                case EK_SX:
                    c = e.kp.nj;
                    sm = std::max(sm, e.smem_sx);
                    break;
                case EK_POST:
                    c = quad ? cdiv((long)e.NX * e.NY * (e.NZ / 4), PQ_THREADS) : cdiv((long)e.NX * e.NY, POST_COLS);
                    break;
                case EK_KES: c = cdiv((long)(e.NX - 2) * (e.NY - 2) * (e.NZ - 2), 128); break;
                case EK_FX:
                    c = (long)e.kp.nj * cdiv(e.NZ - 2, KTx);
                    sm = std::max(sm, 2 * (size_t)e.kp.ni * KTx * sizeof(typename V2<T>::t));
                    break;
                case EK_TH:
                    c = cdiv((long)e.kp.ni * e.kp.nj, TC);
                    sm = std::max(sm, (size_t)TC * (e.NZ | 1) * (sizeof(typename V2<T>::t) + sizeof(T)));
                    break;
                }
                pre[m + 1] = pre[m] + c;
            }
            total[k] = pre[n];
            smem[k] = sm;
            if (!d_pre[k]) cudaMalloc(&d_pre[k], sizeof(long) * (n + 1));
            cudaMemcpy(d_pre[k], pre.data(), sizeof(long) * (n + 1), cudaMemcpyHostToDevice);
        }
        auto occ = [&](const void *fn, int threads, size_t sm) {
            int b = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, threads, sm);
            return std::max(1, b) * nsm;
        };
        grid[EK_ADV] = occ(advect_fn(), 256, smem[EK_ADV]);
        grid[EK_MIRROR] = occ((const void *)kb_mirror<T>, 256, 0);
        grid[EK_DIVY] = occ((const void *)kb_div_fft_y<T>, 256, smem[EK_DIVY]);
        grid[EK_SX] = occ((const void *)kb_spectral_x<T>, 256, smem[EK_SX]);
        grid[EK_IFFTY] = occ((const void *)kb_ifft_y_pi<T>, 256, smem[EK_IFFTY]);
        grid[EK_POST] = occ((const void *)kb_post<T>, POST_THREADS, 0);
        if constexpr (sizeof(T) == 4) {
            if (quad) grid[EK_POST] = occ((const void *)kb_post_quad<T>, PQ_THREADS, 0);
        }
        grid[EK_KES] = occ((const void *)kb_kessler<T>, 128, 0);
        grid[EK_FX] = occ((const void *)kb_fft_x<T>, KTx * std::max(1, 256 / KTx), smem[EK_FX]);
        grid[EK_TH] = occ((const void *)kb_thomas<T>, 256, smem[EK_TH]);
        for (int k = 0; k < EK_COUNT; k++) grid[k] = (int)std::min<long>(grid[k], std::max(1L, total[k]));
    }

    // Autotuner of the batched step: the advection tile and the level tile of
    // the y transforms (one for every member), timed over all members on
    // their current state; P, the fall speed and pi of every member are
    // restored afterwards.  Results are bit-identical for every choice.
    int tune() override
    {
        cudaSetDevice(dev);
        refresh_tables();
        const int nf = (moist ? 7 : 4) + 2;
        size_t tot = 0;
        for (auto *e : mem) tot += (size_t)nf * e->N;
        T *snap = nullptr;
        if (cudaMalloc(&snap, tot * sizeof(T)) != cudaSuccess) return GA_ERR_NOMEM;
        auto copy_all = [&](bool save) {
            size_t o = 0;
            for (auto *e : mem) {
                T *ptr[9];
                int np = 0;
                for (int f = 0; f < nf - 2; f++) ptr[np++] = e->buf[f][e->pi_[f]];
                ptr[np++] = e->pi;
                ptr[np++] = e->vt;
                for (int q = 0; q < np; q++, o += e->N) {
                    if (save) cudaMemcpyAsync(snap + o, ptr[q], e->N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
                    else cudaMemcpyAsync(ptr[q], snap + o, e->N * sizeof(T), cudaMemcpyDeviceToDevice, stream);
                }
            }
        };
        copy_all(true);
        cudaEvent_t ea, eb;
        cudaEventCreate(&ea);
        cudaEventCreate(&eb);
        const long long l0 = launches;
        auto timeit = [&](auto fn) {
            fn();
            cudaEventRecord(ea, stream);
            for (int r = 0; r < 3; r++) fn();
            cudaEventRecord(eb, stream);
            cudaEventSynchronize(eb);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ea, eb);
            return cudaGetLastError() == cudaSuccess ? ms / 3.f : 1e30f;
        };
        const int what = ADV_UV | ADV_WB | ADV_TH | (moist ? (ADV_Q | ADV_ZERO) : 0);
        const KFields<T> *F = d_f[rot];
        std::string info;
        char line[160];
        {
            float best = 1e30f;
            int bi = adv_ti, bj = adv_tj, qi = adv_qi, qj = adv_qj, qb = adv_qb;
            bool bq = false;
            adv_quad = false;
            for (auto &tl : Engine<T>::kAdvTiles) {
                bool fits = true;
                for (auto *e : mem) fits = fits && advect_tile_smem(tl[0], tl[1], e->NZ, sizeof(T)) <= 200 * 1024;
                if (!fits) continue;
                adv_ti = tl[0];
                adv_tj = tl[1];
                build_prefixes();
                const float t = timeit([&] { launch_advect(F, 1. / 3., what); });
                if (t < best) { best = t; bi = tl[0]; bj = tl[1]; }
            }
            if (quad) {
                adv_quad = true;
                for (auto &tl : Engine<T>::kQuadTiles) {
                    for (int mb = 3; mb <= 4; mb++) {
                        adv_qi = tl[0];
                        adv_qj = tl[1];
                        adv_qb = mb;
                        if (!quad_applies()) continue;
                        build_prefixes();
                        const float t = timeit([&] { launch_advect(F, 1. / 3., what); });
                        if (t < best) { best = t; bq = true; qi = tl[0]; qj = tl[1]; qb = mb; }
                    }
                }
            }
            adv_ti = bi;
            adv_tj = bj;
            adv_quad = bq;
            adv_qi = qi;
            adv_qj = qj;
            adv_qb = qb;
            build_prefixes();
            if (bq)
                std::snprintf(line, sizeof line, "advect tile %dx%d, four levels per thread, %d blocks/SM (%.3f ms); ", qi,
                              qj, qb, best);
            else std::snprintf(line, sizeof line, "advect tile %dx%d (%.3f ms); ", bi, bj, best);
            info += line;
        }
        {
            std::vector<int> keep(nmem);
            for (int m = 0; m < nmem; m++) keep[m] = mem[m]->KTy;
            auto set_kty = [&](int kt) {
                for (auto *e : mem) {
                    e->KTy = kt;
                    e->smem_y = 2 * (size_t)e->kp.nj * kt * sizeof(T2);
                }
                tables_dirty = true;
                refresh_tables();
                build_prefixes();
            };
            auto chain = [&] {
                const KFields<T> *G = d_f[rot];
                kb_mirror<T><<<grid[EK_MIRROR], 256, 0, stream>>>(d_p, G, d_pre[EK_MIRROR], nmem);
                kb_div_fft_y<T><<<grid[EK_DIVY], dim3(16, 16), smem[EK_DIVY], stream>>>(d_p, G, d_aux,
                                                                                       d_pre[EK_DIVY], nmem, 1. / 3.);
                launch_sx();
                kb_ifft_y_pi<T><<<grid[EK_IFFTY], dim3(16, 16), smem[EK_IFFTY], stream>>>(d_p, G, d_aux,
                                                                                         d_pre[EK_IFFTY], nmem);
            };
            float best = 1e30f;
            int bk = -1;
            for (int kt = 1; kt <= 64; kt <<= 1) {
                bool fits = true;
                for (auto *e : mem)
                    fits = fits && kt <= 2 * (e->NZ - 2) && 2 * (size_t)e->kp.nj * kt * sizeof(T2) <= 200 * 1024;
                if (!fits) break;
                set_kty(kt);
                const float t = timeit(chain);
                if (t < best) { best = t; bk = kt; }
            }
            if (bk > 0) {
                set_kty(bk);
            } else {
                for (int m = 0; m < nmem; m++) {
                    mem[m]->KTy = keep[m];
                    mem[m]->smem_y = 2 * (size_t)mem[m]->kp.nj * keep[m] * sizeof(T2);
                }
                tables_dirty = true;
                refresh_tables();
                build_prefixes();
            }
            // the x solve: the fused kernel's block sizes (when every member
            // fits it), then the unfused solve for each x level tile
            float bxs = 1e30f;
            int bu = sx_unfused, bkx = KTx, bt = sx_threads;
            if (fused_ok) {
                sx_unfused = 0;
                for (int nt : {256, 512}) {
                    sx_threads = nt;
                    const float t = timeit(chain);
                    if (t < bxs) { bxs = t; bu = 0; bt = nt; }
                }
            }
            for (int kt = 1; kt <= 64; kt <<= 1) {
                if (!ktx_fits(kt)) break;
                sx_unfused = 1;
                KTx = kt;
                build_prefixes();
                const float t = timeit(chain);
                if (t < bxs) { bxs = t; bu = 1; bkx = kt; }
            }
            sx_unfused = bu;
            KTx = bkx;
            sx_threads = bt;
            build_prefixes();
            best = bxs;
            if (sx_unfused)
                std::snprintf(line, sizeof line, "y level tile %d, x level tile %d (pressure solve %.3f ms)", bk, KTx,
                              best);
            else
                std::snprintf(line, sizeof line, "y level tile %d, x block %d threads (pressure solve %.3f ms)", bk,
                              sx_threads, best);
            info += line;
        }
        copy_all(false);
        cudaError_t e = cudaStreamSynchronize(stream);
        cudaEventDestroy(ea);
        cudaEventDestroy(eb);
        cudaFree(snap);
        launches = l0;
        for (auto &g : graph)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
        tuning = info;
        if (e != cudaSuccess) {
            set_error(std::string("CUDA: ") + cudaGetErrorString(e));
            return GA_ERR_CUDA;
        }
        return GA_OK;
    }

    // member tables: parameters (after basic-state refresh) and both rotation states
    void refresh_tables()
    {
        for (auto *e : mem) {
            if (e->btab_dirty) {
                e->refresh_base();
                tables_dirty = true;
                e->sync_status();
            }
        }
        if (!tables_dirty) return;
        tables_dirty = false;
        std::vector<KParams<T>> hp(nmem);
        std::vector<KFields<T>> f0(nmem), f1(nmem);
        std::vector<MemberAux<T>> ha(nmem);
        for (int m = 0; m < nmem; m++) {
            Engine<T> &e = *mem[m];
            hp[m] = e.kp;
            hp[m].dt_d = e.cfg.dt;
            f0[m] = e.fields();
            f1[m] = f0[m];
            for (int f = 0; f < 7; f++) std::swap(f1[m].cur[f], f1[m].P[f]);
            ha[m].spec = e.spec; ha[m].tw_i = e.tw_i; ha[m].tw_j = e.tw_j;
            ha[m].plan_i = e.plan_i; ha[m].plan_j = e.plan_j;
            ha[m].KTy = e.KTy; ha[m].psx = e.psx;
        }
        cudaMemcpy(d_p, hp.data(), sizeof(KParams<T>) * nmem, cudaMemcpyHostToDevice);
        cudaMemcpy(d_f[0], f0.data(), sizeof(KFields<T>) * nmem, cudaMemcpyHostToDevice);
        cudaMemcpy(d_f[1], f1.data(), sizeof(KFields<T>) * nmem, cudaMemcpyHostToDevice);
        cudaMemcpy(d_aux, ha.data(), sizeof(MemberAux<T>) * nmem, cudaMemcpyHostToDevice);
        build_prefixes();  // a basic state that changed may change the advection kernel
        rot = 0;
        for (auto &g : graph)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    }

    void swap_all()
    {
        rot ^= 1;
        for (auto *e : mem) e->swap_inner(true);
    }

    void rk3_step()
    {
        static const double steps[3] = {1. / 3., 0.5, 1.0};
        for (int s = 0; s < 3; s++) {
            const double st = steps[s];
            KFields<T> *F = d_f[rot];
            const int what = ADV_UV | ADV_WB | ADV_TH | (moist ? (ADV_Q | ADV_ZERO) : 0);
            launch_advect(F, st, what);
            kb_mirror<T><<<grid[EK_MIRROR], 256, 0, stream>>>(d_p, F, d_pre[EK_MIRROR], nmem);
            kb_div_fft_y<T><<<grid[EK_DIVY], dim3(16, 16), smem[EK_DIVY], stream>>>(d_p, F, d_aux, d_pre[EK_DIVY],
                                                                                   nmem, st);
            launch_sx();
            kb_ifft_y_pi<T><<<grid[EK_IFFTY], dim3(16, 16), smem[EK_IFFTY], stream>>>(d_p, F, d_aux, d_pre[EK_IFFTY],
                                                                                     nmem);
            const int fu = PF_PROJECT | PF_SPONGE | PF_VBC, ft = PF_SPONGE | PF_VBC, fq = PF_ZERO | PF_SPONGE | PF_VBC;
            launch_post(F, make_int4(fu, fu, fu, ft), make_int4(fq, fq, fq, 0), st);
            launches += 5 + sx_launches();
            if (s < 2) swap_all();
        }
        KFields<T> *F = d_f[rot];
        if (moist) {
            kb_kessler<T><<<grid[EK_KES], 128, 0, stream>>>(d_p, F, d_pre[EK_KES], nmem, d_err);
            launches++;
        }
        const int fu = PF_SPONGE | PF_VBC | PF_RAYLEIGH | PF_WRITE_M, fq = PF_SPONGE | PF_VBC | PF_WRITE_M;
        launch_post(F, make_int4(fu, fu, fu, fu), make_int4(fq, fq, fq, 0), 1.0);
        launches++;
        swap_all();
        for (auto *e : mem) {
            e->bigcounter++;
            e->mtime += e->cfg.dt;
        }
    }

    int step(int nsteps) override
    {
        cudaSetDevice(dev);
        refresh_tables();
        int n = 0;
        while (nsteps - n >= 2) {
            const int parity = rot;
            if (!graph[parity]) {
                std::vector<long long> bc(nmem);
                std::vector<double> mt(nmem);
                for (int m = 0; m < nmem; m++) { bc[m] = mem[m]->bigcounter; mt[m] = mem[m]->mtime; }
                const long long l0 = launches;
                cudaGraph_t g = nullptr;
                if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) break;
                rk3_step();
                rk3_step();
                if (cudaStreamEndCapture(stream, &g) != cudaSuccess) { cudaGetLastError(); break; }
                cudaError_t e = cudaGraphInstantiate(&graph[parity], g, 0);
                cudaGraphDestroy(g);
                graph_launches[parity] = launches - l0;
                launches = l0;
                for (int m = 0; m < nmem; m++) { mem[m]->bigcounter = bc[m]; mem[m]->mtime = mt[m]; }
                if (e != cudaSuccess) { cudaGetLastError(); graph[parity] = nullptr; break; }
            }
            if (cudaGraphLaunch(graph[parity], stream) != cudaSuccess) break;
            launches += graph_launches[parity];
            for (auto *e : mem) {
                e->bigcounter += 2;
                e->mtime += 2 * e->cfg.dt;
            }
            n += 2;
        }
        for (; n < nsteps; n++) rk3_step();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(std::string("CUDA launch: ") + cudaGetErrorString(e));
            return GA_ERR_CUDA;
        }
        return GA_OK;
    }

    int synchronize() override
    {
        cudaSetDevice(dev);
        cudaError_t e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) {
            set_error(std::string("CUDA: ") + cudaGetErrorString(e));
            return GA_ERR_CUDA;
        }
        int h = 0;
        cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (h) {
            set_error("Kessler evaporation E>100 in an ensemble member (the reference exits here)");
            return GA_ERR_KESSLER;
        }
        return GA_OK;
    }

    EngineBase *member(int m) override { return (m >= 0 && m < nmem) ? mem[m] : nullptr; }
    int size() const override { return nmem; }
    void *stream_handle() override { return stream; }
    void mark_dirty() override { tables_dirty = true; }
};

template <typename T>
EnsembleBase *make_ensemble(const ga_config *cfgs, const ga_columns *cols, int n, int *rc)
{
    Ensemble<T> *e = new Ensemble<T>(cfgs, cols, n, rc);
    if (*rc != GA_OK) {
        delete e;
        return nullptr;
    }
    return e;
}

}  // namespace ga
