// ga_lin.cuh - host side of the tangent-linear model and the adjoint of one
// precision (dry, non-periodic contexts): perturbation / adjoint buffers that
// rotate like the state's, the TLM step, and the checkpointed adjoint sweep.
// Included at the end of ga_engine.cuh; defines Engine<T>'s linearisation
// members.
#pragma once
#include <memory>

#include "ga_engine.cuh"
#include "ga_lin_kernels.cuh"
#include "ga_adj_quad.cuh"

namespace ga {

template <typename T>
struct Lin : LinBase {
    typedef typename V2<T>::t T2;
    Engine<T> &e;
    long N;
    int nf;              // linearised prognostic fields: 4 dry, 7 moist
    T *lb[7][3] = {};
    int lci[7], lpi[7], lmi[7];
    T *lpi_f = nullptr;  // pi (perturbation or adjoint)
    T *dbar = nullptr;   // adjoint of the divergence, real [i][j][k]
    T *coef = nullptr;   // linearised face coefficients of one stage (LIN_NCOEF[_MOIST] fields)
    unsigned char *mask = nullptr;   // clipping record of the trajectory's current stage (TLM)
    unsigned char *mtape = nullptr;  // clipping records of a segment: 3 stages x N per step (adjoint)
    double *rain_keep = nullptr;     // accumulated rain of the final state, kept over the recomputation
    T *tape = nullptr;   // stage-start u, v, w, theta of every step of a segment
    size_t tape_steps = 0;
    T *ckpt = nullptr;   // full states (current, P, M of u, v, w, theta)
    size_t ckpt_slots = 0;
    // two recorded steps into trajectory slots (2m, 2m+1), per rotation parity
    std::vector<cudaGraphExec_t> rec_graph[2];
    std::vector<long long> rec_graph_launches[2];
    // the four-level adjoint advection (FP32, NZ % 4 == 0); GA_ADJ=level keeps
    // the per-level kernel
    bool adj_quad = false;
    // the coefficient pass of a stage needs only the trajectory: it runs on a
    // side stream beside the pressure adjoint
    cudaStream_t side = nullptr;
    cudaEvent_t ev_cols = nullptr, ev_coef = nullptr;

    explicit Lin(Engine<T> &eng) : e(eng), N(eng.N), nf(eng.nprog)
    {
        for (int f = 0; f < nf; f++) {
            for (int s = 0; s < 3; s++) lb[f][s] = e.template dalloc<T>(N);
            lci[f] = 0; lpi[f] = 1; lmi[f] = 2;
        }
        lpi_f = e.template dalloc<T>(N);
        dbar = e.template dalloc<T>(N);
        coef = e.template dalloc<T>((size_t)(nf == 7 ? LIN_NCOEF_MOIST : LIN_NCOEF) * N);
        if (nf == 7) {
            mask = e.template dalloc<unsigned char>(N);
            rain_keep = e.template dalloc<double>((size_t)e.NX * e.NY);
        }
        cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&ev_cols, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev_coef, cudaEventDisableTiming);
        const int optin = 200 * 1024;
        cudaFuncSetAttribute(k_adj_fft_y_in<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_adj_ifft_y_out<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_thomas_adj<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_spectral_x_adj<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_adj_advect<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_adj_advect<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if constexpr (sizeof(T) == 4) {
            const char *ev = std::getenv("GA_ADJ");
            adj_quad = e.NZ % 4 == 0 && !(ev && !std::strcmp(ev, "level"));
            cudaFuncSetAttribute(k_adj_advect_quad<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(k_adj_advect_quad<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        }
    }
    ~Lin() override
    {
        drop_graphs();
        if (tape) cudaFree(tape);
        if (mtape) cudaFree(mtape);
        if (ckpt) cudaFree(ckpt);
        if (side) {
            cudaStreamSynchronize(side);
            cudaStreamDestroy(side);
        }
        if (ev_cols) cudaEventDestroy(ev_cols);
        if (ev_coef) cudaEventDestroy(ev_coef);
    }

    // trajectory fields per step: stage-start prognostic fields, and (moist)
    // the inputs of Kessler
    size_t per_step() const { return (size_t)(3 * nf + (nf == 7 ? 5 : 0)) * N; }
    T *rec_at(int slot) { return tape + (size_t)slot * per_step(); }
    unsigned char *mrec_at(int slot) { return mtape ? mtape + (size_t)slot * 3 * N : nullptr; }

    void drop_graphs() override
    {
        for (int par = 0; par < 2; par++) {
            for (auto &g : rec_graph[par])
                if (g) cudaGraphExecDestroy(g);
            rec_graph[par].clear();
            rec_graph_launches[par].clear();
        }
    }

    // two steps recording into trajectory slots m2, m2+1: replayed from a
    // CUDA graph captured on first use (slots and parity fix every pointer)
    void record_pair(int m2)
    {
        const int par = e.ci[0] == 0 ? 0 : 1;
        const size_t idx = (size_t)m2;
        auto &gs = rec_graph[par];
        auto &ls = rec_graph_launches[par];
        if (gs.size() <= idx) {
            gs.resize(idx + 1, nullptr);
            ls.resize(idx + 1, 0);
        }
        if (!gs[idx] && e.use_graphs) {
            const long long bc = e.bigcounter, l0 = e.launches;
            const double mt = e.mtime;
            cudaGraph_t g = nullptr;
            bool ok = cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                e.rk3_step(rec_at(m2), mrec_at(m2));
                e.rk3_step(rec_at(m2 + 1), mrec_at(m2 + 1));
                ok = cudaStreamEndCapture(e.stream, &g) == cudaSuccess;
            }
            if (ok) ok = cudaGraphInstantiate(&gs[idx], g, 0) == cudaSuccess;
            if (g) cudaGraphDestroy(g);
            ls[idx] = e.launches - l0;
            e.launches = l0;
            e.bigcounter = bc;
            e.mtime = mt;
            if (!ok) {
                cudaGetLastError();
                gs[idx] = nullptr;
            }
        }
        if (gs[idx] && cudaGraphLaunch(gs[idx], e.stream) == cudaSuccess) {
            e.launches += ls[idx];
            e.bigcounter += 2;
            e.mtime += 2 * e.cfg.dt;
        } else {
            e.rk3_step(rec_at(m2), mrec_at(m2));
            e.rk3_step(rec_at(m2 + 1), mrec_at(m2 + 1));
        }
    }

    // steps n0..n1-1 of a segment, recording step n into trajectory slot
    // base + n - n0
    void record_segment(int n0, int n1, int base)
    {
        int n = n0;
        for (; n + 1 < n1; n += 2) record_pair(base + n - n0);
        if (n < n1) e.rk3_step(rec_at(base + n - n0), mrec_at(base + n - n0));
    }
    // bytes of the trajectory of one step (fields and clipping records)
    size_t step_bytes() const { return per_step() * sizeof(T) + (nf == 7 ? 3 * (size_t)N : 0); }

    KFields<T> fields() const
    {
        KFields<T> F;
        std::memset(&F, 0, sizeof(F));
        for (int f = 0; f < nf; f++) {
            F.cur[f] = lb[f][lci[f]];
            F.P[f] = lb[f][lpi[f]];
            F.M[f] = lb[f][lmi[f]];
        }
        for (int b = 0; b < 6; b++) F.bar[b] = e.bar[b];
        F.pi = lpi_f;
        F.vt = e.vt;
        return F;
    }

    T *slot_ptr(int field, int slot)
    {
        if (field == GA_PI) return lpi_f;
        if (field < 0 || field >= nf) return nullptr;
        if (slot == GA_SLOT_CUR) return lb[field][lci[field]];
        if (slot == GA_SLOT_P) return lb[field][lpi[field]];
        if (slot == GA_SLOT_M) return lb[field][lmi[field]];
        return nullptr;
    }

    // run the engine's (linear) forward kernels on these buffers
    void exchange()
    {
        for (int f = 0; f < nf; f++) {
            for (int s = 0; s < 3; s++) std::swap(e.buf[f][s], lb[f][s]);
            std::swap(e.ci[f], lci[f]);
            std::swap(e.pi_[f], lpi[f]);
            std::swap(e.mi[f], lmi[f]);
        }
        std::swap(e.pi, lpi_f);
    }
    void swap_inner()
    {
        for (int f = 0; f < nf; f++) std::swap(lci[f], lpi[f]);
    }

    // the posts of the step as they act on perturbations: zero_moisture is
    // left out (values reaching the post are already clipped, so it is
    // inactive there; the advection's clipping carries the mask)
    static void stage_flags(int *fl)
    {
        for (int f = 0; f < 7; f++) fl[f] = 0;
        fl[FU] = fl[FV] = fl[FW] = PF_PROJECT | PF_SPONGE | PF_VBC;
        fl[FTH] = fl[FQV] = fl[FQC] = fl[FQR] = PF_SPONGE | PF_VBC;
    }
    static void final_flags(int *fl)
    {
        for (int f = 0; f < 7; f++) fl[f] = 0;
        fl[FU] = fl[FV] = fl[FW] = fl[FTH] = PF_SPONGE | PF_VBC | PF_RAYLEIGH | PF_WRITE_M;
        fl[FQV] = fl[FQC] = fl[FQR] = PF_SPONGE | PF_VBC | PF_WRITE_M;
    }

    // one step of the state and of the perturbations together
    void tlm_step()
    {
        static const double steps[3] = {1. / 3., 0.5, 1.0};
        const long tot = (long)(e.NX - 6) * (e.NY - 6) * (e.NZ - 2);
        int fl[7];
        const bool moist = nf == 7;
        for (int s = 0; s < 3; s++) {
            const double st = steps[s];
            const T sdtg = (T)(st * e.cfg.dt * 9.8 * 0.5);
            e.qmask = mask;
            e.advect(st, ADV_UV | ADV_WB | ADV_TH | (moist ? (ADV_Q | ADV_ZERO) : 0));
            e.qmask = nullptr;
            KFields<T> R = e.fields();
            R.qmask = mask;
            k_tl_advect<T><<<cdiv(tot, 128), 128, 0, e.stream>>>(e.kp, R, fields(), (T)st, sdtg);
            e.launches++;
            stage_flags(fl);
            e.solve_pressure(st);
            e.post(fl, 7, st, true);
            exchange();
            e.solve_pressure(st);
            e.post(fl, 7, st, true);
            exchange();
            if (s < 2) {
                e.swap_inner(true);
                swap_inner();
            }
        }
        if (moist) {  // Kessler: the tangent about the trajectory before its own update
            const long tk = (long)(e.NX - 2) * (e.NY - 2) * (e.NZ - 2);
            k_tl_kessler<T><<<cdiv(tk, 128), 128, 0, e.stream>>>(e.kp, e.fields(), fields());
            e.launches++;
            e.kessler();
        }
        final_flags(fl);
        e.post(fl, 7, 1.0, true);
        exchange();
        e.post(fl, 7, 1.0, true);
        exchange();
        e.swap_inner(true);
        swap_inner();
        e.mtime += e.cfg.dt;
        e.bigcounter++;
    }

    // transposed pressure solve: pi-bar -> P-bar of u, v, w (pi-bar is left
    // as read; the next transposed projection overwrites it)
    void adj_pressure(double st)
    {
        KFields<T> A = fields();
        const int nkt_y = cdiv(e.NZ - 2, e.KTy), nkt_x = cdiv(e.NZ - 2, e.KTx);
        const dim3 by_y(e.KTy, std::max(1, 256 / e.KTy)), by_x(e.KTx, std::max(1, 256 / e.KTx));
        cudaStream_t s = e.stream;
        k_adj_fft_y_in<T><<<dim3(nkt_y, e.kp.ni), by_y, e.smem_y, s>>>(e.kp, lpi_f, e.spec, e.plan_j, e.tw_j, e.KTy);
        if (e.psx > 0) {  // x transforms and the solves fused, as in the forward step
            // the adjoint kernel's registers allow blocks of up to 512 threads
            const int nl = e.NZ - 2, bx = std::min(nl, 64), nt = std::min(e.sx_threads, 512);
            k_spectral_x_adj<T><<<e.kp.nj, dim3(bx, std::max(1, nt / bx)), e.smem_sx, s>>>(e.kp, e.spec, e.plan_i,
                                                                                         e.tw_i, e.psx);
            e.launches += 1;
        } else {
            k_fft_x<T><<<dim3(nkt_x, e.kp.nj), by_x, e.smem_x, s>>>(e.kp, e.spec, e.plan_i, e.tw_i, 0, e.KTx);
            const long ncol = (long)e.kp.ni * e.kp.nj;
            k_thomas_adj<T><<<cdiv(ncol, e.TC), 256, e.smem_th, s>>>(e.kp, e.spec, e.TC);
            k_fft_x<T><<<dim3(nkt_x, e.kp.nj), by_x, e.smem_x, s>>>(e.kp, e.spec, e.plan_i, e.tw_i, 1, e.KTx);
            e.launches += 3;
        }
        k_adj_ifft_y_out<T><<<dim3(nkt_y, e.kp.ni), by_y, e.smem_y, s>>>(e.kp, e.spec, dbar, e.plan_j, e.tw_j, e.KTy);
        bool div_quad = false;
        if constexpr (sizeof(T) == 4) div_quad = adj_quad;
        if (div_quad) {
            if constexpr (sizeof(T) == 4)
                k_adj_div_quad<T><<<cdiv(N / 4, 256), 256, 0, s>>>(e.kp, A, dbar, (T)(st * e.cfg.dt));
        } else {
            k_adj_div<T><<<cdiv(N, 256), 256, 0, s>>>(e.kp, A, dbar, (T)(st * e.cfg.dt));
        }
        e.launches += 3;
    }

    // adjoint of one step about the trajectory rec (stage-start u, v, w,
    // theta: rec + (4*stage + field)*N).  first: the adjoint of the final
    // state enters here (the final pi-bar, and a current slot that holds no
    // stale P-bar).
    void adj_step(const T *rec, const unsigned char *mrec, bool first)
    {
        static const double steps[3] = {1. / 3., 0.5, 1.0};
        cudaStream_t s = e.stream;
        const bool moist = nf == 7;
        const dim3 gadv(cdiv(e.NZ, AJ_TK), cdiv(e.NX, AJ_TI), cdiv(e.NY, AJ_TJ));
        const size_t smem_adv = AjCfg<T>::smem;
        swap_inner();  // advance_outer's swap
        const int ncol = cdiv((long)e.NX * e.NY * nf, 128);  // threads of k_adj_cols: (field, column)
        // the column transposes: one (field, column, level quad) per thread in FP32
        auto cols = [&](int fl) {
            if constexpr (sizeof(T) == 4) {
                if (adj_quad) {
                    k_adj_cols_quad<T><<<ncol, 128, 0, s>>>(e.kp, fields(), fl);
                    return;
                }
            }
            k_adj_cols<T><<<ncol, 128, 0, s>>>(e.kp, fields(), fl);
        };
        k_adj_fold_m<T><<<cdiv(N, 256), 256, 0, s>>>(e.kp, fields());  // advance_outer's M <- P
        e.launches++;
        if (moist) {
            // the step-final post, then Kessler (its inputs: rec + 3*nf*N);
            // pi-bar takes Kessler's pi row (first: on top of the final pi-bar)
            cols(AP_RAYLEIGH | AP_VBC | AP_SPONGE);
            k_adj_kessler<T><<<cdiv(N, 128), 128, 0, s>>>(e.kp, e.fields(), rec + (size_t)3 * nf * N, fields(),
                                                         first ? 1 : 0);
            e.launches += 2;
        }
        for (int st = 2; st >= 0; st--) {
            const double step = steps[st];
            if (st < 2) swap_inner();
            // dry: stage 2 shares its buffer with the step-final post, one pass
            int fl = AP_VBC | AP_SPONGE, acc = 0;
            if (st == 2) {
                if (moist) acc = 1;
                else {
                    fl = AP_RAYLEIGH | AP_VBC | AP_SPONGE2;
                    acc = first ? 1 : 0;
                }
            }
            cols(fl);
            // the coefficient pass (trajectory in, coefficients and the clipped
            // points' moisture P-bar out) runs on the side stream beside the
            // pressure adjoint: after the column transposes, which write that
            // P-bar, and after the previous stage's advection adjoint, which
            // read the coefficients
            {
                KFields<T> R = e.fields();
                for (int f = 0; f < nf; f++) R.cur[f] = const_cast<T *>(rec) + (size_t)(nf * st + f) * N;
                const unsigned char *qm = moist ? mrec + (size_t)st * N : nullptr;
                cudaEventRecord(ev_cols, s);
                cudaStreamWaitEvent(side, ev_cols, 0);
                bool coef_quad = false;
                if constexpr (sizeof(T) == 4) coef_quad = adj_quad && e.kp.ubase_adv;
                if (coef_quad) {
                    if constexpr (sizeof(T) == 4)
                        k_lin_coef_quad<T><<<cdiv(N / 4, LQ_THREADS), LQ_THREADS, 0, side>>>(e.kp, R, coef, fields(),
                                                                                            qm);
                } else {
                    k_lin_coef<T><<<cdiv(N, 128), 128, 0, side>>>(e.kp, R, coef, fields(), qm);
                }
                cudaEventRecord(ev_coef, side);
            }
            bool proj_quad = false;
            if constexpr (sizeof(T) == 4) proj_quad = adj_quad;
            if (proj_quad) {
                if constexpr (sizeof(T) == 4)
                    k_adj_project_quad<T><<<cdiv(N / 4, 256), 256, 0, s>>>(e.kp, fields(), (T)step, acc);
            } else {
                k_adj_project<T><<<cdiv(N, 256), 256, 0, s>>>(e.kp, fields(), (T)step, acc);
            }
            e.launches += 2;
            adj_pressure(step);
            cudaStreamWaitEvent(s, ev_coef, 0);
            const T sdtg = (T)(step * e.cfg.dt * 9.8 * 0.5);
            const int zc = (first && st == 2) ? 0 : 1;
            e.launches += 2 + (moist ? 1 : 0);
            if constexpr (sizeof(T) == 4) {
                if (adj_quad) {
                    k_adj_advect_quad<T, 0><<<gadv, AJ_THREADS, QJ_SMEM, s>>>(e.kp, coef, fields(), (T)step, sdtg, zc);
                    if (moist)
                        k_adj_advect_quad<T, 1><<<gadv, AJ_THREADS, QJ_SMEM, s>>>(e.kp, coef, fields(), (T)step, sdtg,
                                                                                 zc);
                    continue;
                }
            }
            k_adj_advect<T, 0><<<gadv, AJ_THREADS, smem_adv, s>>>(e.kp, coef, fields(), (T)step, sdtg, zc);
            if (moist) k_adj_advect<T, 1><<<gadv, AJ_THREADS, smem_adv, s>>>(e.kp, coef, fields(), (T)step, sdtg, zc);
        }
    }

    int reserve(size_t tape_need, size_t ckpt_need)
    {
        if (tape_need > tape_steps) {
            drop_graphs();
            if (tape) cudaFree(tape);
            if (mtape) cudaFree(mtape);
            tape = nullptr;
            mtape = nullptr;
            tape_steps = 0;
            if (cudaMalloc(&tape, tape_need * per_step() * sizeof(T)) != cudaSuccess) return GA_ERR_NOMEM;
            if (nf == 7 && cudaMalloc(&mtape, tape_need * 3 * (size_t)N) != cudaSuccess) return GA_ERR_NOMEM;
            tape_steps = tape_need;
        }
        if (ckpt_need > ckpt_slots) {
            if (ckpt) cudaFree(ckpt);
            ckpt = nullptr;
            ckpt_slots = 0;
            if (cudaMalloc(&ckpt, ckpt_need * 3 * nf * (size_t)N * sizeof(T)) != cudaSuccess) return GA_ERR_NOMEM;
            ckpt_slots = ckpt_need;
        }
        return GA_OK;
    }

    // copy the state (current, P, M of u, v, w, theta) to or from a checkpoint
    void checkpoint(size_t slot, bool save)
    {
        T *base = ckpt + slot * 3 * nf * (size_t)N;
        for (int f = 0; f < nf; f++) {
            const int idx[3] = {e.ci[f], e.pi_[f], e.mi[f]};
            for (int s = 0; s < 3; s++) {
                T *c = base + (size_t)(3 * f + s) * N;
                if (save) cudaMemcpyAsync(c, e.buf[f][idx[s]], N * sizeof(T), cudaMemcpyDeviceToDevice, e.stream);
                else cudaMemcpyAsync(e.buf[f][idx[s]], c, N * sizeof(T), cudaMemcpyDeviceToDevice, e.stream);
            }
        }
    }

    // Segments whose trajectory the first sweep keeps on the tape: the last
    // ones, as many as device memory holds beside the checkpoints with a
    // tenth of the GPU's memory to spare (at least one, at most all).
    // GA_ADJ_RESIDENT=n fixes the count.
    int resident_segments(int nseg, int K)
    {
        int R = 1;
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
            const size_t sb = step_bytes(), cb = 3 * (size_t)nf * N * sizeof(T);
            const size_t have = fr + tape_steps * sb + ckpt_slots * cb;  // the current tape and checkpoints are given back
            const size_t need = (size_t)(nseg + 1) * cb + tot / 10;
            if (have > need) R = (int)std::min<size_t>((size_t)nseg, (have - need) / ((size_t)K * sb));
        } else {
            cudaGetLastError();
        }
        if (const char *ev = std::getenv("GA_ADJ_RESIDENT")) R = std::atoi(ev);
        return std::max(1, std::min(R, nseg));
    }

    // nsteps forward from the current state, then the adjoint back to it.
    // States are checkpointed every K steps.  The first sweep records the
    // stage-start fields of the last `resident` segments; every earlier
    // segment is recomputed from its checkpoint (recording) before its
    // adjoint runs.
    int resident = 1;
    int adjoint(int nsteps, int K)
    {
        if (nsteps <= 0) return GA_OK;
        if (K <= 0 || K > nsteps) K = nsteps;
        const int nseg = (nsteps + K - 1) / K;
        int R = resident_segments(nseg, K);
        if (R > 1 && (size_t)R * K > tape_steps) {  // give the old tape back before the larger one
            drop_graphs();
            if (tape) cudaFree(tape);
            if (mtape) cudaFree(mtape);
            tape = nullptr;
            mtape = nullptr;
            tape_steps = 0;
        }
        int rc = reserve((size_t)R * K, (size_t)nseg + 1);
        if (rc == GA_ERR_NOMEM && R > 1) {
            cudaGetLastError();
            R = 1;
            rc = reserve((size_t)K, (size_t)nseg + 1);
        }
        if (rc) return rc;
        resident = R;
        const int first_res = nseg - R;  // first resident segment
        for (int seg = 0; seg < nseg; seg++) {
            const int n0 = seg * K, n1 = std::min(nsteps, n0 + K);
            checkpoint(seg, true);
            if (seg >= first_res) record_segment(n0, n1, (seg - first_res) * K);
            else if (int rc2 = e.step(n1 - n0)) return rc2;
        }
        checkpoint(nseg, true);
        const long long bc = e.bigcounter;
        const double mt = e.mtime;
        const size_t nrain = (size_t)e.NX * e.NY;
        if (rain_keep)  // the recomputation would accumulate the rain again
            cudaMemcpyAsync(rain_keep, e.accrain, nrain * sizeof(double), cudaMemcpyDeviceToDevice, e.stream);
        for (int seg = nseg - 1; seg >= 0; seg--) {
            const int n0 = seg * K, n1 = std::min(nsteps, n0 + K);
            int base = 0;
            if (seg >= first_res) {
                base = (seg - first_res) * K;
            } else {  // the resident segments' slots are consumed by now
                checkpoint(seg, false);
                record_segment(n0, n1, 0);
            }
            for (int n = n1 - 1; n >= n0; n--)
                adj_step(rec_at(base + n - n0), mrec_at(base + n - n0), n == nsteps - 1);
        }
        const long tot = (long)(e.NX - 6) * (e.NY - 6) * (e.NZ - 2);
        k_adj_zero_cells<T><<<cdiv(tot, 256), 256, 0, e.stream>>>(e.kp, fields());
        e.launches++;
        checkpoint(nseg, false);
        if (rain_keep)
            cudaMemcpyAsync(e.accrain, rain_keep, nrain * sizeof(double), cudaMemcpyDeviceToDevice, e.stream);
        e.bigcounter = bc;
        e.mtime = mt;
        cudaMemsetAsync(lpi_f, 0, N * sizeof(T), e.stream);  // the step does not read pi
        return GA_OK;
    }
};

template <typename T>
Lin<T> *Engine<T>::linear()
{
    if (!lin) lin.reset(new Lin<T>(*this));
    return static_cast<Lin<T> *>(lin.get());
}

template <typename T>
int Engine<T>::lin_supported() const
{
    if (kp.periodic || (kp.moist && kp.rf != 1)) {
        set_error("tangent-linear / adjoint: non-periodic contexts, Eulerian rain fallout (rain_fallout 1) only");
        return GA_ERR_UNSUPPORTED;
    }
    if (cfg.use_explicit_diffusion) {
        set_error("tangent-linear / adjoint: explicit diffusion is not linearised");
        return GA_ERR_UNSUPPORTED;
    }
    if (cfg.turbulence_option) {
        set_error("tangent-linear / adjoint: the turbulence scheme is not linearised");
        return GA_ERR_UNSUPPORTED;
    }
    if (kp.ice) {
        set_error("tangent-linear / adjoint: the ice scheme is not linearised");
        return GA_ERR_UNSUPPORTED;
    }
    if (cfg.linear_model || cfg.hydrostatic) {
        set_error("tangent-linear / adjoint: contexts of the linearised model or the hydrostatic set have none");
        return GA_ERR_UNSUPPORTED;
    }
    return GA_OK;
}

template <typename T>
int Engine<T>::lin_set_field(int field, int slot, const double *host, size_t n)
{
    if (int rc = lin_supported()) return rc;
    if (!host || n != (size_t)N) return GA_ERR_ARG;
    cudaSetDevice(device);
    T *d = linear()->slot_ptr(field, slot);
    if (!d || status) return status ? status : GA_ERR_ARG;
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

template <typename T>
int Engine<T>::lin_get_field(int field, int slot, double *host, size_t n)
{
    if (int rc = lin_supported()) return rc;
    if (!host || n != (size_t)N) return GA_ERR_ARG;
    cudaSetDevice(device);
    T *d = linear()->slot_ptr(field, slot);
    if (!d || status) return status ? status : GA_ERR_ARG;
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

template <typename T>
int Engine<T>::tlm_step(int nsteps)
{
    if (int rc = lin_supported()) return rc;
    cudaSetDevice(device);
    refresh_base();
    Lin<T> *L = linear();
    if (status) return status;
    for (int n = 0; n < nsteps; n++) {
        L->tlm_step();
        if (int rc = launch_status()) return rc;
    }
    return sync_status();
}

template <typename T>
int Engine<T>::adjoint(int nsteps, int checkpoint_every)
{
    if (int rc = lin_supported()) return rc;
    if (nsteps < 0) return GA_ERR_ARG;
    cudaSetDevice(device);
    refresh_base();
    Lin<T> *L = linear();
    if (status) return status;
    int rc = L->adjoint(nsteps, checkpoint_every);
    if (rc) {
        set_error("adjoint: out of device memory for the checkpoints / trajectory");
        return rc;
    }
    if ((rc = launch_status())) return rc;
    return sync_status();
}

}  // namespace ga
