// ga_engine.h - precision-independent interface between the C ABI
// (ga_api.cu) and the per-precision engines (ga_f64.cu, ga_f32.cu).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "ga_anelastic.h"

namespace ga {

// kernel groups timed by the optional event profiler
enum ProfCat { PC_ADVECT = 0, PC_EDGES, PC_DIV_FFT_Y, PC_FFT_X, PC_THOMAS, PC_IFFT_Y_PI, PC_POST, PC_KESSLER,
               PC_PPM, PC_COPY, PC_DIFFUSION, PC_TURBULENCE, PC_COUNT };
static const char *const kProfNames[PC_COUNT] = {"advect", "edges", "div_fft_y", "fft_x", "thomas",
                                                 "ifft_y_pi", "post", "kessler", "ppm", "copy", "diffusion",
                                                 "turbulence"};

// tangent-linear / adjoint state of an engine (ga_lin.cuh)
struct LinBase {
    virtual ~LinBase() {}
    virtual void drop_graphs() {}
};

struct EngineBase {
    virtual ~EngineBase()
    {
        for (auto &r : prof_pending) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
    }
    virtual int set_field(int field, int slot, const double *host, size_t n) = 0;
    virtual int get_field(int field, int slot, double *host, size_t n) = 0;
    virtual int op(int op, double step) = 0;
    virtual int step(int nsteps) = 0;
    virtual int check_finite() = 0;
    virtual int budget(int slot, double *out) = 0;  // GA_NBUDGET FP64 domain sums
    virtual void *field_ptr(int field, int slot) = 0;
    // tangent-linear model and adjoint (dry, non-periodic contexts)
    virtual int lin_set_field(int field, int slot, const double *host, size_t n) = 0;
    virtual int lin_get_field(int field, int slot, double *host, size_t n) = 0;
    virtual int tlm_step(int nsteps) = 0;
    virtual int adjoint(int nsteps, int checkpoint_every) = 0;
    // autotuner: times the candidate tile shapes and FFT plans, keeps the fastest
    virtual int tune() = 0;
    std::string tuning;  // the choice, as text
    cudaStream_t stream = nullptr;
    long long launches = 0;
    long long bigcounter = 0;
    double mtime = 0.0;
    int device = 0;

    // ---- optional per-group timing with CUDA events on the engine stream
    struct ProfRec {
        int cat;
        int nlaunch;
        cudaEvent_t a, b;
    };
    bool prof = false;
    std::vector<ProfRec> prof_pending;
    double prof_ms[PC_COUNT] = {};
    long long prof_n[PC_COUNT] = {};
    int prof_begin(int cat)
    {
        if (!prof) return -1;
        ProfRec r{cat, 0, nullptr, nullptr};
        cudaEventCreate(&r.a);
        cudaEventCreate(&r.b);
        cudaEventRecord(r.a, stream);
        prof_pending.push_back(r);
        return (int)prof_pending.size() - 1;
    }
    void prof_end(int h, int nlaunch)
    {
        if (h < 0) return;
        prof_pending[h].nlaunch = nlaunch;
        cudaEventRecord(prof_pending[h].b, stream);
    }
    void prof_collect()
    {
        cudaStreamSynchronize(stream);
        for (auto &r : prof_pending) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, r.a, r.b);
            prof_ms[r.cat] += ms;
            prof_n[r.cat] += r.nlaunch;
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        prof_pending.clear();
    }
    void prof_reset()
    {
        prof_collect();
        for (int c = 0; c < PC_COUNT; c++) { prof_ms[c] = 0; prof_n[c] = 0; }
    }
};

struct ProfScope {
    EngineBase *e;
    int h, n;
    ProfScope(EngineBase *eng, int cat, int nl) : e(eng), h(eng->prof_begin(cat)), n(nl) {}
    ~ProfScope() { e->prof_end(h, n); }
};

// ensemble of independent members advanced by batched kernels
struct EnsembleBase {
    virtual ~EnsembleBase() {}
    virtual int step(int nsteps) = 0;  // queues work, no final synchronize
    virtual int synchronize() = 0;
    virtual EngineBase *member(int m) = 0;
    virtual int size() const = 0;
    virtual void *stream_handle() = 0;
    virtual void mark_dirty() = 0;
    virtual int tune() = 0;
    std::string tuning;
    long long launches = 0;
};

// set by the engines, read by ga_last_error (thread local)
void set_error(const std::string &msg);

size_t noalloc_bytes_needed(const ga_config *c);
// GA_OK, or GA_ERR_ARG with the reason when the grid needs more scratch or
// shared memory per block than the allocation-free solve has
int noalloc_check(const ga_config *c, std::string *why);
int solve_pressure_noalloc(const ga_config *c, const ga_columns *cols, double *up, double *vp, double *wp,
                           double *pi, double step, cudaStream_t stream);

EnsembleBase *make_ensemble_f64(const ga_config *cfgs, const ga_columns *cols, int n, int *rc);
EnsembleBase *make_ensemble_f32(const ga_config *cfgs, const ga_columns *cols, int n, int *rc);

EngineBase *make_engine_f64(const ga_config *cfg, const ga_columns *cols, int *rc);
EngineBase *make_engine_f32(const ga_config *cfg, const ga_columns *cols, int *rc);

}  // namespace ga
