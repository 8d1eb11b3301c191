// ga_engine.h - precision-independent interface between the C ABI
// (ga_api.cu) and the per-precision engines (ga_f64.cu, ga_f32.cu).
#pragma once
#include <cuda_runtime.h>
#include <string>

#include "../../include/ga_anelastic.h"

namespace ga {

struct EngineBase {
    virtual ~EngineBase() {}
    virtual int set_field(int field, int slot, const double *host, size_t n) = 0;
    virtual int get_field(int field, int slot, double *host, size_t n) = 0;
    virtual int op(int op, double step) = 0;
    virtual int step(int nsteps) = 0;
    virtual int check_finite() = 0;
    virtual void *field_ptr(int field, int slot) = 0;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    long long bigcounter = 0;
    double mtime = 0.0;
    int device = 0;
};

// set by the engines, read by ga_last_error (thread local)
void set_error(const std::string &msg);

EngineBase *make_engine_f64(const ga_config *cfg, const ga_columns *cols, int *rc);
EngineBase *make_engine_f32(const ga_config *cfg, const ga_columns *cols, int *rc);

}  // namespace ga
