// FP32 engine: FP32 storage and arithmetic, with the near-singular low
// horizontal wavenumbers of the pressure solve in FP64.
#include "ga_engine.cuh"

namespace ga {
EngineBase *make_engine_f32(const ga_config *cfg, const ga_columns *cols, int *rc)
{
    return make_engine<float>(cfg, cols, rc);
}
}  // namespace ga
