// FP32 engine: FP32 storage and arithmetic, with the near-singular low
// horizontal wavenumbers of the pressure solve in FP64.
#include "ga_ensemble.cuh"

namespace ga {
EngineBase *make_engine_f32(const ga_config *cfg, const ga_columns *cols, int *rc)
{
    return make_engine<float>(cfg, cols, rc);
}
EnsembleBase *make_ensemble_f32(const ga_config *cfgs, const ga_columns *cols, int n, int *rc)
{
    return make_ensemble<float>(cfgs, cols, n, rc);
}
}  // namespace ga
