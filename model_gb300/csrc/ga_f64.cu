// FP64 engine: the parity path.  Compiled with --fmad=false so that no
// multiply-add is contracted and every expression rounds as the reference's.
#include "ga_ensemble.cuh"

namespace ga {
EngineBase *make_engine_f64(const ga_config *cfg, const ga_columns *cols, int *rc)
{
    return make_engine<double>(cfg, cols, rc);
}
EnsembleBase *make_ensemble_f64(const ga_config *cfgs, const ga_columns *cols, int n, int *rc)
{
    return make_ensemble<double>(cfgs, cols, n, rc);
}
}  // namespace ga
