// ggks_batch_f64.cu -- instantiation of the batched selection for one element
// type (split per type so the build compiles the units in parallel).
#include "ggks_batch_host.cuh"

namespace ggks {
template int select_batch<double>(Context &, const BatchInput &, double *, double *, cudaStream_t,
                               const BatchTune &, float *);
}  // namespace ggks
