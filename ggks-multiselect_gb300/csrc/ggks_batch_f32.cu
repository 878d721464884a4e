// ggks_batch_f32.cu -- instantiation of the batched selection for one element
// type (split per type so the build compiles the units in parallel).
#include "ggks_batch_host.cuh"

namespace ggks {
template int select_batch<float>(Context &, const BatchInput &, float *, float *, cudaStream_t,
                               const BatchTune &, float *);
}  // namespace ggks
