// ggks_batch_u32.cu -- instantiation of the batched selection for one element
// type (split per type so the build compiles the units in parallel).
#include "ggks_batch_host.cuh"

namespace ggks {
template int select_batch<uint32_t>(Context &, const BatchInput &, uint32_t *, uint32_t *, cudaStream_t,
                               const BatchTune &, float *);
}  // namespace ggks
