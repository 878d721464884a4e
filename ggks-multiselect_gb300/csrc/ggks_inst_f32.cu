// ggks_inst_f32.cu -- instantiation of the selection pipeline for one input type
// (split per type so the build compiles the units in parallel).
#include "ggks_pipeline.cuh"

namespace ggks {
template int select<float, float>(Context &, const float *, uint64_t, const ReqSource &, uint32_t,
                            float *, const float **, cudaStream_t, const float *);
// recursive levels run on the keys of oversized segments
template int select<uint32_t, float>(Context &, const uint32_t *, uint64_t, const ReqSource &, uint32_t,
                            float *, const float **, cudaStream_t, const uint32_t *);
}  // namespace ggks
