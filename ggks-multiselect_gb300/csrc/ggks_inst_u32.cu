// ggks_inst_u32.cu -- instantiation of the selection pipeline for one input type
// (split per type so the build compiles the units in parallel).
#include "ggks_pipeline.cuh"

namespace ggks {
template int select<uint32_t, uint32_t>(Context &, const uint32_t *, uint64_t, const ReqSource &, uint32_t,
                            uint32_t *, const uint32_t **, cudaStream_t, const uint32_t *);
}  // namespace ggks
