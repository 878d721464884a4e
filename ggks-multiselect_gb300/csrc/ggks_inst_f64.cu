// ggks_inst_f64.cu -- instantiation of the selection pipeline for one input type
// (split per type so the build compiles the units in parallel).
#include "ggks_pipeline.cuh"

namespace ggks {
template int select<double, double>(Context &, const double *, uint64_t, const ReqSource &, uint32_t,
                            double *, const double **, cudaStream_t, const double *);
// recursive levels run on the keys of oversized segments
template int select<uint64_t, double>(Context &, const uint64_t *, uint64_t, const ReqSource &, uint32_t,
                            double *, const double **, cudaStream_t, const uint64_t *);
}  // namespace ggks
