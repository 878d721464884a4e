// ggks_internal.h -- host-side context and pipeline driver declarations.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>

#include "ggks.h"
#include "ggks_device.cuh"

namespace ggks {

// devices whose per-device launch settings (shared-memory limits, occupancy)
// are remembered; a larger device index is set up again on every call
constexpr int kMaxDevices = 64;

// Tunables of the batched path: bucket budget of a problem is about n / div
// buckets; tiles of the (problem, tile) queue hold `tile` elements.
struct BatchTune {
  uint32_t div = 256;
  uint32_t tile = 1u << 18;
};

// Orders the batched launches of several contexts (a server's lanes) on the
// device.  Under the mutex a launch makes its stream wait for the newest
// launch's kernel-done event, launches with the whole co-resident grid, and
// becomes the newest: the kernels run back to back with the whole device,
// and each lane's planning, uploads, result copies and scatter overlap the
// other lanes' kernels (a lane no longer waits on the host for another
// lane's grid share).
struct LaunchChain {
  std::mutex mu;
  cudaEvent_t last = nullptr;  // kernel-done event of the newest launch (its context's)
  uint64_t queued = 0;         // launches queued behind a kernel still in flight
};

// A context owns one device, one stream, a device arena (per-call scratch), a
// survivor buffer, a device staging buffer for host-vector inputs, pinned host
// staging, and a child context for recursive re-selection of oversized
// segments.
struct Context {
  int device = 0;
  int sm_count = 0;
  int smem_optin = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;

  char *arena = nullptr;  // [slice counts | out | ctrl | reqs | ... ]
  size_t arena_bytes = 0;
  void *surv = nullptr;
  size_t surv_bytes = 0;
  void *dvec = nullptr;
  size_t dvec_bytes = 0;
  char *pin = nullptr;
  size_t pin_bytes = 0;

  std::unique_ptr<Context> child;
  int depth = 0;

  // batched selection: device workspace, pinned staging, kernel events and
  // the autotuner's choices per batch shape
  char *barena = nullptr;
  size_t barena_bytes = 0;
  char *bpin = nullptr;
  size_t bpin_bytes = 0;
  cudaEvent_t bev0 = nullptr, bev1 = nullptr;
  std::map<uint64_t, BatchTune> tuned;
  BatchTune last_tune;
  BatchTune pinned_tune{0, 0};  // div != 0: used for every batch (no autotuning)
  LaunchChain *chain = nullptr;  // shared with other contexts' batched launches, if set
  // when set (a server's lanes), each batched launch's device interval in ms
  // after this event, read once the launch has finished
  cudaEvent_t time_base = nullptr;
  float last_launch_t0 = 0.f, last_launch_t1 = 0.f;
  // host clock when the last batched kernel was launched
  std::chrono::steady_clock::time_point last_launch_wall{};

  ggks_stats stats{};
  uint32_t profiling = 0;  // bit i: time pass i with CUDA events
  bool events_ready = false;
  cudaEvent_t ev0[GGKS_NUM_PASSES]{}, ev1[GGKS_NUM_PASSES]{};
  cudaEvent_t copy_done = nullptr;

  ~Context();
};

// status mapping
int from_cuda(cudaError_t e);

int context_init(Context &ctx, int device);
Context *default_context(int device, int *status);
Context *child_of(Context &ctx, int *status);

cudaError_t ensure_arena(Context &ctx, size_t bytes);
cudaError_t ensure_buffer(Context &ctx, char **p, size_t *have, size_t bytes);
cudaError_t ensure_pinned(Context &ctx, char **p, size_t *have, size_t bytes);
cudaError_t ensure_surv(Context &ctx, size_t bytes);
cudaError_t ensure_dvec(Context &ctx, size_t bytes);
cudaError_t ensure_pin(Context &ctx, size_t bytes);

// fixed-offset persistent state at the start of the arena: k_lut's
// per-slice sample counts, zero between calls
constexpr size_t kSliceCntBytes = kLutIdx * sizeof(uint32_t);

// Where the requests of one selection come from.
struct ReqSource {
  const uint32_t *h_k = nullptr;  // host k list (k-th largest): rank = n - k
  const Req *d_reqs = nullptr;    // device requests (recursive levels)
  bool topk = false;              // ranks n-1 .. n-K into outputs 0 .. K-1
  bool topk_pipeline = false;     // a top-k that does not take the threshold path
  bool no_small = false;          // never the one-launch small-vector path
};

// Run one selection.  Results land in d_out_user (device) or, when it is
// null, in the context's arena.  If host_results is not null the results are
// also copied to pinned host memory and *host_results points there (valid
// until the next call on the context).  The stream is synchronised.
// ingest: when not null, a host vector mapped into the device address space;
// the first passes read it and the histogram pass writes it to d_in (a device
// buffer with the same alignment modulo 16 bytes).
template <class InT, class OutT>
int select(Context &ctx, const InT *d_in, uint64_t n, const ReqSource &src, uint32_t num_req,
           OutT *d_out_user, const OutT **host_results, cudaStream_t s, const InT *ingest);

// One batch: problem p is vecs[p] (device, n[p] elements) with outputs
// [k_off[p], k_off[p + 1]); output j asks for the k[j]-th largest of its
// problem, or, when k is null, output k_off[p] + i is the (i + 1)-th largest
// (top-k).  k values are already checked to lie in [1, n[p]].
struct BatchInput {
  const void *const *vecs = nullptr;
  const uint64_t *n = nullptr;
  uint32_t num_problems = 0;
  const uint32_t *k_off = nullptr;
  const uint32_t *k = nullptr;
  // uint32 batches only, per problem (may be null): the vector holds float32
  // values, selected in float order, whose outputs are float32 bits (host
  // outputs only)
  const uint8_t *is_float = nullptr;
};

// Run one batch in one cooperative launch (plus re-runs on survivor overflow
// and a recursive re-selection of oversized segments).  Results go to
// d_out_user (device) when it is not null, else to the context's workspace;
// h_out (host), when not null, receives them too.  *kernel_ms: device time of
// the launches.  The stream is synchronised.
template <class T>
int select_batch(Context &ctx, const BatchInput &in, T *d_out_user, T *h_out, cudaStream_t s,
                 const BatchTune &tune, float *kernel_ms);

}  // namespace ggks
