// ggks_pipeline.cuh -- host driver of the selection pipeline (templated on the
// input element type and the output value type).  Included by the
// per-type instantiation units.
#pragma once

#include <algorithm>
#include <atomic>
#include <type_traits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ggks_internal.h"
#include "ggks_small.cuh"
#include "ggks_topk.cuh"

namespace ggks {

// keys of needed bins that one finishing CTA holds in shared memory (plus an
// equal scratch area for sorting a large bin)
template <class T>
static inline uint32_t cap_keys_for() {
  return sizeof(typename Traits<T>::K) == 4 ? 4096u : 2048u;
}
// bins (5 arrays), the gather buffer, a scratch half its size for sorting one
// large bin, per-bin key ranges: about 52 KB (f32) / 60 KB (f64), so that
// several finishing CTAs share an SM
template <class T>
static inline int finish_smem_bytes() {
  using K = typename Traits<T>::K;
  return (int)finish_smem_for<K>(cap_keys_for<T>());
}

static inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// k_plan's shared memory: the table, the bucket prefix and flags for the
// largest bucket count, and room for 6144 per-slot request counters (both
// launchers raise the kernel's limit to this one value)
constexpr size_t kPlanSlotBytes = 6144 * 8;
constexpr int kPlanSmemMax = (int)(kLutPadded * sizeof(uint32_t) + (size_t)kMaxNb * 5 + 16 +
                                   kPlanSlotBytes);

struct Plan {
  uint64_t n = 0;
  uint32_t num_req = 0;
  uint32_t S = 0, sample_grid = 0;
  uint32_t nb_max = 0;
  uint32_t G = 0;           // hist / compact grid
  bool unroll8 = true;      // tiles of 8 (else 4) vectors per thread in hist / compact
  uint32_t scan_tiles = 0;
  uint32_t cap_keys = 0;
  uint32_t fin_grid = 0;
  uint64_t surv_cap = 0;
  // arena offsets
  size_t out = 0, ctrl = 0, reqs = 0, hdr = 0, lut = 0, samples = 0, partials = 0,
         bpre = 0, ttot = 0, seg_bucket = 0, seg_off = 0, seg_size = 0, kstart = 0, kcnt = 0, fill = 0,
         kcur = 0, seg_lo = 0, seg_hi = 0, deferred = 0, req_bucket = 0, req_local = 0, klist = 0,
         pm_bits = 0, pm_bcount = 0, pm_bslot = 0, cand_cnt = 0, cand_tab = 0, reps = 0,
         bsingle = 0, bkey = 0, total = 0;
  // speculative compaction: the candidate pool is the survivor buffer from
  // surv_half on, cand_chunks chunks of kCandChunk keys
  uint64_t surv_half = 0;
  uint32_t cand_chunks = 0;
};
static_assert(sizeof(Ctrl) <= 256, "the control block travels in one 256-byte image");

template <class InT, class OutT>
static Plan make_plan(const Context &ctx, uint64_t n, uint32_t num_req) {
  using K = typename Traits<InT>::K;
  Plan p;
  p.n = n;
  p.num_req = num_req;
  p.S = n <= 65536 ? (uint32_t)n : 65536u;
  p.sample_grid = (p.S + 1023) / 1024;
  uint64_t want = n / 32;
  uint32_t nb = 8192;
  while (nb < kMaxNb && (uint64_t)nb * 2 <= want) nb *= 2;
  p.nb_max = nb;
  uint64_t g = (n + 65535) / 65536;
  p.G = (uint32_t)(g < 1 ? 1 : (g > (uint64_t)ctx.sm_count ? ctx.sm_count : g));
  p.scan_tiles = (p.nb_max + kScanTile - 1) / kScanTile;
  // Tiles of 8 vectors per thread stream a little faster than tiles of 4, but
  // the grid's last round of tiles is then coarser: keep 8 unless 4 spreads
  // the tiles over the CTAs better by more than 1 % (the busiest CTA's tiles
  // against the average).
  {
    const double nv = (double)(n * sizeof(InT) / 16);
    auto spread = [&](double tile_v) {
      const double t = std::floor(nv / tile_v);
      return t < 1 ? 1e9 : std::ceil(t / p.G) * p.G / t;
    };
    p.unroll8 = spread(8.0 * 1024) <= spread(4.0 * 1024) * 1.01;
  }
  p.cap_keys = cap_keys_for<InT>();
  uint32_t slots_bound = num_req < p.nb_max ? num_req : p.nb_max;
  uint32_t fg = 5u * (uint32_t)ctx.sm_count;
  p.fin_grid = slots_bound < fg ? (slots_bound ? slots_bound : 1) : fg;
  uint64_t cap = n / 8;
  cap = cap < (1u << 20) ? (1u << 20) : cap;
  if (cap > n) cap = n;
  // survivors below surv_half; from there the candidate pool, which also
  // holds one partly filled chunk per histogram warp
  p.surv_half = (cap / 2) & ~(uint64_t)3;  // 16-byte aligned pool
  p.surv_cap = cap + (uint64_t)p.G * kCandWarps * kCandChunk;
  const uint64_t chunks = (p.surv_cap - p.surv_half) / kCandChunk;
  p.cand_chunks = (uint32_t)(chunks < 0xFFFFFFFFull ? chunks : 0xFFFFFFFFull);

  const size_t A = 256;
  // the arena's head: per-slice sample counts of k_lut, zero between
  // calls (the arena starts zeroed; every call leaves them zero)
  size_t o = kSliceCntBytes;
  p.out = o;
  o = align_up(o + (size_t)num_req * sizeof(OutT), A);
  p.ctrl = o;
  o += A;  // ctrl is followed directly by the requests (one upload)
  p.reqs = o;
  o = align_up(o + (size_t)num_req * sizeof(Req), A);
  p.hdr = o;
  o = align_up(o + sizeof(LutHeader<K>), A);
  p.lut = o;
  o = align_up(o + kLutPadded * sizeof(uint32_t), A);
  p.samples = o;
  o = align_up(o + (size_t)p.S * sizeof(K), A);
  p.partials = o;
  o = align_up(o + (size_t)p.G * p.nb_max * sizeof(uint32_t), A);
  auto arr = [&](size_t &off, size_t elems, size_t esz) {
    off = o;
    o = align_up(o + elems * esz, A);
  };
  arr(p.bpre, p.nb_max, 4);
  arr(p.ttot, p.scan_tiles, 4);
  arr(p.seg_bucket, p.nb_max, 4);
  arr(p.seg_off, p.nb_max, 8);
  arr(p.seg_size, p.nb_max, 4);
  arr(p.kstart, p.nb_max, 4);
  arr(p.kcnt, p.nb_max, 4);
  arr(p.kcur, p.nb_max, 4);
  arr(p.fill, p.nb_max, 4);
  arr(p.seg_lo, p.nb_max, sizeof(K));
  arr(p.seg_hi, p.nb_max, sizeof(K));
  arr(p.deferred, p.nb_max, 4);
  arr(p.req_bucket, num_req, 4);
  arr(p.req_local, num_req, 4);
  arr(p.klist, num_req, sizeof(Req));
  // premapped plan (many requests): bucket bitmap and request counts, zeroed
  // together before each use, and the bucket -> slot map
  p.pm_bits = o;
  p.pm_bcount = o + (size_t)p.nb_max / 8;
  o = align_up(o + (size_t)p.nb_max / 8 + (size_t)p.nb_max * 4, A);
  arr(p.pm_bslot, p.nb_max, 4);
  arr(p.cand_cnt, (size_t)p.G * kCandWarps, 4);
  arr(p.cand_tab, (size_t)p.G * kCandWarps * kCandChunksPerWarp, 4);
  // single-key tracking of tables whose keys repeat often: each CTA's key per
  // bucket, and per bucket whether the vector holds one key there and which
  arr(p.reps, (size_t)p.G * p.nb_max, sizeof(K));
  arr(p.bsingle, p.nb_max, 4);
  arr(p.bkey, p.nb_max, sizeof(K));
  p.total = o;
  return p;
}

// Raise a kernel's dynamic shared-memory limit on the current device.  The
// attribute belongs to the kernel as loaded on one device, so it is set once
// per device (the largest value asked for so far is remembered per device);
// the result of the setting is returned for the caller to check.
template <auto F>
static cudaError_t set_smem_max(int bytes) {
  static std::atomic<int> set_to[kMaxDevices];  // static storage: starts at zero
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const bool tracked = dev >= 0 && dev < kMaxDevices;
  if (tracked && set_to[dev].load(std::memory_order_acquire) >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute((const void *)F, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && tracked) {
    int cur = set_to[dev].load(std::memory_order_acquire);
    while (cur < bytes && !set_to[dev].compare_exchange_weak(cur, bytes)) {
    }
  }
  return e;
}

// Launches a pipeline kernel with programmatic stream serialization: it may be
// scheduled while the previous kernel in the stream still runs, and waits for
// that kernel in its own first instructions (pdl_start).  The arguments are
// converted to the kernel's parameter types.
template <class... P, class... A>
static cudaError_t launch(void (*kern)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                          A &&...args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// Launches k_small as one cluster of kSmCtas CTAs, plainly (no programmatic
// serialization: it follows a copy).
template <class... P, class... A>
static cudaError_t launch_small(void (*kern)(P...), cudaStream_t s, A &&...args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kSmCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kSmCtas);
  cfg.blockDim = dim3(kSmThreads);
  cfg.dynamicSmemBytes = kSmBytes;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// Whether the current device can run k_small<InT, OutT> (once per device):
// its shared memory and the cluster size (16 CTAs, a non-portable size that
// must be allowed first) are set, and the occupancy calculator must find room
// for one such cluster.  false: the small-vector path is not used there.
template <class InT, class OutT>
static std::atomic<int> *small_state() {
  static std::atomic<int> state[kMaxDevices];  // 0 unknown, 1 ready, 2 unavailable
  return state;
}
template <class InT, class OutT>
static bool small_ready() {
  std::atomic<int> *state = small_state<InT, OutT>();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return false;
  const int st = state[dev].load(std::memory_order_acquire);
  if (st) return st == 1;
  auto kern = k_small<InT, OutT>;
  bool ok = cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kSmBytes) == cudaSuccess &&
            cudaFuncSetAttribute((const void *)kern,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  if (ok) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kSmCtas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kSmCtas);
    cfg.blockDim = dim3(kSmThreads);
    cfg.dynamicSmemBytes = kSmBytes;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    ok = cudaOccupancyMaxActiveClusters(&clusters, (const void *)kern, &cfg) == cudaSuccess &&
         clusters >= 1;
  }
  cudaGetLastError();  // a refused attribute or query leaves no error behind
  state[dev].store(ok ? 1 : 2, std::memory_order_release);
  return ok;
}

struct PassTimer {
  Context &ctx;
  cudaStream_t s;
  int pass;
  PassTimer(Context &c, cudaStream_t st, int p) : ctx(c), s(st), pass(p) {
    if (ctx.profiling & (1u << pass)) cudaEventRecord(ctx.ev0[pass], s);
  }
  ~PassTimer() {
    if (ctx.profiling & (1u << pass)) cudaEventRecord(ctx.ev1[pass], s);
    ctx.stats.launches++;
    ctx.stats.pass_launches[pass]++;
  }
};

static void collect_pass_times(Context &ctx, const bool *ran) {
  if (!ctx.profiling) return;
  for (int i = 0; i < GGKS_NUM_PASSES; ++i) {
    if (!ran[i] || !(ctx.profiling & (1u << i))) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx.ev0[i], ctx.ev1[i]) == cudaSuccess) ctx.stats.pass_ms[i] += ms;
  }
}

__global__ void k_make_topk_reqs(Req *reqs, uint64_t n, uint32_t K);

// Rank windows for speculative compaction: one window over all requested
// ranks, or, for up to 64 requests, two windows split at the widest gap
// between neighbouring ranks.  The table builder widens them by the sample's
// error and turns speculation off when they would keep too many elements;
// windows spanning more than n / 16 ranks are not sent at all.
static inline void set_windows_any(Ctrl *ci, const Req *hr, uint32_t num_req) {
  if (num_req == 0) return;
  if (num_req > 64) {
    uint32_t lo = hr[0].rank, hi = hr[0].rank;
    for (uint32_t i = 1; i < num_req; ++i) {
      lo = hr[i].rank < lo ? hr[i].rank : lo;
      hi = hr[i].rank > hi ? hr[i].rank : hi;
    }
    ci->spec_nwin = 1;
    ci->spec_lo[0] = lo;
    ci->spec_hi[0] = hi;
    return;
  }
  uint32_t r[64];
  for (uint32_t i = 0; i < num_req; ++i) r[i] = hr[i].rank;
  std::sort(r, r + num_req);
  uint32_t cut = 0, gap = 0;  // the second window starts at r[cut] (0: one window)
  for (uint32_t i = 1; i < num_req; ++i)
    if (r[i] - r[i - 1] > gap) {
      gap = r[i] - r[i - 1];
      cut = i;
    }
  if (gap <= 1) cut = 0;
  ci->spec_nwin = cut ? 2 : 1;
  ci->spec_lo[0] = r[0];
  ci->spec_hi[0] = cut ? r[cut - 1] : r[num_req - 1];
  if (cut) {
    ci->spec_lo[1] = r[cut];
    ci->spec_hi[1] = r[num_req - 1];
  }
}
static inline void set_windows(Ctrl *ci, const Req *hr, uint32_t num_req, uint64_t n) {
  set_windows_any(ci, hr, num_req);
  uint64_t span = 0;
  for (uint32_t w = 0; w < ci->spec_nwin; ++w) span += ci->spec_hi[w] - ci->spec_lo[w] + 1;
  if (span > n / 16) ci->spec_nwin = 0;
}

// Top-k by a sampled threshold (ggks_topk.cuh): k_sample, k_tau, k_filter,
// k_pick.  *missed: the candidates fell short (or did not fit), nothing is
// answered, and the caller runs the pipeline; d_in then holds the device copy
// of an ingested host vector.
template <class InT>
static int topk_threshold(Context &ctx, const InT *d_in, uint64_t n, uint32_t K, InT *d_out_user,
                          const InT **host_results, cudaStream_t s, const InT *ingest,
                          bool *missed) {
  using Kt = typename Traits<InT>::K;
  *missed = false;
  const Plan p = make_plan<InT, InT>(ctx, n, K);
  cudaError_t e = ensure_arena(ctx, p.total);
  if (e != cudaSuccess) return from_cuda(e);
  e = ensure_surv(ctx, (size_t)p.surv_cap * sizeof(Kt));
  if (e != cudaSuccess) return from_cuda(e);
  char *A = ctx.arena;
  Ctrl *ctrl = reinterpret_cast<Ctrl *>(A + p.ctrl);
  Kt *tau = reinterpret_cast<Kt *>(A + p.hdr);
  Kt *samples = reinterpret_cast<Kt *>(A + p.samples);
  uint32_t *slice_cnt = reinterpret_cast<uint32_t *>(A);
  Kt *arr = reinterpret_cast<Kt *>(ctx.surv);  // the candidate array
  const uint64_t arr_cap = p.surv_cap;
  InT *d_out = d_out_user ? d_out_user : reinterpret_cast<InT *>(A + p.out);
  const size_t out_span = p.ctrl - p.out;
  e = ensure_pin(ctx, 256 + out_span + 256);
  if (e != cudaSuccess) return from_cuda(e);
  char *pin_up = ctx.pin;
  char *pin_down = ctx.pin + 256;
  Ctrl *h_ctrl = reinterpret_cast<Ctrl *>(pin_down + out_span);
  std::memset(pin_up, 0, 256);  // a zeroed control block
  e = cudaMemcpyAsync(ctrl, pin_up, 256, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return from_cuda(e);
  cudaError_t le = cudaSuccess;
  auto L = [&le](cudaError_t r) {
    if (le == cudaSuccess) le = r;
  };
  const int pick_smem = (int)pick_smem_bytes<Kt>();
  const int filt_smem = (int)(kCandWarps * kFiltBuf * sizeof(Kt));
  L(set_smem_max<k_pick<Kt, InT>>(pick_smem));
  L(set_smem_max<k_filter<InT, 8>>(filt_smem));
  L(set_smem_max<k_filter<InT, 4>>(filt_smem));
  bool ran[GGKS_NUM_PASSES] = {false, false, false, false, false, false};
  {
    PassTimer t(ctx, s, GGKS_PASS_SAMPLE);
    L(launch(k_sample<InT>, p.sample_grid, 1024, 0, s, ingest ? ingest : d_in, n, p.S, 0x5EEDu,
             samples, ctrl));
    L(launch(k_tau<Kt>, p.sample_grid, 1024, 0, s, samples, p.S, ctrl, slice_cnt, n, K, tau));
    ctx.stats.launches++;
    ran[GGKS_PASS_SAMPLE] = true;
  }
  {
    PassTimer t(ctx, s, GGKS_PASS_HIST);
    L(launch(p.unroll8 ? k_filter<InT, 8> : k_filter<InT, 4>, p.G, 1024, filt_smem, s,
             ingest ? ingest : d_in, n, tau, arr, arr_cap, &ctrl->cand_next,
             ingest ? const_cast<InT *>(d_in) : nullptr, ctrl));
    ran[GGKS_PASS_HIST] = true;
  }
  {
    PassTimer t(ctx, s, GGKS_PASS_FINISH);
    L(launch(k_pick<Kt, InT>, 1, 1024, pick_smem, s, arr, arr_cap, &ctrl->cand_next, tau, K,
             d_out, ctrl));
    ran[GGKS_PASS_FINISH] = true;
  }
  e = le != cudaSuccess ? le : cudaGetLastError();
  if (e != cudaSuccess) return from_cuda(e);
  const bool want_host = host_results != nullptr;
  if (want_host && !d_out_user)
    e = cudaMemcpyAsync(pin_down, A + p.out, out_span + sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
  else
    e = cudaMemcpyAsync(h_ctrl, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && want_host && d_out_user)
    e = cudaMemcpyAsync(pin_down, d_out, (size_t)K * sizeof(InT), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return from_cuda(e);
  collect_pass_times(ctx, ran);
  const Ctrl c = *h_ctrl;
  if (c.status & ST_FATAL) return (c.status & ST_TIMEOUT) ? GGKS_TIMEOUT : GGKS_INTERNAL;
  if (c.status & ST_TOPK_MISS) {
    *missed = true;
    ctx.stats.topk_misses++;
    return GGKS_OK;
  }
  ctx.stats.topk_threshold_calls++;
  if (want_host) *host_results = reinterpret_cast<const InT *>(pin_down);
  return GGKS_OK;
}

// A small vector in one launch (ggks_small.cuh): host k lists or a top-k of
// at most kSmMaxReq requests on a device vector of at most kSmMaxN
// (kSmMaxTopkN for a top-k) elements.
// *missed: the kernel met a case it leaves to the pipeline (nothing is
// answered; the caller runs the pipeline, which writes every output again).
// Arena: [slice counts | out | ctrl | requests]: the control block and the
// requests go up in one copy, the outputs and the control block come back in
// one.
template <class InT, class OutT>
static int select_small(Context &ctx, const InT *d_in, uint64_t n, const ReqSource &src,
                        uint32_t num_req, OutT *d_out_user, const OutT **host_results,
                        cudaStream_t s, bool *missed) {
  using K = typename Traits<InT>::K;
  *missed = false;
  if (!small_ready<InT, OutT>()) {
    *missed = true;
    return GGKS_OK;
  }
  const size_t out_span = align_up((size_t)num_req * sizeof(OutT), 256);
  const size_t o_out = kSliceCntBytes, o_ctrl = o_out + out_span, o_reqs = o_ctrl + 256;
  const size_t o_chk = align_up(o_reqs + (size_t)num_req * sizeof(Req), 256);
  const size_t up_bytes = 256 + (size_t)num_req * sizeof(Req);
  cudaError_t e = ensure_arena(ctx, o_chk + (size_t)kSmNb * kSmCtas * sizeof(uint32_t));
  if (e == cudaSuccess) e = ensure_surv(ctx, (size_t)n * sizeof(K));
  const size_t down_off = align_up(up_bytes, 256);
  if (e == cudaSuccess) e = ensure_pin(ctx, down_off + out_span + 256);
  if (e != cudaSuccess) return from_cuda(e);
  char *A = ctx.arena;
  Ctrl *ctrl = reinterpret_cast<Ctrl *>(A + o_ctrl);
  OutT *d_out = d_out_user ? d_out_user : reinterpret_cast<OutT *>(A + o_out);
  char *pin_up = ctx.pin;
  char *pin_down = ctx.pin + down_off;
  Ctrl *h_ctrl = reinterpret_cast<Ctrl *>(pin_down + out_span);
  // every call ends with a stream synchronisation: no earlier copy still
  // reads the pinned buffer
  std::memset(pin_up, 0, 256);
  Req *hr = reinterpret_cast<Req *>(pin_up + 256);
  for (uint32_t i = 0; i < num_req; ++i) {
    hr[i].rank = src.topk ? (uint32_t)(n - 1 - i) : (uint32_t)(n - src.h_k[i]);
    hr[i].out = i;
  }
  e = cudaMemcpyAsync(ctrl, pin_up, up_bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return from_cuda(e);
  {
    PassTimer t(ctx, s, GGKS_PASS_SAMPLE);
    e = launch_small(k_small<InT, OutT>, s, d_in, n, reinterpret_cast<const Req *>(A + o_reqs),
                     num_req, d_out, reinterpret_cast<K *>(ctx.surv), ctx.surv_bytes / sizeof(K),
                     reinterpret_cast<uint32_t *>(A + o_chk), ctrl);
  }
  if (e != cudaSuccess) {
    // a cluster launch the device refuses (its SMs held by other work in a
    // way the occupancy query did not foresee): the pipeline runs instead,
    // and this device no longer tries the small path
    cudaGetLastError();
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices)
      small_state<InT, OutT>()[dev].store(2, std::memory_order_release);
    e = cudaStreamSynchronize(s);  // the uploaded requests are no longer needed
    if (e != cudaSuccess) return from_cuda(e);
    *missed = true;
    return GGKS_OK;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return from_cuda(e);
  const bool want_host = host_results != nullptr;
  if (want_host && !d_out_user)
    e = cudaMemcpyAsync(pin_down, A + o_out, out_span + sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
  else
    e = cudaMemcpyAsync(h_ctrl, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && want_host && d_out_user)
    e = cudaMemcpyAsync(pin_down, d_out, (size_t)num_req * sizeof(OutT), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return from_cuda(e);
  bool ran[GGKS_NUM_PASSES] = {true, false, false, false, false, false};
  collect_pass_times(ctx, ran);
#ifdef GGKS_SMALL_TIMING
  fprintf(stderr, "ggks small timing n=%llu req=%u:", (unsigned long long)n, num_req);
  // stamp order: 0 start, 1 sampled, 2 table, 3 histograms, 8 totals, 9 scan,
  // 10 barrier, 11 prefix, 12 requests, 13 cursors, 4 barrier, 5 compacted,
  // 6 checked, 7 finished
  static const int order[14] = {0, 1, 2, 3, 8, 9, 10, 11, 12, 13, 4, 5, 6, 7};
  for (int i = 1; i < 14; ++i)
    fprintf(stderr, " %.2f",
            (double)(h_ctrl->t_ns[order[i]] - h_ctrl->t_ns[order[i - 1]]) * 1e-3);
  fprintf(stderr, " us; first CTA start %.2f us before CTA 0, last CTA end %.2f us after\n",
          (double)(h_ctrl->t_ns[0] - ~h_ctrl->t_ns[14]) * 1e-3,
          (double)(h_ctrl->t_ns[15] - h_ctrl->t_ns[7]) * 1e-3);
#endif
  if (h_ctrl->status & ST_SMALL_MISS) {
    *missed = true;
    ctx.stats.small_misses++;
    return GGKS_OK;
  }
  if (h_ctrl->status & ST_FATAL) return (h_ctrl->status & ST_TIMEOUT) ? GGKS_TIMEOUT : GGKS_INTERNAL;
  ctx.stats.small_calls++;
  if (want_host) *host_results = reinterpret_cast<const OutT *>(pin_down);
  return GGKS_OK;
}

template <class InT, class OutT>
int select(Context &ctx, const InT *d_in, uint64_t n, const ReqSource &src, uint32_t num_req,
           OutT *d_out_user, const OutT **host_results, cudaStream_t s, const InT *ingest) {
  using K = typename Traits<InT>::K;
  if (ctx.depth > 12) return GGKS_INTERNAL;
  // a small device vector with host k's or a top-k: one launch, unless that
  // kernel leaves the case to the pipeline
  if constexpr (std::is_same<InT, OutT>::value) {
    if (ctx.depth == 0 && !ingest && !src.no_small && (src.h_k || src.topk) && num_req >= 1 &&
        num_req <= kSmMaxReq && n <= (src.topk ? kSmMaxTopkN : kSmMaxN)) {
      bool missed = false;
      const int st = select_small<InT, OutT>(ctx, d_in, n, src, num_req, d_out_user,
                                             host_results, s, &missed);
      if (st != GGKS_OK || !missed) return st;
    }
  }
  // a top-k of at most kPickMax values from a vector larger than the sample:
  // the threshold path, unless its candidates fall short
  if constexpr (std::is_same<InT, OutT>::value) {
    if (src.topk && ctx.depth == 0 && num_req <= kPickMax && n > 65536 &&
        (uint64_t)num_req * 64 <= n && !src.topk_pipeline) {
      bool missed = false;
      const int st = topk_threshold<InT>(ctx, d_in, n, num_req, d_out_user, host_results, s,
                                         ingest, &missed);
      if (st != GGKS_OK || !missed) return st;
      ingest = nullptr;  // the filter pass wrote the device copy
    }
  }
  const Plan p = make_plan<InT, OutT>(ctx, n, num_req);
  cudaError_t e = ensure_arena(ctx, p.total);
  if (e != cudaSuccess) return from_cuda(e);
  e = ensure_surv(ctx, (size_t)p.surv_cap * sizeof(K));
  if (e != cudaSuccess) return from_cuda(e);
  char *A = ctx.arena;
  Ctrl *ctrl = reinterpret_cast<Ctrl *>(A + p.ctrl);
  Req *reqs = reinterpret_cast<Req *>(A + p.reqs);
  LutHeader<K> *hdr = reinterpret_cast<LutHeader<K> *>(A + p.hdr);
  uint32_t *lut = reinterpret_cast<uint32_t *>(A + p.lut);
  K *samples = reinterpret_cast<K *>(A + p.samples);
  uint32_t *slice_cnt = reinterpret_cast<uint32_t *>(A);
  uint32_t *partials = reinterpret_cast<uint32_t *>(A + p.partials);
  uint32_t *bpre = reinterpret_cast<uint32_t *>(A + p.bpre);  // prefix inside 64-bucket tiles
  uint32_t *ttot = reinterpret_cast<uint32_t *>(A + p.ttot);  // the tiles' totals
  uint32_t *seg_bucket = reinterpret_cast<uint32_t *>(A + p.seg_bucket);
  uint64_t *seg_off = reinterpret_cast<uint64_t *>(A + p.seg_off);
  uint32_t *seg_size = reinterpret_cast<uint32_t *>(A + p.seg_size);
  uint32_t *kstart = reinterpret_cast<uint32_t *>(A + p.kstart);
  uint32_t *kcnt = reinterpret_cast<uint32_t *>(A + p.kcnt);
  uint32_t *kcur = reinterpret_cast<uint32_t *>(A + p.kcur);
  uint32_t *fill = reinterpret_cast<uint32_t *>(A + p.fill);
  K *seg_lo = reinterpret_cast<K *>(A + p.seg_lo);
  K *seg_hi = reinterpret_cast<K *>(A + p.seg_hi);
  uint32_t *deferred = reinterpret_cast<uint32_t *>(A + p.deferred);
  uint32_t *req_bucket = reinterpret_cast<uint32_t *>(A + p.req_bucket);
  uint32_t *req_local = reinterpret_cast<uint32_t *>(A + p.req_local);
  Req *klist = reinterpret_cast<Req *>(A + p.klist);
  K *surv = reinterpret_cast<K *>(ctx.surv);
  K *cand = surv + p.surv_half;
  uint32_t *cand_cnt = reinterpret_cast<uint32_t *>(A + p.cand_cnt);
  uint32_t *cand_tab = reinterpret_cast<uint32_t *>(A + p.cand_tab);
  K *reps = reinterpret_cast<K *>(A + p.reps);
  uint32_t *bsingle = reinterpret_cast<uint32_t *>(A + p.bsingle);
  K *bkey = reinterpret_cast<K *>(A + p.bkey);
  OutT *d_out = d_out_user ? d_out_user : reinterpret_cast<OutT *>(A + p.out);
  const bool out_in_arena = d_out_user == nullptr;

  // pinned staging: [ctrl image | host requests] up, [out | pad | ctrl] down
  const size_t up_bytes = 256 + (src.h_k ? (size_t)num_req * sizeof(Req) : 0);
  const size_t out_span = p.ctrl - p.out;  // == align_up(num_req * sizeof(OutT), 256)
  const size_t down_off = align_up(up_bytes, 256);
  e = ensure_pin(ctx, down_off + out_span + 256);
  if (e != cudaSuccess) return from_cuda(e);
  char *pin_up = ctx.pin;
  char *pin_down = ctx.pin + down_off;
  Ctrl *h_ctrl = reinterpret_cast<Ctrl *>(pin_down + out_span);
  // every call ends with a stream synchronisation, so no earlier copy still
  // reads the pinned buffer here
  std::memset(pin_up, 0, 256);
  Ctrl *ci = reinterpret_cast<Ctrl *>(pin_up);
  if (src.h_k) {
    Req *hr = reinterpret_cast<Req *>(pin_up + 256);
    for (uint32_t i = 0; i < num_req; ++i) {
      hr[i].rank = (uint32_t)(n - src.h_k[i]);
      hr[i].out = i;
    }
    set_windows(ci, hr, num_req, n);
  } else if (src.topk && num_req && (uint64_t)num_req <= n / 16) {
    ci->spec_nwin = 1;
    ci->spec_lo[0] = n - num_req;
    ci->spec_hi[0] = n - 1;
  }
  e = cudaMemcpyAsync(ctrl, pin_up, up_bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return from_cuda(e);
  const Req *rq = src.d_reqs ? src.d_reqs : reqs;
  bool ran[GGKS_NUM_PASSES] = {false, false, false, false, false, false};
  cudaError_t le = cudaSuccess;  // the first failed launch
  auto L = [&le](cudaError_t r) {
    if (le == cudaSuccess) le = r;
  };
  if (src.topk) {
    L(launch(k_make_topk_reqs, (num_req + 255) / 256, 256, 0, s, reqs, n, num_req));
    ctx.stats.launches++;
  }

  // ---- (b) sample + splitter table
  {
    PassTimer t(ctx, s, GGKS_PASS_SAMPLE);
    L(launch(k_sample<InT>, p.sample_grid, 1024, 0, s, ingest ? ingest : d_in, n, p.S, 0x5EEDu,
             samples, ctrl));
    L(launch(k_lut<K>, p.sample_grid, 1024, 0, s, samples, p.S, ctrl, hdr, lut, p.nb_max,
             slice_cnt, n, p.cand_chunks, p.G));
    ctx.stats.launches++;
    ran[GGKS_PASS_SAMPLE] = true;
  }
  // ---- (c) histogram
  {
    const int smem = (int)(kRepWords * sizeof(uint32_t) + (size_t)p.nb_max * 4);
    L(set_smem_max<k_hist<InT, 8>>((int)(kRepWords * sizeof(uint32_t) + (size_t)kMaxNb * 4)));
    L(set_smem_max<k_hist<InT, 4>>((int)(kRepWords * sizeof(uint32_t) + (size_t)kMaxNb * 4)));
    PassTimer t(ctx, s, GGKS_PASS_HIST);
    // with a mapped host vector, this pass also writes the device copy d_in
    L(launch(p.unroll8 ? k_hist<InT, 8> : k_hist<InT, 4>, p.G, 1024, smem, s, ingest ? ingest : d_in, n, hdr, lut, partials,
             p.nb_max, ctrl, ingest ? const_cast<InT *>(d_in) : nullptr, cand, cand_cnt, cand_tab,
             &ctrl->cand_next, reps));
    ran[GGKS_PASS_HIST] = true;
  }
  // ---- (d) reduce + decoupled look-back scan
  {
    PassTimer t(ctx, s, GGKS_PASS_SCAN);
    L(launch(k_colsum<K>, p.scan_tiles, kScanThreads, 0, s, partials, p.G, p.nb_max, hdr, bpre,
             ttot, ctrl, reps, bsingle, bkey));
    ran[GGKS_PASS_SCAN] = true;
  }
  // ---- (e) plan
  {
    // per-slot request counters in shared memory unless the requests are premapped
    const int smem = (int)(align_up(kLutPadded * sizeof(uint32_t) + (size_t)p.nb_max * 5, 16) +
                           (num_req < kPremapMin ? kPlanSlotBytes : 0));
    L(set_smem_max<k_plan<InT, OutT>>(kPlanSmemMax));
    PassTimer t(ctx, s, GGKS_PASS_PLAN);
    Premap pm;
    const bool premap = num_req >= kPremapMin;
    uint32_t *pm_bits = reinterpret_cast<uint32_t *>(A + p.pm_bits);
    uint32_t *pm_bcount = reinterpret_cast<uint32_t *>(A + p.pm_bcount);
    uint32_t *pm_bslot = reinterpret_cast<uint32_t *>(A + p.pm_bslot);
    if (premap) {
      // many requests: map them with many CTAs (k_reqmap), place them with
      // many CTAs (k_reqplace); the plan CTA only numbers the slots
      e = cudaMemsetAsync(pm_bits, 0, (size_t)p.nb_max / 8 + (size_t)p.nb_max * 4, s);
      if (e != cudaSuccess) return from_cuda(e);
      L(set_smem_max<k_reqmap>((int)(kMaxNb * 4)));
      L(launch(k_reqmap, (num_req + kReqmapPerCta - 1) / kReqmapPerCta, 1024, p.nb_max * 4, s,
               bpre, ttot, ctrl, rq, num_req, req_bucket, req_local, pm_bits, pm_bcount));
      pm.bits = pm_bits;
      pm.bcount = pm_bcount;
      pm.bslot = pm_bslot;
    }
    L(launch(k_plan<InT, OutT>, 1, 1024, smem, s, hdr, lut, bpre, ttot, n, rq, num_req, p.nb_max,
             ctrl, seg_bucket, seg_off, seg_size, kstart, kcnt, kcur, fill, seg_lo, seg_hi,
             req_bucket, req_local, klist, p.surv_cap, pm, bsingle, bkey));
    if (premap) {
      L(launch(k_reqplace, (num_req + 1023) / 1024, 1024, 0, s, ctrl, rq, num_req, req_bucket,
               req_local, pm_bslot, kstart, kcur, klist));
      ctx.stats.launches += 2;
    }
    ran[GGKS_PASS_PLAN] = true;
  }
  uint64_t surv_cap = p.surv_cap;
  const K *cand_live = cand;  // no candidates once the survivor buffer is replaced
  auto launch_tail = [&]() {
    {
      const int smem = (int)compact_smem_bytes(p.nb_max);
      L(set_smem_max<k_compact<InT, 8>>((int)compact_smem_bytes(kMaxNb)));
      L(set_smem_max<k_compact<InT, 4>>((int)compact_smem_bytes(kMaxNb)));
      PassTimer t(ctx, s, GGKS_PASS_COMPACT);
      L(launch(p.unroll8 ? k_compact<InT, 8> : k_compact<InT, 4>, p.G, 1024, smem, s, d_in, n, hdr, lut, seg_bucket, seg_off,
               seg_size, partials, fill, p.nb_max, surv, surv_cap, ctrl, cand_live, cand_cnt,
               cand_tab, p.surv_half));
      ran[GGKS_PASS_COMPACT] = true;
    }
    {
      const int smem = finish_smem_bytes<InT>();
      L(set_smem_max<k_finish<K, OutT>>(smem));
      PassTimer t(ctx, s, GGKS_PASS_FINISH);
      L(launch(k_finish<K, OutT>, p.fin_grid, kFinThreads, smem, s, surv, ctrl, seg_off, seg_size,
               seg_lo, seg_hi, kstart, kcnt, klist, deferred, p.cap_keys, d_out));
      ran[GGKS_PASS_FINISH] = true;
    }
  };
  launch_tail();
  e = le != cudaSuccess ? le : cudaGetLastError();
  if (e != cudaSuccess) return from_cuda(e);

  // results and control block come back in one copy when the output is ours
  auto pull = [&](bool with_out) -> cudaError_t {
    cudaError_t r;
    if (with_out && out_in_arena)
      r = cudaMemcpyAsync(pin_down, A + p.out, out_span + sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
    else
      r = cudaMemcpyAsync(h_ctrl, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
    if (r == cudaSuccess && with_out && !out_in_arena)
      r = cudaMemcpyAsync(pin_down, d_out, (size_t)num_req * sizeof(OutT), cudaMemcpyDeviceToHost, s);
    if (r != cudaSuccess) return r;
    return cudaStreamSynchronize(s);
  };
  const bool want_host = host_results != nullptr;
  e = pull(want_host);
  if (e != cudaSuccess) return from_cuda(e);
  collect_pass_times(ctx, ran);

  for (int round = 0; round < 4; ++round) {
    const Ctrl c = *h_ctrl;
    if (c.status & ST_FATAL) {
      // a stopped call may leave slice counts behind
      cudaMemsetAsync(slice_cnt, 0, kSliceCntBytes, s);
      cudaStreamSynchronize(s);
      return (c.status & ST_TIMEOUT) ? GGKS_TIMEOUT : GGKS_INTERNAL;
    }
    if (c.status & ST_OVERFLOW) {
      // survivors did not fit: grow the buffer, re-run compaction + finish
      const uint64_t need = c.cap_needed + (c.cap_needed >> 3);
      e = ensure_surv(ctx, (size_t)need * sizeof(K));
      if (e != cudaSuccess) return from_cuda(e);
      surv = reinterpret_cast<K *>(ctx.surv);
      surv_cap = need;
      cand_live = nullptr;
      ctx.stats.retries++;
      e = cudaMemsetAsync(&ctrl->status, 0, sizeof(uint32_t), s);
      if (e != cudaSuccess) return from_cuda(e);
      for (int i = 0; i < GGKS_NUM_PASSES; ++i) ran[i] = false;
      launch_tail();
      if (le != cudaSuccess) return from_cuda(le);
      e = pull(want_host);
      if (e != cudaSuccess) return from_cuda(e);
      collect_pass_times(ctx, ran);
      continue;
    }
    if (c.status & ST_DEFERRED) {
      // oversized segments: select each again, recursively, on its keys
      const uint32_t D = c.deferred_count, ns = c.num_slots;
      std::vector<uint32_t> dl(D), sz(ns), ks(ns), kc(ns);
      std::vector<uint64_t> so(ns);
      e = cudaMemcpyAsync(dl.data(), deferred, D * 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(sz.data(), seg_size, ns * 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(so.data(), seg_off, ns * 8, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(ks.data(), kstart, ns * 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(kc.data(), kcnt, ns * 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return from_cuda(e);
      int st = GGKS_OK;
      Context *ch = child_of(ctx, &st);
      if (!ch) return st;
      for (uint32_t d = 0; d < D; ++d) {
        const uint32_t slot = dl[d];
        ReqSource cs;
        cs.d_reqs = klist + ks[slot];
        ctx.stats.recursions++;
        st = select<K, OutT>(*ch, surv + so[slot], sz[slot], cs, kc[slot], d_out, nullptr, s,
                             nullptr);
        if (st != GGKS_OK) return st;
      }
      if (want_host) {
        e = pull(true);
        if (e != cudaSuccess) return from_cuda(e);
      }
    }
    break;
  }
  ctx.stats.survivors += h_ctrl->total_surv;
  ctx.stats.spec_calls += h_ctrl->spec_on;
  ctx.stats.spec_ctas += h_ctrl->spec_ctas;
  if (want_host) *host_results = reinterpret_cast<const OutT *>(pin_down);
  return GGKS_OK;
}

}  // namespace ggks
