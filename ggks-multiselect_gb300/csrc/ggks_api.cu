// ggks_api.cu -- contexts, workspace management and the extern "C" entry
// points declared in include/ggks.h.
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "ggks_internal.h"

namespace ggks {

// ---------------------------------------------------------------------------
// small kernels owned by this unit
// ---------------------------------------------------------------------------
// top-k requests: output i receives the (i+1)-th largest, i.e. ascending rank
// n-1-i (multiselectTimingFunctions.cu:207-209 builds k = 1..K for this)
__global__ void k_make_topk_reqs(Req *reqs, uint64_t n, uint32_t K) {
  pdl_start();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < K) {
    Req r;
    r.rank = (uint32_t)(n - 1 - i);
    r.out = i;
    reqs[i] = r;
  }
}

// ---------------------------------------------------------------------------
// context and workspace
// ---------------------------------------------------------------------------
int from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return GGKS_OK;
  if (e == cudaErrorMemoryAllocation) return GGKS_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GGKS_NO_DEVICE;
  return GGKS_CUDA_ERROR;
}

Context::~Context() {
  int cur = -1;
  cudaGetDevice(&cur);
  cudaSetDevice(device);
  child.reset();
  if (stream) cudaStreamSynchronize(stream);
  if (arena) cudaFree(arena);
  if (surv) cudaFree(surv);
  if (dvec) cudaFree(dvec);
  if (pin) cudaFreeHost(pin);
  if (barena) cudaFree(barena);
  if (bpin) cudaFreeHost(bpin);
  if (bev0) cudaEventDestroy(bev0);
  if (bev1) cudaEventDestroy(bev1);
  if (events_ready) {
    for (int i = 0; i < GGKS_NUM_PASSES; ++i) {
      cudaEventDestroy(ev0[i]);
      cudaEventDestroy(ev1[i]);
    }
  }
  if (copy_done) cudaEventDestroy(copy_done);
  if (stream && depth == 0) cudaStreamDestroy(stream);
  if (cur >= 0) cudaSetDevice(cur);
}

int context_init(Context &ctx, int device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return GGKS_NO_DEVICE;
  if (device < 0 || device >= count) return GGKS_INVALID_ARG;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return from_cuda(e);
  ctx.device = device;
  e = cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&ctx.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx.copy_done, cudaEventDisableTiming);
  return from_cuda(e);
}

// zero: clear the new buffer on `stream` (the stream that uses it), so that
// the clearing is ordered before that stream's work; a plain cudaMemset would
// go to the legacy default stream, which a non-blocking stream does not wait
// for, and could land in the middle of a call while other work keeps the
// default stream busy.
static cudaError_t grow(void **p, size_t *have, size_t need, bool zero,
                        cudaStream_t stream = nullptr) {
  if (need <= *have && *p) return cudaSuccess;
  size_t want = need + need / 4 + 4096;
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
  }
  cudaError_t e = cudaMalloc(p, want);
  if (e != cudaSuccess) {
    *p = nullptr;
    return e;
  }
  *have = want;
  if (zero) e = cudaMemsetAsync(*p, 0, want, stream);
  return e;
}

cudaError_t ensure_arena(Context &ctx, size_t bytes) {
  // the arena's head holds state that must start zeroed (slice counts)
  if (bytes <= ctx.arena_bytes && ctx.arena) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(ctx.stream);
  if (e != cudaSuccess) return e;
  void *p = ctx.arena;
  e = grow(&p, &ctx.arena_bytes, bytes, true, ctx.stream);
  ctx.arena = static_cast<char *>(p);
  return e;
}

cudaError_t ensure_buffer(Context &ctx, char **p, size_t *have, size_t bytes) {
  if (bytes <= *have && *p) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(ctx.stream);
  if (e != cudaSuccess) return e;
  void *v = *p;
  e = grow(&v, have, bytes, false);
  *p = static_cast<char *>(v);
  return e;
}

cudaError_t ensure_pinned(Context &ctx, char **p, size_t *have, size_t bytes) {
  (void)ctx;
  if (bytes <= *have && *p) return cudaSuccess;
  if (*p) {
    cudaFreeHost(*p);
    *p = nullptr;
    *have = 0;
  }
  size_t want = bytes + bytes / 4 + 4096;
  void *v = nullptr;
  cudaError_t e = cudaHostAlloc(&v, want, cudaHostAllocDefault);
  if (e != cudaSuccess) return e;
  *p = static_cast<char *>(v);
  *have = want;
  return cudaSuccess;
}

cudaError_t ensure_surv(Context &ctx, size_t bytes) {
  if (bytes <= ctx.surv_bytes && ctx.surv) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(ctx.stream);
  if (e != cudaSuccess) return e;
  return grow(&ctx.surv, &ctx.surv_bytes, bytes, false);
}

cudaError_t ensure_dvec(Context &ctx, size_t bytes) {
  if (bytes <= ctx.dvec_bytes && ctx.dvec) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(ctx.stream);
  if (e != cudaSuccess) return e;
  return grow(&ctx.dvec, &ctx.dvec_bytes, bytes, false);
}

cudaError_t ensure_pin(Context &ctx, size_t bytes) {
  if (bytes <= ctx.pin_bytes && ctx.pin) return cudaSuccess;
  if (ctx.pin) {
    cudaFreeHost(ctx.pin);
    ctx.pin = nullptr;
    ctx.pin_bytes = 0;
  }
  size_t want = bytes + bytes / 4 + 4096;
  void *p = nullptr;
  cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
  if (e != cudaSuccess) return e;
  ctx.pin = static_cast<char *>(p);
  ctx.pin_bytes = want;
  return cudaSuccess;
}

Context *child_of(Context &ctx, int *status) {
  if (!ctx.child) {
    std::unique_ptr<Context> c(new Context());
    c->device = ctx.device;
    c->sm_count = ctx.sm_count;
    c->smem_optin = ctx.smem_optin;
    c->stream = ctx.stream;  // borrowed: not destroyed by the child
    c->depth = ctx.depth + 1;
    ctx.child = std::move(c);
  }
  *status = GGKS_OK;
  return ctx.child.get();
}

static std::mutex g_default_mu;
static Context *g_default[64];

Context *default_context(int device, int *status) {
  if (device < 0 || device >= 64) {
    *status = GGKS_INVALID_ARG;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default[device]) {
    // default contexts live until process exit (never destroyed: tearing
    // down CUDA state from a static destructor is unsafe)
    Context *c = new Context();
    int st = context_init(*c, device);
    if (st != GGKS_OK) {
      c->stream = nullptr;
      delete c;
      *status = st;
      return nullptr;
    }
    g_default[device] = c;
  }
  *status = GGKS_OK;
  return g_default[device];
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

static Context *resolve(const ggks_opts *opts, int *status) {
  if (opts && opts->ctx) {
    *status = GGKS_OK;
    return reinterpret_cast<Context *>(opts->ctx);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *status = GGKS_NO_DEVICE;
    return nullptr;
  }
  return default_context(dev, status);
}

// ---------------------------------------------------------------------------
// host vectors
// ---------------------------------------------------------------------------
// A pinned (page-locked, mapped) host vector is read by the kernels directly
// over the CPU-GPU link: the histogram pass ingests it and writes the device
// copy in the same pass, so the copy overlaps the first pass.  Any other host
// memory is copied to the device first.  The device copy keeps the host
// vector's alignment modulo 16 bytes, so both are split into the same
// 16-byte vectors.
template <class T>
static int stage_host_vector(Context &ctx, const T *vec, uint64_t n, cudaStream_t s,
                             const T **d_in, const T **ingest) {
  cudaError_t e = ensure_dvec(ctx, n * sizeof(T) + 16);
  if (e != cudaSuccess) return from_cuda(e);
  const uintptr_t mis = (uintptr_t)vec & 15u;
  T *dst = reinterpret_cast<T *>(static_cast<char *>(ctx.dvec) + mis);
  cudaPointerAttributes attr{};
  const bool mapped = cudaPointerGetAttributes(&attr, vec) == cudaSuccess &&
                      attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr &&
                      ((uintptr_t)attr.devicePointer & 15u) == mis;
  cudaGetLastError();  // a plain host pointer is not an error
  if (mapped) {
    *ingest = static_cast<const T *>(attr.devicePointer);
    ctx.stats.host_ingested++;
  } else {
    e = cudaMemcpyAsync(dst, vec, n * sizeof(T), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return from_cuda(e);
    *ingest = nullptr;
    ctx.stats.host_staged++;
  }
  *d_in = dst;
  return GGKS_OK;
}

// ---------------------------------------------------------------------------
// API bodies
// ---------------------------------------------------------------------------
template <class T>
static int api_multiselect(const T *vec, uint64_t n, const uint32_t *h_k, uint32_t num_k, T *out,
                           const ggks_opts *opts, bool host_input) {
  if (!vec || !h_k || !out || n == 0 || n > GGKS_MAX_N || num_k == 0) return GGKS_INVALID_ARG;
  if ((uintptr_t)vec % sizeof(T) != 0) return GGKS_INVALID_ARG;
  for (uint32_t i = 0; i < num_k; ++i)
    if (h_k[i] < 1 || (uint64_t)h_k[i] > n) return GGKS_INVALID_ARG;
  int st = GGKS_OK;
  Context *ctx = resolve(opts, &st);
  if (!ctx) return st;
  std::lock_guard<std::mutex> lk(ctx->mu);
  DeviceGuard dg(ctx->device);
  cudaStream_t s = (opts && opts->stream) ? static_cast<cudaStream_t>(opts->stream) : ctx->stream;
  const T *d_in = vec;
  const T *ingest = nullptr;
  if (host_input) {
    int st2 = stage_host_vector(*ctx, vec, n, s, &d_in, &ingest);
    if (st2 != GGKS_OK) return st2;
  }
  const bool out_dev = opts && (opts->flags & GGKS_FLAG_OUT_DEVICE);
  ReqSource src;
  src.h_k = h_k;
  src.no_small = opts && (opts->flags & GGKS_FLAG_NO_SMALL);
  const T *hres = nullptr;
  st = select<T, T>(*ctx, d_in, n, src, num_k, out_dev ? out : nullptr, out_dev ? nullptr : &hres, s,
                   ingest);
  if (st == GGKS_OK) {
    if (!out_dev) std::memcpy(out, hres, (size_t)num_k * sizeof(T));
    ctx->stats.calls++;
    ctx->stats.bytes_in += n * sizeof(T);
  }
  return st;
}

template <class T>
static int api_topk(const T *vec, uint64_t n, uint32_t K, T *out, const ggks_opts *opts,
                    bool host_input) {
  if (!vec || !out || n == 0 || n > GGKS_MAX_N || K == 0 || (uint64_t)K > n) return GGKS_INVALID_ARG;
  if ((uintptr_t)vec % sizeof(T) != 0) return GGKS_INVALID_ARG;
  int st = GGKS_OK;
  Context *ctx = resolve(opts, &st);
  if (!ctx) return st;
  std::lock_guard<std::mutex> lk(ctx->mu);
  DeviceGuard dg(ctx->device);
  cudaStream_t s = (opts && opts->stream) ? static_cast<cudaStream_t>(opts->stream) : ctx->stream;
  const T *d_in = vec;
  const T *ingest = nullptr;
  if (host_input) {
    int st2 = stage_host_vector(*ctx, vec, n, s, &d_in, &ingest);
    if (st2 != GGKS_OK) return st2;
  }
  const bool out_dev = opts && (opts->flags & GGKS_FLAG_OUT_DEVICE);
  ReqSource src;
  src.topk = true;
  src.topk_pipeline = opts && (opts->flags & GGKS_FLAG_TOPK_PIPELINE);
  src.no_small = opts && (opts->flags & (GGKS_FLAG_NO_SMALL | GGKS_FLAG_TOPK_PIPELINE));
  const T *hres = nullptr;
  st = select<T, T>(*ctx, d_in, n, src, K, out_dev ? out : nullptr, out_dev ? nullptr : &hres, s,
                   ingest);
  if (st == GGKS_OK) {
    if (!out_dev) std::memcpy(out, hres, (size_t)K * sizeof(T));
    ctx->stats.calls++;
    ctx->stats.bytes_in += n * sizeof(T);
  }
  return st;
}

// ---------------------------------------------------------------------------
// batched selection
// ---------------------------------------------------------------------------
// Autotuner candidates: bucket divisor (elements per bucket, roughly) x tile
// size (elements per work item).  Results do not depend on the choice.
static const BatchTune kTuneCandidates[] = {
    {256, 1u << 16},  {256, 1u << 18},  {256, 1u << 20},  {1024, 1u << 16}, {1024, 1u << 18},
    {1024, 1u << 20}, {4096, 1u << 16}, {4096, 1u << 18}, {4096, 1u << 20},
};

static inline uint32_t log2_round(uint64_t v) {
  uint32_t r = 0;
  while (r < 63 && (1ull << (r + 1)) <= v + (v >> 1)) ++r;
  return r;
}

template <class T>
static int api_batch(const T *const *vecs, const uint64_t *n, uint32_t P, const uint32_t *k_off,
                     const uint32_t *h_k, const uint32_t *K, T *out, const ggks_opts *opts) {
  if (!vecs || !n || P == 0 || !out) return GGKS_INVALID_ARG;
  std::vector<uint32_t> off_topk;
  if (K) {
    // top-k: output offsets are the prefix sums of K
    off_topk.resize((size_t)P + 1);
    uint64_t run = 0;
    for (uint32_t p = 0; p < P; ++p) {
      off_topk[p] = (uint32_t)run;
      run += K[p];
      if (run > 0xFFFFFFFFull) return GGKS_INVALID_ARG;
    }
    off_topk[P] = (uint32_t)run;
    k_off = off_topk.data();
  } else if (!k_off || k_off[0] != 0) {
    return GGKS_INVALID_ARG;
  }
  const uint32_t R = k_off[P];
  if (R > 0 && !K && !h_k) return GGKS_INVALID_ARG;
  uint64_t bytes = 0, elems = 0;
  uint32_t active = 0;
  for (uint32_t p = 0; p < P; ++p) {
    if (k_off[p + 1] < k_off[p]) return GGKS_INVALID_ARG;
    const uint32_t nr = k_off[p + 1] - k_off[p];
    if (nr == 0) continue;
    if (!vecs[p] || n[p] == 0 || n[p] > GGKS_MAX_N) return GGKS_INVALID_ARG;
    if ((uintptr_t)vecs[p] % sizeof(T) != 0) return GGKS_INVALID_ARG;
    if (K) {
      if ((uint64_t)K[p] > n[p]) return GGKS_INVALID_ARG;
    } else {
      for (uint32_t j = k_off[p]; j < k_off[p + 1]; ++j)
        if (h_k[j] < 1 || (uint64_t)h_k[j] > n[p]) return GGKS_INVALID_ARG;
    }
    bytes += n[p] * sizeof(T);
    elems += n[p];
    active++;
  }
  if (R == 0) return GGKS_OK;
  int st = GGKS_OK;
  Context *ctx = resolve(opts, &st);
  if (!ctx) return st;
  std::lock_guard<std::mutex> lk(ctx->mu);
  DeviceGuard dg(ctx->device);
  cudaStream_t s = (opts && opts->stream) ? static_cast<cudaStream_t>(opts->stream) : ctx->stream;
  const bool out_dev = opts && (opts->flags & GGKS_FLAG_OUT_DEVICE);
  BatchInput in;
  in.vecs = reinterpret_cast<const void *const *>(vecs);
  in.n = n;
  in.num_problems = P;
  in.k_off = k_off;
  in.k = K ? nullptr : h_k;
  // batch shape: element size, total elements, problems, outputs per problem
  const uint64_t key = ((uint64_t)sizeof(T) << 24) | ((uint64_t)log2_round(elems) << 16) |
                       ((uint64_t)log2_round(active) << 8) | log2_round(R / active);
  auto it = ctx->tuned.find(key);
  BatchTune tune = it != ctx->tuned.end() ? it->second : BatchTune{};
  if (ctx->pinned_tune.div != 0) {
    tune = ctx->pinned_tune;
  } else if (it == ctx->tuned.end() && opts && (opts->flags & GGKS_FLAG_AUTOTUNE)) {
    // whole calls are timed: planning, launches, re-runs and recursion
    double best = -1.0;
    for (const BatchTune &c : kTuneCandidates) {
      const auto t0 = std::chrono::steady_clock::now();
      st = select_batch<T>(*ctx, in, out_dev ? out : nullptr, nullptr, s, c, nullptr);
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (st != GGKS_OK) return st;
      if (best < 0.0 || dt < best) {
        best = dt;
        tune = c;
      }
    }
    ctx->tuned[key] = tune;
  }
  float ms = 0.f;
  st = select_batch<T>(*ctx, in, out_dev ? out : nullptr, out_dev ? nullptr : out, s, tune, &ms);
  if (st == GGKS_OK) {
    ctx->last_tune = tune;
    ctx->stats.calls++;
    ctx->stats.bytes_in += bytes;
  }
  return st;
}

}  // namespace ggks

using namespace ggks;

extern "C" {

int ggks_multiselect_f32(const float *d_vec, uint64_t n, const uint32_t *h_k, uint32_t num_k,
                         float *h_out, const ggks_opts *opts) {
  return api_multiselect<float>(d_vec, n, h_k, num_k, h_out, opts, false);
}
int ggks_multiselect_f64(const double *d_vec, uint64_t n, const uint32_t *h_k, uint32_t num_k,
                         double *h_out, const ggks_opts *opts) {
  return api_multiselect<double>(d_vec, n, h_k, num_k, h_out, opts, false);
}
int ggks_multiselect_u32(const uint32_t *d_vec, uint64_t n, const uint32_t *h_k, uint32_t num_k,
                         uint32_t *h_out, const ggks_opts *opts) {
  return api_multiselect<uint32_t>(d_vec, n, h_k, num_k, h_out, opts, false);
}
int ggks_multiselect_host_f32(const float *h_vec, uint64_t n, const uint32_t *h_k, uint32_t num_k,
                              float *h_out, const ggks_opts *opts) {
  return api_multiselect<float>(h_vec, n, h_k, num_k, h_out, opts, true);
}
int ggks_multiselect_host_f64(const double *h_vec, uint64_t n, const uint32_t *h_k,
                              uint32_t num_k, double *h_out, const ggks_opts *opts) {
  return api_multiselect<double>(h_vec, n, h_k, num_k, h_out, opts, true);
}
int ggks_multiselect_host_u32(const uint32_t *h_vec, uint64_t n, const uint32_t *h_k,
                              uint32_t num_k, uint32_t *h_out, const ggks_opts *opts) {
  return api_multiselect<uint32_t>(h_vec, n, h_k, num_k, h_out, opts, true);
}
int ggks_topk_f32(const float *d_vec, uint64_t n, uint32_t K, float *h_out, const ggks_opts *opts) {
  return api_topk<float>(d_vec, n, K, h_out, opts, false);
}
int ggks_topk_f64(const double *d_vec, uint64_t n, uint32_t K, double *h_out,
                  const ggks_opts *opts) {
  return api_topk<double>(d_vec, n, K, h_out, opts, false);
}
int ggks_topk_u32(const uint32_t *d_vec, uint64_t n, uint32_t K, uint32_t *h_out,
                  const ggks_opts *opts) {
  return api_topk<uint32_t>(d_vec, n, K, h_out, opts, false);
}
int ggks_select_f32(const float *d_vec, uint64_t n, uint32_t k, float *out, const ggks_opts *opts) {
  return api_multiselect<float>(d_vec, n, &k, 1, out, opts, false);
}
int ggks_select_f64(const double *d_vec, uint64_t n, uint32_t k, double *out,
                    const ggks_opts *opts) {
  return api_multiselect<double>(d_vec, n, &k, 1, out, opts, false);
}
int ggks_select_u32(const uint32_t *d_vec, uint64_t n, uint32_t k, uint32_t *out,
                    const ggks_opts *opts) {
  return api_multiselect<uint32_t>(d_vec, n, &k, 1, out, opts, false);
}
int ggks_topk_host_f32(const float *h_vec, uint64_t n, uint32_t K, float *h_out,
                       const ggks_opts *opts) {
  return api_topk<float>(h_vec, n, K, h_out, opts, true);
}
int ggks_topk_host_f64(const double *h_vec, uint64_t n, uint32_t K, double *h_out,
                       const ggks_opts *opts) {
  return api_topk<double>(h_vec, n, K, h_out, opts, true);
}
int ggks_topk_host_u32(const uint32_t *h_vec, uint64_t n, uint32_t K, uint32_t *h_out,
                       const ggks_opts *opts) {
  return api_topk<uint32_t>(h_vec, n, K, h_out, opts, true);
}

int ggks_multiselect_batch_f32(const float *const *d_vecs, const uint64_t *n, uint32_t num_problems,
                               const uint32_t *k_offsets, const uint32_t *h_k, float *out,
                               const ggks_opts *opts) {
  return api_batch<float>(d_vecs, n, num_problems, k_offsets, h_k, nullptr, out, opts);
}
int ggks_multiselect_batch_f64(const double *const *d_vecs, const uint64_t *n,
                               uint32_t num_problems, const uint32_t *k_offsets,
                               const uint32_t *h_k, double *out, const ggks_opts *opts) {
  return api_batch<double>(d_vecs, n, num_problems, k_offsets, h_k, nullptr, out, opts);
}
int ggks_multiselect_batch_u32(const uint32_t *const *d_vecs, const uint64_t *n,
                               uint32_t num_problems, const uint32_t *k_offsets,
                               const uint32_t *h_k, uint32_t *out, const ggks_opts *opts) {
  return api_batch<uint32_t>(d_vecs, n, num_problems, k_offsets, h_k, nullptr, out, opts);
}
int ggks_topk_batch_f32(const float *const *d_vecs, const uint64_t *n, uint32_t num_problems,
                        const uint32_t *K, float *out, const ggks_opts *opts) {
  if (!K) return GGKS_INVALID_ARG;
  return api_batch<float>(d_vecs, n, num_problems, nullptr, nullptr, K, out, opts);
}
int ggks_topk_batch_f64(const double *const *d_vecs, const uint64_t *n, uint32_t num_problems,
                        const uint32_t *K, double *out, const ggks_opts *opts) {
  if (!K) return GGKS_INVALID_ARG;
  return api_batch<double>(d_vecs, n, num_problems, nullptr, nullptr, K, out, opts);
}
int ggks_topk_batch_u32(const uint32_t *const *d_vecs, const uint64_t *n, uint32_t num_problems,
                        const uint32_t *K, uint32_t *out, const ggks_opts *opts) {
  if (!K) return GGKS_INVALID_ARG;
  return api_batch<uint32_t>(d_vecs, n, num_problems, nullptr, nullptr, K, out, opts);
}

static Context *ctx_or_default(ggks_context *ctx, int *st);

int ggks_batch_set_tuning(ggks_context *ctx, uint32_t div, uint32_t tile) {
  if (div != 0 && (div < 16 || div > (1u << 24) || tile < 64)) return GGKS_INVALID_ARG;
  int st = GGKS_OK;
  Context *c = ctx_or_default(ctx, &st);
  if (!c) return st;
  std::lock_guard<std::mutex> lk(c->mu);
  c->pinned_tune.div = div;
  c->pinned_tune.tile = tile;
  return GGKS_OK;
}

int ggks_batch_last_tuning(ggks_context *ctx, uint32_t *div, uint32_t *tile) {
  if (!div || !tile) return GGKS_INVALID_ARG;
  int st = GGKS_OK;
  Context *c = ctx_or_default(ctx, &st);
  if (!c) return st;
  std::lock_guard<std::mutex> lk(c->mu);
  *div = c->last_tune.div;
  *tile = c->last_tune.tile;
  return GGKS_OK;
}

int ggks_context_create(int device, ggks_context **out) {
  if (!out) return GGKS_INVALID_ARG;
  *out = nullptr;
  Context *c = new Context();
  int cur = -1;
  cudaGetDevice(&cur);
  int st = context_init(*c, device);
  if (cur >= 0) cudaSetDevice(cur);
  if (st != GGKS_OK) {
    delete c;
    return st;
  }
  *out = reinterpret_cast<ggks_context *>(c);
  return GGKS_OK;
}

int ggks_context_destroy(ggks_context *ctx) {
  if (!ctx) return GGKS_INVALID_ARG;
  delete reinterpret_cast<Context *>(ctx);
  return GGKS_OK;
}

static Context *ctx_or_default(ggks_context *ctx, int *st) {
  if (ctx) {
    *st = GGKS_OK;
    return reinterpret_cast<Context *>(ctx);
  }
  ggks_opts o{};
  return resolve(&o, st);
}

int ggks_context_get_stats(ggks_context *ctx, ggks_stats *out) {
  if (!out) return GGKS_INVALID_ARG;
  int st = GGKS_OK;
  Context *c = ctx_or_default(ctx, &st);
  if (!c) return st;
  std::lock_guard<std::mutex> lk(c->mu);
  *out = c->stats;
  // kernels of recursive levels count toward the total; the per-pass figures
  // describe the top level only
  for (Context *ch = c->child.get(); ch; ch = ch->child.get()) out->launches += ch->stats.launches;
  return GGKS_OK;
}

int ggks_context_reset_stats(ggks_context *ctx) {
  int st = GGKS_OK;
  Context *c = ctx_or_default(ctx, &st);
  if (!c) return st;
  std::lock_guard<std::mutex> lk(c->mu);
  for (Context *p = c; p; p = p->child.get()) p->stats = ggks_stats{};
  return GGKS_OK;
}

int ggks_context_set_profiling(ggks_context *ctx, int on) {
  int st = GGKS_OK;
  Context *c = ctx_or_default(ctx, &st);
  if (!c) return st;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (on && !c->events_ready) {
    for (int i = 0; i < GGKS_NUM_PASSES; ++i) {
      if (cudaEventCreate(&c->ev0[i]) != cudaSuccess || cudaEventCreate(&c->ev1[i]) != cudaSuccess)
        return GGKS_CUDA_ERROR;
    }
    c->events_ready = true;
  }
  // on: 0 = off; GGKS_PROFILE_PASSES(mask) = the passes in mask; any other
  // value = every pass
  if (on == 0)
    c->profiling = 0;
  else if ((uint32_t)on & 0x80000000u)
    c->profiling = (uint32_t)on & ((1u << GGKS_NUM_PASSES) - 1u);
  else
    c->profiling = (1u << GGKS_NUM_PASSES) - 1u;
  return GGKS_OK;
}

const char *ggks_status_string(int status) {
  switch (status) {
    case GGKS_OK: return "ok";
    case GGKS_INVALID_ARG: return "invalid argument";
    case GGKS_OOM: return "out of memory";
    case GGKS_CUDA_ERROR: return "CUDA error";
    case GGKS_TIMEOUT: return "device-side wait timed out";
    case GGKS_INTERNAL: return "internal consistency check failed";
    case GGKS_NO_DEVICE: return "no CUDA device";
    case GGKS_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

int ggks_version(void) { return GGKS_VERSION; }

}  // extern "C"
