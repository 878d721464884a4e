// ggks_server.cu -- the serving loop: multiselect / top-k requests of mixed
// sizes and element types arrive at any time and are coalesced into batched
// launches (continuous batching).
//
// Host threads per server:
//   admission  takes submitted requests in arrival order while their device
//              bytes (uploaded vector + bucket-state estimate) fit the
//              admission budget -- the HBM cap, and the device's free memory
//              less a reserve -- copies host vectors to the device on a copy
//              stream, and hands requests whose data is on the device to the
//              lanes;
//   lanes      (2 by default) each take every device-ready request (up to
//              max_batch), run one batched selection for their float32 and
//              uint32 requests together (32-bit keys; the float32 problems
//              keep the float order) and one for their float64 requests
//              (select_batch: one persistent launch each; a group of a
//              single request takes the single-vector pipeline, whose latency
//              is lower), scatter the results to the callers' buffers and
//              release the requests' device bytes.  Each lane has its own
//              context (stream and workspace).  The lanes' batched launches
//              form one chain on the device (LaunchChain): each is queued
//              behind the newest kernel of any lane and runs with the whole
//              device as soon as that kernel ends, while the lanes' planning,
//              control-block uploads, result copies and scatter overlap the
//              running kernel -- the device goes from one batch's kernel to
//              the next without a host round trip between them.
// Requests that arrive while batches are on the GPU are admitted and uploaded
// meanwhile and join the next batch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "ggks_internal.h"

namespace ggks {

using Clock = std::chrono::steady_clock;

struct SReq {
  uint64_t ticket = 0;
  int dtype = 0;
  const void *vec = nullptr;  // caller's vector
  bool host = false;          // vec is host memory: copied at admission
  uint64_t n = 0;
  std::vector<uint32_t> k;    // k-th largest, 1-based (top-k: 1 .. K)
  void *out = nullptr;        // caller's host buffer of k.size() values
  uint64_t bytes = 0;         // charge against the cap
  void *dvec = nullptr;       // device copy of a host vector
  cudaEvent_t up = nullptr;   // upload finished
  Clock::time_point t_submit, t_done;
  int status = GGKS_OK;
  bool done = false;
};

struct Lane {
  Context ctx;
  Context ctx64;  // the float64 group's, while the 32-bit group runs on ctx
  std::atomic<bool> ctx64_ready{false};
  std::thread thr;
};

constexpr uint64_t kDefaultReserve = 1ull << 30;
constexpr uint32_t kMaxLanes = 8;

struct Server {
  int device = 0;
  uint64_t cap = 0, used = 0, reserve = kDefaultReserve;
  uint32_t max_batch = 0;
  std::vector<std::unique_ptr<Lane>> lanes;
  LaunchChain chain;
  cudaStream_t copy_stream = nullptr;
  std::mutex mu;
  std::condition_variable cv_admit, cv_exec, cv_done;
  std::deque<SReq *> pending;    // submitted, not admitted
  std::deque<SReq *> uploading;  // admitted, host-to-device copy in flight
  std::deque<SReq *> ready;      // data on the device, waiting for a batch
  std::unordered_map<uint64_t, SReq *> live;
  uint64_t next_ticket = 1;
  bool stopping = false;
  std::thread admit_thr;
  ggks_server_stats st{};
  cudaEvent_t time_base = nullptr;                // recorded once at creation
  std::vector<std::pair<float, float>> launch_ms;  // batched launches' device intervals
  // batch formation: when the device is expected to finish the batches handed
  // out so far, and the device time per input byte of large batched launches
  // (moving average; 0 until one has been measured)
  Clock::time_point dev_free_est{};
  double ns_per_byte = 0.0;
  double prep_ns_per_req = 0.0;  // host time from taking a batch to its first launch, per request
  // the device's free memory as last read, and when (admission reads it
  // again after kFreeMemAge, or whenever a request does not fit)
  uint64_t free_mem = 0;
  Clock::time_point free_mem_t{};
};

constexpr auto kFreeMemAge = std::chrono::milliseconds(1);

// a lane takes its batch this long, plus the measured host preparation of
// as many requests as are ready, before the device is expected to run out of
// queued work: time to plan and upload the batch and queue its launch
constexpr auto kBatchLead = std::chrono::microseconds(400);
// the device's queued work is taken as this fraction of its estimate: a batch
// taken a little early only waits on the device, one taken late leaves the
// device idle for its host preparation
constexpr double kDevEstimateFactor = 0.8;
// expected device time of a batched launch: a fixed part (its latency-bound
// phases) and the slope measured on launches of at least kSlopeBytes
constexpr double kLaunchFixedNs = 100e3;
constexpr uint64_t kSlopeBytes = 64ull << 20;

static size_t elem_size(int dtype) { return dtype == GGKS_DTYPE_F64 ? 8 : 4; }

// device bytes charged for a request: its uploaded vector and an estimate of
// its bucket state (tables, rows, survivors, outputs)
static uint64_t charge_of(const SReq &r) {
  const uint64_t vb = r.n * elem_size(r.dtype);
  return (r.host ? vb : 0) + 65536 + vb / 16 + (uint64_t)r.k.size() * 64;
}

// Admission budget: the cap, and no more than the device's free memory
// (less the reserve) on top of the bytes already admitted.  The free memory
// is read again when the last reading is older than kFreeMemAge or when
// `fresh` (a request did not fit the budget); the bytes admitted since a
// reading count against it through S->used.
static uint64_t admit_budget(Server *S, bool fresh) {
  const auto now = Clock::now();
  uint64_t hbm = S->cap;
  if (fresh || now - S->free_mem_t > kFreeMemAge || S->free_mem_t == Clock::time_point{}) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
      // free memory net of what was admitted then, so that S->used adds back
      S->free_mem = (uint64_t)fr + S->used;
      S->free_mem_t = now;
    } else {
      S->free_mem_t = Clock::time_point{};
    }
  }
  if (S->free_mem_t != Clock::time_point{})
    hbm = S->free_mem > S->reserve ? S->free_mem - S->reserve : 0ull;
  const uint64_t b = std::min(S->cap, hbm);
  S->st.admit_budget_bytes = b;
  return b;
}

static void admit_loop(Server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  bool held = false;       // the head waits for device memory ...
  uint64_t used_at_hold = 0;  // ... since the admitted bytes were this much
  for (;;) {
    // a held head is tried again once admitted bytes have been released
    S->cv_admit.wait(lk, [&] {
      return S->stopping || !S->uploading.empty() ||
             (!S->pending.empty() && S->used + S->pending.front()->bytes <= S->cap &&
              (!held || S->used < used_at_hold));
    });
    if (S->stopping && S->pending.empty() && S->uploading.empty()) return;
    // admit in arrival order while the cap and the free memory allow; the
    // budget is taken once per round (cudaMemGetInfo), again when the head
    // does not fit it
    uint64_t budget = admit_budget(S, false);
    held = false;
    while (!S->pending.empty() && S->used + S->pending.front()->bytes <= S->cap) {
      SReq *r = S->pending.front();
      if (S->used + r->bytes > budget) {
        budget = admit_budget(S, true);
        if (S->used + r->bytes > budget) {
          if (S->used == 0 && S->uploading.empty()) {
            // nothing admitted will free memory: it cannot fit
            S->pending.pop_front();
            r->status = GGKS_OOM;
            r->t_done = Clock::now();
            r->done = true;
            S->st.completed++;
            S->cv_done.notify_all();
            continue;
          }
          S->st.hbm_waits++;
          held = true;  // retried when an admitted request completes
          used_at_hold = S->used;
          break;
        }
      }
      S->pending.pop_front();
      S->used += r->bytes;
      S->st.peak_bytes = std::max(S->st.peak_bytes, S->used);
      if (!r->host) {
        S->ready.push_back(r);
        S->cv_exec.notify_one();
        continue;
      }
      const size_t vb = r->n * elem_size(r->dtype);
      cudaError_t e = cudaMallocAsync(&r->dvec, vb, S->copy_stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(r->dvec, r->vec, vb, cudaMemcpyHostToDevice, S->copy_stream);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->up, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(r->up, S->copy_stream);
      if (e != cudaSuccess) r->status = from_cuda(e);
      S->st.uploads++;
      S->st.upload_bytes += vb;
      S->uploading.push_back(r);
    }
    // hand over the oldest upload once it has landed
    if (!S->uploading.empty()) {
      SReq *r = S->uploading.front();
      lk.unlock();
      if (r->status == GGKS_OK && r->up) {
        const cudaError_t e = cudaEventSynchronize(r->up);
        if (e != cudaSuccess) r->status = from_cuda(e);
      }
      lk.lock();
      S->uploading.pop_front();
      S->ready.push_back(r);
      S->cv_exec.notify_one();
    }
  }
}

// a lone request: the single-vector pipeline has the lower latency
template <class T>
static void run_single(Context &ctx, SReq *r) {
  const T *vec = static_cast<const T *>(r->host ? r->dvec : r->vec);
  ReqSource src;
  src.h_k = r->k.data();
  const T *res = nullptr;
  std::lock_guard<std::mutex> lk(ctx.mu);
  r->status = select<T, T>(ctx, vec, r->n, src, (uint32_t)r->k.size(), nullptr, &res,
                           ctx.stream, nullptr);
  if (r->status == GGKS_OK) std::memcpy(r->out, res, r->k.size() * sizeof(T));
}

// One group: the float64 requests of a batch (T = double), or its float32 and
// uint32 requests together (T = uint32_t: both have 32-bit keys, the float32
// problems are flagged and keep the float order).
template <class T>
static void run_group(Server *S, Context &ctx, std::vector<SReq *> &g) {
  if (g.size() == 1) {
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->st.single_calls++;
    }
    SReq *r = g[0];
    if (r->dtype == GGKS_DTYPE_F32)
      run_single<float>(ctx, r);
    else
      run_single<T>(ctx, r);
    return;
  }
  std::vector<const void *> vecs(g.size());
  std::vector<uint64_t> ns(g.size());
  std::vector<uint32_t> off(g.size() + 1, 0), ks;
  for (size_t i = 0; i < g.size(); ++i) {
    vecs[i] = g[i]->host ? g[i]->dvec : g[i]->vec;
    ns[i] = g[i]->n;
    off[i + 1] = off[i] + (uint32_t)g[i]->k.size();
    ks.insert(ks.end(), g[i]->k.begin(), g[i]->k.end());
  }
  std::vector<T> out(off.back());
  std::vector<uint8_t> flt(g.size(), 0);
  bool any_float = false;
  for (size_t i = 0; i < g.size(); ++i) {
    flt[i] = g[i]->dtype == GGKS_DTYPE_F32 ? 1 : 0;
    any_float |= flt[i] != 0;
  }
  BatchInput in;
  in.vecs = vecs.data();
  in.n = ns.data();
  if (std::is_same<T, uint32_t>::value && any_float) in.is_float = flt.data();
  in.num_problems = (uint32_t)g.size();
  in.k_off = off.data();
  in.k = ks.data();
  std::lock_guard<std::mutex> lk(ctx.mu);
  const BatchTune tune = ctx.pinned_tune.div ? ctx.pinned_tune : BatchTune{};
  float kms = 0.f;
  const int st = select_batch<T>(ctx, in, nullptr, out.data(), ctx.stream, tune, &kms);
  uint64_t bytes = 0;
  for (SReq *r : g) bytes += r->n * elem_size(r->dtype);
  bool newest = false;  // no other lane's launch queued behind this one
  {
    std::lock_guard<std::mutex> lc(S->chain.mu);
    newest = S->chain.last == ctx.bev1;
  }
  {
    std::lock_guard<std::mutex> lk2(S->mu);
    S->st.kernel_ms += kms;
    if (newest && S->dev_free_est > Clock::now()) {
      // the device ran out of work sooner than expected: a lane holding its
      // batch open takes it now
      S->dev_free_est = Clock::now();
      S->cv_exec.notify_all();
    }
    if (st == GGKS_OK && bytes >= kSlopeBytes) {
      const double v = std::max(0.0, (double)kms * 1e6 - kLaunchFixedNs) / (double)bytes;
      S->ns_per_byte = S->ns_per_byte == 0.0 ? v : 0.8 * S->ns_per_byte + 0.2 * v;
    }
    if (st == GGKS_OK) S->launch_ms.emplace_back(ctx.last_launch_t0, ctx.last_launch_t1);
  }
  for (size_t i = 0; i < g.size(); ++i) {
    if (st != GGKS_OK) {
      g[i]->status = st;
      continue;
    }
    std::memcpy(g[i]->out, out.data() + off[i], g[i]->k.size() * sizeof(T));
  }
}

// marks a finished group done: frees its uploads, releases its bytes and
// wakes its waiters and the admission thread
static void complete(Server *S, cudaStream_t stream, std::vector<SReq *> &g, bool launched) {
  for (SReq *r : g)
    if (r->dvec) cudaFreeAsync(r->dvec, stream);
  cudaStreamSynchronize(stream);
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lk(S->mu);
  for (SReq *r : g) {
    if (r->up) cudaEventDestroy(r->up);
    r->up = nullptr;
    r->dvec = nullptr;
    r->t_done = now;
    r->done = true;
    S->used -= r->bytes;
    S->st.completed++;
  }
  if (launched) S->st.launches++;
  S->cv_done.notify_all();
  S->cv_admit.notify_one();
}

// runs one group on a context of a lane
template <class T>
static void run_counted(Server *S, Context &ctx, std::vector<SReq *> &g) {
  const auto t0 = Clock::now();
  run_group<T>(S, ctx, g);
  complete(S, ctx.stream, g, true);
  std::lock_guard<std::mutex> lk(S->mu);
  S->st.group_ms += std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

static void lane_loop(Server *S, Lane *L) {
  cudaSetDevice(S->device);
  std::vector<SReq *> batch;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        S->cv_exec.wait(lk, [&] {
          return !S->ready.empty() ||
                 (S->stopping && S->pending.empty() && S->uploading.empty());
        });
        if (S->ready.empty()) {
          S->cv_exec.notify_all();  // the other lanes stop too
          return;
        }
        // Continuous batching: while the device still has queued work that
        // lasts longer than it takes to plan and launch a batch, the batch
        // is held open and requests arriving meanwhile join it (fewer,
        // larger launches, each with its fixed phases); it is taken in time
        // to keep the device fed, at once when the device is idle, full or
        // the server is stopping.
        const auto hold_until =
            S->dev_free_est - kBatchLead -
            std::chrono::nanoseconds((int64_t)(S->prep_ns_per_req * (double)S->ready.size()));
        if (S->stopping || Clock::now() >= hold_until ||
            (S->max_batch && S->ready.size() >= S->max_batch))
          break;
        S->cv_exec.wait_until(lk, hold_until);
      }
      batch.clear();
      uint64_t bytes = 0;
      while (!S->ready.empty() && (S->max_batch == 0 || batch.size() < S->max_batch)) {
        batch.push_back(S->ready.front());
        bytes += batch.back()->n * elem_size(batch.back()->dtype);
        S->ready.pop_front();
      }
      // the device is expected to run this batch after the work already handed out
      const auto start = std::max(Clock::now() + kBatchLead, S->dev_free_est);
      if (S->ns_per_byte > 0.0)
        S->dev_free_est =
            start + std::chrono::nanoseconds((int64_t)(kDevEstimateFactor *
                                                       (kLaunchFixedNs + S->ns_per_byte * (double)bytes)));
      S->st.batches++;
      S->st.batched_requests += batch.size();
      S->st.max_batch_seen = std::max<uint64_t>(S->st.max_batch_seen, batch.size());
    }
    // float32 and uint32 requests share one launch (32-bit keys); float64
    // requests take their own
    const auto t_take = Clock::now();
    std::vector<SReq *> g32, g64, failed;
    for (SReq *r : batch)
      (r->status != GGKS_OK ? failed : r->dtype == GGKS_DTYPE_F64 ? g64 : g32).push_back(r);
    if (!failed.empty()) complete(S, L->ctx.stream, failed, false);
    const auto launches0 = L->ctx.stats.launches;
    // a float64 group runs at the same time on the lane's second context, so
    // both groups' launches are queued on the device together
    std::thread t64;
    if (!g64.empty() && !g32.empty()) {
      if (!L->ctx64_ready) {
        if (context_init(L->ctx64, S->device) == GGKS_OK) {
          L->ctx64.chain = &S->chain;
          L->ctx64.time_base = S->time_base;
          {
            std::lock_guard<std::mutex> lk(L->ctx.mu);
            L->ctx64.pinned_tune = L->ctx.pinned_tune;
          }
          L->ctx64_ready = true;
        }
      }
      if (L->ctx64_ready) {
        t64 = std::thread([S, L, &g64] {
          cudaSetDevice(S->device);
          run_counted<double>(S, L->ctx64, g64);
        });
      }
    }
    if (!g32.empty()) run_counted<uint32_t>(S, L->ctx, g32);
    // host preparation of the first group, per request of the batch
    if (L->ctx.stats.launches != launches0 && g32.size() > 1 && L->ctx.last_launch_wall > t_take) {
      const double v =
          std::chrono::duration<double, std::nano>(L->ctx.last_launch_wall - t_take).count() /
          (double)batch.size();
      std::lock_guard<std::mutex> lk(S->mu);
      S->prep_ns_per_req = S->prep_ns_per_req == 0.0 ? v : 0.8 * S->prep_ns_per_req + 0.2 * v;
    }
    if (t64.joinable())
      t64.join();
    else if (!g64.empty())
      run_counted<double>(S, L->ctx, g64);
  }
}

}  // namespace ggks

using namespace ggks;

extern "C" {

int ggks_server_create(const ggks_server_config *cfg, ggks_server **out) {
  if (!cfg || !out || cfg->hbm_cap_bytes == 0 || cfg->lanes > kMaxLanes) return GGKS_INVALID_ARG;
  *out = nullptr;
  Server *S = new Server();
  const uint32_t nl = cfg->lanes ? cfg->lanes : 2u;
  int cur = -1;
  cudaGetDevice(&cur);
  int st = GGKS_OK;
  for (uint32_t i = 0; i < nl && st == GGKS_OK; ++i) {
    S->lanes.emplace_back(new Lane());
    st = context_init(S->lanes.back()->ctx, cfg->device);
    S->lanes.back()->ctx.chain = &S->chain;
  }
  if (st == GGKS_OK &&
      cudaStreamCreateWithFlags(&S->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    st = GGKS_CUDA_ERROR;
  // one time base for every lane's launch intervals
  if (st == GGKS_OK && (cudaEventCreate(&S->time_base) != cudaSuccess ||
                        cudaEventRecord(S->time_base, S->copy_stream) != cudaSuccess ||
                        cudaEventSynchronize(S->time_base) != cudaSuccess))
    st = GGKS_CUDA_ERROR;
  if (st == GGKS_OK)
    for (auto &L : S->lanes) L->ctx.time_base = S->time_base;
  if (st != GGKS_OK) {
    if (S->time_base) cudaEventDestroy(S->time_base);
    if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
  }
  if (cur >= 0) cudaSetDevice(cur);
  if (st != GGKS_OK) {
    delete S;
    return st;
  }
  S->device = cfg->device;
  S->cap = cfg->hbm_cap_bytes;
  S->reserve = cfg->hbm_reserve_bytes ? cfg->hbm_reserve_bytes : kDefaultReserve;
  S->max_batch = cfg->max_batch;
  S->admit_thr = std::thread(admit_loop, S);
  for (auto &L : S->lanes) L->thr = std::thread(lane_loop, S, L.get());
  *out = reinterpret_cast<ggks_server *>(S);
  return GGKS_OK;
}

int ggks_server_destroy(ggks_server *srv) {
  if (!srv) return GGKS_INVALID_ARG;
  Server *S = reinterpret_cast<Server *>(srv);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stopping = true;
  }
  S->cv_admit.notify_all();
  S->cv_exec.notify_all();
  S->admit_thr.join();
  {
    std::lock_guard<std::mutex> lk(S->mu);
  }
  S->cv_exec.notify_all();
  for (auto &L : S->lanes) L->thr.join();
  for (auto &kv : S->live) delete kv.second;
  int cur = -1;
  cudaGetDevice(&cur);
  cudaSetDevice(S->device);
  if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
  if (S->time_base) cudaEventDestroy(S->time_base);
  if (cur >= 0) cudaSetDevice(cur);
  delete S;
  return GGKS_OK;
}

int ggks_server_submit(ggks_server *srv, const ggks_request *req, void *out, uint64_t *ticket) {
  if (!srv || !req || !out || !ticket) return GGKS_INVALID_ARG;
  Server *S = reinterpret_cast<Server *>(srv);
  if (req->dtype != GGKS_DTYPE_F32 && req->dtype != GGKS_DTYPE_F64 && req->dtype != GGKS_DTYPE_U32)
    return GGKS_INVALID_ARG;
  if (!req->vec || req->n == 0 || req->n > GGKS_MAX_N || req->num_k == 0) return GGKS_INVALID_ARG;
  if ((uintptr_t)req->vec % elem_size(req->dtype) != 0) return GGKS_INVALID_ARG;
  const bool topk = (req->flags & GGKS_REQ_TOPK) != 0;
  if (topk ? (uint64_t)req->num_k > req->n : !req->k) return GGKS_INVALID_ARG;
  SReq *r = new SReq();
  r->dtype = req->dtype;
  r->vec = req->vec;
  r->host = (req->flags & GGKS_REQ_HOST_VECTOR) != 0;
  r->n = req->n;
  r->out = out;
  r->k.resize(req->num_k);
  for (uint32_t i = 0; i < req->num_k; ++i) {
    const uint32_t k = topk ? i + 1 : req->k[i];
    if (k < 1 || (uint64_t)k > req->n) {
      delete r;
      return GGKS_INVALID_ARG;
    }
    r->k[i] = k;
  }
  r->bytes = charge_of(*r);
  if (r->bytes > S->cap) {
    delete r;
    return GGKS_OOM;  // would never fit the cap
  }
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    r->ticket = S->next_ticket++;
    S->live[r->ticket] = r;
    S->pending.push_back(r);
    S->st.submitted++;
    *ticket = r->ticket;
  }
  S->cv_admit.notify_one();
  return GGKS_OK;
}

int ggks_server_wait(ggks_server *srv, uint64_t ticket, double *latency_ms) {
  if (!srv) return GGKS_INVALID_ARG;
  Server *S = reinterpret_cast<Server *>(srv);
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->live.find(ticket);
  if (it == S->live.end()) return GGKS_INVALID_ARG;
  SReq *r = it->second;
  S->cv_done.wait(lk, [&] { return r->done; });
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  const int st = r->status;
  S->live.erase(it);
  delete r;
  return st;
}

int ggks_server_get_stats(ggks_server *srv, ggks_server_stats *out) {
  if (!srv || !out) return GGKS_INVALID_ARG;
  Server *S = reinterpret_cast<Server *>(srv);
  ggks_server_stats st;
  std::vector<std::pair<float, float>> iv;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    st = S->st;
    st.in_flight_bytes = S->used;
    iv = S->launch_ms;
  }
  {
    std::lock_guard<std::mutex> lk(S->chain.mu);
    st.concurrent_launches = S->chain.queued;
  }
  // device time covered by at least one batched launch
  std::sort(iv.begin(), iv.end());
  double busy = 0.0, end = -1e300;
  for (const auto &p : iv) {
    if (p.first > end) {
      busy += p.second - p.first;
      end = p.second;
    } else if (p.second > end) {
      busy += p.second - end;
      end = p.second;
    }
  }
  st.device_busy_ms = busy;
  st.device_span_ms = iv.empty() ? 0.0 : end - iv.front().first;
  // the lanes' batched phases and recursions, read under each lane's lock
  st.recursions = 0;
  for (int ph = 0; ph < GGKS_NUM_BATCH_PHASES; ++ph) st.batch_phase_ms[ph] = 0.0;
  for (auto &L : S->lanes) {
    Context *cs[2] = {&L->ctx, L->ctx64_ready ? &L->ctx64 : nullptr};
    for (Context *c : cs) {
      if (!c) continue;
      std::lock_guard<std::mutex> lk(c->mu);
      st.recursions += c->stats.recursions;
      for (int ph = 0; ph < GGKS_NUM_BATCH_PHASES; ++ph)
        st.batch_phase_ms[ph] += c->stats.batch_phase_ms[ph];
    }
  }
  *out = st;
  return GGKS_OK;
}

int ggks_server_set_tuning(ggks_server *srv, uint32_t div, uint32_t tile) {
  if (!srv) return GGKS_INVALID_ARG;
  Server *S = reinterpret_cast<Server *>(srv);
  for (auto &L : S->lanes) {
    int st = ggks_batch_set_tuning(reinterpret_cast<ggks_context *>(&L->ctx), div, tile);
    if (st == GGKS_OK && L->ctx64_ready)
      st = ggks_batch_set_tuning(reinterpret_cast<ggks_context *>(&L->ctx64), div, tile);
    if (st != GGKS_OK) return st;
  }
  return GGKS_OK;
}

}  // extern "C"
