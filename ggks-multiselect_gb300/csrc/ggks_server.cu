// ggks_server.cu -- the serving loop: multiselect / top-k requests of mixed
// sizes and element types arrive at any time and are coalesced into batched
// launches (continuous batching).
//
// Two host threads per server:
//   admission  takes submitted requests in arrival order while their device
//              bytes fit the HBM cap (uploaded vector + bucket-state estimate),
//              copies host vectors to the device on a copy stream, and hands
//              requests whose data is on the device to the executor;
//   executor   takes every device-ready request (up to max_batch), runs one
//              batched selection per element type (select_batch: one
//              persistent launch each; a type with a single request takes the
//              single-vector pipeline, whose latency is lower), scatters the
//              results to the callers' buffers, releases the requests' device
//              bytes.
// Requests that arrive while a batch is on the GPU are admitted and uploaded
// meanwhile (the copy stream overlaps the compute stream) and join the next
// batch.  Batches run one after another on the compute stream, so no two
// cooperative launches are ever in flight together.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
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

struct Server {
  int device = 0;
  uint64_t cap = 0, used = 0;
  uint32_t max_batch = 0;
  Context ctx;
  cudaStream_t copy_stream = nullptr;
  std::mutex mu;
  std::condition_variable cv_admit, cv_exec, cv_done;
  std::deque<SReq *> pending;    // submitted, not admitted
  std::deque<SReq *> uploading;  // admitted, host-to-device copy in flight
  std::deque<SReq *> ready;      // data on the device, waiting for a batch
  std::unordered_map<uint64_t, SReq *> live;
  uint64_t next_ticket = 1;
  bool stopping = false;
  std::thread admit_thr, exec_thr;
  ggks_server_stats st{};
};

static size_t elem_size(int dtype) { return dtype == GGKS_DTYPE_F64 ? 8 : 4; }

// device bytes charged for a request: its uploaded vector and an estimate of
// its bucket state (tables, rows, survivors, outputs)
static uint64_t charge_of(const SReq &r) {
  const uint64_t vb = r.n * elem_size(r.dtype);
  return (r.host ? vb : 0) + 65536 + vb / 16 + (uint64_t)r.k.size() * 64;
}

static void admit_loop(Server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_admit.wait(lk, [&] {
      return S->stopping || !S->uploading.empty() ||
             (!S->pending.empty() && S->used + S->pending.front()->bytes <= S->cap);
    });
    if (S->stopping && S->pending.empty() && S->uploading.empty()) return;
    // admit in arrival order while the cap allows
    while (!S->pending.empty() && S->used + S->pending.front()->bytes <= S->cap) {
      SReq *r = S->pending.front();
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

template <class T>
static void run_group(Server *S, std::vector<SReq *> &g) {
  if (g.size() == 1) {
    // a lone request: the single-vector pipeline has the lower latency
    SReq *r = g[0];
    const T *vec = static_cast<const T *>(r->host ? r->dvec : r->vec);
    ReqSource src;
    src.h_k = r->k.data();
    const T *res = nullptr;
    std::lock_guard<std::mutex> lk(S->ctx.mu);
    r->status = select<T, T>(S->ctx, vec, r->n, src, (uint32_t)r->k.size(), nullptr, &res,
                             S->ctx.stream, nullptr);
    if (r->status == GGKS_OK) std::memcpy(r->out, res, r->k.size() * sizeof(T));
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
  BatchInput in;
  in.vecs = vecs.data();
  in.n = ns.data();
  in.num_problems = (uint32_t)g.size();
  in.k_off = off.data();
  in.k = ks.data();
  std::lock_guard<std::mutex> lk(S->ctx.mu);
  const BatchTune tune = S->ctx.pinned_tune.div ? S->ctx.pinned_tune : BatchTune{};
  const int st = select_batch<T>(S->ctx, in, nullptr, out.data(), S->ctx.stream, tune, nullptr);
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
static void complete(Server *S, std::vector<SReq *> &g, bool launched) {
  for (SReq *r : g)
    if (r->dvec) cudaFreeAsync(r->dvec, S->ctx.stream);
  cudaStreamSynchronize(S->ctx.stream);
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

static void exec_loop(Server *S) {
  cudaSetDevice(S->device);
  std::vector<SReq *> batch;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_exec.wait(lk, [&] {
        return !S->ready.empty() ||
               (S->stopping && S->pending.empty() && S->uploading.empty());
      });
      if (S->ready.empty()) return;
      batch.clear();
      while (!S->ready.empty() && (S->max_batch == 0 || batch.size() < S->max_batch)) {
        batch.push_back(S->ready.front());
        S->ready.pop_front();
      }
      S->st.batches++;
      S->st.batched_requests += batch.size();
      S->st.max_batch_seen = std::max<uint64_t>(S->st.max_batch_seen, batch.size());
    }
    std::vector<SReq *> g[3], failed;
    for (SReq *r : batch) (r->status == GGKS_OK ? g[r->dtype] : failed).push_back(r);
    if (!failed.empty()) complete(S, failed, false);
    if (!g[GGKS_DTYPE_F32].empty()) {
      run_group<float>(S, g[GGKS_DTYPE_F32]);
      complete(S, g[GGKS_DTYPE_F32], true);
    }
    if (!g[GGKS_DTYPE_U32].empty()) {
      run_group<uint32_t>(S, g[GGKS_DTYPE_U32]);
      complete(S, g[GGKS_DTYPE_U32], true);
    }
    if (!g[GGKS_DTYPE_F64].empty()) {
      run_group<double>(S, g[GGKS_DTYPE_F64]);
      complete(S, g[GGKS_DTYPE_F64], true);
    }
  }
}

}  // namespace ggks

using namespace ggks;

extern "C" {

int ggks_server_create(const ggks_server_config *cfg, ggks_server **out) {
  if (!cfg || !out || cfg->hbm_cap_bytes == 0) return GGKS_INVALID_ARG;
  *out = nullptr;
  Server *S = new Server();
  int cur = -1;
  cudaGetDevice(&cur);
  int st = context_init(S->ctx, cfg->device);
  if (st == GGKS_OK &&
      cudaStreamCreateWithFlags(&S->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    st = GGKS_CUDA_ERROR;
  if (cur >= 0) cudaSetDevice(cur);
  if (st != GGKS_OK) {
    delete S;
    return st;
  }
  S->device = cfg->device;
  S->cap = cfg->hbm_cap_bytes;
  S->max_batch = cfg->max_batch;
  S->admit_thr = std::thread(admit_loop, S);
  S->exec_thr = std::thread(exec_loop, S);
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
  S->exec_thr.join();
  for (auto &kv : S->live) delete kv.second;
  int cur = -1;
  cudaGetDevice(&cur);
  cudaSetDevice(S->device);
  if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
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
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->st;
  out->in_flight_bytes = S->used;
  return GGKS_OK;
}

int ggks_server_set_tuning(ggks_server *srv, uint32_t div, uint32_t tile) {
  if (!srv) return GGKS_INVALID_ARG;
  Server *S = reinterpret_cast<Server *>(srv);
  return ggks_batch_set_tuning(reinterpret_cast<ggks_context *>(&S->ctx), div, tile);
}

}  // extern "C"
