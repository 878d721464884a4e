// ggks_batch_host.cuh -- host driver of the batched multiselect (one
// cooperative launch of k_batch per batch).  Included by the per-type units.
#pragma once

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "ggks_batch.cuh"
#include "ggks_internal.h"

namespace ggks {

static inline size_t balign(size_t v, size_t a) { return (v + a - 1) / a * a; }

static inline uint32_t pow2_ceil_u32(uint64_t v) {
  uint32_t r = 1;
  while (r < v && r < 0x80000000u) r <<= 1;
  return r;
}

// the batch's shared-memory need: the largest of the phases' layouts
template <class T>
static inline int batch_smem_bytes() {
  using K = typename Traits<T>::K;
  const size_t table = (size_t)kBMaxS * sizeof(K);
  const size_t plan = kLutPadded * 4 + (size_t)kBMaxNb * 5 + (size_t)kBPlanSlots * 8;
  const size_t tiles = (kBTileLut + (size_t)kBMaxNb) * 4 + kBRepBytes;
  const size_t fin = std::max(finish_smem_for<K>(sizeof(K) == 4 ? 4096u : 2048u),
                              (size_t)(kBThreads / 32) *
                                  (kBWarpBytes + (kWarpSelBins + kWarpSelReq) * 4));
  return (int)std::max(std::max(table, tiles), std::max(plan, fin));
}

template <class T>
int select_batch(Context &ctx, const BatchInput &in, T *d_out_user, T *h_out, cudaStream_t s,
                 const BatchTune &tune, float *kernel_ms) {
  using K = typename Traits<T>::K;
  const uint32_t bcap = sizeof(K) == 4 ? 4096u : 2048u;
  const uint32_t R = in.k_off[in.num_problems];
  // float32 problems ride in uint32 batches only, with host outputs
  if (in.is_float && (!std::is_same<T, uint32_t>::value || d_out_user)) return GGKS_INVALID_ARG;

  // co-resident grid: every CTA the SMs hold at once
  const int smem = batch_smem_bytes<T>();
  // the kernel's attributes belong to it as loaded on one device: set up once
  // per device (per instantiation), the resulting occupancy remembered + 1
  static std::atomic<int> bps_plus1[kMaxDevices];  // static storage: starts at zero
  const bool tracked = ctx.device >= 0 && ctx.device < kMaxDevices;
  int blocks_per_sm = tracked ? bps_plus1[ctx.device].load(std::memory_order_acquire) - 1 : -1;
  if (blocks_per_sm < 0) {
    cudaError_t ae = cudaFuncSetAttribute((const void *)k_batch<T>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // two CTAs of about 100 KB each per SM: ask for the largest shared-memory carveout
    if (ae == cudaSuccess)
      ae = cudaFuncSetAttribute((const void *)k_batch<T>,
                                cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (ae != cudaSuccess) return from_cuda(ae);
    int b = 0;
    const cudaError_t oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch<T>, kBThreads,
                                                                           smem);
    if (oe != cudaSuccess) return from_cuda(oe);
    blocks_per_sm = b;
    if (tracked) bps_plus1[ctx.device].store(b + 1, std::memory_order_release);
  }
  if (blocks_per_sm < 1) return GGKS_UNSUPPORTED;
  const uint32_t max_grid = (uint32_t)blocks_per_sm * (uint32_t)ctx.sm_count;

  // ---- plan: problems with requests, their bucket budgets and tiles.  The
  // tile size is the tuned one, or smaller when the batch holds fewer than
  // two tiles per resident CTA of that size (a few large tiles would leave
  // most CTAs idle in the streaming phases).
  uint64_t total_n = 0;
  for (uint32_t p = 0; p < in.num_problems; ++p)
    if (in.k_off[p + 1] > in.k_off[p]) total_n += in.n[p];
  uint64_t tile = std::max<uint64_t>(64, tune.tile & ~63ull);
  while (tile > kBMinTile && total_n / tile < 2ull * max_grid) tile >>= 1;
  std::vector<BProb> probs;
  std::vector<uint32_t> orig;  // problem index in the caller's arrays
  probs.reserve(in.num_problems);
  uint64_t lut_words = 0, cnt_words = 0, row_words = 0, surv_est = 0;
  uint32_t num_tiles = 0;
  for (uint32_t p = 0; p < in.num_problems; ++p) {
    const uint32_t nr = in.k_off[p + 1] - in.k_off[p];
    if (nr == 0) continue;
    BProb b{};
    b.x = in.vecs[p];
    b.n = in.n[p];
    // buckets: about n / div elements each, a power of two in [4, kBMaxNb];
    // half as many slices, at most kBSlices (the table needs nb_max >=
    // slices + 2; the tile phases hold it once per bank)
    uint32_t nbm = pow2_ceil_u32((b.n + tune.div - 1) / tune.div);
    nbm = std::min(kBMaxNb, std::max(4u, nbm));
    uint32_t nsl_bits = 0;
    while ((2u << nsl_bits) < nbm && nsl_bits < kBSliceBits) ++nsl_bits;
    b.nb_max = nbm;
    b.nsl_bits = nsl_bits;
    b.S = (uint32_t)std::min<uint64_t>(b.n, kBMaxS);
    b.ntiles = (uint32_t)((b.n + tile - 1) / tile);
    b.req_off = in.k_off[p];
    b.num_req = nr;
    b.flt = in.is_float ? (in.is_float[p] ? 1u : 0u) : 0u;
    // speculation: requests whose ascending ranks span at most n / 32 (a top-k,
    // k's close together) of a problem larger than eight samples' worth
    {
      uint64_t rmin = ~0ull, rmax = 0;
      for (uint32_t i = 0; i < nr; ++i) {
        const uint64_t k = in.k ? in.k[in.k_off[p] + i] : (uint64_t)i + 1;
        const uint64_t r = b.n - k;
        rmin = std::min(rmin, r);
        rmax = std::max(rmax, r);
      }
      if (b.n > 8ull * kBMaxS && rmax - rmin + 1 <= b.n / 32) {
        b.spec = 1;
        b.spec_lo = (uint32_t)rmin;
        b.spec_hi = (uint32_t)rmax;
      }
    }
    b.lut_off = lut_words;
    lut_words += ((1u << nsl_bits) + 1 + 3) & ~3u;
    b.cnt_off = cnt_words;
    cnt_words += nbm;
    b.row0 = row_words;
    row_words += (uint64_t)b.ntiles * nbm;
    num_tiles += b.ntiles;
    surv_est += std::min<uint64_t>(b.n, (uint64_t)nr * 4 * ((b.n + nbm - 1) / nbm) + 64);
    probs.push_back(b);
    orig.push_back(p);
  }
  const uint32_t P = (uint32_t)probs.size();
  if (P == 0) return GGKS_OK;
  // tiles, largest first, so that the end of each tile phase has the small ones
  std::vector<BTile> tiles;
  tiles.reserve(num_tiles);
  for (uint32_t q = 0; q < P; ++q)
    for (uint32_t r = 0; r < probs[q].ntiles; ++r) {
      BTile t{};
      t.begin = (uint64_t)r * tile;
      t.end = std::min<uint64_t>(probs[q].n, t.begin + tile);
      t.prob = q;
      t.rank = r;
      tiles.push_back(t);
    }
  std::stable_sort(tiles.begin(), tiles.end(), [](const BTile &a, const BTile &b) {
    return (a.end - a.begin) > (b.end - b.begin);
  });
  // candidate areas of speculating problems' tiles: the window and the
  // thresholds' margins (as the kernel places them) spread over the tiles in
  // proportion to their length, with half again and 256 keys to spare; a tile
  // that sees more reads its elements in the compaction phase
  uint64_t cand_words = 0;
  for (BTile &t : tiles) {
    const BProb &b = probs[t.prob];
    t.cand_off = cand_words;
    t.cand_cap = 0;
    if (!b.spec) continue;
    constexpr double CH = 32.0 / sizeof(T);
    const double S = b.S, fc = b.S / CH, n = (double)b.n;
    auto margin = [&](double q) { return CH * (4.0 * std::sqrt(fc * q * (1.0 - q)) + 2.0) + 1.0; };
    const double pl = b.spec_lo / n, ph = (b.spec_hi + 1.0) / n;
    const double expect = (b.spec_hi - b.spec_lo + 1.0) + (margin(pl) + margin(ph)) * n / S;
    const double len = (double)(t.end - t.begin);
    const uint64_t cap = std::min<uint64_t>(t.end - t.begin, (uint64_t)(expect * len / n * 1.5) + 256);
    t.cand_cap = (uint32_t)((cap + 3) & ~3ull);
    cand_words += t.cand_cap;
  }

  // ---- workspace: [ctrl | probs | tiles | reqs] is uploaded in one copy
  const size_t A = 256;
  static_assert(sizeof(BCtrl) <= A, "the control block fills one aligned slot");
  size_t o = 0;
  auto arr = [&](size_t elems, size_t esz) {
    const size_t at = o;
    o = balign(o + elems * esz, A);
    return at;
  };
  const size_t o_ctrl = arr(1, A);
  const size_t o_probs = arr(P, sizeof(BProb));
  const size_t o_tiles = arr(num_tiles, sizeof(BTile));
  const size_t o_reqs = arr(R, sizeof(Req));
  const size_t up_bytes = o;
  const size_t o_hdrs = arr(P, sizeof(BHdr));
  const size_t o_luts = arr(lut_words, 4);
  const size_t o_rows = arr(row_words, 4);
  const size_t o_reps = arr(row_words, sizeof(K));
  const size_t o_counts = arr(cnt_words, 4);
  const size_t o_req_bucket = arr(R, 4), o_req_local = arr(R, 4);
  const size_t o_seg_bucket = arr(R, 4), o_seg_size = arr(R, 4), o_kstart = arr(R, 4),
               o_kcnt = arr(R, 4), o_kcur = arr(R, 4), o_fill = arr(R, 4);
  const size_t o_seg_off = arr(R, 8), o_seg_lo = arr(R, sizeof(K)), o_seg_hi = arr(R, sizeof(K));
  const size_t o_klist = arr(R, sizeof(Req)), o_deferred = arr(R, 4);
  const size_t o_big = arr(R, 4), o_small = arr(R, 4), o_wsel = arr(R, 4),
               o_retry = arr(R, 4);
  const size_t o_out = arr(R, sizeof(T));
  const size_t o_cand = arr(cand_words, sizeof(K)), o_ccnt = arr(num_tiles, 4);
  const size_t total = o;

  cudaError_t e = ensure_buffer(ctx, &ctx.barena, &ctx.barena_bytes, total);
  if (e != cudaSuccess) return from_cuda(e);
  const size_t out_bytes = (size_t)R * sizeof(T);
  e = ensure_pinned(ctx, &ctx.bpin, &ctx.bpin_bytes, up_bytes + A + out_bytes);
  if (e != cudaSuccess) return from_cuda(e);
  uint64_t surv_cap = std::max<uint64_t>(surv_est, 1u << 20);
  if (ctx.surv_bytes / sizeof(K) > surv_cap) surv_cap = ctx.surv_bytes / sizeof(K);
  e = ensure_surv(ctx, (size_t)surv_cap * sizeof(K));
  if (e != cudaSuccess) return from_cuda(e);

  char *hp = ctx.bpin;
  std::memset(hp, 0, A);
  std::memcpy(hp + o_probs, probs.data(), (size_t)P * sizeof(BProb));
  std::memcpy(hp + o_tiles, tiles.data(), (size_t)num_tiles * sizeof(BTile));
  Req *hr = reinterpret_cast<Req *>(hp + o_reqs);
  for (uint32_t q = 0; q < P; ++q) {
    const uint32_t p = orig[q];
    const uint64_t n = probs[q].n;
    const uint32_t off = in.k_off[p], nr = probs[q].num_req;
    for (uint32_t i = 0; i < nr; ++i) {
      // k-th largest (1-based) is ascending rank n - k; top-k output i is
      // the (i + 1)-th largest
      const uint64_t k = in.k ? in.k[off + i] : (uint64_t)i + 1;
      hr[off + i].rank = (uint32_t)(n - k);
      hr[off + i].out = off + i;
    }
  }
  char *D = ctx.barena;
  BCtrl *ctrl = reinterpret_cast<BCtrl *>(D + o_ctrl);
  char *h_ctrl = hp + up_bytes;
  T *h_res = reinterpret_cast<T *>(hp + up_bytes + A);
  e = cudaMemcpyAsync(D, hp, up_bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return from_cuda(e);

  T *d_out = d_out_user ? d_out_user : reinterpret_cast<T *>(D + o_out);
  BArgs a{};
  a.probs = reinterpret_cast<const BProb *>(D + o_probs);
  a.hdrs = reinterpret_cast<BHdr *>(D + o_hdrs);
  a.tiles = reinterpret_cast<const BTile *>(D + o_tiles);
  a.num_probs = P;
  a.num_tiles = num_tiles;
  a.num_req = R;
  a.bcap = bcap;
  a.lut_words = lut_words;
  a.row_words = row_words;
  a.cnt_words = cnt_words;
  a.luts = reinterpret_cast<uint32_t *>(D + o_luts);
  a.rows = reinterpret_cast<uint32_t *>(D + o_rows);
  a.reps = D + o_reps;
  a.counts = reinterpret_cast<uint32_t *>(D + o_counts);
  a.reqs = reinterpret_cast<const Req *>(D + o_reqs);
  a.req_bucket = reinterpret_cast<uint32_t *>(D + o_req_bucket);
  a.req_local = reinterpret_cast<uint32_t *>(D + o_req_local);
  a.seg_bucket = reinterpret_cast<uint32_t *>(D + o_seg_bucket);
  a.seg_size = reinterpret_cast<uint32_t *>(D + o_seg_size);
  a.kstart = reinterpret_cast<uint32_t *>(D + o_kstart);
  a.kcnt = reinterpret_cast<uint32_t *>(D + o_kcnt);
  a.kcur = reinterpret_cast<uint32_t *>(D + o_kcur);
  a.fill = reinterpret_cast<uint32_t *>(D + o_fill);
  a.seg_off = reinterpret_cast<uint64_t *>(D + o_seg_off);
  a.seg_lo = D + o_seg_lo;
  a.seg_hi = D + o_seg_hi;
  a.klist = reinterpret_cast<Req *>(D + o_klist);
  a.big_list = reinterpret_cast<uint32_t *>(D + o_big);
  a.small_list = reinterpret_cast<uint32_t *>(D + o_small);
  a.wsel_list = reinterpret_cast<uint32_t *>(D + o_wsel);
  a.retry_list = reinterpret_cast<uint32_t *>(D + o_retry);
  a.deferred = reinterpret_cast<uint32_t *>(D + o_deferred);
  a.out = d_out;
  a.cand = D + o_cand;
  a.cand_cnt = reinterpret_cast<uint32_t *>(D + o_ccnt);
  a.ctrl = ctrl;


  // every CTA the SMs hold at once, or fewer when the batch has less work
  // (each grid barrier waits for every CTA)
  const uint32_t work = std::max(std::max(num_tiles, P), R / 8);
  const uint32_t grid_want = std::max(1u, std::min(max_grid, work));

  float ms_total = 0.f;
  // the results come back with the control block (one synchronisation); a
  // rerun or a deferred slot makes them stale and they are copied again
  bool res_fresh = false;
  auto launch = [&]() -> cudaError_t {
    a.surv = ctx.surv;
    a.surv_cap = surv_cap;
    void *args[] = {&a};
    if (ctx.bev0 == nullptr) {
      cudaError_t r = cudaEventCreate(&ctx.bev0);
      if (r == cudaSuccess) r = cudaEventCreate(&ctx.bev1);
      if (r != cudaSuccess) return r;
    }
    // with a chain (a server's lanes), the kernel is queued on the device
    // right behind the newest batched kernel of any lane
    const uint32_t grid = grid_want;
    ctx.stats.batch_grid = grid;
    std::unique_lock<std::mutex> chain_lk;
    if (ctx.chain) {
      chain_lk = std::unique_lock<std::mutex>(ctx.chain->mu);
      if (ctx.chain->last) {
        if (cudaEventQuery(ctx.chain->last) == cudaErrorNotReady) ctx.chain->queued++;
        const cudaError_t we = cudaStreamWaitEvent(s, ctx.chain->last, 0);
        if (we != cudaSuccess) return we;
      }
    }
    cudaEventRecord(ctx.bev0, s);
    cudaError_t r = cudaLaunchCooperativeKernel((const void *)k_batch<T>, dim3(grid), dim3(kBThreads),
                                                args, (size_t)smem, s);
    ctx.last_launch_wall = std::chrono::steady_clock::now();
    cudaEventRecord(ctx.bev1, s);
    if (ctx.chain) {
      if (r == cudaSuccess) ctx.chain->last = ctx.bev1;
      chain_lk.unlock();
    }
    ctx.stats.launches++;
    if (r != cudaSuccess) {
      cudaStreamSynchronize(s);
      return r;
    }
    r = cudaMemcpyAsync(h_ctrl, ctrl, sizeof(BCtrl), cudaMemcpyDeviceToHost, s);
    if (r == cudaSuccess && h_out) {
      r = cudaMemcpyAsync(h_res, d_out, out_bytes, cudaMemcpyDeviceToHost, s);
      res_fresh = r == cudaSuccess;
    }
    const cudaError_t rs = cudaStreamSynchronize(s);
    if (r == cudaSuccess) r = rs;
    float ms = 0.f;
    if (r == cudaSuccess && cudaEventElapsedTime(&ms, ctx.bev0, ctx.bev1) == cudaSuccess)
      ms_total += ms;
    if (r == cudaSuccess && ctx.time_base &&
        cudaEventElapsedTime(&ctx.last_launch_t0, ctx.time_base, ctx.bev0) == cudaSuccess)
      ctx.last_launch_t1 = ctx.last_launch_t0 + ms;
    return r;
  };
  e = launch();
  if (e != cudaSuccess) return from_cuda(e);

  for (int round = 0;; ++round) {
    BCtrl c;
    std::memcpy(&c, h_ctrl, sizeof(BCtrl));
#ifdef GGKS_BATCH_TIMING
    fprintf(stderr, "ggks batch timing: %u problems, gather %.0f cycles/problem, table %.0f cycles/problem\n",
            P, (double)c.dbg_a / P, (double)c.dbg_b / P);
#endif
#ifdef GGKS_BATCH_CHECKS
    if (c.dbg_code)
      fprintf(stderr, "ggks batch index check %u failed: %llu %llu (status %u)\n", c.dbg_code,
              (unsigned long long)c.dbg_a, (unsigned long long)c.dbg_b, c.status);
#endif
    if (c.status & ST_FATAL) return (c.status & ST_TIMEOUT) ? GGKS_TIMEOUT : GGKS_INTERNAL;
    if (c.status & ST_OVERFLOW) {
      if (round >= 3) return GGKS_INTERNAL;
      // survivors did not fit: grow the buffer and run the batch again
      surv_cap = c.cap_needed + (c.cap_needed >> 3);
      e = ensure_surv(ctx, (size_t)surv_cap * sizeof(K));
      if (e != cudaSuccess) return from_cuda(e);
      ctx.stats.retries++;
      e = cudaMemsetAsync(ctrl, 0, sizeof(BCtrl), s);
      if (e == cudaSuccess) e = launch();
      if (e != cudaSuccess) return from_cuda(e);
      continue;
    }
    for (int ph = 0; ph < kBPhases; ++ph)
      if (c.t_ns[ph + 1] >= c.t_ns[ph]) ctx.stats.batch_phase_ms[ph] += (c.t_ns[ph + 1] - c.t_ns[ph]) * 1e-6;
    ctx.stats.survivors += c.surv_top;
    ctx.stats.batch_spec_tiles += c.spec_tiles;
    if (c.status & ST_DEFERRED) {
      // slots whose needed bins exceed shared memory: select each again on
      // its survivor keys (recursively, single-vector path)
      res_fresh = false;
      const uint32_t Dn = c.deferred_count;
      std::vector<uint32_t> dl(Dn);
      e = cudaMemcpyAsync(dl.data(), a.deferred, (size_t)Dn * 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return from_cuda(e);
      int st = GGKS_OK;
      Context *ch = child_of(ctx, &st);
      if (!ch) return st;
      for (uint32_t d = 0; d < Dn; ++d) {
        const uint32_t g = dl[d];
        uint64_t so = 0;
        uint32_t sz = 0, ks = 0, kc = 0;
        e = cudaMemcpyAsync(&so, a.seg_off + g, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&sz, a.seg_size + g, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&ks, a.kstart + g, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&kc, a.kcnt + g, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return from_cuda(e);
        ReqSource cs;
        cs.d_reqs = a.klist + ks;
        ctx.stats.recursions++;
        st = select<K, T>(*ch, reinterpret_cast<const K *>(ctx.surv) + so, sz, cs, kc, d_out,
                          nullptr, s, nullptr);
        if (st != GGKS_OK) return st;
      }
    }
    break;
  }
  if (h_out) {
    if (!res_fresh) {
      e = cudaMemcpyAsync(h_res, d_out, out_bytes, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return from_cuda(e);
    }
    std::memcpy(h_out, h_res, out_bytes);
    // float32 problems of a uint32 batch: keys back to float32 bits
    if (in.is_float)
      for (uint32_t p = 0; p < in.num_problems; ++p)
        if (in.is_float[p])
          for (uint32_t i = in.k_off[p]; i < in.k_off[p + 1]; ++i) {
            uint32_t &v = reinterpret_cast<uint32_t *>(h_out)[i];
            v ^= ((v >> 31) - 1u) | 0x80000000u;
          }
  }
  if (kernel_ms) *kernel_ms = ms_total;
  ctx.stats.batch_calls++;
  ctx.stats.batch_problems += P;
  return GGKS_OK;
}

}  // namespace ggks
