// ggks_topk.cuh -- top-k by a sampled threshold: one streaming pass keeps the
// elements at or above a threshold taken from the sample, and one CTA selects
// the K largest of those candidates.
//
// The reference computes top-k as a multiselect of k = 1..K
// (multiselectTimingFunctions.cu:205-231: timeBucketTopkselect builds the k
// list and calls the bucket multiselect, bucketMultiselect.cu:837-871), which
// here is the histogram / plan / compaction / finish pipeline.  For K up to
// kPickMax the K largest are found with less work:
//   k_sample  the sample (shared with the pipeline);
//   k_tau     bins the samples in 4096 fine slices of their span (as k_lut
//             does); the last CTA finds the sample rank below which the K-th
//             largest element's sample rank lies with overwhelming
//             probability (the rank of the K-th largest among S samples is
//             about Binomial(S, 1 - K / n); six standard deviations plus four
//             below its mean) and takes the sample key of that rank as the
//             threshold tau;
//   k_filter  streams the vector once: each key >= tau goes to its warp's
//             candidate list (chunks of the pool), nothing else is written;
//   k_pick    one CTA: a 4096-bin histogram of the candidates over their key
//             range, the bin holding the K-th largest, a gather of every
//             candidate from that bin up into shared memory, a bitonic sort,
//             and the K largest out in descending order.
// Correctness never rests on the prediction: k_pick checks that the lists are
// complete and hold at least K keys, and that the gathered keys fit; else it
// flags ST_TOPK_MISS and the caller runs the pipeline instead.
#pragma once

#include "ggks_device.cuh"

namespace ggks {

constexpr uint32_t kPickMax = 4096;     // largest K of the threshold path
constexpr uint32_t kPickBins = 4096;    // k_pick's histogram
constexpr uint32_t kPickCap = 8192;     // keys k_pick gathers and sorts at most
constexpr uint32_t kTauBuf = 2048;      // samples of the threshold's fine slice k_tau sorts

// ---------------------------------------------------------------------------
// k_tau: the threshold from the sample
// ---------------------------------------------------------------------------
// Grid: ceil(S / 1024) CTAs of 1024 threads, after k_sample (span in Ctrl).
// slice_cnt (global, kLutIdx words) is zero on entry and left zero.  The last
// CTA writes tau (0: no useful threshold, which the caller treats as a miss).
template <class K>
__global__ void __launch_bounds__(1024) k_tau(const K *__restrict__ samples, uint32_t S, Ctrl *ctrl,
                                              uint32_t *slice_cnt, uint64_t n, uint32_t kk,
                                              K *tau) {
  pdl_start();
  __shared__ uint32_t red32[33];
  __shared__ uint32_t s_last, s_jf, s_r, s_cnt;
  __shared__ uint32_t ccnt[kLutIdx];
  __shared__ K buf[kTauBuf];
  const uint32_t tid = threadIdx.x;
  const uint32_t i = blockIdx.x * blockDim.x + tid;
  for (uint32_t j = tid; j < kLutIdx; j += blockDim.x) ccnt[j] = 0;
  const K k = i < S ? __ldcg(samples + i) : K(0);
  const K kmin = (K)~__ldcg((const unsigned long long *)&ctrl->kmin_inv);
  const K kmax = (K)__ldcg((const unsigned long long *)&ctrl->kmax);
  const int bl = bitlen<K>(kmax - kmin);
  const uint32_t fsh = bl > kLutIdxBits ? (uint32_t)(bl - kLutIdxBits) : 0u;
  __syncthreads();
  if (i < S) atomicAdd(&ccnt[(uint32_t)((k - kmin) >> fsh)], 1u);
  __syncthreads();
  for (uint32_t j = tid; j < kLutIdx; j += blockDim.x) {
    const uint32_t c = ccnt[j];
    if (c) atomicAdd(&slice_cnt[j], c);
  }
  if (tid == 0) {
    __threadfence();
    s_last = (atomicAdd(&ctrl->sample_done, 1u) == gridDim.x - 1) ? 1u : 0u;
    if (s_last) __threadfence();
  }
  __syncthreads();
  if (!s_last) return;

  // the sample rank below the K-th largest's, with six standard deviations and
  // four ranks to spare (single precision: ranks need about one unit of 2^16)
  const float dS = (float)S;
  const float pl = (float)(n - kk) / (float)n;
  const float a = pl * dS - (6.0f * sqrtf(dS * pl * (1.0f - pl)) + 4.0f);
  const bool open = !(a > 0.0f);  // the window reaches the smallest sample
  const uint32_t wa = open ? 0u : (a >= dS - 1.0f ? S - 1u : (uint32_t)a);
  // fine slice holding sample rank wa (4 fine slices per thread, in order)
  const uint32_t per = kLutIdx / blockDim.x;
  uint32_t fc[4], fsum = 0;
#pragma unroll
  for (uint32_t q = 0; q < 4; ++q) {
    const uint32_t j = per * tid + q;
    fc[q] = q < per ? __ldcg(slice_cnt + j) : 0u;
    if (q < per) slice_cnt[j] = 0;  // zero for the next call
    fsum += fc[q];
  }
  if (tid == 0) {
    s_jf = 0;
    s_r = 0;
    s_cnt = 0;
  }
  uint32_t ftot;
  uint32_t fpre = block_incl_scan(fsum, &ftot, red32) - fsum;
#pragma unroll
  for (uint32_t q = 0; q < 4; ++q) {
    if (q < per && fc[q] && fpre <= wa && wa < fpre + fc[q]) {
      s_jf = per * tid + q;
      s_r = wa - fpre;
    }
    fpre += fc[q];
  }
  __syncthreads();
  const uint32_t jf = s_jf, r = s_r;
  // the samples of that fine slice; their r-th smallest is tau (16 loads per
  // thread in flight before their compares: a load and a shared atomic in
  // one loop body would complete one at a time)
  for (uint32_t s0 = tid; s0 < S; s0 += 16 * blockDim.x) {
    K xs[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const uint32_t q = s0 + u * blockDim.x;
      xs[u] = q < S ? __ldcg(samples + q) : kmin;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      if (s0 + u * blockDim.x < S && (uint32_t)((xs[u] - kmin) >> fsh) == jf) {
        const uint32_t at = atomicAdd(&s_cnt, 1u);
        if (at < kTauBuf) buf[at] = xs[u];
      }
    }
  }
  __syncthreads();
  const uint32_t cnt = s_cnt;
  K t;
  if (open) {
    t = K(0);
  } else if (cnt > kTauBuf || r >= cnt) {
    t = kmin + ((K)jf << fsh);  // the fine slice's first key: a lower threshold
  } else {
    uint32_t P = 1;
    while (P < cnt) P <<= 1;
    for (uint32_t q = cnt + tid; q < P; q += blockDim.x) buf[q] = KeyMax<K>::v;
    __syncthreads();
    bitonic_sort_smem(buf, P);
    t = buf[r];
  }
  if (tid == 0) {
    *tau = t;
    ctrl->sample_done = 0;  // re-arm for the next call on this workspace
  }
}

// ---------------------------------------------------------------------------
// k_filter: one pass, keys >= tau into per-warp candidate lists
// ---------------------------------------------------------------------------
// Same tiles and lists as k_hist's speculative candidates (cand_put_warp):
// warp w of CTA c leaves its count in cand_cnt[c * kCandWarps + w] and its
// chunk table in cand_tab.  INGEST: x is a mapped host vector, also written to
// copy_to (the device copy, same alignment modulo 16 bytes).
template <class T, int UNROLL, bool INGEST>
__device__ __forceinline__ void filter_body(const T *__restrict__ x, uint64_t n,
                                            typename Traits<T>::K t, T *__restrict__ copy_to,
                                            const CandPool<typename Traits<T>::K> &cp,
                                            CandList &cl, uint32_t *wtab) {
  using K = typename Traits<T>::K;
  using V = typename Traits<T>::Vec;
  constexpr int PV = Traits<T>::kPerVec;
  const Span<T> sp = split_span(x, n);
  const V *xv = reinterpret_cast<const V *>(x + sp.head);
  V *cv = reinterpret_cast<V *>(copy_to + sp.head);
  const uint64_t tile_v = (uint64_t)blockDim.x * UNROLL;
  const uint64_t ntiles = sp.nvec / tile_v;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t off = tile * tile_v + threadIdx.x;
    V v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u)
      v[u] = INGEST ? xv[off + (uint64_t)u * blockDim.x] : ldg_stream(xv + off + (uint64_t)u * blockDim.x);
    if (INGEST) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) cv[off + (uint64_t)u * blockDim.x] = v[u];
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      K k[PV];
      vec_keys<T>(v[u], k);
      bool any = false;
#pragma unroll
      for (int e = 0; e < PV; ++e) any |= k[e] >= t;
      // one vote per vector; the per-key votes only when a lane keeps one
      if (__any_sync(0xffffffffu, any)) {
#pragma unroll
        for (int e = 0; e < PV; ++e) cand_put_warp<K>(cp, k[e], k[e] >= t, cl, wtab);
      }
    }
  }
  // leftover vectors and the scalar head / tail: every lane runs every round
  const uint32_t owner = (uint32_t)(ntiles % gridDim.x);
  if (blockIdx.x == owner) {
    for (uint64_t vb = ntiles * tile_v; vb < sp.nvec; vb += blockDim.x) {
      const uint64_t vi = vb + threadIdx.x;
      const bool valid = vi < sp.nvec;
      V vv{};
      if (valid) {
        vv = INGEST ? xv[vi] : ldg_stream(xv + vi);
        if (INGEST) cv[vi] = vv;
      }
      K k[PV];
      vec_keys<T>(vv, k);
#pragma unroll
      for (int e = 0; e < PV; ++e) cand_put_warp<K>(cp, k[e], valid && k[e] >= t, cl, wtab);
    }
    auto scalar = [&](uint64_t e0, uint64_t e1) {
      for (uint64_t eb = e0; eb < e1; eb += blockDim.x) {
        const uint64_t e = eb + threadIdx.x;
        const bool valid = e < e1;
        K k = 0;
        if (valid) {
          const T v = x[e];
          if (INGEST) copy_to[e] = v;
          k = Traits<T>::key(v);
        }
        cand_put_warp<K>(cp, k, valid && k >= t, cl, wtab);
      }
    };
    scalar(0, sp.head);
    scalar(sp.tail0, n);
  }
}

template <class T, int UNROLL>
__global__ void __launch_bounds__(1024, 1)
    k_filter(const T *__restrict__ x, uint64_t n, const typename Traits<T>::K *tau,
             typename Traits<T>::K *__restrict__ pool, uint32_t pool_chunks, uint32_t *cand_next,
             uint32_t *__restrict__ cand_cnt, uint32_t *__restrict__ cand_tab,
             T *__restrict__ copy_to, const Ctrl *ctrl) {
  pdl_start();
  using K = typename Traits<T>::K;
  __shared__ uint32_t s_wcnt[kCandWarps];
  __shared__ uint32_t s_tab[kCandWarps * kCandChunksPerWarp];
  if (ctrl->status & ST_FATAL) return;
  const K t = *tau;
  CandPool<K> cp;
  cp.pool = pool;
  cp.chunks = pool_chunks;
  cp.next = cand_next;
  CandList cl;
  const uint32_t warp = threadIdx.x >> 5;
  uint32_t *wt = s_tab + warp * kCandChunksPerWarp;
  if (copy_to)
    filter_body<T, UNROLL, true>(x, n, t, copy_to, cp, cl, wt);
  else
    filter_body<T, UNROLL, false>(x, n, t, nullptr, cp, cl, wt);
  if ((threadIdx.x & 31) == 0) s_wcnt[warp] = cl.count;
  __syncthreads();
  if (threadIdx.x < kCandWarps)
    cand_cnt[(uint64_t)blockIdx.x * kCandWarps + threadIdx.x] = s_wcnt[threadIdx.x];
  for (uint32_t i = threadIdx.x; i < kCandWarps * kCandChunksPerWarp; i += blockDim.x)
    cand_tab[(uint64_t)blockIdx.x * kCandWarps * kCandChunksPerWarp + i] = s_tab[i];
}

// ---------------------------------------------------------------------------
// k_pick: the K largest of the candidates
// ---------------------------------------------------------------------------
// One CTA of 1024 threads.  lists = G * kCandWarps candidate lists (at most
// kPickLists).  The candidates are numbered list after list (list offsets in
// shared memory); thread t takes the contiguous numbers [C t / T, C (t+1) / T)
// and walks its lists, with each list's first chunk index staged in shared
// memory (later chunks, of lists holding more than kCandChunk keys, are read
// from the chunk table).  When the C candidates fit the stage (kPickStage
// keys) one walk copies them there and every later pass reads shared memory;
// otherwise every pass walks the lists again.
//
// Dynamic shared memory: list offsets (kPickLists + 1 words), first chunks
// (kPickLists), the histogram (kPickBins), the stage (kPickStage keys) and the
// sort buffer (kPickCap keys).  out[i] = the (i + 1)-th largest, i < kk.
constexpr uint32_t kPickLists = 4864;  // 152 CTAs x 32 warps
template <class K>
struct PickShape {
  static constexpr uint32_t kStage = sizeof(K) == 4 ? 32768u : 12288u;
};
template <class K>
__host__ __device__ constexpr size_t pick_smem_bytes() {
  return ((size_t)kPickLists * 2 + 1 + kPickBins) * sizeof(uint32_t) +
         ((size_t)PickShape<K>::kStage + kPickCap) * sizeof(K) + 16;
}

template <class K, class OutT>
__global__ void __launch_bounds__(1024, 1)
    k_pick(const K *__restrict__ pool, uint32_t pool_chunks, const uint32_t *__restrict__ cand_cnt,
           const uint32_t *__restrict__ cand_tab, uint32_t lists, const K *tau, uint32_t kk,
           OutT *__restrict__ out, Ctrl *ctrl) {
  pdl_start();
  constexpr uint32_t kStage = PickShape<K>::kStage;
  extern __shared__ uint4 smem_raw[];
  uint32_t *loff = reinterpret_cast<uint32_t *>(smem_raw);  // kPickLists + 1
  uint32_t *first = loff + kPickLists + 1;                   // kPickLists
  uint32_t *hist = first + kPickLists;                       // kPickBins
  K *stage = reinterpret_cast<K *>(
      reinterpret_cast<uintptr_t>(hist + kPickBins + 3) & ~uintptr_t(15));
  K *buf = stage + kStage;  // kPickCap
  __shared__ uint32_t red32[33];
  __shared__ K redk[33];
  __shared__ bool s_miss;
  __shared__ uint32_t s_j, s_above, s_cnt;
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  if (ctrl->status & ST_FATAL) return;
  if (tid == 0) s_miss = lists > kPickLists;
  __syncthreads();
  if (s_miss) {
    if (tid == 0) atomicOr(&ctrl->status, ST_TOPK_MISS);
    return;
  }
  // list counts -> offsets (contiguous lists per thread); every list must be
  // complete; first chunks staged
  const uint32_t per = (lists + nt - 1) / nt;
  uint32_t mysum = 0;
  for (uint32_t q = 0; q < per; ++q) {
    const uint32_t L = tid * per + q;
    if (L >= lists) break;
    const uint32_t c = __ldcg(cand_cnt + L);
    const uint32_t nch = (c + kCandChunk - 1) / kCandChunk;
    if (nch > kCandChunksPerWarp) {
      s_miss = true;
    } else {
      for (uint32_t h = 0; h < nch; ++h) {
        const uint32_t ch = __ldcg(cand_tab + (uint64_t)L * kCandChunksPerWarp + h);
        if (ch >= pool_chunks) s_miss = true;
        if (h == 0) first[L] = ch;
      }
    }
    mysum += c;
  }
  uint32_t total;
  uint32_t run = block_incl_scan(mysum, &total, red32) - mysum;
  for (uint32_t q = 0; q < per; ++q) {
    const uint32_t L = tid * per + q;
    if (L >= lists) break;
    loff[L] = run;
    run += __ldcg(cand_cnt + L);
  }
  if (tid == 0) loff[lists] = total;
  for (uint32_t b = tid; b < kPickBins; b += nt) hist[b] = 0;
  __syncthreads();
  if (s_miss || total < kk) {
    if (tid == 0) atomicOr(&ctrl->status, ST_TOPK_MISS);
    return;
  }
  const uint32_t C = total;
  // walk: fn(candidate number, key) for this thread's contiguous numbers, four
  // loads in flight
  auto walk = [&](auto &&fn) {
    const uint32_t i0 = (uint32_t)((uint64_t)C * tid / nt);
    const uint32_t i1 = (uint32_t)((uint64_t)C * (tid + 1) / nt);
    if (i0 >= i1) return;
    uint32_t lo = 0, hi = lists;  // the list holding i0: last L with loff[L] <= i0
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (loff[mid] <= i0)
        lo = mid;
      else
        hi = mid;
    }
    uint32_t L = lo;
    for (uint32_t i = i0; i < i1; i += 4) {
      uint64_t at[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t idx = i + u;
        at[u] = 0;
        if (idx < i1) {
          while (idx >= loff[L + 1]) ++L;
          const uint32_t j = idx - loff[L];
          const uint32_t ch = j < kCandChunk
                                  ? first[L]
                                  : __ldcg(cand_tab + (uint64_t)L * kCandChunksPerWarp + j / kCandChunk);
          at[u] = (uint64_t)ch * kCandChunk + j % kCandChunk;
        }
      }
      K kv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) kv[u] = i + u < i1 ? __ldcg(pool + at[u]) : K(0);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i + u < i1) fn(i + u, kv[u]);
    }
  };
  const bool staged = C <= kStage;
  // every candidate once: fn(key)
  auto each = [&](auto &&fn) {
    if (staged) {
      for (uint32_t i = tid; i < C; i += nt) fn(stage[i]);
    } else {
      walk([&](uint32_t, K k) { fn(k); });
    }
  };
  const K t = *tau;
  K mx = 0;
  if (staged) {
    walk([&](uint32_t i, K k) {
      stage[i] = k;
      mx = k > mx ? k : mx;
    });
  } else {
    walk([&](uint32_t, K k) { mx = k > mx ? k : mx; });
  }
  mx = block_reduce(mx, [](K p, K q) { return p > q ? p : q; }, redk);  // also orders the stage
  const int bl = bitlen<K>(mx - t);
  const uint32_t sh = bl > 12 ? (uint32_t)(bl - 12) : 0u;
  each([&](K k) { atomicAdd(&hist[min((uint32_t)((k - t) >> sh), kPickBins - 1u)], 1u); });
  __syncthreads();
  // the bin holding the kk-th largest: counts from the top, 4 bins per thread
  {
    uint32_t c4[4], sum = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t b = 4 * tid + q;
      c4[q] = b < kPickBins ? hist[kPickBins - 1 - b] : 0u;
      sum += c4[q];
    }
    uint32_t tot;
    uint32_t above = block_incl_scan(sum, &tot, red32) - sum;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (above < kk && kk <= above + c4[q]) {
        s_j = kPickBins - 1 - (4 * tid + q);
        s_above = above;
      }
      above += c4[q];
    }
    if (tid == 0) s_cnt = 0;
  }
  __syncthreads();
  const uint32_t j = s_j, above = s_above;
  const uint32_t in_j = hist[j];
  // one key in bin j (a bin one key wide): only the bins above are gathered
  const bool single = sh == 0;
  const uint32_t need = single ? above : above + in_j;
  if (need > kPickCap) {
    if (tid == 0) atomicOr(&ctrl->status, ST_TOPK_MISS);
    return;
  }
  each([&](K k) {
    const uint32_t b = min((uint32_t)((k - t) >> sh), kPickBins - 1u);
    if (single ? b > j : b >= j) buf[atomicAdd(&s_cnt, 1u)] = k;
  });
  __syncthreads();
  const uint32_t cnt = s_cnt;  // == need
  uint32_t P = 1;
  while (P < cnt) P <<= 1;
  for (uint32_t q = cnt + tid; q < P; q += nt) buf[q] = K(0);
  __syncthreads();
  if (P > 1) bitonic_sort_smem(buf, P);  // ascending; the padding sorts first
  // descending: the (i + 1)-th largest is buf[P - 1 - i]; in the single-key
  // case ranks from `above` on are the bin's key
  for (uint32_t i = tid; i < kk; i += nt) {
    const K k = (single && i >= above) ? (K)(t + (K)j) : buf[P - 1 - i];
    out[i] = Traits<OutT>::value(k);
  }
}

}  // namespace ggks
