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
//             threshold tau (a radix select among the samples of the
//             fine slice holding that rank);
//   k_filter  streams the vector once: each key >= tau is appended to one
//             contiguous candidate array, nothing else is written;
//   k_pick    one CTA: a 4096-bin histogram of the candidates over their key
//             range, the bin holding the K-th largest, a gather of every
//             candidate from that bin up into shared memory, a bitonic sort,
//             and the K largest out in descending order.
// Correctness never rests on the prediction: k_pick checks that every
// candidate was kept and that there are at least K, and that the gathered
// keys fit; else it flags ST_TOPK_MISS and the caller runs the pipeline.
#pragma once

#include <type_traits>

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
  __shared__ uint32_t s_rcnt[256], s_rsel[2];
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
  // every thread's counts before the CTA reports done (the fence below is
  // cumulative over what the barrier ordered)
  __syncthreads();
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
  // the samples of that fine slice; their r-th smallest is tau.  Eight
  // 128-bit loads per thread in flight before their compares (a load and a
  // shared atomic in one loop body would complete one at a time): 65 536
  // four-byte samples take two rounds.  The sample array starts 256-byte aligned; keys
  // past its last whole vector are read one by one.
  using SV = typename std::conditional<sizeof(K) == 4, uint4, ulonglong2>::type;
  constexpr uint32_t PV = 16 / sizeof(K);
  const uint32_t nv = S / PV;
  const SV *sv = reinterpret_cast<const SV *>(samples);
  // the slice holds a few dozen samples: a lane that finds one takes its
  // place with its own shared atomic (no vote per key)
  auto take = [&](K key, bool valid) {
    if (valid && (uint32_t)((key - kmin) >> fsh) == jf) {
      const uint32_t at = atomicAdd(&s_cnt, 1u);
      if (at < kTauBuf) buf[at] = key;
    }
  };
  for (uint32_t v0 = tid; v0 < nv; v0 += 8 * blockDim.x) {
    SV xs[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint32_t q = v0 + u * blockDim.x;
      if (q < nv) xs[u] = __ldcg(sv + q);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool ok = v0 + u * blockDim.x < nv;
      if constexpr (sizeof(K) == 4) {
        take(ok ? (K)xs[u].x : kmin, ok);
        take(ok ? (K)xs[u].y : kmin, ok);
        take(ok ? (K)xs[u].z : kmin, ok);
        take(ok ? (K)xs[u].w : kmin, ok);
      } else {
        take(ok ? (K)xs[u].x : kmin, ok);
        take(ok ? (K)xs[u].y : kmin, ok);
      }
    }
  }
  for (uint32_t q = nv * PV + tid; q < S; q += blockDim.x) take(__ldcg(samples + q), true);
  __syncthreads();
  const uint32_t cnt = s_cnt;
  K t;
  if (open) {
    t = K(0);
  } else if (cnt > kTauBuf || r >= cnt) {
    t = kmin + ((K)jf << fsh);  // the fine slice's first key: a lower threshold
  } else {
    // the r-th smallest of the slice's samples by radix select (16 block
    // barriers for 4-byte keys; a bitonic sort of up to 2048 keys took 66)
    t = cta_select_rank<K>(buf, cnt, r, s_rcnt, s_rsel);
  }
  if (tid == 0) {
    *tau = t;
    ctrl->sample_done = 0;  // re-arm for the next call on this workspace
  }
}

// ---------------------------------------------------------------------------
// k_filter: one pass, keys >= tau appended to one contiguous array
// ---------------------------------------------------------------------------
// Each warp collects its candidates in a 256-key buffer in shared memory and
// moves a buffer that could fill up to the candidate array with one atomic on
// the array's length (cand_next); at the end the CTA's warps move what is left
// with one atomic for the whole CTA.  The candidates are thus one contiguous
// array [0, C), which k_pick reads with coalesced loads (one SM gathering
// scattered 4-byte candidates from per-warp lists was bound by its outstanding
// misses: 43 us for 20 000 keys).  Keys past the array's capacity are counted
// but not written (k_pick then reports a miss).  INGEST: x is a mapped host
// vector, also written to copy_to (the device copy, same alignment modulo 16
// bytes).
constexpr uint32_t kFiltBuf = 256;  // keys of one warp's buffer

template <class K>
struct FiltWarp {
  K *buf;           // this warp's kFiltBuf keys in shared memory
  uint32_t cnt = 0;  // keys in buf (warp-uniform)
  K *arr;           // the candidate array
  uint64_t cap;     // its capacity
  uint32_t *len;    // its length (global)
  // moves the buffer to the array (the whole warp calls this)
  __device__ __forceinline__ void flush() {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(len, cnt);
    base = __shfl_sync(0xffffffffu, base, 0);
    __syncwarp();
    for (uint32_t i = lane; i < cnt; i += 32)
      if ((uint64_t)base + i < cap) arr[base + i] = buf[i];
    __syncwarp();
    cnt = 0;
  }
  // every lane calls this with its key and whether it keeps it
  __device__ __forceinline__ void put(K k, bool keep) {
    const uint32_t m = __ballot_sync(0xffffffffu, keep);
    if (!m) return;
    if (cnt > kFiltBuf - 32) flush();
    const uint32_t lane = threadIdx.x & 31;
    if (keep) buf[cnt + __popc(m & ((1u << lane) - 1u))] = k;
    cnt += __popc(m);
  }
};

template <class T, int UNROLL, bool INGEST>
__device__ __forceinline__ void filter_body(const T *__restrict__ x, uint64_t n,
                                            typename Traits<T>::K t, T *__restrict__ copy_to,
                                            FiltWarp<typename Traits<T>::K> &fw) {
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
        for (int e = 0; e < PV; ++e) fw.put(k[e], k[e] >= t);
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
      for (int e = 0; e < PV; ++e) fw.put(k[e], valid && k[e] >= t);
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
        fw.put(k, valid && k >= t);
      }
    };
    scalar(0, sp.head);
    scalar(sp.tail0, n);
  }
}

// Grid and tiles as k_hist; 1024 threads; dynamic shared memory
// kCandWarps * kFiltBuf keys.  arr[0 .. cap) receives the candidates and
// *len (zero on entry) their count.
template <class T, int UNROLL>
__global__ void __launch_bounds__(1024, 1)
    k_filter(const T *__restrict__ x, uint64_t n, const typename Traits<T>::K *tau,
             typename Traits<T>::K *__restrict__ arr, uint64_t cap, uint32_t *len,
             T *__restrict__ copy_to, const Ctrl *ctrl) {
  pdl_start();
  using K = typename Traits<T>::K;
  extern __shared__ uint4 smem_raw[];
  __shared__ uint32_t s_wcnt[kCandWarps];
  __shared__ uint32_t s_base;
  if (ctrl->status & ST_FATAL) return;
  const K t = *tau;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  FiltWarp<K> fw;
  fw.buf = reinterpret_cast<K *>(smem_raw) + warp * kFiltBuf;
  fw.arr = arr;
  fw.cap = cap;
  fw.len = len;
  if (copy_to)
    filter_body<T, UNROLL, true>(x, n, t, copy_to, fw);
  else
    filter_body<T, UNROLL, false>(x, n, t, nullptr, fw);
  // what the warps hold: one atomic for the CTA
  if (lane == 0) s_wcnt[warp] = fw.cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (uint32_t w = 0; w < kCandWarps; ++w) {
      const uint32_t c = s_wcnt[w];
      s_wcnt[w] = tot;
      tot += c;
    }
    s_base = tot ? atomicAdd(len, tot) : 0u;
  }
  __syncthreads();
  const uint64_t base = (uint64_t)s_base + s_wcnt[warp];
  for (uint32_t i = lane; i < fw.cnt; i += 32)
    if (base + i < cap) arr[base + i] = fw.buf[i];
}

// ---------------------------------------------------------------------------
// k_pick: the K largest of the candidates
// ---------------------------------------------------------------------------
// One CTA of 1024 threads over the contiguous candidate array arr[0, C)
// (coalesced reads).  When C fits the stage (kStage keys) the candidates are
// copied into shared memory once and every later pass reads them there.
// Dynamic shared memory: the histogram and the bins' offsets (kPickBins words
// each), the stage and the sort buffer (kPickCap keys).  out[i] = the (i + 1)-th largest, i < kk.
template <class K>
struct PickShape {
  static constexpr uint32_t kStage = sizeof(K) == 4 ? 36864u : 14336u;
};
constexpr uint32_t kPickBinSort = 32;  // largest bin sorted by one thread
template <class K>
__host__ __device__ constexpr size_t pick_smem_bytes() {
  return (size_t)2 * kPickBins * sizeof(uint32_t) +
         ((size_t)PickShape<K>::kStage + kPickCap) * sizeof(K) + 16;
}

template <class K, class OutT>
__global__ void __launch_bounds__(1024, 1)
    k_pick(const K *__restrict__ arr, uint64_t cap, const uint32_t *len, const K *tau, uint32_t kk,
           OutT *__restrict__ out, Ctrl *ctrl) {
  pdl_start();
  constexpr uint32_t kStage = PickShape<K>::kStage;
  extern __shared__ uint4 smem_raw[];
  uint32_t *hist = reinterpret_cast<uint32_t *>(smem_raw);  // kPickBins
  uint32_t *off = hist + kPickBins;                          // kPickBins
  K *stage = reinterpret_cast<K *>(off + kPickBins);         // 16-byte aligned
  K *buf = stage + kStage;                                   // kPickCap
  __shared__ uint32_t red32[33];
  __shared__ K redk[33];
  __shared__ uint32_t s_j, s_above, s_cnt;
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  if (ctrl->status & ST_FATAL) return;
  const uint32_t C = __ldcg(len);
  const K t = *tau;
  for (uint32_t b = tid; b < kPickBins; b += nt) hist[b] = 0;
  if ((uint64_t)C > cap || C < kk) {  // candidates lost past the capacity, or too few
    if (tid == 0) atomicOr(&ctrl->status, ST_TOPK_MISS);
    return;
  }
  const bool staged = C <= kStage;
  // every candidate once: fn(key); eight loads per thread in flight
  auto each = [&](auto &&fn) {
    if (staged) {
      for (uint32_t i = tid; i < C; i += nt) fn(stage[i]);
      return;
    }
    for (uint32_t i0 = tid; i0 < C; i0 += 8 * nt) {
      K kv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) kv[u] = i0 + u * nt < C ? __ldcg(arr + i0 + u * nt) : K(0);
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (i0 + u * nt < C) fn(kv[u]);
    }
  };
  K mx = 0;
  if (staged) {
    for (uint32_t i0 = tid; i0 < C; i0 += 8 * nt) {
      K kv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) kv[u] = i0 + u * nt < C ? __ldcg(arr + i0 + u * nt) : K(0);
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (i0 + u * nt < C) {
          stage[i0 + u * nt] = kv[u];
          mx = kv[u] > mx ? kv[u] : mx;
        }
    }
  } else {
    each([&](K k) { mx = k > mx ? k : mx; });
  }
  mx = block_reduce(mx, [](K p, K q) { return p > q ? p : q; }, redk);  // also orders the stage
  const int bl = bitlen<K>(mx - t);
  const uint32_t sh = bl > 12 ? (uint32_t)(bl - 12) : 0u;
  each([&](K k) { atomicAdd(&hist[min((uint32_t)((k - t) >> sh), kPickBins - 1u)], 1u); });
  __syncthreads();
  // the bin holding the kk-th largest: counts from the top, 4 bins per
  // thread; off[b] = candidates in the bins above b (their place in
  // descending order)
  uint32_t maxc = 0;
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
      const uint32_t b = 4 * tid + q;
      if (b < kPickBins) off[kPickBins - 1 - b] = above;
      if (above < kk && kk <= above + c4[q]) {
        s_j = kPickBins - 1 - (4 * tid + q);
        s_above = above;
      }
      // a bin holding one of the kk largest and sorted here (not the
      // kk-th's bin when it is one key wide)
      if (above < kk && !(sh == 0 && kk <= above + c4[q])) maxc = max(maxc, c4[q]);
      above += c4[q];
    }
    if (tid == 0) s_cnt = 0;
  }
  maxc = block_reduce(maxc, [](uint32_t p, uint32_t q) { return p > q ? p : q; }, red32);
  const uint32_t j = s_j, above = s_above;
  const uint32_t in_j = hist[j];
  // one key in bin j (a bin one key wide): only the bins above are gathered
  const bool single = sh == 0;
  const uint32_t need = single ? above : above + in_j;
  if (need > kPickCap) {
    if (tid == 0) atomicOr(&ctrl->status, ST_TOPK_MISS);
    return;
  }
  // Bins of at most kPickBinSort keys: each key goes to its bin's place in
  // descending order (the bin's count, counted down, numbers its keys), and
  // one thread sorts each bin's few keys.  Otherwise the gathered keys are
  // sorted together (bitonic).
  const bool by_bin = maxc <= kPickBinSort;
  each([&](K k) {
    const uint32_t b = min((uint32_t)((k - t) >> sh), kPickBins - 1u);
    const bool in = single ? b > j : b >= j;
    if (by_bin) {
      if (in) buf[off[b] + atomicSub(&hist[b], 1u) - 1u] = k;
    } else {
      const uint32_t at = warp_append(&s_cnt, in);
      if (in) buf[at] = k;
    }
  });
  __syncthreads();
  if (by_bin) {
    // bins j .. kPickBins - 1 (j + 1 .. in the single-key case), each sorted
    // descending in place by one thread (insertion sort)
    for (uint32_t b = (single ? j + 1 : j) + tid; b < kPickBins; b += nt) {
      const uint32_t lo = off[b];
      const uint32_t hi = b ? off[b - 1] : need;
      for (uint32_t q = lo + 1; q < hi; ++q) {
        const K v = buf[q];
        uint32_t r = q;
        while (r > lo && buf[r - 1] < v) {
          buf[r] = buf[r - 1];
          --r;
        }
        buf[r] = v;
      }
    }
    __syncthreads();
    for (uint32_t i = tid; i < kk; i += nt) {
      const K k = (single && i >= above) ? (K)(t + (K)j) : buf[i];
      out[i] = Traits<OutT>::value(k);
    }
    return;
  }
  const uint32_t got = s_cnt;  // == need
  uint32_t P = 1;
  while (P < got) P <<= 1;
  for (uint32_t q = got + tid; q < P; q += nt) buf[q] = K(0);
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
