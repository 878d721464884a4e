// ggks_small.cuh -- the selection of a small vector in one launch.
//
// Below a few million elements the pipeline's seven dependent kernels cost
// about 70-95 us whatever the size (each pass's fixed latency, not its
// traffic).  Here one thread-block cluster of kSmCtas CTAs runs the same
// algorithm -- sample, range-adaptive splitter table, bucket histogram,
// k -> bucket plan, compaction of the requested buckets, in-shared-memory
// finish -- with cluster barriers between the phases and distributed shared
// memory for the exchanges, so nothing of the plan goes through global memory
// or the host:
//
//   A  every CTA samples the same keys (pairs of neighbouring elements at
//      hashed positions) and builds the same table with build_lut_cta, the
//      single-vector builder (512 slices, kSmNb buckets): no CTA waits for
//      another's table.
//   B  every CTA holds the table once per bank and counts its contiguous
//      share of the vector into one shared-memory word per bucket.
//   C  bucket b is owned by thread b % 1024 of CTA b / 1024: it sums the
//      bucket's counts over the cluster; a block scan and the CTAs' totals
//      give the bucket's global prefix (its elements' first rank).
//   D  each request is mapped by the CTA whose buckets hold its rank; the
//      owner of a bucket turns its count in every CTA into that CTA's first
//      survivor position -- prefix + the counts of the CTAs before it -- when
//      the bucket is requested, else into an inactive cursor.  A requested
//      bucket's survivors land at [prefix, prefix + count) of the survivor
//      buffer (n keys), the ranks they hold in the sorted vector, so no slot
//      numbering or allocation is needed.
//   E  every CTA compacts its share: one lookup, one shared atomic on the
//      bucket's cursor (inactive cursors carry bit 31), a predicated store.
//   F  the owners check that every CTA's cursor reached its end, then finish
//      their requested buckets: a warp per bucket of at most small_warp_cap
//      keys (finish_warp_select for up to four requests, else finish_warp);
//      the whole CTA for larger ones: a bitonic sort of
//      the segment in shared memory up to small_sort_cap keys, finish_slot
//      beyond.
//
// Anything this layout does not cover -- a bucket whose needed bins do not fit
// (finish_slot asks for a recursive level), cursors that did not reach their
// ends (the input changed between the passes) -- sets ST_SMALL_MISS and the
// host runs the pipeline instead; the outputs are then written again.  Every
// CTA passes every cluster barrier (no early exit), and no CTA reads another's
// shared memory after the last barrier.
#pragma once

#include <cooperative_groups.h>

#include "ggks_batch.cuh"

namespace ggks {

#ifdef GGKS_SMALL_TIMING
#define GGKS_SMALL_STAMP(i)                                                            \
  do {                                                                                 \
    if (r == 0 && tid == 0) {                                                          \
      uint64_t t_;                                                                     \
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_));                           \
      ctrl->t_ns[i] = t_;                                                              \
    }                                                                                  \
  } while (0)
// every CTA: its start (as the complement, so that atomicMax finds the
// earliest) and its end
#define GGKS_SMALL_EDGE(end)                                                           \
  do {                                                                                 \
    if (tid == 0) {                                                                    \
      uint64_t t_;                                                                     \
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_));                           \
      atomicMax((unsigned long long *)&ctrl->t_ns[(end) ? 15 : 14],                    \
                (unsigned long long)((end) ? t_ : ~t_));                               \
    }                                                                                  \
  } while (0)
#else
#define GGKS_SMALL_EDGE(end) \
  do {                       \
  } while (0)
#define GGKS_SMALL_STAMP(i) \
  do {                      \
  } while (0)
#endif

constexpr uint32_t kSmCtas = 16;                  // CTAs of the cluster (a non-portable size)
constexpr uint32_t kSmThreads = 1024;
constexpr uint32_t kSmNb = kSmCtas * kSmThreads;  // bucket budget: one bucket per thread
// samples, taken as pairs at S / 2 positions (16384 four-byte keys gathered
// by all 16 CTAs at once took about 10 us, 8192 about 5)
template <class K>
__host__ __device__ constexpr uint32_t small_samples() {
  return 8192u;
}
constexpr uint32_t kSmMaxReq = kSmThreads;        // one request per thread
// largest vectors taken by this path: multiselects up to 2^20 elements
// (measured on GB300: 2^20 / 101 k's 80 us against 92 us for the pipeline,
// even at 2^21); top-k up to 2^18 (the threshold path is faster above)
constexpr uint64_t kSmMaxN = 1ull << 20;
constexpr uint64_t kSmMaxTopkN = 1ull << 18;
constexpr uint32_t ST_SMALL_MISS = 64u;           // run the pipeline instead

// dynamic shared memory: the table once per bank, then one word per bucket --
// its count after the histogram phase, its compaction cursor after the plan
// (inactive cursors carry bit 31).  CTA 0's samples (phase A) lie over the
// bucket words; the finishers' scratch (phase F) over both.
constexpr size_t kSmHcOff = (size_t)kRepWords * 4;
constexpr size_t kSmBytes = kSmHcOff + (size_t)kSmNb * 4;
// a warp finisher's buffer: a warp sorts at most 256 four-byte keys (a
// one-warp bitonic network over 1024 keys took about 30 us; larger segments
// go to the whole-CTA finisher)
constexpr uint32_t kSmWarpBytes = 1024;
static_assert(kSmHcOff % 16 == 0, "bucket words' alignment");
static_assert((size_t)small_samples<uint32_t>() * 4 <= kSmBytes - kSmHcOff, "samples fit");
static_assert((size_t)small_samples<uint64_t>() * 8 <= kSmBytes - kSmHcOff, "samples fit");
static_assert(kSmThreads / 32 * (kSmWarpBytes + (kWarpSelBins + kWarpSelReq) * 4) <= kSmBytes,
              "warp finishers' buffers and histograms fit");
static_assert(small_samples<uint64_t>() % (2 * kSmThreads) == 0, "whole pairs per thread");

// segments of at most this many keys are finished by one warp
template <class K>
__host__ __device__ constexpr uint32_t small_warp_cap() {
  return kSmWarpBytes / (uint32_t)sizeof(K);
}
// segments of at most this many keys are sorted whole by the CTA in shared
// memory (a bitonic network); larger ones go to finish_slot
template <class K>
__host__ __device__ constexpr uint32_t small_sort_cap() {
  return (uint32_t)(65536 / sizeof(K));
}
// gather buffer of the CTA finisher (finish_slot) for the largest segments
template <class K>
__host__ __device__ constexpr uint32_t small_fin_cap() {
  return sizeof(K) == 4 ? 16384u : 4096u;
}
static_assert(finish_smem_for<uint32_t>(small_fin_cap<uint32_t>()) <= kSmBytes, "finisher fits");
static_assert(small_sort_cap<uint32_t>() * 4 <= kSmBytes && small_sort_cap<uint64_t>() * 8 <= kSmBytes,
              "a sorted segment fits");
static_assert(finish_smem_for<uint64_t>(small_fin_cap<uint64_t>()) <= kSmBytes, "finisher fits");

// Completes the ascending sort of s[0, P) (P a power of two >= 32) whose
// 32-key runs are each sorted ascending (as warp_bitonic32 leaves them):
// merges of doubling width whose first step compares mirrored positions, so
// that every merged run stays ascending (the network finish_warp runs in one
// warp), one __syncthreads per step.
template <class K>
__device__ __forceinline__ void bitonic_merge_smem(K *s, uint32_t P) {
  for (uint32_t k = 64; k <= P; k <<= 1) {
    const uint32_t half = k >> 1;
    for (uint32_t i = threadIdx.x; i < (P >> 1); i += blockDim.x) {
      const uint32_t a = ((i & ~(half - 1)) << 1) | (i & (half - 1));
      const uint32_t b = a ^ (k - 1);
      const K x = s[a], y = s[b];
      if (x > y) {
        s[a] = y;
        s[b] = x;
      }
    }
    __syncthreads();
    for (uint32_t j = k >> 2; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < (P >> 1); i += blockDim.x) {
        const uint32_t a = ((i & ~(j - 1)) << 1) | (i & (j - 1)), b = a + j;
        const K x = s[a], y = s[b];
        if (x > y) {
          s[a] = y;
          s[b] = x;
        }
      }
      __syncthreads();
    }
  }
}

// x: device vector of n elements (1 <= n <= kSmMaxN; the kernel itself takes
// any n below 2^31); reqs: num_req requests
// (ascending 0-based rank, output index; num_req <= kSmMaxReq); out: outputs;
// surv: survivor buffer of surv_cap >= n keys; chk: kSmNb * kSmCtas words
// (each requested bucket's first cursors, for the check); ctrl: status.
// Launched as one cluster of kSmCtas CTAs of kSmThreads threads.
template <class T, class OutT>
__global__ void __launch_bounds__(kSmThreads, 1)
    k_small(const T *__restrict__ x, uint64_t n, const Req *__restrict__ reqs, uint32_t num_req,
            OutT *__restrict__ out, typename Traits<T>::K *__restrict__ surv, uint64_t surv_cap,
            uint32_t *__restrict__ chk, Ctrl *ctrl) {
  namespace cg = cooperative_groups;
  using K = typename Traits<T>::K;
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t r = cl.block_rank();
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  extern __shared__ uint4 smem_raw[];
  uint32_t *rep = reinterpret_cast<uint32_t *>(smem_raw);
  uint32_t *hc = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(smem_raw) + kSmHcOff);
  __shared__ uint32_t s_tab[kSvSlices + 1];  // the splitter table
  __shared__ LutHeader<K> s_hdr;
  __shared__ K redk[33];
  __shared__ uint32_t red32[33];
  __shared__ uint32_t s_ctot;                 // elements in this CTA's buckets
  __shared__ uint32_t s_pre[kSmThreads];      // global prefix of this CTA's buckets
  __shared__ uint32_t s_kcnt[kSmThreads];     // requests per bucket
  __shared__ uint32_t s_kstart[kSmThreads];   // their lists' starts in s_klist
  __shared__ uint32_t s_kcur[kSmThreads];
  __shared__ Req s_klist[kSmMaxReq];          // requests by bucket (ranks local to the bucket)
  __shared__ uint32_t s_slot[kSmThreads];     // requested buckets: small ones up, large down
  __shared__ uint32_t s_nsmall, s_nlarge;
  __shared__ bool s_miss;

  GGKS_SMALL_STAMP(0);
  GGKS_SMALL_EDGE(false);
  // this thread's request, loaded ahead of the phases before its use
  Req q;
  q.rank = 0;
  q.out = 0;
  if (tid < num_req) q = reqs[tid];
  // ---------------- A: sample and table, in every CTA (the same samples and
  // the same deterministic build give every CTA the same table, so no CTA
  // waits for another's)
  constexpr uint32_t kS = small_samples<K>();
  const uint32_t S = n < kS ? (uint32_t)n : kS;
  if (tid == 0) {
    s_nsmall = 0;
    s_nlarge = 0;
    s_miss = false;
  }
  {
    K *samples = reinterpret_cast<K *>(hc);
    K lo = KeyMax<K>::v, hi = 0;
    if ((uint64_t)S >= n) {
      for (uint32_t i = tid; i < S; i += kSmThreads) {
        const K k = Traits<T>::key(x[i]);
        samples[i] = k;
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
      }
    } else {
      // pairs of neighbouring elements at hashed positions (samples 2q and
      // 2q + 1 are neighbours for the table builder's estimate of lanes
      // sharing a bucket); S / 2 independent positions keep the edge buckets
      // (keys beyond the sampled extremes) near n / (S / 2) keys.  Every
      // load of a thread is issued before its keys are used.
      constexpr uint32_t PER = kS / 2 / kSmThreads;  // pairs per thread
      K k[2 * PER];
#pragma unroll
      for (uint32_t u = 0; u < PER; ++u) {
        const uint32_t q = tid + u * kSmThreads;
        const uint64_t pos = ((uint64_t)hash32(q * 0x9E3779B9u + 0x5EEDu) * (n - 1)) >> 32;
        k[2 * u] = Traits<T>::key(x[pos]);
        k[2 * u + 1] = Traits<T>::key(x[pos + 1]);
      }
#pragma unroll
      for (uint32_t u = 0; u < PER; ++u) {
        const uint32_t q = tid + u * kSmThreads;
#pragma unroll
        for (uint32_t e = 0; e < 2; ++e) {
          const K kk = k[2 * u + e];
          samples[2 * q + e] = kk;
          lo = kk < lo ? kk : lo;
          hi = kk > hi ? kk : hi;
        }
      }
    }
    lo = block_reduce(lo, [](K u, K v) { return u < v ? u : v; }, redk);
    hi = block_reduce(hi, [](K u, K v) { return u > v ? u : v; }, redk);
    GGKS_SMALL_STAMP(1);
    build_lut_cta<K, (int)(kLutIdx / kSmThreads), true>(samples, S, lo, hi, kSmNb, s_tab, &s_hdr,
                                                        kSvBits);
  }
  __syncthreads();
  GGKS_SMALL_STAMP(2);

  // ---------------- B: histogram of this CTA's share
  for (uint32_t b = tid; b < kSmNb; b += kSmThreads) hc[b] = 0;
  __syncthreads();
  for (uint32_t i = tid; i < kRepWords; i += kSmThreads) rep[i] = s_tab[i >> 5];
  const LutHeader<K> h = s_hdr;
  const uint64_t a0 = n * r / kSmCtas, a1 = n * (r + 1) / kSmCtas;
  const uint32_t *lut = rep + lane;
  __syncthreads();
  for_range<T>(x, a0, a1, [&](K k, bool) {
    atomicAdd(&hc[bucket_of_rep<K>(k, h.base, h.shift, lut)], 1u);
  });
  cl.sync();  // 1: every histogram is complete (and every CTA has started)
  GGKS_SMALL_STAMP(3);

  // ---------------- C: bucket totals and their global prefix
  const uint32_t b = r * kSmThreads + tid;  // the bucket this thread owns
  uint32_t tot = 0;
#pragma unroll
  for (uint32_t c = 0; c < kSmCtas; ++c) tot += cl.map_shared_rank(hc, c)[b];
  uint32_t ctot;
  GGKS_SMALL_STAMP(8);
  const uint32_t excl = block_incl_scan(tot, &ctot, red32) - tot;
  if (tid == 0) s_ctot = ctot;
  s_kcnt[tid] = 0;
  GGKS_SMALL_STAMP(9);
  cl.sync();  // 2: every CTA's total is published
  GGKS_SMALL_STAMP(10);
  // the totals of the CTAs before this one: one remote load per lane of warp 0
  if (warp == 0) {
    uint32_t v = lane < r ? *cl.map_shared_rank(&s_ctot, lane) : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red32[32] = v;
  }
  __syncthreads();
  const uint32_t coff = red32[32];
  const uint32_t pre = coff + excl;
  s_pre[tid] = pre;
  __syncthreads();
  GGKS_SMALL_STAMP(11);

  // ---------------- D: requests -> buckets, every CTA's cursors
  const bool mine = tid < num_req && q.rank >= coff && q.rank - coff < ctot;
  uint32_t qb = 0;
  if (mine) {
    // the last bucket whose prefix is <= the rank (its count covers the rank)
    uint32_t i = 0;
#pragma unroll
    for (uint32_t step = kSmThreads / 2; step > 0; step >>= 1)
      if (s_pre[i + step] <= q.rank) i += step;
    qb = i;
    q.rank -= s_pre[i];
    atomicAdd(&s_kcnt[i], 1u);
  }
  __syncthreads();
  const uint32_t kc = s_kcnt[tid];
  uint32_t ktot;
  s_kstart[tid] = block_incl_scan(kc, &ktot, red32) - kc;
  s_kcur[tid] = 0;
  __syncthreads();
  if (mine) s_klist[s_kstart[qb] + atomicAdd(&s_kcur[qb], 1u)] = q;
  GGKS_SMALL_STAMP(12);
  // the owner turns its bucket's count in every CTA into that CTA's first
  // survivor position (a requested bucket) or an inactive cursor; each word is
  // read and written by its owner only
  uint32_t *my_chk = chk + (size_t)b * kSmCtas;
  if (kc) {
    // every count first (independent remote loads in flight together)
    uint32_t v[kSmCtas];
#pragma unroll
    for (uint32_t c = 0; c < kSmCtas; ++c) v[c] = cl.map_shared_rank(hc, c)[b];
    uint32_t run = pre;
#pragma unroll
    for (uint32_t c = 0; c < kSmCtas; ++c) {
      cl.map_shared_rank(hc, c)[b] = run;
      my_chk[c] = run;
      run += v[c];
    }
  } else {
#pragma unroll
    for (uint32_t c = 0; c < kSmCtas; ++c) cl.map_shared_rank(hc, c)[b] = kInactive;
  }
  if (kc) {
    if (tot <= small_warp_cap<K>())
      s_slot[atomicAdd(&s_nsmall, 1u)] = tid;
    else
      s_slot[kSmThreads - 1u - atomicAdd(&s_nlarge, 1u)] = tid;
  }
  GGKS_SMALL_STAMP(13);
  cl.sync();  // 3: every cursor is in place
  GGKS_SMALL_STAMP(4);

  // ---------------- E: compaction of this CTA's share
  {
    const uint32_t cap = (uint32_t)(surv_cap < (uint64_t)kInactive ? surv_cap : kInactive);
    for_range<T>(x, a0, a1, [&](K k, bool) {
      const uint32_t pos = atomicAdd(&hc[bucket_of_rep<K>(k, h.base, h.shift, lut)], 1u);
      st_global_if(surv + pos, k, pos < cap);
    });
  }
  cl.sync();  // 4: survivors written, cursors final
  GGKS_SMALL_STAMP(5);

  // ---------------- F: check, then finish the requested buckets
  if (kc) {
    // CTA c's cursor ends where CTA c + 1's started (the last at the bucket's end)
    uint32_t fin[kSmCtas], start[kSmCtas];
#pragma unroll
    for (uint32_t c = 0; c < kSmCtas; ++c) {
      fin[c] = cl.map_shared_rank(hc, c)[b];
      start[c] = my_chk[c];
    }
    bool bad = false;
#pragma unroll
    for (uint32_t c = 0; c < kSmCtas; ++c)
      bad |= fin[c] != (c + 1 < kSmCtas ? start[c + 1] : pre + tot);
    if (bad) s_miss = true;
  }
  cl.sync();  // 5: no shared memory of another CTA is read after this
  GGKS_SMALL_STAMP(6);
  if (!s_miss) {
    uint32_t *scratch = reinterpret_cast<uint32_t *>(smem_raw);
    const uint32_t nsmall = s_nsmall, nlarge = s_nlarge;
    // key range of bucket gb: from its first key to the next bucket's
    auto range = [&](uint32_t gb, K *klo, K *khi) {
      const K lo = bucket_lo<K>(gb, h.base, h.shift, s_tab, kSvSlices);
      const K nx = gb + 1 < h.nb ? bucket_lo<K>(gb + 1, h.base, h.shift, s_tab, kSvSlices) : K(0);
      *klo = lo;
      *khi = nx > lo ? nx - K(1) : KeyMax<K>::v;
    };
    auto size_of = [&](uint32_t t) {
      return (t + 1 < kSmThreads ? s_pre[t + 1] : coff + ctot) - s_pre[t];
    };
    for (uint32_t i = 0; i < nlarge; ++i) {
      const uint32_t t = s_slot[kSmThreads - 1u - i];
      const uint32_t size = size_of(t);
      const Req *rq = s_klist + s_kstart[t];
      const uint32_t m = s_kcnt[t];
      if (size <= small_sort_cap<K>()) {
        // the whole segment, padded to a power of two with the largest key:
        // 32-key runs sorted in registers, then the CTA's bitonic merges
        K *buf = reinterpret_cast<K *>(scratch);
        uint32_t P = 32;
        while (P < size) P <<= 1;
        for (uint32_t c0 = 0; c0 < P; c0 += kSmThreads) {
          const uint32_t j = c0 + tid;
          if (c0 + warp * 32 < P) {  // whole warps: the shuffle network needs all lanes
            const K v = j < size ? __ldcg(surv + s_pre[t] + j) : KeyMax<K>::v;
            buf[j] = warp_bitonic32(v);
          }
        }
        __syncthreads();
        bitonic_merge_smem(buf, P);
        for (uint32_t j = tid; j < m; j += kSmThreads) {
          const Req e = rq[j];
          out[e.out] = Traits<OutT>::value(buf[e.rank]);
        }
        __syncthreads();
      } else {
        K lo, hi;
        range(r * kSmThreads + t, &lo, &hi);
        const bool done = finish_slot<K, OutT, 1>(surv + s_pre[t], size, lo, hi, rq, m,
                                                 small_fin_cap<K>(), scratch, out);
        if (!done && tid == 0) s_miss = true;
      }
    }
    __syncthreads();
    K *wbuf = reinterpret_cast<K *>(scratch) + (size_t)warp * small_warp_cap<K>();
    uint32_t *whist = scratch + (size_t)(kSmThreads / 32) * (kSmWarpBytes / 4) +
                      (size_t)warp * (kWarpSelBins + kWarpSelReq);
    for (uint32_t i = warp; i < nsmall; i += kSmThreads / 32) {
      const uint32_t t = s_slot[i];
      K lo, hi;
      range(r * kSmThreads + t, &lo, &hi);
      const uint32_t size = size_of(t), m = s_kcnt[t];
      const Req *rq = s_klist + s_kstart[t];
      // up to kWarpSelReq requests: radix select, else (or when the needed
      // bins do not fit) the segment is sorted
      if (m > kWarpSelReq || !finish_warp_select<K, OutT>(surv + s_pre[t], size, lo, hi, rq, m,
                                                           wbuf, small_warp_cap<K>(), whist, out))
        finish_warp<K, OutT>(surv + s_pre[t], size, lo, rq, m, wbuf, out);
    }
  }
  __syncthreads();
  GGKS_SMALL_STAMP(7);
  GGKS_SMALL_EDGE(true);
#ifdef GGKS_SMALL_TIMING
  if (tid == 0) {
    uint32_t mx = 0;
    for (uint32_t i = 0; i < s_nsmall; ++i) {
      const uint32_t t = s_slot[i];
      const uint32_t sz = (t + 1 < kSmThreads ? s_pre[t + 1] : coff + ctot) - s_pre[t];
      mx = sz > mx ? sz : mx;
    }
    uint32_t mxl = 0;
    for (uint32_t i = 0; i < s_nlarge; ++i) {
      const uint32_t t = s_slot[kSmThreads - 1u - i];
      const uint32_t sz = (t + 1 < kSmThreads ? s_pre[t + 1] : coff + ctot) - s_pre[t];
      mxl = sz > mxl ? sz : mxl;
    }
    if (n >= (1u << 20))
      printf("cta %u: small %u (max %u keys), large %u (max %u keys), ctot %u\n", r, s_nsmall, mx,
             s_nlarge, mxl, ctot);
  }
#endif
  if (tid == 0 && s_miss) atomicOr(&ctrl->status, ST_SMALL_MISS);
}

}  // namespace ggks
