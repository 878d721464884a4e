// ggks_batch.cuh -- batched multiselect: thousands of independent vectors of
// uneven lengths, each with its own k list, selected in one persistent
// cooperative launch driven by work queues.
//
// The reference selects one vector per call (bucketMultiselectWrapper,
// bucketMultiselect.cu:837-871) and picks its algorithm per size offline
// (analyzeMultiselect.cu:209-274); here every problem of a batch runs the same
// bucket pipeline as the single-vector path, phase by phase across the whole
// batch, inside one kernel:
//
//   1 table    queue over problems: up to kBMaxS keys sampled into shared
//              memory, the problem's splitter table built by build_lut_cta
//              (the single-vector builder) with 2^nsl_bits <= kBSlices slices;
//              the tile phases hold it in shared memory once per bank.
//   2 hist     queue over (problem, tile) items: a tile is a contiguous range
//              of one problem; its shared-memory histogram becomes one row of
//              counts (rows of a problem's tiles are consecutive).  Tiles of a
//              speculating problem also keep the keys inside the problem's
//              candidate window in the tile's candidate area.
//   3 plan     queue over problems: the problem's rows become their exclusive
//              prefix over its tiles (column sums = bucket counts), a block
//              scan gives the bucket prefix, requested ranks map to buckets
//              and slots, the slots' survivors get a range of the shared
//              survivor buffer from a bump allocator, request lists per slot.
//   4 compact  queue over the same (problem, tile) items: cursors start at the
//              tile's prefix row, one shared atomic per element; a tile of a
//              speculating problem whose slots all lie inside the window
//              reads its complete candidate list instead of its elements.
//
// Speculation (top-k and other requests whose ranks cluster): the host sends
// the problem's rank window; phase 1 takes from the sample a key tau_lo below
// the window's lowest rank and a key tau_hi above its highest, with four
// standard deviations of the sample's rank error (counted in sampled chunks)
// and two chunks to spare, and phase 3 checks that every slot's bucket lies
// strictly between the buckets of tau_lo and tau_hi (buckets are monotone in
// the key, so every key of those buckets is then a candidate).  A tile whose
// list overflowed its area, or a problem whose slots fall outside, reads the
// elements as before: correctness never rests on the sample.
//   5 finish   queue over the large slots: finish_slot (the single-vector
//              finisher), a whole CTA each; then a warp queue over the
//              mid-size slots with at most kWarpSelReq requests (radix select
//              by one warp), then a warp queue over the small slots (at most
//              warp_cap keys, the common case); after one more grid barrier,
//              a CTA queue over the mid-size slots whose needed bins did not
//              fit a warp's buffer.  A batch with fewer than kWselPerCta
//              mid-size slots per CTA puts them in the first CTA queue
//              instead, and skips that barrier.
//
// A grid-wide barrier with a bounded wait separates the phases; the grid is
// launched cooperatively (all CTAs co-resident).  No CTA leaves early: a CTA
// that sees an error status skips the remaining work but still passes every
// barrier.  Data written by other CTAs in an earlier phase is read with
// ld.global.cg (L2), never through a possibly stale L1 line.
#pragma once

#include <type_traits>

#include "ggks_device.cuh"

namespace ggks {

constexpr int kBThreads = 512;
// slices of a problem's splitter table: few enough that the tile phases hold
// the table once per bank (entry j of lane l's copy at word 32 j + l), so a
// warp's 32 lookups take one shared-memory wavefront whatever slices its keys
// hit (a single copy of up to 4096 slices took two to three)
constexpr uint32_t kBSliceBits = 7;
constexpr uint32_t kBSlices = 1u << kBSliceBits;
constexpr uint32_t kBRepLut = (kBSlices + 1) * 32;  // words of the per-bank table
// shared-memory words in front of the tile phases' histogram / cursors
constexpr uint32_t kBTileLut = kBRepLut > kLutPadded ? kBRepLut : kLutPadded;
constexpr int kBSpt = (int)kLutIdx / kBThreads;  // slices per thread in the table build
constexpr uint32_t kBMaxNb = 8192;               // bucket budget of one problem
constexpr uint32_t kBMaxS = 8192;                // samples of one problem (shared memory)
constexpr int kBPhases = 5;
constexpr uint64_t kBMinTile = 1u << 16;  // smallest tile the host picks for a small batch
constexpr int kBColBatch = 4;  // tile rows per lane and load step of the plan phase's single-key scan
constexpr uint32_t kBWarpBytes = 2048;  // shared memory of one warp-finisher buffer
// 128-bit vectors in flight per thread in the plain counting loop of the
// tile phases and the plain compaction loop of uint32 and float64 batches
// (the other tile loops keep four)
constexpr int kBTileVecs = 8;
constexpr uint32_t kBRepBytes = 32768;  // per-bucket first keys of a tile (dup problems)
// slots whose request counters fit in the plan phase's spare shared memory
// (after the table, the bucket prefix and the flags: 81936 - 57360 bytes)
constexpr uint32_t kBPlanSlots = 3072;

// segments of at most this many keys are finished by one warp
template <class K>
__host__ __device__ constexpr uint32_t warp_cap() {
  return kBWarpBytes / (uint32_t)sizeof(K);
}

// one problem (host-written, read-only on the device)
struct BProb {
  const void *x;
  uint64_t n;
  uint64_t lut_off;  // u32 index of the splitter table (nsl + 1 entries, 16-byte aligned)
  uint64_t cnt_off;  // u32 index of the bucket counts (nb_max entries)
  uint64_t row0;     // u32 index of the first tile's row (tile r: row0 + r * nb_max)
  uint32_t req_off, num_req;  // requests [req_off, req_off + num_req); slots use the same range
  uint32_t nb_max, nsl_bits;
  uint32_t S, ntiles;
  uint32_t spec;              // 1: keep candidates in [rank spec_lo, rank spec_hi]
  uint32_t spec_lo, spec_hi;  // ascending ranks (0-based) the requests fall in
  uint32_t flt;               // a uint32 batch's float32 problem: keys in float order
};

// splitter-table header and plan results of one problem (device-written)
struct BHdr {
  uint64_t base;
  uint64_t surv_off;
  uint32_t shift, nb, heavy, num_slots;
  uint32_t dup;      // tiles track whether each bucket holds a single key
  uint32_t spec_on;  // phase 1 set the candidate window [tau_lo, tau_hi]
  uint32_t spec_ok;  // phase 3: every slot's bucket lies strictly inside it
  uint32_t pad;
  uint64_t tau_lo, tau_hi;  // keys; tau_lo 0 / tau_hi the largest key: open end
};

// one (problem, tile) work item (host-written)
struct BTile {
  uint64_t begin, end;  // elements [begin, end) of problem prob
  uint32_t prob, rank;  // rank of the tile among its problem's tiles
  uint64_t cand_off;    // key index of the tile's candidate area (speculating problems)
  uint32_t cand_cap, pad;
};

struct BCtrl {
  uint32_t status;
  uint32_t queue[kBPhases];  // work queue counters of the phases
  uint32_t bar_count, bar_gen;
  uint32_t deferred_count;
  uint32_t n_big, n_small;  // slots finished by a whole CTA / by one warp
  uint32_t small_pop;       // warp queue of the small slots
  uint32_t n_wsel, wsel_pop;  // mid-size slots a warp selects in, and their queue
  uint32_t n_retry, retry_pop;  // mid-size slots left to a whole CTA, and their queue
  uint32_t spec_tiles;      // compaction tiles that read their candidates
  uint64_t surv_top;    // survivor bump allocator
  uint64_t cap_needed;  // survivors wanted when they did not fit
  uint64_t t_ns[kBPhases + 1];  // %globaltimer at the start and after each phase (CTA 0)
  uint32_t dbg_code, dbg_pad;   // first failed index check (builds with GGKS_BATCH_CHECKS)
  uint64_t dbg_a, dbg_b;
};

struct BArgs {
  const BProb *probs;
  BHdr *hdrs;
  const BTile *tiles;
  uint32_t num_probs, num_tiles;
  uint32_t num_req;  // requests of all problems (= slot index space)
  uint32_t bcap;     // finisher gather capacity (keys)
  uint64_t surv_cap;
  uint64_t lut_words, row_words, cnt_words;  // sizes, for the index checks
  uint32_t *luts;
  uint32_t *rows;
  void *reps;  // key per row entry: the tile's only key of the bucket (dup problems)
  uint32_t *counts;
  const Req *reqs;  // rank within the problem, output position in out[]
  uint32_t *req_bucket, *req_local;
  uint32_t *seg_bucket, *seg_size, *kstart, *kcnt, *kcur;
  uint32_t *fill;  // per slot: survivor positions handed out to tiles (phase 4)
  uint64_t *seg_off;
  void *seg_lo, *seg_hi;  // key arrays
  Req *klist;
  uint32_t *big_list, *small_list, *wsel_list;  // slot indices by finisher kind
  uint32_t *retry_list;  // mid-size slots whose warp select did not fit
  void *surv;             // key array
  uint32_t *deferred;
  void *out;              // output values
  void *cand;             // key array: the tiles' candidate areas
  uint32_t *cand_cnt;     // per tile: candidates seen (may exceed the area)
  BCtrl *ctrl;
};

// Index checks of the batched kernel, compiled in with GGKS_BATCH_CHECKS: a
// failed check records its code and operands (first failure wins), sets
// ST_INTERNAL, and the guarded access is skipped.  Without the macro every
// check is the constant true.
#ifdef GGKS_BATCH_CHECKS
static __device__ __noinline__ bool bcheck_fail(BCtrl *c, uint32_t code, uint64_t a, uint64_t b) {
  if (atomicCAS(&c->dbg_code, 0u, code) == 0u) {
    c->dbg_a = a;
    c->dbg_b = b;
  }
  atomicOr(&c->status, ST_INTERNAL);
  return false;
}
#define BCHECK(cond, code, a, b) \
  ((cond) ? true : bcheck_fail(A.ctrl, (code), (uint64_t)(a), (uint64_t)(b)))
#else
#define BCHECK(cond, code, a, b) true
#endif

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier of a co-resident grid (generation counter).  A wait that
// runs out sets ST_TIMEOUT and goes on, so every wait ends.  Returns the
// status seen after the barrier (same value in every thread of the CTA).
__device__ __forceinline__ uint32_t grid_barrier(BCtrl *c, uint32_t *s_status, int phase) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t g0 = ld_acquire_u32(&c->bar_gen);
    __threadfence();
    if (atomicAdd(&c->bar_count, 1u) == gridDim.x - 1) {
      atomicExch(&c->bar_count, 0u);
      __threadfence();
      atomicAdd(&c->bar_gen, 1u);
    } else {
      int iters = 0;
      while (ld_acquire_u32(&c->bar_gen) == g0) {
        if (++iters > kSpinLimit) {
          atomicOr(&c->status, ST_TIMEOUT);
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    if (blockIdx.x == 0 && phase >= 0) c->t_ns[phase] = global_ns();
    *s_status = ld_acquire_u32(&c->status);
  }
  __syncthreads();
  return *s_status;
}

// next item of a work queue, shared with the whole CTA
__device__ __forceinline__ uint32_t queue_pop(uint32_t *q, uint32_t *s_item) {
  __syncthreads();
  if (threadIdx.x == 0) *s_item = atomicAdd(q, 1u);
  __syncthreads();
  return *s_item;
}

// Shared-memory position of bucket / slice x in the tile phases: x with its
// low five bits XORed by the next five.  Inputs with few distinct values
// (integer-valued floats, say) put their buckets and slices at regular
// power-of-two strides, which without the swizzle fall into one bank.  A
// permutation inside every group of 32 entries.
__device__ __forceinline__ uint32_t swz(uint32_t x) { return x ^ ((x >> 5) & 31u); }

// bucket_of with the splitter table held once per bank: lane_lut = table +
// (lane index), entry j at lane_lut[32 j]
template <class K>
__device__ __forceinline__ uint32_t bucket_of_lane(K key, K base, uint32_t shift,
                                                   const uint32_t *lane_lut, uint32_t nsl) {
  const K d = key - base;  // wraps for key < base; that result is discarded
  const K idx = d >> shift;
  const uint32_t j = idx < (K)nsl ? (uint32_t)idx : nsl;
  const uint32_t e = lane_lut[32 * j];
  const uint32_t b = (uint32_t)((int32_t)e >> 7) + shr_clamp(d, e & 127u);
  return key < base ? 0u : b;
}

__device__ __forceinline__ uint32_t ldcg_u(const uint32_t *p) { return __ldcg(p); }
__device__ __forceinline__ uint64_t ldcg_u(const uint64_t *p) {
  return __ldcg(reinterpret_cast<const unsigned long long *>(p));
}

__device__ __forceinline__ BHdr load_hdr(const BHdr *h) {
  BHdr r;
  r.base = ldcg_u(&h->base);
  r.surv_off = ldcg_u(&h->surv_off);
  const uint4 w = __ldcg(reinterpret_cast<const uint4 *>(&h->shift));
  r.shift = w.x;
  r.nb = w.y;
  r.heavy = w.z;
  r.num_slots = w.w;
  const uint4 w2 = __ldcg(reinterpret_cast<const uint4 *>(&h->dup));
  r.dup = w2.x;
  r.spec_on = w2.y;
  r.spec_ok = w2.z;
  r.tau_lo = ldcg_u(&h->tau_lo);
  r.tau_hi = ldcg_u(&h->tau_hi);
  return r;
}

// One warp finishes a segment of at most warp_cap<K>() keys: the keys are
// sorted in the warp's shared-memory buffer (32-key runs in registers, then
// bitonic merges whose first step compares mirrored positions, so every run
// stays ascending) and each request reads its rank.  size 0: a flat slot
// whose single key is lo.
template <class K, class OutT>
__device__ __forceinline__ void finish_warp(const K *__restrict__ src, uint32_t size, K lo,
                                            const Req *__restrict__ rq, uint32_t m, K *buf,
                                            OutT *__restrict__ out) {
  const uint32_t lane = threadIdx.x & 31;
  if (size == 0) {
    for (uint32_t j = lane; j < m; j += 32) out[rq[j].out] = Traits<OutT>::value(lo);
    return;
  }
  uint32_t P = 32;
  while (P < size) P <<= 1;
  for (uint32_t c = 0; c < P; c += 32) {
    const K v = c + lane < size ? src[c + lane] : KeyMax<K>::v;
    buf[c + lane] = warp_bitonic32(v);
  }
  __syncwarp();
  for (uint32_t k = 64; k <= P; k <<= 1) {
    const uint32_t half = k >> 1;
    for (uint32_t t = lane; t < (P >> 1); t += 32) {
      const uint32_t a = ((t & ~(half - 1)) << 1) | (t & (half - 1));
      const uint32_t b = a ^ (k - 1);
      const K x = buf[a], y = buf[b];
      if (x > y) {
        buf[a] = y;
        buf[b] = x;
      }
    }
    __syncwarp();
    for (uint32_t j = k >> 2; j > 0; j >>= 1) {
      for (uint32_t t = lane; t < (P >> 1); t += 32) {
        const uint32_t a = ((t & ~(j - 1)) << 1) | (t & (j - 1)), b = a + j;
        const K x = buf[a], y = buf[b];
        if (x > y) {
          buf[a] = y;
          buf[b] = x;
        }
      }
      __syncwarp();
    }
  }
  for (uint32_t j = lane; j < m; j += 32) {
    const Req e = rq[j];
    out[e.out] = Traits<OutT>::value(buf[e.rank]);
  }
  __syncwarp();
}

// requests a warp answers by radix select (more: the segment is sorted)
constexpr uint32_t kWarpSelReq = 4;
constexpr uint32_t kWarpSelBins = 256;  // the select's histogram (one word per bin)
// Segments above warp_cap keys and up to this many, with at most kWarpSelReq
// requests, are selected by one warp (two passes of size / 32 loads per lane)
// instead of a whole CTA; larger ones keep the CTA.
constexpr uint32_t kWarpSelMax = 16384;
// A warp takes about ten times a CTA's time on such a segment, so warps take
// them only when a batch has at least this many per CTA of the grid (a CTA
// queue of fewer ends sooner); otherwise they join the CTA queue.
constexpr uint32_t kWselPerCta = 16;

// One warp answers m <= kWarpSelReq requests of a segment of size > 0 keys, all
// in [lo, hi], by radix select instead of sorting the segment: a histogram of
// (key - lo) in 256 bins, the bin of each requested rank, then only those
// bins' keys gathered into buf (buf_cap keys), each bin sorted (32-key runs in
// registers, the finish_warp merges above that), and each request read from
// its bin.  hist: kWarpSelBins + kWarpSelReq shared words of this warp.
// Returns false, having written nothing, when the needed bins do not fit buf
// (keys spread unevenly over the bucket's range); the caller then sorts the
// segment.  Every index into the per-request arrays is a compile-time one.
template <class K, class OutT>
__device__ __forceinline__ bool finish_warp_select(const K *__restrict__ src, uint32_t size, K lo,
                                                   K hi, const Req *__restrict__ rq, uint32_t m,
                                                   K *buf, uint32_t buf_cap, uint32_t *hist,
                                                   OutT *__restrict__ out) {
  const uint32_t lane = threadIdx.x & 31;
  if (size >= 65536u) return false;  // ranks inside a bin travel in 16 bits
  const int bl = bitlen<K>(hi - lo);
  const uint32_t sh = bl > 8 ? (uint32_t)(bl - 8) : 0u;  // (hi - lo) >> sh < 256
  auto bin_of = [&](K k) -> uint32_t {
    const uint32_t b = (uint32_t)((K)(k - lo) >> sh);
    return b < kWarpSelBins ? b : kWarpSelBins - 1u;  // keys lie in [lo, hi]: never clamped
  };
#pragma unroll
  for (uint32_t q = 0; q < kWarpSelBins / 32; ++q) hist[q * 32 + lane] = 0;
  __syncwarp();
  // U loads in flight per lane in both passes over the segment
  constexpr uint32_t U = sizeof(K) == 4 ? 8u : 4u;
  for (uint32_t i0 = 0; i0 < size; i0 += 32 * U) {
    K v[U];
#pragma unroll
    for (uint32_t u = 0; u < U; ++u) {
      const uint32_t i = i0 + 32 * u + lane;
      v[u] = i < size ? src[i] : K(0);
    }
#pragma unroll
    for (uint32_t u = 0; u < U; ++u)
      if (i0 + 32 * u + lane < size) atomicAdd(&hist[bin_of(v[u])], 1u);
  }
  __syncwarp();
  // exclusive prefix of the bins, lane l holding bins 8 l .. 8 l + 7
  uint32_t c[8], sum = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    c[q] = hist[8 * lane + q];
    sum += c[q];
  }
  const uint32_t run = warp_incl_scan(sum) - sum;
  // each request's bin and rank inside it; its region of buf (a request
  // whose bin an earlier request also needs shares that one's region)
  uint32_t rb[kWarpSelReq], rr[kWarpSelReq], roff[kWarpSelReq], rcnt[kWarpSelReq],
      rP[kWarpSelReq];
  bool own[kWarpSelReq];
  bool ok = true;
  uint32_t used = 0;
#pragma unroll
  for (uint32_t j = 0; j < kWarpSelReq; ++j) {
    rb[j] = 0xFFFFFFFFu;
    rr[j] = 0;
    roff[j] = 0;
    rcnt[j] = 0;
    rP[j] = 0;
    own[j] = false;
    if (j >= m) continue;
    const uint32_t r = rq[j].rank;
    uint32_t acc = run, hit = 0, at = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (c[q] && acc <= r && r < acc + c[q]) {
        hit = 1;
        at = ((8 * lane + q) << 16) | (r - acc);  // bin, rank inside it (< 2^16)
      }
      acc += c[q];
    }
    const uint32_t who = __ballot_sync(0xffffffffu, hit);
    if (who == 0) {
      ok = false;  // a rank outside the segment: leave it to the sort
      continue;
    }
    at = __shfl_sync(0xffffffffu, at, __ffs(who) - 1);
    rb[j] = at >> 16;
    rr[j] = at & 0xFFFFu;
    own[j] = true;
#pragma unroll
    for (uint32_t t = 0; t < j; ++t)
      if (rb[t] == rb[j]) {
        own[j] = false;
        roff[j] = roff[t];
      }
    if (own[j]) {
      rcnt[j] = hist[rb[j]];
      uint32_t P = 32;
      while (P < rcnt[j]) P <<= 1;
      rP[j] = P;
      roff[j] = used;
      used += P;
    }
  }
  if (!ok) return false;
  if (sh == 0) {
    // bins one key wide (the bucket spans under 256 keys): each request's
    // key is its bin's, however many copies the bin holds
#pragma unroll
    for (uint32_t j = 0; j < kWarpSelReq; ++j)
      if (j < m && lane == j) out[rq[j].out] = Traits<OutT>::value((K)(lo + (K)rb[j]));
    __syncwarp();
    return true;
  }
  if (used > buf_cap) return false;
  // gather the needed bins' keys (per-bin counters after the histogram)
  uint32_t *cur = hist + kWarpSelBins;
  if (lane < kWarpSelReq) cur[lane] = 0;
  __syncwarp();
  for (uint32_t i0 = 0; i0 < size; i0 += 32 * U) {
    K v[U];
#pragma unroll
    for (uint32_t u = 0; u < U; ++u) {
      const uint32_t i = i0 + 32 * u + lane;
      v[u] = i < size ? src[i] : K(0);
    }
#pragma unroll
    for (uint32_t u = 0; u < U; ++u) {
      if (i0 + 32 * u >= size) break;  // the same for every lane
      const uint32_t i = i0 + 32 * u + lane;
      const K k = v[u];
      const uint32_t b = i < size ? bin_of(k) : 0xFFFFFFFFu;
#pragma unroll
      for (uint32_t t = 0; t < kWarpSelReq; ++t) {
        if (!own[t]) continue;
        const bool mine = b == rb[t];
        const uint32_t mm = __ballot_sync(0xffffffffu, mine);
        if (mm == 0) continue;
        const int leader = __ffs(mm) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&cur[t], (uint32_t)__popc(mm));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (mine) buf[roff[t] + base + __popc(mm & ((1u << lane) - 1u))] = k;
      }
    }
  }
  __syncwarp();
  // sort each needed bin in its region (the padding sorts last)
#pragma unroll
  for (uint32_t t = 0; t < kWarpSelReq; ++t) {
    if (!own[t]) continue;
    K *s = buf + roff[t];
    const uint32_t P = rP[t];
    for (uint32_t c0 = 0; c0 < P; c0 += 32) {
      const K v = c0 + lane < rcnt[t] ? s[c0 + lane] : KeyMax<K>::v;
      s[c0 + lane] = warp_bitonic32(v);
    }
    __syncwarp();
    for (uint32_t k = 64; k <= P; k <<= 1) {
      const uint32_t half = k >> 1;
      for (uint32_t x = lane; x < (P >> 1); x += 32) {
        const uint32_t a = ((x & ~(half - 1)) << 1) | (x & (half - 1));
        const uint32_t b = a ^ (k - 1);
        const K u = s[a], v = s[b];
        if (u > v) {
          s[a] = v;
          s[b] = u;
        }
      }
      __syncwarp();
      for (uint32_t j = k >> 2; j > 0; j >>= 1) {
        for (uint32_t x = lane; x < (P >> 1); x += 32) {
          const uint32_t a = ((x & ~(j - 1)) << 1) | (x & (j - 1)), b = a + j;
          const K u = s[a], v = s[b];
          if (u > v) {
            s[a] = v;
            s[b] = u;
          }
        }
        __syncwarp();
      }
    }
  }
  // answers: lane j answers request j
#pragma unroll
  for (uint32_t j = 0; j < kWarpSelReq; ++j)
    if (j < m && lane == j) out[rq[j].out] = Traits<OutT>::value(buf[roff[j] + rr[j]]);
  __syncwarp();
  return true;
}

// Elements [a, b) of x (any alignment): scalar head up to a 16-byte boundary,
// a 128-bit body with U vectors in flight per thread, a scalar tail.
// f(key, full) is called once per element; full: all 32 lanes of the warp
// make the same call (the unrolled body), so warp-collective operations are
// allowed.
template <class T, int U = 4, class F>
__device__ __forceinline__ void for_range(const T *__restrict__ x, uint64_t a, uint64_t b, F &&f) {
  using K = typename Traits<T>::K;
  using V = typename Traits<T>::Vec;
  constexpr int PV = Traits<T>::kPerVec;
  uint64_t va = a + (uint64_t)((16u - ((uint32_t)(uintptr_t)(x + a) & 15u)) & 15u) / sizeof(T);
  if (va > b) va = b;
  const uint64_t nvec = (b - va) / PV;
  const uint64_t vb = va + nvec * PV;
  for (uint64_t e = a + threadIdx.x; e < va; e += blockDim.x) f(Traits<T>::key(x[e]), false);
  for (uint64_t e = vb + threadIdx.x; e < b; e += blockDim.x) f(Traits<T>::key(x[e]), false);
  const V *xv = reinterpret_cast<const V *>(x + va);
  const uint64_t step = (uint64_t)U * blockDim.x;
  uint64_t v0 = 0;
  for (; v0 + step <= nvec; v0 += step) {
    V vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) vv[u] = ldg_stream(xv + v0 + (uint64_t)u * blockDim.x + threadIdx.x);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      K k[PV];
      vec_keys<T>(vv[u], k);
#pragma unroll
      for (int e = 0; e < PV; ++e) f(k[e], true);
    }
  }
  for (uint64_t vi = v0 + threadIdx.x; vi < nvec; vi += blockDim.x) {
    K k[PV];
    vec_keys<T>(ldg_stream(xv + vi), k);
#pragma unroll
    for (int e = 0; e < PV; ++e) f(k[e], false);
  }
}

// A uint32 batch also carries float32 problems (flt): both have 32-bit keys,
// so float32 and uint32 requests share one launch; a float32 problem's keys
// take the float order (its outputs are keys, turned back into floats by the
// host).  Key of element i of a problem's vector:
template <class T>
__device__ __forceinline__ typename Traits<T>::K load_key(const void *x, uint64_t i, uint32_t flt) {
  if constexpr (std::is_same<T, uint32_t>::value) {
    const uint32_t b = reinterpret_cast<const uint32_t *>(x)[i];
    return flt ? Traits<float>::key_bits(b) : b;
  } else {
    return Traits<T>::key(reinterpret_cast<const T *>(x)[i]);
  }
}

// for_range over a problem's vector in its own key order
template <class T, int U = 4, class F>
__device__ __forceinline__ void for_range_p(const void *x, uint32_t flt, uint64_t a, uint64_t b,
                                            F &&f) {
  if constexpr (std::is_same<T, uint32_t>::value) {
    if (flt) {
      for_range<float, U>(reinterpret_cast<const float *>(x), a, b, f);
      return;
    }
  }
  for_range<T, U>(reinterpret_cast<const T *>(x), a, b, f);
}

template <class T>
__global__ void __launch_bounds__(kBThreads, 2) k_batch(BArgs A) {
  using K = typename Traits<T>::K;
  using OutT = T;
  extern __shared__ uint4 smem_raw[];
  uint32_t *sm = reinterpret_cast<uint32_t *>(smem_raw);
  __shared__ uint32_t s_item, s_status, s_cur;
  __shared__ K redk[33];
  __shared__ uint32_t red32[33];
  __shared__ uint64_t red64[33];
  __shared__ uint64_t s_base;
  __shared__ uint32_t s_lb[3];
  __shared__ LutHeader<K> s_hdr;
  __shared__ bool s_bad;
  __shared__ uint32_t s_rcnt[256], s_rsel[2], s_ccnt;
  BCtrl *ctrl = A.ctrl;
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  K *surv = reinterpret_cast<K *>(A.surv);
  K *seg_lo = reinterpret_cast<K *>(A.seg_lo);
  K *seg_hi = reinterpret_cast<K *>(A.seg_hi);
  OutT *out = reinterpret_cast<OutT *>(A.out);
  if (blockIdx.x == 0 && tid == 0) ctrl->t_ns[0] = global_ns();
  // candidate counts start at zero (phase 2 adds to them after the barrier)
  for (uint32_t t = blockIdx.x * nt + tid; t < A.num_tiles; t += gridDim.x * nt) A.cand_cnt[t] = 0;

  // ---------------- phase 1: splitter tables
  for (uint32_t p = queue_pop(&ctrl->queue[0], &s_item); p < A.num_probs;
       p = queue_pop(&ctrl->queue[0], &s_item)) {
#ifdef GGKS_BATCH_TIMING
    const long long c0 = clock64();
#endif
    const BProb P = A.probs[p];
    K *samples = reinterpret_cast<K *>(sm);
    K lo = KeyMax<K>::v, hi = 0;
    if ((uint64_t)P.S >= P.n) {
      // small problem: every element is a sample
      for (uint32_t i = tid; i < P.S; i += nt) {
        const K k = load_key<T>(P.x, i, P.flt);
        samples[i] = k;
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
      }
    } else {
      // S / CH chunks of CH consecutive elements (one 32-byte sector's worth)
      // at hashed positions: the whole grid gathers at once, and a sector read
      // for one 4-byte key would spend 8x the DRAM traffic
      constexpr uint32_t CH = 32 / sizeof(T);
      const uint32_t nch = P.S / CH;
      const uint64_t slots = P.n / CH;
      for (uint32_t c = tid; c < nch; c += nt) {
        const uint64_t pos = (((uint64_t)hash32(c * 0x9E3779B9u + 0x5EEDu) * slots) >> 32) * CH;
        K k[CH];
#pragma unroll
        for (uint32_t e = 0; e < CH; ++e) k[e] = load_key<T>(P.x, pos + e, P.flt);
#pragma unroll
        for (uint32_t e = 0; e < CH; ++e) {
          samples[c * CH + e] = k[e];
          lo = k[e] < lo ? k[e] : lo;
          hi = k[e] > hi ? k[e] : hi;
        }
      }
    }
    lo = block_reduce(lo, [](K u, K v) { return u < v ? u : v; }, redk);
    hi = block_reduce(hi, [](K u, K v) { return u > v ? u : v; }, redk);
#ifdef GGKS_BATCH_TIMING
    const long long c1 = clock64();
#endif
    if (!BCHECK(P.lut_off + (1u << P.nsl_bits) < A.lut_words && P.S <= kBMaxS, 1, p, P.lut_off))
      continue;
    build_lut_cta<K, kBSpt, true>(samples, P.S, lo, hi, P.nb_max, A.luts + P.lut_off, &s_hdr,
                                  (int)P.nsl_bits);
    __syncthreads();
    // Speculation: the window's ends as sample ranks, moved outwards by four
    // standard deviations of the number of sampled chunks below them
    // (Binomial(chunks, rank / n)) plus two chunks, in chunk-sized units (a
    // chunk's keys are neighbours, as correlated as sorted input makes them);
    // an end beyond the samples leaves that side open.  A miss costs only the
    // full compaction read.  The same float arithmetic in every thread.
    K tau_lo = 0, tau_hi = KeyMax<K>::v;
    const bool spec_on = P.spec && (uint64_t)P.S < P.n && !s_hdr.dup;
    if (spec_on) {
      constexpr uint32_t CH = 32 / sizeof(T);
      const float fS = (float)P.S, fc = (float)(P.S / CH), fn = (float)P.n;
      const float pl = (float)P.spec_lo / fn, ph = (float)((uint64_t)P.spec_hi + 1) / fn;
      const float al = pl * fS - (float)CH * (4.0f * sqrtf(fc * pl * (1.0f - pl)) + 2.0f);
      const float ah = ph * fS + (float)CH * (4.0f * sqrtf(fc * ph * (1.0f - ph)) + 2.0f);
      if (al >= 1.0f) tau_lo = cta_select_rank<K>(samples, P.S, (uint32_t)al, s_rcnt, s_rsel);
      if (ah <= fS - 2.0f)
        tau_hi = cta_select_rank<K>(samples, P.S, (uint32_t)ah + 1u, s_rcnt, s_rsel);
    }
#ifdef GGKS_BATCH_TIMING
    if (tid == 0) {
      atomicAdd((unsigned long long *)&ctrl->dbg_a, (unsigned long long)(c1 - c0));
      atomicAdd((unsigned long long *)&ctrl->dbg_b, (unsigned long long)(clock64() - c1));
    }
#endif
    if (tid == 0) {
      BHdr h;
      h.base = s_hdr.base;
      h.surv_off = 0;
      h.shift = s_hdr.shift;
      h.nb = s_hdr.nb;
      h.heavy = s_hdr.heavy;
      h.num_slots = 0;
      h.dup = (s_hdr.dup && P.nb_max * sizeof(K) <= kBRepBytes) ? 1u : 0u;
      h.spec_on = spec_on ? 1u : 0u;
      h.spec_ok = 0;
      h.pad = 0;
      h.tau_lo = (uint64_t)tau_lo;
      h.tau_hi = (uint64_t)tau_hi;
      A.hdrs[p] = h;
    }
    // the bucket totals start at zero: the tiles of phase 2 add to them
    for (uint32_t b = tid; b < P.nb_max; b += nt) A.counts[P.cnt_off + b] = 0;
  }
  uint32_t st = grid_barrier(ctrl, &s_status, 1);

  // ---------------- phase 2: one histogram row per tile
  if (tid == 0) s_cur = 0xFFFFFFFFu;  // problem whose table is in shared memory
  uint32_t *lut = sm;                     // the plan phase's single copy
  const uint32_t *lane_lut = sm + (tid & 31);  // the tile phases' per-bank copies
  uint32_t *hist = sm + kBTileLut;
  K *rep = reinterpret_cast<K *>(hist + kBMaxNb);
  K *reps = reinterpret_cast<K *>(A.reps);
  if (!(st & ST_FATAL)) {
    for (uint32_t t = queue_pop(&ctrl->queue[1], &s_item); t < A.num_tiles;
         t = queue_pop(&ctrl->queue[1], &s_item)) {
      const BTile tl = A.tiles[t];
      const BProb P = A.probs[tl.prob];
      const BHdr H = load_hdr(A.hdrs + tl.prob);
      const uint32_t nsl = 1u << P.nsl_bits;
      if (s_cur != tl.prob)
        for (uint32_t w = tid; w < (nsl + 1) * 32; w += nt) sm[w] = __ldcg(A.luts + P.lut_off + (w >> 5));
      for (uint32_t b = tid; b < ((H.nb + 31) & ~31u); b += nt) {
        hist[b] = 0;
        if (H.dup) rep[b] = KeyMax<K>::v;
      }
      if (tid == 0) s_ccnt = 0;
      __syncthreads();
      if (tid == 0) s_cur = tl.prob;
      const K base = (K)H.base;
      const uint32_t shift = H.shift;
      if (H.dup) {
        // count, and keep the bucket's first key; a second distinct key (or
        // the largest key, which marks an empty entry) sets the mixed bit
        for_range_p<T>(P.x, P.flt, tl.begin, tl.end, [&](K k, bool) {
          const uint32_t ub = bucket_of_lane<K>(k, base, shift, lane_lut, nsl);
          if (!BCHECK(ub < H.nb, 2, ub, H.nb)) return;
          const uint32_t b = swz(ub);
          atomicAdd(&hist[b], 1u);
          const K r = rep[b];
          if (r != k || k == KeyMax<K>::v) {
            if (k != KeyMax<K>::v && r == KeyMax<K>::v) {
              const K old = atomic_cas_key(&rep[b], KeyMax<K>::v, k);
              if (old != KeyMax<K>::v && old != k) atomicOr(&hist[b], kMixed);
            } else if (!(hist[b] & kMixed)) {
              atomicOr(&hist[b], kMixed);
            }
          }
        });
      } else if (H.spec_on) {
        // count, and append the keys inside the window to the tile's
        // candidate area: one unsigned compare per key, a shared atomic for
        // each kept key (about one lane in a warp keeps one when it does, so
        // a warp vote would buy nothing); the count goes on past the area's
        // end, so the compaction phase can tell a complete list
        const K tlo = (K)H.tau_lo, span = (K)H.tau_hi - (K)H.tau_lo;
        K *cand = reinterpret_cast<K *>(A.cand) + tl.cand_off;
        const uint32_t ccap = tl.cand_cap;
        for_range_p<T>(P.x, P.flt, tl.begin, tl.end, [&](K k, bool) {
          const uint32_t ub = bucket_of_lane<K>(k, base, shift, lane_lut, nsl);
          if (BCHECK(ub < H.nb, 4, ub, H.nb)) atomicAdd(&hist[swz(ub)], 1u);
          if ((K)(k - tlo) <= span) {
            const uint32_t pos = atomicAdd(&s_ccnt, 1u);
            if (pos < ccap) cand[pos] = k;
          }
        });
      } else {
        // also for heavy problems: the histogram's atomics return nothing, and
        // lanes adding to one counter cost no more than lanes adding to
        // different ones, so warp aggregation (compaction's) would only slow
        // this phase down.  Eight vectors in flight per thread.
        for_range_p<T, kBTileVecs>(P.x, P.flt, tl.begin, tl.end, [&](K k, bool) {
          const uint32_t ub = bucket_of_lane<K>(k, base, shift, lane_lut, nsl);
          if (!BCHECK(ub < H.nb, 4, ub, H.nb)) return;
          atomicAdd(&hist[swz(ub)], 1u);
        });
      }
      __syncthreads();
      if (H.spec_on && tid == 0) A.cand_cnt[t] = s_ccnt;
      const uint64_t ro = P.row0 + (uint64_t)tl.rank * P.nb_max;
      if (!BCHECK(ro + H.nb <= A.row_words && H.nb <= P.nb_max, 5, ro, H.nb)) continue;
      // the tile's row, and its counts added to the problem's bucket totals
      uint32_t *tot = A.counts + P.cnt_off;
      for (uint32_t b = tid; b < H.nb; b += nt) {
        const uint32_t c = hist[swz(b)];
        A.rows[ro + b] = c;
        if (c & ~kMixed) atomicAdd(tot + b, c & ~kMixed);
        if (H.dup) reps[ro + b] = rep[swz(b)];
      }
    }
  }
  st = grid_barrier(ctrl, &s_status, 2);

  // ---------------- phase 3: per-problem scan and plan
  if (!(st & ST_FATAL)) {
    for (uint32_t p = queue_pop(&ctrl->queue[2], &s_item); p < A.num_probs;
         p = queue_pop(&ctrl->queue[2], &s_item)) {
      const BProb P = A.probs[p];
      const BHdr H = load_hdr(A.hdrs + p);
      const uint32_t nb = H.nb, nsl = 1u << P.nsl_bits, nr = P.ntiles;
      uint32_t *excl = sm + kLutPadded;  // bucket prefix; later: slot of each flagged bucket
      uint8_t *flag = reinterpret_cast<uint8_t *>(excl + kBMaxNb);
      uint32_t *cnt = A.counts + P.cnt_off;
      if (!BCHECK(P.row0 + (uint64_t)nr * P.nb_max <= A.row_words && nb <= P.nb_max &&
                      P.cnt_off + P.nb_max <= A.cnt_words && P.req_off + P.num_req <= A.num_req,
                  6, p, nb))
        continue;
      for (uint32_t j = tid; j <= nsl; j += nt) lut[j] = __ldcg(A.luts + P.lut_off + j);
      // bucket totals (added by the tiles of phase 2) -> exclusive prefix in
      // shared memory; the flags start clear
      load_totals(cnt, nb, excl);
      for (uint32_t v = tid; v < ((nb + 3) >> 2); v += nt) reinterpret_cast<uint32_t *>(flag)[v] = 0;
      __syncthreads();
      if (smem_excl_scan(excl, nb, red32) != P.n && tid == 0) atomicOr(&ctrl->status, ST_INTERNAL);
      // contiguous bucket range per thread (slot numbering below)
      const uint32_t per = (nb + nt - 1) / nt;
      const uint32_t b0 = min(nb, tid * per), b1 = min(nb, b0 + per);
      // requests -> bucket (the last b with excl[b] <= rank) and local rank
      const Req *rq = A.reqs + P.req_off;
      for (uint32_t i = tid; i < P.num_req; i += nt) {
        const uint32_t rank = rq[i].rank;
        uint32_t lo = 0, hi = nb;
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (excl[mid] <= rank)
            lo = mid;
          else
            hi = mid;
        }
        flag[lo] |= 1;  // concurrent writers all store the same value
        A.req_bucket[P.req_off + i] = lo;
        A.req_local[P.req_off + i] = rank - excl[lo];
      }
      __syncthreads();
      // flagged buckets -> slots in bucket order; excl[] now maps bucket -> slot
      uint32_t my_slots = 0;
      for (uint32_t b = b0; b < b1; ++b) my_slots += flag[b] & 1u;
      uint32_t tot_slots;
      {
        uint32_t slot = block_incl_scan(my_slots, &tot_slots, red32) - my_slots;
        for (uint32_t b = b0; b < b1; ++b)
          if (flag[b] & 1u) {
            excl[b] = slot;
            if (BCHECK(slot < P.num_req, 7, slot, P.num_req)) A.seg_bucket[P.req_off + slot] = b;
            slot++;
          }
      }
      __syncthreads();
      // Dup problems learn which slot buckets hold one and the same key in
      // every tile: those become flat slots (flag bit 1; the key goes to tile
      // 0's key row).  A warp per slot, its lanes over the tiles, kBColBatch
      // loads per lane in flight.
      if (H.dup) {
        const uint32_t lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
        for (uint32_t q = warp; q < tot_slots; q += nwarps) {
          const uint32_t b = __ldcg(A.seg_bucket + P.req_off + q);
          const uint32_t *col = A.rows + P.row0 + b;
          const K *rcol = reps + P.row0 + b;
          bool mixed = false, any = false;
          K kmin = KeyMax<K>::v, kmax = 0;
          for (uint32_t r0 = 0; r0 < nr; r0 += 32 * kBColBatch) {
            uint32_t v[kBColBatch];
#pragma unroll
            for (int j = 0; j < kBColBatch; ++j) {
              const uint32_t r = r0 + j * 32 + lane;
              v[j] = r < nr ? __ldcg(col + (uint64_t)r * P.nb_max) : 0u;
            }
            K rr[kBColBatch];
#pragma unroll
            for (int j = 0; j < kBColBatch; ++j) {
              const uint32_t r = r0 + j * 32 + lane;
              rr[j] = (r < nr && (v[j] & ~kMixed)) ? ldcg_u(rcol + (uint64_t)r * P.nb_max)
                                                    : KeyMax<K>::v;
            }
#pragma unroll
            for (int j = 0; j < kBColBatch; ++j) {
              mixed |= (v[j] & kMixed) != 0;
              if (v[j] & ~kMixed) {
                any = true;
                kmin = rr[j] < kmin ? rr[j] : kmin;
                kmax = rr[j] > kmax ? rr[j] : kmax;
              }
            }
          }
          mixed = __any_sync(0xffffffffu, mixed);
          any = __any_sync(0xffffffffu, any);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const K a2 = __shfl_xor_sync(0xffffffffu, kmin, o);
            const K z2 = __shfl_xor_sync(0xffffffffu, kmax, o);
            kmin = a2 < kmin ? a2 : kmin;
            kmax = z2 > kmax ? z2 : kmax;
          }
          // one key in every tile that saw the bucket, no tile with two
          if (lane == 0 && any && !mixed && kmin == kmax && kmin != KeyMax<K>::v) {
            flag[b] |= 2;
            reps[P.row0 + b] = kmin;
          }
        }
        __syncthreads();
      }
      // key range, flat test and survivor count of each slot
      const uint32_t sper = (tot_slots + nt - 1) / nt;
      const uint32_t s0 = min(tot_slots, tid * sper), s1 = min(tot_slots, s0 + sper);
      uint64_t my_surv = 0;
      // speculation holds when every slot with survivors lies strictly between
      // the buckets of the window's ends (an open end bounds nothing)
      const bool lo_open = H.tau_lo == 0, hi_open = (K)H.tau_hi == KeyMax<K>::v;
      const uint32_t b_tlo = lo_open ? 0u : bucket_of<K>((K)H.tau_lo, (K)H.base, H.shift, lut, nsl);
      const uint32_t b_thi = hi_open ? 0u : bucket_of<K>((K)H.tau_hi, (K)H.base, H.shift, lut, nsl);
      bool outside = false;
      for (uint32_t q = s0; q < s1; ++q) {
        const uint32_t g = P.req_off + q;
        const uint32_t b = __ldcg(A.seg_bucket + g);
        K klo = bucket_lo<K>(b, (K)H.base, H.shift, lut, nsl);
        const K knext = (b + 1 < nb) ? bucket_lo<K>(b + 1, (K)H.base, H.shift, lut, nsl) : K(0);
        // single key iff the next bucket starts one key later (see k_plan), or
        // every tile saw one and the same key in the bucket
        bool single = (knext > klo) ? (knext - klo == K(1)) : (klo == KeyMax<K>::v);
        if (flag[b] & 2u) {
          single = true;
          klo = ldcg_u(reps + P.row0 + b);
        }
        const uint32_t cb = single ? 0u : __ldcg(cnt + b);
        if (cb && ((!lo_open && b <= b_tlo) || (!hi_open && b >= b_thi))) outside = true;
        A.seg_size[g] = cb;
        seg_lo[g] = klo;
        seg_hi[g] = single ? klo : (knext > klo ? knext - K(1) : KeyMax<K>::v);
        A.kcnt[g] = 0;
        A.kcur[g] = 0;
        A.fill[g] = 0;
        my_surv += cb;
      }
      if (__syncthreads_or(outside) == 0 && H.spec_on && tid == 0) A.hdrs[p].spec_ok = 1u;
      uint64_t tot_surv;
      uint64_t off = block_incl_scan(my_surv, &tot_surv, red64) - my_surv;
      if (tid == 0) {
        const uint64_t base = atomicAdd((unsigned long long *)&ctrl->surv_top,
                                        (unsigned long long)tot_surv);
        if (base + tot_surv > A.surv_cap) {
          atomicOr(&ctrl->status, ST_OVERFLOW);
          atomicMax((unsigned long long *)&ctrl->cap_needed,
                    (unsigned long long)(base + tot_surv));
        }
        // compaction cursors carry the position inside the problem in 31 bits
        if (tot_surv >= (uint64_t)kInactive) atomicOr(&ctrl->status, ST_INTERNAL);
        s_base = base;
        A.hdrs[p].surv_off = base;
        A.hdrs[p].num_slots = tot_slots;
      }
      __syncthreads();
      off += s_base;
      for (uint32_t q = s0; q < s1; ++q) {
        const uint32_t g = P.req_off + q;
        A.seg_off[g] = off;
        off += __ldcg(A.seg_size + g);
      }
      __syncthreads();
      // per-slot request counters: in the shared memory after the flags when
      // the slots fit (a top-k puts thousands of requests in a few slots),
      // else the global ones
      uint32_t *s_cnt = reinterpret_cast<uint32_t *>(flag + kBMaxNb);
      uint32_t *s_cur = s_cnt + kBPlanSlots;
      const bool in_smem = tot_slots <= kBPlanSlots;
      if (in_smem)
        for (uint32_t q = tid; q < tot_slots; q += nt) {
          s_cnt[q] = 0;
          s_cur[q] = 0;
        }
      __syncthreads();
      for (uint32_t i = tid; i < P.num_req; i += nt) {
        const uint32_t q = excl[__ldcg(A.req_bucket + P.req_off + i)];
        atomicAdd(in_smem ? &s_cnt[q] : &A.kcnt[P.req_off + q], 1u);
      }
      __syncthreads();
      {
        uint32_t mine = 0;
        for (uint32_t q = s0; q < s1; ++q)
          mine += in_smem ? s_cnt[q] : __ldcg(A.kcnt + P.req_off + q);
        uint32_t t2;
        uint32_t r2 = block_incl_scan(mine, &t2, red32) - mine + P.req_off;
        for (uint32_t q = s0; q < s1; ++q) {
          const uint32_t c = in_smem ? s_cnt[q] : __ldcg(A.kcnt + P.req_off + q);
          if (in_smem) A.kcnt[P.req_off + q] = c;  // the finisher reads the counts
          A.kstart[P.req_off + q] = r2;
          r2 += c;
        }
      }
      // finisher lists: small segments go to one warp each; mid-size ones
      // with few requests to one warp's radix select; the others to a whole
      // CTA each
      {
        auto kind = [&](uint32_t q) -> uint32_t {  // 0 small, 1 warp select, 2 CTA
          const uint32_t sz = __ldcg(A.seg_size + P.req_off + q);
          if (sz <= warp_cap<K>()) return 0u;
          const uint32_t c = in_smem ? s_cnt[q] : __ldcg(A.kcnt + P.req_off + q);
          return sz <= kWarpSelMax && c <= kWarpSelReq ? 1u : 2u;
        };
        uint32_t my[3] = {0, 0, 0};
        for (uint32_t q = s0; q < s1; ++q) {
          const uint32_t t = kind(q);
          my[0] += t == 0u;
          my[1] += t == 1u;
          my[2] += t == 2u;
        }
        uint32_t tot[3], at[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) at[t] = block_incl_scan(my[t], &tot[t], red32) - my[t];
        if (tid == 0) {
          s_lb[0] = atomicAdd(&ctrl->n_small, tot[0]);
          s_lb[1] = atomicAdd(&ctrl->n_wsel, tot[1]);
          s_lb[2] = atomicAdd(&ctrl->n_big, tot[2]);
        }
        __syncthreads();
#pragma unroll
        for (int t = 0; t < 3; ++t) at[t] += s_lb[t];
        for (uint32_t q = s0; q < s1; ++q) {
          const uint32_t g = P.req_off + q, t = kind(q);
          if (t == 0u)
            A.small_list[at[0]++] = g;
          else if (t == 1u)
            A.wsel_list[at[1]++] = g;
          else
            A.big_list[at[2]++] = g;
        }
      }
      __syncthreads();
      for (uint32_t i = tid; i < P.num_req; i += nt) {
        const uint32_t q = excl[__ldcg(A.req_bucket + P.req_off + i)];
        const uint32_t g = P.req_off + q;
        const uint32_t pos =
            __ldcg(A.kstart + g) + atomicAdd(in_smem ? &s_cur[q] : &A.kcur[g], 1u);
        Req e;
        e.rank = __ldcg(A.req_local + P.req_off + i);
        e.out = rq[i].out;
        if (BCHECK(pos < A.num_req && e.out < A.num_req && g < P.req_off + P.num_req, 8, pos, g))
          A.klist[pos] = e;
      }
    }
  }
  st = grid_barrier(ctrl, &s_status, 3);

  // ---------------- phase 4: compaction, the same (problem, tile) items
  if (!(st & (ST_FATAL | ST_OVERFLOW))) {
    if (tid == 0) {
      s_cur = 0xFFFFFFFFu;
      s_bad = false;
    }
    uint32_t *cursor = sm + kBTileLut;
    for (uint32_t t = queue_pop(&ctrl->queue[3], &s_item); t < A.num_tiles;
         t = queue_pop(&ctrl->queue[3], &s_item)) {
      const BTile tl = A.tiles[t];
      const BProb P = A.probs[tl.prob];
      const BHdr H = load_hdr(A.hdrs + tl.prob);
      const uint32_t nsl = 1u << P.nsl_bits;
      if (s_cur != tl.prob)
        for (uint32_t w = tid; w < (nsl + 1) * 32; w += nt) sm[w] = __ldcg(A.luts + P.lut_off + (w >> 5));
      for (uint32_t b = tid; b < ((H.nb + 31) & ~31u); b += nt) cursor[b] = kInactive;
      __syncthreads();
      if (tid == 0) s_cur = tl.prob;
      uint32_t *row = A.rows + P.row0 + (uint64_t)tl.rank * P.nb_max;
      // Positions relative to the problem's survivor range (flat slots have
      // none): the tile takes its share of each slot's segment with one
      // atomic on the slot's fill counter (tiles take their shares in any
      // order; the order of a segment's keys does not matter), and leaves the
      // end of its share in its row for the check below.
      for (uint32_t s = tid; s < H.num_slots; s += nt) {
        const uint32_t g = P.req_off + s;
        if (__ldcg(A.seg_size + g) == 0) continue;
        const uint32_t b = __ldcg(A.seg_bucket + g);
        if (!BCHECK(b < H.nb && s < P.num_req, 10, b, s)) continue;
        const uint32_t c = __ldcg(row + b) & ~kMixed;
        const uint32_t pre = c ? atomicAdd(A.fill + g, c) : 0u;
        const uint32_t at = (uint32_t)(ldcg_u(A.seg_off + g) - H.surv_off + pre);
        cursor[swz(b)] = at;
        row[b] = at + c;
      }
      __syncthreads();
      K *sp = surv + H.surv_off;
      // inactive cursors carry bit 31, so one compare keeps inactive keys out
      // and every store inside the buffer (see compact_one)
      const uint64_t room = A.surv_cap - H.surv_off;
      const uint32_t cap = (uint32_t)(room < (uint64_t)kInactive ? room : kInactive);
      const K base = (K)H.base;
      const uint32_t shift = H.shift;
      const uint32_t ncand = H.spec_ok ? __ldcg(A.cand_cnt + t) : 0xFFFFFFFFu;
      if (H.spec_ok && ncand <= tl.cand_cap) {
        // the tile's complete candidate list holds every key of its slots'
        // buckets (phase 3's check): read it in place of the elements
        const K *cand = reinterpret_cast<const K *>(A.cand) + tl.cand_off;
        for (uint32_t i = tid; i < ncand; i += nt) {
          const K k = ldcg_u(cand + i);
          const uint32_t ub = bucket_of_lane<K>(k, base, shift, lane_lut, nsl);
          if (!BCHECK(ub < H.nb, 9, ub, H.nb)) continue;
          const uint32_t pos = atomicAdd(&cursor[swz(ub)], 1u);
          st_global_if(sp + pos, k, pos < cap);
        }
        if (tid == 0) atomicAdd(&ctrl->spec_tiles, 1u);
      } else if (H.heavy) {
        // Sorted runs and few distinct keys: the cursor atomics return
        // positions, which lanes of one address receive one at a time, so
        // lanes of a warp sharing a bucket take one atomic (match.any) and
        // consecutive positions.  A key whose bucket fails the check (the call
        // is then failed) stays in the vote under bucket 0 but is not stored.
        for_range_p<T>(P.x, P.flt, tl.begin, tl.end, [&](K k, bool full) {
          uint32_t ub = bucket_of_lane<K>(k, base, shift, lane_lut, nsl);
          const bool ok = BCHECK(ub < H.nb, 9, ub, H.nb);
          if (!ok) ub = 0;
          uint32_t pos;
          if (full) {
            const uint32_t peers = __match_any_sync(0xffffffffu, ub);
            const uint32_t lane = threadIdx.x & 31;
            const int leader = __ffs(peers) - 1;
            uint32_t p0 = 0;
            if ((int)lane == leader) p0 = atomicAdd(&cursor[swz(ub)], (uint32_t)__popc(peers));
            p0 = __shfl_sync(peers, p0, leader);
            pos = p0 + __popc(peers & ((1u << lane) - 1u));
          } else {
            pos = atomicAdd(&cursor[swz(ub)], 1u);
          }
          st_global_if(sp + pos, k, ok && pos < cap);
        });
      } else {
        // eight vectors in flight, four for float batches (whose kernel
        // spills 256 bytes of loads with eight)
        constexpr int CV = std::is_same<T, float>::value ? 4 : kBTileVecs;
        for_range_p<T, CV>(P.x, P.flt, tl.begin, tl.end, [&](K k, bool) {
          uint32_t ub = bucket_of_lane<K>(k, base, shift, lane_lut, nsl);
          if (!BCHECK(ub < H.nb, 9, ub, H.nb)) return;
          const uint32_t pos = atomicAdd(&cursor[swz(ub)], 1u);
          st_global_if(sp + pos, k, pos < cap);
        });
      }
      __syncthreads();
      // each cursor must end where the tile's share of the segment ends
      for (uint32_t s = tid; s < H.num_slots; s += nt) {
        const uint32_t g = P.req_off + s;
        if (__ldcg(A.seg_size + g) == 0) continue;
        const uint32_t b = __ldcg(A.seg_bucket + g);
        if (cursor[swz(b)] != __ldcg(row + b)) s_bad = true;
      }
    }
    __syncthreads();
    if (tid == 0 && s_bad) atomicOr(&ctrl->status, ST_INTERNAL);
  }
  st = grid_barrier(ctrl, &s_status, 4);

  // ---------------- phase 5: finish every slot
  // one slot by the whole CTA; a slot whose needed bins exceed the shared
  // memory goes to the host's recursion
  auto cta_finish = [&](uint32_t g) {
    // one vector per thread and chunk: the kernel's other phases already
    // hold its register budget
    const bool done = finish_slot<K, OutT, 1>(
        surv + ldcg_u(A.seg_off + g), __ldcg(A.seg_size + g), ldcg_u(seg_lo + g), ldcg_u(seg_hi + g),
        A.klist + __ldcg(A.kstart + g), __ldcg(A.kcnt + g), A.bcap, sm, out);
    if (!done && tid == 0) {
      const uint32_t d = atomicAdd(&ctrl->deferred_count, 1u);
      A.deferred[d] = g;
      atomicOr(&ctrl->status, ST_DEFERRED);
    }
  };
  // mid-size slots by warps or, when the batch has few, by CTAs after the
  // large ones.  The count is final since phase 3 and every CTA reads it,
  // whatever the status: one choice for the grid, and so for the barrier
  // that only the warps' fallback needs.
  const uint32_t n_wsel_all = __ldcg(&ctrl->n_wsel);
  const bool wsel_warps = n_wsel_all >= kWselPerCta * gridDim.x;
  if (!(st & (ST_FATAL | ST_OVERFLOW))) {
    const uint32_t n_big = __ldcg(&ctrl->n_big), n_small = __ldcg(&ctrl->n_small);
    const uint32_t n_wsel = wsel_warps ? n_wsel_all : 0u;
    const uint32_t n_cta = n_big + (wsel_warps ? 0u : n_wsel_all);
    // large segments first, a whole CTA each
    for (uint32_t i = queue_pop(&ctrl->queue[4], &s_item); i < n_cta;
         i = queue_pop(&ctrl->queue[4], &s_item)) {
      const uint32_t g = i < n_big ? __ldcg(A.big_list + i) : __ldcg(A.wsel_list + (i - n_big));
      if (!BCHECK(i < A.num_req && g < A.num_req &&
                      ldcg_u(A.seg_off + g) + __ldcg(A.seg_size + g) <= A.surv_cap &&
                      __ldcg(A.kstart + g) + __ldcg(A.kcnt + g) <= A.num_req,
                  11, i, g))
        continue;
#ifdef GGKS_BATCH_CHECKS
      {
        bool bad = false;
        const uint32_t sz = __ldcg(A.seg_size + g), ks = __ldcg(A.kstart + g);
        for (uint32_t j = tid; j < __ldcg(A.kcnt + g); j += nt) {
          const Req e = A.klist[ks + j];
          if (e.out >= A.num_req || (sz && e.rank >= sz)) bad = true;
        }
        if (__syncthreads_or(bad)) {
          if (tid == 0) BCHECK(false, 13, g, sz);
          continue;
        }
      }
#endif
      cta_finish(g);
    }
    // then the mid-size and the small ones, one warp each (the queue pop
    // above ended with a barrier, so no thread of this CTA still uses the
    // shared memory)
    const uint32_t lane = tid & 31;
    K *wbuf = reinterpret_cast<K *>(sm) + (size_t)(tid >> 5) * warp_cap<K>();
    // the select's histogram, after every warp's buffer
    uint32_t *whist = sm + (size_t)(nt / 32) * (kBWarpBytes / 4) +
                      (size_t)(tid >> 5) * (kWarpSelBins + kWarpSelReq);
    // mid-size slots (the longer warp jobs) first: radix select, or to the
    // CTA queue after the next barrier when the needed bins do not fit the
    // warp's buffer
    while (true) {
      uint32_t i = 0;
      if (lane == 0) i = atomicAdd(&ctrl->wsel_pop, 1u);
      i = __shfl_sync(0xffffffffu, i, 0);
      if (i >= n_wsel) break;
      const uint32_t g = __ldcg(A.wsel_list + i);
      if (!BCHECK(i < A.num_req && g < A.num_req && __ldcg(A.seg_size + g) > warp_cap<K>() &&
                      __ldcg(A.seg_size + g) <= kWarpSelMax && __ldcg(A.kcnt + g) <= kWarpSelReq &&
                      ldcg_u(A.seg_off + g) + __ldcg(A.seg_size + g) <= A.surv_cap &&
                      __ldcg(A.kstart + g) + __ldcg(A.kcnt + g) <= A.num_req,
                  15, i, g))
        continue;
#ifdef GGKS_BATCH_CHECKS
      {
        bool bad = false;
        const uint32_t sz = __ldcg(A.seg_size + g), ks = __ldcg(A.kstart + g);
        for (uint32_t j = lane; j < __ldcg(A.kcnt + g); j += 32) {
          const Req e = A.klist[ks + j];
          if (e.out >= A.num_req || e.rank >= sz) bad = true;
        }
        if (__any_sync(0xffffffffu, bad)) {
          if (lane == 0) BCHECK(false, 16, g, sz);
          continue;
        }
      }
#endif
      const bool done = finish_warp_select<K, OutT>(
          surv + ldcg_u(A.seg_off + g), __ldcg(A.seg_size + g), ldcg_u(seg_lo + g),
          ldcg_u(seg_hi + g), A.klist + __ldcg(A.kstart + g), __ldcg(A.kcnt + g), wbuf,
          warp_cap<K>(), whist, out);
      if (!done && lane == 0) A.retry_list[atomicAdd(&ctrl->n_retry, 1u)] = g;
    }
    while (true) {
      uint32_t i = 0;
      if (lane == 0) i = atomicAdd(&ctrl->small_pop, 1u);
      i = __shfl_sync(0xffffffffu, i, 0);
      if (i >= n_small) break;
      const uint32_t g = __ldcg(A.small_list + i);
      if (!BCHECK(i < A.num_req && g < A.num_req && __ldcg(A.seg_size + g) <= warp_cap<K>() &&
                      ldcg_u(A.seg_off + g) + __ldcg(A.seg_size + g) <= A.surv_cap &&
                      __ldcg(A.kstart + g) + __ldcg(A.kcnt + g) <= A.num_req,
                  12, i, g))
        continue;
#ifdef GGKS_BATCH_CHECKS
      {
        bool bad = false;
        const uint32_t sz = __ldcg(A.seg_size + g), ks = __ldcg(A.kstart + g);
        for (uint32_t j = lane; j < __ldcg(A.kcnt + g); j += 32) {
          const Req e = A.klist[ks + j];
          if (e.out >= A.num_req || (sz && e.rank >= sz)) bad = true;
        }
        if (__any_sync(0xffffffffu, bad)) {
          if (lane == 0) BCHECK(false, 14, g, sz);
          continue;
        }
      }
#endif
      // one to kWarpSelReq requests: radix select; more (a top-k's bucket),
      // or needed bins that do not fit: the segment is sorted
      const uint32_t sz = __ldcg(A.seg_size + g), kc = __ldcg(A.kcnt + g);
      const Req *rq = A.klist + __ldcg(A.kstart + g);
      const K *src = surv + ldcg_u(A.seg_off + g);
      if (sz == 0 || kc > kWarpSelReq ||
          !finish_warp_select<K, OutT>(src, sz, ldcg_u(seg_lo + g), ldcg_u(seg_hi + g), rq, kc,
                                       wbuf, warp_cap<K>(), whist, out))
        finish_warp<K, OutT>(src, sz, ldcg_u(seg_lo + g), rq, kc, wbuf, out);
    }
  }
  // the mid-size slots no warp could answer, a whole CTA each
  if (wsel_warps) {
    st = grid_barrier(ctrl, &s_status, -1);
    if (!(st & (ST_FATAL | ST_OVERFLOW))) {
      const uint32_t n_retry = __ldcg(&ctrl->n_retry);
      for (uint32_t i = queue_pop(&ctrl->retry_pop, &s_item); i < n_retry;
           i = queue_pop(&ctrl->retry_pop, &s_item)) {
        const uint32_t g = __ldcg(A.retry_list + i);
        if (!BCHECK(i < A.num_req && g < A.num_req, 17, i, g)) continue;
        cta_finish(g);
      }
    }
  }
  __syncthreads();
  if (blockIdx.x == 0 && tid == 0) ctrl->t_ns[kBPhases] = global_ns();
}

}  // namespace ggks
