// ggks_device.cuh -- device side of the GB300 GGKS bucket multiselect.
//
// The pipeline (one problem; every pass is a kernel on one stream, no host
// round trip between passes):
//
//   (a) keys      order-preserving float/double -> uint key map
//                 (keyConversion.cu:9-23), applied on load, never stored.
//   (b) sample    k_sample_lut: S pseudo-random keys are gathered; the last
//                 CTA builds a range-adaptive splitter table (LUT) from them:
//                 4096 equal-width slices of the sample's key span, each
//                 slice cut into 2^b sub-buckets with b chosen from the
//                 slice's sample count, so that buckets hold about equal
//                 numbers of elements.  Keys below / above the sample span go
//                 to open-ended edge buckets, so no min/max pass is needed.
//                 Replaces the reference's minmax + 1024-sample 17-pivot /
//                 16-slope construction (bucketMultiselect.cu:414-508,
//                 :534-547, :659-667).
//   (c) hist      k_hist: persistent grid-stride pass over the input with
//                 128-bit loads; per-CTA shared-memory histogram of up to
//                 nb_max buckets (warp-aggregated with match.any when the
//                 sample shows heavy duplicates); one row of counts per CTA.
//                 Replaces assignSmartBucket (bucketMultiselect.cu:129-205)
//                 without its 4n-byte element-to-bucket array.
//   (d) scan      k_scan: sums the per-CTA rows per bucket and computes the
//                 global exclusive prefix with a single-pass decoupled
//                 look-back scan (bounded spin).  Replaces sumCounts
//                 (:214-221) and the host walk of findKBuckets (:87-111).
//   (e) plan      k_plan: one CTA maps every requested rank to its bucket and
//                 local rank, answers ranks that fall in single-key buckets
//                 directly, assigns compact slots to the active buckets and
//                 groups the requests by slot.  Replaces the host reindex loop
//                 and reindexCounts (:714-756).
//   (f) compact   k_compact: second pass over the input; elements of active
//                 buckets are appended to their slot's segment of the
//                 survivor buffer (keys).  Replaces copyElements (:249-308).
//   (g) finish    k_finish: per segment, an in-shared-memory sort of the
//                 survivors and a gather of the requested ranks.  Replaces
//                 thrust::sort of all survivors + copyValuesInChunk
//                 (:799-818).  Segments larger than shared memory are listed
//                 for a recursive re-selection by the host.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ggks {

// ---------------------------------------------------------------------------
// constants and shared structs
// ---------------------------------------------------------------------------
constexpr int kLutIdxBits = 12;
constexpr uint32_t kLutIdx = 1u << kLutIdxBits;  // slices over the sample span
constexpr uint32_t kLutEntries = kLutIdx + 1;    // + one for keys above the span
constexpr int kMaxSubBits = 20;                  // at most 2^20 buckets per slice
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;
constexpr int kSpinLimit = 1 << 22;              // bounded device-side waits

// status bits in Ctrl::status
enum : uint32_t {
  ST_OVERFLOW = 1u,  // survivors exceed the survivor buffer: host regrows, re-runs (f)+(g)
  ST_DEFERRED = 2u,  // some segments exceed shared memory: host re-selects them
  ST_TIMEOUT = 4u,   // a bounded wait gave up
  ST_INTERNAL = 8u,  // a consistency check failed (counts do not add up to n)
};
constexpr uint32_t ST_FATAL = ST_TIMEOUT | ST_INTERNAL;

// One selection request: ascending 0-based rank and the output position.
struct Req {
  uint32_t rank;
  uint32_t out;
};

// Device control block (lives in the workspace; zeroed once at allocation).
struct Ctrl {
  uint32_t status;
  uint32_t num_slots;
  uint64_t total_surv;
  uint32_t deferred_count;
  uint32_t sample_done;  // last-CTA ticket of k_sample_lut (reset by that CTA)
  uint32_t scan_ticket;  // dynamic tile ids of k_scan (reset by k_plan)
  uint32_t nb;           // buckets in use
  uint64_t cap_needed;
};

template <class K>
struct LutHeader {
  K base;          // smallest sampled key
  uint32_t shift;  // slice index = (key - base) >> shift
  uint32_t nb;     // number of buckets
  uint32_t heavy;  // 1: warp-aggregate histogram updates
  uint32_t pad;
};

// ---------------------------------------------------------------------------
// (a) order-preserving keys (keyConversion.cu:9-23 preProcess, :29-42
// postProcess).  Key types are unsigned; uint32/uint64 inputs are their own
// keys (the uint64 form carries float64 keys through a recursive level).
// ---------------------------------------------------------------------------
template <class T>
struct Traits;

template <>
struct Traits<float> {
  using K = uint32_t;
  using Vec = uint4;
  static constexpr int kPerVec = 4;
  __device__ __forceinline__ static K key(float v) {
    uint32_t b = __float_as_uint(v);
    return b ^ ((uint32_t)((int32_t)b >> 31) | 0x80000000u);
  }
  __device__ __forceinline__ static K key_bits(uint32_t b) {
    return b ^ ((uint32_t)((int32_t)b >> 31) | 0x80000000u);
  }
  __device__ __forceinline__ static float value(K k) {
    return __uint_as_float(k ^ (((k >> 31) - 1u) | 0x80000000u));
  }
};

template <>
struct Traits<double> {
  using K = uint64_t;
  using Vec = ulonglong2;
  static constexpr int kPerVec = 2;
  __device__ __forceinline__ static K key(double v) {
    uint64_t b = (uint64_t)__double_as_longlong(v);
    return b ^ ((uint64_t)((int64_t)b >> 63) | 0x8000000000000000ull);
  }
  __device__ __forceinline__ static K key_bits(uint64_t b) {
    return b ^ ((uint64_t)((int64_t)b >> 63) | 0x8000000000000000ull);
  }
  __device__ __forceinline__ static double value(K k) {
    return __longlong_as_double((long long)(k ^ (((k >> 63) - 1ull) | 0x8000000000000000ull)));
  }
};

template <>
struct Traits<uint32_t> {
  using K = uint32_t;
  using Vec = uint4;
  static constexpr int kPerVec = 4;
  __device__ __forceinline__ static K key(uint32_t v) { return v; }
  __device__ __forceinline__ static K key_bits(uint32_t b) { return b; }
  __device__ __forceinline__ static uint32_t value(K k) { return k; }
};

template <>
struct Traits<uint64_t> {
  using K = uint64_t;
  using Vec = ulonglong2;
  static constexpr int kPerVec = 2;
  __device__ __forceinline__ static K key(uint64_t v) { return v; }
  __device__ __forceinline__ static K key_bits(uint64_t b) { return b; }
  __device__ __forceinline__ static uint64_t value(K k) { return k; }
};

template <class K>
struct KeyMax;
template <>
struct KeyMax<uint32_t> {
  static constexpr uint32_t v = 0xFFFFFFFFu;
  static constexpr int bits = 32;
};
template <>
struct KeyMax<uint64_t> {
  static constexpr uint64_t v = 0xFFFFFFFFFFFFFFFFull;
  static constexpr int bits = 64;
};

// the four keys held by one 128-bit vector (two for 64-bit types)
template <class T>
__device__ __forceinline__ void vec_keys(const uint4 &v, uint32_t (&k)[4]) {
  k[0] = Traits<T>::key_bits(v.x);
  k[1] = Traits<T>::key_bits(v.y);
  k[2] = Traits<T>::key_bits(v.z);
  k[3] = Traits<T>::key_bits(v.w);
}
template <class T>
__device__ __forceinline__ void vec_keys(const ulonglong2 &v, uint64_t (&k)[2]) {
  k[0] = Traits<T>::key_bits(v.x);
  k[1] = Traits<T>::key_bits(v.y);
}

// ---------------------------------------------------------------------------
// small PTX helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(uint64_t *p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t *p) {
  return *(const volatile uint32_t *)p;
}

// streaming 128-bit load that does not allocate in L1
template <class V>
__device__ __forceinline__ V ldg_stream(const V *p);
template <>
__device__ __forceinline__ uint4 ldg_stream<uint4>(const uint4 *p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}
template <>
__device__ __forceinline__ ulonglong2 ldg_stream<ulonglong2>(const ulonglong2 *p) {
  ulonglong2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u64 {%0,%1}, [%2];"
               : "=l"(v.x), "=l"(v.y)
               : "l"(p));
  return v;
}

// right shift that yields 0 for shift >= width
__device__ __forceinline__ uint32_t shr_clamp(uint32_t d, uint32_t s) {
  return __funnelshift_r(d, 0u, s);  // shf.r.clamp: shift clamped to 32
}
__device__ __forceinline__ uint32_t shr_clamp(uint64_t d, uint32_t s) {
  return s >= 64 ? 0u : (uint32_t)(d >> s);
}

template <class K>
__device__ __forceinline__ int bitlen(K v);
template <>
__device__ __forceinline__ int bitlen<uint32_t>(uint32_t v) {
  return 32 - __clz(v);
}
template <>
__device__ __forceinline__ int bitlen<uint64_t>(uint64_t v) {
  return 64 - __clzll((long long)v);
}

__device__ __forceinline__ uint32_t hash32(uint32_t a) {
  // 32-bit integer finaliser (murmur3 fmix32)
  a ^= a >> 16;
  a *= 0x85ebca6bu;
  a ^= a >> 13;
  a *= 0xc2b2ae35u;
  a ^= a >> 16;
  return a;
}

// ---------------------------------------------------------------------------
// bucket function: slice lookup + sub-bucket by the next bits of the key
// ---------------------------------------------------------------------------
// lut[j] = {C, rs}: bucket = C + ((key - base) >> rs) (mod 2^32).  For a slice
// j cut into 2^b sub-buckets starting at bucket B_j: rs = shift - b and
// C = B_j - (j << b).  Merged empty slices use b = 0; the top entry (keys
// above the sampled span) uses rs = key width, i.e. a constant bucket.
// Bucket 0 holds the keys below `base` (the sampled minimum); the table's
// buckets start at 1, so the first of them starts exactly at `base`.
template <class K>
__device__ __forceinline__ uint32_t bucket_of(K key, K base, uint32_t shift, const uint2 *lut) {
  const K d = key - base;  // wraps for key < base; that result is discarded
  const K idx = d >> shift;
  const uint32_t j = idx < (K)kLutIdx ? (uint32_t)idx : kLutIdx;
  const uint2 e = lut[j];
  const uint32_t b = e.x + shr_clamp(d, e.y);
  return key < base ? 0u : b;
}

// smallest key that maps to bucket b (b < nb); bucket 0 starts at key 0.
template <class K>
__device__ __forceinline__ K bucket_lo(uint32_t b, K base, uint32_t shift, const uint2 *lut) {
  if (b == 0) return K(0);
  // first entry whose last bucket >= b: entries' bucket ranges are
  // non-decreasing in j.  last_bucket(j) = C_j + (((j+1) << shift) - 1) >> rs_j
  uint32_t lo = 0, hi = kLutIdx;  // search over [0, kLutIdx]
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    uint2 e = lut[mid];
    uint32_t last;
    if (mid == kLutIdx) {
      last = e.x;
    } else {
      K dmax = (((K)(mid + 1)) << shift) - 1;
      last = e.x + shr_clamp(dmax, e.y);
    }
    if (last >= b)
      hi = mid;
    else
      lo = mid + 1;
  }
  uint2 e = lut[lo];
  if (lo == kLutIdx) return base + (((K)kLutIdx) << shift);
  K dstart = ((K)lo) << shift;
  uint32_t first = e.x + shr_clamp(dstart, e.y);
  if (first >= b) return base + dstart;
  // within slice lo: sub-bucket (b - first) starts at dstart + ((b - first) << rs)
  return base + dstart + (((K)(b - first)) << e.y);
}

// ---------------------------------------------------------------------------
// block reductions / scans (blockDim.x multiple of 32, <= 1024)
// ---------------------------------------------------------------------------
template <class V>
__device__ __forceinline__ V warp_incl_scan(V v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    V t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// inclusive scan over the block; returns the block total through *total.
template <class V>
__device__ __forceinline__ V block_incl_scan(V v, V *total, V *sh /* >= 33 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  V s = warp_incl_scan(v);
  if (lane == 31) sh[warp] = s;
  __syncthreads();
  if (warp == 0) {
    V w = lane < nwarps ? sh[lane] : V(0);
    V ws = warp_incl_scan(w);
    if (lane < nwarps) sh[lane] = ws - w;  // exclusive warp offsets
    if (lane == nwarps - 1) sh[32] = ws;
  }
  __syncthreads();
  V r = s + sh[warp];
  *total = sh[32];
  __syncthreads();
  return r;
}

template <class V, class Op>
__device__ __forceinline__ V block_reduce(V v, Op op, V *sh /* >= 32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  V r = sh[0];
  for (int w = 1; w < nwarps; ++w) r = op(r, sh[w]);
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// (b) sample + splitter table
// ---------------------------------------------------------------------------
// Grid: ceil(S / 1024) CTAs of 1024 threads.  Every thread gathers one key;
// the last CTA to finish builds the table.
template <class T>
__global__ void __launch_bounds__(1024) k_sample_lut(const T *__restrict__ x, uint64_t n,
                                                     uint32_t S, uint32_t seed,
                                                     typename Traits<T>::K *samples,
                                                     Ctrl *ctrl,
                                                     LutHeader<typename Traits<T>::K> *hdr,
                                                     uint2 *lut, uint32_t nb_max) {
  using K = typename Traits<T>::K;
  __shared__ uint32_t cnt[kLutEntries + 3];
  __shared__ K redk[33];
  __shared__ uint32_t red32[33];
  __shared__ uint32_t s_last;

  const uint32_t tid = threadIdx.x;
  const uint32_t i = blockIdx.x * blockDim.x + tid;
  if (i < S) {
    uint64_t pos;
    if ((uint64_t)S >= n)
      pos = i;
    else
      pos = ((uint64_t)hash32(i * 0x9E3779B9u + seed) * n) >> 32;
    samples[i] = Traits<T>::key(x[pos]);
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&ctrl->sample_done, 1u) == gridDim.x - 1) ? 1u : 0u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // --- span of the sample
  K kmin = KeyMax<K>::v, kmax = 0;
  for (uint32_t s = tid; s < S; s += blockDim.x) {
    K k = __ldcg(samples + s);
    kmin = k < kmin ? k : kmin;
    kmax = k > kmax ? k : kmax;
  }
  kmin = block_reduce(kmin, [](K a, K b) { return a < b ? a : b; }, redk);
  kmax = block_reduce(kmax, [](K a, K b) { return a > b ? a : b; }, redk);
  const int bl = bitlen<K>(kmax - kmin);
  const uint32_t shift = bl > kLutIdxBits ? (uint32_t)(bl - kLutIdxBits) : 0u;
  const int bcap = (int)(shift < (uint32_t)kMaxSubBits ? shift : (uint32_t)kMaxSubBits);

  // --- sample counts per slice
  for (uint32_t j = tid; j < kLutEntries + 3; j += blockDim.x) cnt[j] = 0;
  __syncthreads();
  for (uint32_t s = tid; s < S; s += blockDim.x) {
    K k = __ldcg(samples + s);
    atomicAdd(&cnt[(uint32_t)((k - kmin) >> shift)], 1u);
  }
  __syncthreads();

  // Each thread owns 4 consecutive slices [4 tid, 4 tid + 4); thread 0 also
  // owns the top entry kLutIdx (appended after the scan).
  int lc[4];
  uint32_t c[4];
  bool prev_nonempty[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t j = 4 * tid + q;
    c[q] = cnt[j];
    lc[q] = c[q] ? (c[q] == 1 ? 0 : 32 - __clz(c[q] - 1)) : -1;  // ceil(log2 c)
    prev_nonempty[q] = (j == 0) ? true : (cnt[j - 1] != 0);
  }
  const bool top_run_start = cnt[kLutIdx - 1] != 0;

  auto contrib = [&](int q, int t) -> uint32_t {
    if (c[q]) {
      int b = lc[q] - t;
      b = b < 0 ? 0 : (b > bcap ? bcap : b);
      return 1u << b;
    }
    return prev_nonempty[q] ? 1u : 0u;
  };
  // buckets in use for threshold t: the low-edge bucket 0, the slices, and
  // the top entry when it starts a run of its own
  auto total_for = [&](int t) -> uint32_t {
    uint32_t s = contrib(0, t) + contrib(1, t) + contrib(2, t) + contrib(3, t);
    s = block_reduce(s, [](uint32_t a, uint32_t b) { return a + b; }, red32);
    return 1u + s + (top_run_start ? 1u : 0u);
  };
  // smallest t with total(t) <= nb_max (total is non-increasing in t)
  int tlo = -kMaxSubBits - 1, thi = 33;
  while (tlo < thi) {
    int mid = (tlo + thi) >> 1;  // arithmetic shift: floor for negatives
    if (total_for(mid) <= nb_max)
      thi = mid;
    else
      tlo = mid + 1;
  }
  const int t = tlo;

  uint32_t my[4], mysum = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    my[q] = contrib(q, t);
    mysum += my[q];
  }
  uint32_t total;
  uint32_t incl = block_incl_scan(mysum, &total, red32);
  uint32_t run = incl - mysum + 1u;  // bucket 0 is the low edge
  uint32_t max_per_bucket = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t j = 4 * tid + q;
    uint2 e;
    if (c[q]) {
      int b = lc[q] - t;
      b = b < 0 ? 0 : (b > bcap ? bcap : b);
      e.x = run - (j << b);
      e.y = shift - (uint32_t)b;
      uint32_t per = c[q] >> b;
      max_per_bucket = per > max_per_bucket ? per : max_per_bucket;
    } else {
      uint32_t B = prev_nonempty[q] ? run : run - 1u;
      e.x = B - j;  // (d >> shift) == j on this slice
      e.y = shift;
    }
    lut[j] = e;
    run += my[q];
  }
  max_per_bucket = block_reduce(max_per_bucket, [](uint32_t a, uint32_t b) { return a > b ? a : b; },
                                red32);
  if (tid == 0) {
    const uint32_t nb = 1u + total + (top_run_start ? 1u : 0u);
    uint2 e;
    e.x = top_run_start ? total + 1u : total;
    e.y = (uint32_t)KeyMax<K>::bits;
    lut[kLutIdx] = e;
    LutHeader<K> h;
    h.base = kmin;
    h.shift = shift;
    h.nb = nb;
    // a bucket expected to hold >= 16x the mean: warp-aggregate updates
    h.heavy = ((uint64_t)max_per_bucket * nb >= 16ull * S && S >= 256) ? 1u : 0u;
    h.pad = 0;
    *hdr = h;
    ctrl->nb = nb;
    ctrl->sample_done = 0;  // re-arm for the next call on this workspace
  }
}

// ---------------------------------------------------------------------------
// (c) histogram pass
// ---------------------------------------------------------------------------
// Persistent grid; every CTA owns one row of nb_max counters in `partials`.
// The vector body covers the 16-byte aligned middle of the input in tiles of
// UNROLL vectors per thread; the ragged head/tail go through a scalar path.
template <class T>
struct Span {
  uint64_t head;   // scalar elements before the first aligned vector
  uint64_t nvec;   // aligned vectors
  uint64_t tail0;  // first scalar element after the vectors
};
template <class T>
__device__ __forceinline__ Span<T> split_span(const T *x, uint64_t n) {
  Span<T> s;
  uint64_t mis = (uint64_t)(uintptr_t)x & 15u;
  uint64_t head = mis ? (16u - mis) / sizeof(T) : 0;
  if (head > n) head = n;
  s.head = head;
  s.nvec = (n - head) / Traits<T>::kPerVec;
  s.tail0 = head + s.nvec * Traits<T>::kPerVec;
  return s;
}

template <bool HEAVY>
__device__ __forceinline__ void hist_add(uint32_t *hist, uint32_t b) {
  if (HEAVY) {
    const uint32_t peers = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&hist[b], (uint32_t)__popc(peers));
  } else {
    atomicAdd(&hist[b], 1u);
  }
}

template <class T, int UNROLL, bool HEAVY>
__device__ __forceinline__ void hist_body(const T *__restrict__ x, uint64_t n, uint32_t *hist,
                                          const uint2 *lut, typename Traits<T>::K base,
                                          uint32_t shift) {
  using K = typename Traits<T>::K;
  using V = typename Traits<T>::Vec;
  constexpr int PV = Traits<T>::kPerVec;
  const Span<T> sp = split_span(x, n);
  const V *xv = reinterpret_cast<const V *>(x + sp.head);
  const uint64_t tile_v = (uint64_t)blockDim.x * UNROLL;
  const uint64_t ntiles = sp.nvec / tile_v;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const V *p = xv + tile * tile_v + threadIdx.x;
    V v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) v[u] = ldg_stream(p + (uint64_t)u * blockDim.x);
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      K k[PV];
      vec_keys<T>(v[u], k);
#pragma unroll
      for (int q = 0; q < PV; ++q) hist_add<HEAVY>(hist, bucket_of<K>(k[q], base, shift, lut));
    }
  }
  // leftover vectors (fewer than one tile) and the scalar head / tail
  const uint32_t owner = (uint32_t)(ntiles % gridDim.x);
  if (blockIdx.x == owner) {
    for (uint64_t vi = ntiles * tile_v + threadIdx.x; vi < sp.nvec; vi += blockDim.x) {
      V vv = ldg_stream(xv + vi);
      K k[PV];
      vec_keys<T>(vv, k);
#pragma unroll
      for (int q = 0; q < PV; ++q) atomicAdd(&hist[bucket_of<K>(k[q], base, shift, lut)], 1u);
    }
    for (uint64_t e = threadIdx.x; e < sp.head; e += blockDim.x)
      atomicAdd(&hist[bucket_of<K>(Traits<T>::key(x[e]), base, shift, lut)], 1u);
    for (uint64_t e = sp.tail0 + threadIdx.x; e < n; e += blockDim.x)
      atomicAdd(&hist[bucket_of<K>(Traits<T>::key(x[e]), base, shift, lut)], 1u);
  }
}

template <class T, int UNROLL>
__global__ void __launch_bounds__(1024, 1)
    k_hist(const T *__restrict__ x, uint64_t n, const LutHeader<typename Traits<T>::K> *hdr,
           const uint2 *__restrict__ lut_g, uint32_t *__restrict__ partials, uint32_t nb_max,
           const Ctrl *ctrl) {
  using K = typename Traits<T>::K;
  extern __shared__ uint4 smem_raw[];
  uint2 *lut = reinterpret_cast<uint2 *>(smem_raw);
  uint32_t *hist = reinterpret_cast<uint32_t *>(lut + kLutEntries + 1);
  if (ctrl->status & ST_FATAL) return;
  const LutHeader<K> h = *hdr;
  for (uint32_t j = threadIdx.x; j < kLutEntries; j += blockDim.x) lut[j] = lut_g[j];
  for (uint32_t b = threadIdx.x; b < h.nb; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  if (h.heavy)
    hist_body<T, UNROLL, true>(x, n, hist, lut, h.base, h.shift);
  else
    hist_body<T, UNROLL, false>(x, n, hist, lut, h.base, h.shift);
  __syncthreads();
  uint32_t *row = partials + (uint64_t)blockIdx.x * nb_max;
  for (uint32_t b = threadIdx.x; b < h.nb; b += blockDim.x) row[b] = hist[b];
}

// ---------------------------------------------------------------------------
// (d) reduce the per-CTA rows and scan (decoupled look-back, one pass)
// ---------------------------------------------------------------------------
constexpr int kScanTile = 256;
constexpr uint64_t kFlagAgg = 1ull << 62, kFlagIncl = 2ull << 62;
constexpr uint64_t kValMask = (1ull << 62) - 1;

template <class K>
__global__ void __launch_bounds__(kScanTile)
    k_scan(const uint32_t *__restrict__ partials, uint32_t rows, uint32_t nb_max,
           const LutHeader<K> *hdr, uint32_t *__restrict__ counts, uint32_t *__restrict__ excl,
           uint64_t *tile_state, Ctrl *ctrl) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t red[33];
  __shared__ uint64_t s_prefix;
  if (ctrl->status & ST_FATAL) return;
  const uint32_t nb = hdr->nb;
  if (threadIdx.x == 0) s_tile = atomicAdd(&ctrl->scan_ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  if ((uint64_t)tile * kScanTile >= nb) return;
  const uint32_t b = tile * kScanTile + threadIdx.x;
  uint32_t c = 0;
  if (b < nb) {
    const uint32_t *p = partials + b;
    uint32_t r = 0;
    uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (; r + 8 <= rows; r += 8) {
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] += __ldcg(p + (uint64_t)(r + q) * nb_max);
    }
    for (; r < rows; ++r) acc[0] += __ldcg(p + (uint64_t)r * nb_max);
#pragma unroll
    for (int q = 0; q < 8; ++q) c += acc[q];
  }
  uint32_t agg;
  const uint32_t incl = block_incl_scan(c, &agg, red);

  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    uint64_t prefix = 0;
    if (tile == 0) {
      if (lane == 0) st_release_u64(&tile_state[0], kFlagIncl | agg);
    } else {
      if (lane == 0) st_release_u64(&tile_state[tile], kFlagAgg | agg);
      int64_t pred = (int64_t)tile - 1;
      bool timed_out = false;
      while (true) {
        const int64_t p = pred - lane;
        uint64_t st = 0;
        int iters = 0;
        while (true) {
          st = p >= 0 ? ld_acquire_u64(&tile_state[p]) : kFlagIncl;
          if (__all_sync(0xffffffffu, (st >> 62) != 0)) break;
          if (++iters > kSpinLimit) {
            timed_out = true;
            break;
          }
          __nanosleep(64);
        }
        if (timed_out) break;
        const uint32_t incl_mask = __ballot_sync(0xffffffffu, (st >> 62) == 2);
        const int first = incl_mask ? __ffs(incl_mask) - 1 : 32;
        uint64_t v = (lane <= first) ? (st & kValMask) : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        prefix += v;
        if (incl_mask) break;
        pred -= 32;
      }
      if (timed_out) {
        if (lane == 0) atomicOr(&ctrl->status, ST_TIMEOUT);
        prefix = 0;
      }
      if (lane == 0) st_release_u64(&tile_state[tile], kFlagIncl | (prefix + agg));
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  if (b < nb) {
    counts[b] = c;
    excl[b] = (uint32_t)(s_prefix + incl - c);
  }
}

// ---------------------------------------------------------------------------
// (e) plan: requests -> buckets -> slots; request lists per slot
// ---------------------------------------------------------------------------
// One CTA of 1024 threads.  Dynamic shared memory: excl[nb_max] (u32),
// lut[kLutEntries + 1] (uint2), active flags[nb_max] (u8).
template <class InT, class OutT>
__global__ void __launch_bounds__(1024, 1)
    k_plan(const LutHeader<typename Traits<InT>::K> *hdr, const uint2 *__restrict__ lut_g,
           const uint32_t *__restrict__ counts, const uint32_t *__restrict__ excl_g, uint64_t n,
           const Req *__restrict__ reqs, uint32_t num_req, uint32_t nb_max, Ctrl *ctrl,
           uint64_t *tile_state, uint32_t scan_tiles, uint32_t *__restrict__ slot_of,
           uint64_t *__restrict__ seg_off, uint32_t *__restrict__ seg_size,
           uint32_t *__restrict__ kstart, uint32_t *__restrict__ kcnt,
           uint32_t *__restrict__ kcur, uint32_t *__restrict__ seg_cursor,
           uint32_t *__restrict__ req_bucket, Req *__restrict__ klist, uint64_t surv_cap,
           OutT *__restrict__ out) {
  using K = typename Traits<InT>::K;
  extern __shared__ uint4 smem_raw[];
  uint2 *lut = reinterpret_cast<uint2 *>(smem_raw);
  uint32_t *excl = reinterpret_cast<uint32_t *>(lut + kLutEntries + 1);
  uint8_t *flag = reinterpret_cast<uint8_t *>(excl + nb_max);
  __shared__ uint32_t red32[33];
  __shared__ uint64_t red64[33];
  const uint32_t tid = threadIdx.x, nt = blockDim.x;

  if (ctrl->status & ST_FATAL) return;
  const LutHeader<K> h = *hdr;
  const uint32_t nb = h.nb;
  for (uint32_t j = tid; j < kLutEntries; j += nt) lut[j] = lut_g[j];
  for (uint32_t b = tid; b < nb; b += nt) {
    excl[b] = excl_g[b];
    flag[b] = 0;
  }
  // re-arm the scan's state for the next call on this workspace
  for (uint32_t t = tid; t < scan_tiles; t += nt) tile_state[t] = 0;
  if (tid == 0) {
    ctrl->scan_ticket = 0;
    ctrl->deferred_count = 0;
    if ((uint64_t)excl_g[nb - 1] + counts[nb - 1] != n) atomicOr(&ctrl->status, ST_INTERNAL);
  }
  __syncthreads();

  // requests -> bucket; single-key buckets are answered here
  for (uint32_t i = tid; i < num_req; i += nt) {
    const Req r = reqs[i];
    uint32_t lo = 0, hi = nb;  // last b with excl[b] <= rank
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (excl[mid] <= r.rank)
        lo = mid;
      else
        hi = mid;
    }
    const uint32_t b = lo;
    // bucket b holds a single key iff the next bucket starts one key later.
    // The start of the top entry's bucket can wrap past the key width; then
    // no key reaches it and bucket b runs up to the largest key.
    const K klo = bucket_lo<K>(b, h.base, h.shift, lut);
    const K knext = (b + 1 < nb) ? bucket_lo<K>(b + 1, h.base, h.shift, lut) : K(0);
    const bool single = (knext > klo) ? (knext - klo == K(1)) : (klo == KeyMax<K>::v);
    if (single) {
      out[r.out] = Traits<OutT>::value(klo);
      req_bucket[i] = kNoSlot;
    } else {
      flag[b] = 1;
      req_bucket[i] = b;
    }
  }
  __syncthreads();

  // slots: exclusive scan of active flags and of active counts over buckets
  const uint32_t per = (nb + nt - 1) / nt;
  const uint32_t b0 = tid * per, b1 = min(nb, b0 + per);
  uint32_t my_slots = 0;
  uint64_t my_surv = 0;
  for (uint32_t b = b0; b < b1; ++b)
    if (flag[b]) {
      my_slots++;
      my_surv += counts[b];
    }
  uint32_t tot_slots;
  uint64_t tot_surv;
  uint32_t slot = block_incl_scan(my_slots, &tot_slots, red32) - my_slots;
  uint64_t off = block_incl_scan(my_surv, &tot_surv, red64) - my_surv;
  for (uint32_t b = b0; b < b1; ++b) {
    if (flag[b]) {
      const uint32_t cb = counts[b];
      slot_of[b] = slot;
      seg_off[slot] = off;
      seg_size[slot] = cb;
      kcnt[slot] = 0;
      kcur[slot] = 0;
      seg_cursor[slot] = 0;
      slot++;
      off += cb;
    } else {
      slot_of[b] = kNoSlot;
    }
  }
  if (tid == 0) {
    ctrl->num_slots = tot_slots;
    ctrl->total_surv = tot_surv;
    if (tot_surv > surv_cap) {
      atomicOr(&ctrl->status, ST_OVERFLOW);
      ctrl->cap_needed = tot_surv;
    }
  }
  __syncthreads();

  // requests per slot
  for (uint32_t i = tid; i < num_req; i += nt) {
    const uint32_t b = req_bucket[i];
    if (b != kNoSlot) atomicAdd(&kcnt[slot_of[b]], 1u);
  }
  __syncthreads();
  {
    const uint32_t sper = (tot_slots + nt - 1) / nt;
    const uint32_t s0 = tid * sper, s1 = min(tot_slots, s0 + sper);
    uint32_t mine = 0;
    for (uint32_t s = s0; s < s1; ++s) mine += kcnt[s];
    uint32_t tot;
    uint32_t run = block_incl_scan(mine, &tot, red32) - mine;
    for (uint32_t s = s0; s < s1; ++s) {
      kstart[s] = run;
      run += kcnt[s];
    }
  }
  __syncthreads();
  for (uint32_t i = tid; i < num_req; i += nt) {
    const uint32_t b = req_bucket[i];
    if (b != kNoSlot) {
      const uint32_t s = slot_of[b];
      const uint32_t pos = kstart[s] + atomicAdd(&kcur[s], 1u);
      const Req r = reqs[i];
      Req e;
      e.rank = r.rank - excl[b];
      e.out = r.out;
      klist[pos] = e;
    }
  }
}

// ---------------------------------------------------------------------------
// (f) compaction pass
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void compact_one(typename Traits<T>::K k, typename Traits<T>::K base,
                                            uint32_t shift, const uint2 *lut,
                                            const uint32_t *active,
                                            const uint32_t *__restrict__ slot_of,
                                            const uint64_t *__restrict__ seg_off,
                                            const uint32_t *__restrict__ seg_size,
                                            uint32_t *seg_cursor,
                                            typename Traits<T>::K *__restrict__ surv,
                                            Ctrl *ctrl) {
  const uint32_t b = bucket_of(k, base, shift, lut);
  if ((active[b >> 5] >> (b & 31)) & 1u) {
    const uint32_t s = __ldg(slot_of + b);
    const uint32_t c = atomicAdd(seg_cursor + s, 1u);
    // pass 2 recomputes pass 1's buckets, so c < seg_size[s]; an input changed
    // between the passes is reported instead of writing past the segment
    if (c < __ldg(seg_size + s))
      surv[__ldg(seg_off + s) + c] = k;
    else
      atomicOr(&ctrl->status, ST_INTERNAL);
  }
}

template <class T, int UNROLL>
__global__ void __launch_bounds__(1024, 1)
    k_compact(const T *__restrict__ x, uint64_t n, const LutHeader<typename Traits<T>::K> *hdr,
              const uint2 *__restrict__ lut_g, const uint32_t *__restrict__ slot_of,
              const uint64_t *__restrict__ seg_off, const uint32_t *__restrict__ seg_size,
              uint32_t *seg_cursor, typename Traits<T>::K *__restrict__ surv, uint32_t nb_max,
              Ctrl *ctrl) {
  using K = typename Traits<T>::K;
  using V = typename Traits<T>::Vec;
  constexpr int PV = Traits<T>::kPerVec;
  extern __shared__ uint4 smem_raw[];
  uint2 *lut = reinterpret_cast<uint2 *>(smem_raw);
  uint32_t *active = reinterpret_cast<uint32_t *>(lut + kLutEntries + 1);
  if (ctrl->status & (ST_FATAL | ST_OVERFLOW)) return;
  const LutHeader<K> h = *hdr;
  const uint32_t nwords = (h.nb + 31) >> 5;
  for (uint32_t j = threadIdx.x; j < kLutEntries; j += blockDim.x) lut[j] = lut_g[j];
  // one ballot per 32 buckets (blockDim.x is a multiple of 32)
  for (uint32_t base_b = 0; base_b < nwords * 32; base_b += blockDim.x) {
    const uint32_t b = base_b + threadIdx.x;
    const bool on = b < h.nb && slot_of[b] != kNoSlot;
    const uint32_t bits = __ballot_sync(0xffffffffu, on);
    if ((threadIdx.x & 31) == 0 && (b >> 5) < nwords) active[b >> 5] = bits;
  }
  __syncthreads();

  const Span<T> sp = split_span(x, n);
  const V *xv = reinterpret_cast<const V *>(x + sp.head);
  const uint64_t tile_v = (uint64_t)blockDim.x * UNROLL;
  const uint64_t ntiles = sp.nvec / tile_v;
  // walk the tiles from the end: the tail of the input read by the histogram
  // pass is the part most likely to still be in L2
  for (uint64_t q = blockIdx.x; q < ntiles; q += gridDim.x) {
    const uint64_t tile = ntiles - 1 - q;
    const V *p = xv + tile * tile_v + threadIdx.x;
    V v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) v[u] = ldg_stream(p + (uint64_t)u * blockDim.x);
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      K k[PV];
      vec_keys<T>(v[u], k);
#pragma unroll
      for (int e = 0; e < PV; ++e)
        compact_one<T>(k[e], h.base, h.shift, lut, active, slot_of, seg_off, seg_size, seg_cursor,
                       surv, ctrl);
    }
  }
  const uint32_t owner = (uint32_t)(ntiles % gridDim.x);
  if (blockIdx.x == owner) {
    for (uint64_t vi = ntiles * tile_v + threadIdx.x; vi < sp.nvec; vi += blockDim.x) {
      V vv = ldg_stream(xv + vi);
      K k[PV];
      vec_keys<T>(vv, k);
#pragma unroll
      for (int e = 0; e < PV; ++e)
        compact_one<T>(k[e], h.base, h.shift, lut, active, slot_of, seg_off, seg_size, seg_cursor,
                       surv, ctrl);
    }
    for (uint64_t e = threadIdx.x; e < sp.head; e += blockDim.x)
      compact_one<T>(Traits<T>::key(x[e]), h.base, h.shift, lut, active, slot_of, seg_off,
                     seg_size, seg_cursor, surv, ctrl);
    for (uint64_t e = sp.tail0 + threadIdx.x; e < n; e += blockDim.x)
      compact_one<T>(Traits<T>::key(x[e]), h.base, h.shift, lut, active, slot_of, seg_off,
                     seg_size, seg_cursor, surv, ctrl);
  }
}

// ---------------------------------------------------------------------------
// (g) per-segment finish: shared-memory MSD radix select
// ---------------------------------------------------------------------------
// One CTA per segment (persistent over segments).  The segment's keys are
// read from the survivor buffer (L2-resident) three times: min/max, a
// 2048-bin histogram of the top 11 bits of (key - min), and a gather of only
// the bins that hold requested ranks into shared memory.  Each gathered bin is
// sorted (a warp bitonic network for bins of <= 32 keys, a CTA bitonic sort for
// larger ones) and every request reads its rank.  Segments whose needed bins
// exceed the shared-memory buffer are listed for a recursive re-selection.
constexpr int kFinBins = 2048;
constexpr int kFinBinBits = 11;
constexpr int kFinThreads = 512;

template <class K>
__device__ __forceinline__ K warp_bitonic32(K v) {
  const uint32_t lane = threadIdx.x & 31;
#pragma unroll
  for (uint32_t k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      const K o = __shfl_xor_sync(0xffffffffu, v, j);
      const bool up = (lane & k) == 0;
      const bool lower = (lane & j) == 0;
      const K mn = v < o ? v : o, mx = v < o ? o : v;
      v = (lower == up) ? mn : mx;
    }
  }
  return v;
}

template <class K>
__device__ __forceinline__ void bitonic_sort_smem(K *s, uint32_t P) {
  for (uint32_t k = 2; k <= P; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < (P >> 1); i += blockDim.x) {
        const uint32_t lo = ((i & ~(j - 1)) << 1) | (i & (j - 1));
        const uint32_t hi = lo + j;
        const bool asc = (lo & k) == 0;
        const K a = s[lo], b = s[hi];
        if ((a > b) == asc) {
          s[lo] = b;
          s[hi] = a;
        }
      }
      __syncthreads();
    }
  }
}

// last bin with start[bin] <= r (start is an exclusive scan, start[0] = 0)
__device__ __forceinline__ uint32_t bin_of_rank(const uint32_t *start, uint32_t r) {
  uint32_t lo = 0, hi = kFinBins;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (start[mid] <= r)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

template <class K, class OutT>
__global__ void __launch_bounds__(kFinThreads)
    k_finish(const K *__restrict__ surv, Ctrl *ctrl, const uint64_t *__restrict__ seg_off,
             const uint32_t *__restrict__ seg_size, const uint32_t *__restrict__ kstart,
             const uint32_t *__restrict__ kcnt, const Req *__restrict__ klist,
             uint32_t *__restrict__ deferred, uint32_t bcap, OutT *__restrict__ out) {
  extern __shared__ uint4 smem_raw[];
  uint32_t *hist = reinterpret_cast<uint32_t *>(smem_raw);
  uint32_t *start = hist + kFinBins;
  uint32_t *gofs = start + kFinBins;  // gather offset of a needed bin, else kNoSlot
  uint32_t *cur = gofs + kFinBins;
  K *B = reinterpret_cast<K *>(cur + kFinBins);  // gathered keys of the needed bins
  K *T = B + bcap;                               // scratch for sorting a large bin
  __shared__ K redk[33];
  __shared__ uint32_t red32[33];
  constexpr uint32_t PER = kFinBins / kFinThreads;  // bins per thread

  if (ctrl->status & (ST_FATAL | ST_OVERFLOW)) return;
  const uint32_t num_slots = ctrl->num_slots;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t nwarps = blockDim.x >> 5;
  for (uint32_t slot = blockIdx.x; slot < num_slots; slot += gridDim.x) {
    const uint32_t size = seg_size[slot];
    const K *src = surv + seg_off[slot];
    const Req *rq = klist + kstart[slot];
    const uint32_t m = kcnt[slot];

    // ---- min / max
    K mn = KeyMax<K>::v, mx = 0;
    for (uint32_t i = tid; i < size; i += blockDim.x) {
      const K k = src[i];
      mn = k < mn ? k : mn;
      mx = k > mx ? k : mx;
    }
    mn = block_reduce(mn, [](K a, K b) { return a < b ? a : b; }, redk);
    mx = block_reduce(mx, [](K a, K b) { return a > b ? a : b; }, redk);
    if (mn == mx) {  // one distinct key: every rank is that key
      for (uint32_t j = tid; j < m; j += blockDim.x) out[rq[j].out] = Traits<OutT>::value(mn);
      continue;  // block_reduce ends with a barrier: shared state is free
    }
    const int bl = bitlen<K>(mx - mn);
    const uint32_t sh = bl > kFinBinBits ? (uint32_t)(bl - kFinBinBits) : 0u;

    // ---- histogram
    for (uint32_t i = tid; i < kFinBins; i += blockDim.x) {
      hist[i] = 0;
      cur[i] = 0;
    }
    __syncthreads();
    for (uint32_t i = tid; i < size; i += blockDim.x)
      atomicAdd(&hist[(uint32_t)((src[i] - mn) >> sh)], 1u);
    __syncthreads();
    {
      uint32_t c[PER], sum = 0;
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        c[q] = hist[tid * PER + q];
        sum += c[q];
      }
      uint32_t tot;
      uint32_t run = block_incl_scan(sum, &tot, red32) - sum;
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        start[tid * PER + q] = run;
        gofs[tid * PER + q] = 0;  // "needed" flag until the next scan
        run += c[q];
      }
    }
    __syncthreads();
    for (uint32_t j = tid; j < m; j += blockDim.x) gofs[bin_of_rank(start, rq[j].rank)] = 1u;
    __syncthreads();
    uint32_t V;
    {
      uint32_t c[PER], sum = 0;
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        const uint32_t b = tid * PER + q;
        c[q] = gofs[b] ? hist[b] : 0u;
        sum += c[q];
      }
      uint32_t run = block_incl_scan(sum, &V, red32) - sum;
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        const uint32_t b = tid * PER + q;
        const bool need = gofs[b] != 0u;
        gofs[b] = need ? run : kNoSlot;
        run += c[q];
      }
    }
    __syncthreads();
    if (V > bcap) {  // the needed bins do not fit: re-select on the host side
      if (tid == 0) {
        const uint32_t d = atomicAdd(&ctrl->deferred_count, 1u);
        deferred[d] = slot;
        atomicOr(&ctrl->status, ST_DEFERRED);
      }
      __syncthreads();
      continue;
    }

    // ---- gather the needed bins
    for (uint32_t i = tid; i < size; i += blockDim.x) {
      const K k = src[i];
      const uint32_t b = (uint32_t)((k - mn) >> sh);
      const uint32_t g = gofs[b];
      if (g != kNoSlot) B[g + atomicAdd(&cur[b], 1u)] = k;
    }
    __syncthreads();

    // ---- sort each needed bin: warps take the small ones
    for (uint32_t b = warp; b < kFinBins; b += nwarps) {
      const uint32_t g = gofs[b], c = hist[b];
      if (g == kNoSlot || c < 2 || c > 32) continue;
      K v = lane < c ? B[g + lane] : KeyMax<K>::v;
      v = warp_bitonic32(v);
      if (lane < c) B[g + lane] = v;
    }
    __syncthreads();
    for (uint32_t b = 0; b < kFinBins; ++b) {  // large bins: the whole CTA
      const uint32_t g = gofs[b], c = hist[b];
      if (g == kNoSlot || c <= 32) continue;
      uint32_t P = 64;
      while (P < c) P <<= 1;
      for (uint32_t i = tid; i < P; i += blockDim.x) T[i] = i < c ? B[g + i] : KeyMax<K>::v;
      __syncthreads();
      bitonic_sort_smem(T, P);
      for (uint32_t i = tid; i < c; i += blockDim.x) B[g + i] = T[i];
      __syncthreads();
    }

    // ---- answer
    for (uint32_t j = tid; j < m; j += blockDim.x) {
      const Req e = rq[j];
      const uint32_t b = bin_of_rank(start, e.rank);
      out[e.out] = Traits<OutT>::value(B[gofs[b] + (e.rank - start[b])]);
    }
    __syncthreads();
  }
}

// top-k request builder: rank n-1-i goes to output i (descending)
__global__ void k_topk_reqs(Req *reqs, uint64_t n, uint32_t K);

}  // namespace ggks
