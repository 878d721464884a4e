// ggks_device.cuh -- device side of the GB300 GGKS bucket multiselect.
//
// The pipeline (one problem; every pass is a kernel on one stream, no host
// round trip between passes):
//
//   (a) keys      order-preserving float/double -> uint key map
//                 (keyConversion.cu:9-23), applied on load, never stored.
//   (b) sample    k_sample + k_lut: S pseudo-random keys are gathered; the
//                 last CTA builds a range-adaptive splitter table (LUT) from them:
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
//                 nb_max buckets; one row of counts per CTA.
//                 Replaces assignSmartBucket (bucketMultiselect.cu:129-205)
//                 without its 4n-byte element-to-bucket array.
//   (d) totals    k_colsum: sums the per-CTA rows per bucket.  Replaces
//                 sumCounts (:214-221).
//   (e) plan      k_plan: one CTA takes the exclusive bucket prefix in shared
//                 memory, maps every requested rank to its bucket and local
//                 rank, answers ranks that fall in single-key buckets
//                 directly, assigns compact slots to the active buckets and
//                 groups the requests by slot.  Replaces the host walk of findKBuckets
//                 (:87-111), the host reindex loop and reindexCounts
//                 (:714-756).
//   (f) compact   k_compact: second pass over the input with the same
//                 CTA-to-tile assignment as (c); every CTA takes its share of
//                 each active bucket's segment with one global atomic and
//                 starts a private shared-memory cursor there, so elements of
//                 active buckets land in their segment of the survivor buffer
//                 with shared-memory atomics only.
//                 Replaces copyElements (:249-308) and reindexCounts
//                 (:229-241).
//   (g) finish    k_finish: per segment, an in-shared-memory sort of the
//                 survivors and a gather of the requested ranks.  Replaces
//                 thrust::sort of all survivors + copyValuesInChunk
//                 (:799-818).  Segments larger than shared memory are listed
//                 for a recursive re-selection by the host.
//
// Speculative compaction.  When the requested ranks cluster (top-k, one k, a
// few k's near each other or near both ends), the host sends one or two rank
// windows; (b) widens them by the sample's rank error and, if the predicted
// buckets hold few elements, (c) also lists the elements of those buckets per
// warp, in chunks taken from a pool in the survivor buffer's upper half, and
// (f) reads those candidates in place of the input whenever every active
// bucket was predicted (a CTA with an incomplete list reads its tiles).  The
// result never depends on the prediction, only the second pass's traffic does.
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
constexpr uint32_t kLutPadded = (kLutEntries + 3) & ~3u;  // 16-byte multiple
// at most 2^15 buckets per slice, and 2^(24 - slice bits) so that a packed
// table entry's first-bucket offset fits its signed 25-bit field
constexpr int kMaxSubBits = 15;
// The single-vector path's table: 2^9 slices.  Its streaming passes keep the
// table in shared memory once per bank -- entry j of copy l at word 32 j + l,
// read by lane l only -- so that a warp's 32 lookups take one wavefront
// whatever slices its keys fall in (one shared copy costs about three: the
// lanes' distinct entries pile up in a few banks).  2^9 slices keep the 32
// copies at 64 KB beside the 128 KB histogram.  The sample is still binned in
// 2^12 fine slices, which place the speculative windows (see build_lut_cta).
constexpr int kSvBits = 9;
constexpr uint32_t kSvSlices = 1u << kSvBits;
constexpr uint32_t kRepWords = (kSvSlices + 1) * 32;  // 32 copies of the 2^9 + 1 entries
constexpr uint32_t kMaxNb = 32768;  // buckets of one vector: shared-memory histogram limit (u32)
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;
constexpr uint32_t kInactive = 0x80000000u;  // compaction cursor of an inactive bucket
constexpr int kSpinLimit = 1 << 22;              // bounded device-side waits
constexpr uint32_t kMixed = 0x80000000u;  // count word: the bucket holds more than one key
// Buckets of a table that tracks single-key buckets in the histogram pass:
// its counts and first keys share the shared memory of nb_max counts.  0: no
// tracking (the splitter table needs more than 4098 buckets to be feasible).
template <class K>
__host__ __device__ constexpr uint32_t dup_nb_cap(uint32_t nb_max) {
  return nb_max / (sizeof(K) == 4 ? 2u : 4u) >= 8192u ? nb_max / (sizeof(K) == 4 ? 2u : 4u) : 0u;
}
constexpr uint32_t kCandWarps = 32;  // warps of a histogram / compaction CTA (1024 threads)
constexpr uint32_t kCandChunk = 256;          // candidate keys per pool chunk
constexpr uint32_t kCandChunksPerWarp = 64;   // chunks one warp's list can hold

// Programmatic dependent launch.  The pipeline's kernels are launched so that
// each may be scheduled while its predecessor in the stream still runs;
// griddepcontrol.wait blocks until that predecessor has completed and its
// memory is visible (a no-op after a plain launch), and comes before a
// kernel's first global access.  griddepcontrol.launch_dependents lets the
// successor be scheduled at once: it orders nothing, the successor's own wait
// does.  No kernel of the pipeline waits on other CTAs, so successors that sit
// resident while waiting cannot hold up the running grid.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_start() {
  pdl_trigger();
  pdl_wait();
}

// Bulk asynchronous copies global -> shared (the copy engine's untiled form):
// 16-byte aligned addresses, sizes in multiples of 16 bytes, completion
// counted in bytes on an mbarrier.  One thread initialises the barrier and
// issues the copies; a barrier of the block orders the initialisation before
// any wait; waits are bounded.
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// bytes: a multiple of 16, issued in pieces of at most 32 KB
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  for (uint32_t o = 0; o < bytes; o += 32768u) {
    const uint32_t m = bytes - o < 32768u ? bytes - o : 32768u;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(static_cast<char *>(dst) + o)),
        "l"(static_cast<const char *>(src) + o), "r"(m), "r"(smem_addr(bar))
        : "memory");
  }
}
// true once the barrier's phase `parity` has completed; false after
// kSpinLimit tries
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  for (int i = 0; i < kSpinLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// status bits in Ctrl::status
enum : uint32_t {
  ST_OVERFLOW = 1u,  // survivors exceed the survivor buffer: host regrows, re-runs (f)+(g)
  ST_DEFERRED = 2u,  // some segments exceed shared memory: host re-selects them
  ST_TIMEOUT = 4u,   // a bounded wait gave up
  ST_INTERNAL = 8u,  // a consistency check failed (counts do not add up to n)
  ST_BAD_K = 16u,    // a k outside [1, n] (device-side k lists)
  ST_TOPK_MISS = 32u,  // the threshold top-k's candidates fell short: run the pipeline
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
  uint32_t sample_done;    // last-CTA ticket of k_lut (reset by that CTA)
  uint32_t same_key;       // far-apart sample pairs holding one key (k_lut)
  uint32_t nb;             // buckets in use
  uint64_t cap_needed;
  uint64_t kmin_inv;     // ~(smallest sampled key), by atomicMax
  uint64_t kmax;         // largest sampled key, by atomicMax
  // rank windows of the call's requests, written by the host into the
  // uploaded image (0 windows: the requests are spread out or unknown)
  uint32_t spec_nwin;
  uint32_t spec_pad;
  uint64_t spec_lo[2], spec_hi[2];  // ascending 0-based ranks, inclusive
  uint32_t spec_on;    // the table keeps candidate buckets (k_lut)
  uint32_t spec_ctas;  // compaction CTAs that read candidates
  uint32_t cand_next;  // candidate chunks handed out (k_hist)
  uint64_t t_ns[16];   // phase stamps of the small-vector kernel (GGKS_SMALL_TIMING builds)
};

template <class K>
struct LutHeader {
  K base;          // smallest sampled key
  uint32_t shift;  // slice index = (key - base) >> shift
  uint32_t nb;     // number of buckets
  uint32_t heavy;  // 1: warp-aggregate compaction's cursor updates
  uint32_t dup;    // 1: sampled keys repeat often (at least once per nb pairs)
  // speculative compaction: the histogram pass also keeps every element whose
  // bucket lies in [spec_lo[i], spec_lo[i] + spec_len[i]) (i < 2) in a pool of
  // cand_cap chunks; spec == 0: off
  uint32_t spec;
  uint32_t cand_cap;
  uint32_t spec_lo[2];
  uint32_t spec_len[2];
};

// Inputs of the candidate-window computation (k_lut's last CTA).
struct SpecArgs {
  const Ctrl *ctrl;     // spec_nwin, spec_lo, spec_hi
  uint64_t n;           // elements of the vector
  uint32_t cand_cap;    // candidate chunks in the pool (0: off)
  uint32_t G;           // histogram CTAs
};

template <class K>
__device__ __forceinline__ bool in_spec(const LutHeader<K> &h, uint32_t b) {
  return (b - h.spec_lo[0] < h.spec_len[0]) | (b - h.spec_lo[1] < h.spec_len[1]);
}

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

// predicated global stores (no branch around them)
__device__ __forceinline__ void st_global_if(uint32_t *p, uint32_t v, bool pred) {
  asm volatile(
      "{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %2, 0;\n\t@q st.global.b32 [%0], %1;\n\t}" ::"l"(p),
      "r"(v), "r"((uint32_t)pred)
      : "memory");
}
__device__ __forceinline__ void st_global_if(uint64_t *p, uint64_t v, bool pred) {
  asm volatile(
      "{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %2, 0;\n\t@q st.global.b64 [%0], %1;\n\t}" ::"l"(p),
      "l"(v), "r"((uint32_t)pred)
      : "memory");
}

// right shift that yields 0 for shift >= width (the splitter table's top
// entry shifts by the key width).  __funnelshift_rc clamps the shift to 32;
// __funnelshift_r would wrap it to shift & 31.
__device__ __forceinline__ uint32_t shr_clamp(uint32_t d, uint32_t s) {
  return __funnelshift_rc(d, 0u, s);
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
// lut[j] = (C_j << 7) | rs_j.  For slice j with first bucket B_j cut into 2^b_j
// sub-buckets: rs_j = shift - b_j and C_j = B_j - (j << b_j), a signed 25-bit
// value (|j << b_j| < 2^24 because a table of 2^s slices has j < 2^s and
// b_j <= 24 - s).  Then
//   bucket = C_j + ((key - base) >> rs_j),
// since (key - base) >> rs_j = (j << b_j) + sub-bucket on slice j.  Empty
// slices of one run share a bucket (b = 0); the top entry (keys above the
// sampled span) has rs = key width, i.e. the constant bucket C.  Bucket 0
// holds the keys below `base` (the sampled minimum), so the first slice's
// buckets start at 1 and its first bucket starts exactly at `base`.  One 4-byte
// entry per slice keeps the shared-memory lookup to a single wavefront for
// runs of neighbouring slices; the bucket costs two ALU operations.
//
// nsl (a power of two <= kLutIdx) is the number of slices; the top entry sits
// at lut[nsl].  The single-vector path always uses kLutIdx slices; small
// problems of a batch use fewer.
template <class K>
__device__ __forceinline__ uint32_t bucket_of(K key, K base, uint32_t shift, const uint32_t *lut,
                                              uint32_t nsl = kLutIdx) {
  const K d = key - base;  // wraps for key < base; that result is discarded
  const K idx = d >> shift;
  const uint32_t j = idx < (K)nsl ? (uint32_t)idx : nsl;
  const uint32_t e = lut[j];
  const uint32_t b = (uint32_t)((int32_t)e >> 7) + shr_clamp(d, e & 127u);
  return key < base ? 0u : b;
}

// bucket_of on the single-vector table (kSvSlices slices) replicated once per
// bank in shared memory: lane_lut = table + (lane index), entry j at
// lane_lut[32 j], so the lanes of a warp never share a bank.
template <class K>
__device__ __forceinline__ uint32_t bucket_of_rep(K key, K base, uint32_t shift,
                                                  const uint32_t *lane_lut) {
  const K d = key - base;  // wraps for key < base; that result is discarded
  const K idx = d >> shift;
  const uint32_t j = idx < (K)kSvSlices ? (uint32_t)idx : kSvSlices;
  const uint32_t e = lane_lut[j << 5];
  const uint32_t b = (uint32_t)((int32_t)e >> 7) + shr_clamp(d, e & 127u);
  return key < base ? 0u : b;
}

// Copies the single-vector table (kSvSlices + 1 entries, global) into shared
// memory once per bank (kRepWords words); the caller synchronises.
__device__ __forceinline__ void load_rep_table(uint32_t *rep, const uint32_t *__restrict__ lut_g) {
  for (uint32_t i = threadIdx.x; i < kRepWords; i += blockDim.x) rep[i] = __ldg(lut_g + (i >> 5));
}

__device__ __forceinline__ uint32_t lut_pack(int32_t C, uint32_t rs) {
  return ((uint32_t)C << 7) | rs;
}

// first bucket and sub-bucket bits of entry j
__device__ __forceinline__ void lut_entry(uint32_t e, uint32_t j, uint32_t shift, uint32_t *B,
                                          uint32_t *bb, uint32_t nsl = kLutIdx) {
  const int32_t C = (int32_t)e >> 7;
  if (j == nsl) {
    *B = (uint32_t)C;
    *bb = 0;
  } else {
    *bb = shift - (e & 127u);
    *B = (uint32_t)(C + (int32_t)(j << *bb));
  }
}

// smallest key that maps to bucket b (b < nb); bucket 0 starts at key 0.
template <class K>
__device__ __forceinline__ K bucket_lo(uint32_t b, K base, uint32_t shift, const uint32_t *lut,
                                       uint32_t nsl = kLutIdx) {
  if (b == 0) return K(0);
  // first entry whose last bucket >= b (bucket ranges are non-decreasing in j)
  uint32_t lo = 0, hi = nsl;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    uint32_t B, bb;
    lut_entry(lut[mid], mid, shift, &B, &bb, nsl);
    if (B + (1u << bb) - 1u >= b)
      hi = mid;
    else
      lo = mid + 1;
  }
  uint32_t B, bb;
  lut_entry(lut[lo], lo, shift, &B, &bb, nsl);
  const K dstart = ((K)lo) << shift;  // for lo == nsl this may wrap: see the caller
  if (B >= b) return base + dstart;
  return base + dstart + (((K)(b - B)) << (shift - bb));
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
// each CTA folds its min / max into Ctrl with one atomic each; the last CTA to
// finish counts the samples per slice and builds the table.
//
// Allocation: a slice with c samples gets 2^b sub-buckets,
// b = clamp(ceil(log2 c) - t, 0, min(shift, 15, 24 - slice bits)), and empty
// slices merge into one bucket per run.  The smallest threshold t whose bucket total fits nb_max
// is found from a histogram of ceil(log2 c) over the slices, so each candidate
// t costs a 33-term sum on one thread.
// Builds the splitter table of one problem from its S sampled keys (kmin /
// kmax: the sample's extremes) with one whole CTA of 4096 / SPT threads; the
// table goes to lut[0 .. nsl] with nsl = 2^nsl_bits slices (nb_max >= nsl + 2
// makes every threshold feasible), and thread 0 writes the header.  The
// samples are in shared memory (SMEM) or in global memory written by other
// CTAs (read past L1).
//
// pre_cnt (global, kLutIdx words): the samples already binned in 2^12 fine
// slices of the span ((key - kmin) >> fine shift, fine shift = bit length of
// the span - 12, at least 0); every slice is a run of 2^fold fine slices.
// With pre_cnt a slice's sub-buckets follow its peak density -- its largest
// fine count times 2^fold, in place of its count -- so that a slice whose
// keys crowd into part of its range (the slice holding the sampled maximum,
// whose keys stop there; a steep stretch of a distribution) gets buckets as
// narrow as its densest part needs.
// fine (shared, kLutIdx words, with pre_cnt only): lent by the caller to keep
// the fine counts, which place the speculative windows (sp) at fine-slice
// precision; without it no window is computed.
template <class K, int SPT, bool SMEM>
__device__ void build_lut_cta(const K *samples, uint32_t S, K kmin, K kmax, uint32_t nb_max,
                              uint32_t *lut, LutHeader<K> *hdr, int nsl_bits = kLutIdxBits,
                              uint32_t *pre_cnt = nullptr, int64_t pre_same_key = -1,
                              const SpecArgs *sp = nullptr, uint32_t dup_cap = 0,
                              uint32_t *fine = nullptr) {
  __shared__ uint32_t cnt[kLutIdx];
  __shared__ uint32_t lch[36];  // [0, 33): slices by ceil(log2 c); [34]: empty-run starts
  __shared__ uint32_t red32[33];
  __shared__ int s_t, s_r0;
  __shared__ uint32_t s_tot[54];
  __shared__ uint32_t s_cost[34];
  const uint32_t tid = threadIdx.x;
  const uint32_t nsl = 1u << nsl_bits;
  // A caller that tracks single-key buckets (dup_cap) needs at most dup_cap
  // buckets when keys repeat often; the counted far-apart pairs tell that
  // before the table exists (with nb_max >= the final bucket count, this test
  // holds whenever the table's dup flag will).
  if (dup_cap && pre_same_key >= 0 && S >= 256 &&
      (uint64_t)pre_same_key * nb_max >= (S / 2 < 4096u ? S / 2 : 4096u) && nb_max > dup_cap)
    nb_max = dup_cap;
  const int bl = bitlen<K>(kmax - kmin);
  const uint32_t shift = bl > nsl_bits ? (uint32_t)(bl - nsl_bits) : 0u;
  const uint32_t fsh = bl > kLutIdxBits ? (uint32_t)(bl - kLutIdxBits) : 0u;  // fine slices
  const uint32_t fold = shift - fsh;  // a slice is 2^fold fine slices
  int bcap = (int)(shift < (uint32_t)kMaxSubBits ? shift : (uint32_t)kMaxSubBits);
  if (bcap > 24 - nsl_bits) bcap = 24 - nsl_bits;

  // --- sample counts per slice: counted by the caller in fine slices
  // (pre_cnt, global, left zero here for the next call), or from the samples
  if (tid < 36) lch[tid] = 0;
  if (pre_cnt) {
    for (uint32_t j = tid; j < nsl; j += blockDim.x) cnt[j] = 0;
    __syncthreads();
    for (uint32_t j0 = tid; j0 < kLutIdx; j0 += 4 * blockDim.x) {
      uint32_t c4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t j = j0 + u * blockDim.x;
        c4[u] = j < kLutIdx ? __ldcg(pre_cnt + j) : 0u;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t j = j0 + u * blockDim.x;
        if (j < kLutIdx) {
          if (fine) fine[j] = c4[u];
          if (c4[u] && (j >> fold) < nsl) atomicMax(&cnt[j >> fold], c4[u] << fold);
          pre_cnt[j] = 0;
        }
      }
    }
    __syncthreads();
  } else {
    for (uint32_t j = tid; j < kLutIdx; j += blockDim.x) cnt[j] = 0;
    __syncthreads();
  }
  // 16 loads per thread in flight before their atomics (loads and shared
  // atomics interleaved in one loop body complete one at a time)
  for (uint32_t s0 = tid; s0 < (pre_cnt ? 0u : S); s0 += 16 * blockDim.x) {
    K kk[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const uint32_t s = s0 + u * blockDim.x;
      kk[u] = s < S ? (SMEM ? samples[s] : __ldcg(samples + s)) : kmin;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u)
      if (s0 + u * blockDim.x < S) atomicAdd(&cnt[(uint32_t)((kk[u] - kmin) >> shift)], 1u);
  }
  __syncthreads();

  // Each thread owns SPT consecutive slices [SPT tid, SPT tid + SPT) (those at
  // or beyond nsl are unused); the top entry (keys above the sampled span) is
  // written by thread 0 after the scan.
  int lc[SPT];
  uint32_t c[SPT];
  bool prev_nonempty[SPT];
#pragma unroll
  for (int q = 0; q < SPT; ++q) {
    const uint32_t j = SPT * tid + q;
    const bool in = j < nsl;
    c[q] = in ? cnt[j] : 0u;
    lc[q] = c[q] ? (c[q] == 1 ? 0 : 32 - __clz(c[q] - 1)) : -1;  // ceil(log2 c)
    prev_nonempty[q] = in && ((j == 0) ? true : (cnt[j - 1] != 0));
    if (c[q])
      atomicAdd(&lch[lc[q]], 1u);
    else if (prev_nonempty[q])
      atomicAdd(&lch[34], 1u);
  }
  const bool top_run_start = cnt[nsl - 1] != 0;
  if (tid == 0) s_t = 33;  // total(33) <= 1 + nsl + 1 <= nb_max: always feasible
  if (tid < 34) s_cost[tid] = 0;
  __syncthreads();
  if (tid < 54) {
    // smallest t with total(t) <= nb_max; one candidate t per thread
    const int t = -kMaxSubBits - 1 + (int)tid;
    uint64_t tot = 1u + lch[34] + (top_run_start ? 1u : 0u);
    for (int l = 0; l < 33; ++l) {
      int b = l - t;
      b = b < 0 ? 0 : (b > bcap ? bcap : b);
      tot += (uint64_t)lch[l] << b;
    }
    s_tot[tid] = (uint32_t)(tot < 0xFFFFFFFFull ? tot : 0xFFFFFFFFull);
    if (tot <= nb_max) atomicMin(&s_t, t);
  }
  __syncthreads();
  const int t = s_t;
  const uint32_t spare = nb_max - s_tot[t + kMaxSubBits + 1];

  // Power-of-two rounding leaves part of the budget unused.  Spend it on the
  // slices whose buckets are expected to be the fullest: r = 32 * (samples per
  // bucket) / 2^t in [0, 32]; doubling slice j's buckets costs 2^b_j.  The
  // largest r first, as long as the whole bin of r fits.
  int bq[SPT];
  uint32_t rq[SPT];
#pragma unroll
  for (int q = 0; q < SPT; ++q) {
    int b = lc[q] - t;
    bq[q] = b < 0 ? 0 : (b > bcap ? bcap : b);
    rq[q] = 0xFFFFFFFFu;  // not a candidate
    if (c[q] && bq[q] < bcap) {
      const int e = bq[q] + t - 5;  // r = c * 32 / 2^(b + t)
      uint32_t r = e >= 0 ? (e >= 32 ? 0u : c[q] >> e) : (-e >= 32 ? 32u : c[q] << (-e));
      rq[q] = r > 32u ? 32u : r;
      atomicAdd(&s_cost[rq[q]], 1u << bq[q]);
    }
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t acc = 0;
    int r0 = 33;
    for (int r = 32; r >= 0; --r) {
      if (acc + s_cost[r] > spare) break;
      acc += s_cost[r];
      r0 = r;
    }
    s_r0 = r0;
  }
  __syncthreads();
  const uint32_t r0 = (uint32_t)s_r0;
#pragma unroll
  for (int q = 0; q < SPT; ++q)
    if (rq[q] != 0xFFFFFFFFu && rq[q] >= r0) bq[q] += 1;

  auto bits_of = [&](int q) -> int { return bq[q]; };
  uint32_t my[SPT], mysum = 0;
#pragma unroll
  for (int q = 0; q < SPT; ++q) {
    my[q] = c[q] ? (1u << bits_of(q)) : (prev_nonempty[q] ? 1u : 0u);
    mysum += my[q];
  }
  uint32_t total;
  const uint32_t incl = block_incl_scan(mysum, &total, red32);
  uint32_t run = incl - mysum + 1u;  // bucket 0 is the low edge

  // Candidate windows.  The number of samples below the element of rank r is
  // about Binomial(S, r / n); each window [lo, hi] of ranks is widened to the
  // sample ranks E - 6 sd - 4 .. E + 6 sd + 4 of its ends, and the slices
  // holding those two samples bound its buckets.  A window reaching past the
  // sample's first or last key takes bucket 0 or the top bucket as well.  The
  // prediction only decides what the histogram pass keeps: compaction checks
  // that every segment's bucket was kept before it reads the candidates.
  __shared__ uint32_t s_sp[8];  // per window: first bucket, last bucket, first / end sample rank
  const bool spec_on = sp != nullptr && sp->cand_cap != 0 && sp->ctrl->spec_nwin != 0 &&
                       pre_cnt != nullptr && fine != nullptr;
  uint32_t wa[2] = {0, 0}, wb[2] = {0, 0}, nwin = 0;
  bool wlo_open[2] = {false, false}, whi_open[2] = {false, false};
  if (spec_on) {
    nwin = sp->ctrl->spec_nwin < 2u ? sp->ctrl->spec_nwin : 2u;
    // single precision (float64 is slow on this part; sample ranks need
    // about one unit of 2^16)
    const float dn = (float)sp->n, dS = (float)S;
#pragma unroll
    for (uint32_t w = 0; w < 2; ++w) {
      if (w >= nwin) break;
      const float pl = (float)sp->ctrl->spec_lo[w] / dn;
      const float ph = fminf((float)(sp->ctrl->spec_hi[w] + 1) / dn, 1.0f);
      const float a = pl * dS - (6.0f * sqrtf(dS * pl * (1.0f - pl)) + 4.0f);
      const float b = ph * dS + (6.0f * sqrtf(dS * ph * (1.0f - ph)) + 4.0f);
      wlo_open[w] = a <= 0.0f;
      whi_open[w] = b >= dS - 1.0f;
      wa[w] = wlo_open[w] ? 0u : (a >= dS - 1.0f ? S - 1u : (uint32_t)a);
      wb[w] = whi_open[w] ? S - 1u : (uint32_t)b;
    }
    // defaults (replaced below; no fine slice left unmatched): every bucket, every sample
    if (tid < 8) s_sp[tid] = (tid & 3) == 1 ? 0xFFFFFFFEu : ((tid & 3) == 3 ? S : 0u);
  }
  // the table also goes to cnt[] (its counts are no longer read) for the
  // collision estimate below
#pragma unroll
  for (int q = 0; q < SPT; ++q) {
    const uint32_t j = SPT * tid + q;
    uint32_t e = 0;
    if (j >= nsl) {
      continue;  // unused slice
    } else if (c[q]) {
      const int b = bits_of(q);
      e = lut_pack((int32_t)run - (int32_t)(j << b), shift - (uint32_t)b);
    } else {
      // one bucket per run of empty slices
      e = lut_pack((int32_t)(prev_nonempty[q] ? run : run - 1u) - (int32_t)j, shift);
    }
    lut[j] = e;
    cnt[j] = e;
    run += my[q];
  }
  const uint32_t top = lut_pack((int32_t)(top_run_start ? total + 1u : total),
                                (uint32_t)KeyMax<K>::bits);
  __syncthreads();
  // Warp-aggregated cursor updates in compaction pay off when lanes of a warp
  // often hit the same bucket (its atomics return positions, which lanes of
  // one address receive one at a time): the chance that two elements share a
  // bucket is estimated from neighbouring samples (2q, 2q + 1), which are
  // neighbouring elements when the samples come in pairs or runs, as the
  // passes' warps see them.  The
  // chance that two elements share a key, a property of the whole vector, is
  // estimated from far-apart samples (q, q + S/2).
  uint32_t same = 0, same_key = 0;
  const uint32_t npairs = S / 2 < 4096u ? S / 2 : 4096u;  // enough for a 1/32 estimate
  auto bucket = [&](K k) {
    const K d = k - kmin;
    const K idx = d >> shift;
    const uint32_t j = idx < (K)nsl ? (uint32_t)idx : nsl;
    const uint32_t e = j == nsl ? top : cnt[j];
    return (uint32_t)((int32_t)e >> 7) + shr_clamp(d, e & 127u);
  };
  if (spec_on) {
    // The fine slices split the sample ranks [0, S) in order: the fine slice
    // holding a window's first (last) sample rank gives the window's first
    // (last) bucket, that of the fine slice's first (last) key.  Each thread
    // takes kLutIdx / blockDim.x consecutive fine slices (at most 4).
    const uint32_t per = kLutIdx / blockDim.x;
    uint32_t fc[4], fsum = 0;
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q) {
      fc[q] = q < per ? fine[per * tid + q] : 0u;
      fsum += fc[q];
    }
    uint32_t ftot;
    uint32_t fpre = block_incl_scan(fsum, &ftot, red32) - fsum;
    const K span = kmax - kmin;
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q) {
      if (q >= per || fc[q] == 0) continue;
      const uint32_t jf = per * tid + q;
#pragma unroll
      for (uint32_t w = 0; w < 2; ++w) {
        if (w >= nwin) break;
        if (fpre <= wa[w] && wa[w] < fpre + fc[q]) {
          s_sp[4 * w + 0] = bucket(kmin + ((K)jf << fsh));
          s_sp[4 * w + 2] = fpre;
        }
        if (fpre <= wb[w] && wb[w] < fpre + fc[q]) {
          K dend = ((K)(jf + 1u) << fsh) - K(1);
          dend = dend < span ? dend : span;
          s_sp[4 * w + 1] = bucket(kmin + dend);
          s_sp[4 * w + 3] = fpre + fc[q];
        }
      }
      fpre += fc[q];
    }
    __syncthreads();
  }
  auto ld = [&](uint32_t i) -> K { return SMEM ? samples[i] : __ldcg(samples + i); };
  // four pairs of each kind per thread and step, all loads issued first (the
  // far-apart pairs only when the caller has not counted them)
  const bool far = pre_same_key < 0;
  for (uint32_t q0 = tid; q0 < npairs; q0 += 4 * blockDim.x) {
    K a[4], b[4], c[4], d2[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t q = q0 + u * blockDim.x;
      const bool ok = q < npairs;
      a[u] = ok ? ld(2 * q) : K(0);
      b[u] = ok ? ld(2 * q + 1) : K(0);
      c[u] = ok && far ? ld(q) : K(0);
      d2[u] = ok && far ? ld(q + S / 2) : K(1);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (q0 + u * blockDim.x < npairs) {
        same += bucket(a[u]) == bucket(b[u]) ? 1u : 0u;
        same_key += c[u] == d2[u] ? 1u : 0u;
      }
  }
  same = block_reduce(same, [](uint32_t p, uint32_t q) { return p + q; }, red32);
  same_key = far ? block_reduce(same_key, [](uint32_t p, uint32_t q) { return p + q; }, red32)
                 : (uint32_t)pre_same_key;
  if (tid == 0) {
    const uint32_t nb = 1u + total + (top_run_start ? 1u : 0u);
    lut[nsl] = top;
    LutHeader<K> h;
    h.base = kmin;
    h.shift = shift;
    h.nb = nb;
    // collision chance >= 1/32: with 32 lanes, about 15 same-bucket pairs per
    // warp access
    h.heavy = (S >= 256 && 32ull * same >= npairs) ? 1u : 0u;
    // two elements share a key with chance >= 1 / nb: buckets holding a single
    // key (many copies of it) are likely
    h.dup = (S >= 256 && (uint64_t)same_key * nb >= npairs) ? 1u : 0u;
    h.spec = 0;
    h.cand_cap = 0;
    h.spec_lo[0] = h.spec_lo[1] = 0;
    h.spec_len[0] = h.spec_len[1] = 0;
    if (spec_on) {
      // bucket intervals and the sample ranks they hold, ordered and merged
      uint32_t blo[2], bhi[2], clo[2], chi[2];
#pragma unroll
      for (uint32_t w = 0; w < 2; ++w) {
        if (w >= nwin) break;
        blo[w] = wlo_open[w] ? 0u : s_sp[4 * w + 0];
        bhi[w] = whi_open[w] ? nb - 1u : s_sp[4 * w + 1];
        clo[w] = wlo_open[w] ? 0u : s_sp[4 * w + 2];
        chi[w] = whi_open[w] ? S : s_sp[4 * w + 3];
      }
      uint32_t ni = nwin;
      if (ni == 2) {
        if (blo[1] < blo[0]) {
          uint32_t t0 = blo[0]; blo[0] = blo[1]; blo[1] = t0;
          t0 = bhi[0]; bhi[0] = bhi[1]; bhi[1] = t0;
          t0 = clo[0]; clo[0] = clo[1]; clo[1] = t0;
          t0 = chi[0]; chi[0] = chi[1]; chi[1] = t0;
        }
        if (blo[1] <= bhi[0] + 1u) {
          bhi[0] = bhi[1] > bhi[0] ? bhi[1] : bhi[0];
          chi[0] = chi[1] > chi[0] ? chi[1] : chi[0];
          ni = 1;
        }
      }
      uint32_t pred = 0;  // samples inside the intervals
#pragma unroll
      for (uint32_t i = 0; i < 2; ++i)
        if (i < ni) pred += chi[i] - clo[i];
      // the expected candidates with half as much again, plus one partly
      // filled chunk per histogram warp, must fit the pool
      const float want = 1.5f * (float)sp->n * (float)pred / (float)S +
                         (float)sp->G * kCandWarps * kCandChunk;
      if (want <= (float)sp->cand_cap * kCandChunk) {
        h.spec = ni;
        h.cand_cap = sp->cand_cap;
#pragma unroll
        for (uint32_t i = 0; i < 2; ++i)
          if (i < ni) {
            h.spec_lo[i] = blo[i];
            h.spec_len[i] = bhi[i] - blo[i] + 1u;
          }
      }
    }
    *hdr = h;
  }
}

// Two kernels of ceil(S / 1024) CTAs.  k_sample: each thread gathers one
// sample (pairs of neighbouring elements at hashed positions) and each CTA
// folds its min / max into Ctrl.
// k_lut (after it in the stream): each CTA re-reads its 1024 samples, bins
// them by slice in shared memory against the sample's span, adds its non-zero
// slice counts to slice_cnt (global, zero on entry) and counts the far-apart
// pairs (q, q + S/2) that hold one key; the last CTA to finish builds the
// table from slice_cnt (leaving it zero) and reads back only the neighbouring
// samples its bucket collision estimate needs.  The kernel boundary takes the
// place of a grid barrier, so no launch needs every CTA resident at once.
// The table builder also turns the call's rank windows (Ctrl::spec_*) into
// the candidate buckets of speculative compaction (n, cand_cap: chunks in the
// candidate pool, 0 for none; G: histogram CTAs).
template <class T>
__global__ void __launch_bounds__(1024) k_sample(const T *__restrict__ x, uint64_t n, uint32_t S,
                                                 uint32_t seed,
                                                 typename Traits<T>::K *__restrict__ samples,
                                                 Ctrl *ctrl) {
  pdl_start();
  using K = typename Traits<T>::K;
  __shared__ K redk[33];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  K mine_lo = KeyMax<K>::v, mine_hi = 0;
  if (i < S) {
    uint64_t pos;
    if ((uint64_t)S >= n) {
      pos = i;
    } else {
      // pairs of neighbouring elements at hashed positions: samples 2q and
      // 2q + 1 are neighbours, so the table builder's collision estimate sees
      // runs of equal buckets (sorted input) as the histogram's warps do
      pos = (((uint64_t)hash32((i >> 1) * 0x9E3779B9u + seed) * (n - 1)) >> 32) + (i & 1u);
    }
    const K k = Traits<T>::key(x[pos]);
    samples[i] = k;
    mine_lo = k;
    mine_hi = k;
  }
  mine_lo = block_reduce(mine_lo, [](K p, K q) { return p < q ? p : q; }, redk);
  mine_hi = block_reduce(mine_hi, [](K p, K q) { return p > q ? p : q; }, redk);
  if (threadIdx.x == 0) {
    atomicMax((unsigned long long *)&ctrl->kmin_inv, (unsigned long long)~(uint64_t)mine_lo);
    atomicMax((unsigned long long *)&ctrl->kmax, (unsigned long long)mine_hi);
  }
}

template <class K>
__global__ void __launch_bounds__(1024) k_lut(const K *__restrict__ samples, uint32_t S,
                                              Ctrl *ctrl, LutHeader<K> *hdr, uint32_t *lut,
                                              uint32_t nb_max, uint32_t *slice_cnt, uint64_t n,
                                              uint32_t cand_cap, uint32_t G) {
  pdl_start();
  __shared__ uint32_t red32[33];
  __shared__ uint32_t s_last;
  __shared__ uint32_t ccnt[kLutIdx];

  const uint32_t tid = threadIdx.x;
  const uint32_t i = blockIdx.x * blockDim.x + tid;
  for (uint32_t j = tid; j < kLutIdx; j += blockDim.x) ccnt[j] = 0;
  const uint32_t npairs = S / 2 < 4096u ? S / 2 : 4096u;
  const K k = i < S ? __ldcg(samples + i) : K(0);
  const K other = i < npairs ? __ldcg(samples + i + S / 2) : K(0);
  const K kmin = (K)~__ldcg((const unsigned long long *)&ctrl->kmin_inv);
  const K kmax = (K)__ldcg((const unsigned long long *)&ctrl->kmax);
  const int bl = bitlen<K>(kmax - kmin);
  const uint32_t shift = bl > kLutIdxBits ? (uint32_t)(bl - kLutIdxBits) : 0u;
  __syncthreads();
  if (i < S) atomicAdd(&ccnt[(uint32_t)((k - kmin) >> shift)], 1u);
  // far-apart pairs (q, q + S/2): does the vector hold many copies of a key
  uint32_t sk = i < npairs && other == k ? 1u : 0u;
  sk = block_reduce(sk, [](uint32_t p, uint32_t q) { return p + q; }, red32);
  for (uint32_t j = tid; j < kLutIdx; j += blockDim.x) {
    const uint32_t c = ccnt[j];
    if (c) atomicAdd(&slice_cnt[j], c);
  }
  // every thread's counts before the CTA reports done (the fence below is
  // cumulative over what the barrier ordered)
  __syncthreads();
  if (tid == 0) {
    if (sk) atomicAdd(&ctrl->same_key, sk);
    __threadfence();
    s_last = (atomicAdd(&ctrl->sample_done, 1u) == gridDim.x - 1) ? 1u : 0u;
    if (s_last) __threadfence();
  }
  __syncthreads();
  if (!s_last) return;

  // the table has kSvSlices slices; the fine counts (this CTA's ccnt is free
  // now) place the speculative windows
  __syncthreads();
  const SpecArgs sa{ctrl, n, cand_cap, G};
  build_lut_cta<K, 4, false>(samples, S, kmin, kmax, nb_max, lut, hdr, kSvBits, slice_cnt,
                             (int64_t)__ldcg(&ctrl->same_key), &sa, dup_nb_cap<K>(nb_max), ccnt);
  if (tid == 0) {
    ctrl->nb = hdr->nb;
    ctrl->spec_on = hdr->spec != 0 ? 1u : 0u;
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

// Atomics on order-preserving keys in shared memory.
__device__ __forceinline__ uint32_t atomic_cas_key(uint32_t *p, uint32_t cmp, uint32_t v) {
  return atomicCAS(p, cmp, v);
}
__device__ __forceinline__ uint64_t atomic_cas_key(uint64_t *p, uint64_t cmp, uint64_t v) {
  return atomicCAS(reinterpret_cast<unsigned long long *>(p), (unsigned long long)cmp,
                   (unsigned long long)v);
}
__device__ __forceinline__ void atomic_min_key(uint32_t *p, uint32_t v) { atomicMin(p, v); }
__device__ __forceinline__ void atomic_max_key(uint32_t *p, uint32_t v) { atomicMax(p, v); }
__device__ __forceinline__ void atomic_min_key(uint64_t *p, uint64_t v) {
  atomicMin(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}
__device__ __forceinline__ void atomic_max_key(uint64_t *p, uint64_t v) {
  atomicMax(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}

// Shared-memory position of bucket b in the histogram of a table that tracks
// single-key buckets (its keys repeat often, LutHeader::dup): the low five
// bits XOR the next five (a permutation inside every block of 1024 buckets),
// so that buckets at power-of-two strides -- integer-valued floats put theirs
// 512 apart -- do not all fall into one bank (2^26 floats in [0, 256), counts
// alone: 232 -> 79 us).  Other tables keep plain positions.
__device__ __forceinline__ uint32_t bank_swz(uint32_t b) { return b ^ ((b >> 5) & 31u); }
// buckets [0, nb) occupy positions [0, bank_span(nb)) once swizzled
__device__ __forceinline__ uint32_t bank_span(uint32_t nb) { return (nb + 1023u) & ~1023u; }

// Single-key tracking (a table whose keys repeat often): rep[i] keeps the
// first key counted at position i (KeyMax: none yet); a second distinct key --
// or the largest key, which marks an empty entry -- sets kMixed in the count.
template <class K>
__device__ __forceinline__ void track_key(uint32_t *hist, K *rep, uint32_t i, K k) {
  const K r = rep[i];
  if (r != k || k == KeyMax<K>::v) {
    if (k != KeyMax<K>::v && r == KeyMax<K>::v) {
      const K old = atomic_cas_key(&rep[i], KeyMax<K>::v, k);
      if (old != KeyMax<K>::v && old != k) atomicOr(&hist[i], kMixed);
    } else if (!(hist[i] & kMixed)) {
      atomicOr(&hist[i], kMixed);
    }
  }
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

// A warp's candidates (speculative compaction) go to chunks of kCandChunk
// keys taken from one pool (the upper half of the survivor buffer) with one
// global atomic each and listed in the warp's table of kCandChunksPerWarp
// entries (shared memory while the pass runs).  A chunk index at or past the
// pool's size means the pool ran out, and a count past the table's reach means
// the table did: either way the warp's list is incomplete and compaction reads
// the CTA's tiles instead.  Chunks follow the keys wherever they lie, so a
// sorted input whose candidates fill a few CTAs' tiles still fits.
template <class K>
struct CandPool {
  K *pool;
  uint32_t chunks;  // chunks in the pool
  uint32_t *next;   // chunks handed out so far (global)
  uint32_t lo0, len0, lo1, len1;
  __device__ __forceinline__ bool keep(uint32_t b) const {
    return (b - lo0 < len0) | (b - lo1 < len1);
  }
};

// A warp's list while the pass runs: its length and the chunk holding its
// last key, both warp-uniform in registers.
struct CandList {
  uint32_t count = 0;
  uint32_t cur = 0xFFFFFFFFu;
};

// Every lane of the warp calls this with its key and whether it keeps it:
// the keeping lanes take consecutive positions of the warp's list.  A new
// chunk (a vote adds at most 32 keys, so at most one) is taken by lane 0,
// recorded in the warp's table tab and broadcast; the table is not read here.
template <class K>
__device__ __forceinline__ void cand_put_warp(const CandPool<K> &cp, K k, bool keep,
                                              CandList &cl, uint32_t *tab) {
  const uint32_t m = __ballot_sync(0xffffffffu, keep);
  if (m) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t have = (cl.count + kCandChunk - 1) / kCandChunk;  // chunks the list holds
    const uint32_t end = cl.count + __popc(m);
    uint32_t nxt = cl.cur;
    if (end > have * kCandChunk) {
      uint32_t c = 0xFFFFFFFFu;  // no chunk: the table is full
      if (lane == 0 && have < kCandChunksPerWarp) {
        c = atomicAdd(cp.next, 1u);
        tab[have] = c;
      }
      nxt = __shfl_sync(0xffffffffu, c, 0);
    }
    if (keep) {
      const uint32_t pos = cl.count + __popc(m & ((1u << lane) - 1u));
      const uint32_t c = pos >= have * kCandChunk ? nxt : cl.cur;
      if (c < cp.chunks) cp.pool[(uint64_t)c * kCandChunk + pos % kCandChunk] = k;
    }
    cl.cur = nxt;
    cl.count = end;
  }
}

// INGEST: x is a host vector mapped into the device address space (pinned
// memory read over NVLink-C2C); every tile is also written to copy_to, the
// device copy that the later passes read.  copy_to has the same alignment
// modulo 16 bytes as x.  SPEC: keys of the kept buckets also go to the warp's
// candidate list (cand_put_warp).  SWZ: swizzled positions (bank_swz) and
// single-key tracking in rep (track_key).
template <class T, int UNROLL, bool INGEST, bool SPEC, bool SWZ>
__device__ __forceinline__ void hist_body(const T *__restrict__ x, uint64_t n, uint32_t *hist,
                                          const uint32_t *lut /* lane's table */,
                                          typename Traits<T>::K base,
                                          uint32_t shift, T *__restrict__ copy_to,
                                          const CandPool<typename Traits<T>::K> &cr,
                                          uint32_t *wcount, uint32_t *wtab,
                                          typename Traits<T>::K *rep) {
  using K = typename Traits<T>::K;
  using V = typename Traits<T>::Vec;
  constexpr int PV = Traits<T>::kPerVec;
  const Span<T> sp = split_span(x, n);
  const V *xv = reinterpret_cast<const V *>(x + sp.head);
  V *cv = reinterpret_cast<V *>(copy_to + sp.head);
  const uint64_t tile_v = (uint64_t)blockDim.x * UNROLL;
  const uint64_t ntiles = sp.nvec / tile_v;
  CandList cl;  // this warp's candidates (SPEC)
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t off = tile * tile_v + threadIdx.x;
    V v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      if (INGEST)
        v[u] = xv[off + (uint64_t)u * blockDim.x];
      else
        v[u] = ldg_stream(xv + off + (uint64_t)u * blockDim.x);
    }
    if (INGEST) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) cv[off + (uint64_t)u * blockDim.x] = v[u];
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      K k[PV];
      vec_keys<T>(v[u], k);
      uint32_t b[PV];
      bool any = false;
#pragma unroll
      for (int e = 0; e < PV; ++e) {
        b[e] = bucket_of_rep<K>(k[e], base, shift, lut);
        const uint32_t i = SWZ ? bank_swz(b[e]) : b[e];
        atomicAdd(&hist[i], 1u);
        if (SWZ) track_key<K>(hist, rep, i, k[e]);
        if (SPEC) any |= cr.keep(b[e]);
      }
      // one vote per vector; the per-key votes only when a lane keeps one
      if (SPEC && __any_sync(0xffffffffu, any)) {
#pragma unroll
        for (int e = 0; e < PV; ++e) cand_put_warp<K>(cr, k[e], cr.keep(b[e]), cl, wtab);
      }
    }
  }
  // leftover vectors (fewer than one tile) and the scalar head / tail; every
  // lane runs every round (the candidate votes need the whole warp)
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
      for (int e = 0; e < PV; ++e) {
        const uint32_t b = valid ? bucket_of_rep<K>(k[e], base, shift, lut) : 0u;
        if (valid) {
          const uint32_t i = SWZ ? bank_swz(b) : b;
          atomicAdd(&hist[i], 1u);
          if (SWZ) track_key<K>(hist, rep, i, k[e]);
        }
        if (SPEC) cand_put_warp<K>(cr, k[e], valid && cr.keep(b), cl, wtab);
      }
    }
    auto scalar = [&](uint64_t e0, uint64_t e1) {
      for (uint64_t eb = e0; eb < e1; eb += blockDim.x) {
        const uint64_t e = eb + threadIdx.x;
        const bool valid = e < e1;
        K k = 0;
        uint32_t b = 0;
        if (valid) {
          const T v = x[e];
          if (INGEST) copy_to[e] = v;
          k = Traits<T>::key(v);
          b = bucket_of_rep<K>(k, base, shift, lut);
          const uint32_t i = SWZ ? bank_swz(b) : b;
          atomicAdd(&hist[i], 1u);
          if (SWZ) track_key<K>(hist, rep, i, k);
        }
        if (SPEC) cand_put_warp<K>(cr, k, valid && cr.keep(b), cl, wtab);
      }
    };
    scalar(0, sp.head);
    scalar(sp.tail0, n);
  }
  if (SPEC && (threadIdx.x & 31) == 0) *wcount = cl.count;
}

template <class T, int UNROLL, bool INGEST, bool SPEC>
__device__ __forceinline__ void hist_dispatch(const T *__restrict__ x, uint64_t n, uint32_t *hist,
                                              const uint32_t *lut,
                                              const LutHeader<typename Traits<T>::K> &h,
                                              T *__restrict__ copy_to,
                                              const CandPool<typename Traits<T>::K> &cr,
                                              uint32_t *wcount, uint32_t *wtab,
                                              typename Traits<T>::K *rep) {
  // The histogram's atomics return nothing; lanes of a warp adding to one
  // counter cost no more than lanes adding to different ones, so the warp
  // aggregation that compaction uses (h.heavy) only slows this pass down
  // (measured at 2^26: two-valued, constant and sorted inputs 74 -> 55 us).
  // rep: single-key tracking (and swizzled positions), see k_hist.
  if (rep)
    hist_body<T, UNROLL, INGEST, SPEC, true>(x, n, hist, lut, h.base, h.shift, copy_to, cr,
                                             wcount, wtab, rep);
  else
    hist_body<T, UNROLL, INGEST, SPEC, false>(x, n, hist, lut, h.base, h.shift, copy_to, cr,
                                              wcount, wtab, nullptr);
}

// copy_to == nullptr: x is the device vector.  Otherwise x is a mapped host
// vector and this pass also writes the device copy (see hist_body).  cand:
// the candidate pool (nullptr: no speculation); when the table keeps
// buckets, warp w of CTA c lists its candidates in pool chunks and leaves its
// count in cand_cnt[c * kCandWarps + w] and its chunk table in
// cand_tab[(c * kCandWarps + w) * kCandChunksPerWarp ...); cand_next counts
// the chunks handed out (zero on entry).  reps (nullptr: none): when the
// table's keys repeat often and it has at most dup_nb_cap(nb_max) buckets, the
// CTA also tracks each bucket's key (the first dup_nb_cap counts of the shared
// histogram are followed by as many keys) and writes its row of keys to
// reps[c * nb_max ...), with kMixed in the row's count where a bucket held
// more than one key.
template <class T, int UNROLL>
__global__ void __launch_bounds__(1024, 1)
    k_hist(const T *__restrict__ x, uint64_t n, const LutHeader<typename Traits<T>::K> *hdr,
           const uint32_t *__restrict__ lut_g, uint32_t *__restrict__ partials, uint32_t nb_max,
           const Ctrl *ctrl, T *__restrict__ copy_to, typename Traits<T>::K *__restrict__ cand,
           uint32_t *__restrict__ cand_cnt, uint32_t *__restrict__ cand_tab,
           uint32_t *cand_next, typename Traits<T>::K *__restrict__ reps) {
  pdl_start();
  using K = typename Traits<T>::K;
  extern __shared__ uint4 smem_raw[];
  uint32_t *rep_lut = reinterpret_cast<uint32_t *>(smem_raw);  // one copy per bank
  uint32_t *hist = (rep_lut + kRepWords);
  const uint32_t *lut = rep_lut + (threadIdx.x & 31);  // this lane's copy
  __shared__ uint32_t s_wcnt[kCandWarps];
  __shared__ uint32_t s_tab[kCandWarps * kCandChunksPerWarp];
  if (ctrl->status & ST_FATAL) return;
  const LutHeader<K> h = *hdr;
  load_rep_table(rep_lut, lut_g);
  const uint32_t dcap = dup_nb_cap<K>(nb_max);
  const bool track = reps != nullptr && h.dup && dcap != 0 && h.nb <= dcap;
  K *rep = track ? reinterpret_cast<K *>(hist + dcap) : nullptr;
  const uint32_t span = min(bank_span(h.nb), nb_max);
  for (uint32_t b = threadIdx.x; b < span; b += blockDim.x) {
    hist[b] = 0;
    if (track) rep[b] = KeyMax<K>::v;
  }
  __syncthreads();
  const bool spec = cand != nullptr && h.spec != 0;
  const uint32_t warp = threadIdx.x >> 5;
  CandPool<K> cr;
  cr.pool = cand;
  cr.chunks = h.cand_cap;
  cr.next = cand_next;
  cr.lo0 = h.spec_lo[0];
  cr.len0 = h.spec_len[0];
  cr.lo1 = h.spec_lo[1];
  cr.len1 = h.spec_len[1];
  uint32_t *wc = s_wcnt + warp, *wt = s_tab + warp * kCandChunksPerWarp;
  if (copy_to) {
    if (spec)
      hist_dispatch<T, UNROLL, true, true>(x, n, hist, lut, h, copy_to, cr, wc, wt, rep);
    else
      hist_dispatch<T, UNROLL, true, false>(x, n, hist, lut, h, copy_to, cr, wc, wt, rep);
  } else {
    if (spec)
      hist_dispatch<T, UNROLL, false, true>(x, n, hist, lut, h, nullptr, cr, wc, wt, rep);
    else
      hist_dispatch<T, UNROLL, false, false>(x, n, hist, lut, h, nullptr, cr, wc, wt, rep);
  }
  __syncthreads();
  uint32_t *row = partials + (uint64_t)blockIdx.x * nb_max;
  for (uint32_t b = threadIdx.x; b < h.nb; b += blockDim.x) {
    const uint32_t i = track ? bank_swz(b) : b;
    row[b] = hist[i];
    if (track) reps[(uint64_t)blockIdx.x * nb_max + b] = rep[i];
  }
  if (spec) {
    if (threadIdx.x < kCandWarps)
      cand_cnt[(uint64_t)blockIdx.x * kCandWarps + threadIdx.x] = s_wcnt[threadIdx.x];
    // entries past a warp's chunks are never read
    for (uint32_t i = threadIdx.x; i < kCandWarps * kCandChunksPerWarp; i += blockDim.x)
      cand_tab[(uint64_t)blockIdx.x * kCandWarps * kCandChunksPerWarp + i] = s_tab[i];
  }
}

// ---------------------------------------------------------------------------
// (d) bucket totals: column sums of the per-CTA rows
// ---------------------------------------------------------------------------
// Each CTA sums kScanTile buckets over the rows and writes their exclusive
// prefix inside the tile and the tile's total; the kernels that search the
// bucket prefix (k_plan, k_reqmap: load_prefix) add the tiles' offsets in
// shared memory.  A grid-wide scan here would make every tile wait on its
// predecessors.
constexpr int kScanThreads = 256;
constexpr int kScanTile = 64;  // buckets per CTA

// 16 lanes read a row's 64 buckets of the tile as 16-byte vectors, and the
// CTA's 16 groups of 16 lanes split the rows between them (8 rows per thread
// at once: two rounds of loads for 152 rows; a tracking table reads the rows
// again for the buckets' keys).  The rows are read once;
// compaction later takes each CTA's share of a bucket's segment from its own
// row.
template <class K>
__global__ void __launch_bounds__(kScanThreads, 4)
    k_colsum(const uint32_t *__restrict__ partials, uint32_t rows, uint32_t nb_max,
             const LutHeader<K> *hdr, uint32_t *__restrict__ bpre, uint32_t *__restrict__ ttot,
             const Ctrl *ctrl, const K *__restrict__ reps, uint32_t *__restrict__ bsingle,
             K *__restrict__ bkey) {
  pdl_start();
  constexpr uint32_t kVecs = kScanTile / 4;              // 16-byte vectors per tile row
  constexpr uint32_t kGroups = kScanThreads / kVecs;     // row groups
  constexpr uint32_t kBatch = 8;                         // loads in flight per thread
  __shared__ uint32_t gsum[kGroups][kScanTile];
  __shared__ uint32_t s_w2[2];
  __shared__ uint8_t gstate[kGroups][kScanTile];  // single-key tracking: 0 none, 1 one key, 2 more
  __shared__ K gkey[kGroups][kScanTile];
  if (ctrl->status & ST_FATAL) return;
  const uint32_t nb = hdr->nb;
  if ((uint64_t)blockIdx.x * kScanTile >= nb) return;
  const uint32_t dcap = dup_nb_cap<K>(nb_max);
  const bool track = reps != nullptr && hdr->dup && dcap != 0 && nb <= dcap;
  // thread t sums buckets 4 (t % kVecs) .. + 3 of the tile over row group
  // t / kVecs: a row's 64 buckets are one 256-byte span read by 16 lanes
  const uint32_t v = threadIdx.x % kVecs, grp = threadIdx.x / kVecs;
  const uint32_t b0 = blockIdx.x * kScanTile + 4 * v;
  const uint32_t per = (rows + kGroups - 1) / kGroups;
  const uint32_t r0 = grp * per, r1 = min(rows, r0 + per);
  const uint4 *p = reinterpret_cast<const uint4 *>(partials + b0);
  const uint32_t row4 = nb_max / 4;  // nb_max is a multiple of 4
  uint4 gs = make_uint4(0, 0, 0, 0);
  if (b0 < nb) {
    for (uint32_t r = r0; r < r1; r += kBatch) {
      uint4 e[kBatch];
#pragma unroll
      for (uint32_t q = 0; q < kBatch; ++q)
        e[q] = r + q < r1 ? __ldcg(p + (uint64_t)(r + q) * row4) : make_uint4(0, 0, 0, 0);
#pragma unroll
      for (uint32_t q = 0; q < kBatch; ++q) {
        gs.x += e[q].x & ~kMixed;
        gs.y += e[q].y & ~kMixed;
        gs.z += e[q].z & ~kMixed;
        gs.w += e[q].w & ~kMixed;
      }
    }
  }
  // single-key tracking of the four buckets (a second pass over the rows, in
  // tracking tables only): per row with keys in a bucket, its key or "more
  // than one"
  uint32_t st[4] = {0, 0, 0, 0};  // 0 none, 1 one key (key), 2 more
  K key[4] = {0, 0, 0, 0};
  if (track && b0 < nb) {
    for (uint32_t r = r0; r < r1; ++r) {
      const uint4 e = __ldcg(p + (uint64_t)r * row4);
      const uint32_t c4[4] = {e.x, e.y, e.z, e.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (!(c4[j] & ~kMixed)) continue;
        if (c4[j] & kMixed) {
          st[j] = 2;
        } else if (st[j] != 2) {
          const K rk = __ldcg(reps + (uint64_t)r * nb_max + b0 + j);
          if (st[j] == 0) {
            st[j] = 1;
            key[j] = rk;
          } else if (rk != key[j]) {
            st[j] = 2;
          }
        }
      }
    }
  }
  // rows hold stale counts past nb
  gsum[grp][4 * v + 0] = b0 + 0 < nb ? gs.x : 0u;
  gsum[grp][4 * v + 1] = b0 + 1 < nb ? gs.y : 0u;
  gsum[grp][4 * v + 2] = b0 + 2 < nb ? gs.z : 0u;
  gsum[grp][4 * v + 3] = b0 + 3 < nb ? gs.w : 0u;
  if (track) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      gstate[grp][4 * v + j] = (uint8_t)st[j];
      gkey[grp][4 * v + j] = key[j];
    }
  }
  __syncthreads();
  // the tile's kScanTile buckets (two warps) -> their exclusive prefix inside
  // the tile, and the tile's total
  const uint32_t col = threadIdx.x;
  uint32_t c = 0, incl = 0;
  if (col < kScanTile) {
#pragma unroll
    for (uint32_t g = 0; g < kGroups; ++g) c += gsum[g][col];
    incl = warp_incl_scan(c);
    if ((col & 31) == 31) s_w2[col >> 5] = incl;
  }
  __syncthreads();
  if (col < kScanTile) {
    const uint32_t b = blockIdx.x * kScanTile + col;
    if (b < nb) bpre[b] = incl - c + (col >= 32 ? s_w2[0] : 0u);
    if (col == 0) ttot[blockIdx.x] = s_w2[0] + s_w2[1];
    if (track && b < nb) {
      // one key in the whole vector: every row group saw none or the same one
      uint32_t s1 = 0;
      K k1 = 0;
#pragma unroll
      for (uint32_t g = 0; g < kGroups; ++g) {
        const uint32_t sg = gstate[g][col];
        if (sg == 2 || (sg == 1 && s1 == 1 && gkey[g][col] != k1)) s1 = 2;
        else if (sg == 1 && s1 == 0) {
          s1 = 1;
          k1 = gkey[g][col];
        }
      }
      bsingle[b] = s1 == 1 ? 1u : 0u;
      bkey[b] = k1;
    }
  }
}
static_assert(kScanTile == 64, "k_colsum's tile prefix covers two warps");

// In place: a[0 .. nb) (bucket totals, 16-byte aligned, zero from nb up to
// the next multiple of 4) becomes its exclusive prefix; returns the total.
// Warp w owns a contiguous run of 16-byte vectors, read in rounds of 32
// neighbouring vectors (conflict-free); one pass sums, one pass writes.
static __device__ uint64_t smem_excl_scan(uint32_t *a, uint32_t nb, uint32_t *s_w /* >= 33 */) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint4 *a4 = reinterpret_cast<uint4 *>(a);
  const uint32_t nv = (nb + 3) >> 2;
  const uint32_t span = (((nv + nwarps - 1) / nwarps) + 31) & ~31u;  // vectors per warp
  const uint32_t v0 = warp * span;
  uint32_t mine = 0;
  for (uint32_t r = 0; r < span; r += 32) {
    const uint32_t v = v0 + r + lane;
    if (v < nv) {
      const uint4 c = a4[v];
      mine += c.x + c.y + c.z + c.w;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if (lane == 0) s_w[warp] = mine;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < nwarps ? s_w[lane] : 0u;
    const uint32_t incl = warp_incl_scan(w);
    if (lane < nwarps) s_w[lane] = incl - w;
    if (lane == 31) s_w[32] = incl;
  }
  __syncthreads();
  uint32_t base = s_w[warp];
  for (uint32_t r = 0; r < span; r += 32) {
    const uint32_t v = v0 + r + lane;
    uint4 c = make_uint4(0, 0, 0, 0);
    if (v < nv) c = a4[v];
    const uint32_t sum = c.x + c.y + c.z + c.w;
    const uint32_t incl = warp_incl_scan(sum);
    const uint32_t pre = base + incl - sum;
    if (v < nv) a4[v] = make_uint4(pre, pre + c.x, pre + c.x + c.y, pre + c.x + c.y + c.z);
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
  const uint64_t total = s_w[32];
  __syncthreads();
  return total;
}

// ---------------------------------------------------------------------------
// (e) plan: requests -> buckets -> slots; request lists per slot
// ---------------------------------------------------------------------------
// With tens of thousands of requests the per-request work leaves the single
// plan CTA: k_reqmap (many CTAs) maps every request to its bucket and local
// rank, flags the bucket in a bitmap and counts requests per bucket; k_plan
// then numbers the slots from the bitmap and takes the per-slot counts from
// the bucket counts; k_reqplace (many CTAs) writes the request lists.
constexpr uint32_t kPremapMin = 16384;     // requests from which the mapping is spread out
constexpr uint32_t kReqmapPerCta = 4096;   // requests per k_reqmap CTA (1024 threads)

struct Premap {
  const uint32_t *bits = nullptr;    // bucket flags, one bit each (null: not premapped)
  const uint32_t *bcount = nullptr;  // requests per bucket
  uint32_t *bslot = nullptr;         // slot of each flagged bucket (written by k_plan)
};

// Bucket totals counts_g[0 .. nb) -> a[] (shared, 16-byte aligned), zero up
// to the next multiple of 4; every load of a step in flight before the
// stores.
__device__ __forceinline__ void load_totals(const uint32_t *__restrict__ counts_g, uint32_t nb,
                                            uint32_t *a) {
  const uint32_t nb4 = (nb + 3) >> 2;
  for (uint32_t v0 = threadIdx.x; v0 < nb4; v0 += 4 * blockDim.x) {
    uint4 e[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t v = v0 + u * blockDim.x;
      e[u] = v < nb4 ? __ldcg(reinterpret_cast<const uint4 *>(counts_g) + v) : make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t v = v0 + u * blockDim.x;
      if (v < nb4) {
        if (4 * v + 4 > nb) {  // the last vector: totals past nb are stale
          const uint32_t k = nb - 4 * v;
          if (k < 2) e[u].y = 0;
          if (k < 3) e[u].z = 0;
          e[u].w = 0;
        }
        reinterpret_cast<uint4 *>(a)[v] = e[u];
      }
    }
  }
}

// The exclusive bucket prefix into a[] (shared, 16-byte aligned): bpre_g holds
// each bucket's prefix inside its tile of kScanTile buckets, ttot_g the tiles'
// totals (k_colsum).  The tile totals are scanned (one per thread: at most
// kMaxNb / kScanTile tiles), then every bucket adds its tile's offset.
// Returns the total.
//
// With bar set, the tile prefixes come by one bulk copy that completes on bar
// (phase 0) while the tile totals are scanned: issued here by thread 0 when
// issue is set, else already issued by the caller (bulk_prefix_bytes(nb)
// bytes).  A wait that gives up marks the call timed out in *status.
__device__ __forceinline__ uint32_t bulk_prefix_bytes(uint32_t nb) { return ((nb + 3) >> 2) * 16u; }

static __device__ uint64_t load_prefix(const uint32_t *__restrict__ bpre_g,
                                       const uint32_t *__restrict__ ttot_g, uint32_t nb,
                                       uint32_t *a, uint32_t *s_tile /* kMaxNb / kScanTile */,
                                       uint32_t *red /* 33 */, uint64_t *bar = nullptr,
                                       bool issue = false, uint32_t *status = nullptr) {
  const uint32_t ntile = (nb + kScanTile - 1) / kScanTile;
  if (bar && issue && threadIdx.x == 0) {
    mbar_init(bar);
    mbar_expect_tx(bar, bulk_prefix_bytes(nb));
    bulk_g2s(a, bpre_g, bulk_prefix_bytes(nb), bar);
  }
  const uint32_t t = threadIdx.x < ntile ? __ldcg(ttot_g + threadIdx.x) : 0u;
  if (!bar) load_totals(bpre_g, nb, a);
  uint32_t tot;
  const uint32_t ex = block_incl_scan(t, &tot, red) - t;  // ends with a barrier
  if (bar) {
    if (!mbar_wait(bar, 0)) {
      if (status) atomicOr(status, ST_TIMEOUT);
      mbar_wait(bar, 0);  // once more for the copy in flight, then go on
    }
    // the last vector's entries past nb are stale
    if (threadIdx.x < 4u * ((nb + 3) >> 2) - nb) a[nb + threadIdx.x] = 0;
  }
  if (threadIdx.x < ntile) s_tile[threadIdx.x] = ex;
  __syncthreads();
  uint4 *a4 = reinterpret_cast<uint4 *>(a);
  for (uint32_t v = threadIdx.x; v < ((nb + 3) >> 2); v += blockDim.x) {
    const uint32_t o = s_tile[v / (kScanTile / 4)];  // four buckets of one tile
    uint4 x = a4[v];
    x.x += o;
    x.y += o;
    x.z += o;
    x.w += o;
    a4[v] = x;
  }
  __syncthreads();
  return tot;
}

// Bitmap and counts must start at zero.  Shared memory: the bucket prefix
// (nb_max u32), from the tile prefixes and totals.
static __global__ void __launch_bounds__(1024)
    k_reqmap(const uint32_t *__restrict__ bpre_g, const uint32_t *__restrict__ ttot_g,
             const Ctrl *ctrl, const Req *__restrict__ reqs, uint32_t num_req,
             uint32_t *__restrict__ req_bucket, uint32_t *__restrict__ req_local, uint32_t *bits,
             uint32_t *bcount) {
  pdl_start();
  extern __shared__ uint4 smem_raw[];
  uint32_t *excl = reinterpret_cast<uint32_t *>(smem_raw);
  __shared__ uint32_t s_w[33];
  __shared__ uint32_t s_tile[kMaxNb / kScanTile];
  __shared__ uint64_t s_bar;
  if (ctrl->status & ST_FATAL) return;
  const uint32_t nb = ctrl->nb;
  const bool bulk = aligned16(bpre_g) && aligned16(excl);
  load_prefix(bpre_g, ttot_g, nb, excl, s_tile, s_w, bulk ? &s_bar : nullptr, true,
              const_cast<uint32_t *>(&ctrl->status));
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t u = 0; u < kReqmapPerCta / 1024; ++u) {
    const uint32_t i = blockIdx.x * kReqmapPerCta + u * 1024 + threadIdx.x;
    const bool valid = i < num_req;
    uint32_t b = 0xFFFFFFFFu;
    if (valid) {
      const uint32_t rank = reqs[i].rank;
      uint32_t lo = 0, hi = nb;
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (excl[mid] <= rank)
          lo = mid;
        else
          hi = mid;
      }
      b = lo;
      req_bucket[i] = lo;
      req_local[i] = rank - excl[lo];
    }
    // one count and one flag per bucket per warp (neighbouring requests often
    // share a bucket)
    const uint32_t peers = __match_any_sync(0xffffffffu, b);
    if (valid && (int)lane == __ffs(peers) - 1) {
      atomicAdd(&bcount[b], (uint32_t)__popc(peers));
      atomicOr(&bits[b >> 5], 1u << (b & 31));
    }
  }
}

// klist positions: kstart[slot] + arrival order in the slot (warp-aggregated
// cursors; kcur starts at zero, set by k_plan).
static __global__ void __launch_bounds__(1024)
    k_reqplace(const Ctrl *ctrl, const Req *__restrict__ reqs, uint32_t num_req,
               const uint32_t *__restrict__ req_bucket, const uint32_t *__restrict__ req_local,
               const uint32_t *__restrict__ bslot, const uint32_t *__restrict__ kstart,
               uint32_t *kcur, Req *__restrict__ klist) {
  pdl_start();
  if (ctrl->status & ST_FATAL) return;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < num_req;
  const uint32_t q = valid ? bslot[req_bucket[i]] : 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t peers = __match_any_sync(0xffffffffu, q);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (valid && (int)lane == leader) base = atomicAdd(&kcur[q], (uint32_t)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (valid) {
    Req e;
    e.rank = req_local[i];
    e.out = reqs[i].out;
    klist[kstart[q] + base + __popc(peers & ((1u << lane) - 1u))] = e;
  }
}

// Flag words per lane in k_plan's slot numbering (1024 threads, kMaxNb buckets).
constexpr uint32_t kPlanRounds = kMaxNb / 4 / 1024;
static_assert(kPlanRounds * 4 * 1024 == kMaxNb, "k_plan slot numbering covers kMaxNb buckets");

// k_plan's request mapping: bucket = the last b with excl[b] <= rank (a
// fixed-step search over the prefix in shared memory), the request's rank
// inside it, and the bucket's flag.  R requests per thread and step.
template <int R>
__device__ __forceinline__ void plan_map_requests(const uint32_t *excl, uint32_t nb,
                                                  const Req *__restrict__ reqs, uint32_t num_req,
                                                  uint8_t *flag, uint32_t *__restrict__ req_bucket,
                                                  uint32_t *__restrict__ req_local) {
  const uint32_t nt = blockDim.x;
  const uint32_t top = nb > 1 ? 1u << (31 - __clz(nb - 1)) : 0u;  // largest step
  for (uint32_t i0 = threadIdx.x; i0 < num_req; i0 += R * nt) {
    uint32_t rank[R], lo[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const uint32_t i = i0 + u * nt;
      rank[u] = i < num_req ? reqs[i].rank : 0u;
      lo[u] = 0;
    }
    for (uint32_t step = top; step; step >>= 1) {
#pragma unroll
      for (int u = 0; u < R; ++u) {
        const uint32_t m = lo[u] + step;
        if (m < nb && excl[m] <= rank[u]) lo[u] = m;
      }
    }
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const uint32_t i = i0 + u * nt;
      if (i < num_req) {
        flag[lo[u]] = 1;
        req_bucket[i] = lo[u];
        req_local[i] = rank[u] - excl[lo[u]];
      }
    }
  }
}

// One CTA of 1024 threads.  Dynamic shared memory: lut[kLutEntries + 1] (u32,
// padded to 16 bytes), excl[nb_max] (u32), flags[nb_max] (u8).
//
// Every bucket that holds a requested rank gets a slot, in bucket order.  A
// bucket whose key range is a single key is a "flat" slot: seg_size 0, no
// survivors (compaction skips it), and the finisher answers its requests with
// that key.  Other slots own a segment of the survivor buffer of exactly the
// bucket's count.
template <class InT, class OutT>
__global__ void __launch_bounds__(1024, 1)
    k_plan(const LutHeader<typename Traits<InT>::K> *hdr, const uint32_t *__restrict__ lut_g,
           const uint32_t *__restrict__ bpre, const uint32_t *__restrict__ ttot, uint64_t n,
           const Req *__restrict__ reqs, uint32_t num_req, uint32_t nb_max, Ctrl *ctrl,
           uint32_t *__restrict__ seg_bucket,
           uint64_t *__restrict__ seg_off, uint32_t *__restrict__ seg_size,
           uint32_t *__restrict__ kstart, uint32_t *__restrict__ kcnt,
           uint32_t *__restrict__ kcur, uint32_t *__restrict__ fill,
           typename Traits<InT>::K *__restrict__ seg_lo,
           typename Traits<InT>::K *__restrict__ seg_hi, uint32_t *__restrict__ req_bucket,
           uint32_t *__restrict__ req_local, Req *__restrict__ klist, uint64_t surv_cap,
           Premap pm, const uint32_t *__restrict__ bsingle = nullptr,
           const typename Traits<InT>::K *__restrict__ bkey = nullptr) {
  // The requests are complete before the call's first kernel (uploaded, made
  // by a kernel the plainly launched sample kernel waits for, or left by an
  // earlier call): with at most one per thread, each thread loads its own
  // ahead of the dependency wait.
  pdl_trigger();
  const bool own = num_req <= blockDim.x;
  Req my_rq;
  my_rq.rank = 0;
  my_rq.out = 0;
  if (own && !pm.bits && threadIdx.x < num_req) my_rq = reqs[threadIdx.x];
  pdl_wait();
  using K = typename Traits<InT>::K;
  extern __shared__ uint4 smem_raw[];
  uint32_t *lut = reinterpret_cast<uint32_t *>(smem_raw);
  uint32_t *excl = lut + kLutPadded;  // 16-byte aligned; later: slot of each bucket
  uint8_t *flag = reinterpret_cast<uint8_t *>(excl + nb_max);
  uint32_t *s_segb = reinterpret_cast<uint32_t *>(flag);  // once the flags are in registers
  __shared__ uint32_t red32[33];
  __shared__ uint64_t red64[33];
  __shared__ uint32_t s_wbase[33];
  __shared__ uint32_t s_tile[kMaxNb / kScanTile];
  const uint32_t tid = threadIdx.x, nt = blockDim.x;

  __shared__ uint64_t s_bar;
  if (ctrl->status & ST_FATAL) return;
  const LutHeader<K> h = *hdr;
  const uint32_t nb = h.nb;
  // the table and the tile prefixes come by bulk copies that run while the
  // flags are loaded and the tile totals scanned
  const bool bulk = aligned16(bpre) && aligned16(lut_g) && aligned16(lut) && aligned16(excl);
  if (bulk && tid == 0) {
    mbar_init(&s_bar);
    mbar_expect_tx(&s_bar, bulk_prefix_bytes(nb) + kLutPadded * 4u);
    bulk_g2s(lut, lut_g, kLutPadded * 4u, &s_bar);
    bulk_g2s(excl, bpre, bulk_prefix_bytes(nb), &s_bar);
  }
  // flags, one word per four buckets; every load of a step is issued before
  // the first shared store (loads and stores interleaved in one loop body
  // complete one at a time)
  const uint32_t nb4 = (nb + 3) >> 2;
  for (uint32_t v0 = tid; v0 < nb4; v0 += 4 * nt) {
    uint32_t f[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t v = v0 + u * nt;
      f[u] = v < nb4 && pm.bits ? __ldcg(pm.bits + (v >> 3)) : 0u;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t v = v0 + u * nt;
      if (v < nb4) {
        // flags of buckets 4v .. 4v + 3, one byte each
        const uint32_t f4 = (f[u] >> ((4 * v) & 31)) & 0xFu;
        reinterpret_cast<uint32_t *>(flag)[v] =
            (f4 & 1u) | ((f4 & 2u) << 7) | ((f4 & 4u) << 14) | ((f4 & 8u) << 21);
      }
    }
  }
  for (uint32_t j0 = tid; j0 < (bulk ? 0u : kLutEntries); j0 += 8 * nt) {
    uint32_t e[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const uint32_t j = j0 + u * nt;
      e[u] = j < kLutEntries ? __ldcg(lut_g + j) : 0u;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (j0 + u * nt < kLutEntries) lut[j0 + u * nt] = e[u];
  }
  if (tid == 0) ctrl->deferred_count = 0;
  __syncthreads();
  // the bucket prefix; the totals must add up to n (else the input changed
  // under the histogram)
  if (load_prefix(bpre, ttot, nb, excl, s_tile, s_wbase, bulk ? &s_bar : nullptr, false,
                  &ctrl->status) != n &&
      tid == 0)
    atomicOr(&ctrl->status, ST_INTERNAL);

  // requests -> bucket (the last b with excl[b] <= rank is never empty) and
  // the rank inside it; with many requests, four per thread and step, so that
  // their loads and searches overlap
  uint32_t my_b = 0;  // the bucket of the thread's own request
  if (!pm.bits) {
    if (own) {
      if (tid < num_req) {
        const uint32_t top = nb > 1 ? 1u << (31 - __clz(nb - 1)) : 0u;
        uint32_t lo = 0;
        for (uint32_t step = top; step; step >>= 1) {
          const uint32_t m = lo + step;
          if (m < nb && excl[m] <= my_rq.rank) lo = m;
        }
        flag[lo] = 1;
        my_b = lo;
        my_rq.rank -= excl[lo];  // now the rank inside the bucket
      }
    } else if (num_req >= 4096) {
      plan_map_requests<4>(excl, nb, reqs, num_req, flag, req_bucket, req_local);
    } else {
      plan_map_requests<1>(excl, nb, reqs, num_req, flag, req_bucket, req_local);
    }
  }
  __syncthreads();

  // Slots in bucket order.  Warp w owns the flag words [w wpw, (w + 1) wpw)
  // (one byte per bucket, 0 or 1), read in rounds of 32 neighbouring words;
  // the flags stay in registers, so from the warp-total scan on the flag
  // bytes can hold the slot -> bucket list (s_segb, while it fits).  Once the
  // slots have read their buckets' sizes from excl[], it maps each flagged
  // bucket to its slot.
  const uint32_t lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const uint32_t nw = (nb + 3) >> 2;
  const uint32_t wpw = (((nw + nwarps - 1) / nwarps) + 31) & ~31u;
  const uint32_t rounds = wpw >> 5;  // <= kPlanRounds for 1024 threads
  uint32_t fw[kPlanRounds];
  uint32_t mine = 0;
#pragma unroll
  for (uint32_t r = 0; r < kPlanRounds; ++r) {
    const uint32_t w = warp * wpw + r * 32 + lane;
    fw[r] = (r < rounds && w < nw) ? reinterpret_cast<const uint32_t *>(flag)[w] : 0u;
    mine += __popc(fw[r]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if (lane == 0) s_wbase[warp] = mine;
  __syncthreads();
  if (warp == 0) {
    const uint32_t v = lane < nwarps ? s_wbase[lane] : 0u;
    const uint32_t incl = warp_incl_scan(v);
    if (lane < nwarps) s_wbase[lane] = incl - v;
    if (lane == 31) s_wbase[32] = incl;
  }
  __syncthreads();
  const uint32_t tot_slots = s_wbase[32];
  const bool segb_smem = tot_slots <= nb_max / 4;
  {
    uint32_t slot0 = s_wbase[warp];
#pragma unroll
    for (uint32_t r = 0; r < kPlanRounds; ++r) {
      if (r >= rounds) break;
      const uint32_t c = __popc(fw[r]);
      const uint32_t incl = warp_incl_scan(c);
      uint32_t slot = slot0 + incl - c;
      const uint32_t b4 = 4u * (warp * wpw + r * 32 + lane);
      for (uint32_t bits = fw[r]; bits; bits &= bits - 1u) {
        const uint32_t b = b4 + ((__ffs(bits) - 1) >> 3);
        seg_bucket[slot] = b;
        if (segb_smem) s_segb[slot] = b;
        if (pm.bits) pm.bslot[b] = slot;
        ++slot;
      }
      slot0 += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncthreads();
  // one thread per slot (contiguous slot range per thread for the offsets):
  // key range, flat test, survivor count
  const uint32_t sper = (tot_slots + nt - 1) / nt;
  const uint32_t s0 = min(tot_slots, tid * sper), s1 = min(tot_slots, s0 + sper);
  uint64_t my_surv = 0;
  const uint32_t dcap = dup_nb_cap<K>(nb_max);
  const bool dtrack = bsingle != nullptr && bkey != nullptr && h.dup && dcap != 0 && nb <= dcap;
  for (uint32_t q = s0; q < s1; ++q) {
    const uint32_t b = segb_smem ? s_segb[q] : __ldcg(seg_bucket + q);
    const K klo = bucket_lo<K>(b, h.base, h.shift, lut, kSvSlices);
    const K knext = (b + 1 < nb) ? bucket_lo<K>(b + 1, h.base, h.shift, lut, kSvSlices) : K(0);
    // single key iff the next bucket starts one key later; the start of the
    // top entry's bucket can wrap past the key width, and then bucket b runs
    // up to the largest key
    const bool single = (knext > klo) ? (knext - klo == K(1)) : (klo == KeyMax<K>::v);
    // a wider bucket that the histogram pass saw holding one key (k_colsum)
    const bool one = !single && dtrack && __ldcg(bsingle + b) != 0u;
    const uint32_t cb =
        (single || one) ? 0u : (uint32_t)((b + 1 < nb ? excl[b + 1] : n) - excl[b]);
    const K flat_key = one ? __ldcg(bkey + b) : klo;
    seg_size[q] = cb;  // 0 marks a flat slot
    seg_lo[q] = flat_key;
    seg_hi[q] = (single || one) ? flat_key : (knext > klo ? knext - K(1) : KeyMax<K>::v);
    kcnt[q] = pm.bits ? __ldcg(pm.bcount + b) : 0u;  // premapped: the bucket's request count
    kcur[q] = 0;
    fill[q] = 0;
    my_surv += cb;
  }
  uint64_t tot_surv;
  {
    // the sizes of all but a thread's last slot are read back (none for one
    // slot per thread)
    uint64_t off = block_incl_scan(my_surv, &tot_surv, red64) - my_surv;
    for (uint32_t q = s0; q < s1; ++q) {
      seg_off[q] = off;
      if (q + 1 < s1) off += __ldcg(seg_size + q);
      // the sizes are read (the scan's barriers passed): bucket -> slot
      excl[segb_smem ? s_segb[q] : __ldcg(seg_bucket + q)] = q;
    }
  }
  if (tid == 0) {
    ctrl->num_slots = tot_slots;
    ctrl->total_surv = tot_surv;
    if (tot_surv > surv_cap) {
      atomicOr(&ctrl->status, ST_OVERFLOW);
      ctrl->cap_needed = tot_surv;
    }
    // compaction cursors carry the survivor position in 31 bits
    if (tot_surv >= (uint64_t)kInactive) atomicOr(&ctrl->status, ST_INTERNAL);
  }
  __syncthreads();

  // requests per slot, then the request lists (local ranks).  Many requests
  // in few slots (a top-k) would queue on a few global counters, so the
  // per-slot counters live in shared memory when the launch left room for
  // them after the table, prefix and flags (the room is read from
  // %dynamic_smem_size; a launch without it uses the global counters).
  uint32_t dyn;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
  const uint32_t used = (uint32_t)((kLutPadded * 4 + (size_t)nb_max * 5 + 15) & ~(size_t)15);
  const uint32_t room = dyn > used ? (dyn - used) / 8 : 0u;
  uint32_t *s_cnt = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(smem_raw) + used);
  uint32_t *s_cur = s_cnt + room;  // cursor = slot start + requests placed so far
  const bool in_smem = !pm.bits && tot_slots <= room;
  if (pm.bits) {
    // counted by k_reqmap; kcnt holds them already
  } else if (own) {
    // one request per thread, its bucket in a register
    if (in_smem) {
      for (uint32_t q = tid; q < tot_slots; q += nt) s_cnt[q] = 0;
      __syncthreads();
    }
    if (tid < num_req) atomicAdd(in_smem ? &s_cnt[excl[my_b]] : &kcnt[excl[my_b]], 1u);
  } else if (in_smem) {
    for (uint32_t q = tid; q < tot_slots; q += nt) s_cnt[q] = 0;
    __syncthreads();
    // four requests per thread and step: the global loads overlap
    for (uint32_t i0 = tid; i0 < num_req; i0 += 4 * nt) {
      uint32_t b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) b[u] = i0 + u * nt < num_req ? req_bucket[i0 + u * nt] : 0u;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u * nt < num_req) atomicAdd(&s_cnt[excl[b[u]]], 1u);
    }
  } else {
    for (uint32_t i = tid; i < num_req; i += nt) atomicAdd(&kcnt[excl[req_bucket[i]]], 1u);
  }
  __syncthreads();
  {
    uint32_t mine = 0;
    for (uint32_t q = s0; q < s1; ++q) mine += in_smem ? s_cnt[q] : kcnt[q];
    uint32_t tot;
    uint32_t run = block_incl_scan(mine, &tot, red32) - mine;
    for (uint32_t q = s0; q < s1; ++q) {
      const uint32_t c = in_smem ? s_cnt[q] : kcnt[q];
      if (in_smem) {
        kcnt[q] = c;  // the finisher reads the counts
        s_cur[q] = run;
      }
      kstart[q] = run;
      run += c;
    }
  }
  __syncthreads();
  if (pm.bits) {
    // k_reqplace writes the lists
  } else if (own) {
    if (tid < num_req) {
      const uint32_t q = excl[my_b];
      klist[in_smem ? atomicAdd(&s_cur[q], 1u) : kstart[q] + atomicAdd(&kcur[q], 1u)] = my_rq;
    }
  } else if (in_smem) {
    for (uint32_t i0 = tid; i0 < num_req; i0 += 4 * nt) {
      uint32_t b[4], loc[4], o[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t i = i0 + u * nt;
        const bool ok = i < num_req;
        b[u] = ok ? req_bucket[i] : 0u;
        loc[u] = ok ? req_local[i] : 0u;
        o[u] = ok ? reqs[i].out : 0u;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u * nt < num_req) {
          Req e;
          e.rank = loc[u];
          e.out = o[u];
          klist[atomicAdd(&s_cur[excl[b[u]]], 1u)] = e;
        }
    }
  } else {
    for (uint32_t i = tid; i < num_req; i += nt) {
      const uint32_t q = excl[req_bucket[i]];
      const uint32_t pos = kstart[q] + atomicAdd(&kcur[q], 1u);
      Req e;
      e.rank = req_local[i];
      e.out = reqs[i].out;
      klist[pos] = e;
    }
  }
}

// ---------------------------------------------------------------------------
// (f) compaction pass
// ---------------------------------------------------------------------------
// cursor[b] (shared) = next survivor position of this CTA in bucket b for an
// active bucket (< 2^31), or kInactive + (elements seen so far) for an inactive
// one.  Every element takes one shared atomic on its bucket's cursor and the
// returned value decides whether it is stored: no divergent branch per
// survivor.  cap = min(survivor capacity, kInactive), so the single compare
// pos < cap rejects inactive buckets and keeps every store inside the buffer
// (a position past the capacity can only come from an input that changed
// between the passes; the cursor check at the end of the pass reports it).
// In heavy mode lanes of a warp that hit the same bucket share one atomic
// (match.any) and take consecutive positions.
template <class T, bool HEAVY>
__device__ __forceinline__ void compact_one(typename Traits<T>::K k, typename Traits<T>::K base,
                                            uint32_t shift, const uint32_t *lut /* lane's table */,
                                            uint32_t *cursor,
                                            typename Traits<T>::K *__restrict__ surv, uint32_t cap) {
  const uint32_t b = bucket_of_rep(k, base, shift, lut);
  uint32_t pos;
  if (HEAVY) {
    const uint32_t peers = __match_any_sync(0xffffffffu, b);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t p0 = 0;
    if (lane == leader) p0 = atomicAdd(&cursor[b], (uint32_t)__popc(peers));
    p0 = __shfl_sync(peers, p0, leader);
    pos = p0 + __popc(peers & ((1u << lane) - 1u));
  } else {
    pos = atomicAdd(&cursor[b], 1u);
  }
  // store without a branch: a predicated st.global
  st_global_if(surv + pos, k, pos < cap);
}

// Streams the CTA's tiles (and, in the owner CTA, the leftover vectors and
// the scalar head / tail) through onev(keys of one vector, in_tiles) and
// one(key) for the scalar head and tail.
template <class T, int UNROLL, class FV, class F>
__device__ __forceinline__ void compact_body(const T *__restrict__ x, uint64_t n, FV &&onev,
                                             F &&one) {
  using K = typename Traits<T>::K;
  using V = typename Traits<T>::Vec;
  constexpr int PV = Traits<T>::kPerVec;
  const Span<T> sp = split_span(x, n);
  const V *xv = reinterpret_cast<const V *>(x + sp.head);
  const uint64_t tile_v = (uint64_t)blockDim.x * UNROLL;
  const uint64_t ntiles = sp.nvec / tile_v;
  // The same tiles as the histogram pass (tile = blockIdx.x + q * gridDim.x),
  // visited last-to-first: the tail of the input read by that pass is the part
  // most likely to still be in L2.
  const uint64_t mine = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  for (uint64_t q = mine; q-- > 0;) {
    const uint64_t tile = blockIdx.x + q * gridDim.x;
    const V *p = xv + tile * tile_v + threadIdx.x;
    V v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) v[u] = ldg_stream(p + (uint64_t)u * blockDim.x);
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      K kk[PV];
      vec_keys<T>(v[u], kk);
      onev(kk, true);
    }
  }
  const uint32_t owner = (uint32_t)(ntiles % gridDim.x);
  if (blockIdx.x == owner) {
    for (uint64_t vi = ntiles * tile_v + threadIdx.x; vi < sp.nvec; vi += blockDim.x) {
      V vv = ldg_stream(xv + vi);
      K kk[PV];
      vec_keys<T>(vv, kk);
      onev(kk, false);
    }
    for (uint64_t e = threadIdx.x; e < sp.head; e += blockDim.x) one(Traits<T>::key(x[e]));
    for (uint64_t e = sp.tail0 + threadIdx.x; e < n; e += blockDim.x) one(Traits<T>::key(x[e]));
  }
}

// dynamic shared memory of k_compact: the table once per bank, then one
// cursor per bucket
__host__ __device__ constexpr size_t compact_smem_bytes(uint32_t nb_max) {
  return (size_t)(kRepWords + nb_max) * sizeof(uint32_t);
}

// Grid and tile assignment must equal k_hist's (same G, same owner of the
// leftovers), so that CTA c meets exactly the elements it counted.  CTA c
// takes its share of each slot's segment with one atomic on the slot's fill
// counter (CTAs take their shares in any order: the order of a segment's keys
// never matters) and leaves the share's end in its row of the per-CTA counts
// for the check at the end.  A call that overflows the survivor buffer stops
// here before touching the rows or the counters, so its re-run finds both as
// the plan left them.  In heavy mode (lanes of a warp often share a bucket)
// the cursor updates are warp-aggregated.
//
// A filtered variant was measured and not kept: the active buckets' bitmap
// held once per bank, so that only elements of active buckets take a cursor
// atomic, cut the shared-memory wavefronts per warp of 32 keys from 5.3 to
// 4.5 (atomics 4.0 -> 0.9), but the bitmap read, rank and predicated update
// doubled the instructions per key (18.5 -> 40), and the pass became issue
// bound: 2^27 keys took 194 us against 129 us.  A coarser gate -- per-bucket
// cursors kept, a bitmap of 4096 bucket groups (8 buckets each) held once per
// bank, the atomic and store only for keys of groups holding an active
// bucket (24 % of them at 1001 spread k's) -- was slower too at 2^28: 325 us
// branched (each key's returning atomic serialised behind its branch), 309 us
// predicated, against 225 us; the third dependent shared-memory access per
// key (table, gate, cursor) costs more than the conflicts it saves.
//
// Speculative compaction: when the histogram pass kept candidates (cand not
// null, the table's spec on) and every segment's bucket is a kept one, CTA c's
// candidates hold all of its elements of the segments' buckets, so it reads
// them in place of its tiles -- unless one of its warps' lists is incomplete
// (it reads its tiles).  The candidates lie in the survivor buffer above
// surv_half, so candidate mode also needs the survivors to end below it.
template <class T, int UNROLL>
__global__ void __launch_bounds__(1024, 1)
    k_compact(const T *__restrict__ x, uint64_t n, const LutHeader<typename Traits<T>::K> *hdr,
              const uint32_t *__restrict__ lut_g, const uint32_t *__restrict__ seg_bucket,
              const uint64_t *__restrict__ seg_off, const uint32_t *__restrict__ seg_size,
              uint32_t *__restrict__ rows, uint32_t *__restrict__ fill, uint32_t nb_max,
              typename Traits<T>::K *__restrict__ surv, uint64_t surv_cap, Ctrl *ctrl,
              const typename Traits<T>::K *__restrict__ cand,
              const uint32_t *__restrict__ cand_cnt, const uint32_t *__restrict__ cand_tab,
              uint64_t surv_half) {
  pdl_start();
  using K = typename Traits<T>::K;
  extern __shared__ uint4 smem_raw[];
  uint32_t *rep_lut = reinterpret_cast<uint32_t *>(smem_raw);  // one copy per bank
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t *lut = rep_lut + lane;  // this lane's copy
  uint32_t *cursor = rep_lut + kRepWords;  // per bucket
  __shared__ bool s_bad;
  __shared__ bool s_spec_miss;
  __shared__ uint32_t s_wcnt[kCandWarps];
  __shared__ uint32_t s_tab[kCandWarps * kCandChunksPerWarp];
  // nothing to compact when every slot is a single-key one (answered by the
  // finisher from its key alone), and then no cursor needs checking either
  if ((ctrl->status & (ST_FATAL | ST_OVERFLOW)) || ctrl->total_surv == 0) return;
  const LutHeader<K> h = *hdr;
  const uint32_t c = blockIdx.x;
  load_rep_table(rep_lut, lut_g);
  const uint32_t num_slots = ctrl->num_slots;
  const bool spec = cand != nullptr && h.spec != 0;
  for (uint32_t b = threadIdx.x; b < h.nb; b += blockDim.x) cursor[b] = kInactive;
  if (threadIdx.x == 0) {
    s_bad = false;
    s_spec_miss = false;
  }
  __syncthreads();
  // a warp whose list is incomplete (its table or the pool ran out) sends the
  // CTA to its tiles
  if (spec) {
    const uint32_t *tab = cand_tab + (uint64_t)c * kCandWarps * kCandChunksPerWarp;
    for (uint32_t i = threadIdx.x; i < kCandWarps * kCandChunksPerWarp; i += blockDim.x)
      s_tab[i] = tab[i];
    if (threadIdx.x < kCandWarps) {
      const uint32_t wc = cand_cnt[(uint64_t)c * kCandWarps + threadIdx.x];
      s_wcnt[threadIdx.x] = wc;
      const uint32_t nch = (wc + kCandChunk - 1) / kCandChunk;
      if (nch > kCandChunksPerWarp) {
        s_spec_miss = true;
      } else {
        for (uint32_t q = 0; q < nch; ++q)
          if (tab[threadIdx.x * kCandChunksPerWarp + q] >= h.cand_cap) s_spec_miss = true;
      }
    }
  }
  // flat slots (seg_size 0: a single-key bucket) are answered without survivors
  uint32_t *row = rows + (uint64_t)c * nb_max;
  for (uint32_t s = threadIdx.x; s < num_slots; s += blockDim.x) {
    const uint32_t sz = seg_size[s];
    if (sz == 0) continue;
    const uint32_t b = seg_bucket[s];
    const uint32_t cnt = row[b] & ~kMixed;
    const uint32_t pre = cnt ? atomicAdd(fill + s, cnt) : 0u;
    const uint32_t at = (uint32_t)(seg_off[s] + pre);
    cursor[b] = at;
    row[b] = at + cnt;
    if (spec && !in_spec(h, b)) s_spec_miss = true;
  }
  __syncthreads();
  const uint32_t cap = (uint32_t)(surv_cap < (uint64_t)kInactive ? surv_cap : kInactive);
  if (spec && !s_spec_miss && ctrl->total_surv <= surv_half) {
    // warp w reads the candidates of the histogram pass's warp w
    const uint32_t w = threadIdx.x >> 5;
    const uint32_t *wt = s_tab + w * kCandChunksPerWarp;
    const uint32_t cw = s_wcnt[w];
    const uint32_t cap_lo = (uint32_t)(surv_half < (uint64_t)cap ? surv_half : cap);
    for (uint32_t i = lane; i < cw; i += 32)
      compact_one<T, false>(cand[(uint64_t)wt[i / kCandChunk] * kCandChunk + i % kCandChunk],
                            h.base, h.shift, lut, cursor, surv, cap_lo);
    if (threadIdx.x == 0) atomicAdd(&ctrl->spec_ctas, 1u);
  } else if (h.heavy) {
    constexpr int PV = Traits<T>::kPerVec;
    compact_body<T, UNROLL>(
        x, n,
        [&](const K(&kk)[PV], bool in_tiles) {
#pragma unroll
          for (int e = 0; e < PV; ++e) {
            if (in_tiles)
              compact_one<T, true>(kk[e], h.base, h.shift, lut, cursor, surv, cap);
            else
              compact_one<T, false>(kk[e], h.base, h.shift, lut, cursor, surv, cap);
          }
        },
        [&](K k) { compact_one<T, false>(k, h.base, h.shift, lut, cursor, surv, cap); });
  } else {
    constexpr int PV = Traits<T>::kPerVec;
    compact_body<T, UNROLL>(
        x, n,
        [&](const K(&kk)[PV], bool) {
#pragma unroll
          for (int e = 0; e < PV; ++e)
            compact_one<T, false>(kk[e], h.base, h.shift, lut, cursor, surv, cap);
        },
        [&](K k) { compact_one<T, false>(k, h.base, h.shift, lut, cursor, surv, cap); });
  }
  __syncthreads();
  // every cursor must have reached the end of the CTA's share; anything else
  // means the input changed between the two passes
  for (uint32_t s = threadIdx.x; s < num_slots; s += blockDim.x) {
    if (seg_size[s] == 0) continue;
    const uint32_t b = seg_bucket[s];
    if (cursor[b] != row[b]) s_bad = true;
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_bad) atomicOr(&ctrl->status, ST_INTERNAL);
}

// ---------------------------------------------------------------------------
// (g) per-segment finish: shared-memory MSD radix select
// ---------------------------------------------------------------------------
// One CTA per segment (persistent over segments).  The segment's keys are
// read from the survivor buffer (L2-resident) three times: min/max, a
// histogram of up to 1024 bins over the top bits of (key - min), and a gather of only
// the bins that hold requested ranks into shared memory.  Each gathered bin is
// sorted (a warp bitonic network for bins of <= 32 keys, a CTA bitonic sort for
// larger ones) and every request reads its rank; needed bins beyond the
// shared-memory buffer take further rounds.  Segments with a needed bin larger
// than the sorting scratch are listed for a recursive re-selection.
constexpr int kFinBins = 1024;
constexpr int kFinBinBits = 10;
constexpr int kFinThreads = 256;
constexpr uint32_t kFlatBin = 0xFFFFFFFEu;  // gather offset of a needed bin holding one key

// shared memory of finish_slot with a gather buffer of bcap keys: five bin
// arrays, the buffer, a scratch half its size, per-bin key minima and maxima
template <class K>
__host__ __device__ constexpr size_t finish_smem_for(uint32_t bcap) {
  return 5 * kFinBins * sizeof(uint32_t) + (size_t)bcap * sizeof(K) * 3 / 2 +
         2 * kFinBins * sizeof(K);
}

// Position for a lane appending one item to a shared-memory list whose length
// is *counter, for the lanes of the warp that run this call together (want:
// whether this lane appends; the result is meaningful only then).  One atomic
// per warp: thousands of lanes incrementing one shared counter one by one
// serialise on it (a gather of 4096 keys that way took about 80 us).
__device__ __forceinline__ uint32_t warp_append(uint32_t *counter, bool want) {
  const uint32_t act = __activemask();
  const uint32_t m = __ballot_sync(act, want);
  if (m == 0) return 0;
  const uint32_t lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
  base = __shfl_sync(act, base, leader);
  return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

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

// The r-th smallest (0-based, r < S) of keys[0, S) in shared memory, by the
// whole CTA: MSD radix select, eight bits a round.  cnt: 256 shared words;
// sel: 2 shared words.  Every thread returns the key.
template <class K>
__device__ K cta_select_rank(const K *keys, uint32_t S, uint32_t r, uint32_t *cnt, uint32_t *sel) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  K prefix = 0, mask = 0;
  for (int sh = 8 * (int)sizeof(K) - 8; sh >= 0; sh -= 8) {
    for (uint32_t i = tid; i < 256; i += nt) cnt[i] = 0;
    __syncthreads();
    for (uint32_t i = tid; i < S; i += nt) {
      const K k = keys[i];
      if ((k & mask) == prefix) atomicAdd(&cnt[(uint32_t)(k >> sh) & 255u], 1u);
    }
    __syncthreads();
    if (tid < 32) {
      uint32_t c[8], sum = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        c[j] = cnt[8 * lane + j];
        sum += c[j];
      }
      const uint32_t incl = warp_incl_scan(sum);
      uint32_t acc = incl - sum;
      if (acc <= r && r < incl) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (r >= acc && r < acc + c[j]) {
            sel[0] = 8 * lane + j;
            sel[1] = r - acc;
          }
          acc += c[j];
        }
      }
    }
    __syncthreads();
    prefix |= (K)sel[0] << sh;
    mask |= (K)255 << sh;
    r = sel[1];
    __syncthreads();
  }
  return prefix;
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
__device__ __forceinline__ uint32_t bin_of_rank(const uint32_t *start, uint32_t nbins, uint32_t r) {
  uint32_t lo = 0, hi = nbins;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (start[mid] <= r)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Finishes one slot: its segment src[0 .. size) of survivor keys lies in the
// key range [lo, hi] (size 0: a flat slot whose single key is lo); the m
// requests rq[] hold local ranks and output positions.  Called by a whole CTA
// (a multiple of kFinThreads threads); smem is finish_smem_for<K>(bcap) bytes:
// 5 * kFinBins u32, the gather buffer (bcap keys), the scratch (bcap / 2
// keys), per-bin minima and maxima (kFinBins keys each).  Needed bins that
// together exceed the gather buffer are gathered, sorted and answered in up
// to kFinMaxRounds rounds; returns false when a single needed bin exceeds the
// scratch or more rounds would be needed: the slot needs a recursive
// re-selection.
// 16-byte vectors of survivor keys, read past L1 (the survivors may have been
// written earlier in the same kernel)
template <class K>
struct KeyVec;
template <>
struct KeyVec<uint32_t> {
  using V = uint4;
  static constexpr int kKeys = 4;
  static __device__ __forceinline__ V load(const V *p) { return __ldcg(p); }
  static __device__ __forceinline__ uint32_t key(const V &v, int e) {
    return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
  }
};
template <>
struct KeyVec<uint64_t> {
  using V = ulonglong2;
  static constexpr int kKeys = 2;
  static __device__ __forceinline__ V load(const V *p) { return __ldcg(p); }
  static __device__ __forceinline__ uint64_t key(const V &v, int e) { return e == 0 ? v.x : v.y; }
};
constexpr uint32_t kSpecBins = 24;  // bins kept either side of a request's predicted bin
constexpr uint32_t kFinMaxRounds = 4;  // gather rounds of a slot (more: recursive re-selection)
constexpr int kFinVecs = 2;  // vectors per thread and chunk in k_finish (63 registers)

template <class K, class OutT, int VECS = kFinVecs>
__device__ bool finish_slot(const K *__restrict__ src, uint32_t size, K lo, K hi,
                            const Req *__restrict__ rq, uint32_t m, uint32_t bcap, uint32_t *smem,
                            OutT *__restrict__ out) {
  uint32_t *hist = smem;
  uint32_t *start = hist + kFinBins;
  uint32_t *gofs = start + kFinBins;  // gather offset of a needed bin, else kNoSlot
  uint32_t *cur = gofs + kFinBins;
  uint32_t *small = cur + kFinBins;   // needed bins of 2..32 keys
  K *B = reinterpret_cast<K *>(small + kFinBins);  // gathered keys of the needed bins
  K *T = B + bcap;                                 // scratch for sorting a large bin (tcap keys)
  K *bmin = T + bcap / 2;                          // second attempt: per-bin key range
  K *bmax = bmin + kFinBins;
  constexpr int kMaxBig = 64;
  __shared__ K redk[33];
  __shared__ uint32_t red32[33];
  __shared__ uint32_t big[kMaxBig];
  __shared__ uint32_t s_nbig, s_nsmall, s_maxneed, s_v, s_spec, s_wlo, s_wsp, s_end;
  __shared__ uint32_t s_wn[32];  // speculative gather: keys kept per warp
  constexpr uint32_t PER = kFinBins / kFinThreads;  // bins per thread (at most)
  const uint32_t tcap = bcap / 2;                   // scratch T holds one bin of <= tcap keys
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t nwarps = blockDim.x >> 5;
  // each thread's first request, loaded ahead of the phases that read it
  Req my_rq;
  my_rq.rank = 0;
  my_rq.out = 0;
  if (tid < m) my_rq = rq[tid];
  auto req_at = [&](uint32_t j) -> Req { return j == tid ? my_rq : rq[j]; };
  if (size == 0) {  // flat slot: every rank in the bucket is its single key
    for (uint32_t j = tid; j < m; j += blockDim.x) out[req_at(j).out] = Traits<OutT>::value(lo);
    return true;
  }
  // The segment is read as aligned 16-byte vectors, VECS per thread and
  // chunk, every load of a chunk in flight before its keys are used (each
  // vector in flight costs about 15 registers once its keys' bodies are
  // scheduled).  The first and last vector may hold keys of the neighbouring
  // segments (an aligned 16-byte granule lies within one page, so reading it
  // is safe); those keys are masked out.
  using KV = KeyVec<K>;
  using VecT = typename KV::V;
  constexpr uint32_t KPV = KV::kKeys;
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(src) & ~uintptr_t(15);
  const uint32_t head = (uint32_t)((reinterpret_cast<uintptr_t>(src) - a0) / sizeof(K));
  const VecT *vsrc = reinterpret_cast<const VecT *>(a0);
  const uint32_t nvec = (uint32_t)(((uint64_t)head + size + KPV - 1) / KPV);
  const uint32_t chunk = VECS * blockDim.x;
  auto each_key = [&](auto &&fn) {
    for (uint32_t c0 = 0; c0 < nvec; c0 += chunk) {
      VecT tv[VECS];
#pragma unroll
      for (int u = 0; u < VECS; ++u) {
        const uint32_t v = c0 + u * blockDim.x + tid;
        if (v < nvec) tv[u] = KV::load(vsrc + v);
      }
#pragma unroll
      for (int u = 0; u < VECS; ++u) {
        const uint32_t v = c0 + u * blockDim.x + tid;
        if (v < nvec) {
#pragma unroll
          for (uint32_t e = 0; e < KPV; ++e) {
            const uint32_t i = v * KPV + e;  // key index from the first vector's start
            if (i >= head && i - head < size) fn(KV::key(tv[u], (int)e));
          }
        }
      }
    }
  };
  // about four keys per bin
  uint32_t nbits = 8;
  while (nbits < (uint32_t)kFinBinBits && (4u << nbits) < size) ++nbits;
  const uint32_t nbins = 1u << nbits;

  // digits of (key - mn): first over the bucket's key range; if the needed
  // bins then hold too many keys, over the segment's actual min / max, with
  // each bin's key range tracked: a needed bin holding one distinct key is
  // answered from its range and not gathered
  K mn = lo, mx = hi;
  uint32_t V = 0, sh = 0;
  bool flat = false, fits = false, direct = false;
  for (int attempt = 0; attempt < 2 && !fits && !flat && !direct; ++attempt) {
    if (attempt == 1) {
      K a = KeyMax<K>::v, z = 0;
      each_key([&](K k) {
        a = k < a ? k : a;
        z = k > z ? k : z;
      });
      a = block_reduce(a, [](K p, K q) { return p < q ? p : q; }, redk);
      z = block_reduce(z, [](K p, K q) { return p > q ? p : q; }, redk);
      if (a == z) {
        flat = true;
        mn = a;
        break;
      }
      mn = a;
      mx = z;
    }
    const bool track = attempt == 1;
    const int bl = bitlen<K>(mx - mn);
    sh = bl > (int)nbits ? (uint32_t)(bl - (int)nbits) : 0u;
    for (uint32_t i = tid; i < nbins; i += blockDim.x) {
      hist[i] = 0;
      cur[i] = 0;
      bmin[i] = KeyMax<K>::v;
      bmax[i] = 0;
    }
    // Speculative gather (first attempt, a slot with one request): within a
    // bucket the keys are close to linear in their rank, so the request's bin
    // is predicted from its rank, and the counting pass keeps the keys of the
    // kSpecBins bins either side of it in T (one region per warp).  If the
    // request's bin lies in the window (and no region overflowed), the needed
    // bin is filled from T and the segment is not read a second time.
    const bool spec = attempt == 0 && m == 1;
    if (tid == 0) {
      if (spec) {
        const uint32_t span = min((uint32_t)((mx - mn) >> sh), nbins - 1u) + 1u;  // bins in use
        const float at = ((float)my_rq.rank + 0.5f) * ((float)span / (float)size);
        const uint32_t pb = at < (float)(span - 1) ? (uint32_t)at : span - 1u;
        s_wlo = pb > kSpecBins ? pb - kSpecBins : 0u;
        s_wsp = min(pb + kSpecBins, nbins - 1u) - s_wlo;
      }
      s_nbig = 0;
      s_nsmall = 0;
      s_maxneed = 0;
      s_spec = 0;
    }
    if (spec && tid < nwarps) s_wn[tid] = 0;
    __syncthreads();
    // keys lie in [mn, mx], so the digit is < nbins; the clamp keeps a
    // shared-memory index in range whatever the data
    const uint32_t wlo = spec ? s_wlo : 0u, wsp = spec ? s_wsp : 0u;
    const uint32_t wcap = tcap / nwarps;  // keys per warp region of T
    K *wreg = T + warp * wcap;
    auto count = [&](K k) {
      const uint32_t bb = min((uint32_t)((k - mn) >> sh), nbins - 1u);
      atomicAdd(&hist[bb], 1u);
      if (track) {
        atomic_min_key(&bmin[bb], k);
        atomic_max_key(&bmax[bb], k);
      }
      if (spec && bb - wlo <= wsp) {
        const uint32_t p = atomicAdd(&s_wn[warp], 1u);
        if (p < wcap) wreg[p] = k;
      }
    };
    each_key(count);
    __syncthreads();
    {
      uint32_t cc[PER], sum = 0;
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        const uint32_t bb = tid * PER + q;
        cc[q] = bb < nbins ? hist[bb] : 0u;
        sum += cc[q];
      }
      uint32_t tot;
      uint32_t run = block_incl_scan(sum, &tot, red32) - sum;
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        const uint32_t bb = tid * PER + q;
        if (bb < nbins) {
          start[bb] = run;
          // few requests: "not needed" until warp 0 marks the needed bins;
          // else the "needed" flag until the next scan
          gofs[bb] = m <= 32 ? kNoSlot : 0u;
        }
        run += cc[q];
      }
    }
    __syncthreads();
    if (sh == 0) {  // every bin is a single key: the ranks read their bins
      direct = true;
      break;
    }
    if (m <= 32) {
      // One warp finds the requests' bins, drops repeats (match.any) and
      // numbers the needed bins with a warp scan: no block-wide scan over
      // the bins.  The gather order of the bins does not matter.
      if (warp == 0) {
        const uint32_t bb = lane < m ? bin_of_rank(start, nbins, req_at(lane).rank) : kNoSlot;
        const uint32_t same = __match_any_sync(0xffffffffu, bb);
        const bool lead = bb != kNoSlot && (int)lane == __ffs(same) - 1;
        const bool one = lead && track && bmin[bb] == bmax[bb];
        const uint32_t c = lead && !one ? hist[bb] : 0u;
        const uint32_t incl = warp_incl_scan(c);
        if (lead) {
          gofs[bb] = one ? kFlatBin : incl - c;
          if (!one) {
            atomicMax(&s_maxneed, c);
            if (c > 32) {
              const uint32_t at = atomicAdd(&s_nbig, 1u);
              if (at < kMaxBig) big[at] = bb;
            } else if (c > 1) {
              small[atomicAdd(&s_nsmall, 1u)] = bb;
            }
          }
        }
        if (lane == 31) s_v = incl;
        // the speculative gather holds the needed bin, no region overflowed
        if (spec && lane == 0 && bb - wlo <= wsp) {
          bool fit = true;
          for (uint32_t w = 0; w < nwarps; ++w) fit = fit && s_wn[w] <= wcap;
          s_spec = fit ? 1u : 0u;
        }
      }
      __syncthreads();
      V = s_v;
      fits = V <= bcap && s_maxneed <= tcap;
      continue;
    }
    for (uint32_t j = tid; j < m; j += blockDim.x)
      gofs[bin_of_rank(start, nbins, req_at(j).rank)] = 1u;
    __syncthreads();
    {
      uint32_t cc[PER], sum = 0;
      bool one[PER];  // a needed bin of one distinct key (tracked attempt only)
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        const uint32_t bb = tid * PER + q;
        one[q] = track && bb < nbins && gofs[bb] && bmin[bb] == bmax[bb];
        cc[q] = (bb < nbins && gofs[bb] && !one[q]) ? hist[bb] : 0u;
        sum += cc[q];
      }
      uint32_t run = block_incl_scan(sum, &V, red32) - sum;
#pragma unroll
      for (uint32_t q = 0; q < PER; ++q) {
        const uint32_t bb = tid * PER + q;
        if (bb < nbins) {
          const bool need = gofs[bb] != 0u && !one[q];
          gofs[bb] = one[q] ? kFlatBin : (need ? run : kNoSlot);
          if (need) atomicMax(&s_maxneed, cc[q]);
          if (need && cc[q] > 32) {
            const uint32_t at = atomicAdd(&s_nbig, 1u);
            if (at < kMaxBig) big[at] = bb;
          } else if (need && cc[q] > 1) {
            small[atomicAdd(&s_nsmall, 1u)] = bb;
          }
        }
        run += cc[q];
      }
    }
    __syncthreads();
    fits = V <= bcap && s_maxneed <= tcap;
  }
  if (flat) {  // one distinct key: every rank is that key
    for (uint32_t j = tid; j < m; j += blockDim.x) out[req_at(j).out] = Traits<OutT>::value(mn);
    __syncthreads();
    return true;
  }
  if (direct) {  // bins of one key each (few distinct keys, many copies)
    for (uint32_t j = tid; j < m; j += blockDim.x) {
      const Req e = req_at(j);
      out[e.out] = Traits<OutT>::value(mn + (K)bin_of_rank(start, nbins, e.rank));
    }
    __syncthreads();
    return true;
  }
  // a needed bin that does not fit, or so many needed keys that the rounds
  // would read the segment more than kFinMaxRounds times: the caller
  // re-selects this slot on its keys
  if (s_maxneed > tcap || V > kFinMaxRounds * bcap) {
    __syncthreads();
    return false;
  }
  (void)fits;

  // ---- gather, sort and answer the needed bins in rounds of at most bcap
  // keys, in bin order (one round when they all fit; every further round
  // reads the segment again -- a slot whose ranks are all requested, as a
  // top-k's are, holds more keys than one round)
  const uint32_t nsmall = s_nsmall;
  const uint32_t nbig = s_nbig;
  uint32_t base = 0;
  do {
    uint32_t end = V;
    if (V - base > bcap) {
      // the round ends at the last needed bin that ends within bcap keys (the
      // first bin from base fits: no needed bin exceeds tcap < bcap)
      if (tid == 0) s_end = base;
      __syncthreads();
      for (uint32_t bb = tid; bb < nbins; bb += blockDim.x) {
        const uint32_t g = gofs[bb];
        if (g >= kFlatBin) continue;
        const uint32_t e = g + hist[bb];
        if (g >= base && e <= base + bcap) atomicMax(&s_end, e);
      }
      __syncthreads();
      end = s_end;
    }
    auto in_round = [&](uint32_t g) { return g >= base && g < end; };
    // gather this round's bins
    {
      auto put = [&](K k) {
        const uint32_t bb = min((uint32_t)((k - mn) >> sh), nbins - 1u);
        const uint32_t g = gofs[bb];
        if (in_round(g)) B[g - base + atomicAdd(&cur[bb], 1u)] = k;
      };
      if (s_spec) {
        const uint32_t wcap = tcap / nwarps;
        for (uint32_t w = 0; w < nwarps; ++w)
          for (uint32_t i = tid; i < s_wn[w]; i += blockDim.x) put(T[w * wcap + i]);
      } else {
        each_key(put);
      }
    }
    __syncthreads();

    // sort each needed bin: a warp per bin of 2..32 keys
    for (uint32_t q = warp; q < nsmall; q += nwarps) {
      const uint32_t bb = small[q];
      const uint32_t g = gofs[bb], c = hist[bb];
      if (!in_round(g)) continue;
      K v = lane < c ? B[g - base + lane] : KeyMax<K>::v;
      v = warp_bitonic32(v);
      if (lane < c) B[g - base + lane] = v;
    }
    // larger bins: the whole CTA, one at a time
    for (uint32_t q = 0; q < (nbig <= (uint32_t)kMaxBig ? nbig : nbins); ++q) {
      const uint32_t bb = nbig <= (uint32_t)kMaxBig ? big[q] : q;
      const uint32_t g = gofs[bb], c = hist[bb];
      if (!in_round(g) || c <= 32) continue;
      uint32_t P = 64;
      while (P < c) P <<= 1;
      __syncthreads();
      for (uint32_t i = tid; i < P; i += blockDim.x) T[i] = i < c ? B[g - base + i] : KeyMax<K>::v;
      __syncthreads();
      bitonic_sort_smem(T, P);
      for (uint32_t i = tid; i < c; i += blockDim.x) B[g - base + i] = T[i];
    }
    __syncthreads();

    // answer the requests whose bins this round holds (one-key bins: once)
    for (uint32_t j = tid; j < m; j += blockDim.x) {
      const Req e = req_at(j);
      const uint32_t bb = bin_of_rank(start, nbins, e.rank);
      const uint32_t g = gofs[bb];
      if (g == kFlatBin) {
        if (base == 0) out[e.out] = Traits<OutT>::value(bmin[bb]);
      } else if (in_round(g)) {
        out[e.out] = Traits<OutT>::value(B[g - base + (e.rank - start[bb])]);
      }
    }
    __syncthreads();
    base = end;
  } while (base < V);
  return true;
}

template <class K, class OutT>
__global__ void __launch_bounds__(kFinThreads)
    k_finish(const K *__restrict__ surv, Ctrl *ctrl, const uint64_t *__restrict__ seg_off,
             const uint32_t *__restrict__ seg_size, const K *__restrict__ seg_lo,
             const K *__restrict__ seg_hi, const uint32_t *__restrict__ kstart,
             const uint32_t *__restrict__ kcnt, const Req *__restrict__ klist,
             uint32_t *__restrict__ deferred, uint32_t bcap, OutT *__restrict__ out) {
  pdl_start();
  extern __shared__ uint4 smem_raw[];
  if (ctrl->status & (ST_FATAL | ST_OVERFLOW)) return;
  const uint32_t num_slots = ctrl->num_slots;
  for (uint32_t slot = blockIdx.x; slot < num_slots; slot += gridDim.x) {
    const bool done = finish_slot<K, OutT>(surv + seg_off[slot], seg_size[slot], seg_lo[slot],
                                           seg_hi[slot], klist + kstart[slot], kcnt[slot], bcap,
                                           reinterpret_cast<uint32_t *>(smem_raw), out);
    if (!done && threadIdx.x == 0) {
      const uint32_t d = atomicAdd(&ctrl->deferred_count, 1u);
      deferred[d] = slot;
      atomicOr(&ctrl->status, ST_DEFERRED);
    }
  }
}


}  // namespace ggks
