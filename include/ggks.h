/*
 * ggks.h -- C ABI of the GB300 (sm_103a) GGKS bucket multiselect / top-k.
 *
 * Plain C types only (pointers, sizes, status codes): any FFI can bind it.
 * Paths in the citations are relative to the reference project
 * (uysalere/ggks-multiSelect).
 *
 * Conventions shared by every entry point
 *   - k is the k-th LARGEST element, 1-based, exactly as the reference wrapper
 *     takes it (bucketMultiselect.cu:842-846): out[i] = ascending[n - k[i]].
 *   - Results are bit-exact order statistics under the order-preserving key
 *     order (keyConversion.cu:9-23): -0.0 < +0.0, NaNs beyond the infinities
 *     by sign.  For every other input this is the numeric order.
 *   - The input vector is never modified.  The k array is read, not written.
 *   - Outputs are written in the caller's k order (bucketMultiselect.cu:816-818)
 *     or, for top-k, in descending order (multiselectTimingFunctions.cu:156-177).
 *   - Every call returns a ggks_status; nothing is reported through the
 *     return value of a selection (the reference returns 1 for both success
 *     and failure, bucketMultiselect.cu:30-32, :832).
 *   - Calls are synchronous with respect to the host outputs: when a call
 *     returns GGKS_OK, host outputs are filled.  Work is issued on the
 *     context's stream (or opts->stream).
 *   - n must satisfy 1 <= n <= GGKS_MAX_N; device vectors must be aligned to
 *     their element size.
 */
#ifndef GGKS_H_
#define GGKS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GGKS_VERSION 10000 /* 1.0.0 */
#define GGKS_MAX_N 4294967295ull

typedef enum ggks_status {
  GGKS_OK = 0,
  GGKS_INVALID_ARG = 1,   /* null pointer, n or num_k out of range, k not in [1, n] */
  GGKS_OOM = 2,           /* device or pinned host allocation failed */
  GGKS_CUDA_ERROR = 3,    /* a CUDA runtime call or kernel launch failed */
  GGKS_TIMEOUT = 4,       /* a bounded device-side wait gave up */
  GGKS_INTERNAL = 5,      /* a device-side consistency check failed */
  GGKS_NO_DEVICE = 6,     /* no usable CUDA device */
  GGKS_UNSUPPORTED = 7
} ggks_status;

typedef struct ggks_context ggks_context;

/* Options shared by the selection entry points.  Pass NULL for defaults. */
typedef struct ggks_opts {
  ggks_context *ctx; /* NULL: the calling thread's current device's default context */
  void *stream;      /* cudaStream_t; NULL: the context's own stream */
  uint32_t flags;    /* GGKS_FLAG_* */
  uint32_t reserved;
} ggks_opts;

/* opts->flags: the output pointer is device memory (no device-to-host copy). */
#define GGKS_FLAG_OUT_DEVICE 1u
/* opts->flags for ggks_topk_*: run the histogram / compaction pipeline even
 * where the threshold path (K <= 4096, n > 65536, 64 K <= n) or the
 * one-launch small-vector path applies; the results are the same. */
#define GGKS_FLAG_TOPK_PIPELINE 4u
/* opts->flags for ggks_multiselect_* / ggks_topk_*: run the pipeline even
 * where the one-launch small-vector path applies (a device vector of at most
 * 2^20 elements -- 2^18 for a top-k -- and at most 1024 k's); the results are
 * the same. */
#define GGKS_FLAG_NO_SMALL 8u

/* ------------------------------------------------------------------------ */
/* Multiselect                                                               */
/* ------------------------------------------------------------------------ */

/* Replaces BucketMultiselect::bucketMultiselectWrapper<T>
 * (bucketMultiselect.cu:837-871): d_vec is a device vector of n elements,
 * h_k a host array of num_k k's (k-th largest), h_out a host array of num_k
 * results in the caller's k order.  The reference's blocks/threads launch
 * arguments have no counterpart: launch shapes are chosen per problem. */
int ggks_multiselect_f32(const float *d_vec, uint64_t n, const uint32_t *h_k, uint32_t num_k,
                         float *h_out, const ggks_opts *opts);
int ggks_multiselect_f64(const double *d_vec, uint64_t n, const uint32_t *h_k, uint32_t num_k,
                         double *h_out, const ggks_opts *opts);
int ggks_multiselect_u32(const uint32_t *d_vec, uint64_t n, const uint32_t *h_k,
                         uint32_t num_k, uint32_t *h_out, const ggks_opts *opts);

/* Replaces the timing adapter's host-vector form timeBucketMultiselect<T>
 * (multiselectTimingFunctions.cu:100-122): the vector is in host memory and is
 * copied to the device inside the call (overlapped with the first pass). */
int ggks_multiselect_host_f32(const float *h_vec, uint64_t n, const uint32_t *h_k,
                              uint32_t num_k, float *h_out, const ggks_opts *opts);
int ggks_multiselect_host_f64(const double *h_vec, uint64_t n, const uint32_t *h_k,
                              uint32_t num_k, double *h_out, const ggks_opts *opts);
int ggks_multiselect_host_u32(const uint32_t *h_vec, uint64_t n, const uint32_t *h_k,
                              uint32_t num_k, uint32_t *h_out, const ggks_opts *opts);

/* ------------------------------------------------------------------------ */
/* Top-k                                                                     */
/* ------------------------------------------------------------------------ */

/* Replaces timeBucketTopkselect<T> (multiselectTimingFunctions.cu:205-231),
 * which runs the bucket multiselect with k = 1..K, and the top-k wrapper
 * signature randomizedTopkSelectWrapper<T> (randomizedTopkSelect.cu:210-213):
 * h_out receives the K largest values of d_vec in descending order. */
int ggks_topk_f32(const float *d_vec, uint64_t n, uint32_t K, float *h_out,
                  const ggks_opts *opts);
int ggks_topk_f64(const double *d_vec, uint64_t n, uint32_t K, double *h_out,
                  const ggks_opts *opts);
int ggks_topk_u32(const uint32_t *d_vec, uint64_t n, uint32_t K, uint32_t *h_out,
                  const ggks_opts *opts);

/* Host-vector form of the above (multiselectTimingFunctions.cu:205-231 takes
 * h_vec). */
int ggks_topk_host_f32(const float *h_vec, uint64_t n, uint32_t K, float *h_out,
                       const ggks_opts *opts);
int ggks_topk_host_f64(const double *h_vec, uint64_t n, uint32_t K, double *h_out,
                       const ggks_opts *opts);
int ggks_topk_host_u32(const uint32_t *h_vec, uint64_t n, uint32_t K, uint32_t *h_out,
                       const ggks_opts *opts);

/* ------------------------------------------------------------------------ */
/* Single-k select                                                           */
/* ------------------------------------------------------------------------ */

/* Replaces BucketSelect::bucketSelectWrapper<T> (bucketSelect.cu:453-471) and
 * RandomizedBucketSelect::randomizedBucketSelectWrapper<T>
 * (randomizedBucketSelect.cu:861-881), which return the K-th largest element
 * of a device vector: one output, *out = the k-th largest (1-based), host
 * memory (device memory with GGKS_FLAG_OUT_DEVICE).  A multiselect with one k. */
int ggks_select_f32(const float *d_vec, uint64_t n, uint32_t k, float *out, const ggks_opts *opts);
int ggks_select_f64(const double *d_vec, uint64_t n, uint32_t k, double *out,
                    const ggks_opts *opts);
int ggks_select_u32(const uint32_t *d_vec, uint64_t n, uint32_t k, uint32_t *out,
                    const ggks_opts *opts);

/* ------------------------------------------------------------------------ */
/* Multiselect without allocation                                            */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference.  A float32 multiselect for callers that
 * may not allocate memory when they select: an engine or framework whose
 * device memory all belongs to its own allocator, which budgets every byte (an
 * allocation behind its back can exhaust the device or break its accounting),
 * and latency-bound loops where an allocation would stall on the driver.  It
 * calls no cudaMalloc, cudaFree, cudaHostAlloc or other allocating routine; its
 * scratch is one fixed device array (about 11 MB) that every GPU loading this
 * library holds until the process exits.
 *   d_vec: device vector of n floats; d_k: device array of num_k k's (k-th
 *   largest, 1-based); d_out: device array of num_k results in k order;
 *   stream: a cudaStream_t (NULL: the legacy default stream).  The call
 *   returns when the results are in d_out.
 * Limits: 1 <= n <= GGKS_NOALLOC_MAX_N and 1 <= num_k <= GGKS_NOALLOC_MAX_K,
 * else GGKS_INVALID_ARG (also for a k outside [1, n]); an input whose buckets
 * would need a recursive re-selection (heavy, nearly equal duplicates) returns
 * GGKS_UNSUPPORTED (d_out may then hold partial results; nothing past its
 * num_k entries is written).  The first call on a device looks up the
 * scratch's device address and sets the kernels' shared-memory limits there;
 * make it before any stream capture.  All calls share the scratch, which
 * keeps the last call's contents (each call clears what must start at zero):
 * calls that overlap on the GPU race and must be serialised by the caller. */
#define GGKS_NOALLOC_MAX_N (1ull << 21)
#define GGKS_NOALLOC_MAX_K 2048u
int ggks_multiselect_noalloc_f32(const float *d_vec, uint64_t n, const uint32_t *d_k,
                                 uint32_t num_k, float *d_out, void *stream);

/* ------------------------------------------------------------------------ */
/* Batched selection                                                         */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference, which selects one vector per call
 * (bucketMultiselectWrapper, bucketMultiselect.cu:837-871) and compares
 * algorithms per size in an offline loop (analyzeMultiselect.cu:209-274).
 * Selects many independent vectors of uneven lengths, each with its own k
 * list, in one persistent kernel launch driven by a (problem, tile) work
 * queue.  Results are bit-exact and equal, output for output, to separate
 * ggks_multiselect_* calls.
 *   d_vecs[p]: device vector of n[p] elements (p < num_problems), aligned to
 *   the element size.  k_offsets: num_problems + 1 non-decreasing entries,
 *   k_offsets[0] = 0; the outputs of problem p are
 *   out[k_offsets[p] .. k_offsets[p + 1]) and out[j] is the h_k[j]-th largest
 *   (1-based) of its problem's vector.  A problem without outputs is skipped
 *   (its vector may be NULL, n 0).  out: host array of k_offsets[num_problems]
 *   values, or device memory with GGKS_FLAG_OUT_DEVICE.
 * opts->flags & GGKS_FLAG_AUTOTUNE: the first call for a batch shape (element
 * type, total elements, problems, outputs per problem, each rounded to a power
 * of two) times every candidate bucket budget / tile size and keeps the
 * fastest for later calls of that shape on the context. */
#define GGKS_FLAG_AUTOTUNE 2u
int ggks_multiselect_batch_f32(const float *const *d_vecs, const uint64_t *n,
                               uint32_t num_problems, const uint32_t *k_offsets,
                               const uint32_t *h_k, float *out, const ggks_opts *opts);
int ggks_multiselect_batch_f64(const double *const *d_vecs, const uint64_t *n,
                               uint32_t num_problems, const uint32_t *k_offsets,
                               const uint32_t *h_k, double *out, const ggks_opts *opts);
int ggks_multiselect_batch_u32(const uint32_t *const *d_vecs, const uint64_t *n,
                               uint32_t num_problems, const uint32_t *k_offsets,
                               const uint32_t *h_k, uint32_t *out, const ggks_opts *opts);

/* Batched top-k (no reference counterpart; per vector it matches
 * ggks_topk_*): problem p's K[p] largest values, descending, go to
 * out[off_p .. off_p + K[p]) with off_p = K[0] + ... + K[p - 1].  K[p] = 0
 * skips the problem; K[p] <= n[p]. */
int ggks_topk_batch_f32(const float *const *d_vecs, const uint64_t *n, uint32_t num_problems,
                        const uint32_t *K, float *out, const ggks_opts *opts);
int ggks_topk_batch_f64(const double *const *d_vecs, const uint64_t *n, uint32_t num_problems,
                        const uint32_t *K, double *out, const ggks_opts *opts);
int ggks_topk_batch_u32(const uint32_t *const *d_vecs, const uint64_t *n,
                        uint32_t num_problems, const uint32_t *K, uint32_t *out,
                        const ggks_opts *opts);

/* The bucket divisor (about n / div buckets per problem) and tile size
 * (elements per work item) used by the context's last batched call. */
int ggks_batch_last_tuning(ggks_context *ctx, uint32_t *div, uint32_t *tile);
/* Pin the divisor (16 <= div <= 2^24) and tile size (>= 64 elements, rounded
 * down to a multiple of 64) for every later batched call on the context,
 * instead of the autotuner's choice; div = 0 unpins. */
int ggks_batch_set_tuning(ggks_context *ctx, uint32_t div, uint32_t tile);

/* passes of a single-vector call and phases of a batched launch, as counted
 * by the statistics below */
#define GGKS_NUM_PASSES 6
#define GGKS_NUM_BATCH_PHASES 5

/* ------------------------------------------------------------------------ */
/* Serving loop                                                              */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference (a benchmark harness that runs one
 * selection at a time, compareMultiselect.cu:72-187).  A server accepts
 * multiselect and top-k requests of mixed sizes and element types at any
 * time, from any thread, and coalesces them into batched launches:
 *   - admission: requests are taken in arrival order while the device bytes
 *     of the admitted ones (uploaded vector + bucket-state estimate) stay
 *     within the admission budget, min(hbm_cap_bytes, the device's free
 *     memory - hbm_reserve_bytes + the bytes already admitted); a request
 *     that does not fit waits for earlier ones to finish (GGKS_OOM if nothing
 *     is admitted and it still does not fit).  A host vector is copied to the
 *     device then, on a copy stream that overlaps the running batches;
 *   - execution: `lanes` executors (each with its own stream and workspace)
 *     each take the requests whose data is on the device (at most max_batch,
 *     0 = no limit) and run them as one persistent launch per element type
 *     present.  Batches of different lanes are planned, uploaded and run on
 *     the device at the same time; their persistent grids share the device's
 *     co-resident CTAs, so that every grid is resident at once.  Requests
 *     arriving meanwhile join the next batch.
 * Each result equals the result of the single-vector entry point on the same
 * vector and k's, bit for bit. */
typedef struct ggks_server ggks_server;

typedef struct ggks_server_config {
  int device;
  uint32_t max_batch;         /* requests per batch at most; 0 = no limit */
  uint64_t hbm_cap_bytes;     /* admission cap on the admitted requests' device bytes */
  uint64_t hbm_reserve_bytes; /* device memory admission leaves free; 0 = 1 GiB */
  uint32_t lanes;             /* batches in flight at once, 1..8; 0 = 2 */
  uint32_t reserved;
} ggks_server_config;

#define GGKS_DTYPE_F32 0
#define GGKS_DTYPE_F64 1
#define GGKS_DTYPE_U32 2
/* ggks_request.flags */
#define GGKS_REQ_TOPK 1u        /* the num_k largest, descending (k is ignored) */
#define GGKS_REQ_HOST_VECTOR 2u /* vec is host memory (else device memory) */

typedef struct ggks_request {
  int32_t dtype;      /* GGKS_DTYPE_* */
  uint32_t flags;     /* GGKS_REQ_* */
  const void *vec;    /* n elements; must stay valid until ggks_server_wait returns */
  uint64_t n;
  const uint32_t *k;  /* num_k k's (k-th largest, 1-based); copied by submit */
  uint32_t num_k;     /* outputs; for top-k, K */
  uint32_t reserved;
} ggks_request;

typedef struct ggks_server_stats {
  uint64_t submitted, completed;
  uint64_t batches;          /* batches formed */
  uint64_t batched_requests; /* requests over all batches */
  uint64_t max_batch_seen;
  uint64_t launches;         /* batched selections run (per batch: one for its float32 and
                                uint32 requests together, one for its float64 ones) */
  uint64_t uploads, upload_bytes; /* host vectors copied at admission */
  uint64_t peak_bytes;       /* largest admitted device bytes */
  uint64_t in_flight_bytes;  /* admitted device bytes now */
  uint64_t concurrent_launches; /* batched launches queued on the device behind another
                                   lane's kernel still in flight */
  uint64_t hbm_waits;        /* admissions held back by the device's free memory */
  uint64_t admit_budget_bytes; /* the admission budget at the last admission */
  uint64_t single_calls;     /* lone requests of a type run on the single-vector pipeline */
  uint64_t recursions;       /* oversized segments re-selected, all lanes */
  double batch_phase_ms[GGKS_NUM_BATCH_PHASES]; /* device time per batch phase, all lanes */
  double kernel_ms;          /* device time of the batched launches, all lanes */
  double group_ms;           /* lane wall time per element-type group (plan, run, results) */
  double device_busy_ms;     /* union of the batched launches' device intervals, all lanes */
  double device_span_ms;     /* first batched launch's start to the last one's end */
} ggks_server_stats;

int ggks_server_create(const ggks_server_config *cfg, ggks_server **out);
/* Finishes every submitted request, then stops the server's threads. */
int ggks_server_destroy(ggks_server *srv);
/* out: host buffer of num_k values, written before ggks_server_wait returns.
 * GGKS_OOM: the request alone exceeds the cap. */
int ggks_server_submit(ggks_server *srv, const ggks_request *req, void *out, uint64_t *ticket);
/* Blocks until the request is done; returns its status; *latency_ms (may be
 * NULL): submit to completion.  Each ticket is waited for once. */
int ggks_server_wait(ggks_server *srv, uint64_t ticket, double *latency_ms);
int ggks_server_get_stats(ggks_server *srv, ggks_server_stats *out);
/* Pin the batched path's divisor / tile size (ggks_batch_set_tuning). */
int ggks_server_set_tuning(ggks_server *srv, uint32_t div, uint32_t tile);

/* ------------------------------------------------------------------------ */
/* Contexts, statistics, utilities                                           */
/* ------------------------------------------------------------------------ */

/* A context owns a device, a stream, a device workspace and pinned staging.
 * Calls on one context are serialised by the context; use one context per
 * host thread for concurrency.  (The reference keeps its timer in namespace
 * globals, bucketMultiselect.cu:49-50, and is not thread-safe.) */
int ggks_context_create(int device, ggks_context **out);
int ggks_context_destroy(ggks_context *ctx);

/* Per-pass statistics of a context, accumulated since the last reset
 * (GGKS_NUM_PASSES and GGKS_NUM_BATCH_PHASES are defined with the batched
 * entry points). */
typedef struct ggks_stats {
  uint64_t calls;                     /* selection calls completed */
  uint64_t launches;                  /* kernels launched by this library */
  uint64_t pass_launches[GGKS_NUM_PASSES];
  double pass_ms[GGKS_NUM_PASSES];    /* device time per pass (profiling on) */
  uint64_t bytes_in;                  /* algorithmic input bytes (n * sizeof(T)) */
  uint64_t survivors;                 /* elements compacted into active buckets */
  uint64_t retries;                   /* survivor-buffer regrowth re-runs */
  uint64_t recursions;                /* oversized segments re-selected */
  uint64_t host_ingested;             /* host vectors read in place by the first pass */
  uint64_t host_staged;               /* host vectors copied to the device first */
  uint64_t batch_calls;               /* batched calls completed */
  uint64_t batch_problems;            /* problems selected by batched calls */
  double batch_phase_ms[GGKS_NUM_BATCH_PHASES]; /* device time per batch phase */
  uint64_t batch_grid;                /* CTAs of the last batched launch */
  uint64_t spec_calls;                /* calls whose first pass also kept the predicted
                                         candidates (top-k, few clustered k's) */
  uint64_t spec_ctas;                 /* compaction CTAs that read those candidates
                                         in place of their share of the vector */
  uint64_t topk_threshold_calls;      /* top-k calls answered by the threshold path */
  uint64_t topk_misses;               /* threshold attempts that fell back to the pipeline */
  uint64_t batch_spec_tiles;          /* batched compaction tiles that read their candidates
                                         in place of their elements */
  uint64_t small_calls;               /* calls answered by the one-launch small-vector path */
  uint64_t small_misses;              /* small-vector attempts left to the pipeline */
} ggks_stats;

/* phase indices of ggks_stats.batch_phase_ms (one persistent launch; each
 * phase is timed from the grid barrier before it to the one after it) */
#define GGKS_BATCH_TABLE 0    /* samples + splitter table of every problem */
#define GGKS_BATCH_HIST 1     /* histogram rows of every (problem, tile) */
#define GGKS_BATCH_PLAN 2     /* per-problem bucket prefix, k -> bucket, slots */
#define GGKS_BATCH_COMPACT 3  /* compaction of every (problem, tile) */
#define GGKS_BATCH_FINISH 4   /* every slot's in-shared-memory selection */

/* pass indices of ggks_stats.pass_* */
#define GGKS_PASS_SAMPLE 0   /* sample + splitter table build */
#define GGKS_PASS_HIST 1     /* bucket histogram over the input */
#define GGKS_PASS_SCAN 2     /* bucket totals: column sums of the per-CTA rows */
#define GGKS_PASS_PLAN 3     /* bucket prefix, k -> bucket marker, slot and request
                                layout */
#define GGKS_PASS_COMPACT 4  /* compaction of active-bucket elements */
#define GGKS_PASS_FINISH 5   /* per-segment in-shared-memory selection */

int ggks_context_get_stats(ggks_context *ctx, ggks_stats *out);
int ggks_context_reset_stats(ggks_context *ctx);
/* on != 0: time every pass with CUDA events on the context's stream */
int ggks_context_set_profiling(ggks_context *ctx, int on);
/* value for ggks_context_set_profiling: time only the passes whose bits
 * (1 << GGKS_PASS_*) are set in mask */
#define GGKS_PROFILE_PASSES(mask) ((int)(0x80000000u | (uint32_t)(mask)))
const char *ggks_status_string(int status);
int ggks_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GGKS_H_ */
