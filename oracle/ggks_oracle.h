/*
 * ggks_oracle.h -- CPU oracle for GGKS bucket multiselect / top-k select.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark use it, and only as the checker.
 *
 * What it restates (paths are relative to the reference project root):
 *   - keyConversion.cu:9-42            order-preserving float/double <-> uint keys
 *   - multiselectTimingFunctions.cu:41-95
 *                                      sort-and-choose multiselect, the
 *                                      reference's own oracle:
 *                                      out[i] = ascending[n - k_i]
 *   - multiselectTimingFunctions.cu:155-177
 *                                      sort-and-choose top-k: the K largest,
 *                                      descending
 *   - bucketMultiselect.cu:87-111, :129-205, :249-308, :414-508, :521-871
 *                                      the bucket multiselect algorithm itself
 *                                      (17 sampled pivots, 16 slopes, 8192
 *                                      buckets, k-bucket walk, compaction,
 *                                      sort of survivors, gather), run on the
 *                                      CPU so that its result can be checked
 *                                      against sort-and-choose.
 *
 * Ordering policy: every sort orders by the order-preserving key, so -0.0
 * sorts below +0.0 and NaNs sort by sign beyond the infinities.  The reference
 * compares with the native operator<, which leaves those cases unordered; for
 * all other inputs the two orders are identical.
 *
 * Parity unpinned: the reference ships no golden vectors for this path, and
 * its path (CUDA kernels and Thrust on the device, sort-and-choose included)
 * runs only on a GPU, so no output of the reference itself stands behind this
 * restatement.  It is checked instead against closed-form known-answer
 * vectors built from the reference's deterministic generators
 * (generateProblems.cu) and against an independent sort (numpy) in the tests.
 */
#ifndef GGKS_ORACLE_H_
#define GGKS_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (same values as the product's ggks_status) */
#define GGKS_ORACLE_OK 0
#define GGKS_ORACLE_INVALID_ARG 1
#define GGKS_ORACLE_OOM 2

/* keyConversion.cu:9-23 (preProcess) and :29-42 (postProcess) */
uint32_t ggks_oracle_key_f32(uint32_t bits);
uint64_t ggks_oracle_key_f64(uint64_t bits);
uint32_t ggks_oracle_unkey_f32(uint32_t key);
uint64_t ggks_oracle_unkey_f64(uint64_t key);

/* Sort-and-choose multiselect (multiselectTimingFunctions.cu:51-95).
 * k[i] is the k-th LARGEST, 1-based (bucketMultiselect.cu:845-846);
 * out[i] = ascending[n - k[i]].  threads <= 1 runs single-threaded. */
int ggks_oracle_multiselect_f32(const float *vec, uint64_t n, const uint32_t *k,
                                uint32_t num_k, float *out, int threads);
int ggks_oracle_multiselect_f64(const double *vec, uint64_t n, const uint32_t *k,
                                uint32_t num_k, double *out, int threads);
int ggks_oracle_multiselect_u32(const uint32_t *vec, uint64_t n, const uint32_t *k,
                                uint32_t num_k, uint32_t *out, int threads);

/* Sort-and-choose top-k (multiselectTimingFunctions.cu:155-177): the K
 * largest values in descending order. */
int ggks_oracle_topk_f32(const float *vec, uint64_t n, uint32_t kk, float *out, int threads);
int ggks_oracle_topk_f64(const double *vec, uint64_t n, uint32_t kk, double *out, int threads);
int ggks_oracle_topk_u32(const uint32_t *vec, uint64_t n, uint32_t kk, uint32_t *out, int threads);

/* The reference's bucket multiselect algorithm run on the CPU
 * (bucketMultiselect.cu:521-871), with a seeded sample in place of the
 * time-seeded one (bucketMultiselect.cu:377-389).  Same k convention. */
int ggks_oracle_bucket_multiselect_f32(const float *vec, uint32_t n, const uint32_t *k,
                                       uint32_t num_k, float *out, uint64_t seed);
int ggks_oracle_bucket_multiselect_f64(const double *vec, uint32_t n, const uint32_t *k,
                                       uint32_t num_k, double *out, uint64_t seed);
int ggks_oracle_bucket_multiselect_u32(const uint32_t *vec, uint32_t n, const uint32_t *k,
                                       uint32_t num_k, uint32_t *out, uint64_t seed);

/* Sort-and-choose multiselect on one thread with the C++ standard library's
 * std::sort of the keys (ggks_oracle_stdsort.cpp): the benchmark's CPU
 * baseline.  Same k convention and output as ggks_oracle_multiselect_*. */
int ggks_oracle_multiselect_stdsort_f32(const float *vec, uint64_t n, const uint32_t *k,
                                        uint32_t num_k, float *out);
int ggks_oracle_multiselect_stdsort_f64(const double *vec, uint64_t n, const uint32_t *k,
                                        uint32_t num_k, double *out);
int ggks_oracle_multiselect_stdsort_u32(const uint32_t *vec, uint64_t n, const uint32_t *k,
                                        uint32_t num_k, uint32_t *out);

/* Ascending sort of keys (LSD radix); exposed for tests of the oracle. */
int ggks_oracle_sort_keys_u32(uint32_t *keys, uint64_t n, int threads);
int ggks_oracle_sort_keys_u64(uint64_t *keys, uint64_t n, int threads);

#ifdef __cplusplus
}
#endif
#endif
