/*
 * ggks_oracle.c -- CPU oracle for GGKS bucket multiselect / top-k select.
 *
 * TEST INFRASTRUCTURE ONLY (see ggks_oracle.h).  Plain C11 + pthreads; builds
 * with gcc on x86_64 and aarch64 alike (no intrinsics, no assumptions about
 * the signedness of char).
 */
#define _GNU_SOURCE
#include "ggks_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Order-preserving keys: keyConversion.cu:9-23 (preProcess) flips the sign  */
/* bit of non-negative floats and all bits of negative ones, so that the     */
/* unsigned order of the keys is the numeric order of the values.            */
/* keyConversion.cu:29-42 (postProcess) undoes it.                           */
/* ------------------------------------------------------------------------ */
uint32_t ggks_oracle_key_f32(uint32_t bits) {
  uint32_t mask = (bits & 0x80000000u) ? 0xffffffffu : 0x80000000u;
  return bits ^ mask;
}
uint64_t ggks_oracle_key_f64(uint64_t bits) {
  uint64_t mask = (bits & 0x8000000000000000ull) ? 0xffffffffffffffffull
                                                  : 0x8000000000000000ull;
  return bits ^ mask;
}
uint32_t ggks_oracle_unkey_f32(uint32_t key) {
  uint32_t mask = (key & 0x80000000u) ? 0x80000000u : 0xffffffffu;
  return key ^ mask;
}
uint64_t ggks_oracle_unkey_f64(uint64_t key) {
  uint64_t mask = (key & 0x8000000000000000ull) ? 0x8000000000000000ull
                                                 : 0xffffffffffffffffull;
  return key ^ mask;
}

/* ------------------------------------------------------------------------ */
/* Parallel LSD radix sort of unsigned keys (8-bit digits).  Each pass: every */
/* thread counts its contiguous chunk, the counts are prefix-summed in        */
/* (digit, thread) order, and every thread scatters its chunk stably.  A pass */
/* whose digit is the same for every key is skipped.                          */
/* ------------------------------------------------------------------------ */
#define RADIX_BITS 8
#define RADIX_SIZE (1u << RADIX_BITS)
#define MAX_THREADS 256

typedef struct {
  void *src, *dst;
  uint64_t n;
  int nthreads, keybytes;
  uint64_t (*hist)[RADIX_SIZE]; /* [thread][digit] */
  pthread_barrier_t *bar;
  int *skip;
} sort_shared_t;

typedef struct {
  sort_shared_t *sh;
  int tid;
} sort_arg_t;

static inline uint64_t load_key(const void *p, uint64_t i, int keybytes) {
  return keybytes == 4 ? ((const uint32_t *)p)[i] : ((const uint64_t *)p)[i];
}
static inline void store_key(void *p, uint64_t i, uint64_t v, int keybytes) {
  if (keybytes == 4)
    ((uint32_t *)p)[i] = (uint32_t)v;
  else
    ((uint64_t *)p)[i] = v;
}

static void *radix_worker(void *varg) {
  sort_arg_t *a = (sort_arg_t *)varg;
  sort_shared_t *sh = a->sh;
  const int T = sh->nthreads, t = a->tid, kb = sh->keybytes;
  const uint64_t n = sh->n;
  const uint64_t lo = n * (uint64_t)t / (uint64_t)T;
  const uint64_t hi = n * (uint64_t)(t + 1) / (uint64_t)T;
  const int passes = kb * 8 / RADIX_BITS;
  void *src = sh->src, *dst = sh->dst;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = pass * RADIX_BITS;
    uint64_t *h = sh->hist[t];
    memset(h, 0, sizeof(uint64_t) * RADIX_SIZE);
    if (kb == 4) {
      const uint32_t *s = (const uint32_t *)src;
      for (uint64_t i = lo; i < hi; ++i) h[(s[i] >> shift) & (RADIX_SIZE - 1)]++;
    } else {
      const uint64_t *s = (const uint64_t *)src;
      for (uint64_t i = lo; i < hi; ++i) h[(s[i] >> shift) & (RADIX_SIZE - 1)]++;
    }
    pthread_barrier_wait(sh->bar);
    if (t == 0) {
      /* digit-major exclusive prefix; detect a constant digit */
      uint64_t run = 0;
      int nonzero = 0;
      for (uint32_t d = 0; d < RADIX_SIZE; ++d) {
        uint64_t tot = 0;
        for (int u = 0; u < T; ++u) tot += sh->hist[u][d];
        if (tot) nonzero++;
        for (int u = 0; u < T; ++u) {
          uint64_t c = sh->hist[u][d];
          sh->hist[u][d] = run;
          run += c;
        }
      }
      *sh->skip = (nonzero <= 1);
    }
    pthread_barrier_wait(sh->bar);
    if (!*sh->skip) {
      uint64_t *off = sh->hist[t];
      for (uint64_t i = lo; i < hi; ++i) {
        uint64_t v = load_key(src, i, kb);
        store_key(dst, off[(v >> shift) & (RADIX_SIZE - 1)]++, v, kb);
      }
      void *tmp = src;
      src = dst;
      dst = tmp;
    }
    pthread_barrier_wait(sh->bar);
  }
  if (t == 0) sh->src = src; /* where the sorted keys ended up */
  return NULL;
}

static int radix_sort(void *keys, uint64_t n, int keybytes, int threads) {
  if (n <= 1) return GGKS_ORACLE_OK;
  if (threads < 1) threads = 1;
  if (threads > MAX_THREADS) threads = MAX_THREADS;
  if ((uint64_t)threads > n) threads = (int)n;
  void *tmp = malloc((size_t)n * (size_t)keybytes);
  uint64_t(*hist)[RADIX_SIZE] = calloc((size_t)threads, sizeof(*hist));
  if (!tmp || !hist) {
    free(tmp);
    free(hist);
    return GGKS_ORACLE_OOM;
  }
  pthread_barrier_t bar;
  pthread_barrier_init(&bar, NULL, (unsigned)threads);
  int skip = 0;
  sort_shared_t sh = {keys, tmp, n, threads, keybytes, hist, &bar, &skip};
  sort_arg_t args[MAX_THREADS];
  pthread_t tids[MAX_THREADS];
  for (int t = 0; t < threads; ++t) {
    args[t].sh = &sh;
    args[t].tid = t;
  }
  for (int t = 1; t < threads; ++t) pthread_create(&tids[t], NULL, radix_worker, &args[t]);
  radix_worker(&args[0]);
  for (int t = 1; t < threads; ++t) pthread_join(tids[t], NULL);
  pthread_barrier_destroy(&bar);
  if (sh.src != keys) memcpy(keys, sh.src, (size_t)n * (size_t)keybytes);
  free(tmp);
  free(hist);
  return GGKS_ORACLE_OK;
}

int ggks_oracle_sort_keys_u32(uint32_t *keys, uint64_t n, int threads) {
  return radix_sort(keys, n, 4, threads);
}
int ggks_oracle_sort_keys_u64(uint64_t *keys, uint64_t n, int threads) {
  return radix_sort(keys, n, 8, threads);
}

/* ------------------------------------------------------------------------ */
/* Parallel key conversion of the input copy.                                */
/* ------------------------------------------------------------------------ */
typedef struct {
  const void *in;
  void *out;
  uint64_t lo, hi;
  int kind; /* 0 f32, 1 f64, 2 u32 */
} conv_arg_t;

static void *conv_worker(void *varg) {
  conv_arg_t *a = (conv_arg_t *)varg;
  if (a->kind == 0) {
    const uint32_t *s = (const uint32_t *)a->in;
    uint32_t *d = (uint32_t *)a->out;
    for (uint64_t i = a->lo; i < a->hi; ++i) d[i] = ggks_oracle_key_f32(s[i]);
  } else if (a->kind == 1) {
    const uint64_t *s = (const uint64_t *)a->in;
    uint64_t *d = (uint64_t *)a->out;
    for (uint64_t i = a->lo; i < a->hi; ++i) d[i] = ggks_oracle_key_f64(s[i]);
  } else {
    memcpy((uint32_t *)a->out + a->lo, (const uint32_t *)a->in + a->lo,
           (size_t)(a->hi - a->lo) * 4);
  }
  return NULL;
}

static void *keys_of(const void *vec, uint64_t n, int kind, int threads) {
  const int kb = kind == 1 ? 8 : 4;
  void *keys = malloc((size_t)n * (size_t)kb);
  if (!keys) return NULL;
  if (threads < 1) threads = 1;
  if (threads > MAX_THREADS) threads = MAX_THREADS;
  conv_arg_t args[MAX_THREADS];
  pthread_t tids[MAX_THREADS];
  for (int t = 0; t < threads; ++t) {
    args[t].in = vec;
    args[t].out = keys;
    args[t].lo = n * (uint64_t)t / (uint64_t)threads;
    args[t].hi = n * (uint64_t)(t + 1) / (uint64_t)threads;
    args[t].kind = kind;
  }
  for (int t = 1; t < threads; ++t) pthread_create(&tids[t], NULL, conv_worker, &args[t]);
  conv_worker(&args[0]);
  for (int t = 1; t < threads; ++t) pthread_join(tids[t], NULL);
  return keys;
}

static void value_of_key(const void *keys, uint64_t idx, int kind, void *out, uint64_t oi) {
  if (kind == 0) {
    uint32_t b = ggks_oracle_unkey_f32(((const uint32_t *)keys)[idx]);
    memcpy((uint32_t *)out + oi, &b, 4);
  } else if (kind == 1) {
    uint64_t b = ggks_oracle_unkey_f64(((const uint64_t *)keys)[idx]);
    memcpy((uint64_t *)out + oi, &b, 8);
  } else {
    ((uint32_t *)out)[oi] = ((const uint32_t *)keys)[idx];
  }
}

/* multiselectTimingFunctions.cu:51-95: sort ascending, then
 * out[i] = sorted[n - k_i] (copyInChunk, :42-48). */
static int sort_and_choose(const void *vec, uint64_t n, const uint32_t *k, uint32_t num_k,
                           void *out, int threads, int kind) {
  if (!vec || !k || !out || n == 0 || num_k == 0) return GGKS_ORACLE_INVALID_ARG;
  for (uint32_t i = 0; i < num_k; ++i)
    if (k[i] < 1 || (uint64_t)k[i] > n) return GGKS_ORACLE_INVALID_ARG;
  void *keys = keys_of(vec, n, kind, threads);
  if (!keys) return GGKS_ORACLE_OOM;
  int st = radix_sort(keys, n, kind == 1 ? 8 : 4, threads);
  if (st == GGKS_ORACLE_OK)
    for (uint32_t i = 0; i < num_k; ++i) value_of_key(keys, n - k[i], kind, out, i);
  free(keys);
  return st;
}

/* multiselectTimingFunctions.cu:156-177: sort descending, take the first K. */
static int sort_and_choose_topk(const void *vec, uint64_t n, uint32_t kk, void *out,
                                int threads, int kind) {
  if (!vec || !out || n == 0 || kk == 0 || (uint64_t)kk > n) return GGKS_ORACLE_INVALID_ARG;
  void *keys = keys_of(vec, n, kind, threads);
  if (!keys) return GGKS_ORACLE_OOM;
  int st = radix_sort(keys, n, kind == 1 ? 8 : 4, threads);
  if (st == GGKS_ORACLE_OK)
    for (uint32_t i = 0; i < kk; ++i) value_of_key(keys, n - 1 - i, kind, out, i);
  free(keys);
  return st;
}

int ggks_oracle_multiselect_f32(const float *vec, uint64_t n, const uint32_t *k,
                                uint32_t num_k, float *out, int threads) {
  return sort_and_choose(vec, n, k, num_k, out, threads, 0);
}
int ggks_oracle_multiselect_f64(const double *vec, uint64_t n, const uint32_t *k,
                                uint32_t num_k, double *out, int threads) {
  return sort_and_choose(vec, n, k, num_k, out, threads, 1);
}
int ggks_oracle_multiselect_u32(const uint32_t *vec, uint64_t n, const uint32_t *k,
                                uint32_t num_k, uint32_t *out, int threads) {
  return sort_and_choose(vec, n, k, num_k, out, threads, 2);
}
int ggks_oracle_topk_f32(const float *vec, uint64_t n, uint32_t kk, float *out, int threads) {
  return sort_and_choose_topk(vec, n, kk, out, threads, 0);
}
int ggks_oracle_topk_f64(const double *vec, uint64_t n, uint32_t kk, double *out, int threads) {
  return sort_and_choose_topk(vec, n, kk, out, threads, 1);
}
int ggks_oracle_topk_u32(const uint32_t *vec, uint64_t n, uint32_t kk, uint32_t *out,
                         int threads) {
  return sort_and_choose_topk(vec, n, kk, out, threads, 2);
}

/* ------------------------------------------------------------------------ */
/* The reference's bucket multiselect, restated on the CPU.                  */
/* ------------------------------------------------------------------------ */
#define BMS_NUM_BUCKETS 8192 /* bucketMultiselect.cu:841 */
#define BMS_NUM_PIVOTS 17    /* bucketMultiselect.cu:868 */
#define BMS_SAMPLE 1024      /* bucketMultiselect.cu:562 */
#define BMS_END_OFFSET 22    /* bucketMultiselect.cu:420, :469 */

static uint64_t splitmix64(uint64_t *s) {
  uint64_t z = (*s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* native-type value access as double, as the reference's bucket projection
 * uses (bucketMultiselect.cu:184-186) */
static double as_double(const void *vec, uint64_t i, int kind) {
  if (kind == 0) return (double)((const float *)vec)[i];
  if (kind == 1) return ((const double *)vec)[i];
  return (double)((const uint32_t *)vec)[i];
}
static uint64_t key_at(const void *vec, uint64_t i, int kind) {
  if (kind == 0) {
    uint32_t b;
    memcpy(&b, (const float *)vec + i, 4);
    return ggks_oracle_key_f32(b);
  }
  if (kind == 1) {
    uint64_t b;
    memcpy(&b, (const double *)vec + i, 8);
    return ggks_oracle_key_f64(b);
  }
  return ((const uint32_t *)vec)[i];
}
static void store_from_key(void *out, uint64_t oi, uint64_t key, int kind) {
  if (kind == 0) {
    uint32_t b = ggks_oracle_unkey_f32((uint32_t)key);
    memcpy((uint32_t *)out + oi, &b, 4);
  } else if (kind == 1) {
    uint64_t b = ggks_oracle_unkey_f64(key);
    memcpy((uint64_t *)out + oi, &b, 8);
  } else {
    ((uint32_t *)out)[oi] = (uint32_t)key;
  }
}

typedef struct {
  uint32_t k, idx;
} kpair_t;
static int cmp_kpair(const void *a, const void *b) {
  const kpair_t *x = (const kpair_t *)a, *y = (const kpair_t *)b;
  if (x->k != y->k) return x->k < y->k ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}
static int cmp_double(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

/* bucketMultiselect.cu:129-205 (assignSmartBucket): 4-step binary search over
 * the 17 pivots, then a linear projection with the interval's slope. */
static uint32_t bms_bucket(double x, const double *piv, const double *slope) {
  int lo = 0, hi = BMS_NUM_PIVOTS - 1;
  for (int j = 1; j < BMS_NUM_PIVOTS - 1; j *= 2) {
    int mid = (hi + lo) / 2;
    if (x >= piv[mid])
      lo = mid;
    else
      hi = mid;
  }
  const int small = BMS_NUM_BUCKETS / (BMS_NUM_PIVOTS - 1);
  uint32_t b = (uint32_t)(lo * small) + (uint32_t)(int)((x - piv[lo]) * slope[lo]);
  if (b >= BMS_NUM_BUCKETS) b = BMS_NUM_BUCKETS - 1; /* :188-189 */
  return b;
}

static int bucket_multiselect(const void *vec, uint32_t n, const uint32_t *k_ori,
                              uint32_t num_k, void *out, uint64_t seed, int kind) {
  if (!vec || !k_ori || !out || n == 0 || num_k == 0) return GGKS_ORACLE_INVALID_ARG;
  for (uint32_t i = 0; i < num_k; ++i)
    if (k_ori[i] < 1 || k_ori[i] > n) return GGKS_ORACLE_INVALID_ARG;

  /* STEP 1 (:534-547): extrema; a flat vector answers every k with min. */
  uint64_t kmin = key_at(vec, 0, kind), kmax = kmin;
  uint64_t imin = 0, imax = 0;
  for (uint64_t i = 1; i < n; ++i) {
    uint64_t kk = key_at(vec, i, kind);
    if (kk < kmin) kmin = kk, imin = i;
    if (kk > kmax) kmax = kk, imax = i;
  }
  if (kmin == kmax) {
    for (uint32_t i = 0; i < num_k; ++i) store_from_key(out, i, kmin, kind);
    return GGKS_ORACLE_OK;
  }
  const double dmin = as_double(vec, imin, kind), dmax = as_double(vec, imax, kind);

  /* wrapper (:842-846): k-th largest -> k-th smallest, 1-based */
  kpair_t *ks = malloc(sizeof(kpair_t) * num_k);
  if (!ks) return GGKS_ORACLE_OOM;
  for (uint32_t i = 0; i < num_k; ++i) {
    ks[i].k = n - k_ori[i] + 1;
    ks[i].idx = i;
  }
  /* STEP 3 (:615-646): sort the k's keeping their indices; peel k == n (max)
   * and k == 1 (min). */
  qsort(ks, num_k, sizeof(kpair_t), cmp_kpair);
  uint32_t first = 0, last = num_k;
  while (last > first && ks[last - 1].k == n) {
    store_from_key(out, ks[last - 1].idx, kmax, kind);
    last--;
  }
  while (first < last && ks[first].k == 1) {
    store_from_key(out, ks[first].idx, kmin, kind);
    first++;
  }
  if (first == last) { /* every k was peeled (the reference reads garbage here) */
    free(ks);
    return GGKS_ORACLE_OK;
  }

  /* STEP 4 (:414-508, :665-667): 1024 sampled elements, sorted; pivots at
   * min, s[21], s[21 + 70 (i-1)] (i = 2..14), s[1001], max; slopes
   * 512 / (p_{i+1} - p_i), infinite slopes set to 0. */
  double sample[BMS_SAMPLE];
  uint64_t st = seed ? seed : 0x243f6a8885a308d3ull;
  for (int i = 0; i < BMS_SAMPLE; ++i) {
    uint64_t pos = (splitmix64(&st) >> 11) % n;
    sample[i] = as_double(vec, pos, kind);
  }
  qsort(sample, BMS_SAMPLE, sizeof(double), cmp_double);
  double piv[BMS_NUM_PIVOTS], slope[BMS_NUM_PIVOTS - 1];
  const int pivot_offset = (BMS_SAMPLE - BMS_END_OFFSET * 2) / (BMS_NUM_PIVOTS - 3);
  const double small = (double)(BMS_NUM_BUCKETS / (BMS_NUM_PIVOTS - 1));
  piv[0] = dmin;
  piv[BMS_NUM_PIVOTS - 1] = dmax;
  piv[1] = sample[BMS_END_OFFSET - 1];
  piv[BMS_NUM_PIVOTS - 2] = sample[BMS_SAMPLE - BMS_END_OFFSET - 1];
  for (int i = 2; i < BMS_NUM_PIVOTS - 2; ++i)
    piv[i] = sample[pivot_offset * (i - 1) + BMS_END_OFFSET - 1];
  for (int i = 0; i < BMS_NUM_PIVOTS - 1; ++i) {
    slope[i] = small / (piv[i + 1] - piv[i]);
    if (isinf(slope[i]) || isnan(slope[i])) slope[i] = 0;
  }

  /* STEP 5 (:689-696): per-bucket counts. */
  uint32_t *bucket_of = malloc(sizeof(uint32_t) * (size_t)n);
  uint64_t *count = calloc(BMS_NUM_BUCKETS, sizeof(uint64_t));
  if (!bucket_of || !count) {
    free(ks);
    free(bucket_of);
    free(count);
    return GGKS_ORACLE_OOM;
  }
  for (uint64_t i = 0; i < n; ++i) {
    uint32_t b = bms_bucket(as_double(vec, i, kind), piv, slope);
    bucket_of[i] = b;
    count[b]++;
  }

  /* STEP 6 (:87-111, :714-730): walk the sorted k's over the cumulative
   * counts; each k gets its bucket and the count before it; unique buckets
   * get consecutive output offsets; k' = offset + k - before. */
  const uint32_t nk = last - first;
  uint32_t *kbucket = malloc(sizeof(uint32_t) * nk);
  uint64_t *kbefore = malloc(sizeof(uint64_t) * nk);
  uint64_t *klocal = malloc(sizeof(uint64_t) * nk);
  int64_t *seg_of_bucket = malloc(sizeof(int64_t) * BMS_NUM_BUCKETS);
  uint64_t *seg_off = malloc(sizeof(uint64_t) * (BMS_NUM_BUCKETS + 1));
  if (!kbucket || !kbefore || !klocal || !seg_of_bucket || !seg_off) {
    free(ks), free(bucket_of), free(count), free(kbucket), free(kbefore), free(klocal);
    free(seg_of_bucket), free(seg_off);
    return GGKS_ORACLE_OOM;
  }
  {
    uint32_t kb = 0;
    uint64_t sum = count[0];
    for (uint32_t i = 0; i < nk; ++i) {
      uint64_t kv = ks[first + i].k;
      while (sum < kv && kb < BMS_NUM_BUCKETS - 1) {
        kb++;
        sum += count[kb];
      }
      kbucket[i] = kb;
      kbefore[i] = sum - count[kb];
    }
  }
  for (uint32_t b = 0; b < BMS_NUM_BUCKETS; ++b) seg_of_bucket[b] = -1;
  uint32_t nseg = 0;
  uint64_t total = 0;
  for (uint32_t i = 0; i < nk; ++i) {
    if (i == 0 || kbucket[i] != kbucket[i - 1]) {
      seg_of_bucket[kbucket[i]] = nseg;
      seg_off[nseg] = total;
      total += count[kbucket[i]];
      nseg++;
    }
    klocal[i] = seg_off[seg_of_bucket[kbucket[i]]] + (ks[first + i].k - kbefore[i]);
  }

  /* STEP 7 (:249-308, :777-780): copy the elements of the marked buckets. */
  uint64_t *surv = malloc(sizeof(uint64_t) * (size_t)(total ? total : 1));
  uint64_t *cursor = malloc(sizeof(uint64_t) * (nseg ? nseg : 1));
  if (!surv || !cursor) {
    free(ks), free(bucket_of), free(count), free(kbucket), free(kbefore), free(klocal);
    free(seg_of_bucket), free(seg_off), free(surv), free(cursor);
    return GGKS_ORACLE_OOM;
  }
  for (uint32_t s = 0; s < nseg; ++s) cursor[s] = seg_off[s];
  for (uint64_t i = 0; i < n; ++i) {
    int64_t s = seg_of_bucket[bucket_of[i]];
    if (s >= 0) surv[cursor[s]++] = key_at(vec, i, kind);
  }

  /* STEP 8 (:799-818): sort the survivors, gather out[idx] = surv[k' - 1]. */
  int rc = radix_sort(surv, total, 8, 1);
  if (rc == GGKS_ORACLE_OK)
    for (uint32_t i = 0; i < nk; ++i)
      store_from_key(out, ks[first + i].idx, surv[klocal[i] - 1], kind);

  free(ks), free(bucket_of), free(count), free(kbucket), free(kbefore), free(klocal);
  free(seg_of_bucket), free(seg_off), free(surv), free(cursor);
  return rc;
}

int ggks_oracle_bucket_multiselect_f32(const float *vec, uint32_t n, const uint32_t *k,
                                       uint32_t num_k, float *out, uint64_t seed) {
  return bucket_multiselect(vec, n, k, num_k, out, seed, 0);
}
int ggks_oracle_bucket_multiselect_f64(const double *vec, uint32_t n, const uint32_t *k,
                                       uint32_t num_k, double *out, uint64_t seed) {
  return bucket_multiselect(vec, n, k, num_k, out, seed, 1);
}
int ggks_oracle_bucket_multiselect_u32(const uint32_t *vec, uint32_t n, const uint32_t *k,
                                       uint32_t num_k, uint32_t *out, uint64_t seed) {
  return bucket_multiselect(vec, n, k, num_k, out, seed, 2);
}
