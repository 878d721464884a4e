// ggks_bucket_multiselect.hpp -- C++ mirror of the reference's host interface
// for the bucket multiselect / top-k path, implemented over the C ABI in
// ggks.h.  Code written against the reference's headers compiles against this
// one with the same names and argument meanings:
//
//   BucketMultiselect::bucketMultiselectWrapper<T>   bucketMultiselect.cu:837-871
//   results_t<T>                                     multiselectTimingFunctions.cu:11-14
//   timeBucketMultiselect<T>                         multiselectTimingFunctions.cu:100-122
//   timeBucketTopkselect<T>                          multiselectTimingFunctions.cu:205-231
//   randomizedTopkSelectWrapper<T>                   randomizedTopkSelect.cu:210-213
//   BucketSelect::bucketSelectWrapper<T>             bucketSelect.cu:453-471
//   RandomizedBucketSelect::randomizedBucketSelectWrapper<T>
//                                                    randomizedBucketSelect.cu:861-881
//
// T is float, double or unsigned int (the reference's uint).  Differences:
//   - errors are not silent: the wrapper returns (T)0 instead of (T)1 and
//     BucketMultiselect::lastStatus() holds the ggks_status;
//   - blocks / threads are accepted and ignored (launch shapes are chosen per
//     problem);
//   - the timing adapters time the host-vector entry point, so their time
//     includes the host-to-device copy of the vector, which the reference
//     performs before starting its timer (setupForTiming, :17-26).
#ifndef GGKS_BUCKET_MULTISELECT_HPP_
#define GGKS_BUCKET_MULTISELECT_HPP_

#include <chrono>
#include <cstdint>
#include <cstdlib>

#include "ggks.h"

namespace ggks_detail {
template <typename T>
struct Api;
template <>
struct Api<float> {
  static int ms(const float *d, uint64_t n, const uint32_t *k, uint32_t nk, float *o) {
    return ggks_multiselect_f32(d, n, k, nk, o, nullptr);
  }
  static int ms_host(const float *h, uint64_t n, const uint32_t *k, uint32_t nk, float *o) {
    return ggks_multiselect_host_f32(h, n, k, nk, o, nullptr);
  }
  static int tk(const float *d, uint64_t n, uint32_t K, float *o) {
    return ggks_topk_f32(d, n, K, o, nullptr);
  }
  static int tk_host(const float *h, uint64_t n, uint32_t K, float *o) {
    return ggks_topk_host_f32(h, n, K, o, nullptr);
  }
  static int sel(const float *d, uint64_t n, uint32_t k, float *o) {
    return ggks_select_f32(d, n, k, o, nullptr);
  }
};
template <>
struct Api<double> {
  static int ms(const double *d, uint64_t n, const uint32_t *k, uint32_t nk, double *o) {
    return ggks_multiselect_f64(d, n, k, nk, o, nullptr);
  }
  static int ms_host(const double *h, uint64_t n, const uint32_t *k, uint32_t nk, double *o) {
    return ggks_multiselect_host_f64(h, n, k, nk, o, nullptr);
  }
  static int tk(const double *d, uint64_t n, uint32_t K, double *o) {
    return ggks_topk_f64(d, n, K, o, nullptr);
  }
  static int tk_host(const double *h, uint64_t n, uint32_t K, double *o) {
    return ggks_topk_host_f64(h, n, K, o, nullptr);
  }
  static int sel(const double *d, uint64_t n, uint32_t k, double *o) {
    return ggks_select_f64(d, n, k, o, nullptr);
  }
};
template <>
struct Api<unsigned int> {
  static int ms(const unsigned int *d, uint64_t n, const uint32_t *k, uint32_t nk,
                unsigned int *o) {
    return ggks_multiselect_u32(d, n, k, nk, o, nullptr);
  }
  static int ms_host(const unsigned int *h, uint64_t n, const uint32_t *k, uint32_t nk,
                     unsigned int *o) {
    return ggks_multiselect_host_u32(h, n, k, nk, o, nullptr);
  }
  static int tk(const unsigned int *d, uint64_t n, uint32_t K, unsigned int *o) {
    return ggks_topk_u32(d, n, K, o, nullptr);
  }
  static int tk_host(const unsigned int *h, uint64_t n, uint32_t K, unsigned int *o) {
    return ggks_topk_host_u32(h, n, K, o, nullptr);
  }
  static int sel(const unsigned int *d, uint64_t n, uint32_t k, unsigned int *o) {
    return ggks_select_u32(d, n, k, o, nullptr);
  }
};
inline int &last_status() {
  static thread_local int s = GGKS_OK;
  return s;
}
}  // namespace ggks_detail

namespace BucketMultiselect {

// ggks_status of the calling thread's last call through this header
inline int lastStatus() { return ggks_detail::last_status(); }

// bucketMultiselect.cu:837-871: d_vector is a device vector of `length`
// elements; kVals_ori holds numKs k's (k-th largest, 1-based, host memory,
// not modified); outputs is a host array of numKs values in k order.
template <typename T>
T bucketMultiselectWrapper(T *d_vector, int length, unsigned int *kVals_ori, int numKs,
                           T *outputs, int blocks, int threads) {
  (void)blocks;
  (void)threads;
  if (length <= 0 || numKs <= 0) {
    ggks_detail::last_status() = GGKS_INVALID_ARG;
    return (T)0;
  }
  int st = ggks_detail::Api<T>::ms(d_vector, (uint64_t)length, kVals_ori, (uint32_t)numKs, outputs);
  ggks_detail::last_status() = st;
  return st == GGKS_OK ? (T)1 : (T)0;
}

}  // namespace BucketMultiselect

// multiselectTimingFunctions.cu:11-14
template <typename T>
struct results_t {
  float time;
  T *vals;
};

template <typename T>
inline void freeResults(results_t<T> *r) {
  if (r) {
    std::free(r->vals);
    std::free(r);
  }
}

// multiselectTimingFunctions.cu:100-122 (host vector in, k list, results in
// k order); returns nullptr on error (lastStatus() says why).
template <typename T>
results_t<T> *timeBucketMultiselect(T *h_vec, unsigned int numElements, unsigned int *kVals,
                                    unsigned int kCount) {
  results_t<T> *r = (results_t<T> *)std::malloc(sizeof(results_t<T>));
  if (!r) return nullptr;
  r->vals = (T *)std::malloc(sizeof(T) * (kCount ? kCount : 1));
  auto t0 = std::chrono::steady_clock::now();
  int st = ggks_detail::Api<T>::ms_host(h_vec, numElements, kVals, kCount, r->vals);
  auto t1 = std::chrono::steady_clock::now();
  ggks_detail::last_status() = st;
  if (st != GGKS_OK) {
    freeResults(r);
    return nullptr;
  }
  r->time = std::chrono::duration<float, std::milli>(t1 - t0).count();
  return r;
}

// multiselectTimingFunctions.cu:205-231: the kCount largest, descending.
template <typename T>
results_t<T> *timeBucketTopkselect(T *h_vec, unsigned int numElements, unsigned int kCount) {
  results_t<T> *r = (results_t<T> *)std::malloc(sizeof(results_t<T>));
  if (!r) return nullptr;
  r->vals = (T *)std::malloc(sizeof(T) * (kCount ? kCount : 1));
  auto t0 = std::chrono::steady_clock::now();
  int st = ggks_detail::Api<T>::tk_host(h_vec, numElements, kCount, r->vals);
  auto t1 = std::chrono::steady_clock::now();
  ggks_detail::last_status() = st;
  if (st != GGKS_OK) {
    freeResults(r);
    return nullptr;
  }
  r->time = std::chrono::duration<float, std::milli>(t1 - t0).count();
  return r;
}

// randomizedTopkSelect.cu:210-213 signature: device list in, a malloc'd host
// array of the k largest values (descending) out, owned by the caller.
// Computed by the bucket path (exact), not by the randomized algorithm.
template <typename T>
T *randomizedTopkSelectWrapper(T *list, int size, int k) {
  if (size <= 0 || k <= 0) {
    ggks_detail::last_status() = GGKS_INVALID_ARG;
    return nullptr;
  }
  T *out = (T *)std::malloc(sizeof(T) * (size_t)k);
  if (!out) return nullptr;
  int st = ggks_detail::Api<T>::tk(list, (uint64_t)size, (uint32_t)k, out);
  ggks_detail::last_status() = st;
  if (st != GGKS_OK) {
    std::free(out);
    return nullptr;
  }
  return out;
}

namespace ggks_detail {
template <typename T>
T select_one(T *d_vector, int length, int K) {
  T v = (T)0;
  if (length <= 0 || K <= 0 || K > length) {
    last_status() = GGKS_INVALID_ARG;
    return v;
  }
  last_status() = Api<T>::sel(d_vector, (uint64_t)length, (uint32_t)K, &v);
  return v;
}
}  // namespace ggks_detail

// bucketSelect.cu:453-471: the K-th largest element (1-based) of the device
// vector; BucketMultiselect::lastStatus() reports errors (the value is then 0).
namespace BucketSelect {
template <typename T>
T bucketSelectWrapper(T *d_vector, int length, int K, int blocks, int threads) {
  (void)blocks;
  (void)threads;
  return ggks_detail::select_one(d_vector, length, K);
}
}  // namespace BucketSelect

// randomizedBucketSelect.cu:861-881: same contract; computed by the same
// exact bucket path.
namespace RandomizedBucketSelect {
template <typename T>
T randomizedBucketSelectWrapper(T *d_vector, int length, int K, int blocks, int threads) {
  (void)blocks;
  (void)threads;
  return ggks_detail::select_one(d_vector, length, K);
}
}  // namespace RandomizedBucketSelect

#endif  // GGKS_BUCKET_MULTISELECT_HPP_
