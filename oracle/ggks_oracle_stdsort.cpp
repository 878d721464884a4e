// ggks_oracle_stdsort.cpp -- single-threaded sort-and-choose with std::sort.
//
// TEST INFRASTRUCTURE ONLY (see ggks_oracle.h): the benchmark's CPU baseline
// leg times it.  It restates multiselectTimingFunctions.cu:51-95 (sort the
// whole vector, out[i] = ascending[n - k_i]) with the comparison sort of the
// C++ standard library on one thread, ordering by the order-preserving key as
// the rest of the oracle does.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "ggks_oracle.h"

namespace {

template <class T, class K, K (*Key)(K), K (*Unkey)(K)>
int stdsort_multiselect(const T *vec, uint64_t n, const uint32_t *k, uint32_t num_k, T *out) {
  if ((n && !vec) || (num_k && (!k || !out))) return GGKS_ORACLE_INVALID_ARG;
  for (uint32_t i = 0; i < num_k; ++i)
    if (k[i] < 1 || k[i] > n) return GGKS_ORACLE_INVALID_ARG;
  std::vector<K> keys;
  try {
    keys.resize(n);
  } catch (...) {
    return GGKS_ORACLE_OOM;
  }
  for (uint64_t i = 0; i < n; ++i) {
    K b;
    std::memcpy(&b, vec + i, sizeof(K));
    keys[i] = Key(b);
  }
  std::sort(keys.begin(), keys.end());
  for (uint32_t i = 0; i < num_k; ++i) {
    const K b = Unkey(keys[n - k[i]]);
    std::memcpy(out + i, &b, sizeof(K));
  }
  return GGKS_ORACLE_OK;
}

uint32_t id32(uint32_t v) { return v; }

}  // namespace

extern "C" int ggks_oracle_multiselect_stdsort_f32(const float *vec, uint64_t n, const uint32_t *k,
                                                   uint32_t num_k, float *out) {
  return stdsort_multiselect<float, uint32_t, ggks_oracle_key_f32, ggks_oracle_unkey_f32>(
      vec, n, k, num_k, out);
}

extern "C" int ggks_oracle_multiselect_stdsort_f64(const double *vec, uint64_t n,
                                                   const uint32_t *k, uint32_t num_k, double *out) {
  return stdsort_multiselect<double, uint64_t, ggks_oracle_key_f64, ggks_oracle_unkey_f64>(
      vec, n, k, num_k, out);
}

extern "C" int ggks_oracle_multiselect_stdsort_u32(const uint32_t *vec, uint64_t n,
                                                   const uint32_t *k, uint32_t num_k,
                                                   uint32_t *out) {
  return stdsort_multiselect<uint32_t, uint32_t, id32, id32>(vec, n, k, num_k, out);
}
