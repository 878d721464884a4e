// A caller written against the reference's host interface, built against
// include/ggks_bucket_multiselect.hpp only (plus the CUDA runtime for its
// device buffers): it calls every name the C++ mirror provides on real device
// data and writes the answers for the test to check against the oracle.
//
//   dropin_harness <dir> <n> <numKs> <K>
// reads <dir>/vec_{f32,f64,u32}.bin (n elements each) and <dir>/k.bin (numKs
// k's, k-th largest, 1-based) and writes, per type t:
//   ms_t.bin   BucketMultiselect::bucketMultiselectWrapper   (numKs values)
//   tms_t.bin  timeBucketMultiselect                         (numKs values)
//   ttk_t.bin  timeBucketTopkselect                          (K values, descending)
//   rtk_t.bin  randomizedTopkSelectWrapper                   (K values, descending)
//   sel_t.bin  BucketSelect::bucketSelectWrapper, k = k[0..7]  (8 values)
//   rsel_t.bin RandomizedBucketSelect::randomizedBucketSelectWrapper, same k's
// Exit status 0 only if every call succeeded.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ggks_bucket_multiselect.hpp"

namespace {

template <typename T>
bool read_file(const std::string &path, std::vector<T> &v, size_t count) {
  v.resize(count);
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  const size_t got = std::fread(v.data(), sizeof(T), count, f);
  std::fclose(f);
  return got == count;
}

template <typename T>
bool write_file(const std::string &path, const T *v, size_t count) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const size_t put = std::fwrite(v, sizeof(T), count, f);
  std::fclose(f);
  return put == count;
}

template <typename T>
int run(const std::string &dir, const char *t, int n, std::vector<unsigned int> &k, int K) {
  std::vector<T> h;
  if (!read_file(dir + "/vec_" + t + ".bin", h, (size_t)n)) return 10;
  T *d = nullptr;
  if (cudaMalloc(&d, sizeof(T) * (size_t)n) != cudaSuccess) return 11;
  if (cudaMemcpy(d, h.data(), sizeof(T) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess)
    return 12;
  const int numKs = (int)k.size();
  int rc = 0;

  // bucketMultiselect.cu:837-871 -- the caller passes #SMs and the block size
  cudaDeviceProp dp;
  cudaGetDeviceProperties(&dp, 0);
  std::vector<T> out((size_t)numKs);
  T ret = BucketMultiselect::bucketMultiselectWrapper(d, n, k.data(), numKs, out.data(),
                                                      dp.multiProcessorCount, dp.maxThreadsPerBlock);
  if (ret != (T)1 || BucketMultiselect::lastStatus() != GGKS_OK) rc = 20;
  if (!write_file(dir + "/ms_" + t + ".bin", out.data(), out.size())) rc = 21;

  // multiselectTimingFunctions.cu:100-122 and :205-231 (host vector in)
  results_t<T> *r = timeBucketMultiselect(h.data(), (unsigned)n, k.data(), (unsigned)numKs);
  if (!r || !(r->time >= 0.f)) {
    rc = 30;
  } else if (!write_file(dir + "/tms_" + t + ".bin", r->vals, (size_t)numKs)) {
    rc = 31;
  }
  freeResults(r);
  results_t<T> *tk = timeBucketTopkselect(h.data(), (unsigned)n, (unsigned)K);
  if (!tk) {
    rc = 40;
  } else if (!write_file(dir + "/ttk_" + t + ".bin", tk->vals, (size_t)K)) {
    rc = 41;
  }
  freeResults(tk);

  // randomizedTopkSelect.cu:210-213: caller-owned malloc'd array
  T *rt = randomizedTopkSelectWrapper(d, n, K);
  if (!rt) {
    rc = 50;
  } else if (!write_file(dir + "/rtk_" + t + ".bin", rt, (size_t)K)) {
    rc = 51;
  }
  std::free(rt);

  // bucketSelect.cu:453-471, randomizedBucketSelect.cu:861-881
  T sel[8], rsel[8];
  for (int i = 0; i < 8; ++i) {
    const int kk = (int)k[(size_t)i % k.size()];
    sel[i] = BucketSelect::bucketSelectWrapper(d, n, kk, dp.multiProcessorCount,
                                               dp.maxThreadsPerBlock);
    if (BucketMultiselect::lastStatus() != GGKS_OK) rc = 60;
    rsel[i] = RandomizedBucketSelect::randomizedBucketSelectWrapper(d, n, kk, 0, 0);
    if (BucketMultiselect::lastStatus() != GGKS_OK) rc = 61;
  }
  if (!write_file(dir + "/sel_" + t + ".bin", sel, 8)) rc = 62;
  if (!write_file(dir + "/rsel_" + t + ".bin", rsel, 8)) rc = 63;
  cudaFree(d);
  return rc;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s <dir> <n> <numKs> <K>\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const int n = std::atoi(argv[2]), numKs = std::atoi(argv[3]), K = std::atoi(argv[4]);
  std::vector<unsigned int> k;
  if (!read_file(dir + "/k.bin", k, (size_t)numKs)) return 3;
  int rc = run<float>(dir, "f32", n, k, K);
  if (rc == 0) rc = run<double>(dir, "f64", n, k, K);
  if (rc == 0) rc = run<unsigned int>(dir, "u32", n, k, K);
  if (rc != 0) std::fprintf(stderr, "failed: code %d (last ggks status %d)\n", rc,
                            BucketMultiselect::lastStatus());
  return rc;
}
