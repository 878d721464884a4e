// ref_gpu_host.cu -- test and measurement infrastructure: the reference's
// bucket multiselect run on the GPU with the reference's own kernels.
//
// The reference is a set of .cu drivers whose host and device code compile as
// one unit.  Its kernels come from oracle/_ref/ref_kernels.cubin (built from
// the reference's sources in place by oracle/ref_gpu.py, see ref_kernels.cu).
// Its host code cannot be built where its sources are absent, so this file
// restates it step by step and launches the cubin's kernels with the
// reference's grids, blocks, shared-memory sizes and arguments, on the legacy
// default stream, with the same synchronous copies, allocations and Thrust
// calls (CUDA's own Thrust):
//   phaseOne<T>                 bucketMultiselect.cu:521-833
//   generatePivots<T>           :414-457 (uint), :460-508 (float, double)
//   createRandomVector<T>       :374-386 (the cubin's ggks_ref_random_vector_*)
//   findKBuckets                :87-111
//   bucketMultiselectWrapper<T> :837-871
//   timeBucketMultiselect<T>, timeBucketTopkselect<T>,
//   timeSortAndChooseMultiselect<T>, timeSortAndChooseTopkselect<T>
//                               multiselectTimingFunctions.cu:100-122,
//                               :205-231, :51-95, :156-177
// Two guards, which change nothing for the inputs the tests and the bench use:
//  * the k sort's peeling loops (:633-646) stop at the list's ends, and a list
//    made only of k = 1 and k = n returns after peeling (the reference reads
//    outside its arrays there);
//  * the sampling kernel reads list[(int)(u * size)] with u from Thrust's
//    uniform_real_distribution<float>(0, 1), which returns 1.0f when the
//    engine's draw rounds up to the float denominator (about 3e-8 per draw):
//    that reads list[size], one element past the vector.  The timing adapters
//    here therefore allocate one element more and give it the vector's first
//    value (an element of the vector, so the pivots stay in [min, max]); a
//    caller of the device-vector entries must do the same.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cxxabi.h>
#include <sys/time.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <thrust/device_ptr.h>
#include <thrust/extrema.h>
#include <thrust/functional.h>
#include <thrust/pair.h>
#include <thrust/sort.h>

namespace {

typedef unsigned int uint;
constexpr int kMaxThreadsPerBlock = 1024;  // MAX_THREADS_PER_BLOCK, bucketMultiselect.cu:27

// ---------------------------------------------------------------------------
// the cubin and its kernels
// ---------------------------------------------------------------------------
template <class T> struct TypeIx;
template <> struct TypeIx<float> { static constexpr int v = 0; static constexpr const char *n = "float"; };
template <> struct TypeIx<double> { static constexpr int v = 1; static constexpr const char *n = "double"; };
template <> struct TypeIx<uint> { static constexpr int v = 2; static constexpr const char *n = "unsigned int"; };

struct Kernels {
  CUfunction assign[3] = {}, copy_elements[3] = {}, copy_values[3] = {}, copy_in_chunk[3] = {};
  CUfunction enlarge[2] = {};     // template, float and double
  CUfunction enlarge_uint = {};   // the overload for uint vectors (:402-405)
  CUfunction sum_counts = {}, reindex_counts = {};
  CUfunction random_f32 = {}, random_f64 = {};
};
CUmodule g_mod = nullptr;
Kernels g_k;
std::mutex g_mu;

bool has(const std::string &s, const std::string &what) { return s.find(what) != std::string::npos; }

// Names every kernel of the cubin by its demangled signature.
int bind_kernels() {
  unsigned cnt = 0;
  if (cuModuleGetFunctionCount(&cnt, g_mod) != CUDA_SUCCESS) return -2;
  std::vector<CUfunction> fs(cnt);
  if (cuModuleEnumerateFunctions(fs.data(), cnt, g_mod) != CUDA_SUCCESS) return -3;
  const char *tn[3] = {TypeIx<float>::n, TypeIx<double>::n, TypeIx<uint>::n};
  for (CUfunction f : fs) {
    const char *raw = nullptr;
    if (cuFuncGetName(&raw, f) != CUDA_SUCCESS || !raw) continue;
    int st = 0;
    char *dm = abi::__cxa_demangle(raw, nullptr, nullptr, &st);
    const std::string s = st == 0 && dm ? dm : raw;
    std::free(dm);
    for (int t = 0; t < 3; ++t) {
      const std::string a = std::string("<") + tn[t] + ">(";
      if (has(s, "BucketMultiselect::assignSmartBucket" + a)) g_k.assign[t] = f;
      if (has(s, "BucketMultiselect::copyElements" + a)) g_k.copy_elements[t] = f;
      if (has(s, "BucketMultiselect::copyValuesInChunk" + a)) g_k.copy_values[t] = f;
      if (has(s, "copyInChunk" + a) && !has(s, "copyValuesInChunk")) g_k.copy_in_chunk[t] = f;
      if (t < 2 && has(s, "BucketMultiselect::enlargeIndexAndGetElements" + a)) g_k.enlarge[t] = f;
    }
    if (has(s, "BucketMultiselect::enlargeIndexAndGetElements(float*, unsigned int*")) g_k.enlarge_uint = f;
    if (has(s, "BucketMultiselect::sumCounts(")) g_k.sum_counts = f;
    if (has(s, "BucketMultiselect::reindexCounts(")) g_k.reindex_counts = f;
    if (s == "ggks_ref_random_vector_f32") g_k.random_f32 = f;
    if (s == "ggks_ref_random_vector_f64") g_k.random_f64 = f;
  }
  for (int t = 0; t < 3; ++t)
    if (!g_k.assign[t] || !g_k.copy_elements[t] || !g_k.copy_values[t] || !g_k.copy_in_chunk[t])
      return -4;
  if (!g_k.enlarge[0] || !g_k.enlarge[1] || !g_k.enlarge_uint || !g_k.sum_counts ||
      !g_k.reindex_counts || !g_k.random_f32 || !g_k.random_f64)
    return -4;
  return 0;
}

// <<<grid, block, smem>>> on the legacy default stream, as the reference's
// launches are
bool launch(CUfunction f, unsigned grid, unsigned block, unsigned smem, void **args) {
  return cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, (CUstream)0, args, nullptr) ==
         CUDA_SUCCESS;
}

#define REF_CALL(x)                                                                   \
  do {                                                                                \
    if ((x) != cudaSuccess) {                                                         \
      std::fprintf(stderr, "reference GPU path: CUDA error at %s:%d\n", __FILE__, __LINE__); \
      return EXIT_FAILURE;                                                            \
    }                                                                                 \
  } while (0)
#define REF_LAUNCH(...)                                                               \
  do {                                                                                \
    if (!launch(__VA_ARGS__)) {                                                       \
      std::fprintf(stderr, "reference GPU path: launch failed at %s:%d\n", __FILE__, __LINE__); \
      return EXIT_FAILURE;                                                            \
    }                                                                                 \
  } while (0)

// createRandomVector<T> (:374-386): seeded from the time of day, as there
uint time_seed() {
  timeval t1;
  gettimeofday(&t1, nullptr);
  return (uint)(t1.tv_usec * t1.tv_sec);
}
int random_vector(float *d, int size) {
  uint seed = time_seed();
  void *a[] = {&d, &size, &seed};
  REF_LAUNCH(g_k.random_f32, (unsigned)((size + 255) / 256), 256, 0, a);
  return 0;
}
int random_vector(double *d, int size) {
  uint seed = time_seed();
  void *a[] = {&d, &size, &seed};
  REF_LAUNCH(g_k.random_f64, (unsigned)((size + 255) / 256), 256, 0, a);
  return 0;
}

// pivots[1] and pivots[P-2] are the sample's elements endOffset from its ends,
// the others evenly spaced in between; each slope maps a pivot interval onto
// numSmallBuckets buckets (one single-element copy per pivot, as there)
template <class T, class D>
int pivots_from_sorted_sample(T *pivots, double *slopes, const T *d_sample, int numPivots,
                              int sizeOfSample, int totalSmallBuckets, D diff) {
  const int endOffset = 22;
  const int pivotOffset = (sizeOfSample - endOffset * 2) / (numPivots - 3);
  const int numSmallBuckets = totalSmallBuckets / (numPivots - 1);
  REF_CALL(cudaMemcpy(pivots + 1, d_sample + endOffset - 1, sizeof(T), cudaMemcpyDeviceToHost));
  REF_CALL(cudaMemcpy(pivots + numPivots - 2, d_sample + sizeOfSample - endOffset - 1, sizeof(T),
                      cudaMemcpyDeviceToHost));
  slopes[0] = numSmallBuckets / diff(pivots[1], pivots[0]);
  for (int i = 2; i < numPivots - 2; i++) {
    REF_CALL(cudaMemcpy(pivots + i, d_sample + pivotOffset * (i - 1) + endOffset - 1, sizeof(T),
                        cudaMemcpyDeviceToHost));
    slopes[i - 1] = numSmallBuckets / diff(pivots[i], pivots[i - 1]);
  }
  slopes[numPivots - 3] = numSmallBuckets / diff(pivots[numPivots - 2], pivots[numPivots - 3]);
  slopes[numPivots - 2] = numSmallBuckets / diff(pivots[numPivots - 1], pivots[numPivots - 2]);
  return 0;
}

// generatePivots<float/double> (:460-508)
template <class T>
int generate_pivots(T *pivots, double *slopes, T *d_list, int sizeOfVector, int numPivots,
                    int sizeOfSample, int totalSmallBuckets, T mn, T mx) {
  T *d_randoms = nullptr;
  REF_CALL(cudaMalloc(&d_randoms, sizeof(T) * sizeOfSample));
  if (random_vector(d_randoms, sizeOfSample)) return EXIT_FAILURE;
  void *a[] = {&d_randoms, &d_list, &sizeOfVector};
  REF_LAUNCH(g_k.enlarge[TypeIx<T>::v], (unsigned)(sizeOfSample / kMaxThreadsPerBlock),
             kMaxThreadsPerBlock, 0, a);
  pivots[0] = mn;
  pivots[numPivots - 1] = mx;
  thrust::device_ptr<T> rp(d_randoms);
  thrust::sort(rp, rp + sizeOfSample);
  REF_CALL(cudaDeviceSynchronize());
  if (pivots_from_sorted_sample(pivots, slopes, d_randoms, numPivots, sizeOfSample,
                                totalSmallBuckets,
                                [](T a, T b) { return (double)a - (double)b; }))
    return EXIT_FAILURE;
  cudaFree(d_randoms);
  return 0;
}

// generatePivots for uint vectors (:414-457): float draws, gathered as uint
// into the same buffer; slopes from the unsigned difference
template <>
int generate_pivots<uint>(uint *pivots, double *slopes, uint *d_list, int sizeOfVector,
                          int numPivots, int sizeOfSample, int totalSmallBuckets, uint mn,
                          uint mx) {
  float *d_randomFloats = nullptr;
  REF_CALL(cudaMalloc(&d_randomFloats, sizeof(float) * sizeOfSample));
  uint *d_randomInts = (uint *)d_randomFloats;
  if (random_vector(d_randomFloats, sizeOfSample)) return EXIT_FAILURE;
  void *a[] = {&d_randomFloats, &d_randomInts, &d_list, &sizeOfVector};
  REF_LAUNCH(g_k.enlarge_uint, (unsigned)(sizeOfSample / kMaxThreadsPerBlock),
             kMaxThreadsPerBlock, 0, a);
  pivots[0] = mn;
  pivots[numPivots - 1] = mx;
  thrust::device_ptr<uint> rp(d_randomInts);
  thrust::sort(rp, rp + sizeOfSample);
  REF_CALL(cudaDeviceSynchronize());
  if (pivots_from_sorted_sample(pivots, slopes, d_randomInts, numPivots, sizeOfSample,
                                totalSmallBuckets, [](uint a, uint b) { return (double)(a - b); }))
    return EXIT_FAILURE;
  cudaFree(d_randomFloats);
  return 0;
}

// findKBuckets (:87-111): the last row of the scanned counts holds the
// totals; walk the sorted k's over them
int find_k_buckets(uint *d_bucketCount, uint *h_bucketCount, int numBuckets, const uint *kVals,
                   int numKs, uint *sums, uint *markedBuckets, int numBlocks) {
  const int sumsRowIndex = numBuckets * (numBlocks - 1);
  REF_CALL(cudaMemcpy(h_bucketCount, d_bucketCount + sumsRowIndex, sizeof(uint) * numBuckets,
                      cudaMemcpyDeviceToHost));
  int kBucket = 0;
  uint sum = h_bucketCount[0];
  for (int i = 0; i < numKs; i++) {
    const uint k = kVals[i];
    while ((sum < k) & (kBucket < numBuckets - 1)) {
      kBucket++;
      sum += h_bucketCount[kBucket];
    }
    markedBuckets[i] = kBucket;
    sums[i] = sum - h_bucketCount[kBucket];
  }
  return 0;
}

// phaseOne<T> (:521-833).  kVals: host, k-th smallest, modified in place.
template <class T>
int phase_one(T *d_vector, int length, uint *kVals, int numKs, T *output, int blocks, int threads,
              int numBuckets, int numPivots) {
  // step 1 (:534-547): extrema; a flat vector answers every k
  thrust::device_ptr<T> dev_ptr(d_vector);
  thrust::pair<thrust::device_ptr<T>, thrust::device_ptr<T>> mm =
      thrust::minmax_element(dev_ptr, dev_ptr + length);
  const T minimum = *mm.first;
  const T maximum = *mm.second;
  if (maximum == minimum) {
    for (int i = 0; i < numKs; i++) output[i] = minimum;
    return 1;
  }

  // step 2 (:553-603): launch shape, pivots and slopes, bucket ids, counts
  const int threadsPerBlock = threads;
  const int numBlocks = blocks;
  const int offset = blocks * threads;
  const int sampleSize = 1024;
  std::vector<double> slopes(numPivots - 1);
  std::vector<T> pivots(numPivots);
  double *d_slopes = nullptr;
  T *d_pivots = nullptr;
  uint *d_elementToBucket = nullptr;
  REF_CALL(cudaMalloc(&d_elementToBucket, (size_t)length * sizeof(uint)));
  std::vector<uint> h_bucketCount(numBuckets);
  uint *d_bucketCount = nullptr;
  REF_CALL(cudaMalloc(&d_bucketCount, (size_t)numBlocks * numBuckets * sizeof(uint)));
  uint *d_kVals = nullptr, *d_kIndices = nullptr, *d_uniqueBuckets = nullptr,
       *d_reindexCounter = nullptr;
  std::vector<uint> kthBuckets(numKs), kthBucketScanner(numKs, 0), kIndexStore(numKs),
      uniqueBuckets(numKs), reindexCounter(numKs);
  REF_CALL(cudaMalloc(&d_kVals, numKs * sizeof(uint)));
  REF_CALL(cudaMalloc(&d_kIndices, numKs * sizeof(uint)));
  for (int i = 0; i < numKs; i++) kIndexStore[i] = i;
  uint *kIndices = kIndexStore.data();

  // step 3 (:610-646): sort the k's with their positions; k = n and k = 1
  // are answered by the extrema
  REF_CALL(cudaMemcpy(d_kIndices, kIndices, numKs * sizeof(uint), cudaMemcpyHostToDevice));
  REF_CALL(cudaMemcpy(d_kVals, kVals, numKs * sizeof(uint), cudaMemcpyHostToDevice));
  thrust::device_ptr<uint> kVals_ptr(d_kVals), kIndices_ptr(d_kIndices);
  thrust::sort_by_key(kVals_ptr, kVals_ptr + numKs, kIndices_ptr);
  REF_CALL(cudaMemcpy(kIndices, d_kIndices, numKs * sizeof(uint), cudaMemcpyDeviceToHost));
  REF_CALL(cudaMemcpy(kVals, d_kVals, numKs * sizeof(uint), cudaMemcpyDeviceToHost));
  const int numKsAll = numKs;
  int kMaxIndex = numKs - 1, kOffsetMax = 0;
  while (numKs > 0 && kVals[kMaxIndex] == (uint)length) {
    output[kIndices[numKs - 1]] = maximum;
    numKs--;
    kMaxIndex--;
    kOffsetMax++;
  }
  int kOffsetMin = 0;
  while (numKs > 0 && kVals[0] == 1) {
    output[kIndices[0]] = minimum;
    kIndices++;
    kVals++;
    numKs--;
    kOffsetMin++;
  }
  if (numKs == 0) {  // guard: every k was 1 or n
    cudaFree(d_elementToBucket);
    cudaFree(d_bucketCount);
    cudaFree(d_kVals);
    cudaFree(d_kIndices);
    return 1;
  }

  // step 4 (:651-683): pivots and slopes from a 1024-element sample; an
  // infinite slope (two equal pivots) becomes 0
  REF_CALL(cudaMalloc(&d_slopes, (numPivots - 1) * sizeof(double)));
  REF_CALL(cudaMalloc(&d_pivots, numPivots * sizeof(T)));
  if (generate_pivots<T>(pivots.data(), slopes.data(), d_vector, length, numPivots, sampleSize,
                         numBuckets, minimum, maximum))
    return EXIT_FAILURE;
  for (int i = 0; i < numPivots - 1; i++)
    if (std::isinf(slopes[i])) slopes[i] = 0;
  REF_CALL(cudaMemcpy(d_slopes, slopes.data(), (numPivots - 1) * sizeof(double),
                      cudaMemcpyHostToDevice));
  REF_CALL(cudaMemcpy(d_pivots, pivots.data(), numPivots * sizeof(T), cudaMemcpyHostToDevice));

  // step 5 (:690-704): bucket of every element, per-block counts, their scan
  {
    const unsigned smem = numPivots * sizeof(T) + (numPivots - 1) * sizeof(double) +
                          numBuckets * sizeof(uint);
    int nb = numBuckets, np = numPivots, off = offset, len = length;
    void *a[] = {&d_vector, &len, &nb, &d_slopes, &d_pivots, &np, &d_elementToBucket,
                 &d_bucketCount, &off};
    REF_LAUNCH(g_k.assign[TypeIx<T>::v], numBlocks, threadsPerBlock, smem, a);
    int nbl = numBlocks;
    void *b[] = {&d_bucketCount, &nb, &nbl};
    REF_LAUNCH(g_k.sum_counts, numBuckets / threadsPerBlock, threadsPerBlock, 0, b);
  }

  // step 6 (:711-716): the bucket of every k
  if (find_k_buckets(d_bucketCount, h_bucketCount.data(), numBuckets, kVals, numKs,
                     kthBucketScanner.data(), kthBuckets.data(), numBlocks))
    return EXIT_FAILURE;

  // step 7 (:718-756): distinct k buckets, their offsets in the reduced
  // vector, and each k's rank inside it
  uniqueBuckets[0] = kthBuckets[0];
  reindexCounter[0] = 0;
  int numUniqueBuckets = 1;
  kVals[0] -= kthBucketScanner[0];
  for (int i = 1; i < numKs; i++) {
    if (kthBuckets[i] != kthBuckets[i - 1]) {
      uniqueBuckets[numUniqueBuckets] = kthBuckets[i];
      reindexCounter[numUniqueBuckets] =
          reindexCounter[numUniqueBuckets - 1] + h_bucketCount[kthBuckets[i - 1]];
      numUniqueBuckets++;
    }
    kVals[i] = reindexCounter[numUniqueBuckets - 1] + kVals[i] - kthBucketScanner[i];
  }
  const int newInputLength =
      reindexCounter[numUniqueBuckets - 1] + h_bucketCount[kthBuckets[numKs - 1]];
  REF_CALL(cudaMalloc(&d_reindexCounter, numUniqueBuckets * sizeof(uint)));
  REF_CALL(cudaMalloc(&d_uniqueBuckets, numUniqueBuckets * sizeof(uint)));
  REF_CALL(cudaMemcpy(d_reindexCounter, reindexCounter.data(), numUniqueBuckets * sizeof(uint),
                      cudaMemcpyHostToDevice));
  REF_CALL(cudaMemcpy(d_uniqueBuckets, uniqueBuckets.data(), numUniqueBuckets * sizeof(uint),
                      cudaMemcpyHostToDevice));
  {
    int nb = numBuckets, nbl = numBlocks, nu = numUniqueBuckets;
    void *a[] = {&d_bucketCount, &nb, &nbl, &d_reindexCounter, &d_uniqueBuckets, &nu};
    REF_LAUNCH(g_k.reindex_counts, (unsigned)std::ceil((float)numUniqueBuckets / threadsPerBlock),
               threadsPerBlock, 0, a);
  }

  // step 7, copy (:763-783): the k buckets' elements into a new vector
  T *newInput = nullptr;
  REF_CALL(cudaMalloc(&newInput, (size_t)newInputLength * sizeof(T)));
  {
    int len = length, nu = numUniqueBuckets, nb = numBuckets;
    uint off = (uint)offset;
    void *a[] = {&d_vector, &len, &d_elementToBucket, &d_uniqueBuckets, &nu,
                 &newInput, &off, &d_bucketCount, &nb};
    REF_LAUNCH(g_k.copy_elements[TypeIx<T>::v], numBlocks, threadsPerBlock,
               numUniqueBuckets * sizeof(uint), a);
  }

  // step 8 (:790-830): sort the reduced vector and read every k from it
  cudaFree(d_pivots);
  cudaFree(d_slopes);
  cudaFree(d_bucketCount);
  cudaFree(d_uniqueBuckets);
  cudaFree(d_reindexCounter);
  thrust::device_ptr<T> newInput_ptr(newInput);
  thrust::sort(newInput_ptr, newInput_ptr + newInputLength);
  T *d_output = (T *)d_elementToBucket;
  REF_CALL(cudaMemcpy(d_output, output, (numKs + kOffsetMin + kOffsetMax) * sizeof(T),
                      cudaMemcpyHostToDevice));
  REF_CALL(cudaMemcpy(d_kVals, kVals, numKs * sizeof(uint), cudaMemcpyHostToDevice));
  REF_CALL(cudaMemcpy(d_kIndices, kIndices, numKs * sizeof(uint), cudaMemcpyHostToDevice));
  {
    int nk = numKs;
    void *a[] = {&d_output, &newInput, &d_kVals, &d_kIndices, &nk};
    REF_LAUNCH(g_k.copy_values[TypeIx<T>::v], numBlocks, threadsPerBlock, 0, a);
  }
  REF_CALL(cudaMemcpy(output, d_output, (numKs + kOffsetMin + kOffsetMax) * sizeof(T),
                      cudaMemcpyDeviceToHost));
  (void)numKsAll;
  cudaFree(d_elementToBucket);
  cudaFree(d_kIndices);
  cudaFree(d_kVals);
  cudaFree(newInput);
  return 1;
}

// bucketMultiselectWrapper<T> (:837-871): k-th largest -> k-th smallest;
// 8192 buckets, 17 pivots
template <class T>
int wrapper(T *d_vector, int length, const uint *kVals_ori, int numKs, T *outputs, int blocks,
            int threads) {
  std::vector<uint> kVals(numKs);
  for (int i = 0; i < numKs; i++) kVals[i] = length - kVals_ori[i] + 1;
  return phase_one(d_vector, length, kVals.data(), numKs, outputs, blocks, threads, 8192, 17);
}

int device_shape(int *sms, int *max_threads) {
  cudaDeviceProp dp;
  if (cudaGetDeviceProperties(&dp, 0) != cudaSuccess) return -1;
  *sms = dp.multiProcessorCount;
  *max_threads = dp.maxThreadsPerBlock;
  return 0;
}

// setupForTiming (multiselectTimingFunctions.cu:16-26), with the extra
// element described at the top of this file
template <class T>
T *upload_padded(const T *h_vec, uint n) {
  T *d = nullptr;
  if (cudaMalloc(&d, ((size_t)n + 1) * sizeof(T)) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, h_vec, (size_t)n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d + n, h_vec, sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  return d;
}

struct EventTimer {
  cudaEvent_t a{}, b{};
  EventTimer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, 0);
  }
  float stop() {
    float ms = -1.f;
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~EventTimer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

// timeBucketMultiselect<T> (:100-122)
template <class T>
float time_bucket_multiselect(const T *h_vec, uint n, const uint *k, uint nk, T *out) {
  int sms = 0, mt = 0;
  if (device_shape(&sms, &mt)) return -1.f;
  T *d = upload_padded(h_vec, n);
  if (!d) return -1.f;
  float ms;
  {
    EventTimer t;
    const int rc = wrapper(d, (int)n, k, (int)nk, out, sms, mt);
    ms = t.stop();
    if (rc != 1) ms = -1.f;
  }
  cudaFree(d);
  return ms;
}

// timeBucketTopkselect<T> (:205-231): k = 1..K
template <class T>
float time_bucket_topk(const T *h_vec, uint n, uint K, T *out) {
  std::vector<uint> ks(K);
  for (uint i = 0; i < K; i++) ks[i] = i + 1;
  return time_bucket_multiselect(h_vec, n, ks.data(), K, out);
}

// timeSortAndChooseMultiselect<T> (:51-95)
template <class T>
float time_sort_choose_multiselect(const T *h_vec, uint n, const uint *k, uint nk, T *out) {
  T *d = upload_padded(h_vec, n);
  if (!d) return -1.f;
  float ms;
  {
    EventTimer t;
    thrust::device_ptr<T> p(d);
    thrust::sort(p, p + n);
    T *d_output = nullptr;
    uint *d_kList = nullptr;
    cudaMalloc(&d_output, nk * sizeof(T));
    cudaMalloc(&d_kList, nk * sizeof(uint));
    cudaMemcpy(d_kList, k, nk * sizeof(uint), cudaMemcpyHostToDevice);
    int threads = kMaxThreadsPerBlock;
    if ((int)nk < threads) threads = (int)nk;
    const int blocks = (int)std::ceil(nk / (float)threads);
    uint cnt = nk, ne = n;
    void *a[] = {&d_output, &d, &d_kList, &cnt, &ne};
    const bool ok = launch(g_k.copy_in_chunk[TypeIx<T>::v], blocks, threads, 0, a);
    cudaMemcpy(out, d_output, nk * sizeof(T), cudaMemcpyDeviceToHost);
    cudaFree(d_output);
    cudaFree(d_kList);
    ms = t.stop();
    if (!ok) ms = -1.f;
  }
  cudaFree(d);
  return ms;
}

// timeSortAndChooseTopkselect<T> (:156-177)
template <class T>
float time_sort_choose_topk(const T *h_vec, uint n, uint K, T *out) {
  T *d = upload_padded(h_vec, n);
  if (!d) return -1.f;
  float ms;
  {
    EventTimer t;
    thrust::device_ptr<T> p(d);
    thrust::sort(p, p + n, thrust::greater<T>());
    cudaMemcpy(out, d, K * sizeof(T), cudaMemcpyDeviceToHost);
    ms = t.stop();
  }
  cudaFree(d);
  return ms;
}

}  // namespace

extern "C" {

// Loads the cubin of the reference's kernels into the current device's
// primary context (once per process).  0 on success.
int ggks_refgpu_load(const char *cubin_path) {
  std::lock_guard<std::mutex> g(g_mu);
  if (g_mod) return 0;
  if (cudaFree(0) != cudaSuccess) return -1;  // the runtime's primary context
  if (cuModuleLoad(&g_mod, cubin_path) != CUDA_SUCCESS) {
    g_mod = nullptr;
    return -1;
  }
  const int rc = bind_kernels();
  if (rc) {
    cuModuleUnload(g_mod);
    g_mod = nullptr;
  }
  return rc;
}

int ggks_refgpu_device_shape(int *sms, int *max_threads) { return device_shape(sms, max_threads); }

// bucketMultiselectWrapper<T> on a resident device vector (readable at
// d_vec[n], see the top of this file); k's are k-th largest; the wrapper's
// time under CUDA events on the legacy stream goes to *ms.  Returns 1 (the
// reference's success value) or EXIT_FAILURE.
#define GGKS_REFGPU_ENTRIES(SUF, T)                                                         \
  int ggks_refgpu_bucket_multiselect_##SUF(T *d_vec, int n, const uint *k, int nk, T *out,  \
                                           int blocks, int threads, float *ms) {            \
    EventTimer t;                                                                           \
    const int rc = wrapper(d_vec, n, k, nk, out, blocks, threads);                          \
    const float e = t.stop();                                                               \
    if (ms) *ms = e;                                                                        \
    return rc;                                                                              \
  }                                                                                         \
  float ggks_refgpu_time_bucket_multiselect_##SUF(const T *h, uint n, const uint *k, uint nk, \
                                                  T *out) {                                 \
    return time_bucket_multiselect(h, n, k, nk, out);                                       \
  }                                                                                         \
  float ggks_refgpu_time_bucket_topk_##SUF(const T *h, uint n, uint K, T *out) {            \
    return time_bucket_topk(h, n, K, out);                                                  \
  }                                                                                         \
  float ggks_refgpu_time_sort_choose_multiselect_##SUF(const T *h, uint n, const uint *k,   \
                                                       uint nk, T *out) {                   \
    return time_sort_choose_multiselect(h, n, k, nk, out);                                  \
  }                                                                                         \
  float ggks_refgpu_time_sort_choose_topk_##SUF(const T *h, uint n, uint K, T *out) {       \
    return time_sort_choose_topk(h, n, K, out);                                             \
  }
GGKS_REFGPU_ENTRIES(f32, float)
GGKS_REFGPU_ENTRIES(f64, double)
GGKS_REFGPU_ENTRIES(u32, uint)
#undef GGKS_REFGPU_ENTRIES

}  // extern "C"
