// ref_kernels.cu -- test and measurement infrastructure: the reference's own
// device kernels for its bucket multiselect path, compiled for sm_103a into
// oracle/_ref/ref_kernels.cubin by oracle/ref_gpu.py.  Nothing of the product
// links or loads it.
//
// The reference's sources are read where they lie (their paths come in as
// GGKS_REF_BUCKET_MULTISELECT / GGKS_REF_TIMING_FUNCTIONS; the reference
// directory is not put on the include path, where its vendored Thrust 1.4.0
// would shadow CUDA's; nothing is copied into this tree):
//   bucketMultiselect.cu           assignSmartBucket<T>      (:129-205)
//                                  sumCounts                 (:214-221)
//                                  reindexCounts             (:228-241)
//                                  copyElements<T>           (:249-308)
//                                  copyValuesInChunk<T>      (:315-325)
//                                  enlargeIndexAndGetElements (:402-405, :401-
//                                    as the template at :395-399)
//                                  RandomNumberFunctor       (:350-369)
//   multiselectTimingFunctions.cu  copyInChunk<T>            (:41-48)
// Every kernel template the reference's host code launches is instantiated
// below for the element types the reference's harness uses (float, double,
// uint).  The one device-side step that the reference runs through a Thrust
// algorithm with its own functor -- createRandomVector (:374-386):
// thrust::transform of counting indices through RandomNumberFunctor(seed) --
// is the kernel ggks_ref_random_vector_*, which applies the same functor to
// each index (out[i] = (T) RandomNumberFunctor(seed)(i)).  The host side of
// the path (phaseOne, generatePivots, the wrapper and the timing adapters) is
// restated in ref_gpu_host.cu, which loads this cubin and launches these
// kernels in the reference's order.
#include "ref_gpu_shim.h"

// the includes the reference's harness puts before these sources
// (compareMultiselect.hpp:8-24)
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>
#include <time.h>

#include <algorithm>
#include <thrust/device_ptr.h>
#include <thrust/extrema.h>
#include <thrust/functional.h>
#include <thrust/pair.h>
#include <thrust/random.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/transform_reduce.h>

#include GGKS_REF_BUCKET_MULTISELECT
#include GGKS_REF_TIMING_FUNCTIONS

namespace BucketMultiselect {
#define GGKS_REF_KERNELS(T)                                                                   \
  template __global__ void assignSmartBucket<T>(T *, int, int, double *, T *, int, uint *,   \
                                                uint *, int);                                 \
  template __global__ void copyElements<T>(T *, int, uint *, uint *, const int, T *, uint,   \
                                           uint *, int);                                      \
  template __global__ void copyValuesInChunk<T>(T *, T *, uint *, uint *, int);
GGKS_REF_KERNELS(float)
GGKS_REF_KERNELS(double)
GGKS_REF_KERNELS(uint)
#undef GGKS_REF_KERNELS
// generatePivots<float/double> (:460-508) gathers its sample with the template;
// generatePivots for uint (:414-457) with the non-template overload (:402-405)
template __global__ void enlargeIndexAndGetElements<float>(float *, float *, int);
template __global__ void enlargeIndexAndGetElements<double>(double *, double *, int);
}  // namespace BucketMultiselect

template __global__ void copyInChunk<float>(float *, float *, uint *, uint, uint);
template __global__ void copyInChunk<double>(double *, double *, uint *, uint, uint);
template __global__ void copyInChunk<uint>(uint *, uint *, uint *, uint, uint);

// createRandomVector<T> (bucketMultiselect.cu:374-386): one value per index.
// The functor travels by value, as thrust::transform passes it to its kernel
// (its constructor is host code); the host driver passes its one field, the
// seed.
static_assert(sizeof(BucketMultiselect::RandomNumberFunctor) == sizeof(unsigned),
              "RandomNumberFunctor is passed as its seed");
extern "C" __global__ void ggks_ref_random_vector_f32(float *out, int size,
                                                      BucketMultiselect::RandomNumberFunctor f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < size) out[i] = f((unsigned)i);
}
extern "C" __global__ void ggks_ref_random_vector_f64(double *out, int size,
                                                      BucketMultiselect::RandomNumberFunctor f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < size) out[i] = (double)f((unsigned)i);
}
