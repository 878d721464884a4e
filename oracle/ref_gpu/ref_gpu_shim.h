// ref_gpu_shim.h -- force-included before the reference's sources when they
// are compiled for sm_103a (oracle/ref_gpu/ref_kernels.cu): the names they use
// that CUDA 13 and C++17 no longer provide, and nothing else.
#pragma once
#include <cuda_runtime.h>
#include <thrust/functional.h>

#define register
#define cudaThreadSynchronize cudaDeviceSynchronize
#define cudaThreadExit cudaDeviceReset
#define syncthreads __syncthreads

namespace thrust {
template <typename Arg, typename Result>
struct unary_function {
  typedef Arg argument_type;
  typedef Result result_type;
};
}  // namespace thrust
