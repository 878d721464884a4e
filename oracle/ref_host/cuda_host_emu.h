// cuda_host_emu.h -- test infrastructure: a host-CPU stand-in for the CUDA
// runtime, so that the reference's own CUDA C++ sources for the bucket
// multiselect path run on the CPU and their outputs pin the oracle.
//
// Used only by oracle/build_ref.py, which force-includes this header ahead of
// the reference's bucketMultiselect.cu and multiselectTimingFunctions.cu,
// rewrites their `kernel<<<grid, block, smem>>>(args)` statements into
// `ggks_host_emu::launch(grid, block, smem, [&]{ kernel(args); })` and their
// `extern __shared__ T name[];` declarations into a pointer to the launch's
// dynamic shared memory, and compiles the result with the host compiler into
// oracle/_ref/libggks_ref.so.  Nothing in the product links this file.
//
// Execution model:
//  * device memory is host memory: cudaMalloc/cudaFree/cudaMemcpy/cudaMemset
//    are malloc/free/memcpy/memset;
//  * Thrust runs on its sequential CPP back end (THRUST_DEVICE_SYSTEM_CPP), so
//    thrust::sort / sort_by_key / minmax_element / transform on device_ptr work
//    on that memory;
//  * a launch runs its blocks one after another; the threads of a block are
//    cooperative fibers (ucontext) that switch only at __syncthreads(), so a
//    block's threads see one shared-memory image and every barrier holds;
//  * atomics are plain read-modify-writes (no two fibers run at once), with
//    CUDA's wrap rules for atomicInc / atomicDec;
//  * `__shared__` variables become function-local statics: blocks never run
//    at the same time, so one instance per kernel is one instance per block.
// The emulated device reports GGKS_EMU_SMS multiprocessors (default 152, a GB300) and
// 1024 threads per block.  The reference's results are exact order statistics
// and do not depend on either figure.
#pragma once

#include <cuda_runtime.h>  // types and declarations only; libcudart is never linked

#include <ucontext.h>
#include <sys/time.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

#undef __global__
#undef __device__
#undef __host__
#undef __shared__
#undef __forceinline__
#define __global__
#define __device__
#define __host__
#define __shared__ static
#define __forceinline__ inline

// Names the reference uses that CUDA 13 / C++17 no longer provide.
#define register
#define cudaThreadSynchronize cudaDeviceSynchronize
#define cudaThreadExit cudaDeviceReset
namespace thrust {
template <typename Arg, typename Result>
struct unary_function {
  typedef Arg argument_type;
  typedef Result result_type;
};
}  // namespace thrust

inline uint3 threadIdx;
inline uint3 blockIdx;
inline dim3 blockDim;
inline dim3 gridDim;

namespace ggks_host_emu {

struct Engine {
  static constexpr size_t kStackBytes = 64 * 1024;
  std::vector<ucontext_t> fiber;
  std::vector<unsigned char> done;
  char* stacks = nullptr;
  size_t nstacks = 0;
  ucontext_t sched;
  unsigned cur = 0;
  const std::function<void()>* body = nullptr;
  std::vector<unsigned char> smem;
};

inline Engine& engine() {
  static Engine e;
  return e;
}

inline void fiber_main() {
  Engine& e = engine();
  (*e.body)();
  e.done[e.cur] = 1;  // returning resumes the scheduler through uc_link
}

inline void* dynamic_shared() { return engine().smem.data(); }

// Runs `body` once per thread of every block of the grid.
inline void launch(dim3 grid, dim3 block, size_t smem_bytes,
                   const std::function<void()>& body) {
  Engine& e = engine();
  const unsigned nt = block.x * block.y * block.z;
  if (nt == 0 || nt > 1024) {
    std::fprintf(stderr, "ggks_host_emu: bad block size %u\n", nt);
    std::abort();
  }
  if (e.nstacks < nt) {
    std::free(e.stacks);
    e.stacks = static_cast<char*>(std::malloc(nt * Engine::kStackBytes));
    if (!e.stacks) std::abort();
    e.nstacks = nt;
  }
  e.fiber.resize(nt);
  e.done.assign(nt, 0);
  // Dynamic shared memory starts as a fixed non-zero pattern: the reference
  // must initialise what it reads, as on a GPU.
  e.smem.assign(smem_bytes + 16, 0xA5);
  e.body = &body;
  gridDim = grid;
  blockDim = block;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = make_uint3(bx, by, bz);
        for (unsigned t = 0; t < nt; ++t) {
          getcontext(&e.fiber[t]);
          e.fiber[t].uc_stack.ss_sp = e.stacks + size_t(t) * Engine::kStackBytes;
          e.fiber[t].uc_stack.ss_size = Engine::kStackBytes;
          e.fiber[t].uc_link = &e.sched;
          makecontext(&e.fiber[t], fiber_main, 0);
          e.done[t] = 0;
        }
        // One round resumes every live thread until it reaches the next
        // barrier or returns; rounds repeat until all have returned.
        for (;;) {
          bool live = false;
          for (unsigned t = 0; t < nt; ++t) {
            if (e.done[t]) continue;
            e.cur = t;
            threadIdx = make_uint3(t % block.x, (t / block.x) % block.y,
                                   t / (block.x * block.y));
            swapcontext(&e.sched, &e.fiber[t]);
            if (!e.done[t]) live = true;
          }
          if (!live) break;
        }
      }
  e.body = nullptr;
}

}  // namespace ggks_host_emu

inline void __syncthreads() {
  ggks_host_emu::Engine& e = ggks_host_emu::engine();
  swapcontext(&e.fiber[e.cur], &e.sched);
}
#define syncthreads __syncthreads

inline unsigned int atomicInc(unsigned int* a, unsigned int v) {
  unsigned int old = *a;
  *a = (old >= v) ? 0u : old + 1u;
  return old;
}
inline unsigned int atomicDec(unsigned int* a, unsigned int v) {
  unsigned int old = *a;
  *a = (old == 0u || old > v) ? v : old - 1u;
  return old;
}
inline unsigned int atomicAdd(unsigned int* a, unsigned int v) {
  unsigned int old = *a;
  *a = old + v;
  return old;
}
inline int atomicAdd(int* a, int v) {
  int old = *a;
  *a = old + v;
  return old;
}

// ---- runtime entry points the reference calls (C linkage, as declared) ----

cudaError_t CUDARTAPI cudaMalloc(void** p, size_t n) {
  *p = std::malloc(n ? n : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t CUDARTAPI cudaFree(void* p) {
  std::free(p);
  return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemcpy(void* d, const void* s, size_t n, enum cudaMemcpyKind) {
  if (n) std::memmove(d, s, n);
  return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemset(void* d, int v, size_t n) {
  std::memset(d, v, n);
  return cudaSuccess;
}
cudaError_t CUDARTAPI cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaDeviceReset(void) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaGetDeviceProperties(struct cudaDeviceProp* p, int) {
  std::memset(p, 0, sizeof(*p));
  const char* s = std::getenv("GGKS_EMU_SMS");
  p->multiProcessorCount = (s && std::atoi(s) > 0) ? std::atoi(s) : 152;
  p->maxThreadsPerBlock = 1024;
  p->warpSize = 32;
  return cudaSuccess;
}
cudaError_t CUDARTAPI cudaEventCreate(cudaEvent_t* e) {
  *e = reinterpret_cast<cudaEvent_t>(new double(0.0));
  return cudaSuccess;
}
cudaError_t CUDARTAPI cudaEventRecord(cudaEvent_t e, cudaStream_t) {
  using clk = std::chrono::steady_clock;
  *reinterpret_cast<double*>(e) =
      std::chrono::duration<double, std::milli>(clk::now().time_since_epoch()).count();
  return cudaSuccess;
}
cudaError_t CUDARTAPI cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
  *ms = float(*reinterpret_cast<double*>(b) - *reinterpret_cast<double*>(a));
  return cudaSuccess;
}
cudaError_t CUDARTAPI cudaEventDestroy(cudaEvent_t e) {
  delete reinterpret_cast<double*>(e);
  return cudaSuccess;
}
