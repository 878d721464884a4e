// ggks_noalloc.cu -- a float32 multiselect that allocates no memory.
//
// Who needs it: callers that may not allocate device memory when they
// select -- an engine or framework whose device memory all belongs to its own
// allocator, which budgets every byte (a cudaMalloc behind its back can
// exhaust the device or break that accounting), and latency-bound loops where
// an allocation would stall on the driver.  The regular entry points grow a
// per-context workspace and pinned staging with cudaMalloc / cudaHostAlloc;
// this one does not.
//
// How: all scratch lives in one file-scope __device__ array of fixed size
// (kNaScratchBytes, about 11 MB), which every GPU that loads this library
// holds until the process exits.  The caller passes the input vector, the k
// list and the output array, all in device memory, and a stream.  Sizes are
// capped (n <= GGKS_NOALLOC_MAX_N, num_k <= GGKS_NOALLOC_MAX_K); larger
// requests are rejected with GGKS_INVALID_ARG.
//
// The array's name is only a host-side stand-in for the device symbol; its
// device address comes from cudaGetSymbolAddress, called once per device with
// that device current on the first call there, which also sets the kernels'
// shared-memory limits on that device (so the first call on a device must
// come before any stream capture).  Every call shares the one array, which
// keeps the last call's contents; each call clears the control block and the
// slice counts, the only parts that must start at zero.  Calls whose work
// overlaps on the GPU (different streams, or several host threads) race and
// must be serialised by the caller.
#include <mutex>

#include "ggks_pipeline.cuh"

namespace ggks {
namespace {

constexpr uint64_t kNaMaxN = GGKS_NOALLOC_MAX_N;
constexpr uint32_t kNaMaxK = GGKS_NOALLOC_MAX_K;
constexpr uint32_t kNaNbMax = 8192;  // buckets: keeps the per-CTA rows small
constexpr uint32_t kNaMaxG = 64;     // histogram / compaction CTAs
constexpr uint32_t kNaS = 65536;     // sample size

constexpr size_t na_align(size_t v) { return (v + 255) / 256 * 256; }
// scratch layout (byte offsets); the control block and the slice counts are
// zeroed together at the start of each call
constexpr size_t kNaCtrl = 0;
constexpr size_t kNaSliceCnt = na_align(kNaCtrl + sizeof(Ctrl));
constexpr size_t kNaReqs = na_align(kNaSliceCnt + kSliceCntBytes);
constexpr size_t kNaHdr = na_align(kNaReqs + kNaMaxK * sizeof(Req));
constexpr size_t kNaLut = na_align(kNaHdr + sizeof(LutHeader<uint32_t>));
constexpr size_t kNaSamples = na_align(kNaLut + kLutPadded * sizeof(uint32_t));
constexpr size_t kNaPartials = na_align(kNaSamples + kNaS * sizeof(uint32_t));
constexpr size_t kNaCounts = na_align(kNaPartials + (size_t)kNaMaxG * kNaNbMax * 4);
constexpr size_t kNaTtot = na_align(kNaCounts + kNaNbMax * 4);
constexpr size_t kNaSegBucket = na_align(kNaTtot + kNaNbMax / kScanTile * 4);
constexpr size_t kNaSegOff = na_align(kNaSegBucket + kNaNbMax * 4);
constexpr size_t kNaSegSize = na_align(kNaSegOff + kNaNbMax * 8);
constexpr size_t kNaKstart = na_align(kNaSegSize + kNaNbMax * 4);
constexpr size_t kNaKcnt = na_align(kNaKstart + kNaNbMax * 4);
constexpr size_t kNaKcur = na_align(kNaKcnt + kNaNbMax * 4);
constexpr size_t kNaFill = na_align(kNaKcur + kNaNbMax * 4);
constexpr size_t kNaSegLo = na_align(kNaFill + kNaNbMax * 4);
constexpr size_t kNaSegHi = na_align(kNaSegLo + kNaNbMax * 4);
constexpr size_t kNaDeferred = na_align(kNaSegHi + kNaNbMax * 4);
constexpr size_t kNaReqBucket = na_align(kNaDeferred + kNaNbMax * 4);
constexpr size_t kNaReqLocal = na_align(kNaReqBucket + kNaMaxK * 4);
constexpr size_t kNaKlist = na_align(kNaReqLocal + kNaMaxK * 4);
constexpr size_t kNaSurv = na_align(kNaKlist + kNaMaxK * sizeof(Req));
constexpr size_t kNaScratchBytes = na_align(kNaSurv + kNaMaxN * sizeof(uint32_t));

// the scratch itself (device memory reserved at module load)
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

std::mutex g_na_mu;
char *g_na_base[64];  // device address of g_noalloc_scratch per device

// k list (k-th largest) -> requests; a k outside [1, n] is reported and
// replaced by 1 so that every later index stays in range
__global__ void k_na_reqs(const uint32_t *__restrict__ k, uint32_t num_k, uint64_t n, Req *reqs,
                          Ctrl *ctrl) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_k) return;
  uint32_t kk = k[i];
  if (kk < 1 || (uint64_t)kk > n) {
    atomicOr(&ctrl->status, ST_BAD_K);
    kk = 1;
  }
  Req r;
  r.rank = (uint32_t)(n - kk);
  r.out = i;
  reqs[i] = r;
}

// device address of the scratch on the current device (set up on first use)
int scratch_base(char **base) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return from_cuda(e);
  if (dev < 0 || dev >= 64) return GGKS_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_base[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return e != cudaSuccess ? from_cuda(e) : GGKS_CUDA_ERROR;
    g_na_base[dev] = static_cast<char *>(p);
  }
  *base = g_na_base[dev];
  return GGKS_OK;
}

}  // namespace
}  // namespace ggks

using namespace ggks;

extern "C" int ggks_multiselect_noalloc_f32(const float *d_vec, uint64_t n, const uint32_t *d_k,
                                            uint32_t num_k, float *d_out, void *stream) {
  using K = uint32_t;
  constexpr int UNROLL = 4;
  if (!d_vec || !d_k || !d_out || n == 0 || n > kNaMaxN || num_k == 0 || num_k > kNaMaxK)
    return GGKS_INVALID_ARG;
  if ((uintptr_t)d_vec % sizeof(float) != 0) return GGKS_INVALID_ARG;
  char *A = nullptr;
  int st = scratch_base(&A);
  if (st != GGKS_OK) return st;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return from_cuda(e);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  Ctrl *ctrl = reinterpret_cast<Ctrl *>(A + kNaCtrl);
  Req *reqs = reinterpret_cast<Req *>(A + kNaReqs);
  LutHeader<K> *hdr = reinterpret_cast<LutHeader<K> *>(A + kNaHdr);
  uint32_t *lut = reinterpret_cast<uint32_t *>(A + kNaLut);
  K *samples = reinterpret_cast<K *>(A + kNaSamples);
  uint32_t *partials = reinterpret_cast<uint32_t *>(A + kNaPartials);
  uint32_t *bpre = reinterpret_cast<uint32_t *>(A + kNaCounts);  // prefix inside 64-bucket tiles
  uint32_t *ttot = reinterpret_cast<uint32_t *>(A + kNaTtot);
  uint32_t *seg_bucket = reinterpret_cast<uint32_t *>(A + kNaSegBucket);
  uint64_t *seg_off = reinterpret_cast<uint64_t *>(A + kNaSegOff);
  uint32_t *seg_size = reinterpret_cast<uint32_t *>(A + kNaSegSize);
  uint32_t *kstart = reinterpret_cast<uint32_t *>(A + kNaKstart);
  uint32_t *kcnt = reinterpret_cast<uint32_t *>(A + kNaKcnt);
  uint32_t *kcur = reinterpret_cast<uint32_t *>(A + kNaKcur);
  uint32_t *fill = reinterpret_cast<uint32_t *>(A + kNaFill);
  K *seg_lo = reinterpret_cast<K *>(A + kNaSegLo);
  K *seg_hi = reinterpret_cast<K *>(A + kNaSegHi);
  uint32_t *deferred = reinterpret_cast<uint32_t *>(A + kNaDeferred);
  uint32_t *req_bucket = reinterpret_cast<uint32_t *>(A + kNaReqBucket);
  uint32_t *req_local = reinterpret_cast<uint32_t *>(A + kNaReqLocal);
  Req *klist = reinterpret_cast<Req *>(A + kNaKlist);
  K *surv = reinterpret_cast<K *>(A + kNaSurv);

  // launch shapes for this n (the survivor area holds n keys: no overflow)
  const uint32_t S = n <= kNaS ? (uint32_t)n : kNaS;
  uint64_t g = (n + 65535) / 65536;
  const uint32_t G = (uint32_t)(g < 1 ? 1 : (g > kNaMaxG ? kNaMaxG : (g > (uint64_t)sms ? sms : g)));
  const uint32_t col_tiles = (kNaNbMax + kScanTile - 1) / kScanTile;
  const uint32_t cap_keys = cap_keys_for<float>();
  const uint32_t fg = 5u * (uint32_t)sms;
  const uint32_t fin_grid = num_k < fg ? num_k : fg;

  // the kernels' shared-memory limits on this device (set on its first call)
  e = set_smem_max<k_hist<float, UNROLL>>((int)(kRepWords * sizeof(uint32_t) + (size_t)kMaxNb * 4));
  if (e == cudaSuccess) e = set_smem_max<k_plan<float, float>>(kPlanSmemMax);
  if (e == cudaSuccess)
    e = set_smem_max<k_compact<float, UNROLL>>((int)compact_smem_bytes(kMaxNb));
  if (e == cudaSuccess) e = set_smem_max<k_finish<K, float>>(finish_smem_bytes<float>());
  if (e != cudaSuccess) return from_cuda(e);

  // the control block and the slice counts start at zero
  e = cudaMemsetAsync(A + kNaCtrl, 0, kNaSliceCnt + kSliceCntBytes, s);
  if (e != cudaSuccess) return from_cuda(e);
  k_na_reqs<<<(num_k + 255) / 256, 256, 0, s>>>(d_k, num_k, n, reqs, ctrl);
  k_sample<float><<<(S + 1023) / 1024, 1024, 0, s>>>(d_vec, n, S, 0x5EEDu, samples, ctrl);
  k_lut<K><<<(S + 1023) / 1024, 1024, 0, s>>>(samples, S, ctrl, hdr, lut, kNaNbMax,
                                               reinterpret_cast<uint32_t *>(A + kNaSliceCnt), n,
                                               0u, G);
  {
    const int smem = (int)(kRepWords * sizeof(uint32_t) + (size_t)kNaNbMax * 4);
    k_hist<float, UNROLL><<<G, 1024, smem, s>>>(d_vec, n, hdr, lut, partials, kNaNbMax, ctrl,
                                                nullptr, nullptr, nullptr, nullptr, nullptr,
                                                nullptr);
  }
  k_colsum<K><<<col_tiles, kScanThreads, 0, s>>>(partials, G, kNaNbMax, hdr, bpre, ttot, ctrl,
                                                  nullptr, nullptr, nullptr);
  {
    const int smem = (int)(kLutPadded * sizeof(uint32_t) + (size_t)kNaNbMax * 5);
    k_plan<float, float><<<1, 1024, smem, s>>>(hdr, lut, bpre, ttot, n, reqs, num_k, kNaNbMax,
                                                ctrl, seg_bucket, seg_off,
                                                seg_size, kstart, kcnt, kcur, fill, seg_lo, seg_hi,
                                                req_bucket, req_local, klist, n, Premap{});
  }
  {
    const int smem = (int)compact_smem_bytes(kNaNbMax);
    k_compact<float, UNROLL><<<G, 1024, smem, s>>>(d_vec, n, hdr, lut, seg_bucket, seg_off,
                                                   seg_size, partials, fill, kNaNbMax, surv, n,
                                                   ctrl, nullptr, nullptr, nullptr, 0);
  }
  {
    const int smem = finish_smem_bytes<float>();
    k_finish<K, float><<<fin_grid, kFinThreads, smem, s>>>(surv, ctrl, seg_off, seg_size, seg_lo,
                                                          seg_hi, kstart, kcnt, klist, deferred,
                                                          cap_keys, d_out);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return from_cuda(e);
  Ctrl h;  // host copy of the control block (stack memory)
  e = cudaMemcpyAsync(&h, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return from_cuda(e);
  if (h.status & ST_BAD_K) return GGKS_INVALID_ARG;
  if (h.status & ST_TIMEOUT) return GGKS_TIMEOUT;
  if (h.status & (ST_INTERNAL | ST_OVERFLOW)) return GGKS_INTERNAL;
  // a segment whose needed keys exceed a finishing CTA's shared memory needs a
  // recursive level with its own workspace, which this entry point does not have
  if (h.status & ST_DEFERRED) return GGKS_UNSUPPORTED;
  return GGKS_OK;
}
