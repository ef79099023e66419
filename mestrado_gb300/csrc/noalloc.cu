// noalloc.cu -- pair scoring that allocates nothing.
//
// Some hosts cannot let a library call cudaMalloc or cudaFree: code that runs
// while a CUDA stream is being captured in the global capture mode (where
// those calls are not permitted), and hosts that hand out all device memory
// from their own pool and must not have a cudaFree synchronize the device
// underneath them.  nwg_score_pairs_noalloc serves them: the caller passes
// every input and output as device memory, and the only work memory -- the
// per-pair (H, F) row kept between 16-row strips, the same scratch the
// one-thread-per-pair kernel keeps in a buffer of its context -- is a
// file-scope static device array of kNoallocScratchBytes (32 MiB), which every
// GPU that loads this library holds until the process exits.  No context is
// created, so no context buffer is allocated either.
//
// Set-up: the first call on a device (with that device current) looks the
// array up with cudaGetSymbolAddress once and keeps the address for that
// device; make that first call before any stream capture begins.  The
// address is kept for the life of the process, so a device reset after the
// first call (which reloads the module) is not supported.
//
// Sharing: every call on a device uses the same array and it keeps the last
// call's contents.  Nothing in it has to start at zero: each pair writes the
// part of the row it reads before reading it.  Calls whose kernels overlap on
// the GPU (two streams, or two host threads) race on the array: serialize them.
#include <climits>
#include <mutex>

#include "nwg_matrix.h"
#include "wave_impl.cuh"

namespace nwg {
namespace {

constexpr size_t kNoallocScratchBytes = size_t(32) << 20;
constexpr int64_t kNoallocScratchCells = (int64_t)(kNoallocScratchBytes / sizeof(int2));
constexpr int kNoallocThreads = 128;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) int2 g_noalloc_scratch[kNoallocScratchCells];

// the built-in matrix (blosum64.txt / definitions.cuh:96-121, BLOSUM62 values)
// in static device memory, used when the caller passes no matrix
static __device__ int8_t g_noalloc_sub[kLetters * kLetters] = {NWG_BLOSUM64_VALUES};

struct DeviceSetup {
  std::mutex mu;
  bool done[kMaxDevices] = {};
  int2* scratch[kMaxDevices] = {};
  int8_t* sub[kMaxDevices] = {};
};

DeviceSetup& setup_state() {
  static DeviceSetup s;
  return s;
}

// One pair per thread through the plain form's per-thread scorer (int32,
// 16-row register strip, NeedlemanWunsch.cu:22-161 with the strips widened to
// 16 rows); the (H, F) row between strips lives in the static array at stride
// `stride`.  A thread scores pairs k, k + stride, ... in turn and reuses its
// column of the array for each.
__global__ void __launch_bounds__(kNoallocThreads)
noalloc_pairs_kernel(const int8_t* __restrict__ codes, const int64_t* __restrict__ start,
                     const int32_t* __restrict__ len, const int32_t* __restrict__ pi,
                     const int32_t* __restrict__ pj, int64_t npairs, int32_t* __restrict__ out, int max_len,
                     int go, int ge, const int8_t* __restrict__ sub, int2* __restrict__ scratch, int64_t stride) {
  __shared__ int8_t s_sub[kLetters * kLetters];
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = sub[e];
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int2* sc = scratch + t;
  for (int64_t k = t; k < npairs; k += stride) {
    const int i = pi[k], j = pj[k];
    const int Lx = len[i], Ly = len[j];
    if (Lx < 1 || Ly < 1 || Lx > max_len) {   // outside what the caller declared: no scratch access
      out[k] = INT_MIN;
      continue;
    }
    out[k] = wave::score_thread(codes + start[i], Lx, codes + start[j], Ly, go, ge, s_sub, sc, stride);
  }
}

}  // namespace
}  // namespace nwg

extern "C" int nwg_score_pairs_noalloc(const int8_t* d_codes, const int64_t* d_start, const int32_t* d_len,
                                       const int32_t* d_pi, const int32_t* d_pj, int64_t npairs, int32_t* d_out,
                                       int max_len, int gap_open, int gap_ext, const int8_t* d_sub, void* stream) {
  using namespace nwg;
  if (npairs < 0 || gap_open < 0 || gap_ext < 0 || gap_open > 1000 || gap_ext > 1000) return NWG_ERR_INVALID;
  // the static array holds the (H, F) row of 128 concurrent pairs at the least
  if (max_len < 1 || (int64_t)max_len * kNoallocThreads > kNoallocScratchCells) return NWG_ERR_INVALID;
  if (npairs == 0) return NWG_OK;
  if (!d_codes || !d_start || !d_len || !d_pi || !d_pj || !d_out) return NWG_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return NWG_ERR_NO_DEVICE;
  }
  DeviceSetup& S = setup_state();
  int2* scratch = nullptr;
  int8_t* builtin = nullptr;
  {
    std::lock_guard<std::mutex> lock(S.mu);
    if (!S.done[dev]) {
      void* p = nullptr;
      void* q = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess ||
          cudaGetSymbolAddress(&q, g_noalloc_sub) != cudaSuccess) {
        cudaGetLastError();
        return NWG_ERR_CUDA;
      }
      S.scratch[dev] = (int2*)p;
      S.sub[dev] = (int8_t*)q;
      S.done[dev] = true;
    }
    scratch = S.scratch[dev];
    builtin = S.sub[dev];
  }
  // threads: as many rows of max_len as the array holds, a multiple of the
  // block size, no more than the pairs need
  int64_t threads = kNoallocScratchCells / max_len;
  threads = threads / kNoallocThreads * kNoallocThreads;
  const int64_t need = (npairs + kNoallocThreads - 1) / kNoallocThreads * kNoallocThreads;
  if (threads > need) threads = need;
  const int64_t blocks = threads / kNoallocThreads;
  noalloc_pairs_kernel<<<(unsigned)blocks, kNoallocThreads, 0, (cudaStream_t)stream>>>(
      d_codes, d_start, d_len, d_pi, d_pj, npairs, d_out, max_len, gap_open, gap_ext, d_sub ? d_sub : builtin,
      scratch, threads);
  return cudaGetLastError() == cudaSuccess ? NWG_OK : NWG_ERR_CUDA;
}
