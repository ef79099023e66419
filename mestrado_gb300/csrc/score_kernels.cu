// score_kernels.cu -- sm_103a Needleman-Wunsch (Gotoh) score kernels.
//
// Recurrence of NeedlemanWunschGlobalScoreKernel (NeedlemanWunsch.cu:22-161)
// over reversed 8-bit residue codes, X = columns, Y = rows:
//   H[-1][-1] = 0, H[-1][c] = -ge(c+1), H[r][-1] = -ge(r+1)       (:65-70,:89,:94-99)
//   F[-1][c] = E[r][-1] = -32768+ge                                (:68,:97)
//   F[r][c] = max(F[r-1][c]-ge, H[r-1][c]-go)                      (:142)
//   E[r][c] = max(E[r][c-1]-ge, H[r][c-1]-go)                      (:143)
//   H[r][c] = max(E, F, H[r-1][c-1] + S[y_r][x_c])                 (:145-146)
//   score   = H[Ly-1][Lx-1]                                        (:160)
//
// This file holds the per-thread forms and the dispatch of the batched form
// (whose kernel lives in wave_impl.cuh, one translation unit per template):
//  * plain_kernel: the reference's launch model on sm_103a -- one thread per
//    pair, int32, a 16-row register strip, the per-column (H, F) boundary in
//    global scratch, one launch per length group.  It is the baseline the
//    batched form is measured against.
//  * rerun_kernel: int32 re-run of the pairs the int16 overflow guard queued.
//  * pairlist_kernel: explicit pair lists.
//  * dpx_peak_kernel: the roofline denominator (cell update only).
#include "wave_impl.cuh"

namespace nwg {
namespace {

using wave::Lanes;
using wave::clamp_code;
using wave::put_score;
using wave::score_thread;

// ---- plain form ------------------------------------------------------------

__global__ void __launch_bounds__(kPlainThreads) plain_kernel(const PlainArgs a) {
  __shared__ int8_t s_sub[kLetters * kLetters];
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = a.sub[e];
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.nthreads) return;
  int lo = 0, hi = a.ny_launch - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.y_prefix[mid] <= t) lo = mid; else hi = mid - 1;
  }
  const int y = a.y_begin + lo;
  const int i = (int)(t - a.y_prefix[lo]);
  const int v = score_thread(a.codes + a.xstart[i], a.xlen[i], a.codes + a.ystart[y], a.ylen[y],
                             a.go, a.ge, s_sub, a.scratch + t, a.nthreads);
  const int xo = a.xorig[i], yo = a.yorig[y];
  if (a.triangle) {
    a.D[(int64_t)xo * a.ld + yo] = (float)v;
    a.D[(int64_t)yo * a.ld + xo] = (float)v;
  } else {
    a.D[(int64_t)xo * a.ld + a.col0 + yo] = (float)v;
  }
}

// int32 re-run of the pairs the optimistic int16 groups queued.  The count is
// read on the device, so the launch needs no host round trip.
__global__ void __launch_bounds__(kPlainThreads) rerun_kernel(const WaveArgs a, int2* scratch,
                                                               int64_t nthreads) {
  __shared__ int8_t s_sub[kLetters * kLetters];
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = a.sub[e];
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long cnt = *a.rerun_count;
  if (cnt > (unsigned long long)a.rerun_cap) cnt = (unsigned long long)a.rerun_cap;
  for (int64_t k = t; k < (int64_t)cnt; k += nthreads) {
    const int2 q = a.rerun[k];
    const int v = score_thread(a.codes + a.xstart[q.x], a.xlen[q.x], a.codes + a.ystart[q.y], a.ylen[q.y],
                               a.go, a.ge, s_sub, scratch + t, nthreads);
    put_score(a, a.xorig[q.x], a.yorig[q.y], v);
  }
}

__global__ void __launch_bounds__(kPlainThreads) pairlist_kernel(const PairListArgs a, int64_t count) {
  __shared__ int8_t s_sub[kLetters * kLetters];
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = a.sub[e];
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int64_t k = a.base + t;
  const int i = a.pi[k], j = a.pj[k];
  a.out[k] = score_thread(a.codes + a.start[i], a.len[i], a.codes + a.start[j], a.len[j], a.go,
                          a.ge, s_sub, a.scratch + t, count);
}

// Peak of the cell update alone (roofline denominator): the inner loop of
// wave_band on a 16-row register strip, with the profile words and the
// incoming boundary taken from registers -- no memory, no shuffles.
template <int P, int F>
__global__ void __launch_bounds__(256) dpx_peak_kernel(uint32_t p0, uint32_t p1, uint32_t p2,
                                                       uint32_t p3, int go, int ge, int cols,
                                                       uint32_t* sink) {
  using L = Lanes<P>;
  constexpr int R = 16;
  const uint32_t NGE = L::packed(-ge), NGO = L::arith(-go, -go);
  uint32_t H[R], T[R], E[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    H[r] = L::splat(-ge * (r + 1 + (int)(threadIdx.x & 7)));
    T[r] = L::add(H[r], NGO);
    E[r] = L::splat(kShortMin + ge);
  }
  uint32_t hprev = 0, hin = L::splat(-ge), fin = L::splat(kShortMin + ge);
  const uint32_t pv[4] = {p0, p1, p2, p3};
  const uint32_t NGOP = L::packed(-go);
  for (int c = 0; c < cols; ++c) {
    uint32_t diag = hprev;
    hprev = hin;
    uint32_t f = fin;
    if (F == 3) {
      // shifted form with plain adds and 2-input maxima: 5 adds, 2 max, 1 max3
      const uint32_t NGEA = L::arith(-ge, -ge), NGOA = L::arith(-go, -go);
      uint32_t hup = hin;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        f = L::max2(L::add(f, NGEA), hup);
        const uint32_t e = L::max2(L::add(E[r], NGEA), H[r]);
        const uint32_t h = L::max3(L::add(f, NGOA), L::add(e, NGOA), L::add(diag, pv[r & 3]));
        diag = H[r];
        H[r] = h;
        E[r] = e;
        hup = h;
      }
      hin = H[3];
    } else if (F == 4) {
      // unshifted form with plain adds and 2-input maxima: 4 adds, 2 max, 1 max3
      const uint32_t NGEA = L::arith(-ge, -ge);
      uint32_t tup = L::add(hin, NGO);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        f = L::max2(L::add(f, NGEA), tup);
        const uint32_t e = L::max2(L::add(E[r], NGEA), T[r]);
        const uint32_t h = L::max3(e, f, L::add(diag, pv[r & 3]));
        diag = H[r];
        H[r] = h;
        E[r] = e;
        T[r] = L::add(h, NGO);
        tup = T[r];
      }
      hin = T[3];
    } else if (F == 5) {
      // shifted chain (viaddmax) with the off-chain maxima as adds + max
      const uint32_t NGEA = L::arith(-ge, -ge), NGOA = L::arith(-go, -go);
      uint32_t hup = hin;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        f = L::addmax(f, NGE, hup);
        const uint32_t e = L::max2(L::add(E[r], NGEA), H[r]);
        const uint32_t m = L::max2(L::add(e, NGOA), L::add(diag, pv[r & 3]));
        const uint32_t h = L::addmax(f, NGOP, m);
        diag = H[r];
        H[r] = h;
        E[r] = e;
        hup = h;
      }
      hin = H[3];
    } else if (F == 2) {
      // the shifted form of wave kernel layout V = 2: 4 DPX + 1 add per word
      uint32_t hup = hin;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        f = L::addmax(f, NGE, hup);
        const uint32_t e = L::addmax(E[r], NGE, H[r]);
        const uint32_t m = L::addmax(e, NGOP, L::add(diag, pv[r & 3]));
        const uint32_t h = L::addmax(f, NGOP, m);
        diag = H[r];
        H[r] = h;
        E[r] = e;
        hup = h;
      }
      hin = H[3];
    } else {
      uint32_t tup = L::add(hin, NGO);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        f = L::addmax(f, NGE, tup);
        const uint32_t e = L::addmax(E[r], NGE, T[r]);
        const uint32_t hd = L::add(diag, pv[r & 3]);
        const uint32_t h = L::max3(e, f, hd);
        diag = H[r];
        H[r] = h;
        E[r] = e;
        T[r] = L::add(h, NGO);
        tup = T[r];
      }
      hin = T[3];
    }
    fin = f;
  }
  uint32_t acc = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) acc ^= H[r] ^ E[r];
  if (acc == 0x9E3779B9u) sink[blockIdx.x] = acc;   // keeps the chain live
}

}  // namespace

#define NWG_CASE(r) \
  if (R == r) return wave_launch_r##r(P, V, W, a, grid, s);
cudaError_t launch_wave(int R, int P, int V, int W, const WaveArgs& a, int grid, cudaStream_t s) {
  NWG_WAVE_ROWS(NWG_CASE)
  return cudaErrorInvalidValue;
}
#undef NWG_CASE

#define NWG_CASE(r) \
  if (R == r) {     \
    wave_prepare_r##r(P, V, W); \
    return;         \
  }
void prepare_wave(int R, int P, int V, int W) { NWG_WAVE_ROWS(NWG_CASE) }
#undef NWG_CASE

#define NWG_CASE(r) \
  if (R == r) return wave_occupancy_r##r(P, V, W);
int wave_max_ctas_per_sm(int R, int P, int V, int W) {
  NWG_WAVE_ROWS(NWG_CASE)
  return 1;
}
#undef NWG_CASE

#define NWG_CASE(r) (R == r) ||
bool wave_exists(int R, int P, int V, int W) {
  return (NWG_WAVE_ROWS(NWG_CASE) false) && wave::wave_variant_exists(R, P, V, W);
}
#undef NWG_CASE

template <int P, int F>
static cudaError_t launch_peak_one(int cols, int grid, uint32_t* sink, int go, int ge, cudaStream_t s) {
  const uint32_t p0 = P == 2 ? 4u * 65536u + 3u : 0u, p1 = P == 2 ? (uint32_t)(-2 * 65536 + 1) : 1u,
                 p2 = P == 2 ? (uint32_t)(2 * 65536 - 1) : 0xFFFFFFFEu, p3 = P == 2 ? 5u * 65536u : 3u;
  dpx_peak_kernel<P, F><<<grid, 256, 0, s>>>(p0, p1, p2, p3, go, ge, cols, sink);
  return cudaGetLastError();
}

template <int P, int F>
static int peak_occupancy_one() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dpx_peak_kernel<P, F>, 256, 0);
  return n > 0 ? n : 1;
}

#define NWG_PEAK_FORMS(X) X(0) X(2) X(3) X(4) X(5)
cudaError_t launch_dpx_peak(int P, int form, int cols, int grid, uint32_t* sink, int go, int ge, cudaStream_t s) {
#define NWG_CASE(f) \
  if (form == f) return P == 2 ? launch_peak_one<2, f>(cols, grid, sink, go, ge, s) : launch_peak_one<1, f>(cols, grid, sink, go, ge, s);
  NWG_PEAK_FORMS(NWG_CASE)
#undef NWG_CASE
  return cudaErrorInvalidValue;
}

int dpx_peak_ctas_per_sm(int P, int form) {
#define NWG_CASE(f) \
  if (form == f) return P == 2 ? peak_occupancy_one<2, f>() : peak_occupancy_one<1, f>();
  NWG_PEAK_FORMS(NWG_CASE)
#undef NWG_CASE
  return 1;
}
#undef NWG_PEAK_FORMS

cudaError_t launch_rerun(const WaveArgs& a, int2* scratch, int64_t nthreads, cudaStream_t s) {
  const int64_t blocks = (nthreads + kPlainThreads - 1) / kPlainThreads;
  rerun_kernel<<<(unsigned)blocks, kPlainThreads, 0, s>>>(a, scratch, blocks * kPlainThreads);
  return cudaGetLastError();
}

cudaError_t launch_plain(const PlainArgs& a, cudaStream_t s) {
  const int64_t blocks = (a.nthreads + kPlainThreads - 1) / kPlainThreads;
  plain_kernel<<<(unsigned)blocks, kPlainThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_pairlist(const PairListArgs& a, int64_t count, cudaStream_t s) {
  const int64_t blocks = (count + kPlainThreads - 1) / kPlainThreads;
  pairlist_kernel<<<(unsigned)blocks, kPlainThreads, 0, s>>>(a, count);
  return cudaGetLastError();
}

}  // namespace nwg
