// wave_impl.cuh -- the batched-form kernel (anti-diagonal wavefront per warp),
// instantiated per rows-per-lane template in wave_r*.cu.
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
// A wavefront of W lanes (W = 32, 16 or 8: 32/W wavefronts per warp, each on
// its own X) aligns one X (streamed as columns) against a band of W*R rows:
// lane k of the front owns rows [kR, kR+R) and runs one column behind lane
// k-1; the bottom (H, F) of each lane's strip goes to lane k+1 by
// __shfl_up_sync within the front.  Narrow fronts give bands of 8R and 16R
// rows (finer than 32R) and a ramp of W-1 columns instead of 31.  P = 2 packs
// two Y sequences into the halves of every register (offset-binary int16x2,
// unsigned DPX max + full-rate 32-bit adds), P = 1 runs int32 lanes.  All
// warps of a CTA share one Y group, so the per-letter score profile of the
// band is built once per CTA in shared memory and read as one 128-bit load
// per 4 rows.  CTAs are persistent and pull (Y group, X chunk) jobs from a
// device counter.  V selects the register layout: V = 0 keeps H, H-go and E
// per row (fewest instructions), V = 1 keeps H and E and recomputes H-go with
// one add (fewer registers, more resident warps: min-blocks launch bound).
// V = 2 keeps E' = E + go and F' = F + go instead of E and F:
//   F'[r] = max(F'[r-1] - ge, H[r-1]),  E'[c] = max(E'[c-1] - ge, H[c-1]),
//   H = max(F' - go, max(E' - go, diag + S)),
// the same values (go >= ge is not even needed: it is a change of variables),
// with two dependent operations per row down the strip instead of three.
#pragma once

#include <type_traits>

#include "nwg_internal.h"

namespace nwg {
namespace wave {

__device__ __forceinline__ uint32_t splat16(int v) {
  return (uint32_t)(v & 0xFFFF) | ((uint32_t)(v & 0xFFFF) << 16);
}

template <int P>
struct Lanes;

// Two independent pairs in the halves of every 32-bit word, each half in
// offset binary (value + 32768).  The max operations are unsigned DPX
// (__viaddmax_u16x2 adds per half modulo 2^16, then takes the unsigned max;
// __vimax3_u16x2), and offset-binary order is numeric order.  The two plain
// additions of a cell (H - go, diag + S) are ordinary 32-bit adds of a word
// holding hi*65536 + lo: with every half inside [4, 65524] no carry crosses
// from the low half, which the host's overflow guard guarantees (values stay
// within [-32764, 32756]).  Per word: 2 full-rate adds + 3 DPX.
template <>
struct Lanes<2> {
  static __device__ __forceinline__ uint32_t splat(int v) { return splat16(v + 32768); }
  // word to ADD (32-bit arithmetic) that adds lo to the low half and hi to the high half
  static __device__ __forceinline__ uint32_t arith(int lo, int hi) { return (uint32_t)(hi * 65536 + lo); }
  // per-half operand for addmax (modulo 2^16 in each half)
  static __device__ __forceinline__ uint32_t packed(int v) { return splat16(v); }
  static __device__ __forceinline__ uint32_t add(uint32_t a, uint32_t b) { return a + b; }
  static __device__ __forceinline__ uint32_t addmax(uint32_t a, uint32_t b, uint32_t c) {
    return __viaddmax_u16x2(a, b, c);
  }
  static __device__ __forceinline__ uint32_t max3(uint32_t a, uint32_t b, uint32_t c) {
    return __vimax3_u16x2(a, b, c);
  }
  static __device__ __forceinline__ int lo(uint32_t w) { return (int)(w & 0xFFFFu) - 32768; }
  static __device__ __forceinline__ int hi(uint32_t w) { return (int)(w >> 16) - 32768; }
};

template <>
struct Lanes<1> {
  static __device__ __forceinline__ uint32_t splat(int v) { return (uint32_t)v; }
  static __device__ __forceinline__ uint32_t arith(int lo, int) { return (uint32_t)lo; }
  static __device__ __forceinline__ uint32_t packed(int v) { return (uint32_t)v; }
  static __device__ __forceinline__ uint32_t add(uint32_t a, uint32_t b) { return (uint32_t)((int)a + (int)b); }
  static __device__ __forceinline__ uint32_t addmax(uint32_t a, uint32_t b, uint32_t c) {
    return (uint32_t)__viaddmax_s32((int)a, (int)b, (int)c);
  }
  static __device__ __forceinline__ uint32_t max3(uint32_t a, uint32_t b, uint32_t c) {
    return (uint32_t)__vimax3_s32((int)a, (int)b, (int)c);
  }
  static __device__ __forceinline__ int lo(uint32_t w) { return (int)w; }
  static __device__ __forceinline__ int hi(uint32_t w) { return (int)w; }
};

__device__ __forceinline__ unsigned clamp_code(int c) {
  // Codes are validated on the host (or counted by the bound kernel); the
  // clamp only keeps a bad code from addressing outside the shared tables.
  const unsigned u = (unsigned)c;
  return u < (unsigned)kLetters ? u : (unsigned)(kLetters - 1);
}

template <int R>
__device__ __forceinline__ uint32_t pick(const uint32_t (&H)[R], int idx) {
  uint32_t v = 0;
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (r == idx) v = H[r];
  return v;
}

__device__ __forceinline__ void put_score(const WaveArgs& a, int xo, int yo, int v) {
  if (a.triangle) {
    a.D[(int64_t)xo * a.ld + yo] = (float)v;
    a.D[(int64_t)yo * a.ld + xo] = (float)v;
  } else {
    a.D[(int64_t)xo * a.ld + a.col0 + yo] = (float)v;
  }
}

// Job-relative output (several jobs in one launch): the group's matrix.
__device__ __forceinline__ void put_score_job(const WaveArgs& a, float* D, int64_t ld, int xo, int yo, int v) {
  D[(int64_t)xo * ld + yo] = (float)v;
  D[(int64_t)yo * ld + xo] = (float)v;
}

// Optimistic int16 groups: a pair whose composition bound could exceed the
// int16 range is not reported from the int16 lanes; it goes to the int32
// re-run queue instead.
__device__ __forceinline__ bool int16_safe(const WaveArgs& a, int i, int y) {
  return !a.check_bound || min(a.xbound[i], a.ybound[y]) <= a.max_h;
}

__device__ __forceinline__ void queue_rerun(const WaveArgs& a, int i, int y) {
  const unsigned long long k = atomicAdd(a.rerun_count, 1ull);
  if (k < (unsigned long long)a.rerun_cap) a.rerun[k] = make_int2(i, y);
}

template <int R, int P, int V>
struct BandState {
  uint32_t H[R];
  uint32_t E[R];
  uint32_t T[V == 0 ? R : 1];
};

// One column of the lane's R-row strip: H/E (and H-go for V == 0) updated in
// place; f carries F down the strip; returns the bottom F (F' for V == 2).
// NGO: word added to H to get H - go; NGOP: -go as the per-half addmax operand.
template <int R, int P, int V, int W>
__device__ __forceinline__ uint32_t strip_column(BandState<R, P, V>& s, const uint4* __restrict__ pp,
                                                 uint32_t diag, uint32_t hin, uint32_t fin, uint32_t NGE,
                                                 uint32_t NGO, uint32_t NGOP) {
  using L = Lanes<P>;
  constexpr int Q = R / 4;
  uint32_t f = fin;
  if (V == 2) {
    // fin is F' of the row above the strip, hin its H
    uint32_t hup = hin;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const uint4 pv = pp[q * W];
      const uint32_t sv[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const int r = q * 4 + w;
        f = L::addmax(f, NGE, hup);                                      // F'[r][c]
        const uint32_t e = L::addmax(s.E[r], NGE, s.H[r]);               // E'[r][c]
        const uint32_t m = L::addmax(e, NGOP, L::add(diag, sv[w]));      // max(E, diag + S)
        const uint32_t h = L::addmax(f, NGOP, m);                        // H[r][c]
        diag = s.H[r];
        s.H[r] = h;
        s.E[r] = e;
        hup = h;
      }
    }
    return f;
  }
  uint32_t tup = L::add(hin, NGO);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint4 pv = pp[q * W];
    const uint32_t sv[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int r = q * 4 + w;
      f = L::addmax(f, NGE, tup);                                        // F[r][c]
      const uint32_t tl = (V == 0) ? s.T[(V == 0) ? r : 0] : L::add(s.H[r], NGO);
      const uint32_t e = L::addmax(s.E[r], NGE, tl);                     // E[r][c]
      const uint32_t hd = L::add(diag, sv[w]);                           // H[r-1][c-1] + S
      const uint32_t h = L::max3(e, f, hd);                              // H[r][c]
      diag = s.H[r];
      s.H[r] = h;
      s.E[r] = e;
      tup = L::add(h, NGO);
      if (V == 0) s.T[(V == 0) ? r : 0] = tup;
    }
  }
  return f;
}

// One band (W*R rows starting at b*W*R) of one X for the calling front.
// sl: lane within the front; Lx: this front's X length, 0 when the front has
// no pair to report (its lanes then only take part in the shuffles); Lmin /
// Lmax: smallest / largest Lx over the warp's working fronts (warp-uniform).
template <int R, int P, int V, int W>
__device__ __forceinline__ void wave_band(const WaveArgs& a, int sl, int b, int nb,
                                          const int8_t* __restrict__ X, int Lx, int Lmin, int Lmax,
                                          const uint32_t* __restrict__ prof,
                                          int32_t* __restrict__ scratch, int rowA, int rowB,
                                          bool wantA, bool wantB, int xo, int yoA, int yoB,
                                          float* jobD, int64_t jobld) {
  using L = Lanes<P>;
  constexpr int BAND = W * R;
  constexpr int Q = R / 4;
  const uint32_t NGE = L::packed(-a.ge);        // per-half operand of addmax
  const uint32_t NGO = L::arith(-a.go, -a.go);   // word added to H to get H - go
  const uint32_t NGOP = L::packed(-a.go);        // per-half operand: - go
  const uint32_t NGEA = L::arith(-a.ge, -a.ge);  // word added to H[-1][c] to get H[-1][c+1]
  // E[r][-1] = F[-1][c] = -32768 + ge; V == 2 keeps them shifted by go
  const uint32_t SENT = L::splat(kShortMin + a.ge + (V == 2 ? a.go : 0));

  BandState<R, P, V> s;
  const int rowbase = b * BAND + sl * R;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    s.H[r] = L::splat(-a.ge * (rowbase + r + 1));   // H[row][-1]
    s.E[r] = SENT;                                   // E[row][-1]
    if (V == 0) s.T[(V == 0) ? r : 0] = L::add(s.H[r], NGO);
  }
  uint32_t hprev = L::splat(-a.ge * rowbase);       // H[rowbase-1][-1]: diag of column 0
  uint32_t hbot = 0, fbot = 0;
  uint32_t hb = L::splat(-a.ge);                    // H[-1][c] of the column lane 0 works on (band 0)
  const bool top = b == 0;
  const bool work = Lx > 0;
  const int32_t* rd = scratch + ((b + 1) & 1) * 2 * a.scratch_cols;   // written by band b-1
  int32_t* wr = scratch + (b & 1) * 2 * a.scratch_cols;
  const bool writer = sl == W - 1 && b + 1 < nb && work;
  const uint4* pl = reinterpret_cast<const uint4*>(prof) + sl;
  int xnext = (sl == 0 && work) ? (int)X[0] : 0;

  auto step = [&](int t, auto checked) {
    constexpr bool kChecked = decltype(checked)::value;
    const int c = t - sl;
    uint32_t hin = __shfl_up_sync(0xffffffffu, hbot, 1, W);
    uint32_t fin = __shfl_up_sync(0xffffffffu, fbot, 1, W);
    const int xl = xnext;
    if (kChecked) {
      if (c + 1 >= 0 && c + 1 < Lx) xnext = X[c + 1];
    } else if (W == 32 || work) {
      xnext = X[min(c + 1, Lx - 1)];
    }
    if (kChecked ? (c >= 0 && c < Lx) : (W == 32 || work)) {
      uint32_t bh = hb, bf = SENT;
      if (!top && sl == 0) {
        bh = (uint32_t)rd[2 * c];
        bf = (uint32_t)rd[2 * c + 1];
      }
      if (sl == 0) {
        hin = bh;
        fin = bf;
      }
      hb = L::add(hb, NGEA);
      const uint32_t diag = hprev;
      hprev = hin;
      fbot = strip_column<R, P, V, W>(s, pl + clamp_code(xl) * (Q * W), diag, hin, fin, NGE, NGO, NGOP);
      hbot = s.H[R - 1];
      if (writer) {
        wr[2 * c] = (int32_t)hbot;
        wr[2 * c + 1] = (int32_t)fbot;
      }
    }
  };
  // ramp-up (some lanes before column 0), steady state (every lane of every
  // working front on a column), ramp-down (some lanes past their last column)
  int t = 0;
  const int t1 = Lmin < W - 1 ? Lmin : W - 1;
  for (; t < t1; ++t) step(t, std::true_type{});
  for (; t < Lmin; ++t) step(t, std::false_type{});
  for (; t < Lmax + W - 1; ++t) step(t, std::true_type{});

  // H[] now holds the last column; the lane owning a pair's last row reports.
  if (wantA) {
    const int rr = rowA - b * BAND;
    if (rr >= 0 && rr < BAND && sl == rr / R) {
      const int v = L::lo(pick<R>(s.H, rr % R));
      if (jobD) put_score_job(a, jobD, jobld, xo, yoA, v);
      else put_score(a, xo, yoA, v);
    }
  }
  if (P == 2 && wantB) {
    const int rr = rowB - b * BAND;
    if (rr >= 0 && rr < BAND && sl == rr / R) {
      const int v = L::hi(pick<R>(s.H, rr % R));
      if (jobD) put_score_job(a, jobD, jobld, xo, yoB, v);
      else put_score(a, xo, yoB, v);
    }
  }
}

template <int R, int P, int V>
struct MinBlocks {
  static constexpr int value = V == 0 ? 1 : (R <= 8 ? 4 : (R <= 16 ? 3 : 2));
};

template <int R, int P, int V, int W>
__global__ void __launch_bounds__(kWaveThreads, (MinBlocks<R, P, V>::value)) wave_kernel(const WaveArgs a) {
  constexpr int S = 32 / W;                // fronts per warp
  constexpr int BAND = W * R;
  constexpr int Q = R / 4;
  static_assert(R % 4 == 0, "rows per lane must be a multiple of 4");
  static_assert(W == 8 || W == 16 || W == 32, "front width");
  extern __shared__ __align__(16) uint32_t prof[];   // [letter][Q][front lane][4]
  __shared__ int8_t s_sub[kLetters * kLetters];
  __shared__ long long s_job;

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int sl = lane % W;                 // lane within the front
  const int seg = lane / W;                // front within the warp
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = a.sub[e];
  int32_t* scratch =
      a.scratch + ((size_t)(blockIdx.x * kWaveWarps + warp) * S + seg) * 4 * (size_t)a.scratch_cols;

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_job = (long long)atomicAdd(a.counter, 1ull);
    __syncthreads();
    const long long job = s_job;
    if (job >= a.njobs) break;
    int lo = 0, hi = a.ngroups - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.job_prefix[mid] <= job) lo = mid; else hi = mid - 1;
    }
    const long long chunk = job - a.job_prefix[lo];
    const int g = a.g_begin + lo;
    const int y0 = a.group_y[g];
    const int y1 = (P == 2) ? a.group_y2[g] : -1;
    const bool has_b = y1 >= 0;
    const int nX = a.group_x[g];
    const int xbase = a.group_xbase ? a.group_xbase[g] : 0;
    float* jobD = a.group_dofs ? a.D + a.group_dofs[g] : nullptr;
    const int64_t jobld = a.group_ld ? a.group_ld[g] : a.ld;
    const int i = xbase + (int)(chunk * (kWaveWarps * S)) + warp * S + seg;
    const int LyA = a.ylen[y0];
    const int LyB = has_b ? a.ylen[y1] : 0;
    const int8_t* YA = a.codes + a.ystart[y0];
    const int8_t* YB = has_b ? a.codes + a.ystart[y1] : YA;
    const bool active = i < xbase + nX;
    const int8_t* X = a.codes + (active ? a.xstart[i] : 0);
    bool wantA = active && (!a.triangle || i <= y0);
    bool wantB = active && has_b && (!a.triangle || i <= y1);
    if (P == 2 && a.check_bound && active) {
      // A carry out of an overflowing low half would reach the high half of
      // the same word, so an unsafe A pair also sends B to the re-run queue.
      const bool safeA = int16_safe(a, i, y0);
      const bool safeB = !has_b || int16_safe(a, i, y1);
      if (wantA && !safeA) {
        if (sl == 0) queue_rerun(a, i, y0);
        wantA = false;
      }
      if (wantB && !(safeA && safeB)) {
        if (sl == 0) queue_rerun(a, i, y1);
        wantB = false;
      }
    }
    const int Lx = (wantA || wantB) ? a.xlen[i] : 0;
    const int Lmax = __reduce_max_sync(0xffffffffu, (unsigned)Lx);
    const int Lmin = (int)__reduce_min_sync(0xffffffffu, Lx > 0 ? (unsigned)Lx : 0x7fffffffu);
    const int rows = LyA > LyB ? LyA : LyB;
    const int nb = (rows + BAND - 1) / BAND;
    const int xo = active ? a.xorig[i] : 0;
    const int yoA = a.yorig[y0];
    const int yoB = has_b ? a.yorig[y1] : 0;

    for (int b = 0; b < nb; ++b) {
      if (b > 0) __syncthreads();   // every warp is done with the previous band's profile
      for (int e = threadIdx.x; e < kLetters * BAND; e += kWaveThreads) {
        const int x = e / BAND;
        const int row = e - x * BAND;
        const int k = row / R, r = row - k * R;
        const int grow = b * BAND + row;
        const int sa = grow < LyA ? (int)s_sub[clamp_code(YA[grow]) * kLetters + x] : 0;
        uint32_t w;
        if (P == 2) {
          const int sb = grow < LyB ? (int)s_sub[clamp_code(YB[grow]) * kLetters + x] : 0;
          w = Lanes<2>::arith(sa, sb);
        } else {
          w = (uint32_t)sa;
        }
        prof[((x * Q + (r >> 2)) * W + k) * 4 + (r & 3)] = w;
      }
      __syncthreads();
      if (Lmax > 0)
        wave_band<R, P, V, W>(a, sl, b, nb, X, Lx, Lmin, Lmax, prof, scratch, LyA - 1, LyB - 1, wantA, wantB, xo,
                              yoA, yoB, jobD, jobld);
    }
  }
}

template <int R, int P, int V, int W>
void prepare_one() {
  const size_t smem = (size_t)kLetters * W * R * sizeof(uint32_t);
  cudaFuncSetAttribute(wave_kernel<R, P, V, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int R, int P, int V, int W>
cudaError_t launch_one(const WaveArgs& a, int grid, cudaStream_t s) {
  const size_t smem = (size_t)kLetters * W * R * sizeof(uint32_t);
  wave_kernel<R, P, V, W><<<grid, kWaveThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int R, int P, int V, int W>
int occupancy_one() {
  const size_t smem = (size_t)kLetters * W * R * sizeof(uint32_t);
  cudaFuncSetAttribute(wave_kernel<R, P, V, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wave_kernel<R, P, V, W>, kWaveThreads, smem) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

// The (P, V, W) combinations that exist: W = 32 with every P and V; the
// narrow fronts (W = 16, 8) on int16x2 lanes with V = 0 or 2.
inline bool wave_variant_exists(int P, int V, int W) {
  if (W == 32) return (P == 1 || P == 2) && V >= 0 && V <= 2;
  return (W == 16 || W == 8) && P == 2 && (V == 0 || V == 2);
}

// Entry points of one rows-per-lane template (every existing P, V, W).
template <int R>
struct Entry {
  template <class Fn>
  static auto with(int P, int V, int W, Fn&& fn) {
    if (W == 16) return V == 2 ? fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 2>{},
                                    std::integral_constant<int, 16>{})
                               : fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 0>{},
                                    std::integral_constant<int, 16>{});
    if (W == 8) return V == 2 ? fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 2>{},
                                   std::integral_constant<int, 8>{})
                              : fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 0>{},
                                   std::integral_constant<int, 8>{});
    if (P == 2) {
      if (V == 2) return fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 2>{},
                            std::integral_constant<int, 32>{});
      if (V == 1) return fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 1>{},
                            std::integral_constant<int, 32>{});
      return fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 0>{}, std::integral_constant<int, 32>{});
    }
    if (V == 2) return fn(std::integral_constant<int, 1>{}, std::integral_constant<int, 2>{},
                          std::integral_constant<int, 32>{});
    if (V == 1) return fn(std::integral_constant<int, 1>{}, std::integral_constant<int, 1>{},
                          std::integral_constant<int, 32>{});
    return fn(std::integral_constant<int, 1>{}, std::integral_constant<int, 0>{}, std::integral_constant<int, 32>{});
  }
  static cudaError_t launch(int P, int V, int W, const WaveArgs& a, int grid, cudaStream_t s) {
    if (!wave_variant_exists(P, V, W)) return cudaErrorInvalidValue;
    return with(P, V, W, [&](auto p, auto v, auto w) {
      return launch_one<R, decltype(p)::value, decltype(v)::value, decltype(w)::value>(a, grid, s);
    });
  }
  static void prepare(int P, int V, int W) {
    if (!wave_variant_exists(P, V, W)) return;
    with(P, V, W, [&](auto p, auto v, auto w) {
      prepare_one<R, decltype(p)::value, decltype(v)::value, decltype(w)::value>();
      return 0;
    });
  }
  static int occupancy(int P, int V, int W) {
    if (!wave_variant_exists(P, V, W)) return 1;
    return with(P, V, W, [&](auto p, auto v, auto w) {
      return occupancy_one<R, decltype(p)::value, decltype(v)::value, decltype(w)::value>();
    });
  }
};

}  // namespace wave

// Per-template dispatch tables (one translation unit per R).
#define NWG_WAVE_ROWS(X) X(4) X(8) X(12) X(16) X(20) X(24) X(32)
#define NWG_DECL_WAVE(r)                                                                         \
  cudaError_t wave_launch_r##r(int P, int V, int W, const WaveArgs& a, int grid, cudaStream_t s); \
  void wave_prepare_r##r(int P, int V, int W);                                                  \
  int wave_occupancy_r##r(int P, int V, int W);
NWG_WAVE_ROWS(NWG_DECL_WAVE)
#undef NWG_DECL_WAVE

#define NWG_DEFINE_WAVE(r)                                                                        \
  cudaError_t wave_launch_r##r(int P, int V, int W, const WaveArgs& a, int grid, cudaStream_t s) { \
    return wave::Entry<r>::launch(P, V, W, a, grid, s);                                          \
  }                                                                                              \
  void wave_prepare_r##r(int P, int V, int W) { wave::Entry<r>::prepare(P, V, W); }              \
  int wave_occupancy_r##r(int P, int V, int W) { return wave::Entry<r>::occupancy(P, V, W); }

}  // namespace nwg
