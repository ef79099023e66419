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
// V = 3 keeps T = H - go and E per row and nothing else: the diagonal term
// H[r-1][c-1] + S becomes T[r-1][c-1] + (S + go), with S + go stored in the
// profile, so V = 0's instruction mix (2 adds, 2 viaddmax, 1 vimax3) runs
// with V = 2's register footprint.
// V = 4 is V = 2 with a one-operation F chain, exact when go >= ge: with
// m = max(E, diag + S), H = max(F, m), so F'[r] = max(F'[r-1] - ge, H[r-1])
// = max(F'[r-1] - ge, F'[r-1] - go, m[r-1]) = max(F'[r-1] - ge, m[r-1]);
// m does not depend on F, so only the F' update itself stays on the path
// from one row to the next (and from one lane to the next).
// V = 6 is layout 3 with the lane's strip split in two halves one column
// apart: at step t lane k's upper R/2 rows work on column t - 2k and its lower
// R/2 rows on column t - 2k - 1, fed by the upper half's last row of the step
// before.  The two halves are independent within a step, so the lane has two
// dependency chains of R/2 rows instead of one of R, with layout 3's 3 ALU
// operations per word; the skew between lanes becomes two columns.
// V = 5 is layout 3 with two X per front: every lane runs the strips of two
// X (adjacent in length order) against the same band, row by row
// interleaved, so two independent dependency chains share the lane's issue
// slots.
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
  static __device__ __forceinline__ uint32_t max2(uint32_t a, uint32_t b) { return __vmaxu2(a, b); }
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
  static __device__ __forceinline__ uint32_t max2(uint32_t a, uint32_t b) { return (uint32_t)max((int)a, (int)b); }
  static __device__ __forceinline__ int lo(uint32_t w) { return (int)w; }
  static __device__ __forceinline__ int hi(uint32_t w) { return (int)w; }
};

__device__ __forceinline__ unsigned clamp_code(int c) {
  // Codes are validated on the host (or counted by the bound kernel); the
  // clamp only keeps a bad code from addressing outside the shared tables.
  const unsigned u = (unsigned)c;
  return u < (unsigned)kLetters ? u : (unsigned)(kLetters - 1);
}

// One pair per thread, int32, 16-row register strip; the (H, F) row between
// strips lives in global scratch, one int2 per X column at stride `stride`
// (consecutive threads adjacent: coalesced).  Used by the plain, re-run and
// pair-list kernels and by the allocation-free entry point.  Same loop structure as
// NeedlemanWunschGlobalScoreKernel with its 12-row strips widened to 16.
__device__ __forceinline__ int score_thread(const int8_t* __restrict__ X, int Lx,
                                            const int8_t* __restrict__ Y, int Ly, int go, int ge,
                                            const int8_t* s_sub, int2* sc, int64_t stride) {
  for (int c = 0; c < Lx; ++c) sc[(int64_t)c * stride] = make_int2(-ge * (c + 1), kShortMin + ge);
  int hc = 0;
  for (int y0 = 0; y0 < Ly; y0 += kPlainRows) {
    int yl[kPlainRows], Hs[kPlainRows], Es[kPlainRows];
#pragma unroll
    for (int r = 0; r < kPlainRows; ++r) {
      yl[r] = (y0 + r < Ly) ? (int)clamp_code(Y[y0 + r]) * kLetters : 0;
      Hs[r] = -ge * (y0 + r + 1);
      Es[r] = kShortMin + ge;
    }
    int upleft = -ge * y0;
    const int ymin = min(kPlainRows, Ly - y0);
    for (int c = 0; c < Lx; ++c) {
      int diag = upleft;
      const int2 af = sc[(int64_t)c * stride];
      hc = af.x;
      upleft = af.x;
      int f = af.y;
      const unsigned xc = clamp_code(X[c]);
#pragma unroll
      for (int r = 0; r < kPlainRows; ++r) {
        if (r < ymin) {
          const int s = s_sub[yl[r] + xc];
          f = max(f - ge, hc - go);
          const int e = max(Es[r] - ge, Hs[r] - go);
          hc = max(max(e, f), s + diag);
          diag = Hs[r];
          Hs[r] = hc;
          Es[r] = e;
        }
      }
      sc[(int64_t)c * stride] = make_int2(hc, f);
    }
  }
  return hc;
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

// Shared-memory score profile of one band: per letter, Q = R/4 groups of
// four rows, each group one uint4 per front lane.  With W = 1 (one pair per
// thread) the 32 lanes of a warp read different letters at once, so each
// letter's row of groups is padded by one uint4 to spread them over the banks.
template <int R, int W>
struct Profile {
  static constexpr int Q = (R + 3) / 4;                               // uint4 per lane (last one partly used)
  static constexpr int kLetterStride = W == 1 ? Q + 1 : Q * W;        // uint4 per letter
  static constexpr int kWords = kLetters * kLetterStride * 4;         // 32-bit words
  static constexpr size_t kBytes = sizeof(uint32_t) * (size_t)kWords;
  static __device__ __forceinline__ int index(int x, int row) {       // word of (letter, band row)
    const int k = row / R, r = row - k * R;
    return ((x * kLetterStride + (r >> 2) * W + k)) * 4 + (r & 3);
  }
};

// Words between the band-boundary entries of consecutive columns of one
// front: with W = 1 the CTA's 256 fronts interleave column by column, so a
// warp's 32 fronts read and write 32 consecutive words per column.
template <int W>
constexpr int scratch_stride() { return W == 1 ? kWaveThreads : 1; }

template <int V>
struct Layout {
  static constexpr int K = V == 5 ? 2 : 1;                // X per front
  static constexpr int L = (V == 5 || V == 6) ? 3 : V;    // register layout of each strip
};

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
  constexpr int Q = (R + 3) / 4;   // 4-row profile quads; rows past R of the last one are skipped
  uint32_t f = fin;
  if (V == 3) {
    // s.H holds T = H - go; hin is T of the row above; sv is S + go.  The next
    // row's diag + S is taken from the old T[r] before T[r] is overwritten, so
    // no value has to outlive its register's new contents (the profile quad
    // of the next 4 rows is loaded one quad ahead).
    uint32_t tup = hin;
    uint4 pv = pp[0];
    uint32_t hd = L::add(diag, pv.x);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const uint4 pn = (q + 1 < Q) ? pp[(q + 1) * W] : pv;
      const uint32_t sn[4] = {pv.y, pv.z, pv.w, pn.x};                 // S + go of the row below
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const int r = q * 4 + w;
        if (r >= R) continue;
        f = L::addmax(f, NGE, tup);                                      // F[r][c]
        const uint32_t e = L::addmax(s.E[r], NGE, s.H[r]);               // E[r][c]
        const uint32_t hn = L::add(s.H[r], sn[w]);                       // row r + 1: diag + S
        const uint32_t h = L::max3(e, f, hd);                            // H[r][c]
        s.H[r] = L::add(h, NGO);
        s.E[r] = e;
        tup = s.H[r];
        hd = hn;
      }
      pv = pn;
    }
    return f;
  }
  if (V == 4) {
    // fin is F' of the row above the strip, hin its H; then up carries m
    uint32_t up = hin;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const uint4 pv = pp[q * W];
      const uint32_t sv[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const int r = q * 4 + w;
        if (r >= R) continue;
        f = L::addmax(f, NGE, up);                                       // F'[r][c]
        const uint32_t e = L::addmax(s.E[r], NGE, s.H[r]);               // E'[r][c]
        const uint32_t m = L::addmax(e, NGOP, L::add(diag, sv[w]));      // max(E, diag + S)
        diag = s.H[r];
        s.H[r] = L::addmax(f, NGOP, m);                                  // H[r][c]
        s.E[r] = e;
        up = m;
      }
    }
    return f;
  }
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
        if (r >= R) continue;
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
      if (r >= R) continue;
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

// Two strips of layout 3 (two X, the same rows), interleaved row by row.
template <int R, int P, int W>
__device__ __forceinline__ void strip_column_pair(BandState<R, P, 3> (&s)[2], const uint4* __restrict__ pa,
                                                  const uint4* __restrict__ pb, uint32_t (&diag)[2],
                                                  const uint32_t (&hin)[2], uint32_t (&f)[2], uint32_t NGE,
                                                  uint32_t NGO) {
  using L = Lanes<P>;
  constexpr int Q = (R + 3) / 4;
  uint32_t tup[2] = {hin[0], hin[1]};
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint4 va = pa[q * W], vb = pb[q * W];
    const uint32_t sv[2][4] = {{va.x, va.y, va.z, va.w}, {vb.x, vb.y, vb.z, vb.w}};
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int r = q * 4 + w;
      if (r >= R) continue;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        f[k] = L::addmax(f[k], NGE, tup[k]);
        const uint32_t e = L::addmax(s[k].E[r], NGE, s[k].H[r]);
        const uint32_t h = L::max3(e, f[k], L::add(diag[k], sv[k][w]));
        diag[k] = s[k].H[r];
        s[k].H[r] = L::add(h, NGO);
        s[k].E[r] = e;
        tup[k] = s[k].H[r];
      }
    }
  }
}

// Rows [R0, R0 + RH) (RH a multiple of 4) of a layout-3 strip at one column:
// s.H holds T = H - go; tup is T of the row above, diag T of the row above at
// the previous column, f the F of the row above; pp the column's profile
// (S + go).  Returns F of the last row.
template <int R0, int RH, int R, int P, int W>
__device__ __forceinline__ uint32_t strip_rows3(BandState<R, P, 3>& s, const uint4* __restrict__ pp, uint32_t diag,
                                                uint32_t tup, uint32_t f, uint32_t NGE, uint32_t NGO) {
  using L = Lanes<P>;
  static_assert(R0 % 4 == 0 && RH % 4 == 0 && R0 + RH <= R, "4-row profile quads");
  constexpr int Q0 = R0 / 4, Q1 = (R0 + RH) / 4;
  // The next row's diag + S is taken from the old T[r] before T[r] is
  // overwritten, so no value has to outlive its register's new contents (the
  // profile quad of the next 4 rows is loaded one quad ahead).
  uint4 pv = pp[Q0 * W];
  uint32_t hd = L::add(diag, pv.x);                                    // row R0: diag + S
#pragma unroll
  for (int q = Q0; q < Q1; ++q) {
    const uint4 pn = (q + 1 < Q1) ? pp[(q + 1) * W] : pv;
    const uint32_t sv[4] = {pv.x, pv.y, pv.z, pv.w};
    const uint32_t sn[4] = {pv.y, pv.z, pv.w, pn.x};                   // S + go of the row below
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int r = q * 4 + w;
      f = L::addmax(f, NGE, tup);                                      // F[r][c]
      const uint32_t e = L::addmax(s.E[r], NGE, s.H[r]);               // E[r][c]
      const uint32_t hn = L::add(s.H[r], sn[w]);                       // row r + 1: diag + S
      const uint32_t h = L::max3(e, f, hd);                            // H[r][c]
      s.H[r] = L::add(h, NGO);
      s.E[r] = e;
      tup = s.H[r];
      hd = hn;
      (void)sv;
    }
    pv = pn;
  }
  return f;
}

// One band of layout 6 (layout 3, the lane's strip split in two halves one
// column apart; one X per front, wavefronts of 8 to 32 lanes).  Arguments as
// wave_band's.
template <int R, int P, int W>
__device__ __forceinline__ void wave_band_split(const WaveArgs& a, int sl, int b, int nb, const int8_t* X0, int Lx0,
                                                int Lmin, int Lmax, const uint32_t* __restrict__ prof,
                                                int32_t* __restrict__ scratch, int rowA, int rowB, bool wantA0,
                                                bool wantB0, int xo0, int yoA, int yoB, float* jobD, int64_t jobld) {
  using L = Lanes<P>;
  constexpr int BAND = W * R;
  constexpr int RH = R / 2;
  static_assert(W >= 8 && RH % 4 == 0, "split strips: wavefronts, halves of whole 4-row quads");
  const uint32_t NGE = L::packed(-a.ge);
  const uint32_t NGO = L::arith(-a.go, -a.go);
  const uint32_t NGEA = L::arith(-a.ge, -a.ge);
  const uint32_t SENT = L::splat(kShortMin + a.ge);
  constexpr int LS = Profile<R, W>::kLetterStride;
  BandState<R, P, 3> s;
  const int rowbase = b * BAND + sl * R;
  const int gsh = a.go;   // layout 3 carries T = H - go
#pragma unroll
  for (int r = 0; r < R; ++r) {
    s.H[r] = L::splat(-a.ge * (rowbase + r + 1) - gsh);   // T[row][-1]
    s.E[r] = SENT;
  }
  const bool work = Lx0 > 0;
  const int32_t* rd = scratch + ((b + 1) & 1) * 2 * a.scratch_cols;   // band b-1
  int32_t* wr = scratch + (b & 1) * 2 * a.scratch_cols;
  uint32_t hprev = L::splat(-a.ge * rowbase - gsh);   // T of the row above the strip at column c-1
  uint32_t mid_prev = s.H[RH - 1];                    // T of the upper half's last row at column c-2
  uint32_t fmid = 0;                                   // F of the upper half's last row at column c-1
  uint32_t hbot = 0, fbot = 0;
  int xnext = (sl == 0 && work) ? (int)X0[0] : 0;
  int xcur = 0;                                        // code of the upper half's previous column
  uint32_t hb = L::splat(-a.ge - gsh);                 // T[-1][c] of the column lane 0 works on (band 0)
  const bool top = b == 0;
  const bool last_band = b + 1 >= nb;
  const uint4* pl = reinterpret_cast<const uint4*>(prof) + sl;

  auto step = [&](int t, auto checked) {
    constexpr bool kChecked = decltype(checked)::value;
    const int c = t - 2 * sl;   // the upper half's column; the lower half's is c - 1
    uint32_t hin = __shfl_up_sync(0xffffffffu, hbot, 1, W);
    uint32_t fin = __shfl_up_sync(0xffffffffu, fbot, 1, W);
    const int xl = xnext;
    if (kChecked) {
      if (c + 1 >= 0 && c + 1 < Lx0) xnext = X0[c + 1];
    } else if (W == 32 || work) {
      xnext = X0[min(c + 1, Lx0 - 1)];
    }
    const bool up_on = kChecked ? (c >= 0 && c < Lx0) : (W == 32 || work);
    const bool lo_on = kChecked ? (c >= 1 && c - 1 < Lx0) : (W == 32 || work);
    if (up_on && sl == 0) {
      hin = top ? hb : (uint32_t)rd[2 * c];
      fin = top ? SENT : (uint32_t)rd[2 * c + 1];
    }
    if (!kChecked || c >= 0) hb = L::add(hb, NGEA);
    const uint32_t mid_cur = s.H[RH - 1];   // the upper half's last row at column c-1
    if (lo_on) {
      fbot = strip_rows3<RH, RH, R, P, W>(s, pl + clamp_code(xcur) * LS, mid_prev, mid_cur, fmid, NGE, NGO);
      hbot = s.H[R - 1];
    }
    if (up_on) {
      const uint32_t diag = hprev;
      hprev = hin;
      fmid = strip_rows3<0, RH, R, P, W>(s, pl + clamp_code(xl) * LS, diag, hin, fin, NGE, NGO);
      mid_prev = mid_cur;
      xcur = xl;
    }
    if (sl == W - 1 && !last_band && lo_on) {
      wr[2 * (c - 1)] = (int32_t)hbot;
      wr[2 * (c - 1) + 1] = (int32_t)fbot;
    }
  };
  // ramp-up (lanes before their columns), steady state (both halves of every
  // lane on a column), ramp-down (lanes past their last column)
  int t = 0;
  const int t1 = Lmin < 2 * W - 1 ? Lmin : 2 * W - 1;
  for (; t < t1; ++t) step(t, std::true_type{});
#pragma unroll 2
  for (; t < Lmin; ++t) step(t, std::false_type{});
  for (; t < Lmax + 2 * W - 1; ++t) step(t, std::true_type{});

  // H[] now holds the last column (T = H - go); the lane owning a pair's last row reports.
  if (wantA0) {
    const int rr = rowA - b * BAND;
    if (rr >= 0 && rr < BAND && sl == rr / R) {
      const int v = L::lo(pick<R>(s.H, rr % R)) + gsh;
      if (jobD) put_score_job(a, jobD, jobld, xo0, yoA, v);
      else put_score(a, xo0, yoA, v);
    }
  }
  if (P == 2 && wantB0) {
    const int rr = rowB - b * BAND;
    if (rr >= 0 && rr < BAND && sl == rr / R) {
      const int v = L::hi(pick<R>(s.H, rr % R)) + gsh;
      if (jobD) put_score_job(a, jobD, jobld, xo0, yoB, v);
      else put_score(a, xo0, yoB, v);
    }
  }
}

// One band (W*R rows starting at b*W*R) of the front's K X (K = 2 for V = 5).
// sl: lane within the front; Lx[k]: length of X k, 0 when it has no pair to
// report (its strip is then not computed; the lanes still take part in the
// shuffles); Lmin / Lmax: smallest / largest Lx over the warp's working X
// (warp-uniform).  scratch: the front's band-boundary buffers, 4 words per
// column per X.
template <int R, int P, int V, int W>
__device__ __forceinline__ void wave_band(const WaveArgs& a, int sl, int b, int nb,
                                          const int8_t* const (&X)[Layout<V>::K], const int (&Lx)[Layout<V>::K],
                                          int Lmin, int Lmax, const uint32_t* __restrict__ prof,
                                          int32_t* __restrict__ scratch, int rowA, int rowB,
                                          const bool (&wantA)[Layout<V>::K], const bool (&wantB)[Layout<V>::K],
                                          const int (&xo)[Layout<V>::K], int yoA, int yoB, float* jobD,
                                          int64_t jobld) {
  using L = Lanes<P>;
  constexpr int K = Layout<V>::K;
  constexpr int VL = Layout<V>::L;
  constexpr int BAND = W * R;
  const uint32_t NGE = L::packed(-a.ge);        // per-half operand of addmax
  const uint32_t NGO = L::arith(-a.go, -a.go);   // word added to H to get H - go
  const uint32_t NGOP = L::packed(-a.go);        // per-half operand: - go
  const uint32_t NGEA = L::arith(-a.ge, -a.ge);  // word added to H[-1][c] to get H[-1][c+1]
  // E[r][-1] = F[-1][c] = -32768 + ge; layouts 2 and 4 keep them shifted by go
  const uint32_t SENT = L::splat(kShortMin + a.ge + ((VL == 2 || VL == 4) ? a.go : 0));

  constexpr int SST = scratch_stride<W>();
  constexpr int LS = Profile<R, W>::kLetterStride;
  BandState<R, P, VL> s[K];
  const int rowbase = b * BAND + sl * R;
  const int gsh = VL == 3 ? a.go : 0;               // layout 3 carries T = H - go instead of H
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      s[k].H[r] = L::splat(-a.ge * (rowbase + r + 1) - gsh);   // H[row][-1] (T for layout 3)
      s[k].E[r] = SENT;                                         // E[row][-1]
      if (VL == 0) s[k].T[(VL == 0) ? r : 0] = L::add(s[k].H[r], NGO);
    }
  uint32_t hprev[K], hbot[K], fbot[K];
  int xnext[K];
  bool work[K];
  const int32_t* rd[K];
  int32_t* wr[K];
  const bool top = b == 0;
  const uint4* pl = reinterpret_cast<const uint4*>(prof) + sl;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    hprev[k] = L::splat(-a.ge * rowbase - gsh);     // H[rowbase-1][-1]: diag of column 0
    hbot[k] = fbot[k] = 0;
    work[k] = Lx[k] > 0;
    rd[k] = scratch + ((size_t)k * 4 * a.scratch_cols + ((b + 1) & 1) * 2 * a.scratch_cols) * SST;   // band b-1
    wr[k] = scratch + ((size_t)k * 4 * a.scratch_cols + (b & 1) * 2 * a.scratch_cols) * SST;
    xnext[k] = (sl == 0 && work[k]) ? (int)X[k][0] : 0;
  }
  uint32_t hb = L::splat(-a.ge - gsh);              // H[-1][c] of the column lane 0 works on (band 0)
  const bool last_band = b + 1 >= nb;

  auto step = [&](int t, auto checked) {
    constexpr bool kChecked = decltype(checked)::value;
    const int c = t - sl;
    uint32_t hin[K], fin[K];
    int xl[K];
    bool on[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if constexpr (W > 1) {
        hin[k] = __shfl_up_sync(0xffffffffu, hbot[k], 1, W);
        fin[k] = __shfl_up_sync(0xffffffffu, fbot[k], 1, W);
      } else {
        hin[k] = hbot[k];   // every lane is lane 0 of its own front: read from the band above below
        fin[k] = fbot[k];
      }
      xl[k] = xnext[k];
      if (kChecked) {
        if (c + 1 >= 0 && c + 1 < Lx[k]) xnext[k] = X[k][c + 1];
      } else if ((W == 32 && K == 1) || work[k]) {
        xnext[k] = X[k][min(c + 1, Lx[k] - 1)];
      }
      on[k] = kChecked ? (c >= 0 && c < Lx[k]) : ((W == 32 && K == 1) || work[k]);
      if (on[k] && sl == 0) {
        hin[k] = top ? hb : (uint32_t)rd[k][(size_t)(2 * c) * SST];
        fin[k] = top ? SENT : (uint32_t)rd[k][(size_t)(2 * c + 1) * SST];
      }
    }
    if (!kChecked || c >= 0) hb = L::add(hb, NGEA);
    bool paired = false;
    if constexpr (K == 2) {
      if (!kChecked && on[0] && on[1]) {
        // both strips on a column: interleaved
        uint32_t diag[2] = {hprev[0], hprev[1]};
        uint32_t f[2] = {fin[0], fin[1]};
        hprev[0] = hin[0];
        hprev[1] = hin[1];
        strip_column_pair<R, P, W>(s, pl + clamp_code(xl[0]) * LS, pl + clamp_code(xl[1]) * LS, diag, hin,
                                   f, NGE, NGO);
        fbot[0] = f[0];
        fbot[1] = f[1];
        hbot[0] = s[0].H[R - 1];
        hbot[1] = s[1].H[R - 1];
        paired = true;
      }
    }
    if (!paired) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (!on[k]) continue;
        const uint32_t diag = hprev[k];
        hprev[k] = hin[k];
        fbot[k] = strip_column<R, P, VL, W>(s[k], pl + clamp_code(xl[k]) * LS, diag, hin[k], fin[k], NGE, NGO,
                                            NGOP);
        hbot[k] = s[k].H[R - 1];
      }
    }
    if (sl == W - 1 && !last_band) {
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (on[k]) {
          wr[k][(size_t)(2 * c) * SST] = (int32_t)hbot[k];
          wr[k][(size_t)(2 * c + 1) * SST] = (int32_t)fbot[k];
        }
    }
  };
  // ramp-up (some lanes before column 0), steady state (every lane of every
  // working strip on a column), ramp-down (some lanes past their last column)
  int t = 0;
  const int t1 = Lmin < W - 1 ? Lmin : W - 1;
  for (; t < t1; ++t) step(t, std::true_type{});
#pragma unroll 2
  for (; t < Lmin; ++t) step(t, std::false_type{});
  for (; t < Lmax + W - 1; ++t) step(t, std::true_type{});

  // H[] now holds the last column; the lane owning a pair's last row reports.
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (wantA[k]) {
      const int rr = rowA - b * BAND;
      if (rr >= 0 && rr < BAND && sl == rr / R) {
        const int v = L::lo(pick<R>(s[k].H, rr % R)) + gsh;
        if (jobD) put_score_job(a, jobD, jobld, xo[k], yoA, v);
        else put_score(a, xo[k], yoA, v);
      }
    }
    if (P == 2 && wantB[k]) {
      const int rr = rowB - b * BAND;
      if (rr >= 0 && rr < BAND && sl == rr / R) {
        const int v = L::hi(pick<R>(s[k].H, rr % R)) + gsh;
        if (jobD) put_score_job(a, jobD, jobld, xo[k], yoB, v);
        else put_score(a, xo[k], yoB, v);
      }
    }
  }
}

// Copies the bytes [p, p + n) into shared memory at dst + lead, where p - lead
// is the word at or below p, and returns lead.  The thread takes words w0,
// w0 + stride, ...: a word that lies inside [begin, end) goes by a 4-byte
// cp.async (completed by cp_async_wait_all), the partial words at either edge
// of the buffer by plain byte loads (bytes outside it read as 0); nothing
// outside [begin, end) is read.
__device__ __forceinline__ int stage_bytes(int8_t* dst, const int8_t* p, int n, const int8_t* begin,
                                           const int8_t* end, int w0, int stride) {
  const uintptr_t base = (uintptr_t)p & ~(uintptr_t)3;
  const int lead = (int)((uintptr_t)p - base);
  const int words = (lead + n + 3) >> 2;
  for (int w = w0; w < words; w += stride) {
    const uintptr_t src = base + 4 * (uintptr_t)w;
    if (src >= (uintptr_t)begin && src + 4 <= (uintptr_t)end) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(dst + 4 * w);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uintptr_t q = src + j;
        dst[4 * w + j] = (q >= (uintptr_t)begin && q < (uintptr_t)end) ? *reinterpret_cast<const int8_t*>(q)
                                                                       : (int8_t)0;
      }
    }
  }
  return lead;
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

template <int R, int P, int V>
struct MinBlocks {
  static constexpr int rows = V == 5 ? 2 * R : R;   // register rows per lane
  static constexpr int value = V == 0 ? 1 : (rows <= 8 ? 4 : (rows <= 16 ? 3 : 2));
};

template <int R, int P, int V, int W>
__global__ void __launch_bounds__(kWaveThreads, (MinBlocks<R, P, V>::value)) wave_kernel(const WaveArgs a) {
  constexpr int S = 32 / W;                // fronts per warp
  constexpr int K = Layout<V>::K;          // X per front
  constexpr int BAND = W * R;
  static_assert(R % 2 == 0 && R >= 4 && R <= 32, "rows per lane: even, 4 to 32");
  static_assert(W == 1 || W == 8 || W == 16 || W == 32, "front width");
  static_assert(W > 1 || K == 1, "one pair per thread holds one X per front");
  extern __shared__ __align__(16) uint32_t prof[];   // Profile<R, W>: [letter][Q][front lane][4]
  __shared__ __align__(16) int8_t s_sub[kLetters * kLetters + 4];
  // the rows of the band of both Y sequences, staged by cp.async for the profile build
  constexpr int kTile = (BAND + 8 + 15) / 16 * 16;
  __shared__ __align__(16) int8_t s_ytile[2][kTile];
  __shared__ long long s_job;

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int sl = lane % W;                 // lane within the front
  const int seg = lane / W;                // front within the warp
  // the substitution matrix, staged by cp.async (visible after the job loop's first barrier)
  stage_bytes(s_sub, a.sub, kLetters * kLetters, a.sub, a.sub + kLetters * kLetters, threadIdx.x, blockDim.x);
  cp_async_wait_all();
  // band-boundary scratch of the front: its own block of 4 x scratch_cols
  // words per X, or (W = 1) one column of the CTA's interleaved block
  int32_t* scratch =
      W == 1 ? a.scratch + (size_t)blockIdx.x * kWaveThreads * K * 4 * (size_t)a.scratch_cols + threadIdx.x
             : a.scratch + ((size_t)(blockIdx.x * kWaveWarps + warp) * S + seg) * K * 4 * (size_t)a.scratch_cols;

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
    const int LyA = a.ylen[y0];
    const int LyB = has_b ? a.ylen[y1] : 0;
    const int8_t* YA = a.codes + a.ystart[y0];
    const int8_t* YB = has_b ? a.codes + a.ystart[y1] : YA;
    const int8_t* X[K];
    int Lx[K], xo[K];
    bool wantA[K], wantB[K];
    unsigned lmax = 0, lmin = 0x7fffffffu;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = xbase + (int)(chunk * (kWaveWarps * S * K)) + (warp * S + seg) * K + k;
      const bool active = i < xbase + nX;
      X[k] = a.codes + (active ? a.xstart[i] : 0);
      wantA[k] = active && (!a.triangle || i <= y0);
      wantB[k] = active && has_b && (!a.triangle || i <= y1);
      if (P == 2 && a.check_bound && active) {
        // A carry out of an overflowing low half would reach the high half of
        // the same word, so an unsafe A pair also sends B to the re-run queue.
        const bool safeA = int16_safe(a, i, y0);
        const bool safeB = !has_b || int16_safe(a, i, y1);
        if (wantA[k] && !safeA) {
          if (sl == 0) queue_rerun(a, i, y0);
          wantA[k] = false;
        }
        if (wantB[k] && !(safeA && safeB)) {
          if (sl == 0) queue_rerun(a, i, y1);
          wantB[k] = false;
        }
      }
      Lx[k] = (wantA[k] || wantB[k]) ? a.xlen[i] : 0;
      xo[k] = active ? a.xorig[i] : 0;
      if (Lx[k] > 0) {
        lmax = max(lmax, (unsigned)Lx[k]);
        lmin = min(lmin, (unsigned)Lx[k]);
      }
    }
    const int Lmax = (int)__reduce_max_sync(0xffffffffu, lmax);
    const int Lmin = (int)__reduce_min_sync(0xffffffffu, lmin);
    const int rows = LyA > LyB ? LyA : LyB;
    const int nb = (rows + BAND - 1) / BAND;
    const int yoA = a.yorig[y0];
    const int yoB = has_b ? a.yorig[y1] : 0;

    for (int b = 0; b < nb; ++b) {
      // the band's rows of YA and YB into the tiles (every warp is done with
      // the previous band's profile and tiles after the barrier that follows)
      const int na = min(BAND, LyA - b * BAND), nbr = min(BAND, LyB - b * BAND);
      const int leadA = na > 0 ? stage_bytes(s_ytile[0], YA + b * BAND, na, a.codes, a.codes_end, threadIdx.x,
                                             kWaveThreads)
                               : 0;
      const int leadB = (P == 2 && nbr > 0) ? stage_bytes(s_ytile[1], YB + b * BAND, nbr, a.codes, a.codes_end,
                                                          threadIdx.x, kWaveThreads)
                                            : 0;
      cp_async_wait_all();
      __syncthreads();
      for (int e = threadIdx.x; e < kLetters * BAND; e += kWaveThreads) {
        const int x = e / BAND;
        const int row = e - x * BAND;
        const int grow = b * BAND + row;
        const int gsh = Layout<V>::L == 3 ? a.go : 0;   // layout 3 adds the profile to T = H - go
        const int sa = (grow < LyA ? (int)s_sub[clamp_code(s_ytile[0][leadA + row]) * kLetters + x] : 0) + gsh;
        uint32_t w;
        if (P == 2) {
          const int sb = (grow < LyB ? (int)s_sub[clamp_code(s_ytile[1][leadB + row]) * kLetters + x] : 0) + gsh;
          w = Lanes<2>::arith(sa, sb);
        } else {
          w = (uint32_t)sa;
        }
        prof[Profile<R, W>::index(x, row)] = w;
      }
      __syncthreads();
      if (Lmax > 0) {
        if constexpr (V == 6)
          wave_band_split<R, P, W>(a, sl, b, nb, X[0], Lx[0], Lmin, Lmax, prof, scratch, LyA - 1, LyB - 1, wantA[0],
                                   wantB[0], xo[0], yoA, yoB, jobD, jobld);
        else
          wave_band<R, P, V, W>(a, sl, b, nb, X, Lx, Lmin, Lmax, prof, scratch, LyA - 1, LyB - 1, wantA, wantB, xo,
                                yoA, yoB, jobD, jobld);
      }
    }
  }
}

template <int R, int P, int V, int W>
void prepare_one() {
  const size_t smem = Profile<R, W>::kBytes;
  cudaFuncSetAttribute(wave_kernel<R, P, V, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int R, int P, int V, int W>
cudaError_t launch_one(const WaveArgs& a, int grid, cudaStream_t s) {
  const size_t smem = Profile<R, W>::kBytes;
  wave_kernel<R, P, V, W><<<grid, kWaveThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int R, int P, int V, int W>
int occupancy_one() {
  const size_t smem = Profile<R, W>::kBytes;
  cudaFuncSetAttribute(wave_kernel<R, P, V, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wave_kernel<R, P, V, W>, kWaveThreads, smem) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

// Rows per lane that exist only in the most used forms (int16x2 wavefronts,
// layouts 2 to 4): they refine the band sizes between the multiples of 4.
constexpr bool extra_rows(int R) { return R % 4 != 0 || R == 28; }

// The (P, V, W) combinations that exist for R rows per lane.  For R a multiple
// of 4 (not 28): W = 32 with every P and V; the narrow fronts (W = 16, 8) on
// int16x2 lanes with V = 0, 2, 3, 4 or 5; one pair per thread (W = 1: every
// lane its own front, bands of R rows) on int16x2 lanes with V = 0, 2, 3 or 4.
// The other R: int16x2 wavefronts of 32, 16 or 8 lanes with V = 2, 3 or 4.
inline bool wave_variant_exists(int R, int P, int V, int W) {
  if (V == 6) return !extra_rows(R) && R % 8 == 0 && P == 2 && (W == 32 || W == 16 || W == 8);
  if (extra_rows(R)) return P == 2 && (W == 32 || W == 16 || W == 8) && V >= 2 && V <= 4;
  if (W == 32) return (P == 1 || P == 2) && V >= 0 && V <= 5;
  if (W == 1) return P == 2 && (V == 0 || V == 2 || V == 3 || V == 4);
  return (W == 16 || W == 8) && P == 2 && (V == 0 || V == 2 || V == 3 || V == 4 || V == 5);
}

// Entry points of one rows-per-lane template (every existing P, V, W).
template <int R>
struct Entry {
  static constexpr bool kExtra = extra_rows(R);
  template <int P, int W, class Fn>
  static auto with_v(int V, Fn&& fn) {
    using std::integral_constant;
    if constexpr (W > 1 && !kExtra) {
      if (V == 5) return fn(integral_constant<int, P>{}, integral_constant<int, 5>{}, integral_constant<int, W>{});
    }
    if constexpr (W > 1 && !kExtra && P == 2 && R % 8 == 0) {
      if (V == 6) return fn(integral_constant<int, P>{}, integral_constant<int, 6>{}, integral_constant<int, W>{});
    }
    if (V == 4) return fn(integral_constant<int, P>{}, integral_constant<int, 4>{}, integral_constant<int, W>{});
    if (V == 3) return fn(integral_constant<int, P>{}, integral_constant<int, 3>{}, integral_constant<int, W>{});
    if constexpr (kExtra) {
      return fn(integral_constant<int, P>{}, integral_constant<int, 2>{}, integral_constant<int, W>{});
    } else {
      if (V == 2) return fn(integral_constant<int, P>{}, integral_constant<int, 2>{}, integral_constant<int, W>{});
      if constexpr (W == 32) {
        if (V == 1) return fn(integral_constant<int, P>{}, integral_constant<int, 1>{}, integral_constant<int, W>{});
      }
      return fn(integral_constant<int, P>{}, integral_constant<int, 0>{}, integral_constant<int, W>{});
    }
  }
  template <class Fn>
  static auto with(int P, int V, int W, Fn&& fn) {
    if constexpr (kExtra) {
      if (W == 16) return with_v<2, 16>(V, fn);
      if (W == 8) return with_v<2, 8>(V, fn);
      return with_v<2, 32>(V, fn);
    } else {
      if (W == 1) return with_v<2, 1>(V, fn);
      if (W == 16) return with_v<2, 16>(V, fn);
      if (W == 8) return with_v<2, 8>(V, fn);
      if (P == 2) return with_v<2, 32>(V, fn);
      return with_v<1, 32>(V, fn);
    }
  }
  static cudaError_t launch(int P, int V, int W, const WaveArgs& a, int grid, cudaStream_t s) {
    if (!wave_variant_exists(R, P, V, W)) return cudaErrorInvalidValue;
    return with(P, V, W, [&](auto p, auto v, auto w) {
      return launch_one<R, decltype(p)::value, decltype(v)::value, decltype(w)::value>(a, grid, s);
    });
  }
  static void prepare(int P, int V, int W) {
    if (!wave_variant_exists(R, P, V, W)) return;
    with(P, V, W, [&](auto p, auto v, auto w) {
      prepare_one<R, decltype(p)::value, decltype(v)::value, decltype(w)::value>();
      return 0;
    });
  }
  static int occupancy(int P, int V, int W) {
    if (!wave_variant_exists(R, P, V, W)) return 1;
    return with(P, V, W, [&](auto p, auto v, auto w) {
      return occupancy_one<R, decltype(p)::value, decltype(v)::value, decltype(w)::value>();
    });
  }
};

}  // namespace wave

// Per-template dispatch tables (one translation unit per R).
#define NWG_WAVE_ROWS(X) X(4) X(8) X(12) X(16) X(18) X(20) X(22) X(24) X(26) X(28) X(30) X(32)
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
