// nj.cu -- neighbor joining on the device: the join loop of
// SpeciesBlock::buildTree (SpeciesBlock.cpp:845-1343) with modifyMatrix
// (:710-842), buildGblRowSums (:426-453) and TreeNode::join (TreeNode.cpp:
// 31-58), for one process and one GPU.
//
// Semantics kept from the reference:
//  * D is float, row/column slots; the new node takes the slot of the smaller
//    id and keeps its stale diagonal (:787-841, :952, :1186);
//  * T is double: T[k] += (float)(tmp - (Dik + Djk)) with tmp the float
//    ((Dik + Djk) - d) / 2 (:793-801); the new node's T is the sequential
//    double sum of its tmp values in ascending id order (:799, :818); rebuilds
//    recompute every T as a sequential double sum of its row over active
//    nodes in ascending id order, diagonal included (:432-452);
//  * rebuilds after max(n0*0.5, 200) joins, then every n*0.5, never below
//    200 active nodes (:864, :1226-1247);
//  * the pair chosen is the minimum of q = ((double)d*(n-2) - T[a]) - T[b]
//    with (a, b) the order of the reference's Dij record (node-id order for
//    records made by buildBins, :549-558; row-slot order for records made when
//    a node is inserted, :1280-1292), ties to the larger max(i,j) then the
//    larger min(i,j) (:1165-1179).
// The reference reaches that minimum through bins and heaps (:456-674,
// :1019-1144), which only prune -- except that a pair popped from a heap is
// valued as d*(n-2) - (T[a] + T[b]) (:1119-1121) and more than QDA=8 equal
// values are cut by nth_element (:1148).  Each step therefore also checks
// whether any other pair comes within the two roundings of the winner, or
// more than four pairs tie exactly; such a step is counted as ambiguous (its
// pick is still the exact-argmin one).  The heap-size rebuild trigger
// (:1206-1223) cannot fire while the heaps hold at most the entries pushed
// since the last build; that bound is tracked and any check it cannot exclude
// is counted.
//
// Search per join:
//  1. one streaming pass over the live triangle of D (4 B per live pair):
//     q in float, fl(fl(fl(d*(n-2)) - Tf_r) - Tf_c) with Tf the float copy of
//     T; per row its two smallest q (and the column of the smallest), overall
//     the minimum and the largest magnitude M = |d|(n-2) + |T_r| + |T_c|.
//     Every float q is within E = 8 * 2^-24 * M of the exact q.
//  2. the candidates are the pairs whose float q is at most min + 3E: when
//     each row within that threshold has one such pair (its second smallest q
//     is beyond), they are those rows' minima; otherwise the rows are scanned
//     again into a list (up to 2048 candidates; beyond that, as in the
//     one-CTA form always, the CTAs reduce their first candidates and a
//     second scan counts the ties).  Each candidate gets its exact double q in
//     both roundings.
// The winner follows the tie-break; the ambiguity check runs over the
// candidates: any pair left out has q > winner + E, beyond reach of either
// rounding.  All floating-point operations use the _rn intrinsics in the
// reference's evaluation order (no contraction).
//
// Four launch forms run a job's whole join loop (several jobs per launch in
// the serving loop):
//  * one CTA with the job in its shared memory (up to 160 taxa);
//  * one thread-block cluster with the matrix in its distributed shared
//    memory (up to 768 taxa);
//  * one cluster with the matrix in global memory (up to 2048 taxa);
//  * the whole GPU, one cooperative launch per segment between compactions
//    (compacted to the live slots, in slot order), above that.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "nwg_ctx.h"

namespace nwg {

namespace {

constexpr int kNJMaxN = 8192;
constexpr int kCandCap = 2048;         // candidate list capacity per join (longer lists are not read)

struct NJDev {
  float* D;            // n0 x ld, slots
  double* T;           // per slot
  float* Tf;           // per slot, (float)T; NaN at dead and padding slots (ld entries)
  int* slot;           // per node id (2n0-1), -1 dead
  int* node;           // per slot: node id, -1 dead
  int* act;            // active node ids ascending [n0 + 1]
  int* na;             // active count
  int* g32;            // [2] candidates of the fallback scan
  unsigned long long* stats;  // [0] ambiguous steps, [1] tie steps, [2] internal errors,
                              // [3] open heap-size checks, [4] rebuilds (cluster form)
  nwg_join* joins;
  int n0;              // slots
  int ld;              // row stride of D (floats), a multiple of 4
  int cand_cap;        // candidate list capacity
  int pad;
};

__device__ __forceinline__ int ford(float f) {
  // order-preserving map float -> int (for atomicMin / atomicMax)
  const int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7FFFFFFF;
}


// Exponent of the lowest set bit of a nonzero float (INT_MAX for zero).
__device__ __forceinline__ int low_bit_exp(float f) {
  const unsigned b = __float_as_uint(f) & 0x7FFFFFFFu;
  if (b == 0) return INT_MAX;
  const unsigned e = b >> 23, m = b & 0x7FFFFFu;
  if (e == 0) return -149 + __ffs(m) - 1;
  return (int)e - 150 + __ffs(m | 0x800000u) - 1;
}

// Exponent of the highest set bit of |f| (f = m * 2^(e) with m in [1, 2)),
// INT_MIN for 0.
__device__ __forceinline__ int top_bit_exp(float f) {
  const unsigned b = __float_as_uint(f) & 0x7FFFFFFFu;
  if (b == 0) return INT_MIN;
  const unsigned e = b >> 23, m = b & 0x7FFFFFu;
  if (e == 0) return -149 + (31 - __clz(m));
  return (int)e - 127;
}

// f as a signed integer count of 2^lowexp (exact: lowexp is at most the
// lowest set bit of f, and |f| < 2^(lowexp + 49) is checked by the caller).
__device__ __forceinline__ long long float_units(float f, int lowexp) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
  if (e == 0 && m == 0) return 0;
  const long long mant = e == 0 ? (long long)m : (long long)(m | 0x800000u);
  const int sh = (e == 0 ? -149 : (int)e - 150) - lowexp;   // value = mant * 2^(sh + lowexp)
  // a right shift drops only zero bits: lowexp <= the lowest set bit of f
  const long long v = sh >= 0 ? mant << sh : mant >> (-sh);
  return (b >> 31) ? -v : v;
}

// A sequential double sum of floats equals any-order sum when every partial
// sum is exact: all terms are multiples of 2^lowexp and sum|x| < 2^(53+lowexp)
// (a multiple of 2^lowexp below that magnitude has at most 53 significant
// bits).  absum is itself a rounded sum, hence the 1e-12 slack.
__device__ __forceinline__ bool sum_is_exact(double absum, int lowexp) {
  if (lowexp == INT_MAX) return true;   // every term is zero
  return absum * (1.0 + 1e-12) < ldexp(1.0, 53 + lowexp);
}

// Sequential row sums (buildGblRowSums): one warp per active row; the lanes'
// any-order sum is used when it is provably exact, else lane 0 sums in order.
__global__ void rowsum_kernel(NJDev s, const int* abort) {
  if (*(volatile const int*)abort) return;   // a segment gave up: the lists were never written
  const int na = *s.na;
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (k >= na) return;
  const int sk = s.slot[s.act[k]];
  const float* row = s.D + (size_t)sk * s.ld;
  double part = 0.0, ab = 0.0;
  int lowexp = INT_MAX;
  for (int j = lane; j < na; j += 32) {
    const float x = row[s.slot[s.act[j]]];
    part = __dadd_rn(part, (double)x);
    ab = __dadd_rn(ab, (double)fabsf(x));
    lowexp = min(lowexp, low_bit_exp(x));
  }
  for (int o = 16; o > 0; o >>= 1) {
    part = __dadd_rn(part, __shfl_down_sync(0xffffffffu, part, o));
    ab = __dadd_rn(ab, __shfl_down_sync(0xffffffffu, ab, o));
    lowexp = min(lowexp, __shfl_down_sync(0xffffffffu, lowexp, o));
  }
  if (lane == 0) {
    double sum = part;
    if (!sum_is_exact(ab, lowexp)) {
      sum = 0.0;
      for (int j = 0; j < na; ++j) sum = __dadd_rn(sum, (double)row[s.slot[s.act[j]]]);
    }
    s.T[sk] = sum;
    s.Tf[sk] = (float)sum;
  }
}

// The pick's outcome: the winner's position among the candidates, the
// candidates within rounding of it (itself included) as ties or as pairs the
// reference's heap rounding could have preferred, and a failed pick.
struct PickOut {
  int idx;
  unsigned ties, amb;
  bool error;       // no candidate, or the list overflowed
};

// The pick's statistics: ambiguous step, tie step or internal error.
__device__ __forceinline__ void record_pick(const NJDev& s, const PickOut& r) {
  if (r.error) atomicAdd(&s.stats[2], 1ull);
  else if (r.amb > 0 || r.ties > 4) atomicAdd(&s.stats[0], 1ull);
  else if (r.ties > 1) atomicAdd(&s.stats[1], 1ull);
}

// ---- large n: one cooperative launch over the whole GPU per segment ---------
// Every CTA takes part in every phase of every join, with two grid barriers
// per join in the usual case:
//  P  the live triangle, one row pair (p, n0-1-p) per warp, warps numbered
//     across CTAs first; 16-byte loads (rows are padded to a multiple of 4
//     floats and the padding's float row sums are NaN).  Per row its two
//     smallest float q and the column of the smallest (grmin, grec); per CTA
//     the smallest q and the largest magnitude (part).
//  -- barrier --
//  K  every CTA reduces the CTA partials to the candidate threshold and finds
//     the rows whose minimum is within it.  When each such row's second
//     smallest q is beyond the threshold, the candidates are exactly those
//     rows' minima: every CTA evaluates them (exact q in both roundings) and
//     takes the same winner.  Otherwise (ties, close pairs) every CTA scans
//     its slice of the selected rows into a global list and, after one more
//     barrier, picks from it.
//  J  every CTA applies the join to its own share of the slots (T, the new
//     row and column, the new row's values with their exponent range and
//     integer sum) and of the active list (shifted into the other list).
//  -- barrier --
// At the start of the next join (or at the end of the segment) every CTA
// combines the shares into the new node's row sum and writes it, with the
// dead slot's NaN and the slot -> node map, itself -- the same values in
// every CTA, so each CTA reads its own writes; CTA 0 keeps the join record
// (branch lengths are filled in after the loop) and the id -> slot map.
// Rebuilds (row sums) and compactions run between segments.

struct GCand {
  long long k1, k2;   // order-preserving integer keys of q1 and q2
  double q1;          // record-order rounding of q (SpeciesBlock.cpp:1051)
  double ta, tb;      // T of the slots of a and b
  int a, b;           // node ids, a < b
  int sa, sb;         // their slots
  float d;
  int pad;
};

// An entry of the fallback scan's list: the keys and the node ids (the
// winner's slots, d and row sums are read again after the pick).
struct KCand {
  long long k1, k2;
  int a, b;
};

struct GridNJ {
  unsigned* bar;        // [0] barrier arrivals (counts up from 0 per launch)
  int* abort;           // set when a barrier wait gave up; every CTA then leaves
  int* act2;            // the other active list (the join writes the shifted list there)
  int* grmin;           // per slot: smallest float q of the row's pairs (ordered int)
  int4* grec;           // per slot: second smallest q (ordered int), column and distance of the smallest
  double* tsnap;        // per slot: T as the pass saw it (the pick reads these, never T itself)
  float* tv;            // per slot: the new row's value
  float* part;          // [2 * grid]: per CTA smallest q and largest magnitude
  long long* jsum;      // [2 * grid]: per CTA integer sum and sum of magnitudes (units of 2^jexp)
  int* jexp;            // [2 * grid]: per CTA lowest and highest exponent of its values
  KCand* cand;          // the candidate list of the fallback scan
  KCand* cbest;         // [grid]: per CTA its first candidate of the fallback scan
};

constexpr long long kBarrierSpinCycles = 4000000000ll;   // about two seconds: no phase takes a millisecond
constexpr int kFastRows = 32;                             // candidate rows the direct pick evaluates
constexpr int kGridMax = 256;                             // CTAs of the cooperative launch, at most

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier of a cooperative launch (all CTAs resident): arrivals count up,
// the k-th barrier waits for k * gridDim.x arrivals.  A wait that exceeds the
// spin limit, or sees another CTA's abort, sets the abort flag and returns
// false; the caller then leaves the kernel.
__device__ bool grid_barrier(const GridNJ& g, unsigned& target) {
  __shared__ int s_ok;
  __syncthreads();
  target += gridDim.x;
  if (threadIdx.x == 0) {
    // release: this CTA's writes (ordered before by the CTA barrier) are
    // visible to every CTA that acquires the count
    red_release_add(&g.bar[0], 1u);
    int ok = 1;
    const long long t0 = clock64();
    while ((int)(ld_acquire_u32(&g.bar[0]) - target) < 0) {
      if (*(volatile int*)g.abort) {
        ok = 0;
        break;
      }
      if (clock64() - t0 > kBarrierSpinCycles) {
        atomicExch(g.abort, 1);
        ok = 0;
        break;
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The CTAs that run one job's join loop: the whole cooperative grid (large n)
// or one thread-block cluster (a job per cluster).
struct Team {
  int rank, size;
};

template <bool CL>
__device__ __forceinline__ bool team_sync(const GridNJ& g, unsigned& target) {
  if constexpr (CL) {
    cooperative_groups::this_cluster().sync();
    return true;
  } else {
    return grid_barrier(g, target);
  }
}

// Order-preserving map double -> int64 (finite values; -0 and +0 map alike).
__device__ __forceinline__ long long dkey(double q) {
  long long b = __double_as_longlong(q);
  if ((b & 0x7FFFFFFFFFFFFFFFll) == 0) b = 0;
  return b >= 0 ? b : b ^ 0x7FFFFFFFFFFFFFFFll;
}

// Exact double of u * 2^e (|u| < 2^53, the result a normal double).
__device__ __forceinline__ double units_to_double(long long u, int e) {
  if (u == 0) return 0.0;
  const unsigned long long m = (unsigned long long)(u < 0 ? -u : u);
  const int msb = 63 - __clzll((long long)m);
  const unsigned long long bits = ((unsigned long long)(msb + e + 1023) << 52) |
                                  ((m << (52 - msb)) & 0xFFFFFFFFFFFFFull) | (u < 0 ? (1ull << 63) : 0ull);
  return __longlong_as_double(bits);
}

// One element of P: q, the row's two smallest (with the column of the
// smallest) and the magnitude |x| + |tc| (the row's |tr| is added per row).
// At a dead or padding slot tc is NaN: q and the magnitude are NaN and drop
// out (comparisons with NaN are false; fmaxf ignores NaN).
__device__ __forceinline__ void pass_elem(float d, float tc, int c, float tr, float nm2f, float& m1, float& m2,
                                          int& c1, float& mag) {
  const float x = __fmul_rn(d, nm2f);
  const float q = __fsub_rn(__fsub_rn(x, tr), tc);
  const bool lt = q < m1;
  m2 = lt ? m1 : fminf(m2, q);
  c1 = lt ? c : c1;
  m1 = lt ? q : m1;
  mag = fmaxf(mag, __fadd_rn(fabsf(x), fabsf(tc)));
}

// Odd joins scan every row backwards: the lines the previous pass read last
// are still in L2 when the triangle is a little larger than L2.
__device__ void grid_pass(const NJDev& s, const GridNJ& g, Team tm, float nm2f, bool rev) {
  __shared__ float sq[32], sm[32];
  const int lane = threadIdx.x & 31;
  const int n0 = s.n0, nv = s.ld >> 2;
  const int nw = tm.size * (int)(blockDim.x >> 5);
  const int npairs = (n0 + 1) >> 1;
  const float4* Tf4 = reinterpret_cast<const float4*>(s.Tf);
  float qmin = FLT_MAX, mmax = 0.f;
  for (int p = (int)(threadIdx.x >> 5) * tm.size + tm.rank; p < npairs; p += nw) {
    for (int h = 0; h < 2; ++h) {
      if (n0 - 1 - p == p && h) break;
      const int r = (h != (int)rev) ? n0 - 1 - p : p;
      const float tr = s.Tf[r];
      if (tr != tr) {   // dead slot
        if (lane == 0) g.grmin[r] = 0x7F7FFFFF;
        continue;
      }
      const double Tr = s.T[r];
      const float* row = s.D + (size_t)r * s.ld;
      float m1 = FLT_MAX, m2 = FLT_MAX, mag = 0.f;
      int c1 = -1;
      const int c0 = r + 1, v0 = (c0 + 3) >> 2;
      // columns c0 .. 4*v0-1 (at most three) one by one
      if (lane < 4 * v0 - c0 && c0 + lane < n0)
        pass_elem(row[c0 + lane], s.Tf[c0 + lane], c0 + lane, tr, nm2f, m1, m2, c1, mag);
      const float4* row4 = reinterpret_cast<const float4*>(row);
      auto vec = [&](int v) {
        const float4 d = row4[v];
        const float4 tc = Tf4[v];
        pass_elem(d.x, tc.x, 4 * v, tr, nm2f, m1, m2, c1, mag);
        pass_elem(d.y, tc.y, 4 * v + 1, tr, nm2f, m1, m2, c1, mag);
        pass_elem(d.z, tc.z, 4 * v + 2, tr, nm2f, m1, m2, c1, mag);
        pass_elem(d.w, tc.w, 4 * v + 3, tr, nm2f, m1, m2, c1, mag);
      };
      if (!rev) {
#pragma unroll 4
        for (int v = v0 + lane; v < nv; v += 32) vec(v);
      } else {
#pragma unroll 4
        for (int v = nv - 1 - lane; v >= v0; v -= 32) vec(v);
      }
      // the row's two smallest over the warp (an equal pair makes m2 = m1)
      for (int o = 16; o > 0; o >>= 1) {
        const float om1 = __shfl_xor_sync(0xffffffffu, m1, o);
        const float om2 = __shfl_xor_sync(0xffffffffu, m2, o);
        const int oc1 = __shfl_xor_sync(0xffffffffu, c1, o);
        const bool take = om1 < m1 || (om1 == m1 && oc1 < c1);
        const float lo = take ? om1 : m1, hi = take ? m1 : om1;
        m2 = fminf(hi, fminf(m2, om2));
        m1 = lo;
        c1 = take ? oc1 : c1;
        mag = fmaxf(mag, __shfl_xor_sync(0xffffffffu, mag, o));
      }
      if (lane == 0) {
        // the pick reads only what the pass wrote: a fast CTA's join share may
        // already be changing T and D while a slow one still picks
        g.grmin[r] = ford(m1);
        g.grec[r] = make_int4(ford(m2), c1, __float_as_int(c1 >= 0 ? row[c1] : 0.f), 0);
        g.tsnap[r] = Tr;
      }
      qmin = fminf(qmin, m1);
      mmax = fmaxf(mmax, __fadd_rn(mag, fabsf(tr)));
    }
  }
  if (lane == 0) {
    sq[threadIdx.x >> 5] = qmin;
    sm[threadIdx.x >> 5] = mmax;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nwb = (int)(blockDim.x >> 5);
    qmin = lane < nwb ? sq[lane] : FLT_MAX;
    mmax = lane < nwb ? sm[lane] : 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      qmin = fminf(qmin, __shfl_xor_sync(0xffffffffu, qmin, o));
      mmax = fmaxf(mmax, __shfl_xor_sync(0xffffffffu, mmax, o));
    }
    if (lane == 0) {
      g.part[2 * tm.rank] = qmin;
      g.part[2 * tm.rank + 1] = mmax;
    }
  }
}

// A candidate from its pair: slots r, c with their node ids, T and d.
__device__ __forceinline__ GCand make_cand(int r, int c, int ur, int uc, double Tr, double Tc, float d, double nm2,
                                           int watermark) {
  GCand cd;
  const bool rfirst = ur < uc;
  cd.a = rfirst ? ur : uc;
  cd.b = rfirst ? uc : ur;
  cd.sa = rfirst ? r : c;
  cd.sb = rfirst ? c : r;
  cd.ta = rfirst ? Tr : Tc;
  cd.tb = rfirst ? Tc : Tr;
  cd.d = d;
  cd.pad = 0;
  // record order (SpeciesBlock.cpp:1051): node-id order, except for a record
  // made when the newer node was inserted (row-slot order)
  const bool swap = cd.b >= watermark && cd.sb < cd.sa;
  const double nmd = __dmul_rn((double)d, nm2);
  cd.q1 = swap ? __dsub_rn(__dsub_rn(nmd, cd.tb), cd.ta) : __dsub_rn(__dsub_rn(nmd, cd.ta), cd.tb);
  cd.k1 = dkey(cd.q1);
  cd.k2 = dkey(__dsub_rn(nmd, __dadd_rn(cd.ta, cd.tb)));   // heap rounding (:1119-1121)
  return cd;
}

// Winner (smallest q1, then larger b, then larger a) and the ambiguity / tie
// counts over nc candidates, by one warp; load(k) gives candidate k.
template <class Load>
__device__ PickOut pick_keys(int nc, Load&& load) {   // load(k) has k1, k2, a, b
  const int l = threadIdx.x & 31;
  long long bk = LLONG_MAX, bk2 = LLONG_MAX;
  int ba = INT_MAX, bb = -1, bi = -1;
  for (int k = l; k < nc; k += 32) {
    const auto c = load(k);
    if (c.k1 < bk || (c.k1 == bk && (c.b > bb || (c.b == bb && c.a > ba)))) {
      bk = c.k1;
      bk2 = c.k2;
      ba = c.a;
      bb = c.b;
      bi = k;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const long long q = __shfl_xor_sync(0xffffffffu, bk, o);
    const long long q2 = __shfl_xor_sync(0xffffffffu, bk2, o);
    const int a2 = __shfl_xor_sync(0xffffffffu, ba, o);
    const int b2 = __shfl_xor_sync(0xffffffffu, bb, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
    if (q < bk || (q == bk && (b2 > bb || (b2 == bb && a2 > ba)))) {
      bk = q;
      bk2 = q2;
      ba = a2;
      bb = b2;
      bi = i2;
    }
  }
  // every lane holds the winner; any other candidate whose smaller rounding
  // reaches the winner's larger one could have been picked by the reference
  const long long hiw = max(bk, bk2);
  const bool robust_w = bk == bk2;
  unsigned ties = 0, amb = 0;
  for (int k = l; k < nc; k += 32) {
    const auto c = load(k);
    if (min(c.k1, c.k2) > hiw) continue;
    if (c.a == ba && c.b == bb) ++ties;
    else if (robust_w && c.k1 == c.k2 && c.k1 == bk) ++ties;
    else ++amb;
  }
  for (int o = 16; o > 0; o >>= 1) {
    ties += __shfl_xor_sync(0xffffffffu, ties, o);
    amb += __shfl_xor_sync(0xffffffffu, amb, o);
  }
  PickOut r;
  r.idx = bi;
  r.ties = ties;
  r.amb = amb;
  r.error = bb < 0;
  return r;
}

// Long candidate lists (wide exact ties, e.g. hundreds of identical
// sequences, whose pairs all tie): above kListPickMax candidates one warp's
// pick over the list would be slow, and the list does not hold them.  Instead
// every CTA reduces its threads' first candidates in the pick's order, the
// winner is the first of those, and a second scan counts the ties and
// ambiguous pairs against it with pick_keys' rule.  (The one-CTA form always
// picks this way, without the list.)
constexpr int kListPickMax = kCandCap;

__device__ __forceinline__ KCand kc_none() { return KCand{LLONG_MAX, LLONG_MAX, INT_MAX, -1}; }

// x before y in the pick's order: smaller q1 key, then larger b, then larger a.
__device__ __forceinline__ bool kc_first(const KCand& x, const KCand& y) {
  return x.k1 < y.k1 || (x.k1 == y.k1 && (x.b > y.b || (x.b == y.b && x.a > y.a)));
}

__device__ __forceinline__ KCand ld_kcand(const KCand* p) {   // written by other CTAs: from L2
  return KCand{__ldcg(&p->k1), __ldcg(&p->k2), __ldcg(&p->a), __ldcg(&p->b)};
}

__device__ __forceinline__ KCand warp_first(KCand x) {
  for (int o = 16; o > 0; o >>= 1) {
    KCand y;
    y.k1 = __shfl_xor_sync(0xffffffffu, x.k1, o);
    y.k2 = __shfl_xor_sync(0xffffffffu, x.k2, o);
    y.a = __shfl_xor_sync(0xffffffffu, x.a, o);
    y.b = __shfl_xor_sync(0xffffffffu, x.b, o);
    if (kc_first(y, x)) x = y;
  }
  return x;
}

// The CTA's first candidate, valid in warp 0 (sw: 32 entries of shared memory,
// not reused before the next CTA barrier).
__device__ KCand cta_first(KCand x, KCand* sw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = ((int)blockDim.x + 31) >> 5;
  x = warp_first(x);
  if (lane == 0) sw[warp] = x;
  __syncthreads();
  if (warp == 0) x = warp_first(lane < nw ? sw[lane] : kc_none());
  return x;
}

// pick_keys' tie and ambiguity rule for candidate c against the winner w.
__device__ __forceinline__ void count_vs(const KCand& c, const KCand& w, unsigned& ties, unsigned& amb) {
  if (min(c.k1, c.k2) > max(w.k1, w.k2)) return;
  if (c.a == w.a && c.b == w.b) ++ties;
  else if (w.k1 == w.k2 && c.k1 == c.k2 && c.k1 == w.k1) ++ties;
  else ++amb;
}

// The CTA's counts into cnt[0] (ties) and cnt[1] (ambiguous pairs).
__device__ __forceinline__ void add_counts(unsigned ties, unsigned amb, int* cnt) {
  for (int o = 16; o > 0; o >>= 1) {
    ties += __shfl_xor_sync(0xffffffffu, ties, o);
    amb += __shfl_xor_sync(0xffffffffu, amb, o);
  }
  if ((threadIdx.x & 31) == 0 && (ties | amb)) {
    atomicAdd(&cnt[0], (int)ties);
    atomicAdd(&cnt[1], (int)amb);
  }
}

// K.  Returns 1 when the winner is in *win, 0 when the fallback scan is
// needed (the same in every CTA).
__device__ int grid_pick_direct(const NJDev& s, const GridNJ& g, Team tm, double nm2, float nm2f, int watermark, GCand* win,
                                PickOut* pk, float* sthr) {
  __shared__ int rows[kFastRows];
  __shared__ GCand fc[kFastRows];
  __shared__ int nrows, s_ok;
  const int n0 = s.n0;
  // the row minima load together with the CTA partials (n0 <= 8 * blockDim)
  constexpr int kPerThread = 8;
  int rm[kPerThread];
#pragma unroll
  for (int t = 0; t < kPerThread; ++t) {
    const int p = (int)threadIdx.x + t * (int)blockDim.x;
    rm[t] = p < n0 ? g.grmin[p] : 0x7F7FFFFF;
  }
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    float q = FLT_MAX, m = 0.f;
    // every partial in flight at once (at most kGridMax CTAs)
#pragma unroll
    for (int t = 0; t < kGridMax / 32; ++t) {
      const int b = l + 32 * t;
      if (b < tm.size) {
        const float2 pm = reinterpret_cast<const float2*>(g.part)[b];
        q = fminf(q, pm.x);
        m = fmaxf(m, pm.y);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      q = fminf(q, __shfl_xor_sync(0xffffffffu, q, o));
      m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if (l == 0) {
      *sthr = q + 3.f * (8.f * 5.9604645e-8f * m) + 1e-30f;
      nrows = 0;
    }
  }
  __syncthreads();
  const float thr = *sthr;
  const int othr = ford(thr);
#pragma unroll
  for (int t = 0; t < kPerThread; ++t) {
    if (rm[t] <= othr) {
      const int k = atomicAdd(&nrows, 1);
      if (k < kFastRows) rows[k] = (int)threadIdx.x + t * (int)blockDim.x;
    }
  }
  __syncthreads();
  const int nr = nrows;
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    int ok = nr >= 1 && nr <= kFastRows;
    if (ok && l < nr) {
      const int r = rows[l];
      const int4 rec = g.grec[r];
      const int c = rec.y;
      if (rec.x <= othr || c < 0) {
        ok = 0;   // a second pair of the row within the threshold
      } else {
        const int ur = s.node[r], uc = s.node[c];
        const double Tr = g.tsnap[r], Tc = g.tsnap[c];
        const float d = __int_as_float(rec.z);
        fc[l] = make_cand(r, c, ur, uc, Tr, Tc, d, nm2, watermark);
        if (ur < 0 || uc < 0) ok = 0;
      }
    }
    ok = __all_sync(0xffffffffu, ok);
    PickOut r{};
    if (ok && nr == 1) {
      r.idx = 0;     // one candidate: the winner, a tie with itself only
      r.ties = 1;
      r.amb = 0;
      r.error = false;
    } else if (ok) {
      r = pick_keys(nr, [&](int k) { return fc[k]; });
    }
    if (l == 0) {
      s_ok = ok;
      if (ok) {
        *pk = r;
        *win = fc[r.idx];
      }
    }
  }
  __syncthreads();
  return s_ok;
}

// K, fallback: visit(pred, candidate) for this CTA's share of the pairs of
// every row within the threshold, called by whole warps together (pred is
// false on lanes without a candidate in that step); the same pairs on every
// call of one join.  Up to kSplitRows rows, the team's warps split each row's
// columns; more rows (wide ties), one warp per row, warps numbered across the
// team, lanes over the columns.
constexpr int kSplitRows = 16;

template <class Visit>
__device__ void grid_cand_scan(const NJDev& s, const GridNJ& g, Team tm, float nm2f, double nm2, int watermark,
                               float thr, Visit&& visit) {
  constexpr int kRows = 512;
  __shared__ int rows[kRows];
  __shared__ int nrows;
  const int n0 = s.n0;
  const int othr = ford(thr);
  if (threadIdx.x == 0) nrows = 0;
  __syncthreads();
  for (int p = threadIdx.x; p < n0; p += blockDim.x) {
    if (g.grmin[p] <= othr) {
      const int t = atomicAdd(&nrows, 1);
      if (t < kRows) rows[t] = p;
    }
  }
  __syncthreads();
  const bool all = nrows > kRows;   // more near-minimal rows than the list holds: every row
  const int nr = all ? n0 : nrows;
  const int lane = threadIdx.x & 31;
  const int wpc = (int)blockDim.x >> 5;
  const int gw = tm.rank * wpc + ((int)threadIdx.x >> 5), nw = tm.size * wpc;
  // columns c0 + lane, c0 + cstep + lane, ... of row r (c0 and cstep the same in the warp)
  auto scan_row = [&](int r, int c0, int cstep) {
    const int ur = s.node[r];
    if (ur < 0 || g.grmin[r] > othr) return;
    const float tr = s.Tf[r];
    const double Tr = s.T[r];
    const float* row = s.D + (size_t)r * s.ld;
    for (int cb = c0; cb < n0; cb += cstep) {
      const int c = cb + lane;
      bool pred = false;
      KCand kc = kc_none();
      if (c < n0) {
        const int uc = s.node[c];
        const float d = row[c];
        const float q = __fsub_rn(__fsub_rn(__fmul_rn(d, nm2f), tr), s.Tf[c]);
        if (uc >= 0 && q <= thr) {
          const GCand cd = make_cand(r, c, ur, uc, Tr, s.T[c], d, nm2, watermark);
          kc = KCand{cd.k1, cd.k2, cd.a, cd.b};
          pred = true;
        }
      }
      visit(pred, kc);
    }
  };
  if (nr <= kSplitRows) {
    for (int t = 0; t < nr; ++t) {   // every CTA's list holds the same rows, in its own order
      const int r = all ? t : rows[t];
      scan_row(r, r + 1 + 32 * gw, 32 * nw);
    }
  } else {
    // rows by slot (an order the same in every CTA); scan_row skips the others
    for (int r = gw; r < n0; r += nw) scan_row(r, r + 1, 32);
  }
}

// A warp's candidates of one scan step into the list, one atomic per warp.
// s.g32[2] ends at the number of candidates when that is at most
// kListPickMax, else above kListPickMax: a warp that saw the count pass it
// stops counting (full, the same in the warp).
__device__ __forceinline__ void list_push(const NJDev& s, const GridNJ& g, bool pred, const KCand& c, bool& full) {
  const unsigned bal = __ballot_sync(0xffffffffu, pred);
  if (bal == 0 || full) return;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0) base = atomicAdd(&s.g32[2], __popc(bal));
  base = __shfl_sync(0xffffffffu, base, 0);
  const int idx = base + __popc(bal & ((1u << lane) - 1u));
  if (pred && idx < s.cand_cap) g.cand[idx] = c;
  full = base + __popc(bal) > kListPickMax;
}

// The scan into the candidate list; returns this thread's first candidate
// (reduced over the CTA only when the list is not used).
__device__ KCand grid_cand(const NJDev& s, const GridNJ& g, Team tm, float nm2f, double nm2, int watermark, float thr) {
  KCand first = kc_none();
  bool full = false;
  grid_cand_scan(s, g, tm, nm2f, nm2, watermark, thr, [&](bool pred, const KCand& c) {
    list_push(s, g, pred, c, full);
    if (pred && kc_first(c, first)) first = c;
  });
  return first;
}

// The second scan of a long list: ties and ambiguous pairs against the winner
// w into s.g32[0] and s.g32[1].
__device__ void grid_cand_count(const NJDev& s, const GridNJ& g, Team tm, float nm2f, double nm2, int watermark,
                                float thr, const KCand& w) {
  unsigned ties = 0, amb = 0;
  grid_cand_scan(s, g, tm, nm2f, nm2, watermark, thr, [&](bool pred, const KCand& c) {
    if (pred) count_vs(c, w, ties, amb);
  });
  add_counts(ties, amb, s.g32);
}

// J: this CTA's share of the slots (SpeciesBlock.cpp:787-841: tmp = ((Dik +
// Djk) - d) / 2 in float, T[k] += (float)(tmp - (Dik + Djk)), the new row and
// column of slot si, whose diagonal keeps i's old value) and of the active
// list; the share's exponent range and integer sum go to jexp / jsum.  The
// shares hold at most one slot and one list position per thread (the launch
// has at least n0 / blockDim CTAs).
// An exact sum of floats as u * 2^e (|u| < 2^62), with a = sum of |values| in
// the same units and t the highest exponent; e = INT_MAX for no values.  A
// sum whose values span 48 bits or more is not kept (the row's range then
// rules out the integer sum anyway; e and t stay exact).
struct USum {
  long long u, a;
  int e, t;
};

__device__ __forceinline__ void usum_add(USum& x, const USum& y) {
  if (y.e == INT_MAX) return;
  if (x.e == INT_MAX) {
    x = y;
    return;
  }
  const int e = min(x.e, y.e), t = max(x.t, y.t);
  if (t - e >= 48) {
    x.u = x.a = 0;
  } else {
    const long long mx = 1ll << (x.e - e), my = 1ll << (y.e - e);
    x.u = x.u * mx + y.u * my;
    x.a = x.a * mx + y.a * my;
  }
  x.e = e;
  x.t = t;
}

__device__ __forceinline__ void usum_warp(USum& x) {
  for (int o = 16; o > 0; o >>= 1) {
    USum y;
    y.u = __shfl_xor_sync(0xffffffffu, x.u, o);
    y.a = __shfl_xor_sync(0xffffffffu, x.a, o);
    y.e = __shfl_xor_sync(0xffffffffu, x.e, o);
    y.t = __shfl_xor_sync(0xffffffffu, x.t, o);
    usum_add(x, y);
  }
}

__device__ void grid_join_share(const NJDev& s, const GridNJ& g, Team tm, const GCand& w, int na, const int* act, int* act2) {
  __shared__ USum swarp[32];
  const int i = w.a, j = w.b, si = w.sa, sj = w.sb;
  const float dmin = w.d;
  const int n0 = s.n0;
  const size_t ld = (size_t)s.ld;
  const int per = (n0 + tm.size - 1) / tm.size;
  const int p = tm.rank * per + (int)threadIdx.x;
  USum x;
  x.u = x.a = 0;
  x.e = INT_MAX;
  x.t = INT_MIN;
  if ((int)threadIdx.x < per && p < n0) {
    const int v = s.node[p];
    const float Dik = s.D[(size_t)si * ld + p];
    const float Djk = s.D[(size_t)sj * ld + p];
    const double Tk = s.T[p];
    if (v >= 0 && p != si && p != sj) {
      const float sumf = __fadd_rn(Dik, Djk);
      const float tmp = __fmul_rn(__fsub_rn(sumf, dmin), 0.5f);
      const double t = __dadd_rn(Tk, (double)__fsub_rn(tmp, sumf));
      s.T[p] = t;
      s.Tf[p] = (float)t;
      s.D[(size_t)p * ld + si] = tmp;
      s.D[(size_t)si * ld + p] = tmp;
      g.tv[p] = tmp;
      if (tmp != 0.f) {
        x.e = low_bit_exp(tmp);
        x.t = top_bit_exp(tmp);
        x.u = float_units(tmp, x.e);
        x.a = x.u < 0 ? -x.u : x.u;
      }
    }
  }
  // the active list without i and j (ascending ids), shifted into act2
  const int kper = (na + tm.size - 1) / tm.size;
  const int k = tm.rank * kper + (int)threadIdx.x;
  if ((int)threadIdx.x < kper && k < na) {
    const int v = act[k];
    if (v != i && v != j) act2[k - (v > i) - (v > j)] = v;
  }
  // the share's slots sit in its first warps (per <= blockDim)
  const int nwv = (per + 31) >> 5;
  if ((int)(threadIdx.x >> 5) < nwv) usum_warp(x);
  if (nwv > 1) {
    if ((threadIdx.x & 31) == 0 && (int)(threadIdx.x >> 5) < nwv) swarp[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w2 = 1; w2 < nwv; ++w2) usum_add(x, swarp[w2]);
  }
  if (threadIdx.x == 0) {
    g.jsum[2 * tm.rank] = x.u;
    g.jsum[2 * tm.rank + 1] = x.a;
    g.jexp[2 * tm.rank] = x.e;
    g.jexp[2 * tm.rank + 1] = x.t;
  }
}

// After the barrier that ends join `step`: the new node's row sum
// (SpeciesBlock.cpp:799, :818 -- the sequential double sum in ascending id
// order, taken as the exact integer sum of the shares when that provably
// equals it), written by every CTA for itself; CTA 0 also writes the join
// record (TreeNode::join's inputs; the lengths follow after the loop) and the
// id -> slot map.  When the integer sum cannot be used, CTA 0 runs the
// sequential loop and one more grid barrier follows.
template <bool CL>
__device__ bool grid_join_apply(const NJDev& s, const GridNJ& g, Team tm, const GCand& w, const PickOut& pk, int step,
                                int n, const int* act_old, int* act_new, unsigned& target) {
  __shared__ double s_sum;
  __shared__ int s_exact;
  const int i = w.a, j = w.b, si = w.sa, sj = w.sb;
  const int m_n = n - step, next = n + step;
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    // at most kGridMax CTAs: kGridMax / 32 shares per lane, held in registers
    constexpr int kPer = kGridMax / 32;
    int je[kPer];
    long long jsv[kPer], jav[kPer];
    int lowexp = INT_MAX, topexp = INT_MIN;
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int b = l + 32 * t;
      je[t] = INT_MAX;
      jsv[t] = jav[t] = 0;
      if (b < tm.size) {
        je[t] = g.jexp[2 * b];
        jsv[t] = g.jsum[2 * b];
        jav[t] = g.jsum[2 * b + 1];
        topexp = max(topexp, g.jexp[2 * b + 1]);
      }
      lowexp = min(lowexp, je[t]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      lowexp = min(lowexp, __shfl_xor_sync(0xffffffffu, lowexp, o));
      topexp = max(topexp, __shfl_xor_sync(0xffffffffu, topexp, o));
    }
    // every value below 2^49 units of 2^lowexp: a share's sum (at most 8192
    // values) moved to those units stays below 2^62
    const bool fits = lowexp == INT_MAX || topexp - lowexp < 48;
    long long isum = 0, iabs = 0;
    if (fits && lowexp != INT_MAX) {
#pragma unroll
      for (int t = 0; t < kPer; ++t) {
        if (je[t] == INT_MAX) continue;   // a share without values
        const long long m = 1ll << (je[t] - lowexp);
        isum += jsv[t] * m;
        iabs += jav[t] * m;
      }
      for (int o = 16; o > 0; o >>= 1) {
        isum += __shfl_xor_sync(0xffffffffu, isum, o);
        iabs += __shfl_xor_sync(0xffffffffu, iabs, o);
      }
    }
    if (l == 0) {
      if (lowexp == INT_MAX) {
        s_sum = 0.0;                                 // every value is zero
        s_exact = 1;
      } else if (fits && iabs < (1ll << 53)) {
        s_sum = units_to_double(isum, lowexp);       // exact: |isum| < 2^53
        s_exact = 1;
      } else {
        s_exact = 0;
      }
    }
  }
  __syncthreads();
  const bool exact = s_exact != 0;
  if (threadIdx.x == 0) {
    if (exact) {
      s.T[si] = s_sum;
      s.Tf[si] = __double2float_rn(s_sum);
    } else if (tm.rank == 0) {
      double sum = 0.0;   // the reference's loop: active ids ascending, i and j skipped
      for (int k = 0; k < m_n; ++k) {
        const int v = act_old[k];
        if (v != i && v != j) sum = __dadd_rn(sum, (double)g.tv[s.slot[v]]);
      }
      s.T[si] = sum;
      s.Tf[si] = __double2float_rn(sum);
    }
    s.Tf[sj] = __int_as_float(0x7FC00000);   // dead: NaN
    s.node[sj] = -1;
    s.node[si] = next;
    if (tm.rank == 0) {
      nwg_join& J = s.joins[step];
      J.i = i;
      J.j = j;
      J.node = next;
      J.n = m_n;
      J.d = w.d;
      J.pad = 0.f;
      J.q = w.q1;
      J.ti = w.ta;
      J.tj = w.tb;
      act_new[m_n - 2] = next;
      *s.na = m_n - 1;
      s.slot[j] = -1;
      s.slot[i] = -1;
      s.slot[next] = si;
      s.g32[0] = s.g32[1] = s.g32[2] = 0;   // every CTA took its pick before the barrier
      record_pick(s, pk);
    }
  }
  if (!exact) return team_sync<CL>(g, target);   // T[si] from CTA 0
  __syncthreads();
  return true;
}

// One join of the team: pass, pick, share.  False when the team stops (a
// barrier gave up or the pick failed -- the same in every CTA).
template <bool CL>
__device__ bool team_join(const NJDev& s, const GridNJ& g, Team tm, int step, int n, int watermark, int*& act,
                          int*& act2, PickOut& spick, GCand& swin, float& sthr, unsigned& target) {
  const int m_n = n - step;
  const float nm2f = (float)(m_n - 2);
  const double nm2 = (double)(m_n - 2);
  grid_pass(s, g, tm, nm2f, (step & 1) != 0);
  if (!team_sync<CL>(g, target)) return false;
  if (!grid_pick_direct(s, g, tm, nm2, nm2f, watermark, &swin, &spick, &sthr)) {
    const KCand tfirst = grid_cand(s, g, tm, nm2f, nm2, watermark, sthr);
    if (!team_sync<CL>(g, target)) return false;
    // the winner's pair again, as the scan read it (row = the smaller slot)
    auto rederive = [&](const KCand& w) {
      const int sa = s.slot[w.a], sb = s.slot[w.b];
      const int r0 = min(sa, sb), c0 = max(sa, sb);
      swin = make_cand(r0, c0, s.node[r0], s.node[c0], s.T[r0], s.T[c0], s.D[(size_t)r0 * s.ld + c0], nm2,
                       watermark);
    };
    const int ncount = *(volatile int*)&s.g32[2];   // the same in every CTA
    if (ncount <= min(s.cand_cap, kListPickMax)) {
      if (threadIdx.x < 32) {
        const PickOut r = pick_keys(ncount, [&](int k) { return g.cand[k]; });
        if (threadIdx.x == 0) {
          spick = r;
          if (!r.error) rederive(g.cand[r.idx]);
        }
      }
      __syncthreads();
    } else {
      __shared__ KCand sw[32];
      __shared__ KCand sfirst;
      const KCand cf = cta_first(tfirst, sw);
      if (threadIdx.x == 0) g.cbest[tm.rank] = cf;
      if (!team_sync<CL>(g, target)) return false;
      if (threadIdx.x < 32) {
        const PickOut r = pick_keys(tm.size, [&](int k) { return ld_kcand(&g.cbest[k]); });
        if (threadIdx.x == 0) sfirst = r.error ? kc_none() : ld_kcand(&g.cbest[r.idx]);
      }
      __syncthreads();
      const KCand w = sfirst;
      grid_cand_count(s, g, tm, nm2f, nm2, watermark, sthr, w);
      if (!team_sync<CL>(g, target)) return false;
      if (threadIdx.x == 0) {
        spick.idx = 0;
        spick.ties = (unsigned)__ldcg(&s.g32[0]);
        spick.amb = (unsigned)__ldcg(&s.g32[1]);
        spick.error = w.b < 0;
        if (!spick.error) rederive(w);
      }
      __syncthreads();
    }
  }
  if (spick.error) {
    if (tm.rank == 0 && threadIdx.x == 0) record_pick(s, spick);
    return false;
  }
  grid_join_share(s, g, tm, swin, m_n, act, act2);
  int* t = act;
  act = act2;
  act2 = t;
  return team_sync<CL>(g, target);
}

// Joins step0 .. step1-1 of an n-taxon job over the whole GPU (the active
// count before join t is n - t).
__global__ void __launch_bounds__(1024, 1) nj_grid_kernel(NJDev s, GridNJ g, int step0, int step1, int n,
                                                         int watermark) {
  __shared__ PickOut spick;
  __shared__ GCand swin;
  __shared__ float sthr;
  const Team tm{(int)blockIdx.x, (int)gridDim.x};
  unsigned target = 0;
  if (*(volatile int*)g.abort) return;   // an earlier segment gave up: every CTA leaves
  for (int p = (int)(blockIdx.x * blockDim.x + threadIdx.x); p < s.n0; p += (int)(gridDim.x * blockDim.x))
    g.grmin[p] = 0x7F7FFFFF;   // ordered int of FLT_MAX
  if (blockIdx.x == 0 && threadIdx.x == 0) s.g32[0] = s.g32[1] = s.g32[2] = 0;
  if (!grid_barrier(g, target)) return;
  int* act = s.act;
  int* act2 = g.act2;
  for (int step = step0; step < step1; ++step) {
    // the previous join's new list is act, its old one act2
    if (step > step0 && !grid_join_apply<false>(s, g, tm, swin, spick, step - 1, n, act2, act, target)) return;
    if (!team_join<false>(s, g, tm, step, n, watermark, act, act2, spick, swin, sthr, target)) return;
  }
  if (step1 > step0) grid_join_apply<false>(s, g, tm, swin, spick, step1 - 1, n, act2, act, target);
}

// TreeNode::join (TreeNode.cpp:31-58) for a recorded join: L_i = (d + (T_i -
// T_j)/(n-2)) / 2, L_j likewise, n = 2 gives d/2 each, a negative side is
// clamped to 0 and moved to the other.
__device__ void join_lengths(nwg_join& J) {
  const double half = 0.5;
  double li, lj;
  if (J.n == 2) {
    li = lj = __dmul_rn((double)J.d, half);
  } else {
    const double nm2 = (double)(J.n - 2);
    li = __dmul_rn(half, __dadd_rn((double)J.d, __ddiv_rn(__dsub_rn(J.ti, J.tj), nm2)));
    lj = __dmul_rn(half, __dadd_rn((double)J.d, __ddiv_rn(__dsub_rn(J.tj, J.ti), nm2)));
  }
  if (li < 0.0) {
    lj = __dsub_rn(lj, li);
    li = 0.0;
  } else if (lj < 0.0) {
    li = __dsub_rn(li, lj);
    lj = 0.0;
  }
  J.len_i = li;
  J.len_j = lj;
}

__global__ void nj_lengths_kernel(nwg_join* joins, int count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) join_lengths(joins[k]);
}

// Compaction, part 1 (one CTA): map[p] = new slot of live slot p (ascending),
// T / Tf / node into the new slots, slot[v] of every live node remapped.
__global__ void __launch_bounds__(1024) compact_map_kernel(NJDev s, int* map, double* T2, float* Tf2, int* node2,
                                                           int nslots, const int* abort) {
  if (*(volatile const int*)abort) return;
  __shared__ int wsum[33];
  const int n0 = s.n0;
  const int chunk = (n0 + blockDim.x - 1) / blockDim.x;
  const int p0 = threadIdx.x * chunk;
  int keep = 0;
  for (int p = p0; p < p0 + chunk && p < n0; ++p) keep += s.node[p] >= 0;
  int incl = keep;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if ((threadIdx.x & 31) >= o) incl += y;
  }
  if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      const int t = wsum[w];
      wsum[w] = acc;
      acc += t;
    }
    wsum[32] = acc;
  }
  __syncthreads();
  int q = wsum[threadIdx.x >> 5] + incl - keep;
  for (int p = p0; p < p0 + chunk && p < n0; ++p) {
    const int v = s.node[p];
    if (v >= 0) {
      map[p] = q;
      T2[q] = s.T[p];
      Tf2[q] = s.Tf[p];
      node2[q] = v;
      ++q;
    } else {
      map[p] = -1;
    }
  }
  __syncthreads();
  for (int v = threadIdx.x; v < nslots; v += blockDim.x) {
    const int p = s.slot[v];
    if (p >= 0) s.slot[v] = map[p];
  }
}

// Compaction, part 2: D2[map[p]][map[c]] = D[p][c] for live p, c (one block per old row).
__global__ void __launch_bounds__(256) compact_copy_kernel(NJDev s, const int* map, float* D2, int ld2,
                                                           const int* abort) {
  if (*(volatile const int*)abort) return;
  const int p = blockIdx.x;
  const int np = map[p];
  if (np < 0) return;
  const float* row = s.D + (size_t)p * s.ld;
  float* out = D2 + (size_t)np * ld2;
  for (int c = threadIdx.x; c < s.n0; c += blockDim.x) {
    const int nc = map[c];
    if (nc >= 0) out[nc] = row[c];
  }
}

// ---- one job per thread-block cluster (serving and up to 2048 taxa) --------
// The same phases as the large-n form, with the C CTAs of a cluster as the
// team and hardware cluster barriers between the phases; the reference's
// rebuild schedule runs inside the kernel (row sums over the cluster, no
// compaction: the matrix stays in L2).

struct NJJob {
  NJDev s;
  GridNJ g;
  int n;
  int pad;
};

// Sequential row sums (buildGblRowSums, SpeciesBlock.cpp:426-453) over the
// active list, one warp per row, warps w0, w0 + wstride, ...; the lanes'
// any-order sum is used when it is provably exact, else lane 0 sums in order.
__device__ void team_rowsums(const NJDev& s, const int* act, int w0, int wstride) {
  const int na = *s.na;
  const int lane = threadIdx.x & 31;
  for (int k = w0; k < na; k += wstride) {
    const int sk = s.slot[act[k]];
    const float* row = s.D + (size_t)sk * s.ld;
    double part = 0.0, ab = 0.0;
    int lowexp = INT_MAX;
    for (int j = lane; j < na; j += 32) {
      const float x = row[s.slot[act[j]]];
      part = __dadd_rn(part, (double)x);
      ab = __dadd_rn(ab, (double)fabsf(x));
      lowexp = min(lowexp, low_bit_exp(x));
    }
    for (int o = 16; o > 0; o >>= 1) {
      part = __dadd_rn(part, __shfl_down_sync(0xffffffffu, part, o));
      ab = __dadd_rn(ab, __shfl_down_sync(0xffffffffu, ab, o));
      lowexp = min(lowexp, __shfl_down_sync(0xffffffffu, lowexp, o));
    }
    if (lane == 0) {
      double sum = part;
      if (!sum_is_exact(ab, lowexp)) {
        sum = 0.0;
        for (int j = 0; j < na; ++j) sum = __dadd_rn(sum, (double)row[s.slot[act[j]]]);
      }
      s.T[sk] = sum;
      s.Tf[sk] = __double2float_rn(sum);
    }
  }
}

template <int C>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(1024, 1) nj_cluster_kernel(const NJJob* jobs, int njobs) {
  __shared__ PickOut spick;
  __shared__ GCand swin;
  __shared__ float sthr;
  __shared__ NJJob sjob;   // the job's descriptor (shared memory keeps registers free)
  const int job = (int)blockIdx.x / C;   // the same for every CTA of the cluster
  if (job >= njobs) return;
  if (threadIdx.x == 0) sjob = jobs[job];
  __syncthreads();
  const NJDev& s = sjob.s;
  const GridNJ& g = sjob.g;
  const int n = sjob.n;
  const Team tm{(int)cooperative_groups::this_cluster().block_rank(), C};
  const int w0 = tm.rank * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);
  const int wstride = C * (int)(blockDim.x >> 5);
  const int t0 = tm.rank * (int)blockDim.x + (int)threadIdx.x, tstride = C * (int)blockDim.x;
  unsigned target = 0;   // (grid barriers only)
  for (int k = t0; k < 2 * n - 1; k += tstride) s.slot[k] = k < n ? k : -1;
  for (int k = t0; k < n; k += tstride) {
    s.node[k] = k;
    s.act[k] = k;
    g.grmin[k] = 0x7F7FFFFF;
  }
  for (int k = n + t0; k < s.ld; k += tstride) s.Tf[k] = __int_as_float(0x7FC00000);   // padding: NaN
  if (tm.rank == 0 && threadIdx.x == 0) {
    *s.na = n;
    s.g32[0] = s.g32[1] = s.g32[2] = 0;
    s.stats[0] = s.stats[1] = s.stats[2] = s.stats[3] = s.stats[4] = 0;
  }
  cooperative_groups::this_cluster().sync();
  if (n < 2) return;
  team_rowsums(s, s.act, w0, wstride);
  cooperative_groups::this_cluster().sync();
  // the reference's schedule (SpeciesBlock.cpp:864, :1206-1247)
  const int kBinT = 30 * 31 / 2;
  int steps = max((int)((float)n * 0.5f), 200);
  int pq_ck = 500;
  long long ave0 = (((long long)(n - 1) * n) / 2) / kBinT;
  long long ub = ((long long)n * (n - 1)) / 2;
  int watermark = n;
  int* act = s.act;
  int* act2 = g.act2;
  bool pending = false;   // a join whose row sum and maps are still to be written
  for (int step = 0; step < n - 1; ++step) {
    if (pending) grid_join_apply<true>(s, g, tm, swin, spick, step - 1, n, act2, act, target);
    if (!team_join<true>(s, g, tm, step, n, watermark, act, act2, spick, swin, sthr, target)) return;
    pending = true;
    if (--pq_ck == 0) {
      pq_ck = 500;
      if (steps > 0 && (double)(ub / kBinT) / (double)ave0 > 2.0 && tm.rank == 0 && threadIdx.x == 0) s.stats[3] += 1;
    }
    const int m_after = n - step - 1;
    if (steps == 0) {
      grid_join_apply<true>(s, g, tm, swin, spick, step, n, act2, act, target);
      pending = false;
      cooperative_groups::this_cluster().sync();
      team_rowsums(s, act, w0, wstride);
      if (tm.rank == 0 && threadIdx.x == 0) s.stats[4] += 1;
      watermark = n + step + 1;
      steps = (m_after < 200) ? INT_MAX : (int)((float)m_after * 0.5f);
      ave0 = (((long long)(m_after - 1) * m_after) / 2) / kBinT;
      ub = ((long long)m_after * (m_after - 1)) / 2;
      cooperative_groups::this_cluster().sync();
    } else {
      --steps;
      ub += m_after - 1;
    }
  }
  if (pending) grid_join_apply<true>(s, g, tm, swin, spick, n - 2, n, act2, act, target);
  cooperative_groups::this_cluster().sync();
  for (int k = t0; k < n - 1; k += tstride) join_lengths(s.joins[k]);
}

// ---- small jobs: the whole join loop in one CTA ----------------------------
// Up to kCtaNJMax taxa one CTA holds the job in its shared memory: the rows,
// T, the float row sums, the maps and the active lists.  A thread scans its
// own folded row pair sequentially (no per-row warp reduction), and every
// phase boundary is a CTA barrier; the new node's row sum is complete when the
// join share's block reduction is.  The arithmetic is that of the other forms.

constexpr int kCtaNJMax = 160;   // above it a cluster's shared memory is faster (measured crossover near 170)
constexpr int kCtaThreads = 256;

struct CtaLayout {
  int ldl;
  size_t rows, tf, t, node, slot, act_a, act_b, grm, grc, tv, bytes;
};

__host__ __device__ inline CtaLayout cta_layout(int n) {
  auto al = [](size_t x) { return (x + 15) / 16 * 16; };
  CtaLayout L;
  L.ldl = (n + 3) & ~3;
  size_t o = 0;
  L.rows = o; o += al(sizeof(float) * (size_t)n * L.ldl);
  L.tf = o; o += al(sizeof(float) * L.ldl);
  L.t = o; o += al(sizeof(double) * n);
  L.node = o; o += al(sizeof(int) * n);
  L.slot = o; o += al(sizeof(int) * 2 * n);
  L.act_a = o; o += al(sizeof(int) * (n + 1));
  L.act_b = o; o += al(sizeof(int) * (n + 1));
  L.grm = o; o += al(sizeof(int) * n);
  L.grc = o; o += al(sizeof(int4) * n);
  L.tv = o; o += al(sizeof(float) * n);
  L.bytes = o;
  return L;
}

// Block-wide reduction of a USum over kCtaThreads threads (result in thread 0).
__device__ __forceinline__ USum cta_usum(USum x, USum* swarp) {
  usum_warp(x);
  if ((threadIdx.x & 31) == 0) swarp[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int w = 1; w < kCtaThreads / 32; ++w) usum_add(x, swarp[w]);
  return x;
}

__global__ void __launch_bounds__(kCtaThreads, 1) nj_cta_kernel(const NJJob* jobs, int njobs) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ NJJob sjob;
  __shared__ float wq[kCtaThreads / 32], wm[kCtaThreads / 32];
  __shared__ USum swarp[kCtaThreads / 32];
  __shared__ int rows_sel[kFastRows];
  __shared__ GCand fc[kFastRows];
  __shared__ int nsel, s_ok;
  __shared__ PickOut spick;
  __shared__ GCand swin;
  __shared__ float sthr;
  if ((int)blockIdx.x >= njobs) return;
  if (threadIdx.x == 0) sjob = jobs[blockIdx.x];
  __syncthreads();
  const NJDev& s = sjob.s;
  const GridNJ& g = sjob.g;
  const int n = sjob.n;
  const CtaLayout L = cta_layout(n);
  const int ldl = L.ldl;
  float* rows = reinterpret_cast<float*>(smem + L.rows);
  float* Tf = reinterpret_cast<float*>(smem + L.tf);
  double* T = reinterpret_cast<double*>(smem + L.t);
  int* node = reinterpret_cast<int*>(smem + L.node);
  int* slot = reinterpret_cast<int*>(smem + L.slot);
  int* act = reinterpret_cast<int*>(smem + L.act_a);
  int* act2 = reinterpret_cast<int*>(smem + L.act_b);
  int* grm = reinterpret_cast<int*>(smem + L.grm);
  int4* grc = reinterpret_cast<int4*>(smem + L.grc);
  float* tv = reinterpret_cast<float*>(smem + L.tv);
  const int tid = (int)threadIdx.x, nth = kCtaThreads;
  const int lane = tid & 31, warp = tid >> 5;
  for (int e = tid; e < n * ldl; e += nth) {
    const int r = e / ldl, c = e - r * ldl;
    rows[e] = c < n ? s.D[(size_t)r * s.ld + c] : 0.f;
  }
  for (int k = tid; k < ldl; k += nth) Tf[k] = __int_as_float(0x7FC00000);
  for (int k = tid; k < 2 * n; k += nth) slot[k] = k < n ? k : -1;
  for (int k = tid; k < n; k += nth) {
    node[k] = k;
    act[k] = k;
  }
  if (tid == 0) {
    s.g32[2] = 0;
    s.stats[0] = s.stats[1] = s.stats[2] = s.stats[3] = s.stats[4] = 0;
  }
  __syncthreads();
  // row sums (buildGblRowSums): a thread per row, the reference's sequential
  // double sum over the active list in ascending id order
  auto rowsums = [&](int na) {
    for (int k = tid; k < na; k += nth) {
      const int r = slot[act[k]];
      const float* row = rows + (size_t)r * ldl;
      double sum = 0.0;
      for (int j = 0; j < na; ++j) sum = __dadd_rn(sum, (double)row[slot[act[j]]]);
      T[r] = sum;
      Tf[r] = __double2float_rn(sum);
    }
    __syncthreads();
  };
  if (n >= 2) rowsums(n);
  const int kBinT = 30 * 31 / 2;
  int steps = max((int)((float)n * 0.5f), 200);
  int pq_ck = 500;
  long long ave0 = (((long long)(n - 1) * n) / 2) / kBinT;
  long long ub = ((long long)n * (n - 1)) / 2;
  int watermark = n;
  const int npairs = (n + 1) / 2;
  for (int step = 0; step < n - 1; ++step) {
    const int m_n = n - step, next = n + step;
    const float nm2f = (float)(m_n - 2);
    const double nm2 = (double)(m_n - 2);
    // ---- pass: a thread per folded row pair, its rows scanned sequentially
    float qmin = FLT_MAX, mmax = 0.f;
    if (tid < npairs) {
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        const int r = h ? n - 1 - tid : tid;
        if (h && r == tid) break;
        const float tr = Tf[r];
        if (tr != tr) {   // dead
          grm[r] = 0x7F7FFFFF;
          continue;
        }
        const float* row = rows + (size_t)r * ldl;
        float m1 = FLT_MAX, m2 = FLT_MAX, mag = 0.f;
        int c1 = -1;
        // columns r+1 .. up to the next multiple of 4 one by one, then 16-byte
        // vectors (rows padded to ldl floats, the padding's row sums NaN)
        const int v0 = (r + 4) >> 2;
        for (int c = r + 1; c < 4 * v0 && c < n; ++c) pass_elem(row[c], Tf[c], c, tr, nm2f, m1, m2, c1, mag);
        const float4* row4 = reinterpret_cast<const float4*>(row);
        const float4* Tf4 = reinterpret_cast<const float4*>(Tf);
#pragma unroll 2
        for (int v = v0; v < (ldl >> 2); ++v) {
          const float4 d = row4[v];
          const float4 tc = Tf4[v];
          pass_elem(d.x, tc.x, 4 * v, tr, nm2f, m1, m2, c1, mag);
          pass_elem(d.y, tc.y, 4 * v + 1, tr, nm2f, m1, m2, c1, mag);
          pass_elem(d.z, tc.z, 4 * v + 2, tr, nm2f, m1, m2, c1, mag);
          pass_elem(d.w, tc.w, 4 * v + 3, tr, nm2f, m1, m2, c1, mag);
        }
        grm[r] = ford(m1);
        grc[r] = make_int4(ford(m2), c1, __float_as_int(c1 >= 0 ? row[c1] : 0.f), 0);
        qmin = fminf(qmin, m1);
        mmax = fmaxf(mmax, __fadd_rn(mag, fabsf(tr)));
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      qmin = fminf(qmin, __shfl_xor_sync(0xffffffffu, qmin, o));
      mmax = fmaxf(mmax, __shfl_xor_sync(0xffffffffu, mmax, o));
    }
    if (lane == 0) {
      wq[warp] = qmin;
      wm[warp] = mmax;
    }
    __syncthreads();
    if (tid == 0) {
      float q = FLT_MAX, mm = 0.f;
      for (int w = 0; w < nth / 32; ++w) {
        q = fminf(q, wq[w]);
        mm = fmaxf(mm, wm[w]);
      }
      sthr = q + 3.f * (8.f * 5.9604645e-8f * mm) + 1e-30f;
      nsel = 0;
    }
    __syncthreads();
    // ---- pick
    const float thr = sthr;
    const int othr = ford(thr);
    for (int r = tid; r < n; r += nth) {
      if (grm[r] <= othr) {
        const int k = atomicAdd(&nsel, 1);
        if (k < kFastRows) rows_sel[k] = r;
      }
    }
    __syncthreads();
    const int nr = nsel;
    if (warp == 0) {
      int ok = nr >= 1 && nr <= kFastRows;
      if (ok && lane < nr) {
        const int r = rows_sel[lane];
        const int4 rec = grc[r];
        const int c = rec.y;
        if (rec.x <= othr || c < 0) {
          ok = 0;   // a second pair of the row within the threshold
        } else {
          fc[lane] = make_cand(r, c, node[r], node[c], T[r], T[c], __int_as_float(rec.z), nm2, watermark);
        }
      }
      ok = __all_sync(0xffffffffu, ok);
      PickOut pr{};
      if (ok && nr == 1) {
        pr.idx = 0;
        pr.ties = 1;
        pr.amb = 0;
        pr.error = false;
      } else if (ok) {
        pr = pick_keys(nr, [&](int k) { return fc[k]; });
      }
      if (lane == 0) {
        s_ok = ok;
        if (ok) {
          spick = pr;
          swin = fc[pr.idx];
        }
      }
    }
    __syncthreads();
    if (!s_ok) {
      // fallback: the selected rows' pairs within the threshold, scanned
      // twice: the first candidate in the pick's order (block reduction),
      // then the ties and ambiguous pairs against it (pick_keys' rule)
      auto scan = [&](auto&& visit) {
        for (int r = 0; r < n; ++r) {
          if (grm[r] > othr) continue;
          const int ur = node[r];
          const float tr = Tf[r];
          const float* row = rows + (size_t)r * ldl;
          for (int c = r + 1 + tid; c < n; c += nth) {
            const int uc = node[c];
            if (uc < 0) continue;
            const float d = row[c];
            const float q = __fsub_rn(__fsub_rn(__fmul_rn(d, nm2f), tr), Tf[c]);
            if (q > thr) continue;
            const GCand cd = make_cand(r, c, ur, uc, T[r], T[c], d, nm2, watermark);
            visit(KCand{cd.k1, cd.k2, cd.a, cd.b});
          }
        }
      };
      __shared__ KCand skw[32];
      __shared__ KCand sfirst;
      __shared__ unsigned scnt[2];
      KCand first = kc_none();
      scan([&](const KCand& c) {
        if (kc_first(c, first)) first = c;
      });
      first = cta_first(first, skw);
      if (tid == 0) {
        sfirst = first;
        scnt[0] = scnt[1] = 0;
      }
      __syncthreads();
      const KCand wk = sfirst;
      unsigned ties = 0, amb = 0;
      if (wk.b >= 0) scan([&](const KCand& c) { count_vs(c, wk, ties, amb); });
      for (int o = 16; o > 0; o >>= 1) {
        ties += __shfl_xor_sync(0xffffffffu, ties, o);
        amb += __shfl_xor_sync(0xffffffffu, amb, o);
      }
      if (lane == 0 && (ties | amb)) {
        atomicAdd(&scnt[0], ties);
        atomicAdd(&scnt[1], amb);
      }
      __syncthreads();
      if (tid == 0) {
        spick.idx = 0;
        spick.ties = scnt[0];
        spick.amb = scnt[1];
        spick.error = wk.b < 0;
        if (!spick.error) {
          // the winner's pair again, as the scan read it (row = the smaller slot)
          const int sa = slot[wk.a], sb = slot[wk.b];
          const int r0 = min(sa, sb), c0 = max(sa, sb);
          swin = make_cand(r0, c0, node[r0], node[c0], T[r0], T[c0], rows[(size_t)r0 * ldl + c0], nm2, watermark);
        }
      }
      __syncthreads();
      if (spick.error) {
        if (tid == 0) record_pick(s, spick);
        break;
      }
    }
    // ---- join share: a thread per slot
    const GCand w = swin;
    const int i = w.a, j = w.b, si = w.sa, sj = w.sb;
    USum x;
    x.u = x.a = 0;
    x.e = INT_MAX;
    x.t = INT_MIN;
    for (int p = tid; p < n; p += nth) {
      if (node[p] < 0 || p == si || p == sj) continue;
      float* row = rows + (size_t)p * ldl;
      const float sumf = __fadd_rn(row[si], row[sj]);
      const float tmp = __fmul_rn(__fsub_rn(sumf, w.d), 0.5f);
      const double t = __dadd_rn(T[p], (double)__fsub_rn(tmp, sumf));
      T[p] = t;
      Tf[p] = __double2float_rn(t);
      row[si] = tmp;
      rows[(size_t)si * ldl + p] = tmp;
      tv[p] = tmp;
      if (tmp != 0.f) {
        USum y;
        y.e = low_bit_exp(tmp);
        y.t = top_bit_exp(tmp);
        y.u = float_units(tmp, y.e);
        y.a = y.u < 0 ? -y.u : y.u;
        usum_add(x, y);
      }
    }
    for (int k = tid; k < m_n; k += nth) {
      const int v = act[k];
      if (v != i && v != j) act2[k - (v > i) - (v > j)] = v;
    }
    x = cta_usum(x, swarp);   // ends with every thread past the share
    if (tid == 0) {
      double sum;
      if (x.e == INT_MAX) {
        sum = 0.0;
      } else if (x.t - x.e < 48 && x.a < (1ll << 53)) {
        sum = units_to_double(x.u, x.e);   // exact: the sequential sum's value
      } else {
        sum = 0.0;   // the reference's loop: active ids ascending, i and j skipped
        for (int k = 0; k < m_n; ++k) {
          const int v = act[k];
          if (v != i && v != j) sum = __dadd_rn(sum, (double)tv[slot[v]]);
        }
      }
      T[si] = sum;
      Tf[si] = __double2float_rn(sum);
      Tf[sj] = __int_as_float(0x7FC00000);
      node[sj] = -1;
      node[si] = next;
      slot[j] = -1;
      slot[i] = -1;
      slot[next] = si;
      act2[m_n - 2] = next;
      nwg_join& J = s.joins[step];
      J.i = i;
      J.j = j;
      J.node = next;
      J.n = m_n;
      J.d = w.d;
      J.pad = 0.f;
      J.q = w.q1;
      J.ti = w.ta;
      J.tj = w.tb;
      record_pick(s, spick);
    }
    {
      int* t = act;
      act = act2;
      act2 = t;
    }
    // ---- the reference's rebuild schedule (SpeciesBlock.cpp:864, :1206-1247)
    if (--pq_ck == 0) {
      pq_ck = 500;
      if (steps > 0 && (double)(ub / kBinT) / (double)ave0 > 2.0 && tid == 0) s.stats[3] += 1;
    }
    const int m_after = m_n - 1;
    __syncthreads();
    if (steps == 0) {
      rowsums(m_after);
      if (tid == 0) s.stats[4] += 1;
      watermark = next + 1;
      steps = (m_after < 200) ? INT_MAX : (int)((float)m_after * 0.5f);
      ave0 = (((long long)(m_after - 1) * m_after) / 2) / kBinT;
      ub = ((long long)m_after * (m_after - 1)) / 2;
    } else {
      --steps;
      ub += m_after - 1;
    }
  }
  __syncthreads();
  for (int k = tid; k < n - 1; k += nth) join_lengths(s.joins[k]);
}

// ---- small jobs: the whole join loop in the cluster's shared memory --------
// Up to kSmemNJMax taxa the matrix fits the distributed shared memory of one
// cluster.  CTA q holds the rows of the folded slot pairs p = q, q + C, ...
// (rows p and n-1-p; local row 2*(p/C) + (row != p)); every CTA keeps its own
// copy of the float row sums, the slot -> node and id -> slot maps and the
// active list, updated identically, and reads the other CTAs' row minima,
// partials, row sums and rows through distributed shared memory.  The phases
// and the arithmetic are those of the global forms (pass with the two
// smallest q per row, direct pick or fallback scan, join share, apply, the
// reference's rebuild schedule); only the join records and a fallback
// candidate list use global memory.

constexpr int kSmemNJMax = 768;

struct SmemLayout {
  int ldl;   // local row stride (floats, a multiple of 4)
  int lr;    // local rows per CTA (two per local pair)
  size_t rows, tf, tloc, tsn, node, slot, act_a, act_b, grm, grc, tvl, bytes;   // grm: every slot
};

__host__ __device__ inline SmemLayout smem_layout(int n, int C) {
  auto al = [](size_t x) { return (x + 15) / 16 * 16; };
  SmemLayout L;
  L.ldl = (n + 3) & ~3;
  const int npairs = (n + 1) / 2;
  L.lr = 2 * ((npairs + C - 1) / C);
  size_t o = 0;
  L.rows = o; o += al(sizeof(float) * (size_t)L.lr * L.ldl);
  L.tf = o; o += al(sizeof(float) * L.ldl);
  L.tloc = o; o += al(sizeof(double) * L.lr);
  L.tsn = o; o += al(sizeof(double) * L.lr);
  L.node = o; o += al(sizeof(int) * n);
  L.slot = o; o += al(sizeof(int) * 2 * n);
  L.act_a = o; o += al(sizeof(int) * (n + 1));
  L.act_b = o; o += al(sizeof(int) * (n + 1));
  L.grm = o; o += al(sizeof(int) * n);
  L.grc = o; o += al(sizeof(int4) * L.lr);
  L.tvl = o; o += al(sizeof(float) * L.lr);
  L.bytes = o;
  return L;
}

template <int C>
struct SmemNJ {
  int n, npairs, ldl, lr, rank;
  float* rows;     // local rows, ldl floats each
  float* Tf;       // float row sums of every slot (NaN dead / padding)
  double* Tloc;    // T of the local rows
  double* Tsn;     // T of the local rows as the pass saw it (the pick reads these)
  int* node;       // slot -> node id
  int* slot;       // node id -> slot
  int* grm;        // every slot: smallest float q of its row (ordered int), pushed by the row's owner
  int4* grc;       // local rows: second smallest q (ordered int), column and distance of the smallest
  float* tvl;      // local rows: the new row's value in this join
  // slot -> owner CTA and local row
  __device__ __forceinline__ int owner(int r) const {
    const int p = min(r, n - 1 - r);
    return p % C;
  }
  __device__ __forceinline__ int local_row(int r) const {
    const int p = min(r, n - 1 - r);
    return 2 * (p / C) + (r != p ? 1 : 0);
  }
  // local row lr of CTA q -> slot, or -1
  __device__ __forceinline__ int slot_of(int q, int l) const {
    const int p = (l >> 1) * C + q;
    if (p >= npairs) return -1;
    if (l & 1) return n - 1 - p == p ? -1 : n - 1 - p;
    return p;
  }
  template <class T>
  __device__ __forceinline__ T* at(T* local, int q) const {
    return cooperative_groups::this_cluster().map_shared_rank(local, q);
  }
};

// Row sums of this CTA's live rows over the active list (the reference's
// ascending-id order; any-order lanes when provably exact), with the float
// copies written into every CTA's row-sum array.
template <int C>
__device__ void smem_rowsums(const SmemNJ<C>& m, const int* act, int na) {
  const int lane = threadIdx.x & 31;
  for (int l = (int)(threadIdx.x >> 5); l < m.lr; l += (int)(blockDim.x >> 5)) {
    const int r = m.slot_of(m.rank, l);
    if (r < 0 || m.node[r] < 0) continue;
    const float* row = m.rows + (size_t)l * m.ldl;
    double part = 0.0, ab = 0.0;
    int lowexp = INT_MAX;
    for (int j = lane; j < na; j += 32) {
      const float x = row[m.slot[act[j]]];
      part = __dadd_rn(part, (double)x);
      ab = __dadd_rn(ab, (double)fabsf(x));
      lowexp = min(lowexp, low_bit_exp(x));
    }
    for (int o = 16; o > 0; o >>= 1) {
      part = __dadd_rn(part, __shfl_down_sync(0xffffffffu, part, o));
      ab = __dadd_rn(ab, __shfl_down_sync(0xffffffffu, ab, o));
      lowexp = min(lowexp, __shfl_down_sync(0xffffffffu, lowexp, o));
    }
    double sum = __shfl_sync(0xffffffffu, part, 0);
    if (lane == 0 && !sum_is_exact(ab, lowexp)) {
      sum = 0.0;
      for (int j = 0; j < na; ++j) sum = __dadd_rn(sum, (double)row[m.slot[act[j]]]);
    }
    sum = __shfl_sync(0xffffffffu, sum, 0);
    if (lane == 0) m.Tloc[l] = sum;
    const float tf = __double2float_rn(sum);
    if (lane < C) m.at(m.Tf, lane)[r] = tf;
  }
}

template <int C>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(1024, 1) nj_smem_kernel(const NJJob* jobs, int njobs) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ NJJob sjob;
  __shared__ float sparts[2 * 16];   // every CTA's pass partial (pushed by each CTA)
  __shared__ USum susums[16];        // every CTA's share sum (pushed by each CTA)
  __shared__ int rows_sel[kFastRows];
  __shared__ GCand fc[kFastRows];
  __shared__ int nsel, s_ok;
  __shared__ PickOut spick;
  __shared__ GCand swin;
  __shared__ float sthr;
  __shared__ double s_sum;
  __shared__ int s_exact;
  namespace cg = cooperative_groups;
  const int crank = (int)cg::this_cluster().block_rank();
  const int job = (int)blockIdx.x / C;   // the same for every CTA of the cluster
  if (job >= njobs) return;
  if (threadIdx.x == 0) sjob = jobs[job];
  __syncthreads();
  const NJDev& s = sjob.s;
  const GridNJ& g = sjob.g;
  const int n = sjob.n;
  __shared__ SmemNJ<C> sm;   // the layout's pointers (shared memory keeps registers free)
  const SmemLayout L = smem_layout(n, C);
  if (threadIdx.x == 0) {
    sm.n = n;
    sm.npairs = (n + 1) / 2;
    sm.ldl = L.ldl;
    sm.lr = L.lr;
    sm.rank = crank;
    sm.rows = reinterpret_cast<float*>(smem + L.rows);
    sm.Tf = reinterpret_cast<float*>(smem + L.tf);
    sm.Tloc = reinterpret_cast<double*>(smem + L.tloc);
    sm.node = reinterpret_cast<int*>(smem + L.node);
    sm.slot = reinterpret_cast<int*>(smem + L.slot);
    sm.grm = reinterpret_cast<int*>(smem + L.grm);
    sm.grc = reinterpret_cast<int4*>(smem + L.grc);
    sm.Tsn = reinterpret_cast<double*>(smem + L.tsn);
    sm.tvl = reinterpret_cast<float*>(smem + L.tvl);
  }
  __syncthreads();
  const SmemNJ<C>& m = sm;
  int* act = reinterpret_cast<int*>(smem + L.act_a);
  int* act2 = reinterpret_cast<int*>(smem + L.act_b);
  const int rank = m.rank;
  const int tid = (int)threadIdx.x, nth = (int)blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  // this CTA's rows from the matrix (padding columns 0); maps and lists
  for (int l = 0; l < m.lr; ++l) {
    const int r = m.slot_of(rank, l);
    float* row = m.rows + (size_t)l * m.ldl;
    for (int c = tid; c < m.ldl; c += nth) row[c] = (r >= 0 && c < n) ? s.D[(size_t)r * s.ld + c] : 0.f;
  }
  for (int k = tid; k < m.ldl; k += nth) m.Tf[k] = __int_as_float(0x7FC00000);
  for (int k = tid; k < 2 * n; k += nth) m.slot[k] = k < n ? k : -1;
  for (int k = tid; k < n; k += nth) {
    m.node[k] = k;
    act[k] = k;
  }
  for (int k = tid; k < n; k += nth) m.grm[k] = 0x7F7FFFFF;
  if (rank == 0 && tid == 0) {
    s.g32[0] = s.g32[1] = s.g32[2] = 0;
    s.stats[0] = s.stats[1] = s.stats[2] = s.stats[3] = s.stats[4] = 0;
  }
  cg::this_cluster().sync();   // every CTA's row-sum array is NaN before any broadcast lands
  if (n >= 2) {
    __syncthreads();
    smem_rowsums(m, act, n);
  }
  cg::this_cluster().sync();
  const int kBinT = 30 * 31 / 2;
  int steps = max((int)((float)n * 0.5f), 200);
  int pq_ck = 500;
  long long ave0 = (((long long)(n - 1) * n) / 2) / kBinT;
  long long ub = ((long long)n * (n - 1)) / 2;
  int watermark = n;
  bool failed = false;
  for (int step = 0; step < n - 1 && !failed; ++step) {
    const int m_n = n - step, next = n + step;
    const float nm2f = (float)(m_n - 2);
    const double nm2 = (double)(m_n - 2);
    // ---- pass: each warp one local pair, 16-byte loads from shared memory
    {
      float qmin = FLT_MAX, mmax = 0.f;
      // the layout's fields in registers (shared-memory stores below would
      // otherwise make the compiler reload them)
      const float* const Tfp = m.Tf;
      const float* const rowsp = m.rows;
      const int ldl = m.ldl;
      int* const grmp = m.grm;
      int4* const grcp = m.grc;
      double* const tsnp = m.Tsn;
      const double* const tlocp = m.Tloc;
      const float4* Tf4 = reinterpret_cast<const float4*>(Tfp);
      const int nv = ldl >> 2;
      auto row_pass = [&](int l) {
        const int r = m.slot_of(rank, l);
        if (r < 0) return;
        const float tr = Tfp[r];
        if (tr != tr) {   // dead
          if (lane < C) m.at(grmp, lane)[r] = 0x7F7FFFFF;
          return;
        }
        const float* row = rowsp + (size_t)l * ldl;
        float m1 = FLT_MAX, m2 = FLT_MAX, mag = 0.f;
        int c1 = -1;
        const int c0 = r + 1, v0 = (c0 + 3) >> 2;
        if (lane < 4 * v0 - c0 && c0 + lane < n) pass_elem(row[c0 + lane], Tfp[c0 + lane], c0 + lane, tr, nm2f, m1, m2, c1, mag);
        const float4* row4 = reinterpret_cast<const float4*>(row);
        for (int v = v0 + lane; v < nv; v += 32) {
          const float4 d = row4[v];
          const float4 tc = Tf4[v];
          pass_elem(d.x, tc.x, 4 * v, tr, nm2f, m1, m2, c1, mag);
          pass_elem(d.y, tc.y, 4 * v + 1, tr, nm2f, m1, m2, c1, mag);
          pass_elem(d.z, tc.z, 4 * v + 2, tr, nm2f, m1, m2, c1, mag);
          pass_elem(d.w, tc.w, 4 * v + 3, tr, nm2f, m1, m2, c1, mag);
        }
        for (int o = 16; o > 0; o >>= 1) {
          const float om1 = __shfl_xor_sync(0xffffffffu, m1, o);
          const float om2 = __shfl_xor_sync(0xffffffffu, m2, o);
          const int oc1 = __shfl_xor_sync(0xffffffffu, c1, o);
          const bool take = om1 < m1 || (om1 == m1 && oc1 < c1);
          const float lo = take ? om1 : m1, hi = take ? m1 : om1;
          m2 = fminf(hi, fminf(m2, om2));
          m1 = lo;
          c1 = take ? oc1 : c1;
          mag = fmaxf(mag, __shfl_xor_sync(0xffffffffu, mag, o));
        }
        // the pick reads only what the pass wrote (a fast CTA's join share
        // may already be changing rows and row sums); the row minimum goes to
        // every CTA
        if (lane < C) m.at(grmp, lane)[r] = ford(m1);
        if (lane == 0) {
          grcp[l] = make_int4(ford(m2), c1, __float_as_int(c1 >= 0 ? row[c1] : 0.f), 0);
          tsnp[l] = tlocp[l];
        }
        qmin = fminf(qmin, m1);
        mmax = fmaxf(mmax, __fadd_rn(mag, fabsf(tr)));
      };
      // a row pair per warp, the two rows' warp reductions in the same
      // shuffle rounds
      auto pair_pass = [&](int lp) {
        float m1[2], m2[2], mag[2], trs[2];
        int c1[2], rs[2];
        bool live[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int l = 2 * lp + h;
          rs[h] = m.slot_of(rank, l);
          trs[h] = rs[h] >= 0 ? Tfp[rs[h]] : 0.f;
          live[h] = rs[h] >= 0 && trs[h] == trs[h];
          if (rs[h] >= 0 && !live[h] && lane < C) m.at(grmp, lane)[rs[h]] = 0x7F7FFFFF;   // dead
          m1[h] = m2[h] = FLT_MAX;
          mag[h] = 0.f;
          c1[h] = -1;
          if (!live[h]) continue;
          const int r = rs[h];
          const float tr = trs[h];
          const float* row = rowsp + (size_t)l * ldl;
          const int c0 = r + 1, v0 = (c0 + 3) >> 2;
          if (lane < 4 * v0 - c0 && c0 + lane < n)
            pass_elem(row[c0 + lane], Tfp[c0 + lane], c0 + lane, tr, nm2f, m1[h], m2[h], c1[h], mag[h]);
          const float4* row4 = reinterpret_cast<const float4*>(row);
          for (int v = v0 + lane; v < nv; v += 32) {
            const float4 d = row4[v];
            const float4 tc = Tf4[v];
            pass_elem(d.x, tc.x, 4 * v, tr, nm2f, m1[h], m2[h], c1[h], mag[h]);
            pass_elem(d.y, tc.y, 4 * v + 1, tr, nm2f, m1[h], m2[h], c1[h], mag[h]);
            pass_elem(d.z, tc.z, 4 * v + 2, tr, nm2f, m1[h], m2[h], c1[h], mag[h]);
            pass_elem(d.w, tc.w, 4 * v + 3, tr, nm2f, m1[h], m2[h], c1[h], mag[h]);
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float om1 = __shfl_xor_sync(0xffffffffu, m1[h], o);
            const float om2 = __shfl_xor_sync(0xffffffffu, m2[h], o);
            const int oc1 = __shfl_xor_sync(0xffffffffu, c1[h], o);
            const bool take = om1 < m1[h] || (om1 == m1[h] && oc1 < c1[h]);
            const float lo = take ? om1 : m1[h], hi = take ? m1[h] : om1;
            m2[h] = fminf(hi, fminf(m2[h], om2));
            m1[h] = lo;
            c1[h] = take ? oc1 : c1[h];
            mag[h] = fmaxf(mag[h], __shfl_xor_sync(0xffffffffu, mag[h], o));
          }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!live[h]) continue;
          const int l = 2 * lp + h, r = rs[h];
          if (lane < C) m.at(grmp, lane)[r] = ford(m1[h]);
          if (lane == 0) {
            const float* row = rowsp + (size_t)l * ldl;
            grcp[l] = make_int4(ford(m2[h]), c1[h], __float_as_int(c1[h] >= 0 ? row[c1[h]] : 0.f), 0);
            tsnp[l] = tlocp[l];
          }
          qmin = fminf(qmin, m1[h]);
          mmax = fmaxf(mmax, __fadd_rn(mag[h], fabsf(trs[h])));
        }
      };
      // one row per warp when the CTA's rows fit its warps, else one row pair
      // per warp
      const int nw = nth >> 5;
      if (m.lr <= nw) {
        if (warp < m.lr) row_pass(warp);
      } else {
        for (int lp = warp; 2 * lp < m.lr; lp += nw) pair_pass(lp);
      }
      __shared__ float wq[32], wm[32];
      if (lane == 0) {
        wq[warp] = qmin;
        wm[warp] = mmax;
      }
      __syncthreads();
      if (warp == 0) {
        qmin = lane < (nth >> 5) ? wq[lane] : FLT_MAX;
        mmax = lane < (nth >> 5) ? wm[lane] : 0.f;
        for (int o = 16; o > 0; o >>= 1) {
          qmin = fminf(qmin, __shfl_xor_sync(0xffffffffu, qmin, o));
          mmax = fmaxf(mmax, __shfl_xor_sync(0xffffffffu, mmax, o));
        }
        if (lane < C) {
          float* dst = m.at(sparts, lane);
          dst[2 * rank] = qmin;
          dst[2 * rank + 1] = mmax;
        }
      }
    }
    cg::this_cluster().sync();
    // ---- pick: threshold from the CTA partials, rows within it, candidates
    if (warp == 0) {
      float q = lane < C ? sparts[2 * lane] : FLT_MAX, mm = lane < C ? sparts[2 * lane + 1] : 0.f;
      for (int o = 16; o > 0; o >>= 1) {
        q = fminf(q, __shfl_xor_sync(0xffffffffu, q, o));
        mm = fmaxf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
      }
      if (lane == 0) {
        sthr = q + 3.f * (8.f * 5.9604645e-8f * mm) + 1e-30f;
        nsel = 0;
      }
    }
    __syncthreads();
    const float thr = sthr;
    const int othr = ford(thr);
    for (int r = tid; r < n; r += nth) {
      if (m.grm[r] <= othr) {
        const int k = atomicAdd(&nsel, 1);
        if (k < kFastRows) rows_sel[k] = r;
      }
    }
    __syncthreads();
    const int nr = nsel;
    if (warp == 0) {
      int ok = nr >= 1 && nr <= kFastRows;
      if (ok && lane < nr) {
        const int r = rows_sel[lane];
        const int q = m.owner(r), l = m.local_row(r);
        const int4 rec = m.at(m.grc, q)[l];
        const int c = rec.y;
        if (rec.x <= othr || c < 0) {
          ok = 0;   // a second pair of the row within the threshold
        } else {
          const int qc = m.owner(c), lc = m.local_row(c);
          const double Tr = m.at(m.Tsn, q)[l], Tc = m.at(m.Tsn, qc)[lc];
          const float d = __int_as_float(rec.z);
          const int ur = m.node[r], uc = m.node[c];
          fc[lane] = make_cand(r, c, ur, uc, Tr, Tc, d, nm2, watermark);
          if (ur < 0 || uc < 0) ok = 0;
        }
      }
      ok = __all_sync(0xffffffffu, ok);
      PickOut pr{};
      if (ok && nr == 1) {
        pr.idx = 0;
        pr.ties = 1;
        pr.amb = 0;
        pr.error = false;
      } else if (ok) {
        pr = pick_keys(nr, [&](int k) { return fc[k]; });
      }
      if (lane == 0) {
        s_ok = ok;
        if (ok) {
          spick = pr;
          swin = fc[pr.idx];
        }
      }
    }
    __syncthreads();
    if (!s_ok) {
      // fallback: each CTA scans its own rows within the threshold into the
      // list (as grid_cand does; beyond the list's capacity the winner comes
      // from the CTAs' first candidates and a second scan counts against it)
      // (one warp per local row, lanes over the columns; visit(pred, candidate)
      // by whole warps as in grid_cand_scan)
      auto scan = [&](auto&& visit) {
        for (int l = warp; l < m.lr; l += nth >> 5) {
          const int r = m.slot_of(rank, l);
          if (r < 0 || m.grm[r] > othr) continue;
          const int ur = m.node[r];
          const float tr = m.Tf[r];
          const double Tr = m.Tloc[l];
          const float* row = m.rows + (size_t)l * m.ldl;
          for (int cb = r + 1; cb < n; cb += 32) {
            const int c = cb + lane;
            bool pred = false;
            KCand kc = kc_none();
            if (c < n) {
              const int uc = m.node[c];
              const float d = row[c];
              const float q = __fsub_rn(__fsub_rn(__fmul_rn(d, nm2f), tr), m.Tf[c]);
              if (uc >= 0 && q <= thr) {
                const double Tc = m.at(m.Tloc, m.owner(c))[m.local_row(c)];
                const GCand cd = make_cand(r, c, ur, uc, Tr, Tc, d, nm2, watermark);
                kc = KCand{cd.k1, cd.k2, cd.a, cd.b};
                pred = true;
              }
            }
            visit(pred, kc);
          }
        }
      };
      // the winner's pair again, as the scan read it (row = the smaller slot)
      auto rederive = [&](const KCand& w) {
        const int sa = m.slot[w.a], sb = m.slot[w.b];
        const int r0 = min(sa, sb), c0 = max(sa, sb);
        const int q = m.owner(r0), l = m.local_row(r0);
        const double Tr = m.at(m.Tloc, q)[l], Tc = m.at(m.Tloc, m.owner(c0))[m.local_row(c0)];
        const float d = m.at(m.rows, q)[(size_t)l * m.ldl + c0];
        swin = make_cand(r0, c0, m.node[r0], m.node[c0], Tr, Tc, d, nm2, watermark);
      };
      __shared__ KCand skw[32];
      __shared__ KCand sfirst;
      KCand first = kc_none();
      bool full = false;
      scan([&](bool pred, const KCand& c) {
        list_push(s, g, pred, c, full);
        if (pred && kc_first(c, first)) first = c;
      });
      cg::this_cluster().sync();
      const int ncount = *(volatile int*)&s.g32[2];   // the same in every CTA
      if (ncount <= min(s.cand_cap, kListPickMax)) {
        if (warp == 0) {
          const PickOut pr = pick_keys(ncount, [&](int k) { return g.cand[k]; });
          if (lane == 0) {
            spick = pr;
            if (!pr.error) rederive(g.cand[pr.idx]);
          }
        }
        __syncthreads();
      } else {
        first = cta_first(first, skw);
        if (tid == 0) g.cbest[rank] = first;
        cg::this_cluster().sync();
        if (warp == 0) {
          const PickOut pr = pick_keys(C, [&](int k) { return ld_kcand(&g.cbest[k]); });
          if (lane == 0) sfirst = pr.error ? kc_none() : ld_kcand(&g.cbest[pr.idx]);
        }
        __syncthreads();
        const KCand w = sfirst;
        unsigned ties = 0, amb = 0;
        scan([&](bool pred, const KCand& c) {
          if (pred) count_vs(c, w, ties, amb);
        });
        add_counts(ties, amb, s.g32);
        cg::this_cluster().sync();
        if (tid == 0) {
          spick.idx = 0;
          spick.ties = (unsigned)__ldcg(&s.g32[0]);
          spick.amb = (unsigned)__ldcg(&s.g32[1]);
          spick.error = w.b < 0;
          if (!spick.error) rederive(w);
        }
        __syncthreads();
      }
      if (spick.error) {   // the same in every CTA
        if (rank == 0 && tid == 0) record_pick(s, spick);
        failed = true;
        break;
      }
    }
    // ---- join share: this CTA's rows
    const GCand w = swin;
    const int i = w.a, j = w.b, si = w.sa, sj = w.sb;
    {
      USum x;
      x.u = x.a = 0;
      x.e = INT_MAX;
      x.t = INT_MIN;
      if (tid < m.lr) {
        const int l = tid;
        const int r = m.slot_of(rank, l);
        if (r >= 0 && m.node[r] >= 0 && r != si && r != sj) {
          float* row = m.rows + (size_t)l * m.ldl;
          const float Dik = row[si], Djk = row[sj];
          const float sumf = __fadd_rn(Dik, Djk);
          const float tmp = __fmul_rn(__fsub_rn(sumf, w.d), 0.5f);
          const double t = __dadd_rn(m.Tloc[l], (double)__fsub_rn(tmp, sumf));
          m.Tloc[l] = t;
          const float tf = __double2float_rn(t);
          row[si] = tmp;
          m.at(m.rows, m.owner(si))[(size_t)m.local_row(si) * m.ldl + r] = tmp;   // the new row
#pragma unroll
          for (int q = 0; q < C; ++q) m.at(m.Tf, q)[r] = tf;
          m.tvl[l] = tmp;
          if (tmp != 0.f) {
            x.e = low_bit_exp(tmp);
            x.t = top_bit_exp(tmp);
            x.u = float_units(tmp, x.e);
            x.a = x.u < 0 ? -x.u : x.u;
          }
        }
      }
      const int nwv = (m.lr + 31) >> 5;
      if (warp < nwv) usum_warp(x);
      __shared__ USum swp[32];
      if (lane == 0 && warp < nwv) swp[warp] = x;
      __syncthreads();   // also: every read of this join's maps is done
      if (tid == 0) {
        for (int w2 = 1; w2 < nwv; ++w2) usum_add(x, swp[w2]);
        for (int q = 0; q < C; ++q) m.at(susums, q)[rank] = x;   // to every CTA
      }
      // the maps and the active list, identically in every CTA
      for (int k = tid; k < m_n; k += nth) {
        const int v = act[k];
        if (v != i && v != j) act2[k - (v > i) - (v > j)] = v;
      }
      if (tid == 0) {
        act2[m_n - 2] = next;
        m.node[sj] = -1;
        m.node[si] = next;
        m.slot[j] = -1;
        m.slot[i] = -1;
        m.slot[next] = si;
        m.Tf[sj] = __int_as_float(0x7FC00000);
      }
    }
    cg::this_cluster().sync();
    // ---- apply: the new node's row sum from the CTA sums
    if (warp == 0) {
      USum x;
      x.u = x.a = 0;
      x.e = INT_MAX;
      x.t = INT_MIN;
      if (lane < C) x = susums[lane];
      usum_warp(x);
      if (lane == 0) {
        if (x.e == INT_MAX) {
          s_sum = 0.0;
          s_exact = 1;
        } else if (x.t - x.e < 48 && x.a < (1ll << 53)) {
          s_sum = units_to_double(x.u, x.e);
          s_exact = 1;
        } else {
          s_exact = 0;
        }
      }
    }
    __syncthreads();
    if (s_exact) {
      if (tid == 0) {
        m.Tf[si] = __double2float_rn(s_sum);
        if (m.owner(si) == rank) m.Tloc[m.local_row(si)] = s_sum;
      }
    } else {
      if (rank == 0 && tid == 0) {
        double sum = 0.0;   // the reference's loop: active ids ascending, i and j skipped
        for (int k = 0; k < m_n; ++k) {
          const int v = act[k];
          if (v == i || v == j) continue;
          const int sv = v == next ? si : m.slot[v];
          sum = __dadd_rn(sum, (double)m.at(m.tvl, m.owner(sv))[m.local_row(sv)]);
        }
        const float tf = __double2float_rn(sum);
        for (int q = 0; q < C; ++q) m.at(m.Tf, q)[si] = tf;
        m.at(m.Tloc, m.owner(si))[m.local_row(si)] = sum;
      }
      cg::this_cluster().sync();
    }
    if (rank == 0 && tid == 0) {
      nwg_join& J = s.joins[step];
      J.i = i;
      J.j = j;
      J.node = next;
      J.n = m_n;
      J.d = w.d;
      J.pad = 0.f;
      J.q = w.q1;
      J.ti = w.ta;
      J.tj = w.tb;
      s.g32[0] = s.g32[1] = s.g32[2] = 0;
      record_pick(s, spick);
    }
    {
      int* t = act;
      act = act2;
      act2 = t;
    }
    // ---- the reference's rebuild schedule (SpeciesBlock.cpp:864, :1206-1247)
    if (--pq_ck == 0) {
      pq_ck = 500;
      if (steps > 0 && (double)(ub / kBinT) / (double)ave0 > 2.0 && rank == 0 && tid == 0) s.stats[3] += 1;
    }
    const int m_after = m_n - 1;
    if (steps == 0) {
      cg::this_cluster().sync();   // every CTA's own write of the new row sum lands before the broadcasts
      smem_rowsums(m, act, m_after);
      if (rank == 0 && tid == 0) s.stats[4] += 1;
      watermark = next + 1;
      steps = (m_after < 200) ? INT_MAX : (int)((float)m_after * 0.5f);
      ave0 = (((long long)(m_after - 1) * m_after) / 2) / kBinT;
      ub = ((long long)m_after * (m_after - 1)) / 2;
      cg::this_cluster().sync();
    } else {
      --steps;
      ub += m_after - 1;
      __syncthreads();
    }
  }
  cg::this_cluster().sync();   // every join record is written; no CTA reads another's shared memory after this
  if (!failed)
    for (int k = rank * nth + tid; k < n - 1; k += C * nth) join_lengths(s.joins[k]);
}

}  // namespace

struct NJState {
  DevBuf D, jobws, desc;
  // large-n path: row sums, maps, compaction buffers, candidates, grid partials and barrier words
  DevBuf T, Tf, slot, node, act, na, g32, stats, joins, cand, cbest, tv, grmin, grec, tsnap;
  DevBuf D2, T2, Tf2, node2, map, act2, part, jsum, jexp, gbar;
  ~NJState() {
    for (DevBuf* b : {&D, &jobws, &desc, &T, &Tf, &slot, &node, &act, &na, &g32, &stats, &joins, &cand, &cbest, &tv, &grmin,
                      &grec, &tsnap, &D2, &T2, &Tf2, &node2, &map, &act2, &part, &jsum, &jexp, &gbar})
      b->release();
  }
};

// Up to this many taxa one cluster runs the whole join loop (the matrix stays
// in L2); larger matrices take the whole GPU per join.  The environment
// variable NWG_NJ_CLUSTER_MAX_N overrides the threshold (both forms give the
// same joins; the tests run each form on the same inputs).
int cluster_nj_max_n() {
  static const int v = [] {
    const char* e = std::getenv("NWG_NJ_CLUSTER_MAX_N");
    return e ? std::atoi(e) : 2048;
  }();
  return v;
}

void Ctx::nj_release() {
  delete reinterpret_cast<NJState*>(nj_state);
  nj_state = nullptr;
}

int Ctx::nj(const float* D, int64_t ld, int n, bool device_D, nwg_join* joins, nwg_nj_stats* st) {
  if (n < 1 || !D || ld < n || (!joins && n > 1)) return fail(NWG_ERR_INVALID, "nj arguments");
  if (n > kNJMaxN) return fail(NWG_ERR_INVALID, "neighbor joining on the device supports n <= 8192");
  nwg_nj_stats stats;
  std::memset(&stats, 0, sizeof(stats));
  if (n == 1) {
    stats.reference_identical = 1;
    if (st) *st = stats;
    return NWG_OK;
  }
  if (!nj_state) nj_state = new NJState();
  NJState& S = *reinterpret_cast<NJState*>(nj_state);
  const int nn = 2 * n - 1;
  const bool big = n > cluster_nj_max_n();
  const int ldd = nj_row_stride(n);   // rows padded to a multiple of 4 floats (16-byte loads)
  int rc;
  if ((rc = S.D.ensure(sizeof(float) * (size_t)n * ldd))) return fail(rc, "nj allocation");
  cudaStream_t s = stream;
  const cudaMemcpyKind kind = device_D ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if ((rc = cuda(cudaMemcpy2DAsync(S.D.p, sizeof(float) * ldd, D, sizeof(float) * ld, sizeof(float) * n, n, kind, s),
                 "nj upload")))
    return rc;
  const void* jsrc;   // join records and statistics on the device
  const void* ssrc;
  if (!big) {
    if ((rc = S.jobws.ensure(nj_job_workspace(n))) || (rc = S.desc.ensure(sizeof(NJJob))))
      return fail(rc, "nj allocation");
    NJJob J{};
    nwg_join* jp;
    unsigned long long* sp;
    nj_job_setup(&J, (float*)S.D.p, n, ldd, (char*)S.jobws.p, &jp, &sp);
    jsrc = jp;
    ssrc = sp;
    // the descriptor travels in the stream (a pageable copy is staged at once)
    if ((rc = cuda(cudaMemcpyAsync(S.desc.p, &J, sizeof(J), cudaMemcpyHostToDevice, s), "nj upload"))) return rc;
    if (st) cudaEventRecord(ev0, s);
    const int csm = smem_nj_cluster(n);
    if ((rc = cuda(n <= cta_nj_max_n() ? launch_nj_cta(S.desc.p, 1, n, s)
                   : csm               ? launch_nj_smem(S.desc.p, 1, n, csm, s)
                                       : launch_nj_cluster(S.desc.p, 1, nj_cluster_size(), s),
                   "nj launch")))
      return rc;
    ++launches;
  } else {
    // one CTA of 1024 threads per SM (cooperative launch); every join share
    // then holds at most one slot per thread
    const int grid = std::min(sms, kGridMax);
    if ((rc = S.T.ensure(sizeof(double) * n)) || (rc = S.Tf.ensure(sizeof(float) * ldd)) ||
        (rc = S.slot.ensure(sizeof(int) * nn)) || (rc = S.node.ensure(sizeof(int) * n)) ||
        (rc = S.act.ensure(sizeof(int) * (n + 1))) || (rc = S.na.ensure(sizeof(int))) ||
        (rc = S.g32.ensure(sizeof(int) * 4)) || (rc = S.stats.ensure(sizeof(unsigned long long) * 5)) ||
        (rc = S.joins.ensure(sizeof(nwg_join) * (n - 1))) || (rc = S.cand.ensure(sizeof(KCand) * kCandCap)) ||
        (rc = S.cbest.ensure(sizeof(KCand) * grid)) ||
        (rc = S.tv.ensure(sizeof(float) * n)) || (rc = S.grmin.ensure(sizeof(int) * n)) ||
        (rc = S.grec.ensure(sizeof(int4) * n)) || (rc = S.tsnap.ensure(sizeof(double) * n)) || (rc = S.D2.ensure(sizeof(float) * (size_t)n * ldd)) ||
        (rc = S.T2.ensure(sizeof(double) * n)) || (rc = S.Tf2.ensure(sizeof(float) * ldd)) ||
        (rc = S.node2.ensure(sizeof(int) * n)) || (rc = S.map.ensure(sizeof(int) * n)) ||
        (rc = S.act2.ensure(sizeof(int) * (n + 1))) || (rc = S.part.ensure(sizeof(float) * 2 * grid)) ||
        (rc = S.jsum.ensure(sizeof(long long) * 2 * grid)) || (rc = S.jexp.ensure(sizeof(int) * 2 * grid)) ||
        (rc = S.gbar.ensure(sizeof(int) * 4)))
      return fail(rc, "nj allocation");
    NJDev d{};
    d.D = (float*)S.D.p;
    d.T = (double*)S.T.p;
    d.Tf = (float*)S.Tf.p;
    d.slot = (int*)S.slot.p;
    d.node = (int*)S.node.p;
    d.act = (int*)S.act.p;
    d.na = (int*)S.na.p;
    d.g32 = (int*)S.g32.p;
    d.stats = (unsigned long long*)S.stats.p;
    d.joins = (nwg_join*)S.joins.p;
    d.n0 = n;
    d.ld = ldd;
    d.cand_cap = kCandCap;
    jsrc = S.joins.p;
    ssrc = S.stats.p;
    std::vector<int> slot0(nn, -1), act0(n + 1, 0);
    for (int k = 0; k < n; ++k) slot0[k] = k, act0[k] = k;
    const int na0 = n;
    const int g0[4] = {0, 0, 0, 0};
    if ((rc = cuda(cudaMemcpyAsync(S.slot.p, slot0.data(), sizeof(int) * nn, cudaMemcpyHostToDevice, s), "nj upload")) ||
        (rc = cuda(cudaMemcpyAsync(S.node.p, act0.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s), "nj upload")) ||
        (rc = cuda(cudaMemcpyAsync(S.act.p, act0.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s), "nj upload")) ||
        (rc = cuda(cudaMemcpyAsync(S.na.p, &na0, sizeof(int), cudaMemcpyHostToDevice, s), "nj upload")) ||
        (rc = cuda(cudaMemcpyAsync(S.g32.p, g0, sizeof(g0), cudaMemcpyHostToDevice, s), "nj upload")) ||
        (rc = cuda(cudaMemsetAsync(S.stats.p, 0, sizeof(unsigned long long) * 5, s), "nj upload")) ||
        (rc = cuda(cudaStreamSynchronize(s), "nj upload")))   // the host vectors above are local
      return rc;
    int blocks_per_sm = 0;
    if ((rc = cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, nj_grid_kernel, 1024, 0),
                   "nj occupancy")))
      return rc;
    if (blocks_per_sm < 1 || grid * 1024 < n) return fail(NWG_ERR_CUDA, "neighbor-joining grid kernel does not fit");
    float* Dalt = (float*)S.D2.p;
    double* Talt = (double*)S.T2.p;
    float* Tfalt = (float*)S.Tf2.p;
    int* nodealt = (int*)S.node2.p;
    GridNJ g{};
    g.bar = (unsigned*)S.gbar.p;
    g.abort = (int*)S.gbar.p + 2;
    g.act2 = (int*)S.act2.p;
    g.grmin = (int*)S.grmin.p;
    g.grec = (int4*)S.grec.p;
    g.tsnap = (double*)S.tsnap.p;
    g.cbest = (KCand*)S.cbest.p;
    g.tv = (float*)S.tv.p;
    g.part = (float*)S.part.p;
    g.jsum = (long long*)S.jsum.p;
    g.jexp = (int*)S.jexp.p;
    g.cand = (KCand*)S.cand.p;
    // NaN (all bits set) float row sums at the padding slots; rowsum_kernel
    // fills the live ones
    if ((rc = cuda(cudaMemsetAsync(S.gbar.p, 0, sizeof(int) * 4, s), "nj upload")) ||
        (rc = cuda(cudaMemsetAsync(S.Tf.p, 0xFF, sizeof(float) * ldd, s), "nj upload")))
      return rc;
    if (st) cudaEventRecord(ev0, s);
    rowsum_kernel<<<(n + 7) / 8, 256, 0, s>>>(d, g.abort);
    ++launches;
    // The reference's schedule (deterministic in n): rebuild after
    // max(n*0.5, 200) joins, then every m*0.5 joins, none below 200 active
    // nodes; the joins between two rebuilds are one cooperative launch.
    const int kBinT = 30 * 31 / 2;
    int steps = std::max((int)((float)n * 0.5f), 200);
    int pq_ck = 500;
    long long ave0 = (((long long)(n - 1) * n) / 2) / kBinT;
    long long ub = ((long long)n * (n - 1)) / 2;
    int watermark = n, m_n = n;
    // compaction to the live slots, in slot order (every slot comparison of
    // the record-order rounding is unchanged, so it may run at any step)
    auto compact = [&](int na) -> int {
      const int ld2 = (na + 3) & ~3;
      int e;
      if ((e = cuda(cudaMemsetAsync(Tfalt, 0xFF, sizeof(float) * ld2, s), "nj launch"))) return e;
      compact_map_kernel<<<1, 1024, 0, s>>>(d, (int*)S.map.p, Talt, Tfalt, nodealt, nn, g.abort);
      compact_copy_kernel<<<d.n0, 256, 0, s>>>(d, (const int*)S.map.p, Dalt, ld2, g.abort);
      launches += 2;
      std::swap(d.D, Dalt);
      std::swap(d.T, Talt);
      std::swap(d.Tf, Tfalt);
      std::swap(d.node, nodealt);
      d.n0 = na;
      d.ld = ld2;
      return NWG_OK;
    };
    // Between rebuilds, large matrices are also compacted once a sixteenth of
    // their slots are dead: the pass streams every column of a live row.
    constexpr int kCompactMinSlots = 2048, kCompactFrac = 16;
    int step = 0;
    while (step < n - 1) {
      // the segment ends with the join after which the countdown reaches 0,
      // or at the next compaction
      int seg_end = steps == INT_MAX ? n - 1 : std::min(n - 1, step + steps + 1);
      const bool comp = d.n0 >= kCompactMinSlots && step + d.n0 / kCompactFrac < seg_end;
      if (comp) seg_end = step + d.n0 / kCompactFrac;
      if ((rc = cuda(cudaMemsetAsync(S.gbar.p, 0, sizeof(unsigned) * 2, s), "nj launch"))) return rc;
      // failure injection for the tests (NWG_NJ_INJECT_BARRIER_STALL=1): the
      // arrival count of the first segment starts one short, so its first
      // barrier never completes and every CTA gives up after the spin limit
      if (step == 0 && std::getenv("NWG_NJ_INJECT_BARRIER_STALL") &&
          std::atoi(std::getenv("NWG_NJ_INJECT_BARRIER_STALL")) == 1 &&
          (rc = cuda(cudaMemsetAsync(S.gbar.p, 0xFF, sizeof(unsigned), s), "nj launch")))
        return rc;
      {
        int a0 = step, a1 = seg_end, an = n, aw = watermark;
        void* args[] = {&d, &g, &a0, &a1, &an, &aw};
        if ((rc = cuda(cudaLaunchCooperativeKernel((const void*)nj_grid_kernel, dim3(grid), dim3(1024), args, 0, s),
                       "nj launch")))
          return rc;
        ++launches;
      }
      if ((seg_end - step) & 1) std::swap(d.act, g.act2);   // each join writes the other list
      bool rebuild = false;
      for (; step < seg_end; ++step) {
        if (--pq_ck == 0) {
          pq_ck = 500;
          if (steps > 0) {
            const double r = (double)(ub / kBinT) / (double)ave0;
            if (r > 2.0) ++stats.pq_trigger_open;
          }
        }
        --m_n;
        if (steps == 0) {
          rebuild = true;
        } else {
          if (steps != INT_MAX) --steps;
          ub += m_n - 1;
        }
      }
      if (rebuild) {
        rowsum_kernel<<<(m_n + 7) / 8, 256, 0, s>>>(d, g.abort);
        ++launches;
        if ((rc = compact(m_n))) return rc;
        ++stats.rebuilds;
        watermark = n + step;
        steps = (m_n < 200) ? INT_MAX : (int)((float)m_n * 0.5f);
        ave0 = (((long long)(m_n - 1) * m_n) / 2) / kBinT;
        ub = ((long long)m_n * (m_n - 1)) / 2;
      } else if (comp) {
        if ((rc = compact(m_n))) return rc;
      }
      if ((rc = cuda(cudaGetLastError(), "nj launch"))) return rc;
    }
    nj_lengths_kernel<<<(n - 1 + 255) / 256, 256, 0, s>>>(d.joins, n - 1);
    ++launches;
    if ((rc = cuda(cudaGetLastError(), "nj launch"))) return rc;
  }
  if (st) cudaEventRecord(ev1, s);
  unsigned long long dst[5] = {0, 0, 0, 0, 0};
  if ((rc = cuda(cudaMemcpyAsync(joins, jsrc, sizeof(nwg_join) * (n - 1), cudaMemcpyDeviceToHost, s), "nj download")) ||
      (rc = cuda(cudaMemcpyAsync(dst, ssrc, sizeof(dst), cudaMemcpyDeviceToHost, s), "nj download")) ||
      (rc = cuda(cudaStreamSynchronize(s), "nj sync")))
    return rc;
  if (dst[2]) return fail(NWG_ERR_CUDA, "neighbor joining candidate list empty or overflowing");
  if (big) {
    int gb[4];
    if ((rc = cuda(cudaMemcpy(gb, S.gbar.p, sizeof(gb), cudaMemcpyDeviceToHost), "nj download"))) return rc;
    if (gb[2]) return fail(NWG_ERR_CUDA, "neighbor-joining grid barrier timed out");
  }
  stats.ambiguous_steps = (int64_t)dst[0];
  stats.tie_steps = (int64_t)dst[1];
  if (!big) {
    stats.pq_trigger_open = (int64_t)dst[3];
    stats.rebuilds = (int64_t)dst[4];
  }
  stats.reference_identical = stats.ambiguous_steps == 0 && stats.pq_trigger_open == 0;
  if (st) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    stats.device_ms = ms;
    *st = stats;
  }
  return NWG_OK;
}

// Workspace of one job of the cluster forms, laid out from `base` (256-byte
// aligned pieces); fills *J when given.  The job's matrix is separate (n rows
// of ld floats, ld a multiple of 4; the form over L2 modifies it in place,
// the shared-memory form only reads it).
static size_t job_layout(int n, int ld, char* base, NJJob* J) {
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t cap = std::min<size_t>(kCandCap, (size_t)n * (n - 1) / 2 + 1);
  constexpr int kC = 16;   // partials for the largest cluster
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* q = base ? base + off : nullptr;
    off += al(bytes);
    return q;
  };
  char* T = take(sizeof(double) * n);
  char* Tf = take(sizeof(float) * ld);
  char* slot = take(sizeof(int) * (2 * n));
  char* node = take(sizeof(int) * n);
  char* act = take(sizeof(int) * (n + 1));
  char* act2 = take(sizeof(int) * (n + 1));
  char* na = take(sizeof(int) * 4);
  char* g32 = take(sizeof(int) * 4);
  char* stats = take(sizeof(unsigned long long) * 5);
  char* grmin = take(sizeof(int) * n);
  char* grec = take(sizeof(int4) * n);
  char* tsnap = take(sizeof(double) * n);
  char* tv = take(sizeof(float) * n);
  char* part = take(sizeof(float) * 2 * kC);
  char* jsum = take(sizeof(long long) * 2 * kC);
  char* jexp = take(sizeof(int) * 2 * kC);
  char* cand = take(sizeof(KCand) * cap);
  char* cbest = take(sizeof(KCand) * kC);
  char* joins = take(sizeof(nwg_join) * (n > 1 ? n - 1 : 1));
  if (J) {
    J->s.T = (double*)T;
    J->s.Tf = (float*)Tf;
    J->s.slot = (int*)slot;
    J->s.node = (int*)node;
    J->s.act = (int*)act;
    J->s.na = (int*)na;
    J->s.g32 = (int*)g32;
    J->s.stats = (unsigned long long*)stats;
    J->s.joins = (nwg_join*)joins;
    J->s.n0 = n;
    J->s.ld = ld;
    J->s.cand_cap = (int)cap;
    J->g.act2 = (int*)act2;
    J->g.grmin = (int*)grmin;
    J->g.grec = (int4*)grec;
    J->g.tsnap = (double*)tsnap;
    J->g.tv = (float*)tv;
    J->g.part = (float*)part;
    J->g.jsum = (long long*)jsum;
    J->g.jexp = (int*)jexp;
    J->g.cand = (KCand*)cand;
    J->g.cbest = (KCand*)cbest;
    J->n = n;
  }
  return off;
}

size_t nj_job_workspace(int n) { return job_layout(n, nj_row_stride(n), nullptr, nullptr); }

// Fill the job descriptor for a job of n nodes with matrix D (row stride ld)
// and workspace at base; returns the addresses of its join records and
// statistics.
void nj_job_setup(void* job_out, float* D, int n, int ld, char* base, nwg_join** joins, unsigned long long** stats) {
  NJJob J{};
  job_layout(n, ld, base, &J);
  J.s.D = D;
  *joins = J.s.joins;
  *stats = J.s.stats;
  std::memcpy(job_out, &J, sizeof(J));
}

size_t nj_job_desc_bytes() { return sizeof(NJJob); }

// One job per cluster of C CTAs (C = 8 or 16).
cudaError_t launch_nj_cluster(const void* d_jobs, int njobs, int C, cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const NJJob* jobs = reinterpret_cast<const NJJob*>(d_jobs);
  if (C == 16) {
    cudaError_t e = cudaFuncSetAttribute(nj_cluster_kernel<16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    nj_cluster_kernel<16><<<njobs * 16, 1024, 0, s>>>(jobs, njobs);
  } else {
    nj_cluster_kernel<8><<<njobs * 8, 1024, 0, s>>>(jobs, njobs);
  }
  return cudaGetLastError();
}

// Jobs of at most this many taxa run the join loop in one CTA
// (nj_cta_kernel); NWG_NJ_CTA_MAX_N overrides it (0: never).
int cta_nj_max_n() {
  static const int v = [] {
    const char* e = std::getenv("NWG_NJ_CTA_MAX_N");
    return e ? std::min(std::atoi(e), kCtaNJMax) : kCtaNJMax;
  }();
  return v;
}

cudaError_t launch_nj_cta(const void* d_jobs, int njobs, int nmax, cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const int bytes = (int)cta_layout(std::max(nmax, 2)).bytes;
  cudaError_t e = cudaFuncSetAttribute(nj_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  nj_cta_kernel<<<njobs, kCtaThreads, bytes, s>>>(reinterpret_cast<const NJJob*>(d_jobs), njobs);
  return cudaGetLastError();
}

// Jobs of at most this many taxa run the join loop in the cluster's shared
// memory (nj_smem_kernel); NWG_NJ_SMEM_MAX_N overrides it (0: never).
int smem_nj_max_n() {
  static const int v = [] {
    const char* e = std::getenv("NWG_NJ_SMEM_MAX_N");
    return e ? std::min(std::atoi(e), kSmemNJMax) : kSmemNJMax;
  }();
  return v;
}

// The shared-memory form's cluster size for a launch whose largest job has
// nmax taxa (0 when it does not fit either size).
int smem_nj_cluster(int nmax) {
  const size_t cap = 200 * 1024;   // dynamic shared memory per CTA
  if (nmax > smem_nj_max_n()) return 0;
  const bool fit8 = smem_layout(nmax, 8).bytes <= cap;
  const bool fit16 = nj_cluster_size() == 16 && smem_layout(nmax, 16).bytes <= cap;
  if (nmax < 256 && fit8) return 8;
  if (fit16) return 16;
  return fit8 ? 8 : 0;
}

cudaError_t launch_nj_smem(const void* d_jobs, int njobs, int nmax, int C, cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const NJJob* jobs = reinterpret_cast<const NJJob*>(d_jobs);
  const int bytes = (int)smem_layout(std::max(nmax, 2), C).bytes;
  cudaError_t e;
  if (C == 16) {
    if ((e = cudaFuncSetAttribute(nj_smem_kernel<16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) ||
        (e = cudaFuncSetAttribute(nj_smem_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
      return e;
    nj_smem_kernel<16><<<njobs * 16, 1024, bytes, s>>>(jobs, njobs);
  } else {
    if ((e = cudaFuncSetAttribute(nj_smem_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
    nj_smem_kernel<8><<<njobs * 8, 1024, bytes, s>>>(jobs, njobs);
  }
  return cudaGetLastError();
}

// The largest cluster (16, else 8) that the device schedules for the join loop.
int nj_cluster_size() {
  static int best = 0;
  if (best) return best;
  best = 8;
  const void* fn = (const void*)nj_cluster_kernel<16>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(1024);
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = 16;
    at.val.clusterDim.y = 1;
    at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) == cudaSuccess && clusters > 0) best = 16;
  }
  cudaGetLastError();
  return best;
}

}  // namespace nwg

extern "C" int nwg_nj(nwg_ctx* ctx, const float* D, int64_t ld, int n, nwg_join* joins, nwg_nj_stats* stats) {
  if (!ctx) return NWG_ERR_INVALID;
  nwg::Ctx* c = reinterpret_cast<nwg::Ctx*>(ctx);
  c->launches = 0;
  const int rc = c->nj(D, ld, n, false, joins, stats);
  if (stats) stats->launches = c->launches;
  return rc;
}

extern "C" int nwg_nj_dev(nwg_ctx* ctx, const float* d_D, int64_t ld, int n, nwg_join* joins, nwg_nj_stats* stats) {
  if (!ctx) return NWG_ERR_INVALID;
  nwg::Ctx* c = reinterpret_cast<nwg::Ctx*>(ctx);
  c->launches = 0;
  const int rc = c->nj(d_D, ld, n, true, joins, stats);
  if (stats) stats->launches = c->launches;
  return rc;
}
