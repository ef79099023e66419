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
// Search: RapidNJ-style.  Every row slot keeps its partners sorted by d
// (ascending) when the row is made; a row is scanned in that order while the
// lower bound d*(n-2) - T_row - T_max (minus a rounding margin) stays at or
// under the current upper bound, so a step touches a few entries per row
// instead of the whole matrix.  All floating-point operations use the _rn
// intrinsics in the reference's evaluation order (no contraction).
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstring>
#include <vector>

#include "nwg_ctx.h"

namespace nwg {

namespace {

constexpr int kNJMaxN = 8192;          // row sort in shared memory
constexpr int kScanWarps = 8;

struct Entry {
  float d;
  int v;
};

struct Pick {
  double q1, q2;
  int a, b;      // a < b node ids
};

struct NJDev {
  float* D;            // n0 x n0, slots
  double* T;           // per slot
  int* slot;           // per node id (2n0-1), -1 dead
  int* act;            // active node ids ascending [n0]
  int* na;             // active count
  Entry* rows;         // per slot: n0 entries
  int* rowlen;         // per slot
  int* head;           // per slot: first entry that may be live
  double* rq;          // per active index: best q1 of the row
  int* ra;             // per active index: best pair a
  int* rb;             // per active index: best pair b
  double* gl;          // [0] T max, [1] upper bound, [2] hi of winner
  Pick* win;
  unsigned long long* cnt;   // [0] ties (this step), [1] ambiguous pairs (this step)
  unsigned long long* stats; // [0] ambiguous steps, [1] tie steps
  nwg_join* joins;
  float* vd;           // per slot, new row values
  int n0;
};

__device__ __forceinline__ bool better(double q, int b, int a, double q2, int b2, int a2) {
  if (q < q2) return true;
  if (q > q2) return false;
  return b > b2 || (b == b2 && a > a2);
}

// q as the reference's candidate list computes it (record order).
__device__ __forceinline__ double q_record(const NJDev& s, float d, int u, int v, int watermark, double nm2) {
  const int a = min(u, v), b = max(u, v);
  const int sa = s.slot[a], sb = s.slot[b];
  int f = sa, g = sb;
  if (b >= watermark && sb < sa) {
    f = sb;
    g = sa;
  }
  return __dsub_rn(__dsub_rn(__dmul_rn((double)d, nm2), s.T[f]), s.T[g]);
}

__device__ __forceinline__ double q_heap(const NJDev& s, float d, int u, int v, double nm2) {
  return __dsub_rn(__dmul_rn((double)d, nm2), __dadd_rn(s.T[s.slot[u]], s.T[s.slot[v]]));
}

// rounding margin of the lower bound: generous multiple of the double ulp
__device__ __forceinline__ double margin(double x, double tu, double tmax) {
  return 1e-12 * (fabs(x) + fabs(tu) + fabs(tmax)) + 1e-300;
}

// Sequential row sums (buildGblRowSums): one thread per active row.
__global__ void rowsum_kernel(NJDev s) {
  const int na = *s.na;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= na) return;
  const float* row = s.D + (size_t)s.slot[s.act[k]] * s.n0;
  double sum = 0.0;
  for (int j = 0; j < na; ++j) sum = __dadd_rn(sum, (double)row[s.slot[s.act[j]]]);
  s.T[s.slot[s.act[k]]] = sum;
}

// Bitonic sort of (d, v) pairs in shared memory, n <= kNJMaxN (padded).
__device__ void block_sort(Entry* e, int n) {
  int m = 1;
  while (m < n) m <<= 1;
  for (int k = n + threadIdx.x; k < m; k += blockDim.x) e[k] = Entry{FLT_MAX, INT_MAX};
  __syncthreads();
  for (int size = 2; size <= m; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < m / 2; t += blockDim.x) {
        const int i = 2 * t - (t & (stride - 1));
        const int j = i + stride;
        const bool up = (i & size) == 0;
        const Entry A = e[i], B = e[j];
        const bool gt = A.d > B.d || (A.d == B.d && A.v > B.v);
        if (gt == up) {
          e[i] = B;
          e[j] = A;
        }
      }
      __syncthreads();
    }
  }
}

// Sorted partner list of every leaf row (initial rows).
__global__ void init_rows_kernel(NJDev s) {
  extern __shared__ Entry sh[];
  const int u = blockIdx.x;
  const int n = s.n0;
  int cnt = 0;
  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    const int k = v < u ? v : v - 1;
    if (v != u) sh[k] = Entry{s.D[(size_t)u * n + v], v};
  }
  cnt = n - 1;
  __syncthreads();
  block_sort(sh, cnt);
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) s.rows[(size_t)u * n + k] = sh[k];
  if (threadIdx.x == 0) {
    s.rowlen[u] = cnt;
    s.head[u] = 0;
  }
}

// T max over active rows and a first upper bound: the q of every row's first
// live partner (dead entries at a row's head are skipped for good).
__global__ void prepare_kernel(NJDev s, int watermark, double nm2) {
  __shared__ double red_t[32], red_u[32];
  const int na = *s.na;
  double tmax = -DBL_MAX, ub = DBL_MAX;
  for (int k = threadIdx.x; k < na; k += blockDim.x) {
    const int u = s.act[k];
    const int su = s.slot[u];
    tmax = fmax(tmax, s.T[su]);
    const Entry* row = s.rows + (size_t)su * s.n0;
    int h = s.head[su];
    const int len = s.rowlen[su];
    while (h < len && s.slot[row[h].v] < 0) ++h;
    s.head[su] = h;
    if (h < len) ub = fmin(ub, q_record(s, row[h].d, u, row[h].v, watermark, nm2));
  }
  for (int o = 16; o > 0; o >>= 1) {
    tmax = fmax(tmax, __shfl_down_sync(0xffffffffu, tmax, o));
    ub = fmin(ub, __shfl_down_sync(0xffffffffu, ub, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red_t[threadIdx.x >> 5] = tmax;
    red_u[threadIdx.x >> 5] = ub;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      tmax = fmax(tmax, red_t[w]);
      ub = fmin(ub, red_u[w]);
    }
    tmax = fmax(tmax, red_t[0]);
    ub = fmin(ub, red_u[0]);
    s.gl[0] = tmax;
    s.gl[1] = ub;
    s.cnt[0] = 0;
    s.cnt[1] = 0;
  }
}

// Phase 1: best pair of every active row among entries whose lower bound is
// at most the upper bound.
__global__ void __launch_bounds__(32 * kScanWarps) scan_kernel(NJDev s, int watermark, double nm2) {
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * kScanWarps + (threadIdx.x >> 5);
  const int na = *s.na;
  if (k >= na) return;
  const int u = s.act[k];
  const int su = s.slot[u];
  const double tu = s.T[su], tmax = s.gl[0], ub = s.gl[1];
  const Entry* row = s.rows + (size_t)su * s.n0;
  const int len = s.rowlen[su];
  double bq = DBL_MAX;
  int ba = INT_MAX, bb = -1;
  for (int base = s.head[su]; base < len; base += 32) {
    const int e = base + lane;
    bool go_on = false;
    if (e < len) {
      const Entry en = row[e];
      const double x = __dmul_rn((double)en.d, nm2);
      const double lb = __dsub_rn(__dsub_rn(x, tu), tmax);
      go_on = lb - margin(x, tu, tmax) <= ub;
      if (go_on && s.slot[en.v] >= 0) {
        const double q = q_record(s, en.d, u, en.v, watermark, nm2);
        const int a = min(u, en.v), b = max(u, en.v);
        if (better(q, b, a, bq, bb, ba)) {
          bq = q;
          ba = a;
          bb = b;
        }
      }
    }
    if (!__any_sync(0xffffffffu, go_on)) break;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double q2 = __shfl_down_sync(0xffffffffu, bq, o);
    const int a2 = __shfl_down_sync(0xffffffffu, ba, o);
    const int b2 = __shfl_down_sync(0xffffffffu, bb, o);
    if (better(q2, b2, a2, bq, bb, ba)) {
      bq = q2;
      ba = a2;
      bb = b2;
    }
  }
  if (lane == 0) {
    s.rq[k] = bq;
    s.ra[k] = ba;
    s.rb[k] = bb;
  }
}

// Winner over rows, and the bound of the ambiguity pass.
__global__ void pick_kernel(NJDev s, double nm2) {
  __shared__ double sq[32];
  __shared__ int sa[32], sb[32];
  const int na = *s.na;
  double bq = DBL_MAX;
  int ba = INT_MAX, bb = -1;
  for (int k = threadIdx.x; k < na; k += blockDim.x) {
    if (s.rb[k] >= 0 && better(s.rq[k], s.rb[k], s.ra[k], bq, bb, ba)) {
      bq = s.rq[k];
      ba = s.ra[k];
      bb = s.rb[k];
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double q2 = __shfl_down_sync(0xffffffffu, bq, o);
    const int a2 = __shfl_down_sync(0xffffffffu, ba, o);
    const int b2 = __shfl_down_sync(0xffffffffu, bb, o);
    if (better(q2, b2, a2, bq, bb, ba)) {
      bq = q2;
      ba = a2;
      bb = b2;
    }
  }
  if ((threadIdx.x & 31) == 0) {
    sq[threadIdx.x >> 5] = bq;
    sa[threadIdx.x >> 5] = ba;
    sb[threadIdx.x >> 5] = bb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      if (better(sq[w], sb[w], sa[w], bq, bb, ba)) {
        bq = sq[w];
        ba = sa[w];
        bb = sb[w];
      }
    Pick p;
    p.q1 = bq;
    p.a = ba;
    p.b = bb;
    if (bb < 0) {            // no candidate: cannot happen with >= 2 active nodes
      atomicAdd(&s.stats[2], 1ull);
      *s.win = p;
      s.gl[2] = -DBL_MAX;
      return;
    }
    const float d = s.D[(size_t)s.slot[ba] * s.n0 + s.slot[bb]];
    p.q2 = q_heap(s, d, ba, bb, nm2);
    *s.win = p;
    s.gl[2] = fmax(p.q1, p.q2);
  }
}

// Phase 2: could the heap rounding of another pair, or a wide exact tie,
// change the reference's pick?  Each pair is counted from the row of its
// larger id (that row always holds it).
__global__ void __launch_bounds__(32 * kScanWarps) ambiguity_kernel(NJDev s, int watermark, double nm2) {
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * kScanWarps + (threadIdx.x >> 5);
  const int na = *s.na;
  if (k >= na) return;
  const int u = s.act[k];
  const int su = s.slot[u];
  const double tu = s.T[su], tmax = s.gl[0], hi = s.gl[2];
  const Pick w = *s.win;
  if (w.b < 0) return;
  const bool robust_w = w.q1 == w.q2;
  const Entry* row = s.rows + (size_t)su * s.n0;
  const int len = s.rowlen[su];
  unsigned ties = 0, amb = 0;
  for (int base = s.head[su]; base < len; base += 32) {
    const int e = base + lane;
    bool go_on = false;
    if (e < len) {
      const Entry en = row[e];
      const double x = __dmul_rn((double)en.d, nm2);
      const double lb = __dsub_rn(__dsub_rn(x, tu), tmax);
      go_on = lb - margin(x, tu, tmax) <= hi;
      if (go_on && en.v < u && s.slot[en.v] >= 0) {
        const int a = en.v, b = u;
        const double q1 = q_record(s, en.d, u, en.v, watermark, nm2);
        const double q2 = q_heap(s, en.d, u, en.v, nm2);
        const double lo = fmin(q1, q2);
        if (lo <= hi) {
          if (a == w.a && b == w.b) ++ties;
          else if (robust_w && q1 == q2 && q1 == w.q1) ++ties;
          else ++amb;
        }
      }
    }
    if (!__any_sync(0xffffffffu, go_on)) break;
  }
  for (int o = 16; o > 0; o >>= 1) {
    ties += __shfl_down_sync(0xffffffffu, ties, o);
    amb += __shfl_down_sync(0xffffffffu, amb, o);
  }
  if (lane == 0) {
    if (ties) atomicAdd(&s.cnt[0], (unsigned long long)ties);
    if (amb) atomicAdd(&s.cnt[1], (unsigned long long)amb);
  }
}

// The join: record, modifyMatrix, new sorted row, active list.  One CTA.
__global__ void join_kernel(NJDev s, int step, int next, int m_n) {
  extern __shared__ Entry sh[];
  __shared__ int s_pos[1024 / 32 + 1];
  __shared__ float s_tmp_dummy;
  const Pick w = *s.win;
  if (w.b < 0) return;                 // counted as an internal error by pick_kernel
  const int i = w.a, j = w.b;          // i < j
  const int si = s.slot[i], sj = s.slot[j];
  const int n0 = s.n0;
  const int na = *s.na;
  const float dmin = s.D[(size_t)si * n0 + sj];
  (void)s_tmp_dummy;
  if (threadIdx.x == 0) {
    // TreeNode::join with left = min id, right = max id
    const double Ti = s.T[si], Tj = s.T[sj];
    double li, lj;
    const double half = 0.5;
    if (m_n == 2) {
      li = lj = __dmul_rn((double)dmin, half);
    } else {
      const double nm2 = (double)(m_n - 2);
      li = __dmul_rn(half, __dadd_rn((double)dmin, __ddiv_rn(__dsub_rn(Ti, Tj), nm2)));
      lj = __dmul_rn(half, __dadd_rn((double)dmin, __ddiv_rn(__dsub_rn(Tj, Ti), nm2)));
    }
    if (li < 0.0) {
      lj = __dsub_rn(lj, li);
      li = 0.0;
    } else if (lj < 0.0) {
      li = __dsub_rn(li, lj);
      lj = 0.0;
    }
    nwg_join& J = s.joins[step];
    J.i = i;
    J.j = j;
    J.node = next;
    J.n = m_n;
    J.d = dmin;
    J.q = w.q1;
    J.ti = Ti;
    J.tj = Tj;
    J.len_i = li;
    J.len_j = lj;
    const unsigned long long ties = s.cnt[0], amb = s.cnt[1];
    if (amb > 0 || ties > 4) atomicAdd(&s.stats[0], 1ull);
    else if (ties > 1) atomicAdd(&s.stats[1], 1ull);
  }
  __syncthreads();
  // new row values, T updates, D row/column of slot si (k over active, k != i, j)
  for (int k = threadIdx.x; k < na; k += blockDim.x) {
    const int v = s.act[k];
    if (v == i || v == j) continue;
    const int sk = s.slot[v];
    const float Dik = s.D[(size_t)si * n0 + sk];
    const float Djk = s.D[(size_t)sj * n0 + sk];
    const float sumf = __fadd_rn(Dik, Djk);
    const float tmp = __fmul_rn(__fsub_rn(sumf, dmin), 0.5f);
    s.vd[sk] = tmp;
    s.T[sk] = __dadd_rn(s.T[sk], (double)__fsub_rn(tmp, sumf));
  }
  __syncthreads();
  // sequential sum of tmp in ascending id order (SpeciesBlock.cpp:799)
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int k = 0; k < na; ++k) {
      const int v = s.act[k];
      if (v == i || v == j) continue;
      sum = __dadd_rn(sum, (double)s.vd[s.slot[v]]);
    }
    s.T[si] = sum;
  }
  // D updates and the new node's sorted row (entries: all remaining active)
  int cnt = 0;
  for (int k = threadIdx.x; k < na; k += blockDim.x) {
    const int v = s.act[k];
    if (v == i || v == j) continue;
    const int sk = s.slot[v];
    const float t = s.vd[sk];
    s.D[(size_t)sk * n0 + si] = t;
    s.D[(size_t)si * n0 + sk] = t;
  }
  // compacted active list: ascending ids without i, j, plus next at the end
  {
    // block-wide exclusive scan of keep flags over the ascending list
    const int chunk = (na + blockDim.x - 1) / blockDim.x;
    const int k0 = threadIdx.x * chunk;
    int keep = 0;
    for (int k = k0; k < k0 + chunk && k < na; ++k) keep += (s.act[k] != i && s.act[k] != j);
    // warp scan
    int incl = keep;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((threadIdx.x & 31) >= o) incl += y;
    }
    if ((threadIdx.x & 31) == 31) s_pos[threadIdx.x >> 5] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) {
        const int t = s_pos[w2];
        s_pos[w2] = acc;
        acc += t;
      }
      s_pos[blockDim.x >> 5] = acc;
    }
    __syncthreads();
    int pos = s_pos[threadIdx.x >> 5] + incl - keep;
    // gather into shared first (reads of s.act must finish before writes)
    int* tmp_ids = reinterpret_cast<int*>(sh);
    for (int k = k0; k < k0 + chunk && k < na; ++k)
      if (s.act[k] != i && s.act[k] != j) tmp_ids[pos++] = s.act[k];
    __syncthreads();
    cnt = s_pos[blockDim.x >> 5];
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) s.act[k] = tmp_ids[k];
    __syncthreads();
  }
  // sorted row of the new node in slot si
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
    const int v = s.act[k];
    sh[k] = Entry{s.vd[s.slot[v]], v};
  }
  __syncthreads();
  block_sort(sh, cnt);
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) s.rows[(size_t)si * n0 + k] = sh[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    s.rowlen[si] = cnt;
    s.head[si] = 0;
    s.act[cnt] = next;
    *s.na = cnt + 1;
    s.slot[j] = -1;
    s.slot[i] = -1;
    s.slot[next] = si;
  }
}

}  // namespace

struct NJState {
  DevBuf D, T, slot, act, na, rows, rowlen, head, rq, ra, rb, gl, win, cnt, stats, joins, vd;
  ~NJState() {
    for (DevBuf* b : {&D, &T, &slot, &act, &na, &rows, &rowlen, &head, &rq, &ra, &rb, &gl, &win, &cnt, &stats,
                      &joins, &vd})
      b->release();
  }
};

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
    if (st) *st = stats;
    return NWG_OK;
  }
  if (!nj_state) nj_state = new NJState();
  NJState& S = *reinterpret_cast<NJState*>(nj_state);
  const int nn = 2 * n - 1;
  int rc;
  if ((rc = S.D.ensure(sizeof(float) * (size_t)n * n)) || (rc = S.T.ensure(sizeof(double) * n)) ||
      (rc = S.slot.ensure(sizeof(int) * nn)) || (rc = S.act.ensure(sizeof(int) * (n + 1))) ||
      (rc = S.na.ensure(sizeof(int))) || (rc = S.rows.ensure(sizeof(Entry) * (size_t)n * n)) ||
      (rc = S.rowlen.ensure(sizeof(int) * n)) || (rc = S.head.ensure(sizeof(int) * n)) ||
      (rc = S.rq.ensure(sizeof(double) * n)) || (rc = S.ra.ensure(sizeof(int) * n)) ||
      (rc = S.rb.ensure(sizeof(int) * n)) || (rc = S.gl.ensure(sizeof(double) * 4)) ||
      (rc = S.win.ensure(sizeof(Pick))) || (rc = S.cnt.ensure(sizeof(unsigned long long) * 2)) ||
      (rc = S.stats.ensure(sizeof(unsigned long long) * 3)) ||
      (rc = S.joins.ensure(sizeof(nwg_join) * (n - 1))) || (rc = S.vd.ensure(sizeof(float) * n)))
    return fail(rc, "nj allocation");
  cudaStream_t s = stream;
  const cudaMemcpyKind kind = device_D ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if ((rc = cuda(cudaMemcpy2DAsync(S.D.p, sizeof(float) * n, D, sizeof(float) * ld, sizeof(float) * n, n, kind, s),
                 "nj upload")))
    return rc;
  std::vector<int> slot0(nn, -1), act0(n + 1, 0);
  for (int k = 0; k < n; ++k) slot0[k] = k, act0[k] = k;
  const int na0 = n;
  if ((rc = cuda(cudaMemcpyAsync(S.slot.p, slot0.data(), sizeof(int) * nn, cudaMemcpyHostToDevice, s), "nj upload")) ||
      (rc = cuda(cudaMemcpyAsync(S.act.p, act0.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s), "nj upload")) ||
      (rc = cuda(cudaMemcpyAsync(S.na.p, &na0, sizeof(int), cudaMemcpyHostToDevice, s), "nj upload")) ||
      (rc = cuda(cudaMemsetAsync(S.stats.p, 0, sizeof(unsigned long long) * 3, s), "nj upload")))
    return rc;
  cudaStreamSynchronize(s);   // host vectors above are pageable and local
  NJDev d{};
  d.D = (float*)S.D.p;
  d.T = (double*)S.T.p;
  d.slot = (int*)S.slot.p;
  d.act = (int*)S.act.p;
  d.na = (int*)S.na.p;
  d.rows = (Entry*)S.rows.p;
  d.rowlen = (int*)S.rowlen.p;
  d.head = (int*)S.head.p;
  d.rq = (double*)S.rq.p;
  d.ra = (int*)S.ra.p;
  d.rb = (int*)S.rb.p;
  d.gl = (double*)S.gl.p;
  d.win = (Pick*)S.win.p;
  d.cnt = (unsigned long long*)S.cnt.p;
  d.stats = (unsigned long long*)S.stats.p;
  d.joins = (nwg_join*)S.joins.p;
  d.vd = (float*)S.vd.p;
  d.n0 = n;
  int m = 1;
  while (m < n) m <<= 1;
  const size_t sort_smem = sizeof(Entry) * (size_t)m;
  if ((rc = cuda(cudaFuncSetAttribute(init_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sort_smem),
                 "nj smem")) ||
      (rc = cuda(cudaFuncSetAttribute(join_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sort_smem),
                 "nj smem")))
    return rc;
  if (st) cudaEventRecord(ev0, s);
  rowsum_kernel<<<(n + 127) / 128, 128, 0, s>>>(d);
  init_rows_kernel<<<n, 1024, sort_smem, s>>>(d);
  launches += 2;
  // host-side schedule (deterministic in n, as the reference's)
  const int kBinT = 30 * 31 / 2;
  int steps = std::max((int)((float)n * 0.5f), 200);
  int pq_ck = 500;
  long long ave0 = (((long long)(n - 1) * n) / 2) / kBinT;
  long long ub = ((long long)n * (n - 1)) / 2;
  int watermark = n, next = n, m_n = n, na = n;
  for (int step = 0; step < n - 1; ++step) {
    const double nm2 = (double)(m_n - 2);
    const int sg = (na + kScanWarps - 1) / kScanWarps;
    prepare_kernel<<<1, 1024, 0, s>>>(d, watermark, nm2);
    scan_kernel<<<sg, 32 * kScanWarps, 0, s>>>(d, watermark, nm2);
    pick_kernel<<<1, 1024, 0, s>>>(d, nm2);
    ambiguity_kernel<<<sg, 32 * kScanWarps, 0, s>>>(d, watermark, nm2);
    join_kernel<<<1, 1024, sort_smem, s>>>(d, step, next, m_n);
    launches += 5;
    if (--pq_ck == 0) {
      pq_ck = 500;
      if (steps > 0) {
        const double r = (double)(ub / kBinT) / (double)ave0;
        if (r > 2.0) ++stats.pq_trigger_open;
      }
    }
    --m_n;
    na -= 1;
    ++next;
    if (steps == 0) {
      rowsum_kernel<<<(na + 127) / 128, 128, 0, s>>>(d);
      ++launches;
      ++stats.rebuilds;
      watermark = next;
      steps = (m_n < 200) ? INT_MAX : (int)((float)m_n * 0.5f);
      ave0 = (((long long)(m_n - 1) * m_n) / 2) / kBinT;
      ub = ((long long)m_n * (m_n - 1)) / 2;
    } else {
      --steps;
      ub += na - 1;
    }
    if ((rc = cuda(cudaGetLastError(), "nj launch"))) return rc;
  }
  unsigned long long dst[3] = {0, 0, 0};
  if ((rc = cuda(cudaMemcpyAsync(joins, S.joins.p, sizeof(nwg_join) * (n - 1), cudaMemcpyDeviceToHost, s), "nj download")) ||
      (rc = cuda(cudaMemcpyAsync(dst, S.stats.p, sizeof(dst), cudaMemcpyDeviceToHost, s), "nj download")) ||
      (rc = cuda(cudaStreamSynchronize(s), "nj sync")))
    return rc;
  if (dst[2]) return fail(NWG_ERR_CUDA, "neighbor joining found no candidate pair");
  stats.ambiguous_steps = (int64_t)dst[0];
  stats.tie_steps = (int64_t)dst[1];
  if (st) {
    cudaEventRecord(ev1, s);
    cudaEventSynchronize(ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    stats.device_ms = ms;
    *st = stats;
  }
  return NWG_OK;
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
