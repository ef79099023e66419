// trace.cu -- pairwise alignment with traceback for guide-tree cherries.
//
// Replaces AlignmentMatch::computePairwise (AlignmentMatch.cu:140-317) with
// its three kernels: NeedlemanWunschGlobalMatchKernel (NeedlemanWunsch.cu:
// 184-365), NeedlemanWunschGlobalBackKernel (:393-494) and
// reorderMatchesMemory (:496-563).
//
// match_kernel<W>: a wavefront of W lanes per pair (W = 32, 16 or 8: 32/W
//   pairs per warp), int32 lanes; lane k of a front owns 8 rows of a band of
//   8W rows, one column behind lane k-1, bottom (H, F) passed by
//   __shfl_up_sync within the front.  Narrow fronts cut the rows computed
//   past the end of Y (the last band) and the ramp of W-1 columns per band.
//   Every cell yields the reference's 4-bit flags
//     bit3 L  = (H==E && H!=F) || H==diag        (:330)
//     bit2 U  = H==F || H==diag                  (:332)
//     bit1 cU = F == F_up - ge                   (:315-316, :334)
//     bit0 cL = E == E_left - ge                 (:336)
//   from the sign bits of four differences, appended by funnel shifts.
//   A lane's 8 rows of one column make one 32-bit word; the W lanes of a
//   front store W consecutive words per step: word (b*(Lx+W-1) + t)*W + k
//   holds rows b*8W + 8k .. +7 at column t-k, row r in bits 4(7-r)..4(7-r)+3.
// The walk runs in the same warp right after the pairs' last bands, while
//   their flags are still in L2, from (Lx-1, Ly-1) with the reference's rule
//   set (continue flags of the previous move first, then up, then left, else
//   diagonal); row -1 reads as left+continue, column -1 as up+continue, and
//   an up move out of row 0 ends the walk (the reference's word reload at
//   :456-457 never fires for row -1).  Each front stages the flags of a
//   window of 32 columns x 40 rows ending at its walk's cell in shared memory
//   (one load round trip), with the window's residue codes, and its lane 0
//   walks inside it; a walk leaves a window after 32 to 72 steps.
//   Characters come out in forward order, so the reorder/byte-swap pass is
//   not needed.
#include <algorithm>
#include <cstring>
#include <vector>

#include "nwg_ctx.h"

namespace nwg {

namespace {

constexpr int kTR = 8;                               // rows per lane
constexpr int kTWarps = 4;                           // warps per CTA
constexpr int kTProfBytes = kLetters * 32 * kTR;     // profile bytes per warp (6 KB, every W)

struct TraceArgs {
  const int8_t* codes;
  const int64_t* start;
  const int32_t* len;
  const int32_t* px;
  const int32_t* py;
  const int32_t* order;     // slot -> pair: pairs of similar lengths share a warp
  const int64_t* nib_off;   // per pair: first word of its nibble array
  uint32_t* nib;
  int32_t* scratch;         // per pair slot: 2 buffers x 2 ints x maxlen
  int32_t* score;
  char* outx;
  char* outy;
  int32_t* outlen;
  int64_t stride;
  int npairs;
  int scratch_cols;
  int go, ge;
  const int8_t* sub;
};

__device__ __forceinline__ unsigned tclamp(int c) {
  const unsigned u = (unsigned)c;
  return u < (unsigned)kLetters ? u : (unsigned)(kLetters - 1);
}

__constant__ char c_dec[kLetters + 1] = "ARNDCQEGHILKMFPSTWYVBZX*";   // code -> letter

static_assert(kTR == 8, "a lane's scores of one column are one 8-byte load");

// Shared memory of one front's walk: the flag words of the window (row group
// g0+gi of column x0-j at gi*32 + j) and its residue codes.
struct WalkWindow {
  uint32_t flags[5 * 32];
  int8_t xs[32];   // X[x0 - j]
  int8_t ys[40];   // Y[8*g0 + i]
};

// The backtraces of the warp's fronts (every lane calls it; p < 0: the
// front has no pair).  Lane 0 of each front walks; all lanes of a front load
// its windows.
template <int W>
__device__ void walk_pairs(const TraceArgs& a, int p, int lane, WalkWindow& w) {
  const int sl = lane % W, lead = lane - sl;
  const int8_t* X = nullptr;
  const int8_t* Y = nullptr;
  const uint32_t* nib = nullptr;
  char* ox = nullptr;
  char* oy = nullptr;
  int Lx = 0, Ly = 0;
  if (p >= 0) {
    const int ix = a.px[p], iy = a.py[p];
    X = a.codes + a.start[ix];
    Y = a.codes + a.start[iy];
    Lx = a.len[ix];
    Ly = a.len[iy];
    nib = a.nib + a.nib_off[p];
    ox = a.outx + (size_t)p * a.stride;
    oy = a.outy + (size_t)p * a.stride;
  }
  const int cap = Lx + Ly;
  // walk state (meaningful in the front's lane 0): 1 = needs a window, 2 = done
  int state = p >= 0 ? 1 : 2;
  int x = Lx - 1, y = Ly - 1, k = 0;
  unsigned prev = 12u, cell = 0u;
  bool have_cell = false, stop = false;
  for (;;) {
    const int st = __shfl_sync(0xffffffffu, state, lead);
    if (__all_sync(0xffffffffu, st == 2)) break;
    // (re)load the window ending at (x, y) of the fronts that need one; x, y >= 0 there
    const int x0 = __shfl_sync(0xffffffffu, x, lead);
    const int g0 = (__shfl_sync(0xffffffffu, y, lead) >> 3) - 4;
    if (st == 1) {
#pragma unroll
      for (int j = 0; j < 32 / W; ++j) {
        const int col = sl + j * W, c = x0 - col;
#pragma unroll
        for (int gi = 0; gi < 5; ++gi) {
          const int g = g0 + gi;
          uint32_t v = 0u;
          if (g >= 0 && c >= 0) v = nib[((size_t)(g / W) * (Lx + W - 1) + (c + g % W)) * W + g % W];
          w.flags[gi * 32 + col] = v;
        }
        w.xs[col] = c >= 0 ? X[c] : (int8_t)0;
      }
      for (int i = sl; i < 40; i += W) {
        const int r = 8 * g0 + i;
        w.ys[i] = (r >= 0 && r < Ly) ? Y[r] : (int8_t)0;
      }
    }
    __syncwarp();
    if (sl == 0 && st == 1) {
      for (;;) {
        if (!have_cell) {
          if (stop) {
            cell = 0u;   // no word reload for row -1 after an up move
          } else if (y < 0) {
            cell = x < 0 ? 0u : 9u;   // row -1: left + continue-left; corner: stop
          } else if (x < 0) {
            cell = 6u;                // column -1: up + continue-up
          } else if (x0 - x < 32 && (y >> 3) >= g0) {
            cell = (w.flags[((y >> 3) - g0) * 32 + (x0 - x)] >> (4 * (7 - (y & 7)))) & 15u;
          } else {
            state = 1;
            break;
          }
          have_cell = true;
        }
        if (!((cell & 12u) && k < cap)) {
          state = 2;
          break;
        }
        unsigned todo;
        if (((prev & 12u) == 4u) && (prev & 2u)) todo = 4u;
        else if (((prev & 12u) == 8u) && (prev & 1u)) todo = 8u;
        else if ((cell & 12u) == 4u) todo = 4u;
        else if ((cell & 12u) == 8u) todo = 8u;
        else todo = 12u;
        // a well-formed matrix never asks for a move off the -1 row/column
        // other than the ones handled here; stop rather than read outside
        if ((todo != 4u && x < 0) || (todo != 8u && y < 0)) {
          state = 2;
          break;
        }
        // residue codes: from the window inside it, else (the runs along row
        // -1 and column -1) from the sequences
        const bool xin = x >= 0 && x0 - x < 32;
        const bool yin = y >= 8 * g0 && y - 8 * g0 < 40;
        if (todo == 8u) {
          ox[k] = c_dec[tclamp(xin ? w.xs[x0 - x] : X[x])];
          oy[k] = '-';
          --x;
        } else if (todo == 4u) {
          ox[k] = '-';
          oy[k] = c_dec[tclamp(yin ? w.ys[y - 8 * g0] : Y[y])];
          --y;
          stop = y < 0;
        } else {
          ox[k] = c_dec[tclamp(xin ? w.xs[x0 - x] : X[x])];
          oy[k] = c_dec[tclamp(yin ? w.ys[y - 8 * g0] : Y[y])];
          --x;
          --y;
        }
        prev = todo | (cell & 3u);
        ++k;
        have_cell = false;
      }
      if (state == 2) {
        ox[k] = 0;
        oy[k] = 0;
        a.outlen[p] = k;
      }
    }
    __syncwarp();   // the walkers are done with the windows before they are overwritten
  }
}

template <int W>
__global__ void __launch_bounds__(32 * kTWarps) match_kernel(const TraceArgs a) {
  constexpr int S = 32 / W;         // fronts (pairs) per warp
  constexpr int BAND = W * kTR;     // rows per band
  __shared__ int8_t s_sub[kLetters * kLetters];
  __shared__ __align__(16) int8_t s_prof[kTWarps][kTProfBytes];   // per front [letter][band row]
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = a.sub[e];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int front = lane / W, sl = lane % W;
  const int wslot = (blockIdx.x * kTWarps + warp) * S;
  if (wslot >= a.npairs) return;    // the whole warp is idle
  const int slot = wslot + front;
  const int p = slot < a.npairs ? a.order[slot] : -1;
  const int8_t* X = nullptr;
  const int8_t* Y = nullptr;
  int Lx = 0, Ly = 0;
  if (p >= 0) {
    const int ix = a.px[p], iy = a.py[p];
    X = a.codes + a.start[ix];
    Y = a.codes + a.start[iy];
    Lx = a.len[ix];
    Ly = a.len[iy];
  }
  const int go = a.go, ge = a.ge;
  const int nb = (Ly + BAND - 1) / BAND;
  const int nb_max = __reduce_max_sync(0xffffffffu, (unsigned)nb);
  const int lx_max = __reduce_max_sync(0xffffffffu, (unsigned)Lx);
  int8_t* prof = s_prof[warp] + front * (kLetters * BAND);
  int32_t* scr = p >= 0 ? a.scratch + (size_t)p * 4 * a.scratch_cols : nullptr;
  uint32_t* nib = p >= 0 ? a.nib + a.nib_off[p] : nullptr;
  const int kSent = kShortMin + ge;
  int H[kTR], E[kTR];
  for (int b = 0; b < nb_max; ++b) {
    const bool band_on = b < nb;
    __syncwarp();
    if (band_on)
      for (int e = sl; e < kLetters * BAND; e += W) {
        const int x = e / BAND, row = e - x * BAND, grow = b * BAND + row;
        prof[e] = grow < Ly ? s_sub[tclamp(Y[grow]) * kLetters + x] : (int8_t)0;
      }
    __syncwarp();
    const int rowbase = b * BAND + sl * kTR;
#pragma unroll
    for (int r = 0; r < kTR; ++r) {
      H[r] = -ge * (rowbase + r + 1);
      E[r] = kSent;
    }
    int hprev = -ge * rowbase;
    int hbot = 0, fbot = 0;
    const int32_t* rd = scr + ((b + 1) & 1) * 2 * a.scratch_cols;
    int32_t* wr = scr + (b & 1) * 2 * a.scratch_cols;
    uint32_t* nb_base = nib + (size_t)b * (Lx + W - 1) * W;
    for (int t = 0; t < lx_max + W - 1; ++t) {
      const int c = t - sl;
      int hin = __shfl_up_sync(0xffffffffu, hbot, 1, W);
      int fin = __shfl_up_sync(0xffffffffu, fbot, 1, W);
      if (band_on && c >= 0 && c < Lx) {
        if (sl == 0) {
          if (b == 0) {
            hin = -ge * (c + 1);
            fin = kSent;
          } else {
            hin = rd[2 * c];
            fin = rd[2 * c + 1];
          }
        }
        // the lane's 8 scores of column c: one 8-byte load
        const uint2 pw = *reinterpret_cast<const uint2*>(prof + tclamp(X[c]) * BAND + sl * kTR);
        int diag = hprev;
        hprev = hin;
        int f = fin, hup = hin;
        uint32_t word = 0;
#pragma unroll
        for (int r = 0; r < kTR; ++r) {
          // Each flag is the sign bit of one difference (a - b - 1 < 0 <=> a <= b):
          // cu = (F_up - ge >= H_up - go), cl = (E_left - ge >= H_left - go),
          // pf = (F >= E), ps = (diag + S >= max(F, E)), i.e. H == diag + S;
          // then U = ps || pf and L = ps || !pf, since otherwise H = max(F, E)
          // and H == F <=> pf, (H == E && H != F) <=> !pf.  The bits are
          // appended to the word by funnel shifts: L, U, cU, cL of row r land
          // in bits 4(7-r)+3 .. 4(7-r).
          const int fo = f - ge, hgo = hup - go;
          const uint32_t xcu = (uint32_t)(hgo - fo - 1);
          f = max(fo, hgo);
          const int eo = E[r] - ge, ego = H[r] - go;
          const uint32_t xcl = (uint32_t)(ego - eo - 1);
          const int e = max(eo, ego);
          const int sv = (int)(int8_t)((r < 4 ? pw.x : pw.y) >> (8 * (r & 3)));
          const int sim = diag + sv;
          const uint32_t xpf = (uint32_t)(e - f - 1);
          const int t2 = max(f, e);
          const uint32_t xps = (uint32_t)(t2 - sim - 1);
          const int h = max(sim, t2);
          word = __funnelshift_l(xps | ~xpf, word, 1);   // L
          word = __funnelshift_l(xps | xpf, word, 1);    // U
          word = __funnelshift_l(xcu, word, 1);          // cU
          word = __funnelshift_l(xcl, word, 1);          // cL
          diag = H[r];
          H[r] = h;
          E[r] = e;
          hup = h;
        }
        nb_base[(size_t)t * W + sl] = word;
        hbot = H[kTR - 1];
        fbot = f;
        if (sl == W - 1 && b + 1 < nb) {
          wr[2 * c] = hbot;
          wr[2 * c + 1] = fbot;
        }
      }
    }
    if (band_on) {
      const int rr = (Ly - 1) - b * BAND;
      if (rr >= 0 && rr < BAND && sl == rr / kTR) {
        int v = 0;
#pragma unroll
        for (int r = 0; r < kTR; ++r)
          if (r == rr % kTR) v = H[r];
        a.score[p] = v;
      }
    }
  }
  // the walks, while the pairs' flags are still in L2 (the warp's stores are
  // visible to the warp after the warp barrier); their windows take the
  // place of the fronts' profiles
  __syncwarp();
  static_assert(S * sizeof(WalkWindow) <= kTProfBytes, "walk windows fit the profile's space");
  walk_pairs<W>(a, p, lane, reinterpret_cast<WalkWindow*>(s_prof[warp])[front]);
}

}  // namespace

struct TraceState {
  DevBuf codes, start, len, px, py, order, off, nib, scratch, score, outx, outy, outlen;
  ~TraceState() {
    for (DevBuf* b : {&codes, &start, &len, &px, &py, &order, &off, &nib, &scratch, &score, &outx, &outy, &outlen})
      b->release();
  }
};

namespace {

// Front width of the match kernel for a set of pairs: the least estimated
// cost, in cells, of the rows x columns computed (whole bands of 8W rows,
// ramps of W-1 columns) plus the walks, which run one after another for the
// 32/W fronts of a warp (a walk step costs about as much as kWalkStep cells:
// fitted to the kernel's times at W = 32, 16 and 8 on 3,640 pairs of 100-300
// residues on a GB300: 0.436, 0.422 and 0.652 ms).
constexpr double kWalkStep = 38.0;
int trace_lanes(const std::vector<int32_t>& len, const int32_t* px, const int32_t* py, int npairs) {
  int best = 32;
  double best_cost = 0.0;
  for (int W : {32, 16, 8}) {
    const int band = 8 * W;
    double cost = 0.0;
    for (int k = 0; k < npairs; ++k) {
      const int Lx = len[px[k]], Ly = len[py[k]];
      cost += (double)((Ly + band - 1) / band) * band * (Lx + W - 1) + kWalkStep * (32 / W) * (Lx + Ly);
    }
    if (W == 32 || cost < best_cost) {
      best = W;
      best_cost = cost;
    }
  }
  return best;
}

cudaError_t launch_match(int W, const TraceArgs& a, cudaStream_t s) {
  const int per_cta = kTWarps * (32 / W);
  const int grid = (a.npairs + per_cta - 1) / per_cta;
  if (W == 8) match_kernel<8><<<grid, 32 * kTWarps, 0, s>>>(a);
  else if (W == 16) match_kernel<16><<<grid, 32 * kTWarps, 0, s>>>(a);
  else match_kernel<32><<<grid, 32 * kTWarps, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

void Ctx::extra_release() {
  delete reinterpret_cast<TraceState*>(trace_state);
  trace_state = nullptr;
  nj_release();
  ingest_release();
  msa_release();
}

int Ctx::align_pairs(const int8_t* codes, const int64_t* offsets, int n, const int32_t* px, const int32_t* py,
                     int npairs, char* outx, char* outy, int64_t stride, int32_t* outlen, int32_t* score,
                     nwg_stats* st) {
  if (!codes || !offsets || n < 1 || npairs < 0 || (npairs > 0 && (!px || !py || !outx || !outy || !outlen)))
    return fail(NWG_ERR_INVALID, "align_pairs arguments");
  int maxlen = 0;
  for (int s = 0; s < n; ++s) {
    const int64_t L = offsets[s + 1] - offsets[s];
    if (L <= 0) return fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
    maxlen = std::max<int>(maxlen, (int)L);
  }
  for (int k = 0; k < npairs; ++k) {
    if (px[k] < 0 || px[k] >= n || py[k] < 0 || py[k] >= n) return fail(NWG_ERR_INVALID, "pair index");
    if (stride < offsets[px[k] + 1] - offsets[px[k]] + offsets[py[k] + 1] - offsets[py[k]] + 1)
      return fail(NWG_ERR_INVALID, "output stride shorter than Lx + Ly + 1");
  }
  if (npairs == 0) return NWG_OK;
  const int64_t total = offsets[n];
  for (int64_t k = 0; k < total; ++k)
    if ((unsigned)codes[k] >= (unsigned)kLetters) return fail(NWG_ERR_BAD_RESIDUE, "residue code outside 0..23");
  if (!trace_state) trace_state = new TraceState();
  TraceState& T = *reinterpret_cast<TraceState*>(trace_state);
  std::vector<int32_t> len(n);
  for (int s = 0; s < n; ++s) len[s] = (int32_t)(offsets[s + 1] - offsets[s]);
  int rc;
  if ((rc = T.codes.ensure((size_t)total)) || (rc = T.start.ensure(sizeof(int64_t) * n)) ||
      (rc = T.len.ensure(sizeof(int32_t) * n)))
    return fail(rc, "traceback allocation");
  cudaStream_t s = stream;
  if ((rc = cuda(cudaMemcpyAsync(T.codes.p, codes, (size_t)total, cudaMemcpyHostToDevice, s), "upload")) ||
      (rc = cuda(cudaMemcpyAsync(T.start.p, offsets, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s), "upload")) ||
      (rc = cuda(cudaMemcpyAsync(T.len.p, len.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s), "upload")))
    return rc;
  // batches bounded by the nibble memory (~1 GiB of words per batch)
  const int64_t kBudgetWords = (int64_t)1 << 28;
  // statistics: kernel_ms = the match kernels alone, d2h_ms = the downloads
  cudaEvent_t ev_copied = nullptr;
  if (st && (rc = cuda(cudaEventCreate(&ev_copied), "traceback event"))) return rc;
  struct EventGuard {
    cudaEvent_t e;
    ~EventGuard() {
      if (e) cudaEventDestroy(e);
    }
  } guard{ev_copied};
  const int W = trace_lanes_forced ? trace_lanes_forced : trace_lanes(len, px, py, npairs);
  const int band = 8 * W;
  int k0 = 0;
  while (k0 < npairs) {
    std::vector<int64_t> off;
    int64_t words = 0;
    int k1 = k0;
    while (k1 < npairs) {
      const int Lx = len[px[k1]], Ly = len[py[k1]];
      const int64_t w = (int64_t)((Ly + band - 1) / band) * (Lx + W - 1) * W;
      if (k1 > k0 && words + w > kBudgetWords) break;
      off.push_back(words);
      words += w;
      ++k1;
    }
    const int m = k1 - k0;
    // pairs of similar band counts and X lengths share a warp
    std::vector<int32_t> order((size_t)m);
    for (int k = 0; k < m; ++k) order[(size_t)k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int u, int v) {
      const int bu = (len[py[k0 + u]] + band - 1) / band, bv = (len[py[k0 + v]] + band - 1) / band;
      if (bu != bv) return bu > bv;
      return len[px[k0 + u]] > len[px[k0 + v]];
    });
    if ((rc = T.px.ensure(sizeof(int32_t) * m)) || (rc = T.py.ensure(sizeof(int32_t) * m)) ||
        (rc = T.order.ensure(sizeof(int32_t) * m)) ||
        (rc = T.off.ensure(sizeof(int64_t) * m)) || (rc = T.nib.ensure(sizeof(uint32_t) * (size_t)words)) ||
        (rc = T.scratch.ensure(sizeof(int32_t) * 4 * (size_t)m * maxlen)) ||
        (rc = T.score.ensure(sizeof(int32_t) * m)) || (rc = T.outx.ensure((size_t)m * stride)) ||
        (rc = T.outy.ensure((size_t)m * stride)) || (rc = T.outlen.ensure(sizeof(int32_t) * m)))
      return fail(rc, "traceback allocation");
    if ((rc = cuda(cudaMemcpyAsync(T.px.p, px + k0, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s), "upload")) ||
        (rc = cuda(cudaMemcpyAsync(T.py.p, py + k0, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s), "upload")) ||
        (rc = cuda(cudaMemcpyAsync(T.off.p, off.data(), sizeof(int64_t) * m, cudaMemcpyHostToDevice, s), "upload")) ||
        (rc = cuda(cudaMemcpyAsync(T.order.p, order.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice, s),
                   "upload")))
      return rc;
    TraceArgs a{};
    a.codes = (const int8_t*)T.codes.p;
    a.start = (const int64_t*)T.start.p;
    a.len = (const int32_t*)T.len.p;
    a.px = (const int32_t*)T.px.p;
    a.py = (const int32_t*)T.py.p;
    a.order = (const int32_t*)T.order.p;
    a.nib_off = (const int64_t*)T.off.p;
    a.nib = (uint32_t*)T.nib.p;
    a.scratch = (int32_t*)T.scratch.p;
    a.score = (int32_t*)T.score.p;
    a.outx = (char*)T.outx.p;
    a.outy = (char*)T.outy.p;
    a.outlen = (int32_t*)T.outlen.p;
    a.stride = stride;
    a.npairs = m;
    a.scratch_cols = maxlen;
    a.go = go;
    a.ge = ge;
    a.sub = (const int8_t*)b_sub.p;
    if (st) cudaEventRecord(ev0, s);
    ++launches;
    if ((rc = cuda(launch_match(W, a, s), "traceback launch"))) return rc;
    if (st) cudaEventRecord(ev1, s);
    if ((rc = cuda(cudaMemcpyAsync(outx + (size_t)k0 * stride, T.outx.p, (size_t)m * stride, cudaMemcpyDeviceToHost, s),
                   "download")) ||
        (rc = cuda(cudaMemcpyAsync(outy + (size_t)k0 * stride, T.outy.p, (size_t)m * stride, cudaMemcpyDeviceToHost, s),
                   "download")) ||
        (rc = cuda(cudaMemcpyAsync(outlen + k0, T.outlen.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s),
                   "download")))
      return rc;
    if (score &&
        (rc = cuda(cudaMemcpyAsync(score + k0, T.score.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s), "download")))
      return rc;
    if (st) cudaEventRecord(ev_copied, s);
    if ((rc = cuda(cudaStreamSynchronize(s), "traceback sync"))) return rc;
    if (st) {
      for (int k = k0; k < k1; ++k) st->cells += (int64_t)len[px[k]] * len[py[k]];
      float ms = 0.f, ms2 = 0.f;
      cudaEventElapsedTime(&ms, ev0, ev1);
      cudaEventElapsedTime(&ms2, ev1, ev_copied);
      st->kernel_ms += ms;
      st->d2h_ms += ms2;
    }
    k0 = k1;
  }
  if (st) {
    st->pairs = npairs;
    st->pairs_int32 = npairs;
  }
  return NWG_OK;
}

}  // namespace nwg

namespace {

// Post-order walk of TreeNode::getNodes (TreeNode.cpp:91-117) over the join
// records: left subtree, right subtree, then the node; a node whose two
// children are leaves is a cherry (AlignmentMatch.cu:167-186, vecSize == 2).
int cherries(const int32_t* left, const int32_t* right, int nleaves, int32_t* node, int32_t* l, int32_t* r) {
  if (nleaves < 2) return 0;
  const int nn = 2 * nleaves - 1;
  std::vector<int> stack;
  std::vector<char> expanded((size_t)nn, 0);
  stack.push_back(nn - 1);
  int cnt = 0;
  while (!stack.empty()) {
    const int v = stack.back();
    if (v < nleaves) {
      stack.pop_back();
      continue;
    }
    const int k = v - nleaves;
    if (!expanded[(size_t)v]) {
      expanded[(size_t)v] = 1;
      stack.push_back(right[k]);
      stack.push_back(left[k]);
      continue;
    }
    stack.pop_back();
    if (left[k] < nleaves && right[k] < nleaves) {
      if (node) {
        node[cnt] = v;
        l[cnt] = left[k];
        r[cnt] = right[k];
      }
      ++cnt;
    }
  }
  return cnt;
}

}  // namespace

extern "C" int nwg_cherries(const int32_t* left, const int32_t* right, int nleaves, int32_t* node, int32_t* l,
                            int32_t* r) {
  if (!left || !right || nleaves < 0) return -NWG_ERR_INVALID;
  for (int k = 0; k + 1 < nleaves; ++k) {
    if (left[k] < 0 || right[k] < 0 || left[k] >= nleaves + k || right[k] >= nleaves + k) return -NWG_ERR_INVALID;
  }
  return cherries(left, right, nleaves, node, l, r);
}

extern "C" int nwg_set_trace_lanes(nwg_ctx* ctx, int lanes) {
  if (!ctx || !(lanes == 0 || lanes == 8 || lanes == 16 || lanes == 32)) return NWG_ERR_INVALID;
  reinterpret_cast<nwg::Ctx*>(ctx)->trace_lanes_forced = lanes;
  return NWG_OK;
}

extern "C" int nwg_align_pairs(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n, const int32_t* px,
                               const int32_t* py, int npairs, char* outx, char* outy, int64_t stride, int32_t* len,
                               int32_t* score, nwg_stats* stats) {
  if (!ctx) return NWG_ERR_INVALID;
  nwg::Ctx* c = reinterpret_cast<nwg::Ctx*>(ctx);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  c->launches = 0;
  const int rc = c->align_pairs(codes, offsets, n, px, py, npairs, outx, outy, stride, len, score, stats);
  if (stats) stats->launches = c->launches;
  return rc;
}
