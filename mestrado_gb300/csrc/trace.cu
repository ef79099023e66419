// trace.cu -- pairwise alignment with traceback for guide-tree cherries.
//
// Replaces AlignmentMatch::computePairwise (AlignmentMatch.cu:140-317) with
// its three kernels: NeedlemanWunschGlobalMatchKernel (NeedlemanWunsch.cu:
// 184-365), NeedlemanWunschGlobalBackKernel (:393-494) and
// reorderMatchesMemory (:496-563).
//
// match_kernel: one warp per pair, int32 lanes, the wavefront of the score
//   kernel (lane k owns 8 rows, one column behind lane k-1, bottom (H, F)
//   passed by __shfl_up_sync).  Every cell yields the reference's 4-bit flags
//     bit3 L  = (H==E && H!=F) || H==diag        (:330)
//     bit2 U  = H==F || H==diag                  (:332)
//     bit1 cU = F == F_up - ge                   (:315-316, :334)
//     bit0 cL = E == E_left - ge                 (:336)
//   A lane's 8 rows of one column make one 32-bit word; the 32 lanes of a
//   step store 32 consecutive words (one 128-byte line): word (b*(Lx+31) + t)
//   *32 + k holds rows b*256 + 8k .. +7 at column t-k, row r in bits 4r..4r+3.
// The walk runs in lane 0 of the same warp right after the pair's last band,
//   while its flags are still in L2: one thread per pair walks from (Lx-1, Ly-1) with the
//   reference's rule set (continue flags of the previous move first, then up,
//   then left, else diagonal), row -1 reads as left+continue, column -1 as
//   up+continue, and an up move out of row 0 ends the walk (the reference's
//   word reload at :456-457 never fires for row -1).  Characters come out in
//   forward order, so the reorder/byte-swap pass is not needed.
#include <algorithm>
#include <cstring>
#include <vector>

#include "nwg_ctx.h"

namespace nwg {

namespace {

constexpr int kTR = 8;             // rows per lane
constexpr int kTBand = 32 * kTR;   // rows per band
constexpr int kTWarps = 4;         // warps (pairs) per CTA (6 KB profile per warp)

struct TraceArgs {
  const int8_t* codes;
  const int64_t* start;
  const int32_t* len;
  const int32_t* px;
  const int32_t* py;
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

__device__ __forceinline__ unsigned nibble_at(const uint32_t* nib, int Lx, int x, int y) {
  if (y < 0) return x < 0 ? 0u : 9u;     // row -1: left + continue-left; corner: stop
  if (x < 0) return 6u;                  // column -1: up + continue-up
  const int b = y / kTBand, yy = y - b * kTBand, k = yy / kTR;
  const uint32_t w = nib[((size_t)b * (Lx + 31) + (x + k)) * 32 + k];
  return (w >> (4 * (yy - k * kTR))) & 15u;
}

// The backtrace of pair p from its flags (one thread).
__device__ void walk_pair(const TraceArgs& a, int p) {
  const int ix = a.px[p], iy = a.py[p];
  const int8_t* X = a.codes + a.start[ix];
  const int8_t* Y = a.codes + a.start[iy];
  const int Lx = a.len[ix], Ly = a.len[iy];
  const uint32_t* nib = a.nib + a.nib_off[p];
  char* ox = a.outx + (size_t)p * a.stride;
  char* oy = a.outy + (size_t)p * a.stride;
  int x = Lx - 1, y = Ly - 1, k = 0;
  unsigned prev = 12u;
  unsigned cell = nibble_at(nib, Lx, x, y);
  const int cap = Lx + Ly;
  while ((cell & 12u) && k < cap) {
    unsigned todo;
    if (((prev & 12u) == 4u) && (prev & 2u)) todo = 4u;
    else if (((prev & 12u) == 8u) && (prev & 1u)) todo = 8u;
    else if ((cell & 12u) == 4u) todo = 4u;
    else if ((cell & 12u) == 8u) todo = 8u;
    else todo = 12u;
    // a well-formed matrix never asks for a move off the -1 row/column other
    // than the ones handled below; stop rather than read outside the inputs
    if ((todo != 4u && x < 0) || (todo != 8u && y < 0)) break;
    bool stop = false;
    if (todo == 8u) {
      ox[k] = c_dec[tclamp(X[x])];
      oy[k] = '-';
      --x;
    } else if (todo == 4u) {
      ox[k] = '-';
      oy[k] = c_dec[tclamp(Y[y])];
      --y;
      stop = y < 0;     // no word reload for row -1 after an up move
    } else {
      ox[k] = c_dec[tclamp(X[x])];
      oy[k] = c_dec[tclamp(Y[y])];
      --x;
      --y;
    }
    prev = todo | (cell & 3u);
    ++k;
    cell = stop ? 0u : nibble_at(nib, Lx, x, y);
  }
  ox[k] = 0;
  oy[k] = 0;
  a.outlen[p] = k;
}

__global__ void __launch_bounds__(32 * kTWarps) match_kernel(const TraceArgs a) {
  __shared__ int8_t s_sub[kLetters * kLetters];
  __shared__ __align__(8) int8_t s_prof[kTWarps][kLetters * kTBand];   // per-warp profile [letter][row]
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = a.sub[e];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int p = blockIdx.x * kTWarps + warp;
  if (p >= a.npairs) return;
  const int ix = a.px[p], iy = a.py[p];
  const int8_t* X = a.codes + a.start[ix];
  const int8_t* Y = a.codes + a.start[iy];
  const int Lx = a.len[ix], Ly = a.len[iy];
  const int go = a.go, ge = a.ge;
  const int nb = (Ly + kTBand - 1) / kTBand;
  int8_t* prof = s_prof[warp];
  int32_t* scr = a.scratch + (size_t)p * 4 * a.scratch_cols;
  uint32_t* nib = a.nib + a.nib_off[p];
  const int kSent = kShortMin + ge;
  int H[kTR], E[kTR];
  for (int b = 0; b < nb; ++b) {
    __syncwarp();
    for (int e = lane; e < kLetters * kTBand; e += 32) {
      const int x = e / kTBand, row = e - x * kTBand, grow = b * kTBand + row;
      prof[e] = grow < Ly ? s_sub[tclamp(Y[grow]) * kLetters + x] : (int8_t)0;
    }
    __syncwarp();
    const int rowbase = b * kTBand + lane * kTR;
#pragma unroll
    for (int r = 0; r < kTR; ++r) {
      H[r] = -ge * (rowbase + r + 1);
      E[r] = kSent;
    }
    int hprev = -ge * rowbase;
    int hbot = 0, fbot = 0;
    const int32_t* rd = scr + ((b + 1) & 1) * 2 * a.scratch_cols;
    int32_t* wr = scr + (b & 1) * 2 * a.scratch_cols;
    uint32_t* nb_base = nib + (size_t)b * (Lx + 31) * 32;
    for (int t = 0; t < Lx + 31; ++t) {
      const int c = t - lane;
      int hin = __shfl_up_sync(0xffffffffu, hbot, 1);
      int fin = __shfl_up_sync(0xffffffffu, fbot, 1);
      if (c >= 0 && c < Lx) {
        if (lane == 0) {
          if (b == 0) {
            hin = -ge * (c + 1);
            fin = kSent;
          } else {
            hin = rd[2 * c];
            fin = rd[2 * c + 1];
          }
        }
        // the lane's 8 scores of column c: one 8-byte load
        const uint2 pw = *reinterpret_cast<const uint2*>(prof + tclamp(X[c]) * kTBand + lane * kTR);
        int diag = hprev;
        hprev = hin;
        int f = fin, hup = hin;
        uint32_t word = 0;
#pragma unroll
        for (int r = 0; r < kTR; ++r) {
          const int fo = f - ge;
          f = max(fo, hup - go);
          const int eo = E[r] - ge;
          const int e = max(eo, H[r] - go);
          const int sv = (int)(int8_t)((r < 4 ? pw.x : pw.y) >> (8 * (r & 3)));
          const int sim = diag + sv;
          int h = max(e, f);
          h = max(h, sim);
          const uint32_t L = ((h == e) && (h != f)) || (h == sim);
          const uint32_t U = (h == f) || (h == sim);
          const uint32_t cu = (f == fo);
          const uint32_t cl = (e == eo);
          word |= ((L << 3) | (U << 2) | (cu << 1) | cl) << (4 * r);
          diag = H[r];
          H[r] = h;
          E[r] = e;
          hup = h;
        }
        nb_base[(size_t)t * 32 + lane] = word;
        hbot = H[kTR - 1];
        fbot = f;
        if (lane == 31 && b + 1 < nb) {
          wr[2 * c] = hbot;
          wr[2 * c + 1] = fbot;
        }
      }
    }
    const int rr = (Ly - 1) - b * kTBand;
    if (rr >= 0 && rr < kTBand && lane == rr / kTR) {
      int v = 0;
#pragma unroll
      for (int r = 0; r < kTR; ++r)
        if (r == rr % kTR) v = H[r];
      a.score[p] = v;
    }
  }
  // the walk, while the pair's flags are still in L2 (the warp's stores are
  // visible to lane 0 after the warp barrier)
  __syncwarp();
  if (lane == 0) walk_pair(a, p);
}

}  // namespace

struct TraceState {
  DevBuf codes, start, len, px, py, off, nib, scratch, score, outx, outy, outlen;
  ~TraceState() {
    for (DevBuf* b : {&codes, &start, &len, &px, &py, &off, &nib, &scratch, &score, &outx, &outy, &outlen})
      b->release();
  }
};

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
  const double t0 = st ? 0.0 : 0.0;
  (void)t0;
  if (st) cudaEventRecord(ev0, s);
  int k0 = 0;
  while (k0 < npairs) {
    std::vector<int64_t> off;
    int64_t words = 0;
    int k1 = k0;
    while (k1 < npairs) {
      const int Lx = len[px[k1]], Ly = len[py[k1]];
      const int64_t w = (int64_t)((Ly + kTBand - 1) / kTBand) * (Lx + 31) * 32;
      if (k1 > k0 && words + w > kBudgetWords) break;
      off.push_back(words);
      words += w;
      ++k1;
    }
    const int m = k1 - k0;
    if ((rc = T.px.ensure(sizeof(int32_t) * m)) || (rc = T.py.ensure(sizeof(int32_t) * m)) ||
        (rc = T.off.ensure(sizeof(int64_t) * m)) || (rc = T.nib.ensure(sizeof(uint32_t) * (size_t)words)) ||
        (rc = T.scratch.ensure(sizeof(int32_t) * 4 * (size_t)m * maxlen)) ||
        (rc = T.score.ensure(sizeof(int32_t) * m)) || (rc = T.outx.ensure((size_t)m * stride)) ||
        (rc = T.outy.ensure((size_t)m * stride)) || (rc = T.outlen.ensure(sizeof(int32_t) * m)))
      return fail(rc, "traceback allocation");
    if ((rc = cuda(cudaMemcpyAsync(T.px.p, px + k0, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s), "upload")) ||
        (rc = cuda(cudaMemcpyAsync(T.py.p, py + k0, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s), "upload")) ||
        (rc = cuda(cudaMemcpyAsync(T.off.p, off.data(), sizeof(int64_t) * m, cudaMemcpyHostToDevice, s), "upload")))
      return rc;
    TraceArgs a{};
    a.codes = (const int8_t*)T.codes.p;
    a.start = (const int64_t*)T.start.p;
    a.len = (const int32_t*)T.len.p;
    a.px = (const int32_t*)T.px.p;
    a.py = (const int32_t*)T.py.p;
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
    match_kernel<<<(m + kTWarps - 1) / kTWarps, 32 * kTWarps, 0, s>>>(a);
    ++launches;
    if ((rc = cuda(cudaGetLastError(), "traceback launch"))) return rc;
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
    if ((rc = cuda(cudaStreamSynchronize(s), "traceback sync"))) return rc;
    if (st) {
      for (int k = k0; k < k1; ++k) st->cells += (int64_t)len[px[k]] * len[py[k]];
    }
    k0 = k1;
  }
  if (st) {
    cudaEventRecord(ev1, s);
    cudaEventSynchronize(ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    st->kernel_ms = ms;
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
