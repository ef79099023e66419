// msa.cu -- progressive alignment along the guide tree.
//
// The reference's AlignmentMatch::computeMSA (AlignmentMatch.cu:320-434) is
// an empty loop, so this is the build's own definition (parity unpinned; the
// oracle's nwo_msa is the same algorithm on the CPU): internal node n+k joins
// left[k] (X, columns) and right[k] (Y, rows).  A profile is its columns'
// letter counts (int16 x 24 per column), in reversed column order like the
// codes.  A merge aligns two profiles with the pairwise recurrence and flags
// of the cherry traceback (NeedlemanWunsch.cu:184-365 and :393-494),
// generalised: cell score sum_x sum_y cX[x] cY[y] S[x][y], gap penalties
// go*kX*kY and ge*kX*kY (k = sequences of a profile), 64-bit integers.  Two
// single sequences therefore align exactly as nwg_align_pairs aligns them.
//
// Device work per tree level (every merge whose children are done):
//  1. msa_dp_kernel, one CTA per merge: 256 rows per strip, one thread per
//     row, an anti-diagonal step per __syncthreads; thread r keeps
//     W[x] = sum_y cY[r][y] S[x][y] in registers, so a cell costs 24
//     multiply-adds (in int32 when kX * kY * max|S| < 2^31, which bounds the
//     sum; else in int64), with the next column's counts loaded a step
//     ahead; (H, F) of the row above comes through shared memory, the bottom
//     row of a strip through global scratch; the 4 flag bits of every cell
//     are stored one byte per cell, anti-diagonal major (coalesced); then
//     thread 0 walks the flags with the traceback rules while they are still
//     in L2, ops in forward order (columns the walk leaves are appended
//     opposite gaps);
//  2. msa_build_kernel, one CTA per merge: the merged profile and, for both
//     children, the map of their columns to the new ones.
// At the end the final position of every column is resolved parents first
// (msa_pos_kernel) and every leaf's residues are scattered into its row.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "nwg_ctx.h"

namespace nwg {
namespace {

constexpr int kMR = 256;   // rows per strip = threads per merge CTA

struct MergeDesc {
  int64_t xoff, yoff, ooff;   // first column of X, Y and the new profile in the count pool
  int64_t xmap, ymap;         // X's and Y's column maps (written here)
  int64_t nib;                // first flag byte
  int64_t ops;                // first op byte (capacity lx + ly)
  int64_t scratch;            // first (H, F) pair of the strip-boundary scratch (lx entries)
  int32_t lx, ly, kx, ky;
  int32_t nops;               // written by the walk
  int32_t mac32;              // kx * ky * max|S| < 2^31: a cell's score sum fits int32
};

__device__ __forceinline__ int64_t mx64(int64_t a, int64_t b) { return a > b ? a : b; }

__device__ __forceinline__ unsigned msa_nib(const uint8_t* nib, int lx, int x, int y) {
  if (y < 0) return x < 0 ? 0u : 9u;     // row -1: left + continue-left; corner: stop
  if (x < 0) return 6u;                  // column -1: up + continue-up
  const int s = y / kMR, yl = y - s * kMR;
  return nib[(size_t)s * (size_t)(lx + kMR - 1) * kMR + (size_t)(x + yl) * kMR + yl];
}

// The traceback rules of the cherry alignment over the merge's flags, ops in
// forward order (one thread).
__device__ void msa_walk(MergeDesc& m, const uint8_t* nib, uint8_t* ops) {
  const int lx = m.lx, ly = m.ly;
  const uint8_t* nb = nib + m.nib;
  uint8_t* op = ops + m.ops;
  int x = lx - 1, y = ly - 1, k = 0;
  unsigned prev = 12u;
  unsigned cell = msa_nib(nb, lx, x, y);
  while ((cell & 12u) && k < lx + ly) {
    unsigned todo;
    if (((prev & 12u) == 4u) && (prev & 2u)) todo = 4u;
    else if (((prev & 12u) == 8u) && (prev & 1u)) todo = 8u;
    else if ((cell & 12u) == 4u) todo = 4u;
    else if ((cell & 12u) == 8u) todo = 8u;
    else todo = 12u;
    if ((todo != 4u && x < 0) || (todo != 8u && y < 0)) break;
    bool stop = false;
    op[k++] = (uint8_t)todo;
    if (todo == 8u) {
      --x;
    } else if (todo == 4u) {
      --y;
      stop = y < 0;
    } else {
      --x;
      --y;
    }
    prev = todo | (cell & 3u);
    cell = stop ? 0u : msa_nib(nb, lx, x, y);
  }
  while (x >= 0 && k < lx + ly) {   // columns the walk left, opposite gaps
    op[k++] = 8u;
    --x;
  }
  while (y >= 0 && k < lx + ly) {
    op[k++] = 4u;
    --y;
  }
  m.nops = k;
}

__global__ void __launch_bounds__(kMR) msa_dp_kernel(MergeDesc* md, const int16_t* __restrict__ cnt, uint8_t* nib,
                                                     longlong2* __restrict__ scratch, const int8_t* __restrict__ sub,
                                                     int go, int ge, uint8_t* __restrict__ ops) {
  __shared__ int8_t s_sub[kLetters * kLetters];
  __shared__ int64_t sh_h[2][kMR], sh_f[2][kMR];
  const MergeDesc m = md[blockIdx.x];
  for (int e = threadIdx.x; e < kLetters * kLetters; e += blockDim.x) s_sub[e] = sub[e];
  __syncthreads();
  const int lx = m.lx, ly = m.ly;
  const int64_t kk = (int64_t)m.kx * m.ky;
  const int64_t GO = (int64_t)go * kk, GE = (int64_t)ge * kk;
  const int64_t kSent = -(((int64_t)1) << 60);
  const int16_t* X = cnt + m.xoff * kLetters;
  const int16_t* Y = cnt + m.yoff * kLetters;
  longlong2* bnd = scratch + m.scratch;
  const int tid = threadIdx.x;
  const int nstrips = (ly + kMR - 1) / kMR;
  for (int sidx = 0; sidx < nstrips; ++sidx) {
    const int r = sidx * kMR + tid;       // this thread's row
    const bool live = r < ly;
    int32_t W[kLetters];
#pragma unroll
    for (int x = 0; x < kLetters; ++x) W[x] = 0;
    if (live) {
      const int16_t* cy = Y + (size_t)r * kLetters;
      for (int b = 0; b < kLetters; ++b) {
        const int c = cy[b];
        if (c == 0) continue;
#pragma unroll
        for (int x = 0; x < kLetters; ++x) W[x] += c * (int)s_sub[b * kLetters + x];
      }
    }
    int64_t hleft = -GE * (r + 1), eleft = kSent;
    int64_t diag = -GE * r;               // H[r-1][-1] (0 for row 0)
    uint8_t* nb = nib + m.nib + (size_t)sidx * (size_t)(lx + kMR - 1) * kMR;
    const int steps = lx + kMR - 1;
    // the counts of this thread's column, loaded one step ahead
    auto load_col = [&](int c, uint4 (&v)[3]) {
      if (c >= 0 && c < lx) {
        const uint4* p = reinterpret_cast<const uint4*>(X + (size_t)c * kLetters);
        v[0] = p[0];
        v[1] = p[1];
        v[2] = p[2];
      }
    };
    uint4 cur[3] = {}, nxt[3] = {};
    load_col(-tid, cur);
    for (int t = 0; t < steps; ++t) {
      const int c = t - tid;
      const int par = t & 1;
      load_col(c + 1, nxt);
      if (live && c >= 0 && c < lx) {
        int64_t hup, fup;
        if (tid == 0) {
          if (sidx == 0) {
            hup = -GE * (c + 1);
            fup = kSent;
          } else {
            const longlong2 v = bnd[c];
            hup = v.x;
            fup = v.y;
          }
        } else {
          hup = sh_h[par ^ 1][tid - 1];
          fup = sh_f[par ^ 1][tid - 1];
        }
        int64_t s = 0;
        if (m.mac32) {   // |s| <= kx * ky * max|S| < 2^31
          int32_t s32 = 0;
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const uint32_t w[4] = {cur[q].x, cur[q].y, cur[q].z, cur[q].w};
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              s32 += (int32_t)(int16_t)(w[h] & 0xFFFFu) * W[q * 8 + 2 * h];
              s32 += (int32_t)(int16_t)(w[h] >> 16) * W[q * 8 + 2 * h + 1];
            }
          }
          s = s32;
        } else {
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const uint32_t w[4] = {cur[q].x, cur[q].y, cur[q].z, cur[q].w};
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              s += (int64_t)(int16_t)(w[h] & 0xFFFFu) * W[q * 8 + 2 * h];
              s += (int64_t)(int16_t)(w[h] >> 16) * W[q * 8 + 2 * h + 1];
            }
          }
        }
        const int64_t f = mx64(fup - GE, hup - GO);
        const uint32_t cu = f == fup - GE;
        const int64_t e = mx64(eleft - GE, hleft - GO);
        const uint32_t cl = e == eleft - GE;
        const int64_t sim = diag + s;
        const int64_t h = mx64(mx64(e, f), sim);
        const uint32_t L = ((h == e) && (h != f)) || (h == sim);
        const uint32_t U = (h == f) || (h == sim);
        nb[(size_t)t * kMR + tid] = (uint8_t)((L << 3) | (U << 2) | (cu << 1) | cl);
        diag = hup;
        hleft = h;
        eleft = e;
        sh_h[par][tid] = h;
        sh_f[par][tid] = f;
        if (tid == kMR - 1 && sidx + 1 < nstrips) bnd[c] = make_longlong2(h, f);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) cur[q] = nxt[q];
      __syncthreads();
    }
  }
  // the walk, while the merge's flags are still in L2 (the CTA barrier above
  // makes every thread's flags visible to thread 0)
  if (tid == 0) msa_walk(md[blockIdx.x], nib, ops);
}

// Merged profile and child maps; one CTA per merge, ops scanned in chunks.
__global__ void __launch_bounds__(1024) msa_build_kernel(const MergeDesc* __restrict__ md, int16_t* cnt, int32_t* maps,
                                                         const uint8_t* __restrict__ ops) {
  __shared__ int wx[33], wy[33];
  __shared__ int basex, basey;
  const MergeDesc m = md[blockIdx.x];
  const int k = m.nops;
  const uint8_t* op = ops + m.ops;
  const int16_t* X = cnt + m.xoff * kLetters;
  const int16_t* Y = cnt + m.yoff * kLetters;
  int16_t* O = cnt + m.ooff * kLetters;
  if (threadIdx.x == 0) basex = basey = 0;
  __syncthreads();
  for (int j0 = 0; j0 < k; j0 += blockDim.x) {
    const int j = j0 + threadIdx.x;
    const unsigned o = j < k ? op[j] : 0u;
    const int ux = (o & 8u) ? 1 : 0, uy = (o & 4u) ? 1 : 0;
    int ix = ux, iy = uy;   // inclusive scans over the block
    for (int d = 1; d < 32; d <<= 1) {
      const int a = __shfl_up_sync(0xffffffffu, ix, d), b = __shfl_up_sync(0xffffffffu, iy, d);
      if ((threadIdx.x & 31) >= d) {
        ix += a;
        iy += b;
      }
    }
    if ((threadIdx.x & 31) == 31) {
      wx[threadIdx.x >> 5] = ix;
      wy[threadIdx.x >> 5] = iy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int ax = 0, ay = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        const int tx = wx[w], ty = wy[w];
        wx[w] = ax;
        wy[w] = ay;
        ax += tx;
        ay += ty;
      }
      wx[32] = ax;
      wy[32] = ay;
    }
    __syncthreads();
    if (j < k) {
      // ops run from the last columns of X and Y (reversed storage) forward
      const int before_x = basex + wx[threadIdx.x >> 5] + ix - ux;
      const int before_y = basey + wy[threadIdx.x >> 5] + iy - uy;
      const int col = k - 1 - j;
      int16_t* out = O + (size_t)col * kLetters;
      const int cxi = m.lx - 1 - before_x, cyi = m.ly - 1 - before_y;
      for (int x = 0; x < kLetters; ++x) {
        const int v = (ux ? X[(size_t)cxi * kLetters + x] : 0) + (uy ? Y[(size_t)cyi * kLetters + x] : 0);
        out[x] = (int16_t)v;
      }
      if (ux) maps[m.xmap + cxi] = col;
      if (uy) maps[m.ymap + cyi] = col;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      basex += wx[32];
      basey += wy[32];
    }
    __syncthreads();
  }
}

// Leaf profiles: one column per residue (reversed codes), count 1.
__global__ void msa_leaf_kernel(const int8_t* __restrict__ codes, int64_t total, int16_t* cnt) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= total) return;
  int16_t* o = cnt + c * kLetters;
  int x = codes[c];
  if (x < 0 || x >= kLetters) x = kLetters - 1;
#pragma unroll
  for (int k = 0; k < kLetters; ++k) o[k] = (int16_t)(k == x);
}

struct PosJob {
  int64_t parent_pos;   // parent's positions (first column)
  int64_t child_pos;    // child's positions (written)
  int64_t child_map;    // child's column -> parent column
  int32_t len;          // child columns
  int32_t pad;
};

// pos[child][c] = pos[parent][map[c]]; one CTA per (parent, child).
__global__ void msa_pos_kernel(const PosJob* __restrict__ jobs, int32_t* pos, const int32_t* __restrict__ maps) {
  const PosJob j = jobs[blockIdx.x];
  for (int c = threadIdx.x; c < j.len; c += blockDim.x) pos[j.child_pos + c] = pos[j.parent_pos + maps[j.child_map + c]];
}

__global__ void msa_root_kernel(int32_t* pos, int64_t root_pos, int len) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < len) pos[root_pos + c] = len - 1 - c;
}

// Rows: out[v][pos[v][c]] = letter of residue c of leaf v (one CTA per leaf).
__global__ void msa_rows_kernel(const int8_t* __restrict__ codes, const int64_t* __restrict__ off,
                                const int32_t* __restrict__ pos, char* out, int64_t L) {
  const int v = blockIdx.x;
  const int64_t a = off[v], b = off[v + 1];
  const char kDec[kLetters + 1] = "ARNDCQEGHILKMFPSTWYVBZX*";
  for (int64_t c = a + threadIdx.x; c < b; c += blockDim.x) {
    int x = codes[c];
    if (x < 0 || x >= kLetters) x = kLetters - 1;
    out[(int64_t)v * L + pos[c]] = kDec[x];
  }
}

}  // namespace

struct MsaState {
  DevBuf codes, off, cnt, maps, pos, nib, ops, scratch, md, pj, out;
  int n = 0;
  int64_t L = 0;
  ~MsaState() {
    for (DevBuf* b : {&codes, &off, &cnt, &maps, &pos, &nib, &ops, &scratch, &md, &pj, &out}) b->release();
  }
};

void Ctx::msa_release() {
  delete reinterpret_cast<MsaState*>(msa_state);
  msa_state = nullptr;
}

int Ctx::msa(const int8_t* codes, const int64_t* offsets, int n, const int32_t* left, const int32_t* right,
             int64_t* msa_len, nwg_stats* st) {
  if (!codes || !offsets || n < 1 || (n > 1 && (!left || !right)) || !msa_len) return fail(NWG_ERR_INVALID, "msa arguments");
  const int nn = 2 * n - 1;
  // the tree: children, heights (levels), each node a child at most once
  std::vector<int> height(nn, 0), used(nn, 0), kseq(nn, 1);
  std::vector<int64_t> len(nn, 0);
  for (int v = 0; v < n; ++v) {
    len[v] = offsets[v + 1] - offsets[v];
    if (len[v] <= 0) return fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
  }
  int levels = 0;
  for (int k = 0; k < n - 1; ++k) {
    const int a = left[k], b = right[k], v = n + k;
    if (a < 0 || b < 0 || a >= b || b >= v || used[a] || used[b]) return fail(NWG_ERR_INVALID, "malformed guide tree");
    used[a] = used[b] = 1;
    height[v] = 1 + std::max(height[a], height[b]);
    kseq[v] = kseq[a] + kseq[b];
    levels = std::max(levels, height[v]);
  }
  if (!msa_state) msa_state = new MsaState();
  MsaState& M = *reinterpret_cast<MsaState*>(msa_state);
  const int64_t total = offsets[n] - offsets[0];
  std::vector<int64_t> off0(n + 1);
  for (int v = 0; v <= n; ++v) off0[v] = offsets[v] - offsets[0];
  cudaStream_t s = stream;
  int rc;
  // column pool: leaves first (their columns = residues), internal nodes appended per level
  std::vector<int64_t> col(nn, -1);
  for (int v = 0; v < n; ++v) col[v] = off0[v];
  int64_t pool = total;
  if ((rc = M.codes.ensure((size_t)std::max<int64_t>(total, 1))) || (rc = M.off.ensure(sizeof(int64_t) * (n + 1))))
    return fail(rc, "msa allocation");
  if ((rc = cuda(cudaMemcpyAsync(M.codes.p, codes + offsets[0], (size_t)total, cudaMemcpyHostToDevice, s), "msa upload")) ||
      (rc = cuda(cudaMemcpyAsync(M.off.p, off0.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s),
                 "msa upload")))
    return rc;
  // worst-case pool: every internal node at most the sum of its leaves' lengths
  std::vector<int64_t> leafsum(nn, 0);
  for (int v = 0; v < n; ++v) leafsum[v] = len[v];
  int64_t cap = total;
  for (int k = 0; k < n - 1; ++k) {
    leafsum[n + k] = leafsum[left[k]] + leafsum[right[k]];
    cap += leafsum[n + k];
  }
  if ((rc = M.cnt.ensure(sizeof(int16_t) * kLetters * (size_t)std::max<int64_t>(cap, 1))) ||
      (rc = M.maps.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(cap, 1))) ||
      (rc = M.pos.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(cap, 1))))
    return fail(rc, "msa allocation");
  if (st) cudaEventRecord(ev0, s);
  msa_leaf_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>((const int8_t*)M.codes.p, total, (int16_t*)M.cnt.p);
  ++launches;
  std::vector<std::vector<int>> bylevel(levels + 1);
  for (int k = 0; k < n - 1; ++k) bylevel[height[n + k]].push_back(n + k);
  int64_t cells = 0;
  int64_t smax = 1;   // largest |S| of the context's matrix
  for (int k = 0; k < kLetters * kLetters; ++k) smax = std::max<int64_t>(smax, sub[k] < 0 ? -sub[k] : sub[k]);
  std::vector<MergeDesc> md;
  for (int l = 1; l <= levels; ++l) {
    const std::vector<int>& nodes = bylevel[l];
    const int nm = (int)nodes.size();
    md.assign(nm, MergeDesc{});
    int64_t nib_total = 0, ops_total = 0, scr_total = 0;
    for (int q = 0; q < nm; ++q) {
      const int v = nodes[q], a = left[v - n], b = right[v - n];
      MergeDesc& d = md[q];
      d.xoff = col[a];
      d.yoff = col[b];
      d.lx = (int)len[a];
      d.ly = (int)len[b];
      d.kx = kseq[a];
      d.ky = kseq[b];
      d.mac32 = (int64_t)d.kx * d.ky * smax < ((int64_t)1 << 31) ? 1 : 0;
      d.xmap = col[a];
      d.ymap = col[b];
      d.ooff = pool;
      col[v] = pool;
      pool += len[a] + len[b];   // capacity; the walk's length is read back below
      const int nstr = (d.ly + kMR - 1) / kMR;
      d.nib = nib_total;
      nib_total += (int64_t)nstr * (d.lx + kMR - 1) * kMR;
      d.ops = ops_total;
      ops_total += d.lx + d.ly;
      d.scratch = scr_total;
      scr_total += d.lx;
      cells += (int64_t)d.lx * d.ly;
    }
    if ((rc = M.nib.ensure((size_t)std::max<int64_t>(nib_total, 1))) ||
        (rc = M.ops.ensure((size_t)std::max<int64_t>(ops_total, 1))) ||
        (rc = M.scratch.ensure(sizeof(longlong2) * (size_t)std::max<int64_t>(scr_total, 1))) ||
        (rc = M.md.ensure(sizeof(MergeDesc) * nm)))
      return fail(rc, "msa allocation");
    if ((rc = cuda(cudaMemcpyAsync(M.md.p, md.data(), sizeof(MergeDesc) * nm, cudaMemcpyHostToDevice, s), "msa upload")))
      return rc;
    msa_dp_kernel<<<nm, kMR, 0, s>>>((MergeDesc*)M.md.p, (const int16_t*)M.cnt.p, (uint8_t*)M.nib.p,
                                     (longlong2*)M.scratch.p, (const int8_t*)b_sub.p, go, ge, (uint8_t*)M.ops.p);
    msa_build_kernel<<<nm, 1024, 0, s>>>((const MergeDesc*)M.md.p, (int16_t*)M.cnt.p, (int32_t*)M.maps.p,
                                        (const uint8_t*)M.ops.p);
    launches += 2;
    if ((rc = cuda(cudaGetLastError(), "msa launch"))) return rc;
    // the new profiles' lengths (the next level sizes its work with them)
    if ((rc = cuda(cudaMemcpyAsync(md.data(), M.md.p, sizeof(MergeDesc) * nm, cudaMemcpyDeviceToHost, s), "msa")) ||
        (rc = cuda(cudaStreamSynchronize(s), "msa sync")))
      return rc;
    for (int q = 0; q < nm; ++q) len[nodes[q]] = md[q].nops;
  }
  // final positions, parents first, then the rows
  const int root = nn - 1;
  const int64_t L = len[root];
  std::vector<PosJob> pj;
  if ((rc = cuda(cudaMemsetAsync(M.pos.p, 0, sizeof(int32_t) * (size_t)std::max<int64_t>(pool, 1), s), "msa"))) return rc;
  msa_root_kernel<<<(unsigned)((L + 255) / 256), 256, 0, s>>>((int32_t*)M.pos.p, col[root], (int)L);
  ++launches;
  if ((rc = M.pj.ensure(sizeof(PosJob) * (size_t)std::max(2 * n, 2)))) return fail(rc, "msa allocation");
  for (int l = levels; l >= 1; --l) {
    pj.clear();
    for (int v : bylevel[l]) {
      const int a = left[v - n], b = right[v - n];
      pj.push_back(PosJob{col[v], col[a], col[a], (int32_t)len[a], 0});
      pj.push_back(PosJob{col[v], col[b], col[b], (int32_t)len[b], 0});
    }
    if ((rc = cuda(cudaMemcpyAsync(M.pj.p, pj.data(), sizeof(PosJob) * pj.size(), cudaMemcpyHostToDevice, s), "msa")))
      return rc;
    msa_pos_kernel<<<(unsigned)pj.size(), 256, 0, s>>>((const PosJob*)M.pj.p, (int32_t*)M.pos.p,
                                                      (const int32_t*)M.maps.p);
    ++launches;
    // the job list is reused by the next level: wait for this launch
    if ((rc = cuda(cudaStreamSynchronize(s), "msa sync"))) return rc;
  }
  if ((rc = M.out.ensure((size_t)std::max<int64_t>((int64_t)n * L, 1)))) return fail(rc, "msa allocation");
  if ((rc = cuda(cudaMemsetAsync(M.out.p, '-', (size_t)n * L, s), "msa"))) return rc;
  msa_rows_kernel<<<n, 256, 0, s>>>((const int8_t*)M.codes.p, (const int64_t*)M.off.p, (const int32_t*)M.pos.p,
                                    (char*)M.out.p, L);
  ++launches;
  if (st) cudaEventRecord(ev1, s);
  if ((rc = cuda(cudaStreamSynchronize(s), "msa sync"))) return rc;
  M.n = n;
  M.L = L;
  *msa_len = L;
  if (st) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    st->kernel_ms = ms;
    st->cells = cells;
    st->pairs = n - 1;
  }
  return NWG_OK;
}

int Ctx::msa_rows(char* out, int64_t stride) {
  MsaState* M = reinterpret_cast<MsaState*>(msa_state);
  if (!M || !M->n || !out || stride < M->L) return fail(NWG_ERR_INVALID, "msa rows");
  int rc;
  if ((rc = cuda(cudaMemcpy2DAsync(out, (size_t)stride, M->out.p, (size_t)M->L, (size_t)M->L, (size_t)M->n,
                                   cudaMemcpyDeviceToHost, stream),
                 "msa download")) ||
      (rc = cuda(cudaStreamSynchronize(stream), "msa sync")))
    return rc;
  return NWG_OK;
}

}  // namespace nwg

using nwg::Ctx;

extern "C" {

int nwg_msa(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n, const int32_t* left,
            const int32_t* right, int64_t* msa_len, nwg_stats* stats) {
  if (!ctx) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  c->launches = 0;
  const int rc = c->msa(codes, offsets, n, left, right, msa_len, stats);
  if (stats) stats->launches = c->launches;
  return rc;
}

int nwg_msa_rows(nwg_ctx* ctx, char* out, int64_t row_stride) {
  if (!ctx) return NWG_ERR_INVALID;
  return reinterpret_cast<Ctx*>(ctx)->msa_rows(out, row_stride);
}

}  // extern "C"
