// nwg_internal.h -- shared declarations of libnwgpu (not installed).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/nwgpu.h"

namespace nwg {

constexpr int kLetters = 24;              // alphabet of AlignmentScore.cu:10-27
constexpr int kShortMin = -32768;         // SHORT_MIN of NeedlemanWunsch.cu:12
constexpr int kWaveWarps = 8;             // warps per CTA of the wavefront kernels
constexpr int kWaveThreads = 32 * kWaveWarps;
constexpr int kPlainThreads = 128;
constexpr int kPlainRows = 16;            // rows per thread strip in the plain kernel
// Overflow guard of the int16x2 lanes (offset binary, halves in [4, 65524]),
// per context from (go, ge, matrix) by int16_limits():
//  * lower side: with w = max(ge, -min entry, 1), every H of a pair is
//    >= -(D+2)*w, D = max(Lx, rows) and rows including the band padding
//    (< 32*32 rows): H[-1][c] = -ge(c+1), and each diagonal step loses at most
//    w.  Every other value (E, F, H - go, diag + S, E - ge inside the DPX max)
//    is within go + ge + |min entry| below that, so sequences up to the
//    context's max_len (at most kInt16MaxLen) keep values >= -32764;
//  * upper side: every H of a pair is <= min(bound_x, bound_y), bound = sum of
//    the residues' best matrix scores (floored at 0); H <= max_h keeps
//    diag + S <= 32756.  A pair whose shorter sequence has <= max_h / (best
//    entry) residues is always inside; longer pairs run on int16 lanes
//    optimistically, are checked against the device-side bounds and re-run on
//    int32 lanes when the check fails.
constexpr int kInt16MaxLen = 6900;
struct Int16Limits {
  int max_len;   // longest sequence of a set that may use int16 lanes (0: none)
  int max_h;     // largest H an int16 pair may reach
};
inline Int16Limits int16_limits(int go, int ge, const int8_t* sub) {
  int smin = 127, smax = -128;
  for (int k = 0; k < kLetters * kLetters; ++k) {
    smin = sub[k] < smin ? sub[k] : smin;
    smax = sub[k] > smax ? sub[k] : smax;
  }
  int w = ge > -smin ? ge : -smin;
  w = w > 1 ? w : 1;
  const int slack = go + ge + (smin < 0 ? -smin : 0);
  int len = (32764 - slack) / w - 2 - 32 * 32;
  len = len < 0 ? 0 : (len > kInt16MaxLen ? kInt16MaxLen : len);
  return {len, 32756 - (smax > 0 ? smax : 0)};
}

// Sequence set laid out on the device for one call: sorted by length
// (descending), each start 16-byte aligned.
struct DevSet {
  int n = 0;
  std::vector<int32_t> h_len;     // sorted lengths
  std::vector<int32_t> h_orig;    // sorted -> original index
  std::vector<int64_t> h_start;   // sorted -> start in d_codes
  std::vector<int32_t> h_bound;   // sorted -> H upper bound
  int8_t* d_codes = nullptr;      // aligned, packed codes (owned by ctx arena)
  int64_t* d_start = nullptr;
  int32_t* d_len = nullptr;
  int32_t* d_orig = nullptr;
  int64_t bytes = 0;
};

struct WaveArgs {
  const int8_t* codes;
  const int8_t* codes_end;    // one past the last byte of the codes buffer (staging never reads past it)
  const int64_t* xstart;
  const int32_t* xlen;
  const int32_t* xorig;
  const int64_t* ystart;
  const int32_t* ylen;
  const int32_t* yorig;
  const int32_t* group_y;     // per Y group: first Y (sorted index)
  const int32_t* group_y2;    // per Y group: second Y for int16x2 lanes, or -1
  const int32_t* group_x;     // per Y group: number of X rows (triangle: up to the group's last Y)
  const int64_t* job_prefix;  // per Y group of this bucket: first CTA job; ngroups+1 entries
  // several alignment jobs in one launch (serving): per Y group, the first X
  // (sorted index) of its job, the offset of its job's matrix in D and that
  // matrix's leading dimension; null for a single set
  const int32_t* group_xbase;
  const int64_t* group_dofs;
  const int32_t* group_ld;
  unsigned long long* counter;
  float* D;
  int32_t* scratch;           // per warp: 2 buffers x 2 words x scratch_cols
  int64_t ld;
  int64_t col0;
  int64_t njobs;
  int nx, ny;
  int g_begin, ngroups;
  int triangle;
  int go, ge;
  int scratch_cols;
  const int8_t* sub;          // 24*24 on device, 4-byte aligned (staged by cp.async)
  // overflow guard (optimistic int16 buckets)
  int check_bound;
  int max_h;                  // the context's int16 upper limit of H (checked groups)
  const int32_t* xbound;      // per sorted X: composition bound
  const int32_t* ybound;
  int2* rerun;                // (sorted x, sorted y) pairs to re-run on int32 lanes
  unsigned long long* rerun_count;
  int64_t rerun_cap;
};

struct PlainArgs {
  const int8_t* codes;
  const int64_t* xstart;
  const int32_t* xlen;
  const int32_t* xorig;
  const int64_t* ystart;
  const int32_t* ylen;
  const int32_t* yorig;
  const int64_t* y_prefix;    // per Y in this launch: first thread; ny_launch+1 entries
  int2* scratch;              // [column][thread]
  float* D;
  int64_t ld;
  int64_t col0;
  int64_t nthreads;
  int y_begin, ny_launch;
  int triangle;
  int go, ge;
  const int8_t* sub;
};

struct PairListArgs {
  const int8_t* codes;
  const int64_t* start;
  const int32_t* len;
  const int32_t* pi;
  const int32_t* pj;
  int32_t* out;
  int2* scratch;              // [column][thread]
  int64_t npairs;
  int64_t base;               // first pair of this launch
  int go, ge;
  const int8_t* sub;
};

// Launchers (score_kernels.cu, wave_r*.cu).  R is the rows per lane; P = 2
// for int16x2 lanes (two pairs per warp), 1 for int32 lanes.
// V: register layout of the wave kernel (0: H, H-go, E per row; 1: H, E per
// row with a min-blocks launch bound).
// wave kernel <R rows per lane, P pairs per word, V layout, W lanes per front>
cudaError_t launch_wave(int R, int P, int V, int W, const WaveArgs& a, int grid, cudaStream_t s);
int wave_max_ctas_per_sm(int R, int P, int V, int W);
void prepare_wave(int R, int P, int V, int W);   // sets the dynamic shared memory limit (outside graph capture)
bool wave_exists(int R, int P, int V, int W);
inline int wave_x_per_front(int V) { return V == 5 ? 2 : 1; }
cudaError_t launch_plain(const PlainArgs& a, cudaStream_t s);
cudaError_t launch_rerun(const WaveArgs& a, int2* scratch, int64_t nthreads, cudaStream_t s);
// neighbor joining of many jobs in one launch, one thread-block cluster per job (nj.cu)
// Row stride (floats) of a neighbor-joining matrix on the device: rows padded
// to a multiple of 4 floats for 16-byte loads.
inline int nj_row_stride(int n) { return (n + 3) & ~3; }
size_t nj_job_workspace(int n);
void nj_job_setup(void* job_out, float* D, int n, int ld, char* base, nwg_join** joins, unsigned long long** stats);
size_t nj_job_desc_bytes();
// residue encoding + reversal on the device (ingest.cu): sequence s of src at
// src_off[s] (len[s] bytes) -> dst at dst_off[s]; bad[s] = bytes outside the alphabet
cudaError_t launch_encode(const char* d_src, const int64_t* d_src_off, const int64_t* d_dst_off, const int32_t* d_len,
                          int n, int8_t* d_dst, int* d_bad, cudaStream_t s);
cudaError_t launch_nj_cluster(const void* d_jobs, int njobs, int C, cudaStream_t s);
// jobs of at most cta_nj_max_n() taxa: the join loop in one CTA's shared memory
int cta_nj_max_n();
cudaError_t launch_nj_cta(const void* d_jobs, int njobs, int nmax, cudaStream_t s);
// jobs of at most smem_nj_max_n() taxa: the join loop in the cluster's shared memory
int smem_nj_cluster(int nmax);
cudaError_t launch_nj_smem(const void* d_jobs, int njobs, int nmax, int C, cudaStream_t s);
int nj_cluster_size();
constexpr int kServeMaxN = 8192;   // largest job of the serving loop (neighbor joining on the device)
cudaError_t launch_dpx_peak(int P, int form, int cols, int grid, uint32_t* sink, int go, int ge, cudaStream_t s);
int dpx_peak_ctas_per_sm(int P, int form);
cudaError_t launch_pairlist(const PairListArgs& a, int64_t count, cudaStream_t s);

}  // namespace nwg
