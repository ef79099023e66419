// nwg_ctx.h -- the context behind the opaque nwg_ctx handle (not installed).
#pragma once

#include <string>
#include <vector>

#include "nwg_internal.h"

namespace nwg {

// Grow-only device buffer owned by a context.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes);
  void release();
};

// One sequence set as the kernels see it: sorted by length (descending).
struct SetView {
  int n = 0;
  int maxlen = 0;
  std::vector<int32_t> len, orig, bound;
  std::vector<int64_t> start;
  const int8_t* d_codes = nullptr;
  const int64_t* d_start = nullptr;
  const int32_t* d_len = nullptr;
  const int32_t* d_orig = nullptr;
};

const int8_t* builtin_matrix();
const char* letter_order();

struct TuneChoice {
  int R;   // rows per lane (4 to 32, even; not a multiple of 4, or 28: layouts 2 to 4 on int16x2 lanes only)
  int V;   // register layout (0 to 6)
  int W;   // lanes per wavefront (32, 16, 8): band of W*R rows; 1: one pair per thread, bands of R rows
};
// Rows a Y of `rows` residues occupies under choice t (whole bands).
inline int padded_rows(const TuneChoice& t, int rows) {
  const int band = t.W * t.R;
  return (rows + band - 1) / band * band;
}
// The same band on full-width fronts, for groups that run on int32 lanes
// (the narrow fronts and the rows per lane that are not multiples of 4 exist
// for int16x2 lanes only).
inline TuneChoice int32_choice(TuneChoice t) {
  if (t.V == 6) t.V = 3;   // the split strips exist for int16x2 lanes only
  if (t.W == 32 && t.R % 4 == 0 && t.R != 28) return t;
  const int band = t.W * t.R;
  int R = 32;
  for (int r : {4, 8, 12, 16, 20, 24, 32})
    if (32 * r >= band) { R = r; break; }
  return {R, t.V == 1 ? 0 : t.V, 32};
}
constexpr int kTuneClasses = NWG_TUNE_CLASSES;
// Upper bound of the Y rows of each class; the last class takes every longer Y.
constexpr int kClassRows[kTuneClasses] = {64,  96,  128, 160, 192, 224, 256,  320,
                                          384, 448, 512, 640, 768, 1024, 1536, 1 << 30};
// Defaults before tuning (the table measured on a GB300): one pair per thread
// (W = 1) for the classes up to 96 rows, wavefronts above, mostly the
// layouts with 1.5 ALU operations per cell (3, and 6 where R is a multiple of 8).
constexpr TuneChoice kDefaultTune[kTuneClasses] = {
    {32, 4, 1},  {32, 4, 1},  {16, 5, 8},  {20, 3, 8},  {24, 6, 8},  {28, 3, 8},  {32, 6, 8},  {20, 3, 16},
    {24, 6, 16}, {28, 3, 16}, {32, 6, 16}, {20, 3, 32}, {24, 6, 16}, {32, 3, 32}, {24, 6, 16}, {32, 3, 32}};
// The best wavefront (W >= 8) per class before tuning, for latency-bound
// callers: one pair per thread needs 256 X per CTA and streams a Y in bands,
// so it wins on throughput over many X but lengthens a small job.
constexpr TuneChoice kDefaultTuneWave[kTuneClasses] = {
    {8, 5, 8},   {12, 0, 8},  {16, 5, 8},  {20, 3, 8},  {24, 6, 8},  {28, 3, 8},  {32, 6, 8},  {20, 3, 16},
    {24, 6, 16}, {28, 3, 16}, {32, 6, 16}, {20, 3, 32}, {24, 6, 16}, {32, 3, 32}, {24, 6, 16}, {32, 3, 32}};
int tune_class(int rows);

struct BatchPlan;
struct Ctx;
void destroy_plans(Ctx* c);

struct Ctx {
  int go = 10, ge = 2;
  int8_t sub[kLetters * kLetters];
  Int16Limits i16{kInt16MaxLen, 32756 - 11};   // set from (go, ge, sub) at creation
  int device = 0, sms = 1;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string last_err;
  int launches = 0;
  // Kernel choice per length class of the Y rows (rows <= kClassRows[k]):
  // rows per lane and register layout, set by the autotuner (tune.cu).
  TuneChoice tune[kTuneClasses];
  // The fastest wavefront (W >= 8) per class, for the serving loop, whose
  // small jobs are latency-bound (one pair per thread lengthens them).
  TuneChoice tune_wave[kTuneClasses];
  // Every candidate the autotuner timed per class, with its rate in computed
  // cells per second (band-padded rows x columns / time).  Empty when the
  // table was set by hand or not tuned: tune[] is then used as it is.
  struct Cand {
    TuneChoice t;
    double rate;
  };
  std::vector<Cand> cands[kTuneClasses];
  // The choice for a Y group of this many rows: the class's candidate with
  // the least estimated time (its padded rows / its rate), the class's
  // fastest at the class bound unless another is estimated 2 % faster.
  // Layout 4 is exact only when go >= ge and falls back to layout 2.
  TuneChoice choice(int rows) const {
    const int k = tune_class(rows);
    TuneChoice t = tune[k], fastest = t;
    double pick_est = 0.0, min_est = 0.0;
    for (const Cand& c : cands[k]) {
      const double est = padded_rows(c.t, rows) / c.rate;
      if (c.t.R == t.R && c.t.V == t.V && c.t.W == t.W) pick_est = est;
      if (min_est == 0.0 || est < min_est) {
        min_est = est;
        fastest = c.t;
      }
    }
    if (pick_est > 0.0 && min_est < 0.98 * pick_est) t = fastest;
    if (t.V == 4 && go < ge) t.V = 2;
    return t;
  }
  TuneChoice choice_wave(int rows) const {
    TuneChoice t = tune_wave[tune_class(rows)];
    if (t.V == 4 && go < ge) t.V = 2;
    return t;
  }
  uint64_t tune_version = 0;        // bumped on every change (part of the plan key)
  bool tuned = false;

  DevBuf b_codes, b_start, b_len, b_orig, b_bound, b_bad;
  DevBuf b_start2, b_len2, b_orig2;
  DevBuf b_gy, b_gy2, b_gx, b_jobs, b_counter, b_wscratch, b_pscratch, b_yprefix;
  DevBuf b_D, b_sub, b_rowmax;
  DevBuf b_pi, b_pj, b_out;
  // per-launch event timing (nwg_set_launch_timing)
  bool launch_timing = false;
  std::vector<nwg_launch_rec> recs;
  std::vector<cudaEvent_t> evpool;
  int rec_begin(const nwg_launch_rec& r);   // records the start event; returns record index
  int rec_end(int idx);
  int rec_finalize();
  // batched-form plans (batched.cu): [0] all-pairs triangle, [1] block
  BatchPlan* plans[2] = {nullptr, nullptr};
  bool use_graphs = true;
  std::vector<cudaStream_t> branch;     // parallel branches for bucket launches
  cudaEvent_t fork_ev = nullptr;
  std::vector<cudaEvent_t> join_ev;
  int autotune(bool force, nwg_tune_result* out);
  bool tune_from_cache(nwg_tune_result* res);
  int batched(const int8_t* d_codes, const int64_t* xoff, int nx, const int64_t* yoff, int ny, bool triangle,
              float* d_D, int64_t ld, int64_t col0, int mode, nwg_stats* st);
  // traceback / neighbor joining state (trace.cu, nj.cu)
  void* trace_state = nullptr;
  void* nj_state = nullptr;
  void* ingest_state = nullptr;
  void* msa_state = nullptr;
  void extra_release();
  void nj_release();
  void ingest_release();
  void msa_release();
  int msa(const int8_t* codes, const int64_t* offsets, int n, const int32_t* left, const int32_t* right,
          int64_t* msa_len, nwg_stats* st);
  int msa_rows(char* out, int64_t stride);
  int nj(const float* D, int64_t ld, int n, bool device_D, nwg_join* joins, nwg_nj_stats* st);
  int trace_lanes_forced = 0;   // front width of the traceback kernel (0: chosen per call)
  int align_pairs(const int8_t* codes, const int64_t* offsets, int n, const int32_t* px, const int32_t* py,
                  int npairs, char* outx, char* outy, int64_t stride, int32_t* outlen, int32_t* score,
                  nwg_stats* st);

  ~Ctx();
  int fail(int status, const char* what, cudaError_t e = cudaSuccess);
  int cuda(cudaError_t e, const char* what);
  int prepare_set(const int8_t* d_codes, const int64_t* offsets, int n, SetView& v, DevBuf& bstart,
                  DevBuf& blen, DevBuf& borig, bool want_bounds);
  int run_plain(const SetView& X, const SetView& Y, bool triangle, float* d_D, int64_t ld,
                int64_t col0, nwg_stats* st);
  int score_all_dev(const int8_t* d_codes, const int64_t* offsets, int n, float* d_D, int64_t ld,
                    int mode, nwg_stats* st);
};

}  // namespace nwg
