// api.cu -- C ABI of libnwgpu: contexts, sequence sets, length-bucket plans
// and the scoring entry points (include/nwgpu.h).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "nwg_ctx.h"
#include "nwg_matrix.h"

namespace nwg {

// Residue order of the reference (AlignmentScore.cu:10-27): code k is kOrder[k].
static const char kOrder[kLetters + 1] = "ARNDCQEGHILKMFPSTWYVBZX*";

// blosum64.txt (== definitions.cuh:96-121; BLOSUM62 values) in kOrder.
static const int8_t kBlosum[kLetters * kLetters] = {NWG_BLOSUM64_VALUES};

const int8_t* builtin_matrix() { return kBlosum; }
const char* letter_order() { return kOrder; }

namespace {

double now_ms() {
  using clk = std::chrono::steady_clock;
  return std::chrono::duration<double, std::milli>(clk::now().time_since_epoch()).count();
}

}  // namespace

// ---- context ---------------------------------------------------------------

Ctx::~Ctx() {
  destroy_plans(this);
  for (cudaStream_t b : branch) cudaStreamDestroy(b);
  for (cudaEvent_t e : join_ev) cudaEventDestroy(e);
  if (fork_ev) cudaEventDestroy(fork_ev);
  for (DevBuf* b : {&b_codes, &b_start, &b_len, &b_orig, &b_bound, &b_bad, &b_start2, &b_len2,
                    &b_orig2, &b_gy, &b_gy2, &b_gx, &b_jobs, &b_counter, &b_wscratch, &b_pscratch,
                    &b_yprefix, &b_D, &b_sub, &b_rowmax, &b_pi, &b_pj, &b_out})
    b->release();
  extra_release();
  for (cudaEvent_t e : evpool) cudaEventDestroy(e);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (own_stream) cudaStreamDestroy(own_stream);
}

int Ctx::fail(int status, const char* what, cudaError_t e) {
  last_err = what;
  if (e != cudaSuccess) {
    last_err += ": ";
    last_err += cudaGetErrorString(e);
  }
  return status;
}

int Ctx::cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return NWG_OK;
  return fail(e == cudaErrorMemoryAllocation ? NWG_ERR_OOM : NWG_ERR_CUDA, what, e);
}

int DevBuf::ensure(size_t bytes) {
  if (bytes <= cap) return NWG_OK;
  release();
  size_t want = bytes < 256 ? 256 : bytes;
  if (cudaMalloc(&p, want) != cudaSuccess) {
    p = nullptr;
    cap = 0;
    cudaGetLastError();
    return NWG_ERR_OOM;
  }
  cap = want;
  return NWG_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}

// Sorted, bounded view of one sequence set.  lengths come from the host
// offsets; codes are already on the device at d_codes + offsets[i].
int Ctx::prepare_set(const int8_t* d_codes, const int64_t* offsets, int n, SetView& v,
                     DevBuf& bstart, DevBuf& blen, DevBuf& borig, bool want_bounds) {
  v.n = n;
  v.len.resize(n);
  v.orig.resize(n);
  v.start.resize(n);
  for (int i = 0; i < n; ++i) {
    const int64_t L = offsets[i + 1] - offsets[i];
    if (L <= 0) return fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
    if (L > (int64_t)0x7fffffff) return fail(NWG_ERR_INVALID, "sequence too long");
  }
  std::iota(v.orig.begin(), v.orig.end(), 0);
  std::stable_sort(v.orig.begin(), v.orig.end(), [&](int a, int b) {
    return offsets[a + 1] - offsets[a] > offsets[b + 1] - offsets[b];
  });
  v.maxlen = 0;
  for (int k = 0; k < n; ++k) {
    const int o = v.orig[k];
    v.len[k] = (int32_t)(offsets[o + 1] - offsets[o]);
    v.start[k] = offsets[o];
    v.maxlen = std::max(v.maxlen, v.len[k]);
  }
  int rc;
  if ((rc = bstart.ensure(sizeof(int64_t) * n)) || (rc = blen.ensure(sizeof(int32_t) * n)) ||
      (rc = borig.ensure(sizeof(int32_t) * n)))
    return fail(rc, "set allocation");
  if ((rc = cuda(cudaMemcpyAsync(bstart.p, v.start.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, stream), "set upload")) ||
      (rc = cuda(cudaMemcpyAsync(blen.p, v.len.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream), "set upload")) ||
      (rc = cuda(cudaMemcpyAsync(borig.p, v.orig.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream), "set upload")))
    return rc;
  v.d_codes = d_codes;
  v.d_start = (int64_t*)bstart.p;
  v.d_len = (int32_t*)blen.p;
  v.d_orig = (int32_t*)borig.p;
  v.bound.assign(n, 0);
  (void)want_bounds;
  return NWG_OK;
}

int tune_class(int rows) {
  for (int k = 0; k < kTuneClasses; ++k)
    if (rows <= kClassRows[k]) return k;
  return kTuneClasses - 1;
}

// Build and launch the batched (wavefront) plan for X rows against Y groups.
int Ctx::run_plain(const SetView& X, const SetView& Y, bool triangle, float* d_D, int64_t ld,
                   int64_t col0, nwg_stats* st) {
  // one launch per group of consecutive (similar-length) Ys, <= kMaxThreads pairs each
  const int64_t kMaxThreads = (int64_t)sms * 512;
  int rc;
  PlainArgs a{};
  a.codes = X.d_codes;
  a.xstart = X.d_start; a.xlen = X.d_len; a.xorig = X.d_orig;
  a.ystart = Y.d_start; a.ylen = Y.d_len; a.yorig = Y.d_orig;
  a.scratch = (int2*)b_pscratch.p;
  a.D = d_D; a.ld = ld; a.col0 = col0;
  a.triangle = triangle ? 1 : 0;
  a.go = go; a.ge = ge;
  a.sub = (const int8_t*)b_sub.p;
  // all launches' prefixes go to one upload
  std::vector<int64_t> pre;
  struct L { int y0, ny; int64_t off, threads; };
  std::vector<L> ls;
  for (int y = 0; y < Y.n;) {
    L l{y, 0, (int64_t)pre.size(), 0};
    while (y < Y.n) {
      const int64_t nx = triangle ? y + 1 : X.n;
      if (l.ny > 0 && l.threads + nx > kMaxThreads) break;
      pre.push_back(l.threads);
      l.threads += nx;
      ++l.ny;
      ++y;
    }
    pre.push_back(l.threads);
    ls.push_back(l);
  }
  int64_t tmax = 0;
  for (const L& l : ls) tmax = std::max(tmax, l.threads);
  if ((rc = b_pscratch.ensure(sizeof(int2) * (size_t)tmax * (size_t)std::max(X.maxlen, 1))))
    return fail(rc, "plain scratch");
  a.scratch = (int2*)b_pscratch.p;
  if ((rc = b_yprefix.ensure(sizeof(int64_t) * pre.size()))) return fail(rc, "plain plan");
  if ((rc = cuda(cudaMemcpyAsync(b_yprefix.p, pre.data(), sizeof(int64_t) * pre.size(), cudaMemcpyHostToDevice, stream), "plain plan")))
    return rc;
  std::vector<double> sx((size_t)X.n + 1, 0.0);
  for (int i = 0; i < X.n; ++i) sx[i + 1] = sx[i] + X.len[i];
  for (const L& l : ls) {
    a.y_begin = l.y0;
    a.ny_launch = l.ny;
    a.y_prefix = (const int64_t*)b_yprefix.p + l.off;
    a.nthreads = l.threads;
    int ri = -1;
    if (launch_timing) {
      nwg_launch_rec r{1, 0, 0, (int32_t)((l.threads + kPlainThreads - 1) / kPlainThreads), 0, 0, 0.0};
      double cells = 0;
      for (int y = l.y0; y < l.y0 + l.ny; ++y) {
        const int cnt = triangle ? y : X.n;
        r.pairs += cnt;
        cells += (double)Y.len[y] * sx[cnt];
      }
      r.cells = (int64_t)cells;
      if ((ri = rec_begin(r)) < 0) return fail(NWG_ERR_CUDA, "launch timing");
    }
    if ((rc = cuda(launch_plain(a, stream), "plain launch"))) return rc;
    if (ri >= 0 && (rc = rec_end(ri))) return rc;
    ++launches;
  }
  if (st) st->pairs_int32 += triangle ? (int64_t)Y.n * (Y.n + 1) / 2 : (int64_t)X.n * Y.n;
  return NWG_OK;
}

int Ctx::rec_begin(const nwg_launch_rec& r) {
  const size_t k = recs.size();
  while (evpool.size() < 2 * (k + 1)) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    evpool.push_back(e);
  }
  recs.push_back(r);
  if (cudaEventRecord(evpool[2 * k], stream) != cudaSuccess) return -1;
  return (int)k;
}

int Ctx::rec_end(int idx) {
  return cuda(cudaEventRecord(evpool[2 * (size_t)idx + 1], stream), "launch timing");
}

int Ctx::rec_finalize() {
  for (size_t k = 0; k < recs.size(); ++k) {
    if (recs[k].ms > 0) continue;
    int rc;
    if ((rc = cuda(cudaEventSynchronize(evpool[2 * k + 1]), "launch timing"))) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, evpool[2 * k], evpool[2 * k + 1]);
    recs[k].ms = ms;
  }
  return NWG_OK;
}

int Ctx::score_all_dev(const int8_t* d_codes, const int64_t* offsets, int n, float* d_D, int64_t ld,
                       int mode, nwg_stats* st) {
  if (n < 1 || !offsets || !d_codes || !d_D || ld < n) return fail(NWG_ERR_INVALID, "score_all arguments");
  if (mode < 0 || mode > 2) return fail(NWG_ERR_INVALID, "mode");
  int rc;
  if (st) {
    double L = 0, L2 = 0;
    for (int i = 0; i < n; ++i) {
      const double l = (double)(offsets[i + 1] - offsets[i]);
      L += l;
      L2 += l * l;
    }
    st->cells += (int64_t)((L * L - L2) / 2);
    st->pairs += (int64_t)n * (n + 1) / 2;
  }
  if (mode == NWG_MODE_PLAIN) {
    SetView S;
    if ((rc = prepare_set(d_codes, offsets, n, S, b_start, b_len, b_orig, false))) return rc;
    if (st && (rc = cuda(cudaEventRecord(ev0, stream), "event"))) return rc;
    if ((rc = run_plain(S, S, true, d_D, ld, 0, st))) return rc;
  } else {
    if (st && (rc = cuda(cudaEventRecord(ev0, stream), "event"))) return rc;
    if ((rc = batched(d_codes, offsets, n, offsets, n, true, d_D, ld, 0, mode, st))) return rc;
  }
  if (st) {
    if ((rc = cuda(cudaEventRecord(ev1, stream), "event")) ||
        (rc = cuda(cudaEventSynchronize(ev1), "kernel sync")))
      return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    st->kernel_ms += ms;
  }
  return NWG_OK;
}

}  // namespace nwg

using nwg::Ctx;

// ---- C ABI -----------------------------------------------------------------

extern "C" {

const char* nwg_status_str(int s) {
  switch (s) {
    case NWG_OK: return "ok";
    case NWG_ERR_NO_DEVICE: return "no CUDA device";
    case NWG_ERR_OOM: return "device out of memory";
    case NWG_ERR_BAD_RESIDUE: return "residue outside the 24-letter alphabet";
    case NWG_ERR_TIMEOUT: return "bounded device wait timed out";
    case NWG_ERR_OVERFLOW: return "score overflow";
    case NWG_ERR_INVALID: return "invalid argument";
    case NWG_ERR_CUDA: return "CUDA runtime error";
    case NWG_ERR_EMPTY_SEQ: return "zero-length sequence";
    case NWG_ERR_NJ_AMBIGUOUS: return "neighbor-joining step ambiguous under the reference's rounding";
    default: return "unknown status";
  }
}

int nwg_ctx_create(int gap_open, int gap_ext, const int8_t* sub, nwg_ctx** out) {
  if (!out) return NWG_ERR_INVALID;
  *out = nullptr;
  if (gap_open < 0 || gap_ext < 0 || gap_open > 1000 || gap_ext > 1000) return NWG_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return NWG_ERR_NO_DEVICE;
  }
  Ctx* c = new Ctx();
  c->go = gap_open;
  c->ge = gap_ext;
  std::memcpy(c->sub, sub ? sub : nwg::kBlosum, sizeof(c->sub));
  c->i16 = nwg::int16_limits(c->go, c->ge, c->sub);
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
  int rc;
  if ((rc = c->cuda(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking), "stream")) ||
      (rc = c->cuda(cudaEventCreate(&c->ev0), "event")) || (rc = c->cuda(cudaEventCreate(&c->ev1), "event"))) {
    delete c;
    return rc;
  }
  c->stream = c->own_stream;
  for (int k = 0; k < nwg::kTuneClasses; ++k) {
    c->tune[k] = nwg::kDefaultTune[k];
    c->tune_wave[k] = nwg::kDefaultTuneWave[k];
  }
  for (int k = 0; k < 2; ++k) {
    cudaStream_t b;
    cudaEvent_t e;
    if ((rc = c->cuda(cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking), "stream")) ||
        (rc = c->cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event"))) {
      delete c;
      return rc;
    }
    c->branch.push_back(b);
    c->join_ev.push_back(e);
  }
  if ((rc = c->cuda(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming), "event"))) {
    delete c;
    return rc;
  }
  int8_t rowmax[nwg::kLetters];
  for (int a = 0; a < nwg::kLetters; ++a) {
    int m = -128;
    for (int b = 0; b < nwg::kLetters; ++b) m = std::max<int>(m, c->sub[a * nwg::kLetters + b]);
    rowmax[a] = (int8_t)std::max(m, 0);
  }
  if ((rc = c->b_sub.ensure(sizeof(c->sub))) || (rc = c->b_rowmax.ensure(sizeof(rowmax)))) {
    delete c;
    return rc;
  }
  cudaMemcpy(c->b_sub.p, c->sub, sizeof(c->sub), cudaMemcpyHostToDevice);
  cudaMemcpy(c->b_rowmax.p, rowmax, sizeof(rowmax), cudaMemcpyHostToDevice);
  *out = reinterpret_cast<nwg_ctx*>(c);
  return NWG_OK;
}

int nwg_ctx_destroy(nwg_ctx* ctx) {
  if (!ctx) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  cudaStreamSynchronize(c->stream);
  delete c;
  return NWG_OK;
}

int nwg_set_stream(nwg_ctx* ctx, void* stream) {
  if (!ctx) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return NWG_OK;
}

const char* nwg_last_error(const nwg_ctx* ctx) {
  return ctx ? reinterpret_cast<const Ctx*>(ctx)->last_err.c_str() : "null context";
}

int nwg_encode(const char* ascii, const int64_t* offsets, int n, int8_t* codes) {
  if (!ascii || !offsets || !codes || n < 0) return NWG_ERR_INVALID;
  int8_t tab[256];
  for (int k = 0; k < 256; ++k) tab[k] = -1;
  for (int k = 0; k < nwg::kLetters; ++k) tab[(unsigned char)nwg::kOrder[k]] = (int8_t)k;
  int bad = 0;
  for (int s = 0; s < n; ++s) {
    const int64_t a = offsets[s], b = offsets[s + 1];
    if (b <= a) return NWG_ERR_EMPTY_SEQ;
    // encode and reverse (AlignmentScore.cu:168-177, every residue encoded)
    for (int64_t k = a; k < b; ++k) {
      const int8_t c = tab[(unsigned char)ascii[b - 1 - (k - a)]];
      bad += c < 0;
      codes[k] = c;
    }
  }
  return bad ? NWG_ERR_BAD_RESIDUE : NWG_OK;
}

int nwg_parse_wire(const char* wire, int n, int8_t* codes, int64_t* offsets) {
  // SpeciesBlock.cpp:309-322 layout, walked as AlignmentScore.cu:149-166 does
  if (!wire || !offsets || n < 0) return NWG_ERR_INVALID;
  const char* p = wire + sizeof(int);
  offsets[0] = 0;
  std::vector<const char*> src(n);
  for (int s = 0; s < n; ++s) {
    int len;
    p += sizeof(int);
    std::memcpy(&len, p, sizeof(int));
    p += sizeof(int);
    if (len <= 0) return NWG_ERR_EMPTY_SEQ;
    src[s] = p;
    offsets[s + 1] = offsets[s] + len;
    p += len + 1;
  }
  if (!codes) return NWG_OK;
  int bad = 0;
  int8_t tab[256];
  for (int k = 0; k < 256; ++k) tab[k] = -1;
  for (int k = 0; k < nwg::kLetters; ++k) tab[(unsigned char)nwg::kOrder[k]] = (int8_t)k;
  for (int s = 0; s < n; ++s) {
    const int64_t a = offsets[s], b = offsets[s + 1];
    for (int64_t k = a; k < b; ++k) {
      const int8_t c = tab[(unsigned char)src[s][b - 1 - k]];
      bad += c < 0;
      codes[k] = c;
    }
  }
  return bad ? NWG_ERR_BAD_RESIDUE : NWG_OK;
}

int nwg_score_all_dev(nwg_ctx* ctx, const int8_t* d_codes, const int64_t* offsets, int n, float* d_D,
                      int64_t ld, int mode, nwg_stats* stats) {
  if (!ctx) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  const double t0 = nwg::now_ms();
  if (stats) std::memset(stats, 0, sizeof(*stats));
  c->launches = 0;
  c->recs.clear();
  int rc = c->score_all_dev(d_codes, offsets, n, d_D, ld, mode, stats);
  if (stats) {
    stats->launches = c->launches;
    stats->total_ms = nwg::now_ms() - t0;
  }
  return rc;
}

int nwg_score_all(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n, float* D,
                  int64_t ld, int mode, nwg_stats* stats) {
  if (!ctx || !codes || !offsets || !D || n < 1 || ld < n) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  const double t0 = nwg::now_ms();
  if (stats) std::memset(stats, 0, sizeof(*stats));
  c->launches = 0;
  c->recs.clear();
  const int64_t total = offsets[n];
  int rc;
  for (int s = 0; s < n; ++s)
    if (offsets[s + 1] <= offsets[s]) return c->fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
  for (int64_t k = 0; k < total; ++k)
    if ((unsigned)codes[k] >= (unsigned)nwg::kLetters) return c->fail(NWG_ERR_BAD_RESIDUE, "residue code outside 0..23");
  if ((rc = c->b_codes.ensure((size_t)std::max<int64_t>(total, 1))) ||
      (rc = c->b_D.ensure(sizeof(float) * (size_t)n * (size_t)n)))
    return c->fail(rc, "score_all allocation");
  double t = nwg::now_ms();
  if ((rc = c->cuda(cudaMemcpyAsync(c->b_codes.p, codes, (size_t)total, cudaMemcpyHostToDevice, c->stream), "codes upload")))
    return rc;
  if (stats) {
    cudaStreamSynchronize(c->stream);
    stats->h2d_ms = nwg::now_ms() - t;
  }
  rc = c->score_all_dev((const int8_t*)c->b_codes.p, offsets, n, (float*)c->b_D.p, n, mode, stats);
  if (rc) return rc;
  t = nwg::now_ms();
  if (ld == n)
    rc = c->cuda(cudaMemcpyAsync(D, c->b_D.p, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToHost, c->stream), "D download");
  else
    rc = c->cuda(cudaMemcpy2DAsync(D, sizeof(float) * ld, c->b_D.p, sizeof(float) * n, sizeof(float) * n, n,
                                   cudaMemcpyDeviceToHost, c->stream), "D download");
  if (rc) return rc;
  if ((rc = c->cuda(cudaStreamSynchronize(c->stream), "score_all sync"))) return rc;
  if (stats) {
    stats->d2h_ms = nwg::now_ms() - t;
    stats->launches = c->launches;
    stats->total_ms = nwg::now_ms() - t0;
  }
  return NWG_OK;
}

int nwg_score_block(nwg_ctx* ctx, const int8_t* xcodes, const int64_t* xoff, int nx,
                    const int8_t* ycodes, const int64_t* yoff, int ny, float* D, int64_t ld,
                    int64_t r0, int mode, nwg_stats* stats) {
  if (!ctx || !xcodes || !xoff || !ycodes || !yoff || !D || nx < 1 || ny < 1 || r0 < 0 || ld < r0 + ny)
    return NWG_ERR_INVALID;
  if (mode < 0 || mode > 2) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  const double t0 = nwg::now_ms();
  if (stats) std::memset(stats, 0, sizeof(*stats));
  c->launches = 0;
  c->recs.clear();
  const int64_t tx = xoff[nx], ty = yoff[ny];
  int rc;
  if ((rc = c->b_codes.ensure((size_t)(tx + ty))) || (rc = c->b_D.ensure(sizeof(float) * (size_t)nx * ny)))
    return c->fail(rc, "score_block allocation");
  int8_t* dc = (int8_t*)c->b_codes.p;
  if ((rc = c->cuda(cudaMemcpyAsync(dc, xcodes, (size_t)tx, cudaMemcpyHostToDevice, c->stream), "upload")) ||
      (rc = c->cuda(cudaMemcpyAsync(dc + tx, ycodes, (size_t)ty, cudaMemcpyHostToDevice, c->stream), "upload")))
    return rc;
  for (int64_t k = 0; k < tx; ++k)
    if ((unsigned)xcodes[k] >= (unsigned)nwg::kLetters) return c->fail(NWG_ERR_BAD_RESIDUE, "residue code");
  for (int64_t k = 0; k < ty; ++k)
    if ((unsigned)ycodes[k] >= (unsigned)nwg::kLetters) return c->fail(NWG_ERR_BAD_RESIDUE, "residue code");
  std::vector<int64_t> yo2(ny + 1);
  for (int k = 0; k <= ny; ++k) yo2[k] = yoff[k] + tx;
  if (stats) {
    double sx = 0, sy = 0;
    for (int k = 0; k < nx; ++k) sx += (double)(xoff[k + 1] - xoff[k]);
    for (int k = 0; k < ny; ++k) sy += (double)(yoff[k + 1] - yoff[k]);
    stats->cells = (int64_t)(sx * sy);
    stats->pairs = (int64_t)nx * ny;
    cudaEventRecord(c->ev0, c->stream);
  }
  // block result in a dense nx x ny device matrix, then one 2D copy into D[:, r0:]
  float* dD = (float*)c->b_D.p;
  if (mode == NWG_MODE_PLAIN) {
    nwg::SetView X, Y;
    if ((rc = c->prepare_set(dc, xoff, nx, X, c->b_start, c->b_len, c->b_orig, false))) return rc;
    if ((rc = c->prepare_set(dc, yo2.data(), ny, Y, c->b_start2, c->b_len2, c->b_orig2, false))) return rc;
    rc = c->run_plain(X, Y, false, dD, ny, 0, stats);
  } else {
    rc = c->batched(dc, xoff, nx, yo2.data(), ny, false, dD, ny, 0, mode, stats);
  }
  if (rc) return rc;
  if (stats) {
    cudaEventRecord(c->ev1, c->stream);
    cudaEventSynchronize(c->ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->kernel_ms = ms;
  }
  if ((rc = c->cuda(cudaMemcpy2DAsync(D + r0, sizeof(float) * ld, dD, sizeof(float) * ny, sizeof(float) * ny, nx,
                                      cudaMemcpyDeviceToHost, c->stream), "block download")) ||
      (rc = c->cuda(cudaStreamSynchronize(c->stream), "block sync")))
    return rc;
  if (stats) {
    stats->launches = c->launches;
    stats->total_ms = nwg::now_ms() - t0;
  }
  return NWG_OK;
}

int nwg_score_pairs(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n, const int32_t* pi,
                    const int32_t* pj, int64_t npairs, int32_t* out, nwg_stats* stats) {
  if (!ctx || !codes || !offsets || !pi || !pj || !out || n < 1 || npairs < 0) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  const double t0 = nwg::now_ms();
  if (stats) std::memset(stats, 0, sizeof(*stats));
  c->launches = 0;
  c->recs.clear();
  for (int64_t k = 0; k < npairs; ++k)
    if (pi[k] < 0 || pi[k] >= n || pj[k] < 0 || pj[k] >= n) return c->fail(NWG_ERR_INVALID, "pair index");
  int maxlen = 0;
  for (int s = 0; s < n; ++s) {
    const int64_t L = offsets[s + 1] - offsets[s];
    if (L <= 0) return c->fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
    maxlen = std::max<int>(maxlen, (int)L);
  }
  if (npairs == 0) return NWG_OK;
  const int64_t total = offsets[n];
  std::vector<int32_t> len(n);
  for (int s = 0; s < n; ++s) len[s] = (int32_t)(offsets[s + 1] - offsets[s]);
  int rc;
  const int64_t kMax = (int64_t)c->sms * 512;
  if ((rc = c->b_codes.ensure((size_t)total)) || (rc = c->b_start.ensure(sizeof(int64_t) * n)) ||
      (rc = c->b_len.ensure(sizeof(int32_t) * n)) || (rc = c->b_pi.ensure(sizeof(int32_t) * npairs)) ||
      (rc = c->b_pj.ensure(sizeof(int32_t) * npairs)) || (rc = c->b_out.ensure(sizeof(int32_t) * npairs)) ||
      (rc = c->b_pscratch.ensure(sizeof(int2) * (size_t)kMax * maxlen)))
    return c->fail(rc, "pair-list allocation");
  cudaStream_t s = c->stream;
  if ((rc = c->cuda(cudaMemcpyAsync(c->b_codes.p, codes, (size_t)total, cudaMemcpyHostToDevice, s), "upload")) ||
      (rc = c->cuda(cudaMemcpyAsync(c->b_start.p, offsets, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s), "upload")) ||
      (rc = c->cuda(cudaMemcpyAsync(c->b_len.p, len.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s), "upload")) ||
      (rc = c->cuda(cudaMemcpyAsync(c->b_pi.p, pi, sizeof(int32_t) * npairs, cudaMemcpyHostToDevice, s), "upload")) ||
      (rc = c->cuda(cudaMemcpyAsync(c->b_pj.p, pj, sizeof(int32_t) * npairs, cudaMemcpyHostToDevice, s), "upload")))
    return rc;
  // validate codes on the host side of the copy
  for (int64_t k = 0; k < total; ++k)
    if ((unsigned)codes[k] >= (unsigned)nwg::kLetters) return c->fail(NWG_ERR_BAD_RESIDUE, "residue code");
  nwg::PairListArgs a{};
  a.codes = (const int8_t*)c->b_codes.p;
  a.start = (const int64_t*)c->b_start.p;
  a.len = (const int32_t*)c->b_len.p;
  a.pi = (const int32_t*)c->b_pi.p;
  a.pj = (const int32_t*)c->b_pj.p;
  a.out = (int32_t*)c->b_out.p;
  a.scratch = (int2*)c->b_pscratch.p;
  a.npairs = npairs;
  a.go = c->go;
  a.ge = c->ge;
  a.sub = (const int8_t*)c->b_sub.p;
  for (int64_t b = 0; b < npairs; b += kMax) {
    a.base = b;
    if ((rc = c->cuda(nwg::launch_pairlist(a, std::min(kMax, npairs - b), s), "pair-list launch"))) return rc;
    ++c->launches;
  }
  if ((rc = c->cuda(cudaMemcpyAsync(out, c->b_out.p, sizeof(int32_t) * npairs, cudaMemcpyDeviceToHost, s), "download")) ||
      (rc = c->cuda(cudaStreamSynchronize(s), "pair-list sync")))
    return rc;
  if (stats) {
    stats->pairs = npairs;
    stats->pairs_int32 = npairs;
    stats->launches = c->launches;
    stats->total_ms = nwg::now_ms() - t0;
  }
  return NWG_OK;
}

int nwg_dpx_peak_form(nwg_ctx* ctx, int lanes16, int form, double* cells_per_s) {
  if (!ctx || !cells_per_s) return NWG_ERR_INVALID;
  if (form != 0 && form != 2 && form != 3 && form != 4 && form != 5) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  const int P = lanes16 ? 2 : 1;
  const int cols = 4096;
  const int grid = c->sms * nwg::dpx_peak_ctas_per_sm(P, form);
  int rc;
  if ((rc = c->b_out.ensure(sizeof(uint32_t) * grid))) return c->fail(rc, "dpx peak");
  for (int rep = 0; rep < 2; ++rep) {      // first launch warms up clocks and caches
    if ((rc = c->cuda(cudaEventRecord(c->ev0, c->stream), "event")) ||
        (rc = c->cuda(nwg::launch_dpx_peak(P, form, cols, grid, (uint32_t*)c->b_out.p, c->go, c->ge, c->stream),
                      "dpx peak")) ||
        (rc = c->cuda(cudaEventRecord(c->ev1, c->stream), "event")) ||
        (rc = c->cuda(cudaEventSynchronize(c->ev1), "dpx peak sync")))
      return rc;
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  const double cells = (double)grid * 256.0 * cols * 16 * P;
  *cells_per_s = cells / (ms * 1e-3);
  return NWG_OK;
}

int nwg_dpx_peak(nwg_ctx* ctx, int lanes16, double* cells_per_s) {
  if (!ctx || !cells_per_s) return NWG_ERR_INVALID;
  double best = 0.0;
  for (int form : {0, 2, 3, 4, 5}) {
    double v = 0.0;
    const int rc = nwg_dpx_peak_form(ctx, lanes16, form, &v);
    if (rc) return rc;
    best = std::max(best, v);
  }
  *cells_per_s = best;
  return NWG_OK;
}

int nwg_set_launch_timing(nwg_ctx* ctx, int on) {
  if (!ctx) return NWG_ERR_INVALID;
  reinterpret_cast<Ctx*>(ctx)->launch_timing = on != 0;
  return NWG_OK;
}

int nwg_launch_records(nwg_ctx* ctx, nwg_launch_rec* out, int cap) {
  if (!ctx) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (c->rec_finalize() != NWG_OK) return -NWG_ERR_CUDA;
  const int n = (int)c->recs.size();
  for (int k = 0; k < n && k < cap && out; ++k) out[k] = c->recs[k];
  return n;
}

}  // extern "C"
