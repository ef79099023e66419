// batched.cu -- the batched form: length-bucketed plans for the persistent
// wavefront kernels, cached per length profile and replayed as a CUDA graph.
//
// A plan depends only on the sequence lengths (and the mode), never on the
// residues: sequences are sorted by length, Y sequences are grouped (two per
// group on int16x2 lanes, one on int32 lanes), groups are bucketed by the
// rows-per-lane template their length needs, and every bucket gets a job
// prefix table and a device job counter.  The residue-dependent overflow
// check runs on the device inside the step (composition bounds + int32
// re-run queue), so one step is a fixed launch sequence:
//   memset counters -> bounds -> wave kernels (buckets on parallel branches)
//   -> int32 re-run
// which is captured once and replayed with cudaGraphLaunch.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "nwg_ctx.h"

namespace nwg {

namespace {

uint64_t fnv(const int64_t* p, int n, uint64_t h = 1469598103934665603ull) {
  for (int k = 0; k <= n; ++k) {
    uint64_t v = (uint64_t)p[k];
    for (int b = 0; b < 8; ++b) {
      h ^= (v >> (8 * b)) & 0xFF;
      h *= 1099511628211ull;
    }
  }
  return h;
}

// Per-sequence sum of row maxima of the matrix over its residues, in sorted
// order; counts codes outside 0..23.
__global__ void set_bound_kernel(const int8_t* __restrict__ codes, const int64_t* __restrict__ start,
                                 const int32_t* __restrict__ len, const int8_t* __restrict__ rowmax,
                                 int n, int32_t* __restrict__ bound, unsigned long long* __restrict__ bad) {
  const int s = blockIdx.x;
  if (s >= n) return;
  const int8_t* p = codes + start[s];
  const int L = len[s];
  int acc = 0, nbad = 0;
  for (int k = threadIdx.x; k < L; k += blockDim.x) {
    const int c = p[k];
    if (c < 0 || c >= kLetters) ++nbad;
    else acc += rowmax[c];
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_down_sync(0xffffffffu, acc, o);
    nbad += __shfl_down_sync(0xffffffffu, nbad, o);
  }
  __shared__ int wa[4], wb[4];
  if ((threadIdx.x & 31) == 0) { wa[threadIdx.x >> 5] = acc; wb[threadIdx.x >> 5] = nbad; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int A = 0, B = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { A += wa[w]; B += wb[w]; }
    bound[s] = A;
    if (B) atomicAdd(bad, (unsigned long long)B);
  }
}

}  // namespace

struct BatchPlan {
  // key
  int nx = -1, ny = -1;
  bool triangle = true;
  int mode = -1;
  uint64_t hx = 0, hy = 0;
  uint64_t tune_version = 0;
  // sorted sets (host copies + device arrays)
  SetView X, Y;
  DevBuf bxs, bxl, bxo, bxb, bys, byl, byo, byb;
  // groups, buckets
  struct Bucket { int R, P, V, W, check, g0, ng; int64_t j0, njobs, pairs; double cells; int grid;
                  size_t scratch_off; int maxrows; };
  std::vector<Bucket> buckets;
  DevBuf gy, gy2, gx, jobs, counters, rerun, rerun_scratch, wscratch;
  int64_t rerun_cap = 0, rerun_threads = 0;
  int64_t pairs16 = 0, pairs32 = 0, pairs_checked = 0;
  int scols = 1;
  int64_t codes_len = 0;   // bytes of the codes buffer the sets reach (one past the last residue)
  // graph
  cudaGraphExec_t exec = nullptr;
  const int8_t* g_codes = nullptr;
  float* g_D = nullptr;
  int64_t g_ld = 0, g_col0 = 0;
  cudaStream_t g_stream = nullptr;
  int graph_launches = 0;

  ~BatchPlan() {
    if (exec) cudaGraphExecDestroy(exec);
    for (DevBuf* b : {&bxs, &bxl, &bxo, &bxb, &bys, &byl, &byo, &byb, &gy, &gy2, &gx, &jobs, &counters,
                      &rerun, &rerun_scratch, &wscratch})
      b->release();
  }
};

void destroy_plans(Ctx* c) {
  for (BatchPlan*& p : c->plans) {
    delete p;
    p = nullptr;
  }
}

static int upload_set(Ctx* c, const int64_t* offsets, int n, SetView& v, DevBuf& bs, DevBuf& bl, DevBuf& bo,
                      DevBuf& bb) {
  v.n = n;
  v.len.resize(n);
  v.orig.resize(n);
  v.start.resize(n);
  for (int i = 0; i < n; ++i) {
    const int64_t L = offsets[i + 1] - offsets[i];
    if (L <= 0) return c->fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
    if (L > (int64_t)0x7fffffff) return c->fail(NWG_ERR_INVALID, "sequence too long");
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
  if ((rc = bs.ensure(sizeof(int64_t) * n)) || (rc = bl.ensure(sizeof(int32_t) * n)) ||
      (rc = bo.ensure(sizeof(int32_t) * n)) || (rc = bb.ensure(sizeof(int32_t) * n)))
    return c->fail(rc, "set allocation");
  if ((rc = c->cuda(cudaMemcpy(bs.p, v.start.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice), "set upload")) ||
      (rc = c->cuda(cudaMemcpy(bl.p, v.len.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice), "set upload")) ||
      (rc = c->cuda(cudaMemcpy(bo.p, v.orig.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice), "set upload")))
    return rc;
  v.d_start = (int64_t*)bs.p;
  v.d_len = (int32_t*)bl.p;
  v.d_orig = (int32_t*)bo.p;
  return NWG_OK;
}

// Build (or fetch) the plan for these lengths.
static int get_plan(Ctx* c, const int64_t* xoff, int nx, const int64_t* yoff, int ny, bool triangle, int mode,
                    BatchPlan** out) {
  const uint64_t hx = fnv(xoff, nx), hy = triangle ? hx : fnv(yoff, ny, 7);
  BatchPlan*& slot = c->plans[triangle ? 0 : 1];
  if (slot && slot->nx == nx && slot->ny == ny && slot->mode == mode && slot->hx == hx && slot->hy == hy &&
      slot->tune_version == c->tune_version) {
    *out = slot;
    return NWG_OK;
  }
  delete slot;
  slot = nullptr;
  BatchPlan* p = new BatchPlan();
  p->nx = nx; p->ny = ny; p->triangle = triangle; p->mode = mode; p->hx = hx; p->hy = hy;
  p->tune_version = c->tune_version;
  int rc;
  if ((rc = upload_set(c, xoff, nx, p->X, p->bxs, p->bxl, p->bxo, p->bxb))) { delete p; return rc; }
  if (triangle) {
    p->Y = p->X;
  } else if ((rc = upload_set(c, yoff, ny, p->Y, p->bys, p->byl, p->byo, p->byb))) {
    delete p;
    return rc;
  }
  const SetView& X = p->X;
  const SetView& Y = p->Y;
  for (int k = 0; k < X.n; ++k) p->codes_len = std::max<int64_t>(p->codes_len, X.start[k] + X.len[k]);
  for (int k = 0; k < Y.n; ++k) p->codes_len = std::max<int64_t>(p->codes_len, Y.start[k] + Y.len[k]);
  const bool force32 = mode == NWG_MODE_BATCHED_INT32 ||
                       std::max(X.maxlen, Y.maxlen) > c->i16.max_len;
  // certain int16: the shorter sequence of every pair is short enough that
  // even its best-case score fits (max matrix entry * length)
  int maxs = 0;
  for (int k = 0; k < kLetters * kLetters; ++k) maxs = std::max<int>(maxs, c->sub[k]);
  const int certain_len = maxs > 0 ? c->i16.max_h / maxs : 1 << 30;

  struct Group { int y, y2, nx, R, V, W, P, check; };
  std::vector<Group> groups;
  groups.reserve((size_t)Y.n / 2 + 1);
  for (int y = 0; y < Y.n;) {
    const TuneChoice tc = c->choice(Y.len[y]);
    if (!force32) {
      const int y2 = y + 1 < Y.n ? y + 1 : -1;
      const int last = y2 >= 0 ? y2 : y;
      const int nxg = triangle ? last + 1 : X.n;
      // Y sorted by length: Y.len[y] is the group's longest; the pair's
      // shorter sequence is at most that long.
      const int check = Y.len[y] > certain_len ? 1 : 0;
      groups.push_back({y, y2, nxg, tc.R, tc.V, tc.W, 2, check});
      y = last + 1;
    } else {
      const TuneChoice t32 = int32_choice(tc);
      groups.push_back({y, -1, triangle ? y + 1 : X.n, t32.R, t32.V, 32, 1, 0});
      ++y;
    }
  }
  std::stable_sort(groups.begin(), groups.end(), [](const Group& a, const Group& b) {
    if (a.R * a.W != b.R * b.W) return a.R * a.W > b.R * b.W;
    if (a.R != b.R) return a.R > b.R;
    if (a.V != b.V) return a.V > b.V;
    if (a.P != b.P) return a.P > b.P;
    return a.check > b.check;
  });
  const int ng = (int)groups.size();
  std::vector<int32_t> gy(ng), gy2(ng), gx(ng);
  for (int k = 0; k < ng; ++k) { gy[k] = groups[k].y; gy2[k] = groups[k].y2; gx[k] = groups[k].nx; }
  std::vector<double> sx((size_t)X.n + 1, 0.0);
  for (int i = 0; i < X.n; ++i) sx[i + 1] = sx[i] + X.len[i];
  std::vector<int64_t> prefix;
  prefix.reserve(ng + 16);
  for (int k = 0; k < ng;) {
    int e = k;
    while (e < ng && groups[e].R == groups[k].R && groups[e].V == groups[k].V && groups[e].W == groups[k].W &&
           groups[e].P == groups[k].P && groups[e].check == groups[k].check)
      ++e;
    BatchPlan::Bucket b{groups[k].R, groups[k].P, groups[k].V, groups[k].W, groups[k].check, k, e - k,
                        (int64_t)prefix.size(), 0, 0, 0.0, 0, 0, 0};
    const int xper = kWaveWarps * (32 / b.W) * wave_x_per_front(b.V);   // X per CTA job
    int64_t acc = 0;
    for (int g = k; g < e; ++g) {
      prefix.push_back(acc);
      acc += (groups[g].nx + xper - 1) / xper;
      b.maxrows = std::max(b.maxrows, Y.len[groups[g].y]);
      for (int yy : {groups[g].y, groups[g].y2}) {
        if (yy < 0) continue;
        const int cnt = triangle ? yy : X.n;   // pairs i<j only (diagonal not counted)
        b.pairs += cnt;
        b.cells += (double)Y.len[yy] * sx[cnt];
        const int64_t all = triangle ? yy + 1 : X.n;
        if (groups[g].P == 2) p->pairs16 += all; else p->pairs32 += all;
        if (groups[g].check) p->pairs_checked += all;
      }
    }
    prefix.push_back(acc);
    b.njobs = acc;
    p->buckets.push_back(b);
    k = e;
  }
  const size_t nb = p->buckets.size();
  if ((rc = p->gy.ensure(sizeof(int32_t) * ng)) || (rc = p->gy2.ensure(sizeof(int32_t) * ng)) ||
      (rc = p->gx.ensure(sizeof(int32_t) * ng)) || (rc = p->jobs.ensure(sizeof(int64_t) * prefix.size())) ||
      (rc = p->counters.ensure(sizeof(unsigned long long) * (nb + 2)))) {
    delete p;
    return c->fail(rc, "plan allocation");
  }
  if ((rc = c->cuda(cudaMemcpy(p->gy.p, gy.data(), sizeof(int32_t) * ng, cudaMemcpyHostToDevice), "plan upload")) ||
      (rc = c->cuda(cudaMemcpy(p->gy2.p, gy2.data(), sizeof(int32_t) * ng, cudaMemcpyHostToDevice), "plan upload")) ||
      (rc = c->cuda(cudaMemcpy(p->gx.p, gx.data(), sizeof(int32_t) * ng, cudaMemcpyHostToDevice), "plan upload")) ||
      (rc = c->cuda(cudaMemcpy(p->jobs.p, prefix.data(), sizeof(int64_t) * prefix.size(), cudaMemcpyHostToDevice),
                    "plan upload"))) {
    delete p;
    return rc;
  }
  // grids (persistent: SMs x resident CTAs, capped by the jobs) and the band
  // boundary scratch: buckets run concurrently, so every bucket with more than
  // one band gets its own region
  p->scols = std::max(X.maxlen, 1);
  size_t scratch_words = 1;
  for (auto& b : p->buckets) {
    b.grid = (int)std::min<int64_t>(b.njobs, (int64_t)c->sms * wave_max_ctas_per_sm(b.R, b.P, b.V, b.W));
    b.grid = std::max(b.grid, 1);
    b.scratch_off = scratch_words;
    if (b.maxrows > b.W * b.R)
      scratch_words += (size_t)b.grid * kWaveWarps * (32 / b.W) * wave_x_per_front(b.V) * 4 * p->scols;
  }
  if ((rc = p->wscratch.ensure(sizeof(int32_t) * scratch_words))) {
    delete p;
    return c->fail(rc, "wave scratch");
  }
  p->rerun_cap = p->pairs_checked;
  if (p->rerun_cap > 0) {
    p->rerun_threads = std::min<int64_t>(p->rerun_cap, (int64_t)c->sms * 512);
    p->rerun_threads = (p->rerun_threads + kPlainThreads - 1) / kPlainThreads * kPlainThreads;
    if ((rc = p->rerun.ensure(sizeof(int2) * (size_t)p->rerun_cap)) ||
        (rc = p->rerun_scratch.ensure(sizeof(int2) * (size_t)p->rerun_threads * p->scols))) {
      delete p;
      return c->fail(rc, "re-run queue");
    }
  }
  slot = p;
  *out = p;
  return NWG_OK;
}

// Queue one batched step on stream s (directly or under graph capture).
static int enqueue_step(Ctx* c, BatchPlan* p, const int8_t* d_codes, float* d_D, int64_t ld, int64_t col0,
                        cudaStream_t s, bool timed) {
  int rc;
  const size_t nb = p->buckets.size();
  unsigned long long* ctr = (unsigned long long*)p->counters.p;
  if ((rc = c->cuda(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long) * (nb + 2), s), "counters"))) return rc;
  set_bound_kernel<<<p->X.n, 128, 0, s>>>(d_codes, p->X.d_start, p->X.d_len, (const int8_t*)c->b_rowmax.p, p->X.n,
                                          (int32_t*)p->bxb.p, ctr + nb + 1);
  ++c->launches;
  if (!p->triangle) {
    set_bound_kernel<<<p->Y.n, 128, 0, s>>>(d_codes, p->Y.d_start, p->Y.d_len, (const int8_t*)c->b_rowmax.p,
                                            p->Y.n, (int32_t*)p->byb.p, ctr + nb + 1);
    ++c->launches;
  }
  if ((rc = c->cuda(cudaGetLastError(), "bound kernel"))) return rc;

  WaveArgs a{};
  a.codes = d_codes;
  a.codes_end = d_codes + p->codes_len;
  a.xstart = p->X.d_start; a.xlen = p->X.d_len; a.xorig = p->X.d_orig;
  a.ystart = p->Y.d_start; a.ylen = p->Y.d_len; a.yorig = p->Y.d_orig;
  a.group_y = (const int32_t*)p->gy.p;
  a.group_y2 = (const int32_t*)p->gy2.p;
  a.group_x = (const int32_t*)p->gx.p;
  a.D = d_D; a.ld = ld; a.col0 = col0;
  a.scratch = (int32_t*)p->wscratch.p;
  a.scratch_cols = p->scols;
  a.nx = p->X.n; a.ny = p->Y.n;
  a.triangle = p->triangle ? 1 : 0;
  a.go = c->go; a.ge = c->ge;
  a.sub = (const int8_t*)c->b_sub.p;
  a.xbound = (const int32_t*)p->bxb.p;
  a.ybound = (const int32_t*)(p->triangle ? p->bxb.p : p->byb.p);
  a.rerun = (int2*)p->rerun.p;
  a.rerun_count = ctr + nb;
  a.rerun_cap = p->rerun_cap;

  // fork: buckets go round-robin onto the context's branch streams so one
  // bucket's tail overlaps the next bucket's start
  const int nbr = timed ? 1 : (int)std::min<size_t>(c->branch.size() + 1, nb);
  if (nbr > 1) {
    if ((rc = c->cuda(cudaEventRecord(c->fork_ev, s), "fork"))) return rc;
    for (int k = 0; k + 1 < nbr; ++k)
      if ((rc = c->cuda(cudaStreamWaitEvent(c->branch[k], c->fork_ev, 0), "fork"))) return rc;
  }
  for (size_t k = 0; k < nb; ++k) {
    const BatchPlan::Bucket& b = p->buckets[k];
    if (b.njobs == 0) continue;
    cudaStream_t bs = (nbr > 1 && (k % nbr) != 0) ? c->branch[(k % nbr) - 1] : s;
    a.job_prefix = (const int64_t*)p->jobs.p + b.j0;
    a.counter = ctr + k;
    a.njobs = b.njobs;
    a.g_begin = b.g0;
    a.ngroups = b.ng;
    a.check_bound = b.check;
    a.max_h = c->i16.max_h;
    a.scratch = (int32_t*)p->wscratch.p + b.scratch_off;
    int ri = -1;
    if (timed) {
      nwg_launch_rec r{0, b.R, b.P == 2 ? 1 : 0, b.grid, b.pairs, (int64_t)b.cells, 0.0, b.V, b.W};
      if ((ri = c->rec_begin(r)) < 0) return c->fail(NWG_ERR_CUDA, "launch timing");
    }
    if ((rc = c->cuda(launch_wave(b.R, b.P, b.V, b.W, a, b.grid, bs), "wave launch"))) return rc;
    if (ri >= 0 && (rc = c->rec_end(ri))) return rc;
    ++c->launches;
  }
  if (nbr > 1) {
    for (int k = 0; k + 1 < nbr; ++k) {
      if ((rc = c->cuda(cudaEventRecord(c->join_ev[k], c->branch[k]), "join")) ||
          (rc = c->cuda(cudaStreamWaitEvent(s, c->join_ev[k], 0), "join")))
        return rc;
    }
  }
  if (p->rerun_cap > 0) {
    if ((rc = c->cuda(launch_rerun(a, (int2*)p->rerun_scratch.p, p->rerun_threads, s), "re-run launch"))) return rc;
    ++c->launches;
  }
  return NWG_OK;
}

int Ctx::batched(const int8_t* d_codes, const int64_t* xoff, int nx, const int64_t* yoff, int ny, bool triangle,
                 float* d_D, int64_t ld, int64_t col0, int mode, nwg_stats* st) {
  BatchPlan* p = nullptr;
  int rc;
  if ((rc = get_plan(this, xoff, nx, yoff, ny, triangle, mode, &p))) return rc;
  for (const auto& b : p->buckets) prepare_wave(b.R, b.P, b.V, b.W);
  if (st) {
    st->pairs_int16 += p->pairs16;
    st->pairs_int32 += p->pairs32;
    st->buckets += (int32_t)p->buckets.size();
  }
  if (launch_timing || !use_graphs) {
    if ((rc = enqueue_step(this, p, d_codes, d_D, ld, col0, stream, launch_timing))) return rc;
  } else {
    if (!p->exec || p->g_codes != d_codes || p->g_D != d_D || p->g_ld != ld || p->g_col0 != col0 ||
        p->g_stream != stream) {
      if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
      }
      cudaGraph_t g;
      if ((rc = cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "graph capture"))) return rc;
      const int saved = launches;
      rc = enqueue_step(this, p, d_codes, d_D, ld, col0, stream, false);
      const cudaError_t e = cudaStreamEndCapture(stream, &g);
      if (rc) return rc;
      if ((rc = cuda(e, "graph capture"))) return rc;
      rc = cuda(cudaGraphInstantiate(&p->exec, g, 0), "graph instantiate");
      cudaGraphDestroy(g);
      if (rc) return rc;
      p->g_codes = d_codes; p->g_D = d_D; p->g_ld = ld; p->g_col0 = col0; p->g_stream = stream;
      p->graph_launches = launches - saved;
      launches = saved;
    }
    if ((rc = cuda(cudaGraphLaunch(p->exec, stream), "graph launch"))) return rc;
    launches += p->graph_launches;
  }
  if (st) {
    // residue check and re-run count (the caller asked for stats: synchronize)
    unsigned long long cnt[2] = {0, 0};
    const size_t nb = p->buckets.size();
    if ((rc = cuda(cudaMemcpyAsync(cnt, (unsigned long long*)p->counters.p + nb, sizeof(cnt), cudaMemcpyDeviceToHost,
                                   stream), "counters")) ||
        (rc = cuda(cudaStreamSynchronize(stream), "counters")))
      return rc;
    if (cnt[1]) return fail(NWG_ERR_BAD_RESIDUE, "residue code outside 0..23");
    st->reruns += (int64_t)cnt[0];
  }
  return NWG_OK;
}

}  // namespace nwg
