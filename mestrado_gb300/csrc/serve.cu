// serve.cu -- continuous batching of alignment jobs (distance matrix + guide
// tree per job) on one GPU.
//
// A job is a set of sequences; its result is the job's distance matrix and its
// neighbor-joining join list, each identical to what nwg_score_all and nwg_nj
// give for that job alone.  Jobs are submitted at any time.  A worker thread
// forms batches from the pending queue: a job is admitted when its HBM
// footprint (n^2 matrix, NJ workspace, codes) fits the budget left by the jobs
// in flight.  A batch is queued on one of four pipeline slots (own stream,
// device arenas, pinned staging):
//   residues in (ASCII; encoded and reversed on the device) -> one
//   multi-job plan: every job's Y groups in shared length buckets, so one
//   persistent launch per bucket interleaves pairs of different jobs ->
//   matrices out -> the join loops, one thread-block cluster per job (jobs
//   that fit, with the matrix in the cluster's shared memory) -> join lists
//   out.
// While one slot's batch is on the device the next batch is formed and queued
// on another free slot, so arrivals overlap the work in flight.  Each slot has
// its own completion thread that waits for that slot's event, hands results
// to their jobs and frees their footprint, so a short batch is returned
// without waiting for a longer one launched before it.  Nothing waits on the
// device except those host-side event waits.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <numeric>
#include <thread>
#include <unordered_map>
#include <vector>

#include "nwg_ctx.h"

namespace nwg {

namespace {

// CTAs per job in the join-loop launch: the O(n^2) passes of one join split
// over 8 SMs (jobs of one batch run side by side).
constexpr int kNJClusterServe = 8;
constexpr int kNJWideN = 256;   // from this job size on, the widest cluster
constexpr int kNJSmemServeMax = 768;   // jobs up to this size: join loop in shared memory

double clock_ms() {
  using clk = std::chrono::steady_clock;
  return std::chrono::duration<double, std::milli>(clk::now().time_since_epoch()).count();
}

struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return NWG_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes, 4096);
    if (cudaMallocHost(&p, want) != cudaSuccess) {
      cudaGetLastError();
      return NWG_ERR_OOM;
    }
    cap = want;
    return NWG_OK;
  }
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
};

}  // namespace

struct ServeJob {
  uint64_t id = 0;
  int n = 0;
  std::vector<char> ascii;    // the job's residues as submitted (encoded on the device)
  std::vector<int64_t> off;
  size_t footprint = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  int batch_jobs = 0;
  int status = NWG_OK;
  bool done = false;
  bool waited = false;   // a nwg_server_wait call holds the job (one waiter at a time)
  std::vector<float> D;
  std::vector<nwg_join> joins;
  unsigned long long njst[5] = {0, 0, 0, 0, 0};
  // placement in its batch
  size_t d_off = 0, nj_off = 0, codes_off = 0, desc_idx = 0, seq_base = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  DevBuf ascii, codes, bad, start, len, orig, gy, gy2, gx, gxb, gdofs, gld, jobsbuf, counters, scratch, D, njws, njdesc;
  HostBuf h_codes, h_plan, h_D, h_joins;
  std::vector<ServeJob*> batch;
  bool busy = false;       // holds a batch (from admission to completion)
  bool launched = false;   // its work is queued on the device
  size_t plan_bytes = 0;
  ~Slot() {
    for (DevBuf* b : {&ascii, &codes, &bad, &start, &len, &orig, &gy, &gy2, &gx, &gxb, &gdofs, &gld, &jobsbuf, &counters,
                      &scratch,
                      &D, &njws, &njdesc})
      b->release();
    if (done) cudaEventDestroy(done);
    if (stream) cudaStreamDestroy(stream);
  }
};

struct Server {
  Ctx* ctx = nullptr;
  int64_t budget = 0;
  int max_batch = 0;
  int64_t in_use = 0;
  uint64_t next_id = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_slot;
  static constexpr int kSlots = 4;   // batches that can be on the device at once
  std::deque<ServeJob*> pending;
  std::unordered_map<uint64_t, ServeJob*> jobs;
  Slot slots[kSlots];
  bool stop = false;
  std::thread worker, completer[kSlots];
  int device = 0;

  size_t footprint(int n) const {
    return sizeof(float) * (size_t)n * nj_row_stride(n) + nj_job_workspace(n) + (size_t)n * 600 + 4096;
  }

  int launch_batch(Slot& S);
  void worker_loop();
  void completer_loop(int si);
  int free_slot() const {
    for (int k = 0; k < kSlots; ++k)
      if (!slots[k].busy) return k;
    return -1;
  }
};

// Build the multi-job plan of the slot's batch and queue all its work.
int Server::launch_batch(Slot& S) {
  Ctx& c = *ctx;
  const int nj = (int)S.batch.size();
  // sequences of all jobs, each job sorted by length (descending)
  int64_t total_codes = 0, total_seqs = 0, total_D = 0, total_ws = 0;
  for (ServeJob* J : S.batch) {
    J->codes_off = (size_t)total_codes;
    J->seq_base = (size_t)total_seqs;
    total_codes += (int64_t)J->ascii.size();
    total_seqs += J->n;
    J->d_off = (size_t)total_D;   // rows padded for the join loop's 16-byte loads
    total_D += (int64_t)J->n * nj_row_stride(J->n);
    J->nj_off = (size_t)total_ws;
    total_ws += (int64_t)nj_job_workspace(J->n);
  }
  std::vector<int64_t> start((size_t)total_seqs);
  std::vector<int32_t> len((size_t)total_seqs), orig((size_t)total_seqs);
  struct Group { int y, y2, nx, xbase, R, V, W, P; int64_t dofs; int ld; };
  std::vector<Group> groups;
  int maxlen = 1;
  int64_t base = 0;
  for (ServeJob* J : S.batch) {
    const int n = J->n;
    const int ldp = nj_row_stride(n);
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int b) { return J->off[a + 1] - J->off[a] > J->off[b + 1] - J->off[b]; });
    for (int k = 0; k < n; ++k) {
      const int o = ord[k];
      start[base + k] = (int64_t)J->codes_off + J->off[o];
      len[base + k] = (int32_t)(J->off[o + 1] - J->off[o]);
      orig[base + k] = o;
      maxlen = std::max(maxlen, len[base + k]);
    }
    const bool long_set = len[base] > c.i16.max_len;
    int maxs = 0;
    for (int k = 0; k < kLetters * kLetters; ++k) maxs = std::max<int>(maxs, c.sub[k]);
    const int certain = maxs > 0 ? c.i16.max_h / maxs : 1 << 30;
    for (int y = 0; y < n;) {
      const int gyi = (int)base + y;
      const TuneChoice tc = c.choice_wave(len[gyi]);   // latency first: wavefronts only
      if (!long_set && len[gyi] <= certain) {
        const int y2 = y + 1 < n ? gyi + 1 : -1;
        const int last = y2 >= 0 ? y + 1 : y;
        groups.push_back({gyi, y2, last + 1, (int)base, tc.R, tc.V, tc.W, 2, (int64_t)J->d_off, ldp});
        y = last + 1;
      } else {
        const TuneChoice t32 = int32_choice(tc);
        groups.push_back({gyi, -1, y + 1, (int)base, t32.R, t32.V, 32, 1, (int64_t)J->d_off, ldp});
        ++y;
      }
    }
    base += n;
  }
  std::stable_sort(groups.begin(), groups.end(), [](const Group& a, const Group& b) {
    if (a.R * a.W != b.R * b.W) return a.R * a.W > b.R * b.W;
    if (a.R != b.R) return a.R > b.R;
    if (a.V != b.V) return a.V > b.V;
    return a.P > b.P;
  });
  const int ng = (int)groups.size();
  struct Bucket { int R, V, W, P, g0, ng; int64_t j0, njobs; int grid; size_t soff; bool multi; };
  std::vector<Bucket> buckets;
  std::vector<int64_t> prefix;
  for (int k = 0; k < ng;) {
    int e = k;
    while (e < ng && groups[e].R == groups[k].R && groups[e].V == groups[k].V && groups[e].W == groups[k].W &&
           groups[e].P == groups[k].P)
      ++e;
    Bucket b{groups[k].R, groups[k].V, groups[k].W, groups[k].P, k, e - k, (int64_t)prefix.size(), 0, 0, 0, false};
    const int xper = kWaveWarps * (32 / b.W) * wave_x_per_front(b.V);   // X per CTA job
    int64_t acc = 0;
    for (int g = k; g < e; ++g) {
      prefix.push_back(acc);
      acc += (groups[g].nx + xper - 1) / xper;
      if (len[groups[g].y] > b.W * groups[g].R) b.multi = true;
    }
    prefix.push_back(acc);
    b.njobs = acc;
    buckets.push_back(b);
    k = e;
  }
  size_t scratch_words = 1;
  for (auto& b : buckets) {
    b.grid = (int)std::max<int64_t>(
        1, std::min<int64_t>(b.njobs, (int64_t)c.sms * wave_max_ctas_per_sm(b.R, b.P, b.V, b.W)));
    b.soff = scratch_words;
    if (b.multi) scratch_words += (size_t)b.grid * kWaveWarps * (32 / b.W) * wave_x_per_front(b.V) * 4 * maxlen;
    prepare_wave(b.R, b.P, b.V, b.W);
  }
  // device buffers of the slot (grow-only)
  int rc;
  const size_t desc = nj_job_desc_bytes();
  if ((rc = S.codes.ensure((size_t)std::max<int64_t>(total_codes, 1))) ||
      (rc = S.ascii.ensure((size_t)std::max<int64_t>(total_codes, 1))) || (rc = S.bad.ensure(sizeof(int) * total_seqs)) ||
      (rc = S.start.ensure(sizeof(int64_t) * total_seqs)) || (rc = S.len.ensure(sizeof(int32_t) * total_seqs)) ||
      (rc = S.orig.ensure(sizeof(int32_t) * total_seqs)) || (rc = S.gy.ensure(sizeof(int32_t) * ng)) ||
      (rc = S.gy2.ensure(sizeof(int32_t) * ng)) || (rc = S.gx.ensure(sizeof(int32_t) * ng)) ||
      (rc = S.gxb.ensure(sizeof(int32_t) * ng)) || (rc = S.gdofs.ensure(sizeof(int64_t) * ng)) ||
      (rc = S.gld.ensure(sizeof(int32_t) * ng)) || (rc = S.jobsbuf.ensure(sizeof(int64_t) * prefix.size())) ||
      (rc = S.counters.ensure(sizeof(unsigned long long) * (buckets.size() + 1))) ||
      (rc = S.scratch.ensure(sizeof(int32_t) * scratch_words)) || (rc = S.D.ensure(sizeof(float) * total_D)) ||
      (rc = S.njws.ensure((size_t)total_ws)) || (rc = S.njdesc.ensure(desc * nj)))
    return rc;
  // pinned staging: codes, then the plan arrays, then NJ descriptors
  // NJ descriptors grouped by launch form: jobs whose join loop runs in one
  // CTA, then in a cluster's shared memory, then the rest (join loop over
  // L2); one launch per group
  int nmax_g[3] = {0, 0, 0}, cnt_g[3] = {0, 0, 0};
  std::vector<int> form(nj);
  for (int k = 0; k < nj; ++k) {
    const int n = S.batch[k]->n;
    form[k] = n <= cta_nj_max_n() ? 0 : (n <= kNJSmemServeMax && smem_nj_cluster(n) ? 1 : 2);
    nmax_g[form[k]] = std::max(nmax_g[form[k]], n);
    ++cnt_g[form[k]];
  }
  const int c_smem = cnt_g[1] ? smem_nj_cluster(nmax_g[1]) : 0;
  std::vector<char> descs(desc * nj);
  std::vector<nwg_join*> jptr(nj);
  std::vector<unsigned long long*> sptr(nj);
  int next_idx[3] = {0, cnt_g[0], cnt_g[0] + cnt_g[1]};
  for (int k = 0; k < nj; ++k) {
    ServeJob* J = S.batch[k];
    J->desc_idx = (size_t)next_idx[form[k]]++;
    nj_job_setup(&descs[desc * J->desc_idx], (float*)S.D.p + J->d_off, J->n, nj_row_stride(J->n),
                 (char*)S.njws.p + J->nj_off, &jptr[k], &sptr[k]);
  }
  std::vector<int32_t> a_gy(ng), a_gy2(ng), a_gx(ng), a_gxb(ng), a_gld(ng);
  std::vector<int64_t> a_gdofs(ng);
  for (int k = 0; k < ng; ++k) {
    a_gy[k] = groups[k].y;
    a_gy2[k] = groups[k].y2;
    a_gx[k] = groups[k].nx;
    a_gxb[k] = groups[k].xbase;
    a_gdofs[k] = groups[k].dofs;
    a_gld[k] = groups[k].ld;
  }
  struct Piece { const void* src; size_t bytes; void* dst; };
  std::vector<Piece> pieces = {
      {start.data(), sizeof(int64_t) * total_seqs, S.start.p}, {len.data(), sizeof(int32_t) * total_seqs, S.len.p},
      {orig.data(), sizeof(int32_t) * total_seqs, S.orig.p},  {a_gy.data(), sizeof(int32_t) * ng, S.gy.p},
      {a_gy2.data(), sizeof(int32_t) * ng, S.gy2.p},          {a_gx.data(), sizeof(int32_t) * ng, S.gx.p},
      {a_gxb.data(), sizeof(int32_t) * ng, S.gxb.p},          {a_gdofs.data(), sizeof(int64_t) * ng, S.gdofs.p},
      {a_gld.data(), sizeof(int32_t) * ng, S.gld.p},          {prefix.data(), sizeof(int64_t) * prefix.size(), S.jobsbuf.p},
      {descs.data(), desc * nj, S.njdesc.p}};
  size_t staged = 0;
  for (auto& pc : pieces) staged += (pc.bytes + 15) / 16 * 16;
  if ((rc = S.h_codes.ensure((size_t)std::max<int64_t>(total_codes, 1))) || (rc = S.h_plan.ensure(staged)) ||
      (rc = S.h_D.ensure(sizeof(float) * total_D)) ||
      (rc = S.h_joins.ensure((sizeof(nwg_join) * (size_t)total_seqs) + sizeof(unsigned long long) * 5 * nj +
                             sizeof(int) * total_seqs)))
    return rc;
  for (ServeJob* J : S.batch)
    std::memcpy((char*)S.h_codes.p + J->codes_off, J->ascii.data(), J->ascii.size());
  size_t o = 0;
  for (auto& pc : pieces) {
    std::memcpy((char*)S.h_plan.p + o, pc.src, pc.bytes);
    o += (pc.bytes + 15) / 16 * 16;
  }
  cudaStream_t st = S.stream;
  if ((rc = c.cuda(cudaMemcpyAsync(S.ascii.p, S.h_codes.p, (size_t)total_codes, cudaMemcpyHostToDevice, st), "serve")))
    return rc;
  o = 0;
  for (auto& pc : pieces) {
    if ((rc = c.cuda(cudaMemcpyAsync(pc.dst, (char*)S.h_plan.p + o, pc.bytes, cudaMemcpyHostToDevice, st), "serve")))
      return rc;
    o += (pc.bytes + 15) / 16 * 16;
  }
  // codes: every sequence encoded and reversed in place of its ASCII (same offsets)
  if ((rc = c.cuda(launch_encode((const char*)S.ascii.p, (const int64_t*)S.start.p, (const int64_t*)S.start.p,
                                 (const int32_t*)S.len.p, (int)total_seqs, (int8_t*)S.codes.p, (int*)S.bad.p, st),
                   "serve encode")))
    return rc;
  if ((rc = c.cuda(cudaMemsetAsync(S.counters.p, 0, sizeof(unsigned long long) * (buckets.size() + 1), st), "serve")))
    return rc;
  WaveArgs a{};
  a.codes = (const int8_t*)S.codes.p;
  a.codes_end = a.codes + total_codes;
  a.xstart = a.ystart = (const int64_t*)S.start.p;
  a.xlen = a.ylen = (const int32_t*)S.len.p;
  a.xorig = a.yorig = (const int32_t*)S.orig.p;
  a.group_y = (const int32_t*)S.gy.p;
  a.group_y2 = (const int32_t*)S.gy2.p;
  a.group_x = (const int32_t*)S.gx.p;
  a.group_xbase = (const int32_t*)S.gxb.p;
  a.group_dofs = (const int64_t*)S.gdofs.p;
  a.group_ld = (const int32_t*)S.gld.p;
  a.D = (float*)S.D.p;
  a.ld = 0;
  a.scratch_cols = maxlen;
  a.nx = a.ny = (int)total_seqs;
  a.triangle = 1;
  a.go = c.go;
  a.ge = c.ge;
  a.sub = (const int8_t*)c.b_sub.p;
  for (size_t k = 0; k < buckets.size(); ++k) {
    const Bucket& b = buckets[k];
    a.job_prefix = (const int64_t*)S.jobsbuf.p + b.j0;
    a.counter = (unsigned long long*)S.counters.p + k;
    a.njobs = b.njobs;
    a.g_begin = b.g0;
    a.ngroups = b.ng;
    a.scratch = (int32_t*)S.scratch.p + b.soff;
    if ((rc = c.cuda(launch_wave(b.R, b.P, b.V, b.W, a, b.grid, st), "serve wave launch"))) return rc;
  }
  if ((rc = c.cuda(cudaMemcpyAsync(S.h_D.p, S.D.p, sizeof(float) * total_D, cudaMemcpyDeviceToHost, st), "serve")))
    return rc;
  // join loops, one CTA or one cluster per job, one launch per form (jobs
  // with 256 sequences or more take the device's largest cluster)
  if (cnt_g[0] && (rc = c.cuda(launch_nj_cta(S.njdesc.p, cnt_g[0], nmax_g[0], st), "serve nj launch"))) return rc;
  if (cnt_g[1] && (rc = c.cuda(launch_nj_smem((const char*)S.njdesc.p + desc * cnt_g[0], cnt_g[1], nmax_g[1], c_smem,
                                              st),
                               "serve nj launch")))
    return rc;
  if (cnt_g[2]) {
    const int csize = nmax_g[2] >= kNJWideN ? nj_cluster_size() : kNJClusterServe;
    if ((rc = c.cuda(launch_nj_cluster((const char*)S.njdesc.p + desc * (cnt_g[0] + cnt_g[1]), cnt_g[2], csize, st),
                     "serve nj launch")))
      return rc;
  }
  char* hj = (char*)S.h_joins.p;
  size_t jo = 0;
  for (int k = 0; k < nj; ++k) {
    ServeJob* J = S.batch[k];
    const size_t bytes = sizeof(nwg_join) * (size_t)std::max(J->n - 1, 0);
    if (bytes && (rc = c.cuda(cudaMemcpyAsync(hj + jo, jptr[k], bytes, cudaMemcpyDeviceToHost, st), "serve"))) return rc;
    jo += bytes;
  }
  for (int k = 0; k < nj; ++k) {
    if ((rc = c.cuda(cudaMemcpyAsync(hj + jo, sptr[k], sizeof(unsigned long long) * 5, cudaMemcpyDeviceToHost, st),
                     "serve")))
      return rc;
    jo += sizeof(unsigned long long) * 5;
  }
  if ((rc = c.cuda(cudaMemcpyAsync(hj + jo, S.bad.p, sizeof(int) * total_seqs, cudaMemcpyDeviceToHost, st), "serve")))
    return rc;
  return c.cuda(cudaEventRecord(S.done, st), "serve event");
}

void Server::worker_loop() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv_work.wait(lk, [&] { return stop || (!pending.empty() && free_slot() >= 0); });
    if (stop) return;
    const int si = free_slot();
    Slot& S = slots[si];
    S.batch.clear();
    const double now = clock_ms();
    // first come, first served: stop at the first job that does not fit
    while (!pending.empty() && (int)S.batch.size() < max_batch &&
           in_use + (int64_t)pending.front()->footprint <= budget) {
      ServeJob* J = pending.front();
      pending.pop_front();
      in_use += (int64_t)J->footprint;
      J->t_admit = now;
      S.batch.push_back(J);
    }
    if (S.batch.empty()) {
      // budget taken by the batches in flight (a job alone always fits: the
      // submit call checks that): wait for a completion
      cv_work.wait(lk);
      continue;
    }
    for (ServeJob* J : S.batch) J->batch_jobs = (int)S.batch.size();
    S.busy = true;
    lk.unlock();
    const int rc = launch_batch(S);
    lk.lock();
    if (rc != NWG_OK) {
      cudaStreamSynchronize(S.stream);
      for (ServeJob* J : S.batch) {
        J->status = rc;
        J->done = true;
        J->t_done = clock_ms();
        in_use -= (int64_t)J->footprint;
      }
      S.batch.clear();
      S.busy = false;
      cv_done.notify_all();
      continue;
    }
    S.launched = true;
    cv_slot.notify_all();
  }
}

// One completion thread per slot: each waits for its own slot's batch, so a
// short batch is handed back while a longer one is still on the device.
void Server::completer_loop(int si) {
  cudaSetDevice(device);
  Slot& S = slots[si];
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv_slot.wait(lk, [&] { return stop || S.launched; });
    if (!S.launched && stop) return;
    lk.unlock();
    const cudaError_t e = cudaEventSynchronize(S.done);
    const double now = clock_ms();
    lk.lock();
    S.launched = false;
    const char* hj = (const char*)S.h_joins.p;
    size_t jo = 0;
    for (ServeJob* J : S.batch) {
      const size_t bytes = sizeof(nwg_join) * (size_t)std::max(J->n - 1, 0);
      J->joins.resize((size_t)std::max(J->n - 1, 0));
      if (bytes) std::memcpy(J->joins.data(), hj + jo, bytes);
      jo += bytes;
    }
    for (ServeJob* J : S.batch) {
      std::memcpy(J->njst, hj + jo, sizeof(J->njst));
      jo += sizeof(J->njst);
    }
    const int* badseq = reinterpret_cast<const int*>(hj + jo);
    for (ServeJob* J : S.batch) {
      int nbad = 0;
      for (int k = 0; k < J->n; ++k) nbad += badseq[J->seq_base + k];
      const int n = J->n, ldp = nj_row_stride(n);
      J->D.resize((size_t)n * n);
      const float* src = (const float*)S.h_D.p + J->d_off;
      for (int r = 0; r < n; ++r) std::memcpy(J->D.data() + (size_t)r * n, src + (size_t)r * ldp, sizeof(float) * n);
      J->status = e != cudaSuccess ? NWG_ERR_CUDA
                  : nbad           ? NWG_ERR_BAD_RESIDUE
                  : J->njst[2]     ? NWG_ERR_CUDA
                                   : NWG_OK;
      J->t_done = now;
      J->done = true;
      in_use -= (int64_t)J->footprint;
    }
    S.batch.clear();
    S.busy = false;
    cv_done.notify_all();
    cv_work.notify_all();
  }
}

}  // namespace nwg

using nwg::Server;

extern "C" {

int nwg_server_create(int gap_open, int gap_ext, int64_t hbm_budget_bytes, int max_batch_jobs, nwg_server** out) {
  if (!out || hbm_budget_bytes <= 0 || max_batch_jobs < 1) return NWG_ERR_INVALID;
  *out = nullptr;
  nwg_ctx* c = nullptr;
  int rc = nwg_ctx_create(gap_open, gap_ext, nullptr, &c);
  if (rc) return rc;
  Server* s = new Server();
  s->ctx = reinterpret_cast<nwg::Ctx*>(c);
  s->budget = hbm_budget_bytes;
  s->max_batch = max_batch_jobs;
  cudaGetDevice(&s->device);
  s->ctx->tune_from_cache(nullptr);   // the device's autotuned table when one is cached
  for (auto& S : s->slots) {
    if (cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&S.done, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      delete s;
      nwg_ctx_destroy(c);
      return NWG_ERR_CUDA;
    }
  }
  s->worker = std::thread([s] { s->worker_loop(); });
  for (int k = 0; k < Server::kSlots; ++k) s->completer[k] = std::thread([s, k] { s->completer_loop(k); });
  *out = reinterpret_cast<nwg_server*>(s);
  return NWG_OK;
}

int nwg_server_submit(nwg_server* srv, const char* ascii, const int64_t* offsets, int n, uint64_t* job_id) {
  if (!srv || !ascii || !offsets || n < 1 || !job_id) return NWG_ERR_INVALID;
  Server* s = reinterpret_cast<Server*>(srv);
  if (n > nwg::kServeMaxN) return NWG_ERR_INVALID;
  auto* J = new nwg::ServeJob();
  J->n = n;
  J->off.assign(offsets, offsets + n + 1);
  for (int k = 0; k <= n; ++k) J->off[k] -= offsets[0];
  for (int k = 0; k < n; ++k)
    if (J->off[k + 1] <= J->off[k]) {
      delete J;
      return NWG_ERR_EMPTY_SEQ;
    }
  J->ascii.assign(ascii + offsets[0], ascii + offsets[n]);
  if (J->ascii.empty()) J->ascii.push_back(0);
  J->footprint = s->footprint(n);
  if ((int64_t)J->footprint > s->budget) {
    delete J;
    return NWG_ERR_OOM;
  }
  J->t_submit = nwg::clock_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    J->id = s->next_id++;
    s->jobs[J->id] = J;
    s->pending.push_back(J);
  }
  s->cv_work.notify_all();
  *job_id = J->id;
  return NWG_OK;
}

int nwg_server_wait(nwg_server* srv, uint64_t job_id, int timeout_ms, float* D, nwg_join* joins,
                    nwg_job_info* info) {
  if (!srv) return NWG_ERR_INVALID;
  Server* s = reinterpret_cast<Server*>(srv);
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end()) return NWG_ERR_INVALID;
  nwg::ServeJob* J = it->second;
  if (J->waited) return NWG_ERR_INVALID;   // another thread is waiting for it and will release it
  J->waited = true;
  const auto pred = [&] { return J->done; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, pred);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) {
    J->waited = false;
    return NWG_ERR_TIMEOUT;
  }
  if (D && !J->D.empty()) std::memcpy(D, J->D.data(), sizeof(float) * J->D.size());
  if (joins && !J->joins.empty()) std::memcpy(joins, J->joins.data(), sizeof(nwg_join) * J->joins.size());
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->n = J->n;
    info->status = J->status;
    info->batch_jobs = J->batch_jobs;
    info->queue_ms = J->t_admit - J->t_submit;
    info->latency_ms = J->t_done - J->t_submit;
    double L = 0, L2 = 0;
    for (int k = 0; k < J->n; ++k) {
      const double l = (double)(J->off[k + 1] - J->off[k]);
      L += l;
      L2 += l * l;
    }
    info->cells = (int64_t)((L * L - L2) / 2);
    info->nj_ambiguous_steps = (int64_t)J->njst[0];
    info->nj_tie_steps = (int64_t)J->njst[1];
    info->nj_rebuilds = (int64_t)J->njst[4];
    info->nj_reference_identical = J->njst[0] == 0 && J->njst[3] == 0;
  }
  const int st = J->status;
  // By key: the wait released the lock, and a submit on another thread may
  // have rehashed the map meanwhile, which invalidates `it`.
  s->jobs.erase(job_id);
  delete J;
  return st;
}

int nwg_server_destroy(nwg_server* srv) {
  if (!srv) return NWG_ERR_INVALID;
  Server* s = reinterpret_cast<Server*>(srv);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_slot.notify_all();
  s->worker.join();
  // the completion threads drain what is in flight
  for (auto& t : s->completer) t.join();
  for (auto& S : s->slots) cudaStreamSynchronize(S.stream);
  for (auto& kv : s->jobs) delete kv.second;
  nwg_ctx* c = reinterpret_cast<nwg_ctx*>(s->ctx);
  delete s;
  nwg_ctx_destroy(c);
  return NWG_OK;
}

}  // extern "C"
