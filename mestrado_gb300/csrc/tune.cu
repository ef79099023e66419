// tune.cu -- autotuner of the batched form: per length class of the Y rows,
// the rows-per-lane template and register layout of the wave kernel.
//
// For class k (Y rows in (lo, hi]) a probe workload is built from uniform
// random residues: 128 Y sequences and enough X sequences of hi + 10 %
// residues for ~1e10 cells, scored in block mode.  Candidates: wavefronts of
// W = 32, 16 or 8 lanes with one, two or three bands whose rows land in
// (lo, hi + hi/8], and, for the classes up to 512 rows, one pair per thread
// (W = 1, bands of 16-32 rows).  Each runs once to warm up and once timed
// with CUDA events, on Y of the longest whole number of its bands in the
// class (else hi), which gives its rate in computed (band-padded) cells per
// second.  The class's pick is the least estimated time at hi (padded rows /
// rate); every candidate's rate is kept, so that a plan can pick per Y group
// the candidate whose bands fit that group best.  The table is written to a
// cache file per device (name + SM count) and read back by later contexts.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nwg_ctx.h"

namespace nwg {

namespace {

std::string cache_path(int device) {
  cudaDeviceProp prop;
  std::memset(&prop, 0, sizeof(prop));
  cudaGetDeviceProperties(&prop, device);
  std::string name(prop.name);
  for (char& ch : name)
    if (!((ch >= 'a' && ch <= 'z') || (ch >= 'A' && ch <= 'Z') || (ch >= '0' && ch <= '9'))) ch = '_';
  std::string dir;
  if (const char* e = std::getenv("NWG_TUNE_CACHE")) dir = e;
  else if (const char* h = std::getenv("HOME")) dir = std::string(h) + "/.cache/nwgpu";
  else dir = "/tmp/nwgpu";
  return dir + "/tune_v1_" + name + "_sm" + std::to_string(prop.multiProcessorCount) + ".txt";
}

void make_parent_dirs(const std::string& file) {
  for (size_t k = 1; k < file.size(); ++k)
    if (file[k] == '/') mkdir(file.substr(0, k).c_str(), 0755);   // existing levels just fail
}

const int kCandR[] = {4, 8, 12, 16, 18, 20, 22, 24, 26, 28, 30, 32};

// Upper bound of a class's Y rows for the probes: its longest Y; the open last
// class probes 2000 rows.
int representative_rows(int k) { return k == kTuneClasses - 1 ? 2000 : kClassRows[k]; }
int class_floor(int k) { return k == 0 ? 0 : kClassRows[k - 1]; }

// Y rows a candidate is probed on in class k, or 0 if it is no candidate there.
int probe_rows(int k, const TuneChoice& t) {
  const int hi = representative_rows(k), lo = class_floor(k);
  const int band = t.W * t.R;
  if (t.W == 1) return (t.R >= 16 && hi <= 512) ? hi : 0;
  if (k == kTuneClasses - 1) return (band * 3 >= hi && band <= 2 * hi + 128) ? hi : 0;
  bool useful = false;
  for (int m = 1; m <= 3; ++m) useful |= lo < m * band && m * band <= hi + hi / 8;
  if (!useful) return 0;
  const int whole = hi / band * band;
  return whole > lo ? whole : hi;
}

const char kCacheTag[] = "nwgpu-tune-7";   // bumped whenever the candidate set changes

}  // namespace

// The cached table of this device, if one exists (no tuning run).
bool Ctx::tune_from_cache(nwg_tune_result* res) {
  const std::string path = cache_path(device);
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return false;
  int ok = 0;
  TuneChoice t[kTuneClasses], tw[kTuneClasses];
  double g[kTuneClasses];
  std::vector<Cand> cc[kTuneClasses];
  char tag[32] = {0};
  if (std::fscanf(f, "%31s", tag) == 1 && std::strcmp(tag, kCacheTag) == 0) {
    for (int k = 0; k < kTuneClasses; ++k) {
      int kk, R, V, W, Rw, Vw, Ww, n;
      double gc;
      if (std::fscanf(f, "%d %d %d %d %lf %d %d %d %d", &kk, &R, &V, &W, &gc, &Rw, &Vw, &Ww, &n) != 9 || kk != k ||
          !wave_exists(R, 2, V, W) || Ww < 8 || !wave_exists(Rw, 2, Vw, Ww) || n < 0 || n > 1000)
        break;
      bool good = true;
      for (int e = 0; e < n && good; ++e) {
        Cand c;
        good = std::fscanf(f, "%d %d %d %lf", &c.t.R, &c.t.V, &c.t.W, &c.rate) == 4 &&
               wave_exists(c.t.R, 2, c.t.V, c.t.W) && c.rate > 0.0;
        cc[k].push_back(c);
      }
      if (!good) break;
      t[k] = {R, V, W};
      tw[k] = {Rw, Vw, Ww};
      g[k] = gc;
      ++ok;
    }
  }
  std::fclose(f);
  if (ok != kTuneClasses) return false;
  for (int k = 0; k < kTuneClasses; ++k) {
    tune[k] = t[k];
    tune_wave[k] = tw[k];
    cands[k] = std::move(cc[k]);
    if (res) {
      res->rows_per_lane[k] = t[k].R;
      res->variant[k] = t[k].V;
      res->lanes[k] = t[k].W;
      res->gcups[k] = g[k];
    }
  }
  ++tune_version;
  tuned = true;
  if (res) res->from_cache = 1;
  return true;
}

int Ctx::autotune(bool force, nwg_tune_result* out) {
  const std::string path = cache_path(device);
  nwg_tune_result res;
  std::memset(&res, 0, sizeof(res));
  res.classes = kTuneClasses;
  for (int k = 0; k < kTuneClasses; ++k) res.max_rows[k] = kClassRows[k] > 1000000 ? 0x7fffffff : kClassRows[k];
  if (!force && tune_from_cache(&res)) {
    if (out) *out = res;
    return NWG_OK;
  }
  const auto t0 = std::chrono::steady_clock::now();
  const bool saved_graphs = use_graphs;
  use_graphs = false;
  uint64_t lcg = 0x243F6A8885A308D3ull;
  auto rnd = [&]() {
    lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
    return (uint32_t)(lcg >> 33);
  };
  int rc = NWG_OK;
  DevBuf probe;
  for (int k = 0; k < kTuneClasses; ++k) cands[k].clear();   // the probes run tune[k] as it is
  std::vector<Cand> found[kTuneClasses];
  for (int k = 0; k < kTuneClasses && rc == NWG_OK; ++k) {
    const int Ly = representative_rows(k);
    const int Lx = Ly + Ly / 10;
    const int ny = 128;
    int nx = (int)std::min<double>(4096.0, std::max<double>(256.0, 1e10 / ((double)ny * Ly * Lx)));
    nx = (nx + kWaveWarps - 1) / kWaveWarps * kWaveWarps;
    std::vector<int64_t> xoff(nx + 1), yoff(ny + 1);
    for (int i = 0; i <= nx; ++i) xoff[i] = (int64_t)i * Lx;
    for (int j = 0; j <= ny; ++j) yoff[j] = (int64_t)nx * Lx + (int64_t)j * Ly;
    const size_t total = (size_t)nx * Lx + (size_t)ny * Ly;
    std::vector<int8_t> codes(total);
    for (auto& ch : codes) ch = (int8_t)(rnd() % 20);
    if ((rc = probe.ensure(total + sizeof(float) * (size_t)nx * ny))) {
      rc = fail(rc, "autotune probe");
      break;
    }
    int8_t* dcodes = (int8_t*)probe.p;
    float* dD = (float*)((char*)probe.p + ((total + 255) / 256) * 256);
    if ((size_t)((char*)dD - (char*)probe.p) + sizeof(float) * (size_t)nx * ny > probe.cap) {
      probe.release();
      if ((rc = probe.ensure(((total + 255) / 256) * 256 + sizeof(float) * (size_t)nx * ny))) {
        rc = fail(rc, "autotune probe");
        break;
      }
      dcodes = (int8_t*)probe.p;
      dD = (float*)((char*)probe.p + ((total + 255) / 256) * 256);
    }
    if ((rc = cuda(cudaMemcpy(dcodes, codes.data(), total, cudaMemcpyHostToDevice), "autotune upload"))) break;
    double best = 0.0, best_wave = 0.0;   // least estimated time at Ly (padded rows / rate)
    TuneChoice pick = kDefaultTune[k], pick_wave = kDefaultTuneWave[k];
    for (int W : {32, 16, 8, 1})
    for (int R : kCandR) {
      for (int V = 0; V <= 6; ++V) {
        const TuneChoice cand{R, V, W};
        const int Lyc = probe_rows(k, cand);
        if (Lyc == 0 || !wave_exists(R, 2, V, W) || (V == 4 && go < ge)) continue;
        for (int j = 0; j <= ny; ++j) yoff[j] = (int64_t)nx * Lx + (int64_t)j * Lyc;
        tune[k] = cand;
        ++tune_version;
        float ms = 0.f;
        for (int rep = 0; rep < 2 && rc == NWG_OK; ++rep) {
          if ((rc = cuda(cudaEventRecord(ev0, stream), "autotune event"))) break;
          if ((rc = batched(dcodes, xoff.data(), nx, yoff.data(), ny, false, dD, ny, 0, NWG_MODE_BATCHED, nullptr)))
            break;
          if ((rc = cuda(cudaEventRecord(ev1, stream), "autotune event")) ||
              (rc = cuda(cudaEventSynchronize(ev1), "autotune sync")))
            break;
          cudaEventElapsedTime(&ms, ev0, ev1);
        }
        if (rc) break;
        if (!(ms > 0.f)) continue;   // no usable timing: not a candidate
        const double rate = (double)nx * ny * padded_rows(cand, Lyc) * Lx / (ms * 1e-3);
        found[k].push_back({cand, rate});
        const double est = padded_rows(cand, Ly) / rate;
        if (best == 0.0 || est < best) {
          best = est;
          pick = cand;
        }
        if (W >= 8 && (best_wave == 0.0 || est < best_wave)) {
          best_wave = est;
          pick_wave = cand;
        }
      }
      if (rc) break;
    }
    tune[k] = pick;
    tune_wave[k] = pick_wave;
    res.rows_per_lane[k] = pick.R;
    res.variant[k] = pick.V;
    res.lanes[k] = pick.W;
    res.gcups[k] = best > 0.0 ? (double)Ly / best / 1e9 : 0.0;   // the pick's GCUPS on Y of the class bound
  }
  probe.release();
  destroy_plans(this);   // the probe plans are of no further use
  use_graphs = saved_graphs;
  ++tune_version;
  if (rc) {
    for (int k = 0; k < kTuneClasses; ++k) {
      tune[k] = kDefaultTune[k];
      tune_wave[k] = kDefaultTuneWave[k];
    }
    return rc;
  }
  for (int k = 0; k < kTuneClasses; ++k) cands[k] = std::move(found[k]);
  tuned = true;
  res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  make_parent_dirs(path);
  if (FILE* f = std::fopen(path.c_str(), "w")) {
    std::fprintf(f, "%s\n", kCacheTag);
    for (int k = 0; k < kTuneClasses; ++k) {
      std::fprintf(f, "%d %d %d %d %.3f %d %d %d %d", k, tune[k].R, tune[k].V, tune[k].W, res.gcups[k],
                   tune_wave[k].R, tune_wave[k].V, tune_wave[k].W, (int)cands[k].size());
      for (const Cand& c : cands[k]) std::fprintf(f, " %d %d %d %.6g", c.t.R, c.t.V, c.t.W, c.rate);
      std::fprintf(f, "\n");
    }
    std::fclose(f);
  }
  if (out) *out = res;
  return NWG_OK;
}

}  // namespace nwg

extern "C" int nwg_autotune(nwg_ctx* ctx, int flags, nwg_tune_result* out) {
  if (!ctx) return NWG_ERR_INVALID;
  return reinterpret_cast<nwg::Ctx*>(ctx)->autotune((flags & 1) != 0, out);
}

extern "C" int nwg_set_tuning_lanes(nwg_ctx* ctx, const int32_t* rows_per_lane, const int32_t* variant,
                                    const int32_t* lanes) {
  if (!ctx || !rows_per_lane || !variant) return NWG_ERR_INVALID;
  nwg::Ctx* c = reinterpret_cast<nwg::Ctx*>(ctx);
  for (int k = 0; k < nwg::kTuneClasses; ++k)
    if (!nwg::wave_exists(rows_per_lane[k], 2, variant[k], lanes ? lanes[k] : 32)) return NWG_ERR_INVALID;
  for (int k = 0; k < nwg::kTuneClasses; ++k) {
    c->tune[k] = {rows_per_lane[k], variant[k], lanes ? lanes[k] : 32};
    c->cands[k].clear();   // a forced table is used as it is
    // a forced table drives the serving loop too where it names wavefronts
    if (c->tune[k].W >= 8) c->tune_wave[k] = c->tune[k];
  }
  ++c->tune_version;
  c->tuned = true;
  return NWG_OK;
}

extern "C" int nwg_set_tuning(nwg_ctx* ctx, const int32_t* rows_per_lane, const int32_t* variant) {
  return nwg_set_tuning_lanes(ctx, rows_per_lane, variant, nullptr);
}
