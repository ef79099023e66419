// synth.cpp -- seeded synthetic protein families (host only).
//
// The reference ships six real FASTA inputs without expected outputs and
// publishes no benchmark suite; the workloads here are seeded synthetic
// families with the shapes the benchmark configurations name.  A family of k
// sequences is a uniform i.i.d. root evolved down a random binary (Yule) tree:
// repeatedly pick a uniformly chosen current leaf and replace it by two
// mutated copies.  On each edge every site is substituted with probability ps
// by a uniformly chosen different residue, and with probability pi per site an
// indel event happens (insertion or deletion 50/50, length geometric with mean
// 3 and support >= 1, inserted residues uniform).  Lengths are clipped to
// [clip_lo, clip_hi].
//
// PRNG: SplitMix64 seeding xoshiro256**.  Everything but the lognormal root
// length is integer arithmetic, so those families are bit-identical on x86-64
// and aarch64; the lognormal draw uses libm (log/cos/exp) and is documented as
// platform-dependent in rare rounding cases.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/nwgpu_synth.h"

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (int k = 0; k < 4; ++k) {
      z += 0x9E3779B97F4A7C15ull;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
      x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
      s[k] = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform integer in [0, n) by rejection (no modulo bias)
  uint32_t below(uint32_t n) {
    uint64_t lim = (~0ull) - ((~0ull) % n);
    uint64_t v;
    do { v = next(); } while (v >= lim);
    return (uint32_t)(v % n);
  }
  // Bernoulli(p) with p given as a 2^-32 fixed-point threshold
  bool bern(uint32_t thr) { return (uint32_t)(next() >> 32) < thr; }
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

uint32_t to_thr(double p) {
  if (p <= 0) return 0;
  if (p >= 1) return 0xFFFFFFFFu;
  return (uint32_t)(p * 4294967296.0);
}

const char kStd[21] = "ARNDCQEGHILKMFPSTWYV";

int geom_len(Rng& r) {
  // P(len = m) = (2/3)^(m-1) * 1/3: mean 3, support >= 1
  int m = 1;
  while (r.below(3) != 0) ++m;
  return m;
}

void mutate(Rng& r, const std::vector<char>& in, std::vector<char>& out, uint32_t ps, uint32_t pi,
            int lo, int hi) {
  out.clear();
  out.reserve(in.size() + 16);
  size_t k = 0;
  while (k < in.size()) {
    char c = in[k];
    if (r.bern(ps)) {
      char d;
      do { d = kStd[r.below(20)]; } while (d == c);
      c = d;
    }
    if (r.bern(pi)) {
      int m = geom_len(r);
      if (r.below(2) == 0) {         // insertion after this site
        out.push_back(c);
        for (int t = 0; t < m; ++t) out.push_back(kStd[r.below(20)]);
        ++k;
      } else {                       // deletion of m sites starting here
        k += (size_t)m;
      }
      continue;
    }
    out.push_back(c);
    ++k;
  }
  if ((int)out.size() > hi) out.resize((size_t)hi);
  while ((int)out.size() < lo) out.push_back(kStd[r.below(20)]);
}

int root_length(Rng& r, const nws_spec& sp) {
  double v;
  switch (sp.root_mode) {
    case NWS_ROOT_FIXED: v = sp.root_a; break;
    case NWS_ROOT_UNIFORM: {
      int a = (int)sp.root_a, b = (int)sp.root_b;
      v = a + (int)r.below((uint32_t)(b - a + 1));
      break;
    }
    default: {  // lognormal(median root_a, sigma root_b), Box-Muller
      double u1 = r.unit(), u2 = r.unit();
      if (u1 < 1e-300) u1 = 1e-300;
      double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
      v = std::floor(std::exp(std::log(sp.root_a) + sp.root_b * z) + 0.5);
      break;
    }
  }
  int L = (int)v;
  if (L < sp.clip_lo) L = sp.clip_lo;
  if (L > sp.clip_hi) L = sp.clip_hi;
  return L;
}

}  // namespace

extern "C" int nws_generate(const nws_spec* sp, uint64_t seed, nws_out* out) {
  if (!sp || !out || sp->families < 1 || sp->per_family < 1 || sp->clip_lo < 1 ||
      sp->clip_hi < sp->clip_lo)
    return 1;
  std::vector<std::vector<char>> all;
  all.reserve((size_t)sp->families * sp->per_family);
  uint32_t ps = to_thr(sp->ps), pi = to_thr(sp->pi);
  for (int f = 0; f < sp->families; ++f) {
    Rng r(seed * 0x100000001B3ull + (uint64_t)f * 0x9E3779B97F4A7C15ull + 1);
    int L = root_length(r, *sp);
    std::vector<char> root((size_t)L);
    for (int k = 0; k < L; ++k) root[(size_t)k] = kStd[r.below(20)];
    std::vector<std::vector<char>> leaves;
    leaves.push_back(root);
    std::vector<char> a, b;
    while ((int)leaves.size() < sp->per_family) {
      uint32_t pick = r.below((uint32_t)leaves.size());
      mutate(r, leaves[pick], a, ps, pi, sp->clip_lo, sp->clip_hi);
      mutate(r, leaves[pick], b, ps, pi, sp->clip_lo, sp->clip_hi);
      leaves[pick].swap(a);
      leaves.push_back(b);
    }
    if (sp->per_family == 1) {
      // a family of one is its (clipped) root
      if ((int)leaves[0].size() > sp->clip_hi) leaves[0].resize((size_t)sp->clip_hi);
    }
    for (auto& s : leaves) all.push_back(s);
  }
  int64_t total = 0;
  for (auto& s : all) total += (int64_t)s.size();
  out->n = (int32_t)all.size();
  out->total = total;
  out->residues = (char*)std::malloc((size_t)(total > 0 ? total : 1));
  out->lengths = (int32_t*)std::malloc(sizeof(int32_t) * all.size());
  if (!out->residues || !out->lengths) return 2;
  int64_t off = 0;
  for (size_t k = 0; k < all.size(); ++k) {
    std::memcpy(out->residues + off, all[k].data(), all[k].size());
    out->lengths[k] = (int32_t)all[k].size();
    off += (int64_t)all[k].size();
  }
  return 0;
}

extern "C" void nws_release(nws_out* out) {
  if (!out) return;
  std::free(out->residues);
  std::free(out->lengths);
  out->residues = nullptr;
  out->lengths = nullptr;
  out->n = 0;
  out->total = 0;
}

extern "C" int nws_config_spec(int cfg, nws_spec* sp) {
  // The five workload shapes of the benchmark configurations.
  std::memset(sp, 0, sizeof(*sp));
  sp->clip_lo = 1;
  sp->clip_hi = 4000;
  switch (cfg) {
    case 0: sp->families = 1; sp->per_family = 64; sp->root_mode = NWS_ROOT_FIXED; sp->root_a = 300;
            sp->ps = 0.05; sp->pi = 0.005; return 0;
    case 1: sp->families = 10; sp->per_family = 200; sp->root_mode = NWS_ROOT_FIXED; sp->root_a = 450;
            sp->ps = 0.08; sp->pi = 0.005; return 0;
    case 2: sp->families = 50; sp->per_family = 200; sp->root_mode = NWS_ROOT_LOGNORMAL;
            sp->root_a = 350; sp->root_b = 0.6; sp->clip_lo = 30; sp->clip_hi = 4000;
            sp->ps = 0.1; sp->pi = 0.01; return 0;
    case 3: sp->families = 40; sp->per_family = 200; sp->root_mode = NWS_ROOT_UNIFORM;
            sp->root_a = 100; sp->root_b = 300; sp->ps = 0.05; sp->pi = 0.005; return 0;
    default: return 1;
  }
}

extern "C" uint64_t nws_config_seed(int cfg) { return 0x6D657374ull + (uint64_t)cfg; }
