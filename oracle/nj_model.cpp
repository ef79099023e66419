/*
 * nj_model.cpp -- neighbor joining as the reference's buildTree runs it, with
 * its bins, bin heaps, candidate list and prediction array.
 *
 * TEST INFRASTRUCTURE ONLY (the library never links it).  nwo_nj in
 * nw_oracle.c picks each join by the exact argmin of q in one rounding; the
 * reference instead values a pair in one of two roundings depending on where
 * the pair sits when the join is chosen, and keeps only eight candidates
 * (SpeciesBlock.cpp:1019-1180).  On inputs where that choice decides the join
 * (tie-heavy matrices: duplicated sequences) only a model of those data
 * structures gives the reference's tree.  This file restates them:
 *
 *   buildGblRowSums  SpeciesBlock.cpp:426-453   row sums, ascending id order
 *   buildBins        :456-674                   T quantile bins, one heap per
 *                                               bin pair, bin visiting order
 *   buildTree        :845-1343                  per join: bin maxima (:996-
 *                                               1013), candidate list scan
 *                                               (:1019-1068), return of stale
 *                                               candidates every 50 joins
 *                                               (:1070-1091), compaction
 *                                               (:1093-1099), heap pops
 *                                               (:1102-1144), the eight kept
 *                                               (:1145-1151) and the final
 *                                               pick (:1160-1180), rebuild
 *                                               schedule (:1204-1247), new
 *                                               pairs into heaps (:1249-1297),
 *                                               prediction update (:1299-1319)
 *   modifyMatrix     :710-842                   new row, T updates
 *   TreeNode::join   TreeNode.cpp:31-58         branch lengths
 *
 * with one rank and the reference's defaults (CmdLineOptions.cpp:37-48:
 * 30 bins, 8 kept candidates, prediction on, allgather pick, rebuild ratio
 * 0.5, heap ratio 2.0; duplicate removal has no zero distances to act on,
 * SpeciesBlock.cpp:884-981).
 *
 * The containers and algorithms are the reference's own (std::priority_queue,
 * std::nth_element, std::partition, std::partial_sort, std::multimap), taken
 * from the same C++ standard library, so every order the reference leaves to
 * its library -- which of more than eight tied candidates survive the cut,
 * the pop order of equal distances in a heap -- is the reference's.  Checked
 * against the reference's own buildTree compiled from its sources
 * (tests/test_nj_model_cpu.py).
 */
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <queue>
#include <vector>

#include "nw_oracle.h"

namespace {

constexpr int kBins = 30;                       // clustSize (CmdLineOptions.cpp:41)
constexpr int kBinT = kBins * (kBins + 1) / 2;  // bin pairs, one rank: all local
constexpr int kQDA = 8;                         // qda (:42)
constexpr int kQDASZ = 512;                     // SpeciesBlock.cpp:847
constexpr int kPqRatioInit = 500;               // :848
constexpr int kCandidateScan = 50;              // :849
constexpr int kMinRebuild = 200;                // :5
constexpr float kRatio = 0.5f;                  // rebuildRatio (CmdLineOptions.cpp:40)
constexpr float kPqRatio = 2.0f;                // pqRatio (:39)

struct Dij {
  float d;
  int i, j;
};
struct ADij {
  float d;
  int i, j;
  bool active;
};
struct QDij {
  float d = FLT_MAX;
  int i = -1, j = -1;
  double q = DBL_MAX;
};

// the reference's heap order (structs.h:121-128): smallest d on top
struct DijCompare {
  bool operator()(const Dij& a, const Dij& b) const { return a.d > b.d; }
};
struct QCompare {
  bool operator()(const QDij& a, const QDij& b) const { return a.q < b.q; }
};

using Heap = std::priority_queue<Dij, std::vector<Dij>, DijCompare>;

class Model {
 public:
  Model(float* D, int n) : D_(D), n0_(n) {}

  void run(nwo_join* joins, nwo_nj_model_stats* st);

 private:
  float& d(int a, int b) { return D_[(int64_t)a * n0_ + b]; }
  void row_sums();
  void build_bins();
  void keep_eight();       // :1145-1151 + :1155
  void pick(QDij& minQ);   // :1160-1180
  void join(const QDij& minQ, nwo_join* J);
  void predict_update();   // :1299-1319

  float* D_;
  int n0_, nn_ = 0, next_ = 0, n_ = 0;
  std::vector<double> T_;
  std::vector<int> slot_, act_, bin_loc_;
  std::vector<float> vd_;
  double bin_range_[kBins], max_t2_[kBins];
  int pair_a_[kBinT], pair_b_[kBinT], idx_[kBins][kBins], bin_order_[kBinT];
  std::vector<Heap> pq_;
  std::vector<ADij> adij_;
  std::vector<QDij> qdA_, qdAg_;
  int nq_ = 0;
  nwo_nj_model_stats st_{};
};

void Model::row_sums() {
  for (int a : act_) {
    const int ra = slot_[a];
    double sum = 0.0;
    for (int b : act_) sum += d(ra, slot_[b]);
    T_[ra] = sum;
  }
}

void Model::build_bins() {
  for (auto& h : pq_) h = Heap();
  double tmin = DBL_MAX, tmax = -DBL_MAX;
  std::vector<double> Tv;
  Tv.reserve(act_.size());
  for (int a : act_) {
    const double t = T_[slot_[a]];
    Tv.push_back(t);
    tmax = t > tmax ? t : tmax;
    tmin = t < tmin ? t : tmin;
  }
  (void)tmin;
  const int rem = n_ % kBins, rdel = n_ / kBins;
  int ir = rdel;
  std::sort(Tv.begin(), Tv.end());
  bin_range_[kBins - 1] = tmax;
  for (int b = 0; b < kBins - 1; ++b) {
    const int irn = std::min(ir + 1, n_ - 1);
    // Below 29 active nodes the reference reads T[m_n], past its vector
    // (:491-494), for the upper bins; the model clamps to the last value.
    if (ir > n_ - 1) ++st_.out_of_range_bins;
    const int irc = std::min(ir, n_ - 1);
    bin_range_[b] = 0.5 * (Tv[(size_t)irc] + Tv[(size_t)irn]);
    ir += rdel + (rem > b);
  }
  for (int a : act_) {
    const int ra = slot_[a];
    int lb = (int)(std::lower_bound(bin_range_, bin_range_ + kBins, T_[ra]) - bin_range_);
    if (lb >= kBins) lb = kBins - 1;
    bin_loc_[ra] = lb;
  }
  // every live pair into its bin pair's heap, in the send-buffer order
  // (:545-561): i ascending, j after i
  for (size_t x = 0; x < act_.size(); ++x) {
    const int i = act_[x], ri = slot_[i];
    for (size_t y = x + 1; y < act_.size(); ++y) {
      const int j = act_[y], rj = slot_[j];
      pq_[(size_t)idx_[bin_loc_[ri]][bin_loc_[rj]]].push(Dij{d(ri, rj), i, j});
    }
  }
  // visiting order: descending bin_range[a] + bin_range[b], ties in bin order
  std::multimap<double, int, std::greater<double> > mm;
  for (int l = 0; l < kBinT; ++l) mm.insert(std::make_pair(bin_range_[pair_a_[l]] + bin_range_[pair_b_[l]], l));
  int c = 0;
  for (auto& kv : mm) bin_order_[c++] = kv.second;
}

void Model::keep_eight() {
  std::nth_element(qdA_.begin(), qdA_.begin() + std::min(nq_, kQDA), qdA_.begin() + nq_, QCompare());
  for (int k = nq_; k < kQDA; ++k) qdA_[(size_t)k].q = DBL_MAX;
}

void Model::pick(QDij& minQ) {
  // MPI_Allgather of the eight (one rank: a copy), then the tie-break loop
  // :1164-1179 -- smallest q, then largest max(i,j), then largest min(i,j)
  for (int k = 0; k < kQDA; ++k) qdAg_[(size_t)k] = qdA_[(size_t)k];
  minQ.q = DBL_MAX;
  int minI = INT_MAX, minJ = INT_MAX;
  for (int k = 0; k < kQDA; ++k) {
    const QDij& c = qdAg_[(size_t)k];
    if (c.q <= minQ.q) {
      const int ni = std::min(c.i, c.j), nj = std::max(c.i, c.j);
      if (c.q < minQ.q || minJ < nj || (minJ == nj && minI < ni)) {
        minQ = c;
        minI = std::min(minQ.i, minQ.j);
        minJ = std::max(minQ.i, minQ.j);
      }
    }
  }
}

void Model::join(const QDij& mq, nwo_join* J) {
  const int i = std::min(mq.i, mq.j), j = std::max(mq.i, mq.j);
  const int ri = slot_[i], rj = slot_[j];
  const double Ti = T_[ri], Tj = T_[rj];
  // TreeNode::join (TreeNode.cpp:31-58)
  double li, lj;
  const double half = 0.5;
  if (n_ == 2) {
    li = lj = mq.d * half;
  } else {
    li = half * (mq.d + (Ti - Tj) / (n_ - 2));
    lj = half * (mq.d + (Tj - Ti) / (n_ - 2));
  }
  if (li < 0.0) {
    lj -= li;
    li = 0.0;
  } else if (lj < 0.0) {
    li -= lj;
    lj = 0.0;
  }
  J->i = i;
  J->j = j;
  J->node = next_;
  J->n = n_;
  J->d = mq.d;
  J->pad = 0.f;
  J->q = mq.q;
  J->ti = Ti;
  J->tj = Tj;
  J->len_i = li;
  J->len_j = lj;
  // modifyMatrix (:710-842)
  act_.erase(std::remove_if(act_.begin(), act_.end(), [&](int k) { return k == i || k == j; }), act_.end());
  slot_[i] = slot_[j] = -1;
  double sum = 0.0;
  for (int k : act_) {
    const int rk = slot_[k];
    const float Dik = d(ri, rk), Djk = d(rj, rk);
    const float tmp = ((Dik + Djk) - mq.d) / 2;
    sum += tmp;
    vd_[(size_t)rk] = tmp;
    T_[rk] += tmp - (Dik + Djk);
  }
  T_[ri] = sum;
  for (int k : act_) {
    const int rk = slot_[k];
    d(rk, ri) = vd_[(size_t)rk];
    d(ri, rk) = vd_[(size_t)rk];
  }
}

void Model::predict_update() {
  for (auto& qd : qdAg_) {
    int ri, rj;
    if (qd.i < 0 || qd.j < 0 || (ri = slot_[qd.i]) == -1 || (rj = slot_[qd.j]) == -1) {
      qd.q = DBL_MAX;
      continue;
    }
    qd.q = ((double)qd.d) * (n_ - 2) - T_[ri] - T_[rj];
  }
  std::partial_sort(qdAg_.begin(), qdAg_.begin() + kQDA, qdAg_.end(), QCompare());
  qdA_[0] = qdAg_[0];
  int jc = 0;
  for (int k = 1; k < kQDA; ++k) {
    if ((qdA_[(size_t)jc].i != qdAg_[(size_t)k].i || qdA_[(size_t)jc].j != qdAg_[(size_t)k].j) &&
        qdAg_[(size_t)k].q != DBL_MAX) {
      qdA_[(size_t)++jc] = qdAg_[(size_t)k];
      if (jc == kQDA - 1) break;
    }
  }
  nq_ = jc + 1;
}

void Model::run(nwo_join* joins, nwo_nj_model_stats* st) {
  if (n0_ <= 1) {
    if (st) *st = st_;
    return;
  }
  nn_ = 2 * n0_ - 1;
  next_ = n0_;
  n_ = n0_;
  T_.assign((size_t)n0_, 0.0);
  vd_.assign((size_t)n0_, 0.f);
  slot_.assign((size_t)nn_, -1);
  bin_loc_.assign((size_t)n0_, 0);
  for (int k = 0; k < n0_; ++k) {
    slot_[(size_t)k] = k;
    act_.push_back(k);
  }
  int g = 0;
  for (int a = 0; a < kBins; ++a)
    for (int b = a; b < kBins; ++b) {
      idx_[a][b] = idx_[b][a] = g;
      pair_a_[g] = a;
      pair_b_[g] = b;
      ++g;
    }
  pq_.assign(kBinT, Heap());
  qdA_.assign(kQDASZ, QDij());
  qdAg_.assign(kQDA, QDij());
  adij_.reserve(1000);

  row_sums();
  build_bins();
  int steps = std::max((int)(n_ * kRatio), kMinRebuild);
  int pq_ck = kPqRatioInit;
  long sz0 = n_;
  long ave0 = (((sz0 - 1) * sz0) / 2) / kBinT;

  while (next_ < nn_) {
    QDij minQ = qdA_[0];
    // bin maxima and second maxima over the active nodes (:996-1013)
    for (int b = 0; b < kBins; ++b) bin_range_[b] = max_t2_[b] = -DBL_MAX;
    for (int k : act_) {
      const int rk = slot_[k], b = bin_loc_[rk];
      if (T_[rk] > max_t2_[b]) {
        if (T_[rk] > bin_range_[b]) {
          max_t2_[b] = bin_range_[b];
          bin_range_[b] = T_[rk];
        } else {
          max_t2_[b] = T_[rk];
        }
      }
    }
    auto max_tsum = [&](int a, int b) { return bin_range_[a] + ((a == b) ? max_t2_[a] : bin_range_[b]); };
    auto push_q = [&](const QDij& e) {
      qdA_[(size_t)nq_++] = e;
      if (nq_ == kQDASZ) {
        std::nth_element(qdA_.begin(), qdA_.begin() + kQDA, qdA_.begin() + nq_, QCompare());
        nq_ = kQDA;
      }
    };
    // drop inactive, dead candidates from the end (:1019-1035)
    {
      int last = (int)adij_.size() - 1, c;
      for (c = last; c >= 0; --c) {
        ADij& a = adij_[(size_t)c];
        if (a.active) break;
        if (slot_[a.i] != -1 && slot_[a.j] != -1) break;
        a.active = false;
      }
      if (c != last) adij_.erase(adij_.begin() + (c + 1), adij_.end());
    }
    // scan the candidate list, newest first (:1037-1068)
    unsigned inactive = 0;
    for (int c = (int)adij_.size() - 1; c >= 0; --c) {
      ADij& a = adij_[(size_t)c];
      if (!a.active) {
        ++inactive;
        continue;
      }
      const int ri = slot_[a.i], rj = slot_[a.j];
      if (ri == -1 || rj == -1) {
        a.active = false;
      } else {
        const double q = ((double)a.d) * (n_ - 2) - T_[ri] - T_[rj];
        if (q <= minQ.q) {
          minQ = QDij{a.d, a.i, a.j, q};
          push_q(minQ);
        }
      }
    }
    // every 50 joins, return candidates that cannot win to their heaps (:1070-1091)
    if ((n0_ - n_) % kCandidateScan == 0 && steps > kCandidateScan / 2) {
      for (int c = (int)adij_.size() - 1; c >= 0; --c) {
        ADij& a = adij_[(size_t)c];
        if (!a.active) continue;
        const int ri = slot_[a.i], rj = slot_[a.j];
        const int bi = bin_loc_[ri], bj = bin_loc_[rj];
        const double qlim = ((double)a.d) * (n_ - 2) - max_tsum(bi, bj);
        if (qlim > minQ.q) {
          a.active = false;
          pq_[(size_t)idx_[bi][bj]].push(Dij{a.d, a.i, a.j});
        }
      }
    }
    // compaction when a fifth is inactive (:1093-1099)
    if (!adij_.empty() && inactive > adij_.size() / 5) {
      auto good = std::partition(adij_.begin(), adij_.end(), [](const ADij& a) { return a.active; });
      adij_.erase(good, adij_.end());
    }
    // pop the bin heaps in visiting order (:1102-1144)
    for (int jb = 0; jb < kBinT; ++jb) {
      const int l = bin_order_[jb];
      Heap& pq = pq_[(size_t)l];
      const double mts = max_tsum(pair_a_[l], pair_b_[l]);
      while (!pq.empty()) {
        const Dij top = pq.top();
        const int ri = slot_[top.i], rj = slot_[top.j];
        if (ri == -1 || rj == -1) {
          pq.pop();
          continue;
        }
        double q = ((double)top.d) * (n_ - 2);
        const double qlim = q - mts;
        q -= T_[ri] + T_[rj];
        if (qlim > minQ.q) break;
        push_q(QDij{top.d, top.i, top.j, q});
        if (q <= minQ.q) minQ = QDij{top.d, top.i, top.j, q};
        adij_.push_back(ADij{top.d, top.i, top.j, true});
        pq.pop();
      }
    }
    keep_eight();
    pick(minQ);
    const int keep = slot_[std::min(minQ.i, minQ.j)];   // the new node's slot
    join(minQ, &joins[next_ - n0_]);

    // heap occupancy check every 500 joins (:1204-1223)
    if (--pq_ck == 0) {
      pq_ck = kPqRatioInit;
      if (steps > 0) {
        long total = 0;
        for (auto& h : pq_) total += (long)h.size();
        total = total / (long)kBinT;
        const double r = (double)total / (double)ave0;
        if (r > kPqRatio) {
          steps = 0;
          ++st_.pq_triggers;
        }
      }
    }
    --n_;
    if (steps == 0) {
      slot_[(size_t)next_] = keep;
      act_.push_back(next_);
      ++next_;
      adij_.clear();
      row_sums();
      build_bins();
      ++st_.rebuilds;
      steps = (n_ < kMinRebuild) ? INT_MAX : (int)(n_ * kRatio);
      sz0 = n_;
      ave0 = (((sz0 - 1) * sz0) / 2) / kBinT;
    } else {
      --steps;
      // the new node's bin from this join's maxima (:1255-1261); above every
      // maximum the slot keeps its previous bin
      for (int b = 0; b < kBins; ++b)
        if (T_[keep] <= bin_range_[b]) {
          bin_loc_[keep] = b;
          break;
        }
      const int bi = bin_loc_[keep];
      slot_[(size_t)next_] = keep;
      for (int k : act_) {
        const int rk = slot_[k];
        const int a = rk < keep ? k : next_, b = rk < keep ? next_ : k;
        pq_[(size_t)idx_[bi][bin_loc_[rk]]].push(Dij{vd_[(size_t)rk], a, b});
      }
      act_.push_back(next_);
      ++next_;
    }
    predict_update();
  }
  if (st) *st = st_;
}

}  // namespace

extern "C" void nwo_nj_model(float* D, int n, nwo_join* joins, nwo_nj_model_stats* stats) {
  Model m(D, n);
  m.run(joins, stats);
}
