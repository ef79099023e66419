/*
 * nw_oracle.c -- CPU restatement of the ptersnow/mestrado hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle.  The product library never
 * links or calls it.  Every function names the reference file:line it
 * restates; the reference's GPU code itself does not build on CUDA 13 and is
 * defective as shipped, so the contract is the reference's recurrence on
 * correctly encoded inputs.
 *
 * Parity pin: nwo_score_pair/nwo_traceback against hand-derived known-answer
 * tests (tests/test_oracle.py); nwo_nj against the reference's own
 * SpeciesBlock::buildTree compiled from its sources through a one-rank MPI
 * shim (oracle/ref_shim -> oracle/_ref/ref_nj) and the golden join lists that
 * run produced (tests/golden/).
 *
 * Built with -O2 -ffp-contract=off so that no multiply-add is fused: the
 * reference was built for x86-64 without FMA.
 */
#include "nw_oracle.h"

#include <limits.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Residue order of AlignmentScore::conversion (AlignmentScore.cu:10-27) and
 * revConvConst (definitions.cuh:134-137): code k is the k-th letter. */
static const char kOrder[NWO_LETTERS + 1] = "ARNDCQEGHILKMFPSTWYVBZX*";

/* definitions.cuh:96-121 (identical to blosum64.txt:1-24; BLOSUM62 values),
 * rows and columns in kOrder. */
static const int8_t kBlosum[NWO_LETTERS * NWO_LETTERS] = {
   4,-1,-2,-2, 0,-1,-1, 0,-2,-1,-1,-1,-1,-2,-1, 1, 0,-3,-2, 0,-2,-1, 0,-4,
  -1, 5, 0,-2,-3, 1, 0,-2, 0,-3,-2, 2,-1,-3,-2,-1,-1,-3,-2,-3,-1, 0,-1,-4,
  -2, 0, 6, 1,-3, 0, 0, 0, 1,-3,-3, 0,-2,-3,-2, 1, 0,-4,-2,-3, 3, 0,-1,-4,
  -2,-2, 1, 6,-3, 0, 2,-1,-1,-3,-4,-1,-3,-3,-1, 0,-1,-4,-3,-3, 4, 1,-1,-4,
   0,-3,-3,-3, 9,-3,-4,-3,-3,-1,-1,-3,-1,-2,-3,-1,-1,-2,-2,-1,-3,-3,-2,-4,
  -1, 1, 0, 0,-3, 5, 2,-2, 0,-3,-2, 1, 0,-3,-1, 0,-1,-2,-1,-2, 0, 3,-1,-4,
  -1, 0, 0, 2,-4, 2, 5,-2, 0,-3,-3, 1,-2,-3,-1, 0,-1,-3,-2,-2, 1, 4,-1,-4,
   0,-2, 0,-1,-3,-2,-2, 6,-2,-4,-4,-2,-3,-3,-2, 0,-2,-2,-3,-3,-1,-2,-1,-4,
  -2, 0, 1,-1,-3, 0, 0,-2, 8,-3,-3,-1,-2,-1,-2,-1,-2,-2, 2,-3, 0, 0,-1,-4,
  -1,-3,-3,-3,-1,-3,-3,-4,-3, 4, 2,-3, 1, 0,-3,-2,-1,-3,-1, 3,-3,-3,-1,-4,
  -1,-2,-3,-4,-1,-2,-3,-4,-3, 2, 4,-2, 2, 0,-3,-2,-1,-2,-1, 1,-4,-3,-1,-4,
  -1, 2, 0,-1,-3, 1, 1,-2,-1,-3,-2, 5,-1,-3,-1, 0,-1,-3,-2,-2, 0, 1,-1,-4,
  -1,-1,-2,-3,-1, 0,-2,-3,-2, 1, 2,-1, 5, 0,-2,-1,-1,-1,-1, 1,-3,-1,-1,-4,
  -2,-3,-3,-3,-2,-3,-3,-3,-1, 0, 0,-3, 0, 6,-4,-2,-2, 1, 3,-1,-3,-3,-1,-4,
  -1,-2,-2,-1,-3,-1,-1,-2,-2,-3,-3,-1,-2,-4, 7,-1,-1,-4,-3,-2,-2,-1,-2,-4,
   1,-1, 1, 0,-1, 0, 0, 0,-1,-2,-2, 0,-1,-2,-1, 4, 1,-3,-2,-2, 0, 0, 0,-4,
   0,-1, 0,-1,-1,-1,-1,-2,-2,-1,-1,-1,-1,-2,-1, 1, 5,-2,-2, 0,-1,-1, 0,-4,
  -3,-3,-4,-4,-2,-2,-3,-2,-2,-3,-2,-3,-1, 1,-4,-3,-2,11, 2,-3,-4,-3,-2,-4,
  -2,-2,-2,-3,-2,-1,-2,-3, 2,-1,-1,-2,-1, 3,-3,-2,-2, 2, 7,-1,-3,-2,-1,-4,
   0,-3,-3,-3,-1,-2,-2,-3,-3, 3, 1,-2, 1,-1,-2,-2, 0,-3,-1, 4,-3,-2,-1,-4,
  -2,-1, 3, 4,-3, 0, 1,-1, 0,-3,-4, 0,-3,-3,-2, 0,-1,-4,-3,-3, 4, 1,-1,-4,
  -1, 0, 0, 1,-3, 3, 4,-2, 0,-3,-3, 1,-1,-3,-1, 0,-1,-3,-2,-2, 1, 4,-1,-4,
   0,-1,-1,-1,-2,-1,-1,-1,-1,-1,-1,-1,-1,-1,-2, 0, 0,-2,-1,-1,-1,-1,-1,-4,
  -4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4, 1,
};

const int8_t* nwo_blosum(void) { return kBlosum; }

void nwo_conversion_table(int8_t out[256]) {
  for (int c = 0; c < 256; ++c) out[c] = -1;
  for (int k = 0; k < NWO_LETTERS; ++k) out[(unsigned char)kOrder[k]] = (int8_t)k;
}

int nwo_encode_reverse(const char* ascii, int len, int8_t* out) {
  int8_t tab[256];
  int bad = 0;
  nwo_conversion_table(tab);
  /* AlignmentScore.cu:168-177 swaps ends while encoding; the intended result
   * is the fully encoded, fully reversed sequence. */
  for (int i = 0; i < len; ++i) {
    int8_t c = tab[(unsigned char)ascii[len - 1 - i]];
    if (c < 0) ++bad;
    out[i] = c;
  }
  return bad;
}

int nwo_parse_wire(const char* buf, int n, int8_t* codes, int64_t* offsets) {
  /* SpeciesBlock.cpp:309-322 writes the block and AlignmentScore::parse
   * (AlignmentScore.cu:149-166)
   * walk: skip the leading rank int, then per sequence skip seqNo, read
   * len, take len chars and step over the NUL. */
  const char* p = buf + sizeof(int);
  int bad = 0;
  int64_t off = 0;
  offsets[0] = 0;
  for (int s = 0; s < n; ++s) {
    int len;
    p += sizeof(int);
    memcpy(&len, p, sizeof(int));
    p += sizeof(int);
    bad += nwo_encode_reverse(p, len, codes + off);
    p += len + 1;
    off += len;
    offsets[s + 1] = off;
  }
  return bad;
}

static inline int imax(int a, int b) { return a > b ? a : b; }

int nwo_score_pair(const int8_t* x, int lx, const int8_t* y, int ly,
                   int go, int ge, const int8_t* sub) {
  /* NeedlemanWunsch.cu:22-161.  Names follow the kernel: AFh/AFf are the
   * (H, F) halves of AF[] (one per X column, carried from strip to strip),
   * AEh/AEe the (H, E) halves of AE_shared[] (one per strip row, carried from
   * column to column), upleft the A_init_upleft pair.  The kernel keeps these
   * in 16-bit storage; for every input whose values fit in 16 bits (all
   * lengths this project accepts, see the int16 bound in nwg_score) the int32
   * arithmetic here gives the same numbers. */
  enum { YSTEPS = 12 };
  const int kShortMin = -32768;
  int* AFh = (int*)malloc(sizeof(int) * (size_t)(lx > 0 ? lx : 1));
  int* AFf = (int*)malloc(sizeof(int) * (size_t)(lx > 0 ? lx : 1));
  int AEh[YSTEPS], AEe[YSTEPS];
  int hcur = 0;
  for (int c = 0; c < lx; ++c) {            /* :65-70 */
    AFh[c] = -ge * (c + 1);
    AFf[c] = kShortMin + ge;
  }
  for (int y0 = 0; y0 < ly; y0 += YSTEPS) { /* :87 */
    int upleft_x = -ge * y0;                /* :89 */
    for (int i = 0; i < YSTEPS; ++i) {      /* :94-99 */
      AEh[i] = -ge * (y0 + i + 1);
      AEe[i] = kShortMin + ge;
    }
    int ymin = ly - y0 < YSTEPS ? ly - y0 : YSTEPS;
    for (int c = 0; c < lx; ++c) {          /* :112 */
      int upleft_y = upleft_x;              /* :115 */
      int xc = x[c];
      int hup = AFh[c];                     /* :121-126 */
      hcur = hup;
      upleft_x = hup;
      int f = AFf[c];
      for (int i = 0; i < ymin; ++i) {      /* :137-150 */
        int s = sub[y[y0 + i] * NWO_LETTERS + xc];
        f = imax(f - ge, hcur - go);
        int e = imax(AEe[i] - ge, AEh[i] - go);
        hcur = imax(e, f);
        hcur = imax(hcur, s + upleft_y);
        upleft_y = AEh[i];
        AEh[i] = hcur;
        AEe[i] = e;
      }
      AFh[c] = hcur;                        /* :152-155 */
      AFf[c] = f;
    }
  }
  free(AFh);
  free(AFf);
  return hcur;                              /* :160 */
}

void nwo_score_all(const int8_t* codes, const int64_t* offsets, int n,
                   int go, int ge, const int8_t* sub, float* D, int64_t ld,
                   int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int i = 0; i < n; ++i) {
    const int8_t* xi = codes + offsets[i];
    int li = (int)(offsets[i + 1] - offsets[i]);
    for (int j = i; j < n; ++j) {
      const int8_t* yj = codes + offsets[j];
      int lj = (int)(offsets[j + 1] - offsets[j]);
      /* D[x][y] = score(X = seq x, Y = seq y) (AlignmentScore.cu:262-264);
       * the score is symmetric so both halves get the same value. */
      int s = nwo_score_pair(xi, li, yj, lj, go, ge, sub);
      D[(int64_t)i * ld + j] = (float)s;
      D[(int64_t)j * ld + i] = (float)s;
    }
  }
  (void)threads;
}

void nwo_score_list(const int8_t* codes, const int64_t* offsets,
                    const int32_t* pi, const int32_t* pj, int64_t npairs,
                    int go, int ge, const int8_t* sub, int32_t* out, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t k = 0; k < npairs; ++k) {
    int i = pi[k], j = pj[k];
    out[k] = nwo_score_pair(codes + offsets[i], (int)(offsets[i + 1] - offsets[i]),
                            codes + offsets[j], (int)(offsets[j + 1] - offsets[j]),
                            go, ge, sub);
  }
  (void)threads;
}

/* ------------------------------------------------------------------------ */
/* Traceback                                                                 */
/* ------------------------------------------------------------------------ */

/* 32-bit BACK(x, y) word of NeedlemanWunsch.cu:182/233-240/329-359: rows of
 * one 8-row strip at one column, row k of the strip in bits (7-k)*4, rows past
 * the end zero; row -1 holds 9 (left + continue-left), column -1 holds
 * 0x66666666 (up + continue-up), the corner holds 0 (stop). */
static uint32_t back_word(const uint8_t* nib, int lx, int ly, int x, int y) {
  if (y == -1) return x == -1 ? 0u : 9u;
  if (x == -1) return 0x66666666u;
  int r0 = (y / 8) * 8;
  uint32_t w = 0;
  for (int k = 0; k < 8; ++k) {
    w <<= 4;
    if (r0 + k < ly) w |= nib[(size_t)(r0 + k) * lx + x];
  }
  return w;
}

int nwo_traceback(const int8_t* x, int lx, const int8_t* y, int ly,
                  int go, int ge, const int8_t* sub,
                  char* outx, char* outy, int* score) {
  const int kShortMin = -32768;
  uint8_t* nib = (uint8_t*)malloc((size_t)lx * ly + 1);
  int* Hrow = (int*)malloc(sizeof(int) * (size_t)lx);
  int* Frow = (int*)malloc(sizeof(int) * (size_t)lx);
  /* Nibble fill, NeedlemanWunschGlobalMatchKernel (:184-365), cell by cell:
   * the values are those of the score kernel; the flags are
   *   bit3 L  = (H==E && H!=F) || H==diag        (:330)
   *   bit2 U  = H==F || H==diag                  (:332)
   *   bit1 cU = F == F_up - ge                   (:315-316, :334)
   *   bit0 cL = E == E_left - ge                 (:336)                    */
  for (int c = 0; c < lx; ++c) { Hrow[c] = -ge * (c + 1); Frow[c] = kShortMin + ge; }
  int h = 0;
  for (int r = 0; r < ly; ++r) {
    int hleft = -ge * (r + 1);        /* H[r][-1] */
    int eleft = kShortMin + ge;       /* E[r][-1] */
    int diag = (r == 0) ? 0 : -ge * r;/* H[r-1][-1] */
    for (int c = 0; c < lx; ++c) {
      int hup = Hrow[c];
      int fup = Frow[c];
      int f = imax(fup - ge, hup - go);
      int cu = (f == fup - ge);
      int e = imax(eleft - ge, hleft - go);
      int cl = (e == eleft - ge);
      int sim = diag + sub[y[r] * NWO_LETTERS + x[c]];
      h = imax(e, f);
      h = imax(h, sim);
      int L = ((h == e) && (h != f)) || (h == sim);
      int U = (h == f) || (h == sim);
      nib[(size_t)r * lx + c] = (uint8_t)((L << 3) | (U << 2) | (cu << 1) | cl);
      diag = hup;
      Hrow[c] = h;
      Frow[c] = f;
      hleft = h;
      eleft = e;
    }
  }
  if (score) *score = h;

  /* Backtrace, NeedlemanWunschGlobalBackKernel (:393-494), including its
   * word-reload rule: an up move reloads BACK only when y crosses into the
   * previous strip ((y % 8) == 7 in C arithmetic), so an up move out of row 0
   * finds an empty word and stops (:451-458). */
  static const char kDec[NWO_LETTERS + 1] = "ARNDCQEGHILKMFPSTWYVBZX*";
  int px = lx - 1, py = ly - 1, k = 0;
  uint32_t b8 = back_word(nib, lx, ly, px, py) >> ((((8 - ((py + 1) % 8)) % 8)) * 4);
  unsigned prev = 12u;
  unsigned b1 = b8 & 15u;
  b8 >>= 4;
  while (b1 & 12u) {
    unsigned todo;
    if (((prev & 12u) == 4u) && (prev & 2u)) todo = 4u;
    else if (((prev & 12u) == 8u) && (prev & 1u)) todo = 8u;
    else if ((b1 & 12u) == 4u) todo = 4u;
    else if ((b1 & 12u) == 8u) todo = 8u;
    else todo = 12u;
    if (todo == 8u) {
      outx[k] = kDec[(int)x[px]];
      outy[k] = '-';
      --px;
      b8 = back_word(nib, lx, ly, px, py) >> ((((8 - ((py + 1) % 8)) % 8)) * 4);
    } else if (todo == 4u) {
      outx[k] = '-';
      outy[k] = kDec[(int)y[py]];
      --py;
      if ((py % 8) == 7) b8 = back_word(nib, lx, ly, px, py);
    } else {
      outx[k] = kDec[(int)x[px]];
      outy[k] = kDec[(int)y[py]];
      --px;
      --py;
      b8 = back_word(nib, lx, ly, px, py) >> ((((8 - ((py + 1) % 8)) % 8)) * 4);
    }
    prev = todo | (b1 & 3u);
    b1 = b8 & 15u;
    b8 >>= 4;
    ++k;
  }
  outx[k] = 0;
  outy[k] = 0;
  free(nib);
  free(Hrow);
  free(Frow);
  return k;
}

/* ------------------------------------------------------------------------ */
/* Neighbor joining                                                          */
/* ------------------------------------------------------------------------ */

/* The reference's q for a pair held in its candidate list or prediction
 * array, ((double)d*(n-2) - T[a]) - T[b] with (a, b) the order of the Dij
 * record (SpeciesBlock.cpp:1051, :1309), and for a pair popped from a bin heap,
 * (double)d*(n-2) - (T[a] + T[b]) (:1119-1121).  Records made by buildBins are
 * in node-id order (:549-558); records made when a new node is inserted are
 * in row-slot order (:1280-1292). */
void nwo_nj(float* D, int n, nwo_join* joins, nwo_nj_stats* stats) {
  if (n <= 1) {
    if (stats) { stats->ambiguous_steps = stats->tie_steps = stats->rebuilds = stats->pq_trigger_open = 0; }
    return;
  }
  const int nn = 2 * n - 1;
  const int kBinT = 30 * 31 / 2;              /* m_binT with 30 bins, 1 rank */
  nwo_nj_stats st = {0, 0, 0, 0};
  int* slot = (int*)malloc(sizeof(int) * (size_t)(nn > 0 ? nn : 1));
  int* act = (int*)malloc(sizeof(int) * (size_t)(nn > 0 ? nn : 1));
  double* T = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  float* vd = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  int na = n;
  for (int i = 0; i < n; ++i) { slot[i] = i; act[i] = i; }
  for (int i = n; i < nn; ++i) slot[i] = -1;

  /* buildGblRowSums (:426-453): sequential double sum over active nodes in
   * ascending id order, diagonal included. */
#define ROW_SUMS()                                                   \
  for (int a = 0; a < na; ++a) {                                     \
    const float* row = D + (int64_t)slot[act[a]] * n;                \
    double sum = 0.0;                                                \
    for (int b = 0; b < na; ++b) sum += row[slot[act[b]]];           \
    T[slot[act[a]]] = sum;                                           \
  }
  ROW_SUMS();

  int next = n;                /* m_nextInternalNodeG */
  int watermark = n;           /* ids below this had their record made by buildBins */
  int steps = (int)((float)n * 0.5f);
  if (steps < 200) steps = 200;                       /* :864 */
  int pq_ck = 500;                                    /* :848, :986 */
  long long sz0 = n;
  long long ave0 = (((sz0 - 1) * sz0) / 2) / kBinT;   /* :988 */
  long long ub = ((long long)n * (n - 1)) / 2;        /* heap entries pushed since the last build */
  int m_n = n;

  while (next < nn) {
    const double nm2 = (double)(m_n - 2);
    /* pass 1: exact argmin of the candidate-list q with the :1169-1179 tie-break */
    double best = DBL_MAX;
    int bi = -1, bj = -1;
    for (int a = 0; a < na; ++a) {
      int u = act[a];
      for (int b = a + 1; b < na; ++b) {
        int v = act[b];                    /* u < v */
        int su = slot[u], sv = slot[v];
        float d = D[(int64_t)su * n + sv];
        int f = su, s = sv;
        if (v >= watermark && sv < su) { f = sv; s = su; }
        double q1 = ((double)d * nm2 - T[f]) - T[s];
        if (q1 < best || (q1 == best && (v > bj || (v == bj && u > bi)))) {
          best = q1; bi = u; bj = v;
        }
      }
    }
    /* pass 2: could the other rounding or a wide exact tie change the pick? */
    {
      int su = slot[bi], sv = slot[bj];
      float dw = D[(int64_t)su * n + sv];
      double q2w = (double)dw * nm2 - (T[su] + T[sv]);
      double hiw = best > q2w ? best : q2w;
      int robust_w = (q2w == best);
      int ties = 0, amb = 0;
      for (int a = 0; a < na && !amb; ++a) {
        int u = act[a];
        for (int b = a + 1; b < na; ++b) {
          int v = act[b];
          int pu = slot[u], pv = slot[v];
          float d = D[(int64_t)pu * n + pv];
          int f = pu, s = pv;
          if (v >= watermark && pv < pu) { f = pv; s = pu; }
          double q1 = ((double)d * nm2 - T[f]) - T[s];
          double q2 = (double)d * nm2 - (T[pu] + T[pv]);
          double lo = q1 < q2 ? q1 : q2;
          if (lo > hiw) continue;
          if (u == bi && v == bj) { ++ties; continue; }
          if (robust_w && q1 == q2 && q1 == best) { ++ties; continue; }
          amb = 1;
          break;
        }
      }
      if (ties > 4) amb = 1;
      if (amb) ++st.ambiguous_steps;
      else if (ties > 1) ++st.tie_steps;
    }

    /* TreeNode::join (TreeNode.cpp:31-58) with left = min id, right = max id
     * (SpeciesBlock.cpp:1182-1201). */
    const int si = slot[bi], sj = slot[bj];
    const float dmin = D[(int64_t)si * n + sj];
    const double Ti = T[si], Tj = T[sj];
    double li, lj;
    const double half = 0.5;
    if (m_n == 2) {
      li = lj = (dmin * half);
    } else {
      li = half * (dmin + (Ti - Tj) / (m_n - 2));
      lj = half * (dmin + (Tj - Ti) / (m_n - 2));
    }
    if (li < 0.0) { lj -= li; li = 0.0; }
    else if (lj < 0.0) { li -= lj; lj = 0.0; }
    nwo_join* J = &joins[next - n];
    J->i = bi; J->j = bj; J->node = next; J->n = m_n; J->d = dmin; J->pad = 0.f;
    J->q = best; J->ti = Ti; J->tj = Tj; J->len_i = li; J->len_j = lj;

    /* modifyMatrix (:710-842): unlink j and i, build the new row from the
     * float update, adjust T by the float-rounded delta, the new node takes
     * row/column slot of min id i and keeps its stale diagonal. */
    {
      int w = 0;
      for (int a = 0; a < na; ++a)
        if (act[a] != bi && act[a] != bj) act[w++] = act[a];
      na = w;
    }
    double sum = 0.0;
    for (int a = 0; a < na; ++a) {
      int sk = slot[act[a]];
      float Dik = D[(int64_t)si * n + sk];
      float Djk = D[(int64_t)sj * n + sk];
      float tmp = ((Dik + Djk) - dmin) / 2;
      sum += tmp;
      vd[sk] = tmp;
      T[sk] += (float)(tmp - (Dik + Djk));
    }
    T[si] = sum;
    for (int a = 0; a < na; ++a) {
      int sk = slot[act[a]];
      D[(int64_t)sk * n + si] = vd[sk];
      D[(int64_t)si * n + sk] = vd[sk];
    }
    slot[bi] = slot[bj] = -1;

    /* rebuild schedule (:1206-1247) */
    if (--pq_ck == 0) {
      pq_ck = 500;
      if (steps > 0) {
        /* The reference compares its heap occupancy to 2x the initial size.
         * Occupancy is at most the entries pushed since the last build; if
         * even that bound stays <= 2 the trigger cannot fire. */
        long long tot = ub / kBinT;
        double r = (double)tot / (double)ave0;
        if (r > 2.0) ++st.pq_trigger_open;
      }
    }
    --m_n;
    slot[next] = si;
    act[na++] = next;
    ++next;
    if (steps == 0) {
      ROW_SUMS();
      ++st.rebuilds;
      watermark = next;
      steps = (m_n < 200) ? INT_MAX : (int)((float)m_n * 0.5f);
      sz0 = m_n;
      ave0 = (((sz0 - 1) * sz0) / 2) / kBinT;
      ub = (sz0 * (sz0 - 1)) / 2;
    } else {
      --steps;
      ub += na - 1;          /* the new node's pairs pushed into the heaps */
    }
  }
#undef ROW_SUMS
  if (stats) *stats = st;
  free(slot); free(act); free(T); free(vd);
}


/* ---- progressive alignment (nwo_msa) ----------------------------------- */

typedef struct {
  int len;          /* columns                                   */
  int k;            /* sequences                                 */
  int32_t* cnt;     /* len x NWO_LETTERS letter counts, reversed  */
  int32_t* mapx;    /* merge: X column -> new column (reversed)   */
  int32_t* mapy;    /* merge: Y column -> new column (reversed)   */
  int left, right;  /* children (internal nodes), -1 for leaves   */
} nwo_prof;

static int64_t i64max(int64_t a, int64_t b) { return a > b ? a : b; }

/* Merge X (columns) and Y (rows) into a new profile; fills the maps. */
static int msa_merge(const nwo_prof* X, const nwo_prof* Y, int go, int ge, const int8_t* sub, nwo_prof* out,
                     int32_t* mapx, int32_t* mapy) {
  const int lx = X->len, ly = Y->len;
  const int64_t kk = (int64_t)X->k * Y->k;
  const int64_t GO = go * kk, GE = ge * kk;
  const int64_t kSent = -(((int64_t)1) << 60);
  /* W[y][x] = sum_b cY[y][b] S[x][b]: the row's score against letter x */
  int64_t* W = (int64_t*)malloc(sizeof(int64_t) * (size_t)ly * NWO_LETTERS);
  for (int r = 0; r < ly; ++r)
    for (int x = 0; x < NWO_LETTERS; ++x) {
      int64_t w = 0;
      for (int b = 0; b < NWO_LETTERS; ++b) w += (int64_t)Y->cnt[(size_t)r * NWO_LETTERS + b] * sub[b * NWO_LETTERS + x];
      W[(size_t)r * NWO_LETTERS + x] = w;
    }
  uint8_t* nib = (uint8_t*)malloc((size_t)lx * ly + 1);
  int64_t* Hrow = (int64_t*)malloc(sizeof(int64_t) * (size_t)lx);
  int64_t* Frow = (int64_t*)malloc(sizeof(int64_t) * (size_t)lx);
  for (int c = 0; c < lx; ++c) { Hrow[c] = -GE * (c + 1); Frow[c] = kSent; }
  for (int r = 0; r < ly; ++r) {
    int64_t hleft = -GE * (r + 1), eleft = kSent, diag = (r == 0) ? 0 : -GE * r;
    const int64_t* w = W + (size_t)r * NWO_LETTERS;
    for (int c = 0; c < lx; ++c) {
      const int32_t* cx = X->cnt + (size_t)c * NWO_LETTERS;
      int64_t s = 0;
      for (int x = 0; x < NWO_LETTERS; ++x) s += (int64_t)cx[x] * w[x];
      const int64_t hup = Hrow[c], fup = Frow[c];
      const int64_t f = i64max(fup - GE, hup - GO);
      const int cu = (f == fup - GE);
      const int64_t e = i64max(eleft - GE, hleft - GO);
      const int cl = (e == eleft - GE);
      const int64_t sim = diag + s;
      const int64_t h = i64max(i64max(e, f), sim);
      const int L = ((h == e) && (h != f)) || (h == sim);
      const int U = (h == f) || (h == sim);
      nib[(size_t)r * lx + c] = (uint8_t)((L << 3) | (U << 2) | (cu << 1) | cl);
      diag = hup;
      Hrow[c] = h;
      Frow[c] = f;
      hleft = h;
      eleft = e;
    }
  }
  /* walk: ops in forward order; 12 = both columns, 8 = X only, 4 = Y only */
  uint8_t* ops = (uint8_t*)malloc((size_t)lx + ly + 1);
  int px = lx - 1, py = ly - 1, k = 0;
  unsigned prev = 12u;
#define NIB(xx, yy) ((yy) < 0 ? ((xx) < 0 ? 0u : 9u) : ((xx) < 0 ? 6u : (unsigned)nib[(size_t)(yy) * lx + (xx)]))
  unsigned cell = NIB(px, py);
  while ((cell & 12u) && k < lx + ly) {
    unsigned todo;
    if (((prev & 12u) == 4u) && (prev & 2u)) todo = 4u;
    else if (((prev & 12u) == 8u) && (prev & 1u)) todo = 8u;
    else if ((cell & 12u) == 4u) todo = 4u;
    else if ((cell & 12u) == 8u) todo = 8u;
    else todo = 12u;
    if ((todo != 4u && px < 0) || (todo != 8u && py < 0)) break;
    int stop = 0;
    ops[k++] = (uint8_t)todo;
    if (todo == 8u) --px;
    else if (todo == 4u) { --py; stop = py < 0; }
    else { --px; --py; }
    prev = todo | (cell & 3u);
    cell = stop ? 0u : NIB(px, py);
  }
#undef NIB
  while (px >= 0) { ops[k++] = 8u; --px; }   /* columns the walk left */
  while (py >= 0) { ops[k++] = 4u; --py; }
  /* merged profile: op j (forward) is new column k-1-j (reversed) */
  out->len = k;
  out->k = X->k + Y->k;
  out->cnt = (int32_t*)calloc((size_t)k * NWO_LETTERS + 1, sizeof(int32_t));
  int ix = lx - 1, iy = ly - 1;
  for (int j = 0; j < k; ++j) {
    const int col = k - 1 - j;
    int32_t* o = out->cnt + (size_t)col * NWO_LETTERS;
    if (ops[j] & 8u) {
      for (int x = 0; x < NWO_LETTERS; ++x) o[x] += X->cnt[(size_t)ix * NWO_LETTERS + x];
      mapx[ix--] = col;
    }
    if (ops[j] & 4u) {
      for (int x = 0; x < NWO_LETTERS; ++x) o[x] += Y->cnt[(size_t)iy * NWO_LETTERS + x];
      mapy[iy--] = col;
    }
  }
  free(W); free(nib); free(Hrow); free(Frow); free(ops);
  return k;
}

int64_t nwo_msa(const int8_t* codes, const int64_t* offsets, int n, const int32_t* left, const int32_t* right,
                int go, int ge, const int8_t* sub, char* out, int64_t cap) {
  if (n < 1) return -1;
  const int nn = 2 * n - 1;
  nwo_prof* P = (nwo_prof*)calloc((size_t)nn, sizeof(nwo_prof));
  for (int v = 0; v < n; ++v) {
    const int L = (int)(offsets[v + 1] - offsets[v]);
    P[v].len = L;
    P[v].k = 1;
    P[v].left = P[v].right = -1;
    P[v].cnt = (int32_t*)calloc((size_t)L * NWO_LETTERS + 1, sizeof(int32_t));
    for (int c = 0; c < L; ++c) {
      int x = codes[offsets[v] + c];
      if (x < 0 || x >= NWO_LETTERS) x = NWO_LETTERS - 1;
      P[v].cnt[(size_t)c * NWO_LETTERS + x] = 1;
    }
  }
  for (int k = 0; k < n - 1; ++k) {
    const int a = left[k], b = right[k], v = n + k;
    if (a < 0 || b < 0 || a >= v || b >= v || a >= b || P[a].cnt == NULL || P[b].cnt == NULL) return -1;
    P[a].mapx = (int32_t*)malloc(sizeof(int32_t) * (size_t)P[a].len + 4);
    P[b].mapy = (int32_t*)malloc(sizeof(int32_t) * (size_t)P[b].len + 4);
    msa_merge(&P[a], &P[b], go, ge, sub, &P[v], P[a].mapx, P[b].mapy);
    P[v].left = a;
    P[v].right = b;
  }
  const int root = nn - 1;
  const int64_t L = P[root].len;
  if (out && cap >= (int64_t)n * L) {
    /* final forward position of every column, parents before children */
    int32_t** pos = (int32_t**)calloc((size_t)nn, sizeof(int32_t*));
    pos[root] = (int32_t*)malloc(sizeof(int32_t) * (size_t)L + 4);
    for (int c = 0; c < L; ++c) pos[root][c] = (int32_t)(L - 1 - c);
    for (int v = root; v >= n; --v) {
      const int a = P[v].left, b = P[v].right;
      pos[a] = (int32_t*)malloc(sizeof(int32_t) * (size_t)P[a].len + 4);
      pos[b] = (int32_t*)malloc(sizeof(int32_t) * (size_t)P[b].len + 4);
      for (int c = 0; c < P[a].len; ++c) pos[a][c] = pos[v][P[a].mapx[c]];
      for (int c = 0; c < P[b].len; ++c) pos[b][c] = pos[v][P[b].mapy[c]];
    }
    static const char kDec[NWO_LETTERS + 1] = "ARNDCQEGHILKMFPSTWYVBZX*";
    memset(out, '-', (size_t)n * L);
    for (int v = 0; v < n; ++v)
      for (int c = 0; c < P[v].len; ++c) {
        int x = codes[offsets[v] + c];
        if (x < 0 || x >= NWO_LETTERS) x = NWO_LETTERS - 1;
        out[(size_t)v * L + pos[v][c]] = kDec[x];
      }
    for (int v = 0; v < nn; ++v) free(pos[v]);
    free(pos);
  }
  for (int v = 0; v < nn; ++v) { free(P[v].cnt); free(P[v].mapx); free(P[v].mapy); }
  free(P);
  return L;
}
