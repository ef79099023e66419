/*
 * nw_oracle.h -- CPU restatement of the ptersnow/mestrado hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, calls or
 * executes this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, always as the oracle and never as the thing measured
 * or shipped.
 *
 * Each function cites the reference file:line whose behaviour it restates.
 * Parity pin: the NW score restatement is checked against hand-derived
 * known-answer tests; the NJ restatement is checked against the reference's
 * own SpeciesBlock.cpp/TreeNode.cpp compiled unchanged through a one-rank MPI
 * shim (oracle/ref_shim, built into oracle/_ref/) and against the golden join
 * lists that build produced (tests/golden/).
 */
#ifndef NW_ORACLE_H
#define NW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Alphabet order of the reference (AlignmentScore.cu:10-27, definitions.cuh:134-137). */
#define NWO_LETTERS 24

/* ASCII -> code table (every unlisted byte maps to -1). */
void nwo_conversion_table(int8_t out[256]);

/* The 24x24 substitution matrix (definitions.cuh:96-121 == blosum64.txt). */
const int8_t* nwo_blosum(void);

/* Encode one ASCII sequence and reverse it, as AlignmentScore::parse intends
 * (AlignmentScore.cu:142-178, with the middle residue of odd lengths encoded
 * too).  Returns the number of residues that mapped to -1 (0 == clean). */
int nwo_encode_reverse(const char* ascii, int len, int8_t* out);

/* Decode the MPI wire buffer of SpeciesBlock.cpp:309-322:
 *   [int rank][{int seqNo, int len, char[len], '\0'} x n]
 * into concatenated reversed codes, offsets[n+1].  Returns bad-residue count. */
int nwo_parse_wire(const char* buf, int n, int8_t* codes, int64_t* offsets);

/* Gotoh global score of one pair, restating NeedlemanWunschGlobalScoreKernel
 * (NeedlemanWunsch.cu:22-161) loop for loop: 12-row strips, one (H,F) pair per
 * X column carried between strips, sentinel -32768+ge.  int32 arithmetic. */
int nwo_score_pair(const int8_t* x, int lx, const int8_t* y, int ly,
                   int go, int ge, const int8_t* sub);

/* All-pairs distance matrix D[i*ld+j] = D[j*ld+i] = (float)score(i,j), diagonal
 * included (AlignmentScore.cu:262-264 with defects 5/6 fixed).  OpenMP over
 * rows when threads > 1. */
void nwo_score_all(const int8_t* codes, const int64_t* offsets, int n,
                   int go, int ge, const int8_t* sub, float* D, int64_t ld,
                   int threads);

/* Score an explicit list of pairs (used for bounded CPU baselines). */
void nwo_score_list(const int8_t* codes, const int64_t* offsets,
                    const int32_t* pi, const int32_t* pj, int64_t npairs,
                    int go, int ge, const int8_t* sub, int32_t* out, int threads);

/* Traceback nibbles of NeedlemanWunschGlobalMatchKernel (NeedlemanWunsch.cu:
 * 184-365) followed by NeedlemanWunschGlobalBackKernel (:393-494), reorder
 * (:496-563) folded in.  Writes two NUL-terminated gapped ASCII strings
 * (capacity lx+ly+1 each) and returns the alignment length; *score gets H. */
int nwo_traceback(const int8_t* x, int lx, const int8_t* y, int ly,
                  int go, int ge, const int8_t* sub,
                  char* outx, char* outy, int* score);

/* One neighbor-joining step record. */
typedef struct {
  int32_t i, j;        /* joined node ids, i < j                          */
  int32_t node;        /* id of the new internal node                      */
  int32_t n;           /* active node count when the join was chosen       */
  float   d;           /* D[i][j]                                          */
  float   pad;
  double  q;           /* winning q value                                  */
  double  ti, tj;      /* row sums T_i, T_j used by TreeNode::join         */
  double  len_i, len_j;/* branch lengths given to i and j                  */
} nwo_join;

typedef struct {
  int64_t ambiguous_steps;   /* steps where the two q roundings or >4 exact ties could change the pick */
  int64_t tie_steps;         /* steps resolved by the (max j, max i) tie-break                       */
  int64_t rebuilds;          /* row-sum rebuilds performed                                           */
  int64_t pq_trigger_open;   /* checks where the heap-size trigger could not be excluded             */
} nwo_nj_stats;

/* Exact-argmin restatement of SpeciesBlock::buildTree (SpeciesBlock.cpp:845-
 * 1343) with modifyMatrix (:710-842), buildGblRowSums (:426-453) and
 * TreeNode::join (TreeNode.cpp:31-58).  D is n x n row-major float and is
 * modified in place.  joins must hold n-1 records. */
void nwo_nj(float* D, int n, nwo_join* joins, nwo_nj_stats* stats);

typedef struct {
  int64_t rebuilds;          /* row-sum and bin rebuilds                                          */
  int64_t pq_triggers;       /* rebuilds started by the heap occupancy check                      */
  int64_t out_of_range_bins; /* bin bounds the reference reads past its T vector (below 29 taxa)  */
} nwo_nj_model_stats;

/* Neighbor joining as SpeciesBlock::buildTree runs it (SpeciesBlock.cpp:
 * 426-1343): bins, bin heaps, candidate list, the eight kept candidates and
 * the prediction array, so that each join is valued in the rounding the
 * reference applies to it, with the reference's own standard containers and
 * algorithms (nj_model.cpp).  D (n x n, row-major float) is modified in place;
 * joins must hold n-1 records. */
void nwo_nj_model(float* D, int n, nwo_join* joins, nwo_nj_model_stats* stats);

/* Progressive alignment along the guide tree (this library's definition: the
 * reference's AlignmentMatch::computeMSA, AlignmentMatch.cu:320-434, is an
 * empty loop -- parity unpinned).  Internal node n+k joins left[k] (X,
 * columns) and right[k] (Y, rows), left[k] < right[k].  A profile is its
 * columns' letter counts, in reversed column order like the codes; a merge
 * aligns two profiles with the pairwise recurrence and flags of
 * nwo_traceback, generalised: the cell score is the sum over residue pairs
 * sum_x sum_y cX[x] cY[y] S[x][y], the gap penalties are go*kX*kY and
 * ge*kX*kY (k = sequences in a profile), all in 64-bit integers.  The walk
 * follows nwo_traceback's rules; columns it leaves (an up move out of row 0)
 * are appended opposite gaps.  Writes n rows of L characters (row k =
 * sequence k in forward order, '-' for gaps) to out when cap >= n*L; returns
 * L (or -1 on a malformed tree). */
int64_t nwo_msa(const int8_t* codes, const int64_t* offsets, int n, const int32_t* left, const int32_t* right,
                int go, int ge, const int8_t* sub, char* out, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
