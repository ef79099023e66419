/*
 * nwgpu.h -- C ABI of the GB300 (sm_103a) all-pairs Needleman-Wunsch,
 * cherry-traceback and neighbor-joining library (libnwgpu.so).
 *
 * Drop-in boundary for the ptersnow/mestrado hot path.  Every entry point is
 * plain C: POD arguments, caller-owned host buffers (or caller-owned device
 * pointers for the *_dev forms), an int status return (0 == NWG_OK) instead of
 * the reference's print-and-exit (AlignmentScore.cu:3-8, :119-122).  The C++
 * classes with the reference's signatures (AlignmentScore, AlignmentMatch) sit
 * on top of this ABI in nwgpu_compat.hpp.
 *
 * Threading: one nwg_ctx per host thread; calls on one context are not
 * re-entrant.  A context owns its CUDA stream (or borrows the caller's, see
 * nwg_set_stream) and all device buffers it needs for its lifetime -- no
 * per-window malloc/free as in AlignmentScore.cu:286-312.
 */
#ifndef NWGPU_H
#define NWGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NWG_OK 0
#define NWG_ERR_NO_DEVICE 1     /* no CUDA device (reference: exit(0), AlignmentScore.cu:119-122) */
#define NWG_ERR_OOM 2           /* device allocation failed                                      */
#define NWG_ERR_BAD_RESIDUE 3   /* byte outside the 24-letter alphabet (AlignmentScore.cu:10-27)  */
#define NWG_ERR_TIMEOUT 4       /* a bounded device wait gave up                                  */
#define NWG_ERR_OVERFLOW 5      /* a score left the int32 range                                   */
#define NWG_ERR_INVALID 6       /* bad argument                                                   */
#define NWG_ERR_CUDA 7          /* CUDA runtime error                                             */
#define NWG_ERR_EMPTY_SEQ 8     /* zero-length sequence (FastaFile.cpp:55 rejects these too)      */
#define NWG_ERR_NJ_AMBIGUOUS 9  /* informational: see nwg_nj_stats.ambiguous_steps               */

/* ---- scoring modes ------------------------------------------------------ */
#define NWG_MODE_BATCHED 0      /* persistent length-bucketed wavefront kernels, int16x2 + int32 */
#define NWG_MODE_PLAIN 1        /* one thread per pair, int32, one launch per length group       */
#define NWG_MODE_BATCHED_INT32 2/* batched kernels with every pair on the int32 lanes            */

typedef struct nwg_ctx nwg_ctx;

typedef struct {
  int64_t pairs;        /* pairs computed, diagonal self-pairs included              */
  int64_t cells;        /* sum over i<j of L_i*L_j: the GCUPS work unit              */
  int64_t pairs_int16;  /* pairs that ran on int16x2 lanes                           */
  int64_t pairs_int32;  /* pairs that ran on int32 lanes                             */
  int64_t reruns;       /* int16 pairs re-run on int32 lanes by the overflow guard   */
  int32_t launches;     /* kernels launched by the call                              */
  int32_t buckets;      /* length buckets                                            */
  double kernel_ms;     /* device time of the scoring launches (events on the stream)*/
  double h2d_ms;        /* host->device copies (host-buffer entry points only)       */
  double d2h_ms;        /* device->host copies (host-buffer entry points only)       */
  double total_ms;      /* host wall time of the call                                */
} nwg_stats;

/* Create a context on the current CUDA device.  gap_open/gap_ext are the
 * penalties of AlignmentScore(gapOpen, gapExt, ...) (AlignmentScore.cu:
 * 110-136; the aligner passes 10 and 2, SpeciesBlock.cpp:361).  sub is the
 * 24x24 substitution matrix in the reference's letter order, or NULL for the
 * built-in blosum64.txt matrix (definitions.cuh:96-121). */
int nwg_ctx_create(int gap_open, int gap_ext, const int8_t* sub, nwg_ctx** out);
int nwg_ctx_destroy(nwg_ctx* ctx);

/* Launch on the caller's cudaStream_t (passed as void*) instead of the
 * context's own stream; NULL restores the context's stream. */
int nwg_set_stream(nwg_ctx* ctx, void* stream);

const char* nwg_status_str(int status);

/* Last CUDA or argument error seen by the context, as text. */
const char* nwg_last_error(const nwg_ctx* ctx);

/* ---- host-side encoding (AlignmentScore::parse, AlignmentScore.cu:142-178) */

/* Decode the wire buffer of SpeciesBlock.cpp:309-322
 * ([int rank][{int seqNo, int len, char[len], '\0'} x n]) into reversed
 * 8-bit codes.  offsets must hold n+1 entries; codes must hold the residue
 * total (pass codes == NULL to only fill offsets). */
int nwg_parse_wire(const char* wire, int n, int8_t* codes, int64_t* offsets);

/* Encode and reverse n ASCII sequences laid end to end (offsets[n+1]). */
int nwg_encode(const char* ascii, const int64_t* offsets, int n, int8_t* codes);

/* The same on the device: d_ascii and d_codes are device buffers, offsets a
 * host array.  Bytes outside the alphabet become -1 as in the reference's
 * table; their count goes to *bad_count (may be NULL) and the call returns
 * NWG_ERR_BAD_RESIDUE.  Synchronizes the context stream. */
int nwg_encode_dev(nwg_ctx* ctx, const char* d_ascii, const int64_t* offsets, int n, int8_t* d_codes,
                   int64_t* bad_count);

/* nwg_parse_wire with the residues encoded on the device: the headers are
 * read from the host copy `wire`, the residues from `d_wire`, a device copy of
 * the same block; offsets (n+1, host) are filled; d_codes may be NULL (offsets
 * only). */
int nwg_parse_wire_dev(nwg_ctx* ctx, const char* wire, const char* d_wire, int n, int8_t* d_codes,
                       int64_t* offsets, int64_t* bad_count);

/* ---- all-pairs distance matrix ----------------------------------------- */

/* Replaces AlignmentScore::loadDB + computeDistanceMtx on one rank
 * (AlignmentScore.cu:180-277, SpeciesBlock.cpp:361-363): fills the full
 * n x n row-major float matrix D (leading dimension ld >= n) with
 * D[i][j] = D[j][i] = (float)score(i, j), diagonal included.  codes/offsets
 * are reversed codes as produced by nwg_parse_wire/nwg_encode.  Host buffers:
 * the call copies the codes in and D out. */
int nwg_score_all(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n,
                  float* D, int64_t ld, int mode, nwg_stats* stats);

/* Same with device-resident codes (d_codes) and matrix (d_D); offsets stay on
 * the host.  Work is queued on the context stream; the call returns once the
 * kernels are queued unless stats != NULL (then it synchronizes to time). */
int nwg_score_all_dev(nwg_ctx* ctx, const int8_t* d_codes, const int64_t* offsets, int n,
                      float* d_D, int64_t ld, int mode, nwg_stats* stats);

/* Rectangular block: D[x][r0 + y] = score(X_x, Y_y) for nx rows of the
 * loaded set X and ny sequences of block Y -- the computeDistanceMtx(rbuf,
 * rSz, distances, r0) shape (AlignmentScore.cu:187-277).  Host buffers. */
int nwg_score_block(nwg_ctx* ctx, const int8_t* xcodes, const int64_t* xoffsets, int nx,
                    const int8_t* ycodes, const int64_t* yoffsets, int ny,
                    float* D, int64_t ld, int64_t r0, int mode, nwg_stats* stats);

/* Score an explicit pair list (pi[k], pj[k]) -> out[k]; host buffers. */
int nwg_score_pairs(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n,
                    const int32_t* pi, const int32_t* pj, int64_t npairs, int32_t* out,
                    nwg_stats* stats);

/* ---- pairwise alignment with traceback ------------------------------------ */

/* Replaces AlignmentMatch::computePairwise (AlignmentMatch.cu:140-317) and
 * its MatchKernel/BacktraceKernel/ReorderMatches launches (NeedlemanWunsch.cu:
 * 592-613): pair k aligns X = sequence px[k] (columns) with Y = sequence
 * py[k] (rows).  Writes the two gapped strings in forward order ('-' for a
 * gap, letters decoded as revConvConst, definitions.cuh:134-137), each
 * NUL-terminated, at outx + k*stride and outy + k*stride (stride >= Lx+Ly+1),
 * the alignment length to len[k] and, if score != NULL, the score to
 * score[k].  codes/offsets are reversed codes (nwg_encode).  Host buffers. */
int nwg_align_pairs(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n,
                    const int32_t* px, const int32_t* py, int npairs, char* outx, char* outy,
                    int64_t stride, int32_t* len, int32_t* score, nwg_stats* stats);

/* Front width of the traceback kernel: lanes per pair (32, 16 or 8; 32/W
 * pairs per warp, bands of 8W rows), or 0 (the default) for the width with
 * the least estimated cost for the call's pairs (rows x columns computed,
 * and the walks of a warp's pairs, which run one after another).  Results
 * do not depend on it.  Not part of the reference's interface. */
int nwg_set_trace_lanes(nwg_ctx* ctx, int lanes);

/* Guide-tree cherries (AlignmentMatch.cu:167-186 over TreeNode::getNodes,
 * TreeNode.cpp:91-117): internal node n_leaves+k joins left[k] and right[k]
 * (node ids: leaves 0..n_leaves-1, internal nodes in creation order).  Lists
 * every internal node whose two children are leaves, in the post-order of
 * getNodes (left subtree, right subtree, node).  Returns the count (outputs may
 * be NULL to only count) or a negative status. */
int nwg_cherries(const int32_t* left, const int32_t* right, int n_leaves, int32_t* node,
                 int32_t* l, int32_t* r);

/* ---- neighbor joining ------------------------------------------------------ */

/* One join: nodes i < j merged into node `node` (= n0 + step) while n nodes
 * were active; d = D[i][j]; q the winning value; ti/tj the row sums and
 * len_i/len_j the branch lengths TreeNode::join gives to i and j
 * (TreeNode.cpp:31-58). */
typedef struct {
  int32_t i, j;
  int32_t node;
  int32_t n;
  float d;
  float pad;
  double q;
  double ti, tj;
  double len_i, len_j;
} nwg_join;

typedef struct {
  int64_t ambiguous_steps;  /* steps where the reference's heap rounding or a >4-way exact tie
                               could pick differently (the exact-argmin pick is kept)          */
  int64_t tie_steps;        /* steps decided by the (max j, max i) tie-break                      */
  int64_t rebuilds;         /* row-sum rebuilds                                                   */
  int64_t pq_trigger_open;  /* heap-size rebuild checks that could not be excluded                */
  double device_ms;         /* device time of the join loop                                       */
  int32_t launches;
  int32_t reference_identical; /* 1: no ambiguous step and no open heap-size check -- every join
                                  is the one the reference's buildTree makes on this matrix;
                                  0: at least one join may differ from the reference's (see below) */
} nwg_nj_stats;

/* Replaces SpeciesBlock::buildTree on one rank (SpeciesBlock.cpp:845-1343):
 * the n-1 joins of neighbor joining on the n x n float matrix D (row-major,
 * leading dimension ld; the caller's matrix is not modified) in the
 * reference's order, with its FP32 matrix updates, FP64 row sums and
 * q = d*(n-2) - T_i - T_j, and its tie-break (larger max(i,j), then larger
 * min(i,j)).  joins must hold n-1 records.  n <= 8192.
 *
 * Each join is the exact argmin of q.  The reference instead values a pair
 * as (d(n-2) - T_i) - T_j in its candidate list and as d(n-2) - (T_i + T_j)
 * when it pops the pair from a bin heap, and cuts its candidates to eight
 * with std::nth_element (SpeciesBlock.cpp:1019-1180).  When no other pair
 * comes within those two roundings of the winner and at most four pairs tie
 * exactly, both give the same join; otherwise the step is counted in
 * stats.ambiguous_steps, and the reference's pick there depends on its heap
 * layouts and on which tied candidates its library's cut keeps (duplicated
 * sequences: tens of tied pairs).  stats.reference_identical is 1 exactly
 * when no step was ambiguous, i.e. when the returned tree is guaranteed to be
 * the reference's. */
int nwg_nj(nwg_ctx* ctx, const float* D, int64_t ld, int n, nwg_join* joins, nwg_nj_stats* stats);

/* Same with D already on the device (d_D). */
int nwg_nj_dev(nwg_ctx* ctx, const float* d_D, int64_t ld, int n, nwg_join* joins, nwg_nj_stats* stats);

/* The Newick text TreeNode::buildTreeOutput writes (TreeNode.cpp:61-81,
 * SpeciesBlock.cpp:1328-1338): "(\n", ",\n", ")\n" separators, lengths as
 * ":" setprecision(4) showpoint setw(8), terminated by ";\n".  names[k] is
 * leaf k's label (the reference uses the whole FASTA header line, '>'
 * included).  Writes at most cap bytes (NUL-terminated) and returns the full
 * length, or a negative status. */
int64_t nwg_newick(const nwg_join* joins, int n, const char* const* names, char* out, int64_t cap);

/* ---- pair scoring without allocation ---------------------------------------
 * No counterpart in the reference: an entry point for hosts that cannot let a
 * library call cudaMalloc or cudaFree -- code running while a stream is
 * captured in the global capture mode, or hosts that hand out all device
 * memory from their own pool and must not have a cudaFree synchronize the
 * device under them.  Same scores as nwg_score_pairs (one pair per thread,
 * int32), but every input and output is caller-provided device memory, no
 * context is used, and the only work memory is a fixed 32 MiB static device
 * array that every GPU loading the library holds until exit.
 *
 *   d_codes/d_start/d_len: reversed codes and per-sequence start and length;
 *   d_pi/d_pj: npairs valid sequence indices; d_out: npairs scores (INT_MIN
 *   for a pair whose X is longer than max_len or has an empty sequence);
 *   max_len: the longest X of the call, at most 32768 (larger values are
 *   rejected with NWG_ERR_INVALID); d_sub: 576-entry device matrix or NULL for
 *   the built-in one; stream: cudaStream_t or NULL.
 *
 * The first call on a device looks the static array up (cudaGetSymbolAddress)
 * with that device current; make it before any stream capture.  All calls on
 * a device share the array and it keeps the last call's contents (nothing in
 * it needs to start at zero); calls whose kernels overlap on the GPU race on
 * it and must be serialized.  The looked-up address is kept for the life of
 * the process: resetting the device (cudaDeviceReset, or a reset of the
 * primary context) after the first call is not supported.  Returns once the
 * kernel is queued. */
int nwg_score_pairs_noalloc(const int8_t* d_codes, const int64_t* d_start, const int32_t* d_len,
                            const int32_t* d_pi, const int32_t* d_pj, int64_t npairs, int32_t* d_out,
                            int max_len, int gap_open, int gap_ext, const int8_t* d_sub, void* stream);

/* ---- measurement ---------------------------------------------------------
 * Not part of the reference's interface (the reference times nothing on the
 * device; timer.h falls back to clock()).  These give the bench its roofline
 * denominator and per-launch device times. */

/* Peak of the cell update alone: every SM runs the cell update on
 * register-resident strips, no memory, no shuffles, in every form of
 * nwg_dpx_peak_form, and the fastest form counts.  lanes16 != 0: int16x2
 * words (2 cells per word), else int32.  Returns cells per second. */
int nwg_dpx_peak(nwg_ctx* ctx, int lanes16, double* cells_per_s);

/* The same for one form of the cell update: 0 = 2 adds + 2 viaddmax + 1
 * vimax3; 2 = 1 add + 4 viaddmax (shifted E', F'); 3 = shifted, 5 adds + 2
 * two-input max + 1 vimax3; 4 = unshifted, 4 adds + 2 max + 1 vimax3;
 * 5 = shifted, viaddmax on the F chain, adds + max off it. */
int nwg_dpx_peak_form(nwg_ctx* ctx, int lanes16, int form, double* cells_per_s);

typedef struct {
  int32_t kind;         /* 0 wave (batched), 1 plain, 2 pair list, 3 other    */
  int32_t rows_per_lane;/* R of the wave kernel                                */
  int32_t lanes16;      /* 1: int16x2 lanes, 0: int32                          */
  int32_t grid;         /* CTAs launched                                       */
  int64_t pairs;        /* pairs (i<j) this launch computes                    */
  int64_t cells;        /* their L_i*L_j sum                                   */
  double ms;            /* device time (events around this launch alone)       */
  int32_t variant;      /* register layout of the wave kernel (0..6)          */
  int32_t lanes;        /* lanes per wavefront (32, 16, 8)                    */
} nwg_launch_rec;

/* Per-launch event timing for the next calls (0 = off, the default: timing
 * inserts events between launches). */
int nwg_set_launch_timing(nwg_ctx* ctx, int on);

/* Records of the launches of the last scoring call; returns how many exist
 * (copies at most cap). */
int nwg_launch_records(nwg_ctx* ctx, nwg_launch_rec* out, int cap);

/* ---- autotuner --------------------------------------------------------------
 * The batched form has a kernel choice per length class of the shorter
 * sequences of a pair (the Y rows): rows per lane (4..32), lanes per
 * wavefront (32, 16 or 8; band = lanes x rows per lane) and register layout.  nwg_autotune times every candidate of every class on
 * synthetic inputs of that class's length and keeps the fastest; the result is
 * cached in a text file per device (directory $NWG_TUNE_CACHE, else
 * $HOME/.cache/nwgpu) and reused by later contexts.  Not part of the
 * reference's interface, which had one fixed window/strip shape
 * (definitions.cuh:26,47-48). */
#define NWG_TUNE_CLASSES 16

typedef struct {
  int32_t classes;                          /* NWG_TUNE_CLASSES                          */
  int32_t from_cache;                       /* 1 if read from the cache file              */
  int32_t max_rows[NWG_TUNE_CLASSES];       /* class k: Y rows <= max_rows[k]             */
  int32_t rows_per_lane[NWG_TUNE_CLASSES];
  int32_t variant[NWG_TUNE_CLASSES];
  int32_t lanes[NWG_TUNE_CLASSES];          /* lanes per wavefront                        */
  int32_t pad;
  double gcups[NWG_TUNE_CLASSES];           /* the winner's throughput on the probe       */
  double seconds;                           /* tuning time (0 from cache)                 */
} nwg_tune_result;

/* flags: 1 = ignore (and overwrite) the cache. */
int nwg_autotune(nwg_ctx* ctx, int flags, nwg_tune_result* out);

/* Set the choice per class explicitly (NWG_TUNE_CLASSES entries each), on
 * 32-lane wavefronts; nwg_set_tuning_lanes also sets the lanes per front
 * (32, 16 or 8; narrow fronts take variant 0 or 2). */
int nwg_set_tuning(nwg_ctx* ctx, const int32_t* rows_per_lane, const int32_t* variant);
int nwg_set_tuning_lanes(nwg_ctx* ctx, const int32_t* rows_per_lane, const int32_t* variant,
                         const int32_t* lanes);

/* ---- progressive alignment ----------------------------------------------------
 * The multiple alignment along the guide tree (the reference's
 * AlignmentMatch::computeMSA, AlignmentMatch.cu:320-434, is an empty loop:
 * this is the library's own definition, the same as the oracle's nwo_msa).
 * Internal node n+k joins left[k] (columns) and right[k] (rows), left[k] <
 * right[k] < n+k -- the (i, j) of nwg_join records.  Profiles are letter
 * counts per column; a merge is the pairwise recurrence and traceback flags
 * of nwg_align_pairs with the cell score sum_x sum_y cX[x] cY[y] S[x][y] and
 * the gap penalties scaled by the product of the two profiles' sequence
 * counts (64-bit integers); columns a walk leaves are appended opposite gaps.
 * codes/offsets: reversed codes (nwg_encode).  Returns the alignment length in
 * *msa_len; nwg_msa_rows then copies the n rows (forward order, '-' for gaps)
 * to out, row k at out + k*row_stride (row_stride >= length). */
int nwg_msa(nwg_ctx* ctx, const int8_t* codes, const int64_t* offsets, int n, const int32_t* left,
            const int32_t* right, int64_t* msa_len, nwg_stats* stats);
int nwg_msa_rows(nwg_ctx* ctx, char* out, int64_t row_stride);

/* ---- serving loop ------------------------------------------------------------
 * Alignment jobs (one sequence family each: distance matrix + guide tree, the
 * work of SpeciesBlock::buildTree up to the join loop, SpeciesBlock.cpp:242-403
 * and wnj.cpp:10-52, for one job) submitted at any time from any thread.
 * A worker thread admits pending jobs while their HBM footprint
 * (n^2 floats of matrix + NJ workspace + codes) fits hbm_budget_bytes and puts
 * up to max_batch_jobs of them into one batch: one persistent launch per
 * length bucket with pairs of all the batch's jobs interleaved, then the
 * join loops, one launch per form: one CTA per job up to 160 sequences, a
 * cluster per job (8 CTAs, 16 from 256 sequences on) with the matrix in its
 * shared memory up to 768, a cluster over L2 above.  Up to four batches
 * can be on the device at once (own streams), so jobs arriving while one batch runs
 * are admitted and overlap it, and each batch is returned as soon as it is done.  Each job's matrix and join list equal what
 * nwg_score_all and nwg_nj return for that job alone.
 * Jobs with n <= 8192 sequences are accepted (larger: NWG_ERR_INVALID).
 * The reference has no serving loop. */
typedef struct nwg_server nwg_server;

typedef struct {
  int32_t n;                   /* sequences                                        */
  int32_t status;              /* NWG_OK or the job's error                         */
  int32_t batch_jobs;          /* jobs in the batch it ran in                       */
  int32_t nj_reference_identical; /* as nwg_nj_stats.reference_identical            */
  double queue_ms;             /* submit -> admitted to a batch                     */
  double latency_ms;           /* submit -> results on the host                     */
  int64_t cells;               /* DP cells of the job's off-diagonal pairs          */
  int64_t nj_ambiguous_steps;  /* as nwg_nj_stats                                   */
  int64_t nj_tie_steps;
  int64_t nj_rebuilds;
} nwg_job_info;

int nwg_server_create(int gap_open, int gap_ext, int64_t hbm_budget_bytes, int max_batch_jobs,
                      nwg_server** out);
/* Copies the job's sequences (ASCII, offsets[0..n]; empty sequences are
 * refused here) and returns at once; the residues are encoded on the device
 * with the batch, so a byte outside the alphabet makes the job's status
 * NWG_ERR_BAD_RESIDUE at nwg_server_wait. */
int nwg_server_submit(nwg_server* srv, const char* ascii, const int64_t* offsets, int n, uint64_t* job_id);
/* Waits up to timeout_ms (< 0: no limit; NWG_ERR_TIMEOUT when it runs out, the
 * job stays queryable) for the job, copies its n*n matrix to D and its n-1
 * joins to joins (either may be NULL) and releases it; returns the job's
 * status.  A second call for a job another thread is waiting for returns
 * NWG_ERR_INVALID at once. */
int nwg_server_wait(nwg_server* srv, uint64_t job_id, int timeout_ms, float* D, nwg_join* joins,
                    nwg_job_info* info);
/* Stops admitting, finishes the batches on the device, frees everything.
 * Jobs not yet waited for are dropped. */
int nwg_server_destroy(nwg_server* srv);

#ifdef __cplusplus
}
#endif
#endif
