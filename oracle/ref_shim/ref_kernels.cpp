/*
 * ref_kernels.cpp -- the reference's own score, match and backtrace kernels
 * run on the host, one sequence pair at a time.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile copies the kernel section of the
 * reference's NeedlemanWunsch.cu (from its first line down to `#undef BACK`,
 * i.e. NeedlemanWunschGlobalScoreKernel :22-161, NeedlemanWunschGlobalMatchKernel
 * :184-365, NeedlemanWunschGlobalBackKernel :393-494 and reorderMatchesMemory
 * :496-563, without the <<<>>> launchers :586-613) from the reference checkout
 * into oracle/_ref/ (git-ignored) and compiles it here unchanged, with the
 * reference's definitions.cuh (substitution matrix, alphabet, constants) read
 * from the checkout too.  Nothing of the reference is copied into this
 * repository.
 *
 * The CUDA constructs are given host meanings:
 *   __global__, __device__, __constant__  -> nothing (plain functions/globals)
 *   __shared__                            -> static (one block's shared array)
 *   threadIdx, blockIdx, blockDim         -> globals set before each call
 *   texSeqsX/Y, tex1Dfetch                -> a bounds-checked byte fetch
 *                                            (0 outside, as a 1D texture bound
 *                                            to linear memory returns)
 *   __syncthreads()                       -> nothing (one thread runs at a time)
 *   max, min                              -> int max/min
 * Each call runs one pair as the only thread of a 1x1 block (window = 1,
 * offset = 1), so thread-local indexing (blockThread = 0) never aliases.
 *
 * Patches, each forced by running the shipped text correctly (the reference's
 * defects):
 *  - a 16x16 block loads only entries 0..287 of the 576-entry matrix
 *    into shmSM (NeedlemanWunsch.cu:26-35, :188-197).  Before the first pair,
 *    each kernel is run once per loader thread idx = 0..559 on an empty pair
 *    (length 0, returns right after the load), which fills all 576 entries of
 *    its static shmSM through the kernel's own load code;
 *  - BLOCK_SIZE 16 with 256 threads overflows AE_shared/sharedYSeq
 *    (:75-77, :243-245).  One thread per block indexes slot 0 only;
 *  - the host-side parse and copy defects (AlignmentScore.cu): not part
 *    of this text; the caller passes correctly encoded, fully reversed codes.
 * Uninitialised locals of the backtrace kernel (tmpMatchX/Y, shifted out
 * before use) are zero-initialised by the compiler flag
 * -ftrivial-auto-var-init=zero; the shipped text relied on the shifts alone.
 */
#include <climits>
#include <cstdint>
#include <cstring>
#include <vector>

#include "vector_types.h"

#define __global__
#define __device__
#define __constant__
#define __shared__ static
#define __syncthreads() ((void)0)

static uint3 threadIdx, blockIdx;
static dim3 blockDim;

struct ShimTexture {
  const char* p;
  int n;
};
static ShimTexture texSeqsX, texSeqsY;
static inline char tex1Dfetch(const ShimTexture& t, int i) { return (i >= 0 && i < t.n) ? t.p[i] : (char)0; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }

#include "nw_kernels.inc"

namespace {

void run_as(unsigned tx, unsigned ty, unsigned bdx, unsigned bdy) {
  threadIdx = {tx, ty, 0};
  blockIdx = {0, 0, 0};
  blockDim = {bdx, bdy, 1};
}

void set_pair(const int8_t* x, int lx, const int8_t* y, int ly, int go, int ge) {
  gapOp = (char)go;
  gapEx = (char)ge;
  window = 1;
  offset = 1;
  std::memset(tex1Starts, 0, sizeof(tex1Starts));
  std::memset(tex2Starts, 0, sizeof(tex2Starts));
  tex1Starts[1] = lx;
  tex2Starts[1] = ly;
  texSeqsX = {reinterpret_cast<const char*>(x), lx};
  texSeqsY = {reinterpret_cast<const char*>(y), ly};
}

// Fill each kernel's static shmSM through its own load code: loader threads
// idx = ty*16 + tx for idx 0..559 (idx + 16 stays below 576), on an empty
// pair so that every call returns right after the load.
bool primed = false;
void prime() {
  if (primed) return;
  std::memset(tex1Starts, 0, sizeof(tex1Starts));
  std::memset(tex2Starts, 0, sizeof(tex2Starts));
  short2 af[1];
  unsigned int back[1];
  int score[1];
  for (unsigned idx = 0; idx < 560; ++idx) {
    run_as(idx % 16, idx / 16, 16, 1);
    NeedlemanWunschGlobalScoreKernel(af, score, false);
    NeedlemanWunschGlobalMatchKernel(af, back, score, 1, false);
  }
  primed = true;
}

}  // namespace

extern "C" {

/* Score of one pair through NeedlemanWunschGlobalScoreKernel.  x (columns)
 * and y (rows) are encoded, reversed codes, 1 <= lx, ly <= 32767. */
int refk_score_pair(const int8_t* x, int lx, const int8_t* y, int ly, int go, int ge) {
  if (lx < 1 || ly < 1 || lx > SHRT_MAX || ly > SHRT_MAX) return INT_MIN;
  prime();
  set_pair(x, lx, y, ly, go, ge);
  std::vector<short2> af((size_t)lx);
  int score = INT_MIN;
  run_as(0, 0, 1, 1);
  NeedlemanWunschGlobalScoreKernel(af.data(), &score, false);
  return score;
}

/* One pair through NeedlemanWunschGlobalMatchKernel (score + 4-bit flags) and
 * NeedlemanWunschGlobalBackKernel (walk, gapped ASCII).  outx/outy receive
 * the two gapped rows (NUL-terminated, capacity lx + ly + 1 each); returns
 * their length, the score in *score. */
int refk_traceback(const int8_t* x, int lx, const int8_t* y, int ly, int go, int ge, char* outx, char* outy,
                   int* score) {
  if (lx < 1 || ly < 1 || lx + ly > SHRT_MAX - 8) return -1;
  prime();
  set_pair(x, lx, y, ly, go, ge);
  const short rowWidth = (short)(lx + 1);
  std::vector<short2> af((size_t)lx);
  std::vector<unsigned int> back((size_t)((ly + 7) / 8 + 1) * (size_t)rowWidth, 0u);
  const size_t words = (size_t)(lx + ly) / 4 + 3;
  std::vector<unsigned int> mx(words, 0u), my(words, 0u);
  run_as(0, 0, 1, 1);
  NeedlemanWunschGlobalMatchKernel(af.data(), back.data(), score, rowWidth, false);
  NeedlemanWunschGlobalBackKernel(back.data(), rowWidth, mx.data(), my.data(), false);
  // word k holds characters 4k..4k+3, the first in its most significant byte
  // (the byte swap reorderMatchesMemory performs)
  int k = 0;
  for (size_t w = 0; w < words; ++w)
    for (int b = 3; b >= 0; --b) {
      const char cx = (char)((mx[w] >> (8 * b)) & 0xFF), cy = (char)((my[w] >> (8 * b)) & 0xFF);
      if (cx == 0 || cy == 0) {
        outx[k] = outy[k] = 0;
        return k;
      }
      outx[k] = cx;
      outy[k] = cy;
      ++k;
    }
  outx[k] = outy[k] = 0;
  return k;
}

}  // extern "C"
