/*
 * nwgpu_compat.hpp -- the reference's CUDA host classes, re-exposed on the
 * libnwgpu C ABI with their signatures unchanged, so that the aligner's host
 * code (SpeciesBlock.cpp:361-363, :395, :1402-1403, :1498, :1583) compiles and
 * links against the GB300 path without edits: include this header where the
 * reference includes AlignmentScore.cuh / AlignmentMatch.cuh (the include
 * guards are the reference's, so either name works) and link libnwgpu.so.
 *
 * Behaviour differences, all deliberate:
 *  - errors: the reference prints and calls exit() (AlignmentScore.cu:3-8);
 *    here a failing call prints the library's status text to stderr and calls
 *    exit() with the status, the same observable contract, unless
 *    NWGPU_COMPAT_THROW is defined, in which case it throws std::runtime_error;
 *  - the window size argument is accepted and ignored (the GPU path has no
 *    windows); copySeqsToTex and the free per-window launchers (ScoreKernel,
 *    MatchKernel, BacktraceKernel, ReorderMatches) exist for source
 *    compatibility only and report that they are not used;
 *  - computeDistanceMtx writes distances[x][r0 + y] for the rows of the loaded
 *    block and the columns of rbuf (the reference wrote the uninitialised
 *    `col` instead of r0, AlignmentScore.cu:195,264);
 *  - AlignmentMatch::computeAlignment aligns every cherry it is handed
 *    (iNode.vecSize == 2): seqs[iSpecies[0]] (X) against seqs[iSpecies[1]]
 *    (Y); both strings are replaced by their gapped rows and the node is
 *    marked aligned.  computeMSA (profile alignment beyond cherries) is not
 *    provided: the reference's is an empty loop (AlignmentMatch.cu:428-430).
 */
#ifndef NWGPU_COMPAT_HPP
#define NWGPU_COMPAT_HPP

#include <string>
#include <vector>

#include "nwgpu.h"

#ifndef DEFINITIONS_CUH
#define DEFINITIONS_CUH
/* the standard headers definitions.cuh:4-13 brings to its includers (the CUDA
 * runtime headers it includes there also bring <climits> and <cfloat>) */
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdio>
#include <cstring>
#include <iostream>
/* definitions.cuh:227-231 */
struct TexVariablesAddresses {
  char* texSeqs1DevPtr;
  char* texSeqs2DevPtr;
};
#endif

#ifndef ALIGNMENTSCORE_CUH
#define ALIGNMENTSCORE_CUH
/* AlignmentScore.cuh:10-38 */
class AlignmentScore {
 public:
  AlignmentScore(int gapOpen, int gapExt, unsigned int wSize, int maxSeqLen);
  ~AlignmentScore();

  void loadDB(char* lbuf, int lSz);
  TexVariablesAddresses copySeqsToTex(int startSeqs1No, int startSeqs2No);
  void parse(std::string seqs, std::vector<int>& starts, std::vector<int>& lenghts, char* input, int size);
  void computeDistanceMtx(char* rbuf, int rSz, std::vector<std::vector<float> >& distances, int r0);

 private:
  nwg_ctx* ctx_;
  int xSize;
  std::vector<char> xWire;
  std::vector<int8_t> xCodes;
  std::vector<int64_t> xOffsets;
};
#endif

#ifndef ALIGNMENTMATCH_CUH
#define ALIGNMENTMATCH_CUH
/* AlignmentMatch.cuh:9-15 */
struct iNode {
  int index;
  int vecSize;
  bool aligned;
  std::vector<int> iSpecies;
};

/* AlignmentMatch.cuh:21-49 */
class AlignmentMatch {
 public:
  AlignmentMatch(int gapOpen, int gapExt, unsigned int wSize, int maxSeqLen);
  ~AlignmentMatch();

  void prepare(std::vector<std::string>& seqs, int myProc);
  void computeAlignment(std::vector<iNode>& aSeqs, std::vector<std::string>& seqs, int myProc);

  TexVariablesAddresses copySeqsToTex(int startSeqs1No, int startSeqs2No);

  void computeMSA(std::vector<iNode>& aSeqs, std::vector<std::string>& seqs, int myProc);
  void computePairwise(std::vector<iNode>& aSeqs, std::vector<std::string>& seqs, int myProc);

 private:
  nwg_ctx* ctx_;
};
#endif

/* The reference's free per-window launchers (AlignmentScore.cuh:40,
 * AlignmentMatch.cuh:51-56), declared when the CUDA vector types are
 * available; they are never called by the GB300 path. */
#if defined(__has_include)
#if __has_include(<vector_types.h>)
#include <vector_types.h>
#define NWGPU_COMPAT_LAUNCHERS 1
void ScoreKernel(dim3 grid, dim3 block, short2* AF, int* scoresDevPtr, bool border);
void MatchKernel(dim3 grid, dim3 block, short2* AF, unsigned int* back, int* scoresDevPtr, short rowWidth,
                 bool border);
void ReorderMatches(dim3 grid, dim3 block, unsigned int* inX, unsigned int* outX, unsigned int* inY,
                    unsigned int* outY, int maxMatchLength);
void BacktraceKernel(dim3 grid, dim3 block, unsigned int* back, short rowWidth, unsigned int* matchesX,
                     unsigned int* matchesY, bool border);
#endif
#endif

#endif
