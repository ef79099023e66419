/*
 * ref_harness.cpp -- runs the reference's own neighbor-joining code.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile together with the
 * reference's SpeciesBlock.cpp, TreeNode.cpp, CmdLineOptions.cpp and
 * FastaFile.cpp, read in place from the reference checkout (never copied into
 * this repository), plus the one-rank mpi.h of this directory.  Replaces
 * wnj.cpp:15-57 for one rank:
 *
 *   [NWG_REF_D=matrix.f32] ref_nj <input.fasta> <out_prefix>
 *
 * readFasta -> buildTree -> buildAlign, with two stand-ins for the CUDA
 * classes: AlignmentScore computes the distance block with the oracle's
 * restated recurrence (nwo_score_pair), AlignmentMatch records the iNode list
 * buildAlign hands it.  Writes
 *   <prefix>.joins   one line per internal node: node left right
 *                    %a(length(left)) %a(length(right))
 *   <prefix>.cherries  the (left,right) pairs with vecSize==2, in order
 *   <prefix>.D       the float distance matrix (n*n, little endian)
 * and the reference writes <basename>.tree itself (SpeciesBlock.cpp:1328-1338).
 */

/* Standard headers first so the access override below touches only the
 * reference's own classes. */
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <queue>
#include <sstream>
#include <string>
#include <unistd.h>
#include <vector>

#include "mpi.h"
#include "../nw_oracle.h"

/* The CUDA headers of the reference cannot be compiled by a host compiler on
 * CUDA 13; their include guards are taken here and the two classes declared
 * with the reference's signatures (AlignmentScore.cuh:10-38,
 * AlignmentMatch.cuh:9-49). */
#define DEFINITIONS_CUH
#define ALIGNMENTSCORE_CUH
#define ALIGNMENTMATCH_CUH

struct TexVariablesAddresses {
  char* texSeqs1DevPtr;
  char* texSeqs2DevPtr;
};

class AlignmentScore {
 public:
  AlignmentScore(int gapOpen, int gapExt, unsigned int wSize, int maxSeqLen)
      : go_(gapOpen), ge_(gapExt), maxSeqLength(maxSeqLen), windowSize(wSize) {}
  ~AlignmentScore() {}
  void loadDB(char* lbuf, int lSz) {
    xSize = lSz;
    parse_block(lbuf, lSz, xCodes, xOff);
  }
  void computeDistanceMtx(char* rbuf, int rSz, std::vector<std::vector<float> >& distances, int r0) {
    /* NWG_REF_D names a float32 n*n matrix already computed by the same
     * restated recurrence (oracle nwo_score_all, multi-threaded); reading it
     * only saves time on large inputs. */
    if (const char* pre = std::getenv("NWG_REF_D")) {
      FILE* f = std::fopen(pre, "rb");
      if (!f) { std::fprintf(stderr, "ref_harness: cannot open %s\n", pre); std::exit(3); }
      for (int x = 0; x < xSize; ++x)
        if (std::fread(&distances[x][r0], sizeof(float), (size_t)rSz, f) != (size_t)rSz) std::exit(3);
      std::fclose(f);
      return;
    }
    std::vector<int8_t> yCodes;
    std::vector<int64_t> yOff;
    parse_block(rbuf, rSz, yCodes, yOff);
    for (int x = 0; x < xSize; ++x)
      for (int y = 0; y < rSz; ++y)
        distances[x][r0 + y] = (float)nwo_score_pair(
            &xCodes[xOff[x]], (int)(xOff[x + 1] - xOff[x]), &yCodes[yOff[y]],
            (int)(yOff[y + 1] - yOff[y]), go_, ge_, nwo_blosum());
  }

 private:
  static void parse_block(char* buf, int n, std::vector<int8_t>& codes, std::vector<int64_t>& off) {
    /* size the code buffer from the wire lengths, then decode */
    const char* p = buf + sizeof(int);
    int64_t total = 0;
    for (int s = 0; s < n; ++s) {
      int len;
      p += sizeof(int);
      std::memcpy(&len, p, sizeof(int));
      p += sizeof(int) + len + 1;
      total += len;
    }
    codes.assign((size_t)(total > 0 ? total : 1), 0);
    off.assign((size_t)n + 1, 0);
    if (nwo_parse_wire(buf, n, codes.data(), off.data()) != 0) {
      std::fprintf(stderr, "ref_harness: residue outside the 24-letter alphabet\n");
      std::exit(3);
    }
  }
  int go_, ge_;
  int maxSeqLength;
  unsigned int windowSize;
  int xSize = 0;
  std::vector<int8_t> xCodes;
  std::vector<int64_t> xOff;
};

struct iNode {
  int index;
  int vecSize;
  bool aligned;
  std::vector<int> iSpecies;
};

static std::vector<iNode> g_align_nodes;

class AlignmentMatch {
 public:
  AlignmentMatch(int, int, unsigned int, int) {}
  ~AlignmentMatch() {}
  void prepare(std::vector<std::string>&, int) {}
  void computeAlignment(std::vector<iNode>& aSeqs, std::vector<std::string>&, int) {
    g_align_nodes = aSeqs;
  }
};

#define private public
#include "SpeciesBlock.h"
#undef private

#include "SpeciesBlock.cpp"

int myProc, nProcs;

int main(int argc, char* argv[]) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_nj <input.fasta> <out_prefix>\n");
    return 2;
  }
  char* cargv[2] = {argv[0], argv[1]};
  CmdLineOptions cmd(2, cargv);
  if (cmd.state() != CmdLineOptions::iGOOD) return 2;
  MPI_Init(&argc, &argv);
  MPI_Comm_size(MPI_COMM_WORLD, &nProcs);
  MPI_Comm_rank(MPI_COMM_WORLD, &myProc);

  SpeciesBlock sb(cmd);
  sb.readFasta();
  const int n0 = sb.m_n0;
  std::string prefix(argv[2]);
  {
    FILE* f = std::fopen((prefix + ".D").c_str(), "wb");
    for (int i = 0; i < n0; ++i) std::fwrite(sb.m_distances[i].data(), sizeof(float), (size_t)n0, f);
    std::fclose(f);
  }
  sb.buildTree();
  {
    FILE* f = std::fopen((prefix + ".joins").c_str(), "w");
    TreeNode* base = &sb.m_nodes[0];
    for (int k = n0; k < 2 * n0 - 1; ++k) {
      TreeNode& t = sb.m_nodes[k];
      int l = (int)(t.mp_left - base), r = (int)(t.mp_right - base);
      std::fprintf(f, "%d %d %d %a %a\n", k, l, r, t.mp_left->m_length, t.mp_right->m_length);
    }
    std::fclose(f);
  }
  sb.freeMemory();
  sb.buildAlign();
  {
    FILE* f = std::fopen((prefix + ".cherries").c_str(), "w");
    for (const iNode& a : g_align_nodes)
      if (a.vecSize == 2) std::fprintf(f, "%d %d %d\n", a.index, a.iSpecies[0], a.iSpecies[1]);
    std::fclose(f);
  }
  MPI_Finalize();
  return 0;
}
