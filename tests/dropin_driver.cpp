// dropin_driver.cpp -- a host program of this project's own that drives the
// GB300 path through the reference's class interface (include/nwgpu_compat.hpp)
// the way the aligner's host code does: AlignmentScore::loadDB with a rank's
// row block and computeDistanceMtx with column blocks at offset r0
// (SpeciesBlock.cpp:356-363, :395), then AlignmentMatch::computeAlignment on
// an iNode list (SpeciesBlock.cpp:1402-1403, :1498).  Test infrastructure:
// built and run by tests/test_dropin_gpu.py.
//
//   dropin_driver <seqs.txt> <cherries.txt> <out_prefix>
//
// seqs.txt: one sequence per line.  cherries.txt: "a b" per line (the two
// leaves of a cherry).  Writes
//   <prefix>.square  n*n float32: loadDB(all), computeDistanceMtx(all, r0 = 0)
//   <prefix>.split   n*n float32: loadDB(all), then the column blocks [0, h)
//                    at r0 = 0 and [h, n) at r0 = h
//   <prefix>.rows    (n-h)*n float32: loadDB(rows [h, n)), columns all
//   <prefix>.aln     per iNode of the list, its two rows after alignment
//                    (cherries) or the untouched sequences (other nodes)
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "nwgpu_compat.hpp"

namespace {

// wire block of SpeciesBlock.cpp:309-322: [int rank][{int seqNo, int len,
// char[len], '\0'} x n]
std::vector<char> wire(const std::vector<std::string>& s, int first, int count) {
  std::vector<char> b(sizeof(int), 0);
  for (int k = first; k < first + count; ++k) {
    const int no = k, len = (int)s[(size_t)k].size();
    const size_t at = b.size();
    b.resize(at + 2 * sizeof(int) + (size_t)len + 1);
    std::memcpy(&b[at], &no, sizeof(int));
    std::memcpy(&b[at + sizeof(int)], &len, sizeof(int));
    std::memcpy(&b[at + 2 * sizeof(int)], s[(size_t)k].data(), (size_t)len);
    b[at + 2 * sizeof(int) + (size_t)len] = 0;
  }
  return b;
}

bool dump(const std::string& path, const std::vector<std::vector<float> >& D) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  for (const auto& row : D)
    if (std::fwrite(row.data(), sizeof(float), row.size(), f) != row.size()) return false;
  return std::fclose(f) == 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s <seqs.txt> <cherries.txt> <out_prefix>\n", argv[0]);
    return 2;
  }
  std::vector<std::string> seqs;
  {
    std::ifstream in(argv[1]);
    std::string line;
    while (std::getline(in, line))
      if (!line.empty()) seqs.push_back(line);
  }
  const int n = (int)seqs.size(), h = n / 2;
  const std::string out = argv[3];
  int maxLen = 0;
  for (const auto& s : seqs) maxLen = s.size() > (size_t)maxLen ? (int)s.size() : maxLen;

  AlignmentScore score(10, 2, 16, maxLen);
  std::vector<char> all = wire(seqs, 0, n), lo = wire(seqs, 0, h), hi = wire(seqs, h, n - h);

  std::vector<std::vector<float> > D(n, std::vector<float>(n, -1.0f));
  score.loadDB(all.data(), n);
  score.computeDistanceMtx(all.data(), n, D, 0);
  if (!dump(out + ".square", D)) return 3;

  std::vector<std::vector<float> > S(n, std::vector<float>(n, -1.0f));
  score.computeDistanceMtx(lo.data(), h, S, 0);
  score.computeDistanceMtx(hi.data(), n - h, S, h);
  if (!dump(out + ".split", S)) return 3;

  std::vector<std::vector<float> > R(n - h, std::vector<float>(n, -1.0f));
  score.loadDB(hi.data(), n - h);
  score.computeDistanceMtx(all.data(), n, R, 0);
  if (!dump(out + ".rows", R)) return 3;

  // iNode list: every cherry, and between them a three-leaf node that the
  // pairwise stage leaves alone
  std::vector<iNode> nodes;
  {
    std::ifstream in(argv[2]);
    int a, b, id = n;
    while (in >> a >> b) {
      iNode c;
      c.index = id++;
      c.vecSize = 2;
      c.aligned = false;
      c.iSpecies = {a, b};
      nodes.push_back(c);
      iNode t;
      t.index = id++;
      t.vecSize = 3;
      t.aligned = false;
      t.iSpecies = {a, b, 0};
      nodes.push_back(t);
    }
  }
  AlignmentMatch match(10, 2, 16, maxLen);
  std::vector<std::string> work = seqs;
  match.prepare(work, 0);
  match.computeAlignment(nodes, work, 0);
  std::ofstream aln(out + ".aln");
  for (const auto& nd : nodes) {
    if (nd.vecSize != 2) continue;
    aln << (nd.aligned ? 1 : 0) << "\n" << work[(size_t)nd.iSpecies[0]] << "\n" << work[(size_t)nd.iSpecies[1]] << "\n";
  }
  return aln.good() ? 0 : 3;
}
