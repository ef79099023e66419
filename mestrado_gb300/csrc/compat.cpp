// compat.cpp -- AlignmentScore / AlignmentMatch (reference signatures) on the
// libnwgpu C ABI.  See include/nwgpu_compat.hpp for the contract.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nwgpu_compat.hpp"

namespace {

void die(int status, nwg_ctx* ctx, const char* where) {
  std::string msg = std::string(where) + ": " + nwg_status_str(status);
  if (ctx) {
    const char* extra = nwg_last_error(ctx);
    if (extra && *extra) msg += std::string(" (") + extra + ")";
  }
#ifdef NWGPU_COMPAT_THROW
  throw std::runtime_error(msg);
#else
  std::fprintf(stderr, "nwgpu: %s\n", msg.c_str());
  std::exit(status);
#endif
}

nwg_ctx* make_ctx(int go, int ge) {
  nwg_ctx* c = nullptr;
  const int rc = nwg_ctx_create(go, ge, nullptr, &c);
  if (rc == NWG_ERR_NO_DEVICE) {
    // AlignmentScore.cu:119-122 prints this and exits with status 0
    std::fprintf(stderr, "There are no available device(s) that support CUDA\n");
    std::exit(0);
  }
  if (rc != NWG_OK) die(rc, nullptr, "nwg_ctx_create");
  // the device's tuned kernel table: read from its cache, or measured once
  // (a few seconds) and cached; on failure the built-in table stays
  nwg_autotune(c, 0, nullptr);
  return c;
}

// byte length of the first n sequences of a wire block (SpeciesBlock.cpp:309-322)
size_t wire_bytes(const char* buf, int n) {
  const char* p = buf + sizeof(int);
  for (int s = 0; s < n; ++s) {
    int len;
    p += sizeof(int);
    std::memcpy(&len, p, sizeof(int));
    p += sizeof(int) + len + 1;
  }
  return (size_t)(p - buf);
}

void decode(const char* buf, int n, std::vector<int8_t>& codes, std::vector<int64_t>& off, nwg_ctx* ctx) {
  off.assign((size_t)n + 1, 0);
  int rc = nwg_parse_wire(buf, n, nullptr, off.data());
  if (rc != NWG_OK) die(rc, ctx, "parse");
  codes.assign((size_t)(off[n] > 0 ? off[n] : 1), 0);
  rc = nwg_parse_wire(buf, n, codes.data(), off.data());
  if (rc != NWG_OK) die(rc, ctx, "parse");
}

}  // namespace

AlignmentScore::AlignmentScore(int gapOpen, int gapExt, unsigned int, int)
    : ctx_(make_ctx(gapOpen, gapExt)), xSize(0) {}

AlignmentScore::~AlignmentScore() { nwg_ctx_destroy(ctx_); }

void AlignmentScore::loadDB(char* lbuf, int lSz) {
  xSize = lSz;
  xWire.assign(lbuf, lbuf + wire_bytes(lbuf, lSz));
  decode(lbuf, lSz, xCodes, xOffsets, ctx_);
}

TexVariablesAddresses AlignmentScore::copySeqsToTex(int, int) {
  std::fprintf(stderr, "nwgpu: copySeqsToTex is not used by the GB300 path (no texture windows)\n");
  TexVariablesAddresses t{nullptr, nullptr};
  return t;
}

void AlignmentScore::parse(std::string seqs, std::vector<int>& starts, std::vector<int>& lengths, char* input,
                           int size) {
  // AlignmentScore.cu:142-178 outputs: starts[size+1], lengths[size]; the
  // encoded sequence text went to a by-value copy in the reference and is not
  // returned here either.
  (void)seqs;
  std::vector<int8_t> codes;
  std::vector<int64_t> off;
  decode(input, size, codes, off, ctx_);
  starts.resize((size_t)size + 1);
  lengths.clear();
  for (int s = 0; s <= size; ++s) starts[(size_t)s] = (int)off[(size_t)s];
  for (int s = 0; s < size; ++s) lengths.push_back((int)(off[(size_t)s + 1] - off[(size_t)s]));
}

void AlignmentScore::computeDistanceMtx(char* rbuf, int rSz, std::vector<std::vector<float> >& distances, int r0) {
  if (xSize < 1 || rSz < 1) return;
  const size_t rb = wire_bytes(rbuf, rSz);
  const bool same = rSz == xSize && rb == xWire.size() && std::memcmp(rbuf, xWire.data(), rb) == 0;
  int rc;
  if (same) {
    // the square block of one rank: every pair once, both halves written
    std::vector<float> D((size_t)xSize * xSize);
    rc = nwg_score_all(ctx_, xCodes.data(), xOffsets.data(), xSize, D.data(), xSize, NWG_MODE_BATCHED, nullptr);
    if (rc != NWG_OK) die(rc, ctx_, "computeDistanceMtx");
    for (int x = 0; x < xSize; ++x)
      std::memcpy(&distances[(size_t)x][(size_t)r0], &D[(size_t)x * xSize], sizeof(float) * (size_t)xSize);
    return;
  }
  std::vector<int8_t> yCodes;
  std::vector<int64_t> yOffsets;
  decode(rbuf, rSz, yCodes, yOffsets, ctx_);
  std::vector<float> D((size_t)xSize * rSz);
  rc = nwg_score_block(ctx_, xCodes.data(), xOffsets.data(), xSize, yCodes.data(), yOffsets.data(), rSz, D.data(),
                       rSz, 0, NWG_MODE_BATCHED, nullptr);
  if (rc != NWG_OK) die(rc, ctx_, "computeDistanceMtx");
  for (int x = 0; x < xSize; ++x)
    std::memcpy(&distances[(size_t)x][(size_t)r0], &D[(size_t)x * rSz], sizeof(float) * (size_t)rSz);
}

AlignmentMatch::AlignmentMatch(int gapOpen, int gapExt, unsigned int, int) : ctx_(make_ctx(gapOpen, gapExt)) {}

AlignmentMatch::~AlignmentMatch() { nwg_ctx_destroy(ctx_); }

void AlignmentMatch::prepare(std::vector<std::string>&, int) {
  // The reference encodes a copy and discards it (AlignmentMatch.cu:115-131);
  // encoding happens inside computeAlignment here.
}

TexVariablesAddresses AlignmentMatch::copySeqsToTex(int, int) {
  std::fprintf(stderr, "nwgpu: copySeqsToTex is not used by the GB300 path (no texture windows)\n");
  TexVariablesAddresses t{nullptr, nullptr};
  return t;
}

void AlignmentMatch::computeAlignment(std::vector<iNode>& aSeqs, std::vector<std::string>& seqs, int myProc) {
  computePairwise(aSeqs, seqs, myProc);
  computeMSA(aSeqs, seqs, myProc);
}

void AlignmentMatch::computePairwise(std::vector<iNode>& aSeqs, std::vector<std::string>& seqs, int) {
  std::vector<int> cherry;
  for (size_t k = 0; k < aSeqs.size(); ++k)
    if (aSeqs[k].vecSize == 2 && aSeqs[k].iSpecies.size() >= 2) cherry.push_back((int)k);
  if (cherry.empty()) return;
  // the sequences the cherries name, encoded once
  std::vector<int> used;
  std::vector<int> local(seqs.size(), -1);
  for (int k : cherry)
    for (int s = 0; s < 2; ++s) {
      const int id = aSeqs[(size_t)k].iSpecies[(size_t)s];
      if (id < 0 || (size_t)id >= seqs.size()) die(NWG_ERR_INVALID, ctx_, "computePairwise: species index");
      if (local[(size_t)id] < 0) {
        local[(size_t)id] = (int)used.size();
        used.push_back(id);
      }
    }
  std::string ascii;
  std::vector<int64_t> off(used.size() + 1, 0);
  for (size_t u = 0; u < used.size(); ++u) {
    ascii += seqs[(size_t)used[u]];
    off[u + 1] = (int64_t)ascii.size();
  }
  std::vector<int8_t> codes(ascii.size() > 0 ? ascii.size() : 1);
  int rc = nwg_encode(ascii.data(), off.data(), (int)used.size(), codes.data());
  if (rc != NWG_OK) die(rc, ctx_, "computePairwise: encode");
  std::vector<int32_t> px, py;
  int64_t stride = 1;
  for (int k : cherry) {
    const int a = local[(size_t)aSeqs[(size_t)k].iSpecies[0]], b = local[(size_t)aSeqs[(size_t)k].iSpecies[1]];
    px.push_back(a);
    py.push_back(b);
    const int64_t need = (off[(size_t)a + 1] - off[(size_t)a]) + (off[(size_t)b + 1] - off[(size_t)b]) + 1;
    if (need > stride) stride = need;
  }
  const int m = (int)px.size();
  std::vector<char> ox((size_t)m * stride), oy((size_t)m * stride);
  std::vector<int32_t> len((size_t)m);
  rc = nwg_align_pairs(ctx_, codes.data(), off.data(), (int)used.size(), px.data(), py.data(), m, ox.data(),
                       oy.data(), stride, len.data(), nullptr, nullptr);
  if (rc != NWG_OK) die(rc, ctx_, "computePairwise");
  for (int c = 0; c < m; ++c) {
    iNode& node = aSeqs[(size_t)cherry[(size_t)c]];
    seqs[(size_t)node.iSpecies[0]].assign(&ox[(size_t)c * stride], (size_t)len[(size_t)c]);
    seqs[(size_t)node.iSpecies[1]].assign(&oy[(size_t)c * stride], (size_t)len[(size_t)c]);
    node.aligned = true;
  }
}

void AlignmentMatch::computeMSA(std::vector<iNode>&, std::vector<std::string>&, int) {
  // Profile alignment beyond cherries is not provided (the reference's job
  // loop is empty, AlignmentMatch.cu:428-430).
}

#ifdef NWGPU_COMPAT_LAUNCHERS
namespace {
void not_used(const char* what) {
  std::fprintf(stderr, "nwgpu: %s is a per-window launcher of the reference; the GB300 path does not use it\n", what);
}
}  // namespace
void ScoreKernel(dim3, dim3, short2*, int*, bool) { not_used("ScoreKernel"); }
void MatchKernel(dim3, dim3, short2*, unsigned int*, int*, short, bool) { not_used("MatchKernel"); }
void ReorderMatches(dim3, dim3, unsigned int*, unsigned int*, unsigned int*, unsigned int*, int) {
  not_used("ReorderMatches");
}
void BacktraceKernel(dim3, dim3, unsigned int*, short, unsigned int*, unsigned int*, bool) {
  not_used("BacktraceKernel");
}
#endif
