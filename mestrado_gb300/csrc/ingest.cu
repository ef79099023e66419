// ingest.cu -- residue encoding and reversal on the device.
//
// AlignmentScore::parse (AlignmentScore.cu:142-178) turns each sequence of
// the wire block into 8-bit codes (the 24-letter order of :10-27, every other
// byte -1) and reverses it; here one CTA per sequence does the same from a
// device copy of the ASCII (or of the wire block itself), so sequences that
// arrive on the device -- or in the serving loop, every job -- skip the host
// pass.  A byte outside the alphabet is stored as -1, as the reference's
// table does, and counted per sequence; the scoring kernels clamp such codes,
// and every entry point reports them (NWG_ERR_BAD_RESIDUE).
#include <cstring>
#include <vector>

#include "nwg_ctx.h"

namespace nwg {
namespace {

__constant__ int8_t c_table[256];

// dst[dst_off[s] + k] = code(src[src_off[s] + len[s] - 1 - k]); bad[s] = count of -1 codes.
__global__ void __launch_bounds__(128) encode_kernel(const char* __restrict__ src, const int64_t* __restrict__ src_off,
                                                     const int64_t* __restrict__ dst_off, const int32_t* __restrict__ len,
                                                     int n, int8_t* __restrict__ dst, int* __restrict__ bad) {
  const int s = blockIdx.x;
  if (s >= n) return;
  const char* in = src + src_off[s];
  int8_t* out = dst + dst_off[s];
  const int L = len[s];
  int nbad = 0;
  for (int k = threadIdx.x; k < L; k += blockDim.x) {
    const int8_t c = c_table[(unsigned char)in[L - 1 - k]];
    nbad += c < 0;
    out[k] = c;
  }
  for (int o = 16; o > 0; o >>= 1) nbad += __shfl_down_sync(0xffffffffu, nbad, o);
  __shared__ int wb[4];
  if ((threadIdx.x & 31) == 0) wb[threadIdx.x >> 5] = nbad;
  __syncthreads();
  if (threadIdx.x == 0 && bad) bad[s] = wb[0] + wb[1] + wb[2] + wb[3];
}

struct IngestState {
  DevBuf src_off, dst_off, len, bad;
  ~IngestState() {
    for (DevBuf* b : {&src_off, &dst_off, &len, &bad}) b->release();
  }
};

int set_table_once() {
  static bool done = false;
  if (done) return NWG_OK;
  int8_t tab[256];
  for (int k = 0; k < 256; ++k) tab[k] = -1;
  const char* order = letter_order();
  for (int k = 0; k < kLetters; ++k) tab[(unsigned char)order[k]] = (int8_t)k;
  if (cudaMemcpyToSymbol(c_table, tab, sizeof(tab)) != cudaSuccess) {
    cudaGetLastError();
    return NWG_ERR_CUDA;
  }
  done = true;
  return NWG_OK;
}

}  // namespace

// Shared by the C entry points and the serving loop: n sequences, their
// positions in src / dst and lengths already on the device (d_* arrays).
cudaError_t launch_encode(const char* d_src, const int64_t* d_src_off, const int64_t* d_dst_off, const int32_t* d_len,
                          int n, int8_t* d_dst, int* d_bad, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (set_table_once() != NWG_OK) return cudaErrorUnknown;
  encode_kernel<<<n, 128, 0, s>>>(d_src, d_src_off, d_dst_off, d_len, n, d_dst, d_bad);
  return cudaGetLastError();
}

// Host arrays of positions and lengths -> device, launch, optional bad count.
static int encode_dev(Ctx* c, const char* d_src, const std::vector<int64_t>& src_off, const int64_t* dst_off, int n,
                      int8_t* d_dst, int64_t* bad_count) {
  auto* st = reinterpret_cast<IngestState*>(c->ingest_state);
  if (!st) c->ingest_state = st = new IngestState();
  int rc;
  if ((rc = st->src_off.ensure(sizeof(int64_t) * n)) || (rc = st->dst_off.ensure(sizeof(int64_t) * n)) ||
      (rc = st->len.ensure(sizeof(int32_t) * n)) || (rc = st->bad.ensure(sizeof(int) * n)))
    return c->fail(rc, "encode allocation");
  std::vector<int32_t> len(n);
  for (int k = 0; k < n; ++k) {
    const int64_t L = dst_off[k + 1] - dst_off[k];
    if (L <= 0) return c->fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
    len[k] = (int32_t)L;
  }
  cudaStream_t s = c->stream;
  if ((rc = c->cuda(cudaMemcpyAsync(st->src_off.p, src_off.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s),
                    "encode upload")) ||
      (rc = c->cuda(cudaMemcpyAsync(st->dst_off.p, dst_off, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s),
                    "encode upload")) ||
      (rc = c->cuda(cudaMemcpyAsync(st->len.p, len.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s),
                    "encode upload")) ||
      (rc = c->cuda(launch_encode(d_src, (const int64_t*)st->src_off.p, (const int64_t*)st->dst_off.p,
                                  (const int32_t*)st->len.p, n, d_dst, (int*)st->bad.p, s),
                    "encode launch")))
    return rc;
  std::vector<int> bad(n);
  if ((rc = c->cuda(cudaMemcpyAsync(bad.data(), st->bad.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s), "encode")) ||
      (rc = c->cuda(cudaStreamSynchronize(s), "encode sync")))
    return rc;
  int64_t nb = 0;
  for (int k = 0; k < n; ++k) nb += bad[k];
  if (bad_count) *bad_count = nb;
  return nb ? NWG_ERR_BAD_RESIDUE : NWG_OK;
}

void Ctx::ingest_release() {
  delete reinterpret_cast<IngestState*>(ingest_state);
  ingest_state = nullptr;
}

}  // namespace nwg

using nwg::Ctx;

extern "C" {

int nwg_encode_dev(nwg_ctx* ctx, const char* d_ascii, const int64_t* offsets, int n, int8_t* d_codes,
                   int64_t* bad_count) {
  if (!ctx || !d_ascii || !offsets || !d_codes || n < 1) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  std::vector<int64_t> src(offsets, offsets + n);
  return nwg::encode_dev(c, d_ascii, src, offsets, n, d_codes, bad_count);
}

int nwg_parse_wire_dev(nwg_ctx* ctx, const char* wire, const char* d_wire, int n, int8_t* d_codes,
                       int64_t* offsets, int64_t* bad_count) {
  if (!ctx || !wire || !d_wire || !offsets || n < 1) return NWG_ERR_INVALID;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  // headers walked on the host (SpeciesBlock.cpp:309-322 layout), residues on the device
  std::vector<int64_t> src(n);
  const char* p = wire + sizeof(int);
  offsets[0] = 0;
  for (int s = 0; s < n; ++s) {
    int len;
    p += sizeof(int);
    std::memcpy(&len, p, sizeof(int));
    p += sizeof(int);
    if (len <= 0) return c->fail(NWG_ERR_EMPTY_SEQ, "zero-length sequence");
    src[s] = (int64_t)(p - wire);
    offsets[s + 1] = offsets[s] + len;
    p += len + 1;
  }
  if (!d_codes) return NWG_OK;
  return nwg::encode_dev(c, d_wire, src, offsets, n, d_codes, bad_count);
}

}  // extern "C"
