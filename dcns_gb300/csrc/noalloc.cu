// dcns_semiglobal_noalloc: the 2-piece affine semi-global DP (score and end position) for one pair, with all of its
// scratch in a fixed device array of this file instead of memory the library allocates.
//
// Who needs it: callers that must not allocate device memory at call time.  A host process whose device memory is
// owned by another allocator (a framework's caching pool, a hard per-process budget already handed out) gets
// cudaMalloc failures or fragmentation from a library that allocates on demand, and a latency-bound serving thread
// cannot afford cudaMalloc/cudaFree, which synchronise the device and stall every other stream.  Such a caller passes
// its own device buffers for the inputs and the output; this entry point calls no cudaMalloc, cudaFree or allocating
// library routine.
//
// Limits and sharing: both sequences at most kNaMaxLen bases.  The scratch array (about 1.6 MB) is held by every GPU
// that loads the library until the process exits, and every call on a device shares it: calls whose work overlaps on
// the GPU (different streams, or different host threads without ordering) race on it.  Calls issued in order on one
// stream do not.  The work counter that must start at zero is cleared by each call's set-up kernel, on the caller's
// stream, before the DP kernel runs.
//
// The first call on each device looks up the scratch array's device address with cudaGetSymbolAddress (with that
// device current) and caches it; make that first call before any stream capture.
#include <mutex>

#include "../../include/dcns_gb300.h"
#include "device_common.cuh"
#include "engine.h"

namespace dcns {

constexpr int kNaMaxLen = 16384;

struct NaScratch {
  SgTask task;
  int idx;
  int counter;
  int bad_code;
  int pad;
  uint32_t pk[(2 * (kNaMaxLen + 64) + 128) / 16];
  uint32_t nm[(2 * (kNaMaxLen + 64) + 128) / 32];
  SgRec bnd[kSgNW * (kNaMaxLen + 2)];  // the semi-global kernel's boundary rows of its one CTA
};

static __device__ __align__(256) unsigned char g_na_scratch[sizeof(NaScratch)];

__device__ __forceinline__ void na_pack(const int8_t *src, int n, int64_t base, NaScratch *S, int *bad) {
  const int ngroups = ((n + 63) / 64) * 2;
  for (int g = threadIdx.x; g < ngroups; g += blockDim.x) {
    uint32_t w0 = 0, w1 = 0, nb = 0;
    for (int t = 0; t < 32; ++t) {
      const int k = g * 32 + t;
      if (k >= n) break;
      const int c = src[k];
      uint32_t two = 0;
      if (c == 1)
        two = 1;
      else if (c == 3)
        two = 2;
      else if (c == 4)
        two = 3;
      else if (c != 0) {
        nb |= 1u << t;
        if (c != 2) *bad = 1;
      }
      if (t < 16)
        w0 |= two << (2 * t);
      else
        w1 |= two << (2 * (t - 16));
    }
    S->pk[(base >> 4) + 2 * g] = w0;
    S->pk[(base >> 4) + 2 * g + 1] = w1;
    S->nm[(base >> 5) + g] = nb;
  }
}

// Packs both sequences into the scratch arena and writes the task record; clears the work counter.
__global__ void na_prepare_kernel(NaScratch *S, const int8_t *s1, int n1, const int8_t *s2, int n2) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const int64_t b2 = ((int64_t)n1 + 63) / 64 * 64;
  na_pack(s1, n1, 0, S, &bad);
  na_pack(s2, n2, b2, S, &bad);
  __syncthreads();
  if (threadIdx.x == 0) {
    SgTask t{};
    t.base1 = 0;
    t.base2 = b2;
    t.a1 = 0;
    t.a2 = 0;
    t.n1 = n1;
    t.n2 = n2;
    t.dir = 0;
    t.want_codes = 0;
    S->task = t;
    S->idx = 0;
    S->counter = 0;
    S->bad_code = bad;
  }
}

// Copies the result to the caller's buffer: {maxScore, endPosition1, endPosition2 (0-based), status}.
__global__ void na_finish_kernel(const NaScratch *S, int32_t *out) {
  if (threadIdx.x == 0) {
    const bool bad = S->bad_code != 0;
    out[0] = bad ? -1 : S->task.score;
    out[1] = bad ? -1 : S->task.end1 - 1;
    out[2] = bad ? -1 : S->task.end2 - 1;
    out[3] = bad ? 1 : 0;
  }
}

namespace {
std::mutex g_na_mu;
NaScratch *g_na_ptr[64] = {};
}  // namespace

}  // namespace dcns

extern "C" int dcns_semiglobal_noalloc(const int8_t *d_seq1, int32_t len1, const int8_t *d_seq2, int32_t len2,
                                       const dcns_params *params, int32_t *d_out, void *stream) {
  using namespace dcns;
  if (!params || !d_out || len1 < 0 || len2 < 0 || (len1 > 0 && !d_seq1) || (len2 > 0 && !d_seq2))
    return DCNS_ERR_INVALID;
  if (len1 > kNaMaxLen || len2 > kNaMaxLen) return DCNS_ERR_INVALID;  // the fixed scratch holds at most this much
  Params P;
  try {  // the parameter checks of the allocating entry points, so both accept and reject the same parameters
    P = to_params(params);
    validate(P);
  } catch (const Error &) {
    return DCNS_ERR_INVALID;
  }
  // An error still pending from the caller's earlier CUDA work is reported and left in place for its owner, so that
  // the check after the launches below reports only this call's own launch errors.
  if (cudaPeekAtLastError() != cudaSuccess) return DCNS_ERR_DEVICE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DCNS_ERR_DEVICE;
  NaScratch *S = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
      // the kernel's boundary scratch for one CTA must fit the fixed array (checked once, with the kernel's own sizing)
      if (sg_bnd_bytes(1, kNaMaxLen, kSgNW) > (int64_t)sizeof(NaScratch::bnd)) return DCNS_ERR_DEVICE;
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_na_scratch) != cudaSuccess || !p) {
        (void)cudaGetLastError();  // the failed lookup's own error
        return DCNS_ERR_DEVICE;
      }
      g_na_ptr[dev] = (NaScratch *)p;
    }
    S = g_na_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  na_prepare_kernel<<<1, 256, 0, st>>>(S, d_seq1, len1, d_seq2, len2);
  Arena ar{S->pk, S->nm};
  launch_semiglobal(&S->task, &S->idx, 1, ar, P, nullptr, S->bnd, kNaMaxLen, &S->counter, 1, kSgNW, st);
  na_finish_kernel<<<1, 32, 0, st>>>(S, d_out);
  return cudaGetLastError() == cudaSuccess ? DCNS_OK : DCNS_ERR_DEVICE;
}
