// es_noalloc.cu -- a primality test over caller-owned device buffers that allocates nothing.
//
// Some callers cannot allocate device memory: code that runs while its host process holds a
// fixed device-memory budget handed out by someone else (a serving process that reserved
// everything up front), code that runs where cudaMalloc is not allowed to block or fail at
// run time, and callers in a framework that owns every device allocation. They already hold
// the input and output buffers on the device and need only the work done.
//
// es_is_prime_noalloc runs the engine's two-pass Miller-Rabin (a base-2 round with a thread
// per value, then the 12-base test with one base per lane of a warp for the values that pass)
// with its scratch -- the list of values that passed the first round and its counter -- in a
// file-scope __device__ array of fixed size instead of in memory from cudaMalloc. That array
// exists once per GPU that loads the library and stays allocated until the process exits.
#include "../../include/es_sieve.h"
#include "es_arith.cuh"
#include "es_tail.cuh"

#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>

namespace es {

// Scratch: word 0 is the counter of values that passed the base-2 round, words
// [NOALLOC_LIST, NOALLOC_LIST + ES_NOALLOC_MAX) their indices.
constexpr u32 NOALLOC_LIST = 64;   // keeps the list 256-byte aligned
static __device__ __align__(256) u32 g_noalloc_scratch[NOALLOC_LIST + ES_NOALLOC_MAX];

__global__ void k_noalloc_round1(const u64 *__restrict__ n, u64 count, unsigned char *__restrict__ out,
                                 u32 *__restrict__ scratch) {
  u32 *cnt = scratch;
  u32 *list = scratch + NOALLOC_LIST;
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (u64)gridDim.x * blockDim.x) {
    if (sprp2_64(n[i])) list[atomicAdd(cnt, 1u)] = (u32)i;   // at most count <= ES_NOALLOC_MAX entries
    else out[i] = 0;
  }
}

__global__ void k_noalloc_round2(const u64 *__restrict__ n, unsigned char *__restrict__ out,
                                 const u32 *__restrict__ scratch) {
  const u32 lane = threadIdx.x & 31;
  const u64 warps = (u64)gridDim.x * blockDim.x / 32;
  const u32 m = scratch[0];
  const u32 *list = scratch + NOALLOC_LIST;
  for (u64 k = ((u64)blockIdx.x * blockDim.x + threadIdx.x) / 32; k < m; k += warps) {
    const u32 i = list[k];
    const bool prime = warp_is_prime(n[i], lane);
    if (lane == 0) out[i] = prime ? 1 : 0;
  }
}

// The device address of the scratch array, looked up once per CUDA context with that
// context current (in host code g_noalloc_scratch names a host-side stand-in, never the device
// array). The cache is keyed by the driver's context id, which no later context reuses: after a
// cudaDeviceReset the device's new primary context gets a new id, so the address is looked up
// again in the new context instead of pointing into the destroyed one.
typedef int (*CtxGetCurrentFn)(void **ctx);
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);
static std::mutex g_noalloc_mu;
static std::unordered_map<unsigned long long, u32 *> g_noalloc_ptr;
static CtxGetCurrentFn g_ctx_get_current = nullptr;
static CtxGetIdFn g_ctx_get_id = nullptr;

static cudaError_t noalloc_scratch(u32 **out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return cudaErrorNotSupported;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != 0 || !ctx || g_ctx_get_id(ctx, &id) != 0) return cudaErrorDeviceUninitialized;
  auto it = g_noalloc_ptr.find(id);
  if (it == g_noalloc_ptr.end()) {
    void *p = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess) return err;
    it = g_noalloc_ptr.emplace(id, static_cast<u32 *>(p)).first;
  }
  *out = it->second;
  return cudaSuccess;
}

}  // namespace es

extern "C" es_status es_is_prime_noalloc(const uint64_t *d_n, size_t count, uint8_t *d_out, void *stream) {
  using namespace es;
  if (count == 0) return ES_OK;
  if (!d_n || !d_out) return ES_ERR_ARG;
  if (count > ES_NOALLOC_MAX) return ES_ERR_ARG;     // the scratch list holds ES_NOALLOC_MAX indices
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ES_ERR_CUDA;
  // makes the device's primary context current on this thread (it allocates nothing)
  if (cudaSetDevice(dev) != cudaSuccess) return ES_ERR_CUDA;
  u32 *scratch = nullptr;
  if (noalloc_scratch(&scratch) != cudaSuccess) return ES_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ES_ERR_CUDA;
  // the counter carries the previous call's value: clear it first, on the caller's stream
  if (cudaMemsetAsync(scratch, 0, sizeof(u32), s) != cudaSuccess) return ES_ERR_CUDA;
  k_noalloc_round1<<<sms * 2, 256, 0, s>>>(reinterpret_cast<const u64 *>(d_n), count, d_out, scratch);
  if (cudaGetLastError() != cudaSuccess) return ES_ERR_CUDA;
  k_noalloc_round2<<<sms * 2, 256, 0, s>>>(reinterpret_cast<const u64 *>(d_n), d_out, scratch);
  if (cudaGetLastError() != cudaSuccess) return ES_ERR_CUDA;
  return ES_OK;
}
