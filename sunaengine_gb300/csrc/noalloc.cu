// State digest of a caller-owned device buffer, with no device allocation.
//
// Who needs this: hosts that cannot call cudaMalloc at the moment they want
// a digest. cudaMalloc can synchronise the device, which a latency-bound
// caller stepping other streams cannot afford, and an embedding host that
// hands out device memory from its own fixed pool may forbid libraries from
// allocating at all. Such a caller owns the state buffer and the 8-word
// result buffer and only needs the engine's digest of it (H_set || H_slot,
// the reference's statehash digest).
//
// The per-block partial digests live in `g_partials`, a fixed array in this
// library's device image: 2048 blocks x 8 words (64 KiB). Every GPU that
// loads the library holds that array until the process exits. Each block
// covers up to 8192 particles, so one call digests at most 16,777,216
// particles; larger requests are refused before anything is launched.
//
// The array is shared by every call on a device. Each call overwrites exactly
// the partials it then reads, so nothing has to start at zero, but two calls
// whose kernels overlap on the GPU (different streams, no ordering between
// them) race on the array and may return wrong digests. Order them on one
// stream, or synchronise between them.
//
// Host code cannot pass `g_partials` itself to a kernel: in host code the
// name denotes a host-side stand-in, not the device address. The device
// address is fetched with cudaGetSymbolAddress, with the caller's context
// current, by the first call made under each CUDA context, and kept under
// that context's process-unique id (cuCtxGetId). A context created later
// (a second context on the same device, or the new primary context after
// cudaDeviceReset) has a new id and gets its own lookup, so an address is
// never reused outside the context it was fetched in.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdio>
#include <mutex>

#include "../../include/suna.h"
#include "statehash.cuh"

namespace {

constexpr uint32_t NA_THREADS = 256;
constexpr uint32_t NA_PER_BLOCK = 8192;  // particles one block digests
constexpr uint32_t NA_MAX_BLOCKS = 2048;
constexpr uint32_t NA_MAX_PARTICLES = NA_PER_BLOCK * NA_MAX_BLOCKS;  // 16,777,216
static_assert(NA_MAX_PARTICLES == SN_NOALLOC_MAX_PARTICLES, "suna.h states the same particle limit");
constexpr int NA_CACHE = 32;  // contexts remembered; older entries are looked up again

static __device__ __align__(256) uint32_t g_partials[NA_MAX_BLOCKS * 8];

struct CtxAddr {
  unsigned long long id;
  uint32_t* addr;
};
std::mutex g_mu;
CtxAddr g_cache[NA_CACHE] = {};
int g_used = 0, g_next = 0;

// Pass 1: block b digests particles [b*8192, (b+1)*8192) and writes its 8
// partial lane sums to partials[b]. u32 addition is commutative, so the split
// gives the same digest as the engine's own accumulation.
__global__ void __launch_bounds__(NA_THREADS) k_na_partial(const int32_t* __restrict__ state, uint32_t n,
                                                           uint32_t nFluid, const uint32_t* __restrict__ bond,
                                                           uint32_t* __restrict__ partials) {
  __shared__ uint32_t ws[NA_THREADS / 32][8];
  uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const uint32_t lo = blockIdx.x * NA_PER_BLOCK;
  const uint32_t hi = min(n, lo + NA_PER_BLOCK);
  for (uint32_t i = lo + threadIdx.x; i < hi; i += NA_THREADS) {
    uint32_t h[8];
    const uint32_t* row = (bond && i < nFluid) ? bond + (size_t)i * sn::BOND_CAP : nullptr;
    sn::d2::particle_digest(state + (size_t)i * 8, i, row, h);
#pragma unroll
    for (int l = 0; l < 8; ++l) acc[l] += h[l];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    uint32_t v = __reduce_add_sync(0xffffffffu, acc[l]);
    if (lane == 0) ws[warp][l] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    uint32_t s = 0;
    for (int w = 0; w < (int)(NA_THREADS / 32); ++w) s += ws[w][threadIdx.x];
    partials[blockIdx.x * 8 + threadIdx.x] = s;
  }
}

// Pass 2: one block adds the partials in block order into out[8].
__global__ void __launch_bounds__(NA_THREADS) k_na_final(const uint32_t* __restrict__ partials, uint32_t blocks,
                                                         uint32_t* __restrict__ out) {
  __shared__ uint32_t ws[NA_THREADS / 32][8];
  uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (uint32_t blk = threadIdx.x; blk < blocks; blk += NA_THREADS)
#pragma unroll
    for (int l = 0; l < 8; ++l) acc[l] += partials[blk * 8 + l];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    uint32_t v = __reduce_add_sync(0xffffffffu, acc[l]);
    if (lane == 0) ws[warp][l] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    uint32_t s = 0;
    for (int w = 0; w < (int)(NA_THREADS / 32); ++w) s += ws[w][threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// The driver's process-unique id of the calling thread's current context, or
// false when no context is current. The two driver calls are fetched through
// the runtime, so the library needs no link against libcuda.
using CtxGetCurrentFn = CUresult(CUDAAPI*)(CUcontext*);
using CtxGetIdFn = CUresult(CUDAAPI*)(CUcontext, unsigned long long*);
bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess)
      return false;
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

// The device address of g_partials in the calling thread's current context.
// The first call under a context looks it up; later calls under the same
// context reuse it.
uint32_t* partials_in_current_context() {
  std::lock_guard<std::mutex> lock(g_mu);
  unsigned long long id = 0;
  const bool known = current_context_id(&id);
  if (known)
    for (int k = 0; k < g_used; ++k)
      if (g_cache[k].id == id) return g_cache[k].addr;
  // With no context current yet, this lookup is the runtime call that binds
  // the device's primary context; the id is read after it.
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
  if (e != cudaSuccess) {
    int dev = -1;
    cudaGetDevice(&dev);
    fprintf(stderr, "[suna] sn_digest_device_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
            cudaGetErrorString(e));
    return nullptr;
  }
  if (!known && !current_context_id(&id)) return static_cast<uint32_t*>(p);  // not cached: looked up next call
  const int k = g_used < NA_CACHE ? g_used++ : (g_next++ % NA_CACHE);
  g_cache[k] = CtxAddr{id, static_cast<uint32_t*>(p)};
  return g_cache[k].addr;
}

}  // namespace

extern "C" int sn_digest_device_noalloc(const int32_t* d_state, uint32_t n, uint32_t n_fluid,
                                        const uint32_t* d_bond, uint32_t* d_out, void* stream) {
  if (!d_state || !d_out || n_fluid > n) return SN_E_INVALID;
  if (n > NA_MAX_PARTICLES) {
    fprintf(stderr,
            "[suna] sn_digest_device_noalloc: n = %u exceeds the no-allocation limit of %u particles "
            "(%u blocks of %u)\n",
            n, NA_MAX_PARTICLES, NA_MAX_BLOCKS, NA_PER_BLOCK);
    return SN_E_CAPACITY;
  }
  uint32_t* partials = partials_in_current_context();
  if (!partials) return SN_E_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint32_t blocks = (n + NA_PER_BLOCK - 1) / NA_PER_BLOCK;
  if (blocks == 0) blocks = 1;  // n == 0: one empty block writes zero partials
  k_na_partial<<<blocks, NA_THREADS, 0, st>>>(d_state, n, n_fluid, d_bond, partials);
  k_na_final<<<1, NA_THREADS, 0, st>>>(partials, blocks, d_out);
  return cudaGetLastError() == cudaSuccess ? SN_OK : SN_E_CUDA;
}
