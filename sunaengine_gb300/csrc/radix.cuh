// Stable, atomic-free LSD radix sort of (u32 key, u32 value) pairs.
//
// This is the grid's counting sort. The reference builds its grid with an
// atomicAdd histogram and an atomic scatter, then restores a canonical order
// with an O(k^2)-per-cell `canonicalize` pass (src/sim.wgsl:1009-1168). Here
// the inputs arrive in slot order and every pass is stable, so the output is
// already in (cell, ascending slot) order: the canonical order, with no
// atomics anywhere. Ranking inside a warp uses __match_any_sync + popc; each
// digit has exactly one leader lane per round, so the per-warp counters in
// shared memory never see a conflicting write.
//
// Per pass: hist (per tile, per digit) -> one-CTA exclusive scan over the
// digit-major [digit][tile] matrix -> scatter.
#pragma once
#include <cstdint>

namespace sn {
namespace radix {
// Internal linkage: every translation unit that sorts gets its own copy of
// these kernels, so several engines can include this header.
namespace {

constexpr int RBITS = 9;
constexpr int RADIX = 1 << RBITS;
constexpr int TPB = 512;                 // threads per tile
constexpr int WARPS = TPB / 32;
constexpr int ITEMS = 16;                // items per thread
constexpr int TILE = TPB * ITEMS;        // 8192 items per tile
constexpr int WARP_ITEMS = 32 * ITEMS;   // 512 items per warp, in 16 rounds of 32
static_assert(TPB == RADIX, "one thread per digit in the histogram and scatter prologues");

__device__ __forceinline__ uint32_t digit_of(const uint32_t* keys, uint32_t idx, uint32_t n, int shift) {
  return idx < n ? ((keys[idx] >> shift) & (RADIX - 1)) : (uint32_t)RADIX;
}

__device__ __forceinline__ void warp_counts(const uint32_t* keys, uint32_t n, int shift, uint32_t tileBase,
                                            uint32_t (*cnt)[RADIX + 1], int warp, int lane) {
  for (int r = 0; r < ITEMS; ++r) {
    uint32_t idx = tileBase + warp * WARP_ITEMS + r * 32 + lane;
    uint32_t d = digit_of(keys, idx, n, shift);
    uint32_t m = __match_any_sync(0xffffffffu, d);
    if (lane == __ffs(m) - 1) cnt[warp][d] += __popc(m);
    __syncwarp();
  }
}

__global__ void __launch_bounds__(TPB) k_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                              uint32_t* __restrict__ hist, uint32_t numTiles) {
  __shared__ uint32_t cnt[WARPS][RADIX + 1];
  int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < WARPS * (RADIX + 1); i += TPB) (&cnt[0][0])[i] = 0;
  __syncthreads();
  uint32_t tile = blockIdx.x;
  warp_counts(keys, n, shift, tile * TILE, cnt, warp, lane);
  __syncthreads();
  uint32_t s = 0;
  for (int w = 0; w < WARPS; ++w) s += cnt[w][tid];
  hist[(uint32_t)tid * numTiles + tile] = s;
}

// Exclusive scan of m words in place, one CTA of 1024 threads: tiles of 8192
// words are staged through shared memory with coalesced loads and stores, each
// thread scans 8 contiguous words, a warp-shuffle scan joins the threads, and
// a carry links the tiles.
constexpr int SCAN_T = 1024, SCAN_I = 8, SCAN_TILE = SCAN_T * SCAN_I;
__global__ void __launch_bounds__(SCAN_T) k_scan(uint32_t* __restrict__ a, uint32_t m) {
  __shared__ uint32_t buf[SCAN_TILE + SCAN_TILE / 32];
  __shared__ uint32_t ws[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto at = [](int i) { return i + (i >> 5); };  // pad one word per 32 against bank conflicts
  uint32_t carry = 0;
  for (uint32_t base = 0; base < m; base += SCAN_TILE) {
    for (int k = 0; k < SCAN_I; ++k) {
      uint32_t i = base + k * SCAN_T + tid;
      buf[at(k * SCAN_T + tid)] = i < m ? a[i] : 0u;
    }
    __syncthreads();
    uint32_t v[SCAN_I], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) { v[k] = buf[at(tid * SCAN_I + k)]; s += v[k]; }
    uint32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = ws[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      ws[lane] = w;
    }
    __syncthreads();
    uint32_t run = carry + x - s + (warp > 0 ? ws[warp - 1] : 0u);
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) { buf[at(tid * SCAN_I + k)] = run; run += v[k]; }
    const uint32_t total = ws[31];
    __syncthreads();
    for (int k = 0; k < SCAN_I; ++k) {
      uint32_t i = base + k * SCAN_T + tid;
      if (i < m) a[i] = buf[at(k * SCAN_T + tid)];
    }
    carry += total;
    __syncthreads();
  }
}

// valsIn == nullptr means the values are the input indices (first pass).
__global__ void __launch_bounds__(TPB) k_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ valsIn,
                                                 uint32_t n, int shift, const uint32_t* __restrict__ offs,
                                                 uint32_t numTiles, uint32_t* __restrict__ keysOut,
                                                 uint32_t* __restrict__ valsOut) {
  __shared__ uint32_t cnt[WARPS][RADIX + 1];
  int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < WARPS * (RADIX + 1); i += TPB) (&cnt[0][0])[i] = 0;
  __syncthreads();
  uint32_t tile = blockIdx.x, tileBase = tile * TILE;
  warp_counts(keys, n, shift, tileBase, cnt, warp, lane);
  __syncthreads();
  {
    uint32_t run = offs[(uint32_t)tid * numTiles + tile];
    for (int w = 0; w < WARPS; ++w) {
      uint32_t t = cnt[w][tid];
      cnt[w][tid] = run;
      run += t;
    }
  }
  __syncthreads();
  const uint32_t ltmask = (1u << lane) - 1u;
  for (int r = 0; r < ITEMS; ++r) {
    uint32_t idx = tileBase + warp * WARP_ITEMS + r * 32 + lane;
    uint32_t d = digit_of(keys, idx, n, shift);
    uint32_t m = __match_any_sync(0xffffffffu, d);
    uint32_t base = cnt[warp][d];
    __syncwarp();
    if (d < (uint32_t)RADIX) {
      uint32_t pos = base + __popc(m & ltmask);
      keysOut[pos] = keys[idx];
      valsOut[pos] = valsIn ? valsIn[idx] : idx;
    }
    if (lane == __ffs(m) - 1) cnt[warp][d] = base + __popc(m);
    __syncwarp();
  }
}

// Sort n pairs. keys0 is consumed; the result lands in (outKeys, outVals).
// tmpK/tmpV are scratch of n words; hist needs RADIX * ceil(n / TILE) words.
inline void sort_pairs(uint32_t* keys0, uint32_t n, int keyBits, uint32_t* outKeys, uint32_t* outVals,
                       uint32_t* tmpK, uint32_t* tmpV, uint32_t* hist, cudaStream_t st) {
  if (n == 0) return;
  uint32_t numTiles = (n + TILE - 1) / TILE;
  int passes = (keyBits + RBITS - 1) / RBITS;
  if (passes < 1) passes = 1;
  const uint32_t* kin = keys0;
  const uint32_t* vin = nullptr;
  for (int p = 0; p < passes; ++p) {
    // ping-pong so that the final pass writes (outKeys, outVals)
    bool toOut = ((passes - 1 - p) % 2) == 0;
    uint32_t* ko = toOut ? outKeys : tmpK;
    uint32_t* vo = toOut ? outVals : tmpV;
    int shift = p * RBITS;
    k_hist<<<numTiles, TPB, 0, st>>>(kin, n, shift, hist, numTiles);
    k_scan<<<1, SCAN_T, 0, st>>>(hist, RADIX * numTiles);
    k_scatter<<<numTiles, TPB, 0, st>>>(kin, vin, n, shift, hist, numTiles, ko, vo);
    kin = ko;
    vin = vo;
  }
}

inline size_t hist_words(uint32_t n) { return (size_t)RADIX * ((n + TILE - 1) / TILE + 1); }

}  // namespace
}  // namespace radix
}  // namespace sn
