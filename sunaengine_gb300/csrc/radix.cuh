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
// Per pass: hist (per tile, per digit) -> exclusive scan of every digit's row
// of tile counts (one CTA per digit) -> scatter, whose prologue scans the
// digit totals itself (one thread per digit). The tile (512 threads x IT
// items) is picked per sort so that even a few hundred thousand keys spread
// over ~128 CTAs.
#pragma once
#include <algorithm>
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
constexpr int MAX_ITEMS = 16;            // items per thread, largest tile
constexpr int MIN_TILES = 128;           // a sort spreads over at least this many tiles when it can
static_assert(TPB == RADIX, "one thread per digit in the histogram and scatter prologues");

__device__ __forceinline__ uint32_t digit_of(const uint32_t* keys, uint32_t idx, uint32_t n, int shift) {
  return idx < n ? ((keys[idx] >> shift) & (RADIX - 1)) : (uint32_t)RADIX;
}

template <int IT>
__device__ __forceinline__ void warp_counts(const uint32_t* keys, uint32_t n, int shift, uint32_t tileBase,
                                            uint32_t (*cnt)[RADIX + 1], int warp, int lane) {
#pragma unroll 4
  for (int r = 0; r < IT; ++r) {
    uint32_t idx = tileBase + warp * (32 * IT) + r * 32 + lane;
    uint32_t d = digit_of(keys, idx, n, shift);
    uint32_t m = __match_any_sync(0xffffffffu, d);
    if (lane == __ffs(m) - 1) cnt[warp][d] += __popc(m);
    __syncwarp();
  }
}

template <int IT>
__global__ void __launch_bounds__(TPB) k_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                              uint32_t* __restrict__ hist, uint32_t numTiles) {
  __shared__ uint32_t cnt[WARPS][RADIX + 1];
  int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < WARPS * (RADIX + 1); i += TPB) (&cnt[0][0])[i] = 0;
  __syncthreads();
  uint32_t tile = blockIdx.x;
  warp_counts<IT>(keys, n, shift, tile * (TPB * IT), cnt, warp, lane);
  __syncthreads();
  uint32_t s = 0;
  for (int w = 0; w < WARPS; ++w) s += cnt[w][tid];
  hist[(uint32_t)tid * numTiles + tile] = s;
}

// One CTA per digit: exclusive scan of that digit's row of tile counts, in
// place; the row total goes to totals[digit].
constexpr int ROW_T = 256;
__global__ void __launch_bounds__(ROW_T) k_scan_rows(uint32_t* __restrict__ hist, uint32_t numTiles,
                                                     uint32_t* __restrict__ totals) {
  __shared__ uint32_t ws[ROW_T / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t* row = hist + (size_t)blockIdx.x * numTiles;
  uint32_t carry = 0;
  for (uint32_t base = 0; base < numTiles; base += ROW_T) {
    const uint32_t i = base + tid;
    const uint32_t v = i < numTiles ? row[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    uint32_t before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < ROW_T / 32; ++w) {
      if (w < warp) before += ws[w];
      all += ws[w];
    }
    if (i < numTiles) row[i] = carry + before + x - v;
    carry += all;
    __syncthreads();
  }
  if (tid == 0) totals[blockIdx.x] = carry;
}

// valsIn == nullptr means the values are the input indices (first pass).
template <int IT>
__global__ void __launch_bounds__(TPB) k_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ valsIn,
                                                 uint32_t n, int shift, const uint32_t* __restrict__ offs,
                                                 const uint32_t* __restrict__ totals, uint32_t numTiles,
                                                 uint32_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut) {
  __shared__ uint32_t cnt[WARPS][RADIX + 1];
  __shared__ uint32_t wsum[WARPS];
  int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < WARPS * (RADIX + 1); i += TPB) (&cnt[0][0])[i] = 0;
  // exclusive scan of the digit totals (k_scan_rows left each row's sum)
  const uint32_t tv = totals[tid];
  uint32_t tx = tv;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, tx, o);
    if (lane >= o) tx += t;
  }
  if (lane == 31) wsum[warp] = tx;
  __syncthreads();
  uint32_t digitBase = tx - tv;
  for (int w = 0; w < warp; ++w) digitBase += wsum[w];
  uint32_t tile = blockIdx.x, tileBase = tile * (TPB * IT);
  warp_counts<IT>(keys, n, shift, tileBase, cnt, warp, lane);
  __syncthreads();
  {
    uint32_t run = digitBase + offs[(uint32_t)tid * numTiles + tile];
    for (int w = 0; w < WARPS; ++w) {
      uint32_t t = cnt[w][tid];
      cnt[w][tid] = run;
      run += t;
    }
  }
  __syncthreads();
  const uint32_t ltmask = (1u << lane) - 1u;
#pragma unroll 4
  for (int r = 0; r < IT; ++r) {
    uint32_t idx = tileBase + warp * (32 * IT) + r * 32 + lane;
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

// Items per thread for n keys: the smallest power of two (1..16) that keeps
// the tile count at or below MIN_TILES, so small sorts still fill the GPU.
inline int items_for(uint32_t n) {
  int it = 1;
  while (it < MAX_ITEMS && (uint64_t)TPB * it * MIN_TILES < n) it <<= 1;
  return it;
}

template <int IT>
inline void sort_pass(const uint32_t* kin, const uint32_t* vin, uint32_t n, int shift, uint32_t* hist,
                      uint32_t* ko, uint32_t* vo, cudaStream_t st) {
  const uint32_t numTiles = (n + TPB * IT - 1) / (TPB * IT);
  uint32_t* totals = hist + (size_t)RADIX * numTiles;
  k_hist<IT><<<numTiles, TPB, 0, st>>>(kin, n, shift, hist, numTiles);
  k_scan_rows<<<RADIX, ROW_T, 0, st>>>(hist, numTiles, totals);
  k_scatter<IT><<<numTiles, TPB, 0, st>>>(kin, vin, n, shift, hist, totals, numTiles, ko, vo);
}

// Sort n pairs. keys0 is consumed; the result lands in (outKeys, outVals).
// tmpK/tmpV are scratch of n words; hist needs hist_words(n) words.
// Kernel launches: 3 per pass of RBITS key bits.
inline void sort_pairs(uint32_t* keys0, uint32_t n, int keyBits, uint32_t* outKeys, uint32_t* outVals,
                       uint32_t* tmpK, uint32_t* tmpV, uint32_t* hist, cudaStream_t st) {
  if (n == 0) return;
  int passes = (keyBits + RBITS - 1) / RBITS;
  if (passes < 1) passes = 1;
  const int it = items_for(n);
  const uint32_t* kin = keys0;
  const uint32_t* vin = nullptr;
  for (int p = 0; p < passes; ++p) {
    // ping-pong so that the final pass writes (outKeys, outVals)
    bool toOut = ((passes - 1 - p) % 2) == 0;
    uint32_t* ko = toOut ? outKeys : tmpK;
    uint32_t* vo = toOut ? outVals : tmpV;
    int shift = p * RBITS;
    switch (it) {
      case 1: sort_pass<1>(kin, vin, n, shift, hist, ko, vo, st); break;
      case 2: sort_pass<2>(kin, vin, n, shift, hist, ko, vo, st); break;
      case 4: sort_pass<4>(kin, vin, n, shift, hist, ko, vo, st); break;
      case 8: sort_pass<8>(kin, vin, n, shift, hist, ko, vo, st); break;
      default: sort_pass<16>(kin, vin, n, shift, hist, ko, vo, st); break;
    }
    kin = ko;
    vin = vo;
  }
}

constexpr int LAUNCHES_PER_PASS = 3;

// Words of `hist` a sort of up to n keys needs (tile counts plus the digit totals).
inline size_t hist_words(uint32_t n) {
  const uint32_t tiles = (n + TPB * items_for(n) - 1) / (TPB * items_for(n));
  return (size_t)RADIX * (std::max<uint32_t>(tiles, MIN_TILES) + 2);
}

}  // namespace
}  // namespace radix
}  // namespace sn
