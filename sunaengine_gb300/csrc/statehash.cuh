// The reference's canonical state digest (src/hash/statehash.js:36-169,
// src/hash/statehash.wgsl:54-170): MurmurHash3_x86_32 body and finalizer run as
// 4 salted lanes over each particle's 8 state words, giving per particle the 8
// words that are u32-added across particles (H_set lanes 0..3, H_slot 4..7),
// with the optional commutative bond fold, plus the per-substep chain fold.
#pragma once
#include <cstdint>
#include "world.cuh"

namespace sn {
namespace d2 {

__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return __funnelshift_l(x, x, r); }
__device__ __forceinline__ uint32_t mm_step(uint32_t h, uint32_t k) {
  k *= 0xcc9e2d51u;
  k = rotl32(k, 15);
  k *= 0x1b873593u;
  h ^= k;
  h = rotl32(h, 13);
  return h * 5u + 0xe6546b64u;
}
__device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}
// The 8 digest lanes one particle contributes (u32-added across particles).
__device__ __forceinline__ void particle_digest(const int32_t* w8, uint32_t idx, const uint32_t* bondRow,
                                                uint32_t out[8]) {
  const uint32_t SEED[4] = {0x9e3779b1u, 0x85ebca77u, 0xc2b2ae3du, 0x27d4eb2fu};
  const uint32_t SALT[4] = {0x00000000u, 0x51633e2du, 0x9c8f2a17u, 0xd0e5b943u};
  uint32_t h[4] = {SEED[0], SEED[1], SEED[2], SEED[3]};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    uint32_t w = (uint32_t)w8[k];
#pragma unroll
    for (int l = 0; l < 4; ++l) h[l] = mm_step(h[l], w ^ SALT[l]);
  }
  uint32_t s[4], t[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) { s[l] = h[l]; t[l] = h[l]; }
  if (bondRow) {
    uint32_t bn = 0, com = 0, scom = 0;
    for (int k = 0; k < BOND_CAP; ++k) {
      uint32_t w = bondRow[k];
      if (w == 0u) break;
      com += fmix32(((w >> 17) & 0x1fffu) ^ 0x5bd1e995u);
      scom += fmix32(w ^ 0x2f5b3c17u);
      bn++;
    }
    if (bn) {
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        s[l] = mm_step(s[l], bn) ^ com;
        t[l] = mm_step(t[l], bn) ^ scom;
      }
    }
  }
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    out[l] = fmix32(s[l] ^ 8u);
    out[4 + l] = fmix32(mm_step(t[l], idx) ^ 9u);
  }
}

// Warp-aggregated u32 add of 8 digest words into acc[scene]. Lanes with
// valid == false contribute nothing. Addition mod 2^32 is commutative, so the
// digest does not depend on the order in which warps land.
__device__ __forceinline__ void digest_add(uint32_t* acc, bool valid, uint32_t scene, const uint32_t h[8]) {
  uint32_t key = valid ? scene : 0xffffffffu;
  uint32_t peers = __match_any_sync(0xffffffffu, key);
  int lane = threadIdx.x & 31;
  bool leader = lane == __ffs(peers) - 1;
  if (peers == 0xffffffffu) {
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      uint32_t t = __reduce_add_sync(0xffffffffu, h[l]);
      if (leader && valid) atomicAdd(acc + scene * 8 + l, t);
    }
    return;
  }
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    uint32_t v = h[l], total = 0, m = peers;
    while (m) {
      int src = __ffs(m) - 1;
      m &= m - 1;
      total += __shfl_sync(peers, v, src);
    }
    if (leader && valid) atomicAdd(acc + scene * 8 + l, total);
  }
}

// Block-level digest accumulation. Almost every warp of a block hashes
// particles of one scene; their warp sums go to 8 shared-memory words (the
// first scene a warp leader claims for the block) and reach global memory with
// 8 atomics per block at the end, instead of 8 same-address global atomics per
// warp. Warps of any other scene add to global memory directly. u32 addition
// is commutative and associative, so the totals are exact in any order.
// digest_block_begin/end must be reached by every thread of the block.
constexpr uint32_t DIGEST_NO_SCENE = 0xffffffffu;
__device__ __forceinline__ void digest_block_begin(uint32_t* sacc, uint32_t* sscene) {
  if (threadIdx.x < 8) sacc[threadIdx.x] = 0u;
  if (threadIdx.x == 0) *sscene = DIGEST_NO_SCENE;
  __syncthreads();
}
__device__ __forceinline__ void digest_add_block(uint32_t* acc, uint32_t* sacc, uint32_t* sscene, bool valid,
                                                 uint32_t scene, const uint32_t h[8]) {
  uint32_t key = valid ? scene : DIGEST_NO_SCENE;
  uint32_t peers = __match_any_sync(0xffffffffu, key);
  int lane = threadIdx.x & 31;
  bool leader = lane == __ffs(peers) - 1;
  uint32_t t[8];
  if (peers == 0xffffffffu) {
#pragma unroll
    for (int l = 0; l < 8; ++l) t[l] = __reduce_add_sync(0xffffffffu, h[l]);
  } else {
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      uint32_t v = h[l], total = 0, m = peers;
      while (m) {
        int src = __ffs(m) - 1;
        m &= m - 1;
        total += __shfl_sync(peers, v, src);
      }
      t[l] = total;
    }
  }
  if (!(leader && valid)) return;
  uint32_t owner = *(volatile uint32_t*)sscene;
  if (owner == DIGEST_NO_SCENE) {
    const uint32_t prev = atomicCAS(sscene, DIGEST_NO_SCENE, scene);
    owner = prev == DIGEST_NO_SCENE ? scene : prev;
  }
  if (owner == scene) {
#pragma unroll
    for (int l = 0; l < 8; ++l) atomicAdd(sacc + l, t[l]);
  } else {
#pragma unroll
    for (int l = 0; l < 8; ++l) atomicAdd(acc + scene * 8 + l, t[l]);
  }
}
__device__ __forceinline__ void digest_block_end(uint32_t* acc, uint32_t* sacc, uint32_t* sscene) {
  __syncthreads();
  const uint32_t owner = *sscene;
  if (threadIdx.x < 8 && owner != DIGEST_NO_SCENE) atomicAdd(acc + owner * 8 + threadIdx.x, sacc[threadIdx.x]);
}

}  // namespace d2
}  // namespace sn
