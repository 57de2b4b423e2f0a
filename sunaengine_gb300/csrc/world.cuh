// Device-side layout of a world: one or more independent 2D scenes advanced
// together, one substep per pass of the kernel sequence.
//
// Two index spaces:
//   * SLOT space: each scene owns a contiguous slot range [slotBase, slotBase+cap).
//     Slot i - slotBase is the reference's particle index (fluid first, then the
//     boundary block), so hashed state words, stAcc and bond rows live here.
//   * SORTED space: every active particle of every scene, ordered by grid key.
//     Keys are colour-major: all scenes' colour-0 cells, then colour-1, ...; a
//     scene's cells of one colour are in (cy/2, cx/2) row-major order; inside
//     a cell, particles are in ascending slot order (the reference's canonical
//     order, src/sim.wgsl:1126-1168). One colour class is therefore one
//     contiguous sorted range, and every solver gather reads neighbours from a
//     few nearby ranges.
#pragma once
#include <cstdint>

namespace sn {

constexpr int MAXNBR = 48;
constexpr int BOND_CAP = 48;
constexpr int MAT_WORDS = 48;
constexpr int MAT_MAX = 64;
constexpr int TN = 3202;
constexpr int LUT_WORDS = 5 * TN;
constexpr uint32_t NBR_BOUNDARY = 0x80000000u;  // set in a neighbour entry when it is a wall particle

// Per-scene parameters (the reference's Params uniform, src/sim.wgsl:225-300,
// plus this layout's key offsets).
struct ScenePar {
  uint32_t slotBase;
  uint32_t cap;        // slots owned
  uint32_t n, nFluid;
  uint32_t gridW, gridH, cellShift, cellTotal;
  int32_t domW, domH, vmax;
  uint32_t weldHold;   // the weld tag a gesture holds open (0: none)
  uint32_t keyOff[4];  // global key of this scene's first colour-c cell
  uint32_t nA[4];      // colour-c cells per grid row: (gridW + 1 - (c & 1)) / 2
  uint32_t formClock;  // formation clock (the engine's `_substep`), advanced on device
  uint32_t bondDirty;  // run formation on the next substep regardless of the clock
  uint32_t formNow;    // formation runs in the substep in flight (set by predict)
  uint32_t active;     // 0 = slot range reserved but not stepped
  uint32_t substep;    // substeps advanced since load (impulse schedule clock)
  uint32_t fuseTag;    // §18.24 armed draw-time fusion tag (0: none)
  uint32_t nJets;      // §23.B jets (setJets): 0..8
  int32_t jet[8][5];   // [x, y, r, fx, fy] ticks
  int32_t userA[2];    // §24 setUserDrive: the drive of user-flagged rigid bodies
};

// World-level totals, written by the host when the scene set changes.
struct WorldPar {
  uint32_t numScenes;
  uint32_t K;              // total grid cells over all scenes = sentinel key
  uint32_t colourBase[5];  // first global key of each colour class; [4] = K
  uint32_t slotEnd;        // 1 + last slot that can be active
  uint32_t nAct;           // active particles (sorted-space length)
  uint32_t hasFriction;    // some material has fric != 0 or bondK != 0
  uint32_t hasBonds;       // some material has bondK != 0
  uint32_t nBodies;        // §20 body records (all scenes)
};

#ifdef __CUDACC__
// cellStart[k] = first sorted position whose key is >= k, for k in [0, K],
// over the n sorted keys. Each CTA (256 threads) first loads 256 pivots,
// skey[j * n / 256], into shared memory; a key's answer lies between the last
// pivot below it and the first at or above it, so the search takes 8 steps in
// shared memory and about log2(n / 256) dependent global loads instead of
// log2(n). Every thread of the CTA must call it.
__device__ __forceinline__ void cell_starts(const uint32_t* __restrict__ skey, uint32_t n, uint32_t K,
                                            uint32_t* __restrict__ cellStart) {
  __shared__ uint32_t piv[256];
  for (uint32_t j = threadIdx.x; j < 256u; j += blockDim.x)
    piv[j] = n ? skey[(uint32_t)(((uint64_t)j * n) >> 8)] : 0xffffffffu;
  __syncthreads();
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= K; k += gridDim.x * blockDim.x) {
    uint32_t c = 0;  // pivots below k
#pragma unroll
    for (uint32_t step = 128; step; step >>= 1)
      if (piv[c + step - 1] < k) c += step;
    if (c == 255u && piv[255] < k) c = 256u;
    uint32_t lo = c ? (uint32_t)(((uint64_t)(c - 1) * n) >> 8) + 1u : 0u;
    uint32_t hi = c < 256u ? (uint32_t)(((uint64_t)c * n) >> 8) : n;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (skey[mid] < k) lo = mid + 1; else hi = mid;
    }
    cellStart[k] = lo;
  }
}
#endif

}  // namespace sn
