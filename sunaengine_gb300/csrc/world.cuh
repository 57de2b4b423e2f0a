// Device-side layout of a world: one or more independent 2D scenes advanced
// together, one substep per pass of the kernel sequence.
//
// Two index spaces:
//   * SLOT space: each scene owns a contiguous slot range [slotBase, slotBase+cap).
//     Slot i - slotBase is the reference's particle index (fluid first, then the
//     boundary block), so hashed state words, stAcc and bond rows live here.
//   * SORTED space: every active particle of every scene, ordered by grid key,
//     in one of two layouts chosen per world.
//     Colour-major (the default): all scenes' colour-0 cells, then colour-1,
//     ...; a scene's cells of one colour are in (cy/2, cx/2) row-major order.
//     One colour class is one contiguous sorted range.
//     Tile-major (the staged gathers): each scene's grid is cut into square
//     tiles of T x T cells (T = 2^tileShift), tiles in row-major order, and
//     inside a tile the four colour classes one after another, each colour's
//     cells in (ly/2, lx/2) row-major order. A tile's particles are one
//     contiguous sorted range, and so is each colour class inside it.
//     In both layouts the particles of a cell are in ascending slot order (the
//     reference's canonical order, src/sim.wgsl:1126-1168).
//
// In the tile-major layout a tile's neighbourhood (the tile plus a one-cell
// ring around it) is 9 + 2T contiguous runs of sorted space: the tile itself,
// the two colour runs of the halo row below and of the row above (a colour's
// cells in one tile row are consecutive keys), and the T + 2 single cells of
// the halo column on each side. The per-substep run table (TR) lists each
// run's first sorted position and its offset in the tile's staged copy; the
// staged kernels copy the runs into shared memory with bulk copies and read
// neighbours there through 16-bit tile-local indices.
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
constexpr uint16_t NBRL_BOUNDARY = 0x8000u;     // the same flag in a tile-local (16-bit) entry
constexpr uint16_t NBRL_INDEX = 0x7fffu;

// Tiles: side 2^tileShift cells, tileShift in [TILE_SHIFT_MIN, TILE_SHIFT_MAX].
constexpr uint32_t TILE_SHIFT_MIN = 2, TILE_SHIFT_MAX = 4;
constexpr uint32_t TR_RUNS_MAX = 9 + 2 * (1u << TILE_SHIFT_MAX);  // 41
constexpr uint32_t TR_STRIDE = 96;   // words per tile: [0, 48) run starts, [48, 96) run offsets (+ total)
constexpr uint32_t TR_BASE = 48;
// A tile whose neighbourhood holds more records than the staged kernels'
// shared-memory copy is gathered from global memory instead.
constexpr uint32_t STAGE_MAX = 2048;

// Per-scene parameters (the reference's Params uniform, src/sim.wgsl:225-300,
// plus this layout's key offsets).
struct ScenePar {
  uint32_t slotBase;
  uint32_t cap;        // slots owned
  uint32_t n, nFluid;
  uint32_t gridW, gridH, cellShift, cellTotal;
  int32_t domW, domH, vmax;
  uint32_t weldHold;   // the weld tag a gesture holds open (0: none)
  uint32_t keyOff[4];  // colour-major layout: global key of this scene's first colour-c cell
  uint32_t nA[4];      // colour-major layout: colour-c cells per grid row, (gridW + 1 - (c & 1)) / 2
  uint32_t tileShift;  // 0: colour-major layout; else tile-major, tile side = 2^tileShift cells
  uint32_t keyBase;    // tile-major layout: global key of this scene's first cell (its first tile)
  uint32_t tileBase;   // tile-major layout: global index of this scene's first tile
  uint32_t tilesX, tilesY;
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
  uint32_t K;              // total grid keys over all scenes = sentinel key
  uint32_t colourBase[5];  // colour-major layout: first key of each colour class; [4] = K
  uint32_t nTiles;         // tile-major layout: tiles over all scenes (0 in the colour-major layout)
  uint32_t stageCap;       // records a staged kernel copies per tile at most (its shared-memory copy)
  uint32_t slotEnd;        // 1 + last slot that can be active
  uint32_t nAct;           // active particles (sorted-space length)
  uint32_t hasFriction;    // some material has fric != 0 or bondK != 0
  uint32_t hasBonds;       // some material has bondK != 0
  uint32_t nBodies;        // §20 body records (all scenes)
};

// One tile of the world: its scene, its tile coordinates and its first key.
struct TileInfo {
  uint32_t scene, tx, ty, key0;
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
