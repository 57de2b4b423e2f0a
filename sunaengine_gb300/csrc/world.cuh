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

}  // namespace sn
