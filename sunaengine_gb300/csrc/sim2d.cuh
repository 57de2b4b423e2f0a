// The 2D substep as sm_103a kernels.
//
// One substep is this kernel sequence (reference pass order,
// src/engine.js:4003-4155, re-cut along true data dependences):
//
//   k_predict_key   predict (src/sim.wgsl:958-1000) + grid key per slot
//   radix sort      stable, atomic-free: replaces gridCount/scan/scatter/canonicalize
//   k_cellstart     cell ranges in sorted space (on a side branch, beside k_gather)
//   k_gather        slot -> sorted-space working set
//   k_cellbox       pred boxes of crowded cells (+ k_cellbox_chunks)
//   k_nbr           neighbour lists, reference traversal order and MAXNBR cut
//   ITERS x { k_solveA; k_colour x 4; [k_friction; k_apply_fric] }
//                   density/lambda, then colour-classed Gauss-Seidel position
//                   correction; solveB and applyDp are fused per colour over a
//                   double-buffered pred (see k_colour), each pass's copy of
//                   the other colours (k_colour_copy) on a side branch beside it
//   k_contain       containment of intruders (when a seal particle is live)
//   k_post1         finalize + xsph + normals + conduct in one neighbour sweep
//   k_post2         surfaceTension + thermal + formation flag clear + state hash
//   [k_form1, k_form2, k_hash]   bond formation for worlds with bonding rows
//   k_fold          per-scene chain fold, formation clock
//
// Sorted-space records are packed so one neighbour costs one or two wide loads:
//   PL[p] = {pred.x, pred.y, lam, info}   info = matId | state bits (INFO_*)
//   RX[p] = {rho, rinv, temp, 0}
//   NQ[p] = {nrm.x, nrm.y, rho, 0}        (written by k_post1 for k_post2)
// The kernel tables are interleaved per LUT index: WG = {W, G}, CA = {C, A}.
//
// Everything is int32 on the integer pipes; no floats, no atomics in the
// physics (the only atomics are the u32 adds of the digest and the debug
// counters, both commutative).
//
// Range facts used by the release build (debug builds keep every saturation
// test so the debug counters stay exact): fluid preds are wall-clamped into
// [0, 2^27] and wall particles lie in [-2^27, 2^27], so pred differences never
// overflow; an accepted neighbour has |d| <= 163848 < 2^18; |G| < 2^27, so a
// gradient term is < 2^19; |lambda| <= 2^22; |vel| <= 2^16; K_ij <= 2^18;
// |T| <= 2^29. Under these bounds every per-pair product below either fits in
// i32 after its shift (mulf) or is clamped at once into an i32 range (mulc).
#pragma once
#include <cstdint>
#include "fixed.cuh"
#include "stage.cuh"
#include "statehash.cuh"
#include "world.cuh"

namespace sn {
namespace d2 {

// ---- constants: src/sim.wgsl:55-175 -----------------------------------------
constexpr int32_t H = 163840;
constexpr int32_t RHO0 = 1048576;
constexpr int32_t TWO_RHO0 = 2097152;
constexpr int32_t HS = 10240;
constexpr int32_t H2S = 104857600;
constexpr int32_t LAM_MAX = 4194304;
constexpr int32_t S_TERM = 16777216;
constexpr int32_t DP_TERM = 2097152;
constexpr int32_t XS_TERM = 2097152;
constexpr int32_t ST_TERM = 4194304;
constexpr int32_t RINV_MAX = 262144;
constexpr int32_t WALL = 32768;
constexpr int32_t C_MAX = 58000;
constexpr int32_t RHO_FLOOR_RINV = 32768;
constexpr int32_t RHO_FLOOR_K = 65536;
constexpr int32_t AMBIENT = 1310720;
constexpr int32_t TEMP_MIN = -33554432, TEMP_MAX = 536870912;
constexpr int32_t DT_CLAMP = 16777216;
constexpr int32_t HT_TERM = 16777216;
constexpr int32_t CORR_TERM = 16777216;
constexpr int32_t CORR_NEVER = 2147483647;
constexpr uint32_t FLAG_BURNING = 1, FLAG_DEAD = 2, FLAG_ANCHOR = 4, FLAG_RIGID = 16;
constexpr uint32_t FLAG_CONGEAL = 32, FLAG_BURST = 64, FLAG_SEAL = 128;
constexpr uint32_t WELD_TAG_MASK = 0x000fff00u;
constexpr uint32_t NBRN_CONGEAL = 0x20000000u;
constexpr uint32_t NBRN_SEAL = 0x40000000u;      // a non-wall neighbour carries FLAG_SEAL (nbr_has_seal)
constexpr uint32_t NBRN_COUNT = 0x1fffffffu;
constexpr int FPRE = 5, RPRE = 3, BPRE = 5;
constexpr int32_t D2_FLOOR = 262144;
constexpr int32_t FR_TERM = 16777216;
constexpr int32_t BOND_R2 = 17623204;
constexpr int32_t HARD_BREAK2 = 26214400;
constexpr int32_t L0_MAX = 5120, L0_MIN = 512;
constexpr uint32_t BOND_J_MASK = 0x0001ffffu, BOND_L0_MASK = 0x3ffe0000u, BOND_TOMB = 0x40000000u;
constexpr int32_t BD_TERM = 16777216;
constexpr uint32_t MAT_PHOTO_ROW = 15;
// info word bits (sorted space)
constexpr uint32_t INFO_MAT = 0xffu;
constexpr uint32_t INFO_BOUNDARY = 0x80000000u;  // a wall particle (slot >= nFluid)
constexpr uint32_t INFO_DEAD = 0x40000000u;      // FLAG_DEAD
constexpr uint32_t INFO_CONGEAL = 0x20000000u;   // FLAG_CONGEAL
constexpr uint32_t INFO_PINNED = 0x10000000u;    // FLAG_ANCHOR | FLAG_RIGID: never moved by dp
constexpr uint32_t INFO_BURST = 0x08000000u;     // FLAG_BURST
constexpr uint32_t INFO_RIGID = 0x04000000u;     // FLAG_RIGID
constexpr uint32_t INFO_SEAL = 0x02000000u;      // FLAG_SEAL
constexpr uint32_t INFO_TAG = 0x000fff00u;       // a rigid member's weld tag (its body id); 0 otherwise

// material words (src/engine.js:678-705)
enum : int {
  M_eps = 0, M_dpMax = 1, M_xsph = 2, M_phantom = 3, M_gammaCoh = 4, M_gammaCur = 5, M_adhesion = 6,
  M_grav = 7, M_cond = 8, M_coolRate = 9, M_meltPt = 11, M_meltTo = 12, M_freezePt = 13, M_freezeTo = 14,
  M_boilPt = 15, M_boilTo = 16, M_condPt = 17, M_condTo = 18, M_ignitePt = 19, M_fuel0 = 20,
  M_burnRate = 21, M_burnHeat = 22, M_burnTo = 23, M_splitTo = 24, M_splitPct = 25, M_spawnTemp = 26,
  M_corrode = 28, M_corrPt = 29, M_corrTo = 30, M_fric = 31, M_bondK = 32, M_bondBreak = 33,
  M_bondReform = 34, M_bondFormV = 35, M_bondFormP = 36, M_bondMu = 37, M_bondGroup = 38, M_rampLo = 39,
  M_rampHi = 40, M_rampInv = 41, M_rampSign = 42, M_solidMode = 43, M_tempTarget = 44, M_tempDrive = 45,
  M_burstP = 46, M_sealMode = 47
};
constexpr int32_t SOLID_RIGID = 2;

// All device buffers of a world, passed by value.
struct Bufs {
  // slot space
  int32_t* state;       // [cap * 8] hashed particle words
  int2* stacc;          // [cap] surface-tension acceleration, consumed next substep
  int2* predSlot;       // [cap] predict output in slot order
  uint32_t* sceneOf;    // [cap]
  uint32_t* keys;       // [cap]
  uint32_t* inv;        // [cap] slot -> sorted position
  uint32_t* bond;       // [cap * 48]
  uint32_t* bondCand;   // [cap * 48]
  // sort
  uint32_t* skey;       // [cap]
  uint32_t* sslot;      // [cap]
  uint32_t* cellStart;  // [K + 1]
  // sorted space
  int4* PL;             // {pred.x, pred.y, lam, info}  (buffer A)
  int4* PL2;            // buffer B of the colour sweep (same layout)
  int4* RX;             // {rho, rinv, temp, 0}
  int4* NQ;             // {nrm.x, nrm.y, rho, 0}
  int2* POS;
  uint32_t* SCN;
  int2* DP;
  int32_t* HEAT;
  int32_t* CORR;
  uint32_t* NBR;        // [MAXNBR][nbrStride] sorted indices | NBR_BOUNDARY
  uint16_t* NBRL;       // [MAXNBR][nbrStride] the same neighbours as tile-local indices | NBRL_BOUNDARY
  uint32_t* NBRN;
  uint32_t nbrStride;
  const TileInfo* tiles;  // [nTiles]
  uint32_t* TR;           // [nTiles][TR_STRIDE] run table of each tile's neighbourhood
  // tables and per-scene data
  const int32_t* luts;  // 5*TN, reference layout
  const int2* WG;       // [TN] {W, G}
  const int2* CA;       // [TN] {C, A}
  const int32_t* mats;
  const uint16_t* rcp;  // [32768] floor(2^30 / dn), dn in [2^15, 2^16)
  ScenePar* scenes;
  WorldPar* world;
  uint32_t* acc;        // [S * 8]
  uint32_t* accLast;    // [S * 8]
  uint32_t* chain;      // [S * 8]
  uint32_t* dbg;        // [16]
  uint32_t* err;        // [4]
  uint32_t* work;       // [8] per-substep flags: [0] = some particle has a friction/bond row,
                        // [1] = some live fluid particle carries INFO_SEAL or INFO_CONGEAL,
                        // [2] = tiles too large to stage (entries of OVF),
                        // [3] = chunks of crowded cells for k_cellbox_chunks,
                        // [5] = some scene forms bonds this substep (formNow);
                        // and, never reset: [4] = some bond row of the world may be
                        // non-empty (set by bond formation and by every host write of
                        // bond rows)
  uint32_t* OVF;        // [nTiles] the tiles of this substep whose neighbourhood exceeds stageCap
  int4* CB;             // [K] pred bounding box of each cell above CELL_BIG particles (k_cellbox)
  // §20 rigid bodies
  int32_t* rbody;       // [bodies * 32] body records (the reference's RB_* words; word 29 = scene)
  int32_t* rdrv;        // [bodies * 10] driver sidecars (RD_* words)
  int2* rest;           // [cap] rest offsets, slot space
  const int32_t* cosT;  // [1026] Q22 quarter-turn cosine table
  uint32_t* rmark;      // [cap] rigidMember's leave marks, slot space
};

enum : uint32_t { ERR_UNSUPPORTED_ROW = 1u, ERR_BOND_PARTNER = 2u, ERR_STAGE_TIMEOUT = 4u, ERR_BARRIER = 8u };

__device__ __forceinline__ int32_t matw(const Bufs& b, uint32_t m, int w) { return __ldg(b.mats + m * MAT_WORDS + w); }

__device__ __forceinline__ uint32_t gstride() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ uint32_t gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }

// pred_i - pred_j. Both lie in [-2^27, 2^27], so the reference's fp_sub_sat
// cannot saturate; debug builds keep the test to count it anyway.
template <bool DBG>
__device__ __forceinline__ int2 pdelta(int2 a, int2 b, const Flags<DBG>& f) {
  if constexpr (DBG) return make_int2(sub_sat(a.x, b.x, f), sub_sat(a.y, b.y, f));
  else return make_int2(a.x - b.x, a.y - b.y);
}
template <bool DBG>
__device__ __forceinline__ int2 delta(int2 a, int2 b, const Flags<DBG>& f) {
  return make_int2(sub_sat(a.x, b.x, f), sub_sat(a.y, b.y, f));
}

// lut_index (src/sim.wgsl:520-527): symmetric rounding of |d| >> PRE, per-axis
// reject, r^2 < H2S, index r^2 >> KSH; -1 outside the kernel.
template <bool DBG>
__device__ __forceinline__ int lut_index(int2 d, const Flags<DBG>& f) {
  int32_t ax, ay;
  if constexpr (DBG) {
    ax = wadd(abs_sat(d.x, f), 8) >> 4;
    ay = wadd(abs_sat(d.y, f), 8) >> 4;
  } else {
    ax = (abs(d.x) + 8) >> 4;
    ay = (abs(d.y) + 8) >> 4;
  }
  if (max(ax, ay) > HS) return -1;
  int32_t r2 = wadd(wmul(ax, ax), wmul(ay, ay));
  if (r2 >= H2S) return -1;
  return r2 >> 15;
}
// lut_index(d) >= 0 without the index, branch-free (release builds): an axis
// above HS is clamped to HS + 1, whose square alone already exceeds H2S, so
// the sum rejects exactly when lut_index does (and cannot wrap).
__device__ __forceinline__ bool in_kernel(int2 d) {
  static_assert((int64_t)(HS + 1) * (HS + 1) >= H2S && 2 * (int64_t)(HS + 1) * (HS + 1) < INT32_MAX, "clamp");
  const int32_t ax = min((abs(d.x) + 8) >> 4, HS + 1), ay = min((abs(d.y) + 8) >> 4, HS + 1);
  return ax * ax + ay * ay < H2S;
}
__device__ __forceinline__ int2 wall_clamp(const ScenePar& S, int2 p) {
  return make_int2(clampi(p.x, WALL, S.domW - WALL), clampi(p.y, WALL, S.domH - WALL));
}
__device__ __forceinline__ int32_t mat_mix(int32_t a, int32_t b) { return wadd(a, b) >> 1; }
template <bool DBG>
__device__ __forceinline__ int32_t sym_k(int32_t ri, int32_t rj, const uint16_t* rcp, const Flags<DBG>& f) {
  int32_t den = max(RHO_FLOOR_K, add_sat(ri, rj, f));
  return clampi(divshift<16>(TWO_RHO0, den, rcp, f), 0, RINV_MAX);
}
// The grid key of cell (cx, cy) (both inside the scene's grid). Colour-major
// layout (tileShift 0): the scene's colour-c cells in (cy/2, cx/2) row-major
// order from keyOff[c]. Tile-major layout: tile, then colour, then the
// colour's cells row-major inside the tile.
__device__ __forceinline__ uint32_t key_of(const ScenePar& S, int32_t cx, int32_t cy) {
  if (S.tileShift == 0u) {
    const uint32_t c = (uint32_t)(cx & 1) | ((uint32_t)(cy & 1) << 1);
    return S.keyOff[c] + (uint32_t)(cy >> 1) * S.nA[c] + (uint32_t)(cx >> 1);
  }
  const uint32_t ts = S.tileShift, T = 1u << ts;
  const uint32_t tx = (uint32_t)cx >> ts, ty = (uint32_t)cy >> ts;
  const uint32_t lx = (uint32_t)cx & (T - 1u), ly = (uint32_t)cy & (T - 1u);
  const uint32_t c = (lx & 1u) | ((ly & 1u) << 1);
  return S.keyBase + ((ty * S.tilesX + tx) << (2u * ts)) + (c << (2u * ts - 2u)) + (ly >> 1) * (T >> 1) +
         (lx >> 1);
}
// Index of the tile (world-wide) holding cell (cx, cy).
__device__ __forceinline__ uint32_t tile_of(const ScenePar& S, int32_t cx, int32_t cy) {
  return S.tileBase + ((uint32_t)cy >> S.tileShift) * S.tilesX + ((uint32_t)cx >> S.tileShift);
}
__device__ __forceinline__ uint32_t tile_runs(uint32_t tileShift) { return 9u + (2u << tileShift); }
// Which run of tile (tx, ty)'s neighbourhood holds cell (gx, gy), a cell of
// the tile or of the one-cell ring around it: 0 = the tile, 1-2 = the halo row
// below (by x parity), 3-4 = the row above, then the left column's T + 2
// cells bottom to top, then the right column's.
__device__ __forceinline__ uint32_t halo_run(uint32_t tileShift, uint32_t tx, uint32_t ty, int32_t gx, int32_t gy) {
  const int32_t T = 1 << tileShift;
  const int32_t lx = gx - (int32_t)(tx << tileShift), ly = gy - (int32_t)(ty << tileShift);
  const bool inx = lx >= 0 && lx < T, iny = ly >= 0 && ly < T;
  if (inx && iny) return 0u;
  if (inx) return (ly < 0 ? 1u : 3u) + (uint32_t)(gx & 1);
  return 5u + (lx < 0 ? 0u : (uint32_t)T + 2u) + (uint32_t)(ly + 1);
}
__device__ __forceinline__ int2 cell_coord(const ScenePar& S, int2 p) {
  int32_t cx = p.x >> S.cellShift;
  int32_t cy = p.y >> S.cellShift;
  return make_int2(clampi(cx, 0, (int32_t)S.gridW - 1), clampi(cy, 0, (int32_t)S.gridH - 1));
}
// A neighbouring cell column (row) whose nearest edge is at least REJECT_D
// ticks from the particle holds no particle the kernel can accept: lut_index
// rejects |d| >= REJECT_D on either axis. Every particle assigned to column
// c >= 1 has x >= c * cell (clamping only moves x < 0 into column 0), and every
// particle of column c <= gridW - 2 has x < (c + 1) * cell, so the test below
// is exact and skipping such a column changes neither the list nor its order.
constexpr int32_t REJECT_D = (HS + 1) * 16 - 8;  // smallest |d| with (|d| + 8) >> 4 > HS
constexpr uint32_t SKIP_LEFT = 1u, SKIP_RIGHT = 2u, SKIP_DOWN = 4u, SKIP_UP = 8u;
__device__ __forceinline__ uint32_t far_sides(const ScenePar& S, int2 p, int2 cc) {
  const int64_t x0 = (int64_t)cc.x << S.cellShift, y0 = (int64_t)cc.y << S.cellShift;
  const int64_t cs = (int64_t)1 << S.cellShift;
  uint32_t m = 0;
  if ((int64_t)p.x - x0 >= REJECT_D) m |= SKIP_LEFT;
  if (x0 + cs - (int64_t)p.x >= REJECT_D) m |= SKIP_RIGHT;
  if ((int64_t)p.y - y0 >= REJECT_D) m |= SKIP_DOWN;
  if (y0 + cs - (int64_t)p.y >= REJECT_D) m |= SKIP_UP;
  return m;
}
__device__ __forceinline__ bool seal_class(const Bufs& b, uint32_t m) {
  return matw(b, m, M_bondK) != 0 && matw(b, m, M_bondReform) == 0 && matw(b, m, M_solidMode) != 0 &&
         matw(b, m, M_phantom) == 0;
}
__device__ __forceinline__ bool fuse_row(const Bufs& b, uint32_t m) {
  return matw(b, m, M_bondK) != 0 && matw(b, m, M_bondReform) == 0 && matw(b, m, M_bondGroup) >= 0 &&
         m != MAT_PHOTO_ROW;
}
__device__ __forceinline__ uint32_t id_hash(uint32_t i) {
  uint32_t x = i + 0x9e3779b9u;
  x = (x ^ (x >> 16)) * 0x21f0aaadu;
  x = (x ^ (x >> 15)) * 0x735a2d97u;
  return x ^ (x >> 15);
}
__device__ __forceinline__ uint32_t pick_product(uint32_t primary, uint32_t splitTo, uint32_t pct, uint32_t i) {
  if (pct == 0u) return primary;
  return (id_hash(i) & 255u) < pct ? splitTo : primary;
}
template <bool DBG>
__device__ __forceinline__ int32_t bond_k(const Bufs& b, uint32_t m, int32_t T, const Flags<DBG>& f) {
  int32_t k = matw(b, m, M_bondK);
  if (k == 0) return 0;
  int32_t sgn = matw(b, m, M_rampSign);
  if (sgn == 0) return k;
  int32_t lo = matw(b, m, M_rampLo);
  int32_t span = sub_sat(matw(b, m, M_rampHi), lo, f);
  int32_t dT = clampi(sub_sat(T, lo, f), 0, span);
  int32_t u = clampi(mul<16>(dT, matw(b, m, M_rampInv), f), 0, 65536);
  if (sgn < 0) u = 65536 - u;
  return mul<16>(k, u, f);
}
__device__ __forceinline__ uint32_t info_of(uint32_t matId, uint32_t flags, bool boundary) {
  return (matId & INFO_MAT) | (boundary ? INFO_BOUNDARY : 0u) | ((flags & FLAG_DEAD) ? INFO_DEAD : 0u) |
         ((flags & FLAG_CONGEAL) ? INFO_CONGEAL : 0u) | ((flags & (FLAG_ANCHOR | FLAG_RIGID)) ? INFO_PINNED : 0u) |
         ((flags & FLAG_BURST) ? INFO_BURST : 0u) | ((flags & FLAG_RIGID) ? INFO_RIGID : 0u) |
         ((flags & FLAG_SEAL) ? INFO_SEAL : 0u) | ((flags & FLAG_RIGID) ? (flags & INFO_TAG) : 0u);
}
// rg_same_body (src/sim.wgsl:891-894) on two info words: both rigid members
// wearing the same nonzero body tag.
__device__ __forceinline__ bool same_body(uint32_t infoI, uint32_t infoJ) {
  return (infoI & infoJ & INFO_RIGID) != 0u && ((infoI ^ infoJ) & INFO_TAG) == 0u && (infoI & INFO_TAG) != 0u;
}
__device__ __forceinline__ int2 xy(int4 v) { return make_int2(v.x, v.y); }
__device__ __forceinline__ int2 ld_pred(const int4* PL, uint32_t q) {
  return *reinterpret_cast<const int2*>(PL + q);
}

// Sum over the L lanes that share one particle (L a power of two, groups are
// aligned within the warp). Wrapping u32 addition, so the split is exact.
template <int L>
__device__ __forceinline__ int32_t gsum(int32_t v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v = wadd(v, __shfl_xor_sync(0xffffffffu, v, o, L));
  return v;
}

// ---- kernels --------------------------------------------------------------------

// jet_accel (src/sim.wgsl:935-949): the saturating sum of the accelerations
// of the scene's jets whose disc holds p; (0, 0) with no jets.
template <bool DBG>
__device__ __forceinline__ int2 jet_accel(const ScenePar& S, int2 p, const Flags<DBG>& f) {
  int2 a = make_int2(0, 0);
  for (uint32_t k = 0; k < S.nJets; ++k) {
    const int32_t dx = sub_sat(p.x, S.jet[k][0], f) >> 9, dy = sub_sat(p.y, S.jet[k][1], f) >> 9;
    const int32_t rr = S.jet[k][2] >> 9;
    if (wadd(wmul(dx, dx), wmul(dy, dy)) <= wmul(rr, rr)) {
      a.x = add_sat(a.x, S.jet[k][3], f);
      a.y = add_sat(a.y, S.jet[k][4], f);
    }
  }
  return a;
}

// predict (src/sim.wgsl:958-1000) + the grid key of every slot.
template <bool DBG>
__global__ void __launch_bounds__(256) k_predict_key(Bufs b) {
  Flags<DBG> f{b.dbg};
  const uint32_t K = b.world->K, slotEnd = b.world->slotEnd;
  if (gtid() == 0) {  // per-substep flags, set again by k_gather, k_tiles and k_cellbox
    b.work[0] = 0u;
    b.work[1] = 0u;
    b.work[2] = 0u;
    b.work[3] = 0u;
    b.work[5] = 0u;
  }
  for (uint32_t slot = gtid(); slot < slotEnd; slot += gstride()) {
    uint32_t s = b.sceneOf[slot];
    const ScenePar& S = b.scenes[s];
    uint32_t i = slot - S.slotBase;
    if (!S.active || i >= S.n) { b.keys[slot] = K; continue; }
    if (i == 0) b.scenes[s].formNow = ((S.formClock & 3u) == 0u || S.bondDirty) ? 1u : 0u;
    const int4* w4 = reinterpret_cast<const int4*>(b.state + (size_t)slot * 8);
    int4 a = w4[0], c = w4[1];
    int2 pos = make_int2(a.x, a.y);
    int2 pred = pos;
    if (i < S.nFluid) {
      uint32_t m = (uint32_t)c.x, fl = (uint32_t)c.y;
      if (matw(b, m, M_phantom) == 0 && !(fl & (FLAG_ANCHOR | FLAG_RIGID))) {
        int2 st = b.stacc[slot];
        int32_t vmax = S.vmax, vmaxN = neg_sat(vmax, f);
        const int2 jf = jet_accel(S, pos, f);
        int32_t vx = add_sat(add_sat(a.z, st.x, f), jf.x, f);
        int32_t vy = add_sat(add_sat(add_sat(a.w, st.y, f), matw(b, m, M_grav), f), jf.y, f);
        vx = clampi(vx, vmaxN, vmax);
        vy = clampi(vy, vmaxN, vmax);
        pred = wall_clamp(S, make_int2(add_sat(pos.x, vx, f), add_sat(pos.y, vy, f)));
      }
    }
    b.predSlot[slot] = pred;
    int2 cc = cell_coord(S, pred);
    b.keys[slot] = key_of(S, cc.x, cc.y);
  }
}

// cellStart[k] = first sorted position whose key is >= k, for k in [0, K].
__global__ void __launch_bounds__(256) k_cellstart(Bufs b) {
  cell_starts(b.skey, b.world->slotEnd, b.world->K, b.cellStart);
}

// Move the working set into sorted space.
__global__ void __launch_bounds__(256) k_gather(Bufs b) {
  const uint32_t nAct = b.world->nAct;
  for (uint32_t p = gtid(); p < nAct; p += gstride()) {
    uint32_t slot = b.sslot[p];
    uint32_t s = b.sceneOf[slot];
    const ScenePar& S = b.scenes[s];
    uint32_t i = slot - S.slotBase;
    const int4* w4 = reinterpret_cast<const int4*>(b.state + (size_t)slot * 8);
    int4 a = w4[0], c = w4[1];
    int2 pr = b.predSlot[slot];
    int4 rec = make_int4(pr.x, pr.y, 0, (int32_t)info_of((uint32_t)c.x, (uint32_t)c.y, i >= S.nFluid));
    b.PL[p] = rec;
    b.PL2[p] = rec;
    b.RX[p] = make_int4(0, 0, c.z, 0);
    b.POS[p] = make_int2(a.x, a.y);
    b.SCN[p] = s;
    b.inv[slot] = p;
    const uint32_t m = (uint32_t)rec.w & INFO_MAT;
    // the particles k_friction or k_apply_fric would touch (a superset of each)
    const bool fr = !((uint32_t)rec.w & INFO_BOUNDARY) && (matw(b, m, M_fric) != 0 || matw(b, m, M_bondK) != 0);
    const unsigned bal = __ballot_sync(__activemask(), fr);
    if (fr && (threadIdx.x & 31u) == (unsigned)(__ffs(bal) - 1) && *(volatile uint32_t*)b.work == 0u)
      atomicOr(b.work, 1u);
    // a live fluid particle a neighbour-list flag can see (buildNbr's sealSeen / congealSeen)
    const bool fl = !((uint32_t)rec.w & (INFO_BOUNDARY | INFO_DEAD)) && ((uint32_t)rec.w & (INFO_SEAL | INFO_CONGEAL));
    const unsigned bfl = __ballot_sync(__activemask(), fl);
    if (fl && (threadIdx.x & 31u) == (unsigned)(__ffs(bfl) - 1) && *(volatile uint32_t*)(b.work + 1) == 0u)
      atomicOr(b.work + 1, 1u);
    // its scene forms bonds this substep (k_predict_key set formNow): k_form1 has work
    const bool fm = S.formNow != 0u;
    const unsigned bfm = __ballot_sync(__activemask(), fm);
    if (fm && (threadIdx.x & 31u) == (unsigned)(__ffs(bfm) - 1) && *(volatile uint32_t*)(b.work + 5) == 0u)
      atomicOr(b.work + 5, 1u);
  }
}

// Cells holding more than CELL_BIG particles get a bounding box of their
// preds each substep (k_cellbox / k_cellbox_chunks); the list build skips such
// a cell when even the box's nearest point fails lut_index's test, since every
// candidate in it would then be rejected. Wall clamping can pile 10^5
// particles into one edge cell, and a particle beside the pile would otherwise
// test every one of them.
constexpr uint32_t CELL_BIG = 64;
constexpr uint32_t CELL_CHUNK = 4096;  // a larger cell is reduced in chunks of this many, one CTA each
// lut_index's rejection is monotone in |d.x| and |d.y|: if the box's nearest
// point (per axis) is rejected, so is every candidate in the box.
__device__ __forceinline__ bool box_reaches(int4 box, int2 pi) {
  const int64_t gx = max(max((int64_t)box.x - pi.x, (int64_t)pi.x - box.z), (int64_t)0);
  const int64_t gy = max(max((int64_t)box.y - pi.y, (int64_t)pi.y - box.w), (int64_t)0);
  if (gx >= REJECT_D || gy >= REJECT_D) return false;
  const int32_t ax = ((int32_t)gx + 8) >> 4, ay = ((int32_t)gy + 8) >> 4;
  return ax * ax + ay * ay < H2S;
}
struct BoxChunk {
  uint32_t key, lo, hi, pad;
};
// One warp per cell (grid-stride over the keys): the pred box of every cell
// above CELL_BIG particles, reduced by the warp itself up to CELL_CHUNK
// particles; a larger cell gets an empty box here and one chunk entry per
// CELL_CHUNK particles in `chunks` (count in work[3]) for k_cellbox_chunks.
__global__ void __launch_bounds__(256) k_cellbox(Bufs b, BoxChunk* __restrict__ chunks) {
  const uint32_t K = b.world->K, lane = threadIdx.x & 31u, warps = gstride() >> 5;
  for (uint32_t k = gtid() >> 5; k < K; k += warps) {
    const uint32_t lo = b.cellStart[k], hi = b.cellStart[k + 1];
    if (hi - lo <= CELL_BIG) continue;
    if (hi - lo > CELL_CHUNK) {
      const uint32_t n = (hi - lo + CELL_CHUNK - 1) / CELL_CHUNK;
      uint32_t base = 0;
      if (lane == 0) {
        b.CB[k] = make_int4(INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN);
        base = atomicAdd(b.work + 3, n);
      }
      base = __shfl_sync(0xffffffffu, base, 0);
      for (uint32_t c = lane; c < n; c += 32)
        chunks[base + c] = BoxChunk{k, lo + c * CELL_CHUNK, min(hi, lo + (c + 1) * CELL_CHUNK), 0u};
      continue;
    }
    int32_t x0 = INT32_MAX, y0 = INT32_MAX, x1 = INT32_MIN, y1 = INT32_MIN;
    for (uint32_t q = lo + lane; q < hi; q += 32) {
      const int2 pq = ld_pred(b.PL, q);
      x0 = min(x0, pq.x);
      y0 = min(y0, pq.y);
      x1 = max(x1, pq.x);
      y1 = max(y1, pq.y);
    }
    x0 = __reduce_min_sync(0xffffffffu, x0);
    y0 = __reduce_min_sync(0xffffffffu, y0);
    x1 = __reduce_max_sync(0xffffffffu, x1);
    y1 = __reduce_max_sync(0xffffffffu, y1);
    if (lane == 0) b.CB[k] = make_int4(x0, y0, x1, y1);
  }
}
// One CTA per chunk of a crowded cell: the chunk's box, merged into the
// cell's with four atomics (min/max are order-free).
__global__ void __launch_bounds__(256) k_cellbox_chunks(Bufs b, const BoxChunk* __restrict__ chunks) {
  __shared__ int32_t red[4][8];
  const uint32_t n = b.work[3], lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t c = blockIdx.x; c < n; c += gridDim.x) {
    const BoxChunk ch = chunks[c];
    int32_t x0 = INT32_MAX, y0 = INT32_MAX, x1 = INT32_MIN, y1 = INT32_MIN;
    for (uint32_t q = ch.lo + threadIdx.x; q < ch.hi; q += blockDim.x) {
      const int2 pq = ld_pred(b.PL, q);
      x0 = min(x0, pq.x);
      y0 = min(y0, pq.y);
      x1 = max(x1, pq.x);
      y1 = max(y1, pq.y);
    }
    x0 = __reduce_min_sync(0xffffffffu, x0);
    y0 = __reduce_min_sync(0xffffffffu, y0);
    x1 = __reduce_max_sync(0xffffffffu, x1);
    y1 = __reduce_max_sync(0xffffffffu, y1);
    if (lane == 0) {
      red[0][warp] = x0;
      red[1][warp] = y0;
      red[2][warp] = x1;
      red[3][warp] = y1;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
      int32_t v = red[threadIdx.x][0];
      for (int w = 1; w < 8; ++w) v = threadIdx.x < 2 ? min(v, red[threadIdx.x][w]) : max(v, red[threadIdx.x][w]);
      int32_t* box = reinterpret_cast<int32_t*>(b.CB + ch.key);
      if (threadIdx.x < 2) atomicMin(box + threadIdx.x, v);
      else atomicMax(box + threadIdx.x, v);
    }
    __syncthreads();
  }
}

// The run table of every tile's neighbourhood for this substep (one warp per
// tile): run r's first sorted position in TR[t][r], its offset in the tile's
// staged copy in TR[t][TR_BASE + r], and the copy's length in
// TR[t][TR_BASE + runs]. Runs outside the scene's grid are empty.
__global__ void __launch_bounds__(256) k_tiles(Bufs b) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nT = b.world->nTiles;
  const uint32_t warps = gstride() >> 5;
  for (uint32_t t = gtid() >> 5; t < nT; t += warps) {
    const TileInfo ti = b.tiles[t];
    const ScenePar& S = b.scenes[ti.scene];
    const uint32_t ts = S.tileShift, T = 1u << ts, H = T >> 1, runs = tile_runs(ts);
    uint32_t* tr = b.TR + (size_t)t * TR_STRIDE;
    uint32_t carry = 0, own = 0;
    for (uint32_t r0 = 0; r0 < runs; r0 += 32) {
      const uint32_t r = r0 + lane;
      uint32_t start = 0, len = 0;
      if (r < runs && S.active) {
        uint32_t k0 = 0, kn = 0;
        bool any = false;
        if (r == 0) {
          k0 = ti.key0;
          kn = T * T;
          any = true;
        } else if (r <= 4) {
          // a colour's cells in one halo row: H consecutive keys of the tile above or below
          const int32_t gy = (int32_t)(ti.ty * T) + (r <= 2 ? -1 : (int32_t)T);
          const uint32_t xpar = (r - 1u) & 1u;
          if (gy >= 0 && gy < (int32_t)S.gridH) {
            const uint32_t ty2 = (uint32_t)gy >> ts, ly = (uint32_t)gy & (T - 1u);
            const uint32_t c = xpar | ((ly & 1u) << 1);
            k0 = S.keyBase + ((ty2 * S.tilesX + ti.tx) << (2u * ts)) + (c << (2u * ts - 2u)) + (ly >> 1) * H;
            kn = H;
            any = true;
          }
        } else {
          const uint32_t j = r - 5u;
          const bool right = j >= T + 2u;
          const int32_t gx = (int32_t)(ti.tx * T) + (right ? (int32_t)T : -1);
          const int32_t gy = (int32_t)(ti.ty * T) - 1 + (int32_t)(right ? j - (T + 2u) : j);
          if (gx >= 0 && gx < (int32_t)S.gridW && gy >= 0 && gy < (int32_t)S.gridH) {
            k0 = key_of(S, gx, gy);
            kn = 1;
            any = true;
          }
        }
        if (any) {
          start = b.cellStart[k0];
          len = b.cellStart[k0 + kn] - start;
        }
      }
      // exclusive prefix of the lengths in run order
      uint32_t inc = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += v;
      }
      if (r < runs) {
        tr[r] = start;
        tr[TR_BASE + r] = carry + inc - len;
      }
      if (r0 == 0) own = __shfl_sync(0xffffffffu, len, 0);
      carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) {
      tr[TR_BASE + runs] = carry;
      // a tile with particles whose neighbourhood cannot be staged is gathered
      // from global memory by every CTA (list order does not matter: each
      // particle's result depends only on its inputs)
      if (own && carry > b.world->stageCap) b.OVF[atomicAdd(b.work + 2, 1u)] = t;
    }
  }
}

// buildNbr (src/sim.wgsl:1190-1254): 3x3 cells, dy outer, dx inner, ascending
// slot inside a cell; skip self and retired particles; keep pairs inside the
// kernel range; keep the first MAXNBR in that order (dbg[6] counts the rest).
// Wall particles only need their truncation count, so their lists are only
// walked in debug mode.
//
// L lanes share one particle: they test L consecutive candidates of a cell at
// once and place the hits with a ballot prefix, so the list keeps exactly the
// sequential order (and the same MAXNBR cut) whatever L is.
template <bool DBG, int L, bool TILED>
__global__ void __launch_bounds__(256, TILED ? 6 : 8) k_nbr(Bufs b) {
  // Once a list is full, a later candidate can only raise a flag bit or the
  // overflow counter. With no live SEAL/CONGEAL fluid particle in the world
  // and no counters kept, nothing it could change remains, so the scan stops:
  // the list, its count and its flags are the full scan's. (A cell crowded by
  // wall clamping can hold 10^5 particles, where the full scan is quadratic.)
  const bool cut = !DBG && b.work[1] == 0u;
  if constexpr (L == 1) {
    Flags<DBG> f{b.dbg};
    const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
    for (uint32_t p = gtid(); p < nAct; p += gstride()) {
      int4 me = b.PL[p];
      uint32_t info = (uint32_t)me.w;
      bool bnd = (info & INFO_BOUNDARY) != 0;
      if ((bnd && !DBG) || (info & INFO_DEAD)) { b.NBRN[p] = 0; continue; }
      const ScenePar& S = b.scenes[b.SCN[p]];
      int2 pi = xy(me);
      int2 cc = cell_coord(S, pi);
      const uint32_t skip = far_sides(S, pi, cc);
      uint32_t cnt = 0;
      bool congeal = false, sealSeen = false;
      uint32_t* out = b.NBR + p;
      // the tile-local list: offsets into this particle's tile's staged neighbourhood
      const uint32_t ts = S.tileShift, tx = (uint32_t)cc.x >> ts, ty = (uint32_t)cc.y >> ts;
      const uint32_t* tr = TILED ? b.TR + (size_t)tile_of(S, cc.x, cc.y) * TR_STRIDE : b.TR;
      const bool local = TILED && !bnd && tr[TR_BASE + tile_runs(ts)] <= b.world->stageCap;
      uint16_t* outl = b.NBRL + p;
      for (int dy = -1; dy <= 1; ++dy) {
        int32_t gy = cc.y + dy;
        if (gy < 0 || gy >= (int32_t)S.gridH) continue;
        if ((dy < 0 && (skip & SKIP_DOWN)) || (dy > 0 && (skip & SKIP_UP))) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          int32_t gx = cc.x + dx;
          if (gx < 0 || gx >= (int32_t)S.gridW) continue;
          if ((dx < 0 && (skip & SKIP_LEFT)) || (dx > 0 && (skip & SKIP_RIGHT))) continue;
          uint32_t key = key_of(S, gx, gy);
          uint32_t lo = b.cellStart[key], hi = b.cellStart[key + 1];
          if (!DBG && hi - lo > CELL_BIG && !box_reaches(b.CB[key], pi)) continue;
          if (!TILED && cut) {
            // The stopping scan: no live fluid particle carries SEAL or
            // CONGEAL (so neither flag can be raised) and the list ends at
            // MAXNBR (so nothing overflows); the next record is loaded one
            // candidate ahead.
            int4 nx = lo < hi ? b.PL[lo] : make_int4(0, 0, 0, 0);
            for (uint32_t q = lo; q < hi; ++q) {
              const int4 o = nx;
              if (q + 1 < hi) nx = b.PL[q + 1];
              const uint32_t iq = (uint32_t)o.w;
              if (q == p || (iq & INFO_DEAD) || !in_kernel(pdelta(pi, xy(o), f))) continue;
              out[(size_t)cnt * stride] = q | (iq & INFO_BOUNDARY);
              if (++cnt >= (uint32_t)MAXNBR) goto listed;
            }
            continue;
          }
          const uint32_t delta = local ? tr[TR_BASE + halo_run(ts, tx, ty, gx, gy)] - tr[halo_run(ts, tx, ty, gx, gy)] : 0u;
          for (uint32_t q = lo; q < hi; ++q) {
            if (q == p) continue;
            const int4 o = b.PL[q];
            uint32_t iq = (uint32_t)o.w;
            if (iq & INFO_DEAD) continue;
            if (lut_index(pdelta(pi, xy(o), f), f) < 0) continue;
            if (!(iq & INFO_BOUNDARY) && (iq & INFO_CONGEAL)) congeal = true;
            if (!(iq & INFO_BOUNDARY) && (iq & INFO_SEAL)) sealSeen = true;
            if (cnt >= (uint32_t)MAXNBR) { f.flag(6); continue; }
            if (!bnd) out[(size_t)cnt * stride] = q | (iq & INFO_BOUNDARY);
            if (TILED && local)
              outl[(size_t)cnt * stride] = (uint16_t)((q + delta) | ((iq & INFO_BOUNDARY) ? NBRL_BOUNDARY : 0u));
            cnt++;
            if (cut && cnt >= (uint32_t)MAXNBR) goto listed;
          }
        }
      }
    listed:
      b.NBRN[p] = bnd ? 0u : (cnt | (congeal ? NBRN_CONGEAL : 0u) | (sealSeen ? NBRN_SEAL : 0u));
    }
    return;
  }
  Flags<DBG> f{b.dbg};
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  const uint32_t lane = threadIdx.x & 31u, sub = lane & (L - 1);
  const uint32_t gmask = (L == 32 ? 0xffffffffu : ((1u << L) - 1u)) << (lane & ~(uint32_t)(L - 1));
  const uint32_t below = (1u << lane) - 1u;
  const uint32_t G = gstride() / L;
  for (uint32_t p = gtid() / L;; p += G) {
    if (__shfl_sync(0xffffffffu, p, 0) >= nAct) break;  // warp-uniform exit
    const bool valid = p < nAct;
    const int4 me = valid ? b.PL[p] : make_int4(0, 0, 0, (int32_t)INFO_DEAD);
    const uint32_t info = (uint32_t)me.w;
    const bool bnd = (info & INFO_BOUNDARY) != 0;
    const bool work = valid && !((bnd && !DBG) || (info & INFO_DEAD));
    const ScenePar& S = b.scenes[work ? b.SCN[p] : 0u];
    const int2 pi = xy(me);
    const int2 cc = work ? cell_coord(S, pi) : make_int2(0, 0);
    const uint32_t skip = work ? far_sides(S, pi, cc) : 0u;
    uint32_t cnt = 0;
    bool congeal = false, sealSeen = false;
    uint32_t* out = b.NBR + p;
    const uint32_t ts = S.tileShift, tx = (uint32_t)cc.x >> ts, ty = (uint32_t)cc.y >> ts;
    const uint32_t* tr = (TILED && work) ? b.TR + (size_t)tile_of(S, cc.x, cc.y) * TR_STRIDE : b.TR;
    const bool local = TILED && work && !bnd && tr[TR_BASE + tile_runs(ts)] <= b.world->stageCap;
    for (int dy = -1; dy <= 1; ++dy) {
      for (int dx = -1; dx <= 1; ++dx) {
        const int32_t gy = cc.y + dy, gx = cc.x + dx;
        uint32_t lo = 0, len = 0, delta = 0;
        const bool far = (dy < 0 && (skip & SKIP_DOWN)) || (dy > 0 && (skip & SKIP_UP)) ||
                         (dx < 0 && (skip & SKIP_LEFT)) || (dx > 0 && (skip & SKIP_RIGHT));
        const bool full = cut && cnt >= (uint32_t)MAXNBR;  // uniform over the particle's lanes
        if (work && !far && !full && gy >= 0 && gy < (int32_t)S.gridH && gx >= 0 && gx < (int32_t)S.gridW) {
          const uint32_t key = key_of(S, gx, gy);
          lo = b.cellStart[key];
          len = b.cellStart[key + 1] - lo;
          if (!DBG && len > CELL_BIG && !box_reaches(b.CB[key], pi)) len = 0;
          if (TILED && local) {
            const uint32_t run = halo_run(ts, tx, ty, gx, gy);
            delta = tr[TR_BASE + run] - tr[run];
          }
        }
        for (uint32_t t = sub;; t += L) {
          // the warp walks on while any of its particles has candidates left
          // in this cell and room (or a reason) to keep them
          const bool more = t < len && !(cut && cnt >= (uint32_t)MAXNBR);
          if (!__any_sync(0xffffffffu, more)) break;
          const uint32_t q = lo + t;
          bool hit = false;
          uint32_t iq = 0;
          if (more && q != p) {
            const int4 o = b.PL[q];
            iq = (uint32_t)o.w;
            hit = !(iq & INFO_DEAD) && lut_index(pdelta(pi, xy(o), f), f) >= 0;
          }
          uint32_t pos = cnt, nhit = hit ? 1u : 0u;
          if (L > 1) {
            const uint32_t bal = __ballot_sync(0xffffffffu, hit) & gmask;
            pos = cnt + __popc(bal & below);
            nhit = __popc(bal);
          }
          if (hit) {
            if (!(iq & INFO_BOUNDARY) && (iq & INFO_CONGEAL)) congeal = true;
            if (!(iq & INFO_BOUNDARY) && (iq & INFO_SEAL)) sealSeen = true;
            if (pos >= (uint32_t)MAXNBR) f.flag(6);
            else if (!bnd) {
              out[(size_t)pos * stride] = q | (iq & INFO_BOUNDARY);
              if (TILED && local)
                b.NBRL[(size_t)pos * stride + p] =
                    (uint16_t)((q + delta) | ((iq & INFO_BOUNDARY) ? NBRL_BOUNDARY : 0u));
            }
          }
          cnt += nhit;
        }
      }
    }
    if (L > 1) {
      congeal = (__ballot_sync(0xffffffffu, congeal) & gmask) != 0u;
      sealSeen = (__ballot_sync(0xffffffffu, sealSeen) & gmask) != 0u;
    }
    if (valid && sub == 0)
      b.NBRN[p] = (bnd || !work) ? 0u
                                 : (min(cnt, (uint32_t)MAXNBR) | (congeal ? NBRN_CONGEAL : 0u) |
                                    (sealSeen ? NBRN_SEAL : 0u));
  }
}

// ---- tile-staged gathers ------------------------------------------------------
//
// solveA and the colour passes run one CTA per tile (grid-stride over the
// world's tiles). The CTA copies its tile's neighbourhood runs from PL into
// shared memory with bulk copies (stage_tile) and reads every neighbour record
// there through the tile-local list NBRL. A tile whose neighbourhood exceeds
// the staging capacity reads neighbours from global memory through the
// sorted-index list NBR instead; both give the same sums.

// Neighbour access for the staged path: records in shared memory, entries of
// the tile-local list.
struct NbrStaged {
  const int4* sm;
  const uint16_t* nl;
  uint32_t stride;
  __device__ __forceinline__ uint32_t entry(uint32_t p, uint32_t k) const { return nl[(size_t)k * stride + p]; }
  __device__ __forceinline__ int4 rec(uint32_t e) const { return sm[e & NBRL_INDEX]; }
  __device__ __forceinline__ int2 pred(uint32_t e) const {
    return *reinterpret_cast<const int2*>(sm + (e & NBRL_INDEX));
  }
  __device__ __forceinline__ bool wall(uint32_t e) const { return (e & NBRL_BOUNDARY) != 0u; }
};
// Neighbour access from global memory: records in PL, sorted-index entries.
struct NbrGlobal {
  const int4* g;
  const uint32_t* nl;
  uint32_t stride;
  __device__ __forceinline__ uint32_t entry(uint32_t p, uint32_t k) const { return nl[(size_t)k * stride + p]; }
  __device__ __forceinline__ int4 rec(uint32_t e) const { return g[e & ~NBR_BOUNDARY]; }
  __device__ __forceinline__ int2 pred(uint32_t e) const { return ld_pred(g, e & ~NBR_BOUNDARY); }
  __device__ __forceinline__ bool wall(uint32_t e) const { return (e & NBR_BOUNDARY) != 0u; }
};

// Copy tile t's neighbourhood (`total` records in `runs` runs) from `from`
// (PL or PL2) into `stg`. Every thread of the CTA calls it; warp 0 arms the barrier and issues
// one bulk copy per non-empty run. Returns false for the whole CTA when the
// copies did not land within the bounded wait (ERR_STAGE_TIMEOUT is raised).
__device__ __forceinline__ bool stage_tile(const Bufs& b, const int4* from, const uint32_t* tr, uint32_t runs,
                                           uint32_t total, int4* stg, uint64_t* bar, uint32_t parity, uint32_t* okS) {
  if (threadIdx.x < 32) {
    // the previous tile's reads of stg (ordered by the CTA barrier that ended
    // it) come before these async writes
    stage::fence_proxy_async_smem();
    if (threadIdx.x == 0) stage::mbar_arrive_expect_tx(bar, total * 16u);
    __syncwarp();
    for (uint32_t r = threadIdx.x; r < runs; r += 32) {
      const uint32_t off = tr[TR_BASE + r], len = tr[TR_BASE + r + 1] - off;
      if (len) stage::bulk_g2s(stg + off, from + tr[r], len * 16u, bar);
    }
    if (threadIdx.x == 0) {
      bool ok = stage::mbar_wait_bounded(bar, parity);
      if (!ok) {
        atomicOr(b.err, ERR_STAGE_TIMEOUT);
        stage::mbar_wait_bounded(bar, parity);  // let copies in flight land before the CTA exits
      }
      *okS = ok ? 1u : 0u;
    }
  }
  __syncthreads();
  return *okS != 0u;
}

// solveA's neighbour sums for one particle (L lanes share its list).
template <bool DBG, int L, class NB>
__device__ __forceinline__ void solveA_sums(const Bufs& b, const NB& nb, uint32_t p, uint32_t cnt, uint32_t sub,
                                            int2 pi, const Flags<DBG>& f, int32_t& rho, int32_t& S, int32_t& sgx,
                                            int32_t& sgy) {
  // one neighbour ahead: its entry and position are in flight while the
  // current pair is computed
  uint32_t en = sub < cnt ? nb.entry(p, sub) : 0u;
  int2 pn = nb.pred(en);
  uint32_t en2 = sub + L < cnt ? nb.entry(p, sub + L) : 0u;
  for (uint32_t k = sub; k < cnt; k += L) {
    const int2 pj = pn;
    if (k + L < cnt) pn = nb.pred(en2);
    if (k + 2 * L < cnt) en2 = nb.entry(p, k + 2 * L);
    const int2 d = pdelta(pi, pj, f);
    const int id = lut_index(d, f);
    if (id < 0) continue;
    const int2 wg = __ldg(b.WG + id);
    rho = wadd(rho, wg.x);
    const int32_t gx = mulf<26>(wg.y, d.x, f), gy = mulf<26>(wg.y, d.y, f);
    sgx = wadd(sgx, gx);
    sgy = wadd(sgy, gy);
    S = wadd(S, wadd(mulfc<11>(gx, gx, 0, S_TERM, f), mulfc<11>(gy, gy, 0, S_TERM, f)));
  }
  if (L > 1) {
    rho = gsum<L>(rho);
    S = gsum<L>(S);
    sgx = gsum<L>(sgx);
    sgy = gsum<L>(sgy);
  }
}

// solveA (src/sim.wgsl:1270-1318) for particles [p0, p0 + n) of one tile,
// `me_of(i)` giving particle p0 + i's own record: density, |grad C|^2,
// lambda. On the last iteration it also stores rinv (finalize's,
// src/sim.wgsl:2261-2262), which depends only on this rho.
template <bool DBG, int L, bool BOTH, class NB, class ME>
__device__ __forceinline__ void solveA_tile(const Bufs& b, const NB& nb, ME me_of, uint32_t p0, uint32_t n,
                                            int lastIter, const Flags<DBG>& f) {
  const int32_t W0 = __ldg(b.luts);
  const uint32_t sub = threadIdx.x & (L - 1);
  for (uint32_t i = threadIdx.x / L;; i += blockDim.x / L) {
    if (__shfl_sync(0xffffffffu, i, 0) >= n) break;  // warp-uniform exit
    const bool valid = i < n;
    const uint32_t p = p0 + (valid ? i : 0u);
    const int4 me = valid ? me_of(i) : make_int4(0, 0, 0, (int32_t)INFO_BOUNDARY);
    const uint32_t info = (uint32_t)me.w;
    const bool act = valid && !(info & INFO_BOUNDARY);
    const uint32_t cnt = act ? (b.NBRN[p] & NBRN_COUNT) : 0u;
    int32_t rho = 0, S = 0, sgx = 0, sgy = 0;
    solveA_sums<DBG, L>(b, nb, p, cnt, sub, xy(me), f, rho, S, sgx, sgy);
    if (!act || sub != 0) continue;
    rho = wadd(rho, W0);
    S = wadd(S, wadd(clampi(mul<11>(sgx, sgx, f), 0, S_TERM), clampi(mul<11>(sgy, sgy, f), 0, S_TERM)));
    const int32_t Cq = clampi(shr_rne<4>(wsub(rho, RHO0)), 0, C_MAX);
    const int32_t eps = matw(b, info & INFO_MAT, M_eps);
    const int32_t lam = clampi(neg_sat(divshift<25>(Cq, wadd(S, eps), b.rcp, f), f), -LAM_MAX, LAM_MAX);
    b.PL[p].z = lam;
    if constexpr (BOTH) b.PL2[p].z = lam;
    int4& rx = b.RX[p];
    rx.x = rho;
    if (lastIter) rx.y = clampi(divshift<16>(RHO0, max(rho, RHO_FLOOR_RINV), b.rcp, f), 0, RINV_MAX);
  }
}

// solveA over the sorted particles, the grid striding over them (colour-major
// layout). lam goes to both buffers of the colour sweep, which copies only
// preds between them.
template <bool DBG, int L>
__device__ __forceinline__ void solveA_all(const Bufs& b, int lastIter, const Flags<DBG>& f) {
  const uint32_t nAct = b.world->nAct;
  const int4* PL = b.PL;
  const uint32_t chunk = blockDim.x / L;
  for (uint32_t i0 = blockIdx.x * chunk; i0 < nAct; i0 += gridDim.x * chunk)
    solveA_tile<DBG, L, true>(b, NbrGlobal{PL, b.NBR, b.nbrStride}, [&](uint32_t i) { return PL[i0 + i]; }, i0,
                              min(nAct - i0, chunk), lastIter, f);
}
template <bool DBG, int L>
__global__ void __launch_bounds__(256) k_solveA(Bufs b, int lastIter) {
  Flags<DBG> f{b.dbg};
  solveA_all<DBG, L>(b, lastIter, f);
}

// solveA over every tile. Only lam (PL.z) is written in PL, and no particle
// reads a neighbour's lam here, so other CTAs may stage records of a tile
// whose lam this pass is writing. Tiles that fit are staged, one CTA per tile;
// then every CTA works through the tiles too large to stage (the OVF list),
// all threads of the grid striding over each one's particles.
template <bool DBG, int L>
__global__ void __launch_bounds__(256, 4) k_solveA_tiled(Bufs b, int lastIter) {
  extern __shared__ int4 stg[];
  __shared__ uint64_t bar;
  __shared__ uint32_t okS;
  Flags<DBG> f{b.dbg};
  if (threadIdx.x == 0) {
    stage::mbar_init(&bar, 1);
    stage::fence_mbar_init();
  }
  __syncthreads();
  uint32_t parity = 0;
  const uint32_t nT = b.world->nTiles, stride = b.nbrStride, cap = b.world->stageCap;
  for (uint32_t t = blockIdx.x; t < nT; t += gridDim.x) {
    const TileInfo ti = b.tiles[t];
    if (!b.scenes[ti.scene].active) continue;
    const uint32_t runs = tile_runs(b.scenes[ti.scene].tileShift);
    const uint32_t* tr = b.TR + (size_t)t * TR_STRIDE;
    const uint32_t p0 = tr[0], n = tr[TR_BASE + 1], total = tr[TR_BASE + runs];
    if (n == 0 || total > cap) continue;
    if (!stage_tile(b, b.PL, tr, runs, total, stg, &bar, parity, &okS)) return;
    parity ^= 1u;
    solveA_tile<DBG, L, false>(b, NbrStaged{stg, b.NBRL, stride}, [&](uint32_t i) { return stg[i]; }, p0, n,
                               lastIter, f);
    __syncthreads();  // stg is read before the next tile's copy lands
  }
  const uint32_t nOvf = b.work[2];
  const int4* PL = b.PL;
  for (uint32_t k = 0; k < nOvf; ++k) {
    const uint32_t* tr = b.TR + (size_t)b.OVF[k] * TR_STRIDE;
    const uint32_t p0 = tr[0], n = tr[TR_BASE + 1];
    // the grid strides over the tile's particles: shift p0 by this CTA's share
    const uint32_t first = blockIdx.x * (blockDim.x / L);
    if (first >= n) continue;
    const uint32_t per = gridDim.x * (blockDim.x / L);
    for (uint32_t i0 = first; i0 < n; i0 += per) {
      const uint32_t m = min(n - i0, blockDim.x / L);
      solveA_tile<DBG, L, false>(b, NbrGlobal{PL, b.NBR, stride}, [&](uint32_t i) { return PL[p0 + i0 + i]; },
                                 p0 + i0, m, lastIter, f);
    }
  }
}

// solveB_at (src/sim.wgsl:1337-1372) for one particle. The S table is all
// zeros in the frozen tables (scorrK = 0, checked at load), so the release
// build drops its term; debug builds still read it.
// RIG: the warp holds a rigid member, whose own correction skips the members
// of its body (src/sim.wgsl:1355-1358).
template <bool DBG, int L, bool RIG, class NB>
__device__ __forceinline__ int2 solveB_dp(const Bufs& b, const NB& nb, uint32_t p, uint32_t cnt, uint32_t sub,
                                          int2 pi, int32_t li, const Flags<DBG>& f, uint32_t infoI = 0u) {
  int32_t dpx = 0, dpy = 0;
  uint32_t en = sub < cnt ? nb.entry(p, sub) : 0u;
  int4 on = nb.rec(en);
  uint32_t en2 = sub + L < cnt ? nb.entry(p, sub + L) : 0u;
  for (uint32_t k = sub; k < cnt; k += L) {
    const uint32_t e = en;
    const int4 o = on;
    if (k + L < cnt) {
      en = en2;
      on = nb.rec(en);
    }
    if (k + 2 * L < cnt) en2 = nb.entry(p, k + 2 * L);
    const bool wall = nb.wall(e);
    if constexpr (RIG) {
      if (!wall && same_body(infoI, (uint32_t)o.w)) continue;
    }
    const int2 d = pdelta(pi, xy(o), f);
    const int id = lut_index(d, f);
    if (id < 0) continue;
    const int32_t lj = wall ? li : o.z;
    int32_t co;
    if constexpr (DBG) co = add_sat(add_sat(li, lj, f), __ldg(b.luts + 4 * TN + id), f);
    else co = li + lj;
    const int32_t gt = __ldg(b.WG + id).y;
    dpx = wadd(dpx, mulfc<12>(co, mulf<26>(gt, d.x, f), -DP_TERM, DP_TERM, f));
    dpy = wadd(dpy, mulfc<12>(co, mulf<26>(gt, d.y, f), -DP_TERM, DP_TERM, f));
  }
  if (L > 1) {
    dpx = gsum<L>(dpx);
    dpy = gsum<L>(dpy);
  }
  return make_int2(dpx, dpy);
}

// applyDp_at (src/sim.wgsl:1418-1434).
template <bool DBG>
__device__ __forceinline__ int2 apply_dp(const Bufs& b, const ScenePar& S, uint32_t m, int2 pr, int2 dp,
                                         const Flags<DBG>& f) {
  int32_t dm = matw(b, m, M_dpMax), dmN = neg_sat(dm, f);
  int32_t dx = clampi(shr_rne<8>(dp.x), dmN, dm);
  int32_t dy = clampi(shr_rne<8>(dp.y), dmN, dm);
  return wall_clamp(S, make_int2(add_sat(pr.x, dx, f), add_sat(pr.y, dy, f)));
}

// The colour class's particles [lo, lo + n) of one tile: dp of each from the
// pre-pass records, then `out(p, me, dp)` stores the result. `me_of(p)` gives
// particle p's own pre-pass record. Walls are not passed to `out`.
template <bool DBG, int L, class NB, class ME, class OUT>
__device__ __forceinline__ void colour_tile(const Bufs& b, const NB& nb, ME me_of, OUT out, uint32_t lo, uint32_t n,
                                            const Flags<DBG>& f) {
  const uint32_t sub = threadIdx.x & (L - 1);
  for (uint32_t i = threadIdx.x / L;; i += blockDim.x / L) {
    if (__shfl_sync(0xffffffffu, i, 0) >= n) break;  // warp-uniform exit
    const bool mine = i < n;
    const uint32_t p = lo + (mine ? i : 0u);
    const int4 me = mine ? me_of(p) : make_int4(0, 0, 0, (int32_t)INFO_BOUNDARY);
    const uint32_t info = (uint32_t)me.w;
    const bool act = mine && !(info & INFO_BOUNDARY);
    const uint32_t cnt = act ? (b.NBRN[p] & NBRN_COUNT) : 0u;
    const bool rigidI = act && (info & INFO_RIGID);
    int2 dp;
    if (__any_sync(0xffffffffu, rigidI))
      dp = solveB_dp<DBG, L, true>(b, nb, p, cnt, sub, xy(me), me.z, f, rigidI ? info : 0u);
    else
      dp = solveB_dp<DBG, L, false>(b, nb, p, cnt, sub, xy(me), me.z, f);
    if (sub != 0 || !act) continue;
    out(p, me, dp);
  }
}

// One colour of the block Gauss-Seidel sweep (colour-major layout):
// solveB_cK + applyDp_cK fused. The pass reads every pred from `src` and
// writes its colour's corrected preds to `dst`, so a particle never reads a
// value written in the same pass: that is the Jacobi-within-a-colour rule the
// reference gets from its separate solveB/applyDp dispatches
// (src/sim.wgsl:1323-1332). `dst` must leave the pass complete, so the pass
// also copies the two colours that are stale in it: the sweep alternates
// A->B, B->A, A->B, B->A, colour c is written in phase c and read again four
// phases later, so phase c copies colours c+1 and c-1. After phase 3 buffer A
// is complete again. A rigid member's dp is not applied: rigidSolve folds it
// into its body at the end of the iteration (src/sim.wgsl:1418-1429).
// (No __restrict__ here: the persistent kernel reads buffers that its own
// earlier phases wrote, which must not go through the non-coherent load path.)
// Phase c's copy of colours c+1 and c-1 (the two stale in dst) from src.
__device__ __forceinline__ void copy_other_colours(const Bufs& b, int colour, const int4* src, int4* dst) {
  const uint32_t* cb = b.world->colourBase;
  const int c1 = (colour + 1) & 3, c3 = (colour + 3) & 3;
  const uint32_t lo1 = b.cellStart[cb[c1]], hi1 = b.cellStart[cb[c1 + 1]];
  const uint32_t lo3 = b.cellStart[cb[c3]], hi3 = b.cellStart[cb[c3 + 1]];
  const uint32_t n1 = hi1 - lo1, n13 = n1 + (hi3 - lo3);
  for (uint32_t i = gtid(); i < n13; i += gstride()) {
    const uint32_t p = i < n1 ? lo1 + i : lo3 + (i - n1);
    *reinterpret_cast<int2*>(dst + p) = *reinterpret_cast<const int2*>(src + p);
  }
}

template <bool DBG, int L>
__device__ __forceinline__ void colour_all(const Bufs& b, int colour, const int4* src, int4* dst,
                                           const Flags<DBG>& f, bool copyOthers = true) {
  const uint32_t* cb = b.world->colourBase;
  const uint32_t lo = b.cellStart[cb[colour]], hi = b.cellStart[cb[colour + 1]];
  // The grid covers this colour's range only (the launch is sized to the
  // resident capacity); the copies of the neighbouring colours follow, or
  // run beside the pass in k_colour_copy.
  const uint32_t chunk = blockDim.x / L;
  const NbrGlobal nb{src, b.NBR, b.nbrStride};
  for (uint32_t i0 = blockIdx.x * chunk; i0 < hi - lo; i0 += gridDim.x * chunk)
    colour_tile<DBG, L>(
        b, nb, [&](uint32_t p) { return src[p]; },
        [&](uint32_t p, int4 me, int2 dp) {
          const uint32_t info = (uint32_t)me.w;
          int2 pr = xy(me);
          if (info & INFO_RIGID) b.DP[p] = dp;
          if (!(info & INFO_PINNED)) pr = apply_dp(b, b.scenes[b.SCN[p]], info & INFO_MAT, pr, dp, f);
          *reinterpret_cast<int2*>(dst + p) = pr;
        },
        lo + i0, min(hi - lo - i0, chunk), f);
  if (copyOthers) copy_other_colours(b, colour, src, dst);
}
template <bool DBG, int L>
__global__ void __launch_bounds__(256, 8) k_colour(Bufs b, int colour, const int4* __restrict__ src,
                                                int4* __restrict__ dst, int copyOthers) {
  Flags<DBG> f{b.dbg};
  colour_all<DBG, L>(b, colour, src, dst, f, copyOthers != 0);
}
// The copy of phase c, launched on a forked branch of the substep so it runs
// in the slots the pass leaves free; it touches none of the words the pass
// reads from dst or writes.
__global__ void __launch_bounds__(256) k_colour_copy(Bufs b, int colour, const int4* __restrict__ src,
                                                     int4* __restrict__ dst) {
  copy_other_colours(b, colour, src, dst);
}

// One colour of the sweep in the tile-major layout, with staged gathers.
// The pass reads every record from `src` and writes every record to `dst`
// (colour c's with their corrected preds, the rest unchanged), so a particle
// never reads a value written in the same pass: that is the Jacobi-within-a-
// colour rule the reference gets from its separate solveB/applyDp dispatches
// (src/sim.wgsl:1323-1332). The sweep alternates A->B, B->A, A->B, B->A, so
// after the fourth colour A is current again. The first pass of an iteration
// (FULL) writes whole records, since B's lam is one iteration old; the others
// write only the preds.
//
// Tiles that fit are staged from `src`, one CTA per tile, which writes its
// whole tile to `dst` from the staged copy; then every CTA works through the
// tiles too large to stage, the grid striding over each one's particles.
// A rigid member's dp is not applied: rigidSolve folds it into its body at the
// end of the iteration (src/sim.wgsl:1418-1429).
template <bool DBG, int L, bool FULL>
__global__ void __launch_bounds__(256, 6) k_colour_tiled(Bufs b, int colour, const int4* __restrict__ src,
                                                      int4* __restrict__ dst) {
  extern __shared__ int4 stg[];
  __shared__ uint64_t bar;
  __shared__ uint32_t okS;
  Flags<DBG> f{b.dbg};
  if (threadIdx.x == 0) {
    stage::mbar_init(&bar, 1);
    stage::fence_mbar_init();
  }
  __syncthreads();
  auto put = [&](uint32_t p, int4 rec) {
    if constexpr (FULL) dst[p] = rec;
    else *reinterpret_cast<int2*>(dst + p) = xy(rec);
  };
  // the corrected record of an active colour-c particle
  auto moved = [&](const ScenePar& S, uint32_t p, int4 me, int2 dp) {
    const uint32_t info = (uint32_t)me.w;
    if (info & INFO_RIGID) b.DP[p] = dp;
    if (!(info & INFO_PINNED)) {
      const int2 pr = apply_dp(b, S, info & INFO_MAT, xy(me), dp, f);
      me.x = pr.x;
      me.y = pr.y;
    }
    put(p, me);
  };
  uint32_t parity = 0;
  const uint32_t nT = b.world->nTiles, stride = b.nbrStride, cap = b.world->stageCap;
  for (uint32_t t = blockIdx.x; t < nT; t += gridDim.x) {
    const TileInfo ti = b.tiles[t];
    const ScenePar& S = b.scenes[ti.scene];
    if (!S.active) continue;
    const uint32_t ts = S.tileShift, runs = tile_runs(ts);
    const uint32_t* tr = b.TR + (size_t)t * TR_STRIDE;
    const uint32_t p0 = tr[0], n0 = tr[TR_BASE + 1], total = tr[TR_BASE + runs];
    if (n0 == 0 || total > cap) continue;
    const uint32_t Q = 1u << (2u * ts - 2u);
    const uint32_t lo = b.cellStart[ti.key0 + colour * Q], n = b.cellStart[ti.key0 + (colour + 1) * Q] - lo;
    if (!stage_tile(b, src, tr, runs, total, stg, &bar, parity, &okS)) return;
    parity ^= 1u;
    colour_tile<DBG, L>(
        b, NbrStaged{stg, b.NBRL, stride}, [&](uint32_t p) { return stg[p - p0]; },
        [&](uint32_t p, int4 me, int2 dp) { moved(S, p, me, dp); }, lo, n, f);
    // the rest of the tile (other colours and walls) unchanged
    for (uint32_t i = threadIdx.x; i < n0; i += blockDim.x) {
      const uint32_t p = p0 + i;
      const int4 me = stg[i];
      if (p - lo < n && !((uint32_t)me.w & INFO_BOUNDARY)) continue;  // written above
      put(p, me);
    }
    __syncthreads();  // stg is read before the next tile's copy lands
  }
  const uint32_t nOvf = b.work[2];
  for (uint32_t k = 0; k < nOvf; ++k) {
    const uint32_t tIdx = b.OVF[k];
    const TileInfo ti = b.tiles[tIdx];
    const ScenePar& S = b.scenes[ti.scene];
    const uint32_t* tr = b.TR + (size_t)tIdx * TR_STRIDE;
    const uint32_t p0 = tr[0], n0 = tr[TR_BASE + 1];
    const uint32_t Q = 1u << (2u * S.tileShift - 2u);
    const uint32_t lo = b.cellStart[ti.key0 + colour * Q], n = b.cellStart[ti.key0 + (colour + 1) * Q] - lo;
    // colour c: the grid strides over the class with L lanes per particle
    const uint32_t first = blockIdx.x * (blockDim.x / L), per = gridDim.x * (blockDim.x / L);
    for (uint32_t i0 = first; i0 < n; i0 += per) {
      const uint32_t m = min(n - i0, blockDim.x / L);
      colour_tile<DBG, L>(
          b, NbrGlobal{src, b.NBR, stride}, [&](uint32_t p) { return src[p]; },
          [&](uint32_t p, int4 me, int2 dp) { moved(S, p, me, dp); }, lo + i0, m, f);
    }
    // every other record of the tile, and the class's walls, copied
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n0; i += gridDim.x * blockDim.x) {
      const uint32_t p = p0 + i;
      const int4 me = src[p];
      if (p - lo < n && !((uint32_t)me.w & INFO_BOUNDARY)) continue;
      put(p, me);
    }
  }
}

// friction + the bond gather (src/sim.wgsl:1673-1934). Rows with fric == 0
// and bondK == 0 take the reference's zero-work path: their dp is 0 and
// applyFric leaves their (already wall-clamped) pred unchanged, so they are
// skipped here and in k_apply_fric. Results go to DP; k_apply_fric applies
// them (applyFric, src/sim.wgsl:1945-1950) after every row has read pred.
__device__ __forceinline__ bool friction_row(const Bufs& b, uint32_t m) {
  return matw(b, m, M_fric) != 0 || matw(b, m, M_bondK) != 0;
}
// L lanes share one particle's neighbour list (the friction sums wrap, so
// any split is exact); a friction row's cost is one chain of dependent
// gathers, which the split shortens L-fold. The bond gather stays on the
// particle's first lane.
template <bool DBG, int L>
__device__ __forceinline__ void friction_all(const Bufs& b, const Flags<DBG>& f) {
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  const uint32_t sub = threadIdx.x & (L - 1), G = gstride() / L;
  for (uint32_t p = gtid() / L;; p += G) {
    if (__shfl_sync(0xffffffffu, p, 0) >= nAct) break;  // warp-uniform exit
    const bool valid = p < nAct;
    const int4 me = valid ? b.PL[p] : make_int4(0, 0, 0, (int32_t)INFO_BOUNDARY);
    const uint32_t info = (uint32_t)me.w;
    const uint32_t m = info & INFO_MAT;
    const bool act = valid && !(info & INFO_BOUNDARY) && friction_row(b, m);
    // a rigid member skips its own body, gathers no bonds and ADDS its friction
    // to the solver dp waiting for rigidSolve (src/sim.wgsl:1680-1688, 1925-1929)
    const bool rigidI = (info & INFO_RIGID) != 0u;
    const int32_t fi = act ? matw(b, m, M_fric) : 0;
    const int2 pi = xy(me);
    const uint32_t pp = act ? p : 0u;
    const int2 dxi = delta(pi, b.POS[pp], f);
    const uint32_t cnt = fi != 0 ? (b.NBRN[p] & NBRN_COUNT) : 0u;
    int32_t fx = 0, fy = 0;
    // one neighbour ahead (record and old position), two ahead (index)
    const uint32_t* np = b.NBR + pp;
    uint32_t en = sub < cnt ? np[(size_t)sub * stride] : 0u;
    int4 on = b.PL[en & ~NBR_BOUNDARY];
    int2 sn = b.POS[en & ~NBR_BOUNDARY];
    uint32_t en2 = sub + L < cnt ? np[(size_t)(sub + L) * stride] : 0u;
    for (uint32_t k = sub; k < cnt; k += L) {
      const uint32_t e = en;
      const int4 o = on;
      const int2 so = sn;
      if (k + L < cnt) {
        en = en2;
        on = b.PL[en & ~NBR_BOUNDARY];
        sn = b.POS[en & ~NBR_BOUNDARY];
      }
      if (k + 2 * L < cnt) en2 = np[(size_t)(k + 2 * L) * stride];
      if (rigidI && !(e & NBR_BOUNDARY) && same_body(info, (uint32_t)o.w)) continue;
      int2 pq = xy(o);
      int2 d = pdelta(pi, pq, f);
      int id = lut_index(d, f);
      if (id < 0) continue;
      int32_t d4x = shr_rne<FPRE>(d.x), d4y = shr_rne<FPRE>(d.y);
      int32_t d2 = wadd(wmul(d4x, d4x), wmul(d4y, d4y));
      if (d2 < D2_FLOOR) continue;
      int2 rel = dxi;
      int32_t mu = fi;
      if (!(e & NBR_BOUNDARY)) {
        int2 dq = delta(pq, so, f);
        rel = make_int2(sub_sat(dxi.x, dq.x, f), sub_sat(dxi.y, dq.y, f));
        mu = mat_mix(fi, matw(b, (uint32_t)o.w & INFO_MAT, M_fric));
      }
      if (mu == 0) continue;
      int32_t r4x = shr_rne<RPRE>(rel.x), r4y = shr_rne<RPRE>(rel.y);
      int32_t dot = wadd(wmul(d4x, r4x), wmul(d4y, r4y));
      int32_t qq = divshift<16>(dot, d2, b.rcp, f);
      int32_t tx = sub_sat(r4x, mul<16>(d4x, qq, f), f);
      int32_t ty = sub_sat(r4y, mul<16>(d4y, qq, f), f);
      int32_t wq = shr_rne<4>(__ldg(b.WG + id).x);
      int32_t sx = mul<16>(mul<5>(tx, wq, f), mu, f);
      int32_t sy = mul<16>(mul<5>(ty, wq, f), mu, f);
      fx = wsub(fx, clampi(sx, -FR_TERM, FR_TERM));
      fy = wsub(fy, clampi(sy, -FR_TERM, FR_TERM));
    }
    if (L > 1) {
      fx = gsum<L>(fx);
      fy = gsum<L>(fy);
    }
    if (!act || sub != 0) continue;
    if (rigidI) {
      const int2 d0 = b.DP[p];
      b.DP[p] = make_int2(add_sat(d0.x, fx, f), add_sat(d0.y, fy, f));
      continue;
    }
    const int32_t bondKi = matw(b, m, M_bondK);
    int32_t bx = 0, by = 0;
    if (bondKi != 0 && !(info & INFO_BURST)) {
      uint32_t slot = b.sslot[p];
      int32_t ki = bond_k(b, m, b.RX[p].z, f);
      const uint32_t base = b.scenes[b.SCN[p]].slotBase;
      uint32_t* row = b.bond + (size_t)slot * BOND_CAP;
      for (int k = 0; k < BOND_CAP; ++k) {
        uint32_t w = row[k];
        if (w == 0u) break;
        if (w & BOND_TOMB) continue;
        uint32_t q = b.inv[base + (w & BOND_J_MASK)];
        int4 o = b.PL[q];
        uint32_t mj = (uint32_t)o.w & INFO_MAT;
        if ((uint32_t)o.w & INFO_BURST) { row[k] = w | BOND_TOMB; continue; }
        if (matw(b, mj, M_bondK) == 0) { row[k] = w | BOND_TOMB; continue; }
        int32_t L0 = (int32_t)((w >> 17) & 0x1fffu);
        int32_t L02 = wmul(L0, L0);
        int2 d = delta(pi, xy(o), f);
        int32_t d4x = shr_rne<BPRE>(d.x), d4y = shr_rne<BPRE>(d.y);
        if (abs(d4x) > L0_MAX || abs(d4y) > L0_MAX) { row[k] = w | BOND_TOMB; continue; }
        int32_t d2 = wadd(wmul(d4x, d4x), wmul(d4y, d4y));
        if (d2 >= HARD_BREAK2) { row[k] = w | BOND_TOMB; continue; }
        int32_t mb = min(matw(b, m, M_bondBreak), matw(b, mj, M_bondBreak));
        int32_t mub = min(matw(b, m, M_bondMu), matw(b, mj, M_bondMu));
        if (mb != 0 && mub != 0) {
          int32_t lp = neg_sat(add_sat(me.z, o.z, f), f);
          int32_t Pq = lp > 0 ? shr_rne<4>(lp) : 0;
          mb = wadd(wadd(65536, wsub(mb, 65536)), mul<16>(Pq, mub, f));
        }
        if (mb != 0 && d2 > mul<16>(L02, mb, f)) { row[k] = w | BOND_TOMB; continue; }
        if (d2 < D2_FLOOR) continue;
        int32_t kj = bond_k(b, mj, b.RX[q].z, f);
        int32_t kp = min(ki, kj);
        if (kp == 0) continue;
        int32_t C = sub_sat(d2, L02, f);
        int32_t qv = divshift<16>(C, wmul(d2, 4), b.rcp, f);
        int32_t qk = mul<16>(qv, kp, f);
        int32_t gx = mul<3>(d4x, qk, f);
        int32_t gy = mul<3>(d4y, qk, f);
        bx = wsub(bx, clampi(gx, -BD_TERM, BD_TERM));
        by = wsub(by, clampi(gy, -BD_TERM, BD_TERM));
      }
    }
    b.DP[p] = make_int2(add_sat(fx, bx, f), add_sat(fy, by, f));
  }
}

template <bool DBG, int L>
__global__ void __launch_bounds__(256) k_friction(Bufs b) {
  if (*b.work == 0u) return;  // no particle has a friction or bond row this substep
  Flags<DBG> f{b.dbg};
  friction_all<DBG, L>(b, f);
}

template <bool DBG>
__device__ __forceinline__ void apply_fric_all(const Bufs& b, const Flags<DBG>& f) {
  const uint32_t nAct = b.world->nAct;
  for (uint32_t p = gtid(); p < nAct; p += gstride()) {
    int4 me = b.PL[p];
    uint32_t info = (uint32_t)me.w;
    if (info & (INFO_BOUNDARY | INFO_PINNED)) continue;
    uint32_t m = info & INFO_MAT;
    if (!friction_row(b, m)) continue;
    const ScenePar& S = b.scenes[b.SCN[p]];
    int2 np = apply_dp(b, S, m, xy(me), b.DP[p], f);
    *reinterpret_cast<int2*>(b.PL + p) = np;
    *reinterpret_cast<int2*>(b.PL2 + p) = np;
  }
}
template <bool DBG>
__global__ void __launch_bounds__(256) k_apply_fric(Bufs b) {
  if (*b.work == 0u) return;
  Flags<DBG> f{b.dbg};
  apply_fric_all<DBG>(b, f);
}

// ---- the persistent form of the solver loop (opt-in, sn_set_persistent) ----
//
// One cooperative launch runs all `iters` iterations of solveA, the four
// colour passes and (when some particle has a friction or bond row this
// substep) friction and applyFric, for worlds with no rigid body (rigidSolve
// keeps the per-phase launches), the phases separated by grid barriers
// instead of kernel boundaries. The barrier counts arrivals monotonically in bar[0] (zeroed
// before each launch) and releases generation g by writing g + 1 to bar[1];
// a CTA that waits longer than BARRIER_WAIT_CYCLES raises ERR_BARRIER and the
// kernel returns (its results are then not valid; sn_check_errors reports it).
constexpr long long BARRIER_WAIT_CYCLES = 1ll << 31;  // about a second
__device__ __forceinline__ bool grid_barrier(uint32_t* bar, uint32_t* err, uint32_t& gen) {
  __shared__ uint32_t okS;
  __syncthreads();
  if (threadIdx.x == 0) {
    okS = 1u;
    __threadfence();
    const uint32_t target = gridDim.x * (gen + 1u);
    if (atomicAdd(bar, 1u) + 1u == target) {
      atomicExch(bar + 1, gen + 1u);
    } else {
      const long long t0 = clock64();
      while (*(volatile uint32_t*)(bar + 1) <= gen) {
        if (clock64() - t0 > BARRIER_WAIT_CYCLES) {
          atomicOr(err, ERR_BARRIER);
          okS = 0u;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  gen += 1u;
  return okS != 0u;
}
template <bool DBG, int L>
__global__ void __launch_bounds__(256, 8) k_iters_persistent(Bufs b, uint32_t iters, uint32_t* bar) {
  Flags<DBG> f{b.dbg};
  uint32_t gen = 0;
  for (uint32_t it = 0; it < iters; ++it) {
    solveA_all<DBG, L>(b, it + 1 == iters ? 1 : 0, f);
    for (int c = 0; c < 4; ++c) {
      if (!grid_barrier(bar, b.err, gen)) return;
      colour_all<DBG, L>(b, c, (c & 1) ? b.PL2 : b.PL, (c & 1) ? b.PL : b.PL2, f);
    }
    // friction and applyFric, when some particle has a friction or bond row
    // this substep (the flag is the same for every CTA)
    if (*(volatile uint32_t*)b.work != 0u) {
      if (!grid_barrier(bar, b.err, gen)) return;
      friction_all<DBG, L>(b, f);
      if (!grid_barrier(bar, b.err, gen)) return;
      apply_fric_all<DBG>(b, f);
    }
    if (it + 1 < iters && !grid_barrier(bar, b.err, gen)) return;
  }
}


// finalize + xsph + normals + conduct (src/sim.wgsl:2245-2582) in one sweep
// over the neighbour list. vtmp_j = clamp(pred_j - pos_j) is finalize's
// velocity, recomputed where it is needed.
template <bool DBG, int L>
__global__ void __launch_bounds__(256, 4) k_post1(Bufs b) {
  Flags<DBG> f{b.dbg};
  __shared__ int4 smat[MAT_MAX];  // {xsph, cond, corrode, corrPt}
  for (int m = threadIdx.x; m < MAT_MAX; m += blockDim.x)
    smat[m] = make_int4(matw(b, m, M_xsph), matw(b, m, M_cond), matw(b, m, M_corrode), matw(b, m, M_corrPt));
  __syncthreads();
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  const uint32_t sub = threadIdx.x & (L - 1), G = gstride() / L;
  for (uint32_t p = gtid() / L;; p += G) {
    if (__shfl_sync(0xffffffffu, p, 0) >= nAct) break;  // warp-uniform exit
    const bool valid = p < nAct;
    const int4 me = valid ? b.PL[p] : make_int4(0, 0, 0, (int32_t)INFO_BOUNDARY);
    const uint32_t info = (uint32_t)me.w;
    const bool act = valid && !(info & INFO_BOUNDARY);
    const uint32_t pp = act ? p : 0u;
    const ScenePar& S = b.scenes[b.SCN[pp]];
    const int32_t vmax = S.vmax, vmaxN = neg_sat(vmax, f);
    const uint32_t m = info & INFO_MAT;
    const int2 pi = xy(me);
    int2 vi = delta(pi, b.POS[pp], f);
    vi.x = clampi(vi.x, vmaxN, vmax);
    vi.y = clampi(vi.y, vmaxN, vmax);
    const bool doX = !(info & INFO_PINNED);
    const int4 mi = smat[m];
    const int4 rxi = b.RX[pp];
    const int32_t rhoi = rxi.x, Ti = rxi.z;
    const uint32_t cnt = act ? (b.NBRN[p] & NBRN_COUNT) : 0u;
    int32_t ax = 0, ay = 0, sx = 0, sy = 0, hq = 0, hc = 0;
    const uint32_t* np = b.NBR + pp;
    // the neighbour's three records (pred/info, rho/rinv/T, old position)
    // one ahead, its index two ahead
    uint32_t en = sub < cnt ? np[(size_t)sub * stride] : 0u;
    int4 on = b.PL[en & ~NBR_BOUNDARY];
    int4 rn = b.RX[en & ~NBR_BOUNDARY];
    int2 sn = b.POS[en & ~NBR_BOUNDARY];
    uint32_t en2 = sub + L < cnt ? np[(size_t)(sub + L) * stride] : 0u;
    for (uint32_t k = sub; k < cnt; k += L) {
      const uint32_t e = en;
      const int4 o = on;
      const int4 rx = rn;
      const int2 so = sn;
      if (k + L < cnt) {
        en = en2;
        on = b.PL[en & ~NBR_BOUNDARY];
        rn = b.RX[en & ~NBR_BOUNDARY];
        sn = b.POS[en & ~NBR_BOUNDARY];
      }
      if (k + 2 * L < cnt) en2 = np[(size_t)(k + 2 * L) * stride];
      if (e & NBR_BOUNDARY) continue;
      const int2 pq = xy(o);
      const int2 d = pdelta(pi, pq, f);
      const int id = lut_index(d, f);
      if (id < 0) continue;
      const int2 wg = __ldg(b.WG + id);
      const int32_t W = wg.x;
      const int4 mj = smat[(uint32_t)o.w & INFO_MAT];
      if (doX) {
        int32_t K = sym_k(rhoi, rx.x, b.rcp, f);
        int32_t wk = mulf<16>(W, K, f);
        int32_t cij = mat_mix(mi.x, mj.x);
        int2 vj = delta(pq, so, f);
        vj.x = clampi(vj.x, vmaxN, vmax);
        vj.y = clampi(vj.y, vmaxN, vmax);
        ax = wadd(ax, mulfc<16>(mulf<12>(sub_sat(vj.x, vi.x, f), wk, f), cij, -XS_TERM, XS_TERM, f));
        ay = wadd(ay, mulfc<16>(mulf<12>(sub_sat(vj.y, vi.y, f), wk, f), cij, -XS_TERM, XS_TERM, f));
      }
      sx = wadd(sx, mulf<16>(mulf<26>(wg.y, d.x, f), rx.y, f));
      sy = wadd(sy, mulf<16>(mulf<26>(wg.y, d.y, f), rx.y, f));
      {
        int32_t cij = mat_mix(mi.y, mj.y);
        int32_t wk = mulf<16>(W, cij, f);
        int32_t dT = clampi(sub_sat(rx.z, Ti, f), -DT_CLAMP, DT_CLAMP);
        hq = wadd(hq, mulfc<12>(dT, wk, -HT_TERM, HT_TERM, f));
        if (((uint32_t)o.w & INFO_MAT) != m) {
          int32_t spend = mj.w != CORR_NEVER ? mi.z : 0;
          int32_t str = wadd(mj.z, spend);
          if (str != 0) hc = wadd(hc, mulfc<12>(W, str, 0, CORR_TERM, f));
        }
      }
    }
    if (L > 1) {
      ax = gsum<L>(ax);
      ay = gsum<L>(ay);
      sx = gsum<L>(sx);
      sy = gsum<L>(sy);
      hq = gsum<L>(hq);
      hc = gsum<L>(hc);
    }
    if (!valid || sub != 0) continue;
    int32_t* w = b.state + (size_t)b.sslot[p] * 8;
    if (!act) {
      *reinterpret_cast<int2*>(w + 2) = make_int2(0, 0);  // finalize: walls end with zero velocity
      continue;
    }
    b.NQ[p] = make_int4(mul<16>(sx, H, f), mul<16>(sy, H, f), rhoi, 0);
    b.HEAT[p] = hq;
    b.CORR[p] = hc;
    int2 vo = vi;
    if (doX) vo = make_int2(add_sat(vi.x, shr_rne<8>(ax), f), add_sat(vi.y, shr_rne<8>(ay), f));
    *reinterpret_cast<int4*>(w) = make_int4(pi.x, pi.y, vo.x, vo.y);
  }
}

// ---- §29 containment (src/sim.wgsl:1953-2235, 2733-2771) ---------------------
constexpr int32_t SEAL_SEG_MAX2 = 8820900, SEAL_SEG_MIN2 = 670761, SEAL_KEEP4 = 717, SEAL_REACH = 95027;
constexpr int32_t SEAL_STRESS4 = 2560;

__device__ __forceinline__ bool seal_liquid(const Bufs& b, uint32_t m) {
  return matw(b, m, M_bondK) == 0 && matw(b, m, M_fric) == 0 && matw(b, m, M_grav) > 0 && matw(b, m, M_phantom) == 0;
}

// fp_div_s with s = 16 (src/fixed.wgsl:219-261): (|a| << 16) / |b| exactly,
// rounded half to even on the exact remainder, signed and saturated. Only
// the rare close-contact case of the keep-out push divides.
template <bool DBG>
__device__ int32_t div_s16(int32_t a, int32_t b, const Flags<DBG>& f) {
  if (b == 0) {
    f.flag(2);
    return a == 0 ? 0 : (a > 0 ? I32_MAX : I32_MIN);
  }
  const bool neg = (a < 0) != (b < 0);
  const uint64_t ua = a < 0 ? (uint64_t)(-(int64_t)a) : (uint64_t)a;
  const uint64_t ub = b < 0 ? (uint64_t)(-(int64_t)b) : (uint64_t)b;
  const uint64_t n = ua << 16;
  const uint64_t q = n / ub, rem = n - q * ub;
  bool ovf = q > 0xffffffffull;
  uint32_t q32 = (uint32_t)q;
  const uint64_t other = ub - rem;
  if (rem > other || (rem == other && (q32 & 1u))) {
    if (q32 == 0xffffffffu) { ovf = true; q32 = 0; } else { ++q32; }
  }
  if (ovf) { f.flag(1); return neg ? I32_MIN : I32_MAX; }
  if (neg) {
    if (q32 > 2147483648u) { f.flag(1); return I32_MIN; }
    if (q32 == 2147483648u) return I32_MIN;
    return -(int32_t)q32;
  }
  if (q32 > 2147483647u) { f.flag(1); return I32_MAX; }
  return (int32_t)q32;
}

// seal_cross_sign: the sign of ax*by - ay*bx, exact in 64 bits.
__device__ __forceinline__ int seal_cross_sign(int32_t ax, int32_t ay, int32_t bx, int32_t by) {
  const int64_t d = (int64_t)ax * by - (int64_t)ay * bx;
  return d == 0 ? 0 : (d < 0 ? -1 : 1);
}

// The geometry contain and containOverflow share: a keep-out push from each
// seal endpoint, then the swept-segment test against every pair of seal
// endpoints, where a crossing reverts this substep's motion. `entry(k)` gives
// the k-th candidate's sorted index with NBR_BOUNDARY set for wall particles;
// `filter` means the list still holds entries that are not seal endpoints.
template <bool DBG, typename Entry>
__device__ int2 contain_core(const Bufs& b, Entry entry, uint32_t n, bool filter, int2 pos, int2 pr, bool liquidI,
                             const Flags<DBG>& f) {
  auto seal_at = [&](uint32_t e) {
    return !(e & NBR_BOUNDARY) && seal_class(b, (uint32_t)b.PL[e & ~NBR_BOUNDARY].w & INFO_MAT);
  };
  bool touched = false;
  for (uint32_t k = 0; k < n; ++k) {
    const uint32_t e = entry(k);
    if (filter && !seal_at(e)) continue;
    touched = true;
    const int2 pj = ld_pred(b.PL, e & ~NBR_BOUNDARY);
    const int32_t dx4 = shr_rne<BPRE>(sub_sat(pr.x, pj.x, f)), dy4 = shr_rne<BPRE>(sub_sat(pr.y, pj.y, f));
    const int32_t d2 = wadd(wmul(dx4, dx4), wmul(dy4, dy4));
    if (d2 > 0 && d2 < SEAL_KEEP4 * SEAL_KEEP4) {
      const int32_t d4 = (int32_t)isqrt32((uint32_t)d2);
      if (d4 > 0) {
        const int32_t ux = div_s16(dx4, d4, f), uy = div_s16(dy4, d4, f);
        const int32_t amt = (int32_t)((uint32_t)(SEAL_KEEP4 - d4) << BPRE);
        pr.x = add_sat(pr.x, mul<16>(ux, amt, f), f);
        pr.y = add_sat(pr.y, mul<16>(uy, amt, f), f);
      }
    }
  }
  if (!touched) return pr;
  for (uint32_t k = 0; k < n; ++k) {
    const uint32_t e = entry(k);
    if (filter && !seal_at(e)) continue;
    const uint32_t j = e & ~NBR_BOUNDARY;
    const int4 oj = b.PL[j];
    const int32_t sealModeJ = matw(b, (uint32_t)oj.w & INFO_MAT, M_sealMode);
    const int2 pj = xy(oj);
    for (uint32_t q = k + 1; q < n; ++q) {
      const uint32_t e2 = entry(q);
      if (filter && !seal_at(e2)) continue;
      const int4 ok = b.PL[e2 & ~NBR_BOUNDARY];
      if (liquidI && sealModeJ != 0 && matw(b, (uint32_t)ok.w & INFO_MAT, M_sealMode) != 0) continue;
      const int2 pk = xy(ok);
      const int32_t ex4 = shr_rne<BPRE>(sub_sat(pk.x, pj.x, f)), ey4 = shr_rne<BPRE>(sub_sat(pk.y, pj.y, f));
      const int32_t el2 = wadd(wmul(ex4, ex4), wmul(ey4, ey4));
      if (el2 > SEAL_SEG_MAX2 || el2 < SEAL_SEG_MIN2) continue;
      if (min(pj.x, pk.x) > max(pos.x, pr.x) || max(pj.x, pk.x) < min(pos.x, pr.x) ||
          min(pj.y, pk.y) > max(pos.y, pr.y) || max(pj.y, pk.y) < min(pos.y, pr.y))
        continue;
      const int32_t ex = sub_sat(pk.x, pj.x, f), ey = sub_sat(pk.y, pj.y, f);
      const int s0 = seal_cross_sign(ex, ey, sub_sat(pos.x, pj.x, f), sub_sat(pos.y, pj.y, f));
      const int s1 = seal_cross_sign(ex, ey, sub_sat(pr.x, pj.x, f), sub_sat(pr.y, pj.y, f));
      if (s0 == 0 || s0 == s1) continue;
      const int32_t mx = sub_sat(pr.x, pos.x, f), my = sub_sat(pr.y, pos.y, f);
      const int t0 = seal_cross_sign(mx, my, sub_sat(pj.x, pos.x, f), sub_sat(pj.y, pos.y, f));
      const int t1 = seal_cross_sign(mx, my, sub_sat(pk.x, pos.x, f), sub_sat(pk.y, pos.y, f));
      if (t0 == t1 && t0 != 0) continue;
      pr = pos;
    }
  }
  return pr;
}

// contain (src/sim.wgsl:2058-2140) + containOverflow (:2144-2235) in one
// launch: each writes only an intruder's pred and reads only seal endpoints'
// preds, which neither moves, so fusing them changes nothing. Runs after the
// last solver iteration, on the final preds in PL.
template <bool DBG>
__global__ void __launch_bounds__(256) k_contain(Bufs b) {
  // a list holds a seal endpoint (NBRN_SEAL) only if some live fluid particle
  // carries SEAL, which k_gather reports in work[1] (with CONGEAL)
  if (b.work[1] == 0u) return;
  Flags<DBG> f{b.dbg};
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  for (uint32_t p = gtid(); p < nAct; p += gstride()) {
    const uint32_t nn = b.NBRN[p];
    if (!(nn & NBRN_SEAL)) continue;
    const int4 me = b.PL[p];
    const uint32_t info = (uint32_t)me.w;
    if (info & (INFO_BOUNDARY | INFO_PINNED)) continue;
    const uint32_t m = info & INFO_MAT;
    if (seal_class(b, m) || matw(b, m, M_phantom) != 0) continue;
    const int2 pos = b.POS[p];
    int2 pr = xy(me);
    const bool liquidI = seal_liquid(b, m);
    const uint32_t cnt = nn & NBRN_COUNT;
    if (cnt < (uint32_t)MAXNBR) {
      const uint32_t* col = b.NBR + p;
      pr = contain_core(b, [&](uint32_t k) { return col[(size_t)k * stride]; }, cnt, true, pos, pr, liquidI, f);
    } else {
      uint32_t seals[MAXNBR];
      uint32_t sealN = 0;
      const int32_t loX = sub_sat(min(pos.x, pr.x), SEAL_REACH, f), hiX = add_sat(max(pos.x, pr.x), SEAL_REACH, f);
      const int32_t loY = sub_sat(min(pos.y, pr.y), SEAL_REACH, f), hiY = add_sat(max(pos.y, pr.y), SEAL_REACH, f);
      const ScenePar& S = b.scenes[b.SCN[p]];
      const int2 cc = cell_coord(S, pr);
      for (int dy = -1; dy <= 1; ++dy) {
        const int32_t gy = cc.y + dy;
        if (gy < 0 || gy >= (int32_t)S.gridH) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          const int32_t gx = cc.x + dx;
          if (gx < 0 || gx >= (int32_t)S.gridW) continue;
          const uint32_t key = key_of(S, gx, gy);
          for (uint32_t q = b.cellStart[key]; q < b.cellStart[key + 1]; ++q) {
            const int4 o = b.PL[q];
            if (((uint32_t)o.w & INFO_BOUNDARY) || !seal_class(b, (uint32_t)o.w & INFO_MAT)) continue;
            if (o.x < loX || o.x > hiX || o.y < loY || o.y > hiY) continue;
            if (sealN < (uint32_t)MAXNBR) seals[sealN++] = q;
          }
        }
      }
      pr = contain_core(b, [&](uint32_t k) { return seals[k]; }, sealN, false, pos, pr, liquidI, f);
    }
    *reinterpret_cast<int2*>(b.PL + p) = pr;
  }
}

// containStress (src/sim.wgsl:2742-2771), after thermal: a held seal particle
// sums nearby intrusion and, past its row's burstP, lets go (FLAG_BURST). It
// writes only its own flags word and reads neighbours' positions and rows.
// Walks slots (one coalesced read of the two words that decide) and visits
// the neighbour list only for held seal particles. L lanes share one slot's
// list (the stress sum wraps, so any split is exact): a seal body's members
// each walk a list, and the split shortens that serial gather chain.
template <bool DBG, int L>
__global__ void __launch_bounds__(256) k_contain_stress(Bufs b) {
  Flags<DBG> f{b.dbg};
  const uint32_t slotEnd = b.world->slotEnd, stride = b.nbrStride;
  const uint32_t sub = threadIdx.x & (L - 1), G = gstride() / L;
  for (uint32_t slot = gtid() / L;; slot += G) {
    if (__shfl_sync(0xffffffffu, slot, 0) >= slotEnd) break;  // warp-uniform exit
    bool act = slot < slotEnd;
    int32_t* w = b.state + (size_t)(act ? slot : 0u) * 8;
    const int2 mf = *reinterpret_cast<const int2*>(w + 4);
    const uint32_t mi = (uint32_t)mf.x, fl = (uint32_t)mf.y;
    act = act && (fl & (FLAG_ANCHOR | FLAG_RIGID));
    int32_t burstP = 0;
    if (act) {
      const ScenePar& S = b.scenes[b.sceneOf[slot]];
      act = S.active && slot - S.slotBase < S.nFluid;
      burstP = act ? matw(b, mi, M_burstP) : 0;
      act = act && seal_class(b, mi) && burstP > 0;
    }
    const uint32_t p = act ? b.inv[slot] : 0u;
    const int32_t px = act ? w[0] : 0, py = act ? w[1] : 0;
    const uint32_t cnt = act ? (b.NBRN[p] & NBRN_COUNT) : 0u;
    int32_t stress = 0;
    for (uint32_t k = sub; k < cnt; k += L) {
      const uint32_t e = b.NBR[(size_t)k * stride + p];
      if (e & NBR_BOUNDARY) continue;
      const int32_t* wj = b.state + (size_t)b.sslot[e] * 8;
      const uint32_t mj = (uint32_t)wj[4];
      if (seal_class(b, mj) || matw(b, mj, M_phantom) != 0) continue;
      const int32_t dx4 = shr_rne<BPRE>(sub_sat(px, wj[0], f)), dy4 = shr_rne<BPRE>(sub_sat(py, wj[1], f));
      const int32_t d2 = wadd(wmul(dx4, dx4), wmul(dy4, dy4));
      if (d2 >= SEAL_STRESS4 * SEAL_STRESS4) continue;
      stress = wadd(stress, SEAL_STRESS4 - (int32_t)isqrt32((uint32_t)d2));
    }
    if (L > 1) stress = gsum<L>(stress);
    if (act && sub == 0 && (int32_t)((uint32_t)stress << BPRE) > burstP)
      w[5] = (int32_t)((fl & ~(FLAG_ANCHOR | FLAG_RIGID | WELD_TAG_MASK)) | FLAG_BURST);
  }
}

// thermal (src/sim.wgsl:2612-2707) for one particle; updates words 4..7.
template <bool DBG>
__device__ __forceinline__ void thermal(const Bufs& b, uint32_t i, int32_t heat, int32_t corr, int32_t* w,
                                        const Flags<DBG>& f) {
  uint32_t mat0 = (uint32_t)w[4];
  int32_t T = add_sat(w[6], shr_rne<8>(heat), f);
  T = add_sat(T, mul<16>(sub_sat(AMBIENT, T, f), matw(b, mat0, M_coolRate), f), f);
  int32_t fuel = w[7];
  uint32_t fl0 = (uint32_t)w[5];
  bool burning = (fl0 & FLAG_BURNING) != 0;
  if (!burning && fuel > 0 && T >= matw(b, mat0, M_ignitePt)) burning = true;
  if (burning) {
    T = add_sat(T, matw(b, mat0, M_burnHeat), f);
    fuel = max(0, sub_sat(fuel, matw(b, mat0, M_burnRate), f));
  }
  T = clampi(T, TEMP_MIN, TEMP_MAX);
  T = add_sat(T, mul<16>(sub_sat(matw(b, mat0, M_tempTarget), T, f), matw(b, mat0, M_tempDrive), f), f);
  int32_t dose = shr_rne<8>(corr);
  uint32_t mat = mat0;
  bool froze = false;
  uint32_t sTo = (uint32_t)matw(b, mat0, M_splitTo), sPct = (uint32_t)matw(b, mat0, M_splitPct);
  if (burning && fuel <= 0) mat = pick_product((uint32_t)matw(b, mat0, M_burnTo), sTo, sPct, i);
  else if (dose >= matw(b, mat0, M_corrPt)) mat = pick_product((uint32_t)matw(b, mat0, M_corrTo), sTo, sPct, i);
  else if (T >= matw(b, mat0, M_boilPt)) mat = pick_product((uint32_t)matw(b, mat0, M_boilTo), sTo, sPct, i);
  else if (T >= matw(b, mat0, M_meltPt)) mat = pick_product((uint32_t)matw(b, mat0, M_meltTo), sTo, sPct, i);
  else if (T <= matw(b, mat0, M_condPt)) mat = pick_product((uint32_t)matw(b, mat0, M_condTo), sTo, sPct, i);
  else if (T <= matw(b, mat0, M_freezePt)) {
    mat = pick_product((uint32_t)matw(b, mat0, M_freezeTo), sTo, sPct, i);
    froze = true;
  }
  if (mat != mat0) { fuel = matw(b, mat, M_fuel0); burning = false; }
  uint32_t fl = fl0 & ~(FLAG_BURNING | FLAG_DEAD | FLAG_SEAL);
  if (mat != mat0) fl &= ~(FLAG_ANCHOR | FLAG_CONGEAL | FLAG_BURST);
  if (froze && mat != mat0 && fuse_row(b, mat)) fl |= FLAG_CONGEAL;
  if (burning) fl |= FLAG_BURNING;
  if (matw(b, mat, M_phantom) != 0) fl |= FLAG_DEAD;
  if (seal_class(b, mat)) fl |= FLAG_SEAL;
  w[4] = (int32_t)mat;
  w[5] = (int32_t)fl;
  w[6] = T;
  w[7] = fuel;
}

// surfaceTension (src/sim.wgsl:2409-2494) + thermal + the formation pass's
// flag update for rows that cannot bond (bondForm2's tail, src/sim.wgsl:
// 3059-3067) + the state digest. HASH=false when bond formation runs as its
// own kernels (the digest then follows them).
template <bool DBG, bool HASH, int L>
__global__ void __launch_bounds__(256, 5) k_post2(Bufs b, int formFlags) {
  Flags<DBG> f{b.dbg};
  __shared__ int4 smat[MAT_MAX];  // {gammaCoh, gammaCur, adhesion, 0}
  for (int m = threadIdx.x; m < MAT_MAX; m += blockDim.x)
    smat[m] = make_int4(matw(b, m, M_gammaCoh), matw(b, m, M_gammaCur), matw(b, m, M_adhesion), 0);
  __syncthreads();
  __shared__ uint32_t dsacc[8], dsscene;
  if (HASH) digest_block_begin(dsacc, &dsscene);
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  const uint32_t sub = threadIdx.x & (L - 1), G = gstride() / L;
  for (uint32_t p = gtid() / L;; p += G) {
    if (__shfl_sync(0xffffffffu, p, 0) >= nAct) break;  // warp-uniform exit
    const bool valid = p < nAct;
    const int4 me = valid ? b.PL[p] : make_int4(0, 0, 0, (int32_t)INFO_BOUNDARY);
    const uint32_t info = (uint32_t)me.w;
    const bool act = valid && !(info & INFO_BOUNDARY);
    const uint32_t pp = act ? p : 0u;
    const int4 mi = smat[info & INFO_MAT];
    const int2 pi = xy(me);
    const int4 nqi = b.NQ[pp];
    const int32_t rhoi = nqi.z;
    const uint32_t cnt = act ? (b.NBRN[p] & NBRN_COUNT) : 0u;
    int32_t ax = 0, ay = 0;
    const uint32_t* np = b.NBR + pp;
    // the neighbour's record and normal/density one ahead, its index two ahead
    uint32_t en = sub < cnt ? np[(size_t)sub * stride] : 0u;
    int4 on = b.PL[en & ~NBR_BOUNDARY];
    int4 nn = b.NQ[en & ~NBR_BOUNDARY];
    uint32_t en2 = sub + L < cnt ? np[(size_t)(sub + L) * stride] : 0u;
    for (uint32_t k = sub; k < cnt; k += L) {
      const uint32_t e = en;
      const int4 o = on;
      const int4 nq = nn;
      if (k + L < cnt) {
        en = en2;
        on = b.PL[en & ~NBR_BOUNDARY];
        nn = b.NQ[en & ~NBR_BOUNDARY];
      }
      if (k + 2 * L < cnt) en2 = np[(size_t)(k + 2 * L) * stride];
      // a rigid member's cohesion skips its own body (src/sim.wgsl:2450-2457)
      if ((info & INFO_RIGID) && !(e & NBR_BOUNDARY) && same_body(info, (uint32_t)o.w)) continue;
      const int2 d = pdelta(pi, xy(o), f);
      const int id = lut_index(d, f);
      if (id < 0) continue;
      const int2 ca = __ldg(b.CA + id);
      if (e & NBR_BOUNDARY) {
        ax = wsub(ax, mulfc<8>(mulf<22>(ca.y, d.x, f), mi.z, -ST_TERM, ST_TERM, f));
        ay = wsub(ay, mulfc<8>(mulf<22>(ca.y, d.y, f), mi.z, -ST_TERM, ST_TERM, f));
        continue;
      }
      const int32_t K = sym_k(rhoi, nq.z, b.rcp, f);
      const int4 mj = smat[(uint32_t)o.w & INFO_MAT];
      const int32_t gCoh = mat_mix(mi.x, mj.x);
      const int32_t gCur = mat_mix(mi.y, mj.y);
      int32_t fx = neg_sat(mulf<16>(mulf<22>(ca.x, d.x, f), gCoh, f), f);
      int32_t fy = neg_sat(mulf<16>(mulf<22>(ca.x, d.y, f), gCoh, f), f);
      const int32_t cx = mulf<16>(sub_sat(nqi.x, nq.x, f), gCur, f);
      const int32_t cy = mulf<16>(sub_sat(nqi.y, nq.y, f), gCur, f);
      fx = add_sat(fx, neg_sat(cx, f), f);
      fy = add_sat(fy, neg_sat(cy, f), f);
      ax = wadd(ax, mulc<8>(fx, K, -ST_TERM, ST_TERM, f));
      ay = wadd(ay, mulc<8>(fy, K, -ST_TERM, ST_TERM, f));
    }
    if (L > 1) {
      ax = gsum<L>(ax);
      ay = gsum<L>(ay);
    }
    const bool lead = valid && sub == 0;
    uint32_t scene = 0, idx = 0;
    int32_t w8[8];
    if (lead) {
      const uint32_t slot = b.sslot[p];
      scene = b.SCN[p];
      const ScenePar& S = b.scenes[scene];
      idx = slot - S.slotBase;
      int32_t* w = b.state + (size_t)slot * 8;
      if (act) {
        b.stacc[slot] = make_int2(shr_rne<8>(ax), shr_rne<8>(ay));
        thermal(b, idx, b.HEAT[p], b.CORR[p], w, f);
        if (formFlags && S.formNow) {
          uint32_t fo = (uint32_t)w[5] & ~FLAG_CONGEAL;
          if (!(fo & FLAG_RIGID) && (fo & WELD_TAG_MASK) != S.weldHold) fo &= ~WELD_TAG_MASK;
          w[5] = (int32_t)fo;
        }
      }
      if (HASH) {
        int4 a = reinterpret_cast<const int4*>(w)[0], c = reinterpret_cast<const int4*>(w)[1];
        w8[0] = a.x; w8[1] = a.y; w8[2] = a.z; w8[3] = a.w;
        w8[4] = c.x; w8[5] = c.y; w8[6] = c.z; w8[7] = c.w;
      }
    }
    if (HASH) {
      uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (lead) particle_digest(w8, idx, nullptr, h);
      digest_add_block(b.acc, dsacc, &dsscene, lead, scene, h);
    }
  }
  if (HASH) digest_block_end(b.acc, dsacc, &dsscene);
}

// Digest of the current state of every active scene, in slot order
// (statehash.wgsl `digest`, src/hash/statehash.wgsl:83-159).
__global__ void __launch_bounds__(256) k_hash(Bufs b, uint32_t* __restrict__ acc) {
  __shared__ uint32_t dsacc[8], dsscene;
  digest_block_begin(dsacc, &dsscene);
  const uint32_t slotEnd = b.world->slotEnd;
  const uint32_t nIter = (slotEnd + gstride() - 1) / gstride() * gstride();
  for (uint32_t slot = gtid(); slot < nIter; slot += gstride()) {
    bool valid = false;
    uint32_t s = 0, i = 0;
    uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (slot < slotEnd) {
      s = b.sceneOf[slot];
      const ScenePar& S = b.scenes[s];
      i = slot - S.slotBase;
      valid = S.active && i < S.n;
      if (valid) {
        const uint32_t* row = (b.bond && i < S.nFluid) ? b.bond + (size_t)slot * BOND_CAP : nullptr;
        particle_digest(b.state + (size_t)slot * 8, i, row, h);
      }
    }
    digest_add_block(acc, dsacc, &dsscene, valid, s, h);
  }
  digest_block_end(acc, dsacc, &dsscene);
}

// fold_chain (src/hash/statehash.wgsl:164-170) per scene, then advance the
// formation clock exactly as `_encodeSubstep` does (src/engine.js:4145-4151).
__global__ void k_fold(Bufs b, int doChain) {
  uint32_t s = gtid();
  if (s >= b.world->numScenes) return;
  ScenePar& S = b.scenes[s];
  if (!S.active) return;
  if (doChain) {
    uint32_t a[8], next[8];
    for (int j = 0; j < 8; ++j) a[j] = b.acc[s * 8 + j];
    for (int j = 0; j < 8; ++j) next[j] = mm_step(b.chain[s * 8 + j], a[j] ^ rotl32(a[(j + 1) & 7], 7));
    for (int j = 0; j < 8; ++j) {
      b.chain[s * 8 + j] = next[j];
      b.accLast[s * 8 + j] = a[j];
      b.acc[s * 8 + j] = 0;
    }
  }
  if (S.formNow) S.bondDirty = 0;
  S.formClock += 1;
  S.substep += 1;
}

// markCongealNbr + bondForm1 (src/sim.wgsl:2714-2989), sorted space.
template <bool DBG>
__global__ void __launch_bounds__(256) k_form1(Bufs b) {
  if (b.work[5] == 0u) return;  // no scene forms bonds this substep
  Flags<DBG> f{b.dbg};
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  for (uint32_t p = gtid(); p < nAct; p += gstride()) {
    int4 me = b.PL[p];
    if ((uint32_t)me.w & INFO_BOUNDARY) continue;
    const ScenePar& S = b.scenes[b.SCN[p]];
    if (!S.formNow) continue;
    uint32_t slot = b.sslot[p];
    const int32_t* wi = b.state + (size_t)slot * 8;
    uint32_t* cand = b.bondCand + (size_t)slot * BOND_CAP;
    const uint32_t* brow = b.bond + (size_t)slot * BOND_CAP;
    const uint32_t flI = (uint32_t)wi[5], matI = (uint32_t)wi[4];
    // Rigid members and rows that do not bond propose nothing: their list is
    // empty. Candidate rows are dense (entries first, zeros after), so a row
    // whose first word is zero is already empty and is not rewritten.
    if ((flI & FLAG_RIGID) || matw(b, matI, M_bondK) == 0 || matw(b, matI, M_bondGroup) < 0) {
      if (cand[0] != 0u)
        for (int k = 0; k < BOND_CAP; ++k) cand[k] = 0;
      continue;
    }
    uint32_t cnt = b.NBRN[p] & NBRN_COUNT;
    // markCongealNbr: refresh the congeal bit from the post-thermal flags
    bool seen = false;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t e = b.NBR[(size_t)k * stride + p];
      if (e & NBR_BOUNDARY) continue;
      uint32_t qs = b.sslot[e];
      if ((uint32_t)b.state[(size_t)qs * 8 + 5] & FLAG_CONGEAL) { seen = true; break; }
    }
    bool anchoredI = (flI & FLAG_ANCHOR) != 0;
    uint32_t cn = 0;
    {
      for (int k = 0; k < BOND_CAP; ++k) {
        uint32_t w = brow[k];
        if (w == 0u) break;
        if (w & BOND_TOMB) continue;
        if (cn >= (uint32_t)BOND_CAP) { f.flag(8); break; }
        cand[cn++] = w;
      }
      uint32_t tagI = flI & WELD_TAG_MASK;
      int32_t ki = bond_k(b, matI, wi[6], f);
      bool canReform = (!anchoredI && matw(b, matI, M_bondReform) != 0 && ki != 0);
      bool fuseArmed = S.fuseTag != 0u && fuse_row(b, matI);
      bool congealI = (flI & FLAG_CONGEAL) && fuse_row(b, matI);
      bool congealNear = seen && fuse_row(b, matI);
      if (canReform || (!anchoredI && tagI != 0u) || fuseArmed || congealI || congealNear) {
        for (uint32_t k = 0; k < cnt; ++k) {
          if (cn >= (uint32_t)BOND_CAP) { f.flag(8); break; }
          uint32_t e = b.NBR[(size_t)k * stride + p];
          if (e & NBR_BOUNDARY) continue;
          uint32_t qs = b.sslot[e];
          const int32_t* wj = b.state + (size_t)qs * 8;
          uint32_t j = qs - S.slotBase;
          uint32_t mj = (uint32_t)wj[4];
          uint32_t fJ = (uint32_t)wj[5];
          uint32_t tagJ = fJ & WELD_TAG_MASK;
          bool weld = (!anchoredI && tagI != 0u && tagI == tagJ);
          bool fuse = false;
          if (fuseArmed && !(fJ & FLAG_RIGID) && fuse_row(b, mj) && (!anchoredI || !(fJ & FLAG_ANCHOR)))
            fuse = (tagI == S.fuseTag && tagJ == 0u) || (tagJ == S.fuseTag && tagI == 0u) ||
                   (tagI == S.fuseTag && tagJ == S.fuseTag);
          bool congealJ = (fJ & FLAG_CONGEAL) && fuse_row(b, mj);
          bool congeal = ((congealI || congealJ) && !weld && !fuse && mj == matI && !(fJ & FLAG_RIGID));
          if (!fuse && !congeal && matw(b, mj, M_bondGroup) != matw(b, matI, M_bondGroup)) continue;
          if (!weld && !fuse && !congeal) {
            if (!canReform) continue;
            if (bond_k(b, mj, wj[6], f) == 0) continue;
          }
          bool dup = false;
          for (uint32_t q2 = 0; q2 < cn; ++q2)
            if ((cand[q2] & BOND_J_MASK) == j) { dup = true; break; }
          if (dup) continue;
          int32_t d4x = shr_rne<BPRE>(sub_sat(wi[0], wj[0], f));
          int32_t d4y = shr_rne<BPRE>(sub_sat(wi[1], wj[1], f));
          if (abs(d4x) > L0_MAX || abs(d4y) > L0_MAX) continue;
          int32_t d2 = wadd(wmul(d4x, d4x), wmul(d4y, d4y));
          if (d2 < D2_FLOOR || d2 > BOND_R2) continue;
          if (!weld && !fuse && !congeal) {
            int32_t vl = min(matw(b, matI, M_bondFormV), matw(b, mj, M_bondFormV));
            int32_t vl4 = shr_rne<RPRE>(vl);
            int32_t r4x = shr_rne<RPRE>(sub_sat(wi[2], wj[2], f));
            int32_t r4y = shr_rne<RPRE>(sub_sat(wi[3], wj[3], f));
            if (abs(r4x) > vl4 || abs(r4y) > vl4) continue;
            if (wadd(wmul(r4x, r4x), wmul(r4y, r4y)) > wmul(vl4, vl4)) continue;
            int32_t pl = min(matw(b, matI, M_bondFormP), matw(b, mj, M_bondFormP));
            if (pl != 0 && (neg_sat(me.z, f) < pl || neg_sat(b.PL[e].z, f) < pl)) continue;
          }
          int32_t L0 = (int32_t)isqrt32((uint32_t)d2);
          if (L0 < L0_MIN || L0 > L0_MAX) continue;
          if (j > BOND_J_MASK) { atomicOr(b.err, ERR_BOND_PARTNER); continue; }
          cand[cn++] = (((uint32_t)L0 & 0x1fffu) << 17) | (j & BOND_J_MASK);
        }
      }
    }
    for (uint32_t k = cn; k < (uint32_t)BOND_CAP; ++k) cand[k] = 0;
  }
}

// bondForm2 (src/sim.wgsl:3001-3068): keep mutual proposals, clear weld
// tags. It is the last pass of the substep that writes hashed words, so with
// HASH it also folds every particle's digest (the state hash of the substep).
template <bool HASH>
__global__ void __launch_bounds__(256) k_form2(Bufs b, uint32_t* __restrict__ acc) {
  __shared__ uint32_t dsacc[8], dsscene;
  if (HASH) digest_block_begin(dsacc, &dsscene);
  // While no bond row of the world has ever been non-empty (work[4] clear),
  // the digest needs no row reads: an empty row folds nothing. A row this
  // launch forms is read by the thread that formed it.
  const bool rowsLive = b.work[4] != 0u;
  const uint32_t slotEnd = b.world->slotEnd;
  const uint32_t nIter = HASH ? (slotEnd + gstride() - 1) / gstride() * gstride() : slotEnd;
  for (uint32_t slot = gtid(); slot < nIter; slot += gstride()) {
    bool valid = false, formed = false;
    uint32_t s = 0;
    uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (slot < slotEnd) {
      s = b.sceneOf[slot];
      const ScenePar& S = b.scenes[s];
      const uint32_t i = slot - S.slotBase;
      uint32_t* row = b.bond + (size_t)slot * BOND_CAP;
      if (S.active && i < S.nFluid && S.formNow) {
        const uint32_t* cand = b.bondCand + (size_t)slot * BOND_CAP;
        uint32_t nn = 0;
        for (int k = 0; k < BOND_CAP; ++k) {
          uint32_t w = cand[k];
          if (w == 0u) break;
          uint32_t j = w & BOND_J_MASK;
          const uint32_t* cj = b.bondCand + (size_t)(S.slotBase + j) * BOND_CAP;
          bool ok = false;
          for (int q = 0; q < BOND_CAP; ++q) {
            uint32_t v = cj[q];
            if (v == 0u) break;
            if ((v & BOND_J_MASK) == i) { ok = ((v & BOND_L0_MASK) == (w & BOND_L0_MASK)); break; }
          }
          if (ok) row[nn++] = w & ~BOND_TOMB;
        }
        // bond rows are dense too: an empty row stays as it is
        if (nn != 0u || row[0] != 0u)
          for (int k = nn; k < BOND_CAP; ++k) row[k] = 0;
        if (nn != 0u) {
          formed = true;
          if (!rowsLive) b.work[4] = 1u;
        }
        int32_t* w = b.state + (size_t)slot * 8;
        uint32_t fo = (uint32_t)w[5] & ~FLAG_CONGEAL;
        if (!(fo & FLAG_RIGID) && (fo & WELD_TAG_MASK) != S.weldHold) fo &= ~WELD_TAG_MASK;
        w[5] = (int32_t)fo;
      }
      if (HASH) {
        valid = S.active && i < S.n;
        if (valid)
          particle_digest(b.state + (size_t)slot * 8, i, (i < S.nFluid && (rowsLive || formed)) ? row : nullptr, h);
      }
    }
    if (HASH) digest_add_block(acc, dsacc, &dsscene, valid, s, h);
  }
  if (HASH) digest_block_end(acc, dsacc, &dsscene);
}

}  // namespace d2
}  // namespace sn
