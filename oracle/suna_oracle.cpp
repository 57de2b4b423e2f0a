// ORACLE — test infrastructure only.
//
// A scalar CPU restatement of SunaEngine's deterministic Q16.16 PBF substep,
// used as the parity checker for the CUDA engine and as the timed CPU
// baseline. Only the test suite, the smoke check and the benchmark's CPU
// baseline leg load it; the product library never links or calls it.
//
// It follows the reference pass by pass, with the reference's own data layout
// (AoS particles, 16-word derived rows, MAXNBR-strided neighbour lists, the
// ping-pong state pair), so that it reads against the WGSL line by line:
//   src/fixed.wgsl                        -> fixed_ref.h
//   src/sim.wgsl  predict ... bondForm2   -> the pass functions below
//   src/hash/statehash.js                 -> digest(), fold_chain()
//   src/engine.js loadScene/_encodeSubstep/spawnFluid/applyImpulse
//
// Scope: the fluid, friction, bond, thermal and formation passes, containment
// (src/sim.wgsl section 29) and rigid bodies (section 20, with the host's body
// record math from src/engine.js:2050-2150 and 5452-5811).
//
// Parity is pinned by the reference's frozen dambreak_v1 chain
// (test/extraction_gate.md:62-68).
#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>
#include "fixed_ref.h"
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace ofx;

namespace {

// ---- world constants: src/sim.wgsl:55-113 ----------------------------------
constexpr int32_t H = 163840;
constexpr int32_t RHO0 = 1048576;
constexpr int32_t TWO_RHO0 = 2097152;
constexpr uint32_t PRE = 4;
constexpr int32_t HS = 10240;
constexpr int32_t H2S = 104857600;
constexpr uint32_t KSH = 15;
constexpr uint32_t GF = 22;
constexpr uint32_t CF = 22;
constexpr uint32_t ACC = 8;
constexpr uint32_t MAXNBR = 48;
constexpr uint32_t TN = 3202;
constexpr uint32_t OFF_W = 0, OFF_G = 3202, OFF_C = 6404, OFF_A = 9606, OFF_S = 12808;
constexpr int32_t LAM_MAX = 4194304, NEG_LAM_MAX = -4194304;
constexpr int32_t S_TERM = 16777216;
constexpr int32_t DP_TERM = 2097152, NEG_DP_TERM = -2097152;
constexpr int32_t XS_TERM = 2097152, NEG_XS_TERM = -2097152;
constexpr int32_t ST_TERM = 4194304, NEG_ST_TERM = -4194304;
constexpr int32_t RINV_MAX = 262144;
constexpr int32_t WALL = 32768;
constexpr int32_t CUR_SIGN = -1;
constexpr int32_t C_MAX = 58000;
constexpr int32_t RHO_FLOOR_RINV = 32768;
constexpr int32_t RHO_FLOOR_K = 65536;
constexpr int32_t AMBIENT = 1310720;
constexpr int32_t TEMP_MIN = -33554432, TEMP_MAX = 536870912;
constexpr int32_t DT_CLAMP = 16777216, NEG_DT_CLAMP = -16777216;
constexpr int32_t HT_TERM = 16777216, NEG_HT_TERM = -16777216;
constexpr int32_t CORR_TERM = 16777216;
constexpr int32_t CORR_NEVER = 2147483647;
constexpr uint32_t FLAG_BURNING = 1, FLAG_DEAD = 2, FLAG_ANCHOR = 4, FLAG_RIGID = 16;
constexpr uint32_t FLAG_CONGEAL = 32, FLAG_BURST = 64, FLAG_SEAL = 128;
constexpr uint32_t WELD_TAG_MASK = 0x000fff00u;
constexpr uint32_t NBR_SEAL_BIT = 0x80000000u, NBR_EXT_SEAL_BIT = 0x40000000u, NBR_CONGEAL_BIT = 0x20000000u;
// friction / bonds: src/sim.wgsl:1569-1640
constexpr uint32_t FPRE = 5, RPRE = 3, BPRE = 5;
constexpr int32_t D2_FLOOR = 262144;
constexpr int32_t FR_TERM = 16777216, NEG_FR_TERM = -16777216;
constexpr uint32_t BOND_CAP = 48;
constexpr int32_t BOND_R2 = 17623204;
constexpr int32_t HARD_BREAK2 = 26214400;
constexpr int32_t L0_MAX = 5120, L0_MIN = 512;
constexpr uint32_t BOND_J_MASK = 0x0001ffffu, BOND_L0_SH = 17, BOND_L0_MASK = 0x3ffe0000u, BOND_TOMB = 0x40000000u;
constexpr int32_t BD_TERM = 16777216, NEG_BD_TERM = -16777216;
constexpr uint32_t MAT_PHOTO_ROW = 15;
constexpr uint32_t BOND_PERIOD = 4;
constexpr int32_t VMAX = 65536;
constexpr uint32_t MAT_WORDS = 48;
constexpr uint32_t MAT_MAX = 64;

// Mat word indices: src/sim.wgsl:315-431 / src/engine.js:678-705
enum MatW {
  M_eps, M_dpMax, M_xsph, M_phantom, M_gammaCoh, M_gammaCur, M_adhesion, M_grav,
  M_cond, M_coolRate, M_heatCap, M_meltPt, M_meltTo, M_freezePt, M_freezeTo, M_boilPt, M_boilTo,
  M_condPt, M_condTo, M_ignitePt, M_fuel0, M_burnRate, M_burnHeat, M_burnTo, M_splitTo, M_splitPct,
  M_spawnTemp, M_tint, M_corrode, M_corrPt, M_corrTo, M_fric, M_bondK, M_bondBreak, M_bondReform,
  M_bondFormV, M_bondFormP, M_bondMu, M_bondGroup, M_rampLo, M_rampHi, M_rampInv, M_rampSign,
  M_solidMode, M_tempTarget, M_tempDrive, M_burstP, M_sealMode
};

struct Particle { int32_t px, py, vx, vy; uint32_t matId, flags; int32_t temp, fuel; };
struct Derived {
  int32_t predx, predy, dpx, dpy, vtmpx, vtmpy, nrmx, nrmy, stx, sty, rho, lam, rinv, heat, corr;
  uint32_t pad1;
};
static_assert(sizeof(Particle) == 32, "particle layout");
static_assert(sizeof(Derived) == 64, "derived layout");

struct V2 { int32_t x, y; };

}  // namespace

struct SnoEngine {
  uint32_t maxParticles = 0, iters = 4;
  int32_t luts[5 * 3202];
  int32_t mats[MAT_MAX][MAT_WORDS];      // the table the passes read (grav scaled)
  int32_t matsAuth[MAT_MAX][MAT_WORDS];  // rows as authored or minted
  uint32_t matCount = 0, authoredCount = 0;
  int32_t gravQ = 65536;                 // setGravityScale (src/engine.js:4843), Q16
  int threads = 1;
  bool nbrCut = false;  // stop a full list's scan when no flag can change (pass_buildNbr)
  // params
  uint32_t n = 0, nFluid = 0, gridW = 1, gridH = 1, cellTotal = 1, cellShift = 18;
  int32_t originX = 0, originY = 0, domW = 0, domH = 0, vmax = VMAX;
  uint32_t weldHold = 0, fuseTag = 0;
  uint32_t weldSeq = 1, weldHoldSeq = 0, lastWeldTag = 0;  // weld-group host state (src/engine.js:4570-4680)
  // buffers
  std::vector<Particle> st[2];
  std::vector<Derived> der;
  std::vector<uint32_t> cellCount, cellStart, cellOf, sortedIds, nbr, nbrN, bond, bondCand;
  uint32_t dbg[16];
  // Per-thread counters, merged into dbg at the end of every substep and
  // before any read: a counter that fires on many pairs would otherwise be an
  // atomic on one shared line for every thread. Counts are order-free sums.
  static constexpr int DBG_THREADS = 256;
  alignas(64) uint32_t dbgT[DBG_THREADS][16] = {};
  void merge_dbg() {
    for (int t = 0; t < DBG_THREADS; ++t)
      for (int k = 0; k < 16; ++k) {
        dbg[k] += dbgT[t][k];
        dbgT[t][k] = 0;
      }
  }
  uint32_t chain[8];
  uint32_t acc[8];
  int parity = 0;
  uint64_t substepCount = 0;
  uint64_t formationClock = 0;  // engine `_substep`
  bool bondDirty = true;
  bool wallsOn = true;
  uint32_t unsupported = 0;     // nonzero: a transition produced a row this oracle does not restate
  // §23.B jets (setJets, src/engine.js:4740-4770): [x, y, r, fx, fy] ticks
  int32_t jets[8][5] = {};
  uint32_t nJets = 0;
  // §20 rigid bodies (src/sim.wgsl:670-821): body records in the reference's
  // 32-word layout, the 10-word driver sidecars, rest offsets per slot, the
  // Q22 quarter-turn cosine table, and the host's body list (`_bodies`).
  struct BodyDesc {
    uint32_t tag = 0, first = 0, last = 0, n = 0;
    bool axis = false, user = false;
  };
  std::vector<int32_t> rbody, rdrive, rest;
  std::vector<BodyDesc> bodies;
  int32_t cosT[1026];
  int32_t userA[2] = {0, 0};
  // the loaded scene's boundary block, for spawnFluid's relocation
  std::vector<int32_t> scenePos, sceneTemp, sceneFuel;
  std::vector<uint32_t> sceneMat;
  uint32_t sceneNFluid = 0;
  bool sceneHasTemp = false, sceneHasFuel = false;

  Dbg D() {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
    return Dbg{t < DBG_THREADS ? dbgT[t] : dbg};
#else
    return Dbg{dbgT[0]};
#endif
  }
  const int32_t* M(uint32_t m) const { return mats[m]; }
};

namespace {

using E = SnoEngine;

inline bool seal_class_row(const int32_t* m) {
  return m[M_bondK] != 0 && m[M_bondReform] == 0 && m[M_solidMode] != 0 && m[M_phantom] == 0;
}
inline bool spawn_welds(const int32_t* m) { return m[M_bondGroup] >= 0 && m[M_bondReform] == 0; }
// Rows whose passes this oracle does not restate: rigid bodies (§20).
constexpr int32_t SOLID_RIGID = 2;
inline bool rigid_row(const int32_t* m) { return m[M_solidMode] == SOLID_RIGID; }
inline bool seal_liquid_row(const int32_t* m) {
  return m[M_bondK] == 0 && m[M_fric] == 0 && m[M_grav] > 0 && m[M_phantom] == 0;
}
inline bool fuse_row(const int32_t* m, uint32_t id) {
  return m[M_bondK] != 0 && m[M_bondReform] == 0 && m[M_bondGroup] >= 0 && id != MAT_PHOTO_ROW;
}

// src/sim.wgsl:477-482 (whitelisted floor shift)
inline V2 cell_coord(const E& e, V2 p) {
  int32_t cx = wsub(p.x, e.originX) >> e.cellShift;
  int32_t cy = wsub(p.y, e.originY) >> e.cellShift;
  return V2{clampi(cx, 0, (int32_t)e.gridW - 1), clampi(cy, 0, (int32_t)e.gridH - 1)};
}
inline uint32_t cell_index(const E& e, V2 c) { return (uint32_t)c.y * e.gridW + (uint32_t)c.x; }
inline uint32_t cell_colour(const E& e, uint32_t i) {
  uint32_t c = e.cellOf[i];
  uint32_t cx = c % e.gridW, cy = c / e.gridW;
  return (cx & 1u) | ((cy & 1u) << 1);
}
// src/sim.wgsl:520-527
inline int32_t lut_index(V2 d, const Dbg& g) {
  int32_t ax = wadd(fp_abs(d.x, g), 8) >> PRE;
  int32_t ay = wadd(fp_abs(d.y, g), 8) >> PRE;
  if (ax > HS || ay > HS) return -1;
  int32_t r2 = wadd(wmul(ax, ax), wmul(ay, ay));
  if (r2 >= H2S) return -1;
  return r2 >> KSH;
}
inline int32_t grad_q16(int32_t gt, int32_t d, const Dbg& g) { return fp_mul_s(gt, d, GF + 4u, g); }
inline bool is_boundary(const E& e, uint32_t j) { return j >= e.nFluid; }
inline uint32_t nbr_count(const E& e, uint32_t i) {
  return e.nbrN[i] & ~(NBR_SEAL_BIT | NBR_EXT_SEAL_BIT | NBR_CONGEAL_BIT);
}
inline V2 pred_of(const E& e, uint32_t j) { return V2{e.der[j].predx, e.der[j].predy}; }
inline V2 pred_delta(const E& e, V2 pi, uint32_t j, const Dbg& g) {
  V2 pj = pred_of(e, j);
  return V2{fp_sub_sat(pi.x, pj.x, g), fp_sub_sat(pi.y, pj.y, g)};
}
inline V2 wall_clamp(const E& e, V2 p) {
  return V2{clampi(p.x, WALL, e.domW - WALL), clampi(p.y, WALL, e.domH - WALL)};
}
inline int32_t mat_mix(int32_t a, int32_t b) { return wadd(a, b) >> 1; }
inline int32_t sym_k(int32_t rhoi, int32_t rhoj, const Dbg& g) {
  int32_t den = std::max(RHO_FLOOR_K, fp_add_sat(rhoi, rhoj, g));
  return clampi(fp_divshift(TWO_RHO0, den, 16u, g), 0, RINV_MAX);
}
// src/sim.wgsl:579-594
inline uint32_t id_hash(uint32_t i) {
  uint32_t x = i + 0x9e3779b9u;
  x = (x ^ (x >> 16)) * 0x21f0aaadu;
  x = (x ^ (x >> 15)) * 0x735a2d97u;
  return x ^ (x >> 15);
}
inline uint32_t pick_product(uint32_t primary, uint32_t splitTo, uint32_t splitPct, uint32_t i) {
  if (splitPct == 0u) return primary;
  if ((id_hash(i) & 255u) < splitPct) return splitTo;
  return primary;
}
inline uint32_t weld_tag(uint32_t f) { return f & WELD_TAG_MASK; }
inline bool rg_same_body(uint32_t fi, uint32_t fj) {
  return (fi & FLAG_RIGID) && (fj & FLAG_RIGID) && weld_tag(fi) == weld_tag(fj) && weld_tag(fi) != 0u;
}
// src/sim.wgsl:1663-1671
inline int32_t bond_k(const int32_t* m, int32_t T, const Dbg& g) {
  if (m[M_bondK] == 0) return 0;
  if (m[M_rampSign] == 0) return m[M_bondK];
  int32_t span = fp_sub_sat(m[M_rampHi], m[M_rampLo], g);
  int32_t dT = clampi(fp_sub_sat(T, m[M_rampLo], g), 0, span);
  int32_t u = clampi(fp_mul_s(dT, m[M_rampInv], 16u, g), 0, 65536);
  if (m[M_rampSign] < 0) u = 65536 - u;
  return fp_mul_s(m[M_bondK], u, 16u, g);
}
inline uint32_t bond_j(uint32_t w) { return w & BOND_J_MASK; }
inline int32_t bond_l0(uint32_t w) { return (int32_t)((w >> BOND_L0_SH) & 0x1fffu); }
inline uint32_t bond_pack(uint32_t j, int32_t l0) { return (((uint32_t)l0 & 0x1fffu) << BOND_L0_SH) | (j & BOND_J_MASK); }
inline int32_t iabs(int32_t x) { return x < 0 ? (int32_t)(0u - (uint32_t)x) : x; }  // WGSL abs wraps

#ifdef _OPENMP
#define PFOR _Pragma("omp parallel for schedule(static) num_threads(e.threads)")
#else
#define PFOR
#endif

// ---- passes ------------------------------------------------------------------

// src/sim.wgsl:958-1000
// _nextWeldSeq (src/engine.js:4570-4580): the next tag sequence that is neither
// held open nor worn by a body of the host's body list.
inline bool weld_seq_taken(const E& e, uint32_t q) {
  if (q == e.weldHoldSeq) return true;
  for (const auto& b : e.bodies)
    if ((b.tag >> 8) == q) return true;
  return false;
}
inline uint32_t next_weld_seq(E& e) {
  const uint32_t MAXS = 4095;
  uint32_t q = (e.weldSeq % MAXS) + 1;
  for (uint32_t guard = 0; guard <= MAXS && weld_seq_taken(e, q); ++guard) q = (q % MAXS) + 1;
  e.weldSeq = q;
  return q;
}

// jet_accel (src/sim.wgsl:935-949): the sum of the accelerations of the jets
// whose disc holds p; saturating, so overlapping jets never flip sign.
constexpr uint32_t JET_SH = 9;
inline V2 jet_accel(const E& e, int32_t px, int32_t py, const Dbg& g) {
  V2 a{0, 0};
  for (uint32_t k = 0; k < e.nJets; ++k) {
    const int32_t* j = e.jets[k];
    const int32_t dx = fp_sub_sat(px, j[0], g) >> JET_SH, dy = fp_sub_sat(py, j[1], g) >> JET_SH;
    const int32_t rr = j[2] >> JET_SH;
    if (wadd(wmul(dx, dx), wmul(dy, dy)) <= wmul(rr, rr)) {
      a.x = fp_add_sat(a.x, j[3], g);
      a.y = fp_add_sat(a.y, j[4], g);
    }
  }
  return a;
}

void pass_predict(E& e, const std::vector<Particle>& in) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    const Particle& p = in[i];
    const int32_t* Mt = e.M(p.matId);
    Derived& d = e.der[i];
    if (Mt[M_phantom] != 0) { d.predx = p.px; d.predy = p.py; continue; }
    if (p.flags & FLAG_ANCHOR) { d.predx = p.px; d.predy = p.py; continue; }
    if (p.flags & FLAG_RIGID) continue;
    int32_t vmaxN = fp_neg_sat(e.vmax, g);
    const V2 jf = jet_accel(e, p.px, p.py, g);
    int32_t vx = fp_add_sat(fp_add_sat(p.vx, d.stx, g), jf.x, g);
    int32_t vy = fp_add_sat(fp_add_sat(fp_add_sat(p.vy, d.sty, g), Mt[M_grav], g), jf.y, g);
    vx = clampi(vx, vmaxN, e.vmax);
    vy = clampi(vy, vmaxN, e.vmax);
    V2 pr{fp_add_sat(p.px, vx, g), fp_add_sat(p.py, vy, g)};
    V2 w = wall_clamp(e, pr);
    d.predx = w.x; d.predy = w.y;
  }
}

// gridCount + scanBlock/Top/Add + scatter + canonicalize, src/sim.wgsl:1009-1168.
// The result is what canonicalize produces: cells in index order, occupants
// in ascending id order.
void pass_grid(E& e) {
  std::fill(e.cellCount.begin(), e.cellCount.begin() + e.cellTotal, 0u);
  for (uint32_t i = 0; i < e.n; ++i) {
    uint32_t c = cell_index(e, cell_coord(e, pred_of(e, i)));
    e.cellOf[i] = c;
    e.cellCount[c]++;
  }
  uint32_t run = 0;
  for (uint32_t c = 0; c < e.cellTotal; ++c) { e.cellStart[c] = run; run += e.cellCount[c]; }
  e.cellStart[e.cellTotal] = e.n;
  std::fill(e.cellCount.begin(), e.cellCount.begin() + e.cellTotal, 0u);
  for (uint32_t i = 0; i < e.n; ++i) {  // ascending id == canonical order
    uint32_t c = e.cellOf[i];
    e.sortedIds[e.cellStart[c] + e.cellCount[c]++] = i;
  }
}

// src/sim.wgsl:1190-1254. With e.nbrCut set (sno_set_nbr_cut) the scan of a
// particle's cells stops once its list holds MAXNBR entries, when no live fluid
// particle carries FLAG_SEAL or FLAG_CONGEAL: every later candidate could only
// be truncated away, so the list, its count and its flag bits are what the full
// scan gives; only the overflow counter (debug flag 6) stops counting. The full
// scan is O(occupancy^2) in a crowded cell.
void pass_buildNbr(E& e, const std::vector<Particle>& in) {
  bool flagsLive = false;
  for (uint32_t j = 0; j < e.nFluid && !flagsLive; ++j)
    flagsLive = !(in[j].flags & FLAG_DEAD) && (in[j].flags & (FLAG_SEAL | FLAG_CONGEAL));
  const bool cut = e.nbrCut && !flagsLive;
  PFOR for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    if (in[i].flags & FLAG_DEAD) { e.nbrN[i] = 0; continue; }
    V2 pi = pred_of(e, i);
    V2 cc = cell_coord(e, pi);
    uint32_t base = i * MAXNBR;
    uint32_t cnt = 0;
    bool sealSeen = false, extSeen = false, congealSeen = false;
    for (int32_t dy = -1; dy <= 1; ++dy) {
      int32_t gy = cc.y + dy;
      if (gy < 0 || gy >= (int32_t)e.gridH) continue;
      for (int32_t dx = -1; dx <= 1; ++dx) {
        int32_t gx = cc.x + dx;
        if (gx < 0 || gx >= (int32_t)e.gridW) continue;
        uint32_t c = (uint32_t)gy * e.gridW + (uint32_t)gx;
        for (uint32_t s = e.cellStart[c]; s < e.cellStart[c + 1]; ++s) {
          uint32_t j = e.sortedIds[s];
          if (j == i) continue;
          if (in[j].flags & FLAG_DEAD) continue;
          if (lut_index(pred_delta(e, pi, j, g), g) < 0) continue;
          if (j < e.nFluid && (in[j].flags & FLAG_SEAL)) {
            sealSeen = true;
            if ((in[i].flags & FLAG_RIGID) && (in[j].flags & FLAG_ANCHOR) && !rg_same_body(in[i].flags, in[j].flags))
              extSeen = true;
          }
          if (j < e.nFluid && (in[j].flags & FLAG_CONGEAL)) congealSeen = true;
          if (cnt >= MAXNBR) { g.flag(6); continue; }
          e.nbr[base + cnt] = j;
          cnt++;
          if (cut && cnt >= MAXNBR) goto listed;
        }
      }
    }
  listed:
    e.nbrN[i] = cnt | (sealSeen ? NBR_SEAL_BIT : 0u) | (extSeen ? NBR_EXT_SEAL_BIT : 0u) |
                (congealSeen ? NBR_CONGEAL_BIT : 0u);
  }
}

// src/sim.wgsl:1270-1318
void pass_solveA(E& e, const std::vector<Particle>& in) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    const int32_t* Mt = e.M(in[i].matId);
    V2 pi = pred_of(e, i);
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    int32_t rho = e.luts[OFF_W], S = 0, sgx = 0, sgy = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      V2 d = pred_delta(e, pi, j, g);
      int32_t id = lut_index(d, g);
      if (id < 0) continue;
      uint32_t ui = (uint32_t)id;
      rho = wadd(rho, e.luts[OFF_W + ui]);
      int32_t gt = e.luts[OFF_G + ui];
      int32_t gx = grad_q16(gt, d.x, g), gy = grad_q16(gt, d.y, g);
      sgx = wadd(sgx, gx);
      sgy = wadd(sgy, gy);
      S = wadd(S, wadd(clampi(fp_mul_s(gx, gx, 11u, g), 0, S_TERM), clampi(fp_mul_s(gy, gy, 11u, g), 0, S_TERM)));
    }
    S = wadd(S, wadd(clampi(fp_mul_s(sgx, sgx, 11u, g), 0, S_TERM), clampi(fp_mul_s(sgy, sgy, 11u, g), 0, S_TERM)));
    int32_t Cq = clampi(fp_shr_rne(wsub(rho, RHO0), 4u), 0, C_MAX);
    e.der[i].rho = rho;
    e.der[i].lam = clampi(fp_neg_sat(fp_divshift(Cq, wadd(S, Mt[M_eps]), 25u, g), g), NEG_LAM_MAX, LAM_MAX);
  }
}

// src/sim.wgsl:1337-1407
void pass_solveB(E& e, const std::vector<Particle>& in, uint32_t colour) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    if (cell_colour(e, i) != colour) continue;
    Dbg g = e.D();
    V2 pi = pred_of(e, i);
    int32_t li = e.der[i].lam;
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    uint32_t fi = in[i].flags;
    bool rigidI = (fi & FLAG_RIGID) != 0;
    int32_t dpx = 0, dpy = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      if (rigidI && !is_boundary(e, j) && rg_same_body(fi, in[j].flags)) continue;
      V2 d = pred_delta(e, pi, j, g);
      int32_t id = lut_index(d, g);
      if (id < 0) continue;
      uint32_t ui = (uint32_t)id;
      int32_t lj = is_boundary(e, j) ? li : e.der[j].lam;
      int32_t co = fp_add_sat(fp_add_sat(li, lj, g), e.luts[OFF_S + ui], g);
      int32_t gt = e.luts[OFF_G + ui];
      dpx = wadd(dpx, clampi(fp_mul_s(co, grad_q16(gt, d.x, g), 20u - ACC, g), NEG_DP_TERM, DP_TERM));
      dpy = wadd(dpy, clampi(fp_mul_s(co, grad_q16(gt, d.y, g), 20u - ACC, g), NEG_DP_TERM, DP_TERM));
    }
    e.der[i].dpx = dpx;
    e.der[i].dpy = dpy;
  }
}

// src/sim.wgsl:1418-1434 (applyDp_at)
inline void applyDp_at(E& e, const std::vector<Particle>& in, uint32_t i, const Dbg& g) {
  if (in[i].flags & FLAG_RIGID) return;
  if (in[i].flags & FLAG_ANCHOR) return;
  const int32_t* Mt = e.M(in[i].matId);
  int32_t dm = Mt[M_dpMax], dmN = fp_neg_sat(dm, g);
  Derived& d = e.der[i];
  V2 dd{clampi(fp_shr_rne(d.dpx, ACC), dmN, dm), clampi(fp_shr_rne(d.dpy, ACC), dmN, dm)};
  V2 np{fp_add_sat(d.predx, dd.x, g), fp_add_sat(d.predy, dd.y, g)};
  V2 w = wall_clamp(e, np);
  d.predx = w.x; d.predy = w.y;
}

void pass_applyDp(E& e, const std::vector<Particle>& in, int colour /* -1: applyFric */) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    if (colour >= 0 && cell_colour(e, i) != (uint32_t)colour) continue;
    Dbg g = e.D();
    applyDp_at(e, in, i, g);
  }
}

// src/sim.wgsl:1673-1934 (friction + the section-18 bond gather)
void pass_friction(E& e, const std::vector<Particle>& in) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    const int32_t* Mi = e.M(in[i].matId);
    int32_t fi = Mi[M_fric];
    uint32_t flagsI = in[i].flags;
    bool rigidI = (flagsI & FLAG_RIGID) != 0;
    Derived& di = e.der[i];
    if (fi == 0 && Mi[M_bondK] == 0) {
      if (!rigidI) { di.dpx = 0; di.dpy = 0; }
      continue;
    }
    V2 pi = pred_of(e, i);
    V2 dxi{fp_sub_sat(pi.x, in[i].px, g), fp_sub_sat(pi.y, in[i].py, g)};
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    int32_t fx = 0, fy = 0;
    if (fi != 0) {
      for (uint32_t k = 0; k < cnt; ++k) {
        uint32_t j = e.nbr[base + k];
        if (rigidI && !is_boundary(e, j) && rg_same_body(flagsI, in[j].flags)) continue;
        V2 d = pred_delta(e, pi, j, g);
        int32_t id = lut_index(d, g);
        if (id < 0) continue;
        uint32_t ui = (uint32_t)id;
        int32_t d4x = fp_shr_rne(d.x, FPRE), d4y = fp_shr_rne(d.y, FPRE);
        int32_t d2 = wadd(wmul(d4x, d4x), wmul(d4y, d4y));
        if (d2 < D2_FLOOR) continue;
        V2 rel = dxi;
        int32_t mu = fi;
        if (!is_boundary(e, j)) {
          V2 pj = pred_of(e, j);
          rel = V2{fp_sub_sat(dxi.x, fp_sub_sat(pj.x, in[j].px, g), g),
                   fp_sub_sat(dxi.y, fp_sub_sat(pj.y, in[j].py, g), g)};
          mu = mat_mix(fi, e.M(in[j].matId)[M_fric]);
        }
        if (mu == 0) continue;
        int32_t r4x = fp_shr_rne(rel.x, RPRE), r4y = fp_shr_rne(rel.y, RPRE);
        int32_t dot = wadd(wmul(d4x, r4x), wmul(d4y, r4y));
        int32_t q = fp_divshift(dot, d2, 16u, g);
        int32_t tx = fp_sub_sat(r4x, fp_mul_s(d4x, q, 16u, g), g);
        int32_t ty = fp_sub_sat(r4y, fp_mul_s(d4y, q, 16u, g), g);
        int32_t wq = fp_shr_rne(e.luts[OFF_W + ui], 4u);
        int32_t sx = fp_mul_s(fp_mul_s(tx, wq, 16u - ACC - RPRE, g), mu, 16u, g);
        int32_t sy = fp_mul_s(fp_mul_s(ty, wq, 16u - ACC - RPRE, g), mu, 16u, g);
        fx = wsub(fx, clampi(sx, NEG_FR_TERM, FR_TERM));
        fy = wsub(fy, clampi(sy, NEG_FR_TERM, FR_TERM));
      }
    }
    int32_t ki = bond_k(Mi, in[i].temp, g);
    int32_t bx = 0, by = 0;
    if (Mi[M_bondK] != 0 && !rigidI && (flagsI & FLAG_BURST) == 0u) {
      uint32_t bb = i * BOND_CAP;
      for (uint32_t k = 0; k < BOND_CAP; ++k) {
        uint32_t w = e.bond[bb + k];
        if (w == 0u) break;
        if (w & BOND_TOMB) continue;
        uint32_t j = bond_j(w);
        const int32_t* Mj = e.M(in[j].matId);
        if (in[j].flags & FLAG_BURST) { e.bond[bb + k] = w | BOND_TOMB; continue; }
        if (Mj[M_bondK] == 0) { e.bond[bb + k] = w | BOND_TOMB; continue; }
        int32_t L0 = bond_l0(w);
        int32_t L02 = wmul(L0, L0);
        V2 d = pred_delta(e, pi, j, g);
        int32_t d4x = fp_shr_rne(d.x, BPRE), d4y = fp_shr_rne(d.y, BPRE);
        if (iabs(d4x) > L0_MAX || iabs(d4y) > L0_MAX) { e.bond[bb + k] = w | BOND_TOMB; continue; }
        int32_t d2 = wadd(wmul(d4x, d4x), wmul(d4y, d4y));
        if (d2 >= HARD_BREAK2) { e.bond[bb + k] = w | BOND_TOMB; continue; }
        int32_t mb = std::min(Mi[M_bondBreak], Mj[M_bondBreak]);
        int32_t mub = std::min(Mi[M_bondMu], Mj[M_bondMu]);
        if (mb != 0 && mub != 0) {
          int32_t lp = fp_neg_sat(fp_add_sat(e.der[i].lam, e.der[j].lam, g), g);
          int32_t Pq = 0;
          if (lp > 0) Pq = fp_shr_rne(lp, 4u);
          mb = wadd(wadd(65536, wsub(mb, 65536)), fp_mul_s(Pq, mub, 16u, g));
        }
        if (mb != 0 && d2 > fp_mul_s(L02, mb, 16u, g)) { e.bond[bb + k] = w | BOND_TOMB; continue; }
        if (d2 < D2_FLOOR) continue;
        int32_t kj = bond_k(Mj, in[j].temp, g);
        int32_t kp = std::min(ki, kj);
        if (kp == 0) continue;
        int32_t C = fp_sub_sat(d2, L02, g);
        int32_t q = fp_divshift(C, wmul(d2, 4), 16u, g);
        int32_t qk = fp_mul_s(q, kp, 16u, g);
        int32_t gx = fp_mul_s(d4x, qk, 16u - BPRE - ACC, g);
        int32_t gy = fp_mul_s(d4y, qk, 16u - BPRE - ACC, g);
        bx = wsub(bx, clampi(gx, NEG_BD_TERM, BD_TERM));
        by = wsub(by, clampi(gy, NEG_BD_TERM, BD_TERM));
      }
    }
    if (rigidI) {
      di.dpx = fp_add_sat(di.dpx, fx, g);
      di.dpy = fp_add_sat(di.dpy, fy, g);
    } else {
      di.dpx = fp_add_sat(fx, bx, g);
      di.dpy = fp_add_sat(fy, by, g);
    }
  }
}

// src/sim.wgsl:2245-2265
void pass_finalize(E& e, const std::vector<Particle>& in, std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    Particle o = in[i];
    if (i < e.nFluid) {
      int32_t vmaxN = fp_neg_sat(e.vmax, g);
      Derived& d = e.der[i];
      int32_t vx = clampi(fp_sub_sat(d.predx, o.px, g), vmaxN, e.vmax);
      int32_t vy = clampi(fp_sub_sat(d.predy, o.py, g), vmaxN, e.vmax);
      o.px = d.predx; o.py = d.predy;
      o.vx = vx; o.vy = vy;
      d.vtmpx = vx; d.vtmpy = vy;
      d.rinv = clampi(fp_divshift(RHO0, std::max(d.rho, RHO_FLOOR_RINV), 16u, g), 0, RINV_MAX);
    } else {
      o.vx = 0; o.vy = 0;
    }
    out[i] = o;
  }
}

// src/sim.wgsl:2300-2348
void pass_xsph(E& e, std::vector<Particle>& out) {
  // reads other particles' vtmp (not vel), writes only its own vel
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    if (out[i].flags & FLAG_RIGID) continue;
    if (out[i].flags & FLAG_ANCHOR) continue;
    int32_t ci = e.M(out[i].matId)[M_xsph];
    V2 pi = pred_of(e, i);
    int32_t vix = e.der[i].vtmpx, viy = e.der[i].vtmpy;
    int32_t rhoi = e.der[i].rho;
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    int32_t ax = 0, ay = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      if (is_boundary(e, j)) continue;
      V2 d = pred_delta(e, pi, j, g);
      int32_t id = lut_index(d, g);
      if (id < 0) continue;
      uint32_t ui = (uint32_t)id;
      int32_t K = sym_k(rhoi, e.der[j].rho, g);
      int32_t w = fp_mul_s(e.luts[OFF_W + ui], K, 16u, g);
      int32_t cij = mat_mix(ci, e.M(out[j].matId)[M_xsph]);
      ax = wadd(ax, clampi(fp_mul_s(fp_mul_s(fp_sub_sat(e.der[j].vtmpx, vix, g), w, 20u - ACC, g), cij, 16u, g), NEG_XS_TERM, XS_TERM));
      ay = wadd(ay, clampi(fp_mul_s(fp_mul_s(fp_sub_sat(e.der[j].vtmpy, viy, g), w, 20u - ACC, g), cij, 16u, g), NEG_XS_TERM, XS_TERM));
    }
    out[i].vx = fp_add_sat(out[i].vx, fp_shr_rne(ax, ACC), g);
    out[i].vy = fp_add_sat(out[i].vy, fp_shr_rne(ay, ACC), g);
  }
}

// src/sim.wgsl:2357-2384
void pass_normals(E& e) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    V2 pi = pred_of(e, i);
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    int32_t sx = 0, sy = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      if (is_boundary(e, j)) continue;
      V2 d = pred_delta(e, pi, j, g);
      int32_t id = lut_index(d, g);
      if (id < 0) continue;
      int32_t gt = e.luts[OFF_G + (uint32_t)id];
      int32_t rj = e.der[j].rinv;
      sx = wadd(sx, fp_mul_s(grad_q16(gt, d.x, g), rj, 16u, g));
      sy = wadd(sy, fp_mul_s(grad_q16(gt, d.y, g), rj, 16u, g));
    }
    e.der[i].nrmx = fp_mul_s(sx, H, 16u, g);
    e.der[i].nrmy = fp_mul_s(sy, H, 16u, g);
  }
}

// src/sim.wgsl:2409-2494
void pass_surfaceTension(E& e, const std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    const int32_t* Mt = e.M(out[i].matId);
    V2 pi = pred_of(e, i);
    int32_t nix = e.der[i].nrmx, niy = e.der[i].nrmy;
    int32_t rhoi = e.der[i].rho;
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    bool stRigidI = (out[i].flags & FLAG_RIGID) != 0;
    int32_t ax = 0, ay = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      if (stRigidI && !is_boundary(e, j) && rg_same_body(out[i].flags, out[j].flags)) continue;
      V2 d = pred_delta(e, pi, j, g);
      int32_t id = lut_index(d, g);
      if (id < 0) continue;
      uint32_t ui = (uint32_t)id;
      if (is_boundary(e, j)) {
        int32_t at = e.luts[OFF_A + ui];
        ax = wsub(ax, clampi(fp_mul_s(fp_mul_s(at, d.x, CF, g), Mt[M_adhesion], 16u - ACC, g), NEG_ST_TERM, ST_TERM));
        ay = wsub(ay, clampi(fp_mul_s(fp_mul_s(at, d.y, CF, g), Mt[M_adhesion], 16u - ACC, g), NEG_ST_TERM, ST_TERM));
        continue;
      }
      int32_t K = sym_k(rhoi, e.der[j].rho, g);
      int32_t ct = e.luts[OFF_C + ui];
      const int32_t* Mj = e.M(out[j].matId);
      int32_t gCoh = mat_mix(Mt[M_gammaCoh], Mj[M_gammaCoh]);
      int32_t gCur = mat_mix(Mt[M_gammaCur], Mj[M_gammaCur]);
      int32_t fx = fp_neg_sat(fp_mul_s(fp_mul_s(ct, d.x, CF, g), gCoh, 16u, g), g);
      int32_t fy = fp_neg_sat(fp_mul_s(fp_mul_s(ct, d.y, CF, g), gCoh, 16u, g), g);
      int32_t cx = fp_mul_s(fp_sub_sat(nix, e.der[j].nrmx, g), gCur, 16u, g);
      int32_t cy = fp_mul_s(fp_sub_sat(niy, e.der[j].nrmy, g), gCur, 16u, g);
      // select(cx, fp_neg_sat(cx), CUR_SIGN < 0): WGSL evaluates both arms.
      int32_t ncx = fp_neg_sat(cx, g), ncy = fp_neg_sat(cy, g);
      fx = fp_add_sat(fx, CUR_SIGN < 0 ? ncx : cx, g);
      fy = fp_add_sat(fy, CUR_SIGN < 0 ? ncy : cy, g);
      ax = wadd(ax, clampi(fp_mul_s(fx, K, 16u - ACC, g), NEG_ST_TERM, ST_TERM));
      ay = wadd(ay, clampi(fp_mul_s(fy, K, 16u - ACC, g), NEG_ST_TERM, ST_TERM));
    }
    e.der[i].stx = fp_shr_rne(ax, ACC);
    e.der[i].sty = fp_shr_rne(ay, ACC);
  }
}

// src/sim.wgsl:2528-2582
void pass_conduct(E& e, const std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    uint32_t mi = out[i].matId;
    const int32_t* Mi = e.M(mi);
    int32_t ki = Mi[M_cond];
    int32_t Ti = out[i].temp;
    V2 pi = pred_of(e, i);
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    int32_t q = 0, c = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      if (is_boundary(e, j)) continue;
      V2 d = pred_delta(e, pi, j, g);
      int32_t id = lut_index(d, g);
      if (id < 0) continue;
      int32_t W = e.luts[OFF_W + (uint32_t)id];
      uint32_t mj = out[j].matId;
      const int32_t* Mj = e.M(mj);
      int32_t cij = mat_mix(ki, Mj[M_cond]);
      int32_t wk = fp_mul_s(W, cij, 16u, g);
      int32_t dT = clampi(fp_sub_sat(out[j].temp, Ti, g), NEG_DT_CLAMP, DT_CLAMP);
      q = wadd(q, clampi(fp_mul_s(dT, wk, 20u - ACC, g), NEG_HT_TERM, HT_TERM));
      if (mj != mi) {
        int32_t attack = Mj[M_corrode];
        int32_t spend = (Mj[M_corrPt] != CORR_NEVER) ? Mi[M_corrode] : 0;
        int32_t str = wadd(attack, spend);
        if (str != 0) c = wadd(c, clampi(fp_mul_s(W, str, 20u - ACC, g), 0, CORR_TERM));
      }
    }
    e.der[i].heat = q;
    e.der[i].corr = c;
  }
}

// src/sim.wgsl:2612-2707
void pass_thermal(E& e, std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    Particle& p = out[i];
    uint32_t mat0 = p.matId;
    const int32_t* Mt = e.M(mat0);
    int32_t T = fp_add_sat(p.temp, fp_shr_rne(e.der[i].heat, ACC), g);
    T = fp_add_sat(T, fp_mul_s(fp_sub_sat(AMBIENT, T, g), Mt[M_coolRate], 16u, g), g);
    int32_t fuel = p.fuel;
    bool burning = (p.flags & FLAG_BURNING) != 0;
    if (!burning && fuel > 0 && T >= Mt[M_ignitePt]) burning = true;
    if (burning) {
      T = fp_add_sat(T, Mt[M_burnHeat], g);
      fuel = std::max(0, fp_sub_sat(fuel, Mt[M_burnRate], g));
    }
    T = clampi(T, TEMP_MIN, TEMP_MAX);
    T = fp_add_sat(T, fp_mul_s(fp_sub_sat(Mt[M_tempTarget], T, g), Mt[M_tempDrive], 16u, g), g);
    int32_t dose = fp_shr_rne(e.der[i].corr, ACC);
    uint32_t mat = mat0;
    bool froze = false;
    uint32_t sTo = (uint32_t)Mt[M_splitTo], sPct = (uint32_t)Mt[M_splitPct];
    if (burning && fuel <= 0) mat = pick_product((uint32_t)Mt[M_burnTo], sTo, sPct, i);
    else if (dose >= Mt[M_corrPt]) mat = pick_product((uint32_t)Mt[M_corrTo], sTo, sPct, i);
    else if (T >= Mt[M_boilPt]) mat = pick_product((uint32_t)Mt[M_boilTo], sTo, sPct, i);
    else if (T >= Mt[M_meltPt]) mat = pick_product((uint32_t)Mt[M_meltTo], sTo, sPct, i);
    else if (T <= Mt[M_condPt]) mat = pick_product((uint32_t)Mt[M_condTo], sTo, sPct, i);
    else if (T <= Mt[M_freezePt]) { mat = pick_product((uint32_t)Mt[M_freezeTo], sTo, sPct, i); froze = true; }
    if (mat != mat0) { fuel = e.M(mat)[M_fuel0]; burning = false; }
    uint32_t fl = p.flags & ~(FLAG_BURNING | FLAG_DEAD | FLAG_SEAL);
    if (mat != mat0) fl &= ~(FLAG_ANCHOR | FLAG_CONGEAL | FLAG_BURST);
    if (froze && mat != mat0 && fuse_row(e.M(mat), mat)) fl |= FLAG_CONGEAL;
    if (burning) fl |= FLAG_BURNING;
    if (e.M(mat)[M_phantom] != 0) fl |= FLAG_DEAD;
    if (seal_class_row(e.M(mat))) fl |= FLAG_SEAL;
    p.matId = mat; p.flags = fl; p.temp = T; p.fuel = fuel;
  }
}

// src/sim.wgsl:2714-2730
void pass_markCongealNbr(E& e, const std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    bool seen = false;
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      if (j < e.nFluid && (out[j].flags & FLAG_CONGEAL)) { seen = true; break; }
    }
    e.nbrN[i] = (e.nbrN[i] & ~NBR_CONGEAL_BIT) | (seen ? NBR_CONGEAL_BIT : 0u);
  }
}

// src/sim.wgsl:2794-2989
void pass_bondForm1(E& e, const std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    uint32_t cb = i * BOND_CAP;
    if (out[i].flags & FLAG_RIGID) {
      for (uint32_t k = 0; k < BOND_CAP; ++k) e.bondCand[cb + k] = 0;
      continue;
    }
    bool anchoredI = (out[i].flags & FLAG_ANCHOR) != 0;
    uint32_t matI = out[i].matId;
    const int32_t* Mi = e.M(matI);
    uint32_t cn = 0;
    if (Mi[M_bondK] != 0 && Mi[M_bondGroup] >= 0) {
      for (uint32_t k = 0; k < BOND_CAP; ++k) {
        uint32_t w = e.bond[cb + k];
        if (w == 0u) break;
        if (w & BOND_TOMB) continue;
        if (cn >= BOND_CAP) { g.flag(8); break; }
        e.bondCand[cb + cn++] = w;
      }
      uint32_t tagI = weld_tag(out[i].flags);
      int32_t ki = bond_k(Mi, out[i].temp, g);
      bool canReform = (!anchoredI && Mi[M_bondReform] != 0 && ki != 0);
      bool fuseArmed = (e.fuseTag != 0u && fuse_row(Mi, matI));
      bool congealI = ((out[i].flags & FLAG_CONGEAL) != 0u && fuse_row(Mi, matI));
      bool congealNear = ((e.nbrN[i] & NBR_CONGEAL_BIT) != 0u && fuse_row(Mi, matI));
      if (canReform || (!anchoredI && tagI != 0u) || fuseArmed || congealI || congealNear) {
        uint32_t cnt = nbr_count(e, i), nb = i * MAXNBR;
        for (uint32_t k = 0; k < cnt; ++k) {
          if (cn >= BOND_CAP) { g.flag(8); break; }
          uint32_t j = e.nbr[nb + k];
          if (j >= e.nFluid) continue;
          const int32_t* Mj = e.M(out[j].matId);
          uint32_t fJ = out[j].flags;
          uint32_t tagJ = weld_tag(fJ);
          bool weld = (!anchoredI && tagI != 0u && tagI == tagJ);
          bool fuse = false;
          if (fuseArmed && (fJ & FLAG_RIGID) == 0u && fuse_row(Mj, out[j].matId) &&
              (!anchoredI || (fJ & FLAG_ANCHOR) == 0u)) {
            fuse = ((tagI == e.fuseTag && tagJ == 0u) || (tagJ == e.fuseTag && tagI == 0u) ||
                    (tagI == e.fuseTag && tagJ == e.fuseTag));
          }
          bool congealJ = ((fJ & FLAG_CONGEAL) != 0u && fuse_row(Mj, out[j].matId));
          bool congeal = ((congealI || congealJ) && !weld && !fuse && out[j].matId == matI && (fJ & FLAG_RIGID) == 0u);
          if (!fuse && !congeal && Mj[M_bondGroup] != Mi[M_bondGroup]) continue;
          if (!weld && !fuse && !congeal) {
            if (!canReform) continue;
            if (bond_k(Mj, out[j].temp, g) == 0) continue;
          }
          bool dup = false;
          for (uint32_t q = 0; q < cn; ++q) if (bond_j(e.bondCand[cb + q]) == j) { dup = true; break; }
          if (dup) continue;
          V2 d{fp_sub_sat(out[i].px, out[j].px, g), fp_sub_sat(out[i].py, out[j].py, g)};
          int32_t d4x = fp_shr_rne(d.x, BPRE), d4y = fp_shr_rne(d.y, BPRE);
          if (iabs(d4x) > L0_MAX || iabs(d4y) > L0_MAX) continue;
          int32_t d2 = wadd(wmul(d4x, d4x), wmul(d4y, d4y));
          if (d2 < D2_FLOOR || d2 > BOND_R2) continue;
          if (!weld && !fuse && !congeal) {
            int32_t vl = std::min(Mi[M_bondFormV], Mj[M_bondFormV]);
            int32_t vl4 = fp_shr_rne(vl, RPRE);
            int32_t r4x = fp_shr_rne(fp_sub_sat(out[i].vx, out[j].vx, g), RPRE);
            int32_t r4y = fp_shr_rne(fp_sub_sat(out[i].vy, out[j].vy, g), RPRE);
            if (iabs(r4x) > vl4 || iabs(r4y) > vl4) continue;
            if (wadd(wmul(r4x, r4x), wmul(r4y, r4y)) > wmul(vl4, vl4)) continue;
            int32_t pl = std::min(Mi[M_bondFormP], Mj[M_bondFormP]);
            if (pl != 0 && (fp_neg_sat(e.der[i].lam, g) < pl || fp_neg_sat(e.der[j].lam, g) < pl)) continue;
          }
          int32_t L0 = (int32_t)isqrt64((uint64_t)(uint32_t)d2);
          if (L0 < L0_MIN || L0 > L0_MAX) continue;
          e.bondCand[cb + cn++] = bond_pack(j, L0);
        }
      }
    }
    for (uint32_t k = cn; k < BOND_CAP; ++k) e.bondCand[cb + k] = 0;
  }
}

// src/sim.wgsl:3001-3068
void pass_bondForm2(E& e, std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    uint32_t i = (uint32_t)ii;
    uint32_t cb = i * BOND_CAP;
    uint32_t nn = 0;
    for (uint32_t k = 0; k < BOND_CAP; ++k) {
      uint32_t w = e.bondCand[cb + k];
      if (w == 0u) break;
      uint32_t j = bond_j(w), jb = j * BOND_CAP;
      bool ok = false;
      for (uint32_t q = 0; q < BOND_CAP; ++q) {
        uint32_t v = e.bondCand[jb + q];
        if (v == 0u) break;
        if (bond_j(v) == i) { ok = ((v & BOND_L0_MASK) == (w & BOND_L0_MASK)); break; }
      }
      if (ok) e.bond[cb + nn++] = w & ~BOND_TOMB;
    }
    for (uint32_t k = nn; k < BOND_CAP; ++k) e.bond[cb + k] = 0;
    uint32_t fOut = out[i].flags & ~FLAG_CONGEAL;
    if ((fOut & FLAG_RIGID) == 0u && weld_tag(fOut) != e.weldHold) fOut &= ~WELD_TAG_MASK;
    out[i].flags = fOut;
  }
}

// ---- state hash: src/hash/statehash.js:36-169 --------------------------------
constexpr uint32_t LANE_SEED[4] = {0x9e3779b1u, 0x85ebca77u, 0xc2b2ae3du, 0x27d4eb2fu};
constexpr uint32_t LANE_SALT[4] = {0x00000000u, 0x51633e2du, 0x9c8f2a17u, 0xd0e5b943u};
constexpr uint32_t CHAIN_INIT[8] = {0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u,
                                    0xa4093822u, 0x299f31d0u, 0x082efa98u, 0xec4e6c89u};
constexpr uint32_t BOND_SALT = 0x5bd1e995u, BOND_SALT2 = 0x2f5b3c17u;
inline uint32_t rotl32(uint32_t x, uint32_t r) { return (x << (r & 31)) | (x >> ((32 - r) & 31)); }
inline uint32_t mm_step(uint32_t h, uint32_t k) {
  k *= 0xcc9e2d51u; k = rotl32(k, 15); k *= 0x1b873593u;
  h ^= k; h = rotl32(h, 13); return h * 5u + 0xe6546b64u;
}
inline uint32_t fmix32(uint32_t h) {
  h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16; return h;
}

void digest(const E& e, const std::vector<Particle>& s, uint32_t acc[8]) {
  for (int l = 0; l < 8; ++l) acc[l] = 0;
  const uint32_t nw = 8, m = 9;
  for (uint32_t i = 0; i < e.n; ++i) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(&s[i]);
    uint32_t h[4] = {LANE_SEED[0], LANE_SEED[1], LANE_SEED[2], LANE_SEED[3]};
    for (uint32_t k = 0; k < nw; ++k)
      for (int l = 0; l < 4; ++l) h[l] = mm_step(h[l], w[k] ^ LANE_SALT[l]);
    uint32_t sl[4], ll[4];
    for (int l = 0; l < 4; ++l) { sl[l] = h[l]; ll[l] = h[l]; }
    if (i < e.nFluid) {
      uint32_t bn = 0, com = 0, scom = 0;
      for (uint32_t k = 0; k < BOND_CAP; ++k) {
        uint32_t w2 = e.bond[i * BOND_CAP + k];
        if (w2 == 0u) break;
        com += fmix32(((w2 >> 17) & 0x1fffu) ^ BOND_SALT);
        scom += fmix32(w2 ^ BOND_SALT2);
        bn++;
      }
      if (bn != 0) {
        for (int l = 0; l < 4; ++l) { sl[l] = mm_step(sl[l], bn) ^ com; ll[l] = mm_step(ll[l], bn) ^ scom; }
      }
    }
    for (int l = 0; l < 4; ++l) {
      acc[l] += fmix32(sl[l] ^ nw);
      acc[4 + l] += fmix32(mm_step(ll[l], i) ^ m);
    }
  }
}

void fold_chain(uint32_t chain[8], const uint32_t acc[8]) {
  uint32_t next[8];
  for (int j = 0; j < 8; ++j) next[j] = mm_step(chain[j], acc[j] ^ rotl32(acc[(j + 1) & 7], 7));
  for (int j = 0; j < 8; ++j) chain[j] = next[j];
}

// fp_div_s (src/fixed.wgsl:219-261): (|a| << s) / |b| exactly, rounded half
// to even on the exact remainder, signed and saturated.
inline int32_t fp_div_s(int32_t a, int32_t b, uint32_t s, const Dbg& d) {
  if (b == 0) {
    d.flag(2);
    return a == 0 ? 0 : (a > 0 ? I32_MAX : I32_MIN);
  }
  const bool neg = (a < 0) != (b < 0);
  const uint64_t ua = a < 0 ? (uint64_t)(-(int64_t)a) : (uint64_t)a;
  const uint64_t ub = b < 0 ? (uint64_t)(-(int64_t)b) : (uint64_t)b;
  const uint64_t n = ua << s;
  const uint64_t q = n / ub, rem = n % ub;
  bool ovf = q > 0xffffffffull;
  uint32_t q32 = (uint32_t)q;
  const uint64_t other = ub - rem;
  if (rem > other || (rem == other && (q32 & 1u))) {
    if (q32 == 0xffffffffu) { ovf = true; q32 = 0; } else { ++q32; }
  }
  if (ovf) { d.flag(1); return neg ? I32_MIN : I32_MAX; }
  if (neg) {
    if (q32 > 2147483648u) { d.flag(1); return I32_MIN; }
    if (q32 == 2147483648u) return I32_MIN;
    return -(int32_t)q32;
  }
  if (q32 > 2147483647u) { d.flag(1); return I32_MAX; }
  return (int32_t)q32;
}

// §29 containment (src/sim.wgsl:1953-2235, 2733-2771).
constexpr int32_t SEAL_SEG_MAX2 = 8820900, SEAL_SEG_MIN2 = 670761, SEAL_KEEP4 = 717, SEAL_REACH = 95027;
constexpr int32_t SEAL_STRESS4 = 2560;

// seal_cross_sign: the sign of ax*by - ay*bx, exact in 64 bits.
inline int seal_cross_sign(int32_t ax, int32_t ay, int32_t bx, int32_t by) {
  const int64_t d = (int64_t)ax * by - (int64_t)ay * bx;
  return d == 0 ? 0 : (d < 0 ? -1 : 1);
}

// The geometry shared by contain and containOverflow: the keep-out push from
// each seal endpoint, then the swept-segment test against every pair of seal
// endpoints (a crossing reverts the motion). `filter` = the list still holds
// non-seal entries to skip (contain's neighbour list).
V2 contain_core(const E& e, const std::vector<Particle>& in, const uint32_t* list, uint32_t n, bool filter, V2 pos,
                V2 pr, bool liquidI, const Dbg& g) {
  auto sealj = [&](uint32_t j) { return !is_boundary(e, j) && seal_class_row(e.M(in[j].matId)); };
  bool touched = false;
  for (uint32_t k = 0; k < n; ++k) {
    const uint32_t j = list[k];
    if (filter && !sealj(j)) continue;
    touched = true;
    const V2 pj = pred_of(e, j);
    const int32_t dx4 = fp_shr_rne(fp_sub_sat(pr.x, pj.x, g), BPRE);
    const int32_t dy4 = fp_shr_rne(fp_sub_sat(pr.y, pj.y, g), BPRE);
    const int32_t d2 = wadd(wmul(dx4, dx4), wmul(dy4, dy4));
    if (d2 > 0 && d2 < SEAL_KEEP4 * SEAL_KEEP4) {
      const int32_t d4 = (int32_t)isqrt64((uint64_t)(uint32_t)d2);
      if (d4 > 0) {
        const int32_t ux = fp_div_s(dx4, d4, 16, g), uy = fp_div_s(dy4, d4, 16, g);
        const int32_t amt = (int32_t)((uint32_t)(SEAL_KEEP4 - d4) << BPRE);
        pr.x = fp_add_sat(pr.x, fp_mul_s(ux, amt, 16, g), g);
        pr.y = fp_add_sat(pr.y, fp_mul_s(uy, amt, 16, g), g);
      }
    }
  }
  if (!touched) return pr;
  for (uint32_t k = 0; k < n; ++k) {
    const uint32_t j = list[k];
    if (filter && !sealj(j)) continue;
    const int32_t* Mj = e.M(in[j].matId);
    const V2 pj = pred_of(e, j);
    for (uint32_t q = k + 1; q < n; ++q) {
      const uint32_t k2 = list[q];
      if (filter && !sealj(k2)) continue;
      const int32_t* Mk = e.M(in[k2].matId);
      if (liquidI && Mj[M_sealMode] != 0 && Mk[M_sealMode] != 0) continue;
      const V2 pk = pred_of(e, k2);
      const int32_t ex4 = fp_shr_rne(fp_sub_sat(pk.x, pj.x, g), BPRE);
      const int32_t ey4 = fp_shr_rne(fp_sub_sat(pk.y, pj.y, g), BPRE);
      const int32_t e2 = wadd(wmul(ex4, ex4), wmul(ey4, ey4));
      if (e2 > SEAL_SEG_MAX2 || e2 < SEAL_SEG_MIN2) continue;
      if (std::min(pj.x, pk.x) > std::max(pos.x, pr.x) || std::max(pj.x, pk.x) < std::min(pos.x, pr.x) ||
          std::min(pj.y, pk.y) > std::max(pos.y, pr.y) || std::max(pj.y, pk.y) < std::min(pos.y, pr.y))
        continue;
      const int32_t ex = fp_sub_sat(pk.x, pj.x, g), ey = fp_sub_sat(pk.y, pj.y, g);
      const int s0 = seal_cross_sign(ex, ey, fp_sub_sat(pos.x, pj.x, g), fp_sub_sat(pos.y, pj.y, g));
      const int s1 = seal_cross_sign(ex, ey, fp_sub_sat(pr.x, pj.x, g), fp_sub_sat(pr.y, pj.y, g));
      if (s0 == 0 || s0 == s1) continue;
      const int32_t mx = fp_sub_sat(pr.x, pos.x, g), my = fp_sub_sat(pr.y, pos.y, g);
      const int t0 = seal_cross_sign(mx, my, fp_sub_sat(pj.x, pos.x, g), fp_sub_sat(pj.y, pos.y, g));
      const int t1 = seal_cross_sign(mx, my, fp_sub_sat(pk.x, pos.x, g), fp_sub_sat(pk.y, pos.y, g));
      if (t0 == t1 && t0 != 0) continue;
      pr = pos;
    }
  }
  return pr;
}

// contain (src/sim.wgsl:2058-2140) and containOverflow (:2144-2235). Each
// writes only an intruder's pred and reads only seal endpoints' preds, which
// neither pass moves, so one in-place sweep equals the two dispatches.
void pass_contain(E& e, const std::vector<Particle>& in) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    const uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    if (!(e.nbrN[i] & NBR_SEAL_BIT)) continue;
    const int32_t* Mi = e.M(in[i].matId);
    if (seal_class_row(Mi) || Mi[M_phantom] != 0) continue;
    if (in[i].flags & (FLAG_ANCHOR | FLAG_RIGID)) continue;
    const V2 pos{in[i].px, in[i].py};
    V2 pr = pred_of(e, i);
    const bool liquidI = seal_liquid_row(Mi);
    const uint32_t cnt = nbr_count(e, i);
    if (cnt < MAXNBR) {
      pr = contain_core(e, in, &e.nbr[(size_t)i * MAXNBR], cnt, true, pos, pr, liquidI, g);
    } else {
      uint32_t seals[MAXNBR];
      uint32_t sealN = 0;
      const int32_t loX = fp_sub_sat(std::min(pos.x, pr.x), SEAL_REACH, g);
      const int32_t hiX = fp_add_sat(std::max(pos.x, pr.x), SEAL_REACH, g);
      const int32_t loY = fp_sub_sat(std::min(pos.y, pr.y), SEAL_REACH, g);
      const int32_t hiY = fp_add_sat(std::max(pos.y, pr.y), SEAL_REACH, g);
      const V2 cc = cell_coord(e, pr);
      for (int32_t gy = cc.y - 1; gy <= cc.y + 1; ++gy) {
        if (gy < 0 || gy >= (int32_t)e.gridH) continue;
        for (int32_t gx = cc.x - 1; gx <= cc.x + 1; ++gx) {
          if (gx < 0 || gx >= (int32_t)e.gridW) continue;
          const uint32_t c = (uint32_t)gy * e.gridW + (uint32_t)gx;
          for (uint32_t t = e.cellStart[c]; t < e.cellStart[c + 1]; ++t) {
            const uint32_t j = e.sortedIds[t];
            if (is_boundary(e, j) || !seal_class_row(e.M(in[j].matId))) continue;
            const V2 pj = pred_of(e, j);
            if (pj.x < loX || pj.x > hiX || pj.y < loY || pj.y > hiY) continue;
            if (sealN < MAXNBR) seals[sealN++] = j;
          }
        }
      }
      pr = contain_core(e, in, seals, sealN, false, pos, pr, liquidI, g);
    }
    e.der[i].predx = pr.x;
    e.der[i].predy = pr.y;
  }
}

// containStress (src/sim.wgsl:2742-2771): a held seal particle sums nearby
// intrusion and, past its row's burstP, lets go (FLAG_BURST).
void pass_containStress(E& e, std::vector<Particle>& out) {
  PFOR for (int64_t ii = 0; ii < (int64_t)e.nFluid; ++ii) {
    const uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    const int32_t* Mi = e.M(out[i].matId);
    if (!seal_class_row(Mi) || Mi[M_burstP] <= 0) continue;
    const uint32_t fl = out[i].flags;
    if (!(fl & (FLAG_ANCHOR | FLAG_RIGID))) continue;
    const V2 pi{out[i].px, out[i].py};
    const uint32_t cnt = nbr_count(e, i), base = i * MAXNBR;
    int32_t stress = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
      const uint32_t j = e.nbr[base + k];
      if (is_boundary(e, j)) continue;
      const int32_t* Mj = e.M(out[j].matId);
      if (seal_class_row(Mj) || Mj[M_phantom] != 0) continue;
      const int32_t dx4 = fp_shr_rne(fp_sub_sat(pi.x, out[j].px, g), BPRE);
      const int32_t dy4 = fp_shr_rne(fp_sub_sat(pi.y, out[j].py, g), BPRE);
      const int32_t d2 = wadd(wmul(dx4, dx4), wmul(dy4, dy4));
      if (d2 >= SEAL_STRESS4 * SEAL_STRESS4) continue;
      const int32_t d4 = (int32_t)isqrt64((uint64_t)(uint32_t)d2);
      stress = wadd(stress, SEAL_STRESS4 - d4);
    }
    if ((int32_t)((uint32_t)stress << BPRE) > Mi[M_burstP])
      out[i].flags = (fl & ~(FLAG_ANCHOR | FLAG_RIGID | WELD_TAG_MASK)) | FLAG_BURST;
  }
}

// ---- §20 rigid bodies (src/sim.wgsl:670-821, 3070-3747) ----------------------
// One body at a time, members enumerated by [first, last] plus the tag, sums
// in wrapping i32 (the reference's workgroup tree is exact integer addition,
// so the order of the terms does not matter).
constexpr uint32_t RB_LIVE = 0, RB_TAG = 1, RB_FIRST = 2, RB_LAST = 3, RB_CX = 4, RB_CY = 5, RB_VX = 6,
                   RB_VY = 7, RB_THETA = 8, RB_OMEGA = 9, RB_RESX = 10, RB_RESY = 11, RB_RESVX = 12,
                   RB_RESVY = 13, RB_N = 14, RB_SUMIS2 = 15, RB_GSUM = 16, RB_INVI = 17, RB_IQ = 18,
                   RB_RSH = 19, RB_ISH = 20, RB_OMEGAM = 21, RB_RMAX = 22, RB_OSH = 23, RB_CQX = 24,
                   RB_CQY = 25, RB_THETAQ = 26, RB_AXIS = 27, RB_USER = 28;
constexpr uint32_t RG_BODY_WORDS = 32, RG_MAX_BODIES = 1024, RG_DRIVER_WORDS = 10;
constexpr uint32_t RD_MASK = 0, RD_PX = 1, RD_PY = 2, RD_A = 3, RD_VX = 4, RD_VY = 5, RD_W = 6, RD_FX = 7,
                   RD_FY = 8, RD_TQ = 9;
constexpr int32_t RD_HAS_PX = 1, RD_HAS_PY = 2, RD_HAS_A = 4, RD_HAS_VX = 8, RD_HAS_VY = 16, RD_HAS_W = 32,
                  RD_HAS_FX = 64, RD_HAS_FY = 128, RD_HAS_TQ = 256;
constexpr int32_t BAM_QUARTER = 1073741824, BAM_PER_RAD = 683565276;
constexpr uint32_t RG_QSH = 20, COS_Q = 22, RG_QN = 1024;
constexpr int32_t RG_QMASK = 1048575, COS_ONE = 4194304;
constexpr int32_t RS_TARGET = 2048, TQ_TERM_R = 134217728, NEG_TQ_TERM = -134217728;
constexpr uint32_t TQ_HI_SH = 15;
constexpr int32_t RIGID_MIN_MEMBERS = 4, SUMI_MAX = 1073741824;
constexpr int32_t RG_IQ_MIN = 16, RG_IQ_MAX = 31;
constexpr int32_t SEAL_R4 = 1126;

// fp_shr_rne with a per-body shift: WGSL takes a shift amount modulo 32, so
// s = 0 returns x unchanged (rem = 0 and the half-point is 2^31).
inline int32_t shr_rne_rt(int32_t x, uint32_t s) { return s == 0 ? x : fp_shr_rne(x, s); }

// rg_cos (src/sim.wgsl:836-852): quarter-turn fold + linear interpolation.
inline int32_t rg_cos(const E& e, int32_t a, const Dbg& g) {
  const uint32_t q = ((uint32_t)a >> 30) & 3u;
  const int32_t w = a & 1073741823;
  int32_t u;
  bool neg;
  if (q == 0u) { u = w; neg = false; }
  else if (q == 1u) { u = BAM_QUARTER - w; neg = true; }
  else if (q == 2u) { u = w; neg = true; }
  else { u = BAM_QUARTER - w; neg = false; }
  const uint32_t idx = (uint32_t)u >> RG_QSH;
  const int32_t frac = u & RG_QMASK;
  const int32_t c0 = e.cosT[idx], c1 = e.cosT[idx + 1];
  const int32_t v = wadd(c0, fp_mul_s(wsub(c1, c0), frac, RG_QSH, g));
  return neg ? wsub(0, v) : v;
}
inline int32_t rg_sin(const E& e, int32_t a, const Dbg& g) { return rg_cos(e, wsub(a, BAM_QUARTER), g); }

// rg_idiv_rne (src/sim.wgsl:862-872): round-half-even divide, sign-symmetric.
inline int32_t rg_idiv_rne(int32_t a, int32_t n) {
  if (n <= 0) return 0;
  const bool neg = a < 0;
  const int32_t x = neg ? wsub(0, a) : a;
  int32_t q = (int32_t)((int64_t)x / n);
  const int32_t r2 = wmul(2, wsub(x, wmul(q, n)));
  if (r2 > n || (r2 == n && (q & 1) == 1)) q = wadd(q, 1);
  return neg ? wsub(0, q) : q;
}

// rg_inv_inertia (src/sim.wgsl:3141-3154)
inline void rg_inv_inertia(int32_t s, int32_t rsh, int32_t ish, int32_t& invI, int32_t& iq, const Dbg& g) {
  invI = 0;
  iq = 0;
  if (s <= 0) return;
  const int32_t bl = 32 - (int32_t)clz32((uint32_t)s);
  const int32_t iqNat = bl - 1 + 2 * ish - rsh;
  const int32_t q = std::min(iqNat, RG_IQ_MAX);
  const int32_t E_ = q + rsh - 2 * ish;
  if (iqNat < RG_IQ_MIN || E_ < 1 || E_ > 62) { g.flag(10); return; }
  invI = fp_div_s(BAM_PER_RAD, s, (uint32_t)E_, g);
  iq = q;
}
// rg_mul_shr (src/sim.wgsl:3167-3169)
inline int32_t rg_mul_shr(int32_t a, int32_t b, int32_t s, const Dbg& g) {
  return i64_shr_rne_sat((int64_t)a * (int64_t)b, (uint32_t)clampi(s, 1, 31), g);
}
inline bool rg_is_member(const std::vector<Particle>& st, uint32_t i, int32_t tag) {
  const uint32_t f = st[i].flags;
  return (f & FLAG_RIGID) != 0u && (int32_t)weld_tag(f) == tag;
}
inline int32_t* body_rec(E& e, uint32_t b) { return e.rbody.data() + (size_t)b * RG_BODY_WORDS; }
inline const int32_t* body_drv(const E& e, uint32_t b) { return e.rdrive.data() + (size_t)b * RG_DRIVER_WORDS; }

// rg_place (src/sim.wgsl:3193-3206): pred = c + R(theta) * o for every member.
void rg_place(E& e, const std::vector<Particle>& in, int32_t tag, uint32_t first, uint32_t last, int32_t cx,
              int32_t cy, int32_t th, const Dbg& g) {
  const int32_t c = rg_cos(e, th, g), s = rg_sin(e, th, g);
  for (uint32_t i = first; i <= last && i < e.nFluid; ++i) {
    if (!rg_is_member(in, i, tag)) continue;
    const int32_t ox = e.rest[2 * (size_t)i], oy = e.rest[2 * (size_t)i + 1];
    e.der[i].predx = fp_add_sat(cx, fp_sub_sat(fp_mul_s(ox, c, COS_Q, g), fp_mul_s(oy, s, COS_Q, g), g), g);
    e.der[i].predy = fp_add_sat(cy, fp_add_sat(fp_mul_s(ox, s, COS_Q, g), fp_mul_s(oy, c, COS_Q, g), g), g);
  }
}

// rigidStep (src/sim.wgsl:3226-3440), before predict.
void pass_rigidStep(E& e, const std::vector<Particle>& in) {
  Dbg g = e.D();
  for (uint32_t b = 0; b < (uint32_t)e.bodies.size(); ++b) {
    int32_t* R = body_rec(e, b);
    const int32_t* D = body_drv(e, b);
    const int32_t tag = R[RB_TAG], n = R[RB_N], axis = R[RB_AXIS], usr = R[RB_USER], dmask = D[RD_MASK];
    const uint32_t first = (uint32_t)R[RB_FIRST], last = (uint32_t)R[RB_LAST], rsh = (uint32_t)R[RB_RSH];
    const bool ok = R[RB_LIVE] != 0 && n >= RIGID_MIN_MEMBERS;
    if (!ok) continue;
    int32_t cx = R[RB_CX], cy = R[RB_CY];
    if (dmask & RD_HAS_PX) cx = D[RD_PX];
    if (dmask & RD_HAS_PY) cy = D[RD_PY];
    int32_t fx = 0, fy = 0, thi = 0, tlo = 0;
    for (uint32_t i = first; i <= last && i < e.nFluid; ++i) {
      if (!rg_is_member(in, i, tag)) continue;
      const Derived& d = e.der[i];
      const int32_t gI = axis != 0 ? e.M(in[i].matId)[M_grav] : 0;
      const int32_t sy0 = fp_add_sat(d.sty, gI, g);
      const V2 jm = jet_accel(e, in[i].px, in[i].py, g);
      const int32_t jx0 = fp_add_sat(d.stx, jm.x, g), jy0 = fp_add_sat(sy0, jm.y, g);
      const int32_t sx = clampi(jx0, -32768, 32768), sy = clampi(jy0, -32768, 32768);
      if (sx != jx0 || sy != jy0) g.flag(11);
      fx = wadd(fx, sx);
      fy = wadd(fy, sy);
      const int32_t rx = shr_rne_rt(fp_sub_sat(in[i].px, cx, g), rsh);
      const int32_t ry = shr_rne_rt(fp_sub_sat(in[i].py, cy, g), rsh);
      const int32_t raw = wsub(wmul(rx, sy), wmul(ry, sx));
      if (raw > TQ_TERM_R || raw < NEG_TQ_TERM) g.flag(9);
      const int32_t t = clampi(raw, NEG_TQ_TERM, TQ_TERM_R);
      const int32_t hi = t >> TQ_HI_SH;
      thi = wadd(thi, hi);
      tlo = wadd(tlo, wsub(t, (int32_t)((uint32_t)hi << TQ_HI_SH)));
    }
    const int32_t invI = R[RB_INVI], iq = R[RB_IQ], gS = R[RB_GSUM];
    const bool holdX = axis != 0 || (dmask & RD_HAS_PX), holdY = axis != 0 || (dmask & RD_HAS_PY);
    int32_t dvx = 0, dvy = 0;
    if (axis == 0) {
      const int32_t ax = wadd(R[RB_RESVX], fx), ay = wadd(wadd(R[RB_RESVY], fy), gS);
      dvx = rg_idiv_rne(ax, n);
      dvy = rg_idiv_rne(ay, n);
      R[RB_RESVX] = wsub(ax, wmul(dvx, n));
      R[RB_RESVY] = wsub(ay, wmul(dvy, n));
      const int32_t uax = usr != 0 ? e.userA[0] : 0, uay = usr != 0 ? e.userA[1] : 0;
      dvx = fp_add_sat(dvx, uax, g);
      dvy = fp_add_sat(dvy, uay, g);
    }
    if (dmask & RD_HAS_FX) dvx = fp_add_sat(dvx, D[RD_FX], g);
    if (dmask & RD_HAS_FY) dvy = fp_add_sat(dvy, D[RD_FY], g);
    int32_t vx0 = R[RB_VX], vy0 = R[RB_VY];
    if (dmask & RD_HAS_VX) vx0 = D[RD_VX];
    if (dmask & RD_HAS_VY) vy0 = D[RD_VY];
    const int32_t vmaxN = fp_neg_sat(e.vmax, g);
    const int32_t vx = clampi(fp_add_sat(vx0, dvx, g), vmaxN, e.vmax);
    const int32_t vy = clampi(fp_add_sat(vy0, dvy, g), vmaxN, e.vmax);
    if (holdX) {
      R[RB_VX] = 0; R[RB_RESVX] = 0; R[RB_CQX] = cx; R[RB_CX] = cx;
    } else {
      R[RB_VX] = vx;
      R[RB_CQX] = clampi(fp_add_sat(cx, vx, g), WALL, wsub(e.domW, WALL));
    }
    if (holdY) {
      R[RB_VY] = 0; R[RB_RESVY] = 0; R[RB_CQY] = cy; R[RB_CY] = cy;
    } else {
      R[RB_VY] = vy;
      R[RB_CQY] = clampi(fp_add_sat(cy, vy, g), WALL, wsub(e.domH, WALL));
    }
    int32_t dth = 0;
    if (invI != 0)
      dth = fp_add_sat(rg_mul_shr(thi, invI, iq - (int32_t)TQ_HI_SH, g), rg_mul_shr(tlo, invI, iq, g), g);
    if (dmask & RD_HAS_TQ) dth = fp_add_sat(dth, D[RD_TQ], g);
    int32_t theta = R[RB_THETA], w0 = R[RB_OMEGA];
    if (dmask & RD_HAS_A) theta = D[RD_A];
    if (dmask & RD_HAS_W) w0 = D[RD_W];
    const int32_t om = R[RB_OMEGAM];
    const int32_t w = clampi(fp_add_sat(w0, dth, g), wsub(0, om), om);
    if (dmask & RD_HAS_A) {
      R[RB_THETA] = theta; R[RB_THETAQ] = theta; R[RB_OMEGA] = 0;
    } else {
      R[RB_OMEGA] = w;
      R[RB_THETAQ] = wadd(theta, w);
    }
    rg_place(e, in, tag, first, last, R[RB_CQX], R[RB_CQY], R[RB_THETAQ], g);
  }
}

// rigid_seal_delta (src/sim.wgsl:2001-2051): a member's swept segment against
// the anchored seal particles of the cells its expanded AABB touches; a hit
// returns the reversion pos - pred, which rigidSolve folds into the body.
V2 rigid_seal_delta(const E& e, const std::vector<Particle>& in, uint32_t i, int32_t bodyTag, const Dbg& g) {
  const V2 pos{in[i].px, in[i].py}, pr{e.der[i].predx, e.der[i].predy};
  const int32_t mx4 = fp_shr_rne(fp_sub_sat(pr.x, pos.x, g), BPRE), my4 = fp_shr_rne(fp_sub_sat(pr.y, pos.y, g), BPRE);
  const int32_t ml2 = wadd(wmul(mx4, mx4), wmul(my4, my4));
  const V2 lo = cell_coord(e, V2{fp_sub_sat(std::min(pos.x, pr.x), SEAL_REACH, g),
                                 fp_sub_sat(std::min(pos.y, pr.y), SEAL_REACH, g)});
  const V2 hi = cell_coord(e, V2{fp_add_sat(std::max(pos.x, pr.x), SEAL_REACH, g),
                                 fp_add_sat(std::max(pos.y, pr.y), SEAL_REACH, g)});
  for (int32_t gy = lo.y; gy <= hi.y; ++gy)
    for (int32_t gx = lo.x; gx <= hi.x; ++gx) {
      const uint32_t c = (uint32_t)gy * e.gridW + (uint32_t)gx;
      for (uint32_t t = e.cellStart[c]; t < e.cellStart[c + 1]; ++t) {
        const uint32_t j = e.sortedIds[t];
        if (j == i || is_boundary(e, j)) continue;
        const uint32_t fj = in[j].flags;
        if ((fj & (FLAG_ANCHOR | FLAG_SEAL)) != (FLAG_ANCHOR | FLAG_SEAL) || !seal_class_row(e.M(in[j].matId)))
          continue;
        if ((fj & FLAG_RIGID) && (int32_t)weld_tag(fj) == bodyTag) continue;
        const int32_t px4 = fp_shr_rne(fp_sub_sat(e.der[j].predx, pos.x, g), BPRE);
        const int32_t py4 = fp_shr_rne(fp_sub_sat(e.der[j].predy, pos.y, g), BPRE);
        int32_t dx4 = px4, dy4 = py4;
        if (ml2 > 0) {
          const int32_t dot = wadd(wmul(px4, mx4), wmul(py4, my4));
          if (dot >= ml2) {
            dx4 = wsub(px4, mx4);
            dy4 = wsub(py4, my4);
          } else if (dot > 0) {
            const int32_t tq = fp_div_s(dot, ml2, 16, g);
            dx4 = wsub(px4, fp_mul_s(mx4, tq, 16, g));
            dy4 = wsub(py4, fp_mul_s(my4, tq, 16, g));
          }
        }
        if (wadd(wmul(dx4, dx4), wmul(dy4, dy4)) < SEAL_R4 * SEAL_R4)
          return V2{fp_sub_sat(pos.x, pr.x, g), fp_sub_sat(pos.y, pr.y, g)};
      }
    }
  return V2{0, 0};
}

// rigidSolve (src/sim.wgsl:3459-3573), once per iteration after applyFric.
void pass_rigidSolve(E& e, const std::vector<Particle>& in) {
  Dbg g = e.D();
  for (uint32_t b = 0; b < (uint32_t)e.bodies.size(); ++b) {
    int32_t* R = body_rec(e, b);
    const int32_t* D = body_drv(e, b);
    const int32_t tag = R[RB_TAG], n = R[RB_N], axis = R[RB_AXIS], dmask = D[RD_MASK];
    const uint32_t first = (uint32_t)R[RB_FIRST], last = (uint32_t)R[RB_LAST], rsh = (uint32_t)R[RB_RSH];
    const int32_t cqx = R[RB_CQX], cqy = R[RB_CQY];
    if (!(R[RB_LIVE] != 0 && n >= RIGID_MIN_MEMBERS)) continue;
    int32_t fx = 0, fy = 0, sx = 0, sy = 0, sn = 0, thi = 0, tlo = 0;
    for (uint32_t i = first; i <= last && i < e.nFluid; ++i) {
      if (!rg_is_member(in, i, tag)) continue;
      const int32_t dm = e.M(in[i].matId)[M_dpMax], dmN = fp_neg_sat(dm, g);
      const Derived& d = e.der[i];
      const V2 seal = rigid_seal_delta(e, in, i, tag, g);
      const int32_t dx = clampi(fp_shr_rne(d.dpx, ACC), dmN, dm), dy = clampi(fp_shr_rne(d.dpy, ACC), dmN, dm);
      fx = wadd(fx, dx);
      fy = wadd(fy, dy);
      if (seal.x != 0 || seal.y != 0) {
        sx = wadd(sx, seal.x);
        sy = wadd(sy, seal.y);
        sn = wadd(sn, 1);
      }
      const int32_t tx = fp_add_sat(dx, seal.x, g), ty = fp_add_sat(dy, seal.y, g);
      const int32_t rx = shr_rne_rt(fp_sub_sat(d.predx, cqx, g), rsh);
      const int32_t ry = shr_rne_rt(fp_sub_sat(d.predy, cqy, g), rsh);
      const int32_t raw = wsub(wmul(rx, ty), wmul(ry, tx));
      if (raw > TQ_TERM_R || raw < NEG_TQ_TERM) g.flag(9);
      const int32_t t = clampi(raw, NEG_TQ_TERM, TQ_TERM_R);
      const int32_t hi = t >> TQ_HI_SH;
      thi = wadd(thi, hi);
      tlo = wadd(tlo, wsub(t, (int32_t)((uint32_t)hi << TQ_HI_SH)));
    }
    const int32_t invI = R[RB_INVI], iq = R[RB_IQ];
    if (axis == 0) {
      const int32_t ax = wadd(R[RB_RESX], fx), ay = wadd(R[RB_RESY], fy);
      int32_t dcx = rg_idiv_rne(ax, n), dcy = rg_idiv_rne(ay, n);
      R[RB_RESX] = wsub(ax, wmul(dcx, n));
      R[RB_RESY] = wsub(ay, wmul(dcy, n));
      if (sn > 0) {
        dcx = fp_add_sat(dcx, rg_idiv_rne(sx, sn), g);
        dcy = fp_add_sat(dcy, rg_idiv_rne(sy, sn), g);
      }
      if (!(dmask & RD_HAS_PX)) R[RB_CQX] = clampi(fp_add_sat(cqx, dcx, g), WALL, wsub(e.domW, WALL));
      else R[RB_RESX] = 0;
      if (!(dmask & RD_HAS_PY)) R[RB_CQY] = clampi(fp_add_sat(cqy, dcy, g), WALL, wsub(e.domH, WALL));
      else R[RB_RESY] = 0;
    }
    int32_t dth = 0;
    if (invI != 0)
      dth = fp_add_sat(rg_mul_shr(thi, invI, iq - (int32_t)TQ_HI_SH, g), rg_mul_shr(tlo, invI, iq, g), g);
    if (!(dmask & RD_HAS_A)) R[RB_THETAQ] = wadd(R[RB_THETAQ], dth);
    rg_place(e, in, tag, first, last, R[RB_CQX], R[RB_CQY], R[RB_THETAQ], g);
  }
}

// rigidMember (src/sim.wgsl:3610-3747), after containStress. The leave step
// decides every member against the membership the pass began with, then
// clears: the reference's workgroup clears FLAG_RIGID in the same loop that
// other lanes read it, which only matters when a leaving member is another
// member's sole same-body neighbour within bond range; here that read is
// defined as the state at the start of the pass.
void pass_rigidMember(E& e, std::vector<Particle>& out) {
  Dbg g = e.D();
  for (uint32_t b = 0; b < (uint32_t)e.bodies.size(); ++b) {
    int32_t* R = body_rec(e, b);
    if (R[RB_LIVE] == 0) continue;
    const int32_t tag = R[RB_TAG], axis = R[RB_AXIS];
    const uint32_t first = (uint32_t)R[RB_FIRST], last = (uint32_t)R[RB_LAST];
    const uint32_t ish = (uint32_t)R[RB_ISH], osh = (uint32_t)R[RB_OSH];
    // 1. close the substep
    const int32_t vmaxN = fp_neg_sat(e.vmax, g);
    R[RB_VX] = clampi(fp_sub_sat(R[RB_CQX], R[RB_CX], g), vmaxN, e.vmax);
    R[RB_VY] = clampi(fp_sub_sat(R[RB_CQY], R[RB_CY], g), vmaxN, e.vmax);
    R[RB_OMEGA] = wsub(R[RB_THETAQ], R[RB_THETA]);
    R[RB_CX] = R[RB_CQX];
    R[RB_CY] = R[RB_CQY];
    R[RB_THETA] = R[RB_THETAQ];
    // 2. leave
    std::vector<uint32_t> leaving;
    for (uint32_t i = first; i <= last && i < e.nFluid; ++i) {
      if (!rg_is_member(out, i, tag)) continue;
      const int32_t* M = e.M(out[i].matId);
      bool leave = M[M_solidMode] != SOLID_RIGID || M[M_phantom] != 0;
      if (!leave) {
        bool touched = false;
        const uint32_t cnt = nbr_count(e, i);
        for (uint32_t k = 0; k < cnt; ++k) {
          const uint32_t j = e.nbr[(size_t)i * MAXNBR + k];
          if (j >= e.nFluid) continue;
          if (!rg_is_member(out, j, tag)) continue;
          const int32_t dx = fp_shr_rne(fp_sub_sat(out[i].px, out[j].px, g), BPRE);
          const int32_t dy = fp_shr_rne(fp_sub_sat(out[i].py, out[j].py, g), BPRE);
          if (iabs(dx) > L0_MAX || iabs(dy) > L0_MAX) continue;
          if (wadd(wmul(dx, dx), wmul(dy, dy)) <= BOND_R2) { touched = true; break; }
        }
        leave = !touched;
      }
      if (leave) leaving.push_back(i);
    }
    for (uint32_t i : leaving) out[i].flags &= ~FLAG_RIGID;
    // 3. recount and re-base
    int32_t cn = 0, sox = 0, soy = 0, si2 = 0, gsm = 0;
    for (uint32_t i = first; i <= last && i < e.nFluid; ++i) {
      if (!rg_is_member(out, i, tag)) continue;
      const int32_t ox = e.rest[2 * (size_t)i], oy = e.rest[2 * (size_t)i + 1];
      cn = wadd(cn, 1);
      sox = wadd(sox, ox >> osh);
      soy = wadd(soy, oy >> osh);
      const int32_t a = ox >> ish, c = oy >> ish;
      si2 = wadd(si2, wadd(wmul(a, a), wmul(c, c)));
      gsm = wadd(gsm, e.M(out[i].matId)[M_grav]);
    }
    const int32_t nLive = cn;
    const bool dissolve = nLive < RIGID_MIN_MEMBERS;
    int32_t dx = 0, dy = 0;
    if (!dissolve && axis == 0) {
      dx = (int32_t)((uint32_t)rg_idiv_rne(sox, nLive) << osh);
      dy = (int32_t)((uint32_t)rg_idiv_rne(soy, nLive) << osh);
    }
    if (dissolve) {
      R[RB_LIVE] = 0;
      R[RB_N] = 0;
    } else {
      if (dx != 0 || dy != 0) {
        const int32_t th = R[RB_THETA];
        const int32_t c = rg_cos(e, th, g), s = rg_sin(e, th, g);
        R[RB_CX] = fp_add_sat(R[RB_CX], fp_sub_sat(fp_mul_s(dx, c, COS_Q, g), fp_mul_s(dy, s, COS_Q, g), g), g);
        R[RB_CY] = fp_add_sat(R[RB_CY], fp_add_sat(fp_mul_s(dx, s, COS_Q, g), fp_mul_s(dy, c, COS_Q, g), g), g);
      }
      R[RB_N] = nLive;
      R[RB_SUMIS2] = si2;
      R[RB_GSUM] = gsm;
      int32_t invI, iq;
      rg_inv_inertia(si2, R[RB_RSH], R[RB_ISH], invI, iq, g);
      R[RB_INVI] = invI;
      R[RB_IQ] = iq;
    }
    for (uint32_t i = first; i <= last && i < e.nFluid; ++i) {
      if (!rg_is_member(out, i, tag)) continue;
      if (dissolve) {
        out[i].flags &= ~FLAG_RIGID;
      } else if (dx != 0 || dy != 0) {
        e.rest[2 * (size_t)i] = wsub(e.rest[2 * (size_t)i], dx);
        e.rest[2 * (size_t)i + 1] = wsub(e.rest[2 * (size_t)i + 1], dy);
      }
    }
  }
}

// ---- §20 host math (src/engine.js:2050-2150, 5452-5811) ------------------------
// Math.round: the integral value closest to x, ties towards +infinity.
inline double js_round(double x) {
  const double r = std::floor(x);
  return (x - r >= 0.5) ? r + 1.0 : r;
}
// buildCosTable (src/engine.js:2062-2068)
void build_cos_table(int32_t T[1026]) {
  for (uint32_t k = 0; k <= RG_QN; ++k)
    T[k] = (int32_t)js_round(std::cos(((double)k * M_PI) / (double)(2 * RG_QN)) * (double)COS_ONE);
  T[RG_QN] = 0;
  T[RG_QN + 1] = 0;
}
// idivRne (src/engine.js:2074-2080) on the host's exact integers.
inline int64_t idiv_rne64(int64_t a, int64_t n) {
  if (n <= 0) return 0;
  const bool neg = a < 0;
  const int64_t x = neg ? -a : a;
  int64_t q = x / n;
  const int64_t r2 = 2 * (x - q * n);
  if (r2 > n || (r2 == n && (q & 1) == 1)) q += 1;
  return neg ? -q : q;
}
// isqrt64 (src/engine.js:2083-2089) on a double, with the reference's own
// float seed and integer correction.
inline double isqrt_js(double x) {
  if (x <= 0) return 0;
  double r = std::floor(std::sqrt(x));
  while (r > 0 && r * r > x) r -= 1;
  while ((r + 1) * (r + 1) <= x) r += 1;
  return r;
}
struct Shifts { int32_t rMax, rsh, ish, osh; };
// rigidShifts (src/engine.js:2106-2128), in the same double arithmetic.
bool rigid_shifts(const std::vector<int32_t>& ox, const std::vector<int32_t>& oy, Shifts& out) {
  const size_t N = ox.size();
  double rMax = 0;
  for (size_t k = 0; k < N; ++k) {
    const double a = std::fabs((double)ox[k]), b = std::fabs((double)oy[k]);
    const double m = isqrt_js(a * a + b * b);
    if (m > rMax) rMax = m;
  }
  const int32_t rm = (int32_t)(int64_t)rMax;
  int32_t rsh = 0;
  while ((rm >> rsh) > RS_TARGET) ++rsh;
  int32_t ish = 0;
  for (;;) {
    double sum = 0;
    for (size_t k = 0; k < N; ++k) {
      const double a = (double)(ox[k] >> ish), b = (double)(oy[k] >> ish);
      sum += a * a + b * b;
    }
    if (sum < (double)SUMI_MAX) break;
    if (++ish > 30) return false;
  }
  int32_t osh = 0;
  while ((double)N * (double)(rm >> osh) >= (double)SUMI_MAX) ++osh;
  out = Shifts{rm, rsh, ish, osh};
  return true;
}
// rigidInvInertia (src/engine.js:2135-2150): exact, like the BigInt original.
void rigid_inv_inertia_host(int32_t s, int32_t rsh, int32_t ish, int32_t& invI, int32_t& iq) {
  invI = 0;
  iq = 0;
  if (s <= 0) return;
  const int32_t bl = 32 - (int32_t)clz32((uint32_t)s);
  const int32_t iqNat = bl - 1 + 2 * ish - rsh;
  const int32_t q0 = std::min(iqNat, RG_IQ_MAX);
  const int32_t E_ = q0 + rsh - 2 * ish;
  if (iqNat < RG_IQ_MIN || E_ < 1 || E_ > 62) return;
  const unsigned __int128 num = (unsigned __int128)BAM_PER_RAD << E_, den = (unsigned __int128)s;
  unsigned __int128 q = num / den;
  const unsigned __int128 r = num - q * den;
  if (2 * r > den || (2 * r == den && (q & 1))) q += 1;
  if (q > 2147483647u) q = 2147483647u;
  invI = (int32_t)q;
  iq = q0;
}

// _writeBodyRecord (src/engine.js:5452-5580). `st` is the current state;
// `members` ascending fluid slots. Returns the body index or -1.
int32_t write_body_record(E& e, const std::vector<uint32_t>& members, const std::vector<Particle>& st, uint32_t tag,
                          const int32_t* pivot, bool user) {
  const size_t N = members.size();
  if (N < (size_t)RIGID_MIN_MEMBERS) return -1;
  if (e.bodies.size() >= RG_MAX_BODIES) return -1;
  int64_t sx = 0, sy = 0, svx = 0, svy = 0;
  for (uint32_t i : members) { sx += st[i].px; sy += st[i].py; svx += st[i].vx; svy += st[i].vy; }
  const bool axis = pivot != nullptr;
  const int32_t cx = axis ? pivot[0] : (int32_t)idiv_rne64(sx, (int64_t)N);
  const int32_t cy = axis ? pivot[1] : (int32_t)idiv_rne64(sy, (int64_t)N);
  const int32_t vx = axis ? 0 : (int32_t)idiv_rne64(svx, (int64_t)N);
  const int32_t vy = axis ? 0 : (int32_t)idiv_rne64(svy, (int64_t)N);
  std::vector<int32_t> ox(N), oy(N);
  for (size_t k = 0; k < N; ++k) {
    ox[k] = (int32_t)((int64_t)st[members[k]].px - cx);
    oy[k] = (int32_t)((int64_t)st[members[k]].py - cy);
  }
  Shifts sh;
  if (!rigid_shifts(ox, oy, sh)) return -1;
  int64_t sumIs2 = 0, gSum = 0;
  for (size_t k = 0; k < N; ++k) {
    const int64_t a = ox[k] >> sh.ish, b = oy[k] >> sh.ish;
    sumIs2 += a * a + b * b;
    gSum += e.M(st[members[k]].matId)[M_grav];
  }
  int32_t invI, iq;
  rigid_inv_inertia_host((int32_t)sumIs2, sh.rsh, sh.ish, invI, iq);
  int64_t acc = 0;
  for (size_t k = 0; k < N; ++k) {
    const Particle& p = st[members[k]];
    acc += (int64_t)(ox[k] >> sh.rsh) * ((int64_t)p.vy - vy) - (int64_t)(oy[k] >> sh.rsh) * ((int64_t)p.vx - vx);
  }
  int64_t omega = 0;
  if (invI != 0) {
    const __int128 num = (__int128)acc * invI, den = (__int128)1 << iq;
    __int128 q = num / den, r = num - q * den;
    if (r < 0) { q -= 1; r += den; }
    if (2 * r > den || (2 * r == den && (q & 1))) q += 1;
    omega = (int64_t)q;
  }
  const int64_t omegaMax =
      std::max<int64_t>(1, std::min<int64_t>(BAM_QUARTER, ((int64_t)VMAX * BAM_PER_RAD) / std::max<int64_t>(1, sh.rMax)));
  omega = std::max(-omegaMax, std::min(omegaMax, omega));
  const uint32_t idx = (uint32_t)e.bodies.size();
  e.rbody.resize((size_t)(idx + 1) * RG_BODY_WORDS, 0);
  e.rdrive.resize((size_t)(idx + 1) * RG_DRIVER_WORDS, 0);
  int32_t* R = body_rec(e, idx);
  std::fill(R, R + RG_BODY_WORDS, 0);
  std::fill(e.rdrive.begin() + (size_t)idx * RG_DRIVER_WORDS, e.rdrive.begin() + (size_t)(idx + 1) * RG_DRIVER_WORDS, 0);
  R[RB_LIVE] = 1; R[RB_TAG] = (int32_t)tag;
  R[RB_FIRST] = (int32_t)members.front(); R[RB_LAST] = (int32_t)members.back();
  R[RB_CX] = cx; R[RB_CY] = cy; R[RB_VX] = vx; R[RB_VY] = vy;
  R[RB_THETA] = 0; R[RB_OMEGA] = (int32_t)omega;
  R[RB_N] = (int32_t)N; R[RB_SUMIS2] = (int32_t)sumIs2; R[RB_GSUM] = (int32_t)(uint32_t)(uint64_t)gSum;
  R[RB_INVI] = invI; R[RB_IQ] = iq; R[RB_RSH] = sh.rsh; R[RB_ISH] = sh.ish; R[RB_OSH] = sh.osh;
  R[RB_OMEGAM] = (int32_t)omegaMax; R[RB_RMAX] = sh.rMax;
  R[RB_CQX] = cx; R[RB_CQY] = cy; R[RB_THETAQ] = 0;
  R[RB_AXIS] = axis ? 1 : 0; R[RB_USER] = user ? 1 : 0;
  for (size_t k = 0; k < N; ++k) {
    e.rest[2 * (size_t)members[k]] = ox[k];
    e.rest[2 * (size_t)members[k] + 1] = oy[k];
  }
  E::BodyDesc d;
  d.tag = tag; d.first = members.front(); d.last = members.back(); d.n = (uint32_t)N; d.axis = axis; d.user = user;
  e.bodies.push_back(d);
  return (int32_t)idx;
}

// eraseWhere's body repair (src/engine.js:6526-6610) after a compaction with
// survivors `surv` (old slots, ascending).
void repair_bodies_after_erase(E& e, const std::vector<uint32_t>& surv) {
  if (e.bodies.empty()) return;
  std::vector<Particle>& st = e.st[e.parity];
  const uint32_t newF = (uint32_t)surv.size();
  std::vector<int32_t> restOut(e.rest.size(), 0);
  for (uint32_t k = 0; k < newF; ++k) {
    restOut[2 * (size_t)k] = e.rest[2 * (size_t)surv[k]];
    restOut[2 * (size_t)k + 1] = e.rest[2 * (size_t)surv[k] + 1];
  }
  std::vector<int32_t> recs, drvs;
  std::vector<E::BodyDesc> kept;
  Dbg g = e.D();
  for (size_t bi = 0; bi < e.bodies.size(); ++bi) {
    const E::BodyDesc& b = e.bodies[bi];
    std::vector<uint32_t> mem;
    for (uint32_t k = 0; k < newF; ++k) {
      const uint32_t f = st[k].flags;
      if ((f & FLAG_RIGID) && (f & WELD_TAG_MASK) == b.tag) mem.push_back(k);
    }
    if (mem.size() < (size_t)RIGID_MIN_MEMBERS) {
      for (uint32_t k : mem) {
        st[k].flags &= ~FLAG_RIGID;
        e.st[1 - e.parity][k].flags &= ~FLAG_RIGID;
      }
      continue;
    }
    std::vector<int32_t> rec(e.rbody.begin() + bi * RG_BODY_WORDS, e.rbody.begin() + (bi + 1) * RG_BODY_WORDS);
    const int32_t ish = rec[RB_ISH];
    int64_t sumIs2 = 0, gSum = 0;
    for (uint32_t k : mem) {
      const int64_t a = restOut[2 * (size_t)k] >> ish, c = restOut[2 * (size_t)k + 1] >> ish;
      sumIs2 += a * a + c * c;
      gSum += e.M(st[k].matId)[M_grav];
    }
    int32_t invI, iq;
    rigid_inv_inertia_host((int32_t)sumIs2, rec[RB_RSH], ish, invI, iq);
    rec[RB_FIRST] = (int32_t)mem.front(); rec[RB_LAST] = (int32_t)mem.back();
    rec[RB_N] = (int32_t)mem.size(); rec[RB_SUMIS2] = (int32_t)sumIs2;
    rec[RB_GSUM] = (int32_t)(uint32_t)(uint64_t)gSum; rec[RB_INVI] = invI; rec[RB_IQ] = iq;
    recs.insert(recs.end(), rec.begin(), rec.end());
    drvs.insert(drvs.end(), e.rdrive.begin() + bi * RG_DRIVER_WORDS, e.rdrive.begin() + (bi + 1) * RG_DRIVER_WORDS);
    E::BodyDesc d = b;
    d.first = mem.front(); d.last = mem.back(); d.n = (uint32_t)mem.size();
    kept.push_back(d);
  }
  (void)g;
  e.rbody = recs;
  e.rdrive = drvs;
  e.bodies = kept;
  e.rest = restOut;
}

// One substep, in _encodeSubstep's order (src/engine.js:4003-4155).
void substep(E& e) {
  std::vector<Particle>& in = e.st[e.parity];
  std::vector<Particle>& out = e.st[1 - e.parity];
  pass_rigidStep(e, in);
  pass_predict(e, in);
  pass_grid(e);
  pass_buildNbr(e, in);
  for (uint32_t it = 0; it < e.iters; ++it) {
    pass_solveA(e, in);
    for (uint32_t c = 0; c < 4; ++c) {
      pass_solveB(e, in, c);
      pass_applyDp(e, in, (int)c);
    }
    pass_friction(e, in);
    pass_applyDp(e, in, -1);
    pass_rigidSolve(e, in);
  }
  pass_contain(e, in);
  pass_finalize(e, in, out);
  pass_xsph(e, out);
  pass_normals(e);
  pass_surfaceTension(e, out);
  pass_conduct(e, out);
  pass_thermal(e, out);
  pass_containStress(e, out);
  pass_rigidMember(e, out);
  if ((e.formationClock % BOND_PERIOD) == 0 || e.bondDirty) {
    pass_markCongealNbr(e, out);
    pass_bondForm1(e, out);
    pass_bondForm2(e, out);
    e.bondDirty = false;
  }
  e.formationClock++;
  digest(e, out, e.acc);
  fold_chain(e.chain, e.acc);
  e.parity = 1 - e.parity;
  e.substepCount++;
  e.merge_dbg();
}

}  // namespace

// ---- C ABI -------------------------------------------------------------------
extern "C" {

SnoEngine* sno_create(uint32_t maxParticles, const int32_t* luts, const int32_t* mats, uint32_t matCount,
                      uint32_t iters, int threads) {
  if (matCount == 0 || matCount > MAT_MAX || iters < 1 || iters > 16) return nullptr;
  SnoEngine* e = new SnoEngine();
  e->maxParticles = maxParticles;
  e->iters = iters;
  e->threads = threads < 1 ? 1 : threads;
  std::memcpy(e->luts, luts, sizeof(e->luts));
  std::memset(e->mats, 0, sizeof(e->mats));
  std::memcpy(e->mats, mats, sizeof(int32_t) * MAT_WORDS * matCount);
  std::memcpy(e->matsAuth, e->mats, sizeof(e->mats));
  e->matCount = e->authoredCount = matCount;
  std::memset(e->dbg, 0, sizeof(e->dbg));
  std::memset(e->dbgT, 0, sizeof(e->dbgT));
  build_cos_table(e->cosT);
  return e;
}

void sno_destroy(SnoEngine* e) { delete e; }
void sno_set_nbr_cut(SnoEngine* e, int on) { e->nbrCut = on != 0; }

// setJets (src/engine.js:4740-4770): the first JET_MAX = 8 jets, [x, y, r, fx, fy] each.
uint32_t sno_set_jets(SnoEngine* e, const int32_t* q, uint32_t k) {
  if (k > 8) k = 8;
  for (uint32_t j = 0; j < k; ++j)
    for (int w = 0; w < 5; ++w) e->jets[j][w] = q[j * 5 + w];
  e->nJets = k;
  return k;
}

// loadScene, src/engine.js:3704-3951. Returns 0 or a negative error code:
// -1 bad sizes, -2 matId out of range, -3 position out of range, -4 flags,
// -5 temp, -6 fuel, -7 cellShift, -8 too many cells, -9 a row this oracle
// does not restate (a rigid-body row, solidMode 2).
int sno_load_scene(SnoEngine* e, uint32_t n, uint32_t nFluid, const int32_t* pos, const int32_t* vel,
                   const uint32_t* matId, const uint32_t* flags, const int32_t* temp, const int32_t* fuel,
                   int32_t domW, int32_t domH, uint32_t cellShift) {
  if (n > e->maxParticles || nFluid > n) return -1;
  const int32_t MAX_POS = 134217728;
  for (uint32_t i = 0; i < n; ++i) {
    if (matId[i] >= e->matCount) return -2;
    int32_t lo = i < nFluid ? 0 : -MAX_POS;
    if (pos[2 * i] < lo || pos[2 * i] > MAX_POS || pos[2 * i + 1] < lo || pos[2 * i + 1] > MAX_POS) return -3;
    if (flags && (flags[i] & ~7u)) return -4;
    if (temp && (temp[i] < TEMP_MIN || temp[i] > TEMP_MAX)) return -5;
    if (fuel && fuel[i] < 0) return -6;
  }
  if (cellShift < 1 || cellShift > 27 || (1u << cellShift) < (uint32_t)H) return -7;
  uint32_t cs = 1u << cellShift;
  uint32_t gW = std::max<uint32_t>(1, (uint32_t)((domW + (int64_t)cs - 1) / cs));
  uint32_t gH = std::max<uint32_t>(1, (uint32_t)((domH + (int64_t)cs - 1) / cs));
  uint64_t ct = (uint64_t)gW * gH;
  if (ct > (1u << 24)) return -8;
  e->n = n; e->nFluid = nFluid; e->gridW = gW; e->gridH = gH; e->cellTotal = (uint32_t)ct;
  e->cellShift = cellShift; e->domW = domW; e->domH = domH; e->originX = 0; e->originY = 0;
  e->vmax = VMAX; e->weldHold = 0; e->fuseTag = 0; e->wallsOn = true;
  e->weldSeq = 1; e->weldHoldSeq = 0; e->lastWeldTag = 0;
  e->substepCount = 0; e->parity = 0; e->formationClock = 0; e->bondDirty = true;
  e->unsupported = 0;
  uint32_t cap = e->maxParticles;
  // a scene load dissolves every body and resets the drive (src/engine.js:3811-3813, 3849)
  e->bodies.clear();
  e->rbody.clear();
  e->rdrive.clear();
  e->rest.assign((size_t)cap * 2, 0);
  e->userA[0] = e->userA[1] = 0;
  for (int p = 0; p < 2; ++p) e->st[p].assign(cap, Particle{});
  e->der.assign(cap, Derived{});
  e->cellCount.assign(ct + 1, 0);
  e->cellStart.assign(ct + 1, 0);
  e->cellOf.assign(cap, 0);
  e->sortedIds.assign(cap, 0);
  e->nbr.assign((size_t)cap * MAXNBR, 0);
  e->nbrN.assign(cap, 0);
  e->bond.assign((size_t)cap * BOND_CAP, 0);
  e->bondCand.assign((size_t)cap * BOND_CAP, 0);
  std::memset(e->dbg, 0, sizeof(e->dbg));
  std::memset(e->dbgT, 0, sizeof(e->dbgT));
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t m = matId[i];
    const int32_t* row = e->mats[m];
    uint32_t want = row[M_phantom] != 0 ? FLAG_DEAD : 0u;
    uint32_t given = flags ? flags[i] : 0u;
    if ((given & FLAG_DEAD) && want == 0) return -4;
    Particle p;
    p.px = pos[2 * i]; p.py = pos[2 * i + 1];
    p.vx = vel[2 * i]; p.vy = vel[2 * i + 1];
    p.matId = m;
    uint32_t tag = (i < nFluid && spawn_welds(row)) ? (1u << 8) : 0u;
    p.flags = given | want | (seal_class_row(row) ? FLAG_SEAL : 0u) | tag;
    p.temp = temp ? temp[i] : AMBIENT;
    p.fuel = fuel ? fuel[i] : row[M_fuel0];
    e->st[0][i] = p;
    e->st[1][i] = p;
    e->der[i].predx = p.px;
    e->der[i].predy = p.py;
  }
  e->sceneNFluid = nFluid;
  e->scenePos.assign(pos, pos + 2 * (size_t)n);
  e->sceneMat.assign(matId, matId + n);
  e->sceneHasTemp = temp != nullptr;
  e->sceneHasFuel = fuel != nullptr;
  e->sceneTemp.assign(n, 0);
  e->sceneFuel.assign(n, 0);
  if (temp) e->sceneTemp.assign(temp, temp + n);
  if (fuel) e->sceneFuel.assign(fuel, fuel + n);
  std::memcpy(e->chain, CHAIN_INIT, sizeof(e->chain));
  return 0;
}

int sno_step(SnoEngine* e, uint32_t count) {
  if (e->n == 0) return -1;
  for (uint32_t s = 0; s < count; ++s) substep(*e);
  // step() (src/engine.js:3990-3997): the arm dies with the formation pass
  // after its gesture was released.
  if (count > 0 && e->fuseTag != 0 && e->weldHold == 0) e->fuseTag = 0;
  return e->unsupported ? -9 : 0;
}

// Weld groups (src/engine.js:4570-4680).
int sno_hold_weld_group(SnoEngine* e, uint32_t tag) {
  const uint32_t t = tag & WELD_TAG_MASK;
  if (t == 0) return -1;
  e->weldHold = t;
  e->weldHoldSeq = t >> 8;
  return (int)t;
}
uint32_t sno_end_weld_group(SnoEngine* e) {
  if (e->weldHold == 0) return 0;
  const uint32_t was = e->weldHold;
  e->weldHold = 0;
  e->weldHoldSeq = 0;
  e->bondDirty = true;
  return was;
}
uint32_t sno_begin_weld_group(SnoEngine* e) {
  if (e->weldHold != 0) sno_end_weld_group(e);
  if (e->fuseTag != 0) e->fuseTag = 0;
  return (uint32_t)sno_hold_weld_group(e, (next_weld_seq(*e) << 8) & WELD_TAG_MASK);
}
int sno_arm_fuse(SnoEngine* e) {
  if (e->weldHold == 0) return -1;
  e->fuseTag = e->weldHold;
  return (int)e->fuseTag;
}
void sno_weld_state(SnoEngine* e, uint32_t out[4]) {
  out[0] = e->weldHold; out[1] = e->fuseTag; out[2] = e->lastWeldTag; out[3] = e->weldSeq;
}

void sno_digest(SnoEngine* e, uint32_t acc[8]) { digest(*e, e->st[e->parity], acc); }
void sno_chain(SnoEngine* e, uint32_t chain[8]) { std::memcpy(chain, e->chain, sizeof(e->chain)); }
void sno_reset_chain(SnoEngine* e) { std::memcpy(e->chain, CHAIN_INIT, sizeof(e->chain)); }
void sno_dbg(SnoEngine* e, uint32_t out[16]) {
  e->merge_dbg();
  std::memcpy(out, e->dbg, sizeof(e->dbg));
}
uint32_t sno_n(SnoEngine* e) { return e->n; }
uint32_t sno_nfluid(SnoEngine* e) { return e->nFluid; }
uint64_t sno_substeps(SnoEngine* e) { return e->substepCount; }
uint64_t sno_formation_clock(SnoEngine* e) { return e->formationClock; }

int sno_read_state(SnoEngine* e, int32_t* out, size_t words) {
  if (words < (size_t)e->n * 8) return -1;
  std::memcpy(out, e->st[e->parity].data(), (size_t)e->n * 32);
  return 0;
}
int sno_read_derived(SnoEngine* e, int32_t* out, size_t words) {
  if (words < (size_t)e->n * 16) return -1;
  std::memcpy(out, e->der.data(), (size_t)e->n * 64);
  return 0;
}
// readNbrN's count field (src/engine.js:4291) and readCellStart (:4292).
int sno_read_nbr_counts(SnoEngine* e, uint32_t* out, size_t words) {
  if (words < (size_t)e->n) return -1;
  for (uint32_t i = 0; i < e->n; ++i) out[i] = e->nbrN[i] & ~(NBR_SEAL_BIT | NBR_EXT_SEAL_BIT | NBR_CONGEAL_BIT);
  return 0;
}
int sno_read_cell_start(SnoEngine* e, uint32_t* out, size_t words) {
  if (words < (size_t)e->cellTotal + 1) return -1;
  std::memcpy(out, e->cellStart.data(), ((size_t)e->cellTotal + 1) * 4);
  return 0;
}
int sno_read_bonds(SnoEngine* e, uint32_t* out, size_t words) {
  if (words < (size_t)e->nFluid * BOND_CAP) return -1;
  std::memcpy(out, e->bond.data(), (size_t)e->nFluid * BOND_CAP * 4);
  return 0;
}
// Exact keyframe restore (state words into both parities + derived rows),
// src/demo_boot.js:308-320.
int sno_write_state(SnoEngine* e, const int32_t* state, const int32_t* derived) {
  std::memcpy(e->st[0].data(), state, (size_t)e->n * 32);
  std::memcpy(e->st[1].data(), state, (size_t)e->n * 32);
  if (derived) std::memcpy(e->der.data(), derived, (size_t)e->n * 64);
  return 0;
}
int sno_write_bonds(SnoEngine* e, const uint32_t* in, size_t words) {
  if (words < (size_t)e->nFluid * BOND_CAP) return -1;
  std::memcpy(e->bond.data(), in, (size_t)e->nFluid * BOND_CAP * 4);
  return 0;
}

// eraseWhere's compaction (src/engine.js:6460-6650): keep[i] for each fluid
// slot; survivors keep their order, the boundary block follows them; state and
// derived rows are permuted, bond contents are renumbered (tombstones and
// bonds to erased partners dropped), and formation runs on the next substep.
// Returns the number of particles removed.
int64_t sno_erase(SnoEngine* e, const uint8_t* keep) {
  const uint32_t oldF = e->nFluid, nB = e->n - e->nFluid;
  std::vector<uint32_t> surv;
  for (uint32_t i = 0; i < oldF; ++i)
    if (keep[i]) surv.push_back(i);
  const uint32_t newF = (uint32_t)surv.size(), removed = oldF - newF;
  if (removed == 0) return 0;
  const uint32_t newN = newF + nB;
  std::vector<Particle>& cur = e->st[e->parity];
  std::vector<Particle> st(e->maxParticles);
  std::vector<Derived> dv(e->maxParticles);
  for (uint32_t k = 0; k < newF; ++k) { st[k] = cur[surv[k]]; dv[k] = e->der[surv[k]]; }
  for (uint32_t b = 0; b < nB; ++b) { st[newF + b] = cur[oldF + b]; dv[newF + b] = e->der[oldF + b]; }
  std::vector<int32_t> oldToNew(oldF, -1);
  for (uint32_t k = 0; k < newF; ++k) oldToNew[surv[k]] = (int32_t)k;
  std::vector<uint32_t> bo(e->bond.size(), 0), bc(e->bondCand.size(), 0);
  for (int which = 0; which < 2; ++which) {
    const std::vector<uint32_t>& src = which ? e->bondCand : e->bond;
    std::vector<uint32_t>& dst = which ? bc : bo;
    for (uint32_t k = 0; k < newF; ++k) {
      uint32_t so = surv[k] * BOND_CAP, c = 0;
      for (uint32_t q = 0; q < BOND_CAP; ++q) {
        uint32_t w = src[so + q];
        if (w == 0u) break;
        if (w & BOND_TOMB) continue;
        int32_t nj = oldToNew[w & BOND_J_MASK];
        if (nj < 0) continue;
        dst[k * BOND_CAP + c++] = (w & BOND_L0_MASK) | (uint32_t)nj;
      }
    }
  }
  e->st[0] = st;
  e->st[1] = st;
  e->der = dv;
  e->bond = bo;
  e->bondCand = bc;
  e->n = newN;
  e->nFluid = newF;
  e->bondDirty = true;
  repair_bodies_after_erase(*e, surv);
  return removed;
}

void sno_set_formation_clock(SnoEngine* e, uint64_t clk, int dirty) {
  e->formationClock = clk;
  e->bondDirty = dirty != 0;
}

// spawnFluid, src/engine.js:5901-6020. Particles are (x, y, vx, vy, mat,
// flags, temp, fuel) rows; hasTemp/hasFuel say whether temp/fuel were given.
// Returns the new n (unchanged when the cap refuses), or negative on error.
int64_t sno_spawn(SnoEngine* e, const int32_t* rows, uint32_t k, int hasTemp, int hasFuel, int noWeld) {
  if (k == 0) return e->n;
  uint32_t nB = e->n - e->nFluid;
  uint32_t newFluid = e->nFluid + k, newN = newFluid + nB;
  if (newN > e->maxParticles) return e->n;
  std::vector<Particle>& stb = e->st[e->parity];
  // noWeld bit 0: {noWeld: true}; bit 1: {ownGroup: true}
  // §18.2 W1 + §18.22 (src/engine.js:5925-5935): one gesture is one group.
  const uint32_t seq = (e->weldHoldSeq != 0 && !(noWeld & 2)) ? e->weldHoldSeq : next_weld_seq(*e);
  const uint32_t tagNow = (seq << 8) & WELD_TAG_MASK;
  e->lastWeldTag = tagNow;
  for (uint32_t i = 0; i < k; ++i) {
    const int32_t* r = rows + 8 * i;
    int32_t mm = r[4] < 0 ? 0 : r[4];
    uint32_t m = (uint32_t)std::min<int32_t>((int32_t)e->matCount - 1, mm);
    const int32_t* row = e->mats[m];
    Particle p;
    p.px = r[0]; p.py = r[1]; p.vx = r[2]; p.vy = r[3]; p.matId = m;
    const uint32_t weldTag = (!(noWeld & 1) && spawn_welds(row)) ? tagNow : 0u;
    p.flags = ((uint32_t)r[5] & (FLAG_BURNING | FLAG_ANCHOR)) | (row[M_phantom] != 0 ? FLAG_DEAD : 0u) |
              (seal_class_row(row) ? FLAG_SEAL : 0u) | weldTag;
    int32_t t = hasTemp ? r[6] : row[M_spawnTemp];
    p.temp = clampi(t, TEMP_MIN, TEMP_MAX);
    p.fuel = std::max(0, hasFuel ? r[7] : row[M_fuel0]);
    stb[e->nFluid + i] = p;
  }
  for (uint32_t b = 0; b < nB; ++b) {
    uint32_t src = e->sceneNFluid + b;
    Particle p{};
    p.px = e->scenePos[2 * src]; p.py = e->scenePos[2 * src + 1];
    p.matId = e->sceneMat[src];
    p.temp = e->sceneHasTemp ? e->sceneTemp[src] : AMBIENT;
    p.fuel = e->sceneHasFuel ? e->sceneFuel[src] : e->mats[p.matId][M_fuel0];
    stb[e->nFluid + k + b] = p;
  }
  for (uint32_t i = e->nFluid; i < newN; ++i) {
    Derived d{};
    d.predx = stb[i].px; d.predy = stb[i].py;
    e->der[i] = d;
  }
  for (uint32_t i = e->nFluid; i < newFluid; ++i)
    for (uint32_t q = 0; q < BOND_CAP; ++q) { e->bond[i * BOND_CAP + q] = 0; e->bondCand[i * BOND_CAP + q] = 0; }
  e->n = newN; e->nFluid = newFluid;
  e->bondDirty = true;
  return e->n;
}

// setWalls, src/engine.js:5262-5305: remove the boundary block (n = nFluid)
// or rewrite it from the loaded scene and put it back. Returns walls-on.
int sno_set_walls(SnoEngine* e, int on) {
  uint32_t nB = (uint32_t)e->scenePos.size() / 2 - e->sceneNFluid;
  bool want = on != 0;
  if (nB == 0) { e->wallsOn = want; return want; }
  if (want == e->wallsOn) return e->wallsOn;
  if (!want) { e->n = e->nFluid; e->wallsOn = false; return 0; }
  if (e->nFluid + nB > e->maxParticles) return e->wallsOn;
  std::vector<Particle>& stb = e->st[e->parity];
  for (uint32_t b = 0; b < nB; ++b) {
    uint32_t src = e->sceneNFluid + b;
    Particle p{};
    p.px = e->scenePos[2 * src]; p.py = e->scenePos[2 * src + 1];
    p.matId = e->sceneMat[src];
    p.temp = e->sceneHasTemp ? e->sceneTemp[src] : AMBIENT;
    p.fuel = e->sceneHasFuel ? e->sceneFuel[src] : e->mats[p.matId][M_fuel0];
    stb[e->nFluid + b] = p;
    Derived d{};
    d.predx = p.px; d.predy = p.py;
    e->der[e->nFluid + b] = d;
  }
  e->n = e->nFluid + nB;
  e->wallsOn = true;
  return 1;
}

// applyImpulse, src/engine.js:6077-6098, on the current state (the mirror the
// reference reads is synced at the substep boundary). The disc test uses IEEE
// double arithmetic exactly as the reference's JS numbers do.
int64_t sno_impulse(SnoEngine* e, int32_t cx, int32_t cy, int32_t radius, int32_t ix, int32_t iy, uint32_t limit) {
  std::vector<Particle>& s = e->st[e->parity];
  volatile double r = (double)radius;
  volatile double r2 = r * r;
  uint32_t hits = 0;
  for (uint32_t i = 0; i < e->nFluid && hits < limit; ++i) {
    volatile double dx = (double)s[i].px - (double)cx;
    volatile double dy = (double)s[i].py - (double)cy;
    volatile double a = dx * dx;
    volatile double b = dy * dy;
    volatile double sum = a + b;
    if (sum > r2) continue;
    int64_t vx = (int64_t)s[i].vx + ix, vy = (int64_t)s[i].vy + iy;
    vx = std::max<int64_t>(-VMAX, std::min<int64_t>(VMAX, vx));
    vy = std::max<int64_t>(-VMAX, std::min<int64_t>(VMAX, vy));
    s[i].vx = (int32_t)vx; s[i].vy = (int32_t)vy;
    hits++;
  }
  return hits;
}


// ---- §20 rigid bodies: the host calls (src/engine.js:5452-5811) ----------------
// pivot: NULL for a free body, else {x, y} ticks (an axis body, §19.B).
// Each returns the new body's index, or -1 where the reference returns null.
int32_t sno_make_rigid_body(SnoEngine* e, const uint32_t* slots, uint32_t k, const int32_t* pivot, int user) {
  if (k == 0 || e->nFluid == 0) return -1;
  std::vector<Particle>& st = e->st[e->parity];
  std::vector<uint32_t> members;
  for (uint32_t q = 0; q < k; ++q) {
    const uint32_t i = slots[q];
    if (i >= e->nFluid) continue;
    if (e->M(st[i].matId)[M_solidMode] != SOLID_RIGID) continue;
    if (st[i].flags & (FLAG_RIGID | FLAG_ANCHOR)) continue;
    members.push_back(i);
  }
  std::sort(members.begin(), members.end());
  if (members.size() < (size_t)RIGID_MIN_MEMBERS) return -1;
  std::vector<bool> inUse(4096, false);
  for (uint32_t i = 0; i < e->nFluid; ++i) inUse[(st[i].flags & WELD_TAG_MASK) >> 8] = true;
  uint32_t seq = 0;
  for (uint32_t g = 0; g <= 4095; ++g) {
    const uint32_t q = next_weld_seq(*e);
    if (!inUse[q]) { seq = q; break; }
  }
  if (seq == 0) return -2;
  const uint32_t tag = (seq << 8) & WELD_TAG_MASK;
  std::vector<Particle> st2 = st;
  for (uint32_t i : members) st2[i].flags = (st2[i].flags & ~WELD_TAG_MASK) | tag | FLAG_RIGID;
  const int32_t idx = write_body_record(*e, members, st2, tag, pivot, user != 0);
  if (idx < 0) return -1;
  st = st2;
  e->st[1 - e->parity] = st2;
  e->bondDirty = true;
  return idx;
}
int32_t sno_promote_weld_group(SnoEngine* e, uint32_t tag, const int32_t* pivot, int user) {
  const uint32_t t = (tag == 0 ? e->weldHold : tag) & WELD_TAG_MASK;
  if (t == 0 || e->nFluid == 0) return -1;
  std::vector<Particle>& st = e->st[e->parity];
  std::vector<uint32_t> members;
  for (uint32_t i = 0; i < e->nFluid; ++i) {
    const uint32_t f = st[i].flags;
    if ((f & WELD_TAG_MASK) != t) continue;
    if (f & (FLAG_RIGID | FLAG_ANCHOR)) continue;
    if (e->M(st[i].matId)[M_solidMode] != SOLID_RIGID) continue;
    members.push_back(i);
  }
  const int32_t idx = write_body_record(*e, members, st, t, pivot, user != 0);
  if (idx < 0) return -1;
  for (uint32_t i : members) {
    st[i].flags |= FLAG_RIGID;
    e->st[1 - e->parity][i].flags = st[i].flags;
  }
  e->bondDirty = true;
  return idx;
}
// _writeBodyRecord as the host-side rebuilds call it (members as given, tag 0
// draws _nextWeldSeq, FLAG_RIGID and the tag set). *tagOut = the tag.
int32_t sno_write_body(SnoEngine* e, const uint32_t* slots, uint32_t k, uint32_t tag, const int32_t* pivot, int user,
                       uint32_t* tagOut) {
  std::vector<uint32_t> members(slots, slots + k);
  std::sort(members.begin(), members.end());
  members.erase(std::unique(members.begin(), members.end()), members.end());
  if (!members.empty() && members.back() >= e->nFluid) return -3;
  const uint32_t t = tag != 0 ? (tag & WELD_TAG_MASK) : ((next_weld_seq(*e) << 8) & WELD_TAG_MASK);
  if (tagOut) *tagOut = t;
  if (members.empty()) return -1;
  std::vector<Particle>& st = e->st[e->parity];
  for (uint32_t i : members) {
    st[i].flags = (st[i].flags & ~WELD_TAG_MASK) | t | FLAG_RIGID;
    e->st[1 - e->parity][i].flags = st[i].flags;
  }
  e->bondDirty = true;
  return write_body_record(*e, members, st, t, pivot, user != 0);
}
int32_t sno_end_weld_group_and_promote(SnoEngine* e, const int32_t* pivot, int user) {
  const uint32_t was = sno_end_weld_group(e);
  if (was == 0) return -1;
  return sno_promote_weld_group(e, was, pivot, user);
}
uint32_t sno_dissolve_all_bodies(SnoEngine* e) {
  if (e->bodies.empty()) return 0;
  uint32_t k = 0;
  for (uint32_t i = 0; i < e->nFluid; ++i) {
    if (!(e->st[e->parity][i].flags & FLAG_RIGID)) continue;
    e->st[0][i].flags &= ~FLAG_RIGID;
    e->st[1][i].flags &= ~FLAG_RIGID;
    ++k;
  }
  e->bodies.clear();
  e->rbody.clear();
  e->rdrive.clear();
  return k;
}
uint32_t sno_body_count(SnoEngine* e) { return (uint32_t)e->bodies.size(); }
int sno_read_bodies(SnoEngine* e, int32_t* out, size_t words) {
  if (words < e->rbody.size()) return -1;
  std::memcpy(out, e->rbody.data(), e->rbody.size() * 4);
  return 0;
}
int sno_read_rest(SnoEngine* e, int32_t* out, size_t words) {
  if (words < (size_t)e->n * 2) return -1;
  std::memcpy(out, e->rest.data(), (size_t)e->n * 8);
  return 0;
}
int sno_set_body_user(SnoEngine* e, uint32_t index, int on) {
  if (index >= e->bodies.size()) return 0;
  e->bodies[index].user = on != 0;
  body_rec(*e, index)[RB_USER] = on ? 1 : 0;
  return 1;
}
// One body's driver sidecar: mask (RD_HAS_* bits) and the nine values.
int sno_set_body_driver(SnoEngine* e, uint32_t index, int32_t mask, const int32_t* values) {
  if (index >= e->bodies.size() || mask < 0 || mask >= 512) return -1;
  int32_t* D = e->rdrive.data() + (size_t)index * RG_DRIVER_WORDS;
  D[0] = mask;
  for (int q = 0; q < 9; ++q) D[1 + q] = values ? values[q] : 0;
  return 0;
}
int sno_clear_body_drivers(SnoEngine* e) {
  std::fill(e->rdrive.begin(), e->rdrive.end(), 0);
  return 0;
}
int32_t sno_set_user_drive(SnoEngine* e, int32_t ax, int32_t ay) {
  const int32_t M = 32768;
  e->userA[0] = std::max(-M, std::min(M, ax));
  e->userA[1] = std::max(-M, std::min(M, ay));
  return 0;
}
// dragGrab's rigid branch (src/engine.js:6111-6140): the body wearing `tag`
// is put one velocity behind the target and its translational remainders are
// dropped. Returns 1 if a free body was moved.
int sno_drag_body(SnoEngine* e, uint32_t tag, int32_t tx, int32_t ty, int32_t vx, int32_t vy) {
  for (size_t b = 0; b < e->bodies.size(); ++b) {
    if (e->bodies[b].tag != tag) continue;
    if (e->bodies[b].axis) return 0;
    const int32_t cvx = std::max(-VMAX, std::min(VMAX, vx)), cvy = std::max(-VMAX, std::min(VMAX, vy));
    const int32_t ONE = 65536;
    const int32_t cx = (int32_t)std::max<int64_t>(ONE, std::min<int64_t>((int64_t)e->domW - ONE, (int64_t)tx - cvx));
    const int32_t cy = (int32_t)std::max<int64_t>(ONE, std::min<int64_t>((int64_t)e->domH - ONE, (int64_t)ty - cvy));
    int32_t* R = body_rec(*e, (uint32_t)b);
    R[RB_CX] = cx; R[RB_CY] = cy; R[RB_VX] = cvx; R[RB_VY] = cvy;
    R[RB_RESX] = R[RB_RESY] = R[RB_RESVX] = R[RB_RESVY] = 0;
    return 1;
  }
  return 0;
}
// restoreAuthoringSnapshot's rigid part (src/engine.js:5838-5880): body
// records (n x 32 words) and rest offsets (n_particles x 2); drivers cleared.
int sno_restore_bodies(SnoEngine* e, const int32_t* records, uint32_t nBodies, const int32_t* rest, size_t restWords) {
  if (nBodies > RG_MAX_BODIES || restWords > e->rest.size()) return -1;
  e->rbody.assign(records, records + (size_t)nBodies * RG_BODY_WORDS);
  e->rdrive.assign((size_t)nBodies * RG_DRIVER_WORDS, 0);
  e->bodies.clear();
  for (uint32_t b = 0; b < nBodies; ++b) {
    const int32_t* R = records + (size_t)b * RG_BODY_WORDS;
    E::BodyDesc d;
    d.tag = (uint32_t)R[RB_TAG]; d.first = (uint32_t)R[RB_FIRST]; d.last = (uint32_t)R[RB_LAST];
    d.n = (uint32_t)R[RB_N]; d.axis = R[RB_AXIS] != 0; d.user = R[RB_USER] != 0;
    e->bodies.push_back(d);
  }
  if (rest) std::copy(rest, rest + restWords, e->rest.begin());
  return 0;
}


// ---- material rows at run time (src/engine.js:4843-4855, 5115-5245) -----------
// _internUpload: a row past the authored ones (the next free row appends),
// rampInv baked, grav scaled by the gravity scale. Returns the table size or
// a negative code (-1 bad row id, -2 a product outside the table).
int sno_set_material(SnoEngine* e, uint32_t row, const int32_t* w) {
  if (row < e->authoredCount || row > e->matCount || row >= MAT_MAX) return -1;
  const uint32_t count = std::max(e->matCount, row + 1);
  for (int f : {M_meltTo, M_freezeTo, M_boilTo, M_condTo, M_burnTo, M_splitTo, M_corrTo})
    if (w[f] < 0 || (uint32_t)w[f] >= count) return -2;
  std::memcpy(e->matsAuth[row], w, sizeof(int32_t) * MAT_WORDS);
  const int64_t span = (int64_t)w[M_rampHi] - w[M_rampLo];
  e->matsAuth[row][M_rampInv] = span > 0 ? (int32_t)(4294967296LL / span) : 0;
  std::memcpy(e->mats[row], e->matsAuth[row], sizeof(int32_t) * MAT_WORDS);
  e->mats[row][M_grav] = (int32_t)idiv_rne64((int64_t)w[M_grav] * e->gravQ, 65536);
  e->matCount = count;
  return (int)count;
}
void sno_clear_materials(SnoEngine* e) {
  for (uint32_t m = e->authoredCount; m < MAT_MAX; ++m) {
    std::memset(e->mats[m], 0, sizeof(e->mats[m]));
    std::memset(e->matsAuth[m], 0, sizeof(e->matsAuth[m]));
  }
  e->matCount = e->authoredCount;
}
int32_t sno_set_gravity_scale(SnoEngine* e, int32_t q) {
  const int32_t qq = std::max(0, std::min(4 * 65536, q));
  e->gravQ = qq;
  for (uint32_t m = 0; m < e->matCount; ++m)
    e->mats[m][M_grav] = (int32_t)idiv_rne64((int64_t)e->matsAuth[m][M_grav] * qq, 65536);
  return qq;
}
uint32_t sno_mat_count(SnoEngine* e) { return e->matCount; }

}  // extern "C"
