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
// Scope: the fluid, friction, bond, thermal and formation passes. Rigid bodies
// (src/sim.wgsl section 20) and containment (section 29) are not restated;
// rows that would activate them are refused at load/spawn and a transition
// into one raises an error word (see `unsupported`).
//
// Parity is pinned by the reference's frozen dambreak_v1 chain
// (test/extraction_gate.md:62-68).
#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>
#include "fixed_ref.h"

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
  int32_t mats[MAT_MAX][MAT_WORDS];
  uint32_t matCount = 0;
  int threads = 1;
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
  // the loaded scene's boundary block, for spawnFluid's relocation
  std::vector<int32_t> scenePos, sceneTemp, sceneFuel;
  std::vector<uint32_t> sceneMat;
  uint32_t sceneNFluid = 0;
  bool sceneHasTemp = false, sceneHasFuel = false;

  Dbg D() { return Dbg{dbg}; }
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
// _nextWeldSeq (src/engine.js:4570-4580): the next tag sequence not held open.
inline uint32_t next_weld_seq(E& e) {
  const uint32_t MAXS = 4095;
  uint32_t q = (e.weldSeq % MAXS) + 1;
  for (uint32_t guard = 0; guard <= MAXS && q == e.weldHoldSeq; ++guard) q = (q % MAXS) + 1;
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

// src/sim.wgsl:1190-1254
void pass_buildNbr(E& e, const std::vector<Particle>& in) {
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
        }
      }
    }
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
    if (rigid_row(e.M(mat))) {
#ifdef _OPENMP
#pragma omp atomic
#endif
      e.unsupported |= 1u;
    }
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

// One substep, in _encodeSubstep's order (src/engine.js:4003-4155).
void substep(E& e) {
  std::vector<Particle>& in = e.st[e.parity];
  std::vector<Particle>& out = e.st[1 - e.parity];
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
  }
  pass_contain(e, in);
  pass_finalize(e, in, out);
  pass_xsph(e, out);
  pass_normals(e);
  pass_surfaceTension(e, out);
  pass_conduct(e, out);
  pass_thermal(e, out);
  pass_containStress(e, out);
  // rigidMember: inert (no rigid-body rows are admitted)
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
  e->matCount = matCount;
  std::memset(e->dbg, 0, sizeof(e->dbg));
  return e;
}

void sno_destroy(SnoEngine* e) { delete e; }

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
    if (rigid_row(e->mats[matId[i]])) return -9;
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
void sno_dbg(SnoEngine* e, uint32_t out[16]) { std::memcpy(out, e->dbg, sizeof(e->dbg)); }
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
  for (uint32_t i = 0; i < k; ++i) {
    const int32_t* r = rows + 8 * i;
    int32_t mm = r[4] < 0 ? 0 : r[4];
    uint32_t m = (uint32_t)std::min<int32_t>((int32_t)e->matCount - 1, mm);
    if (rigid_row(e->mats[m])) return -9;
  }
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

}  // extern "C"
