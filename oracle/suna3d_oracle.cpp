// ORACLE — test infrastructure only. Never linked into the product library.
//
// Scalar CPU restatement of SunaEngine's 3D solver, 3d/sim3d.wgsl (Jacobi PBF
// with half-space walls) driven as 3d/app.js drives it (predict, grid,
// canonical neighbour lists, iters x (density, solveDp, applyDp), integrate),
// plus its striped FNV-1a digest (3d/sim3d.wgsl:555-590) folded as
// 3d/app.js:717-744 does. The 3D path has no golden values in the reference,
// so this restatement is the parity anchor for it ("parity unpinned").
//
// Build-defined additions (no reference counterpart): a per-substep chain of
// the 2D engine's Murmur H_set/H_slot digest over each particle's 8 words
// [p.x, p.y, p.z, mat, v.x, v.y, v.z, 0], so the 3D path can be checked every
// substep like the 2D one; a per-substep stir phase; and bonds, the 2D
// engine's bond distance constraint (src/sim.wgsl:1594-1671, the bond gather
// of friction at :1880-1934) restated over three axes and added to solveDp's
// correction of each bonded particle (bond3 below).
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include "fixed_ref.h"

using namespace ofx;

namespace {

constexpr uint32_t MAXNBR = 48;
constexpr int32_t H = 131072;
constexpr int32_t H2Q = 262144;
constexpr uint32_t LUT_SHIFT = 7;
constexpr uint32_t OFF_W = 0, OFF_G = 2049, OFF_P = 4098, OFF_PG = 4611;
constexpr int32_t RHO0 = 1048576;
constexpr int32_t C_MAX = 1048576;
constexpr int32_t LAM_MAX = 4194304;
constexpr int32_t EPS_S = 524288;
constexpr uint32_t GRAD_S = 16, S_ACC_S = 16, LAM_S = 24, DP_S = 20;
constexpr int32_t S_TERM = 8388608;
constexpr int32_t MARGIN = 32768;
// bonds (build-defined): rows of 6 entries {partner + 1 | TOMB, L0}
constexpr uint32_t BOND3_CAP = 6, BOND3_WORDS = 12, BOND3_TOMB = 0x80000000u, BOND3_J = 0x7fffffffu;
constexpr uint32_t BOND3_PRE = 5;
constexpr int32_t BOND3_L0_MIN = 512, BOND3_L0_MAX = 5120, BOND3_HARD_BREAK2 = 26214400, BOND3_D2_FLOOR = 262144;
constexpr int32_t BOND3_TERM = 16777216, BOND3_DP_MAX = 16384;

struct V3 { int32_t x, y, z; };

struct P3 { V3 p; uint32_t mat; V3 v; V3 pr; int32_t lam; V3 dp; int32_t rho; };

}  // namespace

struct Sno3 {
  uint32_t maxN = 0, iters = 4;
  int threads = 1;
  std::vector<int32_t> luts;
  std::vector<int32_t> mats;  // rows of 4: grav, rhoW, damp, f0
  uint32_t matCount = 0;
  uint32_t n = 0, gx = 1, gy = 1, gz = 1, cellTotal = 1;
  int32_t stirAmp = 0;
  int32_t stirPhase = 0;  // fixed for one step() call, as the reference writes params once per batch
  uint32_t frame = 0;     // > 0: the phase is fixed per frame of `frame` substeps instead
  bool ballOn = false;
  V3 ballPos{0, 0, 0};
  int32_t ballReach = 0;
  std::vector<int32_t> ballW, ballG;  // 1024 each, indexed by r2q >> 12
  std::vector<P3> ps;
  std::vector<uint32_t> cellOf, cellStart, cellCount, sorted, nbr, nbrN;
  std::vector<uint32_t> bond;  // [maxN * BOND3_WORDS]
  int32_t bondK = 0, bondBrk = 0;
  uint32_t dbg[16];
  uint32_t chain[8];
  uint64_t substeps = 0;
  Dbg D() { return Dbg{dbg}; }
  int32_t grav(uint32_t m) const { return mats[m * 4 + 0]; }
  int32_t rhoW(uint32_t m) const { return mats[m * 4 + 1]; }
  int32_t damp(uint32_t m) const { return mats[m * 4 + 2]; }
  int32_t world_max(int axis) const { return (int32_t)(axis == 0 ? gx : axis == 1 ? gy : gz) * H; }
};

namespace {

#ifdef _OPENMP
#define PFOR3 _Pragma("omp parallel for schedule(static) num_threads(e.threads)")
#else
#define PFOR3
#endif

inline V3 clamp_world(const Sno3& e, V3 p) {
  return V3{clampi(p.x, MARGIN, e.world_max(0) - MARGIN), clampi(p.y, MARGIN, e.world_max(1) - MARGIN),
            clampi(p.z, MARGIN, e.world_max(2) - MARGIN)};
}
inline uint32_t cell_index(const Sno3& e, int32_t cx, int32_t cy, int32_t cz) {
  return ((uint32_t)cz * e.gy + (uint32_t)cy) * e.gx + (uint32_t)cx;
}

// wall_of (3d/sim3d.wgsl:127-141): distance to wall w and its signed gradient.
struct Wall { int32_t dist; V3 dir; };
inline Wall wall_of(const Sno3& e, V3 p, uint32_t w, int32_t gm, const Dbg& g) {
  uint32_t axis = w >> 1;
  bool hi = (w & 1u) == 1u;
  int32_t pos = axis == 0 ? p.x : (axis == 1 ? p.y : p.z);
  int32_t d = hi ? wsub(e.world_max((int)axis), pos) : pos;
  int32_t s = hi ? gm : fp_neg_sat(gm, g);  // select(neg, gm, hi): both arms evaluated
  if (hi) (void)fp_neg_sat(gm, g);
  V3 dir{0, 0, 0};
  if (axis == 0) dir.x = s; else if (axis == 1) dir.y = s; else dir.z = s;
  return Wall{std::max(d, 0), dir};
}

// predict (3d/sim3d.wgsl:188-215)
void predict3(Sno3& e) {
  int32_t phase = e.stirPhase;
  PFOR3 for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    Dbg g = e.D();
    P3& q = e.ps[ii];
    V3 v = q.v;
    v.y = fp_sub_sat(v.y, e.grav(q.mat), g);
    if (e.stirAmp != 0) {
      int32_t t0 = ((phase + 32768) & 131071) - 65536;
      int32_t tri = (t0 < 0 ? -t0 : t0) - 32768;
      v.x = fp_add_sat(v.x, fp_mul_s(tri, e.stirAmp, 16, g), g);
    }
    int32_t dm = e.damp(q.mat);
    v = V3{fp_mul_s(v.x, dm, 16, g), fp_mul_s(v.y, dm, 16, g), fp_mul_s(v.z, dm, 16, g)};
    q.pr = clamp_world(e, V3{fp_add_sat(q.p.x, v.x, g), fp_add_sat(q.p.y, v.y, g), fp_add_sat(q.p.z, v.z, g)});
    q.lam = 0;
    q.v = v;
  }
}

// gridCount .. canonicalize (3d/sim3d.wgsl:229-334): canonical ascending id per cell.
void grid3(Sno3& e) {
  std::fill(e.cellCount.begin(), e.cellCount.end(), 0u);
  for (uint32_t i = 0; i < e.n; ++i) {
    const V3& p = e.ps[i].pr;
    uint32_t c = cell_index(e, p.x / H, p.y / H, p.z / H);
    e.cellOf[i] = c;
    e.cellCount[c]++;
  }
  uint32_t run = 0;
  for (uint32_t c = 0; c < e.cellTotal; ++c) { e.cellStart[c] = run; run += e.cellCount[c]; }
  e.cellStart[e.cellTotal] = e.n;
  std::fill(e.cellCount.begin(), e.cellCount.end(), 0u);
  for (uint32_t i = 0; i < e.n; ++i) {
    uint32_t c = e.cellOf[i];
    e.sorted[e.cellStart[c] + e.cellCount[c]++] = i;
  }
}

// buildNbr (3d/sim3d.wgsl:341-390)
void nbr3(Sno3& e) {
  PFOR3 for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    V3 pi = e.ps[i].pr;
    int32_t cx0 = pi.x / H, cy0 = pi.y / H, cz0 = pi.z / H;
    uint32_t base = i * MAXNBR, cnt = 0;
    for (int dz = -1; dz <= 1; ++dz) {
      int32_t cz = cz0 + dz;
      if (cz < 0 || cz >= (int32_t)e.gz) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        int32_t cy = cy0 + dy;
        if (cy < 0 || cy >= (int32_t)e.gy) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          int32_t cx = cx0 + dx;
          if (cx < 0 || cx >= (int32_t)e.gx) continue;
          uint32_t cc = cell_index(e, cx, cy, cz);
          for (uint32_t s = e.cellStart[cc]; s < e.cellStart[cc + 1]; ++s) {
            uint32_t j = e.sorted[s];
            if (j == i) continue;
            const V3& pj = e.ps[j].pr;
            V3 d{wsub(pj.x, pi.x), wsub(pj.y, pi.y), wsub(pj.z, pi.z)};
            if (fp_abs(d.x, g) >= H || fp_abs(d.y, g) >= H || fp_abs(d.z, g) >= H) continue;
            int32_t qx = d.x >> 8, qy = d.y >> 8, qz = d.z >> 8;
            int32_t r2q = wadd(wadd(wmul(qx, qx), wmul(qy, qy)), wmul(qz, qz));
            if (r2q >= H2Q) continue;
            if (cnt >= MAXNBR) { g.flag(6); continue; }
            e.nbr[base + cnt++] = j;
          }
        }
      }
    }
    e.nbrN[i] = cnt;
  }
}

inline int32_t s_term(int32_t a, const Dbg& g) { return clampi(fp_mul_s(a, a, S_ACC_S, g), 0, S_TERM); }

// ball_term (3d/sim3d.wgsl:154-176): the cursor sphere, a table indexed by the
// centre distance squared.
constexpr int32_t BALL_R2MAX = 4194304;
struct Ball { bool hit; int32_t w; V3 g; };
inline Ball ball_term(const Sno3& e, V3 pi, const Dbg& g) {
  Ball t{false, 0, {0, 0, 0}};
  if (!e.ballOn) return t;
  V3 dc{wsub(e.ballPos.x, pi.x), wsub(e.ballPos.y, pi.y), wsub(e.ballPos.z, pi.z)};
  if (fp_abs(dc.x, g) >= e.ballReach || fp_abs(dc.y, g) >= e.ballReach || fp_abs(dc.z, g) >= e.ballReach) return t;
  int32_t qx = dc.x >> 8, qy = dc.y >> 8, qz = dc.z >> 8;
  int32_t r2q = wadd(wadd(wmul(qx, qx), wmul(qy, qy)), wmul(qz, qz));
  if (r2q >= BALL_R2MAX) return t;
  uint32_t bi = (uint32_t)r2q >> 12;
  int32_t gt = e.ballG[bi];
  t.hit = true;
  t.w = e.ballW[bi];
  t.g = V3{fp_mul_s(gt, dc.x, GRAD_S, g), fp_mul_s(gt, dc.y, GRAD_S, g), fp_mul_s(gt, dc.z, GRAD_S, g)};
  return t;
}

// density (3d/sim3d.wgsl:397-468), ball off
void density3(Sno3& e) {
  PFOR3 for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    P3& q = e.ps[i];
    V3 pi = q.pr;
    uint32_t cnt = e.nbrN[i], base = i * MAXNBR;
    int32_t rho = wmul(e.luts[OFF_W], 256 + e.rhoW(q.mat)) >> 8;
    int32_t S = 0;
    V3 sg{0, 0, 0};
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      const V3& pj = e.ps[j].pr;
      V3 d{wsub(pj.x, pi.x), wsub(pj.y, pi.y), wsub(pj.z, pi.z)};
      int32_t qx = d.x >> 8, qy = d.y >> 8, qz = d.z >> 8;
      int32_t r2q = wadd(wadd(wmul(qx, qx), wmul(qy, qy)), wmul(qz, qz));
      if (r2q >= H2Q) continue;
      uint32_t ui = (uint32_t)r2q >> LUT_SHIFT;
      rho = wadd(rho, wmul(e.luts[OFF_W + ui], 256 + e.rhoW(e.ps[j].mat)) >> 8);
      int32_t gt = e.luts[OFF_G + ui];
      V3 gv{fp_mul_s(gt, d.x, GRAD_S, g), fp_mul_s(gt, d.y, GRAD_S, g), fp_mul_s(gt, d.z, GRAD_S, g)};
      sg = V3{wadd(sg.x, gv.x), wadd(sg.y, gv.y), wadd(sg.z, gv.z)};
      S = wadd(S, wadd(wadd(s_term(gv.x, g), s_term(gv.y, g)), s_term(gv.z, g)));
    }
    for (uint32_t w = 0; w < 6; ++w) {
      Wall probe = wall_of(e, pi, w, 0, g);
      if (probe.dist >= H) continue;
      uint32_t b = (uint32_t)probe.dist >> 8;
      rho = wadd(rho, e.luts[OFF_P + b]);
      V3 gv = wall_of(e, pi, w, e.luts[OFF_PG + b], g).dir;
      sg = V3{wadd(sg.x, gv.x), wadd(sg.y, gv.y), wadd(sg.z, gv.z)};
      S = wadd(S, wadd(wadd(s_term(gv.x, g), s_term(gv.y, g)), s_term(gv.z, g)));
    }
    Ball bt = ball_term(e, pi, g);
    if (bt.hit) {
      rho = wadd(rho, bt.w);
      sg = V3{wadd(sg.x, bt.g.x), wadd(sg.y, bt.g.y), wadd(sg.z, bt.g.z)};
      S = wadd(S, wadd(wadd(s_term(bt.g.x, g), s_term(bt.g.y, g)), s_term(bt.g.z, g)));
    }
    S = wadd(S, wadd(wadd(s_term(sg.x, g), s_term(sg.y, g)), s_term(sg.z, g)));
    int32_t Cq = clampi(fp_shr_rne(wsub(rho, RHO0), 4), 0, C_MAX);
    q.rho = rho;
    q.lam = clampi(fp_neg_sat(fp_divshift(Cq, wadd(S, EPS_S), LAM_S, g), g), fp_neg_sat(LAM_MAX, g), LAM_MAX);
  }
}

inline int32_t iabs3(int32_t x) { return x < 0 ? (int32_t)(0u - (uint32_t)x) : x; }

// A bonded particle's correction from the iteration's starting positions,
// its row walked in order. Per bond: d4 = (p_i - p_j) >> 5 (round half even);
// a bond whose ends are too far apart is tombstoned in this end's row (the
// test is symmetric, so the other end drops its copy in the same pass);
// C = |d4|^2 - L0^2, q = C / (4 |d4|^2) in Q16 (the solver divide), and each
// axis sums -clamp(d4 * (q * k >> 16) >> 3). The 2D constraint, src/sim.wgsl:
// 1880-1934, with the material stiffness replaced by the scene's.
V3 bond3(Sno3& e, uint32_t i, V3 pi, const Dbg& g) {
  uint32_t* row = e.bond.data() + (size_t)i * BOND3_WORDS;
  int32_t bx = 0, by = 0, bz = 0;
  for (uint32_t k = 0; k < BOND3_CAP; ++k) {
    const uint32_t w = row[2 * k];
    if (w == 0u) break;
    if (w & BOND3_TOMB) continue;
    const int32_t L0 = (int32_t)row[2 * k + 1];
    const int32_t L02 = wmul(L0, L0);
    const V3& pj = e.ps[(w & BOND3_J) - 1u].pr;
    const int32_t d4x = fp_shr_rne(fp_sub_sat(pi.x, pj.x, g), BOND3_PRE);
    const int32_t d4y = fp_shr_rne(fp_sub_sat(pi.y, pj.y, g), BOND3_PRE);
    const int32_t d4z = fp_shr_rne(fp_sub_sat(pi.z, pj.z, g), BOND3_PRE);
    if (iabs3(d4x) > BOND3_L0_MAX || iabs3(d4y) > BOND3_L0_MAX || iabs3(d4z) > BOND3_L0_MAX) {
      row[2 * k] = w | BOND3_TOMB;
      continue;
    }
    const int32_t d2 = wadd(wadd(wmul(d4x, d4x), wmul(d4y, d4y)), wmul(d4z, d4z));
    if (d2 >= BOND3_HARD_BREAK2 || (e.bondBrk != 0 && d2 > fp_mul_s(L02, e.bondBrk, 16u, g))) {
      row[2 * k] = w | BOND3_TOMB;
      continue;
    }
    if (d2 < BOND3_D2_FLOOR) continue;
    const int32_t C = fp_sub_sat(d2, L02, g);
    const int32_t q = fp_divshift(C, wmul(d2, 4), 16u, g);
    const int32_t qk = fp_mul_s(q, e.bondK, 16u, g);
    bx = wsub(bx, clampi(fp_mul_s(d4x, qk, 3u, g), -BOND3_TERM, BOND3_TERM));
    by = wsub(by, clampi(fp_mul_s(d4y, qk, 3u, g), -BOND3_TERM, BOND3_TERM));
    bz = wsub(bz, clampi(fp_mul_s(d4z, qk, 3u, g), -BOND3_TERM, BOND3_TERM));
  }
  return V3{clampi(fp_shr_rne(bx, 8u), -BOND3_DP_MAX, BOND3_DP_MAX), clampi(fp_shr_rne(by, 8u), -BOND3_DP_MAX, BOND3_DP_MAX),
            clampi(fp_shr_rne(bz, 8u), -BOND3_DP_MAX, BOND3_DP_MAX)};
}

// solveDp + applyDp (3d/sim3d.wgsl:476-537): gather with a saturating running
// sum in canonical neighbour order, then the walls, the ball and (build-
// defined) the bonds, then apply.
void solve3(Sno3& e) {
  PFOR3 for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    uint32_t i = (uint32_t)ii;
    Dbg g = e.D();
    P3& q = e.ps[i];
    V3 pi = q.pr;
    int32_t lami = q.lam;
    uint32_t cnt = e.nbrN[i], base = i * MAXNBR;
    V3 acc{0, 0, 0};
    for (uint32_t k = 0; k < cnt; ++k) {
      uint32_t j = e.nbr[base + k];
      const V3& pj = e.ps[j].pr;
      V3 d{wsub(pj.x, pi.x), wsub(pj.y, pi.y), wsub(pj.z, pi.z)};
      int32_t qx = d.x >> 8, qy = d.y >> 8, qz = d.z >> 8;
      int32_t r2q = wadd(wadd(wmul(qx, qx), wmul(qy, qy)), wmul(qz, qz));
      if (r2q >= H2Q) continue;
      uint32_t ui = (uint32_t)r2q >> LUT_SHIFT;
      int32_t gt = e.luts[OFF_G + ui];
      V3 gv{fp_mul_s(gt, d.x, GRAD_S, g), fp_mul_s(gt, d.y, GRAD_S, g), fp_mul_s(gt, d.z, GRAD_S, g)};
      int32_t lsum = fp_add_sat(lami, e.ps[j].lam, g);
      acc = V3{fp_add_sat(acc.x, fp_mul_s(lsum, gv.x, DP_S, g), g), fp_add_sat(acc.y, fp_mul_s(lsum, gv.y, DP_S, g), g),
               fp_add_sat(acc.z, fp_mul_s(lsum, gv.z, DP_S, g), g)};
    }
    for (uint32_t w = 0; w < 6; ++w) {
      Wall probe = wall_of(e, pi, w, 0, g);
      if (probe.dist >= H) continue;
      uint32_t b = (uint32_t)probe.dist >> 8;
      V3 gv = wall_of(e, pi, w, e.luts[OFF_PG + b], g).dir;
      acc = V3{fp_add_sat(acc.x, fp_mul_s(lami, gv.x, DP_S, g), g), fp_add_sat(acc.y, fp_mul_s(lami, gv.y, DP_S, g), g),
               fp_add_sat(acc.z, fp_mul_s(lami, gv.z, DP_S, g), g)};
    }
    Ball bt = ball_term(e, pi, g);
    if (bt.hit)
      acc = V3{fp_add_sat(acc.x, fp_mul_s(lami, bt.g.x, DP_S, g), g), fp_add_sat(acc.y, fp_mul_s(lami, bt.g.y, DP_S, g), g),
               fp_add_sat(acc.z, fp_mul_s(lami, bt.g.z, DP_S, g), g)};
    if (!e.bond.empty() && e.bond[(size_t)i * BOND3_WORDS] != 0u) {
      const V3 bd = bond3(e, i, pi, g);
      acc = V3{fp_add_sat(acc.x, bd.x, g), fp_add_sat(acc.y, bd.y, g), fp_add_sat(acc.z, bd.z, g)};
    }
    q.dp = acc;
  }
  PFOR3 for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    Dbg g = e.D();
    P3& q = e.ps[ii];
    q.pr = clamp_world(e, V3{fp_add_sat(q.pr.x, q.dp.x, g), fp_add_sat(q.pr.y, q.dp.y, g),
                             fp_add_sat(q.pr.z, q.dp.z, g)});
  }
}

// integrate (3d/sim3d.wgsl:542-552)
void integrate3(Sno3& e) {
  PFOR3 for (int64_t ii = 0; ii < (int64_t)e.n; ++ii) {
    Dbg g = e.D();
    P3& q = e.ps[ii];
    q.v = V3{fp_sub_sat(q.pr.x, q.p.x, g), fp_sub_sat(q.pr.y, q.p.y, g), fp_sub_sat(q.pr.z, q.p.z, g)};
    q.p = q.pr;
  }
}

// Murmur digest over [p.x, p.y, p.z, mat, v.x, v.y, v.z, 0] (the 2D engine's
// statehash lanes, src/hash/statehash.js:80-159, applied to the 3D words).
constexpr uint32_t SEED[4] = {0x9e3779b1u, 0x85ebca77u, 0xc2b2ae3du, 0x27d4eb2fu};
constexpr uint32_t SALT[4] = {0x00000000u, 0x51633e2du, 0x9c8f2a17u, 0xd0e5b943u};
constexpr uint32_t CHAIN_INIT[8] = {0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u,
                                    0xa4093822u, 0x299f31d0u, 0x082efa98u, 0xec4e6c89u};
inline uint32_t rotl(uint32_t x, uint32_t r) { return (x << r) | (x >> ((32 - r) & 31)); }
inline uint32_t mm(uint32_t h, uint32_t k) {
  k *= 0xcc9e2d51u; k = rotl(k, 15); k *= 0x1b873593u;
  h ^= k; h = rotl(h, 13); return h * 5u + 0xe6546b64u;
}
inline uint32_t fmix(uint32_t h) {
  h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16; return h;
}
void words3(const P3& q, uint32_t w[8]) {
  w[0] = (uint32_t)q.p.x; w[1] = (uint32_t)q.p.y; w[2] = (uint32_t)q.p.z; w[3] = q.mat;
  w[4] = (uint32_t)q.v.x; w[5] = (uint32_t)q.v.y; w[6] = (uint32_t)q.v.z; w[7] = 0;
}
void murmur3(const Sno3& e, uint32_t acc[8]) {
  for (int l = 0; l < 8; ++l) acc[l] = 0;
  for (uint32_t i = 0; i < e.n; ++i) {
    uint32_t w[8];
    words3(e.ps[i], w);
    uint32_t h[4] = {SEED[0], SEED[1], SEED[2], SEED[3]};
    for (int k = 0; k < 8; ++k)
      for (int l = 0; l < 4; ++l) h[l] = mm(h[l], w[k] ^ SALT[l]);
    for (int l = 0; l < 4; ++l) {
      acc[l] += fmix(h[l] ^ 8u);
      acc[4 + l] += fmix(mm(h[l], i) ^ 9u);
    }
  }
}
void fold(uint32_t chain[8], const uint32_t a[8]) {
  uint32_t nx[8];
  for (int j = 0; j < 8; ++j) nx[j] = mm(chain[j], a[j] ^ rotl(a[(j + 1) & 7], 7));
  std::memcpy(chain, nx, sizeof(nx));
}

}  // namespace

extern "C" {

Sno3* sno3_create(uint32_t maxN, const int32_t* luts, uint32_t lutWords, const int32_t* mats, uint32_t matCount,
                  uint32_t iters, int threads) {
  Sno3* e = new Sno3();
  e->maxN = maxN;
  e->iters = iters;
  e->threads = threads < 1 ? 1 : threads;
  e->luts.assign(luts, luts + lutWords);
  e->mats.assign(mats, mats + 4 * matCount);
  e->matCount = matCount;
  std::memset(e->dbg, 0, sizeof(e->dbg));
  return e;
}
void sno3_destroy(Sno3* e) { delete e; }

int sno3_load(Sno3* e, uint32_t n, const int32_t* pos, const int32_t* vel, const uint32_t* mat, uint32_t gx,
              uint32_t gy, uint32_t gz, int32_t stirAmp, uint32_t frame) {
  if (n > e->maxN || gx == 0 || gy == 0 || gz == 0) return -1;
  e->n = n; e->gx = gx; e->gy = gy; e->gz = gz; e->cellTotal = gx * gy * gz;
  e->bond.clear();
  e->bondK = e->bondBrk = 0;
  e->stirAmp = stirAmp;
  e->frame = frame;
  e->ps.assign(n, P3{});
  for (uint32_t i = 0; i < n; ++i) {
    if (mat[i] >= e->matCount) return -2;
    P3& q = e->ps[i];
    q.p = V3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    q.v = V3{vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
    q.mat = mat[i];
    q.pr = q.p;
  }
  e->cellOf.assign(n, 0);
  e->cellStart.assign(e->cellTotal + 1, 0);
  e->cellCount.assign(e->cellTotal, 0);
  e->sorted.assign(n, 0);
  e->nbr.assign((size_t)n * MAXNBR, 0);
  e->nbrN.assign(n, 0);
  e->substeps = 0;
  std::memset(e->dbg, 0, sizeof(e->dbg));
  std::memcpy(e->chain, CHAIN_INIT, sizeof(e->chain));
  return 0;
}

int sno3_step(Sno3* e, uint32_t count) {
  e->stirPhase = (int32_t)((e->substeps * 384) & 131071);
  for (uint32_t s = 0; s < count; ++s) {
    if (e->frame) e->stirPhase = (int32_t)(((e->substeps - e->substeps % e->frame) * 384) & 131071);
    predict3(*e);
    grid3(*e);
    nbr3(*e);
    for (uint32_t it = 0; it < e->iters; ++it) {
      density3(*e);
      solve3(*e);
    }
    integrate3(*e);
    e->substeps++;
    uint32_t a[8];
    murmur3(*e, a);
    fold(e->chain, a);
  }
  return 0;
}

// digestStripe + the host fold (3d/sim3d.wgsl:555-590, 3d/app.js:717-744).
void sno3_fnv(Sno3* e, uint32_t out[8]) {
  uint32_t words[256];
  uint32_t per = (e->n + 255) / 256;
  for (uint32_t k = 0; k < 256; ++k) {
    uint32_t lo = k * per, hi = std::min(e->n, lo + per);
    uint32_t h = 2166136261u;
    for (uint32_t i = lo; i < hi; ++i) {
      const P3& q = e->ps[i];
      uint32_t vals[6] = {(uint32_t)q.p.x, (uint32_t)q.p.y, (uint32_t)q.p.z,
                          (uint32_t)q.v.x, (uint32_t)q.v.y, (uint32_t)q.v.z};
      for (uint32_t w : vals)
        for (int b = 0; b < 4; ++b) h = (h ^ ((w >> (8 * b)) & 0xffu)) * 16777619u;
    }
    words[k] = h;
  }
  for (uint32_t L = 0; L < 8; ++L) out[L] = 2166136261u ^ (L * 0x9e3779b9u);
  for (uint32_t k = 0; k < 256; ++k)
    for (uint32_t L = 0; L < 8; ++L) {
      uint32_t h = out[L] ^ words[k];
      h = h * 16777619u;
      h = h ^ (h >> 13);
      out[L] = h;
    }
}
// spawn (3d/app.js:575-597): append k particles (positions from the host,
// velocity zero) past the live count; refused past capacity.
uint32_t sno3_spawn(Sno3* e, const int32_t* pos, const uint32_t* mat, uint32_t k) {
  uint32_t room = e->maxN - e->n;
  if (k > room) k = room;
  for (uint32_t i = 0; i < k; ++i) {
    if (mat[i] >= e->matCount) return 0;
  }
  for (uint32_t i = 0; i < k; ++i) {
    P3 q{};
    q.p = V3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    q.mat = mat[i];
    e->ps.push_back(q);
  }
  e->n += k;
  e->cellOf.assign(e->n, 0);
  e->sorted.assign(e->n, 0);
  e->nbr.assign((size_t)e->n * MAXNBR, 0);
  e->nbrN.assign(e->n, 0);
  return k;
}
void sno3_set_ball(Sno3* e, int on, int32_t x, int32_t y, int32_t z, int32_t reach, const int32_t* w1024,
                   const int32_t* g1024) {
  e->ballOn = on != 0;
  e->ballPos = V3{x, y, z};
  e->ballReach = reach;
  e->ballW.assign(w1024, w1024 + 1024);
  e->ballG.assign(g1024, g1024 + 1024);
}
uint32_t sno3_n(Sno3* e) { return e->n; }
// Build-defined bonds: n * 12 words of rows (see bond3), the scene's stiffness
// (Q16) and break ratio; replaces all rows. -1 on a malformed row.
int sno3_write_bonds(Sno3* e, const uint32_t* rows, size_t words, int32_t k, int32_t brk) {
  if (words != (size_t)e->n * BOND3_WORDS || k < 0 || k > 65536 || brk < 0) return -1;
  for (uint32_t i = 0; i < e->n; ++i)
    for (uint32_t t = 0; t < BOND3_CAP; ++t) {
      const uint32_t w = rows[(size_t)i * BOND3_WORDS + 2 * t], L0 = rows[(size_t)i * BOND3_WORDS + 2 * t + 1];
      if (w == 0u) continue;
      const uint32_t j = (w & BOND3_J) - 1u;
      if (j >= e->n || j == i || (int32_t)L0 < BOND3_L0_MIN || (int32_t)L0 > BOND3_L0_MAX) return -1;
    }
  e->bond.assign((size_t)e->maxN * BOND3_WORDS, 0u);
  std::memcpy(e->bond.data(), rows, words * 4);
  e->bondK = k;
  e->bondBrk = brk;
  return 0;
}
int sno3_read_bonds(Sno3* e, uint32_t* out, size_t words) {
  if (words < (size_t)e->n * BOND3_WORDS) return -1;
  if (e->bond.empty()) std::memset(out, 0, (size_t)e->n * BOND3_WORDS * 4);
  else std::memcpy(out, e->bond.data(), (size_t)e->n * BOND3_WORDS * 4);
  return 0;
}
int sno3_write_state(Sno3* e, const int32_t* words, uint32_t n, uint64_t substeps, const uint32_t* chain) {
  if (n > e->maxN) return -1;
  e->ps.assign(n, P3{});
  for (uint32_t i = 0; i < n; ++i) {
    const int32_t* w = words + 8 * (size_t)i;
    P3& q = e->ps[i];
    q.p = V3{w[0], w[1], w[2]};
    q.mat = (uint32_t)w[3];
    q.v = V3{w[4], w[5], w[6]};
    q.pr = q.p;
  }
  e->n = n;
  e->cellOf.assign(n, 0);
  e->sorted.assign(n, 0);
  e->nbr.assign((size_t)n * MAXNBR, 0);
  e->nbrN.assign(n, 0);
  e->substeps = substeps;
  if (chain) std::memcpy(e->chain, chain, 32);
  return 0;
}
uint64_t sno3_substeps(Sno3* e) { return e->substeps; }
void sno3_digest(Sno3* e, uint32_t acc[8]) { murmur3(*e, acc); }
void sno3_chain(Sno3* e, uint32_t c[8]) { std::memcpy(c, e->chain, 32); }
void sno3_dbg(Sno3* e, uint32_t out[16]) { std::memcpy(out, e->dbg, 64); }
int sno3_read_state(Sno3* e, int32_t* out, size_t words) {
  if (words < (size_t)e->n * 8) return -1;
  for (uint32_t i = 0; i < e->n; ++i) words3(e->ps[i], reinterpret_cast<uint32_t*>(out + 8 * (size_t)i));
  return 0;
}

}  // extern "C"
