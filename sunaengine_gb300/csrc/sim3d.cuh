// Device kernels of the 3D solver on sm_103a.
//
// Semantics are those of the reference's 3D Jacobi PBF (3d/sim3d.wgsl:188-552,
// driven by 3d/app.js:672-698): predict, grid, canonical neighbour lists,
// ITERS x (density, solveDp, applyDp), integrate; plus the 2D engine's Murmur
// state hash applied to each particle's 8 words [p.xyz, mat, v.xyz, 0] once per
// substep, folded into a per-scene chain.
//
// Layout (the reference keeps one 64-byte AoS record per particle and an index
// buffer; here the state is slot order and the solver runs in sorted space):
//   state[slot]  = {p.x, p.y, p.z, mat, v.x, v.y, v.z, 0}           32 B, slot order
//   PRS[slot]    = {pr.x, pr.y, pr.z, tag}                           predict output
//   PW[s], PW2[s]= {pr.x, pr.y, pr.z, tag}   sorted space, ping-pong across iterations
//   PL[s]        = {pr.x, pr.y, pr.z, lambda}                        density output
//   tag          = (256 + rhoW(mat)) | scene << 12  (the volume-claim weight and the scene)
//   NBR[k][s]    = sorted index of neighbour k (column-major, coalesced across s)
// Sorted space is all scenes' particles ordered by (scene key offset + cell,
// slot): the stable radix sort of slot-ordered keys leaves every cell in
// ascending particle id, which is the reference's canonical order (its
// `canonicalize` pass, 3d/sim3d.wgsl:296-334), and cells (cx-1, cx, cx+1) are
// adjacent keys, so each (dz, dy) row of the 3x3x3 stencil is one contiguous
// run of sorted indices in the reference's dz, dy, dx, ascending-id order.
//
// solveDp accumulates with a saturating add (order dependent); see k3_solve
// for how the sum stays exact under a lane split.
//
// Range facts used by the release build (debug builds keep every saturation
// test so the debug counters match the reference's fp_flag counts): positions
// are clamped into [MARGIN, 52 * H - MARGIN], so coordinate differences fit
// easily and the wrapping r2q of any in-world pair is non-negative; a pair
// that passes r2q < H2Q has |d| < H = 2^17 on every axis (so the reference's
// per-axis reject is implied); |G| < 2^24, so a gradient term G*d >> 16 is
// below 2^25 and never saturates; its square may, and is clamped at once into
// [0, S_TERM]; |lambda| <= 2^22, so lambda_i + lambda_j never saturates and
// (lambda sum) * gradient >> 20 is below 2^28.
#pragma once
#include <cstdint>
#include "fixed.cuh"
#include "statehash.cuh"

namespace sn {
namespace d3 {

constexpr uint32_t MAXNBR = 48;
constexpr int32_t H = 131072;          // smoothing radius and cell edge, 2 wu
constexpr int HSHIFT = 17;             // H == 1 << 17
constexpr int32_t H2Q = 262144;        // (H >> 8)^2
constexpr int LUT_N = 2049, PLANE_N = 513, BALL_N = 1024;
constexpr int LUT_WORDS = 2 * LUT_N + 2 * PLANE_N;
constexpr int32_t RHO0 = 1048576, C_MAX = 1048576, LAM_MAX = 4194304, EPS_S = 524288;
constexpr int32_t S_TERM = 8388608, MARGIN = 32768, BALL_R2MAX = 4194304;
constexpr uint32_t TAG_W = 0xfffu, TAG_SHIFT = 12;
constexpr uint32_t TAG_BONDED = 0x80000000u;  // the particle's slot has a bond row
constexpr uint32_t TAG_SCENE = 0x7ffffu;      // (tag >> TAG_SHIFT) & TAG_SCENE = scene
__device__ __forceinline__ uint32_t scene_of_tag(uint32_t tag) { return (tag >> TAG_SHIFT) & TAG_SCENE; }

// Bonds (build-defined; the reference's 3D page has none): the 2D engine's
// bond distance constraint (src/sim.wgsl:1594-1671, the bond gather of
// friction at :1880-1934) restated over three axes. Each slot has a row of
// BOND3_CAP entries of two words, {partner + 1 | BOND3_TOMB, L0}: the partner's
// scene-local index plus one (0 ends the row), and the rest length in ticks
// >> 5. A bond is stored in both ends' rows.
constexpr uint32_t BOND3_CAP = 6, BOND3_WORDS = 2 * BOND3_CAP;
constexpr uint32_t BOND3_TOMB = 0x80000000u, BOND3_J = 0x7fffffffu;
constexpr int BOND3_PRE = 5;               // d4 = d >> 5 (round half even)
constexpr int32_t BOND3_L0_MIN = 512, BOND3_L0_MAX = 5120;
constexpr int32_t BOND3_HARD_BREAK2 = 26214400;  // L0_MAX^2
constexpr int32_t BOND3_D2_FLOOR = 262144;
constexpr int32_t BOND3_TERM = 16777216;
constexpr int32_t BOND3_DP_MAX = 16384;    // a bond moves a particle at most 1/4 wu per iteration
constexpr uint32_t NO_SCENE = 0xffffffffu;
constexpr uint32_t MAX_AXIS_CELLS = 52;  // keeps the reference's wrapping r2q of any in-world pair non-negative

struct Scene3 {
  uint32_t slotBase, cap, n, keyOff;
  uint32_t gx, gy, gz, cellTotal;
  int32_t wmax[3];
  int32_t stirPhase, stirAmp;
  uint32_t ballOn;
  int32_t ball[3];
  int32_t reach;
  uint32_t active;
  uint32_t substep;  // this scene's substep counter (low 32 bits), advanced by k3_fold
  uint32_t frame;    // 0: stir phase fixed per step call; F > 0: fixed per frame of F substeps
  int32_t bondK;     // bond stiffness, Q16 (0..65536)
  int32_t bondBrk;   // a bond breaks when d^2 > L0^2 * bondBrk / 2^16 (0: never, by ratio)
  uint32_t pad[3];
};

struct World3 {
  uint32_t numScenes, K, slotEnd, nAct;
};

struct Bufs3 {
  int32_t* state;
  uint32_t* sceneOf;
  uint32_t* bond;     // [cap * BOND3_WORDS] bond rows, slot order
  uint32_t* bflag;    // [cap] 1 when the slot's row holds an entry
  uint32_t* inv;      // [cap] slot -> sorted position (this substep)
  int4* PRS;
  uint32_t *keys, *skey, *sslot, *cellStart;
  int4 *PW, *PW2, *PL;
  uint32_t *NBR, *NBRN;
  uint32_t nbrStride;
  const int2* WG;     // {W, G}, 2049
  const int2* PG;     // {planeW, planeG}, 513
  const int2* BALL;   // per scene {w, g}, 1024
  const int32_t* mats;
  const uint16_t* rcp;
  Scene3* scenes;
  World3* world;
  uint32_t *acc, *accLast, *chain, *dbg;
};

__device__ __forceinline__ uint32_t gstride3() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ uint32_t gtid3() { return blockIdx.x * blockDim.x + threadIdx.x; }

__device__ __forceinline__ int32_t wall_max(const Scene3& S, int axis) { return S.wmax[axis]; }

__device__ __forceinline__ int3 clamp_world(const Scene3& S, int32_t x, int32_t y, int32_t z) {
  return make_int3(clampi(x, MARGIN, S.wmax[0] - MARGIN), clampi(y, MARGIN, S.wmax[1] - MARGIN),
                   clampi(z, MARGIN, S.wmax[2] - MARGIN));
}

// Squared distance in reduced units with the reference's wrapping i32
// arithmetic. Scenes are at most MAX_AXIS_CELLS cells per axis, so for any two
// in-world points the sum stays below 2^31 and is never negative.
__device__ __forceinline__ int32_t r2q_of(int32_t dx, int32_t dy, int32_t dz) {
  int32_t qx = dx >> 8, qy = dy >> 8, qz = dz >> 8;
  return wadd(wadd(wmul(qx, qx), wmul(qy, qy)), wmul(qz, qz));
}

template <bool DBG>
__device__ __forceinline__ int32_t s_term(int32_t a, const Flags<DBG>& f) {
  return clampi(mul<16>(a, a, f), 0, S_TERM);
}

// The cursor ball (ball_term, 3d/sim3d.wgsl:154-176).
template <bool DBG>
__device__ __forceinline__ bool ball_term(const Bufs3& b, const Scene3& S, uint32_t sc, int32_t px, int32_t py,
                                          int32_t pz, int32_t& w, int3& g, const Flags<DBG>& f) {
  if (S.ballOn != 1u) return false;
  int32_t dx = wsub(S.ball[0], px), dy = wsub(S.ball[1], py), dz = wsub(S.ball[2], pz);
  if (abs_sat(dx, f) >= S.reach || abs_sat(dy, f) >= S.reach || abs_sat(dz, f) >= S.reach) return false;
  int32_t r2q = r2q_of(dx, dy, dz);
  if (r2q >= BALL_R2MAX) return false;
  int2 t = __ldg(b.BALL + (size_t)sc * BALL_N + ((uint32_t)r2q >> 12));
  w = t.x;
  g = make_int3(mul<16>(t.y, dx, f), mul<16>(t.y, dy, f), mul<16>(t.y, dz, f));
  return true;
}

// predict (3d/sim3d.wgsl:188-215) and the grid key of the predicted position.
template <bool DBG>
__global__ void __launch_bounds__(256) k3_predict(Bufs3 b) {
  const World3 W = *b.world;
  Flags<DBG> f{b.dbg};
  for (uint32_t slot = gtid3(); slot < W.slotEnd; slot += gstride3()) {
    uint32_t sc = b.sceneOf[slot];
    if (sc == NO_SCENE) { b.keys[slot] = W.K; continue; }
    const Scene3& S = b.scenes[sc];
    if (slot - S.slotBase >= S.n) { b.keys[slot] = W.K; continue; }
    const int4* w4 = reinterpret_cast<const int4*>(b.state + (size_t)slot * 8);
    int4 p = w4[0], v4 = w4[1];
    uint32_t m = (uint32_t)p.w;
    const int32_t grav = __ldg(b.mats + m * 4 + 0), rhoW = __ldg(b.mats + m * 4 + 1), damp = __ldg(b.mats + m * 4 + 2);
    int32_t vx = v4.x, vy = sub_sat(v4.y, grav, f), vz = v4.z;
    if (S.stirAmp != 0) {
      const int32_t phase =
          S.frame ? (int32_t)(((S.substep - S.substep % S.frame) * 384u) & 131071u) : S.stirPhase;
      int32_t t0 = ((phase + 32768) & 131071) - 65536;
      int32_t tri = (t0 < 0 ? -t0 : t0) - 32768;
      vx = add_sat(vx, mul<16>(tri, S.stirAmp, f), f);
    }
    vx = mul<16>(vx, damp, f);
    vy = mul<16>(vy, damp, f);
    vz = mul<16>(vz, damp, f);
    int3 pr = clamp_world(S, add_sat(p.x, vx, f), add_sat(p.y, vy, f), add_sat(p.z, vz, f));
    const uint32_t bonded = b.bflag[slot] ? TAG_BONDED : 0u;
    b.PRS[slot] = make_int4(pr.x, pr.y, pr.z, (int32_t)((uint32_t)(256 + rhoW) | (sc << TAG_SHIFT) | bonded));
    uint32_t cx = (uint32_t)pr.x >> HSHIFT, cy = (uint32_t)pr.y >> HSHIFT, cz = (uint32_t)pr.z >> HSHIFT;
    b.keys[slot] = S.keyOff + (cz * S.gy + cy) * S.gx + cx;
  }
}

// cellStart[k] = first sorted index with key >= k, for k in [0, K].
__global__ void __launch_bounds__(256) k3_cellstart(Bufs3 b) {
  cell_starts(b.skey, b.world->slotEnd, b.world->K, b.cellStart);
}

__global__ void __launch_bounds__(256) k3_gather(Bufs3 b) {
  const uint32_t nAct = b.world->nAct;
  for (uint32_t s = gtid3(); s < nAct; s += gstride3()) {
    const uint32_t slot = b.sslot[s];
    b.PW[s] = b.PRS[slot];
    b.inv[slot] = s;
  }
}

// buildNbr (3d/sim3d.wgsl:341-390): dz, dy, dx, ascending id; MAXNBR cut
// drops the tail of that order and raises dbg[6]. With L > 1 the L lanes of
// a particle test L consecutive candidates of a row at once and place the
// hits with a ballot prefix, so the list is the same for every L.
template <bool DBG, int L>
__global__ void __launch_bounds__(256) k3_nbr(Bufs3 b) {
  if constexpr (L == 1) {
    const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
    Flags<DBG> f{b.dbg};
    for (uint32_t s = gtid3(); s < nAct; s += gstride3()) {
      const int4 me = b.PW[s];
      const uint32_t sc = scene_of_tag((uint32_t)me.w);
      const Scene3& S = b.scenes[sc];
      const int32_t cx = me.x >> HSHIFT, cy = me.y >> HSHIFT, cz = me.z >> HSHIFT;
      const int32_t x0 = max(cx - 1, 0), x1 = min(cx + 1, (int32_t)S.gx - 1);
      uint32_t cnt = 0;
      for (int dz = -1; dz <= 1; ++dz) {
        int32_t z = cz + dz;
        if (z < 0 || z >= (int32_t)S.gz) continue;
        for (int dy = -1; dy <= 1; ++dy) {
          int32_t y = cy + dy;
          if (y < 0 || y >= (int32_t)S.gy) continue;
          uint32_t row = S.keyOff + ((uint32_t)z * S.gy + (uint32_t)y) * S.gx;
          uint32_t lo = b.cellStart[row + x0], hi = b.cellStart[row + x1 + 1];
          for (uint32_t t = lo; t < hi; ++t) {
            if (t == s) continue;
            int4 o = b.PW[t];
            int32_t dx = wsub(o.x, me.x), dy2 = wsub(o.y, me.y), dz2 = wsub(o.z, me.z);
            if constexpr (DBG)
              if (abs_sat(dx, f) >= H || abs_sat(dy2, f) >= H || abs_sat(dz2, f) >= H) continue;
            if (r2q_of(dx, dy2, dz2) >= H2Q) continue;
            if (cnt >= MAXNBR) { f.flag(6); continue; }
            b.NBR[(size_t)cnt * stride + s] = t;
            ++cnt;
          }
        }
      }
      b.NBRN[s] = cnt;
    }
    return;
  }
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  Flags<DBG> f{b.dbg};
  const uint32_t lane = threadIdx.x & 31u, sub = lane & (L - 1);
  const uint32_t gmask = ((L == 32) ? 0xffffffffu : ((1u << L) - 1u)) << (lane & ~(uint32_t)(L - 1));
  const uint32_t below = (1u << lane) - 1u;
  const uint32_t G = gstride3() / L;
  for (uint32_t s = gtid3() / L;; s += G) {
    if (__shfl_sync(0xffffffffu, s, 0) >= nAct) break;  // warp-uniform exit
    const bool valid = s < nAct;
    const int4 me = valid ? b.PW[s] : make_int4(0, 0, 0, 0);
    const uint32_t sc = scene_of_tag((uint32_t)me.w);
    const Scene3& S = b.scenes[sc];
    const int32_t cx = me.x >> HSHIFT, cy = me.y >> HSHIFT, cz = me.z >> HSHIFT;
    const int32_t x0 = max(cx - 1, 0), x1 = min(cx + 1, (int32_t)S.gx - 1);
    uint32_t cnt = 0;
    for (int dz = -1; dz <= 1; ++dz) {
      for (int dy = -1; dy <= 1; ++dy) {
        const int32_t z = cz + dz, y = cy + dy;
        uint32_t lo = 0, len = 0;
        if (valid && z >= 0 && z < (int32_t)S.gz && y >= 0 && y < (int32_t)S.gy) {
          const uint32_t row = S.keyOff + ((uint32_t)z * S.gy + (uint32_t)y) * S.gx;
          lo = b.cellStart[row + x0];
          len = b.cellStart[row + x1 + 1] - lo;
        }
        const uint32_t maxLen = L == 1 ? len : __reduce_max_sync(0xffffffffu, len);
        for (uint32_t k = sub; k - sub < maxLen; k += L) {
          const uint32_t t = lo + k;
          bool hit = false;
          if (k < len && t != s) {
            const int4 o = b.PW[t];
            const int32_t dx = wsub(o.x, me.x), dy2 = wsub(o.y, me.y), dz2 = wsub(o.z, me.z);
            hit = abs_sat(dx, f) < H && abs_sat(dy2, f) < H && abs_sat(dz2, f) < H && r2q_of(dx, dy2, dz2) < H2Q;
          }
          uint32_t pos = cnt, nhit = hit ? 1u : 0u;
          if (L > 1) {
            const uint32_t bal = __ballot_sync(0xffffffffu, hit) & gmask;
            pos = cnt + __popc(bal & below);
            nhit = __popc(bal);
          }
          if (hit) {
            if (pos >= MAXNBR) f.flag(6);
            else b.NBR[(size_t)pos * stride + s] = t;
          }
          cnt += nhit;
        }
      }
    }
    if (valid && sub == 0) b.NBRN[s] = min(cnt, MAXNBR);
  }
}

// Distance to wall w (axis w >> 1, high side when bit 0 is set) and the signed
// gradient toward it (wall_of, 3d/sim3d.wgsl:127-141). Positions are clamped
// into [MARGIN, wmax - MARGIN], so the distance is positive.
__device__ __forceinline__ int32_t wall_dist(const Scene3& S, int32_t x, int32_t y, int32_t z, int w) {
  int axis = w >> 1;
  int32_t pos = axis == 0 ? x : (axis == 1 ? y : z);
  return (w & 1) ? wsub(S.wmax[axis], pos) : pos;
}

// Sum over the L lanes that share one particle (wrapping u32 addition, so
// the split is exact); OR-reduction for magnitude bounds.
template <int L>
__device__ __forceinline__ int32_t gsum3(int32_t v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v = wadd(v, __shfl_xor_sync(0xffffffffu, v, o, L));
  return v;
}
template <int L>
__device__ __forceinline__ uint32_t gor3(uint32_t v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o, L);
  return v;
}

// density (3d/sim3d.wgsl:397-468). L lanes share a particle's neighbour list;
// every sum here is a wrapping i32 sum (per-term clamps only), so any split is
// exact.
template <bool DBG, int L>
__global__ void __launch_bounds__(256) k3_density(Bufs3 b, const int4* __restrict__ PW) {
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  Flags<DBG> f{b.dbg};
  const uint32_t sub = threadIdx.x & (L - 1), G = gstride3() / L;
  const int32_t W0 = __ldg(&b.WG[0].x);
  for (uint32_t s = gtid3() / L;; s += G) {
    if (__shfl_sync(0xffffffffu, s, 0) >= nAct) break;  // warp-uniform exit
    const bool valid = s < nAct;
    const int4 me = valid ? PW[s] : make_int4(0, 0, 0, 0);
    int32_t rho = 0, St = 0, sgx = 0, sgy = 0, sgz = 0;
    const uint32_t cnt = valid ? b.NBRN[s] : 0u;
    // one neighbour record and two indices ahead (as in the 2D sweeps)
    int4 on = PW[sub < cnt ? b.NBR[(size_t)sub * stride + s] : 0u];
    uint32_t tn2 = sub + L < cnt ? b.NBR[(size_t)(sub + L) * stride + s] : 0u;
    for (uint32_t k = sub; k < cnt; k += L) {
      const int4 o = on;
      if (k + L < cnt) on = PW[tn2];
      if (k + 2 * L < cnt) tn2 = b.NBR[(size_t)(k + 2 * L) * stride + s];
      int32_t dx = wsub(o.x, me.x), dy = wsub(o.y, me.y), dz = wsub(o.z, me.z);
      int32_t r2q = r2q_of(dx, dy, dz);
      if (r2q >= H2Q) continue;
      int2 wg = __ldg(b.WG + ((uint32_t)r2q >> 7));
      rho = wadd(rho, wmul(wg.x, (int32_t)((uint32_t)o.w & TAG_W)) >> 8);
      int32_t gx = mulf<16>(wg.y, dx, f), gy = mulf<16>(wg.y, dy, f), gz = mulf<16>(wg.y, dz, f);
      sgx = wadd(sgx, gx);
      sgy = wadd(sgy, gy);
      sgz = wadd(sgz, gz);
      St = wadd(St, wadd(wadd(mulc<16>(gx, gx, 0, S_TERM, f), mulc<16>(gy, gy, 0, S_TERM, f)),
                         mulc<16>(gz, gz, 0, S_TERM, f)));
    }
    if (L > 1) {
      rho = gsum3<L>(rho);
      St = gsum3<L>(St);
      sgx = gsum3<L>(sgx);
      sgy = gsum3<L>(sgy);
      sgz = gsum3<L>(sgz);
    }
    if (!valid || sub != 0) continue;
    const uint32_t sc = scene_of_tag((uint32_t)me.w);
    const Scene3& S = b.scenes[sc];
    rho = wadd(rho, wmul(W0, (int32_t)((uint32_t)me.w & TAG_W)) >> 8);
#pragma unroll
    for (int w = 0; w < 6; ++w) {
      int32_t dist = wall_dist(S, me.x, me.y, me.z, w);
      if (dist >= H) continue;
      int2 pg = __ldg(b.PG + ((uint32_t)dist >> 8));
      rho = wadd(rho, pg.x);
      int32_t gm = (w & 1) ? pg.y : neg_sat(pg.y, f);
      if (w & 1) (void)neg_sat(pg.y, f);  // select() evaluates both arms
      int axis = w >> 1;
      if (axis == 0) sgx = wadd(sgx, gm); else if (axis == 1) sgy = wadd(sgy, gm); else sgz = wadd(sgz, gm);
      St = wadd(St, s_term(gm, f));  // the two zero components contribute clamp(0) = 0
    }
    int32_t bw;
    int3 bg;
    if (ball_term(b, S, sc, me.x, me.y, me.z, bw, bg, f)) {
      rho = wadd(rho, bw);
      sgx = wadd(sgx, bg.x);
      sgy = wadd(sgy, bg.y);
      sgz = wadd(sgz, bg.z);
      St = wadd(St, wadd(wadd(s_term(bg.x, f), s_term(bg.y, f)), s_term(bg.z, f)));
    }
    St = wadd(St, wadd(wadd(s_term(sgx, f), s_term(sgy, f)), s_term(sgz, f)));
    int32_t Cq = clampi(shr_rne<4>(wsub(rho, RHO0)), 0, C_MAX);
    int32_t lam = clampi(neg_sat(divshift<24>(Cq, wadd(St, EPS_S), b.rcp, f), f), -LAM_MAX, LAM_MAX);
    b.PL[s] = make_int4(me.x, me.y, me.z, lam);
  }
}

// One solveDp pair term (3d/sim3d.wgsl:493-509); false when the pair is out
// of range (it adds nothing).
template <bool DBG>
__device__ __forceinline__ bool dp_term(const Bufs3& b, const int4& me, const int4& o, int32_t& tx, int32_t& ty,
                                        int32_t& tz, const Flags<DBG>& f) {
  int32_t dx = wsub(o.x, me.x), dy = wsub(o.y, me.y), dz = wsub(o.z, me.z);
  int32_t r2q = r2q_of(dx, dy, dz);
  if (r2q >= H2Q) return false;
  int32_t gt = __ldg(&b.WG[(uint32_t)r2q >> 7].y);
  int32_t lsum = DBG ? add_sat(me.w, o.w, f) : wadd(me.w, o.w);
  tx = mulf<20>(lsum, mulf<16>(gt, dx, f), f);
  ty = mulf<20>(lsum, mulf<16>(gt, dy, f), f);
  tz = mulf<20>(lsum, mulf<16>(gt, dz, f), f);
  return true;
}

// The bond correction of one bonded particle from the iteration's starting
// positions (PL), its row walked in order; a bond whose ends have parted too
// far is tombstoned in this end's row (the test is symmetric, so the other end
// tombstones its copy in the same pass). Per bond, as the 2D constraint:
// d4 = (p_i - p_j) >> 5, C = |d4|^2 - L0^2, q = C / (4 |d4|^2) (Q16), and
// each axis sums -clamp(d4 * q * k >> 3); the sum moves the particle by
// clamp(sum >> 8 (round half even), +-BOND3_DP_MAX).
template <bool DBG>
__device__ __forceinline__ int3 bond_dp(const Bufs3& b, const Scene3& S, uint32_t slot, const int4& me,
                                        const Flags<DBG>& f) {
  uint32_t* row = b.bond + (size_t)slot * BOND3_WORDS;
  int32_t bx = 0, by = 0, bz = 0;
  for (uint32_t k = 0; k < BOND3_CAP; ++k) {
    const uint32_t w = row[2 * k];
    if (w == 0u) break;
    if (w & BOND3_TOMB) continue;
    const int32_t L0 = (int32_t)row[2 * k + 1];
    const int32_t L02 = wmul(L0, L0);
    const int4 o = b.PL[b.inv[S.slotBase + (w & BOND3_J) - 1u]];
    const int32_t d4x = shr_rne<BOND3_PRE>(sub_sat(me.x, o.x, f));
    const int32_t d4y = shr_rne<BOND3_PRE>(sub_sat(me.y, o.y, f));
    const int32_t d4z = shr_rne<BOND3_PRE>(sub_sat(me.z, o.z, f));
    if (abs(d4x) > BOND3_L0_MAX || abs(d4y) > BOND3_L0_MAX || abs(d4z) > BOND3_L0_MAX) {
      row[2 * k] = w | BOND3_TOMB;
      continue;
    }
    const int32_t d2 = wadd(wadd(wmul(d4x, d4x), wmul(d4y, d4y)), wmul(d4z, d4z));
    if (d2 >= BOND3_HARD_BREAK2 || (S.bondBrk != 0 && d2 > mul<16>(L02, S.bondBrk, f))) {
      row[2 * k] = w | BOND3_TOMB;
      continue;
    }
    if (d2 < BOND3_D2_FLOOR) continue;
    const int32_t C = sub_sat(d2, L02, f);
    const int32_t qv = divshift<16>(C, wmul(d2, 4), b.rcp, f);
    const int32_t qk = mul<16>(qv, S.bondK, f);
    bx = wsub(bx, clampi(mul<3>(d4x, qk, f), -BOND3_TERM, BOND3_TERM));
    by = wsub(by, clampi(mul<3>(d4y, qk, f), -BOND3_TERM, BOND3_TERM));
    bz = wsub(bz, clampi(mul<3>(d4z, qk, f), -BOND3_TERM, BOND3_TERM));
  }
  return make_int3(clampi(shr_rne<8>(bx), -BOND3_DP_MAX, BOND3_DP_MAX),
                   clampi(shr_rne<8>(by), -BOND3_DP_MAX, BOND3_DP_MAX),
                   clampi(shr_rne<8>(bz), -BOND3_DP_MAX, BOND3_DP_MAX));
}

// solveDp + applyDp (3d/sim3d.wgsl:476-537), fused over a double buffer:
// every read is of the PL / PW written by the previous kernel, the new
// position goes to PWout.
//
// solveDp's running sum saturates, which makes it order-dependent in general.
// The lanes keep wrapping partial sums and an OR of the terms' magnitudes:
// when cnt x max|term| <= INT_MAX no prefix of the sequential sum can leave
// i32, every saturating add is an exact add, and the wrapping total IS the
// sequential result. Otherwise (never seen in practice) lane 0 redoes the sum
// sequentially with saturation in the canonical order.
template <bool DBG, int L>
__global__ void __launch_bounds__(256) k3_solve(Bufs3 b, const int4* __restrict__ PWin, int4* __restrict__ PWout) {
  const uint32_t nAct = b.world->nAct, stride = b.nbrStride;
  Flags<DBG> f{b.dbg};
  const uint32_t sub = threadIdx.x & (L - 1), G = gstride3() / L;
  for (uint32_t s = gtid3() / L;; s += G) {
    if (__shfl_sync(0xffffffffu, s, 0) >= nAct) break;  // warp-uniform exit
    const bool valid = s < nAct;
    const int4 me = valid ? b.PL[s] : make_int4(0, 0, 0, 0);
    const uint32_t cnt = valid ? b.NBRN[s] : 0u;
    int32_t ax = 0, ay = 0, az = 0;
    uint32_t mag = 0;
    int4 on = b.PL[sub < cnt ? b.NBR[(size_t)sub * stride + s] : 0u];
    uint32_t tn2 = sub + L < cnt ? b.NBR[(size_t)(sub + L) * stride + s] : 0u;
    for (uint32_t k = sub; k < cnt; k += L) {
      const int4 o = on;
      if (k + L < cnt) on = b.PL[tn2];
      if (k + 2 * L < cnt) tn2 = b.NBR[(size_t)(k + 2 * L) * stride + s];
      int32_t tx, ty, tz;
      if (!dp_term(b, me, o, tx, ty, tz, f)) continue;
      if constexpr (DBG) {
        if (L == 1) {
          ax = add_sat(ax, tx, f);
          ay = add_sat(ay, ty, f);
          az = add_sat(az, tz, f);
          continue;
        }
      }
      ax = wadd(ax, tx);
      ay = wadd(ay, ty);
      az = wadd(az, tz);
      mag |= (uint32_t)abs(tx) | (uint32_t)abs(ty) | (uint32_t)abs(tz);
    }
    if (L > 1) {
      ax = gsum3<L>(ax);
      ay = gsum3<L>(ay);
      az = gsum3<L>(az);
      mag = gor3<L>(mag);
    }
    if (!valid || sub != 0) continue;
    const bool exact = (DBG && L == 1) || (uint64_t)mag * cnt <= 0x7fffffffull;
    if (!exact) {
      // the terms' own events were counted in the lane pass; recount only the sum's
      const Flags<false> quiet{nullptr};
      ax = ay = az = 0;
      for (uint32_t k = 0; k < cnt; ++k) {
        int4 o = b.PL[b.NBR[(size_t)k * stride + s]];
        int32_t tx, ty, tz;
        if (!dp_term(b, me, o, tx, ty, tz, quiet)) continue;
        ax = add_sat(ax, tx, f);
        ay = add_sat(ay, ty, f);
        az = add_sat(az, tz, f);
      }
    }
    const int32_t tag = PWin[s].w;
    const uint32_t sc = scene_of_tag((uint32_t)tag);
    const Scene3& S = b.scenes[sc];
    const int32_t lami = me.w;
#pragma unroll
    for (int w = 0; w < 6; ++w) {
      int32_t dist = wall_dist(S, me.x, me.y, me.z, w);
      if (dist >= H) continue;
      int32_t pg = __ldg(&b.PG[(uint32_t)dist >> 8].y);
      int32_t gm = (w & 1) ? pg : neg_sat(pg, f);
      if (w & 1) (void)neg_sat(pg, f);
      int axis = w >> 1;
      // the zero components add fp_mul_s(lami, 0) = 0
      int32_t c = mul<20>(lami, gm, f);
      if (axis == 0) ax = add_sat(ax, c, f); else if (axis == 1) ay = add_sat(ay, c, f); else az = add_sat(az, c, f);
    }
    int32_t bw;
    int3 bg;
    if (ball_term(b, S, sc, me.x, me.y, me.z, bw, bg, f)) {
      ax = add_sat(ax, mul<20>(lami, bg.x, f), f);
      ay = add_sat(ay, mul<20>(lami, bg.y, f), f);
      az = add_sat(az, mul<20>(lami, bg.z, f), f);
    }
    if ((uint32_t)tag & TAG_BONDED) {
      const int3 bd = bond_dp(b, S, b.sslot[s], me, f);
      ax = add_sat(ax, bd.x, f);
      ay = add_sat(ay, bd.y, f);
      az = add_sat(az, bd.z, f);
    }
    int3 pr = clamp_world(S, add_sat(me.x, ax, f), add_sat(me.y, ay, f), add_sat(me.z, az, f));
    PWout[s] = make_int4(pr.x, pr.y, pr.z, tag);
  }
}

// integrate (3d/sim3d.wgsl:542-552) back into slot order, with the per-substep
// state hash of the new state when HASH is set.
template <bool DBG, bool HASH>
__global__ void __launch_bounds__(256) k3_integrate(Bufs3 b, const int4* __restrict__ PW) {
  __shared__ uint32_t dsacc[8], dsscene;
  if (HASH) d2::digest_block_begin(dsacc, &dsscene);
  const uint32_t nAct = b.world->nAct;
  Flags<DBG> f{b.dbg};
  const uint32_t nIter = (nAct + gstride3() - 1) / gstride3() * gstride3();
  for (uint32_t s = gtid3(); s < nIter; s += gstride3()) {
    const bool valid = s < nAct;
    uint32_t sc = 0, local = 0;
    int32_t w8[8];
    if (valid) {
      uint32_t slot = b.sslot[s];
      int4 pr = PW[s];
      sc = scene_of_tag((uint32_t)pr.w);
      local = slot - b.scenes[sc].slotBase;
      int4* w4 = reinterpret_cast<int4*>(b.state + (size_t)slot * 8);
      int4 p = w4[0];
      int4 v = make_int4(sub_sat(pr.x, p.x, f), sub_sat(pr.y, p.y, f), sub_sat(pr.z, p.z, f), 0);
      int4 np = make_int4(pr.x, pr.y, pr.z, p.w);
      w4[0] = np;
      w4[1] = v;
      w8[0] = np.x; w8[1] = np.y; w8[2] = np.z; w8[3] = np.w;
      w8[4] = v.x; w8[5] = v.y; w8[6] = v.z; w8[7] = 0;
    }
    if constexpr (HASH) {
      uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (valid) d2::particle_digest(w8, local, nullptr, h);
      d2::digest_add_block(b.acc, dsacc, &dsscene, valid, sc, h);
    }
  }
  if (HASH) d2::digest_block_end(b.acc, dsacc, &dsscene);
}

// State hash of every active scene's slots, on demand.
__global__ void __launch_bounds__(256) k3_hash(Bufs3 b, uint32_t* __restrict__ acc) {
  __shared__ uint32_t dsacc[8], dsscene;
  d2::digest_block_begin(dsacc, &dsscene);
  const uint32_t slotEnd = b.world->slotEnd;
  const uint32_t nIter = (slotEnd + gstride3() - 1) / gstride3() * gstride3();
  for (uint32_t slot = gtid3(); slot < nIter; slot += gstride3()) {
    bool valid = false;
    uint32_t sc = 0, local = 0;
    if (slot < slotEnd) {
      sc = b.sceneOf[slot];
      if (sc != NO_SCENE) {
        local = slot - b.scenes[sc].slotBase;
        valid = local < b.scenes[sc].n;
      }
    }
    uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (valid) d2::particle_digest(b.state + (size_t)slot * 8, local, nullptr, h);
    d2::digest_add_block(acc, dsacc, &dsscene, valid, valid ? sc : 0u, h);
  }
  d2::digest_block_end(acc, dsacc, &dsscene);
}

// Per-scene chain fold of this substep's digest (src/engine.js:4154 semantics)
// and the scene's substep counter.
__global__ void k3_fold(Bufs3 b, int doChain) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.world->numScenes || !b.scenes[s].active) return;
  b.scenes[s].substep += 1u;
  if (!doChain) return;
  uint32_t a[8], nx[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = b.acc[s * 8 + j];
#pragma unroll
  for (int j = 0; j < 8; ++j) nx[j] = d2::mm_step(b.chain[s * 8 + j], a[j] ^ d2::rotl32(a[(j + 1) & 7], 7));
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    b.chain[s * 8 + j] = nx[j];
    b.accLast[s * 8 + j] = a[j];
    b.acc[s * 8 + j] = 0u;
  }
}

// digestStripe (3d/sim3d.wgsl:555-590): 256 fixed contiguous stripes of
// FNV-1a over the bytes of p.xyz and v.xyz, one word per stripe.
__global__ void __launch_bounds__(256) k3_fnv(const int32_t* __restrict__ state, uint32_t base, uint32_t n,
                                              uint32_t* __restrict__ out) {
  const uint32_t k = threadIdx.x;
  const uint32_t per = (n + 255u) / 256u, lo = k * per, hi = min(n, lo + per);
  uint32_t h = 2166136261u;
  for (uint32_t i = lo; i < hi; ++i) {
    const int32_t* w = state + (size_t)(base + i) * 8;
    const uint32_t vals[6] = {(uint32_t)w[0], (uint32_t)w[1], (uint32_t)w[2],
                              (uint32_t)w[4], (uint32_t)w[5], (uint32_t)w[6]};
#pragma unroll
    for (int q = 0; q < 6; ++q)
#pragma unroll
      for (int by = 0; by < 4; ++by) h = (h ^ ((vals[q] >> (8 * by)) & 0xffu)) * 16777619u;
  }
  out[k] = h;
}

}  // namespace d3
}  // namespace sn
