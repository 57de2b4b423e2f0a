// §20 rigid bodies on the GPU (src/sim.wgsl:670-821, 2001-2051, 3070-3747).
//
// One CTA of 256 threads per body, as in the reference: the members are the
// slots of [first, last] that wear FLAG_RIGID and the body's tag; the CTA sums
// their forces and torques (wrapping i32 sums, so the reduction order is
// free), one thread updates the 32-word body record, and every thread then
// places its share of the members at c + R(theta) * o.
//
//   k_rigid_step    rigidStep, after k_predict_key: integrates V and omega,
//                   places members into predSlot and re-keys them
//   k_rigid_solve   rigidSolve, after each solver iteration: folds the
//                   members' dp (solver + friction, kept in DP by the colour
//                   and friction passes) and swept seal contacts into the
//                   body, places members into both pred buffers
//   k_rigid_member  rigidMember, after thermal: closes the substep, lets
//                   members leave, re-bases and recounts
//
// The rest of a body's state is in the particles' own words (FLAG_RIGID and
// the weld tag), which the other passes read through the INFO_RIGID/INFO_TAG
// bits of the sorted records.
#pragma once
#include "sim2d.cuh"

namespace sn {
namespace d2 {

constexpr int RB_LIVE = 0, RB_TAG = 1, RB_FIRST = 2, RB_LAST = 3, RB_CX = 4, RB_CY = 5, RB_VX = 6, RB_VY = 7,
              RB_THETA = 8, RB_OMEGA = 9, RB_RESX = 10, RB_RESY = 11, RB_RESVX = 12, RB_RESVY = 13, RB_N = 14,
              RB_SUMIS2 = 15, RB_GSUM = 16, RB_INVI = 17, RB_IQ = 18, RB_RSH = 19, RB_ISH = 20, RB_OMEGAM = 21,
              RB_RMAX = 22, RB_OSH = 23, RB_CQX = 24, RB_CQY = 25, RB_THETAQ = 26, RB_AXIS = 27, RB_USER = 28,
              RB_SCENE = 29;  // this layout's own word: the world scene the body belongs to
constexpr int RG_BODY_WORDS = 32, RG_MAX_BODIES = 1024, RG_DRIVER_WORDS = 10, RG_COS_N = 1026;
constexpr int RD_MASK = 0, RD_PX = 1, RD_PY = 2, RD_A = 3, RD_VX = 4, RD_VY = 5, RD_W = 6, RD_FX = 7, RD_FY = 8,
              RD_TQ = 9;
constexpr int32_t RD_HAS_PX = 1, RD_HAS_PY = 2, RD_HAS_A = 4, RD_HAS_VX = 8, RD_HAS_VY = 16, RD_HAS_W = 32,
                  RD_HAS_FX = 64, RD_HAS_FY = 128, RD_HAS_TQ = 256;
constexpr int32_t BAM_QUARTER = 1073741824, BAM_PER_RAD = 683565276;
constexpr int RG_QSH = 20, COS_Q = 22;
constexpr int32_t RG_QMASK = 1048575;
constexpr int32_t TQ_TERM_R = 134217728;
constexpr int TQ_HI_SH = 15;
constexpr int32_t RIGID_MIN_MEMBERS = 4;
constexpr int32_t RG_IQ_MIN = 16, RG_IQ_MAX = 31;
constexpr int32_t SEAL_R4 = 1126;  // 0.55 wu
constexpr int RG_THREADS = 256;

// fp_shr_rne with a per-body shift; WGSL shift amounts wrap modulo 32, so
// s = 0 leaves x unchanged.
__device__ __forceinline__ int32_t shr_rne_rt(int32_t x, uint32_t s) {
  if (s == 0u) return x;
  const int32_t q = x >> s;
  const uint32_t rem = (uint32_t)x & ((1u << s) - 1u), half = 1u << (s - 1u);
  return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

// fp_div_s (src/fixed.wgsl:219-261) with a runtime shift: RNE((|a| << s) / |b|)
// of the 64-bit dividend, signed and saturated.
template <bool DBG>
__device__ int32_t div_s(int32_t a, int32_t b, uint32_t s, const Flags<DBG>& f) {
  if (b == 0) {
    f.flag(2);
    return a == 0 ? 0 : (a > 0 ? I32_MAX : I32_MIN);
  }
  const bool neg = (a < 0) != (b < 0);
  const uint64_t ua = a < 0 ? (uint64_t)(-(int64_t)a) : (uint64_t)a;
  const uint64_t ub = b < 0 ? (uint64_t)(-(int64_t)b) : (uint64_t)b;
  const uint64_t n = s < 64u ? ua << s : 0u;
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

// rg_cos / rg_sin (src/sim.wgsl:836-853): quarter-turn fold of the Q22 table.
template <bool DBG>
__device__ __forceinline__ int32_t rg_cos(const int32_t* __restrict__ T, int32_t a, const Flags<DBG>& f) {
  const uint32_t q = ((uint32_t)a >> 30) & 3u;
  const int32_t w = a & 1073741823;
  const int32_t u = (q == 0u || q == 2u) ? w : BAM_QUARTER - w;
  const bool neg = (q == 1u || q == 2u);
  const uint32_t idx = (uint32_t)u >> RG_QSH;
  const int32_t frac = u & RG_QMASK;
  const int32_t c0 = __ldg(T + idx), c1 = __ldg(T + idx + 1);
  const int32_t v = wadd(c0, mul<RG_QSH>(wsub(c1, c0), frac, f));
  return neg ? wsub(0, v) : v;
}
template <bool DBG>
__device__ __forceinline__ int32_t rg_sin(const int32_t* __restrict__ T, int32_t a, const Flags<DBG>& f) {
  return rg_cos(T, wsub(a, BAM_QUARTER), f);
}

// rg_idiv_rne (src/sim.wgsl:862-872)
__device__ __forceinline__ int32_t rg_idiv_rne(int32_t a, int32_t n) {
  if (n <= 0) return 0;
  const bool neg = a < 0;
  const int32_t x = neg ? wsub(0, a) : a;
  int32_t q = (int32_t)((int64_t)x / n);
  const int32_t r2 = wmul(2, wsub(x, wmul(q, n)));
  if (r2 > n || (r2 == n && (q & 1) == 1)) q = wadd(q, 1);
  return neg ? wsub(0, q) : q;
}

// rg_inv_inertia (src/sim.wgsl:3141-3154)
template <bool DBG>
__device__ void rg_inv_inertia(int32_t s, int32_t rsh, int32_t ish, int32_t& invI, int32_t& iq, const Flags<DBG>& f) {
  invI = 0;
  iq = 0;
  if (s <= 0) return;
  const int32_t bl = 32 - __clz(s);
  const int32_t iqNat = bl - 1 + 2 * ish - rsh;
  const int32_t q = min(iqNat, RG_IQ_MAX);
  const int32_t E = q + rsh - 2 * ish;
  if (iqNat < RG_IQ_MIN || E < 1 || E > 62) { f.flag(10); return; }
  invI = div_s(BAM_PER_RAD, s, (uint32_t)E, f);
  iq = q;
}

// rg_mul_shr (src/sim.wgsl:3167-3169)
template <bool DBG>
__device__ __forceinline__ int32_t rg_mul_shr(int32_t a, int32_t b, int32_t s, const Flags<DBG>& f) {
  return shr_rne_sat64((int64_t)a * (int64_t)b, clampi(s, 1, 31), f);
}

__device__ __forceinline__ bool rg_member(const Bufs& b, uint32_t slot, int32_t tag) {
  const uint32_t fl = (uint32_t)b.state[(size_t)slot * 8 + 5];
  return (fl & FLAG_RIGID) != 0u && (int32_t)(fl & WELD_TAG_MASK) == tag;
}

// Sum K wrapping i32 values over the CTA; every thread gets the totals.
template <int K>
__device__ __forceinline__ void rg_block_sum(int32_t (&v)[K], int32_t (*sh)[K]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] = wadd(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sh[warp][k] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    int32_t t = 0;
    for (int w = 0; w < RG_THREADS / 32; ++w) t = wadd(t, sh[w][k]);
    v[k] = t;
  }
  __syncthreads();
}

// pred = c + R(theta) * o (rg_place, src/sim.wgsl:3193-3206)
template <bool DBG>
__device__ __forceinline__ int2 rg_at(int32_t cx, int32_t cy, int32_t c, int32_t s, int2 o, const Flags<DBG>& f) {
  return make_int2(add_sat(cx, sub_sat(mul<COS_Q>(o.x, c, f), mul<COS_Q>(o.y, s, f), f), f),
                   add_sat(cy, add_sat(mul<COS_Q>(o.x, s, f), mul<COS_Q>(o.y, c, f), f), f));
}

// rigidStep (src/sim.wgsl:3226-3440). Runs after k_predict_key, which gave
// every member pred = pos; the placement overwrites predSlot and the grid key.
template <bool DBG>
__global__ void __launch_bounds__(RG_THREADS) k_rigid_step(Bufs b) {
  Flags<DBG> f{b.dbg};
  __shared__ int32_t sh[RG_THREADS / 32][4];
  int32_t* R = b.rbody + (size_t)blockIdx.x * RG_BODY_WORDS;
  const int32_t* D = b.rdrv + (size_t)blockIdx.x * RG_DRIVER_WORDS;
  const ScenePar& S = b.scenes[R[RB_SCENE]];
  const int32_t tag = R[RB_TAG], n = R[RB_N], axis = R[RB_AXIS], dmask = D[RD_MASK];
  if (!(R[RB_LIVE] != 0 && n >= RIGID_MIN_MEMBERS) || !S.active) return;
  const uint32_t first = (uint32_t)R[RB_FIRST], last = (uint32_t)R[RB_LAST], rsh = (uint32_t)R[RB_RSH];
  int32_t cx = R[RB_CX], cy = R[RB_CY];
  if (dmask & RD_HAS_PX) cx = D[RD_PX];
  if (dmask & RD_HAS_PY) cy = D[RD_PY];
  int32_t v[4] = {0, 0, 0, 0};  // fx, fy, thi, tlo
  for (uint32_t i = first + threadIdx.x; i <= last && i < S.nFluid; i += RG_THREADS) {
    const uint32_t slot = S.slotBase + i;
    if (!rg_member(b, slot, tag)) continue;
    const int32_t* w = b.state + (size_t)slot * 8;
    const int2 st0 = b.stacc[slot];
    const int32_t gI = axis != 0 ? matw(b, (uint32_t)w[4], M_grav) : 0;
    const int32_t sy0 = add_sat(st0.y, gI, f);
    const int2 jm = jet_accel(S, make_int2(w[0], w[1]), f);
    const int32_t jx0 = add_sat(st0.x, jm.x, f), jy0 = add_sat(sy0, jm.y, f);
    const int32_t sx = clampi(jx0, -32768, 32768), sy = clampi(jy0, -32768, 32768);
    if (sx != jx0 || sy != jy0) f.flag(11);
    v[0] = wadd(v[0], sx);
    v[1] = wadd(v[1], sy);
    const int32_t rx = shr_rne_rt(sub_sat(w[0], cx, f), rsh), ry = shr_rne_rt(sub_sat(w[1], cy, f), rsh);
    const int32_t raw = wsub(wmul(rx, sy), wmul(ry, sx));
    if (raw > TQ_TERM_R || raw < -TQ_TERM_R) f.flag(9);
    const int32_t t = clampi(raw, -TQ_TERM_R, TQ_TERM_R);
    const int32_t hi = t >> TQ_HI_SH;
    v[2] = wadd(v[2], hi);
    v[3] = wadd(v[3], wsub(t, (int32_t)((uint32_t)hi << TQ_HI_SH)));
  }
  rg_block_sum<4>(v, sh);
  if (threadIdx.x == 0) {
    const int32_t invI = R[RB_INVI], iq = R[RB_IQ], gS = R[RB_GSUM];
    const bool holdX = axis != 0 || (dmask & RD_HAS_PX), holdY = axis != 0 || (dmask & RD_HAS_PY);
    int32_t dvx = 0, dvy = 0;
    if (axis == 0) {
      const int32_t ax = wadd(R[RB_RESVX], v[0]), ay = wadd(wadd(R[RB_RESVY], v[1]), gS);
      dvx = rg_idiv_rne(ax, n);
      dvy = rg_idiv_rne(ay, n);
      R[RB_RESVX] = wsub(ax, wmul(dvx, n));
      R[RB_RESVY] = wsub(ay, wmul(dvy, n));
      const bool usr = R[RB_USER] != 0;
      dvx = add_sat(dvx, usr ? S.userA[0] : 0, f);
      dvy = add_sat(dvy, usr ? S.userA[1] : 0, f);
    }
    if (dmask & RD_HAS_FX) dvx = add_sat(dvx, D[RD_FX], f);
    if (dmask & RD_HAS_FY) dvy = add_sat(dvy, D[RD_FY], f);
    const int32_t vx0 = (dmask & RD_HAS_VX) ? D[RD_VX] : R[RB_VX];
    const int32_t vy0 = (dmask & RD_HAS_VY) ? D[RD_VY] : R[RB_VY];
    const int32_t vmaxN = neg_sat(S.vmax, f);
    const int32_t vx = clampi(add_sat(vx0, dvx, f), vmaxN, S.vmax);
    const int32_t vy = clampi(add_sat(vy0, dvy, f), vmaxN, S.vmax);
    if (holdX) {
      R[RB_VX] = 0; R[RB_RESVX] = 0; R[RB_CQX] = cx; R[RB_CX] = cx;
    } else {
      R[RB_VX] = vx;
      R[RB_CQX] = clampi(add_sat(cx, vx, f), WALL, wsub(S.domW, WALL));
    }
    if (holdY) {
      R[RB_VY] = 0; R[RB_RESVY] = 0; R[RB_CQY] = cy; R[RB_CY] = cy;
    } else {
      R[RB_VY] = vy;
      R[RB_CQY] = clampi(add_sat(cy, vy, f), WALL, wsub(S.domH, WALL));
    }
    int32_t dth = 0;
    if (invI != 0) dth = add_sat(rg_mul_shr(v[2], invI, iq - TQ_HI_SH, f), rg_mul_shr(v[3], invI, iq, f), f);
    if (dmask & RD_HAS_TQ) dth = add_sat(dth, D[RD_TQ], f);
    const int32_t theta = (dmask & RD_HAS_A) ? D[RD_A] : R[RB_THETA];
    const int32_t w0 = (dmask & RD_HAS_W) ? D[RD_W] : R[RB_OMEGA];
    const int32_t om = R[RB_OMEGAM];
    const int32_t wv = clampi(add_sat(w0, dth, f), wsub(0, om), om);
    if (dmask & RD_HAS_A) {
      R[RB_THETA] = theta; R[RB_THETAQ] = theta; R[RB_OMEGA] = 0;
    } else {
      R[RB_OMEGA] = wv;
      R[RB_THETAQ] = wadd(theta, wv);
    }
  }
  __syncthreads();
  const int32_t qx = R[RB_CQX], qy = R[RB_CQY], th = R[RB_THETAQ];
  const int32_t c = rg_cos(b.cosT, th, f), s = rg_sin(b.cosT, th, f);
  for (uint32_t i = first + threadIdx.x; i <= last && i < S.nFluid; i += RG_THREADS) {
    const uint32_t slot = S.slotBase + i;
    if (!rg_member(b, slot, tag)) continue;
    const int2 pr = rg_at(qx, qy, c, s, b.rest[slot], f);
    b.predSlot[slot] = pr;
    const int2 cc = cell_coord(S, pr);
    b.keys[slot] = key_of(S, cc.x, cc.y);
  }
}

// rigid_seal_delta (src/sim.wgsl:2001-2051): the member's swept segment
// against held seal particles in the cells its expanded AABB touches. Every
// hit returns the same reversion (pos - pred), so the scan is an existence
// test and its order does not matter: lane `sub` of a group of L lanes tests
// every L-th candidate of each cell, and the group ORs the answers.
template <bool DBG>
__device__ bool rigid_seal_hit(const Bufs& b, const ScenePar& S, uint32_t p, int2 pos, int2 pr, int32_t tag,
                               uint32_t sub, uint32_t L, const Flags<DBG>& f) {
  const int32_t mx4 = shr_rne<BPRE>(sub_sat(pr.x, pos.x, f)), my4 = shr_rne<BPRE>(sub_sat(pr.y, pos.y, f));
  const int32_t ml2 = wadd(wmul(mx4, mx4), wmul(my4, my4));
  const int2 lo = cell_coord(S, make_int2(sub_sat(min(pos.x, pr.x), SEAL_REACH, f), sub_sat(min(pos.y, pr.y), SEAL_REACH, f)));
  const int2 hi = cell_coord(S, make_int2(add_sat(max(pos.x, pr.x), SEAL_REACH, f), add_sat(max(pos.y, pr.y), SEAL_REACH, f)));
  for (int32_t gy = lo.y; gy <= hi.y; ++gy)
    for (int32_t gx = lo.x; gx <= hi.x; ++gx) {
      const uint32_t key = key_of(S, gx, gy);
      for (uint32_t t = b.cellStart[key] + sub; t < b.cellStart[key + 1]; t += L) {
        if (t == p) continue;
        const int4 o = b.PL[t];
        const uint32_t info = (uint32_t)o.w;
        // a held seal particle wears FLAG_SEAL and FLAG_ANCHOR, so its sorted
        // record carries INFO_SEAL and INFO_PINNED; only those read their flags
        if ((info & INFO_BOUNDARY) || !(info & INFO_SEAL) || !(info & INFO_PINNED)) continue;
        const uint32_t fj = (uint32_t)b.state[(size_t)b.sslot[t] * 8 + 5];
        if ((fj & (FLAG_ANCHOR | FLAG_SEAL)) != (FLAG_ANCHOR | FLAG_SEAL) || !seal_class(b, info & INFO_MAT)) continue;
        if ((fj & FLAG_RIGID) && (int32_t)(fj & WELD_TAG_MASK) == tag) continue;
        const int32_t px4 = shr_rne<BPRE>(sub_sat(o.x, pos.x, f)), py4 = shr_rne<BPRE>(sub_sat(o.y, pos.y, f));
        int32_t dx4 = px4, dy4 = py4;
        if (ml2 > 0) {
          const int32_t dot = wadd(wmul(px4, mx4), wmul(py4, my4));
          if (dot >= ml2) {
            dx4 = wsub(px4, mx4);
            dy4 = wsub(py4, my4);
          } else if (dot > 0) {
            const int32_t tq = div_s(dot, ml2, 16u, f);
            dx4 = wsub(px4, mul<16>(mx4, tq, f));
            dy4 = wsub(py4, mul<16>(my4, tq, f));
          }
        }
        if (wadd(wmul(dx4, dx4), wmul(dy4, dy4)) < SEAL_R4 * SEAL_R4)
          return true;
      }
    }
  return false;
}

// rigidSolve (src/sim.wgsl:3459-3573), after each iteration's friction pass.
// `seal`: the world has seal-class rows (else no contact can exist).
template <bool DBG>
__global__ void __launch_bounds__(RG_THREADS, 1) k_rigid_solve(Bufs b, int seal) {
  Flags<DBG> f{b.dbg};
  __shared__ int32_t sh[RG_THREADS / 32][7];
  int32_t* R = b.rbody + (size_t)blockIdx.x * RG_BODY_WORDS;
  const int32_t* D = b.rdrv + (size_t)blockIdx.x * RG_DRIVER_WORDS;
  const ScenePar& S = b.scenes[R[RB_SCENE]];
  const int32_t tag = R[RB_TAG], n = R[RB_N], axis = R[RB_AXIS], dmask = D[RD_MASK];
  if (!(R[RB_LIVE] != 0 && n >= RIGID_MIN_MEMBERS) || !S.active) return;
  const uint32_t first = (uint32_t)R[RB_FIRST], last = (uint32_t)R[RB_LAST], rsh = (uint32_t)R[RB_RSH];
  const int32_t cqx = R[RB_CQX], cqy = R[RB_CQY];
  int32_t v[7] = {0, 0, 0, 0, 0, 0, 0};  // fx, fy, thi, tlo, sn, sx, sy
  // With seal contacts possible, a body whose slot range leaves threads idle
  // gives each member a group of L lanes for the contact search (debug builds
  // keep one lane, so their event counts follow the sequential scan).
  const uint32_t span = last >= first ? last - first + 1u : 0u;
  uint32_t L = 1;
  if (!DBG && seal)
    while (L < 8u && span * (L * 2u) <= (uint32_t)RG_THREADS) L *= 2u;
  const uint32_t lane = threadIdx.x & 31u, sub = threadIdx.x & (L - 1u);
  const uint32_t gmask = ((1u << L) - 1u) << (lane & ~(L - 1u));
  for (uint32_t base = first; base <= last && base < S.nFluid; base += RG_THREADS / L) {
    const uint32_t i = base + threadIdx.x / L;
    const uint32_t slot = S.slotBase + i;
    const bool mem = i <= last && i < S.nFluid && rg_member(b, slot, tag);
    const int32_t* w = b.state + (size_t)(mem ? slot : S.slotBase) * 8;
    const uint32_t p = mem ? b.inv[slot] : 0u;
    const int2 pr = ld_pred(b.PL, p);
    const int2 pos = make_int2(w[0], w[1]);
    bool hit = seal && mem && rigid_seal_hit(b, S, p, pos, pr, tag, sub, L, f);
    if (L > 1u) hit = (__ballot_sync(0xffffffffu, hit) & gmask) != 0u;
    if (!mem || sub != 0u) continue;
    const int32_t dm = matw(b, (uint32_t)w[4], M_dpMax), dmN = neg_sat(dm, f);
    const int2 dp = b.DP[p];
    const int2 sd = hit ? make_int2(sub_sat(pos.x, pr.x, f), sub_sat(pos.y, pr.y, f)) : make_int2(0, 0);
    const int32_t dx = clampi(shr_rne<8>(dp.x), dmN, dm), dy = clampi(shr_rne<8>(dp.y), dmN, dm);
    v[0] = wadd(v[0], dx);
    v[1] = wadd(v[1], dy);
    if (sd.x != 0 || sd.y != 0) {
      v[4] = wadd(v[4], 1);
      v[5] = wadd(v[5], sd.x);
      v[6] = wadd(v[6], sd.y);
    }
    const int32_t tx = add_sat(dx, sd.x, f), ty = add_sat(dy, sd.y, f);
    const int32_t rx = shr_rne_rt(sub_sat(pr.x, cqx, f), rsh), ry = shr_rne_rt(sub_sat(pr.y, cqy, f), rsh);
    const int32_t raw = wsub(wmul(rx, ty), wmul(ry, tx));
    if (raw > TQ_TERM_R || raw < -TQ_TERM_R) f.flag(9);
    const int32_t t = clampi(raw, -TQ_TERM_R, TQ_TERM_R);
    const int32_t hi = t >> TQ_HI_SH;
    v[2] = wadd(v[2], hi);
    v[3] = wadd(v[3], wsub(t, (int32_t)((uint32_t)hi << TQ_HI_SH)));
  }
  rg_block_sum<7>(v, sh);
  if (threadIdx.x == 0) {
    const int32_t invI = R[RB_INVI], iq = R[RB_IQ];
    if (axis == 0) {
      const int32_t ax = wadd(R[RB_RESX], v[0]), ay = wadd(R[RB_RESY], v[1]);
      int32_t dcx = rg_idiv_rne(ax, n), dcy = rg_idiv_rne(ay, n);
      R[RB_RESX] = wsub(ax, wmul(dcx, n));
      R[RB_RESY] = wsub(ay, wmul(dcy, n));
      if (v[4] > 0) {
        dcx = add_sat(dcx, rg_idiv_rne(v[5], v[4]), f);
        dcy = add_sat(dcy, rg_idiv_rne(v[6], v[4]), f);
      }
      if (!(dmask & RD_HAS_PX)) R[RB_CQX] = clampi(add_sat(cqx, dcx, f), WALL, wsub(S.domW, WALL));
      else R[RB_RESX] = 0;
      if (!(dmask & RD_HAS_PY)) R[RB_CQY] = clampi(add_sat(cqy, dcy, f), WALL, wsub(S.domH, WALL));
      else R[RB_RESY] = 0;
    }
    int32_t dth = 0;
    if (invI != 0) dth = add_sat(rg_mul_shr(v[2], invI, iq - TQ_HI_SH, f), rg_mul_shr(v[3], invI, iq, f), f);
    if (!(dmask & RD_HAS_A)) R[RB_THETAQ] = wadd(R[RB_THETAQ], dth);
  }
  __syncthreads();
  const int32_t qx = R[RB_CQX], qy = R[RB_CQY], th = R[RB_THETAQ];
  const int32_t c = rg_cos(b.cosT, th, f), s = rg_sin(b.cosT, th, f);
  for (uint32_t i = first + threadIdx.x; i <= last && i < S.nFluid; i += RG_THREADS) {
    const uint32_t slot = S.slotBase + i;
    if (!rg_member(b, slot, tag)) continue;
    const uint32_t p = b.inv[slot];
    const int2 pr = rg_at(qx, qy, c, s, b.rest[slot], f);
    *reinterpret_cast<int2*>(b.PL + p) = pr;
    *reinterpret_cast<int2*>(b.PL2 + p) = pr;
  }
}

// rigidMember (src/sim.wgsl:3610-3747), after thermal and containStress.
// Leave decisions read the membership the pass began with (marks first, then
// the clears, across a CTA barrier); the reference's single loop clears
// FLAG_RIGID while other lanes of its workgroup read it.
template <bool DBG>
__global__ void __launch_bounds__(RG_THREADS) k_rigid_member(Bufs b) {
  Flags<DBG> f{b.dbg};
  __shared__ int32_t sh[RG_THREADS / 32][5];
  int32_t* R = b.rbody + (size_t)blockIdx.x * RG_BODY_WORDS;
  const ScenePar& S = b.scenes[R[RB_SCENE]];
  if (R[RB_LIVE] == 0 || !S.active) return;
  const int32_t tag = R[RB_TAG], axis = R[RB_AXIS];
  const uint32_t first = (uint32_t)R[RB_FIRST], last = (uint32_t)R[RB_LAST];
  const uint32_t ish = (uint32_t)R[RB_ISH], osh = (uint32_t)R[RB_OSH];
  const uint32_t stride = b.nbrStride;
  if (threadIdx.x == 0) {  // 1. close the substep
    const int32_t vmaxN = neg_sat(S.vmax, f);
    R[RB_VX] = clampi(sub_sat(R[RB_CQX], R[RB_CX], f), vmaxN, S.vmax);
    R[RB_VY] = clampi(sub_sat(R[RB_CQY], R[RB_CY], f), vmaxN, S.vmax);
    R[RB_OMEGA] = wsub(R[RB_THETAQ], R[RB_THETA]);
    R[RB_CX] = R[RB_CQX];
    R[RB_CY] = R[RB_CQY];
    R[RB_THETA] = R[RB_THETAQ];
  }
  // 2. leave: a member whose row is no longer rigid (or retired), or with no
  // same-body neighbour within bond range
  for (uint32_t i = first + threadIdx.x; i <= last && i < S.nFluid; i += RG_THREADS) {
    const uint32_t slot = S.slotBase + i;
    if (!rg_member(b, slot, tag)) continue;
    const int32_t* w = b.state + (size_t)slot * 8;
    const uint32_t m = (uint32_t)w[4];
    bool leave = matw(b, m, M_solidMode) != SOLID_RIGID || matw(b, m, M_phantom) != 0;
    if (!leave) {
      bool touched = false;
      const uint32_t p = b.inv[slot], cnt = b.NBRN[p] & NBRN_COUNT;
      for (uint32_t k = 0; k < cnt && !touched; ++k) {
        const uint32_t e = b.NBR[(size_t)k * stride + p];
        if (e & NBR_BOUNDARY) continue;
        const uint32_t js = b.sslot[e];
        if (!rg_member(b, js, tag)) continue;
        const int32_t* wj = b.state + (size_t)js * 8;
        const int32_t dx = shr_rne<BPRE>(sub_sat(w[0], wj[0], f)), dy = shr_rne<BPRE>(sub_sat(w[1], wj[1], f));
        if (abs(dx) > L0_MAX || abs(dy) > L0_MAX) continue;
        if (wadd(wmul(dx, dx), wmul(dy, dy)) <= BOND_R2) touched = true;
      }
      leave = !touched;
    }
    b.rmark[slot] = leave ? 1u : 0u;
  }
  __syncthreads();
  for (uint32_t i = first + threadIdx.x; i <= last && i < S.nFluid; i += RG_THREADS) {
    const uint32_t slot = S.slotBase + i;
    if (!rg_member(b, slot, tag)) continue;
    if (b.rmark[slot]) b.state[(size_t)slot * 8 + 5] &= ~(int32_t)FLAG_RIGID;
  }
  __syncthreads();
  // 3. recount and re-base
  int32_t v[5] = {0, 0, 0, 0, 0};  // n, sum ox>>osh, sum oy>>osh, sum (o>>ish)^2, sum grav
  for (uint32_t i = first + threadIdx.x; i <= last && i < S.nFluid; i += RG_THREADS) {
    const uint32_t slot = S.slotBase + i;
    if (!rg_member(b, slot, tag)) continue;
    const int2 o = b.rest[slot];
    v[0] = wadd(v[0], 1);
    v[1] = wadd(v[1], o.x >> osh);
    v[2] = wadd(v[2], o.y >> osh);
    const int32_t a = o.x >> ish, c = o.y >> ish;
    v[3] = wadd(v[3], wadd(wmul(a, a), wmul(c, c)));
    v[4] = wadd(v[4], matw(b, (uint32_t)b.state[(size_t)slot * 8 + 4], M_grav));
  }
  rg_block_sum<5>(v, sh);
  const int32_t nLive = v[0];
  const bool dissolve = nLive < RIGID_MIN_MEMBERS;
  int32_t dx = 0, dy = 0;
  if (!dissolve && axis == 0) {
    dx = (int32_t)((uint32_t)rg_idiv_rne(v[1], nLive) << osh);
    dy = (int32_t)((uint32_t)rg_idiv_rne(v[2], nLive) << osh);
  }
  if (threadIdx.x == 0) {
    if (dissolve) {
      R[RB_LIVE] = 0;
      R[RB_N] = 0;
    } else {
      if (dx != 0 || dy != 0) {
        const int32_t th = R[RB_THETA];
        const int32_t c = rg_cos(b.cosT, th, f), s = rg_sin(b.cosT, th, f);
        R[RB_CX] = add_sat(R[RB_CX], sub_sat(mul<COS_Q>(dx, c, f), mul<COS_Q>(dy, s, f), f), f);
        R[RB_CY] = add_sat(R[RB_CY], add_sat(mul<COS_Q>(dx, s, f), mul<COS_Q>(dy, c, f), f), f);
      }
      R[RB_N] = nLive;
      R[RB_SUMIS2] = v[3];
      R[RB_GSUM] = v[4];
      int32_t invI, iq;
      rg_inv_inertia(v[3], R[RB_RSH], R[RB_ISH], invI, iq, f);
      R[RB_INVI] = invI;
      R[RB_IQ] = iq;
    }
  }
  if (!dissolve && dx == 0 && dy == 0) return;
  for (uint32_t i = first + threadIdx.x; i <= last && i < S.nFluid; i += RG_THREADS) {
    const uint32_t slot = S.slotBase + i;
    if (!rg_member(b, slot, tag)) continue;
    if (dissolve) {
      b.state[(size_t)slot * 8 + 5] &= ~(int32_t)FLAG_RIGID;
    } else {
      const int2 o = b.rest[slot];
      b.rest[slot] = make_int2(wsub(o.x, dx), wsub(o.y, dy));
    }
  }
}

}  // namespace d2
}  // namespace sn
