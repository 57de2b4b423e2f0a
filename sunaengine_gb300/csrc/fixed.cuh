// Q16.16 fixed-point core for sm_103a.
//
// Semantics are those of the reference's integer core (src/fixed.wgsl): exact
// 32x32->64 products, arithmetic right shifts rounded half to even, saturation
// to i32, wrapping i32 +,-,*. The implementation is GB300-native: one
// IMAD.WIDE for the product and a branch-free biased-shift rounding
//   RNE(p / 2^s) = (p + 2^(s-1) - 1 + ((p >> s) & 1)) >> s
// instead of the reference's 16-bit-limb emulation.
//
// Debug counters (src/fixed.wgsl:62-77): with DBG = true every saturation,
// bad divide and truncation bumps the same slot the reference's fp_flag does;
// with DBG = false the counting compiles away. Results are identical.
#pragma once
#include <cstdint>

#ifndef SN_HD
#define SN_HD __host__ __device__ __forceinline__
#endif

namespace sn {

constexpr int32_t I32_MAX = 2147483647;
constexpr int32_t I32_MIN = -2147483647 - 1;

template <bool DBG>
struct Flags {
  uint32_t* dbg;
  __device__ __forceinline__ void flag(int slot) const {
    if constexpr (DBG) atomicAdd(dbg + slot, 1u);
  }
};

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
__device__ __forceinline__ int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return min(max(x, lo), hi); }

// RNE shift of a 64-bit value by a runtime s in 1..31, saturated to i32.
template <bool DBG>
__device__ __forceinline__ int32_t shr_rne_sat64(int64_t p, int s, const Flags<DBG>& f) {
  int64_t bias = ((int64_t)1 << (s - 1)) - 1 + ((p >> s) & 1);
  int64_t q = (p + bias) >> s;
  int32_t lo = (int32_t)q;
  if ((int64_t)lo != q) {
    f.flag(0);
    return q < 0 ? I32_MIN : I32_MAX;
  }
  return lo;
}

// fp_mul_s with a compile-time shift (src/fixed.wgsl:168).
template <int S, bool DBG>
__device__ __forceinline__ int32_t mul(int32_t a, int32_t b, const Flags<DBG>& f) {
  static_assert(S >= 1 && S <= 31, "shift");
  int64_t p = (int64_t)a * (int64_t)b;
  int64_t q = (p + ((((int64_t)1) << (S - 1)) - 1) + ((p >> S) & 1)) >> S;
  int32_t lo = (int32_t)q;
  if ((int64_t)lo != q) {
    f.flag(0);
    return q < 0 ? I32_MIN : I32_MAX;
  }
  return lo;
}

// Release-build helpers for products whose range is known from the operand
// bounds. The rounding is computed as round-half-up, t = a*b + 2^(S-1) (one
// IMAD.WIDE with the bias as addend), q = t >> S, then an exact tie (the low S
// bits of t all zero) clears q's low bit: RNE picks the even neighbour, which
// is q & ~1 for both signs in two's complement.
//   mulf : the RNE result provably fits in i32 (no saturation test needed);
//   mulfc: fits in i32 and is then clamped into [lo, hi];
//   mulc : may exceed i32, clamped into [lo, hi] inside i32 (clamping the exact
//          value equals clamping the saturated one).
// Debug builds use the saturating form so the debug counters see every event.
template <int S>
__device__ __forceinline__ int32_t rne_lo(int32_t a, int32_t b) {
  int64_t t = (int64_t)a * (int64_t)b + (((int64_t)1) << (S - 1));
  uint32_t lo = (uint32_t)t, hi = (uint32_t)((uint64_t)t >> 32);
  uint32_t q = __funnelshift_r(lo, hi, S);
  if ((lo & ((1u << S) - 1u)) == 0u) q &= ~1u;
  return (int32_t)q;
}
template <int S>
__device__ __forceinline__ int64_t rne64(int64_t p) {
  int64_t t = p + (((int64_t)1) << (S - 1));
  int64_t q = t >> S;
  if (((uint32_t)t & ((1u << S) - 1u)) == 0u) q &= ~(int64_t)1;
  return q;
}
template <int S, bool DBG>
__device__ __forceinline__ int32_t mulf(int32_t a, int32_t b, const Flags<DBG>& f) {
  if constexpr (DBG) return mul<S>(a, b, f);
  else return rne_lo<S>(a, b);
}
template <int S, bool DBG>
__device__ __forceinline__ int32_t mulfc(int32_t a, int32_t b, int32_t lo, int32_t hi, const Flags<DBG>& f) {
  if constexpr (DBG) return min(max(mul<S>(a, b, f), lo), hi);
  else return min(max(rne_lo<S>(a, b), lo), hi);
}
template <int S, bool DBG>
__device__ __forceinline__ int32_t mulc(int32_t a, int32_t b, int32_t lo, int32_t hi, const Flags<DBG>& f) {
  if constexpr (DBG) {
    return min(max(mul<S>(a, b, f), lo), hi);
  } else {
    int64_t q = rne64<S>((int64_t)a * (int64_t)b);
    return (int32_t)min(max(q, (int64_t)lo), (int64_t)hi);
  }
}

template <bool DBG>
__device__ __forceinline__ int32_t add_sat(int32_t a, int32_t b, const Flags<DBG>& f) {
  int32_t s = wadd(a, b);
  if (((a ^ s) & (b ^ s)) < 0) { f.flag(5); return a < 0 ? I32_MIN : I32_MAX; }
  return s;
}
template <bool DBG>
__device__ __forceinline__ int32_t sub_sat(int32_t a, int32_t b, const Flags<DBG>& f) {
  int32_t s = wsub(a, b);
  if (((a ^ b) & (a ^ s)) < 0) { f.flag(5); return a < 0 ? I32_MIN : I32_MAX; }
  return s;
}
template <bool DBG>
__device__ __forceinline__ int32_t neg_sat(int32_t a, const Flags<DBG>& f) {
  if (a == I32_MIN) { f.flag(5); return I32_MAX; }
  return -a;
}
template <bool DBG>
__device__ __forceinline__ int32_t abs_sat(int32_t a, const Flags<DBG>& f) {
  return a < 0 ? neg_sat(a, f) : a;
}

// fp_shr_rne on i32 (src/fixed.wgsl:205-213): floor shift, then +1 when the
// remainder is above half, or exactly half with an odd quotient.
template <int S>
__device__ __forceinline__ int32_t shr_rne(int32_t x) {
  int32_t q = x >> S;
  uint32_t r = (uint32_t)x & ((1u << S) - 1u);
  return q + (int32_t)((r + (uint32_t)(q & 1)) > (1u << (S - 1)));
}

// fp_divshift (src/fixed.wgsl:285-309): ~floor(num * 2^k / den) through the
// clz-normalised 15-bit reciprocal Rn = floor(2^30 / dn), dn in [2^15, 2^16).
// Rn comes from a 32768-entry table of exact quotients (built on the host by
// integer division), so the solver's per-pair divides cost one cached load.
template <int K, bool DBG>
__device__ __forceinline__ int32_t divshift(int32_t num, int32_t den, const uint16_t* __restrict__ rcp,
                                            const Flags<DBG>& f) {
  if (den == 0) {
    f.flag(2);
    return num == 0 ? 0 : (num > 0 ? I32_MAX : I32_MIN);
  }
  int32_t d = den, nn = num;
  if (d < 0) { f.flag(1); d = abs_sat(d, f); nn = neg_sat(nn, f); }
  int32_t e = 16 - __clz(d);
  int32_t dn = e >= 0 ? (d >> e) : (d << (-e));
  int32_t Rn = (int32_t)__ldg(rcp + (dn - 32768));
  int32_t s = 30 + e - K;
  if (s > 31) { f.flag(1); return 0; }
  if (s < 1) {
    f.flag(1);
    return nn == 0 ? 0 : (nn > 0 ? I32_MAX : I32_MIN);
  }
  return shr_rne_sat64((int64_t)nn * (int64_t)Rn, s, f);
}

// floor(sqrt(x)) for x < 2^32, exact, by bit-by-bit digit recurrence (the
// same mathematical result as src/fixed.wgsl:318-332's isqrt64).
__device__ __forceinline__ uint32_t isqrt32(uint32_t x) {
  uint32_t rem = 0, root = 0;
#pragma unroll
  for (int i = 15; i >= 0; --i) {
    rem = (rem << 2) | ((x >> (2 * i)) & 3u);
    uint32_t trial = (root << 2) | 1u;
    root <<= 1;
    if (rem >= trial) { rem -= trial; root |= 1u; }
  }
  return root;
}

}  // namespace sn
