// ORACLE — test infrastructure only. Never linked into the product library.
//
// Scalar CPU restatement of the reference's integer numeric core,
// src/fixed.wgsl (SunaEngine). Every function follows the WGSL semantics the
// reference relies on: i32 +,-,* wrap mod 2^32, `>>` on i32 is arithmetic,
// integer `/` truncates. Signed overflow is undefined in C++, so wrapping
// arithmetic is done on uint32_t.
//
// The debug counters (fp_flag, src/fixed.wgsl:62-77) are mirrored: every
// function takes the 16-slot counter array and bumps the same slot the
// reference bumps. Counting never changes a result.
#pragma once
#include <cstdint>

namespace ofx {

constexpr int32_t I32_MAX = 2147483647;
constexpr int32_t I32_MIN = -2147483647 - 1;

struct Dbg {
  uint32_t* slots;  // 16 counters, may be shared between threads
  void flag(uint32_t s) const {
#ifdef _OPENMP
#pragma omp atomic
#endif
    slots[s] += 1u;
  }
};

inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
inline int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return x < lo ? lo : (x > hi ? hi : x); }

// i64_mul_i32 + i64_shr_rne_sat (src/fixed.wgsl:131-164): exact signed product,
// arithmetic shift by s in 1..31 rounding half to even, saturate to i32 with
// dbg[0] on saturation.
inline int32_t i64_shr_rne_sat(int64_t v, uint32_t s, const Dbg& d) {
  uint64_t u = (uint64_t)v;
  uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
  uint32_t hiS = (uint32_t)((int32_t)hi >> s);
  uint32_t loS = (lo >> s) | (hi << (32u - s));
  uint32_t mask = (1u << s) - 1u;
  uint32_t rem = lo & mask;
  uint32_t half = 1u << (s - 1u);
  uint32_t inc = 0;
  if (rem > half) inc = 1;
  else if (rem == half) inc = loS & 1u;
  uint32_t lo2 = loS + inc;
  uint32_t hi2 = hiS;
  if (inc == 1u && lo2 == 0u) hi2 += 1u;
  uint32_t sgn = lo2 >> 31;
  if (hi2 == 0u && sgn == 0u) return (int32_t)lo2;
  if (hi2 == 0xFFFFFFFFu && sgn == 1u) return (int32_t)lo2;
  d.flag(0);
  if ((int32_t)hi < 0) return I32_MIN;
  return I32_MAX;
}

inline int32_t fp_mul_s(int32_t a, int32_t b, uint32_t s, const Dbg& d) {
  return i64_shr_rne_sat((int64_t)a * (int64_t)b, s, d);
}

// src/fixed.wgsl:175-200
inline int32_t fp_add_sat(int32_t a, int32_t b, const Dbg& d) {
  int32_t s = wadd(a, b);
  if (((a ^ s) & (b ^ s)) < 0) { d.flag(5); return a < 0 ? I32_MIN : I32_MAX; }
  return s;
}
inline int32_t fp_neg_sat(int32_t a, const Dbg& d) {
  if (a == I32_MIN) { d.flag(5); return I32_MAX; }
  return -a;
}
inline int32_t fp_sub_sat(int32_t a, int32_t b, const Dbg& d) {
  int32_t s = wsub(a, b);
  if (((a ^ b) & (a ^ s)) < 0) { d.flag(5); return a < 0 ? I32_MIN : I32_MAX; }
  return s;
}
inline int32_t fp_abs(int32_t a, const Dbg& d) { return a < 0 ? fp_neg_sat(a, d) : a; }

// src/fixed.wgsl:205-213
inline int32_t fp_shr_rne(int32_t x, uint32_t s) {
  int32_t q = x >> s;
  uint32_t rem = (uint32_t)x & ((1u << s) - 1u);
  uint32_t half = 1u << (s - 1u);
  int32_t inc = 0;
  if (rem > half) inc = 1;
  else if (rem == half && (q & 1) == 1) inc = 1;
  return q + inc;
}

inline uint32_t clz32(uint32_t x) { return x == 0 ? 32u : (uint32_t)__builtin_clz(x); }

// src/fixed.wgsl:285-309 — the solver divide: ~floor(num * 2^k / den) through a
// clz-normalised 15-bit reciprocal.
inline int32_t fp_divshift(int32_t num, int32_t den, uint32_t k, const Dbg& d) {
  if (den == 0) {
    d.flag(2);
    if (num == 0) return 0;
    return num > 0 ? I32_MAX : I32_MIN;
  }
  int32_t dd = den, nn = num;
  if (dd < 0) { d.flag(1); dd = fp_abs(dd, d); nn = fp_neg_sat(nn, d); }
  int32_t e = 16 - (int32_t)clz32((uint32_t)dd);
  int32_t dn = e >= 0 ? (dd >> e) : (int32_t)((uint32_t)dd << (uint32_t)(-e));
  int32_t Rn = 1073741824 / dn;
  int32_t s = 30 + e - (int32_t)k;
  if (s > 31) { d.flag(1); return 0; }
  if (s < 1) {
    d.flag(1);
    if (nn == 0) return 0;
    return nn > 0 ? I32_MAX : I32_MIN;
  }
  return i64_shr_rne_sat((int64_t)nn * (int64_t)Rn, (uint32_t)s, d);
}

// src/fixed.wgsl:318-332 — floor(sqrt(n)) for a 64-bit unsigned n, digit
// recurrence. Only used on values below 2^32 here.
inline uint32_t isqrt64(uint64_t n) {
  uint64_t rem = 0;
  uint32_t root = 0;
  for (int i = 31; i >= 0; --i) {
    uint32_t bits = (uint32_t)((n >> (2 * i)) & 3u);
    rem = (rem << 2) + bits;
    uint64_t trial = ((uint64_t)root << 2) + 1u;
    root <<= 1;
    if (rem >= trial) { rem -= trial; root |= 1u; }
  }
  return root;
}

}  // namespace ofx
