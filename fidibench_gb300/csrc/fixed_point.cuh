// fixed_point.cuh -- 64-bit block-fixed-point helpers of the temporally
// blocked upwind kernel (host and device).
//
// A field value f is carried as the integer F = round(f * 2^s) for one scale
// s shared by the whole launch (chosen from max|f| so that |F| < 2^60 / G^K,
// G the step's max-norm growth bound).  Conversions are done with integer
// operations on the IEEE-754 bit pattern (the FP64 pipe of GB300 retires only
// ~2 conversions per clock per SM, the integer pipes ~64-128 operations).
//
// The update F' = F + sum_j a_j (F_up_j - F) multiplies 64-bit differences
// D_j (|D_j| < 2^60) by coefficients a_j in [0, 1] held in Q1.62 (A = a 2^62),
// split as A = a1 2^32 + a0 with a0 in [-2^31, 2^31) (balanced halves, so
// 0 <= a1 <= 2^30).  With D = d1 2^32 + d0 (d1 signed, d0 unsigned):
//   A D / 2^64 = a1 d1 + (a1 d0 + a0 d1) / 2^32 + a0 d0 / 2^64.
// fixed_update sums the a1 d1 products exactly, sums the six a1 d0 and a0 d1
// products exactly in one unsigned 64-bit word (offset so that the sum lies
// in [0, 2^64)), rounds that sum once to nearest (2 units of F after the
// final x4), drops the a0 d0 terms (below 2 units of F each) and returns
// F + 4 * sum: within 8 units of the exact F + sum_j a_j D_j, and exactly F
// when every D_j is zero.  Every product is
// a 32 x 32 -> 64-bit multiply (IMAD.WIDE without an addend, which runs at
// about twice the rate of the accumulating form on GB300).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define FDB_HD __host__ __device__ __forceinline__
#else
#define FDB_HD inline
#endif

namespace fdb {

// Bits 2^-1022 .. : values whose binary exponent field is zero (zero and
// subnormals) map to 0; the fixed path never sees non-finite values because
// the scale pre-pass rejects them.
FDB_HD int64_t to_fixed(double f, int s) {
#ifdef __CUDA_ARCH__
  const uint64_t b = (uint64_t)__double_as_longlong(f);
#else
  uint64_t b;
  __builtin_memcpy(&b, &f, 8);
#endif
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0;
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = e - 1075 + s;  // |F| = m * 2^sh
  uint64_t mag;
  if (sh >= 0) {
    mag = (sh < 11) ? (m << sh) : 0x0FFFFFFFFFFFFFFFull;  // cannot happen for |f| <= max
  } else if (sh > -63) {
    mag = (m + (1ull << (-sh - 1))) >> (-sh);  // round half away from zero
  } else {
    mag = 0;
  }
  return (b >> 63) ? -(int64_t)mag : (int64_t)mag;
}

FDB_HD int clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return a ? __builtin_clzll(a) : 64;
#endif
}

// F * 2^-s rounded to nearest even.  Results below 2^-1022 flush to zero.
FDB_HD double to_double(int64_t F, int s) {
  if (F == 0) return 0.0;
  const uint64_t sign = (F < 0) ? 0x8000000000000000ull : 0ull;
  uint64_t a = (F < 0) ? (uint64_t)(-F) : (uint64_t)F;
  const int lz = clz64(a);
  a <<= lz;                          // bit 63 set: |F| = a * 2^-lz
  uint64_t m = a >> 11;              // 53 significant bits
  const uint64_t rem = a & 0x7FF;
  m += (rem > 0x400 || (rem == 0x400 && (m & 1))) ? 1 : 0;
  const int E = 1086 - lz - s;       // biased exponent for m in [2^52, 2^53]
  uint64_t bits;
  if (E <= 0) return 0.0;
  if (E >= 2047) bits = sign | 0x7FF0000000000000ull;
  else bits = sign | ((((uint64_t)(E - 1)) << 52) + m);
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)bits);
#else
  double d;
  __builtin_memcpy(&d, &bits, 8);
  return d;
#endif
}

// Coefficient a in [0, 1] as balanced Q1.62 halves.
struct QCoeff {
  int32_t a1;
  int32_t a0;
};

inline QCoeff make_qcoeff(double a) {
  // a * 2^62 is exact for a >= 2^-10 (53-bit mantissa); smaller a round down.
  const double scaled = a * 4611686018427387904.0;  // 2^62
  uint64_t A = (uint64_t)scaled;
  int64_t lo = (int64_t)(A & 0xFFFFFFFFull);
  int64_t hi = (int64_t)(A >> 32);
  if (lo >= 0x80000000ll) {
    lo -= 0x100000000ll;
    hi += 1;
  }
  QCoeff q;
  q.a1 = (int32_t)hi;
  q.a0 = (int32_t)lo;
  return q;
}

// 32 x 32 -> 64-bit products (one IMAD.WIDE each on the device)
FDB_HD int64_t mulw_s(int32_t a, int32_t b) {
#ifdef __CUDA_ARCH__
  int64_t d;
  asm("mul.wide.s32 %0, %1, %2;" : "=l"(d) : "r"(a), "r"(b));
  return d;
#else
  return (int64_t)a * (int64_t)b;
#endif
}
FDB_HD uint64_t mulw_u(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  uint64_t d;
  asm("mul.wide.u32 %0, %1, %2;" : "=l"(d) : "r"(a), "r"(b));
  return d;
#else
  return (uint64_t)a * (uint64_t)b;
#endif
}

// One cell from its upstream differences D_j = F_up_j - F (|F| < 2^59 for
// the cell and its upstream values): F + sum_j a_j D_j.
FDB_HD int64_t fixed_update_d(int64_t c, int64_t Dz, int64_t Dy, int64_t Dx, const QCoeff& qz,
                              const QCoeff& qy, const QCoeff& qx) {
  const int32_t z1 = (int32_t)(Dz >> 32), y1 = (int32_t)(Dy >> 32), x1 = (int32_t)(Dx >> 32);
  const uint32_t z0 = (uint32_t)Dz, y0 = (uint32_t)Dy, x0 = (uint32_t)Dx;
  // |a1 d1| <= 2^58
  const int64_t hi = mulw_s(qz.a1, z1) + mulw_s(qy.a1, y1) + mulw_s(qx.a1, x1);
  // sum of a1 d0 in [0, 3 2^62), of a0 d1 in (-3 2^59, 3 2^59); with the
  // offset 3 2^59 + 2^31 the total lies in (0, 2^64): exact modulo 2^64
  const uint64_t lo1 = mulw_u((uint32_t)qz.a1, z0) + mulw_u((uint32_t)qy.a1, y0) +
                       mulw_u((uint32_t)qx.a1, x0);
  const uint64_t lo2 = (uint64_t)(mulw_s(qz.a0, z1) + mulw_s(qy.a0, y1) + mulw_s(qx.a0, x1));
  const uint64_t lo = lo1 + lo2 + ((3ull << 59) + 0x80000000ull);
  const int64_t r = hi + (int64_t)(lo >> 32) - (3ll << 27);
  return c + r * 4;
}

// One cell: F' = F + sum_j a_j (F_up_j - F) for the z, y and x upstream
// values zb, up, left.
FDB_HD int64_t fixed_update(int64_t c, int64_t zb, int64_t up, int64_t left, const QCoeff& qz,
                            const QCoeff& qy, const QCoeff& qx) {
  return fixed_update_d(c, zb - c, up - c, left - c, qz, qy, qx);
}

}  // namespace fdb
