// bin_coord.h -- window start and fraction of a node coordinate on a power-of-two grid,
// from the bits of x (integer arithmetic only).
//
// The reference's rule (src/cunfft_kernel.cu:175-182) for grid size n:
//     u = llrint(n x) - signbit(x) - m,    c = n x - u,
// evaluated there in FP64.  For n = 2^k the product n x is exact, so u and the fraction
// c - m follow exactly from the sign, exponent and mantissa of x: with x = (-1)^s M 2^-(sh+k)
// (M the 53-bit significand), n x = (-1)^s M 2^-sh, llrint rounds M 2^-sh half to even, and
//     c - m = n x - llrint(n x) + s = v 2^-sh
// with v an integer below 2^63.  GB300's FP64 pipe is narrow; this form leaves it idle.
// Compiled for the device (binning kernels) and the host (its check against the FP64
// rule on the CPU).
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define CG_BIN_HD __host__ __device__
#else
#define CG_BIN_HD
#endif

namespace cg {

struct CoordPow2 {
  int64_t u;  // window start llrint(n x) - signbit(x) - m
  int64_t v;  // (c - m) 2^sh, exact
  int sh;     // 1 .. 62
};

// false when x is zero, subnormal, not finite, |n x| >= 2^52 or |n x| < 2^-10: the
// caller then takes the FP64 form
CG_BIN_HD inline bool coord_pow2(double x, int k, int m, CoordPow2& out) {
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  const int s = (int)(b >> 63), e = (int)((b >> 52) & 0x7FF);
  if (e == 0 || e == 0x7FF) return false;
  const uint64_t mant = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = 1075 - k - e;  // n x = (-1)^s mant 2^-sh
  if (sh < 1 || sh > 62) return false;
  const uint64_t q = mant >> sh, rem = mant & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  const uint64_t up = (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;  // round half to even
  const int64_t ra = (int64_t)(q + up);
  out.u = (s ? -ra : ra) - s - m;
  const int64_t d = (int64_t)rem - (int64_t)(up << sh);  // |n x| - |llrint(n x)|, times 2^sh
  out.v = s ? (int64_t)(1ull << sh) - d : d;
  out.sh = sh;
  return true;
}

// v 2^-sh rounded once to FP32
CG_BIN_HD inline float coord_pow2_frac(const CoordPow2& c) {
  uint32_t sb = (uint32_t)(127 - c.sh) << 23;  // 2^-sh, a normal float for sh <= 62
  float scale;
  memcpy(&scale, &sb, sizeof(scale));
  return (float)c.v * scale;
}

}  // namespace cg
