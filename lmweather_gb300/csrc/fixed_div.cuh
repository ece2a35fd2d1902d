// Correctly rounded division by a divisor fixed for a run (FP64), shared by the plane stencil and the FP64
// sphere synthesis.
#pragma once
#include <cmath>

namespace lmw {

constexpr unsigned long long kDivAbs = 0x7fffffffffffffffull, kDivMant = 0x000fffffffffffffull;

// x / y correctly rounded (round to nearest even), for a divisor y fixed for the run. GB300's FP64 pipe is narrow
// and an IEEE division costs several FP64 operations with a reciprocal seed; this costs three. The host stores the
// reciprocal as an unevaluated sum zh + zl (zh = RN(1/y), zl = RN(1/y - zh), formed exactly with an FMA), and
// q = RN(x zh + RN(x zl)) approximates x / y to about 2^-105 relative (the fixed-divisor scheme of N. Brisebarre,
// J.-M. Muller and S. K. Raina, "Accelerating correctly rounded floating-point division when the divisor is known
// in advance", IEEE Trans. Computers 53(8), 2004). q is ACCEPTED only on a proof that it is the rounded quotient:
// with gap the distance from |q| to the next double toward zero (the smaller of its two neighbour gaps) and
// T = |y| gap / 2 (a power-of-two scaling of y, formed exactly on the integer pipe), the FMA residual
// r = RN(x - q y) satisfies |r| < T only if |x - q y| < T (rounding is monotone and T is a double), that is
// |x / y - q| < gap / 2, which puts x / y strictly inside q's rounding interval. Zero dividends give the signed
// zero directly; everything else that is not accepted (ties, non-finite values, quotients or bounds outside the
// normal range) takes the IEEE division, so the result is RN(x / y) for every x.
__device__ __forceinline__ double div_fixed(double x, double y, double zh, double zl, int &fast) {
  const double q = __fma_rn(x, zh, __dmul_rn(x, zl));
  const double r = __fma_rn(-q, y, x);
  const unsigned long long bx = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long by0 = static_cast<unsigned long long>(__double_as_longlong(y));
  const unsigned long long bq = static_cast<unsigned long long>(__double_as_longlong(q)) & kDivAbs;
  const unsigned long long by = by0 & kDivAbs;
  const unsigned long long br = static_cast<unsigned long long>(__double_as_longlong(r)) & kDivAbs;
  if ((bx & kDivAbs) == 0) {
    fast = 1;
    return __longlong_as_double(static_cast<long long>((bx ^ by0) & ~kDivAbs));
  }
  const int eq = static_cast<int>(bq >> 52);
  // biased exponent of T: |y| times 2^(exponent of gap - 1), gap = ulp(q), halved when q is a power of two
  const int et = static_cast<int>(by >> 52) + eq - 1023 - 53 - ((bq & kDivMant) == 0 ? 1 : 0);
  if (eq >= 1 && eq <= 2046 && et >= 1 && et <= 2046 &&
      br < ((static_cast<unsigned long long>(et) << 52) | (by & kDivMant))) {
    fast = 1;
    return q;
  }
  fast = 0;
  return x / y;
}

// the two-term reciprocal div_fixed needs: zh = RN(1/y), zl = RN(1/y - zh) (1 - y zh is exact for zh = RN(1/y), so
// the FMA forms it without error and the division rounds 1/y - zh once); false when y or zh is not a normal number
// (then divide plainly). A subnormal zl (|y| above about 2^969) only makes the fast path's answer rarer: the
// acceptance test does not depend on it.
inline bool fixed_div_reciprocal(double y, double &zh, double &zl) {
  zh = 1.0 / y;
  zl = std::fma(-y, zh, 1.0) / y;
  return std::fpclassify(y) == FP_NORMAL && std::fpclassify(zh) == FP_NORMAL && std::isfinite(zl);
}

}  // namespace lmw
