// Definitions shared by the sphere kernels (sphere.cu) and the split-precision Legendre path (sphere_split.cuh).
#pragma once
#include <cuda_runtime.h>

namespace lmw {
namespace {

struct SphDev {
  int N, M, nlat, nlon, nh, ntri, logn;
  double a, g;
  const double *Ps, *Hs, *Pa, *Ha, *mu, *w, *wd, *cosl, *r2om, *kfac, *lapl;
  const double2 *tw;
  const int *trim, *trin, *tri;
  // per member: bit 0 = the Coriolis grid is tilted (read fgrid, else f = om2 mu), bit 1 = orography (read hsgrid)
  const int *gflag;
  const double *om2;  // 2 Omega per member
  float inv_a_f;      // 1/a rounded to FP32 once on the host (the FP32 kernels' metric factor)
  double inv_a, inv_a_l;  // 1/a as a two-term sum, for the FP64 synthesis's correctly rounded division (div_fixed)
  int div_a;          // a and 1/a are normal numbers (else the synthesis divides plainly)
};

template <class R> struct V2;
template <> struct V2<double> { using type = double2; };
template <> struct V2<float> { using type = float2; };
__device__ __forceinline__ double2 mk2(double x, double y) { return make_double2(x, y); }
__device__ __forceinline__ float2 mk2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cfma(float2 acc, float2 a, float s) { return make_float2(fmaf(a.x, s, acc.x), fmaf(a.y, s, acc.y)); }
__device__ __forceinline__ float2 conjd(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 imul(float2 z, float m) { return make_float2(-m * z.y, m * z.x); }
// Legendre tables, weights and twiddles in the compute precision of a stage kernel
template <class R> struct SphTab {
  const R *Ps, *Hs, *Pa, *Ha, *w, *wd, *r2om, *kfac, *lapl;
  const typename V2<R>::type *tw;
};

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cfma(double2 acc, double2 a, double s) { return make_double2(fma(a.x, s, acc.x), fma(a.y, s, acc.y)); }
__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }
// (i m) z
__device__ __forceinline__ double2 imul(double2 z, double m) { return make_double2(-m * z.y, m * z.x); }

// IEEE 754 conversions between binary32 and binary64 on the integer pipe. GB300 executes FP64 arithmetic and
// FP64 conversions on a narrow pipe (about 2 operations per clock per SM), so the split path's FP64 epilogues
// convert with integer operations instead; the results are those of the hardware conversions, bit for bit.
// float -> double is exact: the exponent is rebiased by 1023 - 127 = 896 and the 23 fraction bits become the top
// of the 52. Zeros, subnormals, infinities and NaNs (exponent field 0 or 255) take the hardware conversion.
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return static_cast<double>(f);
  const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  const unsigned lo = u << 29;
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}
// double -> float, rounded to nearest with ties to even, for results in the normal binary32 range: binary64
// exponents 897..1150 become binary32 exponents 1..254, the fraction keeps its top 23 bits and the 29 dropped
// bits decide the rounding; a carry out of the fraction raises the exponent (to infinity past 254), as IEEE
// rounding does. Other exponents (zeros, subnormal results, overflow, infinities, NaNs) take the hardware
// conversion.
__device__ __forceinline__ float d2f_int(double x) {
  const unsigned hi = static_cast<unsigned>(__double2hiint(x)), lo = static_cast<unsigned>(__double2loint(x));
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e < 897u || e > 1150u) return static_cast<float>(x);
  unsigned r = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rem = lo & 0x1fffffffu;
  r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
  return __uint_as_float(r | (hi & 0x80000000u));
}

// a double in the kernel's arithmetic type: itself for FP64, d2f_int (the hardware's rounding) for FP32
template <class R> __device__ __forceinline__ R to_arith(double x);
template <> __device__ __forceinline__ double to_arith<double>(double x) { return x; }
template <> __device__ __forceinline__ float to_arith<float>(double x) { return d2f_int(x); }
// a value of the kernel's arithmetic type widened to double: itself for FP64, f2d_int (exact) for FP32
__device__ __forceinline__ double from_arith(double x) { return x; }
__device__ __forceinline__ double from_arith(float x) { return f2d_int(x); }

constexpr int NSLOT = 5;  // A, B, U Phi, V Phi (times w/((1-mu^2)a)) and the Bernoulli function (times w)

struct StageArgs {
  int stage;        // 0..3
  double c;         // 0.5 dt, 0.5 dt, dt, dt/6
  float c32 = 0.0f;    // c rounded to FP32 (the split path's stages 0-2)
  const double *filt;  // [2][M]: zeta/delta and phi factors by n (last stage)
  int zero = 0;        // advect-only: the flow's tendencies are zero (cpp/sphere.cpp:411-415)
};

}  // namespace
}  // namespace lmw
