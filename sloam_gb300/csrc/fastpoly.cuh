// fastpoly.cuh — the projection's first-try arctangent: an odd polynomial
// in FP32, fitted here by iteratively reweighted least squares on Chebyshev
// nodes (relative error), evaluated by Horner's rule with fma.
//
//   atan(a) = a * P(a^2),  0 <= a <= 1,    P of degree 8.
//
// Measured in emulated FP32 over 8 M arguments: at most 1.6 ulp
// (1.27e-7 relative) from the exact value.  atan2 is rebuilt from atan on
// min/max of |x|, |y| with an approximate quotient (2 ulp): 4.9e-7 relative
// at most from the correctly rounded float.  The projection accepts these
// values only where a 1.2e-6 relative margin cannot change the pixel, so
// the pixel equals the one of the correctly rounded angle; other points
// take the exact path.  tests/test_fastpoly.py re-checks the bounds from the
// coefficient lists below.
#pragma once

namespace sg {

// Coefficients, constant term first.
#define SG_ATAN_P                                                              \
  9.999999848e-01f, -3.333307364e-01f, 1.999262348e-01f, -1.420367011e-01f,    \
      1.064101933e-01f, -7.504455481e-02f, 4.269324857e-02f, -1.606961499e-02f, \
      2.850121155e-03f

__device__ __forceinline__ float atan01_poly(float a) {
  constexpr float c[9] = {SG_ATAN_P};
  const float s = a * a;
  float p = c[8];
#pragma unroll
  for (int k = 7; k >= 0; --k) p = fmaf(p, s, c[k]);
  return a * p;
}

// atan2(y, x) for finite nonzero x, y with 1e-18 <= min(|x|,|y|) and
// max(|x|,|y|) <= 1e18 (the quotient stays a normal float; __fdividef's
// 2-ulp bound holds for divisors in (2^-126, 2^126)).
__device__ __forceinline__ float atan2_poly(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  float t = atan01_poly(__fdividef(mn, mx));
  t = ay > ax ? 1.57079637f - t : t;
  t = x < 0.0f ? 3.14159274f - t : t;
  return copysignf(t, y);
}

}  // namespace sg
