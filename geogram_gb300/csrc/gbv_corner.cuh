// Corners of a cell from three planes, with the error bound that lets the
// clipping kernels decide most conflict signs in floating point
// (declarations shared by the fixed-shape and the unbounded clipping
// kernels).
#pragma once

#include "gbv_refgeom.cuh"

namespace gbv {

template <typename Real>
struct Consts;
template <>
struct Consts<double> {
  // error-bound factors in units of 2^-53, about twice the rounding counts
  // of the evaluation: 3x3 determinant (5 levels), dot product (3 levels)
  static constexpr double kDet = 12.0 * 1.1102230246251565e-16;
  static constexpr double kDot = 8.0 * 1.1102230246251565e-16;
  static constexpr double kUlp = 1.1102230246251565e-16;
};
template <>
struct Consts<float> {
  // units of 2^-24; includes the rounding of the FP32 planes themselves
  static constexpr float kDet = 32.0f * 5.9604645e-8f;
  static constexpr float kDot = 16.0f * 5.9604645e-8f;
  static constexpr float kUlp = 5.9604645e-8f;
};

// Error bound of a corner obtained by Cramer's rule from its homogeneous
// coordinates with denominator W, the permanents (pX, pY, pZ, pW) of the
// four 3x3 minors and cm = max |corner coordinate|: a bound on
// |corner - exact corner| per coordinate plus the rounding of a later
// 4-term dot product with the corner.  +inf when the sign of W is not sure.
template <typename Real>
__device__ __forceinline__ Real cramer_bound(Real W, Real pX, Real pY, Real pZ, Real pW, Real cm) {
  using K = Consts<Real>;
  const Real den = fabs(W) - K::kDet * pW;
  if (!(den > Real(0))) return Real(INFINITY);
  const Real pm = fmax(pX, fmax(pY, pZ));
  return (K::kDet * (pm + cm * pW) / den + Real(2) * K::kUlp * cm + K::kDot * cm) * Real(1.0001);
}

// Permanents of the 3x3 minors of rows a, b, c used by Cramer's rule.
template <typename Real, typename R4>
__device__ __forceinline__ void cramer_perms(const R4& a, const R4& b, const R4& c, Real& pX,
                                             Real& pY, Real& pZ, Real& pW) {
  const Real pxy = fabs(b.x * c.y) + fabs(b.y * c.x), pxz = fabs(b.x * c.z) + fabs(b.z * c.x);
  const Real pxw = fabs(b.x * c.w) + fabs(b.w * c.x), pyz = fabs(b.y * c.z) + fabs(b.z * c.y);
  const Real pyw = fabs(b.y * c.w) + fabs(b.w * c.y), pzw = fabs(b.z * c.w) + fabs(b.w * c.z);
  pW = fabs(a.x) * pyz + fabs(a.y) * pxz + fabs(a.z) * pxy;
  pX = fabs(a.w) * pyz + fabs(a.y) * pzw + fabs(a.z) * pyw;
  pY = fabs(a.x) * pzw + fabs(a.w) * pxz + fabs(a.z) * pxw;
  pZ = fabs(a.x) * pyw + fabs(a.y) * pxw + fabs(a.w) * pxy;
}

// FP32 corner: Cramer's rule through the 2x2 minors of rows b, c.
__device__ __forceinline__ void corner_fp32(const float4& a, const float4& b, const float4& c,
                                            float& x, float& y, float& z, float& eps) {
  const float mxy = b.x * c.y - b.y * c.x, mxz = b.x * c.z - b.z * c.x;
  const float mxw = b.x * c.w - b.w * c.x, myz = b.y * c.z - b.z * c.y;
  const float myw = b.y * c.w - b.w * c.y, mzw = b.z * c.w - b.w * c.z;
  const float W = a.x * myz - a.y * mxz + a.z * mxy;
  const float X = -(a.w * myz + a.y * mzw - a.z * myw);
  const float Y = a.x * mzw + a.w * mxz - a.z * mxw;
  const float Z = -(a.x * myw - a.y * mxw + a.w * mxy);
  const float inv = 1.0f / W;
  x = X * inv;
  y = Y * inv;
  z = Z * inv;
  float pX, pY, pZ, pW;
  cramer_perms<float>(a, b, c, pX, pY, pZ, pW);
  eps = cramer_bound<float>(W, pX, pY, pZ, pW, fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z))));
}

// FP64 corner exactly as the reference computes it, with its error bound.
__device__ __forceinline__ void corner_fp64(const double4& a, const double4& b,
                                            const double4& c, double& x, double& y, double& z,
                                            float& eps) {
  const double4 p = r_triangle_point(a, b, c);
  x = __ddiv_rn(p.x, p.w);
  y = __ddiv_rn(p.y, p.w);
  z = __ddiv_rn(p.z, p.w);
  double pX, pY, pZ, pW;
  cramer_perms<double>(a, b, c, pX, pY, pZ, pW);
  const double e =
      cramer_bound<double>(p.w, pX, pY, pZ, pW, fmax(fabs(x), fmax(fabs(y), fabs(z))));
  eps = __double2float_ru(e);
}

}  // namespace gbv
