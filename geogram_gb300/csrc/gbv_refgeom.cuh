// Device versions of the reference's FP64 cell-geometry formulas,
// evaluated operation for operation as the reference writes them (explicit
// round-to-nearest intrinsics, so no multiply-add is fused), which makes
// corners, radii, volumes, centroids and facet areas bit-identical to the
// reference's for the same combinatorics:
//   det2x2 / det3x3 ............ voronoi/convex_cell.h:356-368
//   compute_triangle_point ..... voronoi/convex_cell.cpp:1055-1081
//   squared_distance ........... voronoi/convex_cell.h:186-191
//   triangle_area .............. voronoi/convex_cell.cpp:1147-1158
//   tet_volume ................. voronoi/convex_cell.cpp:1193-1213
#pragma once

namespace gbv {

__device__ __forceinline__ double r_det2(double a11, double a12, double a21, double a22) {
  return __dsub_rn(__dmul_rn(a11, a22), __dmul_rn(a12, a21));
}

__device__ __forceinline__ double r_det3(double a11, double a12, double a13, double a21,
                                         double a22, double a23, double a31, double a32,
                                         double a33) {
  const double t1 = __dmul_rn(a11, r_det2(a22, a23, a32, a33));
  const double t2 = __dmul_rn(a21, r_det2(a12, a13, a32, a33));
  const double t3 = __dmul_rn(a31, r_det2(a12, a13, a22, a23));
  return __dadd_rn(__dsub_rn(t1, t2), t3);
}

// Homogeneous intersection of the planes of a triangle (rows a, b, c).
__device__ __forceinline__ double4 r_triangle_point(const double4& a, const double4& b,
                                                    const double4& c) {
  double4 r;
  r.x = -r_det3(a.w, a.y, a.z, b.w, b.y, b.z, c.w, c.y, c.z);
  r.y = -r_det3(a.x, a.w, a.z, b.x, b.w, b.z, c.x, c.w, c.z);
  r.z = -r_det3(a.x, a.y, a.w, b.x, b.y, b.w, c.x, c.y, c.w);
  r.w = r_det3(a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z);
  return r;
}

// The corner as compute_geometry stores it: (x/w, y/w, z/w).
__device__ __forceinline__ double3 r_corner(const double4& a, const double4& b,
                                            const double4& c) {
  const double4 p = r_triangle_point(a, b, c);
  return make_double3(__ddiv_rn(p.x, p.w), __ddiv_rn(p.y, p.w), __ddiv_rn(p.z, p.w));
}

// squared_distance(center, p): dx = p - center, dx*dx + dy*dy + dz*dz.
__device__ __forceinline__ double r_sqdist(double cx, double cy, double cz, const double3& p) {
  const double dx = __dsub_rn(p.x, cx), dy = __dsub_rn(p.y, cy), dz = __dsub_rn(p.z, cz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ double r_triangle_area(const double3& p1, const double3& p2,
                                                  const double3& p3) {
  const double Ux = __dsub_rn(p2.x, p1.x), Uy = __dsub_rn(p2.y, p1.y), Uz = __dsub_rn(p2.z, p1.z);
  const double Vx = __dsub_rn(p3.x, p1.x), Vy = __dsub_rn(p3.y, p1.y), Vz = __dsub_rn(p3.z, p1.z);
  const double Wx = __dsub_rn(__dmul_rn(Uy, Vz), __dmul_rn(Uz, Vy));
  const double Wy = __dsub_rn(__dmul_rn(Uz, Vx), __dmul_rn(Ux, Vz));
  const double Wz = __dsub_rn(__dmul_rn(Ux, Vy), __dmul_rn(Uy, Vx));
  const double s =
      __dadd_rn(__dadd_rn(__dmul_rn(Wx, Wx), __dmul_rn(Wy, Wy)), __dmul_rn(Wz, Wz));
  return __dmul_rn(0.5, __dsqrt_rn(s));
}

__device__ __forceinline__ double r_tet_volume(const double3& p1, const double3& p2,
                                               const double3& p3, const double3& p4) {
  const double Ux = __dsub_rn(p2.x, p1.x), Uy = __dsub_rn(p2.y, p1.y), Uz = __dsub_rn(p2.z, p1.z);
  const double Vx = __dsub_rn(p3.x, p1.x), Vy = __dsub_rn(p3.y, p1.y), Vz = __dsub_rn(p3.z, p1.z);
  const double Wx = __dsub_rn(p4.x, p1.x), Wy = __dsub_rn(p4.y, p1.y), Wz = __dsub_rn(p4.z, p1.z);
  const double UVx = __dsub_rn(__dmul_rn(Uy, Vz), __dmul_rn(Uz, Vy));
  const double UVy = __dsub_rn(__dmul_rn(Uz, Vx), __dmul_rn(Ux, Vz));
  const double UVz = __dsub_rn(__dmul_rn(Ux, Vy), __dmul_rn(Uy, Vx));
  const double d =
      __dadd_rn(__dadd_rn(__dmul_rn(UVx, Wx), __dmul_rn(UVy, Wy)), __dmul_rn(UVz, Wz));
  return __ddiv_rn(fabs(d), 6.0);
}

// det4x4 of convex_cell.h:383-402 with the reference's operation order (no
// fused multiply-add): the sign of the fast-predicate conflict test
// (convex_cell.cpp:947-966, conflict iff > 0).  Columns: the planes of the
// triangle's three vertices and the clipping plane.
__device__ __forceinline__ double r_det4x4(const double4& p1, const double4& p2,
                                           const double4& p3, const double4& e) {
  const double a11 = p1.x, a12 = p2.x, a13 = p3.x, a14 = e.x;
  const double a21 = p1.y, a22 = p2.y, a23 = p3.y, a24 = e.y;
  const double a31 = p1.z, a32 = p2.z, a33 = p3.z, a34 = e.z;
  const double a41 = p1.w, a42 = p2.w, a43 = p3.w, a44 = e.w;
  const double m12 = __dsub_rn(__dmul_rn(a21, a12), __dmul_rn(a11, a22));
  const double m13 = __dsub_rn(__dmul_rn(a31, a12), __dmul_rn(a11, a32));
  const double m14 = __dsub_rn(__dmul_rn(a41, a12), __dmul_rn(a11, a42));
  const double m23 = __dsub_rn(__dmul_rn(a31, a22), __dmul_rn(a21, a32));
  const double m24 = __dsub_rn(__dmul_rn(a41, a22), __dmul_rn(a21, a42));
  const double m34 = __dsub_rn(__dmul_rn(a41, a32), __dmul_rn(a31, a42));
  const double m123 =
      __dadd_rn(__dsub_rn(__dmul_rn(m23, a13), __dmul_rn(m13, a23)), __dmul_rn(m12, a33));
  const double m124 =
      __dadd_rn(__dsub_rn(__dmul_rn(m24, a13), __dmul_rn(m14, a23)), __dmul_rn(m12, a43));
  const double m134 =
      __dadd_rn(__dsub_rn(__dmul_rn(m34, a13), __dmul_rn(m14, a33)), __dmul_rn(m13, a43));
  const double m234 =
      __dadd_rn(__dsub_rn(__dmul_rn(m34, a23), __dmul_rn(m24, a33)), __dmul_rn(m23, a43));
  return __dsub_rn(__dadd_rn(__dsub_rn(__dmul_rn(m234, a14), __dmul_rn(m134, a24)),
                             __dmul_rn(m124, a34)),
                   __dmul_rn(m123, a44));
}

// With the fast predicates a conflict test whose filter margin is below
// this multiple of its error bound is decided by r_det4x4 (whose own
// rounding could then differ from the exact sign); beyond it every
// evaluation has the exact sign.
constexpr double kFastPredWide = 64.0;

}  // namespace gbv
