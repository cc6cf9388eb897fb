// Exact sign of a 4x4 determinant of doubles, on the device.
//
// The reference decides every clipping conflict of VBW::ConvexCell with
// PCK::det_4d (voronoi/convex_cell.cpp:870-912, numerics/predicates.cpp:
// 2073-2110): a floating-point filter, then exact expansion arithmetic when
// the filter cannot decide.  This is the exact part, written from
// Shewchuk's published algorithms (J. R. Shewchuk, "Adaptive Precision
// Floating-Point Arithmetic and Fast Robust Geometric Predicates",
// Discrete Comput. Geom. 18, 1997): Two-Sum, Two-Product (exact with a
// fused multiply-add), Grow-Expansion and Scale-Expansion with zero
// elimination.  Expansions are kept in increasing magnitude order and are
// nonoverlapping, so the sign is the sign of the last component.
#pragma once

namespace gbv {

__device__ __forceinline__ void x_two_sum(double a, double b, double& x, double& y) {
  x = __dadd_rn(a, b);
  double bv = __dsub_rn(x, a);
  double av = __dsub_rn(x, bv);
  y = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
}

__device__ __forceinline__ void x_two_prod(double a, double b, double& x, double& y) {
  x = __dmul_rn(a, b);
  y = __fma_rn(a, b, -x);
}

// h = e + b (h may not alias e); returns the length of h.
__device__ __forceinline__ int x_grow(int en, const double* e, double b, double* h) {
  double q = b;
  int hn = 0;
  for (int i = 0; i < en; ++i) {
    double qn, hh;
    x_two_sum(q, e[i], qn, hh);
    q = qn;
    if (hh != 0.0) h[hn++] = hh;
  }
  if (q != 0.0 || hn == 0) h[hn++] = q;
  return hn;
}

// h = e + f (repeated growth through tmp; h may not alias e or f).
__device__ __forceinline__ int x_sum(int en, const double* e, int fn, const double* f,
                                     double* h, double* tmp) {
  for (int i = 0; i < en; ++i) h[i] = e[i];
  int hn = en;
  for (int i = 0; i < fn; ++i) {
    hn = x_grow(hn, h, f[i], tmp);
    for (int j = 0; j < hn; ++j) h[j] = tmp[j];
  }
  return hn;
}

// h = b * e; returns the length of h.
__device__ __forceinline__ int x_scale(int en, const double* e, double b, double* h) {
  int hn = 0;
  double q, hh;
  x_two_prod(e[0], b, q, hh);
  if (hh != 0.0) h[hn++] = hh;
  for (int i = 1; i < en; ++i) {
    double p1, p0, s;
    x_two_prod(e[i], b, p1, p0);
    x_two_sum(q, p0, s, hh);
    if (hh != 0.0) h[hn++] = hh;
    x_two_sum(p1, s, q, hh);
    if (hh != 0.0) h[hn++] = hh;
  }
  if (q != 0.0 || hn == 0) h[hn++] = q;
  return hn;
}

// Exact sign of det [r0; r1; r2; r3] (rows of four doubles): 2x2 minors of
// rows 0-1, 3x3 minors of rows 0-2 expanded along row 2, the 4x4
// determinant expanded along row 3.  Kept out of line: it only runs when
// the floating-point filter of the clipping kernel cannot decide.
static __device__ __noinline__ int det4_sign_exact(const double* r0, const double* r1,
                                            const double* r2, const double* r3) {
  double m[6][4];
  int mn[6];
  // pair index of columns (a<b): 01 02 03 12 13 23
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
  for (int k = 0; k < 6; ++k) {
    double p[2], q[2], t[8];
    x_two_prod(r0[pa[k]], r1[pb[k]], p[1], p[0]);
    x_two_prod(-r0[pb[k]], r1[pa[k]], q[1], q[0]);
    mn[k] = x_sum(2, p, 2, q, m[k], t);
  }
  auto pidx = [](int a, int b) { return a == 0 ? b - 1 : (a == 1 ? b + 1 : 5); };
  const int cols[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  double acc[192], tmp[192];
  int an = 1;
  acc[0] = 0.0;
  for (int s = 0; s < 4; ++s) {
    const int a = cols[s][0], b = cols[s][1], c = cols[s][2];
    double t1[8], t2[8], t3[8], u[16], d3[24], t4[32];
    const int kbc = pidx(b, c), kac = pidx(a, c), kab = pidx(a, b);
    int n1 = x_scale(mn[kbc], m[kbc], r2[a], t1);
    int n2 = x_scale(mn[kac], m[kac], -r2[b], t2);
    int n3 = x_scale(mn[kab], m[kab], r2[c], t3);
    int nu = x_sum(n1, t1, n2, t2, u, t4);
    int nd = x_sum(nu, u, n3, t3, d3, t4);
    double f = (s % 2 == 0) ? -r3[s] : r3[s];
    double term[48];
    int tn = x_scale(nd, d3, f, term);
    for (int i = 0; i < tn; ++i) {
      an = x_grow(an, acc, term[i], tmp);
      for (int j = 0; j < an; ++j) acc[j] = tmp[j];
    }
  }
  const double top = acc[an - 1];
  return (top > 0.0) - (top < 0.0);
}

}  // namespace gbv
