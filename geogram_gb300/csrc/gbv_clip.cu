// Laguerre cell clipping: one thread per cell, the polytope in shared
// memory laid out [slot][thread] so that a warp's 32 cells touch 32
// consecutive words.
//
// The cell is kept in the dual form of the reference's VBW::ConvexCell
// (voronoi/convex_cell.h:419-1436): every clipping plane is a vertex,
// every corner of the polytope is a triangle of three planes, with the
// three adjacent triangles.  Clipping by a plane (convex_cell.cpp:461-516,
// 761-865) removes the triangles whose corner is on the negative side and
// fans new triangles from the new plane around the border of the removed
// zone.  What differs from the CPU code is the layout and the bookkeeping:
//   - triangles live in fixed slots tracked by bit masks instead of linked
//     lists, planes in slots recycled once no triangle uses them;
//   - each triangle caches its corner and a bound on the corner's rounding
//     error, so a conflict test is three FMAs and a compare; when the
//     bound cannot decide the sign, the FP64 kernel evaluates the exact
//     determinant sign (the reference's PCK::det_4d decision) and the FP32
//     kernel marks the cell for an FP64 re-clip;
//   - the security-radius test (generic_RVD.h:2278-2352) reads the
//     cached corner radii.
#include <cfloat>
#include <cmath>
#include <type_traits>

#include "gbv_clip.cuh"
#include "gbv_exact.cuh"

namespace gbv {

constexpr uint32_t kBoxBase = 0xFFFFFF00u;  // pslot of box plane b is kBoxBase + b
cudaError_t last_launch_error = cudaSuccess;
constexpr int kClipThreads = 32;

// ---------------------------------------------------------------------
// Small fixed-capacity bit sets
// ---------------------------------------------------------------------
template <int NW>
struct Bits {
  uint64_t w[NW];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int i = 0; i < NW; ++i) w[i] = 0;
  }
  __device__ __forceinline__ bool test(int i) const { return (w[i >> 6] >> (i & 63)) & 1ull; }
  __device__ __forceinline__ void set(int i) { w[i >> 6] |= 1ull << (i & 63); }
  __device__ __forceinline__ int popc() const {
    int c = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) c += __popcll(w[i]);
    return c;
  }
  __device__ __forceinline__ bool any() const {
    uint64_t a = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) a |= w[i];
    return a != 0;
  }
  __device__ __forceinline__ bool equals(const Bits& o) const {
    bool e = true;
#pragma unroll
    for (int i = 0; i < NW; ++i) e = e && (w[i] == o.w[i]);
    return e;
  }
  // lowest set bit, -1 if none
  __device__ __forceinline__ int first() const {
#pragma unroll
    for (int i = 0; i < NW; ++i)
      if (w[i]) return i * 64 + __ffsll((long long)w[i]) - 1;
    return -1;
  }
};

template <int NW>
__device__ __forceinline__ Bits<NW> andnot(const Bits<NW>& a, const Bits<NW>& b) {
  Bits<NW> r;
#pragma unroll
  for (int i = 0; i < NW; ++i) r.w[i] = a.w[i] & ~b.w[i];
  return r;
}

template <int NW>
__device__ __forceinline__ Bits<NW> full_bits(int n) {
  Bits<NW> r;
#pragma unroll
  for (int i = 0; i < NW; ++i) {
    int lo = i * 64;
    r.w[i] = (n >= lo + 64) ? ~0ull : (n <= lo ? 0ull : ((1ull << (n - lo)) - 1ull));
  }
  return r;
}

// ---------------------------------------------------------------------
// Per-thread cell storage in shared memory
// ---------------------------------------------------------------------
template <typename Real, int BS, int T, int P>
struct CellSmem;

template <int BS, int T, int P>
struct CellSmem<double, BS, T, P> {
  double4 corner[T][BS];  // x, y, z (global frame); w packs (r2, eps) floats
  uint32_t tv[T][BS];     // planes i | j << 8 | k << 16
  uint32_t ta[T][BS];     // adjacent triangles across the edges opposite i, j, k
  uint32_t pslot[P][BS];  // neighbour's sorted slot, or kBoxBase + box face
  uint16_t prank[P][BS];  // position in the neighbour list
  uint16_t pnb[P][BS];    // border scratch: triangle | edge << 8
  uint8_t pnext[P][BS];   // border scratch: next border plane / facet triangle
};

template <int BS, int T, int P>
struct CellSmem<float, BS, T, P> {
  float4 corner[T][BS];   // x, y, z (frame centred on the seed), eps
  float4 plane[P][BS];    // local-frame plane equations
  uint32_t tv[T][BS];
  uint32_t ta[T][BS];
  uint32_t pslot[P][BS];
  uint16_t prank[P][BS];
  uint16_t pnb[P][BS];
  uint8_t pnext[P][BS];
};

template <typename Real>
struct Consts;
template <>
struct Consts<double> {
  // error-bound factors (units of 2^-53), inflated about twice over the
  // rounding counts of the evaluation: det3 (5 levels), dot (3 levels)
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

__device__ __forceinline__ double pack2f(float lo, float hi) {
  return __hiloint2double(__float_as_int(hi), __float_as_int(lo));
}
__device__ __forceinline__ float unpack_lo(double d) { return __int_as_float(__double2loint(d)); }
__device__ __forceinline__ float unpack_hi(double d) { return __int_as_float(__double2hiint(d)); }

template <typename R4>
__device__ __forceinline__ auto pabs1(const R4& p) -> decltype(p.x) {
  return fabs(p.x) + fabs(p.y) + fabs(p.z);
}

// Intersection of the three planes a, b, c (rows), by Cramer's rule as in
// ConvexCell::compute_triangle_point (convex_cell.cpp:1055-1081), with the
// permanents of the 3x3 minors that bound the rounding error.  Returns the
// corner (x, y, z) and eps, a bound on |corner - exact corner| per
// coordinate plus the rounding of a later dot product with it; eps is +inf
// when the sign of the denominator cannot be certified.
template <typename Real, typename R4>
__device__ __forceinline__ void cramer(const R4& a, const R4& b, const R4& c, Real& x,
                                       Real& y, Real& z, Real& eps) {
  using K = Consts<Real>;
  const Real mxy = b.x * c.y - b.y * c.x, pxy = fabs(b.x * c.y) + fabs(b.y * c.x);
  const Real mxz = b.x * c.z - b.z * c.x, pxz = fabs(b.x * c.z) + fabs(b.z * c.x);
  const Real mxw = b.x * c.w - b.w * c.x, pxw = fabs(b.x * c.w) + fabs(b.w * c.x);
  const Real myz = b.y * c.z - b.z * c.y, pyz = fabs(b.y * c.z) + fabs(b.z * c.y);
  const Real myw = b.y * c.w - b.w * c.y, pyw = fabs(b.y * c.w) + fabs(b.w * c.y);
  const Real mzw = b.z * c.w - b.w * c.z, pzw = fabs(b.z * c.w) + fabs(b.w * c.z);
  const Real W = a.x * myz - a.y * mxz + a.z * mxy;
  const Real X = -(a.w * myz + a.y * mzw - a.z * myw);
  const Real Y = a.x * mzw + a.w * mxz - a.z * mxw;
  const Real Z = -(a.x * myw - a.y * mxw + a.w * mxy);
  const Real pW = fabs(a.x) * pyz + fabs(a.y) * pxz + fabs(a.z) * pxy;
  const Real pX = fabs(a.w) * pyz + fabs(a.y) * pzw + fabs(a.z) * pyw;
  const Real pY = fabs(a.x) * pzw + fabs(a.w) * pxz + fabs(a.z) * pxw;
  const Real pZ = fabs(a.x) * pyw + fabs(a.y) * pxw + fabs(a.w) * pxy;
  const Real inv = Real(1) / W;
  x = X * inv;
  y = Y * inv;
  z = Z * inv;
  const Real cm = fmax(fabs(x), fmax(fabs(y), fabs(z)));
  const Real den = fabs(W) - K::kDet * pW;
  if (!(den > Real(0))) {
    eps = Real(INFINITY);
  } else {
    const Real pm = fmax(pX, fmax(pY, pZ));
    eps = (K::kDet * (pm + cm * pW) / den + Real(2) * K::kUlp * cm + K::kDot * cm) *
          Real(1.0001);
  }
}

// ---------------------------------------------------------------------
// Plane equations
// ---------------------------------------------------------------------
struct SeedCtx {
  double4 pi;   // x, y, z, h
  double qi;    // w - |p|^2
  double wi;
  double box[6];
};

// Power bisector of seed i and the plane's owner in the reference's global
// frame, periodic_delaunay_3d.cpp:3722-3726, or a box face
// (convex_cell.cpp:189-194).  Bit-identical to the reference's plane.
__device__ __forceinline__ double4 plane_fp64(uint32_t ps, const SeedCtx& sc,
                                              const SortedSeeds& S) {
  if (ps >= kBoxBase) {
    switch (ps - kBoxBase) {
      case 0: return make_double4(1.0, 0.0, 0.0, -sc.box[0]);
      case 1: return make_double4(-1.0, 0.0, 0.0, sc.box[3]);
      case 2: return make_double4(0.0, 1.0, 0.0, -sc.box[1]);
      case 3: return make_double4(0.0, -1.0, 0.0, sc.box[4]);
      case 4: return make_double4(0.0, 0.0, 1.0, -sc.box[2]);
      default: return make_double4(0.0, 0.0, -1.0, sc.box[5]);
    }
  }
  const double4 pj = S.xd[ps];
  const double qj = S.q[ps];
  return make_double4(2.0 * __dsub_rn(sc.pi.x, pj.x), 2.0 * __dsub_rn(sc.pi.y, pj.y),
                      2.0 * __dsub_rn(sc.pi.z, pj.z), __dsub_rn(sc.qi, qj));
}

// The same plane translated to the frame centred on seed i, in FP32:
// (-2 d, |d|^2 + w_i - w_j) with d = p_j - p_i rounded from FP64.
__device__ __forceinline__ float4 plane_fp32(uint32_t ps, const SeedCtx& sc,
                                             const SortedSeeds& S, const double* wsorted) {
  if (ps >= kBoxBase) {
    switch (ps - kBoxBase) {
      case 0: return make_float4(1.f, 0.f, 0.f, (float)(sc.pi.x - sc.box[0]));
      case 1: return make_float4(-1.f, 0.f, 0.f, (float)(sc.box[3] - sc.pi.x));
      case 2: return make_float4(0.f, 1.f, 0.f, (float)(sc.pi.y - sc.box[1]));
      case 3: return make_float4(0.f, -1.f, 0.f, (float)(sc.box[4] - sc.pi.y));
      case 4: return make_float4(0.f, 0.f, 1.f, (float)(sc.pi.z - sc.box[2]));
      default: return make_float4(0.f, 0.f, -1.f, (float)(sc.box[5] - sc.pi.z));
    }
  }
  const double4 pj = S.xd[ps];
  const float dx = (float)(pj.x - sc.pi.x), dy = (float)(pj.y - sc.pi.y),
              dz = (float)(pj.z - sc.pi.z);
  const float dw = wsorted ? (float)(wsorted[ps] - sc.wi) : 0.f;
  return make_float4(-2.f * dx, -2.f * dy, -2.f * dz, (dx * dx + dy * dy + dz * dz) - dw);
}

// ---------------------------------------------------------------------
// Geometry of the final cell (FP64): volume, mg and facet areas with the
// fans of ConvexCell::compute_mg / facet_area (convex_cell.cpp:1160-1307).
// ---------------------------------------------------------------------
template <int T, int P, class CornerFn, class TvFn, class TaFn>
struct Geometry {
  CornerFn corner;
  TvFn tv;
  TaFn ta;
  __device__ __forceinline__ int find_vertex(uint32_t t, uint32_t v) const {
    const uint32_t x = tv(t);
    return ((x >> 8 & 0xFF) == v) + 2 * ((x >> 16 & 0xFF) == v);
  }
  __device__ __forceinline__ uint32_t adj(uint32_t t, int e) const {
    return (ta(t) >> (8 * e)) & 0xFF;
  }
};

__device__ __forceinline__ double tet_vol6(double3 p, double3 q, double3 r, double3 s) {
  const double ux = q.x - p.x, uy = q.y - p.y, uz = q.z - p.z;
  const double vx = r.x - p.x, vy = r.y - p.y, vz = r.z - p.z;
  const double wx = s.x - p.x, wy = s.y - p.y, wz = s.z - p.z;
  const double cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
  return fabs(cx * wx + cy * wy + cz * wz);
}

__device__ __forceinline__ double tri_area2(double3 p, double3 q, double3 r) {
  const double ux = q.x - p.x, uy = q.y - p.y, uz = q.z - p.z;
  const double vx = r.x - p.x, vy = r.y - p.y, vz = r.z - p.z;
  const double wx = uy * vz - uz * vy, wy = uz * vx - ux * vz, wz = ux * vy - uy * vx;
  return sqrt(wx * wx + wy * wy + wz * wz);
}

// ---------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------
template <typename Real, int T, int P>
__global__ void __launch_bounds__(kClipThreads)
clip_kernel(ClipArgs a) {
  constexpr int BS = kClipThreads;
  constexpr int NWT = (T + 63) / 64;
  using Smem = CellSmem<Real, BS, T, P>;
  using R4 = typename std::conditional<std::is_same<Real, double>::value, double4, float4>::type;
  constexpr bool kFP64 = std::is_same<Real, double>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  const int tid = threadIdx.x;
  const uint32_t qi = blockIdx.x * BS + tid;
  if (qi >= a.nq) return;
  const SortedSeeds& S = a.S;
  const uint32_t s = a.qlist ? a.qlist[qi] : qi;

  SeedCtx sc;
  sc.pi = S.xd[s];
  sc.qi = S.q[s];
  sc.wi = S.ws ? S.ws[s] : 0.0;
#pragma unroll
  for (int c = 0; c < 6; ++c) sc.box[c] = a.box[c];
  const double hi2 = sc.pi.w * sc.pi.w;

  auto plane_of = [&](uint32_t p) -> R4 {
    if constexpr (kFP64) {
      return plane_fp64(sm.pslot[p][tid], sc, S);
    } else {
      return sm.plane[p][tid];
    }
  };
  auto r2_of = [&](uint32_t t) -> float {
    if constexpr (kFP64) {
      return unpack_lo(sm.corner[t][tid].w);
    } else {
      const float4 c = sm.corner[t][tid];
      return c.x * c.x + c.y * c.y + c.z * c.z;
    }
  };
  // stores the corner of triangle t from its three planes; returns its r2
  auto make_corner = [&](uint32_t t, const R4& pa, const R4& pb, const R4& pc) -> float {
    Real x, y, z, eps;
    cramer<Real>(pa, pb, pc, x, y, z, eps);
    if constexpr (kFP64) {
      const double dx = x - sc.pi.x, dy = y - sc.pi.y, dz = z - sc.pi.z;
      const float r2 = __double2float_ru(dx * dx + dy * dy + dz * dz) * 1.0000002f;
      sm.corner[t][tid] = make_double4(x, y, z, pack2f(r2, __double2float_ru(eps)));
      return r2;
    } else {
      sm.corner[t][tid] = make_float4(x, y, z, eps);
      return x * x + y * y + z * z;
    }
  };

  // ---- init_with_box (convex_cell.cpp:175-215): 6 planes, 8 corners
#pragma unroll
  for (int b = 0; b < 6; ++b) {
    sm.pslot[b][tid] = kBoxBase + b;
    sm.prank[b][tid] = 0xFFFF;
    if constexpr (!kFP64) sm.plane[b][tid] = plane_fp32(kBoxBase + b, sc, S, S.ws);
  }
  {
    // triangles and adjacency of the box, in the reference's order
    const uint32_t bt[8] = {2 | 5 << 8 | 0 << 16, 5 | 3 << 8 | 0 << 16, 1 | 5 << 8 | 2 << 16,
                            5 | 1 << 8 | 3 << 16, 4 | 2 << 8 | 0 << 16, 4 | 0 << 8 | 3 << 16,
                            2 | 4 << 8 | 1 << 16, 4 | 3 << 8 | 1 << 16};
    const uint32_t ba[8] = {1 | 4 << 8 | 2 << 16, 5 | 0 << 8 | 3 << 16, 0 | 6 << 8 | 3 << 16,
                            7 | 1 << 8 | 2 << 16, 0 | 5 << 8 | 6 << 16, 1 | 7 << 8 | 4 << 16,
                            7 | 2 << 8 | 4 << 16, 3 | 6 << 8 | 5 << 16};
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      sm.tv[t][tid] = bt[t];
      sm.ta[t][tid] = ba[t];
    }
  }
  Bits<NWT> valid;
  valid.clear();
  float R2 = 0.f;
  for (int t = 0; t < 8; ++t) {
    valid.set(t);
    const uint32_t v = sm.tv[t][tid];
    float r2 = make_corner(t, plane_of(v & 0xFF), plane_of(v >> 8 & 0xFF), plane_of(v >> 16 & 0xFF));
    R2 = fmaxf(R2, r2);
  }
  uint64_t pused = 0x3Full;
  bool recycled = false;

  const uint32_t row = a.qrow ? a.qrow[qi] : qi;
  const uint32_t cnt_raw = a.nbr_cnt[row];
  const bool dup = (cnt_raw >> 31) != 0;
  const uint32_t cnt = dup ? 0u : cnt_raw;
  int32_t st;
  uint32_t jj = 0;
  uint32_t stop_slot = kNone;
  unsigned long long n_exact = 0;

  if (dup) {
    st = CELL_DUPLICATE;
  } else {
    st = -1;
    for (; jj < cnt; ++jj) {
      const uint32_t j = a.nbr[(size_t)jj * a.nbr_stride + row];
      const double4 pj = S.xd[j];
      // ---- security radius (generic_RVD.h:2300-2324)
      if (a.check_sr) {
        if constexpr (kFP64) {
          const double dij = dist2_exact(sc.pi, pj);
          if (dij > 4.1 * ((double)R2 + hi2)) {
            st = CELL_CERTIFIED;
            stop_slot = j;
            break;
          }
        } else {
          const float dx = (float)(pj.x - sc.pi.x), dy = (float)(pj.y - sc.pi.y),
                      dz = (float)(pj.z - sc.pi.z), dh = (float)(pj.w - sc.pi.w);
          const float dij = dx * dx + dy * dy + dz * dz + dh * dh;
          if (dij > 4.1f * (R2 + (float)hi2)) {
            st = CELL_CERTIFIED;
            stop_slot = j;
            break;
          }
        }
      }
      if (!valid.any()) continue;  // empty cell: nothing left to clip
      // ---- the plane
      R4 Pn;
      Real bw;
      if constexpr (kFP64) {
        Pn = plane_fp64(j, sc, S);
        bw = Consts<double>::kDot * fabs(Pn.w);
      } else {
        Pn = plane_fp32(j, sc, S, S.ws);
        const double qj = S.q[j];
        // rounding of the reference's FP64 planes, seen from FP32
        const float ref_term = (float)(3.5527136788005009e-15 *
                                       (fabs(sc.qi) + fabs(qj) +
                                        (double)pabs1(Pn) * (fmax(fabs(sc.pi.x), fmax(fabs(sc.pi.y), fabs(sc.pi.z))) + 1.0)));
        bw = Consts<float>::kDot * fabsf(Pn.w) + ref_term;
      }
      const Real pa1 = pabs1(Pn) * Real(1.0001);
      bw *= Real(1.0001);
      // ---- conflict scan (triangle_is_in_conflict, convex_cell.cpp:870-912)
      Bits<NWT> conflict;
      conflict.clear();
      float newR2 = 0.f;
      bool uncertain = false;
#pragma unroll
      for (int wi = 0; wi < NWT; ++wi) {
        uint64_t m = valid.w[wi];
        while (m) {
          const int t = wi * 64 + __ffsll((long long)m) - 1;
          m &= m - 1;
          const R4 c = sm.corner[t][tid];
          Real eps;
          if constexpr (kFP64) eps = (double)unpack_hi(c.w);
          else eps = c.w;
          const Real sv = fma(Pn.z, c.z, fma(Pn.y, c.y, fma(Pn.x, c.x, Pn.w)));
          const Real bound = fma(pa1, eps, bw);
          bool in_conflict;
          if (sv < -bound) {
            in_conflict = true;
          } else if (sv > bound) {
            in_conflict = false;
          } else {
            if constexpr (kFP64) {
              const uint32_t v = sm.tv[t][tid];
              const double4 p0 = plane_of(v & 0xFF), p1 = plane_of(v >> 8 & 0xFF),
                            p2 = plane_of(v >> 16 & 0xFF);
              const double r0[4] = {p0.x, p0.y, p0.z, p0.w}, r1[4] = {p1.x, p1.y, p1.z, p1.w},
                           rr2[4] = {p2.x, p2.y, p2.z, p2.w}, r3[4] = {Pn.x, Pn.y, Pn.z, Pn.w};
              in_conflict = det4_sign_exact(r0, r1, rr2, r3) >= 0;
              ++n_exact;
            } else {
              uncertain = true;
              in_conflict = false;
            }
          }
          if (in_conflict) conflict.set(t);
          else newR2 = fmaxf(newR2, r2_of(t));
        }
      }
      if (!kFP64 && uncertain) {
        st = CELL_RECHECK;
        break;
      }
      if (!conflict.any()) continue;
      if (conflict.equals(valid)) {  // the whole cell is clipped away
        valid.clear();
        R2 = 0.f;
        continue;
      }
      // ---- a slot for the new plane (recycle planes no triangle uses)
      uint64_t freep = ~pused & (P >= 64 ? ~0ull : ((1ull << P) - 1ull));
      if (!freep) {
        uint64_t used = 0;
        Bits<NWT> keep = andnot(valid, conflict);
#pragma unroll
        for (int wi = 0; wi < NWT; ++wi) {
          uint64_t m = keep.w[wi];
          while (m) {
            const int t = wi * 64 + __ffsll((long long)m) - 1;
            m &= m - 1;
            const uint32_t v = sm.tv[t][tid];
            used |= (1ull << (v & 0xFF)) | (1ull << (v >> 8 & 0xFF)) | (1ull << (v >> 16 & 0xFF));
          }
        }
        pused = used;
        recycled = true;
        freep = ~pused & (P >= 64 ? ~0ull : ((1ull << P) - 1ull));
        if (!freep) {
          st = CELL_OVERFLOW;
          break;
        }
      }
      const uint32_t lv = (uint32_t)(__ffsll((long long)freep) - 1);
      pused |= 1ull << lv;
      sm.pslot[lv][tid] = j;
      sm.prank[lv][tid] = (uint16_t)jj;
      if constexpr (!kFP64) sm.plane[lv][tid] = Pn;
      // ---- border of the conflict zone (triangulate_conflict_zone)
      int nborder = 0;
      uint32_t first_v = 0;
#pragma unroll
      for (int wi = 0; wi < NWT; ++wi) {
        uint64_t m = conflict.w[wi];
        while (m) {
          const int t = wi * 64 + __ffsll((long long)m) - 1;
          m &= m - 1;
          const uint32_t v = sm.tv[t][tid], ad = sm.ta[t][tid];
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            const uint32_t nb = (ad >> (8 * e)) & 0xFF;
            if (conflict.test((int)nb)) continue;
            // edge opposite vertex e runs v[e+1] -> v[e+2] in t; the kept
            // triangle nb holds it reversed, so walking the border along
            // nb's orientation goes v[e+2] -> v[e+1]
            const uint32_t x = (v >> (8 * ((e + 1) % 3))) & 0xFF;
            const uint32_t y = (v >> (8 * ((e + 2) % 3))) & 0xFF;
            const uint32_t an = sm.ta[nb][tid];
            const uint32_t eb = ((an >> 8 & 0xFF) == (uint32_t)t) + 2 * ((an >> 16 & 0xFF) == (uint32_t)t);
            sm.pnext[y][tid] = (uint8_t)x;
            sm.pnb[y][tid] = (uint16_t)(nb | (eb << 8));
            first_v = y;
            ++nborder;
          }
        }
      }
      const int nkeep = valid.popc() - conflict.popc();
      if (nkeep + nborder > T) {
        st = CELL_OVERFLOW;
        break;
      }
      // ---- fan new triangles (lv, next, v) around the border
      Bits<NWT> freet = andnot(full_bits<NWT>(T), andnot(valid, conflict));
      valid = andnot(valid, conflict);
      R2 = newR2;
      uint32_t v = first_v;
      int prev_t = -1, first_t = -1;
      R4 Pv = plane_of(v);
      int steps = 0;
      do {
        if (++steps > nborder) break;  // not a simple cycle: reported below
        const uint32_t x = sm.pnext[v][tid];
        const uint32_t nbinfo = sm.pnb[v][tid];
        const uint32_t tn = nbinfo & 0xFF, eb = nbinfo >> 8;
        const int nt = freet.first();
        freet.w[nt >> 6] &= ~(1ull << (nt & 63));
        valid.set(nt);
        sm.tv[nt][tid] = lv | (x << 8) | (v << 16);
        sm.ta[nt][tid] = tn | ((uint32_t)(prev_t < 0 ? 0 : prev_t) << 8);
        {
          uint32_t an = sm.ta[tn][tid];
          an = (an & ~(0xFFu << (8 * eb))) | ((uint32_t)nt << (8 * eb));
          sm.ta[tn][tid] = an;
        }
        const R4 Px = plane_of(x);
        const float r2 = make_corner(nt, Pn, Px, Pv);
        R2 = fmaxf(R2, r2);
        if (prev_t >= 0) {
          uint32_t ap = sm.ta[prev_t][tid];
          sm.ta[prev_t][tid] = (ap & 0x0000FFFFu) | ((uint32_t)nt << 16);
        } else {
          first_t = nt;
        }
        prev_t = nt;
        v = x;
        Pv = Px;
      } while (v != first_v);
      if (v != first_v || steps != nborder) {
        st = CELL_ERROR;
        break;
      }
      {
        uint32_t ap = sm.ta[prev_t][tid];
        sm.ta[prev_t][tid] = (ap & 0x0000FFFFu) | ((uint32_t)first_t << 16);
        uint32_t af = sm.ta[first_t][tid];
        sm.ta[first_t][tid] = (af & 0xFFFF00FFu) | ((uint32_t)prev_t << 8);
      }
    }
    if (st < 0) {
      // list exhausted without certification
      const bool complete = (cnt < a.list_k) || (a.list_k >= a.n_total - 1);
      st = (complete || !a.check_sr) ? (a.check_sr ? CELL_ALL_NEIGHBOURS : CELL_CERTIFIED)
                                     : CELL_NEED_MORE_K;
    }
  }
  if (a.counters) {
    if (n_exact) atomicAdd(&a.counters[0], n_exact);
    const unsigned amask = __activemask();
    const unsigned mx = __reduce_max_sync(amask, jj);
    if ((unsigned)(tid & 31) == (unsigned)(__ffs(amask) - 1))
      atomicMax(&a.counters[1], (unsigned long long)mx);
  }

  if (st == CELL_RECHECK || st == CELL_OVERFLOW || st == CELL_NEED_MORE_K ||
      st == CELL_ERROR) {
    a.status[s] = st;
    a.nclip[s] = jj;
    return;
  }

  // ---- FP64 corners of the final cell
  // FP64 kernel: cached.  FP32 kernel: recomputed from the reference's
  // FP64 planes into the space of the FP32 corners and planes.
  auto corner64 = [&](uint32_t t) -> double3 {
    if constexpr (kFP64) {
      const double4 c = sm.corner[t][tid];
      return make_double3(c.x, c.y, c.z);
    } else {
      const double2 xy = reinterpret_cast<const double2(*)[BS]>(&sm.corner[0][0])[t][tid];
      const double zz = reinterpret_cast<const double(*)[BS]>(&sm.plane[0][0])[t][tid];
      return make_double3(xy.x, xy.y, zz);
    }
  };
  if constexpr (!kFP64) {
    static_assert(sizeof(sm.plane) >= sizeof(double) * T * BS, "plane space too small");
    double R2_64 = 0.0;
#pragma unroll
    for (int wi = 0; wi < NWT; ++wi) {
      uint64_t m = valid.w[wi];
      while (m) {
        const int t = wi * 64 + __ffsll((long long)m) - 1;
        m &= m - 1;
        const uint32_t v = sm.tv[t][tid];
        const double4 p0 = plane_fp64(sm.pslot[v & 0xFF][tid], sc, S);
        const double4 p1 = plane_fp64(sm.pslot[v >> 8 & 0xFF][tid], sc, S);
        const double4 p2 = plane_fp64(sm.pslot[v >> 16 & 0xFF][tid], sc, S);
        double x, y, z, eps;
        cramer<double>(p0, p1, p2, x, y, z, eps);
        reinterpret_cast<double2(*)[BS]>(&sm.corner[0][0])[t][tid] = make_double2(x, y);
        reinterpret_cast<double(*)[BS]>(&sm.plane[0][0])[t][tid] = z;
        const double dx = x - sc.pi.x, dy = y - sc.pi.y, dz = z - sc.pi.z;
        R2_64 = fmax(R2_64, dx * dx + dy * dy + dz * dz);
      }
    }
    // the FP32 stop must also hold in FP64
    if (st == CELL_CERTIFIED && stop_slot != kNone) {
      const double dij = dist2_exact(sc.pi, S.xd[stop_slot]);
      if (!(dij > 4.1 * (R2_64 + hi2))) {
        a.status[s] = CELL_RECHECK;
        a.nclip[s] = jj;
        return;
      }
    }
  }

  // ---- v2t (pnext reused): one triangle per contributing plane
#pragma unroll
  for (int p = 0; p < P; ++p) sm.pnext[p][tid] = 0xFF;
#pragma unroll
  for (int wi = 0; wi < NWT; ++wi) {
    uint64_t m = valid.w[wi];
    while (m) {
      const int t = wi * 64 + __ffsll((long long)m) - 1;
      m &= m - 1;
      const uint32_t v = sm.tv[t][tid];
      sm.pnext[v & 0xFF][tid] = (uint8_t)t;
      sm.pnext[v >> 8 & 0xFF][tid] = (uint8_t)t;
      sm.pnext[v >> 16 & 0xFF][tid] = (uint8_t)t;
    }
  }
  auto find_vertex = [&](uint32_t t, uint32_t v) -> int {
    const uint32_t x = sm.tv[t][tid];
    return ((x >> 8 & 0xFF) == v) + 2 * ((x >> 16 & 0xFF) == v);
  };
  auto adjacent = [&](uint32_t t, int e) -> uint32_t { return (sm.ta[t][tid] >> (8 * e)) & 0xFF; };

  // ---- volume and mg (compute_mg): fans of tets from one corner
  double m = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
  {
    int t_origin = -1;
    double3 po = make_double3(0, 0, 0);
    for (int p = 0; p < P; ++p) {
      const uint32_t t0 = sm.pnext[p][tid];
      if (t0 == 0xFF) continue;
      if (t_origin < 0) {
        t_origin = (int)t0;
        po = corner64(t0);
        continue;
      }
      uint32_t t = t0;
      int cur = 0;
      double3 q1 = make_double3(0, 0, 0), q2 = q1;
      int guard = 0;
      do {
        const double3 pt = corner64(t);
        if (cur == 0) q1 = pt;
        else if (cur == 1) q2 = pt;
        else {
          const double cm = tet_vol6(po, q1, q2, pt) / 6.0;
          m += cm;
          gx += cm * (po.x + q1.x + q2.x + pt.x) / 4.0;
          gy += cm * (po.y + q1.y + q2.y + pt.y) / 4.0;
          gz += cm * (po.z + q1.z + q2.z + pt.z) / 4.0;
          q2 = pt;
        }
        ++cur;
        const int lvx = find_vertex(t, (uint32_t)p);
        t = adjacent(t, (lvx + 1) % 3);
      } while (t != t0 && ++guard < T);
    }
  }
  a.vol[s] = m;
  a.mg[s] = gx;
  a.mg[(size_t)a.out_stride + s] = gy;
  a.mg[2 * (size_t)a.out_stride + s] = gz;

  // ---- facets between seeds, in the reference's order (clipping order)
  uint32_t nfac = 0;
  for (int p = 0; p < P; ++p) {
    const uint32_t t0 = sm.pnext[p][tid];
    const uint32_t ps = sm.pslot[p][tid];
    if (t0 == 0xFF || ps >= kBoxBase) continue;
    double area = 0.0;
    uint32_t t = t0;
    int cur = 0;
    double3 q0 = make_double3(0, 0, 0), q1 = q0;
    int guard = 0;
    do {
      const double3 pt = corner64(t);
      if (cur == 0) q0 = pt;
      else if (cur == 1) q1 = pt;
      else {
        area += 0.5 * tri_area2(q0, q1, pt);
        q1 = pt;
      }
      ++cur;
      const int lvx = find_vertex(t, (uint32_t)p);
      t = adjacent(t, (lvx + 1) % 3);
    } while (t != t0 && ++guard < T);
    uint32_t pos = nfac;
    if (recycled) {
      // order among contributing seed planes by list position
      pos = 0;
      const uint16_t rk = sm.prank[p][tid];
      for (int p2 = 0; p2 < P; ++p2) {
        if (sm.pnext[p2][tid] == 0xFF || sm.pslot[p2][tid] >= kBoxBase) continue;
        pos += (sm.prank[p2][tid] < rk);
      }
    }
    a.f_nbr[(size_t)pos * a.out_stride + s] = S.perm[ps];
    a.f_area[(size_t)pos * a.out_stride + s] = area;
    ++nfac;
  }
  a.nf[s] = nfac;
  a.nclip[s] = jj;
  a.status[s] = st;
}

template <typename Real, int T, int P>
static void launch_clip(const ClipArgs& a, cudaStream_t st) {
  if (a.nq == 0) return;
  const size_t sh = sizeof(CellSmem<Real, kClipThreads, T, P>);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(clip_kernel<Real, T, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sh);
    configured = true;
  }
  const unsigned nb = (a.nq + kClipThreads - 1) / kClipThreads;
  clip_kernel<Real, T, P><<<nb, kClipThreads, sh, st>>>(a);
  last_launch_error = cudaGetLastError();
}

void launch_clip_fp64(const ClipArgs& a, int shape, cudaStream_t st) {
  if (shape == CLIP_SMALL) launch_clip<double, kSmallT, kSmallP>(a, st);
  else launch_clip<double, kLargeT, kLargeP>(a, st);
}

void launch_clip_fp32(const ClipArgs& a, cudaStream_t st) {
  launch_clip<float, kSmallT, kSmallP>(a, st);
}

}  // namespace gbv
