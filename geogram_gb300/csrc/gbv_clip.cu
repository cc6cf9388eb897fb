// Laguerre cell clipping: one thread per cell, the polytope in shared
// memory laid out [slot][thread] so that a warp's 32 cells touch 32
// consecutive words.
//
// The cell is kept in the dual form of the reference's VBW::ConvexCell
// (voronoi/convex_cell.h:419-1436): every clipping plane is a vertex,
// every corner of the polytope is a triangle of three planes with its three
// adjacent triangles.  Clipping by a plane (convex_cell.cpp:461-516,
// 761-865) removes the triangles whose corner lies on the negative side and
// fans new triangles from the new plane around the border of the removed
// zone.  What differs from the CPU code is layout and bookkeeping:
//   - triangles live in fixed slots tracked by bit masks instead of linked
//     lists; planes in slots recycled once no triangle uses them;
//   - the reference's valid-list order, which decides how its geometry
//     fans are rooted, is carried as one key per triangle (see below);
//   - each triangle caches its corner and a bound on the corner's rounding
//     error, so a conflict test is three FMAs and a compare.  When the
//     bound cannot decide the sign, the FP64 kernel evaluates the exact
//     determinant sign (the reference's PCK::det_4d decision) and the FP32
//     kernel marks the cell for an FP64 re-clip;
//   - the security-radius test (generic_RVD.h:2278-2352) reads the cached
//     corner radii.
// The kernel writes the cell's combinatorics; gbv_geom.cu turns them into
// volume, centroid and facet areas.
//
// List-order keys.  The reference rebuilds its valid-triangle list at every
// clip: survivors are relinked in reverse order, then the new triangles are
// pushed at the head in creation order; the border walk starts at the
// border edge met last while scanning that list.  With an "effective key"
// eff = parity * key per triangle and the list read in ascending eff, one
// clip is: parity flips (survivors reversed, nothing rewritten), the c-th
// new triangle gets eff = -(max eff of the survivors) - 1 - c, and the walk
// starts at the border edge maximising (new eff of the kept triangle, edge).
#include <cfloat>
#include <cmath>
#include <type_traits>

#include "gbv_clip.cuh"
#include "gbv_exact.cuh"
#include "gbv_refgeom.cuh"
#include "gbv_corner.cuh"

namespace gbv {

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
  __device__ __forceinline__ void reset(int i) { w[i >> 6] &= ~(1ull << (i & 63)); }
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
// Per-thread cell storage in shared memory, [slot][thread]
// ---------------------------------------------------------------------
template <typename Real, int BS, int T, int P>
struct CellSmem;

template <int BS, int T, int P>
struct CellSmem<double, BS, T, P> {
  double2 cxy[T][BS];     // corner x, y (reference frame and arithmetic)
  double2 czr[T][BS];     // corner z, squared distance to the seed
  float eps[T][BS];       // corner error bound (cramer_bound)
  uint32_t tv[T][BS];     // planes i | j << 8 | k << 16
  uint32_t ta[T][BS];     // triangles across the edges opposite i, j, k
  int16_t key[T][BS];
  uint32_t pown[P][BS];   // plane owner: seed slot or kBoxBase + face
  uint16_t prank[P][BS];  // list position of the plane's seed
  uint16_t pnb[P][BS];    // border scratch: kept triangle | edge << 8
  uint8_t pnext[P][BS];   // border scratch: next border plane
};

template <int BS, int T, int P>
struct CellSmem<float, BS, T, P> {
  float4 c4[T][BS];       // corner x, y, z (frame centred on the seed), eps
  uint32_t tv[T][BS];
  uint32_t ta[T][BS];
  int16_t key[T][BS];
  float4 pl[P][BS];       // local-frame plane equations
  uint16_t prank[P][BS];
  uint16_t pnb[P][BS];
  uint8_t pnext[P][BS];
};

// ---------------------------------------------------------------------
// Plane equations
// ---------------------------------------------------------------------
struct SeedCtx {
  double4 pi;     // x, y, z, h
  double qi;      // w - |p|^2
  float4 fh, fl;  // FP32 value and remainder of (x, y, z, h)
  float2 fw;      // FP32 value and remainder of w
  double box[6];
};

// Power bisector of seed i and the plane's owner in the reference's global
// frame, periodic_delaunay_3d.cpp:3722-3726, or a box face
// (convex_cell.cpp:189-194).  Bit-identical to the reference's plane.
__device__ __forceinline__ double4 plane_fp64(uint32_t own, const double4& pi, double qi,
                                              const double* box, const SortedSeeds& S) {
  if (own >= kBoxBase) {
    switch (own - kBoxBase) {
      case 0: return make_double4(1.0, 0.0, 0.0, -box[0]);
      case 1: return make_double4(-1.0, 0.0, 0.0, box[3]);
      case 2: return make_double4(0.0, 1.0, 0.0, -box[1]);
      case 3: return make_double4(0.0, -1.0, 0.0, box[4]);
      case 4: return make_double4(0.0, 0.0, 1.0, -box[2]);
      default: return make_double4(0.0, 0.0, -1.0, box[5]);
    }
  }
  const double4 pj = S.xd[own];
  const double qj = S.q[own];
  return make_double4(2.0 * __dsub_rn(pi.x, pj.x), 2.0 * __dsub_rn(pi.y, pj.y),
                      2.0 * __dsub_rn(pi.z, pj.z), __dsub_rn(qi, qj));
}

// A box face in the frame centred on the seed, in FP32.
__device__ __forceinline__ float4 box_plane_fp32(int b, const SeedCtx& sc) {
  switch (b) {
    case 0: return make_float4(1.f, 0.f, 0.f, (sc.fh.x - (float)sc.box[0]) + sc.fl.x);
    case 1: return make_float4(-1.f, 0.f, 0.f, ((float)sc.box[3] - sc.fh.x) - sc.fl.x);
    case 2: return make_float4(0.f, 1.f, 0.f, (sc.fh.y - (float)sc.box[1]) + sc.fl.y);
    case 3: return make_float4(0.f, -1.f, 0.f, ((float)sc.box[4] - sc.fh.y) - sc.fl.y);
    case 4: return make_float4(0.f, 0.f, 1.f, (sc.fh.z - (float)sc.box[2]) + sc.fl.z);
    default: return make_float4(0.f, 0.f, -1.f, ((float)sc.box[5] - sc.fh.z) - sc.fl.z);
  }
}

// The reference's conflict decision for the triangle of planes p0, p1, p2
// and the clipping plane pj: det4 >= 0 exactly (PCK::det_4d), or the FP64
// det4x4 > 0 with the fast predicates.  Out of line: the FP32 kernel needs
// it only when its own bound cannot decide, and its expansion arithmetic
// would otherwise weigh on the registers of the conflict loop.
__device__ __noinline__ bool exact_conflict(double4 p0, double4 p1, double4 p2, double4 pj,
                                            int fast) {
  if (fast) return r_det4x4(p0, p1, p2, pj) > 0.0;
  const double r0[4] = {p0.x, p0.y, p0.z, p0.w}, r1[4] = {p1.x, p1.y, p1.z, p1.w},
               r2[4] = {p2.x, p2.y, p2.z, p2.w}, r3[4] = {pj.x, pj.y, pj.z, pj.w};
  return det4_sign_exact(r0, r1, r2, r3) >= 0;
}

// ---------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------
// XF (FP32 only): a sign the FP32 bound cannot decide is taken exactly from
// the FP64 planes; without it the cell is marked for a recheck (a leaner
// loop for the first pass over every cell).
template <typename Real, int T, int P, bool XF>
__global__ void __launch_bounds__(kClipThreads) clip_kernel(ClipArgs a) {
  constexpr int BS = kClipThreads;
  constexpr int NWT = (T + 63) / 64;
  constexpr bool kFP64 = std::is_same<Real, double>::value;
  using Smem = CellSmem<Real, BS, T, P>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  const int tid = threadIdx.x;
  const uint32_t qi = blockIdx.x * BS + tid;
  if (qi >= a.nq) return;
  const SortedSeeds& S = a.S;
  const uint32_t s = a.qlist ? a.qlist[qi] : qi;
  const uint32_t row = a.qrow ? a.qrow[qi] : qi;

  SeedCtx sc;
  sc.pi = S.xd[s];
#pragma unroll
  for (int c = 0; c < 6; ++c) sc.box[c] = a.box[c];
  if constexpr (kFP64) {
    sc.qi = S.q[s];
  } else {
    sc.fh = S.xf[s];
    sc.fl = S.xl[s];
    sc.fw = S.wf ? S.wf[s] : make_float2(0.f, 0.f);
  }
  const double hi2 = __dmul_rn(sc.pi.w, sc.pi.w);
  const float hi2f = sc.fh.w * sc.fh.w;

  // Plane p's equation (FP64: recomputed from its owner, FP32: stored).
  auto plane_of = [&](uint32_t p) {
    if constexpr (kFP64) return plane_fp64(sm.pown[p][tid], sc.pi, sc.qi, sc.box, S);
    else return sm.pl[p][tid];
  };
  // The reference's FP64 plane of plane slot p (FP32 kernel: from its list
  // position, box faces keep their slots 0-5) and of seed slot j.
  auto plane64_of = [&](uint32_t j) -> double4 {
    return plane_fp64(j, sc.pi, S.q[s], sc.box, S);
  };
  auto plane64 = [&](uint32_t p) -> double4 {
    if constexpr (kFP64) {
      return plane_fp64(sm.pown[p][tid], sc.pi, sc.qi, sc.box, S);
    } else {
      const uint16_t rk = sm.prank[p][tid];
      const uint32_t own =
          (rk == 0xFFFF) ? kBoxBase + p : a.nbr[(size_t)rk * a.nbr_stride + row];
      return plane_fp64(own, sc.pi, S.q[s], sc.box, S);
    }
  };
  // Creates the corner of triangle t from its planes; returns its r2.
  auto make_corner = [&](uint32_t t, const auto& pa, const auto& pb, const auto& pc) -> Real {
    if constexpr (kFP64) {
      double x, y, z;
      float e;
      corner_fp64(pa, pb, pc, x, y, z, e);
      const double r2 = r_sqdist(sc.pi.x, sc.pi.y, sc.pi.z, make_double3(x, y, z));
      sm.cxy[t][tid] = make_double2(x, y);
      sm.czr[t][tid] = make_double2(z, r2);
      sm.eps[t][tid] = e;
      return r2;
    } else {
      float x, y, z, e;
      corner_fp32(pa, pb, pc, x, y, z, e);
      sm.c4[t][tid] = make_float4(x, y, z, e);
      return x * x + y * y + z * z;
    }
  };

  // ---- init_with_box (convex_cell.cpp:175-215): 6 planes, 8 corners
#pragma unroll
  for (int b = 0; b < 6; ++b) {
    sm.prank[b][tid] = 0xFFFF;
    if constexpr (kFP64) sm.pown[b][tid] = kBoxBase + b;
    else sm.pl[b][tid] = box_plane_fp32(b, sc);
  }
  {
    // triangles and adjacency of the box corners, in the reference's order
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
      sm.key[t][tid] = (int16_t)(-t);  // each pushed at the head of the list
    }
  }
  Bits<NWT> valid;
  valid.clear();
  Real R2 = 0;
  for (int t = 0; t < 8; ++t) {
    valid.set(t);
    const uint32_t v = sm.tv[t][tid];
    const Real r2 = make_corner(t, plane_of(v & 0xFF), plane_of(v >> 8 & 0xFF),
                                plane_of(v >> 16 & 0xFF));
    R2 = fmax(R2, r2);
  }
  uint64_t pused = 0x3Full;
  int parity = 1;

  const uint32_t cnt_raw = a.nbr_cnt[row];
  const bool dup = (cnt_raw >> 31) != 0;
  const uint32_t copies = (cnt_raw >> 24) & 0x7Fu;
  // a seed with higher-index copies: the reference stops growing its list
  // at reference_list_cap, certified or not
  const uint32_t cap = copies ? reference_list_cap(a.k0, a.n_total, copies, a.check_sr != 0)
                              : 0xFFFFFFFFu;
  const uint32_t cnt = dup ? 0u : min(cnt_raw & kCntMask, cap);
  int32_t st = -1;
  uint32_t jj = 0;
  unsigned long long n_exact = 0;
  uint32_t n_tests = 0, n_created = 0;  // conflict tests, corners made (the flop model)

  if (dup) {
    st = CELL_DUPLICATE;
  } else {
    for (; jj < cnt; ++jj) {
      const uint32_t j = a.nbr[(size_t)jj * a.nbr_stride + row];
      // ---- security radius (generic_RVD.h:2300-2324) and the plane
      float4 Pf = make_float4(0.f, 0.f, 0.f, 0.f);
      double4 Pd = make_double4(0.0, 0.0, 0.0, 0.0);
      if constexpr (kFP64) {
        const double4 pj = S.xd[j];
        if (a.check_sr) {
          const double dij = dist2_exact(sc.pi, pj);
          if (dij > __dmul_rn(4.1, __dadd_rn(R2, hi2))) {
            st = CELL_CERTIFIED;
            break;
          }
        }
        Pd = make_double4(2.0 * __dsub_rn(sc.pi.x, pj.x), 2.0 * __dsub_rn(sc.pi.y, pj.y),
                          2.0 * __dsub_rn(sc.pi.z, pj.z), __dsub_rn(sc.qi, S.q[j]));
      } else {
        // d = p_j - p_i from the value/remainder pairs keeps FP32 relative
        // accuracy however close the two seeds are
        const float4 jh = S.xf[j], jl = S.xl[j];
        const float dx = (jh.x - sc.fh.x) + (jl.x - sc.fl.x);
        const float dy = (jh.y - sc.fh.y) + (jl.y - sc.fl.y);
        const float dz = (jh.z - sc.fh.z) + (jl.z - sc.fl.z);
        const float dh = (jh.w - sc.fh.w) + (jl.w - sc.fl.w);
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (a.check_sr && d2 + dh * dh > 4.1f * (R2 + hi2f)) {
          st = CELL_CERTIFIED;
          break;
        }
        float dw = 0.f;
        if (S.wf) {
          const float2 wj = S.wf[j];
          dw = (wj.x - sc.fw.x) + (wj.y - sc.fw.y);
        }
        // (-2 d, |d|^2 + w_i - w_j): the bisector in the seed's frame
        Pf = make_float4(-2.f * dx, -2.f * dy, -2.f * dz, d2 - dw);
      }
      // every clip relinks the reference's valid list in reverse order
      const int par_old = parity;
      parity = -parity;
      if (!valid.any()) continue;  // empty cell: nothing left to clip
      Real pa1, bw;
      if constexpr (kFP64) {
        pa1 = (fabs(Pd.x) + fabs(Pd.y) + fabs(Pd.z)) * 1.0001;
        bw = Consts<double>::kDot * fabs(Pd.w) * 1.0001;
      } else {
        pa1 = (fabsf(Pf.x) + fabsf(Pf.y) + fabsf(Pf.z)) * 1.0001f;
        // the reference's own FP64 planes carry a rounding of about
        // 2^-52 (|w_i| + |w_j| + |p_i|^2 + |p_j|^2) in their offset
        const float wj = S.wf ? S.wf[j].x : 0.f;
        const float pn = sc.fh.x * sc.fh.x + sc.fh.y * sc.fh.y + sc.fh.z * sc.fh.z;
        const float qmag = fabsf(sc.fw.x) + fabsf(wj) + 2.f * pn + 1.f;
        bw = (Consts<float>::kDot * fabsf(Pf.w) + 3.5527137e-15f * qmag) * 1.0001f;
      }
      // ---- conflict scan (triangle_is_in_conflict, convex_cell.cpp:870-912)
      Bits<NWT> conflict;
      conflict.clear();
      Real keepR2 = 0;
      int keep_max_eff = -0x7FFF;
      bool uncertain = false;
      auto test = [&](int t) {
        ++n_tests;
        Real cx, cy, cz, r2, eps;
        if constexpr (kFP64) {
          const double2 xy = sm.cxy[t][tid], zr = sm.czr[t][tid];
          cx = xy.x;
          cy = xy.y;
          cz = zr.x;
          r2 = zr.y;
          eps = (double)sm.eps[t][tid];
        } else {
          const float4 c = sm.c4[t][tid];
          cx = c.x;
          cy = c.y;
          cz = c.z;
          eps = c.w;
          r2 = cx * cx + cy * cy + cz * cz;
        }
        Real sv;
        if constexpr (kFP64) sv = fma(Pd.z, cz, fma(Pd.y, cy, fma(Pd.x, cx, Pd.w)));
        else sv = fmaf(Pf.z, cz, fmaf(Pf.y, cy, fmaf(Pf.x, cx, Pf.w)));
        const Real bound = fma(pa1, eps, bw) * (a.fast_pred ? (Real)kFastPredWide : (Real)1);
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
            if (a.fast_pred) {
              in_conflict = r_det4x4(p0, p1, p2, Pd) > 0.0;
            } else {
              const double r0[4] = {p0.x, p0.y, p0.z, p0.w}, r1[4] = {p1.x, p1.y, p1.z, p1.w},
                           rr2[4] = {p2.x, p2.y, p2.z, p2.w}, r3[4] = {Pd.x, Pd.y, Pd.z, Pd.w};
              in_conflict = det4_sign_exact(r0, r1, rr2, r3) >= 0;
            }
            ++n_exact;
          } else if constexpr (XF) {
            // FP32 cannot decide: the exact sign of the reference's FP64
            // planes decides, as in the FP64 kernel
            const uint32_t v = sm.tv[t][tid];
            in_conflict = exact_conflict(plane64(v & 0xFF), plane64(v >> 8 & 0xFF),
                                         plane64(v >> 16 & 0xFF), plane64_of(j), a.fast_pred);
            ++n_exact;
          } else {
            uncertain = true;
            in_conflict = false;
          }
        }
        if (in_conflict) {
          conflict.set(t);
        } else {
          keepR2 = fmax(keepR2, r2);
          keep_max_eff = max(keep_max_eff, par_old * (int)sm.key[t][tid]);
        }
      };
#pragma unroll
      for (int wi = 0; wi < NWT; ++wi) {
        uint64_t m = valid.w[wi];
        while (m) {
          // four triangles per iteration, so that their loads overlap
          const int t0 = wi * 64 + __ffsll((long long)m) - 1;
          m &= m - 1;
          int t1 = -1, t2 = -1, t3 = -1;
          if (m) { t1 = wi * 64 + __ffsll((long long)m) - 1; m &= m - 1; }
          if (m) { t2 = wi * 64 + __ffsll((long long)m) - 1; m &= m - 1; }
          if (m) { t3 = wi * 64 + __ffsll((long long)m) - 1; m &= m - 1; }
          test(t0);
          if (t1 >= 0) test(t1);
          if (t2 >= 0) test(t2);
          if (t3 >= 0) test(t3);
        }
      }
      if (!kFP64 && uncertain) {
        st = CELL_RECHECK;
        break;
      }
      if (!conflict.any()) continue;
      if (conflict.equals(valid)) {  // the whole cell is clipped away
        valid.clear();
        R2 = 0;
        continue;
      }
      // ---- a slot for the new plane (recycle planes no triangle uses)
      const uint64_t pmask = (P >= 64) ? ~0ull : ((1ull << P) - 1ull);
      uint64_t freep = ~pused & pmask;
      if (!freep) {
        uint64_t used = 0;
        const Bits<NWT> keep = andnot(valid, conflict);
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
        freep = ~pused & pmask;
        if (!freep) {
          st = CELL_OVERFLOW;
          break;
        }
      }
      const uint32_t lv = (uint32_t)(__ffsll((long long)freep) - 1);
      pused |= 1ull << lv;
      sm.prank[lv][tid] = (uint16_t)jj;
      if constexpr (kFP64) sm.pown[lv][tid] = j;
      else sm.pl[lv][tid] = Pf;
      // ---- border of the conflict zone (triangulate_conflict_zone)
      int nborder = 0;
      uint32_t first_v = 0;
      int best = -0x7FFFFFFF;
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
            // triangle nb holds it reversed, so the border walk, which
            // follows nb's orientation, goes from y = v[e+2] to x = v[e+1]
            const uint32_t x = (v >> (8 * ((e + 1) % 3))) & 0xFF;
            const uint32_t y = (v >> (8 * ((e + 2) % 3))) & 0xFF;
            const uint32_t an = sm.ta[nb][tid];
            const uint32_t eb =
                ((an >> 8 & 0xFF) == (uint32_t)t) + 2 * ((an >> 16 & 0xFF) == (uint32_t)t);
            sm.pnext[y][tid] = (uint8_t)x;
            sm.pnb[y][tid] = (uint16_t)(nb | (eb << 8));
            // the reference starts its walk at the border edge it meets last
            // while scanning the relinked list (new eff = -old eff)
            const int score = -par_old * (int)sm.key[nb][tid] * 4 + (int)eb;
            if (score > best) {
              best = score;
              first_v = y;
            }
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
      R2 = keepR2;
      const int key_base = -keep_max_eff - 1;
      uint32_t v = first_v;
      int prev_t = -1, first_t = -1, created = 0;
      auto Pv = plane_of(v);
      do {
        if (created >= nborder) break;  // not a simple cycle: reported below
        const uint32_t x = sm.pnext[v][tid];
        const uint32_t nbinfo = sm.pnb[v][tid];
        const uint32_t tn = nbinfo & 0xFF, eb = nbinfo >> 8;
        const int nt = freet.first();
        freet.reset(nt);
        valid.set(nt);
        sm.tv[nt][tid] = lv | (x << 8) | (v << 16);
        sm.ta[nt][tid] = tn | ((uint32_t)(prev_t < 0 ? 0 : prev_t) << 8);
        sm.key[nt][tid] = (int16_t)(parity * (key_base - created));
        {
          uint32_t an = sm.ta[tn][tid];
          an = (an & ~(0xFFu << (8 * eb))) | ((uint32_t)nt << (8 * eb));
          sm.ta[tn][tid] = an;
        }
        const auto Px = plane_of(x);
        Real r2;
        if constexpr (kFP64) r2 = make_corner(nt, Pd, Px, Pv);
        else r2 = make_corner(nt, Pf, Px, Pv);
        R2 = fmax(R2, r2);
        if (prev_t >= 0) {
          const uint32_t ap = sm.ta[prev_t][tid];
          sm.ta[prev_t][tid] = (ap & 0x0000FFFFu) | ((uint32_t)nt << 16);
        } else {
          first_t = nt;
        }
        prev_t = nt;
        ++created;
        ++n_created;
        v = x;
        Pv = Px;
      } while (v != first_v);
      if (v != first_v || created != nborder) {
        st = CELL_ERROR;
        break;
      }
      {
        const uint32_t ap = sm.ta[prev_t][tid];
        sm.ta[prev_t][tid] = (ap & 0x0000FFFFu) | ((uint32_t)first_t << 16);
        const uint32_t af = sm.ta[first_t][tid];
        sm.ta[first_t][tid] = (af & 0xFFFF00FFu) | ((uint32_t)prev_t << 8);
      }
    }
    if (st < 0) {
      // list exhausted without certification
      const bool complete = ((cnt_raw & kCntMask) < a.list_k) || (a.list_k >= a.n_total - 1);
      if (!a.check_sr) st = CELL_CERTIFIED;
      else if (copies && cnt == cap) st = (cap == 0) ? CELL_DUPLICATE : CELL_STALLED;
      else st = complete ? CELL_ALL_NEIGHBOURS : CELL_NEED_MORE_K;
    }
  }
  if (a.counters) {
    if (n_exact) atomicAdd(&a.counters[0], n_exact);
    const unsigned amask = __activemask();
    const unsigned mx = __reduce_max_sync(amask, jj);
    const unsigned nt = __reduce_add_sync(amask, n_tests);
    const unsigned nc = __reduce_add_sync(amask, n_created);
    if ((unsigned)(tid & 31) == (unsigned)(__ffs(amask) - 1)) {
      atomicMax(&a.counters[1], (unsigned long long)mx);
      atomicAdd(&a.counters[2], (unsigned long long)nt);
      atomicAdd(&a.counters[3], (unsigned long long)nc);
    }
  }
  a.status[s] = st;
  a.nclip[s] = jj;
  if (st == CELL_RECHECK || st == CELL_OVERFLOW || st == CELL_NEED_MORE_K || st == CELL_ERROR)
    return;

  // ---- the combinatorics, for the geometry kernel
  const CombBuf& cb = a.comb;
  const size_t tb = (size_t)s * kTMax, pb = (size_t)s * kPMax;
#pragma unroll
  for (int wi = 0; wi < NWT; ++wi) {
    uint64_t m = valid.w[wi];
    while (m) {
      const int t = wi * 64 + __ffsll((long long)m) - 1;
      m &= m - 1;
      cb.tv[tb + t] = sm.tv[t][tid];
      cb.ta[tb + t] = sm.ta[t][tid];
      cb.key[tb + t] = sm.key[t][tid];
    }
  }
  for (uint64_t m = pused; m; m &= m - 1) {
    const int p = __ffsll((long long)m) - 1;
    const uint16_t rk = sm.prank[p][tid];
    uint32_t own;
    if constexpr (kFP64) {
      own = sm.pown[p][tid];
    } else {
      // box faces only ever occupy their initial slots 0-5
      own = (rk == 0xFFFF) ? kBoxBase + (uint32_t)p : a.nbr[(size_t)rk * a.nbr_stride + row];
    }
    cb.pown[pb + p] = own;
    cb.prank[pb + p] = rk;
  }
  cb.tmask[s] = make_ulonglong2(valid.w[0], NWT > 1 ? valid.w[NWT - 1] : 0ull);
  cb.pmask[s] = pused;
  cb.flags[s] = parity < 0 ? 1u : 0u;
}

template <typename Real, int T, int P, bool XF>
static void launch_clip(const ClipArgs& a, cudaStream_t st) {
  if (a.nq == 0) return;
  const size_t sh = sizeof(CellSmem<Real, kClipThreads, T, P>);
  cudaFuncSetAttribute(clip_kernel<Real, T, P, XF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sh);
  const unsigned nb = (a.nq + kClipThreads - 1) / kClipThreads;
  clip_kernel<Real, T, P, XF><<<nb, kClipThreads, sh, st>>>(a); count_launch();
  last_launch_error = cudaGetLastError();
}

void launch_clip_fp64(const ClipArgs& a, int shape, cudaStream_t st) {
  if (shape == CLIP_SMALL) launch_clip<double, kSmallT, kSmallP, false>(a, st);
  else launch_clip<double, kLargeT, kLargeP, false>(a, st);
}

void launch_clip_fp32(const ClipArgs& a, int shape, bool exact_fallback, cudaStream_t st) {
  if (shape == CLIP_SMALL) {
    if (exact_fallback) launch_clip<float, kSmallT, kSmallP, true>(a, st);
    else launch_clip<float, kSmallT, kSmallP, false>(a, st);
  } else {
    launch_clip<float, kLargeT, kLargeP, true>(a, st);
  }
}

}  // namespace gbv
