// Laguerre cell clipping: one warp per cell, the polytope in a shared
// memory record of the warp, its triangles spread over the lanes.
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
//   - the lanes test the triangles against a plane together (one or more
//     triangles each, a ballot gives the conflict zone), find the border
//     of the zone together, and create the new triangles together once one
//     lane has walked the border; the planes of the next 32 list positions
//     are computed one per lane ahead of the loop;
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
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <type_traits>

#include "gbv_clip.cuh"
#include "gbv_exact.cuh"
#include "gbv_refgeom.cuh"
#include "gbv_corner.cuh"

namespace gbv {

cudaError_t last_launch_error = cudaSuccess;
constexpr int kClipWarps = 8;  // cells in flight per block, one per warp
// resident blocks per SM the registers must allow: 3 (80 registers) for the
// lean FP32 loop that runs every cell, 2 where the exact-sign fallback's
// registers would spill
template <typename Real, bool XF>
constexpr int clip_min_blocks() {
  return (std::is_same<Real, float>::value && !XF) ? 3 : 2;
}

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

// k-th (0-based) set bit of m; the bit must exist
__device__ __forceinline__ int select32(uint32_t m, int k) {
  int base = 0;
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1) {
    const uint32_t low = m & ((1u << w) - 1u);
    const int c = __popc(low);
    if (k >= c) {
      k -= c;
      m >>= w;
      base += w;
    } else {
      m = low;
    }
  }
  return base;
}

template <int NW>
__device__ __forceinline__ int select_bit(const Bits<NW>& b, int k) {
#pragma unroll
  for (int i = 0; i < NW; ++i) {
    const uint32_t lo = (uint32_t)b.w[i], hi = (uint32_t)(b.w[i] >> 32);
    const int cl = __popc(lo), ch = __popc(hi);
    if (k < cl) return 64 * i + select32(lo, k);
    k -= cl;
    if (k < ch) return 64 * i + 32 + select32(hi, k);
    k -= ch;
  }
  return -1;
}

// The n lowest set bits of b.
template <int NW>
__device__ __forceinline__ Bits<NW> lowest_bits(const Bits<NW>& b, int n) {
  Bits<NW> r;
#pragma unroll
  for (int i = 0; i < NW; ++i) {
    const int c = __popcll(b.w[i]);
    if (n >= c) {
      r.w[i] = b.w[i];
      n -= c;
    } else if (n > 0) {
      const uint32_t lo = (uint32_t)b.w[i];
      const int cl = __popc(lo);
      const int pos = n <= cl ? select32(lo, n - 1) : 32 + select32((uint32_t)(b.w[i] >> 32), n - 1 - cl);
      r.w[i] = b.w[i] & (pos >= 63 ? ~0ull : ((2ull << pos) - 1ull));
      n = 0;
    } else {
      r.w[i] = 0;
    }
  }
  return r;
}

template <int NW>
__device__ __forceinline__ void or_into(Bits<NW>& a, const Bits<NW>& b) {
#pragma unroll
  for (int i = 0; i < NW; ++i) a.w[i] |= b.w[i];
}

template <typename R>
__device__ __forceinline__ R warp_max(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}
__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}
__device__ __forceinline__ double warp_maxf(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}
__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// ---------------------------------------------------------------------
// Cell record in shared memory, one per warp
// ---------------------------------------------------------------------
template <typename Real, int T, int P>
struct CellRec;

template <int T, int P>
struct __align__(16) CellRec<double, T, P> {
  double2 cxy[T];     // corner x, y (reference frame and arithmetic)
  double2 czr[T];     // corner z, squared distance to the seed
  float eps[T];       // corner error bound (cramer_bound)
  uint32_t tv[T];     // planes i | j << 8 | k << 16
  uint32_t ta[T];     // triangles across the edges opposite i, j, k (bytes 0-2)
  uint32_t pown[P];   // plane owner: seed slot or kBoxBase + face
  int16_t key[T];
  uint16_t prank[P];  // list position of the plane's seed
  uint16_t pnb[P];    // border scratch: kept triangle | edge << 8
  uint8_t pnext[P];   // border scratch: next border plane
  uint8_t order[T];   // border planes in walk order
};

template <int T, int P>
struct __align__(16) CellRec<float, T, P> {
  float4 c4[T];       // corner x, y, z (frame centred on the seed), eps
  float4 pl[P];       // local-frame plane equations
  uint32_t tv[T];
  uint32_t ta[T];
  int16_t key[T];
  uint16_t prank[P];
  uint16_t pnb[P];
  uint8_t pnext[P];
  uint8_t order[T];
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
// loop for the first pass over every cell).  The warps stride over the
// queries; every lane holds the cell's bookkeeping (valid triangles, used
// planes, parity, R2), so control flow stays uniform across the warp.
template <typename Real, int T, int P, bool XF>
__global__ void __launch_bounds__(kClipWarps * 32, clip_min_blocks<Real, XF>()) clip_kernel(ClipArgs a) {
  constexpr int NWT = (T + 63) / 64;
  constexpr int NS = T / 32;  // triangle slots per lane: slot t on lane t % 32
  constexpr bool kFP64 = std::is_same<Real, double>::value;
  using Rec = CellRec<Real, T, P>;
  using Plane = typename std::conditional<kFP64, double4, float4>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  Rec& g = reinterpret_cast<Rec*>(smem_raw)[threadIdx.x >> 5];
  const SortedSeeds& S = a.S;
  const uint32_t nwarps = gridDim.x * kClipWarps;
  unsigned long long n_exact = 0, n_tests = 0, n_created = 0;
  uint32_t max_jj = 0;

  for (uint32_t qi = blockIdx.x * kClipWarps + (threadIdx.x >> 5); qi < a.nq; qi += nwarps) {
    if (a.abort_on_empty && *(volatile unsigned int*)a.abort_on_empty) break;
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
    const float pn = sc.fh.x * sc.fh.x + sc.fh.y * sc.fh.y + sc.fh.z * sc.fh.z;

    // Plane p's equation (FP64: recomputed from its owner, FP32: stored).
    auto plane_of = [&](uint32_t p) {
      if constexpr (kFP64) return plane_fp64(g.pown[p], sc.pi, sc.qi, sc.box, S);
      else return g.pl[p];
    };
    // The reference's FP64 plane of plane slot p (FP32 kernel: from its
    // list position, box faces keep their slots 0-5) and of seed slot j.
    auto plane64_of = [&](uint32_t j) -> double4 {
      return plane_fp64(j, sc.pi, S.q[s], sc.box, S);
    };
    auto plane64 = [&](uint32_t p) -> double4 {
      if constexpr (kFP64) {
        return plane_fp64(g.pown[p], sc.pi, sc.qi, sc.box, S);
      } else {
        const uint16_t rk = g.prank[p];
        const uint32_t own =
            (rk == 0xFFFF) ? kBoxBase + p : a.nbr[(size_t)rk * a.nbr_stride + row];
        return plane_fp64(own, sc.pi, S.q[s], sc.box, S);
      }
    };
    // FP32 bisector of the seed and seed slot j in the seed's frame,
    // (-2 d, |d|^2 + w_i - w_j) with d = p_j - p_i taken from the
    // value/remainder pairs (FP32 relative accuracy however close the two
    // seeds are); d2h = |d|^2 + (h_j - h_i)^2, wj = w_j.
    auto seed_plane32 = [&](uint32_t j, float& d2h, float& wj) -> float4 {
      const float4 jh = S.xf[j], jl = S.xl[j];
      const float dx = (jh.x - sc.fh.x) + (jl.x - sc.fl.x);
      const float dy = (jh.y - sc.fh.y) + (jl.y - sc.fl.y);
      const float dz = (jh.z - sc.fh.z) + (jl.z - sc.fl.z);
      const float dh = (jh.w - sc.fh.w) + (jl.w - sc.fl.w);
      const float d2 = dx * dx + dy * dy + dz * dz;
      d2h = d2 + dh * dh;
      float dw = 0.f;
      wj = 0.f;
      if (S.wf) {
        const float2 w2 = S.wf[j];
        dw = (w2.x - sc.fw.x) + (w2.y - sc.fw.y);
        wj = w2.x;
      }
      return make_float4(-2.f * dx, -2.f * dy, -2.f * dz, d2 - dw);
    };
    // Creates the corner of triangle t from its planes; returns its r2.
    auto make_corner = [&](uint32_t t, const auto& pa, const auto& pb, const auto& pc) -> Real {
      if constexpr (kFP64) {
        double x, y, z;
        float e;
        corner_fp64(pa, pb, pc, x, y, z, e);
        const double r2 = r_sqdist(sc.pi.x, sc.pi.y, sc.pi.z, make_double3(x, y, z));
        g.cxy[t] = make_double2(x, y);
        g.czr[t] = make_double2(z, r2);
        g.eps[t] = e;
        return r2;
      } else {
        float x, y, z, e;
        corner_fp32(pa, pb, pc, x, y, z, e);
        g.c4[t] = make_float4(x, y, z, e);
        return x * x + y * y + z * z;
      }
    };

    // ---- init_with_box (convex_cell.cpp:175-215): 6 planes, 8 corners,
    // triangles and adjacency in the reference's order, each pushed at the
    // head of the list
    if (lane < 6) {
      g.prank[lane] = 0xFFFF;
      if constexpr (kFP64) g.pown[lane] = kBoxBase + lane;
      else g.pl[lane] = box_plane_fp32(lane, sc);
    }
    if (lane < 8) {
      const uint32_t bt[8] = {2 | 5 << 8 | 0 << 16, 5 | 3 << 8 | 0 << 16, 1 | 5 << 8 | 2 << 16,
                              5 | 1 << 8 | 3 << 16, 4 | 2 << 8 | 0 << 16, 4 | 0 << 8 | 3 << 16,
                              2 | 4 << 8 | 1 << 16, 4 | 3 << 8 | 1 << 16};
      const uint32_t ba[8] = {1 | 4 << 8 | 2 << 16, 5 | 0 << 8 | 3 << 16, 0 | 6 << 8 | 3 << 16,
                              7 | 1 << 8 | 2 << 16, 0 | 5 << 8 | 6 << 16, 1 | 7 << 8 | 4 << 16,
                              7 | 2 << 8 | 4 << 16, 3 | 6 << 8 | 5 << 16};
      g.tv[lane] = bt[lane];
      g.ta[lane] = ba[lane];
      g.key[lane] = (int16_t)(-lane);
    }
    __syncwarp();
    Real R2 = 0;
    if (lane < 8) {
      const uint32_t v = g.tv[lane];
      R2 = make_corner(lane, plane_of(v & 0xFF), plane_of(v >> 8 & 0xFF), plane_of(v >> 16 & 0xFF));
    }
    R2 = warp_maxf(R2);
    Bits<NWT> valid;
    valid.clear();
    valid.w[0] = 0xFFull;
    // this lane's slots (t = lane + 32 q) among the valid triangles, bit q
    auto lane_bits = [&](const Bits<NWT>& b) {
      uint32_t m = 0;
#pragma unroll
      for (int q = 0; q < NS; ++q)
        m |= (uint32_t)((b.w[q >> 1] >> (lane + 32 * (q & 1))) & 1ull) << q;
      return m;
    };
    uint32_t vm = lane_bits(valid);
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

    if (dup) {
      st = CELL_DUPLICATE;
    } else {
      // the plane of list position jj0 + lane, its security-radius
      // distance and its conflict bound terms
      uint32_t bj = 0;
      Plane bP{};
      Real bd = 0, bpa = 0, bbw = 0;
      // the conflict bound's terms carry the fast predicates' widening
      // (a power of two: the scaled bound rounds as the unscaled one)
      const Real wide = a.fast_pred ? (Real)kFastPredWide : (Real)1;
      if (a.resume) {
        // ---- continue from the stored polytope of the list's first `done`
        // positions (the lists only grow at their end, so clipping on from
        // there gives the polytope a clipping from the box would give: the
        // same planes in the same order, each conflict sign exact)
        const CombBuf& cb = a.comb;
        const uint32_t fl = cb.flags[s];
        const uint32_t done = fl >> 8;
        const ulonglong2 tm = cb.tmask[s];
        const uint64_t pm = cb.pmask[s];
        if ((fl & 2u) && done > 0 && done <= cnt && (NWT > 1 || tm.y == 0) &&
            (P >= 64 || (pm >> (P & 63)) == 0)) {
          jj = done;
          parity = (fl & 1u) ? -1 : 1;
          pused = pm;
          valid.clear();
          valid.w[0] = tm.x;
          if (NWT > 1) valid.w[NWT - 1] = tm.y;
          const size_t tb = (size_t)s * kTMax, pb = (size_t)s * kPMax;
          for (int p = lane; p < P; p += 32) {
            if (!((pm >> p) & 1ull)) continue;
            const uint16_t rk = cb.prank[pb + p];
            g.prank[p] = rk;
            if constexpr (kFP64) {
              g.pown[p] = cb.pown[pb + p];
            } else {
              float d2h, wj;
              g.pl[p] = (rk == 0xFFFF) ? box_plane_fp32(p, sc)
                                       : seed_plane32(a.nbr[(size_t)rk * a.nbr_stride + row],
                                                      d2h, wj);
            }
          }
#pragma unroll
          for (int q = 0; q < NS; ++q) {
            const int t = lane + 32 * q;
            if (!valid.test(t)) continue;
            g.tv[t] = cb.tv[tb + t];
            g.ta[t] = cb.ta[tb + t];
            g.key[t] = cb.key[tb + t];
          }
          __syncwarp();
          Real r2 = 0;
#pragma unroll
          for (int q = 0; q < NS; ++q) {
            const int t = lane + 32 * q;
            if (!valid.test(t)) continue;
            const uint32_t v = g.tv[t];
            r2 = fmax(r2, make_corner(t, plane_of(v & 0xFF), plane_of(v >> 8 & 0xFF),
                                      plane_of(v >> 16 & 0xFF)));
          }
          R2 = warp_maxf(r2);
          vm = lane_bits(valid);
          __syncwarp();
        }
      }
      // the first iteration loads a batch (unsigned: jj - jj0 == 32)
      uint32_t jj0 = jj - 32u;
      for (; jj < cnt; ++jj) {
        if (jj - jj0 == 32) {
          jj0 = jj;
          const uint32_t pos = jj0 + lane;
          if (pos < cnt) {
            const uint32_t j = a.nbr[(size_t)pos * a.nbr_stride + row];
            bj = j;
            if constexpr (kFP64) {
              const double4 pj = S.xd[j];
              bd = a.check_sr ? dist2_exact(sc.pi, pj) : 0.0;
              bP = make_double4(2.0 * __dsub_rn(sc.pi.x, pj.x), 2.0 * __dsub_rn(sc.pi.y, pj.y),
                                2.0 * __dsub_rn(sc.pi.z, pj.z), __dsub_rn(sc.qi, S.q[j]));
              bpa = (fabs(bP.x) + fabs(bP.y) + fabs(bP.z)) * 1.0001 * wide;
              bbw = Consts<double>::kDot * fabs(bP.w) * 1.0001 * wide;
            } else {
              float wj;
              bP = seed_plane32(j, bd, wj);
              bpa = (fabsf(bP.x) + fabsf(bP.y) + fabsf(bP.z)) * 1.0001f * wide;
              // the reference's own FP64 planes carry a rounding of about
              // 2^-52 (|w_i| + |w_j| + |p_i|^2 + |p_j|^2) in their offset
              const float qmag = fabsf(sc.fw.x) + fabsf(wj) + 2.f * pn + 1.f;
              bbw = (Consts<float>::kDot * fabsf(bP.w) + 3.5527137e-15f * qmag) * 1.0001f * wide;
            }
          }
        }
        const int src = (int)(jj - jj0);
        const uint32_t j = __shfl_sync(FULL, bj, src);
        // ---- security radius (generic_RVD.h:2300-2324)
        if (a.check_sr) {
          const Real dj = __shfl_sync(FULL, bd, src);
          bool stop;
          if constexpr (kFP64) stop = dj > __dmul_rn(4.1, __dadd_rn(R2, hi2));
          else stop = dj > 4.1f * (R2 + hi2f);
          if (stop) {
            st = CELL_CERTIFIED;
            break;
          }
        }
        // every clip relinks the reference's valid list in reverse order
        const int par_old = parity;
        parity = -parity;
        if (!valid.any()) continue;  // empty cell: nothing left to clip
        Plane Pn;
        Pn.x = __shfl_sync(FULL, bP.x, src);
        Pn.y = __shfl_sync(FULL, bP.y, src);
        Pn.z = __shfl_sync(FULL, bP.z, src);
        Pn.w = __shfl_sync(FULL, bP.w, src);
        const Real pa1 = __shfl_sync(FULL, bpa, src), bw = __shfl_sync(FULL, bbw, src);

        // ---- conflict scan (triangle_is_in_conflict, convex_cell.cpp:870-912)
        bool cf[NS];
        bool uncertain = false;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
          const int t = lane + 32 * q;
          cf[q] = false;
          if (!((vm >> q) & 1u)) continue;
          Real cx, cy, cz, eps;
          if constexpr (kFP64) {
            const double2 xy = g.cxy[t];
            cx = xy.x;
            cy = xy.y;
            cz = g.czr[t].x;
            eps = (double)g.eps[t];
          } else {
            const float4 c = g.c4[t];
            cx = c.x;
            cy = c.y;
            cz = c.z;
            eps = c.w;
          }
          Real sv;
          if constexpr (kFP64) sv = fma(Pn.z, cz, fma(Pn.y, cy, fma(Pn.x, cx, Pn.w)));
          else sv = fmaf(Pn.z, cz, fmaf(Pn.y, cy, fmaf(Pn.x, cx, Pn.w)));
          const Real bound = fma(pa1, eps, bw);
          bool in_conflict;
          if (sv < -bound) {
            in_conflict = true;
          } else if (sv > bound) {
            in_conflict = false;
          } else {
            if constexpr (kFP64) {
              const uint32_t v = g.tv[t];
              in_conflict = exact_conflict(plane_of(v & 0xFF), plane_of(v >> 8 & 0xFF),
                                           plane_of(v >> 16 & 0xFF), Pn, a.fast_pred);
              ++n_exact;
            } else if constexpr (XF) {
              // FP32 cannot decide: the exact sign of the reference's FP64
              // planes decides, as in the FP64 kernel
              const uint32_t v = g.tv[t];
              in_conflict = exact_conflict(plane64(v & 0xFF), plane64(v >> 8 & 0xFF),
                                           plane64(v >> 16 & 0xFF), plane64_of(j), a.fast_pred);
              ++n_exact;
            } else {
              uncertain = true;
              in_conflict = false;
            }
          }
          cf[q] = in_conflict;
        }
        if (lane == 0) n_tests += (unsigned)valid.popc();
        if (!kFP64 && !XF && __any_sync(FULL, uncertain)) {
          st = CELL_RECHECK;
          break;
        }
        Bits<NWT> conflict;
        conflict.clear();
#pragma unroll
        for (int q = 0; q < NS; ++q)
          conflict.w[q >> 1] |= (uint64_t)__ballot_sync(FULL, cf[q]) << (32 * (q & 1));
        if (!conflict.any()) continue;
        if (conflict.equals(valid)) {  // the whole cell is clipped away
          valid.clear();
          vm = 0;
          R2 = 0;
          if (a.abort_on_empty) {
            if (lane == 0) atomicExch(a.abort_on_empty, 1u);
            st = CELL_RECHECK;  // not a result: the caller stops
            break;
          }
          continue;
        }
        // the kept triangles: largest corner radius and list key
        Real kr2 = 0;
        int kme = -0x7FFF;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
          const int t = lane + 32 * q;
          if (!((vm >> q) & 1u) || cf[q]) continue;
          Real r2;
          if constexpr (kFP64) {
            r2 = g.czr[t].y;
          } else {
            const float4 c = g.c4[t];
            r2 = c.x * c.x + c.y * c.y + c.z * c.z;
          }
          kr2 = fmax(kr2, r2);
          kme = max(kme, par_old * (int)g.key[t]);
        }
        const Real keepR2 = warp_maxf(kr2);
        const int keep_max_eff = __reduce_max_sync(FULL, kme);
        // ---- a slot for the new plane (recycle planes no triangle uses)
        const uint64_t pmask = (P >= 64) ? ~0ull : ((1ull << P) - 1ull);
        uint64_t freep = ~pused & pmask;
        if (!freep) {
          uint64_t used = 0;
#pragma unroll
          for (int q = 0; q < NS; ++q) {
            const int t = lane + 32 * q;
            if (!((vm >> q) & 1u) || cf[q]) continue;
            const uint32_t v = g.tv[t];
            used |= (1ull << (v & 0xFF)) | (1ull << (v >> 8 & 0xFF)) | (1ull << (v >> 16 & 0xFF));
          }
          pused = (uint64_t)__reduce_or_sync(FULL, (uint32_t)used) |
                  ((uint64_t)__reduce_or_sync(FULL, (uint32_t)(used >> 32)) << 32);
          freep = ~pused & pmask;
          if (!freep) {
            st = CELL_OVERFLOW;
            break;
          }
        }
        // list positions are stored in 16 bits (0xFFFF marks a box face):
        // a plane further down the list sends the cell to the huge-cell
        // kernel, which keeps them in 32 bits
        if (jj >= 0xFFFFu) {
          st = CELL_OVERFLOW;
          break;
        }
        const uint32_t lv = (uint32_t)(__ffsll((long long)freep) - 1);
        pused |= 1ull << lv;
        if (lane == 0) {
          g.prank[lv] = (uint16_t)jj;
          if constexpr (kFP64) g.pown[lv] = j;
          else g.pl[lv] = Pn;
        }
        // ---- border of the conflict zone (triangulate_conflict_zone)
        int nb_lane = 0;
        long long best = LLONG_MIN;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
          if (!cf[q]) continue;
          const int t = lane + 32 * q;
          const uint32_t v = g.tv[t], ad = g.ta[t];
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            const uint32_t nb = (ad >> (8 * e)) & 0xFF;
            if (conflict.test((int)nb)) continue;
            // edge opposite vertex e runs v[e+1] -> v[e+2] in t; the kept
            // triangle nb holds it reversed, so the border walk, which
            // follows nb's orientation, goes from y = v[e+2] to x = v[e+1]
            const uint32_t x = (v >> (8 * ((e + 1) % 3))) & 0xFF;
            const uint32_t y = (v >> (8 * ((e + 2) % 3))) & 0xFF;
            const uint32_t an = g.ta[nb];
            const uint32_t eb =
                ((an >> 8 & 0xFF) == (uint32_t)t) + 2 * ((an >> 16 & 0xFF) == (uint32_t)t);
            g.pnext[y] = (uint8_t)x;
            g.pnb[y] = (uint16_t)(nb | (eb << 8));
            // the reference starts its walk at the border edge it meets
            // last while scanning the relinked list (new eff = -old eff);
            // ties (none occur: keys are distinct) would go to the lowest
            // (triangle, edge)
            const int score = -par_old * (int)g.key[nb] * 4 + (int)eb;
            const long long cand = ((long long)score << 24) |
                                   ((long long)(0xFFFF - (t * 3 + e)) << 8) | (long long)y;
            best = max(best, cand);
            ++nb_lane;
          }
        }
        const int nborder = __reduce_add_sync(FULL, nb_lane);
        const uint32_t first_v = (uint32_t)(warp_max(best) & 0xFF);
        const int nkeep = valid.popc() - conflict.popc();
        if (nkeep + nborder > T) {
          st = CELL_OVERFLOW;
          break;
        }
        const Bits<NWT> freet = andnot(full_bits<NWT>(T), andnot(valid, conflict));
        valid = andnot(valid, conflict);
        R2 = keepR2;
        const int key_base = -keep_max_eff - 1;
        if (key_base - nborder < -0x7FFF) {  // keys are stored in 16 bits
          st = CELL_OVERFLOW;
          break;
        }
        __syncwarp();
        // ---- the border in walk order: one lane follows it
        int ok = 1;
        if (lane == 0) {
          uint32_t v = first_v;
          for (int i = 0; i < nborder; ++i) {
            g.order[i] = (uint8_t)v;
            v = g.pnext[v];
            if (v == first_v && i + 1 < nborder) {  // closes early: not a simple cycle
              ok = 0;
              break;
            }
          }
          if (v != first_v) ok = 0;
        }
        ok = __shfl_sync(FULL, ok, 0);
        if (!ok) {
          st = CELL_ERROR;
          break;
        }
        __syncwarp();
        // ---- fan new triangles (lv, next, v) around the border: the i-th
        // takes the i-th free slot, its neighbours the slots of i - 1 and
        // i + 1 along the border
        Real r2n = 0;
        for (int i0 = 0; i0 < nborder; i0 += 32) {
          const int i = i0 + lane;
          // slots of border positions i and, through the lanes beside it
          // (or directly at the ends of a 32-position round), i - 1 and i + 1
          const int nt = i < nborder ? select_bit(freet, i) : -1;
          int ntp = __shfl_up_sync(FULL, nt, 1), ntn = __shfl_down_sync(FULL, nt, 1);
          if (i >= nborder) continue;
          if (lane == 0 || i == 0) ntp = select_bit(freet, i > 0 ? i - 1 : nborder - 1);
          if (lane == 31 || i + 1 == nborder) ntn = select_bit(freet, i + 1 < nborder ? i + 1 : 0);
          const uint32_t v = g.order[i];
          const uint32_t x = g.order[i + 1 < nborder ? i + 1 : 0];
          const uint32_t nbinfo = g.pnb[v];
          const uint32_t tn = nbinfo & 0xFF, eb = nbinfo >> 8;
          g.tv[nt] = lv | (x << 8) | (v << 16);
          g.ta[nt] = tn | ((uint32_t)ntp << 8) | ((uint32_t)ntn << 16);
          g.key[nt] = (int16_t)(parity * (key_base - i));
          reinterpret_cast<uint8_t*>(&g.ta[tn])[eb] = (uint8_t)nt;
          r2n = fmax(r2n, make_corner(nt, Pn, plane_of(x), plane_of(v)));
        }
        R2 = fmax(R2, warp_maxf(r2n));
        or_into(valid, lowest_bits(freet, nborder));
        vm = lane_bits(valid);
        if (lane == 0) n_created += (unsigned)nborder;
        __syncwarp();
      }
      if (st < 0) {
        // list exhausted without certification
        const bool complete = ((cnt_raw & kCntMask) < a.list_k) || (a.list_k >= a.n_total - 1);
        if (!a.check_sr) st = CELL_CERTIFIED;
        else if (copies && cnt == cap) st = (cap == 0) ? CELL_DUPLICATE : CELL_STALLED;
        else st = complete ? CELL_ALL_NEIGHBOURS : CELL_NEED_MORE_K;
      }
    }
    max_jj = max(max_jj, jj);
    if (lane == 0) {
      a.status[s] = st;
      a.nclip[s] = jj;
    }
    if (!(st == CELL_RECHECK || st == CELL_OVERFLOW || st == CELL_NEED_MORE_K ||
          st == CELL_ERROR)) {
      // ---- the combinatorics, for the geometry kernel
      const CombBuf& cb = a.comb;
      const size_t tb = (size_t)s * kTMax, pb = (size_t)s * kPMax;
#pragma unroll
      for (int q = 0; q < NS; ++q) {
        const int t = lane + 32 * q;
        if (!valid.test(t)) continue;
        cb.tv[tb + t] = g.tv[t];
        cb.ta[tb + t] = g.ta[t];
        cb.key[tb + t] = g.key[t];
      }
      for (int p = lane; p < P; p += 32) {
        if (!((pused >> p) & 1ull)) continue;
        const uint16_t rk = g.prank[p];
        uint32_t own;
        if constexpr (kFP64) {
          own = g.pown[p];
        } else {
          // box faces only ever occupy their initial slots 0-5
          own = (rk == 0xFFFF) ? kBoxBase + (uint32_t)p : a.nbr[(size_t)rk * a.nbr_stride + row];
        }
        cb.pown[pb + p] = own;
        cb.prank[pb + p] = rk;
      }
      if (lane == 0) {
        cb.tmask[s] = make_ulonglong2(valid.w[0], NWT > 1 ? valid.w[NWT - 1] : 0ull);
        cb.pmask[s] = pused;
        // parity, and the list positions this polytope has clipped
        cb.flags[s] = (parity < 0 ? 1u : 0u) | (jj <= 0xFFFFFFu ? 2u | jj << 8 : 0u);
      }
    }
    __syncwarp();  // the record is reused by the warp's next cell
  }
  if (a.counters) {
    const unsigned long long ne = warp_sum(n_exact), nt = warp_sum(n_tests),
                             nc = warp_sum(n_created);
    if (lane == 0) {
      if (ne) atomicAdd(&a.counters[0], ne);
      atomicMax(&a.counters[1], (unsigned long long)max_jj);
      atomicAdd(&a.counters[2], nt);
      atomicAdd(&a.counters[3], nc);
    }
  }
}

template <typename Real, int T, int P, bool XF>
static void launch_clip(const ClipArgs& a, cudaStream_t st) {
  if (a.nq == 0) return;
  const size_t sh = sizeof(CellRec<Real, T, P>) * kClipWarps;
  cudaFuncSetAttribute(clip_kernel<Real, T, P, XF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sh);
  static int resident = 0;  // blocks the device holds at once
  if (resident == 0) {
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, clip_kernel<Real, T, P, XF>,
                                                  kClipWarps * 32, sh);
    resident = std::max(1, per_sm) * std::max(1, sms);
  }
  const unsigned need = (a.nq + kClipWarps - 1) / kClipWarps;
  const unsigned nb = std::min<unsigned>(need, (unsigned)resident);
  clip_kernel<Real, T, P, XF><<<nb, kClipWarps * 32, sh, st>>>(a); count_launch();
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
