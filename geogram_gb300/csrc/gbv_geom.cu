// Geometry of the clipped cells: one warp per cell, FP64.
//
// From the combinatorics written by the clipping kernels, this computes
// what the reference's VBW::ConvexCell reports, with its formulas and its
// summation order, so the results are bit-identical to the reference's:
//   compute_geometry (convex_cell.cpp:1125-1145): every corner by Cramer's
//     rule from the three planes, and v2t[v] = the last triangle of the
//     valid list that holds v (here: the largest effective list key);
//   compute_mg (convex_cell.cpp:1267-1307): planes in creation order, the
//     first contributing one gives the fan origin t_origin, every other
//     facet is fanned from v2t[v] around the plane;
//   facet_area (convex_cell.cpp:1160-1191) for the seed facets.
// The lanes compute corners and tetrahedron terms in parallel; one lane
// adds the terms in the reference's order.  For cells clipped in FP32 the
// kernel also checks, in FP64, that the reference's security-radius loop
// would have stopped at the same neighbour, and sends the cell back to
// FP64 clipping otherwise.
#include <cfloat>

#include "gbv_clip.cuh"
#include "gbv_refgeom.cuh"

namespace gbv {

constexpr int kGeomWarps = 4;
constexpr int kMaxTerms = 2 * kTMax;  // tetrahedra of one cell, at most 2 nt - 4

struct GeomWarpSmem {
  double px[kTMax], py[kTMax], pz[kTMax];  // corners
  double4 plane[kPMax];
  int v2t[kPMax];                           // (eff + 32768) << 8 | triangle, -1: none
  uint16_t prank[kPMax];                    // list position (0xFFFF: box face)
  int16_t ntets[kPMax];                     // per rank
  int16_t toff[kPMax + 1];                  // term offsets per rank
  uint8_t order[kPMax];                     // contributing planes in creation order
  double tm[kMaxTerms], tx[kMaxTerms], ty[kMaxTerms], tz[kMaxTerms];
};

__device__ __forceinline__ double plane_from_owner_w(double qi, double qj) { return __dsub_rn(qi, qj); }

__global__ void __launch_bounds__(kGeomWarps * 32) geom_kernel(GeomArgs a) {
  extern __shared__ __align__(16) unsigned char geom_smem[];
  GeomWarpSmem* smw = reinterpret_cast<GeomWarpSmem*>(geom_smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t ci = blockIdx.x * kGeomWarps + warp;
  if (ci >= a.nq) return;
  GeomWarpSmem& g = smw[warp];
  const SortedSeeds& S = a.S;
  const uint32_t s = a.qlist ? a.qlist[ci] : ci;
  const int32_t st = a.status[s];
  if (st >= CELL_NEED_MORE_K) return;  // not final: handled by another pass
  const CombBuf& cb = a.comb;
  const size_t tb = (size_t)s * kTMax, pb = (size_t)s * kPMax;
  const ulonglong2 tm2 = cb.tmask[s];
  const uint64_t pm = cb.pmask[s];
  const int parity = (cb.flags[s] & 1u) ? -1 : 1;
  const double4 pi = S.xd[s];
  const double qi = S.q[s];

  // ---- planes (FP64, the reference's global frame) and v2t init
  for (int p = lane; p < kPMax; p += 32) {
    g.v2t[p] = -1;
    g.prank[p] = 0xFFFF;
    if ((pm >> p) & 1ull) {
      g.prank[p] = cb.prank[pb + p];
      const uint32_t own = cb.pown[pb + p];
      double4 P;
      if (own >= kBoxBase) {
        switch (own - kBoxBase) {
          case 0: P = make_double4(1.0, 0.0, 0.0, -a.box[0]); break;
          case 1: P = make_double4(-1.0, 0.0, 0.0, a.box[3]); break;
          case 2: P = make_double4(0.0, 1.0, 0.0, -a.box[1]); break;
          case 3: P = make_double4(0.0, -1.0, 0.0, a.box[4]); break;
          case 4: P = make_double4(0.0, 0.0, 1.0, -a.box[2]); break;
          default: P = make_double4(0.0, 0.0, -1.0, a.box[5]); break;
        }
      } else {
        const double4 pj = S.xd[own];
        P = make_double4(2.0 * __dsub_rn(pi.x, pj.x), 2.0 * __dsub_rn(pi.y, pj.y),
                         2.0 * __dsub_rn(pi.z, pj.z), plane_from_owner_w(qi, S.q[own]));
      }
      g.plane[p] = P;
    }
  }
  __syncwarp();
  // ---- corners (compute_geometry) and v2t
  double R2 = 0.0;
  for (int t = lane; t < kTMax; t += 32) {
    const uint64_t w = (t < 64) ? tm2.x : tm2.y;
    if (!((w >> (t & 63)) & 1ull)) continue;
    const uint32_t v = cb.tv[tb + t];
    const int a0 = v & 0xFF, a1 = v >> 8 & 0xFF, a2 = v >> 16 & 0xFF;
    const double3 c = r_corner(g.plane[a0], g.plane[a1], g.plane[a2]);
    g.px[t] = c.x;
    g.py[t] = c.y;
    g.pz[t] = c.z;
    R2 = fmax(R2, r_sqdist(pi.x, pi.y, pi.z, c));
    const int eff = parity * (int)cb.key[tb + t];
    const int packed = ((eff + 32768) << 8) | t;
    atomicMax(&g.v2t[a0], packed);
    atomicMax(&g.v2t[a1], packed);
    atomicMax(&g.v2t[a2], packed);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) R2 = fmax(R2, __shfl_xor_sync(0xFFFFFFFFu, R2, o));
  __syncwarp();

  // ---- FP32 clipping: the reference stops at the same neighbour only if
  // d(stop) > 4.1 (R2 + h^2) and d(last clipped) <= 4.1 (R2 + h^2) with the
  // final cell's R2 (R2 only shrinks while clipping)
  if (a.verify_sr &&
      (st == CELL_CERTIFIED || st == CELL_ALL_NEIGHBOURS || st == CELL_STALLED)) {
    const uint32_t row = a.qrow ? a.qrow[ci] : ci;
    const uint32_t jj = a.nclip[s];
    const double thr = __dmul_rn(4.1, __dadd_rn(R2, __dmul_rn(pi.w, pi.w)));
    bool ok = true;
    if (st == CELL_CERTIFIED) {
      const uint32_t js = a.nbr[(size_t)jj * a.nbr_stride + row];
      ok = dist2_exact(pi, S.xd[js]) > thr;
    }
    if (ok && jj > 0) {
      const uint32_t jl = a.nbr[(size_t)(jj - 1) * a.nbr_stride + row];
      ok = !(dist2_exact(pi, S.xd[jl]) > thr);
    }
    if (!ok) {
      if (lane == 0) a.status[s] = CELL_RECHECK;
      return;
    }
  }

  // ---- planes in the reference's creation order: box faces 0-5 (their
  // slots), then the seeds in clipping order (list position)
  int rank_of[2] = {-1, -1};
  int nseed_before[2] = {0, 0};
  bool is_seed[2] = {false, false};
  int ncontrib = 0;
  {
    int cidx[2] = {0x7FFFFFFF, 0x7FFFFFFF};
    for (int h = 0; h < 2; ++h) {
      const int p = lane + 32 * h;
      if (g.v2t[p] >= 0) {
        is_seed[h] = g.prank[p] != 0xFFFF;
        cidx[h] = is_seed[h] ? 6 + g.prank[p] : p;
        rank_of[h] = 0;
      }
    }
    for (int q = 0; q < kPMax; ++q) {
      if (g.v2t[q] < 0) continue;
      ++ncontrib;
      const bool qseed = g.prank[q] != 0xFFFF;
      const int iq = qseed ? 6 + g.prank[q] : q;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (rank_of[h] < 0) continue;
        if (iq < cidx[h]) {
          ++rank_of[h];
          if (qseed) ++nseed_before[h];
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
      if (rank_of[h] >= 0) g.order[rank_of[h]] = (uint8_t)(lane + 32 * h);
  }
  __syncwarp();
  if (ncontrib == 0) {
    if (lane == 0) {
      a.vol[s] = 0.0;
      a.mg[s] = 0.0;
      a.mg[(size_t)a.out_stride + s] = 0.0;
      a.mg[2 * (size_t)a.out_stride + s] = 0.0;
      a.nf[s] = 0;
    }
    return;
  }
  const int t_origin = g.v2t[g.order[0]] & 0xFF;
  auto find_vertex = [&](uint32_t t, uint32_t v) -> int {
    const uint32_t x = cb.tv[tb + t];
    return ((x >> 8 & 0xFF) == v) + 2 * ((x >> 16 & 0xFF) == v);
  };
  auto adjacent = [&](uint32_t t, int e) -> uint32_t {
    return (cb.ta[tb + t] >> (8 * e)) & 0xFF;
  };
  auto corner = [&](int t) { return make_double3(g.px[t], g.py[t], g.pz[t]); };

  // ---- fan sizes per rank (the origin facet, rank 0, adds no term)
  for (int r = lane; r < kPMax; r += 32) {
    int cnt = 0;
    if (r >= 1 && r < ncontrib) {
      const int p = g.order[r];
      const int t0 = g.v2t[p] & 0xFF;
      int t = t0, deg = 0;
      do {
        ++deg;
        t = adjacent(t, (find_vertex(t, p) + 1) % 3);
      } while (t != t0 && deg < 2 * kTMax);
      cnt = deg - 2;
    }
    g.ntets[r] = (int16_t)cnt;
  }
  __syncwarp();
  if (lane == 0) {
    int acc = 0;
    for (int r = 0; r < ncontrib; ++r) {
      g.toff[r] = (int16_t)acc;
      acc += g.ntets[r];
    }
    g.toff[ncontrib] = (int16_t)min(acc, kMaxTerms);
  }
  __syncwarp();
  // ---- tetrahedron terms of compute_mg, written at their sequence position
  const double3 po = corner(t_origin);
  for (int r = lane; r < ncontrib; r += 32) {
    if (r == 0) continue;
    const int p = g.order[r];
    const int t0 = g.v2t[p] & 0xFF;
    int t = t0, cur = 0, k = g.toff[r];
    double3 q1 = po, q2 = po;
    int guard = 0;
    do {
      const double3 pt = corner(t);
      if (cur == 0) {
        q1 = pt;
      } else if (cur == 1) {
        q2 = pt;
      } else if (k < kMaxTerms) {
        const double cm = r_tet_volume(po, q1, q2, pt);
        g.tm[k] = cm;
        g.tx[k] = __ddiv_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(po.x, q1.x), q2.x), pt.x)), 4.0);
        g.ty[k] = __ddiv_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(po.y, q1.y), q2.y), pt.y)), 4.0);
        g.tz[k] = __ddiv_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(po.z, q1.z), q2.z), pt.z)), 4.0);
        ++k;
        q2 = pt;
      }
      ++cur;
      t = adjacent(t, (find_vertex(t, p) + 1) % 3);
    } while (t != t0 && ++guard < 2 * kTMax);
  }
  __syncwarp();
  if (lane == 0) {
    double m = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    const int nterm = g.toff[ncontrib];
    for (int k = 0; k < nterm; ++k) {
      m = __dadd_rn(m, g.tm[k]);
      gx = __dadd_rn(gx, g.tx[k]);
      gy = __dadd_rn(gy, g.ty[k]);
      gz = __dadd_rn(gz, g.tz[k]);
    }
    a.vol[s] = m;
    a.mg[s] = gx;
    a.mg[(size_t)a.out_stride + s] = gy;
    a.mg[2 * (size_t)a.out_stride + s] = gz;
  }
  // ---- facets shared with other seeds (facet_area), clipping order
  int nfac_lane = 0;
  for (int h = 0; h < 2; ++h) {
    const int p = lane + 32 * h;
    if (rank_of[h] < 0 || !is_seed[h]) continue;
    ++nfac_lane;
    const int t0 = g.v2t[p] & 0xFF;
    int t = t0, cur = 0, guard = 0;
    double3 q0 = po, q1 = po;
    double area = 0.0;
    do {
      const double3 pt = corner(t);
      if (cur == 0) {
        q0 = pt;
      } else if (cur == 1) {
        q1 = pt;
      } else {
        area = __dadd_rn(area, r_triangle_area(q0, q1, pt));
        q1 = pt;
      }
      ++cur;
      t = adjacent(t, (find_vertex(t, p) + 1) % 3);
    } while (t != t0 && ++guard < 2 * kTMax);
    const int pos = nseed_before[h];
    a.f_nbr[(size_t)pos * a.out_stride + s] = S.perm[cb.pown[pb + p]];
    a.f_area[(size_t)pos * a.out_stride + s] = area;
  }
  int nfac = nfac_lane;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nfac += __shfl_xor_sync(0xFFFFFFFFu, nfac, o);
  if (lane == 0) a.nf[s] = (uint32_t)nfac;
}

void launch_geometry(const GeomArgs& a, cudaStream_t st) {
  if (a.nq == 0) return;
  const size_t sh = sizeof(GeomWarpSmem) * kGeomWarps;
  cudaFuncSetAttribute(geom_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
  const unsigned nb = (a.nq + kGeomWarps - 1) / kGeomWarps;
  geom_kernel<<<nb, kGeomWarps * 32, sh, st>>>(a); count_launch();
  last_launch_error = cudaGetLastError();
}

}  // namespace gbv
