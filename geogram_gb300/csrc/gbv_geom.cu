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
// The FP64 work is spread over the lanes: one corner, one tetrahedron or
// one facet triangle per lane, from fan sequences walked in shared memory;
// four lanes then add the tetrahedron terms in the reference's order (one
// accumulator each), one lane per facet adds its area terms.  For cells
// clipped in FP32 the kernel also checks, in FP64, that the reference's
// security-radius loop would have stopped at the same neighbour, and sends
// the cell back to FP64 clipping otherwise.
//
// FP32 geometry (G32, the precision mode GBV_PRECISION_FP32_GEOMETRY): the
// same combinatorics and fans, but corners, tetrahedra and facet triangles
// in FP32 in the frame centred on the seed (the planes as the FP32
// clipping kernel forms them), the terms added in FP64; the security-radius
// stop is verified with the corners' error bounds, and a cell it cannot
// verify goes back to the FP64 re-clip.
#include <cfloat>

#include "gbv_clip.cuh"
#include "gbv_corner.cuh"
#include "gbv_refgeom.cuh"

namespace gbv {

constexpr int kGeomWarps = 8;

// T, P: the capacities of the clipping shape whose cells are processed.
template <int T, int P>
struct GeomWarpSmem {
  static constexpr int kTerms = 2 * T;   // fan triangles of one cell, at most 2 nt - 4
  double px[T], py[T], pz[T];            // corners
  double4 plane[P];
  double tm[kTerms], tx[kTerms], ty[kTerms], tz[kTerms];  // volume terms
  double ta[kTerms];                     // area terms
  uint32_t tv[T], tadj[T];               // the cell's triangles
  int v2t[P];                            // (eff + 32768) << 8 | triangle, -1: none
  uint16_t prank[P];                     // list position (0xFFFF: box face)
  int16_t fstart[P + 1];                 // fan sequence offsets per rank
  int16_t vofs[P + 1];                   // volume-term offsets per rank
  int16_t aofs[P + 1];                   // area-term offsets per rank (seed facets)
  uint8_t fan[3 * T];                    // fan sequences (triangles around planes)
  uint8_t order[P];                      // contributing planes in creation order
  uint8_t tlist[T];                      // used triangle slots, compacted
  float4 cf[T];                          // corners (FP32) and their best power bound
  float4 stkl[96];                       // per stack entry, read when it is pushed: the
  uint32_t stkb[96], stke[96];           //   node's linear weight bound, its seed range,
  float stkw[96], stkx[96];              //   its largest weight and the bound's excess
  uint32_t cbest[T];                     // best seed of each corner (certification)
  uint32_t stk[96];                      // octree traversal stack
  uint32_t owner[P];                     // seed slot of each live plane (kNone: none)
};

// Whether the bisector pj of the cell's seed and another seed may put the
// corner of planes p0, p1, p2 in conflict: false only when the FP64 corner
// and its error bound show the corner strictly on the kept side, the test
// the clipping kernels apply before their exact sign (convex_cell.cpp:
// 870-912).  Where the bound cannot decide, the answer is "may": the seed
// is then reported, which costs at most a round.
__device__ __forceinline__ bool corner_in_conflict(double4 p0, double4 p1, double4 p2, double4 pj) {
  double x, y, z;
  float e;
  corner_fp64(p0, p1, p2, x, y, z, e);
  const double sv = fma(pj.z, z, fma(pj.y, y, fma(pj.x, x, pj.w)));
  const double bound = fma((fabs(pj.x) + fabs(pj.y) + fabs(pj.z)) * 1.0001, (double)e,
                           Consts<double>::kDot * fabs(pj.w) * 1.0001);
  return !(sv > bound);
}

// Cell-centred certification.  A seed j cuts the cell only if for some
// corner c its power pi_j(c) = |c - p_j|^2 - w_j is below the seed's own,
// pi_i(c) = |c - p_i|^2 - w_i.  For every corner the warp looks for the
// seed of least power at c among those that may be below pi_i(c) and are
// not yet in the candidate list -- the seed whose Laguerre cell holds c,
// hence a neighbour of the final cell -- and reports the distinct ones as
// extra candidates.  Clipping by them and certifying again ends in a few
// rounds; a round that finds none certifies the cell.
//
// The octree walk is a best-bound search shared by the warp: a node whose
// seeds all have w <= W_B cannot improve corner c when dist(c, box)^2 - W_B
// >= best(c), and is skipped when that holds for every corner (each lane
// tests its own corners).  best(c) starts at pi_i(c) plus a wide FP32
// margin.  Leaves are scanned one seed per lane against every corner, in
// the seed's frame: with c' = c - p_i, q = p_j - p_i and dw = w_j - w_i
// formed from FP32 value/remainder pairs, d = |c' - q|^2 - dw is pi_j(c) -
// pi_i(c) + |c'|^2 within 1e-6 (|c'|^2 + |d| + |dw|) (coordinates,
// squares and the subtraction each round to 2^-24 relative; |c' - q|^2 <=
// |d| + |dw|), so the test d - 4e-6 (|d| + |dw|) <= |c'|^2 (1 + 4e-6) +
// 1e-12 (the floor for the FP64 corner's own rounding) never drops a seed
// that cuts.  Each seed it keeps at some corner and that is not in the list
// yet is broadcast; the corners' owners count the seeds that may cut there
// and keep the least-power one.  After the walk, a corner whose only such
// seed does not cut in FP64 (the corner against its error bound,
// corner_in_conflict) reports nothing: optimal transport cells lie far from
// their seeds, so their corners' powers are large next to the gaps between
// them, and FP32 alone would report many seeds that do not cut.
template <int T, int P, int NCL, typename Sm>
__device__ __forceinline__ void certify_cell(const GeomArgs& a, const SortedSeeds& S,
                                             const GridDesc& gd, uint32_t s, uint32_t row,
                                             int ntri, float4 (&mine)[NCL], Sm& g, int lane) {
  float4* cf = g.cf;
  uint32_t* cbest = g.cbest;
  uint32_t* stk = g.stk;
  const uint32_t* owner = g.owner;
  const unsigned FULL = 0xFFFFFFFFu;
  const float hf = gd.h_f;
  const uint32_t ncand = a.cand_cnt[row] & kCntMask;
  const double4 pi_d = S.xd[s];
  const float4 pi_f = S.xf[s], pi_l = S.xl[s];
  const float2 wi_f = S.wf ? S.wf[s] : make_float2(0.f, 0.f);
  const double qi_d = S.q[s];
  // the reference's FP64 bisector of the cell's seed and seed slot j
  auto seed_plane64 = [&](uint32_t j) {
    const double4 pj = S.xd[j];
    return make_double4(2.0 * __dsub_rn(pi_d.x, pj.x), 2.0 * __dsub_rn(pi_d.y, pj.y),
                        2.0 * __dsub_rn(pi_d.z, pj.z), __dsub_rn(qi_d, S.q[j]));
  };
  // the FP64 test at compacted corner k (corner_in_conflict)
  auto cuts_corner = [&](int k, const double4& pj) {
    const uint32_t v = g.tv[g.tlist[k]];
    return corner_in_conflict(g.plane[v & 0xFF], g.plane[v >> 8 & 0xFF],
                              g.plane[v >> 16 & 0xFF], pj);
  };
  uint32_t bj[NCL], bperm[NCL];  // best seed of each corner and its original index
  float bd[NCL];                 // its d (seed frame)
  uint32_t npos = 0;             // per corner (2 bits): seeds that may cut there, 0, 1, 2+
#pragma unroll
  for (int q = 0; q < NCL; ++q) {
    bj[q] = kNone;
    bperm[q] = 0;
    bd[q] = INFINITY;
    if (mine[q].w > -INFINITY) mine[q].w += 1e-5f * fabsf(mine[q].w) + 1e-7f;
  }
  bool overflow = false;
  unsigned long long n_nodes = 0, n_seeds = 0;
  const bool have_lin = a.node_lin_f != nullptr;
  int sp = 0;
  if (lane == 0) {
    stk[0] = 0u;
    g.stkb[0] = S.cell_start[0];
    g.stke[0] = S.cell_start[1u << (3 * gd.L)];
    g.stkw[0] = a.node_wmax_f[node_offset(0)];
    if (have_lin) {
      g.stkl[0] = a.node_lin_f[node_offset(0)];
      g.stkx[0] = a.node_ex_f[node_offset(0)];
    }
  }
  sp = 1;
  __syncwarp();
  while (sp > 0) {
    const uint32_t e = stk[sp - 1];
    const uint32_t b = g.stkb[sp - 1], en = g.stke[sp - 1];
    const float WB = g.stkw[sp - 1];
    float4 fl = make_float4(0.f, 0.f, 0.f, 0.f);
    float fe = 0.f;
    if (have_lin) {
      fl = g.stkl[sp - 1];
      fe = g.stkx[sp - 1];
    }
    __syncwarp();
    --sp;
    const int lev = (int)(e & 15u);
    const uint32_t code = e >> 4;
    const int shift = gd.L - lev;
    if (b == en) continue;
    ++n_nodes;
    const float side = hf * (float)(1u << shift);
    const float bx = gd.lo_f[0] + (float)compact3(code) * side;
    const float by = gd.lo_f[1] + (float)compact3(code >> 1) * side;
    const float bz = gd.lo_f[2] + (float)compact3(code >> 2) * side;
    const float pad = 1e-6f * (1.f + fabsf(bx) + fabsf(by) + fabsf(bz)) + 1e-5f * side;
    bool ok = true;
#pragma unroll
    for (int q = 0; q < NCL; ++q) {
      const float4 c = mine[q];
      if (!(c.w > -INFINITY)) continue;  // unused slot
      const float dx = fmaxf(fmaxf(bx - pad - c.x, c.x - (bx + side + pad)), 0.f);
      const float dy = fmaxf(fmaxf(by - pad - c.y, c.y - (by + side + pad)), 0.f);
      const float dz = fmaxf(fmaxf(bz - pad - c.z, c.z - (bz + side + pad)), 0.f);
      const float d2 = dx * dx + dy * dy + dz * dz;
      const float need = (c.w + WB) + 1e-5f * (fabsf(c.w) + fabsf(WB) + d2) + 1e-7f;
      const bool clear = (d2 >= need) ||
                         (have_lin && linear_bound_clears(c.x, c.y, c.z, c.w, bx, by, bz, side,
                                                          pad, fl, fe));
      ok = ok && clear;
    }
    if (__all_sync(FULL, ok)) continue;
    if (en - b <= 32u || lev == gd.L) {
      n_seeds += en - b;
      for (uint32_t base = b; base < en; base += 32) {
        const uint32_t j = base + lane;
        bool cut = false;
        float jx = 0.f, jy = 0.f, jz = 0.f, dw = 0.f, sj = 0.f;
        uint32_t jperm = 0;
        if (j < en && j != s) {
          // the seed in the cell seed's frame (the FP64 copy only for a
          // possible copy)
          const float4 jf = S.xf[j], jl = S.xl[j];
          jx = (jf.x - pi_f.x) + (jl.x - pi_l.x);
          jy = (jf.y - pi_f.y) + (jl.y - pi_l.y);
          jz = (jf.z - pi_f.z) + (jl.z - pi_l.z);
          if (S.wf) {
            const float2 w2 = S.wf[j];
            dw = (w2.x - wi_f.x) + (w2.y - wi_f.y);
          }
          // the test's slack for |dw|, with d - 4e-6 |d| folded into the
          // corner's bound (d >= 0; a negative d passes anyway)
          sj = 4.1e-6f * fabsf(dw);
          // a copy of the seed is no neighbour (delaunay_nn.cpp:126-133)
          bool same = false;
          if (jf.x == pi_f.x && jf.y == pi_f.y && jf.z == pi_f.z) {
            const double4 pj = S.xd[j];
            same = pj.x == pi_d.x && pj.y == pi_d.y && pj.z == pi_d.z;
          }
          for (int k = 0; k < ntri && !cut && !same; ++k) {
            const float4 c = cf[k];
            const float dx = c.x - jx, dy = c.y - jy, dz = c.z - jz;
            cut = dx * dx + dy * dy + dz * dz - dw <= c.w + sj;
          }
          if (cut) {
            // already in the candidate list (clipped, cutting or not)?  The
            // seeds of the cell's facets first (shared memory), which are
            // what the corners' bounds meet most; then the whole list
            bool listed = false;
#pragma unroll
            for (int p = 0; p < P; ++p) listed = listed || owner[p] == j;
            if (listed) cut = false;
            for (uint32_t k = 0; k < ncand && cut; ++k)
              if (a.nbr[(size_t)k * a.nbr_stride + row] == j) cut = false;
            if (cut) jperm = S.perm[j];
          }
        }
        unsigned m = __ballot_sync(FULL, cut);
        while (m) {
          const int src = __ffs(m) - 1;
          m &= m - 1;
          const float sx = __shfl_sync(FULL, jx, src), sy = __shfl_sync(FULL, jy, src),
                      sz = __shfl_sync(FULL, jz, src), sw = __shfl_sync(FULL, dw, src),
                      ss = __shfl_sync(FULL, sj, src);
          const uint32_t sid = __shfl_sync(FULL, j, src);
          const uint32_t sperm = __shfl_sync(FULL, jperm, src);
#pragma unroll
          for (int q = 0; q < NCL; ++q) {
            if (!(mine[q].w > -INFINITY)) continue;
            const float4 c = cf[lane + 32 * q];
            const float dx = c.x - sx, dy = c.y - sy, dz = c.z - sz;
            const float d = dx * dx + dy * dy + dz * dz - sw;
            if (!(d <= c.w + ss)) continue;  // cannot cut at this corner
            if (((npos >> (2 * q)) & 3u) < 2u) npos += 1u << (2 * q);
            // the least power so far (ties to the lower original index: the
            // result does not depend on the scan order of the seeds)
            if (d < bd[q] || (d == bd[q] && bj[q] != kNone && sperm < bperm[q])) {
              bd[q] = d;
              bj[q] = sid;
              bperm[q] = sperm;
              // the walk's bound, in the global frame (w_i rounded)
              mine[q].w = fminf(mine[q].w, d - wi_f.x);
            }
          }
        }
        __syncwarp();
      }
      continue;
    }
    if (sp + 8 > 96) {
      overflow = true;
      break;
    }
    // children nearest to the seed (power lower bound) popped first: the
    // corners' bounds then shrink early and prune the rest
    {
      float key = INFINITY;
      bool live = false;
      uint32_t cb0 = 0, ce0 = 0;
      float cw = 0.f;
      if (lane < 8) {
        const uint32_t cc = (code << 3) | (uint32_t)lane;
        const int csh = shift - 1;
        cb0 = S.cell_start[cc << (3 * csh)];
        ce0 = S.cell_start[(cc + 1u) << (3 * csh)];
        live = cb0 != ce0;
        if (live) {
          const float cs = 0.5f * side;
          const float qx = bx + (float)(lane & 1) * cs, qy = by + (float)((lane >> 1) & 1) * cs,
                      qz = bz + (float)((lane >> 2) & 1) * cs;
          const float sx = (float)pi_d.x, sy = (float)pi_d.y, sz = (float)pi_d.z;
          const float ex = fmaxf(fmaxf(qx - sx, sx - (qx + cs)), 0.f);
          const float ey = fmaxf(fmaxf(qy - sy, sy - (qy + cs)), 0.f);
          const float ez = fmaxf(fmaxf(qz - sz, sz - (qz + cs)), 0.f);
          cw = a.node_wmax_f[node_offset(lev + 1) + cc];
          key = ex * ex + ey * ey + ez * ez - cw;
        }
      }
      const unsigned lm = __ballot_sync(FULL, live);
      // rank among the live children, descending key (ties by child index)
      int rank = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float kk = __shfl_sync(FULL, key, k);
        if (((lm >> k) & 1u) && (kk > key || (kk == key && k < lane))) ++rank;
      }
      if (live) {
        const int at = sp + rank;
        const uint32_t cc = (code << 3) | (uint32_t)lane;
        stk[at] = (cc << 4) | (uint32_t)(lev + 1);
        g.stkb[at] = cb0;
        g.stke[at] = ce0;
        g.stkw[at] = cw;
        if (have_lin) {
          g.stkl[at] = a.node_lin_f[node_offset(lev + 1) + cc];
          g.stkx[at] = a.node_ex_f[node_offset(lev + 1) + cc];
        }
      }
      __syncwarp();
      sp += __popc(lm);
    }
  }
  // A corner whose only possible cutter does not cut in FP64 has none.
  // (With two or more, the least-power one in FP32 is reported as it is:
  // another may cut.)
  {
    uint32_t chk = 0;
#pragma unroll
    for (int q = 0; q < NCL; ++q)
      if (bj[q] != kNone && ((npos >> (2 * q)) & 3u) == 1u) chk |= 1u << q;
    while (chk) {  // one corner at a time: the FP64 test once in the code
      const int qn = __ffs(chk) - 1;
      chk &= chk - 1;
      uint32_t sid = kNone;
#pragma unroll
      for (int q = 0; q < NCL; ++q)
        if (q == qn) sid = bj[q];
      if (cuts_corner(lane + 32 * qn, seed_plane64(sid))) continue;
#pragma unroll
      for (int q = 0; q < NCL; ++q)
        if (q == qn) bj[q] = kNone;
    }
  }
  // the distinct best seeds, in corner order
#pragma unroll
  for (int q = 0; q < NCL; ++q)
    if (lane + 32 * q < T) cbest[lane + 32 * q] = (lane + 32 * q < ntri) ? bj[q] : kNone;
  __syncwarp();
  uint32_t found = 0;
#pragma unroll
  for (int q = 0; q < NCL; ++q) {
    const int i = lane + 32 * q;
    const uint32_t v = (i < ntri) ? bj[q] : kNone;
    bool take = v != kNone;
    for (int k = 0; k < i && take; ++k)
      if (cbest[k] == v) take = false;
    const unsigned m = __ballot_sync(FULL, take);
    if (take) {
      const uint32_t pos = found + __popc(m & ((1u << lane) - 1u));
      if (pos < a.max_extra) a.extra[(size_t)pos * a.nbr_stride + row] = v;
    }
    found += __popc(m);
  }
  if (lane == 0) {
    const bool more = overflow || found > a.max_extra;
    a.extra_cnt[row] = (found < a.max_extra ? found : a.max_extra) | (more ? 0x80000000u : 0u);
    if (a.cert_stats) {
      atomicAdd(&a.cert_stats[0], n_nodes);
      atomicAdd(&a.cert_stats[1], n_seeds);
      atomicMax(&a.cert_stats[2], n_nodes);
      atomicMax(&a.cert_stats[3], n_seeds);
      atomicAdd(&a.cert_stats[4], 1ull);
    }
  }
  __syncwarp();
}

// The FP32 plane of owner `own` in the frame centred on seed s (value and
// remainder of the coordinates, as the FP32 clipping kernel forms it).
__device__ __forceinline__ float4 local_plane32(uint32_t own, uint32_t s, const SortedSeeds& S,
                                                const double* box) {
  const float4 fh = S.xf[s], fl = S.xl[s];
  if (own >= kBoxBase) {
    switch (own - kBoxBase) {
      case 0: return make_float4(1.f, 0.f, 0.f, (fh.x - (float)box[0]) + fl.x);
      case 1: return make_float4(-1.f, 0.f, 0.f, ((float)box[3] - fh.x) - fl.x);
      case 2: return make_float4(0.f, 1.f, 0.f, (fh.y - (float)box[1]) + fl.y);
      case 3: return make_float4(0.f, -1.f, 0.f, ((float)box[4] - fh.y) - fl.y);
      case 4: return make_float4(0.f, 0.f, 1.f, (fh.z - (float)box[2]) + fl.z);
      default: return make_float4(0.f, 0.f, -1.f, ((float)box[5] - fh.z) - fl.z);
    }
  }
  const float4 jh = S.xf[own], jl = S.xl[own];
  const float dx = (jh.x - fh.x) + (jl.x - fl.x);
  const float dy = (jh.y - fh.y) + (jl.y - fl.y);
  const float dz = (jh.z - fh.z) + (jl.z - fl.z);
  float dw = 0.f;
  if (S.wf) {
    const float2 wi = S.wf[s], wj = S.wf[own];
    dw = (wj.x - wi.x) + (wj.y - wi.y);
  }
  return make_float4(-2.f * dx, -2.f * dy, -2.f * dz, dx * dx + dy * dy + dz * dz - dw);
}

__device__ __forceinline__ float4 to_f4(const double4& q) {
  return make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
}

// CERT: the power-range certification (a.node_wmax set); its walk is kept
// out of the plain kernels, whose registers it would raise.
template <int T, int P, bool G32, bool CERT>
__global__ void __launch_bounds__(kGeomWarps * 32) geom_kernel(GeomArgs a) {
  constexpr int NH = (P + 31) / 32;  // planes (and ranks) per lane
  using Sm = GeomWarpSmem<T, P>;
  extern __shared__ __align__(16) unsigned char geom_smem[];
  Sm* smw = reinterpret_cast<Sm*>(geom_smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t ci = blockIdx.x * kGeomWarps + warp;
  if (ci >= a.nq) return;
  Sm& g = smw[warp];
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
  const unsigned FULL = 0xFFFFFFFFu;

  // ---- used triangles, compacted; planes (FP64, the reference's frame)
  const int nt0 = __popcll(tm2.x);
  const int ntri = nt0 + (T > 64 ? __popcll(tm2.y) : 0);
  for (int h = 0; h < (T > 64 ? 2 : 1); ++h) {
    const uint64_t w = h ? tm2.y : tm2.x;
    for (int b = 2 * lane; b < 2 * lane + 2; ++b) {
      if (!((w >> b) & 1ull)) continue;
      const int pos = (h ? nt0 : 0) + __popcll(w & ((1ull << b) - 1ull));
      const int t = 64 * h + b;
      g.tlist[pos] = (uint8_t)t;
      g.tv[t] = cb.tv[tb + t];
      g.tadj[t] = cb.ta[tb + t];
    }
  }
  for (int p = lane; p < P; p += 32) {
    g.v2t[p] = -1;
    g.prank[p] = 0xFFFF;
    g.owner[p] = kNone;
    if ((pm >> p) & 1ull) {
      g.prank[p] = cb.prank[pb + p];
      const uint32_t own = cb.pown[pb + p];
      g.owner[p] = own;
      double4 Q;
      if constexpr (G32) {
        const float4 f = local_plane32(own, s, S, a.box);
        Q = make_double4(f.x, f.y, f.z, f.w);
      } else if (own >= kBoxBase) {
        switch (own - kBoxBase) {
          case 0: Q = make_double4(1.0, 0.0, 0.0, -a.box[0]); break;
          case 1: Q = make_double4(-1.0, 0.0, 0.0, a.box[3]); break;
          case 2: Q = make_double4(0.0, 1.0, 0.0, -a.box[1]); break;
          case 3: Q = make_double4(0.0, -1.0, 0.0, a.box[4]); break;
          case 4: Q = make_double4(0.0, 0.0, 1.0, -a.box[2]); break;
          default: Q = make_double4(0.0, 0.0, -1.0, a.box[5]); break;
        }
      } else {
        const double4 pj = S.xd[own];
        Q = make_double4(2.0 * __dsub_rn(pi.x, pj.x), 2.0 * __dsub_rn(pi.y, pj.y),
                         2.0 * __dsub_rn(pi.z, pj.z), __dsub_rn(qi, S.q[own]));
      }
      g.plane[p] = Q;
    }
  }
  __syncwarp();
  // ---- corners (compute_geometry) and v2t
  double R2 = 0.0, R2lo = 0.0;  // G32: bounds on the reference's R2 (R2 the upper one)
  for (int i = lane; i < ntri; i += 32) {
    const int t = g.tlist[i];
    const uint32_t v = g.tv[t];
    const int a0 = v & 0xFF, a1 = v >> 8 & 0xFF, a2 = v >> 16 & 0xFF;
    if constexpr (G32) {
      float x, y, z, e;
      corner_fp32(to_f4(g.plane[a0]), to_f4(g.plane[a1]), to_f4(g.plane[a2]), x, y, z, e);
      g.px[t] = x;
      g.py[t] = y;
      g.pz[t] = z;
      // |c|^2 within 2 |c|_1 e + 3 e^2 of the exact corner's, plus its own
      // FP32 rounding; FP64 slack for the reference's own rounding
      const double r2 = (double)x * x + (double)y * y + (double)z * z;
      const double m1 = fabs((double)x) + fabs((double)y) + fabs((double)z);
      const double er = 2.0 * m1 * e + 3.0 * (double)e * e + r2 * 1e-12;
      R2 = fmax(R2, r2 + er);
      R2lo = fmax(R2lo, r2 - er);
    } else {
      const double3 c = r_corner(g.plane[a0], g.plane[a1], g.plane[a2]);
      g.px[t] = c.x;
      g.py[t] = c.y;
      g.pz[t] = c.z;
      R2 = fmax(R2, r_sqdist(pi.x, pi.y, pi.z, c));
    }
    const int eff = parity * (int)cb.key[tb + t];
    const int packed = ((eff + 32768) << 8) | t;
    atomicMax(&g.v2t[a0], packed);
    atomicMax(&g.v2t[a1], packed);
    atomicMax(&g.v2t[a2], packed);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R2 = fmax(R2, __shfl_xor_sync(FULL, R2, o));
    if constexpr (G32) R2lo = fmax(R2lo, __shfl_xor_sync(FULL, R2lo, o));
  }
  __syncwarp();

  // ---- cell-centred certification (power range query)
  if constexpr (CERT && !G32) {
    constexpr int NCL = (T + 31) / 32;
    const double wi = S.ws ? S.ws[s] : 0.0;
    float4 mine[NCL];
#pragma unroll
    for (int q = 0; q < NCL; ++q) {
      const int i = lane + 32 * q;
      mine[q] = make_float4(0.f, 0.f, 0.f, -INFINITY);
      if (i < ntri) {
        const int t = g.tlist[i];
        const double dx = g.px[t] - pi.x, dy = g.py[t] - pi.y, dz = g.pz[t] - pi.z;
        const double r2 = dx * dx + dy * dy + dz * dz;
        mine[q] = make_float4((float)g.px[t], (float)g.py[t], (float)g.pz[t], (float)(r2 - wi));
        // the corner in the seed's frame and the bound on a candidate's
        // power there (certify_cell)
        const float lx = (float)dx, ly = (float)dy, lz = (float)dz;
        const float base = lx * lx + ly * ly + lz * lz;
        g.cf[i] = make_float4(lx, ly, lz, (base * (1.f + 4e-6f) + 1e-12f) * (1.f + 5e-6f));
      }
    }
    __syncwarp();
    const GridDesc gd = *S.gd;
    const uint32_t row = a.qrow ? a.qrow[ci] : ci;
    certify_cell<T, P, NCL>(a, S, gd, s, row, ntri, mine, g, lane);
    __syncwarp();
  }

  // ---- FP32 clipping: the reference stops at the same neighbour only if
  // d(stop) > 4.1 (R2 + h^2) and d(last clipped) <= 4.1 (R2 + h^2) with the
  // final cell's R2 (R2 only shrinks while clipping)
  if (a.verify_sr &&
      (st == CELL_CERTIFIED || st == CELL_ALL_NEIGHBOURS || st == CELL_STALLED)) {
    const uint32_t row = a.qrow ? a.qrow[ci] : ci;
    const uint32_t jj = a.nclip[s];
    // G32: the reference's threshold lies between these two (rounding is
    // monotonic); the FP64 corners give it exactly
    const double thr = __dmul_rn(4.1, __dadd_rn(R2, __dmul_rn(pi.w, pi.w)));
    const double thr_lo = G32 ? __dmul_rn(4.1, __dadd_rn(R2lo, __dmul_rn(pi.w, pi.w))) : thr;
    bool ok = true;
    if (st == CELL_CERTIFIED) {
      const uint32_t js = a.nbr[(size_t)jj * a.nbr_stride + row];
      ok = dist2_exact(pi, S.xd[js]) > thr;
    }
    if (ok && jj > 0) {
      const uint32_t jl = a.nbr[(size_t)(jj - 1) * a.nbr_stride + row];
      ok = !(dist2_exact(pi, S.xd[jl]) > thr_lo);
    }
    if (!ok) {
      if (lane == 0) a.status[s] = CELL_RECHECK;
      return;
    }
  }

  // ---- planes in the reference's creation order: box faces 0-5 (their
  // slots), then the seeds in clipping order (list position)
  int rank_of[NH], nseed_before[NH];
  bool is_seed[NH];
  int ncontrib = 0;
  {
    int cidx[NH];
#pragma unroll
    for (int h = 0; h < NH; ++h) {
      const int p = lane + 32 * h;
      rank_of[h] = -1;
      nseed_before[h] = 0;
      is_seed[h] = false;
      cidx[h] = 0x7FFFFFFF;
      if (p < P && g.v2t[p] >= 0) {
        is_seed[h] = g.prank[p] != 0xFFFF;
        cidx[h] = is_seed[h] ? 6 + g.prank[p] : p;
        rank_of[h] = 0;
      }
    }
    for (int q = 0; q < P; ++q) {
      if (g.v2t[q] < 0) continue;
      ++ncontrib;
      const bool qseed = g.prank[q] != 0xFFFF;
      const int iq = qseed ? 6 + g.prank[q] : q;
#pragma unroll
      for (int h = 0; h < NH; ++h) {
        if (rank_of[h] < 0) continue;
        if (iq < cidx[h]) {
          ++rank_of[h];
          if (qseed) ++nseed_before[h];
        }
      }
    }
#pragma unroll
    for (int h = 0; h < NH; ++h)
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
  auto next_around = [&](uint32_t t, uint32_t v) -> uint32_t {
    const uint32_t x = g.tv[t];
    const int lv = ((x >> 8 & 0xFF) == v) + 2 * ((x >> 16 & 0xFF) == v);
    return (g.tadj[t] >> (8 * ((lv + 1) % 3))) & 0xFF;
  };
  // ---- fan lengths per rank
  int deg_r[NH], vol_r[NH], area_r[NH];
#pragma unroll
  for (int h = 0; h < NH; ++h) {
    const int r = lane + 32 * h;
    deg_r[h] = 0;
    if (r < ncontrib) {
      const int p = g.order[r];
      const uint32_t t0 = g.v2t[p] & 0xFF;
      uint32_t t = t0;
      int deg = 0;
      do {
        ++deg;
        t = next_around(t, p);
      } while (t != t0 && deg < 3 * T);
      deg_r[h] = deg;
    }
    vol_r[h] = (r < ncontrib && r > 0) ? deg_r[h] - 2 : 0;
    area_r[h] = (r < ncontrib && g.prank[g.order[r]] != 0xFFFF) ? deg_r[h] - 2 : 0;
  }
  // exclusive scans over the ranks of: fan length, volume terms, area terms
  {
    int base_f = 0, base_v = 0, base_a = 0;
#pragma unroll
    for (int h = 0; h < NH; ++h) {
      int f = deg_r[h], v = vol_r[h], ar = area_r[h];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int yf = __shfl_up_sync(FULL, f, o), yv = __shfl_up_sync(FULL, v, o),
                  ya = __shfl_up_sync(FULL, ar, o);
        if (lane >= o) {
          f += yf;
          v += yv;
          ar += ya;
        }
      }
      const int r = lane + 32 * h;
      if (r < P) {
        g.fstart[r] = (int16_t)(base_f + f - deg_r[h]);
        g.vofs[r] = (int16_t)(base_v + v - vol_r[h]);
        g.aofs[r] = (int16_t)(base_a + ar - area_r[h]);
      }
      base_f += __shfl_sync(FULL, f, 31);
      base_v += __shfl_sync(FULL, v, 31);
      base_a += __shfl_sync(FULL, ar, 31);
    }
    if (lane == 0) {
      g.fstart[P] = (int16_t)base_f;
      g.vofs[P] = (int16_t)base_v;
      g.aofs[P] = (int16_t)base_a;
    }
  }
  __syncwarp();
  // ---- fan sequences (triangles around each plane from v2t)
#pragma unroll
  for (int h = 0; h < NH; ++h) {
    const int r = lane + 32 * h;
    if (r >= ncontrib) continue;
    const int p = g.order[r];
    const uint32_t t0 = g.v2t[p] & 0xFF;
    uint32_t t = t0;
    int k = g.fstart[r];
    const int kend = k + deg_r[h];
    do {
      g.fan[k++] = (uint8_t)t;
      t = next_around(t, p);
    } while (t != t0 && k < kend);
  }
  __syncwarp();
  const int nvol = min((int)g.vofs[P], Sm::kTerms), narea = min((int)g.aofs[P], Sm::kTerms);
  const int t_origin = g.v2t[g.order[0]] & 0xFF;
  const double3 po = make_double3(g.px[t_origin], g.py[t_origin], g.pz[t_origin]);
  auto corner = [&](int t) { return make_double3(g.px[t], g.py[t], g.pz[t]); };
  // the rank owning term k: the last rank whose offset is <= k
  auto rank_of_term = [&](const int16_t* ofs, int k) -> int {
    int lo = 0, hi = ncontrib - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ofs[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  };
  // ---- tetrahedron terms of compute_mg: tet j of rank r is
  // (t_origin, fan[0], fan[j+1], fan[j+2])
  for (int k = lane; k < nvol; k += 32) {
    const int r = rank_of_term(g.vofs, k);
    const int j = k - g.vofs[r];
    const uint8_t* fan = &g.fan[g.fstart[r]];
    const double3 q1 = corner(fan[0]), q2 = corner(fan[j + 1]), q3 = corner(fan[j + 2]);
    if constexpr (G32) {
      const float ux = (float)q1.x - (float)po.x, uy = (float)q1.y - (float)po.y,
                  uz = (float)q1.z - (float)po.z;
      const float vx = (float)q2.x - (float)po.x, vy = (float)q2.y - (float)po.y,
                  vz = (float)q2.z - (float)po.z;
      const float wx = (float)q3.x - (float)po.x, wy = (float)q3.y - (float)po.y,
                  wz = (float)q3.z - (float)po.z;
      const float d = (uy * vz - uz * vy) * wx + (uz * vx - ux * vz) * wy + (ux * vy - uy * vx) * wz;
      const float cm = fabsf(d) * (1.f / 6.f);
      g.tm[k] = cm;
      g.tx[k] = cm * ((float)po.x + (float)q1.x + (float)q2.x + (float)q3.x) * 0.25f;
      g.ty[k] = cm * ((float)po.y + (float)q1.y + (float)q2.y + (float)q3.y) * 0.25f;
      g.tz[k] = cm * ((float)po.z + (float)q1.z + (float)q2.z + (float)q3.z) * 0.25f;
    } else {
      const double cm = r_tet_volume(po, q1, q2, q3);
      g.tm[k] = cm;
      // cm * (p + q + r + s) / 4.0: the division by 4 is the exact product by 0.25
      g.tx[k] = __dmul_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(po.x, q1.x), q2.x), q3.x)), 0.25);
      g.ty[k] = __dmul_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(po.y, q1.y), q2.y), q3.y)), 0.25);
      g.tz[k] = __dmul_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(po.z, q1.z), q2.z), q3.z)), 0.25);
    }
  }
  // ---- facet-area terms: triangle j of a seed facet is (fan[0], fan[j+1], fan[j+2])
  for (int k = lane; k < narea; k += 32) {
    const int r = rank_of_term(g.aofs, k);
    const int j = k - g.aofs[r];
    const uint8_t* fan = &g.fan[g.fstart[r]];
    if constexpr (G32) {
      const double3 p1 = corner(fan[0]), p2 = corner(fan[j + 1]), p3 = corner(fan[j + 2]);
      const float ux = (float)p2.x - (float)p1.x, uy = (float)p2.y - (float)p1.y,
                  uz = (float)p2.z - (float)p1.z;
      const float vx = (float)p3.x - (float)p1.x, vy = (float)p3.y - (float)p1.y,
                  vz = (float)p3.z - (float)p1.z;
      const float cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
      g.ta[k] = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
    } else {
      g.ta[k] = r_triangle_area(corner(fan[0]), corner(fan[j + 1]), corner(fan[j + 2]));
    }
  }
  __syncwarp();
  // ---- sums in the reference's order: one accumulator per lane 0-3
  if (lane < 4) {
    const double* src = lane == 0 ? g.tm : (lane == 1 ? g.tx : (lane == 2 ? g.ty : g.tz));
    double acc = 0.0;
    for (int k = 0; k < nvol; ++k) acc = __dadd_rn(acc, src[k]);
    if constexpr (G32) {
      // back from the seed's frame: mg = mg_local + m p_i
      const double m = __shfl_sync(0xFu, acc, 0, 4);
      const double pc = lane == 1 ? pi.x : (lane == 2 ? pi.y : pi.z);
      if (lane > 0) acc = fma(m, pc, acc);
    }
    if (lane == 0) a.vol[s] = acc;
    else a.mg[(size_t)(lane - 1) * a.out_stride + s] = acc;
  }
  // ---- facets shared with other seeds, in clipping order
  int nfac_lane = 0;
#pragma unroll
  for (int h = 0; h < NH; ++h) {
    const int p = lane + 32 * h;
    if (rank_of[h] < 0 || !is_seed[h]) continue;
    ++nfac_lane;
    const int r = rank_of[h];
    double area = 0.0;
    const int k1 = min((int)g.aofs[r + 1], narea);
    for (int k = g.aofs[r]; k < k1; ++k) area = __dadd_rn(area, g.ta[k]);
    const int pos = nseed_before[h];
    a.f_nbr[(size_t)pos * a.out_stride + s] = S.perm[cb.pown[pb + p]];
    a.f_area[(size_t)pos * a.out_stride + s] = area;
  }
  int nfac = nfac_lane;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nfac += __shfl_xor_sync(FULL, nfac, o);
  if (lane == 0) a.nf[s] = (uint32_t)nfac;
}

template <int T, int P, bool G32, bool CERT>
static void launch_geom(const GeomArgs& a, cudaStream_t st) {
  const size_t sh = sizeof(GeomWarpSmem<T, P>) * kGeomWarps;
  cudaFuncSetAttribute(geom_kernel<T, P, G32, CERT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sh);
  const unsigned nb = (a.nq + kGeomWarps - 1) / kGeomWarps;
  geom_kernel<T, P, G32, CERT><<<nb, kGeomWarps * 32, sh, st>>>(a); count_launch();
  last_launch_error = cudaGetLastError();
}

void launch_geometry(const GeomArgs& a, cudaStream_t st) {
  if (a.nq == 0) return;
  const bool large = a.shape == CLIP_LARGE;
  if (a.g32) {
    if (large) launch_geom<kLargeT, kLargeP, true, false>(a, st);
    else launch_geom<kSmallT, kSmallP, true, false>(a, st);
  } else if (a.node_wmax) {
    if (large) launch_geom<kLargeT, kLargeP, false, true>(a, st);
    else launch_geom<kSmallT, kSmallP, false, true>(a, st);
  } else {
    if (large) launch_geom<kLargeT, kLargeP, false, false>(a, st);
    else launch_geom<kSmallT, kSmallP, false, false>(a, st);
  }
}

}  // namespace gbv
