// Laguerre / Voronoi cells restricted to a tetrahedral mesh: what the
// reference's volumetric RestrictedVoronoiDiagram integrates
// (voronoi/RVD.cpp: compute_centroids_in_volume :500-530 with
// ComputeCentroidsVolumetric :429-497, compute_CVT_func_grad_in_volume
// :878-910 with ComputeCVTFuncGradVolumetric :792-870).
//
// The reference walks the mesh and the Delaunay triangulation together
// (generic_RVD.h).  Here every seed's cell is first certified in the mesh's
// bounding box by the meshless engine; the cell is then the box cut by the
// bisectors of its facet neighbours, so its part in a tetrahedron T is T cut
// by those bisectors alone.  One thread per cell finds the tetrahedra that
// may meet the cell in a grid of bins (every tetrahedron is listed in the
// bins its bounding box overlaps, bins sorted, each tetrahedron taken in
// the first bin it shares with the cell), clips each one by the cell's
// planes (a small polyhedron clipper on outward-oriented polygons), and
// integrates the pieces in that fixed order: mass, first moment, and the
// CVT energy int |x - p_i|^2 and its gradient by tetrahedra from the seed
// to the border of the restricted cell, as the reference forms them (fi =
// m/10 (U.U + V.V + W.W + U.V + V.W + W.U), gi = 2 m (p - centroid), m
// unsigned: exact for cells star-shaped from their seed, and the
// reference's value otherwise).  FP64 throughout; the decomposition
// differs from the reference's, so results agree to rounding, not bit for
// bit.
#include <cfloat>

#include "gbv_context.cuh"
#include "gbv_refgeom.cuh"

namespace gbv {
namespace {

constexpr int kRvMaxV = 96;    // vertices of a piece while clipping
constexpr int kRvMaxF = 40;    // polygons
constexpr int kRvMaxFV = 320;  // polygon entries
constexpr int kRvMaxCut = 48;  // edges cut by one plane

struct Piece {
  double3 v[kRvMaxV];
  uint16_t fs[kRvMaxF + 1];  // polygon f: fv[fs[f] .. fs[f + 1])
  uint8_t fv[kRvMaxFV];
  uint8_t tag[kRvMaxF];      // 0-3: on that face of the tetrahedron, 4: on a bisector
  int nv, nf;
};

// The tetrahedron's faces as outward counter-clockwise polygons of a
// positively oriented tetrahedron (a, b, c, d).
__constant__ uint8_t kTetFace[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {1, 2, 3}};

struct RestrictArgs {
  uint32_t n;
  const double* xyz;       // seeds, caller order [n][3]
  const double* w;         // weights or null
  const uint32_t* rowptr;  // cell facets (CSR, caller order)
  const uint32_t* nbr;
  const uint32_t* slot_of;
  const uint32_t* nf;      // per slot (bit kHugeFacets: no stored polytope)
  CombBuf cb;
  const double4* xd;       // sorted seeds (for the cell's corners)
  const double* q;
  double box[6];
  const double* mv;        // mesh vertices [nv][3]
  const uint32_t* tets;    // [nt][4], positively oriented
  uint32_t nt;
  int G;                   // bins per axis
  double bin_lo[3], bin_h[3];
  const uint32_t* bin_start;  // G^3 + 1
  const uint32_t* bin_tets;
  const uint8_t* bmask;    // per tetrahedron: bit k set when face k is on the mesh boundary
  double* m;
  double* mg;              // [n][3]
  double* F;               // per cell CVT energy
  double* g;               // [n][3] CVT gradient
  uint32_t* err;           // [0] pieces beyond the clipper's capacity
};

__device__ __forceinline__ int bin_of(double x, double lo, double h, int G) {
  int b = (int)floor((x - lo) / h);
  return b < 0 ? 0 : (b >= G ? G - 1 : b);
}

// Plane n.x <= c of the bisector of seed i against seed j (the part of
// space where i's power is the smaller one).
__device__ __forceinline__ void bisector(const double* pi, double wi, const double* pj, double wj,
                                         double3& nrm, double& c) {
  nrm = make_double3(2.0 * (pj[0] - pi[0]), 2.0 * (pj[1] - pi[1]), 2.0 * (pj[2] - pi[2]));
  const double li = pi[0] * pi[0] + pi[1] * pi[1] + pi[2] * pi[2];
  const double lj = pj[0] * pj[0] + pj[1] * pj[1] + pj[2] * pj[2];
  c = (lj - wj) - (li - wi);
}

__device__ void tet_piece(Piece& P, const double3& a, const double3& b, const double3& c,
                          const double3& d) {
  P.v[0] = a;
  P.v[1] = b;
  P.v[2] = c;
  P.v[3] = d;
  P.nv = 4;
  for (int k = 0; k < 4; ++k) {
    for (int e = 0; e < 3; ++e) P.fv[3 * k + e] = kTetFace[k][e];
    P.tag[k] = (uint8_t)k;
  }
  for (int k = 0; k <= 4; ++k) P.fs[k] = (uint16_t)(3 * k);
  P.nf = 4;
}

// Keeps the part of P where nrm.x <= c.  Returns false when nothing is left
// (or sets *overflow when the piece outgrows the fixed capacity).
__device__ bool clip_piece(Piece& P, const double3& nrm, double c, bool* overflow) {
  double sv[kRvMaxV];
  bool any_out = false, any_in = false;
  for (int i = 0; i < P.nv; ++i) {
    sv[i] = c - (nrm.x * P.v[i].x + nrm.y * P.v[i].y + nrm.z * P.v[i].z);
    if (sv[i] < 0.0) any_out = true;
    else any_in = true;
  }
  if (!any_out) return true;
  if (!any_in) return false;
  // kept vertices renumbered first, then one new vertex per cut edge
  int remap[kRvMaxV];
  double3 nvx[kRvMaxV];
  int nn = 0;
  for (int i = 0; i < P.nv; ++i) {
    remap[i] = sv[i] >= 0.0 ? nn : -1;
    if (sv[i] >= 0.0) nvx[nn++] = P.v[i];
  }
  int cut_a[kRvMaxCut], cut_b[kRvMaxCut], cut_id[kRvMaxCut];
  int ncut = 0;
  int cap_next[kRvMaxV];
  for (int i = 0; i < kRvMaxV; ++i) cap_next[i] = -1;
  auto cut_vertex = [&](int u, int x) -> int {
    const int lo = min(u, x), hi = max(u, x);
    for (int k = 0; k < ncut; ++k)
      if (cut_a[k] == lo && cut_b[k] == hi) return cut_id[k];
    if (ncut == kRvMaxCut || nn == kRvMaxV) {
      *overflow = true;
      return 0;
    }
    const double t = sv[u] / (sv[u] - sv[x]);
    const double3 pu = P.v[u], px = P.v[x];
    nvx[nn] = make_double3(pu.x + t * (px.x - pu.x), pu.y + t * (px.y - pu.y),
                           pu.z + t * (px.z - pu.z));
    cut_a[ncut] = lo;
    cut_b[ncut] = hi;
    cut_id[ncut++] = nn;
    return nn++;
  };
  uint16_t nfs[kRvMaxF + 1];
  uint8_t nfv[kRvMaxFV];
  uint8_t ntag[kRvMaxF];
  int nnf = 0, nfe = 0;
  for (int f = 0; f < P.nf; ++f) {
    const int b = P.fs[f], e = P.fs[f + 1], len = e - b;
    const int start = nfe;
    int exitv = -1, entryv = -1;
    for (int k = 0; k < len; ++k) {
      const int u = P.fv[b + k], x = P.fv[b + (k + 1) % len];
      const bool iu = sv[u] >= 0.0, ix = sv[x] >= 0.0;
      if (iu) {
        if (nfe == kRvMaxFV) { *overflow = true; return false; }
        nfv[nfe++] = (uint8_t)remap[u];
      }
      if (iu != ix) {
        const int cv = cut_vertex(u, x);
        if (*overflow || nfe == kRvMaxFV) { *overflow = true; return false; }
        nfv[nfe++] = (uint8_t)cv;
        if (iu) exitv = cv;
        else entryv = cv;
      }
    }
    if (nfe - start >= 3) {
      if (nnf == kRvMaxF) { *overflow = true; return false; }
      ntag[nnf] = P.tag[f];
      nfs[nnf++] = (uint16_t)start;
      // the new polygon runs the cut edge exit -> entry the other way
      if (exitv >= 0 && entryv >= 0) cap_next[entryv] = exitv;
    } else {
      nfe = start;
    }
  }
  // the cap polygon on the plane, chained through the reversed cut edges
  int first = -1;
  for (int k = 0; k < ncut; ++k)
    if (cap_next[cut_id[k]] >= 0) { first = cut_id[k]; break; }
  if (first >= 0) {
    const int start = nfe;
    int v = first, steps = 0;
    do {
      if (nfe == kRvMaxFV) { *overflow = true; return false; }
      nfv[nfe++] = (uint8_t)v;
      v = cap_next[v];
    } while (v >= 0 && v != first && ++steps < kRvMaxCut);
    if (nfe - start >= 3 && nnf < kRvMaxF) {
      ntag[nnf] = 4;
      nfs[nnf++] = (uint16_t)start;
    } else {
      nfe = start;
    }
  }
  nfs[nnf] = (uint16_t)nfe;
  for (int i = 0; i < nn; ++i) P.v[i] = nvx[i];
  for (int f = 0; f <= nnf; ++f) P.fs[f] = nfs[f];
  for (int f = 0; f < nnf; ++f) P.tag[f] = ntag[f];
  for (int k = 0; k < nfe; ++k) P.fv[k] = nfv[k];
  P.nv = nn;
  P.nf = nnf;
  return nnf >= 4;
}

// Adds the piece's mass and first moment (tetrahedra from p to the fans of
// its outward polygons, signed: exact for any piece), and the CVT energy and
// gradient terms as the reference forms them: tetrahedra from the seed p to
// the polygons on the border of the restricted cell only (on a bisector, or
// on a face of the mesh's boundary: bmask bit k for tetrahedron face k),
// each polygon counted with the absolute volumes of its cones (Geom::
// tetra_volume is unsigned; the cones of one planar polygon share a sign).
__device__ void integrate_piece(const Piece& P, const double* p, uint32_t bmask, double& m,
                                double3& mg, double& F, double3& gv) {
  for (int f = 0; f < P.nf; ++f) {
    const int b = P.fs[f], e = P.fs[f + 1];
    const double3 v0 = P.v[P.fv[b]];
    double fm = 0.0, fF = 0.0;
    double3 fg = make_double3(0.0, 0.0, 0.0);
    for (int k = b + 1; k + 1 < e; ++k) {
      const double3 v1 = P.v[P.fv[k]], v2 = P.v[P.fv[k + 1]];
      const double Ux = v0.x - p[0], Uy = v0.y - p[1], Uz = v0.z - p[2];
      const double Vx = v1.x - p[0], Vy = v1.y - p[1], Vz = v1.z - p[2];
      const double Wx = v2.x - p[0], Wy = v2.y - p[1], Wz = v2.z - p[2];
      const double vol = (Ux * (Vy * Wz - Vz * Wy) - Uy * (Vx * Wz - Vz * Wx) +
                          Uz * (Vx * Wy - Vy * Wx)) / 6.0;
      fm += vol;
      const double s = vol / 4.0;
      mg.x += s * (p[0] + v0.x + v1.x + v2.x);
      mg.y += s * (p[1] + v0.y + v1.y + v2.y);
      mg.z += s * (p[2] + v0.z + v1.z + v2.z);
      const double q = Ux * Ux + Uy * Uy + Uz * Uz + Vx * Vx + Vy * Vy + Vz * Vz + Wx * Wx +
                       Wy * Wy + Wz * Wz + (Ux * Vx + Uy * Vy + Uz * Vz) +
                       (Vx * Wx + Vy * Wy + Vz * Wz) + (Wx * Ux + Wy * Uy + Wz * Uz);
      fF += vol / 10.0 * q;
      // 2 m (p - (p + v0 + v1 + v2) / 4)
      fg.x += 2.0 * vol * (0.75 * p[0] - 0.25 * v0.x - 0.25 * v1.x - 0.25 * v2.x);
      fg.y += 2.0 * vol * (0.75 * p[1] - 0.25 * v0.y - 0.25 * v1.y - 0.25 * v2.y);
      fg.z += 2.0 * vol * (0.75 * p[2] - 0.25 * v0.z - 0.25 * v1.z - 0.25 * v2.z);
    }
    m += fm;
    const uint8_t tg = P.tag[f];
    if (tg == 4 || ((bmask >> tg) & 1u)) {
      const double sg = fm >= 0.0 ? 1.0 : -1.0;
      F += sg * fF;
      gv.x += sg * fg.x;
      gv.y += sg * fg.y;
      gv.z += sg * fg.z;
    }
  }
}

__device__ __forceinline__ double4 restrict_plane(const RestrictArgs& a, uint32_t own,
                                                  const double4& pi, double qi) {
  if (own >= kBoxBase) {
    switch (own - kBoxBase) {
      case 0: return make_double4(1.0, 0.0, 0.0, -a.box[0]);
      case 1: return make_double4(-1.0, 0.0, 0.0, a.box[3]);
      case 2: return make_double4(0.0, 1.0, 0.0, -a.box[1]);
      case 3: return make_double4(0.0, -1.0, 0.0, a.box[4]);
      case 4: return make_double4(0.0, 0.0, 1.0, -a.box[2]);
      default: return make_double4(0.0, 0.0, -1.0, a.box[5]);
    }
  }
  const double4 pj = a.xd[own];
  return make_double4(2.0 * __dsub_rn(pi.x, pj.x), 2.0 * __dsub_rn(pi.y, pj.y),
                      2.0 * __dsub_rn(pi.z, pj.z), __dsub_rn(qi, a.q[own]));
}

__global__ void __launch_bounds__(64) restrict_kernel(RestrictArgs a) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double* p = a.xyz + 3 * (size_t)i;
  const double wi = a.w ? a.w[i] : 0.0;
  const uint32_t s = a.slot_of[i];
  // bounding box of the cell: its corners, or the whole box for a cell of
  // the unbounded path (no stored polytope)
  double lo[3] = {a.box[0], a.box[1], a.box[2]}, hi[3] = {a.box[3], a.box[4], a.box[5]};
  if (!(a.nf[s] & kHugeFacets)) {
    const ulonglong2 tm = a.cb.tmask[s];
    const size_t tb = (size_t)s * kTMax, pb = (size_t)s * kPMax;
    const double4 pis = a.xd[s];
    const double qis = a.q[s];
    lo[0] = lo[1] = lo[2] = DBL_MAX;
    hi[0] = hi[1] = hi[2] = -DBL_MAX;
    bool none = true;
    for (int h = 0; h < 2; ++h) {
      uint64_t wbits = h ? tm.y : tm.x;
      while (wbits) {
        const int t = 64 * h + __ffsll((long long)wbits) - 1;
        wbits &= wbits - 1;
        const uint32_t v = a.cb.tv[tb + t];
        const double3 c = r_corner(restrict_plane(a, a.cb.pown[pb + (v & 0xFF)], pis, qis),
                                   restrict_plane(a, a.cb.pown[pb + (v >> 8 & 0xFF)], pis, qis),
                                   restrict_plane(a, a.cb.pown[pb + (v >> 16 & 0xFF)], pis, qis));
        lo[0] = fmin(lo[0], c.x); hi[0] = fmax(hi[0], c.x);
        lo[1] = fmin(lo[1], c.y); hi[1] = fmax(hi[1], c.y);
        lo[2] = fmin(lo[2], c.z); hi[2] = fmax(hi[2], c.z);
        none = false;
      }
    }
    if (none) {  // empty cell
      a.m[i] = 0.0;
      a.mg[3 * (size_t)i] = a.mg[3 * (size_t)i + 1] = a.mg[3 * (size_t)i + 2] = 0.0;
      a.g[3 * (size_t)i] = a.g[3 * (size_t)i + 1] = a.g[3 * (size_t)i + 2] = 0.0;
      a.F[i] = 0.0;
      return;
    }
    const double pad = 1e-9 * (1.0 + fabs(a.box[3] - a.box[0]));
    for (int k = 0; k < 3; ++k) {
      lo[k] -= pad;
      hi[k] += pad;
    }
  }
  int b0[3], b1[3];
  for (int k = 0; k < 3; ++k) {
    b0[k] = bin_of(lo[k], a.bin_lo[k], a.bin_h[k], a.G);
    b1[k] = bin_of(hi[k], a.bin_lo[k], a.bin_h[k], a.G);
  }
  const uint32_t r0 = a.rowptr[i], r1 = a.rowptr[i + 1];
  double m = 0.0, F = 0.0;
  double3 mg = make_double3(0.0, 0.0, 0.0), gv = make_double3(0.0, 0.0, 0.0);
  bool overflow = false;
  Piece P;
  for (int bz = b0[2]; bz <= b1[2]; ++bz)
    for (int by = b0[1]; by <= b1[1]; ++by)
      for (int bx = b0[0]; bx <= b1[0]; ++bx) {
        const uint32_t bin = ((uint32_t)bz * a.G + by) * a.G + bx;
        for (uint32_t e = a.bin_start[bin]; e < a.bin_start[bin + 1]; ++e) {
          const uint32_t t = a.bin_tets[e];
          const uint32_t* tv = a.tets + 4 * (size_t)t;
          double3 c[4];
          double tl[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, th[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
          for (int k = 0; k < 4; ++k) {
            const double* vv = a.mv + 3 * (size_t)tv[k];
            c[k] = make_double3(vv[0], vv[1], vv[2]);
            for (int d = 0; d < 3; ++d) {
              tl[d] = fmin(tl[d], vv[d]);
              th[d] = fmax(th[d], vv[d]);
            }
          }
          // the first bin the tetrahedron shares with the cell takes it
          int first[3];
          bool overlap = true;
          for (int d = 0; d < 3; ++d) {
            first[d] = max(bin_of(tl[d], a.bin_lo[d], a.bin_h[d], a.G), b0[d]);
            overlap = overlap && tl[d] <= hi[d] && th[d] >= lo[d];
          }
          if (!overlap || first[0] != bx || first[1] != by || first[2] != bz) continue;
          tet_piece(P, c[0], c[1], c[2], c[3]);
          bool alive = true;
          for (uint32_t r = r0; r < r1 && alive; ++r) {
            const uint32_t j = a.nbr[r];
            double3 nrm;
            double cc;
            bisector(p, wi, a.xyz + 3 * (size_t)j, a.w ? a.w[j] : 0.0, nrm, cc);
            alive = clip_piece(P, nrm, cc, &overflow);
          }
          if (overflow) break;
          if (alive) integrate_piece(P, p, a.bmask[t], m, mg, F, gv);
        }
        if (overflow) break;
      }
  if (overflow) atomicAdd(&a.err[0], 1u);
  a.m[i] = m;
  a.mg[3 * (size_t)i] = mg.x;
  a.mg[3 * (size_t)i + 1] = mg.y;
  a.mg[3 * (size_t)i + 2] = mg.z;
  a.F[i] = F;
  a.g[3 * (size_t)i] = gv.x;
  a.g[3 * (size_t)i + 1] = gv.y;
  a.g[3 * (size_t)i + 2] = gv.z;
}

// ---- bins of tetrahedra
__global__ void orient_tets_kernel(const double* __restrict__ mv, const uint32_t* __restrict__ in,
                                   uint32_t nt, uint32_t nv, uint32_t* __restrict__ out,
                                   uint32_t* __restrict__ err) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  uint32_t v[4];
  for (int k = 0; k < 4; ++k) {
    v[k] = in[4 * (size_t)t + k];
    if (v[k] >= nv) {
      atomicAdd(&err[1], 1u);
      v[k] = 0;
    }
  }
  const double* A = mv + 3 * (size_t)v[0];
  const double* B = mv + 3 * (size_t)v[1];
  const double* C = mv + 3 * (size_t)v[2];
  const double* D = mv + 3 * (size_t)v[3];
  const double ux = B[0] - A[0], uy = B[1] - A[1], uz = B[2] - A[2];
  const double vx = C[0] - A[0], vy = C[1] - A[1], vz = C[2] - A[2];
  const double wx = D[0] - A[0], wy = D[1] - A[1], wz = D[2] - A[2];
  const double det = ux * (vy * wz - vz * wy) - uy * (vx * wz - vz * wx) + uz * (vx * wy - vy * wx);
  if (det < 0.0) {
    const uint32_t tmp = v[1];
    v[1] = v[2];
    v[2] = tmp;
  }
  for (int k = 0; k < 4; ++k) out[4 * (size_t)t + k] = v[k];
}

template <bool FILL>
__global__ void bin_tets_kernel(const double* __restrict__ mv, const uint32_t* __restrict__ tets,
                                uint32_t nt, RestrictArgs a, uint32_t* __restrict__ count,
                                uint32_t* __restrict__ cursor, uint32_t* __restrict__ list) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  double tl[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, th[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int k = 0; k < 4; ++k) {
    const double* vv = mv + 3 * (size_t)tets[4 * (size_t)t + k];
    for (int d = 0; d < 3; ++d) {
      tl[d] = fmin(tl[d], vv[d]);
      th[d] = fmax(th[d], vv[d]);
    }
  }
  int b0[3], b1[3];
  for (int d = 0; d < 3; ++d) {
    b0[d] = bin_of(tl[d], a.bin_lo[d], a.bin_h[d], a.G);
    b1[d] = bin_of(th[d], a.bin_lo[d], a.bin_h[d], a.G);
  }
  for (int bz = b0[2]; bz <= b1[2]; ++bz)
    for (int by = b0[1]; by <= b1[1]; ++by)
      for (int bx = b0[0]; bx <= b1[0]; ++bx) {
        const uint32_t bin = ((uint32_t)bz * a.G + by) * a.G + bx;
        if (FILL) list[atomicAdd(&cursor[bin], 1u)] = t;
        else atomicAdd(&count[bin], 1u);
      }
}

// each bin's list in ascending order (the fill order depends on atomics)
__global__ void sort_bins_kernel(const uint32_t* __restrict__ start, uint32_t nbins,
                                 uint32_t* __restrict__ list) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const uint32_t lo = start[b], hi = start[b + 1];
  for (uint32_t i = lo + 1; i < hi; ++i) {
    const uint32_t v = list[i];
    uint32_t j = i;
    while (j > lo && list[j - 1] > v) {
      list[j] = list[j - 1];
      --j;
    }
    list[j] = v;
  }
}

// Bit k of bmask[t]: face k of tetrahedron t is on the mesh's boundary (no
// other tetrahedron has its three vertices).  Both tetrahedra of an inner
// face are listed in the bin of the face's centroid.
__global__ void tet_boundary_kernel(const double* __restrict__ mv,
                                    const uint32_t* __restrict__ tets, uint32_t nt, RestrictArgs a,
                                    uint8_t* __restrict__ bmask) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  uint8_t mask = 0;
  for (int k = 0; k < 4; ++k) {
    uint32_t fvx[3];
    double cen[3] = {0.0, 0.0, 0.0};
    for (int e = 0; e < 3; ++e) {
      fvx[e] = tets[4 * (size_t)t + kTetFace[k][e]];
      for (int d = 0; d < 3; ++d) cen[d] += mv[3 * (size_t)fvx[e] + d] / 3.0;
    }
    const uint32_t bin = ((uint32_t)bin_of(cen[2], a.bin_lo[2], a.bin_h[2], a.G) * a.G +
                          bin_of(cen[1], a.bin_lo[1], a.bin_h[1], a.G)) * a.G +
                         bin_of(cen[0], a.bin_lo[0], a.bin_h[0], a.G);
    bool shared = false;
    for (uint32_t e = a.bin_start[bin]; e < a.bin_start[bin + 1] && !shared; ++e) {
      const uint32_t u = a.bin_tets[e];
      if (u == t) continue;
      int hits = 0;
      for (int q = 0; q < 4; ++q) {
        const uint32_t vu = tets[4 * (size_t)u + q];
        hits += (vu == fvx[0]) + (vu == fvx[1]) + (vu == fvx[2]);
      }
      shared = hits == 3;
    }
    if (!shared) mask |= (uint8_t)(1u << k);
  }
  bmask[t] = mask;
}

}  // namespace

// The cells of the seeds restricted to the mesh (host arrays); cells first
// computed with `cells` (the orchestration of gbv_api.cu) on the box given.
void restricted_cells(gbv_context* c, const double* d_xyz, const double* d_w, uint32_t n,
                      const double* d_mv, uint32_t nv, const uint32_t* d_tets_in, uint32_t nt,
                      cudaStream_t st, double* d_m, double* d_mg, double* d_F, double* d_g) {
  RestrictArgs a{};
  a.n = n;
  a.xyz = d_xyz;
  a.w = d_w;
  a.rowptr = c->rowptr;
  a.nbr = c->nbr;
  a.slot_of = c->S.slot_of;
  a.nf = c->buf<uint32_t>("nf", n);
  a.cb.tv = c->buf<uint32_t>("cb_tv", (size_t)kTMax * n);
  a.cb.ta = c->buf<uint32_t>("cb_ta", (size_t)kTMax * n);
  a.cb.key = c->buf<int16_t>("cb_key", (size_t)kTMax * n);
  a.cb.pown = c->buf<uint32_t>("cb_pown", (size_t)kPMax * n);
  a.cb.prank = c->buf<uint16_t>("cb_prank", (size_t)kPMax * n);
  a.cb.tmask = c->buf<ulonglong2>("cb_tmask", n);
  a.cb.pmask = c->buf<uint64_t>("cb_pmask", n);
  a.cb.flags = c->buf<uint32_t>("cb_flags", n);
  a.xd = c->S.xd;
  a.q = c->S.q;
  for (int k = 0; k < 6; ++k) a.box[k] = c->box[k];
  a.mv = d_mv;
  a.nt = nt;
  uint32_t* err = c->buf<uint32_t>("rv_err", 2);
  GBV_CUDA(cudaMemsetAsync(err, 0, 2 * sizeof(uint32_t), st));
  a.err = err;
  uint32_t* tets = c->buf<uint32_t>("rv_tets", 4 * (size_t)nt);
  const unsigned ntb = (nt + 127) / 128;
  orient_tets_kernel<<<ntb, 128, 0, st>>>(d_mv, d_tets_in, nt, nv, tets, err); count_launch();
  a.tets = tets;
  int G = (int)std::cbrt((double)nt / 2.0);
  G = std::max(1, std::min(G, 64));
  a.G = G;
  for (int k = 0; k < 3; ++k) {
    a.bin_lo[k] = c->box[k];
    a.bin_h[k] = (c->box[3 + k] - c->box[k]) / G * (1.0 + 1e-12);
  }
  const uint32_t nbins = (uint32_t)(G * G * G);
  uint32_t* start = c->buf<uint32_t>("rv_bin_start", (size_t)nbins + 1);
  uint32_t* cursor = c->buf<uint32_t>("rv_bin_cursor", nbins);
  GBV_CUDA(cudaMemsetAsync(start, 0, sizeof(uint32_t) * ((size_t)nbins + 1), st));
  bin_tets_kernel<false><<<ntb, 128, 0, st>>>(d_mv, tets, nt, a, start, nullptr, nullptr); count_launch();
  uint32_t* tmp = c->buf<uint32_t>("rv_scan", scan_tmp_elems((size_t)nbins + 1));
  exclusive_scan_u32(start, (size_t)nbins + 1, tmp, st);
  GBV_CUDA(cudaMemcpyAsync(cursor, start, sizeof(uint32_t) * nbins, cudaMemcpyDeviceToDevice, st));
  uint32_t total = 0;
  GBV_CUDA(cudaMemcpyAsync(&total, start + nbins, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GBV_CUDA(cudaStreamSynchronize(st));
  uint32_t* list = c->buf<uint32_t>("rv_bin_tets", std::max<uint32_t>(total, 1));
  bin_tets_kernel<true><<<ntb, 128, 0, st>>>(d_mv, tets, nt, a, nullptr, cursor, list); count_launch();
  sort_bins_kernel<<<(nbins + 127) / 128, 128, 0, st>>>(start, nbins, list); count_launch();
  a.bin_start = start;
  a.bin_tets = list;
  uint8_t* bmask = c->buf<uint8_t>("rv_bmask", nt);
  tet_boundary_kernel<<<ntb, 128, 0, st>>>(d_mv, tets, nt, a, bmask); count_launch();
  a.bmask = bmask;
  a.m = d_m;
  a.mg = d_mg;
  a.F = d_F;
  a.g = d_g;
  restrict_kernel<<<(n + 63) / 64, 64, 0, st>>>(a); count_launch();
  uint32_t h_err[2] = {0, 0};
  GBV_CUDA(cudaMemcpyAsync(h_err, err, sizeof h_err, cudaMemcpyDeviceToHost, st));
  GBV_CUDA(cudaStreamSynchronize(st));
  GBV_CUDA(cudaGetLastError());
  if (h_err[1])
    throw StatusError{GBV_ERR_INVALID_ARGUMENT, std::to_string(h_err[1]) +
                                                    " tetrahedron vertex index(es) out of range"};
  if (h_err[0])
    throw StatusError{GBV_ERR_CAPACITY, std::to_string(h_err[0]) +
                                            " cell piece(s) beyond the clipper's " +
                                            std::to_string(kRvMaxV) + " vertices"};
}

}  // namespace gbv
