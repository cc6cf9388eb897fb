// Cells beyond the capacity of the clipping kernels (more than 128 corners
// or 64 live planes): one single-thread block per cell, the polytope in global memory
// with room for kHugeT corners and kHugeV planes, FP64 with exact conflict
// signs, and the reference's own list discipline, so that the results are
// those of the other paths (and of the reference) bit for bit.
//
// The reference's VBW::ConvexCell grows its arrays without bound
// (voronoi/convex_cell.cpp:1086-1101).  Such cells are rare -- seeds at
// the edge of dense clusters whose cells face hundreds of cluster cells --
// but they do occur in clustered inputs and in the first iterations of
// optimal transport, where the other paths would stop with a capacity
// error.
//
// The cell is the dual polytope of ConvexCell (voronoi/convex_cell.h:
// 1350-1433): planes are vertices, corners are triangles with their three
// adjacent triangles, and the valid triangles form a singly linked list
// through the fourth 16-bit field.  Clipping (clip_by_plane,
// convex_cell.cpp:467-516) walks the list, moves the triangles in conflict
// to a conflict list and relinks the others in reverse order; the border of
// the conflict zone is fanned from the last border edge met
// (triangulate_conflict_zone, convex_cell.cpp:761-865); freed triangles
// are reused first (new_triangle, convex_cell.h:1143-1166).  Corners,
// radii, volumes, centroids and facet areas use the reference's FP64
// formulas operation for operation (gbv_refgeom.cuh), and compute_mg and
// facet_area walk the same fans in the same order (convex_cell.cpp:
// 1160-1191, 1215-1253), so every output is the reference's.
//
// A plane that cuts nothing takes no slot here (the reference stores it
// and never uses it); slots keep clipping order, which is the order in
// which facets are reported, so nothing observable changes.
#include "gbv_clip.cuh"
#include "gbv_corner.cuh"
#include "gbv_exact.cuh"
#include "gbv_refgeom.cuh"

namespace gbv {

namespace {

constexpr uint16_t kEnd = 16383;     // END_OF_LIST of the 14-bit links
constexpr uint16_t kConf = 32768;    // link flag: the triangle is in conflict

struct HugeCell {
  ushort4* t;     // plane slots i, j, k and the list link
  ushort4* adj;   // adjacent triangles across the edges opposite i, j, k
  double4* cor;   // corner (x, y, z) and its squared distance to the seed
  float* eps;     // error bound of the corner (cramer_bound)
  double4* pl;    // plane equations
  uint32_t* vg;   // plane slot -> neighbour slot (kNone for the box)
  uint16_t* v2t;
  uint8_t* v2e;
  int nb_t, nb_v, first_free, first_valid;
  bool full;
  unsigned long long tests, nodes, seeds;  // work counters
};

__device__ __forceinline__ int vtx(const ushort4& t, int lv) {
  return lv == 0 ? t.x : (lv == 1 ? t.y : t.z);
}
__device__ __forceinline__ int adj_of(const ushort4& a, int le) {
  return le == 0 ? a.x : (le == 1 ? a.y : a.z);
}
__device__ __forceinline__ void set_adj(ushort4& a, int le, int v) {
  if (le == 0) a.x = (uint16_t)v;
  else if (le == 1) a.y = (uint16_t)v;
  else a.z = (uint16_t)v;
}
__device__ __forceinline__ int find_vtx(const ushort4& t, int v) {
  return (t.y == v) + 2 * (t.z == v);
}

__device__ __forceinline__ void set_corner(HugeCell& C, int t, const double4& pi) {
  const ushort4 tv = C.t[t];
  double x, y, z;
  float e;
  corner_fp64(C.pl[tv.x], C.pl[tv.y], C.pl[tv.z], x, y, z, e);
  C.cor[t] = make_double4(x, y, z, r_sqdist(pi.x, pi.y, pi.z, make_double3(x, y, z)));
  C.eps[t] = e;
}

// new_triangle: the most recently freed slot first, pushed at the head of
// the valid list.  Returns -1 when the capacity is exhausted.
__device__ int new_triangle(HugeCell& C, int i, int j, int k) {
  int r = C.first_free;
  if (r == kEnd) {
    if (C.nb_t >= (int)kHugeT) {
      C.full = true;
      return -1;
    }
    r = C.nb_t++;
  } else {
    C.first_free = C.t[r].w & ~kConf;
  }
  C.t[r] = make_ushort4((uint16_t)i, (uint16_t)j, (uint16_t)k, (uint16_t)C.first_valid);
  C.first_valid = r;
  return r;
}

__device__ void init_box(HugeCell& C, const double* box, const double4& pi) {
  C.nb_t = 0;
  C.first_free = kEnd;
  C.first_valid = kEnd;
  C.full = false;
  C.pl[0] = make_double4(0.0, 0.0, 0.0, 0.0);
  C.pl[1] = make_double4(1.0, 0.0, 0.0, -box[0]);
  C.pl[2] = make_double4(-1.0, 0.0, 0.0, box[3]);
  C.pl[3] = make_double4(0.0, 1.0, 0.0, -box[1]);
  C.pl[4] = make_double4(0.0, -1.0, 0.0, box[4]);
  C.pl[5] = make_double4(0.0, 0.0, 1.0, -box[2]);
  C.pl[6] = make_double4(0.0, 0.0, -1.0, box[5]);
  for (int v = 0; v < 7; ++v) C.vg[v] = kNone;
  C.nb_v = 7;
  // the 8 box corners as triangles of face planes, with their adjacency
  const uint16_t tri[8][6] = {{3, 6, 1, 1, 4, 2}, {6, 4, 1, 5, 0, 3}, {2, 6, 3, 0, 6, 3},
                              {6, 2, 4, 7, 1, 2}, {5, 3, 1, 0, 5, 6}, {5, 1, 4, 1, 7, 4},
                              {3, 5, 2, 7, 2, 4}, {5, 4, 2, 3, 6, 5}};
  for (int q = 0; q < 8; ++q) {
    const int r = new_triangle(C, tri[q][0], tri[q][1], tri[q][2]);
    C.adj[r] = make_ushort4(tri[q][3], tri[q][4], tri[q][5], 0);
    set_corner(C, r, pi);
  }
}

// Conflict of triangle t with plane P: det [P_i; P_j; P_k; P] >= 0, exact.
// Decided, as in the clipping kernels, from the cached corner c: the sign
// of P . (c, 1) when it exceeds the corner's error bound, else exactly.
// With the fast predicates, tests near the bound are decided by the
// reference's FP64 det4x4 instead (conflict iff > 0).
__device__ __forceinline__ bool in_conflict(const HugeCell& C, int t, const double4& P,
                                            double pa1, double bw, bool fast,
                                            unsigned long long& n_exact) {
  const double4 c = C.cor[t];
  const double sv = fma(P.z, c.z, fma(P.y, c.y, fma(P.x, c.x, P.w)));
  const double bound = fma(pa1, (double)C.eps[t], bw) * (fast ? kFastPredWide : 1.0);
  if (sv < -bound) return true;
  if (sv > bound) return false;
  const ushort4 tv = C.t[t];
  const double4 a = C.pl[tv.x], b = C.pl[tv.y], d = C.pl[tv.z];
  ++n_exact;
  if (fast) return r_det4x4(a, b, d, P) > 0.0;
  const double r0[4] = {a.x, a.y, a.z, a.w}, r1[4] = {b.x, b.y, b.z, b.w},
               r2[4] = {d.x, d.y, d.z, d.w}, r3[4] = {P.x, P.y, P.z, P.w};
  return det4_sign_exact(r0, r1, r2, r3) >= 0;
}

// clip_by_plane.  Returns false when a capacity is exhausted.  R2 receives
// the squared radius of the clipped cell (max over its corners).
__device__ bool clip(HugeCell& C, const double4& P, uint32_t j, const double4& pi, double& R2,
                     bool fast, unsigned long long& n_exact) {
  int head = kEnd, tail = kEnd;
  int t = C.first_valid;
  C.first_valid = kEnd;
  double keep = 0.0;
  const double pa1 = (fabs(P.x) + fabs(P.y) + fabs(P.z)) * 1.0001;
  const double bw = Consts<double>::kDot * fabs(P.w) * 1.0001;
  while (t != kEnd) {
    const int next = C.t[t].w;
    ++C.tests;
    if (in_conflict(C, t, P, pa1, bw, fast, n_exact)) {
      C.t[t].w = (uint16_t)(head | kConf);
      head = t;
      if (tail == kEnd) tail = t;
    } else {
      C.t[t].w = (uint16_t)C.first_valid;
      C.first_valid = t;
      keep = fmax(keep, C.cor[t].w);
    }
    t = next;
  }
  R2 = keep;
  if (head == kEnd) return true;  // nothing cut: no plane slot needed
  if (C.nb_v >= (int)kHugeV) {
    C.full = true;
    return false;
  }
  const int lv = C.nb_v++;
  C.pl[lv] = P;
  C.vg[lv] = j;
  // border of the conflict zone; the walk starts at the last border edge met
  int first_v = kEnd;
  for (int u = C.first_valid; u != kEnd; u = C.t[u].w) {
    const ushort4 a = C.adj[u];
    const ushort4 tv = C.t[u];
    if (C.t[a.x].w & kConf) {
      first_v = tv.y;
      C.v2t[first_v] = (uint16_t)u;
      C.v2e[first_v] = 0;
    }
    if (C.t[a.y].w & kConf) {
      first_v = tv.z;
      C.v2t[first_v] = (uint16_t)u;
      C.v2e[first_v] = 1;
    }
    if (C.t[a.z].w & kConf) {
      first_v = tv.x;
      C.v2t[first_v] = (uint16_t)u;
      C.v2e[first_v] = 2;
    }
  }
  if (first_v != kEnd) {
    int v = first_v, prev_new = -1, first_new = -1;
    int guard = 0;
    do {
      const int tt = C.v2t[v], e = C.v2e[v];
      const int v2 = vtx(C.t[tt], (e + 2) % 3);
      const int nt = new_triangle(C, lv, v2, v);
      if (nt < 0) return false;
      C.adj[nt] = make_ushort4((uint16_t)tt, 0, 0, 0);
      set_adj(C.adj[tt], e, nt);
      if (prev_new == -1) {
        first_new = nt;
      } else {
        set_adj(C.adj[prev_new], 2, nt);
        set_adj(C.adj[nt], 1, prev_new);
      }
      set_corner(C, nt, pi);
      R2 = fmax(R2, C.cor[nt].w);
      prev_new = nt;
      v = v2;
      if (++guard > (int)kHugeT) {  // not a simple cycle
        C.full = true;
        return false;
      }
    } while (v != first_v);
    set_adj(C.adj[prev_new], 2, first_new);
    set_adj(C.adj[first_new], 1, prev_new);
  }
  C.t[tail].w = (uint16_t)C.first_free;
  C.first_free = head;
  return true;
}

// Certification as in the geometry kernel (FP32 with the same margins),
// one corner at a time: for every corner, a best-bound octree search for
// the seed of least power at the corner among those below the seed's own
// power there and not in the candidate list; the distinct ones are the
// extra candidates.
__device__ void certify(const HugeArgs& a, HugeCell& C, uint32_t s, uint32_t row,
                        const double4& pi, double wi) {
  const SortedSeeds& S = a.S;
  const GridDesc& gd = *S.gd;
  const float hf = gd.h_f;
  const uint32_t ncand = a.nbr_cnt[row] & kCntMask;
  uint32_t found = 0;
  bool more = false;
  uint32_t stk[96];
  for (int t = C.first_valid; t != kEnd; t = C.t[t].w) {
    const double4 cd = C.cor[t];
    const float cx = (float)cd.x, cy = (float)cd.y, cz = (float)cd.z;
    const float rho = (float)(cd.w - wi);
    float best = rho + 1e-5f * fabsf(rho) + 1e-7f;
    uint32_t bj = kNone;
    int sp = 0;
    stk[sp++] = 0u;
    while (sp > 0) {
      const uint32_t e = stk[--sp];
      const int lev = (int)(e & 15u);
      const uint32_t code = e >> 4;
      const int shift = gd.L - lev;
      const uint32_t b = S.cell_start[code << (3 * shift)];
      const uint32_t en = S.cell_start[(code + 1u) << (3 * shift)];
      if (b == en) continue;
      ++C.nodes;
      const float WB = (float)a.node_wmax[node_offset(lev) + code];
      const float side = hf * (float)(1u << shift);
      const float bx = gd.lo_f[0] + (float)compact3(code) * side;
      const float by = gd.lo_f[1] + (float)compact3(code >> 1) * side;
      const float bz = gd.lo_f[2] + (float)compact3(code >> 2) * side;
      const float pad = 1e-6f * (1.f + fabsf(bx) + fabsf(by) + fabsf(bz)) + 1e-5f * side;
      const float dx = fmaxf(fmaxf(bx - pad - cx, cx - (bx + side + pad)), 0.f);
      const float dy = fmaxf(fmaxf(by - pad - cy, cy - (by + side + pad)), 0.f);
      const float dz = fmaxf(fmaxf(bz - pad - cz, cz - (bz + side + pad)), 0.f);
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 >= (best + WB) + 1e-5f * (fabsf(best) + fabsf(WB) + d2) + 1e-7f) continue;
      if (a.node_lin) {
        const double4 l = a.node_lin[node_offset(lev) + code];
        if (linear_bound_clears(cx, cy, cz, best, bx, by, bz, side, pad,
                                make_float4((float)l.x, (float)l.y, (float)l.z, (float)l.w),
                                (float)a.node_ex[node_offset(lev) + code]))
          continue;
      }
      if (en - b <= 32u || lev == gd.L) {
        C.seeds += en - b;
        for (uint32_t jn = b; jn < en; ++jn) {
          if (jn == s) continue;
          const double4 pj = S.xd[jn];
          if (pj.x == pi.x && pj.y == pi.y && pj.z == pi.z) continue;
          const float wj = S.ws ? (float)S.ws[jn] : 0.f;
          const float ex = cx - (float)pj.x, ey = cy - (float)pj.y, ez = cz - (float)pj.z;
          const float d = ex * ex + ey * ey + ez * ez - wj;
          // ties with the current best go to the lower original index, so
          // that the result does not depend on the order of the slots
          if (!(d < best || (d == best && bj != kNone && S.perm[jn] < S.perm[bj]))) continue;
          bool member = false;
          for (uint32_t k = 0; k < ncand && !member; ++k)
            member = a.nbr[(size_t)k * a.nbr_stride + row] == jn;
          if (member) continue;
          best = d;
          bj = jn;
        }
        continue;
      }
      if (sp + 8 > 96) {
        more = true;
        break;
      }
      // children by their lower bound on the power at c, the most promising
      // popped first; children that cannot improve are not pushed
      float lb[8];
      int ord[8], nk = 0;
      const float cs = 0.5f * side;
      for (int ch = 0; ch < 8; ++ch) {
        const uint32_t cc = (code << 3) | (uint32_t)ch;
        const int csh = shift - 1;
        if (S.cell_start[cc << (3 * csh)] == S.cell_start[(cc + 1u) << (3 * csh)]) continue;
        const float qx = bx + (float)(ch & 1) * cs, qy = by + (float)((ch >> 1) & 1) * cs,
                    qz = bz + (float)((ch >> 2) & 1) * cs;
        const float ex = fmaxf(fmaxf(qx - pad - cx, cx - (qx + cs + pad)), 0.f);
        const float ey = fmaxf(fmaxf(qy - pad - cy, cy - (qy + cs + pad)), 0.f);
        const float ez = fmaxf(fmaxf(qz - pad - cz, cz - (qz + cs + pad)), 0.f);
        const float v = ex * ex + ey * ey + ez * ez -
                        (float)a.node_wmax[node_offset(lev + 1) + cc];
        int q = nk++;
        while (q > 0 && lb[q - 1] < v) {  // descending: the smallest is pushed last
          lb[q] = lb[q - 1];
          ord[q] = ord[q - 1];
          --q;
        }
        lb[q] = v;
        ord[q] = ch;
      }
      for (int k = 0; k < nk; ++k)
        stk[sp++] = (((code << 3) | (uint32_t)ord[k]) << 4) | (uint32_t)(lev + 1);
    }
    if (bj == kNone) continue;
    bool dup = false;
    for (uint32_t k = 0; k < found && k < a.max_extra && !dup; ++k)
      dup = a.extra[(size_t)k * a.nbr_stride + row] == bj;
    if (dup) continue;
    if (found < a.max_extra) a.extra[(size_t)found * a.nbr_stride + row] = bj;
    else more = true;
    ++found;
  }
  a.extra_cnt[row] = (found < a.max_extra ? found : a.max_extra) | (more ? 0x80000000u : 0u);
}

// One cell per block of one thread: cells walk different lists, and the
// threads of a warp would run their divergent walks one after the other.
__global__ void __launch_bounds__(1) huge_kernel(HugeArgs a) {
  const uint32_t qi = blockIdx.x;
  if (qi >= a.nq) return;
  const SortedSeeds& S = a.S;
  const uint32_t s = a.qlist[qi];
  const uint32_t row = a.qrow ? a.qrow[qi] : qi;
  HugeCell C;
  C.t = a.scr_t + (size_t)qi * kHugeT;
  C.adj = a.scr_adj + (size_t)qi * kHugeT;
  C.cor = a.scr_cor + (size_t)qi * kHugeT;
  C.eps = a.scr_eps + (size_t)qi * kHugeT;
  C.pl = a.scr_pl + (size_t)qi * kHugeV;
  C.vg = a.scr_vg + (size_t)qi * kHugeV;
  C.v2t = a.scr_v2t + (size_t)qi * kHugeV;
  C.v2e = a.scr_v2e + (size_t)qi * kHugeV;
  const double4 pi = S.xd[s];
  const double qi_ = S.q[s];
  const double hi2 = __dmul_rn(pi.w, pi.w);
  C.tests = C.nodes = C.seeds = 0;
  const long long c0 = clock64();
  init_box(C, a.box, pi);
  double R2 = 0.0;
  for (int t = C.first_valid; t != kEnd; t = C.t[t].w) R2 = fmax(R2, C.cor[t].w);

  const uint32_t cnt_raw = a.nbr_cnt[row];
  const bool dup = (cnt_raw >> 31) != 0;
  const uint32_t copies = (cnt_raw >> 24) & 0x7Fu;
  const uint32_t cap = copies ? reference_list_cap(a.k0, a.n_total, copies, a.check_sr != 0)
                              : 0xFFFFFFFFu;
  const uint32_t cnt = dup ? 0u : min(cnt_raw & kCntMask, cap);
  int32_t st = -1;
  uint32_t jj = 0;
  unsigned long long n_exact = 0;
  if (dup) {
    st = CELL_DUPLICATE;
  } else {
    for (; jj < cnt; ++jj) {
      const uint32_t j = a.nbr[(size_t)jj * a.nbr_stride + row];
      const double4 pj = S.xd[j];
      if (a.check_sr) {
        const double dij = dist2_exact(pi, pj);
        if (dij > __dmul_rn(4.1, __dadd_rn(R2, hi2))) {
          st = CELL_CERTIFIED;
          break;
        }
      }
      const double4 P = make_double4(2.0 * __dsub_rn(pi.x, pj.x), 2.0 * __dsub_rn(pi.y, pj.y),
                                     2.0 * __dsub_rn(pi.z, pj.z), __dsub_rn(qi_, S.q[j]));
      if (!clip(C, P, j, pi, R2, a.fast_pred != 0, n_exact)) {
        st = CELL_OVERFLOW;
        break;
      }
    }
    if (st < 0) {
      const bool complete = ((cnt_raw & kCntMask) < a.list_k) || (a.list_k >= a.n_total - 1);
      if (!a.check_sr) st = CELL_CERTIFIED;
      else if (copies && cnt == cap) st = (cap == 0) ? CELL_DUPLICATE : CELL_STALLED;
      else st = complete ? CELL_ALL_NEIGHBOURS : CELL_NEED_MORE_K;
    }
  }
  if (a.counters) {
    if (n_exact) atomicAdd(&a.counters[0], n_exact);
    atomicMax(&a.counters[1], (unsigned long long)jj);
  }
  a.status[s] = st;
  a.nclip[s] = jj;
  const long long c1 = clock64();
  if (a.stats) {
    unsigned long long* o = a.stats + (size_t)qi * kHugeStats;
    o[0] = (unsigned long long)(c1 - c0);
    o[3] = jj;
    o[4] = C.tests;
    o[5] = (unsigned long long)C.nb_t;
    o[6] = (unsigned long long)C.nb_v;
  }
  if (st == CELL_OVERFLOW || st == CELL_NEED_MORE_K) return;

  // ---- geometry: compute_geometry, compute_mg, facet_area
  for (int v = 0; v < C.nb_v; ++v) C.v2t[v] = kEnd;
  for (int t = C.first_valid; t != kEnd; t = C.t[t].w) {
    const ushort4 tv = C.t[t];
    C.v2t[tv.x] = (uint16_t)t;
    C.v2t[tv.y] = (uint16_t)t;
    C.v2t[tv.z] = (uint16_t)t;
  }
  auto P3 = [&](int t) {
    const double4 c = C.cor[t];
    return make_double3(c.x, c.y, c.z);
  };
  double m = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
  int t_origin = kEnd;
  bool bad = false;
  for (int v = 0; v < C.nb_v && !bad; ++v) {
    if (C.v2t[v] == kEnd) continue;
    if (t_origin == kEnd) {
      t_origin = C.v2t[v];
      continue;
    }
    int t1 = 0, t2 = 0, cur = 0, guard = 0;
    int t = C.v2t[v];
    const double3 p = P3(t_origin);
    do {
      if (cur == 0) t1 = t;
      else if (cur == 1) t2 = t;
      else {
        const double3 q = P3(t1), r = P3(t2), w = P3(t);
        const double cm = r_tet_volume(p, q, r, w);
        m = __dadd_rn(m, cm);
        gx = __dadd_rn(gx, __ddiv_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(p.x, q.x), r.x), w.x)), 4.0));
        gy = __dadd_rn(gy, __ddiv_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(p.y, q.y), r.y), w.y)), 4.0));
        gz = __dadd_rn(gz, __ddiv_rn(__dmul_rn(cm, __dadd_rn(__dadd_rn(__dadd_rn(p.z, q.z), r.z), w.z)), 4.0));
        t2 = t;
      }
      ++cur;
      const int lv = find_vtx(C.t[t], v);
      t = adj_of(C.adj[t], (lv + 1) % 3);
      if (++guard > (int)kHugeT) bad = true;
    } while (t != C.v2t[v] && !bad);
  }
  uint32_t* fn = a.fac_nbr + (size_t)qi * kHugeV;
  double* fa = a.fac_area + (size_t)qi * kHugeV;
  uint32_t nfac = 0;
  for (int v = 1; v < C.nb_v && !bad; ++v) {
    if (C.v2t[v] == kEnd || C.vg[v] == kNone) continue;
    double area = 0.0;
    int t1 = 0, t2 = 0, cur = 0, guard = 0;
    int t = C.v2t[v];
    do {
      if (cur == 0) t1 = t;
      else if (cur == 1) t2 = t;
      else {
        area = __dadd_rn(area, r_triangle_area(P3(t1), P3(t2), P3(t)));
        t2 = t;
      }
      ++cur;
      const int lv = find_vtx(C.t[t], v);
      t = adj_of(C.adj[t], (lv + 1) % 3);
      if (++guard > (int)kHugeT) bad = true;
    } while (t != C.v2t[v] && !bad);
    fn[nfac] = S.perm[C.vg[v]];
    fa[nfac] = area;
    ++nfac;
  }
  if (bad) {
    a.status[s] = CELL_ERROR;
    return;
  }
  a.vol[s] = m;
  a.mg[s] = gx;
  a.mg[(size_t)a.out_stride + s] = gy;
  a.mg[2 * (size_t)a.out_stride + s] = gz;
  a.nf[s] = nfac | kHugeFacets;
  a.hp_nbr[s] = fn;
  a.hp_area[s] = fa;
  const long long c2 = clock64();
  if (a.node_wmax) certify(a, C, s, row, pi, S.ws ? S.ws[s] : 0.0);
  if (a.stats) {
    unsigned long long* o = a.stats + (size_t)qi * kHugeStats;
    o[1] = (unsigned long long)(c2 - c1);
    o[2] = (unsigned long long)(clock64() - c2);
    o[7] = C.nodes;
    o[8] = C.seeds;
  }
}

}  // namespace

void launch_huge(const HugeArgs& a, cudaStream_t st) {
  if (a.nq == 0) return;
  huge_kernel<<<a.nq, 1, 0, st>>>(a);
  count_launch();
  last_launch_error = cudaGetLastError();
}

}  // namespace gbv
