// Cell polytopes of the last computed cells, as the reference writes them:
// ConvexCell::save (voronoi/convex_cell.cpp:282-352) and append_to_mesh
// (:371-444).  Both list one vertex per valid triangle in the order of the
// valid list (here: ascending effective list key, the order the geometry
// kernel also recovers), with coordinates from compute_triangle_point divided
// by w (gbv_refgeom.cuh, bit-identical), then one polygon per plane that
// still bounds the cell, in plane creation order (box faces, then the seeds
// in clipping order), walked from v2t[v] -- the last valid triangle holding
// the plane -- to triangle_adjacent(t, (lv + 1) % 3) until it closes.
//
// One thread per requested cell; a count pass sizes the outputs (a cell of
// nt corners has nt vertices and 3 nt polygon entries), a fill pass writes
// them.  The combinatorics come from the clipping kernels' records (by
// sorted slot), which stay valid until the seeds are sorted again; cells of
// the unbounded single-thread path keep theirs in scratch that is gone, so
// they are reported and not exported.
#include "gbv_context.cuh"
#include "gbv_refgeom.cuh"

namespace gbv {
namespace {

struct MeshArgs {
  const uint32_t* cells;  // original indices (nullptr: 0..m-1)
  uint32_t m;
  uint32_t n;
  const uint32_t* slot_of;
  const uint32_t* perm;
  const double4* xd;
  const double* q;
  CombBuf cb;
  const uint32_t* nf;
  double box[6];
  uint32_t* nv;            // count pass: corners per cell
  uint32_t* nfc;           // count pass: polygons per cell
  const uint32_t* vofs;    // fill pass: exclusive scans of nv and nfc
  const uint32_t* fofs;
  double* verts;           // [3][..] row-major x, y, z per vertex
  uint32_t* face_ptr;
  uint32_t* face_vtx;      // cell-local vertex numbers
  uint32_t* face_seed;     // original index of the seed across the face, kNone: box
  uint32_t* err;           // [0] unbounded-path cells, [1] indices >= n, [2] open fans
};

__device__ __forceinline__ double4 mesh_plane(const MeshArgs& a, uint32_t own, const double4& pi,
                                              double qi) {
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

template <bool FILL>
__global__ void cell_mesh_kernel(MeshArgs a) {
  const uint32_t qc = blockIdx.x * blockDim.x + threadIdx.x;
  if (qc >= a.m) return;
  const uint32_t i = a.cells ? a.cells[qc] : qc;
  bool skip = false;
  uint32_t s = 0;
  if (i >= a.n) {
    if (!FILL) atomicAdd(&a.err[1], 1u);
    skip = true;
  } else {
    s = a.slot_of[i];
    if (a.nf[s] & kHugeFacets) {
      if (!FILL) atomicAdd(&a.err[0], 1u);
      skip = true;
    }
  }
  if (skip) {
    if (!FILL) {
      a.nv[qc] = 0;
      a.nfc[qc] = 0;
    }
    return;
  }
  const size_t tb = (size_t)s * kTMax, pb = (size_t)s * kPMax;
  const ulonglong2 tm = a.cb.tmask[s];
  const uint64_t pm = a.cb.pmask[s];
  const int parity = (a.cb.flags[s] & 1u) ? -1 : 1;

  // valid triangles in list order: ascending effective key
  uint8_t ord[kTMax];
  int eff[kTMax];
  int nt = 0;
  for (int h = 0; h < 2; ++h) {
    uint64_t w = h ? tm.y : tm.x;
    while (w) {
      const int t = 64 * h + __ffsll((long long)w) - 1;
      w &= w - 1;
      const int e = parity * (int)a.cb.key[tb + t];
      int p = nt++;
      while (p > 0 && eff[p - 1] > e) {
        eff[p] = eff[p - 1];
        ord[p] = ord[p - 1];
        --p;
      }
      eff[p] = e;
      ord[p] = (uint8_t)t;
    }
  }
  // v2t: the last triangle of the list that holds the plane
  int v2t[kPMax];
  for (int p = 0; p < kPMax; ++p) v2t[p] = -1;
  for (int r = 0; r < nt; ++r) {
    const uint32_t v = a.cb.tv[tb + ord[r]];
    v2t[v & 0xFF] = ord[r];
    v2t[v >> 8 & 0xFF] = ord[r];
    v2t[v >> 16 & 0xFF] = ord[r];
  }
  // planes that bound the cell, in creation order: box faces (their own
  // slots 0-5), then the seeds by clipping position
  uint8_t po[kPMax];
  int nfaces = 0;
  for (int p = 0; p < kPMax; ++p) {
    if (!((pm >> p) & 1ull) || v2t[p] < 0) continue;
    const uint16_t rk = a.cb.prank[pb + p];
    const int key = rk == 0xFFFF ? p : 6 + rk;
    int j = nfaces++;
    while (j > 0) {
      const uint16_t rj = a.cb.prank[pb + po[j - 1]];
      const int kj = rj == 0xFFFF ? po[j - 1] : 6 + rj;
      if (kj < key) break;
      po[j] = po[j - 1];
      --j;
    }
    po[j] = (uint8_t)p;
  }
  if (!FILL) {
    a.nv[qc] = (uint32_t)nt;
    a.nfc[qc] = (uint32_t)nfaces;
    return;
  }

  uint8_t tix[kTMax];
  for (int r = 0; r < nt; ++r) tix[ord[r]] = (uint8_t)r;
  const double4 pi = a.xd[s];
  const double qi = a.q[s];
  const size_t v0 = a.vofs[qc];
  for (int r = 0; r < nt; ++r) {
    const uint32_t v = a.cb.tv[tb + ord[r]];
    const double3 c = r_corner(mesh_plane(a, a.cb.pown[pb + (v & 0xFF)], pi, qi),
                               mesh_plane(a, a.cb.pown[pb + (v >> 8 & 0xFF)], pi, qi),
                               mesh_plane(a, a.cb.pown[pb + (v >> 16 & 0xFF)], pi, qi));
    a.verts[3 * (v0 + r)] = c.x;
    a.verts[3 * (v0 + r) + 1] = c.y;
    a.verts[3 * (v0 + r) + 2] = c.z;
  }
  size_t f = a.fofs[qc];
  size_t idx = 3 * v0;
  const size_t idx_end = 3 * (v0 + (size_t)nt);
  bool open = false;
  for (int k = 0; k < nfaces; ++k) {
    const int p = po[k];
    const uint32_t own = a.cb.pown[pb + p];
    a.face_ptr[f] = (uint32_t)idx;
    a.face_seed[f] = own >= kBoxBase ? kNone : a.perm[own];
    ++f;
    const int t0 = v2t[p];
    int t = t0, steps = 0;
    do {
      if (idx >= idx_end) {
        open = true;
        break;
      }
      a.face_vtx[idx++] = tix[t];
      const uint32_t v = a.cb.tv[tb + t];
      const int lv = ((v & 0xFF) == (uint32_t)p) ? 0 : (((v >> 8 & 0xFF) == (uint32_t)p) ? 1 : 2);
      t = (int)((a.cb.ta[tb + t] >> (8 * ((lv + 1) % 3))) & 0xFF);
    } while (t != t0 && ++steps < kTMax);
    if (t != t0) open = true;
  }
  if (open || idx != idx_end) atomicAdd(&a.err[2], 1u);
}

}  // namespace
}  // namespace gbv

using namespace gbv;

extern "C" gbv_status gbv_cells_mesh(gbv_context* c, const uint32_t* cells, uint32_t m,
                                     gbv_mesh_sizes* sizes, double* vertices,
                                     uint32_t* cell_vertex_ptr, uint32_t* cell_face_ptr,
                                     uint32_t* face_ptr, uint32_t* face_vertices,
                                     uint32_t* face_seed) {
  auto fail = [](gbv_status st, const std::string& msg) {
    set_last_error(msg.c_str());
    return st;
  };
  if (!c) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL context");
  if (!c->has_cells) return fail(GBV_ERR_STATE, "no cells computed");
  if (!cells) m = c->n;
  try {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const uint32_t n = c->n;
    MeshArgs a{};
    a.m = m;
    a.n = n;
    a.slot_of = c->S.slot_of;
    a.perm = c->S.perm;
    a.xd = c->S.xd;
    a.q = c->S.q;
    a.cb.tv = c->buf<uint32_t>("cb_tv", (size_t)kTMax * n);
    a.cb.ta = c->buf<uint32_t>("cb_ta", (size_t)kTMax * n);
    a.cb.key = c->buf<int16_t>("cb_key", (size_t)kTMax * n);
    a.cb.pown = c->buf<uint32_t>("cb_pown", (size_t)kPMax * n);
    a.cb.prank = c->buf<uint16_t>("cb_prank", (size_t)kPMax * n);
    a.cb.tmask = c->buf<ulonglong2>("cb_tmask", n);
    a.cb.pmask = c->buf<uint64_t>("cb_pmask", n);
    a.cb.flags = c->buf<uint32_t>("cb_flags", n);
    a.nf = c->buf<uint32_t>("nf", n);
    for (int k = 0; k < 6; ++k) a.box[k] = c->box[k];
    if (cells) {
      uint32_t* dc = c->buf<uint32_t>("mesh_cells", std::max<uint32_t>(m, 1));
      if (m) GBV_CUDA(cudaMemcpyAsync(dc, cells, 4 * (size_t)m, cudaMemcpyHostToDevice, st));
      a.cells = dc;
    }
    uint32_t* nv = c->buf<uint32_t>("mesh_nv", (size_t)m + 1);
    uint32_t* nfc = c->buf<uint32_t>("mesh_nf", (size_t)m + 1);
    a.err = c->buf<uint32_t>("mesh_err", 4);
    a.nv = nv;
    a.nfc = nfc;
    GBV_CUDA(cudaMemsetAsync(a.err, 0, 4 * sizeof(uint32_t), st));
    GBV_CUDA(cudaMemsetAsync(nv + m, 0, sizeof(uint32_t), st));
    GBV_CUDA(cudaMemsetAsync(nfc + m, 0, sizeof(uint32_t), st));
    const unsigned nb = (m + 127) / 128;
    if (m) {
      cell_mesh_kernel<false><<<nb, 128, 0, st>>>(a);
      count_launch();
    }
    GBV_CUDA(cudaGetLastError());
    uint32_t* tmp = c->buf<uint32_t>("mesh_scan", scan_tmp_elems((size_t)m + 1));
    exclusive_scan_u32(nv, (size_t)m + 1, tmp, st);
    exclusive_scan_u32(nfc, (size_t)m + 1, tmp, st);
    uint32_t h[6] = {0, 0, 0, 0, 0, 0};
    GBV_CUDA(cudaMemcpyAsync(h, a.err, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaMemcpyAsync(h + 4, nv + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaMemcpyAsync(h + 5, nfc + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    if (h[1]) return fail(GBV_ERR_INVALID_ARGUMENT, std::to_string(h[1]) +
                                                        " cell index(es) beyond the cells");
    if (h[0])
      return fail(GBV_ERR_CAPACITY,
                  std::to_string(h[0]) + " cell(s) beyond " + std::to_string(kTMax) +
                      " corners: the unbounded path keeps no polytope to export");
    const uint64_t NV = h[4], NF = h[5];
    if (sizes) {
      sizes->n_vertices = NV;
      sizes->n_faces = NF;
      sizes->n_face_vertices = 3 * NV;
    }
    if (3 * NV > 0xFFFFFFFFull)
      return fail(GBV_ERR_CAPACITY, "more than 2^32 polygon entries: export fewer cells");
    if (!(vertices || cell_vertex_ptr || cell_face_ptr || face_ptr || face_vertices || face_seed))
      return GBV_OK;
    a.vofs = nv;
    a.fofs = nfc;
    a.verts = c->buf<double>("mesh_verts", 3 * NV);
    a.face_ptr = c->buf<uint32_t>("mesh_fptr", NF + 1);
    a.face_vtx = c->buf<uint32_t>("mesh_fvtx", 3 * NV);
    a.face_seed = c->buf<uint32_t>("mesh_fseed", NF);
    if (m) {
      cell_mesh_kernel<true><<<nb, 128, 0, st>>>(a);
      count_launch();
    }
    GBV_CUDA(cudaGetLastError());
    const uint32_t tot = (uint32_t)(3 * NV);
    GBV_CUDA(cudaMemcpyAsync(a.face_ptr + NF, &tot, sizeof(uint32_t), cudaMemcpyHostToDevice,
                             st));
    GBV_CUDA(cudaMemcpyAsync(h, a.err + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (vertices && NV)
      GBV_CUDA(cudaMemcpyAsync(vertices, a.verts, 24 * NV, cudaMemcpyDeviceToHost, st));
    if (cell_vertex_ptr)
      GBV_CUDA(cudaMemcpyAsync(cell_vertex_ptr, nv, 4 * ((size_t)m + 1), cudaMemcpyDeviceToHost,
                               st));
    if (cell_face_ptr)
      GBV_CUDA(cudaMemcpyAsync(cell_face_ptr, nfc, 4 * ((size_t)m + 1), cudaMemcpyDeviceToHost,
                               st));
    if (face_ptr)
      GBV_CUDA(cudaMemcpyAsync(face_ptr, a.face_ptr, 4 * (NF + 1), cudaMemcpyDeviceToHost, st));
    if (face_vertices && NV)
      GBV_CUDA(cudaMemcpyAsync(face_vertices, a.face_vtx, 12 * NV, cudaMemcpyDeviceToHost, st));
    if (face_seed && NF)
      GBV_CUDA(cudaMemcpyAsync(face_seed, a.face_seed, 4 * NF, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    if (h[0]) return fail(GBV_ERR_STATE, std::to_string(h[0]) + " polygon fan(s) did not close");
    return GBV_OK;
  } catch (const CudaError& e) {
    return fail(GBV_ERR_CUDA, e.where + ": " + cudaGetErrorString(e.e));
  } catch (const StatusError& e) {
    return fail(e.st, e.msg);
  }
}
