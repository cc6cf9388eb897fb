/*
 * Oracle reference harness -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is compiled together with geogram's own sources, straight from
 * the reference checkout, into oracle/_ref/libgbv_ref.so (recipe:
 * oracle/ref/Makefile).  It validates the CPU restatement in
 * oracle/gbv_oracle.c and for the GPU path; nothing in the product links or
 * calls it.
 *
 * What runs here is the reference's code:
 *   - kNN: GEO::NearestNeighborSearch::create(dim, "BNN") -> BalancedKdTree
 *     (points/nn_search.cpp:118-149, points/kd_tree.cpp:156-387);
 *   - cells: VBW::ConvexCell with exact predicates (voronoi/convex_cell.cpp:
 *     init_with_box :175-215, clip_by_plane :461-516, compute_geometry
 *     :1125-1145, compute_mg :1267-1307, facet_area :1160-1191,
 *     squared_radius :1312-1330), and its output ConvexCell::save
 *     (:282-352).
 * What is composed here (the reference has no meshless Laguerre driver):
 *   - the per-seed neighbour list of Delaunay_NearestNeighbors
 *     (delaunay/delaunay_nn.cpp:104-145: ask k+1, drop self, a duplicate
 *     with a lower index empties the list);
 *   - the security-radius loop of generic_RVD.h:2278-2352 (stop when
 *     d2(pi,pj) > 4.1 R2, grow k by k/8 when k>8 else by 1);
 *   - the power bisector of periodic_delaunay_3d.cpp:3722-3726;
 *   - for weights, the 4-d lift used by compute_OTM/main.cpp:280-283:
 *     h_i = sqrt(W - w_i), W = max w; kNN and the security radius are taken
 *     in 4-d (R2 = squared_radius(p_i) + h_i^2).
 */
#include <geogram/basic/common.h>
#include <geogram/basic/logger.h>
#include <geogram/basic/process.h>
#include <geogram/basic/command_line.h>
#include <geogram/basic/command_line_args.h>
#include <geogram/basic/file_system.h>
#include <geogram/basic/progress.h>
#include <geogram/basic/stopwatch.h>
#include <geogram/numerics/predicates.h>
#include <geogram/points/nn_search.h>
#include <geogram/voronoi/convex_cell.h>
#include <geogram/voronoi/RVD.h>
#include <geogram/voronoi/CVT.h>
#include <geogram/delaunay/delaunay.h>
#include <geogram/delaunay/periodic_delaunay_3d.h>
#include <geogram/mesh/mesh.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <sstream>
#include <thread>
#include <vector>

namespace {

bool g_initialised = false;
// 1: clip with ConvexCell::clip_by_plane_fast (convex_cell.cpp:599-757)
int g_walk = 0;

void ensure_init() {
    if (g_initialised) return;
    GEO::FileSystem::initialize();
    GEO::Logger::initialize();
    GEO::Process::initialize(0);
    GEO::Progress::initialize();
    GEO::CmdLine::initialize();
    GEO::Stopwatch::initialize();
    GEO::PCK::initialize();
    GEO::Delaunay::initialize();
    // the argument groups the Delaunay and RVD factories read
    // (algo:delaunay, algo:predicates, dbg:*), with their defaults
    GEO::CmdLine::import_arg_group("standard");
    GEO::CmdLine::import_arg_group("algo");
    GEO::Logger::instance()->set_quiet(true);
    g_initialised = true;
}

template <class F>
void run_threads(unsigned n, int nthreads, F&& body) {
    if (nthreads <= 1 || n < 64) {
        body(0u, n);
        return;
    }
    std::atomic<unsigned> next(0);
    const unsigned chunk = 256;
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) {
        pool.emplace_back([&]() {
            for (;;) {
                unsigned b = next.fetch_add(chunk);
                if (b >= n) break;
                body(b, std::min(n, b + chunk));
            }
        });
    }
    for (auto& th : pool) th.join();
}

/* Neighbour list of one seed, as Delaunay_NearestNeighbors builds it
 * (delaunay_nn.cpp:104-145). Returns the list length. */
unsigned seed_neighbours(const GEO::NearestNeighborSearch* nn, unsigned n,
                         unsigned i, unsigned nb, std::vector<GEO::index_t>& ix,
                         std::vector<double>& dd, std::vector<GEO::index_t>& out) {
    nb = std::min(nb + 1, n);
    ix.resize(nb);
    dd.resize(nb);
    nn->get_nearest_neighbors(nb, i, ix.data(), dd.data());
    out.clear();
    for (unsigned j = 0; j < nb; ++j) {
        if (ix[j] == i) continue;
        if (dd[j] == 0.0) {
            if (ix[j] < i) { out.clear(); return 0; }
            continue;
        }
        out.push_back(ix[j]);
        if (out.size() == nb - 1) break;
    }
    return unsigned(out.size());
}

/* The lifted points (4-d when weighted) of the seeds. */
unsigned lifted_points(const double* xyz, const double* w, unsigned n, std::vector<double>& pts,
                       std::vector<double>& h) {
    unsigned dim = (w != nullptr) ? 4u : 3u;
    pts.assign(size_t(n) * dim, 0.0);
    h.assign(n, 0.0);
    if (w != nullptr) {
        double W = w[0];
        for (unsigned i = 1; i < n; ++i) W = std::max(W, w[i]);
        for (unsigned i = 0; i < n; ++i) h[i] = ::sqrt(W - w[i]);
    }
    for (unsigned i = 0; i < n; ++i) {
        for (unsigned c = 0; c < 3; ++c) pts[size_t(i) * dim + c] = xyz[3 * size_t(i) + c];
        if (dim == 4) pts[size_t(i) * dim + 3] = h[i];
    }
    return dim;
}

/* Clips the box [0,1]^3 to the cell of seed i with the security-radius
 * loop; returns the status, *list_out the list length, *clips_out the
 * planes clipped. */
int clip_cell(VBW::ConvexCell& C, const GEO::NearestNeighborSearch* nn, const double* xyz,
              const double* w, const std::vector<double>& pts, const std::vector<double>& h,
              unsigned dim, unsigned n, unsigned i, unsigned k0, int check_sr,
              std::vector<GEO::index_t>& ix, std::vector<double>& dd,
              std::vector<GEO::index_t>& nbrs, unsigned* list_out, unsigned* clips_out) {
    const double* pi = &pts[size_t(i) * dim];
    const double wi = (w != nullptr) ? w[i] : 0.0;
    const double pi_len2 = xyz[3 * i] * xyz[3 * i] +
                           xyz[3 * i + 1] * xyz[3 * i + 1] +
                           xyz[3 * i + 2] * xyz[3 * i + 2];
    C.init_with_box(0.0, 0.0, 0.0, 1.0, 1.0, 1.0);
    int st = 1;
    unsigned jj = 0, prev = 0, nb_req = std::min(k0, n - 1);
    nbrs.clear();
    unsigned list = seed_neighbours(nn, n, i, nb_req, ix, dd, nbrs);
    bool done = false;
    while (!done) {
        if (list == 0) { st = 2; break; }
        if (prev == list) { st = 3; break; }
        for (; jj < list; ++jj) {
            GEO::index_t j = nbrs[jj];
            double R2 = C.squared_radius(
                VBW::make_vec3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
            if (dim == 4) R2 += h[i] * h[i];
            const double* pj = &pts[size_t(j) * dim];
            double dij = 0.0;
            for (unsigned c = 0; c < dim; ++c) dij += (pj[c] - pi[c]) * (pj[c] - pi[c]);
            if (check_sr && dij > 4.1 * R2) { st = 0; done = true; break; }
            const double wj = (w != nullptr) ? w[j] : 0.0;
            const double pj_len2 = xyz[3 * j] * xyz[3 * j] +
                                   xyz[3 * j + 1] * xyz[3 * j + 1] +
                                   xyz[3 * j + 2] * xyz[3 * j + 2];
            VBW::vec4 P = VBW::make_vec4(
                2.0 * (xyz[3 * i] - xyz[3 * j]),
                2.0 * (xyz[3 * i + 1] - xyz[3 * j + 1]),
                2.0 * (xyz[3 * i + 2] - xyz[3 * j + 2]),
                (wi - pi_len2) - (wj - pj_len2));
            if (g_walk) C.clip_by_plane_fast(P, j);
            else C.clip_by_plane(P, j);
        }
        if (done) break;
        if (!check_sr) { st = 0; break; }
        if (list >= n - 1) { st = 1; break; }
        prev = list;
        unsigned nb = list;
        nb = (nb > 8) ? nb + nb / 8 : nb + 1;
        nb = std::min(nb, n - 1);
        list = seed_neighbours(nn, n, i, nb, ix, dd, nbrs);
    }
    *list_out = list;
    *clips_out = jj;
    return st;
}

}  // namespace

extern "C" {

int ref_init(void) {
    ensure_init();
    return 0;
}

/* Selects clip_by_plane_fast (walk = 1) or clip_by_plane (walk = 0) for
 * the cell functions below. */
int ref_set_walk(int walk) {
    g_walk = walk;
    return 0;
}

/* k nearest neighbours of every point (self included), ascending d2. */
int ref_knn(const double* pts, unsigned dim, unsigned n, unsigned k,
            unsigned* idx, double* d2, int nthreads) {
    ensure_init();
    if (k > n) return 1;
    GEO::NearestNeighborSearch_var nn =
        GEO::NearestNeighborSearch::create(GEO::coord_index_t(dim), "BNN");
    nn->set_points(n, pts);
    run_threads(n, nthreads, [&](unsigned b, unsigned e) {
        for (unsigned i = b; i < e; ++i) {
            nn->get_nearest_neighbors(k, i, idx + size_t(i) * k,
                                      d2 + size_t(i) * k);
        }
    });
    nn.reset();
    return 0;
}

/*
 * Certified Laguerre cells clipped to the box [0,1]^3.
 *   xyz    : 3n seeds; w: n weights or NULL (Voronoi)
 *   k0     : initial neighbour count (20 in Delaunay_NearestNeighbors)
 *   check_sr: 1 = grow k until the security radius certifies the cell
 *   exact  : 1 = exact predicates (the ConvexCell default)
 * Outputs (per seed i):
 *   vol[i], mg[3i..3i+2] (volume-weighted centroid, compute_mg),
 *   nbr_count[i] and, in nbr_idx/nbr_area[i*max_nbr ...], the contributing
 *   seed facets in clipping order, k_list[i] (list length when stopped),
 *   n_clip[i] (planes clipped), status[i]:
 *     0 certified, 1 all n-1 neighbours clipped, 2 empty neighbour list
 *     (duplicate seed), 3 list stopped growing, 4 more facets than max_nbr.
 */
int ref_cells(const double* xyz, const double* w, unsigned n, unsigned k0,
              int check_sr, int exact, int nthreads, double* vol, double* mg,
              unsigned* nbr_count, unsigned* nbr_idx, double* nbr_area,
              unsigned max_nbr, unsigned* k_list, unsigned* n_clip,
              int* status) {
    ensure_init();
    if (n < 2) return 1;
    std::vector<double> pts, h;
    const unsigned dim = lifted_points(xyz, w, n, pts, h);
    GEO::NearestNeighborSearch_var nn =
        GEO::NearestNeighborSearch::create(GEO::coord_index_t(dim), "BNN");
    nn->set_points(n, pts.data());

    run_threads(n, nthreads, [&](unsigned b, unsigned e) {
        VBW::ConvexCell C(VBW::WithVGlobal);
        C.use_exact_predicates(exact != 0);
        std::vector<GEO::index_t> ix, nbrs;
        std::vector<double> dd;
        for (unsigned i = b; i < e; ++i) {
            unsigned list = 0, jj = 0;
            int st = clip_cell(C, nn, xyz, w, pts, h, dim, n, i, k0, check_sr, ix, dd, nbrs,
                               &list, &jj);
            C.compute_geometry();
            double m = 0.0;
            VBW::vec3 g = VBW::make_vec3(0.0, 0.0, 0.0);
            C.compute_mg(m, g);
            vol[i] = m;
            mg[3 * i] = g.x;
            mg[3 * i + 1] = g.y;
            mg[3 * i + 2] = g.z;
            unsigned cnt = 0;
            for (VBW::index_t v = 1; v < C.nb_v(); ++v) {
                if (!C.vertex_is_contributing(v)) continue;
                VBW::global_index_t j = C.v_global_index(v);
                if (j == VBW::global_index_t(-1)) continue;
                if (cnt < max_nbr) {
                    nbr_idx[size_t(i) * max_nbr + cnt] = unsigned(j);
                    nbr_area[size_t(i) * max_nbr + cnt] = C.facet_area(v);
                }
                ++cnt;
            }
            if (cnt > max_nbr) st = 4;
            nbr_count[i] = cnt;
            k_list[i] = list;
            n_clip[i] = jj;
            status[i] = st;
        }
    });
    nn.reset();
    return 0;
}

/*
 * The cells of seeds which[0 .. m) written one after the other by
 * ConvexCell::save (voronoi/convex_cell.cpp:282-352) into out (at most cap
 * bytes, NUL-terminated), vertex numbers continuing from one cell to the
 * next (v_offset 1, then 1 + the vertices written so far), with the given
 * shrink factor.  Returns the text length, or -1 when cap is too small.
 */
long ref_cells_save(const double* xyz, const double* w, unsigned n, unsigned k0,
                    int check_sr, const unsigned* which, unsigned m, double shrink,
                    char* out, size_t cap) {
    ensure_init();
    if (n < 2) return -1;
    std::vector<double> pts, h;
    const unsigned dim = lifted_points(xyz, w, n, pts, h);
    GEO::NearestNeighborSearch_var nn =
        GEO::NearestNeighborSearch::create(GEO::coord_index_t(dim), "BNN");
    nn->set_points(n, pts.data());
    VBW::ConvexCell C(VBW::WithVGlobal);
    std::vector<GEO::index_t> ix, nbrs;
    std::vector<double> dd;
    std::ostringstream os;
    GEO::index_t v_offset = 1;
    for (unsigned q = 0; q < m; ++q) {
        unsigned list = 0, jj = 0;
        clip_cell(C, nn, xyz, w, pts, h, dim, n, which[q], k0, check_sr, ix, dd, nbrs, &list,
                  &jj);
        v_offset += C.save(os, v_offset, shrink);
    }
    nn.reset();
    const std::string txt = os.str();
    if (txt.size() + 1 > cap) return -1;
    std::memcpy(out, txt.c_str(), txt.size() + 1);
    return long(txt.size());
}

/*
 * Voronoi cells restricted to a tetrahedral mesh (volumetric RVD,
 * voronoi/RVD.cpp compute_centroids_in_volume :500-530 and
 * compute_CVT_func_grad_in_volume :878-910) of the seeds, with the
 * reference's own Delaunay triangulation ("BDEL") and
 * RestrictedVoronoiDiagram.
 *   verts[3 nv], tets[4 nt] (vertex indices), seeds[3 n]
 * Outputs: mg[3 n], m[n] (mass and first moment of each restricted cell),
 * *f and g[3 n] (the CVT energy sum_i int |x - p_i|^2 over the restricted
 * cells and its gradient).  nthreads = 1 keeps the reference single-threaded.
 */
int ref_rvd_volume(const double* verts, unsigned nv, const unsigned* tets, unsigned nt,
                   const double* seeds, unsigned n, double* mg, double* m, double* f,
                   double* g) {
    ensure_init();
    GEO::Process::set_max_threads(1);
    GEO::Mesh M(3);
    M.vertices.create_vertices(nv);
    for (unsigned v = 0; v < nv; ++v)
        for (unsigned c = 0; c < 3; ++c) M.vertices.point_ptr(v)[c] = verts[3 * size_t(v) + c];
    M.cells.create_tets(nt);
    for (unsigned t = 0; t < nt; ++t)
        for (unsigned k = 0; k < 4; ++k) M.cells.set_vertex(t, k, tets[4 * size_t(t) + k]);
    M.cells.connect();
    // the RVD configures the triangulation it observes: created first, as
    // compute_RVD/main.cpp and CVT.cpp:55-75 do, then the seeds are set
    GEO::Delaunay_var del = GEO::Delaunay::create(3, "BDEL");
    GEO::RestrictedVoronoiDiagram_var rvd = GEO::RestrictedVoronoiDiagram::create(del, &M);
    del->set_vertices(n, seeds);
    rvd->set_volumetric(true);
    for (size_t k = 0; k < size_t(n); ++k) {
        m[k] = 0.0;
        for (int c = 0; c < 3; ++c) {
            mg[3 * k + c] = 0.0;
            g[3 * k + c] = 0.0;
        }
    }
    rvd->compute_centroids(mg, m);
    double fv = 0.0;
    rvd->compute_CVT_func_grad(fv, g);
    *f = fv;
    return 0;
}

/*
 * CentroidalVoronoiTesselation::Newton_iterations(nb_iter, m) (voronoi/
 * CVT.cpp:272-307, HLBFGS) on the volumetric tet mesh: seeds[3 n] hold the
 * start and receive the result; *f the CVT energy at the result.
 */
int ref_cvt_newton(const double* verts, unsigned nv, const unsigned* tets, unsigned nt,
                   double* seeds, unsigned n, unsigned nb_iter, unsigned m, double* f) {
    ensure_init();
    GEO::Process::set_max_threads(1);
    GEO::Mesh M(3);
    M.vertices.create_vertices(nv);
    for (unsigned v = 0; v < nv; ++v)
        for (unsigned c = 0; c < 3; ++c) M.vertices.point_ptr(v)[c] = verts[3 * size_t(v) + c];
    M.cells.create_tets(nt);
    for (unsigned t = 0; t < nt; ++t)
        for (unsigned k = 0; k < 4; ++k) M.cells.set_vertex(t, k, tets[4 * size_t(t) + k]);
    M.cells.connect();
    {
        GEO::CentroidalVoronoiTesselation cvt(&M, 3, "BDEL");
        cvt.set_volumetric(true);
        cvt.set_points(n, seeds);
        cvt.Newton_iterations(nb_iter, m);
        for (unsigned i = 0; i < n; ++i)
            for (unsigned c = 0; c < 3; ++c) seeds[3 * size_t(i) + c] = cvt.embedding(i)[c];
    }
    std::vector<double> mg(3 * size_t(n)), mm(n), g(3 * size_t(n));
    return ref_rvd_volume(verts, nv, tets, nt, seeds, n, mg.data(), mm.data(), f, g.data());
}

/*
 * Laguerre cells of the seeds in the periodic cube [0, period)^3, by the
 * reference's PeriodicDelaunay3d (delaunay/periodic_delaunay_3d.cpp:
 * compute, copy_Laguerre_cell_from_Delaunay :3634-3734) and ConvexCell
 * geometry.  Per seed i: vol[i], mg[3i..], and its facets (at most max_nbr):
 * the real index of the seed across the facet, the translation of that
 * image as the code (tx+1)*9 + (ty+1)*3 + (tz+1) (13: none), the facet's
 * area.  xyz must lie in [0, period).
 */
int ref_periodic_cells(const double* xyz, const double* w, unsigned n, double period,
                       double* vol, double* mg, unsigned* nbr_count, unsigned* nbr_idx,
                       unsigned char* nbr_shift, double* nbr_area, unsigned max_nbr) {
    ensure_init();
    if (n < 2) return 1;
    // reference-counted: heap-allocated and held by a SmartPointer
    GEO::SmartPointer<GEO::PeriodicDelaunay3d> dp = new GEO::PeriodicDelaunay3d(true, period);
    GEO::PeriodicDelaunay3d& del = *dp;
    del.set_vertices(n, xyz);
    if (w != nullptr) del.set_weights(w);
    del.compute();
    VBW::ConvexCell C(VBW::WithVGlobal);
    for (unsigned i = 0; i < n; ++i) {
        del.copy_Laguerre_cell_from_Delaunay(i, C);
        C.compute_geometry();
        double m = 0.0;
        VBW::vec3 g = VBW::make_vec3(0.0, 0.0, 0.0);
        C.compute_mg(m, g);
        vol[i] = m;
        mg[3 * i] = g.x;
        mg[3 * i + 1] = g.y;
        mg[3 * i + 2] = g.z;
        unsigned cnt = 0;
        for (VBW::index_t v = 1; v < C.nb_v(); ++v) {
            if (!C.vertex_is_contributing(v)) continue;
            const VBW::global_index_t j = C.v_global_index(v);
            if (j == VBW::global_index_t(-1)) continue;
            if (cnt < max_nbr) {
                const unsigned inst = unsigned(j) / n;
                const int* T = GEO::Periodic::translation[inst];
                nbr_idx[size_t(i) * max_nbr + cnt] = unsigned(j) % n;
                nbr_shift[size_t(i) * max_nbr + cnt] =
                    (unsigned char)((T[0] + 1) * 9 + (T[1] + 1) * 3 + (T[2] + 1));
                nbr_area[size_t(i) * max_nbr + cnt] = C.facet_area(v);
            }
            ++cnt;
        }
        nbr_count[i] = cnt;
    }
    return 0;
}

}  // extern "C"
