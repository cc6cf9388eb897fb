/*
 * gbv.h -- C ABI of the GB300 meshless Voronoi/Laguerre cell engine.
 *
 * A drop-in for geogram's meshless cell path.  Every entry point below
 * replaces one reference interface; the citation is given beside it
 * (paths relative to geogram's src/lib/).  Plain pointers and sizes only:
 * no C++ or torch types cross this boundary, no exception leaves it, and
 * every call returns a gbv_status (the message of the last failure on the
 * calling thread is in gbv_last_error()).
 *
 * Ownership follows the reference: input arrays stay caller-owned; the
 * context copies them to the GPU and owns its device buffers until
 * gbv_destroy().  Host output arrays are caller-allocated.  Calls on one
 * context are synchronous and must not be made concurrently; separate
 * contexts may be used from separate threads.
 */
#ifndef GBV_H
#define GBV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBV_OK = 0,
    GBV_ERR_INVALID_ARGUMENT = 1,
    GBV_ERR_CUDA = 2,
    GBV_ERR_NO_DEVICE = 3,
    GBV_ERR_CAPACITY = 4,
    GBV_ERR_NOT_CONVERGED = 5,
    GBV_ERR_STATE = 6
} gbv_status;

/* Per-cell outcome (cell_status).  0-2 are the outcomes of the reference's
 * security-radius loop, generic_RVD.h (geogram/voronoi) :2278-2352, with
 * the neighbour lists of delaunay_nn.cpp:104-145. */
enum {
    GBV_CELL_CERTIFIED = 0,       /* stopped by d2(pi,pj) > 4.1 R2          */
    GBV_CELL_ALL_NEIGHBOURS = 1,  /* every other seed was clipped           */
    GBV_CELL_DUPLICATE = 2,       /* a lower-index seed at distance 0: the
                                     neighbour list is empty, the cell is
                                     the unclipped box (as the reference)   */
    GBV_CELL_STALLED = 3,         /* the seed has higher-index copies: its
                                     lists are shorter than asked for, their
                                     growth stalls before certification and
                                     the reference stops there (the cell is
                                     not certified; delaunay_nn.cpp:104-145,
                                     generic_RVD.h:2297-2299)               */
    GBV_CELL_NEED_MORE_K = 16,    /* internal: list exhausted, retried      */
    GBV_CELL_OVERFLOW = 17,       /* internal: capacity exceeded, retried   */
    GBV_CELL_RECHECK = 18,        /* internal: FP32 could not certify       */
    GBV_CELL_ERROR = 19           /* the conflict zone was not a disk (never
                                     seen with exact signs; reported as an
                                     error by the compute call)             */
};

typedef enum {
    GBV_PRECISION_FP64 = 0,          /* all clipping in FP64, exact signs   */
    GBV_PRECISION_FP32_RECHECK = 1,  /* FP32 clipping with certified signs,
                                        FP64 geometry, FP64 re-clip of every
                                        cell FP32 could not certify: results
                                        identical to GBV_PRECISION_FP64     */
    GBV_PRECISION_FP32_GEOMETRY = 2  /* as FP32_RECHECK (same cells, same
                                        neighbours and facets, same status),
                                        but volumes, centroids and facet
                                        areas from FP32 corners in each
                                        seed's frame, summed in FP64: volumes
                                        and centroids within 1e-4 s, facet
                                        areas within 1e-3 s^(2/3), s the
                                        larger of the cell's volume and the
                                        mean cell volume.  For
                                        gbv_cells_* and Lloyd with the
                                        security radius (power-range cells
                                        keep FP64 geometry)                 */
} gbv_precision;

typedef struct gbv_context gbv_context;

typedef struct {
    double box_min[3];   /* clipping box (init_with_box, convex_cell.cpp:175) */
    double box_max[3];
    uint32_t k0;         /* first neighbour list length (20, delaunay_nn.cpp:50) */
    uint32_t check_sr;   /* 1: grow the list until certified (set_check_SR) */
    uint32_t precision;  /* gbv_precision */
    uint32_t certification; /* gbv_certification */
    uint32_t first_k;    /* no counterpart in the reference: neighbours fetched
                            by the first kNN pass of the security-radius loop
                            (the reference starts at k0 and grows by k/8; a
                            longer first list gives the same cells with fewer
                            passes); 0: automatic (96 without weights, 128
                            with), at most 128 */
    uint32_t predicates; /* gbv_predicates */
} gbv_cell_options;

typedef enum {
    /* PCK::det_4d, the ConvexCell default (convex_cell.cpp:873-912) */
    GBV_PREDICATES_EXACT = 0,
    /* use_exact_predicates(false): the FP64 det4x4 of convex_cell.h:383-402,
     * conflict iff > 0 (convex_cell.cpp:947-966); differs from the exact
     * mode only on degenerate configurations */
    GBV_PREDICATES_FAST = 1
} gbv_predicates;

typedef enum {
    /* the reference's security-radius loop (generic_RVD.h:2278-2352) on
     * the 4-d lift for weights: its results, bit for bit */
    GBV_CERTIFY_SECURITY_RADIUS = 0,
    /* no security radius: candidates from the kNN, then every seed that
     * could still cut the cell is found by a power range query around the
     * cell's corners (octree with per-node maximum weight) and clipped.
     * Same cells in exact arithmetic; needed when weights vary widely (the
     * lifted radius then spans most seeds), e.g. optimal transport. */
    GBV_CERTIFY_POWER_RANGE = 1
} gbv_certification;

typedef struct {
    uint64_t nnz;              /* facets between seeds (CSR entries)        */
    uint32_t n_cells;
    uint32_t n_recheck_fp64;   /* cells re-clipped in FP64 (precision mode) */
    uint32_t n_more_k;         /* cells that needed a longer list           */
    uint32_t n_overflow;       /* cells re-run with the large capacity      */
    uint32_t max_clips;        /* most neighbours visited by one cell       */
    uint32_t knn_k;            /* list length of the first pass             */
    double mean_clips;         /* mean neighbours visited per cell          */
    double volume_sum;         /* compensated FP64 sum of cell volumes      */
    uint64_t n_exact;          /* exact (expansion) predicate evaluations   */
    double ms_grid, ms_knn, ms_clip, ms_retry, ms_total;
    uint32_t n_huge;     /* cells beyond 128 corners / 64 planes (one-thread path) */
    uint32_t n_knn_exact; /* first-pass queries the FP32 kNN screening passed to
                             the exact search                          */
    uint64_t n_conflict_tests;  /* corner-versus-plane tests (triangle_is_in_conflict)
                                   of the first clipping pass over every cell */
    uint64_t n_corners_created; /* corners that pass created             */
    double ms_clip_kernel;      /* that pass's kernel alone               */
} gbv_cell_report;

/* ---------------------------------------------------------------- */
/* Context                                                          */
/* ---------------------------------------------------------------- */

/* Last error message of the calling thread ("" if none). */
const char* gbv_last_error(void);

/* Number of CUDA kernels this library has launched since it was loaded
 * (all contexts).  Replaces nothing in the reference; used to account for
 * the GPU work of a call. */
uint64_t gbv_kernel_launches(void);

/* Device memory the context holds now (its buffers are kept between calls
 * and grown on demand); *peak (optional) receives the most it held at
 * once.  No reference counterpart (a footprint report). */
uint64_t gbv_device_bytes(const gbv_context* ctx, uint64_t* peak);

/* Creates a context on CUDA device `device`.  Replaces nothing in the
 * reference (its engines are plain C++ objects); the context owns one
 * CUDA stream and the device buffers. */
gbv_status gbv_create(int device, gbv_context** out);
gbv_status gbv_destroy(gbv_context* ctx);

/* Fills the defaults: unit box, k0 = 20, check_sr = 1, FP64. */
void gbv_cell_options_default(gbv_cell_options* opt);

/* ---------------------------------------------------------------- */
/* NearestNeighborSearch (points/nn_search.h:69-262)                 */
/* ---------------------------------------------------------------- */

/* NearestNeighborSearch::set_points(n, pts, stride), nn_search.h:96-121.
 * dim = 3 (the reference's kd-tree takes any dimension; this engine takes
 * 3, or 4 for the lifted power-diagram points).  stride is in doubles,
 * >= dim (stride_supported() is true).  The points are copied to the GPU
 * and the search structure is built there. */
gbv_status gbv_nn_set_points(gbv_context* ctx, uint32_t n, const double* pts,
                             uint32_t dim, uint32_t stride);

/* NearestNeighborSearch::get_nearest_neighbors(k, q, idx, d2) for nq query
 * points (nn_search.h:131-160): the k nearest stored points of each query,
 * ascending squared distance, ties by point index.  q is nq*dim doubles;
 * idx and d2 are nq*k. */
gbv_status gbv_nn_get_nearest_neighbors(gbv_context* ctx, uint32_t nq,
                                        const double* q, uint32_t k,
                                        uint32_t* idx, double* d2);

/* get_nearest_neighbors(k, q_index, idx, d2) (nn_search.h:166-176) for
 * every stored point at once: row i holds the k nearest of point i, the
 * point itself included (d2 = 0), as the reference returns it.  This is
 * the batch table from which per-query calls are served. */
gbv_status gbv_nn_get_nearest_neighbors_all(gbv_context* ctx, uint32_t k,
                                            uint32_t* idx, double* d2);

/* ---------------------------------------------------------------- */
/* Laguerre cells (VBW::ConvexCell results, voronoi/convex_cell.h)   */
/* ---------------------------------------------------------------- */

/* For every seed: clip the box by the power bisectors of its nearest
 * neighbours (convex_cell.cpp:461-516, plane periodic_delaunay_3d.cpp:
 * 3722-3726) until the security radius certifies the cell
 * (generic_RVD.h:2278-2352).  xyz: 3n doubles; w: n weights or NULL
 * (Voronoi).  Inputs are host pointers; results stay on the device until
 * gbv_cells_fetch().  The report may be NULL.  GBV_ERR_CAPACITY when the
 * cells' facets total 2^32 or more (the CSR offsets are 32-bit). */
gbv_status gbv_cells_compute(gbv_context* ctx, const double* xyz,
                             const double* w, uint32_t n,
                             const gbv_cell_options* opt,
                             gbv_cell_report* report);

/* Same with device pointers, ordered on `stream` (a cudaStream_t, NULL =
 * the context's stream). */
gbv_status gbv_cells_compute_device(gbv_context* ctx, const double* d_xyz,
                                    const double* d_w, uint32_t n,
                                    const gbv_cell_options* opt, void* stream,
                                    gbv_cell_report* report);

/* Copies the last results to host arrays (each may be NULL):
 *   vol[n]           ConvexCell::volume()      (convex_cell.cpp:1215-1253)
 *   mg[3n]           ConvexCell::compute_mg()  (convex_cell.cpp:1267-1307)
 *   nbr_rowptr[n+1], nbr_idx[nnz], nbr_area[nnz]: the facets shared with
 *                    other seeds, i.e. v_global_index(v) and facet_area(v)
 *                    (convex_cell.h:768-830) for every contributing v,
 *                    in the reference's order (clipping order);
 *   cell_status[n]   GBV_CELL_*. */
gbv_status gbv_cells_fetch(gbv_context* ctx, double* vol, double* mg,
                           uint32_t* nbr_rowptr, uint32_t* nbr_idx,
                           double* nbr_area, int32_t* cell_status);

/* Device pointers of the last results (valid until the next compute). */
gbv_status gbv_cells_device_results(gbv_context* ctx, const double** vol,
                                    const double** mg,
                                    const uint32_t** nbr_rowptr,
                                    const uint32_t** nbr_idx,
                                    const double** nbr_area,
                                    const int32_t** cell_status);

/* ---------------------------------------------------------------- */
/* CVT Lloyd step (voronoi/CVT.cpp:133-167)                          */
/* ---------------------------------------------------------------- */

/* One Lloyd iteration on the meshless cells: computes the cells of xyz
 * (weights w or NULL) and replaces every seed by its centroid mg/m when
 * m > 1e-30 (CVT.cpp:150-160).  xyz is updated in place (host array). */
gbv_status gbv_lloyd_step(gbv_context* ctx, double* xyz, const double* w,
                          uint32_t n, const gbv_cell_options* opt,
                          gbv_cell_report* report);

/* Same on device arrays (d_xyz updated in place) for `iters` iterations. */
gbv_status gbv_lloyd_device(gbv_context* ctx, double* d_xyz, const double* d_w,
                            uint32_t n, uint32_t iters,
                            const gbv_cell_options* opt, void* stream,
                            gbv_cell_report* report);

/* ---------------------------------------------------------------- */
/* Semi-discrete optimal transport (OptimalTransportMap3d, exploragram;
 * program compute_OTM/main.cpp:280-296).  The exploragram sources are not in
 * the reference checkout; the solver follows the published method it
 * implements: damped Newton on the Kantorovich dual with FP64 conjugate
 * gradient on the Laguerre Hessian.                                  */
/* ---------------------------------------------------------------- */

typedef struct {
    double box_min[3];   /* source: uniform density on this machine */
    double box_max[3];
    double tol;          /* stop when max_i |vol_i - nu_i| / nu_i < tol (1e-6) */
    uint32_t max_newton; /* Newton iterations (100) */
    uint32_t max_cg;     /* CG iterations per Newton step (4000) */
    uint32_t precision;  /* gbv_precision of the cell computations */
    uint32_t reserved;
    /* CG stops at ||r|| <= cg_rtol ||b|| (default and 0: 1e-4; measured at
       1M clustered seeds: 30 Newton steps / 17.4 s against 64 / 23.8 s at
       1e-3, no gain below 1e-4) */
    double cg_rtol;
    /* the line search of a Newton step starts at min(1, step_growth * the
     * previous step) (default 4); 0: always at 1 */
    double step_growth;
} gbv_ot_options;

typedef struct {
    uint32_t converged;
    uint32_t newton_iters;
    uint32_t cg_iters;        /* total */
    uint32_t halvings;        /* damping steps of the line search */
    uint32_t cell_calls;      /* Laguerre diagrams computed */
    uint32_t levels;          /* 1, or the levels of gbv_ot_solve_levels */
    double mass_error_inf;    /* max_i |vol_i - nu_i| / nu_i at the end */
    double mass_error_l2;     /* ||vol - nu|| / ||nu|| at the end */
    double min_volume;
    double ms_total, ms_cells, ms_linear;
    /* the given start was multiplied by this so that every cell keeps at
     * least 1e-8 min(nu) (1: used as given, 0: replaced by zeros) */
    double start_scale;
    double ms_start;          /* learned start: features, network and solve */
    uint32_t start_cg_iters;  /* learned start: CG iterations of its solve */
    uint32_t reserved2;
} gbv_ot_report;

void gbv_ot_options_default(gbv_ot_options* opt);

/* Weights w such that every Laguerre cell of seed i (clipped to the box)
 * has volume nu_i (nu NULL: box volume / n each; sum nu must equal the box
 * volume).  w_inout holds the starting weights (zeros, or a warm start) and
 * receives the solution.  Host arrays; the report may be NULL. */
gbv_status gbv_ot_solve(gbv_context* ctx, const double* xyz, const double* nu, uint32_t n,
                        const gbv_ot_options* opt, double* w_inout, gbv_ot_report* report);

/* Multilevel solve, as optimize_levels in the reference's compute_OTM
 * (compute_OTM/main.cpp:292-294): nested random subsets of n / ratio^l
 * seeds (the coarsest at least min_level), each solved to a relative mass
 * error of max(tol, 1e-3) and the finest to tol; every level starts from
 * the coarser weights interpolated at its seeds (a Gaussian-weighted local
 * linear fit over the 16 nearest coarser seeds).  w_out: output only.
 * Totals in the report (newton_iters and the errors are the finest level's). */
gbv_status gbv_ot_solve_levels(gbv_context* ctx, const double* xyz, const double* nu, uint32_t n,
                               const gbv_ot_options* opt, uint32_t ratio, uint32_t min_level,
                               double* w_out, gbv_ot_report* report);
gbv_status gbv_ot_solve_levels_device(gbv_context* ctx, const double* d_xyz, const double* d_nu,
                                      uint32_t n, const gbv_ot_options* opt, uint32_t ratio,
                                      uint32_t min_level, double* d_w, void* stream,
                                      gbv_ot_report* report);

/* Same on device arrays, ordered on `stream` (NULL: the context's). */
gbv_status gbv_ot_solve_device(gbv_context* ctx, const double* d_xyz, const double* d_nu,
                               uint32_t n, const gbv_ot_options* opt, double* d_w_inout,
                               void* stream, gbv_ot_report* report);

/* The callback of OptimalTransportMap3d's optimiser at weights w: the
 * gradient g_i = nu_i - |Lag_i(w)| and the Hessian of the dual (CSR in
 * the caller's seed order, off-diagonal -A_ij / (2 |p_i - p_j|), diagonal
 * minus the row sum).  Host arrays.  Call with h_capacity = 0 to get *nnz;
 * GBV_ERR_CAPACITY when h_capacity < *nnz. */
gbv_status gbv_ot_gradient_hessian(gbv_context* ctx, const double* xyz, const double* w,
                                   const double* nu, uint32_t n, const gbv_ot_options* opt,
                                   double* g, uint32_t* h_rowptr, uint32_t* h_col,
                                   double* h_val, double* h_diag, uint64_t h_capacity,
                                   uint64_t* nnz);

/* ---------------------------------------------------------------- */
/* Learned warm start for gbv_ot_solve.  No counterpart in the        */
/* reference: the reference's solver starts from zero weights (or     */
/* from a coarser level).  A small MLP predicts each seed's weight    */
/* from its position and the distances to its 16 nearest seeds; its   */
/* forward and backward passes run on the tensor cores (BF16 in,      */
/* FP32 accumulation).  All pointers are device pointers.             */
/* ---------------------------------------------------------------- */

#define GBV_MLP_INPUTS 19
/* FP32 parameters: W1[128][32] (inputs padded to 32 columns, the padding
 * kept at zero), b1[128], W2[128][128], b2[128], W3[128][128], b3[128],
 * W4[128], b4 */
#define GBV_MLP_PARAMS 37377
/* normalisation: input mean[19], input std[19], output mean, output std */
#define GBV_MLP_NORM 40
/* rows per gbv_mlp_loss_grad call */
#define GBV_MLP_MAX_BATCH 65536u

/* Raw features [n][19] of the seeds d_xyz [n][3]: x, y, z, then the 16
 * nearest distances to other seeds times n^(1/3), ascending.  n >= 17. */
gbv_status gbv_mlp_features(gbv_context* ctx, const double* d_xyz, uint32_t n, float* d_raw,
                            void* stream);
/* Network output (standardised) for n rows of raw features. */
gbv_status gbv_mlp_forward(gbv_context* ctx, const float* d_params, const float* d_norm,
                           const float* d_raw, uint32_t n, float* d_y, void* stream);
/* Gradient (FP32, layout of the parameters) of the mean squared error
 * between the output and the standardised targets (d_target are weights;
 * the normalisation maps them); *loss receives the error.  n <=
 * GBV_MLP_MAX_BATCH. */
gbv_status gbv_mlp_loss_grad(gbv_context* ctx, const float* d_params, const float* d_norm,
                             const float* d_raw, const float* d_target, uint32_t n,
                             float* d_grad, double* loss, void* stream);
/* One Adam step (bias-corrected) on the parameters; step counts from 1. */
gbv_status gbv_mlp_adam(gbv_context* ctx, float* d_params, float* d_m, float* d_v,
                        const float* d_grad, uint32_t step, float lr, float beta1, float beta2,
                        float eps, void* stream);
/* The learned start: cells and Hessian H0 at zero weights, the network's
 * prediction of t_i = (H0 w*)_i / vol_i(0) (the cell-averaged Laplacian of
 * the optimal weights; by the Monge-Ampere relation a function of the local
 * density its inputs see), then w = H0^+ (t vol(0)) by conjugate gradient,
 * scaled toward zero if a cell would fall below 1e-8 min(nu).
 * d_w [n] receives the weights. */
gbv_status gbv_ot_warm_start(gbv_context* ctx, const double* d_xyz, uint32_t n,
                             const gbv_ot_options* opt, const float* d_params,
                             const float* d_norm, double* d_w, void* stream);
/* gbv_ot_solve_device from the learned start (d_w: output only). */
gbv_status gbv_ot_solve_learned_device(gbv_context* ctx, const double* d_xyz, const double* d_nu,
                                       uint32_t n, const gbv_ot_options* opt,
                                       const float* d_params, const float* d_norm, double* d_w,
                                       void* stream, gbv_ot_report* report);
/* Separable start (no reference counterpart: the reference's solver starts
 * from zero): w_i = |p_i|^2 - 2 sum_a Phi_a(p_ia), Phi_a' the piecewise-
 * linear empirical CDF of axis a mapped onto the box of opt (the seed of
 * rank k to box_min + (k + 1/2)/n (box_max - box_min)).  For distinct seeds
 * no cell of these weights is empty.  d_xyz [3n] device seeds, d_w [n]
 * receives the weights (not centred), 1 <= n <= 2^31. */
gbv_status gbv_ot_separable_start(gbv_context* ctx, const double* d_xyz, uint32_t n,
                                  const gbv_ot_options* opt, double* d_w, void* stream);
/* The tensor-core product the network uses, exposed for testing:
 * C[M][N] (FP32, ldc) = A[M][K] Bt[N][K]^T, A and Bt BF16 row-major, K a
 * multiple of 32, lda and ldb multiples of 8. */
gbv_status gbv_mlp_gemm_nt(gbv_context* ctx, const void* d_a, int lda, const void* d_bt,
                           int ldb, float* d_c, int ldc, int M, int N, int K, void* stream);

/* ---------------------------------------------------------------- */
/* Periodic cells                                                    */
/* ---------------------------------------------------------------- */

/* Replaces PeriodicDelaunay3d(periodic = true, period) with
 * copy_Laguerre_cell_from_Delaunay (delaunay/periodic_delaunay_3d.h:126-156,
 * periodic_delaunay_3d.cpp:3634-3734): the Laguerre cells of the seeds
 * xyz[3 n] (in [0, period)^3; weights w[n] or NULL) in the periodic cube.
 * opt gives k0 and precision (security-radius certification; its box is
 * ignored).  The cells are computed here and kept in the context; read
 * them with gbv_periodic_fetch (report->nnz facets). */
gbv_status gbv_periodic_cells(gbv_context* ctx, const double* xyz, const double* w, uint32_t n,
                              double period, const gbv_cell_options* opt,
                              gbv_cell_report* report);

/* The last periodic cells, host arrays (any may be NULL): vol[n], mg[3 n]
 * (about the seed's own position, which may lie outside the cube for a
 * cell that wraps), rowptr[n + 1], and per facet the seed across it
 * (nbr, an index < n), the translation of that seed's image as
 * shift = (tx + 1) * 9 + (ty + 1) * 3 + (tz + 1) with t in {-1, 0, 1}
 * periods (13: no translation; the reference's instance, translated by
 * Periodic::translation), and the facet area. */
gbv_status gbv_periodic_fetch(gbv_context* ctx, double* vol, double* mg, uint32_t* rowptr,
                              uint32_t* nbr, uint8_t* shift, double* area);

/* ---------------------------------------------------------------- */
/* Cells restricted to a tetrahedral mesh                            */
/* ---------------------------------------------------------------- */

/* Replaces RestrictedVoronoiDiagram with set_volumetric(true)
 * (voronoi/RVD.h:180) and its compute_centroids (RVD.h:284-290;
 * RVD.cpp:429-530) and compute_CVT_func_grad (RVD.h:295-320;
 * RVD.cpp:792-910): the cells of the seeds (Voronoi, or Laguerre with
 * weights w) restricted to the union of the tetrahedra, for CVT and optimal
 * transport on non-cube domains.  Host arrays: mesh_xyz[3 nv], tets[4 nt]
 * (vertex indices, any orientation), xyz[3 n], w[n] or NULL.  opt gives
 * k0, check_sr and precision; its box is replaced by the bounding box of
 * the mesh and the seeds.  Outputs (any may be NULL): m[n] and mg[3 n], the
 * mass and first moment of each restricted cell; *f and g[3 n], the CVT
 * energy sum_i int_{cell_i} |x - p_i|^2 and its gradient formed as the
 * reference forms them: cones from each seed to the border of its
 * restricted cell with unsigned volumes (for a cell star-shaped from its
 * seed, the exact integral and 2 (m_i p_i - mg_i)).  Afterwards the
 * context holds the unrestricted cells (gbv_cells_fetch). */
gbv_status gbv_restricted_cells(gbv_context* ctx, const double* mesh_xyz, uint32_t nv,
                                const uint32_t* tets, uint32_t nt, const double* xyz,
                                const double* w, uint32_t n, const gbv_cell_options* opt,
                                double* m, double* mg, double* f, double* g,
                                gbv_cell_report* report);

/* Replaces CentroidalVoronoiTesselation::Newton_iterations(nb_iter, m)
 * (voronoi/CVT.cpp:272-307) on a tetrahedral mesh: L-BFGS keeping m pairs
 * (the reference's HLBFGS with its default line search, epsg = epsf =
 * epsx = 0: nb_iter iterations unless the line search fails) on the CVT
 * energy and gradient of gbv_restricted_cells, evaluated on the GPU at
 * every step.  HLBFGS stops once its iteration count exceeds nb_iter, so
 * the reference takes nb_iter + 1 steps; so does this.  xyz[3 n] holds the
 * start and receives the result; opt gives k0 and precision (security
 * radius).  energy[nb_iter + 2] (or NULL): the energy at the start and
 * after each step; *iterations (or NULL): the steps done. */
gbv_status gbv_cvt_newton(gbv_context* ctx, const double* mesh_xyz, uint32_t nv,
                          const uint32_t* tets, uint32_t nt, double* xyz, uint32_t n,
                          const gbv_cell_options* opt, uint32_t nb_iter, uint32_t m,
                          double* energy, uint32_t* iterations);

/* ---------------------------------------------------------------- */
/* Cell polytopes (output formats)                                   */
/* ---------------------------------------------------------------- */

typedef struct {
    uint64_t n_vertices;       /* corners of the requested cells            */
    uint64_t n_faces;          /* polygons                                  */
    uint64_t n_face_vertices;  /* polygon entries (3 per corner)            */
} gbv_mesh_sizes;

/* Replaces ConvexCell::save / append_to_mesh (voronoi/convex_cell.cpp:
 * 282-352, 371-444) for the cells of the last compute on ctx: cells[0..m)
 * (original seed indices; NULL = every cell, m ignored).  Per cell, its
 * corners in the reference's order (the valid-triangle list; coordinates
 * bit-identical to compute_triangle_point / w) and one polygon per plane
 * that bounds it, in plane creation order (box faces, then the seeds in
 * clipping order), each walked as the reference walks it.  Host arrays:
 *   vertices[3 * n_vertices]       x, y, z of each corner, cell after cell
 *   cell_vertex_ptr[m + 1]         first corner of each cell
 *   cell_face_ptr[m + 1]           first polygon of each cell
 *   face_ptr[n_faces + 1]          first entry of each polygon
 *   face_vertices[n_face_vertices] corner numbers local to the cell
 *   face_seed[n_faces]             v_global_index of the plane: the seed
 *                                  across the face, 0xFFFFFFFF for the box
 * Call once with the arrays NULL to get *sizes, then with arrays of those
 * sizes (any may be NULL).  Cells beyond 128 corners return GBV_ERR_CAPACITY
 * (their polytope is not kept). */
gbv_status gbv_cells_mesh(gbv_context* ctx, const uint32_t* cells, uint32_t m,
                          gbv_mesh_sizes* sizes, double* vertices, uint32_t* cell_vertex_ptr,
                          uint32_t* cell_face_ptr, uint32_t* face_ptr, uint32_t* face_vertices,
                          uint32_t* face_seed);

/* ---------------------------------------------------------------- */
/* Allocation-free kNN                                               */
/* ---------------------------------------------------------------- */

/* Largest point count gbv_knn_noalloc accepts. */
#define GBV_NOALLOC_MAX_POINTS 32768u

/* No counterpart in the reference: an allocation-free variant of the kNN
 * search for callers that must not allocate GPU memory while they run
 * (code under a strict device-memory budget or using its own memory pool,
 * regions where an allocation's implicit synchronisation is not allowed,
 * latency-bound loops).  Same result as gbv_nn_set_points followed by
 * gbv_nn_get_nearest_neighbors_all: row i of d_idx / d_d2 (n rows of k)
 * holds the k nearest of point i, the point itself included, ascending
 * (d2, index).  All arrays are device pointers; the work is enqueued on
 * `stream` (a cudaStream_t, NULL = the legacy default stream) and the call
 * does not wait for it.  It calls no cudaMalloc or cudaFree: its scratch is
 * a fixed array inside the library (about 3.2 MB, held on every device that
 * loads the library until the process exits).  Limits: 1 <= n <=
 * GBV_NOALLOC_MAX_POINTS (larger n returns GBV_ERR_CAPACITY), dim 3 or 4,
 * stride >= dim doubles, 1 <= k <= min(n, 64).  The scratch is shared by
 * every call and keeps the last call's contents: calls whose work overlaps
 * on the GPU race and corrupt each other's results, so order them on one
 * stream.  Every call looks up the scratch's address in the current
 * context, so it stays right after cudaDeviceReset.  The first call in a
 * context loads the library's device code there, scratch included: that
 * load allocates the 3.2 MB and can synchronise, so make the first call on
 * each device outside any region that must not allocate, and before any
 * stream capture.  d_pts, d_idx and d_d2 must be device (or managed) memory
 * of the current device; anything else returns GBV_ERR_INVALID_ARGUMENT
 * before any work is enqueued. */
gbv_status gbv_knn_noalloc(const double* d_pts, uint32_t n, uint32_t dim, uint32_t stride,
                           uint32_t k, uint32_t* d_idx, double* d_d2, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBV_H */
