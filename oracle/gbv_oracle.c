/*
 * gbv_oracle.c -- CPU restatement of geogram's meshless Laguerre cell path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of the GPU kernels' tests and the timed
 * CPU baseline ("port") of bench.py.  Nothing in the product (the
 * geogram_gb300 package and its CUDA library) links, imports or calls it.
 *
 * Pinned against the reference itself: oracle/ref/Makefile compiles
 * geogram's BalancedKdTree and VBW::ConvexCell from the reference sources
 * into oracle/_ref/libgbv_ref.so, and tests/test_oracle_pin.py checks that
 * this file reproduces its kNN lists, neighbour lists, volumes, centroids
 * and facet areas bit for bit on seeded inputs (fixtures in tests/golden/).
 *
 * What is restated (reference file:line):
 *   kNN ........ KdTree::get_nearest_neighbors, kd_tree.cpp:156-387 (exact
 *                FP64 squared distance geometry_nd.h:65-73; ties here are
 *                ordered by point index)
 *   neighbours . Delaunay_NearestNeighbors::get_neighbors_internal,
 *                delaunay_nn.cpp:104-145
 *   cell ....... VBW::ConvexCell: init_with_box convex_cell.cpp:175-215,
 *                new_triangle convex_cell.h:1143-1166, clip_by_plane
 *                convex_cell.cpp:467-516, triangulate_conflict_zone :761-865,
 *                triangle_is_in_conflict (exact) :870-912,
 *                compute_triangle_point :971-1082, compute_geometry
 *                :1125-1145, facet_area :1160-1191, compute_mg :1267-1307,
 *                squared_radius :1312-1330
 *   SR loop .... clip_by_cell_SR, generic_RVD.h:2278-2352
 *   plane ...... power bisector, periodic_delaunay_3d.cpp:3722-3726
 *   lift ....... 4-d lift h_i = sqrt(W - w_i), compute_OTM/main.cpp:280-283
 *   exact sign . PCK::det_4d (predicates.cpp:2073-2110) is restated as a
 *                floating-point filter plus Shewchuk's expansion arithmetic
 *                (J. R. Shewchuk, "Adaptive Precision Floating-Point
 *                Arithmetic and Fast Robust Geometric Predicates", 1997):
 *                Two-Sum, Two-Product (via a correctly rounded fma), grow-
 *                and scale-expansion with zero elimination.
 *
 * Build with -ffp-contract=off (oracle/Makefile) so that a*b+c is never
 * fused and the results match on every host.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double x, y, z, w; } v4;
typedef struct { double x, y, z; } v3;

/* ------------------------------------------------------------------ */
/* Exact sign of a 4x4 determinant                                     */
/* ------------------------------------------------------------------ */

static void two_sum(double a, double b, double* x, double* y) {
    double s = a + b;
    double bv = s - a;
    double av = s - bv;
    *x = s;
    *y = (a - av) + (b - bv);
}

static void two_prod(double a, double b, double* x, double* y) {
    double p = a * b;
    *x = p;
    *y = fma(a, b, -p);
}

/* h = e + b; e nonoverlapping, increasing magnitude; returns length. */
static int grow_exp(int elen, const double* e, double b, double* h) {
    double q = b;
    int hn = 0;
    for (int i = 0; i < elen; ++i) {
        double qn, hh;
        two_sum(q, e[i], &qn, &hh);
        q = qn;
        if (hh != 0.0) h[hn++] = hh;
    }
    if (q != 0.0 || hn == 0) h[hn++] = q;
    return hn;
}

/* h = e + f by repeated growth; h must not alias e or f. */
static int sum_exp(int elen, const double* e, int flen, const double* f,
                   double* h, double* tmp) {
    int hn = elen;
    memcpy(h, e, sizeof(double) * (size_t)elen);
    for (int i = 0; i < flen; ++i) {
        hn = grow_exp(hn, h, f[i], tmp);
        memcpy(h, tmp, sizeof(double) * (size_t)hn);
    }
    return hn;
}

/* h = b * e; returns length. */
static int scale_exp(int elen, const double* e, double b, double* h) {
    int hn = 0;
    double q, hh;
    two_prod(e[0], b, &q, &hh);
    if (hh != 0.0) h[hn++] = hh;
    for (int i = 1; i < elen; ++i) {
        double p1, p0, s;
        two_prod(e[i], b, &p1, &p0);
        two_sum(q, p0, &s, &hh);
        if (hh != 0.0) h[hn++] = hh;
        two_sum(p1, s, &q, &hh);
        if (hh != 0.0) h[hn++] = hh;
    }
    if (q != 0.0 || hn == 0) h[hn++] = q;
    return hn;
}

static int exp_sign(int n, const double* e) {
    double top = e[n - 1];
    return (top > 0.0) - (top < 0.0);
}

/* 2x2 minor of rows r0, r1 on columns (a, b): r0[a] r1[b] - r0[b] r1[a]. */
static int minor2_exp(const double* r0, const double* r1, int a, int b, double* h) {
    double p[2], q[2], t[8];
    two_prod(r0[a], r1[b], &p[1], &p[0]);
    two_prod(-r0[b], r1[a], &q[1], &q[0]);
    int pn = (p[0] != 0.0) ? 2 : 1;
    double* pp = (p[0] != 0.0) ? p : &p[1];
    int qn = (q[0] != 0.0) ? 2 : 1;
    double* qq = (q[0] != 0.0) ? q : &q[1];
    return sum_exp(pn, pp, qn, qq, h, t);
}

/* Exact sign of det [p0; p1; p2; p3] (rows are 4-vectors). */
static int det4_exact_sign(const double* p0, const double* p1,
                           const double* p2, const double* p3) {
    double m[4][4][4];
    int mn[4][4];
    for (int a = 0; a < 4; ++a)
        for (int b = a + 1; b < 4; ++b) mn[a][b] = minor2_exp(p0, p1, a, b, m[a][b]);
    /* 3x3 minors of rows 0..2 on column triples (a<b<c), expanded along
     * row 2: p2[a] m_bc - p2[b] m_ac + p2[c] m_ab. */
    double d3[4][24];
    int d3n[4];
    static const int cols[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    for (int s = 0; s < 4; ++s) {
        int a = cols[s][0], b = cols[s][1], c = cols[s][2];
        double t1[8], t2[8], t3[8], u[16], tmp[32];
        int n1 = scale_exp(mn[b][c], m[b][c], p2[a], t1);
        int n2 = scale_exp(mn[a][c], m[a][c], -p2[b], t2);
        int n3 = scale_exp(mn[a][b], m[a][b], p2[c], t3);
        int nu = sum_exp(n1, t1, n2, t2, u, tmp);
        d3n[s] = sum_exp(nu, u, n3, t3, d3[s], tmp);
    }
    /* Expand along row 3 with signs (-, +, -, +). */
    double acc[192], nxt[192], term[48], tmp[192];
    int an = 1;
    acc[0] = 0.0;
    for (int s = 0; s < 4; ++s) {
        double f = (s % 2 == 0) ? -p3[s] : p3[s];
        int tn = scale_exp(d3n[s], d3[s], f, term);
        an = sum_exp(an, acc, tn, term, nxt, tmp);
        memcpy(acc, nxt, sizeof(double) * (size_t)an);
    }
    return exp_sign(an, acc);
}

/* Sign of det [p0; p1; p2; p3]: a floating-point evaluation whose error
 * is bounded by 2^-48 times the permanent of |entries| (a generous bound
 * for the 9 rounding levels of the cofactor evaluation), then the exact
 * expansion when the filter cannot decide. */
static int det4_sign(const double* p0, const double* p1, const double* p2,
                     const double* p3, long* n_exact) {
    double m[4][4], pm[4][4];
    for (int a = 0; a < 4; ++a)
        for (int b = a + 1; b < 4; ++b) {
            m[a][b] = p0[a] * p1[b] - p0[b] * p1[a];
            pm[a][b] = fabs(p0[a] * p1[b]) + fabs(p0[b] * p1[a]);
        }
    static const int cols[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    double det = 0.0, perm = 0.0;
    for (int s = 0; s < 4; ++s) {
        int a = cols[s][0], b = cols[s][1], c = cols[s][2];
        double d3 = p2[a] * m[b][c] - p2[b] * m[a][c] + p2[c] * m[a][b];
        double q3 = fabs(p2[a]) * pm[b][c] + fabs(p2[b]) * pm[a][c] + fabs(p2[c]) * pm[a][b];
        double f = (s % 2 == 0) ? -p3[s] : p3[s];
        det += f * d3;
        perm += fabs(f) * q3;
    }
    double bound = perm * 0x1p-48;
    if (det > bound) return 1;
    if (det < -bound) return -1;
    if (perm == 0.0) return 0;
    if (n_exact) ++*n_exact;
    return det4_exact_sign(p0, p1, p2, p3);
}

/* Exported for the tests: exact sign of det [p0;p1;p2;p3]. */
int orc_det4_sign(const double* p0, const double* p1, const double* p2,
                  const double* p3) {
    return det4_sign(p0, p1, p2, p3, NULL);
}

/* ------------------------------------------------------------------ */
/* The convex cell (dual form: planes are vertices, corners triangles) */
/* ------------------------------------------------------------------ */

enum { CONFLICT_MASK = 32768, END_OF_LIST = 16383 };

typedef struct { uint16_t i, j, k, flags; } tri_t;
typedef struct { uint16_t i, j, k; } adj_t;

typedef struct {
    int max_t, max_v, nb_t, nb_v;
    int first_free, first_valid;
    tri_t* t;
    adj_t* adj;
    v4* plane;
    uint32_t* vglobal;
    uint16_t* v2t;
    uint8_t* v2e;
    v3* tpoint;
    long n_exact;
} cell_t;

static void cell_init(cell_t* C) {
    memset(C, 0, sizeof(*C));
    C->max_t = 64;
    C->max_v = 32;
    C->t = (tri_t*)calloc((size_t)C->max_t, sizeof(tri_t));
    C->adj = (adj_t*)calloc((size_t)C->max_t, sizeof(adj_t));
    C->tpoint = (v3*)calloc((size_t)C->max_t, sizeof(v3));
    C->plane = (v4*)calloc((size_t)C->max_v, sizeof(v4));
    C->vglobal = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)C->max_v);
    C->v2t = (uint16_t*)malloc(sizeof(uint16_t) * (size_t)C->max_v);
    C->v2e = (uint8_t*)malloc((size_t)C->max_v);
    for (int v = 0; v < C->max_v; ++v) {
        C->vglobal[v] = 0xFFFFFFFFu;
        C->v2t[v] = 0xFFFF;
        C->v2e[v] = 0xFF;
    }
}

static void cell_free(cell_t* C) {
    free(C->t); free(C->adj); free(C->tpoint); free(C->plane);
    free(C->vglobal); free(C->v2t); free(C->v2e);
}

static void grow_v(cell_t* C) {
    int old = C->max_v;
    C->max_v *= 2;
    C->plane = (v4*)realloc(C->plane, sizeof(v4) * (size_t)C->max_v);
    C->vglobal = (uint32_t*)realloc(C->vglobal, sizeof(uint32_t) * (size_t)C->max_v);
    C->v2t = (uint16_t*)realloc(C->v2t, sizeof(uint16_t) * (size_t)C->max_v);
    C->v2e = (uint8_t*)realloc(C->v2e, (size_t)C->max_v);
    for (int v = old; v < C->max_v; ++v) {
        C->vglobal[v] = 0xFFFFFFFFu;
        C->v2t[v] = 0xFFFF;
        C->v2e[v] = 0xFF;
    }
}

static void grow_t(cell_t* C) {
    C->max_t *= 2;
    C->t = (tri_t*)realloc(C->t, sizeof(tri_t) * (size_t)C->max_t);
    C->adj = (adj_t*)realloc(C->adj, sizeof(adj_t) * (size_t)C->max_t);
    C->tpoint = (v3*)realloc(C->tpoint, sizeof(v3) * (size_t)C->max_t);
}

static int new_triangle(cell_t* C, int i, int j, int k) {
    int r = C->first_free;
    if (r == END_OF_LIST) {
        r = C->nb_t;
        ++C->nb_t;
        if (C->nb_t > C->max_t) grow_t(C);
    } else {
        C->first_free = C->t[C->first_free].flags & ~CONFLICT_MASK;
    }
    C->t[r].i = (uint16_t)i;
    C->t[r].j = (uint16_t)j;
    C->t[r].k = (uint16_t)k;
    C->t[r].flags = (uint16_t)C->first_valid;
    C->first_valid = r;
    return r;
}

static void new_triangle_adj(cell_t* C, int i, int j, int k, int a0, int a1, int a2) {
    int r = new_triangle(C, i, j, k);
    C->adj[r].i = (uint16_t)a0;
    C->adj[r].j = (uint16_t)a1;
    C->adj[r].k = (uint16_t)a2;
}

static void init_with_box(cell_t* C, double xmin, double ymin, double zmin,
                          double xmax, double ymax, double zmax) {
    C->nb_t = 0;
    C->nb_v = 0;
    C->first_free = END_OF_LIST;
    C->first_valid = END_OF_LIST;
    C->plane[0] = (v4){0, 0, 0, 0};
    C->plane[1] = (v4){1.0, 0.0, 0.0, -xmin};
    C->plane[2] = (v4){-1.0, 0.0, 0.0, xmax};
    C->plane[3] = (v4){0.0, 1.0, 0.0, -ymin};
    C->plane[4] = (v4){0.0, -1.0, 0.0, ymax};
    C->plane[5] = (v4){0.0, 0.0, 1.0, -zmin};
    C->plane[6] = (v4){0.0, 0.0, -1.0, zmax};
    for (int v = 0; v < 7; ++v) C->vglobal[v] = 0xFFFFFFFFu;
    /* The 8 box corners, as triangles of the 6 face planes. */
    new_triangle_adj(C, 3, 6, 1, 1, 4, 2);
    new_triangle_adj(C, 6, 4, 1, 5, 0, 3);
    new_triangle_adj(C, 2, 6, 3, 0, 6, 3);
    new_triangle_adj(C, 6, 2, 4, 7, 1, 2);
    new_triangle_adj(C, 5, 3, 1, 0, 5, 6);
    new_triangle_adj(C, 5, 1, 4, 1, 7, 4);
    new_triangle_adj(C, 3, 5, 2, 7, 2, 4);
    new_triangle_adj(C, 5, 4, 2, 3, 6, 5);
    C->nb_v = 7;
}

static int tri_vertex(const cell_t* C, int t, int lv) {
    return lv == 0 ? C->t[t].i : (lv == 1 ? C->t[t].j : C->t[t].k);
}
static int tri_adjacent(const cell_t* C, int t, int le) {
    return le == 0 ? C->adj[t].i : (le == 1 ? C->adj[t].j : C->adj[t].k);
}
static void set_tri_adjacent(cell_t* C, int t, int le, int a) {
    if (le == 0) C->adj[t].i = (uint16_t)a;
    else if (le == 1) C->adj[t].j = (uint16_t)a;
    else C->adj[t].k = (uint16_t)a;
}
static int tri_find_vertex(const cell_t* C, int t, int v) {
    return (C->t[t].j == v) + 2 * (C->t[t].k == v);
}
static int is_conflict(const cell_t* C, int t) {
    return (C->t[t].flags & CONFLICT_MASK) != 0;
}

/* Exact mode only (all triangles of a box-initialised cell are finite). */
static int triangle_in_conflict(cell_t* C, int t, v4 eqn, int exact) {
    v4 p1 = C->plane[C->t[t].i], p2 = C->plane[C->t[t].j], p3 = C->plane[C->t[t].k];
    if (exact) {
        return det4_sign(&p1.x, &p2.x, &p3.x, &eqn.x, &C->n_exact) >= 0;
    }
    /* Fast mode: det4x4 of convex_cell.h:383-402 evaluated as written. */
    double a11 = p1.x, a12 = p2.x, a13 = p3.x, a14 = eqn.x;
    double a21 = p1.y, a22 = p2.y, a23 = p3.y, a24 = eqn.y;
    double a31 = p1.z, a32 = p2.z, a33 = p3.z, a34 = eqn.z;
    double a41 = p1.w, a42 = p2.w, a43 = p3.w, a44 = eqn.w;
    double m12 = a21 * a12 - a11 * a22;
    double m13 = a31 * a12 - a11 * a32;
    double m14 = a41 * a12 - a11 * a42;
    double m23 = a31 * a22 - a21 * a32;
    double m24 = a41 * a22 - a21 * a42;
    double m34 = a41 * a32 - a31 * a42;
    double m123 = m23 * a13 - m13 * a23 + m12 * a33;
    double m124 = m24 * a13 - m14 * a23 + m12 * a43;
    double m134 = m34 * a13 - m14 * a33 + m13 * a43;
    double m234 = m34 * a23 - m24 * a33 + m23 * a43;
    double det = m234 * a14 - m134 * a24 + m124 * a34 - m123 * a44;
    return det > 0.0;
}

static void triangulate_conflict_zone(cell_t* C, int lv, int head, int tail) {
    if (head == END_OF_LIST) return;
    int first_v = END_OF_LIST;
    for (int t = C->first_valid; t != END_OF_LIST; t = C->t[t].flags) {
        if (is_conflict(C, tri_adjacent(C, t, 0))) {
            first_v = tri_vertex(C, t, 1);
            C->v2t[first_v] = (uint16_t)t;
            C->v2e[first_v] = 0;
        }
        if (is_conflict(C, tri_adjacent(C, t, 1))) {
            first_v = tri_vertex(C, t, 2);
            C->v2t[first_v] = (uint16_t)t;
            C->v2e[first_v] = 1;
        }
        if (is_conflict(C, tri_adjacent(C, t, 2))) {
            first_v = tri_vertex(C, t, 0);
            C->v2t[first_v] = (uint16_t)t;
            C->v2e[first_v] = 2;
        }
    }
    if (first_v != END_OF_LIST) {
        int v = first_v;
        int prev_new = -1, first_new = -1;
        do {
            int t = C->v2t[v];
            int e = C->v2e[v];
            int v2 = tri_vertex(C, t, (e + 2) % 3);
            int nt = new_triangle(C, lv, v2, v);
            set_tri_adjacent(C, nt, 0, t);
            set_tri_adjacent(C, t, e, nt);
            if (prev_new == -1) {
                first_new = nt;
            } else {
                set_tri_adjacent(C, prev_new, 2, nt);
                set_tri_adjacent(C, nt, 1, prev_new);
            }
            prev_new = nt;
            v = v2;
        } while (v != first_v);
        set_tri_adjacent(C, prev_new, 2, first_new);
        set_tri_adjacent(C, first_new, 1, prev_new);
    }
    C->t[tail].flags = (uint16_t)C->first_free;
    C->first_free = head;
}

static void clip_by_plane(cell_t* C, v4 eqn, uint32_t j, int exact) {
    int lv = C->nb_v;
    if (lv == C->max_v) grow_v(C);
    C->plane[lv] = eqn;
    ++C->nb_v;
    int head = END_OF_LIST, tail = END_OF_LIST;
    int t = C->first_valid;
    C->first_valid = END_OF_LIST;
    while (t != END_OF_LIST) {
        int next = C->t[t].flags;
        if (triangle_in_conflict(C, t, eqn, exact)) {
            C->t[t].flags = (uint16_t)(head | CONFLICT_MASK);
            head = t;
            if (tail == END_OF_LIST) tail = t;
        } else {
            C->t[t].flags = (uint16_t)C->first_valid;
            C->first_valid = t;
        }
        t = next;
    }
    if (head == END_OF_LIST) {
        /* The plane cuts nothing.  The reference keeps it as an unused
         * vertex (convex_cell.cpp:467-476); no triangle refers to it and the
         * facets are read in insertion order, so dropping it changes no
         * output, and it keeps the 16-bit plane indices of the triangles
         * (convex_cell.h:309-321) from wrapping in cells clipped by more
         * than 65535 neighbours. */
        --C->nb_v;
        return;
    }
    triangulate_conflict_zone(C, lv, head, tail);
    C->vglobal[lv] = j;
}

static double det2x2(double a11, double a12, double a21, double a22) {
    return a11 * a22 - a12 * a21;
}
static double det3x3(double a11, double a12, double a13, double a21, double a22,
                     double a23, double a31, double a32, double a33) {
    return a11 * det2x2(a22, a23, a32, a33) - a21 * det2x2(a12, a13, a32, a33) +
           a31 * det2x2(a12, a13, a22, a23);
}

static v4 triangle_point(const cell_t* C, int t) {
    v4 a = C->plane[C->t[t].i], b = C->plane[C->t[t].j], c = C->plane[C->t[t].k];
    v4 r;
    r.x = -det3x3(a.w, a.y, a.z, b.w, b.y, b.z, c.w, c.y, c.z);
    r.y = -det3x3(a.x, a.w, a.z, b.x, b.w, b.z, c.x, c.w, c.z);
    r.z = -det3x3(a.x, a.y, a.w, b.x, b.y, b.w, c.x, c.y, c.w);
    r.w = det3x3(a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z);
    return r;
}

static double squared_radius(const cell_t* C, v3 c) {
    double r = 0.0;
    for (int t = C->first_valid; t != END_OF_LIST; t = C->t[t].flags) {
        v4 p = triangle_point(C, t);
        double dx = p.x / p.w - c.x, dy = p.y / p.w - c.y, dz = p.z / p.w - c.z;
        double d = dx * dx + dy * dy + dz * dz;
        if (r < d) r = d;
    }
    return r;
}

static void compute_geometry(cell_t* C) {
    for (int v = 0; v < C->max_v; ++v) C->v2t[v] = END_OF_LIST;
    for (int t = C->first_valid; t != END_OF_LIST; t = C->t[t].flags) {
        v4 p = triangle_point(C, t);
        C->tpoint[t] = (v3){p.x / p.w, p.y / p.w, p.z / p.w};
        C->v2t[C->t[t].i] = (uint16_t)t;
        C->v2t[C->t[t].j] = (uint16_t)t;
        C->v2t[C->t[t].k] = (uint16_t)t;
    }
}

static double triangle_area(v3 p1, v3 p2, v3 p3) {
    double Ux = p2.x - p1.x, Uy = p2.y - p1.y, Uz = p2.z - p1.z;
    double Vx = p3.x - p1.x, Vy = p3.y - p1.y, Vz = p3.z - p1.z;
    double Wx = Uy * Vz - Uz * Vy, Wy = Uz * Vx - Ux * Vz, Wz = Ux * Vy - Uy * Vx;
    return 0.5 * sqrt(Wx * Wx + Wy * Wy + Wz * Wz);
}

static double tet_volume(v3 p1, v3 p2, v3 p3, v3 p4) {
    double Ux = p2.x - p1.x, Uy = p2.y - p1.y, Uz = p2.z - p1.z;
    double Vx = p3.x - p1.x, Vy = p3.y - p1.y, Vz = p3.z - p1.z;
    double Wx = p4.x - p1.x, Wy = p4.y - p1.y, Wz = p4.z - p1.z;
    double UVx = Uy * Vz - Uz * Vy, UVy = Uz * Vx - Ux * Vz, UVz = Ux * Vy - Uy * Vx;
    return fabs(UVx * Wx + UVy * Wy + UVz * Wz) / 6.0;
}

static double facet_area(const cell_t* C, int v) {
    int t1t2[2] = {0, 0};
    int cur = 0;
    double r = 0.0;
    if (C->v2t[v] != END_OF_LIST) {
        int t = C->v2t[v];
        do {
            if (cur < 2) {
                t1t2[cur] = t;
            } else {
                r += triangle_area(C->tpoint[t1t2[0]], C->tpoint[t1t2[1]], C->tpoint[t]);
                t1t2[1] = t;
            }
            ++cur;
            int lv = tri_find_vertex(C, t, v);
            t = tri_adjacent(C, t, (lv + 1) % 3);
        } while (t != C->v2t[v]);
    }
    return r;
}

static void compute_mg(const cell_t* C, double* m, v3* g) {
    *m = 0.0;
    *g = (v3){0.0, 0.0, 0.0};
    int t_origin = END_OF_LIST;
    for (int v = 0; v < C->nb_v; ++v) {
        if (C->v2t[v] == END_OF_LIST) continue;
        if (t_origin == END_OF_LIST) {
            t_origin = C->v2t[v];
            continue;
        }
        int t1t2[2] = {0, 0};
        int cur = 0;
        int t = C->v2t[v];
        do {
            if (cur < 2) {
                t1t2[cur] = t;
            } else {
                v3 p = C->tpoint[t_origin], q = C->tpoint[t1t2[0]];
                v3 r = C->tpoint[t1t2[1]], s = C->tpoint[t];
                double cm = tet_volume(p, q, r, s);
                *m += cm;
                g->x += cm * (p.x + q.x + r.x + s.x) / 4.0;
                g->y += cm * (p.y + q.y + r.y + s.y) / 4.0;
                g->z += cm * (p.z + q.z + r.z + s.z) / 4.0;
                t1t2[1] = t;
            }
            ++cur;
            int lv = tri_find_vertex(C, t, v);
            t = tri_adjacent(C, t, (lv + 1) % 3);
        } while (t != C->v2t[v]);
    }
}

/* ------------------------------------------------------------------ */
/* kNN: uniform grid over the first three coordinates, exact FP64      */
/* distances in all `dim` coordinates, ties ordered by point index.    */
/* ------------------------------------------------------------------ */

typedef struct {
    const double* pts;
    unsigned dim, n, G;
    double lo[3], h;
    uint32_t* start;  /* G^3 + 1 */
    uint32_t* items;  /* n */
} grid_t;

static int gclamp(long v, int G) { return v < 0 ? 0 : (v >= G ? G - 1 : (int)v); }

static void grid_build(grid_t* g, const double* pts, unsigned dim, unsigned n) {
    g->pts = pts;
    g->dim = dim;
    g->n = n;
    double lo[3] = {pts[0], pts[1], pts[2]}, hi[3] = {pts[0], pts[1], pts[2]};
    for (unsigned i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            double v = pts[(size_t)i * dim + c];
            if (v < lo[c]) lo[c] = v;
            if (v > hi[c]) hi[c] = v;
        }
    double ext = fmax(hi[0] - lo[0], fmax(hi[1] - lo[1], hi[2] - lo[2]));
    if (ext <= 0.0) ext = 1.0;
    unsigned G = (unsigned)cbrt((double)n / 2.0);
    if (G < 1) G = 1;
    if (G > 256) G = 256;
    g->G = G;
    g->h = ext / G * (1.0 + 1e-9);
    for (int c = 0; c < 3; ++c) g->lo[c] = lo[c];
    size_t nc = (size_t)G * G * G;
    g->start = (uint32_t*)calloc(nc + 1, sizeof(uint32_t));
    g->items = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    uint32_t* cid = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    for (unsigned i = 0; i < n; ++i) {
        int c3[3];
        for (int c = 0; c < 3; ++c)
            c3[c] = gclamp((long)floor((pts[(size_t)i * dim + c] - lo[c]) / g->h), (int)G);
        cid[i] = (uint32_t)(((size_t)c3[2] * G + c3[1]) * G + c3[0]);
        g->start[cid[i] + 1]++;
    }
    for (size_t c = 0; c < nc; ++c) g->start[c + 1] += g->start[c];
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * nc);
    memcpy(fill, g->start, sizeof(uint32_t) * nc);
    for (unsigned i = 0; i < n; ++i) g->items[fill[cid[i]]++] = i;
    free(fill);
    free(cid);
}

static void grid_free(grid_t* g) { free(g->start); free(g->items); }

static double dist2(const double* a, const double* b, unsigned dim) {
    double r = 0.0;
    for (unsigned c = 0; c < dim; ++c) r += (b[c] - a[c]) * (b[c] - a[c]);
    return r;
}

/* k nearest of point q (index qi) among all points, self included,
 * ascending (d2, index). */
static void grid_knn(const grid_t* g, const double* q, unsigned k, uint32_t* idx,
                     double* d2) {
    unsigned cnt = 0;
    int G = (int)g->G;
    int qc[3];
    for (int c = 0; c < 3; ++c) qc[c] = gclamp((long)floor((q[c] - g->lo[c]) / g->h), G);
    for (int r = 0;; ++r) {
        for (int z = qc[2] - r; z <= qc[2] + r; ++z) {
            if (z < 0 || z >= G) continue;
            for (int y = qc[1] - r; y <= qc[1] + r; ++y) {
                if (y < 0 || y >= G) continue;
                for (int x = qc[0] - r; x <= qc[0] + r; ++x) {
                    if (x < 0 || x >= G) continue;
                    if (abs(x - qc[0]) != r && abs(y - qc[1]) != r && abs(z - qc[2]) != r) continue;
                    size_t cell = ((size_t)z * G + y) * G + x;
                    for (uint32_t s = g->start[cell]; s < g->start[cell + 1]; ++s) {
                        uint32_t j = g->items[s];
                        double d = dist2(q, g->pts + (size_t)j * g->dim, g->dim);
                        if (cnt == k && (d > d2[k - 1] || (d == d2[k - 1] && j > idx[k - 1]))) continue;
                        int pos = (cnt < k) ? (int)cnt : (int)k - 1;
                        while (pos > 0 && (d2[pos - 1] > d || (d2[pos - 1] == d && idx[pos - 1] > j))) {
                            d2[pos] = d2[pos - 1];
                            idx[pos] = idx[pos - 1];
                            --pos;
                        }
                        d2[pos] = d;
                        idx[pos] = j;
                        if (cnt < k) ++cnt;
                    }
                }
            }
        }
        if (qc[0] - r <= 0 && qc[1] - r <= 0 && qc[2] - r <= 0 && qc[0] + r >= G - 1 &&
            qc[1] + r >= G - 1 && qc[2] + r >= G - 1)
            break; /* whole grid visited */
        if (cnt == k) {
            double b = INFINITY;
            for (int c = 0; c < 3; ++c) {
                double lo = g->lo[c] + (qc[c] - r) * g->h, hi = g->lo[c] + (qc[c] + r + 1) * g->h;
                if (qc[c] - r > 0) b = fmin(b, q[c] - lo);
                if (qc[c] + r < G - 1) b = fmin(b, hi - q[c]);
            }
            if (b > 0.0 && d2[k - 1] < b * b * (1.0 - 1e-12)) break;
        }
    }
}

/* ------------------------------------------------------------------ */
/* Threading                                                           */
/* ------------------------------------------------------------------ */

typedef void (*range_fn)(void* ctx, unsigned b, unsigned e);
typedef struct { range_fn fn; void* ctx; unsigned n; unsigned* next; } job_t;

static void* job_main(void* arg) {
    job_t* j = (job_t*)arg;
    for (;;) {
        unsigned b = __atomic_fetch_add(j->next, 128u, __ATOMIC_RELAXED);
        if (b >= j->n) break;
        unsigned e = b + 128u < j->n ? b + 128u : j->n;
        j->fn(j->ctx, b, e);
    }
    return NULL;
}

static void run_parallel_range(range_fn fn, void* ctx, unsigned b0, unsigned n, int nthreads) {
    if (nthreads <= 1 || n - b0 < 256) {
        fn(ctx, b0, n);
        return;
    }
    unsigned next = b0;
    job_t job = {fn, ctx, n, &next};
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, job_main, &job);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
}

static void run_parallel(range_fn fn, void* ctx, unsigned n, int nthreads) {
    if (nthreads <= 1 || n < 256) {
        fn(ctx, 0, n);
        return;
    }
    unsigned next = 0;
    job_t job = {fn, ctx, n, &next};
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, job_main, &job);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
}

/* ------------------------------------------------------------------ */
/* Public entry points                                                 */
/* ------------------------------------------------------------------ */

typedef struct { grid_t* g; unsigned k; uint32_t* idx; double* d2; } knn_ctx;

static void knn_range(void* vctx, unsigned b, unsigned e) {
    knn_ctx* c = (knn_ctx*)vctx;
    for (unsigned i = b; i < e; ++i)
        grid_knn(c->g, c->g->pts + (size_t)i * c->g->dim, c->k, c->idx + (size_t)i * c->k,
                 c->d2 + (size_t)i * c->k);
}

/* k nearest neighbours of every point (self included), ascending (d2, idx). */
int orc_knn(const double* pts, unsigned dim, unsigned n, unsigned k, uint32_t* idx,
            double* d2, int nthreads) {
    if (dim < 3 || k > n || n == 0) return 1;
    grid_t g;
    grid_build(&g, pts, dim, n);
    knn_ctx c = {&g, k, idx, d2};
    run_parallel(knn_range, &c, n, nthreads);
    grid_free(&g);
    return 0;
}

typedef struct {
    const double* xyz;
    const double* w;
    const double* pts;
    const double* hl;
    unsigned dim, n, k0, max_nbr;
    int check_sr, exact;
    grid_t* g;
    double* vol;
    double* mg;
    uint32_t *nbr_count, *nbr_idx, *k_list, *n_clip;
    double* nbr_area;
    int* status;
    long n_exact;
    unsigned off;  /* outputs of seed i go to index i - off */
} cells_ctx;

/* Neighbour list of seed i (delaunay_nn.cpp:104-145). */
static unsigned seed_neighbours(const cells_ctx* c, unsigned i, unsigned nb,
                                uint32_t* ix, double* dd, uint32_t* out) {
    nb = nb + 1 < c->n ? nb + 1 : c->n;
    grid_knn(c->g, c->pts + (size_t)i * c->dim, nb, ix, dd);
    unsigned m = 0;
    for (unsigned j = 0; j < nb; ++j) {
        if (ix[j] == i) continue;
        if (dd[j] == 0.0) {
            if (ix[j] < i) return 0;
            continue;
        }
        out[m++] = ix[j];
        if (m == nb - 1) break;
    }
    return m;
}

static void cells_range(void* vctx, unsigned b, unsigned e) {
    cells_ctx* c = (cells_ctx*)vctx;
    cell_t C;
    cell_init(&C);
    /* room for the first request (k0 + 1 points) and then some */
    unsigned cap = c->k0 + 2 > 64 ? c->k0 + 2 : 64;
    uint32_t* ix = (uint32_t*)malloc(sizeof(uint32_t) * (cap + 1));
    double* dd = (double*)malloc(sizeof(double) * (cap + 1));
    uint32_t* nb = (uint32_t*)malloc(sizeof(uint32_t) * (cap + 1));
    const unsigned n = c->n;
    for (unsigned i = b; i < e; ++i) {
        const double* xi = c->xyz + 3 * (size_t)i;
        const double* pi = c->pts + (size_t)i * c->dim;
        const double wi = c->w ? c->w[i] : 0.0;
        const double pi_len2 = xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2];
        init_with_box(&C, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0);
        int st = 1;
        unsigned jj = 0, prev = 0;
        unsigned req = c->k0 < n - 1 ? c->k0 : n - 1;
        unsigned list = seed_neighbours(c, i, req, ix, dd, nb);
        int done = 0;
        while (!done) {
            if (list == 0) { st = 2; break; }
            if (prev == list) { st = 3; break; }
            for (; jj < list; ++jj) {
                /* Beyond the 16-bit indices (65535 planes; triangle links
                 * below END_OF_LIST, and one clip at most doubles the
                 * triangles): status 5, the cell as clipped so far. */
                if (C.nb_v >= 65534 || C.nb_t >= END_OF_LIST / 2) { st = 5; done = 1; break; }
                uint32_t j = nb[jj];
                double R2 = squared_radius(&C, (v3){xi[0], xi[1], xi[2]});
                if (c->dim == 4) R2 += c->hl[i] * c->hl[i];
                double dij = dist2(pi, c->pts + (size_t)j * c->dim, c->dim);
                if (c->check_sr && dij > 4.1 * R2) { st = 0; done = 1; break; }
                const double* xj = c->xyz + 3 * (size_t)j;
                const double wj = c->w ? c->w[j] : 0.0;
                const double pj_len2 = xj[0] * xj[0] + xj[1] * xj[1] + xj[2] * xj[2];
                v4 P = {2.0 * (xi[0] - xj[0]), 2.0 * (xi[1] - xj[1]), 2.0 * (xi[2] - xj[2]),
                        (wi - pi_len2) - (wj - pj_len2)};
                clip_by_plane(&C, P, j, c->exact);
            }
            if (done) break;
            if (!c->check_sr) { st = 0; break; }
            if (list >= n - 1) { st = 1; break; }
            prev = list;
            unsigned want = list > 8 ? list + list / 8 : list + 1;
            if (want > n - 1) want = n - 1;
            if (want + 1 > cap) {
                cap = 2 * (want + 1);
                ix = (uint32_t*)realloc(ix, sizeof(uint32_t) * (cap + 1));
                dd = (double*)realloc(dd, sizeof(double) * (cap + 1));
                nb = (uint32_t*)realloc(nb, sizeof(uint32_t) * (cap + 1));
            }
            list = seed_neighbours(c, i, want, ix, dd, nb);
        }
        compute_geometry(&C);
        double m;
        v3 g;
        compute_mg(&C, &m, &g);
        const size_t o = (size_t)(i - c->off);
        c->vol[o] = m;
        c->mg[3 * o] = g.x;
        c->mg[3 * o + 1] = g.y;
        c->mg[3 * o + 2] = g.z;
        unsigned cnt = 0;
        for (int v = 1; v < C.nb_v; ++v) {
            if (C.v2t[v] == END_OF_LIST) continue;
            uint32_t j = C.vglobal[v];
            if (j == 0xFFFFFFFFu) continue;
            if (cnt < c->max_nbr) {
                c->nbr_idx[o * c->max_nbr + cnt] = j;
                c->nbr_area[o * c->max_nbr + cnt] = facet_area(&C, v);
            }
            ++cnt;
        }
        if (cnt > c->max_nbr && st != 5) st = 4;
        c->nbr_count[o] = cnt;
        c->k_list[o] = list;
        c->n_clip[o] = jj;
        c->status[o] = st;
    }
    __atomic_fetch_add(&c->n_exact, C.n_exact, __ATOMIC_RELAXED);
    free(ix);
    free(dd);
    free(nb);
    cell_free(&C);
}

/* Seeds, their 4-d lift and the grid, built once for any number of cell
 * ranges (the reference builds its kd-tree once per point set too). */
typedef struct {
    const double* xyz;
    const double* w;
    double* pts;
    double* hl;
    unsigned dim, n;
    grid_t g;
} prepared_t;

void* orc_cells_prepare(const double* xyz, const double* w, unsigned n) {
    if (n < 2) return NULL;
    prepared_t* p = (prepared_t*)calloc(1, sizeof(prepared_t));
    unsigned dim = w ? 4u : 3u;
    p->xyz = xyz;
    p->w = w;
    p->dim = dim;
    p->n = n;
    p->pts = (double*)malloc(sizeof(double) * (size_t)n * dim);
    p->hl = (double*)calloc(n, sizeof(double));
    if (w) {
        double W = w[0];
        for (unsigned i = 1; i < n; ++i) W = w[i] > W ? w[i] : W;
        for (unsigned i = 0; i < n; ++i) p->hl[i] = sqrt(W - w[i]);
    }
    for (unsigned i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) p->pts[(size_t)i * dim + c] = xyz[3 * (size_t)i + c];
        if (dim == 4) p->pts[(size_t)i * dim + 3] = p->hl[i];
    }
    grid_build(&p->g, p->pts, dim, n);
    return p;
}

void orc_cells_release(void* h) {
    prepared_t* p = (prepared_t*)h;
    if (!p) return;
    grid_free(&p->g);
    free(p->pts);
    free(p->hl);
    free(p);
}

/* Cells of seeds [i0, i1) of a prepared seed set (all n seeds take part
 * as neighbours); outputs are indexed i - i0.  Same per-seed contract as
 * ref_cells in oracle/ref/ref_harness.cpp.  *n_exact receives the number
 * of exact (expansion) predicate evaluations.  status: 0 certified, 1
 * every seed used, 2 duplicate, 3 list growth stalled, 4 more facets than
 * max_nbr, 5 beyond the 16-bit plane / triangle indices of the
 * reference's cell (the cell as clipped until then). */
int orc_cells_prepared_range(void* h, unsigned i0, unsigned i1, unsigned k0, int check_sr,
                             int exact, int nthreads, double* vol, double* mg,
                             uint32_t* nbr_count, uint32_t* nbr_idx, double* nbr_area,
                             unsigned max_nbr, uint32_t* k_list, uint32_t* n_clip, int* status,
                             long* n_exact) {
    prepared_t* p = (prepared_t*)h;
    if (!p || i0 > i1 || i1 > p->n) return 1;
    cells_ctx c = {p->xyz, p->w, p->pts, p->hl, p->dim, p->n, k0, max_nbr, check_sr, exact,
                   &p->g, vol, mg, nbr_count, nbr_idx, k_list, n_clip, nbr_area, status, 0, i0};
    run_parallel_range(cells_range, &c, i0, i1, nthreads);
    if (n_exact) *n_exact = c.n_exact;
    return 0;
}

/* Cells of seeds [i0, i1) of the n seeds: prepare, range, release. */
int orc_cells_range(const double* xyz, const double* w, unsigned n, unsigned i0, unsigned i1,
                    unsigned k0, int check_sr, int exact, int nthreads, double* vol, double* mg,
                    uint32_t* nbr_count, uint32_t* nbr_idx, double* nbr_area, unsigned max_nbr,
                    uint32_t* k_list, uint32_t* n_clip, int* status, long* n_exact) {
    if (n < 2 || i0 > i1 || i1 > n) return 1;
    void* h = orc_cells_prepare(xyz, w, n);
    int r = orc_cells_prepared_range(h, i0, i1, k0, check_sr, exact, nthreads, vol, mg,
                                     nbr_count, nbr_idx, nbr_area, max_nbr, k_list, n_clip,
                                     status, n_exact);
    orc_cells_release(h);
    return r;
}

/* All n cells; same contract as ref_cells in oracle/ref/ref_harness.cpp. */
int orc_cells(const double* xyz, const double* w, unsigned n, unsigned k0, int check_sr,
              int exact, int nthreads, double* vol, double* mg, uint32_t* nbr_count,
              uint32_t* nbr_idx, double* nbr_area, unsigned max_nbr, uint32_t* k_list,
              uint32_t* n_clip, int* status, long* n_exact) {
    return orc_cells_range(xyz, w, n, 0, n, k0, check_sr, exact, nthreads, vol, mg, nbr_count,
                           nbr_idx, nbr_area, max_nbr, k_list, n_clip, status, n_exact);
}
