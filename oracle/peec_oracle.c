/*
 * CPU oracle for the PEEC hot path.  TEST INFRASTRUCTURE ONLY: loaded by
 * tests/, the smoke check and the bench's CPU-baseline leg as the checker,
 * never by the GPU library.
 *
 * Restates the reference algorithms in the reference's operation order; built
 * with ISO C flags (-std=c17 turns floating-point contraction off in gcc) it
 * matches the reference bit for bit on the same machine.  The comment above
 * each function names the reference file:line it follows (paths inside the
 * reference project).
 */
#include "peec_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../peeeeeeeeeeeeeeeeeeec_gb300/csrc/gauss_legendre_table.h"

#define MU0_OVER_4PI 1.0e-7                 /* inductance.c:24 */
#define INV_4PI_EPS0 8.987551792261171e9    /* potential.c:26  */

/* ------------------------------------------------------------------ */
/* small vector helpers (quadrature.c:18-72)                           */
/* ------------------------------------------------------------------ */

static double v_dist(const double a[3], const double b[3])
{
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

static void v_cross(const double a[3], const double b[3], double c[3])
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static double v_norm(const double a[3])
{
    return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
}

static double v_dot(const double a[3], const double b[3])
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* quadrature.c:80-86: vertices coincide within 1e-12 m */
static int same_point(const double a[3], const double b[3])
{
    return v_dist(a, b) <= 1.0e-12;
}

static void corner(const QuadPatch *p, int k, double out[3])
{
    out[0] = p->points[3 * k + 0];
    out[1] = p->points[3 * k + 1];
    out[2] = p->points[3 * k + 2];
}

/* ------------------------------------------------------------------ */
/* Gauss-Legendre (quadrature.c:94-313)                                */
/* ------------------------------------------------------------------ */

int oracle_gauss_legendre_rule(int order, double *x, double *w)
{
    if (x == NULL || w == NULL) return -1;
    for (int r = 0; r < GL_NUM_ORDERS; ++r) {
        if (GL_ORDERS[r] != order) continue;
        for (int i = 0; i < order; ++i) {
            x[i] = GL_NODES[r][i];
            w[i] = GL_WEIGHTS[r][i];
        }
        return 0;
    }
    return -1;
}

static int order_ok(int order)
{
    return order == 2 || order == 3 || order == 4 || order == 5 || order == 6
        || order == 8 || order == 10 || order == 12 || order == 16;
}

/* ------------------------------------------------------------------ */
/* classification (quadrature.c:384-416, 466-607)                      */
/* ------------------------------------------------------------------ */

static double patch_size(const QuadPatch *p)
{
    double c[4][3], longest = 0.0;
    for (int i = 0; i < 4; ++i) corner(p, i, c[i]);
    for (int i = 0; i < 4; ++i) {
        double s = v_dist(c[i], c[(i + 1) % 4]);
        if (s > longest) longest = s;
    }
    return longest;
}

static int shared_vertex_count(const QuadPatch *a, const QuadPatch *b)
{
    int shared = 0;
    for (int i = 0; i < 4; ++i) {
        double pa[3];
        corner(a, i, pa);
        for (int j = 0; j < 4; ++j) {
            double pb[3];
            corner(b, j, pb);
            if (same_point(pa, pb)) { ++shared; break; }
        }
    }
    return shared;
}

static int same_vertex_set(const QuadPatch *a, const QuadPatch *b)
{
    int used[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) {
        double pa[3];
        int hit = 0;
        corner(a, i, pa);
        for (int j = 0; j < 4 && !hit; ++j) {
            double pb[3];
            if (used[j]) continue;
            corner(b, j, pb);
            if (same_point(pa, pb)) { used[j] = 1; hit = 1; }
        }
        if (!hit) return 0;
    }
    return 1;
}

int oracle_classify_pair(const QuadPatch *a, const QuadPatch *b, double near_factor)
{
    if (a == NULL || b == NULL) return 3;
    if (a == b) return 0;
    if (same_vertex_set(a, b)) return 0;
    if (shared_vertex_count(a, b) > 0) return 1;
    double gap2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        double alo = a->points[k], ahi = alo, blo = b->points[k], bhi = blo;
        for (int i = 1; i < 4; ++i) {
            alo = fmin(alo, a->points[3 * i + k]);
            ahi = fmax(ahi, a->points[3 * i + k]);
            blo = fmin(blo, b->points[3 * i + k]);
            bhi = fmax(bhi, b->points[3 * i + k]);
        }
        double g = fmax(0.0, fmax(alo - bhi, blo - ahi));
        gap2 += g * g;
    }
    double gap = sqrt(gap2);
    double ha = patch_size(a), hb = patch_size(b);
    double h = (ha > hb) ? ha : hb;
    if (h > 0.0 && gap < near_factor * h) return 2;
    return 3;
}

/* ------------------------------------------------------------------ */
/* far rule (quadrature.c:632-783)                                     */
/* ------------------------------------------------------------------ */

static void tri_point(const double p0[3], const double p1[3], const double p2[3],
                      double u, double v, double r[3], double *jac)
{
    double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    double e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double xi = u, eta = (1.0 - u) * v;
    for (int k = 0; k < 3; ++k) r[k] = p0[k] + xi * e1[k] + eta * e2[k];
    double n[3];
    v_cross(e1, e2, n);
    *jac = v_norm(n) * (1.0 - u);
}

static double far_rule(double a[3][3], double b[3][3], int order)
{
    double x[16], w[16];
    if (order <= 0 || order > 16 || oracle_gauss_legendre_rule(order, x, w) != 0) return NAN;
    double sum = 0.0;
    for (int iu = 0; iu < order; ++iu) {
        double ua = 0.5 * (x[iu] + 1.0), wua = 0.5 * w[iu];
        for (int iv = 0; iv < order; ++iv) {
            double va = 0.5 * (x[iv] + 1.0), wva = 0.5 * w[iv];
            double ra[3], ja = 0.0;
            tri_point(a[0], a[1], a[2], ua, va, ra, &ja);
            for (int ju = 0; ju < order; ++ju) {
                double ub = 0.5 * (x[ju] + 1.0), wub = 0.5 * w[ju];
                for (int jv = 0; jv < order; ++jv) {
                    double vb = 0.5 * (x[jv] + 1.0), wvb = 0.5 * w[jv];
                    double rb[3], jb = 0.0;
                    tri_point(b[0], b[1], b[2], ub, vb, rb, &jb);
                    double R = v_dist(ra, rb);
                    if (R <= 0.0) continue;
                    double wt = wua * wva * wub * wvb * ja * jb;
                    sum += wt / R;
                }
            }
        }
    }
    return sum;
}

/* ------------------------------------------------------------------ */
/* analytic triangle potential + adaptive outer rule                   */
/* (quadrature.c:842-973)                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    double p[3][3], unit[3][3], outward[3][3], length[3], normal[3];
    double twice_area;
} Tri;

static _Thread_local unsigned long long potential_evals = 0;

unsigned long long oracle_potential_evaluations(int reset)
{
    unsigned long long v = potential_evals;
    if (reset) potential_evals = 0;
    return v;
}

static void tri_prepare(double p[3][3], Tri *t)
{
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            t->p[i][k] = p[i][k];
            t->unit[i][k] = p[(i + 1) % 3][k] - p[i][k];
        }
    v_cross(t->unit[0], t->unit[1], t->normal);
    t->twice_area = v_norm(t->normal);
    if (t->twice_area == 0.0) return;
    for (int k = 0; k < 3; ++k) t->normal[k] /= t->twice_area;
    for (int i = 0; i < 3; ++i) {
        t->length[i] = v_norm(t->unit[i]);
        for (int k = 0; k < 3; ++k) t->unit[i][k] /= t->length[i];
        v_cross(t->unit[i], t->normal, t->outward[i]);
    }
}

static double tri_potential(const Tri *t, const double r[3])
{
    double v[3][3], rad[3];
    ++potential_evals;
    for (int i = 0; i < 3; ++i) {
        for (int k = 0; k < 3; ++k) v[i][k] = t->p[i][k] - r[k];
        rad[i] = v_norm(v[i]);
    }
    double h = v_dot(v[0], t->normal);
    double acc = 0.0;
    for (int i = 0; i < 3; ++i) {
        double d = v_dot(v[i], t->outward[i]);
        if (d == 0.0) continue;
        double s = v_dot(v[i], t->unit[i]);
        double q = hypot(d, h);
        double e = asinh((s + t->length[i]) / q) - asinh(s / q);
        acc += d * e;
    }
    if (h != 0.0) {
        double c[3];
        v_cross(v[1], v[2], c);
        double den = rad[0] * rad[1] * rad[2] + v_dot(v[0], v[1]) * rad[2]
                   + v_dot(v[1], v[2]) * rad[0] + v_dot(v[2], v[0]) * rad[1];
        double omega = 2.0 * atan2(v_dot(v[0], c), den);
        acc -= fabs(h * omega);
    }
    return acc;
}

static double outer_rule(double a[3][3], const Tri *b, int order)
{
    double x[16], w[16];
    if (oracle_gauss_legendre_rule(order, x, w) != 0) return NAN;
    double sum = 0.0;
    for (int i = 0; i < order; ++i)
        for (int j = 0; j < order; ++j) {
            double r[3], jac;
            tri_point(a[0], a[1], a[2], 0.5 * (x[i] + 1), 0.5 * (x[j] + 1), r, &jac);
            sum += 0.25 * w[i] * w[j] * jac * tri_potential(b, r);
        }
    return sum;
}

static double outer_adaptive(double a[3][3], const Tri *b, int order, double abs_tol,
                             int depth)
{
    double lo = outer_rule(a, b, order <= 6 ? 3 : 4);
    double hi = outer_rule(a, b, order);
    if (!isfinite(lo) || !isfinite(hi)) return NAN;
    if (fabs(hi - lo) <= abs_tol + 2e-5 * fabs(hi)) return hi;
    if (depth >= 24) return NAN;
    int e = 0;
    double longest = 0.0;
    for (int i = 0; i < 3; ++i) {
        double s = v_dist(a[i], a[(i + 1) % 3]);
        if (s > longest) { longest = s; e = i; }
    }
    int j = (e + 1) % 3, k = (e + 2) % 3;
    double left[3][3], right[3][3];
    for (int d = 0; d < 3; ++d) {
        double mid = 0.5 * (a[e][d] + a[j][d]);
        left[0][d] = a[e][d];
        left[1][d] = mid;
        left[2][d] = a[k][d];
        right[0][d] = mid;
        right[1][d] = a[j][d];
        right[2][d] = a[k][d];
    }
    return outer_adaptive(left, b, order, abs_tol * 0.5, depth + 1)
         + outer_adaptive(right, b, order, abs_tol * 0.5, depth + 1);
}

/* near_class: 0 = far rule, 1 = SELF, 2 = TOUCHING, 3 = NEAR */
static double tri_pair(double a[3][3], double b[3][3], int far_order, int near_order,
                       int touching_order, int self_order, int near_class)
{
    if (!near_class) return far_rule(a, b, far_order);
    Tri ta, tb;
    tri_prepare(a, &ta);
    tri_prepare(b, &tb);
    if (ta.twice_area == 0.0 || tb.twice_area == 0.0) return 0.0;
    int identical = 1;
    for (int i = 0; i < 3; ++i) {
        int hit = 0;
        for (int j = 0; j < 3; ++j)
            if (same_point(a[i], b[j])) hit = 1;
        if (!hit) identical = 0;
    }
    if (identical) {
        double s = 0.0;
        for (int i = 0; i < 3; ++i) s += tri_potential(&tb, a[i]);
        return ta.twice_area * s / 3.0;
    }
    int order = near_class == 1 ? self_order : near_class == 2 ? touching_order : near_order;
    if (order < 6) order = 6;
    double scale = ta.twice_area * tb.twice_area / sqrt(fmax(ta.twice_area, tb.twice_area));
    double ab = outer_adaptive(a, &tb, order, 2e-5 * scale, 0);
    double ba = outer_adaptive(b, &ta, order, 2e-5 * scale, 0);
    return 0.5 * (ab + ba);
}

double oracle_patch_kernel(const QuadPatch *a, const QuadPatch *b, int far_order,
                           int near_order, int touching_order, int self_order,
                           double near_factor)
{
    if (a == NULL || b == NULL) return NAN;
    if (!order_ok(far_order) || !order_ok(near_order) || !order_ok(touching_order)
        || !order_ok(self_order) || !isfinite(near_factor) || near_factor < 0.0)
        return NAN;
    double pa[4][3], pb[4][3];
    for (int i = 0; i < 4; ++i) {
        corner(a, i, pa[i]);
        corner(b, i, pb[i]);
    }
    /* split (0,1,2) + (0,2,3) */
    static const int split[2][3] = {{0, 1, 2}, {0, 2, 3}};
    double ta[2][3][3], tb[2][3][3];
    for (int t = 0; t < 2; ++t)
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k) {
                ta[t][v][k] = pa[split[t][v]][k];
                tb[t][v][k] = pb[split[t][v]][k];
            }
    int cls = oracle_classify_pair(a, b, near_factor);
    int near_class = cls == 3 ? 0 : cls + 1;
    double sum = 0.0;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            double v = tri_pair(ta[i], tb[j], far_order, near_order, touching_order,
                                self_order, near_class);
            if (!isfinite(v)) return NAN;
            sum += v;
        }
    return sum;
}

/* ------------------------------------------------------------------ */
/* Lp (inductance.c:152-167, 221-382, 390-560)                        */
/* ------------------------------------------------------------------ */

static int region_integral(const PatchList *ra, const PatchList *rb, const int orders[4],
                           double near_factor, double *out)
{
    double sum = 0.0;
    for (size_t i = 0; i < ra->count; ++i)
        for (size_t j = 0; j < rb->count; ++j) {
            double k = oracle_patch_kernel(&ra->patches[i], &rb->patches[j], orders[0],
                                           orders[1], orders[2], orders[3], near_factor);
            if (!isfinite(k)) return -1;
            sum += k;
        }
    *out = sum;
    return 0;
}

int oracle_inductance_pair(const Mesh *mesh, const DualMesh *dual, size_t a, size_t b,
                           const int orders[4], double near_factor,
                           double direction_tolerance, double *value)
{
    if (!mesh || !dual || !orders || !value) return -1;
    if (a >= mesh->n_edges || b >= mesh->n_edges) return -1;
    double dot = v_dot(&mesh->edge_directions[3 * a], &mesh->edge_directions[3 * b]);
    if (fabs(dot) < direction_tolerance) {
        *value = 0.0;
        return 0;
    }
    double sa = dual->edge_region_areas[a], la = mesh->edge_lengths[a];
    double sb = dual->edge_region_areas[b], lb = mesh->edge_lengths[b];
    double wa = (sa <= 0.0 || la <= 0.0) ? 0.0 : sa / la;
    double wb = (sb <= 0.0 || lb <= 0.0) ? 0.0 : sb / lb;
    if (wa <= 0.0 || wb <= 0.0) return -1;
    const PatchList *ra = &dual->edge_patches[a], *rb = &dual->edge_patches[b];
    if (ra->count == 0 || rb->count == 0) return -1;
    double g;
    if (region_integral(ra, rb, orders, near_factor, &g) != 0) return -1;
    *value = MU0_OVER_4PI * dot * g / (wa * wb);
    return isfinite(*value) ? 0 : -1;
}

int oracle_inductance_rows(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                           double near_factor, double direction_tolerance, int threads,
                           size_t row_begin, size_t row_end, double *data)
{
    if (!mesh || !dual || !data || threads < 1) return -1;
    size_t ne = mesh->n_edges;
    int failed = 0;
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (long long as = (long long)row_begin; as < (long long)row_end; ++as) {
        size_t a = (size_t)as;
        for (size_t b = a; b < ne; ++b) {
            int stop;
#pragma omp atomic read
            stop = failed;
            if (stop) break;
            double v = 0.0;
            if (oracle_inductance_pair(mesh, dual, a, b, orders, near_factor,
                                       direction_tolerance, &v) != 0) {
#pragma omp atomic write
                failed = 1;
                break;
            }
            data[a * ne + b] = v;
            data[b * ne + a] = v;
        }
    }
    return failed ? -1 : 0;
}

int oracle_inductance_matrix(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                             double near_factor, double direction_tolerance, int threads,
                             double *data)
{
    if (!mesh) return -1;
    return oracle_inductance_rows(mesh, dual, orders, near_factor, direction_tolerance,
                                  threads, 0, mesh->n_edges, data);
}

/* ------------------------------------------------------------------ */
/* P (potential.c:139-253, 261-395)                                    */
/* ------------------------------------------------------------------ */

int oracle_potential_pair(const Mesh *mesh, const DualMesh *dual, size_t i, size_t j,
                          const int orders[4], double near_factor, double *value)
{
    if (!mesh || !dual || !orders || !value) return -1;
    if (i >= mesh->n_nodes || j >= mesh->n_nodes) return -1;
    double si = dual->node_region_areas[i], sj = dual->node_region_areas[j];
    if (si <= 0.0 || sj <= 0.0) return -1;
    const PatchList *ri = &dual->node_patches[i], *rj = &dual->node_patches[j];
    if (ri->count == 0 || rj->count == 0) return -1;
    double g;
    if (region_integral(ri, rj, orders, near_factor, &g) != 0) return -1;
    *value = INV_4PI_EPS0 * g / (si * sj);
    return isfinite(*value) ? 0 : -1;
}

int oracle_potential_rows(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                          double near_factor, int threads, size_t row_begin,
                          size_t row_end, double *data)
{
    if (!mesh || !dual || !data || threads < 1) return -1;
    size_t nv = mesh->n_nodes;
    int failed = 0;
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (long long is = (long long)row_begin; is < (long long)row_end; ++is) {
        size_t i = (size_t)is;
        for (size_t j = i; j < nv; ++j) {
            int stop;
#pragma omp atomic read
            stop = failed;
            if (stop) break;
            double v = 0.0;
            if (oracle_potential_pair(mesh, dual, i, j, orders, near_factor, &v) != 0) {
#pragma omp atomic write
                failed = 1;
                break;
            }
            data[i * nv + j] = v;
            data[j * nv + i] = v;
        }
    }
    return failed ? -1 : 0;
}

int oracle_potential_matrix(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                            double near_factor, int threads, double *data)
{
    if (!mesh) return -1;
    return oracle_potential_rows(mesh, dual, orders, near_factor, threads, 0,
                                 mesh->n_nodes, data);
}

/* Rows of Lp (kind 0) or P (kind 1) for a timing sample: the upper-
 * triangle pairs (a, b >= a) of the given rows with the default orders
 * (4, 10, 12, 8), near factor 0.5 and direction tolerance 1e-10, the pairs
 * of all sampled rows spread over `threads` threads.  out[k * n + b]
 * receives row rows[k].  Returns 0, or -1 when a pair fails. */
int oracle_sample_rows(const Mesh *mesh, const DualMesh *dual, int kind, const size_t *rows, size_t nrows,
                       int threads, double *out)
{
    static const int orders[4] = {4, 10, 12, 8};
    size_t n = kind == 0 ? mesh->n_edges : mesh->n_nodes;
    size_t *start = malloc((nrows + 1) * sizeof(size_t));
    if (!start) return -1;
    start[0] = 0;
    for (size_t k = 0; k < nrows; ++k) start[k + 1] = start[k] + (rows[k] < n ? n - rows[k] : 0);
    int failed = 0;
    long long total = (long long)start[nrows];
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
    for (long long t = 0; t < total; ++t) {
        size_t lo = 0, hi = nrows;
        while (hi - lo > 1) {
            size_t mid = (lo + hi) / 2;
            if (start[mid] <= (size_t)t) lo = mid; else hi = mid;
        }
        size_t a = rows[lo], b = a + ((size_t)t - start[lo]);
        double v = 0.0;
        int st = kind == 0 ? oracle_inductance_pair(mesh, dual, a, b, orders, 0.5, 1e-10, &v)
                           : oracle_potential_pair(mesh, dual, a, b, orders, 0.5, &v);
        if (st != 0) {
#pragma omp atomic write
            failed = 1;
        }
        out[lo * n + b] = v;
    }
    free(start);
    return failed ? -1 : 0;
}

/* ------------------------------------------------------------------ */
/* real LU (lu.c:194-479, 494-653)                                     */
/* ------------------------------------------------------------------ */

int oracle_lu_factorize(const double *input, size_t n, double pivot_tolerance,
                        int threads, double *a, size_t *piv, size_t *swap_count,
                        double *matrix_scale)
{
    if (!input || !a || !piv || n == 0 || threads < 1) return -1;
    memcpy(a, input, n * n * sizeof(double));
    double scale = 0.0;
    for (size_t t = 0; t < n * n; ++t) {
        double m = fabs(input[t]);
        if (m > scale) scale = m;
    }
    *matrix_scale = scale;
    *swap_count = 0;
    if (!isfinite(scale) || scale <= 0.0) return -2;
    double limit = pivot_tolerance * scale;
    for (size_t k = 0; k < n; ++k) {
        size_t p = k;
        double best = fabs(a[k * n + k]);
        for (size_t i = k + 1; i < n; ++i) {
            double c = fabs(a[i * n + k]);
            if (c > best) { best = c; p = i; }
        }
        if (!isfinite(best) || best <= limit) return -2;
        piv[k] = p;
        if (p != k) {
            for (size_t j = 0; j < n; ++j) {
                double t = a[k * n + j];
                a[k * n + j] = a[p * n + j];
                a[p * n + j] = t;
            }
            ++*swap_count;
        }
        if (k + 1 >= n) continue;
        double pv = a[k * n + k];
        if (!isfinite(pv) || fabs(pv) <= limit) return -2;
#pragma omp parallel for schedule(static) num_threads(threads) if (n - k - 1 >= 64)
        for (long long is = (long long)k + 1; is < (long long)n; ++is) {
            size_t i = (size_t)is;
            double m = a[i * n + k] / pv;
            a[i * n + k] = m;
            for (size_t j = k + 1; j < n; ++j) a[i * n + j] -= m * a[k * n + j];
        }
    }
    for (size_t i = 0; i < n; ++i) {
        double d = a[i * n + i];
        if (!isfinite(d) || fabs(d) <= limit) return -2;
    }
    return 0;
}

int oracle_lu_solve(const double *a, const size_t *piv, size_t n, const double *b,
                    double *x)
{
    if (!a || !piv || !b || !x) return -1;
    if (x != b) memcpy(x, b, n * sizeof(double));
    for (size_t k = 0; k < n; ++k)
        if (piv[k] != k) {
            double t = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = t;
        }
    for (size_t i = 0; i < n; ++i) {
        double c = 0.0;
        for (size_t j = 0; j < i; ++j) c += a[i * n + j] * x[j];
        x[i] -= c;
    }
    for (size_t ii = n; ii-- > 0;) {
        double c = 0.0;
        for (size_t j = ii + 1; j < n; ++j) c += a[ii * n + j] * x[j];
        double d = a[ii * n + ii];
        if (d == 0.0 || !isfinite(d)) return -1;
        x[ii] = (x[ii] - c) / d;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* complex LU (complex_lu.c:208-550, 598-778)                          */
/* ------------------------------------------------------------------ */

int oracle_complex_lu_factorize(const Complex *input, size_t n, double pivot_tolerance,
                                int threads, Complex *a, size_t *piv, size_t *swap_count,
                                double *matrix_scale, double *row_scale,
                                double *column_scale)
{
    if (!input || !a || !piv || !row_scale || !column_scale || n == 0 || threads < 1
        || !isfinite(pivot_tolerance) || pivot_tolerance < 0.0)
        return -1;
    *swap_count = 0;
    *matrix_scale = 0.0;
    for (size_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (size_t j = 0; j < n; ++j) {
            double m = hypot(input[i * n + j].re, input[i * n + j].im);
            if (!isfinite(m)) return -2;
            s = fmax(s, m);
        }
        if (s == 0.0) return -2;
        row_scale[i] = s;
        for (size_t j = 0; j < n; ++j) {
            a[i * n + j].re = input[i * n + j].re / s;
            a[i * n + j].im = input[i * n + j].im / s;
        }
    }
    for (size_t j = 0; j < n; ++j) {
        double s = 0.0;
        for (size_t i = 0; i < n; ++i) s = fmax(s, hypot(a[i * n + j].re, a[i * n + j].im));
        if (s == 0.0) return -2;
        column_scale[j] = s;
        for (size_t i = 0; i < n; ++i) {
            a[i * n + j].re /= s;
            a[i * n + j].im /= s;
        }
    }
    double scale = 0.0;
    for (size_t t = 0; t < n * n; ++t) {
        double m = hypot(a[t].re, a[t].im);
        if (m > scale) scale = m;
    }
    *matrix_scale = scale;
    if (!isfinite(scale) || scale <= 0.0) return -2;
    double limit = pivot_tolerance * scale;
    for (size_t k = 0; k < n; ++k) {
        size_t p = k;
        double best = hypot(a[k * n + k].re, a[k * n + k].im);
        for (size_t i = k + 1; i < n; ++i) {
            double m = hypot(a[i * n + k].re, a[i * n + k].im);
            if (m > best) { best = m; p = i; }
        }
        if (!isfinite(best) || best <= limit) return -2;
        piv[k] = p;
        if (p != k) {
            for (size_t j = 0; j < n; ++j) {
                Complex t = a[k * n + j];
                a[k * n + j] = a[p * n + j];
                a[p * n + j] = t;
            }
            ++*swap_count;
        }
        if (k + 1 >= n) continue;
        Complex pv = a[k * n + k];
        double pm = hypot(pv.re, pv.im);
        if (!isfinite(pm) || pm <= limit) return -2;
#pragma omp parallel for schedule(static) num_threads(threads) if (n - k - 1 >= 64)
        for (long long is = (long long)k + 1; is < (long long)n; ++is) {
            size_t i = (size_t)is;
            Complex q = a[i * n + k], m;
            double den = pv.re * pv.re + pv.im * pv.im;
            m.re = (q.re * pv.re + q.im * pv.im) / den;
            m.im = (q.im * pv.re - q.re * pv.im) / den;
            a[i * n + k] = m;
            for (size_t j = k + 1; j < n; ++j) {
                Complex u = a[k * n + j];
                double pr = m.re * u.re - m.im * u.im;
                double pi = m.re * u.im + m.im * u.re;
                a[i * n + j].re -= pr;
                a[i * n + j].im -= pi;
            }
        }
    }
    for (size_t i = 0; i < n; ++i) {
        double m = hypot(a[i * n + i].re, a[i * n + i].im);
        if (!isfinite(m) || m <= limit) return -2;
    }
    return 0;
}

int oracle_complex_lu_solve(const Complex *a, const size_t *piv, const double *row_scale,
                            const double *column_scale, size_t n, const Complex *b,
                            Complex *x)
{
    if (!a || !piv || !row_scale || !column_scale || !b || !x) return -1;
    for (size_t i = 0; i < n; ++i) {
        x[i].re = b[i].re / row_scale[i];
        x[i].im = b[i].im / row_scale[i];
    }
    for (size_t k = 0; k < n; ++k)
        if (piv[k] != k) {
            Complex t = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = t;
        }
    for (size_t i = 0; i < n; ++i) {
        double cr = 0.0, ci = 0.0;
        for (size_t j = 0; j < i; ++j) {
            Complex l = a[i * n + j], v = x[j];
            cr += l.re * v.re - l.im * v.im;
            ci += l.re * v.im + l.im * v.re;
        }
        x[i].re -= cr;
        x[i].im -= ci;
    }
    for (size_t ii = n; ii-- > 0;) {
        double cr = 0.0, ci = 0.0;
        for (size_t j = ii + 1; j < n; ++j) {
            Complex u = a[ii * n + j], v = x[j];
            cr += u.re * v.re - u.im * v.im;
            ci += u.re * v.im + u.im * v.re;
        }
        Complex r = {x[ii].re - cr, x[ii].im - ci}, d = a[ii * n + ii];
        double den = d.re * d.re + d.im * d.im;
        if (!isfinite(den) || den == 0.0) return -1;
        x[ii].re = (r.re * d.re + r.im * d.im) / den;
        x[ii].im = (r.im * d.re - r.re * d.im) / den;
    }
    for (size_t i = 0; i < n; ++i) {
        x[i].re /= column_scale[i];
        x[i].im /= column_scale[i];
    }
    return 0;
}


/* ===================================================================== */
/* transient stage 1                                                      */
/* ===================================================================== */

/* transient.c:19-35 */
static double transient_theta(int scheme)
{
    return scheme == 1 ? 1.0 : scheme == 2 ? 0.5 : NAN;
}

/* dense incidence row e: A[e][a] = -1, A[e][b] = +1 (incidence.c:34-115) */
static double incidence_entry(const int *edges, size_t e, size_t j)
{
    if ((size_t)edges[2 * e + 1] == j) return 1.0;
    if ((size_t)edges[2 * e + 0] == j) return -1.0;
    return 0.0;
}

int oracle_transient_stage1_matrix(const double *L, const double *P, const int *edges,
                                   const double *R, size_t ne, size_t nv, int scheme,
                                   double dt, double *M, double *F, double *AS)
{
    double theta = transient_theta(scheme);
    if (!L || !P || !edges || !M || !F || !AS || ne == 0 || nv == 0 || isnan(theta) ||
        !isfinite(dt) || dt <= 0.0)
        return -1;
    size_t nt = ne + nv;
    /* potential.c:483-520 */
    for (size_t j = 0; j < nv; ++j) {
        double d = P[j * nv + j];
        if (!isfinite(d) || d <= 0.0) return -1;
        F[j] = 1.0 / d;
    }
    /* incidence.c:593-741: AS[e][a] = (P[plus][a] - P[minus][a]) / P[a][a] */
    for (size_t e = 0; e < ne; ++e) {
        int a = edges[2 * e + 0], b = edges[2 * e + 1];
        if (a < 0 || b < 0 || (size_t)a >= nv || (size_t)b >= nv || a == b) return -1;
        for (size_t k = 0; k < nv; ++k)
            AS[e * nv + k] = (P[(size_t)b * nv + k] - P[(size_t)a * nv + k]) / P[k * nv + k];
    }
    memset(M, 0, nt * nt * sizeof(double));
    for (size_t i = 0; i < ne; ++i)
        for (size_t j = 0; j < ne; ++j) {
            double v = L[i * ne + j] / dt;
            if (i == j) v += theta * (R ? R[i] : 0.0);
            M[i * nt + j] = v;
        }
    for (size_t e = 0; e < ne; ++e)
        for (size_t j = 0; j < nv; ++j) M[e * nt + ne + j] = theta * AS[e * nv + j];
    for (size_t j = 0; j < nv; ++j)
        for (size_t e = 0; e < ne; ++e) M[(ne + j) * nt + e] = -theta * incidence_entry(edges, e, j);
    for (size_t r = 0; r < nv; ++r)
        for (size_t c = 0; c < nv; ++c) {
            double v = 0.0;
            if (r == c) v += F[r];
            M[(ne + r) * nt + ne + c] = v / dt;
        }
    return 0;
}

int oracle_transient_rhs_stage1(const double *L, const double *R, const double *AS,
                                const double *F, const int *edges, size_t ne, size_t nv,
                                int scheme, double dt, const double *I, const double *V,
                                const double *Jn, const double *Jnp1, double *rhs)
{
    double theta = transient_theta(scheme);
    if (!L || !AS || !F || !edges || !I || !V || !rhs || isnan(theta)) return -1;
    double omt = 1.0 - theta;
    for (size_t i = 0; i < ne; ++i) {
        double v = 0.0;
        for (size_t j = 0; j < ne; ++j) v += L[i * ne + j] * I[j] / dt;
        v -= omt * (R ? R[i] : 0.0) * I[i];
        for (size_t j = 0; j < nv; ++j) v -= omt * AS[i * nv + j] * V[j];
        rhs[i] = v;
    }
    for (size_t j = 0; j < nv; ++j) {
        double v = F[j] * V[j] / dt;
        for (size_t e = 0; e < ne; ++e) v += omt * incidence_entry(edges, e, j) * I[e];
        if (Jn) v += omt * Jn[j];
        if (Jnp1) v += theta * Jnp1[j];
        rhs[ne + j] = v;
    }
    return 0;
}

double oracle_lightning_current(double K, double alpha, double beta, double delay, double t)
{
    if (!isfinite(t)) return NAN;
    if (t < delay) return 0.0;
    double tau = t - delay;
    return K * (exp(-alpha * tau) - exp(-beta * tau));
}

int oracle_transient_lightning(const double *L, const double *P, const int *edges,
                               const double *R, size_t ne, size_t nv, int scheme, double dt,
                               double K, double alpha, double beta, double delay,
                               size_t strike_node, size_t return_node, size_t n_steps,
                               double *I, double *V, const int *probe_nodes,
                               size_t n_probe_nodes, const int *probe_edges,
                               size_t n_probe_edges, double *probe_out)
{
    if (strike_node >= nv || return_node >= nv || strike_node == return_node) return -1;
    size_t nt = ne + nv;
    double *M = malloc(nt * nt * sizeof(double)), *F = malloc(nv * sizeof(double));
    double *AS = malloc(ne * nv * sizeof(double)), *lu = malloc(nt * nt * sizeof(double));
    double *rhs = malloc(nt * sizeof(double)), *x = malloc(nt * sizeof(double));
    double *Jn = calloc(nv, sizeof(double)), *Jnp1 = calloc(nv, sizeof(double));
    size_t *piv = malloc(nt * sizeof(size_t));
    int status = -1;
    if (!M || !F || !AS || !lu || !rhs || !x || !Jn || !Jnp1 || !piv) goto done;
    if (oracle_transient_stage1_matrix(L, P, edges, R, ne, nv, scheme, dt, M, F, AS) != 0) goto done;
    size_t swaps;
    double scale;
    status = oracle_lu_factorize(M, nt, 1.0e-14, 1, lu, piv, &swaps, &scale);
    if (status != 0) goto done;
    size_t np = n_probe_nodes + n_probe_edges;
    for (size_t step = 0; step < n_steps; ++step) {
        double tn = step * dt, tnp1 = (step + 1) * dt;
        /* lightning.c:310-373 */
        double cn = oracle_lightning_current(K, alpha, beta, delay, tn);
        double cnp1 = oracle_lightning_current(K, alpha, beta, delay, tnp1);
        memset(Jn, 0, nv * sizeof(double));
        memset(Jnp1, 0, nv * sizeof(double));
        Jn[strike_node] = cn;
        Jn[return_node] = -cn;
        Jnp1[strike_node] = cnp1;
        Jnp1[return_node] = -cnp1;
        oracle_transient_rhs_stage1(L, R, AS, F, edges, ne, nv, scheme, dt, I, V, Jn, Jnp1, rhs);
        if (oracle_lu_solve(lu, piv, nt, rhs, x) != 0) {
            status = -1;
            goto done;
        }
        memcpy(I, x, ne * sizeof(double));
        memcpy(V, x + ne, nv * sizeof(double));
        if (probe_out) {
            for (size_t k = 0; k < n_probe_nodes; ++k) probe_out[step * np + k] = V[probe_nodes[k]];
            for (size_t k = 0; k < n_probe_edges; ++k)
                probe_out[step * np + n_probe_nodes + k] = I[probe_edges[k]];
        }
    }
done:
    free(M);
    free(F);
    free(AS);
    free(lu);
    free(rhs);
    free(x);
    free(Jn);
    free(Jnp1);
    free(piv);
    return status;
}


/* ===================================================================== */
/* retarded kernel (extension; the reference's retardation.c is empty)    */
/* ===================================================================== */

/* far-rule points of a patch: triangles (0,1,2), (0,2,3), order^2 mapped
 * Gauss points each with weight w_u w_v J (quadrature.c:632-666) */
static int patch_points(const QuadPatch *p, int order, double *pts /* [2 order^2][4] */)
{
    double x[16], w[16];
    if (order <= 0 || order > 16 || oracle_gauss_legendre_rule(order, x, w) != 0) return -1;
    double c[4][3];
    for (int i = 0; i < 4; ++i) corner(p, i, c[i]);
    int k = 0;
    for (int t = 0; t < 2; ++t) {
        const double *p0 = c[0], *p1 = c[t == 0 ? 1 : 2], *p2 = c[t == 0 ? 2 : 3];
        for (int iu = 0; iu < order; ++iu)
            for (int iv = 0; iv < order; ++iv, ++k) {
                double u = 0.5 * (x[iu] + 1.0), wu = 0.5 * w[iu];
                double v = 0.5 * (x[iv] + 1.0), wv = 0.5 * w[iv];
                double r[3], jac;
                tri_point(p0, p1, p2, u, v, r, &jac);
                pts[4 * k + 0] = r[0];
                pts[4 * k + 1] = r[1];
                pts[4 * k + 2] = r[2];
                pts[4 * k + 3] = wu * wv * jac;
            }
    }
    return k;
}

/* sum over point pairs of w_a w_b (exp(-jkR) - 1) / R
 * = w_a w_b (-2 sin^2(kR/2) - j sin kR) / R, limit -jk w_a w_b at R = 0 */
static int retard_correction(const QuadPatch *a, const QuadPatch *b, int order, double k,
                             double *re, double *im)
{
    double pa[2 * 16 * 16 * 4], pb[2 * 16 * 16 * 4];
    int na = patch_points(a, order, pa), nb = patch_points(b, order, pb);
    if (na < 0 || nb < 0) return -1;
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
            double d[3] = {pa[4 * i] - pb[4 * j], pa[4 * i + 1] - pb[4 * j + 1], pa[4 * i + 2] - pb[4 * j + 2]};
            double R = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double ww = pa[4 * i + 3] * pb[4 * j + 3];
            if (R <= 0.0) {
                si += -k * ww;
                continue;
            }
            double s = sin(0.5 * k * R), c = cos(0.5 * k * R);
            sr += ww * (-2.0 * s * s) / R;
            si += ww * (-2.0 * s * c) / R;
        }
    *re = sr;
    *im = si;
    return 0;
}

int oracle_retarded_matrix(const Mesh *mesh, const DualMesh *dual, int kind, const int orders[4],
                           double near_factor, double direction_tolerance, double wave_number,
                           int threads, double *out)
{
    if (!mesh || !dual || !orders || !out || threads < 1 || (kind != 0 && kind != 1) ||
        !isfinite(wave_number) || wave_number < 0.0)
        return -1;
    size_t n = kind == 0 ? mesh->n_edges : mesh->n_nodes;
    double *stat = malloc(n * n * sizeof(double));
    if (!stat) return -1;
    int s = kind == 0 ? oracle_inductance_matrix(mesh, dual, orders, near_factor, direction_tolerance,
                                                 threads, stat)
                      : oracle_potential_matrix(mesh, dual, orders, near_factor, threads, stat);
    if (s != 0) {
        free(stat);
        return -1;
    }
    int failed = 0;
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (long long as = 0; as < (long long)n; ++as) {
        size_t a = (size_t)as;
        for (size_t b = a; b < n; ++b) {
            double scale, dre = 0.0, dim = 0.0;
            const PatchList *ra, *rb;
            if (kind == 0) {
                double dot = v_dot(&mesh->edge_directions[3 * a], &mesh->edge_directions[3 * b]);
                double wa = dual->edge_region_areas[a] / mesh->edge_lengths[a];
                double wb = dual->edge_region_areas[b] / mesh->edge_lengths[b];
                scale = fabs(dot) < direction_tolerance ? 0.0 : MU0_OVER_4PI * dot / (wa * wb);
                ra = &dual->edge_patches[a];
                rb = &dual->edge_patches[b];
            } else {
                scale = INV_4PI_EPS0 / (dual->node_region_areas[a] * dual->node_region_areas[b]);
                ra = &dual->node_patches[a];
                rb = &dual->node_patches[b];
            }
            if (scale != 0.0 && wave_number != 0.0) {
                for (size_t i = 0; i < ra->count; ++i)
                    for (size_t j = 0; j < rb->count; ++j) {
                        double r, m;
                        if (retard_correction(&ra->patches[i], &rb->patches[j], orders[0], wave_number,
                                              &r, &m) != 0) {
#pragma omp atomic write
                            failed = 1;
                        }
                        dre += r;
                        dim += m;
                    }
            }
            double vr = stat[a * n + b] + scale * dre, vi = scale * dim;
            out[2 * (a * n + b)] = vr;
            out[2 * (a * n + b) + 1] = vi;
            out[2 * (b * n + a)] = vr;
            out[2 * (b * n + a) + 1] = vi;
        }
    }
    free(stat);
    return failed ? -1 : 0;
}


/* ------------------------------------------------------------------ */
/* RCS radiation vector, dual-patch quadrature (rcs.c:238-1000)        */
/* ------------------------------------------------------------------ */

/* integral over triangle (p0, p1, p2) of exp(j k dir.r) dS by the
 * collapsed-square Gauss rule of `order` (rcs.c:238-362): the points in
 * (iu, iv) order, cos / sin of the phase, weight (0.5 w_u)(0.5 w_v) J. */
static int rcs_triangle(const double p0[3], const double p1[3], const double p2[3], double k,
                        const double dir[3], int order, double *re, double *im)
{
    double x[16], w[16];
    if (order <= 0 || order > 16 || oracle_gauss_legendre_rule(order, x, w) != 0) return -1;
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
        a[d] = p1[d] - p0[d];
        b[d] = p2[d] - p0[d];
    }
    v_cross(a, b, c);
    const double area2 = v_norm(c);
    double sr = 0.0, si = 0.0;
    for (int iu = 0; iu < order; ++iu) {
        const double u = 0.5 * (x[iu] + 1.0), wu = 0.5 * w[iu];
        for (int iv = 0; iv < order; ++iv) {
            const double v = 0.5 * (x[iv] + 1.0), wv = 0.5 * w[iv];
            const double xi = u, eta = (1.0 - u) * v;
            double r[3];
            for (int d = 0; d < 3; ++d) r[d] = p0[d] + xi * a[d] + eta * b[d];
            const double jac = area2 * (1.0 - u);
            const double phase = k * v_dot(dir, r);
            const double weight = wu * wv * jac;
            sr += weight * cos(phase);
            si += weight * sin(phase);
        }
    }
    *re = sr;
    *im = si;
    return 0;
}

int oracle_rcs_radiation_vector(const Mesh *mesh, const DualMesh *dual, const Complex *current,
                                double wave_number, const double dir[3], int order, Complex out[3])
{
    if (!mesh || !dual || !current || !dir || !out || !mesh->edge_vectors || !dual->edge_patches ||
        !dual->edge_region_areas || dual->n_edges != mesh->n_edges)
        return -1;
    if (!isfinite(wave_number) || wave_number <= 0.0 || !order_ok(order)) return -1;
    double F[6] = {0, 0, 0, 0, 0, 0};  /* x re, x im, y re, y im, z re, z im */
    for (size_t e = 0; e < mesh->n_edges; ++e) {
        const double *ev = mesh->edge_vectors + 3 * e;
        const double len = v_norm(ev);
        if (len <= 0.0) continue;                              /* rcs.c:801-806 */
        const double ed[3] = {ev[0] / len, ev[1] / len, ev[2] / len};
        const double area = dual->edge_region_areas[e];
        if (area <= 0.0) continue;                             /* rcs.c:866-869 */
        const double width = area / len;
        /* G_e: patches in list order, triangles (0,1,2) then (0,2,3) */
        double gr = 0.0, gi = 0.0;
        const PatchList *list = &dual->edge_patches[e];
        for (size_t q = 0; q < list->count; ++q) {
            double p[4][3];
            for (int i = 0; i < 4; ++i) corner(&list->patches[q], i, p[i]);
            double r0, i0, r1, i1;
            if (rcs_triangle(p[0], p[1], p[2], wave_number, dir, order, &r0, &i0) != 0 ||
                rcs_triangle(p[0], p[2], p[3], wave_number, dir, order, &r1, &i1) != 0)
                return -1;
            gr += r0 + r1;
            gi += i0 + i1;
        }
        /* (I_e / w_e) G_e along the edge direction (rcs.c:920-990) */
        const double cr = current[e].re / width, ci = current[e].im / width;
        const double sr = cr * gr - ci * gi, si = cr * gi + ci * gr;
        for (int d = 0; d < 3; ++d) {
            F[2 * d] += sr * ed[d];
            F[2 * d + 1] += si * ed[d];
        }
    }
    for (int d = 0; d < 3; ++d) {
        out[d].re = F[2 * d];
        out[d].im = F[2 * d + 1];
    }
    return 0;
}

/* ---- incidence products (incidence.c:242-741), test oracle ---- */

/* incidence.c:298-330: K[e][f] = P[a][c] - P[a][d] - P[b][c] + P[b][d] for
 * e <= f, written to both triangles */
void oracle_incidence_apat(const double *P, const int *edges, size_t nv, size_t ne, double *K) {
    for (size_t e = 0; e < ne; ++e) {
        const size_t a = (size_t)edges[2 * e], b = (size_t)edges[2 * e + 1];
        for (size_t f = e; f < ne; ++f) {
            const size_t c = (size_t)edges[2 * f], d = (size_t)edges[2 * f + 1];
            const double v = P[a * nv + c] - P[a * nv + d] - P[b * nv + c] + P[b * nv + d];
            K[e * ne + f] = v;
            K[f * ne + e] = v;
        }
    }
}

/* incidence.c:475-589: PAT[j][e] = P[j][b] - P[j][a], NaN for an edge out of
 * range; the first non-finite entry in row-major order fails the call */
int oracle_incidence_pat(const double *P, const int *edges, size_t nv, size_t ne, double *out,
                         long long *first_bad) {
    for (size_t j = 0; j < nv; ++j)
        for (size_t e = 0; e < ne; ++e) {
            const int a = edges[2 * e], b = edges[2 * e + 1];
            out[j * ne + e] = (a < 0 || b < 0 || (size_t)a >= nv || (size_t)b >= nv)
                                  ? NAN
                                  : P[j * nv + (size_t)b] - P[j * nv + (size_t)a];
        }
    *first_bad = -1;
    for (size_t t = 0; t < nv * ne; ++t)
        if (!isfinite(out[t])) {
            *first_bad = (long long)t;
            return -1;
        }
    return 0;
}

/* incidence.c:641-729 with node_minus / node_plus = the edge's (a, b):
 * AS[e][k] = (P[b][k] - P[a][k]) / P[k][k]; NaN and failure where P[k][k] is
 * not finite or <= 0 */
int oracle_incidence_as(const double *P, const int *edges, size_t nv, size_t ne, double *AS) {
    int status = 0;
    for (size_t e = 0; e < ne; ++e) {
        const size_t m = (size_t)edges[2 * e], n = (size_t)edges[2 * e + 1];
        for (size_t k = 0; k < nv; ++k) {
            const double pkk = P[k * nv + k];
            if (!isfinite(pkk) || pkk <= 0.0) {
                AS[e * nv + k] = NAN;
                status = -1;
                continue;
            }
            AS[e * nv + k] = (P[n * nv + k] - P[m * nv + k]) / pkk;
        }
    }
    return status;
}
