/*
 * CPU oracle for the PEEC hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain C restatement of the reference algorithms (quadrature, Lp and P
 * assembly, real and complex LU), written to follow the reference's
 * operation order so that, built with ISO C flags (no FP contraction), it
 * reproduces the reference bit for bit.  Only tests/, the smoke check and the
 * bench's CPU baseline may load it; the GPU library never links or calls it.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef PEEC_ORACLE_H
#define PEEC_ORACLE_H

#include <stddef.h>

#include "../include/complex_matrix.h"
#include "../include/dual_mesh.h"
#include "../include/mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* quadrature.c:94-313 */
int oracle_gauss_legendre_rule(int order, double *x, double *w);
/* quadrature.c:550-607; returns 0 SELF, 1 TOUCHING, 2 NEAR, 3 FAR */
int oracle_classify_pair(const QuadPatch *a, const QuadPatch *b, double near_factor);
/* quadrature.c:975-1079 */
double oracle_patch_kernel(const QuadPatch *a, const QuadPatch *b, int far_order,
                           int near_order, int touching_order, int self_order,
                           double near_factor);
/* Number of triangle_potential_at() evaluations made by this thread since the
 * last reset (work counter for the near-field roofline). */
unsigned long long oracle_potential_evaluations(int reset);

/* inductance.c:221-382 and :390-560.  orders[4] = far, near, touching, self.
 * data must hold Ne*Ne doubles; threads >= 1 (OpenMP rows, dynamic). */
int oracle_inductance_pair(const Mesh *mesh, const DualMesh *dual, size_t a, size_t b,
                           const int orders[4], double near_factor,
                           double direction_tolerance, double *value);
int oracle_inductance_matrix(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                             double near_factor, double direction_tolerance,
                             int threads, double *data);
/* Same, for the rows [row_begin, row_end) only (upper triangle b >= a, both
 * mirrors written): a bounded sample for CPU timing. */
int oracle_inductance_rows(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                           double near_factor, double direction_tolerance, int threads,
                           size_t row_begin, size_t row_end, double *data);

/* potential.c:139-253 and :261-395 */
int oracle_potential_pair(const Mesh *mesh, const DualMesh *dual, size_t i, size_t j,
                          const int orders[4], double near_factor, double *value);
/* Upper-triangle pairs of sampled rows of Lp (kind 0) or P (kind 1), default
 * options, for the CPU timing sample; out[k * n + b] = row rows[k]. */
int oracle_sample_rows(const Mesh *mesh, const DualMesh *dual, int kind, const size_t *rows,
                       size_t nrows, int threads, double *out);
int oracle_potential_matrix(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                            double near_factor, int threads, double *data);
int oracle_potential_rows(const Mesh *mesh, const DualMesh *dual, const int orders[4],
                          double near_factor, int threads, size_t row_begin,
                          size_t row_end, double *data);

/* lu.c:194-479: factor in place of a copy.  lu (n*n) receives packed L\U,
 * pivots (n) the pivot rows.  Returns 0 / -1 / -2 like the reference. */
int oracle_lu_factorize(const double *input, size_t n, double pivot_tolerance,
                        int threads, double *lu, size_t *pivots, size_t *swap_count,
                        double *matrix_scale);
/* lu.c:494-653 */
int oracle_lu_solve(const double *lu, const size_t *pivots, size_t n, const double *b,
                    double *x);

/* complex_lu.c:208-550 */
int oracle_complex_lu_factorize(const Complex *input, size_t n, double pivot_tolerance,
                                int threads, Complex *lu, size_t *pivots,
                                size_t *swap_count, double *matrix_scale,
                                double *row_scale, double *column_scale);
/* complex_lu.c:598-778 */
int oracle_complex_lu_solve(const Complex *lu, const size_t *pivots,
                            const double *row_scale, const double *column_scale,
                            size_t n, const Complex *b, Complex *x);

/* ---- transient stage 1 (lightning current at nodes) ----
 * scheme 1 backward Euler (theta 1), 2 trapezoidal (theta 1/2); edges holds
 * (a, b) per edge (current a -> b); R is the edge resistance diagonal or
 * NULL for PEC (zeros).
 *
 * transient.c:1020-1110 stage-1 blocks, with F = 1/diag(P)
 * (potential.c:483-520) and AS = A S (incidence.c:593-741):
 * M = [L/dt + theta R, theta AS; -theta A^T, F/dt], nt = ne + nv.
 * F (nv) and AS (ne x nv) are returned as well. */
int oracle_transient_stage1_matrix(const double *L, const double *P, const int *edges,
                                   const double *R, size_t ne, size_t nv, int scheme,
                                   double dt, double *M, double *F, double *AS);
/* transient.c:1421-1631 (edge voltages absent): rhs (nt) of one step */
int oracle_transient_rhs_stage1(const double *L, const double *R, const double *AS,
                                const double *F, const int *edges, size_t ne, size_t nv,
                                int scheme, double dt, const double *I, const double *V,
                                const double *Jn, const double *Jnp1, double *rhs);
/* lightning.c:184-212: K (exp(-alpha tau) - exp(-beta tau)), tau = t - delay */
double oracle_lightning_current(double K, double alpha, double beta, double delay, double t);
/* main.c:3139-3400: factor M once, then n_steps of source, rhs, solve and
 * extract, starting from I and V (updated in place).  probe_out receives,
 * after every step, V at the probe nodes then I at the probe edges
 * ([n_steps][n_probe_nodes + n_probe_edges]); it may be NULL. */
int oracle_transient_lightning(const double *L, const double *P, const int *edges,
                               const double *R, size_t ne, size_t nv, int scheme, double dt,
                               double K, double alpha, double beta, double delay,
                               size_t strike_node, size_t return_node, size_t n_steps,
                               double *I, double *V, const int *probe_nodes,
                               size_t n_probe_nodes, const int *probe_edges,
                               size_t n_probe_edges, double *probe_out);

/* ---- retarded kernel exp(-jkR)/R (no reference counterpart) ----
 * K_k = K_0 + D_k: K_0 the static patch-pair integral above (exact near
 * field), D_k the integral of (exp(-jkR) - 1)/R, smooth and bounded (limit
 * -jk at R = 0), by the far product rule of order far_order over both
 * patches' triangles for every patch pair.  Entries are scaled as Lp
 * (kind 0, zero for orthogonal edges) or P (kind 1).  out: n x n complex,
 * interleaved.  Parity unpinned: the reference has no retarded kernel; at
 * k = 0 this is the static matrix exactly. */
int oracle_retarded_matrix(const Mesh *mesh, const DualMesh *dual, int kind, const int orders[4],
                           double near_factor, double direction_tolerance, double wave_number,
                           int threads, double *out);

/* RCS radiation vector F(dir) = sum_e (I_e / w_e) G_e(dir) e_hat of one edge
 * current vector, dual-patch quadrature of `order` (rcs.c:701-1000). */
int oracle_rcs_radiation_vector(const Mesh *mesh, const DualMesh *dual, const Complex *current,
                                double wave_number, const double dir[3], int order, Complex out[3]);

#ifdef __cplusplus
}
#endif

/* Incidence products from an edge list (a, b), current a -> b
 * (incidence.c:242-415, 417-591, 593-741): K = A P A^T (ne x ne, e <= f
 * evaluated, mirrored); PAT = P A^T (nv x ne, NaN for an edge out of range;
 * returns -1 with *first_bad = the row-major index of the first non-finite
 * entry); AS = A S (ne x nv; returns -1 if a P[a][a] is not finite or <= 0). */
void oracle_incidence_apat(const double *P, const int *edges, size_t nv, size_t ne, double *K);
int oracle_incidence_pat(const double *P, const int *edges, size_t nv, size_t ne, double *out,
                         long long *first_bad);
int oracle_incidence_as(const double *P, const int *edges, size_t nv, size_t ne, double *AS);

#endif
