/*
 * Runs the reference's own harmonic scattering chain (TEST INFRASTRUCTURE
 * ONLY).  Compiled by `make -C oracle ref` against the reference's headers
 * and linked with its sources into oracle/_ref/libpeec_ref*.so.  The calls
 * follow the reference's driver (main.c:700-830 assembly, main.c:1266-1480
 * solve_harmonic_scattering): inductance_compute_matrix,
 * potential_compute_matrix, incidence_build_PAT, resistance_compute_matrix,
 * incident_field_configure_harmonic (COMPLEX wave) +
 * scattering_build_harmonic_excitation (analytic plane-wave edge integral),
 * harmonic_build_system, harmonic_factorize, harmonic_solve,
 * harmonic_compute_residual.  Each stage is timed with omp_get_wtime, as
 * the driver times it.
 *
 * residual[7] = {absolute_residual, rhs_relative_residual, backward_error,
 *                edge_absolute_residual, node_absolute_residual,
 *                edge_backward_error, node_backward_error}
 * times[8]    = {L, P, PAT, R + A, build, factor, solve, residual} seconds
 */
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "dual_mesh.h"
#include "harmonic.h"
#include "incidence.h"
#include "incident_field.h"
#include "inductance.h"
#include "mesh.h"
#include "potential.h"
#include "resistance.h"
#include "scattering.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static void residual_out(const HarmonicResidual *r, double out[7])
{
    out[0] = r->absolute_residual;
    out[1] = r->rhs_relative_residual;
    out[2] = r->backward_error;
    out[3] = r->edge_absolute_residual;
    out[4] = r->node_absolute_residual;
    out[5] = r->edge_backward_error;
    out[6] = r->node_backward_error;
}

/* Unit-amplitude COMPLEX plane wave (theta, phi in degrees; polarization 1
 * vertical e_theta, 0 horizontal e_phi), zero phase; U_inc per edge by the
 * analytic edge integral (analytic = 1) or the midpoint rule (0).  k_hat and
 * E0 of the configured field are returned when not NULL. */
int ref_plane_wave_excitation(const Mesh *mesh, double frequency, double theta_deg, double phi_deg,
                              int polarization, int analytic, int threads, Complex *U, double k_hat[3],
                              double E0[3])
{
    IncidentField field;
    incident_field_init(&field);
    if (incident_field_configure_harmonic(&field, INCIDENT_WAVE_COMPLEX, (IncidentPolarization)polarization, 1.0,
                                          frequency, theta_deg, phi_deg, 0.0) != 0)
        return -1;
    ScatteringOptions so;
    scattering_options_default(&so, threads);
    so.integration = analytic ? SCATTERING_EDGE_ANALYTIC_PLANE_WAVE : SCATTERING_EDGE_MIDPOINT;
    if (scattering_build_harmonic_excitation(mesh, &field, &so, U) != 0) return -1;
    for (int k = 0; k < 3; ++k) {
        if (k_hat) k_hat[k] = field.k_hat[k];
        if (E0) E0[k] = field.E0[k];
    }
    return 0;
}

/* Z of harmonic_build_system from given Lp, P and edge resistances (R NULL:
 * PEC), with A and P A^T built by the reference's incidence functions. */
int ref_harmonic_build(const Mesh *mesh, const double *L, const double *P, const double *R, double frequency,
                       int threads, Complex *Z)
{
    size_t ne = mesh->n_edges, nv = mesh->n_nodes, n = ne + nv;
    InductanceMatrix Lm = {.n = ne, .data = (double *)L};
    PotentialMatrix Pm = {.n = nv, .data = (double *)P};
    double *rdiag = calloc(ne, sizeof(double));
    if (!rdiag) return -1;
    if (R) memcpy(rdiag, R, ne * sizeof(double));
    ResistanceMatrix Rm = {.n = ne, .diagonal = rdiag};
    IncidenceMatrix A;
    incidence_init(&A);
    Matrix PAT;
    matrix_init(&PAT);
    HarmonicSystem sys;
    harmonic_system_init(&sys);
    int status = -1;
    if (incidence_build(mesh, &A) != 0 || incidence_build_PAT(mesh, &Pm, &PAT, threads) != 0 ||
        harmonic_build_system(&Lm, &Rm, &A, &PAT, frequency, threads, &sys) != 0)
        goto done;
    memcpy(Z, sys.matrix.data, n * n * sizeof(Complex));
    status = 0;
done:
    harmonic_system_free(&sys);
    matrix_free(&PAT);
    incidence_free(&A);
    free(rdiag);
    return status;
}

/* harmonic_compute_residual of a given Z (n = Ne + Nv, row-major), P, edge
 * excitation U (b = [-U; 0]) and solution x = [I; V]. */
int ref_harmonic_residual(const Complex *Z, size_t ne, size_t nv, double frequency, const double *P,
                          const Complex *U, const Complex *x, int threads, double residual[7])
{
    HarmonicSystem sys;
    harmonic_system_init(&sys);
    sys.n_edges = ne;
    sys.n_nodes = nv;
    sys.system_size = ne + nv;
    sys.frequency = frequency;
    sys.omega = 2.0 * M_PI * frequency;
    sys.matrix.rows = sys.matrix.cols = ne + nv;
    sys.matrix.data = (Complex *)Z;
    sys.matrix_built = 1;
    PotentialMatrix Pm = {.n = nv, .data = (double *)P};
    HarmonicExcitation ex = {.n_edges = ne, .n_nodes = nv, .edge_voltage = U, .node_current = NULL};
    HarmonicSolution sol = {.n_edges = ne, .n_nodes = nv, .edge_current = (Complex *)x,
                            .node_voltage = (Complex *)x + ne};
    HarmonicResidual r;
    if (harmonic_compute_residual(&sys, &Pm, &ex, &sol, threads, &r) != 0) return -1;
    residual_out(&r, residual);
    return 0;
}

/* The whole chain on one mesh.  sheet_resistance <= 0 means PEC.  Every
 * output pointer may be NULL except x. */
int ref_harmonic_pipeline(const Mesh *mesh, const DualMesh *dual, double frequency, double theta_deg,
                          double phi_deg, int polarization, double sheet_resistance, int threads,
                          double *L_out, double *P_out, double *R_out, Complex *Z_out, Complex *U_out,
                          Complex *x, size_t *piv_out, double *row_scale_out, double *column_scale_out,
                          double residual[7], double times[8])
{
    size_t ne = mesh->n_edges, nv = mesh->n_nodes, n = ne + nv;
    InductanceMatrix L;
    inductance_init(&L);
    PotentialMatrix P;
    potential_init(&P);
    Matrix PAT;
    matrix_init(&PAT);
    ResistanceMatrix R;
    resistance_init(&R);
    IncidenceMatrix A;
    incidence_init(&A);
    HarmonicSystem sys;
    harmonic_system_init(&sys);
    HarmonicSolution sol;
    harmonic_solution_init(&sol);
    Complex *U = malloc(ne * sizeof(Complex));
    double t[9];
    int status = -1;
    if (!U) return -1;

    t[0] = omp_get_wtime();
    InductanceOptions lo;
    inductance_options_default(&lo, threads);
    if (inductance_compute_matrix(mesh, dual, &lo, &L) != 0) goto done;
    t[1] = omp_get_wtime();
    PotentialOptions po;
    potential_options_default(&po, threads);
    if (potential_compute_matrix(mesh, dual, &po, &P) != 0) goto done;
    t[2] = omp_get_wtime();
    if (incidence_build_PAT(mesh, &P, &PAT, threads) != 0) goto done;
    t[3] = omp_get_wtime();
    ResistanceOptions ro;
    resistance_options_default(&ro, threads);
    if (sheet_resistance > 0.0) {
        ro.model = PEEC_CONDUCTOR_SHEET_RESISTANCE;
        ro.sheet_resistance = sheet_resistance;
    } else {
        ro.model = PEEC_CONDUCTOR_PEC;
    }
    if (resistance_compute_matrix(mesh, dual, &ro, &R) != 0 || incidence_build(mesh, &A) != 0) goto done;
    t[4] = omp_get_wtime();
    if (ref_plane_wave_excitation(mesh, frequency, theta_deg, phi_deg, polarization, 1, threads, U, NULL,
                                  NULL) != 0 ||
        harmonic_build_system(&L, &R, &A, &PAT, frequency, threads, &sys) != 0)
        goto done;
    t[5] = omp_get_wtime();
    if (Z_out) memcpy(Z_out, sys.matrix.data, n * n * sizeof(Complex));
    if (harmonic_factorize(&sys, threads) != 0) goto done;
    t[6] = omp_get_wtime();
    HarmonicExcitation ex = {.n_edges = ne, .n_nodes = nv, .edge_voltage = U, .node_current = NULL};
    if (harmonic_solve(&sys, &P, &ex, &sol, threads) != 0) goto done;
    t[7] = omp_get_wtime();
    HarmonicResidual r;
    if (harmonic_compute_residual(&sys, &P, &ex, &sol, threads, &r) != 0) goto done;
    t[8] = omp_get_wtime();

    memcpy(x, sol.edge_current, ne * sizeof(Complex));
    memcpy(x + ne, sol.node_voltage, nv * sizeof(Complex));
    if (L_out) memcpy(L_out, L.data, ne * ne * sizeof(double));
    if (P_out) memcpy(P_out, P.data, nv * nv * sizeof(double));
    if (R_out) memcpy(R_out, R.diagonal, ne * sizeof(double));
    if (U_out) memcpy(U_out, U, ne * sizeof(Complex));
    if (piv_out) memcpy(piv_out, sys.lu.pivots, n * sizeof(size_t));
    if (row_scale_out) memcpy(row_scale_out, sys.lu.row_scale, n * sizeof(double));
    if (column_scale_out) memcpy(column_scale_out, sys.lu.column_scale, n * sizeof(double));
    if (residual) residual_out(&r, residual);
    if (times)
        for (int k = 0; k < 8; ++k) times[k] = t[k + 1] - t[k];
    status = 0;
done:
    harmonic_solution_free(&sol);
    harmonic_system_free(&sys);
    incidence_free(&A);
    resistance_free(&R);
    matrix_free(&PAT);
    potential_free(&P);
    inductance_free(&L);
    free(U);
    return status;
}

/* Rows of Lp (kind 0) or P (kind 1) for a timing sample: the upper-triangle
 * pairs (a, b >= a) of the given rows with the reference's own per-pair
 * functions and default options, i.e. the work inductance_compute_matrix /
 * potential_compute_matrix do for those rows (inductance.c:390-560,
 * potential.c:261-395); the pairs of all sampled rows are spread over
 * `threads` OpenMP threads (dynamic schedule).  out[k * n + b] receives row
 * rows[k].  Returns 0, or -1 when a pair fails. */
int ref_sample_rows(const Mesh *mesh, const DualMesh *dual, int kind, const size_t *rows, size_t nrows,
                    int threads, double *out)
{
    size_t n = kind == 0 ? mesh->n_edges : mesh->n_nodes;
    size_t *start = malloc((nrows + 1) * sizeof(size_t));
    if (!start) return -1;
    start[0] = 0;
    for (size_t k = 0; k < nrows; ++k) start[k + 1] = start[k] + (rows[k] < n ? n - rows[k] : 0);
    InductanceOptions lo;
    inductance_options_default(&lo, 1);
    PotentialOptions po;
    potential_options_default(&po, 1);
    int failed = 0;
    long long total = (long long)start[nrows];
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
    for (long long t = 0; t < total; ++t) {
        size_t lo_k = 0, hi_k = nrows;
        while (hi_k - lo_k > 1) {
            size_t mid = (lo_k + hi_k) / 2;
            if (start[mid] <= (size_t)t) lo_k = mid; else hi_k = mid;
        }
        size_t a = rows[lo_k], b = a + ((size_t)t - start[lo_k]);
        double v = 0.0;
        int s = kind == 0 ? inductance_compute_pair(mesh, dual, a, b, &lo, &v)
                          : potential_compute_pair(mesh, dual, a, b, &po, &v);
        if (s != 0) {
#pragma omp atomic write
            failed = 1;
        }
        out[lo_k * n + b] = v;
    }
    free(start);
    return failed ? -1 : 0;
}

/* The solve part of the chain from given Lp, P and R (NULL: PEC), timed per
 * stage like the driver: incidence_build + incidence_build_PAT, the
 * excitation + harmonic_build_system, harmonic_factorize, harmonic_solve,
 * harmonic_compute_residual.  times[5] seconds; x (Ne + Nv) and residual[7]
 * as ref_harmonic_pipeline. */
int ref_harmonic_from_matrices(const Mesh *mesh, const double *L, const double *P, const double *R, double frequency,
                               double theta_deg, double phi_deg, int polarization, int threads, Complex *x,
                               double residual[7], double times[5])
{
    size_t ne = mesh->n_edges, nv = mesh->n_nodes;
    InductanceMatrix Lm = {.n = ne, .data = (double *)L};
    PotentialMatrix Pm = {.n = nv, .data = (double *)P};
    double *rdiag = calloc(ne, sizeof(double));
    Complex *U = malloc(ne * sizeof(Complex));
    IncidenceMatrix A;
    incidence_init(&A);
    Matrix PAT;
    matrix_init(&PAT);
    HarmonicSystem sys;
    harmonic_system_init(&sys);
    HarmonicSolution sol;
    harmonic_solution_init(&sol);
    int status = -1;
    double t[6];
    if (!rdiag || !U) goto done;
    if (R) memcpy(rdiag, R, ne * sizeof(double));
    ResistanceMatrix Rm = {.n = ne, .diagonal = rdiag};
    t[0] = omp_get_wtime();
    if (incidence_build(mesh, &A) != 0 || incidence_build_PAT(mesh, &Pm, &PAT, threads) != 0) goto done;
    t[1] = omp_get_wtime();
    if (ref_plane_wave_excitation(mesh, frequency, theta_deg, phi_deg, polarization, 1, threads, U, NULL, NULL) != 0 ||
        harmonic_build_system(&Lm, &Rm, &A, &PAT, frequency, threads, &sys) != 0)
        goto done;
    t[2] = omp_get_wtime();
    if (harmonic_factorize(&sys, threads) != 0) goto done;
    t[3] = omp_get_wtime();
    HarmonicExcitation ex = {.n_edges = ne, .n_nodes = nv, .edge_voltage = U, .node_current = NULL};
    if (harmonic_solve(&sys, &Pm, &ex, &sol, threads) != 0) goto done;
    t[4] = omp_get_wtime();
    HarmonicResidual r;
    if (harmonic_compute_residual(&sys, &Pm, &ex, &sol, threads, &r) != 0) goto done;
    t[5] = omp_get_wtime();
    memcpy(x, sol.edge_current, ne * sizeof(Complex));
    memcpy(x + ne, sol.node_voltage, nv * sizeof(Complex));
    if (residual) residual_out(&r, residual);
    for (int k = 0; k < 5; ++k) times[k] = t[k + 1] - t[k];
    status = 0;
done:
    harmonic_solution_free(&sol);
    harmonic_system_free(&sys);
    matrix_free(&PAT);
    incidence_free(&A);
    free(rdiag);
    free(U);
    return status;
}
