/*
 * Runs the reference's own stage-1 lightning transient (TEST INFRASTRUCTURE
 * ONLY).  Compiled by `make -C oracle ref` against the reference's headers
 * and linked with its sources into oracle/_ref/libpeec_ref.so; it drives the
 * reference API the way its driver does (main.c:3139-3400):
 * transient_system_create_stage1, transient_factorize, then per step
 * lightning_build_node_current at t_n and t_n+1, transient_build_rhs_stage1,
 * transient_solve_step and transient_extract_stage1_solution.
 */
#include <stdlib.h>
#include <string.h>

#include "incidence.h"
#include "inductance.h"
#include "lightning.h"
#include "mesh.h"
#include "potential.h"
#include "resistance.h"
#include "transient.h"

int ref_transient_lightning(const double *L, const double *P, const int *edges, const double *R,
                            size_t ne, size_t nv, int scheme, double dt, double K, double alpha,
                            double beta, double delay, size_t strike_node, size_t return_node,
                            size_t n_steps, double *I, double *V, const int *probe_nodes,
                            size_t n_probe_nodes, const int *probe_edges, size_t n_probe_edges,
                            double *probe_out)
{
    Mesh mesh;
    memset(&mesh, 0, sizeof(mesh));
    mesh.n_edges = ne;
    mesh.n_nodes = nv;
    mesh.edges = (int *)edges;
    IncidenceMatrix A;
    incidence_init(&A);
    if (incidence_build(&mesh, &A) != 0) return -1;
    double *rdiag = calloc(ne, sizeof(double));
    double *src_n = calloc(nv, sizeof(double)), *src_np1 = calloc(nv, sizeof(double));
    if (!rdiag || !src_n || !src_np1) return -1;
    if (R) memcpy(rdiag, R, ne * sizeof(double));
    InductanceMatrix Lm = {.n = ne, .data = (double *)L};
    PotentialMatrix Pm = {.n = nv, .data = (double *)P};
    ResistanceMatrix Rm = {.n = ne, .diagonal = rdiag};
    LightningSource src;
    lightning_source_default(&src);
    src.K = K;
    src.alpha = alpha;
    src.beta = beta;
    src.delay = delay;
    src.strike_node = strike_node;
    src.return_node = return_node;
    TransientSystem sys;
    transient_system_init(&sys);
    int status = -1;
    if (transient_system_create_stage1(&sys, &Lm, &Rm, &A, &Pm, (TransientScheme)scheme, dt) != 0 ||
        transient_factorize(&sys, 1) != 0)
        goto done;
    size_t np = n_probe_nodes + n_probe_edges;
    for (size_t step = 0; step < n_steps; ++step) {
        double t_n = step * dt, t_np1 = (step + 1) * dt;
        if (lightning_build_node_current(&src, nv, t_n, src_n) != 0 ||
            lightning_build_node_current(&src, nv, t_np1, src_np1) != 0 ||
            transient_build_rhs_stage1(&sys, I, V, src_n, src_np1, NULL, NULL) != 0 ||
            transient_solve_step(&sys) != 0 || transient_extract_stage1_solution(&sys, I, V) != 0)
            goto done;
        if (probe_out) {
            for (size_t k = 0; k < n_probe_nodes; ++k) probe_out[step * np + k] = V[probe_nodes[k]];
            for (size_t k = 0; k < n_probe_edges; ++k)
                probe_out[step * np + n_probe_nodes + k] = I[probe_edges[k]];
        }
    }
    status = 0;
done:
    transient_system_free(&sys);
    incidence_free(&A);
    free(rdiag);
    free(src_n);
    free(src_np1);
    return status;
}
