/*
 * Potential-coefficient matrix P (Nv x Nv, row-major, 1/F) and the small
 * helpers built on it.
 *
 * Drop-in for the reference's include/potential.h (types at
 * potential.h:15-78, functions at potential.h:84-239 of the reference
 * project).  The matrix is assembled on the GPU.
 *
 *   P_ij = 1/(4 pi eps0) / (S_i S_j) * sum_{patch pairs} K,
 *   S = node region area.
 */
#ifndef PEEC_POTENTIAL_H
#define PEEC_POTENTIAL_H

#include "dual_mesh.h"
#include "mesh.h"

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
    int far_order;
    int near_order;
    int touching_order;
    int self_order;
    double near_factor;
    int parallel_threads;       /* kept for ABI; must be >= 1 */
} PotentialOptions;

typedef struct
{
    size_t n;                   /* Nv                         */
    double *data;               /* P(i,j) = data[i*n + j]     */
} PotentialMatrix;

/* Orders 4/10/12/8, near_factor 0.5 (reference potential.c:38-58). */
void potential_options_default(PotentialOptions *options, int parallel_threads);

void potential_init(PotentialMatrix *P);
void potential_free(PotentialMatrix *P);

/* One entry P_ij on the GPU; 0 / -1 (reference potential.c:139-253). */
int potential_compute_pair(const Mesh *mesh, const DualMesh *dual,
                           size_t node_i, size_t node_j,
                           const PotentialOptions *options, double *value);

/* Whole matrix on the GPU; same ownership and error contract as
 * inductance_compute_matrix (reference potential.c:261-395). */
int potential_compute_matrix(const Mesh *mesh, const DualMesh *dual,
                             const PotentialOptions *options,
                             PotentialMatrix *P);

/* Reference potential.c:403-475. */
void potential_print_info(const PotentialMatrix *P);

/* F_j = 1/P_jj into caller memory; -1 if any P_jj <= 0 or non-finite
 * (reference potential.c:483-520). */
int potential_build_self_capacitance(const PotentialMatrix *P, double *F);

/* q_j = V_c,j / P_jj (reference potential.c:528-559). */
int potential_self_voltage_to_charge(const PotentialMatrix *P,
                                     const double *V_c, double *charge);

/* phi_j = sum_a P_ja V_c,a / P_aa (reference potential.c:567-612). */
int potential_self_voltage_to_full_potential(const PotentialMatrix *P,
                                             const double *V_c, double *phi);

#ifdef __cplusplus
}
#endif

#endif
