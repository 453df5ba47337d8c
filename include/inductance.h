/*
 * Partial-inductance matrix Lp (Ne x Ne, row-major, henry).
 *
 * Drop-in for the reference's include/inductance.h (types at
 * inductance.h:15-87, functions at inductance.h:95-180 of the reference
 * project).  Same structs, same signatures, same return codes; the matrix is
 * assembled on the GPU and returned in a malloc'ed host array that the
 * caller releases with inductance_free().
 *
 *   L_ab = mu0/(4 pi) * (e_a . e_b) / (w_a w_b) * sum_{patch pairs} K,
 *   w = (edge region area) / (edge length),
 *   L_ab = 0 exactly when |e_a . e_b| < direction_tolerance.
 */
#ifndef PEEC_INDUCTANCE_H
#define PEEC_INDUCTANCE_H

#include "dual_mesh.h"
#include "mesh.h"

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
    int far_order;              /* Gauss-Legendre order, FAR pairs      */
    int near_order;             /* outer order, NEAR pairs              */
    int touching_order;         /* outer order, TOUCHING pairs          */
    int self_order;             /* outer order, SELF pairs              */
    double near_factor;         /* NEAR if gap < near_factor * size     */
    int parallel_threads;       /* kept for ABI; must be >= 1           */
    double direction_tolerance; /* orthogonality cut-off for e_a . e_b  */
} InductanceOptions;

typedef struct
{
    size_t n;                   /* Ne                                   */
    double *data;               /* L(a,b) = data[a*n + b]               */
} InductanceMatrix;

/* Orders 4/10/12/8, near_factor 0.5, direction_tolerance 1e-10
 * (reference inductance.c:46-97). */
void inductance_options_default(InductanceOptions *options, int parallel_threads);

/* Zero the struct; does not free (reference inductance.c:105-113). */
void inductance_init(InductanceMatrix *L);

/* free(data) and zero the struct (reference inductance.c:121-131). */
void inductance_free(InductanceMatrix *L);

/* One entry L_ab computed on the GPU.  0 on success; -1 on bad arguments,
 * empty regions, non-positive widths or a non-finite integral
 * (reference inductance.c:221-382). */
int inductance_compute_pair(const Mesh *mesh, const DualMesh *dual,
                            size_t edge_a, size_t edge_b,
                            const InductanceOptions *options, double *value);

/* Whole matrix on the GPU.  Starts with inductance_init(L) (no free),
 * allocates L->data with calloc; on any failure prints an "ERROR:" line,
 * frees the data and returns -1 (reference inductance.c:390-560). */
int inductance_compute_matrix(const Mesh *mesh, const DualMesh *dual,
                              const InductanceOptions *options,
                              InductanceMatrix *L);

/* Size, range, diagonal range and symmetry error on stdout
 * (reference inductance.c:568-646). */
void inductance_print_info(const InductanceMatrix *L);

#ifdef __cplusplus
}
#endif

#endif
