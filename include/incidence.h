/* Drop-in for the reference's include/incidence.h: the edge-node incidence
 * matrix A (Ne x Nv, A[e][a] = -1, A[e][b] = +1 for the globally oriented
 * edge e = a -> b) and the dense products the PEEC systems use.  The O(N^2)
 * products run on the GPU (csrc/incidence.cu); results are host arrays as in
 * the reference.  Device-resident forms are in peec_gb300.h. */
#ifndef PEEC_INCIDENCE_H
#define PEEC_INCIDENCE_H

#include <stddef.h>

#include "matrix.h"
#include "mesh.h"
#include "potential.h"

#ifdef __cplusplus
extern "C" {
#endif

/* incidence.h:47-54 */
typedef struct {
    size_t rows;
    size_t cols;
    double *data;
} IncidenceMatrix;

/* incidence.h:62-76: zero the struct / free data and zero it */
void incidence_init(IncidenceMatrix *A);
void incidence_free(IncidenceMatrix *A);

/* incidence.c:34-115: A = Ne x Nv, calloc'ed, two entries per row; -1 on a
 * missing topology or a node index out of range (with an ERROR message). */
int incidence_build(const Mesh *mesh, IncidenceMatrix *A);

/* incidence.c:117-154: max over rows of |sum of the row| (-1 for NULL). */
double incidence_check_row_sum(const IncidenceMatrix *A);

/* incidence.c:156-187: size, non-zero count and the expected 2 Ne on stdout. */
void incidence_print_info(const IncidenceMatrix *A);

/* incidence.c:242-415: K = A P A^T (Ne x Ne), K[e][f] = P[a][c] - P[a][d]
 * - P[b][c] + P[b][d] evaluated for e <= f and mirrored.  -1 on NULL input,
 * parallel_threads < 1, P->n != Nv, Ne or Nv = 0. */
int incidence_build_APAT(const Mesh *mesh, const PotentialMatrix *P, Matrix *K, int parallel_threads);

/* incidence.c:417-591: PAT = P A^T (Nv x Ne), PAT[j][e] = P[j][b] - P[j][a];
 * a column of an edge with a node out of range is NaN, and any non-finite
 * entry fails the call (-1, "invalid value in P A^T at [j,e]" for the first
 * in row-major order, PAT freed). */
int incidence_build_PAT(const Mesh *mesh, const PotentialMatrix *P, Matrix *PAT, int parallel_threads);

/* incidence.c:593-741: AS = A S (Ne x Nv), AS[e][a] = (P[n][a] - P[m][a]) /
 * P[a][a] with m / n the last columns of row e holding -1 / +1; -1 (AS
 * freed) when a row of A has another non-zero value or lacks -1 or +1, or a
 * P[a][a] is not finite or <= 0. */
int incidence_build_AS(const IncidenceMatrix *A, const PotentialMatrix *P, Matrix *AS, int parallel_threads);

#ifdef __cplusplus
}
#endif

#endif
