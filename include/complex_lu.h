/*
 * Dense complex LU with row/column equilibration and partial pivoting.
 *
 * Drop-in for the reference's include/complex_lu.h (types at
 * complex_lu.h:14-71, functions at complex_lu.h:77-161 of the reference
 * project).  Runs on the GPU; results in host arrays:
 *   Aeq = diag(1/row_scale) A diag(1/column_scale),  P Aeq = L U,
 *   row_scale[i]    = max_j |A_ij|,
 *   column_scale[j] = max_i |A_ij / row_scale[i]|,
 *   data packed L\U of Aeq, row-major, interleaved {re, im}.
 * Return codes as for the real LU; a zero row or column, or a non-finite
 * entry, gives -2.
 */
#ifndef PEEC_COMPLEX_LU_H
#define PEEC_COMPLEX_LU_H

#include "complex_matrix.h"

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
    int parallel_threads;       /* kept for ABI; must be >= 1               */
    double pivot_tolerance;     /* relative to max|Aeq_ij|; finite and >= 0  */
    size_t parallel_threshold;  /* kept for ABI; no effect on the GPU        */
} ComplexLUOptions;

typedef struct
{
    size_t n;
    Complex *data;
    size_t *pivots;
    size_t swap_count;
    double matrix_scale;        /* max|Aeq_ij|                               */
    double *row_scale;          /* [n]                                       */
    double *column_scale;       /* [n]                                       */
    int factorized;
} ComplexLUFactorization;

/* tolerance 1e-14, threshold 64 (reference complex_lu.c:16-29). */
void complex_lu_options_default(ComplexLUOptions *options, int parallel_threads);

void complex_lu_init(ComplexLUFactorization *lu);
void complex_lu_free(ComplexLUFactorization *lu);

/* Reference complex_lu.c:208-550. */
int complex_lu_factorize(const Complex *input, size_t n,
                         const ComplexLUOptions *options,
                         ComplexLUFactorization *lu);

/* x = column-unscale( LU-solve( row-scale(b) ) ) (reference complex_lu.c:724-778). */
int complex_lu_solve(const ComplexLUFactorization *lu, const Complex *b, Complex *x);

/* B[r*n + i] layout (reference complex_lu.c:786-840). */
int complex_lu_solve_multiple(const ComplexLUFactorization *lu, const Complex *B,
                              Complex *X, size_t rhs_count, int parallel_threads);

/* Reference complex_lu.c:848-897. */
void complex_lu_print_info(const ComplexLUFactorization *lu);

#ifdef __cplusplus
}
#endif

#endif
