/*
 * Dense real LU with partial pivoting, P A = L U.
 *
 * Drop-in for the reference's include/lu.h (types at lu.h:12-116, functions
 * at lu.h:122-253 of the reference project).  Factorisation and solves run
 * on the GPU; the packed factors and pivots are returned in host arrays with
 * the reference's layout:
 *   data   row-major n x n, unit-lower L below the diagonal, U on and above;
 *   pivots[k] = row swapped with row k at step k (applied in order k=0..n-1).
 * Return codes: 0 ok, -1 bad arguments / allocation, -2 numerically singular
 * (|pivot| <= pivot_tolerance * max|A|, or a non-finite pivot).
 */
#ifndef PEEC_LU_H
#define PEEC_LU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
    int parallel_threads;       /* kept for ABI; must be >= 1            */
    double pivot_tolerance;     /* relative to max|A_ij|                  */
    size_t parallel_threshold;  /* kept for ABI; no effect on the GPU     */
} LUOptions;

typedef struct
{
    size_t n;
    double *data;               /* packed L\U, row-major                  */
    size_t *pivots;             /* [n]                                     */
    size_t swap_count;          /* number of k with pivots[k] != k         */
    double matrix_scale;        /* max|A_ij| of the input                  */
    int factorized;
} LUFactorization;

/* tolerance 1e-14, threshold 64 (reference lu.c:16-48). */
void lu_options_default(LUOptions *options, int parallel_threads);

void lu_init(LUFactorization *lu);
void lu_free(LUFactorization *lu);

/* Factor a copy of input (input is not modified); starts with lu_init(lu)
 * (reference lu.c:194-479). */
int lu_factorize(const double *input, size_t n, const LUOptions *options,
                 LUFactorization *lu);

/* A x = b; x == b allowed (reference lu.c:603-653). */
int lu_solve(const LUFactorization *lu, const double *b, double *x);

/* A X = B for rhs_count right-hand sides stored one after another,
 * B[r*n + i] (reference lu.c:672-724). */
int lu_solve_multiple(const LUFactorization *lu, const double *B, double *X,
                      size_t rhs_count, int parallel_threads);

/* sign(P) * prod U_ii; NaN if not factorised (reference lu.c:732-754). */
double lu_determinant(const LUFactorization *lu);

/* Reference lu.c:762-793. */
void lu_print_info(const LUFactorization *lu);

#ifdef __cplusplus
}
#endif

#endif
