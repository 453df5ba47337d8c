/* Drop-in for the reference's include/matrix_export.h: PEEC matrices in the
 * Matrix Market text format (readable by scipy.io.mmread, MATLAB, Octave).
 * Dense matrices as "array real general" (column-major values, "%.17e"), the
 * incidence and resistance matrices as "coordinate real general".  Files are
 * byte-identical to the reference's; dense values are formatted by parallel
 * host threads and written in order.  Return 0, or -1 on NULL / empty input
 * or a file that cannot be opened. */
#ifndef PEEC_MATRIX_EXPORT_H
#define PEEC_MATRIX_EXPORT_H

#include <stddef.h>

#include "inductance.h"
#include "matrix.h"
#include "mesh.h"
#include "potential.h"
#include "resistance.h"

#ifdef __cplusplus
extern "C" {
#endif

/* matrix_export.c:105-176: rows x cols row-major data as an array */
int matrix_export_dense_mtx(const char *filename, const double *data, size_t rows, size_t cols);

/* matrix_export.c:178-258: A (Ne x Nv) as 2 Ne coordinates, 1-based */
int matrix_export_incidence_mtx(const char *filename, const Mesh *mesh);

/* matrix_export.c:260-321: diagonal R as n coordinates */
int matrix_export_resistance_mtx(const char *filename, const ResistanceMatrix *R);

/* matrix_export.c:323-432: directory (created with its parents, mode 0755)
 * with L.mtx, A.mtx, P.mtx, PAT.mtx, R.mtx, in that order; stops at the
 * first failure. */
int matrix_export_peec_set(const char *directory, const Mesh *mesh, const InductanceMatrix *L,
                           const PotentialMatrix *P, const Matrix *PAT, const ResistanceMatrix *R);

#ifdef __cplusplus
}
#endif

#endif
