/*
 * Extension API of the GB300 PEEC library (no counterpart in the reference).
 *
 * The drop-in headers (inductance.h, potential.h, lu.h, complex_lu.h,
 * quadrature.h) keep the reference's host-array contract.  This header adds
 * what a GPU-resident caller needs: device buffers, the library stream, CUDA
 * event timing, assembly straight into device memory and work counters.
 * Unchanged reference drivers never include it.
 */
#ifndef PEEC_GB300_H
#define PEEC_GB300_H

#include <stddef.h>

#include "dual_mesh.h"
#include "inductance.h"
#include "mesh.h"
#include "potential.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Work and timing of one assembly (filled when a pointer is passed). */
typedef struct
{
    unsigned long long near_pairs;             /* non-FAR patch pairs integrated analytically */
    unsigned long long potential_evaluations;  /* analytic triangle-potential evaluations     */
    double ms_prepare;                         /* patch prep + near-pair discovery (CUDA events) */
    double ms_near;                            /* adaptive near-field kernels                 */
    double ms_far;                             /* tiled far-field + combine kernel            */
} PeecAssemblyStats;

/* 1 if a CUDA device is usable by the library, else 0. */
int peec_gb300_device_ready(void);

/* Text of the last error recorded on this thread. */
const char *peec_gb300_last_error(void);

/* Number of kernels this library has launched since it was loaded. */
unsigned long long peec_gb300_launch_count(void);

/* The library's CUDA stream (cudaStream_t), on which every call enqueues. */
void *peec_gb300_stream(void);

void *peec_gb300_device_alloc(size_t bytes);
void peec_gb300_device_free(void *p);
void *peec_gb300_host_alloc_pinned(size_t bytes);
void peec_gb300_host_free_pinned(void *p);
/* Synchronous copies on the library stream; 0 or -1. */
int peec_gb300_copy_to_device(void *dst, const void *src, size_t bytes);
int peec_gb300_copy_to_host(void *dst, const void *src, size_t bytes);
int peec_gb300_synchronize(void);

/* CUDA events recorded on the library stream. */
void *peec_gb300_event_record(void);
double peec_gb300_event_elapsed_ms(void *start, void *stop);
void peec_gb300_event_destroy(void *event);

/* Lp / P written to device memory d_out (n*n doubles, row-major) with the
 * same options, numerics and errors as inductance_compute_matrix /
 * potential_compute_matrix. */
int peec_gb300_inductance_device(const Mesh *mesh, const DualMesh *dual,
                                 const InductanceOptions *options, double *d_out,
                                 PeecAssemblyStats *stats);
int peec_gb300_potential_device(const Mesh *mesh, const DualMesh *dual,
                                const PotentialOptions *options, double *d_out,
                                PeecAssemblyStats *stats);

#ifdef __cplusplus
}
#endif

#endif
