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

#include "complex_matrix.h"
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
    unsigned long long far_point_pairs;        /* far-rule 1/R point pairs (FAR patch pairs x (2q^2)^2) */
    unsigned long long near_pairs_evaluated;   /* near pairs integrated (the rest reuse a translated copy) */
    unsigned long long near_pairs_reevaluated; /* of those: copies integrated again because their
                                                  representative's adaptive decisions were marginal */
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

/* The calling host thread's CUDA stream (cudaStream_t): each host thread has
 * its own, every call from that thread enqueues on it, and calls from
 * different threads overlap on the device. */
void *peec_gb300_stream(void);

void *peec_gb300_device_alloc(size_t bytes);
void peec_gb300_device_free(void *p);
void *peec_gb300_host_alloc_pinned(size_t bytes);
void peec_gb300_host_free_pinned(void *p);
/* Synchronous copies on the library stream; 0 or -1. */
int peec_gb300_copy_to_device(void *dst, const void *src, size_t bytes);
int peec_gb300_copy_to_host(void *dst, const void *src, size_t bytes);
/* Asynchronous device-to-device copy on the library stream. */
int peec_gb300_copy_device(void *dst, const void *src, size_t bytes);
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

/* Far-rule arithmetic of later assemblies (all entry points): 0 native FP64,
 * 1 double-float on the FP32 pipes (default; FP64-accurate, parity 1e-12),
 * 2 FP32 with FP32 accumulation (mixed-precision path, ~1e-7 relative).
 * Returns the previous mode.  Not thread-safe against concurrent assemblies. */
int peec_gb300_set_far_precision(int mode);

/* Reuse of translated near pairs (default on): near patch pairs whose
 * corners are translated copies of each other (to a few ulps of the largest
 * coordinate) share one adaptive evaluation.  Returns the previous setting. */
int peec_gb300_set_near_reuse(int on);

/* ---- dense factorisations of device-resident matrices (in place) ----
 * Same algorithm, numerics and error codes as lu_factorize /
 * complex_lu_factorize.  d_piv (n int64) receives the pivot rows, d_perm (n
 * int32) the combined row permutation the solves use.  failed_column is the
 * column of a singular pivot, or -1. */
int peec_gb300_lu_factor_device(double *d_a, size_t n, double pivot_tolerance,
                                long long *d_piv, int *d_perm, double *matrix_scale,
                                int *failed_column);
int peec_gb300_complex_lu_factor_device(Complex *d_a, size_t n, double pivot_tolerance,
                                        long long *d_piv, int *d_perm,
                                        double *d_row_scale, double *d_column_scale,
                                        double *matrix_scale, int *failed_column);
/* Same as peec_gb300_lu_factor_device, but allocates no device memory (no
 * cudaMalloc, cudaFree or allocating library call), for callers that own all
 * device memory through their own pool or hard budget, or that must not let
 * cudaMalloc / cudaFree synchronise the device inside a solver loop.  Its
 * scratch (status, scale reduction, panel exchange slots) lives in one
 * 256 KiB static device array that every GPU loading the library keeps until
 * the process exits; n is limited to 50000 (larger n returns -1 with a
 * message, see peec_gb300_last_error).  Each call looks up the array's
 * device address on the current device.  Every call reuses the same array and
 * clears it on entry, so calls that overlap on the GPU (for instance from two
 * host threads) race with each other: serialise them.  The call synchronises
 * the library stream before returning (it reads the matrix scale and the
 * status back). */
int peec_gb300_lu_factor_device_noalloc(double *d_a, size_t n, double pivot_tolerance,
                                        long long *d_piv, int *d_perm,
                                        double *matrix_scale, int *failed_column);
/* Device copies of host factorisations (lu_factorize / complex_lu_factorize
 * results) stay registered for later lu_solve / complex_lu_solve calls.
 * trust = 0 (default): every solve uploads the caller's current host factor
 * into the registered buffers, so edits of the factor between calls are
 * seen.  trust = 1: a registered copy is reused without re-reading the host
 * factor while the pointer, size, pivots, scales, diagonal and a strided
 * sample of 4093 entries are unchanged; set it only if no factor is edited
 * between solves.  Returns the previous setting. */
int peec_gb300_set_factor_cache(int trust);

/* nrhs right-hand sides stored one after another; d_b != d_x. */
int peec_gb300_lu_solve_device(const double *d_lu, const int *d_perm, size_t n,
                               const double *d_b, double *d_x, size_t nrhs);
int peec_gb300_complex_lu_solve_device(const Complex *d_lu, const int *d_perm,
                                       const double *d_row_scale,
                                       const double *d_column_scale, size_t n,
                                       const Complex *d_b, Complex *d_x, size_t nrhs);

/* Per-phase timing of the allocating factorisations (events around each
 * block column's panel, swaps + triangular solve, trailing update).
 * peec_gb300_lu_timing returns -1 unless enabled. */
void peec_gb300_lu_timing_enable(int on);
int peec_gb300_lu_timing(double *ms_panel, double *ms_swap_trsm, double *ms_update,
                         double *update_flops);
/* Of the last timed mixed-precision factorisation: the time (ms) and issued
 * BF16 tensor flops of the outer-block trailing GEMMs alone (K = 6 x 256,
 * operand splits excluded); -1 unless timing is enabled. */
int peec_gb300_lu_timing_trailing(double *ms, double *issued_flops);

/* Measured FMA issue rates of this GPU's FP64 and FP32 pipes (TFLOP/s). */
int peec_gb300_pipe_peaks(double *fp64_tflops, double *fp32_tflops);

/* ---- tensor-core building block ----
 * C_j (FP32, row-major, leading dimension ldc) -= A B_j^T for device BF16
 * matrices A [m][k] and B_j [n][k] (K contiguous), j < J (J = 1 or 2), on
 * tcgen05 with TMA-fed operands and FP32 accumulation in tensor memory.
 * k must be a multiple of 64; A, B_j 16-byte aligned. */
int peec_gb300_tc_gemm(const void *d_a, const void *d_b0, const void *d_b1, float *d_c0,
                       float *d_c1, int m, int n, int k, long long ldc, int J);

/* Complex form used by the mixed-precision LU: C (interleaved FP32 complex,
 * leading dimension ldc complex elements) [row0 + i][col0 + j] -=
 * (A Br^T)[i][j] + j (A Bi^T)[i][j] for i < m, j < n; BF16 A [m][k],
 * Br / Bi [n][k].  A 16-byte aligned block with an even ldc runs on the
 * persistent kernel (TMEM double-buffered accumulators, TMA epilogue). */
int peec_gb300_tc_gemm_cplx(const void *d_a, const void *d_br, const void *d_bi, float *d_c, int m,
                            int n, int k, int row0, int col0, long long ldc);

/* ---- RCS radiation vectors (rcs.c:701-1000, dual-patch quadrature) ----
 * For every direction d (directions: host [n_dir][3], unit vectors) and
 * every solution s (edge currents on the device, solution s at
 * d_current + s * current_stride, current_stride >= n_edges: e.g. the
 * harmonic solution vectors, whose first n_edges entries are the edge
 * currents), radiation[(d * n_rhs + s) * 3 + c] (host) =
 * sum_e (I_e / w_e) G_e(d) e_hat_c with G_e the surface_order Gauss rule of
 * exp(j k d.r) over the edge's dual patches, w_e = S_e / l_e; edges with
 * l_e <= 0 or S_e <= 0 contribute nothing.  FP64; returns 0, or -1 on
 * invalid input (k <= 0, unsupported order, mesh and dual mismatch). */
int peec_gb300_rcs_radiation_device(const Mesh *mesh, const DualMesh *dual, const Complex *d_current,
                                    size_t n_rhs, size_t current_stride, double wave_number,
                                    const double *directions, size_t n_dir, int order,
                                    Complex *radiation);

/* ---- incidence products (incidence.h) on device-resident P ----
 * d_P: nv x nv FP64 row-major; d_edges: [2 ne] (a, b) node pairs, current
 * a -> b.  Outputs are device arrays, row-major, bit-identical to the
 * reference's expressions.
 * P A^T (nv x ne): d_out[j][e] = P[j][b] - P[j][a], NaN for an edge with a
 * node out of range; returns 0, 1 when an entry is not finite (*first_bad =
 * its row-major index, else -1; may be NULL), -1 on invalid arguments. */
int peec_gb300_pat_device(const double *d_P, const int *d_edges, size_t nv, size_t ne, double *d_out,
                          long long *first_bad);
/* A P A^T (ne x ne): d_K[e][f] = P[a][c] - P[a][d] - P[b][c] + P[b][d] for
 * e <= f, mirrored.  Returns 0, or -1 on invalid arguments or a node index
 * out of range. */
int peec_gb300_apat_device(const double *d_P, const int *d_edges, size_t nv, size_t ne, double *d_K);
/* A S (ne x nv): d_AS[e][a] = (P[b][a] - P[a'][a]) / P[a][a] for edge
 * e = a' -> b.  Returns 0, 1 when a P[a][a] is not finite or <= 0 (those
 * entries NaN), -1 on invalid arguments or edges (a node out of range or
 * a' == b). */
int peec_gb300_as_device(const double *d_P, const int *d_edges, size_t nv, size_t ne, double *d_AS);

/* ---- mixed precision complex solve ----
 * The FP32 rounding used by the mixed-precision solve's equilibration:
 * d_y[i] = d_x[i] * 2^-shift rounded to the nearest FP32 (ties to even) by
 * integer operations on the FP64 bits; results below 2^-126 flush to zero,
 * beyond the FP32 range give +-inf, NaN stays NaN. */
int peec_gb300_round_to_f32_device(const double *d_x, float *d_y, size_t count, int shift);

/* Solves Z X = B (n x n FP64 complex, nrhs right-hand sides stored one after
 * another) to a componentwise backward error <= tol: row and column
 * equilibration by powers of two, FP32 LU whose trailing updates run on the
 * tensor cores as split-BF16x3 products (FP32 accumulation), then FP64
 * iterative refinement r = B - Z X from X = 0.  When the refinement stalls
 * (a backward error that is not finite, or a smallest backward error so far
 * not a factor 4 below the smallest three sweeps earlier) or the FP32 pivots
 * break down, the FP32 copy of Z is factored again with split-BF16x6
 * products (three-part operands, FP32-equivalent) and refined again from
 * X = 0, until the gate, max_iter sweeps, or no factor 2 of progress over
 * six sweeps.  If that stalls too, FGMRES-IR with the BF16x6 factor as the
 * preconditioner (per right-hand side from X = 0: FP64 residual, inner
 * flexible GMRES on the row-equilibrated correction equation to 1e-6
 * relative or 40 steps, at most 10 outer steps).  d_Z and d_b are not modified.  Returns 0 when converged, 1 when
 * the refinement did not reach tol (X holds the last iterate), -2 for a zero /
 * non-finite row or column or a singular FP32 pivot, -1 on other errors.
 * backward_error / iterations (sweeps of all attempts) may be NULL. */
int peec_gb300_complex_solve_mixed_device(const Complex *d_Z, size_t n, const Complex *d_b,
                                          Complex *d_x, size_t nrhs, double tol, int max_iter,
                                          double *backward_error, int *iterations);
/* Split-BF16 product terms (3 or 6) of the last mixed solve's final
 * factorisation on this host thread. */
int peec_gb300_mixed_split_terms(void);
/* Inner FGMRES steps of the last mixed solve on this host thread (0 unless
 * refinement from the BF16x6 factor stalled and FGMRES-IR ran); one step
 * serves up to 8 right-hand sides in lockstep. */
int peec_gb300_mixed_gmres_iterations(void);
/* FP64 iterative refinement of d_x (in: a solution, out: the refined one)
 * with an FP64 factor of Z from peec_gb300_complex_lu_factor_device:
 * r = b - Z x, x += (LU)^-1 r until the componentwise backward error
 * <= tol.  Returns 0 when reached, 1 when not after max_iter corrections,
 * -1 on errors.  The server uses it when a mixed solve falls back to FP64. */
int peec_gb300_complex_refine_device(const Complex *d_Z, const Complex *d_lu, const int *d_perm,
                                     const double *d_row_scale, const double *d_column_scale,
                                     size_t n, const Complex *d_b, Complex *d_x, size_t nrhs,
                                     double tol, int max_iter, double *backward_error,
                                     int *iterations);
/* Phase times (ms) of the last mixed solve; returns its iteration count. */
int peec_gb300_mixed_timing(double *ms_prepare, double *ms_factor, double *ms_refine);

/* ---- harmonic system on the device ----
 * Z = [R + j w L, A; -P A^T, j w I] (N = Ne + Nv) from device Lp, P and the
 * edge list (2*Ne int32, a -> b); d_R (Ne diagonal) may be NULL for PEC.
 * Mirrors the reference's harmonic_build_system. */
int peec_gb300_harmonic_build_device(const double *d_L, const double *d_P,
                                     const int *d_edges, const double *d_R,
                                     size_t n_edges, size_t n_nodes, double frequency,
                                     Complex *d_Z);
/* [-U_e; 0] for a plane wave e_hat exp(-j k0 k_hat.r), U_e the field at the
 * edge centre projected on the edge vector times sinc(k0 k_hat.l / 2): the
 * reference's scattering_build_harmonic_excitation with the analytic edge
 * integral (scattering.c:140-336) for a COMPLEX wave of zero phase whose
 * k_hat and E0 (= e_hat) come from incident_field_configure_harmonic. */
int peec_gb300_plane_wave_rhs_device(const double *d_edge_centers,
                                     const double *d_edge_vectors, size_t n_edges,
                                     size_t n_nodes, const double k_hat[3],
                                     const double e_hat[3], double wave_number,
                                     Complex *d_rhs);
/* out[0] = max_i |r_i| / (sum_j |Z_ij||x_j| + |b_i|) over all right-hand
 * sides (r = b - Z x in FP64; the denominator's sum from FP32 magnitudes,
 * ~1e-7 relative, which only matters for a gate on eta), out[1] = max |r_i|,
 * out[2] = max |b_i|. */
int peec_gb300_backward_error_device(const Complex *d_Z, size_t n, const Complex *d_x,
                                     const Complex *d_b, size_t nrhs, double out[3]);

/* ---- batched frequency sweep (no reference counterpart) ----
 * The harmonic systems of one mesh at many frequencies, each with nrhs
 * plane waves, solved by the mixed-precision solve recorded once into a
 * CUDA graph and replayed per frequency (omega and k0 are device data of the
 * graph).  A plan keeps pointers to the caller's device Lp, P, edge list,
 * resistance diagonal (NULL: PEC), edge centres and edge vectors (keep them
 * valid while it lives) and copies the waves (k_hat, e_hat: host [nrhs][3]).
 * Different meshes' plans run from different host threads to overlap. */
typedef struct
{
    int split_terms; /* split-BF16 products of the FP32 factorisation: 3 or 6 */
    int sweeps;      /* FP64 refinement sweeps recorded in the graph (at most; a
                        sweep after the one that reaches 1e-10 does nothing) */
    int tile_bn;     /* width of the wide tensor-core update tiles: 64, 128, or 0 (by shape) */
} PeecSweepTuning;

/* NULL on invalid input or allocation failure.  tuning NULL: {3, 10, 0}. */
void *peec_gb300_sweep_create(const double *d_L, const double *d_P, const int *d_edges, const double *d_R,
                              const double *d_edge_centers, const double *d_edge_vectors, size_t n_edges,
                              size_t n_nodes, size_t nrhs, const double *k_hat, const double *e_hat,
                              const PeecSweepTuning *tuning);
/* Autotuner: replays a fast graph (BF16x3, up to 10 sweeps; sweeps after
 * the one that reaches 1e-10 do nothing) at the probe frequencies (at most
 * 64); the lowest frequency from which every probe reaches 1e-10 becomes
 * the split frequency, below which a robust graph (BF16x6, up to 16 sweeps)
 * runs; the 128- and 64-column tiles of the wide updates are timed at the
 * top probe and the faster kept.  chosen (the fast graph's tuning) and
 * ms_per_system (its replay time) may be NULL. */
int peec_gb300_sweep_tune(void *plan, const double *probe_frequencies, size_t n_probe,
                          PeecSweepTuning *chosen, double *ms_per_system);
/* Solves every frequency: d_X (device) [n_freq][nrhs][Ne + Nv].  A system
 * that the fast graph leaves above tol is replayed with the robust graph
 * (recorded then if the tuner did not need it); one still above tol is solved
 * again outside the graphs (mixed solve with its precision ladder; then the
 * FP64 LU with FP64 refinement).  backward_error[f] (host) is its final
 * componentwise backward error; fallback[f] 0 graph, 3 robust graph after
 * the fast one, 1 mixed ladder, 2 FP64.  Returns 0 when every system reached
 * tol, 1 when some did not, -1 on errors. */
int peec_gb300_sweep_run(void *plan, const double *frequencies, size_t n_freq, double tol,
                         Complex *d_X, double *backward_error, int *fallback);
int peec_gb300_sweep_tuning(void *plan, PeecSweepTuning *tuning);
/* The frequency below which the plan replays its robust graph (BF16x6, more
 * sweeps; 0 when it has none) and that graph's tuning. */
int peec_gb300_sweep_split(void *plan, double *split_frequency, PeecSweepTuning *robust);
void peec_gb300_sweep_destroy(void *plan);

/* ---- retarded Lp / P (no reference counterpart: the reference's
 * retardation.c is empty) ----
 * Lp and P with the kernel exp(-jkR)/R, k = wave_number (rad/m, >= 0),
 * n x n complex in device memory.  Each patch-pair integral is the static
 * one of peec_gb300_inductance_device / _potential_device (exact near field,
 * FP64) plus the integral of (exp(-jkR) - 1)/R -- smooth and bounded -- by
 * the far product rule over every patch pair, evaluated on the FP32 pipes
 * (~1e-6 relative error on that correction).  k = 0 gives the static
 * matrices exactly, with zero imaginary parts. */
int peec_gb300_inductance_retarded_device(const Mesh *mesh, const DualMesh *dual,
                                          const InductanceOptions *options, double wave_number,
                                          Complex *d_out, PeecAssemblyStats *stats);
int peec_gb300_potential_retarded_device(const Mesh *mesh, const DualMesh *dual,
                                         const PotentialOptions *options, double wave_number,
                                         Complex *d_out, PeecAssemblyStats *stats);
/* Z of peec_gb300_harmonic_build_device from complex Lp and P. */
int peec_gb300_harmonic_build_retarded_device(const Complex *d_L, const Complex *d_P,
                                              const int *d_edges, const double *d_R,
                                              size_t n_edges, size_t n_nodes, double frequency,
                                              Complex *d_Z);

/* ---- stage-1 transient (lightning) on the device ----
 * The reference's transient_system_create_stage1 + transient_factorize
 * (transient.c:385-480, 1020-1110, 2014-2066): M = [L/dt + theta R,
 * theta A S; -theta A^T, F/dt] built from device Lp (kept by pointer: it
 * must stay valid while the system lives), P, the edge list (2*Ne int32,
 * a -> b) and the edge resistance diagonal d_R (NULL: PEC), then factorised
 * and kept on the device.  scheme 1 backward Euler, 2 trapezoidal.  Returns
 * 0, -1 (invalid input or CUDA error), -2 (singular system). */
int peec_gb300_transient_create(const double *d_L, const double *d_P, const int *d_edges,
                                const double *d_R, size_t n_edges, size_t n_nodes, int scheme,
                                double dt, void **system);
/* n_steps steps starting at t = step0*dt under the double-exponential
 * lightning current K (exp(-alpha tau) - exp(-beta tau)), tau = t - delay,
 * injected at strike_node and returned at return_node (per step:
 * lightning_build_node_current at t_n and t_n+1, transient_build_rhs_stage1,
 * transient_solve_step).  d_I (Ne) and d_V (Nv, node self-voltages) hold the
 * state on entry and on exit.  d_probes, if the probe counts are not zero,
 * receives after every step V at the probe nodes then I at the probe edges
 * ([n_steps][n_probe_nodes + n_probe_edges]; an index outside the mesh
 * records NaN).  Several runs may use one system at once (each call keeps
 * its own state and scratch). */
int peec_gb300_transient_lightning(void *system, double K, double alpha, double beta,
                                   double delay, size_t strike_node, size_t return_node,
                                   size_t step0, size_t n_steps, double *d_I, double *d_V,
                                   const int *d_probe_nodes, size_t n_probe_nodes,
                                   const int *d_probe_edges, size_t n_probe_edges,
                                   double *d_probes);
/* nrun (1 to 8) lightning runs on one system stepped together: run r has
 * its own source (K[r], alpha[r], beta[r], delay[r], strike_node[r],
 * return_node[r]) and state d_X + r (Ne + Nv) = [I; V] (in and out); every
 * step reads Lp, A S and the system's inverse once for all runs.  d_probes:
 * [n_steps][nrun][n_probe_nodes + n_probe_edges].  Each run's result is the
 * one a single run gives, bit for bit. */
int peec_gb300_transient_lightning_batch(void *system, int nrun, const double *K,
                                         const double *alpha, const double *beta,
                                         const double *delay, const size_t *strike_node,
                                         const size_t *return_node, size_t step0, size_t n_steps,
                                         double *d_X, const int *d_probe_nodes,
                                         size_t n_probe_nodes, const int *d_probe_edges,
                                         size_t n_probe_edges, double *d_probes);
void peec_gb300_transient_destroy(void *system);

/* ---- serving loop ----
 * A server admits harmonic solve requests from a FIFO onto worker threads,
 * each with its own CUDA stream, as soon as a worker is free and the
 * request's device-memory estimate fits the HBM budget.  Lp and P assembled
 * for one mesh_key stay in device memory and serve every later request with
 * that key (any frequency) until evicted, least recently used first, to make
 * room.  Each request builds Z = harmonic_build_system(frequency), nrhs
 * plane-wave right-hand sides, and solves by the plain FP64 complex LU
 * (mixed = 0) or the mixed-precision solve (mixed = 1, tolerance 0 means
 * 1e-10), then copies X to the caller's host array. */
typedef struct
{
    const Mesh *mesh;            /* read when the key is first assembled: keep valid until done */
    const DualMesh *dual;
    unsigned long long mesh_key; /* same key = same mesh (the caller's promise) */
    double frequency;            /* Hz, > 0 */
    size_t nrhs;                 /* plane waves                               */
    const double *k_hat;         /* [3*nrhs] propagation directions (copied at submit) */
    const double *e_hat;         /* [3*nrhs] polarisations (copied at submit)  */
    int mixed;                   /* 0 plain FP64 LU, 1 mixed precision         */
    double tolerance;            /* mixed: backward-error target (0 = 1e-10)   */
    Complex *x;                  /* host output [nrhs][Ne+Nv]                  */
} PeecHarmonicRequest;

typedef struct
{
    int status;            /* 0 solved, 1 mixed refinement did not converge, -2 singular, -1 error */
    int iterations;        /* mixed refinement iterations (0 for plain)     */
    int fallback;          /* 1: the mixed solve did not reach the tolerance
                              (or met a singular FP32 pivot) and the request
                              was solved again by the plain FP64 LU          */
    double backward_error; /* componentwise, over all right-hand sides      */
    double t_submit, t_start, t_end; /* seconds on the server's clock       */
} PeecRequestResult;

/* A lightning run on a PEC mesh (R = 0): n_steps of the stage-1 transient
 * (scheme 1 backward Euler, 2 trapezoidal, step dt) from rest, under the
 * double-exponential current K (exp(-alpha tau) - exp(-beta tau)),
 * tau = t - delay, injected at strike_node and returned at return_node.
 * The factorised system of (mesh_key, scheme, dt) stays resident for later
 * runs.  Probe lists are copied at submit; probes (host [n_steps][n_probe_
 * nodes + n_probe_edges]), I (Ne) and V (Nv) receive the waveforms and the
 * final state when not NULL. */
typedef struct
{
    const Mesh *mesh;
    const DualMesh *dual;
    unsigned long long mesh_key;
    int scheme;
    double dt;
    size_t n_steps;
    double K, alpha, beta, delay;
    size_t strike_node, return_node;
    const int *probe_nodes;
    size_t n_probe_nodes;
    const int *probe_edges;
    size_t n_probe_edges;
    double *probes;
    double *I;
    double *V;
} PeecTransientRequest;

/* Returns NULL on failure.  workers >= 1 host threads (and streams). */
void *peec_gb300_server_create(size_t hbm_budget_bytes, int workers);
/* Ticket >= 0, or -1 for an invalid request or one that can never fit. */
long long peec_gb300_server_submit(void *server, const PeecHarmonicRequest *request);
long long peec_gb300_server_submit_transient(void *server, const PeecTransientRequest *request);
/* Blocks until the request is done; 0, or -1 for an unknown ticket.  For a
 * transient request iterations is the step count and backward_error 0. */
int peec_gb300_server_wait(void *server, long long ticket, PeecRequestResult *result);
/* Seconds since the server was created (the clock of the result times). */
double peec_gb300_server_clock(void *server);
/* Finishes every queued request, then stops the workers and frees the cache. */
void peec_gb300_server_destroy(void *server);

#ifdef __cplusplus
}
#endif

#endif
