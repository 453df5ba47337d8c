// Incidence matrix and its dense products with P (drop-in for the
// reference's include/incidence.h, plus device-resident forms).
//
// Reference (paths inside the reference project):
//   src/peec/incidence.c:34-115    incidence_build: A[e][a] = -1, A[e][b] = +1
//   src/peec/incidence.c:117-187   row-sum check, info
//   src/peec/incidence.c:242-415   K = A P A^T: K[e][f] = P[a][c] - P[a][d]
//                                  - P[b][c] + P[b][d], e <= f, mirrored
//   src/peec/incidence.c:417-591   P A^T: PAT[j][e] = P[j][b] - P[j][a]
//                                  (NaN for an edge out of range, then any
//                                  non-finite entry fails the call)
//   src/peec/incidence.c:593-741   A S: AS[e][a] = (P[n][a] - P[m][a]) / P[a][a]
//   src/math/matrix.c:63-129       matrix_alloc (free, then calloc) / matrix_free
//
// The products are gathers from P: HBM-bound, one thread per output entry,
// consecutive threads on consecutive output columns (coalesced stores; the
// P reads of a row are contiguous for PAT and AS, two rows for APAT).  Every
// entry is the reference's expression in the same order, so results are
// bit-identical.  incidence_build itself is O(Ne) writes into a calloc'ed
// host array and stays on the host.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>


#include "../../include/incidence.h"
#include "../../include/peec_gb300.h"
#include "common.cuh"

namespace peec {

// Output rows r = blockIdx.y (+ k gridDim.y), columns blockIdx.x * 256 +
// threadIdx.x: no 64-bit division per entry.
//
// PAT[j][e] = P[j][b] - P[j][a]; NaN for an edge with a node out of range.
// *bad = smallest linear index of a non-finite entry (row-major).
__global__ void k_pat(const double *P, const int *edges, int nv, int ne, double *out, unsigned long long *bad) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int a = edges[2 * e], b = edges[2 * e + 1];
    const bool in = a >= 0 && b >= 0 && a < nv && b < nv;
    for (int j = blockIdx.y; j < nv; j += gridDim.y) {
        const size_t t = (size_t)j * ne + e;
        const double *row = P + (size_t)j * nv;
        const double v = in ? row[b] - row[a] : NAN;
        out[t] = v;
        if (!isfinite(v)) atomicMin(bad, (unsigned long long)t);
    }
}

// K = A P A^T by 32 x 32 tiles of the upper triangle (tile column >= tile
// row): each entry e <= f is P[a][c] - P[a][d] - P[b][c] + P[b][d], written
// along the row (coalesced) and, through shared memory, to the mirrored tile
// along its rows; *err = 1 for a node index out of range (entry NaN).
__global__ void __launch_bounds__(256) k_apat_tiles(const double *P, const int *edges, int nv, int ne, double *K,
                                                    int *err) {
    __shared__ double t[32][33];
    const int te = blockIdx.y, tf = blockIdx.x;
    if (tf < te) return;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int f = tf * 32 + tx;
    const bool fok = f < ne;
    const int c = fok ? edges[2 * f] : 0, d = fok ? edges[2 * f + 1] : 0;
    for (int i = ty; i < 32; i += 8) {
        const int e = te * 32 + i;
        double v = 0.0;
        if (e < ne && fok) {
            const int a = edges[2 * e], b = edges[2 * e + 1];
            if (a >= 0 && b >= 0 && c >= 0 && d >= 0 && a < nv && b < nv && c < nv && d < nv) {
                const double *pa = P + (size_t)a * nv, *pb = P + (size_t)b * nv;
                v = pa[c] - pa[d] - pb[c] + pb[d];
            } else {
                v = NAN;
                atomicExch(err, 1);
            }
            if (e <= f) K[(size_t)e * ne + f] = v;
        }
        t[i][tx] = v;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        const int fr = tf * 32 + i, ec = te * 32 + tx;  // K[f][e] = v(e, f), e < f
        if (fr < ne && ec < fr) K[(size_t)fr * ne + ec] = t[tx][i];
    }
}

// minus[e] / plus[e]: the last column of row e of A holding -1 / +1 (-1 if
// none); *err = 1 for any other non-zero value.  One warp per row.
__global__ void k_as_nodes(const double *A, long long ne, long long nv, long long *minus, long long *plus, int *err) {
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= ne) return;
    const double *row = A + warp * nv;
    long long m = -1, p = -1;
    bool other = false;
    for (long long j = lane; j < nv; j += 32) {
        const double v = row[j];
        if (v == -1.0)
            m = j;
        else if (v == 1.0)
            p = j;
        else if (v != 0.0)
            other = true;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        m = max(m, __shfl_xor_sync(0xffffffffu, m, s));
        p = max(p, __shfl_xor_sync(0xffffffffu, p, s));
    }
    other = __any_sync(0xffffffffu, other);
    if (lane == 0) {
        minus[warp] = m;
        plus[warp] = p;
        if (other || m < 0 || p < 0) atomicExch(err, 1);
    }
}

// AS[e][a] = (P[n][a] - P[m][a]) / P[a][a]; NaN and *err = 1 where P[a][a] is
// not finite or <= 0.  Rows without both nodes are left as written (the call
// fails for them).
__global__ void k_as(const double *P, const long long *minus, const long long *plus, int ne, int nv, double *AS,
                     int *err) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nv) return;
    const double paa = P[(size_t)a * nv + a];
    const bool good = isfinite(paa) && paa > 0.0;
    for (int e = blockIdx.y; e < ne; e += gridDim.y) {
        const long long m = minus[e], n = plus[e];
        if (m < 0 || n < 0) continue;
        const size_t t = (size_t)e * nv + a;
        if (!good) {
            AS[t] = NAN;
            atomicExch(err, 1);
            continue;
        }
        AS[t] = (P[(size_t)n * nv + a] - P[(size_t)m * nv + a]) / paa;
    }
}

// A S straight from the edge list: AS[e][k] = (P[b][k] - P[a][k]) / P[k][k]
// for e = a -> b; *err |= 1 for a bad P[k][k] (entry NaN), |= 2 for an edge
// with a node out of range or a == b (row left as written).
__global__ void k_as_edges(const double *P, const int *edges, int ne, int nv, double *AS, int *err) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nv) return;
    const double pkk = P[(size_t)k * nv + k];
    const bool good = isfinite(pkk) && pkk > 0.0;
    for (int e = blockIdx.y; e < ne; e += gridDim.y) {
        const int m = edges[2 * e], n = edges[2 * e + 1];
        if (m < 0 || n < 0 || m >= nv || n >= nv || m == n) {
            atomicOr(err, 2);
            continue;
        }
        const size_t t = (size_t)e * nv + k;
        if (!good) {
            AS[t] = NAN;
            atomicOr(err, 1);
            continue;
        }
        AS[t] = (P[(size_t)n * nv + k] - P[(size_t)m * nv + k]) / pkk;
    }
}

// grid of one output: 256 columns per CTA, rows over gridDim.y
static dim3 grid2(long long cols, long long rows) {
    const long long gx = (cols + 255) / 256;
    long long gy = rows < 65535 ? rows : 65535;
    while (gx * gy > 152 * 64 && gy > 1) gy = (gy + 1) / 2;
    return dim3((unsigned)gx, (unsigned)(gy < 1 ? 1 : gy));
}

// matrix.c:63-110: free what M holds, then rows x cols zeros (calloc)
static bool matrix_alloc_host(Matrix *M, size_t rows, size_t cols) {
    if (rows == 0 || cols == 0 || rows > (size_t)-1 / cols / sizeof(double)) {
        fprintf(stderr, "ERROR: invalid matrix allocation size %zu x %zu.\n", rows, cols);
        return false;
    }
    free(M->data);
    memset(M, 0, sizeof(*M));
    M->data = static_cast<double *>(calloc(rows * cols, sizeof(double)));
    if (!M->data) {
        fprintf(stderr, "ERROR: cannot allocate matrix %zu x %zu.\n", rows, cols);
        return false;
    }
    M->rows = rows;
    M->cols = cols;
    return true;
}

static void matrix_release(Matrix *M) {
    free(M->data);
    memset(M, 0, sizeof(*M));
}

}  // namespace peec

using namespace peec;

// ---------------------------------------------------------------------
// device-resident forms (peec_gb300.h)
// ---------------------------------------------------------------------
extern "C" int peec_gb300_pat_device(const double *d_P, const int *d_edges, size_t nv, size_t ne, double *d_out,
                                     long long *first_bad) {
    if (!d_P || !d_edges || !d_out || nv == 0 || ne == 0) return -1;
    DBuf<unsigned long long> bad(1);
    if (!bad.p) return -1;
    cudaMemsetAsync(bad.p, 0xff, sizeof(unsigned long long), stream());
    if (nv > 0x7fffffff || ne > 0x7fffffff) return -1;
    PEEC_LAUNCH(k_pat, grid2(ne, nv), 256, 0, d_P, d_edges, (int)nv, (int)ne, d_out, bad.p);
    unsigned long long hb = 0;
    cudaMemcpyAsync(&hb, bad.p, sizeof(hb), cudaMemcpyDeviceToHost, stream());
    if (!launch_ok("P A^T") || !sync("P A^T")) return -1;
    if (first_bad) *first_bad = hb == ~0ull ? -1 : (long long)hb;
    return hb == ~0ull ? 0 : 1;
}

extern "C" int peec_gb300_apat_device(const double *d_P, const int *d_edges, size_t nv, size_t ne, double *d_K) {
    if (!d_P || !d_edges || !d_K || nv == 0 || ne == 0) return -1;
    if (nv > 0x7fffffff || ne > 0x7fffffff || (ne + 31) / 32 > 65535) return -1;
    DBuf<int> err(1);
    if (!err.p) return -1;
    cudaMemsetAsync(err.p, 0, sizeof(int), stream());
    const unsigned tiles = (unsigned)((ne + 31) / 32);
    PEEC_LAUNCH(k_apat_tiles, dim3(tiles, tiles), 256, 0, d_P, d_edges, (int)nv, (int)ne, d_K, err.p);
    int he = 0;
    cudaMemcpyAsync(&he, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!launch_ok("A P A^T") || !sync("A P A^T")) return -1;
    return he ? -1 : 0;
}

extern "C" int peec_gb300_as_device(const double *d_P, const int *d_edges, size_t nv, size_t ne, double *d_AS) {
    if (!d_P || !d_edges || !d_AS || nv == 0 || ne == 0) return -1;
    if (nv > 0x7fffffff || ne > 0x7fffffff) return -1;
    DBuf<int> err(1);
    if (!err.p) return -1;
    cudaMemsetAsync(err.p, 0, sizeof(int), stream());
    PEEC_LAUNCH(k_as_edges, grid2(nv, ne), 256, 0, d_P, d_edges, (int)ne, (int)nv, d_AS, err.p);
    int he = 0;
    cudaMemcpyAsync(&he, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!launch_ok("A S") || !sync("A S")) return -1;
    return (he & 2) ? -1 : (he & 1) ? 1 : 0;
}

// ---------------------------------------------------------------------
// drop-in (incidence.h)
// ---------------------------------------------------------------------
extern "C" {

void incidence_init(IncidenceMatrix *A) {
    if (A) memset(A, 0, sizeof(*A));
}

void incidence_free(IncidenceMatrix *A) {
    if (!A) return;
    free(A->data);
    incidence_init(A);
}

int incidence_build(const Mesh *mesh, IncidenceMatrix *A) {
    if (!mesh || !A) return -1;
    if (!mesh->edges || mesh->n_edges == 0 || mesh->n_nodes == 0) {
        fprintf(stderr, "ERROR: mesh topology is not available.\n");
        return -1;
    }
    incidence_init(A);
    A->rows = mesh->n_edges;
    A->cols = mesh->n_nodes;
    A->data = static_cast<double *>(calloc(A->rows * A->cols, sizeof(double)));
    if (!A->data) {
        fprintf(stderr, "ERROR: cannot allocate incidence matrix.\n");
        incidence_free(A);
        return -1;
    }
    for (size_t e = 0; e < mesh->n_edges; ++e) {
        const int a = mesh->edges[2 * e], b = mesh->edges[2 * e + 1];
        if (a < 0 || b < 0) {
            fprintf(stderr, "ERROR: negative node index in edge %zu.\n", e);
            incidence_free(A);
            return -1;
        }
        if ((size_t)a >= mesh->n_nodes || (size_t)b >= mesh->n_nodes) {
            fprintf(stderr, "ERROR: node index out of range in edge %zu.\n", e);
            incidence_free(A);
            return -1;
        }
        A->data[e * A->cols + (size_t)a] = -1.0;
        A->data[e * A->cols + (size_t)b] = +1.0;
    }
    return 0;
}

double incidence_check_row_sum(const IncidenceMatrix *A) {
    if (!A || !A->data) return -1.0;
    double worst = 0.0;
    for (size_t r = 0; r < A->rows; ++r) {
        double sum = 0.0;
        for (size_t c = 0; c < A->cols; ++c) sum += A->data[r * A->cols + c];
        if (fabs(sum) > worst) worst = fabs(sum);
    }
    return worst;
}

void incidence_print_info(const IncidenceMatrix *A) {
    if (!A) return;
    size_t nonzero = 0;
    if (A->data)
        for (size_t i = 0; i < A->rows * A->cols; ++i) nonzero += A->data[i] != 0.0;
    printf("\nincidence matrix A: Ne = %zu rows, Nv = %zu columns, %zu non-zeros (expected %zu)\n", A->rows, A->cols,
           nonzero, 2 * A->rows);
}

int incidence_build_APAT(const Mesh *mesh, const PotentialMatrix *P, Matrix *K, int parallel_threads) {
    if (!mesh || !P || !K || !P->data || parallel_threads < 1) return -1;
    if (P->n != mesh->n_nodes) {
        fprintf(stderr, "ERROR: incompatible P matrix size in incidence_build_APAT.\n");
        return -1;
    }
    const size_t ne = mesh->n_edges, nv = mesh->n_nodes;
    if (ne == 0 || nv == 0 || !mesh->edges) return -1;
    for (size_t e = 0; e < 2 * ne; ++e)
        if (mesh->edges[e] < 0 || (size_t)mesh->edges[e] >= nv) {
            fprintf(stderr, "ERROR: node index out of range in edge %zu.\n", e / 2);
            return -1;
        }
    if (!matrix_alloc_host(K, ne, ne)) return -1;
    DBuf<double> dP(nv * nv), dK(ne * ne);
    DBuf<int> dE(2 * ne);
    int s = -1;
    if (dP.p && dK.p && dE.p && dP.upload(P->data, nv * nv) && dE.upload(mesh->edges, 2 * ne))
        s = peec_gb300_apat_device(dP.p, dE.p, nv, ne, dK.p);
    if (s == 0 && !(dK.download(K->data, ne * ne) && sync("A P A^T download"))) s = -1;
    if (s != 0) {
        matrix_release(K);
        return -1;
    }
    return 0;
}

int incidence_build_PAT(const Mesh *mesh, const PotentialMatrix *P, Matrix *PAT, int parallel_threads) {
    if (!mesh || !P || !PAT || parallel_threads < 1) return -1;
    if (!mesh->edges || !P->data) {
        fprintf(stderr, "ERROR: invalid input in incidence_build_PAT().\n");
        return -1;
    }
    if (P->n != mesh->n_nodes) {
        fprintf(stderr, "ERROR: P size does not match mesh nodes in incidence_build_PAT().\n");
        return -1;
    }
    const size_t nv = mesh->n_nodes, ne = mesh->n_edges;
    if (!matrix_alloc_host(PAT, nv, ne)) {
        fprintf(stderr, "ERROR: cannot allocate P A^T matrix.\n");
        return -1;
    }
    DBuf<double> dP(nv * nv), dO(nv * ne);
    DBuf<int> dE(2 * ne);
    long long bad = -1;
    int s = -1;
    if (dP.p && dO.p && dE.p && dP.upload(P->data, nv * nv) && dE.upload(mesh->edges, 2 * ne))
        s = peec_gb300_pat_device(dP.p, dE.p, nv, ne, dO.p, &bad);
    if (s == 1) {
        fprintf(stderr, "ERROR: invalid value in P A^T at [%zu,%zu].\n", (size_t)bad / ne, (size_t)bad % ne);
        matrix_release(PAT);
        return -1;
    }
    if (s == 0 && !(dO.download(PAT->data, nv * ne) && sync("P A^T download"))) s = -1;
    if (s != 0) {
        matrix_release(PAT);
        return -1;
    }
    return 0;
}

int incidence_build_AS(const IncidenceMatrix *A, const PotentialMatrix *P, Matrix *AS, int parallel_threads) {
    if (!A || !P || !AS || !A->data || !P->data || parallel_threads < 1) return -1;
    if (A->cols != P->n || A->rows == 0 || A->cols == 0) {
        fprintf(stderr, "ERROR: incompatible dimensions in incidence_build_AS().\n");
        return -1;
    }
    const size_t ne = A->rows, nv = A->cols;
    if (ne > 0x7fffffff || nv > 0x7fffffff) return -1;
    if (!matrix_alloc_host(AS, ne, nv)) {
        fprintf(stderr, "ERROR: cannot allocate A S matrix.\n");
        return -1;
    }
    DBuf<double> dA(ne * nv), dP(nv * nv), dO(ne * nv);
    DBuf<long long> minus(ne), plus(ne);
    DBuf<int> err(1);
    int herr = 0;
    bool ok = dA.p && dP.p && dO.p && minus.p && plus.p && err.p && dA.upload(A->data, ne * nv) &&
              dP.upload(P->data, nv * nv) &&
              cuda_ok(cudaMemsetAsync(dO.p, 0, ne * nv * sizeof(double), stream()), "A S clear") &&
              cuda_ok(cudaMemsetAsync(err.p, 0, sizeof(int), stream()), "A S flag");
    if (ok) {
        PEEC_LAUNCH(k_as_nodes, (unsigned)(((long long)ne * 32 + 255) / 256), 256, 0, dA.p, (long long)ne,
                    (long long)nv, minus.p, plus.p, err.p);
        PEEC_LAUNCH(k_as, grid2(nv, ne), 256, 0, dP.p, minus.p, plus.p, (int)ne, (int)nv, dO.p, err.p);
        cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
        ok = launch_ok("A S") && sync("A S");
    }
    if (ok && herr) {
        fprintf(stderr, "ERROR: cannot build A S matrix.\n");
        ok = false;
    }
    if (ok) ok = dO.download(AS->data, ne * nv) && sync("A S download");
    if (!ok) {
        matrix_release(AS);
        return -1;
    }
    return 0;
}

}  // extern "C"
