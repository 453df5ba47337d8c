// Stage-1 transient stepping on the device: the reference's
// transient_system_create_stage1 + transient_factorize (transient.c:385-480,
// 1020-1110, 2014-2066) and, per step, lightning_build_node_current
// (lightning.c:184-373), transient_build_rhs_stage1 (transient.c:1421-1660)
// and transient_solve_step (transient.c:2068-2097).
//
// The system matrix M = [L/dt + theta R, theta AS; -theta A^T, F/dt] is
// filled and LU-factorised once on the device (the reference's pivoting),
// and its inverse is formed from the factor once (blocked substitution of
// the permuted identity, about 2 n^3 FP64 flops); the factor is then freed
// and the inverse stays resident.  Every step is HBM-bound matrix-vector
// work, all runs of a batch at once: the right-hand side (Lp and AS read
// once, the node rows gathered through a node -> edge adjacency instead of
// the dense incidence), x0 = M^-1 b, the residual r = b - M x0 (Lp and AS
// again) and x = x0 + M^-1 r -- one step of iterative refinement, which
// keeps the step backward stable like the reference's LU solve
// (transient_solve_step) while reading 2 (n^2 + Ne^2 + Ne Nv) doubles
// instead of walking a chain of dependent triangular blocks.  The state
// x = [I; V] never leaves HBM between steps.
#include <math.h>
#include <string.h>

#include <vector>

#include "../../include/peec_gb300.h"
#include "common.cuh"

namespace peec {

bool inverse_from_lu_real(const double *lu, const int *perm, int n, double *Minv);

struct TransientSystem {
    int ne = 0, nv = 0, nt = 0, scheme = 0;
    int ldm = 0;  // row stride of M^-1's copies: nt rounded up to 4 (16-byte aligned rows, zero padding)
    int lde = 0, ldn = 0;  // row strides of Lf and ASf: ne and nv rounded up to 2 (zero padding)
    double theta = 0.0, dt = 0.0;
    const double *L = nullptr;  // caller's Lp (kept by pointer)
    double *R = nullptr, *F = nullptr, *AS = nullptr, *lu = nullptr, *dinv = nullptr;
    float2 *minv = nullptr;  // M^-1 as float pairs (hi, lo), nt rows of ldm
    float *minv_hi = nullptr;  // their high parts alone, for the correction's FP32 apply
    float2 *Lf = nullptr, *ASf = nullptr;  // Lp (ne x ne) and A S (ne x nv) as float pairs
    long long *piv = nullptr;
    int *perm = nullptr, *edges = nullptr;
    int *adj_ptr = nullptr, *adj = nullptr;  // node j: edges +(e+1) entering (b = j), -(e+1) leaving (a = j)
    void release() {
        for (void *p : {(void *)R, (void *)F, (void *)AS, (void *)lu, (void *)dinv, (void *)minv, (void *)minv_hi,
                        (void *)Lf,
                        (void *)ASf, (void *)piv,
                        (void *)perm, (void *)edges, (void *)adj_ptr, (void *)adj})
            dfree(p);
        R = F = AS = lu = dinv = nullptr;
        minv = Lf = ASf = nullptr;
        minv_hi = nullptr;
        piv = nullptr;
        perm = edges = adj_ptr = adj = nullptr;
    }
};

// F_j = 1 / P_jj (potential.c:483-520); a non-finite or non-positive
// diagonal sets *bad
__global__ void k_self_capacitance(const double *P, int nv, double *F, int *bad) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nv) return;
    double d = P[(size_t)j * nv + j];
    if (!isfinite(d) || d <= 0.0) {
        atomicExch(bad, 1);
        F[j] = NAN;
        return;
    }
    F[j] = 1.0 / d;
}

// AS[e][k] = (P[b][k] - P[a][k]) / P[k][k] (incidence.c:593-741), k fastest
__global__ void k_as_build(const double *P, const int *edges, int ne, int nv, double *AS) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)ne * nv) return;
    int e = (int)(t / nv), k = (int)(t % nv);
    int a = edges[2 * e], b = edges[2 * e + 1];
    AS[t] = (P[(size_t)b * nv + k] - P[(size_t)a * nv + k]) / P[(size_t)k * nv + k];
}

// M, row-major nt x nt (transient.c:1020-1110, stage 1)
__global__ void k_transient_fill(const double *L, const double *R, const double *AS, const double *F, const int *edges,
                                 int ne, int nv, double theta, double dt, double *M) {
    const int nt = ne + nv;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)nt * nt;
         t += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(t / nt), j = (int)(t % nt);
        double v;
        if (i < ne && j < ne) {
            v = L[(size_t)i * ne + j] / dt;
            if (i == j) v += theta * R[i];
        } else if (i < ne) {
            v = theta * AS[(size_t)i * nv + (j - ne)];
        } else if (j < ne) {
            int node = i - ne;
            double a = edges[2 * j + 1] == node ? 1.0 : edges[2 * j] == node ? -1.0 : 0.0;
            v = -theta * a;
        } else {
            v = (i == j ? F[i - ne] : 0.0) / dt;
        }
        M[t] = v;
    }
}

struct LightningArgs {
    double K, alpha, beta, delay;
    int strike, ret;
    long long start;  // the global step at which this run's own step 0 falls
};

// lightning.c:184-212
__device__ __forceinline__ double lightning_current(const LightningArgs &s, double t) {
    if (t < s.delay) return 0.0;
    double tau = t - s.delay;
    return s.K * (exp(-s.alpha * tau) - exp(-s.beta * tau));
}

// Several lightning runs on one system are stepped together (up to kMaxRuns):
// every matrix of a step (Lp and A S in the right-hand side and the
// residual, M^-1 twice) is read once for all of them.  A run may join a
// batch mid-way: its source time counts from its own start step, and its
// state starts at rest.
static const int kMaxRuns = 8;

struct StepArgs {
    const double *R, *F;
    const float2 *Lf, *ASf;  // Lp and A S as float pairs
    const float2 *xI, *xV;   // the states' I and V parts as float pairs, [run][lde] / [run][ldn]
    int lde, ldn;
    const int *adj_ptr, *adj;
    int ne, nv, nrun;
    double theta, dt;
    const double *x;  // states [nrun][I; V] after the previous step
    double *rhs;      // [nrun][ne + nv]
    LightningArgs src[kMaxRuns];
    long long step;
    // probes of the previous step's state (record_row >= 0): [row][run][np]
    const int *probe_nodes, *probe_edges;
    int n_probe_nodes, n_probe_edges;
    double *probes;
    long long record_row;
};

__device__ __forceinline__ void record_probes(const StepArgs &A, long long row) {
    const int np = A.n_probe_nodes + A.n_probe_edges, nt = A.ne + A.nv;
    for (int t = threadIdx.x; t < np * A.nrun; t += blockDim.x) {
        const int r = t / np, k = t % np;
        const double *x = A.x + (size_t)r * nt;
        double v = NAN;  // an index outside the mesh records NaN
        if (k < A.n_probe_nodes) {
            int j = A.probe_nodes[k];
            if (j >= 0 && j < A.nv) v = x[A.ne + j];
        } else {
            int e = A.probe_edges[k - A.n_probe_nodes];
            if (e >= 0 && e < A.ne) v = x[e];
        }
        A.probes[(row * A.nrun + r) * np + k] = v;
    }
}

// The step's matrix-vector products (M^-1, Lp, A S against every run's
// vector) run in double-float arithmetic on the FP32 pipes, the matrices
// stored as float pairs (8 B an element, as FP64): one FP64 FMA per element
// and run would hold them to GB300's FP64 rate (two per clock per SM), so a
// batch of 8 runs would cost 8x one run; here a batch streams each matrix
// once at about the cost of one run.  Each sum is exact to ~2^-48 of
// sum |a||v|; the FP64 residual of the refinement step and the FP64
// diagonal and adjacency terms keep the step's result to ~1e-14 of the
// FP64 recursion (the waveforms stay within 1e-11 of the reference's).

__global__ void k_split_pairs(const double *v, size_t count, float2 *out) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const double x = v[t];
    const float h = (float)x;
    out[t] = make_float2(h, (float)(x - (double)h));
}

// rows x cols FP64 -> float pairs with row stride ld (ld >= cols, the pad
// columns zero); hi (optional): the high parts alone, same layout
__global__ void k_split_rows(const double *v, int rows, int cols, int ld, float2 *out, float *hi) {
    pdl_wait();
    pdl_trigger();
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)rows * ld) return;
    const int r = (int)(t / ld), c = (int)(t % ld);
    float2 p = make_float2(0.0f, 0.0f);
    if (c < cols) {
        const double x = v[(size_t)r * cols + c];
        const float h = (float)x;
        p = make_float2(h, (float)(x - (double)h));
    }
    out[t] = p;
    if (hi) hi[t] = p.x;
}

// the states x [run][nt] (FP64) as float pairs in two padded parts: the
// currents [run][lde] and the potentials [run][ldn] (pad entries zero), so
// that Lp and A S rows meet 16-byte aligned vectors
__global__ void k_split_state(const double *x, int runs, int ne, int nv, int lde, int ldn, float2 *xI, float2 *xV) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x, per = lde + ldn;
    if (t >= runs * per) return;
    const int r = t / per, c = t % per;
    const bool cur = c < lde;
    const int j = cur ? c : c - lde;
    float2 p = make_float2(0.0f, 0.0f);
    if (j < (cur ? ne : nv)) {
        const double v = x[(size_t)r * (ne + nv) + (cur ? j : ne + j)];
        const float h = (float)v;
        p = make_float2(h, (float)(v - (double)h));
    }
    if (cur)
        xI[(size_t)r * lde + j] = p;
    else
        xV[(size_t)r * ldn + j] = p;
}

// the high parts of float pairs
__global__ void k_pairs_hi(const float2 *in, size_t count, float *out) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) out[t] = in[t].x;
}

// s += (a.x + a.y)(b.x + b.y) with the high parts two-summed into s.x and
// every low-order term in s.y (a.y b.y dropped)
__device__ __forceinline__ void pair_mac(float2 &s, float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    const float t = s.x + p;
    const float bp = t - s.x;
    const float err = (s.x - (t - bp)) + (p - bp);
    s.x = t;
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    s.y += e + err;
}

// out[r] = sum_j row[j] v[r][j] (j < n) for every run r < R, by the whole
// warp (every lane returns the sums).  Each lane reads two elements at a
// time (16 B) and keeps up to 8 such loads in flight (4 KB per warp and
// iteration), so the memory system, not each warp's load-to-use latency,
// sets the pace.  v: run r's vector at v + r ldv (float pairs); ALIGNED:
// row and v + r ldv 16-byte aligned and n even (M^-1's padded layout), the
// vector then read two pairs at a time too.
template <int R, bool ALIGNED = false>
__device__ __forceinline__ void row_dot_df(const float2 *row, int n, const float2 *v, size_t ldv, int lane,
                                           double *out) {
    // loads in flight: fewer with more runs, whose products give each load
    // more work (and whose accumulators need the registers)
    constexpr int kDotDepth = R >= 8 ? 4 : 8;
    float2 acc[2][R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[0][r] = acc[1][r] = make_float2(0.0f, 0.0f);
    // 16-byte loads start at the first 16-byte aligned element of the row
    const int head = n > 0 && (reinterpret_cast<uintptr_t>(row) & 8) ? 1 : 0;
    if (head && lane == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) pair_mac(acc[0][r], row[0], v[(size_t)r * ldv]);
    }
    const int body = (n - head) / 2;  // float4 pairs of elements after the head
    const float4 *row4 = reinterpret_cast<const float4 *>(row + head);
    int t = lane;
    for (; t + 32 * (kDotDepth - 1) < body; t += 32 * kDotDepth) {
        float4 m[kDotDepth];
#pragma unroll
        for (int u = 0; u < kDotDepth; ++u) m[u] = __ldcs(row4 + t + 32 * u);
#pragma unroll
        for (int u = 0; u < kDotDepth; ++u) {
            const int j = head + 2 * (t + 32 * u);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float2 *vr = v + (size_t)r * ldv + j;
                if constexpr (ALIGNED) {  // both pairs in one 16-byte load
                    const float4 w = *reinterpret_cast<const float4 *>(vr);
                    pair_mac(acc[u & 1][r], make_float2(m[u].x, m[u].y), make_float2(w.x, w.y));
                    pair_mac(acc[u & 1][r], make_float2(m[u].z, m[u].w), make_float2(w.z, w.w));
                } else {
                    pair_mac(acc[u & 1][r], make_float2(m[u].x, m[u].y), vr[0]);
                    pair_mac(acc[u & 1][r], make_float2(m[u].z, m[u].w), vr[1]);
                }
            }
        }
    }
    for (; t < body; t += 32) {
        const float4 m = __ldcs(row4 + t);
        const int j = head + 2 * t;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float2 *vr = v + (size_t)r * ldv + j;
            pair_mac(acc[0][r], make_float2(m.x, m.y), vr[0]);
            pair_mac(acc[0][r], make_float2(m.z, m.w), vr[1]);
        }
    }
    const int tail = head + 2 * body;  // one element left when n - head is odd
    if (tail < n && lane == 1) {
#pragma unroll
        for (int r = 0; r < R; ++r) pair_mac(acc[1][r], row[tail], v[(size_t)r * ldv + tail]);
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
        out[r] = warp_sum(((double)acc[0][r].x + (double)acc[1][r].x) + ((double)acc[0][r].y + (double)acc[1][r].y));
}

// Right-hand side of one step for every run (transient.c:1421-1631, edge
// voltages absent): blocks [0, eb) take the edge rows, one warp per row and
// all runs; the rest the (node, run) pairs.
template <int R>
__global__ void __launch_bounds__(256) k_transient_rhs(StepArgs A, int eb) {
    pdl_wait();
    pdl_trigger();
    const double omt = 1.0 - A.theta;
    const int nt = A.ne + A.nv;
    if (blockIdx.x == 0 && A.probes && A.record_row >= 0) record_probes(A, A.record_row);
    if ((int)blockIdx.x < eb) {
        const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
        if (i >= A.ne) return;
        double s[R], sa[R];
        row_dot_df<R, true>(A.Lf + (size_t)i * A.lde, A.lde, A.xI, A.lde, lane, s);
        if (omt != 0.0)
            row_dot_df<R, true>(A.ASf + (size_t)i * A.ldn, A.ldn, A.xV, A.ldn, lane, sa);
        else
#pragma unroll
            for (int r = 0; r < R; ++r) sa[r] = 0.0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const double ls = s[r], as = sa[r];
            if (lane == 0 && r < A.nrun) {
                const double *I = A.x + (size_t)r * nt;
                A.rhs[(size_t)r * nt + i] = ls / A.dt - omt * A.R[i] * I[i] - omt * as;
            }
        }
        return;
    }
    const int t = (blockIdx.x - eb) * blockDim.x + threadIdx.x;
    if (t >= A.nv * A.nrun) return;
    const int r = t / A.nv, j = t % A.nv;
    const double *x = A.x + (size_t)r * nt;
    const LightningArgs &src = A.src[r];
    const long long own = A.step - src.start;  // the run's own step number
    const double tn = (double)own * A.dt, tnp1 = (double)(own + 1) * A.dt;
    double jn = 0.0, jnp1 = 0.0;
    if (j == src.strike || j == src.ret) {
        jn = lightning_current(src, tn);
        jnp1 = lightning_current(src, tnp1);
        if (j == src.ret) {
            jn = -jn;
            jnp1 = -jnp1;
        }
    }
    double v = A.F[j] * x[A.ne + j] / A.dt;
    double at = 0.0;  // (A^T I)_j
    for (int k = A.adj_ptr[j]; k < A.adj_ptr[j + 1]; ++k) {
        int e = A.adj[k];
        at += e > 0 ? x[e - 1] : -x[-e - 1];
    }
    v += omt * at;
    v += omt * jn;
    v += A.theta * jnp1;
    A.rhs[(size_t)r * nt + A.ne + j] = v;
}

// y[r][i] = y0[r][i] (when set) + sum_q Minv[i][q] v[r][q] for every run,
// one warp per row of M^-1 (streamed once for all runs); vs: v as float
// pairs (k_split_rows), [run][ldm] with zero padding.
template <int R>
__global__ void __launch_bounds__(256) k_minv_apply(const float2 *Minv, int nt, int ldm, const float2 *vs,
                                                    const double *y0, double *y, int nrun) {
    pdl_wait();
    pdl_trigger();
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= nt) return;
    double s[R];
    row_dot_df<R, true>(Minv + (size_t)i * ldm, ldm, vs, ldm, lane, s);
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (lane == 0 && r < nrun) y[(size_t)r * nt + i] = (y0 ? y0[(size_t)r * nt + i] : 0.0) + s[r];
}

// out[r] = sum_j row[j] v[r][j] (j < n) in FP32 (FP64 across the warp),
// for the correction x = x0 + M^-1 r of the refinement step: r is ~2^-48
// of b, so the correction needs only a few correct digits, and its FP32
// apply streams half the bytes (the high parts alone).  row and v + r ldv
// 16-byte aligned, n a multiple of 4 (M^-1's padded layout): matrix and
// vector are read four elements at a time.
template <int R>
__device__ __forceinline__ void row_dot_f32(const float *row, int n, const float *v, size_t ldv, int lane,
                                            double *out) {
    float acc[2][R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[0][r] = acc[1][r] = 0.0f;
    const int body = n / 4;
    const float4 *row4 = reinterpret_cast<const float4 *>(row);
    constexpr int kDepth = 4;
    int t = lane;
    for (; t + 32 * (kDepth - 1) < body; t += 32 * kDepth) {
        float4 m[kDepth];
#pragma unroll
        for (int u = 0; u < kDepth; ++u) m[u] = __ldcs(row4 + t + 32 * u);
#pragma unroll
        for (int u = 0; u < kDepth; ++u) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float4 w = reinterpret_cast<const float4 *>(v + (size_t)r * ldv)[t + 32 * u];
                float a = acc[u & 1][r];
                a = fmaf(m[u].x, w.x, a);
                a = fmaf(m[u].y, w.y, a);
                a = fmaf(m[u].z, w.z, a);
                a = fmaf(m[u].w, w.w, a);
                acc[u & 1][r] = a;
            }
        }
    }
    for (; t < body; t += 32) {
        const float4 m = __ldcs(row4 + t);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float4 w = reinterpret_cast<const float4 *>(v + (size_t)r * ldv)[t];
            float a = acc[0][r];
            a = fmaf(m.x, w.x, a);
            a = fmaf(m.y, w.y, a);
            a = fmaf(m.z, w.z, a);
            a = fmaf(m.w, w.w, a);
            acc[0][r] = a;
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) out[r] = warp_sum((double)acc[0][r] + (double)acc[1][r]);
}

// y[r][i] = y0[r][i] + sum_q Minv_hi[i][q] v[r][q] for every run (the
// refinement step's correction), one warp per row; vh: the high parts of
// the vector, [run][ldm] with zero padding.
template <int R>
__global__ void __launch_bounds__(256) k_minv_apply_hi(const float *Mh, int nt, int ldm, const float *vh,
                                                       const double *y0, double *y, int nrun) {
    pdl_wait();
    pdl_trigger();
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= nt) return;
    double s[R];
    row_dot_f32<R>(Mh + (size_t)i * ldm, ldm, vh, ldm, lane, s);
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (lane == 0 && r < nrun) y[(size_t)r * nt + i] = y0[(size_t)r * nt + i] + s[r];
}

// res = b - M x for every run (M of k_transient_fill applied from its
// blocks: Lp / dt, theta R, theta AS, -theta A^T through the adjacency,
// F / dt), rows split as in k_transient_rhs.
template <int R>
__global__ void __launch_bounds__(256) k_transient_resid(StepArgs A, const double *b, double *res, int eb) {
    pdl_wait();
    pdl_trigger();
    const int nt = A.ne + A.nv;
    if ((int)blockIdx.x < eb) {
        const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
        if (i >= A.ne) return;
        double s[R], sa[R];
        row_dot_df<R, true>(A.Lf + (size_t)i * A.lde, A.lde, A.xI, A.lde, lane, s);
        row_dot_df<R, true>(A.ASf + (size_t)i * A.ldn, A.ldn, A.xV, A.ldn, lane, sa);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const double ls = s[r], as = sa[r];
            if (lane == 0 && r < A.nrun) {
                const double *x = A.x + (size_t)r * nt;
                const double mx = ls / A.dt + A.theta * A.R[i] * x[i] + A.theta * as;
                res[(size_t)r * nt + i] = b[(size_t)r * nt + i] - mx;
            }
        }
        return;
    }
    const int t = (blockIdx.x - eb) * blockDim.x + threadIdx.x;
    if (t >= A.nv * A.nrun) return;
    const int r = t / A.nv, j = t % A.nv;
    const double *x = A.x + (size_t)r * nt;
    double at = 0.0;  // (A^T I)_j
    for (int k = A.adj_ptr[j]; k < A.adj_ptr[j + 1]; ++k) {
        int e = A.adj[k];
        at += e > 0 ? x[e - 1] : -x[-e - 1];
    }
    const double mx = -A.theta * at + A.F[j] * x[A.ne + j] / A.dt;
    res[(size_t)r * nt + A.ne + j] = b[(size_t)r * nt + A.ne + j] - mx;
}

__global__ void k_transient_probe(StepArgs A) { record_probes(A, A.record_row); }

static int create(const double *d_L, const double *d_P, const int *d_edges, const double *d_R, size_t ne_, size_t nv_,
                  int scheme, double dt, TransientSystem &S) {
    if (!d_L || !d_P || !d_edges || ne_ == 0 || nv_ == 0 || ne_ + nv_ > 200000 || (scheme != 1 && scheme != 2) ||
        !isfinite(dt) || dt <= 0.0) {
        set_error("transient: invalid arguments (scheme 1 or 2, dt > 0, non-empty mesh)");
        return -1;
    }
    const int ne = (int)ne_, nv = (int)nv_, nt = ne + nv;
    S.ne = ne;
    S.nv = nv;
    S.nt = nt;
    S.scheme = scheme;
    S.theta = scheme == 1 ? 1.0 : 0.5;
    S.dt = dt;
    S.L = d_L;
    // edge list on the host for the node -> edge adjacency (A^T)
    std::vector<int> edges(2 * (size_t)ne);
    if (!cuda_ok(cudaMemcpyAsync(edges.data(), d_edges, edges.size() * sizeof(int), cudaMemcpyDeviceToHost, stream()),
                 "transient edges") ||
        !sync("transient edges"))
        return -1;
    std::vector<int> ptr(nv + 1, 0), adj(2 * (size_t)ne);
    for (int e = 0; e < ne; ++e) {
        int a = edges[2 * e], b = edges[2 * e + 1];
        if (a < 0 || b < 0 || a >= nv || b >= nv || a == b) {
            set_error("transient: edge with an invalid node pair");
            return -1;
        }
        ptr[a + 1]++;
        ptr[b + 1]++;
    }
    for (int j = 0; j < nv; ++j) ptr[j + 1] += ptr[j];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int e = 0; e < ne; ++e) {  // increasing edge order within each node
        adj[fill[edges[2 * e]]++] = -(e + 1);
        adj[fill[edges[2 * e + 1]]++] = e + 1;
    }
    S.R = static_cast<double *>(dalloc(sizeof(double) * ne));
    S.F = static_cast<double *>(dalloc(sizeof(double) * nv));
    S.AS = static_cast<double *>(dalloc(sizeof(double) * (size_t)ne * nv));
    S.lu = static_cast<double *>(dalloc(sizeof(double) * (size_t)nt * nt));
    S.piv = static_cast<long long *>(dalloc(sizeof(long long) * nt));
    S.perm = static_cast<int *>(dalloc(sizeof(int) * nt));
    S.edges = static_cast<int *>(dalloc(sizeof(int) * 2 * (size_t)ne));
    S.adj_ptr = static_cast<int *>(dalloc(sizeof(int) * (nv + 1)));
    S.adj = static_cast<int *>(dalloc(sizeof(int) * 2 * (size_t)ne));
    DBuf<int> bad(1);
    if (!S.R || !S.F || !S.AS || !S.lu || !S.piv || !S.perm || !S.edges || !S.adj_ptr || !S.adj || !bad.p) return -1;
    cudaStream_t st = stream();
    if (d_R)
        cudaMemcpyAsync(S.R, d_R, sizeof(double) * ne, cudaMemcpyDeviceToDevice, st);
    else
        cudaMemsetAsync(S.R, 0, sizeof(double) * ne, st);
    cudaMemcpyAsync(S.edges, edges.data(), edges.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(S.adj_ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(S.adj, adj.data(), adj.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(bad.p, 0, sizeof(int), st);
    PEEC_LAUNCH(k_self_capacitance, (nv + 255) / 256, 256, 0, d_P, nv, S.F, bad.p);
    size_t nas = (size_t)ne * nv;
    PEEC_LAUNCH(k_as_build, (unsigned)((nas + 255) / 256), 256, 0, d_P, S.edges, ne, nv, S.AS);
    PEEC_LAUNCH(k_transient_fill, 152 * 16, 256, 0, d_L, S.R, S.AS, S.F, S.edges, ne, nv, S.theta, dt, S.lu);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!launch_ok("transient system") || !sync("transient system")) return -1;
    if (hbad) {
        set_error("transient: invalid diagonal of P (non-finite or not positive)");
        return -1;
    }
    // Lp and A S as float pairs for the steps' double-float products; the
    // FP64 A S served the fill only
    S.lde = (ne + 1) & ~1;
    S.ldn = (nv + 1) & ~1;
    S.Lf = static_cast<float2 *>(dalloc(sizeof(float2) * (size_t)ne * S.lde));
    S.ASf = static_cast<float2 *>(dalloc(sizeof(float2) * (size_t)ne * S.ldn));
    if (!S.Lf || !S.ASf) return -1;
    PEEC_LAUNCH(k_split_rows, (unsigned)(((size_t)ne * S.lde + 255) / 256), 256, 0, d_L, ne, ne, S.lde, S.Lf,
                (float *)nullptr);
    PEEC_LAUNCH(k_split_rows, (unsigned)(((size_t)ne * S.ldn + 255) / 256), 256, 0, S.AS, ne, nv, S.ldn, S.ASf,
                (float *)nullptr);
    if (!launch_ok("transient split") || !sync("transient split")) return -1;
    dfree(S.AS);
    S.AS = nullptr;
    double scale;
    int col;
    int s = peec_gb300_lu_factor_device(S.lu, nt, 1.0e-14, S.piv, S.perm, &scale, &col);
    if (s != 0) return s == -2 ? -2 : -1;
    // M^-1 from the factor, once (the factor is not needed afterwards), kept
    // as float pairs for the double-float applies
    const size_t nn = (size_t)nt * nt;
    double *inv = static_cast<double *>(dalloc(sizeof(double) * nn));
    if (!inv || !inverse_from_lu_real(S.lu, S.perm, nt, inv) || !sync("transient inverse")) {
        dfree(inv);
        return -1;
    }
    dfree(S.lu);
    S.lu = nullptr;
    S.ldm = (nt + 3) & ~3;
    const size_t np_ = (size_t)nt * S.ldm;
    S.minv = static_cast<float2 *>(dalloc(sizeof(float2) * np_));
    if (!S.minv) {
        dfree(inv);
        return -1;
    }
    PEEC_LAUNCH(k_split_rows, (unsigned)((np_ + 255) / 256), 256, 0, inv, nt, nt, S.ldm, S.minv, (float *)nullptr);
    dfree(inv);  // before the high parts' copy: the peak stays at two FP64 matrices
    S.minv_hi = static_cast<float *>(dalloc(sizeof(float) * np_));
    if (!S.minv_hi) return -1;
    PEEC_LAUNCH(k_pairs_hi, (unsigned)((np_ + 255) / 256), 256, 0, S.minv, np_, S.minv_hi);
    return launch_ok("transient inverse") && sync("transient inverse") ? 0 : -1;
}

// One step for R run slots (the states padded with zero runs): split x,
// right-hand side, x0 = M^-1 b (double-float), split x0, r = b - M x0
// (double-float), x = x0 + M^-1 r (FP32: the correction is ~2^-48 of x).
struct StepBuffers {
    double *x, *rhs, *x0, *res;
    float2 *vs;             // [run][ldm]: the applies' vector
    float2 *xI, *xV, *x0I, *x0V;  // x's and x0's parts: [run][lde], [run][ldn]
    float *vh;              // the high parts of vs
};
template <int R>
static void launch_step(const TransientSystem &S, const StepArgs &A, const StepArgs &Ares, const StepBuffers &b,
                        int grid, int eb, int mgrid, int nrun) {
    const int nt = S.nt;
    const unsigned xgrid = (unsigned)(((size_t)R * (S.lde + S.ldn) + 255) / 256);
    // the step's chain as programmatic dependents: each kernel waits for the
    // one before it (pdl_wait) and lets the next be scheduled at once
    pdl_launch(k_split_state, dim3(xgrid), dim3(256), 0, (const double *)b.x, R, S.ne, S.nv, S.lde, S.ldn, b.xI,
               b.xV);
    pdl_launch(k_transient_rhs<R>, dim3(grid), dim3(256), 0, A, eb);
    const int ldm = S.ldm;
    const unsigned pgrid = (unsigned)(((size_t)R * ldm + 255) / 256);
    pdl_launch(k_split_rows, dim3(pgrid), dim3(256), 0, (const double *)b.rhs, R, nt, ldm, b.vs, (float *)nullptr);
    pdl_launch(k_minv_apply<R>, dim3(mgrid), dim3(256), 0, (const float2 *)S.minv, nt, ldm, (const float2 *)b.vs,
               (const double *)nullptr, b.x0, nrun);
    pdl_launch(k_split_state, dim3(xgrid), dim3(256), 0, (const double *)b.x0, R, S.ne, S.nv, S.lde, S.ldn, b.x0I,
               b.x0V);
    pdl_launch(k_transient_resid<R>, dim3(grid), dim3(256), 0, Ares, (const double *)b.rhs, b.res, eb);
    pdl_launch(k_split_rows, dim3(pgrid), dim3(256), 0, (const double *)b.res, R, nt, ldm, b.vs, b.vh);
    pdl_launch(k_minv_apply_hi<R>, dim3(mgrid), dim3(256), 0, (const float *)S.minv_hi, nt, ldm,
               (const float *)b.vh, (const double *)b.x0, b.x, nrun);
}

// nrun runs (states d_X[r] = [I; V], sources src[r]) stepped together
static int run_lightning(const TransientSystem &S, const LightningArgs *src, int nrun, long long step0,
                         long long n_steps, double *d_X, const int *probe_nodes, int n_probe_nodes,
                         const int *probe_edges, int n_probe_edges, double *probes) {
    const int ne = S.ne, nv = S.nv, nt = S.nt;
    // the step kernels are instantiated for 1, 2, 4 or 8 runs and read that
    // many states: pad with zero states (measured: a 16-run instantiation
    // stepped 16 runs slower than two batches of 8)
    const int cap = nrun <= 1 ? 1 : nrun <= 2 ? 2 : nrun <= 4 ? 4 : 8;
    DBuf<double> x((size_t)nt * cap), rhs((size_t)nt * cap), x0((size_t)nt * cap), res((size_t)nt * cap);
    // float pairs of the vectors: of an apply (vs), of the state x (xs) and of
    // x0 (x0s) for the right-hand side and the residual products
    DBuf<float2> vs((size_t)S.ldm * cap), xI((size_t)S.lde * cap), xV((size_t)S.ldn * cap),
        x0I((size_t)S.lde * cap), x0V((size_t)S.ldn * cap);
    DBuf<float> vh((size_t)S.ldm * cap);
    if (!x.p || !rhs.p || !x0.p || !res.p || !vs.p || !xI.p || !xV.p || !x0I.p || !x0V.p || !vh.p) return -1;
    cudaStream_t st = stream();
    if (cap > nrun) {
        for (double *p : {x.p, rhs.p, x0.p, res.p})
            cudaMemsetAsync(p + (size_t)nt * nrun, 0, sizeof(double) * nt * (cap - nrun), st);
    }
    cudaMemcpyAsync(x.p, d_X, sizeof(double) * nt * nrun, cudaMemcpyDeviceToDevice, st);
    StepArgs A{};
    A.R = S.R;
    A.F = S.F;
    A.Lf = S.Lf;
    A.ASf = S.ASf;
    A.xI = xI.p;
    A.xV = xV.p;
    A.lde = S.lde;
    A.ldn = S.ldn;
    A.adj_ptr = S.adj_ptr;
    A.adj = S.adj;
    A.ne = ne;
    A.nv = nv;
    A.nrun = nrun;
    A.theta = S.theta;
    A.dt = S.dt;
    A.x = x.p;
    A.rhs = rhs.p;
    for (int r = 0; r < nrun; ++r) A.src[r] = src[r];
    A.probe_nodes = probe_nodes;
    A.probe_edges = probe_edges;
    A.n_probe_nodes = n_probe_nodes;
    A.n_probe_edges = n_probe_edges;
    A.probes = (n_probe_nodes + n_probe_edges) > 0 ? probes : nullptr;
    const int eb = (ne + 7) / 8, grid = eb + (nv * nrun + 255) / 256;
    const int mgrid = (nt + 7) / 8;
    StepArgs Ares = A;  // the residual reads x0 as its state
    Ares.x = x0.p;
    Ares.xI = x0I.p;
    Ares.xV = x0V.p;
    const StepBuffers bufs{x.p, rhs.p, x0.p, res.p, vs.p, xI.p, xV.p, x0I.p, x0V.p, vh.p};
    for (long long k = 0; k < n_steps; ++k) {
        A.step = step0 + k;
        A.record_row = k - 1;
        switch (cap) {
            case 1: launch_step<1>(S, A, Ares, bufs, grid, eb, mgrid, nrun); break;
            case 2: launch_step<2>(S, A, Ares, bufs, grid, eb, mgrid, nrun); break;
            case 4: launch_step<4>(S, A, Ares, bufs, grid, eb, mgrid, nrun); break;
            default: launch_step<8>(S, A, Ares, bufs, grid, eb, mgrid, nrun); break;
        }
        if ((k & 255) == 255 && !launch_ok("transient step")) return -1;
    }
    if (A.probes && n_steps > 0) {
        A.record_row = n_steps - 1;
        PEEC_LAUNCH(k_transient_probe, 1, 256, 0, A);
    }
    cudaMemcpyAsync(d_X, x.p, sizeof(double) * nt * nrun, cudaMemcpyDeviceToDevice, st);
    if (!launch_ok("transient steps") || !sync("transient steps")) return -1;
    return 0;
}

// lightning.c:66-171
static bool source_ok(const TransientSystem &S, double K, double alpha, double beta, double delay, size_t strike,
                      size_t ret) {
    return isfinite(K) && K > 0.0 && isfinite(alpha) && isfinite(beta) && alpha > 0.0 && beta > 0.0 &&
           beta > alpha && isfinite(delay) && delay >= 0.0 && strike < (size_t)S.nv && ret < (size_t)S.nv &&
           strike != ret;
}

// The batch entry with each run's start step (null: all 0); the server's
// continuous batching admits runs into a stepping batch at chunk
// boundaries with start = the current global step.
int transient_lightning_runs(void *system, int nrun, const double *K, const double *alpha, const double *beta,
                             const double *delay, const size_t *strike_node, const size_t *return_node,
                             const long long *start, size_t step0, size_t n_steps, double *d_X,
                             const int *d_probe_nodes, size_t n_probe_nodes, const int *d_probe_edges,
                             size_t n_probe_edges, double *d_probes) {
    auto *S = static_cast<TransientSystem *>(system);
    if (!S || !d_X || nrun < 1 || nrun > kMaxRuns || !K || !alpha || !beta || !delay || !strike_node ||
        !return_node) {
        set_error("transient: missing system, state or sources (1 to 8 runs)");
        return -1;
    }
    LightningArgs src[kMaxRuns];
    for (int r = 0; r < nrun; ++r) {
        if (!source_ok(*S, K[r], alpha[r], beta[r], delay[r], strike_node[r], return_node[r])) {
            set_error("transient: invalid lightning source (K > 0, 0 < alpha < beta, delay >= 0, two distinct nodes)");
            return -1;
        }
        if (start && (start[r] < 0 || start[r] > (long long)step0)) {
            set_error("transient: a run's start step lies after the batch's first step");
            return -1;
        }
        src[r] = LightningArgs{K[r], alpha[r], beta[r], delay[r], (int)strike_node[r], (int)return_node[r],
                               start ? start[r] : 0};
    }
    if ((n_probe_nodes && !d_probe_nodes) || (n_probe_edges && !d_probe_edges) ||
        ((n_probe_nodes || n_probe_edges) && !d_probes) || n_probe_nodes + n_probe_edges > (1u << 20)) {
        set_error("transient: probe arrays missing");
        return -1;
    }
    return run_lightning(*S, src, nrun, (long long)step0, (long long)n_steps, d_X, d_probe_nodes, (int)n_probe_nodes,
                         d_probe_edges, (int)n_probe_edges, d_probes);
}

}  // namespace peec

using namespace peec;

extern "C" {

int peec_gb300_transient_create(const double *d_L, const double *d_P, const int *d_edges, const double *d_R,
                                size_t n_edges, size_t n_nodes, int scheme, double dt, void **system) {
    if (!system) return -1;
    *system = nullptr;
    auto *S = new TransientSystem();
    int s = create(d_L, d_P, d_edges, d_R, n_edges, n_nodes, scheme, dt, *S);
    if (s != 0) {
        S->release();
        sync("transient release");
        delete S;
        return s;
    }
    *system = S;
    return 0;
}

int peec_gb300_transient_lightning(void *system, double K, double alpha, double beta, double delay,
                                   size_t strike_node, size_t return_node, size_t step0, size_t n_steps, double *d_I,
                                   double *d_V, const int *d_probe_nodes, size_t n_probe_nodes,
                                   const int *d_probe_edges, size_t n_probe_edges, double *d_probes) {
    auto *S = static_cast<TransientSystem *>(system);
    if (!S || !d_I || !d_V) {
        set_error("transient: missing system or state");
        return -1;
    }
    DBuf<double> X((size_t)S->nt);
    if (!X.p) return -1;
    cudaMemcpyAsync(X.p, d_I, sizeof(double) * S->ne, cudaMemcpyDeviceToDevice, stream());
    cudaMemcpyAsync(X.p + S->ne, d_V, sizeof(double) * S->nv, cudaMemcpyDeviceToDevice, stream());
    size_t strike = strike_node, ret = return_node;
    int s = peec_gb300_transient_lightning_batch(system, 1, &K, &alpha, &beta, &delay, &strike, &ret, step0, n_steps,
                                                 X.p, d_probe_nodes, n_probe_nodes, d_probe_edges, n_probe_edges,
                                                 d_probes);
    if (s != 0) return s;
    cudaMemcpyAsync(d_I, X.p, sizeof(double) * S->ne, cudaMemcpyDeviceToDevice, stream());
    cudaMemcpyAsync(d_V, X.p + S->ne, sizeof(double) * S->nv, cudaMemcpyDeviceToDevice, stream());
    return sync("transient state") ? 0 : -1;
}

int peec_gb300_transient_lightning_batch(void *system, int nrun, const double *K, const double *alpha,
                                         const double *beta, const double *delay, const size_t *strike_node,
                                         const size_t *return_node, size_t step0, size_t n_steps, double *d_X,
                                         const int *d_probe_nodes, size_t n_probe_nodes, const int *d_probe_edges,
                                         size_t n_probe_edges, double *d_probes) {
    return peec::transient_lightning_runs(system, nrun, K, alpha, beta, delay, strike_node, return_node, nullptr,
                                          step0, n_steps, d_X, d_probe_nodes, n_probe_nodes, d_probe_edges,
                                          n_probe_edges, d_probes);
}

void peec_gb300_transient_destroy(void *system) {
    auto *S = static_cast<TransientSystem *>(system);
    if (!S) return;
    S->release();
    sync("transient release");
    delete S;
}

}  // extern "C"
