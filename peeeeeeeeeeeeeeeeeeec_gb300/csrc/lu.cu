// Dense real and complex LU with partial pivoting on sm_103a (FP64).
//
// Reference path (paths inside the reference project):
//   src/math/lu.c:194-479          real factorisation
//   src/math/lu.c:494-724          pivots, forward/backward substitution, solves
//   src/math/complex_lu.c:208-550  equilibration + complex factorisation
//   src/math/complex_lu.c:598-840  complex solves
//
// Layout: the device keeps the matrix row-major, exactly as the host ABI
// (data[i*n+j], complex interleaved {re, im}), so the packed L\U factor is
// downloaded without any transpose.  Blocked right-looking algorithm with
// panel width NB:
//   k_panel     one CTA factors rows k0..n-1 of columns k0..k0+NB-1 column by
//               column: argmax (first maximum wins, as the reference), row
//               swap inside the panel, multipliers, rank-1 update of the
//               remaining panel columns;
//   k_laswp     replays the panel's row swaps on the columns left and right
//               of the panel;
//   k_trsm      U12 = L11^-1 A12 (one thread per column, L11 in shared memory);
//   k_gemm_*    A22 -= L21 U12, register-tiled FP64 (complex: 4 real FMAs
//               per complex multiply-add).
// A device status word stops every later kernel after a singular pivot, so
// the host synchronises once per factorisation.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <complex>
#include <list>
#include <mutex>
#include <type_traits>
#include <vector>

#include "../../include/complex_lu.h"
#include "mixed_capture.cuh"
#include "../../include/lu.h"
#include "../../include/peec_gb300.h"
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace peec {

static const int NB = 32;  // panel width
static const int kPS = NB + 1;  // padded row stride of panel rows in shared memory

struct cplx {
    double re, im;
};

// ---- scalar traits --------------------------------------------------
__device__ __forceinline__ double mag(double v) { return fabs(v); }
__device__ __forceinline__ double mag(cplx v) { return hypot_cr(v.re, v.im); }
__device__ __forceinline__ double divide(double a, double b) { return a / b; }
// complex_lu.c:168-190: (a conj(b)) / |b|^2 without scaling
__device__ __forceinline__ cplx divide(cplx a, cplx b) {
    double den = b.re * b.re + b.im * b.im;
    cplx z;
    z.re = (a.re * b.re + a.im * b.im) / den;
    z.im = (a.im * b.re - a.re * b.im) / den;
    return z;
}
// c - m*u
__device__ __forceinline__ double msub(double c, double m, double u) { return fma(-m, u, c); }
__device__ __forceinline__ cplx msub(cplx c, cplx m, cplx u) {
    c.re = fma(-m.re, u.re, c.re);
    c.re = fma(m.im, u.im, c.re);
    c.im = fma(-m.re, u.im, c.im);
    c.im = fma(-m.im, u.re, c.im);
    return c;
}

// FP32 complex, for the mixed-precision factorisation
struct cplxf {
    float re, im;
};
__device__ __forceinline__ double mag(cplxf v) { return (double)hypotf(v.re, v.im); }
__device__ __forceinline__ cplxf divide(cplxf a, cplxf b) {
    float den = b.re * b.re + b.im * b.im;
    cplxf z;
    z.re = (a.re * b.re + a.im * b.im) / den;
    z.im = (a.im * b.re - a.re * b.im) / den;
    return z;
}
__device__ __forceinline__ cplxf msub(cplxf c, cplxf m, cplxf u) {
    c.re = fmaf(-m.re, u.re, c.re);
    c.re = fmaf(m.im, u.im, c.re);
    c.im = fmaf(-m.re, u.im, c.im);
    c.im = fmaf(-m.im, u.re, c.im);
    return c;
}
// component-wise warp sums and additions
__device__ __forceinline__ double warp_sum_t(double v) { return warp_sum(v); }
__device__ __forceinline__ cplx warp_sum_t(cplx v) {
    v.re = warp_sum(v.re);
    v.im = warp_sum(v.im);
    return v;
}
__device__ __forceinline__ cplxf warp_sum_t(cplxf v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        v.re += __shfl_xor_sync(0xffffffffu, v.re, m);
        v.im += __shfl_xor_sync(0xffffffffu, v.im, m);
    }
    return v;
}
__device__ __forceinline__ double addv(double a, double b) { return a + b; }
__device__ __forceinline__ cplx addv(cplx a, cplx b) { return cplx{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cplxf addv(cplxf a, cplxf b) { return cplxf{a.re + b.re, a.im + b.im}; }

struct Status {
    int code;    // 0 ok, 2 singular / invalid pivot
    int column;  // failing column
    double value;
};

// ---- scale ----------------------------------------------------------
// max over entries of |a| ignoring NaN (the reference's `if (v > max)` never
// takes a NaN), as IEEE bits: non-negative doubles order like integers.
template <class T>
__global__ void k_max_mag(const T *a, size_t count, unsigned long long *out) {
    double best = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x) {
        double m = mag(a[t]);
        if (m > best) best = m;
    }
    for (int s = 16; s > 0; s >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, s));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

// ---- panel ----------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(1024) k_panel(T *a, int n, int k0, int kb, double limit, long long *piv,
                                                Status *st) {
    __shared__ double s_val[32];
    __shared__ int s_idx[32];
    __shared__ int s_pivot;
    __shared__ int s_fail;
    __shared__ T s_row[NB];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nthr = blockDim.x;
    if (st->code != 0) return;
    for (int kk = 0; kk < kb; ++kk) {
        const int k = k0 + kk;
        // argmax |a[i][k]|, i >= k; ties -> lowest row; NaN below the diagonal
        // never wins, a NaN diagonal is kept (and rejected below)
        double best = -1.0;
        int bi = n;
        for (int i = k + tid; i < n; i += nthr) {
            double m = mag(a[(size_t)i * n + k]);
            if (i == k && isnan(m)) m = INFINITY;  // forces rejection
            if (isnan(m)) continue;
            if (m > best || (m == best && i < bi)) {
                best = m;
                bi = i;
            }
        }
        for (int s = 16; s > 0; s >>= 1) {
            double ov = __shfl_xor_sync(0xffffffffu, best, s);
            int oi = __shfl_xor_sync(0xffffffffu, bi, s);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_val[warp] = best;
            s_idx[warp] = bi;
        }
        __syncthreads();
        if (warp == 0) {
            int nw = nthr >> 5;
            best = lane < nw ? s_val[lane] : -1.0;
            bi = lane < nw ? s_idx[lane] : n;
            for (int s = 16; s > 0; s >>= 1) {
                double ov = __shfl_xor_sync(0xffffffffu, best, s);
                int oi = __shfl_xor_sync(0xffffffffu, bi, s);
                if (ov > best || (ov == best && oi < bi)) {
                    best = ov;
                    bi = oi;
                }
            }
            if (lane == 0) {
                double dm = mag(a[(size_t)k * n + k]);
                double pv = isnan(dm) ? dm : best;
                s_fail = 0;
                if (!isfinite(pv) || pv <= limit || bi >= n) {
                    s_fail = 1;
                    st->code = 2;
                    st->column = k;
                    st->value = pv;
                } else {
                    piv[k] = bi;
                }
                s_pivot = bi;
            }
        }
        __syncthreads();
        if (s_fail) return;
        const int p = s_pivot;
        if (p != k) {
            for (int j = k0 + tid; j < k0 + kb; j += nthr) {
                T t = a[(size_t)k * n + j];
                a[(size_t)k * n + j] = a[(size_t)p * n + j];
                a[(size_t)p * n + j] = t;
            }
        }
        __syncthreads();
        if (k + 1 >= n) break;
        for (int j = kk + tid; j < kb; j += nthr) s_row[j] = a[(size_t)k * n + k0 + j];
        __syncthreads();
        const T pivot = s_row[kk];
        for (int i = k + 1 + tid; i < n; i += nthr) {
            T *row = a + (size_t)i * n + k0;
            T m = divide(row[kk], pivot);
            row[kk] = m;
            for (int j = kk + 1; j < kb; ++j) row[j] = msub(row[j], m, s_row[j]);
        }
        __syncthreads();
    }
}

// ---- cooperative panel ------------------------------------------------
// The panel (rows k0..n-1, columns k0..k0+kb-1) spread over G co-resident
// CTAs, each holding a contiguous block of rows in shared memory, so the
// rank-1 panel updates use every SM's FP64 units.  One grid barrier per
// column: before it every CTA publishes its best candidate (value, row and
// the candidate row's panel segment) and the owner of row k publishes row k;
// after it every CTA picks the same pivot (first maximum wins), the two
// owners exchange rows k and p, and all update their rows.  Publication
// slots alternate by column parity so a CTA that runs ahead never
// overwrites slots still being read.  The barrier spin is bounded: on
// timeout the status word reports it and every CTA leaves.
// loads that bypass L1 (other SMs wrote the data this barrier epoch)
template <class T>
__device__ __forceinline__ T ld_volatile(const T *p) {
    if constexpr (sizeof(T) == 8) {
        long long v = __ldcg(reinterpret_cast<const long long *>(p));
        return *reinterpret_cast<T *>(&v);
    } else if constexpr (sizeof(T) == 16) {
        longlong2 v = __ldcg(reinterpret_cast<const longlong2 *>(p));
        return *reinterpret_cast<T *>(&v);
    } else {
        int v = __ldcg(reinterpret_cast<const int *>(p));
        return *reinterpret_cast<T *>(&v);
    }
}

// Pivot magnitudes: FP64 hypot for the FP64 factorisations (the reference's
// pivot choice), FP32 for the FP32 factorisation of the mixed path (no FP64
// instructions there: on GB300 one warp-wide FP64 compare costs 64 cycles).
template <class T>
struct MagType {
    using type = double;
};
template <>
struct MagType<cplxf> {
    using type = float;
};
__device__ __forceinline__ double mag_t(double v) { return fabs(v); }
__device__ __forceinline__ double mag_t(cplx v) { return hypot_cr(v.re, v.im); }
__device__ __forceinline__ float mag_t(cplxf v) { return hypotf(v.re, v.im); }

struct PanelSlots {
    unsigned int count;
    unsigned int gen;
    int timeout;
    int pad;
};

static const long long kSpinLimit = 1LL << 26;

__device__ __forceinline__ bool grid_barrier(PanelSlots *ps, unsigned int nblocks, unsigned int &gen) {
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = &ps->gen;
        __threadfence();
        unsigned int arrived = atomicAdd(&ps->count, 1u);
        int ok = 1;
        if (arrived == nblocks - 1) {
            ps->count = 0;
            __threadfence();
            atomicExch(&ps->gen, gen + 1);
        } else {
            long long spins = 0;
            while (*vgen == gen) {
                if (++spins > kSpinLimit || *(volatile int *)&ps->timeout) {
                    atomicExch(&ps->timeout, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    ++gen;
    return s_ok;
}

template <class T>
__global__ void __launch_bounds__(256) k_panel_coop(T *a, int n, int k0, int kb, int rows_per_cta, double limit,
                                                    long long *piv, Status *st, PanelSlots *ps, double *cand_val,
                                                    int *cand_idx, T *cand_row, T *krow) {
    extern __shared__ unsigned char smem_raw[];
    T *tile = reinterpret_cast<T *>(smem_raw);  // [rows_per_cta][kPS] (padded rows: no bank conflicts)
    using M = typename MagType<T>::type;  // FP32 magnitudes for the FP32 factorisation
    M *cval = reinterpret_cast<M *>(cand_val);
    __shared__ T s_prow[NB];
    __shared__ M s_val[8];
    __shared__ int s_idx[8];
    __shared__ int s_cta[8];
    __shared__ int s_p, s_fail, s_pc;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned int G = gridDim.x;
    const int c = blockIdx.x;
    const int r0 = k0 + c * rows_per_cta, r1 = min(n, r0 + rows_per_cta);
    const int nrows = r1 > r0 ? r1 - r0 : 0;
    if (st->code != 0) return;  // uniform across CTAs (set before launch)
    unsigned int gen = *(volatile unsigned int *)&ps->gen;  // stable between launches
    for (int t = tid; t < nrows * kb; t += blockDim.x) {
        int i = t / kb, j = t % kb;
        tile[i * kPS + j] = a[(size_t)(r0 + i) * n + k0 + j];
    }
    __syncthreads();
    for (int kk = 0; kk < kb; ++kk) {
        const int k = k0 + kk, par = kk & 1;
        // local argmax over this CTA's rows i >= k (NaN below the diagonal
        // never wins; a NaN diagonal becomes +inf and is rejected)
        M best = -1;
        int bi = n;
        for (int i = max(r0, k) + tid; i < r1; i += blockDim.x) {
            M m = mag_t(tile[(i - r0) * kPS + kk]);
            if (i == k && isnan(m)) m = INFINITY;
            if (isnan(m)) continue;
            if (m > best || (m == best && i < bi)) {
                best = m;
                bi = i;
            }
        }
        for (int s = 16; s > 0; s >>= 1) {
            M ov = __shfl_xor_sync(0xffffffffu, best, s);
            int oi = __shfl_xor_sync(0xffffffffu, bi, s);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_val[warp] = best;
            s_idx[warp] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
                if (s_val[w] > best || (s_val[w] == best && s_idx[w] < bi)) {
                    best = s_val[w];
                    bi = s_idx[w];
                }
            s_val[0] = best;
            s_idx[0] = bi;
            cval[par * G + c] = best;
            cand_idx[par * G + c] = bi;
        }
        __syncthreads();
        bi = s_idx[0];
        // publish the candidate row's segment and, if owned here, row k
        if (bi < n)
            for (int j = tid; j < kb; j += blockDim.x)
                cand_row[((size_t)par * G + c) * NB + j] = tile[(bi - r0) * kPS + j];
        if (k >= r0 && k < r1)
            for (int j = tid; j < kb; j += blockDim.x) krow[(size_t)par * NB + j] = tile[(k - r0) * kPS + j];
        if (!grid_barrier(ps, G, gen)) {
            if (c == 0 && tid == 0) atomicCAS(&st->code, 0, 6);
            return;
        }
        // global pivot, identical in every CTA: the G candidates are loaded
        // in parallel and reduced (largest value, then lowest row)
        {
            M gb = -1;
            int gi = n, gc = -1;
            for (unsigned int q = tid; q < G; q += blockDim.x) {
                M v = ld_volatile(cval + par * G + q);
                int ix = ld_volatile(cand_idx + par * G + q);
                if (ix >= n) continue;
                if (v > gb || (v == gb && ix < gi)) {
                    gb = v;
                    gi = ix;
                    gc = (int)q;
                }
            }
            for (int sh = 16; sh > 0; sh >>= 1) {
                M ov = __shfl_xor_sync(0xffffffffu, gb, sh);
                int oi = __shfl_xor_sync(0xffffffffu, gi, sh);
                int oc = __shfl_xor_sync(0xffffffffu, gc, sh);
                if (ov > gb || (ov == gb && oi < gi)) {
                    gb = ov;
                    gi = oi;
                    gc = oc;
                }
            }
            __syncthreads();  // s_val / s_idx of the local argmax are consumed
            if (lane == 0) {
                s_val[warp] = gb;
                s_idx[warp] = gi;
                s_cta[warp] = gc;
            }
            __syncthreads();
        }
        if (tid == 0) {
            M gb = s_val[0];
            int gi = s_idx[0], gc = s_cta[0];
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
                if (s_val[w] > gb || (s_val[w] == gb && s_idx[w] < gi)) {
                    gb = s_val[w];
                    gi = s_idx[w];
                    gc = s_cta[w];
                }
            s_fail = 0;
            if (gc < 0 || !isfinite(gb) || (double)gb <= limit) {
                s_fail = 1;
                if (c == 0) {
                    st->code = 2;
                    st->column = k;
                    st->value = (double)gb;
                }
            } else if (c == 0) {
                piv[k] = gi;
            }
            s_p = gi;
            s_pc = gc;
        }
        __syncthreads();
        if (s_fail) return;
        const int p = s_p, pc = s_pc;
        // the new row k is the published row p (full panel width: columns
        // < kk hold earlier multipliers and move with the row)
        const T *prow_g = cand_row + ((size_t)par * G + pc) * NB;
        for (int j = tid; j < kb; j += blockDim.x) s_prow[j] = ld_volatile(prow_g + j);
        __syncthreads();
        if (p != k) {
            if (k >= r0 && k < r1)
                for (int j = tid; j < kb; j += blockDim.x) tile[(k - r0) * kPS + j] = s_prow[j];
            if (p >= r0 && p < r1)
                for (int j = tid; j < kb; j += blockDim.x)
                    tile[(p - r0) * kPS + j] = ld_volatile(krow + (size_t)par * NB + j);
        }
        __syncthreads();
        if (k + 1 >= n) break;
        const T pivot = s_prow[kk];
        for (int i = max(r0, k + 1) + tid; i < r1; i += blockDim.x) {
            T *row = tile + (i - r0) * kPS;
            T m = divide(row[kk], pivot);
            row[kk] = m;
            for (int j = kk + 1; j < kb; ++j) row[j] = msub(row[j], m, s_prow[j]);
        }
        __syncthreads();
    }
    for (int t = tid; t < nrows * kb; t += blockDim.x) {
        int i = t / kb, j = t % kb;
        a[(size_t)(r0 + i) * n + k0 + j] = tile[i * kPS + j];
    }
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// ---- lean FP32 panel (the mixed path) ------------------------------
// The same partial pivoting (first maximum of |z| in FP32 wins) with the
// per-column critical path cut down, from measurements of the cooperative
// panel on GB300 (8402 rows, 152 CTAs, per column: local argmax + publish
// 0.94 us, grid barrier 2.3 us, candidate read + selection by 256 threads
// 1.4 us, pivot row 0.2 us, update 0.6 us):
//  * 64 threads per CTA, one row each: the argmax is a warp shuffle plus one
//    two-warp exchange, and the next column's magnitude comes out of the
//    update itself;
//  * no grid barrier: each CTA publishes its candidate (row segment, index)
//    and then one epoch-tagged flag word carrying the FP32 magnitude; one
//    warp polls the G flags (a flag per 128-byte line), which synchronises
//    and delivers the magnitudes in one step;
//  * multipliers by one complex reciprocal of the pivot instead of a
//    division per row.
// Epochs grow monotonically (base from the slots word, advanced by CTA 0 at
// the end), so flags of earlier columns or launches never match.  Every
// wait is bounded (status 6).
static const int kLeanThreads = 64;
static const int kLeanPoll = 8;  // flags per polling lane (two per 16-byte load): at most 256 CTAs

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acquire_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void ld_relaxed_v2u64(const unsigned long long *p, unsigned long long &a,
                                                 unsigned long long &b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}

// The largest FP32 value f with f <= x: for an FP32 g, g <= f exactly when
// (double)g <= x, so the per-column pivot test needs no FP64 instruction.
__device__ __forceinline__ float float_at_most(double x) {
    float f = (float)x;
    if ((double)f > x) f = nextafterf(f, -INFINITY);
    return f;
}

__device__ __forceinline__ float lean_mag(cplxf v, bool diag) {
    float m = hypotf(v.re, v.im);
    if (isnan(m)) m = diag ? INFINITY : -1.0f;  // NaN below the diagonal never wins; on it, +inf is rejected
    return m;
}

__global__ void __launch_bounds__(kLeanThreads) k_panel_lean(cplxf *a, int n, int k0, int kb, double limit,
                                                             long long *piv, Status *st, PanelSlots *ps,
                                                             unsigned long long *flag, int flag_stride,
                                                             int *cand_idx, cplxf *cand_row, cplxf *krow) {
    __shared__ cplxf tile[kLeanThreads][kPS];
    __shared__ cplxf s_prow[2][NB];  // pivot rows of the current and the previous column
    __shared__ float s_wv[2], s_fb;
    __shared__ int s_wi[2], s_gc, s_p, s_timeout;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned G = gridDim.x;
    const int c = blockIdx.x;
    const int r0 = k0 + c * kLeanThreads, r1 = min(n, r0 + kLeanThreads);
    const int nrows = r1 > r0 ? r1 - r0 : 0;
    if (st->code != 0) return;  // uniform across CTAs (set before launch)
    const float limf = float_at_most(limit);
    const unsigned gen0 = *(volatile unsigned *)&ps->gen;
    for (int t = tid; t < nrows * kb; t += kLeanThreads) {
        const int ii = t / kb, j = t % kb;
        tile[ii][j] = a[(size_t)(r0 + ii) * n + k0 + j];
    }
    if (tid == 0) s_timeout = 0;
    __syncthreads();
    const int i = r0 + tid;
    const bool mine = tid < nrows;
    cplxf *row = tile[tid];
    float mv = mine ? lean_mag(row[0], i == k0) : -1.0f;
    cplxf mreg = {0.0f, 0.0f};  // this row's multiplier of the previous column (its update is deferred)
    for (int kk = 0; kk < kb; ++kk) {
        const int k = k0 + kk, par = kk & 1;
        const unsigned epoch = gen0 + (unsigned)kk + 1u;
        const cplxf *pprev = s_prow[par ^ 1];  // pivot row of column kk - 1
        // this CTA's candidate (column kk is up to date): largest magnitude, lowest row
        float bv = (mine && i >= k) ? mv : -1.0f;
        int bi = bv >= 0.0f ? i : n;
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, sh);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, sh);
            if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_wv[warp] = bv;
            s_wi[warp] = bi;
        }
        __syncthreads();
        if (s_wv[1] > s_wv[0] || (s_wv[1] == s_wv[0] && s_wi[1] < s_wi[0])) {
            bv = s_wv[1];
            bi = s_wi[1];
        } else {
            bv = s_wv[0];
            bi = s_wi[0];
        }
        // publish the candidate row and, if owned here, row k as they are
        // (columns > kk still lack the previous column's update, which the
        // readers apply), then the flag with the magnitude
        if (warp == 0 && bi < n && lane < kb) cand_row[((size_t)par * G + c) * NB + lane] = tile[bi - r0][lane];
        if (warp == 1 && k >= r0 && k < r1 && lane < kb) krow[(size_t)par * NB + lane] = tile[k - r0][lane];
        if (tid == 0) cand_idx[par * G + c] = bi;
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            st_relaxed_u64(flag + (size_t)par * flag_stride + c,
                           ((unsigned long long)epoch << 32) | __float_as_uint(bi < n ? bv : -1.0f));
        }
        // the previous column's deferred update of this CTA's rows, while
        // the flags travel
        if (kk > 0 && mine && i >= k) {
#pragma unroll 4
            for (int j = kk + 1; j < kb; ++j) row[j] = msub(row[j], mreg, pprev[j]);
        }
        // warp 0 polls the G flags (dense: a sweep is a few coalesced 16-byte
        // loads per lane, flags q = 64 u + 2 lane + {0, 1}), then one acquire
        // fence: (largest magnitude, lowest CTA)
        if (warp == 0) {
            float fb = -2.0f;
            int fq = -1;
            unsigned long long v[kLeanPoll];
            unsigned pending = 0;
#pragma unroll
            for (int u = 0; u < kLeanPoll; ++u)
                if (64 * (u >> 1) + 2 * lane + (u & 1) < (int)G) pending |= 1u << u;
            for (long long spin = 0; pending && spin < kSpinLimit; ++spin) {
#pragma unroll
                for (int u = 0; u < kLeanPoll; u += 2)
                    if (pending & (3u << u))
                        ld_relaxed_v2u64(flag + (size_t)par * flag_stride + 64 * (u >> 1) + 2 * lane, v[u], v[u + 1]);
#pragma unroll
                for (int u = 0; u < kLeanPoll; ++u)
                    if ((pending & (1u << u)) && (unsigned)(v[u] >> 32) == epoch) pending &= ~(1u << u);
                if ((spin & 1023) == 1023 && *(volatile int *)&ps->timeout) break;
            }
            fence_acquire_gpu();
            const bool ok = pending == 0;
#pragma unroll
            for (int u = 0; u < kLeanPoll; ++u) {
                const int q = 64 * (u >> 1) + 2 * lane + (u & 1);
                if (q >= (int)G) continue;
                const float f = __uint_as_float((unsigned)v[u]);
                if (ok && f >= 0.0f && (f > fb || (f == fb && q < fq))) {
                    fb = f;
                    fq = q;
                }
            }
            if (!ok) atomicExch(&ps->timeout, 1);
            const bool any_fail = __any_sync(0xffffffffu, !ok);
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
                const float ov = __shfl_xor_sync(0xffffffffu, fb, sh);
                const int oq = __shfl_xor_sync(0xffffffffu, fq, sh);
                if (oq >= 0 && (fq < 0 || ov > fb || (ov == fb && oq < fq))) {
                    fb = ov;
                    fq = oq;
                }
            }
            if (lane == 0) {
                s_gc = fq;
                s_fb = fb;
                s_timeout = any_fail ? 1 : 0;
            }
        }
        __syncthreads();
        if (s_timeout) {
            if (tid == 0) atomicCAS(&st->code, 0, 6);
            return;
        }
        const int gc = s_gc;
        const float gb = s_fb;
        if (gc < 0 || !isfinite(gb) || gb <= limf) {
            if (c == 0 && tid == 0) {
                st->code = 2;
                st->column = k;
                st->value = gc < 0 ? -1.0 : (double)gb;
            }
            return;
        }
        // the winner's row (with the pending update applied, exactly as its
        // owner applied it) and index; the owner of p takes row k
        cplxf *pcur = s_prow[par];
        cplxf kval = {0.0f, 0.0f};
        if (gc == c) {
            if (warp == 0 && lane < kb) pcur[lane] = tile[bi - r0][lane];
            if (tid == 0) s_p = bi;
            if (warp == 1 && bi != k && lane < kb) {
                if (k >= r0 && k < r1) {
                    kval = tile[k - r0][lane];  // updated above by its own thread
                } else {
                    kval = ld_volatile(krow + (size_t)par * NB + lane);
                    if (kk > 0 && lane > kk) {
                        const cplxf km = ld_volatile(krow + (size_t)par * NB + kk - 1);
                        kval = msub(kval, km, pprev[lane]);
                    }
                }
            }
        } else {
            if (warp == 0 && lane < kb) {
                cplxf v = ld_volatile(cand_row + ((size_t)par * G + gc) * NB + lane);
                if (kk > 0 && lane > kk) {
                    const cplxf cm = ld_volatile(cand_row + ((size_t)par * G + gc) * NB + kk - 1);
                    v = msub(v, cm, pprev[lane]);
                }
                pcur[lane] = v;
            }
            if (warp == 1 && lane == 0) s_p = ld_volatile(cand_idx + par * G + gc);
        }
        __syncthreads();
        const int p = s_p;
        if (p != k) {
            if (warp == 0 && k >= r0 && k < r1 && lane < kb) tile[k - r0][lane] = pcur[lane];
            if (warp == 1 && gc == c && lane < kb) tile[p - r0][lane] = kval;
        }
        if (c == 0 && tid == 0) piv[k] = p;
        __syncthreads();
        if (k + 1 >= n) break;
        // this row's multiplier and its next column (the rest of the row is
        // updated in the next step, off the critical path)
        if (mine && i > k) {
            const cplxf pv = pcur[kk];
            const float den = pv.re * pv.re + pv.im * pv.im;
            const cplxf inv = {pv.re / den, -pv.im / den};
            const cplxf x = row[kk];
            mreg = cplxf{x.re * inv.re - x.im * inv.im, x.re * inv.im + x.im * inv.re};
            row[kk] = mreg;
            if (kk + 1 < kb) {
                row[kk + 1] = msub(row[kk + 1], mreg, pcur[kk + 1]);
                mv = lean_mag(row[kk + 1], i == k + 1);
            } else {
                mv = -1.0f;
            }
        } else {
            mv = -1.0f;
        }
    }
    __syncthreads();
    for (int t = tid; t < nrows * kb; t += kLeanThreads) {
        const int ii = t / kb, j = t % kb;
        a[(size_t)(r0 + ii) * n + k0 + j] = tile[ii][j];
    }
    // every CTA read the base epoch before publishing column 0, and CTA 0
    // gets here only after every CTA published the last column
    if (c == 0 && tid == 0) atomicExch(&ps->gen, gen0 + (unsigned)kb);
}

// ---- lean FP64 panel (the plain LU) --------------------------------
// The lean panel's structure for the FP64 factorisations, with the
// reference's arithmetic kept bit for bit (FP64 |z|, first maximum wins,
// NaN never wins, L = a / pivot by the same complex division, one msub per
// pivot and element in pivot order): 64 rows per CTA, one per thread;
// candidates published with an epoch-tagged flag carrying the magnitude
// rounded to FP32 (monotonic: the FP32 maximum identifies the winner unless
// several candidates share it, then their exact FP64 magnitudes decide);
// the previous column's row update deferred to run while the flags travel.
template <class T>
__device__ __forceinline__ double lean64_mag(T v, bool diag) {
    double m = mag_t(v);
    if (isnan(m)) m = diag ? INFINITY : -1.0;
    return m;
}

template <class T>
__global__ void __launch_bounds__(kLeanThreads) k_panel_lean64(T *a, int n, int k0, int kb, double limit,
                                                               long long *piv, Status *st, PanelSlots *ps,
                                                               unsigned long long *flag, int flag_stride,
                                                               int *cand_idx, double *cand_val, T *cand_row,
                                                               T *krow) {
    __shared__ T tile[kLeanThreads][kPS];
    __shared__ T s_prow[2][NB];
    __shared__ double s_wv[2], s_gb;
    __shared__ int s_wi[2], s_gc, s_p, s_timeout;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned G = gridDim.x;
    const int c = blockIdx.x;
    const int r0 = k0 + c * kLeanThreads, r1 = min(n, r0 + kLeanThreads);
    const int nrows = r1 > r0 ? r1 - r0 : 0;
    if (st->code != 0) return;  // uniform across CTAs (set before launch)
    const unsigned gen0 = *(volatile unsigned *)&ps->gen;
    for (int t = tid; t < nrows * kb; t += kLeanThreads) {
        const int ii = t / kb, j = t % kb;
        tile[ii][j] = a[(size_t)(r0 + ii) * n + k0 + j];
    }
    if (tid == 0) s_timeout = 0;
    __syncthreads();
    const int i = r0 + tid;
    const bool mine = tid < nrows;
    T *row = tile[tid];
    double mv = mine ? lean64_mag(row[0], i == k0) : -1.0;
    T mreg = T{};
    for (int kk = 0; kk < kb; ++kk) {
        const int k = k0 + kk, par = kk & 1;
        const unsigned epoch = gen0 + (unsigned)kk + 1u;
        const T *pprev = s_prow[par ^ 1];
        double bv = (mine && i >= k) ? mv : -1.0;
        int bi = bv >= 0.0 ? i : n;
        for (int sh = 16; sh > 0; sh >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, bv, sh);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, sh);
            if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_wv[warp] = bv;
            s_wi[warp] = bi;
        }
        __syncthreads();
        if (s_wv[1] > s_wv[0] || (s_wv[1] == s_wv[0] && s_wi[1] < s_wi[0])) {
            bv = s_wv[1];
            bi = s_wi[1];
        } else {
            bv = s_wv[0];
            bi = s_wi[0];
        }
        if (warp == 0 && bi < n && lane < kb) cand_row[((size_t)par * G + c) * NB + lane] = tile[bi - r0][lane];
        if (warp == 1 && k >= r0 && k < r1 && lane < kb) krow[(size_t)par * NB + lane] = tile[k - r0][lane];
        if (tid == 0) {
            cand_idx[par * G + c] = bi;
            cand_val[par * G + c] = bv;
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            st_relaxed_u64(flag + (size_t)par * flag_stride + c,
                           ((unsigned long long)epoch << 32) | __float_as_uint(bi < n ? (float)bv : -1.0f));
        }
        if (kk > 0 && mine && i >= k)
            for (int j = kk + 1; j < kb; ++j) row[j] = msub(row[j], mreg, pprev[j]);
        if (warp == 0) {
            unsigned long long v[kLeanPoll];
            unsigned pending = 0;
#pragma unroll
            for (int u = 0; u < kLeanPoll; ++u)
                if (64 * (u >> 1) + 2 * lane + (u & 1) < (int)G) pending |= 1u << u;
            for (long long spin = 0; pending && spin < kSpinLimit; ++spin) {
#pragma unroll
                for (int u = 0; u < kLeanPoll; u += 2)
                    if (pending & (3u << u))
                        ld_relaxed_v2u64(flag + (size_t)par * flag_stride + 64 * (u >> 1) + 2 * lane, v[u], v[u + 1]);
#pragma unroll
                for (int u = 0; u < kLeanPoll; ++u)
                    if ((pending & (1u << u)) && (unsigned)(v[u] >> 32) == epoch) pending &= ~(1u << u);
                if ((spin & 1023) == 1023 && *(volatile int *)&ps->timeout) break;
            }
            fence_acquire_gpu();
            const bool ok = pending == 0;
            // FP32 maximum, then the exact FP64 maximum among those sharing it
            float fb = -2.0f;
#pragma unroll
            for (int u = 0; u < kLeanPoll; ++u) {
                const int q = 64 * (u >> 1) + 2 * lane + (u & 1);
                const float f = __uint_as_float((unsigned)v[u]);
                if (ok && q < (int)G && f >= 0.0f && f > fb) fb = f;
            }
            for (int sh = 16; sh > 0; sh >>= 1) fb = fmaxf(fb, __shfl_xor_sync(0xffffffffu, fb, sh));
            double eb = -1.0;
            int eq = -1;
#pragma unroll
            for (int u = 0; u < kLeanPoll; ++u) {
                const int q = 64 * (u >> 1) + 2 * lane + (u & 1);
                if (!ok || q >= (int)G || fb < 0.0f || __uint_as_float((unsigned)v[u]) != fb) continue;
                const double ev = ld_volatile(cand_val + par * G + q);
                if (eq < 0 || ev > eb || (ev == eb && q < eq)) {
                    eb = ev;
                    eq = q;
                }
            }
            for (int sh = 16; sh > 0; sh >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, eb, sh);
                const int oq = __shfl_xor_sync(0xffffffffu, eq, sh);
                if (oq >= 0 && (eq < 0 || ov > eb || (ov == eb && oq < eq))) {
                    eb = ov;
                    eq = oq;
                }
            }
            if (!ok) atomicExch(&ps->timeout, 1);
            const bool any_fail = __any_sync(0xffffffffu, !ok);
            if (lane == 0) {
                s_gc = eq;
                s_gb = eb;
                s_timeout = any_fail ? 1 : 0;
            }
        }
        __syncthreads();
        if (s_timeout) {
            if (tid == 0) atomicCAS(&st->code, 0, 6);
            return;
        }
        const int gc = s_gc;
        const double gb = s_gb;
        if (gc < 0 || !isfinite(gb) || gb <= limit) {
            if (c == 0 && tid == 0) {
                st->code = 2;
                st->column = k;
                st->value = gc < 0 ? -1.0 : gb;
            }
            return;
        }
        T *pcur = s_prow[par];
        T kval = T{};
        if (gc == c) {
            if (warp == 0 && lane < kb) pcur[lane] = tile[bi - r0][lane];
            if (tid == 0) s_p = bi;
            if (warp == 1 && bi != k && lane < kb) {
                if (k >= r0 && k < r1) {
                    kval = tile[k - r0][lane];
                } else {
                    kval = ld_volatile(krow + (size_t)par * NB + lane);
                    if (kk > 0 && lane > kk) kval = msub(kval, ld_volatile(krow + (size_t)par * NB + kk - 1), pprev[lane]);
                }
            }
        } else {
            if (warp == 0 && lane < kb) {
                const T *cr = cand_row + ((size_t)par * G + gc) * NB;
                T vv = ld_volatile(cr + lane);
                if (kk > 0 && lane > kk) vv = msub(vv, ld_volatile(cr + kk - 1), pprev[lane]);
                pcur[lane] = vv;
            }
            if (warp == 1 && lane == 0) s_p = ld_volatile(cand_idx + par * G + gc);
        }
        __syncthreads();
        const int p = s_p;
        if (p != k) {
            if (warp == 0 && k >= r0 && k < r1 && lane < kb) tile[k - r0][lane] = pcur[lane];
            if (warp == 1 && gc == c && lane < kb) tile[p - r0][lane] = kval;
        }
        if (c == 0 && tid == 0) piv[k] = p;
        __syncthreads();
        if (k + 1 >= n) break;
        if (mine && i > k) {
            mreg = divide(row[kk], pcur[kk]);
            row[kk] = mreg;
            if (kk + 1 < kb) {
                row[kk + 1] = msub(row[kk + 1], mreg, pcur[kk + 1]);
                mv = lean64_mag(row[kk + 1], i == k + 1);
            } else {
                mv = -1.0;
            }
        } else {
            mv = -1.0;
        }
    }
    __syncthreads();
    for (int t = tid; t < nrows * kb; t += kLeanThreads) {
        const int ii = t / kb, j = t % kb;
        a[(size_t)(r0 + ii) * n + k0 + j] = tile[ii][j];
    }
    if (c == 0 && tid == 0) atomicExch(&ps->gen, gen0 + (unsigned)kb);
}

// ---- cluster FP32 panel (the mixed path) ---------------------------
// The lean panel's per-column exchange still crosses the GPU: measured on
// GB300, a release store takes ~2 us to reach pollers on other SMs, while a
// thread-block cluster barrier takes 0.2 us and a distributed-shared-memory
// load 0.1 us.  Here the whole panel lives in one cluster of C (1-16) CTAs,
// one row per thread (up to 640 rows per CTA), candidates in each CTA's
// shared memory: per column a CTA argmax, one split cluster barrier (the
// previous column's deferred update runs between arrive and wait), the
// winner read from its CTA's shared memory, the swap, and the multiplier
// plus next column of every row.  Published rows are copied before the
// deferred update; readers apply it (the row's multiplier in column kk-1
// times the previous pivot row), exactly as the owner does.  The pivot rule
// is the lean panel's (first maximum of |z| in FP32, lowest row on ties).
struct ClSlot {
    cplxf row[2][NB];   // candidate row, by column parity
    cplxf krow[2][NB];  // row k when owned here
    float val[2];
    int idx[2];
};

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

static const int kClMaxThreads = 640;  // rows per CTA at most (registers: 102 a thread)
static const int kClStride = NB + 2;   // tile row stride (complex): 16-byte aligned rows

__global__ void __launch_bounds__(kClMaxThreads) k_panel_cl(cplxf *a, int n, int k0, int kb, int rows_per_cta,
                                                            double limit, long long *piv, Status *st) {
    pdl_wait();
    pdl_trigger();
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char cl_smem[];
    cplxf(*tile)[kClStride] = reinterpret_cast<cplxf(*)[kClStride]>(cl_smem);  // [rows_per_cta][kClStride]
    __shared__ ClSlot slot;
    __shared__ __align__(16) cplxf s_prow[2][NB];
    __shared__ float s_wv[32], s_gb;
    __shared__ int s_wi[32], s_gc, s_p;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int C = (int)cluster.num_blocks(), c = (int)cluster.block_rank();
    const int r0 = k0 + c * rows_per_cta, r1 = min(n, r0 + rows_per_cta);
    const int nrows = r1 > r0 ? r1 - r0 : 0;
    if (st->code != 0) return;  // uniform over the cluster (set before launch)
    const float limf = float_at_most(limit);
    for (int t = tid; t < nrows * kb; t += blockDim.x) {
        const int ii = t / kb, j = t % kb;
        tile[ii][j] = a[(size_t)(r0 + ii) * n + k0 + j];
    }
    __syncthreads();
    const int i = r0 + tid;
    const bool mine = tid < nrows;
    cplxf *row = tile[mine ? tid : 0];
    float mv = mine ? lean_mag(row[0], i == k0) : -1.0f;
    cplxf mreg = {0.0f, 0.0f};
    bool failed = false;
    for (int kk = 0; kk < kb; ++kk) {
        const int k = k0 + kk, par = kk & 1;
        const cplxf *pprev = s_prow[par ^ 1];
        // CTA candidate (largest magnitude, lowest row)
        float bv = (mine && i >= k) ? mv : -1.0f;
        int bi = bv >= 0.0f ? i : n;
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, sh);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, sh);
            if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            s_wv[warp] = bv;
            s_wi[warp] = bi;
        }
        __syncthreads();
        if (warp == 0) {
            bv = lane < nwarps ? s_wv[lane] : -1.0f;
            bi = lane < nwarps ? s_wi[lane] : n;
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
                const float ov = __shfl_xor_sync(0xffffffffu, bv, sh);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, sh);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            // publish: the candidate as it is (pending the previous column's update)
            if (lane < kb) slot.row[par][lane] = bi < n ? tile[bi - r0][lane] : cplxf{0.0f, 0.0f};
            if (lane == 0) {
                slot.val[par] = bi < n ? bv : -1.0f;
                slot.idx[par] = bi;
            }
        }
        if (warp == 1 && k >= r0 && k < r1 && lane < kb) slot.krow[par][lane] = tile[k - r0][lane];
        __syncthreads();
        cluster_arrive();
        // the previous column's deferred update, between arrive and wait: the
        // row in registers (16-byte shared-memory accesses, compile-time
        // column indices), columns kk+1 .. kb-1 only
        if (kk > 0 && mine && i >= k) {
            float4 *r4 = reinterpret_cast<float4 *>(row);
            const float4 *p4 = reinterpret_cast<const float4 *>(pprev);
#pragma unroll
            for (int q = 0; q < NB / 2; ++q) {
                if (2 * q + 1 <= kk || 2 * q >= kb) continue;
                float4 r = r4[q];
                const float4 u = p4[q];
                if (2 * q > kk) {
                    r.x = fmaf(-mreg.re, u.x, r.x);
                    r.x = fmaf(mreg.im, u.y, r.x);
                    r.y = fmaf(-mreg.re, u.y, r.y);
                    r.y = fmaf(-mreg.im, u.x, r.y);
                }
                if (2 * q + 1 < kb) {
                    r.z = fmaf(-mreg.re, u.z, r.z);
                    r.z = fmaf(mreg.im, u.w, r.z);
                    r.w = fmaf(-mreg.re, u.w, r.w);
                    r.w = fmaf(-mreg.im, u.z, r.w);
                }
                r4[q] = r;
            }
        }
        __syncwarp();
        cluster_wait();

        // the winner over the cluster
        if (warp == 0) {
            float fv = -1.0f;
            int fi = n, fq = -1;
            if (lane < C) {
                const ClSlot *rs = cluster.map_shared_rank(&slot, lane);
                fv = rs->val[par];
                fi = rs->idx[par];
                fq = fi < n ? lane : -1;
                if (fq < 0) fv = -1.0f;
            }
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
                const float ov = __shfl_xor_sync(0xffffffffu, fv, sh);
                const int oi = __shfl_xor_sync(0xffffffffu, fi, sh);
                const int oq = __shfl_xor_sync(0xffffffffu, fq, sh);
                if (oq >= 0 && (fq < 0 || ov > fv || (ov == fv && oi < fi))) {
                    fv = ov;
                    fi = oi;
                    fq = oq;
                }
            }
            if (lane == 0) {
                s_gc = fq;
                s_gb = fv;
                s_p = fi;
            }
        }
        __syncthreads();
        const int gc = s_gc, p = s_p;
        const float gb = s_gb;
        if (gc < 0 || !isfinite(gb) || gb <= limf) {
            if (c == 0 && tid == 0) {
                st->code = 2;
                st->column = k;
                st->value = gc < 0 ? -1.0 : (double)gb;
            }
            failed = true;
            break;  // uniform over the cluster: every CTA read the same slots
        }
        // the pivot row, and row k for the owner of p, with the pending update
        cplxf *pcur = s_prow[par];
        cplxf kval = {0.0f, 0.0f};
        if (warp == 0 && lane < kb) {
            const ClSlot *ws = cluster.map_shared_rank(&slot, gc);
            cplxf v = ws->row[par][lane];
            if (kk > 0 && lane > kk) v = msub(v, ws->row[par][kk - 1], pprev[lane]);
            pcur[lane] = v;
        }
        if (warp == 1 && gc == c && p != k && lane < kb) {
            const ClSlot *ks = cluster.map_shared_rank(&slot, (k - k0) / rows_per_cta);
            kval = ks->krow[par][lane];
            if (kk > 0 && lane > kk) kval = msub(kval, ks->krow[par][kk - 1], pprev[lane]);
        }
        __syncthreads();
        if (p != k) {
            if (warp == 0 && k >= r0 && k < r1 && lane < kb) tile[k - r0][lane] = pcur[lane];
            if (warp == 1 && gc == c && lane < kb) tile[p - r0][lane] = kval;
        }
        if (c == 0 && tid == 0) piv[k] = p;
        __syncthreads();
        if (k + 1 >= n) break;
        if (mine && i > k) {
            const cplxf pv = pcur[kk];
            const float den = pv.re * pv.re + pv.im * pv.im;
            const cplxf inv = {pv.re / den, -pv.im / den};
            const cplxf x = row[kk];
            mreg = cplxf{x.re * inv.re - x.im * inv.im, x.re * inv.im + x.im * inv.re};
            row[kk] = mreg;
            if (kk + 1 < kb) {
                row[kk + 1] = msub(row[kk + 1], mreg, pcur[kk + 1]);
                mv = lean_mag(row[kk + 1], i == k + 1);
            } else {
                mv = -1.0f;
            }
        } else {
            mv = -1.0f;
        }
    }
    if (!failed) {
        __syncthreads();
        for (int t = tid; t < nrows * kb; t += blockDim.x) {
            const int ii = t / kb, j = t % kb;
            a[(size_t)(r0 + ii) * n + k0 + j] = tile[ii][j];
        }
    }
    // no CTA leaves while another may still read its shared memory
    __syncthreads();
    cluster_arrive();
    cluster_wait();
}


// Cluster FP32 panel for m rows: one CTA up to 640 rows, else C = 16 CTAs
// (8 where 16 is not available), one row per thread; false when it does
// not apply.
static bool launch_cl_panel(cplxf *a, int n, int k0, int kb, double limit, long long *piv, Status *st) {
    const int m = n - k0;
    if (m < 1) return false;
    static const size_t kMaxSmem = 200 * 1024;
    static const int max_c = [] {
        cudaFuncSetAttribute(k_panel_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
        cudaFuncSetAttribute(k_panel_cl, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(16);
        cfg.blockDim = dim3(kClMaxThreads);
        cfg.dynamicSmemBytes = kMaxSmem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int c = 0;
        if (cudaOccupancyMaxPotentialClusterSize(&c, k_panel_cl, &cfg) != cudaSuccess) c = 0;
        cudaGetLastError();
        return c >= 16 ? 16 : c >= 8 ? 8 : 0;
    }();
    if (max_c == 0) return false;
    // a panel of up to kClMaxThreads rows fits one CTA: a cluster of one,
    // whose barriers are the CTA's own (measured: the tail panels of a small
    // system take ~30 us instead of ~240 us with the single-CTA global-
    // memory panel, and the SMs left free serve the other streams of a
    // batched sweep).  Larger panels take the widest cluster: intermediate
    // sizes (2-8 CTAs) made the 8402-unknown factorisation 2 ms slower.
    const int C = m <= kClMaxThreads ? 1 : max_c;
    const int rows = (m + C - 1) / C;
    if (rows > kClMaxThreads) return false;
    const size_t smem = (size_t)rows * kClStride * sizeof(cplxf);
    if (smem > kMaxSmem) return false;
    const int threads = std::max(64, (rows + 31) / 32 * 32);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream();
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;  // a programmatic dependent (pdl_wait)
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 2;
    note_launch();
    return cuda_ok(cudaLaunchKernelEx(&cfg, k_panel_cl, a, n, k0, kb, rows, limit, piv, st), "cluster FP32 panel launch");
}


// ---- row swaps outside the panel -------------------------------------
static const int kLaswpCols = 32;  // columns per k_laswp block (shared memory 2 NB x 32 x 16 bytes at most)

template <class T>
__global__ void __launch_bounds__(256) k_laswp(T *a, int n, int k0, int kb, const long long *piv, const Status *st) {
    pdl_wait();
    pdl_trigger();
    // The kb interchanges (k, piv[k]) applied in order move at most 2 kb
    // rows.  Warp 0 composes them into (destination, source) pairs; then the
    // block stages its kLaswpCols columns of the source rows in shared memory
    // (independent, coalesced loads) and writes them to the destinations.
    // Same result as the sequential interchanges, one memory round trip.
    extern __shared__ __align__(16) unsigned char laswp_smem[];
    T *buf = reinterpret_cast<T *>(laswp_smem);  // [2 NB][kLaswpCols]
    __shared__ int s_pos[2 * NB], s_src[2 * NB], s_cnt;
    if (st->code != 0) return;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < 32) {
        // positions k0 .. k0+kb-1 first, others appended as they appear
        for (int t = lane; t < kb; t += 32) {
            s_pos[t] = k0 + t;
            s_src[t] = k0 + t;
        }
        int cnt = kb;
        // the kb pivots in one load (lane l holds piv[k0 + l]); the steps below
        // take them by shuffle instead of one dependent load each
        const int my_p = lane < kb ? (int)piv[k0 + lane] : 0;
        __syncwarp();
        for (int kk = 0; kk < kb; ++kk) {
            const int k = k0 + kk, p = __shfl_sync(0xffffffffu, my_p, kk);
            if (p == k) continue;
            int ip;
            if (p < k0 + kb) {
                ip = p - k0;
            } else {
                int f = -1;
                for (int t = lane; t < cnt; t += 32)
                    if (s_pos[t] == p) f = t;
                const unsigned hit = __ballot_sync(0xffffffffu, f >= 0);
                if (hit) {
                    ip = __shfl_sync(0xffffffffu, f, __ffs(hit) - 1);
                } else {
                    ip = cnt;
                    if (lane == 0) {
                        s_pos[cnt] = p;
                        s_src[cnt] = p;
                    }
                    ++cnt;
                }
            }
            __syncwarp();
            if (lane == 0) {
                const int t = s_src[kk];
                s_src[kk] = s_src[ip];
                s_src[ip] = t;
            }
            __syncwarp();
        }
        if (lane == 0) s_cnt = cnt;
    }
    __syncthreads();
    const int cnt = s_cnt, j0 = blockIdx.x * kLaswpCols;
    for (int e = tid; e < cnt * kLaswpCols; e += blockDim.x) {
        const int r = e / kLaswpCols, jj = e % kLaswpCols, j = j0 + jj;
        if (j < n && !(j >= k0 && j < k0 + kb)) buf[r * kLaswpCols + jj] = a[(size_t)s_src[r] * n + j];
    }
    __syncthreads();
    for (int e = tid; e < cnt * kLaswpCols; e += blockDim.x) {
        const int r = e / kLaswpCols, jj = e % kLaswpCols, j = j0 + jj;
        if (j < n && !(j >= k0 && j < k0 + kb)) a[(size_t)s_pos[r] * n + j] = buf[r * kLaswpCols + jj];
    }
}

// ---- U12 = L11^-1 A12 ------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_trsm(T *a, int n, int k0, int kb, int c0, int c1, const Status *st) {
    pdl_wait();
    pdl_trigger();
    __shared__ T L[NB][NB];
    if (st->code != 0) return;
    for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
        int i = t / kb, m = t % kb;
        L[i][m] = a[(size_t)(k0 + i) * n + k0 + m];
    }
    __syncthreads();
    int j = c0 + blockIdx.x * blockDim.x + threadIdx.x;  // columns c0 .. c1-1 (all right of the panel)
    if (j >= c1) return;
    // all loads first (independent), the substitution in registers, then the
    // stores: the loads no longer wait behind the previous rows' stores
    T x[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i)
        if (i < kb) x[i] = a[(size_t)(k0 + i) * n + j];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        if (i < kb) {
            T v = x[i];
#pragma unroll
            for (int m = 0; m < NB; ++m)
                if (m < i) v = msub(v, L[i][m], x[m]);
            x[i] = v;
        }
    }
#pragma unroll
    for (int i = 0; i < NB; ++i)
        if (i < kb) a[(size_t)(k0 + i) * n + j] = x[i];
}

// ---- A22 -= L21 U12 --------------------------------------------------
// Real: 64x64 C tile per 256-thread CTA, 4x4 per thread.
__global__ void __launch_bounds__(256) k_gemm_real(double *a, int n, int k0, int kb, const Status *st) {
    __shared__ double As[NB][64 + 1];
    __shared__ double Bs[NB][64];
    if (st->code != 0) return;
    const int r0 = k0 + kb + blockIdx.y * 64, c0 = k0 + kb + blockIdx.x * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    for (int t = threadIdx.x; t < 64 * NB; t += 256) {
        int r = t / NB, m = t % NB;  // A tile: rows r0.., cols k0..
        As[m][r] = (r0 + r < n && m < kb) ? a[(size_t)(r0 + r) * n + k0 + m] : 0.0;
        int mm = t / 64, c = t % 64;  // B tile: rows k0.., cols c0..
        Bs[mm][c] = (c0 + c < n && mm < kb) ? a[(size_t)(k0 + mm) * n + c0 + c] : 0.0;
    }
    __syncthreads();
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int r = r0 + ty + 16 * i, c = c0 + tx + 16 * j;
            acc[i][j] = (r < n && c < n) ? a[(size_t)r * n + c] : 0.0;
        }
#pragma unroll 8
    for (int m = 0; m < NB; ++m) {
        double av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = As[m][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = Bs[m][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fma(-av[i], bv[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int r = r0 + ty + 16 * i, c = c0 + tx + 16 * j;
            if (r < n && c < n) a[(size_t)r * n + c] = acc[i][j];
        }
}

// Complex: 32x64 C tile per 256-thread CTA, 2x4 per thread.
__global__ void __launch_bounds__(256) k_gemm_cplx(cplx *a, int n, int k0, int kb, const Status *st) {
    __shared__ cplx As[NB][32 + 1];
    __shared__ cplx Bs[NB][64];
    if (st->code != 0) return;
    const int r0 = k0 + kb + blockIdx.y * 32, c0 = k0 + kb + blockIdx.x * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const cplx z = {0.0, 0.0};
    for (int t = threadIdx.x; t < 32 * NB; t += 256) {
        int r = t / NB, m = t % NB;
        As[m][r] = (r0 + r < n && m < kb) ? a[(size_t)(r0 + r) * n + k0 + m] : z;
    }
    for (int t = threadIdx.x; t < 64 * NB; t += 256) {
        int mm = t / 64, c = t % 64;
        Bs[mm][c] = (c0 + c < n && mm < kb) ? a[(size_t)(k0 + mm) * n + c0 + c] : z;
    }
    __syncthreads();
    cplx acc[2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int r = r0 + ty + 16 * i, c = c0 + tx + 16 * j;
            acc[i][j] = (r < n && c < n) ? a[(size_t)r * n + c] : z;
        }
#pragma unroll 4
    for (int m = 0; m < NB; ++m) {
        cplx av[2], bv[4];
#pragma unroll
        for (int i = 0; i < 2; ++i) av[i] = As[m][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = Bs[m][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = msub(acc[i][j], av[i], bv[j]);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int r = r0 + ty + 16 * i, c = c0 + tx + 16 * j;
            if (r < n && c < n) a[(size_t)r * n + c] = acc[i][j];
        }
}

// Complex, 3 real products per complex multiply-add (Gauss / 3M):
//   T1 = Ar Br, T2 = Ai Bi, T3 = (Ar + Ai)(Br + Bi),
//   C -= (T1 - T2) + j (T3 - T1 - T2),
// 25% fewer FP64 operations than the 4-product form; the sums Ar + Ai and
// Br + Bi are formed once per tile in shared memory.  32x64 C tile per
// 256-thread CTA, 2x4 per thread.
__global__ void __launch_bounds__(256) k_gemm_cplx3m(cplx *a, int n, int k0, int kb, const Status *st) {
    extern __shared__ double sm3[];
    double *Ar = sm3, *Ai = Ar + NB * 33, *As = Ai + NB * 33;  // [NB][33]
    double *Br = As + NB * 33, *Bi = Br + NB * 64, *Bs = Bi + NB * 64;  // [NB][64]
    if (st->code != 0) return;
    const int r0 = k0 + kb + blockIdx.y * 32, c0 = k0 + kb + blockIdx.x * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    for (int t = threadIdx.x; t < 32 * NB; t += 256) {
        int r = t / NB, m = t % NB;
        cplx v = (r0 + r < n && m < kb) ? a[(size_t)(r0 + r) * n + k0 + m] : cplx{0.0, 0.0};
        Ar[m * 33 + r] = v.re;
        Ai[m * 33 + r] = v.im;
        As[m * 33 + r] = v.re + v.im;
    }
    for (int t = threadIdx.x; t < 64 * NB; t += 256) {
        int mm = t / 64, c = t % 64;
        cplx v = (c0 + c < n && mm < kb) ? a[(size_t)(k0 + mm) * n + c0 + c] : cplx{0.0, 0.0};
        Br[mm * 64 + c] = v.re;
        Bi[mm * 64 + c] = v.im;
        Bs[mm * 64 + c] = v.re + v.im;
    }
    __syncthreads();
    double t1[2][4], t2[2][4], t3[2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) t1[i][j] = t2[i][j] = t3[i][j] = 0.0;
#pragma unroll 4
    for (int m = 0; m < NB; ++m) {
        double ar[2], ai[2], as[2], br[4], bi[4], bs[4];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            ar[i] = Ar[m * 33 + ty + 16 * i];
            ai[i] = Ai[m * 33 + ty + 16 * i];
            as[i] = As[m * 33 + ty + 16 * i];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            br[j] = Br[m * 64 + tx + 16 * j];
            bi[j] = Bi[m * 64 + tx + 16 * j];
            bs[j] = Bs[m * 64 + tx + 16 * j];
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                t1[i][j] = fma(ar[i], br[j], t1[i][j]);
                t2[i][j] = fma(ai[i], bi[j], t2[i][j]);
                t3[i][j] = fma(as[i], bs[j], t3[i][j]);
            }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int r = r0 + ty + 16 * i, c = c0 + tx + 16 * j;
            if (r < n && c < n) {
                cplx v = a[(size_t)r * n + c];
                v.re -= t1[i][j] - t2[i][j];
                v.im -= (t3[i][j] - t1[i][j]) - t2[i][j];
                a[(size_t)r * n + c] = v;
            }
        }
}

static const size_t kGemm3mSmem = (size_t)NB * 33 * 3 * 8 + (size_t)NB * 64 * 3 * 8;

// ---- final diagonal check (lu.c:455-476) -----------------------------
template <class T>
__global__ void k_check_diag(const T *a, int n, double limit, Status *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || st->code != 0) return;
    double m = mag(a[(size_t)i * n + i]);
    if (!isfinite(m) || m <= limit) {
        if (atomicCAS(&st->code, 0, 3) == 0) {
            st->column = i;
            st->value = m;
        }
    }
}

// ---- complex equilibration (complex_lu.c:275-302) ---------------------
// row scales: one warp per row, max of hypot; non-finite -> status 4,
// zero row -> status 5
__global__ void k_row_scale(const cplx *in, cplx *out, int n, double *row_scale, Status *st) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const cplx *row = in + (size_t)warp * n;
    double s = 0.0;
    int bad = 0;
    for (int j = lane; j < n; j += 32) {
        double m = hypot_cr(row[j].re, row[j].im);
        if (!isfinite(m)) bad = 1;
        s = fmax(s, m);
    }
    for (int d = 16; d > 0; d >>= 1) {
        s = fmax(s, __shfl_xor_sync(0xffffffffu, s, d));
        bad |= __shfl_xor_sync(0xffffffffu, bad, d);
    }
    if (bad || s == 0.0) {
        if (lane == 0) atomicCAS(&st->code, 0, bad ? 4 : 5);
        return;
    }
    if (lane == 0) row_scale[warp] = s;
    cplx *orow = out + (size_t)warp * n;
    for (int j = lane; j < n; j += 32) {
        cplx v = row[j];
        orow[j] = cplx{v.re / s, v.im / s};
    }
}

// column scales on the row-scaled matrix: one CTA per 32 columns, its 8
// warps striding over the rows (coalesced 32-column row segments), max
// reduced in shared memory; then every entry is divided by its column scale.
__global__ void __launch_bounds__(256) k_col_max(const cplx *a, int n, double *col_scale, Status *st) {
    __shared__ double part[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane;
    double s = 0.0;
    if (j < n)
        for (int i = warp; i < n; i += 8) s = fmax(s, hypot_cr(a[(size_t)i * n + j].re, a[(size_t)i * n + j].im));
    part[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && j < n) {
        for (int w = 1; w < 8; ++w) s = fmax(s, part[w][lane]);
        if (s == 0.0) atomicCAS(&st->code, 0, 5);
        col_scale[j] = s;
    }
}

__global__ void k_col_divide(cplx *a, int n, const double *col_scale, const Status *st) {
    if (st->code != 0) return;
    size_t nn = (size_t)n * n;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nn; t += (size_t)gridDim.x * blockDim.x) {
        double c = col_scale[t % n];
        cplx v = a[t];
        a[t] = cplx{v.re / c, v.im / c};
    }
}

// ---- solves ------------------------------------------------------------
// permutation of the sequential swaps (lu.c:494-510), one thread in shared
// memory: perm[i] = source row of position i after all swaps.
// Runs only after a successful factorisation (st == nullptr or code 0):
// after a singular pivot the later pivot entries were never written.
__global__ void k_perm(const long long *piv, int n, int *perm, const Status *st) {
    extern __shared__ int sp[];
    if (st && st->code != 0) return;
    for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < n; ++k) {
            long long pl = piv[k];
            int p = (pl >= k && pl < n) ? (int)pl : k;  // pivots are rows k..n-1
            if (p != k) {
                int t = sp[k];
                sp[k] = sp[p];
                sp[p] = t;
            }
        }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

// ---------------------------------------------------------------------
// wavefront triangular solves: one cooperative launch does the forward
// (unit L) and backward (U) substitution for all right-hand sides, NR at a
// time.  Row blocks of kRB rows are owned round-robin by the CTAs (forward
// in increasing, backward in decreasing block order).  A block streams its
// off-diagonal tiles from HBM as soon as the x block they multiply is
// published (the tile itself is loaded before waiting), then applies the
// precomputed inverse of its diagonal block (k_diag_inverse) as one more
// tile and publishes x with a per-block ready flag.  The inverse turns the
// 64-step dependent substitution, which on one warp would run at a quarter
// of the SM's small FP64 rate, into a product spread over all warps.  The
// FP32 factor of the mixed path (WaveArgs::subst) solves its upper blocks by
// substitution instead, one warp per right-hand side: an FP32 inverse of an
// ill-conditioned upper block (condition numbers near 1e7 at kHz
// frequencies) is not backward stable, and iterative refinement from it
// stalls; unit lower blocks with |l_ij| <= 1 keep the inverse.
// Every task waits only on earlier tasks of the global order (forward
// 0..nb-1, then backward nb-1..0) and each CTA runs its tasks in that order,
// so with all CTAs co-resident the earliest unfinished task can always
// proceed.  Waits are bounded: on timeout the kernel records code 6 in
// *error and returns.
// ---------------------------------------------------------------------
static const int kRB = 64;
static const int kRS = kRB + 1;  // padded row stride of a block in shared memory

template <class T>
struct WaveArgs {
    const T *lu;
    const T *dinv;            // [nb][2][kRB][kRB]: L_bb^-1, U_bb^-1 (k_diag_inverse)
    int n, nb, nrhs;
    const int *perm;          // forward rhs_i = b[perm[i]] (NULL: b[i])
    const double *row_scale;  // complex: rhs divided by row_scale[perm[i]]
    const double *col_scale;  // if set, out[i] = x[i] / col_scale[i]
    const T *b;
    T *x;                     // working solution (may equal b when perm is NULL)
    T *out;                   // unscaled copy (col_scale set), else unused
    unsigned *flags;          // [nchunks][2][nb], zero on entry
    int *error;
    int subst;                // upper blocks by substitution (dinv's upper half from k_diag_copy_upper)
    const int *refine_blocks;  // if set: [nb][2] (lower, upper), 1 = that diagonal block's solve takes one
                               // step of iterative refinement after the inverse (k_diag_flags)
    const int *skip;           // if set and *skip != 0 the launch does nothing (a converged graph sweep)
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <class T>
__device__ __forceinline__ T zero_t() {
    T z;
    memset(&z, 0, sizeof(T));
    return z;
}
__device__ __forceinline__ double one_t(double) { return 1.0; }
__device__ __forceinline__ cplx one_t(cplx) { return cplx{1.0, 0.0}; }
__device__ __forceinline__ cplxf one_t(cplxf) { return cplxf{1.0f, 0.0f}; }
__device__ __forceinline__ double neg_t(double v) { return -v; }
__device__ __forceinline__ cplx neg_t(cplx v) { return cplx{-v.re, -v.im}; }
__device__ __forceinline__ cplxf neg_t(cplxf v) { return cplxf{-v.re, -v.im}; }
__device__ __forceinline__ double ldcg_t(const double *p) { return __ldcg(p); }
__device__ __forceinline__ cplx ldcg_t(const cplx *p) {
    double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
    return cplx{v.x, v.y};
}
__device__ __forceinline__ cplxf ldcg_t(const cplxf *p) {
    float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
    return cplxf{v.x, v.y};
}
__device__ __forceinline__ double scale_div(double v, double s) { return v / s; }
__device__ __forceinline__ cplx scale_div(cplx v, double s) { return cplx{v.re / s, v.im / s}; }
__device__ __forceinline__ cplxf scale_div(cplxf v, double s) {
    return cplxf{(float)(v.re / s), (float)(v.im / s)};
}

// Inverses of the diagonal blocks of a packed LU factor, one CTA per block:
// threads 0..63 each solve one column of L_bb X = I (unit lower), threads
// 64..127 one column of U_bb X = I, from the block staged in shared memory.
// Entries outside the matrix are zero.
template <class T>
__global__ void __launch_bounds__(128) k_diag_inverse(const T *lu, int n, T *dinv) {
    extern __shared__ __align__(16) unsigned char inv_smem[];
    T *blk = reinterpret_cast<T *>(inv_smem);  // kRB x kRS
    T *XL = blk + kRB * kRS, *XU = XL + kRB * kRS;
    const int b = blockIdx.x, r0 = b * kRB, nrow = min(kRB, n - r0);
    for (int t = threadIdx.x; t < kRB * kRB; t += blockDim.x) {
        int i = t / kRB, j = t % kRB;
        blk[i * kRS + j] = (i < nrow && j < nrow) ? lu[(size_t)(r0 + i) * n + r0 + j] : zero_t<T>();
        XL[i * kRS + j] = zero_t<T>();
        XU[i * kRS + j] = zero_t<T>();
    }
    __syncthreads();
    const int c = threadIdx.x & (kRB - 1);
    if (c < nrow) {
        if (threadIdx.x < kRB) {  // column c of L^-1: rows c..nrow-1
            XL[c * kRS + c] = one_t(T{});
            for (int i = c + 1; i < nrow; ++i) {
                T s = zero_t<T>();
                for (int k = c; k < i; ++k) s = msub(s, blk[i * kRS + k], XL[k * kRS + c]);
                XL[i * kRS + c] = s;
            }
        } else {  // column c of U^-1: rows c..0
            XU[c * kRS + c] = divide(one_t(T{}), blk[c * kRS + c]);
            for (int i = c - 1; i >= 0; --i) {
                T s = zero_t<T>();
                for (int k = i + 1; k <= c; ++k) s = msub(s, blk[i * kRS + k], XU[k * kRS + c]);
                XU[i * kRS + c] = divide(s, blk[i * kRS + i]);
            }
        }
    }
    __syncthreads();
    T *dl = dinv + (size_t)b * 2 * kRB * kRB, *du = dl + kRB * kRB;
    for (int t = threadIdx.x; t < kRB * kRB; t += blockDim.x) {
        int i = t / kRB, j = t % kRB;
        dl[t] = XL[i * kRS + j];
        du[t] = XU[i * kRS + j];
    }
}

// The upper diagonal blocks of a packed LU factor for substitution, over
// the U_bb^-1 half of dinv, transposed (column j of a block is row j of its
// copy): the strict upper part of U_bb with 1 / u_jj on the diagonal, zeros
// elsewhere and outside the matrix.  One CTA per block.
template <class T>
__global__ void __launch_bounds__(256) k_diag_copy_upper(const T *lu, int n, T *dinv) {
    const int b = blockIdx.x, r0 = b * kRB, nrow = min(kRB, n - r0);
    T *du = dinv + ((size_t)b * 2 + 1) * kRB * kRB;
    for (int t = threadIdx.x; t < kRB * kRB; t += blockDim.x) {
        const int j = t / kRB, i = t % kRB;  // entry (i, j) of the block goes to du[j][i]
        T u = zero_t<T>();
        if (i < nrow && j < nrow && i <= j) {
            const T v = lu[(size_t)(r0 + i) * n + r0 + j];
            u = i < j ? v : divide(one_t(T{}), v);
        }
        du[t] = u;
    }
}

// FP64 factors: the diagonal blocks whose inverse would cost the solve its
// backward stability take one step of refinement after the inverse
// (wave_block).  Per block and triangle, kappa = ||T||_inf ||T^-1||_inf
// (|re| + |im| for complex entries); applying a computed inverse perturbs
// the block's solution by up to about 64 kappa eps relative (7e-15 kappa),
// so blocks with kappa above kRefineCondition = 1e3 (or a non-finite one)
// get flag 1 (the step costs two more 64 x 64 products on the solve's
// critical path, where FP64 runs at 2 FMA per clock per SM):
// flag[2 b] for the unit lower block, flag[2 b + 1] for the upper.
static const double kRefineCondition = 1.0e3;

__device__ __forceinline__ double abs1(double v) { return fabs(v); }
__device__ __forceinline__ double abs1(cplx v) { return fabs(v.re) + fabs(v.im); }

template <class T>
__global__ void __launch_bounds__(256) k_diag_flags(const T *lu, int n, const T *dinv, int *flag) {
    __shared__ double nrm[4][kRB];  // row sums: |L|, |L^-1|, |U|, |U^-1|
    const int b = blockIdx.x, r0 = b * kRB, nrow = min(kRB, n - r0);
    const T *dl = dinv + (size_t)b * 2 * kRB * kRB, *du = dl + kRB * kRB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = warp; i < kRB; i += 8) {
        double sl = 0.0, sli = 0.0, su = 0.0, sui = 0.0;
        if (i < nrow)
            for (int j = lane; j < nrow; j += 32) {
                const double a = abs1(lu[(size_t)(r0 + i) * n + r0 + j]);
                if (j < i) sl += a;
                if (j == i) sl += 1.0;
                if (j >= i) su += a;
                sli += abs1(dl[i * kRB + j]);
                sui += abs1(du[i * kRB + j]);
            }
        for (int d = 16; d > 0; d >>= 1) {
            sl += __shfl_xor_sync(0xffffffffu, sl, d);
            sli += __shfl_xor_sync(0xffffffffu, sli, d);
            su += __shfl_xor_sync(0xffffffffu, su, d);
            sui += __shfl_xor_sync(0xffffffffu, sui, d);
        }
        if (lane == 0) {
            nrm[0][i] = sl;
            nrm[1][i] = sli;
            nrm[2][i] = su;
            nrm[3][i] = sui;
        }
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        const int t = threadIdx.x;  // 0 lower, 1 upper
        double a = 0.0, ai = 0.0;
        for (int i = 0; i < nrow; ++i) {
            a = fmax(a, nrm[2 * t][i]);
            ai = fmax(ai, nrm[2 * t + 1][i]);
        }
        const double kappa = a * ai;
        flag[2 * b + t] = !(kappa <= kRefineCondition);
    }
}

// bounded wait for *flag != 0 by one thread; false on timeout / abort
__device__ __forceinline__ bool wave_wait(const unsigned *flag, int *error) {
    long long spins = 0;
    while (ld_acquire_u32(flag) == 0u) {
        if (++spins > kSpinLimit || *(volatile int *)error) {
            atomicExch(error, 6);
            return false;
        }
        __nanosleep(32);
    }
    return true;
}

// c + m*u
__device__ __forceinline__ double mac(double c, double m, double u) { return fma(m, u, c); }
__device__ __forceinline__ cplx mac(cplx c, cplx m, cplx u) {
    c.re = fma(m.re, u.re, c.re);
    c.re = fma(-m.im, u.im, c.re);
    c.im = fma(m.re, u.im, c.im);
    c.im = fma(m.im, u.re, c.im);
    return c;
}
__device__ __forceinline__ cplxf mac(cplxf c, cplxf m, cplxf u) {
    c.re = fmaf(m.re, u.re, c.re);
    c.re = fmaf(-m.im, u.im, c.re);
    c.im = fmaf(m.re, u.im, c.im);
    c.im = fmaf(m.im, u.re, c.im);
    return c;
}
template <class T>
__device__ __forceinline__ T shfl_xor_t(T v, int m) {
    T r;
    const unsigned *pv = reinterpret_cast<const unsigned *>(&v);
    unsigned *pr = reinterpret_cast<unsigned *>(&r);
#pragma unroll
    for (int w = 0; w < (int)(sizeof(T) / 4); ++w) pr[w] = __shfl_xor_sync(0xffffffffu, pv[w], m);
    return r;
}

template <class T>
__device__ __forceinline__ T shfl_t(T v, int src) {
    T r;
    const unsigned *pv = reinterpret_cast<const unsigned *>(&v);
    unsigned *pr = reinterpret_cast<unsigned *>(&r);
#pragma unroll
    for (int w = 0; w < (int)(sizeof(T) / 4); ++w) pr[w] = __shfl_sync(0xffffffffu, pv[w], src);
    return r;
}

// shared memory of one wavefront CTA: the diagonal-block inverse (staged by
// cp.async while the off-diagonal tiles stream), the per-lane partial sums
// and the block's right-hand sides
static const int kDS = kRB + 4;  // row stride of the staged inverse (bank-conflict free)
template <class T, int NR>
struct WaveSmem {
    T dinv[kRB * kDS];
    T part[NR][kRB][33];
    T y[NR][kRB];
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <class T, int NR, bool LOWER>
__device__ bool wave_block(const WaveArgs<T> &A, int blk, int c0, int nr, unsigned *flags, WaveSmem<T, NR> &S,
                           int *s_ok) {
    constexpr int RPW = kRB / 8;  // rows per warp in the tile loop
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = A.n, nb = A.nb;
    const int r0 = blk * kRB, nrow = min(kRB, n - r0);
    // stage the inverse of the diagonal block (64 x 64, 16-byte pieces)
    {
        const T *D = A.dinv + ((size_t)blk * 2 + (LOWER ? 0 : 1)) * kRB * kRB;
        constexpr int per_row = kRB * (int)sizeof(T) / 16;
        for (int t = threadIdx.x; t < kRB * per_row; t += blockDim.x) {
            const int r = t / per_row, c = t % per_row;
            cp_async16(reinterpret_cast<char *>(S.dinv + r * kDS) + 16 * c,
                       reinterpret_cast<const char *>(D + r * kRB) + 16 * c);
        }
    }
    T acc[RPW][NR];
#pragma unroll
    for (int r = 0; r < RPW; ++r)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[r][q] = zero_t<T>();
    // off-diagonal tiles: forward j = 0..blk-1, backward j = nb-1..blk+1
    const int ntiles = LOWER ? blk : nb - 1 - blk;
    for (int t = 0; t < ntiles; ++t) {
        const int jb = LOWER ? t : nb - 1 - t;
        const int c = jb * kRB + lane;
        T a0[RPW], a1[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            const int row = r0 + warp * RPW + r;
            const bool ok = row < r0 + nrow;
            const T *ar = A.lu + (size_t)(ok ? row : r0) * n;
            a0[r] = (ok && c < n) ? ar[c] : zero_t<T>();
            a1[r] = (ok && c + 32 < n) ? ar[c + 32] : zero_t<T>();
        }
        if (threadIdx.x == 0) *s_ok = wave_wait(flags + jb, A.error);
        __syncthreads();
        if (!*s_ok) return false;
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            if (q >= nr) break;
            const T *xr = A.x + (size_t)(c0 + q) * n;
            T x0 = c < n ? ldcg_t(xr + c) : zero_t<T>();
            T x1 = c + 32 < n ? ldcg_t(xr + c + 32) : zero_t<T>();
#pragma unroll
            for (int r = 0; r < RPW; ++r) {
                acc[r][q] = msub(acc[r][q], a0[r], x0);
                acc[r][q] = msub(acc[r][q], a1[r], x1);
            }
        }
    }
    // lane partials -> shared memory (no FP64 shuffle trees: the FP64 pipe
    // is the scarce resource here)
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        if (q >= nr) break;
#pragma unroll
        for (int r = 0; r < RPW; ++r) S.part[q][warp * RPW + r][lane] = acc[r][q];
    }
    __syncthreads();
    // row sums: four threads per row, eight partials each, then two shuffles
    const int row = threadIdx.x >> 2, qq = threadIdx.x & 3;
    for (int q = 0; q < nr; ++q) {
        T s = S.part[q][row][qq * 8];
#pragma unroll
        for (int l = 1; l < 8; ++l) s = addv(s, S.part[q][row][qq * 8 + l]);
        s = addv(s, shfl_xor_t(s, 1));
        s = addv(s, shfl_xor_t(s, 2));
        if (qq == 0) {
            T v = zero_t<T>();
            if (row < nrow) {
                const int i = r0 + row;
                T rhs;
                if (LOWER && A.perm) {
                    const int src = A.perm[i];
                    rhs = ldcg_t(A.b + (size_t)(c0 + q) * n + src);
                    if (A.row_scale) rhs = scale_div(rhs, A.row_scale[src]);
                } else if (LOWER) {
                    rhs = ldcg_t(A.b + (size_t)(c0 + q) * n + i);
                } else {
                    rhs = ldcg_t(A.x + (size_t)(c0 + q) * n + i);
                }
                v = addv(rhs, s);
            }
            S.y[q][row] = v;
        }
    }
    cp_async_wait_all();
    __syncthreads();
    if (!LOWER && A.subst) {
        // x_b from U_b x_b = y by substitution, warp q for right-hand side q,
        // lane l holding rows l and l + 32; S.dinv holds U_b transposed
        // (k_diag_copy_upper), so step j reads column j as one conflict-free row
        if (warp < nr) {
            const int q = warp;
            T v0 = S.y[q][lane], v1 = S.y[q][lane + 32];
            for (int j = nrow - 1; j >= 0; --j) {
                const T *col = S.dinv + j * kDS;
                const T xj = mac(zero_t<T>(), shfl_t(j < 32 ? v0 : v1, j & 31), col[j]);
                v0 = msub(v0, col[lane], xj);
                v1 = msub(v1, col[lane + 32], xj);
                if (lane == (j & 31)) {  // row j is final: x_j (its own update above is discarded)
                    if (j < 32)
                        v0 = xj;
                    else
                        v1 = xj;
                }
            }
            T *xq = A.x + (size_t)(c0 + q) * n + r0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = lane + 32 * h;
                const T v = h ? v1 : v0;
                if (row < nrow) {
                    xq[row] = v;
                    if (A.col_scale)
                        A.out[(size_t)(c0 + q) * n + r0 + row] = scale_div(v, A.col_scale[r0 + row]);
                }
            }
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) st_release_u32(flags + blk, 1u);
        return true;
    }
    if (A.refine_blocks && A.refine_blocks[2 * blk + (LOWER ? 0 : 1)]) {
        // ill-conditioned diagonal block: x0 = D_b^-1 y, r = y - T_b x0 with
        // the block T_b of the factor (unit lower or upper), x = x0 + D_b^-1 r
        // -- one step of refinement makes the inverse-based block solve
        // backward stable (its error shrinks by kappa(T_b) eps per step).
        // S.part is free here: x0 in part[q][i][0], r in part[q][i][1].
        for (int q = 0; q < nr; ++q) {
            T v = zero_t<T>();
#pragma unroll
            for (int k = 0; k < kRB / 4; ++k) v = mac(v, S.dinv[row * kDS + qq + 4 * k], S.y[q][qq + 4 * k]);
            v = addv(v, shfl_xor_t(v, 1));
            v = addv(v, shfl_xor_t(v, 2));
            if (qq == 0) S.part[q][row][0] = row < nrow ? v : zero_t<T>();
        }
        __syncthreads();
        const T *trow = A.lu + (size_t)(r0 + (row < nrow ? row : 0)) * n + r0;
        for (int q = 0; q < nr; ++q) {
            T v = zero_t<T>();
#pragma unroll
            for (int k = 0; k < kRB / 4; ++k) {
                const int c = qq + 4 * k;
                if (row < nrow && c < nrow) {
                    T t = zero_t<T>();
                    if (LOWER)
                        t = c < row ? trow[c] : (c == row ? one_t(T{}) : zero_t<T>());
                    else if (c >= row)
                        t = trow[c];
                    v = mac(v, t, S.part[q][c][0]);
                }
            }
            v = addv(v, shfl_xor_t(v, 1));
            v = addv(v, shfl_xor_t(v, 2));
            if (qq == 0) S.part[q][row][1] = row < nrow ? addv(S.y[q][row], neg_t(v)) : zero_t<T>();
        }
        __syncthreads();
        for (int q = 0; q < nr; ++q) {
            T v = zero_t<T>();
#pragma unroll
            for (int k = 0; k < kRB / 4; ++k) v = mac(v, S.dinv[row * kDS + qq + 4 * k], S.part[q][qq + 4 * k][1]);
            v = addv(v, shfl_xor_t(v, 1));
            v = addv(v, shfl_xor_t(v, 2));
            if (qq == 0 && row < nrow) {
                v = addv(S.part[q][row][0], v);
                A.x[(size_t)(c0 + q) * n + r0 + row] = v;
                if (!LOWER && A.col_scale)
                    A.out[(size_t)(c0 + q) * n + r0 + row] = scale_div(v, A.col_scale[r0 + row]);
            }
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) st_release_u32(flags + blk, 1u);
        return true;
    }
    // x_b = D_b^-1 y: four threads per row, interleaved columns qq + 4k
    for (int q = 0; q < nr; ++q) {
        T v = zero_t<T>();
#pragma unroll
        for (int k = 0; k < kRB / 4; ++k) v = mac(v, S.dinv[row * kDS + qq + 4 * k], S.y[q][qq + 4 * k]);
        v = addv(v, shfl_xor_t(v, 1));
        v = addv(v, shfl_xor_t(v, 2));
        if (qq == 0 && row < nrow) {
            A.x[(size_t)(c0 + q) * n + r0 + row] = v;
            if (!LOWER && A.col_scale) A.out[(size_t)(c0 + q) * n + r0 + row] = scale_div(v, A.col_scale[r0 + row]);
        }
    }
    __threadfence();
    __syncthreads();  // every x of the block written; shared memory free for reuse
    if (threadIdx.x == 0) st_release_u32(flags + blk, 1u);
    return true;
}

// Tasks in ticket order: per chunk of NR right-hand sides, the forward
// blocks 0..nb-1, then the backward blocks nb-1..0.  A CTA takes the next
// ticket from a counter when it is free and every task waits only on tasks
// of lower tickets, all taken by CTAs already running, so the solve needs no
// co-residency: it is an ordinary launch, which starts on whatever SMs are
// free (under concurrent streams a cooperative launch waits until the whole
// grid fits at once).
template <class T, int NR>
__global__ void __launch_bounds__(256) k_trsv_wave(WaveArgs<T> A) {
    if (A.skip && *A.skip) return;  // uniform: written before the launch
    extern __shared__ __align__(16) unsigned char wave_smem[];
    WaveSmem<T, NR> &S = *reinterpret_cast<WaveSmem<T, NR> *>(wave_smem);
    __shared__ int s_ok, s_task;
    const int nb = A.nb;
    const int nchunks = (A.nrhs + NR - 1) / NR, total = nchunks * 2 * nb;
    unsigned *ticket = A.flags + (size_t)nchunks * 2 * nb;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(ticket, 1u);
        __syncthreads();
        const int t = s_task;
        __syncthreads();  // every thread has read s_task before the next ticket
        if (t >= total) return;
        const int chunk = t / (2 * nb), u = t - chunk * 2 * nb, c0 = chunk * NR;
        const int nr = min(NR, A.nrhs - c0);
        unsigned *ff = A.flags + (size_t)chunk * 2 * nb, *bf = ff + nb;
        if (u < nb) {
            if (!wave_block<T, NR, true>(A, u, c0, nr, ff, S, &s_ok)) return;
        } else {
            const int blk = 2 * nb - 1 - u;
            // the last block's backward step also needs the whole forward pass
            if (blk == nb - 1) {
                if (threadIdx.x == 0) s_ok = wave_wait(ff + nb - 1, A.error);
                __syncthreads();
                if (!s_ok) return;
            }
            if (!wave_block<T, NR, false>(A, blk, c0, nr, bf, S, &s_ok)) return;
        }
    }
}

template <class T>
static constexpr int wave_nr() {  // right-hand sides per wave: 8-byte scalars 4, FP64 complex 2
    return sizeof(T) == 8 ? 4 : 2;
}

// Flag words of one wavefront solve of n unknowns and nrhs right-hand sides
// (one per block and direction, then the ticket counter).
template <class T>
static size_t wave_flag_count(int n, int nrhs) {
    int nb = (n + kRB - 1) / kRB;
    return (size_t)((nrhs + wave_nr<T>() - 1) / wave_nr<T>()) * 2 * nb + 1;
}

// Elements of the diagonal-block inverses of an n x n factor.
// Elements (of 8 bytes or more) of the diagonal-block inverses of an n x n
// factor, followed by 2 nb ints: the per-block refinement flags of the FP64
// solves (k_diag_flags).
static size_t wave_dinv_count(int n) {
    int nb = (n + kRB - 1) / kRB;
    return (size_t)nb * 2 * kRB * kRB + ((size_t)2 * nb * sizeof(int) + 7) / 8;
}

template <class T>
static int *wave_refine_flags(T *dinv, int n) {
    int nb = (n + kRB - 1) / kRB;
    return reinterpret_cast<int *>(dinv + (size_t)nb * 2 * kRB * kRB);
}

// Computes the diagonal-block inverses of the factor into dinv; with subst
// the upper half then holds the transposed upper blocks for substitution
// (WaveArgs::subst).  FP64 factors also get the per-block refinement flags
// (k_diag_flags; WaveArgs::refine_blocks = wave_refine_flags(dinv)).
template <class T>
static bool wave_prepare(const T *lu, int n, T *dinv, bool subst = false) {
    constexpr size_t smem = (size_t)3 * kRB * kRS * sizeof(T);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_diag_inverse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!cuda_ok(attr, "diagonal block inverse smem attribute")) return false;
    int nb = (n + kRB - 1) / kRB;
    PEEC_LAUNCH(k_diag_inverse<T>, nb, 128, smem, lu, n, dinv);
    if (subst) {
        PEEC_LAUNCH(k_diag_copy_upper<T>, nb, 256, 0, lu, n, dinv);
    } else if constexpr (sizeof(T) == sizeof(double) || sizeof(T) == sizeof(cplx)) {
        if constexpr (!std::is_same<T, cplxf>::value)
            PEEC_LAUNCH(k_diag_flags<T>, nb, 256, 0, lu, n, dinv, wave_refine_flags(dinv, n));
    }
    return launch_ok("diagonal block inverses");
}

// Launches the wavefront solve (A.dinv from wave_prepare; flags / error as
// wave_flag_count words and one int).  Returns false on a launch failure.
template <class T>
static bool wave_solve(WaveArgs<T> A) {
    constexpr int NR = wave_nr<T>();
    static int capacity = [] {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_trsv_wave<T, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(WaveSmem<T, NR>));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_wave<T, NR>, 256, sizeof(WaveSmem<T, NR>));
        return sms * per_sm;
    }();
    if (capacity < 1) {
        set_error("triangular solve: kernel does not fit on an SM");
        return false;
    }
    A.nb = (A.n + kRB - 1) / kRB;
    const int tasks = (A.nrhs + NR - 1) / NR * 2 * A.nb;
    const int grid = std::min(tasks, capacity);
    cudaMemsetAsync(A.flags, 0, wave_flag_count<T>(A.n, A.nrhs) * sizeof(unsigned), stream());
    PEEC_LAUNCH((k_trsv_wave<T, NR>), grid, 256, sizeof(WaveSmem<T, NR>), A);
    return launch_ok("triangular solve launch");
}


// ---------------------------------------------------------------------
// registry: device copies of factorisations, keyed by the host data
// pointer and checked by a fingerprint before reuse
// ---------------------------------------------------------------------
struct Resident {
    const void *host_data = nullptr;
    size_t n = 0;
    bool complex_ = false;
    void *d_lu = nullptr;
    long long *d_piv = nullptr;
    int *d_perm = nullptr;
    double *d_row = nullptr, *d_col = nullptr;
    unsigned long long fingerprint = 0;
    size_t bytes = 0;
};

// Reuse of device factor copies across *_solve calls without re-reading the
// host factor (peec_gb300_set_factor_cache): off by default, so every solve
// uploads the caller's current host factor into the registered device
// buffers.  When on, a registered copy is reused while the host pointer,
// size, pivots, scales, diagonal and a strided sample of the factor are
// unchanged, which is only safe for callers that never edit a factor's
// other entries between solves.
static std::atomic<int> g_trust_factor_cache{0};

static std::mutex g_reg_mu;
static std::list<Resident> g_reg;
static size_t g_reg_bytes = 0;
static const size_t kRegLimit = (size_t)96 << 30;  // device bytes kept for reuse

static unsigned long long mix(unsigned long long h, unsigned long long v) {
    h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h;
}

// pivots, scales, the diagonal and a strided sample of the packed factor
static unsigned long long fingerprint(const void *data, const size_t *piv, const double *rs, const double *cs,
                                      size_t n, bool cx) {
    unsigned long long h = n;
    const unsigned long long *d = (const unsigned long long *)data;
    size_t w = cx ? 2 : 1, total = n * n * w;
    for (size_t k = 0; k < n; ++k) {
        h = mix(h, piv[k]);
        h = mix(h, d[(k * n + k) * w]);
        if (cx) h = mix(h, d[(k * n + k) * w + 1]);
        if (rs) h = mix(h, ((const unsigned long long *)rs)[k]);
        if (cs) h = mix(h, ((const unsigned long long *)cs)[k]);
    }
    size_t step = total / 4093 + 1;
    for (size_t t = 0; t < total; t += step) h = mix(h, d[t]);
    return h;
}

static void release(Resident &r) {
    dfree(r.d_lu);
    dfree(r.d_piv);
    dfree(r.d_perm);
    dfree(r.d_row);
    dfree(r.d_col);
}

static void registry_drop(const void *host_data) {
    std::lock_guard<std::mutex> g(g_reg_mu);
    for (auto it = g_reg.begin(); it != g_reg.end(); ++it)
        if (it->host_data == host_data) {
            g_reg_bytes -= it->bytes;
            release(*it);
            g_reg.erase(it);
            return;
        }
}

static void registry_put(Resident r) {
    registry_drop(r.host_data);
    std::lock_guard<std::mutex> g(g_reg_mu);
    while (!g_reg.empty() && g_reg_bytes + r.bytes > kRegLimit) {
        g_reg_bytes -= g_reg.back().bytes;
        release(g_reg.back());
        g_reg.pop_back();
    }
    g_reg_bytes += r.bytes;
    g_reg.push_front(r);
}

static void registry_set_fingerprint(const void *host_data, unsigned long long fp) {
    std::lock_guard<std::mutex> g(g_reg_mu);
    for (auto &r : g_reg)
        if (r.host_data == host_data) r.fingerprint = fp;
}

// The registered copy of host_data with this size and type; with
// any_content false its fingerprint must also equal fp.
static bool registry_get(const void *host_data, size_t n, bool cx, unsigned long long fp, bool any_content,
                         Resident &out) {
    std::lock_guard<std::mutex> g(g_reg_mu);
    for (auto it = g_reg.begin(); it != g_reg.end(); ++it)
        if (it->host_data == host_data) {
            if (it->n != n || it->complex_ != cx || (!any_content && it->fingerprint != fp)) return false;
            g_reg.splice(g_reg.begin(), g_reg, it);
            out = *it;
            return true;
        }
    return false;
}

// ---------------------------------------------------------------------
// factorisation driver
// ---------------------------------------------------------------------
// Cooperative-panel launch plan for rows m: G co-resident CTAs of 256
// threads with rows_per_cta rows each in shared memory; G = 0 if it does not
// fit (the single-CTA panel is used then).
template <class T>
struct CoopPlan {
    int G = 0, rows = 0;
    size_t smem = 0;
};

template <class T>
static CoopPlan<T> coop_plan(int m) {
    CoopPlan<T> pl;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop || m < 2 * 64) return pl;  // small panels: one CTA is faster
    int G = std::min(sms, (m + 31) / 32);
    int rows = (m + G - 1) / G;
    size_t smem = (size_t)rows * kPS * sizeof(T);
    if (smem > 200 * 1024) return pl;
    static const cudaError_t attr =  // once per type (thread-safe static initialisation)
        cudaFuncSetAttribute(k_panel_coop<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (attr != cudaSuccess) return pl;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel_coop<T>, 256, smem);
    if (per_sm < 1) return pl;
    pl.G = G;
    pl.rows = rows;
    pl.smem = smem;
    return pl;
}

// Host-side phase trace of the mixed solve on stderr (PEEC_GB300_TRACE set):
// wall milliseconds since the previous mark, after synchronising the stream.
static bool trace_enabled() {
    static const bool on = getenv("PEEC_GB300_TRACE") != nullptr;
    return on;
}

struct PhaseTrace {
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    void mark(const char *what) {
        if (!trace_enabled()) return;
        cudaStreamSynchronize(stream());
        const auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "[peec trace] %-32s %10.3f ms\n", what,
                std::chrono::duration<double, std::milli>(now - t).count());
        t = now;
    }
};

// Split-BF16 terms the mixed path's first factorisation uses: 3 (BF16x3),
// or 6 (BF16x6) with PEEC_GB300_MIXED_SPLIT=6.
static thread_local int g_start_terms = 0;  // set_mixed_start_terms
static int mixed_split_terms() {
    static const int t = [] {
        const char *e = getenv("PEEC_GB300_MIXED_SPLIT");
        return e && strcmp(e, "6") == 0 ? 6 : 3;
    }();
    return g_start_terms ? g_start_terms : t;
}

// The split terms this host thread's next mixed solves start with (3 or 6;
// 0: the default).  The batched sweep starts its fallback solves with
// BF16x6: a system its graph did not bring to the gate gains nothing from
// another BF16x3 attempt.  Returns the previous setting.
int set_mixed_start_terms(int t) {
    const int prev = g_start_terms;
    g_start_terms = (t == 3 || t == 6) ? t : 0;
    return prev;
}

// FP32 panel of the mixed path: the cluster panel (k_panel_cl) where the
// panel fits one cluster's shared memory, else the lean grid panel, else the
// cooperative one.  PEEC_GB300_MIXED_PANEL=lean / coop selects a form.
static bool cl_panel_enabled() {
    static const bool on = [] {
        const char *e = getenv("PEEC_GB300_MIXED_PANEL");
        return !(e && (strcmp(e, "lean") == 0 || strcmp(e, "coop") == 0));
    }();
    return on;
}

// CTAs of the lean FP32 panel for m rows (0: use another form); the grid
// must be co-resident.
static int lean_panel_ctas(int m) {
    static const int cap = [] {
        const char *e = getenv("PEEC_GB300_MIXED_PANEL");
        if (e && strcmp(e, "coop") == 0) return 0;
        int dev = 0, sms = 0, coop = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (!coop || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel_lean, kLeanThreads, 0) != cudaSuccess)
            return 0;
        return per_sm * sms;
    }();
    if (m < 2 * kLeanThreads) return 0;  // small panels: one CTA
    const int g = (m + kLeanThreads - 1) / kLeanThreads;
    return g <= cap && g <= 32 * kLeanPoll ? g : 0;
}

// CTAs of the lean FP64 panel (k_panel_lean64) for m rows, 0 where it does
// not apply (PEEC_GB300_PANEL=coop selects the cooperative grid panel).
template <class T>
static int lean64_panel_ctas(int m) {
    static const int cap = [] {
        const char *e = getenv("PEEC_GB300_PANEL");
        if (e && strcmp(e, "coop") == 0) return 0;
        int dev = 0, sms = 0, coop = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (!coop ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel_lean64<T>, kLeanThreads, 0) != cudaSuccess)
            return 0;
        return per_sm * sms;
    }();
    if (m < 2 * kLeanThreads) return 0;
    const int g = (m + kLeanThreads - 1) / kLeanThreads;
    return g <= cap && g <= 32 * kLeanPoll ? g : 0;
}

// Complex trailing update form: the direct 4-product form (default; it keeps
// the reference's backward error, 1.5e-11 on the 8402-unknown box) or 3 real
// products when PEEC_GB300_CGEMM=3m (17% faster, backward error 3.4e-11).
static bool complex_gemm_3m() {
    static int mode = -1;
    if (mode < 0) {
        const char *e = getenv("PEEC_GB300_CGEMM");
        mode = (e && strcmp(e, "3m") == 0) ? 1 : 0;
    }
    return mode == 1;
}

struct PanelScratch {
    PanelSlots *ps = nullptr;
    double *cand_val = nullptr;
    int *cand_idx = nullptr;
    void *cand_row = nullptr, *krow = nullptr;
};

// Optional phase timing of factor_device (extension: peec_gb300_lu_timing):
// CUDA events around the panel, swap + triangular solve, and trailing update
// launches of every block column, summed at the end of the factorisation.
struct LuTiming {
    bool enabled = false;
    double ms[4] = {0, 0, 0, 0};  // panel, swaps + trsm (+ splits), update, outer-block trailing GEMM
    double flops_update = 0.0;    // flops of the trailing updates (algorithmic, or issued BF16 for the mixed path)
    double flops_outer = 0.0;     // issued BF16 flops of the mixed path's outer-block trailing GEMMs
    std::vector<cudaEvent_t> ev;
    std::vector<int> cat;       // category of the interval that ends at each event (-1: none)
    void reset() {
        for (auto e : ev) cudaEventDestroy(e);
        ev.clear();
        cat.clear();
        ms[0] = ms[1] = ms[2] = ms[3] = 0.0;
        flops_update = flops_outer = 0.0;
    }
    void mark(int c) {
        if (!enabled) return;
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, stream());
        ev.push_back(e);
        cat.push_back(c);
    }
    void finish() {
        if (!enabled || ev.empty()) return;
        cudaEventSynchronize(ev.back());
        for (size_t i = 1; i < ev.size(); ++i) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[i - 1], ev[i]);
            if (cat[i] >= 0) ms[cat[i]] += t;
        }
    }
};
static thread_local LuTiming g_lu_timing;  // per host thread, like the stream

template <class T>
static bool factor_device(T *d_a, int n, double limit, long long *d_piv, Status *d_st) {
    LuTiming &tm = g_lu_timing;
    if (tm.enabled) tm.reset();
    DBuf<unsigned char> scratch;
    PanelScratch sc;
    // lean FP64 panel slots: ceil(n / 64) CTAs at most
    const size_t GL = (size_t)(n + kLeanThreads - 1) / kLeanThreads;
    const int lean_stride = (int)((GL + 63) / 64 * 64);
    DBuf<unsigned long long> lean_flag(2 * (size_t)lean_stride);
    DBuf<int> lean_idx(2 * GL);
    DBuf<double> lean_val(2 * GL);
    DBuf<T> lean_rows(2 * GL * NB + 2 * NB);
    if (!lean_flag.p || !lean_idx.p || !lean_val.p || !lean_rows.p) return false;
    cudaMemsetAsync(lean_flag.p, 0, lean_flag.n * sizeof(unsigned long long), stream());
    {
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        size_t G = (size_t)sms;
        size_t bytes = 256 + 2 * G * 8 + 2 * G * 4 + 2 * G * NB * sizeof(T) + 2 * NB * sizeof(T) + 64;
        if (!scratch.alloc(bytes)) return false;
        cudaMemsetAsync(scratch.p, 0, bytes, stream());
        unsigned char *b = scratch.p;
        sc.ps = (PanelSlots *)b;
        sc.cand_val = (double *)(b + 256);
        sc.cand_idx = (int *)(b + 256 + 2 * G * 8);
        size_t off = 256 + 2 * G * 8 + 2 * G * 4;
        off = (off + 15) & ~(size_t)15;
        sc.cand_row = b + off;
        sc.krow = b + off + 2 * G * NB * sizeof(T);
    }
    for (int k0 = 0; k0 < n; k0 += NB) {
        int kb = std::min(NB, n - k0);
        tm.mark(2);
        CoopPlan<T> pl = coop_plan<T>(n - k0);
        const int lean_g = lean64_panel_ctas<T>(n - k0);
        if (lean_g > 0) {
            unsigned long long *fl = lean_flag.p;
            int fls = lean_stride;
            int *li = lean_idx.p;
            double *lv = lean_val.p;
            T *lr = lean_rows.p, *lk = lean_rows.p + 2 * GL * NB;
            void *args[] = {&d_a, &n, (void *)&k0, &kb, &limit, &d_piv, &d_st, &sc.ps, &fl, &fls, &li, &lv, &lr, &lk};
            if (!cuda_ok(cudaLaunchCooperativeKernel((const void *)k_panel_lean64<T>, dim3(lean_g), dim3(kLeanThreads),
                                                     args, 0, stream()),
                         "lean FP64 panel launch"))
                return false;
            note_launch();
        } else if (pl.G > 0) {
            int rows = pl.rows;
            T *cr = (T *)sc.cand_row, *kr = (T *)sc.krow;
            void *args[] = {&d_a, &n, (void *)&k0, &kb, &rows, &limit, &d_piv, &d_st, &sc.ps, &sc.cand_val,
                            &sc.cand_idx, &cr, &kr};
            if (!cuda_ok(cudaLaunchCooperativeKernel((const void *)k_panel_coop<T>, dim3(pl.G), dim3(256), args,
                                                     pl.smem, stream()),
                         "cooperative panel launch"))
                return false;
            note_launch();
        } else {
            PEEC_LAUNCH(k_panel<T>, 1, 1024, 0, d_a, n, k0, kb, limit, d_piv, d_st);
        }
        tm.mark(0);
        PEEC_LAUNCH(k_laswp<T>, (n + kLaswpCols - 1) / kLaswpCols, 256, 2 * NB * kLaswpCols * sizeof(T), d_a, n, k0, kb,
                    d_piv, d_st);
        int rest = n - (k0 + kb);
        if (rest > 0) {
            PEEC_LAUNCH(k_trsm<T>, (rest + 255) / 256, 256, 0, d_a, n, k0, kb, k0 + kb, n, d_st);
        }
        tm.mark(1);
        if (tm.enabled) tm.flops_update += (sizeof(T) == sizeof(double) ? 2.0 : 8.0) * (double)rest * rest * kb;
        if (rest > 0) {
            if constexpr (sizeof(T) == sizeof(double)) {
                dim3 g((rest + 63) / 64, (rest + 63) / 64);
                PEEC_LAUNCH(k_gemm_real, g, 256, 0, (double *)d_a, n, k0, kb, d_st);
            } else {
                dim3 g((rest + 63) / 64, (rest + 31) / 32);
                if (complex_gemm_3m()) {
                    static const cudaError_t attr = cudaFuncSetAttribute(
                        k_gemm_cplx3m, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemm3mSmem);
                    (void)attr;
                    PEEC_LAUNCH(k_gemm_cplx3m, g, 256, kGemm3mSmem, (cplx *)d_a, n, k0, kb, d_st);
                } else {
                    PEEC_LAUNCH(k_gemm_cplx, g, 256, 0, (cplx *)d_a, n, k0, kb, d_st);
                }
            }
        }
    }
    tm.mark(2);
    tm.finish();
    PEEC_LAUNCH(k_check_diag<T>, (n + 255) / 256, 256, 0, d_a, n, limit, d_st);
    return launch_ok("LU kernels");
}

template <class T>
static bool solve_device(const T *d_lu, const int *d_perm, const double *d_row, const double *d_col, int n,
                         const T *d_b, T *d_x, int nrhs) {
    constexpr bool cx = sizeof(T) == sizeof(cplx);
    DBuf<unsigned> flags(wave_flag_count<T>(n, nrhs));
    DBuf<int> err(1);
    DBuf<T> work(cx ? (size_t)n * nrhs : 0), dinv(wave_dinv_count(n));
    if (!flags.p || !err.p || (cx && !work.p) || !dinv.p) return false;
    if (!cuda_ok(cudaMemsetAsync(err.p, 0, sizeof(int), stream()), "solve scratch")) return false;
    if (!wave_prepare(d_lu, n, dinv.p)) return false;
    WaveArgs<T> A{};
    A.lu = d_lu;
    A.dinv = dinv.p;
    A.refine_blocks = wave_refine_flags(dinv.p, n);
    A.n = n;
    A.nrhs = nrhs;
    A.perm = d_perm;
    A.row_scale = cx ? d_row : nullptr;
    A.col_scale = cx ? d_col : nullptr;
    A.b = d_b;
    A.x = cx ? work.p : d_x;  // complex: scaled solution in scratch, unscaled into d_x
    A.out = d_x;
    A.flags = flags.p;
    A.error = err.p;
    if (!wave_solve(A)) return false;
    int herr = 0;
    cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!launch_ok("LU solve kernels") || !sync("LU solve")) return false;
    if (herr) {
        set_error("triangular solve: a wait for an earlier row block timed out");
        return false;
    }
    return true;
}

}  // namespace peec

using namespace peec;

// =====================================================================
// C ABI: lu.h
// =====================================================================
extern "C" {

int peec_gb300_set_factor_cache(int trust) { return g_trust_factor_cache.exchange(trust ? 1 : 0); }

void lu_options_default(LUOptions *options, int parallel_threads) {
    if (!options) return;
    options->parallel_threads = parallel_threads;
    options->pivot_tolerance = 1.0e-14;
    options->parallel_threshold = 64;
}

void lu_init(LUFactorization *lu) {
    if (lu) memset(lu, 0, sizeof(*lu));
}

void lu_free(LUFactorization *lu) {
    if (!lu) return;
    if (lu->data) registry_drop(lu->data);
    free(lu->data);
    free(lu->pivots);
    lu_init(lu);
}

}  // extern "C"

namespace peec {

// Equilibrate (complex), scale, factor and build the solve permutation of a
// device-resident matrix in place.  Returns -1 on a CUDA failure, else 0
// with *hs holding the device status (code 0 ok) and *scale max|A| (NaN
// ignored).  A zero / non-finite complex row or column gives hs->code 4/5
// before any factorisation.
template <class T>
static int factor_inplace(T *d_a, int n, double pivot_tolerance, bool cx, long long *d_piv, int *d_perm,
                          double *d_row, double *d_col, double *scale, Status *hs) {
    size_t nn = (size_t)n * n;
    DBuf<Status> st(1);
    DBuf<unsigned long long> mx(1);
    if (!st.p || !mx.p) return -1;
    cudaMemsetAsync(st.p, 0, sizeof(Status), stream());
    cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), stream());
    if (cx) {
        // complex_lu.c:275-302: row scales, then column scales of the row-scaled matrix
        PEEC_LAUNCH(k_row_scale, (unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, (const cplx *)d_a, (cplx *)d_a, n,
                    d_row, st.p);
        PEEC_LAUNCH(k_col_max, (n + 31) / 32, 256, 0, (const cplx *)d_a, n, d_col, st.p);
        PEEC_LAUNCH(k_col_divide, 152 * 16, 256, 0, (cplx *)d_a, n, d_col, st.p);
    }
    PEEC_LAUNCH(k_max_mag<T>, 152 * 8, 256, 0, d_a, nn, mx.p);
    unsigned long long bits = 0;
    cudaMemcpyAsync(&bits, mx.p, sizeof(bits), cudaMemcpyDeviceToHost, stream());
    cudaMemcpyAsync(hs, st.p, sizeof(Status), cudaMemcpyDeviceToHost, stream());
    if (!sync("LU scale")) return -1;
    memcpy(scale, &bits, sizeof(double));
    if (hs->code != 0 || !isfinite(*scale) || *scale <= 0.0) return 0;
    double limit = pivot_tolerance * *scale;
    if (!factor_device<T>(d_a, n, limit, d_piv, st.p)) return -1;
    size_t perm_smem = (size_t)n * sizeof(int);
    if (perm_smem > 48 * 1024) cudaFuncSetAttribute(k_perm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)perm_smem);
    PEEC_LAUNCH(k_perm, 1, 1024, perm_smem, d_piv, n, d_perm, st.p);
    cudaMemcpyAsync(hs, st.p, sizeof(Status), cudaMemcpyDeviceToHost, stream());
    if (!launch_ok("LU permutation") || !sync("LU factorisation")) return -1;
    if (hs->code == 6) {
        set_error("LU panel synchronisation timed out");
        return -1;
    }
    return 0;
}

static void report_status(const Status &hs, bool cx) {
    if (hs.code == 2)
        fprintf(stderr, cx ? "ERROR: complex LU matrix is singular or nearly singular at column %d, |pivot| = %.9e.\n"
                           : "ERROR: LU matrix is singular or nearly singular at column %d, |pivot| = %.9e.\n",
                hs.column, hs.value);
    else if (hs.code == 3)
        fprintf(stderr, cx ? "ERROR: invalid complex U diagonal at [%d,%d], |Uii| = %.9e.\n"
                           : "ERROR: invalid diagonal U[%d,%d] = %.9e.\n",
                hs.column, hs.column, hs.value);
}

// Shared host driver for both factorisations.  On success the factor stays
// resident on the device (registry) for the solves.
template <class T>
static int factorize_common(const T *input, size_t n, double pivot_tolerance, bool cx, T *host_lu, size_t *host_piv,
                            size_t *swap_count, double *matrix_scale, double *row_scale, double *col_scale) {
    int ni = (int)n;
    size_t nn = n * n;
    Resident r;
    r.n = n;
    r.complex_ = cx;
    r.bytes = nn * sizeof(T) + n * (sizeof(long long) + sizeof(int) + (cx ? 2 * sizeof(double) : 0));
    r.d_lu = dalloc(nn * sizeof(T));
    r.d_piv = (long long *)dalloc(n * sizeof(long long));
    r.d_perm = (int *)dalloc(n * sizeof(int));
    if (cx) {
        r.d_row = (double *)dalloc(n * sizeof(double));
        r.d_col = (double *)dalloc(n * sizeof(double));
    }
    if (!r.d_lu || !r.d_piv || !r.d_perm || (cx && (!r.d_row || !r.d_col))) {
        release(r);
        return -1;
    }
    T *d_a = (T *)r.d_lu;
    if (!cuda_ok(cudaMemcpyAsync(d_a, input, nn * sizeof(T), cudaMemcpyHostToDevice, stream()), "LU upload")) {
        release(r);
        return -1;
    }
    Status hs;
    double scale = 0.0;
    if (factor_inplace<T>(d_a, ni, pivot_tolerance, cx, r.d_piv, r.d_perm, r.d_row, r.d_col, &scale, &hs) != 0) {
        release(r);
        return -1;
    }
    if (hs.code == 4 || hs.code == 5) {  // zero or non-finite row / column of the complex input
        release(r);
        return -2;
    }
    *matrix_scale = scale;
    if (!isfinite(scale) || scale <= 0.0) {
        fprintf(stderr, cx ? "ERROR: complex LU input matrix is invalid or zero.\n"
                           : "ERROR: LU input matrix is zero or contains invalid values.\n");
        release(r);
        return -2;
    }
    std::vector<long long> piv(n);
    bool copied = cuda_ok(cudaMemcpyAsync(host_lu, d_a, nn * sizeof(T), cudaMemcpyDeviceToHost, stream()), "LU download") &&
                  cuda_ok(cudaMemcpyAsync(piv.data(), r.d_piv, n * sizeof(long long), cudaMemcpyDeviceToHost, stream()),
                          "pivot download");
    if (cx && copied)
        copied = cuda_ok(cudaMemcpyAsync(row_scale, r.d_row, n * sizeof(double), cudaMemcpyDeviceToHost, stream()), "scale") &&
                 cuda_ok(cudaMemcpyAsync(col_scale, r.d_col, n * sizeof(double), cudaMemcpyDeviceToHost, stream()), "scale");
    if (!sync("LU download") || !copied) {
        release(r);
        return -1;
    }
    size_t done = hs.code == 0 ? n : (size_t)hs.column;
    size_t swaps = 0;
    for (size_t k = 0; k < n; ++k) {
        host_piv[k] = k < done ? (size_t)piv[k] : k;
        if (k < done && host_piv[k] != k) ++swaps;
    }
    *swap_count = swaps;
    if (hs.code != 0) {
        report_status(hs, cx);
        release(r);
        return -2;
    }
    r.host_data = host_lu;
    r.fingerprint = fingerprint(host_lu, host_piv, cx ? row_scale : nullptr, cx ? col_scale : nullptr, n, cx);
    registry_put(r);
    return 0;
}

template <class T>
static bool upload_factor(Resident &r, const T *data, const size_t *pivots, const double *rs, const double *cs,
                          size_t n, bool cx) {
    std::vector<long long> piv(n);
    for (size_t k = 0; k < n; ++k) {
        if (pivots[k] >= n) return false;
        piv[k] = (long long)pivots[k];
    }
    bool ok = cuda_ok(cudaMemcpyAsync(r.d_lu, data, n * n * sizeof(T), cudaMemcpyHostToDevice, stream()), "factor upload") &&
              cuda_ok(cudaMemcpyAsync(r.d_piv, piv.data(), n * sizeof(long long), cudaMemcpyHostToDevice, stream()),
                      "pivot upload");
    if (cx && ok)
        ok = cuda_ok(cudaMemcpyAsync(r.d_row, rs, n * sizeof(double), cudaMemcpyHostToDevice, stream()), "scale upload") &&
             cuda_ok(cudaMemcpyAsync(r.d_col, cs, n * sizeof(double), cudaMemcpyHostToDevice, stream()), "scale upload");
    size_t perm_smem = n * sizeof(int);
    if (perm_smem > 48 * 1024) cudaFuncSetAttribute(k_perm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)perm_smem);
    if (ok) PEEC_LAUNCH(k_perm, 1, 1024, perm_smem, r.d_piv, (int)n, r.d_perm, (const Status *)nullptr);
    return ok && sync("factor upload");
}

// Device copy of a host factorisation: the registered buffers, refreshed
// from the host factor (or reused unread when the cache is trusted and the
// fingerprint matches), else new buffers uploaded now and registered.
template <class T>
static bool resident_for(const T *data, const size_t *pivots, const double *rs, const double *cs, size_t n, bool cx,
                         Resident &out) {
    unsigned long long fp = fingerprint(data, pivots, rs, cs, n, cx);
    Resident r;
    if (registry_get(data, n, cx, g_trust_factor_cache.load() ? fp : 0, !g_trust_factor_cache.load(), r)) {
        if (g_trust_factor_cache.load()) {
            out = r;
            return true;
        }
        if (!upload_factor<T>(r, data, pivots, rs, cs, n, cx)) {
            registry_drop(data);
            return false;
        }
        registry_set_fingerprint(data, fp);
        out = r;
        return true;
    }
    r = Resident();
    r.host_data = data;
    r.n = n;
    r.complex_ = cx;
    r.fingerprint = fp;
    r.bytes = n * n * sizeof(T) + n * (sizeof(long long) + sizeof(int) + (cx ? 2 * sizeof(double) : 0));
    r.d_lu = dalloc(n * n * sizeof(T));
    r.d_piv = (long long *)dalloc(n * sizeof(long long));
    r.d_perm = (int *)dalloc(n * sizeof(int));
    if (cx) {
        r.d_row = (double *)dalloc(n * sizeof(double));
        r.d_col = (double *)dalloc(n * sizeof(double));
    }
    if (!r.d_lu || !r.d_piv || !r.d_perm || (cx && (!r.d_row || !r.d_col)) ||
        !upload_factor<T>(r, data, pivots, rs, cs, n, cx)) {
        release(r);
        return false;
    }
    registry_put(r);
    out = r;
    return true;
}

template <class T>
static int solve_common(const T *data, const size_t *pivots, const double *rs, const double *cs, size_t n, bool cx,
                        const T *B, T *X, size_t nrhs) {
    if (n > (size_t)0x7fffffff || nrhs > (size_t)0x7fffffff) return -1;
    Resident r;
    if (!resident_for<T>(data, pivots, rs, cs, n, cx, r)) return -1;
    size_t tot = n * nrhs;
    DBuf<T> db(tot), dx(tot);
    if (!db.p || !dx.p) return -1;
    if (!db.upload(B, tot)) return -1;
    if (!solve_device<T>((const T *)r.d_lu, r.d_perm, r.d_row, r.d_col, (int)n, db.p, dx.p, (int)nrhs)) return -1;
    if (!dx.download(X, tot) || !sync("LU solve")) return -1;
    for (size_t t = 0; t < tot; ++t) {
        const double *v = (const double *)&X[t];
        for (size_t w = 0; w < sizeof(T) / 8; ++w)
            if (!isfinite(v[w])) return -1;  // zero / non-finite diagonal reached
    }
    return 0;
}

}  // namespace peec

extern "C" {

int lu_factorize(const double *input, size_t n, const LUOptions *options, LUFactorization *lu) {
    if (!input || !options || !lu || n == 0) return -1;
    if (options->parallel_threads < 1) return -1;
    if (n > (size_t)0x7fffffff || n > SIZE_MAX / n || n * n > SIZE_MAX / sizeof(double)) {
        fprintf(stderr, "ERROR: LU matrix size overflow.\n");
        return -1;
    }
    lu_init(lu);
    lu->n = n;
    lu->data = (double *)malloc(n * n * sizeof(double));
    lu->pivots = (size_t *)malloc(n * sizeof(size_t));
    if (!lu->data || !lu->pivots) {
        fprintf(stderr, "ERROR: cannot allocate LU factorization.\n");
        lu_free(lu);
        return -1;
    }
    int s = factorize_common<double>(input, n, options->pivot_tolerance, false, lu->data, lu->pivots,
                                     &lu->swap_count, &lu->matrix_scale, nullptr, nullptr);
    if (s == -1 || (s == -2 && !isfinite(lu->matrix_scale)) || (s == -2 && lu->matrix_scale <= 0.0)) {
        lu_free(lu);
        return s;
    }
    lu->factorized = s == 0;
    return s;
}

int lu_solve(const LUFactorization *lu, const double *b, double *x) {
    if (!lu || !b || !x || !lu->data || !lu->pivots || !lu->factorized) return -1;
    return solve_common<double>(lu->data, lu->pivots, nullptr, nullptr, lu->n, false, b, x, 1);
}

int lu_solve_multiple(const LUFactorization *lu, const double *B, double *X, size_t rhs_count, int parallel_threads) {
    if (!lu || !B || !X || rhs_count == 0 || parallel_threads < 1 || !lu->factorized) return -1;
    if (!lu->data || !lu->pivots) return -1;
    return solve_common<double>(lu->data, lu->pivots, nullptr, nullptr, lu->n, false, B, X, rhs_count);
}

double lu_determinant(const LUFactorization *lu) {
    if (!lu || !lu->data || !lu->factorized) return NAN;
    double det = (lu->swap_count % 2 == 0) ? 1.0 : -1.0;
    for (size_t i = 0; i < lu->n; ++i) det *= lu->data[i * lu->n + i];
    return det;
}

void lu_print_info(const LUFactorization *lu) {
    if (!lu) return;
    printf("\n========================================\n");
    printf("LU FACTORIZATION (GPU)\n");
    printf("========================================\n");
    printf("Size         : %zu x %zu\n", lu->n, lu->n);
    printf("Swap count   : %zu\n", lu->swap_count);
    printf("Matrix scale : %.9e\n", lu->matrix_scale);
    printf("Factorized   : %s\n", lu->factorized ? "yes" : "no");
    if (lu->data && lu->n > 0)
        printf("LU memory    : %.3f MiB\n", ((double)lu->n * (double)lu->n * sizeof(double)) / (1024.0 * 1024.0));
    printf("========================================\n");
}

// =====================================================================
// C ABI: complex_lu.h
// =====================================================================
void complex_lu_options_default(ComplexLUOptions *options, int parallel_threads) {
    if (!options) return;
    options->parallel_threads = parallel_threads;
    options->pivot_tolerance = 1.0e-14;
    options->parallel_threshold = 64;
}

void complex_lu_init(ComplexLUFactorization *lu) {
    if (lu) memset(lu, 0, sizeof(*lu));
}

void complex_lu_free(ComplexLUFactorization *lu) {
    if (!lu) return;
    if (lu->data) registry_drop(lu->data);
    free(lu->data);
    free(lu->pivots);
    free(lu->row_scale);
    free(lu->column_scale);
    complex_lu_init(lu);
}

int complex_lu_factorize(const Complex *input, size_t n, const ComplexLUOptions *options,
                         ComplexLUFactorization *lu) {
    if (!input || !options || !lu || n == 0 || options->parallel_threads < 1 || !isfinite(options->pivot_tolerance) ||
        options->pivot_tolerance < 0.0)
        return -1;
    if (n > (size_t)0x7fffffff || n > SIZE_MAX / n || n * n > SIZE_MAX / sizeof(Complex)) {
        fprintf(stderr, "ERROR: complex LU matrix size overflow.\n");
        return -1;
    }
    complex_lu_init(lu);
    lu->n = n;
    lu->data = (Complex *)malloc(n * n * sizeof(Complex));
    lu->pivots = (size_t *)malloc(n * sizeof(size_t));
    lu->row_scale = (double *)malloc(n * sizeof(double));
    lu->column_scale = (double *)malloc(n * sizeof(double));
    if (!lu->data || !lu->pivots || !lu->row_scale || !lu->column_scale) {
        fprintf(stderr, "ERROR: cannot allocate complex LU factorization.\n");
        complex_lu_free(lu);
        return -1;
    }
    lu->matrix_scale = 0.0;
    int s = factorize_common<cplx>((const cplx *)input, n, options->pivot_tolerance, true, (cplx *)lu->data,
                                   lu->pivots, &lu->swap_count, &lu->matrix_scale, lu->row_scale, lu->column_scale);
    // equilibration / scale failures release everything (complex_lu.c:275-320);
    // a singular pivot keeps the partial factor for the caller to free
    if (s == -1 || (s == -2 && (!isfinite(lu->matrix_scale) || lu->matrix_scale <= 0.0))) {
        complex_lu_free(lu);
        return s;
    }
    lu->factorized = s == 0;
    return s;
}

int complex_lu_solve(const ComplexLUFactorization *lu, const Complex *b, Complex *x) {
    if (!lu || !b || !x || !lu->data || !lu->pivots || !lu->factorized) return -1;
    if (!lu->row_scale || !lu->column_scale) return -1;
    return solve_common<cplx>((const cplx *)lu->data, lu->pivots, lu->row_scale, lu->column_scale, lu->n, true,
                              (const cplx *)b, (cplx *)x, 1);
}

int complex_lu_solve_multiple(const ComplexLUFactorization *lu, const Complex *B, Complex *X, size_t rhs_count,
                              int parallel_threads) {
    if (!lu || !B || !X || rhs_count == 0 || parallel_threads < 1 || !lu->factorized) return -1;
    if (!lu->data || !lu->pivots || !lu->row_scale || !lu->column_scale) return -1;
    return solve_common<cplx>((const cplx *)lu->data, lu->pivots, lu->row_scale, lu->column_scale, lu->n, true,
                              (const cplx *)B, (cplx *)X, rhs_count);
}

void complex_lu_print_info(const ComplexLUFactorization *lu) {
    if (!lu) return;
    printf("\n========================================\n");
    printf("COMPLEX LU FACTORIZATION (GPU)\n");
    printf("========================================\n");
    printf("Size         : %zu x %zu\n", lu->n, lu->n);
    printf("Swap count   : %zu\n", lu->swap_count);
    printf("Matrix scale : %.9e\n", lu->matrix_scale);
    printf("Factorized   : %s\n", lu->factorized ? "yes" : "no");
    if (lu->data && lu->n > 0)
        printf("LU memory    : %.3f MiB\n", ((double)lu->n * (double)lu->n * sizeof(Complex)) / (1024.0 * 1024.0));
    printf("========================================\n");
}

}  // extern "C"

// =====================================================================
// extension: factor / solve matrices that already live on the device
// =====================================================================
extern "C" {

int peec_gb300_lu_factor_device(double *d_a, size_t n, double pivot_tolerance, long long *d_piv, int *d_perm,
                                double *matrix_scale, int *failed_column) {
    if (!d_a || !d_piv || !d_perm || n == 0 || n > (size_t)0x7fffffff) return -1;
    Status hs;
    double scale = 0.0;
    if (factor_inplace<double>(d_a, (int)n, pivot_tolerance, false, d_piv, d_perm, nullptr, nullptr, &scale, &hs) != 0)
        return -1;
    if (matrix_scale) *matrix_scale = scale;
    if (failed_column) *failed_column = hs.code ? hs.column : -1;
    if (!isfinite(scale) || scale <= 0.0) return -2;
    if (hs.code) {
        report_status(hs, false);
        return -2;
    }
    return 0;
}

int peec_gb300_complex_lu_factor_device(Complex *d_a, size_t n, double pivot_tolerance, long long *d_piv, int *d_perm,
                                        double *d_row_scale, double *d_column_scale, double *matrix_scale,
                                        int *failed_column) {
    if (!d_a || !d_piv || !d_perm || !d_row_scale || !d_column_scale || n == 0 || n > (size_t)0x7fffffff) return -1;
    Status hs;
    double scale = 0.0;
    if (factor_inplace<cplx>((cplx *)d_a, (int)n, pivot_tolerance, true, d_piv, d_perm, d_row_scale, d_column_scale,
                             &scale, &hs) != 0)
        return -1;
    if (matrix_scale) *matrix_scale = scale;
    if (failed_column) *failed_column = hs.code ? hs.column : -1;
    if (hs.code == 4 || hs.code == 5 || !isfinite(scale) || scale <= 0.0) return -2;
    if (hs.code) {
        report_status(hs, true);
        return -2;
    }
    return 0;
}

int peec_gb300_lu_solve_device(const double *d_lu, const int *d_perm, size_t n, const double *d_b, double *d_x,
                               size_t nrhs) {
    if (!d_lu || !d_perm || !d_b || !d_x || n == 0 || nrhs == 0 || d_b == d_x) return -1;
    if (!solve_device<double>(d_lu, d_perm, nullptr, nullptr, (int)n, d_b, d_x, (int)nrhs)) return -1;
    return 0;
}

int peec_gb300_complex_lu_solve_device(const Complex *d_lu, const int *d_perm, const double *d_row_scale,
                                       const double *d_column_scale, size_t n, const Complex *d_b, Complex *d_x,
                                       size_t nrhs) {
    if (!d_lu || !d_perm || !d_row_scale || !d_column_scale || !d_b || !d_x || n == 0 || nrhs == 0 || d_b == d_x)
        return -1;
    if (!solve_device<cplx>((const cplx *)d_lu, d_perm, d_row_scale, d_column_scale, (int)n, (const cplx *)d_b,
                            (cplx *)d_x, (int)nrhs))
        return -1;
    return 0;
}

}  // extern "C"

// =====================================================================
// Allocation-free real factorisation
//
// Some callers cannot let a library allocate device memory: applications
// that own every byte of the GPU through their own pool or hard budget (a
// hidden cudaMalloc would break their accounting or fail under the cap), and
// tight solver loops where cudaMalloc / cudaFree would synchronise the
// device.  For them peec_gb300_lu_factor_device_noalloc keeps all of its
// scratch -- the status word, the scale reduction and the cooperative
// panel's exchange slots -- in one file-scope device array of fixed size,
// which every GPU that loads this library holds until the process exits.
// =====================================================================
namespace peec {

static const size_t kNoAllocScratchBytes = 256 * 1024;
static const size_t kNoAllocMaxN = 50000;  // the permutation kernel keeps n ints in shared memory
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host-side name of the array is not a device address: resolve it on every
// call with the caller's device current (no allocation, and no address kept
// across a device reset or a reload of the module).
static unsigned char *noalloc_scratch() {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        set_error("cudaGetSymbolAddress of the static LU scratch failed: %s", cudaGetErrorString(e));
        return nullptr;
    }
    return (unsigned char *)p;
}

}  // namespace peec

extern "C" int peec_gb300_lu_factor_device_noalloc(double *d_a, size_t n, double pivot_tolerance, long long *d_piv,
                                                   int *d_perm, double *matrix_scale, int *failed_column) {
    if (!d_a || !d_piv || !d_perm || n == 0) return -1;
    if (n > kNoAllocMaxN) {
        set_error("peec_gb300_lu_factor_device_noalloc: n = %zu exceeds the maximum %zu", n, kNoAllocMaxN);
        return -1;
    }
    int dev = 0, sms = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "current device") ||
        !cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))
        return -1;
    // layout: status | scale word | panel slots | candidates | candidate rows | row k
    const size_t G = (size_t)sms;
    const size_t off_mx = 64, off_ps = 128, off_val = 256, off_idx = off_val + 2 * G * 8;
    const size_t off_row = (off_idx + 2 * G * 4 + 15) & ~(size_t)15;
    const size_t off_krow = off_row + 2 * G * NB * sizeof(double);
    const size_t need = off_krow + 2 * NB * sizeof(double);
    if (need > kNoAllocScratchBytes) {
        set_error("peec_gb300_lu_factor_device_noalloc: %d SMs need %zu scratch bytes, the maximum is %zu", sms, need,
                  kNoAllocScratchBytes);
        return -1;
    }
    unsigned char *base = noalloc_scratch();
    if (!base) return -1;
    Status *st = (Status *)base;
    unsigned long long *mx = (unsigned long long *)(base + off_mx);
    PanelScratch sc;
    sc.ps = (PanelSlots *)(base + off_ps);
    sc.cand_val = (double *)(base + off_val);
    sc.cand_idx = (int *)(base + off_idx);
    sc.cand_row = base + off_row;
    sc.krow = base + off_krow;
    // the array keeps the previous call's contents: clear what must start at zero
    if (!cuda_ok(cudaMemsetAsync(base, 0, need, stream()), "scratch reset")) return -1;
    const int ni = (int)n;
    PEEC_LAUNCH(k_max_mag<double>, 152 * 8, 256, 0, d_a, n * n, mx);
    unsigned long long bits = 0;
    Status hs;
    cudaMemcpyAsync(&bits, mx, sizeof(bits), cudaMemcpyDeviceToHost, stream());
    if (!sync("LU scale")) return -1;
    double scale;
    memcpy(&scale, &bits, sizeof(scale));
    if (matrix_scale) *matrix_scale = scale;
    if (failed_column) *failed_column = -1;
    if (!isfinite(scale) || scale <= 0.0) return -2;
    double limit = pivot_tolerance * scale;
    for (int k0 = 0; k0 < ni; k0 += NB) {
        int kb = std::min(NB, ni - k0);
        CoopPlan<double> pl = coop_plan<double>(ni - k0);
        if (pl.G > 0) {
            int rows = pl.rows;
            double *cr = (double *)sc.cand_row, *kr = (double *)sc.krow;
            void *args[] = {&d_a, (void *)&ni, (void *)&k0, &kb, &rows, &limit, &d_piv, &st, &sc.ps, &sc.cand_val,
                            &sc.cand_idx, &cr, &kr};
            if (!cuda_ok(cudaLaunchCooperativeKernel((const void *)k_panel_coop<double>, dim3(pl.G), dim3(256), args,
                                                     pl.smem, stream()),
                         "cooperative panel launch"))
                return -1;
            note_launch();
        } else {
            PEEC_LAUNCH(k_panel<double>, 1, 1024, 0, d_a, ni, k0, kb, limit, d_piv, st);
        }
        PEEC_LAUNCH(k_laswp<double>, (ni + kLaswpCols - 1) / kLaswpCols, 256, 2 * NB * kLaswpCols * sizeof(double), d_a,
                    ni, k0, kb, d_piv, st);
        int rest = ni - (k0 + kb);
        if (rest > 0) {
            PEEC_LAUNCH(k_trsm<double>, (rest + 255) / 256, 256, 0, d_a, ni, k0, kb, k0 + kb, ni, st);
            dim3 g((rest + 63) / 64, (rest + 63) / 64);
            PEEC_LAUNCH(k_gemm_real, g, 256, 0, d_a, ni, k0, kb, st);
        }
    }
    PEEC_LAUNCH(k_check_diag<double>, (ni + 255) / 256, 256, 0, d_a, ni, limit, st);
    size_t perm_smem = n * sizeof(int);
    if (perm_smem > 48 * 1024) cudaFuncSetAttribute(k_perm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)perm_smem);
    PEEC_LAUNCH(k_perm, 1, 1024, perm_smem, d_piv, ni, d_perm, st);
    cudaMemcpyAsync(&hs, st, sizeof(Status), cudaMemcpyDeviceToHost, stream());
    if (!launch_ok("LU kernels") || !sync("LU factorisation")) return -1;
    if (hs.code == 6) {
        set_error("LU panel synchronisation timed out");
        return -1;
    }
    if (failed_column) *failed_column = hs.code ? hs.column : -1;
    if (hs.code) {
        report_status(hs, false);
        return -2;
    }
    return 0;
}

extern "C" {

// Turn per-phase timing of the allocating factorisations on (1) or off (0).
void peec_gb300_lu_timing_enable(int on) { g_lu_timing.enabled = on != 0; }

// Phase times of the last timed factorisation (ms) and the algorithmic
// flops of its trailing updates.
int peec_gb300_lu_timing(double *ms_panel, double *ms_swap_trsm, double *ms_update, double *update_flops) {
    if (!g_lu_timing.enabled) return -1;
    if (ms_panel) *ms_panel = g_lu_timing.ms[0];
    if (ms_swap_trsm) *ms_swap_trsm = g_lu_timing.ms[1];
    if (ms_update) *ms_update = g_lu_timing.ms[2] + g_lu_timing.ms[3];
    if (update_flops) *update_flops = g_lu_timing.flops_update;
    return 0;
}

// Of the last timed mixed factorisation: time (ms) and issued BF16 flops of
// the outer-block trailing GEMMs alone (K = 6 x 256; no operand splits).
int peec_gb300_lu_timing_trailing(double *ms, double *issued_flops) {
    if (!g_lu_timing.enabled) return -1;
    if (ms) *ms = g_lu_timing.ms[3];
    if (issued_flops) *issued_flops = g_lu_timing.flops_outer;
    return 0;
}

}  // extern "C"

// =====================================================================
// Mixed precision: FP32 complex LU with a split-BF16x3 tensor-core
// trailing update, then FP64 iterative refinement against the FP64 matrix.
//
//   equilibrate by powers of two (row scales, then column scales of the
//   row-scaled matrix, in integer exponent arithmetic), round to FP32 complex;
//   per block column: cooperative FP32 panel (same pivot rule), row swaps,
//   U12 = L11^-1 A12 in FP32, then split L21 and U12 into BF16 hi/lo parts,
//     A'  = [Lr_h Lr_h Lr_l Li_h Li_h Li_l]            (K' = 6 x 32)
//     Br' = [Ur_h Ur_l Ur_h -Ui_h -Ui_l -Ui_h]
//     Bi' = [Ui_h Ui_l Ui_h  Ur_h  Ur_l  Ur_h]
//   so that one tcgen05 GEMM with two TMEM accumulators gives
//     C -= (Lr Ur - Li Ui) + j (Lr Ui + Li Ur)   to ~2^-16 per product;
//   refinement: x = 0, r = b; repeat { d = LU^-1 r (FP32); x += d;
//     r = b - Z x (FP64); stop when the componentwise backward error
//     max |r_i| / (sum_j |Z_ij||x_j| + |b_i|) <= tol }.
// =====================================================================
namespace peec {

bool tc_gemm_update_cplx(const void *a, const void *br, const void *bi, float *c, int m, int n, int k, int row0,
                         int col0, long long ldc, int *d_err);

// x * 2^-shift rounded to FP32 (nearest, ties to even) by integer operations
// on the bits: no FP64 instruction (one warp-wide FP64 operation costs ~64
// cycles on GB300).  Zero and subnormal inputs and results below 2^-126
// give (signed) zero; results beyond the FP32 range give +-inf; NaN stays NaN.
__device__ __forceinline__ float f64_to_f32_scaled(double x, int shift) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7ff);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    if (ex == 0x7ff) return __uint_as_float(sign | (m ? 0x7fc00000u : 0x7f800000u));
    if (ex == 0) return __uint_as_float(sign);
    int e = ex - 1023 - shift;
    if (e < -126) return __uint_as_float(sign);
    unsigned m23 = (unsigned)(m >> 29);
    const unsigned long long rem = m & 0x1FFFFFFFull;
    if (rem > 0x10000000ull || (rem == 0x10000000ull && (m23 & 1u))) {
        if (++m23 == 0x800000u) {
            m23 = 0;
            ++e;
        }
    }
    if (e > 127) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned)(e + 127) << 23) | m23);
}

// |z| in FP32 for the backward error's denominator sum |Z||x| + |b| (a
// stopping test: FP32 relative error there moves eta by ~1e-7 of itself);
// values beyond the FP32 range clamp to 3e38, which can only shrink the
// denominator, i.e. overstate eta.
__device__ __forceinline__ float abs_f32(cplx z) {
    const float m = hypotf(f64_to_f32_scaled(z.re, 0), f64_to_f32_scaled(z.im, 0));
    return m < 3.0e38f ? m : 3.0e38f;
}

// Equilibration of the mixed path with power-of-two scales, in integer
// exponent arithmetic: R_i = the largest exponent of row i (of max(|re|,
// |im|)), C_j = max_i (E_ij - R_i) <= 0 over column j; the scaled entries
// z 2^-(R_i + C_j) have magnitude < 2 with every column's largest >= 1, and
// the scalings are exact.  Status 4: a non-finite entry; 5: a zero row or
// column (as the FP64 equilibration).
__device__ __forceinline__ int exp_of(double x) { return (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff); }

__global__ void k_eq2_row(const cplx *z, int n, int *er, double *rs, Status *st) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const cplx *row = z + (size_t)warp * n;
    int e = 0;
    for (int j = lane; j < n; j += 32) e = max(e, max(exp_of(row[j].re), exp_of(row[j].im)));
    for (int d = 16; d > 0; d >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, d));
    if (lane == 0) {
        if (e == 0x7ff || e == 0) atomicCAS(&st->code, 0, e ? 4 : 5);
        const int ee = (e == 0x7ff || e == 0) ? 1023 : e;
        er[warp] = ee;
        rs[warp] = __longlong_as_double((long long)ee << 52);  // 2^(R_i)
    }
}

__global__ void __launch_bounds__(256) k_eq2_col(const cplx *z, int n, const int *er, int *ec, double *cs,
                                                 Status *st) {
    __shared__ int part[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane;
    int c = -100000;
    if (j < n)
        for (int i = warp; i < n; i += 8) {
            const cplx v = z[(size_t)i * n + j];
            const int e = max(exp_of(v.re), exp_of(v.im));
            if (e != 0) c = max(c, e - er[i]);
        }
    part[warp][lane] = c;
    __syncthreads();
    if (warp == 0 && j < n) {
        for (int w = 1; w < 8; ++w) c = max(c, part[w][lane]);
        if (c < -1022) {
            atomicCAS(&st->code, 0, 5);
            c = 0;
        }
        ec[j] = c;
        cs[j] = __longlong_as_double((long long)(c + 1023) << 52);  // 2^(C_j)
    }
}

// f = z 2^-(R_i + C_j) in FP32 and |z| in FP32 (the backward error's
// denominator), one pass over Z
__global__ void k_eq2_to_float(const cplx *z, int n, const int *er, const int *ec, cplxf *f, float *absz) {
    const size_t nn = (size_t)n * n;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nn; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / n), j = (int)(t % n);
        const cplx v = z[t];
        const int shift = (er[i] - 1023) + ec[j];
        f[t] = cplxf{f64_to_f32_scaled(v.re, shift), f64_to_f32_scaled(v.im, shift)};
        if (absz) absz[t] = abs_f32(v);
    }
}

// x = h + m (+ l): each part the BF16 rounding of what the earlier parts
// leave (x - h and x - h - m are exact in FP32).
template <int P>
__device__ __forceinline__ void split_parts(float x, __nv_bfloat16 (&v)[P]) {
#pragma unroll
    for (int p = 0; p < P; ++p) {
        v[p] = __float2bfloat16_rn(x);
        x -= __bfloat162float(v[p]);
    }
}

// The products of one split-BF16 real product a b: T = 3 terms (BF16x3,
// two-part operands: h h + h m + m h, about 16 bits) or T = 6 terms (BF16x6,
// three-part operands: h h + h m + m h + h l + m m + l h, the products the
// FP32 rounding of a b keeps).  Term t multiplies part split_pa(t) of a by
// part split_pb(t) of b.
template <int T> struct SplitScheme {
    static constexpr int parts = T == 3 ? 2 : 3;
    static constexpr int planes = 2 * T;  // K = planes x KW
    __host__ __device__ static constexpr int pa(int t) { return t == 2 || t == 4 ? 1 : t == 5 ? 2 : 0; }
    __host__ __device__ static constexpr int pb(int t) { return t == 1 || t == 4 ? 1 : t == 3 ? 2 : 0; }
};

// Split operands of one complex trailing update C -= L U, K = 2 T KW:
// A' row r (0..m-1) <- L[row0 + r][col0 .. col0+kw-1] (zero-padded to KW) as
// 2 T planes KW wide, [re part pa(0) .. re part pa(T-1) | im part pa(0) ..],
// e.g. [re_h | re_h | re_l | im_h | im_h | im_l] for T = 3.
template <int T>
__global__ void k_split_a(const cplxf *a, int n, int row0, int m, int col0, int kw, int KW, __nv_bfloat16 *out) {
    pdl_wait();
    pdl_trigger();
    using S = SplitScheme<T>;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)m * KW) return;
    int r = (int)(t / KW), c = (int)(t % KW);
    cplxf x = c < kw ? a[(size_t)(row0 + r) * n + col0 + c] : cplxf{0.0f, 0.0f};
    __nv_bfloat16 re[S::parts], im[S::parts];
    split_parts(x.re, re);
    split_parts(x.im, im);
    __nv_bfloat16 *row = out + (size_t)r * S::planes * KW;
#pragma unroll
    for (int q = 0; q < T; ++q) {
        row[q * KW + c] = re[S::pa(q)];
        row[(T + q) * KW + c] = im[S::pa(q)];
    }
}

// Br', Bi' row j (0..nc-1) <- U[row0 .. row0+kw-1][col0 + j] as 2 T planes:
// Br' = [re part pb(q) | -im part pb(q)], Bi' = [im part pb(q) | re part pb(q)]
// (q = 0 .. T-1), so that A' Br' = Re(L U) and A' Bi' = Im(L U); for T = 3
// Br' = [re_h | re_l | re_h | -im_h | -im_l | -im_h].
// A 64 (K) x 32 (columns) tile per CTA goes through shared memory: rows of U
// are read along the columns (coalesced), the BF16 parts are kept as
// K-contiguous planes, and the K-major outputs are written as 128-byte
// segments of 16-byte stores.  grid (ceil(nc / 32), ceil(KW / 64)), 256 threads.
static const int kSbK = 64, kSbJ = 32, kSbPad = 72;  // plane row: 72 BF16 = 144 bytes (16-byte aligned)
template <int T>
__global__ void __launch_bounds__(256) k_split_b(const cplxf *a, int n, int row0, int kw, int KW, int col0, int nc,
                                                 __nv_bfloat16 *br, __nv_bfloat16 *bi) {
    pdl_wait();
    pdl_trigger();
    using S = SplitScheme<T>;
    constexpr int NP = S::parts;
    __shared__ __align__(16) __nv_bfloat16 pl[2 * NP][kSbJ][kSbPad];  // re parts, then im parts
    const int t = threadIdx.x, j0 = blockIdx.x * kSbJ, c0 = blockIdx.y * kSbK;
    {
        const int j = t & 31;
        for (int rr = 0; rr < kSbK / 8; ++rr) {
            const int c = rr * 8 + (t >> 5);
            cplxf x = (c0 + c < kw && j0 + j < nc) ? a[(size_t)(row0 + c0 + c) * n + col0 + j0 + j]
                                                   : cplxf{0.0f, 0.0f};
            __nv_bfloat16 re[NP], im[NP];
            split_parts(x.re, re);
            split_parts(x.im, im);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                pl[p][j][c] = re[p];
                pl[NP + p][j][c] = im[p];
            }
        }
    }
    __syncthreads();
    // output segment seg (0 .. 4T-1): br planes 0..2T-1, then bi planes;
    // within 2T planes, the parts pb(q) of the first then the second component
    for (int q = t; q < 2 * S::planes * kSbJ * (kSbK / 8); q += blockDim.x) {
        const int e = q & 7, j = (q >> 3) & (kSbJ - 1), seg = q >> 8;
        const int c = c0 + 8 * e;
        if (j0 + j >= nc || c >= KW) continue;
        const bool is_bi = seg >= S::planes;
        const int p = seg % S::planes, second = p / T, part = S::pb(p % T);
        const int imag = is_bi ? 1 - second : second;
        uint4 v = *reinterpret_cast<const uint4 *>(&pl[NP * imag + part][j][8 * e]);
        const unsigned m = (!is_bi && second) ? 0x80008000u : 0u;
        v.x ^= m;
        v.y ^= m;
        v.z ^= m;
        v.w ^= m;
        __nv_bfloat16 *out = (is_bi ? bi : br) + (size_t)(j0 + j) * S::planes * KW + p * KW + c;
        *reinterpret_cast<uint4 *>(out) = v;
    }
}

// N = I - L^-1 for the unit lower triangle L = a[K0 + i][K0 + k] (i, k < kw,
// kw <= 256), FP32 complex, row-major kw x kw; N is strictly lower.
// Blocked in 32 x 32 blocks: CTA (jb, g) computes the columns 32 jb + 8 g ..
// +7 of X = L^-1.  Phase 1: warp w inverts the diagonal block D = L_ii^-1,
// i = jb + w (one lane per column, forward substitution in registers).
// Phase 2, block rows i = jb+1 ..: X_i = -D_i sum_{k<i} L_ik X_k (the sum in
// shared memory, one output per thread).  grid (ceil(kw / 32), 4), 256
// threads, dynamic shared memory k_lower_inv_smem().
static const int kLiPad = 33, kLiX = 9, kLiRow = 225;
static constexpr size_t k_lower_inv_smem() {
    return sizeof(cplxf) * ((size_t)8 * 32 * kLiPad + 256 * kLiX + 32 * kLiRow + 32 * kLiX);
}
__global__ void __launch_bounds__(256) k_lower_inv(const cplxf *a, int n, int K0, int kw, cplxf *N) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(16) unsigned char li_smem[];
    cplxf *blk = reinterpret_cast<cplxf *>(li_smem);  // [8][32][kLiPad]: L_ii, then L_ii^-1
    cplxf *X = blk + 8 * 32 * kLiPad;                 // [256][kLiX]: rows 32 jb.., this CTA's 8 columns
    cplxf *Lr = X + 256 * kLiX;                       // [32][kLiRow]: L_i,jb..i-1
    cplxf *S = Lr + 32 * kLiRow;                      // [32][kLiX]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int jb = blockIdx.x, g = blockIdx.y, nb = (kw + 31) / 32;
    // phase 1: diagonal block inverses (rows past kw: identity)
    {
        const int i = jb + warp;
        if (i < nb) {
            cplxf *B = blk + warp * 32 * kLiPad;
            for (int r = 0; r < 32; ++r) {
                const int gr = 32 * i + r, gq = 32 * i + lane;
                B[r * kLiPad + lane] = (lane < r && gr < kw) ? a[(size_t)(K0 + gr) * n + K0 + gq] : cplxf{0.0f, 0.0f};
            }
            __syncwarp();
            cplxf d[32];
#pragma unroll
            for (int r = 0; r < 32; ++r) {
                cplxf s = {r == lane ? 1.0f : 0.0f, 0.0f};
#pragma unroll
                for (int q = 0; q < r; ++q) {
                    const cplxf l = B[r * kLiPad + q];
                    s.re = fmaf(-l.re, d[q].re, s.re);
                    s.re = fmaf(l.im, d[q].im, s.re);
                    s.im = fmaf(-l.re, d[q].im, s.im);
                    s.im = fmaf(-l.im, d[q].re, s.im);
                }
                d[r] = r >= lane ? s : cplxf{0.0f, 0.0f};
            }
            __syncwarp();
#pragma unroll
            for (int r = 0; r < 32; ++r) B[r * kLiPad + lane] = d[r];
        }
    }
    __syncthreads();
    const int r = tid >> 3, cc = tid & 7;
    X[r * kLiX + cc] = blk[r * kLiPad + 8 * g + cc];  // X_jb = columns of D_jb
    for (int i = jb + 1; i < nb; ++i) {
        const int len = 32 * (i - jb);
        for (int q = tid; q < 32 * len; q += blockDim.x) {
            const int rr = q / len, qq = q % len, gr = 32 * i + rr;
            Lr[rr * kLiRow + qq] = gr < kw ? a[(size_t)(K0 + gr) * n + K0 + 32 * jb + qq] : cplxf{0.0f, 0.0f};
        }
        __syncthreads();
        cplxf s0 = {0.0f, 0.0f}, s1 = {0.0f, 0.0f};
        for (int q = 0; q < len; q += 2) {
            s0 = mac(s0, Lr[r * kLiRow + q], X[q * kLiX + cc]);
            s1 = mac(s1, Lr[r * kLiRow + q + 1], X[(q + 1) * kLiX + cc]);
        }
        S[r * kLiX + cc] = cplxf{s0.re + s1.re, s0.im + s1.im};
        __syncthreads();
        const cplxf *D = blk + (i - jb) * 32 * kLiPad;
        cplxf x = {0.0f, 0.0f};
        for (int q = 0; q < 32; ++q) x = mac(x, D[r * kLiPad + q], S[q * kLiX + cc]);
        X[(len + r) * kLiX + cc] = cplxf{-x.re, -x.im};
        __syncthreads();
    }
    // N[row][col] = -X for row > col, 0 otherwise (rows above the block: 0)
    const int col = 32 * jb + 8 * g + cc;
    if (col >= kw) return;
    for (int row = r; row < kw; row += 32) {
        cplxf v = {0.0f, 0.0f};
        if (row > col) {
            const cplxf xv = X[(row - 32 * jb) * kLiX + cc];
            v = cplxf{-xv.re, -xv.im};
        }
        N[(size_t)row * kw + col] = v;
    }
}

// y = P D_r^-1 r in FP32 (the permuted, row-scaled residual)
__global__ void k_mix_rhs(const cplx *r, const int *perm, const double *rs, int n, int nrhs, cplxf *y,
                          const int *skip) {
    if (skip && *skip) return;
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)n * nrhs) return;
    int q = (int)(t / n), i = (int)(t % n), src = perm[i];
    cplx v = r[(size_t)q * n + src];
    double s = rs[src];
    y[t] = cplxf{(float)(v.re / s), (float)(v.im / s)};
}

__global__ void k_abs_matrix(const cplx *Z, size_t count, float *out) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
        out[t] = abs_f32(Z[t]);
}

// x += D_c^-1 y  (FP64 accumulation of the FP32 correction)
__global__ void k_mix_update(cplx *x, const cplxf *y, const double *cs, int n, int nrhs, float *absx,
                             const int *skip) {
    if (skip && *skip) return;
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)n * nrhs) return;
    int i = (int)(t % n);
    double s = cs[i];
    cplx v = x[t];
    v.re += (double)y[t].re / s;
    v.im += (double)y[t].im / s;
    x[t] = v;
    absx[t] = abs_f32(v);
}

// r = b - Z x in FP64 (one warp per row and right-hand side) and the
// componentwise backward error |r_i| / (sum_j |Z_ij||x_j| + |b_i|), the
// denominator from FP32 magnitudes, max-reduced as IEEE bits.
__global__ void k_residual(const cplx *Z, const float *absZ, const cplx *x, const float *absx, const cplx *b, int n,
                           int nrhs, cplx *r, unsigned long long *be, const int *skip) {
    if (skip && *skip) return;
    long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= (long long)n * nrhs) return;
    int q = (int)(warp / n), i = (int)(warp % n);
    const cplx *row = Z + (size_t)i * n, *xr = x + (size_t)q * n;
    const float *arow = absZ + (size_t)i * n, *ax = absx + (size_t)q * n;
    double yr = 0.0, yi = 0.0;
    float den = 0.0f;
    for (int j = lane; j < n; j += 32) {
        cplx z = row[j], v = xr[j];
        yr = fma(z.re, v.re, yr);
        yr = fma(-z.im, v.im, yr);
        yi = fma(z.re, v.im, yi);
        yi = fma(z.im, v.re, yi);
        den = fmaf(arow[j], ax[j], den);
    }
    yr = warp_sum(yr);
    yi = warp_sum(yi);
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) den += __shfl_xor_sync(0xffffffffu, den, m);
    if (lane == 0) {
        cplx bi = b[(size_t)q * n + i];
        cplx ri = cplx{bi.re - yr, bi.im - yi};
        r[(size_t)q * n + i] = ri;
        double res = sqrt(fma(ri.re, ri.re, ri.im * ri.im)), babs = hypot(bi.re, bi.im);
        double d = (double)den + babs;
        double eta = d > 0.0 ? res / d : res;
        if (!isfinite(eta)) eta = INFINITY;
        atomicMax(be, (unsigned long long)__double_as_longlong(eta));
    }
}

// A graph sweep's convergence flag: *done = (backward error <= tol); the
// backward error accumulator is zeroed for the next residual unless done.
__global__ void k_sweep_done(const unsigned long long *be, double tol, int *done) {
    if (*done) return;
    double eta;
    memcpy(&eta, be, sizeof(eta));
    *done = eta <= tol;
}
__global__ void k_zero_unless_done(unsigned long long *be, const int *done) {
    if (!*done) *be = 0ull;
}

__global__ void k_abs_x(const cplx *x, size_t count, float *absx) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t < count) absx[t] = abs_f32(x[t]);
}

__global__ void k_add_cplx(cplx *x, const cplx *dx, size_t count) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    x[t].re += dx[t].re;
    x[t].im += dx[t].im;
}

// ---- FGMRES-IR: flexible GMRES on D_r^-1 Z d = D_r^-1 r, preconditioned by
// the FP32 factor applied in FP32 (Arioli and Duff, "Using FGMRES to obtain
// backward stability in mixed precision", ETNA 33, 2009) ----

// The right-hand sides of one FGMRES chunk run in lockstep: every vector
// argument below is nq column blocks of n (block q at offset q n), nq <=
// kGmresChunk, and each block sees the arithmetic of a solve of its own.
static const int kGmresChunk = 8;
struct GmresScalars {
    double v[kGmresChunk];
};
struct GmresCounts {
    int v[kGmresChunk];
};

// y_q = D_r^-1 Z v_q in FP64, one warp per row (Z read once for all q)
__global__ void k_zmv_scaled(const cplx *Z, const cplx *v, const double *rs, int n, int nq, cplx *y) {
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const cplx *row = Z + (size_t)warp * n;
    double yr[kGmresChunk], yi[kGmresChunk];
#pragma unroll
    for (int q = 0; q < kGmresChunk; ++q) yr[q] = yi[q] = 0.0;
    for (int j = lane; j < n; j += 32) {
        const cplx z = row[j];
#pragma unroll
        for (int q = 0; q < kGmresChunk; ++q) {
            if (q >= nq) break;
            const cplx u = v[(size_t)q * n + j];
            yr[q] = fma(z.re, u.re, yr[q]);
            yr[q] = fma(-z.im, u.im, yr[q]);
            yi[q] = fma(z.re, u.im, yi[q]);
            yi[q] = fma(z.im, u.re, yi[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < kGmresChunk; ++q) {
        if (q >= nq) break;
        const double a = warp_sum(yr[q]), c = warp_sum(yi[q]);
        if (lane == 0) y[(size_t)q * n + warp] = cplx{a / rs[warp], c / rs[warp]};
    }
}

// y_q = P v_q rounded to FP32 (v already row-scaled); grid.y = q
__global__ void k_perm_f32(const cplx *v, const int *perm, int n, cplxf *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t o = (size_t)blockIdx.y * n;
    const cplx u = v[o + perm[i]];
    y[o + i] = cplxf{(float)u.re, (float)u.im};
}

// v = D_r^-1 r
__global__ void k_scale_rows(const cplx *r, const double *rs, int n, cplx *v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = cplx{r[i].re / rs[i], r[i].im / rs[i]};
}

// w_q = D_c^-1 y_q: the FP32 correction solve's result in FP64; grid.y = q
__global__ void k_mix_out(const cplxf *y, const double *cs, int n, cplx *w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t o = (size_t)blockIdx.y * n;
    w[o + i] = cplx{(double)y[o + i].re / cs[i], (double)y[o + i].im / cs[i]};
}

// h_q[j] = v_{j,q}^H w_q for j < k (basis vector j of block q at V + (j nq +
// q) n), one CTA per (j, q), a fixed reduction order; h_q at h + q ld
__global__ void __launch_bounds__(256) k_gs_dots(const cplx *V, int n, int nq, const cplx *w, cplx *h, int ld) {
    __shared__ double sr[8], si[8];
    const int q = blockIdx.y;
    const cplx *v = V + ((size_t)blockIdx.x * nq + q) * n, *wq = w + (size_t)q * n;
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) {
        const cplx a = v[i], b = wq[i];
        re = fma(a.re, b.re, re);
        re = fma(a.im, b.im, re);
        im = fma(a.re, b.im, im);
        im = fma(-a.im, b.re, im);
    }
    re = warp_sum(re);
    im = warp_sum(im);
    if ((threadIdx.x & 31) == 0) {
        sr[threadIdx.x >> 5] = re;
        si[threadIdx.x >> 5] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int t = 0; t < 8; ++t) {
            a += sr[t];
            b += si[t];
        }
        h[(size_t)q * ld + blockIdx.x] = cplx{a, b};
    }
}

// w_q -= sum_{j<k} h_q[j] v_{j,q}; grid.y = q
__global__ void k_gs_update(const cplx *V, int n, int nq, int k, const cplx *h, int ld, cplx *w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int q = blockIdx.y;
    const cplx *hq = h + (size_t)q * ld;
    cplx s = w[(size_t)q * n + i];
    for (int j = 0; j < k; ++j) {
        const cplx hj = hq[j], v = V[((size_t)j * nq + q) * n + i];
        s.re -= hj.re * v.re - hj.im * v.im;
        s.im -= hj.re * v.im + hj.im * v.re;
    }
    w[(size_t)q * n + i] = s;
}

// out[q] = ||w_q||_2, one CTA of 1024 threads per q
__global__ void __launch_bounds__(1024) k_norm2(const cplx *w, int n, double *out) {
    __shared__ double part[32];
    const cplx *wq = w + (size_t)blockIdx.x * n;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 1024) s = fma(wq[i].re, wq[i].re, fma(wq[i].im, wq[i].im, s));
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < 32; ++q) t += part[q];
        out[blockIdx.x] = sqrt(t);
    }
}

// v_q = w_q * scale_q; grid.y = q
__global__ void k_cscale(const cplx *w, int n, GmresScalars scale, cplx *v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t o = (size_t)blockIdx.y * n;
    const double sc = scale.v[blockIdx.y];
    v[o + i] = cplx{w[o + i].re * sc, w[o + i].im * sc};
}

// x_q += sum_{j<k_q} y_q[j] z_{j,q} (z_{j,q} at Zk + (j nq + q) n, y_q at y + q
// ld); grid.y = q
__global__ void k_gmres_update(const cplx *Zk, int n, int nq, GmresCounts k, const cplx *y, int ld, cplx *x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int q = blockIdx.y;
    const cplx *yq = y + (size_t)q * ld;
    cplx s = x[(size_t)q * n + i];
    for (int j = 0; j < k.v[q]; ++j) {
        const cplx a = yq[j], v = Zk[((size_t)j * nq + q) * n + i];
        s.re += a.re * v.re - a.im * v.im;
        s.im += a.re * v.im + a.im * v.re;
    }
    x[(size_t)q * n + i] = s;
}

struct MixedTiming {
    double ms_prepare = 0, ms_factor = 0, ms_refine = 0;
    int iterations = 0, split_terms = 3, gmres_iterations = 0;
};
static thread_local MixedTiming g_mixed_timing;  // last mixed solve of this host thread

}  // namespace peec

// FP64 iterative refinement of a solution from an FP64 complex factor of Z
// (peec_gb300_complex_lu_factor_device): r = b - Z x, x += LU^-1 r until the
// componentwise backward error <= tol.  Returns 0 when reached, 1 when not
// after max_iter corrections (x holds the last iterate), -1 on errors.
extern "C" int peec_gb300_complex_refine_device(const Complex *d_Z, const Complex *d_lu, const int *d_perm,
                                                const double *d_row_scale, const double *d_column_scale, size_t n_,
                                                const Complex *d_b, Complex *d_x, size_t nrhs_, double tol,
                                                int max_iter, double *backward_error, int *iterations) {
    using namespace peec;
    if (!d_Z || !d_lu || !d_perm || !d_row_scale || !d_column_scale || !d_b || !d_x || n_ == 0 || nrhs_ == 0 ||
        n_ > (size_t)0x7fffffff || max_iter < 0)
        return -1;
    const int n = (int)n_, nrhs = (int)nrhs_;
    const size_t nn = n_ * n_, nv = n_ * nrhs_;
    const cplx *Z = (const cplx *)d_Z;
    cplx *x = (cplx *)d_x;
    DBuf<float> absZ(nn), absx(nv);
    DBuf<cplx> r(nv), dx(nv);
    DBuf<unsigned long long> be(1);
    if (!absZ.p || !absx.p || !r.p || !dx.p || !be.p) return -1;
    PEEC_LAUNCH(k_abs_matrix, 152 * 8, 256, 0, Z, nn, absZ.p);
    double eta = INFINITY;
    int it = 0;
    for (;; ++it) {
        cudaMemsetAsync(be.p, 0, sizeof(unsigned long long), stream());
        PEEC_LAUNCH(k_abs_x, (unsigned)((nv + 255) / 256), 256, 0, x, nv, absx.p);
        PEEC_LAUNCH(k_residual, (unsigned)((nv * 32 + 255) / 256), 256, 0, Z, absZ.p, x, absx.p, (const cplx *)d_b, n,
                    nrhs, r.p, be.p, (const int *)nullptr);
        unsigned long long hb = 0;
        cudaMemcpyAsync(&hb, be.p, sizeof(hb), cudaMemcpyDeviceToHost, stream());
        if (!launch_ok("refinement") || !sync("refinement")) return -1;
        memcpy(&eta, &hb, sizeof(eta));
        if (eta <= tol || it >= max_iter) break;
        if (!solve_device<cplx>((const cplx *)d_lu, d_perm, d_row_scale, d_column_scale, n, r.p, dx.p, nrhs))
            return -1;
        PEEC_LAUNCH(k_add_cplx, (unsigned)((nv + 255) / 256), 256, 0, x, dx.p, nv);
    }
    if (backward_error) *backward_error = eta;
    if (iterations) *iterations = it;
    return eta <= tol ? 0 : 1;
}

namespace peec {

__global__ void k_capture_status(const Status *st, const int *werr, const unsigned long long *be,
                                 unsigned long long *eta_out, int *status_out) {
    *status_out = st->code ? st->code : (*werr ? 6 : 0);
    *eta_out = *be;
}

bool mrhs_split_z(const void *Z, size_t count, void *Zs);
bool mrhs_sweep(const void *Zs, const void *lu, const int *perm, const double *rs, const double *cs, int n, int nrhs,
                const void *b, void *x, void *r, void *Y, void *xs, unsigned long long *be, unsigned long long *be_q,
                int *done, double tol);
// from this many right-hand sides on, the refinement sweeps use the blocked
// many-right-hand-side form (multirhs.cu) instead of the wavefront solve
// (NR right-hand sides per pass) and the per-row residual
static const int kManyRhs = 32;

int mixed_solve_impl(const Complex *d_Z, size_t n_, const Complex *d_b, Complex *d_x, size_t nrhs_, double tol,
                     int max_iter, double *backward_error, int *iterations, const MixedCapture *cap) {
    if (!d_Z || !d_b || !d_x || n_ == 0 || nrhs_ == 0 || n_ > (size_t)0x7fffffff || max_iter < 1) return -1;
    const int n = (int)n_, nrhs = (int)nrhs_;
    const size_t nn = n_ * n_, nv = n_ * nrhs_;
    const cplx *Z = (const cplx *)d_Z;
    const cplx *b = (const cplx *)d_b;
    cplx *x = (cplx *)d_x;
    DBuf<cplxf> f(nn), y(nv);
    DBuf<cplx> r(nv);
    DBuf<double> rs(n), cs(n);
    DBuf<long long> piv(n);
    DBuf<int> perm(n), err(1);
    DBuf<Status> st(1);
    DBuf<unsigned long long> mx(1), be(1);
    // two-level blocking: 32-column panels inside 256-column outer blocks, so
    // the bulk of the trailing update runs with K = 6 x 256 on the tensor cores
    const int OB = 256;
    DBuf<__nv_bfloat16> ap((size_t)n * 12 * OB), bpr((size_t)n * 12 * OB), bpi((size_t)n * 12 * OB);
    DBuf<cplxf> linv((size_t)OB * OB);  // I - L11^-1 of one outer block
    DBuf<unsigned char> scratch;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t G = (size_t)sms;
    size_t sbytes = 256 + 2 * G * 8 + 2 * G * 4 + 16 + 2 * G * NB * sizeof(cplxf) + 2 * NB * sizeof(cplxf) + 64;
    // lean panel slots: G_lean = ceil(n / 64) CTAs at most
    const size_t GL = (size_t)(n + kLeanThreads - 1) / kLeanThreads;
    const int lean_stride = (int)((GL + 63) / 64 * 64);  // flags of one parity, a multiple of 64 (16-byte loads)
    DBuf<unsigned long long> lean_flag(2 * (size_t)lean_stride);
    DBuf<int> lean_idx(2 * GL);
    DBuf<cplxf> lean_rows(2 * GL * NB + 2 * NB);
    if (!f.p || !y.p || !r.p || !rs.p || !cs.p || !piv.p || !perm.p || !err.p || !st.p || !mx.p || !be.p || !ap.p ||
        !bpr.p || !bpi.p || !linv.p || !scratch.alloc(sbytes) ||
        !lean_flag.p || !lean_idx.p || !lean_rows.p)
        return -1;
    cudaMemsetAsync(lean_flag.p, 0, lean_flag.n * sizeof(unsigned long long), stream());
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    if (!cap) {
        for (auto &e : ev) cudaEventCreate(&e);
        cudaEventRecord(ev[0], stream());
    }
    cudaMemsetAsync(scratch.p, 0, sbytes, stream());
    cudaMemsetAsync(st.p, 0, sizeof(Status), stream());
    cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), stream());
    cudaMemsetAsync(err.p, 0, sizeof(int), stream());
    PanelScratch sc;
    {
        unsigned char *bb = scratch.p;
        sc.ps = (PanelSlots *)bb;
        sc.cand_val = (double *)(bb + 256);
        sc.cand_idx = (int *)(bb + 256 + 2 * G * 8);
        size_t off = (256 + 2 * G * 8 + 2 * G * 4 + 15) & ~(size_t)15;
        sc.cand_row = bb + off;
        sc.krow = bb + off + 2 * G * NB * sizeof(cplxf);
    }
    // equilibrate by powers of two, round to FP32; |Z| in FP32 in the same pass
    DBuf<int> er(n), ec(n);
    DBuf<float> absZ(nn);
    if (!er.p || !ec.p || !absZ.p) return -1;
    PEEC_LAUNCH(k_eq2_row, (unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, Z, n, er.p, rs.p, st.p);
    PEEC_LAUNCH(k_eq2_col, (n + 31) / 32, 256, 0, Z, n, er.p, ec.p, cs.p, st.p);
    PEEC_LAUNCH(k_eq2_to_float, 152 * 16, 256, 0, Z, n, er.p, ec.p, f.p, absZ.p);
    PEEC_LAUNCH(k_max_mag<cplxf>, 152 * 8, 256, 0, f.p, nn, mx.p);
    unsigned long long bits = 0;
    Status hs;
    double scale = 1.0;
    if (!cap) {
        cudaMemcpyAsync(&bits, mx.p, sizeof(bits), cudaMemcpyDeviceToHost, stream());
        cudaMemcpyAsync(&hs, st.p, sizeof(hs), cudaMemcpyDeviceToHost, stream());
        if (!sync("mixed equilibration")) return -1;
        if (hs.code != 0) return -2;
        memcpy(&scale, &bits, sizeof(scale));
        if (!isfinite(scale) || scale <= 0.0) return -2;
        cudaEventRecord(ev[1], stream());
    }
    const double limit = 1e-14 * scale;
    cplxf *a = f.p;
    LuTiming &tm = g_lu_timing;
    // split-BF16 terms of the trailing update products: BF16x3 first (about
    // 16 bits), BF16x6 (FP32-equivalent) when refinement from the BF16x3
    // factor stalls; PEEC_GB300_MIXED_SPLIT=6 starts with BF16x6
    // (many right-hand sides: BF16x6 from the start -- the factorisation is
    // a small part of such a solve, every refinement sweep reads Z for all
    // right-hand sides, and the BF16x6 factor needs fewer sweeps)
    int T = cap ? cap->split_terms : (nrhs >= kManyRhs ? 6 : mixed_split_terms());
    // FP32 factorisation of f, trailing updates on the tensor cores: 0, -2 on
    // a pivot breakdown, -1 on errors
    auto factor = [&]() -> int {
        if (tm.enabled) tm.reset();
        // C[row0.., col0..] -= L[row0.., kc..kc+kw) U[kc..kc+kw, col0..), split-BF16 with T terms
        // (the L operand may come from another matrix: lsrc with leading dimension
        // ld, its rows lrow0.., columns lcol0..)
        auto tc_update_from = [&](const cplxf *lsrc, int ld, int lrow0, int lcol0, int row0, int m, int col0, int nc,
                                  int kc, int kw) -> bool {
            if (m <= 0 || nc <= 0) return true;
            const int KW = (kw + 31) / 32 * 32;
            if (T == 6)
                pdl_launch(k_split_a<6>, dim3((unsigned)(((long long)m * KW + 255) / 256)), dim3(256), 0, lsrc, ld, lrow0, m, lcol0, kw, KW,
                        ap.p);
            else
                pdl_launch(k_split_a<3>, dim3((unsigned)(((long long)m * KW + 255) / 256)), dim3(256), 0, lsrc, ld, lrow0, m, lcol0, kw, KW,
                        ap.p);
            if (T == 6)
                pdl_launch(k_split_b<6>, dim3((nc + kSbJ - 1) / kSbJ, (KW + kSbK - 1) / kSbK), dim3(256), 0, a, n, kc, kw, KW, col0, nc,
                        bpr.p, bpi.p);
            else
                pdl_launch(k_split_b<3>, dim3((nc + kSbJ - 1) / kSbJ, (KW + kSbK - 1) / kSbK), dim3(256), 0, a, n, kc, kw, KW, col0, nc,
                        bpr.p, bpi.p);
            if (tm.enabled) tm.flops_update += 2.0 * 2.0 * (double)m * nc * (2.0 * T * KW);  // issued BF16 tensor flops
            return tc_gemm_update_cplx(ap.p, bpr.p, bpi.p, (float *)a, m, nc, 2 * T * KW, row0, col0, n, err.p);
        };
        auto tc_update = [&](int row0, int m, int col0, int nc, int kc, int kw, bool outer = false) -> bool {
            if (m <= 0 || nc <= 0) return true;
            const int KW = (kw + 31) / 32 * 32;
            if (T == 6)
                pdl_launch(k_split_a<6>, dim3((unsigned)(((long long)m * KW + 255) / 256)), dim3(256), 0, a, n, row0, m, kc, kw, KW, ap.p);
            else
                pdl_launch(k_split_a<3>, dim3((unsigned)(((long long)m * KW + 255) / 256)), dim3(256), 0, a, n, row0, m, kc, kw, KW, ap.p);
            if (T == 6)
                pdl_launch(k_split_b<6>, dim3((nc + kSbJ - 1) / kSbJ, (KW + kSbK - 1) / kSbK), dim3(256), 0, a, n, kc, kw, KW, col0, nc,
                        bpr.p, bpi.p);
            else
                pdl_launch(k_split_b<3>, dim3((nc + kSbJ - 1) / kSbJ, (KW + kSbK - 1) / kSbK), dim3(256), 0, a, n, kc, kw, KW, col0, nc,
                        bpr.p, bpi.p);
            if (tm.enabled) tm.flops_update += 2.0 * 2.0 * (double)m * nc * (2.0 * T * KW);  // issued BF16 tensor flops
            if (!outer) return tc_gemm_update_cplx(ap.p, bpr.p, bpi.p, (float *)a, m, nc, 2 * T * KW, row0, col0, n, err.p);
            tm.mark(2);
            if (tm.enabled) tm.flops_outer += 2.0 * 2.0 * (double)m * nc * (2.0 * T * KW);
            const bool ok = tc_gemm_update_cplx(ap.p, bpr.p, bpi.p, (float *)a, m, nc, 2 * T * KW, row0, col0, n, err.p);
            tm.mark(3);
            return ok;
        };
        for (int K0 = 0; K0 < n; K0 += OB) {
            const int E = std::min(n, K0 + OB);  // the outer block is columns [K0, E)
            for (int k0 = K0; k0 < E; k0 += NB) {
                const int kb = std::min(NB, E - k0);
                tm.mark(2);
                CoopPlan<cplxf> pl = coop_plan<cplxf>(n - k0);
                const int lean_g = lean_panel_ctas(n - k0);
                if (cl_panel_enabled() && launch_cl_panel(a, n, k0, kb, limit, piv.p, st.p)) {
                } else if (lean_g > 0) {
                    Status *stp = st.p;
                    long long *pivp = piv.p;
                    int kbv = kb;
                    unsigned long long *fl = lean_flag.p;
                    int *li = lean_idx.p;
                    cplxf *lr = lean_rows.p, *lk = lean_rows.p + 2 * GL * NB;
                    int fls = lean_stride;
                    void *args[] = {&a, (void *)&n, (void *)&k0, &kbv, (void *)&limit, &pivp, &stp, &sc.ps, &fl, &fls, &li,
                                    &lr, &lk};
                    if (!cuda_ok(cudaLaunchCooperativeKernel((const void *)k_panel_lean, dim3(lean_g), dim3(kLeanThreads),
                                                             args, 0, stream()),
                                 "lean panel launch"))
                        return -1;
                    note_launch();
                } else if (pl.G > 0) {
                    int rows = pl.rows;
                    cplxf *cr = (cplxf *)sc.cand_row, *kr = (cplxf *)sc.krow;
                    Status *stp = st.p;
                    long long *pivp = piv.p;
                    int kbv = kb;
                    void *args[] = {&a, (void *)&n, (void *)&k0, &kbv, &rows, (void *)&limit, &pivp, &stp, &sc.ps,
                                    &sc.cand_val, &sc.cand_idx, &cr, &kr};
                    if (!cuda_ok(cudaLaunchCooperativeKernel((const void *)k_panel_coop<cplxf>, dim3(pl.G), dim3(256),
                                                             args, pl.smem, stream()),
                                 "cooperative panel launch"))
                        return -1;
                    note_launch();
                } else {
                    PEEC_LAUNCH(k_panel<cplxf>, 1, 1024, 0, a, n, k0, kb, limit, piv.p, st.p);
                }
                tm.mark(0);
                pdl_launch(k_laswp<cplxf>, dim3((n + kLaswpCols - 1) / kLaswpCols), dim3(256),
                           2 * NB * kLaswpCols * sizeof(cplxf), a, n, k0, kb, (const long long *)piv.p,
                           (const Status *)st.p);
                // the rest of the outer block's columns: U12 rows, then the narrow update
                const int rin = E - (k0 + kb);
                if (rin > 0)
                    pdl_launch(k_trsm<cplxf>, dim3((rin + 255) / 256), dim3(256), 0, a, n, k0, kb, k0 + kb, E,
                               (const Status *)st.p);
                tm.mark(1);
                if (!tc_update(k0 + kb, n - (k0 + kb), k0 + kb, rin, k0, kb)) return -1;
            }
            if (E < n) {
                // U12 of the outer block for the columns right of it in one
                // tensor-core update: U12 = L11^-1 A12 = A12 - (I - L11^-1) A12
                const int kw = E - K0;
                static const cudaError_t li_attr = cudaFuncSetAttribute(
                    k_lower_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k_lower_inv_smem());
                if (!cuda_ok(li_attr, "lower-inverse smem attribute")) return -1;
                pdl_launch(k_lower_inv, dim3((kw + 31) / 32, 4), dim3(256), k_lower_inv_smem(), (const cplxf *)a, n, K0,
                           kw, linv.p);
                tm.mark(1);
                if (!tc_update_from(linv.p, kw, 0, 0, K0, kw, E, n - E, K0, kw)) return -1;
                tm.mark(2);
                // trailing update with K = 6 x (E - K0)
                if (!tc_update(E, n - E, E, n - E, K0, E - K0, true)) return -1;
            }
        }
        tm.mark(2);
        tm.finish();
        PEEC_LAUNCH(k_check_diag<cplxf>, (n + 255) / 256, 256, 0, a, n, limit, st.p);
        size_t perm_smem = n_ * sizeof(int);
        if (perm_smem > 48 * 1024) cudaFuncSetAttribute(k_perm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)perm_smem);
        PEEC_LAUNCH(k_perm, 1, 1024, perm_smem, piv.p, n, perm.p, st.p);
        if (cap) return launch_ok("mixed factorisation") ? 0 : -1;
        int herr = 0;
        cudaMemcpyAsync(&hs, st.p, sizeof(hs), cudaMemcpyDeviceToHost, stream());
        cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
        if (!launch_ok("mixed factorisation") || !sync("mixed factorisation")) return -1;
        if (herr) {
            set_error("tcgen05 trailing update: a pipeline wait timed out");
            return -1;
        }
        if (hs.code == 6) {
            set_error("LU panel synchronisation timed out");
            return -1;
        }
        if (hs.code != 0) return -2;
        return 0;
    };
    // FP64 iterative refinement from x = 0: 0 at the gate; 1 when max_iter
    // sweeps end or the refinement stalls (a backward error that is not
    // finite, or a smallest backward error so far that is not a factor 4
    // below the smallest three sweeps earlier with BF16x3 -- the BF16x6
    // factor is the better choice then -- or a factor 2 below the smallest
    // six sweeps earlier with BF16x6); -1 on errors
    DBuf<unsigned> wflags(wave_flag_count<cplxf>(n, nrhs));
    DBuf<int> werr(1), done(1);  // done: a graph sweep converged (later sweeps are no-ops)
    DBuf<cplxf> wdinv(wave_dinv_count(n));
    DBuf<float> absx(nv);
    if (!wflags.p || !werr.p || !wdinv.p || !absx.p) return -1;
    // many right-hand sides: Z and x as float pairs for the double-float residual
    const bool many = nrhs >= kManyRhs;
    DBuf<float4> zsp(many ? nn : 0), xsp(many ? nv : 0);
    DBuf<unsigned long long> be_q(many ? nrhs_ : 0);  // per right-hand side backward errors
    DBuf<int> rhs_done(many ? nrhs_ : 0);             // right-hand sides at the gate
    if (many && (!zsp.p || !xsp.p || !be_q.p || !rhs_done.p)) return -1;
    double eta = INFINITY;
    int total_it = 0;
    auto refine = [&]() -> int {
        PhaseTrace tr;
        cudaMemsetAsync(x, 0, nv * sizeof(cplx), stream());
        cudaMemcpyAsync(r.p, b, nv * sizeof(cplx), cudaMemcpyDeviceToDevice, stream());
        cudaMemsetAsync(werr.p, 0, sizeof(int), stream());
        if (!wave_prepare(a, n, wdinv.p, true)) return -1;
        if (many && !mrhs_split_z(Z, nn, zsp.p)) return -1;
        if (many) cudaMemsetAsync(rhs_done.p, 0, nrhs_ * sizeof(int), stream());
        if (!cap) tr.mark("refine: set-up");
        // one refinement sweep (FP32 correction solve, FP64 update, FP64
        // residual + backward error): captured once as a CUDA graph and
        // replayed per iteration
        auto sweep = [&]() {
            if (many) {
                // many right-hand sides: blocked substitution with GEMM updates
                // and the residual in GEMM form (multirhs.cu)
                cudaMemsetAsync(be.p, 0, sizeof(unsigned long long), stream());
                mrhs_sweep(zsp.p, a, perm.p, rs.p, cs.p, n, nrhs, b, x, r.p, y.p, xsp.p, be.p, be_q.p, rhs_done.p,
                           tol);
                return;
            }
            const int *skip = cap ? done.p : nullptr;
            PEEC_LAUNCH(k_mix_rhs, (unsigned)((nv + 255) / 256), 256, 0, r.p, perm.p, rs.p, n, nrhs, y.p, skip);
            WaveArgs<cplxf> W{};
            W.skip = skip;
            W.lu = a;
            W.dinv = wdinv.p;
            W.n = n;
            W.nrhs = nrhs;
            W.b = y.p;  // already permuted and row-scaled by k_mix_rhs
            W.x = y.p;
            W.flags = wflags.p;
            W.error = werr.p;
            W.subst = 1;  // backward stable for ill-conditioned diagonal blocks of the FP32 factor
            wave_solve(W);
            PEEC_LAUNCH(k_mix_update, (unsigned)((nv + 255) / 256), 256, 0, x, y.p, cs.p, n, nrhs, absx.p, skip);
            if (cap)
                PEEC_LAUNCH(k_zero_unless_done, 1, 1, 0, be.p, (const int *)done.p);
            else
                cudaMemsetAsync(be.p, 0, sizeof(unsigned long long), stream());
            PEEC_LAUNCH(k_residual, (unsigned)((nv * 32 + 255) / 256), 256, 0, Z, absZ.p, x, absx.p, b, n, nrhs, r.p,
                        be.p, skip);
            if (cap) PEEC_LAUNCH(k_sweep_done, 1, 1, 0, (const unsigned long long *)be.p, cap->tol, done.p);
        };
        if (cap) {
            cudaMemsetAsync(done.p, 0, sizeof(int), stream());
            for (int it = 0; it < cap->sweeps; ++it) sweep();
            total_it = cap->sweeps;
            return launch_ok("refinement") ? 0 : -1;
        }
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t gexec = nullptr;
        if (!sync("refinement setup")) return -1;
        unsigned long long sweep_launches = 0;
        if (cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            unsigned long long l0 = launch_count();
            sweep();
            sweep_launches = launch_count() - l0;
            if (cudaStreamEndCapture(stream(), &graph) != cudaSuccess ||
                cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) {
                gexec = nullptr;
            }
        }
        cudaGetLastError();  // a failed capture falls back to direct launches
        tr.mark(gexec ? "refine: sweep graph recorded" : "refine: capture failed");
        const int window = T == 6 ? 6 : 3;
        const double gain = T == 6 ? 0.5 : 0.25;
        double best = INFINITY, back[6];  // back[it % window]: the best after sweep it - window
        for (double &v : back) v = INFINITY;
        int out = 1, it = 1;
        eta = INFINITY;
        for (; it <= max_iter; ++it) {
            if (gexec) {
                if (!cuda_ok(cudaGraphLaunch(gexec, stream()), "refinement graph")) {
                    out = -1;
                    break;
                }
                note_launch((int)sweep_launches);  // the replayed kernels
            } else {
                sweep();
            }
            unsigned long long hb = 0;
            int hw = 0;
            cudaMemcpyAsync(&hb, be.p, sizeof(hb), cudaMemcpyDeviceToHost, stream());
            cudaMemcpyAsync(&hw, werr.p, sizeof(hw), cudaMemcpyDeviceToHost, stream());
            if (!launch_ok("refinement") || !sync("refinement") || hw) {
                if (hw) set_error("triangular solve: a wait for an earlier row block timed out");
                out = -1;
                break;
            }
            memcpy(&eta, &hb, sizeof(eta));
            tr.mark("refine: sweep");
            if (eta <= tol) {
                out = 0;
                break;
            }
            if (!isfinite(eta)) break;
            best = fmin(best, eta);
            if (best > gain * back[it % window]) break;
            back[it % window] = best;
        }
        total_it += it > max_iter ? max_iter : it;
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        if (many && out != -1) {
            // the last backward error of every right-hand side (those that
            // stopped earlier were not recomputed in the last sweeps)
            std::vector<unsigned long long> hq(nrhs_);
            if (!be_q.download(hq.data(), nrhs_) || !sync("per right-hand side errors")) return -1;
            double worst = 0.0;
            for (unsigned long long bits : hq) {
                double e;
                memcpy(&e, &bits, sizeof(e));
                worst = fmax(worst, e);
            }
            eta = worst;
            out = eta <= tol ? 0 : 1;
        }
        return out;
    };
    // FGMRES-IR with the BF16x6 factor, the last rung: per right-hand side
    // from x = 0, outer FP64 residuals r = b - Z x and inner flexible GMRES
    // on D_r^-1 Z d = D_r^-1 r (the equilibrated rows), preconditioned by the
    // FP32 factor in FP32 (z_k = D_c^-1 U^-1 L^-1 P v_k, kept for the update
    // d = Z_k y since the preconditioner is not exactly linear); classical
    // Gram-Schmidt twice, Givens rotations on the host; 1e-6 relative
    // residual or 40 steps per inner solve.  A right-hand side stops at the
    // gate, after 10 outer steps, or when its backward error no longer
    // halves.  Up to kGmresChunk right-hand sides run in lockstep: one
    // triangular solve, one pass over Z and one host round trip per step
    // serve them all, each with its own Krylov basis, rotations and stopping
    // (a finished one rides along on zero vectors).  0 at the gate, 1 when
    // not, -1 on errors.
    int gmres_total = 0;
    auto gmres_ir = [&]() -> int {
        constexpr int m = 40, ld = m + 1;
        const int Q = std::min(nrhs, kGmresChunk);
        DBuf<cplx> V((size_t)(m + 1) * Q * n), Zk((size_t)m * Q * n), w((size_t)Q * n), hd((size_t)2 * Q * ld),
            yd((size_t)Q * ld);
        DBuf<double> nrm(Q);
        DBuf<unsigned long long> beq(Q);
        if (!V.p || !Zk.p || !w.p || !hd.p || !yd.p || !nrm.p || !beq.p) return -1;
        const unsigned gn = (unsigned)((n + 255) / 256), gw = (unsigned)(((size_t)n * 32 + 255) / 256);
        using zc = std::complex<double>;
        auto host_sync = [&](const char *what) -> bool {
            int hw = 0;
            cudaMemcpyAsync(&hw, werr.p, sizeof(hw), cudaMemcpyDeviceToHost, stream());
            if (!launch_ok(what) || !sync(what)) return false;
            if (hw) set_error("triangular solve: a wait for an earlier row block timed out");
            return hw == 0;
        };
        double eta_max = 0.0;
        for (int q0 = 0; q0 < nrhs; q0 += Q) {
            const int nq = std::min(Q, nrhs - q0);
            const dim3 gq(gn, (unsigned)nq);
            // z_q = D_c^-1 U^-1 L^-1 P v_q in FP32, returned in FP64, for all q at once
            auto precondition = [&](const cplx *v, cplx *z) -> bool {
                PEEC_LAUNCH(k_perm_f32, gq, 256, 0, v, perm.p, n, y.p);
                WaveArgs<cplxf> W{};
                W.lu = a;
                W.dinv = wdinv.p;
                W.n = n;
                W.nrhs = nq;
                W.b = y.p;
                W.x = y.p;
                W.flags = wflags.p;
                W.error = werr.p;
                W.subst = 1;
                if (!wave_solve(W)) return false;
                PEEC_LAUNCH(k_mix_out, gq, 256, 0, y.p, cs.p, n, z);
                return true;
            };
            cplx *xc = x + (size_t)q0 * n;
            const cplx *bc = b + (size_t)q0 * n;
            cudaMemsetAsync(xc, 0, (size_t)nq * n * sizeof(cplx), stream());
            std::vector<double> eta_q(nq, INFINITY), prev(nq, INFINITY), beta(nq), hn(nq);
            std::vector<unsigned long long> hb(nq);
            std::vector<char> live(nq, 1);  // still iterating (outer)
            for (int outer = 0; outer < 10; ++outer) {
                cudaMemsetAsync(beq.p, 0, nq * sizeof(unsigned long long), stream());
                for (int q = 0; q < nq; ++q) {
                    const size_t o = (size_t)q * n;
                    PEEC_LAUNCH(k_abs_x, gn, 256, 0, xc + o, (size_t)n, absx.p + o);
                    PEEC_LAUNCH(k_residual, gw, 256, 0, Z, absZ.p, xc + o, absx.p + o, bc + o, n, 1, r.p + o,
                                beq.p + q, (const int *)nullptr);
                    PEEC_LAUNCH(k_scale_rows, gn, 256, 0, r.p + o, rs.p, n, V.p + o);
                }
                PEEC_LAUNCH(k_norm2, nq, 1024, 0, V.p, n, nrm.p);
                cudaMemcpyAsync(hb.data(), beq.p, nq * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream());
                cudaMemcpyAsync(beta.data(), nrm.p, nq * sizeof(double), cudaMemcpyDeviceToHost, stream());
                if (!host_sync("GMRES-IR residual")) return -1;
                GmresScalars sc0{};
                bool any = false;
                for (int q = 0; q < nq; ++q) {
                    if (!live[q]) continue;
                    memcpy(&eta_q[q], &hb[q], sizeof(double));
                    if (eta_q[q] <= tol || !isfinite(eta_q[q]) || eta_q[q] > 0.5 * prev[q] || !(beta[q] > 0.0) ||
                        !isfinite(beta[q])) {
                        live[q] = 0;
                        continue;
                    }
                    prev[q] = eta_q[q];
                    sc0.v[q] = 1.0 / beta[q];
                    any = true;
                }
                if (!any) break;
                PEEC_LAUNCH(k_cscale, gq, 256, 0, V.p, n, sc0, V.p);
                std::vector<std::vector<zc>> H(nq, std::vector<zc>((size_t)(m + 1) * m)), g(nq), sn(nq);
                std::vector<std::vector<double>> c(nq, std::vector<double>(m));
                std::vector<cplx> hh((size_t)2 * Q * ld);
                std::vector<char> inner(live);
                GmresCounts kk{};
                for (int q = 0; q < nq; ++q) {
                    g[q].assign(m + 1, zc(0.0));
                    sn[q].assign(m, zc(0.0));
                    g[q][0] = beta[q];
                }
                for (int k = 0; k < m; ++k) {
                    cplx *zk = Zk.p + (size_t)k * nq * n;
                    const cplx *vk = V.p + (size_t)k * nq * n;
                    if (!precondition(vk, zk)) return -1;
                    PEEC_LAUNCH(k_zmv_scaled, gw, 256, 0, Z, zk, rs.p, n, nq, w.p);
                    for (int pass = 0; pass < 2; ++pass) {
                        PEEC_LAUNCH(k_gs_dots, dim3((unsigned)(k + 1), (unsigned)nq), 256, 0, V.p, n, nq, w.p,
                                    hd.p + (size_t)pass * Q * ld, ld);
                        PEEC_LAUNCH(k_gs_update, gq, 256, 0, V.p, n, nq, k + 1, hd.p + (size_t)pass * Q * ld, ld, w.p);
                    }
                    PEEC_LAUNCH(k_norm2, nq, 1024, 0, w.p, n, nrm.p);
                    cudaMemcpyAsync(hh.data(), hd.p, hh.size() * sizeof(cplx), cudaMemcpyDeviceToHost, stream());
                    cudaMemcpyAsync(hn.data(), nrm.p, nq * sizeof(double), cudaMemcpyDeviceToHost, stream());
                    if (!host_sync("GMRES-IR step")) return -1;
                    ++gmres_total;
                    GmresScalars sck{};
                    bool more = false;
                    for (int q = 0; q < nq; ++q) {
                        if (!inner[q]) continue;
                        zc *col = &H[q][(size_t)k * (m + 1)];
                        const cplx *h0 = &hh[(size_t)q * ld], *h1 = &hh[(size_t)(Q + q) * ld];
                        for (int j = 0; j <= k; ++j) col[j] = zc(h0[j].re + h1[j].re, h0[j].im + h1[j].im);
                        const double hq = hn[q];
                        if (hq > 0.0 && isfinite(hq)) sck.v[q] = 1.0 / hq;
                        // earlier rotations, then a new one zeroing the subdiagonal hq
                        for (int j = 0; j < k; ++j) {
                            const zc u = c[q][j] * col[j] + sn[q][j] * col[j + 1];
                            col[j + 1] = -std::conj(sn[q][j]) * col[j] + c[q][j] * col[j + 1];
                            col[j] = u;
                        }
                        const double aa = std::abs(col[k]), rr = std::hypot(aa, hq);
                        if (aa == 0.0) {
                            c[q][k] = 0.0;
                            sn[q][k] = 1.0;
                            col[k] = hq;
                        } else {
                            const zc ph = col[k] / aa;
                            c[q][k] = aa / rr;
                            sn[q][k] = ph * (hq / rr);
                            col[k] = ph * rr;
                        }
                        g[q][k + 1] = -std::conj(sn[q][k]) * g[q][k];
                        g[q][k] = c[q][k] * g[q][k];
                        kk.v[q] = k + 1;
                        if (!(hq > 0.0) || !isfinite(hq) || std::abs(g[q][k + 1]) <= 1e-6 * beta[q]) {
                            inner[q] = 0;
                            sck.v[q] = 0.0;
                        } else {
                            more = true;
                        }
                    }
                    PEEC_LAUNCH(k_cscale, gq, 256, 0, w.p, n, sck, V.p + (size_t)(k + 1) * nq * n);
                    if (!more) break;
                }
                // y_q from the triangular H_q, x_q += Z_k y_q
                std::vector<cplx> yh((size_t)Q * ld, cplx{0.0, 0.0});
                for (int q = 0; q < nq; ++q) {
                    if (!live[q]) continue;
                    const int kq = kk.v[q];
                    std::vector<zc> yv(kq);
                    for (int i = kq - 1; i >= 0; --i) {
                        zc sum = g[q][i];
                        for (int j = i + 1; j < kq; ++j) sum -= H[q][(size_t)j * (m + 1) + i] * yv[j];
                        yv[i] = sum / H[q][(size_t)i * (m + 1) + i];
                    }
                    for (int i = 0; i < kq; ++i) yh[(size_t)q * ld + i] = cplx{yv[i].real(), yv[i].imag()};
                }
                cudaMemcpyAsync(yd.p, yh.data(), yh.size() * sizeof(cplx), cudaMemcpyHostToDevice, stream());
                PEEC_LAUNCH(k_gmres_update, gq, 256, 0, Zk.p, n, nq, kk, yd.p, ld, xc);
                if (!host_sync("GMRES-IR update")) return -1;
            }
            for (int q = 0; q < nq; ++q) {
                if (!(eta_q[q] <= tol)) {
                    eta = eta_q[q];
                    return 1;
                }
                eta_max = std::max(eta_max, eta_q[q]);
            }
        }
        eta = eta_max;
        return 0;
    };
    float t01 = -1.0f, ms_factor = 0.0f, ms_refine = 0.0f;
    int outcome;
    if (cap) {
        outcome = factor();
        if (outcome == 0) outcome = refine();
        if (outcome != 0) return -1;
        PEEC_LAUNCH(k_capture_status, 1, 1, 0, st.p, werr.p, be.p, cap->d_eta_bits, cap->d_status);
        return launch_ok("mixed solve (graph form)") ? 0 : -1;
    }
    for (;;) {
        outcome = factor();
        cudaEventRecord(ev[2], stream());
        if (outcome == 0) outcome = refine();
        cudaEventRecord(ev[3], stream());
        cudaEventSynchronize(ev[3]);
        if (t01 < 0.0f) cudaEventElapsedTime(&t01, ev[0], ev[1]);
        float t12 = 0.0f, t23 = 0.0f;
        cudaEventElapsedTime(&t12, ev[1], ev[2]);
        cudaEventElapsedTime(&t23, ev[2], ev[3]);
        ms_factor += t12;
        ms_refine += t23;
        if (outcome == -1 || outcome == 0 || T == 6) break;
        // stalled (or an FP32 pivot breakdown) with BF16x3: factor the FP32
        // copy of the equilibrated Z again with BF16x6 products
        T = 6;
        cudaEventRecord(ev[1], stream());
        cudaMemsetAsync(scratch.p, 0, sbytes, stream());
        cudaMemsetAsync(st.p, 0, sizeof(Status), stream());
        cudaMemsetAsync(err.p, 0, sizeof(int), stream());
        cudaMemsetAsync(lean_flag.p, 0, lean_flag.n * sizeof(unsigned long long), stream());
        PEEC_LAUNCH(k_eq2_to_float, 152 * 16, 256, 0, Z, n, er.p, ec.p, f.p, (float *)nullptr);
    }
    if (outcome == 1 && T == 6) {
        // still stalled with BF16x6: GMRES-IR with the same factor
        cudaEventRecord(ev[2], stream());
        outcome = gmres_ir();
        cudaEventRecord(ev[3], stream());
        cudaEventSynchronize(ev[3]);
        float t23 = 0.0f;
        cudaEventElapsedTime(&t23, ev[2], ev[3]);
        ms_refine += t23;
        total_it += gmres_total;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (outcome == -1) return -1;
    g_mixed_timing.gmres_iterations = gmres_total;
    g_mixed_timing.ms_prepare = t01;
    g_mixed_timing.ms_factor = ms_factor;
    g_mixed_timing.ms_refine = ms_refine;
    g_mixed_timing.iterations = total_it;
    g_mixed_timing.split_terms = T;
    if (backward_error) *backward_error = eta;
    if (iterations) *iterations = total_it;
    if (outcome == -2) return -2;
    return outcome == 0 ? 0 : 1;
}

}  // namespace peec

extern "C" int peec_gb300_complex_solve_mixed_device(const Complex *d_Z, size_t n_, const Complex *d_b, Complex *d_x,
                                                     size_t nrhs_, double tol, int max_iter, double *backward_error,
                                                     int *iterations) {
    return peec::mixed_solve_impl(d_Z, n_, d_b, d_x, nrhs_, tol, max_iter, backward_error, iterations, nullptr);
}

namespace peec {
__global__ void k_round_f32(const double *x, float *y, size_t count, int shift) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
        y[t] = f64_to_f32_scaled(x[t], shift);
}
}  // namespace peec

// The FP32 rounding of the mixed path's equilibration: y = x 2^-shift to the
// nearest FP32 (ties to even), subnormal results flushed to zero.
extern "C" int peec_gb300_round_to_f32_device(const double *d_x, float *d_y, size_t count, int shift) {
    using namespace peec;
    if ((!d_x || !d_y) && count) return -1;
    if (!count) return 0;
    PEEC_LAUNCH(k_round_f32, 152 * 4, 256, 0, d_x, d_y, count, shift);
    return sync("FP32 rounding") ? 0 : -1;
}

extern "C" int peec_gb300_mixed_split_terms(void) { return peec::g_mixed_timing.split_terms; }

extern "C" int peec_gb300_mixed_gmres_iterations(void) { return peec::g_mixed_timing.gmres_iterations; }

extern "C" int peec_gb300_mixed_timing(double *ms_prepare, double *ms_factor, double *ms_refine) {
    if (ms_prepare) *ms_prepare = peec::g_mixed_timing.ms_prepare;
    if (ms_factor) *ms_factor = peec::g_mixed_timing.ms_factor;
    if (ms_refine) *ms_refine = peec::g_mixed_timing.ms_refine;
    return peec::g_mixed_timing.iterations;
}
