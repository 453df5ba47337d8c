// Lp / P assembly on sm_103a: the 1/R panel integrals of the dual mesh.
//
// Reference path (paths inside the reference project):
//   src/peec/inductance.c:221-560  Lp entries and matrix
//   src/peec/potential.c:139-395   P entries and matrix
//   src/peec/quadrature.c:550-1079 pair classification, far rule, analytic
//                                  triangle potential, adaptive outer rule
//
// Pipeline for one matrix (all on the library stream):
//   1. k_patch_prep      per patch: bounding box, longest side
//   2. k_far_points      per patch: the far-rule points and weights of its two
//                        triangles (x, y, z, w) -- reused by every pair
//   3. k_near_scan       per patch i: every partner j of the upper triangle
//                        whose class is not FAR (counted, scanned, filled:
//                        a deterministic, i-major, j-sorted list)
//   4. k_near_eval       one warp per (near pair, triangle pair, direction):
//                        adaptive outer Gauss rule over the analytic inner
//                        potential, depth-first with an explicit stack
//   5. k_near_finalize   per near pair: the 4 triangle-pair values combined in
//                        the reference's order (both orientations)
//   6. k_assemble_tiles  one CTA per 32x32 tile of the upper triangle, one
//                        warp per entry: sums its patch pairs in the
//                        reference's (i, j) order, far pairs by the product
//                        rule with a warp-shuffle reduction, near pairs from
//                        step 5; the tile and its mirror are written with
//                        coalesced row stores.
// Everything is FP64.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/dual_mesh.h"
#include "../../include/inductance.h"
#include "../../include/mesh.h"
#include "../../include/peec_gb300.h"
#include "../../include/potential.h"
#include "../../include/quadrature.h"
#include "common.cuh"
#include "geometry.cuh"

namespace peec {

static const double kMu0Over4Pi = 1.0e-7;               // inductance.c:24
static const double kInv4PiEps0 = 8.987551792261171e9;  // potential.c:26

__constant__ double c_gl_x[GL_NUM_ORDERS][16];
__constant__ double c_gl_w[GL_NUM_ORDERS][16];

static bool upload_gl_tables() {
    static std::once_flag once;
    static bool ok = false;
    std::call_once(once, [] {
        ok = cuda_ok(cudaMemcpyToSymbol(c_gl_x, GL_NODES, sizeof(GL_NODES)), "GL table") &&
             cuda_ok(cudaMemcpyToSymbol(c_gl_w, GL_WEIGHTS, sizeof(GL_WEIGHTS)), "GL table");
    });
    return ok;
}

enum Kind { KIND_INDUCTANCE = 0, KIND_POTENTIAL = 1, KIND_RAW = 2 };

// Device-resident region set: the patches of all edge (or node) regions,
// region-contiguous, plus per-region scale data.
struct RegionsDev {
    int n = 0;             // regions
    int np = 0;            // patches
    int *off = nullptr;    // [n+1]
    int *owner = nullptr;  // [np]
    double *corner = nullptr;  // [np*12]
    double *box = nullptr;     // [np*6]
    double *size = nullptr;    // [np]
    double *dir = nullptr;     // [n*3]   (inductance)
    double *scale = nullptr;   // [n]     width w (inductance) or area S (potential); <= 0 marks a bad region
    int *same_obj = nullptr;   // [np]    object id for the reference's pointer test
    float4 *boxf = nullptr;    // [np*2]  box rounded to FP32: (lo, size), (hi, 0) -- the scan's far filter
    int *axis = nullptr;       // [n]     0/1/2 when dir is exactly +-e_axis, else -1 (inductance)
    double cmax = 0.0;         // largest |corner coordinate| (scale of the rounding noise)
};

// one far-rule point: position and weight (32-byte aligned for vector loads)
struct alignas(32) FarPt {
    double x, y, z, w;
};

// The same point as unevaluated float pairs (hi + lo == the double to 2^-48
// relative): the far rule runs on the FP32 pipes in double-float arithmetic.
struct alignas(32) FarPtF {
    float xh, yh, zh, wh, xl, yl, zl, wl;
};

__device__ __forceinline__ void split_df(double v, float &h, float &l) {
    h = __double2float_rn(v);
    l = __double2float_rn(v - (double)h);
}

struct NearRec {
    int i, j, cls, pad;
};

// ---------------------------------------------------------------------
// 1-2. per-patch preparation
// ---------------------------------------------------------------------
__global__ void k_patch_prep(RegionsDev R) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= R.np) return;
    const double *c = R.corner + 12 * (size_t)p;
    double *b = R.box + 6 * (size_t)p;
    patch_aabb(c, b);
    R.size[p] = patch_size(c);
    R.boxf[2 * p] = make_float4((float)b[0], (float)b[1], (float)b[2], (float)R.size[p]);
    R.boxf[2 * p + 1] = make_float4((float)b[3], (float)b[4], (float)b[5], 0.0f);
}

// Far-rule points of patch p: triangle t (0: corners 0,1,2; 1: 0,2,3), point
// (iu, iv) at index t*q*q + iu*q + iv; weight (0.5 w_iu)(0.5 w_iv) J
// (reference quadrature.c:679-783 evaluates the same points per pair).
__global__ void k_far_points(RegionsDev R, int q, int row, FarPt *pts, FarPtF *ptf) {
    int np = R.np, per = 2 * q * q;
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)np * per) return;
    int p = (int)(g / per), k = (int)(g % per);
    int t = k / (q * q), iu = (k / q) % q, iv = k % q;
    const double *c = R.corner + 12 * (size_t)p;
    const double *p0 = c, *p1 = c + (t == 0 ? 3 : 6), *p2 = c + (t == 0 ? 6 : 9);
    double u = 0.5 * (c_gl_x[row][iu] + 1.0), wu = 0.5 * c_gl_w[row][iu];
    double v = 0.5 * (c_gl_x[row][iv] + 1.0), wv = 0.5 * c_gl_w[row][iv];
    double r[3], jac;
    tri_map(p0, p1, p2, u, v, r, &jac);
    double w = wu * wv * jac;
    pts[g] = FarPt{r[0], r[1], r[2], w};
    FarPtF f;
    split_df(r[0], f.xh, f.xl);
    split_df(r[1], f.yh, f.yl);
    split_df(r[2], f.zh, f.zl);
    split_df(w, f.wh, f.wl);
    ptf[g] = f;
}

// ---------------------------------------------------------------------
// 3. near-pair discovery
// ---------------------------------------------------------------------
struct ScanArgs {
    RegionsDev R;
    int kind;
    double near_factor;
    double dir_tol;
    int only_a, only_b;  // >= 0: restrict to the single entry (only_a, only_b)
};

__device__ __forceinline__ bool region_pair_skipped(const ScanArgs &s, int a, int b) {
    if (s.only_a >= 0) {
        int lo = s.only_a < s.only_b ? s.only_a : s.only_b, hi = s.only_a < s.only_b ? s.only_b : s.only_a;
        if (!(a == lo && b == hi)) return true;
    }
    if (s.kind == KIND_INDUCTANCE) {
        // axis-aligned directions: the FP64 dot product is exactly 0 or +-1
        const int xa = s.R.axis[a], xb = s.R.axis[b];
        if (xa >= 0 && xb >= 0) return (xa != xb ? 0.0 : 1.0) < s.dir_tol;
        double d = dot3(s.R.dir + 3 * a, s.R.dir + 3 * b);
        if (fabs(d) < s.dir_tol) return true;  // entry is exactly 0, no integral
    }
    return false;
}

// pass 0 counts, pass 1 writes (count[i] -> offsets in off[i]).  One warp
// per patch i, the lanes over consecutive partners j: the partners found in
// a chunk of 32 are ranked by ballot, so the list keeps the j order.
__global__ void k_near_scan(ScanArgs s, int pass, int *count, const int *off, NearRec *out,
                            unsigned long long *far_pairs) {
    const int lane = threadIdx.x & 31;
    const int i = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const RegionsDev &R = s.R;
    if (i >= R.np) return;
    const int a = R.owner[i];
    const double *ci = R.corner + 12 * (size_t)i, *bi = R.box + 6 * (size_t)i;
    const double hi = R.size[i];
    // FP32 filter: a pair whose FP32 gap exceeds the FP32 threshold by more
    // than the rounding of both (boxes rounded to FP32 move by <= 2^-24 cmax
    // per coordinate; the margins below are 4x the worst case) is FAR in the
    // exact FP64 test as well; every other pair takes the exact test.
    const float4 la = R.boxf[2 * i], ha4 = R.boxf[2 * i + 1];
    const float nf = (float)s.near_factor;
    const float slack = (float)(9.5367431640625e-07 * R.cmax);  // 2^-20 cmax
    const int same_i = R.same_obj[i];
    const int w = pass ? off[i] : 0;
    int found = 0;
    unsigned long long nfar = 0;
    int b_prev = -1;
    bool skip_b = false;
    for (int jb = R.off[a]; jb < R.np; jb += 32) {
        const int j = jb + lane;
        bool near = false;
        int cls = CLS_FAR;
        if (j < R.np) {
            const int b = R.owner[j];
            if (b != b_prev) {
                skip_b = region_pair_skipped(s, a, b);
                b_prev = b;
            }
            if (!skip_b && !(b == a && j < i)) {
                const bool same = same_i == R.same_obj[j];
                bool far = false;
                if (!same) {
                    const float4 lb = R.boxf[2 * j], hb4 = R.boxf[2 * j + 1];
                    float gx = fmaxf(0.0f, fmaxf(la.x - hb4.x, lb.x - ha4.x));
                    float gy = fmaxf(0.0f, fmaxf(la.y - hb4.y, lb.y - ha4.y));
                    float gz = fmaxf(0.0f, fmaxf(la.z - hb4.z, lb.z - ha4.z));
                    float gap = sqrtf(gx * gx + gy * gy + gz * gz);
                    float h = fmaxf(la.w, lb.w);
                    far = gap * (1.0f - 9.5367431640625e-07f) - slack > nf * h * (1.0f + 9.5367431640625e-07f);
                }
                if (!far)
                    cls = classify_pair(ci, bi, hi, R.corner + 12 * (size_t)j, R.box + 6 * (size_t)j, R.size[j],
                                        s.near_factor, same);
                if (cls == CLS_FAR)
                    ++nfar;
                else
                    near = true;
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, near);
        if (pass && near) out[w + found + __popc(bal & ((1u << lane) - 1u))] = NearRec{i, j, cls, 0};
        found += __popc(bal);
    }
    if (!pass) {
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) nfar += __shfl_xor_sync(0xffffffffu, nfar, sh);
        if (lane == 0) {
            count[i] = found;
            if (far_pairs && nfar) atomicAdd(far_pairs, nfar);
        }
    }
}

// exclusive scan of count[0..n) into off[0..n], single CTA of 1024 threads
__global__ void k_exclusive_scan(const int *count, int *off, int n) {
    __shared__ long long part[1024];
    int t = threadIdx.x;
    int chunk = (n + 1023) / 1024;
    int lo = t * chunk, hi = min(n, lo + chunk);
    long long s = 0;
    for (int k = lo; k < hi; ++k) s += count[k];
    part[t] = s;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        long long v = (t >= d) ? part[t - d] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    long long base = part[t] - s;
    for (int k = lo; k < hi; ++k) {
        off[k] = (int)base;
        base += count[k];
    }
    if (t == 1023) off[n] = (int)part[1023];
}

// ---------------------------------------------------------------------
// 4. analytic potential + adaptive outer rule (quadrature.c:842-938)
// ---------------------------------------------------------------------
struct TriPot {
    double p[3][3], unit[3][3], outw[3][3], len[3], nrm[3];
    double twice_area;
};

__device__ void tri_prepare(const double *v, TriPot &t) {
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            t.p[i][k] = v[3 * i + k];
            t.unit[i][k] = v[3 * ((i + 1) % 3) + k] - v[3 * i + k];
        }
    cross3(t.unit[0], t.unit[1], t.nrm);
    t.twice_area = norm3(t.nrm);
    if (t.twice_area == 0.0) return;
    for (int k = 0; k < 3; ++k) t.nrm[k] /= t.twice_area;
    for (int i = 0; i < 3; ++i) {
        t.len[i] = norm3(t.unit[i]);
        for (int k = 0; k < 3; ++k) t.unit[i][k] /= t.len[i];
        cross3(t.unit[i], t.nrm, t.outw[i]);
    }
}

// \int_T 1/|r - r0| dS exactly: sum over edges of d_e * (asinh terms) minus
// |h * solid angle| (van Oosterom's uniform-layer formula, as the reference).
__device__ double tri_potential(const TriPot &t, const double *r) {
    double v[3][3], rad[3];
    for (int i = 0; i < 3; ++i) {
        for (int k = 0; k < 3; ++k) v[i][k] = t.p[i][k] - r[k];
        rad[i] = norm3(v[i]);
    }
    double h = dot3(v[0], t.nrm);
    double acc = 0.0;
    for (int i = 0; i < 3; ++i) {
        double d = dot3(v[i], t.outw[i]);
        if (d == 0.0) continue;  // finite limit d log(.) = 0, as the reference
        // Edge integral asinh((s+L)/q) - asinh(s/q), q = hypot(d, h), as
        // log(A2/A1) with A = s + sqrt(s^2 + q^2) (= q e^asinh(s/q)); for
        // s < 0 the equal form q^2 / (sqrt(s^2 + q^2) - s) avoids the
        // cancellation.  The square roots use the same s and q as the
        // asinh arguments (not the vertex distances, which disagree by
        // rounding when the point lies on the edge's line).  One log and two
        // square roots instead of two asinh and a hypot.
        double s = dot3(v[i], t.unit[i]);
        double s2 = s + t.len[i];
        double q2 = d * d + h * h;
        double e;
        if (q2 > 1e-280) {
            double r1 = sqrt(fma(s, s, q2)), r2 = sqrt(fma(s2, s2, q2));
            double a1 = s >= 0.0 ? s + r1 : q2 / (r1 - s);
            double a2 = s2 >= 0.0 ? s2 + r2 : q2 / (r2 - s2);
            e = log(a2 / a1);
        } else {  // q^2 underflows: the reference's form
            double q = hypot(d, h);
            e = asinh(s2 / q) - asinh(s / q);
        }
        acc += d * e;
    }
    if (h != 0.0) {
        double c[3];
        cross3(v[1], v[2], c);
        double den = rad[0] * rad[1] * rad[2] + dot3(v[0], v[1]) * rad[2] + dot3(v[1], v[2]) * rad[0] +
                     dot3(v[2], v[0]) * rad[1];
        double omega = 2.0 * atan2(dot3(v[0], c), den);
        acc -= fabs(h * omega);
    }
    return acc;
}

struct AdaptNode {
    double v[9];
    double tol;
    int depth;
    int pad;
};

static const int kStackCap = 28;  // depth <= 24 => at most 26 pending nodes

struct NearWarpSmem {
    TriPot inner;
    AdaptNode stack[kStackCap];
};

// Depth-first adaptive integration of triangle `outer` against the inner
// potential, by one warp: the low and high rules of a node are spread over
// the lanes and reduced with shuffles; accepted nodes add `high` left to
// right.  Returns NaN if a rule is non-finite or depth 24 is exceeded
// (reference quadrature.c:915-938).
// Decision flags for the reuse of translated copies (see 5b below).
enum : int { MARG_THRESHOLD = 1, MARG_TIE = 2, MARG_TRACE_FULL = 4 };
static const int kTraceCap = 256;       // decisions recorded per job
static const unsigned char kAccept = 0xFF;

__device__ double warp_adaptive(const double *outer, NearWarpSmem &sm, int order, double abs_tol,
                                unsigned long long &evals, int &mflags, unsigned char *trace, int &trace_len) {
    const int lane = threadIdx.x & 31;
    const int ql = order <= 6 ? 3 : 4;
    const int rl = gl_row(ql), rh = gl_row(order);
    const int nlo = ql * ql, ntot = nlo + order * order;
    if (lane == 0) {
        for (int k = 0; k < 9; ++k) sm.stack[0].v[k] = outer[k];
        sm.stack[0].tol = abs_tol;
        sm.stack[0].depth = 0;
    }
    __syncwarp();
    int sp = 1;
    double acc = 0.0;
    while (sp > 0) {
        AdaptNode nd = sm.stack[sp - 1];
        --sp;
        __syncwarp();
        const double *a0 = nd.v, *a1 = nd.v + 3, *a2 = nd.v + 6;
        double lo = 0.0, hi = 0.0;
        for (int k = lane; k < ntot; k += 32) {
            int ord, row, idx;
            if (k < nlo) {
                ord = ql;
                row = rl;
                idx = k;
            } else {
                ord = order;
                row = rh;
                idx = k - nlo;
            }
            int i = idx / ord, j = idx % ord;
            double xi = c_gl_x[row][i], xj = c_gl_x[row][j];
            double wi = c_gl_w[row][i], wj = c_gl_w[row][j];
            double r[3], jac;
            tri_map(a0, a1, a2, 0.5 * (xi + 1.0), 0.5 * (xj + 1.0), r, &jac);
            double val = 0.25 * wi * wj * jac * tri_potential(sm.inner, r);
            if (k < nlo)
                lo += val;
            else
                hi += val;
        }
        evals += (unsigned long long)ntot;
        lo = warp_sum(lo);
        hi = warp_sum(hi);
        if (!isfinite(lo) || !isfinite(hi)) return nan("");
        // a decision within 1e-6 of its threshold could go the other way for
        // a copy of this pair that differs only by rounding of its corners
        double thr = nd.tol + 2e-5 * fabs(hi), gap = fabs(hi - lo);
        if (fabs(gap - thr) <= 1e-6 * thr) mflags |= MARG_THRESHOLD;
        if (fabs(hi - lo) <= nd.tol + 2e-5 * fabs(hi)) {
            acc += hi;
            if (trace) {
                if (trace_len < kTraceCap) {
                    if (lane == 0) trace[trace_len] = kAccept;
                    ++trace_len;
                } else {
                    mflags |= MARG_TRACE_FULL;
                }
            }
            continue;
        }
        if (nd.depth >= 24 || sp + 2 > kStackCap) return nan("");
        int e = 0;
        double longest = 0.0, len[3];
        for (int i = 0; i < 3; ++i) {
            double s = dist3(nd.v + 3 * i, nd.v + 3 * ((i + 1) % 3));
            len[i] = s;
            if (s > longest) {
                longest = s;
                e = i;
            }
        }
        // two (nearly) equal longest edges: which one is bisected is decided
        // by rounding, so a translated copy may subdivide differently
        for (int i = 0; i < 3; ++i)
            if (i != e && len[i] >= longest * (1.0 - 1e-10)) mflags |= MARG_TIE;
        if (trace) {
            if (trace_len < kTraceCap) {
                if (lane == 0) trace[trace_len] = (unsigned char)e;
                ++trace_len;
            } else {
                mflags |= MARG_TRACE_FULL;
            }
        }
        int j = (e + 1) % 3, k = (e + 2) % 3;
        if (lane == 0) {
            AdaptNode &left = sm.stack[sp + 1], &right = sm.stack[sp];
            for (int d = 0; d < 3; ++d) {
                double mid = 0.5 * (nd.v[3 * e + d] + nd.v[3 * j + d]);
                left.v[d] = nd.v[3 * e + d];
                left.v[3 + d] = mid;
                left.v[6 + d] = nd.v[3 * k + d];
                right.v[d] = mid;
                right.v[3 + d] = nd.v[3 * j + d];
                right.v[6 + d] = nd.v[3 * k + d];
            }
            left.tol = right.tol = nd.tol * 0.5;
            left.depth = right.depth = nd.depth + 1;
        }
        __syncwarp();
        sp += 2;
    }
    return acc;
}

// Triangle t of a patch: 0 -> corners (0,1,2), 1 -> (0,2,3).
__device__ __forceinline__ void patch_triangle(const double *c, int t, double *v) {
    const int idx[2][3] = {{0, 1, 2}, {0, 2, 3}};
    for (int m = 0; m < 3; ++m)
        for (int k = 0; k < 3; ++k) v[3 * m + k] = c[3 * idx[t][m] + k];
}

struct NearEvalArgs {
    const double *corner;
    const NearRec *rec;
    const int *job_rec;  // records to evaluate (representatives), or null for all
    int nrec;            // number of records to evaluate
    int orders[4];  // far, near, touching, self
    double *slot;   // [records*4*2]
    int *kind;      // [nrec*4]: 0 adaptive, 1 zero area, 2 identical triangles
    int *next_job;  // work counter
    unsigned long long *evals;
    int *marginal;  // [nrec] MARG_* flags of the record's jobs (null: not recorded)
    unsigned char *trace;  // [jobs * kTraceCap] decision traces (null: not recorded)
    int *trace_len;        // [jobs]
};

// One warp per job (record, triangle pair t = s*2+u, direction d); warps
// fetch jobs dynamically because refinement depth varies a lot.
__global__ void __launch_bounds__(256, 2) k_near_eval(NearEvalArgs A) {
    extern __shared__ unsigned char smem_raw[];
    NearWarpSmem *all = reinterpret_cast<NearWarpSmem *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    NearWarpSmem &sm = all[warp];
    const long long njobs = (long long)A.nrec * 8;
    unsigned long long evals = 0;
    for (;;) {
        long long job = 0;
        if (lane == 0) job = atomicAdd(A.next_job, 1);
        job = __shfl_sync(0xffffffffu, job, 0);
        if (job >= njobs) break;
        int r = (int)(job >> 3), t = (int)((job >> 1) & 3), d = (int)(job & 1);
        if (A.job_rec) r = A.job_rec[r];
        NearRec rec = A.rec[r];
        double ta[9], tb[9];
        patch_triangle(A.corner + 12 * (size_t)rec.i, t >> 1, ta);
        patch_triangle(A.corner + 12 * (size_t)rec.j, t & 1, tb);
        // outer = the triangle integrated by the rule, inner = the potential source
        const double *outer = d == 0 ? ta : tb, *inner = d == 0 ? tb : ta;
        TriPot po;  // outer's own prepared form (area, identity test)
        tri_prepare(outer, po);
        if (lane == 0) tri_prepare(inner, sm.inner);
        __syncwarp();
        double out;
        int kind;
        if (po.twice_area == 0.0 || sm.inner.twice_area == 0.0) {
            kind = 1;
            out = 0.0;
        } else {
            bool identical = true;
            for (int m = 0; m < 3; ++m) {
                bool hit = false;
                for (int q = 0; q < 3; ++q)
                    if (same_point(ta + 3 * m, tb + 3 * q)) hit = true;
                if (!hit) identical = false;
            }
            if (identical) {
                // K(T,T) = (2 area / 3) * sum over the outer vertices of the
                // inner potential (quadrature.c:948-956); d = 1 gives the
                // value with the roles of the two triangles swapped.
                kind = 2;
                double s = 0.0;
                for (int m = 0; m < 3; ++m) s += tri_potential(sm.inner, outer + 3 * m);
                out = po.twice_area * s / 3.0;
                evals += 3;
            } else {
                kind = 0;
                int cls = rec.cls;
                int order = cls == CLS_SELF ? A.orders[3] : cls == CLS_TOUCHING ? A.orders[2] : A.orders[1];
                if (order < 6) order = 6;
                double aa = d == 0 ? po.twice_area : sm.inner.twice_area;
                double ab = d == 0 ? sm.inner.twice_area : po.twice_area;
                double scale = aa * ab / sqrt(fmax(aa, ab));
                int mflags = 0, tlen = 0;
                unsigned char *tr = A.trace ? A.trace + (size_t)job * kTraceCap : nullptr;
                out = warp_adaptive(outer, sm, order, 2e-5 * scale, evals, mflags, tr, tlen);
                if (lane == 0 && A.marginal && mflags) atomicOr(A.marginal + r, mflags);
                if (lane == 0 && A.trace_len) A.trace_len[job] = tlen;
            }
        }
        if (lane == 0) {
            A.slot[(size_t)r * 8 + t * 2 + d] = out;
            if (d == 0) A.kind[(size_t)r * 4 + t] = kind;
            if (kind != 0 && A.trace_len) A.trace_len[job] = 0;
        }
        __syncwarp();
    }
    if (lane == 0 && evals) atomicAdd(A.evals, evals);
}

// K for each near record in both orientations (quadrature.c:1060-1076 sums
// the triangle pairs (0,0),(0,1),(1,0),(1,1); the swapped patch order visits
// the same values as (0,0),(1,0),(0,1),(1,1)).
__global__ void k_near_finalize(int nrec, const double *slot, const int *kind, double2 *kval) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    double fwd[4], rev[4];
    for (int t = 0; t < 4; ++t) {
        double s0 = slot[(size_t)r * 8 + t * 2], s1 = slot[(size_t)r * 8 + t * 2 + 1];
        int k = kind[(size_t)r * 4 + t];
        if (k == 1) {
            fwd[t] = rev[t] = 0.0;
        } else if (k == 2) {
            fwd[t] = s0;
            rev[t] = s1;
        } else {
            fwd[t] = rev[t] = 0.5 * (s0 + s1);
        }
    }
    double kf = 0.0, kr = 0.0;
    const int rev_order[4] = {0, 2, 1, 3};
    bool bad_f = false, bad_r = false;
    for (int t = 0; t < 4; ++t) {
        if (!isfinite(fwd[t])) bad_f = true;
        kf += fwd[t];
        double v = rev[rev_order[t]];
        if (!isfinite(v)) bad_r = true;
        kr += v;
    }
    kval[r] = make_double2(bad_f ? nan("") : kf, bad_r ? nan("") : kr);
}

// ---------------------------------------------------------------------
// 5a. level-synchronous form of the adaptive rule
//
// The depth-first warp above serialises a job's whole refinement tree, and a
// few deep jobs (edge- and vertex-touching pairs refine towards the shared
// edge to depth ~20) set the time of the launch.  Here the trees of all
// jobs grow one level per launch: every node of the level is one warp (the
// same low / high rules and decisions as the reference's recursion), accepted
// nodes keep `high`, refined nodes append their two children to the next
// level.  The value is then formed bottom-up exactly as the recursion returns
// it, value(node) = value(left) + value(right) (quadrature.c:936-937), and a
// top-down pass numbers the nodes in depth-first order to write the decision
// trace the reuse replay reads.  The critical path is the tree depth
// (<= 24 levels) instead of the largest tree's node count.
struct LevelJob {
    TriPot inner;
    int order;
    int slot;  // r * 8 + t * 2 + d
    int rec;   // record (marginal flags)
};

struct LevelNode {
    double v[9];
    double tol;
    double val;
    int job;    // index into the chunk's LevelJob array
    int depth;
    int child;  // first child (left; right = child + 1) or -1
    int size;   // nodes in the subtree
    int pos;    // depth-first position in the job's tree
    int edge;   // bisected edge of a refined node
};

struct LevelArgs {
    const double *corner;
    const NearRec *rec;
    const int *job_rec;
    long long job0, njob;  // jobs [job0, job0 + njob) of the launch's job numbering
    int orders[4];
    double *slot;
    int *kind;
    int *marginal;
    unsigned char *trace;  // [jobs * kTraceCap] or null
    int *trace_len;
    LevelJob *jobs;        // [njob]
    LevelNode *pool;
    int *count;            // nodes appended to the next level
    int *overflow;
    unsigned long long *evals;
};

// One thread per job: zero-area and identical-triangle jobs are finished
// here (as in k_near_eval); adaptive jobs get their root node.
__global__ void k_level_init(LevelArgs A, int base0, int cap) {
    long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= A.njob) return;
    const long long job = A.job0 + g;
    int r = (int)(job >> 3), t = (int)((job >> 1) & 3), d = (int)(job & 1);
    if (A.job_rec) r = A.job_rec[r];
    NearRec rec = A.rec[r];
    double ta[9], tb[9];
    patch_triangle(A.corner + 12 * (size_t)rec.i, t >> 1, ta);
    patch_triangle(A.corner + 12 * (size_t)rec.j, t & 1, tb);
    const double *outer = d == 0 ? ta : tb, *inner = d == 0 ? tb : ta;
    LevelJob &J = A.jobs[g];
    TriPot po;
    tri_prepare(outer, po);
    tri_prepare(inner, J.inner);
    J.slot = r * 8 + t * 2 + d;
    J.rec = r;
    int kind;
    if (po.twice_area == 0.0 || J.inner.twice_area == 0.0) {
        kind = 1;
        A.slot[J.slot] = 0.0;
    } else {
        bool identical = true;
        for (int m = 0; m < 3; ++m) {
            bool hit = false;
            for (int q = 0; q < 3; ++q)
                if (same_point(ta + 3 * m, tb + 3 * q)) hit = true;
            if (!hit) identical = false;
        }
        if (identical) {
            kind = 2;
            double s = 0.0;
            for (int m = 0; m < 3; ++m) s += tri_potential(J.inner, outer + 3 * m);
            A.slot[J.slot] = po.twice_area * s / 3.0;
            atomicAdd(A.evals, 3ull);
        } else {
            kind = 0;
            int order = rec.cls == CLS_SELF ? A.orders[3] : rec.cls == CLS_TOUCHING ? A.orders[2] : A.orders[1];
            if (order < 6) order = 6;
            J.order = order;
            double aa = d == 0 ? po.twice_area : J.inner.twice_area;
            double ab = d == 0 ? J.inner.twice_area : po.twice_area;
            double scale = aa * ab / sqrt(fmax(aa, ab));
            int at = atomicAdd(A.count, 1);
            if (at >= cap) {
                atomicExch(A.overflow, 1);
            } else {
                LevelNode &nd = A.pool[base0 + at];
                for (int k = 0; k < 9; ++k) nd.v[k] = outer[k];
                nd.tol = 2e-5 * scale;
                nd.job = (int)g;
                nd.depth = 0;
                nd.child = -1;
                nd.pos = 0;
            }
        }
    }
    if (d == 0) A.kind[(size_t)r * 4 + t] = kind;
    if (kind != 0 && A.trace_len) A.trace_len[job] = 0;
}

// One warp per node of one level.
__global__ void __launch_bounds__(256, 2) k_level_eval(LevelArgs A, int base, int n, int next_base, int cap) {
    __shared__ TriPot s_inner[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long w = blockIdx.x * 8ll + warp;
    if (w >= n) return;
    LevelNode &nd = A.pool[base + w];
    const LevelJob &J = A.jobs[nd.job];
    TriPot &inner = s_inner[warp];
    {
        const double *src = reinterpret_cast<const double *>(&J.inner);
        double *dst = reinterpret_cast<double *>(&inner);
        for (int k = lane; k < (int)(sizeof(TriPot) / sizeof(double)); k += 32) dst[k] = src[k];
    }
    double v[9];
    for (int k = 0; k < 9; ++k) v[k] = nd.v[k];
    const double tol = nd.tol;
    const int depth = nd.depth, order = J.order;
    __syncwarp();
    const int ql = order <= 6 ? 3 : 4;
    const int rl = gl_row(ql), rh = gl_row(order);
    const int nlo = ql * ql, ntot = nlo + order * order;
    double lo = 0.0, hi = 0.0;
    for (int k = lane; k < ntot; k += 32) {
        int ord, row, idx;
        if (k < nlo) {
            ord = ql;
            row = rl;
            idx = k;
        } else {
            ord = order;
            row = rh;
            idx = k - nlo;
        }
        int i = idx / ord, j = idx % ord;
        double xi = c_gl_x[row][i], xj = c_gl_x[row][j];
        double wi = c_gl_w[row][i], wj = c_gl_w[row][j];
        double r[3], jac;
        tri_map(v, v + 3, v + 6, 0.5 * (xi + 1.0), 0.5 * (xj + 1.0), r, &jac);
        double val = 0.25 * wi * wj * jac * tri_potential(inner, r);
        if (k < nlo)
            lo += val;
        else
            hi += val;
    }
    lo = warp_sum(lo);
    hi = warp_sum(hi);
    if (lane != 0) return;
    atomicAdd(A.evals, (unsigned long long)ntot);
    nd.child = -1;
    if (!isfinite(lo) || !isfinite(hi)) {
        nd.val = nan("");
        return;
    }
    int mflags = 0;
    double thr = tol + 2e-5 * fabs(hi), gap = fabs(hi - lo);
    if (fabs(gap - thr) <= 1e-6 * thr) mflags |= MARG_THRESHOLD;
    if (gap <= thr) {
        nd.val = hi;
    } else if (depth >= 24) {
        nd.val = nan("");  // quadrature.c:922
    } else {
        int e = 0;
        double longest = 0.0, len[3];
        for (int i = 0; i < 3; ++i) {
            double sl = dist3(v + 3 * i, v + 3 * ((i + 1) % 3));
            len[i] = sl;
            if (sl > longest) {
                longest = sl;
                e = i;
            }
        }
        for (int i = 0; i < 3; ++i)
            if (i != e && len[i] >= longest * (1.0 - 1e-10)) mflags |= MARG_TIE;
        nd.edge = e;
        int at = atomicAdd(A.count, 2);
        if (at + 2 > cap) {
            atomicExch(A.overflow, 1);
            nd.val = nan("");
        } else {
            nd.child = next_base + at;
            LevelNode &left = A.pool[next_base + at], &right = A.pool[next_base + at + 1];
            int j = (e + 1) % 3, k = (e + 2) % 3;
            for (int dd = 0; dd < 3; ++dd) {
                double mid = 0.5 * (v[3 * e + dd] + v[3 * j + dd]);
                left.v[dd] = v[3 * e + dd];
                left.v[3 + dd] = mid;
                left.v[6 + dd] = v[3 * k + dd];
                right.v[dd] = mid;
                right.v[3 + dd] = v[3 * j + dd];
                right.v[6 + dd] = v[3 * k + dd];
            }
            left.tol = right.tol = tol * 0.5;
            left.depth = right.depth = depth + 1;
            left.job = right.job = nd.job;
            left.child = right.child = -1;
        }
    }
    if (mflags && A.marginal) atomicOr(A.marginal + J.rec, mflags);
}

// value(node) = value(left) + value(right); subtree sizes
__global__ void k_level_up(LevelNode *pool, int base, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    LevelNode &nd = pool[base + i];
    if (nd.child >= 0) {
        const LevelNode &l = pool[nd.child], &r = pool[nd.child + 1];
        nd.val = l.val + r.val;
        nd.size = 1 + l.size + r.size;
    } else {
        nd.size = 1;
    }
}

// depth-first positions of the children; the decision trace
__global__ void k_level_down(LevelArgs A, int base, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const LevelNode &nd = A.pool[base + i];
    if (A.trace && nd.pos < kTraceCap)
        A.trace[(size_t)(A.job0 + nd.job) * kTraceCap + nd.pos] = nd.child >= 0 ? (unsigned char)nd.edge : kAccept;
    if (nd.child >= 0) {
        LevelNode &l = A.pool[nd.child], &r = A.pool[nd.child + 1];
        l.pos = nd.pos + 1;
        r.pos = nd.pos + 1 + l.size;
    }
}

// roots: the job's value, trace length, full-trace flag
__global__ void k_level_roots(LevelArgs A, int base, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const LevelNode &nd = A.pool[base + i];
    const LevelJob &J = A.jobs[nd.job];
    A.slot[J.slot] = nd.val;
    if (A.trace_len) A.trace_len[A.job0 + nd.job] = nd.size < kTraceCap ? nd.size : kTraceCap;
    if (A.marginal && A.trace && nd.size > kTraceCap) atomicOr(A.marginal + J.rec, MARG_TRACE_FULL);
}

// PEEC_GB300_NEAR_LEVELS=0 keeps the depth-first warp form (k_near_eval).
static bool near_levels_enabled() {
    static const bool on = [] {
        const char *e = getenv("PEEC_GB300_NEAR_LEVELS");
        return !(e && strcmp(e, "0") == 0);
    }();
    return on;
}

// All 8 jobs of the first nrec records of E's list, level by level, in
// chunks whose trees fit the node pool (a chunk that overflows is retried
// with half the jobs).
static bool near_eval_levels(const NearEvalArgs &E, int nrec) {
    static const int kPoolNodes = 1 << 21;
    const long long total = (long long)nrec * 8;
    if (total == 0) return true;
    long long chunk = total < (1 << 16) ? total : (1 << 16);
    DBuf<LevelNode> pool(kPoolNodes);
    DBuf<LevelJob> jobs((size_t)chunk);
    DBuf<int> cnt(1), ovf(1);
    if (!pool.p || !jobs.p || !cnt.p || !ovf.p) return false;
    LevelArgs L;
    L.corner = E.corner;
    L.rec = E.rec;
    L.job_rec = E.job_rec;
    for (int k = 0; k < 4; ++k) L.orders[k] = E.orders[k];
    L.slot = E.slot;
    L.kind = E.kind;
    L.marginal = E.marginal;
    L.trace = E.trace;
    L.trace_len = E.trace_len;
    L.jobs = jobs.p;
    L.pool = pool.p;
    L.count = cnt.p;
    L.overflow = ovf.p;
    L.evals = E.evals;
    std::vector<int> base, cnt_l;
    for (long long job0 = 0; job0 < total;) {
        const long long nj = std::min(chunk, total - job0);
        L.job0 = job0;
        L.njob = nj;
        base.assign(1, 0);
        cnt_l.clear();
        int h[2] = {0, 0};
        cudaMemsetAsync(cnt.p, 0, sizeof(int), stream());
        cudaMemsetAsync(ovf.p, 0, sizeof(int), stream());
        PEEC_LAUNCH(k_level_init, (unsigned)((nj + 127) / 128), 128, 0, L, 0, kPoolNodes);
        cudaMemcpyAsync(&h[0], cnt.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
        cudaMemcpyAsync(&h[1], ovf.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
        if (!sync("near-field roots")) return false;
        bool overflow = h[1] != 0;
        cnt_l.push_back(h[0]);
        while (!overflow && cnt_l.back() > 0) {
            const int lv = (int)cnt_l.size() - 1;
            const int next_base = base[lv] + cnt_l[lv];
            cudaMemsetAsync(cnt.p, 0, sizeof(int), stream());
            PEEC_LAUNCH(k_level_eval, (unsigned)((cnt_l[lv] + 7) / 8), 256, 0, L, base[lv], cnt_l[lv], next_base,
                        kPoolNodes - next_base);
            cudaMemcpyAsync(&h[0], cnt.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
            cudaMemcpyAsync(&h[1], ovf.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
            if (!sync("near-field level")) return false;
            overflow = h[1] != 0;
            base.push_back(next_base);
            cnt_l.push_back(h[0]);
        }
        if (overflow) {
            if (nj == 1) {
                set_error("near-field quadrature: one refinement tree exceeds %d nodes", kPoolNodes);
                return false;
            }
            chunk = (nj + 1) / 2;
            continue;
        }
        const int levels = (int)cnt_l.size() - 1;  // the last level is empty
        for (int lv = levels - 1; lv >= 0; --lv)
            PEEC_LAUNCH(k_level_up, (unsigned)((cnt_l[lv] + 255) / 256), 256, 0, pool.p, base[lv], cnt_l[lv]);
        for (int lv = 0; lv < levels; ++lv)
            PEEC_LAUNCH(k_level_down, (unsigned)((cnt_l[lv] + 255) / 256), 256, 0, L, base[lv], cnt_l[lv]);
        if (cnt_l[0] > 0) PEEC_LAUNCH(k_level_roots, (unsigned)((cnt_l[0] + 255) / 256), 256, 0, L, base[0], cnt_l[0]);
        if (!launch_ok("near-field levels")) return false;
        job0 += nj;
    }
    return true;
}

// ---------------------------------------------------------------------
// 5b. reuse of translated near pairs
//
// The near-pair integral depends only on the two patches' corners relative
// to each other.  On meshes with repeated cells most near pairs are
// translated copies of a few hundred configurations (5 cm box: 56 k P pairs,
// 251 distinct; 69 k Lp pairs, 318 distinct).  Each record gets a key: its
// 21 corner offsets relative to corner 0 of patch i, quantised to delta (a
// few ulps of the largest coordinate, so copies that differ only by rounding
// share a key), plus its class and same-object flag.  Records with equal
// keys share one evaluation: the representative is the lowest record index
// of the group (deterministic), and a full-key comparison guards against
// hash collisions.  Copies differ from their representative by at most
// delta in each offset, far below the parity tolerance.
// ---------------------------------------------------------------------
static const int kKeyLen = 21;

// strided int fill (used to initialise the representative field of the table)
__global__ void k_fill_int(int *base, long long count, int stride_ints, int value) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < count) base[t * stride_ints] = value;
}

struct MemoSlot {
    unsigned long long hash;  // 0 = empty
    int rep;
    int pad;
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long h, unsigned long long v) {
    h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    h *= 0xff51afd7ed558ccdull;
    return h ^ (h >> 29);
}

// keys[r*22]: 21 quantised offsets + (cls | same_object << 8); ok[r] = 0 if
// an offset does not fit the quantisation range (the record is then never
// shared)
__global__ void k_memo_keys(const double *corner, const int *same_obj, const NearRec *rec, int nrec, double delta,
                            long long *keys, unsigned long long *hash, int *ok) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    NearRec q = rec[r];
    const double *ci = corner + 12 * (size_t)q.i, *cj = corner + 12 * (size_t)q.j;
    long long *key = keys + (size_t)r * (kKeyLen + 1);
    unsigned long long h = 0x1234567ull;
    int good = 1;
    for (int t = 0; t < kKeyLen; ++t) {
        double v = t < 9 ? ci[3 + t] - ci[t % 3] : cj[t - 9] - ci[(t - 9) % 3];
        double qv = rint(v / delta);
        if (!(fabs(qv) < 9.0e15)) {
            good = 0;
            qv = 0.0;
        }
        key[t] = (long long)qv;
        h = mix64(h, (unsigned long long)key[t]);
    }
    long long tag = (long long)q.cls | ((long long)(same_obj[q.i] == same_obj[q.j]) << 8);
    key[kKeyLen] = tag;
    h = mix64(h, (unsigned long long)tag);
    hash[r] = h | 1ull;
    ok[r] = good;
}

__global__ void k_memo_insert(int nrec, const unsigned long long *hash, const int *ok, MemoSlot *tab,
                              unsigned long long mask, int *slot_of) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    if (!ok[r]) {
        slot_of[r] = -1;
        return;
    }
    unsigned long long h = hash[r], s = h & mask;
    for (unsigned long long probe = 0; probe <= mask; ++probe) {  // bounded: the table is never full
        unsigned long long prev = atomicCAS(&tab[s].hash, 0ull, h);
        if (prev == 0ull || prev == h) {
            atomicMin(&tab[s].rep, r);
            slot_of[r] = (int)s;
            return;
        }
        s = (s + 1) & mask;
    }
    slot_of[r] = -1;
}

// rep[r] = representative record; is_rep[r] = 1 for representatives
__global__ void k_memo_resolve(int nrec, const long long *keys, const MemoSlot *tab, const int *slot_of, int *rep,
                               int *is_rep) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    int rr = r;
    if (slot_of[r] >= 0) {
        int r0 = tab[slot_of[r]].rep;
        if (r0 != r) {
            const long long *a = keys + (size_t)r * (kKeyLen + 1), *b = keys + (size_t)r0 * (kKeyLen + 1);
            bool same = true;
            for (int t = 0; t <= kKeyLen; ++t)
                if (a[t] != b[t]) same = false;
            if (same) rr = r0;
        }
    }
    rep[r] = rr;
    is_rep[r] = rr == r;
}

__global__ void k_memo_compact(int nrec, const int *is_rep, const int *off, int *list) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec || !is_rep[r]) return;
    list[off[r]] = r;
}

// ---- multi-round reuse ------------------------------------------------
// A copy whose replay of its representative's trace fails takes the
// representative's value only if it follows the same subdivision tree, so
// copies that fail are regrouped by (representative, first divergence:
// job, trace position, the copy's own edge choice); each new group's
// lowest record is integrated with traces on, and the remaining members
// replay against it -- a few rounds settle almost every tie pattern, and
// what is left is integrated directly.  src[r] is the record whose value r
// takes (r itself when integrated).
static const int kNoFail = 0x7fffffff;

// copies whose representative was integrated in this round: classify
__global__ void k_round_classify(int nrec, const int *rep, const int *rep_pos, const int *marginal, int *src,
                                 int *eval, int *replay, int *fcode) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    replay[r] = 0;
    if (src[r] >= 0) return;  // decided (a representative or an earlier round)
    int r0 = rep[r];
    if (r0 == r || rep_pos[r0] < 0) return;  // representative not integrated in this round
    int m = marginal[r0];
    if (m & (MARG_THRESHOLD | MARG_TRACE_FULL)) {
        src[r] = r;
        eval[r] = 1;
    } else if (!(m & MARG_TIE)) {
        src[r] = r0;
    } else {
        replay[r] = 1;
        fcode[r] = kNoFail;
    }
}

// replay of the representative's trace per (record, job); the first
// divergence (lowest job, then trace position) goes to fcode
__global__ void k_round_replay(int nrec, const int *rep, const int *rep_pos, const int *replay, const double *corner,
                               const NearRec *rec, const unsigned char *trace, const int *trace_len, int *fcode) {
    long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= (long long)nrec * 8) return;
    int r = (int)(g >> 3), jb = (int)(g & 7), t = jb >> 1, d = jb & 1;
    if (!replay[r]) return;
    int r0 = rep[r];
    long long job = (long long)rep_pos[r0] * 8 + jb;
    int len = trace_len[job];
    if (len <= 0) return;  // zero-area or identical triangles: no subdivision
    const unsigned char *tr = trace + (size_t)job * kTraceCap;
    NearRec q = rec[r];
    double ta[9], tb[9];
    patch_triangle(corner + 12 * (size_t)q.i, t >> 1, ta);
    patch_triangle(corner + 12 * (size_t)q.j, t & 1, tb);
    double stack[kStackCap][9];
    for (int k = 0; k < 9; ++k) stack[0][k] = d == 0 ? ta[k] : tb[k];
    int sp = 1, pos = 0, code = kNoFail;
    while (sp > 0) {
        double v[9];
        --sp;
        for (int k = 0; k < 9; ++k) v[k] = stack[sp][k];
        if (pos >= len) {
            code = (jb << 12) | (pos << 2) | 3;
            break;
        }
        unsigned char c = tr[pos];
        if (c == kAccept) {
            ++pos;
            continue;
        }
        int e = 0;
        double longest = 0.0;
        for (int i = 0; i < 3; ++i) {
            double sl = dist3(v + 3 * i, v + 3 * ((i + 1) % 3));
            if (sl > longest) {
                longest = sl;
                e = i;
            }
        }
        if (e != (int)c || sp + 2 > kStackCap) {
            code = (jb << 12) | (pos << 2) | (e & 3);
            break;
        }
        ++pos;
        int j = (e + 1) % 3, k = (e + 2) % 3;
        double *left = stack[sp + 1], *right = stack[sp];
        for (int dd = 0; dd < 3; ++dd) {
            double mid = 0.5 * (v[3 * e + dd] + v[3 * j + dd]);
            left[dd] = v[3 * e + dd];
            left[3 + dd] = mid;
            left[6 + dd] = v[3 * k + dd];
            right[dd] = mid;
            right[3 + dd] = v[3 * j + dd];
            right[6 + dd] = v[3 * k + dd];
        }
        sp += 2;
    }
    if (code == kNoFail && pos != len) code = (jb << 12) | (pos << 2) | 3;
    if (code != kNoFail) atomicMin(fcode + r, code);
}

// after the replay: reuse, or join a new group keyed by (rep, fcode)
__global__ void k_round_regroup(int nrec, const int *replay, const int *fcode, const int *rep, int *src, int *failed,
                                unsigned long long *key) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    failed[r] = 0;
    if (!replay[r]) return;
    if (fcode[r] == kNoFail) {
        src[r] = rep[r];
        return;
    }
    failed[r] = 1;
    key[r] = ((unsigned long long)(unsigned)rep[r] << 32) | (unsigned)fcode[r];
}

// exact-key hash insert of the failed records: lowest record per key
struct RoundSlot {
    unsigned long long key;  // ~0 = empty
    int rep;
    int pad;
};
__global__ void k_round_insert(int nrec, const int *failed, const unsigned long long *key, RoundSlot *tab,
                               unsigned long long mask, int *slot_of) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec || !failed[r]) return;
    unsigned long long kk = key[r], s = mix64(0x51ull, kk) & mask;
    for (unsigned long long probe = 0; probe <= mask; ++probe) {  // bounded: the table is never full
        unsigned long long prev = atomicCAS(&tab[s].key, ~0ull, kk);
        if (prev == ~0ull || prev == kk) {
            atomicMin(&tab[s].rep, r);
            slot_of[r] = (int)s;
            return;
        }
        s = (s + 1) & mask;
    }
    slot_of[r] = -1;
}

// new representatives of the failed records (integrated next, src = self)
__global__ void k_round_resolve(int nrec, const int *failed, const RoundSlot *tab, const int *slot_of, int *rep,
                                int *src, int *is_new, int *eval) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    is_new[r] = 0;
    if (!failed[r]) return;
    if (slot_of[r] < 0) {  // (cannot happen: the table has 4x the records) integrate directly
        src[r] = r;
        eval[r] = 1;
        return;
    }
    int r0 = tab[slot_of[r]].rep;
    rep[r] = r0;
    if (r0 == r) {
        src[r] = r;
        is_new[r] = 1;
    }
}

// representatives integrated in the first reuse pass take their own value
__global__ void k_round_self(int nrec, const int *rep_pos, int *src) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec && rep_pos[r] >= 0) src[r] = r;
}

__global__ void k_round_fail_to_eval(int nrec, const int *failed, int *src, int *eval) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec || !failed[r]) return;
    src[r] = r;
    eval[r] = 1;
}

__global__ void k_round_scatter(int nrec, const int *src, double2 *kval) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    int s = src[r];
    if (s >= 0 && s != r) kval[r] = kval[s];
}

__global__ void k_round_positions(const int *list, int n, int *pos) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pos[list[i]] = i;
}

// ---------------------------------------------------------------------
// 6. tiled assembly
// ---------------------------------------------------------------------
struct TileArgs {
    RegionsDev R;
    int kind;
    double dir_tol;
    const FarPt *pts;
    const FarPtF *ptf;
    int npts;
    int far_df;  // 1: double-float far rule, 0: FP64, 2: FP32
    const int *near_off;
    const NearRec *near_rec;
    const double2 *near_k;
    double *out;  // n*n row-major
    int n;
    int only_a, only_b;
    unsigned long long *err;  // min over failing entries of a*n+b; ~0ull = none
};

static const int kTile = 32;
static const int kTileWarps = 8;

// far-rule integral of one patch pair, all 4 triangle pairs at once:
// sum_p W_p sum_q W_q / |r_p - r_q| over the 2q^2 points of each patch
// (reference quadrature.c:679-783 sums the same products per triangle pair).
// FP64 form: kept for comparison runs (PEEC_GB300_FAR=fp64).
__device__ __forceinline__ double far_pair_fp64(const FarPt *pa, const FarPt *pb, int npts) {
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int p = lane; p < npts; p += 32) {
        FarPt A = pa[p];
        double s = 0.0;
#pragma unroll 4
        for (int q = 0; q < npts; ++q) {
            FarPt B = pb[q];
            double dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
            double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
            if (!(r2 <= 0.0)) s = fma(B.w, rsqrt(r2), s);  // NaN propagates, as the reference's R <= 0 test
        }
        acc = fma(A.w, s, acc);
    }
    return warp_sum(acc);
}

// ---- double-float arithmetic (Dekker / Knuth error-free transforms) ----
// The library is built without implicit FMA contraction, so a + b and a * b
// below round exactly as written; fmaf() is explicit.
struct f2 {
    float h, l;
};
__device__ __forceinline__ f2 two_sum(float a, float b) {
    float s = a + b, v = s - a;
    return f2{s, (a - (s - v)) + (b - v)};
}
__device__ __forceinline__ f2 quick_two_sum(float a, float b) {  // |a| >= |b|
    float s = a + b;
    return f2{s, b - (s - a)};
}
__device__ __forceinline__ f2 df_sub(f2 a, f2 b) {
    f2 s = two_sum(a.h, -b.h);
    return quick_two_sum(s.h, s.l + (a.l - b.l));
}
__device__ __forceinline__ f2 df_add(f2 a, f2 b) {
    f2 s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, s.l + (a.l + b.l));
}
__device__ __forceinline__ f2 df_sqr(f2 a) {
    float p = a.h * a.h;
    float e = fmaf(a.h, a.h, -p);
    e = fmaf(a.h + a.h, a.l, e);
    return quick_two_sum(p, e);
}
__device__ __forceinline__ f2 df_mul(f2 a, f2 b) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return quick_two_sum(p, e);
}
// The hardware reciprocal square root as one instruction: rsqrtf() wraps it
// in a rescaling for subnormal inputs, which the far rule never sees (a FAR
// point pair is at least near_factor patch sizes apart) and which would
// otherwise add ~5 instructions to a loop body of 9.  Subnormal inputs
// flush to zero (result +inf, which the entry's finiteness check reports).
__device__ __forceinline__ float rsqrt_hw(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1/sqrt(x) for x > 0 to ~1e-14 relative: hardware rsqrtf seed y, residual
// r = 1 - x y^2 in double-float, one Halley step y (1 + r/2 + 3 r^2 / 8)
// (third-order convergence from the 2^-22 seed).
__device__ __forceinline__ f2 df_rsqrt(f2 x) {
    float y = rsqrt_hw(x.h);
    float yy = y * y;
    f2 y2 = f2{yy, fmaf(y, y, -yy)};
    f2 t = df_mul(x, y2);
    float r = (1.0f - t.h) - t.l;
    float c = y * fmaf(0.375f * r, r, 0.5f * r);
    return quick_two_sum(y, c);
}

// FP32 form accumulating into this lane's running double-float sum `acc`
// (reduced across the warp once per entry): each lane's point sum over the
// partner patch is FP32; adding it into a (hi, lo) pair keeps the entry's
// sum of ~16 k products at FP32 accuracy.  NaN propagates into `acc`.
__device__ __forceinline__ void far_pair_f32_acc(const FarPtF *pa, const FarPtF *pb, int npts, f2 &acc) {
    // The reference skips R <= 0; two FAR patches of nonzero size are apart
    // (their boxes have a positive gap), so no point pair coincides and the
    // loop needs no test (patches of zero size are skipped by the caller:
    // their weights are all zero).  NaN still propagates through rsqrt.
    const int lane = threadIdx.x & 31;
    for (int p = lane; p < npts; p += 32) {
        const float4 A = *reinterpret_cast<const float4 *>(pa + p);  // xh, yh, zh, wh
        float s0 = 0.0f, s1 = 0.0f;
        int q = 0;
        for (; q + 1 < npts; q += 2) {
            const float4 B0 = *reinterpret_cast<const float4 *>(pb + q);
            const float4 B1 = *reinterpret_cast<const float4 *>(pb + q + 1);
            float dx = A.x - B0.x, dy = A.y - B0.y, dz = A.z - B0.z;
            s0 = fmaf(B0.w, rsqrt_hw(fmaf(dz, dz, fmaf(dy, dy, dx * dx))), s0);
            dx = A.x - B1.x;
            dy = A.y - B1.y;
            dz = A.z - B1.z;
            s1 = fmaf(B1.w, rsqrt_hw(fmaf(dz, dz, fmaf(dy, dy, dx * dx))), s1);
        }
        if (q < npts) {
            const float4 B0 = *reinterpret_cast<const float4 *>(pb + q);
            const float dx = A.x - B0.x, dy = A.y - B0.y, dz = A.z - B0.z;
            s0 = fmaf(B0.w, rsqrt_hw(fmaf(dz, dz, fmaf(dy, dy, dx * dx))), s0);
        }
        acc = df_add(acc, two_sum(A.w * s0, A.w * s1));
    }
}

// The FP32 form at the far order 4 (32 points a patch, one per lane), in
// coordinates local to the pair: with O = the first point of patch A (its
// float pair), a = A - O and b = B - O are formed from the float pairs (so
// they carry FP32 accuracy relative to the patch size and the distance, not
// to the absolute position), and R^2 = |a|^2 + |b|^2 - 2 a.b takes one add
// and three FMAs per point pair.  Its rounding stays a few units of 2^-24 of
// (|a| + |b|)^2 <= (R + 2h)^2, i.e. below 1.5e-6 of R^2 at the closest FAR
// pairs (R >= near_factor h with the default 0.5) -- the absolute-coordinate
// form it replaces rounded each difference to 2^-24 of the coordinate.
// Lane q prepares (b, |b|^2) and the weight of partner point q in the warp's
// shared slot; every lane then reads them as broadcasts.
__device__ __forceinline__ void far_pair_f32_acc32(const FarPtF *pa, const FarPtF *pb, float4 *slot, f2 &acc) {
    const int lane = threadIdx.x & 31;
    const FarPtF A = pa[lane];
    const FarPtF B = pb[lane];
    const float oxh = __shfl_sync(0xffffffffu, A.xh, 0), oxl = __shfl_sync(0xffffffffu, A.xl, 0);
    const float oyh = __shfl_sync(0xffffffffu, A.yh, 0), oyl = __shfl_sync(0xffffffffu, A.yl, 0);
    const float ozh = __shfl_sync(0xffffffffu, A.zh, 0), ozl = __shfl_sync(0xffffffffu, A.zl, 0);
    const float bx = (B.xh - oxh) + (B.xl - oxl), by = (B.yh - oyh) + (B.yl - oyl), bz = (B.zh - ozh) + (B.zl - ozl);
    const float ax = (A.xh - oxh) + (A.xl - oxl), ay = (A.yh - oyh) + (A.yl - oyl), az = (A.zh - ozh) + (A.zl - ozl);
    const float a2 = fmaf(az, az, fmaf(ay, ay, ax * ax));
    const float mx = -2.0f * ax, my = -2.0f * ay, mz = -2.0f * az;
    __syncwarp();  // the slot's previous partner is read by every lane
    slot[lane] = make_float4(bx, by, bz, fmaf(bz, bz, fmaf(by, by, bx * bx)));
    reinterpret_cast<float *>(slot + 32)[lane] = B.wh;
    __syncwarp();
    float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int q4 = 0; q4 < 8; ++q4) {
        const float4 w = slot[32 + q4];
        const float ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float4 b = slot[4 * q4 + u];
            const float r2 = fmaf(mz, b.z, fmaf(my, b.y, fmaf(mx, b.x, a2 + b.w)));
            s[u] = fmaf(ws[u], rsqrt_hw(r2), s[u]);
        }
    }
    acc = df_add(acc, two_sum(A.wh * (s[0] + s[1]), A.wh * (s[2] + s[3])));
}

// The FP32 far rule of a whole entry at the far order 4 (regions of at most
// four patches a side), after its near pairs: farmask bit 4 ii + jj marks the
// far patch pair (off[a] + ii, off[b] + jj).  One origin O for the entry (the
// first point of the entry's first A patch) lets every partner patch be
// staged once per entry and every A point be prepared once per A patch; the
// point loop is far_pair_f32_acc32's.  With |a| below the region size s and
// R >= near_factor s_patch, the rounding of R^2 stays below ~3e-6 of R^2 at
// the closest FAR pairs (typically 1e-7).  slot: 4 x 40 float4 of the warp.
__device__ __forceinline__ void far_entry_f32(const FarPtF *ptf, int i0, int ni, int j0, int nj, unsigned farmask,
                                              float4 *slot, f2 &acc) {
    const int lane = threadIdx.x & 31;
    const FarPtF O = ptf[(size_t)i0 * 32];  // the same address in every lane: one broadcast load
    __syncwarp();  // the previous entry's partner points are read by every lane
    for (int jj = 0; jj < nj; ++jj) {
        if (!((farmask >> jj) & 0x1111u)) continue;  // no far pair with this partner patch
        const FarPtF B = ptf[(size_t)(j0 + jj) * 32 + lane];
        const float bx = (B.xh - O.xh) + (B.xl - O.xl), by = (B.yh - O.yh) + (B.yl - O.yl),
                    bz = (B.zh - O.zh) + (B.zl - O.zl);
        slot[40 * jj + lane] = make_float4(bx, by, bz, fmaf(bz, bz, fmaf(by, by, bx * bx)));
        reinterpret_cast<float *>(slot + 40 * jj + 32)[lane] = B.wh;
    }
    __syncwarp();
    for (int ii = 0; ii < ni; ++ii) {
        const unsigned row = (farmask >> (4 * ii)) & 0xFu;
        if (!row) continue;
        const FarPtF A = ptf[(size_t)(i0 + ii) * 32 + lane];
        const float ax = (A.xh - O.xh) + (A.xl - O.xl), ay = (A.yh - O.yh) + (A.yl - O.yl),
                    az = (A.zh - O.zh) + (A.zl - O.zl);
        const float a2 = fmaf(az, az, fmaf(ay, ay, ax * ax));
        const float mx = -2.0f * ax, my = -2.0f * ay, mz = -2.0f * az;
        for (int jj = 0; jj < nj; ++jj) {
            if (!((row >> jj) & 1u)) continue;
            const float4 *bs = slot + 40 * jj;
            float s4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int q4 = 0; q4 < 8; ++q4) {
                const float4 w = bs[32 + q4];
                const float ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4 b = bs[4 * q4 + u];
                    const float r2 = fmaf(mz, b.z, fmaf(my, b.y, fmaf(mx, b.x, a2 + b.w)));
                    s4[u] = fmaf(ws[u], rsqrt_hw(r2), s4[u]);
                }
            }
            acc = df_add(acc, two_sum(A.wh * (s4[0] + s4[1]), A.wh * (s4[2] + s4[3])));
        }
    }
}

// The double-float form at the far order 4, with the partner's points
// staged in the warp's shared slot (two float4 a point) as above.
__device__ __forceinline__ void far_pair_df_acc32(const FarPtF *pa, const FarPtF *pb, float4 *slot, f2 &acc) {
    const int lane = threadIdx.x & 31;
    const FarPtF A = pa[lane];
    const float4 *pbv = reinterpret_cast<const float4 *>(pb);
    const float4 b0 = pbv[lane], b1 = pbv[32 + lane];
    __syncwarp();
    slot[lane] = b0;
    slot[32 + lane] = b1;
    __syncwarp();
    const f2 ax = {A.xh, A.xl}, ay = {A.yh, A.yl}, az = {A.zh, A.zl};
    f2 s0 = {0.0f, 0.0f}, s1 = {0.0f, 0.0f};
#pragma unroll 4
    for (int q = 0; q < 32; ++q) {
        // point q: float4 2q (xh, yh, zh, wh) and 2q + 1 (xl, yl, zl, wl)
        const float4 h = slot[2 * q], l = slot[2 * q + 1];
        const f2 dx = df_sub(ax, f2{h.x, l.x});
        const f2 dy = df_sub(ay, f2{h.y, l.y});
        const f2 dz = df_sub(az, f2{h.z, l.z});
        const f2 r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
        const f2 t = df_mul(f2{h.w, l.w}, df_rsqrt(r2));
        if (q & 1)
            s1 = df_add(s1, t);
        else
            s0 = df_add(s0, t);
    }
    acc = df_add(acc, df_mul(f2{A.wh, A.wl}, df_add(s0, s1)));
}

// Double-float form, accumulating into this lane's running sum `acc` (the
// entry's far part is reduced across lanes once, after all its patch pairs):
// every point difference, square, the reciprocal square root and the sums
// carry ~48 significant bits on the FP32 pipes; two independent partial sums
// per lane keep the dependent add chains short.  A NaN propagates into `acc`.
__device__ __forceinline__ void far_pair_df_acc(const FarPtF *pa, const FarPtF *pb, int npts, f2 &acc) {
    const int lane = threadIdx.x & 31;
    for (int p = lane; p < npts; p += 32) {
        FarPtF A = pa[p];
        f2 ax = {A.xh, A.xl}, ay = {A.yh, A.yl}, az = {A.zh, A.zl};
        f2 s0 = {0.0f, 0.0f}, s1 = {0.0f, 0.0f};
        for (int q = 0; q < npts; q += 2) {
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (q + u >= npts) break;
                FarPtF B = pb[q + u];
                f2 dx = df_sub(ax, f2{B.xh, B.xl});
                f2 dy = df_sub(ay, f2{B.yh, B.yl});
                f2 dz = df_sub(az, f2{B.zh, B.zl});
                // no R <= 0 test: FAR patches of nonzero size never share a
                // point (the caller skips zero-size patches, whose weights are
                // zero), and a NaN reaches the entry's sum, which the epilogue
                // checks
                f2 r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
                f2 t = df_mul(f2{B.wh, B.wl}, df_rsqrt(r2));
                if (u == 0)
                    s0 = df_add(s0, t);
                else
                    s1 = df_add(s1, t);
            }
        }
        acc = df_add(acc, df_mul(f2{A.wh, A.wl}, df_add(s0, s1)));
    }
}

__device__ __forceinline__ f2 warp_sum_df2(f2 v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        f2 o = {__shfl_xor_sync(0xffffffffu, v.h, m), __shfl_xor_sync(0xffffffffu, v.l, m)};
        v = df_add(v, o);
    }
    return v;
}

__device__ __forceinline__ double warp_sum_df(f2 v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        f2 o = {__shfl_xor_sync(0xffffffffu, v.h, m), __shfl_xor_sync(0xffffffffu, v.l, m)};
        v = df_add(v, o);
    }
    return (double)v.h + (double)v.l;
}

// Double-float form of the same sum: every point difference, square, the
// reciprocal square root and the accumulation carry ~48 significant bits,
// on the FP32 pipes; per-lane partial sums are combined in FP64.
__device__ __forceinline__ double far_pair_df(const FarPtF *pa, const FarPtF *pb, int npts) {
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int p = lane; p < npts; p += 32) {
        FarPtF A = pa[p];
        f2 ax = {A.xh, A.xl}, ay = {A.yh, A.yl}, az = {A.zh, A.zl};
        f2 s = {0.0f, 0.0f};
        bool bad = false;
#pragma unroll 2
        for (int q = 0; q < npts; ++q) {
            FarPtF B = pb[q];
            f2 dx = df_sub(ax, f2{B.xh, B.xl});
            f2 dy = df_sub(ay, f2{B.yh, B.yl});
            f2 dz = df_sub(az, f2{B.zh, B.zl});
            f2 r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
            if (r2.h <= 0.0f) continue;  // the reference skips R <= 0
            if (!(r2.h == r2.h) || !(B.wh == B.wh)) bad = true;  // NaN, as the reference propagates it
            s = df_add(s, df_mul(f2{B.wh, B.wl}, df_rsqrt(r2)));
        }
        double sd = (double)s.h + (double)s.l;
        if (bad) sd = nan("");
        acc = fma((double)A.wh + (double)A.wl, sd, acc);
    }
    return warp_sum(acc);
}

__device__ __forceinline__ bool near_lookup(const TileArgs &T, int i, int j, double &k) {
    int p = i, q = j;
    bool rev = false;
    if (T.R.owner[i] == T.R.owner[j] && i > j) {
        p = j;
        q = i;
        rev = true;
    }
    int lo = T.near_off[p], hi = T.near_off[p + 1];
    for (int m = lo; m < hi; ++m) {
        int jj = T.near_rec[m].j;
        if (jj == q) {
            double2 kv = T.near_k[m];
            k = rev ? kv.y : kv.x;
            return true;
        }
        if (jj > q) break;
    }
    return false;
}

__global__ void __launch_bounds__(kTileWarps * 32) k_assemble_tiles(TileArgs T) {
    __shared__ double tile[kTile][kTile + 1];
    __shared__ float4 stage[kTileWarps][160];  // partner patches' far points, per warp
    const int ta = blockIdx.y, tb = blockIdx.x;
    if (tb < ta) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const RegionsDev &R = T.R;
    const int n = T.n;
    for (int e = warp; e < kTile * kTile; e += kTileWarps) {
        int r = e / kTile, c = e % kTile;
        int a = ta * kTile + r, b = tb * kTile + c;
        double val = 0.0;
        bool active = a < n && b < n && !(ta == tb && c < r);
        if (active && T.only_a >= 0) {
            int lo = min(T.only_a, T.only_b), hi = max(T.only_a, T.only_b);
            active = (a == lo && b == hi);
        }
        if (active) {
            double dot = 0.0, sa = R.scale[a], sb = R.scale[b];
            bool skip = false;
            if (T.kind == KIND_INDUCTANCE) {
                const int xa = R.axis[a], xb = R.axis[b];
                if (xa >= 0 && xb >= 0) {
                    // axis directions: the dot product is exactly 0 or +-1
                    dot = xa != xb ? 0.0 : R.dir[3 * a + xa] * R.dir[3 * b + xb];
                } else {
                    dot = dot3(R.dir + 3 * a, R.dir + 3 * b);
                }
                skip = fabs(dot) < T.dir_tol;
            }
            bool bad = false;
            if (!skip) {
                if (T.kind != KIND_RAW && (sa <= 0.0 || sb <= 0.0)) bad = true;
                double integral = 0.0;
                // double-float mode: far patch pairs accumulate per lane and
                // are reduced across the warp once per entry; near pairs (and
                // the other modes) add in the reference's (i, j) order
                f2 facc = {0.0f, 0.0f};
                // FP32 far rule at order 4 with regions of at most 4 patches:
                // far pairs are collected in farmask and run per entry below
                const int ni = R.off[a + 1] - R.off[a], nj = R.off[b + 1] - R.off[b];
                const bool per_entry = T.far_df == 2 && T.npts == 32 && ni <= 4 && nj <= 4;
                unsigned farmask = 0;
                for (int i = R.off[a]; i < R.off[a + 1] && !bad; ++i) {
                    // i's near partners are sorted by j (the scan's list):
                    // a cursor from the first partner in region b
                    const int mhi = T.near_off[i + 1];
                    int m = T.near_off[i];
                    for (int hi = mhi; m < hi;) {
                        const int mid = (m + hi) >> 1;
                        if (T.near_rec[mid].j < R.off[b])
                            m = mid + 1;
                        else
                            hi = mid;
                    }
                    for (int j = R.off[b]; j < R.off[b + 1]; ++j) {
                        double k;
                        bool near;
                        if (a == b && i > j) {
                            near = near_lookup(T, i, j, k);  // (j, i), reversed, in j's list
                        } else {
                            while (m < mhi && T.near_rec[m].j < j) ++m;
                            near = m < mhi && T.near_rec[m].j == j;
                            if (near) k = T.near_k[m].x;
                        }
                        if (!near) {
                            if (T.far_df == 1) {
                                if (R.boxf[2 * i].w != 0.0f && R.boxf[2 * j].w != 0.0f) {  // zero-size patches add 0
                                    if (T.npts == 32)
                                        far_pair_df_acc32(T.ptf + (size_t)i * 32, T.ptf + (size_t)j * 32,
                                                          stage[warp], facc);
                                    else
                                        far_pair_df_acc(T.ptf + (size_t)i * T.npts, T.ptf + (size_t)j * T.npts,
                                                        T.npts, facc);
                                }
                                continue;
                            }
                            if (T.far_df == 2) {
                                if (R.boxf[2 * i].w != 0.0f && R.boxf[2 * j].w != 0.0f) {  // zero-size patches add 0
                                    if (per_entry)
                                        farmask |= 1u << (4 * (i - R.off[a]) + (j - R.off[b]));
                                    else if (T.npts == 32)
                                        far_pair_f32_acc32(T.ptf + (size_t)i * 32, T.ptf + (size_t)j * 32,
                                                           stage[warp], facc);
                                    else
                                        far_pair_f32_acc(T.ptf + (size_t)i * T.npts, T.ptf + (size_t)j * T.npts,
                                                         T.npts, facc);
                                }
                                continue;
                            }
                            k = far_pair_fp64(T.pts + (size_t)i * T.npts, T.pts + (size_t)j * T.npts, T.npts);
                        }
                        if (!isfinite(k)) {
                            bad = true;
                            break;
                        }
                        integral += k;
                    }
                }
                if (farmask && !bad) far_entry_f32(T.ptf, R.off[a], ni, R.off[b], nj, farmask, stage[warp], facc);
                if (T.far_df == 1 || T.far_df == 2) {
                    const f2 far2 = warp_sum_df2(facc);
                    if (lane == 0) {  // the entry's FP64 epilogue on one lane
                        const double far = (double)far2.h + (double)far2.l;
                        if (!isfinite(far)) bad = true;
                        integral += far;
                    }
                }
                if (lane == 0) {
                    if (T.kind == KIND_INDUCTANCE)
                        val = kMu0Over4Pi * dot * integral / (sa * sb);
                    else if (T.kind == KIND_POTENTIAL)
                        val = kInv4PiEps0 * integral / (sa * sb);
                    else
                        val = integral;
                    if (!isfinite(val)) bad = true;
                }
            }
            if (bad) {
                if (lane == 0) atomicMin(T.err, (unsigned long long)a * (unsigned long long)n + b);
                val = 0.0;
            }
        }
        if (lane == 0) tile[r][c] = val;
    }
    __syncthreads();
    // coalesced writes: the tile rows, then (off the diagonal) the mirror rows
    const int rows = min(kTile, n - ta * kTile), cols = min(kTile, n - tb * kTile);
    if (ta == tb) {
        for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
            int r = e / kTile, c = e % kTile;
            if (c < r) tile[r][c] = tile[c][r];
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
        int r = e / kTile, c = e % kTile;
        if (r < rows && c < cols) T.out[(size_t)(ta * kTile + r) * n + tb * kTile + c] = tile[r][c];
    }
    if (ta != tb) {
        for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
            int c = e / kTile, r = e % kTile;  // output row = column c of the tile
            if (r < rows && c < cols) T.out[(size_t)(tb * kTile + c) * n + ta * kTile + r] = tile[r][c];
        }
    }
}

// ---------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------
struct HostRegions {
    std::vector<int> off, owner, same_obj;
    std::vector<double> corner, dir, scale;
    int n = 0;
};

// Gathers the patch lists of `kind` regions; `scale` <= 0 marks a region
// whose entries must fail (no patches, or non-positive width / area).
static bool gather_regions(const Mesh *mesh, const DualMesh *dual, int kind, HostRegions &H) {
    bool edges = kind == KIND_INDUCTANCE;
    size_t n = edges ? mesh->n_edges : mesh->n_nodes;
    const PatchList *lists = edges ? dual->edge_patches : dual->node_patches;
    if (!lists || n == 0 || n > 0x7fffffff) return false;
    H.n = (int)n;
    H.off.assign(n + 1, 0);
    H.scale.assign(n, 0.0);
    if (edges) H.dir.assign(3 * n, 0.0);
    size_t total = 0;
    for (size_t r = 0; r < n; ++r) {
        H.off[r] = (int)total;
        total += lists[r].count;
        if (total > 0x7fffffff / 12) return false;
    }
    H.off[n] = (int)total;
    H.corner.resize(12 * total);
    H.owner.resize(total);
    H.same_obj.resize(total);
    for (size_t r = 0; r < n; ++r) {
        const PatchList &L = lists[r];
        for (size_t k = 0; k < L.count; ++k) {
            size_t p = (size_t)H.off[r] + k;
            memcpy(&H.corner[12 * p], L.patches[k].points, 12 * sizeof(double));
            H.owner[p] = (int)r;
            H.same_obj[p] = (int)p;
        }
        if (edges) {
            double area = dual->edge_region_areas[r], length = mesh->edge_lengths[r];
            double w = (area <= 0.0 || length <= 0.0) ? 0.0 : area / length;  // inductance.c:152-167
            H.scale[r] = (L.count == 0) ? 0.0 : w;
            for (int k = 0; k < 3; ++k) H.dir[3 * r + k] = mesh->edge_directions[3 * r + k];
        } else {
            double area = dual->node_region_areas[r];
            H.scale[r] = (L.count == 0 || !(area > 0.0)) ? 0.0 : area;
        }
    }
    return true;
}

struct DeviceRegions {
    DBuf<int> off, owner, same_obj;
    DBuf<double> corner, box, size, dir, scale;
    DBuf<float4> boxf;
    DBuf<int> axis;
    RegionsDev view;
    bool upload(const HostRegions &H) {
        int np = H.off[H.n];
        if (!off.alloc(H.n + 1) || !owner.alloc(np) || !same_obj.alloc(np) || !corner.alloc(12 * (size_t)np) ||
            !box.alloc(6 * (size_t)np) || !size.alloc(np) || !scale.alloc(H.n) || !boxf.alloc(2 * (size_t)np) ||
            !axis.alloc(H.n) ||
            !dir.alloc(H.dir.empty() ? 0 : H.dir.size()))
            return false;
        bool ok = off.upload(H.off.data(), H.off.size()) && scale.upload(H.scale.data(), H.scale.size());
        if (np) ok = ok && owner.upload(H.owner.data(), np) && same_obj.upload(H.same_obj.data(), np) &&
                     corner.upload(H.corner.data(), H.corner.size());
        if (!H.dir.empty()) ok = ok && dir.upload(H.dir.data(), H.dir.size());
        {
            // exact axis directions (one nonzero component of magnitude 1)
            std::vector<int> ax(H.n, -1);
            for (int r = 0; r < H.n && !H.dir.empty(); ++r) {
                const double *d = H.dir.data() + 3 * (size_t)r;
                int nz = 0, k = -1;
                for (int q = 0; q < 3; ++q)
                    if (d[q] != 0.0) {
                        ++nz;
                        k = q;
                    }
                if (nz == 1 && fabs(d[k]) == 1.0) ax[r] = k;
            }
            ok = ok && axis.upload(ax.data(), ax.size());
        }
        view.n = H.n;
        view.np = np;
        view.off = off.p;
        view.owner = owner.p;
        view.same_obj = same_obj.p;
        view.corner = corner.p;
        view.box = box.p;
        view.size = size.p;
        view.boxf = boxf.p;
        view.axis = axis.p;
        view.dir = dir.p;
        view.scale = scale.p;
        view.cmax = 0.0;
        for (double v : H.corner) view.cmax = fmax(view.cmax, fabs(v));
        if (ok && np) {
            PEEC_LAUNCH(k_patch_prep, (np + 127) / 128, 128, 0, view);
            ok = launch_ok("patch preparation");
        }
        return ok;
    }
};

struct AssemblyOptions {
    int orders[4];  // far, near, touching, self
    double near_factor;
    double dir_tol;
};

// Far rule arithmetic: 1 double-float on the FP32 pipes (default), 0 native
// FP64 (PEEC_GB300_FAR=fp64), 2 FP32 (PEEC_GB300_FAR=fp32, or
// peec_gb300_set_far_precision for the mixed-precision path).
static std::atomic<int> g_near_reuse{-1};
// Reuse of translated near pairs: on unless PEEC_GB300_NEAR_REUSE=0 or
// peec_gb300_set_near_reuse(0).
static bool near_reuse_enabled() {
    if (g_near_reuse < 0) {
        const char *e = getenv("PEEC_GB300_NEAR_REUSE");
        g_near_reuse = (e && strcmp(e, "0") == 0) ? 0 : 1;
    }
    return g_near_reuse == 1;
}

static std::atomic<int> g_far_mode{-1};
static int far_mode_df() {
    if (g_far_mode < 0) {
        const char *e = getenv("PEEC_GB300_FAR");
        g_far_mode = (e && strcmp(e, "fp64") == 0) ? 0 : (e && strcmp(e, "fp32") == 0) ? 2 : 1;
    }
    return g_far_mode;
}

static bool orders_valid(const AssemblyOptions &o) {
    for (int k = 0; k < 4; ++k)
        if (gl_row(o.orders[k]) < 0) return false;
    return isfinite(o.near_factor) && o.near_factor >= 0.0;
}

// Runs steps 2-6 into d_out (n*n on the device).  Returns 0, or -1 with
// *bad_entry = a*n+b of one failing entry (or -1 if the failure is not tied
// to an entry).
static int run_assembly(DeviceRegions &D, int kind, const AssemblyOptions &o, double *d_out, int only_a,
                        int only_b, long long *bad_entry, PeecAssemblyStats *stats) {
    *bad_entry = -1;
    if (!upload_gl_tables()) return -1;
    const RegionsDev &R = D.view;
    const int n = R.n, np = R.np;
    const int q = o.orders[0], npts = 2 * q * q;
    cudaEvent_t ev[4];
    for (auto &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], stream());

    DBuf<FarPt> pts((size_t)np * npts);
    DBuf<FarPtF> ptf((size_t)np * npts);
    DBuf<int> count(np + 1), near_off(np + 1), counter(1);
    DBuf<unsigned long long> err(1), evals(1), farcount(1);
    if ((np && (!pts.p || !ptf.p || !count.p || !near_off.p)) || !counter.p || !err.p || !evals.p || !farcount.p)
        return -1;
    cudaMemsetAsync(farcount.p, 0, sizeof(unsigned long long), stream());
    cudaMemsetAsync(err.p, 0xff, sizeof(unsigned long long), stream());
    cudaMemsetAsync(evals.p, 0, sizeof(unsigned long long), stream());
    cudaMemsetAsync(counter.p, 0, sizeof(int), stream());
    if (np) {
        long long tot = (long long)np * npts;
        PEEC_LAUNCH(k_far_points, (unsigned)((tot + 255) / 256), 256, 0, R, q, gl_row(q), pts.p, ptf.p);
        ScanArgs s{R, kind, o.near_factor, o.dir_tol, only_a, only_b};
        PEEC_LAUNCH(k_near_scan, (unsigned)(((long long)np * 32 + 255) / 256), 256, 0, s, 0, count.p, nullptr, nullptr,
                    farcount.p);
        PEEC_LAUNCH(k_exclusive_scan, 1, 1024, 0, count.p, near_off.p, np);
    } else {
        cudaMemsetAsync(near_off.p, 0, sizeof(int), stream());
    }
    int nrec = 0;
    if (!cuda_ok(cudaMemcpyAsync(&nrec, near_off.p + np, sizeof(int), cudaMemcpyDeviceToHost, stream()),
                 "near count") ||
        !sync("near-pair discovery"))
        return -1;
    DBuf<NearRec> rec(nrec);
    DBuf<double> slot((size_t)nrec * 8);
    DBuf<int> kindbuf((size_t)nrec * 4);
    DBuf<double2> kval(nrec);
    if (nrec && (!rec.p || !slot.p || !kindbuf.p || !kval.p)) return -1;
    cudaEventRecord(ev[1], stream());
    DBuf<long long> mkeys;
    DBuf<unsigned long long> mhash;
    DBuf<int> mok, mslot, mrep, misrep, moff, mlist;
    DBuf<MemoSlot> mtab;
    int njobrec = nrec;
    const int *job_rec = nullptr;
    if (nrec) {
        ScanArgs s{R, kind, o.near_factor, o.dir_tol, only_a, only_b};
        PEEC_LAUNCH(k_near_scan, (unsigned)(((long long)np * 32 + 255) / 256), 256, 0, s, 1, nullptr, near_off.p,
                    rec.p, nullptr);
        if (near_reuse_enabled() && nrec > 1) {
            unsigned long long cap = 1;
            while (cap < 4ull * (unsigned long long)nrec) cap <<= 1;
            double delta = 8.0 * 2.220446049250313e-16 * (R.cmax > 0.0 ? R.cmax : 1.0);
            bool ok = mkeys.alloc((size_t)nrec * (kKeyLen + 1)) && mhash.alloc(nrec) && mok.alloc(nrec) &&
                      mslot.alloc(nrec) && mrep.alloc(nrec) && misrep.alloc(nrec) && moff.alloc(nrec + 1) &&
                      mtab.alloc(cap);
            if (!ok) return -1;
            cudaMemsetAsync(mtab.p, 0, cap * sizeof(MemoSlot), stream());
            PEEC_LAUNCH(k_fill_int, (unsigned)((cap + 255) / 256), 256, 0, &mtab.p[0].rep, (long long)cap,
                        (int)sizeof(MemoSlot) / (int)sizeof(int), 0x7fffffff);
            unsigned g = (nrec + 255) / 256;
            PEEC_LAUNCH(k_memo_keys, g, 256, 0, R.corner, R.same_obj, rec.p, nrec, delta, mkeys.p, mhash.p, mok.p);
            PEEC_LAUNCH(k_memo_insert, g, 256, 0, nrec, mhash.p, mok.p, mtab.p, cap - 1, mslot.p);
            PEEC_LAUNCH(k_memo_resolve, g, 256, 0, nrec, mkeys.p, mtab.p, mslot.p, mrep.p, misrep.p);
            PEEC_LAUNCH(k_exclusive_scan, 1, 1024, 0, misrep.p, moff.p, nrec);
            int nreps = 0;
            cudaMemcpyAsync(&nreps, moff.p + nrec, sizeof(int), cudaMemcpyDeviceToHost, stream());
            if (!sync("near-pair reuse")) return -1;
            if (!mlist.alloc(nreps > 0 ? nreps : 1)) return -1;
            PEEC_LAUNCH(k_memo_compact, g, 256, 0, nrec, misrep.p, moff.p, mlist.p);
            njobrec = nreps;
            job_rec = mlist.p;
        }
        DBuf<int> marginal(nrec);
        if (!marginal.p) return -1;
        cudaMemsetAsync(marginal.p, 0, (size_t)nrec * sizeof(int), stream());
        DBuf<unsigned char> trace;
        DBuf<int> trace_len;
        if (job_rec) {
            if (!trace.alloc((size_t)njobrec * 8 * kTraceCap) || !trace_len.alloc((size_t)njobrec * 8)) return -1;
            cudaMemsetAsync(trace_len.p, 0, (size_t)njobrec * 8 * sizeof(int), stream());
        }
        NearEvalArgs A;
        A.corner = R.corner;
        A.rec = rec.p;
        A.job_rec = job_rec;
        A.nrec = njobrec;
        A.marginal = marginal.p;
        A.trace = job_rec ? trace.p : nullptr;
        A.trace_len = job_rec ? trace_len.p : nullptr;
        for (int k = 0; k < 4; ++k) A.orders[k] = o.orders[k];
        A.slot = slot.p;
        A.kind = kindbuf.p;
        A.next_job = counter.p;
        A.evals = evals.p;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        size_t smem = 8 * sizeof(NearWarpSmem);
        static std::once_flag attr_once;
        std::call_once(attr_once, [smem] {
            cudaFuncSetAttribute(k_near_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        });
        auto launch_eval = [&](int nj) -> bool {
            if (near_levels_enabled()) return near_eval_levels(A, nj);
            long long jobs = (long long)nj * 8;
            long long want = (jobs + 7) / 8;
            int grid = (int)(want < (long long)sms * 8 ? want : (long long)sms * 8);
            if (grid > 0) PEEC_LAUNCH(k_near_eval, grid, 256, smem, A);
            return true;
        };
        if (!launch_eval(njobrec)) return -1;
        DBuf<int> src, evalf, rpos, replay, fcode, failed, slot_of2, isnew, off2, list2, elist;
        DBuf<unsigned long long> key2;
        DBuf<RoundSlot> tab2;
        unsigned long long evaluated = (unsigned long long)njobrec;
        if (job_rec) {
            const unsigned g = (nrec + 255) / 256;
            unsigned long long cap = 1;
            while (cap < 4ull * (unsigned long long)nrec) cap <<= 1;
            if (!src.alloc(nrec) || !evalf.alloc(nrec) || !rpos.alloc(nrec) || !replay.alloc(nrec) ||
                !fcode.alloc(nrec) || !failed.alloc(nrec) || !slot_of2.alloc(nrec) || !isnew.alloc(nrec) ||
                !off2.alloc(nrec + 1) || !key2.alloc(nrec) || !tab2.alloc(cap))
                return -1;
            // first reuse pass: the representatives just integrated decide for themselves
            PEEC_LAUNCH(k_fill_int, g, 256, 0, src.p, (long long)nrec, 1, -1);
            PEEC_LAUNCH(k_fill_int, g, 256, 0, rpos.p, (long long)nrec, 1, -1);
            cudaMemsetAsync(evalf.p, 0, (size_t)nrec * sizeof(int), stream());
            PEEC_LAUNCH(k_round_positions, (njobrec + 255) / 256, 256, 0, job_rec, njobrec, rpos.p);
            PEEC_LAUNCH(k_round_self, g, 256, 0, nrec, rpos.p, src.p);
            DBuf<unsigned char> rtrace;
            DBuf<int> rtrace_len;
            const unsigned char *cur_trace = trace.p;
            const int *cur_len = trace_len.p;
            const int kRounds = 6;
            for (int round = 1; round <= kRounds; ++round) {
                PEEC_LAUNCH(k_round_classify, g, 256, 0, nrec, mrep.p, rpos.p, marginal.p, src.p, evalf.p, replay.p,
                            fcode.p);
                PEEC_LAUNCH(k_round_replay, (unsigned)(((long long)nrec * 8 + 127) / 128), 128, 0, nrec, mrep.p,
                            rpos.p, replay.p, R.corner, rec.p, cur_trace, cur_len, fcode.p);
                PEEC_LAUNCH(k_round_regroup, g, 256, 0, nrec, replay.p, fcode.p, mrep.p, src.p, failed.p, key2.p);
                if (round == kRounds) {
                    // last round: what still fails is integrated directly
                    PEEC_LAUNCH(k_round_fail_to_eval, g, 256, 0, nrec, failed.p, src.p, evalf.p);
                    break;
                }
                cudaMemsetAsync(tab2.p, 0xff, cap * sizeof(RoundSlot), stream());
                PEEC_LAUNCH(k_fill_int, (unsigned)((cap + 255) / 256), 256, 0, &tab2.p[0].rep, (long long)cap,
                            (int)sizeof(RoundSlot) / (int)sizeof(int), 0x7fffffff);
                PEEC_LAUNCH(k_round_insert, g, 256, 0, nrec, failed.p, key2.p, tab2.p, cap - 1, slot_of2.p);
                PEEC_LAUNCH(k_round_resolve, g, 256, 0, nrec, failed.p, tab2.p, slot_of2.p, mrep.p, src.p, isnew.p,
                            evalf.p);
                PEEC_LAUNCH(k_exclusive_scan, 1, 1024, 0, isnew.p, off2.p, nrec);
                int nnew = 0;
                cudaMemcpyAsync(&nnew, off2.p + nrec, sizeof(int), cudaMemcpyDeviceToHost, stream());
                if (!sync("near-pair reuse round")) return -1;
                if (nnew == 0) break;
                if (!list2.alloc(nnew) || !rtrace.alloc((size_t)nnew * 8 * kTraceCap) ||
                    !rtrace_len.alloc((size_t)nnew * 8))
                    return -1;
                PEEC_LAUNCH(k_memo_compact, g, 256, 0, nrec, isnew.p, off2.p, list2.p);
                PEEC_LAUNCH(k_fill_int, g, 256, 0, rpos.p, (long long)nrec, 1, -1);
                PEEC_LAUNCH(k_round_positions, (nnew + 255) / 256, 256, 0, list2.p, nnew, rpos.p);
                cudaMemsetAsync(rtrace_len.p, 0, (size_t)nnew * 8 * sizeof(int), stream());
                cudaMemsetAsync(counter.p, 0, sizeof(int), stream());
                A.job_rec = list2.p;
                A.nrec = nnew;
                A.trace = rtrace.p;
                A.trace_len = rtrace_len.p;
                if (!launch_eval(nnew)) return -1;
                evaluated += (unsigned long long)nnew;
                cur_trace = rtrace.p;
                cur_len = rtrace_len.p;
            }
            // records marked for direct integration
            PEEC_LAUNCH(k_exclusive_scan, 1, 1024, 0, evalf.p, off2.p, nrec);
            int nre = 0;
            cudaMemcpyAsync(&nre, off2.p + nrec, sizeof(int), cudaMemcpyDeviceToHost, stream());
            if (!sync("near-pair reuse check")) return -1;
            if (nre > 0) {
                if (!elist.alloc(nre)) return -1;
                PEEC_LAUNCH(k_memo_compact, g, 256, 0, nrec, evalf.p, off2.p, elist.p);
                cudaMemsetAsync(counter.p, 0, sizeof(int), stream());
                A.job_rec = elist.p;
                A.nrec = nre;
                A.marginal = nullptr;
                A.trace = nullptr;
                A.trace_len = nullptr;
                if (!launch_eval(nre)) return -1;
                evaluated += (unsigned long long)nre;
            }
            if (stats) {
                stats->near_pairs_evaluated = evaluated;
                stats->near_pairs_reevaluated = evaluated - (unsigned long long)njobrec;
            }
        } else if (stats) {
            stats->near_pairs_evaluated = (unsigned long long)nrec;
            stats->near_pairs_reevaluated = 0;
        }
        PEEC_LAUNCH(k_near_finalize, (nrec + 127) / 128, 128, 0, nrec, slot.p, kindbuf.p, kval.p);
        if (job_rec) PEEC_LAUNCH(k_round_scatter, (nrec + 255) / 256, 256, 0, nrec, src.p, kval.p);
    }
    cudaEventRecord(ev[2], stream());
    TileArgs T;
    T.R = R;
    T.kind = kind;
    T.dir_tol = o.dir_tol;
    T.pts = pts.p;
    T.ptf = ptf.p;
    T.npts = npts;
    // The double-float and FP32 far loops carry no R <= 0 test, which relies
    // on FAR patches being apart: true for near_factor > 0 (a positive box
    // gap).  With near_factor == 0 overlapping patches are FAR, so the FP64
    // form, which skips R <= 0 as the reference does, takes them.
    T.far_df = o.near_factor > 0.0 ? far_mode_df() : 0;
    T.near_off = near_off.p;
    T.near_rec = rec.p;
    T.near_k = kval.p;
    T.out = d_out;
    T.n = n;
    T.only_a = only_a;
    T.only_b = only_b;
    T.err = err.p;
    int nt = (n + kTile - 1) / kTile;
    PEEC_LAUNCH(k_assemble_tiles, dim3(nt, nt), kTileWarps * 32, 0, T);
    cudaEventRecord(ev[3], stream());
    if (!launch_ok("assembly kernels")) return -1;
    unsigned long long e = 0, ne = 0, nf = 0;
    cudaMemcpyAsync(&nf, farcount.p, sizeof(nf), cudaMemcpyDeviceToHost, stream());
    cudaMemcpyAsync(&e, err.p, sizeof(e), cudaMemcpyDeviceToHost, stream());
    cudaMemcpyAsync(&ne, evals.p, sizeof(ne), cudaMemcpyDeviceToHost, stream());
    if (!sync("assembly")) return -1;
    if (stats) {
        float t01 = 0, t12 = 0, t23 = 0;
        cudaEventElapsedTime(&t01, ev[0], ev[1]);
        cudaEventElapsedTime(&t12, ev[1], ev[2]);
        cudaEventElapsedTime(&t23, ev[2], ev[3]);
        stats->near_pairs = (unsigned long long)nrec;
        stats->potential_evaluations = ne;
        stats->far_point_pairs = nf * (unsigned long long)npts * (unsigned long long)npts;
        stats->ms_prepare = t01;
        stats->ms_near = t12;
        stats->ms_far = t23;
    }
    for (auto &ev_ : ev) cudaEventDestroy(ev_);
    if (e != ~0ull) {
        *bad_entry = (long long)e;
        return -1;
    }
    return 0;
}

// ---------------------------------------------------------------------
// 7. retarded kernel exp(-jkR)/R (extension; the reference has none)
//
// K_k = K_0 + D_k with K_0 the static integral of this pipeline (exact near
// field, FP64) and D_k = integral of (exp(-jkR) - 1)/R, which is smooth and
// bounded (limit -jk at R = 0), by the far product rule over every patch
// pair, on the FP32 pipes: (exp(-jkR) - 1)/R = (-2 sin^2(kR/2) - j sin kR)/R
// from one sincosf, FP32 sums per lane and across the warp.  D_k carries
// ~1e-6 relative FP32 error; at k = 0 the result is the static matrix exactly.
//
// The order of the correction's product rule follows the smoothness of the
// integrand over the patch pair: with s the longer patch size and d the
// distance of the patch centres, pairs with d >= 8 s and k s <= 0.1 take
// order 2 (8 points a patch), pairs with d >= 3 s and k s <= 0.8 order 3
// (18 points), the rest the far order (32 points at order 4).  Against the
// far order everywhere, the measured difference stays below 1e-6 of the
// largest |D_k| entry (plates and boxes, k s from 0.01 to 1.1); at 2.5 cm
// cells and 100 MHz about 90% of the pairs take order 2.
// ---------------------------------------------------------------------
struct Cplx {
    double re, im;
};

struct RetardArgs {
    RegionsDev R;
    const FarPtF *ptf;   // far-order points (npts a patch)
    const FarPtF *ptf3;  // order-3 points (18 a patch), or null
    const FarPtF *ptf2;  // order-2 points (8 a patch), or null
    int npts, n, kind;
    double dir_tol;
    float k;
    const double *stat;  // static matrix, n x n
    Cplx *out;           // n x n complex
};

// one point pair's correction with weight w, accumulated in FP32
__device__ __forceinline__ void retard_point_pair(const float4 A, const float4 B, float w, float k, float &sr,
                                                  float &si) {
    const float dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    if (r2 > 0.0f) {
        float inv = rsqrt_hw(r2), sn, cs;
        sincosf(0.5f * k * (r2 * inv), &sn, &cs);
        const float wi = w * inv;
        sr = fmaf(wi, -2.0f * sn * sn, sr);
        si = fmaf(wi, -2.0f * sn * cs, si);
    } else {
        si = fmaf(w, -k, si);
    }
}

// per-lane FP32 sums of one patch pair's correction at the far order: lane
// p holds A point p, the partner's points are read in turn (no FP64
// instructions in the point loop: on GB300 they would cost 64 cycles per
// warp each)
__device__ __forceinline__ void retard_pair(const FarPtF *pa, const FarPtF *pb, int npts, float k, float &re,
                                            float &im) {
    const int lane = threadIdx.x & 31;
    for (int p = lane; p < npts; p += 32) {
        const float4 A = *reinterpret_cast<const float4 *>(pa + p);  // xh, yh, zh, wh
        float sr = 0.0f, si = 0.0f;
#pragma unroll 4
        for (int q = 0; q < npts; ++q) {
            const float4 B = *reinterpret_cast<const float4 *>(pb + q);
            retard_point_pair(A, B, B.w, k, sr, si);
        }
        re = fmaf(A.w, sr, re);
        im = fmaf(A.w, si, im);
    }
}

// the same at a lower order with NP points a patch: the NP x NP point pairs
// spread over the lanes
template <int NP>
__device__ __forceinline__ void retard_pair_low(const FarPtF *pa, const FarPtF *pb, float k, float &re, float &im) {
    const int lane = threadIdx.x & 31;
#pragma unroll 2
    for (int t = lane; t < NP * NP; t += 32) {
        const int a = t / NP, b = t - a * NP;
        const float4 A = *reinterpret_cast<const float4 *>(pa + a);
        const float4 B = *reinterpret_cast<const float4 *>(pb + b);
        retard_point_pair(A, B, A.w * B.w, k, re, im);
    }
}

__global__ void __launch_bounds__(kTileWarps * 32) k_retard_tiles(RetardArgs T) {
    __shared__ Cplx tile[kTile][kTile + 1];
    const int ta = blockIdx.y, tb = blockIdx.x;
    if (tb < ta) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const RegionsDev &R = T.R;
    const int n = T.n;
    for (int e = warp; e < kTile * kTile; e += kTileWarps) {
        int r = e / kTile, c = e % kTile;
        int a = ta * kTile + r, b = tb * kTile + c;
        Cplx val = {0.0, 0.0};
        if (a < n && b < n && !(ta == tb && c < r)) {
            // the entry's FP64 scale in lane 0 only: FP64 instructions are
            // scarce on GB300, the point loop below is all FP32
            double scale = 0.0;
            int skip = 0;
            if (lane == 0) {
                if (T.kind == KIND_INDUCTANCE) {
                    double dot = dot3(R.dir + 3 * a, R.dir + 3 * b);
                    scale = fabs(dot) < T.dir_tol ? 0.0 : kMu0Over4Pi * dot / (R.scale[a] * R.scale[b]);
                } else {
                    scale = kInv4PiEps0 / (R.scale[a] * R.scale[b]);
                }
                skip = scale == 0.0 || T.k == 0.0f;
            }
            skip = __shfl_sync(0xffffffffu, skip, 0);
            float fre = 0.0f, fim = 0.0f;
            if (!skip)
                for (int i = R.off[a]; i < R.off[a + 1]; ++i) {
                    const float4 li = R.boxf[2 * i], hi = R.boxf[2 * i + 1];
                    for (int j = R.off[b]; j < R.off[b + 1]; ++j) {
                        const float4 lj = R.boxf[2 * j], hj = R.boxf[2 * j + 1];
                        const float dx = (li.x + hi.x) - (lj.x + hj.x), dy = (li.y + hi.y) - (lj.y + hj.y),
                                    dz = (li.z + hi.z) - (lj.z + hj.z);
                        const float d = 0.5f * sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
                        const float sz = fmaxf(li.w, lj.w), ks = T.k * sz;
                        if (T.ptf2 && d >= 8.0f * sz && ks <= 0.1f)
                            retard_pair_low<8>(T.ptf2 + (size_t)i * 8, T.ptf2 + (size_t)j * 8, T.k, fre, fim);
                        else if (T.ptf3 && d >= 3.0f * sz && ks <= 0.8f)
                            retard_pair_low<18>(T.ptf3 + (size_t)i * 18, T.ptf3 + (size_t)j * 18, T.k, fre, fim);
                        else
                            retard_pair(T.ptf + (size_t)i * T.npts, T.ptf + (size_t)j * T.npts, T.npts, T.k, fre,
                                        fim);
                    }
                }
#pragma unroll
            for (int m = 16; m > 0; m >>= 1) {
                fre += __shfl_xor_sync(0xffffffffu, fre, m);
                fim += __shfl_xor_sync(0xffffffffu, fim, m);
            }
            if (lane == 0) {
                val.re = T.stat[(size_t)a * n + b] + scale * (double)fre;
                val.im = scale * (double)fim;
            }
        }
        if (lane == 0) tile[r][c] = val;
    }
    __syncthreads();
    const int rows = min(kTile, n - ta * kTile), cols = min(kTile, n - tb * kTile);
    if (ta == tb) {
        for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
            int r = e / kTile, c = e % kTile;
            if (c < r) tile[r][c] = tile[c][r];
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
        int r = e / kTile, c = e % kTile;
        if (r < rows && c < cols) T.out[(size_t)(ta * kTile + r) * n + tb * kTile + c] = tile[r][c];
    }
    if (ta != tb) {
        for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
            int c = e / kTile, r = e % kTile;
            if (r < rows && c < cols) T.out[(size_t)(tb * kTile + c) * n + ta * kTile + r] = tile[r][c];
        }
    }
}

static int assemble_retarded(const Mesh *mesh, const DualMesh *dual, int kind, const AssemblyOptions &o,
                             double wave_number, Complex *d_out, PeecAssemblyStats *stats) {
    if (!isfinite(wave_number) || wave_number < 0.0) {
        set_error("retarded assembly: the wave number must be finite and >= 0");
        return -1;
    }
    HostRegions H;
    if (!gather_regions(mesh, dual, kind, H)) return -1;
    DeviceRegions D;
    if (!D.upload(H)) return -1;
    const int n = H.n, q = o.orders[0], npts = 2 * q * q;
    DBuf<double> stat((size_t)n * n);
    if (!stat.p) return -1;
    long long bad;
    if (run_assembly(D, kind, o, stat.p, -1, -1, &bad, stats) != 0) return -1;
    const RegionsDev &R = D.view;
    // far-order points, and the order-3 / order-2 sets where the far order is higher
    auto points = [&](int order, DBuf<FarPt> &pts, DBuf<FarPtF> &ptf) -> bool {
        const long long tot = (long long)R.np * 2 * order * order;
        if (!tot) return true;
        pts.alloc((size_t)tot);
        ptf.alloc((size_t)tot);
        if (!pts.p || !ptf.p) return false;
        PEEC_LAUNCH(k_far_points, (unsigned)((tot + 255) / 256), 256, 0, R, order, gl_row(order), pts.p, ptf.p);
        return true;
    };
    DBuf<FarPt> pts, pts3, pts2;
    DBuf<FarPtF> ptf, ptf3, ptf2;
    if (!points(q, pts, ptf) || (q > 3 && !points(3, pts3, ptf3)) || (q > 2 && !points(2, pts2, ptf2))) return -1;
    RetardArgs T{R,    ptf.p,       q > 3 ? ptf3.p : nullptr, q > 2 ? ptf2.p : nullptr, npts, n, kind, o.dir_tol,
                 (float)wave_number, stat.p, reinterpret_cast<Cplx *>(d_out)};
    int nt = (n + kTile - 1) / kTile;
    PEEC_LAUNCH(k_retard_tiles, dim3(nt, nt), kTileWarps * 32, 0, T);
    if (!launch_ok("retarded assembly") || !sync("retarded assembly")) return -1;
    return 0;
}

// Counts the far-rule point evaluations of a matrix on the host from the
// region sizes and the near list size (algorithmic work for the roofline).
}  // namespace peec

using namespace peec;

// ---------------------------------------------------------------------
// C ABI: quadrature.h
// ---------------------------------------------------------------------
extern "C" {

int gauss_legendre_rule(int order, double *x, double *w) {
    if (x == NULL || w == NULL) return -1;
    int row = gl_row(order);
    if (row < 0) {
        fprintf(stderr, "ERROR: unsupported Gauss-Legendre order: %d.\n", order);
        return -1;
    }
    for (int i = 0; i < order; ++i) {
        x[i] = GL_NODES[row][i];
        w[i] = GL_WEIGHTS[row][i];
    }
    return 0;
}

double triangle_area(const double p0[3], const double p1[3], const double p2[3]) {
    double a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    double b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double c[3];
    cross3(a, b, c);
    return 0.5 * norm3(c);
}

double quad_patch_area(const QuadPatch *patch) {
    if (patch == NULL) return 0.0;
    const double *c = patch->points;
    return triangle_area(c, c + 3, c + 6) + triangle_area(c, c + 6, c + 9);
}

double quad_patch_size(const QuadPatch *patch) {
    if (patch == NULL) return 0.0;
    return patch_size(patch->points);
}

double quad_patch_min_vertex_distance(const QuadPatch *a, const QuadPatch *b) {
    if (a == NULL || b == NULL) return 0.0;
    double best = HUGE_VAL;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double d = dist3(a->points + 3 * i, b->points + 3 * j);
            if (d < best) best = d;
        }
    return best;
}

QuadPairType quad_patch_classify_pair(const QuadPatch *a, const QuadPatch *b, double near_factor) {
    if (a == NULL || b == NULL) return QUAD_PAIR_FAR;
    double ba[6], bb[6];
    patch_aabb(a->points, ba);
    patch_aabb(b->points, bb);
    return (QuadPairType)classify_pair(a->points, ba, patch_size(a->points), b->points, bb, patch_size(b->points),
                                       near_factor, a == b);
}

double quad_patch_kernel_1_over_r(const QuadPatch *a, const QuadPatch *b, int far_order, int near_order,
                                  int touching_order, int self_order, double near_factor) {
    if (a == NULL || b == NULL) return nan("");
    AssemblyOptions o = {{far_order, near_order, touching_order, self_order}, near_factor, 0.0};
    if (!orders_valid(o)) return nan("");
    HostRegions H;
    bool same = (a == b);
    H.n = same ? 1 : 2;
    H.off = same ? std::vector<int>{0, 1} : std::vector<int>{0, 1, 2};
    H.owner = same ? std::vector<int>{0} : std::vector<int>{0, 1};
    H.same_obj = H.owner;
    H.scale.assign(H.n, 1.0);
    H.corner.assign(a->points, a->points + 12);
    if (!same) H.corner.insert(H.corner.end(), b->points, b->points + 12);
    DeviceRegions D;
    if (!D.upload(H)) return nan("");
    DBuf<double> out((size_t)H.n * H.n);
    if (!out.p) return nan("");
    long long bad = -1;
    int oa = 0, ob = same ? 0 : 1;
    if (run_assembly(D, KIND_RAW, o, out.p, oa, ob, &bad, nullptr) != 0) return nan("");
    double v = 0.0;
    if (!cuda_ok(cudaMemcpyAsync(&v, out.p + ob, sizeof(double), cudaMemcpyDeviceToHost, stream()), "copy") ||
        !sync("pair kernel"))
        return nan("");
    return v;
}

// ---------------------------------------------------------------------
// C ABI: inductance.h / potential.h
// ---------------------------------------------------------------------
void inductance_options_default(InductanceOptions *options, int parallel_threads) {
    if (options == NULL) return;
    options->far_order = 4;
    options->near_order = 10;
    options->touching_order = 12;
    options->self_order = 8;
    options->near_factor = 0.5;
    options->parallel_threads = parallel_threads;
    options->direction_tolerance = 1.0e-10;
}

void inductance_init(InductanceMatrix *L) {
    if (L) memset(L, 0, sizeof(*L));
}

void inductance_free(InductanceMatrix *L) {
    if (!L) return;
    free(L->data);
    inductance_init(L);
}

void potential_options_default(PotentialOptions *options, int parallel_threads) {
    if (options == NULL) return;
    options->far_order = 4;
    options->near_order = 10;
    options->touching_order = 12;
    options->self_order = 8;
    options->near_factor = 0.5;
    options->parallel_threads = parallel_threads;
}

void potential_init(PotentialMatrix *P) {
    if (P) memset(P, 0, sizeof(*P));
}

void potential_free(PotentialMatrix *P) {
    if (!P) return;
    free(P->data);
    potential_init(P);
}

}  // extern "C"

namespace peec {

// Assemble one matrix of `kind` into host memory `host_out` (n*n), or into
// device memory `dev_out` if given.  Single entry when only_a >= 0.
static int assemble(const Mesh *mesh, const DualMesh *dual, int kind, const AssemblyOptions &o, double *host_out,
                    double *dev_out, int only_a, int only_b, long long *bad, PeecAssemblyStats *stats) {
    *bad = -1;
    HostRegions H;
    if (!gather_regions(mesh, dual, kind, H)) return -1;
    DeviceRegions D;
    if (!D.upload(H)) return -1;
    size_t nn = (size_t)H.n * H.n;
    DBuf<double> tmp;
    double *d = dev_out;
    if (!d) {
        if (!tmp.alloc(nn)) return -1;
        d = tmp.p;
    }
    if (run_assembly(D, kind, o, d, only_a, only_b, bad, stats) != 0) return -1;
    if (host_out) {
        if (only_a >= 0) {
            size_t idx = (size_t)(only_a < only_b ? only_a : only_b) * H.n + (only_a < only_b ? only_b : only_a);
            if (!cuda_ok(cudaMemcpyAsync(host_out, d + idx, sizeof(double), cudaMemcpyDeviceToHost, stream()),
                         "copy"))
                return -1;
        } else if (!cuda_ok(cudaMemcpyAsync(host_out, d, nn * sizeof(double), cudaMemcpyDeviceToHost, stream()),
                            "copy")) {
            return -1;
        }
        if (!sync("matrix download")) return -1;
    }
    return 0;
}

}  // namespace peec

extern "C" {

int inductance_compute_pair(const Mesh *mesh, const DualMesh *dual, size_t edge_a, size_t edge_b,
                            const InductanceOptions *options, double *value) {
    if (!mesh || !dual || !options || !value) return -1;
    if (edge_a >= mesh->n_edges || edge_b >= mesh->n_edges) return -1;
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, options->direction_tolerance};
    // orthogonal edges: exact zero before any integral (inductance.c:272-277)
    double dot = dot3(&mesh->edge_directions[3 * edge_a], &mesh->edge_directions[3 * edge_b]);
    if (fabs(dot) < options->direction_tolerance) {
        *value = 0.0;
        return 0;
    }
    if (!orders_valid(o)) return -1;
    long long bad;
    double v = 0.0;
    if (assemble(mesh, dual, KIND_INDUCTANCE, o, &v, nullptr, (int)edge_a, (int)edge_b, &bad, nullptr) != 0)
        return -1;
    *value = v;
    return 0;
}

int inductance_compute_matrix(const Mesh *mesh, const DualMesh *dual, const InductanceOptions *options,
                              InductanceMatrix *L) {
    if (!mesh || !dual || !options || !L) return -1;
    if (mesh->n_edges == 0) return -1;
    inductance_init(L);
    size_t ne = mesh->n_edges;
    L->n = ne;
    L->data = (double *)calloc(ne * ne, sizeof(double));
    if (!L->data) {
        fprintf(stderr, "ERROR: cannot allocate inductance matrix.\n");
        return -1;
    }
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, options->direction_tolerance};
    long long bad = -1;
    int status = orders_valid(o) ? assemble(mesh, dual, KIND_INDUCTANCE, o, L->data, nullptr, -1, -1, &bad, nullptr)
                                 : -1;
    if (status != 0) {
        if (bad >= 0)
            fprintf(stderr, "\nERROR: inductance calculation failed for edges %zu, %zu.\n", (size_t)(bad / ne),
                    (size_t)(bad % ne));
        else
            fprintf(stderr, "\nERROR: inductance calculation failed.\n");
        inductance_free(L);
        return -1;
    }
    return 0;
}

int potential_compute_pair(const Mesh *mesh, const DualMesh *dual, size_t node_i, size_t node_j,
                           const PotentialOptions *options, double *value) {
    if (!mesh || !dual || !options || !value) return -1;
    if (node_i >= mesh->n_nodes || node_j >= mesh->n_nodes) return -1;
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, 0.0};
    if (!orders_valid(o)) return -1;
    long long bad;
    double v = 0.0;
    if (assemble(mesh, dual, KIND_POTENTIAL, o, &v, nullptr, (int)node_i, (int)node_j, &bad, nullptr) != 0)
        return -1;
    *value = v;
    return 0;
}

int potential_compute_matrix(const Mesh *mesh, const DualMesh *dual, const PotentialOptions *options,
                             PotentialMatrix *P) {
    if (!mesh || !dual || !options || !P) return -1;
    if (mesh->n_nodes == 0) return -1;
    potential_init(P);
    size_t nv = mesh->n_nodes;
    P->n = nv;
    P->data = (double *)calloc(nv * nv, sizeof(double));
    if (!P->data) {
        fprintf(stderr, "ERROR: cannot allocate potential matrix.\n");
        return -1;
    }
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, 0.0};
    long long bad = -1;
    int status =
        orders_valid(o) ? assemble(mesh, dual, KIND_POTENTIAL, o, P->data, nullptr, -1, -1, &bad, nullptr) : -1;
    if (status != 0) {
        if (bad >= 0)
            fprintf(stderr, "\nERROR: potential calculation failed for nodes %zu, %zu.\n", (size_t)(bad / nv),
                    (size_t)(bad % nv));
        else
            fprintf(stderr, "\nERROR: potential calculation failed.\n");
        potential_free(P);
        return -1;
    }
    return 0;
}

// Extension: assemble straight into device memory (n*n doubles).
int peec_gb300_inductance_device(const Mesh *mesh, const DualMesh *dual, const InductanceOptions *options,
                                 double *d_out, PeecAssemblyStats *stats) {
    if (!mesh || !dual || !options || !d_out || mesh->n_edges == 0) return -1;
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, options->direction_tolerance};
    if (!orders_valid(o)) return -1;
    long long bad;
    return assemble(mesh, dual, KIND_INDUCTANCE, o, nullptr, d_out, -1, -1, &bad, stats);
}

int peec_gb300_potential_device(const Mesh *mesh, const DualMesh *dual, const PotentialOptions *options,
                                double *d_out, PeecAssemblyStats *stats) {
    if (!mesh || !dual || !options || !d_out || mesh->n_nodes == 0) return -1;
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, 0.0};
    if (!orders_valid(o)) return -1;
    long long bad;
    return assemble(mesh, dual, KIND_POTENTIAL, o, nullptr, d_out, -1, -1, &bad, stats);
}

}  // extern "C"

extern "C" int peec_gb300_inductance_retarded_device(const Mesh *mesh, const DualMesh *dual,
                                                    const InductanceOptions *options, double wave_number,
                                                    Complex *d_out, PeecAssemblyStats *stats) {
    if (!mesh || !dual || !options || !d_out || mesh->n_edges == 0) return -1;
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, options->direction_tolerance};
    if (!orders_valid(o)) return -1;
    return assemble_retarded(mesh, dual, KIND_INDUCTANCE, o, wave_number, d_out, stats);
}

extern "C" int peec_gb300_potential_retarded_device(const Mesh *mesh, const DualMesh *dual,
                                                   const PotentialOptions *options, double wave_number,
                                                   Complex *d_out, PeecAssemblyStats *stats) {
    if (!mesh || !dual || !options || !d_out || mesh->n_nodes == 0) return -1;
    AssemblyOptions o = {{options->far_order, options->near_order, options->touching_order, options->self_order},
                         options->near_factor, 0.0};
    if (!orders_valid(o)) return -1;
    return assemble_retarded(mesh, dual, KIND_POTENTIAL, o, wave_number, d_out, stats);
}

// Select the far-rule arithmetic of later assemblies: 0 FP64, 1 double-float
// (default, FP64-accurate), 2 FP32 (mixed-precision path).  Returns the
// previous mode.
extern "C" int peec_gb300_set_far_precision(int mode) {
    int prev = far_mode_df();
    if (mode >= 0 && mode <= 2) g_far_mode = mode;
    return prev;
}

// Turn the reuse of translated near pairs on (1) or off (0) for later
// assemblies; returns the previous setting.
extern "C" int peec_gb300_set_near_reuse(int on) {
    int prev = near_reuse_enabled() ? 1 : 0;
    g_near_reuse = on ? 1 : 0;
    return prev;
}
