// Mixed-precision building blocks on the tensor cores (tcgen05 + TMA).
//
//   tensor maps      cuTensorMapEncodeTiled through the runtime's driver entry
//                    point (no link-time dependency on libcuda)
//   tc_gemm_update   C_j[row0.., col0..] -= A B_j^T with BF16 operands and FP32
//                    accumulation in TMEM (tc_gemm.cuh)
//   split kernels    FP32 -> BF16 hi + lo, the hi/lo parts laid out along K so
//                    that one GEMM computes the split-BF16x3 product
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "../../include/peec_gb300.h"
#include "common.cuh"
#include "tc_gemm.cuh"

namespace peec {

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static bool encoder() {
    static std::once_flag once;
    std::call_once(once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    if (!g_encode) set_error("cuTensorMapEncodeTiled is not available");
    return g_encode != nullptr;
}

// 2-D BF16 K-major matrix [rows][k], box {64, box_rows}, 128-byte swizzle.
static bool launch_tc_ok() { return launch_ok("tcgen05 GEMM"); }

static bool make_map_bf16(CUtensorMap *map, const void *base, int rows, int k, int box_rows) {
    if (!encoder()) return false;
    if (((uintptr_t)base & 15) || (k * 2) % 16 != 0) {
        set_error("tensor map: base must be 16-byte aligned and the row pitch a multiple of 16 bytes");
        return false;
    }
    cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)k * 2};
    cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return false;
    }
    return true;
}

template <int BN, int J, int S>
static bool launch_tc(const void *a, const void *b0, const void *b1, float *c0, float *c1, int m, int n, int k,
                      int row0, int col0, long long ldc, int *d_err, int interleaved = 0) {
    CUtensorMap ma, mb0, mb1;
    if (!make_map_bf16(&ma, a, m, k, tc::kBM) || !make_map_bf16(&mb0, b0, n, k, BN)) return false;
    if (!make_map_bf16(&mb1, J > 1 ? b1 : b0, n, k, BN)) return false;
    tc::GemmArgs g;
    g.m = m;
    g.n = n;
    g.k = k;
    g.row0 = row0;
    g.col0 = col0;
    g.c[0] = c0;
    g.c[1] = c1;
    g.ldc = ldc;
    g.interleaved = interleaved;
    g.error = d_err;
    constexpr size_t smem = tc::smem_bytes<BN, J, S>();
    // set once per instantiation (thread-safe static initialisation)
    static const cudaError_t attr =
        cudaFuncSetAttribute(tc::k_tc_gemm<BN, J, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!cuda_ok(attr, "tcgen05 GEMM smem attribute")) return false;
    dim3 grid((n + BN - 1) / BN, (m + tc::kBM - 1) / tc::kBM);
    PEEC_LAUNCH((tc::k_tc_gemm<BN, J, S>), grid, 128, smem, ma, mb0, mb1, g);
    return launch_tc_ok();
}

// C_j -= A B_j^T; J = 1 or 2; K multiple of 64; returns false on failure.
bool tc_gemm_update(const void *a, const void *b0, const void *b1, float *c0, float *c1, int m, int n, int k,
                    int row0, int col0, long long ldc, int J, int *d_err) {
    if (k % tc::kBK != 0 || m <= 0 || n <= 0) {
        set_error("tcgen05 GEMM: K must be a positive multiple of 64");
        return false;
    }
    if (J == 1) return launch_tc<128, 1, 4>(a, b0, nullptr, c0, nullptr, m, n, k, row0, col0, ldc, d_err);
    return launch_tc<128, 2, 4>(a, b0, b1, c0, c1, m, n, k, row0, col0, ldc, d_err);
}

// FP32 interleaved complex block C[row0.., col0..] (m x n, leading dimension
// ldc complex) as a 2-D FP32 map, box 32 floats x 128 rows, 128-byte swizzle.
static bool make_map_c(CUtensorMap *map, float *c, long long ldc, int row0, int col0, int m, int n) {
    if (!encoder()) return false;
    float *base = c + 2 * ((size_t)row0 * ldc + col0);
    if (((uintptr_t)base & 15) || (ldc * 8) % 16 != 0) {
        set_error("tensor map: C block must start 16-byte aligned with an even leading dimension");
        return false;
    }
    cuuint64_t dims[2] = {(cuuint64_t)2 * n, (cuuint64_t)m};
    cuuint64_t strides[1] = {(cuuint64_t)ldc * 8};
    cuuint32_t box[2] = {32, (cuuint32_t)tc::kBM};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (C) failed (%d)", (int)r);
        return false;
    }
    return true;
}

// Persistent form (tc_gemm.cuh): one CTA per SM, TMEM double-buffered
// accumulators, TMA epilogue.  Needs the C block 16-byte aligned.
static bool persistent_ok(const float *c, long long ldc, int row0, int col0) {
    const float *base = c + 2 * ((size_t)row0 * ldc + col0);
    return ((uintptr_t)base & 15) == 0 && (ldc & 1) == 0;
}

template <int BN, int S>
static bool launch_tc_persistent(const void *a, const void *br, const void *bi, float *c, int m, int n, int k,
                                 int row0, int col0, long long ldc, int *d_err) {
    CUtensorMap ma, mbr, mbi, mc;
    if (!make_map_bf16(&ma, a, m, k, tc::kBM) || !make_map_bf16(&mbr, br, n, k, BN) ||
        !make_map_bf16(&mbi, bi, n, k, BN) || !make_map_c(&mc, c, ldc, row0, col0, m, n))
        return false;
    constexpr size_t smem = tc::smem_bytes_persistent<BN, S>();
    static const cudaError_t attr = cudaFuncSetAttribute(tc::k_tc_gemm_cplx_persistent<BN, S>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!cuda_ok(attr, "tcgen05 persistent GEMM smem attribute")) return false;
    static const int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    const long long tiles = (long long)((m + tc::kBM - 1) / tc::kBM) * ((n + BN - 1) / BN);
    const int grid = (int)std::min<long long>(tiles, sms);
    tc::PersistentArgs g{m, n, k, d_err};
    pdl_launch(tc::k_tc_gemm_cplx_persistent<BN, S>, dim3(grid), dim3(192), smem, ma, mbr, mbi, mc, g);
    return launch_tc_ok();
}

// PEEC_GB300_TC_PERSISTENT=0 keeps the one-tile-per-CTA kernel everywhere.
static bool persistent_enabled() {
    static const bool on = [] {
        const char *e = getenv("PEEC_GB300_TC_PERSISTENT");
        return !(e && strcmp(e, "0") == 0);
    }();
    return on;
}

// Tile width of the wide (trailing) updates on this host thread: 0 picks by
// shape (128 columns), 64 or 128 forces it.  The batched sweep's autotuner
// sets it while it records a graph, so the choice is baked into the graph.
static thread_local int g_tc_wide_bn = 0;
int set_tc_wide_tile(int bn) {
    const int prev = g_tc_wide_bn;
    g_tc_wide_bn = (bn == 64 || bn == 128) ? bn : 0;
    return prev;
}

// Complex C (interleaved FP32, leading dimension ldc complex elements)
// [row0.., col0..] -= (A Br^T) + j (A Bi^T).
bool tc_gemm_update_cplx(const void *a, const void *br, const void *bi, float *c, int m, int n, int k, int row0,
                         int col0, long long ldc, int *d_err) {
    if (k % tc::kBK != 0 || m <= 0 || n <= 0) {
        set_error("tcgen05 GEMM: K must be a positive multiple of 64");
        return false;
    }
    // narrow updates (the panel's K = 6 or 12 x 32, at most 256 columns):
    // 64-column tiles
    const bool narrow = k <= 192 || (k <= 384 && n <= 256) || (g_tc_wide_bn == 64);
    if (persistent_enabled() && persistent_ok(c, ldc, row0, col0))
        return narrow ? launch_tc_persistent<64, 4>(a, br, bi, c, m, n, k, row0, col0, ldc, d_err)
                      : launch_tc_persistent<128, 4>(a, br, bi, c, m, n, k, row0, col0, ldc, d_err);
    if (narrow) return launch_tc<64, 2, 3>(a, br, bi, c, c, m, n, k, row0, col0, ldc, d_err, 1);
    return launch_tc<128, 2, 4>(a, br, bi, c, c, m, n, k, row0, col0, ldc, d_err, 1);
}

}  // namespace peec

using namespace peec;

// Test / building-block entry point: complex C (interleaved FP32, leading
// dimension ldc complex) [row0.., col0..] -= A Br^T + j A Bi^T, m x n block.
extern "C" int peec_gb300_tc_gemm_cplx(const void *d_a, const void *d_br, const void *d_bi, float *d_c, int m, int n,
                                       int k, int row0, int col0, long long ldc) {
    if (!d_a || !d_br || !d_bi || !d_c || m <= 0 || n <= 0 || row0 < 0 || col0 < 0 || ldc < col0 + n) return -1;
    DBuf<int> err(1);
    if (!err.p) return -1;
    cudaMemsetAsync(err.p, 0, sizeof(int), stream());
    if (!tc_gemm_update_cplx(d_a, d_br, d_bi, d_c, m, n, k, row0, col0, ldc, err.p)) return -1;
    int h = 0;
    cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!sync("tcgen05 complex GEMM")) return -1;
    if (h) {
        set_error("tcgen05 complex GEMM: a pipeline wait timed out");
        return -1;
    }
    return 0;
}

// Test / building-block entry point: C_j (FP32 row-major, ld = ldc) -= A B_j^T
// for device BF16 matrices A [m][k] and B_j [n][k].
extern "C" int peec_gb300_tc_gemm(const void *d_a, const void *d_b0, const void *d_b1, float *d_c0, float *d_c1,
                                  int m, int n, int k, long long ldc, int J) {
    if (!d_a || !d_b0 || !d_c0 || (J == 2 && (!d_b1 || !d_c1)) || (J != 1 && J != 2)) return -1;
    DBuf<int> err(1);
    if (!err.p) return -1;
    cudaMemsetAsync(err.p, 0, sizeof(int), stream());
    if (!tc_gemm_update(d_a, d_b0, d_b1, d_c0, d_c1, m, n, k, 0, 0, ldc, J, err.p)) return -1;
    int h = 0;
    cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream());
    if (!sync("tcgen05 GEMM")) return -1;
    if (h) {
        set_error("tcgen05 GEMM: a pipeline wait timed out");
        return -1;
    }
    return 0;
}
