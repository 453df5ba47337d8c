// tcgen05 tensor-core GEMM for sm_103a: TMA-fed shared-memory operands, FP32
// accumulators in tensor memory (TMEM), one elected thread issuing the MMAs.
//
//   D_j[128 x BN] = A[128 x K] * B_j[BN x K]^T      (j < J, BF16 in, FP32 acc)
//   C_j[rows, cols] -= D_j                            (epilogue, FP32 in HBM)
//
// A and every B_j are K-major BF16 matrices in global memory described by TMA
// tensor maps (box 64 x rows, 128-byte swizzle).  Splitting FP32 operands
// into BF16 hi/lo parts and concatenating the parts along K turns one call
// into the split-BF16x3 product  Ah Bh + Ah Bl + Al Bh  (FP32-equivalent),
// and stacking real / imaginary parts along K gives the complex update with
// J = 2 accumulators that share the A tile.
//
// Warp roles (4 warps, 128 threads): warp 0 allocates TMEM and one of its
// lanes drives TMA; one lane of warp 1 issues tcgen05.mma; after the last MMA
// commits, all four warps read their 32 TMEM lanes (tcgen05.ld 32x32b) and
// update C.  Every mbarrier wait is bounded: on timeout the kernel records
// an error, stops issuing work, waits (bounded) for what it issued, frees
// TMEM and returns.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace peec {
namespace tc {

static const int kBM = 128;       // rows per tile (one TMEM lane each)
static const int kBK = 64;        // K per stage: 64 BF16 = one 128-byte swizzle row
static const int kMaxStages = 4;
static const long long kWaitLimit = 1LL << 26;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    for (long long i = 0; i < kWaitLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 1023) == 1023 && *abort_flag) return false;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *smem_dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor, K-major, 128-byte swizzle: 8-row groups of
// 128-byte rows, 1024 bytes apart (SBO); start address in 16-byte units.
__device__ __forceinline__ uint64_t smem_desc_sw128(const void *smem) {
    uint64_t addr = smem_u32(smem);
    uint64_t d = 0;
    d |= (addr >> 4) & 0x3FFFull;        // start address
    d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
    d |= (uint64_t)1 << 46;              // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;              // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: BF16 x BF16 -> FP32, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4)                       // D format F32
           | (1u << 7)                     // A format BF16
           | (1u << 10)                    // B format BF16
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t *smem_result, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_result)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct GemmArgs {
    int m, n;           // rows of A / C block and rows of B / columns of the C block
    int k;              // K (multiple of 64)
    int row0, col0;     // offset of the updated block in C (A and B start at row 0)
    float *c[2];        // C_j, row-major
    long long ldc;      // leading dimension of C (in complex elements when interleaved)
    int interleaved;    // 1: J = 2 accumulators are the re / im parts of one complex C
    int *error;         // set to 1 on a wait timeout
};

// grid: (ceil(n / BN), ceil(m / 128)); block 128; dynamic smem =
// smem_bytes<BN, J, S>() for an S-stage pipeline (S = min(4, K / 64))
template <int BN, int J, int S>
__host__ __device__ constexpr size_t smem_bytes() {
    return (size_t)S * ((size_t)kBM * kBK * 2 + (size_t)J * BN * kBK * 2) + 1024 + 256;
}

template <int BN, int J, int kStages>
__global__ void __launch_bounds__(128, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b0,
              const __grid_constant__ CUtensorMap map_b1, GemmArgs args) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // stage buffers on a 1024-byte boundary (128-byte swizzle atoms)
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const size_t a_bytes = (size_t)kBM * kBK * 2, b_bytes = (size_t)BN * kBK * 2;
    const size_t stage_bytes = a_bytes + J * b_bytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(base + kStages * stage_bytes);
    uint64_t *empty = full + kStages;
    uint64_t *done = empty + kStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile_n = blockIdx.x * BN, tile_m = blockIdx.y * kBM;
    const int ktiles = args.k / kBK;
    constexpr uint32_t kTmemCols = (J * BN <= 32) ? 32 : (J * BN <= 64) ? 64 : (J * BN <= 128) ? 128 : (J * BN <= 256) ? 256 : 512;

    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    volatile int *abort_flag = &s_abort;

    if (warp == 0 && lane == 0) {
        // TMA producer
        for (int kt = 0; kt < ktiles; ++kt) {
            int s = kt % kStages;
            if (kt >= kStages) {
                if (!mbar_wait(&empty[s], ((kt / kStages) - 1) & 1, abort_flag)) {
                    s_abort = 1;
                    break;
                }
            }
            unsigned char *sa = base + s * stage_bytes;
            mbar_expect_tx(&full[s], (uint32_t)stage_bytes);
            tma_load_2d(sa, &map_a, kt * kBK, tile_m, &full[s]);
            tma_load_2d(sa + a_bytes, &map_b0, kt * kBK, tile_n, &full[s]);
            if (J > 1) tma_load_2d(sa + a_bytes + b_bytes, &map_b1, kt * kBK, tile_n, &full[s]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        constexpr uint32_t idesc = idesc_bf16_f32(kBM, BN);
        for (int kt = 0; kt < ktiles; ++kt) {
            int s = kt % kStages;
            if (!mbar_wait(&full[s], (kt / kStages) & 1, abort_flag)) {
                s_abort = 1;
                break;
            }
            fence_after_sync();
            unsigned char *sa = base + s * stage_bytes;
            uint64_t ad = smem_desc_sw128(sa);
#pragma unroll
            for (int j = 0; j < J; ++j) {
                uint64_t bd = smem_desc_sw128(sa + a_bytes + j * b_bytes);
#pragma unroll
                for (int kk = 0; kk < kBK / 16; ++kk) {
                    // +32 bytes along K inside the swizzle row = +2 in 16-byte units
                    mma_bf16(tmem + j * BN, ad + 2 * kk, bd + 2 * kk, idesc, (kt > 0 || kk > 0) ? 1u : 0u);
                }
            }
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    }
    __syncwarp();
    // epilogue: wait for the accumulators
    bool ok = mbar_wait(done, 0, abort_flag);
    if (!ok) s_abort = 1;
    fence_after_sync();
    __syncthreads();
    if (!s_abort && J == 2 && args.interleaved) {
        // complex C: both accumulators of 32 columns, then one float2 read-
        // modify-write per element (256 contiguous bytes per thread; all
        // loads issued before the first store)
        const int row = tile_m + warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float vr[32], vi[32];
            tmem_ld32(lane_addr + c0, vr);
            tmem_ld32(lane_addr + BN + c0, vi);
            if (row < args.m) {
                int lim = args.n - (tile_n + c0);
                float2 *crow = reinterpret_cast<float2 *>(args.c[0]) + (size_t)(args.row0 + row) * args.ldc +
                               args.col0 + tile_n + c0;
                if (lim >= 32) {
                    float2 cv[32];
#pragma unroll
                    for (int t = 0; t < 32; ++t) cv[t] = crow[t];
#pragma unroll
                    for (int t = 0; t < 32; ++t) {
                        cv[t].x -= vr[t];
                        cv[t].y -= vi[t];
                        crow[t] = cv[t];
                    }
                } else {
#pragma unroll
                    for (int t = 0; t < 32; ++t)
                        if (t < lim) {
                            float2 v = crow[t];
                            v.x -= vr[t];
                            v.y -= vi[t];
                            crow[t] = v;
                        }
                }
            }
        }
    } else if (!s_abort) {
        const int row = tile_m + warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int j = 0; j < J; ++j) {
            for (int c0 = 0; c0 < BN; c0 += 32) {
                float v[32];
                tmem_ld32(lane_addr + j * BN + c0, v);
                if (row < args.m) {
                    int lim = args.n - (tile_n + c0);
                    if (args.interleaved) {
                        float *crow =
                            args.c[0] + ((size_t)(args.row0 + row) * args.ldc + args.col0 + tile_n + c0) * 2 + j;
#pragma unroll
                        for (int t = 0; t < 32; ++t)
                            if (t < lim) crow[2 * t] -= v[t];
                    } else {
                        float *crow = args.c[j] + (size_t)(args.row0 + row) * args.ldc + args.col0 + tile_n + c0;
#pragma unroll
                        for (int t = 0; t < 32; ++t)
                            if (t < lim) crow[t] -= v[t];
                    }
                }
            }
        }
    } else {
        if (threadIdx.x == 0) atomicExch(args.error, 1);
        // give copies already issued time to land before the CTA's shared
        // memory and TMEM are released (bounded)
        for (int i = 0; i < 20000; ++i) __nanosleep(1000);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// ---------------------------------------------------------------------
// Persistent complex update with an overlapped TMA epilogue.
//
//   C[row0 + i][col0 + j] -= (A Br^T)[i][j] + i (A Bi^T)[i][j]
//
// C is interleaved complex FP32 (described by its own tensor map over the
// m x n block, so stores clip at the block's edge).  One CTA per SM loops
// over 128 x BN tiles (t = blockIdx.x, + gridDim.x, ...).  Six warps:
//   warp 0   lane 0 TMA producer of the A / B stages (runs ahead across tiles)
//   warp 1   lane 0 MMA issuer; the two accumulators (re, im) of a tile live
//            in one of two TMEM buffers, so the MMAs of tile t+1 run while
//            the epilogue drains tile t
//   warps 2-5 epilogue: C is brought into shared memory by TMA in 16-column
//            chunks (128 rows x 128 bytes, 128-byte swizzle, double
//            buffered), each thread subtracts its TMEM row, and the chunk
//            goes back by a TMA store -- C is read and written once, in
//            full lines.
// Every wait is bounded; a timeout stops all roles at the next uniform
// point, records the error, lets work in flight drain, and frees TMEM.
static const int kEpiCols = 16;  // complex columns per C chunk (32 floats = one 128-byte row)

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, int x, int y, const void *smem_src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(smem_u32(smem_src))
                 : "memory");
}
// L2 policies: the A / B operands are re-read by every tile row / column and
// should stay in L2 while C streams through once.
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void tma_load_2d_hint(void *smem_dst, const CUtensorMap *map, int x, int y, uint64_t *bar,
                                                 uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, "
        "%3}], [%4], %5;" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}
__device__ __forceinline__ void tma_store_2d_hint(const CUtensorMap *map, int x, int y, const void *smem_src,
                                                  uint64_t policy) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group.L2::cache_hint [%0, {%1, %2}], [%3], %4;" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(smem_u32(smem_src)), "l"(policy)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void epi_barrier() { asm volatile("bar.sync 1, 128;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Tile t of the persistent schedule in groups of kGroupM tile rows: the
// tiles in flight at once (one per SM) cover ~kGroupM rows x 152/kGroupM
// columns of C, so their A and B tiles stay in L2 while C streams.
static const int kGroupM = 8;
__device__ __forceinline__ void tile_of(int t, int tiles_m, int tiles_n, int &tm, int &tn) {
    const int per_group = kGroupM * tiles_n;
    const int first = (t / per_group) * kGroupM;
    const int gm = min(tiles_m - first, kGroupM);
    const int r = t % per_group;
    tm = first + r % gm;
    tn = r / gm;
}

template <int BN, int S>
__host__ __device__ constexpr size_t smem_bytes_persistent() {
    return (size_t)S * ((size_t)kBM * kBK * 2 + (size_t)2 * BN * kBK * 2) + (size_t)2 * kBM * 128 + 1024 + 256;
}

struct PersistentArgs {
    int m, n, k;  // C block m x n, K
    int *error;
};

template <int BN, int kStages>
__global__ void __launch_bounds__(192, 1)
    k_tc_gemm_cplx_persistent(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_br,
                              const __grid_constant__ CUtensorMap map_bi, const __grid_constant__ CUtensorMap map_c,
                              PersistentArgs args) {
    // launched as a programmatic dependent: wait for the split kernels
    // before the barriers, TMEM or any load
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr size_t a_bytes = (size_t)kBM * kBK * 2, b_bytes = (size_t)BN * kBK * 2;
    constexpr size_t stage_bytes = a_bytes + 2 * b_bytes;
    constexpr uint32_t chunk_bytes = kBM * 128;
    unsigned char *cbuf = base + kStages * stage_bytes;  // 2 x [128 rows][128 bytes], swizzled
    uint64_t *full = reinterpret_cast<uint64_t *>(cbuf + 2 * chunk_bytes);
    uint64_t *empty = full + kStages;
    uint64_t *tfull = empty + kStages;
    uint64_t *tempty = tfull + 2;
    uint64_t *cfull = tempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(cfull + 2);
    __shared__ int s_abort, s_epi_fail;
    constexpr uint32_t kTmemCols = 4 * BN;  // two buffers x (re, im)
    static_assert(kTmemCols <= 512 && (kTmemCols & (kTmemCols - 1)) == 0, "TMEM columns");

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_m = (args.m + kBM - 1) / kBM, tiles_n = (args.n + BN - 1) / BN;
    const int ntiles = tiles_m * tiles_n, ktiles = args.k / kBK;
    if (threadIdx.x == 0) {
        s_abort = 0;
        s_epi_fail = 0;
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 4);
            mbar_init(&cfull[b], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    volatile int *abort_flag = &s_abort;

    if (warp == 0) {
        if (lane == 0) {
            long long it = 0;
            const uint64_t keep = policy_evict_last();
            for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x) {
                int tm, tn;
                tile_of(t, tiles_m, tiles_n, tm, tn);
                tm *= kBM;
                tn *= BN;
                for (int kt = 0; kt < ktiles; ++kt, ++it) {
                    const int s = (int)(it % kStages);
                    if (it >= kStages && !mbar_wait(&empty[s], (uint32_t)((it / kStages) - 1) & 1, abort_flag)) {
                        s_abort = 1;
                        break;
                    }
                    unsigned char *sa = base + s * stage_bytes;
                    mbar_expect_tx(&full[s], (uint32_t)stage_bytes);
                    tma_load_2d_hint(sa, &map_a, kt * kBK, tm, &full[s], keep);
                    tma_load_2d_hint(sa + a_bytes, &map_br, kt * kBK, tn, &full[s], keep);
                    tma_load_2d_hint(sa + a_bytes + b_bytes, &map_bi, kt * kBK, tn, &full[s], keep);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16_f32(kBM, BN);
            long long it = 0;
            int lt = 0;
            for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x, ++lt) {
                const int b = lt & 1;
                if (lt >= 2 && !mbar_wait(&tempty[b], (uint32_t)((lt >> 1) - 1) & 1, abort_flag)) {
                    s_abort = 1;
                    break;
                }
                fence_after_sync();
                const uint32_t acc = tmem + (uint32_t)(b * 2 * BN);
                bool ok = true;
                for (int kt = 0; kt < ktiles; ++kt, ++it) {
                    const int s = (int)(it % kStages);
                    if (!mbar_wait(&full[s], (uint32_t)(it / kStages) & 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    fence_after_sync();
                    unsigned char *sa = base + s * stage_bytes;
                    const uint64_t ad = smem_desc_sw128(sa);
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const uint64_t bd = smem_desc_sw128(sa + a_bytes + j * b_bytes);
#pragma unroll
                        for (int kk = 0; kk < kBK / 16; ++kk)
                            mma_bf16(acc + j * BN, ad + 2 * kk, bd + 2 * kk, idesc, (kt > 0 || kk > 0) ? 1u : 0u);
                    }
                    mma_commit(&empty[s]);
                }
                if (!ok) {
                    s_abort = 1;
                    break;
                }
                mma_commit(&tfull[b]);
            }
        }
    } else {
        // epilogue warps 2..5: TMEM lanes 32 (warp % 4) .. + 31.  A failed
        // wait is made uniform over the 128 epilogue threads (flag written
        // before one named barrier, read between it and the next) so that
        // they leave the loop together.
        const int q = warp & 3;
        const int row = 32 * q + lane;  // row within the tile
        const bool leader = (warp == 2 && lane == 0);
        const int chunks = BN / kEpiCols;
        long long gi = 0;  // C chunk sequence number (buffer gi & 1)
        int lt = 0;
        int t = blockIdx.x;
        const uint64_t stream_c = policy_evict_first();
        auto uniform_fail = [&](bool ok) -> bool {
            if (!ok) {
                s_epi_fail = 1;
                s_abort = 1;
            }
            if (leader && s_abort) s_epi_fail = 1;
            __syncwarp();
            epi_barrier();
            const bool f = s_epi_fail != 0;
            epi_barrier();
            return f;
        };
        // prefetch the first chunk
        if (leader && t < ntiles) {
            mbar_expect_tx(&cfull[0], chunk_bytes);
            int tm0, tn0;
            tile_of(t, tiles_m, tiles_n, tm0, tn0);
            tma_load_2d_hint(cbuf, &map_c, 2 * (tn0 * BN), tm0 * kBM, &cfull[0], stream_c);
        }
        for (; t < ntiles; t += gridDim.x, ++lt) {
            const int b = lt & 1;
            int tm, tn;
            tile_of(t, tiles_m, tiles_n, tm, tn);
            tm *= kBM;
            tn *= BN;
            if (uniform_fail(mbar_wait(&tfull[b], (uint32_t)(lt >> 1) & 1, abort_flag))) break;
            fence_after_sync();
            const uint32_t acc = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 2 * BN);
            bool failed = false;
            for (int ch = 0; ch < chunks; ++ch, ++gi) {
                // issue the next chunk's load once its buffer's previous store has read it
                if (leader) {
                    bulk_wait_read0();
                    int nt = t, nch = ch + 1;
                    if (nch == chunks) {
                        nch = 0;
                        nt = t + gridDim.x;
                    }
                    if (nt < ntiles) {
                        const int nb = (int)((gi + 1) & 1);
                        mbar_expect_tx(&cfull[nb], chunk_bytes);
                        int ntm, ntn;
                        tile_of(nt, tiles_m, tiles_n, ntm, ntn);
                        tma_load_2d_hint(cbuf + nb * chunk_bytes, &map_c, 2 * (ntn * BN + nch * kEpiCols), ntm * kBM,
                                         &cfull[nb], stream_c);
                    }
                }
                __syncwarp();
                float vr[kEpiCols], vi[kEpiCols];
                tmem_ld16(acc + ch * kEpiCols, vr);
                tmem_ld16(acc + BN + ch * kEpiCols, vi);
                const int cb = (int)(gi & 1);
                if (uniform_fail(mbar_wait(&cfull[cb], (uint32_t)(gi >> 1) & 1, abort_flag))) {
                    failed = true;
                    break;
                }
                unsigned char *rowp = cbuf + cb * chunk_bytes + row * 128;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    float4 *p = reinterpret_cast<float4 *>(rowp + ((u ^ (row & 7)) << 4));
                    float4 v = *p;
                    v.x -= vr[2 * u];
                    v.y -= vi[2 * u];
                    v.z -= vr[2 * u + 1];
                    v.w -= vi[2 * u + 1];
                    *p = v;
                }
                fence_proxy_async_smem();
                __syncwarp();
                epi_barrier();
                if (leader) {
                    tma_store_2d_hint(&map_c, 2 * (tn + ch * kEpiCols), tm, cbuf + cb * chunk_bytes, stream_c);
                    bulk_commit();
                }
            }
            if (failed) break;
            // this tile's accumulators are read: hand the TMEM buffer back
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
        }
        if (leader) bulk_wait0();
    }
    __syncwarp();
    __syncthreads();
    if (s_abort) {
        if (threadIdx.x == 0) atomicExch(args.error, 1);
        for (int i = 0; i < 20000; ++i) __nanosleep(1000);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

}  // namespace tc
}  // namespace peec
