// mpgpu_tc.cuh -- building blocks of the tcgen05 3xTF32 tile products
// (dense Cholesky trailing update, mpgpu_dense.cu; blocked inverse,
// mpgpu_inverse.cu): 128 x 128 FP32 accumulators in tensor memory, operand
// chunks of 128 rows x 16 K staged in shared memory by cp.async in the
// K-major no-swizzle core-matrix layout, one elected thread issuing the
// MMAs, and mbarrier waits with an iteration limit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tc {

constexpr int kNB = 128;   // tile size (rows and columns of an accumulator)

// C tile (cRow, cCol) = alpha sum_{k0 <= k < k1} A(aRow, k) B(bRow, k)^T + beta C
struct TileTask {
    int32_t aRow, bRow, k0, k1, cRow, cCol;
};

// Tile-major TF32 operands: tile (r, c) of an array with nt tiles per row at
// ((r * nt + c) << 14) floats, row-major inside the tile.
struct TcOp {
    const float *hi, *lo;
    int64_t nt;
};

// Operands stream in chunks of K = 16 through a 3-stage cp.async pipeline;
// one thread issues the tcgen05.mma of a chunk (hi*hi, hi*lo, lo*hi for two
// K = 8 steps) and commits them to the stage's mbarrier, which frees the
// stage for the chunk three ahead.  Shared-memory operand layout: K-major,
// no swizzle, core matrices of 8 rows x 16 bytes; core (row group g, k
// group c) at (g * 4 + c) * 128 bytes: leading (K) byte offset 128, stride
// (row) byte offset 512.
constexpr int kTK = 16;                          // K per chunk
constexpr int kStages = 3;
constexpr int kOpBytes = kNB * kTK * 4;          // 8 KB per operand chunk
constexpr int kStageBytes = 4 * kOpBytes;        // hi/lo of both operands
constexpr int kTcSmem = kStages * kStageBytes;  // the epilogue transposes reuse stage 0
constexpr int kTcThreads = 128;
constexpr int kWaitLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(512 >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor: D f32, A/B tf32, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kNB >> 3) << 17) |
                            ((uint32_t)(kNB >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (int i = 0; i < kWaitLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// asynchronous copy of a 128 x 16 fp32 chunk (rows of 128 in global) into
// the core-matrix layout; 4 x 16-byte copies per thread
__device__ __forceinline__ void load_chunk_async(const float *g, int kc0, uint32_t s) {
#pragma unroll
    for (int i = 0; i < kNB * (kTK / 4) / kTcThreads; ++i) {
        const int idx = threadIdx.x + i * kTcThreads;
        const int row = idx >> 2, k4 = idx & 3;
        const float *src = g + (int64_t)row * kNB + kc0 + k4 * 4;
        const uint32_t dst = s + ((row >> 3) * 4 + k4) * 128 + (row & 7) * 16;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
    }
}


}  // namespace tc

// tile products and operand splits (mpgpu_inverse.cu)
cudaError_t tc_split_tiles(const double *M, int64_t ld, int32_t r0, int32_t r1, int32_t c0, int32_t c1, float *hi,
                           float *lo, int64_t ntDst, int32_t cOff, cudaStream_t s);
cudaError_t tc_tile_gemm(const tc::TcOp &A, const tc::TcOp &B, double *C, int64_t ldc, const tc::TileTask *tasks,
                         int64_t ntask, int32_t trail0, int32_t trailK, double alpha, double beta, int32_t *err,
                         cudaStream_t s);
cudaError_t fp64_tile_gemm(const double *A, int64_t lda, int32_t ta, const double *B, int64_t ldb, int32_t tb,
                           double *C, int64_t ldc, const tc::TileTask *tasks, int64_t ntask, double alpha,
                           double beta, cudaStream_t s);
