// mpgpu_dense.cu -- blocked dense Cholesky of the global matrix (the dense
// solve of `method cholesky`, pede.f90:7951-8054 / chdec2 mpnum.f90:891-987,
// re-blocked for the GPU) in two forms:
//   mode 0: FP64 throughout (panel, triangular solve, trailing update on the
//           FP64 CUDA cores);
//   mode 1: FP64 panel factorisation and triangular solve; the trailing
//           update A22 -= L21 L21^T, which carries the N^3/3 work, on the
//           tcgen05 tensor cores in 3xTF32 (x = hi + lo, products
//           hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory) and
//           subtracted from the FP64 matrix.
// The matrix is dense row-major (lower triangle used), padded to a multiple
// of 128 with identity rows.  The factor of mode 1 is accurate to about the
// TF32x3 product precision; solves refine it in FP64 (mpgpu_solve,
// metsol 31).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "mpgpu_ctx.h"
#include "mpgpu_tc.cuh"

namespace {

constexpr int kNB = 128;   // panel width = tile size

// ------------------------------------------------------------ panel kernels
// Cholesky of the 128 x 128 diagonal block at (k0, k0), in shared memory.
__global__ void __launch_bounds__(512) k_potrf128(double *A, int64_t ld, int64_t k0, int32_t *err) {
    extern __shared__ __align__(16) double sa[];   // 128 x 129
    constexpr int S = kNB + 1;
    __shared__ int bad;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) bad = 0;
    for (int e = tid; e < kNB * kNB; e += nt) {
        const int i = e / kNB, j = e % kNB;
        sa[i * S + j] = j <= i ? A[(k0 + i) * ld + k0 + j] : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < kNB; ++j) {
        if (tid == 0) {
            const double d = sa[j * S + j];
            if (!(d > 0.0)) { bad = 1; sa[j * S + j] = 1.0; }
            else sa[j * S + j] = sqrt(d);
        }
        __syncthreads();
        const double inv = 1.0 / sa[j * S + j];
        for (int i = j + 1 + tid; i < kNB; i += nt) sa[i * S + j] *= inv;
        __syncthreads();
        const int m = kNB - 1 - j;
        for (int e = tid; e < m * m; e += nt) {
            const int i = j + 1 + e / m, k = j + 1 + e % m;
            if (k <= i) sa[i * S + k] -= sa[i * S + j] * sa[k * S + j];
        }
        __syncthreads();
    }
    for (int e = tid; e < kNB * kNB; e += nt) {
        const int i = e / kNB, j = e % kNB;
        if (j <= i) A[(k0 + i) * ld + k0 + j] = sa[i * S + j];
    }
    if (tid == 0 && bad) atomicExch(err, (int)(k0 / kNB) + 1);
}

// L21 = A21 L11^-T: one warp per row below the diagonal block; L11 held
// transposed in shared memory so that a column of L11 is contiguous.
__global__ void __launch_bounds__(256) k_trsm128(double *A, int64_t ld, int64_t k0, int64_t nrows) {
    extern __shared__ __align__(16) double lt[];   // 128 x 128 (lt[j * 128 + c] = L11[c][j]) + 128 inverse diagonal
    double *dinv = lt + kNB * kNB;
    const int tid = threadIdx.x, ln = tid & 31, wib = tid >> 5;
    for (int e = tid; e < kNB * kNB; e += blockDim.x) {
        const int c = e / kNB, j = e % kNB;
        lt[j * kNB + c] = j <= c ? A[(k0 + c) * ld + k0 + j] : 0.0;
    }
    __syncthreads();
    for (int j = tid; j < kNB; j += blockDim.x) dinv[j] = 1.0 / lt[j * kNB + j];
    __syncthreads();
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib; r < nrows; r += nw) {
        double *row = A + (k0 + kNB + r) * ld + k0;
        double a[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = row[q * 32 + ln];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            for (int l = 0; l < 32; ++l) {
                const int j = q * 32 + l;
                const double xj = __shfl_sync(0xffffffffu, a[q], l) * dinv[j];
                if (ln == l) a[q] = xj;
#pragma unroll
                for (int q2 = 0; q2 < 4; ++q2) {
                    if (q2 < q) continue;
                    const int c = q2 * 32 + ln;
                    if (c > j) a[q2] -= xj * lt[j * kNB + c];
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) row[q * 32 + ln] = a[q];
    }
}

// L21 rows as TF32 pairs (hi, lo), row-major with 128 columns
__global__ void k_split_tf32(const double *A, int64_t ld, int64_t k0, int64_t nrows, float *hi, float *lo) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nrows * kNB) return;
    const int64_t r = e / kNB;
    const int k = (int)(e % kNB);
    const double x = A[(k0 + kNB + r) * ld + k0 + k];
    uint32_t h, l;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"((float)x));
    const double rest = x - (double)__uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"((float)rest));
    hi[e] = __uint_as_float(h);
    lo[e] = __uint_as_float(l);
}

// --------------------------------------------- tcgen05 3xTF32 trailing update
using tc::kTK;
using tc::kStages;
using tc::kOpBytes;
using tc::kStageBytes;
using tc::kTcSmem;
using tc::kTcThreads;
using tc::smem_u32;
using tc::umma_desc;
using tc::mma_tf32;
using tc::mbar_wait;
using tc::tmem_ld32;
using tc::load_chunk_async;

// One CTA per 128 x 128 tile (bi >= bj) of the trailing matrix:
// C -= L_i L_j^T with K = 128 (the chunk pipeline of mpgpu_tc.cuh).
__global__ void __launch_bounds__(kTcThreads) k_syrk_tc(double *A, int64_t ld, int64_t r0, int32_t T,
                                                        const float *hi, const float *lo, int32_t *err) {
    extern __shared__ __align__(128) char tsm[];
    __shared__ uint64_t mbar[kStages];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, wib = tid >> 5, ln = tid & 31;
    const int64_t t = blockIdx.x;
    int bi = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((int64_t)bi * (bi + 1) / 2 > t) bi--;
    while ((int64_t)(bi + 1) * (bi + 2) / 2 <= t) bi++;
    const int bj = (int)(t - (int64_t)bi * (bi + 1) / 2);
    if (bi >= T) return;
    const uint32_t sbase = smem_u32(tsm);
    float *epi = reinterpret_cast<float *>(tsm) + wib * 32 * 33;   // after the last MMA only
    if (wib == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tbase)),
                     "r"(kNB));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int st = 0; st < kStages; ++st)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[st])));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tbase;
    const float *ops[4] = {hi + (int64_t)bi * kNB * kNB, lo + (int64_t)bi * kNB * kNB,
                           hi + (int64_t)bj * kNB * kNB, lo + (int64_t)bj * kNB * kNB};
    constexpr int nch = kNB / kTK;
    uint32_t ph = 0;   // bit st: parity of the next completion of stage st's barrier
    bool ok = true;
    for (int c = 0; c < kStages - 1; ++c) {
#pragma unroll
        for (int o = 0; o < 4; ++o) load_chunk_async(ops[o], c * kTK, sbase + c * kStageBytes + o * kOpBytes);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    for (int c = 0; c < nch; ++c) {
        const int st = c % kStages;
        asm volatile("cp.async.wait_group %0;\n" ::"n"(kStages - 2) : "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sb = sbase + st * kStageBytes;
#pragma unroll
            for (int kk = 0; kk < kTK / 8; ++kk) {
                const uint32_t off = kk * 256;   // 8 tf32 = 2 core matrices along K
                const uint64_t dah = umma_desc(sb + off), dal = umma_desc(sb + kOpBytes + off);
                const uint64_t dbh = umma_desc(sb + 2 * kOpBytes + off), dbl = umma_desc(sb + 3 * kOpBytes + off);
                mma_tf32(tmem, dah, dbh, (c > 0 || kk > 0) ? 1u : 0u);
                mma_tf32(tmem, dah, dbl, 1u);
                mma_tf32(tmem, dal, dbh, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&mbar[st]))
                         : "memory");
        }
        // the stage of chunk c + kStages - 1 held chunk c - 1: wait for its MMAs
        const int cn = c + kStages - 1;
        if (cn < nch) {
            const int sn = cn % kStages;
            if (c >= 1) {
                if (!mbar_wait(smem_u32(&mbar[sn]), (ph >> sn) & 1)) { ok = false; }
                ph ^= 1u << sn;
            }
            if (ok)
#pragma unroll
                for (int o = 0; o < 4; ++o)
                    load_chunk_async(ops[o], cn * kTK, sbase + sn * kStageBytes + o * kOpBytes);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        if (!__syncthreads_and(ok)) { ok = false; break; }
    }
    // wait for the MMAs of the chunks not yet waited for (the last kStages-1)
    if (ok) {
        for (int c = (nch > kStages - 1 ? nch - (kStages - 1) : 0); c < nch; ++c) {
            const int st = c % kStages;
            if (!mbar_wait(smem_u32(&mbar[st]), (ph >> st) & 1)) ok = false;
            ph ^= 1u << st;
        }
    } else {
        for (int st = 0; st < kStages; ++st) mbar_wait(smem_u32(&mbar[st]), (ph >> st) & 1);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (__syncthreads_and(ok)) {   // every MMA done: the stages are free for the transposes
        // rows of warp w = tensor-memory lanes 32w .. 32w+31; transpose each
        // 32 x 32 block through shared memory so the FP64 update is coalesced
        const int64_t rowBase = r0 + (int64_t)bi * kNB + wib * 32;
        const int64_t colBase = r0 + (int64_t)bj * kNB;
        for (int cb = 0; cb < kNB / 32; ++cb) {
            uint32_t v[32];
            tmem_ld32(tmem + ((uint32_t)(wib * 32) << 16) + (uint32_t)(cb * 32), v);
#pragma unroll
            for (int q = 0; q < 32; ++q) epi[ln * 33 + q] = __uint_as_float(v[q]);
            __syncwarp();
            // all 32 loads in flight before the subtractions
            double cv[32];
            double *cp = A + rowBase * ld + colBase + cb * 32 + ln;
#pragma unroll
            for (int r = 0; r < 32; ++r) cv[r] = cp[r * ld];
#pragma unroll
            for (int r = 0; r < 32; ++r) cp[r * ld] = cv[r] - (double)epi[r * 33 + ln];
            __syncwarp();
        }
    } else if (tid == 0) {
        atomicExch(err, -1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (wib == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kNB));
}

// ------------------------------------------------ FP64 trailing update
// 64 x 64 tiles (bi >= bj), 256 threads with 4 x 4 outputs each, K = 128
// in chunks of 16 from the FP64 panel.
__global__ void __launch_bounds__(256) k_syrk_fp64(double *A, int64_t ld, int64_t k0, int64_t r0, int32_t T) {
    __shared__ double sa[16][64 + 1], sb[16][64 + 1];
    const int64_t t = blockIdx.x;
    int bi = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((int64_t)bi * (bi + 1) / 2 > t) bi--;
    while ((int64_t)(bi + 1) * (bi + 2) / 2 <= t) bi++;
    const int bj = (int)(t - (int64_t)bi * (bi + 1) / 2);
    if (bi >= T) return;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t i0 = r0 + (int64_t)bi * 64, j0 = r0 + (int64_t)bj * 64;
    double acc[4][4] = {};
    for (int kc = 0; kc < kNB; kc += 16) {
        for (int e = tid; e < 64 * 16; e += 256) {
            const int r = e >> 4, k = e & 15;
            sa[k][r] = A[(i0 + r) * ld + k0 + kc + k];
            sb[k][r] = A[(j0 + r) * ld + k0 + kc + k];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            double a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) { a[q] = sa[k][ty * 4 + q]; b[q] = sb[k][tx * 4 + q]; }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) A[(i0 + ty * 4 + p) * ld + j0 + tx * 4 + q] -= acc[p][q];
}

__global__ void k_pad_identity(double *A, int64_t ld, int64_t n, int64_t npad) {
    const int64_t i = n + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npad) A[i * ld + i] = 1.0;
}

}  // namespace

// Factorise the dense padded matrix A (npad x npad, row-major, lower
// triangle) in place.  Returns 0, MPGPU_ERR_FACTOR (non-positive pivot in
// panel *badPanel) or a CUDA/timeout error.
int32_t dense_cholesky_device(mpgpu_ctx *c, double *A, int64_t npad, int mode, float *hiBuf, float *loBuf,
                              int32_t *dErr, int32_t *badPanel) {
    cudaStream_t s = c->stream;
    const int64_t ld = npad;
    const int64_t np = npad / kNB;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    const int potrfSmem = kNB * (kNB + 1) * (int)sizeof(double);
    const int trsmSmem = (kNB * kNB + kNB) * (int)sizeof(double);
    const int tcSmem = kTcSmem;
    MPG_CUDA(c, cudaFuncSetAttribute(k_potrf128, cudaFuncAttributeMaxDynamicSharedMemorySize, potrfSmem));
    MPG_CUDA(c, cudaFuncSetAttribute(k_trsm128, cudaFuncAttributeMaxDynamicSharedMemorySize, trsmSmem));
    MPG_CUDA(c, cudaFuncSetAttribute(k_syrk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tcSmem));
    MPG_CUDA(c, cudaMemsetAsync(dErr, 0, sizeof(int32_t), s));
    for (int64_t p = 0; p < np; ++p) {
        const int64_t k0 = p * kNB;
        k_potrf128<<<1, 512, potrfSmem, s>>>(A, ld, k0, dErr);
        const int64_t rows = npad - k0 - kNB;
        if (rows <= 0) break;
        const int64_t tb = std::min<int64_t>((rows + 7) / 8, (int64_t)nsm);
        k_trsm128<<<(unsigned)tb, 256, trsmSmem, s>>>(A, ld, k0, rows);
        const int64_t r0 = k0 + kNB;
        if (mode == 1) {
            k_split_tf32<<<(unsigned)((rows * kNB + 255) / 256), 256, 0, s>>>(A, ld, k0, rows, hiBuf, loBuf);
            const int32_t T = (int32_t)(rows / kNB);
            const int64_t ntile = (int64_t)T * (T + 1) / 2;
            k_syrk_tc<<<(unsigned)ntile, kTcThreads, tcSmem, s>>>(A, ld, r0, T, hiBuf, loBuf, dErr);
        } else {
            const int32_t T = (int32_t)(rows / 64);
            const int64_t ntile = (int64_t)T * (T + 1) / 2;
            k_syrk_fp64<<<(unsigned)ntile, 256, 0, s>>>(A, ld, k0, r0, T);
        }
        MPG_CUDA(c, cudaGetLastError());
    }
    int32_t h = 0;
    MPG_CUDA(c, cudaMemcpyAsync(&h, dErr, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    if (h < 0) return set_err(c, MPGPU_ERR_TIMEOUT, "tensor-core update: barrier wait ran out");
    if (h > 0) {
        if (badPanel) *badPanel = h - 1;
        return set_err(c, MPGPU_ERR_FACTOR, "non-positive pivot in the dense Cholesky");
    }
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_dense_cholesky(mpgpu_ctx *c, int32_t n, const double *A, double *L, int32_t mode,
                                        double *ms) {
    if (!c || n <= 0 || !A || !L || (mode != 0 && mode != 1)) return MPGPU_ERR_ARG;
    MPG_CUDA(c, cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int64_t npad = ((int64_t)n + kNB - 1) / kNB * kNB;
    double *dA = nullptr;
    float *hi = nullptr, *lo = nullptr;
    int32_t *dErr = nullptr;
    int32_t rc = MPGPU_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto fail = [&](cudaError_t e, const char *w) { rc = cuda_err(c, e, w); };
    cudaError_t e = cudaMalloc(&dA, sizeof(double) * npad * npad);
    if (e == cudaSuccess) e = cudaMalloc(&hi, sizeof(float) * npad * kNB);
    if (e == cudaSuccess) e = cudaMalloc(&lo, sizeof(float) * npad * kNB);
    if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(dA, 0, sizeof(double) * npad * npad, s);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(dA, sizeof(double) * npad, A, sizeof(double) * n, sizeof(double) * n, n,
                              cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && npad > n)
        k_pad_identity<<<(unsigned)((npad - n + 255) / 256), 256, 0, s>>>(dA, npad, n, npad);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) fail(e, "mpgpu_dense_cholesky setup");
    if (rc == MPGPU_OK) {
        cudaEventRecord(e0, s);
        int32_t bad = -1;
        rc = dense_cholesky_device(c, dA, npad, mode, hi, lo, dErr, &bad);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        if (ms) *ms = t;
    }
    if (rc == MPGPU_OK) {
        e = cudaMemcpy2DAsync(L, sizeof(double) * n, dA, sizeof(double) * npad, sizeof(double) * n, n,
                              cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) fail(e, "mpgpu_dense_cholesky download");
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(dA);
    cudaFree(hi);
    cudaFree(lo);
    cudaFree(dErr);
    return rc;
}

// ======================================================================
// Refined dense solve: the factor of dense_cholesky_device (FP64 or
// tensor-core 3xTF32) preconditions conjugate gradients in FP64 on the
// original matrix, so the solution reaches the FP64 residual whatever the
// precision of the factor.
namespace {

constexpr int kDotBlk = 304;   // fixed reduction shape: deterministic sums
// the refined solves stop only when the last CG correction is below this
// fraction of the solution (in addition to the residual test)
constexpr double kRefineXtol = 1e-13;

// packed lower triangle (n) -> dense lower (factor) and dense full (for the
// matrix-vector products), both npad x npad row-major; scaled diagonal
__global__ void k_packed_to_dense(const double *Ap, int64_t n, int64_t npad, double *Lo, double *F) {
    const int64_t nn = n * (n + 1) / 2;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = (int64_t)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
        while (i * (i + 1) / 2 > e) i--;
        while ((i + 1) * (i + 2) / 2 <= e) i++;
        const int64_t j = e - i * (i + 1) / 2;
        const double v = Ap[e];
        Lo[i * npad + j] = v;
        F[i * npad + j] = v;
        F[j * npad + i] = v;
    }
}

__global__ void k_copy_lower_shift(const double *F, double *Lo, int64_t npad, double shift) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < npad * npad;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / npad, j = e % npad;
        Lo[e] = j < i ? F[e] : (j == i ? F[e] * (1.0 + shift) : 0.0);
    }
}

// inverses of the 128 x 128 diagonal blocks of L, stored transposed:
// DinvT[p][r][*] = column r of L_pp^-1 (one CTA per block, one warp per r)
__global__ void __launch_bounds__(256) k_trtri_blocks(const double *A, int64_t ld, double *DinvT) {
    extern __shared__ __align__(16) double lt[];   // lt[j * 128 + c] = L_pp[c][j], then 1 / diagonal
    double *dinv = lt + kNB * kNB;
    const int64_t k0 = (int64_t)blockIdx.x * kNB;
    const int tid = threadIdx.x, ln = tid & 31, wib = tid >> 5;
    for (int e = tid; e < kNB * kNB; e += blockDim.x) {
        const int c = e / kNB, j = e % kNB;
        lt[j * kNB + c] = j <= c ? A[(k0 + c) * ld + k0 + j] : 0.0;
    }
    __syncthreads();
    for (int j = tid; j < kNB; j += blockDim.x) dinv[j] = 1.0 / lt[j * kNB + j];
    __syncthreads();
    double *out = DinvT + (int64_t)blockIdx.x * kNB * kNB;
    for (int r = wib; r < kNB; r += blockDim.x >> 5) {
        double a[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = (q * 32 + ln == r) ? 1.0 : 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            for (int l = 0; l < 32; ++l) {
                const int j = q * 32 + l;
                const double xj = __shfl_sync(0xffffffffu, a[q], l) * dinv[j];
                if (ln == l) a[q] = xj;
#pragma unroll
                for (int q2 = 0; q2 < 4; ++q2) {
                    if (q2 < q) continue;
                    const int c = q2 * 32 + ln;
                    if (c > j) a[q2] -= xj * lt[j * kNB + c];
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) out[(int64_t)r * kNB + q * 32 + ln] = a[q];
    }
}

// forward solve, block p: y_p <- L_pp^-1 y_p
__global__ void k_fwd_diag(const double *DinvT, int64_t p, double *y) {
    __shared__ double yp[kNB];
    const int i = threadIdx.x;
    double *yb = y + p * kNB;
    yp[i] = yb[i];
    __syncthreads();
    const double *D = DinvT + p * kNB * kNB;
    double s = 0.0;
    for (int m = 0; m <= i; ++m) s += D[(int64_t)m * kNB + i] * yp[m];
    yb[i] = s;
}

// forward solve, rows below block p: y_R -= L[R][block p] y_p (warp per row)
__global__ void k_fwd_upd(const double *L, int64_t ld, int64_t p, int64_t npad, double *y) {
    __shared__ double yp[kNB];
    const int ln = threadIdx.x & 31;
    if (threadIdx.x < kNB) yp[threadIdx.x] = y[p * kNB + threadIdx.x];
    __syncthreads();
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t R = (p + 1) * kNB + w; R < npad; R += nw) {
        const double *row = L + R * ld + p * kNB;
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) s += row[q * 32 + ln] * yp[q * 32 + ln];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (ln == 0) y[R] -= s;
    }
}

// backward solve, block p: y_p <- L_pp^-T y_p
__global__ void k_bwd_diag(const double *DinvT, int64_t p, double *y) {
    __shared__ double yp[kNB];
    const int i = threadIdx.x;
    double *yb = y + p * kNB;
    yp[i] = yb[i];
    __syncthreads();
    const double *D = DinvT + p * kNB * kNB + (int64_t)i * kNB;
    double s = 0.0;
    for (int m = i; m < kNB; ++m) s += D[m] * yp[m];
    yb[i] = s;
}

// backward solve, columns left of block p: y_c -= sum_m L[p*128+m][c] x_p[m]
__global__ void k_bwd_upd(const double *L, int64_t ld, int64_t p, double *y) {
    __shared__ double xp[kNB];
    if (threadIdx.x < kNB) xp[threadIdx.x] = y[p * kNB + threadIdx.x];
    __syncthreads();
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p * kNB) return;
    const double *col = L + p * kNB * ld + c;
    double s = 0.0;
    for (int m = 0; m < kNB; ++m) s += col[(int64_t)m * ld] * xp[m];
    y[c] -= s;
}

// y = F x, dense full matrix, one warp per row
__global__ void k_gemv(const double *F, int64_t ld, int64_t npad, const double *x, double *y) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = w; r < npad; r += nw) {
        const double *row = F + r * ld;
        double s = 0.0;
        for (int64_t j = ln; j < npad; j += 32) s += row[j] * x[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (ln == 0) y[r] = s;
    }
}

__global__ void k_dotp(int64_t n, const double *a, const double *b, double *part) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_dotf(const double *part, double *out) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < kDotBlk; i += blockDim.x) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// scalars: [0] rz, [1] pq, [2] rz new, [3] rr, [4] bb, [5] squared length of the
// last correction alpha p, [6] p.p, [7] x.x
__global__ void k_cg_step(int64_t n, double *x, double *r, const double *p, const double *q, double *sc) {
    const double alpha = sc[1] != 0.0 ? sc[0] / sc[1] : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[5] = alpha * alpha * sc[6];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        r[i] -= alpha * q[i];
    }
}

__global__ void k_cg_dir(int64_t n, double *p, const double *z, double *sc) {
    const double beta = sc[0] != 0.0 ? sc[2] / sc[0] : 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

__global__ void k_cg_roll(double *sc) {
    if (threadIdx.x == 0 && blockIdx.x == 0) sc[0] = sc[2];
}

__global__ void k_sub_vec(int64_t n, const double *b, const double *ax, double *r) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - ax[i];
}

struct DenseWork {
    int64_t npad = 0, np = 0;
    double *L = nullptr, *F = nullptr, *DinvT = nullptr;
    float *hi = nullptr, *lo = nullptr;
    double *b = nullptr, *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
    double *part = nullptr, *sc = nullptr;
    int32_t *err = nullptr;
    void release() {
        cudaFree(L); cudaFree(F); cudaFree(DinvT); cudaFree(hi); cudaFree(lo);
        cudaFree(b); cudaFree(x); cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q);
        cudaFree(part); cudaFree(sc); cudaFree(err);
    }
};

void precond(const DenseWork &w, const double *in, double *out, cudaStream_t s) {
    cudaMemcpyAsync(out, in, sizeof(double) * w.npad, cudaMemcpyDeviceToDevice, s);
    for (int64_t p = 0; p < w.np; ++p) {
        k_fwd_diag<<<1, kNB, 0, s>>>(w.DinvT, p, out);
        const int64_t rows = w.npad - (p + 1) * kNB;
        if (rows > 0)
            k_fwd_upd<<<(unsigned)std::min<int64_t>((rows + 7) / 8, 1216), 256, 0, s>>>(w.L, w.npad, p, w.npad, out);
    }
    for (int64_t p = w.np - 1; p >= 0; --p) {
        k_bwd_diag<<<1, kNB, 0, s>>>(w.DinvT, p, out);
        if (p > 0) k_bwd_upd<<<(unsigned)((p * kNB + 255) / 256), 256, 0, s>>>(w.L, w.npad, p, out);
    }
}

void dotv(const DenseWork &w, const double *a, const double *b, double *out, cudaStream_t s) {
    k_dotp<<<kDotBlk, 256, 0, s>>>(w.npad, a, b, w.part);
    k_dotf<<<1, 256, 0, s>>>(w.part, out);
}

}  // namespace

// Solve A x = b for the packed SPD matrix Ap (n, device) and the device
// vector bx (b in, x out).  mode 0: FP64 factor, mode 1: tensor-core
// factor; both refined by preconditioned CG in FP64 to rtol.
int32_t dense_solve_pcg(mpgpu_ctx *c, int32_t n, const double *Ap, double *bx, int mode, double rtol,
                        int32_t itnlim, mpgpu_solveinfo *info, double *invOut) {
    cudaStream_t s = c->stream;
    DenseWork w;
    w.npad = ((int64_t)n + kNB - 1) / kNB * kNB;
    w.np = w.npad / kNB;
    const int64_t nn = w.npad * w.npad;
    int32_t rc = MPGPU_OK;
    cudaError_t e = cudaMalloc(&w.L, sizeof(double) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&w.F, sizeof(double) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&w.DinvT, sizeof(double) * w.np * kNB * kNB);
    if (e == cudaSuccess) e = cudaMalloc(&w.hi, sizeof(float) * w.npad * kNB);
    if (e == cudaSuccess) e = cudaMalloc(&w.lo, sizeof(float) * w.npad * kNB);
    for (double **v : {&w.b, &w.x, &w.r, &w.z, &w.p, &w.q})
        if (e == cudaSuccess) e = cudaMalloc(v, sizeof(double) * w.npad);
    if (e == cudaSuccess) e = cudaMalloc(&w.part, sizeof(double) * kDotBlk);
    if (e == cudaSuccess) e = cudaMalloc(&w.sc, sizeof(double) * 16);
    if (e == cudaSuccess) e = cudaMalloc(&w.err, sizeof(int32_t));
    if (e != cudaSuccess) { w.release(); return cuda_err(c, e, "dense solve allocation"); }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    cudaMemsetAsync(w.F, 0, sizeof(double) * nn, s);
    k_packed_to_dense<<<4096, 256, 0, s>>>(Ap, n, w.npad, w.L, w.F);
    if (w.npad > n) k_pad_identity<<<(unsigned)((w.npad - n + 255) / 256), 256, 0, s>>>(w.F, w.npad, n, w.npad);
    cudaMemsetAsync(w.b, 0, sizeof(double) * w.npad, s);
    cudaMemcpyAsync(w.b, bx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    // factorisation; a non-positive pivot of the low-precision factor is
    // cured by a growing diagonal shift (the CG iterations remove it)
    double shift = 0.0;
    int tries = 0;
    for (;; ++tries) {
        k_copy_lower_shift<<<4096, 256, 0, s>>>(w.F, w.L, w.npad, shift);
        int32_t bad = -1;
        rc = dense_cholesky_device(c, w.L, w.npad, mode, w.hi, w.lo, w.err, &bad);
        if (rc != MPGPU_ERR_FACTOR || tries >= 6) break;
        shift = shift == 0.0 ? 1e-7 : shift * 10.0;
    }
    if (rc != MPGPU_OK) { w.release(); return rc; }
    cudaEvent_t eF;
    cudaEventCreate(&eF);
    cudaEventRecord(eF, s);
    const int trtriSmem = (kNB * kNB + kNB) * (int)sizeof(double);
    MPG_CUDA(c, cudaFuncSetAttribute(k_trtri_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, trtriSmem));
    k_trtri_blocks<<<(unsigned)w.np, 256, trtriSmem, s>>>(w.L, w.npad, w.DinvT);
    // x0 = M^-1 b, r = b - A x0, z = M^-1 r, p = z
    precond(w, w.b, w.x, s);
    const unsigned gv = (unsigned)std::min<int64_t>((w.npad + 7) / 8, 4096);
    k_gemv<<<gv, 256, 0, s>>>(w.F, w.npad, w.npad, w.x, w.q);
    k_sub_vec<<<(unsigned)((w.npad + 255) / 256), 256, 0, s>>>(w.npad, w.b, w.q, w.r);
    precond(w, w.r, w.z, s);
    cudaMemcpyAsync(w.p, w.z, sizeof(double) * w.npad, cudaMemcpyDeviceToDevice, s);
    dotv(w, w.r, w.z, w.sc + 0, s);
    dotv(w, w.b, w.b, w.sc + 4, s);
    // one CG iteration as a CUDA graph (its ~600 launches replayed cheaply)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    const unsigned ge = (unsigned)std::min<int64_t>((w.npad + 255) / 256, 4096);
    MPG_CUDA(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    k_gemv<<<gv, 256, 0, s>>>(w.F, w.npad, w.npad, w.p, w.q);
    dotv(w, w.p, w.q, w.sc + 1, s);
    dotv(w, w.p, w.p, w.sc + 6, s);
    k_cg_step<<<ge, 256, 0, s>>>(w.npad, w.x, w.r, w.p, w.q, w.sc);
    dotv(w, w.x, w.x, w.sc + 7, s);
    precond(w, w.r, w.z, s);
    dotv(w, w.r, w.z, w.sc + 2, s);
    k_cg_dir<<<ge, 256, 0, s>>>(w.npad, w.p, w.z, w.sc);
    k_cg_roll<<<1, 32, 0, s>>>(w.sc);
    dotv(w, w.r, w.r, w.sc + 3, s);
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&gexec, graph, 0);
    if (ce != cudaSuccess) { w.release(); return cuda_err(c, ce, "CG graph"); }
    // stop when the relative residual is below rtol AND the last correction
    // is below kRefineXtol of the solution: a residual test alone leaves an
    // error of about cond(A) * rtol, which differs between factors of
    // different precision; the correction test brings every form to the
    // same FP64 solution
    int itn = 0, istop = 0;
    double hs[8];
    const double tol2 = rtol * rtol, xtol2 = kRefineXtol * kRefineXtol;
    while (itn < itnlim) {
        const int batch = std::min(4, itnlim - itn);
        for (int k = 0; k < batch; ++k) cudaGraphLaunch(gexec, s);
        itn += batch;
        MPG_CUDA(c, cudaMemcpyAsync(hs, w.sc, sizeof(hs), cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        if (!(hs[3] == hs[3]) || !(hs[5] == hs[5])) { istop = 9; break; }
        if (hs[3] <= tol2 * hs[4] && hs[5] <= xtol2 * hs[7]) { istop = 1; break; }
    }
    if (istop == 0) istop = 3;
    cudaMemcpyAsync(bx, w.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    // the inverse from the same factor (inversion forms): X = L^-1, Z = X^T X
    cudaEvent_t eR;
    cudaEventCreate(&eR);
    cudaEventRecord(eR, s);
    int32_t rcInv = MPGPU_OK;
    if (invOut && istop != 9) rcInv = dense_inverse_device(c, w.L, w.npad, n, mode, w.DinvT, w.F, invOut, w.err);
    cudaEventRecord(e1, s);
    MPG_CUDA(c, cudaStreamSynchronize(s));
    float ms = 0.0f, msF = 0.0f, msR = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventElapsedTime(&msF, e0, eF);
    cudaEventElapsedTime(&msR, e0, eR);
    cudaEventDestroy(eF);
    cudaEventDestroy(eR);
    if (rcInv != MPGPU_OK) {
        cudaGraphExecDestroy(gexec);
        cudaGraphDestroy(graph);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        w.release();
        return rcInv;
    }
    if (info) {
        info->msFactor = msF;
        info->msRefine = msR - msF;
        info->msInverse = ms - msR;
        info->itn = itn;
        info->istop = istop;
        info->nrank = n;
        info->evmin = shift;
        info->evmax = hs[4] > 0.0 ? std::sqrt(hs[3] / hs[4]) : 0.0;
        info->dxRel = hs[7] > 0.0 ? std::sqrt(hs[5] / hs[7]) : 0.0;
        info->ms = ms;
    }
    cudaGraphExecDestroy(gexec);
    cudaGraphDestroy(graph);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    w.release();
    return istop == 9 ? set_err(c, MPGPU_ERR_NAN, "NaN in the refined dense solve") : MPGPU_OK;
}
