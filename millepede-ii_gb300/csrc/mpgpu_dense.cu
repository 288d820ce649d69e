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
constexpr int kSuperPanels = 4;   // panels per block column of the tensor-core factorisation

// ------------------------------------------------------------ panel kernels
// Cholesky of the 128 x 128 diagonal block at (k0, k0), in shared memory.
__global__ void __launch_bounds__(512) k_potrf128(double *A, int64_t ld, int64_t k0, int32_t *err) {
    extern __shared__ __align__(16) double sa[];   // 128 x 129
    constexpr int S = kNB + 1;
    __shared__ int bad;
    __shared__ double sinv;   // reciprocal of the pivot: one FP64 division per column, not one per thread
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
            const double piv = d > 0.0 ? sqrt(d) : 1.0;
            if (!(d > 0.0)) bad = 1;
            sa[j * S + j] = piv;
            sinv = 1.0 / piv;
        }
        __syncthreads();
        const double inv = sinv;
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
// mode 0: right-looking by 128-wide panels, FP64 trailing updates.
// mode 1: block columns of kSuperPanels panels: inside a block column the
// 128-wide panels are factorised and update the rest of the block column;
// the trailing matrix then receives the whole block column at once, K = 512
// accumulated in tensor memory before one FP64 read-modify-write per tile
// (tcgen05 3xTF32 tile products, mpgpu_inverse.cu).  hiBuf/loBuf hold the
// TF32 split of one block column: npad x (128 * kSuperPanels) floats each.
int32_t dense_cholesky_device(mpgpu_ctx *c, double *A, int64_t npad, int mode, float *hiBuf, float *loBuf,
                              int32_t *dErr, int32_t *badPanel) {
    cudaStream_t s = c->stream;
    const int64_t ld = npad;
    const int32_t np = (int32_t)(npad / kNB);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    const int potrfSmem = kNB * (kNB + 1) * (int)sizeof(double);
    const int trsmSmem = (kNB * kNB + kNB) * (int)sizeof(double);
    MPG_CUDA(c, smem_optin((const void *)k_potrf128));
    MPG_CUDA(c, smem_optin((const void *)k_trsm128));
    MPG_CUDA(c, cudaMemsetAsync(dErr, 0, sizeof(int32_t), s));
    auto panel = [&](int32_t p, cudaStream_t st) -> int64_t {   // potrf + trsm of panel p; rows below it
        const int64_t k0 = (int64_t)p * kNB;
        k_potrf128<<<1, 512, potrfSmem, st>>>(A, ld, k0, dErr);
        const int64_t rows = npad - k0 - kNB;
        if (rows > 0) {
            const int64_t tb = std::min<int64_t>((rows + 7) / 8, (int64_t)nsm);
            k_trsm128<<<(unsigned)tb, 256, trsmSmem, st>>>(A, ld, k0, rows);
        }
        return rows;
    };
    if (mode == 0) {
        for (int32_t p = 0; p < np; ++p) {
            const int64_t rows = panel(p, s);
            if (rows <= 0) break;
            const int32_t T = (int32_t)(rows / 64);
            const int64_t ntile = (int64_t)T * (T + 1) / 2;
            k_syrk_fp64<<<(unsigned)ntile, 256, 0, s>>>(A, ld, (int64_t)p * kNB, (int64_t)(p + 1) * kNB, T);
            MPG_CUDA(c, cudaGetLastError());
        }
    } else {
        // Task lists, copied once: (1) the updates inside every block
        // column (panel p updates the tiles (i, j) of the later panels j of
        // its block column, i >= j); (2) per block column, the trailing
        // tiles of the next block column, which the next panels need first.
        std::vector<tc::TileTask> tk;
        std::vector<int64_t> off(np + 1, 0);
        const int32_t nbc = (np + kSuperPanels - 1) / kSuperPanels;
        std::vector<int64_t> offN(nbc + 1, 0);
        for (int32_t s0 = 0; s0 < np; s0 += kSuperPanels) {
            const int32_t e = std::min(s0 + kSuperPanels, np);
            for (int32_t p = s0; p < e; ++p) {
                off[p] = (int64_t)tk.size();
                for (int32_t jj = p + 1; jj < e; ++jj)
                    for (int32_t i = jj; i < np; ++i) tk.push_back({i, jj, p - s0, p - s0 + 1, i, jj});
            }
        }
        off[np] = (int64_t)tk.size();
        for (int32_t b = 0; b < nbc; ++b) {
            const int32_t s0 = b * kSuperPanels, e = std::min(s0 + kSuperPanels, np);
            const int32_t e2 = std::min(e + kSuperPanels, np);
            offN[b] = (int64_t)tk.size();
            for (int32_t jj = e; jj < e2; ++jj)
                for (int32_t i = jj; i < np; ++i) tk.push_back({i, jj, 0, e - s0, i, jj});
        }
        offN[nbc] = (int64_t)tk.size();
        // panels (and the tiles the next panels need) on a high-priority
        // stream, the bulk of each trailing update on a second stream: the
        // panels of block column b + 1 run while the bulk of block column b
        // is updated (look-ahead); the TF32 split of a block column is
        // double-buffered for that overlap
        struct Res {
            tc::TileTask *task = nullptr;
            float *hl[4] = {nullptr, nullptr, nullptr, nullptr};
            cudaStream_t sp = nullptr, sb = nullptr;
            cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
            cudaStream_t s0 = nullptr;   // the caller's stream (the buffers are ordered on it)
            ~Res() {
                if (sp) cudaStreamSynchronize(sp);
                if (sb) cudaStreamSynchronize(sb);
                for (void *p : {(void *)task, (void *)hl[2], (void *)hl[3]})   // hl[0], hl[1] are the caller's
                    if (p) cudaFreeAsync(p, s0);
                for (cudaEvent_t e : ev)
                    if (e) cudaEventDestroy(e);
                if (sp) cudaStreamDestroy(sp);
                if (sb) cudaStreamDestroy(sb);
            }
        } R;
        const int64_t splitLen = npad * kNB * kSuperPanels;
        R.s0 = s;
        MPG_CUDA(c, cudaMallocAsync(&R.task, sizeof(tc::TileTask) * std::max<size_t>(tk.size(), 1), s));
        R.hl[0] = hiBuf;
        R.hl[1] = loBuf;
        MPG_CUDA(c, cudaMallocAsync(&R.hl[2], sizeof(float) * splitLen, s));
        MPG_CUDA(c, cudaMallocAsync(&R.hl[3], sizeof(float) * splitLen, s));
        int lo = 0, hiPrio = 0;
        MPG_CUDA(c, cudaDeviceGetStreamPriorityRange(&lo, &hiPrio));
        MPG_CUDA(c, cudaStreamCreateWithPriority(&R.sp, cudaStreamNonBlocking, hiPrio));
        MPG_CUDA(c, cudaStreamCreateWithPriority(&R.sb, cudaStreamNonBlocking, lo));
        for (cudaEvent_t &e : R.ev) MPG_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        cudaEvent_t evStart = R.ev[0], evBulk = R.ev[1], evPanels = R.ev[2], evEnd = R.ev[3];
        if (!tk.empty())
            MPG_CUDA(c, cudaMemcpyAsync(R.task, tk.data(), sizeof(tc::TileTask) * tk.size(), cudaMemcpyHostToDevice,
                                        s));
        MPG_CUDA(c, cudaEventRecord(evStart, s));
        MPG_CUDA(c, cudaStreamWaitEvent(R.sp, evStart, 0));
        MPG_CUDA(c, cudaStreamWaitEvent(R.sb, evStart, 0));
        MPG_CUDA(c, cudaEventRecord(evBulk, R.sb));
        hiBuf = nullptr;   // the buffers are R.hl from here on
        loBuf = nullptr;
        for (int32_t b = 0; b < nbc; ++b) {
            const int32_t s0 = b * kSuperPanels, e = std::min(s0 + kSuperPanels, np);
            const int32_t e2 = std::min(e + kSuperPanels, np);
            float *hb = R.hl[2 * (b & 1)], *lb = R.hl[2 * (b & 1) + 1];
            const tc::TcOp op{hb, lb, kSuperPanels};
            bool last = false;
            for (int32_t p = s0; p < e; ++p) {
                const int64_t rows = panel(p, R.sp);
                if (rows <= 0) { last = true; break; }
                MPG_CUDA(c, tc_split_tiles(A, ld, p + 1, np, p, p + 1, hb, lb, kSuperPanels, s0, R.sp));
                MPG_CUDA(c, tc_tile_gemm(op, op, A, ld, R.task + off[p], off[p + 1] - off[p], 0, 0, -1.0, 1.0,
                                         dErr, R.sp));
            }
            if (last) break;
            if (e >= np) break;
            // the next block column's tiles, after the previous bulk update
            MPG_CUDA(c, cudaStreamWaitEvent(R.sp, evBulk, 0));
            MPG_CUDA(c, tc_tile_gemm(op, op, A, ld, R.task + offN[b], offN[b + 1] - offN[b], 0, 0, -1.0, 1.0, dErr,
                                     R.sp));
            MPG_CUDA(c, cudaEventRecord(evPanels, R.sp));
            // the bulk: tiles (i, j >= e2), on the second stream
            const int64_t T = np - e2;
            MPG_CUDA(c, cudaStreamWaitEvent(R.sb, evPanels, 0));
            if (T > 0)
                MPG_CUDA(c, tc_tile_gemm(op, op, A, ld, nullptr, T * (T + 1) / 2, e2, e - s0, -1.0, 1.0, dErr, R.sb));
            MPG_CUDA(c, cudaEventRecord(evBulk, R.sb));
        }
        MPG_CUDA(c, cudaGetLastError());
        MPG_CUDA(c, cudaEventRecord(evEnd, R.sb));
        MPG_CUDA(c, cudaStreamWaitEvent(s, evEnd, 0));
        MPG_CUDA(c, cudaEventRecord(evPanels, R.sp));
        MPG_CUDA(c, cudaStreamWaitEvent(s, evPanels, 0));
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
    if (e == cudaSuccess) e = cudaMalloc(&hi, sizeof(float) * npad * kNB * kSuperPanels);
    if (e == cudaSuccess) e = cudaMalloc(&lo, sizeof(float) * npad * kNB * kSuperPanels);
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

// packed lower triangle (n) -> dense lower (factor; not written when Lo is
// null) and dense full (for the matrix-vector products), both npad x npad
// row-major
__global__ void k_packed_to_dense(const double *Ap, int64_t n, int64_t npad, double *Lo, double *F) {
    const int64_t nn = n * (n + 1) / 2;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = (int64_t)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
        while (i * (i + 1) / 2 > e) i--;
        while ((i + 1) * (i + 2) / 2 <= e) i++;
        const int64_t j = e - i * (i + 1) / 2;
        const double v = Ap[e];
        if (Lo) Lo[i * npad + j] = v;
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

// ---- the preconditioner's triangular solves by super-blocks of kSB rows:
// X_b = L_bb^-1 of every diagonal super-block (from the 128-row inverse
// blocks by block forward substitution in FP64 tile products), then each
// solve is nsb steps of (X_b times the block, update of the rows below or
// the columns left) instead of np steps of 128 rows: a quarter of the
// dependent launches of a CG iteration
constexpr int kSB = 4 * kNB;   // rows of a super-block

// XS rows of panel p, local columns of its 128-column slot: L_pp^-1 (lower)
__global__ void k_sb_set_diag(const double *DinvT, int64_t np, double *XS) {
    const int64_t total = np * kNB * kNB;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = e / (kNB * kNB);
        const int r = (int)(e % (kNB * kNB)) / kNB, c = (int)(e % kNB);
        const double v = c <= r ? DinvT[p * kNB * kNB + (int64_t)c * kNB + r] : 0.0;
        XS[(p * kNB + r) * kSB + (p % 4) * kNB + c] = v;
    }
}

// XT_b = X_b^T per super-block (rows of the super-block, kSB columns each)
__global__ void k_sb_transpose(const double *XS, int64_t npad, double *XT) {
    const int64_t total = npad * kSB;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = e / kSB;
        const int c = (int)(e % kSB);
        const int64_t b0 = row / kSB * kSB;
        const int r = (int)(row - b0);
        if (b0 + c < npad) XT[(b0 + c) * kSB + r] = XS[e];
    }
}

// out[row0 + r] = sum_c X[row0 + r][c] in[row0 + c] over c <= r (lower) or
// c >= r, c < size; a warp per row, lanes over c, tree sum over the lanes
__global__ void k_sb_diag(const double *X, int64_t row0, int size, const double *in, double *out, int lower) {
    const int ln = threadIdx.x & 31;
    const int r = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (r >= size) return;
    const double *xr = X + (row0 + r) * kSB;
    const int c0 = lower ? 0 : r, c1 = lower ? r + 1 : size;
    double sum = 0.0;
    for (int c = c0 + ln; c < c1; c += 32) sum += xr[c] * in[row0 + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (ln == 0) out[row0 + r] = sum;
}

// v_R -= L[R][row0 .. row0 + size) z_b for the rows R >= row0 + size (warp per row)
__global__ void k_sb_fwd_upd(const double *L, int64_t ld, int64_t row0, int size, int64_t npad, const double *z,
                             double *v) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t R = row0 + size + w; R < npad; R += nw) {
        const double *row = L + R * ld + row0;
        double sum = 0.0;
        for (int c = ln; c < size; c += 32) sum += row[c] * z[row0 + c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (ln == 0) v[R] -= sum;
    }
}

// z_c -= sum_m L[row0 + m][c] o[row0 + m] for the columns c < row0: 64
// columns per CTA, the m range in four quarters summed in order
__global__ void __launch_bounds__(256) k_sb_bwd_upd(const double *L, int64_t ld, int64_t row0, int size,
                                                    const double *o, double *z) {
    __shared__ double part[4][64];
    const int cl = threadIdx.x & 63, g = threadIdx.x >> 6;
    const int64_t c = (int64_t)blockIdx.x * 64 + cl;
    const int q = (size + 3) / 4, m0 = g * q, m1 = min(size, m0 + q);
    double sum = 0.0;
    if (c < row0) {
        const double *col = L + row0 * ld + c;
#pragma unroll 8
        for (int m = m0; m < m1; ++m) sum += col[(int64_t)m * ld] * o[row0 + m];
    }
    part[g][cl] = sum;
    __syncthreads();
    if (g == 0 && c < row0) z[c] -= ((part[0][cl] + part[1][cl]) + part[2][cl]) + part[3][cl];
}

struct DenseWork {
    int64_t npad = 0, np = 0;
    double *L = nullptr, *F = nullptr, *DinvT = nullptr;   // factor, matrix, inverse 128-row blocks (transposed)
    double *XS = nullptr, *XT = nullptr, *XW = nullptr;    // super-block inverses, their transposes, scratch
    tc::TileTask *sbTask = nullptr;                        // task lists of the super-block inverses
    float *hi = nullptr, *lo = nullptr;
    double *b = nullptr, *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
    double *t1 = nullptr, *t2 = nullptr;                   // the preconditioner's working vectors
    double *part = nullptr, *sc = nullptr;
    int32_t *err = nullptr;
    void release() {
        cudaFree(L); cudaFree(F); cudaFree(DinvT); cudaFree(XS); cudaFree(XT); cudaFree(XW); cudaFree(sbTask);
        cudaFree(hi); cudaFree(lo);
        cudaFree(b); cudaFree(x); cudaFree(r); cudaFree(z); cudaFree(p); cudaFree(q); cudaFree(t1); cudaFree(t2);
        cudaFree(part); cudaFree(sc); cudaFree(err);
    }
};

// X_b for every super-block from L and the 128-row inverse blocks:
// X_jj = L_jj^-1, and for i = j + d (d = 1, 2, 3) T = sum_{k=j}^{i-1} L_ik X_kj,
// X_ij = -L_ii^-1 T (one wave of tile products per d over all super-blocks)
cudaError_t build_super_inverse(DenseWork &w, cudaStream_t s) {
    const int64_t np = w.np, nsb = (np + 3) / 4;
    cudaError_t e = cudaMemsetAsync(w.XS, 0, sizeof(double) * w.npad * kSB, s);
    if (e != cudaSuccess) return e;
    k_sb_set_diag<<<(unsigned)std::min<int64_t>(np * 64, 4096), 256, 0, s>>>(w.DinvT, np, w.XS);
    std::vector<tc::TileTask> tk;
    std::vector<int64_t> wave(7, 0);
    for (int d = 1; d <= 3; ++d) {
        wave[2 * d - 2] = (int64_t)tk.size();
        for (int64_t b = 0; b < nsb; ++b) {
            const int32_t t0 = (int32_t)(4 * b), npb = (int32_t)std::min<int64_t>(4, np - 4 * b);
            for (int32_t j = 0; j + d < npb; ++j) tk.push_back({t0 + j + d, j, t0 + j, t0 + j + d, t0 + j + d, j});
        }
        wave[2 * d - 1] = (int64_t)tk.size();
        for (int64_t b = 0; b < nsb; ++b) {
            const int32_t t0 = (int32_t)(4 * b), npb = (int32_t)std::min<int64_t>(4, np - 4 * b);
            for (int32_t j = 0; j + d < npb; ++j) tk.push_back({0, j, t0 + j + d, t0 + j + d + 1, t0 + j + d, j});
        }
    }
    wave[6] = (int64_t)tk.size();
    if (!tk.empty()) {
        e = cudaMemcpyAsync(w.sbTask, tk.data(), sizeof(tc::TileTask) * tk.size(), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        for (int d = 1; d <= 3 && e == cudaSuccess; ++d) {
            const int64_t a0 = wave[2 * d - 2], a1 = wave[2 * d - 1], a2 = wave[2 * d];
            e = fp64_tile_gemm(w.L, w.npad, 0, w.XS, kSB, 1, w.XW, kSB, w.sbTask + a0, a1 - a0, 1.0, 0.0, s);
            if (e == cudaSuccess)
                e = fp64_tile_gemm(w.DinvT, kNB, 1, w.XW, kSB, 1, w.XS, kSB, w.sbTask + a1, a2 - a1, -1.0, 0.0, s);
        }
        // the host task list must live until the copy has run
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e != cudaSuccess) return e;
    k_sb_transpose<<<(unsigned)std::min<int64_t>((w.npad * kSB + 255) / 256, 8192), 256, 0, s>>>(w.XS, w.npad, w.XT);
    return cudaGetLastError();
}

// out = L^-T L^-1 in by super-block steps (in is not modified)
void precond(const DenseWork &w, const double *in, double *out, cudaStream_t s) {
    const int64_t nsb = (w.np + 3) / 4;
    double *v = w.t1, *zz = w.t2;
    cudaMemcpyAsync(v, in, sizeof(double) * w.npad, cudaMemcpyDeviceToDevice, s);
    for (int64_t b = 0; b < nsb; ++b) {
        const int64_t row0 = b * kSB;
        const int size = (int)std::min<int64_t>(kSB, w.npad - row0);
        k_sb_diag<<<(unsigned)((size + 7) / 8), 256, 0, s>>>(w.XS, row0, size, v, zz, 1);
        const int64_t rows = w.npad - row0 - size;
        if (rows > 0)
            k_sb_fwd_upd<<<(unsigned)std::min<int64_t>((rows + 7) / 8, 1216), 256, 0, s>>>(w.L, w.npad, row0, size,
                                                                                           w.npad, zz, v);
    }
    for (int64_t b = nsb - 1; b >= 0; --b) {
        const int64_t row0 = b * kSB;
        const int size = (int)std::min<int64_t>(kSB, w.npad - row0);
        k_sb_diag<<<(unsigned)((size + 7) / 8), 256, 0, s>>>(w.XT, row0, size, zz, out, 0);
        if (row0 > 0) k_sb_bwd_upd<<<(unsigned)((row0 + 63) / 64), 256, 0, s>>>(w.L, w.npad, row0, size, out, zz);
    }
}

void dotv(const DenseWork &w, const double *a, const double *b, double *out, cudaStream_t s) {
    k_dotp<<<kDotBlk, 256, 0, s>>>(w.npad, a, b, w.part);
    k_dotf<<<1, 256, 0, s>>>(w.part, out);
}

// ---- constraint elimination in compact WY form (Q = H_1 ... H_m = I - U T U^T)
constexpr int kWy = 128;      // padded number of constraints (columns of U)
constexpr int kWyBlk = 152;   // fixed reduction shape of U^T x

// U (npad x 128, row-major) and U^T (128 x npad) from the Householder
// vectors: u_k = V_k on [0, kn_k), Vk_k at kn_k = npar - ncon + k, 0 beyond
__global__ void k_build_u(const double *V, const double *Vk, int32_t npar, int32_t m, int64_t npad, double *U,
                          double *UT) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < npad * kWy;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / kWy;
        const int k = (int)(e % kWy);
        double u = 0.0;
        if (k < m && i < npar) {
            const int64_t kn = npar - m + k;
            u = i < kn ? V[(int64_t)k * npar + i] : (i == kn ? Vk[k] : 0.0);
        }
        U[e] = u;
        UT[(int64_t)k * npad + i] = u;
    }
}

// T padded to 128 x 128, and its transpose
__global__ void k_pad_t(const double *T, int32_t m, double *T128, double *TT128) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kWy * kWy; e += gridDim.x * blockDim.x) {
        const int r = e / kWy, c = e % kWy;
        const double t = (r < m && c < m) ? T[r * m + c] : 0.0;
        T128[e] = t;
        TT128[c * kWy + r] = t;
    }
}

// C (128 x 128) = op(A) op(B) for 128 x 128 row-major A, B (op: transpose when t)
__global__ void k_small_mm(const double *A, int ta, const double *B, int tb, double *C) {
    const int r = blockIdx.x, cc = threadIdx.x;
    double acc = 0.0;
    for (int k = 0; k < kWy; ++k)
        acc = fma(ta ? A[k * kWy + r] : A[r * kWy + k], tb ? B[cc * kWy + k] : B[k * kWy + cc], acc);
    C[r * kWy + cc] = acc;
}

// M = U^T W (128 x 128): block a, thread b, rows in order
__global__ void k_utw(int64_t npad, const double *U, const double *W, double *M) {
    const int a = blockIdx.x, b = threadIdx.x;
    double acc = 0.0;
    for (int64_t i = 0; i < npad; ++i) acc = fma(U[i * kWy + a], W[i * kWy + b], acc);
    M[a * kWy + b] = acc;
}

// Z = W T^T - 1/2 U S (TT = T^T), then ZU = [Z | U] and UZ = [U | Z] (npad x 256)
__global__ void k_wy_z(int64_t npad, const double *W, const double *U, const double *TT, const double *S, double *ZU,
                       double *UZ) {
    const int a = threadIdx.x;
    for (int64_t i = blockIdx.x; i < npad; i += gridDim.x) {
        double z = 0.0, h = 0.0;
        for (int b = 0; b < kWy; ++b) {
            z = fma(W[i * kWy + b], TT[b * kWy + a], z);
            h = fma(U[i * kWy + b], S[b * kWy + a], h);
        }
        z -= 0.5 * h;
        const double u = U[i * kWy + a];
        ZU[i * 2 * kWy + a] = z;
        ZU[i * 2 * kWy + kWy + a] = u;
        UZ[i * 2 * kWy + a] = u;
        UZ[i * 2 * kWy + kWy + a] = z;
    }
}

// the eliminated rows and columns of the factor's input set to the identity
__global__ void k_identity_rows(double *L, int64_t ld, int64_t nfit, int64_t npad) {
    for (int64_t i = nfit + blockIdx.x; i < npad; i += gridDim.x)
        for (int64_t j = threadIdx.x; j <= i; j += blockDim.x) L[i * ld + j] = i == j ? 1.0 : 0.0;
}

__global__ void k_scale_diag(double *L, int64_t ld, int64_t n, double f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) L[i * ld + i] *= f;
}

// partial sums of U^T x over fixed row ranges (block b: rows b, b + kWyBlk, ...)
__global__ void k_ut_x(int64_t npad, const double *U, const double *x, double *part) {
    const int k = threadIdx.x;
    double acc = 0.0;
    for (int64_t i = blockIdx.x; i < npad; i += kWyBlk) acc = fma(U[i * kWy + k], x[i], acc);
    part[blockIdx.x * kWy + k] = acc;
}

// v = T t or T^T t, t = sum of the partials in block order
__global__ void k_t_coef(const double *part, const double *T, int trans, double *v) {
    __shared__ double t[kWy];
    const int k = threadIdx.x;
    double acc = 0.0;
    for (int b = 0; b < kWyBlk; ++b) acc += part[b * kWy + k];
    t[k] = acc;
    __syncthreads();
    double r = 0.0;
    for (int c = 0; c < kWy; ++c) r = fma(trans ? T[c * kWy + k] : T[k * kWy + c], t[c], r);
    v[k] = r;
}

// x -= U v
__global__ void k_sub_uv(int64_t npad, const double *U, const double *v, double *x) {
    __shared__ double sv[kWy];
    if (threadIdx.x < kWy) sv[threadIdx.x] = v[threadIdx.x];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int k = 0; k < kWy; ++k) acc = fma(U[i * kWy + k], sv[k], acc);
        x[i] -= acc;
    }
}

// y = P b + (I - P) x, P keeping the first nfit components
__global__ void k_reduce_op(int64_t npad, int64_t nfit, const double *b, const double *x, double *y) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = i < nfit ? b[i] : x[i];
}

// a = P x (first nfit components, zeros beyond), or with y: [x_fit; y] at nfit..
__global__ void k_expand(int64_t npad, int64_t nfit, int64_t nfull, const double *x, const double *y, double *a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = i < nfit ? (x ? x[i] : 0.0) : ((y && i < nfull) ? y[i - nfit] : 0.0);
}

__global__ void k_sub_to(int64_t n, const double *a, const double *b, double *r) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = a[i] - b[i];
}

// WY buffers of the constraint elimination: U, U^T, T, T^T, W, M, S, the
// split operands, scratch
struct WyBufs {
    double *U = nullptr, *UT = nullptr, *T = nullptr, *TT = nullptr, *W = nullptr, *M = nullptr, *S = nullptr,
           *X = nullptr, *ZU = nullptr, *UZ = nullptr, *a = nullptr, *part = nullptr, *v = nullptr;
    float *zh = nullptr, *zl = nullptr, *uh = nullptr, *ul = nullptr;
    void release() {
        for (double *p : {U, UT, T, TT, W, M, S, X, ZU, UZ, a, part, v}) cudaFree(p);
        for (float *p : {zh, zl, uh, ul}) cudaFree(p);
        *this = WyBufs();
    }
};

// CG iterations a solve spends on the previous solve's factor before it
// factorises its own matrix
constexpr int kReuseItn = 40;

}  // namespace

// Workspace of the refined dense solve, kept in the context between the
// solves of a job: F (full FP64 matrix), L (the factor; also the split area
// of the WY products), the inverted diagonal blocks, the CG vectors and the
// WY buffers.  factorValid: L and DinvT hold the factor of an earlier solve
// with these sizes (cleared by a new layout or constraint set).
struct DenseResident {
    DenseWork w;
    WyBufs y;
    bool haveWy = false;
    bool factorValid = false;
    int factorMode = -1;
    int32_t factorN = 0, factorM = 0;
    double factorShift = 0.0;
};

void dense_release(mpgpu_ctx *c) {
    if (!c->dense) return;
    cudaStreamSynchronize(c->stream);
    c->dense->w.release();
    c->dense->y.release();
    delete c->dense;
    c->dense = nullptr;
}

void dense_invalidate(mpgpu_ctx *c) {
    if (c->dense) c->dense->factorValid = false;
}

namespace {
// the context's workspace for npad rows (with the WY buffers when wy),
// reallocated when the sizes differ
int32_t dense_workspace(mpgpu_ctx *c, int64_t npad, bool wy, DenseResident *&out) {
    if (c->dense && c->dense->w.npad == npad && (c->dense->haveWy || !wy)) {
        out = c->dense;
        return MPGPU_OK;
    }
    dense_release(c);
    DenseResident *D = new DenseResident();
    DenseWork &w = D->w;
    WyBufs &y = D->y;
    w.npad = npad;
    w.np = npad / kNB;
    const int64_t nn = npad * npad;
    cudaError_t e = cudaMalloc(&w.L, sizeof(double) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&w.F, sizeof(double) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&w.DinvT, sizeof(double) * w.np * kNB * kNB);
    for (double **v : {&w.XS, &w.XT, &w.XW})
        if (e == cudaSuccess) e = cudaMalloc(v, sizeof(double) * w.npad * kSB);
    if (e == cudaSuccess) e = cudaMalloc(&w.sbTask, sizeof(tc::TileTask) * (12 * ((w.np + 3) / 4) + 1));
    if (e == cudaSuccess) e = cudaMalloc(&w.hi, sizeof(float) * w.npad * kNB * kSuperPanels);
    if (e == cudaSuccess) e = cudaMalloc(&w.lo, sizeof(float) * w.npad * kNB * kSuperPanels);
    for (double **v : {&w.b, &w.x, &w.r, &w.z, &w.p, &w.q, &w.t1, &w.t2})
        if (e == cudaSuccess) e = cudaMalloc(v, sizeof(double) * w.npad);
    if (e == cudaSuccess) e = cudaMalloc(&w.part, sizeof(double) * kDotBlk);
    if (e == cudaSuccess) e = cudaMalloc(&w.sc, sizeof(double) * 16);
    if (e == cudaSuccess) e = cudaMalloc(&w.err, sizeof(int32_t));
    if (wy) {
        for (double **v : {&y.U, &y.UT, &y.W, &y.ZU, &y.UZ}) {
            const int64_t len = (v == &y.ZU || v == &y.UZ) ? 2 * w.npad * kWy : w.npad * kWy;
            if (e == cudaSuccess) e = cudaMalloc(v, sizeof(double) * len);
        }
        for (double **v : {&y.T, &y.TT, &y.M, &y.S, &y.X, &y.v})
            if (e == cudaSuccess) e = cudaMalloc(v, sizeof(double) * kWy * kWy);
        if (e == cudaSuccess) e = cudaMalloc(&y.a, sizeof(double) * w.npad);
        if (e == cudaSuccess) e = cudaMalloc(&y.part, sizeof(double) * kWyBlk * kWy);
        for (float **v : {&y.zh, &y.zl, &y.uh, &y.ul})
            if (e == cudaSuccess) e = cudaMalloc(v, sizeof(float) * w.npad * 2 * kWy);
    }
    D->haveWy = wy;
    if (e != cudaSuccess) {
        w.release();
        y.release();
        delete D;
        return cuda_err(c, e, "dense solve allocation");
    }
    c->dense = D;
    out = D;
    return MPGPU_OK;
}
}  // namespace

// Solve A x = b for the packed SPD matrix Ap (n, device) and the device
// vector bx (b in, x out).  mode 0: FP64 factor, mode 1: tensor-core
// factor; both refined by preconditioned CG in FP64 to rtol.
// With wy (mode 1): Ap is the original packed matrix of all n = N
// parameters and the ncon constraints are eliminated inside the solve.
// With P = H_1 ... H_m = I - U T U^T (compact WY of the QL reflections; P A
// P^T is what qlssq forms, P x what qlmlq calls Q^T x), the factor is that
// of the reduced matrix P A P^T formed by tensor-core 3xTF32 products (A' =
// A - Z U^T - U Z^T), a preconditioner only; CG runs in FP64 on the
// operator x -> (P A P^T x) restricted to the nfit = N - ncon fit
// parameters, with A the FP64 matrix and P applied in FP64.  bx: in the
// vector g of all N parameters, out the full correction P^T [x; y] (y:
// wy->y, the constraint part).  invOut: the inverse of the reduced matrix
// from the factor, packed over the nfit fit parameters.
// Mode 1 without invOut first preconditions with the factor of the
// previous solve of the same sizes (the matrix of the previous outlier
// iteration, kept in the context's workspace) and factorises only when CG
// has not converged within kReuseItn iterations; the stop rule is the same,
// so either way the solution is the refined FP64 one (MPGPU_FLAG_FRESH_FACTOR
// factorises at every solve).
int32_t dense_solve_pcg(mpgpu_ctx *c, int32_t n, const double *Ap, double *bx, int mode, double rtol,
                        int32_t itnlim, mpgpu_solveinfo *info, double *invOut, const DenseWyElim *wy) {
    cudaStream_t s = c->stream;
    const int64_t npadN = ((int64_t)n + kNB - 1) / kNB * kNB;
    DenseResident *D = nullptr;
    int32_t rc = dense_workspace(c, npadN, wy != nullptr, D);
    if (rc != MPGPU_OK) return rc;
    DenseWork &w = D->w;
    WyBufs &y = D->y;
    const int64_t nn = w.npad * w.npad;
    const int32_t m = wy ? wy->ncon : 0;
    const int64_t nfit = n - m;
    const bool tryReuse = mode == 1 && !invOut && !(c->flags & MPGPU_FLAG_FRESH_FACTOR) && D->factorValid &&
                          D->factorMode == mode && D->factorN == n && D->factorM == m;
    const unsigned gv = (unsigned)std::min<int64_t>((w.npad + 7) / 8, 4096);
    const unsigned ge = (unsigned)std::min<int64_t>((w.npad + 255) / 256, 4096);
    // x -= U op(T) U^T x: with P = H_1 ... H_m = I - U T U^T, op = T gives
    // P x (qlmlq's "Q^T x", reflections m..1) and op = T^T gives P^T x
    auto qapply = [&](double *xv, bool transT) {
        k_ut_x<<<kWyBlk, kWy, 0, s>>>(w.npad, y.U, xv, y.part);
        k_t_coef<<<1, kWy, 0, s>>>(y.part, y.T, transT ? 1 : 0, y.v);
        k_sub_uv<<<ge, 256, 0, s>>>(w.npad, y.U, y.v, xv);
    };
    // the CG operator: F x, or with wy the reduced matrix (P A P^T)_fit x
    // on the first nfit components and the identity on the others
    auto op = [&](const double *xin, double *out) {
        if (!wy) {
            k_gemv<<<gv, 256, 0, s>>>(w.F, w.npad, w.npad, xin, out);
            return;
        }
        k_expand<<<ge, 256, 0, s>>>(w.npad, nfit, n, xin, nullptr, y.a);
        qapply(y.a, true);
        k_gemv<<<gv, 256, 0, s>>>(w.F, w.npad, w.npad, y.a, out);
        qapply(out, false);
        k_reduce_op<<<ge, 256, 0, s>>>(w.npad, nfit, out, xin, out);
    };
    struct Ev {
        cudaEvent_t e[6] = {};
        Ev() { for (cudaEvent_t &x : e) cudaEventCreate(&x); }
        ~Ev() { for (cudaEvent_t x : e) cudaEventDestroy(x); }
    } ev;
    cudaEvent_t e0 = ev.e[0], e1 = ev.e[1], eFa = ev.e[2], eFb = ev.e[3], eR = ev.e[4];
    cudaEventRecord(e0, s);
    cudaMemsetAsync(w.F, 0, sizeof(double) * nn, s);
    k_packed_to_dense<<<4096, 256, 0, s>>>(Ap, n, w.npad, nullptr, w.F);
    if (w.npad > n) k_pad_identity<<<(unsigned)((w.npad - n + 255) / 256), 256, 0, s>>>(w.F, w.npad, n, w.npad);
    cudaMemsetAsync(w.b, 0, sizeof(double) * w.npad, s);
    if (!wy) {
        cudaMemcpyAsync(w.b, bx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    } else {
        // reduced right-hand side (P (g - A P^T [0; y]))_fit
        k_build_u<<<2048, 256, 0, s>>>(wy->V, wy->Vk, n, m, w.npad, y.U, y.UT);
        k_pad_t<<<64, 256, 0, s>>>(wy->T, m, y.T, y.TT);
        k_expand<<<ge, 256, 0, s>>>(w.npad, nfit, n, nullptr, wy->y, y.a);
        qapply(y.a, true);
        k_gemv<<<gv, 256, 0, s>>>(w.F, w.npad, w.npad, y.a, w.q);
        cudaMemcpyAsync(w.r, bx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
        if (w.npad > n) cudaMemsetAsync(w.r + n, 0, sizeof(double) * (w.npad - n), s);
        k_sub_to<<<ge, 256, 0, s>>>(w.npad, w.r, w.q, w.r);
        qapply(w.r, false);
        k_expand<<<ge, 256, 0, s>>>(w.npad, nfit, n, w.r, nullptr, w.b);
    }
    MPG_CUDA(c, cudaGetLastError());
    // the factorisation of this solve's matrix: with wy the WY products of
    // P A P^T first (W = A U by tensor-core 3xTF32 tile products, A split
    // tile by tile into L's area, which the factor overwrites below)
    auto factorise = [&]() -> int32_t {
        D->factorValid = false;
        if (wy) {
            const int64_t np_ = w.np;
            float *fh = reinterpret_cast<float *>(w.L), *fl = fh + nn;
            MPG_CUDA(c, tc_split_tiles(w.F, w.npad, 0, (int32_t)np_, 0, (int32_t)np_, fh, fl, np_, 0, s));
            MPG_CUDA(c, tc_split_tiles(y.UT, w.npad, 0, 1, 0, (int32_t)np_, y.uh, y.ul, np_, 0, s));
            std::vector<tc::TileTask> tk(np_);
            for (int64_t i = 0; i < np_; ++i) tk[i] = {(int32_t)i, 0, 0, (int32_t)np_, (int32_t)i, 0};
            tc::TileTask *dt = nullptr;
            MPG_CUDA(c, cudaMallocAsync(&dt, sizeof(tc::TileTask) * np_, s));
            struct G { tc::TileTask *p; cudaStream_t s; ~G() { cudaFreeAsync(p, s); } } gd{dt, s};
            MPG_CUDA(c, cudaMemcpyAsync(dt, tk.data(), sizeof(tc::TileTask) * np_, cudaMemcpyHostToDevice, s));
            MPG_CUDA(c, cudaMemsetAsync(w.err, 0, sizeof(int32_t), s));
            MPG_CUDA(c, tc_tile_gemm(tc::TcOp{fh, fl, np_}, tc::TcOp{y.uh, y.ul, np_}, y.W, kWy, dt, np_, 0, 0, 1.0,
                                     0.0, w.err, s));
            MPG_CUDA(c, cudaStreamSynchronize(s));   // the task list is released below
            // M = U^T W, S = T M T^T, Z = W T^T - S U / 2 (FP64, m x m sized)
            k_utw<<<kWy, kWy, 0, s>>>(w.npad, y.U, y.W, y.M);
            k_small_mm<<<kWy, kWy, 0, s>>>(y.T, 0, y.M, 0, y.X);
            k_small_mm<<<kWy, kWy, 0, s>>>(y.X, 0, y.T, 1, y.S);
            k_wy_z<<<(unsigned)std::min<int64_t>(w.npad, 4096), kWy, 0, s>>>(w.npad, y.W, y.U, y.TT, y.S, y.ZU,
                                                                                  y.UZ);
            MPG_CUDA(c, tc_split_tiles(y.ZU, 2 * kWy, 0, (int32_t)np_, 0, 2, y.zh, y.zl, 2, 0, s));
            MPG_CUDA(c, tc_split_tiles(y.UZ, 2 * kWy, 0, (int32_t)np_, 0, 2, y.uh, y.ul, 2, 0, s));
            MPG_CUDA(c, cudaGetLastError());
        }
        // the matrix to factorise: A, or A' = A - Z U^T - U Z^T with the
        // eliminated rows and columns replaced by the identity
        auto prepare = [&](double sh) -> int32_t {
            if (!wy) {
                k_copy_lower_shift<<<4096, 256, 0, s>>>(w.F, w.L, w.npad, sh);
                return MPGPU_OK;
            }
            k_copy_lower_shift<<<4096, 256, 0, s>>>(w.F, w.L, w.npad, 0.0);
            const int64_t T = w.np;
            MPG_CUDA(c, tc_tile_gemm(tc::TcOp{y.zh, y.zl, 2}, tc::TcOp{y.uh, y.ul, 2}, w.L, w.npad, nullptr,
                                     T * (T + 1) / 2, 0, 2, -1.0, 1.0, w.err, s));
            k_identity_rows<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(w.npad - nfit, 4096)), 256, 0, s>>>(
                w.L, w.npad, nfit, w.npad);
            if (sh != 0.0)
                k_scale_diag<<<(unsigned)((nfit + 255) / 256), 256, 0, s>>>(w.L, w.npad, nfit, 1.0 + sh);
            // a tile product whose barrier wait ran out has flagged w.err
            int32_t h = 0;
            MPG_CUDA(c, cudaMemcpyAsync(&h, w.err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            MPG_CUDA(c, cudaStreamSynchronize(s));
            if (h < 0) return set_err(c, MPGPU_ERR_TIMEOUT, "tensor-core tile product: barrier wait ran out");
            return MPGPU_OK;
        };
        // a non-positive pivot of the low-precision factor is cured by a
        // growing diagonal shift (the CG iterations remove it)
        double shift = 0.0;
        int32_t r = MPGPU_OK;
        for (int tries = 0;; ++tries) {
            r = prepare(shift);
            if (r != MPGPU_OK) break;
            int32_t bad = -1;
            r = dense_cholesky_device(c, w.L, w.npad, mode, w.hi, w.lo, w.err, &bad);
            if (r != MPGPU_ERR_FACTOR || tries >= 6) break;
            shift = shift == 0.0 ? 1e-7 : shift * 10.0;
        }
        if (r != MPGPU_OK) return r;
        const int trtriSmem = (kNB * kNB + kNB) * (int)sizeof(double);
        MPG_CUDA(c, smem_optin((const void *)k_trtri_blocks));
        k_trtri_blocks<<<(unsigned)w.np, 256, trtriSmem, s>>>(w.L, w.npad, w.DinvT);
        MPG_CUDA(c, build_super_inverse(w, s));
        MPG_CUDA(c, cudaGetLastError());
        D->factorValid = true;
        D->factorMode = mode;
        D->factorN = n;
        D->factorM = m;
        D->factorShift = shift;
        return MPGPU_OK;
    };
    // preconditioned CG from x0 = M^-1 b; stop when the relative residual
    // is below rtol AND the last correction is below kRefineXtol of the
    // solution: a residual test alone leaves an error of about cond(A) *
    // rtol, which differs between factors of different precision; the
    // correction test brings every form to the same FP64 solution
    double hs[8] = {};
    auto run_cg = [&](int32_t limit, int32_t &itn, int32_t &istop) -> int32_t {
        precond(w, w.b, w.x, s);
        op(w.x, w.q);
        k_sub_vec<<<(unsigned)((w.npad + 255) / 256), 256, 0, s>>>(w.npad, w.b, w.q, w.r);
        precond(w, w.r, w.z, s);
        cudaMemcpyAsync(w.p, w.z, sizeof(double) * w.npad, cudaMemcpyDeviceToDevice, s);
        dotv(w, w.r, w.z, w.sc + 0, s);
        dotv(w, w.b, w.b, w.sc + 4, s);
        // one CG iteration as a CUDA graph (its ~600 launches replayed cheaply)
        struct Gr {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t x = nullptr;
            ~Gr() { if (x) cudaGraphExecDestroy(x); if (g) cudaGraphDestroy(g); }
        } gr;
        MPG_CUDA(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        op(w.p, w.q);
        dotv(w, w.p, w.q, w.sc + 1, s);
        dotv(w, w.p, w.p, w.sc + 6, s);
        k_cg_step<<<ge, 256, 0, s>>>(w.npad, w.x, w.r, w.p, w.q, w.sc);
        dotv(w, w.x, w.x, w.sc + 7, s);
        precond(w, w.r, w.z, s);
        dotv(w, w.r, w.z, w.sc + 2, s);
        k_cg_dir<<<ge, 256, 0, s>>>(w.npad, w.p, w.z, w.sc);
        k_cg_roll<<<1, 32, 0, s>>>(w.sc);
        dotv(w, w.r, w.r, w.sc + 3, s);
        cudaError_t ce = cudaStreamEndCapture(s, &gr.g);
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&gr.x, gr.g, 0);
        if (ce != cudaSuccess) return cuda_err(c, ce, "CG graph");
        itn = 0;
        istop = 0;
        const double tol2 = rtol * rtol, xtol2 = kRefineXtol * kRefineXtol;
        while (itn < limit) {
            const int batch = std::min(4, limit - itn);
            for (int k = 0; k < batch; ++k) cudaGraphLaunch(gr.x, s);
            itn += batch;
            MPG_CUDA(c, cudaMemcpyAsync(hs, w.sc, sizeof(hs), cudaMemcpyDeviceToHost, s));
            MPG_CUDA(c, cudaStreamSynchronize(s));
            if (!(hs[3] == hs[3]) || !(hs[5] == hs[5])) { istop = 9; break; }
            if (hs[3] <= tol2 * hs[4] && hs[5] <= xtol2 * hs[7]) { istop = 1; break; }
        }
        if (istop == 0) istop = 3;
        return MPGPU_OK;
    };
    int32_t itn = 0, istop = 0, reused = 0, itnReuse = 0;
    bool factored = false;
    if (tryReuse) {
        rc = run_cg(std::min<int32_t>(itnlim, kReuseItn), itn, istop);
        if (rc != MPGPU_OK) return rc;
        if (istop == 1) {
            reused = 1;
        } else {
            reused = 2;
            itnReuse = itn;
        }
    }
    if (reused != 1) {
        cudaEventRecord(eFa, s);
        rc = factorise();
        if (rc != MPGPU_OK) return rc;
        cudaEventRecord(eFb, s);
        factored = true;
        rc = run_cg(itnlim, itn, istop);
        if (rc != MPGPU_OK) return rc;
    }
    if (!wy) {
        cudaMemcpyAsync(bx, w.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    } else {
        // the full correction P^T [x; y]
        k_expand<<<ge, 256, 0, s>>>(w.npad, nfit, n, w.x, wy->y, y.a);
        qapply(y.a, true);
        cudaMemcpyAsync(bx, y.a, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    }
    // the inverse from the same factor (inversion forms): X = L^-1, Z = X^T X
    cudaEventRecord(eR, s);
    int32_t rcInv = MPGPU_OK;
    if (invOut && istop != 9) {
        rcInv = dense_inverse_device(c, w.L, w.npad, nfit, mode, w.DinvT, w.F, invOut, w.err);
        // the inverse overwrites L and F
        D->factorValid = false;
    }
    cudaEventRecord(e1, s);
    MPG_CUDA(c, cudaStreamSynchronize(s));
    if (rcInv != MPGPU_OK) return rcInv;
    float ms = 0.0f, msF = 0.0f, msR = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (factored) cudaEventElapsedTime(&msF, eFa, eFb);
    cudaEventElapsedTime(&msR, e0, eR);
    if (info) {
        info->msFactor = msF;
        info->msRefine = msR - msF;
        info->msInverse = ms - msR;
        info->itn = itn + itnReuse;
        info->istop = istop;
        info->nrank = (int32_t)nfit;
        info->evmin = D->factorShift;
        info->evmax = hs[4] > 0.0 ? std::sqrt(hs[3] / hs[4]) : 0.0;
        info->dxRel = hs[7] > 0.0 ? std::sqrt(hs[5] / hs[7]) : 0.0;
        info->ms = ms;
        info->factorReused = reused;
        info->itnReuse = itnReuse;
    }
    return istop == 9 ? set_err(c, MPGPU_ERR_NAN, "NaN in the refined dense solve") : MPGPU_OK;
}
