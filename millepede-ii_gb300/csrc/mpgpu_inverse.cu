// mpgpu_inverse.cu -- inverse of the QL-reduced global matrix from its
// blocked Cholesky factor: the dense form of the inversion that gives pede
// its parameter errors (minver, pede.f90:7838-7945, which inverts with
// sqminl, mpnum.f90:230-355).  With A = L L^T (mpgpu_dense.cu):
//   trtri  X = L^-1, in place, block column by block column from the last
//          (LAPACK's blocked order): for panel p, T = X_trail P (the panel
//          P below the diagonal block times the already inverted trailing
//          part, lower triangular), then X_panel = -T D_p with D_p = L_pp^-1;
//   lauum  Z = X^T X (lower part), Z_ij = sum_{k >= i} X_ki^T X_kj.
// Both are lists of 128 x 128 tile products C = alpha sum_k A_k B_k^T +
// beta C run by one of two kernels: FP64 on the CUDA cores (64 x 64 per CTA,
// the form of the FP64 trailing update) or tcgen05 3xTF32 with FP32
// accumulation in tensor memory over the whole K range (operands split
// once into TF32 hi/lo tiles).  Work: N^3/3 for each of trtri and lauum.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "mpgpu_ctx.h"
#include "mpgpu_tc.cuh"

namespace {

using tc::kNB;
using tc::kStageBytes;
using tc::kStages;
using tc::kTcSmem;
using tc::kTcThreads;
using tc::kOpBytes;
using tc::kTK;
constexpr int64_t kTileEl = (int64_t)kNB * kNB;

using tc::TileTask;

// ------------------------------------------------------------ FP64 form
// An operand tile (row, k) of a dense row-major FP64 matrix M, or of M^T
// (trans: element (m, kk) of the tile is M[k*128 + kk][row*128 + m]).
struct Fp64Op {
    const double *M;
    int64_t ld;
    int32_t trans;
};

__global__ void __launch_bounds__(256) k_tile_gemm_fp64(Fp64Op A, Fp64Op B, double *C, int64_t ldc,
                                                        const TileTask *tasks, double alpha, double beta) {
    __shared__ double sa[16][64 + 1], sb[16][64 + 1];
    const TileTask t = tasks[blockIdx.x >> 2];
    const int sub = blockIdx.x & 3, si = sub >> 1, sj = sub & 1;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t ar = (int64_t)t.aRow * kNB + si * 64, br = (int64_t)t.bRow * kNB + sj * 64;
    double acc[4][4] = {};
    for (int k = t.k0; k < t.k1; ++k) {
        for (int kc = 0; kc < kNB; kc += 16) {
            const int64_t kb = (int64_t)k * kNB + kc;
            for (int e = tid; e < 64 * 16; e += 256) {
                if (!A.trans) {
                    const int r = e >> 4, kk = e & 15;
                    sa[kk][r] = A.M[(ar + r) * A.ld + kb + kk];
                } else {
                    const int r = e & 63, kk = e >> 6;
                    sa[kk][r] = A.M[(kb + kk) * A.ld + ar + r];
                }
                if (!B.trans) {
                    const int r = e >> 4, kk = e & 15;
                    sb[kk][r] = B.M[(br + r) * B.ld + kb + kk];
                } else {
                    const int r = e & 63, kk = e >> 6;
                    sb[kk][r] = B.M[(kb + kk) * B.ld + br + r];
                }
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < 16; ++kk) {
                double a[4], b[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) { a[q] = sa[kk][ty * 4 + q]; b[q] = sb[kk][tx * 4 + q]; }
#pragma unroll
                for (int p = 0; p < 4; ++p)
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double *cp = C + ((int64_t)t.cRow * kNB + si * 64 + ty * 4 + p) * ldc + (int64_t)t.cCol * kNB + sj * 64 +
                         tx * 4 + q;
            *cp = beta != 0.0 ? alpha * acc[p][q] + beta * *cp : alpha * acc[p][q];
        }
}

}  // namespace

// FP64 tile products C(cRow, cCol) = alpha sum_k op(A)(aRow, k) op(B)(k, bRow)
// + beta C over a device task list (op: trans 0 takes tile (r, k) of A or
// (bRow, k) of B transposed, trans 1 the tile as stored)
cudaError_t fp64_tile_gemm(const double *A, int64_t lda, int32_t ta, const double *B, int64_t ldb, int32_t tb,
                           double *C, int64_t ldc, const tc::TileTask *tasks, int64_t ntask, double alpha,
                           double beta, cudaStream_t s) {
    if (ntask <= 0) return cudaSuccess;
    k_tile_gemm_fp64<<<(unsigned)(ntask * 4), 256, 0, s>>>(Fp64Op{A, lda, ta}, Fp64Op{B, ldb, tb}, C, ldc, tasks,
                                                            alpha, beta);
    return cudaGetLastError();
}

namespace {
// ------------------------------------------------------------ tensor-core form
using tc::TcOp;

// Tiles rows [r0, r1) x columns [c0, c1) of the dense FP64 matrix M (or
// the tiles of M^T: tile (c, r) of the destination receives tile (r, c) of
// M transposed) split into TF32 hi + lo; the destination's tile column is
// the source's column less cOff (rows keep their index).
__global__ void k_split_tiles(const double *M, int64_t ld, int32_t r0, int32_t r1, int32_t c0, int32_t c1,
                              int32_t trans, float *hi, float *lo, int64_t ntDst, int32_t cOff) {
    const int64_t nc = c1 - c0;
    const int32_t tr = r0 + (int32_t)(blockIdx.x / nc), tcc = c0 + (int32_t)(blockIdx.x % nc);
    if (tr >= r1) return;
    const int64_t dst = trans ? ((int64_t)tcc * ntDst + tr) * kTileEl
                              : ((int64_t)tr * ntDst + (tcc - cOff)) * kTileEl;
    for (int e = threadIdx.x; e < kTileEl; e += blockDim.x) {
        // destination element (u, v) contiguous; source element (u, v) or (v, u)
        const int u = e / kNB, v = e % kNB;
        const int64_t src = trans ? ((int64_t)tr * kNB + v) * ld + (int64_t)tcc * kNB + u
                                  : ((int64_t)tr * kNB + u) * ld + (int64_t)tcc * kNB + v;
        const double x = M[src];
        uint32_t h, l;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"((float)x));
        const double rest = x - (double)__uint_as_float(h);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"((float)rest));
        hi[dst + e] = __uint_as_float(h);
        lo[dst + e] = __uint_as_float(l);
    }
}

// One CTA per task: the K range of the task streamed chunk by chunk (16
// columns of one K tile per chunk) through the 3-stage pipeline, hi*hi +
// hi*lo + lo*hi accumulated in one FP32 tensor-memory accumulator over all
// chunks, then C = alpha acc + beta C in FP64 (coalesced through shared
// memory).  Bounded mbarrier waits: a wait that runs out sets *err = -1
// and the CTA finishes without writing C.  Without a task list the CTAs
// take the lower triangle of tiles from tile (trail0, trail0) on, each
// with K tiles [0, trailK) of rows i and j: the trailing update of a
// block column.
__global__ void __launch_bounds__(kTcThreads) k_tile_gemm_tc(TcOp A, TcOp B, double *C, int64_t ldc,
                                                             const TileTask *tasks, int32_t trail0, int32_t trailK,
                                                             double alpha, double beta, int32_t *err) {
    extern __shared__ __align__(128) char tsm[];
    __shared__ uint64_t mbar[kStages];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, wib = tid >> 5, ln = tid & 31;
    TileTask t;
    if (tasks) {
        t = tasks[blockIdx.x];
    } else {
        const int64_t q = blockIdx.x;
        int bi = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
        while ((int64_t)bi * (bi + 1) / 2 > q) bi--;
        while ((int64_t)(bi + 1) * (bi + 2) / 2 <= q) bi++;
        const int bj = (int)(q - (int64_t)bi * (bi + 1) / 2);
        t = TileTask{trail0 + bi, trail0 + bj, 0, trailK, trail0 + bi, trail0 + bj};
    }
    const int per = kNB / kTK;   // chunks per K tile
    const int nch = (t.k1 - t.k0) * per;
    if (nch <= 0) return;
    const uint32_t sbase = tc::smem_u32(tsm);
    float *epi = reinterpret_cast<float *>(tsm) + wib * 32 * 33;   // after the last MMA only
    if (wib == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc::smem_u32(&tbase)),
                     "r"(kNB));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int st = 0; st < kStages; ++st)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(tc::smem_u32(&mbar[st])));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tbase;
    auto load = [&](int c, int st) {
        const int64_t k = t.k0 + c / per;
        const int kc0 = (c % per) * kTK;
        const int64_t ta = ((int64_t)t.aRow * A.nt + k) * kTileEl, tb = ((int64_t)t.bRow * B.nt + k) * kTileEl;
        const uint32_t s0 = sbase + st * kStageBytes;
        tc::load_chunk_async(A.hi + ta, kc0, s0);
        tc::load_chunk_async(A.lo + ta, kc0, s0 + kOpBytes);
        tc::load_chunk_async(B.hi + tb, kc0, s0 + 2 * kOpBytes);
        tc::load_chunk_async(B.lo + tb, kc0, s0 + 3 * kOpBytes);
    };
    uint32_t ph = 0;   // bit st: parity of the next completion of stage st's barrier
    bool ok = true;
    for (int c = 0; c < kStages - 1; ++c) {
        if (c < nch) load(c, c);
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
                const uint64_t dah = tc::umma_desc(sb + off), dal = tc::umma_desc(sb + kOpBytes + off);
                const uint64_t dbh = tc::umma_desc(sb + 2 * kOpBytes + off), dbl = tc::umma_desc(sb + 3 * kOpBytes + off);
                tc::mma_tf32(tmem, dah, dbh, (c > 0 || kk > 0) ? 1u : 0u);
                tc::mma_tf32(tmem, dah, dbl, 1u);
                tc::mma_tf32(tmem, dal, dbh, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             tc::smem_u32(&mbar[st]))
                         : "memory");
        }
        // the stage of chunk c + kStages - 1 held chunk c - 1: wait for its MMAs
        const int cn = c + kStages - 1;
        if (cn < nch) {
            const int sn = cn % kStages;
            if (c >= 1) {
                if (!tc::mbar_wait(tc::smem_u32(&mbar[sn]), (ph >> sn) & 1)) ok = false;
                ph ^= 1u << sn;
            }
            if (ok) load(cn, sn);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        if (!__syncthreads_and(ok)) { ok = false; break; }
    }
    // the MMAs of the chunks not yet waited for (the last kStages - 1)
    if (ok) {
        for (int c = (nch > kStages - 1 ? nch - (kStages - 1) : 0); c < nch; ++c) {
            const int st = c % kStages;
            if (!tc::mbar_wait(tc::smem_u32(&mbar[st]), (ph >> st) & 1)) ok = false;
            ph ^= 1u << st;
        }
    } else {
        for (int st = 0; st < kStages; ++st) tc::mbar_wait(tc::smem_u32(&mbar[st]), (ph >> st) & 1);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (__syncthreads_and(ok)) {
        const int64_t rowBase = (int64_t)t.cRow * kNB + wib * 32;
        const int64_t colBase = (int64_t)t.cCol * kNB;
        for (int cb = 0; cb < kNB / 32; ++cb) {
            uint32_t v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(wib * 32) << 16) + (uint32_t)(cb * 32), v);
#pragma unroll
            for (int q = 0; q < 32; ++q) epi[ln * 33 + q] = __uint_as_float(v[q]);
            __syncwarp();
            double *cp = C + rowBase * ldc + colBase + cb * 32 + ln;
            if (beta != 0.0) {
                double cv[32];
#pragma unroll
                for (int r = 0; r < 32; ++r) cv[r] = cp[r * ldc];
#pragma unroll
                for (int r = 0; r < 32; ++r) cp[r * ldc] = alpha * (double)epi[r * 33 + ln] + beta * cv[r];
            } else {
#pragma unroll
                for (int r = 0; r < 32; ++r) cp[r * ldc] = alpha * (double)epi[r * 33 + ln];
            }
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

// diagonal block p of X: D_p = L_pp^-1 from its transposed copy
// (DinvT[p][r][c] = D_p[c][r]), zero above the diagonal
__global__ void k_set_diag_inverse(double *L, int64_t ld, int32_t p, const double *DinvT) {
    const double *D = DinvT + (int64_t)p * kTileEl;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kTileEl; e += gridDim.x * blockDim.x) {
        const int i = e / kNB, j = e % kNB;
        L[((int64_t)p * kNB + i) * ld + (int64_t)p * kNB + j] = j <= i ? D[(int64_t)j * kNB + i] : 0.0;
    }
}

__global__ void k_dense_lower_to_packed(const double *Z, int64_t ld, int64_t n, double *Zp) {
    const int64_t nn = n * (n + 1) / 2;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = (int64_t)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
        while (i * (i + 1) / 2 > e) i--;
        while ((i + 1) * (i + 2) / 2 <= e) i++;
        const int64_t j = e - i * (i + 1) / 2;
        Zp[e] = Z[i * ld + j];
    }
}

}  // namespace

// L (npad x npad, dense row-major, the lower Cholesky factor with the
// inverses of its diagonal blocks in DinvT) is replaced by X = L^-1; Z =
// X^T X (lower part) is written to Zd and its leading n x n block packed
// into Zp.  mode 0: FP64 tile products; mode 1: tensor-core 3xTF32.
int32_t dense_inverse_device(mpgpu_ctx *c, double *L, int64_t npad, int64_t n, int mode, const double *DinvT,
                             double *Zd, double *Zp, int32_t *dErr) {
    cudaStream_t s = c->stream;
    const int32_t np = (int32_t)(npad / kNB);
    const int64_t ld = npad;
    // tasks of every trtri step (T products, then the panel scaling) and of lauum
    std::vector<TileTask> tk;
    std::vector<int64_t> stepT(np + 1), stepS(np + 1);
    for (int32_t p = np - 1; p >= 0; --p) {
        stepT[p] = (int64_t)tk.size();
        for (int32_t r = p + 1; r < np; ++r) tk.push_back({r, p, p + 1, r + 1, r - p - 1, 0});
        stepS[p] = (int64_t)tk.size();
        for (int32_t r = p + 1; r < np; ++r) tk.push_back({r - p - 1, 0, 0, 1, r, p});
    }
    const int64_t lauum0 = (int64_t)tk.size();
    {
        // longest K first
        std::vector<TileTask> la;
        for (int32_t i = 0; i < np; ++i)
            for (int32_t j = 0; j <= i; ++j) la.push_back({i, j, i, np, i, j});
        std::stable_sort(la.begin(), la.end(),
                         [](const TileTask &a, const TileTask &b) { return a.k1 - a.k0 > b.k1 - b.k0; });
        tk.insert(tk.end(), la.begin(), la.end());
    }
    TileTask *dTask = nullptr;
    double *T = nullptr;
    float *xhi = nullptr, *xlo = nullptr, *thi = nullptr, *tlo = nullptr, *phi = nullptr, *plo = nullptr,
          *dhi = nullptr, *dlo = nullptr;
    auto release = [&] {
        cudaFree(dTask); cudaFree(T);
        cudaFree(xhi); cudaFree(xlo); cudaFree(thi); cudaFree(tlo); cudaFree(phi); cudaFree(plo);
        cudaFree(dhi); cudaFree(dlo);
    };
    cudaError_t e = cudaMalloc(&dTask, sizeof(TileTask) * tk.size());
    if (e == cudaSuccess) e = cudaMalloc(&T, sizeof(double) * npad * kNB);
    const int64_t full = (int64_t)np * np * kTileEl;
    if (mode == 1) {
        // X (non-transposed) and L^T, later X^T, split tile by tile; the
        // panel T and the diagonal inverse D_p split per step
        if (e == cudaSuccess) e = cudaMalloc(&xhi, sizeof(float) * full);
        if (e == cudaSuccess) e = cudaMalloc(&xlo, sizeof(float) * full);
        if (e == cudaSuccess) e = cudaMalloc(&phi, sizeof(float) * full);
        if (e == cudaSuccess) e = cudaMalloc(&plo, sizeof(float) * full);
        if (e == cudaSuccess) e = cudaMalloc(&thi, sizeof(float) * (int64_t)np * kTileEl);
        if (e == cudaSuccess) e = cudaMalloc(&tlo, sizeof(float) * (int64_t)np * kTileEl);
        if (e == cudaSuccess) e = cudaMalloc(&dhi, sizeof(float) * kTileEl);
        if (e == cudaSuccess) e = cudaMalloc(&dlo, sizeof(float) * kTileEl);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dTask, tk.data(), sizeof(TileTask) * tk.size(), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { release(); return cuda_err(c, e, "blocked inverse workspace"); }
    if (mode == 1) {
        MPG_CUDA(c, smem_optin((const void *)k_tile_gemm_tc));
        // L^T tiles (p, k) for k > p: the panels of the original factor
        for (int32_t p = 0; p < np - 1; ++p)
            k_split_tiles<<<np - 1 - p, 256, 0, s>>>(L, ld, p + 1, np, p, p + 1, 1, phi, plo, np, 0);
    }
    MPG_CUDA(c, cudaMemsetAsync(dErr, 0, sizeof(int32_t), s));
    // ---- trtri, panels from the last
    for (int32_t p = np - 1; p >= 0; --p) {
        const int32_t m = np - 1 - p;
        if (m > 0) {
            if (mode == 1) {
                k_tile_gemm_tc<<<m, kTcThreads, kTcSmem, s>>>(TcOp{xhi, xlo, np}, TcOp{phi, plo, np}, T, kNB,
                                                              dTask + stepT[p], 0, 0, 1.0, 0.0, dErr);
                k_split_tiles<<<m, 256, 0, s>>>(T, kNB, 0, m, 0, 1, 0, thi, tlo, 1, 0);
                k_split_tiles<<<1, 256, 0, s>>>(DinvT + (int64_t)p * kTileEl, kNB, 0, 1, 0, 1, 0, dhi, dlo, 1, 0);
                k_tile_gemm_tc<<<m, kTcThreads, kTcSmem, s>>>(TcOp{thi, tlo, 1}, TcOp{dhi, dlo, 1}, L, ld,
                                                              dTask + stepS[p], 0, 0, -1.0, 0.0, dErr);
            } else {
                k_tile_gemm_fp64<<<4 * m, 256, 0, s>>>(Fp64Op{L, ld, 0}, Fp64Op{L, ld, 1}, T, kNB, dTask + stepT[p],
                                                       1.0, 0.0);
                k_tile_gemm_fp64<<<4 * m, 256, 0, s>>>(Fp64Op{T, kNB, 0},
                                                       Fp64Op{DinvT + (int64_t)p * kTileEl, kNB, 0}, L, ld,
                                                       dTask + stepS[p], -1.0, 0.0);
            }
        }
        k_set_diag_inverse<<<16, 256, 0, s>>>(L, ld, p, DinvT);
        // the finished column of X, split for the later steps' products
        if (mode == 1) k_split_tiles<<<m + 1, 256, 0, s>>>(L, ld, p, np, p, p + 1, 0, xhi, xlo, np, 0);
        MPG_CUDA(c, cudaGetLastError());
    }
    // ---- lauum
    const int64_t nla = (int64_t)np * (np + 1) / 2;
    if (mode == 1) {
        // X^T tiles (i, k) for k >= i (into the L^T area)
        for (int32_t i = 0; i < np; ++i)
            k_split_tiles<<<np - i, 256, 0, s>>>(L, ld, i, np, i, i + 1, 1, phi, plo, np, 0);
        k_tile_gemm_tc<<<(unsigned)nla, kTcThreads, kTcSmem, s>>>(TcOp{phi, plo, np}, TcOp{phi, plo, np}, Zd, ld,
                                                                  dTask + lauum0, 0, 0, 1.0, 0.0, dErr);
    } else {
        k_tile_gemm_fp64<<<(unsigned)(4 * nla), 256, 0, s>>>(Fp64Op{L, ld, 1}, Fp64Op{L, ld, 1}, Zd, ld,
                                                             dTask + lauum0, 1.0, 0.0);
    }
    MPG_CUDA(c, cudaGetLastError());
    k_dense_lower_to_packed<<<4096, 256, 0, s>>>(Zd, ld, n, Zp);
    int32_t h = 0;
    e = cudaMemcpyAsync(&h, dErr, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    release();
    if (e != cudaSuccess) return cuda_err(c, e, "blocked inverse");
    if (h < 0) return set_err(c, MPGPU_ERR_TIMEOUT, "tensor-core tile product: barrier wait ran out");
    return MPGPU_OK;
}

// Launchers for the blocked Cholesky (mpgpu_dense.cu).
cudaError_t tc_split_tiles(const double *M, int64_t ld, int32_t r0, int32_t r1, int32_t c0, int32_t c1, float *hi,
                           float *lo, int64_t ntDst, int32_t cOff, cudaStream_t s) {
    const int64_t n = (int64_t)(r1 - r0) * (c1 - c0);
    if (n <= 0) return cudaSuccess;
    k_split_tiles<<<(unsigned)n, 256, 0, s>>>(M, ld, r0, r1, c0, c1, 0, hi, lo, ntDst, cOff);
    return cudaGetLastError();
}

cudaError_t tc_tile_gemm(const TcOp &A, const TcOp &B, double *C, int64_t ldc, const TileTask *tasks, int64_t ntask,
                         int32_t trail0, int32_t trailK, double alpha, double beta, int32_t *err, cudaStream_t s) {
    if (ntask <= 0) return cudaSuccess;
    cudaError_t e = smem_optin((const void *)k_tile_gemm_tc);
    if (e != cudaSuccess) return e;
    k_tile_gemm_tc<<<(unsigned)ntask, kTcThreads, kTcSmem, s>>>(A, B, C, ldc, tasks, trail0, trailK, alpha, beta, err);
    return cudaGetLastError();
}
