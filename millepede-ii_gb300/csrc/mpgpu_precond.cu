// mpgpu_precond.cu -- the variable-band preconditioner of MINRES
// (pede's "bandwidth" option: equdecs/equslvs with the constraints
// eliminated, mpnum.f90:2486-2678, on the band of Q^T A Q that the
// preconditioner fill and qlpssq give, pede.f90:2639-2651, 8304-8311).
//
// Layout: row i of the band holds w+1 doubles, entry t for column
// i - w + t (w = mbandw - 1; entry w is the diagonal).  The factor F has
// the same layout with the diagonal replaced by 1/sqrt as lltdec leaves it.
//
// lltdec (mpnum.f90:2155-2209) is a chain over the rows; it runs on one
// warp with the (w+1) x (w+1) window of rows k..k+w in shared memory,
// right-looking: column k is scaled and subtracted from the window, which
// performs the subtractions of lltdec's left-looking loops in the same
// order, so the factor equals lltdec's bit for bit.
//
// The solve (L L^T)^-1 x runs on blocks of s rows at once: within a block
// one warp solves along the rows with the w previous (or next) values in
// its lanes; the coupling to the neighbouring block passes through w
// values per block ("spikes" G = L_bb^-1 C_b and H = L_bb^-T C_{b+1}^T,
// computed once with the factor), so only a w x w step per block is
// sequential.
#include <cuda_pipeline.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "mpgpu_ctx.h"

namespace {
constexpr int kT = 256;
constexpr unsigned kFull = 0xffffffffu;

inline int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    return (int)std::min<int64_t>(std::max<int64_t>(g, 1), 152 * 16);
}

// band of the global matrix over all nVar rows; sparse storage through the
// block table of the row groups (blocks of group I ordered by column group)
__global__ void k_band_fill(int32_t nVar, int32_t w, int32_t matsto, const double *matD, const int32_t *aig,
                            const int32_t *p2g, const int64_t *rowStart, const int32_t *bcol,
                            const int64_t *boff, const int32_t *bld, double *B) {
    const int32_t W1 = w + 1;
    const int64_t tot = (int64_t)nVar * W1;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = (int32_t)(e / W1);
        const int32_t j = i - w + (int32_t)(e - (int64_t)i * W1);
        double a = 0.0;
        if (j >= 0) {
            if (matsto != 2) {
                a = matD[(int64_t)i * (i + 1) / 2 + j];
            } else if (i == j) {
                a = matD[i];
            } else {
                const int32_t I = p2g[i], J = p2g[j];  // 1-based groups, J <= I
                int64_t lo = rowStart[I - 1], hi = rowStart[I] - 1;
                while (lo <= hi) {
                    const int64_t mid = (lo + hi) >> 1;
                    const int32_t Jm = bcol[mid];
                    if (Jm == J) {
                        a = matD[boff[mid] + (int64_t)(i - (aig[I - 1] - 1)) * bld[mid] + (j - (aig[J - 1] - 1))];
                        break;
                    }
                    if (Jm < J) lo = mid + 1;
                    else hi = mid - 1;
                }
            }
        }
        B[e] = a;
    }
}

// one Householder reflection H = I - 2 v v^T applied to the band:
// (i,j) += -2 (v_i y_j + y_i v_j) + 4 beta v_i v_j, y = A' v, beta = v.y
__global__ void k_band_reflect(int32_t nVar, int32_t w, double *B, const double *v, const double *y,
                               const double *betap) {
    const double beta = *betap;
    const int32_t W1 = w + 1;
    const int64_t tot = (int64_t)nVar * W1;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = (int32_t)(e / W1);
        const int32_t j = i - w + (int32_t)(e - (int64_t)i * W1);
        if (j < 0) continue;
        const double vi = v[i], vj = v[j];
        if (vi == 0.0 && vj == 0.0) continue;
        B[e] += -2.0 * (vi * y[j] + y[i] * vj) + 4.0 * beta * (vi * vj);
    }
}

// lltdec on rows 0..n-1 of B into F (F zeroed before); one warp.
// Shared memory: window (w+1)^2 doubles, ring slot m % (w+1) for row m,
// entry t for column m - w + t; pair table of the trailing update.
__global__ void __launch_bounds__(32) k_lltdec(int32_t n, int32_t w, const double *B, double *F, int32_t iopt,
                                               int32_t *nrkdOut) {
    extern __shared__ double win[];
    const int W1 = w + 1;
    uint16_t *pairs = reinterpret_cast<uint16_t *>(win + W1 * W1);
    const int ln = threadIdx.x;
    const int npair = w * (w + 1) / 2;
    // pairs (qm, ql), 1 <= ql <= qm <= w, row-major
    for (int qm = 1, e = 0; qm <= w; ++qm)
        for (int ql = 1; ql <= qm; ++ql, ++e)
            if ((e & 31) == ln) pairs[e] = (uint16_t)(qm << 8 | ql);
    for (int e = ln; e < W1 * W1; e += 32) {
        const int m = e / W1;
        win[e] = m < n ? B[(int64_t)m * W1 + (e - m * W1)] : 0.0;
    }
    int32_t nrkd = 0;
    const double eps = 16.0 * 2.220446049250313e-16;
    double origNext = (ln == 0 && n > 0) ? B[w] : 0.0;
    __syncwarp();
    for (int32_t k = 0; k < n; ++k) {
        const int sk = k % W1;
        // row k + w + 1 (enters the window at the end of this step) and the
        // original diagonal of row k + 1
        const int32_t mn = k + W1;
        double nxt = 0.0;
        if (mn < n && ln < W1) nxt = B[(int64_t)mn * W1 + ln];
        const double orig = origNext;
        if (ln == 0 && k + 1 < n) origNext = B[(int64_t)(k + 1) * W1 + w];
        double d = 0.0;
        int reset = 0;
        if (ln == 0) {
            const double a = win[sk * W1 + w];
            if (k == 0) {
                if (a > 0.0) d = 1.0 / sqrt(a);
                else nrkd = -1;
            } else if (a > eps * orig) {
                d = 1.0 / sqrt(a);
            } else {
                reset = 1;
                if (iopt > 0 && orig > 0.0) {
                    d = 1.0 / sqrt(orig);
                } else if (nrkd == 0) {
                    nrkd = -(k + 1);
                } else {
                    if (nrkd < 0) nrkd = 1;
                    nrkd = nrkd + 1;
                }
            }
            F[(int64_t)k * W1 + w] = d;
        }
        d = __shfl_sync(kFull, d, 0);
        reset = __shfl_sync(kFull, reset, 0);
        if (reset)
            for (int t = ln; t < w; t += 32) F[(int64_t)k * W1 + t] = 0.0;
        // column k of rows k+1 .. k+mmax goes to F only (later steps use
        // columns right of k); each lane forms the column entries it needs
        // for the trailing update again, the same product; a reset row k
        // leaves them (a_mk - 0) * d with the original a_mk
        const int mmax = min(w, n - 1 - k);
        for (int q = 1 + ln; q <= mmax; q += 32) {
            const int32_t m = k + q;
            const double a = reset ? B[(int64_t)m * W1 + (w - q)] : win[(m % W1) * W1 + (w - q)];
            F[(int64_t)m * W1 + (w - q)] = __dmul_rn(a, d);
        }
        // trailing update of the window: (m, l) -= c_mk c_lk, k < l <= m
        for (int e = ln; e < npair; e += 32) {
            const int qm = pairs[e] >> 8, ql = pairs[e] & 0xff;
            if (qm > mmax) continue;
            const int rm = ((k + qm) % W1) * W1, rl = ((k + ql) % W1) * W1;
            const double am = reset ? B[(int64_t)(k + qm) * W1 + (w - qm)] : win[rm + (w - qm)];
            const double al = reset ? B[(int64_t)(k + ql) * W1 + (w - ql)] : win[rl + (w - ql)];
            const double cm = __dmul_rn(am, d), cl = __dmul_rn(al, d);
            double &x = win[rm + (w - qm + ql)];
            x = __dsub_rn(x, __dmul_rn(cm, cl));
        }
        // row k's slot takes row k + w + 1 (no lane reads it in this step)
        if (mn < n && ln < W1) win[sk * W1 + ln] = nxt;
        __syncwarp();
    }
    if (ln == 0) *nrkdOut = nrkd;
}

// L_bb z = x on rows [b0, b1) in place (x[row * xs]), lltfwd's order:
// lane t holds the partial value of row k + t
__device__ void warp_fwd(const double *F, int w, int32_t b0, int32_t b1, double *x, int64_t xs) {
    const int ln = threadIdx.x & 31;
    const int W1 = w + 1;
    double v = (ln <= w && b0 + ln < b1) ? x[(int64_t)(b0 + ln) * xs] : 0.0;
    double dn = F[(int64_t)b0 * W1 + w];
    double ln_c = (ln >= 1 && ln <= w && b0 + ln < b1) ? F[(int64_t)(b0 + ln) * W1 + (w - ln)] : 0.0;
    for (int32_t k = b0; k < b1; ++k) {
        const double d = dn, c = ln_c;
        // the coefficients of the next step
        if (k + 1 < b1) {
            dn = F[(int64_t)(k + 1) * W1 + w];
            ln_c = (ln >= 1 && ln <= w && k + 1 + ln < b1) ? F[(int64_t)(k + 1 + ln) * W1 + (w - ln)] : 0.0;
        }
        const double xk = __dmul_rn(__shfl_sync(kFull, v, 0), d);
        if (ln == 0) x[(int64_t)k * xs] = xk;
        if (ln >= 1 && ln <= w) v = __dsub_rn(v, __dmul_rn(c, xk));
        v = __shfl_down_sync(kFull, v, 1);
        if (ln == w) v = (k + 1 + w < b1) ? x[(int64_t)(k + 1 + w) * xs] : 0.0;
    }
}

// L_bb^T u = y on rows [b0, b1) in place, lltbwd's order: lane t holds the
// partial value of row k - w + t
__device__ void warp_bwd(const double *F, int w, int32_t b0, int32_t b1, double *x, int64_t xs) {
    const int ln = threadIdx.x & 31;
    const int W1 = w + 1;
    int32_t k = b1 - 1;
    double v = (ln <= w && k - w + ln >= b0) ? x[(int64_t)(k - w + ln) * xs] : 0.0;
    double dn = F[(int64_t)k * W1 + w];
    double cn = (ln < w) ? F[(int64_t)k * W1 + ln] : 0.0;
    for (; k >= b0; --k) {
        const double d = dn, c = cn;
        if (k - 1 >= b0) {
            dn = F[(int64_t)(k - 1) * W1 + w];
            cn = (ln < w) ? F[(int64_t)(k - 1) * W1 + ln] : 0.0;
        }
        const double xk = __dmul_rn(__shfl_sync(kFull, v, w), d);
        if (ln == 0) x[(int64_t)k * xs] = xk;
        if (ln < w && k - w + ln >= b0) v = __dsub_rn(v, __dmul_rn(c, xk));
        v = __shfl_up_sync(kFull, v, 1);
        if (ln == 0) v = (k - 1 - w >= b0) ? x[(int64_t)(k - 1 - w) * xs] : 0.0;
    }
}

// the same two solves with the coefficients and the entering values of
// R rows at a time staged in shared memory (one coalesced load per chunk
// instead of a dependent global load per row).  Forward reads the column
// band Fc (Fc[k][0] = d_k, Fc[k][t] = L(k+t, k)), backward the row band F.
constexpr int kChunk = 32;

// chunk c of a block's rows copied asynchronously: coefficient rows
// [r0, r0 + nr) of Fb (w+1 each) and nr entering values starting at row xr
// (zero outside [lo, hi))
__device__ void stage_rows(const double *Fb, int W1, int32_t r0, int nr, const double *x, int32_t xr, int32_t lo,
                           int32_t hi, double *sF, double *sX) {
    const int ln = threadIdx.x & 31;
    for (int e = ln; e < nr * W1; e += 32) __pipeline_memcpy_async(sF + e, Fb + (int64_t)r0 * W1 + e, sizeof(double));
    for (int e = ln; e < nr; e += 32) {
        const int32_t r = xr + e;
        if (r >= lo && r < hi) __pipeline_memcpy_async(sX + e, x + r, sizeof(double));
        else sX[e] = 0.0;
    }
    __pipeline_commit();
}

__device__ void warp_fwd_staged(const double *Fc, int w, int32_t b0, int32_t b1, double *x, double *sF,
                                double *sX) {
    const int ln = threadIdx.x & 31;
    const int W1 = w + 1;
    double v = (ln <= w && b0 + ln < b1) ? x[b0 + ln] : 0.0;
    const int nch = (b1 - b0 + kChunk - 1) / kChunk;
    stage_rows(Fc, W1, b0, min(kChunk, b1 - b0), x, b0 + w + 1, b0, b1, sF, sX);
    for (int ch = 0; ch < nch; ++ch) {
        const int32_t c0 = b0 + ch * kChunk, ce = min(b1, c0 + kChunk);
        const int buf = ch & 1;
        if (ch + 1 < nch) {
            const int32_t n0 = ce, nr = min(kChunk, b1 - n0);
            stage_rows(Fc, W1, n0, nr, x, n0 + w + 1, b0, b1, sF + (buf ^ 1) * kChunk * W1, sX + (buf ^ 1) * kChunk);
            __pipeline_wait_prior(1);
        } else {
            __pipeline_wait_prior(0);
        }
        __syncwarp();
        const double *cF = sF + buf * kChunk * W1, *cX = sX + buf * kChunk;
        for (int32_t k = c0; k < ce; ++k) {
            const int kk = k - c0;
            const double d = cF[kk * W1];
            const double c = (ln >= 1 && ln <= w && k + ln < b1) ? cF[kk * W1 + ln] : 0.0;
            const double xk = __dmul_rn(__shfl_sync(kFull, v, 0), d);
            if (ln == 0) x[k] = xk;
            if (ln >= 1 && ln <= w) v = __dsub_rn(v, __dmul_rn(c, xk));
            v = __shfl_down_sync(kFull, v, 1);
            if (ln == w) v = cX[kk];
        }
        __syncwarp();
    }
}

__device__ void warp_bwd_staged(const double *F, int w, int32_t b0, int32_t b1, double *x, double *sF,
                                double *sX) {
    const int ln = threadIdx.x & 31;
    const int W1 = w + 1;
    double v = (ln <= w && b1 - 1 - w + ln >= b0) ? x[b1 - 1 - w + ln] : 0.0;
    const int nch = (b1 - b0 + kChunk - 1) / kChunk;
    {
        const int32_t c0 = max(b0, b1 - kChunk);
        stage_rows(F, W1, c0, b1 - c0, x, c0 - 1 - w, b0, b1, sF, sX);
    }
    for (int ch = 0; ch < nch; ++ch) {
        const int32_t c1 = b1 - ch * kChunk, c0 = max(b0, c1 - kChunk);
        const int buf = ch & 1;
        if (ch + 1 < nch) {
            const int32_t n1 = c0, n0 = max(b0, n1 - kChunk);
            stage_rows(F, W1, n0, n1 - n0, x, n0 - 1 - w, b0, b1, sF + (buf ^ 1) * kChunk * W1,
                       sX + (buf ^ 1) * kChunk);
            __pipeline_wait_prior(1);
        } else {
            __pipeline_wait_prior(0);
        }
        __syncwarp();
        const double *cF = sF + buf * kChunk * W1, *cX = sX + buf * kChunk;
        for (int32_t k = c1 - 1; k >= c0; --k) {
            const int kk = k - c0;
            const double d = cF[kk * W1 + w];
            const double c = ln < w ? cF[kk * W1 + ln] : 0.0;
            const double xk = __dmul_rn(__shfl_sync(kFull, v, w), d);
            if (ln == 0) x[k] = xk;
            if (ln < w && k - w + ln >= b0) v = __dsub_rn(v, __dmul_rn(c, xk));
            v = __shfl_up_sync(kFull, v, 1);
            if (ln == 0) v = cX[kk];
        }
        __syncwarp();
    }
}

// column band: Fc[k][0] = d_k, Fc[k][t] = L(k+t, k) (0 beyond row n)
__global__ void k_band_colcopy(int32_t n, int32_t w, const double *F, double *Fc) {
    const int32_t W1 = w + 1;
    const int64_t tot = (int64_t)n * W1;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = (int32_t)(e / W1), t = (int32_t)(e - (int64_t)k * W1);
        Fc[e] = t == 0 ? F[(int64_t)k * W1 + w] : (k + t < n ? F[(int64_t)(k + t) * W1 + (w - t)] : 0.0);
    }
}

struct BlockMap {
    int32_t n, s, p;
    __device__ int32_t b0(int32_t b) const { return b * s; }
    __device__ int32_t b1(int32_t b) const { return min(n, (b + 1) * s); }
};

// spikes: G_b[:, q] = L_bb^-1 (column q of the coupling of block b to the
// last w rows of block b-1), H_b[:, r] = L_bb^-T (coupling of row r of
// block b+1 into the last w rows of block b); one warp per (block, column)
__device__ void spike_column(BlockMap M, int32_t w, const double *F, double *G, double *H, int64_t wid) {
    const int32_t W1 = w + 1;
    const int ln = threadIdx.x & 31;
    const int64_t per = (int64_t)M.p * w;
    const bool fwd = wid < per;
    const int64_t u = fwd ? wid : wid - per;
    const int32_t b = (int32_t)(u / w), q = (int32_t)(u - (int64_t)b * w);
    const int32_t b0 = M.b0(b), b1 = M.b1(b);
    if (fwd) {
        if (b == 0) return;
        // rhs: rows b0 + r (r <= q, r < w): L(b0 + r, b0 - w + q) = F[(b0 + r), q - r]
        for (int32_t r = ln; b0 + r < b1; r += 32)
            G[(int64_t)(b0 + r) * w + q] = (r <= q) ? F[(int64_t)(b0 + r) * W1 + (q - r)] : 0.0;
        __syncwarp();
        warp_fwd(F, w, b0, b1, G + q, w);
    } else {
        if (b >= M.p - 1) return;
        // rhs column r = q: rows b1 - w + c (c >= r): L(b1 + r, b1 - w + c) = F[(b1 + r), c - r]
        const int32_t r = q;
        const bool rowOk = b1 + r < M.n;
        for (int32_t i = ln; b0 + i < b1; i += 32) {
            const int32_t row = b0 + i, cidx = row - (b1 - w);
            H[(int64_t)row * w + r] = (rowOk && cidx >= r) ? F[(int64_t)(b1 + r) * W1 + (cidx - r)] : 0.0;
        }
        __syncwarp();
        warp_bwd(F, w, b0, b1, H + r, w);
    }
}

__global__ void k_spikes(BlockMap M, int32_t w, const double *F, double *G, double *H) {
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wid < 2 * (int64_t)M.p * w;
         wid += nwarp)
        spike_column(M, w, F, G, H, wid);
}

constexpr int kSolveWarps = 4;

__global__ void __launch_bounds__(32 * kSolveWarps) k_bsolve_fwd_local(BlockMap M, int32_t w, const double *Fc,
                                                                       const int *done, double *y) {
    if (done && *done) return;
    extern __shared__ double sm[];
    const int wib = threadIdx.x >> 5;
    double *sF = sm + (int64_t)wib * 2 * kChunk * (w + 2), *sX = sF + 2 * kChunk * (w + 1);
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < M.p; b += nwarp)
        warp_fwd_staged(Fc, w, M.b0((int32_t)b), M.b1((int32_t)b), y, sF, sX);
}

// the coupling rows (w x w, contiguous in G or H) and the w values of a
// run of blocks, copied asynchronously into one of two shared buffers:
// block q of the run at sg + q*w*w and sy + q*w; rows past a block's
// nrow are zero
template <class RowOf, class NrowOf, class UseG>
__device__ void stage_run(const double *G, const double *y, int32_t w, int32_t bfirst, int nblk, int dir,
                          RowOf rowOf, NrowOf nrowOf, UseG useG, double *sg, double *sy) {
    const int ln = threadIdx.x & 31;
    const int ww = w * w;
    for (int q = 0; q < nblk; ++q) {
        const int32_t b = bfirst + dir * q;
        const int32_t r0 = rowOf(b);
        const int nrow = nrowOf(b);
        const bool g = useG(b);
        for (int e = ln; e < ww; e += 32) {
            if (g && e < nrow * w) __pipeline_memcpy_async(sg + q * ww + e, G + (int64_t)r0 * w + e, sizeof(double));
            else sg[q * ww + e] = 0.0;
        }
        for (int e = ln; e < w; e += 32) {
            if (e < nrow) __pipeline_memcpy_async(sy + q * w + e, y + r0 + e, sizeof(double));
            else sy[q * w + e] = 0.0;
        }
    }
    __pipeline_commit();
}

// blocks per staged run: two runs of (w*w + w) doubles in 32 KB
__host__ __device__ inline int run_blocks(int w) { return max(1, min(64, 2048 / max(1, w * w + w))); }

// tails t_b = y_b[last w] - G_b[last w] t_{b-1}, sequential over blocks;
// the next run of blocks is copied while the current one is computed
__global__ void k_bsolve_tails(BlockMap M, int32_t w, const double *G, const int *done, const double *y,
                               double *T) {
    if (done && *done) return;
    extern __shared__ double sm[];
    __shared__ double tp[32];
    const int D = run_blocks(w), ww = w * w;
    double *sg = sm, *sy = sm + 2 * D * ww;
    const int ln = threadIdx.x;
    tp[ln] = 0.0;
    const int32_t nb = M.p - 1;
    auto rowOf = [&](int32_t b) { return M.b1(b) - w; };
    auto nrowOf = [&](int32_t) { return w; };
    auto useG = [&](int32_t) { return true; };
    const int nrun = (nb + D - 1) / D;
    if (nrun > 0) stage_run(G, y, w, 0, min(D, nb), 1, rowOf, nrowOf, useG, sg, sy);
    for (int r = 0; r < nrun; ++r) {
        const int buf = r & 1;
        if (r + 1 < nrun) {
            const int32_t f = (r + 1) * D;
            stage_run(G, y, w, f, min(D, nb - f), 1, rowOf, nrowOf, useG, sg + (buf ^ 1) * D * ww,
                      sy + (buf ^ 1) * D * w);
            __pipeline_wait_prior(1);
        } else {
            __pipeline_wait_prior(0);
        }
        __syncwarp();
        const int32_t f = r * D, cntb = min(D, nb - f);
        for (int q = 0; q < cntb; ++q) {
            const int32_t b = f + q;
            const double *g = sg + buf * D * ww + q * ww;
            double t = 0.0;
            if (ln < w) {
                double a0 = 0.0, a1 = 0.0;
                if (b > 0) {
                    const double *gr = g + ln * w;
                    int c = 0;
                    for (; c + 1 < w; c += 2) {
                        a0 = __fma_rn(gr[c], tp[c], a0);
                        a1 = __fma_rn(gr[c + 1], tp[c + 1], a1);
                    }
                    if (c < w) a0 = __fma_rn(gr[c], tp[c], a0);
                }
                t = sy[buf * D * w + q * w + ln] - (a0 + a1);
                T[(int64_t)b * w + ln] = t;
            }
            __syncwarp();
            if (ln < w) tp[ln] = t;
            __syncwarp();
        }
    }
}

// y_b -= G_b t_{b-1}, then L_bb^T u_b = y_b in place
__global__ void __launch_bounds__(32 * kSolveWarps) k_bsolve_bwd_local(BlockMap M, int32_t w, const double *F,
                                                                       const double *G, const double *T,
                                                                       const int *done, double *y) {
    if (done && *done) return;
    extern __shared__ double sm[];
    const int wib = threadIdx.x >> 5;
    double *sF = sm + (int64_t)wib * 2 * kChunk * (w + 2), *sX = sF + 2 * kChunk * (w + 1);
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int ln = threadIdx.x & 31;
    for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < M.p; b += nwarp) {
        const int32_t b0 = M.b0((int32_t)b), b1 = M.b1((int32_t)b);
        if (b > 0 && G) {
            const double *t = T + (b - 1) * w;
            for (int32_t r = b0 + ln; r < b1; r += 32) {
                const double *g = G + (int64_t)r * w;
                double a = 0.0;
                for (int q = 0; q < w; ++q) a = __fma_rn(g[q], t[q], a);
                y[r] -= a;
            }
            __syncwarp();
        }
        warp_bwd_staged(F, w, b0, b1, y, sF, sX);
    }
}

// heads h_b = u_b[first w] - H_b[first w] h_{b+1}, sequential downwards
// with the same staging (the last block has no H rows)
__global__ void k_bsolve_heads(BlockMap M, int32_t w, const double *H, const int *done, const double *y,
                               double *Hd) {
    if (done && *done) return;
    extern __shared__ double sm[];
    __shared__ double hp[32];
    const int D = run_blocks(w), ww = w * w;
    double *sg = sm, *sy = sm + 2 * D * ww;
    const int ln = threadIdx.x;
    hp[ln] = 0.0;
    const int32_t nb = M.p;
    auto rowOf = [&](int32_t b) { return M.b0(b); };
    auto nrowOf = [&](int32_t b) { return min(w, M.b1(b) - M.b0(b)); };
    auto useG = [&](int32_t b) { return b < M.p - 1; };
    const int nrun = (nb + D - 1) / D;
    // runs downwards: run r holds blocks p-1-r*D, p-2-r*D, ...
    stage_run(H, y, w, nb - 1, min(D, nb), -1, rowOf, nrowOf, useG, sg, sy);
    for (int r = 0; r < nrun; ++r) {
        const int buf = r & 1;
        if (r + 1 < nrun) {
            const int32_t f = nb - 1 - (r + 1) * D;
            stage_run(H, y, w, f, min(D, f + 1), -1, rowOf, nrowOf, useG, sg + (buf ^ 1) * D * ww,
                      sy + (buf ^ 1) * D * w);
            __pipeline_wait_prior(1);
        } else {
            __pipeline_wait_prior(0);
        }
        __syncwarp();
        const int32_t f = nb - 1 - r * D, cntb = min(D, f + 1);
        for (int q = 0; q < cntb; ++q) {
            const int32_t b = f - q;
            const int32_t b0 = M.b0(b), b1 = M.b1(b);
            const double *g = sg + buf * D * ww + q * ww;
            double h = 0.0;
            if (ln < w && b0 + ln < b1) {
                double a0 = 0.0, a1 = 0.0;
                if (b < M.p - 1) {
                    const double *gr = g + ln * w;
                    int c = 0;
                    for (; c + 1 < w; c += 2) {
                        a0 = __fma_rn(gr[c], hp[c], a0);
                        a1 = __fma_rn(gr[c + 1], hp[c + 1], a1);
                    }
                    if (c < w) a0 = __fma_rn(gr[c], hp[c], a0);
                }
                h = sy[buf * D * w + q * w + ln] - (a0 + a1);
            }
            if (ln < w) Hd[(int64_t)b * w + ln] = h;
            __syncwarp();
            if (ln < w) hp[ln] = h;
            __syncwarp();
        }
    }
}

// x_b = u_b - H_b h_{b+1}
__global__ void k_bsolve_fix(BlockMap M, int32_t w, const double *H, const double *Hd, const int *done,
                             double *y) {
    if (done && *done) return;
    const int32_t rowsCoupled = min(M.n, (M.p - 1) * M.s);
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rowsCoupled;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = (int32_t)(r / M.s);
        const double *g = H + r * w, *h = Hd + (int64_t)(b + 1) * w;
        double a = 0.0;
        for (int q = 0; q < w; ++q) a = __fma_rn(g[q], h[q], a);
        y[r] -= a;
    }
}

BlockMap block_map(const BandPre &P) { return BlockMap{P.n, P.s, P.p}; }
}  // namespace

int32_t band_alloc(BandPre &P, int32_t nVar, int32_t nfit, int32_t w) {
    band_free(P);
    P.n = nfit;
    P.w = w;
    // rows per block: about sqrt(2 n) (balances the per-block chains against
    // the sequential w x w steps), a multiple of 32, at least 64 and w
    int64_t s = (int64_t)std::llround(std::sqrt(2.0 * std::max(nfit, 1)) / 32.0) * 32;
    s = std::max<int64_t>(std::max<int64_t>(s, 64), w);
    P.s = (int32_t)s;
    P.p = (int32_t)((std::max(nfit, 1) + s - 1) / s);
    const int64_t W1 = w + 1;
    auto al = [](double *&d, int64_t len) {
        return cudaMalloc(&d, sizeof(double) * std::max<int64_t>(len, 1)) == cudaSuccess;
    };
    bool ok = al(P.B, (int64_t)nVar * W1) && al(P.F, (int64_t)std::max(nfit, 1) * W1) &&
              al(P.Fc, (int64_t)std::max(nfit, 1) * W1) &&
              al(P.G, (int64_t)std::max(nfit, 1) * std::max(w, 1)) &&
              al(P.H, (int64_t)std::max(nfit, 1) * std::max(w, 1)) &&
              al(P.T, (int64_t)P.p * std::max(w, 1)) && al(P.Hd, (int64_t)P.p * std::max(w, 1));
    ok = ok && cudaMalloc(&P.nrkd, sizeof(int32_t)) == cudaSuccess;
    if (!ok) {
        band_free(P);
        return MPGPU_ERR_ALLOC;
    }
    return MPGPU_OK;
}

void band_free(BandPre &P) {
    for (double **p : {&P.B, &P.F, &P.Fc, &P.G, &P.H, &P.T, &P.Hd}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    if (P.nrkd) cudaFree(P.nrkd);
    P.nrkd = nullptr;
}

cudaError_t band_fill(const BandPre &P, int32_t nVar, int32_t matsto, const double *matD, const int32_t *aig,
                      const int32_t *p2g, const int64_t *rowStart, const int32_t *bcol, const int64_t *boff,
                      const int32_t *bld, cudaStream_t s) {
    k_band_fill<<<grid_for((int64_t)nVar * (P.w + 1), kT), kT, 0, s>>>(nVar, P.w, matsto, matD, aig, p2g,
                                                                        rowStart, bcol, boff, bld, P.B);
    return cudaGetLastError();
}

cudaError_t band_reflect(const BandPre &P, int32_t nVar, const double *v, const double *y, const double *beta,
                         cudaStream_t s) {
    k_band_reflect<<<grid_for((int64_t)nVar * (P.w + 1), kT), kT, 0, s>>>(nVar, P.w, P.B, v, y, beta);
    return cudaGetLastError();
}

cudaError_t band_factor(const BandPre &P, int32_t lprecm, cudaStream_t s) {
    const int W1 = P.w + 1;
    cudaError_t e = cudaMemsetAsync(P.F, 0, sizeof(double) * (size_t)std::max(P.n, 1) * W1, s);
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(double) * W1 * W1 + sizeof(uint16_t) * (P.w * (P.w + 1) / 2 + 1);
    k_lltdec<<<1, 32, smem, s>>>(P.n, P.w, P.B, P.F, lprecm, P.nrkd);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_band_colcopy<<<grid_for((int64_t)P.n * W1, kT), kT, 0, s>>>(P.n, P.w, P.F, P.Fc);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (P.p > 1 && P.w > 0) {
        const int64_t warps = 2 * (int64_t)P.p * P.w;
        k_spikes<<<grid_for(warps * 32, kT), kT, 0, s>>>(block_map(P), P.w, P.F, P.G, P.H);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t band_solve(const BandPre &P, const int *done, double *y, cudaStream_t s) {
    const BlockMap M = block_map(P);
    // warps per CTA: as many as fit two chunks each in 48 KB (at most 4)
    const size_t perWarp = sizeof(double) * 2 * kChunk * (P.w + 2);
    const int wpc = (int)std::max<size_t>(1, std::min<size_t>(kSolveWarps, (48 * 1024) / perWarp));
    const int gw = (int)((P.p + wpc - 1) / wpc);
    const size_t smem = perWarp * wpc;
    k_bsolve_fwd_local<<<gw, 32 * wpc, smem, s>>>(M, P.w, P.Fc, done, y);
    const bool coupled = P.p > 1 && P.w > 0;
    const size_t srun = sizeof(double) * 2 * run_blocks(P.w) * (P.w * P.w + P.w);
    if (coupled) k_bsolve_tails<<<1, 32, srun, s>>>(M, P.w, P.G, done, y, P.T);
    k_bsolve_bwd_local<<<gw, 32 * wpc, smem, s>>>(M, P.w, P.F, coupled ? P.G : nullptr, P.T, done, y);
    if (coupled) {
        k_bsolve_heads<<<1, 32, srun, s>>>(M, P.w, P.H, done, y, P.Hd);
        k_bsolve_fix<<<grid_for((int64_t)(P.p - 1) * P.s, kT), kT, 0, s>>>(M, P.w, P.H, P.Hd, done, y);
    }
    return cudaGetLastError();
}
