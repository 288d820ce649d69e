// mpgpu_solve.cu -- global solvers on the device: QL constraint
// elimination products, packed Gauss-Jordan inversion (sqminl), root-free
// Cholesky (chdec2/chslv2), the sparse and packed symmetric matrix-vector
// product (avprd0) and preconditioned MINRES.  All reductions have a fixed
// shape, so repeated solves give bit-identical results.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mpgpu_ctx.h"

namespace {

constexpr int kDotBlocks = 304;   // 2 x 152 SMs, fixed for determinism
constexpr int kThreads = 256;

template <class T>
void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double block_sum(double v, double *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    double r = sh[0];
    __syncthreads();
    return r;
}

__global__ void k_dot_partial(int64_t n, const double *a, const double *b, double *part) {
    __shared__ double sh[kThreads];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_sum_final(const double *part, int n, double *out) {
    __shared__ double sh[kThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) *out = s;
}

void dot(const double *a, const double *b, int64_t n, double *part, double *out, cudaStream_t s) {
    k_dot_partial<<<kDotBlocks, kThreads, 0, s>>>(n, a, b, part);
    k_sum_final<<<1, kThreads, 0, s>>>(part, kDotBlocks, out);
}

// ---------------------------------------------------------------- QL products
// qlmlq (mpqldec.f90:404-454) for one vector, one CTA walking the
// reflections k = kfirst, kfirst+step, ..., klast in that order
// (Q x: 1..ncon; Q^T x: ncon..1).
__global__ void k_qlapply(double *x, const double *V, const double *Vk, const int32_t *r2, int32_t npar,
                          int32_t ncon, int kfirst, int klast, int step) {
    __shared__ double sh[1024];
    if (step == 0) return;
    for (int k = kfirst; step > 0 ? k <= klast : k >= klast; k += step) {
        const int kn = npar + k - ncon;
        const int ilast = r2[k - 1];
        const double *v = V + (int64_t)(k - 1) * npar;
        const double vk = Vk[k - 1];
        double s = 0.0;
        for (int i = threadIdx.x; i < ilast; i += blockDim.x) s += v[i] * x[i];
        s = block_sum(s, sh);
        const double sp = s + vk * x[kn - 1];
        __syncthreads();
        for (int i = threadIdx.x; i < ilast; i += blockDim.x) x[i] = x[i] - 2.0 * v[i] * sp;
        if (threadIdx.x == 0) x[kn - 1] = x[kn - 1] - 2.0 * vk * sp;
        __syncthreads();
    }
}

// qlmlq in the compact WY form: Q^T x = x - U T (U^T x), Q x = x - U T^T
// (U^T x), U = the reflection vectors (rows of V with Vk at position
// npar - ncon + k).  Pass 1: per CTA the partial products of eight vectors
// at a time over a fixed row partition; pass 2 (one CTA): the sums in CTA
// order plus the Vk terms, then t = T s or T^T s; pass 3: x -= U t.
constexpr int kWyBlocks = 304;

__global__ void __launch_bounds__(256) k_wy_dots(int32_t n, int32_t m, const double *V, const double *x,
                                                  double *part) {
    __shared__ double sh[8][8];
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int32_t k0 = 0; k0 < m; k0 += 8) {
        const int kc = min(8, m - k0);
        double acc[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = 0.0;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const double xi = x[i];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q < kc) acc[q] += V[(int64_t)(k0 + q) * n + i] * xi;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            double v = acc[q];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (ln == 0) sh[q][wib] = v;
        }
        __syncthreads();
        if ((int)threadIdx.x < kc) {
            double v = 0.0;
            for (int w8 = 0; w8 < (int)(blockDim.x >> 5); ++w8) v += sh[threadIdx.x][w8];
            part[(int64_t)blockIdx.x * m + k0 + threadIdx.x] = v;
        }
        __syncthreads();
    }
}

__global__ void k_wy_coef(int32_t n, int32_t m, int32_t nblk, const double *part, const double *Vk,
                          const double *T, const double *x, int transT, double *tv) {
    extern __shared__ double sv[];
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * m + k];
        sv[k] = s + Vk[k] * x[n - m + k];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double t = 0.0;
        if (transT)
            for (int c = 0; c <= k; ++c) t += T[(int64_t)c * m + k] * sv[c];
        else
            for (int c = k; c < m; ++c) t += T[(int64_t)k * m + c] * sv[c];
        tv[k] = t;
    }
}

__global__ void k_wy_apply(int32_t n, int32_t m, const double *V, const double *Vk, const double *tv, double *x) {
    extern __shared__ double st[];
    for (int k = threadIdx.x; k < m; k += blockDim.x) st[k] = tv[k];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = 0.0;
        for (int k = 0; k < m; ++k) a += V[(int64_t)k * n + i] * st[k];
        const int64_t kk = i - (n - m);
        if (kk >= 0) a += Vk[kk] * st[kk];
        x[i] -= a;
    }
}

// ---------------------------------------------------------------- packed products
// y = A x for the packed symmetric matrix in two deterministic passes.
// Pass 1, one CTA per block of 64 rows: the lower part of each row (one
// warp per row, contiguous) and, per column j left of the block's last row,
// the partial column sum over the block's rows (one thread per column,
// contiguous across threads).  Pass 2 adds, per j, the row part and the
// partial column sums of the blocks below j in block order.
constexpr int kMvRows = 16;

__global__ void __launch_bounds__(256) k_pmv_blocks(int32_t n, const double *A, const double *x, double *yrow,
                                                     double *part) {
    const int64_t b = blockIdx.x;
    const int64_t i0 = b * kMvRows, i1 = min((int64_t)n, i0 + kMvRows);
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    __shared__ double xs[kMvRows];
    if (threadIdx.x < kMvRows) xs[threadIdx.x] = i0 + threadIdx.x < n ? x[i0 + threadIdx.x] : 0.0;
    __syncthreads();
    for (int64_t i = i0 + wib; i < i1; i += 8) {
        const double *row = A + i * (i + 1) / 2;
        double s = 0.0;
        for (int64_t j = ln; j <= i; j += 32) s += row[j] * x[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (ln == 0) yrow[i] = s;
    }
    for (int64_t j = threadIdx.x; j < i1 - 1; j += blockDim.x) {
        double s = 0.0;
        const int64_t ifirst = j + 1 > i0 ? j + 1 : i0;
        for (int64_t i = ifirst; i < i1; ++i) s += A[i * (i + 1) / 2 + j] * xs[i - i0];
        part[b * (int64_t)n + j] = s;
    }
}

__global__ void k_pmv_final(int32_t n, int64_t nb, const double *yrow, const double *part, double *y) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = yrow[j];
    for (int64_t b = (j + 1) / kMvRows; b < nb; ++b) {
        const int64_t i1 = min((int64_t)n, (b + 1) * kMvRows);
        if (j < i1 - 1) s += part[b * (int64_t)n + j];
    }
    y[j] = s;
}

// qlssq update of one reflection on the packed matrix (mpqldec.f90:
// 644-686): rows 1..kn get 2(2 v_i vtAv - Av_i) v_c for c in [1, min(ilast,i)],
// rows ilast and below in [1, ilast] get -2 Av_c v_i, the diagonal (kn,kn)
// its combined term and rows > kn their -2 v_c Av_i parts.
__global__ void k_qlssq_update(int32_t n, double *A, const double *v, double vk, const double *Av,
                               const double *vtAvp, int32_t ilast, int32_t kn) {
    const double vtAv = *vtAvp;
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i1 = 1 + w; i1 <= n; i1 += nw) {   // 1-based row
        double *row = A + (i1 * i1 - i1) / 2 - 1;     // row[c] = A(i1, c), c 1-based
        const double vi = (i1 <= ilast) ? v[i1 - 1] : (i1 == kn ? vk : 0.0);
        if (i1 <= ilast) {
            // both corrections of the reference, in its order, in one pass
            const double f = 2.0 * vi * vtAv - Av[i1 - 1];
            for (int64_t cc = 1 + ln; cc <= i1; cc += 32)
                row[cc] = (row[cc] + 2.0 * (f * v[cc - 1])) - 2.0 * Av[cc - 1] * vi;
        } else if (i1 <= kn) {
            const double f = 2.0 * vi * vtAv - Av[i1 - 1];
            for (int64_t cc = 1 + ln; cc <= ilast; cc += 32) row[cc] = row[cc] + 2.0 * (f * v[cc - 1]);
        }
        if (i1 == kn && ln == 0) row[kn] = row[kn] + 2.0 * ((2.0 * vk * vtAv - Av[kn - 1]) * vk - Av[kn - 1] * vk);
        if (i1 > kn) {
            const double avi = Av[i1 - 1];
            for (int64_t cc = 1 + ln; cc <= ilast; cc += 32) row[cc] = row[cc] - 2.0 * v[cc - 1] * avi;
            if (ln == 0) row[kn] = row[kn] - 2.0 * vk * avi;
        }
    }
}

__global__ void k_vec_with_kn(const double *v, int32_t ilast, double vk, int32_t kn, int32_t n, double *out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = i < ilast ? v[i] : (i == kn - 1 ? vk : 0.0);
}

// sqminl pivot step part 1 (one CTA): choose the pivot (first remaining
// index with the largest |v_jj| above 1e-10 * |original diagonal|, the
// choice of the reference's linked-list scan), scale the pivot row/column.
__global__ void k_sqminl_pivot(int32_t n, double *v, double *b, const double *diag, int32_t *used,
                               double *vk, double *scal, int32_t *pivot) {
    __shared__ double sb[1024];
    __shared__ int sk[1024];
    const double eps = 1.0E-10;
    double best = -1.0;
    int bk = -1;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        if (used[j]) continue;
        const double a = fabs(v[(int64_t)(j + 1) * (j + 2) / 2 - 1]);
        if (a > eps * diag[j] && a > best) { best = a; bk = j; }
    }
    sb[threadIdx.x] = best;
    sk[threadIdx.x] = bk;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            const double ob = sb[threadIdx.x + s];
            const int ok = sk[threadIdx.x + s];
            if (ob > sb[threadIdx.x] || (ob == sb[threadIdx.x] && ok >= 0 && (sk[threadIdx.x] < 0 || ok < sk[threadIdx.x]))) {
                sb[threadIdx.x] = ob;
                sk[threadIdx.x] = ok;
            }
        }
        __syncthreads();
    }
    const int k = sk[0];
    if (threadIdx.x == 0) *pivot = k;
    if (k < 0) return;
    const int64_t kk = (int64_t)(k + 1) * (k + 2) / 2 - 1;
    const double vkk = 1.0 / v[kk];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        if (j == k) { vk[j] = 0.0; continue; }
        const int64_t jk = j > k ? (int64_t)j * (j + 1) / 2 + k : (int64_t)k * (k + 1) / 2 + j;
        const double s = v[jk] * vkk;
        v[jk] = s;
        vk[j] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        v[kk] = -vkk;
        b[k] = b[k] * vkk;
        used[k] = 1;
        scal[0] = vkk;
    }
}

// sqminl pivot step part 2: rank-1 elimination of rows j != k
__global__ void k_sqminl_elim(int32_t n, double *v, double *b, const double *vk, const double *scal,
                              const int32_t *pivot) {
    const int k = *pivot;
    if (k < 0) return;
    const double vkk = scal[0];
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const double bk = b[k];
    for (int64_t j = w; j < n; j += nw) {
        if (j == k) continue;
        const double vjk = vk[j] / vkk;
        if (ln == 0) b[j] = b[j] - bk * vjk;
        double *row = v + j * (j + 1) / 2;
        for (int64_t c = ln; c <= j; c += 32) row[c] = row[c] - vk[c] * vjk;
    }
}

__global__ void k_sqminl_deficit(int32_t n, double *v, double *b, const int32_t *used, const int32_t *pivot) {
    if (*pivot >= 0) return;
    for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
        if (used[j]) continue;
        if (threadIdx.x == 0) b[j] = 0.0;
        double *row = v + j * (j + 1) / 2;
        for (int64_t c = threadIdx.x; c <= j; c += blockDim.x)
            if (!used[c]) row[c] = 0.0;
    }
}

__global__ void k_negate(int64_t n, double *v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = -v[i];
}

__global__ void k_diag_abs(int32_t n, const double *v, double *d) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = fabs(v[(i + 1) * (i + 2) / 2 - 1]);
}

// chdec2 step i (1-based): pivot, then the rank-1 update of rows 1..i-1
__global__ void k_chdec_pivot(int64_t i, double *g, double *stat) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int64_t ii = i * (i + 1) / 2 - 1;
    if (g[ii] > 0.0) {
        const double d = g[ii];
        if (stat[2] == 0.0) { stat[0] = d; stat[1] = d; }
        else { stat[0] = fmax(stat[0], d); stat[1] = fmin(stat[1], d); }
        stat[2] += 1.0;
        g[ii] = 1.0 / d;
    }
}

__global__ void k_chdec_update(int64_t i, double *g) {
    const int64_t rowi = (i * i - i) / 2 - 1;   // g[rowi + c] = G(i, c), c 1-based
    const double gii = g[rowi + i];
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = 1 + w; j <= i - 1; j += nw) {
        const double ratio = g[rowi + j] * gii;
        if (ratio == 0.0) continue;
        double *rowj = g + (j * j - j) / 2 - 1;
        for (int64_t c = 1 + ln; c <= j; c += 32) rowj[c] = rowj[c] - g[rowi + c] * ratio;
    }
}

__global__ void k_chdec_scale(int64_t i, double *g) {
    const int64_t rowi = (i * i - i) / 2 - 1;
    const double gii = g[rowi + i];
    for (int64_t c = 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c <= i - 1; c += (int64_t)gridDim.x * blockDim.x)
        g[rowi + c] = g[rowi + c] * gii;
}

// chslv2 (mpnum.f90:953-987), one CTA: backward then forward substitution
__global__ void k_chslv2(const double *g, double *x, int32_t n) {
    __shared__ double sh[1024];
    // backward: x(i) -= sum_{k>i} G(k,i) x(k)
    for (int64_t i = n; i >= 1; --i) {
        double s = 0.0;
        for (int64_t k = i + 1 + threadIdx.x; k <= n; k += blockDim.x) s += g[(k * k - k) / 2 + i - 1] * x[k - 1];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) x[i - 1] = x[i - 1] - s;
        __syncthreads();
    }
    for (int64_t i = 1; i <= n; ++i) {
        const int64_t ro = (i * i - i) / 2 - 1;
        double s = 0.0;
        for (int64_t k = 1 + threadIdx.x; k <= i - 1; k += blockDim.x) s += g[ro + k] * x[k - 1];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) x[i - 1] = x[i - 1] * g[ro + i] - s;
        __syncthreads();
    }
}

// corr(i) -= sum_j A'(nfit+j, i) y(j), i <= nfit (minver/mchdec rhs)
__global__ void k_cons_rhs(int32_t nfit, int32_t ncon, const double *A, const double *y, double *corr) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nfit; i += (int64_t)gridDim.x * blockDim.x) {
        double cval = corr[i];
        for (int j = 0; j < ncon; ++j) {
            const int64_t r = nfit + j + 1;
            cval = cval - A[(r * r - r) / 2 + i] * y[j];
        }
        corr[i] = cval;
    }
}

__global__ void k_zero_rows(int32_t nfit, int32_t n, double *A) {
    for (int64_t r = nfit + 1 + blockIdx.x; r <= n; r += gridDim.x) {
        double *row = A + (r * r - r) / 2;
        for (int64_t c = threadIdx.x; c < r; c += blockDim.x) row[c] = 0.0;
    }
}

__global__ void k_get_diag(int32_t n, const double *A, double *d) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = A[(i + 1) * (i + 2) / 2 - 1];
}

// ---------------------------------------------------------------- sparse SpMV
// Block table of the mpbits storage: for every stored block (I, J <= I) the
// 0-based offset of element (0,0) in globalMatD and the row stride.
struct SparseBlocks {
    int64_t nblk = 0;
    int64_t *rowStart = nullptr;   // [nG+1] blocks of row group I
    int32_t *bcol = nullptr;       // column group
    int64_t *boff = nullptr;
    int32_t *bld = nullptr;
    int64_t *tOff = nullptr;       // transposed-product buffer offset (off-diagonal blocks)
    int64_t *colStart = nullptr;   // [nG+1] incoming blocks of column group J
    int64_t *colBlk = nullptr;     // block ids ordered by (J, I)
    int64_t *tBase = nullptr;      // [nG] first transposed product of column group J
    double *tbuf = nullptr;
    int64_t tlen = 0;
    bool smallGroups = false;     // every group has at most kSmallGroup parameters
    // small groups: per block its row group (brow), its partial row sums
    // (rowPart, kSmallGroup each) and the stride of its transposed products
    // (tStr: the column group's incoming block count, parameter-major)
    int32_t *brow = nullptr;       // [nblk]
    int32_t *tStr = nullptr;       // [nblk]
    double *rowPart = nullptr;     // [nblk * kSmallGroup]
    // column items: at most kColItem incoming blocks of one column group
    int64_t nColItem = 0;
    int32_t *colItemJ = nullptr;   // [nColItem]
    int64_t *colItemQ0 = nullptr;  // [nColItem] first incoming block (0-based within the group)
    int64_t *colItemQ1 = nullptr;  // [nColItem] end
    int64_t *colItemBeg = nullptr; // [nG+1] first item of column group J
    double *colPart = nullptr;     // [nColItem * kSmallGroup]
    int uniform = 0;               // every group has this many parameters (0: mixed)
};

// phase 1: warp per row group I: y_I = D_I x_I + sum_J A_IJ x_J, the
// strictly-lower part of the diagonal block also transposed into y_I, and
// t_IJ = A_IJ^T x_I for J < I into tbuf
__global__ void k_spmv_rows(int32_t nG, const int32_t *aig, const int64_t *rowStart, const int32_t *bcol,
                            const int64_t *boff, const int32_t *bld, const int64_t *tOff,
                            const double *matD, const double *x, double *y, double *tbuf) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t I = 1 + w; I <= nG; I += nw) {
        const int32_t ia = aig[I - 1] - 1, np = aig[I] - 1 - ia;
        for (int ii = 0; ii < np; ++ii) {
            double s = 0.0;
            for (int64_t bl = rowStart[I - 1]; bl < rowStart[I]; ++bl) {
                const int32_t J = bcol[bl];
                const int32_t ja = aig[J - 1] - 1, nj = aig[J] - 1 - ja;
                const double *row = matD + boff[bl] + (int64_t)ii * bld[bl];
                if (J == I) {
                    for (int jj = ln; jj < ii; jj += 32) s += row[jj] * x[ja + jj];
                    // transposed strictly-lower part: A(r, ii) for r > ii
                    for (int rr = ii + 1 + ln; rr < np; rr += 32)
                        s += matD[boff[bl] + (int64_t)rr * bld[bl] + ii] * x[ia + rr];
                } else {
                    for (int jj = ln; jj < nj; jj += 32) s += row[jj] * x[ja + jj];
                }
            }
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (ln == 0) y[ia + ii] = matD[ia + ii] * x[ia + ii] + s;
        }
        // transposed products of the off-diagonal blocks
        for (int64_t bl = rowStart[I - 1]; bl < rowStart[I]; ++bl) {
            const int32_t J = bcol[bl];
            if (J == I) continue;
            const int32_t nj = aig[J] - aig[J - 1];
            for (int jj = ln; jj < nj; jj += 32) {
                double t = 0.0;
                for (int ii = 0; ii < np; ++ii) t += matD[boff[bl] + (int64_t)ii * bld[bl] + jj] * x[ia + ii];
                tbuf[tOff[bl] + jj] = t;
            }
        }
    }
}

// phase 2: warp per column group J adds the transposed products in a fixed order
__global__ void k_spmv_cols(int32_t nG, const int32_t *aig, const int64_t *colStart, const int64_t *colBlk,
                            const int64_t *tOff, const double *tbuf, double *y) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t J = 1 + w; J <= nG; J += nw) {
        const int32_t ja = aig[J - 1] - 1, nj = aig[J] - 1 - ja;
        for (int jj = ln; jj < nj; jj += 32) {
            double s = y[ja + jj];
            for (int64_t q = colStart[J - 1]; q < colStart[J]; ++q) s += tbuf[tOff[colBlk[q]] + jj];
            y[ja + jj] = s;
        }
    }
}

// the same two phases for row groups of at most 8 parameters.  Phase 1,
// one thread per stored block (all blocks of all row groups, so the lanes
// stay full whatever the row lengths): the block's rows times x_J into its
// partial row sums (rowPart, 8 per block; the diagonal block adds both
// triangles of its strictly-lower part there) and its columns times x_I
// into tbuf (parameter-major per column group).  G > 0: every group has G
// parameters (loops fully unrolled); G = 0: at most 8, predicated.  Phase
// 2: the partial row sums of a group's blocks and the transposed products
// of its incoming blocks summed by column items (long columns split over
// several warps), then y = D x + the group's items in item order; no
// atomics, the sums are reproducible.
constexpr int kSmallGroup = 8;

template <int G>
__global__ void __launch_bounds__(256) k_spmv_blocks(int64_t nb, const int32_t *brow, const int32_t *aig,
                                                     const int32_t *bcol, const int64_t *boff, const int32_t *bld,
                                                     const int64_t *tOff, const int32_t *tStr,
                                                     const double *matD, const double *x, double *tbuf,
                                                     double *rowPart) {
    constexpr int M = G > 0 ? G : kSmallGroup;
    for (int64_t bl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; bl < nb;
         bl += (int64_t)gridDim.x * blockDim.x) {
        const int32_t I = brow[bl], J = bcol[bl];
        const int32_t ia = aig[I - 1] - 1, ja = aig[J - 1] - 1;
        const int np = G > 0 ? G : aig[I] - 1 - ia;
        const int nj = G > 0 ? G : aig[J] - 1 - ja;
        const double *blk = matD + boff[bl];
        const int32_t ld = bld[bl];
        double xi[M], sr[M];
#pragma unroll
        for (int ii = 0; ii < M; ++ii) {
            xi[ii] = ii < np ? x[ia + ii] : 0.0;
            sr[ii] = 0.0;
        }
        if (J != I) {
            double xj[M], tc[M];
#pragma unroll
            for (int jj = 0; jj < M; ++jj) {
                xj[jj] = jj < nj ? x[ja + jj] : 0.0;
                tc[jj] = 0.0;
            }
#pragma unroll
            for (int ii = 0; ii < M; ++ii) {
                if (ii < np) {
#pragma unroll
                    for (int jj = 0; jj < M; ++jj) {
                        if (jj < nj) {
                            const double a = blk[(int64_t)ii * ld + jj];
                            sr[ii] += a * xj[jj];
                            tc[jj] += a * xi[ii];
                        }
                    }
                }
            }
            double *tb = tbuf + tOff[bl];
            const int32_t st = tStr[bl];
#pragma unroll
            for (int jj = 0; jj < M; ++jj)
                if (jj < nj) tb[(int64_t)jj * st] = tc[jj];
        } else {
#pragma unroll
            for (int ii = 1; ii < M; ++ii) {
                if (ii < np) {
#pragma unroll
                    for (int jj = 0; jj < ii; ++jj) {
                        const double a = blk[(int64_t)ii * ld + jj];
                        sr[ii] += a * xi[jj];
                        sr[jj] += a * xi[ii];
                    }
                }
            }
        }
        double *rp = rowPart + bl * kSmallGroup;
#pragma unroll
        for (int ii = 0; ii < M; ++ii) rp[ii] = sr[ii];
    }
}

// phase 2a, one warp per column item (at most kColItem incoming blocks of
// one column group; the first item of a group also takes the partial row
// sums of the group's own blocks): lanes with four independent partial
// sums, a fixed shuffle tree, into colPart (8 per item)
constexpr int kColItem = 128;

__global__ void __launch_bounds__(256) k_spmv_colitems(int64_t nItem, const int32_t *itemJ, const int64_t *itemQ0,
                                                       const int64_t *itemQ1, const int32_t *aig,
                                                       const int64_t *rowStart, const double *rowPart,
                                                       const int64_t *colStart, const int64_t *tBase,
                                                       const double *tbuf, double *colPart) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t it = w; it < nItem; it += nw) {
        const int32_t J = itemJ[it];
        const int32_t nj = aig[J] - aig[J - 1];
        const int64_t q0 = itemQ0[it], q1 = itemQ1[it];
        const bool first = q0 == 0;
        const int64_t r0 = rowStart[J - 1], nr = first ? rowStart[J] - r0 : 0;
        const int64_t cnt = colStart[J] - colStart[J - 1];
        const double *t = tbuf + tBase[J - 1];
        for (int jj = 0; jj < kSmallGroup; ++jj) {
            double v = 0.0;
            if (jj < nj) {
                double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
                for (int64_t q = ln; q < nr; q += 32) v0 += rowPart[(r0 + q) * kSmallGroup + jj];
                const double *tj = t + (int64_t)jj * cnt;
                int64_t q = q0 + ln;
                for (; q + 96 < q1; q += 128) {
                    v0 += tj[q];
                    v1 += tj[q + 32];
                    v2 += tj[q + 64];
                    v3 += tj[q + 96];
                }
                for (; q < q1; q += 32) v1 += tj[q];
                v = (v0 + v1) + (v2 + v3);
            }
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (ln == 0) colPart[it * kSmallGroup + jj] = v;
        }
    }
}

// phase 2b, one thread per parameter: y = D x + the column items of its
// group in item order
__global__ void k_spmv_final(int32_t n, const int32_t *aig, const int32_t *p2g, const int64_t *colItemBeg,
                             const double *colPart, const double *matD, const double *x, double *y) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t J = p2g[j];
        const int32_t jj = (int32_t)j - (aig[J - 1] - 1);
        double r = matD[j] * x[j];
        for (int64_t it = colItemBeg[J - 1]; it < colItemBeg[J]; ++it) r += colPart[it * kSmallGroup + jj];
        y[j] = r;
    }
}

// ---------------------------------------------------------------- MINRES state
struct MinresState {
    double beta1, beta, oldb, alfa, dbar, epsln, oldeps, delta, gbar, root, gamma, cs, sn, phi, phibar;
    double tnorm2, gmax, gmin, Anorm, ynorm, rnorm, denom, rtol;
    double dotv;       // scratch result of the last dot
    int itn, itnlim, istop, done;
};

__global__ void k_mr_init(MinresState *S, double rtol, int itnlim) {
    if (threadIdx.x) return;
    // beta1 = sqrt(r1 . y) is in S->dotv
    double b1 = S->dotv;
    memset(S, 0, sizeof(MinresState));
    S->rtol = rtol;
    S->itnlim = itnlim;
    S->cs = -1.0;
    S->gmin = 1.0e300;
    if (b1 <= 0.0) { S->istop = b1 < 0.0 ? 9 : 0; S->done = 1; return; }
    b1 = sqrt(b1);
    S->beta1 = b1;
    S->beta = b1;
    S->phibar = b1;
}

__global__ void k_mr_scale_v(int32_t n, const MinresState *S, const double *y, double *v) {
    if (S->done) return;
    const double s = 1.0 / S->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = s * y[i];
}

__global__ void k_mr_y1(int32_t n, const MinresState *S, double *y, const double *r1) {
    if (S->done || S->itn < 1) return;   // itn counts completed iterations
    const double f = S->beta / S->oldb;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = y[i] - f * r1[i];
}

__global__ void k_mr_alfa(MinresState *S) {
    if (threadIdx.x || S->done) return;
    S->alfa = S->dotv;
}

__global__ void k_mr_y2(int32_t n, const MinresState *S, double *y, double *r1, double *r2, const double *cu) {
    if (S->done) return;
    const double f = S->alfa / S->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double yi = y[i] - f * r2[i];
        r1[i] = r2[i];
        r2[i] = yi;
        y[i] = (yi * cu[i]) * cu[i];
    }
}

__device__ void mr_rot_body(MinresState *S) {
    double b2 = S->dotv;
    if (b2 < 0.0) { S->istop = 9; S->done = 1; return; }
    S->oldb = S->beta;
    S->beta = sqrt(b2);
    S->tnorm2 += S->alfa * S->alfa + S->oldb * S->oldb + S->beta * S->beta;
    S->oldeps = S->epsln;
    S->delta = S->cs * S->dbar + S->sn * S->alfa;
    S->gbar = S->sn * S->dbar - S->cs * S->alfa;
    S->epsln = S->sn * S->beta;
    S->dbar = -S->cs * S->beta;
    S->root = sqrt(S->gbar * S->gbar + S->dbar * S->dbar);
    double gamma = sqrt(S->gbar * S->gbar + S->beta * S->beta);
    if (gamma < 2.220446049250313e-16) gamma = 2.220446049250313e-16;
    S->gamma = gamma;
    S->cs = S->gbar / gamma;
    S->sn = S->beta / gamma;
    S->phi = S->cs * S->phibar;
    S->phibar = S->sn * S->phibar;
    S->denom = 1.0 / gamma;
    S->gmax = fmax(S->gmax, gamma);
    S->gmin = fmin(S->gmin, gamma);
}

__global__ void k_mr_rot(MinresState *S) {
    if (threadIdx.x || S->done) return;
    mr_rot_body(S);
}

__global__ void k_mr_w(int32_t n, const MinresState *S, const double *v, double *w, double *w1, double *w2,
                       double *x) {
    if (S->done) return;
    const double oe = S->oldeps, de = S->delta, dn = S->denom, ph = S->phi;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = w2[i], b = w[i];
        w1[i] = a;
        w2[i] = b;
        const double wn = (v[i] - oe * a - de * b) * dn;
        w[i] = wn;
        x[i] = x[i] + ph * wn;
    }
}

__device__ void mr_test_body(MinresState *S) {
    S->itn += 1;
    S->Anorm = sqrt(S->tnorm2);
    S->ynorm = sqrt(S->dotv);
    S->rnorm = S->phibar;
    const double test1 = S->rnorm / (S->Anorm * S->ynorm);
    const double test2 = S->root / S->Anorm;
    const double Acond = S->gmax / S->gmin;
    int istop = 0;
    if (S->itn >= S->itnlim) istop = 6;
    if (Acond >= 0.1 / 2.220446049250313e-16) istop = 4;
    if (test2 <= S->rtol) istop = 2;
    if (test1 <= S->rtol) istop = 1;
    if (istop) { S->istop = istop; S->done = 1; }
}

__global__ void k_mr_test(MinresState *S) {
    if (threadIdx.x || S->done) return;
    mr_test_body(S);
}

// Fused forms of one MINRES iteration (diagonal or no preconditioner): each
// vector update also forms its dot product's partial sums with the grid and
// element order of k_dot_partial (kDotBlocks x kThreads, grid-stride), and
// each scalar step sums the partials as k_sum_final does, so the iterates
// are bit-identical to the unfused sequence with half the launches.
__global__ void k_mr_v_pad(int32_t nfit, int32_t n, const MinresState *S, const double *y, double *v, double *xa) {
    if (S->done) return;
    const double s = 1.0 / S->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double vi = 0.0;
        if (i < nfit) {
            vi = s * y[i];
            v[i] = vi;
        }
        xa[i] = vi;
    }
}

// y = ba - (beta / oldbeta) r1 (from the second iteration on), partials of v . y
__global__ void k_mr_y1_dot(int32_t n, const MinresState *S, const double *ba, double *y, const double *r1,
                            const double *v, double *part) {
    __shared__ double sh[kThreads];
    if (S->done) return;
    const bool upd = S->itn >= 1;
    const double f = upd ? S->beta / S->oldb : 0.0;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double yi = ba[i];
        if (upd) yi = yi - f * r1[i];
        y[i] = yi;
        acc += v[i] * yi;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// k_mr_y2, partials of r2 . y
__global__ void k_mr_y2_dot(int32_t n, const MinresState *S, double *y, double *r1, double *r2, const double *cu,
                            double *part) {
    __shared__ double sh[kThreads];
    if (S->done) return;
    const double f = S->alfa / S->beta;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double yi = y[i] - f * r2[i];
        r1[i] = r2[i];
        r2[i] = yi;
        const double zi = (yi * cu[i]) * cu[i];
        y[i] = zi;
        acc += yi * zi;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// k_mr_w, partials of x . x
__global__ void k_mr_w_dot(int32_t n, const MinresState *S, const double *v, double *w, double *w1, double *w2,
                           double *x, double *part) {
    __shared__ double sh[kThreads];
    if (S->done) return;
    const double oe = S->oldeps, de = S->delta, dn = S->denom, ph = S->phi;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = w2[i], b = w[i];
        w1[i] = a;
        w2[i] = b;
        const double wn = (v[i] - oe * a - de * b) * dn;
        w[i] = wn;
        const double xi = x[i] + ph * wn;
        x[i] = xi;
        acc += xi * xi;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// the partials summed as k_sum_final, then the scalar step: 0 alfa, 1 the
// rotation, 2 the convergence test
__global__ void k_mr_sum_step(const double *part, int np, MinresState *S, int step) {
    __shared__ double sh[kThreads];
    if (S->done) return;
    double acc = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc += part[i];
    acc = block_sum(acc, sh);
    if (threadIdx.x) return;
    S->dotv = acc;
    if (step == 0) S->alfa = acc;
    else if (step == 1) mr_rot_body(S);
    else mr_test_body(S);
}

// MINRES-QLP (Choi, Paige & Saunders 2011; minresqlpModule.f90:411-1333 in
// the reference): the Lanczos scalars of MinresState plus the rows of the
// lower-triangular L = R P not yet final, the final u values and the
// rotations of the current iteration for the vector kernel
struct QlpState {
    double etaA, thA, gA, tauA, etaB, thB, gB, tauB, uF1, uF2;
    double c1, s1, c2, s2, uA, uB, uC;
    int k, commit;
};

__device__ __forceinline__ void d_sym_ortho(double a, double b, double *c, double *s, double *r) {
    *r = sqrt(a * a + b * b);
    if (*r == 0.0) { *c = 1.0; *s = 0.0; return; }
    *c = a / *r;
    *s = b / *r;
}

__global__ void k_qlp_init(QlpState *Q) {
    if (threadIdx.x) return;
    memset(Q, 0, sizeof(QlpState));
}

// beta_{k+1}, the left reflection (column k of R, tau_k), the right
// reflections P(k-2,k), P(k-1,k) and u; the same arithmetic as the oracle
__global__ void k_qlp_rot(MinresState *S, QlpState *Q) {
    if (threadIdx.x || S->done) return;
    double b2 = S->dotv;
    if (b2 < 0.0) { S->istop = 9; S->done = 1; return; }
    const int k = S->itn + 1;
    Q->k = k;
    S->oldb = S->beta;
    S->beta = sqrt(b2);
    S->tnorm2 += S->alfa * S->alfa + S->oldb * S->oldb + S->beta * S->beta;
    S->Anorm = sqrt(S->tnorm2);
    const double epsk = S->epsln;
    const double delta = S->cs * S->dbar + S->sn * S->alfa;
    const double gbar = S->sn * S->dbar - S->cs * S->alfa;
    S->epsln = S->sn * S->beta;
    S->dbar = -S->cs * S->beta;
    S->root = sqrt(gbar * gbar + S->dbar * S->dbar);
    double cs, sn, gamma;
    d_sym_ortho(gbar, S->beta, &cs, &sn, &gamma);
    S->cs = cs;
    S->sn = sn;
    const double tau = cs * S->phibar;
    S->phibar = sn * S->phibar;
    S->gmax = fmax(S->gmax, gamma);
    S->gmin = fmin(S->gmin, gamma);
    double c1 = 1, s1 = 0, c2 = 1, s2 = 0, etaC = 0, thC = 0, gC, dk = delta, gk = gamma;
    if (k >= 3) {
        double r;
        d_sym_ortho(Q->gA, epsk, &c1, &s1, &r);
        Q->gA = r;
        const double th = c1 * Q->thB + s1 * dk;
        dk = s1 * Q->thB - c1 * dk;
        Q->thB = th;
        etaC = s1 * gk;
        gk = -c1 * gk;
    }
    if (k >= 2) {
        double r;
        d_sym_ortho(Q->gB, dk, &c2, &s2, &r);
        Q->gB = r;
        thC = s2 * gk;
        gC = -c2 * gk;
    } else {
        gC = gk;
    }
    const double tiny = 2.220446049250313e-16 * S->Anorm;
    double uA = 0.0, uB = 0.0, uC;
    if (k >= 3) uA = fabs(Q->gA) > tiny ? (Q->tauA - Q->etaA * Q->uF2 - Q->thA * Q->uF1) / Q->gA : 0.0;
    if (k >= 2) uB = fabs(Q->gB) > tiny ? (Q->tauB - Q->etaB * Q->uF1 - Q->thB * uA) / Q->gB : 0.0;
    uC = fabs(gC) > tiny ? (tau - etaC * uA - thC * uB) / gC : 0.0;
    Q->c1 = c1; Q->s1 = s1; Q->c2 = c2; Q->s2 = s2;
    Q->uA = uA; Q->uB = uB; Q->uC = uC;
    if (k >= 3) { Q->uF2 = Q->uF1; Q->uF1 = uA; }
    Q->etaA = Q->etaB; Q->thA = Q->thB; Q->gA = Q->gB; Q->tauA = Q->tauB;
    Q->etaB = etaC; Q->thB = thC; Q->gB = gC; Q->tauB = tau;
}

// W = V P (w_{k-2} final into xp) and the candidate iterate xc
__global__ void k_qlp_w(int32_t n, const MinresState *S, const QlpState *Q, const double *v, double *wa,
                        double *wb, double *xp, double *xc) {
    if (S->done) return;
    const int k = Q->k;
    const double c1 = Q->c1, s1 = Q->s1, c2 = Q->c2, s2 = Q->s2, uA = Q->uA, uB = Q->uB, uC = Q->uC;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = wa[i], bb = wb[i], c = v[i];
        if (k >= 3) {
            const double a2 = c1 * a + s1 * c;
            c = s1 * a - c1 * c;
            a = a2;
            xp[i] = xp[i] + uA * a;
        }
        if (k >= 2) {
            const double b2 = c2 * bb + s2 * c;
            c = s2 * bb - c2 * c;
            bb = b2;
        }
        wa[i] = bb;
        wb[i] = c;
        xc[i] = xp[i] + uB * bb + uC * c;
    }
}

__global__ void k_qlp_test(MinresState *S, QlpState *Q, double maxxnorm) {
    if (threadIdx.x || S->done) return;
    Q->commit = 0;
    const double xnorm = sqrt(S->dotv);
    if (xnorm > maxxnorm) { S->istop = 5; S->done = 1; S->itn += 1; return; }
    Q->commit = 1;
    S->itn += 1;
    S->ynorm = xnorm;
    S->rnorm = S->phibar;
    const double test1 = S->rnorm / (S->Anorm * xnorm);
    const double test2 = S->root / S->Anorm;
    const double Acond = S->gmax / S->gmin;
    int istop = 0;
    if (S->itn >= S->itnlim) istop = 6;
    if (Acond >= 0.1 / 2.220446049250313e-16) istop = 4;
    if (test2 <= S->rtol) istop = 2;
    if (test1 <= S->rtol) istop = 1;
    if (istop) { S->istop = istop; S->done = 1; }
}

__global__ void k_qlp_commit(int32_t n, const QlpState *Q, const double *xc, double *x) {
    if (!Q->commit) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = xc[i];
}

__global__ void k_copy_pad(int32_t n, int32_t ntot, const double *x, double *xa) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ntot; i += (int64_t)gridDim.x * blockDim.x)
        xa[i] = i < n ? x[i] : 0.0;
}

__global__ void k_copy_if(int32_t n, const MinresState *S, const double *a, double *b) {
    if (S && S->done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

__global__ void k_apply_precond(int32_t n, const double *r, const double *cu, double *y) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (r[i] * cu[i]) * cu[i];
}

__global__ void k_precond(int32_t n, const double *dg, double *cu) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        cu[i] = dg[i] > 0.0 ? 1.0 / sqrt(dg[i]) : 0.0;
}

__global__ void k_diag_update(int32_t n, double *dg, const double *v, const double *y, const double *betap) {
    const double beta = *betap;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dg[i] = dg[i] - 4.0 * v[i] * y[i] + 4.0 * beta * v[i] * v[i];
}

__global__ void k_sparse_diag(int32_t n, const double *matD, double *dg) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dg[i] = matD[i];
}

__global__ void k_fill(int32_t n, double v, double *a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

__global__ void k_sub(int32_t n, double *a, const double *b) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = a[i] - b[i];
}

// ---------------------------------------------------------------- helpers
struct Solver {
    mpgpu_ctx *c;
    DevJob &j;
    cudaStream_t s;
    int nsm;
    SparseBlocks sb;
    double *part = nullptr;
    explicit Solver(mpgpu_ctx *cc) : c(cc), j(cc->j), s(cc->stream) {
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    }
    ~Solver() {
        // part is stream-ordered (cudaMallocAsync on the context's stream)
        if (part) cudaFreeAsync(part, s);
        part = nullptr;
        dfree(wyPart); dfree(wyT);
        dfree(sb.rowStart); dfree(sb.bcol); dfree(sb.boff); dfree(sb.bld); dfree(sb.tOff);
        dfree(sb.colStart); dfree(sb.colBlk); dfree(sb.tBase); dfree(sb.tbuf); dfree(part);
        dfree(sb.tStr); dfree(sb.brow); dfree(sb.rowPart);
        dfree(sb.colItemJ); dfree(sb.colItemQ0); dfree(sb.colItemQ1); dfree(sb.colItemBeg); dfree(sb.colPart);
        dfree(pmvRow); dfree(pmvPart);
    }
    unsigned grid(int64_t n, int per = kThreads) const {
        int64_t g = (n + per - 1) / per;
        int64_t m = (int64_t)nsm * 8;
        if (g > m) g = m;
        return (unsigned)(g < 1 ? 1 : g);
    }
    unsigned wgrid(int64_t nwarp) const { return grid(nwarp * 32); }

    // packed symmetric product (two passes; buffers kept for the solve)
    double *pmvRow = nullptr, *pmvPart = nullptr;
    int64_t pmvN = 0;
    // scratch of the packed product; a failed allocation leaves none (the
    // product is then not launched and pmvFailed is set)
    cudaError_t alloc_pmv(int32_t n) {
        if (pmvN == n && pmvRow && pmvPart) return cudaSuccess;
        const int64_t nb = ((int64_t)n + kMvRows - 1) / kMvRows;
        dfree(pmvRow);
        dfree(pmvPart);
        pmvN = -1;
        cudaError_t e = cudaMalloc(&pmvRow, sizeof(double) * std::max<int64_t>(n, 1));
        if (e == cudaSuccess) e = cudaMalloc(&pmvPart, sizeof(double) * std::max<int64_t>(nb * n, 1));
        if (e != cudaSuccess) {
            dfree(pmvRow);
            dfree(pmvPart);
            pmvFailed = true;
            return e;
        }
        pmvN = n;
        return cudaSuccess;
    }
    bool pmvFailed = false;
    void packed_matvec(int32_t n, const double *A, const double *x, double *y) {
        const int64_t nb = ((int64_t)n + kMvRows - 1) / kMvRows;
        if (alloc_pmv(n) != cudaSuccess) return;
        k_pmv_blocks<<<(unsigned)nb, 256, 0, s>>>(n, A, x, pmvRow, pmvPart);
        k_pmv_final<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, nb, pmvRow, pmvPart, y);
    }

    // block table of the sparse storage, built from the host copies
    int32_t build_blocks() {
        std::vector<int64_t> off(2 * (j.nG + 1));
        std::vector<int32_t> col(std::max<int64_t>(j.ncolw, 1));
        cudaMemcpy(off.data(), j.off, sizeof(int64_t) * off.size(), cudaMemcpyDeviceToHost);
        if (j.ncolw > 0) cudaMemcpy(col.data(), j.col, sizeof(int32_t) * j.ncolw, cudaMemcpyDeviceToHost);
        const std::vector<int32_t> &aig = j.hAig;
        std::vector<int64_t> rowStart(1, 0), boff, tOff;
        std::vector<int32_t> bcol, bld;
        int64_t tl = 0;
        for (int32_t I = 1; I <= j.nG; ++I) {
            const int32_t np = aig[I] - aig[I - 1];
            const int64_t kk = off[2 * (I - 1)], ll = off[2 * (I - 1) + 1];
            const int64_t ku = off[2 * I] - kk;
            if (ku > 0) {
                if (col[kk] != 0) {  // uncompressed: one (np x ku) matrix
                    int64_t k = 0;
                    while (k < ku) {
                        const int32_t first = col[kk + k];
                        // group of this column
                        int32_t J = (int32_t)(std::upper_bound(aig.begin(), aig.end(), first) - aig.begin());
                        const int32_t nj = aig[J] - aig[J - 1];
                        bcol.push_back(J);
                        boff.push_back(ll + k);
                        bld.push_back((int32_t)ku);
                        tOff.push_back(J == I ? -1 : tl);
                        if (J != I) tl += nj;
                        k += nj;
                    }
                } else {  // compressed: regions (offset, first group) ... (end offset, n+1)
                    for (int64_t k = 2; k <= ku - 2; k += 2) {
                        const int32_t g0 = col[kk + k - 1];
                        const int32_t o0 = col[kk + k - 2];
                        const int32_t o1 = col[kk + k];
                        const int32_t width = o1 - o0;
                        int32_t inreg = 0, J = g0;
                        while (inreg < width) {
                            const int32_t nj = aig[J] - aig[J - 1];
                            bcol.push_back(J);
                            boff.push_back(ll + (int64_t)o0 * np + inreg);
                            bld.push_back(width);
                            tOff.push_back(J == I ? -1 : tl);
                            if (J != I) tl += nj;
                            inreg += nj;
                            J++;
                        }
                    }
                }
            }
            rowStart.push_back((int64_t)bcol.size());
        }
        // incoming (transposed) blocks per column group, ordered by row group
        const int64_t nb = (int64_t)bcol.size();
        std::vector<int64_t> cnt(j.nG + 2, 0);
        std::vector<int32_t> brow(nb);
        for (int32_t I = 1; I <= j.nG; ++I)
            for (int64_t b = rowStart[I - 1]; b < rowStart[I]; ++b) brow[b] = I;
        for (int64_t b = 0; b < nb; ++b)
            if (bcol[b] != brow[b]) cnt[bcol[b]]++;
        std::vector<int64_t> colStart(j.nG + 1, 0);
        for (int32_t J = 1; J <= j.nG; ++J) colStart[J] = colStart[J - 1] + cnt[J];
        std::vector<int64_t> fill(colStart.begin(), colStart.end() - 1), colBlk(std::max<int64_t>(colStart[j.nG], 1));
        for (int64_t b = 0; b < nb; ++b)
            if (bcol[b] != brow[b]) colBlk[fill[bcol[b] - 1]++] = b;
        int32_t maxnp = 0;
        for (int32_t I = 1; I <= j.nG; ++I) maxnp = std::max(maxnp, aig[I] - aig[I - 1]);
        sb.smallGroups = maxnp <= kSmallGroup && nb < (int64_t)0xffffffff;
        // transposed products stored by column group, incoming blocks in row
        // group order: block after block (general kernels) or parameter-major
        // with the group's block count as stride (small groups)
        std::vector<int64_t> tBase(std::max(j.nG, 1));
        std::vector<int32_t> tStr(std::max<int64_t>(nb, 1), 1);
        {
            int64_t off = 0;
            for (int32_t J = 1; J <= j.nG; ++J) {
                tBase[J - 1] = off;
                const int32_t nj = aig[J] - aig[J - 1];
                const int64_t cnt = colStart[J] - colStart[J - 1];
                for (int64_t q = colStart[J - 1]; q < colStart[J]; ++q) {
                    const int64_t r = q - colStart[J - 1];
                    tOff[colBlk[q]] = sb.smallGroups ? off + r : off + r * nj;
                    tStr[colBlk[q]] = (int32_t)cnt;
                }
                off += cnt * nj;
            }
        }
        std::vector<int32_t> ciJ;
        std::vector<int64_t> ciQ0, ciQ1, ciBeg(j.nG + 1, 0);
        for (int32_t J = 1; J <= j.nG; ++J) {
            ciBeg[J - 1] = (int64_t)ciJ.size();
            const int64_t cnt = colStart[J] - colStart[J - 1];
            int64_t q = 0;
            do {
                ciJ.push_back(J);
                ciQ0.push_back(q);
                ciQ1.push_back(std::min<int64_t>(cnt, q + kColItem));
                q += kColItem;
            } while (q < cnt);
        }
        ciBeg[j.nG] = (int64_t)ciJ.size();
        sb.nColItem = (int64_t)ciJ.size();
        int32_t minnp = maxnp;
        for (int32_t I = 1; I <= j.nG; ++I) minnp = std::min(minnp, aig[I] - aig[I - 1]);
        sb.uniform = (sb.smallGroups && minnp == maxnp) ? maxnp : 0;
        sb.nblk = nb;
        sb.tlen = tl;
        auto up = [&](auto *&d, const auto &h) -> cudaError_t {
            cudaError_t e = cudaMalloc((void **)&d, sizeof(h[0]) * std::max<size_t>(h.size(), 1));
            if (e != cudaSuccess) return e;
            return cudaMemcpy(d, h.data(), sizeof(h[0]) * h.size(), cudaMemcpyHostToDevice);
        };
        MPG_CUDA(c, up(sb.rowStart, rowStart));
        MPG_CUDA(c, up(sb.bcol, bcol));
        MPG_CUDA(c, up(sb.boff, boff));
        MPG_CUDA(c, up(sb.bld, bld));
        MPG_CUDA(c, up(sb.tOff, tOff));
        MPG_CUDA(c, up(sb.colStart, colStart));
        MPG_CUDA(c, up(sb.colBlk, colBlk));
        MPG_CUDA(c, up(sb.tBase, tBase));
        if (sb.smallGroups) {
            MPG_CUDA(c, up(sb.tStr, tStr));
            MPG_CUDA(c, up(sb.brow, brow));
            MPG_CUDA(c, cudaMalloc((void **)&sb.rowPart, sizeof(double) * std::max<int64_t>(nb, 1) * kSmallGroup));
            MPG_CUDA(c, up(sb.colItemJ, ciJ));
            MPG_CUDA(c, up(sb.colItemQ0, ciQ0));
            MPG_CUDA(c, up(sb.colItemQ1, ciQ1));
            MPG_CUDA(c, up(sb.colItemBeg, ciBeg));
            MPG_CUDA(c, cudaMalloc((void **)&sb.colPart, sizeof(double) * std::max<int64_t>(sb.nColItem, 1) * kSmallGroup));
        }
        MPG_CUDA(c, cudaMalloc((void **)&sb.tbuf, sizeof(double) * std::max<int64_t>(tl, 1)));
        return MPGPU_OK;
    }

    // y = A x (full parameter space)
    void avprd0(const double *x, double *y) {
        if (j.matsto == 2 && sb.smallGroups) {
            const unsigned gb = grid(sb.nblk);
#define MPG_SPMV_BLOCKS(G)                                                                                  \
    k_spmv_blocks<G><<<gb, kThreads, 0, s>>>(sb.nblk, sb.brow, j.aig, sb.bcol, sb.boff, sb.bld, sb.tOff, sb.tStr, \
                                             j.matD, x, sb.tbuf, sb.rowPart)
            switch (sb.uniform) {
            case 1: MPG_SPMV_BLOCKS(1); break;
            case 2: MPG_SPMV_BLOCKS(2); break;
            case 3: MPG_SPMV_BLOCKS(3); break;
            case 4: MPG_SPMV_BLOCKS(4); break;
            case 5: MPG_SPMV_BLOCKS(5); break;
            case 6: MPG_SPMV_BLOCKS(6); break;
            case 7: MPG_SPMV_BLOCKS(7); break;
            case 8: MPG_SPMV_BLOCKS(8); break;
            default: MPG_SPMV_BLOCKS(0); break;
            }
#undef MPG_SPMV_BLOCKS
            k_spmv_colitems<<<wgrid(sb.nColItem), kThreads, 0, s>>>(sb.nColItem, sb.colItemJ, sb.colItemQ0,
                                                                    sb.colItemQ1, j.aig, sb.rowStart, sb.rowPart,
                                                                    sb.colStart, sb.tBase, sb.tbuf, sb.colPart);
            k_spmv_final<<<grid(j.nVar), kThreads, 0, s>>>(j.nVar, j.aig, j.p2g, sb.colItemBeg, sb.colPart, j.matD,
                                                           x, y);
        } else if (j.matsto == 2) {
            k_spmv_rows<<<wgrid(j.nG), kThreads, 0, s>>>(j.nG, j.aig, sb.rowStart, sb.bcol, sb.boff, sb.bld,
                                                         sb.tOff, j.matD, x, y, sb.tbuf);
            k_spmv_cols<<<wgrid(j.nG), kThreads, 0, s>>>(j.nG, j.aig, sb.colStart, sb.colBlk, sb.tOff,
                                                         sb.tbuf, y);
        } else {
            packed_matvec(j.nVar, j.matD, x, y);
        }
    }
    // the reflections of qlssq in its order (k = m..1): v = v_k, yk =
    // P^T A P v_k with P = H_m ... H_{k+1}, *dsc = v.yk; apply() after each
    template <class Fn>
    void reflections(double *v, double *tmp, double *yk, double *dsc, Fn &&apply) {
        const int32_t n = j.nVar, ncon = j.ncon;
        for (int k = ncon; k >= 1; --k) {
            const int kn = n + k - ncon;
            const double *vr = j.qlV + (int64_t)(k - 1) * n;
            k_vec_with_kn<<<grid(n), kThreads, 0, s>>>(vr, j.hR2[k - 1], j.hVk[k - 1], kn, n, v);
            cudaMemcpyAsync(tmp, v, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
            if (k < ncon) k_qlapply<<<1, 1024, 0, s>>>(tmp, j.qlV, j.qlVk, j.qlR2, n, ncon, k + 1, ncon, 1);
            avprd0(tmp, yk);
            if (k < ncon) k_qlapply<<<1, 1024, 0, s>>>(yk, j.qlV, j.qlVk, j.qlR2, n, ncon, ncon, k + 1, -1);
            dot(v, yk, n, part, dsc, s);
            apply();
        }
    }
    // band of Q^T A Q (pede's preconditioner fill and qlpssq with band
    // width mbandw) and its lltdec factor with the block spikes
    int32_t band_build(BandPre &P, int32_t mbandw, int32_t lprecm, double *v, double *tmp, double *yk,
                       double *dsc) {
        const int32_t n = j.nVar, nfit = j.nVar - j.ncon;
        if (mbandw > MPGPU_BAND_MAX) return set_err(c, MPGPU_ERR_LIMIT, "band preconditioner wider than 32");
        if (band_alloc(P, n, nfit, mbandw - 1)) return set_err(c, MPGPU_ERR_ALLOC, "band preconditioner");
        MPG_CUDA(c, band_fill(P, n, j.matsto, j.matD, j.aig, j.p2g, sb.rowStart, sb.bcol, sb.boff, sb.bld, s));
        cudaError_t e = cudaSuccess;
        reflections(v, tmp, yk, dsc, [&] {
            if (e == cudaSuccess) e = band_reflect(P, n, v, yk, dsc, s);
        });
        MPG_CUDA(c, e);
        MPG_CUDA(c, band_factor(P, lprecm, s));
        return MPGPU_OK;
    }
    // qlmlq (mpqldec.f90:404-454): t = 1 Q^T x (reflections ncon..1), t = 0
    // Q x (1..ncon), in the compact WY form
    double *wyPart = nullptr, *wyT = nullptr;
    void qlmlq(double *x, int t) {
        if (j.ncon <= 0) return;
        const int32_t m = j.ncon, n = j.nVar;
        if (!wyPart && m <= 4096) {
            if (cudaMalloc(&wyPart, sizeof(double) * (size_t)kWyBlocks * m) != cudaSuccess ||
                cudaMalloc(&wyT, sizeof(double) * m) != cudaSuccess) {
                dfree(wyPart);
                dfree(wyT);
                cudaGetLastError();
            }
        }
        // coefficients beyond the shared memory of one CTA, or no workspace:
        // the reflections one after the other in one CTA
        if (m > 4096 || !wyPart || !wyT) {
            if (t) k_qlapply<<<1, 1024, 0, s>>>(x, j.qlV, j.qlVk, j.qlR2, n, m, m, 1, -1);
            else k_qlapply<<<1, 1024, 0, s>>>(x, j.qlV, j.qlVk, j.qlR2, n, m, 1, m, 1);
            return;
        }
        const int nb = (int)std::min<int64_t>(kWyBlocks, std::max<int64_t>(1, n / 512));
        k_wy_dots<<<nb, 256, 0, s>>>(n, m, j.qlV, x, wyPart);
        k_wy_coef<<<1, 256, sizeof(double) * m, s>>>(n, m, nb, wyPart, j.qlVk, j.qlT, x, t ? 0 : 1, wyT);
        k_wy_apply<<<grid(n), kThreads, sizeof(double) * m, s>>>(n, m, j.qlV, j.qlVk, wyT, x);
    }
};

}  // namespace

// ---------------------------------------------------------------- inversion / Cholesky
// minver / mchdec (pede.f90:7838-8054) on the packed matrix
int32_t solve_inversion(mpgpu_ctx *c, const double *consResiduals, double *corrOut, double *errs,
                        mpgpu_solveinfo *info, bool decomposition, int dense, double rtol, int32_t itnlim) {
    Solver S(c);
    DevJob &j = c->j;
    cudaStream_t s = c->stream;
    const int32_t n = j.nVar, ncon = j.ncon, nfit = n - ncon;
    if (j.matsto != 2 && ncon > 0) MPG_CUDA(c, S.alloc_pmv(n));   // the packed products of qlssq
    // per-solve vectors from the stream-ordered pool: a cudaFree would wait
    // for the whole device, i.e. for the other jobs' work in a served mix
    struct Tmp {
        cudaStream_t s;
        double *corr = nullptr, *vbuf = nullptr, *Av = nullptr, *vk = nullptr, *diag = nullptr, *yv = nullptr;
        int32_t *used = nullptr, *piv = nullptr;
        ~Tmp() {
            for (void *p : {(void *)corr, (void *)vbuf, (void *)Av, (void *)vk, (void *)diag, (void *)yv,
                            (void *)used, (void *)piv})
                if (p) cudaFreeAsync(p, s);
        }
    } T{s};
    double *&corr = T.corr, *&vbuf = T.vbuf, *&Av = T.Av, *&vk = T.vk, *&diag = T.diag, *&yv = T.yv;
    int32_t *&used = T.used, *&piv = T.piv;
    MPG_CUDA(c, cudaMallocAsync(&corr, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMallocAsync(&vbuf, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMallocAsync(&Av, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMallocAsync(&vk, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMallocAsync(&diag, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMallocAsync(&yv, sizeof(double) * (ncon + 1), s));
    MPG_CUDA(c, cudaMallocAsync(&used, sizeof(int32_t) * n, s));
    MPG_CUDA(c, cudaMallocAsync(&piv, sizeof(int32_t) * 4, s));
    MPG_CUDA(c, cudaMallocAsync(&S.part, sizeof(double) * (kDotBlocks + 8), s));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    MPG_CUDA(c, cudaMemcpyAsync(corr, j.gvec, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    double *scal = c->scal + 300;   // device scalars
    // Q^T A Q (qlssq, reflections k = ncon .. 1)
    auto qlssq = [&](int t) {
        for (int jj = 1; jj <= ncon; ++jj) {
            const int k = t ? ncon + 1 - jj : jj;
            const int kn = n + k - ncon;
            const int ilast = j.hR2[k - 1];
            const double vkv = j.hVk[k - 1];
            const double *v = j.qlV + (int64_t)(k - 1) * n;
            k_vec_with_kn<<<S.grid(n), kThreads, 0, s>>>(v, ilast, vkv, kn, n, vbuf);
            S.avprd0(vbuf, Av);
            dot(vbuf, Av, n, S.part, scal, s);   // vtAv
            k_qlssq_update<<<S.wgrid(n), kThreads, 0, s>>>(n, j.matD, v, vkv, Av, scal, ilast, kn);
        }
    };
    // tensor-core forms with up to 128 constraints: Q^T A Q is formed inside
    // the dense solve for the preconditioner only (compact WY, 3xTF32) and
    // the refinement applies Q in FP64; no FP64 sweep of the matrix here
    const bool wyElim = dense == 1 && ncon >= 1 && ncon <= 128;
    std::vector<double> y(ncon > 0 ? ncon : 1, 0.0);
    if (ncon > 0) {
        if (!wyElim) qlssq(1);
        // qlbsub (mpqldec.f90:991-1014) on the host
        for (int k = ncon; k >= 1; --k) {
            double d = 0.0;
            for (int cc = 1; cc <= ncon - k; ++cc) d = d + j.hL[(size_t)(k - 1) * ncon + k - 1 + cc] * y[k - 1 + cc];
            y[k - 1] = ((consResiduals ? consResiduals[k - 1] : 0.0) - d) / j.hL[(size_t)(k - 1) * ncon + k - 1];
        }
        MPG_CUDA(c, cudaMemcpyAsync(yv, y.data(), sizeof(double) * ncon, cudaMemcpyHostToDevice, s));
        if (!wyElim) {
            S.qlmlq(corr, 1);
            k_cons_rhs<<<S.grid(nfit), kThreads, 0, s>>>(nfit, ncon, j.matD, yv, corr);
        }
    }
    if (S.pmvFailed) return set_err(c, MPGPU_ERR_ALLOC, "packed product scratch");
    int nrank = 0;
    if (!decomposition && dense < 0) {
        // sqminl (mpnum.f90:230-355) on the leading nfit x nfit block
        k_diag_abs<<<S.grid(nfit), kThreads, 0, s>>>(nfit, j.matD, diag);
        MPG_CUDA(c, cudaMemsetAsync(used, 0, sizeof(int32_t) * nfit, s));
        MPG_CUDA(c, cudaMemsetAsync(piv, 0, sizeof(int32_t) * 4, s));
        for (int i = 0; i < nfit; ++i) {
            k_sqminl_pivot<<<1, 1024, 0, s>>>(nfit, j.matD, corr, diag, used, vk, scal + 8, piv);
            k_sqminl_elim<<<S.wgrid(nfit), kThreads, 0, s>>>(nfit, j.matD, corr, vk, scal + 8, piv);
        }
        k_sqminl_deficit<<<S.grid(nfit, 1), kThreads, 0, s>>>(nfit, j.matD, corr, used, piv);
        k_negate<<<S.grid((int64_t)nfit * (nfit + 1) / 2), kThreads, 0, s>>>((int64_t)nfit * (nfit + 1) / 2, j.matD);
        std::vector<int32_t> hu(nfit);
        MPG_CUDA(c, cudaMemcpyAsync(hu.data(), used, sizeof(int32_t) * nfit, cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        for (int32_t u : hu) nrank += u;
    } else if (dense >= 0) {
        // blocked dense Cholesky (FP64, or tensor-core 3xTF32) refined by
        // preconditioned CG in FP64
        // (inversion forms: the inverse from the same factor replaces the
        // leading block of the packed matrix, where sqminl leaves it)
        const double tol = rtol > 0.0 ? rtol : 1e-13;
        const DenseWyElim wye{ncon, j.qlV, j.qlVk, j.qlT, yv};
        const int32_t rcd = wyElim ? dense_solve_pcg(c, n, j.matD, corr, dense, tol, itnlim > 0 ? itnlim : 2000,
                                                     info, decomposition ? nullptr : j.matD, &wye)
                                   : dense_solve_pcg(c, nfit, j.matD, corr, dense, tol, itnlim > 0 ? itnlim : 2000,
                                                     info, decomposition ? nullptr : j.matD);
        if (rcd != MPGPU_OK) return rcd;
        nrank = info->nrank;
    } else {
        // chdec2 + chslv2 (mpnum.f90:891-987)
        MPG_CUDA(c, cudaMemsetAsync(scal + 16, 0, sizeof(double) * 3, s));
        for (int64_t i = nfit; i >= 1; --i) {
            k_chdec_pivot<<<1, 32, 0, s>>>(i, j.matD, scal + 16);
            if (i > 1) {
                k_chdec_update<<<S.wgrid(i - 1), kThreads, 0, s>>>(i, j.matD);
                k_chdec_scale<<<S.grid(i - 1), kThreads, 0, s>>>(i, j.matD);
            }
        }
        k_chslv2<<<1, 1024, 0, s>>>(j.matD, corr, nfit);
        double st[3];
        MPG_CUDA(c, cudaMemcpyAsync(st, scal + 16, sizeof(double) * 3, cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        info->evmax = st[0];
        info->evmin = st[1];
        nrank = (int)st[2];
    }
    info->nrank = nrank;
    if (ncon > 0 && !wyElim) {   // (the WY form returns the full correction)
        MPG_CUDA(c, cudaMemcpyAsync(corr + nfit, yv, sizeof(double) * ncon, cudaMemcpyDeviceToDevice, s));
        S.qlmlq(corr, 0);
    }
    if (!decomposition && errs) {
        // covariance Q A^-1 Q^T with the constraint rows zeroed (xloopn,
        // pede.f90:9094-9121); its diagonal gives the parameter errors
        if (ncon > 0) {
            k_zero_rows<<<S.grid(ncon, 1), kThreads, 0, s>>>(nfit, n, j.matD);
            qlssq(0);
        }
        k_get_diag<<<S.grid(n), kThreads, 0, s>>>(n, j.matD, diag);
        MPG_CUDA(c, cudaMemcpyAsync(errs, diag, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    }
    MPG_CUDA(c, cudaMemcpyAsync(corrOut, corr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    cudaEventRecord(e1, s);
    MPG_CUDA(c, cudaStreamSynchronize(s));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    info->ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return MPGPU_OK;
}

// ---------------------------------------------------------------- MINRES
// mminrs (pede.f90:8243-8333) with the diagonal preconditioner of the
// QL-reduced matrix and MINRES (Paige & Saunders 1975) kept on the device;
// with qlp, MINRES-QLP on the same Lanczos process (mminrsqlp, the method's
// QLP steps from the first iteration, maxxnorm = nfit / sqrt(eps) as
// pede.f90:626 sets it).
int32_t solve_minres(mpgpu_ctx *c, const double *consResiduals, double rtol, int32_t itnlim,
                     double *corrOut, mpgpu_solveinfo *info, bool qlp) {
    Solver S(c);
    DevJob &j = c->j;
    cudaStream_t s = c->stream;
    const int32_t n = j.nVar, ncon = j.ncon, nfit = n - ncon;
    if (j.matsto == 2) {
        int32_t rc = S.build_blocks();
        if (rc) return rc;
    } else {
        MPG_CUDA(c, S.alloc_pmv(n));
    }
    MPG_CUDA(c, cudaMallocAsync(&S.part, sizeof(double) * (kDotBlocks + 8), s));
    // workspace released on every return
    struct Scratch {
        std::vector<double *> bufs;
        MinresState *St = nullptr;
        QlpState *Qs = nullptr;
        cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
        ~Scratch() {
            for (double *p : bufs) cudaFree(p);
            if (St) cudaFree(St);
            if (Qs) cudaFree(Qs);
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
        }
    } W;
    auto vec = [&](int64_t len) -> double * {
        double *p = nullptr;
        if (cudaMalloc(&p, sizeof(double) * std::max<int64_t>(len, 1)) != cudaSuccess) return nullptr;
        W.bufs.push_back(p);
        return p;
    };
    double *rhs = vec(n), *xa = vec(n), *ba = vec(n), *dg = vec(n), *cu = vec(n), *tmp = vec(n), *yk = vec(n);
    double *r1 = vec(n), *r2 = vec(n), *y = vec(n), *v = vec(n), *w = vec(n), *w1 = vec(n), *w2 = vec(n);
    double *x = vec(n);
    double *wa = nullptr, *wb = nullptr, *xp = nullptr, *xc = nullptr;
    if (qlp) { wa = vec(n); wb = vec(n); xp = vec(n); xc = vec(n); }
    MinresState *&St = W.St;
    QlpState *&Qs = W.Qs;
    MPG_CUDA(c, cudaMalloc(&St, sizeof(MinresState)));
    if (qlp) MPG_CUDA(c, cudaMalloc(&Qs, sizeof(QlpState)));
    for (double *p : W.bufs)
        if (!p) return set_err(c, MPGPU_ERR_ALLOC, "MINRES workspace");
    cudaEvent_t &e0 = W.ev[0], &e1 = W.ev[1], &ep = W.ev[2];
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    MPG_CUDA(c, cudaMemcpyAsync(rhs, j.gvec, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    std::vector<double> yc(ncon > 0 ? ncon : 1, 0.0);
    double *dsc = c->scal + 300;
    if (ncon > 0) {
        for (int k = ncon; k >= 1; --k) {
            double d = 0.0;
            for (int cc = 1; cc <= ncon - k; ++cc) d = d + j.hL[(size_t)(k - 1) * ncon + k - 1 + cc] * yc[k - 1 + cc];
            yc[k - 1] = ((consResiduals ? consResiduals[k - 1] : 0.0) - d) / j.hL[(size_t)(k - 1) * ncon + k - 1];
        }
        // rhs - A Q [0; y], then Q^T
        MPG_CUDA(c, cudaMemsetAsync(xa, 0, sizeof(double) * n, s));
        MPG_CUDA(c, cudaMemcpyAsync(xa + nfit, yc.data(), sizeof(double) * ncon, cudaMemcpyHostToDevice, s));
        S.qlmlq(xa, 0);
        S.avprd0(xa, ba);
        k_sub<<<S.grid(n), kThreads, 0, s>>>(n, rhs, ba);
        S.qlmlq(rhs, 1);
    }
    // preconditioner (pede.f90:8292-8316 by mbandw): < 0 none (M = I), 0
    // the diagonal of Q^T A Q (the band-width-1 case of qlpssq,
    // mpqldec.f90:711-950: dg -= 4 v y - 4 (v.y) v^2 per reflection), > 0
    // the variable-band Cholesky factor of its band (equdecs/equslvs)
    const int32_t mbandw = c->mbandw;
    BandPre P;
    struct BandGuard { BandPre &p; ~BandGuard() { band_free(p); } } bandGuard{P};
    cudaEventCreate(&ep);
    if (mbandw == 0) {
        if (j.matsto == 2) k_sparse_diag<<<S.grid(n), kThreads, 0, s>>>(n, j.matD, dg);
        else k_get_diag<<<S.grid(n), kThreads, 0, s>>>(n, j.matD, dg);
        S.reflections(v, tmp, yk, dsc, [&] { k_diag_update<<<S.grid(n), kThreads, 0, s>>>(n, dg, v, yk, dsc); });
        k_precond<<<S.grid(nfit), kThreads, 0, s>>>(nfit, dg, cu);
    } else {
        k_fill<<<S.grid(nfit), kThreads, 0, s>>>(nfit, 1.0, cu);
        if (mbandw > 0) {
            int32_t rc = S.band_build(P, mbandw, c->lprecm, v, tmp, yk, dsc);
            if (rc) return rc;
        }
    }
    cudaEventRecord(ep, s);
    const int *doneFlag = &St->done;
    // MINRES state: x = 0, r1 = r2 = b, y = M^-1 r1, beta1 = sqrt(r1.y)
    MPG_CUDA(c, cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMemsetAsync(w, 0, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMemsetAsync(w1, 0, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMemsetAsync(w2, 0, sizeof(double) * n, s));
    MPG_CUDA(c, cudaMemcpyAsync(r1, rhs, sizeof(double) * nfit, cudaMemcpyDeviceToDevice, s));
    MPG_CUDA(c, cudaMemcpyAsync(r2, rhs, sizeof(double) * nfit, cudaMemcpyDeviceToDevice, s));
    k_apply_precond<<<S.grid(nfit), kThreads, 0, s>>>(nfit, r1, cu, y);
    if (mbandw > 0) MPG_CUDA(c, band_solve(P, nullptr, y, s));
    dot(r1, y, nfit, S.part, &St->dotv, s);
    k_mr_init<<<1, 32, 0, s>>>(St, rtol, itnlim);
    const double maxxnorm = (double)nfit / sqrt(2.220446049250313e-16);
    if (qlp) {
        k_qlp_init<<<1, 32, 0, s>>>(Qs);
        MPG_CUDA(c, cudaMemsetAsync(wa, 0, sizeof(double) * n, s));
        MPG_CUDA(c, cudaMemsetAsync(wb, 0, sizeof(double) * n, s));
        MPG_CUDA(c, cudaMemsetAsync(xp, 0, sizeof(double) * n, s));
    }
    MinresState hs;
    int it = 0;
    const int batch = 16;
    // the iterations of one batch are recorded once as a CUDA graph and
    // replayed (all scalars live on the device); direct launches if the
    // capture is refused
    const bool fused = !qlp && mbandw <= 0;
    auto batchBody = [&] {
        for (int q = 0; q < batch; ++q) {
            if (fused) {
                k_mr_v_pad<<<S.grid(n), kThreads, 0, s>>>(nfit, n, St, y, v, xa);
                S.qlmlq(xa, 0);
                S.avprd0(xa, ba);
                S.qlmlq(ba, 1);
                k_mr_y1_dot<<<kDotBlocks, kThreads, 0, s>>>(nfit, St, ba, y, r1, v, S.part);
                k_mr_sum_step<<<1, kThreads, 0, s>>>(S.part, kDotBlocks, St, 0);
                k_mr_y2_dot<<<kDotBlocks, kThreads, 0, s>>>(nfit, St, y, r1, r2, cu, S.part);
                k_mr_sum_step<<<1, kThreads, 0, s>>>(S.part, kDotBlocks, St, 1);
                k_mr_w_dot<<<kDotBlocks, kThreads, 0, s>>>(nfit, St, v, w, w1, w2, x, S.part);
                k_mr_sum_step<<<1, kThreads, 0, s>>>(S.part, kDotBlocks, St, 2);
                continue;
            }
            k_mr_scale_v<<<S.grid(nfit), kThreads, 0, s>>>(nfit, St, y, v);
            // y = (Q^T A Q v)(1:nfit)
            k_copy_pad<<<S.grid(n), kThreads, 0, s>>>(nfit, n, v, xa);
            S.qlmlq(xa, 0);
            S.avprd0(xa, ba);
            S.qlmlq(ba, 1);
            k_copy_if<<<S.grid(nfit), kThreads, 0, s>>>(nfit, St, ba, y);
            k_mr_y1<<<S.grid(nfit), kThreads, 0, s>>>(nfit, St, y, r1);
            dot(v, y, nfit, S.part, &St->dotv, s);
            k_mr_alfa<<<1, 32, 0, s>>>(St);
            k_mr_y2<<<S.grid(nfit), kThreads, 0, s>>>(nfit, St, y, r1, r2, cu);
            if (mbandw > 0) band_solve(P, doneFlag, y, s);
            dot(r2, y, nfit, S.part, &St->dotv, s);
            if (!qlp) {
                k_mr_rot<<<1, 32, 0, s>>>(St);
                k_mr_w<<<S.grid(nfit), kThreads, 0, s>>>(nfit, St, v, w, w1, w2, x);
                dot(x, x, nfit, S.part, &St->dotv, s);
                k_mr_test<<<1, 32, 0, s>>>(St);
            } else {
                k_qlp_rot<<<1, 32, 0, s>>>(St, Qs);
                k_qlp_w<<<S.grid(nfit), kThreads, 0, s>>>(nfit, St, Qs, v, wa, wb, xp, xc);
                dot(xc, xc, nfit, S.part, &St->dotv, s);
                k_qlp_test<<<1, 32, 0, s>>>(St, Qs, maxxnorm);
                k_qlp_commit<<<S.grid(nfit), kThreads, 0, s>>>(nfit, Qs, xc, x);
            }
        }
    };
    if (j.matsto != 2) MPG_CUDA(c, S.alloc_pmv(n));  // no allocation while the graph is recorded
    struct GraphGuard {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t e = nullptr;
        ~GraphGuard() {
            if (e) cudaGraphExecDestroy(e);
            if (g) cudaGraphDestroy(g);
        }
    } gg;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        batchBody();
        if (cudaStreamEndCapture(s, &gg.g) != cudaSuccess || cudaGraphInstantiate(&gg.e, gg.g, 0) != cudaSuccess)
            gg.e = nullptr;
        cudaGetLastError();
    }
    for (;;) {
        if (gg.e) MPG_CUDA(c, cudaGraphLaunch(gg.e, s));
        else batchBody();
        it += batch;
        MPG_CUDA(c, cudaMemcpyAsync(&hs, St, sizeof(MinresState), cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        if (hs.done || it > itnlim + batch) break;
    }
    info->itn = hs.itn;
    info->istop = hs.istop;
    if (ncon > 0) {
        MPG_CUDA(c, cudaMemcpyAsync(x + nfit, yc.data(), sizeof(double) * ncon, cudaMemcpyHostToDevice, s));
        S.qlmlq(x, 0);
    }
    MPG_CUDA(c, cudaMemcpyAsync(corrOut, x, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    cudaEventRecord(e1, s);
    MPG_CUDA(c, cudaStreamSynchronize(s));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    info->ms = ms;
    cudaEventElapsedTime(&ms, e0, ep);
    info->msFactor = ms;
    if (mbandw > 0) cudaMemcpy(&info->nrkd, P.nrkd, sizeof(int32_t), cudaMemcpyDeviceToHost);
    return MPGPU_OK;
}

int32_t avprod_host(mpgpu_ctx *c, int32_t n, const double *x, double *b) {
    Solver S(c);
    DevJob &j = c->j;
    cudaStream_t s = c->stream;
    if (j.matsto == 2) {
        int32_t rc = S.build_blocks();
        if (rc) return rc;
    } else {
        MPG_CUDA(c, S.alloc_pmv(j.nVar));
    }
    double *xa = nullptr, *ba = nullptr;
    MPG_CUDA(c, cudaMalloc(&xa, sizeof(double) * j.nVar));
    MPG_CUDA(c, cudaMalloc(&ba, sizeof(double) * j.nVar));
    MPG_CUDA(c, cudaMemsetAsync(xa, 0, sizeof(double) * j.nVar, s));
    MPG_CUDA(c, cudaMemcpyAsync(xa, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    S.qlmlq(xa, 0);
    S.avprd0(xa, ba);
    S.qlmlq(ba, 1);
    MPG_CUDA(c, cudaMemcpyAsync(b, ba, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    cudaFree(xa);
    cudaFree(ba);
    return MPGPU_OK;
}

// the band preconditioner alone (equdecs on pede's matPreCond): band of
// Q^T A Q and its lltdec factor, returned in the variable-band layout of
// indPreCond (pede.f90:7705-7717) for the nfit rows
int32_t band_precond_factor(mpgpu_ctx *c, int32_t mbandw, int32_t lprecm, double *cOut, int32_t *nrkd) {
    Solver S(c);
    DevJob &j = c->j;
    cudaStream_t s = c->stream;
    const int32_t n = j.nVar, nfit = n - j.ncon;
    if (mbandw <= 0) return set_err(c, MPGPU_ERR_ARG, "band width must be positive");
    if (j.matsto == 2) {
        int32_t rc = S.build_blocks();
        if (rc) return rc;
    } else {
        MPG_CUDA(c, S.alloc_pmv(n));
    }
    MPG_CUDA(c, cudaMallocAsync(&S.part, sizeof(double) * (kDotBlocks + 8), s));
    struct Bufs {
        double *v = nullptr, *tmp = nullptr, *yk = nullptr;
        BandPre P;
        ~Bufs() {
            cudaFree(v); cudaFree(tmp); cudaFree(yk);
            band_free(P);
        }
    } bb;
    double *&v = bb.v, *&tmp = bb.tmp, *&yk = bb.yk;
    MPG_CUDA(c, cudaMalloc(&v, sizeof(double) * std::max(n, 1)));
    MPG_CUDA(c, cudaMalloc(&tmp, sizeof(double) * std::max(n, 1)));
    MPG_CUDA(c, cudaMalloc(&yk, sizeof(double) * std::max(n, 1)));
    BandPre &P = bb.P;
    int32_t rc = S.band_build(P, mbandw, lprecm, v, tmp, yk, c->scal + 300);
    if (!rc) {
        const int W1 = P.w + 1;
        std::vector<double> F((size_t)std::max(nfit, 1) * W1);
        cudaMemcpyAsync(F.data(), P.F, sizeof(double) * F.size(), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(nrkd, P.nrkd, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = cuda_err(c, cudaGetLastError(), "band factor");
        int64_t pos = 0;  // india(i) - i + j, 0-based running position
        for (int32_t i = 0; !rc && i < nfit; ++i)
            for (int32_t t = std::max(0, P.w - i); t <= P.w; ++t) cOut[pos++] = F[(size_t)i * W1 + t];
    }
    return rc;
}
