// mpgpu_fit.cu -- per-record local fit and Schur-complement update.
//
// One warp per record (records of one chunk distributed grid-stride).  The
// record words, its measurement table and slot lists are staged in shared
// memory; all decision-relevant arithmetic (global-parameter subtraction,
// normal equations, Gauss-Jordan inversion, residuals, chi2 sums, down-
// weighting, cuts) keeps the operation order of pede's loopbf
// (pede.f90:3387-4442) and this file is compiled with -fmad=false, so the
// accept/reject decision of every record is bit-identical to the reference
// arithmetic.  The update  -Gt W G + B Gamma^-1 Bt  is then formed with
// fused multiply-adds and written to the chunk staging buffer (packed over
// the record's sorted variable parameters) for the deterministic owner-
// computes accumulation (mpgpu_accum.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <math.h>

#include "mpgpu_ctx.h"

namespace {

constexpr double kChuber = 1.345;   // Huber constant (pede.f90:3515)
constexpr double kCauchy = 2.3849;  // Cauchy constant (pede.f90:3516)

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// chindl (mpnum.f90:2078-2115), single precision
__device__ float d_chindl(int n, int nd) {
    const float sn[3] = {0.47523f, 1.690140f, 2.782170f};
    const float t3[30] = {9.0000f, 5.9146f, 4.7184f, 4.0628f, 3.6410f, 3.3436f, 3.1209f,
                          2.9468f, 2.8063f, 2.6902f, 2.5922f, 2.5082f, 2.4352f, 2.3711f,
                          2.3143f, 2.2635f, 2.2178f, 2.1764f, 2.1386f, 2.1040f, 2.0722f,
                          2.0428f, 2.0155f, 1.9901f, 1.9665f, 1.9443f, 1.9235f, 1.9040f,
                          1.8855f, 1.8681f};
    const float t2[30] = {4.0000f, 3.0900f, 2.6750f, 2.4290f, 2.2628f, 2.1415f, 2.0481f,
                          1.9736f, 1.9124f, 1.8610f, 1.8171f, 1.7791f, 1.7457f, 1.7161f,
                          1.6897f, 1.6658f, 1.6442f, 1.6246f, 1.6065f, 1.5899f, 1.5745f,
                          1.5603f, 1.5470f, 1.5346f, 1.5230f, 1.5120f, 1.5017f, 1.4920f,
                          1.4829f, 1.4742f};
    const float t1[30] = {1.0000f, 1.1479f, 1.1753f, 1.1798f, 1.1775f, 1.1730f, 1.1680f,
                          1.1630f, 1.1581f, 1.1536f, 1.1493f, 1.1454f, 1.1417f, 1.1383f,
                          1.1351f, 1.1321f, 1.1293f, 1.1266f, 1.1242f, 1.1218f, 1.1196f,
                          1.1175f, 1.1155f, 1.1136f, 1.1119f, 1.1101f, 1.1085f, 1.1070f,
                          1.1055f, 1.1040f};
    if (nd < 1) return 0.0f;
    int m = n < 3 ? n : 3;
    if (m < 1) m = 1;
    if (nd <= 30) return m == 3 ? t3[nd - 1] : (m == 2 ? t2[nd - 1] : t1[nd - 1]);
    float x = sn[m - 1] + sqrtf((float)(nd + nd - 1));
    return (x * x) / (float)(nd + nd);
}

// ------------------------------------------------------------------------
// Gauss-Jordan inversion with diagonal pivoting (sqminv, mpnum.f90:97-213),
// warp-parallel over the packed elements.  v, b, diag 0-based; used[] flags.
// The pivot is the first remaining index with the largest |v_jj| among
// those above 16*eps*|original diagonal|, which is what the sequential
// linked-list scan of the reference selects.
// The comparisons of the pivot search run on the bit patterns: for
// non-negative doubles that are not NaN the unsigned order of the bits is
// the numeric order, so the search (and its warp argmax) needs no FP64
// instruction; a NaN on either side never passes, as in the FP64 compare.
// diag[] holds the bits of the thresholds 16 eps |v_jj| of the original
// diagonal.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

__device__ void warp_sqminv(double *v, double *b, int n, int *nrank_out, double *diag,
                            double *ocol, double *scol, int *used) {
    const int ln = lane_id();
    const double eps = 16.0 * 2.220446049250313e-16;
    constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;
    const int np = (n * n + n) / 2;
    unsigned long long *thr = reinterpret_cast<unsigned long long *>(diag);
    for (int i = ln; i < n; i += 32) {
        thr[i] = abs_bits(eps * fabs(v[(i + 1) * (i + 2) / 2 - 1]));
        used[i] = 0;
    }
    __syncwarp();
    int nrank = 0;
    bool deficient = false;
    for (int it = 0; it < n; ++it) {
        // pivot search: per lane best candidate, then warp argmax (ties -> low index)
        unsigned long long best = 0;
        int bk = -1;
        for (int j = ln; j < n; j += 32) {
            if (used[j]) continue;
            const unsigned long long a = abs_bits(v[(j + 1) * (j + 2) / 2 - 1]), t = thr[j];
            if (a <= kInfBits && t <= kInfBits && a > t && (bk < 0 || a > best)) { best = a; bk = j; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
            if (ok >= 0 && (bk < 0 || ob > best || (ob == best && ok < bk))) { best = ob; bk = ok; }
        }
        if (bk < 0) { deficient = true; break; }
        const int k = bk;              // 0-based pivot
        const int kk = (k + 1) * (k + 2) / 2 - 1;
        const double vkk = 1.0 / v[kk];
        // stage the pivot column (original) and its scaled copy
        for (int j = ln; j < n; j += 32) {
            if (j == k) continue;
            int jk = j > k ? (j * (j + 1)) / 2 + k : (k * (k + 1)) / 2 + j;
            double o = v[jk];
            ocol[j] = o;
            scol[j] = vkk * o;
        }
        __syncwarp();
        if (ln == 0) {
            used[k] = 1;
        }
        const double bk_new = b[k] * vkk;
        // elimination of every element not in row/column k
        {
            int r = 0, c = ln;
            while (c > r) { c -= r + 1; r++; }
            for (int idx = ln; idx < np; idx += 32) {
                if (r != k && c != k) v[idx] = v[idx] - scol[c] * ocol[r];
                c += 32;
                while (c > r) { c -= r + 1; r++; }
            }
        }
        for (int j = ln; j < n; j += 32) {
            if (j == k) continue;
            b[j] = b[j] - bk_new * ocol[j];
            int jk = j > k ? (j * (j + 1)) / 2 + k : (k * (k + 1)) / 2 + j;
            v[jk] = scol[j];
        }
        __syncwarp();
        if (ln == 0) {
            b[k] = bk_new;
            v[kk] = -vkk;
        }
        nrank++;
        __syncwarp();
    }
    if (deficient) {
        // clear the rows/columns that found no pivot
        int r = 0, c = ln;
        while (c > r) { c -= r + 1; r++; }
        for (int idx = ln; idx < np; idx += 32) {
            if (!used[r] && !used[c]) v[idx] = 0.0;
            c += 32;
            while (c > r) { c -= r + 1; r++; }
        }
        for (int j = ln; j < n; j += 32)
            if (!used[j]) b[j] = 0.0;
        __syncwarp();
    }
    // negation as a sign flip of the bits (exact, like the FP64 negation)
    for (int idx = ln; idx < np; idx += 32)
        v[idx] = __longlong_as_double(__double_as_longlong(v[idx]) ^ (long long)0x8000000000000000ull);
    __syncwarp();
    *nrank_out = nrank;
}

// ------------------------------------------------------------------------

// sequential sqminv for the border part (1-based)
__device__ void s_sqminv(double *v, double *b, int n, int *nrank, double *diag, int *next) {
    const double eps = 16.0 * 2.220446049250313e-16;
    int next0 = 1, l = 1;
    for (int i = 1; i <= n; i++) { next[i] = i + 1; diag[i] = fabs(v[(i * i + i) / 2]); }
    next[n] = -1;
    *nrank = 0;
    for (int i = 1; i <= n; i++) {
        int k = 0, j = next0, last = 0;
        double vkk = 0.0;
        while (j > 0) {
            int jj = (j * j + j) / 2;
            double lim = fabs(vkk) > eps * diag[j] ? fabs(vkk) : eps * diag[j];
            if (fabs(v[jj]) > lim) { vkk = v[jj]; k = j; l = last; }
            last = j;
            j = next[last];
        }
        if (k != 0) {
            int kk = (k * k + k) / 2;
            if (l == 0) next0 = next[k]; else next[l] = next[k];
            next[k] = 0;
            (*nrank)++;
            vkk = 1.0 / vkk;
            v[kk] = -vkk;
            b[k] = b[k] * vkk;
            int jk = kk - k, jl = 0;
            for (j = 1; j <= n; j++) {
                if (j == k) { jk = kk; jl = jl + j; continue; }
                if (j < k) jk = jk + 1; else jk = jk + j - 1;
                double vjk = v[jk];
                v[jk] = vkk * vjk;
                b[j] = b[j] - b[k] * vjk;
                int lk = kk - k;
                for (int ll = 1; ll <= j; ll++) {
                    jl = jl + 1;
                    if (ll == k) { lk = kk; continue; }
                    if (ll < k) lk = lk + 1; else lk = lk + ll - 1;
                    v[jl] = v[jl] - v[lk] * vjk;
                }
            }
        } else {
            for (k = 1; k <= n; k++)
                if (next[k] != 0) {
                    b[k] = 0.0;
                    for (j = 1; j <= k; j++) if (next[j] != 0) v[(k * k - k) / 2 + j] = 0.0;
                }
            break;
        }
    }
    for (int ij = 1; ij <= (n * n + n) / 2; ij++) v[ij] = -v[ij];
}

struct BandWork {
    double *vbnd, *vbdr, *aux, *vbk, *vzru, *scdiag;
    int *scflag;
};

// ------------------------------------------------------------------------
// shared-memory carve-up of one warp
struct WarpMem {
    double *gl, *rm1, *lcor, *lwgt, *res, *t1, *t2, *w0, *clmat, *blvec, *diag, *ocol, *scol;
    double *B, *W;
    double *bnd;   // band scratch (may be null)
    int32_t *in, *mq, *slots, *swS, *sw, *used, *goff;
};

__device__ WarpMem carve(char *base, const FitParams &p) {
    WarpMem m;
    double *d = (double *)base;
    m.gl = d; d += p.wmax;
    m.rm1 = d; d += p.neqmax;
    m.lcor = d; d += p.neqmax;
    m.lwgt = d; d += p.neqmax;
    m.res = d; d += p.neqmax;
    m.t1 = d; d += p.neqmax;
    m.t2 = d; d += p.neqmax;
    m.w0 = d; d += p.neqmax;
    m.clmat = d; d += (int64_t)p.nalcmax * (p.nalcmax + 1) / 2;
    m.blvec = d; d += p.nalcmax;
    m.diag = d; d += p.nalcmax;
    m.ocol = d; d += p.nalcmax;
    m.scol = d; d += p.nalcmax;
    if (!p.bigMode) {
        m.B = d; d += (int64_t)p.nalcmax * p.nalgmax;
        m.W = d; d += (int64_t)p.nalcmax * p.nalgmax;
    } else {
        m.B = m.W = nullptr;   // per record in global memory
    }
    m.bnd = p.bandmax >= 0 ? d : nullptr;
    d += band_doubles(p.nalcmax, p.bandmax, p.bdrmax);
    int32_t *q = (int32_t *)d;
    m.in = q; q += p.wmax;
    m.mq = q; q += 3 * p.neqmax;
    m.slots = q; q += p.nalgmax;
    m.swS = q; q += p.nalgmax + 1;
    m.sw = q; q += p.wmax;
    m.used = q; q += p.nalcmax + 2;
    m.goff = q;
    return m;
}

// Walk over the update elements of one record in block-major order: group
// pairs (qa >= qb), inside a pair row-major (ii, jj) with jj <= ii when
// qa == qb.  goff[q] = first slot of group q, goff[ngrp] = nalg.
struct BlockWalk {
    const int32_t *goff;
    int ngrp;
    int qa = 0, qb = 0, e = 0;     // current pair and element inside it
    int ii = 0, jj = 0;
    __device__ __forceinline__ BlockWalk(const int32_t *g, int n) : goff(g), ngrp(n) {}
    __device__ __forceinline__ int size(int q) const { return goff[q + 1] - goff[q]; }
    __device__ __forceinline__ int nel() const {
        const int na = size(qa);
        return qa == qb ? na * (na + 1) / 2 : na * size(qb);
    }
    // move n elements ahead (n <= 32)
    __device__ __forceinline__ void advance(int n) {
        if (qa >= ngrp) return;
        e += n;
        if (e < nel()) {  // same block: step the row and column
            jj += n;
            if (qa == qb) {
                while (jj > ii) { jj -= ii + 1; ii++; }
            } else {
                const int nj = size(qb);
                ii += jj / nj;
                jj -= (jj / nj) * nj;
            }
            return;
        }
        for (int guard = 0; guard < 1 << 20; ++guard) {
            const int ne = nel();
            if (e < ne) break;
            e -= ne;
            if (++qb > qa) { qa++; qb = 0; }
            if (qa >= ngrp) return;
        }
        // e < 32 here
        if (qa == qb) {
            int r = 0;
            while ((r + 1) * (r + 2) / 2 <= e) r++;
            ii = r;
            jj = e - r * (r + 1) / 2;
        } else {
            const int nj = size(qb);
            ii = e / nj;
            jj = e - ii * nj;
        }
    }
    __device__ __forceinline__ int a() const { return goff[qa] + ii; }
    __device__ __forceinline__ int b() const { return goff[qb] + jj; }
    __device__ __forceinline__ int pair() const { return qa * (qa + 1) / 2 + qb; }
};


// ------------------------------------------------------------------------
// Warp-cooperative sqmibb / sqmibb2 (mpnum.f90:3118-3600) with inv = 0
// (solution, rank and
// eigenvalue bounds; factors left in the band work areas).  Every element
// receives the same operations in the same order as in the reference's
// sequential routine, so the results are bit-identical to it; the lanes take the operations that are
// independent: the updates of one column step of the band LDL^T, the
// forward substitutions, the right-hand sides (border columns and b) of the
// backward substitutions, the border Schur products and the final updates.
#define WB2(r, c) w[((c) - 1) * mp1 + (r)]
__device__ void w_dbcdec(double *w, int mp1, int n, double *aux, double *rx) {
    const int ln = lane_id();
    for (int i = 1 + ln; i <= n; i += 32) aux[i] = 16.0 * WB2(1, i);
    __syncwarp();
    for (int i = 1; i <= n; i++) {
        const int mj = (mp1 - 1 < n - i) ? mp1 - 1 : n - i;
        if (ln == 0) {
            if (WB2(1, i) + aux[i] != aux[i]) WB2(1, i) = 1.0 / WB2(1, i);
            else WB2(1, i) = 0.0;
        }
        __syncwarp();
        const double piv = WB2(1, i);
        for (int j = 1 + ln; j <= mj; j += 32) rx[j] = WB2(j + 1, i) * piv;
        __syncwarp();
        // pair (j, k), k = 1..mj+1-j, updates WB(k, i+j) from column i
        const int npair = mj * (mj + 1) / 2;
        for (int q = ln; q < npair; q += 32) {
            int j = 1, rem = q, cnt = mj;
            while (rem >= cnt) { rem -= cnt; cnt--; j++; }
            const int k = rem + 1;
            WB2(k, i + j) = WB2(k, i + j) - WB2(k + j, i) * rx[j];
        }
        __syncwarp();
        for (int j = 1 + ln; j <= mj; j += 32) WB2(j + 1, i) = rx[j];
        __syncwarp();
    }
}

// nrhs right-hand sides: r < nrhs - extra from inBase + r * stride into
// outBase + r * stride, and (extra = 1) one more from bIn into bOut;
// x = b, then the forward and backward substitutions of s_dbcslv
__device__ void w_dbcslv_multi(const double *w, int mp1, int n, int nrhs, int extra, const double *inBase,
                               double *outBase, int64_t stride, const double *bIn, double *bOut) {
    const int ln = lane_id();
    const int nb = nrhs - extra;
    auto in_of = [&](int r) { return r < nb ? inBase + r * stride : bIn; };
    auto out_of = [&](int r) { return r < nb ? outBase + r * stride : bOut; };
    for (int q = ln; q < nrhs * n; q += 32) {
        const int r = q / n, i = 1 + q % n;
        out_of(r)[i] = in_of(r)[i];
    }
    __syncwarp();
    for (int i = 1; i <= n; i++) {
        const int mj = (mp1 - 1 < n - i) ? mp1 - 1 : n - i;
        for (int q = ln; q < nrhs * mj; q += 32) {
            const int r = q / mj, j = 1 + q % mj;
            double *x = out_of(r);
            x[j + i] = x[j + i] - WB2(j + 1, i) * x[i];
        }
        __syncwarp();
    }
    for (int r = ln; r < nrhs; r += 32) {
        double *x = out_of(r);
        for (int i = n; i >= 1; i--) {
            double rxw = x[i] * WB2(1, i);
            const int mj = (mp1 - 1 < n - i) ? mp1 - 1 : n - i;
            for (int j = 1; j <= mj; j++) rxw = rxw - WB2(j + 1, i) * x[j + i];
            x[i] = rxw;
        }
    }
    __syncwarp();
}
#undef WB2

__device__ void w_sqmibb0(int side, double *v, double *b, int n, int nbdr, int nbnd, int *nrank, double *evdmin,
                          double *evdmax, const BandWork &wk) {
    const int ln = lane_id();
    double *vbnd = wk.vbnd, *vbdr = wk.vbdr, *aux = wk.aux, *vbk = wk.vbk, *vzru = wk.vzru;
    const int mp1 = nbnd + 1, nmb = n - nbdr;
    if (side == 1) {
        const int nb1 = nbdr + 1;
        for (int q = ln; q < nmb * mp1; q += 32) {
            const int i = nb1 + q / mp1, d = q % mp1, j = i + d;
            if (j <= n) vbnd[d + 1 + (i - nb1) * mp1] = v[(j * j - j) / 2 + i];
        }
        for (int q = ln; q < nbdr * n; q += 32) {
            const int i = 1 + q / n, j = 1 + q % n;
            if (j >= i) vbdr[(i - 1) * n + j] = v[(j * j - j) / 2 + i];
        }
    } else {
        const int nb1 = nmb + 1;
        for (int q = ln; q < nmb * mp1; q += 32) {
            const int i = 1 + q / mp1, d = q % mp1, j = i + d;
            if (j <= nmb) vbnd[d + 1 + (i - 1) * mp1] = v[(j * j - j) / 2 + i];
        }
        for (int q = ln; q < nbdr * n; q += 32) {
            const int i = nb1 + q / n, j = 1 + q % n;
            if (j <= i) vbdr[(i - nb1) * n + j] = v[(i * i - i) / 2 + j];
        }
    }
    __syncwarp();
    w_dbcdec(vbnd, mp1, nmb, aux, wk.scdiag);
    // pivots: all positive, else rank 0 and everything zeroed
    int bad = 0;
    double lo = 0.0, hi = 0.0;
    for (int i = 1 + ln; i <= nmb; i += 32) {
        const double d = vbnd[(i - 1) * mp1 + 1];
        if (d <= 0.0) bad = 1;
        if (i == 1 + ln) { lo = d; hi = d; }
        else { if (d < lo) lo = d; if (d > hi) hi = d; }
    }
    const bool any = nmb > 0;
    const bool have = 1 + ln <= nmb;
    // exact min / max over the lanes that hold pivots
    double mn = 0.0, mx = 0.0;
    {
        double l0 = have ? lo : 1.0e308, h0 = have ? hi : -1.0e308;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double a = __shfl_xor_sync(0xffffffffu, l0, o), c = __shfl_xor_sync(0xffffffffu, h0, o);
            l0 = a < l0 ? a : l0;
            h0 = c > h0 ? c : h0;
        }
        mn = any ? l0 : 0.0;
        mx = any ? h0 : 0.0;
    }
    if (__any_sync(0xffffffffu, bad)) {
        for (int q = 1 + ln; q <= n; q += 32) b[q] = 0.0;
        for (int q = 1 + ln; q <= (n * n + n) / 2; q += 32) v[q] = 0.0;
        __syncwarp();
        *nrank = 0;
        *evdmin = 0.0;
        *evdmax = 0.0;
        return;
    }
    *nrank = nmb;
    *evdmin = mn;
    *evdmax = mx;
    if (nbdr == 0) {
        w_dbcslv_multi(vbnd, mp1, nmb, 1, 1, nullptr, nullptr, 0, b, b);
        return;
    }
    double *xb = wk.scdiag;   // solution of the band part of b (b itself is still needed)
    int nrankb = 0;
    if (side == 1) {
        const int nb1 = nbdr + 1;
        w_dbcslv_multi(vbnd, mp1, nmb, nbdr + 1, 1, vbdr + nb1 - 1, aux + nb1 - 1, n, b + nb1 - 1, xb);
        for (int ib = 1 + ln; ib <= nbdr; ib += 32) {
            const int ioff = nb1 + (ib - 1) * n;
            double z = b[ib];
            for (int i = 0; i <= nmb - 1; i++) z = z - b[nb1 + i] * aux[ioff + i];
            vzru[ib] = z;
        }
        __syncwarp();
        for (int i = 1 + ln; i <= nmb; i += 32) b[nb1 + i - 1] = xb[i];
        const int np = nbdr * (nbdr + 1) / 2;
        for (int q = ln; q < np; q += 32) {
            int ib = 1, rem = q;
            while (rem >= ib) { rem -= ib; ib++; }
            const int jb = rem + 1, ip = q + 1;
            const int ioff = nb1 + (ib - 1) * n, joff = nb1 + (jb - 1) * n;
            double t = v[ip];
            for (int i = 0; i <= nmb - 1; i++) t = t - vbdr[ioff + i] * aux[joff + i];
            vbk[ip] = t;
        }
        __syncwarp();
        if (ln == 0) s_sqminv(vbk, vzru, nbdr, &nrankb, wk.scdiag, wk.scflag);
        nrankb = __shfl_sync(0xffffffffu, nrankb, 0);
        __syncwarp();
        if (nrankb == nbdr) *nrank += nbdr;
        else {
            for (int ib = 1 + ln; ib <= nbdr; ib += 32) vzru[ib] = 0.0;
            for (int q = 1 + ln; q <= (nbdr * nbdr + nbdr) / 2; q += 32) vbk[q] = 0.0;
        }
        __syncwarp();
        for (int ib = 1 + ln; ib <= nbdr; ib += 32) b[ib] = vzru[ib];
        __syncwarp();
        for (int i = ln; i <= nmb - 1; i += 32) {
            double t = b[nb1 + i];
            for (int ib = 1; ib <= nbdr; ib++) t = t - b[ib] * aux[nb1 + (ib - 1) * n + i];
            b[nb1 + i] = t;
        }
        __syncwarp();
    } else {
        w_dbcslv_multi(vbnd, mp1, nmb, nbdr + 1, 1, vbdr, aux, n, b, xb);
        for (int ib = 1 + ln; ib <= nbdr; ib += 32) {
            const int ioff = (ib - 1) * n;
            double z = b[nmb + ib];
            for (int i = 1; i <= nmb; i++) z = z - b[i] * aux[ioff + i];
            vzru[ib] = z;
        }
        __syncwarp();
        for (int i = 1 + ln; i <= nmb; i += 32) b[i] = xb[i];
        const int np = nbdr * (nbdr + 1) / 2;
        for (int q = ln; q < np; q += 32) {
            int ib = 1, rem = q;
            while (rem >= ib) { rem -= ib; ib++; }
            const int jb = rem + 1, ip = q + 1;
            const int ioff = (ib - 1) * n, joff = (jb - 1) * n, koff = nmb + (ib - 1) * n;
            double t = vbdr[koff + jb];
            for (int i = 1; i <= nmb; i++) t = t - vbdr[ioff + i] * aux[joff + i];
            vbk[ip] = t;
        }
        __syncwarp();
        if (ln == 0) s_sqminv(vbk, vzru, nbdr, &nrankb, wk.scdiag, wk.scflag);
        nrankb = __shfl_sync(0xffffffffu, nrankb, 0);
        __syncwarp();
        if (nrankb == nbdr) *nrank += nbdr;
        else {
            for (int ib = 1 + ln; ib <= nbdr; ib += 32) vzru[ib] = 0.0;
            for (int q = 1 + ln; q <= (nbdr * nbdr + nbdr) / 2; q += 32) vbk[q] = 0.0;
        }
        __syncwarp();
        for (int i = 1 + ln; i <= nmb; i += 32) {
            double t = b[i];
            for (int ib = 1; ib <= nbdr; ib++) t = t - vzru[ib] * aux[(ib - 1) * n + i];
            b[i] = t;
        }
        for (int ib = 1 + ln; ib <= nbdr; ib += 32) b[nmb + ib] = vzru[ib];
        __syncwarp();
    }
}

// Full inverse of the bordered band matrix factorised by w_sqmibb0,
// warp-parallel; the same matrix as sqmibb's inv = 2 path
// (dbcinv plus the border terms, mpnum.f90:3118-3600) up to rounding.  The
// inverse enters only the Schur complement, not the fit decisions.
// (1) lane per column c: band inverse column by (L D L^T) x = e_c with the
//     factored band; (2) lane per packed element: band inverse plus the
//     border terms, border rows from vbk and aux.  v: 0-based packed n x n;
//     X: 32 x nalcmax per-lane vectors, Vs: nmb (nmb+1) / 2 (global scratch).
#define WB(r, c) w[((c) - 1) * mp1 + (r)]
__device__ void w_band_inverse(int side, double *v, int n, int nbdr, int nbnd, const BandWork &wk, double *X,
                               int xstride, double *Vs) {
    const int ln = threadIdx.x & 31;
    const int mp1 = nbnd + 1, nmb = n - nbdr;
    const double *w = wk.vbnd, *aux = wk.aux, *vbk = wk.vbk;
    for (int c0 = 1; c0 <= nmb; c0 += 32) {
        const int c = c0 + ln;
        if (c <= nmb) {
            double *x = X + ln * xstride - 1;   // 1-based
            for (int i = 1; i <= nmb; ++i) x[i] = i == c ? 1.0 : 0.0;
            for (int i = c; i <= nmb; ++i) {
                const int mj = (mp1 - 1 < nmb - i) ? mp1 - 1 : nmb - i;
                const double xi = x[i];
                for (int j = 1; j <= mj; ++j) x[j + i] = x[j + i] - WB(j + 1, i) * xi;
            }
            for (int i = nmb; i >= 1; --i) {
                double rxw = x[i] * WB(1, i);
                const int mj = (mp1 - 1 < nmb - i) ? mp1 - 1 : nmb - i;
                for (int j = 1; j <= mj; ++j) rxw = rxw - WB(j + 1, i) * x[j + i];
                x[i] = rxw;
            }
            for (int r = c; r <= nmb; ++r) Vs[(r * (r - 1)) / 2 + c] = x[r];   // Vs 1-based packed
        }
    }
    __syncwarp();
    const int total = n * (n + 1) / 2;
    const int ab = side == 1 ? nbdr + 1 : 1;   // aux position of band index 0
    // border products P(ib, i) = sum_jb K(ib, jb) aux(jb, i) with K = vbk,
    // once per record in the per-lane vector area (free after the column
    // solves): the border-band elements are -P, the band elements
    // Vs + sum_ib aux(ib, i) P(ib, j)
    const bool useP = nbdr <= 32;
    double *P = X;
    if (useP) {
        for (int q = ln; q < nbdr * nmb; q += 32) {
            const int ib = 1 + q / nmb, i = q % nmb;
            double t = 0.0;
            for (int jb = 1; jb <= nbdr; ++jb) {
                const int hi = ib > jb ? ib : jb, lo = ib > jb ? jb : ib;
                t = t + vbk[(hi * hi - hi) / 2 + lo] * aux[ab + (jb - 1) * n + i];
            }
            P[(ib - 1) * nmb + i] = t;
        }
        __syncwarp();
    }
    for (int e = ln; e < total; e += 32) {
        int R = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
        while (R > 0 && R * (R + 1) / 2 > e) R--;
        while ((R + 1) * (R + 2) / 2 <= e) R++;
        const int C = e - R * (R + 1) / 2 + 1;
        R += 1;                                   // 1-based (R, C), C <= R
        const bool rB = side == 1 ? R <= nbdr : R > nmb;
        const bool cB = side == 1 ? C <= nbdr : C > nmb;
        double val;
        if (rB && cB) {
            const int ib = side == 1 ? R : R - nmb, jb = side == 1 ? C : C - nmb;
            val = vbk[(ib * (ib - 1)) / 2 + jb];
        } else if (rB || cB) {
            const int ib = rB ? (side == 1 ? R : R - nmb) : (side == 1 ? C : C - nmb);
            const int i = (rB ? C : R) - (side == 1 ? nbdr + 1 : 1);   // band index, 0-based
            if (useP) {
                val = -P[(ib - 1) * nmb + i];
            } else {
                val = 0.0;
                for (int jb = 1; jb <= nbdr; ++jb) {
                    const int hi = ib > jb ? ib : jb, lo = ib > jb ? jb : ib;
                    val = val - vbk[(hi * hi - hi) / 2 + lo] * aux[ab + (jb - 1) * n + i];
                }
            }
        } else {
            const int i = R - (side == 1 ? nbdr + 1 : 1), j = C - (side == 1 ? nbdr + 1 : 1);
            val = Vs[((i + 1) * i) / 2 + j + 1];
            if (useP) {
                for (int ib = 1; ib <= nbdr; ++ib) val = val + aux[ab + (ib - 1) * n + i] * P[(ib - 1) * nmb + j];
            } else {
                for (int ib = 1; ib <= nbdr; ++ib)
                    for (int jb = 1; jb <= nbdr; ++jb) {
                        const int hi = ib > jb ? ib : jb, lo = ib > jb ? jb : ib;
                        val = val + vbk[(hi * hi - hi) / 2 + lo] * aux[ab + (ib - 1) * n + i] *
                                        aux[ab + (jb - 1) * n + j];
                    }
            }
        }
        v[e] = val;
    }
    __syncwarp();
}
#undef WB

__device__ __forceinline__ double wsum_serial(const double *a, int n) {
    // sequential sum in index order on lane 0, broadcast to the warp
    double s = 0.0;
    if (lane_id() == 0)
        for (int e = 0; e < n; ++e) s = s + a[e];
    return __shfl_sync(0xffffffffu, s, 0);
}

// shared-memory work areas of the bordered band solver (1-based views)
__device__ __forceinline__ BandWork band_work(const WarpMem &m, const RecInfo &ri, int n) {
    const int nb = ri.mbdr, nbd = ri.mbnd;
    BandWork wk;
    double *q = m.bnd;
    wk.vbnd = q - 1; q += (int64_t)n * (nbd + 1) + 1;
    wk.vbdr = q - 1; q += (int64_t)n * nb + 1;
    wk.aux = q - 1; q += (int64_t)n * nb + n + 1;
    wk.vbk = q - 1; q += (int64_t)nb * nb + 1;
    wk.vzru = q - 1; q += n + 1;
    wk.scdiag = q - 1; q += n + 1;
    wk.scflag = m.used - 1;
    return wk;
}

// one entry of monitoring histogram h: bins 1..nbins cover [-range, range),
// bin 0 and nbins + 1 take what falls below and above; NaN is not entered
__device__ __forceinline__ void mon_hist(const FitParams &p, int h, float x) {
    if (!(x == x)) return;
    int b;
    if (x < -p.monRange) b = 0;
    else if (x >= p.monRange) b = p.monBins + 1;
    else {
        b = 1 + (int)((x + p.monRange) * ((float)p.monBins / (2.0f * p.monRange)));
        if (b > p.monBins) b = p.monBins;
    }
    atomicAdd(&p.monHist[h * (p.monBins + 2) + b], 1ull);
}

// -sum over the equations shared by slots a and b of dw1 w g_a g_b (the
// G^T W G part of one update element): merge of the equation-ordered word
// lists, the pair taken in the reference's order (later word first); for
// two slots of one group with simple word lists one word per equation
__device__ __forceinline__ double gtwg_element(const WarpMem &m, int a, int b, bool sameGroupSimple) {
    double u = 0.0;
    int qa = m.swS[a], qae = m.swS[a + 1];
    int qb = m.swS[b], qbe = m.swS[b + 1];
    if (sameGroupSimple) {
        for (; qa < qae; ++qa, ++qb) {
            const int ea = m.sw[qa] >> 16;
            const double ca = m.w0[ea] * m.gl[m.sw[qa] & 0xffff];
            u = __fma_rn(-ca, m.gl[m.sw[qb] & 0xffff], u);
        }
        return u;
    }
    while (qa < qae && qb < qbe) {
        const int ea = m.sw[qa] >> 16, eb = m.sw[qb] >> 16;
        if (ea < eb) { qa++; continue; }
        if (eb < ea) { qb++; continue; }
        int qa2 = qa, qb2 = qb;
        while (qa2 < qae && (m.sw[qa2] >> 16) == ea) qa2++;
        while (qb2 < qbe && (m.sw[qb2] >> 16) == ea) qb2++;
        const double cw = m.w0[ea];
        for (int x = qa; x < qa2; ++x)
            for (int y = qb; y < qb2; ++y) {
                const int wa = m.sw[x] & 0xffff, wb = m.sw[y] & 0xffff;
                if (a == b && wb > wa) continue;  // pair once
                const int wj = wa > wb ? wa : wb, wk = wa > wb ? wb : wa;
                const double gj = m.gl[wj];
                if (gj == 0.0) continue;
                u = u - cw * gj * m.gl[wk];
            }
        qa = qa2;
        qb = qb2;
    }
    return u;
}

constexpr int kSformMaxEq = 8;   // equations per group of the S-form update

// whether slots a and c have an equation in common (both lists ordered by
// equation): when not, the G^T W G part of every element of a with the
// group of c (whose slots all share c's list) is the empty sum 0
__device__ __forceinline__ bool eq_lists_meet(const WarpMem &m, int a, int c) {
    int qa = m.swS[a], qae = m.swS[a + 1], qc = m.swS[c], qce = m.swS[c + 1];
    while (qa < qae && qc < qce) {
        const int ea = m.sw[qa] >> 16, ec = m.sw[qc] >> 16;
        if (ea == ec) return true;
        if (ea < ec) qa++;
        else qc++;
    }
    return false;
}

// one S-form task: row a of block (pg, q) with MQ equations in group q.
// Off-diagonal blocks (q < pg): U(a, b) = G^T W G part (the equations the
// two slots share) + sum_f Z_f g_bf with Z_f = sum_{e in E_a} g_ae S_ef.
// Diagonal blocks (q == pg, simple word lists: the slots of the group sit in
// the same MQ equations, one word each): the G^T W G part -sum_f w_f g_af
// g_bf is folded into Z (Z_f -= w_f g_af), U(a, b) = sum_f Z_f g_bf for
// b <= a.  The two kinds run in separate passes over the lanes, so that
// every lane of a pass has the same work.
template <int MQ, bool DIAG>
__device__ __forceinline__ void sform_task(const WarpMem &m, const double *S, int neq, int a, int pg, int q,
                                           const int64_t *pdst, double *stage) {
    const int c0 = m.goff[q], c1 = DIAG ? a + 1 : m.goff[q + 1];
    const int qa0 = m.swS[a], ma = m.swS[a + 1] - qa0, qc0 = m.swS[c0];
    double Z[MQ];
#pragma unroll
    for (int f = 0; f < MQ; ++f) {
        const int ef = m.sw[qc0 + f] >> 16;
        double z = 0.0;
        for (int i = 0; i < ma; ++i) {
            const int ent = m.sw[qa0 + i];
            z = __fma_rn(m.gl[ent & 0xffff], S[(ent >> 16) * neq + ef], z);
        }
        if (DIAG) z = __fma_rn(-m.w0[ef], m.gl[m.sw[qa0 + f] & 0xffff], z);
        Z[f] = z;
    }
    const int ii = a - m.goff[pg];
    const int64_t base = __ldg(pdst + pg * (pg + 1) / 2 + q) +
                         (DIAG ? (int64_t)ii * (ii + 1) / 2 : (int64_t)ii * (m.goff[q + 1] - c0));
    const bool meet = !DIAG && eq_lists_meet(m, a, c0);
    for (int b = c0; b < c1; ++b) {
        double u = meet ? gtwg_element(m, a, b, false) : 0.0;
        const int qb0 = m.swS[b];
#pragma unroll
        for (int f = 0; f < MQ; ++f) u = __fma_rn(Z[f], m.gl[m.sw[qb0 + f] & 0xffff], u);
        stage[base + (b - c0)] = u;
    }
}

// sform_task for groups in 5 to kSformMaxEq equations (a group hit more
// than twice, e.g. a module crossed again by a looping track): the same
// operations with the equation count at run time
template <bool DIAG>
__device__ void sform_task_var(const WarpMem &m, const double *S, int neq, int a, int pg, int q, int mq,
                               const int64_t *pdst, double *stage) {
    const int c0 = m.goff[q], c1 = DIAG ? a + 1 : m.goff[q + 1];
    const int qa0 = m.swS[a], ma = m.swS[a + 1] - qa0, qc0 = m.swS[c0];
    double Z[kSformMaxEq];
#pragma unroll
    for (int f = 0; f < kSformMaxEq; ++f) {
        if (f >= mq) break;
        const int ef = m.sw[qc0 + f] >> 16;
        double z = 0.0;
        for (int i = 0; i < ma; ++i) {
            const int ent = m.sw[qa0 + i];
            z = __fma_rn(m.gl[ent & 0xffff], S[(ent >> 16) * neq + ef], z);
        }
        if (DIAG) z = __fma_rn(-m.w0[ef], m.gl[m.sw[qa0 + f] & 0xffff], z);
        Z[f] = z;
    }
    const int ii = a - m.goff[pg];
    const int64_t base = __ldg(pdst + pg * (pg + 1) / 2 + q) +
                         (DIAG ? (int64_t)ii * (ii + 1) / 2 : (int64_t)ii * (m.goff[q + 1] - c0));
    const bool meet = !DIAG && eq_lists_meet(m, a, c0);
    for (int b = c0; b < c1; ++b) {
        double u = meet ? gtwg_element(m, a, b, false) : 0.0;
        const int qb0 = m.swS[b];
#pragma unroll
        for (int f = 0; f < kSformMaxEq; ++f) {
            if (f >= mq) break;
            u = __fma_rn(Z[f], m.gl[m.sw[qb0 + f] & 0xffff], u);
        }
        stage[base + (b - c0)] = u;
    }
}

// one off-diagonal S-form block (groups pg > q) by one lane: the block of S
// over the equations of the two groups is loaded once into registers
// (large records keep S in global memory), then the rows a of pg as in
// sform_task: Z_f = sum_i g_ai S(e_i, f), U(a, b) = G^T W G part + sum_f Z_f
// g_bf; the same operations in the same order as the per-row tasks
template <int MP, int MQ>
__device__ __forceinline__ void sform_block(const WarpMem &m, const double *S, int neq, int pg, int q,
                                            const int64_t *pdst, double *stage) {
    const int a0 = m.goff[pg], a1 = m.goff[pg + 1], c0 = m.goff[q], c1 = m.goff[q + 1];
    const int qa0 = m.swS[a0], qc0 = m.swS[c0];
    double Sb[MP][MQ];
#pragma unroll
    for (int i = 0; i < MP; ++i) {
        const int ei = m.sw[qa0 + i] >> 16;
#pragma unroll
        for (int f = 0; f < MQ; ++f) Sb[i][f] = S[ei * neq + (m.sw[qc0 + f] >> 16)];
    }
    const bool meet = eq_lists_meet(m, a0, c0);
    const int ncol = c1 - c0;
    const int64_t base = __ldg(pdst + pg * (pg + 1) / 2 + q);
    for (int a = a0; a < a1; ++a) {
        const int qa = m.swS[a];
        double Z[MQ];
#pragma unroll
        for (int f = 0; f < MQ; ++f) {
            double z = 0.0;
#pragma unroll
            for (int i = 0; i < MP; ++i) z = __fma_rn(m.gl[m.sw[qa + i] & 0xffff], Sb[i][f], z);
            Z[f] = z;
        }
        const int64_t row = base + (int64_t)(a - a0) * ncol;
        for (int b = c0; b < c1; ++b) {
            double u = meet ? gtwg_element(m, a, b, false) : 0.0;
            const int qb0 = m.swS[b];
#pragma unroll
            for (int f = 0; f < MQ; ++f) u = __fma_rn(Z[f], m.gl[m.sw[qb0 + f] & 0xffff], u);
            stage[row + (b - c0)] = u;
        }
    }
}

__device__ __forceinline__ void sform_block_dispatch(const WarpMem &m, const double *S, int neq, int pg, int q,
                                                     const int64_t *pdst, double *stage) {
    const int mp = m.swS[m.goff[pg] + 1] - m.swS[m.goff[pg]];
    const int mq = m.swS[m.goff[q] + 1] - m.swS[m.goff[q]];
    if (mp > 4 || mq > 4) {
        // a group in more than four equations: row by row with S read as needed
        for (int a = m.goff[pg]; a < m.goff[pg + 1]; ++a) sform_task_var<false>(m, S, neq, a, pg, q, mq, pdst, stage);
        return;
    }
    switch ((mp - 1) * 4 + (mq - 1)) {
        case 0: sform_block<1, 1>(m, S, neq, pg, q, pdst, stage); break;
        case 1: sform_block<1, 2>(m, S, neq, pg, q, pdst, stage); break;
        case 2: sform_block<1, 3>(m, S, neq, pg, q, pdst, stage); break;
        case 3: sform_block<1, 4>(m, S, neq, pg, q, pdst, stage); break;
        case 4: sform_block<2, 1>(m, S, neq, pg, q, pdst, stage); break;
        case 5: sform_block<2, 2>(m, S, neq, pg, q, pdst, stage); break;
        case 6: sform_block<2, 3>(m, S, neq, pg, q, pdst, stage); break;
        case 7: sform_block<2, 4>(m, S, neq, pg, q, pdst, stage); break;
        case 8: sform_block<3, 1>(m, S, neq, pg, q, pdst, stage); break;
        case 9: sform_block<3, 2>(m, S, neq, pg, q, pdst, stage); break;
        case 10: sform_block<3, 3>(m, S, neq, pg, q, pdst, stage); break;
        case 11: sform_block<3, 4>(m, S, neq, pg, q, pdst, stage); break;
        case 12: sform_block<4, 1>(m, S, neq, pg, q, pdst, stage); break;
        case 13: sform_block<4, 2>(m, S, neq, pg, q, pdst, stage); break;
        case 14: sform_block<4, 3>(m, S, neq, pg, q, pdst, stage); break;
        default: sform_block<4, 4>(m, S, neq, pg, q, pdst, stage); break;
    }
}

template <bool DIAG>
__device__ __forceinline__ void sform_dispatch(const WarpMem &m, const double *S, int neq, int a, int pg, int q,
                                               const int64_t *pdst, double *stage) {
    const int c0 = m.goff[q];
    const int mq = m.swS[c0 + 1] - m.swS[c0];
    switch (mq) {
        case 1: sform_task<1, DIAG>(m, S, neq, a, pg, q, pdst, stage); break;
        case 2: sform_task<2, DIAG>(m, S, neq, a, pg, q, pdst, stage); break;
        case 3: sform_task<3, DIAG>(m, S, neq, a, pg, q, pdst, stage); break;
        case 4: sform_task<4, DIAG>(m, S, neq, a, pg, q, pdst, stage); break;
        default: sform_task_var<DIAG>(m, S, neq, a, pg, q, mq, pdst, stage); break;
    }
}

template <bool BIG>
__global__ void __launch_bounds__(32 * MPG_WARPS_FIT, 2)
k_fit(FitParams p, int perWarp) {
    extern __shared__ __align__(16) char smem[];
    const int ln = lane_id();
    const int wib = threadIdx.x >> 5, wpc = blockDim.x >> 5;
    WarpMem m = carve(smem + (int64_t)wib * perWarp, p);
    const int64_t nwarps = (int64_t)gridDim.x * wpc;

    for (int64_t it = p.r0 + (int64_t)blockIdx.x * wpc + wib; it < p.r1; it += nwarps) {
        const int64_t r = p.recList ? (int64_t)p.recList[it] : it;
        const RecInfo ri = p.rec[r];
        const int nw = ri.nw, neq = ri.neq, nalc = ri.nalc, nalg = ri.nalg;
        for (int i = ln; i < nw; i += 32) {
            m.gl[i] = p.glder[ri.w0 + i];
            m.in[i] = p.inder[ri.w0 + i];
        }
        for (int i = ln; i < 3 * neq; i += 32) m.mq[i] = p.meas[3 * ri.measOff + i];
        for (int i = ln; i < nalg; i += 32) m.slots[i] = p.slots[ri.slotOff + i];
        for (int i = ln; i <= nalg; i += 32) m.swS[i] = p.swStart[ri.slotOff + i];
        const int ngrp = ri.ngrp;
        const int64_t *pdst = p.pairDst + ri.pairOff;  // staging offset per group pair
        double *mB = m.B, *mW = m.W;   // large records: this record's slot in global memory
        if (BIG) {
            mB = p.bw + (it - p.r0) * p.bwStride;
            mW = mB + (int64_t)nalc * nalg;
        }
        if (p.icalcm == 1 && nalc > 0) {
            for (int i = ln; i < ngrp; i += 32) m.goff[i] = p.grpSlot[ri.grpOff + i];
            if (ln == 0) m.goff[ngrp] = nalg;
        }
        __syncwarp();
        const int nswr = m.swS[nalg];
        for (int i = ln; i < nswr; i += 32) m.sw[i] = p.sw[ri.swOff + i];

        int st = 0;          // 0 accepted, 1..6 rejection class, -1 no locals
        double chi2add = 0.0;
        int ndfadd = 0;
        float chndf = 0.0f;
        if (nalc <= 0) {
            st = -1;
        } else {
            const double dw1 = p.fileWeight ? p.fileWeight[ri.file - 1] : 1.0;
            const double dw2 = sqrt(dw1);
            // ---- first loop: subtract the current global parameters
            for (int e = ln; e < neq; e += 32) {
                const int sl = m.mq[3 * e], sg = m.mq[3 * e + 1], lg = m.mq[3 * e + 2];
                double rm = m.gl[sl];
                for (int j = 1; j <= lg - sg; ++j) {
                    const int li = m.in[sg + j];
                    rm = rm - m.gl[sg + j] * p.gpar[li - 1];
                }
                m.rm1[e] = rm;
                m.lcor[e] = 0.0;
                const double rerr = m.gl[sg];
                m.w0[e] = 1.0 / (rerr * rerr);   // weight from the error, same value in every loop
            }
            __syncwarp();
            const int nter = (p.nloopn != 1 && p.lhuber != 0) ? p.lhuber : 1;
            const bool band = ri.mbnd >= 0 && p.lfitbb > 0 && nalc > 5;
            const bool seqNormal = ((ri.mside >> 8) & 1) != 0;
            const bool denseLoc = ((ri.mside >> 9) & 1) != 0;
            const bool simpleWords = ((ri.mside >> 10) & 1) != 0;
            const bool needResing = p.lhuber > 1 && p.dwcut != 0.0f;
            const int npk = (nalc * nalc + nalc) / 2;
            int nrank = 0, ndf = 0;
            double summ = 0.0;
            float cndl10 = 0.0f, resing = 0.0f;
            for (int iter = 1; iter <= nter; ++iter) {
                const bool down = (p.nloopn != 1 && iter != 1 && p.lhuber != 0);
                for (int e = ln; e < neq; e += 32) {
                    const int sg = m.mq[3 * e + 1];
                    const double rerr = m.gl[sg];
                    double wght = m.w0[e];
                    const double resid = m.rm1[e] - m.lcor[e];
                    if (down) {
                        if (iter <= 3) {
                            if (fabs(resid) > kChuber * rerr) wght = wght * kChuber * rerr / fabs(resid);
                        } else {
                            const double t = resid / rerr / kCauchy;
                            wght = wght / (1.0 + t * t);
                        }
                    }
                    m.lwgt[e] = wght;
                }
                // ---- second loop: normal equations
                // room for the products w g_j and w r of every equation in the
                // B/W area, which the local fit does not use otherwise
                const bool preW = !BIG && (int64_t)neq * (nalc + 1) <= 2 * (int64_t)p.nalcmax * p.nalgmax;
                if (denseLoc && preW) {
                    // every equation has the locals 1..nalc: the first products
                    // c_ej = w_e g_ej and c_e0 = w_e r_e once per equation, then
                    // a lane per element of clmat (row j >= column k) or blvec,
                    // equations added in order, each term c_ej g_ek resp.
                    // c_e0 g_ej: the operations of the equation-by-equation
                    // form, (w g_j) g_k and (w r) g_j
                    double *cw = mB;   // neq x (nalc + 1)
                    for (int t = ln; t < neq * (nalc + 1); t += 32) {
                        const int e = t / (nalc + 1), j = t - e * (nalc + 1);
                        cw[t] = m.lwgt[e] * (j == 0 ? m.rm1[e] : m.gl[m.mq[3 * e] + j]);
                    }
                    __syncwarp();
                    const int nq = npk + nalc;
                    for (int q = ln; q < nq; q += 32) {
                        const bool isC = q < npk;
                        int j = q - npk + 1, k = 1;
                        if (isC) {
                            j = 1;
                            k = q + 1;
                            while (k > j) { k -= j; j++; }
                        }
                        double acc = 0.0;
                        for (int e = 0; e < neq; ++e) {
                            const double c = cw[e * (nalc + 1) + (isC ? j : 0)];
                            acc = acc + c * m.gl[m.mq[3 * e] + (isC ? k : j)];
                        }
                        if (isC) m.clmat[q] = acc;
                        else m.blvec[j - 1] = acc;
                    }
                    __syncwarp();
                } else if (denseLoc) {
                    // every equation has the locals 1..nalc: lane per element
                    // of clmat (row j >= column k) or blvec, equations added in
                    // order, each term (w g_j) g_k resp. (w r) g_j as in the
                    // equation-by-equation form
                    const int nq = npk + nalc;
                    for (int q = ln; q < nq; q += 32) {
                        const bool isC = q < npk;
                        int j = q - npk + 1, k = 1;
                        if (isC) {
                            j = 1;
                            k = q + 1;
                            while (k > j) { k -= j; j++; }
                        }
                        double acc = 0.0;
                        for (int e = 0; e < neq; ++e) {
                            const int sl = m.mq[3 * e];
                            const double x = isC ? m.gl[sl + j] : m.rm1[e];
                            const double y = isC ? m.gl[sl + k] : m.gl[sl + j];
                            acc = acc + m.lwgt[e] * x * y;
                        }
                        if (isC) m.clmat[q] = acc;
                        else m.blvec[j - 1] = acc;
                    }
                    __syncwarp();
                } else {
                for (int i = ln; i < npk; i += 32) m.clmat[i] = 0.0;
                for (int i = ln; i < nalc; i += 32) m.blvec[i] = 0.0;
                __syncwarp();
                for (int e = 0; e < neq; ++e) {
                    const int sl = m.mq[3 * e], sg = m.mq[3 * e + 1];
                    const int nl = sg - sl - 1;
                    const double wght = m.lwgt[e], rm = m.rm1[e];
                    if (!seqNormal) {
                        const int npair = (nl * nl + nl) / 2;
                        int j = 1, k = 1 + ln;
                        while (k > j) { k -= j; j++; }
                        for (int q = ln; q < npair; q += 32) {
                            const int ij = m.in[sl + j], ik = m.in[sl + k];
                            const int jk = (ij * ij - ij) / 2 + ik;
                            m.clmat[jk - 1] = m.clmat[jk - 1] + wght * m.gl[sl + j] * m.gl[sl + k];
                            k += 32;
                            while (k > j) { k -= j; j++; }
                        }
                        for (int jj = 1 + ln; jj <= nl; jj += 32) {
                            const int ij = m.in[sl + jj];
                            m.blvec[ij - 1] = m.blvec[ij - 1] + wght * rm * m.gl[sl + jj];
                        }
                    } else if (ln == 0) {
                        // local indices not strictly increasing: reference order, one lane
                        for (int jj = 1; jj <= nl; ++jj) {
                            const int ij = m.in[sl + jj];
                            m.blvec[ij - 1] = m.blvec[ij - 1] + wght * rm * m.gl[sl + jj];
                            for (int kk = 1; kk <= jj; ++kk) {
                                const int ik = m.in[sl + kk];
                                const int jk = (ij * ij - ij) / 2 + ik;
                                m.clmat[jk - 1] = m.clmat[jk - 1] + wght * m.gl[sl + jj] * m.gl[sl + kk];
                            }
                        }
                    }
                    __syncwarp();
                }
                }
                // ---- local solve
                if (band) {
                    // the solution and the factors (the arithmetic of the
                    // decisions, bit-identical to the one-lane form); the
                    // inverse, needed for the update only, is formed
                    // warp-parallel after the iterations
                    double evdmin = 0.0, evdmax = 0.0;
                    int nr = 0;
                    const BandWork wk = band_work(m, ri, nalc);
                    w_sqmibb0(ri.mside & 0xff, m.clmat - 1, m.blvec - 1, nalc, ri.mbdr, ri.mbnd, &nr, &evdmin,
                              &evdmax, wk);
                    cndl10 = evdmin > 0.0 ? log10f((float)(evdmax / evdmin)) : 0.0f;
                    nrank = nr;
                    if (p.monOn && p.monPull && iter == 1 && nr == nalc) {
                        // the local covariance for the pulls (rebuilt from the
                        // normal equations in later iterations)
                        const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
                        double *X = p.bscr + wid * p.bscrStride;
                        w_band_inverse(ri.mside & 0xff, m.clmat, nalc, ri.mbdr, ri.mbnd, wk, X, p.nalcmax,
                                       X + 32 * (int64_t)p.nalcmax);
                    }
                } else {
                    cndl10 = 0.0f;
                    warp_sqminv(m.clmat, m.blvec, nalc, &nrank, m.diag, m.ocol, m.scol, m.used);
                }
                int nanl = 0;
                for (int k = ln; k < nalc; k += 32) {
                    const double bv = m.blvec[k];
                    if (!(bv <= 0.0) && !(bv > 0.0)) nanl = 1;
                }
                const bool nan = __any_sync(0xffffffffu, nanl) != 0;
                // ---- third loop: residuals and chi2
                for (int e = ln; e < neq; e += 32) {
                    const int sl = m.mq[3 * e], sg = m.mq[3 * e + 1];
                    const double rerr = m.gl[sg];
                    double wght = m.w0[e];
                    double rmloc = 0.0;
                    for (int j = 1; j <= sg - sl - 1; ++j) {
                        const int ij = m.in[sl + j];
                        rmloc = rmloc + m.gl[sl + j] * m.blvec[ij - 1];
                    }
                    m.lcor[e] = rmloc;
                    const double rm = m.rm1[e] - rmloc;
                    if (p.monOn && iter == 1) {
                        // monitoring (pede.f90:3938-3980, 4025-4032): normalized
                        // residual; pull rm / sqrt(1/w - l^T C l) where variance is
                        // left, binned per group of the first global label
                        const bool withGlobal = sg < m.mq[3 * e + 2];
                        mon_hist(p, withGlobal ? 0 : 1, (float)(rm / rerr));
                        if (p.monPull && (!band || nrank == nalc)) {
                            double dvar = 0.0;
                            for (int j = 1; j <= sg - sl - 1; ++j) {
                                const int ij = m.in[sl + j];
                                const int jk = (ij * ij - ij) / 2;
                                for (int k = 1; k <= j - 1; ++k) {
                                    const int ik = m.in[sl + k];
                                    dvar = dvar + m.clmat[jk + ik - 1] * m.gl[sl + j] * m.gl[sl + k] * 2.0;
                                }
                                dvar = dvar + m.clmat[jk + ij - 1] * m.gl[sl + j] * m.gl[sl + j];
                            }
                            if (0.999999 / wght > dvar) {
                                const double pull = rm / sqrt(1.0 / wght - dvar);
                                mon_hist(p, withGlobal ? 2 : 3, (float)pull);
                                if (withGlobal && p.measIndex) {
                                    const int g = p.measIndex[m.in[sg + 1] - 1];
                                    if (g > 0) {
                                        const double half = 0.5 * (double)p.monMeasBins;
                                        const double x = p.monMode == 0 ? pull * rerr / p.measRes[g - 1] / 0.1 + half
                                                                        : pull / 0.1 + half;
                                        int irbin = x == x ? (int)x : 1;
                                        irbin = irbin < 1 ? 1 : (irbin > p.monMeasBins ? p.monMeasBins : irbin);
                                        atomicAdd(&p.measHists[(int64_t)(g - 1) * p.monMeasBins + irbin - 1], 1ull);
                                    }
                                }
                            }
                        }
                    }
                    double dchi2 = wght * rm * rm;
                    if (down) {
                        if (iter <= 3) {
                            if (fabs(rm) > kChuber * rerr) {
                                wght = wght * kChuber * rerr / fabs(rm);
                                dchi2 = 2.0 * kChuber * (fabs(rm) / rerr - 0.5 * kChuber);
                            }
                        } else {
                            const double t = rm / rerr / kCauchy;
                            wght = wght / (1.0 + t * t);
                            dchi2 = log(1.0 + t * t) * (kCauchy * kCauchy);
                        }
                    }
                    m.t1[e] = dchi2;
                    if (needResing) {
                        const double dn = 1.0 / sqrt(wght);
                        m.t2[e] = rerr / dn;
                    }
                }
                __syncwarp();
                summ = wsum_serial(m.t1, neq);
                ndf = neq - nrank;
                if (needResing) {
                    // down-weight fraction, used only by the dwcut decision
                    const double suwt = wsum_serial(m.t2, neq);
                    resing = ((float)neq - (float)suwt) / (float)neq;
                }
                if (nan) { st = 1; break; }
                if (nrank != nalc) { st = 2; break; }
                if (cndl10 > p.cndlmx) { st = 3; break; }
                if (ndf <= 0) { st = 4; break; }
                chndf = (float)(summ / (double)ndf);
            }
            // ---- rejection cuts (pede.f90:4106-4144)
            if (st == 0) {
                const float chichi = d_chindl(3, ndf) * (float)ndf;
                if (p.chicut >= 0.0f) {
                    if (summ > (double)(p.chhuge * chichi)) {
                        st = 5;
                    } else if (p.chicut > 0.0f) {
                        const float chlimt = p.chicut * chichi;
                        if (summ > (double)chlimt) {
                            st = 6;
                            chi2add = (double)chlimt;
                            ndfadd = ndf;
                        }
                    }
                }
                if (st == 0 && p.lhuber > 1 && p.dwcut != 0.0f && resing > p.dwcut) {
                    st = 6;
                    chi2add = summ;
                    ndfadd = ndf;
                }
            }
            if (st == 0) {
                // ---- fourth loop: residuals, weights and chi2 of the accepted fit
                for (int e = ln; e < neq; e += 32) {
                    const int sg = m.mq[3 * e + 1];
                    const double rm = m.rm1[e] - m.lcor[e];
                    const double rerr = m.gl[sg];
                    double wght = m.w0[e];
                    double dchi2 = wght * rm * rm;
                    if (p.nloopn != 1 && p.lhuber != 0) {
                        const double resid = fabs(rm);
                        if (nter <= 3) {
                            if (resid > kChuber * rerr)
                                dchi2 = 2.0 * kChuber * (resid / rerr - 0.5 * kChuber);
                        } else {
                            const double t = resid / rerr / kCauchy;
                            dchi2 = log(1.0 + t * t) * (kCauchy * kCauchy);
                        }
                        wght = m.lwgt[e];
                    }
                    m.res[e] = rm;
                    m.lwgt[e] = wght;
                    m.t1[e] = dchi2;
                }
                __syncwarp();
                // without down-weighting in this loop the terms equal those of
                // the last third-loop pass, so is their ordered sum
                chi2add = (p.nloopn != 1 && p.lhuber != 0) ? wsum_serial(m.t1, neq) : summ;
                ndfadd = ndf;
                // per-equation factors of the vector and B terms, (dw1 w) r and
                // dw2 w, and of the G^T W G term, dw1 w
                __syncwarp();
                for (int e = ln; e < neq; e += 32) {
                    const double wv = m.lwgt[e];
                    m.t1[e] = dw1 * wv * m.res[e];
                    m.t2[e] = dw2 * wv;
                    m.w0[e] = dw1 * wv;
                }
                __syncwarp();
                // ---- form of the Schur term B Gamma^-1 B^T.  With T_ek = t2_e
                // l_ek (weighted local derivatives) B = G T, so the term is
                // G S G^T with S = T Gamma^-1 T^T (neq x neq), and the block of
                // groups (p, q) is G_p S(E_p, E_q) G_q^T over the equations
                // E_p, E_q of the two groups: cheaper than the rank-nalc form
                // when groups sit in few equations (one hit: two).  Taken for
                // records with simple word lists, at most four equations per
                // group, room for Y and S in the B/W area and a lower count.
                bool sform = false;
                if (p.icalcm == 1 && simpleWords) {
                    int mmax = 0, nnz = 0;
                    for (int g = ln; g < ngrp; g += 32) {
                        const int c0 = m.goff[g];
                        mmax = max(mmax, m.swS[c0 + 1] - m.swS[c0]);
                    }
                    for (int e = ln; e < neq; e += 32) nnz += m.mq[3 * e + 1] - m.mq[3 * e] - 1;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        mmax = max(mmax, __shfl_xor_sync(0xffffffffu, mmax, o));
                        nnz += __shfl_xor_sync(0xffffffffu, nnz, o);
                    }
                    // Y, S and the task prefix in the B/W area (large records:
                    // the record's slot in global memory)
                    const int64_t room = BIG ? p.bwStride : 2 * (int64_t)p.nalcmax * p.nalgmax;
                    const int64_t need = (int64_t)neq * nalc + (int64_t)neq * neq + (ngrp + 2) / 2 + 1 +
                                         (neq + 2) / 2 + 1;
                    if (mmax >= 1 && mmax <= kSformMaxEq && need <= room) {
                        const int64_t ngg = ((int64_t)nalg * nalg + nalg) / 2;
                        const int64_t costB = (int64_t)nalg * nalc * (nalc + 1) + ngg * nalc;
                        // tasks (slot a, group q <= group of a): about nalg * ngrp / 2
                        const int64_t ntask = (int64_t)nalg * (ngrp + 1) / 2;
                        const int64_t costS = (int64_t)nnz * nalc + (int64_t)neq * (neq + 1) / 2 * (nnz / neq + 1) +
                                              ngg * mmax + ntask * mmax * mmax;
                        sform = costS < costB;
                    }
                }
                // ---- global vector and local-global matrix B, one lane per slot
                for (int s = ln; s < nalg; s += 32) {
                    double v = 0.0;
                    if (p.icalcm == 1 && !sform)
                        for (int k = 0; k < nalc; ++k) mB[k * nalg + s] = 0.0;
                    for (int q = m.swS[s]; q < m.swS[s + 1]; ++q) {
                        const int ent = m.sw[q];
                        const int e = ent >> 16, wp = ent & 0xffff;
                        const double g = m.gl[wp];
                        if (g != 0.0) v = v + m.t1[e] * g;
                        if (p.icalcm == 1 && !sform) {
                            const double cb = m.t2[e] * g;
                            const int sl = m.mq[3 * e], sg = m.mq[3 * e + 1];
                            for (int jj = 1; jj <= sg - sl - 1; ++jj) {
                                const int k = m.in[sl + jj] - 1;
                                mB[k * nalg + s] = __fma_rn(cb, m.gl[sl + jj], mB[k * nalg + s]);
                            }
                        }
                    }
                    p.vstage[ri.slotOff + s] = v;
                }
                __syncwarp();
                if (p.icalcm == 1 && band) {
                    const BandWork wk = band_work(m, ri, nalc);
                    const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
                    double *X = p.bscr + wid * p.bscrStride;
                    w_band_inverse(ri.mside & 0xff, m.clmat, nalc, ri.mbdr, ri.mbnd, wk, X, p.nalcmax,
                                   X + 32 * (int64_t)p.nalcmax);
                }
                if (p.icalcm == 1 && sform) {
                    double *Y = mB;                               // neq x nalc: L Gamma^-1
                    double *S = mB + (int64_t)neq * nalc;         // neq x neq
                    int32_t *tpre = reinterpret_cast<int32_t *>(S + (int64_t)neq * neq);   // ngrp + 1
                    // the equations with global parameters, in order: the
                    // update reads Y and S only on those (a broken-line
                    // record's kink equations have none)
                    int32_t *geq = tpre + ngrp + 2;
                    int nge = 0;
                    for (int base = 0; base < neq; base += 32) {
                        const int e = base + ln;
                        const bool has = e < neq && m.mq[3 * e + 2] > m.mq[3 * e + 1];
                        const unsigned bal = __ballot_sync(0xffffffffu, has);
                        if (has) geq[nge + __popc(bal & ((1u << ln) - 1u))] = e;
                        nge += __popc(bal);
                    }
                    __syncwarp();
                    // Y_ek = sum over the locals j of equation e of l_ej Gamma^-1_jk
                    for (int t = ln; t < nge * nalc; t += 32) {
                        const int e = geq[t / nalc], k = t - (t / nalc) * nalc + 1;
                        const int sl = m.mq[3 * e], sg = m.mq[3 * e + 1];
                        double y = 0.0;
                        for (int jj = 1; jj <= sg - sl - 1; ++jj) {
                            const int l = m.in[sl + jj];
                            const double g = l <= k ? m.clmat[(k * k - k) / 2 + l - 1] : m.clmat[(l * l - l) / 2 + k - 1];
                            y = __fma_rn(m.gl[sl + jj], g, y);
                        }
                        Y[e * nalc + k - 1] = y;
                    }
                    // prefix of the off-diagonal tasks over groups: group g
                    // has (rows of g) x g of them (columns groups q < g)
                    if (!BIG && ln == 0) {
                        int acc = 0;
                        for (int g = 0; g < ngrp; ++g) {
                            tpre[g] = acc;
                            acc += (m.goff[g + 1] - m.goff[g]) * g;
                        }
                        tpre[ngrp] = acc;
                    }
                    __syncwarp();
                    // S_ef = t2_e t2_f sum over the locals k of equation f of Y_ek l_fk
                    const int ns = nge * (nge + 1) / 2;
                    for (int t = ln; t < ns; t += 32) {
                        int ie = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
                        while (ie > 0 && ie * (ie + 1) / 2 > t) ie--;
                        while ((ie + 1) * (ie + 2) / 2 <= t) ie++;
                        const int e = geq[ie], f = geq[t - ie * (ie + 1) / 2];
                        const int sl = m.mq[3 * f], sg = m.mq[3 * f + 1];
                        double acc = 0.0;
                        for (int jj = 1; jj <= sg - sl - 1; ++jj)
                            acc = __fma_rn(Y[e * nalc + m.in[sl + jj] - 1], m.gl[sl + jj], acc);
                        const double v = m.t2[e] * m.t2[f] * acc;
                        S[e * neq + f] = v;
                        S[f * neq + e] = v;
                    }
                    __syncwarp();
                    // tasks (slot a, group q <= group p of a): Z_f = sum_{e in
                    // E_p} g_ae S_ef over the equations f of q, then the row of
                    // a in block (p, q).  Off-diagonal blocks first (every
                    // task the same size), then the diagonal ones, one per slot
                    const int ntask = BIG ? 0 : tpre[ngrp];
                    if (BIG) {
                        // large records (S in global memory): a lane per
                        // off-diagonal block (pg, q), q < pg, t = pg (pg - 1) / 2 + q
                        const int nblk = ngrp * (ngrp - 1) / 2;
                        for (int t = ln; t < nblk; t += 32) {
                            int pg = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)t)) * 0.5f);
                            while (pg > 1 && pg * (pg - 1) / 2 > t) pg--;
                            while ((pg + 1) * pg / 2 <= t) pg++;
                            sform_block_dispatch(m, S, neq, pg, t - pg * (pg - 1) / 2, pdst, p.stage);
                        }
                    }
                    for (int t = ln; t < ntask; t += 32) {
                        int lo = 0, hi = ngrp - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (tpre[mid] <= t) lo = mid;
                            else hi = mid - 1;
                        }
                        const int pg = lo, loc = t - tpre[pg];
                        const int a = m.goff[pg] + loc / pg, q = loc % pg;
                        sform_dispatch<false>(m, S, neq, a, pg, q, pdst, p.stage);
                    }
                    for (int a = ln; a < nalg; a += 32) {
                        int lo = 0, hi = ngrp - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (m.goff[mid] <= a) lo = mid;
                            else hi = mid - 1;
                        }
                        sform_dispatch<true>(m, S, neq, a, lo, lo, pdst, p.stage);
                    }
                } else if (p.icalcm == 1) {
                    // W = B Gamma^-1 (dbavat's c_ik, mpnum.f90:1422-1432):
                    // eight k at a time, each c_ik summed over l = 1..nalc in
                    // order, every B(l, s) loaded once per eight products
                    constexpr int KB = 8;
                    for (int s = ln; s < nalg; s += 32) {
                        for (int k0 = 1; k0 <= nalc; k0 += KB) {
                            double cik[KB];
#pragma unroll
                            for (int t = 0; t < KB; ++t) cik[t] = 0.0;
                            for (int l = 1; l <= nalc; ++l) {
                                const double bl = mB[(l - 1) * nalg + s];
                                const int ll = (l * l - l) / 2;
#pragma unroll
                                for (int t = 0; t < KB; ++t) {
                                    const int k = k0 + t;
                                    if (k > nalc) break;
                                    // Gamma^-1(l, k) of the packed lower triangle
                                    const double g = l <= k ? m.clmat[(k * k - k) / 2 + l - 1] : m.clmat[ll + k - 1];
                                    cik[t] = __fma_rn(bl, g, cik[t]);
                                }
                            }
#pragma unroll
                            for (int t = 0; t < KB; ++t)
                                if (k0 + t <= nalc) mW[s * nalc + k0 + t - 1] = cik[t];
                        }
                    }
                    __syncwarp();
                    // U(a,b) = -sum_eq dw1 w g_a g_b + sum_k W(a,k) B(b,k), a >= b,
                    // written block by block (group pairs qa >= qb, rows ii,
                    // columns jj <= ii on diagonal blocks) to the staging
                    // position of the block's record list
                    BlockWalk bw(m.goff, ngrp);
                    bw.advance(ln);
                    const int64_t ngg = ((int64_t)nalg * nalg + nalg) / 2;
                    for (int64_t idx = ln; idx < ngg; idx += 32) {
                        const int a = bw.a(), b = bw.b();
                        double u = gtwg_element(m, a, b, simpleWords && bw.qa == bw.qb);
                        if (!BIG) {   // large records: W B^T added by k_update_big
                            const double *wa = mW + a * nalc;
                            for (int k = 0; k < nalc; ++k) u = __fma_rn(wa[k], mB[k * nalg + b], u);
                        }
                        p.stage[__ldg(pdst + bw.pair()) + bw.e] = u;
                        bw.advance(32);
                    }
                }
                // large records: the update kernel adds W B^T unless the
                // fit wrote the whole update here
                if (BIG && p.icalcm == 1 && ln == 0) p.bigDone[it - p.r0] = sform ? 1 : 0;
            }
        }
        if (st != 0 && p.icalcm == 1 && nalc > 0) {
            // a rejected record contributes an all-zero update
            BlockWalk bw(m.goff, ngrp);
            bw.advance(ln);
            const int64_t ngg = ((int64_t)nalg * nalg + nalg) / 2;
            for (int64_t idx = ln; idx < ngg; idx += 32) {
                p.stage[__ldg(pdst + bw.pair()) + bw.e] = 0.0;
                bw.advance(32);
            }
        }
        if (ln == 0) {
            p.status[r] = (int8_t)st;
            p.chi2add[r] = chi2add;
            p.ndfadd[r] = ndfadd;
            p.chndf[r] = st == 0 ? chndf : 0.0f;
        }
        __syncwarp();
    }
}

}  // namespace

// W B^T of one accepted large record per CTA, in 64 x 64 tiles of the
// lower triangle (256 threads, 4 x 4 elements each, K in chunks of 16
// through shared memory), added to the record's block-major staging, which
// already holds its G^T W G part.
namespace {
constexpr int kUbT = 64, kUbK = 16;
__global__ void __launch_bounds__(256) k_update_big(FitParams p) {
    __shared__ double ws[kUbK][kUbT + 1], bs[kUbK][kUbT + 1];
    __shared__ int32_t goffs[MPG_NGRP_MAX + 2];
    extern __shared__ int32_t gidx[];   // group of each slot
    const int64_t it = p.r0 + blockIdx.x;
    const int64_t r = p.recList ? (int64_t)p.recList[it] : it;
    const RecInfo ri = p.rec[r];
    if (ri.nalc <= 0 || p.status[r] != 0 || p.bigDone[blockIdx.x]) return;
    const int nalg = ri.nalg, nalc = ri.nalc, ngrp = ri.ngrp;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    for (int g = tid; g < ngrp; g += blockDim.x) goffs[g] = p.grpSlot[ri.grpOff + g];
    if (tid == 0) goffs[ngrp] = nalg;
    __syncthreads();
    for (int sl = tid; sl < nalg; sl += blockDim.x) {
        int g = 0;
        while (g + 1 < ngrp && goffs[g + 1] <= sl) g++;
        gidx[sl] = g;
    }
    __syncthreads();
    const double *B = p.bw + (it - p.r0) * p.bwStride;  // B[k * nalg + s]
    const double *W = B + (int64_t)nalc * nalg;          // W[s * nalc + k]
    const int64_t *pdst = p.pairDst + ri.pairOff;
    const int T = (nalg + kUbT - 1) / kUbT;
    for (int ti = 0; ti < T; ++ti)
        for (int tj = 0; tj <= ti; ++tj) {
            double acc[4][4] = {};
            for (int k0 = 0; k0 < nalc; k0 += kUbK) {
                for (int e = tid; e < kUbT * kUbK; e += blockDim.x) {
                    const int rr = e / kUbK, kk = e % kUbK;
                    const int a = ti * kUbT + rr, k = k0 + kk;
                    ws[kk][rr] = (a < nalg && k < nalc) ? W[(int64_t)a * nalc + k] : 0.0;
                    const int kb = e / kUbT, cb = e % kUbT;
                    const int b = tj * kUbT + cb, k2 = k0 + kb;
                    bs[kb][cb] = (b < nalg && k2 < nalc) ? B[(int64_t)k2 * nalg + b] : 0.0;
                }
                __syncthreads();
#pragma unroll
                for (int kk = 0; kk < kUbK; ++kk) {
                    double av[4], bv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) { av[q] = ws[kk][ty * 4 + q]; bv[q] = bs[kk][tx * 4 + q]; }
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = __fma_rn(av[i], bv[j], acc[i][j]);
                }
                __syncthreads();
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int a = ti * kUbT + ty * 4 + i, b = tj * kUbT + tx * 4 + j;
                    if (a >= nalg || b > a) continue;
                    const int qa = gidx[a], qb = gidx[b];
                    const int ii = a - goffs[qa], jj = b - goffs[qb];
                    const int64_t e = qa == qb ? (int64_t)ii * (ii + 1) / 2 + jj
                                               : (int64_t)ii * (goffs[qb + 1] - goffs[qb]) + jj;
                    p.stage[pdst[qa * (qa + 1) / 2 + qb] + e] += acc[i][j];
                }
        }
}
}  // namespace

cudaError_t launch_update_big(const FitParams &p, cudaStream_t s) {
    const int64_t n = p.r1 - p.r0;
    if (n <= 0) return cudaSuccess;
    k_update_big<<<(unsigned)n, 256, sizeof(int32_t) * std::max(p.nalgmax, 1), s>>>(p);
    return cudaGetLastError();
}

int fit_smem_per_warp(const FitParams &p) {
    return (int)warp_bytes(p.wmax, p.neqmax, p.nalcmax, p.nalgmax, p.bandmax, p.bdrmax, p.ngrpmax,
                           p.bigMode != 0);
}

// warps per CTA so that one CTA fits the 227 KB of shared memory (at most
// p.wpc when that is set; one for the one-record-per-block form)
int fit_warps_per_cta(const FitParams &p) {
    const int per = fit_smem_per_warp(p);
    int wpc = p.onePerBlock ? 1 : (p.wpc > 0 ? std::min(p.wpc, MPG_WARPS_FIT) : MPG_WARPS_FIT);
    while (wpc > 1 && (int64_t)per * wpc > 220 * 1024) wpc--;
    return (int64_t)per * wpc > 220 * 1024 ? 0 : wpc;
}

cudaError_t launch_fit(const FitParams &p, int nsm, int maxPerSM, cudaStream_t s) {
    const int per = fit_smem_per_warp(p);
    void (*kern)(FitParams, int) = p.bigMode ? k_fit<true> : k_fit<false>;
    const int wpc = fit_warps_per_cta(p);
    if (wpc < 1) return cudaErrorInvalidConfiguration;
    const int bytes = per * wpc;
    cudaError_t e = smem_optin((const void *)kern);
    if (e != cudaSuccess) return e;
    int perSM = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, 32 * wpc, bytes);
    if (perSM < 1) perSM = 1;
    if (maxPerSM > 0 && perSM > maxPerSM) perSM = maxPerSM;
    int64_t nrec = p.r1 - p.r0;
    int64_t grid = (int64_t)nsm * perSM;
    int64_t need = (nrec + wpc - 1) / wpc;
    if (grid > need || p.onePerBlock) grid = need;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, 32 * wpc, bytes, s>>>(p, per);
    return cudaGetLastError();
}
