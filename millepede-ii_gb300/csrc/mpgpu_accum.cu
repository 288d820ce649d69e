// mpgpu_accum.cu -- deterministic accumulation of the per-record updates
// into the global matrix and vector, the per-loop statistics and mupdat.
//
// Owner computes: the contributions to one parameter group's block row of
// the lower-triangular global matrix (and its slice of the vector) are
// summed by fixed work items in record order, then the items of a row are
// combined in item order.  Every element therefore receives its sum in the
// same order on every run, independent of scheduling, and no atomics are
// used on floating-point data.  This replaces the write cache and the
// row-owner flush of loopbf/mgupdt (pede.f90:4280-4421, 3219-3357).
#include <cuda_runtime.h>

#include "mpgpu_ctx.h"

// ijpgrp, pede.f90:5371-5461 (single storage precision)
__device__ int64_t d_ijpgrp(int32_t itema, int32_t itemb, int32_t nG, const int32_t *aig,
                            const int64_t *off, const int32_t *col, int32_t *lr) {
    const int32_t item1 = itema > itemb ? itema : itemb;
    const int32_t item2 = itema > itemb ? itemb : itema;
    *lr = 0;
    if (item2 <= 0 || item1 > nG) return 0;
    const int32_t *npgrp = aig - 1;  // 1-based
    const int32_t *c1 = col - 1;
    const int32_t np = npgrp[item1 + 1] - npgrp[item1];
    const int64_t kk = off[2 * (item1 - 1)], ll = off[2 * (item1 - 1) + 1];
    int64_t kl = 1, ku = off[2 * item1] - kk, k;
    if (ku <= 0) return 0;
    if (c1[kk + 1] == 0) {  // compressed: regions (offset, first group) pairs
        kl = 2;
        ku = ku - 2;
        if (ku < kl) return 0;
        int32_t jtem;
        for (int guard = 0; guard < 64; ++guard) {
            k = 2 * ((kl + ku) / 4);
            jtem = c1[kk + k];
            const int32_t jtemn = c1[kk + k + 2];
            if (item2 >= jtem && item2 < jtemn) {
                *lr = c1[kk + k + 1] - c1[kk + k - 1];
                if (npgrp[item2] - npgrp[jtem] >= *lr) return 0;
                return ll + (int64_t)c1[kk + k - 1] * np + npgrp[item2] - npgrp[jtem] + 1;
            }
            if (item2 < jtem) ku = k - 2;
            else if (item2 >= jtemn) kl = k + 2;
            if (kl > ku) return 0;
        }
        return 0;
    }
    const int32_t itemc = npgrp[item2];
    *lr = (int32_t)ku;
    for (int guard = 0; guard < 64; ++guard) {
        k = (kl + ku) / 2;
        const int32_t jtem = c1[kk + k];
        if (itemc == jtem) return ll + k;
        if (itemc < jtem) ku = k - 1;
        else kl = k + 1;
        if (kl > ku) return 0;
    }
    return 0;
}

namespace {

// Work item = (row group I, a record-ordered range of the records that
// contain I).  One warp sums, in record order, the rows of group I of every
// accepted record's update into a private partial block row (dense row
// layout of I: the stored column blocks side by side) and the vector slice.
// Hot row groups (modules crossed by many tracks) are split into several
// items, so the work is balanced over the GPU; k_acc_reduce then adds the
// partials of a row group in item order.  Fixed item boundaries make the
// result independent of scheduling.
constexpr int kAccWarps = 8;
constexpr int kAccSmem = 768;    // doubles of shared-memory partial per warp

__global__ void __launch_bounds__(32 * kAccWarps) k_acc_items(AccParams p) {
    extern __shared__ __align__(16) double sacc[];
    __shared__ int32_t s_off[kAccWarps][MPG_NGRP_MAX + 2];
    __shared__ int32_t s_col[kAccWarps][MPG_NGRP_MAX + 1];
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * kAccWarps + wib;
    const int64_t nw = (int64_t)gridDim.x * kAccWarps;
    double *mine = sacc + (int64_t)wib * kAccSmem;
    for (int64_t it = p.item0 + w; it < p.item0 + p.nitem; it += nw) {
        const int32_t I = p.itRow[it];
        const int32_t ia = p.aig[I - 1] - 1, np = p.aig[I] - p.aig[I - 1];
        const int32_t width = p.rowWidth[I - 1];
        const int64_t psz = (int64_t)np * width, total = psz + 2 * np;
        double *P = total <= kAccSmem ? mine : p.partial + p.itPOff[it];
        for (int64_t q = ln; q < total; q += 32) P[q] = 0.0;
        __syncwarp();
        const int64_t kb0 = p.matsto == 2 ? p.rowBlk0[I - 1] : 0;
        const int64_t kb1 = p.matsto == 2 ? p.rowBlk0[I] : 0;
        for (int64_t e = p.itE0[it]; e < p.itE1[it]; ++e) {
            const int64_t ent = p.entries[e];
            const int64_t r = ent >> 8;
            const int a = (int)(ent & 0xff);
            if (p.status[r] != 0) continue;
            const int64_t updOff = p.rec[r].updOff, grpOff = p.rec[r].grpOff;
            const int64_t slotOff = p.rec[r].slotOff;
            for (int b = ln; b <= a; b += 32) {
                const int32_t J = p.grpId[grpOff + b];
                s_off[wib][b] = p.grpSlot[grpOff + b];
                int32_t col = -1;
                if (p.matsto == 2) {
                    int64_t lo = kb0, hi = kb1 - 1;
                    while (lo <= hi) {
                        const int64_t mid = (lo + hi) >> 1;
                        const int32_t jm = p.blkJ[mid];
                        if (jm == J) { col = p.blkCol[mid]; break; }
                        if (jm < J) lo = mid + 1; else hi = mid - 1;
                    }
                    if (col < 0) *p.errFlag = 23;
                } else {
                    col = p.aig[J - 1] - 1;
                }
                s_col[wib][b] = col < 0 ? 0 : col;
            }
            __syncwarp();
            if (ln == 0) s_off[wib][a + 1] = s_off[wib][a] + np;
            __syncwarp();
            const int32_t offa = s_off[wib][a];
            if (p.icalcm == 1) {
                const int64_t s0 = (int64_t)offa * (offa + 1) / 2;
                const int64_t s1 = (int64_t)(offa + np) * (offa + np + 1) / 2;
                const double *U = p.stage + updOff;
                int ra = offa, cb = ln;
                while (cb > ra) { cb -= ra + 1; ra++; }
                int b = 0;
                for (int64_t idx = s0 + ln; idx < s1; idx += 32) {
                    while (cb >= s_off[wib][b + 1]) b++;
                    while (cb < s_off[wib][b]) b--;
                    const int ii = ra - offa, jj = cb - s_off[wib][b];
                    P[(int64_t)ii * width + s_col[wib][b] + jj] += U[idx];
                    cb += 32;
                    while (cb > ra) { cb -= ra + 1; ra++; }
                }
            }
            for (int ii = ln; ii < np; ii += 32) {
                P[psz + ii] += p.vstage[slotOff + offa + ii];
                P[psz + np + ii] += (double)p.slotCnt[slotOff + offa + ii];
            }
            __syncwarp();
        }
        if (total <= kAccSmem) {
            double *G = p.partial + p.itPOff[it];
            for (int64_t q = ln; q < total; q += 32) G[q] = P[q];
        }
        __syncwarp();
    }
}

// Warp per row group: partials of its items in item (= record) order,
// subtracted from the block row of the global matrix; vector and counts.
__global__ void __launch_bounds__(256) k_acc_reduce(AccParams p) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t I = 1 + w; I <= p.nG; I += nw) {
        const int64_t i0 = p.rowItem0[I - 1], i1 = p.rowItem0[I];
        if (i1 <= i0) continue;
        const int32_t ia = p.aig[I - 1] - 1, np = p.aig[I] - p.aig[I - 1];
        const int32_t width = p.rowWidth[I - 1];
        const int64_t psz = (int64_t)np * width;
        if (p.icalcm == 1) {
            if (p.matsto == 2) {
                for (int64_t k = p.rowBlk0[I - 1]; k < p.rowBlk0[I]; ++k) {
                    const int32_t J = p.blkJ[k];
                    const int32_t nj = p.aig[J] - p.aig[J - 1];
                    const int64_t boff = p.blkOff[k];
                    const int32_t ld = p.blkLd[k], col0 = p.blkCol[k];
                    for (int q = ln; q < np * nj; q += 32) {
                        const int ii = q / nj, jj = q - ii * nj;
                        if (J == I && jj > ii) continue;
                        double sum = 0.0;
                        for (int64_t it = i0; it < i1; ++it)
                            sum += p.partial[p.itPOff[it] + (int64_t)ii * width + col0 + jj];
                        if (J == I && jj == ii) p.matD[ia + ii] -= sum;
                        else p.matD[boff + (int64_t)ii * ld + jj] -= sum;
                    }
                }
            } else {
                for (int64_t q = ln; q < psz; q += 32) {
                    const int64_t ii = q / width, col = q - ii * width;
                    const int64_t gi = ia + ii + 1, gj = col + 1;
                    if (gj > gi) continue;
                    double sum = 0.0;
                    for (int64_t it = i0; it < i1; ++it) sum += p.partial[p.itPOff[it] + q];
                    p.matD[(gi * gi - gi) / 2 + gj - 1] -= sum;
                }
            }
        }
        for (int ii = ln; ii < np; ii += 32) {
            double v = 0.0, cn = 0.0;
            for (int64_t it = i0; it < i1; ++it) {
                v += p.partial[p.itPOff[it] + psz + ii];
                cn += p.partial[p.itPOff[it] + psz + np + ii];
            }
            p.gvec[ia + ii] += v;
            p.gcnt[ia + ii] += (int64_t)cn;
        }
    }
}

// Per-record outcome -> loop statistics.  Integer quantities by atomics
// (exact); the fractional chi2 parts and the weighted ndf by a fixed-shape
// tree (block partials in a fixed order, then one block).
__global__ void k_stats_partial(StatParams p, double *part, float *fpart) {
    __shared__ double sf[256], sw[256];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double frac = 0.0, wndf = 0.0;
    if (i < p.nrec) {
        const int st = p.status[i];
        const RecInfo ri = p.rec[i];
        const double dw = p.fileWeight ? p.fileWeight[ri.file - 1] : 1.0;
        if (st >= 1 && st <= 6) atomicAdd((unsigned long long *)&p.iout[1 + st], 1ull);
        if (st == 0) {
            atomicAdd((unsigned long long *)&p.iout[8], 1ull);
            atomicAdd((unsigned long long *)&p.iout[9 + ri.file - 1], 1ull);
            atomicAdd((unsigned long long *)&p.iout[9 + p.nfiles + ri.file - 1],
                      (unsigned long long)(long long)p.ndfadd[i]);
        }
        if (p.ndfadd[i] > 0 || p.chi2add[i] != 0.0) {
            const double add = p.chi2add[i] * dw;
            const long long nadd = (long long)add;
            atomicAdd((unsigned long long *)&p.iout[0], (unsigned long long)nadd);
            atomicAdd((unsigned long long *)&p.iout[1], (unsigned long long)(long long)p.ndfadd[i]);
            frac = add - (double)nadd;
            wndf = (double)p.ndfadd[i] * dw;
        }
    }
    sf[threadIdx.x] = frac;
    sw[threadIdx.x] = wndf;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sf[threadIdx.x] += sf[threadIdx.x + s];
            sw[threadIdx.x] += sw[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = sf[0];
        part[2 * blockIdx.x + 1] = sw[0];
    }
    // per-file chi2/ndf sums (single precision like the reference's cfd)
    for (int f = 0; f < p.nfiles; ++f) {
        __syncthreads();
        float v = 0.0f;
        if (i < p.nrec && p.status[i] == 0 && p.rec[i].file == f + 1) v = p.chndf[i];
        sf[threadIdx.x] = (double)v;
        __syncthreads();
        for (int s = 128; s > 0; s >>= 1) {
            if (threadIdx.x < s) sf[threadIdx.x] = (double)((float)sf[threadIdx.x] + (float)sf[threadIdx.x + s]);
            __syncthreads();
        }
        if (threadIdx.x == 0) fpart[(int64_t)f * gridDim.x + blockIdx.x] = (float)sf[0];
    }
}

__global__ void k_stats_final(StatParams p, const double *part, const float *fpart, int nblk) {
    if (threadIdx.x != 0) return;
    double f = 0.0, w = 0.0;
    for (int b = 0; b < nblk; ++b) {
        f += part[2 * b];
        w += part[2 * b + 1];
    }
    p.out[0] = f;
    p.out[1] = w;
    for (int fi = 0; fi < p.nfiles; ++fi) {
        float s = 0.0f;
        for (int b = 0; b < nblk; ++b) s += fpart[(int64_t)fi * nblk + b];
        p.fout[fi] = s;
    }
}

__global__ void k_mupdat(int32_t n, const int32_t *iv, const int32_t *jv, const double *add,
                         int32_t matsto, int32_t nG, const int32_t *aig, const int32_t *p2g,
                         const int64_t *off, const int32_t *col, double *matD, int32_t nVar,
                         int32_t *errFlag) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int32_t q = 0; q < n; ++q) {
        const int32_t i = iv[q], j = jv[q];
        const double a = add[q];
        if (i <= 0 || j <= 0 || a == 0.0) continue;
        if (i > nVar || j > nVar) { *errFlag = 23; continue; }
        const int64_t ia = i > j ? i : j, ja = i > j ? j : i;
        if (matsto == 2) {
            if (ia == ja) { matD[ia - 1] += a; continue; }
            int32_t lr;
            const int32_t g1 = p2g[ia - 1], g2 = p2g[ja - 1];
            const int64_t ij = d_ijpgrp(g1, g2, nG, aig, off, col, &lr);
            if (ij == 0) continue;  // pair not stored (suppressed)
            matD[ij + (ja - aig[g2 - 1]) + (ia - aig[g1 - 1]) * (int64_t)lr - 1] += a;
        } else {
            matD[(ia * ia - ia) / 2 + ja - 1] += a;
        }
    }
}

}  // namespace

cudaError_t launch_accumulate(const AccParams &p, int nsm, cudaStream_t s) {
    const int smem = kAccWarps * kAccSmem * (int)sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(k_acc_items, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (p.nitem > 0) {
        int64_t blocks = (p.nitem + kAccWarps - 1) / kAccWarps;
        const int64_t maxb = (int64_t)nsm * 4;
        if (blocks > maxb) blocks = maxb;
        k_acc_items<<<(unsigned)blocks, 32 * kAccWarps, smem, s>>>(p);
    }
    int64_t rb = (p.nG + 7) / 8;
    if (rb > (int64_t)nsm * 8) rb = (int64_t)nsm * 8;
    if (rb < 1) rb = 1;
    k_acc_reduce<<<(unsigned)rb, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_stats(const StatParams &p, cudaStream_t s) {
    const int nblk = (int)((p.nrec + 255) / 256);
    double *part = nullptr;
    float *fpart = nullptr;
    cudaError_t e = cudaMallocAsync(&part, sizeof(double) * 2 * (nblk + 1), s);
    if (e != cudaSuccess) return e;
    e = cudaMallocAsync(&fpart, sizeof(float) * (size_t)(p.nfiles > 0 ? p.nfiles : 1) * (nblk + 1), s);
    if (e != cudaSuccess) return e;
    if (nblk > 0) k_stats_partial<<<nblk, 256, 0, s>>>(p, part, fpart);
    k_stats_final<<<1, 32, 0, s>>>(p, part, fpart, nblk);
    cudaFreeAsync(part, s);
    cudaFreeAsync(fpart, s);
    return cudaGetLastError();
}

cudaError_t launch_mupdat(int32_t n, const int32_t *i, const int32_t *j, const double *add,
                          const DevJob &d, int32_t *errFlag, cudaStream_t s) {
    k_mupdat<<<1, 32, 0, s>>>(n, i, j, add, d.matsto, d.nG, d.aig, d.p2g, d.off, d.col, d.matD,
                             d.nVar, errFlag);
    return cudaGetLastError();
}
