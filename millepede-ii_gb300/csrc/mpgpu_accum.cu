// mpgpu_accum.cu -- deterministic accumulation of the per-record updates
// into the global matrix and vector, the per-loop statistics and mupdat.
//
// Owner computes: one warp owns one parameter group (a block row of the
// lower-triangular global matrix and the matching slice of the vector) and
// walks the records that contain the group in record order.  No two warps
// write the same element and every element receives its contributions in
// record order, so the result does not depend on scheduling and no atomics
// are used on floating-point data.  This replaces the write cache and the
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

// Warp per parameter group I.  Entries (record, group position a) of this
// chunk in record order; for an accepted record the rows of group a of its
// packed update matrix (one contiguous segment) are subtracted from the
// block row of I, and its vector slice is added.
__global__ void __launch_bounds__(256) k_accumulate(AccParams p) {
    const int ln = threadIdx.x & 31;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    __shared__ int64_t s_ij[8][MPG_NGRP_MAX + 1];
    __shared__ int32_t s_lr[8][MPG_NGRP_MAX + 1];
    __shared__ int32_t s_off[8][MPG_NGRP_MAX + 2];
    __shared__ int32_t s_gf[8][MPG_NGRP_MAX + 1];
    const int wib = threadIdx.x >> 5;
    for (int64_t I = 1 + wg; I <= p.nG; I += nwarp) {
        const int32_t ia = p.aig[I - 1];           // first variable index (1-based)
        const int32_t np = p.aig[I] - ia;
        const int64_t e0 = p.eStart[I - 1], e1 = p.eStart[I];
        for (int64_t e = e0; e < e1; ++e) {
            const int64_t ent = p.entries[e];
            const int64_t r = ent >> 8;
            const int a = (int)(ent & 0xff);
            if (p.status[r] != 0) continue;
            const RecInfo ri = p.rec[r];
            // block locations of (I, J_b) for the record's groups b <= a
            for (int b = ln; b <= a; b += 32) {
                const int32_t J = p.grpId[ri.grpOff + b];
                s_off[wib][b] = p.grpSlot[ri.grpOff + b];
                s_gf[wib][b] = p.aig[J - 1];
                if (p.matsto == 2 && p.icalcm == 1) {
                    int32_t lr = 0;
                    int64_t ij = (J == I) ? -1 : d_ijpgrp((int32_t)I, J, p.nG, p.aig, p.off, p.col, &lr);
                    if (J == I) {  // diagonal block: strictly-lower part stored like others
                        ij = d_ijpgrp((int32_t)I, (int32_t)I, p.nG, p.aig, p.off, p.col, &lr);
                    }
                    s_ij[wib][b] = ij;
                    s_lr[wib][b] = lr;
                }
            }
            if (ln == 0) s_off[wib][a + 1] = s_off[wib][a] + np;
            __syncwarp();
            const int32_t offa = s_off[wib][a];
            // vector slice and counts
            for (int ii = ln; ii < np; ii += 32) {
                p.gvec[ia - 1 + ii] += p.vstage[ri.slotOff + offa + ii];
                p.gcnt[ia - 1 + ii] += p.slotCnt[ri.slotOff + offa + ii];
            }
            if (p.icalcm == 1) {
                // segment: packed rows offa .. offa+np-1, columns 0 .. row
                const int64_t s0 = (int64_t)offa * (offa + 1) / 2;
                const int64_t s1 = (int64_t)(offa + np) * (offa + np + 1) / 2;
                const double *U = p.stage + ri.updOff;
                int ra = offa, cb = ln;
                while (cb > ra) { cb -= ra + 1; ra++; }
                int b = 0;
                for (int64_t idx = s0 + ln; idx < s1; idx += 32) {
                    while (cb >= s_off[wib][b + 1]) b++;
                    while (cb < s_off[wib][b]) b--;
                    const int ii = ra - offa, jj = cb - s_off[wib][b];
                    const double u = U[idx];
                    if (p.matsto == 2) {
                        if (b == a && jj == ii) {
                            p.matD[ia - 1 + ii] -= u;
                        } else {
                            const int64_t t = s_ij[wib][b] + jj + (int64_t)ii * s_lr[wib][b] - 1;
                            if (s_ij[wib][b] <= 0) { *p.errFlag = 23; }
                            else p.matD[t] -= u;
                        }
                    } else {
                        const int64_t gi = ia + ii, gj = s_gf[wib][b] + jj;
                        p.matD[(gi * gi - gi) / 2 + gj - 1] -= u;
                    }
                    cb += 32;
                    while (cb > ra) { cb -= ra + 1; ra++; }
                }
            }
            __syncwarp();
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
    int64_t warps = p.nG;
    int64_t blocks = (warps + 7) / 8;
    int64_t maxb = (int64_t)nsm * 8;
    if (blocks > maxb) blocks = maxb;
    if (blocks < 1) blocks = 1;
    k_accumulate<<<(unsigned)blocks, 256, 0, s>>>(p);
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
