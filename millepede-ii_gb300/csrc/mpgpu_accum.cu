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

// Work item = (block (I, J <= I) of the global matrix, a record-ordered
// range of the records containing both groups).  The fit kernel writes the
// part of each record's update that falls in a block to the staging position
// base + k * nel, k the record's rank among the block's records of the chunk
// (elements row-major, lower triangle on diagonal blocks), so an item is one
// contiguous cnt x nel array.
//
// Flat mode (L = lcm(32, nel) <= kFlatMax): the warp streams the array as
// flat words f = lane + 32 k; word f belongs to element f mod nel and is
// added to the shared-memory slot f mod L, which the same lane always owns.
// Every lane does useful work on every load whatever nel is, and each slot
// sums its records in record order.  The L / nel slots of an element are
// then added in slot order.  Larger blocks: lane per element, records in
// order.  Blocks crossed by many tracks are split into several items whose
// sums are added in item order by k_acc_block_reduce.  Item boundaries are
// fixed, so every element receives its sum in the same order on every run.
// Rejected records carry zeros.
constexpr int kAccWarps = 8;
constexpr int kFlatMax = 768;   // slots per warp (6 KB)
constexpr int kLaneEl = 4;      // element accumulators per lane (128 elements per pass)
constexpr int kUnroll = 4;      // loads issued ahead of the adds
constexpr int kTileV = 8;       // vector elements per pass

__host__ __device__ inline int gcd32(int nel) {
    int g = 32;
    while ((nel % g) != 0) g >>= 1;
    return g;
}

// element t of a block (row-major, lower triangle when diagonal) -> (ii, jj)
__device__ __forceinline__ void blk_elem(int32_t t, bool diag, int32_t nj, int32_t &ii, int32_t &jj) {
    if (diag) {
        int32_t r = (int32_t)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
        while (r > 0 && r * (r + 1) / 2 > t) r--;
        while ((r + 1) * (r + 2) / 2 <= t) r++;
        ii = r;
        jj = t - r * (r + 1) / 2;
    } else {
        ii = t / nj;
        jj = t - ii * nj;
    }
}

__device__ __forceinline__ void blk_store(const AccParams &p, int32_t blk, int64_t slot, int32_t t,
                                          bool diag, int32_t ia, int32_t ja, int32_t nj, double sum) {
    if (slot >= 0) {
        p.partial[slot * p.pstride + t] = sum;
        return;
    }
    int32_t ii, jj;
    blk_elem(t, diag, nj, ii, jj);
    if (p.matsto == 2) {
        if (diag && ii == jj) p.matD[ia + ii] -= sum;
        else p.matD[p.bkOff[blk] + (int64_t)ii * p.bkLd[blk] + jj] -= sum;
    } else {
        const int64_t gi = ia + ii + 1, gj = ja + jj + 1;
        p.matD[(gi * gi - gi) / 2 + gj - 1] -= sum;
    }
}

// lane-per-element pass over nq (1..kLaneEl) accumulators per lane
template <int NQ>
__device__ __forceinline__ void acc_lane_elements(const AccParams &p, const double *col, int32_t cnt,
                                                  int32_t nel, int32_t lim, int32_t t, int32_t blk,
                                                  int64_t slot, bool diag, int32_t ia, int32_t ja,
                                                  int32_t nj) {
    double a[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) a[q] = 0.0;
    int32_t r = 0;
    for (; r + kUnroll <= cnt; r += kUnroll) {
        double v[kUnroll][NQ];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int q = 0; q < NQ; ++q)
                v[u][q] = 32 * q < lim ? __ldg(col + (int64_t)(r + u) * nel + 32 * q) : 0.0;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int q = 0; q < NQ; ++q) a[q] += v[u][q];
    }
    for (; r < cnt; ++r)
#pragma unroll
        for (int q = 0; q < NQ; ++q)
            if (32 * q < lim) a[q] += __ldg(col + (int64_t)r * nel + 32 * q);
#pragma unroll
    for (int q = 0; q < NQ; ++q)
        if (32 * q < lim) blk_store(p, blk, slot, t + 32 * q, diag, ia, ja, nj, a[q]);
}

__global__ void __launch_bounds__(32 * kAccWarps) k_acc_blocks(AccParams p) {
    extern __shared__ __align__(16) double accs[];
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    double *acc = accs + wib * kFlatMax;
    const int64_t w = (int64_t)blockIdx.x * kAccWarps + wib;
    const int64_t nw = (int64_t)gridDim.x * kAccWarps;
    for (int64_t it = p.item0 + w; it < p.item0 + p.nitem; it += nw) {
        const int32_t blk = p.itBlk[it];
        const int32_t I = p.bkI[blk], J = p.bkJ[blk];
        const int32_t ia = p.aig[I - 1] - 1, np = p.aig[I] - p.aig[I - 1];
        const int32_t ja = p.aig[J - 1] - 1, nj = p.aig[J] - p.aig[J - 1];
        const bool diag = I == J;
        const int32_t nel = diag ? np * (np + 1) / 2 : np * nj;
        const int64_t slot = p.itSlot[it];
        const int32_t cnt = p.itCnt[it];
        const double *src = p.stage + p.itBase[it];
        const int32_t L = 32 * (nel / gcd32(nel));
        // FP64 adds issued per warp: flat ~ cnt nel / 32 + L / nel (slot
        // reduction), lane per element cnt ceil(nel / 32)
        const int64_t costFlat = ((int64_t)cnt * nel + 31) / 32 + L / nel;
        const int64_t costLane = (int64_t)cnt * ((nel + 31) / 32);
        if (L <= kFlatMax && costFlat < costLane) {
            const int32_t R = L / 32;
            for (int32_t q = ln; q < L; q += 32) acc[q] = 0.0;
            __syncwarp();
            const int64_t total = (int64_t)cnt * nel;
            double *mine = acc + ln;
            int32_t kr = 0;
            int64_t f = ln;
            for (; f + 32 * (kUnroll - 1) < total; f += 32 * kUnroll) {
                double v[kUnroll];
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) v[u] = __ldg(src + f + 32 * u);
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) {
                    mine[32 * kr] += v[u];
                    kr = kr + 1 == R ? 0 : kr + 1;
                }
            }
            for (; f < total; f += 32) {
                mine[32 * kr] += __ldg(src + f);
                kr = kr + 1 == R ? 0 : kr + 1;
            }
            __syncwarp();
            const int32_t per = L / nel;
            for (int32_t t = ln; t < nel; t += 32) {
                double sum = 0.0;
                for (int32_t m = 0; m < per; ++m) sum += acc[t + nel * m];
                blk_store(p, blk, slot, t, diag, ia, ja, nj, sum);
            }
            __syncwarp();
            continue;
        }
        for (int32_t t0 = 0; t0 < nel; t0 += 32 * kLaneEl) {
            const int32_t lim = nel - t0 - ln;  // element q of the lane valid when 32 q < lim
            const int32_t nq = min(kLaneEl, (nel - t0 + 31) / 32);
            const double *col = src + t0 + ln;
            if (nq == 1) acc_lane_elements<1>(p, col, cnt, nel, lim, t0 + ln, blk, slot, diag, ia, ja, nj);
            else if (nq == 2) acc_lane_elements<2>(p, col, cnt, nel, lim, t0 + ln, blk, slot, diag, ia, ja, nj);
            else if (nq == 3) acc_lane_elements<3>(p, col, cnt, nel, lim, t0 + ln, blk, slot, diag, ia, ja, nj);
            else acc_lane_elements<4>(p, col, cnt, nel, lim, t0 + ln, blk, slot, diag, ia, ja, nj);
        }
    }
}

__global__ void __launch_bounds__(256) k_acc_block_reduce(AccParams p) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = p.red0 + w; r < p.red0 + p.nred; r += nw) {
        const int32_t blk = p.rdBlk[r];
        const int64_t s0 = p.rdSlot0[r];
        const int32_t ns = p.rdN[r];
        const int32_t I = p.bkI[blk], J = p.bkJ[blk];
        const int32_t ia = p.aig[I - 1] - 1, np = p.aig[I] - p.aig[I - 1];
        const int32_t ja = p.aig[J - 1] - 1, nj = p.aig[J] - p.aig[J - 1];
        const bool diag = I == J;
        // element order of k_acc_blocks: rows ii, columns jj (jj <= ii on the diagonal)
        int32_t q = 0;
        for (int32_t ii = 0; ii < np; ++ii)
            for (int32_t jj = 0; jj < nj; ++jj) {
                if (diag && jj > ii) continue;
                if ((q & 31) == ln) {
                    double sum = 0.0;
                    for (int32_t k = 0; k < ns; ++k) sum += p.partial[(s0 + k) * p.pstride + q];
                    if (p.matsto == 2) {
                        if (diag && ii == jj) p.matD[ia + ii] -= sum;
                        else p.matD[p.bkOff[blk] + (int64_t)ii * p.bkLd[blk] + jj] -= sum;
                    } else {
                        const int64_t gi = ia + ii + 1, gj = ja + jj + 1;
                        p.matD[(gi * gi - gi) / 2 + gj - 1] -= sum;
                    }
                }
                q++;
            }
    }
}

// vector slices and counts: one CTA of 256 threads per row group; thread t
// sums the accepted records t, t+256, ... of the group in registers (loads
// of four entries issued together), then the threads' sums are added by a
// fixed tree (warp shuffles, then the eight warp sums in order), so every
// loop adds in the same order
constexpr int kVecThreads = 256;
__global__ void __launch_bounds__(kVecThreads) k_acc_vector(AccParams p) {
    __shared__ double wsum[kVecThreads / 32][kTileV];
    __shared__ long long wcnt[kVecThreads / 32][kTileV];
    const int tid = threadIdx.x, ln = tid & 31, wib = tid >> 5;
    for (int64_t I = 1 + blockIdx.x; I <= p.nG; I += gridDim.x) {
        const int64_t e0 = p.vStart[I - 1], e1 = p.vStart[I];
        if (e1 <= e0) continue;
        const int32_t ia = p.aig[I - 1] - 1, np = p.aig[I] - p.aig[I - 1];
        for (int32_t t0 = 0; t0 < np; t0 += kTileV) {
            const int32_t tn = np - t0 < kTileV ? np - t0 : kTileV;
            double acc[kTileV];
            long long cn[kTileV];
#pragma unroll
            for (int q = 0; q < kTileV; ++q) { acc[q] = 0.0; cn[q] = 0; }
            for (int64_t e = e0 + tid; e < e1; e += 4 * kVecThreads) {
                int64_t vo[4];
                bool ok[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t eu = e + (int64_t)u * kVecThreads;
                    const int64_t ent = eu < e1 ? p.vEntries[eu] : -1;
                    vo[u] = ent & ((int64_t(1) << 40) - 1);
                    ok[u] = ent >= 0 && p.status[ent >> 40] == 0;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (!ok[u]) continue;
#pragma unroll
                    for (int q = 0; q < kTileV; ++q) {
                        if (q >= tn) break;
                        acc[q] += p.vstage[vo[u] + t0 + q];
                        cn[q] += p.slotCnt[vo[u] + t0 + q];
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kTileV; ++q) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
                    cn[q] += __shfl_xor_sync(0xffffffffu, cn[q], o);
                }
            }
            if (ln == 0)
#pragma unroll
                for (int q = 0; q < kTileV; ++q) { wsum[wib][q] = acc[q]; wcnt[wib][q] = cn[q]; }
            __syncthreads();
            if (tid < tn) {
                double v = 0.0;
                long long c = 0;
                for (int w = 0; w < kVecThreads / 32; ++w) { v += wsum[w][tid]; c += wcnt[w][tid]; }
                p.gvec[ia + t0 + tid] += v;
                p.gcnt[ia + t0 + tid] += c;
            }
            __syncthreads();
        }
    }
}

// Per-record outcome -> loop statistics.  Integer quantities by atomics
// (exact); the fractional chi2 parts and the weighted ndf by a fixed-shape
// tree (block partials in a fixed order, then one block).
__global__ void k_stats_partial(StatParams p, double *part, float *fpart) {
    __shared__ double sf[256], sw[256];
    // integer counters of the block (exact), one global atomic each at the end
    __shared__ unsigned long long ic[9];
    extern __shared__ unsigned long long fc[];   // 2 * nfiles: accepted, ndf per file
    for (int k = threadIdx.x; k < 9; k += blockDim.x) ic[k] = 0;
    for (int k = threadIdx.x; k < 2 * p.nfiles; k += blockDim.x) fc[k] = 0;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double frac = 0.0, wndf = 0.0;
    int st = -1, file = 0;
    if (i < p.nrec) {
        st = p.status[i];
        file = p.rec[i].file;
        const double dw = p.fileWeight ? p.fileWeight[file - 1] : 1.0;
        const int ndfa = p.ndfadd[i];
        const double c2 = p.chi2add[i];
        if (st >= 1 && st <= 6) atomicAdd(&ic[1 + st], 1ull);
        if (st == 0) {
            atomicAdd(&ic[8], 1ull);
            atomicAdd(&fc[file - 1], 1ull);
            atomicAdd(&fc[p.nfiles + file - 1], (unsigned long long)(long long)ndfa);
        }
        if (ndfa > 0 || c2 != 0.0) {
            const double add = c2 * dw;
            const long long nadd = (long long)add;
            atomicAdd(&ic[0], (unsigned long long)nadd);
            atomicAdd(&ic[1], (unsigned long long)(long long)ndfa);
            frac = add - (double)nadd;
            wndf = (double)ndfa * dw;
        }
    }
    sf[threadIdx.x] = frac;
    sw[threadIdx.x] = wndf;
    __syncthreads();
    for (int k = threadIdx.x; k < 9; k += blockDim.x)
        if (ic[k]) atomicAdd((unsigned long long *)&p.iout[k], ic[k]);
    for (int k = threadIdx.x; k < 2 * p.nfiles; k += blockDim.x)
        if (fc[k]) atomicAdd((unsigned long long *)&p.iout[9 + k], fc[k]);
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
        if (st == 0 && file == f + 1) v = p.chndf[i];
        sf[threadIdx.x] = (double)v;
        __syncthreads();
        for (int s = 128; s > 0; s >>= 1) {
            if (threadIdx.x < s) sf[threadIdx.x] = (double)((float)sf[threadIdx.x] + (float)sf[threadIdx.x + s]);
            __syncthreads();
        }
        if (threadIdx.x == 0) fpart[(int64_t)f * gridDim.x + blockIdx.x] = (float)sf[0];
    }
}

// block partials summed by 256 threads: thread t adds partials t, t+256,
// ... in order, then a fixed tree (warp shuffles, warp sums in order)
__global__ void __launch_bounds__(256) k_stats_final(StatParams p, const double *part, const float *fpart,
                                                     int nblk) {
    __shared__ double ws[8][2];
    __shared__ float wf[8];
    const int tid = threadIdx.x, ln = tid & 31, wib = tid >> 5;
    double f = 0.0, w = 0.0;
    for (int b = tid; b < nblk; b += 256) {
        f += part[2 * b];
        w += part[2 * b + 1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        f += __shfl_xor_sync(0xffffffffu, f, o);
        w += __shfl_xor_sync(0xffffffffu, w, o);
    }
    if (ln == 0) { ws[wib][0] = f; ws[wib][1] = w; }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, c = 0.0;
        for (int q = 0; q < 8; ++q) { a += ws[q][0]; c += ws[q][1]; }
        p.out[0] = a;
        p.out[1] = c;
    }
    for (int fi = 0; fi < p.nfiles; ++fi) {
        __syncthreads();
        float sfl = 0.0f;
        for (int b = tid; b < nblk; b += 256) sfl += fpart[(int64_t)fi * nblk + b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sfl += __shfl_xor_sync(0xffffffffu, sfl, o);
        if (ln == 0) wf[wib] = sfl;
        __syncthreads();
        if (tid == 0) {
            float a = 0.0f;
            for (int q = 0; q < 8; ++q) a += wf[q];
            p.fout[fi] = a;
        }
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
    if (p.icalcm == 1 && p.nitem > 0) {
        const int smem = kAccWarps * kFlatMax * (int)sizeof(double);
        cudaError_t e = smem_optin((const void *)k_acc_blocks);
        if (e != cudaSuccess) return e;
        int64_t blocks = (p.nitem + kAccWarps - 1) / kAccWarps;
        const int64_t maxb = (int64_t)nsm * 4;
        if (blocks > maxb) blocks = maxb;
        k_acc_blocks<<<(unsigned)blocks, 32 * kAccWarps, smem, s>>>(p);
        if (p.nred > 0) {
            int64_t rb = (p.nred + 7) / 8;
            if (rb > (int64_t)nsm * 8) rb = (int64_t)nsm * 8;
            k_acc_block_reduce<<<(unsigned)rb, 256, 0, s>>>(p);
        }
    }
    int64_t vb = p.nG;
    if (vb > (int64_t)nsm * 16) vb = (int64_t)nsm * 16;
    if (vb < 1) vb = 1;
    k_acc_vector<<<(unsigned)vb, kVecThreads, 0, s>>>(p);
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
    const size_t fsm = sizeof(unsigned long long) * 2 * (size_t)(p.nfiles > 0 ? p.nfiles : 1);
    if (nblk > 0) k_stats_partial<<<nblk, 256, fsm, s>>>(p, part, fpart);
    k_stats_final<<<1, 256, 0, s>>>(p, part, fpart, nblk);
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
