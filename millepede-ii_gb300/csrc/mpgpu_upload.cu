// mpgpu_upload.cu -- record preparation on the device (the per-record part
// of readFromBinary/prepareRecords and of loopbf's stage 1, pede.f90:1714-2075,
// 2428-2468, 3655-3741, mppar.f90:282-321).
//
// The records arrive as the Mille words (inder/glder, labels already
// translated to total indices).  Everything the data loop needs is derived
// on the GPU:
//   1. k_up_scan (one warp per record; a compact variant for typical
//      records and a large one for the records it hands over): decode the measurements, count the
//      locals, the variable global words and the distinct variable
//      parameters (sorted), form the parameter groups, check the record
//      (codes as the host checks: 20 malformed, 23 bad index, 35 incomplete
//      groups, 45 limits), choose the bordered-band structure of the local
//      system, and write the per-record counts;
//   2. exclusive scans of the counts give every table offset;
//   3. k_up_fill (one warp per record): the equation table, sorted slots,
//      per-slot word lists in equation order, group list;
//   4. k_up_pairs: the global-matrix block of every record group pair;
//   5. per chunk of records: a stable radix sort of the pairs by block puts
//      the records of one block in record order; from it the staging
//      position of every record block (block-major staging), the work items
//      of the accumulation and the vector entries per group.
// All steps are deterministic: integer counts, order-independent integer
// atomics only for histograms and maxima, and stable sorts.
#include "mpgpu_records.cuh"

namespace {

// record index of work step `it`: all records (compact) or the overflow list (large)
template <bool BIG>
__device__ __forceinline__ int64_t up_steps(const UpParams &P) {
    return BIG ? (int64_t)*P.ovCount : P.rEnd - P.rBegin;
}

template <bool BIG>
__global__ void __launch_bounds__(32 * kUpWarps, UpCap<BIG>::kMinBlocks) k_up_scan(UpParams P) {
    extern __shared__ __align__(16) char upsm[];
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    UpWarp<BIG> &W = reinterpret_cast<UpWarp<BIG> *>(upsm)[wib];
    const int64_t nwarps = (int64_t)gridDim.x * kUpWarps;
    const int64_t nsteps = up_steps<BIG>(P);
    for (int64_t it = (int64_t)blockIdx.x * kUpWarps + wib; it < nsteps; it += nwarps) {
        const int64_t r = BIG ? P.ovList[it] : P.rBegin + it;
        RecShape R = analyze<BIG>(P, r, W, true);
        if (!BIG && R.code == kOverflow) {
            if (ln == 0) P.ovList[atomicAdd(P.ovCount, 1)] = r;
            __syncwarp();
            continue;
        }
        const int file = P.recFile ? P.recFile[r] : 1;
        if (R.code == 0 && (file < 1 || file > P.nfiles)) R.code = MPGPU_ERR_BADRECORD;
        if (R.code == 0 && R.nalc > MPG_NALC_MAX) R.code = MPGPU_ERR_LIMIT;
        int mbnd = -1, mbdr = R.nalc, side = -1;
        if (R.code == 0 && R.nalc > 5) {
            // bordered band structure of the local matrix (pede.f90:3812-3874)
            const int nalc = R.nalc;
            const int32_t *in =
                R.nw <= UpCap<BIG>::kWords ? W.words : P.inder + (P.recPtr[r] - P.recPtr[0]);
            int32_t *band = reinterpret_cast<int32_t *>(W.key);
            __syncwarp();
            for (int i = ln; i < 2 * nalc + 2; i += 32) band[i] = 0;
            __syncwarp();
            for (int e = ln; e < R.neq; e += 32) {
                const int sl = W.eq[3 * e], sg = W.eq[3 * e + 1];
                for (int jq = sl + 1; jq < sg; ++jq)
                    for (int kq = sl + 1; kq <= jq; ++kq) {
                        const int ij = in[jq], ik = in[kq];
                        const int id = abs(ij - ik) + 1;
                        atomicMax(&band[id], min(ij, ik));
                        atomicMax(&band[nalc + id], min(nalc + 1 - ij, nalc + 1 - ik));
                    }
            }
            __syncwarp();
            if (ln == 0) {
                int kx = -1, kbdrx = 0, kbdr = 0;
                int64_t icmn = (int64_t)nalc * nalc * nalc;
                for (int k = nalc; k >= 2; --k) {
                    const int kbnd = k - 2;
                    kbdr = max(kbdr, band[k]);
                    const int64_t wd = kbnd + kbdr + 1;
                    const int64_t icost = 6 * (int64_t)(nalc - kbdr) * wd * wd + 2 * (int64_t)kbdr * kbdr * kbdr;
                    if (icost < icmn) { icmn = icost; kx = k; kbdrx = kbdr; side = 1; }
                }
                if (kx < 0) {
                    kbdr = 0;
                    for (int k = nalc; k >= 2; --k) {
                        const int kbnd = k - 2;
                        kbdr = max(kbdr, band[k + nalc]);
                        const int64_t wd = kbnd + kbdr + 1;
                        const int64_t icost = 6 * (int64_t)(nalc - kbdr) * wd * wd + 2 * (int64_t)kbdr * kbdr * kbdr;
                        if (icost < icmn) { icmn = icost; kx = k; kbdrx = kbdr; side = 2; }
                    }
                }
                if (kx > 0) { mbnd = kx - 2; mbdr = kbdrx; }
                else side = -1;
                W.misc[1] = mbnd; W.misc[2] = mbdr; W.misc[3] = side;
            }
            __syncwarp();
            mbnd = W.misc[1]; mbdr = W.misc[2]; side = W.misc[3];
        }
        if (ln == 0) {
            const int64_t n1 = P.nrec + 1;
            if (R.code != 0) {
                atomicMin(P.err, ((unsigned long long)r << 8) | (unsigned long long)R.code);
                for (int k = 0; k < 6; ++k) P.cnt[k * n1 + r] = 0;
            } else {
                RecInfo ri;
                memset(&ri, 0, sizeof(ri));
                ri.w0 = P.recPtr[r] - P.recPtr[0];
                ri.nw = R.nw; ri.neq = R.neq; ri.nalc = R.nalc; ri.nalg = R.nalg; ri.ngrp = R.ngrp;
                ri.mbnd = (int16_t)mbnd; ri.mbdr = (int16_t)mbdr;
                ri.mside = (side & 0xff) | (R.nonmono ? 0x100 : 0) | (R.denseLoc ? 0x200 : 0) |
                           (R.simpleWords ? 0x400 : 0);
                ri.file = file;
                P.rec[r] = ri;
                const int64_t ng = R.nalc > 0 ? R.ngrp : 0;
                P.cnt[0 * n1 + r] = R.neq;
                P.cnt[1 * n1 + r] = R.nalg + 1;
                P.cnt[2 * n1 + r] = R.nsw;
                P.cnt[3 * n1 + r] = R.ngrp;
                P.cnt[4 * n1 + r] = ng * (ng + 1) / 2;
                P.cnt[5 * n1 + r] = R.nalc > 0 ? (int64_t)R.nalg * (R.nalg + 1) / 2 : 0;
                atomicMax(&P.maxv[0], R.nw);
                atomicMax(&P.maxv[1], R.neq);
                atomicMax(&P.maxv[2], R.nalc);
                atomicMax(&P.maxv[3], R.nalg);
                atomicMax(&P.maxv[4], R.ngrp);
                if (mbnd >= 0) {
                    atomicMax(&P.maxv[5], mbnd);
                    atomicMax(&P.maxv[6], mbdr);
                    atomicAdd(&P.maxv[6 + side], 1);
                }
            }
        }
        __syncwarp();
    }
}

template <bool BIG>
__global__ void __launch_bounds__(32 * kUpWarps, UpCap<BIG>::kMinBlocks) k_up_fill(UpParams P) {
    extern __shared__ __align__(16) char upsm[];
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const unsigned lt = (1u << ln) - 1u;
    UpWarp<BIG> &W = reinterpret_cast<UpWarp<BIG> *>(upsm)[wib];
    const int64_t nwarps = (int64_t)gridDim.x * kUpWarps;
    const int64_t n1 = P.nrec + 1;
    const int64_t nsteps = up_steps<BIG>(P);
    for (int64_t it = (int64_t)blockIdx.x * kUpWarps + wib; it < nsteps; it += nwarps) {
        const int64_t r = BIG ? P.ovList[it] : P.rBegin + it;
        const RecShape R = analyze<BIG>(P, r, W, false);
        if (!BIG && R.code == kOverflow) {  // the large kernel fills it
            __syncwarp();
            continue;
        }
        const int64_t oEq = P.off[0 * n1 + r], oSlot = P.off[1 * n1 + r], oSw = P.off[2 * n1 + r];
        const int64_t oGrp = P.off[3 * n1 + r], oPair = P.off[4 * n1 + r];
        if (ln == 0) {
            RecInfo &ri = P.rec[r];
            ri.measOff = oEq; ri.slotOff = oSlot; ri.swOff = oSw; ri.grpOff = oGrp; ri.pairOff = oPair;
        }
        const double *gl = P.glder + (P.recPtr[r] - P.recPtr[0]);
        for (int i = ln; i < 3 * R.neq; i += 32) P.meas[3 * oEq + i] = W.eq[i];
        for (int i = ln; i < R.nsw; i += 32) {
            const uint64_t k = W.key[i];
            P.sw[oSw + i] = (key_eq(k) << 16) | key_word(k);
        }
        for (int s = ln; s <= R.nalg; s += 32) {
            if (s == R.nalg) {
                P.slots[oSlot + s] = 0;
                P.swStart[oSlot + s] = R.nsw;
                P.slotCnt[oSlot + s] = 0;
                continue;
            }
            const int a = W.slotStart[s], b = W.slotStart[s + 1];
            int nz = 0;
            for (int q = a; q < b; ++q) nz += gl[key_word(W.key[q])] != 0.0;
            P.slots[oSlot + s] = key_var(W.key[a]);
            P.swStart[oSlot + s] = a;
            P.slotCnt[oSlot + s] = nz;
        }
        // group list: heads of the group runs of the sorted slots
        int g0 = 0;
        for (int base = 0; base < R.nalg; base += 32) {
            const int s = base + ln;
            int g = 0;
            bool head = false;
            if (s < R.nalg) {
                g = P.p2g[key_var(W.key[W.slotStart[s]]) - 1];
                head = s == 0 || g != P.p2g[key_var(W.key[W.slotStart[s - 1]]) - 1];
            }
            const unsigned m = __ballot_sync(kFull, head);
            if (head) {
                const int gi = g0 + __popc(m & lt);
                P.grpId[oGrp + gi] = g;
                P.grpSlot[oGrp + gi] = s;
                P.grpRec[oGrp + gi] = (int32_t)r;
            }
            g0 += __popc(m);
        }
        __syncwarp();
    }
}

// block of every record group pair: sparse storage by the row's block list,
// packed storage as a key (I, J) sorted later
struct PairParams {
    int64_t nrec;
    const RecInfo *rec;
    const int32_t *grpId;
    int32_t matsto, nG;
    const int64_t *rowBlk0;
    const int32_t *blkJ;
    uint64_t *key;             // [npairs]
    unsigned long long *err;
};

__global__ void k_up_pairs(PairParams P) {
    const int ln = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = w; r < P.nrec; r += nw) {
        const RecInfo ri = P.rec[r];
        if (ri.nalc <= 0) continue;
        const int ng = ri.ngrp, npair = ng * (ng + 1) / 2;
        for (int p = ln; p < npair; p += 32) {
            int qa = 0;
            while ((qa + 1) * (qa + 2) / 2 <= p) qa++;
            const int qb = p - qa * (qa + 1) / 2;
            const int I = P.grpId[ri.grpOff + qa], J = P.grpId[ri.grpOff + qb];
            uint64_t key;
            if (P.matsto == 2) {
                int64_t lo = P.rowBlk0[I - 1], hi = P.rowBlk0[I] - 1, k = -1;
                while (lo <= hi) {
                    const int64_t mid = (lo + hi) >> 1;
                    const int32_t bj = P.blkJ[mid];
                    if (bj == J) { k = mid; break; }
                    if (bj < J) lo = mid + 1;
                    else hi = mid - 1;
                }
                if (k < 0) {
                    atomicMin(P.err, ((unsigned long long)r << 8) | MPGPU_ERR_BADINDEX);
                    k = 0;
                }
                key = (uint64_t)k;
            } else {
                key = (uint64_t)I * (uint64_t)(P.nG + 1) + (uint64_t)J;
            }
            P.key[ri.pairOff + p] = key;
        }
    }
}

__global__ void k_iota(uint32_t *v, int64_t n, uint32_t base) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = base + (uint32_t)i;
}

__global__ void k_copy_keys(const uint64_t *src, uint64_t *dst, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

// packed storage: distinct sorted keys -> block table, block id per pair
__global__ void k_key_heads(const uint64_t *k, int64_t n, int64_t *head) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) head[i] = (i == 0 || k[i] != k[i - 1]) ? 1 : 0;
    if (i == n) head[n] = 0;
}

__global__ void k_packed_blocks(const uint64_t *k, const uint32_t *v, const int64_t *headEx, int64_t n,
                                int32_t nG, uint64_t *pairKey, int32_t *bkI, int32_t *bkJ, int32_t *bkLd,
                                int64_t *bkOff) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool head = i == 0 || k[i] != k[i - 1];
    const int64_t id = headEx[i] + (head ? 0 : -1);
    pairKey[v[i]] = (uint64_t)id;
    if (head) {
        bkI[id] = (int32_t)(k[i] / (uint64_t)(nG + 1));
        bkJ[id] = (int32_t)(k[i] % (uint64_t)(nG + 1));
        bkLd[id] = 0;
        bkOff[id] = 0;
    }
}

__global__ void k_sparse_blocks(const int64_t *rowBlk0, int32_t nG, int32_t *bkI) {
    const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (I > nG) return;
    for (int64_t k = rowBlk0[I - 1]; k < rowBlk0[I]; ++k) bkI[k] = (int32_t)I;
}

__global__ void k_block_nel(const int32_t *bkI, const int32_t *bkJ, const int32_t *aig, int64_t nblk,
                            int64_t *nel, int32_t *pmax) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nblk) return;
    const int64_t ni = aig[bkI[k]] - aig[bkI[k] - 1], nj = aig[bkJ[k]] - aig[bkJ[k] - 1];
    nel[k] = bkI[k] == bkJ[k] ? ni * (ni + 1) / 2 : ni * nj;
    atomicMax(pmax, (int32_t)nel[k]);
}

// per chunk: segment bounds of the sorted pairs
__global__ void k_seg_bounds(const uint64_t *k, int64_t n, int64_t *segStart, int64_t *segEnd) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i == 0 || k[i] != k[i - 1]) segStart[k[i]] = i;
    if (i == n - 1 || k[i] != k[i + 1]) segEnd[k[i]] = i + 1;
}

struct ChunkParams {
    int64_t nblk;
    const int64_t *nel, *segStart, *segEnd;
    int64_t *cnt, *sb, *nit, *nslot, *nred;   // [nblk + 1] each
};

__global__ void k_chunk_counts(ChunkParams P) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > P.nblk) return;
    if (k == P.nblk) { P.cnt[k] = 0; P.sb[k] = 0; P.nit[k] = 0; P.nslot[k] = 0; P.nred[k] = 0; return; }
    const int64_t c = P.segEnd[k] - P.segStart[k];
    const int64_t nel = P.nel[k] > 0 ? P.nel[k] : 1;
    const int64_t per = max((int64_t)32, (int64_t)16384 / nel);
    const int64_t ni = c > 0 ? (c + per - 1) / per : 0;
    P.cnt[k] = c;
    P.sb[k] = c * P.nel[k];
    P.nit[k] = ni;
    P.nslot[k] = ni > 1 ? ni : 0;
    P.nred[k] = ni > 1 ? 1 : 0;
}

__global__ void k_pair_dst(const uint64_t *k, const uint32_t *v, int64_t n, const int64_t *segStart,
                           const int64_t *bBase, const int64_t *nel, int64_t *pairDst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t b = k[i];
    pairDst[v[i]] = bBase[b] + (i - segStart[b]) * nel[b];
}

struct ItemParams {
    int64_t nblk, item0, red0;
    const int64_t *cnt, *nel, *bBase, *itemOff, *slotOff, *redOff;
    int32_t *itBlk, *itCnt, *rdBlk, *rdN;
    int64_t *itBase, *itSlot, *rdSlot0;
};

__global__ void k_items(ItemParams P) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.nblk) return;
    const int64_t c = P.cnt[k];
    if (c <= 0) return;
    const int64_t nel = P.nel[k] > 0 ? P.nel[k] : 1;
    const int64_t per = max((int64_t)32, (int64_t)16384 / nel);
    const int64_t ni = (c + per - 1) / per;
    for (int64_t m = 0; m < ni; ++m) {
        const int64_t it = P.item0 + P.itemOff[k] + m;
        P.itBlk[it] = (int32_t)k;
        P.itBase[it] = P.bBase[k] + m * per * P.nel[k];
        P.itCnt[it] = (int32_t)min(per, c - m * per);
        P.itSlot[it] = ni > 1 ? P.slotOff[k] + m : -1;
    }
    if (ni > 1) {
        const int64_t rd = P.red0 + P.redOff[k];
        P.rdBlk[rd] = (int32_t)k;
        P.rdSlot0[rd] = P.slotOff[k];
        P.rdN[rd] = (int32_t)ni;
    }
}

// vector entries: group of every record group entry (records with locals)
__global__ void k_grp_keys(const int32_t *grpId, const int32_t *grpRec, const RecInfo *rec, int64_t g0,
                           int64_t n, int32_t nG, uint64_t *key, uint32_t *val) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t q = g0 + i;
    key[i] = rec[grpRec[q]].nalc > 0 ? (uint64_t)grpId[q] : (uint64_t)(nG + 1);
    val[i] = (uint32_t)q;
}

__global__ void k_grp_count(const uint64_t *key, int64_t n, int32_t nG, int64_t *cntG) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t g = key[i];
    if (g >= 1 && g <= (uint64_t)nG && (i == n - 1 || key[i + 1] != g)) cntG[g - 1] = i + 1;
}

__global__ void k_vstart(const int64_t *cntEnd, int32_t nG, int64_t vbase, int64_t *vs) {
    // vs[0] = vbase, vs[g] = vbase + end of group g (groups without entries
    // take the previous end); sequential over groups in one thread block
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int64_t e = 0;
    vs[0] = vbase;
    for (int32_t g = 1; g <= nG; ++g) {
        if (cntEnd[g - 1] > e) e = cntEnd[g - 1];
        vs[g] = vbase + e;
    }
}

__global__ void k_ventries(const uint64_t *key, const uint32_t *val, int64_t n, int32_t nG,
                           const int32_t *grpRec, const int32_t *grpSlot, const RecInfo *rec,
                           int64_t vbase, int64_t *vEntries) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || key[i] > (uint64_t)nG) return;
    const uint32_t q = val[i];
    const int64_t r = grpRec[q];
    vEntries[vbase + i] = (r << 40) | (rec[r].slotOff + grpSlot[q]);
}


// fit size class of every record (the shared memory of its fit: power-of-two
// classes from 4 KB, the last for records beyond one CTA), sort key (chunk,
// class) and the maxima of each class (reduced per block in shared memory)
__global__ void k_fit_bucket(const RecInfo *rec, int64_t nrec, const int64_t *chunkB, int nchunk, uint64_t *key,
                             uint32_t *val, int32_t *bmax) {
    __shared__ int32_t sm[MPG_FIT_BUCKETS * 7];
    for (int i = threadIdx.x; i < MPG_FIT_BUCKETS * 7; i += blockDim.x) sm[i] = 0;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += stride) {
        const RecInfo ri = rec[r];
        int lo = 0, hi = nchunk - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (chunkB[mid] <= r) lo = mid;
            else hi = mid - 1;
        }
        const bool band = ri.mbnd >= 0;
        const int64_t bytes = warp_bytes(max(ri.nw, 1), max(ri.neq, 1), max(ri.nalc, 1), max(ri.nalg, 1),
                                         band ? ri.mbnd : -1, band ? ri.mbdr : 0, max(ri.ngrp, 1), false);
        int b = 0;
        if (bytes > 220 * 1024) b = MPG_FIT_BUCKETS - 1;
        else
            while (b < MPG_FIT_BUCKETS - 2 && ((int64_t)4096 << b) < bytes) b++;
        key[r] = (uint64_t)lo * MPG_FIT_BUCKETS + (uint64_t)b;
        val[r] = (uint32_t)r;
        int32_t *m = sm + 7 * b;
        atomicMax(&m[0], ri.nw);
        atomicMax(&m[1], ri.neq);
        atomicMax(&m[2], ri.nalc);
        atomicMax(&m[3], ri.nalg);
        if (band) {
            atomicMax(&m[4], ri.mbnd + 1);
            atomicMax(&m[5], ri.mbdr);
        }
        atomicMax(&m[6], ri.ngrp);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < MPG_FIT_BUCKETS * 7; i += blockDim.x)
        if (sm[i] > 0) atomicMax(&bmax[i], sm[i]);
}

__global__ void k_key_ends(const uint64_t *k, int64_t n, int64_t *ends) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && (i == n - 1 || k[i] != k[i + 1])) ends[k[i]] = i + 1;
}

__global__ void k_u32_copy(const uint32_t *src, uint32_t *dst, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

}  // namespace

int32_t upload_records_device(mpgpu_ctx *c, int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                              const double *glder, const int32_t *recFile, int32_t nfiles,
                              const double *fileWeight) {
    DevJob &j = c->j;
    UpTmp &t = j.tmp;
    cudaStream_t s = c->stream;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    j.nfiles = nfiles;
    j.nrec = nrec;
    j.nw = recPtr[nrec] - recPtr[0];
    const int64_t n1 = nrec + 1;
    // ---- records to the device
    MPG_CUDA(c, dgrow(j, j.inder, j.nw));
    MPG_CUDA(c, dgrow(j, j.glder, j.nw));
    MPG_CUDA(c, dgrow(j, t.recPtr, n1));
    cudaEvent_t ev[3];
    for (auto &x : ev) cudaEventCreate(&x);
    cudaEventRecord(ev[0], s);
    MPG_CUDA(c, cudaMemcpyAsync(t.recPtr, recPtr, sizeof(int64_t) * n1, cudaMemcpyHostToDevice, s));
    // the words in chunks of records on the second stream; the scan of a
    // chunk starts as soon as its copy is done (the link, not the decode,
    // bounds the upload)
    const int nchunkCopy = (inder && j.nw > ((int64_t)64 << 20)) ? 8 : 1;
    std::vector<int64_t> cr(nchunkCopy + 1);
    for (int k = 0; k <= nchunkCopy; ++k) cr[k] = nrec * k / nchunkCopy;
    std::vector<cudaEvent_t> evc(nchunkCopy);
    for (auto &x : evc) cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    struct EvFree {
        std::vector<cudaEvent_t> &e;
        ~EvFree() {
            for (auto x : e) cudaEventDestroy(x);
        }
    } evFree{evc};
    cudaStream_t sc = inder ? c->stream2 : s;
    MPG_CUDA(c, cudaEventRecord(ev[1], s));
    MPG_CUDA(c, cudaStreamWaitEvent(sc, ev[1], 0));
    for (int k = 0; k < nchunkCopy; ++k) {
        const int64_t a = recPtr[cr[k]], b = recPtr[cr[k + 1]];
        if (inder && b > a) {
            MPG_CUDA(c, cudaMemcpyAsync(j.inder + (a - recPtr[0]), inder + a, sizeof(int32_t) * (b - a),
                                        cudaMemcpyHostToDevice, sc));
            MPG_CUDA(c, cudaMemcpyAsync(j.glder + (a - recPtr[0]), glder + a, sizeof(double) * (b - a),
                                        cudaMemcpyHostToDevice, sc));
        }
        MPG_CUDA(c, cudaEventRecord(evc[k], sc));
    }
    int32_t *dRecFile = nullptr;
    if (recFile) {
        MPG_CUDA(c, dgrow(j, t.recFile, nrec));
        MPG_CUDA(c, cudaMemcpyAsync(t.recFile, recFile, sizeof(int32_t) * nrec, cudaMemcpyHostToDevice, s));
        dRecFile = t.recFile;
    }
    MPG_CUDA(c, dgrow(j, j.rec, nrec));
    MPG_CUDA(c, dgrow(j, t.cnt, 6 * n1));
    MPG_CUDA(c, dgrow(j, t.scanTmp, scan_tmp_len(std::max<int64_t>(n1, 256 * 8))));
    // scalars: the error word (min over record << 8 | code) and 16 maxima
    MPG_CUDA(c, dgrow(j, t.scal, 16));
    unsigned long long *dErr = (unsigned long long *)t.scal;
    int32_t *dMax = (int32_t *)(t.scal + 2);
    MPG_CUDA(c, cudaMemsetAsync(dErr, 0xff, 8, s));
    MPG_CUDA(c, cudaMemsetAsync(dMax, 0, 16 * sizeof(int32_t), s));
    MPG_CUDA(c, cudaMemsetAsync(t.cnt, 0, sizeof(int64_t) * 6 * n1, s));
    // records beyond the compact kernels' capacity: list and count
    MPG_CUDA(c, dgrow(j, t.ovList, nrec));
    int32_t *dOvN = (int32_t *)(t.scal + 12);
    MPG_CUDA(c, cudaMemsetAsync(dOvN, 0, sizeof(int32_t), s));
    UpParams P{};
    P.nrec = nrec; P.recPtr = t.recPtr; P.inder = j.inder; P.glder = j.glder; P.recFile = dRecFile;
    P.nfiles = nfiles; P.varOfTot = j.varOfTot; P.nTotal = j.nTotal; P.p2g = j.p2g; P.aig = j.aig;
    P.nVar = j.nVar; P.nG = j.nG; P.rec = j.rec; P.cnt = t.cnt; P.err = dErr; P.maxv = dMax;
    P.ovList = t.ovList; P.ovCount = dOvN;
    // compact kernels: one wave of persistent CTAs at their occupancy;
    // large kernels: two CTAs per SM over the overflow list
    const int smemS = kUpWarps * (int)sizeof(UpWarp<false>);
    const int smemB = kUpWarps * (int)sizeof(UpWarp<true>);
    MPG_CUDA(c, smem_optin((const void *)k_up_scan<false>));
    MPG_CUDA(c, smem_optin((const void *)k_up_fill<false>));
    MPG_CUDA(c, smem_optin((const void *)k_up_scan<true>));
    MPG_CUDA(c, smem_optin((const void *)k_up_fill<true>));
    int perSm = 0;
    MPG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_up_scan<false>, 32 * kUpWarps, smemS));
    const unsigned upBlocks = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((nrec + kUpWarps - 1) / kUpWarps, (int64_t)nsm * std::max(perSm, 1)));
    const unsigned upBlocksBig = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nrec, (int64_t)nsm * 2));
    for (int k = 0; k < nchunkCopy; ++k) {
        MPG_CUDA(c, cudaStreamWaitEvent(s, evc[k], 0));
        P.rBegin = cr[k];
        P.rEnd = cr[k + 1];
        const unsigned g = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>((P.rEnd - P.rBegin + kUpWarps - 1) / kUpWarps, (int64_t)upBlocks));
        if (P.rEnd > P.rBegin) k_up_scan<false><<<g, 32 * kUpWarps, smemS, s>>>(P);
    }
    // copy time: until the last chunk has arrived
    cudaEventRecord(ev[1], sc);
    if (nrec > 0) k_up_scan<true><<<upBlocksBig, 32 * kUpWarps, smemB, s>>>(P);
    P.rBegin = 0;
    P.rEnd = nrec;
    MPG_CUDA(c, cudaGetLastError());
    // offsets: exclusive scans of the six count arrays (the spare last
    // element of each receives the total)
    MPG_CUDA(c, dgrow(j, t.off, 6 * n1));
    for (int k = 0; k < 6; ++k) MPG_CUDA(c, scan_ex(t.cnt + k * n1, t.off + k * n1, n1, t.scanTmp, s));
    int64_t tot[6];
    for (int k = 0; k < 6; ++k)
        MPG_CUDA(c, cudaMemcpyAsync(&tot[k], t.off + k * n1 + nrec, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    unsigned long long herr = 0;
    int32_t hmax[16];
    MPG_CUDA(c, cudaMemcpyAsync(&herr, dErr, 8, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaMemcpyAsync(hmax, dMax, sizeof(hmax), cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    if (herr != ~0ull) {
        char buf[128];
        snprintf(buf, sizeof buf, "record %lld rejected at upload (code %d)", (long long)(herr >> 8),
                 (int)(herr & 0xff));
        return set_err(c, (int32_t)(herr & 0xff), buf);
    }
    j.maxNw = hmax[0]; j.maxNeq = hmax[1]; j.maxNalc = hmax[2]; j.maxNalg = hmax[3];
    j.maxNgrp = std::max(hmax[4], 1);
    j.maxBand = (hmax[7] + hmax[8]) > 0 ? hmax[5] : -1;
    j.maxBdr = hmax[6];
    j.nbndr[0] = hmax[7]; j.nbndr[1] = hmax[8];
    j.nbdrx = hmax[6]; j.nbndx = (hmax[7] + hmax[8]) > 0 ? hmax[5] : 0;
    const int64_t neqT = tot[0], nslotT = tot[1], nswT = tot[2], ngrpT = tot[3], npairs = tot[4],
                  stageAll = tot[5];
    j.neqTot = neqT; j.nslotTot = nslotT; j.nswTot = nswT; j.ngrpTot = ngrpT;
    if (npairs >= ((int64_t)1 << 32) || ngrpT >= ((int64_t)1 << 32))
        return set_err(c, MPGPU_ERR_LIMIT, "too many record group pairs for one upload");
    // ---- tables
    MPG_CUDA(c, dgrow(j, j.meas, 3 * neqT));
    MPG_CUDA(c, dgrow(j, j.slots, nslotT));
    MPG_CUDA(c, dgrow(j, j.slotCnt, nslotT));
    MPG_CUDA(c, dgrow(j, j.swStart, nslotT));
    MPG_CUDA(c, dgrow(j, j.vstage, nslotT));
    MPG_CUDA(c, dgrow(j, j.sw, nswT));
    MPG_CUDA(c, dgrow(j, j.grpId, ngrpT));
    MPG_CUDA(c, dgrow(j, j.grpSlot, ngrpT));
    MPG_CUDA(c, dgrow(j, t.grpRec, ngrpT));
    P.off = t.off; P.meas = j.meas; P.slots = j.slots; P.slotCnt = j.slotCnt; P.swStart = j.swStart;
    P.sw = j.sw; P.grpId = j.grpId; P.grpSlot = j.grpSlot; P.grpRec = t.grpRec;
    if (nrec > 0) {
        k_up_fill<false><<<upBlocks, 32 * kUpWarps, smemS, s>>>(P);
        k_up_fill<true><<<upBlocksBig, 32 * kUpWarps, smemB, s>>>(P);
    }
    MPG_CUDA(c, cudaGetLastError());
    // ---- blocks of the record pairs
    const int64_t nsort = std::max<int64_t>({npairs, ngrpT, nrec, 1});
    MPG_CUDA(c, dgrow(j, t.k0, nsort));
    MPG_CUDA(c, dgrow(j, t.k1, nsort));
    MPG_CUDA(c, dgrow(j, t.v0, nsort));
    MPG_CUDA(c, dgrow(j, t.v1, nsort));
    MPG_CUDA(c, dgrow(j, t.pairKey, npairs));
    const int64_t ntiles = (nsort + kRsTile - 1) / kRsTile;
    MPG_CUDA(c, dgrow(j, t.hist, 256 * ntiles + 1));
    // scan scratch for every later scan: histograms, pair heads, blocks
    const int64_t nblkMax = j.matsto == 2 ? (int64_t)j.hBlkJ.size() : npairs;
    const int64_t scanMax = std::max({256 * ntiles + 1, n1, npairs + 1, nblkMax + 1});
    MPG_CUDA(c, dgrow(j, t.scanTmp, scan_tmp_len(scanMax)));
    SortBufs sb{t.k0, t.k1, t.v0, t.v1, t.hist, t.scanTmp};
    PairParams pp{nrec, j.rec, j.grpId, j.matsto, j.nG, j.rowBlk0, j.blkJ, t.pairKey, dErr};
    if (nrec > 0) k_up_pairs<<<blocks_for(32 * std::min<int64_t>(nrec, (int64_t)nsm * 64)), 256, 0, s>>>(pp);
    MPG_CUDA(c, cudaGetLastError());
    int64_t nblk = 0;
    if (j.matsto == 2) {
        nblk = (int64_t)j.hBlkJ.size();
        MPG_CUDA(c, dgrow(j, j.bkI, nblk));
        MPG_CUDA(c, dgrow(j, j.bkJ, nblk));
        MPG_CUDA(c, dgrow(j, j.bkLd, nblk));
        MPG_CUDA(c, dgrow(j, j.bkOff, nblk));
        k_sparse_blocks<<<blocks_for(j.nG), 256, 0, s>>>(j.rowBlk0, j.nG, j.bkI);
        MPG_CUDA(c, cudaMemcpyAsync(j.bkJ, j.blkJ, sizeof(int32_t) * nblk, cudaMemcpyDeviceToDevice, s));
        MPG_CUDA(c, cudaMemcpyAsync(j.bkLd, j.blkLd, sizeof(int32_t) * nblk, cudaMemcpyDeviceToDevice, s));
        MPG_CUDA(c, cudaMemcpyAsync(j.bkOff, j.blkOff, sizeof(int64_t) * nblk, cudaMemcpyDeviceToDevice, s));
    } else if (npairs > 0) {
        // packed storage: the group pairs met in the records, sorted
        k_copy_keys<<<blocks_for(npairs), 256, 0, s>>>(t.pairKey, sb.k0, npairs);
        k_iota<<<blocks_for(npairs), 256, 0, s>>>(sb.v0, npairs, 0);
        MPG_CUDA(c, radix_sort(sb, npairs, bits_for((uint64_t)(j.nG + 1) * (uint64_t)(j.nG + 1)), s));
        MPG_CUDA(c, dgrow(j, t.head, npairs + 1));
        k_key_heads<<<blocks_for(npairs + 1), 256, 0, s>>>(sb.k0, npairs, t.head);
        MPG_CUDA(c, scan_ex(t.head, t.head, npairs + 1, t.scanTmp, s));
        MPG_CUDA(c, cudaMemcpyAsync(&nblk, t.head + npairs, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        MPG_CUDA(c, dgrow(j, j.bkI, nblk));
        MPG_CUDA(c, dgrow(j, j.bkJ, nblk));
        MPG_CUDA(c, dgrow(j, j.bkLd, nblk));
        MPG_CUDA(c, dgrow(j, j.bkOff, nblk));
        k_packed_blocks<<<blocks_for(npairs), 256, 0, s>>>(sb.k0, sb.v0, t.head, npairs, j.nG, t.pairKey,
                                                           j.bkI, j.bkJ, j.bkLd, j.bkOff);
    }
    MPG_CUDA(c, cudaGetLastError());
    j.nblk = nblk;
    MPG_CUDA(c, dgrow(j, t.nel, nblk + 1));
    int32_t *dPmax = dMax + 12;
    MPG_CUDA(c, cudaMemsetAsync(dPmax, 0, sizeof(int32_t), s));
    if (nblk > 0) k_block_nel<<<blocks_for(nblk), 256, 0, s>>>(j.bkI, j.bkJ, j.aig, nblk, t.nel, dPmax);
    // ---- chunks by staging size
    int64_t stageElems = std::max<int64_t>(c->stagingBytes / 8, 1);
    bool oneChunk = false;
    if (c->stagingBytes <= 0) {
        size_t freeB = 0, totalB = 0;
        MPG_CUDA(c, cudaMemGetInfo(&freeB, &totalB));
        // memory the staging may take: the free memory (plus the current
        // staging, which is reused) less what the per-chunk buffers need
        const int64_t current = j.cap.count((const void *)&j.stage) ? j.cap[(const void *)&j.stage] * 8 : 0;
        const int64_t others = 48 * nblk + 40 * (npairs / 32 + nblk) + ((int64_t)1 << 30);
        const int64_t room = std::max<int64_t>(((int64_t)freeB + current - others) / 10 * 9, (int64_t)256 << 20);
        if (stageAll * 8 <= room) {
            stageElems = std::max<int64_t>(stageAll, 1);
            oneChunk = true;
        } else {
            stageElems = room / 16;
        }
    } else if (stageAll <= stageElems) {
        oneChunk = true;
    }
    j.chunkRec.assign(1, 0);
    int64_t maxStage = 0;
    if (oneChunk) {
        j.chunkRec.push_back(nrec);
        maxStage = stageAll;
    } else {
        std::vector<int64_t> hs(n1);
        MPG_CUDA(c, cudaMemcpyAsync(hs.data(), t.cnt + 5 * n1, sizeof(int64_t) * n1, cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        int64_t upd = 0;
        for (int64_t r = 0; r < nrec; ++r) {
            const int64_t ngg = hs[r];
            if (ngg > stageElems) return set_err(c, MPGPU_ERR_LIMIT, "record update larger than the staging buffer");
            if (upd + ngg > stageElems) { j.chunkRec.push_back(r); maxStage = std::max(maxStage, upd); upd = 0; }
            upd += ngg;
        }
        j.chunkRec.push_back(nrec);
        maxStage = std::max(maxStage, upd);
    }
    const int64_t nchunk = (int64_t)j.chunkRec.size() - 1;
    // pair and group-entry ranges of the chunks
    std::vector<int64_t> pOff(nchunk + 1), gOff(nchunk + 1);
    for (int64_t ch = 0; ch <= nchunk; ++ch) {
        MPG_CUDA(c, cudaMemcpyAsync(&pOff[ch], t.off + 4 * n1 + j.chunkRec[ch], sizeof(int64_t),
                                    cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaMemcpyAsync(&gOff[ch], t.off + 3 * n1 + j.chunkRec[ch], sizeof(int64_t),
                                    cudaMemcpyDeviceToHost, s));
    }
    int32_t hPmax = 1;
    MPG_CUDA(c, cudaMemcpyAsync(&hPmax, dPmax, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaMemcpyAsync(&herr, dErr, 8, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    if (herr != ~0ull) return set_err(c, MPGPU_ERR_BADINDEX, "record group pair not in the sparse structure");
    j.pstride = std::max(hPmax, 1);
    // ---- per chunk: staging positions, work items, vector entries
    MPG_CUDA(c, dgrow(j, j.pairDst, npairs));
    MPG_CUDA(c, dgrow(j, t.segStart, nblk + 1));
    MPG_CUDA(c, dgrow(j, t.segEnd, nblk + 1));
    MPG_CUDA(c, dgrow(j, t.bcnt, 5 * (nblk + 1)));
    MPG_CUDA(c, dgrow(j, t.bscan, 4 * (nblk + 1)));
    const int64_t itemCap = npairs / 32 + nchunk * (nblk + 1) + 1;
    MPG_CUDA(c, dgrow(j, j.itBlk, itemCap));
    MPG_CUDA(c, dgrow(j, j.itBase, itemCap));
    MPG_CUDA(c, dgrow(j, j.itCnt, itemCap));
    MPG_CUDA(c, dgrow(j, j.itSlot, itemCap));
    MPG_CUDA(c, dgrow(j, j.rdBlk, itemCap));
    MPG_CUDA(c, dgrow(j, j.rdSlot0, itemCap));
    MPG_CUDA(c, dgrow(j, j.rdN, itemCap));
    MPG_CUDA(c, dgrow(j, j.vEntries, ngrpT));
    MPG_CUDA(c, dgrow(j, j.vStart, nchunk * (j.nG + 1)));
    MPG_CUDA(c, dgrow(j, t.cntG, j.nG + 1));
    j.chunkItem.assign(1, 0);
    j.chunkRed.assign(1, 0);
    int64_t maxSlots = 1, vbase = 0, item0 = 0, red0 = 0;
    const int blkBits = bits_for((uint64_t)std::max<int64_t>(nblk, 1));
    const int grpBits = bits_for((uint64_t)j.nG + 1);
    const int64_t nb1 = nblk + 1;
    int64_t *bc = t.bcnt, *bs = t.bscan;
    ChunkParams cp{nblk, t.nel, t.segStart, t.segEnd, bc, bc + nb1, bc + 2 * nb1, bc + 3 * nb1, bc + 4 * nb1};
    for (int64_t ch = 0; ch < nchunk; ++ch) {
        const int64_t p0 = pOff[ch], np = pOff[ch + 1] - pOff[ch];
        MPG_CUDA(c, cudaMemsetAsync(t.segStart, 0, sizeof(int64_t) * nb1, s));
        MPG_CUDA(c, cudaMemsetAsync(t.segEnd, 0, sizeof(int64_t) * nb1, s));
        if (np > 0) {
            k_copy_keys<<<blocks_for(np), 256, 0, s>>>(t.pairKey + p0, sb.k0, np);
            k_iota<<<blocks_for(np), 256, 0, s>>>(sb.v0, np, (uint32_t)p0);
            MPG_CUDA(c, radix_sort(sb, np, blkBits, s));
            k_seg_bounds<<<blocks_for(np), 256, 0, s>>>(sb.k0, np, t.segStart, t.segEnd);
        }
        k_chunk_counts<<<blocks_for(nb1), 256, 0, s>>>(cp);
        // bBase, item, slot and reduction offsets
        MPG_CUDA(c, scan_ex(cp.sb, bs, nb1, t.scanTmp, s));
        MPG_CUDA(c, scan_ex(cp.nit, bs + nb1, nb1, t.scanTmp, s));
        MPG_CUDA(c, scan_ex(cp.nslot, bs + 2 * nb1, nb1, t.scanTmp, s));
        MPG_CUDA(c, scan_ex(cp.nred, bs + 3 * nb1, nb1, t.scanTmp, s));
        if (np > 0)
            k_pair_dst<<<blocks_for(np), 256, 0, s>>>(sb.k0, sb.v0, np, t.segStart, bs, t.nel, j.pairDst);
        int64_t h4[4];
        for (int k = 0; k < 4; ++k)
            MPG_CUDA(c, cudaMemcpyAsync(&h4[k], bs + k * nb1 + nblk, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        if (h4[0] > maxStage) return set_err(c, MPGPU_ERR_LIMIT, "staging layout exceeds the chunk size");
        if (item0 + h4[1] > itemCap || red0 + h4[3] > itemCap)
            return set_err(c, MPGPU_ERR_LIMIT, "work-item table overflow");
        ItemParams ip{nblk, item0, red0, cp.cnt, t.nel, bs, bs + nb1, bs + 2 * nb1, bs + 3 * nb1,
                      j.itBlk, j.itCnt, j.rdBlk, j.rdN, j.itBase, j.itSlot, j.rdSlot0};
        if (nblk > 0) k_items<<<blocks_for(nblk), 256, 0, s>>>(ip);
        item0 += h4[1];
        red0 += h4[3];
        maxSlots = std::max(maxSlots, h4[2]);
        j.chunkItem.push_back(item0);
        j.chunkRed.push_back(red0);
        // vector entries of the chunk by group, in record order
        const int64_t g0 = gOff[ch], ng = gOff[ch + 1] - gOff[ch];
        MPG_CUDA(c, cudaMemsetAsync(t.cntG, 0, sizeof(int64_t) * (j.nG + 1), s));
        if (ng > 0) {
            k_grp_keys<<<blocks_for(ng), 256, 0, s>>>(j.grpId, t.grpRec, j.rec, g0, ng, j.nG, sb.k0, sb.v0);
            MPG_CUDA(c, radix_sort(sb, ng, grpBits, s));
            k_grp_count<<<blocks_for(ng), 256, 0, s>>>(sb.k0, ng, j.nG, t.cntG);
            k_ventries<<<blocks_for(ng), 256, 0, s>>>(sb.k0, sb.v0, ng, j.nG, t.grpRec, j.grpSlot, j.rec, vbase,
                                                      j.vEntries);
        }
        int64_t *vs = j.vStart + ch * (j.nG + 1);
        k_vstart<<<1, 32, 0, s>>>(t.cntG, j.nG, vbase, vs);
        int64_t vend = 0;
        MPG_CUDA(c, cudaMemcpyAsync(&vend, vs + j.nG, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        vbase = vend;
    }
    MPG_CUDA(c, cudaGetLastError());
    // ---- fit buckets: records ordered by (chunk, size class, record)
    {
        const int64_t nkey = nchunk * MPG_FIT_BUCKETS;
        MPG_CUDA(c, dgrow(j, t.chunkB, nchunk + 1));
        MPG_CUDA(c, dgrow(j, t.bmax, MPG_FIT_BUCKETS * 7));
        MPG_CUDA(c, dgrow(j, t.keyEnd, nkey));
        MPG_CUDA(c, dgrow(j, j.recList, nrec));
        MPG_CUDA(c, cudaMemcpyAsync(t.chunkB, j.chunkRec.data(), sizeof(int64_t) * (nchunk + 1),
                                    cudaMemcpyHostToDevice, s));
        MPG_CUDA(c, cudaMemsetAsync(t.bmax, 0, sizeof(int32_t) * MPG_FIT_BUCKETS * 7, s));
        MPG_CUDA(c, cudaMemsetAsync(t.keyEnd, 0, sizeof(int64_t) * nkey, s));
        if (nrec > 0) {
            k_fit_bucket<<<(unsigned)std::min<int64_t>(blocks_for(nrec), (int64_t)nsm * 4), 256, 0, s>>>(
                j.rec, nrec, t.chunkB, (int)nchunk, sb.k0, sb.v0, t.bmax);
            MPG_CUDA(c, radix_sort(sb, nrec, bits_for((uint64_t)std::max<int64_t>(nkey - 1, 1)), s));
            k_key_ends<<<blocks_for(nrec), 256, 0, s>>>(sb.k0, nrec, t.keyEnd);
            k_u32_copy<<<blocks_for(nrec), 256, 0, s>>>(sb.v0, j.recList, nrec);
        }
        std::vector<int64_t> ends(nkey);
        std::vector<int32_t> prevMax = j.bucketMax;
        j.bucketMax.assign(MPG_FIT_BUCKETS * 7, 0);
        MPG_CUDA(c, cudaMemcpyAsync(ends.data(), t.keyEnd, sizeof(int64_t) * nkey, cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaMemcpyAsync(j.bucketMax.data(), t.bmax, sizeof(int32_t) * MPG_FIT_BUCKETS * 7,
                                    cudaMemcpyDeviceToHost, s));
        MPG_CUDA(c, cudaStreamSynchronize(s));
        j.bucketOff.assign(nkey + 1, 0);
        for (int64_t k = 0; k < nkey; ++k) j.bucketOff[k + 1] = ends[k] > 0 ? ends[k] : j.bucketOff[k];
        // tuned warps per CTA stay valid for a class whose maxima (and so
        // its shared-memory arena) did not change
        if (j.bucketWpc.size() != MPG_FIT_BUCKETS || prevMax.size() != j.bucketMax.size()) {
            j.bucketWpc.assign(MPG_FIT_BUCKETS, 0);
            j.bucketTuneMs.assign(MPG_FIT_BUCKETS * 4, 0.0);
        } else {
            for (int b = 0; b < MPG_FIT_BUCKETS; ++b)
                if (!std::equal(prevMax.begin() + 7 * b, prevMax.begin() + 7 * b + 7, j.bucketMax.begin() + 7 * b)) {
                    j.bucketWpc[b] = 0;
                    for (int k = 0; k < 4; ++k) j.bucketTuneMs[4 * b + k] = 0.0;
                }
        }
    }
    // ---- per-loop outputs, file weights, staging and partial sums
    std::vector<double> fw(nfiles, 1.0);
    if (fileWeight) fw.assign(fileWeight, fileWeight + nfiles);
    MPG_CUDA(c, dgrow(j, j.fileWeight, nfiles));
    MPG_CUDA(c, cudaMemcpyAsync(j.fileWeight, fw.data(), sizeof(double) * nfiles, cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, dgrow(j, j.status, nrec));
    MPG_CUDA(c, dgrow(j, j.chi2add, nrec));
    MPG_CUDA(c, dgrow(j, j.ndfadd, nrec));
    MPG_CUDA(c, dgrow(j, j.chndf, nrec));
    j.partialLen = maxSlots * j.pstride;
    MPG_CUDA(c, dgrow(j, j.partial, j.partialLen));
    j.stageLen = std::max<int64_t>(maxStage, 1);
    MPG_CUDA(c, dgrow(j, j.stage, (nchunk > 1 ? 2 : 1) * j.stageLen));
    cudaEventRecord(ev[2], s);
    MPG_CUDA(c, cudaStreamSynchronize(s));
    float t01 = 0.0f, t12 = 0.0f;
    cudaEventElapsedTime(&t01, ev[0], ev[1]);
    cudaEventElapsedTime(&t12, ev[1], ev[2]);
    j.msUploadCopy = t01;
    j.msUploadPrepare = t12;
    j.uploadChunks = (int32_t)nchunk;
    for (auto &x : ev) cudaEventDestroy(x);
    return MPGPU_OK;
}
