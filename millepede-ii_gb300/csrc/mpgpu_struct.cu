// mpgpu_struct.cu -- pede's structure passes on the device.
//
// loop1 (mpgpu_loop1_device): the label table, the entries per label, the
// variable numbering and the parameter groups, with the results of
// mpgpu_host_labels (label table mppar.f90:117-252, entries cut
// pede.f90:5958-5971, pargrp pede.f90:2311-2404, variable groups
// pede.f90:6509-6545), and the translation of the records to total indices
// (prepareRecords(1), mppar.f90:282-321) in place on a device copy that the
// context keeps for loop2 and for the record preparation.
//   1. one warp per record decodes the measurements and inserts the labels
//      of the global words into an open-addressing hash set in HBM, chunk by
//      chunk of records as their copy to the device completes
//      (multiplicative hash, linear probing, lanes holding the same label
//      insert once); a set more than half full is rebuilt eight times larger;
//   2. the occupied slots are compacted and radix-sorted by label: the rank
//      of a label is its total index, stored beside the slot;
//   3. one warp per record translates its global words through the set and
//      counts, per measurement and non-zero derivative, the entries and the
//      group cuts (after x when x+1 is not in the measurement, before x when
//      x-1 is not, both when x occurs twice: the cuts of a sorted index list
//      at its ends and gaps);
//   4. the per-label arrays go to the host, where the last step is the code
//      of mpgpu_host_labels (labels_finish).
//
// loop2 (mpgpu_loop2_device): the mpbits structure of mpgpu_host_mpbits
// (pede.f90:6889-6908, ndbits/spbits mpbits.f90:305-566, 1220-1350) from
// the kept records: one warp per record gathers its distinct parameter
// groups and sets the bits of their pairs in a lower-triangular bitmap, one
// warp per row group counts its
// columns and regions and chooses list or region form, scans give the
// offsets, and one warp per row writes its columns.
//
// Everything is deterministic: set membership and integer counts only.
#include "mpgpu_records.cuh"

#include <cstdio>

#include "host_struct.h"

namespace {

constexpr int kHashProbeMax = 4096;
constexpr int kL1Warps = 4;
static_assert(UpCap<false>::kWords / 32 <= UpCap<false>::kSw + 1 && UpCap<true>::kWords / 32 <= UpCap<true>::kSw + 1,
              "non-zero mask of the words in the slot-start array");

__device__ __forceinline__ uint64_t label_hash(int32_t x) {
    uint32_t h = (uint32_t)x * 2654435761u;
    return (uint64_t)(h ^ (h >> 15));
}

// insert a label (> 0) into the set; false when the probe limit is reached
__device__ bool hash_insert(int32_t *tab, uint64_t mask, int32_t key, unsigned int *count) {
    uint64_t s = label_hash(key) & mask;
    for (int i = 0; i < kHashProbeMax; ++i) {
        const int32_t cur = tab[s];
        if (cur == key) return true;
        if (cur == 0) {
            const int32_t old = atomicCAS(&tab[s], 0, key);
            if (old == 0) {
                atomicAdd(count, 1u);
                return true;
            }
            if (old == key) return true;
        }
        s = (s + 1) & mask;
    }
    return false;
}

// lookup in a set that no thread modifies during the kernel
__device__ int64_t hash_find(const int32_t *tab, uint64_t mask, int32_t key) {
    uint64_t s = label_hash(key) & mask;
    for (int i = 0; i < kHashProbeMax; ++i) {
        const int32_t cur = __ldg(&tab[s]);
        if (cur == key) return (int64_t)s;
        if (cur == 0) return -1;
        s = (s + 1) & mask;
    }
    return -1;
}

struct L1Params {
    int64_t nrec;
    const int64_t *recPtr;       // nrec + 1, absolute word offsets
    int32_t *inder;              // device copy from recPtr[0]; translated by k_l1_translate
    const double *glder;
    int32_t *tab;                // hash set of labels
    uint64_t mask;
    const int32_t *slotIdx;      // total index (0-based) of the label in each slot
    unsigned int *count;         // distinct labels inserted
    int *fail;                   // probe limit reached
    unsigned long long *err;     // min over (record << 8 | code)
    unsigned long long *cnt;     // entries per label, cntCopies copies of ncnt (chosen by block)
    int64_t ncnt;
    int cntCopies;
    uint8_t *seen, *cut;
    int64_t rBegin, rEnd;        // records of the compact kernels' launch
    int64_t *ovList;             // records beyond the compact capacity
    int32_t *ovCount;
};

__device__ __forceinline__ void l1_error(const L1Params &P, int64_t r, int code) {
    atomicMin(P.err, ((unsigned long long)r << 8) | (unsigned long long)code);
}

// words in shared memory (when they fit) and the measurements of record r;
// returns 0, a status code or kOverflow; nw 0 means an empty record
template <bool BIG>
__device__ int l1_decode(const L1Params &P, int64_t r, UpWarp<BIG> &W, const int32_t *&in, int &neq,
                         int64_t &w0, int &nw) {
    const int ln = threadIdx.x & 31;
    w0 = P.recPtr[r] - P.recPtr[0];
    const int64_t nw64 = P.recPtr[r + 1] - P.recPtr[r];
    neq = 0;
    nw = 0;
    in = P.inder + w0;
    if (nw64 <= 0) return nw64 == 0 ? 0 : MPGPU_ERR_BADRECORD;
    if (nw64 > MPG_WORDS_MAX) return MPGPU_ERR_LIMIT;
    nw = (int)nw64;
    if (nw <= UpCap<BIG>::kWords) {
        for (int i = ln; i < nw; i += 32) W.words[i] = in[i];
        __syncwarp();
        in = W.words;
    }
    return decode_measurements<BIG>(in, P.glder + w0, nw - 1, W, neq);
}

template <bool BIG>
__device__ __forceinline__ int64_t l1_steps(const L1Params &P) {
    return BIG ? (int64_t)*P.ovCount : P.rEnd - P.rBegin;
}

template <bool BIG>
__global__ void __launch_bounds__(32 * kL1Warps, UpCap<BIG>::kMinBlocks) k_l1_collect(L1Params P) {
    extern __shared__ __align__(16) char smem[];
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    UpWarp<BIG> &W = reinterpret_cast<UpWarp<BIG> *>(smem)[wib];
    const int64_t nwarps = (int64_t)gridDim.x * kL1Warps, nsteps = l1_steps<BIG>(P);
    for (int64_t it = (int64_t)blockIdx.x * kL1Warps + wib; it < nsteps; it += nwarps) {
        const int64_t r = BIG ? P.ovList[it] : P.rBegin + it;
        const int32_t *in;
        int neq, nw;
        int64_t w0;
        const int code = l1_decode<BIG>(P, r, W, in, neq, w0, nw);
        if (code == kOverflow) {
            if (ln == 0) P.ovList[atomicAdd(P.ovCount, 1)] = r;
            __syncwarp();
            continue;
        }
        if (code != 0) {
            if (ln == 0) l1_error(P, r, code);
            __syncwarp();
            continue;
        }
        int bad = 0, fail = 0;
        for (int e0 = 0; e0 < neq; e0 += 32) {
            const int e = e0 + ln;
            int q0 = 0, len = 0;
            if (e < neq) {
                q0 = W.eq[3 * e + 1] + 1;
                len = W.eq[3 * e + 2] - q0 + 1;
            }
            const int lmax = warp_max(len);
            for (int t = 0; t < lmax; ++t) {
                const int lab = t < len ? in[q0 + t] : 0;
                if (t < len && lab <= 0) bad = 1;
                const bool valid = t < len && lab > 0;
                const unsigned peers = __match_any_sync(kFull, valid ? lab : 0);
                if (valid && (__ffs(peers) - 1) == ln && !hash_insert(P.tab, P.mask, lab, P.count)) fail = 1;
            }
        }
        if (__any_sync(kFull, bad) && ln == 0) l1_error(P, r, MPGPU_ERR_BADINDEX);
        if (__any_sync(kFull, fail) && ln == 0) atomicExch(P.fail, 1);
        __syncwarp();
    }
}

// entries: sum of the per-block copies into the first
__global__ void k_l1_cnt_sum(unsigned long long *cnt, int64_t n, int copies) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long t = cnt[i];
    for (int k = 1; k < copies; ++k) t += cnt[(int64_t)k * n + i];
    cnt[i] = t;
}

__global__ void k_l1_steer(const int32_t *steer, int32_t n, int32_t *tab, uint64_t mask, unsigned int *count,
                           int *fail) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && steer[i] > 0 && !hash_insert(tab, mask, steer[i], count)) atomicExch(fail, 1);
}

__global__ void k_l1_occupied(const int32_t *tab, int64_t n, int64_t *flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = tab[i] != 0;
    if (i == n) flag[n] = 0;
}

__global__ void k_l1_compact(const int32_t *tab, int64_t n, const int64_t *pos, uint64_t *key, uint32_t *slot) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || tab[i] == 0) return;
    key[pos[i]] = (uint64_t)(uint32_t)tab[i];
    slot[pos[i]] = (uint32_t)i;
}

__global__ void k_l1_index(const uint64_t *key, const uint32_t *slot, int64_t n, int32_t *slotIdx,
                           int32_t *labels) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    slotIdx[slot[i]] = (int32_t)i;
    labels[i] = (int32_t)key[i];
}

template <bool BIG>
__global__ void __launch_bounds__(32 * kL1Warps, UpCap<BIG>::kMinBlocks) k_l1_translate(L1Params P) {
    extern __shared__ __align__(16) char smem[];
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    UpWarp<BIG> &W = reinterpret_cast<UpWarp<BIG> *>(smem)[wib];
    const int64_t nwarps = (int64_t)gridDim.x * kL1Warps, nsteps = l1_steps<BIG>(P);
    for (int64_t it = (int64_t)blockIdx.x * kL1Warps + wib; it < nsteps; it += nwarps) {
        const int64_t r = BIG ? P.ovList[it] : P.rBegin + it;
        const int32_t *in;
        int neq, nw;
        int64_t w0;
        const int code = l1_decode<BIG>(P, r, W, in, neq, w0, nw);
        if (code != 0) {  // overflow: the large kernel translates it; errors were reported
            __syncwarp();
            continue;
        }
        const bool smemWords = nw <= UpCap<BIG>::kWords;
        const double *gl = P.glder + w0;
        int32_t *out = P.inder + w0;
        // non-zero derivatives as a bit mask in shared memory (one
        // coalesced pass; the cut tests below read it many times)
        uint32_t *nzm = reinterpret_cast<uint32_t *>(W.slotStart);
        if (smemWords) {
            for (int i0 = 0; i0 < nw; i0 += 32) {
                const int i = i0 + ln;
                const unsigned b = __ballot_sync(kFull, i < nw && gl[i] != 0.0);
                if (ln == 0) nzm[i0 >> 5] = b;
            }
            __syncwarp();
        }
        auto nonzero = [&](int q) { return smemWords ? ((nzm[q >> 5] >> (q & 31)) & 1u) != 0 : gl[q] != 0.0; };
        for (int e0 = 0; e0 < neq; e0 += 32) {
            const int e = e0 + ln;
            int q0 = 0, q1 = -1;
            if (e < neq) {
                q0 = W.eq[3 * e + 1] + 1;
                q1 = W.eq[3 * e + 2];
            }
#pragma unroll 4
            for (int q = q0; q <= q1; ++q) {
                const int64_t s = hash_find(P.tab, P.mask, in[q]);
                const int32_t x = s >= 0 ? __ldg(&P.slotIdx[s]) : -1;
                out[q] = x + 1;
                if (smemWords) W.words[q] = x + 1;
            }
            // entries and group cuts over the non-zero derivatives, word
            // position by word position across the lanes so that lanes
            // holding the same index make one update
            const int len = q1 - q0 + 1, lmax = warp_max(len);
            for (int t = 0; t < lmax; ++t) {
                const int q = q0 + t;
                int x = -1;
                bool ca = false, cb = false;
                if (t < len && nonzero(q)) {
                    x = in[q] - 1;
                    bool prev = false, next = false, dup = false;
                    for (int u = q0; u <= q1; ++u) {
                        if (u == q || !nonzero(u)) continue;
                        const int y = in[u] - 1;
                        prev |= y == x - 1;
                        next |= y == x + 1;
                        dup |= y == x;
                    }
                    ca = !next || dup;
                    cb = x > 0 && (!prev || dup);
                }
                const unsigned peers = __match_any_sync(kFull, x);
                const unsigned mca = __ballot_sync(kFull, ca), mcb = __ballot_sync(kFull, cb);
                if (x >= 0 && (__ffs(peers) - 1) == ln) {
                    atomicAdd(&P.cnt[(int64_t)(blockIdx.x % P.cntCopies) * P.ncnt + x],
                              (unsigned long long)__popc(peers));
                    if (!P.seen[x]) P.seen[x] = 1;
                    if ((mca & peers) && !P.cut[x]) P.cut[x] = 1;
                    if ((mcb & peers) && !P.cut[x - 1]) P.cut[x - 1] = 1;
                }
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ loop2
struct L2Params {
    UpParams up;                        // record analysis (tables of the layout)
    const uint64_t *rowWord;            // first bitmap word of row group I, [nG + 2]
    unsigned long long *bits;
};

// distinct parameter groups of every record (ascending), the bits of all
// their pairs set in the bitmap.  The group ids of the variable global words
// are gathered per measurement, leaving out repeats of the measurement's
// previous group, then sorted and made unique.
template <bool BIG>
__global__ void __launch_bounds__(32 * kL1Warps, UpCap<BIG>::kMinBlocks) k_l2_bits(L2Params Q) {
    extern __shared__ __align__(16) char smem[];
    constexpr int CAPW = UpCap<BIG>::kWords, CAPSW = UpCap<BIG>::kSw;
    const int ln = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const unsigned lt = (1u << ln) - 1u;
    UpWarp<BIG> &W = reinterpret_cast<UpWarp<BIG> *>(smem)[wib];
    const UpParams &P = Q.up;
    const int64_t nwarps = (int64_t)gridDim.x * kL1Warps;
    const int64_t nsteps = BIG ? (int64_t)*P.ovCount : P.nrec;
    for (int64_t it = (int64_t)blockIdx.x * kL1Warps + wib; it < nsteps; it += nwarps) {
        const int64_t r = BIG ? P.ovList[it] : it;
        const int64_t w0 = P.recPtr[r] - P.recPtr[0];
        const int64_t nw64 = P.recPtr[r + 1] - P.recPtr[r];
        if (nw64 <= 0) continue;   // empty record
        int code = nw64 > MPG_WORDS_MAX ? MPGPU_ERR_LIMIT : 0;
        const int nw = (int)min(nw64, (int64_t)MPG_WORDS_MAX);
        const int32_t *in = P.inder + w0;
        int neq = 0;
        if (code == 0) {
            if (nw <= CAPW) {
                for (int i = ln; i < nw; i += 32) W.words[i] = in[i];
                __syncwarp();
                in = W.words;
            }
            code = decode_measurements<BIG>(in, P.glder + w0, nw - 1, W, neq);
        }
        int m = 0, bad = 0;
        if (code == 0) {
            for (int e0 = 0; e0 < neq; e0 += 32) {
                const int e = e0 + ln;
                int q0 = 0, len = 0;
                if (e < neq) {
                    q0 = W.eq[3 * e + 1] + 1;
                    len = W.eq[3 * e + 2] - q0 + 1;
                }
                const int lmax = warp_max(len);
                int lastG = 0;
                for (int t = 0; t < lmax; ++t) {
                    int g = 0;
                    if (t < len) {
                        const int ti = in[q0 + t];
                        if (ti < 1 || ti > P.nTotal) bad = 1;
                        else {
                            const int v = P.varOfTot[ti - 1];
                            if (v > 0) g = P.p2g[v - 1];
                        }
                    }
                    const bool add = g > 0 && g != lastG;
                    if (g > 0) lastG = g;
                    const unsigned msk = __ballot_sync(kFull, add);
                    if (add && m + __popc(msk & lt) < CAPSW) W.key[m + __popc(msk & lt)] = (uint64_t)g;
                    m += __popc(msk);
                }
            }
            __syncwarp();
            if (__any_sync(kFull, bad)) code = MPGPU_ERR_BADINDEX;
            else if (m > CAPSW) code = cap_code<BIG>();
        }
        if (!BIG && code == kOverflow) {
            if (ln == 0) P.ovList[atomicAdd(P.ovCount, 1)] = r;
            __syncwarp();
            continue;
        }
        if (code != 0) {
            if (ln == 0) atomicMin(P.err, ((unsigned long long)r << 8) | (unsigned long long)code);
            __syncwarp();
            continue;
        }
        if (m <= 32) sort_keys_regs<1>(W, m);
        else if (m <= 64) sort_keys_regs<2>(W, m);
        else if (m <= 128) sort_keys_regs<4>(W, m);
        else if (m <= 256) sort_keys_regs<8>(W, m);
        else if constexpr (BIG) sort_keys_smem<BIG>(W, m);
        int32_t *G = W.eq;
        int ng = 0;
        for (int base = 0; base < m; base += 32) {
            const int i = base + ln;
            const bool head = i < m && (i == 0 || W.key[i] != W.key[i - 1]);
            const unsigned msk = __ballot_sync(kFull, head);
            if (head) G[ng + __popc(msk & lt)] = (int32_t)W.key[i];
            ng += __popc(msk);
        }
        __syncwarp();
        for (int a = ln; a < ng; a += 32) {
            const int I = G[a];
            const uint64_t b0 = Q.rowWord[I] * 64;
            for (int b = 0; b <= a; ++b) {
                const uint64_t bit = b0 + (uint64_t)(G[b] - 1);
                unsigned long long *wd = Q.bits + (bit >> 6);
                const unsigned long long msk = 1ull << (bit & 63);
                if (!(*wd & msk)) atomicOr(wd, msk);
            }
        }
        __syncwarp();
    }
}

__device__ __forceinline__ int64_t warp_sum64(int64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__device__ __forceinline__ int64_t warp_incl64(int64_t v) {
    const int ln = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(kFull, v, o);
        if (ln >= o) v += y;
    }
    return v;
}

// per row group I: stored parameters of the row (inr), regions, list or
// region form, column words and matrix elements (ndbits, mpbits.f90:305-566)
__global__ void k_l2_rows(const unsigned long long *bits, const uint64_t *rowWord, const int32_t *aig, int32_t nG,
                          int64_t *nwOut, int64_t *nmOut, uint8_t *comp) {
    const int ln = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nG; w += nwarps) {
        const int I = (int)w + 1;
        const uint64_t r0 = rowWord[I];
        const int nwords = (I + 63) / 64;
        int64_t inr = 0, starts = 0;
        for (int k = ln; k < nwords; k += 32) {
            uint64_t m = bits[r0 + k];
            const uint64_t prevTop = k > 0 ? (bits[r0 + k - 1] >> 63) : 0ull;
            starts += __popcll(m & ~((m << 1) | prevTop));
            while (m) {
                const int J = 64 * k + __ffsll((long long)m);
                inr += aig[J] - aig[J - 1];
                m &= m - 1;
            }
        }
        inr = warp_sum64(inr);
        starts = warp_sum64(starts);
        if (ln == 0) {
            const int64_t irgn = 1 + starts;
            const bool c = inr > 0 && 2 * irgn < inr;
            nwOut[I - 1] = c ? 2 * irgn : inr;
            nmOut[I - 1] = inr * (int64_t)(aig[I] - aig[I - 1]);
            comp[I - 1] = c ? 1 : 0;
        }
    }
}

__global__ void k_l2_offsets(const int64_t *lb, const int64_t *ll, int64_t nd, int32_t nG, int64_t *offsets) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > nG) return;
    offsets[2 * i] = lb[i];
    offsets[2 * i + 1] = nd + ll[i];
}

// columns of row group I: parameter indices (list form) or (width before,
// first group) per region closed by (width, nG + 1) (region form)
__global__ void k_l2_columns(const unsigned long long *bits, const uint64_t *rowWord, const int32_t *aig,
                             int32_t nG, const int64_t *lb, const uint8_t *comp, int32_t *columns) {
    const int ln = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nG; w += nwarps) {
        const int I = (int)w + 1;
        const uint64_t r0 = rowWord[I];
        const int nwords = (I + 63) / 64;
        const int64_t kb = lb[I - 1];
        const bool c = comp[I - 1] != 0;
        int64_t width = 0, nst = 0;
        for (int base = 0; base < nwords; base += 32) {
            const int k = base + ln;
            const uint64_t m = k < nwords ? bits[r0 + k] : 0ull;
            const uint64_t prevTop = (k > 0 && k < nwords) ? (bits[r0 + k - 1] >> 63) : 0ull;
            const uint64_t st = m & ~((m << 1) | prevTop);
            int64_t wsum = 0;
            for (uint64_t t = m; t; t &= t - 1) {
                const int J = 64 * k + __ffsll((long long)t);
                wsum += aig[J] - aig[J - 1];
            }
            const int64_t ssum = __popcll(st);
            const int64_t wi = warp_incl64(wsum), si = warp_incl64(ssum);
            int64_t wpre = width + wi - wsum, spre = nst + si - ssum;
            width += __shfl_sync(kFull, wi, 31);
            nst += __shfl_sync(kFull, si, 31);
            for (uint64_t t = m; t; t &= t - 1) {
                const int b = __ffsll((long long)t) - 1;
                const int J = 64 * k + b + 1;
                const int32_t a0 = aig[J - 1], nj = aig[J] - a0;
                if (c) {
                    if ((st >> b) & 1ull) {
                        columns[kb + 2 * spre] = (int32_t)wpre;
                        columns[kb + 2 * spre + 1] = J;
                        spre++;
                    }
                } else {
                    for (int32_t q = 0; q < nj; ++q) columns[kb + wpre + q] = a0 + q;
                }
                wpre += nj;
            }
        }
        if (c && ln == 0) {
            columns[kb + 2 * nst] = (int32_t)width;
            columns[kb + 2 * nst + 1] = nG + 1;
        }
    }
}

// device buffers of one structure pass, freed at the end
struct Scratch {
    std::vector<void *> p;
    ~Scratch() {
        for (void *x : p) cudaFree(x);
    }
    template <class T>
    cudaError_t get(T *&out, int64_t n) {
        out = nullptr;
        if (n <= 0) n = 1;
        cudaError_t e = cudaMalloc((void **)&out, sizeof(T) * (size_t)n);
        if (e == cudaSuccess) p.push_back(out);
        return e;
    }
};

int32_t l1_status(unsigned long long err) {
    const int code = (int)(err & 0xff);
    if (code == MPGPU_ERR_BADINDEX) return -23;
    if (code == MPGPU_ERR_LIMIT) return -45;
    return -20;
}

}  // namespace

// ------------------------------------------------------------------ entries
void free_resident(ResidentRecords &R) {
    if (R.recPtr) cudaFree(R.recPtr);
    if (R.inder) cudaFree(R.inder);
    if (R.glder) cudaFree(R.glder);
    R = ResidentRecords{};
}

int32_t loop1_device(mpgpu_ctx *c, int64_t nrec, const int64_t *recPtr, const int32_t *inder, const double *glder,
                     int32_t nsteer, const int32_t *steerLabels, int32_t npre, const int32_t *preLabel,
                     const double *preSigma, int32_t mreqenf, int32_t cap, int32_t *labels, int64_t *counter,
                     int32_t *varIndex, int32_t *totGroup, int32_t *nVar, int32_t *nVarGroups) {
    cudaStream_t s = c->stream;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    ResidentRecords &R = c->res;
    free_resident(R);
    const int64_t nw = recPtr[nrec] - recPtr[0];
    if (nw < 0) return -20;
    auto cu = [&](cudaError_t e) { return e == cudaSuccess; };
    if (!cu(cudaMalloc((void **)&R.recPtr, sizeof(int64_t) * (size_t)(nrec + 1))) ||
        !cu(cudaMalloc((void **)&R.inder, sizeof(int32_t) * (size_t)std::max<int64_t>(nw, 1))) ||
        !cu(cudaMalloc((void **)&R.glder, sizeof(double) * (size_t)std::max<int64_t>(nw, 1)))) {
        free_resident(R);
        set_err(c, MPGPU_ERR_ALLOC, "loop1: records do not fit on the device");
        return -30;
    }
    R.nrec = nrec;
    R.nw = nw;
    R.w0 = recPtr[0];
    Scratch S;
    int32_t rc = 0;
#define L1_CUDA(x)                                                   \
    do {                                                             \
        cudaError_t e_ = (x);                                        \
        if (e_ != cudaSuccess) {                                     \
            set_err(c, MPGPU_ERR_CUDA, cudaGetErrorString(e_));      \
            free_resident(R);                                        \
            return -43;                                              \
        }                                                            \
    } while (0)
    L1_CUDA(cudaMemcpyAsync(R.recPtr, recPtr, sizeof(int64_t) * (nrec + 1), cudaMemcpyHostToDevice, s));
    // the records in chunks on the second stream; the label collection of a
    // chunk starts when its copy is done
    const int nchunk = nw > ((int64_t)64 << 20) ? 8 : 1;
    std::vector<int64_t> cr(nchunk + 1);
    for (int k = 0; k <= nchunk; ++k) cr[k] = nrec * k / nchunk;
    struct Events {
        std::vector<cudaEvent_t> e;
        ~Events() {
            for (auto x : e) cudaEventDestroy(x);
        }
    } ev;
    ev.e.resize(nchunk);
    for (auto &x : ev.e) L1_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    for (int k = 0; k < nchunk; ++k) {
        const int64_t a = recPtr[cr[k]], b = recPtr[cr[k + 1]];
        if (b > a) {
            L1_CUDA(cudaMemcpyAsync(R.inder + (a - recPtr[0]), inder + a, sizeof(int32_t) * (b - a),
                                    cudaMemcpyHostToDevice, c->stream2));
            L1_CUDA(cudaMemcpyAsync(R.glder + (a - recPtr[0]), glder + a, sizeof(double) * (b - a),
                                    cudaMemcpyHostToDevice, c->stream2));
        }
        L1_CUDA(cudaEventRecord(ev.e[k], c->stream2));
    }
    // scalars: error word, distinct count, probe failure, overflow count
    unsigned long long *dErr;
    L1_CUDA(S.get(dErr, 4));
    unsigned int *dCount = (unsigned int *)(dErr + 1);
    int *dFail = (int *)(dErr + 2);
    int32_t *dOvN = (int32_t *)(dErr + 3);
    int64_t *ovList;
    L1_CUDA(S.get(ovList, nrec));
    int32_t *dSteer = nullptr;
    if (nsteer > 0) {
        L1_CUDA(S.get(dSteer, nsteer));
        L1_CUDA(cudaMemcpyAsync(dSteer, steerLabels, sizeof(int32_t) * nsteer, cudaMemcpyHostToDevice, s));
    }
    L1Params P{};
    P.nrec = nrec; P.recPtr = R.recPtr; P.inder = R.inder; P.glder = R.glder;
    P.count = dCount; P.fail = dFail; P.err = dErr; P.ovList = ovList; P.ovCount = dOvN;
    const int smemS = kL1Warps * (int)sizeof(UpWarp<false>), smemB = kL1Warps * (int)sizeof(UpWarp<true>);
    L1_CUDA(smem_optin((const void *)k_l1_collect<false>));
    L1_CUDA(smem_optin((const void *)k_l1_collect<true>));
    L1_CUDA(smem_optin((const void *)k_l1_translate<false>));
    L1_CUDA(smem_optin((const void *)k_l1_translate<true>));
    int perSm = 0;
    L1_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_l1_collect<false>, 32 * kL1Warps, smemS));
    const unsigned gS = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((nrec + kL1Warps - 1) / kL1Warps, (int64_t)nsm * std::max(perSm, 1)));
    const unsigned gB = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nrec, (int64_t)nsm * 2));
    // ---- 1. hash set of the labels (rebuilt larger when too full)
    int64_t H = (int64_t)1 << 22;
    while (H < 4 * (int64_t)nsteer) H <<= 1;
    int32_t *tab = nullptr;
    unsigned int hCount = 0;
    for (;;) {
        if (tab) {
            cudaFree(tab);
            S.p.erase(std::find(S.p.begin(), S.p.end(), (void *)tab));
        }
        L1_CUDA(S.get(tab, H));
        L1_CUDA(cudaMemsetAsync(tab, 0, sizeof(int32_t) * H, s));
        L1_CUDA(cudaMemsetAsync(dErr, 0xff, 8, s));
        L1_CUDA(cudaMemsetAsync(dErr + 1, 0, 24, s));
        P.tab = tab;
        P.mask = (uint64_t)(H - 1);
        if (nsteer > 0) k_l1_steer<<<blocks_for(nsteer), 256, 0, s>>>(dSteer, nsteer, tab, P.mask, dCount, dFail);
        for (int k = 0; k < nchunk; ++k) {
            L1_CUDA(cudaStreamWaitEvent(s, ev.e[k], 0));
            P.rBegin = cr[k];
            P.rEnd = cr[k + 1];
            if (P.rEnd > P.rBegin) k_l1_collect<false><<<gS, 32 * kL1Warps, smemS, s>>>(P);
        }
        if (nrec > 0) k_l1_collect<true><<<gB, 32 * kL1Warps, smemB, s>>>(P);
        L1_CUDA(cudaGetLastError());
        unsigned long long h[4];
        L1_CUDA(cudaMemcpyAsync(h, dErr, sizeof(h), cudaMemcpyDeviceToHost, s));
        L1_CUDA(cudaStreamSynchronize(s));
        if (h[0] != ~0ull) {
            rc = l1_status(h[0]);
            char buf[96];
            snprintf(buf, sizeof buf, "loop1: record %lld rejected (code %d)", (long long)(h[0] >> 8),
                     (int)(h[0] & 0xff));
            set_err(c, rc == -23 ? MPGPU_ERR_BADINDEX : rc == -45 ? MPGPU_ERR_LIMIT : MPGPU_ERR_BADRECORD, buf);
            free_resident(R);
            return rc;
        }
        hCount = (unsigned int)(h[1] & 0xffffffffu);
        const int fail = (int)(h[2] & 0xffffffffu);
        if (!fail && 2 * (int64_t)hCount <= H) break;
        if (H >= ((int64_t)1 << 31)) {
            set_err(c, MPGPU_ERR_LIMIT, "loop1: too many distinct labels for the label set");
            free_resident(R);
            return -45;
        }
        H = std::min<int64_t>(H << 3, (int64_t)1 << 31);
    }
    const int64_t n = hCount;
    if (n > cap) {
        free_resident(R);
        return -1;
    }
    // ---- 2. distinct labels, sorted; total index beside each slot
    int64_t *flag, *scanTmp, *hist;
    L1_CUDA(S.get(flag, H + 1));
    L1_CUDA(S.get(scanTmp, scan_tmp_len(std::max<int64_t>(H + 1, 256 * ((n + kRsTile - 1) / kRsTile) + 1))));
    k_l1_occupied<<<blocks_for(H + 1), 256, 0, s>>>(tab, H, flag);
    L1_CUDA(scan_ex(flag, flag, H + 1, scanTmp, s));
    uint64_t *k0, *k1;
    uint32_t *v0, *v1;
    L1_CUDA(S.get(k0, n)); L1_CUDA(S.get(k1, n)); L1_CUDA(S.get(v0, n)); L1_CUDA(S.get(v1, n));
    L1_CUDA(S.get(hist, 256 * ((n + kRsTile - 1) / kRsTile) + 1));
    k_l1_compact<<<blocks_for(H), 256, 0, s>>>(tab, H, flag, k0, v0);
    SortBufs sb{k0, k1, v0, v1, hist, scanTmp};
    L1_CUDA(radix_sort(sb, n, 31, s));
    int32_t *slotIdx, *dLabels;
    L1_CUDA(S.get(slotIdx, H));
    L1_CUDA(S.get(dLabels, n));
    if (n > 0) k_l1_index<<<blocks_for(n), 256, 0, s>>>(sb.k0, sb.v0, n, slotIdx, dLabels);
    // ---- 3. translation, entries, group cuts
    // entries in 32 copies (fewer for large tables), chosen by the block, so
    // that the increments of one label spread over several addresses
    const int copies = n <= ((int64_t)1 << 20) ? 32 : 1;
    unsigned long long *cnt;
    uint8_t *seen, *cut;
    L1_CUDA(S.get(cnt, copies * n));
    L1_CUDA(S.get(seen, n));
    L1_CUDA(S.get(cut, n + 1));
    L1_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * std::max<int64_t>(copies * n, 1), s));
    L1_CUDA(cudaMemsetAsync(seen, 0, std::max<int64_t>(n, 1), s));
    L1_CUDA(cudaMemsetAsync(cut, 0, n + 1, s));
    P.slotIdx = slotIdx; P.cnt = cnt; P.ncnt = n; P.cntCopies = copies; P.seen = seen; P.cut = cut;
    P.rBegin = 0;
    P.rEnd = nrec;
    if (nrec > 0) {
        k_l1_translate<false><<<gS, 32 * kL1Warps, smemS, s>>>(P);
        k_l1_translate<true><<<gB, 32 * kL1Warps, smemB, s>>>(P);
    }
    if (n > 0 && copies > 1) k_l1_cnt_sum<<<blocks_for(n), 256, 0, s>>>(cnt, n, copies);
    L1_CUDA(cudaGetLastError());
    // ---- 4. the per-label arrays to the host; last step as on the host
    std::vector<int32_t> all(n);
    std::vector<int64_t> hcnt(n);
    std::vector<uint8_t> hseen(n), hcut(n + 1);
    if (n > 0) {
        L1_CUDA(cudaMemcpyAsync(all.data(), dLabels, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
        L1_CUDA(cudaMemcpyAsync(hcnt.data(), cnt, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
        L1_CUDA(cudaMemcpyAsync(hseen.data(), seen, n, cudaMemcpyDeviceToHost, s));
        L1_CUDA(cudaMemcpyAsync(hcut.data(), cut, n + 1, cudaMemcpyDeviceToHost, s));
    }
    L1_CUDA(cudaStreamSynchronize(s));
#undef L1_CUDA
    R.translated = true;
    R.nTotal = (int32_t)n;
    return labels_finish(all, hcnt, hcut, hseen, npre, preLabel, preSigma, mreqenf, labels, counter, varIndex,
                         totGroup, nVar, nVarGroups);
}

int32_t loop2_device(mpgpu_ctx *c, const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                     const int32_t *allIndexGroups, int64_t cap, int64_t *offsets, int32_t *columns,
                     int64_t *ncolw, int64_t *nmat) {
    ResidentRecords &R = c->res;
    if (!R.translated || R.nrec < 0) {
        set_err(c, MPGPU_ERR_ARG, "loop2: no records kept by mpgpu_loop1_device");
        return MPGPU_ERR_ARG;
    }
    cudaStream_t s = c->stream;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    const int64_t nrec = R.nrec;
    std::vector<int32_t> p2g(std::max(nVar, 1));
    for (int32_t g = 1; g <= nG; ++g)
        for (int32_t v = allIndexGroups[g - 1]; v < allIndexGroups[g]; ++v) {
            if (v < 1 || v > nVar) return set_err(c, MPGPU_ERR_SIZE, "loop2: bad group table");
            p2g[v - 1] = g;
        }
    std::vector<uint64_t> rowWord(nG + 2, 0);
    for (int32_t I = 1; I <= nG; ++I) rowWord[I + 1] = rowWord[I] + ((uint64_t)I + 63) / 64;
    const int64_t nbits = (int64_t)rowWord[nG + 1] + 1;
    Scratch S;
    int32_t *dVar, *dAig, *dP2g;
    uint64_t *dRow;
    unsigned long long *bits, *dErr;
    int64_t *ovList, *nwA, *nmA, *scanTmp, *dOff;
    uint8_t *comp;
    MPG_CUDA(c, S.get(dVar, R.nTotal));
    MPG_CUDA(c, S.get(dAig, nG + 1));
    MPG_CUDA(c, S.get(dP2g, nVar));
    MPG_CUDA(c, S.get(dRow, nG + 2));
    MPG_CUDA(c, S.get(bits, nbits));
    MPG_CUDA(c, S.get(dErr, 2));
    MPG_CUDA(c, S.get(ovList, nrec));
    MPG_CUDA(c, S.get(nwA, nG + 1));
    MPG_CUDA(c, S.get(nmA, nG + 1));
    MPG_CUDA(c, S.get(comp, nG));
    MPG_CUDA(c, S.get(dOff, 2 * (int64_t)(nG + 1)));
    MPG_CUDA(c, S.get(scanTmp, scan_tmp_len(nG + 1)));
    MPG_CUDA(c, cudaMemcpyAsync(dVar, varIndexOfTotal, sizeof(int32_t) * R.nTotal, cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, cudaMemcpyAsync(dAig, allIndexGroups, sizeof(int32_t) * (nG + 1), cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, cudaMemcpyAsync(dP2g, p2g.data(), sizeof(int32_t) * nVar, cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, cudaMemcpyAsync(dRow, rowWord.data(), sizeof(uint64_t) * (nG + 2), cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, cudaMemsetAsync(bits, 0, sizeof(unsigned long long) * nbits, s));
    MPG_CUDA(c, cudaMemsetAsync(dErr, 0xff, 8, s));
    MPG_CUDA(c, cudaMemsetAsync(dErr + 1, 0, 8, s));
    MPG_CUDA(c, cudaMemsetAsync(nwA, 0, sizeof(int64_t) * (nG + 1), s));
    MPG_CUDA(c, cudaMemsetAsync(nmA, 0, sizeof(int64_t) * (nG + 1), s));
    L2Params Q{};
    UpParams &P = Q.up;
    P.nrec = nrec; P.recPtr = R.recPtr; P.inder = R.inder; P.glder = R.glder;
    P.varOfTot = dVar; P.nTotal = R.nTotal; P.p2g = dP2g; P.aig = dAig; P.nVar = nVar; P.nG = nG;
    P.err = dErr; P.ovList = ovList; P.ovCount = (int32_t *)(dErr + 1);
    Q.rowWord = dRow;
    Q.bits = bits;
    const int smemS = kL1Warps * (int)sizeof(UpWarp<false>), smemB = kL1Warps * (int)sizeof(UpWarp<true>);
    MPG_CUDA(c, smem_optin((const void *)k_l2_bits<false>));
    MPG_CUDA(c, smem_optin((const void *)k_l2_bits<true>));
    int perSm = 0;
    MPG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_l2_bits<false>, 32 * kL1Warps, smemS));
    const unsigned gS = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((nrec + kL1Warps - 1) / kL1Warps, (int64_t)nsm * std::max(perSm, 1)));
    const unsigned gB = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nrec, (int64_t)nsm * 2));
    if (nrec > 0) {
        k_l2_bits<false><<<gS, 32 * kL1Warps, smemS, s>>>(Q);
        k_l2_bits<true><<<gB, 32 * kL1Warps, smemB, s>>>(Q);
    }
    const unsigned gRows = blocks_for(32 * (int64_t)std::max(nG, 1));
    k_l2_rows<<<gRows, 256, 0, s>>>(bits, dRow, dAig, nG, nwA, nmA, comp);
    MPG_CUDA(c, scan_ex(nwA, nwA, nG + 1, scanTmp, s));
    MPG_CUDA(c, scan_ex(nmA, nmA, nG + 1, scanTmp, s));
    const int64_t nd = allIndexGroups[nG] - allIndexGroups[0];
    k_l2_offsets<<<blocks_for(nG + 1), 256, 0, s>>>(nwA, nmA, nd, nG, dOff);
    MPG_CUDA(c, cudaGetLastError());
    unsigned long long herr = 0;
    MPG_CUDA(c, cudaMemcpyAsync(&herr, dErr, 8, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaMemcpyAsync(offsets, dOff, sizeof(int64_t) * 2 * (nG + 1), cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    if (herr != ~0ull) {
        char buf[96];
        snprintf(buf, sizeof buf, "loop2: record %lld rejected (code %d)", (long long)(herr >> 8),
                 (int)(herr & 0xff));
        return set_err(c, (int32_t)(herr & 0xff), buf);
    }
    const int64_t lb = offsets[2 * nG];
    *ncolw = lb;
    *nmat = offsets[2 * nG + 1];
    if (lb > cap) return -1;
    int32_t *dCol;
    MPG_CUDA(c, S.get(dCol, lb));
    k_l2_columns<<<gRows, 256, 0, s>>>(bits, dRow, dAig, nG, nwA, comp, dCol);
    MPG_CUDA(c, cudaGetLastError());
    if (lb > 0) MPG_CUDA(c, cudaMemcpyAsync(columns, dCol, sizeof(int32_t) * lb, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    return 0;
}
