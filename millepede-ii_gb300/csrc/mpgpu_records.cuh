// mpgpu_records.cuh -- device building blocks shared by the record
// preparation (mpgpu_upload.cu) and the structure passes (mpgpu_struct.cu):
// exclusive scan, stable LSD radix sort, and the per-record analysis
// (measurement decode, sorted variable words, slots, parameter groups),
// run by one warp per record.  Everything is internal to the including
// translation unit.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "mpgpu_ctx.h"

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kUpWarps = 4;          // warps per CTA of the record kernels
constexpr int kEqMax = 512;          // measurements per record
constexpr int kSwMax = 512;          // variable global words per record
constexpr int kWordsMax = 2048;      // records up to this length are decoded from shared memory

// ------------------------------------------------------------ exclusive scan
constexpr int kScanThreads = 256, kScanItems = 16, kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int64_t *in, int64_t *out, int64_t n,
                                                             int64_t *tileSum) {
    __shared__ int64_t ws[kScanThreads / 32];
    const int ln = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    int64_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(kFull, x, o);
        if (ln >= o) x += y;
    }
    if (ln == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t t = ln < kScanThreads / 32 ? ws[ln] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(kFull, t, o);
            if (ln >= o) t += y;
        }
        if (ln < kScanThreads / 32) ws[ln] = t;
    }
    __syncthreads();
    int64_t e = x - s + (w > 0 ? ws[w - 1] : 0);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = e;
        e += v[i];
    }
    if (threadIdx.x == kScanThreads - 1) tileSum[blockIdx.x] = e;
}

__global__ void k_scan_add(int64_t *out, int64_t n, const int64_t *tileOff) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tileOff[i / kScanTile];
}

int64_t scan_tmp_len(int64_t n) {
    int64_t t = 0;
    while (n > 1) {
        n = (n + kScanTile - 1) / kScanTile;
        t += n + 1;
    }
    return t + 2;
}

// out[i] = sum of in[0..i) for i < n (in place allowed); tmp holds
// scan_tmp_len(n) elements
cudaError_t scan_ex(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t nt = (n + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<(unsigned)nt, kScanThreads, 0, s>>>(in, out, n, tmp);
    if (nt > 1) {
        cudaError_t e = scan_ex(tmp, tmp, nt, tmp + nt + 1, s);
        if (e != cudaSuccess) return e;
        k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, tmp);
    }
    return cudaGetLastError();
}

// ------------------------------------------------- stable LSD radix sort
constexpr int kRsThreads = 256, kRsItems = 16, kRsTile = kRsThreads * kRsItems;

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint64_t *keys, int64_t n, int shift,
                                                        int64_t ntiles, int64_t *hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * kRsTile;
    for (int i = 0; i < kRsItems; ++i) {
        const int64_t idx = t0 + (int64_t)i * kRsThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Entries of a tile are taken in index order (16 rounds of 256); the rank
// of an entry among equal digits is its warp rank plus the counts of the
// earlier warps of the round and of the earlier rounds: stable.
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint64_t *kin, const uint32_t *vin,
                                                           uint64_t *kout, uint32_t *vout, int64_t n,
                                                           int shift, int64_t ntiles, const int64_t *off) {
    __shared__ int wcnt[kRsThreads / 32][256];
    __shared__ int pre[kRsThreads / 32][256];
    __shared__ int run[256];
    const int t = threadIdx.x, w = t >> 5, ln = t & 31;
    run[t] = 0;
    const int64_t t0 = (int64_t)blockIdx.x * kRsTile;
    for (int rd = 0; rd < kRsItems; ++rd) {
        const int64_t idx = t0 + (int64_t)rd * kRsThreads + t;
        const bool valid = idx < n;
        const uint64_t k = valid ? kin[idx] : 0;
        const uint32_t v = valid ? vin[idx] : 0;
        const int d = valid ? (int)((k >> shift) & 255) : 256;
#pragma unroll
        for (int q = 0; q < kRsThreads / 32; ++q) wcnt[q][t] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(kFull, d);
        const int rank = __popc(peers & ((1u << ln) - 1));
        if (valid && ln == __ffs(peers) - 1) wcnt[w][d] = __popc(peers);
        __syncthreads();
        int acc = run[t];
#pragma unroll
        for (int q = 0; q < kRsThreads / 32; ++q) {
            pre[q][t] = acc;
            acc += wcnt[q][t];
        }
        run[t] = acc;
        __syncthreads();
        if (valid) {
            const int64_t pos = off[(int64_t)d * ntiles + blockIdx.x] + pre[w][d] + rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

struct SortBufs {
    uint64_t *k0, *k1;
    uint32_t *v0, *v1;
    int64_t *hist;     // 256 * ntiles + 1
    int64_t *scanTmp;
};

int bits_for(uint64_t maxKey) {
    int b = 1;
    while (b < 64 && (maxKey >> b) != 0) b++;
    return b;
}

// sorts (k0, v0)[0..n) by the low `bits` bits of the key, stably; the result
// is left in (k0, v0) (buffers are swapped as needed)
cudaError_t radix_sort(SortBufs &b, int64_t n, int bits, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    const int64_t nt = (n + kRsTile - 1) / kRsTile;
    for (int shift = 0; shift < bits; shift += 8) {
        k_rs_hist<<<(unsigned)nt, kRsThreads, 0, s>>>(b.k0, n, shift, nt, b.hist);
        cudaError_t e = scan_ex(b.hist, b.hist, 256 * nt, b.scanTmp, s);
        if (e != cudaSuccess) return e;
        k_rs_scatter<<<(unsigned)nt, kRsThreads, 0, s>>>(b.k0, b.v0, b.k1, b.v1, n, shift, nt, b.hist);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(b.k0, b.k1);
        std::swap(b.v0, b.v1);
    }
    return cudaSuccess;
}

// ------------------------------------------------------------ record kernels
struct UpParams {
    int64_t nrec;
    const int64_t *recPtr;     // device, nrec + 1 (absolute word offsets)
    const int32_t *inder;      // device words from recPtr[0]
    const double *glder;
    const int32_t *recFile;    // may be null
    int32_t nfiles;
    const int32_t *varOfTot;
    int32_t nTotal;
    const int32_t *p2g;        // [nVar]
    const int32_t *aig;        // [nG+1]
    int32_t nVar, nG;
    RecInfo *rec;
    int64_t *cnt;              // 6 arrays of nrec + 1: eq, slot, sw, grp, pair, stage
    unsigned long long *err;   // min over (record << 8 | code)
    int32_t *maxv;             // nw neq nalc nalg ngrp band bdr nbndr1 nbndr2
    int64_t *ovList;           // records beyond the compact capacity (filled by k_up_scan<false>)
    int64_t rBegin, rEnd;      // records of a compact-kernel launch
    int32_t *ovCount;
    // tables (fill)
    const int64_t *off;        // 6 scanned arrays of nrec + 1
    int32_t *meas, *slots, *slotCnt, *swStart, *sw, *grpId, *grpSlot, *grpRec;
};

// Two variants of the record kernels.  The compact one keeps the shared
// memory of a warp small enough for 32 warps per SM (records of up to 512
// words, 128 measurements, 256 variable global words: tracks of a few tens
// of hits); the large one takes records up to the global limits at 8 warps
// per SM.  The compact kernels hand every record beyond their capacity to
// the large ones through an overflow list.  Both run the same analysis, so
// a record's tables and status do not depend on the variant.
template <bool BIG> struct UpCap;
template <> struct UpCap<false> {
    static constexpr int kWords = 512, kEq = 128, kSw = 256, kMinBlocks = 8;
};
template <> struct UpCap<true> {
    static constexpr int kWords = kWordsMax, kEq = kEqMax, kSw = kSwMax, kMinBlocks = 1;
};
constexpr int kOverflow = -1;   // analysis result: beyond the compact capacity

template <bool BIG> struct UpWarp {
    int32_t words[UpCap<BIG>::kWords];
    int32_t eq[3 * UpCap<BIG>::kEq];
    uint64_t key[UpCap<BIG>::kSw];     // after the analysis: band table of k_up_scan
    int32_t slotStart[UpCap<BIG>::kSw + 1];
    int32_t misc[4];
};
static_assert(sizeof(uint64_t) * 256 >= sizeof(int32_t) * (2 * MPG_NALC_MAX + 4), "band table in the key array");

// the large kernels reject what exceeds their capacity, the compact ones defer it
template <bool BIG> __device__ __forceinline__ int cap_code() { return BIG ? MPGPU_ERR_LIMIT : kOverflow; }

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

__device__ __forceinline__ int key_var(uint64_t k) { return (int)(k >> 40); }
__device__ __forceinline__ int key_eq(uint64_t k) { return (int)((k >> 16) & 0xffffff); }
__device__ __forceinline__ int key_word(uint64_t k) { return (int)(k & 0xffff); }

// first p in [from, end] with in[p] == 0, or -1 (warp-wide)
__device__ int next_zero(const int32_t *in, int from, int end) {
    const int ln = threadIdx.x & 31;
    for (int b = from; b <= end; b += 32) {
        const int p = b + ln;
        const bool z = p <= end && in[p] == 0;
        const unsigned m = __ballot_sync(kFull, z);
        if (m) return b + __ffs(m) - 1;
    }
    return -1;
}

// decodeNextMeasurement (pede.f90:2428-2468) over the whole record: the
// measurements as (sl, sg, lg) word triples in W.eq.  The zero index words delimit the
// blocks; without special data blocks they alternate local start, global
// start, so one ballot pass over the record gives every triple.  A record
// with a possible special block (two adjacent zero words, the second with a
// negative value), an odd number of zero words or none takes the sequential
// decode, which also reports malformed records.
template <bool BIG>
__device__ int decode_measurements(const int32_t *in, const double *gl, int end, UpWarp<BIG> &W,
                                   int &neqOut) {
    constexpr int CAP = UpCap<BIG>::kEq;
    const int ln = threadIdx.x & 31;
    const unsigned lt = (1u << ln) - 1u;
    int nz = 0, cand = 0;
    for (int b = 1; b <= end; b += 32) {
        const int p = b + ln;
        const bool z = p <= end && in[p] == 0;
        const unsigned m = __ballot_sync(kFull, z);
        if (z) {
            const int idx = nz + __popc(m & lt), e = idx >> 1;
            if (e < CAP) W.eq[3 * e + (idx & 1)] = p;
            // a local start closes the previous measurement
            if ((idx & 1) == 0 && e >= 1 && e <= CAP) W.eq[3 * (e - 1) + 2] = p - 1;
            if (p >= 2 && in[p - 1] == 0 && gl[p] < 0.0) cand = 1;
        }
        nz += __popc(m);
    }
    cand = __any_sync(kFull, cand);
    if (!cand && (nz & 1) == 0 && (nz > 0 || end <= 0)) {
        const int neq = nz >> 1;
        if (neq > CAP) return cap_code<BIG>();
        if (ln == 0 && neq > 0) W.eq[3 * (neq - 1) + 2] = end;
        __syncwarp();
        neqOut = neq;
        return 0;
    }
    __syncwarp();
    int lg = 0, neq = 0;
    for (int guard = 0; guard < MPG_WORDS_MAX + 2; ++guard) {
        if (lg >= end) break;
        const int sl = next_zero(in, lg + 1, end);
        if (sl < 0) return MPGPU_ERR_BADRECORD;
        const int sg = next_zero(in, sl + 1, end);
        if (sg < 0) return MPGPU_ERR_BADRECORD;
        if (sl + 1 == sg && gl[sg] < 0.0) {  // special data block
            lg = sg + (int)(-gl[sg] + 0.5);
            continue;
        }
        const int nzp = next_zero(in, sg + 1, end);
        lg = nzp < 0 ? end : nzp - 1;
        if (neq >= CAP) return cap_code<BIG>();
        if (ln == 0) {
            W.eq[3 * neq] = sl;
            W.eq[3 * neq + 1] = sg;
            W.eq[3 * neq + 2] = lg;
        }
        neq++;
    }
    __syncwarp();
    neqOut = neq;
    return 0;
}

// ascending bitonic sort of 32 * PER keys held in registers, element
// lane * PER + k in a[k]: strides below PER inside a lane, the others by
// shuffles between lanes
template <int PER>
__device__ __forceinline__ void sort_regs(uint64_t (&a)[PER]) {
    const int ln = threadIdx.x & 31;
#pragma unroll
    for (int kk = 2; kk <= 32 * PER; kk <<= 1) {
#pragma unroll
        for (int jj = kk >> 1; jj > 0; jj >>= 1) {
            if (jj >= PER) {
                const int lm = jj / PER;
                const bool lower = (ln & lm) == 0;
#pragma unroll
                for (int k = 0; k < PER; ++k) {
                    const bool up = ((ln * PER + k) & kk) == 0;
                    const uint64_t b = __shfl_xor_sync(kFull, a[k], lm);
                    const bool takeMin = lower == up;
                    const bool bSmaller = b < a[k];
                    a[k] = (takeMin == bSmaller) ? b : a[k];
                }
            } else {
#pragma unroll
                for (int k = 0; k < PER; ++k) {
                    const int k2 = k ^ jj;
                    if (k2 > k) {
                        const bool up = ((ln * PER + k) & kk) == 0;
                        const uint64_t x = a[k], y = a[k2];
                        const bool sw = (x > y) == up;
                        a[k] = sw ? y : x;
                        a[k2] = sw ? x : y;
                    }
                }
            }
        }
    }
}

template <int PER, bool BIG>
__device__ __forceinline__ void sort_keys_regs(UpWarp<BIG> &W, int nsw) {
    const int ln = threadIdx.x & 31;
    uint64_t a[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int i = ln * PER + k;
        a[k] = i < nsw ? W.key[i] : ~0ull;
    }
    sort_regs<PER>(a);
    __syncwarp();
#pragma unroll
    for (int k = 0; k < PER; ++k) W.key[ln * PER + k] = a[k];
    __syncwarp();
}

// bitonic sort in shared memory (large records beyond 256 keys)
template <bool BIG>
__device__ void sort_keys_smem(UpWarp<BIG> &W, int nsw) {
    const int ln = threadIdx.x & 31;
    int P2 = 32;
    while (P2 < nsw) P2 <<= 1;
    for (int i = nsw + ln; i < P2; i += 32) W.key[i] = ~0ull;
    __syncwarp();
    for (int k = 2; k <= P2; k <<= 1)
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int i = ln; i < P2; i += 32) {
                const int ixj = i ^ jj;
                if (ixj > i) {
                    const uint64_t a = W.key[i], b = W.key[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) { W.key[i] = b; W.key[ixj] = a; }
                }
            }
            __syncwarp();
        }
}

struct RecShape {
    int code;          // 0, a status code or kOverflow
    int nw, neq, nalc, nsw, nalg, ngrp;
    bool nonmono, denseLoc, simpleWords;
};

// decode + sorted variable words + slots + groups of record r (warp-wide);
// the SMEM of the warp holds the equations, the sorted keys and the slot
// starts afterwards
template <bool BIG>
__device__ RecShape analyze(const UpParams &P, int64_t r, UpWarp<BIG> &W, bool checks) {
    constexpr int CAPW = UpCap<BIG>::kWords, CAPSW = UpCap<BIG>::kSw;
    const int ln = threadIdx.x & 31;
    const unsigned lt = (1u << ln) - 1u;
    RecShape R{};
    const int64_t w0 = P.recPtr[r] - P.recPtr[0];
    const int64_t nw64 = P.recPtr[r + 1] - P.recPtr[r];
    const int32_t *in = P.inder + w0;
    const double *gl = P.glder + w0;
    if (nw64 < 1 || nw64 > MPG_WORDS_MAX) { R.code = MPGPU_ERR_BADRECORD; return R; }
    const int nw = (int)nw64, end = nw - 1;
    R.nw = nw;
    // the record's index words in shared memory (one coalesced pass) when
    // they fit; the decode then reads shared memory only
    if (nw <= CAPW) {
        for (int i = ln; i < nw; i += 32) W.words[i] = in[i];
        __syncwarp();
        in = W.words;
    }
    int neq = 0;
    R.code = decode_measurements<BIG>(in, gl, end, W, neq);
    if (R.code != 0) return R;
    R.neq = neq;
    // locals
    int nalc = 0, nonmono = 0, badl = 0;
    for (int e = ln; e < neq; e += 32) {
        const int sl = W.eq[3 * e], sg = W.eq[3 * e + 1];
        int prev = 0;
        for (int q = sl + 1; q < sg; ++q) {
            const int li = in[q];
            if (li <= 0) badl = 1;
            nalc = max(nalc, li);
            if (li <= prev) nonmono = 1;
            prev = li;
        }
    }
    if (__any_sync(kFull, badl)) { R.code = MPGPU_ERR_BADRECORD; return R; }
    nalc = warp_max(nalc);
    R.nalc = nalc;
    R.nonmono = __any_sync(kFull, nonmono) != 0;
    int notDense = nalc <= 0;
    for (int e = ln; e < neq; e += 32) {
        const int sl = W.eq[3 * e], sg = W.eq[3 * e + 1];
        if (sg - sl - 1 != nalc) notDense = 1;
        for (int q = sl + 1; !notDense && q < sg; ++q)
            if (in[q] != q - sl) notDense = 1;
    }
    R.denseLoc = !__any_sync(kFull, notDense);
    // variable global words as sort keys (var, equation, word), placed by
    // ballots (lane = measurement, step = word of the measurement); the
    // loads of eight words are issued together
    int nsw = 0, badg = 0;
    for (int e0 = 0; e0 < neq; e0 += 32) {
        const int e = e0 + ln;
        int q0 = 0, len = 0;
        if (e < neq) {
            q0 = W.eq[3 * e + 1] + 1;
            len = W.eq[3 * e + 2] - q0 + 1;
        }
        const int lmax = warp_max(len);
        for (int t0 = 0; t0 < lmax; t0 += 8) {
            int v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                v[u] = 0;
                if (t0 + u < len) {
                    const int ti = in[q0 + t0 + u];
                    if (ti < 1 || ti > P.nTotal) badg = 1;
                    else v[u] = P.varOfTot[ti - 1];
                }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const unsigned m = __ballot_sync(kFull, v[u] > 0);
                if (v[u] > 0) {
                    const int k = nsw + __popc(m & lt);
                    if (k < CAPSW)
                        W.key[k] = ((uint64_t)v[u] << 40) | ((uint64_t)e << 16) | (uint64_t)(q0 + t0 + u);
                }
                nsw += __popc(m);
            }
        }
    }
    __syncwarp();
    if (__any_sync(kFull, badg)) { R.code = MPGPU_ERR_BADINDEX; return R; }
    if (nsw > CAPSW) { R.code = cap_code<BIG>(); return R; }
    R.nsw = nsw;
    // sort of the keys (they are distinct: the word position is part of them)
    if (nsw <= 32) sort_keys_regs<1>(W, nsw);
    else if (nsw <= 64) sort_keys_regs<2>(W, nsw);
    else if (nsw <= 128) sort_keys_regs<4>(W, nsw);
    else if (nsw <= 256) sort_keys_regs<8>(W, nsw);
    else if constexpr (BIG) sort_keys_smem<BIG>(W, nsw);
    // distinct variables (slots) and their word-list starts
    int nalg = 0, dup = 0;
    for (int base = 0; base < nsw; base += 32) {
        const int i = base + ln;
        bool head = false;
        if (i < nsw) {
            head = i == 0 || key_var(W.key[i]) != key_var(W.key[i - 1]);
            if (!head && key_eq(W.key[i]) == key_eq(W.key[i - 1])) dup = 1;
        }
        const unsigned m = __ballot_sync(kFull, head);
        if (head) W.slotStart[nalg + __popc(m & lt)] = i;
        nalg += __popc(m);
    }
    if (ln == 0) W.slotStart[nalg] = nsw;
    __syncwarp();
    R.nalg = nalg;
    // groups of the sorted slots; every slot of a group must have the
    // equation list of the group's first slot for the lockstep update
    int ngrp = 0, npar = 0, notSimple = dup;
    int lastHead = 0;
    for (int base = 0; base < nalg; base += 32) {
        const int s = base + ln;
        int g = 0;
        bool head = false;
        if (s < nalg) {
            g = P.p2g[key_var(W.key[W.slotStart[s]]) - 1];
            head = s == 0 || g != P.p2g[key_var(W.key[W.slotStart[s - 1]]) - 1];
            if (head) npar += P.aig[g] - P.aig[g - 1];
        }
        const unsigned m = __ballot_sync(kFull, head);
        ngrp += __popc(m);
        // first slot of the group of s
        const unsigned le = m & (ln == 31 ? kFull : ((1u << (ln + 1)) - 1));
        const int h = le ? base + 31 - __clz(le) : lastHead;
        if (s < nalg && !head && checks) {
            const int a0 = W.slotStart[h], a1 = W.slotStart[h + 1];
            const int b0 = W.slotStart[s], b1 = W.slotStart[s + 1];
            if (a1 - a0 != b1 - b0) notSimple = 1;
            else
                for (int q = 0; q < a1 - a0; ++q)
                    if (key_eq(W.key[a0 + q]) != key_eq(W.key[b0 + q])) { notSimple = 1; break; }
        }
        lastHead = __shfl_sync(kFull, h, 31);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) npar += __shfl_xor_sync(kFull, npar, o);
    R.ngrp = ngrp;
    R.simpleWords = !__any_sync(kFull, notSimple);
    if (checks) {
        if (nalc > 0 && npar != nalg) { R.code = MPGPU_ERR_GROUPS; return R; }
        if (ngrp > MPG_NGRP_MAX) { R.code = MPGPU_ERR_LIMIT; return R; }
    }
    return R;
}

unsigned blocks_for(int64_t n, int t = 256) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

}  // namespace
