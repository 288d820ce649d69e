// mpgpu_ctx.h -- device-resident state of one alignment job and the kernel
// interfaces shared by the translation units of libmpgpu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <set>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/mpgpu.h"

#define MPG_WARPS_FIT 8        // warps per CTA of the local-fit kernel
#define MPG_FIT_BUCKETS 8      // size classes of records for the fit launches
#define MPG_NALC_MAX 96        // largest local system handled by the fit kernel
#define MPG_NGRP_MAX 255       // parameter groups per record (entry encoding)
#define MPG_WORDS_MAX 65535    // words per record (16-bit word positions)

// Per-record description built once at upload (host pass over the records).
struct alignas(16) RecInfo {
    int64_t w0;        // first word (error-count word) in the record arrays
    int64_t measOff;   // first equation in the measurement table
    int64_t slotOff;   // first entry of the per-slot arrays (stride nalg+1)
    int64_t pairOff;   // first of the record's group pairs in the pair-destination table
    int64_t swOff;     // first entry of the slot-word lists
    int64_t grpOff;    // first entry of the group list
    int32_t nw, neq, nalc, nalg;
    int32_t ngrp;
    int16_t mbnd, mbdr;   // bordered band structure (mbnd < 0: dense)
    int32_t mside;        // low byte: 1 upper/left, 2 lower/right border; bit 8 local indices not
                          // increasing; bit 9 dense locals (1..nalc in every equation);
                          // bit 10 no variable parameter twice in one equation
    int32_t file;         // 1-based file index
};

// Work arrays of the device-side record preparation (kept between uploads).
struct UpTmp {
    int64_t *recPtr = nullptr;
    int32_t *recFile = nullptr;
    int64_t *cnt = nullptr, *off = nullptr;   // 6 x (nrec + 1) counts and offsets
    int64_t *scanTmp = nullptr;
    int32_t *grpRec = nullptr;                // record of each group entry
    uint64_t *k0 = nullptr, *k1 = nullptr;    // radix-sort keys
    uint32_t *v0 = nullptr, *v1 = nullptr;    // radix-sort values
    uint64_t *pairKey = nullptr;              // block of each record group pair
    int64_t *hist = nullptr, *head = nullptr;
    int64_t *nel = nullptr, *segStart = nullptr, *segEnd = nullptr;
    int64_t *bcnt = nullptr, *bscan = nullptr, *cntG = nullptr;
    int64_t *scal = nullptr;                  // error word and maxima
    int64_t *ovList = nullptr;                // records handed to the large record kernels
    int64_t *chunkB = nullptr, *keyEnd = nullptr;  // chunk boundaries, fit-bucket ends
    int32_t *bmax = nullptr;                  // maxima per fit bucket
};

// Device arrays of one job.  Every pointer is owned by the context.
struct DevJob {
    // layout
    int32_t nTotal = 0, nVar = 0, nG = 0, matsto = 1;
    int64_t nmat = 0, ncolw = 0;
    int32_t *varOfTot = nullptr;   // [nTotal]
    int32_t *aig = nullptr;        // [nG+1] first variable index of each group
    int32_t *p2g = nullptr;        // [nVar]
    int64_t *off = nullptr;        // [2*(nG+1)] sparseMatrixOffsets
    int32_t *col = nullptr;        // [ncolw] sparseMatrixColumns
    double *matD = nullptr;        // [nmat]
    double *gvec = nullptr;        // [nVar]
    int64_t *gcnt = nullptr;       // [nVar]
    double *gpar = nullptr;        // [nTotal]
    // block rows of the global matrix: blocks (I, J <= I) of row group I,
    // ordered by J, with the offset of element (0,0) in globalMatD and the
    // row stride (the blocks of pairs left out by pairentries point at the
    // discard area after the nmat elements, mpgpu_set_suppressed_pairs)
    int64_t *rowBlk0 = nullptr;    // [nG+1]
    int32_t *blkJ = nullptr;
    int64_t *blkOff = nullptr;
    int32_t *blkLd = nullptr;
    int32_t *rowWidth = nullptr;   // [nG] columns of the dense row layout
    std::vector<int32_t> hRowWidth;
    std::vector<int64_t> hRowBlk0, hBlkOff;
    std::vector<int32_t> hBlkJ, hBlkLd;
    // records
    int64_t nrec = 0, nw = 0, neqTot = 0, nslotTot = 0, nswTot = 0, ngrpTot = 0;
    int32_t nfiles = 1;
    int32_t *inder = nullptr;
    double *glder = nullptr;
    RecInfo *rec = nullptr;
    int32_t *meas = nullptr;       // 3 per equation: startLocal, startGlobal, lastGlobal
    int32_t *slots = nullptr;      // sorted variable indices per record (+1 spare)
    int32_t *slotCnt = nullptr;    // accepted-entry count per slot (structural)
    int32_t *swStart = nullptr;    // per slot: start of its word list (relative)
    int32_t *sw = nullptr;         // (eq << 16) | word position
    int32_t *grpId = nullptr;      // group of each record group entry
    int32_t *grpSlot = nullptr;    // first slot of each record group entry
    double *fileWeight = nullptr;  // [nfiles]
    // per-loop outputs
    int8_t *status = nullptr;
    double *chi2add = nullptr;
    int32_t *ndfadd = nullptr;
    float *chndf = nullptr;
    double *vstage = nullptr;      // per-slot vector contributions
    // chunks of records sharing one update staging buffer
    std::vector<int64_t> chunkRec;     // [nchunk+1] record boundaries
    // fit buckets: records classed by the shared memory their fit needs
    // (power-of-two classes from 4 KB; the last class for records beyond one
    // CTA), ordered by (chunk, class, record) in recList
    uint32_t *recList = nullptr;
    std::vector<int64_t> bucketOff;    // [nchunk * MPG_FIT_BUCKETS + 1] positions in recList
    std::vector<int32_t> bucketMax;    // [MPG_FIT_BUCKETS * 7] nw neq nalc nalg band bdr ngrp
    std::vector<int32_t> bucketWpc;    // [MPG_FIT_BUCKETS] tuned warps per CTA (0: not tuned)
    std::vector<double> bucketTuneMs;  // [MPG_FIT_BUCKETS * 4] sample times of wpc 1, 2, 4, 8
    // matrix accumulation: the group-pair blocks (I, J <= I) met in records,
    // per chunk the records of each block (packed U offset << 16 | row slot)
    // cut into work items; items of a block share partial sums when a block
    // has more than one item
    int64_t nblk = 0;
    int32_t *bkI = nullptr, *bkJ = nullptr, *bkLd = nullptr;
    int64_t *bkOff = nullptr;          // sparse: offset of element (0,0)
    std::vector<int64_t> chunkItem;    // [nchunk+1]
    int32_t *itBlk = nullptr;
    int64_t *itBase = nullptr;         // staging offset of the item's first record block
    int32_t *itCnt = nullptr;          // records in the item
    int64_t *itSlot = nullptr;         // partial slot, -1: write the matrix directly
    int64_t *pairDst = nullptr;        // per record group pair: staging offset of its block
    std::vector<int64_t> chunkRed;     // [nchunk+1] blocks with several items
    int32_t *rdBlk = nullptr;
    int64_t *rdSlot0 = nullptr;
    int32_t *rdN = nullptr;
    double *partial = nullptr;
    int64_t partialLen = 0, pstride = 1;
    // vector accumulation: per chunk and row group the records in order
    // (record << 40 | vstage offset)
    int64_t *vEntries = nullptr;
    int64_t *vStart = nullptr;         // [nchunk*(nG+1)]
    double *stage = nullptr;
    int64_t stageLen = 0;
    UpTmp tmp;
    double *bw = nullptr;              // large-record mode: B and W of a record range
    uint8_t *bigDone = nullptr;        // large-record mode: records whose fit wrote the whole update
    double *bscr = nullptr;            // band records: per-warp inverse scratch
    double msUploadCopy = 0.0, msUploadPrepare = 0.0;   // device time of the last upload
    int32_t uploadChunks = 0;
    std::unordered_map<const void *, int64_t> cap;   // capacities of the arrays kept between uploads
    // limits over the job (fit kernel shared memory sizing)
    int32_t maxNw = 0, maxNeq = 0, maxNalc = 0, maxNalg = 0, maxBand = -1, maxBdr = 0, maxNgrp = 1;
    int32_t nbndr[2] = {0, 0}, nbdrx = 0, nbndx = 0;
    // constraints (QL of the constraint matrix, kept on the device)
    int32_t ncon = 0;
    double *qlV = nullptr;         // [ncon*nVar] Householder vectors (row k)
    double *qlVk = nullptr;        // [ncon]
    int32_t *qlR2 = nullptr;       // [ncon] last non-zero index of each vector
    double *qlT = nullptr;         // [ncon*ncon] compact WY factor: H_1 ... H_m = I - U T U^T
    std::vector<double> hL;        // [ncon*ncon] lower triangle L (host)
    std::vector<double> hV, hVk;
    std::vector<int32_t> hR1, hR2;
    // host copies needed by the host-side control
    std::vector<int32_t> hAig;
    // solver workspace
    double *work = nullptr;
    int64_t workLen = 0;
};

// Records kept on the device by mpgpu_loop1_device: copied once,
// translated to total indices in place, used by mpgpu_loop2_device and
// taken over by the next mpgpu_upload_records called with inder = glder =
// NULL.  Not released by mpgpu_set_layout.
struct ResidentRecords {
    int64_t nrec = -1, nw = 0, w0 = 0;   // w0: recPtr[0] of the loop1 call
    int64_t *recPtr = nullptr;           // [nrec + 1], as passed to loop1
    int32_t *inder = nullptr;            // [nw]
    double *glder = nullptr;             // [nw]
    int32_t nTotal = 0;                  // labels of the loop1 table
    bool translated = false;
};

// monitoring of the data loop (mpgpu_set_monitor)
struct Monitor {
    bool on = false;
    int32_t nbins = 100, measBins = 100, mode = 0, lfitnp = 1 << 30, numMeas = 0;
    float range = 5.0f;
    int32_t *measIndex = nullptr;        // device [nTotal]
    double *measRes = nullptr;           // device [numMeas]
    unsigned long long *hist = nullptr;  // device [4 * (nbins + 2)]
    unsigned long long *meas = nullptr;  // device [numMeas * measBins]
};

struct DenseResident;   // workspace of the refined dense solves (mpgpu_dense.cu)
struct mpgpu_ctx {
    int device = 0;
    int32_t flags = 0;                 // mpgpu_cfg.flags
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;   // accumulation, overlapped with the fits
    int64_t stagingBytes = 0;
    std::string err;
    DevJob j;
    ResidentRecords res;
    Monitor mon;
    double *scal = nullptr;      // small device scalar area
    double *hscal = nullptr;     // pinned mirror
    int64_t lastNaccepted = 0;
    int32_t mbandw = 0;          // MINRES preconditioner: < 0 none, 0 diagonal, > 0 band width
    int32_t lprecm = 0;          // lltdec option of the band preconditioner
    DenseResident *dense = nullptr;  // kept between the dense solves of a job
};

// variable-band preconditioner of MINRES (mpgpu_precond.cu): band of
// Q^T A Q over nVar rows (B), its lltdec factor over the nfit rows (F by
// rows, Fc by columns), the block spikes (G, H: nfit x w) and the
// per-block coupling values (T, Hd)
#define MPGPU_BAND_MAX 32
struct BandPre {
    int32_t n = 0, w = 0, s = 0, p = 0;  // rows, lower width, rows per block, blocks
    double *B = nullptr, *F = nullptr, *Fc = nullptr, *G = nullptr, *H = nullptr, *T = nullptr, *Hd = nullptr;
    int32_t *nrkd = nullptr;
};
int32_t band_alloc(BandPre &P, int32_t nVar, int32_t nfit, int32_t w);
void band_free(BandPre &P);
cudaError_t band_fill(const BandPre &P, int32_t nVar, int32_t matsto, const double *matD, const int32_t *aig,
                      const int32_t *p2g, const int64_t *rowStart, const int32_t *bcol, const int64_t *boff,
                      const int32_t *bld, cudaStream_t s);
cudaError_t band_reflect(const BandPre &P, int32_t nVar, const double *v, const double *y, const double *beta,
                         cudaStream_t s);
cudaError_t band_factor(const BandPre &P, int32_t lprecm, cudaStream_t s);
// y := (L L^T)^-1 y on the nfit rows; nothing when *done is set
cudaError_t band_solve(const BandPre &P, const int *done, double *y, cudaStream_t s);
int32_t band_precond_factor(mpgpu_ctx *c, int32_t mbandw, int32_t lprecm, double *cOut, int32_t *nrkd);

// Raises a kernel's dynamic shared-memory limit to what the device allows
// (its opt-in maximum less the kernel's static shared memory), once per
// kernel and device.  The limit is an attribute of the function, not of a
// launch: set per launch to the launch's size, two host threads (the
// serving workers) launching the same kernel with different sizes could
// each find the other's smaller limit in place.
inline cudaError_t smem_optin(const void *kern) {
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({dev, kern})) return cudaSuccess;
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kern);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) done.insert({dev, kern});
    return e;
}

// Device allocation that keeps its capacity between uploads and loops (no
// free / alloc when the next request fits).
template <class T>
inline cudaError_t dgrow(DevJob &j, T *&p, int64_t n) {
    const void *key = (const void *)&p;
    if (n <= 0) n = 1;
    auto it = j.cap.find(key);
    if (p && it != j.cap.end() && it->second >= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cudaError_t e = cudaMalloc((void **)&p, sizeof(T) * (size_t)n);
    if (e != cudaSuccess) { j.cap.erase(key); return e; }
    j.cap[key] = n;
    return cudaSuccess;
}

// shared memory of one fit warp for records up to the given sizes (the
// carve-up of mpgpu_fit.cu); also used to class records by size
__host__ __device__ inline int64_t align8(int64_t x) { return (x + 7) & ~int64_t(7); }

__host__ __device__ inline int64_t band_doubles(int nalc, int bandmax, int bdrmax) {
    if (bandmax < 0) return 0;
    int64_t n = nalc, b = bandmax, d = bdrmax;
    // vbnd n*(b+1), vbdr n*d, aux n*d+n, vbk d*d, vzru n, scdiag n (+1 each)
    return n * (b + 1) + 2 * n * d + 3 * n + d * d + 16;
}

__host__ __device__ inline int64_t warp_bytes(int wmax, int neqmax, int nalcmax, int nalgmax,
                                              int bandmax, int bdrmax, int ngrpmax, bool big = false) {
    int64_t d = 0;
    d += wmax;                          // gl
    d += 7 * (int64_t)neqmax;           // rm1 lcor lwgt res t1 t2 w0
    d += (int64_t)nalcmax * (nalcmax + 1) / 2 + 4 * (int64_t)nalcmax;  // clmat blvec diag ocol scol
    if (!big) d += 2 * (int64_t)nalcmax * nalgmax;  // B W (global memory for large records)
    d += band_doubles(nalcmax, bandmax, bdrmax);
    int64_t i = 0;
    i += wmax;            // in
    i += 3 * (int64_t)neqmax;
    i += nalgmax;         // slots
    i += nalgmax + 1;     // swS
    i += wmax;            // sw
    i += nalcmax + 2;     // used / scflag
    i += ngrpmax + 2;     // goff
    return align8(d * 8 + i * 4 + 64);
}

// ---------------------------------------------------------------- kernels
struct FitParams {
    const RecInfo *rec;
    const int32_t *inder;
    const double *glder;
    const int32_t *meas;
    const int32_t *slots;
    const int32_t *swStart;
    const int32_t *sw;
    const int32_t *grpSlot;
    const int64_t *pairDst;
    const double *gpar;
    const int32_t *varOfTot;
    const double *fileWeight;
    int64_t r0, r1;           // record range, or positions r0..r1 of recList
    const uint32_t *recList;  // records in fit order (null: r0..r1 are records)
    int32_t wpc;              // warps per CTA (0: as many as the shared memory allows)
    int32_t onePerBlock;      // one record per CTA of one warp, no persistent loop
    int32_t icalcm, nloopn, lhuber, lfitbb;
    float chicut, chhuge, dwcut, cndlmx;
    double *stage;            // update staging of this chunk
    double *vstage;
    int8_t *status;
    double *chi2add;
    int32_t *ndfadd;
    float *chndf;
    int32_t wmax, neqmax, nalcmax, nalgmax, bandmax, bdrmax, ngrpmax;  // shared-memory sizing
    // large records: B and W of each record of the range in global memory
    // (stride bwStride doubles per record); the update kernel adds W B^T
    int32_t bigMode;
    double *bw;
    int64_t bwStride;
    uint8_t *bigDone;         // per position of the launch: update fully written by the fit
    // monitoring (first local-fit iteration): normalized residuals and pulls
    // with/without global derivatives (4 histograms of monBins + 2 bins:
    // underflow, bins, overflow) and the pulls or scaled residuals of the
    // monitored measurement groups (measBins per group)
    int32_t monOn, monPull, monBins, monMeasBins, monMode;
    float monRange;
    const int32_t *measIndex;       // [nTotal] group (1-based) of the first global label, 0: none
    const double *measRes;          // [numMeas] mean error of the group
    unsigned long long *monHist, *measHists;
    // band records: per-warp scratch of the warp-parallel band inverse
    double *bscr;
    int64_t bscrStride;
    int32_t *errFlag;
};

int fit_smem_per_warp(const FitParams &p);
int fit_warps_per_cta(const FitParams &p);
cudaError_t launch_fit(const FitParams &p, int nsm, int maxPerSM, cudaStream_t s);
// W B^T of the accepted records r0..r1 added to their block-major staging
// (large-record mode, one CTA per record, 64 x 64 FP64 tiles)
cudaError_t launch_update_big(const FitParams &p, cudaStream_t s);

struct AccParams {
    const int32_t *bkI, *bkJ, *bkLd;
    const int64_t *bkOff;
    const int32_t *itBlk, *itCnt;
    const int64_t *itBase, *itSlot;
    int64_t item0, nitem;          // items of this chunk
    const int32_t *rdBlk;
    const int64_t *rdSlot0;
    const int32_t *rdN;
    int64_t red0, nred;            // multi-item blocks of this chunk
    double *partial;
    int64_t pstride;               // partial slot stride (elements of the largest block)
    const int64_t *vEntries;
    const int64_t *vStart;         // this chunk, [nG+1]
    const int8_t *status;
    const double *stage;
    const double *vstage;
    const int32_t *slotCnt;
    const int32_t *aig;
    int32_t nG, matsto, icalcm;
    double *matD;
    double *gvec;
    int64_t *gcnt;
    int32_t *errFlag;
};
cudaError_t launch_accumulate(const AccParams &p, int nsm, cudaStream_t s);

struct StatParams {
    const int8_t *status;
    const double *chi2add;
    const int32_t *ndfadd;
    const float *chndf;
    const RecInfo *rec;
    const double *fileWeight;
    int64_t nrec;
    int32_t nfiles;
    double *out;     // device: [0] fraction sum, [1] ndfSumW
    int64_t *iout;   // device: [0] chi2 int, [1] ndf, [2..7] nrej, [8] naccepted,
                     //         then naccf[nfiles], ndff[nfiles]
    float *fout;     // device: chi2f[nfiles]
};
cudaError_t launch_stats(const StatParams &p, cudaStream_t s);

// matrix-element updates (mupdat), applied in order by one thread
cudaError_t launch_mupdat(int32_t n, const int32_t *i, const int32_t *j, const double *add,
                          const DevJob &d, int32_t *errFlag, cudaStream_t s);

// device version of ijpgrp (pede.f90:5371-5461); returns the 1-based index
// of the first element of block (itema, itemb) and its row length
__device__ int64_t d_ijpgrp(int32_t itema, int32_t itemb, int32_t nG, const int32_t *aig,
                            const int64_t *off, const int32_t *col, int32_t *lr);

// ---------------------------------------------------------------- solvers
int32_t solve_inversion(mpgpu_ctx *c, const double *consResiduals, double *corr, double *errs,
                        mpgpu_solveinfo *info, bool decomposition, int dense = -1, double rtol = 1e-13,
                        int32_t itnlim = 2000);
// dense blocked Cholesky (mpgpu_dense.cu): mode 0 FP64, mode 1 tensor-core 3xTF32 trailing updates
int32_t dense_cholesky_device(mpgpu_ctx *c, double *A, int64_t npad, int mode, float *hiBuf, float *loBuf,
                              int32_t *dErr, int32_t *badPanel);
// constraint elimination inside the dense solve (device arrays): the
// Householder vectors of the QL decomposition (V, Vk), the compact WY factor
// T (ncon x ncon) and the constraint part y of the solution
struct DenseWyElim {
    int32_t ncon;
    const double *V, *Vk, *T, *y;
};
// packed SPD solve refined by preconditioned CG in FP64 (b in, x out, device);
// with invOut, also the inverse of Ap from the same factor (packed, n);
// with wy, the constraints are eliminated inside (mpgpu_dense.cu)
int32_t dense_solve_pcg(mpgpu_ctx *c, int32_t n, const double *Ap, double *bx, int mode, double rtol,
                        int32_t itnlim, mpgpu_solveinfo *info, double *invOut = nullptr,
                        const DenseWyElim *wy = nullptr);
// frees the dense-solve workspace (and with it the kept factor)
void dense_release(mpgpu_ctx *c);
// the kept factor no longer belongs to the job's matrix (new constraints)
void dense_invalidate(mpgpu_ctx *c);
// blocked inverse from the dense Cholesky factor (mpgpu_inverse.cu)
int32_t dense_inverse_device(mpgpu_ctx *c, double *L, int64_t npad, int64_t n, int mode, const double *DinvT,
                             double *Zd, double *Zp, int32_t *dErr);
int32_t solve_minres(mpgpu_ctx *c, const double *consResiduals, double rtol, int32_t itnlim,
                     double *corr, mpgpu_solveinfo *info, bool qlp = false);
int32_t avprod_host(mpgpu_ctx *c, int32_t n, const double *x, double *b);

// record preparation on the device (mpgpu_upload.cu)
int32_t upload_records_device(mpgpu_ctx *c, int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                              const double *glder, const int32_t *recFile, int32_t nfiles,
                              const double *fileWeight);

// resolves the device address of mpgpu_mupdat_noalloc's static area on the
// context's device (mpgpu_noalloc.cu; called by mpgpu_create)
int32_t noalloc_prepare(mpgpu_ctx *c);

// error helpers
int32_t set_err(mpgpu_ctx *c, int32_t code, const std::string &msg);
void free_resident(ResidentRecords &R);
int32_t loop1_device(mpgpu_ctx *c, int64_t nrec, const int64_t *recPtr, const int32_t *inder, const double *glder,
                     int32_t nsteer, const int32_t *steerLabels, int32_t npre, const int32_t *preLabel,
                     const double *preSigma, int32_t mreqenf, int32_t cap, int32_t *labels, int64_t *counter,
                     int32_t *varIndex, int32_t *totGroup, int32_t *nVar, int32_t *nVarGroups);
int32_t loop2_device(mpgpu_ctx *c, const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                     const int32_t *allIndexGroups, int64_t cap, int64_t *offsets, int32_t *columns,
                     int64_t *ncolw, int64_t *nmat);
int32_t cuda_err(mpgpu_ctx *c, cudaError_t e, const char *where);
#define MPG_CUDA(c, call)                                      \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_err((c), e_, #call); \
    } while (0)
