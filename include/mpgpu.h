/*
 * mpgpu.h -- C-ABI of the GB300 implementation of Millepede-II pede's hot
 * path: per-record local fits, deterministic accumulation of the
 * Schur-complement updates into the packed or mpbits-sparse global matrix,
 * and the global solve (QL constraint elimination, inversion, Cholesky,
 * MINRES).
 *
 * Every entry point returns an int32 status: 0 on success, otherwise a code
 * that follows pede's exit codes (doc/exitCodes.md, peend in
 * pede.f90:11390-11409) where one exists.  No exception or abort crosses
 * this boundary.  Arrays are plain host pointers owned by the caller; the
 * context owns all device memory and keeps it resident between calls.
 * Index arrays hold the reference's 1-based parameter / group numbers.
 * One host thread per context; several contexts may run concurrently.
 *
 * The seams replaced (file:line in the Millepede-II sources):
 *   mpgpu_loop1_device    loop1 label passes, pargrp, prepareRecords(1)
 *                         translation (mppar.f90:117-321, pede.f90:2311-2404,
 *                         5958-5971)
 *   mpgpu_loop2_device    loop2 mpbits structure (pede.f90:6889-6908,
 *                         mpbits.f90:305-566, 1220-1350)
 *   mpgpu_set_layout      loop2 results: globalAllIndexGroups,
 *                         sparseMatrixOffsets/Columns (pede.f90:6509-6545,
 *                         7174, 7426)
 *   mpgpu_set_suppressed_pairs  pairs left out by pairentries, whose
 *                         updates mupdat drops (pede.f90:3172, mpbits.f90:409)
 *   mpgpu_set_constraints feasma / qldecb (pede.f90:1377-1544,
 *                         mpqldec.f90:219-393)
 *   mpgpu_upload_records  readFromBinary + prepareRecords(1) buffers
 *                         (pede.f90:1714-2075, mppar.f90:282-321)
 *   mpgpu_loopbf          CALL loopbf(nrejec,nfiles,jfd,cfd,dfd)
 *                         (pede.f90:2613; routine at 3387-4442) with the
 *                         mgupdt flush (pede.f90:3219-3357)
 *   mpgpu_mupdat          CALL mupdat(i,j,add) (pede.f90:3134-3204)
 *   mpgpu_solve           CALL minver / mchdec / mminrs / mminrsqlp
 *                         (pede.f90:8832-8855)
 *   mpgpu_set_preconditioner  steering "bandwidth mbandw lprecm"
 *                         (pede.f90:10495-10503), used by mminrs 8292-8316
 *   mpgpu_band_factor     CALL equdecs on matPreCond (pede.f90:8309,
 *                         mpnum.f90:2486-2592)
 *   mpgpu_avprod          SUBROUTINE avprod(n,x,b) (pede.f90:5331-5358)
 *   mpgpu_download_matrix globalMatD after the data loop
 *   mpgpu_set_monitor /   measIndex/measRes and measHists of
 *   mpgpu_get_monitor     monitorresiduals/monitorpulls (pede.f90:6571-6579,
 *                         3967-3990); mpgpu_write_mon: monres (7533-7633)
 *   mpgpu_read_mille      readC / readF of the binary files (pede.f90:1714-2075)
 *   mpgpu_write_res       prtglo (pede.f90:4477-4651)
 */
#ifndef MPGPU_H
#define MPGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MPGPU_OK 0
#define MPGPU_ERR_BADRECORD 20     /* malformed record (pede code 20) */
#define MPGPU_ERR_BADINDEX 23      /* index outside the matrix (pede 23) */
#define MPGPU_ERR_SIZE 24          /* size mismatch (pede 24) */
#define MPGPU_ERR_NAN 25           /* NaN in the solution (pede 25) */
#define MPGPU_ERR_TOOMANYREJ 26    /* more than 1/3 of records rejected (pede 26) */
#define MPGPU_ERR_QL 27            /* singular constraints (pede 27) */
#define MPGPU_ERR_FACTOR 29        /* factorisation failed */
#define MPGPU_ERR_ALLOC 30         /* device allocation failed */
#define MPGPU_ERR_GROUPS 35        /* record/group mismatch (pede 35) */
#define MPGPU_ERR_TIMEOUT 41       /* a bounded device wait ran out */
#define MPGPU_ERR_BUDGET 42        /* job rejected by the HBM budget */
#define MPGPU_ERR_CUDA 43          /* CUDA runtime error */
#define MPGPU_ERR_ARG 44           /* invalid argument / call order */
#define MPGPU_ERR_LIMIT 45         /* record larger than the kernel limits */

typedef struct mpgpu_ctx mpgpu_ctx;

/* cfg flags: run every record through the large-record path (B and W of a
 * record in global memory, W B^T by a tiled kernel), which is otherwise
 * chosen only when the records are too large for the per-warp form */
#define MPGPU_FLAG_LARGE_RECORDS 1
/* one fit launch per chunk with the shared memory sized for the job's
 * largest record (no size classes); for comparison */
#define MPGPU_FLAG_NO_BUCKETS 2
/* one record per CTA of one warp (no persistent loop), no size classes: the
 * plain launch form, for comparison */
#define MPGPU_FLAG_ONE_RECORD_PER_BLOCK 4
/* no timing of warps-per-CTA candidates on the first data loop */
#define MPGPU_FLAG_NO_AUTOTUNE 8
/* the tensor-core dense solve (metsol 31) factorises at every solve instead
 * of first preconditioning with the factor of the job's previous solve */
#define MPGPU_FLAG_FRESH_FACTOR 16

typedef struct mpgpu_cfg {
    int32_t device;             /* CUDA device ordinal */
    int32_t flags;              /* MPGPU_FLAG_* */
    int64_t staging_bytes;      /* update staging per chunk (0: sized per job, one chunk when it fits) */
} mpgpu_cfg;

int32_t mpgpu_create(mpgpu_ctx **ctx, const mpgpu_cfg *cfg);
int32_t mpgpu_destroy(mpgpu_ctx *ctx);
/* last error message of the context (static storage inside ctx) */
const char *mpgpu_last_error(const mpgpu_ctx *ctx);

/* Frees the device memory of the context's current job (records, layout,
 * global matrix, constraints, dense-solve workspace with its kept factor);
 * the context stays usable for the next job.  No reference counterpart:
 * pede runs one job per process. */
int32_t mpgpu_release(mpgpu_ctx *ctx);

/* Global-parameter layout.  varIndexOfTotal[nTotal]: variable index (1..nVar)
 * of each total parameter index, <=0 for fixed (globalParLabelIndex(2,:)).
 * allIndexGroups[nGroups+1]: first variable index of each parameter group,
 * last entry nVar+1.  matsto 1: packed lower triangle; matsto 2: mpbits
 * sparse storage described by sparseOffsets[2*(nGroups+1)] (column-major
 * 2 x (nGroups+1), sparseMatrixOffsets) and sparseColumns[ncolw]
 * (sparseMatrixColumns); nmat = length of globalMatD. */
int32_t mpgpu_set_layout(mpgpu_ctx *ctx, int32_t nTotal, const int32_t *varIndexOfTotal,
                         int32_t nVar, int32_t nGroups, const int32_t *allIndexGroups,
                         int32_t matsto, const int64_t *sparseOffsets,
                         const int32_t *sparseColumns, int64_t ncolw, int64_t nmat);

/* pairentries: the group pairs met in the records that the sparse layout
 * leaves out (the list of mpgpu_host_mpbits_pairentries, 1-based group
 * numbers, either order).  The records' updates of these pairs are dropped,
 * as mupdat drops an element that is not stored (pede.f90:3172); without
 * this call such a pair is an upload error (23).  Call after
 * mpgpu_set_layout (sparse) and before mpgpu_upload_records; records
 * uploaded earlier are released; a later call replaces the list.  A pair
 * that the layout stores is refused (24). */
int32_t mpgpu_set_suppressed_pairs(mpgpu_ctx *ctx, int64_t npair, const int32_t *pairs);

/* Linear constraints over the variable parameters, eliminated by QL:
 * A[ncon*nVar], row k = constraint k (the reference's matConstraintsT). */
int32_t mpgpu_set_constraints(mpgpu_ctx *ctx, int32_t ncon, const double *A);

/* Records in the Mille layout (pede.f90:1693-1713) with labels already
 * translated to total parameter indices (prepareRecords(1)).  Record r
 * occupies words [recPtr[r], recPtr[r+1]); recFile[nrec] holds the 1-based
 * file of each record (NULL: all file 1), fileWeight[nfiles] the file
 * weights (NULL: 1).  Replaces any previously uploaded records.  With
 * inder = glder = NULL the records kept (translated) by mpgpu_loop1_device
 * are taken over without a copy; recPtr must be the one given there and the
 * layout must use loop1's label table. */
int32_t mpgpu_upload_records(mpgpu_ctx *ctx, int64_t nrec, const int64_t *recPtr,
                             const int32_t *inder, const double *glder,
                             const int32_t *recFile, int32_t nfiles,
                             const double *fileWeight);

/* Monitoring of the data loop (pede's histograms 3, 12, 13, 14 and its
 * measurement monitor, pede.f90:3938-3980, 4025-4032, 7533-7633), filled
 * by the device fit in the first local-fit iteration of every record:
 * normalized residuals r/sigma and pulls r/sqrt(sigma^2 - l^T C l) (where
 * variance is left), each for measurements with and without global
 * derivatives, and per monitored group (the first global label of the
 * measurement, mpgpu_monitor_groups) the pulls (mode 1, monitorpulls) or
 * the residuals scaled by the group's mean error (mode 0,
 * monitorresiduals) in measBins bins of 0.1.  Pulls are formed in loops
 * nloopn <= lfitnp (0: all).  The histograms are reset by every
 * mpgpu_loopbf.  No counterpart as a C-ABI in the reference. */
typedef struct mpgpu_monitor_cfg {
    int32_t nbins;      /* bins of the four histograms, over [-range, range) */
    float range;
    int32_t measBins;   /* bins per monitored group (pede's measBins, 100) */
    int32_t mode;       /* 0 scaled residuals, 1 pulls */
    int32_t lfitnp;
} mpgpu_monitor_cfg;
/* cfg NULL switches monitoring off.  measIndex[nTotal]: group 1..numMeas
 * of each total parameter index as first global label (0: none); measRes
 * [numMeas] the groups' mean errors (both from mpgpu_monitor_groups). */
int32_t mpgpu_set_monitor(mpgpu_ctx *ctx, const mpgpu_monitor_cfg *cfg, const int32_t *measIndex,
                          const double *measRes, int32_t numMeas);
/* hist[4 * (nbins + 2)]: residuals with globals, residuals without,
 * pulls with globals, pulls without; each underflow, bins, overflow.
 * measHists[numMeas * measBins] (may be NULL). */
int32_t mpgpu_get_monitor(mpgpu_ctx *ctx, int64_t *hist, int64_t *measHists);
/* loop2's grouping of the monitor (pede.f90:6700-6710, 7075-7081): the
 * measurements with local and global derivatives of the (translated)
 * records by their first global label, counted and their errors averaged
 * in record order; measIndex[nTotal] numbers the groups in index order.
 * Returns 0 or a status. */
int32_t mpgpu_monitor_groups(int64_t nrec, const int64_t *recPtr, const int32_t *inder, const double *glder,
                             int32_t nTotal, int32_t *measIndex, double *measRes, int32_t *numMeas);
/* monres (pede.f90:7533-7633): one line per group with the loop number,
 * its label, entries, median and 1.4826 x median absolute deviation of the
 * binned values, and the group's mean error, appended to path (header
 * lines when header != 0). */
int32_t mpgpu_write_mon(const char *path, int32_t header, int32_t mode, int32_t nloopn, int32_t numMeas,
                        const int32_t *groupLabel, const int64_t *measHists, int32_t measBins,
                        const double *measRes);

/* Fit size classes of the uploaded records (the shared memory each fit
 * needs: class k < 7 up to 4 KB << k, class 7 beyond one CTA): records per
 * class, warps per CTA chosen by the tuner on the first data loop (0: not
 * yet tuned, -1: no candidate fitted) and the sample times (ms) of 1, 2, 4
 * and 8 warps per CTA; arrays of MPGPU_FIT_BUCKETS (and 4x that for
 * tuneMs).  No counterpart in the reference. */
#define MPGPU_FIT_BUCKETS 8
int32_t mpgpu_fit_buckets(const mpgpu_ctx *ctx, int64_t *count, int32_t *wpc, double *tuneMs);

/* Device time of the last mpgpu_upload_records: the host-to-device copy of
 * the records and the record preparation on the device, and the number of
 * chunks the loop will run in (no counterpart in the reference). */
int32_t mpgpu_upload_timing(const mpgpu_ctx *ctx, double *msCopy, double *msPrepare, int32_t *nchunk);

typedef struct mpgpu_fitopts {
    int32_t icalcm;    /* 1: build the global matrix */
    int32_t nloopn;    /* data-loop counter (1 = first) */
    int32_t lhuber;    /* outlier down-weighting iterations */
    int32_t lfitbb;    /* bordered-band detection for the local fit */
    float chicut;      /* chi2 cut factor (<0: none) */
    float chhuge;      /* cut for unreasonable chi2 */
    float dwcut;       /* down-weight fraction cut */
    float cndlmx;      /* max log10(condition) of the band part */
} mpgpu_fitopts;

typedef struct mpgpu_fitstats {
    int64_t nrej[6];    /* NaN, rank, condition, ndf<=0, huge chi2, chi2 cut */
    int64_t chi2SumI;   /* integer part of sum(chi2*w) (addsums) */
    double chi2SumD;    /* remainder */
    int64_t ndfSum;
    double ndfSumW;
    int32_t nbndr[2];   /* records solved as bordered band (left / right) */
    int32_t nbdrx, nbndx;
    int64_t naccepted;
    double msFit;       /* device time of the local-fit kernels (CUDA events) */
    double msAccum;     /* device time of the accumulation kernels */
    double msLoop;      /* device time of the whole data loop */
    int32_t launches;   /* kernels launched by the loop */
    int32_t pad;
} mpgpu_fitstats;

/* One data loop (loopbf): local fits of all records with the given global
 * parameters (globalParameter[nTotal], host), then - if icalcm == 1 - the
 * deterministic accumulation of the updates into the device-resident global
 * matrix (zeroed first).  globalVector[nVar] / globalCounter[nVar] (host,
 * may be NULL) receive the gradient and the entry counts; naccf/chi2f/ndff
 * [nfiles] (may be NULL) the per-file statistics.  The vector stays on the
 * device for mpgpu_solve. */
int32_t mpgpu_loopbf(mpgpu_ctx *ctx, const mpgpu_fitopts *opt, const double *globalParameter,
                     double *globalVector, int64_t *globalCounter, mpgpu_fitstats *stats,
                     int32_t *naccf, float *chi2f, int32_t *ndff);

/* Same loop with the global parameters, vector and counters left on the
 * device (device pointers; globalParameter is read, the others written). */
int32_t mpgpu_loopbf_device(mpgpu_ctx *ctx, const mpgpu_fitopts *opt,
                            const double *d_globalParameter, mpgpu_fitstats *stats);

/* mupdat for n elements: matrix(i[k], j[k]) += add[k] (1-based variable
 * indices), applied in order on the device; the vector side (globalVector
 * += vadd) is applied when vidx != NULL. */
int32_t mpgpu_mupdat(mpgpu_ctx *ctx, int32_t n, const int32_t *i, const int32_t *j,
                     const double *add);

/* mpgpu_mupdat without any device allocation.  This entry point has no
 * counterpart in the reference (pede's mupdat adds to host memory).  It is
 * for callers that must not allocate or free device memory during the call:
 * a host loop that adds terms while other streams keep the device busy
 * (cudaFree would wait for all of them), or a job whose matrix and staging
 * fill the device memory.  The triplets are staged in a fixed device area of
 * MPGPU_MUPDAT_NOALLOC_MAX elements, one per device; CUDA reserves it when it
 * loads the library's module holding it, which mpgpu_create forces on its
 * device (the area is in place before the job's large allocations, and
 * mpgpu_mupdat_noalloc itself never loads a module or reserves memory).
 * Larger n returns MPGPU_ERR_LIMIT and changes nothing.  The area is shared
 * by all contexts on a device: calls that overlap in time on the same device
 * race on it, so serialise them.  Same result and error codes as
 * mpgpu_mupdat. */
#define MPGPU_MUPDAT_NOALLOC_MAX 65536
int32_t mpgpu_mupdat_noalloc(mpgpu_ctx *ctx, int32_t n, const int32_t *i, const int32_t *j,
                             const double *add);
int32_t mpgpu_vector_add(mpgpu_ctx *ctx, int32_t n, const int32_t *vidx, const double *vadd);

int32_t mpgpu_download_matrix(mpgpu_ctx *ctx, double *globalMatD);
/* diagonal[nVar] of the current global matrix (matij(i,i), the diagonal
 * minver saves before the inversion, pede.f90:7864-7866) */
int32_t mpgpu_matrix_diagonal(mpgpu_ctx *ctx, double *diagonal);
int32_t mpgpu_download_vector(mpgpu_ctx *ctx, double *globalVector, int64_t *globalCounter);
/* per-record outcome of the last loop: 0 accepted, 1..6 rejection class
 * (nrej index + 1), -1 no local parameters */
int32_t mpgpu_download_record_status(mpgpu_ctx *ctx, int32_t *status);

typedef struct mpgpu_solveinfo {
    int32_t nrank;      /* rank found by inversion / decomposition */
    int32_t itn;        /* MINRES iterations */
    int32_t istop;      /* MINRES stop reason */
    int32_t nrkd;       /* band preconditioner: lltdec's rank-deficit code */
    double evmin, evmax;  /* decomposition pivot range */
    double ms;          /* device time of the solve */
    double msFactor;    /* dense solves: device time of the factorisation; MINRES: of the
                           preconditioner set-up */
    double msRefine;    /* dense solves: device time of the CG refinement */
    double dxRel;       /* dense solves: size of the last CG correction relative to the
                           solution (|alpha p| / |x|) */
    double msInverse;   /* blocked inversions (metsol 11, 12): device time of the inverse
                           from the factor */
    int32_t factorReused;  /* metsol 31: 1 the previous solve's factor preconditioned this
                              one, 2 it was tried and dropped, 0 not tried */
    int32_t itnReuse;      /* CG iterations spent on a dropped factor (included in itn) */
} mpgpu_solveinfo;

/* Global solve (metsol 1 inversion, 3 decomposition = Cholesky, 4 MINRES,
 * 5 MINRES-QLP) of the matrix built by the last mpgpu_loopbf plus mupdat
 * calls.  MINRES-QLP (mminrsqlp, pede.f90 method 5) takes QLP steps from
 * the first iteration (pede's mrmode 2) with maxxnorm = nfit / sqrt(eps);
 * info->istop 1 residual test, 2 least-squares test, 4 condition limit,
 * 5 iterate longer than maxxnorm (the previous one is returned), 6
 * iteration limit.
 * Inversion also in blocked dense form (no counterpart in the reference):
 * metsol 12 the inverse from the FP64 blocked Cholesky factor, metsol 11
 * from the factor with tensor-core 3xTF32 trailing updates, its inverse
 * (trtri, lauum) with 3xTF32 tile products too; the solution is refined as
 * for metsol 31/32, the errors are the diagonal of the inverse (FP64 form:
 * FP64 accuracy; tensor-core form: about the 3xTF32 product precision times
 * the condition number, not refined).
 * Decomposition also in blocked dense form (no counterpart in the
 * reference, same solution): metsol 32 FP64 blocked Cholesky, metsol 31
 * Cholesky with tensor-core 3xTF32 trailing updates; both refine the
 * solution by preconditioned CG in FP64 until the relative residual is
 * below rtol and the last correction is below 1e-13 of the solution, so
 * that factors of either precision reach the same FP64 solution
 * (info->itn iterations, info->istop 1 converged / 3 limit, info->evmin the
 * diagonal shift the low-precision factor needed, info->evmax the final
 * relative residual, info->dxRel the last relative correction).  metsol 31
 * keeps its factor in the context: the next solve of a matrix of the same
 * sizes (the job's next outlier iteration) is first preconditioned with it
 * and factorises only when CG has not converged within 40 iterations
 * (info->factorReused; MPGPU_FLAG_FRESH_FACTOR turns this off).
 * consResiduals[ncon] = d - C p (addcst); correction[nVar] receives the
 * step; errors[nVar] (metsol 1, may be NULL) the diagonal of the covariance
 * (sqrt gives the parameter errors).  rtol/itnlim: MINRES(-QLP) tolerance and
 * iteration limit.  The matrix is consumed (factorised in place). */
int32_t mpgpu_solve(mpgpu_ctx *ctx, int32_t metsol, const double *consResiduals,
                    double rtol, int32_t itnlim, double *correction, double *errors,
                    mpgpu_solveinfo *info);

/* Preconditioner of MINRES / MINRES-QLP (pede's "bandwidth mbandw lprecm",
 * pede.f90:10495-10503, used in mminrs/mminrsqlp 8292-8316): mbandw < 0
 * none, 0 the diagonal (default, precons), 1..MPGPU_BAND_WIDTH_MAX the
 * variable-band Cholesky factor of the band of Q^T A Q (equdecs/equslvs with
 * the constraints eliminated, mpnum.f90:2486-2678); lprecm > 0 is lltdec's
 * skyline option (a dependent row keeps the root of its own diagonal).
 * Kept by the context for the following solves; wider bands return
 * MPGPU_ERR_LIMIT from the solve. */
#define MPGPU_BAND_WIDTH_MAX 32
int32_t mpgpu_set_preconditioner(mpgpu_ctx *ctx, int32_t mbandw, int32_t lprecm);

/* The band preconditioner alone (equdecs on matPreCond): the band of
 * width mbandw > 0 of Q^T A Q of the current matrix factorised by lltdec,
 * written to c in pede's variable-band layout (indPreCond, pede.f90:
 * 7705-7717: rows 1..mbandw triangular, then mbandw per row, the diagonal
 * last in each row and replaced by 1/sqrt) for the nVar - ncon fit
 * parameters; *nrkd receives lltdec's rank-deficit code. */
int32_t mpgpu_band_factor(mpgpu_ctx *ctx, int32_t mbandw, int32_t lprecm, double *c, int32_t *nrkd);

/* Page-lock (register) / release a caller-owned host buffer so that the
 * uploads from it run at full host-device bandwidth. */
int32_t mpgpu_host_register(void *ptr, int64_t bytes);
int32_t mpgpu_host_unregister(void *ptr);
/* Page-locked host memory allocated by the runtime, for record buffers
 * that are uploaded repeatedly (released with mpgpu_host_free). */
int32_t mpgpu_host_alloc(void **ptr, int64_t bytes);
int32_t mpgpu_host_free(void *ptr);

/* Measured FP64 fused-multiply-add throughput of the device (TFLOP/s),
 * used as the roofline denominator of the FP64-bound local-fit kernel. */
int32_t mpgpu_probe_fp64(int32_t device, double *tflops);

/* Dense Cholesky factor L (L L^T = A) of a symmetric positive definite
 * n x n matrix (row-major, lower triangle read; L written row-major, lower
 * triangle), blocked in 128 x 128 tiles (the dense form of chdec2,
 * mpnum.f90:891-987).  mode 0: FP64 throughout; mode 1: trailing updates on
 * the tensor cores in 3xTF32 (about 1e-6 relative accuracy of the factor,
 * used as the preconditioner of the refined solve).  *ms receives the device
 * time.  Returns MPGPU_ERR_FACTOR on a non-positive pivot. */
int32_t mpgpu_dense_cholesky(mpgpu_ctx *ctx, int32_t n, const double *A, double *L, int32_t mode,
                             double *ms);

/* b = Q^T A Q x restricted to the first n = nVar - ncon components
 * (avprod), x and b host arrays of length n. */
int32_t mpgpu_avprod(mpgpu_ctx *ctx, int32_t n, const double *x, double *b);

/* ------------------------------------------------------------------
 * Host side of pede (stand-in for the Fortran host): label table, groups,
 * sparse structure, iteration control and millepede.res.
 * ---------------------------------------------------------------- */
typedef struct mpgpu_steer {
    int32_t metsol;     /* 1 inversion, 3 decomposition, 4 MINRES, 5 MINRES-QLP, 31/32 dense */
    int32_t matsto;     /* 1 packed, 2 sparse */
    int32_t mitera;     /* number of iterations (solutions) */
    int32_t lhuber;     /* outlierdownweighting */
    float chicut, chirem, chhuge, dwcut, cndlmx;
    int32_t lfitbb;
    int32_t mreqenf, mreqena, mreqpe;   /* mreqpe: pede's pairentries (sparse storage):
                                           group pairs met in fewer records are left out
                                           of the matrix and their updates dropped; 1
                                           stores every pair met.  The structure passes
                                           then run on the host. */
    double mrestl;
    int32_t itnlim;
    int32_t nthreads;   /* host threads for the structure passes */
    int32_t structDevice; /* 1: structure passes on the device (mpgpu_loop1_device,
                             mpgpu_loop2_device) when mpgpu_pede_run is called
                             directly; 0: on the host */
    int32_t monitor;      /* imonit of monitorresiduals / monitorpulls: bit 0 writes the
                             millepede.mon lines (job->monPath) after the first data loop,
                             bit 1 after the last, < 0 after every loop; 0 off */
    int32_t monitorPulls; /* imonmd: 1 pulls (monitorpulls), 0 normalised residuals */
    int32_t monitorBins;  /* measBins, bins of 0.1 per group histogram (>= 2, pede's 100) */
    int32_t mbandw;       /* MINRES preconditioner (mpgpu_set_preconditioner): < 0 none,
                             0 diagonal, > 0 band width */
    int32_t lprecm;       /* lltdec skyline option of the band preconditioner */
} mpgpu_steer;

typedef struct mpgpu_job {
    int64_t nrec; const int64_t *recPtr; const int32_t *inder; const double *glder;
    const int32_t *recFile; int32_t nfiles; const double *fileWeight;
    int32_t npar; const int32_t *parLabel; const double *parValue; const double *parSigma;
    int32_t ncon; const int32_t *conStart; const int32_t *conLabel; const double *conCoef;
    const double *conRhs;
    int32_t nmeas; const int32_t *msStart; const int32_t *msLabel; const double *msCoef;
    const double *msRhs; const double *msSigma;
    const char *monPath;  /* millepede.mon of the monitor (steer monitor != 0), NULL: none */
} mpgpu_job;

typedef struct mpgpu_result {
    int32_t cap;
    int32_t nTotal, nVar, nVarGroups, nFit;
    int32_t *labels; double *parameter; double *presigma; double *error; int64_t *counts;
    int32_t *varIndex;
    int64_t nrej[6];
    double fvalue; int64_t ndf;
    int32_t nrank; int32_t minresItn, minresIstop;
    int32_t nloopn;
    int32_t exitCode;
    double msBuild, msSolve;   /* device time of the last build / solve */
    /* optional per-label outputs of mpgpu_pede_run (NULL: not written):
     * start values (globalParStart: the steering's values, set in loop1,
     * pede.f90:5916-5930, before feasib), the global correlation of each variable
     * parameter after an inversion (sqrt(1 - 1/(C_ii A_ii)) with the saved
     * diagonal A_ii of the matrix, prtglo pede.f90:4537-4544; -1 where it
     * is not defined) and the entries of each label in the records
     * (globalParLabelCounter, counted in loop1, pede.f90:2334) */
    double *start;
    double *gcor;
    int64_t *fileCounts;
    /* where the job's time went (mpgpu_pede_run): host wall of the
     * structure passes (labels, translation, sparse structure), host wall of
     * the record upload, device time of all data loops and of all solves,
     * wall of the host work between them (constraint residuals, feasib,
     * measurement lines), wall of the whole job */
    double msStructure, msUpload, msLoops, msSolves, msHostIter, msJob;
} mpgpu_result;

/* loop1 equivalent: label table (sorted), entries per label, parameter
 * groups and variable indices.  Returns nTotal or <0: -1 more labels than
 * cap, -20 malformed record, -23 a global word with a label <= 0. */
int32_t mpgpu_host_labels(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                          const double *glder, int32_t nsteer, const int32_t *steerLabels,
                          int32_t npre, const int32_t *preLabel, const double *preSigma,
                          int32_t mreqenf, int32_t cap, int32_t *labels, int64_t *counter,
                          int32_t *varIndex, int32_t *totGroup, int32_t *nVar,
                          int32_t *nVarGroups);
/* translation labels -> total indices (prepareRecords(1)) */
int32_t mpgpu_host_translate(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                             const double *glder, int32_t nTotal, const int32_t *labels,
                             int32_t *outInder);
/* loop2 sparse structure (matsto 2, mreqpe 1): sparseMatrixOffsets /
 * Columns; returns 0 or <0 (capacity) */
int32_t mpgpu_host_mpbits(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                          const double *glder, const int32_t *varIndexOfTotal, int32_t nVar,
                          int32_t nG, const int32_t *allIndexGroups, int64_t cap,
                          int64_t *offsets, int32_t *columns, int64_t *ncolw, int64_t *nmat);
/* loop2 sparse structure with pairentries mreqpe (clbits/inbits/ndbits,
 * mpbits.f90:73-142, 182-243, 305-566; record pairs pede.f90:6889-6908):
 * every group pair is counted once per record, records nrecData..nrec-1
 * (the structure-only records of the measurement lines) count mreqpe
 * (pede.f90:7036); pairs counted at least mreqpe times are stored, the
 * others met are listed in suppressed[2*k], [2*k+1] (row group >= column
 * group, by row, then column) for mpgpu_set_suppressed_pairs.  Returns 0,
 * 44 on bad arguments, or -1 when columns needs more than cap words or the
 * list more than capSup pairs (*ncolw, *nmat and *nsup then hold the sizes;
 * call again with larger arrays).  mreqpe <= 1 is mpgpu_host_mpbits. */
int32_t mpgpu_host_mpbits_pairentries(int64_t nrec, int64_t nrecData, const int64_t *recPtr,
                                      const int32_t *inder, const double *glder,
                                      const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                                      const int32_t *allIndexGroups, int32_t mreqpe, int64_t cap,
                                      int64_t *offsets, int32_t *columns, int64_t *ncolw,
                                      int64_t *nmat, int64_t capSup, int32_t *suppressed,
                                      int64_t *nsup);

/* loop1 on the device: the tables of mpgpu_host_labels (same arguments,
 * outputs and results) for the label passes of pede's loop1 (label table
 * mppar.f90:117-252, entries cut pede.f90:5958-5971, pargrp
 * pede.f90:2311-2404, variable groups pede.f90:6509-6545).  The records are
 * copied to the device once and kept there, translated to total indices in
 * place (prepareRecords(1), mppar.f90:282-321; the words of
 * mpgpu_host_translate), for mpgpu_loop2_device and for the next
 * mpgpu_upload_records called with inder = glder = NULL.  Records follow the
 * device limits (at most 65535 words and 512 measurements).  Returns nTotal
 * or <0: -1 more labels than cap, -20 malformed record, -23 a global word
 * with a label <= 0, -30 device memory, -43 CUDA, -44 arguments, -45 a
 * record beyond the device limits. */
int32_t mpgpu_loop1_device(mpgpu_ctx *ctx, int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                           const double *glder, int32_t nsteer, const int32_t *steerLabels,
                           int32_t npre, const int32_t *preLabel, const double *preSigma,
                           int32_t mreqenf, int32_t cap, int32_t *labels, int64_t *counter,
                           int32_t *varIndex, int32_t *totGroup, int32_t *nVar, int32_t *nVarGroups);
/* loop2 on the device: sparseMatrixOffsets/Columns of mpgpu_host_mpbits
 * (pede.f90:6889-6908, mpbits.f90:305-566, 1220-1350) from the records kept
 * by mpgpu_loop1_device.  Returns 0, -1 when the columns need more than cap
 * words (offsets, *ncolw and *nmat are set; call again with a larger
 * array), or a status. */
int32_t mpgpu_loop2_device(mpgpu_ctx *ctx, const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                           const int32_t *allIndexGroups, int64_t cap, int64_t *offsets,
                           int32_t *columns, int64_t *ncolw, int64_t *nmat);

/* Mille binary files (C or Fortran record framing, float or double words,
 * plain or gzip-compressed; recognised per file, compressed files through
 * the zlib runtime library libz.so.1) into record arrays, the file part of
 * readFromBinary (pede.f90:1714-2075).  First call with inder == NULL: *nrec and *nw
 * receive the sizes.  Second call: recPtr[nrec+1], inder[nw], glder[nw]
 * (float words widened to double) and recFile[nrec] (1-based file index,
 * may be NULL) are filled; cap is the length of inder/glder.  maxRec > 0
 * limits the records read per file.  Status 20 on a damaged record. */
#define MPGPU_FILE_WORDS_MAX 16777216
int32_t mpgpu_read_mille(int32_t nfiles, const char *const *files, int64_t maxRec, int64_t cap,
                         int64_t *nrec, int64_t *nw, int64_t *recPtr, int32_t *inder, double *glder,
                         int32_t *recFile);

/* Whole alignment job on the GPU (iteration control of xloopn without line
 * search); ctx may be NULL (a private context is created). */
int32_t mpgpu_pede_run(mpgpu_ctx *ctx, const mpgpu_steer *st, const mpgpu_job *job,
                       mpgpu_result *res);
/* millepede.res (prtglo, pede.f90:4477-4651): label, value and pre-sigma
 * of every parameter, and for variable ones the difference to the start
 * value (res->start; the value itself when start is NULL), the error
 * (errors != 0) in pede's G14.5 layout (format 102). */
int32_t mpgpu_write_res(const char *path, const mpgpu_result *res, int32_t errors);
/* The same with pede's printing options: ipcntr (steering "printcounts n",
 * pede.f90:10592-10596) 0 no counts, 1 the entries of the last local fits
 * (res->counts), > 1 the entries in the records (res->fileCounts); counts
 * of variable parameters below mreqena are written as -(count+1), pede's
 * lowstat flag (formats 110-112, pede.f90:4546-4590).  igcorr (steering
 * "globalcorr") adds the global correlation column res->gcor (F8.3,
 * format 102) when errors are written and ipcntr is 0.  ipcntr < 0 (the
 * counts of zero derivatives) is not kept by this library: status 44. */
typedef struct mpgpu_res_opts {
    int32_t errors;
    int32_t ipcntr;
    int32_t igcorr;
    int32_t mreqena;
} mpgpu_res_opts;
int32_t mpgpu_write_res_opts(const char *path, const mpgpu_result *res, const mpgpu_res_opts *opts);

/* ------------------------------------------------------------------
 * Serving: a resident loop that runs alignment jobs as they arrive (no
 * counterpart in the reference, which runs one job per process).  maxActive
 * worker contexts run jobs concurrently on the device; a job is admitted
 * when its device footprint fits in budgetBytes next to the running jobs,
 * in submission order.  A job's result does not depend on the other jobs.
 * ---------------------------------------------------------------- */
typedef struct mpgpu_server mpgpu_server;
typedef struct mpgpu_server_cfg {
    int32_t device;
    int32_t maxActive;      /* jobs on the device at once (0: 4) */
    int64_t budgetBytes;    /* device memory budget for admitted jobs (0: 150 GB) */
} mpgpu_server_cfg;
int32_t mpgpu_server_create(mpgpu_server **srv, const mpgpu_server_cfg *cfg);
/* Queue a job (as mpgpu_pede_run); st, job, res and all arrays they point
 * to must stay valid until mpgpu_server_wait has returned for the ticket. */
int32_t mpgpu_server_submit(mpgpu_server *srv, const mpgpu_steer *st, const mpgpu_job *job,
                            mpgpu_result *res, int64_t *ticket);
/* Wait for a job (timeoutMs <= 0: no limit; MPGPU_ERR_TIMEOUT when it ran
 * out); returns the job's status and its latency (submission to end), its
 * wait for a worker and its admitted device footprint. */
int32_t mpgpu_server_wait(mpgpu_server *srv, int64_t ticket, double timeoutMs, double *msLatency,
                          double *msQueue, int64_t *bytes);
/* Message of the last job that ended with an error ("ticket N: ...";
 * empty when none has); valid until the next call on the server. */
const char *mpgpu_server_last_error(mpgpu_server *srv);
/* Runs the queued jobs to the end, then releases the workers. */
int32_t mpgpu_server_destroy(mpgpu_server *srv);

/* ------------------------------------------------------------------
 * Synthetic Mille data (role of pede -t / mptest1 / mptest2)
 * ---------------------------------------------------------------- */
typedef struct mpgen_cfg {
    int32_t kind;        /* 1 telescope, 2 barrel helices, 3 barrel broken lines */
    int32_t nlayers;     /* telescope layers */
    int32_t nmod;        /* telescope: modules per layer; barrel: total modules */
    int32_t minHits, maxHits;  /* broken lines */
    int64_t ntracks;
    uint64_t seed;
    double sigma1, sigma2;     /* hit resolutions (cm) */
    double misal;              /* misalignment scale (cm) */
    double outlierFrac;        /* fraction of hits with 20x wider noise */
    double theta0;             /* multiple-scattering angle (rad) */
    int32_t threads;           /* > 1: tracks generated on that many threads, each
                                  track from its own random stream (seed, track);
                                  other data than the sequential stream of <= 1 */
} mpgen_cfg;

int mpgen_count(const mpgen_cfg *cfg, int64_t *nrec, int64_t *nwords, int32_t *nlabels);
int mpgen_fill(const mpgen_cfg *cfg, int64_t *recPtr, int32_t *inder, double *glder,
               double *truth);
int mpgen_constraints(const mpgen_cfg *cfg, int32_t *ncon, int32_t *conStart,
                      int32_t *conLabel, double *conCoef);
int mpgen_constraint_words(const mpgen_cfg *cfg);

#ifdef __cplusplus
}
#endif
#endif
