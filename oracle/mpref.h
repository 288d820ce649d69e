/*
 * mpref -- CPU oracle for the pede hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C, FP64 restatement of Millepede-II pede's local fit,
 * Schur-complement accumulation, sparse structure build and global solvers.
 * It exists only to check the GB300 implementation: tests, the smoke check
 * and the CPU-baseline leg of bench.py may call it; the product library never
 * links or calls it.
 *
 * Each function cites the reference routine (file:line, paths relative to the
 * Millepede-II source tree) whose algorithm and operation order it follows.
 * Floating-point expressions keep the reference's evaluation order and the
 * file is compiled with -ffp-contract=off, so the local-fit decisions are
 * reproducible bit for bit.
 *
 * Conventions: arrays crossing this interface are 0-based C arrays whose
 * CONTENT follows the reference (1-based parameter / group indices, reference
 * storage offsets).  Element k of a Fortran array a(1:n) is a[k-1].
 */
#ifndef MPREF_H
#define MPREF_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------
 * Record buffer (Mille record content; pede.f90:1693-1713).
 * Record r occupies words [recPtr[r], recPtr[r+1]); word recPtr[r] is the
 * error-count word.  inder holds labels (raw) or total indices (translated).
 * ------------------------------------------------------------------- */

/* decodeNextMeasurement (pede.f90:2428-2468).  Positions are absolute word
 * positions; *startLocal = -1 signals the end of the record.  Returns 0, or
 * 20 for a record whose zero markers run past its end. */
int mpref_decode(const int32_t *inder, const double *glder, int64_t endOfEntry,
                 int64_t *lastGlobal, int64_t *startLocal, int64_t *startGlobal,
                 int64_t *startSpecial);

/* ---------------------------------------------------------------------
 * loop1 (pede.f90:5777-6146) with indexOfGlobalLabel/useone/upone
 * (mppar.f90:89-252), updateParGroups (pede.f90:2157-2302, mcount=0) and
 * pargrp (pede.f90:2311-2404), all records read as one chunk.
 *
 * steerLabels: labels named in steering lines (registered first).
 * preLabel/preSigma: pre-sigmas (<0 fixes the parameter).
 * Outputs (capacity cap): labels[] sorted ascending, counter[] entries per
 * equation, varIndex[] = globalParLabelIndex(2,:), grpStart[] =
 * globalParLabelIndex(3,:), totGroup[] = globalParLabelIndex(4,:).
 * Returns nTotal (>=0) or -1 on capacity overflow / bad record.
 * ------------------------------------------------------------------- */
int mpref_loop1(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                const double *glder, int32_t nsteer, const int32_t *steerLabels,
                int32_t npre, const int32_t *preLabel, const double *preSigma,
                int32_t mreqenf, int32_t cap, int32_t *labels, int64_t *counter,
                int32_t *varIndex, int32_t *grpStart, int32_t *totGroup,
                int32_t *nVar, int32_t *nVarGroups);

/* globalAllIndexGroups (pede.f90:6509-6524), constraints eliminated:
 * allIndexGroups[nVarGroups+1] (1-based first var index of each group). */
void mpref_var_groups(int32_t nTotal, const int32_t *varIndex, const int32_t *totGroup,
                      int32_t nVar, int32_t nVarGroups, int32_t *allIndexGroups,
                      int32_t *parToGroup);

/* Translate labels -> total indices (prepareRecords(1), mppar.f90:282-321)
 * into outInder (same length as inder).  labels[] sorted.  Returns 0 or 20. */
int mpref_translate(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                    const double *glder, int32_t nTotal, const int32_t *labels,
                    int32_t *outInder);

/* ---------------------------------------------------------------------
 * Sparse structure (matsto=2): clbits/inbits/ndbits/spbits
 * (mpbits.f90:73-142,182-243,305-566,1220-1350) with the record pair fill
 * of loop2 (pede.f90:6889-6908).  nspc=1 (msngpe < 1), mextnd=0.  Records
 * hold total indices; records from nrecData on are the structure-only
 * records of the measurement lines, whose pairs count mreqpe
 * (pede.f90:7036).  Group pairs counted fewer than mreqpe times
 * (pairentries) are left out.
 * Outputs: offsets[2*(nG+1)] = sparseMatrixOffsets (column-major 2 x (nG+1)),
 * columns[] (cap words) = sparseMatrixColumns; *ncolw words used;
 * *nmat = length of globalMatD (diagonal + off-diagonal).
 * Returns 0 or -1 (capacity).
 * ------------------------------------------------------------------- */
int mpref_mpbits(int64_t nrec, int64_t nrecData, const int64_t *recPtr, const int32_t *inder,
                 const double *glder, const int32_t *varIndexOfTotal, int32_t nVar,
                 int32_t nG, const int32_t *allIndexGroups, const int32_t *parToGroup,
                 int32_t mreqpe, int64_t cap, int64_t *offsets, int32_t *columns,
                 int64_t *ncolw, int64_t *nmat);

/* ijpgrp (pede.f90:5371-5461) / ijadd (pede.f90:5498-5537): 1-based index
 * into globalMatD for variable parameters (i,j); 0 if not stored. */
int64_t mpref_ijadd(int32_t i, int32_t j, int32_t nG, const int32_t *allIndexGroups,
                    const int32_t *parToGroup, const int64_t *offsets,
                    const int32_t *columns);

/* ---------------------------------------------------------------------
 * loopbf (pede.f90:3387-4442) + mgupdt (pede.f90:3219-3357)
 * ------------------------------------------------------------------- */
typedef struct mpref_fitopt {
    int32_t icalcm;   /* 1: build matrix */
    int32_t nloopn;   /* data-loop counter (1 = first loop) */
    int32_t lhuber;   /* outlier down-weighting iterations */
    int32_t lfitbb;   /* bordered band detection (>0 on) */
    int32_t matsto;   /* 1 packed, 2 sparse */
    float chicut;     /* chi2 cut factor (<0 none) */
    float chhuge;     /* huge chi2 cut factor */
    float dwcut;      /* down-weight fraction cut */
    float cndlmx;     /* max log10(cond) of band part */
    int32_t mreqpe;   /* pairentries: above 1 (sparse), the updates of group
                         pairs left out of the structure are dropped as mupdat
                         drops them (pede.f90:3172); otherwise a pair missing
                         from the structure is error 23 */
} mpref_fitopt;

typedef struct mpref_fitout {
    int64_t nrej[6];
    int64_t chi2SumI;   /* addsums integer part */
    double chi2SumD;    /* addsums remainder */
    int64_t ndfSum;
    double ndfSumW;
    int32_t nbndr[2];
    int32_t nbdrx, nbndx;
} mpref_fitout;

/* Records must hold total indices.  globalParameter[nTotal];
 * varIndexOfTotal[nTotal]; recFile[nrec] (1-based) or NULL; fileWeight[nfiles]
 * or NULL.  globalVector[nVar], globalCounter[nVar] and matD[] are ADDED to
 * (zero them for a fresh loop).  recStatus[nrec] (optional): 0 accepted,
 * 1..6 rejection class, -1 no local parameters.  naccf/chi2f/ndff[nfiles]
 * optional (added to).  Returns 0, or an error code (23 bad index, 20 bad
 * record, 35 group mismatch). */
int mpref_loopbf(const mpref_fitopt *opt, int64_t nrec, const int64_t *recPtr,
                 const int32_t *inder, const double *glder, const int32_t *recFile,
                 int32_t nfiles, const double *fileWeight, const double *globalParameter,
                 const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                 const int32_t *allIndexGroups, const int32_t *parToGroup,
                 const int64_t *offsets, const int32_t *columns, double *globalVector,
                 int64_t *globalCounter, double *matD, mpref_fitout *out,
                 int32_t *recStatus, int32_t *naccf, float *chi2f, int32_t *ndff);

/* Same loop, records split over nthreads OpenMP threads with per-thread
 * matrices/vectors that are summed at the end (CPU baseline timing). */
int mpref_loopbf_omp(int32_t nthreads, const mpref_fitopt *opt, int64_t nrec,
                     const int64_t *recPtr, const int32_t *inder, const double *glder,
                     const int32_t *recFile, int32_t nfiles, const double *fileWeight,
                     const double *globalParameter, const int32_t *varIndexOfTotal,
                     int32_t nVar, int32_t nG, const int32_t *allIndexGroups,
                     const int32_t *parToGroup, const int64_t *offsets,
                     const int32_t *columns, int64_t nmat, double *globalVector,
                     int64_t *globalCounter, double *matD, mpref_fitout *out, int32_t *status);

/* mupdat (pede.f90:3134-3204): add `add` to element (i,j) (1-based var). */
void mpref_mupdat(int32_t matsto, int32_t i, int32_t j, double add, int32_t nG,
                  const int32_t *allIndexGroups, const int32_t *parToGroup,
                  const int64_t *offsets, const int32_t *columns, double *matD);

/* chindl (mpnum.f90:2078-2115) */
float mpref_chindl(int32_t n, int32_t nd);

/* ---------------------------------------------------------------------
 * Local solvers (exposed for unit tests)
 * ------------------------------------------------------------------- */
/* sqminv (mpnum.f90:97-213): packed v[(n*n+n)/2], b[n] in place. */
void mpref_sqminv(double *v, double *b, int32_t n, int32_t *nrank);
/* sqmibb / sqmibb2 (mpnum.f90:3118-3354 / 3390-3600) */
void mpref_sqmibb(double *v, double *b, int32_t n, int32_t nbdr, int32_t nbnd,
                  int32_t inv, int32_t *nrank, double *evdmin, double *evdmax);
void mpref_sqmibb2(double *v, double *b, int32_t n, int32_t nbdr, int32_t nbnd,
                   int32_t inv, int32_t *nrank, double *evdmin, double *evdmax);

/* ---------------------------------------------------------------------
 * Global solvers
 * ------------------------------------------------------------------- */
/* sqminl (mpnum.f90:230-355): packed in-place inverse + solution. */
void mpref_sqminl(double *v, double *b, int32_t n, int32_t *nrank);
/* chdec2 / chslv2 (mpnum.f90:891-987) */
void mpref_chdec2(double *g, int32_t n, int32_t *nrank, double *evmax, double *evmin);
void mpref_chslv2(const double *g, double *x, int32_t n);

/* QL decomposition of the constraint matrix (mpqldec.f90 qldec 125-196,
 * single block).  A is ncon rows of npar (row k = constraint k, i.e. the
 * reference's matConstraintsT).  State is kept in an opaque object. */
typedef struct mpref_ql mpref_ql;
mpref_ql *mpref_ql_create(int32_t npar, int32_t ncon, const double *A);
void mpref_ql_destroy(mpref_ql *q);
/* qlmlq (mpqldec.f90:404-454): x <- Q x (t=0) or Q^T x (t=1) */
void mpref_ql_mlq(const mpref_ql *q, double *x, int32_t t);
/* qlbsub (mpqldec.f90:991-1014) */
void mpref_ql_bsub(const mpref_ql *q, const double *d, double *y);
/* qlgete (mpqldec.f90:955-981) */
void mpref_ql_gete(const mpref_ql *q, double *emin, double *emax);
/* qlssq (mpqldec.f90:573-698) on a packed matrix (t=1: Q^T A Q, t=0: Q A Q^T) */
void mpref_ql_ssq_packed(const mpref_ql *q, double *A, int32_t t);
/* raw access for parity tests: V (ncon*npar), vecVk (ncon), L (ncon*ncon) */
void mpref_ql_export(const mpref_ql *q, double *V, double *Vk, double *L);

/* avprd0 (pede.f90:5069-5232): b = A x for packed (matsto 1) or sparse. */
/* host threads of the sparse avprd0 (CPU baseline timing; default 1) */
void mpref_set_threads(int32_t n);
void mpref_avprd0(int32_t matsto, int32_t n, const double *x, double *b, int32_t nG,
                  const int32_t *allIndexGroups, const int64_t *offsets,
                  const int32_t *columns, const double *matD);

/* Monitoring of the first local-fit iteration (pede.f90:3938-3980,
 * 4025-4032) for the following loopbf calls: hist[4 * (nbins + 2)]
 * (residuals with/without globals, pulls with/without globals) and
 * meas[numMeas * measBins] are incremented (caller zeroes them). */
void mpref_set_monitor(int32_t on, int32_t pull, int32_t nbins, float range, int32_t measBins, int32_t mode,
                       const int32_t *measIndex, const double *measRes, int64_t *hist, int64_t *meas);

/* MINRES (Paige & Saunders 1975) with a diagonal preconditioner (precons
 * with no constraint blocks, mpnum.f90:2881-3080) on the QL-reduced sparse
 * system (avprod, pede.f90:5331-5358).  Returns istop; *itn iterations. */
int32_t mpref_minres_sparse(int32_t matsto, int32_t nVar, int32_t nG,
                            const int32_t *allIndexGroups, const int64_t *offsets,
                            const int32_t *columns, const double *matD,
                            const mpref_ql *q, const double *rhs, double *x,
                            double rtol, int32_t itnlim, int32_t *itn);

/* MINRES-QLP (the published method; the reference vendors
 * minresqlpModule.f90:411-1333) on the same preconditioned reduced system:
 * minimum-length solution of singular systems.  Returns istop. */
int32_t mpref_minresqlp_sparse(int32_t matsto, int32_t nVar, int32_t nG,
                               const int32_t *allIndexGroups, const int64_t *offsets,
                               const int32_t *columns, const double *matD,
                               const mpref_ql *q, const double *rhs, double *x,
                               double rtol, int32_t itnlim, int32_t *itn);

/* MINRES (qlp 0) or MINRES-QLP (qlp 1) with the preconditioner chosen by
 * mbandw as pede's "bandwidth" option (pede.f90:8292-8316): < 0 none, 0 the
 * diagonal, > 0 the variable-band Cholesky factor of the band of Q^T A Q
 * (equdecs/equslvs with constraints eliminated, lltdec option lprecm).
 * *nrkd receives lltdec's rank-deficit code (may be NULL). */
int32_t mpref_minres_precond(int32_t qlp, int32_t matsto, int32_t nVar, int32_t nG,
                             const int32_t *allIndexGroups, const int64_t *offsets,
                             const int32_t *columns, const double *matD, const mpref_ql *q,
                             const double *rhs, double *x, double rtol, int32_t itnlim,
                             int32_t mbandw, int32_t lprecm, int32_t *itn, int32_t *nrkd);

/* The band preconditioner alone: band of Q^T A Q (mbandw > 0) factorised by
 * lltdec; c receives the first nfit rows in the variable-band layout of
 * mpref_band_index (india[nfit-1] doubles). */
int32_t mpref_band_precond(int32_t matsto, int32_t nVar, int32_t nG, const int32_t *allIndexGroups,
                           const int64_t *offsets, const int32_t *columns, const double *matD,
                           const mpref_ql *q, int32_t mbandw, int32_t lprecm, double *c, int32_t *nrkd);
void mpref_band_index(int32_t n, int32_t mbandw, int64_t *india);
/* 1: form the preconditioner of the QL-reduced system (diagonal and band)
 * by qlpssq's own route (mpqldec.f90:711-945) instead of the exact band of
 * Q^T A Q; 0 (default): exact band, as the device does. */
void mpref_set_qlpssq_literal(int32_t on);
int32_t mpref_lltdec(int32_t n, double *c, const int64_t *india, int32_t iopt);
void mpref_lltslv(int32_t n, const double *c, const int64_t *india, double *x);

/* ---------------------------------------------------------------------
 * Whole job (xloopn/loopn/addcst control without line search) and
 * millepede.res writer (prtglo, pede.f90:4477-4651).
 * ------------------------------------------------------------------- */
typedef struct mpref_steer {
    int32_t metsol;     /* 1 inversion, 3 decomposition, 4 MINRES */
    int32_t matsto;     /* 1 packed, 2 sparse */
    int32_t mitera;     /* number of solutions (iterations) */
    int32_t lhuber;     /* outlierdownweighting */
    float chicut, chirem, chhuge, dwcut, cndlmx;
    int32_t lfitbb;
    int32_t mreqenf, mreqena, mreqpe;
    double mrestl;
    int32_t itnlim;
    int32_t nthreads;   /* OpenMP threads for the data loop (1 = literal) */
    int32_t mbandw;     /* MINRES preconditioner: < 0 none, 0 diagonal, > 0 band width */
    int32_t lprecm;     /* lltdec option of the band preconditioner (skyline) */
} mpref_steer;

typedef struct mpref_job {
    int64_t nrec; const int64_t *recPtr; const int32_t *inder; const double *glder;
    const int32_t *recFile; int32_t nfiles; const double *fileWeight;
    int32_t npar; const int32_t *parLabel; const double *parValue; const double *parSigma;
    int32_t ncon; const int32_t *conStart; const int32_t *conLabel; const double *conCoef;
    const double *conRhs;
    int32_t nmeas; const int32_t *msStart; const int32_t *msLabel; const double *msCoef;
    const double *msRhs; const double *msSigma;
} mpref_job;

typedef struct mpref_result {
    int32_t cap;            /* capacity of the per-label arrays */
    int32_t nTotal, nVar, nVarGroups, nFit;
    int32_t *labels;        /* [cap] */
    double *parameter;      /* [cap] final values */
    double *presigma;       /* [cap] */
    double *error;          /* [cap] (0 where not computed) */
    int64_t *counts;        /* [cap] accepted entries (globalCounter) */
    int32_t *varIndex;      /* [cap] */
    int64_t nrej[6];
    double fvalue; int64_t ndf;
    int32_t nrank;          /* rank of the reduced matrix (inversion/cholesky) */
    int32_t minresItn, minresIstop;
    int32_t nloopn;
    int32_t exitCode;       /* peend code (0 ok) */
    double *start;          /* [cap] start values of the steering, globalParStart (may be NULL) */
    double *gcor;           /* [cap] global correlations of the inversion, -1 undefined (may be NULL) */
    int64_t *fileCounts;    /* [cap] entries in the records, globalParLabelCounter (may be NULL) */
} mpref_result;

int mpref_run(const mpref_steer *st, const mpref_job *job, mpref_result *res);
int mpref_write_res(const char *path, const mpref_result *res, int32_t errors);
/* prtglo with printcounts (ipcntr 0, 1, > 1) and globalcorr (igcorr),
 * formats 102 and 110-112 (pede.f90:4546-4590, 4643-4650) */
int mpref_write_res_opts(const char *path, const mpref_result *res, int32_t errors, int32_t ipcntr,
                         int32_t igcorr, int32_t mreqena);

#ifdef __cplusplus
}
#endif
#endif
