/*
 * mpref_run.c -- oracle: one whole alignment job and the millepede.res
 * writer.  TEST INFRASTRUCTURE ONLY.
 *
 * Control flow follows mptwo/xloopn/loopn/addcst (pede.f90:33-528,
 * 8501-9334, 2479-2885, 704-771) without the line search and the
 * function-value loops: every iteration rebuilds the matrix, solves and adds
 * the correction.  The chi2-cut schedule per data loop is the one of loopn
 * (pede.f90:2583-2593).  feasib (pede.f90:1553-1680) makes the start values
 * feasible before the first data loop (cut 1e-12, pede.f90:8693, 8730) and
 * every corrected parameter set after a solution (cut 1e-6, 8865-8866).
 */
#include "mpref.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int32_t find_label(const int32_t *labels, int32_t n, int32_t item)
{
    int32_t lo = 0, hi = n - 1;
    while (lo <= hi) {
        int32_t mid = (lo + hi) / 2;
        if (labels[mid] == item) return mid;
        if (labels[mid] < item) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

/* feasib (pede.f90:1553-1680) for one constraint group: residuals
 * r = rhs - C p over all labels, rms test against concut in the first of two
 * iterations, then p_var += C^T (C C^T)^-1 r.  pinv: the inverse of the
 * product matrix C C^T (packed, inverted by sqminv as feasma does,
 * pede.f90:1466-1478); dbsvx (mpnum.f90:1264-1297) multiplies it. */
static int feasib(const mpref_job *job, const mpref_result *res, int32_t ntot, const double *pinv,
                  double *gpar, float concut)
{
    int32_t ncon = job->ncon, iact = 0;
    if (ncon <= 0) return 0;
    double *r = (double *)malloc(sizeof(double) * (size_t)ncon);
    double *lam = (double *)malloc(sizeof(double) * (size_t)ncon);
    for (int iter = 1; iter <= 2; iter++) {
        double sum1 = 0.0;
        for (int32_t c = 0; c < ncon; c++) {
            double rhs = job->conRhs ? job->conRhs[c] : 0.0;
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; k++) {
                int32_t li = find_label(res->labels, ntot, job->conLabel[k]);
                if (li >= 0) rhs = rhs - job->conCoef[k] * gpar[li];
            }
            r[c] = rhs;
            sum1 = sum1 + rhs * rhs;
        }
        sum1 = sqrt(sum1 / (double)ncon);
        if (iter == 1 && sum1 < concut) break;
        iact = 1;
        /* dbsvx: lam = V r with V packed symmetric */
        int64_t ijs = 0;
        for (int32_t i = 0; i < ncon; i++) {
            double dsum = 0.0;
            int64_t ij = ijs;
            for (int32_t j = 0; j < ncon; j++) {
                dsum = dsum + pinv[ij] * r[j];
                if (j < i) ij += 1; else ij += j + 1;
            }
            lam[i] = dsum;
            ijs += i + 1;
        }
        for (int32_t c = 0; c < ncon; c++)
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; k++) {
                int32_t li = find_label(res->labels, ntot, job->conLabel[k]);
                if (li >= 0 && res->varIndex[li] > 0) gpar[li] = gpar[li] + lam[c] * job->conCoef[k];
            }
    }
    free(r);
    free(lam);
    return iact;
}

int mpref_run(const mpref_steer *st, const mpref_job *job, mpref_result *res)
{
    int rc = 0;
    int64_t nw = job->recPtr[job->nrec];
    int32_t nsteer = 0, i, j;
    int32_t *steer = (int32_t *)malloc(sizeof(int32_t) *
        (size_t)(job->npar + (job->ncon ? job->conStart[job->ncon] : 0) +
                 (job->nmeas ? job->msStart[job->nmeas] : 0) + 1));
    for (i = 0; i < job->npar; i++) steer[nsteer++] = job->parLabel[i];
    if (job->ncon) for (i = 0; i < job->conStart[job->ncon]; i++) steer[nsteer++] = job->conLabel[i];
    if (job->nmeas) for (i = 0; i < job->msStart[job->nmeas]; i++) steer[nsteer++] = job->msLabel[i];

    int32_t cap = res->cap;
    int32_t *grpStart = (int32_t *)malloc(sizeof(int32_t) * (size_t)cap);
    int32_t *totGroup = (int32_t *)malloc(sizeof(int32_t) * (size_t)cap);
    int64_t *counter = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
    int32_t nVar = 0, nG = 0;
    int32_t ntot = mpref_loop1(job->nrec, job->recPtr, job->inder, job->glder, nsteer, steer,
                               job->npar, job->parLabel, job->parSigma, st->mreqenf, cap,
                               res->labels, counter, res->varIndex, grpStart, totGroup,
                               &nVar, &nG);
    free(steer);
    if (ntot < 0) { res->exitCode = 20; free(grpStart); free(totGroup); free(counter); return 20; }
    res->nTotal = ntot;
    res->nVar = nVar;
    res->nVarGroups = nG;
    if (nVar <= 0) { res->exitCode = 22; free(grpStart); free(totGroup); free(counter); return 22; }

    int32_t *aig = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nG + 1));
    int32_t *p2g = (int32_t *)malloc(sizeof(int32_t) * (size_t)nVar);
    mpref_var_groups(ntot, res->varIndex, totGroup, nVar, nG, aig, p2g);
    int32_t *tinder = (int32_t *)malloc(sizeof(int32_t) * (size_t)nw);
    mpref_translate(job->nrec, job->recPtr, job->inder, job->glder, ntot, res->labels, tinder);

    int64_t *offsets = NULL, nmat, ncolw = 0;
    int32_t *columns = NULL;
    if (st->matsto == 2) {
        /* the pairs of the measurement lines belong to the sparse structure
         * whatever the records hold (pede.f90:7007-7042, with the
         * increment mreqpe, so they are always kept): one structure-only
         * record per measurement line, its labels as global words, after
         * the data records */
        int64_t nrecS = job->nrec, *rpS = (int64_t *)job->recPtr;
        int32_t *inS = tinder;
        double *glS = (double *)job->glder;
        if (job->nmeas > 0) {
            int64_t extra = 0;
            for (int32_t m = 0; m < job->nmeas; m++) extra += 3 + (job->msStart[m + 1] - job->msStart[m]);
            nrecS = job->nrec + job->nmeas;
            rpS = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nrecS + 1));
            inS = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nw + extra));
            glS = (double *)malloc(sizeof(double) * (size_t)(nw + extra));
            int32_t *raw = (int32_t *)malloc(sizeof(int32_t) * (size_t)extra);
            int64_t *rpRaw = (int64_t *)malloc(sizeof(int64_t) * ((size_t)job->nmeas + 1));
            memcpy(rpS, job->recPtr, sizeof(int64_t) * ((size_t)job->nrec + 1));
            memcpy(inS, tinder, sizeof(int32_t) * (size_t)nw);
            memcpy(glS, job->glder, sizeof(double) * (size_t)nw);
            int64_t q = 0;
            for (int32_t m = 0; m < job->nmeas; m++) {
                rpRaw[m] = q;
                /* header, value, sigma (positive: not a special block), labels */
                raw[q] = 0; glS[nw + q] = 0.0; q++;
                raw[q] = 0; glS[nw + q] = 0.0; q++;
                raw[q] = 0; glS[nw + q] = 1.0; q++;
                for (int32_t k = job->msStart[m]; k < job->msStart[m + 1]; k++) {
                    raw[q] = job->msLabel[k];
                    glS[nw + q] = 1.0;
                    q++;
                }
            }
            rpRaw[job->nmeas] = q;
            mpref_translate(job->nmeas, rpRaw, raw, glS + nw, ntot, res->labels, inS + nw);
            for (int32_t m = 0; m <= job->nmeas; m++) rpS[job->nrec + m] = nw + rpRaw[m];
            free(raw);
            free(rpRaw);
        }
        int64_t capc = 64 + 4 * (int64_t)nVar * 64;
        offsets = (int64_t *)malloc(sizeof(int64_t) * 2 * ((size_t)nG + 1));
        for (;;) {
            columns = (int32_t *)malloc(sizeof(int32_t) * (size_t)capc);
            if (mpref_mpbits(nrecS, job->nrec, rpS, inS, glS, res->varIndex, nVar, nG,
                             aig, p2g, st->mreqpe, capc, offsets, columns, &ncolw, &nmat) == 0)
                break;
            free(columns);
            capc *= 4;
        }
        if (job->nmeas > 0) { free(rpS); free(inS); free(glS); }
    } else {
        nmat = (int64_t)nVar * (nVar + 1) / 2;
    }

    /* constraints -> matConstraintsT rows over variable parameters */
    int32_t ncon = job->ncon;
    mpref_ql *q = NULL;
    double *A = NULL;
    if (ncon > 0) {
        A = (double *)calloc((size_t)ncon * (size_t)nVar, sizeof(double));
        for (int32_t c = 0; c < ncon; c++)
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; k++) {
                int32_t li = find_label(res->labels, ntot, job->conLabel[k]);
                if (li < 0) continue;
                int32_t iv = res->varIndex[li];
                if (iv > 0) A[(int64_t)c * nVar + iv - 1] += job->conCoef[k];
            }
        q = mpref_ql_create(nVar, ncon, A);
    }
    int32_t nfit = nVar - ncon;
    res->nFit = nfit;

    double *gpar = (double *)calloc((size_t)ntot, sizeof(double));
    double *gstart = (double *)calloc((size_t)ntot, sizeof(double));
    double *psig = (double *)calloc((size_t)ntot, sizeof(double));
    for (i = 0; i < job->npar; i++) {
        int32_t li = find_label(res->labels, ntot, job->parLabel[i]);
        if (li < 0) continue;
        if (job->parValue) { gpar[li] = job->parValue[i]; gstart[li] = job->parValue[i]; }
        if (job->parSigma) psig[li] = job->parSigma[i];
    }
    /* product matrix of the constraints over the variable parameters,
     * summed parameter by parameter (feasma, pede.f90:1466-1476), inverted */
    double *pinv = NULL;
    if (ncon > 0) {
        pinv = (double *)calloc((size_t)ncon * (ncon + 1) / 2, sizeof(double));
        double *dummy = (double *)calloc((size_t)ncon, sizeof(double));
        int32_t prank = 0;
        for (int32_t l = 0; l < nVar; l++) {
            int64_t ij = 0;
            for (int32_t a = 0; a < ncon; a++)
                for (int32_t b = 0; b <= a; b++, ij++)
                    pinv[ij] = pinv[ij] + A[(int64_t)a * nVar + l] * A[(int64_t)b * nVar + l];
        }
        mpref_sqminv(pinv, dummy, ncon, &prank);
        free(dummy);
        feasib(job, res, ntot, pinv, gpar, 1.0e-12f);
    }
    double *diag0 = (double *)calloc((size_t)nVar, sizeof(double));
    double *pw = (double *)calloc((size_t)nVar, sizeof(double));
    int32_t *v2t = (int32_t *)malloc(sizeof(int32_t) * (size_t)nVar);
    for (i = 0; i < ntot; i++)
        if (res->varIndex[i] > 0) v2t[res->varIndex[i] - 1] = i;
    for (i = 0; i < nVar; i++) {
        double s = psig[v2t[i]];
        pw[i] = s > 0.0 ? 1.0 / (s * s) : 0.0;
    }

    double *gvec = (double *)malloc(sizeof(double) * (size_t)nVar);
    int64_t *gcnt = (int64_t *)malloc(sizeof(int64_t) * (size_t)nVar);
    double *matD = (double *)malloc(sizeof(double) * (size_t)nmat);
    double *corr = (double *)malloc(sizeof(double) * (size_t)nVar);
    double *cres = (double *)calloc((size_t)(ncon > 0 ? ncon : 1), sizeof(double));
    double *csol = (double *)calloc((size_t)(ncon > 0 ? ncon : 1), sizeof(double));
    double *err = (double *)calloc((size_t)nVar, sizeof(double));
    int haveErr = 0;
    float chicut = st->chicut;
    int64_t nrejTot = 0;
    memset(res->nrej, 0, sizeof(res->nrej));

    for (int32_t iter = 1; iter <= st->mitera; iter++) {
        int32_t nloopn = iter;
        if (nloopn > 1) {
            if (nloopn == 2) chicut = st->chirem;
            else {
                chicut = sqrtf(chicut);
                if (chicut != 0.0f && chicut < 1.5f) chicut = 1.0f;
                if (chicut != 0.0f && nrejTot == 0) chicut = 1.0f;
            }
        }
        mpref_fitopt fo = {1, nloopn, st->lhuber, st->lfitbb, st->matsto,
                           chicut, st->chhuge, st->dwcut, st->cndlmx,
                           st->matsto == 2 ? st->mreqpe : 1};
        mpref_fitout out;
        memset(&out, 0, sizeof(out));
        memset(gvec, 0, sizeof(double) * (size_t)nVar);
        memset(gcnt, 0, sizeof(int64_t) * (size_t)nVar);
        memset(matD, 0, sizeof(double) * (size_t)nmat);
        if (st->nthreads > 1)
            rc = mpref_loopbf_omp(st->nthreads, &fo, job->nrec, job->recPtr, tinder, job->glder,
                                  job->recFile, job->nfiles, job->fileWeight, gpar, res->varIndex,
                                  nVar, nG, aig, p2g, offsets, columns, nmat, gvec, gcnt, matD,
                                  &out, NULL);
        else
            rc = mpref_loopbf(&fo, job->nrec, job->recPtr, tinder, job->glder, job->recFile,
                              job->nfiles, job->fileWeight, gpar, res->varIndex, nVar, nG, aig,
                              p2g, offsets, columns, gvec, gcnt, matD, &out, NULL, NULL, NULL,
                              NULL);
        if (rc) break;
        nrejTot = 0;
        for (i = 0; i < 6; i++) { res->nrej[i] = out.nrej[i]; nrejTot += out.nrej[i]; }
        if (3 * nrejTot > job->nrec) { rc = 26; break; }
        /* pre-sigmas (loopn, pede.f90:2711-2718) */
        for (i = 0; i < nVar; i++)
            if (pw[i] != 0.0)
                mpref_mupdat(st->matsto, i + 1, i + 1, pw[i], nG, aig, p2g, offsets, columns, matD);
        /* measurement lines (loopn, pede.f90:2743-2798) */
        for (int32_t m = 0; m < job->nmeas; m++) {
            double rhs = job->msRhs[m], sgm = job->msSigma[m];
            double weight = sgm > 0.0 ? 1.0 / (sgm * sgm) : 0.0, dsum = -rhs;
            int32_t ia = job->msStart[m], ib = job->msStart[m + 1];
            for (j = ia; j < ib; j++) {
                int32_t li = find_label(res->labels, ntot, job->msLabel[j]);
                if (li >= 0) dsum = dsum + job->msCoef[j] * gpar[li];
            }
            for (j = ia; j < ib; j++) {
                double fj = job->msCoef[j];
                if (fj == 0.0) continue;
                int32_t li = find_label(res->labels, ntot, job->msLabel[j]);
                int32_t ivj = li >= 0 ? res->varIndex[li] : 0;
                if (ivj > 0) {
                    gvec[ivj - 1] = gvec[ivj - 1] - weight * dsum * fj;
                    gcnt[ivj - 1] += 1;
                    for (int32_t k = ia; k <= j; k++) {
                        int32_t lk = find_label(res->labels, ntot, job->msLabel[k]);
                        int32_t ivk = lk >= 0 ? res->varIndex[lk] : 0;
                        if (ivk > 0)
                            mpref_mupdat(st->matsto, ivj, ivk, weight * fj * job->msCoef[k], nG,
                                         aig, p2g, offsets, columns, matD);
                    }
                }
            }
            double adder = weight * dsum * dsum;
            double add = adder;
            int64_t nadd = (int64_t)add;
            out.chi2SumI += nadd;
            out.chi2SumD += add - (double)nadd;
            out.ndfSum += 1;
            out.ndfSumW += 1.0;
        }
        res->fvalue = out.chi2SumD + (double)out.chi2SumI;
        res->ndf = out.ndfSum;
        /* addcst (pede.f90:704-771): constraint residuals */
        for (int32_t c = 0; c < ncon; c++) {
            double rhs = job->conRhs ? job->conRhs[c] : 0.0;
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; k++) {
                int32_t li = find_label(res->labels, ntot, job->conLabel[k]);
                if (li >= 0) rhs = rhs - job->conCoef[k] * gpar[li];
            }
            cres[c] = rhs;
        }
        for (i = 0; i < nVar; i++) corr[i] = gvec[i];

        if (st->metsol == 1 || st->metsol == 3) {
            /* minver saves the diagonal for the global correlations
             * (pede.f90:7864-7866) */
            for (int64_t r = 1; r <= nVar; r++) diag0[r - 1] = matD[(r * r - r) / 2 + r - 1];
            if (ncon > 0) {
                mpref_ql_ssq_packed(q, matD, 1);
                mpref_ql_bsub(q, cres, csol);
                mpref_ql_mlq(q, corr, 1);
                for (i = 1; i <= nfit; i++)
                    for (j = 1; j <= ncon; j++) {
                        int64_t r = nfit + j;
                        corr[i - 1] = corr[i - 1] - matD[(r * r - r) / 2 + i - 1] * csol[j - 1];
                    }
            }
            int32_t nrank = 0;
            if (st->metsol == 1) {
                mpref_sqminl(matD, corr, nfit, &nrank);
            } else {
                double evmax, evmin;
                mpref_chdec2(matD, nfit, &nrank, &evmax, &evmin);
                mpref_chslv2(matD, corr, nfit);
            }
            res->nrank = nrank;
            if (ncon > 0) {
                for (j = 0; j < ncon; j++) corr[nfit + j] = csol[j];
                mpref_ql_mlq(q, corr, 0);
            }
            if (st->metsol == 1 && iter == st->mitera) {
                /* errors: Q A^-1 Q^T with the constraint rows zeroed
                 * (xloopn, pede.f90:9094-9121) */
                if (ncon > 0) {
                    for (int64_t r = nfit + 1; r <= nVar; r++)
                        for (int64_t c = 1; c <= r; c++) matD[(r * r - r) / 2 + c - 1] = 0.0;
                    mpref_ql_ssq_packed(q, matD, 0);
                }
                for (int64_t r = 1; r <= nVar; r++) err[r - 1] = matD[(r * r - r) / 2 + r - 1];
                haveErr = 1;
            }
        } else if (st->metsol == 4 || st->metsol == 5) {
            double *rhs = (double *)malloc(sizeof(double) * (size_t)nVar);
            for (i = 0; i < nVar; i++) rhs[i] = corr[i];
            if (ncon > 0) {
                double *xav = (double *)calloc((size_t)nVar, sizeof(double));
                double *bav = (double *)calloc((size_t)nVar, sizeof(double));
                mpref_ql_bsub(q, cres, csol);
                for (j = 0; j < ncon; j++) xav[nfit + j] = csol[j];
                mpref_ql_mlq(q, xav, 0);
                mpref_avprd0(st->matsto, nVar, xav, bav, nG, aig, offsets, columns, matD);
                for (i = 0; i < nVar; i++) rhs[i] = rhs[i] - bav[i];
                mpref_ql_mlq(q, rhs, 1);
                free(xav);
                free(bav);
            }
            int32_t itn = 0;
            res->minresIstop = mpref_minres_precond(st->metsol == 5, st->matsto, nVar, nG, aig, offsets,
                                                    columns, matD, q, rhs, corr, st->mrestl, st->itnlim,
                                                    st->mbandw, st->lprecm, &itn, NULL);
            res->minresItn = itn;
            if (ncon > 0) {
                for (j = 0; j < ncon; j++) corr[nfit + j] = csol[j];
                mpref_ql_mlq(q, corr, 0);
            }
            free(rhs);
        }
        for (i = 0; i < nVar; i++) {
            if (!(corr[i] <= 0.0) && !(corr[i] > 0.0)) { rc = 25; break; }
            gpar[v2t[i]] += corr[i];
        }
        res->nloopn = nloopn;
        if (rc) break;
        if (ncon > 0) feasib(job, res, ntot, pinv, gpar, 1.0e-6f);
    }

    for (i = 0; i < ntot; i++) {
        res->parameter[i] = gpar[i];
        res->presigma[i] = psig[i];
        res->error[i] = 0.0;
        res->counts[i] = 0;
        int32_t iv = res->varIndex[i];
        if (res->start) res->start[i] = gstart[i];
        if (res->fileCounts) res->fileCounts[i] = counter[i];
        if (res->gcor) res->gcor[i] = -1.0;
        if (iv > 0) {
            res->counts[i] = gcnt[iv - 1];
            if (haveErr) {
                double e = sqrt(fabs(err[iv - 1]));
                res->error[i] = err[iv - 1] < 0.0 ? -e : e;
                /* global correlation (prtglo, pede.f90:4537-4544) */
                double gmati = err[iv - 1], dg = diag0[iv - 1];
                if (res->gcor && gmati * dg > 0.0) {
                    double gcor2 = 1.0 - 1.0 / (gmati * dg);
                    if (gcor2 >= 0.0 && gcor2 <= 1.0) res->gcor[i] = (double)(float)sqrt(gcor2);
                }
            }
        }
    }
    res->exitCode = rc;
    free(grpStart); free(totGroup); free(counter); free(aig); free(p2g); free(tinder);
    free(offsets); free(columns); free(A); mpref_ql_destroy(q); free(gpar); free(gstart);
    free(psig); free(pw); free(v2t); free(gvec); free(gcnt); free(matD); free(corr);
    free(cres); free(csol); free(err); free(diag0); free(pinv);
    return rc;
}

/* Fortran Gw.d edit descriptor (w=14, d=5) as written by prtglo */
static void fmt_g(char *buf, double v)
{
    const int w = 14, d = 5;
    char t[64];
    if (v == 0.0) {
        snprintf(t, sizeof t, "%.*f    ", d - 1, 0.0);
        snprintf(buf, 32, "%*s", w, t);
        return;
    }
    snprintf(t, sizeof t, "%.*E", d - 1, v);
    char *e = strchr(t, 'E');
    int ex = atoi(e + 1) + 1;  /* value = 0.ddddd * 10^ex */
    if (ex >= 0 && ex <= d) {
        char f[48];
        snprintf(f, sizeof f, "%.*f    ", d - ex, v);
        snprintf(buf, 32, "%*s", w, f);
    } else {
        /* 0.ddddd E+xx */
        char mant[16];
        int neg = v < 0.0;
        int k = 0;
        for (char *p = t; p < e; p++)
            if (*p >= '0' && *p <= '9') mant[k++] = *p;
        mant[k] = 0;
        char f[48];
        snprintf(f, sizeof f, "%s0.%sE%c%02d", neg ? "-" : "", mant, ex < 0 ? '-' : '+',
                 ex < 0 ? -ex : ex);
        snprintf(buf, 32, "%*s", w, f);
    }
}

int mpref_write_res_opts(const char *path, const mpref_result *res, int32_t errors, int32_t ipcntr,
                         int32_t igcorr, int32_t mreqena)
{
    FILE *f;
    char a[32], b[32], c[32], d[32];
    if (ipcntr < 0 || (ipcntr > 1 && !res->fileCounts)) return -1;
    f = fopen(path, "w");
    if (!f) return -1;
    fprintf(f, " Parameter   ! first 3 elements per line are significant (if used as input)\n");
    for (int32_t i = 0; i < res->nTotal; i++) {
        int32_t iv = res->varIndex[i];
        long long icount = 0;
        int lowstat = 0;
        fmt_g(a, (double)(float)res->parameter[i]);
        fmt_g(b, (double)(float)res->presigma[i]);
        if (iv > 0) {
            icount = res->counts[i];
            lowstat = icount < mreqena;
        }
        if (ipcntr > 1) icount = res->fileCounts[i];
        if (lowstat) icount = -(icount + 1);
        if (iv <= 0) {
            if (ipcntr != 0) fprintf(f, "%10d  %s%s%28s%12lld\n", res->labels[i], a, b, "", icount);
            else fprintf(f, "%10d  %s%s\n", res->labels[i], a, b);
            continue;
        }
        fmt_g(c, (double)(float)(res->parameter[i] - (res->start ? res->start[i] : 0.0)));
        if (errors) {
            fmt_g(d, (double)(float)res->error[i]);
            if (ipcntr != 0) fprintf(f, "%10d  %s%s%s%s%12lld\n", res->labels[i], a, b, c, d, icount);
            else if (igcorr && res->gcor)
                fprintf(f, "%10d  %s%s%s%s%8.3f\n", res->labels[i], a, b, c, d, (double)(float)res->gcor[i]);
            else fprintf(f, "%10d  %s%s%s%s\n", res->labels[i], a, b, c, d);
        } else {
            if (ipcntr != 0) fprintf(f, "%10d  %s%s%s%14s%12lld\n", res->labels[i], a, b, c, "", icount);
            else fprintf(f, "%10d  %s%s%s\n", res->labels[i], a, b, c);
        }
    }
    fclose(f);
    return 0;
}

int mpref_write_res(const char *path, const mpref_result *res, int32_t errors)
{
    return mpref_write_res_opts(path, res, errors, 0, 0, 0);
}
