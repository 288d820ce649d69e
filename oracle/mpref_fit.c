/*
 * mpref_fit.c -- oracle: the per-record local fit and global-matrix update
 * (loopbf, pede.f90:3387-4442).  TEST INFRASTRUCTURE ONLY.
 *
 * One record at a time: measurement decode, subtraction of the current global
 * parameters, normal equations, optional bordered-band detection, local
 * solve, outlier down-weighting iterations, rejection cuts, the global vector
 * and the Schur update Gt W G - B Gamma^-1 Bt, which is subtracted from the
 * global matrix in packed (matsto 1) or mpbits-sparse (matsto 2) storage.
 */
#include "mpref.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

void mpref__sqminv1(double *v1, double *b1, int32_t n, int32_t *nrank, double *diag1,
                    int32_t *next1);
void mpref__sqmibb_any(int32_t side, double *v1, double *b1, int32_t n, int32_t nbdr,
                       int32_t nbnd, int32_t inv, int32_t *nrank, double *evdmin,
                       double *evdmax);

/* chindl, mpnum.f90:2078-2115 (single precision) */
float mpref_chindl(int32_t n, int32_t nd)
{
    static const float sn[3] = {0.47523f, 1.690140f, 2.782170f};
    static const float table[3][30] = {
        {1.0000f, 1.1479f, 1.1753f, 1.1798f, 1.1775f, 1.1730f, 1.1680f, 1.1630f,
         1.1581f, 1.1536f, 1.1493f, 1.1454f, 1.1417f, 1.1383f, 1.1351f, 1.1321f,
         1.1293f, 1.1266f, 1.1242f, 1.1218f, 1.1196f, 1.1175f, 1.1155f, 1.1136f,
         1.1119f, 1.1101f, 1.1085f, 1.1070f, 1.1055f, 1.1040f},
        {4.0000f, 3.0900f, 2.6750f, 2.4290f, 2.2628f, 2.1415f, 2.0481f, 1.9736f,
         1.9124f, 1.8610f, 1.8171f, 1.7791f, 1.7457f, 1.7161f, 1.6897f, 1.6658f,
         1.6442f, 1.6246f, 1.6065f, 1.5899f, 1.5745f, 1.5603f, 1.5470f, 1.5346f,
         1.5230f, 1.5120f, 1.5017f, 1.4920f, 1.4829f, 1.4742f},
        {9.0000f, 5.9146f, 4.7184f, 4.0628f, 3.6410f, 3.3436f, 3.1209f, 2.9468f,
         2.8063f, 2.6902f, 2.5922f, 2.5082f, 2.4352f, 2.3711f, 2.3143f, 2.2635f,
         2.2178f, 2.1764f, 2.1386f, 2.1040f, 2.0722f, 2.0428f, 2.0155f, 1.9901f,
         1.9665f, 1.9443f, 1.9235f, 1.9040f, 1.8855f, 1.8681f}};
    int32_t m;
    if (nd < 1) return 0.0f;
    m = n < 3 ? n : 3;
    if (m < 1) m = 1;
    if (nd <= 30) return table[m - 1][nd - 1];
    float x = sn[m - 1] + sqrtf((float)(nd + nd - 1));
    return (x * x) / (float)(nd + nd);
}

/* addsums, pede.f90:11666-11697 (single accumulator) */
/* monitoring of the first local-fit iteration (pede.f90:3938-3980,
 * 4025-4032): the histograms of the device monitor, filled with the same
 * arithmetic; set by mpref_set_monitor (tests only) */
static struct {
    int32_t on, pull, nbins, measBins, mode;
    float range;
    const int32_t *measIndex;
    const double *measRes;
    int64_t *hist, *meas;
} g_mon;

void mpref_set_monitor(int32_t on, int32_t pull, int32_t nbins, float range, int32_t measBins, int32_t mode,
                       const int32_t *measIndex, const double *measRes, int64_t *hist, int64_t *meas)
{
    g_mon.on = on; g_mon.pull = pull; g_mon.nbins = nbins; g_mon.range = range;
    g_mon.measBins = measBins; g_mon.mode = mode; g_mon.measIndex = measIndex;
    g_mon.measRes = measRes; g_mon.hist = hist; g_mon.meas = meas;
}

static void mon_hist(int h, float x)
{
    int b;
    if (!(x == x)) return;
    if (x < -g_mon.range) b = 0;
    else if (x >= g_mon.range) b = g_mon.nbins + 1;
    else {
        b = 1 + (int)((x + g_mon.range) * ((float)g_mon.nbins / (2.0f * g_mon.range)));
        if (b > g_mon.nbins) b = g_mon.nbins;
    }
    __atomic_fetch_add(&g_mon.hist[h * (g_mon.nbins + 2) + b], 1, __ATOMIC_RELAXED);
}

static void addsums(mpref_fitout *o, double chi2, int32_t ndf, double dw)
{
    double add = chi2 * dw;
    int64_t nadd = (int64_t)add;
    o->chi2SumI += nadd;
    o->chi2SumD += (add - (double)nadd);
    if (o->chi2SumD > 16.0) {
        o->chi2SumD -= 16.0;
        o->chi2SumI += 16;
    }
    o->ndfSum += (int64_t)ndf;
    o->ndfSumW += (double)ndf * dw;
}

/* growable per-thread scratch */
typedef struct {
    int64_t cap_eq, cap_alg, cap_alc, cap_var;
    int64_t *eqL, *eqG, *eqE;
    double *rm1, *lcor, *lwgt;
    double *clmat, *blvec;     /* 1-based */
    int32_t *ibandh;           /* 1-based, 2*nalc */
    double *scdiag;
    int32_t *scflag;
    int32_t *usage, *back;     /* usage 1-based; back[1..nVar] */
    int32_t *grp;
    double *lgm;               /* localGlobalMatrix 1-based */
    int32_t *lgmap;            /* localGlobalMap 1-based */
    int32_t *lgs;              /* localGlobalStructure 1-based */
    double *upd;               /* writeBufferUpdates (one record) 1-based */
} scratch;

static void *grow(void *p, int64_t n, size_t sz)
{
    return realloc(p, (size_t)(n + 4) * sz);
}

static int scratch_fit(scratch *s, int64_t neq, int64_t nalg, int64_t nalc, int32_t nVar)
{
    if (neq > s->cap_eq) {
        s->cap_eq = neq * 2;
        s->eqL = grow(s->eqL, s->cap_eq, sizeof(int64_t));
        s->eqG = grow(s->eqG, s->cap_eq, sizeof(int64_t));
        s->eqE = grow(s->eqE, s->cap_eq, sizeof(int64_t));
        s->rm1 = grow(s->rm1, s->cap_eq, sizeof(double));
        s->lcor = grow(s->lcor, s->cap_eq, sizeof(double));
        s->lwgt = grow(s->lwgt, s->cap_eq, sizeof(double));
    }
    if (nalc > s->cap_alc || nalg > s->cap_alg) {
        if (nalc > s->cap_alc) s->cap_alc = nalc * 2;
        if (nalg > s->cap_alg) s->cap_alg = nalg * 2;
        int64_t a = s->cap_alc, g = s->cap_alg;
        s->clmat = grow(s->clmat, a * (a + 1) / 2, sizeof(double));
        s->blvec = grow(s->blvec, a, sizeof(double));
        s->ibandh = grow(s->ibandh, 2 * a, sizeof(int32_t));
        s->scdiag = grow(s->scdiag, a, sizeof(double));
        s->scflag = grow(s->scflag, a, sizeof(int32_t));
        s->usage = grow(s->usage, g, sizeof(int32_t));
        s->grp = grow(s->grp, g, sizeof(int32_t));
        s->lgm = grow(s->lgm, a * g, sizeof(double));
        s->lgmap = grow(s->lgmap, a * g, sizeof(int32_t));
        s->lgs = grow(s->lgs, 2 * a * g + a + g + 1, sizeof(int32_t));
        s->upd = grow(s->upd, g * (g + 1) / 2, sizeof(double));
    }
    if (!s->back) {
        s->cap_var = nVar;
        s->back = (int32_t *)calloc((size_t)nVar + 2, sizeof(int32_t));
    }
    return 1;
}

static void scratch_free(scratch *s)
{
    free(s->eqL); free(s->eqG); free(s->eqE); free(s->rm1); free(s->lcor); free(s->lwgt);
    free(s->clmat); free(s->blvec); free(s->ibandh); free(s->scdiag); free(s->scflag);
    free(s->usage); free(s->back); free(s->grp); free(s->lgm); free(s->lgmap); free(s->lgs);
    free(s->upd);
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* dbavat, mpnum.f90:1389-1447: w += A V At (iopt=1).  1-based, A is m x n
 * row-major (a(il+l), il=(i-1)*n). */
static void dbavat(const double *v, const double *a, double *w, int32_t n, int32_t m)
{
    int32_t i, k, l, j, il = -n, ijs = 0, lkl, lk, jk, ij;
    double cik;
    for (i = 1; i <= m; i++) {
        ijs = ijs + i - 1;
        il = il + n;
        lkl = 0;
        for (k = 1; k <= n; k++) {
            cik = 0.0;
            lkl = lkl + k - 1;
            lk = lkl;
            for (l = 1; l <= k; l++) {
                lk = lk + 1;
                cik = cik + a[il + l] * v[lk];
            }
            for (l = k + 1; l <= n; l++) {
                lk = lk + l - 1;
                cik = cik + a[il + l] * v[lk];
            }
            jk = k;
            ij = ijs;
            for (j = 1; j <= i; j++) {
                ij = ij + 1;
                w[ij] = w[ij] + cik * a[jk];
                jk = jk + n;
            }
        }
    }
}

/* dbavats, mpnum.f90:1470-1528 (sparse A described by is[]) */
static void dbavats(const double *v, const double *a, const int32_t *is, double *w,
                    int32_t n, int32_t m, int32_t *sc)
{
    int32_t i, k, l, j, ijs = 0, ic, in, lk, ir, ij;
    double cik;
    sc[1] = 0;
    for (k = 2; k <= n; k++) sc[k] = sc[k - 1] + k - 1;
    for (i = 1; i <= m; i++) {
        ijs = ijs + i - 1;
        for (k = 1; k <= n; k++) {
            cik = 0.0;
            for (l = is[i] + 1; l <= is[i + 1]; l += 2) {
                ic = is[l];
                in = is[l + 1];
                lk = sc[k > ic ? k : ic] + (k > ic ? ic : k);
                cik = cik + a[in] * v[lk];
            }
            for (j = is[m + k] + 1; j <= is[m + k + 1]; j += 2) {
                ir = is[j];
                in = is[j + 1];
                if (ir > i) break;
                ij = ijs + ir;
                w[ij] = w[ij] + cik * a[in];
            }
        }
    }
}

typedef struct {
    const mpref_fitopt *opt;
    const int64_t *recPtr;
    const int32_t *inder;
    const double *glder;
    const int32_t *recFile;
    const double *fileWeight;
    const double *gpar;
    const int32_t *vidx;
    int32_t nVar, nG;
    const int32_t *aig;    /* allIndexGroups */
    const int32_t *p2g;    /* parToGroup */
    const int64_t *off;
    const int32_t *col;
} ctx_t;

/* subtract one record's update (packed nalg x nalg over the sorted variable
 * indices usage[1..nalg]) from the global matrix (mgupdt semantics; an
 * element of a pair left out by pairentries is dropped as mupdat drops it,
 * pede.f90:3172, where mgupdt itself stops, pede.f90:3313-3319) */
static int apply_update(const ctx_t *c, const int32_t *usage, int32_t nalg, const double *upd,
                        double *matD)
{
    int32_t i, j;
    for (i = 1; i <= nalg; i++) {
        int64_t gi = usage[i];
        for (j = 1; j <= i; j++) {
            int64_t gj = usage[j];
            double s = upd[(i * i - i) / 2 + j];
            if (c->opt->matsto == 2) {
                if (gi == gj) {
                    matD[gi - 1] -= s;
                } else {
                    int64_t ij = mpref_ijadd((int32_t)gi, (int32_t)gj, c->nG, c->aig, c->p2g,
                                             c->off, c->col);
                    if (ij <= 0) {
                        if (c->opt->mreqpe > 1) continue;  /* pair left out (pairentries) */
                        return 23;
                    }
                    matD[ij - 1] -= s;
                }
            } else {
                int64_t ia = gi > gj ? gi : gj, ja = gi > gj ? gj : gi;
                matD[(ia * ia - ia) / 2 + ja - 1] -= s;
            }
        }
    }
    return 0;
}

/* One record of loopbf.  Returns 0 or an error code; *status set. */
static int fit_record(const ctx_t *c, int64_t r, scratch *s, double *gvec, int64_t *gcnt,
                      double *matD, mpref_fitout *out, int32_t *status, int32_t *naccf,
                      float *chi2f, int32_t *ndff)
{
    const mpref_fitopt *o = c->opt;
    const int32_t *inder = c->inder;
    const double *glder = c->glder;
    const double chuber = 1.345, cauchy = 2.3849;
    int64_t endOfEntry = c->recPtr[r + 1] - 1, lastGlobal, startLocal, startGlobal, sp;
    int32_t kfl = c->recFile ? c->recFile[r] : 1;
    double dw1 = c->fileWeight ? c->fileWeight[kfl - 1] : 1.0;
    double dw2 = sqrt(dw1);
    int32_t nalg = 0, nalc = 0, neq = 0, i, j, k, ieq, rc = 0;

    /* sizes first (neq, nalc upper bound) so scratch can be sized */
    lastGlobal = c->recPtr[r];
    {
        int64_t nw = c->recPtr[r + 1] - c->recPtr[r];
        scratch_fit(s, nw, nw, nw, c->nVar);
    }
    /* ----- first loop: decode, subtract global parameters, collect nalg */
    for (;;) {
        if (mpref_decode(inder, glder, endOfEntry, &lastGlobal, &startLocal, &startGlobal, &sp))
            return 20;
        if (startLocal < 0) break;
        double rmeas = glder[startLocal];
        neq++;
        s->eqL[neq] = startLocal;
        s->eqG[neq] = startGlobal;
        s->eqE[neq] = lastGlobal;
        for (j = 1; j <= lastGlobal - startGlobal; j++) {
            int32_t li = inder[startGlobal + j];
            rmeas = rmeas - glder[startGlobal + j] * c->gpar[li - 1];
            if (o->icalcm == 1) {
                int32_t ij = c->vidx[li - 1];
                if (ij > 0 && s->back[ij] == 0) {
                    nalg++;
                    s->usage[nalg] = ij;
                    s->back[ij] = nalg;
                }
            }
        }
        s->rm1[neq] = rmeas;
        for (j = 1; j <= startGlobal - startLocal - 1; j++) {
            int32_t ij = inder[startLocal + j];
            if (ij > nalc) nalc = ij;
        }
    }
    *status = -1;
    if (nalc <= 0) goto done;
    scratch_fit(s, neq, nalg, nalc, c->nVar);

    int32_t ngg = (nalg * nalg + nalg) / 2, ngrp = 0;
    if (o->icalcm == 1) {
        memset(s->lgm + 1, 0, sizeof(double) * (size_t)(nalg * nalc));
        memset(s->lgmap + 1, 0, sizeof(int32_t) * (size_t)(nalg * nalc));
        qsort(s->usage + 1, (size_t)nalg, sizeof(int32_t), cmp_i32);
        int32_t prev = -1, npar = 0;
        for (k = 1; k <= nalg; k++) {
            int32_t iext = s->usage[k];
            s->back[iext] = k;
            int32_t g = c->p2g[iext - 1];
            if (g != prev) {
                ngrp++;
                s->grp[ngrp] = g;
                prev = g;
                npar += c->aig[g] - c->aig[g - 1];
            }
        }
        if (npar != nalg) { rc = 35; goto done; }
        for (k = 1; k <= ngg; k++) s->upd[k] = 0.0;
    }

    /* ----- iterations */
    int32_t nter = 1;
    if (o->nloopn != 1 && o->lhuber != 0) nter = o->lhuber;
    for (ieq = 1; ieq <= neq; ieq++) s->lcor[ieq] = 0.0;
    int32_t mbnd = -1, mbdr = nalc, mside = -1;
    for (i = 1; i <= 2 * nalc; i++) s->ibandh[i] = 0;
    int32_t iter = 0, nrank = 0, ndf = 0, nan = 0, inv;
    double summ = 0.0, suwt;
    float cndl10 = 0.0f, chndf = 0.0f, resing = 0.0f;
    int32_t nweig;
    double *clmat = s->clmat, *blvec = s->blvec;
    while (iter < nter) {
        iter++;
        for (i = 1; i <= nalc; i++) blvec[i] = 0.0;
        for (i = 1; i <= (nalc * nalc + nalc) / 2; i++) clmat[i] = 0.0;
        nweig = 0;
        cndl10 = 0.0f;
        for (ieq = 1; ieq <= neq; ieq++) {
            startLocal = s->eqL[ieq];
            startGlobal = s->eqG[ieq];
            double rmeas = s->rm1[ieq];
            double rerr = glder[startGlobal];
            double wght = 1.0 / (rerr * rerr);
            nweig++;
            double resid = rmeas - s->lcor[ieq];
            if (o->nloopn != 1 && iter != 1 && o->lhuber != 0) {
                if (iter <= 3) {
                    if (fabs(resid) > chuber * rerr) wght = wght * chuber * rerr / fabs(resid);
                } else {
                    double t = resid / rerr / cauchy;
                    wght = wght / (1.0 + t * t);
                }
            }
            s->lwgt[ieq] = wght;
            for (j = 1; j <= startGlobal - startLocal - 1; j++) {
                int32_t ij = inder[startLocal + j];
                blvec[ij] = blvec[ij] + wght * rmeas * glder[startLocal + j];
                for (k = 1; k <= j; k++) {
                    int32_t ik = inder[startLocal + k];
                    int32_t jk = (ij * ij - ij) / 2 + ik;
                    clmat[jk] = clmat[jk] + wght * glder[startLocal + j] * glder[startLocal + k];
                    if (iter == 1) {
                        int32_t id = abs(ij - ik) + 1;
                        int32_t im = ij < ik ? ij : ik;
                        if (im > s->ibandh[id]) s->ibandh[id] = im;
                        im = (nalc + 1 - ij) < (nalc + 1 - ik) ? (nalc + 1 - ij) : (nalc + 1 - ik);
                        if (im > s->ibandh[nalc + id]) s->ibandh[nalc + id] = im;
                    }
                }
            }
        }
        /* bordered band detection (pede.f90:3838-3874) */
        if (iter == 1 && nalc > 5 && o->lfitbb > 0) {
            int32_t kx = -1, kbdrx = 0, kbdr, kbnd;
            int64_t icmn = (int64_t)nalc * nalc * nalc, icost;
            kbdr = 0;
            for (k = nalc; k >= 2; k--) {
                kbnd = k - 2;
                if (s->ibandh[k] > kbdr) kbdr = s->ibandh[k];
                icost = 6 * (int64_t)(nalc - kbdr) * (int64_t)(kbnd + kbdr + 1) *
                            (int64_t)(kbnd + kbdr + 1) +
                        2 * (int64_t)kbdr * kbdr * kbdr;
                if (icost < icmn) {
                    icmn = icost;
                    kx = k;
                    kbdrx = kbdr;
                    mside = 1;
                }
            }
            if (kx < 0) {
                kbdr = 0;
                for (k = nalc; k >= 2; k--) {
                    kbnd = k - 2;
                    if (s->ibandh[k + nalc] > kbdr) kbdr = s->ibandh[k + nalc];
                    icost = 6 * (int64_t)(nalc - kbdr) * (int64_t)(kbnd + kbdr + 1) *
                                (int64_t)(kbnd + kbdr + 1) +
                            2 * (int64_t)kbdr * kbdr * kbdr;
                    if (icost < icmn) {
                        icmn = icost;
                        kx = k;
                        kbdrx = kbdr;
                        mside = 2;
                    }
                }
            }
            if (kx > 0) {
                mbnd = kx - 2;
                mbdr = kbdrx;
            }
        }
        if (mbnd >= 0) {
            double evdmin, evdmax;
            if (o->nloopn == 1) {
                out->nbndr[mside - 1]++;
                if (mbdr > out->nbdrx) out->nbdrx = mbdr;
                if (mbnd > out->nbndx) out->nbndx = mbnd;
            }
            inv = 0;
            if (iter == 1) inv = 1;   /* lfitnp defaults to huge: pulls always */
            if (o->icalcm == 1) inv = 2;
            mpref__sqmibb_any(mside, clmat, blvec, nalc, mbdr, mbnd, inv, &nrank, &evdmin,
                              &evdmax);
            if (evdmin > 0.0) cndl10 = log10f((float)(evdmax / evdmin));
        } else {
            inv = 2;
            mpref__sqminv1(clmat, blvec, nalc, &nrank, s->scdiag, s->scflag);
        }
        nan = 0;
        for (k = 1; k <= nalc; k++)
            if (!(blvec[k] <= 0.0) && !(blvec[k] > 0.0)) nan++;

        /* third loop: residuals and chi2 */
        summ = 0.0;
        suwt = 0.0;
        for (ieq = 1; ieq <= neq; ieq++) {
            startLocal = s->eqL[ieq];
            startGlobal = s->eqG[ieq];
            double rmeas = s->rm1[ieq];
            double rerr = glder[startGlobal];
            double wght = 1.0 / (rerr * rerr);
            double rmloc = 0.0;
            for (j = 1; j <= startGlobal - startLocal - 1; j++) {
                int32_t ij = inder[startLocal + j];
                rmloc = rmloc + glder[startLocal + j] * blvec[ij];
            }
            s->lcor[ieq] = rmloc;
            rmeas = rmeas - rmloc;
            if (g_mon.on && iter == 1) {
                const int withGlobal = startGlobal < s->eqE[ieq];
                mon_hist(withGlobal ? 0 : 1, (float)(rmeas / rerr));
                if (g_mon.pull && (mbnd < 0 || nrank == nalc)) {
                    double dvar = 0.0;
                    for (j = 1; j <= startGlobal - startLocal - 1; j++) {
                        int32_t ij = inder[startLocal + j];
                        int32_t jk = (ij * ij - ij) / 2;
                        for (k = 1; k <= j - 1; k++) {
                            int32_t ik = inder[startLocal + k];
                            dvar = dvar + clmat[jk + ik] * glder[startLocal + j] * glder[startLocal + k] * 2.0;
                        }
                        dvar = dvar + clmat[jk + ij] * glder[startLocal + j] * glder[startLocal + j];
                    }
                    if (0.999999 / wght > dvar) {
                        double pull = rmeas / sqrt(1.0 / wght - dvar);
                        mon_hist(withGlobal ? 2 : 3, (float)pull);
                        if (withGlobal && g_mon.measIndex) {
                            int32_t g = g_mon.measIndex[inder[startGlobal + 1] - 1];
                            if (g > 0) {
                                double half = 0.5 * (double)g_mon.measBins;
                                double x = g_mon.mode == 0 ? pull * rerr / g_mon.measRes[g - 1] / 0.1 + half
                                                           : pull / 0.1 + half;
                                int irbin = x == x ? (int)x : 1;
                                irbin = irbin < 1 ? 1 : (irbin > g_mon.measBins ? g_mon.measBins : irbin);
                                __atomic_fetch_add(&g_mon.meas[(int64_t)(g - 1) * g_mon.measBins + irbin - 1], 1,
                                                   __ATOMIC_RELAXED);
                            }
                        }
                    }
                }
            }
            double dchi2 = wght * rmeas * rmeas;
            double resid = rmeas;
            if (o->nloopn != 1 && iter != 1 && o->lhuber != 0) {
                if (iter <= 3) {
                    if (fabs(resid) > chuber * rerr) {
                        wght = wght * chuber * rerr / fabs(resid);
                        dchi2 = 2.0 * chuber * (fabs(resid) / rerr - 0.5 * chuber);
                    }
                } else {
                    double t = resid / rerr / cauchy;
                    wght = wght / (1.0 + t * t);
                    dchi2 = log(1.0 + t * t) * (cauchy * cauchy);
                }
            }
            double down = 1.0 / sqrt(wght);
            suwt = suwt + rerr / down;
            summ = summ + dchi2;
        }
        ndf = neq - nrank;
        resing = ((float)nweig - (float)suwt) / (float)nweig;
        if (nan > 0) { out->nrej[0]++; *status = 1; goto done; }
        if (nrank != nalc) { out->nrej[1]++; *status = 2; goto done; }
        if (cndl10 > o->cndlmx) { out->nrej[2]++; *status = 3; goto done; }
        if (ndf <= 0) { out->nrej[3]++; *status = 4; goto done; }
        chndf = (float)(summ / (double)ndf);
    }

    /* ----- rejection cuts (pede.f90:4106-4144) */
    {
        float chichi = mpref_chindl(3, ndf) * (float)ndf;
        if (o->chicut >= 0.0f) {
            if (summ > (double)(o->chhuge * chichi)) {
                out->nrej[4]++;
                *status = 5;
                goto done;
            }
            if (o->chicut > 0.0f) {
                float chlimt = o->chicut * chichi;
                if (summ > (double)chlimt) {
                    addsums(out, (double)chlimt, ndf, dw1);
                    out->nrej[5]++;
                    *status = 6;
                    goto done;
                }
            }
        }
        if (o->lhuber > 1 && o->dwcut != 0.0f && resing > o->dwcut) {
            addsums(out, summ, ndf, dw1);
            out->nrej[5]++;
            *status = 6;
            goto done;
        }
    }
    *status = 0;
    if (naccf) naccf[kfl - 1] += 1;
    if (ndff) ndff[kfl - 1] += ndf;
    if (chi2f) chi2f[kfl - 1] += chndf;

    /* ----- fourth loop: global vector, Gt W G, local-global matrix */
    summ = 0.0;
    for (ieq = 1; ieq <= neq; ieq++) {
        startLocal = s->eqL[ieq];
        startGlobal = s->eqG[ieq];
        lastGlobal = s->eqE[ieq];
        double rmeas = s->rm1[ieq] - s->lcor[ieq];   /* residual after the last fit */
        double rerr = glder[startGlobal];
        double wght = 1.0 / (rerr * rerr);
        double dchi2 = wght * rmeas * rmeas;
        if (o->nloopn != 1 && o->lhuber != 0) {
            double resid = fabs(rmeas);
            if (nter <= 3) {
                if (resid > chuber * rerr) dchi2 = 2.0 * chuber * (resid / rerr - 0.5 * chuber);
            } else {
                double t = resid / rerr / cauchy;
                dchi2 = log(1.0 + t * t) * (cauchy * cauchy);
            }
            wght = s->lwgt[ieq];
        }
        summ = summ + dchi2;
        for (j = 1; j <= lastGlobal - startGlobal; j++) {
            int32_t ivgbj = c->vidx[inder[startGlobal + j] - 1];
            if (glder[startGlobal + j] == 0.0) continue;
            if (ivgbj > 0) {
                gvec[ivgbj - 1] = gvec[ivgbj - 1] + dw1 * wght * rmeas * glder[startGlobal + j];
                gcnt[ivgbj - 1] += 1;
                if (o->icalcm == 1) {
                    int32_t ije = s->back[ivgbj];
                    for (k = 1; k <= j; k++) {
                        int32_t ivgbk = c->vidx[inder[startGlobal + k] - 1];
                        if (ivgbk > 0) {
                            int32_t ike = s->back[ivgbk];
                            int32_t ia = ije > ike ? ije : ike, ib = ije > ike ? ike : ije;
                            int32_t ij = ib + (ia * ia - ia) / 2;
                            s->upd[ij] = s->upd[ij] - dw1 * wght * glder[startGlobal + j] *
                                                          glder[startGlobal + k];
                        }
                    }
                }
            }
        }
        if (o->icalcm != 1) continue;
        for (j = 1; j <= lastGlobal - startGlobal; j++) {
            int32_t ivgbj = c->vidx[inder[startGlobal + j] - 1];
            if (ivgbj > 0) {
                int32_t ije = s->back[ivgbj];
                for (k = 1; k <= startGlobal - startLocal - 1; k++) {
                    int32_t ik = inder[startLocal + k];
                    int32_t jk = ik + (ije - 1) * nalc;
                    s->lgm[jk] = s->lgm[jk] + dw2 * wght * glder[startGlobal + j] *
                                                  glder[startLocal + k];
                    s->lgmap[jk] += 1;
                }
            }
        }
    }
    addsums(out, summ, ndf, dw1);
    if (o->icalcm != 1) goto done;

    /* ----- B Gamma^-1 Bt (dense or sparse product) and matrix update */
    {
        int32_t *lgs = s->lgs;
        int32_t isize = nalc + nalg + 1;
        k = 0;
        for (i = 1; i <= nalg; i++) {
            lgs[i] = isize;
            for (j = 1; j <= nalc; j++) {
                if (s->lgmap[k + j] > 0) {
                    lgs[isize + 1] = j;
                    lgs[isize + 2] = k + j;
                    isize += 2;
                }
            }
            k += nalc;
        }
        if (isize - lgs[1] < nalc * nalg) {
            for (j = 1; j <= nalc; j++) {
                lgs[nalg + j] = isize;
                k = 0;
                for (i = 1; i <= nalg; i++) {
                    if (s->lgmap[k + j] > 0) {
                        lgs[isize + 1] = i;
                        lgs[isize + 2] = k + j;
                        isize += 2;
                    }
                    k += nalc;
                }
            }
            lgs[nalg + nalc + 1] = isize;
            dbavats(clmat, s->lgm, lgs, s->upd, nalc, nalg, s->scflag);
        } else {
            dbavat(clmat, s->lgm, s->upd, nalc, nalg);
        }
        rc = apply_update(c, s->usage, nalg, s->upd, matD);
    }

done:
    for (i = 1; i <= nalg; i++) s->back[s->usage[i]] = 0;
    return rc;
}

int mpref_loopbf(const mpref_fitopt *opt, int64_t nrec, const int64_t *recPtr,
                 const int32_t *inder, const double *glder, const int32_t *recFile,
                 int32_t nfiles, const double *fileWeight, const double *globalParameter,
                 const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                 const int32_t *allIndexGroups, const int32_t *parToGroup,
                 const int64_t *offsets, const int32_t *columns, double *globalVector,
                 int64_t *globalCounter, double *matD, mpref_fitout *out,
                 int32_t *recStatus, int32_t *naccf, float *chi2f, int32_t *ndff)
{
    ctx_t c = {opt, recPtr, inder, glder, recFile, fileWeight, globalParameter,
               varIndexOfTotal, nVar, nG, allIndexGroups, parToGroup, offsets, columns};
    scratch s;
    int rc = 0;
    (void)nfiles;
    memset(&s, 0, sizeof(s));
    for (int64_t r = 0; r < nrec; r++) {
        int32_t st = -1;
        rc = fit_record(&c, r, &s, globalVector, globalCounter, matD, out, &st, naccf, chi2f,
                        ndff);
        if (recStatus) recStatus[r] = st;
        if (rc) break;
    }
    scratch_free(&s);
    return rc;
}

int mpref_loopbf_omp(int32_t nthreads, const mpref_fitopt *opt, int64_t nrec,
                     const int64_t *recPtr, const int32_t *inder, const double *glder,
                     const int32_t *recFile, int32_t nfiles, const double *fileWeight,
                     const double *globalParameter, const int32_t *varIndexOfTotal,
                     int32_t nVar, int32_t nG, const int32_t *allIndexGroups,
                     const int32_t *parToGroup, const int64_t *offsets,
                     const int32_t *columns, int64_t nmat, double *globalVector,
                     int64_t *globalCounter, double *matD, mpref_fitout *out, int32_t *status)
{
    ctx_t c = {opt, recPtr, inder, glder, recFile, fileWeight, globalParameter,
               varIndexOfTotal, nVar, nG, allIndexGroups, parToGroup, offsets, columns};
    int rcall = 0;
    (void)nfiles;
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        scratch s;
        mpref_fitout lo;
        double *lv = (double *)calloc((size_t)nVar, sizeof(double));
        int64_t *lc = (int64_t *)calloc((size_t)nVar, sizeof(int64_t));
        double *lm = (double *)calloc((size_t)nmat, sizeof(double));
        int rc = 0;
        memset(&s, 0, sizeof(s));
        memset(&lo, 0, sizeof(lo));
#pragma omp for schedule(dynamic, 64)
        for (int64_t r = 0; r < nrec; r++) {
            int32_t st = 0;
            if (rc == 0) rc = fit_record(&c, r, &s, lv, lc, lm, &lo, &st, NULL, NULL, NULL);
            if (status) status[r] = st;
        }
#pragma omp critical
        {
            for (int32_t i = 0; i < nVar; i++) {
                globalVector[i] += lv[i];
                globalCounter[i] += lc[i];
            }
            for (int64_t i = 0; i < nmat; i++) matD[i] += lm[i];
            for (int k = 0; k < 6; k++) out->nrej[k] += lo.nrej[k];
            out->chi2SumI += lo.chi2SumI;
            out->chi2SumD += lo.chi2SumD;
            out->ndfSum += lo.ndfSum;
            out->ndfSumW += lo.ndfSumW;
            if (rc) rcall = rc;
        }
        free(lv); free(lc); free(lm);
        scratch_free(&s);
    }
    return rcall;
}
