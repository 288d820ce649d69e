/*
 * mpref_solve.c -- oracle: global solvers.  TEST INFRASTRUCTURE ONLY.
 *
 * Packed Gauss-Jordan inversion (sqminl), root-free Cholesky (chdec2/chslv2),
 * Householder QL elimination of linear constraints (mpqldec.f90, one
 * parameter block), the sparse/packed matrix-vector product (avprd0) and
 * preconditioned MINRES written from Paige & Saunders (1975).
 */
#include "mpref.h"
#ifdef _OPENMP
#include <omp.h>
#endif
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* sqminl, mpnum.f90:230-355 (eps = 1e-10 relative pivot limit) */
void mpref_sqminl(double *v0, double *b0, int32_t n, int32_t *nrank)
{
    double *v = v0 - 1, *b = b0 - 1;
    double *diag = (double *)malloc(sizeof(double) * ((size_t)n + 1));
    double *vk = (double *)malloc(sizeof(double) * ((size_t)n + 1));
    int32_t *next = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n + 1));
    const double eps = 1.0E-10;
    int32_t i, j, k, l = 1, last, next0 = 1;
    double vkk, vjk;
    for (i = 1; i <= n; i++) {
        int64_t i8 = i;
        next[i] = i + 1;
        diag[i] = fabs(v[(i8 * i8 + i8) / 2]);
    }
    next[n] = -1;
    *nrank = 0;
    for (i = 1; i <= n; i++) {
        k = 0;
        vkk = 0.0;
        j = next0;
        last = 0;
        while (j > 0) {
            int64_t j8 = j, jj = (j8 * j8 + j8) / 2;
            double lim = fabs(vkk) > eps * diag[j] ? fabs(vkk) : eps * diag[j];
            if (fabs(v[jj]) > lim) {
                vkk = v[jj];
                k = j;
                l = last;
            }
            last = j;
            j = next[last];
        }
        if (k != 0) {
            int64_t k8 = k, kk = (k8 * k8 + k8) / 2, kkmk = kk - k8, jk;
            if (l == 0) next0 = next[k];
            else next[l] = next[k];
            next[k] = 0;
            (*nrank)++;
            vkk = 1.0 / vkk;
            v[kk] = -vkk;
            b[k] = b[k] * vkk;
            jk = kkmk;
            for (j = 1; j <= n; j++) {
                if (j == k) {
                    jk = kk;
                    vk[j] = 0.0;
                } else {
                    if (j < k) jk = jk + 1;
                    else jk = jk + j - 1;
                    v[jk] = v[jk] * vkk;
                    vk[j] = v[jk];
                }
            }
            for (j = n; j >= 1; j--) {
                if (j == k) continue;
                int64_t j8 = j, jl = j8 * (j8 - 1) / 2;
                vjk = vk[j] / vkk;
                b[j] = b[j] - b[k] * vjk;
                for (int32_t c = 1; c <= j; c++) v[jl + c] = v[jl + c] - vk[c] * vjk;
            }
        } else {
            for (k = 1; k <= n; k++) {
                int64_t k8 = k, kk = (k8 * k8 - k8) / 2;
                if (next[k] != 0) {
                    b[k] = 0.0;
                    for (j = 1; j <= k; j++)
                        if (next[j] != 0) v[kk + j] = 0.0;
                }
            }
            break;
        }
    }
    for (int64_t jj = 1; jj <= (int64_t)n * (int64_t)(n + 1) / 2; jj++) v[jj] = -v[jj];
    free(diag);
    free(vk);
    free(next);
}

/* chdec2, mpnum.f90:891-942 (root-free LDLt of the packed lower triangle,
 * processed from the last row upwards; diagonal replaced by 1/d) */
void mpref_chdec2(double *g0, int32_t n, int32_t *nrank, double *evmax, double *evmin)
{
    double *g = g0 - 1;
    int64_t ii = ((int64_t)n * (int64_t)(n + 1)) / 2, jj;
    int32_t i, j;
    double ratio;
    *nrank = 0;
    *evmax = 0.0;
    *evmin = 0.0;
    for (i = n; i >= 1; i--) {
        if (g[ii] > 0.0) {
            (*nrank)++;
            if (*nrank == 1) {
                *evmax = g[ii];
                *evmin = g[ii];
            } else {
                if (g[ii] > *evmax) *evmax = g[ii];
                if (g[ii] < *evmin) *evmin = g[ii];
            }
            g[ii] = 1.0 / g[ii];
        }
        ii = ii - i;
        for (j = 1; j <= i - 1; j++) {
            ratio = g[ii + j] * g[ii + i];
            if (ratio == 0.0) continue;
            jj = ((int64_t)(j - 1) * (int64_t)j) / 2;
            for (int32_t c = 1; c <= j; c++) g[jj + c] = g[jj + c] - g[ii + c] * ratio;
        }
        for (int32_t c = 1; c <= i - 1; c++) g[ii + c] = g[ii + c] * g[ii + i];
    }
}

/* chslv2, mpnum.f90:953-987 */
void mpref_chslv2(const double *g0, double *x0, int32_t n)
{
    const double *g = g0 - 1;
    double *x = x0 - 1;
    int64_t ii = ((int64_t)n * (int64_t)(n + 1)) / 2, kk;
    int32_t i, k;
    double dsum;
    for (i = n; i >= 1; i--) {
        dsum = x[i];
        kk = ii;
        for (k = i + 1; k <= n; k++) {
            dsum = dsum - g[kk + i] * x[k];
            kk = kk + k;
        }
        x[i] = dsum;
        ii = ii - i;
    }
    for (i = 1; i <= n; i++) {
        dsum = x[i] * g[ii + i];
        for (k = 1; k <= i - 1; k++) dsum = dsum - g[k + ii] * x[k];
        x[i] = dsum;
        ii = ii + i;
    }
}

/* ------------------------------------------------------------------ QL */
struct mpref_ql {
    int32_t npar, ncon;
    double *V;    /* ncon x npar (1-based flat: V[(k-1)*npar + i]) */
    double *Vk;   /* [1..ncon] */
    double *L;    /* ncon x ncon (1-based flat) */
    int32_t *r1, *r2;  /* irangeParNZ */
};

/* qldec, mpqldec.f90:125-196 */
mpref_ql *mpref_ql_create(int32_t npar, int32_t ncon, const double *A)
{
    mpref_ql *q = (mpref_ql *)calloc(1, sizeof(mpref_ql));
    int64_t len = (int64_t)npar * ncon;
    q->npar = npar;
    q->ncon = ncon;
    q->V = (double *)calloc((size_t)len + 1, sizeof(double));
    q->Vk = (double *)calloc((size_t)ncon + 1, sizeof(double));
    q->L = (double *)calloc((size_t)ncon * ncon + 1, sizeof(double));
    q->r1 = (int32_t *)calloc((size_t)ncon + 1, sizeof(int32_t));
    q->r2 = (int32_t *)calloc((size_t)ncon + 1, sizeof(int32_t));
    double *vecN = (double *)calloc((size_t)npar + 1, sizeof(double));
    double *V = q->V;
    for (int64_t i = 0; i < len; i++) V[i + 1] = A[i];
    for (int32_t k = ncon; k >= 1; k--) {
        int32_t kn = npar + k - ncon, i, c;
        int64_t ioff1 = (int64_t)(k - 1) * npar, ioff2, ioff3;
        double nrm = 0.0, sp;
        for (c = 1; c <= kn; c++) vecN[c] = V[ioff1 + c];
        for (c = 1; c <= kn; c++) nrm = nrm + vecN[c] * vecN[c];
        nrm = sqrt(nrm);
        if (nrm == 0.0) continue;
        if (vecN[kn] >= 0.0) vecN[kn] = vecN[kn] + nrm;
        else vecN[kn] = vecN[kn] - nrm;
        nrm = 0.0;
        for (c = 1; c <= kn; c++) nrm = nrm + vecN[c] * vecN[c];
        nrm = sqrt(nrm);
        for (c = 1; c <= kn; c++) vecN[c] = vecN[c] / nrm;
        ioff2 = 0;
        for (i = 1; i <= k; i++) {
            sp = 0.0;
            for (c = 1; c <= kn; c++) sp = sp + vecN[c] * V[ioff2 + c];
            for (c = 1; c <= kn; c++) V[ioff2 + c] = V[ioff2 + c] - 2.0 * vecN[c] * sp;
            ioff2 = ioff2 + npar;
        }
        ioff3 = (int64_t)(k - 1) * ncon;
        for (c = k; c <= ncon; c++) q->L[ioff3 + c] = V[ioff1 + kn + (c - k)];
        for (c = 1; c <= kn - 1; c++) V[ioff1 + c] = vecN[c];
        for (c = kn; c <= npar; c++) V[ioff1 + c] = 0.0;
        q->r1[k] = 1;
        q->r2[k] = kn - 1;
        q->Vk[k] = vecN[kn];
    }
    free(vecN);
    return q;
}

void mpref_ql_destroy(mpref_ql *q)
{
    if (!q) return;
    free(q->V); free(q->Vk); free(q->L); free(q->r1); free(q->r2);
    free(q);
}

void mpref_ql_export(const mpref_ql *q, double *V, double *Vk, double *L)
{
    int64_t len = (int64_t)q->npar * q->ncon;
    if (V) for (int64_t i = 0; i < len; i++) V[i] = q->V[i + 1];
    if (Vk) for (int32_t i = 0; i < q->ncon; i++) Vk[i] = q->Vk[i + 1];
    if (L) for (int64_t i = 0; i < (int64_t)q->ncon * q->ncon; i++) L[i] = q->L[i + 1];
}

/* qlmlq, mpqldec.f90:404-454 (m = 1) */
void mpref_ql_mlq(const mpref_ql *q, double *x0, int32_t t)
{
    double *x = x0 - 1;
    int32_t nconb = q->ncon, nparb = q->npar;
    for (int32_t j = 1; j <= nconb; j++) {
        int32_t k = t ? nconb + 1 - j : j;
        int32_t kn = nparb + k - nconb, ifirst = q->r1[k], ilast = q->r2[k], c;
        const double *vr = q->V + (int64_t)(k - 1) * nparb;   /* vr[1..] */
        double vkn = q->Vk[k];
        if (ifirst <= 0) continue;
        double sp = 0.0;
        for (c = ifirst; c <= ilast; c++) sp = sp + vr[1 + c - ifirst] * x[c];
        sp = sp + vkn * x[kn];
        for (c = ifirst; c <= ilast; c++) x[c] = x[c] - 2.0 * vr[1 + c - ifirst] * sp;
        x[kn] = x[kn] - 2.0 * vkn * sp;
    }
}

/* qlbsub, mpqldec.f90:991-1014 */
void mpref_ql_bsub(const mpref_ql *q, const double *d0, double *y0)
{
    const double *d = d0 - 1;
    double *y = y0 - 1;
    int32_t ncon = q->ncon, nconb = ncon;
    int64_t idiag = (int64_t)ncon * (ncon - 1) + nconb;
    for (int32_t k = nconb; k >= 1; k--) {
        double dot = 0.0;
        for (int32_t c = 1; c <= nconb - k; c++) dot = dot + q->L[idiag + c] * y[k + c];
        y[k] = (d[k] - dot) / q->L[idiag];
        idiag = idiag - ncon - 1;
    }
}

/* qlgete, mpqldec.f90:955-981 */
void mpref_ql_gete(const mpref_ql *q, double *emin, double *emax)
{
    int64_t idiag = 1;
    *emax = q->L[1];
    *emin = *emax;
    for (int32_t i = 1; i <= q->ncon; i++) {
        if (fabs(*emax) < fabs(q->L[idiag])) *emax = q->L[idiag];
        if (fabs(*emin) > fabs(q->L[idiag])) *emin = q->L[idiag];
        idiag = idiag + q->ncon + 1;
    }
}

/* avprds, pede.f90:4855-4930 (packed part): y += A x using only the
 * components x(is..ie); lower part first, then the transposed part */
static void aprod_packed_range(int32_t n, const double *A, const double *x, int32_t is,
                               int32_t ie, double *y)
{
    /* A 1-based packed lower triangle, x, y 1-based */
    for (int32_t i = 1; i <= n; i++) {
        int64_t ij = ((int64_t)i * i - i) / 2;
        int32_t jhi = ie < i ? ie : i;
        for (int32_t j = is; j <= jhi; j++) y[i] = y[i] + A[ij + j] * x[j];
    }
    for (int32_t i = is; i <= ie; i++) {
        int64_t ij = ((int64_t)i * i - i) / 2;
        for (int32_t j = 1; j <= i - 1; j++) y[j] = y[j] + A[ij + j] * x[i];
    }
}

/* qlssq, mpqldec.f90:573-698, packed storage, one block */
void mpref_ql_ssq_packed(const mpref_ql *q, double *A0, int32_t t)
{
    double *A = A0 - 1;
    int32_t nconb = q->ncon, nparb = q->npar;
    double *vecN = (double *)calloc((size_t)nparb + 1, sizeof(double));
    double *Av = (double *)calloc((size_t)nparb + 1, sizeof(double));
    for (int32_t j = 1; j <= nconb; j++) {
        int32_t k = t ? nconb + 1 - j : j;
        int32_t kn = nparb + k - nconb, ifirst = q->r1[k], ilast = q->r2[k], i, c;
        const double *vr = q->V + (int64_t)(k - 1) * nparb;
        double vk = q->Vk[k], vtAv;
        for (c = 1; c <= nparb; c++) vecN[c] = 0.0;
        for (c = ifirst; c <= ilast; c++) vecN[c] = vr[1 + c - ifirst];
        vecN[kn] = vk;
        for (c = 1; c <= nparb; c++) Av[c] = 0.0;
        aprod_packed_range(nparb, A, vecN, ifirst, ilast, Av);
        aprod_packed_range(nparb, A, vecN, kn, kn, Av);
        vtAv = 0.0;
        for (c = ifirst; c <= ilast; c++) vtAv = vtAv + vecN[c] * Av[c];
        vtAv = vtAv + vecN[kn] * Av[kn];
        for (i = 1; i <= kn; i++) {
            int64_t ro = ((int64_t)i * i - i) / 2;
            int32_t ilasti = ilast < i ? ilast : i;
            double f = 2.0 * vecN[i] * vtAv - Av[i];
            for (c = ifirst; c <= ilasti; c++) A[ro + c] = A[ro + c] + 2.0 * (f * vecN[c]);
        }
        for (i = ifirst; i <= ilast; i++) {
            int64_t ro = ((int64_t)i * i - i) / 2;
            for (c = 1; c <= i; c++) A[ro + c] = A[ro + c] - 2.0 * Av[c] * vecN[i];
        }
        {
            int64_t ro = ((int64_t)kn * kn - kn) / 2;
            A[ro + kn] = A[ro + kn] + 2.0 * ((2.0 * vk * vtAv - Av[kn]) * vk - Av[kn] * vk);
        }
        for (i = kn + 1; i <= nparb; i++) {
            int64_t ro = ((int64_t)i * i - i) / 2;
            for (c = ifirst; c <= ilast; c++) A[ro + c] = A[ro + c] - 2.0 * vecN[c] * Av[i];
            A[ro + kn] = A[ro + kn] - 2.0 * vk * Av[i];
        }
    }
    free(vecN);
    free(Av);
}

/* avprd0, pede.f90:5069-5232 (nspc = 1, mextnd = 0) */
/* Host threads of the sparse product (the CPU baseline's timing only; the
 * tests keep the default 1, the reference's sequential order).  With
 * several threads every thread adds its row groups into its own copy of b,
 * and the copies are summed in thread order (the array reduction of the
 * reference's OpenMP loop, pede.f90:5110-5229). */
static int g_avprd0_threads = 1;
void mpref_set_threads(int32_t n) { g_avprd0_threads = n > 1 ? n : 1; }

static void avprd0_groups(int32_t g0, int32_t g1, int32_t nG, const int32_t *allIndexGroups,
                          const int64_t *offsets, const int32_t *columns, const double *matD,
                          const double *x0, double *b0, int first)
{
    const double *x = x0 - 1, *A = matD - 1;
    double *b = b0 - 1;
    int32_t i, j;
    const int32_t *npgrp = allIndexGroups - 1;
    const int32_t *col = columns - 1;
    (void)nG;
    for (int32_t ipg = g0; ipg <= g1; ipg++) {
        int32_t ia = npgrp[ipg], ib = npgrp[ipg + 1] - 1, in = ib - ia + 1;
        for (i = ia; i <= ib; i++) b[i] = (first ? 0.0 : b[i]) + A[i] * x[i];
        int64_t kk = offsets[2 * (ipg - 1)], ll = offsets[2 * (ipg - 1) + 1];
        int64_t ku = offsets[2 * ipg] - kk, indid = kk, indij = ll, k;
        if (ku <= 0) continue;
        if (col[indid + 1] != 0) {
            for (i = ia; i <= ib; i++) {
                for (k = 1; k <= ku; k++) {
                    j = col[indid + k];
                    b[j] = b[j] + A[indij + k] * x[i];
                    b[i] = b[i] + A[indij + k] * x[j];
                }
                indij = indij + ku;
            }
        } else {
            for (k = 2; k <= ku - 2; k += 2) {
                int32_t jg = col[indid + k];
                int32_t ja = npgrp[jg];
                int32_t lj = col[indid + k - 1];
                int32_t jn = col[indid + k + 1] - lj;
                int32_t jb = ja + jn - 1, l;
                lj = 1;
                for (i = ia; i <= ib; i++) {
                    double s = 0.0;
                    for (l = 0; l < jn; l++) s = s + A[indij + lj + l] * x[ja + l];
                    b[i] = b[i] + s;
                    lj = lj + jn;
                }
                lj = 1;
                for (j = ja; j <= jb; j++) {
                    double s = 0.0;
                    for (l = 0; l < in; l++) s = s + A[indij + lj + (int64_t)l * jn] * x[ia + l];
                    b[j] = b[j] + s;
                    lj = lj + 1;
                }
                indij = indij + (int64_t)in * jn;
            }
        }
    }
}

void mpref_avprd0(int32_t matsto, int32_t n, const double *x0, double *b0, int32_t nG,
                  const int32_t *allIndexGroups, const int64_t *offsets,
                  const int32_t *columns, const double *matD)
{
    const double *x = x0 - 1, *A = matD - 1;
    double *b = b0 - 1;
    int32_t i, j;
    if (matsto == 2 && g_avprd0_threads > 1) {
        const int nt = g_avprd0_threads;
        double *copies = (double *)calloc((size_t)nt * (size_t)n, sizeof(double));
#pragma omp parallel num_threads(nt)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double *bt = copies + (size_t)t * (size_t)n;
#pragma omp for schedule(dynamic, 16)
            for (int32_t g = 1; g <= nG; g++)
                avprd0_groups(g, g, nG, allIndexGroups, offsets, columns, matD, x0, bt, 0);
        }
        for (int64_t q = 0; q < n; q++) {
            double v = 0.0;
            for (int t = 0; t < nt; t++) v += copies[(size_t)t * (size_t)n + q];
            b0[q] = v;
        }
        free(copies);
        return;
    }
    if (matsto != 2) {
        for (i = 1; i <= n; i++) {
            int64_t ij = ((int64_t)i * i - i) / 2;
            b[i] = A[ij + i] * x[i];
            for (j = 1; j <= i - 1; j++) {
                b[j] = b[j] + A[ij + j] * x[i];
                b[i] = b[i] + A[ij + j] * x[j];
            }
        }
        return;
    }
    const int32_t *npgrp = allIndexGroups - 1;
    const int32_t *col = columns - 1;
    for (int32_t ipg = 1; ipg <= nG; ipg++) {
        int32_t ia = npgrp[ipg], ib = npgrp[ipg + 1] - 1, in = ib - ia + 1;
        for (i = ia; i <= ib; i++) b[i] = A[i] * x[i];
        int64_t kk = offsets[2 * (ipg - 1)], ll = offsets[2 * (ipg - 1) + 1];
        int64_t ku = offsets[2 * ipg] - kk, indid = kk, indij = ll, k;
        if (ku <= 0) continue;
        if (col[indid + 1] != 0) {
            for (i = ia; i <= ib; i++) {
                for (k = 1; k <= ku; k++) {
                    j = col[indid + k];
                    b[j] = b[j] + A[indij + k] * x[i];
                    b[i] = b[i] + A[indij + k] * x[j];
                }
                indij = indij + ku;
            }
        } else {
            for (k = 2; k <= ku - 2; k += 2) {
                int32_t jg = col[indid + k];
                int32_t ja = npgrp[jg];
                int32_t lj = col[indid + k - 1];
                int32_t jn = col[indid + k + 1] - lj;
                int32_t jb = ja + jn - 1, l;
                lj = 1;
                for (i = ia; i <= ib; i++) {
                    double s = 0.0;
                    for (l = 0; l < jn; l++) s = s + A[indij + lj + l] * x[ja + l];
                    b[i] = b[i] + s;
                    lj = lj + jn;
                }
                lj = 1;
                for (j = ja; j <= jb; j++) {
                    double s = 0.0;
                    for (l = 0; l < in; l++) s = s + A[indij + lj + (int64_t)l * jn] * x[ia + l];
                    b[j] = b[j] + s;
                    lj = lj + 1;
                }
                indij = indij + (int64_t)in * jn;
            }
        }
    }
}

/* ------------------------------------------------------------------
 * Preconditioners of MINRES: none (mbandw < 0), the diagonal of precons
 * (mbandw = 0, no constraint blocks, mpnum.f90:2881-3060: cu = 1/sqrt(c),
 * M^-1 y = (y*cu)*cu) or the variable-band Cholesky factor of equdecs /
 * equslvs with no Lagrange multipliers (mbandw > 0, mpnum.f90:2486-2678:
 * lltdec 2155-2209, lltfwd 2222-2240, lltbwd 2300-2318).
 * ---------------------------------------------------------------- */
typedef struct {
    int32_t kind;          /* -1 none, 0 diagonal, 1 band */
    int32_t n;
    const double *pc;      /* kind 0: cu */
    const double *c;       /* kind 1: factor in the variable-band layout */
    const int64_t *india;  /* kind 1: position of each row's diagonal (1-based) */
} precond;

/* indPreCond (pede.f90:7705-7717): rows 1..mbandw triangular, then a
 * fixed width of mbandw; india[i-1] = 1-based position of c(i,i). */
void mpref_band_index(int32_t n, int32_t mbandw, int64_t *india)
{
    int32_t i;
    for (i = 1; i <= n; i++)
        india[i - 1] = i <= mbandw ? (int64_t)i * (i + 1) / 2 : india[i - 2] + mbandw;
}

/* lltdec (mpnum.f90:2155-2209): c = L L^T of the variable band in place,
 * the diagonal replaced by 1/sqrt; a row whose reduced diagonal is not
 * above 16 eps times its original is reset (iopt > 0: diagonal from the
 * original value, "skyline").  Returns nrkd as lltdec. */
int32_t mpref_lltdec(int32_t n, double *c, const int64_t *india, int32_t iopt)
{
    const double eps = 16.0 * DBL_EPSILON;
    int32_t nrkd = 0, i, j, k;
    double diag = 0.0;
    if (n <= 0) return 0;
#define C_(q) c[(q) - 1]
#define IN_(q) india[(q) - 1]
    if (C_(IN_(1)) > 0.0) {
        C_(IN_(1)) = 1.0 / sqrt(C_(IN_(1)));
    } else {
        C_(IN_(1)) = 0.0;
        nrkd = -1;
    }
    for (k = 2; k <= n; k++) {
        const int32_t mk = (int32_t)(k - IN_(k) + IN_(k - 1) + 1);
        for (j = mk; j <= k; j++) {
            int32_t mj = 1;
            if (j > 1) mj = (int32_t)(j - IN_(j) + IN_(j - 1) + 1);
            const int64_t kj = IN_(k) - k + j;
            diag = C_(IN_(j));
            for (i = (mj > mk ? mj : mk); i <= j - 1; i++) {
                const double prod = C_(IN_(k) - k + i) * C_(IN_(j) - j + i);
                C_(kj) = C_(kj) - prod;
            }
            if (j != k) C_(kj) = C_(kj) * diag;
        }
        if (C_(IN_(k)) > eps * diag) {
            C_(IN_(k)) = 1.0 / sqrt(C_(IN_(k)));
        } else {
            for (j = mk; j <= k; j++) C_(IN_(k) - k + j) = 0.0;
            if (iopt > 0 && diag > 0.0) {
                C_(IN_(k)) = 1.0 / sqrt(diag);
            } else {
                if (nrkd == 0) {
                    nrkd = -k;
                } else {
                    if (nrkd < 0) nrkd = 1;
                    nrkd = nrkd + 1;
                }
            }
        }
    }
    return nrkd;
}

/* lltfwd + lltbwd (mpnum.f90:2222-2240, 2300-2318): x := (L L^T)^-1 x */
void mpref_lltslv(int32_t n, const double *c, const int64_t *india, double *x)
{
    int32_t j, k;
    if (n <= 0) return;
    x[0] = x[0] * C_(IN_(1));
    for (k = 2; k <= n; k++) {
        for (j = (int32_t)(k - IN_(k) + IN_(k - 1) + 1); j <= k - 1; j++) {
            const double prod = C_(IN_(k) - k + j) * x[j - 1];
            x[k - 1] = x[k - 1] - prod;
        }
        x[k - 1] = x[k - 1] * C_(IN_(k));
    }
    for (k = n; k >= 2; k--) {
        x[k - 1] = x[k - 1] * C_(IN_(k));
        for (j = (int32_t)(k - IN_(k) + IN_(k - 1) + 1); j <= k - 1; j++) {
            const double prod = C_(IN_(k) - k + j) * x[k - 1];
            x[j - 1] = x[j - 1] - prod;
        }
    }
    x[0] = x[0] * C_(IN_(1));
#undef C_
#undef IN_
}

static void msolve(const precond *P, const double *r, double *y)
{
    int32_t i, n = P->n;
    if (P->kind < 0) {
        for (i = 0; i < n; i++) y[i] = r[i];
    } else if (P->kind == 0) {
        for (i = 0; i < n; i++) y[i] = (r[i] * P->pc[i]) * P->pc[i];
    } else {
        for (i = 0; i < n; i++) y[i] = r[i];
        mpref_lltslv(n, P->c, P->india, y);
    }
}

/* reduced operator for MINRES: b = (Q^T A Q x)(1:nfit) (avprod) */
typedef struct {
    int32_t matsto, nVar, nG, nfit;
    const int32_t *aig;
    const int64_t *off;
    const int32_t *col;
    const double *matD;
    const mpref_ql *q;
    double *xa, *ba;
} redop;

static void avprod(const redop *o, const double *x, double *b)
{
    int32_t n = o->nfit, i;
    for (i = 0; i < n; i++) o->xa[i] = x[i];
    for (i = n; i < o->nVar; i++) o->xa[i] = 0.0;
    if (o->q) mpref_ql_mlq(o->q, o->xa, 0);
    mpref_avprd0(o->matsto, o->nVar, o->xa, o->ba, o->nG, o->aig, o->off, o->col, o->matD);
    if (o->q) mpref_ql_mlq(o->q, o->ba, 1);
    for (i = 0; i < n; i++) b[i] = o->ba[i];
}

static int g_qlpssq_literal;
static void qlpssq_literal(const redop *o, int32_t mbandw, const int64_t *india, double *c);
static double dotn(const double *a, const double *b, int32_t n)
{
    double s = 0.0;
    for (int32_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* diag(Q^T A Q) by explicit reflection tracking (see qlpssq,
 * mpqldec.f90:711-950, band width 1) */
static void reduced_diag(const redop *o, double *dg)
{
    int32_t nV = o->nVar, i;
    for (i = 0; i < nV; i++) dg[i] = 0.0;
    /* start from diag(A) */
    for (i = 1; i <= nV; i++) {
        if (o->matsto == 2) dg[i - 1] = o->matD[i - 1];
        else dg[i - 1] = o->matD[((int64_t)i * i - i) / 2 + i - 1];
    }
    if (!o->q) return;
    if (g_qlpssq_literal) {  /* qlpssq with band width 1 (pede.f90:8295) */
        int64_t *ind = (int64_t *)calloc((size_t)nV, sizeof(int64_t));
        for (i = 0; i < nV; i++) ind[i] = i + 1;
        qlpssq_literal(o, 1, ind, dg);
        free(ind);
        return;
    }
    const mpref_ql *q = o->q;
    int32_t m = q->ncon;
    double *v = (double *)calloc((size_t)nV, sizeof(double));
    double *y = (double *)calloc((size_t)nV, sizeof(double));
    double *tmp = (double *)calloc((size_t)nV, sizeof(double));
    /* transforms applied in the order k = m, m-1, ..., 1 (qlssq t=true) */
    for (int32_t k = m; k >= 1; k--) {
        int32_t kn = nV + k - m;
        const double *vr = q->V + (int64_t)(k - 1) * nV;
        for (i = 0; i < nV; i++) v[i] = 0.0;
        for (i = q->r1[k]; i <= q->r2[k]; i++) v[i - 1] = vr[1 + i - q->r1[k]];
        v[kn - 1] = q->Vk[k];
        /* P v with P = H_m ... H_{k+1}: apply H_{k+1} first */
        for (i = 0; i < nV; i++) tmp[i] = v[i];
        for (int32_t kk = k + 1; kk <= m; kk++) {
            int32_t knn = nV + kk - m;
            const double *wr = q->V + (int64_t)(kk - 1) * nV;
            double sp = 0.0;
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) sp += wr[1 + i - q->r1[kk]] * tmp[i - 1];
            sp += q->Vk[kk] * tmp[knn - 1];
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) tmp[i - 1] -= 2.0 * wr[1 + i - q->r1[kk]] * sp;
            tmp[knn - 1] -= 2.0 * q->Vk[kk] * sp;
        }
        mpref_avprd0(o->matsto, nV, tmp, y, o->nG, o->aig, o->off, o->col, o->matD);
        for (int32_t kk = m; kk >= k + 1; kk--) {
            int32_t knn = nV + kk - m;
            const double *wr = q->V + (int64_t)(kk - 1) * nV;
            double sp = 0.0;
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) sp += wr[1 + i - q->r1[kk]] * y[i - 1];
            sp += q->Vk[kk] * y[knn - 1];
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) y[i - 1] -= 2.0 * wr[1 + i - q->r1[kk]] * sp;
            y[knn - 1] -= 2.0 * q->Vk[kk] * sp;
        }
        double beta = 0.0;
        for (i = 0; i < nV; i++) beta += v[i] * y[i];
        for (i = 0; i < nV; i++) dg[i] = dg[i] - 4.0 * v[i] * y[i] + 4.0 * beta * v[i] * v[i];
    }
    free(v); free(y); free(tmp);
}

/* Band of Q^T A Q over all nVar rows in the variable-band layout (the
 * preconditioner fill of pede.f90:2639-2651 followed by qlpssq with band
 * width mbandw, mpqldec.f90:711-945).  The reference tracks the products
 * of the reflections through coefficient tables; here each reflection
 * k = m..1 is applied explicitly: with P = H_m ... H_{k+1}, y = P^T A P v
 * and beta = v.y, H A' H changes element (i,j) by
 * -2 (v_i y_j + y_i v_j) + 4 beta v_i v_j.  Same matrix up to rounding. */
static void reduced_band(const redop *o, int32_t mbandw, const int64_t *india, double *c)
{
    int32_t nV = o->nVar, i, j;
    int32_t *p2g = NULL;
    if (o->matsto == 2) {
        p2g = (int32_t *)calloc((size_t)(nV > 0 ? nV : 1), sizeof(int32_t));
        for (int32_t g = 1; g <= o->nG; g++)
            for (int32_t q = o->aig[g - 1]; q < o->aig[g]; q++) p2g[q - 1] = g;
    }
    for (i = 1; i <= nV; i++) {
        const int64_t ia = india[i - 1];
        for (j = (i - mbandw + 1 > 1 ? i - mbandw + 1 : 1); j <= i; j++) {
            double a = 0.0;
            if (o->matsto == 2) {
                const int64_t ij = mpref_ijadd(i, j, o->nG, o->aig, p2g, o->off, o->col);
                if (ij > 0) a = o->matD[ij - 1];
            } else {
                a = o->matD[((int64_t)i * i - i) / 2 + j - 1];
            }
            c[ia - i + j - 1] = a;
        }
    }
    free(p2g);
    if (!o->q) return;
    if (g_qlpssq_literal) {
        qlpssq_literal(o, mbandw, india, c);
        return;
    }
    const mpref_ql *q = o->q;
    int32_t m = q->ncon;
    double *v = (double *)calloc((size_t)nV, sizeof(double));
    double *y = (double *)calloc((size_t)nV, sizeof(double));
    double *tmp = (double *)calloc((size_t)nV, sizeof(double));
    for (int32_t k = m; k >= 1; k--) {
        int32_t kn = nV + k - m;
        const double *vr = q->V + (int64_t)(k - 1) * nV;
        for (i = 0; i < nV; i++) v[i] = 0.0;
        for (i = q->r1[k]; i <= q->r2[k]; i++) v[i - 1] = vr[1 + i - q->r1[k]];
        v[kn - 1] = q->Vk[k];
        for (i = 0; i < nV; i++) tmp[i] = v[i];
        for (int32_t kk = k + 1; kk <= m; kk++) {
            int32_t knn = nV + kk - m;
            const double *wr = q->V + (int64_t)(kk - 1) * nV;
            double sp = 0.0;
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) sp += wr[1 + i - q->r1[kk]] * tmp[i - 1];
            sp += q->Vk[kk] * tmp[knn - 1];
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) tmp[i - 1] -= 2.0 * wr[1 + i - q->r1[kk]] * sp;
            tmp[knn - 1] -= 2.0 * q->Vk[kk] * sp;
        }
        mpref_avprd0(o->matsto, nV, tmp, y, o->nG, o->aig, o->off, o->col, o->matD);
        for (int32_t kk = m; kk >= k + 1; kk--) {
            int32_t knn = nV + kk - m;
            const double *wr = q->V + (int64_t)(kk - 1) * nV;
            double sp = 0.0;
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) sp += wr[1 + i - q->r1[kk]] * y[i - 1];
            sp += q->Vk[kk] * y[knn - 1];
            for (i = q->r1[kk]; i <= q->r2[kk]; i++) y[i - 1] -= 2.0 * wr[1 + i - q->r1[kk]] * sp;
            y[knn - 1] -= 2.0 * q->Vk[kk] * sp;
        }
        double beta = 0.0;
        for (i = 0; i < nV; i++) beta += v[i] * y[i];
        for (i = 1; i <= nV; i++) {
            const int64_t ia = india[i - 1];
            for (j = (i - mbandw + 1 > 1 ? i - mbandw + 1 : 1); j <= i; j++) {
                const double vi = v[i - 1], vj = v[j - 1];
                if (vi == 0.0 && vj == 0.0) continue;
                c[ia - i + j - 1] += -2.0 * (vi * y[j - 1] + y[i - 1] * vj) + 4.0 * beta * (vi * vj);
            }
        }
    }
    free(v); free(y); free(tmp);
}

/* qlpssq (mpqldec.f90:711-945, t = .true.) literally: the band of width
 * mbandw (variable-band layout india, all nVar rows) updated for the
 * reflections through products of the untransformed matrix (first pass)
 * and tables of the vectors' mutual products and coefficients (second
 * pass), as the reference forms the preconditioner of the reduced system.
 * Used when mpref_set_qlpssq_literal(1) is in force. */
static int g_qlpssq_literal = 0;
void mpref_set_qlpssq_literal(int32_t on) { g_qlpssq_literal = on; }

static void qlpssq_literal(const redop *o, int32_t mbandw, const int64_t *india, double *c)
{
    const mpref_ql *q = o->q;
    const int32_t npar = o->nVar, ncon = q->ncon, mbnd = mbandw - 1 > 0 ? mbandw - 1 : 0;
    const double eps16 = 16.0 * DBL_EPSILON;
    double *vtvp = (double *)calloc((size_t)ncon * ncon, sizeof(double));
    double *vtAvp = (double *)calloc((size_t)ncon * ncon, sizeof(double));
    double *coef = (double *)calloc((size_t)ncon * ncon, sizeof(double));
    int32_t *rlo = (int32_t *)calloc((size_t)ncon + 1, sizeof(int32_t));
    int32_t *rhi = (int32_t *)calloc((size_t)ncon + 1, sizeof(int32_t));
    double *vN = (double *)calloc((size_t)npar, sizeof(double));
    double *v2 = (double *)calloc((size_t)npar, sizeof(double));
    double *vAv = (double *)calloc((size_t)npar, sizeof(double));
    int32_t i, l, j, j2;
#define V_(k, vec) do { int32_t ii_; for (ii_ = 0; ii_ < npar; ii_++) (vec)[ii_] = 0.0; \
        for (ii_ = q->r1[k]; ii_ <= q->r2[k]; ii_++) (vec)[ii_ - 1] = q->V[(int64_t)((k) - 1) * npar + 1 + ii_ - q->r1[k]]; \
        (vec)[npar + (k) - ncon - 1] = q->Vk[k]; } while (0)
    /* the band update of mpqldec.f90:838-854 (and 883-898) */
#define BAND_(vtAv, kn) do { int64_t q_ = 0; \
        for (i = 1; i <= npar; i++) { const int64_t ia_ = india[i - 1]; \
            for (l = (i - mbnd > 1 ? i - mbnd : 1); l <= i; l++) { q_ = ia_ - i + l - 1; \
                if (i <= (kn)) c[q_] += 2.0 * ((2.0 * vN[i - 1] * (vtAv) - vAv[i - 1]) * vN[l - 1] - vAv[l - 1] * vN[i - 1]); \
                else c[q_] -= 2.0 * vAv[i - 1] * vN[l - 1]; } } } while (0)
    for (j = 1; j <= ncon; j++) {
        const int32_t k = ncon + 1 - j, kn = npar + k - ncon;
        rlo[k] = ncon;
        rhi[k] = 1;
        V_(k, vN);
        mpref_avprd0(o->matsto, npar, vN, vAv, o->nG, o->aig, o->off, o->col, o->matD);
        for (j2 = j + 1; j2 <= ncon; j2++) {
            const int32_t k2 = ncon + 1 - j2;
            V_(k2, v2);
            const double x = dotn(vN, v2, npar);
            if (fabs(x) > eps16) {
                vtvp[(int64_t)(k - 1) * ncon + k2 - 1] = x;
                vtvp[(int64_t)(k2 - 1) * ncon + k - 1] = x;
            }
        }
        vtvp[(int64_t)(k - 1) * ncon + k - 1] = 1.0;
        for (j2 = 1; j2 <= j; j2++) {
            const int32_t k2 = ncon + 1 - j2;
            V_(k2, v2);
            vtAvp[(int64_t)(k - 1) * ncon + k2 - 1] = dotn(v2, vAv, npar);
        }
        BAND_(vtAvp[(int64_t)(k - 1) * ncon + k - 1], kn);
    }
    for (j = 1; j <= ncon; j++) {
        const int32_t k = ncon + 1 - j, kn = npar + k - ncon;
        const double *ck = coef + (int64_t)(k - 1) * ncon, *vk = vtvp + (int64_t)(k - 1) * ncon;
        int32_t l1 = rlo[k], l2 = rhi[k], k2;
        double vtAv = vtAvp[(int64_t)(k - 1) * ncon + k - 1];
        for (k2 = l1; k2 <= l2; k2++) vtAv += ck[k2 - 1] * vk[k2 - 1];
        V_(k, vN);
        for (i = 0; i < npar; i++) vAv[i] = 0.0;
        for (k2 = l1; k2 <= l2; k2++) {
            if (ck[k2 - 1] == 0.0) continue;
            V_(k2, v2);
            for (i = 0; i < npar; i++) vAv[i] += ck[k2 - 1] * v2[i];
        }
        BAND_(vtAv, kn);
        for (j2 = j + 1; j2 <= ncon; j2++) {
            const int32_t kk2 = ncon + 1 - j2;
            double *c2 = coef + (int64_t)(kk2 - 1) * ncon;
            const double x = vk[kk2 - 1];
            int32_t m1 = rlo[kk2], m2 = rhi[kk2], q2;
            double va = vtAvp[(int64_t)(kk2 - 1) * ncon + k - 1];
            for (q2 = m1; q2 <= m2; q2++) va += c2[q2 - 1] * vk[q2 - 1];
            if (k < m1) m1 = k;
            if (k > m2) m2 = k;
            c2[k - 1] += 2.0 * (2.0 * vtAv * x - va);
            if (x != 0.0) {
                if (rlo[k] < m1) m1 = rlo[k];
                if (rhi[k] > m2) m2 = rhi[k];
                for (q2 = m1; q2 <= m2; q2++) c2[q2 - 1] -= 2.0 * ck[q2 - 1] * x;
            }
            rlo[kk2] = m1;
            rhi[kk2] = m2;
        }
    }
#undef V_
#undef BAND_
    free(vtvp); free(vtAvp); free(coef); free(rlo); free(rhi); free(vN); free(v2); free(vAv);
}

/* Preconditioned MINRES, Paige & Saunders (1975), SIAM J. Numer. Anal. 12,
 * 617-629: Lanczos tridiagonalisation of the preconditioned operator,
 * QR of the tridiagonal by Givens rotations, solution update along the
 * rotated directions.  Stopping: relative residual rnorm/(Anorm*ynorm) <=
 * rtol (istop 1), Arnorm/Anorm <= rtol (istop 2), itn >= itnlim (istop 6). */
static int32_t minres(const redop *o, const precond *pc, const double *b, double *x,
                      double rtol, int32_t itnlim, int32_t *itnout)
{
    int32_t n = o->nfit, i, itn = 0, istop = 0;
    double *r1 = calloc((size_t)n, sizeof(double)), *r2 = calloc((size_t)n, sizeof(double));
    double *y = calloc((size_t)n, sizeof(double)), *v = calloc((size_t)n, sizeof(double));
    double *w = calloc((size_t)n, sizeof(double)), *w1 = calloc((size_t)n, sizeof(double));
    double *w2 = calloc((size_t)n, sizeof(double));
    const double eps = DBL_EPSILON;
    double beta1, beta, oldb, alfa, dbar = 0, epsln = 0, oldeps, delta, gbar, root;
    double gamma, cs = -1, sn = 0, phi, phibar, denom, tnorm2 = 0, gmax = 0, gmin = DBL_MAX;
    double Anorm = 0, ynorm, rnorm, test1, test2, Acond;
    for (i = 0; i < n; i++) { x[i] = 0.0; r1[i] = b[i]; }
    msolve(pc, r1, y);
    beta1 = 0.0;
    for (i = 0; i < n; i++) beta1 += r1[i] * y[i];
    if (beta1 <= 0.0) { *itnout = 0; istop = beta1 < 0.0 ? 9 : 0; goto out; }
    beta1 = sqrt(beta1);
    beta = beta1;
    oldb = 0.0;
    phibar = beta1;
    for (i = 0; i < n; i++) r2[i] = r1[i];
    while (itn < itnlim) {
        itn++;
        double s = 1.0 / beta;
        for (i = 0; i < n; i++) v[i] = s * y[i];
        avprod(o, v, y);
        if (itn >= 2)
            for (i = 0; i < n; i++) y[i] = y[i] - (beta / oldb) * r1[i];
        alfa = 0.0;
        for (i = 0; i < n; i++) alfa += v[i] * y[i];
        for (i = 0; i < n; i++) y[i] = y[i] - (alfa / beta) * r2[i];
        for (i = 0; i < n; i++) { r1[i] = r2[i]; r2[i] = y[i]; }
        msolve(pc, r2, y);
        oldb = beta;
        beta = 0.0;
        for (i = 0; i < n; i++) beta += r2[i] * y[i];
        if (beta < 0.0) { istop = 9; break; }
        beta = sqrt(beta);
        tnorm2 += alfa * alfa + oldb * oldb + beta * beta;
        oldeps = epsln;
        delta = cs * dbar + sn * alfa;
        gbar = sn * dbar - cs * alfa;
        epsln = sn * beta;
        dbar = -cs * beta;
        root = sqrt(gbar * gbar + dbar * dbar);
        gamma = sqrt(gbar * gbar + beta * beta);
        if (gamma < eps) gamma = eps;
        cs = gbar / gamma;
        sn = beta / gamma;
        phi = cs * phibar;
        phibar = sn * phibar;
        denom = 1.0 / gamma;
        for (i = 0; i < n; i++) {
            w1[i] = w2[i];
            w2[i] = w[i];
            w[i] = (v[i] - oldeps * w1[i] - delta * w2[i]) * denom;
            x[i] = x[i] + phi * w[i];
        }
        if (gamma > gmax) gmax = gamma;
        if (gamma < gmin) gmin = gamma;
        Anorm = sqrt(tnorm2);
        ynorm = 0.0;
        for (i = 0; i < n; i++) ynorm += x[i] * x[i];
        ynorm = sqrt(ynorm);
        rnorm = phibar;
        test1 = rnorm / (Anorm * ynorm);
        test2 = root / Anorm;
        Acond = gmax / gmin;
        if (itn >= itnlim) istop = 6;
        if (Acond >= 0.1 / eps) istop = 4;
        if (test2 <= rtol) istop = 2;
        if (test1 <= rtol) istop = 1;
        if (istop) break;
    }
    *itnout = itn;
out:
    free(r1); free(r2); free(y); free(v); free(w); free(w1); free(w2);
    return istop;
}

/* MINRES-QLP (Choi, Paige & Saunders, SIAM J. Sci. Comput. 33 (2011)
 * 1810-1836; the reference vendors it as minresqlpModule.f90:411-1333),
 * restated from the method: the preconditioned Lanczos process and the left
 * reflections of MINRES give the upper-triangular R_k (column k: eps_k in
 * row k-2, delta_k in row k-1, gamma_k in row k) and the right-hand side
 * tau_k; two right reflections per iteration (columns k-2,k then k-1,k) turn
 * R_k into the lower-triangular L_k = R_k P_k (diagonal g, sub-diagonals
 * theta and eta).  With L u = tau and W = V P, x_k = W u: the first k-2
 * components of u and columns of W are final and accumulate in xp, the
 * last two are recomputed each iteration.  A diagonal of L at the rounding
 * level of |T| gives a zero component, which leaves the minimum-length
 * solution of a singular system.  An iterate longer than maxxnorm is not
 * taken (x keeps the previous one).  QLP steps are taken from the first
 * iteration (the reference's mode 2; in exact arithmetic the iterates equal
 * those of MINRES where the system is nonsingular).  istop: 1 residual
 * test, 2 least-squares test, 4 condition limit, 5 |x| above maxxnorm,
 * 6 iteration limit, 9 indefinite preconditioner. */
static void sym_ortho(double a, double b, double *c, double *s, double *r)
{
    *r = sqrt(a * a + b * b);
    if (*r == 0.0) { *c = 1.0; *s = 0.0; return; }
    *c = a / *r;
    *s = b / *r;
}

static int32_t minresqlp(const redop *o, const precond *pc, const double *b, double *x,
                         double rtol, int32_t itnlim, double maxxnorm, int32_t *itnout)
{
    int32_t n = o->nfit, i, itn = 0, istop = 0;
    double *r1 = calloc((size_t)n, sizeof(double)), *r2 = calloc((size_t)n, sizeof(double));
    double *y = calloc((size_t)n, sizeof(double)), *v = calloc((size_t)n, sizeof(double));
    double *wa = calloc((size_t)n, sizeof(double)), *wb = calloc((size_t)n, sizeof(double));
    double *xp = calloc((size_t)n, sizeof(double)), *xc = calloc((size_t)n, sizeof(double));
    const double eps = DBL_EPSILON;
    double beta1, beta, oldb, alfa, dbar = 0, epsln = 0, epsk, delta, gbar, root;
    double gamma, cs = -1, sn = 0, tau, phibar, tnorm2 = 0, gmax = 0, gmin = DBL_MAX;
    double Anorm = 0, xnorm, test1, test2, Acond;
    /* rows k-2 (A) and k-1 (B) of L: eta, theta, diagonal, tau */
    double etaA = 0, thA = 0, gA = 0, tauA = 0, etaB = 0, thB = 0, gB = 0, tauB = 0;
    double uF1 = 0, uF2 = 0;   /* final u_{k-3}, u_{k-4} */
    for (i = 0; i < n; i++) { x[i] = 0.0; r1[i] = b[i]; }
    msolve(pc, r1, y);
    beta1 = 0.0;
    for (i = 0; i < n; i++) beta1 += r1[i] * y[i];
    if (beta1 <= 0.0) { *itnout = 0; istop = beta1 < 0.0 ? 9 : 0; goto out; }
    beta1 = sqrt(beta1);
    beta = beta1;
    oldb = 0.0;
    phibar = beta1;
    for (i = 0; i < n; i++) r2[i] = r1[i];
    while (itn < itnlim) {
        itn++;
        /* Lanczos step (as MINRES) */
        double s = 1.0 / beta;
        for (i = 0; i < n; i++) v[i] = s * y[i];
        avprod(o, v, y);
        if (itn >= 2)
            for (i = 0; i < n; i++) y[i] = y[i] - (beta / oldb) * r1[i];
        alfa = 0.0;
        for (i = 0; i < n; i++) alfa += v[i] * y[i];
        for (i = 0; i < n; i++) y[i] = y[i] - (alfa / beta) * r2[i];
        for (i = 0; i < n; i++) { r1[i] = r2[i]; r2[i] = y[i]; }
        msolve(pc, r2, y);
        oldb = beta;
        beta = 0.0;
        for (i = 0; i < n; i++) beta += r2[i] * y[i];
        if (beta < 0.0) { istop = 9; break; }
        beta = sqrt(beta);
        tnorm2 += alfa * alfa + oldb * oldb + beta * beta;
        Anorm = sqrt(tnorm2);
        /* left reflection: column k of R and tau_k */
        epsk = epsln;
        delta = cs * dbar + sn * alfa;
        gbar = sn * dbar - cs * alfa;
        epsln = sn * beta;
        dbar = -cs * beta;
        root = sqrt(gbar * gbar + dbar * dbar);
        sym_ortho(gbar, beta, &cs, &sn, &gamma);
        tau = cs * phibar;
        phibar = sn * phibar;
        if (gamma > gmax) gmax = gamma;
        if (gamma < gmin) gmin = gamma;
        /* right reflections: P(k-2,k) zeroes eps_k in row k-2, P(k-1,k)
         * the updated delta in row k-1; row k gets eta, theta, g */
        double c1 = 1, s1 = 0, c2 = 1, s2 = 0, etaC = 0, thC = 0, gC, dk = delta, gk = gamma;
        if (itn >= 3) {
            double r;
            sym_ortho(gA, epsk, &c1, &s1, &r);
            gA = r;
            const double th = c1 * thB + s1 * dk;
            dk = s1 * thB - c1 * dk;
            thB = th;
            etaC = s1 * gk;
            gk = -c1 * gk;
        }
        if (itn >= 2) {
            double r;
            sym_ortho(gB, dk, &c2, &s2, &r);
            gB = r;
            thC = s2 * gk;
            gC = -c2 * gk;
        } else {
            gC = gk;
        }
        /* u: row k-2 final, rows k-1 and k provisional */
        const double tiny = eps * Anorm;
        double uA = 0, uB, uC;
        if (itn >= 3) {
            uA = fabs(gA) > tiny ? (tauA - etaA * uF2 - thA * uF1) / gA : 0.0;
        }
        if (itn >= 2) uB = fabs(gB) > tiny ? (tauB - etaB * uF1 - thB * uA) / gB : 0.0;
        else uB = 0.0;
        uC = fabs(gC) > tiny ? (tau - etaC * uA - thC * uB) / gC : 0.0;
        /* W = V P: w_{k-2} final (into xp), w_{k-1}, w_k provisional */
        for (i = 0; i < n; i++) {
            double a = wa[i], bb = wb[i], c = v[i];
            if (itn >= 3) {
                const double a2 = c1 * a + s1 * c;
                c = s1 * a - c1 * c;
                a = a2;
                xp[i] = xp[i] + uA * a;
            }
            if (itn >= 2) {
                const double b2 = c2 * bb + s2 * c;
                c = s2 * bb - c2 * c;
                bb = b2;
            }
            wa[i] = bb;
            wb[i] = c;
            xc[i] = xp[i] + uB * bb + uC * c;
        }
        /* shift the rows: B becomes A, row k becomes B */
        if (itn >= 3) { uF2 = uF1; uF1 = uA; }
        etaA = etaB; thA = thB; gA = gB; tauA = tauB;
        etaB = etaC; thB = thC; gB = gC; tauB = tau;
        xnorm = 0.0;
        for (i = 0; i < n; i++) xnorm += xc[i] * xc[i];
        xnorm = sqrt(xnorm);
        /* an iterate longer than maxxnorm is not taken: x keeps the last one */
        if (xnorm > maxxnorm) { istop = 5; break; }
        for (i = 0; i < n; i++) x[i] = xc[i];
        test1 = phibar / (Anorm * xnorm);
        test2 = root / Anorm;
        Acond = gmax / gmin;
        if (itn >= itnlim) istop = 6;
        if (Acond >= 0.1 / eps) istop = 4;
        if (test2 <= rtol) istop = 2;
        if (test1 <= rtol) istop = 1;
        if (istop) break;
    }
    *itnout = itn;
out:
    free(r1); free(r2); free(y); free(v); free(wa); free(wb); free(xp); free(xc);
    return istop;
}

static void redop_init(redop *o, int32_t matsto, int32_t nVar, int32_t nG, const int32_t *aig,
                       const int64_t *offsets, const int32_t *columns, const double *matD, const mpref_ql *q)
{
    int32_t ncon = q ? q->ncon : 0;
    o->matsto = matsto; o->nVar = nVar; o->nG = nG; o->nfit = nVar - ncon;
    o->aig = aig; o->off = offsets; o->col = columns; o->matD = matD; o->q = q;
    o->xa = (double *)calloc((size_t)(nVar > 0 ? nVar : 1), sizeof(double));
    o->ba = (double *)calloc((size_t)(nVar > 0 ? nVar : 1), sizeof(double));
}

int32_t mpref_band_precond(int32_t matsto, int32_t nVar, int32_t nG, const int32_t *allIndexGroups,
                           const int64_t *offsets, const int32_t *columns, const double *matD,
                           const mpref_ql *q, int32_t mbandw, int32_t lprecm, double *c, int32_t *nrkd)
{
    redop o;
    if (mbandw <= 0) return -1;
    redop_init(&o, matsto, nVar, nG, allIndexGroups, offsets, columns, matD, q);
    int64_t *india = (int64_t *)calloc((size_t)(nVar > 0 ? nVar : 1), sizeof(int64_t));
    mpref_band_index(nVar, mbandw, india);
    double *cf = (double *)calloc((size_t)(nVar > 0 ? india[nVar - 1] : 1), sizeof(double));
    reduced_band(&o, mbandw, india, cf);
    *nrkd = mpref_lltdec(o.nfit, cf, india, lprecm);
    if (o.nfit > 0) memcpy(c, cf, sizeof(double) * (size_t)india[o.nfit - 1]);
    free(cf); free(india); free(o.xa); free(o.ba);
    return 0;
}

int32_t mpref_minres_precond(int32_t qlp, int32_t matsto, int32_t nVar, int32_t nG,
                             const int32_t *allIndexGroups, const int64_t *offsets,
                             const int32_t *columns, const double *matD, const mpref_ql *q,
                             const double *rhs, double *x, double rtol, int32_t itnlim,
                             int32_t mbandw, int32_t lprecm, int32_t *itn, int32_t *nrkd)
{
    redop o;
    int32_t i;
    redop_init(&o, matsto, nVar, nG, allIndexGroups, offsets, columns, matD, q);
    precond P;
    P.kind = mbandw < 0 ? -1 : (mbandw == 0 ? 0 : 1);
    P.n = o.nfit;
    P.pc = NULL; P.c = NULL; P.india = NULL;
    double *pc = NULL, *cf = NULL, *dg = NULL;
    int64_t *india = NULL;
    if (nrkd) *nrkd = 0;
    if (P.kind == 0) {
        dg = (double *)calloc((size_t)(nVar > 0 ? nVar : 1), sizeof(double));
        pc = (double *)calloc((size_t)(nVar > 0 ? nVar : 1), sizeof(double));
        reduced_diag(&o, dg);
        for (i = 0; i < o.nfit; i++) pc[i] = dg[i] > 0.0 ? 1.0 / sqrt(dg[i]) : 0.0;
        P.pc = pc;
    } else if (P.kind == 1) {
        india = (int64_t *)calloc((size_t)(nVar > 0 ? nVar : 1), sizeof(int64_t));
        mpref_band_index(nVar, mbandw, india);
        cf = (double *)calloc((size_t)(nVar > 0 ? india[nVar - 1] : 1), sizeof(double));
        reduced_band(&o, mbandw, india, cf);
        const int32_t r = mpref_lltdec(o.nfit, cf, india, lprecm);
        if (nrkd) *nrkd = r;
        P.c = cf; P.india = india;
    }
    int32_t istop;
    if (qlp) {
        /* maxxnorm as pede sets it (pede.f90:626) */
        const double maxxnorm = (double)o.nfit / sqrt(DBL_EPSILON);
        istop = minresqlp(&o, &P, rhs, x, rtol, itnlim, maxxnorm, itn);
    } else {
        istop = minres(&o, &P, rhs, x, rtol, itnlim, itn);
    }
    free(o.xa); free(o.ba); free(dg); free(pc); free(cf); free(india);
    return istop;
}

int32_t mpref_minresqlp_sparse(int32_t matsto, int32_t nVar, int32_t nG,
                               const int32_t *allIndexGroups, const int64_t *offsets,
                               const int32_t *columns, const double *matD,
                               const mpref_ql *q, const double *rhs, double *x,
                               double rtol, int32_t itnlim, int32_t *itn)
{
    return mpref_minres_precond(1, matsto, nVar, nG, allIndexGroups, offsets, columns, matD, q, rhs, x,
                                rtol, itnlim, 0, 0, itn, NULL);
}

int32_t mpref_minres_sparse(int32_t matsto, int32_t nVar, int32_t nG,
                            const int32_t *allIndexGroups, const int64_t *offsets,
                            const int32_t *columns, const double *matD,
                            const mpref_ql *q, const double *rhs, double *x,
                            double rtol, int32_t itnlim, int32_t *itn)
{
    return mpref_minres_precond(0, matsto, nVar, nG, allIndexGroups, offsets, columns, matD, q, rhs, x,
                                rtol, itnlim, 0, 0, itn, NULL);
}
