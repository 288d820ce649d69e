/*
 * mpref_local.c -- oracle: local (per-record) solvers.  TEST INFRASTRUCTURE.
 *
 * Gauss-Jordan inversion with diagonal pivoting, root-free band Cholesky and
 * the bordered-band combination, restated from mpnum.f90 and
 * Dbandmatrix.f90 keeping the reference's operation order.
 * Internal work arrays are 1-based (pointer decremented by one).
 */
#include "mpref.h"
#include <float.h>
#include <math.h>
#include <stdlib.h>

/* sqminv, mpnum.f90:97-213.  v, b are 1-based here. */
static void sqminv1(double *v, double *b, int32_t n, int32_t *nrank, double *diag,
                    int32_t *next)
{
    int32_t i, j, k, l, last, next0, jj, kk, jk, jl, lk;
    double vkk, vjk;
    const double eps = 16.0 * DBL_EPSILON;
    next0 = 1;
    l = 1;
    for (i = 1; i <= n; i++) {
        next[i] = i + 1;
        diag[i] = fabs(v[(i * i + i) / 2]);
    }
    next[n] = -1;
    *nrank = 0;
    for (i = 1; i <= n; i++) {
        k = 0;
        vkk = 0.0;
        j = next0;
        last = 0;
        while (j > 0) {
            jj = (j * j + j) / 2;
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
            kk = (k * k + k) / 2;
            if (l == 0) next0 = next[k];
            else next[l] = next[k];
            next[k] = 0;
            (*nrank)++;
            vkk = 1.0 / vkk;
            v[kk] = -vkk;
            b[k] = b[k] * vkk;
            jk = kk - k;
            jl = 0;
            for (j = 1; j <= n; j++) {
                if (j == k) {
                    jk = kk;
                    jl = jl + j;
                } else {
                    if (j < k) jk = jk + 1;
                    else jk = jk + j - 1;
                    vjk = v[jk];
                    v[jk] = vkk * vjk;
                    b[j] = b[j] - b[k] * vjk;
                    lk = kk - k;
                    for (l = 1; l <= j; l++) {
                        jl = jl + 1;
                        if (l == k) {
                            lk = kk;
                        } else {
                            if (l < k) lk = lk + 1;
                            else lk = lk + l - 1;
                            v[jl] = v[jl] - v[lk] * vjk;
                        }
                    }
                }
            }
        } else {
            for (k = 1; k <= n; k++) {
                if (next[k] != 0) {
                    b[k] = 0.0;
                    for (j = 1; j <= k; j++)
                        if (next[j] != 0) v[(k * k - k) / 2 + j] = 0.0;
                }
            }
            break;
        }
    }
    for (int32_t ij = 1; ij <= (n * n + n) / 2; ij++) v[ij] = -v[ij];
}

void mpref_sqminv(double *v, double *b, int32_t n, int32_t *nrank)
{
    double *diag = (double *)malloc(sizeof(double) * ((size_t)n + 1));
    int32_t *next = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n + 1));
    sqminv1(v - 1, b - 1, n, nrank, diag, next);
    free(diag);
    free(next);
}

/* band matrix w(mp1, n) column-major: W(r,c) = w[(c-1)*mp1 + r] (1-based w) */
#define W(r, c) w[((c) - 1) * mp1 + (r)]

/* dbcdec, Dbandmatrix.f90:459-493 */
static void dbcdec(double *w, int32_t mp1, int32_t n, double *aux)
{
    int32_t i, j, k;
    double rxw;
    for (i = 1; i <= n; i++) aux[i] = 16.0 * W(1, i);
    for (i = 1; i <= n; i++) {
        if (W(1, i) + aux[i] != aux[i]) W(1, i) = 1.0 / W(1, i);
        else W(1, i) = 0.0;
        int32_t mj = (mp1 - 1 < n - i) ? mp1 - 1 : n - i;
        for (j = 1; j <= mj; j++) {
            rxw = W(j + 1, i) * W(1, i);
            for (k = 1; k <= mj + 1 - j; k++) W(k, i + j) = W(k, i + j) - W(k + j, i) * rxw;
            W(j + 1, i) = rxw;
        }
    }
}

/* dbcslv, Dbandmatrix.f90:503-533 (b and x may alias) */
static void dbcslv(const double *w, int32_t mp1, int32_t n, const double *b, double *x)
{
    int32_t i, j;
    double rxw;
    for (i = 1; i <= n; i++) x[i] = b[i];
    for (i = 1; i <= n; i++) {
        int32_t mj = (mp1 - 1 < n - i) ? mp1 - 1 : n - i;
        for (j = 1; j <= mj; j++) x[j + i] = x[j + i] - W(j + 1, i) * x[i];
    }
    for (i = n; i >= 1; i--) {
        rxw = x[i] * W(1, i);
        int32_t mj = (mp1 - 1 < n - i) ? mp1 - 1 : n - i;
        for (j = 1; j <= mj; j++) rxw = rxw - W(j + 1, i) * x[j + i];
        x[i] = rxw;
    }
}

/* dbcinb, Dbandmatrix.f90:576-604 (band part of the inverse) */
static void dbcinb(const double *w, int32_t mp1, int32_t n, double *vs)
{
    int32_t i, j, k;
    double rxw;
    for (i = n; i >= 1; i--) {
        rxw = W(1, i);
        int32_t jlo = (1 > i - mp1 + 1) ? 1 : i - mp1 + 1;
        for (j = i; j >= jlo; j--) {
            int32_t khi = (n < j + mp1 - 1) ? n : j + mp1 - 1;
            for (k = j + 1; k <= khi; k++) {
                int32_t a = i > k ? i : k, c = i > k ? k : i;
                rxw = rxw - vs[(a * (a - 1)) / 2 + c] * W(1 + k - j, j);
            }
            vs[(i * i - i) / 2 + j] = rxw;
            rxw = 0.0;
        }
    }
}

/* dbcinv, Dbandmatrix.f90:613-638 (complete inverse) */
static void dbcinv(const double *w, int32_t mp1, int32_t n, double *vs)
{
    int32_t i, j, k;
    double rxw;
    for (i = n; i >= 1; i--) {
        rxw = W(1, i);
        for (j = i; j >= 1; j--) {
            int32_t khi = (n < j + mp1 - 1) ? n : j + mp1 - 1;
            for (k = j + 1; k <= khi; k++) {
                int32_t a = i > k ? i : k, c = i > k ? k : i;
                rxw = rxw - vs[(a * (a - 1)) / 2 + c] * W(1 + k - j, j);
            }
            vs[(i * i - i) / 2 + j] = rxw;
            rxw = 0.0;
        }
    }
}
#undef W

typedef struct {
    double *vbnd, *vbdr, *aux, *vbk, *vzru, *scdiag;
    int32_t *scflag;
} bbwork;

static int bbwork_alloc(bbwork *wk, int32_t n, int32_t nbdr, int32_t nbnd)
{
    size_t nb = (size_t)nbdr > 0 ? (size_t)nbdr : 1;
    wk->vbnd = (double *)calloc((size_t)n * (size_t)(nbnd + 1) + 2, sizeof(double));
    wk->vbdr = (double *)calloc((size_t)n * nb + 2, sizeof(double));
    wk->aux = (double *)calloc((size_t)n * nb + (size_t)n + 2, sizeof(double));
    wk->vbk = (double *)calloc(nb * (nb + 1) / 2 + 2, sizeof(double));
    wk->vzru = (double *)calloc(nb + 2, sizeof(double));
    wk->scdiag = (double *)calloc(nb + 2, sizeof(double));
    wk->scflag = (int32_t *)calloc(nb + 2, sizeof(int32_t));
    return wk->vbnd && wk->vbdr && wk->aux && wk->vbk && wk->vzru && wk->scdiag && wk->scflag;
}

static void bbwork_free(bbwork *wk)
{
    free(wk->vbnd); free(wk->vbdr); free(wk->aux); free(wk->vbk);
    free(wk->vzru); free(wk->scdiag); free(wk->scflag);
}

/* sqmibb, mpnum.f90:3118-3354 (upper/left border).  v, b 1-based. */
static void sqmibb1(double *v, double *b, int32_t n, int32_t nbdr, int32_t nbnd, int32_t inv,
                    int32_t *nrank, double *evdmin, double *evdmax, bbwork *wk)
{
    double *vbnd = wk->vbnd, *vbdr = wk->vbdr, *aux = wk->aux, *vbk = wk->vbk, *vzru = wk->vzru;
    int32_t i, j, ib, jb, ip, is, ioff, joff, ij, ip1, ip2, j0, nrankb;
    int32_t nb1 = nbdr + 1, mp1 = nbnd + 1, nmb = n - nbdr;
    *nrank = 0;
    for (i = nb1; i <= n; i++) {
        ip = (i * (i + 1)) / 2;
        is = 0;
        int32_t jhi = (n < i + nbnd) ? n : i + nbnd;
        for (j = i; j <= jhi; j++) {
            ip = ip + is;
            is = j;
            ib = j - i + 1;
            vbnd[ib + (i - nb1) * mp1] = v[ip];
        }
    }
    if (nbdr > 0) {
        ioff = 0;
        for (i = 1; i <= nbdr; i++) {
            ip = (i * (i + 1)) / 2;
            is = 0;
            for (j = i; j <= n; j++) {
                ip = ip + is;
                is = j;
                vbdr[ioff + j] = v[ip];
            }
            ioff = ioff + n;
        }
    }
    dbcdec(vbnd, mp1, nmb, aux);
    ip = 1;
    *nrank = 0;
    *evdmin = 0.0;
    *evdmax = 0.0;
    for (i = 1; i <= nmb; i++) {
        if (vbnd[ip] <= 0.0) {
            for (ip = 1; ip <= n; ip++) b[ip] = 0.0;
            for (ip = 1; ip <= (n * n + n) / 2; ip++) v[ip] = 0.0;
            return;
        }
        (*nrank)++;
        if (*nrank == 1) {
            *evdmin = vbnd[ip];
            *evdmax = vbnd[ip];
        } else {
            if (vbnd[ip] < *evdmin) *evdmin = vbnd[ip];
            if (vbnd[ip] > *evdmax) *evdmax = vbnd[ip];
        }
        ip = ip + mp1;
    }
    if (nbdr == 0) {
        dbcslv(vbnd, mp1, nmb, b, b);
        if (inv > 0) {
            if (inv > 1) dbcinv(vbnd, mp1, nmb, v);
            else dbcinb(vbnd, mp1, nmb, v);
        }
        return;
    }
    ioff = nb1;
    for (ib = 1; ib <= nbdr; ib++) {
        dbcslv(vbnd, mp1, nmb, vbdr + ioff - 1, aux + ioff - 1);
        vzru[ib] = b[ib];
        for (i = 0; i <= nmb - 1; i++) vzru[ib] = vzru[ib] - b[nb1 + i] * aux[ioff + i];
        ioff = ioff + n;
    }
    dbcslv(vbnd, mp1, nmb, b + nb1 - 1, b + nb1 - 1);
    ip = 0;
    ioff = nb1;
    for (ib = 1; ib <= nbdr; ib++) {
        joff = nb1;
        for (jb = 1; jb <= ib; jb++) {
            ip = ip + 1;
            vbk[ip] = v[ip];
            for (i = 0; i <= nmb - 1; i++) vbk[ip] = vbk[ip] - vbdr[ioff + i] * aux[joff + i];
            joff = joff + n;
        }
        ioff = ioff + n;
    }
    sqminv1(vbk, vzru, nbdr, &nrankb, wk->scdiag, wk->scflag);
    if (nrankb == nbdr) {
        *nrank = *nrank + nbdr;
    } else {
        for (ib = 1; ib <= nbdr; ib++) vzru[ib] = 0.0;
        for (ip = (nbdr * nbdr + nbdr) / 2; ip >= 1; ip--) vbk[ip] = 0.0;
    }
    ioff = nb1;
    for (ib = 1; ib <= nbdr; ib++) {
        b[ib] = vzru[ib];
        for (i = 0; i <= nmb - 1; i++) b[nb1 + i] = b[nb1 + i] - b[ib] * aux[ioff + i];
        ioff = ioff + n;
    }
    if (inv > 0) {
        if (inv > 1) dbcinv(vbnd, mp1, nmb, v);
        else dbcinb(vbnd, mp1, nmb, v);
        ip1 = (nmb * nmb + nmb) / 2;
        ip2 = (n * n + n) / 2;
        for (i = nmb - 1; i >= 0; i--) {
            j0 = 0;
            if (inv == 1) j0 = (0 > i - nbnd) ? 0 : i - nbnd;
            for (j = i; j >= j0; j--) {
                v[ip2] = v[ip1];
                ioff = nb1;
                for (ib = 1; ib <= nbdr; ib++) {
                    joff = nb1;
                    for (jb = 1; jb <= nbdr; jb++) {
                        ij = ib > jb ? ib : jb;
                        ij = (ij * ij - ij) / 2 + (ib > jb ? jb : ib);
                        v[ip2] = v[ip2] + vbk[ij] * aux[ioff + i] * aux[joff + j];
                        joff = joff + n;
                    }
                    ioff = ioff + n;
                }
                ip1 = ip1 - 1;
                ip2 = ip2 - 1;
            }
            ip1 = ip1 - j0;
            ip2 = ip2 - j0;
            for (ib = nbdr; ib >= 1; ib--) {
                v[ip2] = 0.0;
                joff = nb1;
                for (jb = 1; jb <= nbdr; jb++) {
                    ij = ib > jb ? ib : jb;
                    ij = (ij * ij - ij) / 2 + (ib > jb ? jb : ib);
                    v[ip2] = v[ip2] - vbk[ij] * aux[i + joff];
                    joff = joff + n;
                }
                ip2 = ip2 - 1;
            }
        }
        for (ip = (nbdr * nbdr + nbdr) / 2; ip >= 1; ip--) {
            v[ip2] = vbk[ip];
            ip2 = ip2 - 1;
        }
    }
}

/* sqmibb2, mpnum.f90:3390-3600 (lower/right border).  v, b 1-based. */
static void sqmibb21(double *v, double *b, int32_t n, int32_t nbdr, int32_t nbnd, int32_t inv,
                     int32_t *nrank, double *evdmin, double *evdmax, bbwork *wk)
{
    double *vbnd = wk->vbnd, *vbdr = wk->vbdr, *aux = wk->aux, *vbk = wk->vbk, *vzru = wk->vzru;
    int32_t i, j, ib, jb, ip, is, ioff, joff, koff, ij, ip1, j0, nrankb;
    int32_t mp1 = nbnd + 1, nmb = n - nbdr, nb1 = nmb + 1;
    *nrank = 0;
    for (i = 1; i <= nmb; i++) {
        ip = (i * (i + 1)) / 2;
        is = 0;
        int32_t jhi = (nmb < i + nbnd) ? nmb : i + nbnd;
        for (j = i; j <= jhi; j++) {
            ip = ip + is;
            is = j;
            ib = j - i + 1;
            vbnd[ib + (i - 1) * mp1] = v[ip];
        }
    }
    if (nbdr > 0) {
        ioff = 0;
        for (i = nb1; i <= n; i++) {
            ip = (i * (i - 1)) / 2;
            for (j = 1; j <= i; j++) vbdr[ioff + j] = v[ip + j];
            ioff = ioff + n;
        }
    }
    dbcdec(vbnd, mp1, nmb, aux);
    ip = 1;
    *nrank = 0;
    *evdmin = 0.0;
    *evdmax = 0.0;
    for (i = 1; i <= nmb; i++) {
        if (vbnd[ip] <= 0.0) {
            for (ip = 1; ip <= n; ip++) b[ip] = 0.0;
            for (ip = 1; ip <= (n * n + n) / 2; ip++) v[ip] = 0.0;
            return;
        }
        (*nrank)++;
        if (*nrank == 1) {
            *evdmin = vbnd[ip];
            *evdmax = vbnd[ip];
        } else {
            if (vbnd[ip] < *evdmin) *evdmin = vbnd[ip];
            if (vbnd[ip] > *evdmax) *evdmax = vbnd[ip];
        }
        ip = ip + mp1;
    }
    if (nbdr == 0) {
        dbcslv(vbnd, mp1, nmb, b, b);
        if (inv > 0) {
            if (inv > 1) dbcinv(vbnd, mp1, nmb, v);
            else dbcinb(vbnd, mp1, nmb, v);
        }
        return;
    }
    ioff = 0;
    for (ib = 1; ib <= nbdr; ib++) {
        dbcslv(vbnd, mp1, nmb, vbdr + ioff, aux + ioff);
        vzru[ib] = b[nmb + ib];
        for (i = 1; i <= nmb; i++) vzru[ib] = vzru[ib] - b[i] * aux[ioff + i];
        ioff = ioff + n;
    }
    dbcslv(vbnd, mp1, nmb, b, b);
    ip = 0;
    ioff = 0;
    koff = nmb;
    for (ib = 1; ib <= nbdr; ib++) {
        joff = 0;
        for (jb = 1; jb <= ib; jb++) {
            ip = ip + 1;
            vbk[ip] = vbdr[koff + jb];
            for (i = 1; i <= nmb; i++) vbk[ip] = vbk[ip] - vbdr[ioff + i] * aux[joff + i];
            joff = joff + n;
        }
        ioff = ioff + n;
        koff = koff + n;
    }
    sqminv1(vbk, vzru, nbdr, &nrankb, wk->scdiag, wk->scflag);
    if (nrankb == nbdr) {
        *nrank = *nrank + nbdr;
    } else {
        for (ib = 1; ib <= nbdr; ib++) vzru[ib] = 0.0;
        for (ip = (nbdr * nbdr + nbdr) / 2; ip >= 1; ip--) vbk[ip] = 0.0;
    }
    ioff = 0;
    for (ib = 1; ib <= nbdr; ib++) {
        for (i = 1; i <= nmb; i++) b[i] = b[i] - vzru[ib] * aux[ioff + i];
        ioff = ioff + n;
        b[nmb + ib] = vzru[ib];
    }
    if (inv > 0) {
        if (inv > 1) dbcinv(vbnd, mp1, nmb, v);
        else dbcinb(vbnd, mp1, nmb, v);
        ip1 = (nmb * nmb + nmb) / 2;
        for (i = nmb - 1; i >= 0; i--) {
            j0 = 0;
            if (inv == 1) j0 = (0 > i - nbnd) ? 0 : i - nbnd;
            for (j = i; j >= j0; j--) {
                ioff = 1;
                for (ib = 1; ib <= nbdr; ib++) {
                    joff = 1;
                    for (jb = 1; jb <= nbdr; jb++) {
                        ij = ib > jb ? ib : jb;
                        ij = (ij * ij - ij) / 2 + (ib > jb ? jb : ib);
                        v[ip1] = v[ip1] + vbk[ij] * aux[ioff + i] * aux[joff + j];
                        joff = joff + n;
                    }
                    ioff = ioff + n;
                }
                ip1 = ip1 - 1;
            }
            ip1 = ip1 - j0;
        }
        ip1 = (nmb * nmb + nmb) / 2;
        ip = 0;
        for (ib = 1; ib <= nbdr; ib++) {
            for (i = 1; i <= nmb; i++) {
                ip1 = ip1 + 1;
                v[ip1] = 0.0;
                joff = 0;
                for (jb = 1; jb <= nbdr; jb++) {
                    ij = ib > jb ? ib : jb;
                    ij = (ij * ij - ij) / 2 + (ib > jb ? jb : ib);
                    v[ip1] = v[ip1] - vbk[ij] * aux[i + joff];
                    joff = joff + n;
                }
            }
            for (jb = 1; jb <= ib; jb++) {
                ip1 = ip1 + 1;
                ip = ip + 1;
                v[ip1] = vbk[ip];
            }
        }
    }
}

/* 1-based entry points used by the record loop */
void mpref__sqminv1(double *v1, double *b1, int32_t n, int32_t *nrank, double *diag1,
                    int32_t *next1)
{
    sqminv1(v1, b1, n, nrank, diag1, next1);
}

void mpref__sqmibb_any(int32_t side, double *v1, double *b1, int32_t n, int32_t nbdr,
                       int32_t nbnd, int32_t inv, int32_t *nrank, double *evdmin,
                       double *evdmax)
{
    bbwork wk;
    bbwork_alloc(&wk, n, nbdr, nbnd);
    if (side == 1) sqmibb1(v1, b1, n, nbdr, nbnd, inv, nrank, evdmin, evdmax, &wk);
    else sqmibb21(v1, b1, n, nbdr, nbnd, inv, nrank, evdmin, evdmax, &wk);
    bbwork_free(&wk);
}

void mpref_sqmibb(double *v, double *b, int32_t n, int32_t nbdr, int32_t nbnd,
                  int32_t inv, int32_t *nrank, double *evdmin, double *evdmax)
{
    mpref__sqmibb_any(1, v - 1, b - 1, n, nbdr, nbnd, inv, nrank, evdmin, evdmax);
}

void mpref_sqmibb2(double *v, double *b, int32_t n, int32_t nbdr, int32_t nbnd,
                   int32_t inv, int32_t *nrank, double *evdmin, double *evdmax)
{
    mpref__sqmibb_any(2, v - 1, b - 1, n, nbdr, nbnd, inv, nrank, evdmin, evdmax);
}
