/*
 * mpref_struct.c -- oracle: record decoding, label table, parameter groups,
 * mpbits sparse structure and matrix addressing.  TEST INFRASTRUCTURE ONLY.
 *
 * Internally 1-based work arrays are used (element 0 unused) so the loops
 * read like the reference routines they restate.
 */
#include "mpref.h"
#include <stdlib.h>
#include <string.h>

/* decodeNextMeasurement, pede.f90:2428-2468 (bounded scans added: a zero
 * marker missing before endOfEntry is reported as a bad record). */
int mpref_decode(const int32_t *inder, const double *glder, int64_t endOfEntry,
                 int64_t *lastGlobal, int64_t *startLocal, int64_t *startGlobal,
                 int64_t *startSpecial)
{
    int64_t lg = *lastGlobal;
    *startSpecial = -1;
    for (;;) {
        *startLocal = -1;
        *startGlobal = -1;
        if (lg >= endOfEntry) { *lastGlobal = lg; return 0; }
        do { lg++; if (lg > endOfEntry) return 20; } while (inder[lg] != 0);
        int64_t sl = lg;
        do { lg++; if (lg > endOfEntry) return 20; } while (inder[lg] != 0);
        int64_t sg = lg;
        *startLocal = sl;
        *startGlobal = sg;
        if (sl + 1 == sg && glder[sg] < 0.0) {
            /* special data block: skip NSP words */
            *startSpecial = sg;
            double nsp = -glder[sg];
            lg = lg + (int64_t)(nsp + 0.5);
            continue;
        }
        while (lg < endOfEntry && inder[lg + 1] != 0) lg++;
        *lastGlobal = lg;
        return 0;
    }
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* position (1-based) of label in sorted labels[1..n], 0 if absent */
static int32_t label_index(const int32_t *lab1, int32_t n, int32_t item)
{
    int32_t lo = 1, hi = n;
    if (item <= 0) return 0;
    while (lo <= hi) {
        int32_t mid = (lo + hi) / 2;
        if (lab1[mid] == item) return mid;
        if (lab1[mid] < item) lo = mid + 1; else hi = mid - 1;
    }
    return 0;
}

/* pargrp, pede.f90:2311-2404.  list[1..n] sorted total indices of one
 * equation; gs[] = group start label, lab[] = labels, cnt[] counters. */
static void pargrp(const int32_t *list, int32_t n, int32_t ntot, const int32_t *lab,
                   int32_t *gs, int64_t *cnt)
{
    int32_t j, li, ltgbi, lstart, istart, jstart, jt;
    if (n <= 0) return;
    ltgbi = -1;
    lstart = -1;
    for (j = 1; j <= n; j++) {
        li = list[j];
        cnt[li] += 1;
        istart = gs[li];
        if (istart == 0) {
            if (li != ltgbi + 1) {
                gs[li] = lab[li];
            } else {
                if (lstart == 0) gs[li] = gs[ltgbi];
                else gs[li] = lab[li];
            }
        }
        ltgbi = li;
        lstart = istart;
    }
    li = list[1];
    istart = gs[li];
    jstart = lab[li];
    if (istart != jstart) {
        while (gs[li] == istart) {
            gs[li] = jstart;
            li++;
            if (li > ntot) break;
        }
    }
    ltgbi = list[1];
    for (j = 2; j <= n; j++) {
        li = list[j];
        if (li != ltgbi + 1) {
            lstart = gs[ltgbi];
            jt = ltgbi + 1;
            jstart = lab[jt];
            while (gs[jt] == lstart) {
                gs[jt] = jstart;
                jt++;
                if (jt > ntot) break;
                if (jt == li) jstart = lab[jt];
            }
            jt = li;
            istart = gs[jt];
            jstart = lab[jt];
            if (istart != jstart) {
                while (gs[jt] == istart) {
                    gs[jt] = jstart;
                    jt++;
                    if (jt > ntot) break;
                }
            }
        }
        ltgbi = li;
    }
    li = list[n];
    if (li < ntot) {
        istart = gs[li];
        li++;
        jstart = lab[li];
        while (gs[li] == istart) {
            gs[li] = jstart;
            li++;
            if (li > ntot) break;
        }
    }
}

int mpref_loop1(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                const double *glder, int32_t nsteer, const int32_t *steerLabels,
                int32_t npre, const int32_t *preLabel, const double *preSigma,
                int32_t mreqenf, int32_t cap, int32_t *labels, int64_t *counter,
                int32_t *varIndex, int32_t *grpStart, int32_t *totGroup,
                int32_t *nVar, int32_t *nVarGroups)
{
    int64_t r, nall = 0, k;
    int64_t lastGlobal, startLocal, startGlobal, startSpecial, endOfEntry;
    int32_t *all;
    int32_t ntot, i, j;

    /* phase 1: every label of steering lines and of all global derivatives
     * (indexOfGlobalLabel via prepareRecords(0), mppar.f90:324-357) */
    for (r = 0; r < nrec; r++) nall += recPtr[r + 1] - recPtr[r];
    all = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nall + nsteer + 1));
    if (!all) return -1;
    k = 0;
    for (i = 0; i < nsteer; i++)
        if (steerLabels[i] > 0) all[k++] = steerLabels[i];
    for (r = 0; r < nrec; r++) {
        endOfEntry = recPtr[r + 1] - 1;
        lastGlobal = recPtr[r];
        for (;;) {
            if (mpref_decode(inder, glder, endOfEntry, &lastGlobal, &startLocal,
                             &startGlobal, &startSpecial)) { free(all); return -1; }
            if (startGlobal < 0) break;
            for (int64_t w = startGlobal + 1; w <= lastGlobal; w++)
                if (inder[w] > 0) all[k++] = inder[w];
        }
    }
    qsort(all, (size_t)k, sizeof(int32_t), cmp_i32);
    ntot = 0;
    for (int64_t q = 0; q < k; q++)
        if (ntot == 0 || all[q] != all[ntot - 1]) all[ntot++] = all[q];
    if (ntot > cap) { free(all); return -1; }

    /* 1-based work arrays */
    int32_t *lab = (int32_t *)calloc((size_t)ntot + 2, sizeof(int32_t));
    int32_t *gs = (int32_t *)calloc((size_t)ntot + 2, sizeof(int32_t));
    int64_t *cnt = (int64_t *)calloc((size_t)ntot + 2, sizeof(int64_t));
    int32_t *list = (int32_t *)malloc(sizeof(int32_t) * ((size_t)ntot + 2));
    for (i = 1; i <= ntot; i++) lab[i] = all[i - 1];
    free(all);

    /* phase 2: updateParGroups with mcount=0 (pede.f90:2227-2289): per
     * equation the non-zero-derivative indices, sorted, then pargrp */
    for (r = 0; r < nrec; r++) {
        endOfEntry = recPtr[r + 1] - 1;
        lastGlobal = recPtr[r];
        for (;;) {
            mpref_decode(inder, glder, endOfEntry, &lastGlobal, &startLocal,
                         &startGlobal, &startSpecial);
            if (startGlobal < 0) break;
            if (lastGlobal > startGlobal) {
                int32_t nnz = 0;
                for (int64_t w = startGlobal + 1; w <= lastGlobal; w++) {
                    if (glder[w] == 0.0) continue;
                    list[++nnz] = label_index(lab, ntot, inder[w]);
                }
                if (nnz == 0) continue;
                qsort(list + 1, (size_t)nnz, sizeof(int32_t), cmp_i32);
                pargrp(list, nnz, ntot, lab, gs, cnt);
            }
        }
    }

    /* phase 3: variable parameters (loop1, pede.f90:5938-5956) */
    double *ps = (double *)calloc((size_t)ntot + 2, sizeof(double));
    for (i = 0; i < npre; i++) {
        int32_t li = label_index(lab, ntot, preLabel[i]);
        if (li) ps[li] = preSigma[i];
    }
    int32_t nv = 0;
    for (i = 1; i <= ntot; i++) {
        if (ps[i] < 0.0) varIndex[i - 1] = -1;
        else if (cnt[i] < mreqenf) varIndex[i - 1] = -2;
        else varIndex[i - 1] = ++nv;
    }
    /* groups (pede.f90:5969-5985) */
    int32_t ntg = 0;
    for (j = 1; j <= ntot; j++) {
        totGroup[j - 1] = 0;
        if (gs[j] == 0) continue;
        if (lab[j] == gs[j]) ntg++;
        totGroup[j - 1] = ntg;
    }
    int32_t nvg = 0, lgrp = -1;
    for (j = 1; j <= ntot; j++) {
        if (varIndex[j - 1] <= 0) continue;
        if (totGroup[j - 1] != lgrp) nvg++;
        lgrp = totGroup[j - 1];
    }
    for (i = 1; i <= ntot; i++) {
        labels[i - 1] = lab[i];
        counter[i - 1] = cnt[i];
        grpStart[i - 1] = gs[i];
    }
    *nVar = nv;
    *nVarGroups = nvg;
    free(lab); free(gs); free(cnt); free(list); free(ps);
    return ntot;
}

/* loop2, pede.f90:6509-6530 (icelim>0: no Lagrange groups) */
void mpref_var_groups(int32_t nTotal, const int32_t *varIndex, const int32_t *totGroup,
                      int32_t nVar, int32_t nVarGroups, int32_t *allIndexGroups,
                      int32_t *parToGroup)
{
    int32_t cur = 0, prev = -1, i, j;
    for (i = 0; i < nTotal; i++) {
        int32_t ij = varIndex[i];
        if (ij <= 0) continue;
        if (totGroup[i] != prev) {
            cur++;
            allIndexGroups[cur - 1] = ij;
            prev = totGroup[i];
        }
    }
    allIndexGroups[nVarGroups] = nVar + 1;
    for (i = 1; i <= nVarGroups; i++)
        for (j = allIndexGroups[i - 1]; j < allIndexGroups[i]; j++) parToGroup[j - 1] = i;
}

int mpref_translate(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                    const double *glder, int32_t nTotal, const int32_t *labels,
                    int32_t *outInder)
{
    int64_t r, lastGlobal, startLocal, startGlobal, startSpecial, endOfEntry;
    const int32_t *lab1 = labels - 1;
    for (r = 0; r < nrec; r++)
        for (int64_t w = recPtr[r]; w < recPtr[r + 1]; w++) outInder[w] = inder[w];
    for (r = 0; r < nrec; r++) {
        endOfEntry = recPtr[r + 1] - 1;
        lastGlobal = recPtr[r];
        for (;;) {
            if (mpref_decode(inder, glder, endOfEntry, &lastGlobal, &startLocal,
                             &startGlobal, &startSpecial)) return 20;
            if (startGlobal < 0) break;
            for (int64_t w = startGlobal + 1; w <= lastGlobal; w++)
                outInder[w] = label_index(lab1, nTotal, inder[w]);
        }
    }
    return 0;
}

/* ---------------- mpbits (nspc=1, mextnd=0) ---------------- */
#define BS 32

/* bit m (may pass the end of the word) counted from bit 0 of word l */
static int bit_get(const uint32_t *bits, int64_t l, int32_t m)
{
    return (int)((bits[l + m / BS] >> (m % BS)) & 1u);
}

static void bit_put(uint32_t *bits, int64_t l, int32_t m, int v)
{
    uint32_t *w = &bits[l + m / BS];
    if (v) *w |= 1u << (m % BS);
    else *w &= ~(1u << (m % BS));
}

/* inbits (mpbits.f90:73-142), lower triangle: the counter of the group
 * pair (i, j) is the ibfw-bit field at bit (j-1)*ibfw of row i, whose bits
 * start at word noffi/BS + i (each row in words of its own); it is raised
 * by inc and saturates at mxcnt.  With ibfw = 1 the field is a flag. */
static void inbits(uint32_t *bits, int32_t n, int32_t ibfw, int32_t mxcnt, int32_t im, int32_t jm,
                   int32_t inc)
{
    int32_t j = im < jm ? im : jm, i = im < jm ? jm : im, b, icount = 0, jcount;
    if (j <= 0 || i > n) return;
    int64_t noffi = (int64_t)(i - 1) * (int64_t)i * ibfw / 2;
    int64_t noffj = (int64_t)(j - 1) * ibfw;
    int64_t l = noffi / BS + i + noffj / BS;             /* 1-based word */
    int32_t m = (int32_t)(noffj % BS);
    if (ibfw <= 1) { bits[l] |= (1u << m); return; }
    for (b = 0; b < ibfw; b++)
        if (bit_get(bits, l, m + b)) icount |= 1 << b;
    jcount = icount;
    icount = icount + inc < mxcnt ? icount + inc : mxcnt;
    if (icount != jcount)
        for (b = 0; b < ibfw; b++) bit_put(bits, l, m + b, (icount >> b) & 1);
}

int mpref_mpbits(int64_t nrec, int64_t nrecData, const int64_t *recPtr, const int32_t *inder,
                 const double *glder, const int32_t *varIndexOfTotal, int32_t nVar,
                 int32_t nG, const int32_t *allIndexGroups, const int32_t *parToGroup,
                 int32_t mreqpe, int64_t cap, int64_t *offsets, int32_t *columns,
                 int64_t *ncolw, int64_t *nmat)
{
    int32_t n = nG, i, j;
    const int32_t *npgrp = allIndexGroups - 1;  /* npgrp[1..n+1] */
    /* clbits (mpbits.f90:182-243) with msngpe = mhispe = 0: counters wide
     * enough to count to mreqpe */
    int32_t ireqpe = mreqpe > 1 ? mreqpe : 1, ibfw = 1, mxcnt = 1;
    for (i = 1; i <= 30; i++)
        if (ireqpe > mxcnt) { ibfw++; mxcnt = mxcnt * 2 + 1; }
    int64_t noffd = (int64_t)n * (int64_t)(n + 1) / 2;
    int64_t ndimb = noffd / BS + n;
    int64_t ndimc = noffd * ibfw / BS + n;
    uint32_t *bits = (uint32_t *)calloc((size_t)ndimb + 2, sizeof(uint32_t));
    uint32_t *cnt = (uint32_t *)calloc((size_t)ndimc + 2, sizeof(uint32_t));
    int32_t *back = (int32_t *)calloc((size_t)nVar + 2, sizeof(int32_t));
    int32_t *use = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nVar + 2));
    int32_t *grp = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nG + 2));
    int64_t r, lastGlobal, startLocal, startGlobal, startSpecial, endOfEntry;
    if (!bits || !cnt || !back || !use || !grp) return -1;

    /* loop2 second pass (pede.f90:6700-6862, 6889-6908): sorted variable
     * indices per record -> groups -> all group pairs, each counted once per
     * record; records from nrecData on are measurement lines, whose pairs
     * count mreqpe (pede.f90:7036) and so are always kept */
    for (r = 0; r < nrec; r++) {
        int32_t ng = 0, ngrp = 0, inc = r < nrecData ? 1 : ireqpe;
        endOfEntry = recPtr[r + 1] - 1;
        lastGlobal = recPtr[r];
        for (;;) {
            mpref_decode(inder, glder, endOfEntry, &lastGlobal, &startLocal,
                         &startGlobal, &startSpecial);
            if (startLocal < 0 && startGlobal < 0) break;
            if (startLocal >= 0) {
                for (int64_t w = startGlobal + 1; w <= lastGlobal; w++) {
                    int32_t ij = varIndexOfTotal[inder[w] - 1];
                    if (ij > 0 && back[ij] == 0) {
                        use[++ng] = ij;
                        back[ij] = ng;
                    }
                }
            }
        }
        qsort(use + 1, (size_t)ng, sizeof(int32_t), cmp_i32);
        int32_t prev = -1;
        for (i = 1; i <= ng; i++) {
            back[use[i]] = 0;
            int32_t g = parToGroup[use[i] - 1];
            if (g != prev) { grp[++ngrp] = g; prev = g; }
        }
        for (i = 1; i <= ngrp; i++)
            for (j = 1; j <= i; j++) inbits(cnt, n, ibfw, mxcnt, grp[i], grp[j], inc);
    }

    /* ndbits (mpbits.f90:305-566): a pair is kept when its counter reaches
     * mreqpe (mpbits.f90:409); the kept flags go to `bits` (one bit per
     * pair, the layout of ibfw = 1) for the column lists of spbits */
    int64_t *nsparr = offsets;  /* nsparr(1,k) = offsets[2*(k-1)], (2,k) = offsets[2*(k-1)+1] */
#define NS1(k) nsparr[2 * ((k) - 1)]
#define NS2(k) nsparr[2 * ((k) - 1) + 1]
    int64_t nd = npgrp[n + 1] - npgrp[1];
    for (i = 1; i <= n; i++) {
        int64_t noffi = (int64_t)(i - 1) * (int64_t)i * ibfw / 2;
        int64_t ll = noffi / BS + i;
        int64_t lk = (int64_t)(i - 1) * (int64_t)i / 2 / BS + i;
        int32_t mm = 0, last = 0, next, ib;
        int64_t inr = 0, irgn = 1;
        for (j = 1; j <= i; j++) {
            int32_t icount = 0;
            for (ib = 0; ib < ibfw; ib++) {
                if ((cnt[ll] >> mm) & 1u) icount |= 1 << ib;
                mm++;
                if (mm >= BS) { ll++; mm -= BS; }
            }
            next = 0;
            if (icount >= ireqpe) {
                next = 1;
                bit_put(bits, lk, j - 1, 1);
                inr += npgrp[j + 1] - npgrp[j];
                if (next != last) irgn++;
            }
            last = next;
        }
        NS1(i + 1) = irgn;
        NS2(i + 1) = inr;
    }
    free(cnt);
    int64_t ncw = 0;
    for (i = 1; i <= n; i++) {
        int64_t irgn = NS1(i + 1), inr = NS2(i + 1);
        int64_t nw0 = inr, nw1, nwcp;
        int32_t icp = 0;
        nwcp = nw0;
        if (inr > 0) {
            nw1 = irgn * 2;
            if (nw1 < nw0) icp = 1;
            nwcp = icp ? nw1 : nw0;
            ncw += nwcp;
        }
        NS1(i + 1) = nwcp;
        NS2(i + 1) = nw0 * (npgrp[i + 1] - npgrp[i]);
    }
    {
        int64_t lb = 0, ll = nd;
        int32_t n1 = 0;
        for (i = 1; i <= n; i++) {
            n1++;
            NS1(n1) = lb;
            NS2(n1) = ll;
            lb += NS1(n1 + 1);
            ll += NS2(n1 + 1);
        }
        n1++;
        NS1(n1) = lb;
        NS2(n1) = ll;
    }
    if (NS1(n + 1) > cap) { free(bits); free(back); free(use); free(grp); return -1; }

    /* spbits (mpbits.f90:1220-1350), nspc = 1 */
    int32_t *nsparc = columns - 1;  /* 1-based */
    for (i = 1; i <= n; i++) {
        int64_t noffi = (int64_t)(i - 1) * (int64_t)i / 2;
        int64_t l = noffi / BS + i;
        int32_t m = 0, last = 0, next;
        int64_t kl = NS1(i), l1 = NS2(i);
        int64_t ndiff = (NS1(i + 1) - kl) * (npgrp[i + 1] - npgrp[i]) - (NS2(i + 1) - l1);
        int64_t ll = l1;
        for (j = 1; j <= i; j++) {
            next = 0;
            if (bits[l] != 0 && ((bits[l] >> m) & 1u)) {
                if (ndiff == 0) {
                    for (int32_t kk = npgrp[j]; kk < npgrp[j + 1]; kk++) nsparc[++kl] = kk;
                } else {
                    next = 1;
                    if (last == 0) {
                        nsparc[++kl] = (int32_t)(ll - l1);
                        nsparc[++kl] = j;
                    }
                }
                ll += npgrp[j + 1] - npgrp[j];
            }
            last = next;
            m++;
            if (m >= BS) { m -= BS; l++; }
        }
        if (ndiff != 0) {
            nsparc[++kl] = (int32_t)(ll - l1);
            nsparc[++kl] = n + 1;
        }
    }
    *ncolw = NS1(n + 1);
    *nmat = NS2(n + 1);
#undef NS1
#undef NS2
    free(bits); free(back); free(use); free(grp);
    return 0;
}

/* ijpgrp, pede.f90:5371-5461 (nspc = 1).  Groups 1-based. */
static void ijpgrp(int32_t itema, int32_t itemb, int32_t nG, const int32_t *npgrp,
                   const int64_t *offsets, const int32_t *columns, int64_t *ij,
                   int32_t *lr)
{
    int32_t item1 = itema > itemb ? itema : itemb;
    int32_t item2 = itema > itemb ? itemb : itema;
    const int32_t *col = columns - 1;  /* 1-based */
    int64_t kk, ll, kl, ku, k;
    int32_t np, jtem, jtemn;
    *ij = 0;
    *lr = 0;
    if (item2 <= 0 || item1 > nG) return;
    np = npgrp[item1 + 1] - npgrp[item1];
    kk = offsets[2 * (item1 - 1)];
    ll = offsets[2 * (item1 - 1) + 1];
    kl = 1;
    ku = offsets[2 * item1] - kk;
    if (ku <= 0) return;
    if (col[kk + 1] == 0) {  /* compressed */
        kl = 2;
        ku = ku - 2;
        if (ku < kl) return;
        for (;;) {
            k = 2 * ((kl + ku) / 4);
            jtem = col[kk + k];
            jtemn = col[kk + k + 2];
            if (item2 >= jtem && item2 < jtemn) {
                *lr = col[kk + k + 1] - col[kk + k - 1];
                if (npgrp[item2] - npgrp[jtem] >= *lr) return;
                break;
            }
            if (item2 < jtem) ku = k - 2;
            else if (item2 >= jtemn) kl = k + 2;
            if (kl <= ku) continue;
            return;
        }
        *ij = ll + (int64_t)col[kk + k - 1] * np + npgrp[item2] - npgrp[jtem] + 1;
    } else {
        int32_t itemc = npgrp[item2];
        *lr = (int32_t)ku;
        for (;;) {
            k = (kl + ku) / 2;
            jtem = col[kk + k];
            if (itemc == jtem) break;
            if (itemc < jtem) ku = k - 1;
            else kl = k + 1;
            if (kl <= ku) continue;
            return;
        }
        *ij = ll + k;
    }
}

int64_t mpref_ijadd(int32_t i, int32_t j, int32_t nG, const int32_t *allIndexGroups,
                    const int32_t *parToGroup, const int64_t *offsets,
                    const int32_t *columns)
{
    const int32_t *npgrp = allIndexGroups - 1;
    int32_t item1 = i > j ? i : j, item2 = i > j ? j : i, lr;
    int32_t nAll = npgrp[nG + 1] - 1;
    int64_t ij;
    if (item2 <= 0 || item1 > nAll) return 0;
    if (item1 == item2) return item1;
    int32_t ipg1 = parToGroup[item1 - 1], ipg2 = parToGroup[item2 - 1];
    ijpgrp(ipg1, ipg2, nG, npgrp, offsets, columns, &ij, &lr);
    if (ij == 0) return 0;
    return ij + (item2 - npgrp[ipg2]) + (int64_t)(item1 - npgrp[ipg1]) * lr;
}

/* mupdat, pede.f90:3134-3204 (matsto 1 and 2, no preconditioner copy) */
void mpref_mupdat(int32_t matsto, int32_t i, int32_t j, double add, int32_t nG,
                  const int32_t *allIndexGroups, const int32_t *parToGroup,
                  const int64_t *offsets, const int32_t *columns, double *matD)
{
    int64_t ia = i > j ? i : j, ja = i > j ? j : i, ij;
    if (i <= 0 || j <= 0 || add == 0.0) return;
    if (matsto == 2) {
        ij = mpref_ijadd(i, j, nG, allIndexGroups, parToGroup, offsets, columns);
        if (ij == 0) return;
        matD[ij - 1] += add;
    } else {
        ij = (ia * ia - ia) / 2 + ja;
        matD[ij - 1] += add;
    }
}
