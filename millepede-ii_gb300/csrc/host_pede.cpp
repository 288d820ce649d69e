// host_pede.cpp -- host side of pede around the device hot path: label
// table and parameter groups (loop1), the mpbits sparse structure (loop2),
// the iteration control (xloopn/loopn/addcst without line search) and the
// millepede.res writer (prtglo).  In a Fortran pede build these steps stay
// in pede itself; this C++ version drives the C-ABI for tests, the
// benchmark and the pede_gpu command.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <functional>
#include <vector>

#include "../../include/mpgpu.h"
#include "host_struct.h"

namespace {

// measurement boundaries of one record (decodeNextMeasurement,
// pede.f90:2428-2468); positions absolute
template <class F>
bool for_each_measurement(const int32_t *in, const double *gl, int64_t w0, int64_t w1, F f) {
    int64_t lg = w0;
    const int64_t end = w1 - 1;
    for (;;) {
        if (lg >= end) return true;
        do { lg++; if (lg > end) return false; } while (in[lg] != 0);
        const int64_t sl = lg;
        do { lg++; if (lg > end) return false; } while (in[lg] != 0);
        const int64_t sg = lg;
        if (sl + 1 == sg && gl[sg] < 0.0) {
            lg = lg + (int64_t)(-gl[sg] + 0.5);
            continue;
        }
        while (lg < end && in[lg + 1] != 0) lg++;
        f(sl, sg, lg);
    }
}

int32_t find_label(const std::vector<int32_t> &lab, int32_t item) {
    auto it = std::lower_bound(lab.begin(), lab.end(), item);
    if (it == lab.end() || *it != item) return -1;
    return (int32_t)(it - lab.begin());
}

// label -> 0-based total index: direct table for compact label ranges,
// binary search otherwise
struct LabelMap {
    const std::vector<int32_t> &lab;
    std::vector<int32_t> direct;
    int32_t lo = 0;
    explicit LabelMap(const std::vector<int32_t> &l) : lab(l) {
        if (lab.empty()) return;
        const int64_t span = (int64_t)lab.back() - lab.front() + 1;
        if (span <= (int64_t)64 << 20) {
            lo = lab.front();
            direct.assign((size_t)span, -1);
            for (size_t i = 0; i < lab.size(); ++i) direct[(size_t)(lab[i] - lo)] = (int32_t)i;
        }
    }
    int32_t find(int32_t item) const {
        if (!direct.empty()) {
            const int64_t k = (int64_t)item - lo;
            return (k < 0 || k >= (int64_t)direct.size()) ? -1 : direct[(size_t)k];
        }
        return find_label(lab, item);
    }
};

int host_threads(int64_t nwork) {
    int n = (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (nwork < 20000) n = 1;
    return n;
}

template <class F>
void run_threads(int nt, F f) {
    if (nt <= 1) { f(0); return; }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back([&f, t] { f(t); });
    for (auto &x : th) x.join();
}

}  // namespace

// loop1: labels (ascending order defines the total index), entries per
// label counted per equation over non-zero derivatives (mcount = 0), the
// parameter groups and the variable-parameter numbering.  A group is a
// maximal run of consecutive total indices that no equation splits: every
// equation's sorted index list cuts before its first element, after its
// last element and at each of its gaps (the fixed point of pargrp,
// pede.f90:2311-2404, over all equations).
extern "C" int32_t mpgpu_host_labels(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                                     const double *glder, int32_t nsteer,
                                     const int32_t *steerLabels, int32_t npre,
                                     const int32_t *preLabel, const double *preSigma,
                                     int32_t mreqenf, int32_t cap, int32_t *labels,
                                     int64_t *counter, int32_t *varIndex, int32_t *totGroup,
                                     int32_t *nVar, int32_t *nVarGroups) {
    const int nt = host_threads(nrec);
    // distinct labels: per-thread sort/unique of the record labels, merged
    std::vector<std::vector<int32_t>> part(nt);
    std::vector<int> bad(nt, 0);
    run_threads(nt, [&](int t) {
        std::vector<int32_t> &v = part[t];
        int32_t last = 0;
        for (int64_t r = nrec * t / nt; r < nrec * (t + 1) / nt; ++r) {
            bool ok = for_each_measurement(inder, glder, recPtr[r], recPtr[r + 1],
                                           [&](int64_t, int64_t sg, int64_t lg) {
                                               for (int64_t w = sg + 1; w <= lg; ++w)
                                                   if (inder[w] > 0 && inder[w] != last) {
                                                       v.push_back(inder[w]);
                                                       last = inder[w];
                                                   }
                                           });
            if (!ok) { bad[t] = 1; return; }
            if (v.size() > (1u << 22)) {
                std::sort(v.begin(), v.end());
                v.erase(std::unique(v.begin(), v.end()), v.end());
            }
        }
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    });
    for (int t = 0; t < nt; ++t)
        if (bad[t]) return -20;
    std::vector<int32_t> all;
    for (int32_t i = 0; i < nsteer; ++i)
        if (steerLabels[i] > 0) all.push_back(steerLabels[i]);
    for (auto &v : part) all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
    const int32_t n = (int32_t)all.size();
    if (n > cap) return -1;
    LabelMap lmap(all);
    // entries and group cuts per equation (non-zero derivatives), per thread
    // partial arrays merged at the end: cut[i] = boundary between i and i+1
    std::vector<std::vector<uint8_t>> cutP(nt), seenP(nt);
    std::vector<std::vector<int64_t>> cntP(nt);
    run_threads(nt, [&](int t) {
        std::vector<uint8_t> &cut = cutP[t], &seen = seenP[t];
        std::vector<int64_t> &cnt = cntP[t];
        cut.assign(n + 1, 0);
        seen.assign(n, 0);
        cnt.assign(n, 0);
        std::vector<int32_t> list;
        for (int64_t r = nrec * t / nt; r < nrec * (t + 1) / nt; ++r) {
            for_each_measurement(inder, glder, recPtr[r], recPtr[r + 1], [&](int64_t, int64_t sg, int64_t lg) {
                list.clear();
                for (int64_t w = sg + 1; w <= lg; ++w) if (inder[w] <= 0) bad[t] = 1;
                if (bad[t]) return;
                for (int64_t w = sg + 1; w <= lg; ++w) {
                    if (glder[w] == 0.0) continue;
                    list.push_back(lmap.find(inder[w]));
                }
                if (list.empty()) return;
                std::sort(list.begin(), list.end());
                for (int32_t x : list) { cnt[x]++; seen[x] = 1; }
                if (list.front() > 0) cut[list.front() - 1] = 1;
                for (size_t q = 0; q + 1 < list.size(); ++q)
                    if (list[q + 1] != list[q] + 1) {
                        cut[list[q]] = 1;
                        if (list[q + 1] > 0) cut[list[q + 1] - 1] = 1;
                    }
                cut[list.back()] = 1;
            });
        }
    });
    for (int t = 0; t < nt; ++t)
        if (bad[t]) return -23;
    std::vector<uint8_t> cut(n + 1, 0), seen(n, 0);
    std::vector<int64_t> cnt(n, 0);
    for (int t = 0; t < nt; ++t)
        for (int32_t i = 0; i < n; ++i) {
            cut[i] |= cutP[t][i];
            seen[i] |= seenP[t][i];
            cnt[i] += cntP[t][i];
        }
    return labels_finish(all, cnt, cut, seen, npre, preLabel, preSigma, mreqenf, labels, counter, varIndex,
                         totGroup, nVar, nVarGroups);
}

int32_t labels_finish(const std::vector<int32_t> &all, const std::vector<int64_t> &cnt,
                      const std::vector<uint8_t> &cut, const std::vector<uint8_t> &seen, int32_t npre,
                      const int32_t *preLabel, const double *preSigma, int32_t mreqenf, int32_t *labels,
                      int64_t *counter, int32_t *varIndex, int32_t *totGroup, int32_t *nVar,
                      int32_t *nVarGroups) {
    const int32_t n = (int32_t)all.size();
    LabelMap lmap(all);
    std::vector<double> ps(n, 0.0);
    for (int32_t i = 0; i < npre; ++i) {
        int32_t li = lmap.find(preLabel[i]);
        if (li >= 0) ps[li] = preSigma[i];
    }
    int32_t nv = 0, ntg = 0;
    for (int32_t i = 0; i < n; ++i) {
        labels[i] = all[i];
        counter[i] = cnt[i];
        if (ps[i] < 0.0) varIndex[i] = -1;
        else if (cnt[i] < mreqenf) varIndex[i] = -2;
        else varIndex[i] = ++nv;
        totGroup[i] = 0;
        if (!seen[i]) continue;
        if (i == 0 || cut[i - 1] || !seen[i - 1]) ntg++;
        totGroup[i] = ntg;
    }
    int32_t nvg = 0, lgrp = -1;
    for (int32_t i = 0; i < n; ++i) {
        if (varIndex[i] <= 0) continue;
        if (totGroup[i] != lgrp) nvg++;
        lgrp = totGroup[i];
    }
    *nVar = nv;
    *nVarGroups = nvg;
    return n;
}

extern "C" int32_t mpgpu_host_translate(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                                        const double *glder, int32_t nTotal, const int32_t *labels,
                                        int32_t *outInder) {
    std::vector<int32_t> lab(labels, labels + nTotal);
    LabelMap lmap(lab);
    const int nt = host_threads(nrec);
    std::vector<int> bad(nt, 0);
    run_threads(nt, [&](int t) {
        const int64_t a = nrec * t / nt, b = nrec * (t + 1) / nt;
        if (b <= a) return;
        std::memcpy(outInder + recPtr[a], inder + recPtr[a], sizeof(int32_t) * (size_t)(recPtr[b] - recPtr[a]));
        for (int64_t r = a; r < b; ++r) {
            bool ok = for_each_measurement(inder, glder, recPtr[r], recPtr[r + 1],
                                           [&](int64_t, int64_t sg, int64_t lg) {
                                               for (int64_t w = sg + 1; w <= lg; ++w)
                                                   outInder[w] = lmap.find(inder[w]) + 1;
                                           });
            if (!ok) { bad[t] = 1; return; }
        }
    });
    for (int t = 0; t < nt; ++t)
        if (bad[t]) return 20;
    return 0;
}

// loop2 sparse structure: the pairs of parameter groups met in the records
// (each counted once per record, pede.f90:6889-6908; the structure-only
// records of the measurement lines from nrecData on count mreqpe,
// pede.f90:7036) whose count reaches mreqpe are stored (clbits/inbits/ndbits,
// mpbits.f90:73-142, 182-243, 305-566); per row group the columns are kept
// either as a list of parameter indices or, when that is shorter, as regions
// of consecutive groups (offset, first group) closed by (end offset, nG+1)
// (spbits, mpbits.f90:1220-1350).  The counters saturate at the largest
// value of their bit field, which is at least mreqpe, as pede's do; the
// fields are a power of two bits wide so that none crosses a 64-bit word.
extern "C" int32_t mpgpu_host_mpbits_pairentries(int64_t nrec, int64_t nrecData, const int64_t *recPtr,
                                                 const int32_t *inder, const double *glder,
                                                 const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                                                 const int32_t *allIndexGroups, int32_t mreqpe, int64_t cap,
                                                 int64_t *offsets, int32_t *columns, int64_t *ncolw,
                                                 int64_t *nmat, int64_t capSup, int32_t *suppressed,
                                                 int64_t *nsup) {
    if (nrec < 0 || nG <= 0 || nVar <= 0 || !recPtr || !allIndexGroups || !offsets || !ncolw || !nmat ||
        (capSup > 0 && !suppressed))
        return MPGPU_ERR_ARG;
    const uint64_t req = (uint64_t)std::max<int32_t>(mreqpe, 1);
    uint32_t fw = 1;
    while (fw < 32 && ((1ull << fw) - 1) < req) fw *= 2;
    const uint64_t mx = (1ull << fw) - 1;
    std::vector<int32_t> p2g(nVar);
    for (int32_t g = 1; g <= nG; ++g)
        for (int32_t v = allIndexGroups[g - 1]; v < allIndexGroups[g]; ++v) p2g[v - 1] = g;
    // lower-triangular counters over group pairs, row I holds J = 1..I
    std::vector<uint64_t> rowWord(nG + 2, 0);   // first word of row I
    for (int32_t I = 1; I <= nG; ++I) rowWord[I + 1] = rowWord[I] + ((uint64_t)I * fw + 63) / 64;
    std::vector<uint64_t> bits(rowWord[nG + 1] + 1, 0);
    const int nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    // records split over threads; a counter is raised by compare-and-swap of
    // its word (saturating adds commute, so the counts do not depend on the
    // order)
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        th.emplace_back([&, t] {
            std::vector<int32_t> grp;
            for (int64_t r = nrec * t / nt; r < nrec * (t + 1) / nt; ++r) {
                const uint64_t inc = r < nrecData ? 1 : req;
                grp.clear();
                for_each_measurement(inder, glder, recPtr[r], recPtr[r + 1], [&](int64_t, int64_t sg, int64_t lg) {
                    for (int64_t w = sg + 1; w <= lg; ++w) {
                        const int32_t v = varIndexOfTotal[inder[w] - 1];
                        if (v > 0) grp.push_back(p2g[v - 1]);
                    }
                });
                std::sort(grp.begin(), grp.end());
                grp.erase(std::unique(grp.begin(), grp.end()), grp.end());
                for (size_t a = 0; a < grp.size(); ++a)
                    for (size_t b = 0; b <= a; ++b) {
                        const uint64_t pos = rowWord[grp[a]] * 64 + (uint64_t)(grp[b] - 1) * fw;
                        uint64_t *word = &bits[pos >> 6];
                        const uint32_t sh = (uint32_t)(pos & 63);
                        if (fw == 1) {
                            __atomic_fetch_or(word, 1ull << sh, __ATOMIC_RELAXED);
                            continue;
                        }
                        uint64_t old = __atomic_load_n(word, __ATOMIC_RELAXED);
                        for (;;) {
                            const uint64_t c = (old >> sh) & mx;
                            if (c >= mx) break;
                            const uint64_t nc = std::min(c + inc, mx);
                            const uint64_t nw = (old & ~(mx << sh)) | (nc << sh);
                            if (__atomic_compare_exchange_n(word, &old, nw, true, __ATOMIC_RELAXED,
                                                            __ATOMIC_RELAXED))
                                break;
                        }
                    }
            }
        });
    }
    for (auto &x : th) x.join();
    auto count = [&](int32_t I, int32_t J) {
        const uint64_t pos = rowWord[I] * 64 + (uint64_t)(J - 1) * fw;
        return (bits[pos >> 6] >> (pos & 63)) & mx;
    };
    auto test = [&](int32_t I, int32_t J) { return count(I, J) >= req; };
    const int64_t nd = allIndexGroups[nG] - allIndexGroups[0];
    std::vector<int64_t> nw(nG + 1), nm(nG + 1);
    std::vector<uint8_t> comp(nG + 1, 0);
    int64_t ns = 0;
    for (int32_t I = 1; I <= nG; ++I) {
        int64_t inr = 0, irgn = 1;
        bool last = false;
        for (int32_t J = 1; J <= I; ++J) {
            const uint64_t c = count(I, J);
            const bool on = c >= req;
            if (on) {
                inr += allIndexGroups[J] - allIndexGroups[J - 1];
                if (!last) irgn++;
            } else if (c > 0) {
                if (ns < capSup) { suppressed[2 * ns] = I; suppressed[2 * ns + 1] = J; }
                ns++;
            }
            last = on;
        }
        const int64_t np = allIndexGroups[I] - allIndexGroups[I - 1];
        comp[I] = inr > 0 && 2 * irgn < inr;
        nw[I] = comp[I] ? 2 * irgn : inr;
        nm[I] = inr * np;
    }
    if (nsup) *nsup = ns;
    int64_t lb = 0, ll = nd;
    for (int32_t I = 1; I <= nG; ++I) {
        offsets[2 * (I - 1)] = lb;
        offsets[2 * (I - 1) + 1] = ll;
        lb += nw[I];
        ll += nm[I];
    }
    offsets[2 * nG] = lb;
    offsets[2 * nG + 1] = ll;
    *ncolw = lb;
    *nmat = ll;
    if (lb > cap || ns > capSup) return -1;
    for (int32_t I = 1; I <= nG; ++I) {
        int64_t k = offsets[2 * (I - 1)];
        int64_t width = 0;
        bool last = false;
        for (int32_t J = 1; J <= I; ++J) {
            const bool on = test(I, J);
            const int32_t nj = allIndexGroups[J] - allIndexGroups[J - 1];
            if (on) {
                if (comp[I]) {
                    if (!last) { columns[k++] = (int32_t)width; columns[k++] = J; }
                } else {
                    for (int32_t q = 0; q < nj; ++q) columns[k++] = allIndexGroups[J - 1] + q;
                }
                width += nj;
            }
            last = on;
        }
        if (comp[I]) { columns[k++] = (int32_t)width; columns[k++] = nG + 1; }
    }
    return 0;
}

// every pair met stored (pairentries 1)
extern "C" int32_t mpgpu_host_mpbits(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                                     const double *glder, const int32_t *varIndexOfTotal,
                                     int32_t nVar, int32_t nG, const int32_t *allIndexGroups,
                                     int64_t cap, int64_t *offsets, int32_t *columns,
                                     int64_t *ncolw, int64_t *nmat) {
    int64_t nsup = 0;
    return mpgpu_host_mpbits_pairentries(nrec, nrec, recPtr, inder, glder, varIndexOfTotal, nVar, nG,
                                         allIndexGroups, 1, cap, offsets, columns, ncolw, nmat, 0, nullptr,
                                         &nsup);
}

// ------------------------------------------------------------------ job

namespace {
// feasib (pede.f90:1553-1680), one constraint group: residuals r = rhs - C p
// over all labels; when their rms is at least concut (first of two
// iterations), p_var += C^T (C C^T)^-1 r.  cinv holds the Cholesky factor
// of the product matrix C C^T (rows of ncon); pede inverts that matrix with
// sqminv (feasma, pede.f90:1466-1478) and multiplies with dbsvx, the same
// solution up to rounding.
void feasib(const mpgpu_job *job, const std::vector<int32_t> &lab, const int32_t *varIndex,
            const std::vector<double> &cfac, std::vector<double> &gpar, float concut) {
    const int32_t ncon = job->ncon;
    if (ncon <= 0) return;
    std::vector<double> r(ncon), lam(ncon);
    for (int iter = 1; iter <= 2; ++iter) {
        double sum1 = 0.0;
        for (int32_t c = 0; c < ncon; ++c) {
            double rhs = job->conRhs ? job->conRhs[c] : 0.0;
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; ++k) {
                const int32_t li = find_label(lab, job->conLabel[k]);
                if (li >= 0) rhs = rhs - job->conCoef[k] * gpar[li];
            }
            r[c] = rhs;
            sum1 = sum1 + rhs * rhs;
        }
        sum1 = std::sqrt(sum1 / (double)ncon);
        if (iter == 1 && sum1 < concut) return;
        // (L L^T) lam = r
        for (int32_t a = 0; a < ncon; ++a) {
            double t = r[a];
            for (int32_t b = 0; b < a; ++b) t -= cfac[(size_t)a * ncon + b] * lam[b];
            lam[a] = t / cfac[(size_t)a * ncon + a];
        }
        for (int32_t a = ncon - 1; a >= 0; --a) {
            double t = lam[a];
            for (int32_t b = a + 1; b < ncon; ++b) t -= cfac[(size_t)b * ncon + a] * lam[b];
            lam[a] = t / cfac[(size_t)a * ncon + a];
        }
        for (int32_t c = 0; c < ncon; ++c)
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; ++k) {
                const int32_t li = find_label(lab, job->conLabel[k]);
                if (li >= 0 && varIndex[li] > 0) gpar[li] = gpar[li] + lam[c] * job->conCoef[k];
            }
    }
}
}  // namespace

// Whole alignment job: structure on the host, data loops and solves on the
// device.  Iteration control of xloopn (pede.f90:8501-9334) without line
// search and function-value loops: every iteration rebuilds the matrix,
// solves and adds the correction; chi2-cut factors per loop as in loopn
// (pede.f90:2583-2593).
// Whole job; `admit`, when given, is asked for the job's device footprint
// after the host structure passes and before any device allocation of the
// job, and may block until that much of the device budget is free (the
// serving loop, mpgpu_serve.cpp); it returns false when the job can never
// fit.
int32_t pede_run_admitted(mpgpu_ctx *ctxIn, const mpgpu_steer *st, const mpgpu_job *job, mpgpu_result *res,
                          const std::function<bool(int64_t)> &admit) {
    if (!st || !job || !res) return MPGPU_ERR_ARG;
    using Clock = std::chrono::steady_clock;
    const auto msSince = [](Clock::time_point a) {
        return std::chrono::duration<double, std::milli>(Clock::now() - a).count();
    };
    const Clock::time_point tJob = Clock::now();
    res->msStructure = res->msUpload = res->msLoops = res->msSolves = res->msHostIter = res->msJob = 0.0;
    mpgpu_ctx *ctx = ctxIn;
    if (!ctx) {
        mpgpu_cfg cfg{0, 0, 0};
        int32_t rc = mpgpu_create(&ctx, &cfg);
        if (rc) return rc;
    }
    int32_t rc = 0;
    std::vector<int32_t> steer;
    for (int32_t i = 0; i < job->npar; ++i) steer.push_back(job->parLabel[i]);
    if (job->ncon) for (int32_t i = 0; i < job->conStart[job->ncon]; ++i) steer.push_back(job->conLabel[i]);
    if (job->nmeas) for (int32_t i = 0; i < job->msStart[job->nmeas]; ++i) steer.push_back(job->msLabel[i]);
    const int32_t cap = res->cap;
    std::vector<int64_t> counter(cap);
    std::vector<int32_t> totGroup(cap);
    int32_t nVar = 0, nG = 0;
    // structure passes on the device: the records are copied once and stay
    // there translated (not under an admission hook, which must see the
    // footprint before any device allocation of the job)
    // (measurement lines in sparse storage add structure-only records, which
    // the host passes take)
    // pairentries (mreqpe > 1, sparse storage only as in pede) counts the
    // group pairs on the host
    const int32_t mreqpe = st->matsto == 2 ? std::max<int32_t>(st->mreqpe, 1) : 1;
    const bool onDevice =
        st->structDevice != 0 && !admit && !(st->matsto == 2 && job->nmeas > 0) && mreqpe == 1;
    int32_t ntot = onDevice
                       ? mpgpu_loop1_device(ctx, job->nrec, job->recPtr, job->inder, job->glder,
                                            (int32_t)steer.size(), steer.data(), job->npar, job->parLabel,
                                            job->parSigma, st->mreqenf, cap, res->labels, counter.data(),
                                            res->varIndex, totGroup.data(), &nVar, &nG)
                       : mpgpu_host_labels(job->nrec, job->recPtr, job->inder, job->glder, (int32_t)steer.size(),
                                           steer.data(), job->npar, job->parLabel, job->parSigma, st->mreqenf,
                                           cap, res->labels, counter.data(), res->varIndex, totGroup.data(),
                                           &nVar, &nG);
    if (ntot < 0) {
        const int32_t code = ntot == -23 ? MPGPU_ERR_BADINDEX : ntot <= -30 ? -ntot : 20;
        res->exitCode = code;
        if (!ctxIn) mpgpu_destroy(ctx);
        return code;
    }
    res->nTotal = ntot;
    res->nVar = nVar;
    res->nVarGroups = nG;
    std::vector<int32_t> lab(res->labels, res->labels + ntot);
    std::vector<int32_t> aig(nG + 1);
    {
        int32_t cur = 0, prev = -1;
        for (int32_t i = 0; i < ntot; ++i) {
            if (res->varIndex[i] <= 0) continue;
            if (totGroup[i] != prev) { aig[cur++] = res->varIndex[i]; prev = totGroup[i]; }
        }
        aig[nG] = nVar + 1;
    }
    const int64_t nw = job->recPtr[job->nrec];
    std::vector<int32_t> tinder;
    if (!onDevice) {
        tinder.resize(nw);
        mpgpu_host_translate(job->nrec, job->recPtr, job->inder, job->glder, ntot, res->labels, tinder.data());
    }
    std::vector<int64_t> offsets;
    std::vector<int32_t> columns, suppressed;
    int64_t ncolw = 0, nmat = 0, nsup = 0;
    // the parameter pairs of the measurement lines belong to the sparse
    // structure whatever the records hold (pede.f90:7007-7042, increment
    // mreqpe: always kept): one structure-only record per measurement line
    // (header, value, positive sigma, its labels as global words)
    int64_t nrecS = job->nrec;
    const int64_t *rpS = job->recPtr;
    const int32_t *inS = tinder.data();
    const double *glS = job->glder;
    std::vector<int64_t> rpA;
    std::vector<int32_t> inA;
    std::vector<double> glA;
    if (st->matsto == 2 && job->nmeas > 0) {
        std::vector<int64_t> rpRaw(1, 0);
        std::vector<int32_t> raw;
        std::vector<double> glRaw;
        for (int32_t m = 0; m < job->nmeas; ++m) {
            for (int k = 0; k < 3; ++k) {
                raw.push_back(0);
                glRaw.push_back(k == 2 ? 1.0 : 0.0);
            }
            for (int32_t q = job->msStart[m]; q < job->msStart[m + 1]; ++q) {
                raw.push_back(job->msLabel[q]);
                glRaw.push_back(1.0);
            }
            rpRaw.push_back((int64_t)raw.size());
        }
        std::vector<int32_t> trRaw(raw.size());
        mpgpu_host_translate(job->nmeas, rpRaw.data(), raw.data(), glRaw.data(), ntot, res->labels, trRaw.data());
        rpA.assign(job->recPtr, job->recPtr + job->nrec + 1);
        for (int32_t m = 1; m <= job->nmeas; ++m) rpA.push_back(nw + rpRaw[m]);
        inA.assign(tinder.begin(), tinder.end());
        inA.insert(inA.end(), trRaw.begin(), trRaw.end());
        glA.assign(job->glder, job->glder + nw);
        glA.insert(glA.end(), glRaw.begin(), glRaw.end());
        nrecS = job->nrec + job->nmeas;
        rpS = rpA.data();
        inS = inA.data();
        glS = glA.data();
    }
    if (st->matsto == 2) {
        offsets.resize(2 * (nG + 1));
        int64_t capc = 1 << 20, caps = mreqpe > 1 ? 1 << 18 : 0;
        for (;;) {
            columns.assign(capc, 0);
            suppressed.assign(2 * std::max<int64_t>(caps, 1), 0);
            const int32_t r2 =
                onDevice ? mpgpu_loop2_device(ctx, res->varIndex, nVar, nG, aig.data(), capc, offsets.data(),
                                              columns.data(), &ncolw, &nmat)
                         : mpgpu_host_mpbits_pairentries(nrecS, job->nrec, rpS, inS, glS, res->varIndex, nVar,
                                                         nG, aig.data(), mreqpe, capc, offsets.data(),
                                                         columns.data(), &ncolw, &nmat, caps,
                                                         suppressed.data(), &nsup);
            if (r2 == 0) break;
            if (r2 != -1) {
                res->exitCode = r2;
                if (!ctxIn) mpgpu_destroy(ctx);
                return r2;
            }
            capc = std::max<int64_t>(ncolw, 1);
            caps = nsup;
        }
    }
    res->msStructure = msSince(tJob);
    if (admit) {
        // device footprint: records and their tables, update staging
        // (bounded by the squared words per record), matrix, dense solve
        int64_t stage = 0;
        for (int64_t r = 0; r < job->nrec; ++r) {
            const int64_t w = job->recPtr[r + 1] - job->recPtr[r];
            stage += (w / 2) * (w / 2 + 1) / 2;
        }
        const int64_t nm = st->matsto == 2 ? nmat : (int64_t)nVar * (nVar + 1) / 2;
        const int64_t npad = ((int64_t)nVar + 127) / 128 * 128;
        // dense forms: F and L (npad^2 each), the split panels, the WY
        // buffers of the constraint elimination and the preconditioner's
        // super-block inverses (about 40 KB per row)
        const int64_t dense = (st->metsol == 31 || st->metsol == 32) ? 2 * npad * npad + 5120 * npad : 0;
        const int64_t stageCap = (int64_t)2 << 30;   // 2 x 8 GiB staging buffers at most (in doubles)
        const int64_t bytes = 40 * nw + 8 * (std::min(stage, stageCap) + nm + dense) + 64 * (int64_t)nVar +
                              ((int64_t)64 << 20);
        if (!admit(bytes)) {
            res->exitCode = MPGPU_ERR_BUDGET;
            if (!ctxIn) mpgpu_destroy(ctx);
            return MPGPU_ERR_BUDGET;
        }
    }
    rc = mpgpu_set_layout(ctx, ntot, res->varIndex, nVar, nG, aig.data(), st->matsto,
                          offsets.empty() ? nullptr : offsets.data(), columns.empty() ? nullptr : columns.data(),
                          ncolw, nmat);
    // the records' updates of the pairs left out are summed apart and dropped
    if (!rc && nsup > 0) rc = mpgpu_set_suppressed_pairs(ctx, nsup, suppressed.data());
    const int32_t ncon = job->ncon;
    std::vector<double> A;
    if (!rc && ncon > 0) {
        A.assign((size_t)ncon * nVar, 0.0);
        for (int32_t c = 0; c < ncon; ++c)
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; ++k) {
                int32_t li = find_label(lab, job->conLabel[k]);
                if (li < 0) continue;
                if (res->varIndex[li] > 0) A[(size_t)c * nVar + res->varIndex[li] - 1] += job->conCoef[k];
            }
        rc = mpgpu_set_constraints(ctx, ncon, A.data());
    }
    const Clock::time_point tUp = Clock::now();
    if (!rc)
        rc = mpgpu_upload_records(ctx, job->nrec, job->recPtr, onDevice ? nullptr : tinder.data(),
                                  onDevice ? nullptr : job->glder, job->recFile, job->nfiles, job->fileWeight);
    res->msUpload = msSince(tUp);
    const int32_t nfit = nVar - ncon;
    res->nFit = nfit;
    std::vector<double> gpar(ntot, 0.0), psig(ntot, 0.0);
    for (int32_t i = 0; i < job->npar; ++i) {
        int32_t li = find_label(lab, job->parLabel[i]);
        if (li < 0) continue;
        if (job->parValue) gpar[li] = job->parValue[i];
        if (job->parSigma) psig[li] = job->parSigma[i];
    }
    const std::vector<double> gstart(gpar);   // globalParStart (loop1, pede.f90:5916-5930)
    // product matrix C C^T of the constraints over the variable parameters
    // (feasma, pede.f90:1466-1476) and its Cholesky factor for feasib; the
    // start values are made feasible before the first data loop (cut 1e-12,
    // xloopn pede.f90:8693, 8730)
    std::vector<double> cfac;
    if (!rc && ncon > 0) {
        cfac.assign((size_t)ncon * ncon, 0.0);
        for (int32_t l = 0; l < nVar; ++l)
            for (int32_t a = 0; a < ncon; ++a)
                for (int32_t b = 0; b <= a; ++b)
                    cfac[(size_t)a * ncon + b] = cfac[(size_t)a * ncon + b] + A[(size_t)a * nVar + l] * A[(size_t)b * nVar + l];
        for (int32_t a = 0; a < ncon && !rc; ++a) {
            for (int32_t b = 0; b <= a; ++b) {
                double t = cfac[(size_t)a * ncon + b];
                for (int32_t k = 0; k < b; ++k) t -= cfac[(size_t)a * ncon + k] * cfac[(size_t)b * ncon + k];
                if (a == b) {
                    if (!(t > 0.0)) { rc = MPGPU_ERR_QL; break; }
                    cfac[(size_t)a * ncon + a] = std::sqrt(t);
                } else {
                    cfac[(size_t)a * ncon + b] = t / cfac[(size_t)b * ncon + b];
                }
            }
        }
        if (!rc) feasib(job, lab, res->varIndex, cfac, gpar, 1.0e-12f);
    }
    std::vector<int32_t> v2t(nVar);
    for (int32_t i = 0; i < ntot; ++i)
        if (res->varIndex[i] > 0) v2t[res->varIndex[i] - 1] = i;
    std::vector<int32_t> pi, pj;
    std::vector<double> pa;
    for (int32_t i = 0; i < nVar; ++i) {
        const double s = psig[v2t[i]];
        if (s > 0.0) { pi.push_back(i + 1); pj.push_back(i + 1); pa.push_back(1.0 / (s * s)); }
    }
    // monitorresiduals / monitorpulls (pede.f90:6571-6579, 2879, 9011):
    // groups of the first global labels from the translated records; the
    // group histograms of one data loop are written as millepede.mon lines
    // after the first loop (bit 0), the last (bit 1) or every loop (< 0)
    const bool monitor = !rc && st->monitor != 0 && job->monPath;
    const int32_t monBins = std::max<int32_t>(st->monitorBins, 2);
    std::vector<int32_t> measIndex, groupLabel;
    std::vector<double> measRes;
    int32_t numMeas = 0;
    bool monHeader = true;
    if (monitor) {
        std::vector<int32_t> tr;
        const int32_t *tin = tinder.data();
        if (onDevice) {
            tr.resize(nw);
            mpgpu_host_translate(job->nrec, job->recPtr, job->inder, job->glder, ntot, res->labels, tr.data());
            tin = tr.data();
        }
        measIndex.assign(ntot, 0);
        measRes.assign(ntot, 0.0);
        rc = mpgpu_monitor_groups(job->nrec, job->recPtr, tin, job->glder, ntot, measIndex.data(), measRes.data(),
                                  &numMeas);
        groupLabel.assign(std::max(numMeas, 1), 0);
        for (int32_t i = 0; i < ntot; ++i)
            if (measIndex[i] > 0) groupLabel[measIndex[i] - 1] = res->labels[i];
        mpgpu_monitor_cfg mc{100, 5.0f, monBins, st->monitorPulls ? 1 : 0, 0};
        if (!rc) rc = mpgpu_set_monitor(ctx, &mc, measIndex.data(), measRes.data(), numMeas);
    }
    std::vector<int64_t> monHist(4 * 102), monMeas((size_t)std::max(numMeas, 1) * monBins);
    int32_t monLoop = 0;
    auto writeMon = [&](int32_t loop) {
        const int32_t r = mpgpu_write_mon(job->monPath, monHeader ? 1 : 0, st->monitorPulls ? 1 : 0, loop, numMeas,
                                          groupLabel.data(), monMeas.data(), monBins, measRes.data());
        monHeader = false;
        return r;
    };
    std::vector<double> gvec(nVar), corr(nVar), err(nVar, 0.0), diag0(nVar, 0.0), cres(ncon > 0 ? ncon : 1, 0.0);
    std::vector<int64_t> gcnt(nVar);
    bool haveErr = false;
    float chicut = st->chicut;
    int64_t nrejTot = 0;
    std::memset(res->nrej, 0, sizeof(res->nrej));
    res->msBuild = res->msSolve = 0.0;
    if (!rc && (st->metsol == 4 || st->metsol == 5)) rc = mpgpu_set_preconditioner(ctx, st->mbandw, st->lprecm);
    const Clock::time_point tIter = Clock::now();
    double msLoopWall = 0.0, msSolveWall = 0.0;
    for (int32_t iter = 1; !rc && iter <= st->mitera; ++iter) {
        const int32_t nloopn = iter;
        if (nloopn > 1) {
            if (nloopn == 2) chicut = st->chirem;
            else {
                chicut = std::sqrt(chicut);
                if (chicut != 0.0f && chicut < 1.5f) chicut = 1.0f;
                if (chicut != 0.0f && nrejTot == 0) chicut = 1.0f;
            }
        }
        mpgpu_fitopts fo{1, nloopn, st->lhuber, st->lfitbb, chicut, st->chhuge, st->dwcut, st->cndlmx};
        mpgpu_fitstats fs;
        const Clock::time_point tL = Clock::now();
        rc = mpgpu_loopbf(ctx, &fo, gpar.data(), nullptr, nullptr, &fs, nullptr, nullptr, nullptr);
        msLoopWall += msSince(tL);
        if (rc) break;
        res->msBuild = fs.msLoop;
        res->msLoops += fs.msLoop;
        if (monitor) {
            rc = mpgpu_get_monitor(ctx, monHist.data(), monMeas.data());
            monLoop = nloopn;
            if (!rc && (st->monitor < 0 || (nloopn == 1 && (st->monitor & 1)))) rc = writeMon(nloopn);
            if (rc) break;
        }
        nrejTot = 0;
        for (int k = 0; k < 6; ++k) { res->nrej[k] = fs.nrej[k]; nrejTot += fs.nrej[k]; }
        if (3 * nrejTot > job->nrec) { rc = MPGPU_ERR_TOOMANYREJ; break; }
        if (!pi.empty()) rc = mpgpu_mupdat(ctx, (int32_t)pi.size(), pi.data(), pj.data(), pa.data());
        if (rc) break;
        double chi2D = fs.chi2SumD;
        int64_t chi2I = fs.chi2SumI, ndfS = fs.ndfSum;
        // measurement lines (loopn, pede.f90:2743-2798)
        std::vector<int32_t> vi;   // their variable entries (each adds 1 to globalCounter)
        if (job->nmeas > 0) {
            std::vector<int32_t> mi, mj;
            std::vector<double> ma, va;
            for (int32_t m = 0; m < job->nmeas; ++m) {
                const double rhs = job->msRhs[m], sgm = job->msSigma[m];
                const double weight = sgm > 0.0 ? 1.0 / (sgm * sgm) : 0.0;
                double dsum = -rhs;
                const int32_t ia = job->msStart[m], ib = job->msStart[m + 1];
                for (int32_t q = ia; q < ib; ++q) {
                    int32_t li = find_label(lab, job->msLabel[q]);
                    if (li >= 0) dsum = dsum + job->msCoef[q] * gpar[li];
                }
                for (int32_t q = ia; q < ib; ++q) {
                    const double fj = job->msCoef[q];
                    if (fj == 0.0) continue;
                    int32_t li = find_label(lab, job->msLabel[q]);
                    const int32_t ivj = li >= 0 ? res->varIndex[li] : 0;
                    if (ivj <= 0) continue;
                    vi.push_back(ivj);
                    va.push_back(-weight * dsum * fj);
                    for (int32_t k = ia; k <= q; ++k) {
                        int32_t lk = find_label(lab, job->msLabel[k]);
                        const int32_t ivk = lk >= 0 ? res->varIndex[lk] : 0;
                        if (ivk > 0) { mi.push_back(ivj); mj.push_back(ivk); ma.push_back(weight * fj * job->msCoef[k]); }
                    }
                }
                const double add = weight * dsum * dsum;
                const int64_t nadd = (int64_t)add;
                chi2I += nadd;
                chi2D += add - (double)nadd;
                ndfS += 1;
            }
            rc = mpgpu_vector_add(ctx, (int32_t)vi.size(), vi.data(), va.data());
            if (!rc) rc = mpgpu_mupdat(ctx, (int32_t)mi.size(), mi.data(), mj.data(), ma.data());
            if (rc) break;
        }
        res->fvalue = chi2D + (double)chi2I;
        res->ndf = ndfS;
        rc = mpgpu_download_vector(ctx, nullptr, gcnt.data());
        if (rc) break;
        for (int32_t iv : vi) gcnt[iv - 1] += 1;
        // addcst: constraint residuals d - C p
        for (int32_t c = 0; c < ncon; ++c) {
            double rhs = job->conRhs ? job->conRhs[c] : 0.0;
            for (int32_t k = job->conStart[c]; k < job->conStart[c + 1]; ++k) {
                int32_t li = find_label(lab, job->conLabel[k]);
                if (li >= 0) rhs = rhs - job->conCoef[k] * gpar[li];
            }
            cres[c] = rhs;
        }
        mpgpu_solveinfo si;
        const bool wantErr = (st->metsol == 1 && iter == st->mitera);
        // minver saves the diagonal for the global correlations (pede.f90:7864-7866)
        if (wantErr && res->gcor) {
            rc = mpgpu_matrix_diagonal(ctx, diag0.data());
            if (rc) break;
        }
        const Clock::time_point tS = Clock::now();
        rc = mpgpu_solve(ctx, st->metsol, cres.data(), st->mrestl, st->itnlim, corr.data(),
                         wantErr ? err.data() : nullptr, &si);
        msSolveWall += msSince(tS);
        if (rc) break;
        res->msSolve = si.ms;
        res->msSolves += si.ms;
        res->nrank = si.nrank;
        res->minresItn = si.itn;
        res->minresIstop = si.istop;
        if (wantErr) haveErr = true;
        for (int32_t i = 0; i < nVar; ++i) {
            if (!(corr[i] <= 0.0) && !(corr[i] > 0.0)) { rc = MPGPU_ERR_NAN; break; }
            gpar[v2t[i]] += corr[i];
        }
        res->nloopn = nloopn;
        // the corrected parameters made feasible (cut 1e-6, pede.f90:8865-8866)
        if (!rc && ncon > 0) feasib(job, lab, res->varIndex, cfac, gpar, 1.0e-6f);
    }
    res->msHostIter = msSince(tIter) - msLoopWall - msSolveWall;
    if (!rc && monitor && st->monitor > 0 && (st->monitor & 2) && monLoop > 0) rc = writeMon(monLoop);
    for (int32_t i = 0; i < ntot; ++i) {
        res->parameter[i] = gpar[i];
        res->presigma[i] = psig[i];
        res->error[i] = 0.0;
        res->counts[i] = 0;
        if (res->start) res->start[i] = gstart[i];
        if (res->fileCounts) res->fileCounts[i] = counter[i];
        if (res->gcor) res->gcor[i] = -1.0;
        const int32_t iv = res->varIndex[i];
        if (iv > 0) {
            res->counts[i] = gcnt[iv - 1];
            if (haveErr && res->gcor) {
                // global correlation (prtglo, pede.f90:4537-4544)
                const double gmati = err[iv - 1], dg = diag0[iv - 1];
                if (gmati * dg > 0.0) {
                    const double gcor2 = 1.0 - 1.0 / (gmati * dg);
                    if (gcor2 >= 0.0 && gcor2 <= 1.0) res->gcor[i] = (double)(float)std::sqrt(gcor2);
                }
            }
            if (haveErr) {
                const double e = std::sqrt(std::fabs(err[iv - 1]));
                res->error[i] = err[iv - 1] < 0.0 ? -e : e;
            }
        }
    }
    res->exitCode = rc;
    if (!ctxIn) mpgpu_destroy(ctx);
    res->msJob = msSince(tJob);
    return rc;
}

extern "C" int32_t mpgpu_pede_run(mpgpu_ctx *ctx, const mpgpu_steer *st, const mpgpu_job *job,
                                  mpgpu_result *res) {
    return pede_run_admitted(ctx, st, job, res, nullptr);
}

namespace {
// Fortran G14.5 edit descriptor as used by prtglo (pede.f90:4643)
std::string fmt_g145(double v) {
    char t[64], f[64], out[64];
    if (v == 0.0) {
        snprintf(out, sizeof out, "%14s", "0.0000    ");
        return out;
    }
    snprintf(t, sizeof t, "%.4E", v);
    const char *e = std::strchr(t, 'E');
    const int ex = std::atoi(e + 1) + 1;  // v = 0.ddddd * 10^ex
    if (ex >= 0 && ex <= 5) {
        snprintf(f, sizeof f, "%.*f    ", 5 - ex, v);
    } else {
        std::string mant;
        for (const char *p = t; p < e; ++p)
            if (*p >= '0' && *p <= '9') mant += *p;
        snprintf(f, sizeof f, "%s0.%sE%c%02d", v < 0 ? "-" : "", mant.c_str(), ex < 0 ? '-' : '+',
                 ex < 0 ? -ex : ex);
    }
    snprintf(out, sizeof out, "%14s", f);
    return out;
}
}  // namespace

// millepede.res in the layout of prtglo (pede.f90:4477-4651, formats
// 102 and 110-112 at 4643-4650): label, value, pre-sigma and, for variable
// parameters, the difference to the start value and (inversion) the error,
// in single precision; optionally the entries (printcounts) or the global
// correlation (globalcorr).
extern "C" int32_t mpgpu_write_res_opts(const char *path, const mpgpu_result *res, const mpgpu_res_opts *o) {
    if (!path || !res || !o) return MPGPU_ERR_ARG;
    if (o->ipcntr < 0) return MPGPU_ERR_ARG;   // zero-derivative counts are not kept
    if (o->ipcntr > 1 && !res->fileCounts) return MPGPU_ERR_ARG;
    if (o->igcorr && o->errors && o->ipcntr == 0 && !res->gcor) return MPGPU_ERR_ARG;
    FILE *f = std::fopen(path, "w");
    if (!f) return MPGPU_ERR_ARG;
    std::fprintf(f, " Parameter   ! first 3 elements per line are significant (if used as input)\n");
    for (int32_t i = 0; i < res->nTotal; ++i) {
        const std::string a = fmt_g145((double)(float)res->parameter[i]);
        const std::string b = fmt_g145((double)(float)res->presigma[i]);
        const int32_t iv = res->varIndex[i];
        int64_t icount = 0;
        bool lowstat = false;
        if (iv > 0) {
            icount = res->counts[i];
            lowstat = icount < o->mreqena;
        }
        if (o->ipcntr > 1) icount = res->fileCounts[i];
        if (lowstat) icount = -(icount + 1);
        if (iv <= 0) {
            if (o->ipcntr != 0)
                std::fprintf(f, "%10d  %s%s%28s%12lld\n", res->labels[i], a.c_str(), b.c_str(), "", (long long)icount);
            else
                std::fprintf(f, "%10d  %s%s\n", res->labels[i], a.c_str(), b.c_str());
            continue;
        }
        const double start = res->start ? res->start[i] : 0.0;
        const std::string d = fmt_g145((double)(float)(res->parameter[i] - start));
        if (o->errors) {
            const std::string e = fmt_g145((double)(float)res->error[i]);
            if (o->ipcntr != 0)
                std::fprintf(f, "%10d  %s%s%s%s%12lld\n", res->labels[i], a.c_str(), b.c_str(), d.c_str(), e.c_str(),
                             (long long)icount);
            else if (o->igcorr)
                std::fprintf(f, "%10d  %s%s%s%s%8.3f\n", res->labels[i], a.c_str(), b.c_str(), d.c_str(), e.c_str(),
                             (double)(float)res->gcor[i]);
            else
                std::fprintf(f, "%10d  %s%s%s%s\n", res->labels[i], a.c_str(), b.c_str(), d.c_str(), e.c_str());
        } else {
            if (o->ipcntr != 0)
                std::fprintf(f, "%10d  %s%s%s%14s%12lld\n", res->labels[i], a.c_str(), b.c_str(), d.c_str(), "",
                             (long long)icount);
            else
                std::fprintf(f, "%10d  %s%s%s\n", res->labels[i], a.c_str(), b.c_str(), d.c_str());
        }
    }
    std::fclose(f);
    return 0;
}

extern "C" int32_t mpgpu_write_res(const char *path, const mpgpu_result *res, int32_t errors) {
    const mpgpu_res_opts o{errors, 0, 0, 0};
    return mpgpu_write_res_opts(path, res, &o);
}

// ------------------------------------------------------------------ monitor
extern "C" int32_t mpgpu_monitor_groups(int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                                        const double *glder, int32_t nTotal, int32_t *measIndex, double *measRes,
                                        int32_t *numMeas) {
    if (nrec < 0 || !recPtr || !inder || !glder || nTotal <= 0 || !measIndex || !measRes || !numMeas)
        return MPGPU_ERR_ARG;
    std::vector<int64_t> cnt(nTotal, 0);
    std::vector<double> sum(nTotal, 0.0);
    int32_t bad = 0;
    for (int64_t r = 0; r < nrec && !bad; ++r) {
        const bool ok = for_each_measurement(inder, glder, recPtr[r], recPtr[r + 1],
                                             [&](int64_t, int64_t sg, int64_t lg) {
                                                 if (lg <= sg) return;   // no global derivative
                                                 const int32_t ij = inder[sg + 1];
                                                 if (ij < 1 || ij > nTotal) { bad = 1; return; }
                                                 cnt[ij - 1]++;
                                                 sum[ij - 1] = sum[ij - 1] + glder[sg];
                                             });
        if (!ok) return MPGPU_ERR_BADRECORD;
    }
    if (bad) return MPGPU_ERR_BADINDEX;
    int32_t n = 0;
    for (int32_t i = 0; i < nTotal; ++i) {
        measIndex[i] = 0;
        if (cnt[i] > 0) {
            measRes[n] = sum[i] / (double)cnt[i];
            measIndex[i] = ++n;
        }
    }
    *numMeas = n;
    return MPGPU_OK;
}

// location (median) and scale (1.4826 x median absolute deviation) of one
// group's binned values as monres computes them: medians of the cumulative
// bin counts with linear interpolation inside the bin, the deviations by
// folding the bins around the median bin; single precision
extern "C" int32_t mpgpu_write_mon(const char *path, int32_t header, int32_t mode, int32_t nloopn, int32_t numMeas,
                                   const int32_t *groupLabel, const int64_t *measHists, int32_t measBins,
                                   const double *measRes) {
    if (!path || numMeas < 0 || measBins < 2 || (numMeas > 0 && (!groupLabel || !measHists || !measRes)))
        return MPGPU_ERR_ARG;
    FILE *f = std::fopen(path, "a");
    if (!f) return MPGPU_ERR_ARG;
    if (header) {
        std::fprintf(f, "%s\n", mode == 0 ? "*** Normalized residuals grouped by first global label (per local fit cycle) ***"
                                          : "*** Pulls grouped by first global label (per local fit cycle) ***");
        std::fprintf(f, "%s\n", "! LFC     Label   Entries        Median  RMS(MAD)          <error>");
    }
    const float binSize = 0.1f;
    std::vector<int64_t> isuml(measBins + 2), isums(measBins + 2);
    for (int32_t g = 0; g < numMeas; ++g) {
        const int64_t *h = measHists + (int64_t)g * measBins;   // h[j - 1]: bin j
        float amed = 0.0f, amad = 0.0f;
        isuml[1] = h[0];
        for (int32_t j = 2; j <= measBins; ++j) isuml[j] = isuml[j - 1] + h[j - 1];
        const int64_t nent = isuml[measBins];
        if (nent > 0) {
            int32_t j = 2;
            for (; j <= measBins; ++j)
                if (2 * isuml[j] > nent) break;
            const int32_t imed = j;
            amed = (float)j;
            if (j <= measBins && isuml[j] > isuml[j - 1])
                amed = amed + (float)(nent - 2 * isuml[j - 1]) / (float)(2 * isuml[j] - 2 * isuml[j - 1]);
            amed = binSize * (amed - (float)(measBins / 2));
            for (int32_t k = 0; k <= measBins; ++k) isums[k] = 0;
            for (int32_t jj = imed; jj <= measBins; ++jj) isums[jj - imed + 1] += h[jj - 1];
            for (int32_t jj = imed - 1; jj >= 1; --jj) isums[imed - jj] += h[jj - 1];
            for (int32_t k = 2; k <= measBins; ++k) isums[k] = isums[k] + isums[k - 1];
            for (j = 2; j <= measBins; ++j)
                if (2 * isums[j] > nent) break;
            amad = (float)(j - 1);
            if (j <= measBins && isums[j] > isums[j - 1])
                amad = amad + (float)(nent - 2 * isums[j - 1]) / (float)(2 * isums[j] - 2 * isums[j - 1]);
            amad = binSize * amad;
        }
        std::fprintf(f, "%5d%10d%10lld%s%s%s\n", nloopn, groupLabel[g], (long long)nent,
                     fmt_g145((double)amed).c_str(), fmt_g145((double)(amad * 1.4826f)).c_str(),
                     fmt_g145((double)(float)measRes[g]).c_str());
    }
    std::fclose(f);
    return MPGPU_OK;
}
