// mpgpu_api.cu -- the C-ABI entry points (include/mpgpu.h): context,
// layout, constraints, record upload, the data loop and the solver dispatch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "mpgpu_ctx.h"

// ------------------------------------------------------------------ errors
int32_t set_err(mpgpu_ctx *c, int32_t code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

int32_t cuda_err(mpgpu_ctx *c, cudaError_t e, const char *where) {
    if (c) c->err = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? MPGPU_ERR_ALLOC : MPGPU_ERR_CUDA;
}

namespace {

template <class T>
void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

template <class T>
cudaError_t dalloc(T *&p, int64_t n) {
    dfree(p);
    if (n <= 0) n = 1;
    return cudaMalloc((void **)&p, sizeof(T) * (size_t)n);
}

template <class T>
cudaError_t dupload(T *&p, const T *h, int64_t n, cudaStream_t s) {
    cudaError_t e = dalloc(p, n);
    if (e != cudaSuccess) return e;
    if (n > 0 && h) return cudaMemcpyAsync(p, h, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, s);
    return cudaSuccess;
}

int nthreads_host() {
    unsigned n = std::thread::hardware_concurrency();
    if (n < 1) n = 1;
    if (n > 64) n = 64;
    return (int)n;
}

template <class F>
void parallel_for(int64_t n, F f) {
    const int nt = nthreads_host();
    if (n < 4096 || nt == 1) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        int64_t a = n * t / nt, b = n * (t + 1) / nt;
        th.emplace_back([=, &f] { f(a, b, t); });
    }
    for (auto &x : th) x.join();
}

void free_records(DevJob &j) {
    dfree(j.inder); dfree(j.glder); dfree(j.rec); dfree(j.meas); dfree(j.slots);
    dfree(j.slotCnt); dfree(j.swStart); dfree(j.sw); dfree(j.grpId); dfree(j.grpSlot);
    dfree(j.fileWeight); dfree(j.status); dfree(j.chi2add); dfree(j.ndfadd); dfree(j.chndf);
    dfree(j.vstage); dfree(j.stage);
    dfree(j.bkI); dfree(j.bkJ); dfree(j.bkLd); dfree(j.bkOff);
    dfree(j.itBlk); dfree(j.itBase); dfree(j.itCnt); dfree(j.itSlot); dfree(j.pairDst);
    dfree(j.rdBlk); dfree(j.rdSlot0); dfree(j.rdN); dfree(j.partial);
    dfree(j.vEntries); dfree(j.vStart);
    j.chunkRec.clear();
    j.chunkItem.clear();
    j.chunkRed.clear();
    j.nrec = 0;
}

void free_layout(DevJob &j) {
    dfree(j.varOfTot); dfree(j.aig); dfree(j.p2g); dfree(j.off); dfree(j.col);
    dfree(j.matD); dfree(j.gvec); dfree(j.gcnt); dfree(j.gpar); dfree(j.work);
    dfree(j.rowBlk0); dfree(j.blkJ); dfree(j.blkOff); dfree(j.blkLd); dfree(j.blkCol);
    dfree(j.rowWidth);
}

void free_constraints(DevJob &j) {
    dfree(j.qlV); dfree(j.qlVk); dfree(j.qlR2);
    j.ncon = 0;
}

// decodeNextMeasurement (pede.f90:2428-2468) on one record; positions
// relative to the record start; returns false for a malformed record
struct Eq { int32_t sl, sg, lg; };
bool decode_record(const int32_t *in, const double *gl, int32_t nw, std::vector<Eq> &eqs) {
    eqs.clear();
    int32_t lg = 0;
    const int32_t end = nw - 1;
    for (;;) {
        if (lg >= end) return true;
        do { lg++; if (lg > end) return false; } while (in[lg] != 0);
        const int32_t sl = lg;
        do { lg++; if (lg > end) return false; } while (in[lg] != 0);
        const int32_t sg = lg;
        if (sl + 1 == sg && gl[sg] < 0.0) {
            lg = lg + (int32_t)(-gl[sg] + 0.5);  // special data block
            continue;
        }
        while (lg < end && in[lg + 1] != 0) lg++;
        eqs.push_back({sl, sg, lg});
    }
}

}  // namespace

// ------------------------------------------------------------------ context
extern "C" int32_t mpgpu_create(mpgpu_ctx **out, const mpgpu_cfg *cfg) {
    if (!out) return MPGPU_ERR_ARG;
    *out = nullptr;
    mpgpu_ctx *c = new mpgpu_ctx();
    c->device = cfg ? cfg->device : 0;
    c->stagingBytes = (cfg && cfg->staging_bytes > 0) ? cfg->staging_bytes : 0;  // 0: sized per job
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->scal, 4096);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&c->hscal, 4096);
    if (e != cudaSuccess) {
        int32_t rc = cuda_err(c, e, "mpgpu_create");
        delete c;
        return rc;
    }
    *out = c;
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_destroy(mpgpu_ctx *c) {
    if (!c) return MPGPU_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_records(c->j);
    free_layout(c->j);
    free_constraints(c->j);
    if (c->scal) cudaFree(c->scal);
    if (c->hscal) cudaFreeHost(c->hscal);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    delete c;
    return MPGPU_OK;
}

extern "C" const char *mpgpu_last_error(const mpgpu_ctx *c) { return c ? c->err.c_str() : ""; }

// ------------------------------------------------------------------ layout
extern "C" int32_t mpgpu_set_layout(mpgpu_ctx *c, int32_t nTotal, const int32_t *varIndexOfTotal,
                                    int32_t nVar, int32_t nGroups, const int32_t *allIndexGroups,
                                    int32_t matsto, const int64_t *sparseOffsets,
                                    const int32_t *sparseColumns, int64_t ncolw, int64_t nmat) {
    if (!c || nTotal <= 0 || nVar <= 0 || nGroups <= 0 || !varIndexOfTotal || !allIndexGroups)
        return set_err(c, MPGPU_ERR_ARG, "mpgpu_set_layout: bad arguments");
    if (matsto != 1 && matsto != 2) return set_err(c, MPGPU_ERR_ARG, "matsto must be 1 or 2");
    if (matsto == 2 && (!sparseOffsets || !sparseColumns))
        return set_err(c, MPGPU_ERR_ARG, "sparse storage needs offsets and columns");
    if (matsto == 1) nmat = (int64_t)nVar * (nVar + 1) / 2;
    if (allIndexGroups[nGroups] != nVar + 1) return set_err(c, MPGPU_ERR_SIZE, "groups do not end at nVar+1");
    cudaSetDevice(c->device);
    DevJob &j = c->j;
    free_layout(j);
    free_records(j);
    j.nTotal = nTotal; j.nVar = nVar; j.nG = nGroups; j.matsto = matsto;
    j.nmat = nmat; j.ncolw = ncolw;
    j.hAig.assign(allIndexGroups, allIndexGroups + nGroups + 1);
    std::vector<int32_t> p2g(nVar);
    for (int32_t g = 1; g <= nGroups; ++g)
        for (int32_t v = allIndexGroups[g - 1]; v < allIndexGroups[g]; ++v) {
            if (v < 1 || v > nVar) return set_err(c, MPGPU_ERR_SIZE, "bad group table");
            p2g[v - 1] = g;
        }
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(j.varOfTot, varIndexOfTotal, nTotal, s));
    MPG_CUDA(c, dupload(j.aig, allIndexGroups, nGroups + 1, s));
    MPG_CUDA(c, dupload(j.p2g, p2g.data(), nVar, s));
    if (matsto == 2) {
        MPG_CUDA(c, dupload(j.off, sparseOffsets, 2 * (int64_t)(nGroups + 1), s));
        MPG_CUDA(c, dupload(j.col, sparseColumns, ncolw, s));
    }
    // block rows (dense row layout of each row group; for the sparse storage
    // the blocks of sparseMatrixOffsets/Columns, ijpgrp pede.f90:5371-5461)
    {
        std::vector<int64_t> rowBlk0(nGroups + 1, 0), bOff;
        std::vector<int32_t> bJ, bLd, bCol, width(nGroups, 0);
        for (int32_t I = 1; I <= nGroups; ++I) {
            const int32_t np = allIndexGroups[I] - allIndexGroups[I - 1];
            if (matsto == 2) {
                const int64_t kk = sparseOffsets[2 * (I - 1)], ll = sparseOffsets[2 * (I - 1) + 1];
                const int64_t ku = sparseOffsets[2 * I] - kk;
                if (ku > 0 && sparseColumns[kk] != 0) {
                    int64_t k = 0;
                    while (k < ku) {
                        const int32_t first = sparseColumns[kk + k];
                        if (first < 1 || first > nVar) return set_err(c, MPGPU_ERR_SIZE, "bad sparse columns");
                        const int32_t J = p2g[first - 1];
                        const int32_t nj = allIndexGroups[J] - allIndexGroups[J - 1];
                        bJ.push_back(J); bOff.push_back(ll + k); bLd.push_back((int32_t)ku);
                        bCol.push_back((int32_t)k);
                        k += nj;
                    }
                    width[I - 1] = (int32_t)ku;
                } else if (ku > 0) {
                    for (int64_t k = 2; k <= ku - 2; k += 2) {
                        const int32_t o0 = sparseColumns[kk + k - 2], g0 = sparseColumns[kk + k - 1];
                        const int32_t o1 = sparseColumns[kk + k];
                        int32_t inreg = 0, J = g0;
                        while (inreg < o1 - o0) {
                            if (J < 1 || J > nGroups) return set_err(c, MPGPU_ERR_SIZE, "bad sparse regions");
                            const int32_t nj = allIndexGroups[J] - allIndexGroups[J - 1];
                            bJ.push_back(J); bOff.push_back(ll + (int64_t)o0 * np + inreg);
                            bLd.push_back(o1 - o0); bCol.push_back(o0 + inreg);
                            inreg += nj;
                            J++;
                        }
                        width[I - 1] = o1;
                    }
                }
            } else {
                width[I - 1] = allIndexGroups[I] - 1;
            }
            rowBlk0[I] = (int64_t)bJ.size();
        }
        j.hRowWidth = width;
        j.hRowBlk0 = rowBlk0;
        j.hBlkJ = bJ;
        j.hBlkOff = bOff;
        j.hBlkLd = bLd;
        MPG_CUDA(c, dupload(j.rowWidth, width.data(), nGroups, s));
        if (matsto == 2) {
            MPG_CUDA(c, dupload(j.rowBlk0, rowBlk0.data(), nGroups + 1, s));
            MPG_CUDA(c, dupload(j.blkJ, bJ.data(), (int64_t)bJ.size(), s));
            MPG_CUDA(c, dupload(j.blkOff, bOff.data(), (int64_t)bOff.size(), s));
            MPG_CUDA(c, dupload(j.blkLd, bLd.data(), (int64_t)bLd.size(), s));
            MPG_CUDA(c, dupload(j.blkCol, bCol.data(), (int64_t)bCol.size(), s));
            MPG_CUDA(c, cudaStreamSynchronize(s));
        }
    }
    MPG_CUDA(c, dalloc(j.matD, nmat));
    MPG_CUDA(c, cudaMemsetAsync(j.matD, 0, sizeof(double) * (size_t)nmat, s));
    MPG_CUDA(c, dalloc(j.gvec, nVar));
    MPG_CUDA(c, dalloc(j.gcnt, nVar));
    MPG_CUDA(c, dalloc(j.gpar, nTotal));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    return MPGPU_OK;
}

// ------------------------------------------------------------------ constraints
// QL decomposition of the constraint matrix (qldec, mpqldec.f90:125-196,
// one parameter block) done on the host at set-up; the Householder vectors
// stay on the device for the Q / Q^T products of every solve.
extern "C" int32_t mpgpu_set_constraints(mpgpu_ctx *c, int32_t ncon, const double *A) {
    if (!c) return MPGPU_ERR_ARG;
    DevJob &j = c->j;
    if (j.nVar <= 0) return set_err(c, MPGPU_ERR_ARG, "set the layout before the constraints");
    free_constraints(j);
    if (ncon <= 0) return MPGPU_OK;
    if (ncon >= j.nVar) return set_err(c, MPGPU_ERR_SIZE, "more constraints than parameters");
    const int32_t npar = j.nVar;
    std::vector<double> V(A, A + (size_t)ncon * npar), L((size_t)ncon * ncon, 0.0), Vk(ncon, 0.0);
    std::vector<int32_t> r1(ncon, 1), r2(ncon, 0);
    std::vector<double> vn(npar);
    for (int32_t k = ncon; k >= 1; --k) {
        const int32_t kn = npar + k - ncon;
        double *row = &V[(size_t)(k - 1) * npar];
        double nrm = 0.0;
        for (int32_t q = 0; q < kn; ++q) { vn[q] = row[q]; nrm = nrm + vn[q] * vn[q]; }
        nrm = std::sqrt(nrm);
        if (nrm == 0.0) return set_err(c, MPGPU_ERR_QL, "empty constraint");
        if (vn[kn - 1] >= 0.0) vn[kn - 1] = vn[kn - 1] + nrm;
        else vn[kn - 1] = vn[kn - 1] - nrm;
        nrm = 0.0;
        for (int32_t q = 0; q < kn; ++q) nrm = nrm + vn[q] * vn[q];
        nrm = std::sqrt(nrm);
        for (int32_t q = 0; q < kn; ++q) vn[q] = vn[q] / nrm;
        for (int32_t i = 1; i <= k; ++i) {
            double *ri = &V[(size_t)(i - 1) * npar];
            double sp = 0.0;
            for (int32_t q = 0; q < kn; ++q) sp = sp + vn[q] * ri[q];
            for (int32_t q = 0; q < kn; ++q) ri[q] = ri[q] - 2.0 * vn[q] * sp;
        }
        for (int32_t cc = k; cc <= ncon; ++cc) L[(size_t)(k - 1) * ncon + cc - 1] = row[kn - 1 + cc - k];
        for (int32_t q = 0; q < kn - 1; ++q) row[q] = vn[q];
        for (int32_t q = kn - 1; q < npar; ++q) row[q] = 0.0;
        r2[k - 1] = kn - 1;
        Vk[k - 1] = vn[kn - 1];
    }
    for (int32_t k = 0; k < ncon; ++k)
        if (L[(size_t)k * ncon + k] == 0.0) return set_err(c, MPGPU_ERR_QL, "singular constraints");
    j.ncon = ncon;
    j.hV = V; j.hVk = Vk; j.hL = L; j.hR1 = r1; j.hR2 = r2;
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(j.qlV, V.data(), (int64_t)ncon * npar, s));
    MPG_CUDA(c, dupload(j.qlVk, Vk.data(), ncon, s));
    MPG_CUDA(c, dupload(j.qlR2, r2.data(), ncon, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    return MPGPU_OK;
}

// ------------------------------------------------------------------ records
// One host pass builds the per-record tables the kernels need (measurement
// boundaries, sorted variable parameters, parameter groups, band structure
// of the local matrix, owner lists per parameter group); the records then
// stay resident on the device for all data loops of the job.
extern "C" int32_t mpgpu_upload_records(mpgpu_ctx *c, int64_t nrec, const int64_t *recPtr,
                                        const int32_t *inder, const double *glder,
                                        const int32_t *recFile, int32_t nfiles,
                                        const double *fileWeight) {
    if (!c || nrec < 0 || !recPtr || !inder || !glder) return MPGPU_ERR_ARG;
    DevJob &j = c->j;
    if (j.nVar <= 0) return set_err(c, MPGPU_ERR_ARG, "set the layout before the records");
    cudaSetDevice(c->device);
    free_records(j);
    if (nfiles < 1) nfiles = 1;
    j.nfiles = nfiles;
    j.nrec = nrec;
    j.nw = recPtr[nrec] - recPtr[0];
    const int32_t nVar = j.nVar, nTotal = j.nTotal;
    std::vector<int32_t> varOfTot(nTotal);
    MPG_CUDA(c, cudaMemcpy(varOfTot.data(), j.varOfTot, sizeof(int32_t) * nTotal, cudaMemcpyDeviceToHost));
    const std::vector<int32_t> &aig = j.hAig;
    std::vector<int32_t> p2g(nVar);
    for (int32_t g = 1; g <= j.nG; ++g)
        for (int32_t v = aig[g - 1]; v < aig[g]; ++v) p2g[v - 1] = g;

    // ---- pass A: sizes and structure per record
    std::vector<RecInfo> rec(nrec);
    std::vector<int32_t> errRec(nthreads_host() + 1, 0);
    std::vector<int64_t> errAt(nthreads_host() + 1, -1);
    parallel_for(nrec, [&](int64_t a, int64_t b, int t) {
        std::vector<Eq> eqs;
        std::vector<int32_t> stamp(nVar + 1, 0), ibandh, eqStamp(nVar + 1, 0);
        std::vector<int32_t> gStamp(j.nG + 1, 0), gCnt(j.nG + 1, 0), eqGroups;
        int32_t eqTag = 0;
        std::vector<int32_t> sl;
        for (int64_t r = a; r < b; ++r) {
            RecInfo &ri = rec[r];
            memset(&ri, 0, sizeof(ri));
            const int64_t w0 = recPtr[r];
            const int64_t nw64 = recPtr[r + 1] - w0;
            const int32_t *in = inder + w0;
            const double *gl = glder + w0;
            ri.w0 = w0 - recPtr[0];
            ri.file = recFile ? recFile[r] : 1;
            if (nw64 < 1 || nw64 > MPG_WORDS_MAX || ri.file < 1 || ri.file > nfiles ||
                !decode_record(in, gl, (int32_t)nw64, eqs)) {
                errRec[t] = MPGPU_ERR_BADRECORD; errAt[t] = r; return;
            }
            ri.nw = (int32_t)nw64;
            ri.neq = (int32_t)eqs.size();
            int32_t nalc = 0, nalg = 0, nsw = 0;
            bool nonmono = false;
            sl.clear();
            for (const Eq &e : eqs) {
                int32_t prev = 0;
                for (int32_t q = e.sl + 1; q < e.sg; ++q) {
                    const int32_t li = in[q];
                    if (li <= 0) { errRec[t] = MPGPU_ERR_BADRECORD; errAt[t] = r; return; }
                    if (li > nalc) nalc = li;
                    if (li <= prev) nonmono = true;
                    prev = li;
                }
                for (int32_t q = e.sg + 1; q <= e.lg; ++q) {
                    const int32_t ti = in[q];
                    if (ti < 1 || ti > nTotal) { errRec[t] = MPGPU_ERR_BADINDEX; errAt[t] = r; return; }
                    const int32_t v = varOfTot[ti - 1];
                    if (v > 0) {
                        nsw++;
                        if (stamp[v] != (int32_t)(r - a + 1)) { stamp[v] = (int32_t)(r - a + 1); sl.push_back(v); }
                    }
                }
            }
            nalg = (int32_t)sl.size();
            ri.nalc = nalc;
            ri.nalg = nalg;
            // every equation carries the local derivatives 1..nalc in order
            // (fast normal equations); no variable parameter twice in one
            // equation (lockstep word lists in the update)
            bool denseLoc = nalc > 0, simpleWords = true;
            for (const Eq &e : eqs) {
                if (e.sg - e.sl - 1 != nalc) denseLoc = false;
                for (int32_t q = e.sl + 1; denseLoc && q < e.sg; ++q)
                    if (in[q] != q - e.sl) denseLoc = false;
                // ... and every group it touches complete (then all slots of a
                // group have the same equation list)
                ++eqTag;
                eqGroups.clear();
                for (int32_t q = e.sg + 1; q <= e.lg; ++q) {
                    const int32_t v = varOfTot[in[q] - 1];
                    if (v <= 0) continue;
                    if (eqStamp[v] == eqTag) simpleWords = false;
                    eqStamp[v] = eqTag;
                    const int32_t g = p2g[v - 1];
                    if (gStamp[g] != eqTag) { gStamp[g] = eqTag; gCnt[g] = 0; eqGroups.push_back(g); }
                    gCnt[g]++;
                }
                for (int32_t g : eqGroups)
                    if (gCnt[g] != aig[g] - aig[g - 1]) simpleWords = false;
            }
            // groups of the sorted variable parameters; the record must hold
            // complete groups (loopbf's npar == nalg check, pede.f90:3710-3724)
            std::sort(sl.begin(), sl.end());
            int32_t ngrp = 0, prevg = -1, npar = 0;
            for (int32_t v : sl) {
                const int32_t g = p2g[v - 1];
                if (g != prevg) { ngrp++; prevg = g; npar += aig[g] - aig[g - 1]; }
            }
            if (nalc > 0 && npar != nalg) { errRec[t] = MPGPU_ERR_GROUPS; errAt[t] = r; return; }
            if (ngrp > MPG_NGRP_MAX) { errRec[t] = MPGPU_ERR_LIMIT; errAt[t] = r; return; }
            ri.ngrp = ngrp;
            // bordered band structure of the local matrix (pede.f90:3812-3874)
            ri.mbnd = -1; ri.mbdr = (int16_t)nalc; ri.mside = -1;
            if (nalc > 5) {
                ibandh.assign(2 * nalc + 2, 0);
                for (const Eq &e : eqs)
                    for (int32_t jq = e.sl + 1; jq < e.sg; ++jq)
                        for (int32_t kq = e.sl + 1; kq <= jq; ++kq) {
                            const int32_t ij = in[jq], ik = in[kq];
                            const int32_t id = std::abs(ij - ik) + 1;
                            int32_t im = std::min(ij, ik);
                            ibandh[id] = std::max(ibandh[id], im);
                            im = std::min(nalc + 1 - ij, nalc + 1 - ik);
                            ibandh[nalc + id] = std::max(ibandh[nalc + id], im);
                        }
                int32_t kx = -1, kbdrx = 0, kbdr = 0, side = -1;
                int64_t icmn = (int64_t)nalc * nalc * nalc;
                for (int32_t k = nalc; k >= 2; --k) {
                    const int32_t kbnd = k - 2;
                    kbdr = std::max(kbdr, ibandh[k]);
                    const int64_t w = kbnd + kbdr + 1;
                    const int64_t icost = 6 * (int64_t)(nalc - kbdr) * w * w + 2 * (int64_t)kbdr * kbdr * kbdr;
                    if (icost < icmn) { icmn = icost; kx = k; kbdrx = kbdr; side = 1; }
                }
                if (kx < 0) {
                    kbdr = 0;
                    for (int32_t k = nalc; k >= 2; --k) {
                        const int32_t kbnd = k - 2;
                        kbdr = std::max(kbdr, ibandh[k + nalc]);
                        const int64_t w = kbnd + kbdr + 1;
                        const int64_t icost = 6 * (int64_t)(nalc - kbdr) * w * w + 2 * (int64_t)kbdr * kbdr * kbdr;
                        if (icost < icmn) { icmn = icost; kx = k; kbdrx = kbdr; side = 2; }
                    }
                }
                if (kx > 0) { ri.mbnd = (int16_t)(kx - 2); ri.mbdr = (int16_t)kbdrx; ri.mside = side; }
            }
            ri.mside = (ri.mside & 0xff) | (nonmono ? 0x100 : 0) | (denseLoc ? 0x200 : 0) |
                       (simpleWords ? 0x400 : 0);
            ri.measOff = nsw;  // temporarily: number of slot words
        }
    });
    for (size_t t = 0; t < errRec.size(); ++t)
        if (errRec[t]) {
            char buf[128];
            snprintf(buf, sizeof buf, "record %lld rejected at upload (code %d)", (long long)errAt[t], errRec[t]);
            return set_err(c, errRec[t], buf);
        }

    // ---- pass B: offsets, maxima, chunks by staging size
    int64_t neqT = 0, nslotT = 0, nswT = 0, ngrpT = 0;
    j.maxNw = j.maxNeq = j.maxNalc = j.maxNalg = 0;
    j.maxBand = -1; j.maxBdr = 0; j.maxNgrp = 1;
    j.nbndr[0] = j.nbndr[1] = 0; j.nbdrx = j.nbndx = 0;
    int64_t stageElems = std::max<int64_t>(c->stagingBytes / 8, 1);
    if (c->stagingBytes <= 0) {
        // sized per job: all updates of the loop in one chunk when that fits
        // in the free device memory left after the record tables (estimated
        // generously as twice the record words), else two chunk buffers of
        // half the room each
        int64_t need = 0;
        for (int64_t r = 0; r < nrec; ++r)
            if (rec[r].nalc > 0) need += (int64_t)rec[r].nalg * (rec[r].nalg + 1) / 2;
        size_t freeB = 0, totalB = 0;
        MPG_CUDA(c, cudaMemGetInfo(&freeB, &totalB));
        const int64_t others = 2 * 12 * j.nw + (int64_t)nrec * 512 + ((int64_t)1 << 30);
        const int64_t room = std::max<int64_t>(((int64_t)freeB - others) / 10 * 9, (int64_t)256 << 20);
        stageElems = need * 8 <= room ? std::max<int64_t>(need, 1) : room / 16;
    }
    j.chunkRec.assign(1, 0);
    int64_t upd = 0, maxStage = 0;
    for (int64_t r = 0; r < nrec; ++r) {
        RecInfo &ri = rec[r];
        const int64_t nsw = ri.measOff;
        ri.measOff = neqT; neqT += ri.neq;
        ri.slotOff = nslotT; nslotT += ri.nalg + 1;
        ri.swOff = nswT; nswT += nsw;
        ri.grpOff = ngrpT; ngrpT += ri.ngrp;
        // records without local parameters leave no update in the staging
        const int64_t ngg = ri.nalc > 0 ? (int64_t)ri.nalg * (ri.nalg + 1) / 2 : 0;
        if (ngg > stageElems) return set_err(c, MPGPU_ERR_LIMIT, "record update larger than the staging buffer");
        if (upd + ngg > stageElems) { j.chunkRec.push_back(r); maxStage = std::max(maxStage, upd); upd = 0; }
        upd += ngg;
        j.maxNgrp = std::max(j.maxNgrp, ri.ngrp);
        j.maxNw = std::max(j.maxNw, ri.nw);
        j.maxNeq = std::max(j.maxNeq, ri.neq);
        j.maxNalc = std::max(j.maxNalc, ri.nalc);
        j.maxNalg = std::max(j.maxNalg, ri.nalg);
        if (ri.mbnd >= 0) {
            j.maxBand = std::max<int32_t>(j.maxBand, ri.mbnd);
            j.maxBdr = std::max<int32_t>(j.maxBdr, ri.mbdr);
            j.nbndr[(ri.mside & 0xff) - 1]++;
            j.nbdrx = std::max<int32_t>(j.nbdrx, ri.mbdr);
            j.nbndx = std::max<int32_t>(j.nbndx, ri.mbnd);
        }
    }
    j.chunkRec.push_back(nrec);
    maxStage = std::max(maxStage, upd);
    j.neqTot = neqT; j.nslotTot = nslotT; j.nswTot = nswT; j.ngrpTot = ngrpT;
    if (j.maxNalc > MPG_NALC_MAX) return set_err(c, MPGPU_ERR_LIMIT, "local system larger than the fit kernel limit");

    // ---- pass C: fill the tables
    std::vector<int32_t> meas(3 * neqT), slots(nslotT), slotCnt(nslotT), swStart(nslotT), sw(nswT);
    std::vector<int32_t> grpId(ngrpT), grpSlot(ngrpT);
    parallel_for(nrec, [&](int64_t a, int64_t b, int) {
        std::vector<Eq> eqs;
        std::vector<int32_t> pos(nVar + 1, -1), cnt;
        for (int64_t r = a; r < b; ++r) {
            const RecInfo &ri = rec[r];
            const int32_t *in = inder + recPtr[r];
            const double *gl = glder + recPtr[r];
            decode_record(in, gl, ri.nw, eqs);
            for (int32_t e = 0; e < ri.neq; ++e) {
                meas[3 * (ri.measOff + e)] = eqs[e].sl;
                meas[3 * (ri.measOff + e) + 1] = eqs[e].sg;
                meas[3 * (ri.measOff + e) + 2] = eqs[e].lg;
            }
            // sorted slots
            int32_t *sl = &slots[ri.slotOff];
            int32_t n = 0;
            for (const Eq &e : eqs)
                for (int32_t q = e.sg + 1; q <= e.lg; ++q) {
                    const int32_t v = varOfTot[in[q] - 1];
                    if (v > 0 && pos[v] < 0) { pos[v] = 0; sl[n++] = v; }
                }
            std::sort(sl, sl + n);
            sl[n] = 0;
            for (int32_t s = 0; s < n; ++s) pos[sl[s]] = s;
            // word lists per slot, in equation order (counting sort)
            cnt.assign(n + 1, 0);
            int32_t *cs = &slotCnt[ri.slotOff];
            for (int32_t s = 0; s <= n; ++s) cs[s] = 0;
            for (const Eq &e : eqs)
                for (int32_t q = e.sg + 1; q <= e.lg; ++q) {
                    const int32_t v = varOfTot[in[q] - 1];
                    if (v > 0) {
                        cnt[pos[v] + 1]++;
                        if (gl[q] != 0.0) cs[pos[v]]++;
                    }
                }
            int32_t *ss = &swStart[ri.slotOff];
            ss[0] = 0;
            for (int32_t s = 0; s < n; ++s) ss[s + 1] = ss[s] + cnt[s + 1];
            std::vector<int32_t> fillp(ss, ss + n);
            for (int32_t e = 0; e < ri.neq; ++e)
                for (int32_t q = eqs[e].sg + 1; q <= eqs[e].lg; ++q) {
                    const int32_t v = varOfTot[in[q] - 1];
                    if (v > 0) sw[ri.swOff + fillp[pos[v]]++] = (e << 16) | q;
                }
            // groups
            int32_t g = 0, prevg = -1;
            for (int32_t s = 0; s < n; ++s) {
                const int32_t gg = p2g[sl[s] - 1];
                if (gg != prevg) {
                    grpId[ri.grpOff + g] = gg;
                    grpSlot[ri.grpOff + g] = s;
                    g++;
                    prevg = gg;
                }
            }
            for (int32_t s = 0; s < n; ++s) pos[sl[s]] = -1;
        }
    });

    // ---- pass D: blocks of the global matrix met in the records
    const int64_t nchunk = (int64_t)j.chunkRec.size() - 1;
    const int32_t nG = j.nG;
    std::vector<int64_t> pairOff(nrec + 1, 0);
    for (int64_t r = 0; r < nrec; ++r) {
        const int64_t ng = rec[r].nalc > 0 ? rec[r].ngrp : 0;
        rec[r].pairOff = pairOff[r];
        pairOff[r + 1] = pairOff[r] + ng * (ng + 1) / 2;
    }
    const int64_t npairs = pairOff[nrec];
    std::vector<int32_t> bkI, bkJ, bkLd;
    std::vector<int64_t> bkOff, packedKey;
    if (j.matsto == 2) {
        const int64_t nb = (int64_t)j.hBlkJ.size();
        bkI.resize(nb);
        for (int32_t I = 1; I <= nG; ++I)
            for (int64_t k = j.hRowBlk0[I - 1]; k < j.hRowBlk0[I]; ++k) bkI[k] = I;
        bkJ = j.hBlkJ;
        bkLd = j.hBlkLd;
        bkOff = j.hBlkOff;
    } else {
        // packed storage: the group pairs that occur in records
        std::vector<std::vector<int64_t>> keys(nthreads_host());
        parallel_for(nrec, [&](int64_t a, int64_t b, int t) {
            std::vector<int64_t> &kv = keys[t];
            for (int64_t r = a; r < b; ++r) {
                if (rec[r].nalc <= 0) continue;
                for (int32_t qa = 0; qa < rec[r].ngrp; ++qa)
                    for (int32_t qb = 0; qb <= qa; ++qb)
                        kv.push_back((int64_t)grpId[rec[r].grpOff + qa] * (nG + 1) + grpId[rec[r].grpOff + qb]);
                if (kv.size() > (1u << 24)) {
                    std::sort(kv.begin(), kv.end());
                    kv.erase(std::unique(kv.begin(), kv.end()), kv.end());
                }
            }
            std::sort(kv.begin(), kv.end());
            kv.erase(std::unique(kv.begin(), kv.end()), kv.end());
        });
        for (auto &kv : keys) packedKey.insert(packedKey.end(), kv.begin(), kv.end());
        std::sort(packedKey.begin(), packedKey.end());
        packedKey.erase(std::unique(packedKey.begin(), packedKey.end()), packedKey.end());
        for (int64_t key : packedKey) {
            bkI.push_back((int32_t)(key / (nG + 1)));
            bkJ.push_back((int32_t)(key % (nG + 1)));
            bkLd.push_back(0);
            bkOff.push_back(0);
        }
    }
    const int64_t nblk = (int64_t)bkI.size();
    // block of every record pair (a >= b)
    std::vector<int32_t> pairBlk(std::max<int64_t>(npairs, 1));
    std::vector<int> pbad(nthreads_host() + 1, 0);
    parallel_for(nrec, [&](int64_t a, int64_t b, int t) {
        for (int64_t r = a; r < b; ++r) {
            if (rec[r].nalc <= 0) continue;
            int64_t q = pairOff[r];
            for (int32_t qa = 0; qa < rec[r].ngrp; ++qa) {
                const int32_t I = grpId[rec[r].grpOff + qa];
                for (int32_t qb = 0; qb <= qa; ++qb) {
                    const int32_t J = grpId[rec[r].grpOff + qb];
                    int64_t k = -1;
                    if (j.matsto == 2) {
                        auto b0 = j.hBlkJ.begin() + j.hRowBlk0[I - 1], b1 = j.hBlkJ.begin() + j.hRowBlk0[I];
                        auto itb = std::lower_bound(b0, b1, J);
                        if (itb != b1 && *itb == J) k = itb - j.hBlkJ.begin();
                    } else {
                        const int64_t key = (int64_t)I * (nG + 1) + J;
                        auto itb = std::lower_bound(packedKey.begin(), packedKey.end(), key);
                        k = itb - packedKey.begin();
                    }
                    if (k < 0) { pbad[t] = 1; k = 0; }
                    pairBlk[q++] = (int32_t)k;
                }
            }
        }
    });
    for (int v : pbad)
        if (v) return set_err(c, MPGPU_ERR_BADINDEX, "record group pair not in the sparse structure");
    int32_t maxEl = 1;
    for (int64_t k = 0; k < nblk; ++k) {
        const int32_t ni = aig[bkI[k]] - aig[bkI[k] - 1], nj = aig[bkJ[k]] - aig[bkJ[k] - 1];
        maxEl = std::max(maxEl, bkI[k] == bkJ[k] ? ni * (ni + 1) / 2 : ni * nj);
    }
    j.pstride = maxEl;
    // per chunk: staging position of every record block (the records of one
    // global-matrix block contiguous in record order), work items and
    // reduction lists; vector entries per row group in record order
    std::vector<int64_t> nelOf(std::max<int64_t>(nblk, 1));
    for (int64_t k = 0; k < nblk; ++k) {
        const int32_t ni = aig[bkI[k]] - aig[bkI[k] - 1], nj = aig[bkJ[k]] - aig[bkJ[k] - 1];
        nelOf[k] = bkI[k] == bkJ[k] ? (int64_t)ni * (ni + 1) / 2 : (int64_t)ni * nj;
    }
    std::vector<int64_t> pairDst(std::max<int64_t>(npairs, 1));
    std::vector<int32_t> itBlk, itCnt, rdBlk, rdN;
    std::vector<int64_t> itBase, itSlot, rdSlot0;
    int64_t nvent = 0;
    for (int64_t r = 0; r < nrec; ++r) if (rec[r].nalc > 0) nvent += rec[r].ngrp;
    std::vector<int64_t> vEntries(std::max<int64_t>(nvent, 1)), vStart((size_t)nchunk * (nG + 1));
    j.chunkItem.assign(1, 0);
    j.chunkRed.assign(1, 0);
    int64_t maxSlots = 1, vbase = 0;
    std::vector<int64_t> cnt(nblk + 1), bBase(nblk + 1);
    for (int64_t ch = 0; ch < nchunk; ++ch) {
        const int64_t r0 = j.chunkRec[ch], r1 = j.chunkRec[ch + 1];
        const int64_t p0 = pairOff[r0], p1 = pairOff[r1];
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int64_t q = p0; q < p1; ++q) cnt[pairBlk[q]]++;
        bBase[0] = 0;
        for (int64_t k = 0; k < nblk; ++k) bBase[k + 1] = bBase[k] + cnt[k] * nelOf[k];
        if (bBase[nblk] > maxStage) return set_err(c, MPGPU_ERR_LIMIT, "staging layout exceeds the chunk size");
        std::vector<int64_t> fill(bBase.begin(), bBase.end() - 1);
        for (int64_t q = p0; q < p1; ++q) {
            const int32_t k = pairBlk[q];
            pairDst[q] = fill[k];
            fill[k] += nelOf[k];
        }
        int64_t slot = 0;
        for (int64_t k = 0; k < nblk; ++k) {
            const int64_t n = cnt[k];
            if (n <= 0) continue;
            const int64_t nel = std::max<int64_t>(nelOf[k], 1);
            const int64_t per = std::max<int64_t>(32, 16384 / nel);
            const int64_t nitem = (n + per - 1) / per;
            for (int64_t m = 0; m < nitem; ++m) {
                itBlk.push_back((int32_t)k);
                itBase.push_back(bBase[k] + m * per * nelOf[k]);
                itCnt.push_back((int32_t)std::min(per, n - m * per));
                itSlot.push_back(nitem > 1 ? slot + m : -1);
            }
            if (nitem > 1) {
                rdBlk.push_back((int32_t)k);
                rdSlot0.push_back(slot);
                rdN.push_back((int32_t)nitem);
                slot += nitem;
            }
        }
        maxSlots = std::max(maxSlots, slot);
        j.chunkItem.push_back((int64_t)itBlk.size());
        j.chunkRed.push_back((int64_t)rdBlk.size());
        // vector entries of the chunk by row group
        int64_t *vs = &vStart[(size_t)ch * (nG + 1)];
        std::vector<int64_t> vc(nG + 1, 0);
        for (int64_t r = r0; r < r1; ++r)
            if (rec[r].nalc > 0)
                for (int32_t qa = 0; qa < rec[r].ngrp; ++qa) vc[grpId[rec[r].grpOff + qa]]++;
        vs[0] = vbase;
        for (int32_t g = 1; g <= nG; ++g) vs[g] = vs[g - 1] + vc[g];
        std::vector<int64_t> vf(vs, vs + nG);
        for (int64_t r = r0; r < r1; ++r)
            if (rec[r].nalc > 0)
                for (int32_t qa = 0; qa < rec[r].ngrp; ++qa) {
                    const int32_t g = grpId[rec[r].grpOff + qa];
                    vEntries[vf[g - 1]++] = (r << 40) | (rec[r].slotOff + grpSlot[rec[r].grpOff + qa]);
                }
        vbase = vs[nG];
    }

    // ---- upload
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(j.inder, inder + recPtr[0], j.nw, s));
    MPG_CUDA(c, dupload(j.glder, glder + recPtr[0], j.nw, s));
    MPG_CUDA(c, dupload(j.rec, rec.data(), nrec, s));
    MPG_CUDA(c, dupload(j.meas, meas.data(), 3 * neqT, s));
    MPG_CUDA(c, dupload(j.slots, slots.data(), nslotT, s));
    MPG_CUDA(c, dupload(j.slotCnt, slotCnt.data(), nslotT, s));
    MPG_CUDA(c, dupload(j.swStart, swStart.data(), nslotT, s));
    MPG_CUDA(c, dupload(j.sw, sw.data(), nswT, s));
    MPG_CUDA(c, dupload(j.grpId, grpId.data(), ngrpT, s));
    MPG_CUDA(c, dupload(j.grpSlot, grpSlot.data(), ngrpT, s));
    j.nblk = nblk;
    MPG_CUDA(c, dupload(j.bkI, bkI.data(), nblk, s));
    MPG_CUDA(c, dupload(j.bkJ, bkJ.data(), nblk, s));
    MPG_CUDA(c, dupload(j.bkLd, bkLd.data(), nblk, s));
    MPG_CUDA(c, dupload(j.bkOff, bkOff.data(), nblk, s));
    MPG_CUDA(c, dupload(j.pairDst, pairDst.data(), npairs, s));
    MPG_CUDA(c, dupload(j.itBlk, itBlk.data(), (int64_t)itBlk.size(), s));
    MPG_CUDA(c, dupload(j.itBase, itBase.data(), (int64_t)itBase.size(), s));
    MPG_CUDA(c, dupload(j.itCnt, itCnt.data(), (int64_t)itCnt.size(), s));
    MPG_CUDA(c, dupload(j.itSlot, itSlot.data(), (int64_t)itSlot.size(), s));
    MPG_CUDA(c, dupload(j.rdBlk, rdBlk.data(), (int64_t)rdBlk.size(), s));
    MPG_CUDA(c, dupload(j.rdSlot0, rdSlot0.data(), (int64_t)rdSlot0.size(), s));
    MPG_CUDA(c, dupload(j.rdN, rdN.data(), (int64_t)rdN.size(), s));
    MPG_CUDA(c, dupload(j.vEntries, vEntries.data(), nvent, s));
    MPG_CUDA(c, dupload(j.vStart, vStart.data(), (int64_t)vStart.size(), s));
    j.partialLen = maxSlots * j.pstride;
    MPG_CUDA(c, dalloc(j.partial, j.partialLen));
    std::vector<double> fw(nfiles, 1.0);
    if (fileWeight) fw.assign(fileWeight, fileWeight + nfiles);
    MPG_CUDA(c, dupload(j.fileWeight, fw.data(), nfiles, s));
    MPG_CUDA(c, dalloc(j.status, nrec));
    MPG_CUDA(c, dalloc(j.chi2add, nrec));
    MPG_CUDA(c, dalloc(j.ndfadd, nrec));
    MPG_CUDA(c, dalloc(j.chndf, nrec));
    MPG_CUDA(c, dalloc(j.vstage, nslotT));
    // two staging buffers when there are several chunks: the fits of chunk
    // k+1 overlap the accumulation of chunk k
    j.stageLen = maxStage;
    MPG_CUDA(c, dalloc(j.stage, (j.chunkRec.size() > 2 ? 2 : 1) * maxStage));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    return MPGPU_OK;
}

// ------------------------------------------------------------------ data loop
static int32_t run_loop(mpgpu_ctx *c, const mpgpu_fitopts *opt, mpgpu_fitstats *stats,
                        int32_t *naccf, float *chi2f, int32_t *ndff) {
    DevJob &j = c->j;
    cudaStream_t s = c->stream;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    int32_t *errFlag = (int32_t *)c->scal;
    MPG_CUDA(c, cudaMemsetAsync(errFlag, 0, 64, s));
    MPG_CUDA(c, cudaMemsetAsync(j.gvec, 0, sizeof(double) * j.nVar, s));
    MPG_CUDA(c, cudaMemsetAsync(j.gcnt, 0, sizeof(int64_t) * j.nVar, s));
    if (opt->icalcm == 1) MPG_CUDA(c, cudaMemsetAsync(j.matD, 0, sizeof(double) * (size_t)j.nmat, s));
    FitParams fp{};
    fp.rec = j.rec; fp.inder = j.inder; fp.glder = j.glder; fp.meas = j.meas;
    fp.slots = j.slots; fp.swStart = j.swStart; fp.sw = j.sw; fp.gpar = j.gpar;
    fp.grpSlot = j.grpSlot; fp.pairDst = j.pairDst;
    fp.varOfTot = j.varOfTot; fp.fileWeight = j.fileWeight;
    fp.icalcm = opt->icalcm; fp.nloopn = opt->nloopn; fp.lhuber = opt->lhuber; fp.lfitbb = opt->lfitbb;
    fp.chicut = opt->chicut; fp.chhuge = opt->chhuge; fp.dwcut = opt->dwcut; fp.cndlmx = opt->cndlmx;
    fp.stage = j.stage; fp.vstage = j.vstage; fp.status = j.status; fp.chi2add = j.chi2add;
    fp.ndfadd = j.ndfadd; fp.chndf = j.chndf;
    fp.wmax = std::max(j.maxNw, 1); fp.neqmax = std::max(j.maxNeq, 1);
    fp.nalcmax = std::max(j.maxNalc, 1); fp.nalgmax = std::max(j.maxNalg, 1);
    fp.bandmax = opt->lfitbb > 0 ? j.maxBand : -1; fp.bdrmax = j.maxBdr;
    fp.ngrpmax = std::max(j.maxNgrp, 1);
    fp.errFlag = errFlag;
    if (fit_warps_per_cta(fp) < 1) return set_err(c, MPGPU_ERR_LIMIT, "records too large for the fit kernel");
    AccParams ap{};
    ap.bkI = j.bkI; ap.bkJ = j.bkJ; ap.bkLd = j.bkLd; ap.bkOff = j.bkOff;
    ap.itBlk = j.itBlk; ap.itBase = j.itBase; ap.itCnt = j.itCnt; ap.itSlot = j.itSlot;
    ap.rdBlk = j.rdBlk; ap.rdSlot0 = j.rdSlot0; ap.rdN = j.rdN;
    ap.partial = j.partial; ap.pstride = j.pstride; ap.vEntries = j.vEntries;
    ap.status = j.status; ap.stage = j.stage; ap.vstage = j.vstage; ap.slotCnt = j.slotCnt;
    ap.aig = j.aig; ap.nG = j.nG; ap.matsto = j.matsto;
    ap.icalcm = opt->icalcm; ap.matD = j.matD; ap.gvec = j.gvec; ap.gcnt = j.gcnt; ap.errFlag = errFlag;
    const int64_t nchunk = (int64_t)j.chunkRec.size() - 1;
    // fits on stream 1, accumulation on stream 2; with several chunks the
    // staging alternates between two buffers and the fit of chunk k+1 runs
    // while chunk k is accumulated (the fit kernel then keeps one CTA per SM
    // so the memory-bound accumulation can share the SMs)
    cudaStream_t s2 = c->stream2;
    const bool overlap = nchunk > 1;
    std::vector<cudaEvent_t> evF0(nchunk), evF1(nchunk), evA0(nchunk), evA1(nchunk);
    cudaEvent_t evStart, evZero, evEnd;
    cudaEventCreate(&evStart);
    cudaEventCreateWithFlags(&evZero, cudaEventDisableTiming);
    cudaEventCreate(&evEnd);
    for (int64_t ch = 0; ch < nchunk; ++ch) {
        cudaEventCreate(&evF0[ch]); cudaEventCreate(&evF1[ch]);
        cudaEventCreate(&evA0[ch]); cudaEventCreate(&evA1[ch]);
    }
    cudaEventRecord(evStart, s);
    cudaEventRecord(evZero, s);
    MPG_CUDA(c, cudaStreamWaitEvent(s2, evZero, 0));
    int32_t launches = 0;
    for (int64_t ch = 0; ch < nchunk; ++ch) {
        fp.r0 = j.chunkRec[ch];
        fp.r1 = j.chunkRec[ch + 1];
        double *stg = j.stage + (overlap ? (ch & 1) * j.stageLen : 0);
        if (overlap && ch >= 2) MPG_CUDA(c, cudaStreamWaitEvent(s, evA1[ch - 2], 0));
        fp.stage = stg;
        cudaEventRecord(evF0[ch], s);
        if (fp.r1 > fp.r0) { MPG_CUDA(c, launch_fit(fp, nsm, 0, s)); launches++; }
        cudaEventRecord(evF1[ch], s);
        MPG_CUDA(c, cudaStreamWaitEvent(s2, evF1[ch], 0));
        ap.stage = stg;
        ap.vStart = j.vStart + ch * (j.nG + 1);
        ap.item0 = j.chunkItem[ch];
        ap.nitem = j.chunkItem[ch + 1] - j.chunkItem[ch];
        ap.red0 = j.chunkRed[ch];
        ap.nred = j.chunkRed[ch + 1] - j.chunkRed[ch];
        cudaEventRecord(evA0[ch], s2);
        if (fp.r1 > fp.r0) { MPG_CUDA(c, launch_accumulate(ap, nsm, s2)); launches += 3; }
        cudaEventRecord(evA1[ch], s2);
    }
    if (nchunk > 0) MPG_CUDA(c, cudaStreamWaitEvent(s, evA1[nchunk - 1], 0));
    // statistics
    const int32_t nf = j.nfiles;
    int64_t *iout = (int64_t *)(c->scal + 8);
    double *dout = c->scal + 4;
    float *fout = (float *)(c->scal + 256);
    const int64_t nint = 9 + 2 * (int64_t)nf;
    if (nint > 240 || nf > 400) return set_err(c, MPGPU_ERR_LIMIT, "too many files for the statistics buffer");
    MPG_CUDA(c, cudaMemsetAsync(iout, 0, sizeof(int64_t) * nint, s));
    StatParams sp{j.status, j.chi2add, j.ndfadd, j.chndf, j.rec, j.fileWeight, j.nrec, nf,
                  dout, iout, fout};
    MPG_CUDA(c, launch_stats(sp, s));
    launches += 2;
    cudaEventRecord(evEnd, s);
    MPG_CUDA(c, cudaMemcpyAsync(c->hscal, c->scal, 4096, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    double msFit = 0.0, msAcc = 0.0;
    float t = 0.0f;
    for (int64_t ch = 0; ch < nchunk; ++ch) {
        cudaEventElapsedTime(&t, evF0[ch], evF1[ch]);
        msFit += t;
        cudaEventElapsedTime(&t, evA0[ch], evA1[ch]);
        msAcc += t;
    }
    cudaEventElapsedTime(&t, evStart, evEnd);
    const double msLoop = t;
    for (int64_t ch = 0; ch < nchunk; ++ch) {
        cudaEventDestroy(evF0[ch]); cudaEventDestroy(evF1[ch]);
        cudaEventDestroy(evA0[ch]); cudaEventDestroy(evA1[ch]);
    }
    cudaEventDestroy(evStart); cudaEventDestroy(evZero); cudaEventDestroy(evEnd);
    const int32_t *hflag = (const int32_t *)c->hscal;
    if (hflag[0]) return set_err(c, hflag[0], "device index error in the data loop");
    const int64_t *hi = (const int64_t *)(c->hscal + 8);
    const double *hd = c->hscal + 4;
    const float *hf = (const float *)(c->hscal + 256);
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        for (int k = 0; k < 6; ++k) stats->nrej[k] = hi[2 + k];
        stats->chi2SumI = hi[0];
        stats->chi2SumD = hd[0];
        stats->ndfSum = hi[1];
        stats->ndfSumW = hd[1];
        if (opt->nloopn == 1 && opt->lfitbb > 0) {
            stats->nbndr[0] = j.nbndr[0]; stats->nbndr[1] = j.nbndr[1];
            stats->nbdrx = j.nbdrx; stats->nbndx = j.nbndx;
        }
        stats->naccepted = hi[8];
        stats->msFit = msFit;
        stats->msAccum = msAcc;
        stats->msLoop = msLoop;
        stats->launches = launches;
    }
    c->lastNaccepted = hi[8];
    for (int32_t f = 0; f < nf; ++f) {
        if (naccf) naccf[f] += (int32_t)hi[9 + f];
        if (ndff) ndff[f] += (int32_t)hi[9 + nf + f];
        if (chi2f) chi2f[f] += hf[f];
    }
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_loopbf_device(mpgpu_ctx *c, const mpgpu_fitopts *opt,
                                       const double *d_globalParameter, mpgpu_fitstats *stats) {
    if (!c || !opt) return MPGPU_ERR_ARG;
    if (c->j.nrec <= 0 || !c->j.rec) return set_err(c, MPGPU_ERR_ARG, "no records uploaded");
    cudaSetDevice(c->device);
    if (d_globalParameter && d_globalParameter != c->j.gpar)
        MPG_CUDA(c, cudaMemcpyAsync(c->j.gpar, d_globalParameter, sizeof(double) * c->j.nTotal,
                                    cudaMemcpyDeviceToDevice, c->stream));
    return run_loop(c, opt, stats, nullptr, nullptr, nullptr);
}

extern "C" int32_t mpgpu_loopbf(mpgpu_ctx *c, const mpgpu_fitopts *opt, const double *globalParameter,
                                double *globalVector, int64_t *globalCounter, mpgpu_fitstats *stats,
                                int32_t *naccf, float *chi2f, int32_t *ndff) {
    if (!c || !opt || !globalParameter) return MPGPU_ERR_ARG;
    if (c->j.nrec <= 0 || !c->j.rec) return set_err(c, MPGPU_ERR_ARG, "no records uploaded");
    cudaSetDevice(c->device);
    DevJob &j = c->j;
    MPG_CUDA(c, cudaMemcpyAsync(j.gpar, globalParameter, sizeof(double) * j.nTotal,
                                cudaMemcpyHostToDevice, c->stream));
    int32_t rc = run_loop(c, opt, stats, naccf, chi2f, ndff);
    if (rc) return rc;
    if (globalVector)
        MPG_CUDA(c, cudaMemcpyAsync(globalVector, j.gvec, sizeof(double) * j.nVar, cudaMemcpyDeviceToHost, c->stream));
    if (globalCounter)
        MPG_CUDA(c, cudaMemcpyAsync(globalCounter, j.gcnt, sizeof(int64_t) * j.nVar, cudaMemcpyDeviceToHost, c->stream));
    MPG_CUDA(c, cudaStreamSynchronize(c->stream));
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_mupdat(mpgpu_ctx *c, int32_t n, const int32_t *i, const int32_t *jj,
                                const double *add) {
    if (!c || n < 0) return MPGPU_ERR_ARG;
    if (n == 0) return MPGPU_OK;
    DevJob &j = c->j;
    int32_t *di = nullptr, *dj = nullptr;
    double *da = nullptr;
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(di, i, n, s));
    MPG_CUDA(c, dupload(dj, jj, n, s));
    MPG_CUDA(c, dupload(da, add, n, s));
    int32_t *errFlag = (int32_t *)c->scal;
    MPG_CUDA(c, cudaMemsetAsync(errFlag, 0, 4, s));
    MPG_CUDA(c, launch_mupdat(n, di, dj, da, j, errFlag, s));
    int32_t h = 0;
    MPG_CUDA(c, cudaMemcpyAsync(&h, errFlag, 4, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    dfree(di); dfree(dj); dfree(da);
    if (h) return set_err(c, h, "mupdat index outside the matrix");
    return MPGPU_OK;
}

namespace {
__global__ void k_vadd(int32_t n, const int32_t *idx, const double *v, double *gvec, int32_t nVar) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int32_t q = 0; q < n; ++q)
        if (idx[q] >= 1 && idx[q] <= nVar) gvec[idx[q] - 1] += v[q];
}
}  // namespace

extern "C" int32_t mpgpu_vector_add(mpgpu_ctx *c, int32_t n, const int32_t *vidx, const double *vadd) {
    if (!c || n < 0) return MPGPU_ERR_ARG;
    if (n == 0) return MPGPU_OK;
    int32_t *di = nullptr;
    double *da = nullptr;
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(di, vidx, n, s));
    MPG_CUDA(c, dupload(da, vadd, n, s));
    k_vadd<<<1, 32, 0, s>>>(n, di, da, c->j.gvec, c->j.nVar);
    MPG_CUDA(c, cudaGetLastError());
    MPG_CUDA(c, cudaStreamSynchronize(s));
    dfree(di); dfree(da);
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_download_matrix(mpgpu_ctx *c, double *globalMatD) {
    if (!c || !globalMatD) return MPGPU_ERR_ARG;
    MPG_CUDA(c, cudaMemcpy(globalMatD, c->j.matD, sizeof(double) * (size_t)c->j.nmat, cudaMemcpyDeviceToHost));
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_download_vector(mpgpu_ctx *c, double *globalVector, int64_t *globalCounter) {
    if (!c) return MPGPU_ERR_ARG;
    if (globalVector)
        MPG_CUDA(c, cudaMemcpy(globalVector, c->j.gvec, sizeof(double) * c->j.nVar, cudaMemcpyDeviceToHost));
    if (globalCounter)
        MPG_CUDA(c, cudaMemcpy(globalCounter, c->j.gcnt, sizeof(int64_t) * c->j.nVar, cudaMemcpyDeviceToHost));
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_download_record_status(mpgpu_ctx *c, int32_t *status) {
    if (!c || !status) return MPGPU_ERR_ARG;
    std::vector<int8_t> st(c->j.nrec);
    MPG_CUDA(c, cudaMemcpy(st.data(), c->j.status, c->j.nrec, cudaMemcpyDeviceToHost));
    for (int64_t r = 0; r < c->j.nrec; ++r) status[r] = st[r];
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_solve(mpgpu_ctx *c, int32_t metsol, const double *consResiduals,
                               double rtol, int32_t itnlim, double *correction, double *errors,
                               mpgpu_solveinfo *info) {
    if (!c || !correction) return MPGPU_ERR_ARG;
    cudaSetDevice(c->device);
    mpgpu_solveinfo tmp;
    if (!info) info = &tmp;
    memset(info, 0, sizeof(*info));
    if (metsol == 1 || metsol == 3) {
        if (c->j.matsto != 1) return set_err(c, MPGPU_ERR_ARG, "inversion/decomposition need packed storage");
        return solve_inversion(c, consResiduals, correction, errors, info, metsol == 3);
    }
    if (metsol == 4) return solve_minres(c, consResiduals, rtol, itnlim, correction, info);
    return set_err(c, MPGPU_ERR_ARG, "unsupported solution method");
}

extern "C" int32_t mpgpu_avprod(mpgpu_ctx *c, int32_t n, const double *x, double *b) {
    if (!c || !x || !b) return MPGPU_ERR_ARG;
    if (n != c->j.nVar - c->j.ncon) return set_err(c, MPGPU_ERR_SIZE, "avprod: vector/matrix size mismatch");
    cudaSetDevice(c->device);
    return avprod_host(c, n, x, b);
}

// ------------------------------------------------------------------ FP64 peak
namespace {
// independent fused multiply-add chains (8 per thread) keep the FP64 pipe busy
__global__ void k_dfma_chain(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
    double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) out[0] = s;  // keeps the chains live
}
}  // namespace

extern "C" int32_t mpgpu_probe_fp64(int32_t device, double *tflops) {
    if (!tflops) return MPGPU_ERR_ARG;
    *tflops = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) return MPGPU_ERR_CUDA;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    double *d = nullptr;
    if (cudaMalloc(&d, 8) != cudaSuccess) return MPGPU_ERR_ALLOC;
    const int iters = 4096, threads = 256, blocks = nsm * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        k_dfma_chain<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
        if (rep > 0 && ms > 0.0f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    *tflops = best;
    return cudaGetLastError() == cudaSuccess ? MPGPU_OK : MPGPU_ERR_CUDA;
}

extern "C" int32_t mpgpu_host_register(void *ptr, int64_t bytes) {
    if (!ptr || bytes <= 0) return MPGPU_ERR_ARG;
    return cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault) == cudaSuccess ? MPGPU_OK : MPGPU_ERR_CUDA;
}

extern "C" int32_t mpgpu_host_unregister(void *ptr) {
    if (!ptr) return MPGPU_ERR_ARG;
    return cudaHostUnregister(ptr) == cudaSuccess ? MPGPU_OK : MPGPU_ERR_CUDA;
}
