// mpgpu_api.cu -- the C-ABI entry points (include/mpgpu.h): context,
// layout, constraints, record upload, the data loop and the solver dispatch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
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

void free_records(DevJob &j) {
    UpTmp &t = j.tmp;
    dfree(t.recPtr); dfree(t.recFile); dfree(t.cnt); dfree(t.off); dfree(t.scanTmp); dfree(t.grpRec);
    dfree(t.k0); dfree(t.k1); dfree(t.v0); dfree(t.v1); dfree(t.pairKey); dfree(t.hist); dfree(t.head);
    dfree(t.nel); dfree(t.segStart); dfree(t.segEnd); dfree(t.bcnt); dfree(t.bscan); dfree(t.cntG); dfree(t.scal);
    dfree(t.ovList); dfree(t.chunkB); dfree(t.keyEnd); dfree(t.bmax); dfree(j.recList);
    dfree(j.bigDone);
    j.cap.clear();
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
    dfree(j.rowBlk0); dfree(j.blkJ); dfree(j.blkOff); dfree(j.blkLd);
    dfree(j.rowWidth);
}

void free_constraints(DevJob &j) {
    dfree(j.qlV); dfree(j.qlVk); dfree(j.qlR2); dfree(j.qlT);
    j.ncon = 0;
}

}  // namespace

// ------------------------------------------------------------------ context
extern "C" int32_t mpgpu_create(mpgpu_ctx **out, const mpgpu_cfg *cfg) {
    if (!out) return MPGPU_ERR_ARG;
    *out = nullptr;
    mpgpu_ctx *c = new mpgpu_ctx();
    c->device = cfg ? cfg->device : 0;
    c->stagingBytes = (cfg && cfg->staging_bytes > 0) ? cfg->staging_bytes : 0;  // 0: sized per job
    c->flags = cfg ? cfg->flags : 0;
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->scal, 4096);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&c->hscal, 4096);
    if (e != cudaSuccess) {
        int32_t rc = cuda_err(c, e, "mpgpu_create");
        mpgpu_destroy(c);
        return rc;
    }
    // the static area of mpgpu_mupdat_noalloc is reserved now, before the
    // job's large allocations (its module would otherwise load lazily, on
    // the first call, when the device memory may be full)
    const int32_t rc = noalloc_prepare(c);
    if (rc != MPGPU_OK) {
        mpgpu_destroy(c);
        return rc;
    }
    *out = c;
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_destroy(mpgpu_ctx *c) {
    if (!c) return MPGPU_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    dense_release(c);
    free_records(c->j);
    free_layout(c->j);
    free_constraints(c->j);
    free_resident(c->res);
    if (c->mon.measIndex) cudaFree(c->mon.measIndex);
    if (c->mon.measRes) cudaFree(c->mon.measRes);
    if (c->mon.hist) cudaFree(c->mon.hist);
    if (c->mon.meas) cudaFree(c->mon.meas);
    if (c->scal) cudaFree(c->scal);
    if (c->hscal) cudaFreeHost(c->hscal);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    delete c;
    return MPGPU_OK;
}

// the device memory of the current job (records, layout, matrix,
// constraints, resident structure, dense workspace); streams and the
// static areas stay, so the context takes the next job as a fresh one
extern "C" int32_t mpgpu_release(mpgpu_ctx *c) {
    if (!c) return MPGPU_ERR_ARG;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->stream2) cudaStreamSynchronize(c->stream2);
    dense_release(c);
    free_records(c->j);
    free_layout(c->j);
    free_constraints(c->j);
    free_resident(c->res);
    c->j.nVar = 0;
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
    dense_release(c);
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
        std::vector<int32_t> bJ, bLd, width(nGroups, 0);
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
                            bLd.push_back(o1 - o0);
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

// ------------------------------------------------------------------ pairentries
// Group pairs met in the records but left out of the sparse structure
// (pairentries: counted fewer than mreqpe times, clbits/ndbits
// mpbits.f90:182-243, 305-566).  Their blocks join the accumulation table
// of their row, in column order, with the offset of a discard area after
// the nmat matrix elements and the row stride of their own column group, so
// the records' updates of those pairs are summed there and dropped, as
// mupdat drops an element of a pair that is not stored (pede.f90:3172); the
// diagonal elements of a left-out diagonal pair still reach the diagonal.
// The discard area is as large as the largest of these blocks, the blocks
// share it and nothing reads it; the sparse products, preconditioners and
// downloads use offsets and columns, which hold only the stored pairs.  A
// later call replaces the list.
extern "C" int32_t mpgpu_set_suppressed_pairs(mpgpu_ctx *c, int64_t npair, const int32_t *pairs) {
    if (!c) return MPGPU_ERR_ARG;
    DevJob &j = c->j;
    if (j.matsto != 2 || !j.matD) return set_err(c, MPGPU_ERR_ARG, "suppressed pairs need a sparse layout");
    if (npair < 0 || (npair > 0 && !pairs))
        return set_err(c, MPGPU_ERR_ARG, "mpgpu_set_suppressed_pairs: bad arguments");
    cudaSetDevice(c->device);
    const int32_t nG = j.nG;
    const std::vector<int32_t> &aig = j.hAig;
    std::vector<std::vector<int32_t>> add(nG + 1);
    for (int64_t q = 0; q < npair; ++q) {
        const int32_t I = std::max(pairs[2 * q], pairs[2 * q + 1]);
        const int32_t J = std::min(pairs[2 * q], pairs[2 * q + 1]);
        if (J < 1 || I > nG) return set_err(c, MPGPU_ERR_SIZE, "suppressed pair outside the groups");
        add[I].push_back(J);
    }
    std::vector<int64_t> rowBlk0(nG + 1, 0), bOff;
    std::vector<int32_t> bJ, bLd;
    int64_t area = 0;
    for (int32_t I = 1; I <= nG; ++I) {
        std::vector<int32_t> &a = add[I];
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
        const int64_t ni = aig[I] - aig[I - 1];
        int64_t k = j.hRowBlk0[I - 1];
        const int64_t ke = j.hRowBlk0[I];
        size_t q = 0;
        while (k < ke || q < a.size()) {
            if (q < a.size() && (k >= ke || a[q] < j.hBlkJ[k])) {
                const int32_t J = a[q++];
                const int32_t nj = aig[J] - aig[J - 1];
                bJ.push_back(J);
                bOff.push_back(j.nmat);
                bLd.push_back(nj);
                area = std::max<int64_t>(area, ni * nj);
            } else if (j.hBlkOff[k] >= j.nmat) {
                ++k;   // a block of an earlier call: the new list replaces it
            } else {
                if (q < a.size() && a[q] == j.hBlkJ[k])
                    return set_err(c, MPGPU_ERR_SIZE, "a suppressed pair is stored in the structure");
                bJ.push_back(j.hBlkJ[k]);
                bOff.push_back(j.hBlkOff[k]);
                bLd.push_back(j.hBlkLd[k]);
                ++k;
            }
        }
        rowBlk0[I] = (int64_t)bJ.size();
    }
    // block ids change: records uploaded before are released
    dense_release(c);
    free_records(j);
    cudaStream_t s = c->stream;
    j.hRowBlk0 = rowBlk0;
    j.hBlkJ = bJ;
    j.hBlkOff = bOff;
    j.hBlkLd = bLd;
    MPG_CUDA(c, dupload(j.rowBlk0, rowBlk0.data(), nG + 1, s));
    MPG_CUDA(c, dupload(j.blkJ, bJ.data(), (int64_t)bJ.size(), s));
    MPG_CUDA(c, dupload(j.blkOff, bOff.data(), (int64_t)bOff.size(), s));
    MPG_CUDA(c, dupload(j.blkLd, bLd.data(), (int64_t)bLd.size(), s));
    MPG_CUDA(c, dalloc(j.matD, j.nmat + area));
    MPG_CUDA(c, cudaMemsetAsync(j.matD, 0, sizeof(double) * (size_t)(j.nmat + area), s));
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
    dense_invalidate(c);
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
    // compact WY form of the reflections (Schreiber & Van Loan 1989):
    // H_1 H_2 ... H_m = I - U T U^T with u_k = (V_k, Vk_k at kn_k), T upper
    // triangular, T_kk = 2, T(0:k, k) = -2 T(0:k, 0:k) U(:, 0:k)^T u_k; the
    // Gram matrix U^T U from the vectors' common support
    std::vector<double> G((size_t)ncon * ncon), T((size_t)ncon * ncon, 0.0);
    auto kn0 = [&](int32_t k) { return npar - ncon + k; };  // 0-based position of Vk_k
    for (int32_t a = 0; a < ncon; ++a)
        for (int32_t b = a; b < ncon; ++b) {
            const double *va = &V[(size_t)a * npar], *vb = &V[(size_t)b * npar];
            double g = 0.0;
            const int32_t lim = std::min(kn0(a), kn0(b));
            for (int32_t q = 0; q < lim; ++q) g += va[q] * vb[q];
            // the Vk entries: u_a at kn0(a) meets u_b there (V row of b or Vk_b)
            g += Vk[a] * (kn0(a) == kn0(b) ? Vk[b] : (kn0(a) < kn0(b) ? vb[kn0(a)] : 0.0));
            if (kn0(b) < kn0(a)) g += Vk[b] * va[kn0(b)];
            G[(size_t)a * ncon + b] = G[(size_t)b * ncon + a] = g;
        }
    for (int32_t k = 0; k < ncon; ++k) {
        T[(size_t)k * ncon + k] = 2.0;
        for (int32_t r = 0; r < k; ++r) {
            double acc = 0.0;
            for (int32_t cc = r; cc < k; ++cc) acc += T[(size_t)r * ncon + cc] * G[(size_t)cc * ncon + k];
            T[(size_t)r * ncon + k] = -2.0 * acc;
        }
    }
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(j.qlT, T.data(), (int64_t)ncon * ncon, s));
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
    if (!c || nrec < 0 || !recPtr || (!inder) != (!glder)) return MPGPU_ERR_ARG;
    DevJob &j = c->j;
    if (j.nVar <= 0) return set_err(c, MPGPU_ERR_ARG, "set the layout before the records");
    if (nfiles < 1) nfiles = 1;
    MPG_CUDA(c, cudaSetDevice(c->device));
    j.nrec = 0;  // no records until the upload succeeds
    if (!inder) {
        // the records kept by mpgpu_loop1_device become the job's records
        ResidentRecords &R = c->res;
        if (!R.translated || R.nrec != nrec || R.w0 != recPtr[0] || R.nw != recPtr[nrec] - recPtr[0])
            return set_err(c, MPGPU_ERR_ARG, "no matching records kept by mpgpu_loop1_device");
        if (R.nTotal != j.nTotal) return set_err(c, MPGPU_ERR_SIZE, "layout and loop1 label tables differ");
        dfree(j.inder);
        dfree(j.glder);
        j.inder = R.inder;
        j.glder = R.glder;
        j.cap[(const void *)&j.inder] = std::max<int64_t>(R.nw, 1);
        j.cap[(const void *)&j.glder] = std::max<int64_t>(R.nw, 1);
        R.inder = nullptr;
        R.glder = nullptr;
        free_resident(R);
    }
    const int32_t rc = upload_records_device(c, nrec, recPtr, inder, glder, recFile, nfiles, fileWeight);
    if (rc != MPGPU_OK) j.nrec = 0;
    return rc;
}

// ------------------------------------------------------------ structure passes
extern "C" int32_t mpgpu_loop1_device(mpgpu_ctx *c, int64_t nrec, const int64_t *recPtr, const int32_t *inder,
                                      const double *glder, int32_t nsteer, const int32_t *steerLabels,
                                      int32_t npre, const int32_t *preLabel, const double *preSigma,
                                      int32_t mreqenf, int32_t cap, int32_t *labels, int64_t *counter,
                                      int32_t *varIndex, int32_t *totGroup, int32_t *nVar,
                                      int32_t *nVarGroups) {
    if (!c || nrec < 0 || !recPtr || (nrec > 0 && (!inder || !glder)) || (nsteer > 0 && !steerLabels) ||
        (npre > 0 && (!preLabel || !preSigma)) || !labels || !counter || !varIndex || !totGroup || !nVar ||
        !nVarGroups)
        return -44;
    if (cudaSetDevice(c->device) != cudaSuccess) return -43;
    return loop1_device(c, nrec, recPtr, inder, glder, nsteer, steerLabels, npre, preLabel, preSigma, mreqenf,
                        cap, labels, counter, varIndex, totGroup, nVar, nVarGroups);
}

extern "C" int32_t mpgpu_loop2_device(mpgpu_ctx *c, const int32_t *varIndexOfTotal, int32_t nVar, int32_t nG,
                                      const int32_t *allIndexGroups, int64_t cap, int64_t *offsets,
                                      int32_t *columns, int64_t *ncolw, int64_t *nmat) {
    if (!c || !varIndexOfTotal || nVar <= 0 || nG <= 0 || !allIndexGroups || !offsets || !ncolw || !nmat ||
        (cap > 0 && !columns))
        return MPGPU_ERR_ARG;
    if (allIndexGroups[nG] != nVar + 1) return set_err(c, MPGPU_ERR_SIZE, "groups do not end at nVar+1");
    MPG_CUDA(c, cudaSetDevice(c->device));
    return loop2_device(c, varIndexOfTotal, nVar, nG, allIndexGroups, cap, offsets, columns, ncolw, nmat);
}

extern "C" int32_t mpgpu_set_monitor(mpgpu_ctx *c, const mpgpu_monitor_cfg *cfg, const int32_t *measIndex,
                                     const double *measRes, int32_t numMeas) {
    if (!c) return MPGPU_ERR_ARG;
    MPG_CUDA(c, cudaSetDevice(c->device));
    Monitor &M = c->mon;
    if (M.measIndex) cudaFree(M.measIndex);
    if (M.measRes) cudaFree(M.measRes);
    if (M.hist) cudaFree(M.hist);
    if (M.meas) cudaFree(M.meas);
    M = Monitor{};
    if (!cfg) return MPGPU_OK;   // monitoring off
    if (cfg->nbins < 1 || cfg->nbins > (1 << 20) || !(cfg->range > 0.0f) || cfg->measBins < 1 ||
        cfg->measBins > (1 << 20) || numMeas < 0 || (numMeas > 0 && (!measIndex || !measRes)))
        return set_err(c, MPGPU_ERR_ARG, "mpgpu_set_monitor: bad configuration");
    DevJob &j = c->j;
    if (numMeas > 0 && j.nTotal <= 0) return set_err(c, MPGPU_ERR_ARG, "set the layout before the monitor groups");
    M.nbins = cfg->nbins;
    M.range = cfg->range;
    M.measBins = cfg->measBins;
    M.mode = cfg->mode;
    M.lfitnp = cfg->lfitnp > 0 ? cfg->lfitnp : (1 << 30);
    M.numMeas = numMeas;
    MPG_CUDA(c, cudaMalloc(&M.hist, sizeof(unsigned long long) * 4 * (M.nbins + 2)));
    if (numMeas > 0) {
        for (int32_t i = 0; i < j.nTotal; ++i)
            if (measIndex[i] < 0 || measIndex[i] > numMeas) return set_err(c, MPGPU_ERR_ARG, "bad monitor group");
        MPG_CUDA(c, cudaMalloc(&M.measIndex, sizeof(int32_t) * j.nTotal));
        MPG_CUDA(c, cudaMalloc(&M.measRes, sizeof(double) * numMeas));
        MPG_CUDA(c, cudaMalloc(&M.meas, sizeof(unsigned long long) * (size_t)numMeas * M.measBins));
        MPG_CUDA(c, cudaMemcpy(M.measIndex, measIndex, sizeof(int32_t) * j.nTotal, cudaMemcpyHostToDevice));
        MPG_CUDA(c, cudaMemcpy(M.measRes, measRes, sizeof(double) * numMeas, cudaMemcpyHostToDevice));
    }
    M.on = true;
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_get_monitor(mpgpu_ctx *c, int64_t *hist, int64_t *measHists) {
    if (!c || !c->mon.on) return c ? set_err(c, MPGPU_ERR_ARG, "monitoring is off") : MPGPU_ERR_ARG;
    MPG_CUDA(c, cudaSetDevice(c->device));
    const Monitor &M = c->mon;
    if (hist)
        MPG_CUDA(c, cudaMemcpy(hist, M.hist, sizeof(int64_t) * 4 * (M.nbins + 2), cudaMemcpyDeviceToHost));
    if (measHists && M.numMeas > 0)
        MPG_CUDA(c, cudaMemcpy(measHists, M.meas, sizeof(int64_t) * (size_t)M.numMeas * M.measBins,
                               cudaMemcpyDeviceToHost));
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_fit_buckets(const mpgpu_ctx *c, int64_t *count, int32_t *wpc, double *tuneMs) {
    static_assert(MPGPU_FIT_BUCKETS == MPG_FIT_BUCKETS, "bucket count of the ABI");
    if (!c) return MPGPU_ERR_ARG;
    const DevJob &j = c->j;
    const int64_t nchunk = (int64_t)j.chunkRec.size() - 1;
    for (int b = 0; b < MPG_FIT_BUCKETS; ++b) {
        int64_t n = 0;
        if (!j.bucketOff.empty())
            for (int64_t ch = 0; ch < nchunk; ++ch)
                n += j.bucketOff[ch * MPG_FIT_BUCKETS + b + 1] - j.bucketOff[ch * MPG_FIT_BUCKETS + b];
        if (count) count[b] = n;
        if (wpc) wpc[b] = j.bucketWpc.empty() ? 0 : j.bucketWpc[b];
        if (tuneMs)
            for (int k = 0; k < 4; ++k) tuneMs[4 * b + k] = j.bucketTuneMs.empty() ? 0.0 : j.bucketTuneMs[4 * b + k];
    }
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_upload_timing(const mpgpu_ctx *c, double *msCopy, double *msPrepare,
                                       int32_t *nchunk) {
    if (!c) return MPGPU_ERR_ARG;
    if (msCopy) *msCopy = c->j.msUploadCopy;
    if (msPrepare) *msPrepare = c->j.msUploadPrepare;
    if (nchunk) *nchunk = c->j.uploadChunks;
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
    const Monitor &mon = c->mon;
    if (mon.on) {
        fp.monOn = 1;
        fp.monPull = opt->nloopn <= mon.lfitnp ? 1 : 0;
        fp.monBins = mon.nbins;
        fp.monMeasBins = mon.measBins;
        fp.monMode = mon.mode;
        fp.monRange = mon.range;
        fp.measIndex = mon.numMeas > 0 ? mon.measIndex : nullptr;
        fp.measRes = mon.measRes;
        fp.monHist = mon.hist;
        fp.measHists = mon.meas;
        MPG_CUDA(c, cudaMemsetAsync(mon.hist, 0, sizeof(unsigned long long) * 4 * (mon.nbins + 2), s));
        if (mon.numMeas > 0)
            MPG_CUDA(c, cudaMemsetAsync(mon.meas, 0, sizeof(unsigned long long) * (size_t)mon.numMeas * mon.measBins,
                                        s));
    }
    // fit launches per size class of records (fit buckets, ordered at
    // upload): each class gets shared memory for its own largest record;
    // classes whose B and W do not fit a warp's shared memory with four
    // warps per CTA take the large-record path
    const bool onePer = (c->flags & MPGPU_FLAG_ONE_RECORD_PER_BLOCK) != 0;
    const bool bucketed = !onePer && !(c->flags & MPGPU_FLAG_NO_BUCKETS) && !j.bucketOff.empty();
    const int nb = bucketed ? MPG_FIT_BUCKETS : 1;
    const int64_t nchunk = (int64_t)j.chunkRec.size() - 1;
    std::vector<FitParams> bfp(nb, fp);
    std::vector<int64_t> bsub(nb, 0);
    int64_t bwNeed = 0;
    for (int b = 0; b < nb; ++b) {
        FitParams &q = bfp[b];
        if (bucketed) {
            if (j.bucketOff[nchunk * nb] == 0) continue;
            int64_t cnt = 0;
            for (int64_t ch = 0; ch < nchunk; ++ch) cnt += j.bucketOff[ch * nb + b + 1] - j.bucketOff[ch * nb + b];
            if (cnt == 0) continue;
            const int32_t *m = &j.bucketMax[7 * b];
            q.wmax = std::max(m[0], 1); q.neqmax = std::max(m[1], 1);
            q.nalcmax = std::max(m[2], 1); q.nalgmax = std::max(m[3], 1);
            q.bandmax = opt->lfitbb > 0 ? m[4] - 1 : -1; q.bdrmax = m[5];
            q.ngrpmax = std::max(m[6], 1);
            q.recList = j.recList;
        }
        q.onePerBlock = onePer ? 1 : 0;
        // the path is chosen by the arena's capacity (not by a tuned warp
        // count), so that every loop of a job takes the same path
        q.bigMode = 0;
        q.wpc = 0;
        FitParams cap = q;
        cap.onePerBlock = 0;
        q.bigMode = (c->flags & MPGPU_FLAG_LARGE_RECORDS) || fit_warps_per_cta(cap) < 4 ? 1 : 0;
        if (bucketed && !j.bucketWpc.empty() && j.bucketWpc[b] > 0) q.wpc = j.bucketWpc[b];
        if (q.bigMode) {
            // B and W, or the S-form's Y (neq x nalc), S (neq x neq) and its
            // group and equation lists, whichever is larger, so that the
            // S-form is not ruled out by the room of a class whose records
            // have more equations than global slots (broken lines)
            const int64_t sNeed = (int64_t)q.neqmax * q.nalcmax + (int64_t)q.neqmax * q.neqmax +
                                  (q.ngrpmax + 2) / 2 + (q.neqmax + 2) / 2 + 2;
            q.bwStride = std::max<int64_t>(2 * (int64_t)q.nalgmax * q.nalcmax, sNeed);
            // records per fit launch: their B and W within 2 GiB
            bsub[b] = std::max<int64_t>(1, ((int64_t)2 << 30) / (8 * std::max<int64_t>(q.bwStride, 1)));
            bwNeed = std::max(bwNeed, bsub[b] * q.bwStride);
        }
        if (fit_warps_per_cta(q) < 1) return set_err(c, MPGPU_ERR_LIMIT, "records too large for the fit kernel");
    }
    if (bwNeed > 0) {
        int64_t subMax = 1;
        for (int b = 0; b < nb; ++b) subMax = std::max(subMax, bsub[b]);
        MPG_CUDA(c, dgrow(j, j.bw, bwNeed));
        MPG_CUDA(c, dgrow(j, j.bigDone, subMax));
        for (auto &q : bfp) { q.bw = j.bw; q.bigDone = j.bigDone; }
    }
    if (fp.bandmax >= 0 && (opt->icalcm == 1 || mon.on)) {
        // every warp that can be resident: 64 per SM (one-record-per-block
        // launches take at most that many records)
        const int64_t stride = 32 * (int64_t)fp.nalcmax + (int64_t)fp.nalcmax * (fp.nalcmax + 1) / 2 + 2;
        MPG_CUDA(c, dgrow(j, j.bscr, (int64_t)nsm * 64 * stride));
        for (auto &q : bfp) { q.bscr = j.bscr; q.bscrStride = stride; }
    }
    // warps per CTA of each class, timed on a sample of the class on the
    // first loop with matrix after an upload that changed the class's
    // maxima; the records' results do not depend on it
    if (bucketed && opt->icalcm == 1 && !(c->flags & MPGPU_FLAG_NO_AUTOTUNE) && nchunk > 0) {
        for (int b = 0; b < nb; ++b) {
            if (j.bucketWpc[b] != 0 || bfp[b].recList == nullptr) continue;
            // sample: four waves of the most warps an SM holds
            const int64_t sample = bfp[b].bigMode ? std::min<int64_t>(bsub[b], (int64_t)nsm * 64)
                                                  : (int64_t)nsm * 64 * 4;
            const int64_t i0 = j.bucketOff[b], i1 = std::min(j.bucketOff[b + 1], i0 + sample);
            if (i1 <= i0) continue;
            FitParams q = bfp[b];
            q.stage = j.stage;
            q.r0 = i0;
            q.r1 = i1;
            q.monOn = 0;   // sample fits leave the monitor alone
            const int cand[4] = {1, 2, 4, 8};
            float best = 0.0f;
            int bestW = 0;
            // more warps per CTA are kept unless fewer are at least 3 % faster
            cudaEvent_t t0, t1;
            cudaEventCreate(&t0);
            cudaEventCreate(&t1);
            bool warm = false;
            for (int k = 0; k < 4; ++k) {
                q.wpc = cand[k];
                if (fit_warps_per_cta(q) != cand[k]) continue;
                if (!warm) MPG_CUDA(c, launch_fit(q, nsm, 0, s));   // caches and first-launch costs
                warm = true;
                cudaEventRecord(t0, s);
                MPG_CUDA(c, launch_fit(q, nsm, 0, s));
                cudaEventRecord(t1, s);
                MPG_CUDA(c, cudaEventSynchronize(t1));
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, t0, t1);
                j.bucketTuneMs[4 * b + k] = ms;
                if (bestW == 0 || ms <= best * 1.03f) {
                    if (bestW == 0 || ms < best) best = ms;
                    bestW = cand[k];
                }
            }
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            j.bucketWpc[b] = bestW > 0 ? bestW : -1;
            bfp[b].wpc = bestW > 0 ? bestW : 0;
        }
    }
    AccParams ap{};
    ap.bkI = j.bkI; ap.bkJ = j.bkJ; ap.bkLd = j.bkLd; ap.bkOff = j.bkOff;
    ap.itBlk = j.itBlk; ap.itBase = j.itBase; ap.itCnt = j.itCnt; ap.itSlot = j.itSlot;
    ap.rdBlk = j.rdBlk; ap.rdSlot0 = j.rdSlot0; ap.rdN = j.rdN;
    ap.partial = j.partial; ap.pstride = j.pstride; ap.vEntries = j.vEntries;
    ap.status = j.status; ap.stage = j.stage; ap.vstage = j.vstage; ap.slotCnt = j.slotCnt;
    ap.aig = j.aig; ap.nG = j.nG; ap.matsto = j.matsto;
    ap.icalcm = opt->icalcm; ap.matD = j.matD; ap.gvec = j.gvec; ap.gcnt = j.gcnt; ap.errFlag = errFlag;
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
    int32_t launches = 0;
    const int32_t nf = j.nfiles;
    int64_t *iout = (int64_t *)(c->scal + 8);
    double *dout = c->scal + 4;
    float *fout = (float *)(c->scal + 256);
    const int64_t nint = 9 + 2 * (int64_t)nf;
    if (nint > 240 || nf > 400) return set_err(c, MPGPU_ERR_LIMIT, "too many files for the statistics buffer");
    auto body = [&]() -> int32_t {
    launches = 0;
    cudaEventRecord(evStart, s);
    cudaEventRecord(evZero, s);
    MPG_CUDA(c, cudaStreamWaitEvent(s2, evZero, 0));
    for (int64_t ch = 0; ch < nchunk; ++ch) {
        fp.r0 = j.chunkRec[ch];
        fp.r1 = j.chunkRec[ch + 1];
        double *stg = j.stage + (overlap ? (ch & 1) * j.stageLen : 0);
        if (overlap && ch >= 2) MPG_CUDA(c, cudaStreamWaitEvent(s, evA1[ch - 2], 0));
        fp.stage = stg;
        cudaEventRecord(evF0[ch], s);
        for (int b = 0; b < nb; ++b) {
            FitParams q = bfp[b];
            const int64_t i0 = bucketed ? j.bucketOff[ch * nb + b] : fp.r0;
            const int64_t i1 = bucketed ? j.bucketOff[ch * nb + b + 1] : fp.r1;
            if (i1 <= i0) continue;
            q.stage = stg;
            int64_t step = q.bigMode ? bsub[b] : i1 - i0;
            if (onePer) step = std::min<int64_t>(step, (int64_t)nsm * 64);
            for (int64_t a = i0; a < i1; a += step) {
                q.r0 = a;
                q.r1 = std::min(i1, a + step);
                MPG_CUDA(c, launch_fit(q, nsm, 0, s));
                launches++;
                if (q.bigMode) {
                    MPG_CUDA(c, launch_update_big(q, s));
                    launches++;
                }
            }
        }
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
    MPG_CUDA(c, cudaMemsetAsync(iout, 0, sizeof(int64_t) * nint, s));
    StatParams sp{j.status, j.chi2add, j.ndfadd, j.chndf, j.rec, j.fileWeight, j.nrec, nf,
                  dout, iout, fout};
    MPG_CUDA(c, launch_stats(sp, s));
    launches += 2;
    cudaEventRecord(evEnd, s);
    return MPGPU_OK;
    };
    {
        // direct launches: the per-chunk fit and accumulation times come
        // from events on the launching streams, which a captured graph's
        // event nodes do not give
        const int32_t rcb = body();
        if (rcb != MPGPU_OK) return rcb;
    }
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
    // the per-call buffers are released on every return
    struct Bufs {
        int32_t *di = nullptr, *dj = nullptr;
        double *da = nullptr;
        ~Bufs() { dfree(di); dfree(dj); dfree(da); }
    } b;
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(b.di, i, n, s));
    MPG_CUDA(c, dupload(b.dj, jj, n, s));
    MPG_CUDA(c, dupload(b.da, add, n, s));
    int32_t *errFlag = (int32_t *)c->scal;
    MPG_CUDA(c, cudaMemsetAsync(errFlag, 0, 4, s));
    MPG_CUDA(c, launch_mupdat(n, b.di, b.dj, b.da, j, errFlag, s));
    int32_t h = 0;
    MPG_CUDA(c, cudaMemcpyAsync(&h, errFlag, 4, cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
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
    struct Bufs {
        int32_t *di = nullptr;
        double *da = nullptr;
        ~Bufs() { dfree(di); dfree(da); }
    } b;
    cudaStream_t s = c->stream;
    MPG_CUDA(c, dupload(b.di, vidx, n, s));
    MPG_CUDA(c, dupload(b.da, vadd, n, s));
    k_vadd<<<1, 32, 0, s>>>(n, b.di, b.da, c->j.gvec, c->j.nVar);
    MPG_CUDA(c, cudaGetLastError());
    MPG_CUDA(c, cudaStreamSynchronize(s));
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_download_matrix(mpgpu_ctx *c, double *globalMatD) {
    if (!c || !globalMatD) return MPGPU_ERR_ARG;
    MPG_CUDA(c, cudaMemcpy(globalMatD, c->j.matD, sizeof(double) * (size_t)c->j.nmat, cudaMemcpyDeviceToHost));
    return MPGPU_OK;
}

namespace {
// diagonal of the packed (row i at i(i+1)/2) or sparse (diagonal first) matrix
__global__ void k_matrix_diag(int32_t n, int32_t matsto, const double *m, double *d) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = matsto == 2 ? m[i] : m[i * (i + 1) / 2 + i];
}
}  // namespace

extern "C" int32_t mpgpu_matrix_diagonal(mpgpu_ctx *c, double *diagonal) {
    if (!c || !diagonal) return MPGPU_ERR_ARG;
    DevJob &j = c->j;
    if (!j.matD || j.nVar <= 0) return set_err(c, MPGPU_ERR_ARG, "no matrix");
    MPG_CUDA(c, cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    double *d = nullptr;
    MPG_CUDA(c, cudaMalloc(&d, sizeof(double) * j.nVar));
    k_matrix_diag<<<(j.nVar + 255) / 256, 256, 0, s>>>(j.nVar, j.matsto, j.matD, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(diagonal, d, sizeof(double) * j.nVar, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    return e == cudaSuccess ? MPGPU_OK : cuda_err(c, e, "mpgpu_matrix_diagonal");
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
    if (metsol == 1 || metsol == 3 || metsol == 31 || metsol == 32 || metsol == 11 || metsol == 12) {
        if (c->j.matsto != 1) return set_err(c, MPGPU_ERR_ARG, "inversion/decomposition need packed storage");
        const int dense = (metsol == 31 || metsol == 11) ? 1 : ((metsol == 32 || metsol == 12) ? 0 : -1);
        const bool inversion = metsol == 1 || metsol == 11 || metsol == 12;
        return solve_inversion(c, consResiduals, correction, errors, info, !inversion, dense, rtol, itnlim);
    }
    if (metsol == 4 || metsol == 5)
        return solve_minres(c, consResiduals, rtol, itnlim, correction, info, metsol == 5);
    return set_err(c, MPGPU_ERR_ARG, "unsupported solution method");
}

extern "C" int32_t mpgpu_set_preconditioner(mpgpu_ctx *c, int32_t mbandw, int32_t lprecm) {
    if (!c) return MPGPU_ERR_ARG;
    if (mbandw > MPGPU_BAND_WIDTH_MAX) return set_err(c, MPGPU_ERR_LIMIT, "band preconditioner wider than 32");
    c->mbandw = mbandw < 0 ? -1 : mbandw;
    c->lprecm = lprecm;
    return MPGPU_OK;
}

extern "C" int32_t mpgpu_band_factor(mpgpu_ctx *c, int32_t mbandw, int32_t lprecm, double *cOut, int32_t *nrkd) {
    if (!c || !cOut || !nrkd) return MPGPU_ERR_ARG;
    if (mbandw <= 0 || mbandw > MPGPU_BAND_WIDTH_MAX)
        return set_err(c, MPGPU_ERR_LIMIT, "band width outside 1..32");
    if (!c->j.matD) return set_err(c, MPGPU_ERR_ARG, "no matrix");
    cudaSetDevice(c->device);
    return band_precond_factor(c, mbandw, lprecm, cOut, nrkd);
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

extern "C" int32_t mpgpu_host_alloc(void **ptr, int64_t bytes) {
    if (!ptr || bytes <= 0) return MPGPU_ERR_ARG;
    *ptr = nullptr;
    return cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocPortable) == cudaSuccess ? MPGPU_OK : MPGPU_ERR_ALLOC;
}

extern "C" int32_t mpgpu_host_free(void *ptr) {
    if (!ptr) return MPGPU_ERR_ARG;
    return cudaFreeHost(ptr) == cudaSuccess ? MPGPU_OK : MPGPU_ERR_CUDA;
}
