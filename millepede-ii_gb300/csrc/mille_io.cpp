// mille_io.cpp -- Mille binary files into record arrays (the file part of
// readFromBinary, pede.f90:1714-2075; record layout of mille.f90:27-59).
//
// A C-format record is an int32 header n (negative: double precision
// words), then |n|/2 float or double values (glder) and |n|/2 int32 values
// (inder).  A Fortran-format (sequential unformatted) record has the same
// payload framed by its byte length before and after.  The format is
// recognised per file from its first record.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/mpgpu.h"

namespace {

struct MilleFile {
    FILE *f = nullptr;
    bool fortran = false;
    ~MilleFile() {
        if (f) std::fclose(f);
    }
};

bool read_i32(FILE *f, int32_t &v) { return std::fread(&v, 4, 1, f) == 1; }

// format of the file from its first record: Fortran when the leading word
// equals the payload length implied by the header that follows it
int open_mille(const char *path, MilleFile &mf) {
    mf.f = std::fopen(path, "rb");
    if (!mf.f) return MPGPU_ERR_ARG;
    int32_t a = 0, b = 0;
    if (!read_i32(mf.f, a)) { mf.fortran = false; std::rewind(mf.f); return MPGPU_OK; }
    if (read_i32(mf.f, b) && b != 0) {
        const int64_t nw = b < 0 ? -(int64_t)b / 2 : (int64_t)b / 2;
        const int64_t bytes = 4 + nw * (b < 0 ? 8 : 4) + nw * 4;
        mf.fortran = (int64_t)a == bytes;
    }
    std::rewind(mf.f);
    return MPGPU_OK;
}

// next record: returns 1 with the words appended, 0 at the end, <0 on a
// damaged record
int next_record(MilleFile &mf, std::vector<int32_t> &in, std::vector<double> &gl) {
    int32_t lead = 0, n = 0;
    if (mf.fortran) {
        if (!read_i32(mf.f, lead)) return 0;
        if (!read_i32(mf.f, n)) return -1;
    } else {
        if (!read_i32(mf.f, n)) return 0;
    }
    if (n == 0 || n == INT32_MIN) return -1;
    const bool dbl = n < 0;
    const int64_t nw = (dbl ? -(int64_t)n : (int64_t)n) / 2;
    if (nw <= 0 || nw > MPGPU_FILE_WORDS_MAX) return -1;
    const size_t g0 = gl.size(), i0 = in.size();
    gl.resize(g0 + nw);
    in.resize(i0 + nw);
    if (dbl) {
        if (std::fread(gl.data() + g0, 8, nw, mf.f) != (size_t)nw) return -1;
    } else {
        std::vector<float> tmp(nw);
        if (std::fread(tmp.data(), 4, nw, mf.f) != (size_t)nw) return -1;
        for (int64_t k = 0; k < nw; ++k) gl[g0 + k] = tmp[k];
    }
    if (std::fread(in.data() + i0, 4, nw, mf.f) != (size_t)nw) return -1;
    if (mf.fortran) {
        int32_t trail = 0;
        if (!read_i32(mf.f, trail) || trail != lead) return -1;
    }
    return 1;
}

}  // namespace

extern "C" int32_t mpgpu_read_mille(int32_t nfiles, const char *const *files, int64_t maxRec, int64_t cap,
                                    int64_t *nrec, int64_t *nw, int64_t *recPtr, int32_t *inder,
                                    double *glder, int32_t *recFile) {
    if (nfiles < 1 || !files || !nrec || !nw) return MPGPU_ERR_ARG;
    *nrec = 0;
    *nw = 0;
    int64_t r = 0, w = 0;
    std::vector<int32_t> in;
    std::vector<double> gl;
    if (recPtr) recPtr[0] = 0;
    for (int32_t fi = 0; fi < nfiles; ++fi) {
        MilleFile mf;
        const int32_t rc = open_mille(files[fi], mf);
        if (rc) return rc;
        int64_t rf = 0;
        for (;;) {
            if (maxRec > 0 && rf >= maxRec) break;
            in.clear();
            gl.clear();
            const int st = next_record(mf, in, gl);
            if (st == 0) break;
            if (st < 0) return MPGPU_ERR_BADRECORD;
            const int64_t k = (int64_t)in.size();
            if (inder) {
                if (w + k > cap) return MPGPU_ERR_SIZE;
                std::memcpy(inder + w, in.data(), 4 * k);
                std::memcpy(glder + w, gl.data(), 8 * k);
                recPtr[r + 1] = w + k;
                if (recFile) recFile[r] = fi + 1;
            }
            w += k;
            r++;
            rf++;
        }
    }
    *nrec = r;
    *nw = w;
    return MPGPU_OK;
}
