// mille_io.cpp -- Mille binary files into record arrays (the file part of
// readFromBinary, pede.f90:1714-2075; record layout of mille.f90:27-59).
//
// A C-format record is an int32 header n (negative: double precision
// words), then |n|/2 float or double values (glder) and |n|/2 int32 values
// (inder).  A Fortran-format (sequential unformatted) record has the same
// payload framed by its byte length before and after.  The format is
// recognised per file from its first record.  Files compressed with gzip
// (recognised by their first two bytes; pede reads them through zlib) are
// read through the zlib runtime library, loaded when the first such file
// is met.
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/mpgpu.h"

namespace {

// the zlib calls used here, resolved from libz.so.1
struct Zlib {
    void *(*gzopen)(const char *, const char *) = nullptr;
    int (*gzread)(void *, void *, unsigned) = nullptr;
    int (*gzrewind)(void *) = nullptr;
    int (*gzclose)(void *) = nullptr;
    bool ok = false;
    Zlib() {
        void *h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) return;
        gzopen = (void *(*)(const char *, const char *))dlsym(h, "gzopen");
        gzread = (int (*)(void *, void *, unsigned))dlsym(h, "gzread");
        gzrewind = (int (*)(void *))dlsym(h, "gzrewind");
        gzclose = (int (*)(void *))dlsym(h, "gzclose");
        ok = gzopen && gzread && gzrewind && gzclose;
    }
};

const Zlib &zlib() {
    static Zlib z;
    return z;
}

struct MilleFile {
    FILE *f = nullptr;
    void *gz = nullptr;
    bool fortran = false;
    ~MilleFile() {
        if (f) std::fclose(f);
        if (gz) zlib().gzclose(gz);
    }
    bool read(void *dst, size_t bytes) {
        if (gz) {
            char *d = static_cast<char *>(dst);
            while (bytes > 0) {
                const unsigned part = bytes > (1u << 30) ? (1u << 30) : (unsigned)bytes;
                if (zlib().gzread(gz, d, part) != (int)part) return false;
                d += part;
                bytes -= part;
            }
            return true;
        }
        return std::fread(dst, 1, bytes, f) == bytes;
    }
    void rewind() {
        if (gz) zlib().gzrewind(gz);
        else std::rewind(f);
    }
};

bool read_i32(MilleFile &mf, int32_t &v) { return mf.read(&v, 4); }

// format of the file from its first record: Fortran when the leading word
// equals the payload length implied by the header that follows it
int open_mille(const char *path, MilleFile &mf) {
    mf.f = std::fopen(path, "rb");
    if (!mf.f) return MPGPU_ERR_ARG;
    unsigned char magic[2] = {0, 0};
    const bool gzip = std::fread(magic, 1, 2, mf.f) == 2 && magic[0] == 0x1f && magic[1] == 0x8b;
    if (gzip) {
        std::fclose(mf.f);
        mf.f = nullptr;
        if (!zlib().ok) return MPGPU_ERR_ARG;
        mf.gz = zlib().gzopen(path, "rb");
        if (!mf.gz) return MPGPU_ERR_ARG;
    }
    mf.rewind();
    int32_t a = 0, b = 0;
    if (!read_i32(mf, a)) { mf.fortran = false; mf.rewind(); return MPGPU_OK; }
    if (read_i32(mf, b) && b != 0) {
        const int64_t nw = b < 0 ? -(int64_t)b / 2 : (int64_t)b / 2;
        const int64_t bytes = 4 + nw * (b < 0 ? 8 : 4) + nw * 4;
        mf.fortran = (int64_t)a == bytes;
    }
    mf.rewind();
    return MPGPU_OK;
}

// next record: returns 1 with the words appended, 0 at the end, <0 on a
// damaged record
int next_record(MilleFile &mf, std::vector<int32_t> &in, std::vector<double> &gl) {
    int32_t lead = 0, n = 0;
    if (mf.fortran) {
        if (!read_i32(mf, lead)) return 0;
        if (!read_i32(mf, n)) return -1;
    } else {
        if (!read_i32(mf, n)) return 0;
    }
    if (n == 0 || n == INT32_MIN) return -1;
    const bool dbl = n < 0;
    const int64_t nw = (dbl ? -(int64_t)n : (int64_t)n) / 2;
    if (nw <= 0 || nw > MPGPU_FILE_WORDS_MAX) return -1;
    const size_t g0 = gl.size(), i0 = in.size();
    gl.resize(g0 + nw);
    in.resize(i0 + nw);
    if (dbl) {
        if (!mf.read(gl.data() + g0, 8 * (size_t)nw)) return -1;
    } else {
        std::vector<float> tmp(nw);
        if (!mf.read(tmp.data(), 4 * (size_t)nw)) return -1;
        for (int64_t k = 0; k < nw; ++k) gl[g0 + k] = tmp[k];
    }
    if (!mf.read(in.data() + i0, 4 * (size_t)nw)) return -1;
    if (mf.fortran) {
        int32_t trail = 0;
        if (!read_i32(mf, trail) || trail != lead) return -1;
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
