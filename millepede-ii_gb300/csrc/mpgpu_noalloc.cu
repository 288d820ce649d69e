// mpgpu_noalloc.cu -- mupdat that stages its input in a fixed, statically
// reserved device area instead of device memory allocated per call.
//
// mpgpu_mupdat copies the caller's (i, j, add) triplets into device buffers
// that it allocates and frees on every call.  Two kinds of caller cannot
// accept that:
//  * a host loop that adds measurement lines or presigma terms to the
//    global matrix while the same device still runs other work on another
//    stream: cudaFree waits for the whole device, so every call would stall
//    the overlapped work;
//  * a job sized so that the global matrix and the update staging fill the
//    device memory: a small allocation in the middle of the run can then
//    fail, or fragment the memory the next large allocation needs.
// mpgpu_mupdat_noalloc stages the triplets in one file-scope __device__
// array of fixed size and runs the same k_mupdat kernel on them.  It never
// allocates or frees device memory.
//
// Limits and rules of use:
//  * at most MPGPU_MUPDAT_NOALLOC_MAX triplets per call; a larger call is
//    rejected with MPGPU_ERR_LIMIT before anything is copied or launched;
//  * the area is one per device, shared by every context on that device:
//    calls that overlap in time on one device (from two host threads, or
//    through two contexts) race on it and can apply each other's triplets,
//    so the caller must serialise them;
//  * the area's device memory is reserved when the CUDA module holding it
//    is loaded; CUDA loads modules lazily (on first use), so mpgpu_create
//    looks up the area's address on its device right away
//    (noalloc_prepare): from the first context on a device onward the area
//    is in place, before the job's large allocations, and no call of
//    mpgpu_mupdat_noalloc loads a module or reserves memory.  The address
//    is kept per device; a call on a device without a context made there
//    first looks it up itself, and should then come before any stream
//    capture is begun on that device.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "mpgpu_ctx.h"

namespace {
constexpr int64_t kNoallocMax = MPGPU_MUPDAT_NOALLOC_MAX;
// area layout: status word in the first 256 bytes, then i[kNoallocMax],
// j[kNoallocMax] (int32) and add[kNoallocMax] (double)
constexpr size_t kOffI = 256;
constexpr size_t kOffJ = kOffI + sizeof(int32_t) * kNoallocMax;
constexpr size_t kOffA = kOffJ + sizeof(int32_t) * kNoallocMax;
constexpr size_t kScratchBytes = kOffA + sizeof(double) * kNoallocMax;
static_assert(kOffA % alignof(double) == 0, "add[] must be 8-byte aligned");
}  // namespace

// 1 MiB + 256 bytes per device, reserved when the module is loaded (at
// mpgpu_create on that device, through noalloc_prepare)
static __device__ __align__(256) unsigned char g_mupdatScratch[kScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setupLock;
unsigned char *g_scratchAddr[kMaxDevices] = {};

// device address of the area on the context's device (the device must be
// current); looked up once per device
int32_t scratch_address(mpgpu_ctx *c, unsigned char **out) {
    if (c->device < 0 || c->device >= kMaxDevices)
        return set_err(c, MPGPU_ERR_ARG, "mupdat_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> guard(g_setupLock);
    if (!g_scratchAddr[c->device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_mupdatScratch);
        if (e != cudaSuccess) return cuda_err(c, e, "cudaGetSymbolAddress(mupdat scratch)");
        if (!p) return set_err(c, MPGPU_ERR_CUDA, "mupdat_noalloc: null scratch address");
        g_scratchAddr[c->device] = static_cast<unsigned char *>(p);
    }
    *out = g_scratchAddr[c->device];
    return MPGPU_OK;
}
}  // namespace

// Called by mpgpu_create with the context's device current: loads the
// module and resolves the area's address once per device.
int32_t noalloc_prepare(mpgpu_ctx *c) {
    unsigned char *base = nullptr;
    return scratch_address(c, &base);
}

extern "C" int32_t mpgpu_mupdat_noalloc(mpgpu_ctx *c, int32_t n, const int32_t *i, const int32_t *jj,
                                        const double *add) {
    if (!c || n < 0) return MPGPU_ERR_ARG;
    if (n > kNoallocMax)
        return set_err(c, MPGPU_ERR_LIMIT,
                       "mupdat_noalloc: " + std::to_string(n) + " elements exceed the scratch capacity of " +
                           std::to_string(kNoallocMax));
    if (n == 0) return MPGPU_OK;
    if (!i || !jj || !add) return set_err(c, MPGPU_ERR_ARG, "mupdat_noalloc: null input array");
    DevJob &j = c->j;
    if (!j.matD) return set_err(c, MPGPU_ERR_ARG, "mupdat_noalloc: no layout set");
    MPG_CUDA(c, cudaSetDevice(c->device));
    unsigned char *base = nullptr;
    const int32_t rc = scratch_address(c, &base);
    if (rc) return rc;
    int32_t *dStatus = reinterpret_cast<int32_t *>(base);
    int32_t *di = reinterpret_cast<int32_t *>(base + kOffI);
    int32_t *dj = reinterpret_cast<int32_t *>(base + kOffJ);
    double *da = reinterpret_cast<double *>(base + kOffA);
    cudaStream_t s = c->stream;
    // the status word must start at zero: the kernel only ever sets it
    MPG_CUDA(c, cudaMemsetAsync(dStatus, 0, sizeof(int32_t), s));
    MPG_CUDA(c, cudaMemcpyAsync(di, i, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, cudaMemcpyAsync(dj, jj, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, cudaMemcpyAsync(da, add, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    MPG_CUDA(c, launch_mupdat(n, di, dj, da, j, dStatus, s));
    int32_t h = 0;
    MPG_CUDA(c, cudaMemcpyAsync(&h, dStatus, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    MPG_CUDA(c, cudaStreamSynchronize(s));
    if (h) return set_err(c, h, "mupdat index outside the matrix");
    return MPGPU_OK;
}
