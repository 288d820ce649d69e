"""ctypes binding of libmpgpu.so (include/mpgpu.h).

The Python side is a thin caller of the C-ABI, the same entry points the
Fortran pede host binds through ISO_C_BINDING.  Loading fails loudly when the
library has not been built: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")
LIBPATH = os.path.join(LIBDIR, "libmpgpu.so")

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)


# mpgpu_cfg flags (include/mpgpu.h)
FLAG_LARGE_RECORDS = 1
FLAG_NO_BUCKETS = 2
FLAG_ONE_RECORD_PER_BLOCK = 4
FLAG_NO_AUTOTUNE = 8


class MonitorCfg(C.Structure):
    _fields_ = [("nbins", C.c_int32), ("range", C.c_float), ("measBins", C.c_int32),
                ("mode", C.c_int32), ("lfitnp", C.c_int32)]


def monitor_groups(S):
    """Monitor groups of a HostStructure's translated records:
    (measIndex[nTotal], measRes[numMeas])."""
    mi = np.zeros(S.nTotal, np.int32)
    mr = np.zeros(max(S.nTotal, 1), np.float64)
    n = C.c_int32()
    rc = lib().mpgpu_monitor_groups(C.c_int64(len(S.recPtr) - 1), ptr(S.recPtr, i64p), ptr(S.tinder, i32p),
                                    ptr(S.glder, f64p), C.c_int32(S.nTotal), ptr(mi, i32p), ptr(mr, f64p),
                                    C.byref(n))
    if rc:
        raise RuntimeError(f"mpgpu_monitor_groups failed ({rc})")
    return mi, mr[:n.value].copy()


def write_mon(path, header, mode, nloopn, group_labels, meas_hists, meas_res):
    gl = np.ascontiguousarray(group_labels, np.int32)
    mh = np.ascontiguousarray(meas_hists, np.int64)
    mr = np.ascontiguousarray(meas_res, np.float64)
    rc = lib().mpgpu_write_mon(str(path).encode(), C.c_int32(header), C.c_int32(mode), C.c_int32(nloopn),
                               C.c_int32(len(gl)), ptr(gl, i32p), ptr(mh.reshape(-1), i64p),
                               C.c_int32(mh.shape[1] if mh.ndim == 2 else 100), ptr(mr, f64p))
    if rc:
        raise RuntimeError(f"mpgpu_write_mon failed ({rc})")


class MpgpuCfg(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_int32), ("staging_bytes", C.c_int64)]


class FitOpts(C.Structure):
    _fields_ = [("icalcm", C.c_int32), ("nloopn", C.c_int32), ("lhuber", C.c_int32),
                ("lfitbb", C.c_int32), ("chicut", C.c_float), ("chhuge", C.c_float),
                ("dwcut", C.c_float), ("cndlmx", C.c_float)]


class FitStats(C.Structure):
    _fields_ = [("nrej", C.c_int64 * 6), ("chi2SumI", C.c_int64), ("chi2SumD", C.c_double),
                ("ndfSum", C.c_int64), ("ndfSumW", C.c_double), ("nbndr", C.c_int32 * 2),
                ("nbdrx", C.c_int32), ("nbndx", C.c_int32), ("naccepted", C.c_int64),
                ("msFit", C.c_double), ("msAccum", C.c_double), ("msLoop", C.c_double),
                ("launches", C.c_int32), ("pad", C.c_int32)]


class SolveInfo(C.Structure):
    _fields_ = [("nrank", C.c_int32), ("itn", C.c_int32), ("istop", C.c_int32),
                ("nrkd", C.c_int32), ("evmin", C.c_double), ("evmax", C.c_double),
                ("ms", C.c_double), ("msFactor", C.c_double), ("msRefine", C.c_double),
                ("dxRel", C.c_double), ("msInverse", C.c_double), ("factorReused", C.c_int32),
                ("itnReuse", C.c_int32)]


class Steer(C.Structure):
    _fields_ = [("metsol", C.c_int32), ("matsto", C.c_int32), ("mitera", C.c_int32),
                ("lhuber", C.c_int32), ("chicut", C.c_float), ("chirem", C.c_float),
                ("chhuge", C.c_float), ("dwcut", C.c_float), ("cndlmx", C.c_float),
                ("lfitbb", C.c_int32), ("mreqenf", C.c_int32), ("mreqena", C.c_int32),
                ("mreqpe", C.c_int32), ("mrestl", C.c_double), ("itnlim", C.c_int32),
                ("nthreads", C.c_int32), ("structDevice", C.c_int32), ("monitor", C.c_int32),
                ("monitorPulls", C.c_int32), ("monitorBins", C.c_int32),
                ("mbandw", C.c_int32), ("lprecm", C.c_int32)]


class Job(C.Structure):
    _fields_ = [("nrec", C.c_int64), ("recPtr", i64p), ("inder", i32p), ("glder", f64p),
                ("recFile", i32p), ("nfiles", C.c_int32), ("fileWeight", f64p),
                ("npar", C.c_int32), ("parLabel", i32p), ("parValue", f64p),
                ("parSigma", f64p),
                ("ncon", C.c_int32), ("conStart", i32p), ("conLabel", i32p),
                ("conCoef", f64p), ("conRhs", f64p),
                ("nmeas", C.c_int32), ("msStart", i32p), ("msLabel", i32p),
                ("msCoef", f64p), ("msRhs", f64p), ("msSigma", f64p), ("monPath", C.c_char_p)]


class Result(C.Structure):
    _fields_ = [("cap", C.c_int32), ("nTotal", C.c_int32), ("nVar", C.c_int32),
                ("nVarGroups", C.c_int32), ("nFit", C.c_int32),
                ("labels", i32p), ("parameter", f64p), ("presigma", f64p), ("error", f64p),
                ("counts", i64p), ("varIndex", i32p),
                ("nrej", C.c_int64 * 6), ("fvalue", C.c_double), ("ndf", C.c_int64),
                ("nrank", C.c_int32), ("minresItn", C.c_int32), ("minresIstop", C.c_int32),
                ("nloopn", C.c_int32), ("exitCode", C.c_int32),
                ("msBuild", C.c_double), ("msSolve", C.c_double),
                ("start", f64p), ("gcor", f64p), ("fileCounts", i64p),
                ("msStructure", C.c_double), ("msUpload", C.c_double), ("msLoops", C.c_double),
                ("msSolves", C.c_double), ("msHostIter", C.c_double), ("msJob", C.c_double)]


class ResOpts(C.Structure):
    _fields_ = [("errors", C.c_int32), ("ipcntr", C.c_int32), ("igcorr", C.c_int32),
                ("mreqena", C.c_int32)]


class GenCfg(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nlayers", C.c_int32), ("nmod", C.c_int32),
                ("minHits", C.c_int32), ("maxHits", C.c_int32), ("ntracks", C.c_int64),
                ("seed", C.c_uint64), ("sigma1", C.c_double), ("sigma2", C.c_double),
                ("misal", C.c_double), ("outlierFrac", C.c_double), ("theta0", C.c_double),
                ("threads", C.c_int32)]


def ptr(a, t):
    """ctypes pointer to a contiguous numpy array (None -> NULL)."""
    if a is None:
        return C.cast(None, t)
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(t)


_lib = None


def lib():
    """Load libmpgpu.so; raises when it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"libmpgpu.so not built ({LIBPATH}); run __graft_entry__.build()")
        L = C.CDLL(LIBPATH)
        for f in ("mpgpu_last_error", "mpgpu_server_last_error"):
            if hasattr(L, f):
                getattr(L, f).restype = C.c_char_p
        _lib = L
    return _lib


EXPORTS = [
    "mpgpu_create", "mpgpu_destroy", "mpgpu_last_error", "mpgpu_set_layout",
    "mpgpu_set_constraints", "mpgpu_upload_records", "mpgpu_loopbf", "mpgpu_loopbf_device",
    "mpgpu_mupdat", "mpgpu_mupdat_noalloc", "mpgpu_set_preconditioner", "mpgpu_band_factor", "mpgpu_vector_add", "mpgpu_download_matrix", "mpgpu_download_vector",
    "mpgpu_download_record_status", "mpgpu_solve", "mpgpu_avprod", "mpgpu_probe_fp64",
    "mpgpu_dense_cholesky", "mpgpu_upload_timing", "mpgpu_fit_buckets",
    "mpgpu_set_monitor", "mpgpu_get_monitor", "mpgpu_monitor_groups", "mpgpu_write_mon",
    "mpgpu_server_create", "mpgpu_server_submit", "mpgpu_server_wait", "mpgpu_server_destroy",
    "mpgpu_server_last_error",
    "mpgpu_read_mille",
    "mpgpu_host_register", "mpgpu_host_unregister", "mpgpu_host_alloc", "mpgpu_host_free",
    "mpgpu_host_labels",
    "mpgpu_host_translate", "mpgpu_host_mpbits", "mpgpu_host_mpbits_pairentries",
    "mpgpu_set_suppressed_pairs", "mpgpu_loop1_device", "mpgpu_loop2_device", "mpgpu_pede_run", "mpgpu_write_res",
    "mpgpu_write_res_opts", "mpgpu_matrix_diagonal", "mpgpu_release",
    "mpgen_count", "mpgen_fill", "mpgen_constraints", "mpgen_constraint_words",
]


# ----------------------------------------------------------------- data
def gen_config(name, ntracks=None, seed=None):
    """Named synthetic workloads (sizes of the benchmark configurations)."""
    if name == "telescope":      # 10 layers x 20 modules, 200 x-shifts
        c = GenCfg(kind=1, nlayers=10, nmod=20, ntracks=5000, seed=1, sigma1=0.005,
                   sigma2=0.005, misal=0.01)
    elif name == "barrel":       # 5000 modules x 6 dof = 30000 globals
        c = GenCfg(kind=2, nmod=5000, ntracks=2_000_000, seed=2, sigma1=0.002, sigma2=0.008,
                   misal=0.005)
    elif name == "brokenlines":  # barrel, 4..40 hits, nloc 8..84
        c = GenCfg(kind=3, nmod=5000, minHits=4, maxHits=40, ntracks=1_000_000, seed=3,
                   sigma1=0.002, sigma2=0.008, misal=0.005, theta0=0.001)
    elif name == "telescope_dense":  # telescope scaled up in module count
        c = GenCfg(kind=1, nlayers=10, nmod=2000, ntracks=400_000, seed=4, sigma1=0.005,
                   sigma2=0.005, misal=0.01)
    else:
        raise ValueError(name)
    if ntracks is not None:
        c.ntracks = ntracks
    if seed is not None:
        c.seed = seed
    return c


def generate(cfg):
    """Mille records (recPtr, inder, glder), true misalignments, constraints."""
    L = lib()
    nrec, nw, nlab = C.c_int64(), C.c_int64(), C.c_int32()
    rc = L.mpgen_count(C.byref(cfg), C.byref(nrec), C.byref(nw), C.byref(nlab))
    assert rc == 0, rc
    recPtr = np.zeros(nrec.value + 1, np.int64)
    inder = np.zeros(nw.value, np.int32)
    glder = np.zeros(nw.value, np.float64)
    truth = np.zeros(nlab.value, np.float64)
    rc = L.mpgen_fill(C.byref(cfg), ptr(recPtr, i64p), ptr(inder, i32p), ptr(glder, f64p),
                      ptr(truth, f64p))
    assert rc == 0, rc
    ncon = C.c_int32()
    L.mpgen_constraints(C.byref(cfg), C.byref(ncon), None, None, None)
    nwc = L.mpgen_constraint_words(C.byref(cfg))
    conStart = np.zeros(ncon.value + 1, np.int32)
    conLabel = np.zeros(nwc, np.int32)
    conCoef = np.zeros(nwc, np.float64)
    L.mpgen_constraints(C.byref(cfg), C.byref(ncon), ptr(conStart, i32p), ptr(conLabel, i32p),
                        ptr(conCoef, f64p))
    return dict(recPtr=recPtr, inder=inder, glder=glder, truth=truth, conStart=conStart,
                conLabel=conLabel, conCoef=conCoef, ncon=ncon.value)


def write_mille_c(path, recPtr, inder, glder):
    """Write records as a C-format double-precision Mille binary file
    (int32 header -2*w, w doubles, w int32; python/readMilleBinary.py)."""
    with open(path, "wb") as f:
        for r in range(len(recPtr) - 1):
            a, b = recPtr[r], recPtr[r + 1]
            np.array([-2 * (b - a)], np.int32).tofile(f)
            glder[a:b].tofile(f)
            inder[a:b].tofile(f)


def read_mille(paths, max_rec=0):
    """Records of Mille binary files through mpgpu_read_mille (C or Fortran
    framing, float or double): (recPtr, inder, glder, recFile)."""
    L = lib()
    arr = (C.c_char_p * len(paths))(*[p.encode() for p in paths])
    nrec, nw = C.c_int64(), C.c_int64()
    rc = L.mpgpu_read_mille(C.c_int32(len(paths)), arr, C.c_int64(max_rec), C.c_int64(0), C.byref(nrec),
                            C.byref(nw), None, None, None, None)
    if rc != 0:
        raise RuntimeError(f"mpgpu_read_mille: {rc}")
    recPtr = np.zeros(nrec.value + 1, np.int64)
    inder = np.zeros(nw.value, np.int32)
    glder = np.zeros(nw.value, np.float64)
    recFile = np.zeros(nrec.value, np.int32)
    rc = L.mpgpu_read_mille(C.c_int32(len(paths)), arr, C.c_int64(max_rec), C.c_int64(nw.value),
                            C.byref(nrec), C.byref(nw), ptr(recPtr, i64p), ptr(inder, i32p),
                            ptr(glder, f64p), ptr(recFile, i32p))
    if rc != 0:
        raise RuntimeError(f"mpgpu_read_mille: {rc}")
    return recPtr, inder, glder, recFile


def read_mille_c(path):
    """Read a C-format Mille binary file (float or double records)."""
    data = open(path, "rb").read()
    pos, ptrs, ints, dbls = 0, [0], [], []
    while pos < len(data):
        h = int(np.frombuffer(data, np.int32, 1, pos)[0]); pos += 4
        w = abs(h) // 2
        if h < 0:
            d = np.frombuffer(data, np.float64, w, pos); pos += 8 * w
        else:
            d = np.frombuffer(data, np.float32, w, pos).astype(np.float64); pos += 4 * w
        i = np.frombuffer(data, np.int32, w, pos); pos += 4 * w
        ints.append(i); dbls.append(d); ptrs.append(ptrs[-1] + w)
    return (np.array(ptrs, np.int64), np.concatenate(ints).astype(np.int32),
            np.concatenate(dbls).astype(np.float64))


# ----------------------------------------------------------------- host side
class HostStructure:
    """loop1/loop2 products computed by the library's host side:
    sorted labels, entries, variable indices, parameter groups, translated
    records and (sparse storage) the mpbits row structure; with mreqpe > 1
    (pairentries) the group pairs met fewer times are left out and listed in
    `suppressed` (one (row group, column group) pair per row)."""

    def __init__(self, data, mreqenf=25, steerLabels=(), preLabel=(), preSigma=(), sparse=True,
                 mreqpe=1):
        L = lib()
        self.recPtr = np.ascontiguousarray(data["recPtr"], np.int64)
        inder = np.ascontiguousarray(data["inder"], np.int32)
        self.glder = np.ascontiguousarray(data["glder"], np.float64)
        nrec = len(self.recPtr) - 1
        cap = len(inder) + len(steerLabels) + 16
        labels = np.zeros(cap, np.int32)
        counter = np.zeros(cap, np.int64)
        varIndex = np.zeros(cap, np.int32)
        totGroup = np.zeros(cap, np.int32)
        nVar, nG = C.c_int32(), C.c_int32()
        sl = np.ascontiguousarray(steerLabels, np.int32)
        pl = np.ascontiguousarray(preLabel, np.int32)
        ps = np.ascontiguousarray(preSigma, np.float64)
        n = L.mpgpu_host_labels(C.c_int64(nrec), ptr(self.recPtr, i64p), ptr(inder, i32p),
                                ptr(self.glder, f64p), C.c_int32(len(sl)), ptr(sl, i32p),
                                C.c_int32(len(pl)), ptr(pl, i32p), ptr(ps, f64p),
                                C.c_int32(mreqenf), C.c_int32(cap), ptr(labels, i32p),
                                ptr(counter, i64p), ptr(varIndex, i32p), ptr(totGroup, i32p),
                                C.byref(nVar), C.byref(nG))
        if n < 0:
            raise RuntimeError(f"mpgpu_host_labels failed ({n})")
        self._tables(n, labels, counter, varIndex, totGroup, nVar.value, nG.value)
        self.rawInder = inder
        self.tinder = np.zeros_like(inder)
        rc = L.mpgpu_host_translate(C.c_int64(nrec), ptr(self.recPtr, i64p), ptr(inder, i32p),
                                    ptr(self.glder, f64p), C.c_int32(n), ptr(self.labels, i32p),
                                    ptr(self.tinder, i32p))
        if rc:
            raise RuntimeError(f"mpgpu_host_translate failed ({rc})")
        self.offsets = np.zeros(2 * (self.nG + 1), np.int64)
        self.columns = np.zeros(1, np.int32)
        self.suppressed = np.zeros((0, 2), np.int32)
        self.ncolw = 0
        self.nmatSparse = 0
        if sparse:
            capc, caps = 1 << 20, 0
            while True:
                cols = np.zeros(capc, np.int32)
                sup = np.zeros(2 * max(caps, 1), np.int32)
                ncolw, nmat, nsup = C.c_int64(), C.c_int64(), C.c_int64()
                if mreqpe > 1:
                    rc = L.mpgpu_host_mpbits_pairentries(
                        C.c_int64(nrec), C.c_int64(nrec), ptr(self.recPtr, i64p),
                        ptr(self.tinder, i32p), ptr(self.glder, f64p), ptr(self.varIndex, i32p),
                        C.c_int32(self.nVar), C.c_int32(self.nG), ptr(self.aig, i32p),
                        C.c_int32(mreqpe), C.c_int64(capc), ptr(self.offsets, i64p),
                        ptr(cols, i32p), C.byref(ncolw), C.byref(nmat), C.c_int64(caps),
                        ptr(sup, i32p), C.byref(nsup))
                else:
                    rc = L.mpgpu_host_mpbits(C.c_int64(nrec), ptr(self.recPtr, i64p),
                                             ptr(self.tinder, i32p), ptr(self.glder, f64p),
                                             ptr(self.varIndex, i32p), C.c_int32(self.nVar),
                                             C.c_int32(self.nG), ptr(self.aig, i32p), C.c_int64(capc),
                                             ptr(self.offsets, i64p), ptr(cols, i32p),
                                             C.byref(ncolw), C.byref(nmat))
                if rc == 0:
                    break
                if rc != -1:
                    raise RuntimeError(f"mpgpu_host_mpbits failed ({rc})")
                capc, caps = max(capc * 4, ncolw.value), nsup.value
            self.suppressed = sup[:2 * nsup.value].reshape(-1, 2).copy()
            self.columns = cols[:max(ncolw.value, 1)].copy()
            self.ncolw, self.nmatSparse = ncolw.value, nmat.value
        self.nmatPacked = self.nVar * (self.nVar + 1) // 2


    def _tables(self, n, labels, counter, varIndex, totGroup, nVar, nG):
        self.nTotal = n
        self.labels, self.counter = labels[:n].copy(), counter[:n].copy()
        self.varIndex, self.totGroup = varIndex[:n].copy(), totGroup[:n].copy()
        self.nVar, self.nG = nVar, nG
        var = self.varIndex > 0
        tg = self.totGroup[var]
        heads = np.ones(len(tg), bool)
        heads[1:] = tg[1:] != tg[:-1]
        self.aig = np.append(self.varIndex[var][heads], self.nVar + 1).astype(np.int32)


class DeviceStructure(HostStructure):
    """The tables of HostStructure computed on the device
    (mpgpu_loop1_device, mpgpu_loop2_device).  The translated records stay
    on the context's device; ctx.upload(S) takes them over without a copy
    (once)."""

    def __init__(self, ctx, data, mreqenf=25, steerLabels=(), preLabel=(), preSigma=(), sparse=True):
        L = lib()
        self.resident = True
        self.recPtr = np.ascontiguousarray(data["recPtr"], np.int64)
        inder = np.ascontiguousarray(data["inder"], np.int32)
        self.glder = np.ascontiguousarray(data["glder"], np.float64)
        nrec = len(self.recPtr) - 1
        cap = len(inder) + len(steerLabels) + 16
        labels = np.zeros(cap, np.int32)
        counter = np.zeros(cap, np.int64)
        varIndex = np.zeros(cap, np.int32)
        totGroup = np.zeros(cap, np.int32)
        nVar, nG = C.c_int32(), C.c_int32()
        sl = np.ascontiguousarray(steerLabels, np.int32)
        pl = np.ascontiguousarray(preLabel, np.int32)
        ps = np.ascontiguousarray(preSigma, np.float64)
        n = L.mpgpu_loop1_device(ctx.h, C.c_int64(nrec), ptr(self.recPtr, i64p), ptr(inder, i32p),
                                 ptr(self.glder, f64p), C.c_int32(len(sl)), ptr(sl, i32p),
                                 C.c_int32(len(pl)), ptr(pl, i32p), ptr(ps, f64p),
                                 C.c_int32(mreqenf), C.c_int32(cap), ptr(labels, i32p),
                                 ptr(counter, i64p), ptr(varIndex, i32p), ptr(totGroup, i32p),
                                 C.byref(nVar), C.byref(nG))
        if n < 0:
            raise RuntimeError(f"mpgpu_loop1_device failed ({n}): {ctx.last_error()}")
        self._tables(n, labels, counter, varIndex, totGroup, nVar.value, nG.value)
        self.tinder = None
        self.offsets = np.zeros(2 * (self.nG + 1), np.int64)
        self.columns = np.zeros(1, np.int32)
        self.ncolw = 0
        self.nmatSparse = 0
        if sparse:
            ncolw, nmat = C.c_int64(), C.c_int64()
            cols = np.zeros(1 << 20, np.int32)
            for _ in range(2):
                rc = L.mpgpu_loop2_device(ctx.h, ptr(self.varIndex, i32p), C.c_int32(self.nVar),
                                          C.c_int32(self.nG), ptr(self.aig, i32p),
                                          C.c_int64(len(cols)), ptr(self.offsets, i64p),
                                          ptr(cols, i32p), C.byref(ncolw), C.byref(nmat))
                if rc != -1:
                    break
                cols = np.zeros(max(ncolw.value, 1), np.int32)
            if rc != 0:
                raise RuntimeError(f"mpgpu_loop2_device failed ({rc}): {ctx.last_error()}")
            self.columns = cols[:max(ncolw.value, 1)].copy()
            self.ncolw, self.nmatSparse = ncolw.value, nmat.value
        self.nmatPacked = self.nVar * (self.nVar + 1) // 2


class Context:
    """One device context with a layout and uploaded records."""

    def __init__(self, device=0, staging_bytes=0, flags=0):
        self.L = lib()
        self.h = C.c_void_p()
        cfg = MpgpuCfg(device=device, flags=flags, staging_bytes=staging_bytes)
        self.check(self.L.mpgpu_create(C.byref(self.h), C.byref(cfg)))

    def last_error(self):
        msg = self.L.mpgpu_last_error(self.h) if self.h else b""
        return msg.decode() if msg else ""

    def check(self, rc):
        if rc != 0:
            msg = self.L.mpgpu_last_error(self.h) if self.h else b""
            raise RuntimeError(f"mpgpu error {rc}: {msg.decode() if msg else ''}")

    def close(self):
        if self.h:
            self.L.mpgpu_destroy(self.h)
            self.h = C.c_void_p()

    def release(self):
        """Free the current job's device memory (mpgpu_release)."""
        self.check(self.L.mpgpu_release(self.h))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_layout(self, S, matsto):
        self.nVar, self.nTotal, self.matsto = S.nVar, S.nTotal, matsto
        self.ncon = 0
        self.nmat = S.nmatSparse if matsto == 2 else S.nmatPacked
        self.check(self.L.mpgpu_set_layout(
            self.h, C.c_int32(S.nTotal), ptr(S.varIndex, i32p), C.c_int32(S.nVar),
            C.c_int32(S.nG), ptr(S.aig, i32p), C.c_int32(matsto),
            ptr(S.offsets if matsto == 2 else None, i64p),
            ptr(S.columns if matsto == 2 else None, i32p), C.c_int64(S.ncolw),
            C.c_int64(self.nmat)))
        sup = getattr(S, "suppressed", None)
        if matsto == 2 and sup is not None and len(sup) > 0:
            self.set_suppressed_pairs(sup)

    def set_suppressed_pairs(self, pairs):
        p = np.ascontiguousarray(pairs, np.int32).reshape(-1)
        self.check(self.L.mpgpu_set_suppressed_pairs(self.h, C.c_int64(len(p) // 2), ptr(p, i32p)))

    def set_constraints(self, A):
        A = np.ascontiguousarray(A, np.float64)
        self.ncon = A.shape[0]
        self.check(self.L.mpgpu_set_constraints(self.h, C.c_int32(A.shape[0]), ptr(A, f64p)))

    def upload(self, S, recFile=None, fileWeight=None):
        self.nrec = len(S.recPtr) - 1
        rf = None if recFile is None else np.ascontiguousarray(recFile, np.int32)
        fw = None if fileWeight is None else np.ascontiguousarray(fileWeight, np.float64)
        self.nfiles = 1 if fw is None else len(fw)
        resident = getattr(S, "resident", False)
        self.check(self.L.mpgpu_upload_records(
            self.h, C.c_int64(self.nrec), ptr(S.recPtr, i64p), ptr(None if resident else S.tinder, i32p),
            ptr(None if resident else S.glder, f64p), ptr(rf, i32p), C.c_int32(self.nfiles), ptr(fw, f64p)))

    def set_monitor(self, nbins=100, rng=5.0, meas_bins=100, mode=1, lfitnp=0, meas_index=None,
                    meas_res=None):
        """Monitoring of the following data loops (None as nbins: off)."""
        if nbins is None:
            self.check(self.L.mpgpu_set_monitor(self.h, None, None, None, C.c_int32(0)))
            self.mon = None
            return
        cfg = MonitorCfg(nbins=nbins, range=rng, measBins=meas_bins, mode=mode, lfitnp=lfitnp)
        mi = None if meas_index is None else np.ascontiguousarray(meas_index, np.int32)
        mr = None if meas_res is None else np.ascontiguousarray(meas_res, np.float64)
        nmeas = 0 if mr is None else len(mr)
        self.check(self.L.mpgpu_set_monitor(self.h, C.byref(cfg), ptr(mi, i32p), ptr(mr, f64p),
                                            C.c_int32(nmeas)))
        self.mon = (nbins, meas_bins, nmeas)

    def get_monitor(self):
        """(hist[4, nbins + 2], measHists[numMeas, measBins]) of the last loop."""
        nbins, mb, nmeas = self.mon
        h = np.zeros(4 * (nbins + 2), np.int64)
        mh = np.zeros(max(nmeas * mb, 1), np.int64)
        self.check(self.L.mpgpu_get_monitor(self.h, ptr(h, i64p), ptr(mh, i64p)))
        return h.reshape(4, nbins + 2), mh[:nmeas * mb].reshape(nmeas, mb)

    def fit_buckets(self):
        """(records, tuned warps per CTA, sample ms [k][1,2,4,8 warps]) per fit size class."""
        cnt = np.zeros(8, np.int64)
        wpc = np.zeros(8, np.int32)
        tms = np.zeros(32, np.float64)
        self.check(self.L.mpgpu_fit_buckets(self.h, ptr(cnt, i64p), ptr(wpc, i32p), ptr(tms, f64p)))
        return cnt, wpc, tms.reshape(8, 4)

    def upload_timing(self):
        """(ms copy, ms prepare, chunks) of the last upload."""
        a, b, n = C.c_double(), C.c_double(), C.c_int32()
        self.check(self.L.mpgpu_upload_timing(self.h, C.byref(a), C.byref(b), C.byref(n)))
        return a.value, b.value, n.value

    def loopbf(self, gpar, **kw):
        o = dict(icalcm=1, nloopn=1, lhuber=0, lfitbb=1, chicut=0.0, chhuge=50.0, dwcut=0.0,
                 cndlmx=100.0)
        o.update(kw)
        fo = FitOpts(**o)
        st = FitStats()
        gvec = np.zeros(self.nVar, np.float64)
        gcnt = np.zeros(self.nVar, np.int64)
        naccf = np.zeros(self.nfiles, np.int32)
        chi2f = np.zeros(self.nfiles, np.float32)
        ndff = np.zeros(self.nfiles, np.int32)
        gpar = np.ascontiguousarray(gpar, np.float64)
        self.check(self.L.mpgpu_loopbf(self.h, C.byref(fo), ptr(gpar, f64p), ptr(gvec, f64p),
                                       ptr(gcnt, i64p), C.byref(st), ptr(naccf, i32p),
                                       ptr(chi2f, f32p), ptr(ndff, i32p)))
        return dict(gvec=gvec, gcnt=gcnt, nrej=list(st.nrej), chi2=st.chi2SumD + st.chi2SumI,
                    ndf=st.ndfSum, naccepted=st.naccepted, nbndr=list(st.nbndr),
                    nbdrx=st.nbdrx, nbndx=st.nbndx, naccf=naccf, chi2f=chi2f, ndff=ndff,
                    msFit=st.msFit, msAccum=st.msAccum, msLoop=st.msLoop, launches=st.launches)

    def matrix(self):
        m = np.zeros(self.nmat, np.float64)
        self.check(self.L.mpgpu_download_matrix(self.h, ptr(m, f64p)))
        return m

    def matrix_diagonal(self):
        m = np.zeros(self.nVar, np.float64)
        self.check(self.L.mpgpu_matrix_diagonal(self.h, ptr(m, f64p)))
        return m

    def status(self):
        s = np.zeros(self.nrec, np.int32)
        self.check(self.L.mpgpu_download_record_status(self.h, ptr(s, i32p)))
        return s

    def mupdat(self, i, j, add):
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        add = np.ascontiguousarray(add, np.float64)
        self.check(self.L.mpgpu_mupdat(self.h, C.c_int32(len(i)), ptr(i, i32p), ptr(j, i32p),
                                       ptr(add, f64p)))

    def dense_cholesky(self, A, mode):
        """Cholesky factor of a dense SPD matrix on the device (mode 0 FP64,
        mode 1 tensor-core 3xTF32 trailing updates); returns (L, ms)."""
        A = np.ascontiguousarray(A, np.float64)
        n = A.shape[0]
        L = np.zeros_like(A)
        ms = C.c_double()
        self.check(self.L.mpgpu_dense_cholesky(self.h, C.c_int32(n), ptr(A, f64p), ptr(L, f64p),
                                               C.c_int32(mode), C.byref(ms)))
        return np.tril(L), ms.value

    def mupdat_noalloc(self, i, j, add):
        """mupdat through the entry point that stages in a fixed device area."""
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        add = np.ascontiguousarray(add, np.float64)
        self.check(self.L.mpgpu_mupdat_noalloc(self.h, C.c_int32(len(i)), ptr(i, i32p),
                                               ptr(j, i32p), ptr(add, f64p)))

    def solve(self, metsol, consResiduals=None, rtol=1e-10, itnlim=2000, errors=False):
        corr = np.zeros(self.nVar, np.float64)
        err = np.zeros(self.nVar, np.float64) if errors else None
        cr = None if consResiduals is None else np.ascontiguousarray(consResiduals, np.float64)
        info = SolveInfo()
        self.check(self.L.mpgpu_solve(self.h, C.c_int32(metsol), ptr(cr, f64p), C.c_double(rtol),
                                      C.c_int32(itnlim), ptr(corr, f64p), ptr(err, f64p),
                                      C.byref(info)))
        return corr, err, info

    def set_preconditioner(self, mbandw, lprecm=0):
        self.check(self.L.mpgpu_set_preconditioner(self.h, C.c_int32(mbandw), C.c_int32(lprecm)))

    def band_factor(self, mbandw, lprecm=0):
        """lltdec factor of the band of Q^T A Q in pede's variable-band layout
        (rows 1..mbandw triangular, then mbandw per row) and nrkd."""
        nfit = self.nVar - self.ncon
        k = min(mbandw, nfit)
        size = k * (k + 1) // 2 + max(nfit - k, 0) * mbandw
        c = np.zeros(max(size, 1), np.float64)
        nrkd = C.c_int32()
        self.check(self.L.mpgpu_band_factor(self.h, C.c_int32(mbandw), C.c_int32(lprecm), ptr(c, f64p),
                                            C.byref(nrkd)))
        return c[:size], nrkd.value

    def avprod(self, x):
        x = np.ascontiguousarray(x, np.float64)
        b = np.zeros_like(x)
        self.check(self.L.mpgpu_avprod(self.h, C.c_int32(len(x)), ptr(x, f64p), ptr(b, f64p)))
        return b


def constraint_matrix(data, S):
    """Rows of the constraint matrix over the variable parameters."""
    A = np.zeros((data["ncon"], S.nVar))
    pos = {int(l): i for i, l in enumerate(S.labels)}
    cs, cl, cc = data["conStart"], data["conLabel"], data["conCoef"]
    for c in range(data["ncon"]):
        for k in range(cs[c], cs[c + 1]):
            li = pos.get(int(cl[k]))
            if li is not None and S.varIndex[li] > 0:
                A[c, S.varIndex[li] - 1] += cc[k]
    return A


# ----------------------------------------------------------------- whole jobs
class JobData:
    """A job's C structures (mpgpu_steer, mpgpu_job, mpgpu_result) with the
    numpy arrays they point to kept alive."""

    def __init__(self, data, constraints=None, params=None, measurements=None, **steer):
        st = dict(metsol=1, matsto=1, mitera=1, lhuber=0, chicut=0.0, chirem=0.0, chhuge=50.0,
                  dwcut=0.0, cndlmx=100.0, lfitbb=1, mreqenf=25, mreqena=10, mreqpe=1,
                  mrestl=1e-10, itnlim=2000, nthreads=0, structDevice=0, monitor=0,
                  monitorPulls=0, monitorBins=100, mbandw=0, lprecm=0)
        st.update(steer)
        self.steer = Steer(**st)
        self.recPtr = np.ascontiguousarray(data["recPtr"], np.int64)
        self.inder = np.ascontiguousarray(data["inder"], np.int32)
        self.glder = np.ascontiguousarray(data["glder"], np.float64)
        j = Job()
        j.nrec = len(self.recPtr) - 1
        j.recPtr, j.inder, j.glder = ptr(self.recPtr, i64p), ptr(self.inder, i32p), ptr(self.glder, f64p)
        j.nfiles = 1
        if constraints is None and data.get("ncon", 0) > 0:
            constraints = (data["conStart"], data["conLabel"], data["conCoef"])
        if constraints is not None:
            self.conStart = np.ascontiguousarray(constraints[0], np.int32)
            self.conLabel = np.ascontiguousarray(constraints[1], np.int32)
            self.conCoef = np.ascontiguousarray(constraints[2], np.float64)
            self.conRhs = np.zeros(len(self.conStart) - 1)
            j.ncon = len(self.conStart) - 1
            j.conStart, j.conLabel = ptr(self.conStart, i32p), ptr(self.conLabel, i32p)
            j.conCoef, j.conRhs = ptr(self.conCoef, f64p), ptr(self.conRhs, f64p)
        if params is not None:
            # steering "Parameter" lines: labels, start values, pre-sigmas
            self.parLabel = np.ascontiguousarray(params[0], np.int32)
            self.parValue = np.ascontiguousarray(params[1], np.float64)
            self.parSigma = np.ascontiguousarray(params[2], np.float64)
            j.npar = len(self.parLabel)
            j.parLabel, j.parValue = ptr(self.parLabel, i32p), ptr(self.parValue, f64p)
            j.parSigma = ptr(self.parSigma, f64p)
        if measurements is not None:
            # steering "measurement" lines: (start, labels, coefficients, rhs, sigma)
            self.msStart = np.ascontiguousarray(measurements[0], np.int32)
            self.msLabel = np.ascontiguousarray(measurements[1], np.int32)
            self.msCoef = np.ascontiguousarray(measurements[2], np.float64)
            self.msRhs = np.ascontiguousarray(measurements[3], np.float64)
            self.msSigma = np.ascontiguousarray(measurements[4], np.float64)
            j.nmeas = len(self.msStart) - 1
            j.msStart, j.msLabel = ptr(self.msStart, i32p), ptr(self.msLabel, i32p)
            j.msCoef, j.msRhs = ptr(self.msCoef, f64p), ptr(self.msRhs, f64p)
            j.msSigma = ptr(self.msSigma, f64p)
        self.job = j
        cap = len(self.inder) + 16
        self.labels = np.zeros(cap, np.int32)
        self.parameter = np.zeros(cap)
        self.presigma = np.zeros(cap)
        self.error = np.zeros(cap)
        self.counts = np.zeros(cap, np.int64)
        self.varIndex = np.zeros(cap, np.int32)
        self.start = np.zeros(cap)
        self.gcor = np.zeros(cap)
        self.fileCounts = np.zeros(cap, np.int64)
        r = Result()
        r.cap = cap
        r.start, r.gcor = ptr(self.start, f64p), ptr(self.gcor, f64p)
        r.fileCounts = ptr(self.fileCounts, i64p)
        r.labels, r.parameter = ptr(self.labels, i32p), ptr(self.parameter, f64p)
        r.presigma, r.error = ptr(self.presigma, f64p), ptr(self.error, f64p)
        r.counts, r.varIndex = ptr(self.counts, i64p), ptr(self.varIndex, i32p)
        self.res = r

    def parameters(self):
        n = self.res.nTotal
        return self.labels[:n].copy(), self.parameter[:n].copy()

    def write_res(self, path, errors=0, ipcntr=0, igcorr=0, mreqena=10):
        """millepede.res of the job (mpgpu_write_res_opts)."""
        o = ResOpts(errors=errors, ipcntr=ipcntr, igcorr=igcorr, mreqena=mreqena)
        return lib().mpgpu_write_res_opts(str(path).encode(), C.byref(self.res), C.byref(o))


class ServerCfg(C.Structure):
    _fields_ = [("device", C.c_int32), ("maxActive", C.c_int32), ("budgetBytes", C.c_int64)]


class Server:
    """Resident request loop (mpgpu_server_*): submit JobData, wait by ticket."""

    def __init__(self, device=0, max_active=4, budget_bytes=0):
        self.L = lib()
        self.h = C.c_void_p()
        cfg = ServerCfg(device=device, maxActive=max_active, budgetBytes=budget_bytes)
        rc = self.L.mpgpu_server_create(C.byref(self.h), C.byref(cfg))
        if rc != 0:
            raise RuntimeError(f"mpgpu_server_create: {rc}")

    def submit(self, jd):
        t = C.c_int64()
        rc = self.L.mpgpu_server_submit(self.h, C.byref(jd.steer), C.byref(jd.job), C.byref(jd.res),
                                        C.byref(t))
        if rc != 0:
            raise RuntimeError(f"mpgpu_server_submit: {rc}")
        return t.value

    def wait(self, ticket, timeout_ms=0.0):
        lat, q, b = C.c_double(), C.c_double(), C.c_int64()
        rc = self.L.mpgpu_server_wait(self.h, C.c_int64(ticket), C.c_double(timeout_ms), C.byref(lat),
                                      C.byref(q), C.byref(b))
        return rc, lat.value, q.value, b.value

    def last_error(self):
        msg = self.L.mpgpu_server_last_error(self.h) if self.h else b""
        return msg.decode() if msg else ""

    def close(self):
        if self.h:
            self.L.mpgpu_server_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run_job(jd, ctx=None):
    """Whole job through mpgpu_pede_run (private context when ctx is None)."""
    return lib().mpgpu_pede_run(ctx.h if ctx is not None else None, C.byref(jd.steer), C.byref(jd.job),
                                C.byref(jd.res))


class PinnedArray:
    """numpy array in page-locked memory from mpgpu_host_alloc."""

    def __init__(self, src):
        src = np.ascontiguousarray(src)
        self.L = lib()
        self.p = C.c_void_p()
        rc = self.L.mpgpu_host_alloc(C.byref(self.p), C.c_int64(max(src.nbytes, 1)))
        if rc != 0:
            raise RuntimeError(f"mpgpu_host_alloc: {rc}")
        buf = (C.c_char * max(src.nbytes, 1)).from_address(self.p.value)
        self.a = np.frombuffer(buf, dtype=src.dtype, count=src.size).reshape(src.shape)
        self.a[...] = src

    def free(self):
        if self.p:
            self.a = None
            self.L.mpgpu_host_free(self.p)
            self.p = C.c_void_p()
