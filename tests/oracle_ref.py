"""ctypes binding of the CPU oracle (oracle/_build/libmpref.so).

Test infrastructure only: the oracle is the checker the GPU results are
compared with; nothing in the product imports this module.
"""
import ctypes as C
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBPATH = os.path.join(ROOT, "oracle", "_build", "libmpref.so")

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)


class FitOpt(C.Structure):
    _fields_ = [("icalcm", C.c_int32), ("nloopn", C.c_int32), ("lhuber", C.c_int32),
                ("lfitbb", C.c_int32), ("matsto", C.c_int32), ("chicut", C.c_float),
                ("chhuge", C.c_float), ("dwcut", C.c_float), ("cndlmx", C.c_float),
                ("mreqpe", C.c_int32)]


class FitOut(C.Structure):
    _fields_ = [("nrej", C.c_int64 * 6), ("chi2SumI", C.c_int64), ("chi2SumD", C.c_double),
                ("ndfSum", C.c_int64), ("ndfSumW", C.c_double), ("nbndr", C.c_int32 * 2),
                ("nbdrx", C.c_int32), ("nbndx", C.c_int32)]


class Steer(C.Structure):
    _fields_ = [("metsol", C.c_int32), ("matsto", C.c_int32), ("mitera", C.c_int32),
                ("lhuber", C.c_int32), ("chicut", C.c_float), ("chirem", C.c_float),
                ("chhuge", C.c_float), ("dwcut", C.c_float), ("cndlmx", C.c_float),
                ("lfitbb", C.c_int32), ("mreqenf", C.c_int32), ("mreqena", C.c_int32),
                ("mreqpe", C.c_int32), ("mrestl", C.c_double), ("itnlim", C.c_int32),
                ("nthreads", C.c_int32), ("mbandw", C.c_int32), ("lprecm", C.c_int32)]


class Job(C.Structure):
    _fields_ = [("nrec", C.c_int64), ("recPtr", i64p), ("inder", i32p), ("glder", f64p),
                ("recFile", i32p), ("nfiles", C.c_int32), ("fileWeight", f64p),
                ("npar", C.c_int32), ("parLabel", i32p), ("parValue", f64p),
                ("parSigma", f64p),
                ("ncon", C.c_int32), ("conStart", i32p), ("conLabel", i32p),
                ("conCoef", f64p), ("conRhs", f64p),
                ("nmeas", C.c_int32), ("msStart", i32p), ("msLabel", i32p),
                ("msCoef", f64p), ("msRhs", f64p), ("msSigma", f64p)]


class Result(C.Structure):
    _fields_ = [("cap", C.c_int32), ("nTotal", C.c_int32), ("nVar", C.c_int32),
                ("nVarGroups", C.c_int32), ("nFit", C.c_int32),
                ("labels", i32p), ("parameter", f64p), ("presigma", f64p), ("error", f64p),
                ("counts", i64p), ("varIndex", i32p),
                ("nrej", C.c_int64 * 6), ("fvalue", C.c_double), ("ndf", C.c_int64),
                ("nrank", C.c_int32), ("minresItn", C.c_int32), ("minresIstop", C.c_int32),
                ("nloopn", C.c_int32), ("exitCode", C.c_int32),
                ("start", f64p), ("gcor", f64p), ("fileCounts", i64p)]


def ptr(a, t):
    if a is None:
        return C.cast(None, t)
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(t)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError("oracle not built: run __graft_entry__.build()")
        L = C.CDLL(LIBPATH)
        L.mpref_chindl.restype = C.c_float
        L.mpref_ijadd.restype = C.c_int64
        L.mpref_ql_create.restype = C.c_void_p
        L.mpref_ql_create.argtypes = [C.c_int32, C.c_int32, f64p]
        for fn in ("mpref_ql_mlq", "mpref_ql_bsub", "mpref_ql_destroy", "mpref_ql_export",
                   "mpref_ql_ssq_packed", "mpref_ql_gete"):
            getattr(L, fn).argtypes = None
        _lib = L
    return _lib


def make_steer(**kw):
    d = dict(metsol=1, matsto=1, mitera=1, lhuber=0, chicut=0.0, chirem=0.0, chhuge=50.0,
             dwcut=0.0, cndlmx=100.0, lfitbb=1, mreqenf=25, mreqena=10, mreqpe=1,
             mrestl=1e-6, itnlim=2000, nthreads=1)
    d.update(kw)
    return Steer(**d)


class Arrays:
    """keeps numpy arrays alive while ctypes structs point to them"""


def make_job(data, parLabel=None, parValue=None, parSigma=None, constraints=True,
             recFile=None, fileWeight=None, measurements=None):
    keep = Arrays()
    keep.recPtr = np.ascontiguousarray(data["recPtr"], np.int64)
    keep.inder = np.ascontiguousarray(data["inder"], np.int32)
    keep.glder = np.ascontiguousarray(data["glder"], np.float64)
    j = Job()
    j.nrec = len(keep.recPtr) - 1
    j.recPtr = ptr(keep.recPtr, i64p)
    j.inder = ptr(keep.inder, i32p)
    j.glder = ptr(keep.glder, f64p)
    if recFile is not None:
        keep.recFile = np.ascontiguousarray(recFile, np.int32)
        keep.fileWeight = np.ascontiguousarray(fileWeight, np.float64)
        j.recFile = ptr(keep.recFile, i32p)
        j.fileWeight = ptr(keep.fileWeight, f64p)
        j.nfiles = len(keep.fileWeight)
    else:
        j.nfiles = 1
    if parLabel is not None:
        keep.parLabel = np.ascontiguousarray(parLabel, np.int32)
        keep.parValue = np.ascontiguousarray(parValue, np.float64)
        keep.parSigma = np.ascontiguousarray(parSigma, np.float64)
        j.npar = len(keep.parLabel)
        j.parLabel = ptr(keep.parLabel, i32p)
        j.parValue = ptr(keep.parValue, f64p)
        j.parSigma = ptr(keep.parSigma, f64p)
    if constraints and data.get("ncon", 0) > 0:
        keep.conStart = np.ascontiguousarray(data["conStart"], np.int32)
        keep.conLabel = np.ascontiguousarray(data["conLabel"], np.int32)
        keep.conCoef = np.ascontiguousarray(data["conCoef"], np.float64)
        keep.conRhs = np.zeros(data["ncon"], np.float64)
        j.ncon = data["ncon"]
        j.conStart = ptr(keep.conStart, i32p)
        j.conLabel = ptr(keep.conLabel, i32p)
        j.conCoef = ptr(keep.conCoef, f64p)
        j.conRhs = ptr(keep.conRhs, f64p)
    if measurements is not None:
        # steering "measurement" lines: (start, labels, coefficients, rhs, sigma)
        keep.msStart = np.ascontiguousarray(measurements[0], np.int32)
        keep.msLabel = np.ascontiguousarray(measurements[1], np.int32)
        keep.msCoef = np.ascontiguousarray(measurements[2], np.float64)
        keep.msRhs = np.ascontiguousarray(measurements[3], np.float64)
        keep.msSigma = np.ascontiguousarray(measurements[4], np.float64)
        j.nmeas = len(keep.msStart) - 1
        j.msStart, j.msLabel = ptr(keep.msStart, i32p), ptr(keep.msLabel, i32p)
        j.msCoef, j.msRhs = ptr(keep.msCoef, f64p), ptr(keep.msRhs, f64p)
        j.msSigma = ptr(keep.msSigma, f64p)
    return j, keep


def make_result(cap, cls=Result):
    keep = Arrays()
    keep.labels = np.zeros(cap, np.int32)
    keep.parameter = np.zeros(cap, np.float64)
    keep.presigma = np.zeros(cap, np.float64)
    keep.error = np.zeros(cap, np.float64)
    keep.counts = np.zeros(cap, np.int64)
    keep.varIndex = np.zeros(cap, np.int32)
    keep.start = np.zeros(cap, np.float64)
    keep.gcor = np.zeros(cap, np.float64)
    keep.fileCounts = np.zeros(cap, np.int64)
    r = cls()
    r.cap = cap
    r.start = ptr(keep.start, f64p)
    r.gcor = ptr(keep.gcor, f64p)
    r.fileCounts = ptr(keep.fileCounts, i64p)
    r.labels = ptr(keep.labels, i32p)
    r.parameter = ptr(keep.parameter, f64p)
    r.presigma = ptr(keep.presigma, f64p)
    r.error = ptr(keep.error, f64p)
    r.counts = ptr(keep.counts, i64p)
    r.varIndex = ptr(keep.varIndex, i32p)
    return r, keep


def run(data, steer, **jobkw):
    """Whole job through the oracle; returns (Result, arrays)."""
    L = lib()
    job, kj = make_job(data, **jobkw)
    cap = int(len(data["inder"]) + 16)
    res, kr = make_result(cap)
    rc = L.mpref_run(C.byref(steer), C.byref(job), C.byref(res))
    n = res.nTotal
    out = dict(rc=rc, labels=kr.labels[:n].copy(), parameter=kr.parameter[:n].copy(),
               error=kr.error[:n].copy(), counts=kr.counts[:n].copy(),
               start=kr.start[:n].copy(), gcor=kr.gcor[:n].copy(),
               fileCounts=kr.fileCounts[:n].copy(), result=res, arrays=kr,
               varIndex=kr.varIndex[:n].copy(), nrej=list(res.nrej), fvalue=res.fvalue,
               ndf=res.ndf, nrank=res.nrank, itn=res.minresItn, istop=res.minresIstop,
               nVar=res.nVar, nFit=res.nFit, nVarGroups=res.nVarGroups)
    return out


class Structure:
    """loop1 + loop2 products computed by the oracle for one record set."""

    def __init__(self, data, mreqenf=25, steerLabels=(), preLabel=(), preSigma=(), sparse=True,
                 mreqpe=1):
        L = lib()
        recPtr = np.ascontiguousarray(data["recPtr"], np.int64)
        inder = np.ascontiguousarray(data["inder"], np.int32)
        glder = np.ascontiguousarray(data["glder"], np.float64)
        nrec = len(recPtr) - 1
        cap = len(inder) + len(steerLabels) + 16
        self.labels = np.zeros(cap, np.int32)
        self.counter = np.zeros(cap, np.int64)
        self.varIndex = np.zeros(cap, np.int32)
        self.grpStart = np.zeros(cap, np.int32)
        self.totGroup = np.zeros(cap, np.int32)
        nVar, nG = C.c_int32(), C.c_int32()
        sl = np.ascontiguousarray(steerLabels, np.int32)
        pl = np.ascontiguousarray(preLabel, np.int32)
        ps = np.ascontiguousarray(preSigma, np.float64)
        n = L.mpref_loop1(C.c_int64(nrec), ptr(recPtr, i64p), ptr(inder, i32p),
                          ptr(glder, f64p), C.c_int32(len(sl)), ptr(sl, i32p),
                          C.c_int32(len(pl)), ptr(pl, i32p), ptr(ps, f64p), C.c_int32(mreqenf),
                          C.c_int32(cap), ptr(self.labels, i32p), ptr(self.counter, i64p),
                          ptr(self.varIndex, i32p), ptr(self.grpStart, i32p),
                          ptr(self.totGroup, i32p), C.byref(nVar), C.byref(nG))
        assert n >= 0
        self.nTotal = n
        for a in ("labels", "counter", "varIndex", "grpStart", "totGroup"):
            setattr(self, a, getattr(self, a)[:n].copy())
        self.nVar, self.nG = nVar.value, nG.value
        self.aig = np.zeros(self.nG + 1, np.int32)
        self.p2g = np.zeros(max(self.nVar, 1), np.int32)
        L.mpref_var_groups(C.c_int32(n), ptr(self.varIndex, i32p), ptr(self.totGroup, i32p),
                           C.c_int32(self.nVar), C.c_int32(self.nG), ptr(self.aig, i32p),
                           ptr(self.p2g, i32p))
        self.tinder = np.zeros_like(inder)
        rc = L.mpref_translate(C.c_int64(nrec), ptr(recPtr, i64p), ptr(inder, i32p),
                               ptr(glder, f64p), C.c_int32(n), ptr(self.labels, i32p),
                               ptr(self.tinder, i32p))
        assert rc == 0
        self.recPtr, self.glder = recPtr, glder
        self.mreqpe = mreqpe
        self.offsets = np.zeros(2 * (self.nG + 1), np.int64)
        self.columns = np.zeros(1, np.int32)
        if sparse:
            capc = 1 << 20
            while True:
                self.columns = np.zeros(capc, np.int32)
                ncolw, nmat = C.c_int64(), C.c_int64()
                rc = L.mpref_mpbits(C.c_int64(nrec), C.c_int64(nrec), ptr(recPtr, i64p),
                                    ptr(self.tinder, i32p),
                                    ptr(glder, f64p), ptr(self.varIndex, i32p),
                                    C.c_int32(self.nVar), C.c_int32(self.nG),
                                    ptr(self.aig, i32p), ptr(self.p2g, i32p), C.c_int32(mreqpe),
                                    C.c_int64(capc), ptr(self.offsets, i64p),
                                    ptr(self.columns, i32p), C.byref(ncolw), C.byref(nmat))
                if rc == 0:
                    break
                capc *= 4
            self.columns = self.columns[:max(ncolw.value, 1)].copy()
            self.ncolw, self.nmatSparse = ncolw.value, nmat.value
        self.nmatPacked = self.nVar * (self.nVar + 1) // 2

    def loopbf(self, gpar, matsto=2, nthreads=1, **opt):
        L = lib()
        o = dict(icalcm=1, nloopn=1, lhuber=0, lfitbb=1, matsto=matsto, chicut=0.0,
                 chhuge=50.0, dwcut=0.0, cndlmx=100.0, mreqpe=self.mreqpe)
        o.update(opt)
        fo = FitOpt(**o)
        out = FitOut()
        nrec = len(self.recPtr) - 1
        nmat = self.nmatSparse if matsto == 2 else self.nmatPacked
        gvec = np.zeros(self.nVar, np.float64)
        gcnt = np.zeros(self.nVar, np.int64)
        matD = np.zeros(nmat, np.float64)
        status = np.zeros(nrec, np.int32)
        gpar = np.ascontiguousarray(gpar, np.float64)
        if nthreads > 1:
            rc = L.mpref_loopbf_omp(C.c_int32(nthreads), C.byref(fo), C.c_int64(nrec),
                                    ptr(self.recPtr, i64p), ptr(self.tinder, i32p),
                                    ptr(self.glder, f64p), None, C.c_int32(1), None,
                                    ptr(gpar, f64p), ptr(self.varIndex, i32p),
                                    C.c_int32(self.nVar), C.c_int32(self.nG),
                                    ptr(self.aig, i32p), ptr(self.p2g, i32p),
                                    ptr(self.offsets, i64p), ptr(self.columns, i32p),
                                    C.c_int64(nmat), ptr(gvec, f64p), ptr(gcnt, i64p),
                                    ptr(matD, f64p), C.byref(out), ptr(status, i32p))
        else:
            rc = L.mpref_loopbf(C.byref(fo), C.c_int64(nrec), ptr(self.recPtr, i64p),
                                ptr(self.tinder, i32p), ptr(self.glder, f64p), None,
                                C.c_int32(1), None, ptr(gpar, f64p), ptr(self.varIndex, i32p),
                                C.c_int32(self.nVar), C.c_int32(self.nG), ptr(self.aig, i32p),
                                ptr(self.p2g, i32p), ptr(self.offsets, i64p),
                                ptr(self.columns, i32p), ptr(gvec, f64p), ptr(gcnt, i64p),
                                ptr(matD, f64p), C.byref(out), ptr(status, i32p), None, None,
                                None)
        return dict(rc=rc, gvec=gvec, gcnt=gcnt, matD=matD, status=status,
                    nrej=list(out.nrej), chi2=out.chi2SumD + out.chi2SumI, ndf=out.ndfSum,
                    nbndr=list(out.nbndr), nbdrx=out.nbdrx, nbndx=out.nbndx)
