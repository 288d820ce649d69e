"""The structure passes on the device (mpgpu_loop1_device,
mpgpu_loop2_device) against the host versions (mpgpu_host_labels,
mpgpu_host_translate, mpgpu_host_mpbits), which the CPU tests hold against
the oracle: every table identical (labels, entries, variable indices,
groups, sparse offsets and columns), and a data loop over the records kept
and translated on the device identical, bit for bit, to one over the
host-translated upload."""
import ctypes as C

import numpy as np
import pytest

from test_gpu_loopbf import with_special_blocks

pytestmark = pytest.mark.gpu


def same_tables(Hs, Ds, sparse):
    assert Ds.nTotal == Hs.nTotal and Ds.nVar == Hs.nVar and Ds.nG == Hs.nG
    for k in ("labels", "counter", "varIndex", "totGroup", "aig"):
        np.testing.assert_array_equal(getattr(Ds, k), getattr(Hs, k), err_msg=k)
    if sparse:
        np.testing.assert_array_equal(Ds.offsets, Hs.offsets)
        assert Ds.ncolw == Hs.ncolw and Ds.nmatSparse == Hs.nmatSparse
        np.testing.assert_array_equal(Ds.columns[:Ds.ncolw], Hs.columns[:Hs.ncolw])


def data_of(mp, kind, ntracks, seed, special=False):
    d = mp.generate(mp.gen_config(kind, ntracks=ntracks, seed=seed))
    return with_special_blocks(d) if special else d


@pytest.mark.parametrize("kind,ntracks,special", [
    ("telescope", 3000, False), ("barrel", 20000, False), ("brokenlines", 1500, False),
    ("barrel", 3000, True)])
def test_tables_match_host(mp, kind, ntracks, special):
    d = data_of(mp, kind, ntracks, 31, special)
    Hs = mp.HostStructure(d, mreqenf=5, sparse=True)
    with mp.Context() as ctx:
        Ds = mp.DeviceStructure(ctx, d, mreqenf=5, sparse=True)
    same_tables(Hs, Ds, True)


def test_steering_labels_and_presigma(mp):
    """Labels named only by the steering (constraints, parameters) join the
    table; fixed parameters and the entries cut give the same variable
    numbering."""
    d = data_of(mp, "telescope", 2000, 32)
    steer = np.array([5, 7, 100000, 100001], np.int32)
    pre = np.array([1, 2, 3, 100001], np.int32)
    sig = np.array([-1.0, 0.0, -1.0, -1.0])
    Hs = mp.HostStructure(d, mreqenf=30, steerLabels=steer, preLabel=pre, preSigma=sig, sparse=False)
    with mp.Context() as ctx:
        Ds = mp.DeviceStructure(ctx, d, mreqenf=30, steerLabels=steer, preLabel=pre, preSigma=sig,
                                sparse=False)
    same_tables(Hs, Ds, False)
    assert 100000 in Ds.labels


@pytest.mark.parametrize("kind,matsto", [("barrel", 2), ("telescope", 1), ("brokenlines", 2)])
def test_resident_records_same_loop(mp, kind, matsto):
    """Layout and records from the device passes: the data loop gives the
    same matrix, vector and decisions as with the host passes."""
    d = data_of(mp, kind, 4000 if kind != "brokenlines" else 800, 33)
    sparse = matsto == 2
    Hs = mp.HostStructure(d, mreqenf=5, sparse=sparse)
    out = []
    for dev in (False, True):
        with mp.Context() as ctx:
            S = mp.DeviceStructure(ctx, d, mreqenf=5, sparse=sparse) if dev else Hs
            ctx.set_layout(S, matsto)
            ctx.upload(S)
            g = ctx.loopbf(np.zeros(S.nTotal))
            out.append((g, ctx.matrix(), ctx.status()))
    (gh, mh, sh), (gd, md, sd) = out
    np.testing.assert_array_equal(sd, sh)
    np.testing.assert_array_equal(md, mh)
    np.testing.assert_array_equal(gd["gvec"], gh["gvec"])
    assert gd["chi2"] == gh["chi2"] and gd["ndf"] == gh["ndf"]


def test_resident_records_taken_once(mp):
    d = data_of(mp, "telescope", 500, 34)
    with mp.Context() as ctx:
        S = mp.DeviceStructure(ctx, d, mreqenf=5, sparse=False)
        ctx.set_layout(S, 1)
        ctx.upload(S)
        with pytest.raises(RuntimeError, match="error 44"):
            ctx.upload(S)


def many_labels(nrec, k, seed):
    """nrec records of one measurement with one local and k global
    derivatives, every label distinct (nrec * k labels)."""
    rng = np.random.default_rng(seed)
    w = 4 + k
    inder = np.zeros(nrec * w, np.int32)
    glder = np.zeros(nrec * w, np.float64)
    lab = rng.permutation(np.arange(1, nrec * k + 1, dtype=np.int32) * 3 + 7)
    for r in range(nrec):
        b = r * w
        inder[b + 2] = 1
        glder[b + 1], glder[b + 2], glder[b + 3] = rng.normal(), 1.0, 0.1
        inder[b + 4:b + w] = lab[r * k:(r + 1) * k]
        glder[b + 4:b + w] = rng.normal(size=k)
    return dict(recPtr=np.arange(nrec + 1, dtype=np.int64) * w, inder=inder, glder=glder)


def test_label_set_rebuilt_larger(mp):
    """2.4 million distinct labels: more than half of the first label set,
    which is rebuilt eight times larger; tables as on the host."""
    d = many_labels(75000, 32, 35)
    Hs = mp.HostStructure(d, mreqenf=1, sparse=False)
    with mp.Context() as ctx:
        Ds = mp.DeviceStructure(ctx, d, mreqenf=1, sparse=False)
    assert Ds.nTotal == 75000 * 32
    same_tables(Hs, Ds, False)


def loop1_rc(mp, ctx, d, cap=None):
    L = mp.lib()
    rp = np.ascontiguousarray(d["recPtr"], np.int64)
    ind = np.ascontiguousarray(d["inder"], np.int32)
    gl = np.ascontiguousarray(d["glder"], np.float64)
    cap = cap or len(ind) + 16
    a32 = [np.zeros(cap, np.int32) for _ in range(3)]
    cnt = np.zeros(cap, np.int64)
    nv, ng = C.c_int32(), C.c_int32()
    i32p, i64p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)
    args = [C.c_int64(len(rp) - 1), rp.ctypes.data_as(i64p), ind.ctypes.data_as(i32p),
            gl.ctypes.data_as(f64p), C.c_int32(0), None, C.c_int32(0), None, None, C.c_int32(1),
            C.c_int32(cap), a32[0].ctypes.data_as(i32p), cnt.ctypes.data_as(i64p),
            a32[1].ctypes.data_as(i32p), a32[2].ctypes.data_as(i32p), C.byref(nv), C.byref(ng)]
    dev = L.mpgpu_loop1_device(ctx.h, *args)
    host = L.mpgpu_host_labels(*args[:])
    return dev, host


def test_error_codes_as_host(mp):
    d = data_of(mp, "telescope", 200, 36)
    with mp.Context() as ctx:
        # capacity
        assert loop1_rc(mp, ctx, d, cap=10) == (-1, -1)
        # a record whose last measurement lacks its second marker
        bad = dict(d)
        rp = d["recPtr"].copy()
        ind = d["inder"].copy()
        r = 7
        a, b = int(rp[r]), int(rp[r + 1])
        zeros = [q for q in range(a + 1, b) if ind[q] == 0]
        ind[zeros[-1]] = 3
        bad["inder"] = ind
        assert loop1_rc(mp, ctx, bad) == (-20, -20)
        # a negative label among the global words
        neg = dict(d)
        ind = d["inder"].copy()
        ind[zeros[-1] + 1] = -4
        neg["inder"] = ind
        assert loop1_rc(mp, ctx, neg) == (-23, -23)
