"""The band preconditioner of MINRES (mpgpu_band_factor,
mpgpu_set_preconditioner; pede's equdecs/equslvs with the constraints
eliminated) against the oracle on the same matrix: the lltdec factor of the
band bit for bit where the band is the stored matrix (no constraints),
within 1e-10 of the largest entry where the constraint reflections reduce
it first; MINRES and MINRES-QLP with band, diagonal and no preconditioner
reach the solution of the oracle's solver with the same preconditioner
within 1e-8 to 1e-7, and whole jobs with the band preconditioner the oracle
job's parameters within 1e-7 (relative to the largest)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

i32p, i64p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)


def build(mp, kind, ntracks, matsto, constraints, seed=61):
    d = mp.generate(mp.gen_config(kind, ntracks=ntracks, seed=seed))
    H = mp.HostStructure(d, mreqenf=5, sparse=(matsto == 2))
    A = mp.constraint_matrix(d, H) if constraints else None
    ctx = mp.Context()
    ctx.set_layout(H, matsto)
    if constraints:
        ctx.set_constraints(A)
    ctx.upload(H)
    lb = ctx.loopbf(np.zeros(H.nTotal))
    return d, H, A, ctx, lb


def oracle_ql(orc, A, n):
    L = orc.lib()
    L.mpref_ql_create.restype = C.c_void_p
    return L.mpref_ql_create(C.c_int32(n), C.c_int32(A.shape[0]), np.ascontiguousarray(A).ctypes.data_as(f64p))


def arrays(H, matsto):
    if matsto == 2:
        return (H.aig.ctypes.data_as(i32p), np.ascontiguousarray(H.offsets, np.int64).ctypes.data_as(i64p),
                np.ascontiguousarray(H.columns, np.int32).ctypes.data_as(i32p))
    return H.aig.ctypes.data_as(i32p), None, None


def oracle_factor(orc, H, matsto, M, q, ncon, mb, lprecm):
    L = orc.lib()
    n = H.nVar
    nfit = n - ncon
    india = np.zeros(n, np.int64)
    L.mpref_band_index(C.c_int32(n), C.c_int32(mb), india.ctypes.data_as(i64p))
    c = np.zeros(int(india[nfit - 1]))
    nrkd = C.c_int32()
    aig, off, col = arrays(H, matsto)
    rc = L.mpref_band_precond(C.c_int32(matsto), C.c_int32(n), C.c_int32(H.nG), aig, off, col,
                              M.ctypes.data_as(f64p), C.c_void_p(q) if q else None, C.c_int32(mb),
                              C.c_int32(lprecm), c.ctypes.data_as(f64p), C.byref(nrkd))
    assert rc == 0
    return c, nrkd.value


@pytest.mark.parametrize("kind,matsto,mb", [("telescope", 1, 6), ("barrel", 2, 12), ("barrel", 2, 32),
                                            ("brokenlines", 2, 1)])
def test_band_factor_exact(mp, orc, kind, matsto, mb):
    """No constraints: the device factor equals the oracle's lltdec bit for bit."""
    _, H, _, ctx, _ = build(mp, kind, 3000 if kind != "brokenlines" else 400, matsto, False)
    with ctx:
        M = ctx.matrix()
        cg, nrkd = ctx.band_factor(mb)
    co, nrkdo = oracle_factor(orc, H, matsto, M, None, 0, mb, 0)
    assert nrkd == nrkdo
    np.testing.assert_array_equal(cg, co)


def reset_rows(c, n, mb):
    """rows whose entries left of the diagonal are all zero (lltdec's reset)"""
    out, pos = [], 0
    for i in range(n):
        k = min(i, mb - 1)
        out.append(not np.any(c[pos:pos + k]))
        pos += k + 1
    return np.array(out)


@pytest.mark.parametrize("lprecm", [0, 1])
def test_band_factor_constraints(mp, orc, lprecm):
    """Constraints eliminated: the band of Q^T A Q, factorised, within 1e-10
    of the largest entry.  The elimination leaves rows that depend on the
    rows before them; the skyline option keeps them with their own diagonal,
    which is itself at the rounding level there, so those rows and the
    columns below them carry rounding-level differences amplified by
    1/sqrt: with the option the same rows are reset and the factors agree
    within 1e-7."""
    _, H, A, ctx, _ = build(mp, "barrel", 4000, 2, True)
    with ctx:
        M = ctx.matrix()
        cg, nrkd = ctx.band_factor(8, lprecm)
    q = oracle_ql(orc, A, H.nVar)
    try:
        co, nrkdo = oracle_factor(orc, H, 2, M, q, A.shape[0], 8, lprecm)
    finally:
        orc.lib().mpref_ql_destroy(C.c_void_p(q))
    assert nrkd == nrkdo
    nfit = H.nVar - A.shape[0]
    np.testing.assert_array_equal(reset_rows(cg, nfit, 8), reset_rows(co, nfit, 8))
    assert np.max(np.abs(cg - co)) <= (1e-7 if lprecm else 1e-10) * np.max(np.abs(co))


def oracle_minres(orc, H, A, M, matsto, gvec, qlp, mbandw, rtol, itnlim):
    """the oracle's MINRES (-QLP) on the QL-reduced system, solution back in
    the full parameter space"""
    L = orc.lib()
    n, ncon = H.nVar, A.shape[0]
    q = oracle_ql(orc, A, n)
    try:
        b = gvec.copy()
        L.mpref_ql_mlq(C.c_void_p(q), b.ctypes.data_as(f64p), C.c_int32(1))
        x = np.zeros(n)
        itn, nrkd = C.c_int32(), C.c_int32()
        aig, off, col = arrays(H, matsto)
        istop = L.mpref_minres_precond(C.c_int32(qlp), C.c_int32(matsto), C.c_int32(n), C.c_int32(H.nG),
                                       aig, off, col, M.ctypes.data_as(f64p), C.c_void_p(q),
                                       b.ctypes.data_as(f64p), x.ctypes.data_as(f64p), C.c_double(rtol),
                                       C.c_int32(itnlim), C.c_int32(mbandw), C.c_int32(0), C.byref(itn),
                                       C.byref(nrkd))
        x[n - ncon:] = 0.0
        L.mpref_ql_mlq(C.c_void_p(q), x.ctypes.data_as(f64p), C.c_int32(0))
    finally:
        L.mpref_ql_destroy(C.c_void_p(q))
    return x, istop, itn.value


@pytest.mark.parametrize("metsol", [4, 5])
def test_minres_band_solve_barrel(mp, orc, metsol):
    """MINRES (-QLP) with "bandwidth 6" on the sparse barrel with constraints
    (30,000 tracks): both converge, the solutions agree within 1e-7 of the
    largest correction, the iteration counts within 10 %, and the band needs
    fewer iterations than the diagonal.  (The system has weakly determined
    modes: solutions with different preconditioners differ at the 1e-4
    level at rtol 1e-12, so each is compared with the oracle's run of the
    same preconditioner.)"""
    _, H, A, ctx, lb = build(mp, "barrel", 30000, 2, True, seed=4)
    ncon = A.shape[0]
    with ctx:
        M = ctx.matrix()
        ctx.set_preconditioner(6)
        corr, _, info = ctx.solve(metsol, consResiduals=np.zeros(ncon), rtol=1e-12, itnlim=6000)
        ctx.set_preconditioner(0)
        _, _, info0 = ctx.solve(metsol, consResiduals=np.zeros(ncon), rtol=1e-12, itnlim=6000)
    x, istop, itn = oracle_minres(orc, H, A, M, 2, lb["gvec"], metsol == 5, 6, 1e-12, 6000)
    assert info.istop in (1, 2) and istop in (1, 2), (info.istop, istop)
    assert np.max(np.abs(corr - x)) <= 1e-7 * np.max(np.abs(x))
    assert abs(info.itn - itn) <= max(3, 0.1 * itn)
    assert info.itn < info0.itn


@pytest.mark.parametrize("metsol,mbandw", [(4, 32), (5, 12), (4, 1)])
def test_minres_band_solve_sparse_telescope(mp, orc, metsol, mbandw):
    """Well-determined sparse system (telescope with constraints, sparse
    storage): the band preconditioners of width 1, 12 and 32 give the
    oracle's solution within 1e-8."""
    _, H, A, ctx, lb = build(mp, "telescope", 5000, 2, True)
    with ctx:
        M = ctx.matrix()
        ctx.set_preconditioner(mbandw)
        corr, _, info = ctx.solve(metsol, consResiduals=np.zeros(A.shape[0]), rtol=1e-13, itnlim=3000)
    x, istop, itn = oracle_minres(orc, H, A, M, 2, lb["gvec"], metsol == 5, mbandw, 1e-13, 3000)
    assert info.istop in (1, 2) and istop in (1, 2), (info.istop, istop)
    assert np.max(np.abs(corr - x)) <= 1e-8 * np.max(np.abs(x))


@pytest.mark.parametrize("mbandw", [-1, 0, 5])
def test_minres_packed_preconditioners(mp, orc, mbandw):
    """Packed telescope with constraints: no, diagonal and band
    preconditioners give the oracle's solution within 1e-8."""
    _, H, A, ctx, lb = build(mp, "telescope", 5000, 1, True)
    with ctx:
        M = ctx.matrix()
        ctx.set_preconditioner(mbandw)
        corr, _, info = ctx.solve(4, consResiduals=np.zeros(A.shape[0]), rtol=1e-13, itnlim=3000)
    x, istop, itn = oracle_minres(orc, H, A, M, 1, lb["gvec"], 0, mbandw, 1e-13, 3000)
    assert info.istop in (1, 2) and istop in (1, 2), (info.istop, istop)
    assert np.max(np.abs(corr - x)) <= 1e-8 * np.max(np.abs(x))


@pytest.mark.parametrize("metsol", [4])
def test_job_band_preconditioner(mp, orc, metsol):
    """Whole sparse job with "bandwidth 6" against the oracle's job driver."""
    from test_gpu_pede import gpu_job
    d = mp.generate(mp.gen_config("barrel", ntracks=30000, seed=4))
    st = orc.make_steer(metsol=metsol, matsto=2, mitera=2, lhuber=2, mrestl=1e-12, itnlim=3000, mreqenf=5,
                        mbandw=6)
    g = gpu_job(mp, orc, d, st)
    o = orc.run(d, st)
    assert g["rc"] == 0 and o["rc"] == 0
    np.testing.assert_array_equal(g["counts"], o["counts"])
    assert g["nrej"] == o["nrej"]
    scale = np.max(np.abs(o["parameter"]))
    assert np.max(np.abs(g["parameter"] - o["parameter"])) <= 1e-7 * scale
