"""Global solves on the GPU (mpgpu_solve) against the oracle on the same
matrix: inversion and decomposition with QL-eliminated constraints,
sparse MINRES, the avprod product."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def build(mp, name, ntracks, matsto, seed=21):
    d = mp.generate(mp.gen_config(name, ntracks=ntracks, seed=seed))
    H = mp.HostStructure(d, mreqenf=5, sparse=(matsto == 2))
    A = mp.constraint_matrix(d, H)
    ctx = mp.Context()
    ctx.set_layout(H, matsto)
    ctx.set_constraints(A)
    ctx.upload(H)
    lb = ctx.loopbf(np.zeros(H.nTotal))
    return d, H, A, ctx, lb


def dense_from_packed(p, n):
    M = np.zeros((n, n))
    M[np.tril_indices(n)] = p
    return M + np.tril(M, -1).T


def kkt_solution(M, A, b):
    n, m = M.shape[0], A.shape[0]
    K = np.block([[M, A.T], [A, np.zeros((m, m))]])
    return np.linalg.solve(K, np.concatenate([b, np.zeros(m)]))[:n]


@pytest.mark.parametrize("metsol", [1, 3])
def test_packed_solvers_vs_oracle(mp, orc, metsol):
    d, H, A, ctx, lb = build(mp, "telescope", 5000, 1)
    with ctx:
        M = ctx.matrix()
        corr, err, info = ctx.solve(metsol, consResiduals=np.zeros(A.shape[0]), errors=(metsol == 1))
    n = H.nVar
    x = kkt_solution(dense_from_packed(M, n), A, lb["gvec"])
    assert np.max(np.abs(corr - x)) <= 1e-9 * np.max(np.abs(x))
    assert info.nrank == n - A.shape[0]
    # oracle: same elimination and solver on the same matrix
    L = orc.lib()
    q = L.mpref_ql_create(n, A.shape[0], orc.ptr(np.ascontiguousarray(A), orc.f64p))
    Mo = M.copy()
    bo = lb["gvec"].copy()
    L.mpref_ql_ssq_packed(C.c_void_p(q), orc.ptr(Mo, orc.f64p), C.c_int32(1))
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(bo, orc.f64p), C.c_int32(1))
    nfit = n - A.shape[0]
    nr = C.c_int32()
    if metsol == 1:
        L.mpref_sqminl(orc.ptr(Mo, orc.f64p), orc.ptr(bo, orc.f64p), C.c_int32(nfit), C.byref(nr))
    else:
        emax, emin = C.c_double(), C.c_double()
        L.mpref_chdec2(orc.ptr(Mo, orc.f64p), C.c_int32(nfit), C.byref(nr), C.byref(emax), C.byref(emin))
        L.mpref_chslv2(orc.ptr(Mo, orc.f64p), orc.ptr(bo, orc.f64p), C.c_int32(nfit))
    bo[nfit:] = 0.0
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(bo, orc.f64p), C.c_int32(0))
    assert nr.value == info.nrank
    assert np.max(np.abs(corr - bo)) <= 1e-10 * np.max(np.abs(bo))
    if metsol == 1:
        # errors: oracle's literal back-transform of the same inverse
        Mo2 = M.copy()
        b2 = lb["gvec"].copy()
        L.mpref_ql_ssq_packed(C.c_void_p(q), orc.ptr(Mo2, orc.f64p), C.c_int32(1))
        L.mpref_sqminl(orc.ptr(Mo2, orc.f64p), orc.ptr(b2, orc.f64p), C.c_int32(nfit), C.byref(nr))
        P = dense_from_packed(Mo2, n)
        P[nfit:, :] = 0.0
        P[:, nfit:] = 0.0
        Mp = P[np.tril_indices(n)].copy()
        L.mpref_ql_ssq_packed(C.c_void_p(q), orc.ptr(Mp, orc.f64p), C.c_int32(0))
        diag = dense_from_packed(Mp, n).diagonal()
        assert np.max(np.abs(err - diag) / np.abs(diag)) <= 1e-9
    L.mpref_ql_destroy(C.c_void_p(q))


def test_minres_sparse(mp, orc):
    d, H, A, ctx, lb = build(mp, "barrel", 40000, 2)
    with ctx:
        M = ctx.matrix()
        corr, _, info = ctx.solve(4, consResiduals=np.zeros(A.shape[0]), rtol=1e-12, itnlim=4000)
        # avprod: Q^T A Q on a random reduced vector
        nfit = H.nVar - A.shape[0]
        xr = np.random.default_rng(1).normal(size=nfit)
        bg = ctx.avprod(xr)
    O = orc.Structure(d, mreqenf=5)
    xo = np.zeros(H.nVar)
    itn = C.c_int32()
    L = orc.lib()
    q = L.mpref_ql_create(H.nVar, A.shape[0], orc.ptr(np.ascontiguousarray(A), orc.f64p))
    rhs = lb["gvec"].copy()
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(rhs, orc.f64p), C.c_int32(1))
    istop = L.mpref_minres_sparse(C.c_int32(2), C.c_int32(H.nVar), C.c_int32(O.nG),
                                  orc.ptr(O.aig, orc.i32p), orc.ptr(O.offsets, orc.i64p),
                                  orc.ptr(O.columns, orc.i32p), orc.ptr(M, orc.f64p),
                                  C.c_void_p(q), orc.ptr(rhs, orc.f64p), orc.ptr(xo, orc.f64p),
                                  C.c_double(1e-12), C.c_int32(4000), C.byref(itn))
    xo[nfit:] = 0.0
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(xo, orc.f64p), C.c_int32(0))
    assert info.istop in (1, 2) and istop in (1, 2)
    assert abs(info.itn - itn.value) <= 0.1 * itn.value  # long Krylov runs drift in rounding
    # two MINRES runs to rtol 1e-12 on a system this ill-conditioned agree to
    # a few 1e-9; the GPU solution's own residual is the sharper check
    assert np.max(np.abs(corr - xo)) <= 1e-8 * np.max(np.abs(xo))
    xr_sol = np.zeros(H.nVar)
    xr_sol[:] = corr
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(xr_sol, orc.f64p), C.c_int32(1))
    with mp.Context() as c2:
        c2.set_layout(H, 2)
        c2.set_constraints(A)
        c2.upload(H)
        c2.loopbf(np.zeros(H.nTotal))
        Ax = c2.avprod(xr_sol[:nfit])
    res = np.linalg.norm(Ax - rhs[:nfit]) / np.linalg.norm(rhs[:nfit])
    assert res <= 1e-9
    # avprod against the oracle's avprd0 with explicit Q
    xa = np.concatenate([xr, np.zeros(A.shape[0])])
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(xa, orc.f64p), C.c_int32(0))
    ba = np.zeros(H.nVar)
    L.mpref_avprd0(C.c_int32(2), C.c_int32(H.nVar), orc.ptr(xa, orc.f64p), orc.ptr(ba, orc.f64p),
                   C.c_int32(O.nG), orc.ptr(O.aig, orc.i32p), orc.ptr(O.offsets, orc.i64p),
                   orc.ptr(O.columns, orc.i32p), orc.ptr(M, orc.f64p))
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(ba, orc.f64p), C.c_int32(1))
    assert np.max(np.abs(bg - ba[:nfit])) <= 1e-12 * np.max(np.abs(ba))
    L.mpref_ql_destroy(C.c_void_p(q))


@pytest.mark.parametrize("metsol", [31, 32])
def test_dense_refined_solvers(mp, metsol):
    """Blocked dense Cholesky (32: FP64, 31: tensor-core 3xTF32) refined by
    FP64 conjugate gradients: the constrained solution agrees with the KKT
    solution of the same matrix within 1e-9 relative (the telescope matrix
    has condition ~1e6 after the elimination)."""
    d, H, A, ctx, lb = build(mp, "telescope", 5000, 1)
    with ctx:
        M = ctx.matrix()
        corr, _, info = ctx.solve(metsol, consResiduals=np.zeros(A.shape[0]), rtol=1e-14, itnlim=500)
    n = H.nVar
    x = kkt_solution(dense_from_packed(M, n), A, lb["gvec"])
    assert info.istop == 1, (info.istop, info.itn)
    assert np.max(np.abs(corr - x)) <= 1e-9 * np.max(np.abs(x))


def test_minresqlp_sparse_vs_minres_and_oracle(mp, orc):
    """MINRES-QLP (metsol 5) on the constrained barrel system: the MINRES
    solution and the oracle's MINRES-QLP within 1e-8 relative, and a
    relative residual of the reduced system below 1e-9."""
    out = {}
    for metsol in (4, 5):
        d, H, A, ctx, lb = build(mp, "barrel", 40000, 2)
        with ctx:
            M = ctx.matrix()
            corr, _, info = ctx.solve(metsol, consResiduals=np.zeros(A.shape[0]), rtol=1e-12, itnlim=4000)
        out[metsol] = (corr, info.istop, info.itn)
    corr, istop, itn = out[5]
    assert istop in (1, 2)
    scale = np.max(np.abs(out[4][0]))
    assert np.max(np.abs(corr - out[4][0])) <= 1e-8 * scale
    O = orc.Structure(d, mreqenf=5)
    nfit = H.nVar - A.shape[0]
    L = orc.lib()
    q = L.mpref_ql_create(H.nVar, A.shape[0], orc.ptr(np.ascontiguousarray(A), orc.f64p))
    rhs = lb["gvec"].copy()
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(rhs, orc.f64p), C.c_int32(1))
    xo = np.zeros(H.nVar)
    it = C.c_int32()
    so = L.mpref_minresqlp_sparse(C.c_int32(2), C.c_int32(H.nVar), C.c_int32(O.nG),
                                  orc.ptr(O.aig, orc.i32p), orc.ptr(O.offsets, orc.i64p),
                                  orc.ptr(O.columns, orc.i32p), orc.ptr(M, orc.f64p),
                                  C.c_void_p(q), orc.ptr(rhs, orc.f64p), orc.ptr(xo, orc.f64p),
                                  C.c_double(1e-12), C.c_int32(4000), C.byref(it))
    xo[nfit:] = 0.0
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(xo, orc.f64p), C.c_int32(0))
    assert so in (1, 2)
    assert np.max(np.abs(corr - xo)) <= 1e-8 * np.max(np.abs(xo))
    xr = corr.copy()
    L.mpref_ql_mlq(C.c_void_p(q), orc.ptr(xr, orc.f64p), C.c_int32(1))
    with mp.Context() as c2:
        c2.set_layout(H, 2)
        c2.set_constraints(A)
        c2.upload(H)
        c2.loopbf(np.zeros(H.nTotal))
        Ax = c2.avprod(xr[:nfit])
    assert np.linalg.norm(Ax - rhs[:nfit]) / np.linalg.norm(rhs[:nfit]) <= 1e-9
    L.mpref_ql_destroy(C.c_void_p(q))


def test_minresqlp_singular_minimum_length(mp):
    """Telescope without constraints: the global shift and shear are free,
    the matrix is singular and the normal equations consistent up to
    rounding (b's null-space part is at the 1e-16 level, which bounds the
    attainable relative residual near 1e-11).  At a tolerance above that
    floor MINRES-QLP returns the minimum-length solution of the diagonally
    preconditioned system, D pinv(D M D) D b (D = 1/sqrt(diag M)), within
    1e-7; a tolerance below it lets the iterations continue into the null
    space."""
    d = mp.generate(mp.gen_config("telescope", ntracks=3000, seed=31))
    H = mp.HostStructure(d, mreqenf=5, sparse=False)
    with mp.Context() as ctx:
        ctx.set_layout(H, 1)
        ctx.upload(H)
        lb = ctx.loopbf(np.zeros(H.nTotal))
        M = dense_from_packed(ctx.matrix(), H.nVar)
        corr, _, info = ctx.solve(5, rtol=1e-10, itnlim=2000)
    b = lb["gvec"]
    Dm = np.diag(1.0 / np.sqrt(np.diag(M)))
    want = Dm @ np.linalg.pinv(Dm @ M @ Dm, rcond=1e-10) @ Dm @ b
    assert np.linalg.matrix_rank(M, tol=1e-9 * np.max(np.abs(M))) <= H.nVar - 2
    assert info.istop in (1, 2, 4)
    assert np.max(np.abs(corr - want)) <= 1e-7 * np.max(np.abs(want))


@pytest.mark.parametrize("nmod", [30, 300])
def test_blocked_inversion_forms(mp, nmod):
    """Inversion from the blocked Cholesky factor (metsol 12 FP64, metsol 11
    tensor-core 3xTF32 with its trtri/lauum tile products in 3xTF32 as
    well) against sqminl (metsol 1) on the same QL-reduced matrix: the
    refined solutions within 1e-10; the FP64 form's errors within 1e-9 (the
    sqminl bar).  The tensor-core form's errors are not refined: their
    relative error is about 1e-7 x the condition number of the reduced
    matrix (6 % for the 3,000-parameter telescope, cond ~ 1e5), asserted
    only within 0.2 here.  Sizes above and below one 128 tile and with
    padding."""
    cfg = mp.gen_config("telescope", ntracks=40 * nmod * 10, seed=23)
    cfg.nmod = nmod
    d = mp.generate(cfg)
    H = mp.HostStructure(d, mreqenf=5, sparse=False)
    A = mp.constraint_matrix(d, H)
    out = {}
    for metsol in (1, 12, 11):
        with mp.Context() as ctx:
            ctx.set_layout(H, 1)
            ctx.set_constraints(A)
            ctx.upload(H)
            ctx.loopbf(np.zeros(H.nTotal))
            corr, err, info = ctx.solve(metsol, consResiduals=np.zeros(A.shape[0]), rtol=1e-13, errors=True)
            out[metsol] = (corr, err, info.nrank, info.msInverse)
    corr1, err1 = out[1][0], out[1][1]
    scale = np.max(np.abs(corr1))
    var = np.abs(err1) > 0
    for metsol, tol in ((12, 1e-9), (11, 0.2)):
        corr, err, nrank, msinv = out[metsol]
        assert nrank == H.nVar - A.shape[0]
        assert np.max(np.abs(corr - corr1)) <= 1e-10 * scale, metsol
        rel = np.max(np.abs(err[var] - err1[var]) / np.abs(err1[var]))
        assert rel <= tol, (metsol, rel)
        assert msinv > 0


def test_mixed_factor_reuse(mp):
    """The tensor-core dense solve (metsol 31) keeps its factor in the
    context: the next outlier iteration's matrix (Huber down-weighting and
    a chi2 cut change the record weights) is first solved with the previous
    factor as the CG preconditioner.  That solution equals the one with a
    fresh factor (MPGPU_FLAG_FRESH_FACTOR) within 1e-10 relative, the solve
    reports the reuse, and a new constraint set drops the kept factor."""
    d = mp.generate(mp.gen_config("telescope", ntracks=20000, seed=23))
    H = mp.HostStructure(d, mreqenf=5)
    A = mp.constraint_matrix(d, H)
    z = np.zeros(A.shape[0])
    sol, infos = {}, {}
    for flags in (0, 16):
        with mp.Context(flags=flags) as ctx:
            ctx.set_layout(H, 1)
            ctx.set_constraints(A)
            ctx.upload(H)
            gpar = np.zeros(H.nTotal)
            got = []
            for it, (hub, cut) in enumerate([(0, 0.0), (2, 6.0), (2, 3.0)], start=1):
                lb = ctx.loopbf(gpar, nloopn=it, lhuber=hub, chicut=cut)
                corr, _, info = ctx.solve(31, consResiduals=z, rtol=1e-12, itnlim=500)
                assert info.istop == 1, (flags, it, info.istop, info.itn)
                got.append((corr, info.factorReused, info.itn, sum(lb["nrej"])))
            # new constraints: the kept factor is not used again
            ctx.set_constraints(A)
            ctx.loopbf(gpar, nloopn=2, lhuber=2, chicut=6.0)
            _, _, info = ctx.solve(31, consResiduals=z, rtol=1e-12, itnlim=500)
            assert info.factorReused == 0
        sol[flags] = got
    assert [g[1] for g in sol[16]] == [0, 0, 0]
    assert sol[0][0][1] == 0
    assert all(g[1] in (1, 2) for g in sol[0][1:])
    assert sol[0][1][1] == 1, sol[0][1][1:]
    for a, b in zip(sol[0], sol[16]):
        x, y = a[0], b[0]
        assert np.max(np.abs(x - y)) <= 1e-10 * np.max(np.abs(y)), (a[1:], b[1:])
