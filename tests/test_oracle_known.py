"""Known-answer tests of the CPU oracle's numerical kernels against numpy /
scipy on the same inputs: the local solvers (sqminv, bordered band
sqmibb/sqmibb2), the global solvers (sqminl, chdec2/chslv2, MINRES), the
QL constraint elimination and the chindl table.  Tolerances: 1e-11
relative for direct solvers on well-conditioned matrices, 1e-9 for MINRES
at rtol 1e-13, 2e-3 for chindl up to 30 degrees of freedom (its table has 4-5
significant digits) and 5e-2 above (Fisher's approximation)."""
import ctypes as C

import numpy as np
import pytest

import oracle_ref as O

f64p = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)


def p(a):
    return a.ctypes.data_as(f64p)


def packed(M):
    """lower triangle by rows, (i*i+i)/2 + j (0-based)"""
    return np.ascontiguousarray(M[np.tril_indices(len(M))], np.float64)


def unpack(v, n):
    M = np.zeros((n, n))
    M[np.tril_indices(n)] = v
    return M + np.tril(M, -1).T


def spd(n, rng, pattern=None):
    A = rng.normal(size=(n, n))
    A = A + A.T
    if pattern is not None:
        A = np.where(pattern, A, 0.0)
    A += np.diag(np.sum(np.abs(A), axis=1) + 1.0)
    return A


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("fn,n", [("mpref_sqminv", 5), ("mpref_sqminv", 17), ("mpref_sqminl", 60)])
def test_gauss_jordan_inverse(orc, fn, n):
    rng = np.random.default_rng(n)
    A = spd(n, rng)
    b = rng.normal(size=n)
    v, x = packed(A), b.copy()
    rank = C.c_int32()
    getattr(O.lib(), fn)(p(v), p(x), C.c_int32(n), C.byref(rank))
    assert rank.value == n
    assert rel(unpack(v, n), np.linalg.inv(A)) <= 1e-11
    assert rel(x, np.linalg.solve(A, b)) <= 1e-11


def test_sqminv_rank_deficit(orc):
    rng = np.random.default_rng(1)
    B = rng.normal(size=(6, 4))
    A = B @ B.T  # rank 4
    v, x = packed(A), rng.normal(size=6)
    rank = C.c_int32()
    O.lib().mpref_sqminv(p(v), p(x), C.c_int32(6), C.byref(rank))
    assert rank.value == 4


@pytest.mark.parametrize("side", [1, 2])
@pytest.mark.parametrize("inv", [1, 2])
def test_bordered_band(orc, side, inv):
    n, nbdr, nbnd = 14, 3, 2
    rng = np.random.default_rng(10 * side + inv)
    idx = np.arange(n)
    bdr = idx < nbdr if side == 1 else idx >= n - nbdr
    band = np.abs(idx[:, None] - idx[None, :]) <= nbnd
    pattern = band | bdr[:, None] | bdr[None, :]
    A = spd(n, rng, pattern)
    b = rng.normal(size=n)
    v, x = packed(A), b.copy()
    rank, emin, emax = C.c_int32(), C.c_double(), C.c_double()
    fn = O.lib().mpref_sqmibb if side == 1 else O.lib().mpref_sqmibb2
    fn(p(v), p(x), C.c_int32(n), C.c_int32(nbdr), C.c_int32(nbnd), C.c_int32(inv),
       C.byref(rank), C.byref(emin), C.byref(emax))
    assert rank.value == n
    assert rel(x, np.linalg.solve(A, b)) <= 1e-11
    Ai = np.linalg.inv(A)
    got = unpack(v, n)
    if inv == 2:
        assert rel(got, Ai) <= 1e-11
    else:  # band part of the inverse and the border rows
        assert rel(got[pattern], Ai[pattern]) <= 1e-11
    assert 0 < emin.value <= emax.value


def test_cholesky(orc):
    n = 40
    rng = np.random.default_rng(7)
    A = spd(n, rng)
    b = rng.normal(size=n)
    g = packed(A)
    rank, evmax, evmin = C.c_int32(), C.c_double(), C.c_double()
    O.lib().mpref_chdec2(p(g), C.c_int32(n), C.byref(rank), C.byref(evmax), C.byref(evmin))
    assert rank.value == n
    x = b.copy()
    O.lib().mpref_chslv2(p(g), p(x), C.c_int32(n))
    assert rel(x, np.linalg.solve(A, b)) <= 1e-11


def ql(npar, ncon, rng):
    A = np.ascontiguousarray(rng.normal(size=(ncon, npar)))
    L = O.lib()
    L.mpref_ql_create.restype = C.c_void_p
    h = L.mpref_ql_create(C.c_int32(npar), C.c_int32(ncon), p(A))
    return A, h


def ql_apply(h, x, t):
    y = np.ascontiguousarray(x, np.float64).copy()
    O.lib().mpref_ql_mlq(C.c_void_p(h), p(y), C.c_int32(t))
    return y


def test_ql_elimination(orc):
    npar, ncon = 30, 4
    rng = np.random.default_rng(3)
    A, h = ql(npar, ncon, rng)
    try:
        Q = np.stack([ql_apply(h, e, 0) for e in np.eye(npar)], axis=1)
        assert rel(Q.T @ Q, np.eye(npar)) <= 1e-13
        # Q^T C^T: the constraints live in the last ncon coordinates only
        QtCt = np.stack([ql_apply(h, A[k], 1) for k in range(ncon)], axis=1)
        assert np.max(np.abs(QtCt[: npar - ncon])) <= 1e-13 * np.max(np.abs(A))
        # qlbsub: y with (Q^T C^T)^T restricted to the last rows times y = d
        d = rng.normal(size=ncon)
        y = np.zeros(ncon)
        O.lib().mpref_ql_bsub(C.c_void_p(h), p(d), p(y))
        x = np.zeros(npar)
        x[npar - ncon:] = y
        assert rel(A @ ql_apply(h, x, 0), d) <= 1e-12
        # qlssq (t=1) gives Q^T M Q on the block that is kept
        M = spd(npar, rng)
        v = packed(M)
        O.lib().mpref_ql_ssq_packed(C.c_void_p(h), p(v), C.c_int32(1))
        m = npar - ncon
        assert rel(unpack(v, npar)[:m, :m], (Q.T @ M @ Q)[:m, :m]) <= 1e-12
    finally:
        O.lib().mpref_ql_destroy(C.c_void_p(h))


def test_minres_packed(orc):
    n = 80
    rng = np.random.default_rng(9)
    A = spd(n, rng)
    b = rng.normal(size=n)
    x = np.zeros(n)
    itn = C.c_int32()
    aig = np.arange(1, n + 2, dtype=np.int32)
    L = O.lib()
    istop = L.mpref_minres_sparse(C.c_int32(1), C.c_int32(n), C.c_int32(n),
                                  aig.ctypes.data_as(i32p), None, None, p(packed(A)), None,
                                  p(b), p(x), C.c_double(1e-13), C.c_int32(1000), C.byref(itn))
    assert istop in (1, 2, 3)
    assert rel(x, np.linalg.solve(A, b)) <= 1e-9


def test_chindl(orc):
    from scipy.stats import chi2, norm
    f = O.lib().mpref_chindl
    f.restype = C.c_float
    for m in (1, 2, 3):
        prob = 2.0 * norm.sf(m)
        for nd in (1, 2, 5, 10, 30, 31, 60, 200):
            want = chi2.isf(prob, nd) / nd
            # above 30 the reference uses Fisher's sqrt(2 chi2) approximation
            tol = 2e-3 if nd <= 30 else 5e-2
            assert abs(f(m, nd) - want) <= tol * want, (m, nd, f(m, nd), want)
            if nd > 30:
                sn = (0.47523, 1.690140, 2.782170)[m - 1]
                fisher = np.float32((sn + np.sqrt(np.float32(2 * nd - 1))) ** 2 / (2 * nd))
                assert abs(f(m, nd) - fisher) <= 1e-6 * fisher


def minres_call(fn, A, b, rtol=1e-13, itnlim=2000):
    n = len(b)
    x = np.zeros(n)
    itn = C.c_int32()
    aig = np.arange(1, n + 2, dtype=np.int32)
    istop = getattr(O.lib(), fn)(C.c_int32(1), C.c_int32(n), C.c_int32(n), aig.ctypes.data_as(i32p), None,
                                 None, p(packed(A)), None, p(np.ascontiguousarray(b)), p(x),
                                 C.c_double(rtol), C.c_int32(itnlim), C.byref(itn))
    return x, istop, itn.value


def test_minresqlp_nonsingular(orc):
    """MINRES-QLP on an SPD system: the solution of numpy within 1e-9, and
    the MINRES solution within 1e-9 (same Krylov iterates)."""
    n = 80
    rng = np.random.default_rng(19)
    A = spd(n, rng)
    b = rng.normal(size=n)
    x, istop, itn = minres_call("mpref_minresqlp_sparse", A, b)
    assert istop in (1, 2) and itn > 0
    assert rel(x, np.linalg.solve(A, b)) <= 1e-9
    xm, _, _ = minres_call("mpref_minres_sparse", A, b)
    assert rel(x, xm) <= 1e-9


def test_minresqlp_singular_minimum_length(orc):
    """Singular consistent system (rank 40 of 60): MINRES-QLP gives the
    minimum-length solution of the diagonally preconditioned system,
    x = D pinv(D A D) D b with D the preconditioner's 1/sqrt(diag A), within
    1e-8."""
    n, r = 60, 40
    rng = np.random.default_rng(23)
    B = rng.normal(size=(n, r))
    A = B @ B.T
    b = A @ rng.normal(size=n)
    x, istop, itn = minres_call("mpref_minresqlp_sparse", A, b, rtol=1e-12, itnlim=500)
    D = np.diag(1.0 / np.sqrt(np.diag(A)))
    want = D @ np.linalg.pinv(D @ A @ D, rcond=1e-10) @ D @ b
    assert istop in (1, 2), istop
    assert rel(x, want) <= 1e-8, (rel(x, want), istop, itn)


def test_minresqlp_maxxnorm_keeps_last_iterate(orc):
    """An inconsistent singular system drives the iterates' length up; the
    solver stops before taking an iterate longer than its limit
    (n / sqrt(eps)) and returns a finite solution."""
    n, r = 60, 40
    rng = np.random.default_rng(29)
    B = rng.normal(size=(n, r))
    A = B @ B.T
    null = np.linalg.svd(B.T)[2][r:].T
    b = A @ rng.normal(size=n) + null @ rng.normal(size=n - r)
    x, istop, itn = minres_call("mpref_minresqlp_sparse", A, b, rtol=1e-14, itnlim=400)
    assert np.all(np.isfinite(x))
    assert np.linalg.norm(x) <= n / np.sqrt(np.finfo(float).eps)


# ---- band preconditioner (equdecs/equslvs with constraints eliminated)
i64p = C.POINTER(C.c_int64)


def band_index(n, mb):
    india = np.zeros(n, np.int64)
    O.lib().mpref_band_index(C.c_int32(n), C.c_int32(mb), india.ctypes.data_as(i64p))
    return india


def band_fill(A, mb):
    n = len(A)
    india = band_index(n, mb)
    c = np.zeros(int(india[-1]))
    for k in range(n):
        for j in range(max(0, k - mb + 1), k + 1):
            c[india[k] - 1 - k + j] = A[k, j]
    return c, india


def band_factor(c, india, mb):
    """dense L from lltdec's band: off-diagonals as stored, diagonal 1/c"""
    n = len(india)
    L = np.zeros((n, n))
    for k in range(n):
        for j in range(max(0, k - mb + 1), k):
            L[k, j] = c[india[k] - 1 - k + j]
        d = c[india[k] - 1]
        L[k, k] = 1.0 / d if d != 0.0 else 0.0
    return L


def band_of(A, mb):
    n = len(A)
    i, j = np.indices((n, n))
    return np.where((i - j < mb) & (j - i < mb), A, 0.0)


def test_lltdec_band_solve(orc):
    """lltdec on an SPD band: L L^T reproduces the band within 1e-13;
    lltfwd + lltbwd solve it within 1e-11."""
    n, mb = 50, 6
    rng = np.random.default_rng(41)
    A = band_of(spd(n, rng), mb)
    c, india = band_fill(A, mb)
    nrkd = O.lib().mpref_lltdec(C.c_int32(n), p(c), india.ctypes.data_as(i64p), C.c_int32(0))
    assert nrkd == 0
    L = band_factor(c, india, mb)
    assert rel(L @ L.T, A) <= 1e-13
    b = rng.normal(size=n)
    x = b.copy()
    O.lib().mpref_lltslv(C.c_int32(n), p(c), india.ctypes.data_as(i64p), p(x))
    assert rel(x, np.linalg.solve(A, b)) <= 1e-11


@pytest.mark.parametrize("iopt", [0, 1])
def test_lltdec_dependent_row(orc, iopt):
    """A row equal to the one before it (an exact 2x2 block [[4,4],[4,4]]):
    its reduced diagonal is exactly 0, the row is reset; without the skyline
    option its diagonal is 0 and nrkd = -row, with it the diagonal is
    1/sqrt(4) and nrkd = 0."""
    n, mb, k = 20, 4, 9
    rng = np.random.default_rng(43)
    A = band_of(spd(n, rng), mb)
    A[k - 1:k + 1, :] = 0.0
    A[:, k - 1:k + 1] = 0.0
    A[k - 1:k + 1, k - 1:k + 1] = 4.0
    c, india = band_fill(A, mb)
    nrkd = O.lib().mpref_lltdec(C.c_int32(n), p(c), india.ctypes.data_as(i64p), C.c_int32(iopt))
    row = c[india[k] - 1 - (min(k, mb - 1)):india[k] - 1]
    assert np.all(row == 0.0)
    if iopt:
        assert nrkd == 0 and c[india[k] - 1] == 0.5
    else:
        assert nrkd == -(k + 1) and c[india[k] - 1] == 0.0


def test_band_precond_of_reduced_matrix(orc):
    """With constraints eliminated, the factor's L L^T is the band of
    (Q^T M Q) restricted to the fit parameters, within 1e-12."""
    npar, ncon, mb = 40, 3, 5
    rng = np.random.default_rng(47)
    Cm, h = ql(npar, ncon, rng)
    try:
        Q = np.stack([ql_apply(h, e, 0) for e in np.eye(npar)], axis=1)
        M = spd(npar, rng)
        m = npar - ncon
        want = band_of((Q.T @ M @ Q)[:m, :m], mb)
        india = band_index(npar, mb)
        c = np.zeros(int(india[m - 1]))
        nrkd = C.c_int32()
        aig = np.arange(1, npar + 2, dtype=np.int32)
        rc = O.lib().mpref_band_precond(C.c_int32(1), C.c_int32(npar), C.c_int32(npar), aig.ctypes.data_as(i32p),
                                        None, None, p(packed(M)), C.c_void_p(h), C.c_int32(mb), C.c_int32(0),
                                        p(c), C.byref(nrkd))
        assert rc == 0 and nrkd.value == 0
        L = band_factor(c, india[:m], mb)
        assert rel(L @ L.T, want) <= 1e-12
    finally:
        O.lib().mpref_ql_destroy(C.c_void_p(h))


@pytest.mark.parametrize("qlp", [0, 1])
@pytest.mark.parametrize("mbandw", [-1, 0, 4, 80])
def test_minres_preconditioners(orc, qlp, mbandw):
    """MINRES and MINRES-QLP with no, diagonal and band preconditioners
    reach numpy's solution within 1e-9; the band as wide as the matrix is
    its exact factor, so one or two iterations suffice."""
    n = 80
    rng = np.random.default_rng(53)
    pat = rng.random((n, n)) < 0.1
    A = spd(n, rng, pattern=pat | pat.T)
    b = rng.normal(size=n)
    x = np.zeros(n)
    itn, nrkd = C.c_int32(), C.c_int32()
    aig = np.arange(1, n + 2, dtype=np.int32)
    istop = O.lib().mpref_minres_precond(C.c_int32(qlp), C.c_int32(1), C.c_int32(n), C.c_int32(n),
                                         aig.ctypes.data_as(i32p), None, None, p(packed(A)), None, p(b), p(x),
                                         C.c_double(1e-13), C.c_int32(1000), C.c_int32(mbandw), C.c_int32(0),
                                         C.byref(itn), C.byref(nrkd))
    assert istop in (1, 2), istop
    assert rel(x, np.linalg.solve(A, b)) <= 1e-9
    if mbandw >= n:
        assert itn.value <= 2


def test_job_band_preconditioner_same_solution(mp):
    """The oracle's job driver with MINRES and pede's "bandwidth 6" reaches
    the parameters of the diagonal preconditioner (well-determined
    telescope with its constraints) within 1e-8."""
    d = mp.generate(mp.gen_config("telescope", ntracks=3000, seed=7))
    out = {}
    for mb in (0, 6, -1):
        st = O.make_steer(metsol=4, matsto=2, mitera=1, mrestl=1e-13, itnlim=3000, mreqenf=5, mbandw=mb)
        out[mb] = O.run(d, st)
        assert out[mb]["rc"] == 0
    scale = np.max(np.abs(out[0]["parameter"]))
    for mb in (6, -1):
        assert np.max(np.abs(out[mb]["parameter"] - out[0]["parameter"])) <= 1e-8 * scale
