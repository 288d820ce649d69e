"""The reference's route to the preconditioner band of Q^T A Q (qlpssq,
mpqldec.f90:711-945), restated step by step in numpy, against the exact
H A H of one reflection.  Its second pass (lines 858-929) applies the band
update with vtAv = v^T A v again while no coefficient has been formed yet,
so the restated route gives band(H A H) + 4 (v^T A v) band(v v^T): the
reference's preconditioner (diagonal, mbandw 0, and band) carries that term
once per reflection.  The preconditioners here use the exact band of
Q^T A Q (tests/test_oracle_known.py); the oracle also carries the literal
route (mpref_set_qlpssq_literal), checked here against the restatement.
The MINRES solution does not depend on the preconditioner, its iteration
count can."""
import numpy as np


def qldec(A):
    """Householder vectors of the QL decomposition (qldec, mpqldec.f90:125-218):
    row k-1 holds v_k below position kn-1, Vk[k-1] its entry at kn-1."""
    ncon, npar = A.shape
    V = A.copy()
    Vk = np.zeros(ncon)
    r2 = np.zeros(ncon, int)
    for k in range(ncon, 0, -1):
        kn = npar + k - ncon
        row = V[k - 1]
        vn = row[:kn].copy()
        nrm = np.sqrt(vn @ vn)
        vn[kn - 1] += nrm if vn[kn - 1] >= 0 else -nrm
        vn /= np.sqrt(vn @ vn)
        for i in range(1, k + 1):
            ri = V[i - 1]
            ri[:kn] -= 2 * vn * (vn @ ri[:kn])
        row[:kn - 1] = vn[:kn - 1]
        row[kn - 1:] = 0.0
        r2[k - 1] = kn - 1
        Vk[k - 1] = vn[kn - 1]
    return V, Vk, r2


def qlpssq_band(M, V, Vk, r2, mb):
    """qlpssq(aprod, B, mb, t=.true.) on the band of M, both passes"""
    npar, ncon = M.shape[0], V.shape[0]
    mbnd = max(0, mb - 1)
    idx = [(i, l) for i in range(1, npar + 1) for l in range(max(1, i - mbnd), i + 1)]
    B = np.array([M[i - 1, l - 1] for (i, l) in idx])
    vtvp = np.zeros((ncon, ncon))
    vtAvp = np.zeros((ncon, ncon))
    coef = np.zeros((ncon, ncon))
    rng = np.zeros((2, ncon), int)

    def vec(k):
        kn = npar + k - ncon
        v = np.zeros(npar)
        v[:r2[k - 1]] = V[k - 1, :r2[k - 1]]
        v[kn - 1] = Vk[k - 1]
        return v, kn

    def order(j):
        return ncon + 1 - j

    def update(vN, vAv, vtAv, kn):
        for q, (i, l) in enumerate(idx):
            if i <= kn:
                B[q] += 2.0 * ((2.0 * vN[i - 1] * vtAv - vAv[i - 1]) * vN[l - 1] - vAv[l - 1] * vN[i - 1])
            else:
                B[q] -= 2.0 * vAv[i - 1] * vN[l - 1]

    for j in range(1, ncon + 1):                       # lines 781-855
        k = order(j)
        vN, kn = vec(k)
        rng[:, k - 1] = (ncon, 1)
        vAv = M @ vN
        for j2 in range(j + 1, ncon + 1):
            k2 = order(j2)
            x = vN @ vec(k2)[0]
            if abs(x) > 16 * np.finfo(float).eps:
                vtvp[k - 1, k2 - 1] = vtvp[k2 - 1, k - 1] = x
        vtvp[k - 1, k - 1] = 1.0
        for j2 in range(1, j + 1):
            k2 = order(j2)
            vtAvp[k - 1, k2 - 1] = vec(k2)[0] @ vAv
        update(vN, vAv, vtAvp[k - 1, k - 1], kn)
    for j in range(1, ncon + 1):                       # lines 858-929
        k = order(j)
        vN, kn = vec(k)
        l1, l2 = rng[:, k - 1]
        vtAv = vtAvp[k - 1, k - 1] + (coef[k - 1, l1 - 1:l2] @ vtvp[k - 1, l1 - 1:l2] if l1 <= l2 else 0.0)
        vAv = np.zeros(npar)
        for k2 in range(l1, l2 + 1):
            if coef[k - 1, k2 - 1] != 0.0:
                vAv += coef[k - 1, k2 - 1] * vec(k2)[0]
        update(vN, vAv, vtAv, kn)
        for j2 in range(j + 1, ncon + 1):
            k2 = order(j2)
            x = vtvp[k - 1, k2 - 1]
            l1, l2 = rng[:, k2 - 1]
            va = vtAvp[k2 - 1, k - 1]
            if l1 <= l2:
                va += coef[k2 - 1, l1 - 1:l2] @ vtvp[k - 1, l1 - 1:l2]
            l1, l2 = min(l1, k), max(l2, k)
            coef[k2 - 1, k - 1] += 2.0 * (2.0 * vtAv * x - va)
            if x != 0.0:
                l1, l2 = min(l1, rng[0, k - 1]), max(l2, rng[1, k - 1])
                coef[k2 - 1, l1 - 1:l2] -= 2.0 * coef[k - 1, l1 - 1:l2] * x
            rng[:, k2 - 1] = (l1, l2)
    out = np.zeros_like(M)
    for q, (i, l) in enumerate(idx):
        out[i - 1, l - 1] = out[l - 1, i - 1] = B[q]
    return out


def test_one_reflection_adds_four_beta_vvT():
    npar, mb = 20, 3
    rng = np.random.default_rng(1)
    V, Vk, r2 = qldec(rng.normal(size=(1, npar)))
    u = np.zeros(npar)
    u[:r2[0]] = V[0, :r2[0]]
    u[npar - 1] = Vk[0]
    M = rng.normal(size=(npar, npar))
    M = M + M.T + npar * np.eye(npar)
    H = np.eye(npar) - 2.0 * np.outer(u, u)
    got = qlpssq_band(M, V, Vk, r2, mb)
    i, j = np.indices(M.shape)
    band = np.abs(i - j) < mb
    extra = 4.0 * (u @ M @ u) * np.outer(u, u)
    assert np.max(np.abs((got - H @ M @ H - extra)[band])) <= 1e-12 * np.max(np.abs(M))
    assert np.max(np.abs((got - H @ M @ H)[band])) > 1e-3 * np.max(np.abs(M))


def test_oracle_literal_route_matches_restatement(orc):
    """The oracle's literal qlpssq route (mpref_set_qlpssq_literal) gives the
    band of the step-by-step restatement above (three constraints, packed
    matrix), compared through lltdec's factor of the fit rows."""
    import ctypes as C
    f64p, i32p, i64p = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
    npar, ncon, mb = 30, 3, 4
    rng = np.random.default_rng(5)
    A = np.ascontiguousarray(rng.normal(size=(ncon, npar)))
    V, Vk, r2 = qldec(A)
    M = rng.normal(size=(npar, npar))
    M = M + M.T + 4 * npar * np.eye(npar)
    want_band = qlpssq_band(M, V, Vk, r2, mb)
    L = orc.lib()
    nfit = npar - ncon
    india = np.zeros(npar, np.int64)
    L.mpref_band_index(C.c_int32(npar), C.c_int32(mb), india.ctypes.data_as(i64p))
    cw = np.zeros(int(india[nfit - 1]))
    for k in range(nfit):
        for jj in range(max(0, k - mb + 1), k + 1):
            cw[india[k] - 1 - k + jj] = want_band[k, jj]
    L.mpref_lltdec(C.c_int32(nfit), cw.ctypes.data_as(f64p), india.ctypes.data_as(i64p), C.c_int32(0))
    L.mpref_ql_create.restype = C.c_void_p
    q = L.mpref_ql_create(C.c_int32(npar), C.c_int32(ncon), A.ctypes.data_as(f64p))
    packed = np.ascontiguousarray(M[np.tril_indices(npar)], np.float64)
    aig = np.arange(1, npar + 2, dtype=np.int32)
    cg = np.zeros_like(cw)
    nrkd = C.c_int32()
    L.mpref_set_qlpssq_literal(C.c_int32(1))
    try:
        rc = L.mpref_band_precond(C.c_int32(1), C.c_int32(npar), C.c_int32(npar), aig.ctypes.data_as(i32p), None,
                                  None, packed.ctypes.data_as(f64p), C.c_void_p(q), C.c_int32(mb), C.c_int32(0),
                                  cg.ctypes.data_as(f64p), C.byref(nrkd))
    finally:
        L.mpref_set_qlpssq_literal(C.c_int32(0))
        L.mpref_ql_destroy(C.c_void_p(q))
    assert rc == 0 and nrkd.value == 0
    assert np.max(np.abs(cg - cw)) <= 1e-10 * np.max(np.abs(cw))


def test_literal_route_same_solution(mp):
    """MINRES on a job's QL-reduced system with the literal route's
    preconditioners (diagonal and band 6) reaches the solution of the exact
    preconditioners within 1e-8; only the iteration counts may differ."""
    import oracle_ref as O
    d = mp.generate(mp.gen_config("telescope", ntracks=3000, seed=9))
    L = O.lib()
    out = {}
    for literal in (0, 1):
        L.mpref_set_qlpssq_literal(literal)
        try:
            for mb in (0, 6):
                st = O.make_steer(metsol=4, matsto=2, mitera=1, mrestl=1e-13, itnlim=3000, mreqenf=5, mbandw=mb)
                r = O.run(d, st)
                assert r["rc"] == 0
                out[(literal, mb)] = r["parameter"]
        finally:
            L.mpref_set_qlpssq_literal(0)
    scale = np.max(np.abs(out[(0, 0)]))
    for key in ((1, 0), (1, 6), (0, 6)):
        assert np.max(np.abs(out[key] - out[(0, 0)])) <= 1e-8 * scale
