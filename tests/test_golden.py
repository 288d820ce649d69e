"""The CPU oracle against golden vectors of the reference's tinypede.py
(tests/golden/make_golden.py): same parameter set, global matrix and vector
within 1e-11 relative (band and dense local fits against tinypede's dense
inversion; packed and mpbits-sparse storage), the same records rejected by
the chi2 cut (a case with outliers), constrained and unconstrained
solutions within 1e-9 relative, errors of the unconstrained fit within 1e-9
relative.

Errors of a constrained fit are not compared tightly: pede's qlssq
(mpqldec.f90:573-698) leaves out the -2 v_kn (A v)_c term in row kn of each
reflection, so its back-transformed covariance is not the exact constrained
covariance that tinypede's bordered inverse gives; the oracle follows pede.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

import sys  # noqa: E402

sys.path.insert(0, GOLD)
import make_golden as G  # noqa: E402


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def products(orc, matsto, matD, n, aig, offsets, columns):
    """(diagonal, M @ probes^T) of the global matrix in packed (matsto 1) or
    mpbits-sparse (matsto 2) storage; the sparse product by the oracle's
    avprd0 (pede.f90:5069-5232)."""
    import ctypes as C
    P = G.probes(n)
    if matsto == 1:
        A = np.zeros((n, n))
        A[np.tril_indices(n)] = matD
        A = A + np.tril(A, -1).T
        return np.diag(A).copy(), A @ P.T
    L = orc.lib()
    aig = np.ascontiguousarray(aig, np.int32)
    off = np.ascontiguousarray(offsets, np.int64)
    col = np.ascontiguousarray(columns, np.int32)
    m = np.ascontiguousarray(matD, np.float64)
    out = np.zeros((n, P.shape[0]))
    for k in range(P.shape[0]):
        x = np.ascontiguousarray(P[k])
        b = np.zeros(n)
        L.mpref_avprd0(C.c_int32(2), C.c_int32(n), orc.ptr(x, orc.f64p), orc.ptr(b, orc.f64p),
                       C.c_int32(len(aig) - 1), orc.ptr(aig, orc.i32p), orc.ptr(off, orc.i64p),
                       orc.ptr(col, orc.i32p), orc.ptr(m, orc.f64p))
        out[:, k] = b
    return m[:n].copy(), out


def check_rejections(nrej, g):
    """chi2 rejections (pede codes 5 and 6) equal to tinypede's, no others"""
    assert nrej[4] + nrej[5] == int(g["nrejects"])
    assert sum(nrej[:4]) == int(g["nbad"])


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def oracle_structure(mp, orc, name):
    c = G.CASES[name]
    d = G.case_data(mp, c)
    g = load(name)
    assert G.record_hash(d) == str(g["record_sha256"]), "generator output changed"
    fixed = np.array(c["fixed"], np.int32)
    S = orc.Structure(d, mreqenf=c["entries"], preLabel=fixed,
                      preSigma=-np.ones(len(fixed)), sparse=c.get("sparse", False))
    return c, d, g, S


@pytest.mark.parametrize("name", list(G.CASES))
def test_matrix_vector(mp, orc, name):
    c, d, g, S = oracle_structure(mp, orc, name)
    var = S.varIndex > 0
    np.testing.assert_array_equal(S.labels[var], g["labels"])
    matsto = 2 if c.get("sparse", False) else 1
    o = S.loopbf(np.zeros(S.nTotal), matsto=matsto, lfitbb=1, chicut=c.get("chicut", 0.0))
    check_rejections(o["nrej"], g)
    n = S.nVar
    dg, pr = products(orc, matsto, o["matD"], n, S.aig, S.offsets, S.columns)
    assert rel(dg, g["diag"]) <= 1e-11
    assert rel(pr, g["probe"]) <= 1e-11
    if "packed" in g:
        assert rel(o["matD"], g["packed"]) <= 1e-11
    assert rel(o["gvec"], g["vector"]) <= 1e-11


@pytest.mark.parametrize("name", ["telescope_con", "telescope_fix"])
def test_solution(mp, orc, name):
    c, d, g, S = oracle_structure(mp, orc, name)
    st = orc.make_steer(metsol=1, matsto=1, mitera=1, mreqenf=c["entries"])
    fixed = np.array(c["fixed"], np.int32)
    kw = {}
    if len(fixed):
        kw = dict(parLabel=fixed, parValue=np.zeros(len(fixed)), parSigma=-np.ones(len(fixed)))
    r = orc.run(d, st, constraints=c["constraints"], **kw)
    assert r["rc"] == 0
    var = r["varIndex"] > 0
    np.testing.assert_array_equal(r["labels"][var], g["labels"])
    assert rel(r["parameter"][var], g["solution"]) <= 1e-9
    if not c["constraints"]:
        assert rel(r["error"][var], g["error"]) <= 1e-9
    else:
        # pede's back-transform (see the module docstring): same scale only
        ratio = r["error"][var] / g["error"]
        assert np.all((ratio > 0.7) & (ratio < 1.3))
