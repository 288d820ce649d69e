"""The CPU oracle against golden vectors of the reference's tinypede.py
(tests/golden/make_golden.py): same parameter set, global matrix and vector
within 1e-11 relative (band and dense local fits against tinypede's dense
inversion), constrained and unconstrained solutions within 1e-9 relative,
errors of the unconstrained fit within 1e-9 relative.

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


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def oracle_structure(mp, orc, name):
    c = G.CASES[name]
    d = G.case_data(mp, c)
    g = load(name)
    assert G.record_hash(d) == str(g["record_sha256"]), "generator output changed"
    fixed = np.array(c["fixed"], np.int32)
    S = orc.Structure(d, mreqenf=c["entries"], preLabel=fixed,
                      preSigma=-np.ones(len(fixed)), sparse=False)
    return c, d, g, S


@pytest.mark.parametrize("name", list(G.CASES))
def test_matrix_vector(mp, orc, name):
    c, d, g, S = oracle_structure(mp, orc, name)
    var = S.varIndex > 0
    np.testing.assert_array_equal(S.labels[var], g["labels"])
    o = S.loopbf(np.zeros(S.nTotal), matsto=1, lfitbb=1)
    assert sum(o["nrej"]) == 0
    n = S.nVar
    A = np.zeros((n, n))
    A[np.tril_indices(n)] = o["matD"]
    A = A + np.tril(A, -1).T
    assert rel(np.diag(A), g["diag"]) <= 1e-11
    assert rel(A @ G.probes(n).T, g["probe"]) <= 1e-11
    if "packed" in g:
        assert rel(A[np.tril_indices(n)], g["packed"]) <= 1e-11
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
