"""The device path through the C-ABI against the golden vectors of the
reference's tinypede.py (tests/golden/make_golden.py): global matrix and
vector from mpgpu_loopbf within 1e-11 relative (packed and mpbits-sparse
storage), the records rejected by the chi2 cut equal; solutions of whole jobs
(mpgpu_pede_run, inversion) within 1e-9 relative; errors of the
unconstrained job within 1e-9 relative (constrained errors follow pede's
qlssq, see test_golden.py)."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as G  # noqa: E402
from test_golden import check_rejections, load, products, rel  # noqa: E402
from test_gpu_pede import gpu_job  # noqa: E402


def case(mp, name):
    c = G.CASES[name]
    d = G.case_data(mp, c)
    g = load(name)
    assert G.record_hash(d) == str(g["record_sha256"]), "generator output changed"
    return c, d, g


@pytest.mark.parametrize("name", list(G.CASES))
def test_device_matrix_vector(mp, orc, name):
    c, d, g = case(mp, name)
    fixed = np.array(c["fixed"], np.int32)
    sparse = c.get("sparse", False)
    H = mp.HostStructure(d, mreqenf=c["entries"], preLabel=fixed, preSigma=-np.ones(len(fixed)),
                         sparse=sparse)
    matsto = 2 if sparse else 1
    with mp.Context() as ctx:
        ctx.set_layout(H, matsto)
        ctx.upload(H)
        o = ctx.loopbf(np.zeros(H.nTotal), chicut=c.get("chicut", 0.0))
        m = ctx.matrix()
    check_rejections(o["nrej"], g)
    n = H.nVar
    dg, pr = products(orc, matsto, m, n, H.aig, H.offsets, H.columns)
    assert rel(dg, g["diag"]) <= 1e-11
    assert rel(pr, g["probe"]) <= 1e-11
    if "packed" in g:
        assert rel(m, g["packed"]) <= 1e-11
    assert rel(o["gvec"], g["vector"]) <= 1e-11


@pytest.mark.parametrize("name", ["telescope_con", "telescope_fix"])
def test_device_solution(mp, orc, name):
    c, d, g = case(mp, name)
    st = orc.make_steer(metsol=1, matsto=1, mitera=1, mreqenf=c["entries"])
    fixed = np.array(c["fixed"], np.int32)
    kw = {}
    if len(fixed):
        kw = dict(parLabel=fixed, parValue=np.zeros(len(fixed)), parSigma=-np.ones(len(fixed)))
    r = gpu_job(mp, orc, d, st, constraints=c["constraints"], **kw)
    assert r["rc"] == 0
    var = r["varIndex"] > 0
    np.testing.assert_array_equal(r["labels"][var], g["labels"])
    assert rel(r["parameter"][var], g["solution"]) <= 1e-9
    if not c["constraints"]:
        assert rel(r["error"][var], g["error"]) <= 1e-9
