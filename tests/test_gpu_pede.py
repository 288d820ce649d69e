"""Whole alignment jobs through mpgpu_pede_run against the oracle's job
driver: label table, counts and rejections exact; parameters 1e-10
relative; inversion errors 1e-9 relative."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gpu_job(mp, orc, d, steer, struct_device=0, **jobkw):
    job, keep = orc.make_job(d, **jobkw)
    cap = len(d["inder"]) + 16
    res, kr = orc.make_result(cap, cls=mp.Result)
    st = mp.Steer(**{f: getattr(steer, f) for f, _ in mp.Steer._fields_ if f not in ("structDevice", "monitor", "monitorPulls", "monitorBins")})
    st.structDevice = struct_device
    jb = mp.Job(**{f: getattr(job, f) for f, _ in mp.Job._fields_ if f != "monPath"})
    rc = mp.lib().mpgpu_pede_run(None, C.byref(st), C.byref(jb), C.byref(res))
    n = res.nTotal
    return dict(rc=rc, labels=kr.labels[:n].copy(), parameter=kr.parameter[:n].copy(),
                error=kr.error[:n].copy(), counts=kr.counts[:n].copy(), nrej=list(res.nrej),
                fvalue=res.fvalue, ndf=res.ndf, nrank=res.nrank, itn=res.minresItn,
                varIndex=kr.varIndex[:n].copy())


def compare(g, o, errors):
    assert g["rc"] == 0 and o["rc"] == 0
    np.testing.assert_array_equal(g["labels"], o["labels"])
    np.testing.assert_array_equal(g["varIndex"], o["varIndex"])
    np.testing.assert_array_equal(g["counts"], o["counts"])
    assert g["nrej"] == o["nrej"]
    assert g["ndf"] == o["ndf"]
    scale = np.max(np.abs(o["parameter"]))
    assert np.max(np.abs(g["parameter"] - o["parameter"])) <= 1e-10 * scale
    assert abs(g["fvalue"] - o["fvalue"]) <= 1e-10 * abs(o["fvalue"])
    if errors:
        assert np.max(np.abs(g["error"] - o["error"]) / np.abs(o["error"])) <= 1e-9


def test_telescope_inversion(mp, orc):
    d = mp.generate(mp.gen_config("telescope", ntracks=5000))
    st = orc.make_steer(metsol=1, matsto=1, mitera=1)
    compare(gpu_job(mp, orc, d, st), orc.run(d, st), errors=True)


def test_telescope_decomposition_iterations(mp, orc):
    cfg = mp.gen_config("telescope", ntracks=5000, seed=3)
    cfg.outlierFrac = 0.02
    d = mp.generate(cfg)
    st = orc.make_steer(metsol=3, matsto=1, mitera=3, lhuber=2, chicut=30.0, chirem=6.0)
    compare(gpu_job(mp, orc, d, st), orc.run(d, st), errors=False)


def test_barrel_sparse_minres(mp, orc):
    d = mp.generate(mp.gen_config("barrel", ntracks=30000, seed=4))
    st = orc.make_steer(metsol=4, matsto=2, mitera=2, lhuber=2, mrestl=1e-12, itnlim=3000,
                        mreqenf=5)
    g = gpu_job(mp, orc, d, st)
    o = orc.run(d, st)
    assert g["rc"] == 0 and o["rc"] == 0
    np.testing.assert_array_equal(g["counts"], o["counts"])
    assert g["nrej"] == o["nrej"]
    scale = np.max(np.abs(o["parameter"]))
    assert np.max(np.abs(g["parameter"] - o["parameter"])) <= 1e-8 * scale


@pytest.mark.parametrize("kind,metsol,matsto", [("barrel", 4, 2), ("telescope", 1, 1)])
def test_structure_on_device_same_job(mp, orc, kind, metsol, matsto):
    """The job with its structure passes on the device (steer structDevice)
    gives the results of the job with host passes, bit for bit."""
    d = mp.generate(mp.gen_config(kind, ntracks=20000 if kind == "barrel" else 5000, seed=5))
    st = orc.make_steer(metsol=metsol, matsto=matsto, mitera=2, lhuber=2, mrestl=1e-12, itnlim=3000,
                        mreqenf=5)
    h = gpu_job(mp, orc, d, st, struct_device=0)
    g = gpu_job(mp, orc, d, st, struct_device=1)
    assert h["rc"] == 0 and g["rc"] == 0
    for k in ("labels", "varIndex", "counts", "parameter", "error"):
        np.testing.assert_array_equal(g[k], h[k], err_msg=k)
    assert g["nrej"] == h["nrej"] and g["ndf"] == h["ndf"] and g["fvalue"] == h["fvalue"]


def test_barrel_sparse_minresqlp(mp, orc):
    """Whole job with MINRES-QLP (metsol 5) against the oracle's job driver."""
    d = mp.generate(mp.gen_config("barrel", ntracks=30000, seed=4))
    st = orc.make_steer(metsol=5, matsto=2, mitera=2, lhuber=2, mrestl=1e-12, itnlim=3000,
                        mreqenf=5)
    g = gpu_job(mp, orc, d, st)
    o = orc.run(d, st)
    assert g["rc"] == 0 and o["rc"] == 0
    np.testing.assert_array_equal(g["counts"], o["counts"])
    assert g["nrej"] == o["nrej"]
    scale = np.max(np.abs(o["parameter"]))
    assert np.max(np.abs(g["parameter"] - o["parameter"])) <= 1e-8 * scale
