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


def test_start_values_feasib_and_res(mp, orc, tmp_path):
    """Start values that violate the constraints (feasib before the first
    data loop), inversion with global correlations: parameters, errors,
    start values, correlations and entries as the oracle's job, and the
    millepede.res written from both results (printcounts, globalcorr)
    identical text."""
    d = mp.generate(mp.gen_config("telescope", ntracks=4000, seed=21))
    labels = np.unique(d["inder"][d["inder"] > 0])[:40]
    rng = np.random.default_rng(5)
    values = rng.normal(0.0, 0.01, len(labels))
    sigmas = np.zeros(len(labels))
    sigmas[::13] = -1.0
    st = orc.make_steer(metsol=1, matsto=1, mitera=2, lhuber=1, chicut=30.0, chirem=6.0)
    kw = dict(parLabel=labels, parValue=values, parSigma=sigmas)
    job, keep = orc.make_job(d, **kw)
    cap = len(d["inder"]) + 16
    res, kr = orc.make_result(cap, cls=mp.Result)
    gst = mp.Steer(**{f: getattr(st, f) for f, _ in mp.Steer._fields_ if hasattr(st, f)})
    gjob = mp.Job(**{f: getattr(job, f) for f, _ in mp.Job._fields_ if hasattr(job, f)})
    assert mp.lib().mpgpu_pede_run(None, C.byref(gst), C.byref(gjob), C.byref(res)) == 0
    o = orc.run(d, st, **kw)
    assert o["rc"] == 0
    n = res.nTotal
    np.testing.assert_array_equal(kr.start[:n], o["start"])
    np.testing.assert_array_equal(kr.fileCounts[:n], o["fileCounts"])
    np.testing.assert_array_equal(kr.counts[:n], o["counts"])
    scale = np.max(np.abs(o["parameter"]))
    assert np.max(np.abs(kr.parameter[:n] - o["parameter"])) <= 1e-10 * scale
    var = o["varIndex"] > 0
    assert np.max(np.abs(kr.error[:n][var] - o["error"][var]) / np.abs(o["error"][var])) <= 1e-9
    assert np.max(np.abs(kr.gcor[:n] - o["gcor"])) <= 1e-6
    for opts in ((1, 1, 0), (1, 0, 1)):
        p1, p2 = tmp_path / "gpu.res", tmp_path / "oracle.res"
        ro = mp.ResOpts(errors=opts[0], ipcntr=opts[1], igcorr=opts[2], mreqena=10)
        assert mp.lib().mpgpu_write_res_opts(str(p1).encode(), C.byref(res), C.byref(ro)) == 0
        assert orc.lib().mpref_write_res_opts(str(p2).encode(), C.byref(o["result"]), C.c_int32(opts[0]),
                                              C.c_int32(opts[1]), C.c_int32(opts[2]), C.c_int32(10)) == 0
        a, b = p1.read_text().splitlines(), p2.read_text().splitlines()
        assert len(a) == len(b)
        # single-precision text of values equal up to the last printed digit
        diff = sum(1 for x, y in zip(a, b) if x != y)
        assert diff <= max(2, len(a) // 100), diff


def test_measurement_lines(mp, orc):
    """Steering measurement lines (pede.f90:2743-2798) in a whole job: the
    GPU job equals the oracle's in packed storage (inversion, with errors)
    and in sparse storage (MINRES), where the pairs of the lines, two
    modules of one telescope layer that no track crosses together, are in
    the structure (pede.f90:7007-7042)."""
    import test_measurement_pairs as T
    d, meas = T.telescope_with_measurements(mp)
    st = orc.make_steer(metsol=1, matsto=1, mitera=1)
    compare(gpu_job(mp, orc, d, st, measurements=meas), orc.run(d, st, measurements=meas), errors=True)
    st = orc.make_steer(metsol=4, matsto=2, mitera=1, mrestl=1e-14, itnlim=4000)
    g = gpu_job(mp, orc, d, st, measurements=meas)
    o = orc.run(d, st, measurements=meas)
    assert g["rc"] == 0 and o["rc"] == 0
    np.testing.assert_array_equal(g["labels"], o["labels"])
    scale = np.max(np.abs(o["parameter"]))
    assert np.max(np.abs(g["parameter"] - o["parameter"])) <= 1e-9 * scale
