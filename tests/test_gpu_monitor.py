"""Monitoring on the device (mpgpu_set_monitor / mpgpu_get_monitor)
against the oracle's restatement on the same records: the normalized
residual and pull histograms and the per-group bins of the measurement
monitor equal, count for count, for dense local fits (pulls and scaled
residuals); for band local fits, whose local covariance the device forms
by another route (the same matrix up to rounding), the residual histograms
equal and at most 0.2 % of the pull entries move between bins."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_both(mp, orc, d, matsto, mode, nbins=80, rng=4.0, meas_bins=100):
    H = mp.HostStructure(d, mreqenf=5, sparse=(matsto == 2))
    mi, mr = mp.monitor_groups(H)
    with mp.Context() as ctx:
        ctx.set_layout(H, matsto)
        ctx.upload(H)
        ctx.set_monitor(nbins=nbins, rng=rng, meas_bins=meas_bins, mode=mode, meas_index=mi, meas_res=mr)
        ctx.loopbf(np.zeros(H.nTotal))
        hg, mg = ctx.get_monitor()
    O = orc.Structure(d, mreqenf=5, sparse=(matsto == 2))
    ho = np.zeros(4 * (nbins + 2), np.int64)
    mo = np.zeros(max(len(mr) * meas_bins, 1), np.int64)
    i32p, i64p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)
    L = orc.lib()
    L.mpref_set_monitor(C.c_int32(1), C.c_int32(1), C.c_int32(nbins), C.c_float(rng), C.c_int32(meas_bins),
                        C.c_int32(mode), mi.ctypes.data_as(i32p), mr.ctypes.data_as(f64p),
                        ho.ctypes.data_as(i64p), mo.ctypes.data_as(i64p))
    try:
        O.loopbf(np.zeros(O.nTotal), matsto=matsto)
    finally:
        L.mpref_set_monitor(C.c_int32(0), C.c_int32(0), C.c_int32(1), C.c_float(1.0), C.c_int32(1), C.c_int32(0),
                            None, None, None, None)
    return hg, mg, ho.reshape(4, nbins + 2), mo[:len(mr) * meas_bins].reshape(len(mr), meas_bins)


@pytest.mark.parametrize("kind,matsto,mode", [("barrel", 2, 1), ("telescope", 1, 0)])
def test_monitor_dense_fits_exact(mp, orc, kind, matsto, mode):
    d = mp.generate(mp.gen_config(kind, ntracks=4000, seed=51))
    hg, mg, ho, mo = run_both(mp, orc, d, matsto, mode)
    assert hg.sum() > 0 and mg.sum() > 0
    np.testing.assert_array_equal(hg, ho)
    np.testing.assert_array_equal(mg, mo)


def test_monitor_band_fits(mp, orc):
    d = mp.generate(mp.gen_config("brokenlines", ntracks=600, seed=52))
    hg, mg, ho, mo = run_both(mp, orc, d, 2, 1)
    np.testing.assert_array_equal(hg[:2], ho[:2])          # residuals: no covariance involved
    assert abs(int(hg[2:].sum()) - int(ho[2:].sum())) <= max(2, 0.001 * ho[2:].sum())
    assert np.abs(hg[2:] - ho[2:]).sum() <= max(2, 0.002 * ho[2:].sum())
    assert np.abs(mg - mo).sum() <= max(2, 0.002 * mo.sum())


def test_job_writes_monitor_file(mp, orc, tmp_path):
    """monitorpulls 3 in a whole job (mpgpu_pede_run): millepede.mon holds
    the header, the group lines after the first data loop, equal to those
    of the oracle's histograms of that loop, and the lines after the last."""
    d = mp.generate(mp.gen_config("telescope", ntracks=3000, seed=53))
    job, keep = orc.make_job(d)
    res, kr = orc.make_result(len(d["inder"]) + 16, cls=mp.Result)
    steer = orc.make_steer(metsol=1, matsto=1, mitera=2)
    st = mp.Steer(**{f: getattr(steer, f) for f, _ in mp.Steer._fields_
                     if f not in ("structDevice", "monitor", "monitorPulls", "monitorBins")})
    st.monitor, st.monitorPulls, st.monitorBins = 3, 1, 100
    path = tmp_path / "millepede.mon"
    jb = mp.Job(**{f: getattr(job, f) for f, _ in mp.Job._fields_ if f != "monPath"})
    jb.monPath = str(path).encode()
    assert mp.lib().mpgpu_pede_run(None, C.byref(st), C.byref(jb), C.byref(res)) == 0
    lines = path.read_text().splitlines()

    H = mp.HostStructure(d, mreqenf=25, sparse=False)
    mi, mr = mp.monitor_groups(H)
    O = orc.Structure(d, mreqenf=25, sparse=False)
    mo = np.zeros(max(len(mr) * 100, 1), np.int64)
    ho = np.zeros(4 * 102, np.int64)
    i32p, i64p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)
    L = orc.lib()
    L.mpref_set_monitor(C.c_int32(1), C.c_int32(1), C.c_int32(100), C.c_float(5.0), C.c_int32(100),
                        C.c_int32(1), mi.ctypes.data_as(i32p), mr.ctypes.data_as(f64p),
                        ho.ctypes.data_as(i64p), mo.ctypes.data_as(i64p))
    try:
        O.loopbf(np.zeros(O.nTotal), matsto=1)
    finally:
        L.mpref_set_monitor(C.c_int32(0), C.c_int32(0), C.c_int32(1), C.c_float(1.0), C.c_int32(1), C.c_int32(0),
                            None, None, None, None)
    glab = np.zeros(len(mr), np.int32)
    for i in np.nonzero(mi > 0)[0]:
        glab[mi[i] - 1] = H.labels[i]
    ref = tmp_path / "ref.mon"
    mp.write_mon(ref, 1, 1, 1, glab, mo[:len(mr) * 100].reshape(len(mr), 100), mr)
    want = ref.read_text().splitlines()
    ng = len(mr)
    assert ng > 0 and len(lines) == 2 + 2 * ng
    assert lines[:2 + ng] == want
    assert all(s.split()[0] == "2" for s in lines[2 + ng:])
    assert [s.split()[1] for s in lines[2 + ng:]] == [s.split()[1] for s in want[2:]]
