"""Steering "measurement" lines in sparse storage (pede.f90:7007-7042): the
parameter pairs of a measurement line belong to the sparse structure even
when no record holds them, so a measurement that links two modules of one
telescope layer (never on one track) contributes its off-diagonal element
as in full storage.  CPU: the oracle's job driver, sparse against packed."""
import numpy as np

import oracle_ref as orc


def telescope_with_measurements(mp):
    d = mp.generate(mp.gen_config("telescope", ntracks=3000, seed=31))
    nmod = 20
    # layer 2: modules 3 and 14 (a track crosses one module per layer);
    # layer 5: modules 0, 7 and 19 in one line
    a, b = 2 * nmod + 3 + 1, 2 * nmod + 14 + 1
    c, e, f = 5 * nmod + 0 + 1, 5 * nmod + 7 + 1, 5 * nmod + 19 + 1
    meas = (np.array([0, 2, 5], np.int32), np.array([a, b, c, e, f], np.int32),
            np.array([1.0, -1.0, 1.0, -2.0, 1.0]), np.array([0.001, -0.0005]),
            np.array([0.0005, 0.001]))
    return d, meas


def test_sparse_equals_packed_with_measurement_lines(mp):
    d, meas = telescope_with_measurements(mp)
    out = {}
    for matsto in (1, 2):
        st = orc.make_steer(metsol=4, matsto=matsto, mitera=1, mrestl=1e-14, itnlim=4000)
        o = orc.run(d, st, measurements=meas)
        assert o["rc"] == 0
        out[matsto] = o
    np.testing.assert_array_equal(out[1]["labels"], out[2]["labels"])
    p1, p2 = out[1]["parameter"], out[2]["parameter"]
    assert np.max(np.abs(p1 - p2)) <= 1e-9 * np.max(np.abs(p1))
    # the measurement lines moved the solution (they are not dropped)
    st = orc.make_steer(metsol=4, matsto=2, mitera=1, mrestl=1e-14, itnlim=4000)
    o0 = orc.run(d, st)
    assert np.max(np.abs(o0["parameter"] - p2)) > 1e-6 * np.max(np.abs(p2))
