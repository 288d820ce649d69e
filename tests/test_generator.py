"""The synthetic Mille generator (csrc/mpgen.cpp), no GPU: the threaded mode
(cfg.threads > 1, each track from its own seeded stream) is deterministic,
independent of the thread count, gives well-formed records with the same
geometry (labels, true misalignments, constraints) as the sequential
stream, and the oracle processes its records like any others."""
import numpy as np
import pytest

import oracle_ref as orc


@pytest.mark.parametrize("kind", ["telescope", "barrel", "brokenlines"])
def test_threaded_generation(mp, kind):
    cfg = mp.gen_config(kind, ntracks=6000, seed=17)
    if kind != "telescope":
        cfg.nmod = 600
    seq = mp.generate(cfg)
    out = {}
    for nt in (2, 5):
        cfg.threads = nt
        out[nt] = mp.generate(cfg)
    a, b = out[2], out[5]
    for k in ("recPtr", "inder", "glder"):
        np.testing.assert_array_equal(a[k], b[k])   # the same for any thread count
    assert len(a["recPtr"]) == len(seq["recPtr"]) == 6001
    assert a["recPtr"][0] == 0 and np.all(np.diff(a["recPtr"]) > 0)
    assert a["recPtr"][-1] == len(a["inder"])
    # the same detector: true misalignments and constraints
    np.testing.assert_array_equal(a["truth"], seq["truth"])
    np.testing.assert_array_equal(a["conLabel"], seq["conLabel"])
    # other tracks than the sequential stream, the same label set
    assert not np.array_equal(a["glder"][:100], seq["glder"][:100])
    la = np.unique(a["inder"][a["inder"] > 0])
    ls = np.unique(seq["inder"][seq["inder"] > 0])
    assert np.array_equal(la, ls) or len(np.setxor1d(la, ls)) < 0.05 * len(ls)


def test_threaded_records_fit(mp):
    """The oracle's data loop on threaded-mode records: every record decodes
    and fits (no rejection without outliers)."""
    cfg = mp.gen_config("barrel", ntracks=3000, seed=19)
    cfg.nmod = 600
    cfg.threads = 4
    d = mp.generate(cfg)
    S = orc.Structure(d, mreqenf=1, sparse=True)
    o = S.loopbf(np.zeros(S.nTotal), matsto=2)
    assert sum(o["nrej"]) == 0
    assert o["ndf"] > 0
