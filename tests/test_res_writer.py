"""millepede.res (prtglo, pede.f90:4477-4651) and feasib (pede.f90:1553-1680)
on the host, no GPU: the oracle's job driver with start values that violate
the constraints (feasib makes them feasible before the first data loop),
the writer's columns ("differ" = parameter - start value, printcounts with
the lowstat sign, globalcorr), the library's writer equal to the oracle's
byte for byte, and the fixed-column layout of the reference's own golden
file CI/refFiles/millepede.res (its layout facts from
tests/golden/millepede_res_layout.json; every line where MILLEPEDE_SOURCES
names the sources)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle_ref as orc

# the reference's golden file, read where the Millepede-II sources are
# (MILLEPEDE_SOURCES, as for tests/golden/make_golden.py)
REF_RES = os.path.join(os.environ.get("MILLEPEDE_SOURCES", ""), "CI", "refFiles", "millepede.res")

# prtglo's record layouts: i10, 2X, then 2..4 G14.5 fields, then either
# F8.3 (102 with globalcorr) or blanks + I12 (110: 28X, 111: 14X, 112: none)
G145 = r"[ -][ 0-9.E+-]{13}"


def parse_line(line):
    """(label, [floats], count or None, gcor or None) of one res line by its
    fixed columns; raises ValueError when the columns do not fit."""
    body = line.rstrip("\n")
    label = int(body[:10])
    if body[10:12] != "  ":
        raise ValueError("no 2X after the label")
    rest = body[12:]
    vals = []
    while len(rest) >= 14 and re.fullmatch(G145, rest[:14]) and rest[:14].strip():
        vals.append(float(rest[:14].replace("E", "e")))
        rest = rest[14:]
    count = gcor = None
    if rest:
        if len(rest) == 8:
            gcor = float(rest)
        else:
            if len(rest) < 12 or rest[:-12].strip():
                raise ValueError("unexpected columns: %r" % rest)
            count = int(rest[-12:])
    return label, vals, count, gcor


def telescope_job(mp, start_shift):
    d = mp.generate(mp.gen_config("telescope", ntracks=3000, seed=21))
    labels = np.unique(d["inder"][d["inder"] > 0])
    labels = labels[labels >= 1][:40]
    rng = np.random.default_rng(5)
    values = rng.normal(0.0, start_shift, len(labels))
    sigmas = np.zeros(len(labels))
    sigmas[::13] = -1.0   # some fixed parameters (pre-sigma < 0)
    return d, labels, values, sigmas


def constraint_residuals(d, out):
    pos = {int(l): i for i, l in enumerate(out["labels"])}
    cs, cl, cc = d["conStart"], d["conLabel"], d["conCoef"]
    r = []
    for c in range(d["ncon"]):
        v = 0.0
        for k in range(cs[c], cs[c + 1]):
            v -= cc[k] * out["parameter"][pos[int(cl[k])]]
        r.append(v)
    return np.array(r)


def test_feasib_and_start_values(mp):
    d, labels, values, sigmas = telescope_job(mp, 0.01)
    st = orc.make_steer(metsol=1, matsto=1, mitera=2)
    o = orc.run(d, st, parLabel=labels, parValue=values, parSigma=sigmas)
    assert o["rc"] == 0
    pos = {int(l): i for i, l in enumerate(o["labels"])}
    # globalParStart are the steering values, not the feasible ones
    for l, v in zip(labels, values):
        assert o["start"][pos[int(l)]] == v
    # the job's result satisfies the constraints
    assert np.max(np.abs(constraint_residuals(d, o))) < 1e-9
    # without constraints the start values are kept as they are by feasib
    o2 = orc.run(d, st, parLabel=labels, parValue=values, parSigma=sigmas, constraints=False)
    assert o2["rc"] == 0
    # global correlations: defined in [0, 1] for variable parameters
    var = o["varIndex"] > 0
    assert np.all((o["gcor"][var] >= 0.0) & (o["gcor"][var] <= 1.0))
    assert np.all(o["gcor"][~var] == -1.0)


def write_both(mp, o, tmp_path, errors, ipcntr, igcorr, mreqena):
    """The oracle's and the library's writer on the same result."""
    L = orc.lib()
    p1 = tmp_path / "oracle.res"
    p2 = tmp_path / "mpgpu.res"
    rc = L.mpref_write_res_opts(str(p1).encode(), C.byref(o["result"]), C.c_int32(errors),
                                C.c_int32(ipcntr), C.c_int32(igcorr), C.c_int32(mreqena))
    assert rc == 0
    # the library's writer reads the same fields (its struct has two more
    # scalars before the optional arrays)
    r = mp.Result()
    for f, _ in orc.Result._fields_:
        setattr(r, f, getattr(o["result"], f))
    opts = mp.ResOpts(errors=errors, ipcntr=ipcntr, igcorr=igcorr, mreqena=mreqena)
    assert mp.lib().mpgpu_write_res_opts(str(p2).encode(), C.byref(r), C.byref(opts)) == 0
    return p1.read_text(), p2.read_text()


@pytest.mark.parametrize("errors,ipcntr,igcorr", [(1, 0, 0), (1, 0, 1), (1, 1, 0), (0, 1, 0),
                                                  (0, 2, 0), (0, 0, 0)])
def test_writer_columns(mp, tmp_path, errors, ipcntr, igcorr):
    d, labels, values, sigmas = telescope_job(mp, 0.002)
    st = orc.make_steer(metsol=1, matsto=1, mitera=1, mreqena=2000)
    o = orc.run(d, st, parLabel=labels, parValue=values, parSigma=sigmas)
    assert o["rc"] == 0
    a, b = write_both(mp, o, tmp_path, errors, ipcntr, igcorr, mreqena=2000)
    assert a == b
    lines = a.splitlines()
    assert lines[0] == " Parameter   ! first 3 elements per line are significant (if used as input)"
    assert len(lines) == 1 + len(o["labels"])
    for k, line in enumerate(lines[1:]):
        lab, vals, count, gcor = parse_line(line)
        assert lab == o["labels"][k]
        np.testing.assert_allclose(vals[0], o["parameter"][k], rtol=5.1e-5, atol=1e-9)
        if o["varIndex"][k] <= 0:
            assert len(vals) == 2
            if ipcntr:
                assert count == (o["fileCounts"][k] if ipcntr > 1 else 0)
            continue
        assert len(vals) == (4 if errors else 3)
        # differ = parameter - start value (pede.f90:4535)
        np.testing.assert_allclose(vals[2], o["parameter"][k] - o["start"][k], rtol=5.1e-5, atol=1e-9)
        if errors:
            np.testing.assert_allclose(vals[3], o["error"][k], rtol=5.1e-5)
        if ipcntr:
            n = o["fileCounts"][k] if ipcntr > 1 else o["counts"][k]
            low = o["counts"][k] < 2000
            assert count == (-(n + 1) if low else n)
        elif igcorr and errors:
            assert gcor == pytest.approx(o["gcor"][k], abs=6e-4)
        else:
            assert count is None and gcor is None
        # the same record width as pede's formats
        width = 12 + 14 * len(vals) + (12 + (14 if not errors else 0) if ipcntr else 0) + \
            (8 if (igcorr and errors and not ipcntr) else 0)
        assert len(line) == width


@pytest.mark.skipif(not os.environ.get("MILLEPEDE_SOURCES") or not os.path.exists(REF_RES),
                    reason="MILLEPEDE_SOURCES not set or without CI/refFiles/millepede.res")
def test_layout_of_reference_golden_file(mp, tmp_path):
    """Every line of the reference's golden millepede.res (printcounts,
    no errors: formats 110/111) parses with the column parser above, and a
    result written with the same options has the same line structure."""
    with open(REF_RES) as f:
        ref = f.read().splitlines()
    assert ref[0].strip().startswith("Parameter")
    shapes = set()
    for line in ref[1:]:
        lab, vals, count, gcor = parse_line(line)
        assert count is not None and gcor is None
        shapes.add((len(vals), len(line)))
    d, labels, values, sigmas = telescope_job(mp, 0.002)
    st = orc.make_steer(metsol=3, matsto=1, mitera=1, mreqena=10)
    o = orc.run(d, st, parLabel=labels, parValue=values, parSigma=sigmas)
    a, _ = write_both(mp, o, tmp_path, errors=0, ipcntr=1, igcorr=0, mreqena=10)
    ours = set()
    for line in a.splitlines()[1:]:
        lab, vals, count, gcor = parse_line(line)
        if len(vals) == 3:
            ours.add((len(vals), len(line)))
    assert ours and ours <= shapes | {(3, 80)}
    assert (3, 80) in shapes


def test_layout_of_reference_golden_fixture(mp, tmp_path):
    """The layout facts of the reference's golden millepede.res
    (tests/golden/millepede_res_layout.json, made by make_res_layout.py):
    its sample lines parse with the column parser above (value, presigma,
    difference and the count of format 110/111), and a result written with
    the same options has lines of the same length."""
    import json
    with open(os.path.join(os.path.dirname(__file__), "golden", "millepede_res_layout.json")) as f:
        fx = json.load(f)
    assert fx["header"].strip().startswith("Parameter")
    assert [s[2] for s in fx["shapes"]] == [fx["nlines"]]
    width = fx["shapes"][0][1]
    for line in fx["samples"]:
        lab, vals, count, gcor = parse_line(line)
        assert len(vals) == 3 and count is not None and gcor is None
        assert len(line) == width
    d, labels, values, sigmas = telescope_job(mp, 0.002)
    st = orc.make_steer(metsol=3, matsto=1, mitera=1, mreqena=10)
    o = orc.run(d, st, parLabel=labels, parValue=values, parSigma=sigmas)
    a, _ = write_both(mp, o, tmp_path, errors=0, ipcntr=1, igcorr=0, mreqena=10)
    ours = [line for line in a.splitlines()[1:] if len(parse_line(line)[1]) == 3]
    assert ours and all(len(line) == width for line in ours)


def test_writer_rejects_zero_counts(mp, tmp_path):
    r = mp.Result()
    opts = mp.ResOpts(errors=0, ipcntr=-1, igcorr=0, mreqena=10)
    assert mp.lib().mpgpu_write_res_opts(str(tmp_path / "x.res").encode(), C.byref(r), C.byref(opts)) == 44
