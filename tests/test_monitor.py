"""Monitoring helpers on the host (no device): the grouping of the
measurements by their first global label (mpgpu_monitor_groups) against a
Python decode of the same records, and the millepede.mon lines
(mpgpu_write_mon) against a numpy restatement of monres's median and
median absolute deviation."""
import numpy as np


def measurements(inder, glder, a, b):
    """(startLocal, startGlobal, lastGlobal) of each measurement of the
    record [a, b) (decodeNextMeasurement, without special blocks)."""
    out, lg, end = [], a, b - 1
    while lg < end:
        sl = next(q for q in range(lg + 1, end + 1) if inder[q] == 0)
        sg = next(q for q in range(sl + 1, end + 1) if inder[q] == 0)
        nz = next((q for q in range(sg + 1, end + 1) if inder[q] == 0), None)
        lg = end if nz is None else nz - 1
        out.append((sl, sg, lg))
    return out


def test_monitor_groups(mp):
    d = mp.generate(mp.gen_config("barrel", ntracks=300, seed=5))
    S = mp.HostStructure(d, mreqenf=1, sparse=False)
    mi, mr = mp.monitor_groups(S)
    cnt, tot = {}, {}
    for r in range(len(S.recPtr) - 1):
        for sl, sg, lg in measurements(S.tinder, S.glder, S.recPtr[r], S.recPtr[r + 1]):
            if lg > sg:
                ij = S.tinder[sg + 1]
                cnt[ij] = cnt.get(ij, 0) + 1
                tot[ij] = tot.get(ij, 0.0) + S.glder[sg]
    keys = sorted(cnt)
    assert len(mr) == len(keys)
    for g, ij in enumerate(keys):
        assert mi[ij - 1] == g + 1
        assert mr[g] == tot[ij] / cnt[ij]
    assert np.count_nonzero(mi) == len(keys)


def median_mad(h, bins=100, size=np.float32(0.1)):
    """monres (pede.f90:7533-7633) for one group, single precision."""
    f = np.float32
    c = np.cumsum(h)
    n = int(c[-1])
    if n == 0:
        return f(0), f(0)
    j = next(k for k in range(2, bins + 1) if 2 * c[k - 1] > n)
    med = f(j)
    if c[j - 1] > c[j - 2]:
        med = f(med + f(n - 2 * c[j - 2]) / f(2 * c[j - 1] - 2 * c[j - 2]))
    med = f(size * f(med - f(bins // 2)))
    s = np.zeros(bins + 1, np.int64)
    for k in range(j, bins + 1):
        s[k - j + 1] += h[k - 1]
    for k in range(j - 1, 0, -1):
        s[j - k] += h[k - 1]
    s = np.cumsum(s)
    jj = next(k for k in range(2, bins + 1) if 2 * s[k] > n)
    mad = f(jj - 1)
    if s[jj] > s[jj - 1]:
        mad = f(mad + f(n - 2 * s[jj - 1]) / f(2 * s[jj] - 2 * s[jj - 1]))
    return med, f(size * mad)


def test_write_mon(mp, tmp_path):
    rng = np.random.default_rng(3)
    hist = np.zeros((3, 100), np.int64)
    for g, (loc, sc, n) in enumerate([(0.0, 1.0, 5000), (0.7, 2.5, 300), (-1.2, 0.5, 50)]):
        x = rng.normal(loc, sc, n)
        b = np.clip((x / 0.1 + 50).astype(np.int64), 1, 100)
        np.add.at(hist[g], b - 1, 1)
    labels = np.array([11, 22, 33], np.int32)
    res = np.array([0.002, 0.004, 0.008])
    p = tmp_path / "millepede.mon"
    mp.write_mon(p, 1, 1, 2, labels, hist, res)
    lines = open(p).read().splitlines()
    assert lines[0].startswith("*** Pulls grouped by first global label")
    assert lines[1].startswith("! LFC     Label   Entries")
    for g, line in enumerate(lines[2:]):
        lfc, lab, nent, med, mad, err = line.split()
        assert int(lfc) == 2 and int(lab) == labels[g] and int(nent) == hist[g].sum()
        wm, wd = median_mad(hist[g])
        assert abs(float(med) - wm) <= 1e-4 * max(1.0, abs(wm))
        assert abs(float(mad) - wd * np.float32(1.4826)) <= 1e-4 * max(1.0, wd)
        assert abs(float(err) - res[g]) <= 1e-6
