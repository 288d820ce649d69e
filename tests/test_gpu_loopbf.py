"""Data loop on the GPU (mpgpu_loopbf through the C-ABI) against the oracle:
record decisions bit-exact, vector / matrix / chi2 within 1e-12 relative
(the Schur products use fused multiply-adds and the accumulation order per
element is record order in both, the vector is summed per record first)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def close(a, b, tol=TOL):
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b)) / scale if a.size else 0.0
    assert err <= tol, f"max rel diff {err:.3e} > {tol:.1e}"


def run_pair(mp, orc, d, matsto, gpar=None, recFile=None, fileWeight=None, **opt):
    H = mp.HostStructure(d, mreqenf=5, sparse=(matsto == 2))
    O = orc.Structure(d, mreqenf=5, sparse=(matsto == 2))
    if gpar is None:
        gpar = np.zeros(H.nTotal)
    o = O.loopbf(gpar, matsto=matsto, **opt) if recFile is None else None
    with mp.Context() as ctx:
        ctx.set_layout(H, matsto)
        ctx.upload(H, recFile=recFile, fileWeight=fileWeight)
        g = ctx.loopbf(gpar, **opt)
        g["matD"] = ctx.matrix()
        g["status"] = ctx.status()
    return g, o, H


def check(g, o):
    np.testing.assert_array_equal(g["status"], o["status"])
    assert g["nrej"] == o["nrej"]
    np.testing.assert_array_equal(g["gcnt"], o["gcnt"])
    close(g["gvec"], o["gvec"])
    close(g["matD"], o["matD"])
    assert g["ndf"] == o["ndf"]
    assert abs(g["chi2"] - o["chi2"]) <= 1e-12 * abs(o["chi2"])


def test_telescope_packed(mp, orc):
    d = mp.generate(mp.gen_config("telescope", ntracks=3000, seed=5))
    g, o, _ = run_pair(mp, orc, d, 1)
    check(g, o)


def test_barrel_sparse(mp, orc):
    d = mp.generate(mp.gen_config("barrel", ntracks=20000, seed=6))
    g, o, _ = run_pair(mp, orc, d, 2)
    check(g, o)


def test_barrel_outliers_downweighting(mp, orc):
    cfg = mp.gen_config("barrel", ntracks=20000, seed=8)
    cfg.outlierFrac = 0.02
    d = mp.generate(cfg)
    rng = np.random.default_rng(3)
    H = mp.HostStructure(d, mreqenf=5)
    gpar = rng.normal(0, 1e-4, H.nTotal)
    for nloopn, lhuber in ((2, 2), (2, 3), (3, 5)):
        g, o, _ = run_pair(mp, orc, d, 2, gpar=gpar, nloopn=nloopn, lhuber=lhuber, chicut=4.0,
                           dwcut=0.2)
        check(g, o)
        assert sum(g["nrej"]) > 0


def test_chi2_cut_and_function_loop(mp, orc):
    cfg = mp.gen_config("telescope", ntracks=4000, seed=9)
    cfg.outlierFrac = 0.05
    d = mp.generate(cfg)
    g, o, _ = run_pair(mp, orc, d, 1, chicut=2.0, chhuge=10.0)
    check(g, o)
    assert g["nrej"][4] + g["nrej"][5] > 0
    # function-value loop: no matrix, vector only
    g, o, _ = run_pair(mp, orc, d, 1, icalcm=0, chicut=2.0)
    np.testing.assert_array_equal(g["status"], o["status"])
    close(g["gvec"], o["gvec"])


def test_deterministic_repeat(mp):
    d = mp.generate(mp.gen_config("barrel", ntracks=30000, seed=10))
    H = mp.HostStructure(d, mreqenf=5)
    with mp.Context(staging_bytes=8 << 20) as ctx:  # several chunks
        ctx.set_layout(H, 2)
        ctx.upload(H)
        a = ctx.loopbf(np.zeros(H.nTotal))
        ma = ctx.matrix()
        b = ctx.loopbf(np.zeros(H.nTotal))
        mb = ctx.matrix()
    assert np.array_equal(ma, mb) and np.array_equal(a["gvec"], b["gvec"])
    # device times of the fit and the accumulation from events on their streams
    assert b["msFit"] > 0 and b["msAccum"] > 0 and b["msLoop"] >= b["msFit"]


def test_chunking_consistent(mp):
    """Different staging sizes (record chunks) change only the grouping of the
    per-element sums: results agree to rounding, each one reproducible."""
    d = mp.generate(mp.gen_config("barrel", ntracks=10000, seed=12))
    H = mp.HostStructure(d, mreqenf=5)
    out = []
    for stage in (1 << 20, 1 << 30):
        with mp.Context(staging_bytes=stage) as ctx:
            ctx.set_layout(H, 2)
            ctx.upload(H)
            ctx.loopbf(np.zeros(H.nTotal))
            out.append(ctx.matrix())
    close(out[0], out[1])


@pytest.mark.parametrize("name,matsto,ntracks", [("barrel", 2, 8000), ("telescope", 1, 3000)])
def test_large_record_path(mp, orc, name, matsto, ntracks):
    """The large-record path (B and W in global memory, W B^T by the tiled
    update kernel), forced on records that also fit the per-warp form:
    same decisions, matrix and vector as the oracle."""
    d = mp.generate(mp.gen_config(name, ntracks=ntracks, seed=12))
    H = mp.HostStructure(d, mreqenf=5, sparse=(matsto == 2))
    O = orc.Structure(d, mreqenf=5, sparse=(matsto == 2))
    gpar = np.zeros(H.nTotal)
    o = O.loopbf(gpar, matsto=matsto)
    with mp.Context(flags=1) as ctx:
        ctx.set_layout(H, matsto)
        ctx.upload(H)
        g = ctx.loopbf(gpar)
        g["matD"] = ctx.matrix()
        g["status"] = ctx.status()
    check(g, o)


def test_brokenlines_large(mp, orc):
    """Broken-line records with up to 40 hits (nloc up to 80, up to 240
    globals): band local fits and the large-record path, against the
    oracle."""
    cfg = mp.gen_config("brokenlines", ntracks=1500, seed=13)
    d = mp.generate(cfg)
    g, o, _ = run_pair(mp, orc, d, 2)
    check(g, o)


def with_special_blocks(d, every_special=3, every_extra=4):
    """The records of d with (a) a special data block of two words, one of
    them a zero index word, after the header of every `every_special`-th
    record, and (b) two more measurements with one local and no global
    words, the second with a negative measured value, at the end of every
    `every_extra`-th record.  Both make the device decode take its
    sequential path (adjacent zero words); (a) is skipped by the decode as
    pede skips special data (pede.f90:2123-2128)."""
    rp, ind, gl = d["recPtr"], d["inder"], d["glder"]
    rp2, ind2, gl2 = [0], [], []
    for r in range(len(rp) - 1):
        a, b = int(rp[r]), int(rp[r + 1])
        wi, wg = list(ind[a:b]), list(gl[a:b])
        if r % every_special == 0:
            wi[1:1] = [0, 0, 3, 0]
            wg[1:1] = [0.0, -2.0, 1.5, 2.5]
        if r % every_extra == 1:
            wi += [0, 1, 0, 0, 1, 0]
            wg += [-0.4, 0.3, 0.2, -0.6, 0.5, 0.2]
        ind2 += wi
        gl2 += wg
        rp2.append(rp2[-1] + len(wi))
    out = dict(d)
    out["recPtr"] = np.array(rp2, np.int64)
    out["inder"] = np.array(ind2, np.int32)
    out["glder"] = np.array(gl2, np.float64)
    return out


@pytest.mark.parametrize("name,matsto", [("barrel", 2), ("telescope", 1)])
def test_special_blocks_sequential_decode(mp, orc, name, matsto):
    d = with_special_blocks(mp.generate(mp.gen_config(name, ntracks=3000, seed=21)))
    g, o, _ = run_pair(mp, orc, d, matsto)
    check(g, o)


def loop_with_flags(mp, d, flags, matsto=2):
    H = mp.HostStructure(d, mreqenf=5, sparse=(matsto == 2))
    with mp.Context(flags=flags) as ctx:
        ctx.set_layout(H, matsto)
        ctx.upload(H)
        gpar = np.zeros(H.nTotal)
        ctx.loopbf(gpar)                     # first loop: the tuner runs here
        g = ctx.loopbf(gpar)
        g["matD"] = ctx.matrix()
        g["status"] = ctx.status()
        g["buckets"] = ctx.fit_buckets()
    return g


def test_fit_buckets_same_loop(mp, orc):
    """Broken-line records of 4-40 hits (nloc 8-84) fall into several size
    classes with their own fit launches (and tuned warps per CTA); the loop
    agrees with the single-launch form, with the one-record-per-block form
    and with the oracle: decisions exactly, sums within 1e-12."""
    cfg = mp.gen_config("brokenlines", ntracks=3000, seed=41)
    d = mp.generate(cfg)
    gb = loop_with_flags(mp, d, 0)
    cnt, wpc, tms = gb["buckets"]
    assert np.count_nonzero(cnt) >= 3 and cnt.sum() == len(d["recPtr"]) - 1
    assert np.all(wpc[cnt > 0] != 0)
    for flags in (mp.FLAG_NO_BUCKETS, mp.FLAG_ONE_RECORD_PER_BLOCK):
        g = loop_with_flags(mp, d, flags)
        np.testing.assert_array_equal(g["status"], gb["status"])
        assert g["nrej"] == gb["nrej"] and g["ndf"] == gb["ndf"]
        close(g["gvec"], gb["gvec"])
        close(g["matD"], gb["matD"])
    O = orc.Structure(d, mreqenf=5, sparse=True)
    H = mp.HostStructure(d, mreqenf=5, sparse=True)
    o = O.loopbf(np.zeros(H.nTotal), matsto=2)
    check(gb, o)
