"""mpgpu_mupdat_noalloc (staging in a fixed device area, no allocation)
against mpgpu_mupdat through the C-ABI: the global matrix after a data loop
plus two update calls in a row agrees within 1e-12 relative (both run the
same kernel in the same order, so it is expected to be identical); both
against the oracle's mupdat (pede.f90:3134-3204) applied to the same
matrix, on packed and on mpbits-sparse storage where most random pairs are
not stored and are suppressed, and on a pairentries layout whose left-out
pairs are dropped; a call above the area's capacity is rejected and leaves
the matrix unchanged."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def close(a, b, tol=TOL):
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b)) / scale
    assert err <= tol, f"max rel diff {err:.3e} > {tol:.1e}"


def batches(nvar, sizes, seed):
    """(i, j, add) triplets: random pairs, diagonal terms, zero adds and
    unused slots (index 0), as mupdat receives them."""
    rng = np.random.default_rng(seed)
    out = []
    for n in sizes:
        i = rng.integers(1, nvar + 1, n).astype(np.int32)
        j = rng.integers(1, nvar + 1, n).astype(np.int32)
        j[::7] = i[::7]
        add = rng.normal(size=n)
        add[::11] = 0.0
        i[::13] = 0
        out.append((i, j, add))
    return out


def setup(mp, kind, matsto, ntracks):
    d = mp.generate(mp.gen_config(kind, ntracks=ntracks, seed=17))
    H = mp.HostStructure(d, mreqenf=5, sparse=(matsto == 2))
    ctx = mp.Context()
    ctx.set_layout(H, matsto)
    ctx.upload(H)
    return ctx, H


@pytest.mark.parametrize("kind,matsto", [("telescope", 1), ("barrel", 2)])
def test_noalloc_matches_mupdat(mp, kind, matsto):
    ctx, H = setup(mp, kind, matsto, 3000)
    with ctx:
        gpar = np.zeros(H.nTotal)
        b1, b2 = batches(ctx.nVar, [5000, 65536], seed=4)
        ctx.loopbf(gpar)
        base = ctx.matrix()
        ctx.mupdat(*b1)
        ctx.mupdat(*b2)
        ref = ctx.matrix()
        ctx.loopbf(gpar)
        np.testing.assert_array_equal(ctx.matrix(), base)
        ctx.mupdat_noalloc(*b1)
        ctx.mupdat_noalloc(*b2)
        got = ctx.matrix()
    assert np.any(ref != base)
    close(got, ref)


def test_noalloc_limits(mp):
    ctx, H = setup(mp, "telescope", 1, 500)
    with ctx:
        ctx.loopbf(np.zeros(H.nTotal))
        base = ctx.matrix()
        nmax = 65536
        i = np.ones(nmax + 1, np.int32)
        with pytest.raises(RuntimeError, match="error 45"):
            ctx.mupdat_noalloc(i, i, np.ones(nmax + 1))
        np.testing.assert_array_equal(ctx.matrix(), base)
        # an index beyond the matrix: code 23, as from mpgpu_mupdat
        bad = np.array([ctx.nVar + 1], np.int32)
        with pytest.raises(RuntimeError, match="error 23"):
            ctx.mupdat_noalloc(bad, bad, np.ones(1))
        with pytest.raises(RuntimeError, match="error 23"):
            ctx.mupdat(bad, bad, np.ones(1))
        ctx.mupdat_noalloc(i[:0], i[:0], np.ones(0))
        np.testing.assert_array_equal(ctx.matrix(), base)


def oracle_mupdat(orc, H, matsto, base, batches_):
    """The oracle's mupdat applied in order to a copy of base."""
    L = orc.lib()
    m = np.ascontiguousarray(base.copy())
    aig = np.ascontiguousarray(H.aig, np.int32)
    p2g = np.zeros(H.nVar, np.int32)
    for g in range(len(aig) - 1):
        p2g[aig[g] - 1:aig[g + 1] - 1] = g + 1
    off = np.ascontiguousarray(H.offsets, np.int64)
    col = np.ascontiguousarray(H.columns, np.int32)
    f64p, i32p, i64p = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
    mp_ = m.ctypes.data_as(f64p)
    args = (C.c_int32(H.nG), aig.ctypes.data_as(i32p), p2g.ctypes.data_as(i32p),
            off.ctypes.data_as(i64p), col.ctypes.data_as(i32p), mp_)
    for i, j, a in batches_:
        for q in range(len(i)):
            L.mpref_mupdat(C.c_int32(matsto), C.c_int32(int(i[q])), C.c_int32(int(j[q])),
                           C.c_double(float(a[q])), *args)
    return m


@pytest.mark.parametrize("kind,matsto", [("telescope", 1), ("barrel", 2)])
def test_noalloc_and_mupdat_match_oracle(mp, orc, kind, matsto):
    ctx, H = setup(mp, kind, matsto, 3000)
    with ctx:
        gpar = np.zeros(H.nTotal)
        bs = batches(ctx.nVar, [4000, 20000], seed=9)
        ctx.loopbf(gpar)
        base = ctx.matrix()
        want = oracle_mupdat(orc, H, matsto, base, bs)
        for call in (ctx.mupdat, ctx.mupdat_noalloc):
            ctx.loopbf(gpar)
            for b in bs:
                call(*b)
            close(ctx.matrix(), want)
    if matsto == 2:
        # most random pairs fall outside the stored blocks and are dropped:
        # the matrix changed, but by fewer elements than there were triplets
        changed = int(np.count_nonzero(want != base))
        assert 0 < changed < sum(len(b[0]) for b in bs) // 2


def test_mupdat_on_pairentries_layout(mp, orc):
    """mpgpu_mupdat and mpgpu_mupdat_noalloc on a sparse layout with
    pairentries 2: elements of the left-out group pairs (pairs the records
    hold) are dropped as the oracle's mupdat drops them
    (pede.f90:3170-3173), the others land as there"""
    d = mp.generate(mp.gen_config("barrel", ntracks=3000, seed=17))
    H = mp.HostStructure(d, mreqenf=5, sparse=True, mreqpe=2)
    sup = H.suppressed
    assert len(sup) > 0
    first = H.aig[sup[:, 0] - 1]
    i = np.where(sup[:, 0] == sup[:, 1], first + 1, first).astype(np.int32)
    j = H.aig[sup[:, 1] - 1].astype(np.int32)
    left = (i, j, np.ones(len(i)))
    bs = [left] + batches(H.nVar, [20000], seed=5)
    with mp.Context() as ctx:
        ctx.set_layout(H, 2)
        ctx.upload(H)
        gpar = np.zeros(H.nTotal)
        ctx.loopbf(gpar)
        base = ctx.matrix()
        np.testing.assert_array_equal(oracle_mupdat(orc, H, 2, base, [left]), base)
        want = oracle_mupdat(orc, H, 2, base, bs)
        for call in (ctx.mupdat, ctx.mupdat_noalloc):
            ctx.loopbf(gpar)
            call(*left)
            np.testing.assert_array_equal(ctx.matrix(), base)
            for b in bs[1:]:
                call(*b)
            close(ctx.matrix(), want)
