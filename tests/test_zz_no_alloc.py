"""mpgpu_mupdat_noalloc (staging in a fixed device area, no allocation)
against mpgpu_mupdat through the C-ABI: the global matrix after a data loop
plus two update calls in a row agrees within 1e-12 relative (both run the
same kernel in the same order, so it is expected to be identical); a call
above the area's capacity is rejected and leaves the matrix unchanged."""
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
