"""Serving loop through the C-ABI (mpgpu_server_*): jobs of different sizes
submitted together, run concurrently on one device; every job's result is
bit-identical to the same job run alone (mpgpu_pede_run), and a job larger
than the memory budget is refused with MPGPU_ERR_BUDGET (42)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def jobs(mp):
    out = []
    for k, (nmod, ntracks, metsol) in enumerate([(20, 3000, 1), (60, 12000, 31), (30, 6000, 3),
                                                 (100, 15000, 32), (40, 8000, 1)]):
        cfg = mp.gen_config("telescope", ntracks=ntracks, seed=100 + k)
        cfg.nmod = nmod
        d = mp.generate(cfg)
        out.append((d, dict(metsol=metsol, matsto=1, mitera=2, mreqenf=5)))
    return out


def test_serve_matches_alone(mp):
    specs = jobs(mp)
    alone = []
    for d, st in specs:
        jd = mp.JobData(d, **st)
        assert mp.run_job(jd) == 0
        alone.append(jd.parameters())
    with mp.Server(max_active=3) as srv:
        jds = [mp.JobData(d, **st) for d, st in specs]
        tickets = [srv.submit(jd) for jd in jds]
        res = [srv.wait(t, timeout_ms=600000.0) for t in tickets]
    for (rc, lat, q, b), jd, (lab, par) in zip(res, jds, alone):
        assert rc == 0
        assert lat > 0 and b > 0
        l2, p2 = jd.parameters()
        np.testing.assert_array_equal(l2, lab)
        np.testing.assert_array_equal(p2, par)


def test_serve_budget_refusal(mp):
    d, st = jobs(mp)[1]
    with mp.Server(max_active=1, budget_bytes=1 << 20) as srv:
        jd = mp.JobData(d, **st)
        rc, lat, q, b = srv.wait(srv.submit(jd), timeout_ms=600000.0)
    assert rc == 42
    assert b > (1 << 20)


def test_serve_mixed_matches_fp64(mp):
    """Every job solved with the tensor-core factor (metsol 31) in the mix
    of the serving loop reaches the parameters of the same job solved with
    the FP64 factor (metsol 32): within 1e-10 relative for one solution
    (the CG refinement stops on the size of its corrections, not on the
    residual alone).  Over three Gauss-Newton iterations each new gradient
    is formed from parameters that differ in their last bits, and the
    solution amplifies that rounding noise by the condition number: there
    the two FP64 forms (blocked, metsol 32, and chdec2, metsol 3) differ by
    about 1e-10 as well, and the mixed form stays within that spread."""
    specs = jobs(mp)
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    for mitera in (1, 3):
        forms = {}
        with mp.Server(max_active=3) as srv:
            for ms in (31, 32, 3):
                forms[ms] = [mp.JobData(d, **dict(st, metsol=ms, mitera=mitera)) for d, st in specs]
            tickets = [srv.submit(jd) for ms in (31, 32, 3) for jd in forms[ms]]
            res = [srv.wait(t, timeout_ms=600000.0) for t in tickets]
        assert all(r[0] == 0 for r in res)
        for a, b, c in zip(forms[31], forms[32], forms[3]):
            np.testing.assert_array_equal(a.parameters()[0], b.parameters()[0])
            mixed = rel(a.parameters()[1], b.parameters()[1])
            spread = rel(b.parameters()[1], c.parameters()[1])
            if mitera == 1:
                assert mixed <= 1e-10, mixed
            else:
                assert mixed <= max(1e-10, 4.0 * spread), (mixed, spread)
            assert a.res.minresItn > 0 and b.res.minresItn > 0
