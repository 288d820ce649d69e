"""Dense blocked Cholesky through the C-ABI (mpgpu_dense_cholesky) against
numpy on seeded SPD matrices (up to n = 2,100: five block columns, the
last one ragged): FP64 form within 1e-12 relative of numpy's
factor; tensor-core 3xTF32 form within 1e-4 relative (its trailing updates
are products of TF32 pairs accumulated in FP32 over a block column of up to
512 columns, then subtracted from the FP64 matrix)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def spd(n, seed, cond=1e4):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    ev = np.geomspace(1.0, 1.0 / cond, n)
    return (Q * ev) @ Q.T


@pytest.mark.parametrize("n", [128, 200, 640, 2100])
@pytest.mark.parametrize("mode,tol", [(0, 1e-12), (1, 1e-4)])
def test_dense_cholesky(mp, n, mode, tol):
    A = spd(n, n)
    ref = np.linalg.cholesky(A)
    with mp.Context() as ctx:
        L, ms = ctx.dense_cholesky(A, mode)
    err = np.max(np.abs(L - ref)) / np.max(np.abs(ref))
    assert err <= tol, err
    assert ms > 0
