"""The POD table pipeline's decomposition on the device (mc_pod_svd, the
one-sided Jacobi SVD in FP64) against LAPACK on the same matrices: singular
values, reconstruction and orthonormality to FP64 accuracy, for tall, wide,
square, rank-deficient and graded matrices, and the pipeline's truncations
through both."""
import numpy as np
import pytest

from minimc_gb300 import Context, pod
from minimc_gb300.engine import MCError

pytestmark = pytest.mark.gpu


def graded(m, n, cond, seed):
    rng = np.random.default_rng(seed)
    Q1, _ = np.linalg.qr(rng.standard_normal((m, min(m, n))))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, min(m, n))))
    s = np.logspace(0, -np.log10(cond), min(m, n))
    return (Q1 * s) @ Q2.T


CASES = {
    "tall": lambda: np.random.default_rng(1).standard_normal((400, 120)),
    "wide": lambda: np.random.default_rng(2).standard_normal((30, 500)),
    "square": lambda: np.random.default_rng(3).standard_normal((64, 64)),
    "column": lambda: np.random.default_rng(4).standard_normal((50, 1)),
    "row": lambda: np.random.default_rng(5).standard_normal((1, 50)),
    "odd": lambda: np.random.default_rng(6).standard_normal((41, 17)),
    "rank7": lambda: np.random.default_rng(7).standard_normal((100, 7)) @ np.random.default_rng(8).standard_normal(
        (7, 40)),
    "graded": lambda: graded(200, 60, 1e12, 9),
    "zero_column": lambda: np.hstack([np.random.default_rng(10).standard_normal((20, 5)), np.zeros((20, 1))]),
}


@pytest.fixture(scope="module")
def ctx(built_library):
    return Context(0)


@pytest.mark.parametrize("name", sorted(CASES))
def test_svd_matches_lapack(ctx, name):
    M = CASES[name]()
    U, S, Vh, sweeps = ctx.pod_svd(M)
    k = min(M.shape)
    assert U.shape == (M.shape[0], k) and S.shape == (k,) and Vh.shape == (k, M.shape[1])
    S_ref = np.linalg.svd(M, compute_uv=False)
    smax = S_ref[0]
    assert np.all(np.diff(S) <= 0)
    np.testing.assert_allclose(S, S_ref, rtol=0, atol=1e-12 * smax)
    np.testing.assert_allclose((U * S) @ Vh, M, rtol=0, atol=1e-12 * smax)
    # right vectors orthonormal; left vectors orthonormal where S > 0
    np.testing.assert_allclose(Vh @ Vh.T, np.eye(k), rtol=0, atol=1e-12)
    live = S > 1e-9 * smax
    Ul = U[:, live]
    np.testing.assert_allclose(Ul.T @ Ul, np.eye(int(live.sum())), rtol=0, atol=1e-10)
    assert 1 <= sweeps < 60


def test_truncate_on_the_device_equals_lapack(ctx):
    rng = np.random.default_rng(12)
    F = np.linspace(0.01, 0.99, 30)
    g = np.linspace(1.0, 3.0, 24)
    T = np.linspace(300.0, 600.0, 5)
    a = rng.uniform(0.5, 1.5, (24, 5))
    vals = np.log(F / (1 - F))[:, None, None] * a[None] * (g[:, None] / 3)[None] + g[None, :, None]
    t = pod.Table(F, g, T, vals)
    for r in (1, 3, 10, 10**6):
        pd = pod.truncate(t, r, "cuda")
        pn = pod.truncate(t, r, "numpy")
        assert pd.rank == pn.rank
        np.testing.assert_allclose(pd.S, pn.S, rtol=0, atol=1e-12 * pn.S[0])
        np.testing.assert_allclose(pd.full_S, pn.full_S, rtol=0, atol=1e-12 * pn.S[0])
        np.testing.assert_allclose(pd.reconstruct(), pn.reconstruct(), rtol=0, atol=1e-11 * np.abs(vals).max())
        assert abs(pd.rel_frobenius_error() - pn.rel_frobenius_error()) < 1e-10


def test_svd_rejects_bad_input(ctx):
    with pytest.raises(MCError, match="non-finite"):
        ctx.pod_svd(np.array([[1.0, np.nan], [0.0, 1.0]]))
