"""The POD table pipeline (minimc_gb300.pod): split, truncate, removal of
non-monotone CDFs, adaptive coarsening to a Frobenius tolerance, and the
partition files the engine reads."""
import numpy as np
import pytest

from minimc_gb300 import pod, synth_tsl


def table(n_F=30, n_g=24, n_T=5, seed=0):
    """A smooth family of increasing inverse CDFs: values[F][g][T]."""
    rng = np.random.default_rng(seed)
    F = synth_tsl.cdf_grid(n_F)
    g = np.linspace(1.0, 3.0, n_g)
    T = np.linspace(300.0, 600.0, n_T)
    a = rng.uniform(0.5, 1.5, (n_g, n_T))
    vals = np.log(F / (1 - F))[:, None, None] * a[None] * (g[:, None] / 3)[None] + g[None, :, None]
    return pod.Table(F, g, T, vals)


def test_split():
    t = table()
    parts = pod.split(t, [5, 11, 20])
    assert [len(p.outer) for p in parts] == [5, 6, 9, 4]
    assert np.array_equal(np.concatenate([p.outer for p in parts]), t.outer)
    assert np.array_equal(np.concatenate([p.values for p in parts], axis=1), t.values)
    with pytest.raises(ValueError):
        pod.split(t, [5, 5])


@pytest.mark.parametrize("device", ["numpy"])
def test_truncate_exact_and_tail(device):
    t = table()
    full = pod.truncate(t, 10**6, device)
    np.testing.assert_allclose(full.reconstruct(), t.values, rtol=0, atol=1e-10)
    for r in (1, 2, 4):
        p = pod.truncate(t, r, device)
        err = np.linalg.norm(p.reconstruct() - t.values) / np.linalg.norm(t.values)
        assert abs(err - p.rel_frobenius_error()) < 1e-10 * max(1.0, err) + 1e-12
        assert p.rank == r


def test_rank_for_tolerance():
    S = np.array([10.0, 1.0, 0.1, 0.01])
    tot = np.sum(S ** 2)
    for r in range(1, 5):
        tail = np.sqrt(np.sum(S[r:] ** 2) / tot)
        assert pod.rank_for_tolerance(S, tail * (1 + 1e-9)) <= r
        if r > 1:
            assert pod.rank_for_tolerance(S, np.sqrt(np.sum(S[r - 1:] ** 2) / tot) * 0.999) >= r


def test_remove_nonmonotonic_cdfs():
    t = table()
    # one outer point whose inverse CDF dips: it goes, the rest stay
    t.values[10:12, 7, 2] -= 5.0
    full = pod.truncate(t, 10**6, "numpy")
    kept = pod.remove_nonmonotonic_cdfs(full)
    assert 7 not in [int(i) for i in np.searchsorted(t.outer, kept.outer)]
    assert len(kept.outer) == len(t.outer) - 1
    assert (np.diff(kept.reconstruct(), axis=0) >= 0).all()
    clean = pod.truncate(table(), 10**6, "numpy")
    assert len(pod.remove_nonmonotonic_cdfs(clean).outer) == len(clean.outer)


def test_adaptive_coarsen_meets_tolerance():
    t = table(n_g=40)
    parts = pod.split(t, [10, 25])
    full = pod.full_decompositions(parts, "numpy")
    prev_ranks = None
    for tol in (1e-2, 1e-3, 1e-5):
        pods = pod.adaptive_coarsen(parts, full, rel_frobenius_norm_tol=tol, device="numpy")
        ranks = [p.rank for p in pods]
        for p, part in zip(pods, parts):
            assert p.rel_frobenius_error() <= tol
            assert (np.diff(p.reconstruct(), axis=0) >= 0).all()
            if p.rank > 1:  # the least rank: one mode fewer misses the tolerance
                q = pod.Pod(p.F, p.outer, p.T, p.cdf[:, :-1], p.S[:-1], p.outer_T[:, :, :-1], p.full_S)
                assert q.rel_frobenius_error() > tol
        if prev_ranks is not None:
            assert all(a >= b for a, b in zip(ranks, prev_ranks))
        prev_ranks = ranks


def test_pipeline_library_loads(tmp_path, built_library):
    """A library written by the pipeline (adaptive ranks) is read by the
    engine's loader like the fixed-rank one."""
    from minimc_gb300.engine import format_output

    tsl = synth_tsl.write_tsl(tmp_path, n_E=16, n_beta_grid=40, n_F_beta=40, n_F_alpha=40,
                              temperatures=np.linspace(283.6, 623.6, 4), rel_tol=1e-3, device="numpy")
    nuc = synth_tsl.moderator_nuclide(tmp_path)
    xml = synth_tsl.broomstick_xml(tsl, nuc, histories=10, cosine_bins=4, energy_bins=4)
    text = format_output(xml, tmp_path, np.zeros(36), np.zeros(36), 10)
    assert text.startswith("10\n")


def test_svd_device_choice(monkeypatch):
    """Without a GPU the pipeline decomposes with LAPACK; an unknown device
    name is refused; "cuda" goes to the project's device kernel."""
    t = table()
    monkeypatch.setattr(pod, "_gpu_present", lambda: False)
    U, S, Vh = pod._svd(t.matrix(), None)
    np.testing.assert_allclose((U * S) @ Vh, t.matrix(), rtol=0, atol=1e-10)
    with pytest.raises(ValueError, match="unknown SVD device"):
        pod._svd(t.matrix(), "cpu")
    called = {}

    def fake(M):
        called["shape"] = M.shape
        return np.linalg.svd(M, full_matrices=False)

    monkeypatch.setattr(pod, "_device_svd", fake)
    pod.truncate(t, 3, "cuda")
    assert called["shape"] == t.matrix().shape
