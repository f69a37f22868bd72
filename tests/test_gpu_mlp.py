"""GPU MLP surrogate of the thermal scattering sampler, through the C ABI.

* Forward outputs and the full parameter gradient of one training step
  (tcgen05 products with FP32 accumulation: FP16 forward operands and
  packed-FP16 hidden SiLU, BF16 backward operands) against a CPU reference
  that applies the same roundings in FP64 arithmetic, and against plain
  FP64 (loose tolerance).
* Training on POD samples of the synthetic library, then sampling: beta and
  alpha distributions against the POD sampler (KS distance, 200-bin
  chi-square at C4's energies with T uniform per sample), the fallback
  outside the trained box, and the speed against the POD GPU forms.
"""
import math
import time

import numpy as np
import pytest
from scipy import stats

from minimc_gb300 import (MLP_PARAMS, RNG_PHILOX, THERMAL_SURROGATE, TSL_FAST, TSL_MLP, TSL_PHILOX, TSL_POD, Context,
                          synth_tsl)

pytestmark = pytest.mark.gpu
EV = 1e-6

W, IN = 128, 16
OFF = {"W1": 0, "b1": W * IN, "W2": W * IN + W, "b2": W * IN + W + W * W, "W3": W * IN + 2 * W + W * W,
       "b3": W * IN + 2 * W + 2 * W * W, "w4": W * IN + 3 * W + 2 * W * W, "b4": W * IN + 4 * W + 2 * W * W}


def bf16(a):
    """Round float32 values to BF16 (nearest even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF["W1"]:OFF["b1"]].reshape(W, IN), p[OFF["b1"]:OFF["W2"]], p[OFF["W2"]:OFF["b2"]].reshape(W, W),
            p[OFF["b2"]:OFF["W3"]], p[OFF["W3"]:OFF["b3"]].reshape(W, W), p[OFF["b3"]:OFF["w4"]],
            p[OFF["w4"]:OFF["b4"]], p[OFF["b4"]])


def silu(z):
    return z / (1 + np.exp(-z))


def f16(a):
    """Round to FP16 (nearest even), returned as float64."""
    return np.asarray(a, np.float64).astype(np.float16).astype(np.float64)


def silu_f16(z):
    """Hidden activations as the kernels form them: h = f16(z / 2), then the
    packed FP16 tanh and fma h + h tanh(h), rounded to FP16."""
    h = f16(np.asarray(z) / 2)
    t = f16(np.tanh(h))
    return f16(h + h * t)


def dsilu(z):
    s = 1 / (1 + np.exp(-z))
    return s * (1 + z * (1 - s))


def reference(p, x, y, emulate=True):
    """Forward and backward of the network; `emulate` applies the kernel's
    roundings: FP16 operands of the forward products, BF16 operands of the
    backward products."""
    ident = lambda a: np.asarray(a, np.float64)  # noqa: E731
    q = bf16 if emulate else ident
    h16 = f16 if emulate else ident
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p)
    n = len(x)
    X = h16(x)
    act = silu_f16 if emulate else silu
    Z1 = X @ h16(W1).T + b1
    H1 = act(Z1)
    Z2 = H1 @ h16(W2).T + b2
    H2 = act(Z2)
    Z3 = H2 @ h16(W3).T + b3
    out = silu(Z3) @ w4 + b4
    e = out - y
    go = 2 * e / n
    g = np.zeros(len(p))
    g[OFF["w4"]:OFF["b4"]] = go @ silu(Z3)
    g[OFF["b4"]] = go.sum()
    dZ3 = go[:, None] * w4[None, :] * dsilu(Z3)
    g[OFF["b3"]:OFF["w4"]] = dZ3.sum(0)
    g[OFF["W3"]:OFF["b3"]] = (q(dZ3).T @ q(H2)).ravel()
    dZ2 = (q(dZ3) @ q(W3)) * dsilu(Z2)
    g[OFF["b2"]:OFF["W3"]] = dZ2.sum(0)
    g[OFF["W2"]:OFF["b2"]] = (q(dZ2).T @ q(H1)).ravel()
    dZ1 = (q(dZ2) @ q(W2)) * dsilu(Z1)
    g[OFF["b1"]:OFF["W2"]] = dZ1.sum(0)
    g[OFF["W1"]:OFF["b1"]] = (q(dZ1).T @ q(X)).ravel()
    return g, float((e * e).sum()), out


def random_case(n, seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(MLP_PARAMS, np.float32)
    p[OFF["W1"]:OFF["b1"]] = (rng.uniform(-0.5, 0.5, (W, IN)) * (np.arange(IN) < 6)).ravel()
    for k, a in (("b1", 0.5), ("b2", 0.09), ("b3", 0.09), ("w4", 0.09)):
        n_ = {"b1": W, "b2": W, "b3": W, "w4": W}[k]
        p[OFF[k]:OFF[k] + n_] = rng.uniform(-a, a, n_)
    p[OFF["W2"]:OFF["b2"]] = rng.uniform(-0.09, 0.09, W * W)
    p[OFF["W3"]:OFF["b3"]] = rng.uniform(-0.09, 0.09, W * W)
    p[OFF["b4"]] = 0.3
    x = np.zeros((n, IN), np.float32)
    x[:, :6] = rng.uniform(-1, 1, (n, 6))
    y = rng.uniform(0, 1, n).astype(np.float32)
    return p, x, y


@pytest.mark.parametrize("n", [128, 1024, 8192])
def test_gradient_matches_cpu_reference(n, built_library):
    p, x, y = random_case(n, seed=n)
    g, loss, out = Context(0).surrogate_grad(p, x, y)
    ge, le, oe = reference(p, x, y, emulate=True)
    np.testing.assert_allclose(out, oe, rtol=2e-3, atol=2e-4)
    assert abs(loss - le) <= 2e-3 * le
    for name, (a, b) in {"W1": (OFF["W1"], OFF["b1"]), "b1": (OFF["b1"], OFF["W2"]), "W2": (OFF["W2"], OFF["b2"]),
                         "b2": (OFF["b2"], OFF["W3"]), "W3": (OFF["W3"], OFF["b3"]), "b3": (OFF["b3"], OFF["w4"]),
                         "w4": (OFF["w4"], OFF["b4"]), "b4": (OFF["b4"], OFF["b4"] + 1)}.items():
        scale = np.abs(ge[a:b]).max() + 1e-12
        err = np.abs(g[a:b] - ge[a:b]).max() / scale
        assert err < 1e-2, (name, err)
    # and against FP64 without BF16 roundings: the same gradient to BF16 accuracy
    gf, _, _ = reference(p, x, y, emulate=False)
    cos = float(g @ gf / (np.linalg.norm(g) * np.linalg.norm(gf)))
    assert cos > 0.999, cos


@pytest.fixture(scope="module")
def trained(tmp_path_factory):
    d = tmp_path_factory.mktemp("tsl")
    tsl = synth_tsl.write_tsl(d)
    nuc = synth_tsl.moderator_nuclide(d)
    xml = synth_tsl.broomstick_xml(tsl, nuc, histories=10)
    ctx = Context(0)
    ctx.load_xml(xml, d)
    t0 = time.perf_counter()
    out = ctx.train_surrogate(0, E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=8192,
                              samples_per_condition=1024, batch=16384, steps=8000, lr=1e-3, seed=3)
    return ctx, out, time.perf_counter() - t0


def test_training_converges(trained):
    """The mean squared quantile error reaches the noise of the targets
    themselves: an empirical quantile of K samples scatters by about
    sqrt(u (1 - u) / K) in CDF units (~2.4e-4 squared for K = 1024)."""
    ctx, out, wall = trained
    assert out.failures == 0
    assert out.loss_beta < 1e-3 and out.loss_alpha < 1e-3, (out.loss_beta, out.loss_alpha)
    assert out.samples == 8192 * 1024


@pytest.mark.parametrize("E", [0.01 * EV, 0.1 * EV, 1.0 * EV])
def test_surrogate_matches_pod(trained, E):
    """C4's incident energies, T uniform in 283.6-623.6 K per sample: the
    surrogate's beta and alpha distributions against the POD sampler's."""
    ctx, _, _ = trained
    n = 200_000
    T = np.random.default_rng(4).uniform(283.6, 623.6, n)
    mb, ma, mf = ctx.sample_tsl(0, np.full(n, E), T, seed=1, method=TSL_MLP)
    pb, pa, pf = ctx.sample_tsl(0, np.full(n, E), T, seed=2, method=TSL_POD | TSL_PHILOX)
    assert mf == 0 and pf == 0
    ks_b = stats.ks_2samp(mb, pb).statistic
    ks_a = stats.ks_2samp(ma, pa).statistic
    assert ks_b < 0.02 and ks_a < 0.02, (ks_b, ks_a)


def test_fallback_outside_box(trained):
    ctx, _, _ = trained
    n = 100_000
    E = np.full(n, 3e-6)  # above the trained box, below the library's cutoff
    mb, ma, _ = ctx.sample_tsl(0, E, 450.0, seed=1, method=TSL_MLP)
    pb, pa, _ = ctx.sample_tsl(0, E, 450.0, seed=5, method=TSL_POD | TSL_PHILOX)
    assert stats.ks_2samp(mb, pb).pvalue > 1e-3
    assert stats.ks_2samp(ma, pa).pvalue > 1e-3


def spectra(ctx, r):
    """Leakage energy and cosine marginals (counts) of the broomstick tally."""
    e = ctx.estimators()[0]
    t = r.sum[e.offset:e.offset + e.n_bins].reshape(int(e.cosine_bins), int(e.energy_bins))
    return t.sum(0), t.sum(1)


def test_surrogate_in_transport(trained):
    """Thermal-scatter queue: the broomstick transported with the surrogate
    sampler (parked particles, one tensor-core launch per round) against the
    POD sampler inside the history kernel: the same events per history, no
    lost particles, and leakage energy / cosine spectra within 0.02 in CDF."""
    ctx, _, _ = trained
    n = 400_000
    pod = ctx.run_fixed_source(rng=RNG_PHILOX, histories=n, seed=5)
    sur = ctx.run_fixed_source(rng=RNG_PHILOX, histories=n, seed=6, thermal=THERMAL_SURROGATE)
    assert sur.raw.lost == 0 and sur.raw.resample_failures == 0 and sur.raw.capped == 0
    assert abs(sur.raw.events / n - pod.raw.events / n) < 0.02
    # leakage probability (most histories leak once after one scatter)
    ls, lp = sur.sum.sum() / n, pod.sum.sum() / n
    assert abs(ls - lp) < 5 * math.sqrt(2 * lp * (1 - lp) / n) + 1e-6, (ls, lp)
    for a, b in zip(spectra(ctx, sur), spectra(ctx, pod)):
        d = np.abs(np.cumsum(a) / a.sum() - np.cumsum(b) / b.sum()).max()
        assert d < 0.02, d
    # the queue really served the scatters: more launches than the POD form
    assert sur.raw.launches > pod.raw.launches


def test_surrogate_transport_reproducible(trained):
    ctx, _, _ = trained
    a = ctx.run_fixed_source(rng=RNG_PHILOX, histories=50_000, seed=9, thermal=THERMAL_SURROGATE)
    b = ctx.run_fixed_source(rng=RNG_PHILOX, histories=50_000, seed=9, thermal=THERMAL_SURROGATE)
    assert np.array_equal(a.sum, b.sum) and a.raw.events == b.raw.events
