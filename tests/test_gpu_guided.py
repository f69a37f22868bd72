"""The guided thermal sampler, through the C ABI.

The guide network (trained on the device from the FP32 POD sampler's own
CDF searches) predicts where ThermalScattering::SampleAlpha's find_cdf
bisection ends for each kinematic bound; the POD reconstructions confirm the
guess or walk from it.  So, for the same random numbers:

* at the sampler level (C4's incident energies 0.01, 0.1 and 1 eV, T uniform
  in 283.6-623.6 K per sample) the guided sampler returns exactly the FP32
  POD sampler's (beta, alpha), sample for sample;
* in transport (the thermal-scatter queue), the broomstick's histories are
  the ones the inline FP32 POD sampler gives: the same events and fate for
  every history and the same leakage tallies -- and the same again for the
  plain POD queue without the network;
* with independent seeds, at 1e7 histories per energy (C4's scale), the
  leakage energy and cosine spectra of the guided form pass a two-sample
  chi-square test against the POD form (p > 0.01), the gate the surrogate
  is held to; and at the sampler level, 1e7 scatters per energy with T
  uniform per sample, its outgoing beta and alpha histograms (200 bins)
  pass the same test against an independent exact-POD sample.
"""
import numpy as np
import pytest
from scipy import stats

from minimc_gb300 import (RNG_PHILOX, THERMAL_GUIDED, THERMAL_POD, THERMAL_POD_QUEUE, TSL_FAST, TSL_GUIDED,
                          TSL_PHILOX, TSL_POD, Context, synth_tsl)

pytestmark = pytest.mark.gpu
RESAMPLE = -6  # MC_ERR_RESAMPLE
EV = 1e-6
ENERGIES = [0.01 * EV, 0.1 * EV, 1.0 * EV]
P_MIN = 0.01  # chi-square gate on the leakage spectra
SUM_RTOL = 1e-12  # tallies of identical histories: summation order only


@pytest.fixture(scope="module")
def library(tmp_path_factory):
    d = tmp_path_factory.mktemp("tsl_guided")
    return d, synth_tsl.write_tsl(d), synth_tsl.moderator_nuclide(d)


def guided_ctx(library, energy=1.0 * EV, histories=10):
    d, tsl, nuc = library
    ctx = Context(0)
    ctx.load_xml(synth_tsl.broomstick_xml(tsl, nuc, histories=histories, energy=energy, temperature=450.0), d)
    out = ctx.train_surrogate_guide(0, E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=4096,
                                    samples_per_condition=512, batch=16384, steps=10000, lr=1e-3, seed=3)
    return ctx, out


@pytest.fixture(scope="module")
def ctx1(library):
    return guided_ctx(library)


def test_guide_training(ctx1):
    """The guide learns where the CDF search ends to about a grid cell:
    (nF + 1) = 161 cells span [0, 1]; an RMS error of two cells leaves the
    walk from the guess far shorter than the bisection's 8 probes."""
    _, out = ctx1
    assert out.failures == 0
    assert out.samples == 2 * 4096 * 512
    assert np.sqrt(out.loss_alpha) < 2.0 / 161, out.loss_alpha


@pytest.mark.parametrize("E", ENERGIES)
def test_guided_samples_are_the_pod_samples(ctx1, E):
    ctx, _ = ctx1
    n = 300_000
    T = np.random.default_rng(8).uniform(283.6, 623.6, n)
    gb, ga, gf = ctx.sample_tsl(0, np.full(n, E), T, seed=21, method=TSL_GUIDED | TSL_FAST)
    pb, pa, pf = ctx.sample_tsl(0, np.full(n, E), T, seed=21, method=TSL_POD | TSL_PHILOX | TSL_FAST)
    assert gf == pf
    assert np.array_equal(gb, pb, equal_nan=True)
    assert np.array_equal(ga, pa, equal_nan=True)


def test_guided_exact_form_samples_are_the_exact_pod_samples(ctx1):
    """The exact (FP64) POD form: the guide starts the same searches over
    its reconstructions, the samples are the exact POD sampler's, bit for
    bit, at C4's energies with T uniform per sample."""
    ctx, _ = ctx1
    n = 100_000
    rng = np.random.default_rng(12)
    E = np.asarray(ENERGIES)[rng.integers(0, 3, n)]
    T = rng.uniform(283.6, 623.6, n)
    gb, ga, gf = ctx.sample_tsl(0, E, T, seed=31, method=TSL_GUIDED)
    pb, pa, pf = ctx.sample_tsl(0, E, T, seed=31, method=TSL_POD | TSL_PHILOX)
    assert gf == pf
    assert np.array_equal(gb, pb, equal_nan=True) and np.array_equal(ga, pa, equal_nan=True)


def test_guided_samples_outside_the_trained_box(ctx1):
    """Outside the guide's (E, T) box the guesses are poorer, the samples
    are still the POD sampler's."""
    ctx, _ = ctx1
    n = 100_000
    E = np.full(n, 3.5e-6)
    T = np.full(n, 700.0)
    gb, ga, _ = ctx.sample_tsl(0, E, T, seed=4, method=TSL_GUIDED | TSL_FAST)
    pb, pa, _ = ctx.sample_tsl(0, E, T, seed=4, method=TSL_POD | TSL_PHILOX | TSL_FAST)
    assert np.array_equal(gb, pb, equal_nan=True) and np.array_equal(ga, pa, equal_nan=True)


def test_guided_transport_is_pod_transport(ctx1):
    """Same seed: every history of the broomstick has the same events and
    fate with the inline FP32 POD sampler, the guided queue and the plain
    POD queue; the tallies agree to summation order."""
    ctx, _ = ctx1
    n = 200_000
    kw = dict(rng=RNG_PHILOX, fast_math=1, histories=n, seed=5, per_history=True)
    pod = ctx.run_fixed_source(thermal=THERMAL_POD, **kw)
    gui = ctx.run_fixed_source(thermal=THERMAL_GUIDED, **kw)
    que = ctx.run_fixed_source(thermal=THERMAL_POD_QUEUE, **kw)
    for r in (gui, que):
        assert r.raw.lost == pod.raw.lost and r.raw.resample_failures == pod.raw.resample_failures
        assert np.array_equal(r.history_events, pod.history_events)
        assert np.array_equal(r.history_fate, pod.history_fate)
        np.testing.assert_allclose(r.sum, pod.sum, rtol=SUM_RTOL, atol=0)
        np.testing.assert_allclose(r.sum_sq, pod.sum_sq, rtol=SUM_RTOL, atol=0)
    # the queue served the scatters (sampler and resume launches)
    assert gui.raw.launches > pod.raw.launches


def test_guided_transport_exact_form_is_pod_transport(ctx1):
    """The exact (FP64) form throughout (fast_math off): the guided queue and
    the plain POD queue give every history the inline exact POD sampler's
    events and fate, tallies to summation order."""
    ctx, _ = ctx1
    n = 200_000
    kw = dict(rng=RNG_PHILOX, fast_math=0, histories=n, seed=7, per_history=True)
    pod = ctx.run_fixed_source(thermal=THERMAL_POD, **kw)
    gui = ctx.run_fixed_source(thermal=THERMAL_GUIDED, **kw)
    que = ctx.run_fixed_source(thermal=THERMAL_POD_QUEUE, **kw)
    for r in (gui, que):
        assert r.raw.lost == pod.raw.lost and r.raw.resample_failures == pod.raw.resample_failures
        assert np.array_equal(r.history_events, pod.history_events)
        assert np.array_equal(r.history_fate, pod.history_fate)
        np.testing.assert_allclose(r.sum, pod.sum, rtol=SUM_RTOL, atol=0)
    assert gui.raw.launches > pod.raw.launches


def spectra(ctx, r):
    """Leakage energy and cosine marginals (counts) of the broomstick tally."""
    e = ctx.estimators()[0]
    t = r.sum[e.offset:e.offset + e.n_bins].reshape(int(e.cosine_bins), int(e.energy_bins))
    return t.sum(0), t.sum(1)


def chi2_two_sample(a, b):
    """Two-sample chi-square of two histograms (bins with >= 10 counts in
    total; the samples' sizes may differ)."""
    keep = (a + b) >= 10
    a, b = a[keep], b[keep]
    ka, kb = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    chi2 = float(np.sum((ka * a - kb * b) ** 2 / (a + b)))
    dof = int(keep.sum()) - 1
    return chi2, dof, float(stats.chi2.sf(chi2, dof))


@pytest.mark.parametrize("E", ENERGIES)
def test_guided_spectra_pass_chi2_against_pod(library, E):
    """Independent seeds, 1e7 histories each: the guided form's leakage
    energy and cosine spectra against the inline POD form's."""
    ctx, _ = guided_ctx(library, energy=E)
    n = 10_000_000
    # at this scale SampleAlpha's resampling limit is reached about once in
    # 1e7 scatters (the reference throws there; the engine kills the
    # particle and reports MC_ERR_RESAMPLE with the count)
    kw = dict(rng=RNG_PHILOX, fast_math=1, histories=n, allow=(RESAMPLE,))
    pod = ctx.run_fixed_source(seed=101, thermal=THERMAL_POD, **kw)
    gui = ctx.run_fixed_source(seed=202, thermal=THERMAL_GUIDED, **kw)
    assert gui.raw.lost == 0
    assert gui.raw.resample_failures <= 10 and pod.raw.resample_failures <= 10
    for name, a, b in zip(("energy", "cosine"), spectra(ctx, gui), spectra(ctx, pod)):
        chi2, dof, p = chi2_two_sample(a, b)
        assert p > P_MIN, (E, name, chi2, dof, p)


@pytest.mark.parametrize("E", ENERGIES)
def test_c4_scale_beta_alpha_histograms(ctx1, E):
    """1e7 scatters at one incident energy, T uniform in 283.6-623.6 K per
    sample: 200-bin beta and alpha histograms (equiprobable edges from one
    exact-POD sample) of the exact guided sampler against an independent
    exact-POD sample."""
    ctx, _ = ctx1
    n = 10_000_000
    T = np.random.default_rng(19).uniform(283.6, 623.6, n)
    ref = ctx.sample_tsl(0, np.full(n, E), T, seed=101, method=TSL_POD | TSL_PHILOX)
    pod = ctx.sample_tsl(0, np.full(n, E), T, seed=202, method=TSL_POD | TSL_PHILOX)
    gui = ctx.sample_tsl(0, np.full(n, E), T, seed=303, method=TSL_GUIDED)
    assert gui[2] <= 10 and pod[2] <= 10  # failed resamples are NaN
    for v, name in ((0, "beta"), (1, "alpha")):
        ok = lambda x: x[~np.isnan(x)]
        edges = np.quantile(ok(ref[v]), np.linspace(0, 1, 201)[1:-1])
        a = np.bincount(np.searchsorted(edges, ok(gui[v])), minlength=200).astype(float)
        b = np.bincount(np.searchsorted(edges, ok(pod[v])), minlength=200).astype(float)
        chi2, dof, p = chi2_two_sample(a, b)
        assert dof >= 150 and p > P_MIN, (E, name, chi2, dof, p)


def test_guide_gains_over_the_bisection(ctx1):
    """What the trained network gains over the method without it: the exact
    (FP64) POD sampler with the guide starting its CDF searches against the
    same sampler bisecting them, on the same 2e6 (E, T) rows on the device
    -- the same samples (tested above), less time.  (In the FP32 form the
    bisection's reconstructions are cheap enough that the network's cost
    outweighs them; the bench line reports both forms.)"""
    torch = pytest.importorskip("torch")
    ctx, _ = ctx1
    n = 2_000_000
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    E = torch.tensor(ENERGIES, dtype=torch.float64, device="cuda")[torch.randint(0, 3, (n,), device="cuda",
                                                                                 generator=g)]
    T = 283.6 + 340.0 * torch.rand(n, dtype=torch.float64, device="cuda", generator=g)
    b = torch.empty_like(E)
    a = torch.empty_like(E)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    def ms(method):
        for _ in range(2):
            ctx.sample_tsl_device(0, E.data_ptr(), T.data_ptr(), n, b.data_ptr(), a.data_ptr(), seed=9, method=method)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(3):
            ctx.sample_tsl_device(0, E.data_ptr(), T.data_ptr(), n, b.data_ptr(), a.data_ptr(), seed=10 + i,
                                  method=method)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    pod, guided = ms(TSL_POD | TSL_PHILOX), ms(TSL_GUIDED)
    assert pod / guided > 1.05, (pod, guided)
