"""GPU thermal scattering parity, through the C ABI.

* ThermalScattering::GetTotal bit-exact against the oracle.
* The sampler with reference streams (minstd seeded seed + i) and the exact
  FP64 POD form: beta and alpha identical to the oracle's, sample by sample.
* Philox streams, exact and FP32 POD forms: two-sample KS tests against
  the oracle at fixed (E, T), and 200-bin beta / alpha histograms with T
  uniform in 283.6-623.6 K per sample (chi-square).
* Broomstick transport: with reference streams the leakage tallies equal the
  oracle's; with Philox and the FP32 form, a chi-square test.
"""
import numpy as np
import pytest
from scipy import stats

from minimc_gb300 import RNG_MINSTD, RNG_PHILOX, TSL_FAST, TSL_PHILOX, TSL_POD, Context, synth_tsl
from oracle.build import Oracle

pytestmark = pytest.mark.gpu
EV = 1e-6


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("tsl")
    tsl = synth_tsl.write_tsl(d)
    nuc = synth_tsl.moderator_nuclide(d)
    return d, tsl, nuc


def ctx_and_oracle(lib, **kw):
    d, tsl, nuc = lib
    xml = synth_tsl.broomstick_xml(tsl, nuc, **kw)
    g = Context(0)
    g.load_xml(xml, d)
    return g, Oracle(xml, d), xml


def test_tsl_total_bit_exact(lib, built_library):
    g, o, _ = ctx_and_oracle(lib, histories=10)
    rng = np.random.default_rng(1)
    E = np.exp(rng.uniform(np.log(1e-11), np.log(4e-6), 20_000))
    T = rng.uniform(200.0, 700.0, 20_000)
    np.testing.assert_array_equal(g.tsl_total(0, E, T), o.tsl_total(0, E, T))


def test_sampler_reference_streams_identical(lib, built_library):
    g, o, _ = ctx_and_oracle(lib, histories=10)
    rng = np.random.default_rng(2)
    n = 50_000
    E = np.exp(rng.uniform(np.log(1e-9), np.log(3e-6), n))
    T = rng.uniform(283.6, 623.6, n)
    gb, ga, gf = g.sample_tsl(0, E, T, seed=7, method=TSL_POD)
    ob_, oa, of = o.sample_tsl(0, E, T, seed=7)
    assert gf == of
    np.testing.assert_array_equal(gb, ob_)
    np.testing.assert_array_equal(ga, oa)


@pytest.mark.parametrize("flags", [TSL_PHILOX, TSL_PHILOX | TSL_FAST])
def test_sampler_philox_ks(lib, flags, built_library):
    g, o, _ = ctx_and_oracle(lib, histories=10)
    n = 100_000
    for E, T in ((0.01 * EV, 300.0), (0.1 * EV, 450.0), (1.0 * EV, 600.0)):
        gb, ga, gf = g.sample_tsl(0, np.full(n, E), T, seed=3, method=TSL_POD | flags)
        ob_, oa, of = o.sample_tsl(0, np.full(n, E), T, seed=3)
        assert gf == 0 and of == 0
        assert stats.ks_2samp(gb, ob_).pvalue > 1e-3, (E, T, flags)
        assert stats.ks_2samp(ga, oa).pvalue > 1e-3, (E, T, flags)


def _hist_chi2(a, b, bins):
    ha, _ = np.histogram(a, bins)
    hb, _ = np.histogram(b, bins)
    keep = (ha + hb) >= 10
    return stats.chi2_contingency(np.vstack([ha[keep], hb[keep]]))[1]


@pytest.mark.parametrize("E", [0.01 * EV, 0.1 * EV, 1.0 * EV])
def test_sampler_continuous_temperature_histograms(lib, E, built_library):
    """T uniform in 283.6-623.6 K per sample; 200-bin beta and alpha
    histograms, FP32 POD form against the oracle."""
    g, o, _ = ctx_and_oracle(lib, histories=10)
    n = 400_000
    T = np.random.default_rng(9).uniform(283.6, 623.6, n)
    gb, ga, _ = g.sample_tsl(0, np.full(n, E), T, seed=5, method=TSL_POD | TSL_PHILOX | TSL_FAST)
    ob_, oa, _ = o.sample_tsl(0, np.full(n, E), T, seed=5)
    bb = np.linspace(min(gb.min(), ob_.min()), max(gb.max(), ob_.max()), 201)
    ab = np.linspace(0, max(ga.max(), oa.max()), 201)
    assert _hist_chi2(gb, ob_, bb) > 1e-3
    assert _hist_chi2(ga, oa, ab) > 1e-3


def test_broomstick_reference_streams_identical(lib, built_library):
    n = 20_000
    g, o, _ = ctx_and_oracle(lib, histories=n, energy=0.1 * EV, temperature=450.0)
    r = g.run_fixed_source(rng=RNG_MINSTD, per_history=True, histories=n)
    ro = o.run_fixed_source(n, 1, threads=8, per_history=True)
    assert np.array_equal(r.history_events, ro["history_events"])
    assert np.array_equal(r.sum, ro["sum"])


def test_broomstick_philox_fast_chi2(lib, built_library):
    n = 200_000
    g, o, _ = ctx_and_oracle(lib, histories=n, energy=1.0 * EV, temperature=450.0, cosine_bins=20, energy_bins=40)
    r = g.run_fixed_source(rng=RNG_PHILOX, fast_math=1, histories=n)
    ro = o.run_fixed_source(n, 1, threads=8)
    a, b = r.sum, ro["sum"]
    keep = (a + b) >= 20
    p = stats.chi2_contingency(np.vstack([a[keep], b[keep]]))[1]
    assert p > 1e-3, p


def test_continuous_temperature_delta_tracking(lib, built_library):
    """The reference's continuous-temperature benchmark shape (oracle pinned
    on the reference by tests/test_reference_cpu.py): cell delta tracking
    with the thermal library's majorant (ThermalScattering::GetMajorant,
    src/ThermalScattering.cpp:106-109), real/virtual rejection at the local
    temperature of a linear 300-600 K field, POD thermal scattering.  With
    reference streams the GPU's histories are the oracle's: the same events
    and fate for at least 99.9 % of histories (the last bits of the CUDA and
    C library erf/exp in the majorant and total may move a rejection), the
    same leakage within 0.2 %."""
    d, tsl, nuc = lib
    n = 20_000
    xml = synth_tsl.continuous_temperature_slab_xml(tsl, nuc, histories=n, thickness=1.0)
    g = Context(0)
    g.load_xml(xml, d)
    r = g.run_fixed_source(rng=RNG_MINSTD, per_history=True, histories=n)
    ro = Oracle(xml, d).run_fixed_source(n, 1, threads=8, per_history=True)
    assert r.raw.lost == 0 and r.raw.resample_failures == ro["resample"]
    assert r.raw.events > 3 * n  # virtual and real collisions, crossings
    agree = np.mean((r.history_events == ro["history_events"]) & (r.history_fate == ro["history_fate"]))
    assert agree > 0.999, agree
    assert abs(r.sum.sum() - ro["sum"].sum()) <= 0.002 * n


def test_continuous_temperature_philox_chi2(lib, built_library):
    """The same problem with Philox streams and the FP32 forms (the
    engine's fast path) against the oracle: leakage spectrum chi-square."""
    d, tsl, nuc = lib
    n = 200_000
    xml = synth_tsl.continuous_temperature_slab_xml(tsl, nuc, histories=n, thickness=1.0, energy_bins=40)
    g = Context(0)
    g.load_xml(xml, d)
    r = g.run_fixed_source(rng=RNG_PHILOX, fast_math=1, histories=n)
    ro = Oracle(xml, d).run_fixed_source(n, 1, threads=8)
    a, b = r.sum, ro["sum"]
    keep = (a + b) >= 20
    p = stats.chi2_contingency(np.vstack([a[keep], b[keep]]))[1]
    assert p > 1e-3, p


def test_pod_pipeline_library(lib, tmp_path, built_library):
    """A library built by the POD pipeline (adaptive ranks at a 1e-4
    relative Frobenius tolerance, decomposed on the GPU, non-monotone CDFs
    removed) samples the same law as the fixed-rank-30 library: KS distances
    at C4's energies within two-sample noise of 2e5 samples."""
    d, tsl, nuc = lib
    ad = tmp_path / "adaptive"
    tsl2 = synth_tsl.write_tsl(ad, rel_tol=1e-4, device=None)
    nuc2 = synth_tsl.moderator_nuclide(ad)
    g1 = Context(0)
    g1.load_xml(synth_tsl.broomstick_xml(tsl, nuc, histories=10), d)
    g2 = Context(0)
    g2.load_xml(synth_tsl.broomstick_xml(tsl2, nuc2, histories=10), ad)
    n = 200_000
    for E in (0.01 * EV, 0.1 * EV, 1.0 * EV):
        T = np.random.default_rng(5).uniform(283.6, 623.6, n)
        b1, a1, f1 = g1.sample_tsl(0, np.full(n, E), T, seed=1, method=TSL_POD | TSL_PHILOX)
        b2, a2, f2 = g2.sample_tsl(0, np.full(n, E), T, seed=2, method=TSL_POD | TSL_PHILOX)
        assert f1 == 0 and f2 == 0
        assert stats.ks_2samp(b1, b2).pvalue > 1e-3
        assert stats.ks_2samp(a1, a2).pvalue > 1e-3
