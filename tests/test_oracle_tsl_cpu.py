"""CPU tests of the oracle's thermal scattering sampler
(ThermalScattering, src/ThermalScattering.cpp) on the synthetic POD library:
the reconstruction against the analytic law it was built from, kinematic
bounds, the direction of energy transfer, the inelastic total, and a
broomstick run (no GPU needed)."""
import math

import numpy as np
import pytest
from scipy import stats

from minimc_gb300 import synth_tsl
from oracle.build import Oracle

KB = 8.617333262145e-11


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("tsl")
    tsl = synth_tsl.write_tsl(d)
    nuc = synth_tsl.moderator_nuclide(d)
    xml = synth_tsl.broomstick_xml(tsl, nuc, histories=20_000)
    return d, tsl, Oracle(xml, d)


def test_beta_marginal_matches_analytic_law(lib):
    """At a tabulated (E, T) the POD sampler reproduces the beta marginal of
    the analytic law (KS distance within sampling noise plus the histogram
    interpolation between CDF points)."""
    d, tsl, o = lib
    E, T = tsl["Es"][70], tsl["Ts"][5]
    b, _, f = o.sample_tsl(0, np.full(50_000, E), T, seed=11)
    assert f == 0
    grid, cdf, tot = synth_tsl.beta_marginal_cdf(E, T, tsl["awr"], tsl["beta_cutoff"])
    ks = stats.kstest(b, lambda x: np.interp(x, grid, cdf / tot))
    assert ks.statistic < 0.01, ks


def test_kinematic_bounds(lib):
    d, tsl, o = lib
    rng = np.random.default_rng(3)
    E = np.exp(rng.uniform(np.log(1e-9), np.log(3e-6), 50_000))
    T = rng.uniform(283.6, 623.6, 50_000)
    b, a, f = o.sample_tsl(0, E, T, seed=5)
    assert f == 0
    kT = KB * T
    assert (b >= -E / kT).all() and (b <= tsl["beta_cutoff"]).all()
    Ep = E + b * kT
    lo = (np.sqrt(E) - np.sqrt(Ep)) ** 2 / (tsl["awr"] * kT)
    hi = (np.sqrt(E) + np.sqrt(Ep)) ** 2 / (tsl["awr"] * kT)
    assert (a >= lo * (1 - 1e-9)).all() and (a <= hi * (1 + 1e-9)).all()
    mu = (E + Ep - a * tsl["awr"] * kT) / (2 * np.sqrt(E * Ep))
    assert (np.abs(mu) <= 1 + 1e-9).all()


def test_energy_transfer_direction(lib):
    """Neutrons well below kT gain energy; well above, they lose it."""
    d, tsl, o = lib
    for E, up in ((1e-8, True), (1e-6, False)):
        b, _, _ = o.sample_tsl(0, np.full(20_000, E), 450.0, seed=2)
        assert (b.mean() > 0) == up


def test_inelastic_total_reconstruction(lib):
    """GetTotal at tabulated points equals the rank-10 reconstruction of the
    law's cross section.  At T >= T_max the reference takes the top
    interval with weight 0, i.e. the second-highest temperature
    (src/ThermalScattering.cpp:129-132, :153-156); kept as written."""
    d, tsl, o = lib
    for i in (0, 30, 78):  # the last energy is the cutoff, outside the library
        got = o.tsl_total(0, np.full(len(tsl["Ts"]), tsl["Es"][i]), tsl["Ts"])
        np.testing.assert_allclose(got[:-1], tsl["xs"][i][:-1], rtol=2e-3)
        assert got[-1] == got[-2]


def test_broomstick_run(lib):
    d, tsl, o = lib
    r = o.run_fixed_source(20_000, 1, threads=4)
    assert r["lost"] == 0 and r["resample"] == 0
    # nearly every neutron leaves through the cylinder (capture is ~1 %)
    assert 0.97 * 20_000 < r["sum"].sum() <= 20_000
