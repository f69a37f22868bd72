"""GPU continuous-energy parity, through the C ABI.

* The unionized-grid energy search equals std::map::upper_bound on every
  table, bit for bit; material cross sections from the exact tables equal
  the oracle's at the evaluation temperature and agree to rounding of the
  free-gas adjustment (CUDA's erf/exp) away from it.
* Reference streams (minstd, exact tables): per-history events and fates,
  fission banks and integer tallies equal the oracle's.
* Philox streams with FP32 union tables: statistical agreement (k within 3
  combined sigma, leakage spectra by a two-sample chi-square test).
"""
import math

import numpy as np
import pytest
from scipy import stats

from minimc_gb300 import BANK_DIRECT, BANK_SLOTS, RNG_MINSTD, RNG_PHILOX, Context, synth_ce
from oracle.build import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ce_data(tmp_path_factory):
    d = tmp_path_factory.mktemp("ce")
    files = synth_ce.write_nuclides(d, n_grid=50_000)
    return d, files


def gpu_ctx(xml, base):
    ctx = Context(0)
    ctx.load_xml(xml, base)
    return ctx


def _energies(x, seed=5):
    lo, hi = x[0], x[-1]
    rng = np.random.default_rng(seed)
    return np.concatenate([x, np.nextafter(x, 0), np.nextafter(x, np.inf), 0.5 * (x[:-1] + x[1:]),
                           np.exp(rng.uniform(np.log(lo / 10), np.log(hi * 10), 100_000)),
                           [lo / 2, hi * 2, lo, hi, np.nextafter(lo, 0), np.nextafter(hi, np.inf)]])


def test_energy_index_bit_exact(ce_data, built_library):
    d, files = ce_data
    xml = synth_ce.ce_problem_xml(files, histories=10)
    g, o = gpu_ctx(xml, d), Oracle(xml, d)
    x = synth_ce.read_table(d / files["U235"]["total"])[0][0]
    E = _energies(x)
    for nuc in range(3):
        np.testing.assert_array_equal(g.energy_index(nuc, E), o.energy_index(nuc, E))


def test_energy_index_distinct_grids(tmp_path, built_library):
    """Tables on different energy axes share one union grid."""
    a = synth_ce.write_flat_nuclide(tmp_path, "A", 1.0, 0.1, 1.0, energies=np.geomspace(1e-11, 20, 7))
    b = synth_ce.write_flat_nuclide(tmp_path, "B", 12.0, 0.2, 2.0, fission=0.3, nubar=2.4,
                                    energies=np.geomspace(3e-10, 5, 11))
    xml = synth_ce.ce_problem_xml({"A": a, "B": b}, histories=10, names=("A", "B"), afrac=(0.5, 0.5))
    g, o = gpu_ctx(xml, tmp_path), Oracle(xml, tmp_path)
    E = _energies(np.union1d(np.geomspace(1e-11, 20, 7), np.geomspace(3e-10, 5, 11)))
    for nuc in range(2):
        np.testing.assert_array_equal(g.energy_index(nuc, E), o.energy_index(nuc, E))


def test_material_xs_bit_exact(ce_data, built_library):
    d, files = ce_data
    xml = synth_ce.ce_problem_xml(files, histories=10)
    g, o = gpu_ctx(xml, d), Oracle(xml, d)
    x = synth_ce.read_table(d / files["H1"]["total"])[0][0]
    E = _energies(x)
    gt, gm = g.material_xs(0, E)
    ot, om = o.material_xs_ce(0, E)
    np.testing.assert_array_equal(gt, ot)
    np.testing.assert_array_equal(gm, om)


def test_material_xs_free_gas_adjusted(ce_data, built_library):
    """At 600 K the totals are sums of reactions with the free-gas factor;
    CUDA's erf/exp may differ from the C library's in the last bit."""
    d, files = ce_data
    xml = synth_ce.ce_problem_xml(files, histories=10, temperature=600.0)
    g, o = gpu_ctx(xml, d), Oracle(xml, d)
    E = np.geomspace(1e-11, 20, 20_000)
    gt, gm = g.material_xs(0, E)
    ot, om = o.material_xs_ce(0, E)
    np.testing.assert_allclose(gt, ot, rtol=1e-14)
    np.testing.assert_allclose(gm, om, rtol=1e-14)


def test_keig_reference_streams_identical(ce_data, built_library):
    d, files = ce_data
    n = 20_000
    xml = synth_ce.ce_problem_xml(files, histories=n, inactive=2, active=3)
    o = Oracle(xml, d).run_keigenvalue(n, 1, 2, 3, threads=8)
    # both bank paths: sites sampled straight into the bank, or per-history
    # slots and a compaction
    for path in (BANK_DIRECT, BANK_SLOTS):
        g = gpu_ctx(xml, d).run_keigenvalue(rng=RNG_MINSTD, bank_path=path)
        assert np.array_equal(g.bank_size, o["bank_size"])
        assert np.array_equal(g.k_cycle, o["k_cycle"])


def test_fixed_source_reference_streams_identical(ce_data, built_library):
    """Leaky box, fission secondaries in their history, energy-binned
    leakage current: events, fates and integer tallies equal the oracle's."""
    d, files = ce_data
    n = 20_000
    xml = synth_ce.ce_problem_xml(files, histories=n, keig=False, reflective=False, half=5.0,
                                  afrac=(0.6, 0.3, 0.001),
                                  estimators=[synth_ce.energy_current("leak", "xhi", bins=40)])
    g = gpu_ctx(xml, d).run_fixed_source(rng=RNG_MINSTD, per_history=True, histories=n)
    o = Oracle(xml, d).run_fixed_source(n, 1, threads=8, per_history=True)
    assert o["secondaries"] > 0
    assert g.raw.secondaries == o["secondaries"]
    assert np.array_equal(g.history_events, o["history_events"])
    assert np.array_equal(g.history_fate, o["history_fate"])
    assert np.array_equal(g.sum, o["sum"])


def test_delta_tracking_reference_streams_identical(ce_data, built_library):
    """Cell delta tracking with a hotter maximum temperature than the
    evaluation: majorants from the free-gas adjustment, virtual collisions."""
    d, files = ce_data
    n = 5_000
    temp = ("  <linear>\n    <gradient x=\"10.0\" y=\"0\" z=\"0\"/>\n    <intercept b=\"293.6\"/>\n"
            "    <bounds upper=\"493.6\" lower=\"93.6\"/>\n  </linear>")
    xml = synth_ce.ce_problem_xml(files, histories=n, keig=False, reflective=False, half=10.0,
                                  afrac=(0.6, 0.3, 0.001), tracking="cell delta", temperature_xml=temp,
                                  estimators=[synth_ce.energy_current("leak", "xhi", bins=40)])
    g = gpu_ctx(xml, d).run_fixed_source(rng=RNG_MINSTD, per_history=True, histories=n)
    o = Oracle(xml, d).run_fixed_source(n, 1, threads=8, per_history=True)
    agree = np.mean((g.history_events == o["history_events"]) & (g.history_fate == o["history_fate"]))
    assert agree > 0.999, agree  # erf/exp last bits may move a rejection
    assert abs(g.sum.sum() - o["sum"].sum()) <= 0.002 * n


def test_keig_fp32_tables_statistical(ce_data, built_library):
    d, files = ce_data
    n, ina, act = 40_000, 4, 20
    xml = synth_ce.ce_problem_xml(files, histories=n, inactive=ina, active=act)
    g = gpu_ctx(xml, d).run_keigenvalue(rng=RNG_PHILOX, fast_math=1)
    o = Oracle(xml, d).run_keigenvalue(n, 1, ina, act, threads=8)
    kg, ko = g.k_cycle[ina:], o["k_cycle"][ina:]
    sig = math.sqrt(kg.var(ddof=1) / len(kg) + ko.var(ddof=1) / len(ko))
    assert abs(kg.mean() - ko.mean()) < 3 * sig + 1e-4, (kg.mean(), ko.mean(), sig)


def test_leakage_spectrum_fp32_tables_chi2(ce_data, built_library):
    d, files = ce_data
    n = 200_000
    xml = synth_ce.ce_problem_xml(files, histories=n, keig=False, reflective=False, half=5.0,
                                  afrac=(0.6, 0.3, 0.001),
                                  estimators=[synth_ce.energy_current("leak", "xhi", bins=40)])
    g = gpu_ctx(xml, d).run_fixed_source(rng=RNG_PHILOX, fast_math=1, histories=n)
    o = Oracle(xml, d).run_fixed_source(n, 1, threads=8)
    a, b = g.sum, o["sum"]
    keep = (a + b) >= 20
    table = np.vstack([a[keep], b[keep]])
    chi2, p, _, _ = stats.chi2_contingency(table)
    assert p > 0.001, (p, a, b)
    assert abs(a.sum() - b.sum()) < 4 * math.sqrt(a.sum() + b.sum())


def test_fp32_tables_off_when_temperature_dependent(ce_data, built_library):
    """Fast mode falls back to the exact tables when cross sections depend
    on temperature, and still agrees statistically."""
    d, files = ce_data
    n, ina, act = 20_000, 3, 12
    xml = synth_ce.ce_problem_xml(files, histories=n, inactive=ina, active=act, temperature=600.0)
    g = gpu_ctx(xml, d).run_keigenvalue(rng=RNG_PHILOX, fast_math=1)
    o = Oracle(xml, d).run_keigenvalue(n, 1, ina, act, threads=8)
    kg, ko = g.k_cycle[ina:], o["k_cycle"][ina:]
    sig = math.sqrt(kg.var(ddof=1) / len(kg) + ko.var(ddof=1) / len(ko))
    assert abs(kg.mean() - ko.mean()) < 3 * sig + 1e-4, (kg.mean(), ko.mean(), sig)


def test_flat_infinite_medium_k(tmp_path, built_library):
    f = synth_ce.write_flat_nuclide(tmp_path, "F", 10.0, capture=0.3, scatter=0.5, fission=0.2, nubar=2.5)
    xml = synth_ce.ce_problem_xml({"F": f}, histories=100_000, names=("F",), afrac=(1.0,), half=5.0,
                                  inactive=2, active=20)
    for fast in (0, 1):
        r = gpu_ctx(xml, tmp_path).run_keigenvalue(rng=RNG_PHILOX, fast_math=fast)
        k = r.k_cycle[2:]
        assert abs(k.mean() - 1.0) < 4 * k.std(ddof=1) / math.sqrt(len(k)) + 1e-4, (fast, k.mean())


def test_transport_bank_direct_path_equals_slot_path(ce_data, built_library):
    """mc_transport_bank on a continuous-energy problem: the sites sampled
    straight into page-locked host output equal the slot path's, site for
    site, for both stream kinds (Philox: one thread per site, in the FP32
    and the FP64 form)."""
    import torch

    from minimc_gb300 import SITE_DTYPE

    d, files = ce_data
    n = 20_000
    ctx = gpu_ctx(synth_ce.ce_problem_xml(files, histories=n, inactive=1, active=1), d)
    rng = np.random.default_rng(9)
    sites = np.zeros(n, SITE_DTYPE)
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    sites["u"], sites["v"], sites["w"] = mu, np.sqrt(1 - mu * mu) * np.cos(ph), np.sqrt(1 - mu * mu) * np.sin(ph)
    sites["energy"] = 2.0
    sites["key"] = np.arange(n, dtype=np.uint64) + 11
    cap = n * max(1, ctx.info.max_yield)
    for opts in (dict(rng=RNG_MINSTD), dict(rng=RNG_PHILOX, fast_math=1), dict(rng=RNG_PHILOX, fast_math=0)):
        ref = np.zeros(cap, SITE_DTYPE)
        m0 = ctx.transport_bank_into(sites, ref, bank_path=BANK_SLOTS, **opts)
        assert m0 > 0
        out = torch.empty(cap * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(SITE_DTYPE)
        m = ctx.transport_bank_into(sites, out, bank_path=BANK_DIRECT, **opts)
        assert m == m0
        assert np.array_equal(out[:m].view(np.uint8), ref[:m0].view(np.uint8))
