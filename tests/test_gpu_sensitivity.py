"""Sensitivity estimators on the GPU (TotalCrossSectionPerturbation and
CurrentTotalCrossSectionSensitivity, src/Perturbation.cpp:68-78,
src/Sensitivity.cpp:55-58), through the C ABI.

With reference streams every history draws the numbers the reference draws,
so the indirect effects, and the sensitivity tallies they score, equal the
oracle's (whose result text the CPU suite pins on the reference's own
output) to the summation order.
"""
import numpy as np
import pytest

from minimc_gb300 import RNG_MINSTD, RNG_PHILOX, Context, synth, synth_ce
from minimc_gb300.engine import Driver, MCError, format_output
from minimc_gb300.synth import with_sensitivities
from oracle.build import Oracle

pytestmark = pytest.mark.gpu
FP_RTOL = 1e-12


def fixed_two_zone(n):
    p = synth.two_zone_cubes(histories=n, groups=4)
    p.problem = "fixedsource"
    for nuc in p.nuclides:
        if nuc.nubar is not None:
            nuc.nubar = nuc.nubar * 0.5  # subcritical chains of secondaries
    p.estimators = [synth.current("leak-xhi", "out-xhi", 4), synth.current("leak-in", "in-xhi")]
    return with_sensitivities(p.xml(), [("dfuel", "fuel"), ("drefl", "reflector")])


def test_multigroup_sensitivities_equal_oracle(built_library):
    n = 20000
    xml = fixed_two_zone(n)
    ctx = Context(0)
    ctx.load_xml(xml)
    assert ctx.info.n_perturbations == 2
    g = ctx.run_fixed_source(rng=RNG_MINSTD, per_history=True, histories=n)
    o = Oracle(xml).run_fixed_source(n, 1, threads=8, per_history=True)
    assert np.array_equal(g.history_events, o["history_events"])
    assert g.raw.secondaries == o["secondaries"] > 0
    np.testing.assert_allclose(g.sum, o["sum"], rtol=FP_RTOL, atol=1e-9)
    np.testing.assert_allclose(g.sum_sq, o["sum_sq"], rtol=FP_RTOL, atol=1e-9)
    est = ctx.estimators()
    assert [e.n_sensitivities for e in est] == [2, 2]
    # every sensitivity block scored
    for e in est:
        for k in range(1, 3):
            assert np.any(g.sum[e.offset + k * e.n_bins: e.offset + (k + 1) * e.n_bins] != 0)


def test_continuous_energy_sensitivities_equal_oracle(built_library, tmp_path):
    files = synth_ce.write_nuclides(tmp_path, n_grid=5000)
    xml = synth_ce.ce_problem_xml(files, histories=4000, keig=False, sphere=6.0, afrac=(0.6, 0.3, 0.001),
                                  estimators=[synth_ce.energy_current("leak", "sphere", bins=20)])
    xml = with_sensitivities(xml, [("dH1", "H1"), ("dU", "U235")])
    ctx = Context(0)
    ctx.load_xml(xml, tmp_path)
    g = ctx.run_fixed_source(rng=RNG_MINSTD, histories=4000)
    o = Oracle(xml, tmp_path).run_fixed_source(4000, 1, threads=8)
    np.testing.assert_allclose(g.sum, o["sum"], rtol=1e-9, atol=1e-9)
    # the result file, sensitivities included
    path = tmp_path / "p.xml"
    path.write_text(xml)
    drv = Driver(ctx)
    assert drv.output_text(g) == format_output(xml, tmp_path, g.sum, g.sum_sq, 4000)
    assert "leak::dH1" in drv.output_text(g) and "leak::dU" in drv.estimator_results(g).keys().__str__()


def test_philox_sensitivities_statistical(built_library):
    """Philox streams: sensitivity means within 5 combined sigma of the
    oracle's."""
    n = 50000
    xml = fixed_two_zone(n)
    ctx = Context(0)
    ctx.load_xml(xml)
    g = ctx.run_fixed_source(rng=RNG_PHILOX, histories=n)
    o = Oracle(xml).run_fixed_source(n, 1, threads=8)
    checked = 0
    for e in ctx.estimators():
        for b in range(e.n_bins):
            # bins with enough crossings for the normal approximation, and
            # the same bin of each sensitivity block
            if min(g.sum[e.offset + b], o["sum"][e.offset + b]) < 50:
                continue
            for k in range(1 + e.n_sensitivities):
                i = e.offset + k * e.n_bins + b
                s, q, so, qo = g.sum[i], g.sum_sq[i], o["sum"][i], o["sum_sq"][i]
                var = (q - s * s / n) + (qo - so * so / n)
                assert abs(s - so) <= 5 * np.sqrt(max(var, 0)) + 1e-9, (e.name, b, k, s, so)
                checked += 1
    assert checked >= 3


def test_keigenvalue_sensitivities_rejected(built_library):
    p = synth.one_group_cube(histories=1000, inactive=1, active=1)
    p.estimators = [synth.current("leak", "cube-xhi")]
    xml = with_sensitivities(p.xml(), [("d", p.nuclides[0].name)])
    ctx = Context(0)
    with pytest.raises(MCError) as e:
        ctx.load_xml(xml)
    assert "fixed-source" in e.value.message
