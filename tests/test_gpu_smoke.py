"""First end-to-end GPU checks: the CUDA path against the CPU oracle."""
import numpy as np
import pytest

from minimc_gb300 import RNG_MINSTD, RNG_PHILOX, Context, synth
from oracle.build import Oracle

pytestmark = pytest.mark.gpu


def test_keig_minstd_identical_to_oracle(built_library):
    p = synth.one_group_cube(histories=5000, inactive=3, active=4)
    xml = p.xml()
    ctx = Context(0)
    ctx.load_xml(xml)
    gpu = ctx.run_keigenvalue(rng=RNG_MINSTD)
    cpu = Oracle(xml).run_keigenvalue(5000, 1, 3, 4, threads=4)
    assert np.array_equal(gpu.bank_size, cpu["bank_size"])
    np.testing.assert_allclose(gpu.sum, cpu["sum"], rtol=1e-12)


def test_fixed_source_leakage_minstd(built_library):
    p = synth.sphere_fixed_source(histories=1000)
    xml = p.xml()
    ctx = Context(0)
    ctx.load_xml(xml)
    r = ctx.run_fixed_source(rng=RNG_MINSTD, per_history=True)
    o = Oracle(xml).run_fixed_source(1000, 1, per_history=True)
    assert np.array_equal(r.history_fate, o["history_fate"])
    assert np.array_equal(r.history_events, o["history_events"])
    assert r.sum[0] == o["sum"][0]


def test_keig_philox_statistical(built_library):
    p = synth.one_group_cube(histories=20000, inactive=10, active=20)
    ctx = Context(0)
    ctx.load_xml(p.xml())
    r = ctx.run_keigenvalue(rng=RNG_PHILOX)
    assert 1.3 < r.k_mean < 1.7
