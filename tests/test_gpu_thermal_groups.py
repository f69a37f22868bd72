"""Thermal groups of the batched multigroup problems (minimc_gb300.thermal_groups),
through the C ABI.

* mc_tsl_group_transfer bins, on the device, exactly the outgoing energies
  E' = E + beta k T of the sampler's own samples (the same streams drawn
  through mc_sample_tsl and binned here on the host give the same counts);
* transfer rows from the MLP surrogate agree with the POD sampler's rows
  at the problems' temperatures, and upscatter out of the lowest group
  grows with temperature;
* batched problems whose thermal groups scatter by the surrogate's rows
  give the k of the same problems with the POD sampler's rows (a
  chi-square over the problems' k differences), and each such problem's
  batched k per cycle equals its single-problem run.
"""
import numpy as np
import pytest
from scipy import stats

from minimc_gb300 import (RNG_PHILOX, TSL_FAST, TSL_MLP, TSL_PHILOX, TSL_POD, Batch, Context, synth, synth_tsl,
                          thermal_groups)

pytestmark = pytest.mark.gpu
BOLTZMANN = 8.617333262145e-11  # MeV/K (the reference's constants::boltzmann)
ROW_TOL = 0.01  # surrogate vs POD transfer fractions (the surrogate's KS distance is ~0.006)


@pytest.fixture(scope="module")
def tsl_ctx(tmp_path_factory):
    d = tmp_path_factory.mktemp("tsl_groups")
    tsl, nuc = synth_tsl.write_tsl(d), synth_tsl.moderator_nuclide(d)
    ctx = Context(0)
    ctx.load_xml(synth_tsl.broomstick_xml(tsl, nuc, histories=10), d)
    return ctx


@pytest.fixture(scope="module")
def trained(tsl_ctx):
    tsl_ctx.train_surrogate(0, E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=8192,
                            samples_per_condition=1024, batch=16384, steps=8000, lr=1e-3, seed=3)
    return tsl_ctx


def host_bins(beta, E, T, bounds):
    ep = E + (beta * BOLTZMANN) * T
    G = len(bounds) - 1
    g = np.zeros(len(ep), dtype=np.int64)
    for k in range(1, G):
        g += ep < bounds[k]
    ok = ~np.isnan(beta)
    return np.bincount(g[ok], minlength=G)


@pytest.mark.parametrize("method", [TSL_POD | TSL_PHILOX | TSL_FAST, TSL_POD | TSL_PHILOX])
def test_transfer_bins_the_sampler_samples(tsl_ctx, method):
    n = 50_000
    E_rows = np.array(thermal_groups.REPRESENTATIVE_MEV + (1e-6,))
    T_rows = np.array([310.0, 455.0, 590.0])
    bounds = thermal_groups.GROUP_BOUNDS_MEV
    probs, fails = tsl_ctx.tsl_group_transfer(0, E_rows, T_rows, n, bounds, seed=17, method=method)
    beta, _, f = tsl_ctx.sample_tsl(0, np.repeat(E_rows, n), np.repeat(T_rows, n), seed=17, method=method)
    assert fails == f
    for r in range(len(E_rows)):
        c = host_bins(beta[r * n:(r + 1) * n], E_rows[r], T_rows[r], bounds)
        assert np.array_equal(probs[r], c / c.sum()), (r, probs[r], c / c.sum())


def test_transfer_rejects_bad_bounds(tsl_ctx):
    from minimc_gb300.engine import MCError

    with pytest.raises(MCError, match="descending"):
        tsl_ctx.tsl_group_transfer(0, [3e-8], [300.0], 100, [1e-6, 1e-5, 1e-11])


def test_surrogate_rows_match_pod_rows(trained):
    T = np.array([300.0, 375.0, 450.0, 525.0, 600.0])
    sur, f1 = thermal_groups.transfer_rows(trained, 0, T, seed=3, method=TSL_MLP)
    pod, f2 = thermal_groups.transfer_rows(trained, 0, T, seed=4, method=TSL_POD | TSL_PHILOX)
    assert f1 == 0 and f2 == 0
    assert np.allclose(sur.sum(-1), 1.0) and np.allclose(pod.sum(-1), 1.0)
    assert np.abs(sur - pod).max() < ROW_TOL, np.abs(sur - pod).max()
    # scatters out of the lowest group: up into group 7 more often when hotter
    up = pod[:, 1, 6]
    assert (np.diff(up) > 0).all(), up
    assert up[0] > 0.01 and up[-1] > 1.5 * up[0]


def thermal_batch(probs, temps, rows, seed_offset=0):
    b = Batch(0)
    made = []
    for i, ((p, h), T) in enumerate(zip(probs, temps)):
        q = thermal_groups.with_thermal_rows(p, T, rows[i])
        b.add(q.xml(), histories=h, seed=p.seed + seed_offset)
        made.append((q, h, p.seed + seed_offset))
    return b, made


def test_thermal_batch_k_surrogate_vs_pod(trained):
    probs = synth.batch_problems(count=16, seed=5, h_min=20_000, h_max=60_000, inactive=5, active=30)
    temps = thermal_groups.problem_temperatures(len(probs), seed=5)
    sur, _ = thermal_groups.transfer_rows(trained, 0, temps, seed=3, method=TSL_MLP)
    pod, _ = thermal_groups.transfer_rows(trained, 0, temps, seed=4, method=TSL_POD | TSL_PHILOX)
    bs, made = thermal_batch(probs, temps, sur)
    bp, _ = thermal_batch(probs, temps, pod, seed_offset=1000)
    rs = bs.run(inactive=5, active=30, fast_math=1)
    rp = bp.run(inactive=5, active=30, fast_math=1)
    assert rs["active_ms"] > 0 and rs["active_ms"] < rs["transport_ms"]
    z = (rs["k_mean"] - rp["k_mean"]) / np.hypot(rs["k_std"], rp["k_std"])
    p = stats.chi2.sf(float(np.sum(z ** 2)), len(z))
    assert p > 1e-3, (p, z)
    # each batched thermal problem is its single-problem run
    for i in (0, 7):
        q, h, seed = made[i]
        ctx = Context(0)
        ctx.load_xml(q.xml())
        s = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=1, histories=h, seed=seed, inactive=5, active=30)
        assert np.array_equal(rs["k_cycle"][i], s.k_cycle)


def test_persistent_batch_very_uneven(built_library):
    """One large problem and fifteen small ones: the small problems' CTAs
    drain their queues and help with the large one; every problem still
    gets its single-run k per cycle."""
    probs = synth.batch_problems(count=16, seed=9, h_min=1_000, h_max=2_000, inactive=2, active=3)
    big = synth.two_zone_cubes(histories=200_000, inactive=2, active=3, seed=99)
    big.estimators = []
    probs = [(big, 200_000)] + probs[1:]
    b = Batch(0)
    for p, h in probs:
        b.add(p.xml(), histories=h, seed=p.seed)
    r = b.run(inactive=2, active=3, fast_math=1)
    for i in (0, 1, 15):
        p, h = probs[i]
        ctx = Context(0)
        ctx.load_xml(p.xml())
        s = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=1, histories=h, seed=p.seed, inactive=2, active=3)
        assert np.array_equal(r["k_cycle"][i], s.k_cycle), i
