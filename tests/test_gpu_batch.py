"""GPU batched problems (mc_batch_*), through the C ABI: per problem the k
per cycle of a batched run equals the single-problem run with the same
seed and Philox streams, with and without the per-cycle CUDA graph."""
import numpy as np
import pytest

from minimc_gb300 import BANK_AUTO, BANK_SLOTS, RNG_PHILOX, Batch, Context, synth

pytestmark = pytest.mark.gpu


def problems(count, h_min, h_max):
    return synth.batch_problems(count=count, seed=11, h_min=h_min, h_max=h_max, inactive=2, active=4)


@pytest.mark.parametrize("graph,bank_path", [(True, BANK_AUTO), (False, BANK_AUTO), (True, BANK_SLOTS)])
def test_batch_equals_single_problem_runs(graph, bank_path, built_library):
    """Both bank paths (sites sampled straight into the concatenated bank,
    or slots and a compaction) give each problem its single-run k."""
    probs = problems(6, 2_000, 30_000)
    b = Batch(0)
    for p, h in probs:
        b.add(p.xml(), histories=h, seed=p.seed)
    r = b.run(inactive=2, active=4, fast_math=1, graph=graph, bank_path=bank_path)
    assert r["graph"] == int(graph)
    for i, (p, h) in enumerate(probs):
        ctx = Context(0)
        ctx.load_xml(p.xml())
        s = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=1, histories=h, seed=p.seed, inactive=2, active=4)
        assert np.array_equal(r["k_cycle"][i], s.k_cycle), (i, r["k_cycle"][i], s.k_cycle)


def test_batch_64_uneven_problems(built_library):
    probs = problems(64, 1_000, 50_000)
    b = Batch(0)
    for p, h in probs:
        b.add(p.xml(), histories=h, seed=p.seed)
    r = b.run(inactive=2, active=4, fast_math=1)
    assert r["histories"] == 6 * sum(h for _, h in probs)
    assert np.isfinite(r["k_cycle"]).all() and (r["k_cycle"] > 0).all()
    assert r["launches"] <= 6 + 2 * 5  # one graph launch per cycle plus the autotuner's runs
