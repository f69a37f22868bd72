"""The benchmark's own configuration against the oracle.

bench.py times the 8-group two-zone k-eigenvalue problem at 1e6 histories
per cycle with Philox streams and FP32 sampling arithmetic (directions,
flight lengths and CDF thresholds in FP32; geometry, positions, k and
tallies in FP64).  Here that exact form runs 30 inactive + 30 active
cycles beside the CPU oracle (the reference's algorithm and random streams,
all host threads) on the same problem, and:

  * the mean k over the active cycles agrees within 3 combined standard
    deviations (per-cycle k values, the usual cycle estimate);
  * the group-binned fuel track-length flux and the x-high leakage current
    agree by a chi-square test (p > 1e-3), with each bin's variance taken
    from the spread of the GPU's per-cycle tallies (which carries the
    cycle-to-cycle correlation a per-history variance would miss).
"""
import math
import os

import numpy as np
import pytest

from minimc_gb300 import RNG_PHILOX, Context, synth
from oracle.build import Oracle

pytestmark = pytest.mark.gpu
N, INACTIVE, ACTIVE = 1_000_000, 30, 30
K_SIGMAS = 3.0
CHI2_P_MIN = 1e-3


def test_two_zone_bench_config_against_oracle(built_library):
    from scipy import stats

    xml = synth.two_zone_cubes(histories=N, inactive=INACTIVE, active=ACTIVE).xml()
    ctx = Context(0)
    ctx.load_xml(xml)
    ctx.keig_begin(rng=RNG_PHILOX, fast_math=1)
    k_gpu, per_cycle = [], []
    prev = np.zeros(ctx.info.total_bins)
    for c in range(INACTIVE + ACTIVE):
        k = ctx.keig_cycle(c >= INACTIVE)
        if c >= INACTIVE:
            k_gpu.append(k)
            s, _ = ctx.tallies()
            per_cycle.append((s - prev) / N)
            prev = s
    out = ctx.keig_end()
    assert out.lost == 0 and out.capped == 0 and out.overflow == 0
    o = Oracle(xml).run_keigenvalue(N, 1, INACTIVE, ACTIVE, threads=os.cpu_count() or 1)
    assert o["lost"] == 0

    kg, ko = np.asarray(k_gpu), o["k_cycle"][INACTIVE:]
    sig = math.sqrt(kg.var(ddof=1) / len(kg) + ko.var(ddof=1) / len(ko))
    assert abs(kg.mean() - ko.mean()) < K_SIGMAS * sig, (kg.mean(), ko.mean(), sig)

    t = np.asarray(per_cycle)                      # [cycle][bin] per-history means
    mean_g = t.mean(axis=0)
    var_g = t.var(axis=0, ddof=1) / len(t)         # of the mean over the active cycles
    mean_o = o["sum"] / (N * ACTIVE)
    keep = var_g > 0
    assert keep.sum() >= 8
    chi2 = float(np.sum((mean_g[keep] - mean_o[keep]) ** 2 / (2 * var_g[keep])))
    p = float(stats.chi2.sf(chi2, int(keep.sum())))
    assert p > CHI2_P_MIN, (chi2, int(keep.sum()), p)
