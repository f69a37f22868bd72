"""Thermal groups of multigroup problems, fed by the thermal-scattering
sampler at each problem's material temperature.

The reference's multigroup data carry no temperature dependence: a
nuclide's scatter matrix (src/Multigroup.cpp:124-147, rows outgoing,
columns incoming) is fixed.  The batched workload gives every problem a
material temperature (300-600 K) and makes the two lowest of its 8 groups
thermal.  A scatter in a thermal group lands in the group of the outgoing
energy that the bound moderator's thermal scattering law gives at a
representative incident energy of the group and the problem's temperature:
E' = E + beta k T (ThermalScattering::Scatter,
src/ThermalScattering.cpp:159-171).  The transfer rows -- the fraction of
scatters from each thermal group into every group -- are sampled on the
device (``Context.tsl_group_transfer``, C ABI ``mc_tsl_group_transfer``),
either from the MLP surrogate (``TSL_MLP``) or from the POD sampler (the
plain form), and written into the problem's scatter matrix; the group's
scattering cross section is kept, only where its scatters go changes.
Multigroup transport then samples the outgoing group per collision from
that matrix exactly as it does for any other group (Multigroup::Scatter,
src/Multigroup.cpp:249-265).  With a fixed representative energy and one
temperature per problem, a thermal group's outgoing-group distribution is
one categorical distribution per problem, so sampling it once with 2^20
scatters per row gives the rows to about 1e-3.
"""
from __future__ import annotations

import copy
import re

import numpy as np

from .engine import TSL_MLP

# 8 groups, boundaries in MeV (descending; group 1 the fastest): groups 7
# (0.1-1 eV) and 8 (below 0.1 eV) are thermal
GROUP_BOUNDS_MEV = np.array([20.0, 2.0, 0.1, 1e-2, 1e-3, 1e-4, 1e-6, 1e-7, 1e-11])
THERMAL_GROUPS = (6, 7)  # 0-based
REPRESENTATIVE_MEV = (3e-7, 3e-8)  # 0.3 eV and 0.03 eV
T_RANGE = (300.0, 600.0)


def problem_temperatures(count: int, seed: int = 11) -> np.ndarray:
    """Material temperatures of `count` problems, uniform in 300-600 K."""
    return np.random.default_rng(seed).uniform(T_RANGE[0], T_RANGE[1], count)


def transfer_rows(ctx, tsl: int, temperatures, samples: int = 1 << 20, seed: int = 1, method: int = TSL_MLP):
    """Transfer rows of the thermal groups at each temperature:
    rows[p, k, g] = fraction of scatters from thermal group THERMAL_GROUPS[k]
    at temperatures[p] that land in group g.  Returns (rows, failures)."""
    T = np.repeat(np.asarray(temperatures, dtype=np.float64), len(THERMAL_GROUPS))
    E = np.tile(np.asarray(REPRESENTATIVE_MEV), len(temperatures))
    probs, fails = ctx.tsl_group_transfer(tsl, E, T, samples, GROUP_BOUNDS_MEV, seed=seed, method=method)
    return probs.reshape(len(temperatures), len(THERMAL_GROUPS), len(GROUP_BOUNDS_MEV) - 1), fails


_CELL = re.compile(r'(<cell name="[^"]*" material="[^"]*")')


def with_thermal_rows(problem, temperature: float, rows):
    """A copy of an 8-group problem whose thermal groups scatter by the given
    transfer rows ([len(THERMAL_GROUPS), 8]) in every nuclide, and whose
    material cells carry the temperature (Cell's temperature attribute,
    src/Cell.cpp:106-112)."""
    if problem.groups != len(GROUP_BOUNDS_MEV) - 1:
        raise ValueError(f"thermal groups need {len(GROUP_BOUNDS_MEV) - 1}-group problems")
    p = copy.deepcopy(problem)
    for nuc in p.nuclides:
        if nuc.scatter is None:
            continue
        S = np.array(nuc.scatter, dtype=np.float64)
        for k, g in enumerate(THERMAL_GROUPS):
            r = np.asarray(rows[k], dtype=np.float64)
            if r.sum() > 0:
                S[:, g] = S[:, g].sum() * r / r.sum()
        nuc.scatter = S
    p.cells = [_CELL.sub(rf'\1 temperature="{float(temperature)!r}"', c) for c in p.cells]
    return p
