"""CPU tests of the oracle's continuous-energy physics (no GPU needed):
ContinuousMap::at's bracket and interpolation, the free-gas temperature
adjustment, free-gas kinematics against the elastic-scattering laws, and an
infinite medium with an analytic k."""
import math

import numpy as np
import pytest

from minimc_gb300 import synth_ce
from oracle import build as ob
from oracle.build import Oracle

KB = 8.617333262145e-11


@pytest.fixture(scope="module")
def ce_data(tmp_path_factory):
    d = tmp_path_factory.mktemp("ce")
    files = synth_ce.write_nuclides(d, n_grid=5000)
    return d, files


def _tables(d, files, name):
    out = {}
    for key in ("total", "capture", "elastic", "fission", "nubar"):
        if key in files[name]:
            axes, v = synth_ce.read_table(d / files[name][key])
            out[key] = (axes[0], v)
    return out


def _energies(x):
    """Grid points, their neighbours, midpoints and out-of-range values."""
    lo, hi = x[0], x[-1]
    mids = 0.5 * (x[:-1] + x[1:])
    return np.concatenate([x, np.nextafter(x, 0), np.nextafter(x, np.inf), mids,
                           [lo / 2, hi * 2, 0.0, lo, hi, np.nextafter(lo, 0), np.nextafter(hi, np.inf)]])


def test_energy_index_is_upper_bound(ce_data):
    d, files = ce_data
    o = Oracle(synth_ce.ce_problem_xml(files, histories=10), d)
    for nuc, name in enumerate(("H1", "O16", "U235")):
        t = _tables(d, files, name)
        E = _energies(t["total"][0])
        got = o.energy_index(nuc, E)
        cols = ["total", "capture", "elastic"] + (["fission", "nubar"] if "fission" in t else [])
        for c, key in enumerate(cols):
            np.testing.assert_array_equal(got[:, c], np.searchsorted(t[key][0], E, side="right"))
        assert (got[:, len(cols):] == -1).all()


def _map_at(x, y, E):
    hi = np.searchsorted(x, E, side="right")
    out = np.empty_like(E)
    top, bot = hi == len(x), hi == 0
    mid = ~(top | bot)
    out[top] = y[-1]
    out[bot] = y[0]
    h = hi[mid]
    k_hi, v_hi, k_lo, v_lo = x[h], y[h], x[h - 1], y[h - 1]
    out[mid] = v_lo + (v_hi - v_lo) / (k_hi - k_lo) * (E[mid] - k_lo)
    return out


def test_material_total_is_continuous_map_at(ce_data):
    """Material::GetMicroscopicTotal at the evaluation temperature: the
    reference's interpolation formula and summation order, bit for bit."""
    d, files = ce_data
    raw = (0.6, 0.3, 0.1)
    o = Oracle(synth_ce.ce_problem_xml(files, histories=10, afrac=raw), d)
    afrac = np.array(raw) / ((raw[0] + raw[1]) + raw[2])  # Material::AssignNuclides normalization
    x = _tables(d, files, "H1")["total"][0]
    E = _energies(x)
    tot, maj = o.material_xs_ce(0, E)
    exp = np.zeros_like(E)
    for k, name in enumerate(("H1", "O16", "U235")):
        xx, yy = _tables(d, files, name)["total"]
        exp = exp + afrac[k] * _map_at(xx, yy, E)
    np.testing.assert_array_equal(tot, exp)
    np.testing.assert_array_equal(maj, exp)


def test_free_gas_adjustment_above_evaluation_temperature(ce_data):
    """At 600 K the 293.6 K totals are not valid: the total becomes the sum
    of the reactions with the scatter cross section rescaled by the free-gas
    factor ratio (src/ContinuousReaction.cpp:225-237)."""
    d, files = ce_data
    o = Oracle(synth_ce.ce_problem_xml(files, histories=10, temperature=600.0, afrac=(1.0, 0.0, 0.0),
                                       names=("H1", "O16", "U235")), d)
    t = _tables(d, files, "H1")
    E = np.geomspace(1e-11, 1e-5, 50)
    tot, _ = o.material_xs_ce(0, E)

    def adj(awr, E, T):
        x = np.sqrt(E / (KB * T))
        arg = awr * x * x
        return (1 + 1 / (2 * arg)) * np.vectorize(math.erf)(np.sqrt(arg)) + np.exp(-arg) / np.sqrt(math.pi * arg)

    awr = files["H1"]["awr"]
    cap = _map_at(*t["capture"], E)
    sc = _map_at(*t["elastic"], E) / adj(awr, E, 293.6) * adj(awr, E, 600.0)
    np.testing.assert_allclose(tot, cap + sc, rtol=1e-13)
    assert (tot > cap + _map_at(*t["elastic"], E)).all()  # hotter target: more collisions


def test_free_gas_kinematics_epithermal():
    """Far above kT the target is at rest: E'/E is uniform on
    [alpha, 1] and the mean lab cosine is 2 / (3A)."""
    for awr in (0.999167339, 15.8575107):
        e, mu = ob.free_gas(awr, 293.6, 1.0, 200_000)
        alpha = ((awr - 1) / (awr + 1)) ** 2
        u = (e - alpha) / (1 - alpha)
        assert abs(u.mean() - 0.5) < 4 * math.sqrt(1 / 12 / len(u))
        assert abs(mu.mean() - 2 / (3 * awr)) < 0.01


def test_free_gas_upscatters_slow_neutrons():
    """A neutron far below kT gains energy from hydrogen (mean about kT)."""
    kT = KB * 293.6
    e, _ = ob.free_gas(0.999167339, 293.6, 1e-3 * kT, 100_000)
    assert 0.9 < e.mean() / kT < 1.1


def test_flat_infinite_medium_k(tmp_path):
    """Energy-independent cross sections in a reflected box: k_inf =
    nu sigma_f / (sigma_c + sigma_f) whatever the scattering does."""
    f = synth_ce.write_flat_nuclide(tmp_path, "F", 10.0, capture=0.3, scatter=0.5, fission=0.2, nubar=2.5)
    xml = synth_ce.ce_problem_xml({"F": f}, histories=4000, names=("F",), afrac=(1.0,), half=5.0)
    r = Oracle(xml, tmp_path).run_keigenvalue(4000, seed=3, inactive=2, active=20, threads=4)
    k = r["k_cycle"][2:]
    assert abs(k.mean() - 1.0) < 4 * k.std(ddof=1) / math.sqrt(len(k)) + 1e-3
