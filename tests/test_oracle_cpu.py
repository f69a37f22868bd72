"""CPU tests: the oracle against the reference's known answers, the random
streams against their published definitions, and the problem loader's
semantic checks (no GPU needed)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from minimc_gb300 import synth
from oracle import build as ob
from oracle.build import Oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
KA = json.loads((GOLDEN / "reference_known_answers.json").read_text())


def _inf(v):
    return math.inf if v == "inf" else v


def test_fixtures_are_current(tmp_path):
    """The committed fixtures are what make_fixtures.py writes."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("mf", GOLDEN / "make_fixtures.py")
    mf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mf)
    assert (GOLDEN / "mg_spheres.xml").read_text() == mf.mg_spheres()
    assert json.loads((GOLDEN / "reference_known_answers.json").read_text()) == json.loads(
        json.dumps(mf.known_answers()))


def test_sphere_distances_known_answers():
    o = Oracle((GOLDEN / "mg_spheres.xml").read_text())
    ka = KA["sphere_distance"]
    for case in ka["cases"]:
        d = o.surface_distance(0, case["p"], case["d"])[0]  # surface 0 = inner shell
        exp = _inf(case["distance"])
        if math.isinf(exp):
            assert math.isinf(d)
        else:
            assert d == pytest.approx(exp, rel=1e-15)


def test_find_cell_known_answers():
    o = Oracle((GOLDEN / "mg_spheres.xml").read_text())
    names = ["pit", "inner shell", "outer shell", ""]
    ka = KA["find_cell"]
    pts = [[x, 0, 0] for x, _ in ka["cases"]]
    cells = o.find_cell(pts)
    assert [names[c] for c in cells] == [name for _, name in ka["cases"]]


def test_nearest_surface_known_answer():
    o = Oracle((GOLDEN / "mg_spheres.xml").read_text())
    ka = KA["nearest_surface"]
    s, d = o.nearest_surface(1, ka["p"], ka["d"])
    assert s[0] == 1  # middle shell
    assert d[0] == pytest.approx(ka["distance"], rel=1e-15)


def test_multigroup_totals_known_answers():
    o = Oracle((GOLDEN / "mg_nuclides.xml").read_text())
    for cell, name in enumerate(["hydrogen", "oxygen", "uranium235"]):
        got = [o.material_total(cell, g) for g in (1, 2)]
        assert got == KA["mg_totals"]["values"][name]


def test_direction_known_answers():
    ka = KA["direction"]
    assert list(ob.normalize(ka["normalize"]["in"])) == ka["normalize"]["out"]
    r = ka["rotate"]
    assert list(ob.rotate(r["d"], r["mu"], r["phi"])) == r["out"]


@pytest.mark.parametrize("name", sorted(KA["errors"]))
def test_reference_error_messages(name):
    with pytest.raises(RuntimeError) as e:
        Oracle((GOLDEN / name).read_text())
    assert str(e.value) == KA["errors"][name]


def test_point_source_leakage_statistical():
    """Reference test: leakage = exp(-1) within 3 sigma (Bernoulli)."""
    ka = KA["point_source_leakage"]
    o = Oracle((GOLDEN / "point_source_leakage.xml").read_text())
    r = o.run_fixed_source(ka["histories"], 1)
    p, n = ka["expected"], ka["histories"]
    est = r["sum"][0] / n
    assert abs(est - p) / p < 3 * math.sqrt((1 - p) / (p * n))


def test_philox_known_answer_vectors():
    """Philox4x32-10 known-answer vectors (Random123 distribution)."""
    assert ob.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert ob.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert ob.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_minstd_generate_canonical_definition():
    """std::uniform_real_distribution over minstd_rand, restated from the C++
    standard: x' = 48271 x mod (2^31-1); U = ((g1-1) + (g2-1) R) / R^2."""
    m, a, r = 2147483647, 48271, 2147483646.0
    for seed in (1, 2, 12345, 2**31 - 2):
        x = seed % m or 1
        ref = []
        for _ in range(50):
            x = x * a % m
            g1 = x
            x = x * a % m
            g2 = x
            s = float(g1 - 1) + float(g2 - 1) * r
            ref.append(s / (r * r))
        assert np.array_equal(ob.minstd_canonical(seed, 50), np.array(ref))


def test_infinite_medium_absorption_fraction():
    """Fixed source in an infinite medium with c = 0.25: every history ends by
    capture after a geometric number of scatters (mean 1/(1-c))."""
    o = Oracle((GOLDEN / "infinite_medium.xml").read_text())
    n = 20000
    r = o.run_fixed_source(n, 1, threads=4, per_history=True)
    assert r["lost"] == 0
    assert np.all(r["history_fate"] == 2)  # capture
    mean_events = r["history_events"].mean()
    assert mean_events == pytest.approx(1 / 0.75, rel=0.03)


def test_keig_reflected_box_equals_k_inf():
    """A reflective cube of the one-group material is an infinite medium:
    k_eff = nu Sigma_f / Sigma_a = 2.5 * 0.2 / 0.3 = 5/3."""
    p = synth.one_group_cube(histories=4000, inactive=5, active=20)
    p.surfaces = synth.box_planes("cube", 10.0, reflective=True)
    o = Oracle(p.xml())
    r = o.run_keigenvalue(4000, 1, 5, 20, threads=4)
    k = r["k_cycle"][5:]
    assert k.mean() == pytest.approx(5 / 3, abs=4 * k.std() / math.sqrt(len(k)) + 1e-3)


def test_robust_geometry_loses_no_particles():
    """Reference semantics lose grazing particles from box cells; the robust
    crossing keeps every particle inside the geometry."""
    p = synth.one_group_cube(histories=5000, inactive=3, active=4)
    ref = Oracle(p.xml())
    ref.set_quirks(True)
    rob = Oracle(p.xml())
    rob.set_quirks(False)
    r_ref = ref.run_keigenvalue(5000, 1, 3, 4, threads=4)
    r_rob = rob.run_keigenvalue(5000, 1, 3, 4, threads=4)
    assert r_rob["lost"] == 0
    assert r_ref["lost"] > 0
    # identical until the first lost particle changes the bank
    assert r_ref["bank_size"][0] == r_rob["bank_size"][0]


def test_two_zone_problem_loads_and_runs():
    p = synth.two_zone_cubes(histories=20000, inactive=2, active=2)
    o = Oracle(p.xml())
    r = o.run_keigenvalue(20000, 1, 2, 2, threads=4)
    assert r["lost"] == 0
    assert 0.7 < r["k_cycle"][-1] < 1.3
