"""GPU parity of the deterministic geometry kernels, through the C ABI:
World::FindCellContaining, Cell::NearestSurface, CSGSurface::Distance and
CSGSurface::Contains must equal the CPU oracle bit for bit on identical
points, and match the reference's known answers."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from minimc_gb300 import GEOMETRY_REFERENCE, GEOMETRY_ROBUST, Context, synth
from oracle.build import Oracle

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
KA = json.loads((GOLDEN / "reference_known_answers.json").read_text())


def broomstick_xml() -> str:
    """A cylinder (x axis) between two planes with voids around it, and a
    sphere cell, to exercise every surface kind."""
    p = synth.one_group_cube(histories=100)
    p.surfaces = ['  <cylinderx name="cyl" r="0.5"/>', '  <planex name="left" x="-3"/>', '  <planex name="right" x="3"/>',
                  '  <sphere name="ball">\n    <center x="10" y="0" z="0"/>\n    <radius r="2"/>\n  </sphere>',
                  '  <cylindery name="cy" r="0.25"/>', '  <cylinderz name="cz" r="0.25"/>',
                  '  <planey name="py" y="0.1"/>', '  <planez name="pz" z="-0.2"/>']
    p.cells = [
        '  <cell name="stick" material="fuel">\n    <surface name="cyl" sense="-1"/>\n'
        '    <surface name="left" sense="+1"/>\n    <surface name="right" sense="-1"/>\n  </cell>',
        '  <cell name="ball" material="fuel">\n    <surface name="ball" sense="-1"/>\n  </cell>',
        '  <cell name="posts" material="fuel">\n    <surface name="cy" sense="-1"/>\n    <surface name="cz" sense="-1"/>\n'
        '    <surface name="py" sense="+1"/>\n    <surface name="pz" sense="-1"/>\n  </cell>',
        '  <void>\n    <surface name="left" sense="-1"/>\n  </void>',
        '  <void>\n    <surface name="right" sense="+1"/>\n  </void>',
        '  <void>\n    <surface name="cyl" sense="+1"/>\n  </void>',
    ]
    p.estimators = []
    return p.xml()


GEOMETRIES = {
    "spheres": lambda: (GOLDEN / "mg_spheres.xml").read_text(),
    "two_zone_boxes": lambda: synth.two_zone_cubes(histories=1000).xml(),
    "cube": lambda: synth.one_group_cube(histories=1000).xml(),
    "mixed": broomstick_xml,
}


def random_points(n, scale, seed):
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(-scale, scale, (n, 3))
    # put a quarter of the points exactly on the coordinate planes used by the
    # geometries (on-surface sense semantics)
    k = n // 4
    xyz[:k, rng.integers(0, 3, k)] = rng.choice([-30.0, -15.0, -10.0, -3.0, 0.0, 0.1, 3.0, 10.0, 15.0, 30.0], k)
    uvw = rng.normal(size=(n, 3))
    uvw /= np.linalg.norm(uvw, axis=1)[:, None]
    uvw[: n // 8] = np.eye(3)[rng.integers(0, 3, n // 8)] * rng.choice([-1.0, 1.0], (n // 8, 1))
    return xyz, uvw


@pytest.mark.parametrize("mode", [GEOMETRY_ROBUST, GEOMETRY_REFERENCE])
@pytest.mark.parametrize("geom", sorted(GEOMETRIES))
def test_geometry_bit_exact(geom, mode, built_library):
    xml = GEOMETRIES[geom]()
    ctx = Context(0)
    ctx.set_geometry_mode(mode)
    ctx.load_xml(xml)
    o = Oracle(xml)
    o.set_quirks(mode == GEOMETRY_REFERENCE)
    scale = {"spheres": 4.0, "two_zone_boxes": 35.0, "cube": 12.0, "mixed": 12.0}[geom]
    xyz, uvw = random_points(100_000, scale, 7)
    cg = ctx.find_cell(xyz)
    co = o.find_cell(xyz)
    assert np.array_equal(cg, co)
    inside = cg >= 0
    sg, dg = ctx.nearest_surface(cg[inside], xyz[inside], uvw[inside])
    so, do = o.nearest_surface(co[inside], xyz[inside], uvw[inside])
    assert np.array_equal(sg, so)
    assert np.array_equal(dg.view(np.int64), do.view(np.int64))  # bit-exact, incl. inf
    for s in range(ctx.info.n_surfaces):
        dg = ctx.surface_distance(s, xyz, uvw)
        do = o.surface_distance(s, xyz, uvw)
        assert np.array_equal(dg.view(np.int64), do.view(np.int64)), s
        assert np.array_equal(ctx.surface_contains(s, xyz), o.surface_contains(s, xyz)), s


def test_reference_known_answers_on_gpu(built_library):
    ctx = Context(0)
    ctx.load_xml((GOLDEN / "mg_spheres.xml").read_text())
    ka = KA["sphere_distance"]
    for case in ka["cases"]:
        d = ctx.surface_distance(0, case["p"], case["d"])[0]
        exp = math.inf if case["distance"] == "inf" else case["distance"]
        assert (math.isinf(d) and math.isinf(exp)) or d == pytest.approx(exp, rel=1e-15)
    names = ["pit", "inner shell", "outer shell", ""]
    cells = ctx.find_cell([[x, 0, 0] for x, _ in KA["find_cell"]["cases"]])
    assert [names[c] for c in cells] == [n for _, n in KA["find_cell"]["cases"]]
    assert ctx.info.n_cells == KA["find_cell"]["n_cells"]
    nk = KA["nearest_surface"]
    s, d = ctx.nearest_surface(1, nk["p"], nk["d"])
    assert ctx.object_name(1, int(s[0])) == nk["surface"] and d[0] == pytest.approx(nk["distance"], rel=1e-15)


def test_multigroup_totals_on_gpu(built_library):
    ctx = Context(0)
    ctx.load_xml((GOLDEN / "mg_nuclides.xml").read_text())
    for cell, name in enumerate(["hydrogen", "oxygen", "uranium235"]):
        tot, maj = ctx.material_xs(cell, [1.0, 2.0])
        assert list(tot) == KA["mg_totals"]["values"][name]
        assert list(maj) == list(tot)
