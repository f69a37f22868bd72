"""Writes the XML fixtures and known answers used by the parity tests.

The problems restate the data of the reference's own unit-test inputs so the
reference's known answers apply to them:

* ``mg_spheres.xml`` -- three concentric spheres (r = 1, 2, 3) filled with
  two-group hydrogen / water / hydrogen and a void outside, with the nuclide
  data of the reference's multigroup test input;
* ``mg_nuclides.xml`` -- the same three nuclides, each alone in a material,
  so that material totals equal nuclide totals;
* ``point_source_leakage.xml`` -- a point source in a unit sphere of a pure
  one-group absorber (Sigma = 1);
* ``infinite_medium.xml`` -- a one-group medium in a sphere of radius 1e10;
* ``error_*.xml`` -- inputs the reference rejects, with its message text.

``reference_known_answers.json`` holds the expected values with the
reference test (file:line) each comes from.  Run:
``python tests/golden/make_fixtures.py``.
"""
from __future__ import annotations

import json
from pathlib import Path

HERE = Path(__file__).resolve().parent

HEAD = '<minimc>\n<general>\n  <particles>neutron</particles>\n  <histories>{hist}</histories>\n  <threads>2</threads>\n  <chunksize>100</chunksize>\n</general>\n'

MG_NUCLIDES = """<nuclides>
  <multigroup groups="2">
    <nuclide name="hydrogen">
      <neutron>
        <capture>0 1</capture>
        <scatter>
          0 0
          1 0
        </scatter>
      </neutron>
    </nuclide>
    <nuclide name="oxygen">
      <neutron>
        <capture>0.5 0.5</capture>
        <scatter>
          0.5 0.0
          0.5 0.5
        </scatter>
      </neutron>
    </nuclide>
    <nuclide name="uranium235">
      <neutron>
        <capture>0.33 0.67</capture>
        <scatter>
          1 0
          0 1
        </scatter>
        <fission>
          <xs>0 1</xs>
          <nubar>0 2.43</nubar>
          <chi>
            0 0.5
            0 0.5
          </chi>
        </fission>
      </neutron>
    </nuclide>
  </multigroup>
</nuclides>
"""

SPHERES = """<surfaces>
  <sphere name="inner shell"><center x="0" y="0" z="0"/><radius r="1"/></sphere>
  <sphere name="middle shell"><center x="0" y="0" z="0"/><radius r="2"/></sphere>
  <sphere name="outer shell"><center x="0" y="0" z="0"/><radius r="3"/></sphere>
</surfaces>
"""

SOURCE = """<problemtype>
  <fixedsource>
    <position><constant x="0" y="0" z="0"/></position>
    <direction><isotropic/></direction>
    <energy><constant energy="{energy}"/></energy>
    <particletype><constant type="neutron"/></particletype>
  </fixedsource>
</problemtype>
"""


def mg_spheres(cells_override: str | None = None, nuclides: str = MG_NUCLIDES, hist: int = 100000) -> str:
    materials = """<materials>
  <material name="water" aden="2">
    <nuclide name="hydrogen" afrac="0.67"/>
    <nuclide name="oxygen" afrac="0.33"/>
  </material>
  <material name="hydrogen" aden="1"><nuclide name="hydrogen" afrac="0.1"/></material>
  <material name="oxygen" aden="1"><nuclide name="oxygen" afrac="0.1"/></material>
</materials>
"""
    cells = cells_override or """<cells>
  <cell name="pit" material="hydrogen"><surface name="inner shell" sense="-1"/></cell>
  <cell name="inner shell" material="water">
    <surface name="inner shell" sense="+1"/><surface name="middle shell" sense="-1"/>
  </cell>
  <cell name="outer shell" material="hydrogen">
    <surface name="middle shell" sense="+1"/><surface name="outer shell" sense="-1"/>
  </cell>
  <void><surface name="outer shell" sense="+1"/></void>
</cells>
"""
    return (HEAD.format(hist=hist) + nuclides + materials + SPHERES + cells + SOURCE.format(energy=1) +
            '<estimators>\n  <current name="leakage" surface="outer shell"/>\n</estimators>\n</minimc>\n')


def mg_nuclides() -> str:
    materials = """<materials>
  <material name="m-hydrogen" aden="1"><nuclide name="hydrogen" afrac="1"/></material>
  <material name="m-oxygen" aden="1"><nuclide name="oxygen" afrac="1"/></material>
  <material name="m-uranium235" aden="1"><nuclide name="uranium235" afrac="1"/></material>
</materials>
"""
    cells = """<cells>
  <cell name="c-hydrogen" material="m-hydrogen"><surface name="inner shell" sense="-1"/></cell>
  <cell name="c-oxygen" material="m-oxygen">
    <surface name="inner shell" sense="+1"/><surface name="middle shell" sense="-1"/>
  </cell>
  <cell name="c-uranium235" material="m-uranium235">
    <surface name="middle shell" sense="+1"/><surface name="outer shell" sense="-1"/>
  </cell>
  <void><surface name="outer shell" sense="+1"/></void>
</cells>
"""
    return HEAD.format(hist=1000) + MG_NUCLIDES + materials + SPHERES + cells + SOURCE.format(energy=1) + "</minimc>\n"


def one_group(capture: float, scatter: float | None, radius: str, hist: int, estimator: bool,
              fission: tuple[float, float] | None = None) -> str:
    parts = [f"        <capture>{capture}</capture>"]
    if scatter is not None:
        parts.append(f"        <scatter>{scatter}</scatter>")
    if fission is not None:
        parts.append(f"        <fission><xs>{fission[0]}</xs><nubar>{fission[1]}</nubar><chi>1.0</chi></fission>")
    nuc = ('<nuclides>\n  <multigroup groups="1">\n    <nuclide name="medium">\n      <neutron>\n' +
           "\n".join(parts) + "\n      </neutron>\n    </nuclide>\n  </multigroup>\n</nuclides>\n")
    body = ('<materials>\n  <material name="medium" aden="1"><nuclide name="medium" afrac="1"/></material>\n</materials>\n'
            f'<surfaces>\n  <sphere name="sphere"><center x="0" y="0" z="0"/><radius r="{radius}"/></sphere>\n</surfaces>\n'
            '<cells>\n  <cell name="sphere" material="medium"><surface name="sphere" sense="-1"/></cell>\n'
            '  <void><surface name="sphere" sense="+1"/></void>\n</cells>\n')
    est = '<estimators>\n  <current name="leakage" surface="sphere"/>\n</estimators>\n' if estimator else ""
    return HEAD.format(hist=hist) + nuc + body + SOURCE.format(energy=1) + est + "</minimc>\n"


ERRORS = {
    # cell referencing a surface that <surfaces> does not define
    # (CSGSurface::Create message, src/CSGSurface.cpp:20-30; test_CSGSurface.cpp:14-21)
    "error_nonexistent_surface.xml": (
        mg_spheres(cells_override="""<cells>
  <cell name="pit" material="hydrogen"><surface name="nonexistent" sense="-1"/></cell>
</cells>
"""),
        'Surface node "nonexistent" not found. Must be one of: '
        '["inner shell", "middle shell", "outer shell", ]'),
    # malformed capture (test_Nuclide.cpp:23-31)
    "error_malformed_capture.xml": (
        mg_spheres(nuclides=MG_NUCLIDES.replace("<capture>0 1</capture>", "<capture>0 1 2</capture>")),
        "/minimc/nuclides/multigroup/nuclide/neutron/capture: Expected 2 entries but got 3"),
    # malformed scatter (test_Nuclide.cpp:32-37)
    "error_malformed_scatter.xml": (
        mg_spheres(nuclides=MG_NUCLIDES.replace("          0 0\n          1 0", "          0 0\n          1 0 1")),
        "/minimc/nuclides/multigroup/nuclide/neutron/scatter: Expected 4 entries but got 5"),
    # nuclide without data for the requested particle (test_Nuclide.cpp:38-41)
    "error_missing_particle_data.xml": (
        mg_spheres(nuclides=MG_NUCLIDES.replace(
            """    <nuclide name="hydrogen">
      <neutron>
        <capture>0 1</capture>
        <scatter>
          0 0
          1 0
        </scatter>
      </neutron>
    </nuclide>""", '    <nuclide name="hydrogen">\n    </nuclide>')),
        '/minimc/nuclides/multigroup/nuclide: "neutron" node not found'),
}


def known_answers() -> dict:
    inf = "inf"
    return {
        "sphere_distance": {
            "source": "test/test_CSGSurface.cpp:23-56",
            "surface": "inner shell",
            "cases": [
                {"p": [2, 0, 0], "d": [0, 0, 1], "distance": inf},
                {"p": [1, 0, 0], "d": [0, 0, 1], "distance": inf},
                {"p": [0, 0, -2], "d": [0, 0, 1], "distance": 1.0},
                {"p": [0, 0, -1], "d": [0, 0, 1], "distance": 2.0},
                {"p": [0, 0, 0], "d": [0, 0, 1], "distance": 1.0},
                {"p": [0, 0, 1], "d": [0, 0, 1], "distance": inf},
                {"p": [0, 0, 2], "d": [0, 0, 1], "distance": inf},
            ],
        },
        "find_cell": {
            "source": "test/test_World.cpp:22-53",
            "n_cells": 4,
            "cases": [[0.0, "pit"], [0.5, "pit"], [1.0, "inner shell"], [1.5, "inner shell"],
                      [2.0, "outer shell"], [2.5, "outer shell"]],
        },
        "nearest_surface": {
            "source": "test/test_Cell.cpp:22-27",
            "cell": "inner shell", "p": [1.5, 0, 0], "d": [1, 0, 0], "surface": "middle shell", "distance": 0.5,
        },
        "mg_totals": {
            "source": "test/test_Nuclide.cpp:68-73",
            "values": {"hydrogen": [1.0, 1.0], "oxygen": [1.5, 1.0], "uranium235": [1.33, 2.67]},
        },
        "direction": {
            "source": "test/test_Point.cpp:49-59",
            "normalize": {"in": [2, 3, 6], "out": [2 / 7, 3 / 7, 6 / 7]},
            "rotate": {"d": [0, 1, 0], "mu": 0.0, "phi": 0.0, "out": [0, 0, -1]},
        },
        "point_source_leakage": {
            "source": "test/test_FixedSource.cpp:13-26, test/Statistics.hpp:16-21",
            "histories": 1000, "expected": 0.36787944117144233,
            "rel_tolerance": "3*sqrt((1-p)/(p*N))",
        },
        "errors": {name: msg for name, (_, msg) in ERRORS.items()},
    }


def main() -> None:
    (HERE / "mg_spheres.xml").write_text(mg_spheres())
    (HERE / "mg_nuclides.xml").write_text(mg_nuclides())
    (HERE / "point_source_leakage.xml").write_text(one_group(1, None, "1", 1000, True))
    (HERE / "infinite_medium.xml").write_text(one_group(0.75, 0.25, "1e10", 100000, False, (0, 1)))
    for name, (xml, _) in ERRORS.items():
        (HERE / name).write_text(xml)
    (HERE / "reference_known_answers.json").write_text(json.dumps(known_answers(), indent=1) + "\n")


if __name__ == "__main__":
    main()
