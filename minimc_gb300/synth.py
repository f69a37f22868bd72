"""Seeded synthetic problems in minimc's XML input format.

The reference's nuclear data are Git-LFS pointers that are not present, so
every workload here is generated: multigroup cross sections drawn from a
seeded generator, CSG box geometries, and (see ``tsl``/``ce``) continuous
energy and thermal-scattering tables.  Each builder returns XML text that
both the GPU engine and the CPU oracle read.

Conventions of the reference input (test/minimc.xsd):
  * a multigroup scatter or chi matrix is written with rows = outgoing group,
    columns = incoming group (src/Multigroup.cpp:124-147);
  * groups are 1..G with 1 the fastest;
  * <void> cells mark leakage.
"""
from __future__ import annotations

import re

from dataclasses import dataclass, field

import numpy as np


def _fmt(v) -> str:
    return repr(float(v))


def _vec(a) -> str:
    return " ".join(_fmt(x) for x in np.ravel(a))


def _mat(m) -> str:
    m = np.asarray(m)
    return "\n".join(" ".join(_fmt(x) for x in row) for row in m)


@dataclass
class MGNuclide:
    name: str
    capture: np.ndarray | None = None
    scatter: np.ndarray | None = None   # [g_out, g_in]
    fission: np.ndarray | None = None
    nubar: np.ndarray | None = None
    chi: np.ndarray | None = None       # [g_out, g_in]

    def xml(self) -> str:
        parts = [f'    <nuclide name="{self.name}">', "      <neutron>"]
        if self.capture is not None:
            parts.append(f"        <capture>{_vec(self.capture)}</capture>")
        if self.scatter is not None:
            parts.append(f"        <scatter>\n{_mat(self.scatter)}\n        </scatter>")
        if self.fission is not None:
            parts.append("        <fission>")
            parts.append(f"          <xs>{_vec(self.fission)}</xs>")
            parts.append(f"          <nubar>{_vec(self.nubar)}</nubar>")
            parts.append(f"          <chi>\n{_mat(self.chi)}\n          </chi>")
            parts.append("        </fission>")
        parts += ["      </neutron>", "    </nuclide>"]
        return "\n".join(parts)


@dataclass
class Problem:
    groups: int
    nuclides: list[MGNuclide]
    materials: list[tuple[str, float, list[tuple[str, float]]]]
    surfaces: list[str]
    cells: list[str]
    histories: int
    problem: str
    estimators: list[str] = field(default_factory=list)
    seed: int = 1
    threads: int = 1
    tracking: str | None = None
    source_group: int = 1
    source_position: tuple = (0.0, 0.0, 0.0)
    source_direction: str = "<isotropic/>"

    def xml(self) -> str:
        gen = [f"  <particles>neutron</particles>", f"  <histories>{self.histories}</histories>",
               f"  <threads>{self.threads}</threads>", "  <chunksize>1000</chunksize>",
               f"  <seed>{self.seed}</seed>"]
        if self.tracking:
            gen.append(f"  <tracking>{self.tracking}</tracking>")
        nucs = "\n".join(n.xml() for n in self.nuclides)
        mats = []
        for name, aden, comps in self.materials:
            mats.append(f'  <material name="{name}" aden="{_fmt(aden)}">')
            mats += [f'    <nuclide name="{n}" afrac="{_fmt(a)}"/>' for n, a in comps]
            mats.append("  </material>")
        x, y, z = self.source_position
        src = (f'    <position>\n      <constant x="{_fmt(x)}" y="{_fmt(y)}" z="{_fmt(z)}"/>\n    </position>\n'
               f"    <direction>\n      {self.source_direction}\n    </direction>\n"
               f'    <energy>\n      <constant energy="{self.source_group}"/>\n    </energy>\n'
               f'    <particletype>\n      <constant type="neutron"/>\n    </particletype>')
        if self.problem.startswith("keigenvalue"):
            prob = f"<{self.problem}>\n  <initialsource>\n{src}\n  </initialsource>\n</keigenvalue>"
        else:
            prob = f"<fixedsource>\n{src}\n</fixedsource>"
        est = ""
        if self.estimators:
            est = "<estimators>\n" + "\n".join(self.estimators) + "\n</estimators>\n"
        return (
            "<minimc>\n<general>\n" + "\n".join(gen) + "\n</general>\n"
            f'<nuclides>\n  <multigroup groups="{self.groups}">\n{nucs}\n  </multigroup>\n</nuclides>\n'
            "<materials>\n" + "\n".join(mats) + "\n</materials>\n"
            "<surfaces>\n" + "\n".join(self.surfaces) + "\n</surfaces>\n"
            "<cells>\n" + "\n".join(self.cells) + "\n</cells>\n"
            f"<problemtype>\n{prob}\n</problemtype>\n" + est + "</minimc>\n")


# ---------------------------------------------------------------------------
# geometry helpers


def box_planes(prefix: str, half: float, reflective: bool = False) -> list[str]:
    r = ' reflective="true"' if reflective else ""
    out = []
    for ax in "xyz":
        out.append(f'  <plane{ax} name="{prefix}-{ax}lo" {ax}="{_fmt(-half)}"{r}/>')
        out.append(f'  <plane{ax} name="{prefix}-{ax}hi" {ax}="{_fmt(half)}"{r}/>')
    return out


def box_cell(name: str, material: str, prefix: str) -> str:
    s = [f'  <cell name="{name}" material="{material}">']
    for ax in "xyz":
        s.append(f'    <surface name="{prefix}-{ax}lo" sense="+1"/>')
        s.append(f'    <surface name="{prefix}-{ax}hi" sense="-1"/>')
    s.append("  </cell>")
    return "\n".join(s)


def outside_voids(prefix: str) -> list[str]:
    """Six half-space voids covering everything outside a box (first match
    in XML order makes overlaps harmless)."""
    out = []
    for ax in "xyz":
        out.append(f'  <void>\n    <surface name="{prefix}-{ax}lo" sense="-1"/>\n  </void>')
        out.append(f'  <void>\n    <surface name="{prefix}-{ax}hi" sense="+1"/>\n  </void>')
    return out


def shell_cells(name: str, material: str, inner: str, outer: str) -> list[str]:
    """The region between two concentric boxes as six convex slabs."""
    cells = []
    axes = "xyz"
    for i, ax in enumerate(axes):
        for side, (sin, sout) in (("lo", ("-1", "+1")), ("hi", ("+1", "-1"))):
            s = [f'  <cell name="{name}-{ax}{side}" material="{material}">']
            # along the slab axis: between outer and inner plane on this side
            if side == "lo":
                s.append(f'    <surface name="{outer}-{ax}lo" sense="+1"/>')
                s.append(f'    <surface name="{inner}-{ax}lo" sense="-1"/>')
            else:
                s.append(f'    <surface name="{inner}-{ax}hi" sense="+1"/>')
                s.append(f'    <surface name="{outer}-{ax}hi" sense="-1"/>')
            # earlier axes: restricted to the inner box; later axes: outer box
            for j, bx in enumerate(axes):
                if j == i:
                    continue
                box = inner if j < i else outer
                s.append(f'    <surface name="{box}-{bx}lo" sense="+1"/>')
                s.append(f'    <surface name="{box}-{bx}hi" sense="-1"/>')
            s.append("  </cell>")
            cells.append("\n".join(s))
    return cells


def tracklength(name: str, cell: str, groups: int) -> str:
    return (f'  <tracklength name="{name}" cell="{cell}">\n    <bins>\n      <energy>\n'
            f'        <linspace bins="{groups}" min="0.5" max="{groups + 0.5}"/>\n'
            f"      </energy>\n    </bins>\n  </tracklength>")


def current(name: str, surface: str, groups: int | None = None) -> str:
    if not groups:
        return f'  <current name="{name}" surface="{surface}"/>'
    return (f'  <current name="{name}" surface="{surface}">\n    <bins>\n      <energy>\n'
            f'        <linspace bins="{groups}" min="0.5" max="{groups + 0.5}"/>\n'
            f"      </energy>\n    </bins>\n  </current>")


# ---------------------------------------------------------------------------
# workloads


def one_group_cube(histories: int = 10_000, inactive: int = 50, active: int = 100, side: float = 20.0,
                   seed: int = 1) -> Problem:
    """One-group k-eigenvalue cube: sigma_t = 1.0 /cm = scatter 0.7 + capture
    0.1 + fission 0.2, nu = 2.5, chi = 1, vacuum boundary.  k_inf = 1.6667."""
    fuel = MGNuclide("fuel", capture=np.array([0.1]), scatter=np.array([[0.7]]), fission=np.array([0.2]),
                     nubar=np.array([2.5]), chi=np.array([[1.0]]))
    return Problem(
        groups=1, nuclides=[fuel], materials=[("fuel", 1.0, [("fuel", 1.0)])],
        surfaces=box_planes("cube", side / 2), cells=[box_cell("cube", "fuel", "cube"), *outside_voids("cube")],
        histories=histories, problem=f'keigenvalue inactive="{inactive}" active="{active}"',
        estimators=[tracklength("flux", "cube", 1), current("leak-xhi", "cube-xhi")], seed=seed)


def mg_data(rng: np.random.Generator, G: int, fissile: bool, k_inf: float = 1.2):
    """Seeded G-group data: sigma_t log-uniform in [0.2, 2.0]; downscatter-only
    P0 matrix with scatter ratio U(0.6, 0.95); fission (fuel only) scaled so
    that the infinite-medium k is k_inf; chi uniform over groups 1-3."""
    sig_t = np.exp(rng.uniform(np.log(0.2), np.log(2.0), G))
    ratio = rng.uniform(0.6, 0.95, G)
    S = np.zeros((G, G))  # [g_out, g_in]
    for gi in range(G):
        w = rng.uniform(0.2, 1.0, G - gi)
        w[0] += 1.0  # favour in-group scattering
        S[gi:, gi] = ratio[gi] * sig_t[gi] * w / w.sum()
    sig_a = sig_t - S.sum(axis=0)
    if not fissile:
        return MGNuclide("", capture=sig_a, scatter=S), sig_t
    frac = rng.uniform(0.3, 0.6, G)
    chi_col = np.zeros(G)
    chi_col[: min(3, G)] = 1.0 / min(3, G)
    nu = np.full(G, 2.5)
    # infinite-medium k for a trial fission fraction, then rescale
    T = np.diag(sig_t)
    A = np.linalg.solve(T - S, np.outer(chi_col, nu * frac * sig_a))
    k0 = float(np.max(np.abs(np.linalg.eigvals(A))))
    scale = k_inf / k0
    if np.max(frac * scale) > 0.95:
        s2 = 0.95 / np.max(frac)
        nu = nu * scale / s2
        scale = s2
    sig_f = frac * scale * sig_a
    cap = sig_a - sig_f
    chi = np.tile(chi_col[:, None], (1, G))
    return MGNuclide("", capture=cap, scatter=S, fission=sig_f, nubar=nu, chi=chi), sig_t


def two_zone_cubes(histories: int = 1_000_000, inactive: int = 20, active: int = 50, groups: int = 8,
                   inner: float = 30.0, outer: float = 60.0, seed: int = 2026) -> Problem:
    """8-group two-zone k-eigenvalue problem: a fuel cube (side 30 cm) inside
    a reflector cube (side 60 cm), vacuum outside; seeded cross sections."""
    rng = np.random.default_rng(seed)
    fuel, _ = mg_data(rng, groups, True)
    refl, _ = mg_data(rng, groups, False)
    fuel.name, refl.name = "fuel", "reflector"
    return Problem(
        groups=groups, nuclides=[fuel, refl],
        materials=[("fuel", 1.0, [("fuel", 1.0)]), ("reflector", 1.0, [("reflector", 1.0)])],
        surfaces=box_planes("in", inner / 2) + box_planes("out", outer / 2),
        cells=[box_cell("fuel", "fuel", "in"), *shell_cells("reflector", "reflector", "in", "out"),
               *outside_voids("out")],
        histories=histories, problem=f'keigenvalue inactive="{inactive}" active="{active}"',
        estimators=[tracklength("fuel-flux", "fuel", groups), current("leak-xhi", "out-xhi", groups)], seed=1)


def one_group_slab_sphere(histories: int = 10_000, inactive: int = 50, active: int = 100, half: float = 10.0,
                          radius: float = 12.0, seed: int = 1) -> Problem:
    """The one-group k-eigenvalue problem of ``one_group_cube`` in a geometry
    the reference's own surfaces describe (it has no planey/planez): the
    slab -half < x < half cut by a sphere of the given radius, vacuum
    outside."""
    fuel = MGNuclide("fuel", capture=np.array([0.1]), scatter=np.array([[0.7]]), fission=np.array([0.2]),
                     nubar=np.array([2.5]), chi=np.array([[1.0]]))
    surfaces = [f'  <planex name="xlo" x="{_fmt(-half)}"/>', f'  <planex name="xhi" x="{_fmt(half)}"/>',
                f'  <sphere name="ball">\n    <center x="0" y="0" z="0"/>\n    <radius r="{_fmt(radius)}"/>\n  </sphere>']
    cells = ['  <cell name="fuel" material="fuel">\n    <surface name="xlo" sense="+1"/>\n'
             '    <surface name="xhi" sense="-1"/>\n    <surface name="ball" sense="-1"/>\n  </cell>',
             '  <void>\n    <surface name="xlo" sense="-1"/>\n  </void>',
             '  <void>\n    <surface name="xhi" sense="+1"/>\n  </void>',
             '  <void>\n    <surface name="ball" sense="+1"/>\n  </void>']
    return Problem(
        groups=1, nuclides=[fuel], materials=[("fuel", 1.0, [("fuel", 1.0)])], surfaces=surfaces, cells=cells,
        histories=histories, problem=f'keigenvalue inactive="{inactive}" active="{active}"',
        estimators=[current("leak-xhi", "xhi"), current("leak-ball", "ball")], seed=seed)


def two_zone_spheres(histories: int = 100_000, inactive: int = 20, active: int = 50, groups: int = 8,
                     seed: int = 2026) -> Problem:
    """The 8-group two-zone problem (same seeded cross sections as
    ``two_zone_cubes``) in spheres of the cubes' volumes: a fuel sphere of
    radius 18.6 cm inside a reflector sphere of radius 37.2 cm, vacuum
    outside -- geometry the reference's own surfaces describe."""
    rng = np.random.default_rng(seed)
    fuel, _ = mg_data(rng, groups, True)
    refl, _ = mg_data(rng, groups, False)
    fuel.name, refl.name = "fuel", "reflector"
    r_in = (3 * 30.0 ** 3 / (4 * np.pi)) ** (1 / 3)
    r_out = (3 * 60.0 ** 3 / (4 * np.pi)) ** (1 / 3)
    surfaces = [f'  <sphere name="{n}">\n    <center x="0" y="0" z="0"/>\n    <radius r="{_fmt(r)}"/>\n  </sphere>'
                for n, r in (("inner", r_in), ("outer", r_out))]
    cells = ['  <cell name="fuel" material="fuel">\n    <surface name="inner" sense="-1"/>\n  </cell>',
             '  <cell name="reflector" material="reflector">\n    <surface name="inner" sense="+1"/>\n'
             '    <surface name="outer" sense="-1"/>\n  </cell>',
             '  <void>\n    <surface name="outer" sense="+1"/>\n  </void>']
    return Problem(
        groups=groups, nuclides=[fuel, refl],
        materials=[("fuel", 1.0, [("fuel", 1.0)]), ("reflector", 1.0, [("reflector", 1.0)])],
        surfaces=surfaces, cells=cells, histories=histories,
        problem=f'keigenvalue inactive="{inactive}" active="{active}"',
        estimators=[current("leak", "outer", groups)], seed=1)


def sphere_fixed_source(radius: float = 1.0, capture: float = 1.0, histories: int = 1000) -> Problem:
    """Point source in a pure-absorber sphere (the reference's
    point-source-leakage check: leakage = exp(-capture*radius))."""
    nuc = MGNuclide("absorber", capture=np.array([capture]))
    return Problem(
        groups=1, nuclides=[nuc], materials=[("absorber", 1.0, [("absorber", 1.0)])],
        surfaces=[f'  <sphere name="sphere">\n    <center x="0" y="0" z="0"/>\n    <radius r="{_fmt(radius)}"/>\n  </sphere>'],
        cells=['  <cell name="sphere" material="absorber">\n    <surface name="sphere" sense="-1"/>\n  </cell>',
               '  <void>\n    <surface name="sphere" sense="+1"/>\n  </void>'],
        histories=histories, problem="fixedsource", estimators=[current("leakage", "sphere")])


def infinite_medium(c: float = 0.25, capture: float = 0.75, fission: float = 0.0, nubar: float = 1.0,
                    histories: int = 10_000, keig: tuple[int, int] | None = None) -> Problem:
    """Homogeneous sphere of radius 1e10 cm: an infinite one-group medium."""
    nuc = MGNuclide("fissile", capture=np.array([capture]), scatter=np.array([[c]]),
                    fission=np.array([fission]), nubar=np.array([nubar]), chi=np.array([[1.0]]))
    prob = f'keigenvalue inactive="{keig[0]}" active="{keig[1]}"' if keig else "fixedsource"
    return Problem(
        groups=1, nuclides=[nuc], materials=[("fissile", 1.0, [("fissile", 1.0)])],
        surfaces=['  <sphere name="sphere">\n    <center x="0" y="0" z="0"/>\n    <radius r="1e10"/>\n  </sphere>'],
        cells=['  <cell name="sphere" material="fissile">\n    <surface name="sphere" sense="-1"/>\n  </cell>',
               '  <void>\n    <surface name="sphere" sense="+1"/>\n  </void>'],
        histories=histories, problem=prob)


def batch_problems(count: int = 64, seed: int = 7, h_min: int = 10_000, h_max: int = 1_000_000,
                   side_min: float = 10.0, side_max: float = 80.0, inactive: int = 20, active: int = 50):
    """Independent problems of the two-zone form with their own seeded cross
    sections (seeds 0..count-1), outer cube sides log-uniform in
    [side_min, side_max] cm (fuel cube half the side) and histories per cycle
    log-uniform in [h_min, h_max]: a list of (Problem, histories)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        side = float(np.exp(rng.uniform(np.log(side_min), np.log(side_max))))
        hist = int(np.exp(rng.uniform(np.log(h_min), np.log(h_max))))
        p = two_zone_cubes(histories=hist, inactive=inactive, active=active, inner=side / 2, outer=side, seed=i)
        p.estimators = []
        p.seed = 1 + i
        out.append((p, hist))
    return out


def with_sensitivities(xml: str, perts: list[tuple[str, str]]) -> str:
    """Adds total cross-section perturbations (name, nuclide) to a problem
    and, to every current estimator, a sensitivity to each of them."""
    pxml = "<perturbations>\n" + "".join(f'  <total name="{n}" nuclide="{nuc}"/>\n' for n, nuc in perts) + \
        "</perturbations>\n"
    sens = "<sensitivities>" + "".join(f'<perturbation name="{n}"/>' for n, _ in perts) + "</sensitivities>"
    xml = re.sub(r"(<current [^>]*?[^/]>)", rf"\1{sens}", xml)
    xml = re.sub(r"(<current [^>]*?)/>", rf"\1>{sens}</current>", xml)
    return xml.replace("</minimc>", pxml + "</minimc>")
