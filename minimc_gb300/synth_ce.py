"""Seeded continuous-energy nuclear data and problems.

The reference's ENDF tables are Git-LFS pointers that are not present, so
the continuous-energy workload uses synthetic nuclides: on a log-spaced grid
of 5e4 energies from 1e-5 eV to 20 MeV, capture = a/sqrt(E) plus 200
single-level Breit-Wigner (SLBW) resonance peaks (seeded energies, total
widths 0.01-10 eV), elastic = constant potential scattering plus the
resonances' elastic part, and for the fissile nuclide a fission cross
section of the same form with nubar(E) = 2.43 + 0.15 E/MeV.

Tables are written in the project table container (``.mctab``: magic,
level count, each level's axis, then the values), which the engine and the
oracle read where the reference reads a pandas/HDF5 table
(src/HDF5DataSet.hpp:87-148).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

EV = 1e-6  # MeV


def write_table(path: Path, axes: list[np.ndarray], values: np.ndarray) -> None:
    """One pandas-style MultiIndex table: level axes, then values in
    row-major order with level 0 slowest."""
    values = np.ascontiguousarray(values, dtype="<f8").ravel()
    assert values.size == int(np.prod([len(a) for a in axes]))
    with open(path, "wb") as f:
        f.write(b"MCTAB1\0\0")
        f.write(np.uint64(len(axes)).tobytes())
        for a in axes:
            a = np.ascontiguousarray(a, dtype="<f8")
            f.write(np.uint64(a.size).tobytes())
            f.write(a.tobytes())
        f.write(np.uint64(values.size).tobytes())
        f.write(values.tobytes())


def read_table(path: Path) -> tuple[list[np.ndarray], np.ndarray]:
    data = Path(path).read_bytes()
    assert data[:8] == b"MCTAB1\0\0"
    off = 8
    nl = int(np.frombuffer(data, "<u8", 1, off)[0])
    off += 8
    axes = []
    for _ in range(nl):
        n = int(np.frombuffer(data, "<u8", 1, off)[0])
        off += 8
        axes.append(np.frombuffer(data, "<f8", n, off).copy())
        off += 8 * n
    nv = int(np.frombuffer(data, "<u8", 1, off)[0])
    off += 8
    return axes, np.frombuffer(data, "<f8", nv, off).copy()


def energy_grid(n: int = 50_000, lo: float = 1e-5 * EV, hi: float = 20.0) -> np.ndarray:
    return np.geomspace(lo, hi, n)


def slbw(E: np.ndarray, E0: np.ndarray, gamma: np.ndarray, peak: np.ndarray) -> np.ndarray:
    """Sum of SLBW peaks peak * sqrt(E0/E) / (1 + x^2), x = 2 (E - E0) / Gamma."""
    out = np.zeros_like(E)
    for e0, g, p in zip(E0, gamma, peak):
        x = 2 * (E - e0) / g
        out += p * np.sqrt(e0 / E) / (1 + x * x)
    return out


def nuclide_tables(rng: np.random.Generator, E: np.ndarray, capture_1ev: float, potential: float,
                   res_scale: float, fissile: bool) -> dict[str, np.ndarray]:
    n_res = 200
    E0 = np.exp(rng.uniform(np.log(1.0 * EV), np.log(1e5 * EV), n_res))
    gamma = np.exp(rng.uniform(np.log(0.01 * EV), np.log(10 * EV), n_res))
    peak = res_scale * np.exp(rng.uniform(np.log(1.0), np.log(1e3), n_res))
    frac_c = rng.uniform(0.2, 0.8, n_res)  # capture share of each resonance
    shape = slbw(E, E0, gamma, peak)
    shape_c = slbw(E, E0, gamma, peak * frac_c)
    capture = capture_1ev * np.sqrt(EV / E) + shape_c
    elastic = potential + (shape - shape_c) * 0.5
    t = {"capture": capture, "elastic": elastic}
    if fissile:
        fission = 1.5 * capture_1ev * np.sqrt(EV / E) + slbw(E, E0, gamma, peak * (1 - frac_c) * 0.5)
        t["fission"] = fission
        t["nubar"] = 2.43 + 0.15 * E
    t["total"] = t["capture"] + t["elastic"] + t.get("fission", 0.0)
    return t


def write_nuclides(directory: Path, seed: int = 2027, n_grid: int = 50_000) -> dict:
    """Three nuclides (hydrogen-like, oxygen-like, uranium-like) -> file names."""
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(seed)
    E = energy_grid(n_grid)
    specs = [("H1", 0.999167339, 0.332, 20.0, 0.2, False),
             ("O16", 15.8575107, 0.0002, 3.8, 0.5, False),
             ("U235", 233.024791, 98.0, 10.0, 20.0, True)]
    files = {}
    for name, awr, cap, pot, res, fissile in specs:
        t = nuclide_tables(rng, E, cap, pot, res, fissile)
        files[name] = {"awr": awr}
        for key, vals in t.items():
            fname = f"synth-{name}-{key}.mctab"
            write_table(directory / fname, [E], vals)
            files[name][key] = fname
    return files


def write_flat_nuclide(directory: Path, name: str, awr: float, capture: float, scatter: float,
                       fission: float = 0.0, nubar: float = 0.0, total: float | None = None,
                       energies=(1e-11, 20.0)) -> dict:
    """A nuclide with energy-independent cross sections (two-point tables)."""
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    E = np.asarray(energies, dtype=np.float64)
    t = {"capture": capture, "elastic": scatter}
    if fission > 0:
        t["fission"] = fission
        t["nubar"] = nubar
    t["total"] = capture + scatter + fission if total is None else total
    out = {"awr": awr}
    for key, v in t.items():
        fname = f"flat-{name}-{key}.mctab"
        write_table(directory / fname, [E], np.full(len(E), float(v)))
        out[key] = fname
    return out


def energy_current(name: str, surface: str, bins: int = 40, lo: float = -11.0, hi: float = 1.5) -> str:
    """Current estimator on a surface with log-spaced energy bins (10^lo to
    10^hi MeV, plus the two open-ended bins)."""
    return (f'  <current name="{name}" surface="{surface}">\n    <bins>\n      <energy>\n'
            f'        <logspace bins="{bins}" min="{lo!r}" max="{hi!r}"/>\n'
            f"      </energy>\n    </bins>\n  </current>")


def ce_problem_xml(files: dict, histories: int = 1_000_000, inactive: int = 20, active: int = 50,
                   half: float = 20.0, afrac: tuple = (0.6, 0.3, 0.1), energy: float = 2.0,
                   temperature: float = 293.6, keig: bool = True, reflective: bool = True,
                   names: tuple = ("H1", "O16", "U235"), estimators: list[str] | None = None,
                   tracking: str = "surface", temperature_xml: str | None = None,
                   sphere: float | None = None) -> str:
    """Homogeneous mixture of `names` in a box of side 2 * half cm; reflective
    faces make it an infinite medium.  Free-gas elastic scattering at
    `temperature` (or the given <temperature> body).  With `sphere` (a
    radius) the mixture fills a vacuum-bounded sphere instead, a geometry
    the reference's own surfaces describe (its surface is named "sphere")."""
    nucs = []
    for name in names:
        f = files[name]
        s = [f'    <nuclide name="{name}" awr="{f["awr"]!r}">', "      <neutron>",
             f'        <total file="{f["total"]}" temperature="293.6"/>',
             f'        <capture file="{f["capture"]}" temperature="293.6"/>',
             f'        <scatter>\n          <xs file="{f["elastic"]}" temperature="293.6"/>\n        </scatter>']
        if "fission" in f:
            s.append(f'        <fission>\n          <xs file="{f["fission"]}" temperature="293.6"/>\n'
                     f'          <nubar file="{f["nubar"]}" temperature="293.6"/>\n        </fission>')
        s += ["      </neutron>", "    </nuclide>"]
        nucs.append("\n".join(s))
    if sphere is not None:
        return _sphere_problem(nucs, names, afrac, sphere, histories, inactive, active, energy, temperature, keig,
                               estimators, tracking, temperature_xml)
    r = ' reflective="true"' if reflective else ""
    planes = []
    for ax in "xyz":
        planes.append(f'  <plane{ax} name="{ax}lo" {ax}="{-half!r}"{r}/>')
        planes.append(f'  <plane{ax} name="{ax}hi" {ax}="{half!r}"{r}/>')
    cell = ['  <cell name="box" material="mix">'] + [
        f'    <surface name="{ax}lo" sense="+1"/>\n    <surface name="{ax}hi" sense="-1"/>' for ax in "xyz"
    ] + ["  </cell>"]
    voids = []
    if not reflective:
        for ax in "xyz":
            voids.append(f'  <void>\n    <surface name="{ax}lo" sense="-1"/>\n  </void>')
            voids.append(f'  <void>\n    <surface name="{ax}hi" sense="+1"/>\n  </void>')
    src = ('    <position>\n      <constant x="0" y="0" z="0"/>\n    </position>\n'
           '    <direction>\n      <isotropic/>\n    </direction>\n'
           f'    <energy>\n      <constant energy="{energy!r}"/>\n    </energy>\n'
           '    <particletype>\n      <constant type="neutron"/>\n    </particletype>')
    prob = (f'<keigenvalue inactive="{inactive}" active="{active}">\n  <initialsource>\n{src}\n  </initialsource>\n'
            "</keigenvalue>") if keig else f"<fixedsource>\n{src}\n</fixedsource>"
    mats = "\n".join(f'    <nuclide name="{n}" afrac="{float(a)!r}"/>' for n, a in zip(names, afrac))
    est = ("<estimators>\n" + "\n".join(estimators) + "\n</estimators>\n") if estimators else ""
    temp = temperature_xml if temperature_xml else f'  <constant c="{temperature!r}"/>'
    trk = "" if tracking == "surface" else f"  <tracking>{tracking}</tracking>\n"
    return ("<minimc>\n<general>\n  <particles>neutron</particles>\n"
            f"  <histories>{histories}</histories>\n  <threads>1</threads>\n  <chunksize>1000</chunksize>\n"
            f"  <seed>1</seed>\n{trk}</general>\n"
            "<nuclides>\n  <continuous>\n" + "\n".join(nucs) + "\n  </continuous>\n</nuclides>\n"
            f'<materials>\n  <material name="mix" aden="0.1">\n{mats}\n  </material>\n</materials>\n'
            "<surfaces>\n" + "\n".join(planes) + "\n</surfaces>\n"
            "<cells>\n" + "\n".join(cell) + "\n" + "\n".join(voids) + "\n</cells>\n"
            f"<temperature>\n{temp}\n</temperature>\n" + est +
            f"<problemtype>\n{prob}\n</problemtype>\n</minimc>\n")


def _sphere_problem(nucs, names, afrac, radius, histories, inactive, active, energy, temperature, keig, estimators,
                    tracking, temperature_xml) -> str:
    src = ('    <position>\n      <constant x="0" y="0" z="0"/>\n    </position>\n'
           '    <direction>\n      <isotropic/>\n    </direction>\n'
           f'    <energy>\n      <constant energy="{energy!r}"/>\n    </energy>\n'
           '    <particletype>\n      <constant type="neutron"/>\n    </particletype>')
    prob = (f'<keigenvalue inactive="{inactive}" active="{active}">\n  <initialsource>\n{src}\n  </initialsource>\n'
            "</keigenvalue>") if keig else f"<fixedsource>\n{src}\n</fixedsource>"
    mats = "\n".join(f'    <nuclide name="{n}" afrac="{float(a)!r}"/>' for n, a in zip(names, afrac))
    est = ("<estimators>\n" + "\n".join(estimators) + "\n</estimators>\n") if estimators else ""
    temp = temperature_xml if temperature_xml else f'  <constant c="{temperature!r}"/>'
    trk = "" if tracking == "surface" else f"  <tracking>{tracking}</tracking>\n"
    return ("<minimc>\n<general>\n  <particles>neutron</particles>\n"
            f"  <histories>{histories}</histories>\n  <threads>1</threads>\n  <chunksize>1000</chunksize>\n"
            f"  <seed>1</seed>\n{trk}</general>\n"
            "<nuclides>\n  <continuous>\n" + "\n".join(nucs) + "\n  </continuous>\n</nuclides>\n"
            f'<materials>\n  <material name="mix" aden="0.1">\n{mats}\n  </material>\n</materials>\n'
            f'<surfaces>\n  <sphere name="sphere">\n    <center x="0" y="0" z="0"/>\n    <radius r="{radius!r}"/>\n'
            "  </sphere>\n</surfaces>\n"
            '<cells>\n  <cell name="ball" material="mix">\n    <surface name="sphere" sense="-1"/>\n  </cell>\n'
            '  <void>\n    <surface name="sphere" sense="+1"/>\n  </void>\n</cells>\n'
            f"<temperature>\n{temp}\n</temperature>\n" + est +
            f"<problemtype>\n{prob}\n</problemtype>\n</minimc>\n")
