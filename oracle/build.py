"""Builds the CPU oracle (TEST INFRASTRUCTURE ONLY).

``oracle/_build/libmc_oracle.so`` = oracle/mc_oracle.cpp (restatement of the
reference's transport path) + the project's XML/model loader.  Used by the
tests, by ``__graft_entry__.smoke()`` as the checker, and by bench.py's CPU
baseline leg; the product never loads it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
OUT = ROOT / "oracle" / "_build" / "libmc_oracle.so"
SOURCES = [ROOT / "oracle" / "mc_oracle.cpp", ROOT / "minimc_gb300" / "csrc" / "mc_xml.cpp",
           ROOT / "minimc_gb300" / "csrc" / "mc_model.cpp"]
HEADERS = list((ROOT / "minimc_gb300" / "csrc").glob("*.hpp"))


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(parents=True, exist_ok=True)
    deps = SOURCES + HEADERS
    if force or not OUT.exists() or any(d.stat().st_mtime > OUT.stat().st_mtime for d in deps):
        tmp = OUT.with_suffix(".tmp.so")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
               f"-I{ROOT / 'minimc_gb300' / 'csrc'}", *map(str, SOURCES), "-o", str(tmp)]
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{res.stdout}")
        tmp.replace(OUT)
    return OUT


class OrcStats(C.Structure):
    _fields_ = [("events", C.c_uint64), ("lost", C.c_uint64), ("capped", C.c_uint64),
                ("secondaries", C.c_uint64), ("seconds", C.c_double), ("k_tracklength", C.c_double),
                ("resample", C.c_uint64)]


_D = C.POINTER(C.c_double)
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t]
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_set_quirks.argtypes = [C.c_void_p, C.c_int]
        lib.orc_total_bins.restype = C.c_uint64
        lib.orc_total_bins.argtypes = [C.c_void_p]
        lib.orc_find_cell.argtypes = [C.c_void_p, _D, C.c_uint64, C.POINTER(C.c_int32)]
        lib.orc_nearest_surface.argtypes = [C.c_void_p, C.POINTER(C.c_int32), _D, _D, C.c_uint64,
                                            C.POINTER(C.c_int32), _D]
        lib.orc_surface_distance.argtypes = [C.c_void_p, C.c_int32, _D, _D, C.c_uint64, _D]
        lib.orc_surface_contains.argtypes = [C.c_void_p, C.c_int32, _D, C.c_uint64, C.POINTER(C.c_int8)]
        lib.orc_philox.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32]
        lib.orc_minstd_canonical.argtypes = [C.c_uint64, C.c_uint64, _D]
        lib.orc_rotate.argtypes = [_D, C.c_double, C.c_double, _D]
        lib.orc_normalize.argtypes = [_D, _D]
        lib.orc_material_total.restype = C.c_double
        lib.orc_material_total.argtypes = [C.c_void_p, C.c_int32, C.c_uint64]
        lib.orc_material_xs_ce.restype = C.c_int
        lib.orc_material_xs_ce.argtypes = [C.c_void_p, C.c_int32, _D, _D, C.c_uint64, _D, _D]
        lib.orc_energy_index.restype = C.c_int
        lib.orc_energy_index.argtypes = [C.c_void_p, C.c_int32, _D, C.c_uint64, C.POINTER(C.c_int64)]
        lib.orc_sample_tsl.restype = C.c_int
        lib.orc_sample_tsl.argtypes = [C.c_void_p, C.c_int32, _D, _D, C.c_uint64, C.c_uint64, _D, _D,
                                       C.POINTER(C.c_uint64)]
        lib.orc_tsl_total.restype = C.c_int
        lib.orc_tsl_total.argtypes = [C.c_void_p, C.c_int32, _D, _D, C.c_uint64, _D]
        lib.orc_set_material_order.restype = C.c_int
        lib.orc_set_material_order.argtypes = [C.c_void_p, C.c_int32, C.c_char_p]
        lib.orc_cell_material.restype = C.c_int32
        lib.orc_cell_material.argtypes = [C.c_void_p, C.c_int32]
        lib.orc_free_gas.argtypes = [C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_uint64, _D, _D]
        lib.orc_run_fixed_source.restype = C.c_int
        lib.orc_run_fixed_source.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int, C.c_uint32, _D, _D,
                                             C.POINTER(C.c_uint32), C.POINTER(C.c_int8), C.POINTER(OrcStats)]
        lib.orc_run_keigenvalue.restype = C.c_int
        lib.orc_run_keigenvalue.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int,
                                            C.c_uint32, _D, C.POINTER(C.c_uint64), _D, _D, C.POINTER(OrcStats)]
        _lib = lib
    return _lib


def _d(a):
    return a.ctypes.data_as(_D)


class Oracle:
    """CPU restatement of the reference path for one problem."""

    def __init__(self, xml_text: str, base_dir: str = ""):
        self.lib = load()
        err = C.create_string_buffer(1024)
        h = self.lib.orc_create(xml_text.encode(), str(base_dir).encode(), err, 1024)
        if not h:
            raise RuntimeError(err.value.decode())
        self.h = h
        self.total_bins = int(self.lib.orc_total_bins(h))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def set_quirks(self, q: bool):
        """True: the reference's exact geometry semantics; False: robust."""
        self.lib.orc_set_quirks(self.h, int(q))

    def material_total(self, cell: int, group: int) -> float:
        return float(self.lib.orc_material_total(self.h, cell, group))

    def set_material_order(self, material: int, names):
        """Iterate the material's nuclides in the given order (see
        orc_set_material_order)."""
        rc = self.lib.orc_set_material_order(self.h, material, " ".join(names).encode())
        if rc != 0:
            raise ValueError(f"set_material_order: {rc}")

    def cell_material(self, cell: int) -> int:
        return int(self.lib.orc_cell_material(self.h, cell))

    def material_xs_ce(self, cell, energy, xyz=None):
        """(total, majorant) microscopic cross sections of a continuous-energy
        material for neutrons of the given energies at the given points."""
        energy = np.ascontiguousarray(energy, np.float64).ravel()
        xyz = np.zeros((len(energy), 3)) if xyz is None else np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        tot = np.zeros(len(energy))
        maj = np.zeros(len(energy))
        if self.lib.orc_material_xs_ce(self.h, cell, _d(energy), _d(xyz), len(energy), _d(tot), _d(maj)) != 0:
            raise ValueError("material_xs_ce: not a continuous-energy cell")
        return tot, maj

    def energy_index(self, nuclide, energy):
        """std::map::upper_bound positions of each energy in the nuclide's
        tables: columns total, reactions in input order, nubar (-1: absent)."""
        energy = np.ascontiguousarray(energy, np.float64).ravel()
        out = np.zeros((len(energy), 6), np.int64)
        if self.lib.orc_energy_index(self.h, nuclide, _d(energy), len(energy),
                                     out.ctypes.data_as(C.POINTER(C.c_int64))) != 0:
            raise ValueError("energy_index: not a continuous-energy problem")
        return out

    def sample_tsl(self, tsl, energy, temperature, seed=1):
        """ThermalScattering::SampleBeta then SampleAlpha for each (E, T),
        sample i on minstd seeded with seed + i: (beta, alpha, failures)."""
        E = np.ascontiguousarray(energy, np.float64).ravel()
        T = np.ascontiguousarray(np.broadcast_to(temperature, E.shape), np.float64)
        b, a = np.zeros(len(E)), np.zeros(len(E))
        f = C.c_uint64()
        if self.lib.orc_sample_tsl(self.h, tsl, _d(E), _d(T), len(E), seed, _d(b), _d(a), C.byref(f)) != 0:
            raise ValueError("no such thermal scattering library")
        return b, a, int(f.value)

    def tsl_total(self, tsl, energy, temperature):
        E = np.ascontiguousarray(energy, np.float64).ravel()
        T = np.ascontiguousarray(np.broadcast_to(temperature, E.shape), np.float64)
        out = np.zeros(len(E))
        if self.lib.orc_tsl_total(self.h, tsl, _d(E), _d(T), len(E), _d(out)) != 0:
            raise ValueError("no such thermal scattering library")
        return out

    def find_cell(self, xyz):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.zeros(len(xyz), np.int32)
        self.lib.orc_find_cell(self.h, _d(xyz), len(xyz), out.ctypes.data_as(C.POINTER(C.c_int32)))
        return out

    def nearest_surface(self, cell, xyz, uvw):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        uvw = np.ascontiguousarray(uvw, np.float64).reshape(-1, 3)
        cell = np.ascontiguousarray(np.broadcast_to(cell, (len(xyz),)), np.int32)
        s = np.zeros(len(xyz), np.int32)
        d = np.zeros(len(xyz))
        self.lib.orc_nearest_surface(self.h, cell.ctypes.data_as(C.POINTER(C.c_int32)), _d(xyz), _d(uvw), len(xyz),
                                     s.ctypes.data_as(C.POINTER(C.c_int32)), _d(d))
        return s, d

    def surface_distance(self, surface, xyz, uvw):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        uvw = np.ascontiguousarray(uvw, np.float64).reshape(-1, 3)
        out = np.zeros(len(xyz))
        self.lib.orc_surface_distance(self.h, surface, _d(xyz), _d(uvw), len(xyz), _d(out))
        return out

    def surface_contains(self, surface, xyz):
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.zeros(len(xyz), np.int8)
        self.lib.orc_surface_contains(self.h, surface, _d(xyz), len(xyz), out.ctypes.data_as(C.POINTER(C.c_int8)))
        return out.astype(bool)

    def run_fixed_source(self, n, seed=1, threads=1, max_events=1000000, per_history=False):
        nb = max(1, self.total_bins)
        s, q = np.zeros(nb), np.zeros(nb)
        ev = np.zeros(n, np.uint32) if per_history else None
        fate = np.zeros(n, np.int8) if per_history else None
        st = OrcStats()
        rc = self.lib.orc_run_fixed_source(
            self.h, n, seed, threads, max_events, _d(s), _d(q),
            ev.ctypes.data_as(C.POINTER(C.c_uint32)) if per_history else None,
            fate.ctypes.data_as(C.POINTER(C.c_int8)) if per_history else None, C.byref(st))
        if rc != 0:
            raise RuntimeError(f"oracle fixed source failed ({rc})")
        return {"sum": s[: self.total_bins], "sum_sq": q[: self.total_bins], "events": st.events,
                "lost": st.lost, "capped": st.capped, "secondaries": st.secondaries, "seconds": st.seconds,
                "resample": st.resample,
                "history_events": ev, "history_fate": fate}

    def run_keigenvalue(self, n, seed, inactive, active, threads=1, max_cycles=0):
        ncyc = inactive + active
        k = np.zeros(ncyc)
        bank = np.zeros(ncyc, np.uint64)
        nb = max(1, self.total_bins)
        s, q = np.zeros(nb), np.zeros(nb)
        st = OrcStats()
        rc = self.lib.orc_run_keigenvalue(self.h, n, seed, inactive, active, threads, max_cycles, _d(k),
                                          bank.ctypes.data_as(C.POINTER(C.c_uint64)), _d(s), _d(q), C.byref(st))
        if rc != 0:
            raise RuntimeError(f"oracle k-eigenvalue failed ({rc})")
        return {"k_cycle": k, "bank_size": bank, "sum": s[: self.total_bins], "sum_sq": q[: self.total_bins],
                "events": st.events, "lost": st.lost, "seconds": st.seconds, "k_tracklength": st.k_tracklength,
                "resample": st.resample}


def philox(counter, key):
    c = (C.c_uint32 * 4)(*counter)
    load().orc_philox(c, key[0], key[1])
    return list(c)


def rotate(d, mu: float, phi: float) -> np.ndarray:
    d = np.ascontiguousarray(d, np.float64)
    out = np.zeros(3)
    load().orc_rotate(_d(d), mu, phi, _d(out))
    return out


def normalize(d) -> np.ndarray:
    d = np.ascontiguousarray(d, np.float64)
    out = np.zeros(3)
    load().orc_normalize(_d(d), _d(out))
    return out


def free_gas(awr: float, T: float, E: float, n: int, seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """Free-gas elastic scattering of n neutrons of energy E (MeV) moving
    along +x off a target of mass ratio awr at T kelvin: (E', mu_lab)."""
    e = np.zeros(n)
    mu = np.zeros(n)
    load().orc_free_gas(awr, T, E, n, seed, _d(e), _d(mu))
    return e, mu


def minstd_canonical(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    load().orc_minstd_canonical(seed, n, _d(out))
    return out
