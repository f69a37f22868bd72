"""ctypes binding of the C ABI (include/minimc_gb300.h) and a thin host-side
mirror of minimc's driver interface.

The reference is driven as ``Driver::Create(path)->Solve()``
(src/minimc.cpp:16-21, src/Driver.cpp:18-35), returning an ``EstimatorSet``
whose estimators report ``mean`` and ``std dev`` per bin
(src/Scorable.cpp:51-70).  ``Driver.create`` / ``Driver.solve`` below do the
same through the GPU library; ``World`` exposes the deterministic queries
(``find_cell_containing``, ``nearest_surface``) that the reference's unit
tests exercise.

The library is the CUDA build in ``minimc_gb300/_lib``; there is no CPU
fallback: loading fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libminimc_gb300.so"

MC_OK = 0
ERRORS = {
    -1: "MC_ERR_INPUT", -2: "MC_ERR_OOM", -3: "MC_ERR_DEVICE", -4: "MC_ERR_TIMEOUT",
    -5: "MC_ERR_LOST", -6: "MC_ERR_RESAMPLE", -7: "MC_ERR_STATE", -8: "MC_ERR_OVERFLOW",
    -9: "MC_ERR_EVENT_CAP",
}
RNG_PHILOX, RNG_MINSTD = 0, 1
SCHEDULE_AUTO, SCHEDULE_HISTORY, SCHEDULE_EVENT = 0, 1, 2
TSL_POD, TSL_MLP, TSL_GUIDED = 0, 1, 2
# run option `thermal` (MC_THERMAL_*): inline POD, quantile surrogate on the
# thermal-scatter queue, guided POD-exact sampler on the queue, plain POD on it
THERMAL_POD, THERMAL_SURROGATE, THERMAL_GUIDED, THERMAL_POD_QUEUE = 0, 1, 2, 3
BANK_AUTO, BANK_SLOTS, BANK_DIRECT = 0, 1, 2  # run option `bank_path` (MC_BANK_*)
TSL_PHILOX, TSL_FAST = 0x10, 0x20  # method flags: Philox streams, FP32 POD form
GEOMETRY_ROBUST, GEOMETRY_REFERENCE = 0, 1

# Particle::Event order (src/Particle.hpp:36-44) plus extensions
EVENTS = ["birth", "scatter", "capture", "fission", "surface_cross", "leak", "virtual_collision",
          "reflect", "lost"]


class MCError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code
        self.message = message


class RunOpts(C.Structure):
    _fields_ = [("histories", C.c_uint64), ("seed", C.c_uint64), ("inactive", C.c_uint32),
                ("active", C.c_uint32), ("rng", C.c_int32), ("schedule", C.c_int32),
                ("max_events", C.c_uint32), ("block_size", C.c_int32), ("fast_math", C.c_int32),
                ("variant", C.c_int32), ("thermal", C.c_int32), ("bank_path", C.c_int32),
                ("queue_sort_min", C.c_uint32), ("reserved", C.c_int32 * 3)]


class Site(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("u", C.c_double),
                ("v", C.c_double), ("w", C.c_double), ("energy", C.c_double), ("key", C.c_uint64)]


SITE_DTYPE = np.dtype([("x", "f8"), ("y", "f8"), ("z", "f8"), ("u", "f8"), ("v", "f8"), ("w", "f8"),
                       ("energy", "f8"), ("key", "u8")])


class ProblemInfo(C.Structure):
    _fields_ = [("problem", C.c_int32), ("energy_mode", C.c_int32), ("tracking", C.c_int32),
                ("n_cells", C.c_int32), ("n_surfaces", C.c_int32), ("n_materials", C.c_int32),
                ("n_nuclides", C.c_int32), ("groups", C.c_int32), ("n_estimators", C.c_int32),
                ("n_tsl", C.c_int32), ("histories", C.c_uint64), ("seed", C.c_uint64),
                ("inactive", C.c_uint32), ("active", C.c_uint32), ("total_bins", C.c_uint64),
                ("max_yield", C.c_uint32), ("n_perturbations", C.c_int32), ("reserved", C.c_int32 * 6)]


class EstimatorInfo(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("kind", C.c_int32), ("target", C.c_int32),
                ("offset", C.c_uint64), ("n_bins", C.c_uint64), ("cosine_bins", C.c_uint64),
                ("energy_bins", C.c_uint64), ("n_sensitivities", C.c_int32), ("sensitivity", C.c_int32 * 4),
                ("reserved", C.c_int32)]


class TallyOut(C.Structure):
    _fields_ = [("sum", C.POINTER(C.c_double)), ("sum_sq", C.POINTER(C.c_double)),
                ("history_events", C.POINTER(C.c_uint32)), ("history_fate", C.POINTER(C.c_int8)),
                ("histories", C.c_uint64), ("events", C.c_uint64), ("secondaries", C.c_uint64),
                ("lost", C.c_uint64), ("capped", C.c_uint64), ("overflow", C.c_uint64),
                ("resample_failures", C.c_uint64), ("transport_ms", C.c_double),
                ("launches", C.c_uint64), ("kernel_ms", C.c_double), ("reserved", C.c_double * 3)]


class TrainDesc(C.Structure):
    """mc_train_desc: the surrogate's trained box and training settings."""
    _fields_ = [("E_min", C.c_double), ("E_max", C.c_double), ("T_min", C.c_double), ("T_max", C.c_double),
                ("conditions", C.c_uint64), ("samples_per_condition", C.c_uint32), ("batch", C.c_uint32),
                ("steps", C.c_uint32), ("lr", C.c_float), ("seed", C.c_uint64), ("reserved", C.c_uint64 * 4)]


class TrainOut(C.Structure):
    _fields_ = [("loss_beta", C.c_double), ("loss_alpha", C.c_double), ("data_ms", C.c_double),
                ("train_ms", C.c_double), ("samples", C.c_uint64), ("failures", C.c_uint64),
                ("reserved", C.c_uint64 * 4)]


MLP_PARAMS = 35329  # FP32 parameters per surrogate network


class BatchOpts(C.Structure):
    _fields_ = [("inactive", C.c_uint32), ("active", C.c_uint32), ("fast_math", C.c_int32), ("no_graph", C.c_int32),
                ("variant", C.c_int32), ("max_events", C.c_uint32), ("bank_path", C.c_int32), ("pad", C.c_int32),
                ("reserved", C.c_uint64 * 3)]


class BatchOut(C.Structure):
    _fields_ = [("k_cycle", C.POINTER(C.c_double)), ("k_mean", C.POINTER(C.c_double)),
                ("k_std", C.POINTER(C.c_double)), ("transport_ms", C.c_double), ("tune_ms", C.c_double * 8),
                ("histories", C.c_uint64), ("events", C.c_uint64), ("lost", C.c_uint64), ("capped", C.c_uint64),
                ("overflow", C.c_uint64), ("launches", C.c_uint64), ("variant", C.c_int32), ("graph", C.c_int32),
                ("active_ms", C.c_double), ("reserved", C.c_uint64 * 3)]


class KeigOut(C.Structure):
    _fields_ = [("k_cycle", C.POINTER(C.c_double)), ("bank_size", C.POINTER(C.c_uint64)),
                ("sum", C.POINTER(C.c_double)), ("sum_sq", C.POINTER(C.c_double)),
                ("k_mean", C.c_double), ("k_std", C.c_double), ("k_tracklength_mean", C.c_double),
                ("events", C.c_uint64), ("lost", C.c_uint64), ("capped", C.c_uint64),
                ("overflow", C.c_uint64), ("transport_ms", C.c_double), ("launches", C.c_uint64),
                ("kernel_ms", C.c_double), ("reserved", C.c_double * 3)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_SIGNATURES = {
    "mc_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "mc_destroy": (None, [_P]),
    "mc_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "mc_set_stream": (C.c_int, [_P, _P]),
    "mc_version": (C.c_int, []),
    "mc_load_xml": (C.c_int, [_P, C.c_char_p, C.c_char_p]),
    "mc_problem_info_get": (C.c_int, [_P, C.POINTER(ProblemInfo)]),
    "mc_set_geometry_mode": (C.c_int, [_P, C.c_int32]),
    "mc_estimator_info_get": (C.c_int, [_P, C.c_int32, C.POINTER(EstimatorInfo)]),
    "mc_object_name": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_char_p, C.c_size_t]),
    "mc_run_fixed_source": (C.c_int, [_P, C.POINTER(RunOpts), C.POINTER(TallyOut)]),
    "mc_run_keigenvalue": (C.c_int, [_P, C.POINTER(RunOpts), C.POINTER(KeigOut)]),
    "mc_keig_begin": (C.c_int, [_P, C.POINTER(RunOpts)]),
    "mc_keig_cycle": (C.c_int, [_P, C.c_int32, _D]),
    "mc_keig_cycles": (C.c_int, [_P, C.c_uint32, C.c_int32, _D]),
    "mc_keig_end": (C.c_int, [_P, C.POINTER(KeigOut)]),
    "mc_keig_status": (C.c_int, [_P, C.POINTER(KeigOut)]),
    "mc_keig_checkpoint": (C.c_int, [_P, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "mc_keig_resume": (C.c_int, [_P, C.c_void_p, C.c_uint64]),
    "mc_schedule_info": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32), _D, C.c_int32]),
    "mc_transport_bank": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(RunOpts), _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "mc_transport_bank_noalloc": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(RunOpts), _P, C.c_uint64,
                                            C.POINTER(C.c_uint64)]),
    "mc_tallies_reset": (C.c_int, [_P]),
    "mc_tallies_get": (C.c_int, [_P, _D, _D]),
    "mc_find_cell": (C.c_int, [_P, _D, C.c_uint64, C.POINTER(C.c_int32)]),
    "mc_nearest_surface": (C.c_int, [_P, C.POINTER(C.c_int32), _D, _D, C.c_uint64, C.POINTER(C.c_int32), _D]),
    "mc_surface_distance": (C.c_int, [_P, C.c_int32, _D, _D, C.c_uint64, _D]),
    "mc_surface_contains": (C.c_int, [_P, C.c_int32, _D, C.c_uint64, C.POINTER(C.c_int8)]),
    "mc_material_xs": (C.c_int, [_P, C.c_int32, _D, _D, C.c_uint64, _D, _D]),
    "mc_energy_index": (C.c_int, [_P, C.c_int32, _D, C.c_uint64, C.POINTER(C.c_int64)]),
    "mc_sample_tsl": (C.c_int, [_P, C.c_int32, _D, _D, C.c_uint64, C.c_uint64, C.c_int32, _D, _D,
                                C.POINTER(C.c_uint64)]),
    "mc_sample_tsl_device": (C.c_int, [_P, C.c_int32, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_int32,
                                       C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]),
    "mc_tsl_total": (C.c_int, [_P, C.c_int32, _D, _D, C.c_uint64, _D]),
    "mc_tsl_group_transfer": (C.c_int, [_P, C.c_int32, _D, _D, C.c_uint32, C.c_uint64, _D, C.c_uint32, C.c_uint64,
                                        C.c_int32, _D, C.POINTER(C.c_uint64)]),
    "mc_pod_svd": (C.c_int, [_P, _D, C.c_uint64, C.c_uint64, _D, _D, _D, C.POINTER(C.c_uint32)]),
    "mc_output_text": (C.c_int, [_P, _D, _D, C.c_uint64, C.c_double, C.c_char_p, C.c_size_t,
                                 C.POINTER(C.c_size_t)]),
    "mc_output_format": (C.c_int, [C.c_char_p, C.c_char_p, _D, _D, C.c_uint64, C.c_double, C.c_char_p, C.c_size_t,
                                   C.POINTER(C.c_size_t)]),
    "mc_batch_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "mc_batch_destroy": (None, [_P]),
    "mc_batch_set_stream": (C.c_int, [_P, C.c_void_p]),
    "mc_batch_add": (C.c_int, [_P, C.c_char_p, C.c_char_p, C.c_uint64, C.c_uint64]),
    "mc_batch_run": (C.c_int, [_P, C.POINTER(BatchOpts), C.POINTER(BatchOut)]),
    "mc_batch_last_error": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "mc_train_surrogate": (C.c_int, [_P, C.c_int32, C.POINTER(TrainDesc), C.POINTER(TrainOut)]),
    "mc_train_surrogate_guide": (C.c_int, [_P, C.c_int32, C.POINTER(TrainDesc), C.POINTER(TrainOut)]),
    "mc_surrogate_get": (C.c_int, [_P, _F, _F, C.POINTER(TrainDesc)]),
    "mc_surrogate_set": (C.c_int, [_P, C.c_int32, C.POINTER(TrainDesc), _F, _F]),
    "mc_surrogate_grad": (C.c_int, [_P, _F, _F, _F, C.c_uint64, _F, _F, _F]),
}

_lib = None


def library_path() -> Path:
    return _LIB_PATH


def load_library() -> C.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise RuntimeError(f"minimc_gb300 CUDA library not built: {_LIB_PATH} (run __graft_entry__.build())")
    lib = C.CDLL(str(_LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def format_output(xml_text: str, base_dir, sum, sum_sq, batchsize: int, total_weight: float | None = None) -> str:
    """minimc's result-file text for tallies of the problem in xml_text,
    formatted on the host (mc_output_format; no device needed)."""
    lib = load_library()
    s = _arr(sum, np.float64)
    q = _arr(sum_sq, np.float64)
    w = float(batchsize if total_weight is None else total_weight)
    d = str(base_dir or "").encode()
    need = C.c_size_t()
    rc = lib.mc_output_format(xml_text.encode(), d, _dptr(s), _dptr(q), batchsize, w, None, 0, C.byref(need))
    buf = C.create_string_buffer(need.value + 1)
    rc = lib.mc_output_format(xml_text.encode(), d, _dptr(s), _dptr(q), batchsize, w, buf, need.value + 1,
                              C.byref(need))
    if rc != 0:
        raise MCError(rc, buf.value.decode())
    return buf.value.decode()


# byte offset of the cycle number in a k-eigenvalue checkpoint (after the
# 8-byte magic, five uint64 fields and two uint32 fields)
_CKPT_CYCLE_OFFSET = 8 + 5 * 8 + 2 * 4


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(_F)


def _arr(a, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


class Context:
    """One device context (mc_ctx): owns the device copy of one problem."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = _P()
        rc = self.lib.mc_create(C.byref(h), device)
        if rc != MC_OK:
            raise MCError(rc, "mc_create failed (no usable CUDA device?)")
        self.h = h
        self.info: ProblemInfo | None = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.mc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self) -> str:
        buf = C.create_string_buffer(1024)
        self.lib.mc_last_error(self.h, buf, 1024)
        return buf.value.decode(errors="replace")

    def check(self, rc: int, allow=()):
        if rc != MC_OK and rc not in allow:
            raise MCError(rc, self.error())
        return rc

    def set_stream(self, stream_handle: int):
        self.check(self.lib.mc_set_stream(self.h, _P(stream_handle)))

    def set_geometry_mode(self, mode: int):
        """GEOMETRY_ROBUST (default) or GEOMETRY_REFERENCE (include/minimc_gb300.h)."""
        self.check(self.lib.mc_set_geometry_mode(self.h, mode))

    def load_xml(self, xml_text: str, base_dir: str | os.PathLike | None = None):
        self.check(self.lib.mc_load_xml(self.h, xml_text.encode(), str(base_dir or "").encode()))
        info = ProblemInfo()
        self.check(self.lib.mc_problem_info_get(self.h, C.byref(info)))
        self.info = info
        return info

    def estimators(self) -> list[EstimatorInfo]:
        out = []
        for i in range(self.info.n_estimators):
            e = EstimatorInfo()
            self.check(self.lib.mc_estimator_info_get(self.h, i, C.byref(e)))
            out.append(e)
        return out

    def object_name(self, kind: int, index: int) -> str:
        buf = C.create_string_buffer(256)
        self.check(self.lib.mc_object_name(self.h, kind, index, buf, 256))
        return buf.value.decode()

    # -- solvers -------------------------------------------------------------
    @staticmethod
    def opts(**kw) -> RunOpts:
        o = RunOpts()
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def run_fixed_source(self, per_history: bool = False, allow=(), **kw):
        nb = max(1, self.info.total_bins)
        s = np.zeros(nb)
        s2 = np.zeros(nb)
        out = TallyOut()
        out.sum = _dptr(s)
        out.sum_sq = _dptr(s2)
        n = kw.get("histories") or self.info.histories
        ev = fate = None
        if per_history:
            ev = np.zeros(n, np.uint32)
            fate = np.zeros(n, np.int8)
            out.history_events = ev.ctypes.data_as(C.POINTER(C.c_uint32))
            out.history_fate = fate.ctypes.data_as(C.POINTER(C.c_int8))
        o = self.opts(**kw)
        rc = self.check(self.lib.mc_run_fixed_source(self.h, C.byref(o), C.byref(out)), allow)
        return FixedSourceResult(rc, s[: self.info.total_bins], s2[: self.info.total_bins], out, ev, fate)

    def run_keigenvalue(self, allow=(), **kw):
        o = self.opts(**kw)
        inactive = o.inactive if (o.inactive or o.active) else self.info.inactive
        active = o.active if (o.inactive or o.active) else self.info.active
        ncyc = inactive + active
        k = np.zeros(ncyc)
        bank = np.zeros(ncyc, np.uint64)
        nb = max(1, self.info.total_bins)
        s = np.zeros(nb)
        s2 = np.zeros(nb)
        out = KeigOut()
        out.k_cycle = _dptr(k)
        out.bank_size = bank.ctypes.data_as(C.POINTER(C.c_uint64))
        out.sum = _dptr(s)
        out.sum_sq = _dptr(s2)
        rc = self.check(self.lib.mc_run_keigenvalue(self.h, C.byref(o), C.byref(out)), allow)
        return KeigResult(rc, k, bank, s[: self.info.total_bins], s2[: self.info.total_bins], out,
                          inactive, active)

    def keig_begin(self, **kw):
        o = self.opts(**kw)
        self.check(self.lib.mc_keig_begin(self.h, C.byref(o)))

    def keig_cycle(self, active: bool) -> float:
        k = C.c_double()
        self.check(self.lib.mc_keig_cycle(self.h, int(active), C.byref(k)))
        return k.value

    def keig_cycles(self, n: int, active: bool) -> np.ndarray:
        """n cycles with one synchronisation (mc_keig_cycles): k per cycle."""
        k = np.zeros(max(1, n))
        self.check(self.lib.mc_keig_cycles(self.h, n, int(active), _dptr(k)))
        return k[:n]

    def keig_status(self) -> KeigOut:
        out = KeigOut()
        self.check(self.lib.mc_keig_status(self.h, C.byref(out)))
        return out

    def keig_checkpoint(self) -> bytes:
        """The state of the k-eigenvalue run between cycles (mc_keig_checkpoint)."""
        n = C.c_uint64()
        self.check(self.lib.mc_keig_checkpoint(self.h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self.check(self.lib.mc_keig_checkpoint(self.h, buf, n.value, C.byref(n)))
        return buf.raw[: n.value]

    def keig_resume(self, state: bytes):
        """Continues a run from keig_checkpoint's bytes (replaces keig_begin)."""
        self.check(self.lib.mc_keig_resume(self.h, state, len(state)))

    def run_keigenvalue_checkpointed(self, path, every: int = 1, **kw) -> KeigResult:
        """run_keigenvalue that writes a checkpoint file after every `every`
        cycles and, when `path` already holds one for this problem, resumes
        from it instead of starting over."""
        p = Path(path)
        o = self.opts(**kw)
        inactive = o.inactive if (o.inactive or o.active) else self.info.inactive
        active = o.active if (o.inactive or o.active) else self.info.active
        done = 0
        if p.exists():
            state = p.read_bytes()
            self.keig_resume(state)
            done = int(np.frombuffer(state, np.uint32, count=1, offset=_CKPT_CYCLE_OFFSET)[0])
        else:
            self.keig_begin(**kw)
        ncyc = inactive + active
        for c in range(done, ncyc):
            self.keig_cycle(c >= inactive)
            if (c + 1) % every == 0 and c + 1 < ncyc:
                tmp = p.with_suffix(p.suffix + ".tmp")
                tmp.write_bytes(self.keig_checkpoint())
                os.replace(tmp, p)
        k = np.zeros(ncyc)
        bank = np.zeros(ncyc, np.uint64)
        nb = max(1, self.info.total_bins)
        s, s2 = np.zeros(nb), np.zeros(nb)
        out = KeigOut()
        out.k_cycle = _dptr(k)
        out.bank_size = bank.ctypes.data_as(C.POINTER(C.c_uint64))
        out.sum = _dptr(s)
        out.sum_sq = _dptr(s2)
        self.check(self.lib.mc_keig_end(self.h, C.byref(out)))
        return KeigResult(MC_OK, k, bank, s[: self.info.total_bins], s2[: self.info.total_bins], out,
                          inactive, active)

    def schedule_info(self) -> dict:
        s, v, g, b = (C.c_int32() for _ in range(4))
        t = np.zeros(16)
        self.check(self.lib.mc_schedule_info(self.h, C.byref(s), C.byref(v), C.byref(g), C.byref(b), _dptr(t), 16))
        names = {1: "history", 2: "event"}
        return {"schedule": names.get(s.value, s.value), "variant": v.value, "grid": g.value, "block": b.value,
                "tune_kernel_ms": [round(x, 4) for x in t if x > 0]}

    def keig_end(self) -> KeigOut:
        out = KeigOut()
        self.check(self.lib.mc_keig_end(self.h, C.byref(out)))
        return out

    def transport_bank(self, sites: np.ndarray, cap: int | None = None, **kw):
        """Batched Particle::Transport over a host bank; returns the fission
        sites banked (in source order).  kw: RunOpts fields (rng, fast_math,
        schedule, max_events)."""
        sites = np.ascontiguousarray(sites, dtype=SITE_DTYPE)
        cap = cap if cap is not None else len(sites) * max(1, self.info.max_yield)
        out = np.zeros(cap, SITE_DTYPE)
        n = self.transport_bank_into(sites, out, **kw)
        return out[:n]

    def transport_bank_into(self, sites: np.ndarray, out: np.ndarray, **kw) -> int:
        """Like transport_bank, with caller-owned (e.g. pinned) site arrays;
        returns the number of fission sites written to ``out``."""
        assert sites.dtype == SITE_DTYPE and out.dtype == SITE_DTYPE
        o = self.opts(**kw)
        n_out = C.c_uint64()
        self.check(self.lib.mc_transport_bank(self.h, sites.ctypes.data_as(_P), len(sites), C.byref(o),
                                              out.ctypes.data_as(_P), len(out), C.byref(n_out)))
        return int(n_out.value)

    def transport_bank_noalloc(self, d_sites: int, n: int, d_out: int, cap: int, **kw) -> int:
        """mc_transport_bank_noalloc: device pointers in and out (for callers
        that cannot allocate device memory, e.g. under a memory budget fixed
        at start-up); returns the number of fission sites banked."""
        o = self.opts(**kw)
        n_out = C.c_uint64()
        self.check(self.lib.mc_transport_bank_noalloc(self.h, _P(d_sites), n, C.byref(o), _P(d_out), cap,
                                                      C.byref(n_out)))
        return int(n_out.value)

    def tallies(self):
        nb = max(1, self.info.total_bins)
        s = np.zeros(nb)
        s2 = np.zeros(nb)
        self.check(self.lib.mc_tallies_get(self.h, _dptr(s), _dptr(s2)))
        return s[: self.info.total_bins], s2[: self.info.total_bins]

    def tallies_reset(self):
        self.check(self.lib.mc_tallies_reset(self.h))

    # -- deterministic queries ------------------------------------------------
    def find_cell(self, xyz) -> np.ndarray:
        xyz = _arr(xyz, np.float64).reshape(-1, 3)
        out = np.zeros(len(xyz), np.int32)
        self.check(self.lib.mc_find_cell(self.h, _dptr(xyz), len(xyz), out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def nearest_surface(self, cell, xyz, uvw):
        xyz = _arr(xyz, np.float64).reshape(-1, 3)
        uvw = _arr(uvw, np.float64).reshape(-1, 3)
        cell = _arr(np.broadcast_to(cell, (len(xyz),)), np.int32)
        surf = np.zeros(len(xyz), np.int32)
        dist = np.zeros(len(xyz))
        self.check(self.lib.mc_nearest_surface(self.h, cell.ctypes.data_as(C.POINTER(C.c_int32)), _dptr(xyz),
                                               _dptr(uvw), len(xyz), surf.ctypes.data_as(C.POINTER(C.c_int32)),
                                               _dptr(dist)))
        return surf, dist

    def surface_distance(self, surface: int, xyz, uvw) -> np.ndarray:
        xyz = _arr(xyz, np.float64).reshape(-1, 3)
        uvw = _arr(uvw, np.float64).reshape(-1, 3)
        out = np.zeros(len(xyz))
        self.check(self.lib.mc_surface_distance(self.h, surface, _dptr(xyz), _dptr(uvw), len(xyz), _dptr(out)))
        return out

    def material_xs(self, cell: int, energy, xyz=None) -> tuple[np.ndarray, np.ndarray]:
        """Material::GetMicroscopicTotal / Majorant for neutrons in `cell`
        (energy: group numbers or MeV; xyz: points, for temperature fields)."""
        e = _arr(np.atleast_1d(energy), np.float64)
        tot = np.zeros(len(e))
        maj = np.zeros(len(e))
        xyz = np.zeros((len(e), 3)) if xyz is None else _arr(xyz, np.float64).reshape(-1, 3)
        if len(xyz) != len(e):
            raise ValueError("xyz must hold one point per energy")
        self.check(self.lib.mc_material_xs(self.h, cell, _dptr(xyz), _dptr(e), len(e), _dptr(tot), _dptr(maj)))
        return tot, maj

    def energy_index(self, nuclide: int, energy) -> np.ndarray:
        """std::map::upper_bound position of each energy in each table of a
        continuous-energy nuclide, found through the unionized grid.
        Columns: total, reactions in input order, fission nubar tables;
        -1 past the last table."""
        e = _arr(np.atleast_1d(energy), np.float64)
        out = np.zeros((len(e), 6), np.int64)
        self.check(self.lib.mc_energy_index(self.h, nuclide, _dptr(e), len(e),
                                            out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def output_text(self, sum, sum_sq, batchsize: int, total_weight: float | None = None) -> str:
        """minimc's result-file text (the .out file) for these tallies,
        normalised by total_weight (default: the batch size)."""
        s = _arr(sum, np.float64)
        q = _arr(sum_sq, np.float64)
        w = float(batchsize if total_weight is None else total_weight)
        need = C.c_size_t()
        self.check(self.lib.mc_output_text(self.h, _dptr(s), _dptr(q), batchsize, w, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value + 1)
        self.check(self.lib.mc_output_text(self.h, _dptr(s), _dptr(q), batchsize, w, buf, need.value + 1,
                                           C.byref(need)))
        return buf.value.decode()

    def sample_tsl(self, tsl: int, energy, temperature, seed: int = 1, method: int = TSL_POD):
        """ThermalScattering::SampleBeta then SampleAlpha for each (E, T)
        (host arrays): (beta, alpha, failures)."""
        e = _arr(np.atleast_1d(energy), np.float64)
        t = _arr(np.broadcast_to(temperature, e.shape), np.float64)
        b = np.zeros(len(e))
        a = np.zeros(len(e))
        f = C.c_uint64()
        self.check(self.lib.mc_sample_tsl(self.h, tsl, _dptr(e), _dptr(t), len(e), seed, method, _dptr(b), _dptr(a),
                                          C.byref(f)))
        return b, a, int(f.value)

    def tsl_group_transfer(self, tsl: int, energy, temperature, n: int, bounds, seed: int = 1,
                           method: int = TSL_POD):
        """Multigroup transfer of thermal scatters (mc_tsl_group_transfer):
        for each (E, T) row, the fractions of n sampled outgoing energies
        E' = E + beta k T in each group of `bounds` (MeV, descending); returns
        (probs [rows, groups], failures)."""
        e = _arr(np.atleast_1d(energy), np.float64)
        t = _arr(np.broadcast_to(temperature, e.shape), np.float64)
        b = _arr(np.asarray(bounds), np.float64)
        G = len(b) - 1
        out = np.zeros((len(e), G))
        f = C.c_uint64()
        self.check(self.lib.mc_tsl_group_transfer(self.h, tsl, _dptr(e), _dptr(t), len(e), n, _dptr(b), G, seed,
                                                  method, _dptr(out), C.byref(f)))
        return out, int(f.value)

    def pod_svd(self, M):
        """Thin SVD of a real matrix on the device (mc_pod_svd, FP64,
        one-sided Jacobi): returns (U, S, Vh, sweeps) with M = U diag(S) Vh,
        S descending, U [rows, k], Vh [k, cols], k = min(rows, cols)."""
        M = np.asarray(M, dtype=np.float64)
        if M.ndim != 2 or M.size == 0:
            raise ValueError("pod_svd needs a non-empty 2-D matrix")
        rows, cols = M.shape
        tall = rows >= cols
        # the column-major buffer of A (m >= n): A = M when tall, M^T when wide
        A = _arr(M.T if tall else M, np.float64)
        m, n = (rows, cols) if tall else (cols, rows)
        U = np.zeros(m * n)
        S = np.zeros(n)
        V = np.zeros(n * n)
        sw = C.c_uint32()
        self.check(self.lib.mc_pod_svd(self.h, _dptr(A), m, n, _dptr(U), _dptr(S), _dptr(V), C.byref(sw)))
        Ua = U.reshape(n, m).T  # A's left vectors [m, n]
        Va = V.reshape(n, n).T  # A's right vectors [n, n]
        if tall:
            return Ua, S, Va.T, int(sw.value)
        return Va, S, Ua.T, int(sw.value)

    def sample_tsl_device(self, tsl: int, d_energy: int, d_temperature: int, n: int, d_beta: int, d_alpha: int,
                          seed: int = 1, method: int = TSL_POD) -> int:
        """The sampler on device arrays (raw device addresses); returns the
        failure count."""
        f = C.c_uint64()
        self.check(self.lib.mc_sample_tsl_device(self.h, tsl, C.c_void_p(d_energy), C.c_void_p(d_temperature), n,
                                                 seed, method, C.c_void_p(d_beta), C.c_void_p(d_alpha), C.byref(f)))
        return int(f.value)

    def train_surrogate(self, tsl: int = 0, E_range=(1e-9, 3e-6), T_range=(283.6, 623.6), conditions: int = 0,
                        samples_per_condition: int = 0, batch: int = 0, steps: int = 0, lr: float = 0.0,
                        seed: int = 1) -> TrainOut:
        """Trains the MLP surrogate of thermal library `tsl` on POD samples
        (mc_train_surrogate)."""
        d = TrainDesc(E_min=E_range[0], E_max=E_range[1], T_min=T_range[0], T_max=T_range[1],
                      conditions=conditions, samples_per_condition=samples_per_condition, batch=batch,
                      steps=steps, lr=lr, seed=seed)
        out = TrainOut()
        self.check(self.lib.mc_train_surrogate(self.h, tsl, C.byref(d), C.byref(out)))
        return out

    def train_surrogate_guide(self, tsl: int = 0, E_range=(1e-9, 3e-6), T_range=(283.6, 623.6),
                              conditions: int = 0, samples_per_condition: int = 0, batch: int = 0, steps: int = 0,
                              lr: float = 0.0, seed: int = 1) -> TrainOut:
        """Trains the guide network of the guided (POD-exact) thermal
        sampler of library `tsl` (mc_train_surrogate_guide)."""
        d = TrainDesc(E_min=E_range[0], E_max=E_range[1], T_min=T_range[0], T_max=T_range[1],
                      conditions=conditions, samples_per_condition=samples_per_condition, batch=batch,
                      steps=steps, lr=lr, seed=seed)
        out = TrainOut()
        self.check(self.lib.mc_train_surrogate_guide(self.h, tsl, C.byref(d), C.byref(out)))
        return out

    def surrogate_params(self):
        """(beta params, alpha params, box) of the trained surrogate."""
        b = np.zeros(MLP_PARAMS, np.float32)
        a = np.zeros(MLP_PARAMS, np.float32)
        box = TrainDesc()
        self.check(self.lib.mc_surrogate_get(self.h, _fptr(b), _fptr(a), C.byref(box)))
        return b, a, box

    def set_surrogate(self, tsl: int, box: TrainDesc, beta_params, alpha_params):
        b = _arr(beta_params, np.float32)
        a = _arr(alpha_params, np.float32)
        self.check(self.lib.mc_surrogate_set(self.h, tsl, C.byref(box), _fptr(b), _fptr(a)))

    def surrogate_grad(self, params, x, y):
        """One forward/backward pass: (gradient, loss, outputs)."""
        p = _arr(params, np.float32)
        x = _arr(x, np.float32).reshape(-1, 16)
        y = _arr(y, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        out = np.zeros(len(x), np.float32)
        loss = C.c_float()
        self.check(self.lib.mc_surrogate_grad(self.h, _fptr(p), _fptr(x), _fptr(y), len(x), _fptr(g),
                                              C.cast(C.byref(loss), _F), _fptr(out)))
        return g, float(loss.value), out

    def tsl_total(self, tsl: int, energy, temperature) -> np.ndarray:
        """ThermalScattering::GetTotal at each (E, T)."""
        e = _arr(np.atleast_1d(energy), np.float64)
        t = _arr(np.broadcast_to(temperature, e.shape), np.float64)
        out = np.zeros(len(e))
        self.check(self.lib.mc_tsl_total(self.h, tsl, _dptr(e), _dptr(t), len(e), _dptr(out)))
        return out

    def surface_contains(self, surface: int, xyz) -> np.ndarray:
        xyz = _arr(xyz, np.float64).reshape(-1, 3)
        out = np.zeros(len(xyz), np.int8)
        self.check(self.lib.mc_surface_contains(self.h, surface, _dptr(xyz), len(xyz),
                                                out.ctypes.data_as(C.POINTER(C.c_int8))))
        return out.astype(bool)


@dataclass
class FixedSourceResult:
    status: int
    sum: np.ndarray
    sum_sq: np.ndarray
    raw: TallyOut
    history_events: np.ndarray | None = None
    history_fate: np.ndarray | None = None

    @property
    def histories(self) -> int:
        return int(self.raw.histories)

    def mean(self) -> np.ndarray:
        """Scorable mean: S / N (src/Scorable.cpp:51-58)."""
        return self.sum / self.histories

    def std(self) -> np.ndarray:
        """Scorable std dev: sqrt(S2 - S^2/N) / N (src/Scorable.cpp:59-68)."""
        n = self.histories
        return np.sqrt(np.maximum(self.sum_sq - self.sum * self.sum / n, 0.0)) / n


@dataclass
class KeigResult:
    status: int
    k_cycle: np.ndarray
    bank_size: np.ndarray
    sum: np.ndarray
    sum_sq: np.ndarray
    raw: KeigOut
    inactive: int
    active: int

    @property
    def k_mean(self) -> float:
        return float(self.raw.k_mean)

    @property
    def k_std(self) -> float:
        return float(self.raw.k_std)


class World:
    """Deterministic queries of a loaded problem (World/Cell/CSGSurface)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.cells = [ctx.object_name(0, i) for i in range(ctx.info.n_cells)]
        self.surfaces = [ctx.object_name(1, i) for i in range(ctx.info.n_surfaces)]

    def find_cell_containing(self, point) -> str:
        """World::FindCellContaining (src/World.cpp:26-37)."""
        c = int(self.ctx.find_cell(np.asarray(point, dtype=np.float64).reshape(1, 3))[0])
        if c < 0:
            raise RuntimeError("Point does not belong to any Cell. Please check"
                               "that all space is either assigned a material or void.")
        return self.cells[c]

    def nearest_surface(self, cell: str, point, direction) -> tuple[str, float]:
        """Cell::NearestSurface (src/Cell.cpp:37-51)."""
        ci = self.cells.index(cell)
        s, d = self.ctx.nearest_surface(ci, np.asarray(point, float).reshape(1, 3),
                                        np.asarray(direction, float).reshape(1, 3))
        return self.surfaces[int(s[0])], float(d[0])


class Driver:
    """``Driver::Create(path)`` + ``Solve()`` (src/Driver.cpp:18-35)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.world = World(ctx)

    @classmethod
    def create(cls, xml_path: str | os.PathLike, device: int = 0) -> "Driver":
        p = Path(xml_path)
        ctx = Context(device)
        ctx.load_xml(p.read_text(), p.parent)
        return cls(ctx)

    @classmethod
    def from_text(cls, xml_text: str, base_dir=None, device: int = 0) -> "Driver":
        ctx = Context(device)
        ctx.load_xml(xml_text, base_dir)
        return cls(ctx)

    @property
    def batchsize(self) -> int:
        return int(self.ctx.info.histories)

    def solve(self, **kw):
        if self.ctx.info.problem == 0:
            return self.ctx.run_fixed_source(**kw)
        return self.ctx.run_keigenvalue(**kw)

    def output_text(self, result) -> str:
        """The result file's text (src/minimc.cpp:20-21) for a solve's
        result.  The reference's k-eigenvalue Solve returns its estimators
        untouched (src/KEigenvalue.cpp:36-62); here the active cycles' tallies
        are written, normalised by batch size x active cycles."""
        if isinstance(result, KeigResult):
            w = self.batchsize * result.active
        else:
            w = result.histories
        return self.ctx.output_text(result.sum, result.sum_sq, self.batchsize, w)

    def write_output(self, result, xml_path: str | os.PathLike) -> Path:
        """Writes the result file beside the input, with the extension
        replaced by .out (src/minimc.cpp:16-21); returns its path."""
        out = Path(xml_path).with_suffix(".out")
        out.write_text(self.output_text(result))
        return out

    def estimator_results(self, result) -> dict[str, dict]:
        """Estimator means and std devs by name, normalized per history (fixed
        source: histories; k-eigenvalue: histories per cycle x active cycles)."""
        if isinstance(result, KeigResult):
            n = self.ctx.info.histories * result.active
        else:
            n = result.histories
        out = {}
        for e in self.ctx.estimators():
            # the estimator, then its sensitivities "<estimator>::<perturbation>"
            names = [e.name.decode()] + [e.name.decode() + "::" + self.ctx.object_name(4, e.sensitivity[k])
                                         for k in range(e.n_sensitivities)]
            for k, name in enumerate(names):
                sl = slice(e.offset + k * e.n_bins, e.offset + (k + 1) * e.n_bins)
                s, s2 = result.sum[sl], result.sum_sq[sl]
                out[name] = {
                    "mean": s / n,
                    "std": np.sqrt(np.maximum(s2 - s * s / n, 0.0)) / n,
                    "cosine_bins": int(e.cosine_bins),
                    "energy_bins": int(e.energy_bins),
                }
        return out


class Batch:
    """Many independent multigroup k-eigenvalue problems run together
    (mc_batch_*): one transport launch per cycle for all of them and one
    CUDA graph per cycle."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = _P()
        rc = self.lib.mc_batch_create(C.byref(h), device)
        if rc != MC_OK:
            raise MCError(rc, "mc_batch_create failed")
        self.h = h
        self.histories: list[int] = []

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.mc_batch_destroy(self.h)
            self.h = None

    def error(self) -> str:
        buf = C.create_string_buffer(1024)
        self.lib.mc_batch_last_error(self.h, buf, 1024)
        return buf.value.decode()

    def set_stream(self, stream: int):
        self.lib.mc_batch_set_stream(self.h, C.c_void_p(stream))

    def add(self, xml_text: str, base_dir: str = "", histories: int = 0, seed: int = 0) -> int:
        rc = self.lib.mc_batch_add(self.h, xml_text.encode(), str(base_dir).encode(), histories, seed)
        if rc < 0:
            raise MCError(rc, self.error())
        self.histories.append(histories)
        return rc

    def run(self, inactive: int, active: int, fast_math: int = 1, graph: bool = True, variant: int = 0,
            max_events: int = 0, bank_path: int = BANK_AUTO, allow=()):
        P = len(self.histories)
        ncyc = inactive + active
        k = np.zeros((P, ncyc))
        km = np.zeros(P)
        ks = np.zeros(P)
        o = BatchOpts(inactive=inactive, active=active, fast_math=fast_math, no_graph=0 if graph else 1,
                      variant=variant, max_events=max_events, bank_path=bank_path)
        out = BatchOut()
        out.k_cycle = _dptr(k)
        out.k_mean = _dptr(km)
        out.k_std = _dptr(ks)
        rc = self.lib.mc_batch_run(self.h, C.byref(o), C.byref(out))
        if rc != MC_OK and rc not in allow:
            raise MCError(rc, self.error())
        return {"k_cycle": k, "k_mean": km, "k_std": ks, "transport_ms": out.transport_ms,
                "active_ms": out.active_ms, "histories": out.histories, "events": out.events, "launches": out.launches,
                "variant": out.variant, "graph": out.graph, "tune_ms": list(out.tune_ms), "status": rc}
