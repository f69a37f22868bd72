"""Speed of the CPU restatement (oracle/mc_oracle.cpp) against the
reference's own transport code (oracle/ref/harness.cpp, the k-eigenvalue
loop over Particle::Transport) on problems the reference can express, at
equal thread counts.  bench.py's reference arm times the restatement (the
reference's sources do not travel to the GPU host), so this ratio says how
its histories/s relate to the reference's own.  Test infrastructure only.

    python -m oracle.ref.calibrate [--threads N]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent.parent
sys.path.insert(0, str(ROOT))


def _ref_lib():
    from oracle.ref import build_ref

    path = build_ref.build()
    if path is None:
        raise SystemExit("the reference's sources are not present")
    lib = C.CDLL(str(path))
    lib.ref_keig.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, C.c_int, C.POINTER(C.c_double),
                             C.POINTER(C.c_uint64), C.c_char_p, C.c_uint64, C.POINTER(C.c_double),
                             C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_char_p, C.c_size_t, C.c_char_p,
                             C.c_size_t]
    lib.ref_keig.restype = C.c_int
    return lib


def time_both(lib, xml: str, cycles: int, threads: int) -> dict:
    from oracle.build import Oracle

    n = int(xml.split("<histories>")[1].split("<")[0])
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "problem.xml"
        path.write_text(xml)
        k = np.zeros(cycles)
        bank = np.zeros(cycles, np.uint64)
        secs = C.c_double()
        lost = C.c_uint64()
        err = C.create_string_buffer(2048)
        rc = lib.ref_keig(str(path).encode(), 1, cycles - 1, threads, k.ctypes.data_as(C.POINTER(C.c_double)),
                          bank.ctypes.data_as(C.POINTER(C.c_uint64)), b"", 0, None, C.byref(secs), C.byref(lost),
                          None, 0, err, 2048)
        if rc != 0:
            raise RuntimeError(err.value.decode())
        o = Oracle(xml, d)
        o.set_quirks(True)
        r = o.run_keigenvalue(n, 1, 1, cycles - 1, threads=threads)
    ref_hps = n * cycles / secs.value
    orc_hps = n * cycles / r["seconds"]
    return {"histories_per_cycle": n, "cycles": cycles, "threads": threads,
            "reference_histories_per_s": ref_hps, "restatement_histories_per_s": orc_hps,
            "restatement_over_reference": orc_hps / ref_hps,
            "same_banks": bool(np.array_equal(bank, r["bank_size"]))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    from minimc_gb300 import synth

    lib = _ref_lib()
    out = {
        "one_group_slab_sphere": time_both(lib, synth.one_group_slab_sphere(histories=20_000).xml(), 10,
                                           args.threads),
        "two_zone_spheres": time_both(lib, synth.two_zone_spheres(histories=100_000).xml(), 4, args.threads),
    }
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
