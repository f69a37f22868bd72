"""Builds the reference's own transport code into oracle/_ref/ (a test
oracle only; nothing of it ships).

The reference's sources are compiled unmodified where they lie, with
project-written stand-ins on the include path for the third-party headers
it needs (pugixml, the HDF5 C++ API) and a replacement for its one
Xerces-C++ user (XMLDocument.cpp, which only validates the XML schema).
The stand-ins implement the calls the reference makes over the project's
XML DOM and table container.  Needs the reference checkout; skipped (returns
None) where it is absent.  The checkout is found at $MINIMC_REFERENCE, else
in a directory named `reference` beside this repository's root.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF_SRC = Path(os.environ.get("MINIMC_REFERENCE", ROOT.parent / "reference")) / "src"
OUT = ROOT / "oracle" / "_ref"
LIB = OUT / "libminimc_ref.so"
EXCLUDE = {"minimc.cpp", "XMLDocument.cpp"}
# -O3 as the reference's own release build; no contraction, so every
# product and sum rounds as the reference built for x86-64 rounds them
FLAGS = ["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-w", "-DNDEBUG"]


def sources() -> list[Path]:
    own = [HERE / "XMLDocument.cpp", HERE / "harness.cpp", ROOT / "minimc_gb300" / "csrc" / "mc_xml.cpp"]
    return sorted(p for p in REF_SRC.glob("*.cpp") if p.name not in EXCLUDE) + own


def available() -> bool:
    """True where the reference's sources can be read."""
    return REF_SRC.exists()


def build(force: bool = False) -> Path | None:
    if not available():
        return None
    OUT.mkdir(parents=True, exist_ok=True)
    (OUT / "obj").mkdir(exist_ok=True)
    stamp = OUT / "flags.txt"  # objects built with other flags are rebuilt
    if not stamp.exists() or stamp.read_text() != " ".join(FLAGS):
        force = True
    inc = [f"-I{REF_SRC}", f"-I{HERE / 'shim'}", f"-I{ROOT / 'minimc_gb300' / 'csrc'}"]
    headers = list((HERE / "shim").glob("*")) + list(REF_SRC.glob("*.hpp"))
    newest_header = max((h.stat().st_mtime for h in headers), default=0)
    jobs = []
    objs = []
    for src in sources():
        obj = OUT / "obj" / (src.parent.name + "_" + src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_header):
            jobs.append([*FLAGS, *inc, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(" ".join(cmd) + "\n" + r.stdout)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not LIB.exists():
        run(["g++", "-shared", "-o", str(LIB), *map(str, objs), "-pthread"])
    stamp.write_text(" ".join(FLAGS))
    return LIB


if __name__ == "__main__":
    print(build())
