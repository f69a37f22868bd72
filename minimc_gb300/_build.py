"""In-tree build of the engine's shared library.

Compiles the host C++ (XML parser, problem model) with g++ and the CUDA
sources with nvcc for sm_103a only, in parallel, and links
``minimc_gb300/_lib/libminimc_gb300.so``.  Host code is compiled with
``-ffp-contract=off`` so that table sums are rounded exactly as the reference
(built for x86-64 without FMA) rounds them, on x86 and on Arm alike.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_lib" / "obj"
LIB = OUT_DIR / "libminimc_gb300.so"

HOST_SOURCES = ["mc_xml.cpp", "mc_model.cpp", "mc_ce_tables.cpp", "mc_output.cpp"]
CUDA_SOURCES = ["mc_abi.cu", "mc_transport.cu", "mc_transport_ce.cu", "mc_transport_ce_fx1.cu", "mc_transport_ce_fx2.cu",
                "mc_transport_ce_exact.cu", "mc_transport_ce_ext.cu", "mc_event.cu", "mc_probe.cu", "mc_tsl.cu",
                "mc_mlp.cu", "mc_batch.cu", "mc_pod.cu"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build command failed ({res.returncode}):\n{' '.join(cmd)}\n{res.stdout}")


def compile_commands(extra_nvcc: list[str] | None = None) -> list[tuple[Path, list[str]]]:
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    cmds = []
    for src in HOST_SOURCES:
        obj = OBJ_DIR / (Path(src).stem + ".o")
        cmds.append((obj, ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                           f"-I{INCLUDE}", "-c", str(CSRC / src), "-o", str(obj)]))
    for src in CUDA_SOURCES:
        obj = OBJ_DIR / (Path(src).stem + ".o")
        cmds.append((obj, [nvcc, GENCODE, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
                           "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}",
                           *(extra_nvcc or []), "-c", str(CSRC / src), "-o", str(obj)]))
    return cmds


def build(force: bool = False, verbose: bool = False, extra_nvcc: list[str] | None = None) -> Path:
    """Builds the library if any source changed; returns its path."""
    cmds = compile_commands(extra_nvcc)
    headers = _headers()
    todo = []
    for obj, cmd in cmds:
        src = Path(cmd[cmd.index("-c") + 1])
        if force or _stale(obj, [src, *headers]):
            todo.append(cmd)
    if todo:
        with ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 8, len(todo)))) as ex:
            for cmd in todo:
                if verbose:
                    print(" ".join(cmd), flush=True)
            list(ex.map(_run, todo))
    objs = [obj for obj, _ in cmds]
    if force or todo or _stale(LIB, objs):
        cuda_lib = _cuda_home() / "lib64"
        if not cuda_lib.exists():
            cuda_lib = _cuda_home() / "lib"
        tmp = LIB.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-o", str(tmp), *map(str, objs), f"-L{cuda_lib}", "-lcudart",
              f"-Wl,-rpath,{cuda_lib}"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
