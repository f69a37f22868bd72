"""The C++ drop-in (include/minimc_gb300_driver.hpp) compiled against the
reference's own Driver (src/Driver.hpp:17-50) with the project's pugixml /
HDF5 stand-ins, linked with the engine library and the reference objects.

GpuFixedSource / GpuKEigenvalue derive from the reference's Driver, so their
construction builds the reference's World, estimators and transport method
from the XML root exactly as FixedSource / KEigenvalue do; CreateGpuDriver
selects between them like Driver::Create (src/Driver.cpp:18-35).  Without a
CUDA device the engine context cannot be created and construction fails
with the engine's message (this container has no GPU; the GPU host has no
reference sources, so the drop-in runs here only up to that point).
"""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"

PROGRAM = r'''
#include "minimc_gb300_driver.hpp"

#include <cstdio>
#include <exception>

int main(int argc, char** argv) {
  for (int i = 1; i < argc; i++) {
    try {
      auto d = minimc_gb300::CreateGpuDriver(argv[i]);
      if (auto* k = dynamic_cast<minimc_gb300::GpuKEigenvalue*>(d.get())) {
        k->Solve();
        std::printf("%s: k %.6f +- %.6f\n", argv[i], k->KMean(), k->KStd());
      }
      else {
        d->Solve();
        std::printf("%s\n", static_cast<minimc_gb300::GpuFixedSource*>(d.get())->ResultText().c_str());
      }
    }
    catch (const std::exception& e) {
      std::printf("%s: error: %s\n", argv[i], e.what());
    }
  }
  return 0;
}
'''


@pytest.fixture(scope="module")
def program(tmp_path_factory, built_library):
    try:
        from oracle.ref import build_ref
    except ImportError:
        pytest.skip("reference build recipe unavailable")
    ref_lib = build_ref.build()
    if ref_lib is None:
        pytest.skip("reference sources are not present")
    d = tmp_path_factory.mktemp("driver")
    src = d / "gpu_driver_main.cpp"
    src.write_text(PROGRAM)
    exe = d / "gpu_driver_main"
    cmd = ["g++", "-std=c++17", "-O1", f"-I{build_ref.REF_SRC}", f"-I{ROOT / 'oracle' / 'ref' / 'shim'}",
           f"-I{ROOT / 'include'}", f"-I{ROOT / 'minimc_gb300' / 'csrc'}", str(src), "-o", str(exe),
           f"-L{Path(ref_lib).parent}", "-lminimc_ref", f"-Wl,-rpath,{Path(ref_lib).parent}",
           f"-L{Path(built_library).parent}", "-lminimc_gb300", f"-Wl,-rpath,{Path(built_library).parent}",
           "-pthread"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return exe


def test_drop_in_compiles_and_fails_cleanly_without_a_device(program, tmp_path):
    import torch

    from minimc_gb300 import synth

    keig = tmp_path / "keig.xml"
    keig.write_text(synth.one_group_slab_sphere(histories=100, inactive=1, active=1).xml())
    fixed = GOLDEN / "point_source_leakage.xml"
    r = subprocess.run([str(program), str(fixed), str(keig)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, cwd=GOLDEN, timeout=120)
    assert r.returncode == 0, r.stdout
    lines = r.stdout.strip().splitlines()
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the runs themselves are checked by the GPU tests")
    assert lines[0] == f"{fixed}: error: minimc_gb300: no usable CUDA device", lines
    assert lines[1] == f"{keig}: error: minimc_gb300: no usable CUDA device", lines


def test_drop_in_reports_input_errors_as_the_reference_does(program, tmp_path):
    """A malformed input fails in the reference's own Driver constructor
    (World, Nuclide) with the reference's message, before the engine."""
    bad = GOLDEN / "error_nonexistent_surface.xml"
    r = subprocess.run([str(program), str(bad)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       cwd=GOLDEN, timeout=120)
    assert r.returncode == 0, r.stdout
    assert "error:" in r.stdout and "no usable CUDA device" not in r.stdout, r.stdout
