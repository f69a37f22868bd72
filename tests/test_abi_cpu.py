"""CPU tests of the C ABI library: it builds, loads, and exports every entry
point include/minimc_gb300.h declares; calls without a device fail cleanly."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "minimc_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mc_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_library):
    lib = C.CDLL(str(built_library))
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(built_library):
    from minimc_gb300 import engine

    assert set(declared_functions()) == set(engine.exported_symbols())


def test_calls_without_device_fail_cleanly(built_library):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = C.CDLL(str(built_library))
    lib.mc_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    h = C.c_void_p()
    assert lib.mc_create(C.byref(h), 0) == -3  # MC_ERR_DEVICE
    lib.mc_load_xml.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
    assert lib.mc_load_xml(None, b"<minimc/>", b"") == -1  # MC_ERR_INPUT
    assert lib.mc_version() == 1


def test_product_does_not_link_the_oracle(built_library):
    """The CUDA library must not depend on anything under oracle/."""
    data = Path(built_library).read_bytes()
    assert b"orc_" not in data
    assert b"libmc_oracle" not in data
