"""CPU-side checks of the C-ABI library: it loads without a GPU, exports every
symbol that include/shci_gpu.h declares, and reports the missing device with a
status code instead of crashing."""
import ctypes
import os
import re

import pytest

from dice_gb300 import build as b
from dice_gb300 import engine as eng

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "shci_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void\*|const char\*)\s+(shci_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    b.build()
    return ctypes.CDLL(b.LIB)


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_binding_covers_header():
    bound = {name for name, _, _ in eng.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_no_device_is_a_status_code(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(eng.ShciError) as ei:
        eng.Engine(0)
    assert ei.value.code == 3


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError):
        eng._lib = None
        eng.load_library(str(tmp_path / "nope.so"))
    eng._lib = None
