import gzip
import os
import re
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")
    config.addinivalue_line("markers", "slow: long CPU oracle run")


def golden_case(tmp_path, name, input_name, fcidump=None):
    """Unpack a golden fixture (FCIDUMP + input file) into tmp_path; returns
    the input path. fcidump: the name of another fixture whose FCIDUMP the
    case shares."""
    d = tmp_path / name
    d.mkdir(parents=True, exist_ok=True)
    with gzip.open(os.path.join(GOLDEN, (fcidump or name) + ".FCIDUMP.gz"), "rb") as f, \
            open(d / "FCIDUMP", "wb") as g:
        shutil.copyfileobj(f, g)
    src = os.path.join(GOLDEN, name + "." + input_name)
    text = open(src).read()
    # inputs name their integral file relative to their own directory; the
    # fixture's FCIDUMP sits beside the unpacked input
    text = re.sub(r"(?im)^(\s*orbitals)\s+\S+", r"\1 FCIDUMP", text)
    with open(d / input_name, "w") as f:
        f.write(text)
    return str(d / input_name)


@pytest.fixture
def golden(tmp_path):
    return lambda name, inp, fcidump=None: golden_case(tmp_path, name, inp, fcidump)


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
