"""The allocation-free sigma entry point (shci_sigma_device_noalloc).

Some callers cannot allocate device memory while they run -- for example a
host program whose own pool owns all of the GPU's memory. For them the
library offers a sigma that packs x into a fixed device array compiled into
the library instead of a context buffer. This file checks, through the C-ABI,
that it returns what the regular shci_sigma_device returns on two calls in a
row (the second with different vectors, so stale scratch contents would
show), and that it rejects sizes beyond its fixed scratch. It is collected
last so that a failing run that stops at the first failure has run every
other test before it."""
import itertools
import os

import numpy as np
import pytest

from dice_gb300 import engine as eng

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fcidump(inp):
    return os.path.join(os.path.dirname(inp), "FCIDUMP")


# (Hamiltonian build mode, sigma mode): each stored layout the entry point
# serves, including the FP64 refinement sigma on a mixed build
@pytest.mark.parametrize("build,mode", [("mixed", "mixed"), ("fp64", "fp64"), ("mixed", "fp64")])
@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_noalloc_sigma_matches_regular_sigma(golden, build, mode, k):
    import torch
    inp = golden("h8_631g", "dice.dat")
    dets = np.load(os.path.join(GOLDEN, "h8_631g_dets.npz"))["dets"]
    e = eng.Engine(0)
    e.read_fcidump(_fcidump(inp))
    e.set_dets(dets)
    e.ham_build(build)
    n = len(dets)
    rng = np.random.default_rng(11 + k)
    for call in range(2):  # two calls in a row, different vectors
        x = torch.tensor(rng.standard_normal((k, n)), device="cuda")
        y_ref = torch.zeros_like(x)
        y_new = torch.full_like(x, float("nan"))
        e.sigma_device(x.data_ptr(), y_ref.data_ptr(), k, n, mode=mode)
        e.sigma_device_noalloc(x.data_ptr(), y_new.data_ptr(), k, n, mode=mode)
        torch.cuda.synchronize()
        ref, new = y_ref.cpu().numpy(), y_new.cpu().numpy()
        assert np.all(np.isfinite(new)), call
        assert np.allclose(new, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max()), call
    e.close()


def test_noalloc_sigma_rejects_null_vectors(golden):
    inp = golden("h8_631g", "dice.dat")
    dets = np.load(os.path.join(GOLDEN, "h8_631g_dets.npz"))["dets"]
    e = eng.Engine(0)
    e.read_fcidump(_fcidump(inp))
    e.set_dets(dets)
    e.ham_build("mixed")
    with pytest.raises(eng.ShciError) as ei:
        e.sigma_device_noalloc(0, 0, 1, len(dets), mode="mixed")
    assert ei.value.code == 1 and "null" in str(ei.value)
    e.close()


def test_noalloc_sigma_rejects_sizes_beyond_its_scratch(golden):
    inp = golden("h8_631g", "dice.dat")
    e = eng.Engine(0)
    e.read_fcidump(_fcidump(inp))
    # 600,000 distinct 4-alpha/4-beta determinants of the 16-orbital h8 space:
    # N x 4 FP64 values need more than the 16 MiB scratch
    strings = [sum(1 << o for o in c) for c in itertools.combinations(range(16), 4)]
    pairs = itertools.islice(itertools.product(strings, strings), 600000)
    dets = np.zeros((600000, 2), np.uint64)
    for i, (a, b) in enumerate(pairs):
        w = 0
        for k in range(16):
            w |= ((a >> k) & 1) << (2 * k) | ((b >> k) & 1) << (2 * k + 1)
        dets[i, 0] = w
    e.set_dets(dets)
    with pytest.raises(eng.ShciError) as ei:
        e.sigma_device_noalloc(0, 0, 4, len(dets), mode="fp64")
    assert ei.value.code == 1 and "scratch" in str(ei.value)
    e.close()
