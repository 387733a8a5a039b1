"""GPU reduced density matrices (shci_rdm / shci_run_rdm) against the CPU
oracle and the reference's own fixtures, through the C-ABI.

The oracle's restatement of SHCIrdm::EvaluateRDM / EvaluateOneRDM is pinned by
tests/test_oracle_golden.py (PySCF FCI RDMs of H2He and h2co, the reference's
o2_stoc 2-RDM). Here the GPU RDMs of the GPU run are compared with the
oracle's on the same space and coefficients: the GPU sums in 64-bit fixed
point (units of 2^-58, one rounding of at most 2^-59 per term), the oracle in
FP64, so elements agree to 1e-11."""
import json
import os

import numpy as np
import pytest

from dice_gb300 import engine as eng
from dice_gb300 import synthetic
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
G = json.load(open(os.path.join(GOLDEN, "golden.json")))
ATOL = 1e-11


def _run(inp, mode="fp64"):
    e = eng.Engine(0)
    E = e.run_input(inp, mode=mode)
    return e, E


def _err_per_element(a, b):
    return np.linalg.norm(a - b) / a.size


def _read_dice_2rdm(path):
    lines = open(path).read().split("\n")
    n = int(lines[0].split()[0])
    out = np.zeros((n,) * 4)
    for ln in lines[1:]:
        f = ln.split()
        if len(f) == 5:
            out[int(f[0]), int(f[1]), int(f[2]), int(f[3])] = float(f[4])
    return out


@pytest.mark.parametrize("name", ["h2he_rdm", "h2co_rdm"])
def test_gpu_rdms_match_pyscf_fci(golden, name):
    """H2He and h2co end to end on the GPU: spatial 1- and 2-RDMs against
    PySCF's FCI ones at the reference's tolerances; the energy from the
    2-RDM reproduces E_var."""
    inp = golden(name, "input.dat")
    e, E = _run(inp)
    s2, s1 = e.rdm()
    e.close()
    ref = np.load(os.path.join(GOLDEN, name + "_pyscf.npz"))
    tol = G["rdm"][name]["tol"]
    assert _err_per_element(s1, ref["1RDM"]) < tol["1RDM"]
    assert _err_per_element(s2, ref["2RDM"].transpose(0, 2, 1, 3)) < tol["2RDM"]
    o = orc.Oracle(os.path.join(os.path.dirname(inp), "FCIDUMP"))
    assert abs(o.rdm_energy(s2) - E[0]) < 1e-9


def test_gpu_o2_stoc_2rdm_matches_trusted(golden, tmp_path):
    """tests/SHCI/o2_stoc: the reference's spatialRDM.0.0.txt of the
    variational wavefunction, written in the reference's text format and
    compared at its 1e-8 error-per-element tolerance."""
    e, E = _run(golden("o2_stoc", "input.dat"))
    s2, _ = e.rdm()
    e.close()
    path = str(tmp_path / "spatialRDM.0.0.txt")
    eng.write_spatial_rdm(path, s2)
    ours = _read_dice_2rdm(path)
    ref = _read_dice_2rdm(os.path.join(GOLDEN, "o2_stoc.trusted2RDM.txt"))
    assert _err_per_element(ours, ref) < G["rdm"]["o2_stoc"]["tol"]["2RDM"]


@pytest.mark.parametrize("name,sched,mode,extra", [
    ("mol10", [(0, 2e-2)], "fp64", ()),
    ("hubbard12", [(0, 1e-3)], "mixed", ()),
    ("mol24", [(0, 3e-3)], "mixed", ()),
    ("mol10", [(0, 2e-2)], "fp64", ("DirectDavidson",)),
])
def test_gpu_rdm_matches_oracle(tmp_path, name, sched, mode, extra):
    """The GPU run's determinants and coefficients handed to the oracle; the
    stored Hamiltonian's connection lists (mixed or FP64 build, or built for
    the RDM after a matrix-free run) give the oracle's RDMs to 1e-11.
    Repeated calls are bitwise equal."""
    inp = synthetic.make_workload(name, str(tmp_path / "w"), schedule=sched, maxiter=2, extra=extra)
    e, E = _run(inp, mode)
    dets = e.dets()
    ci = e.run_ci(1)[0]
    s2, s1 = e.rdm()
    s2b, s1b = e.rdm(ci)
    e.close()
    assert np.array_equal(s2, s2b) and np.array_equal(s1, s1b)
    o = orc.Oracle(os.path.join(os.path.dirname(inp), "FCIDUMP"))
    r2, r1 = o.rdm(dets, ci)
    print(name, len(dets), np.abs(s2 - r2).max(), np.abs(s1 - r1).max())
    assert np.abs(s2 - r2).max() < ATOL and np.abs(s1 - r1).max() < ATOL
    assert abs(np.trace(s1) - o.nelec) < 1e-9
