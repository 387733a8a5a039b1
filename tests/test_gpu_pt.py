"""GPU deterministic PT2 (Epstein-Nesbet) against the CPU oracle, through
the C-ABI.

The oracle's restatement of SHCIbasics::DoPerturbativeDeterministic is pinned
by tests/test_oracle_golden.py (o2_det trusted energy; brute-force second-order
sum over a full CI space). Here the GPU path must select the same
perturbative determinants (distinct count and candidate count exactly) and
give E2 to 1e-10 relative: both sum the same FP64 numerators, in a different
order (a tree of block partials on the GPU, a sequential sum on the CPU), and
take E_a from the diagonal formula instead of the incremental one."""
import json
import os
import re

import numpy as np
import pytest

from dice_gb300 import engine as eng
from dice_gb300 import synthetic
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
G = json.load(open(os.path.join(GOLDEN, "golden.json")))

REL = 1e-10


def _gpu_run(inp, mode="fp64"):
    e = eng.Engine(0)
    E = e.run_input(inp, mode=mode)
    return e, E


def _check(e2_gpu, st_gpu, e2_orc, st_orc):
    assert st_gpu["unique"] == st_orc["unique"]
    assert st_gpu["candidates"] == st_orc["outside"]
    assert abs(e2_gpu - e2_orc) <= REL * abs(e2_orc) + 1e-14
    assert abs(st_gpu["psi1_norm"] - st_orc["psi1_norm"]) <= REL * abs(st_orc["psi1_norm"]) + 1e-14


def test_pt_o2_det_matches_trusted(golden):
    """tests/SHCI/o2_det end to end on the GPU: `deterministic`, epsilon2 1e-7;
    E_var + E_PT2 against trusted_hci.e at the reference's tolerance."""
    inp = golden("o2", "input.dat")
    e, E = _gpu_run(inp)
    Ept = e.run_pt()
    st = e.pt_stats()
    e.close()
    assert st["unique"] == 0  # the converged space is closed under H here
    assert abs(Ept[0] - G["o2_det"]["E_total"]) < G["o2_det"]["tol"]


def _restrictions(inp):
    out = []
    for ln in open(inp):
        t = re.split(r"[,\s]+", ln.strip())
        if t and t[0].lower() == "restrict":
            out.append((int(t[1]), int(t[2]), [int(x) for x in t[3:]]))
    return out


@pytest.mark.parametrize("name,sched,eps2,restrict", [
    ("mol10", [(0, 2e-2)], 1e-12, None),
    ("hubbard12", [(0, 1e-3)], 1e-6, None),
    ("mol24", [(0, 3e-3)], 1e-4, None),
    ("mol24", [(0, 3e-3)], 1e-4, "restrict 0 2 16 17 18 19 20 21 22 23"),
])
def test_pt_matches_oracle(tmp_path, name, sched, eps2, restrict):
    """Same variational space and coefficients on both sides (the GPU run's
    determinants and FP64 coefficients are handed to the oracle), so the
    comparison isolates the perturbative stage. The last case limits the
    electrons in orbitals 16-23, which the perturbative candidates obey too."""
    extra = ("epsilon2 %g" % eps2, "deterministic") + ((restrict,) if restrict else ())
    inp = synthetic.make_workload(name, str(tmp_path / "w"), schedule=sched, maxiter=2, extra=extra)
    e, E = _gpu_run(inp)
    dets = e.dets()
    ci = e.run_ci(1)[0]
    Ept = e.run_pt()
    st = e.pt_stats()
    e.close()
    o = orc.Oracle(os.path.join(os.path.dirname(inp), "FCIDUMP"))
    e2o, sto = o.pt_det(dets, ci, E[0], eps2, restrictions=_restrictions(inp))
    print(name, "gpu", Ept[0] - E[0], st, "oracle", e2o, sto)
    assert st["unique"] > 0
    _check(Ept[0] - E[0], st, e2o, sto)


def test_pt_host_coefficients_and_partitions_agree(tmp_path):
    """shci_pt_deterministic with host coefficients equals shci_run_pt; a
    candidate cap that forces several hash partitions gives the same
    determinants and E2 to rounding; repeated calls are bitwise equal."""
    inp = synthetic.make_workload("mol24", str(tmp_path / "w"), schedule=[(0, 3e-3)], maxiter=2,
                                  extra=("epsilon2 1e-4", "deterministic"))
    e, E = _gpu_run(inp)
    ci = e.run_ci(1)[0]
    ref = e.run_pt()[0] - E[0]
    st = e.pt_stats()
    a = e.pt_deterministic(ci, E[0], 1e-4)
    b = e.pt_deterministic(ci, E[0], 1e-4)
    assert a == b
    assert abs(a - ref) <= 4e-16 * abs(E[0])  # run_pt returns E_var + E2
    e.set_pt_batch(st["candidates"] // 5)
    c = e.pt_deterministic(ci, E[0], 1e-4)
    st2 = e.pt_stats()
    e.close()
    assert st["partitions"] == 1 and st2["partitions"] >= 5
    assert st2["unique"] == st["unique"] and st2["candidates"] == st["candidates"]
    assert abs(c - a) <= 1e-12 * abs(a)


def test_pt_with_occupation_restriction(golden):
    """tests/SHCI/n2_RAS (a `restrict` line): the restriction applies to the
    perturbative candidates too (the reference's `restrict` fills both
    lists); GPU against the oracle on the GPU run's space. Within the
    restriction this space is complete, so no candidate survives, while the
    unrestricted oracle finds several hundred."""
    inp = golden("n2_RAS", "input.dat")
    e, E = _gpu_run(inp)
    dets = e.dets()
    ci = e.run_ci(1)[0]
    eps2 = 1e-6
    e2 = e.pt_deterministic(ci, E[0], eps2)
    st = e.pt_stats()
    e.close()
    restr = _restrictions(inp)
    assert restr
    o = orc.Oracle(os.path.join(os.path.dirname(inp), "FCIDUMP"))
    e2o, sto = o.pt_det(dets, ci, E[0], eps2, restrictions=restr)
    e2u, stu = o.pt_det(dets, ci, E[0], eps2)
    print("gpu", e2, st, "oracle", e2o, sto, "unrestricted", e2u, stu["unique"])
    assert stu["unique"] > sto["unique"]
    _check(e2, st, e2o, sto)


def test_pt_multiple_roots(tmp_path):
    """Two roots: shci_run_pt perturbs each root's vector with its own E0."""
    inp = synthetic.make_workload("hubbard12", str(tmp_path / "w"), schedule=[(0, 1e-3)], maxiter=2, nroots=2,
                                  extra=("epsilon2 1e-6", "deterministic"))
    e, E = _gpu_run(inp)
    dets = e.dets()
    ci = e.run_ci(2)
    Ept = e.run_pt()
    e.close()
    o = orc.Oracle(os.path.join(os.path.dirname(inp), "FCIDUMP"))
    assert len(Ept) == 2
    for r in range(2):
        e2o, _ = o.pt_det(dets, ci[r], E[r], 1e-6)
        assert abs((Ept[r] - E[r]) - e2o) <= REL * abs(e2o)


def test_semistochastic_pt_matches_oracle_draw_for_draw(tmp_path):
    """Semistochastic PT on the GPU and in the oracle with the same seed make
    the same draws, so a fixed number of iterations (target 0: no early stop)
    gives the same estimate to 1e-9 relative and the same standard error to
    1e-6 relative; with and without the deterministic part at epsilon2Large."""
    inp = synthetic.make_workload("mol24", str(tmp_path / "w"), schedule=[(0, 3e-3)], maxiter=2)
    e, E = _gpu_run(inp)
    dets = e.dets()
    ci = e.run_ci(1)[0]
    o = orc.Oracle(os.path.join(os.path.dirname(inp), "FCIDUMP"))
    for eL in (1000.0, 1e-3):
        g2, gsd, git = e.pt_semistochastic(ci, E[0], 1e-5, eps2_large=eL, sample_n=100, max_iter=12,
                                           target_error=0.0, seed=11)
        o2, ost = o.pt_stoch(dets, ci, E[0], 1e-5, eps2_large=eL, sample_n=100, max_iter=12, target_error=0.0,
                             seed=11)
        print("eps2Large", eL, "gpu", g2, gsd, git, "oracle", o2, ost)
        assert git == ost["iterations"] == 12
        assert abs(g2 - o2) <= 1e-9 * abs(o2)
        assert abs(gsd - ost["stddev"]) <= 1e-6 * ost["stddev"]
        assert abs(e.pt_error()["e_large"] - ost["e_large"]) <= 1e-10 * abs(ost["e_large"]) + 1e-15
    e.close()


def test_semistochastic_pt_from_input_estimates_deterministic(tmp_path):
    """An input without `deterministic` but with sampleN runs the
    semistochastic PT (the reference's default): its estimate agrees with
    the deterministic PT2 at the same epsilon2 within 4 standard errors, and
    nPTiter 0 skips PT (E = E_var)."""
    extra = ("epsilon2 1e-6", "epsilon2Large 1e-4", "sampleN 50", "targetError 2e-5", "seed 3")
    inp = synthetic.make_workload("mol10", str(tmp_path / "w"), extra=extra)
    e, E = _gpu_run(inp)
    Ept = e.run_pt()
    err = e.pt_error()
    ci = e.run_ci(1)[0]
    ed = e.pt_deterministic(ci, E[0], 1e-6)
    e.close()
    print("semistochastic", Ept[0] - E[0], err, "deterministic", ed)
    assert err["iterations"] >= 5 and err["stddev"] < 2e-5
    assert abs((Ept[0] - E[0]) - ed) < 4 * err["stddev"]
    inp2 = synthetic.make_workload("mol10", str(tmp_path / "w2"), extra=extra + ("nPTiter 0",))
    e, E = _gpu_run(inp2)
    assert e.run_pt()[0] == E[0]
    e.close()
