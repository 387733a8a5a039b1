"""Time-reversal symmetry (Treversal) on the GPU.

The reference keeps one determinant of every alpha <-> beta flipped pair and
works in the basis (D + t p(D) D~)/sqrt(2) (updateHijForTReversal,
SHCI/Determinants.cpp:32-121; fixForTreversal,
SHCI/SHCImakeHamiltonian.cpp:411-483; the standard-form selection at
SHCI/SHCIbasics.cpp:984-997). That basis spans the t-sector of the flip in the
space holding both members of every pair, so the engine keeps both members,
selects from the standard one with the pair's coefficient, and keeps every
Davidson vector in the sector: the same eigenvalue. Pinned to the reference's
own fixture tests/SHCI/restart_trev (trusted E_var, tolerance 5e-5 in its
test script), run as the reference runs it: input2.dat with io, then
input3.dat resuming from the checkpoint."""
import json
import os

import numpy as np
import pytest

from dice_gb300 import engine as eng

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
G = json.load(open(os.path.join(GOLDEN, "golden.json")))


def _flip(d):
    ev, od = np.uint64(0x5555555555555555), np.uint64(0xAAAAAAAAAAAAAAAA)
    return ((d & ev) << np.uint64(1)) | ((d & od) >> np.uint64(1))


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_restart_trev_fixture_end_to_end(golden, mode):
    first = golden("restart_trev", "input2.dat", fcidump="restart")
    second = golden("restart_trev", "input3.dat", fcidump="restart")
    e = eng.Engine(0)
    e.run_input(first, mode=mode)
    E = e.run_input(second, mode=mode)
    dets = e.dets()
    c = e.run_ci(1)[0]
    e.close()
    print(mode, "E_var", E[0], "trusted", G["restart_trev"]["E_var"], "diff", E[0] - G["restart_trev"]["E_var"])
    assert abs(E[0] - G["restart_trev"]["E_var"]) < G["restart_trev"]["tol"]
    # the space is closed under the flip and the state lies in the Treversal 1
    # sector: c(D~) = p(D) c(D), p the reference's parityOfFlipAlphaBeta
    # (SHCI/Determinants.h:284-297) with 5 beta electrons
    key = {tuple(x): i for i, x in enumerate(dets.tolist())}
    f = _flip(dets)
    idx = np.array([key[tuple(x)] for x in f.tolist()])
    a = dets & np.uint64(0x5555555555555555)
    b = (dets & np.uint64(0xAAAAAAAAAAAAAAAA)) >> np.uint64(1)
    paired = np.array([bin(int(x)).count("1") for x in (a & b)[:, 0]]) + \
        np.array([bin(int(x)).count("1") for x in (a & b)[:, 1]])
    parity = np.where(paired % 2 == 0, 1.0, -1.0) * -1.0  # odd number of beta electrons
    assert np.allclose(c[idx], parity * c, atol=1e-9)


def test_trev_minus_one_is_the_other_sector(tmp_path, golden):
    """Treversal -1 keeps the flip sector in which a closed-shell determinant
    has no component, so it cannot hold this closed-shell system's ground
    state: the run (whose first solve starts at random inside the sector,
    the reference determinant having no component there) converges to a
    state above the plain run's."""
    first = golden("restart_trev", "input2.dat", fcidump="restart")
    text = open(first).read().replace("Treversal 1", "Treversal -1").replace("\nio", "\nnoio")
    minus = os.path.join(os.path.dirname(first), "minus.dat")
    with open(minus, "w") as f:
        f.write(text)
    plain = os.path.join(os.path.dirname(first), "plain.dat")
    with open(plain, "w") as f:
        f.write(text.replace("Treversal -1", ""))
    e = eng.Engine(0)
    Em = e.run_input(minus, mode="fp64")
    Ep = e.run_input(plain, mode="fp64")
    e.close()
    assert np.isfinite(Em[0])
    assert Em[0] > Ep[0] + 1e-3
