"""Files the reference writes for other programs, produced through the C-ABI.

dets.bin (writebestdeterminants, SHCI/SHCI.cpp:465-506): the coefficients are
multiplied by the reference's alpha-beta parity, which the h8_631g example's
own `dets` listing (examples/h8_631g/dets, printed with the same parity) pins:
every determinant's signed weight must match the listing up to the global
sign of the eigenvector."""
import os
import struct

import numpy as np
import pytest

from dice_gb300 import engine as eng

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _read_dets_bin(path):
    raw = open(path, "rb").read()
    num, norb = struct.unpack_from("ii", raw, 0)
    off = 8
    out = []
    for _ in range(num):
        (c,) = struct.unpack_from("d", raw, off)
        s = raw[off + 8: off + 8 + norb].decode()
        out.append((c, s))
        off += 8 + norb
    assert off == len(raw)
    return num, norb, out


def _occ_string(w, norb):
    out = []
    for k in range(norb):
        a = (int(w[(2 * k) // 64]) >> ((2 * k) % 64)) & 1
        b = (int(w[(2 * k + 1) // 64]) >> ((2 * k + 1) % 64)) & 1
        out.append("2" if a and b else "a" if a else "b" if b else "0")
    return "".join(out)


def test_dets_bin_matches_reference_listing(golden):
    inp = golden("h8_631g", "dice.dat")
    with open(inp, "a") as f:
        f.write("\nwritebestdeterminants 2470\n")
    e = eng.Engine(0)
    e.run_input(inp, mode="fp64")
    path = os.path.join(os.path.dirname(inp), "dets.bin")
    num, norb, rows = _read_dets_bin(path)
    e.close()
    assert num == 2470 and norb == 16
    mags = [abs(c) for c, _ in rows]
    assert all(mags[i] >= mags[i + 1] for i in range(len(mags) - 1))
    ref = np.load(os.path.join(GOLDEN, "h8_631g_dets.npz"))
    refw = {_occ_string(w, norb): c for w, c in zip(ref["dets"], ref["weights"])}
    assert set(refw) == {s for _, s in rows}
    ours = {s: c for c, s in rows}
    sign = np.sign(ours[max(refw, key=lambda k: abs(refw[k]))]) * np.sign(refw[max(refw, key=lambda k: abs(refw[k]))])
    # the listing prints 9 significant digits; the coefficients themselves
    # agree with the reference's to 1e-6 relative (tests/test_oracle_golden.py)
    bad = [s for s in refw if abs(sign * ours[s] - refw[s]) > 1e-6 * abs(refw[s]) + 2e-9]
    print("signed weights off the listing:", len(bad))
    assert not bad


def _h8_input(golden, name, schedule, maxiter, extra):
    """The h8 example's input with another schedule, io on and extra keywords."""
    src = golden("h8_631g", "dice.dat")
    text = open(src).read()
    text = text.replace("schedule\n0 1e-6\nend", "schedule\n%s\nend" % schedule)
    text = text.replace("noio", "io").replace("maxiter 12", "maxiter %d" % maxiter)
    assert "io\n" in text and ("maxiter %d" % maxiter) in text
    path = os.path.join(os.path.dirname(src), name)
    with open(path, "w") as f:
        f.write(text + "".join(k + "\n" for k in extra))
    return path


def test_checkpoint_restart_and_fullrestart(golden):
    """io writes the variational result after every iteration
    (writeVariationalResult); restart resumes after the saved iteration, or
    ends at once when the saved iteration already used the final threshold;
    fullrestart reruns the schedule from the saved space
    (SHCI/SHCIbasics.cpp:871-943)."""
    sched = "0 1e-4\n2 1e-6"
    full = _h8_input(golden, "full.dat", sched, 12, ())
    e = eng.Engine(0)
    E_full = e.run_input(full, mode="fp64")[0]
    dets_full = e.dets()
    e.close()
    chk = os.path.join(os.path.dirname(full), "shci_gpu-variational.chk")
    assert os.path.exists(chk)

    # the saved iteration is the converged last one: restart does no iteration
    r = eng.Engine(0)
    E_r = r.run_input(_h8_input(golden, "restart.dat", sched, 12, ("restart",)), mode="fp64")[0]
    assert E_r == E_full
    assert np.array_equal(r.dets(), dets_full)
    assert len(r.run_log()["ndets"]) == 0
    r.close()

    # fullrestart from the converged space: the schedule again from there
    f = eng.Engine(0)
    E_f = f.run_input(_h8_input(golden, "fullrestart.dat", sched, 12, ("fullrestart",)), mode="fp64")[0]
    assert abs(E_f - E_full) < 1e-8
    assert set(map(tuple, f.dets().tolist())) == set(map(tuple, dets_full.tolist()))
    f.close()

    # stop after the two eps1 = 1e-4 iterations, then resume at iteration 2
    t = eng.Engine(0)
    E_t = t.run_input(_h8_input(golden, "truncated.dat", sched, 2, ()), mode="fp64")[0]
    n_t = t.ndets()
    t.close()
    assert E_t > E_full + 1e-6
    g = eng.Engine(0)
    E_g = g.run_input(_h8_input(golden, "resume.dat", sched, 12, ("restart",)), mode="fp64")[0]
    log = g.run_log()
    assert len(log["ndets"]) >= 1 and log["ndets"][0] > n_t
    assert abs(E_g - E_full) < 1e-6
    g.close()
