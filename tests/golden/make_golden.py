"""Regenerate the golden fixtures in this directory from a checkout of the
reference (sanshar/Dice).

Usage: python tests/golden/make_golden.py /path/to/Dice

What is copied, and what it pins:
  * examples/h8_631g: FCIDUMP, dice.dat, the per-iteration table of dice.out
    (determinant counts, energies, Davidson iterations) and the final
    determinant set from the `dets` listing (2470 determinants with weights).
  * tests/SHCI/restart_trev: input2.dat and input3.dat with Treversal 1 on the
    restart FCIDUMP; trusted_hci.e holds E_var of 5e-3 -> 1e-3 -> 1e-4.
  * tests/SHCI/restart: FCIDUMP, input2.dat (io run) and input3.dat (restart);
    trusted_hci.e holds E_var of
    the eps1 schedule 5e-3 -> 1e-3 -> 5e-5.
  * tests/SHCI/n2_RAS: FCIDUMP, input.dat (with an occupation restriction),
    trusted_hci.e (E_var).
  * tests/SHCI/o2_det: FCIDUMP and input.dat (`deterministic`, epsilon2
    1e-7); trusted_hci.e holds E_var + E_PT2 of root 0 (runSmallTests.sh
    tolerance 1e-6).
  * Reduced density matrices: tests/SHCI/H2He_rdm and tests/SHCI/h2co_rdm
    (FCIDUMPs from tests/SHCI/integrals, inputs, PySCF FCI 1- and 2-RDMs,
    runTests.sh tolerances on the error per element), tests/SHCI/o2_stoc
    (input and the reference's own spatial 2-RDM, trusted2RDM.txt).
FCIDUMPs are stored gzip-compressed. Energies and tables go to golden.json.
"""
import gzip
import json
import os
import re
import shutil
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def gz(src, dst):
    with open(src, "rb") as f, open(dst, "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
            shutil.copyfileobj(f, g)


def read_e(path):
    with open(path, "rb") as f:
        return struct.unpack("d", f.read(8))[0]


def det_from_string(fields):
    """Spatial-orbital occupation string ('2','a','b','0') -> two uint64 words
    in the interleaved spin-orbital layout (alpha 2k, beta 2k+1)."""
    w = [0, 0]
    for k, c in enumerate(fields):
        for s, on in ((0, c in ("2", "a")), (1, c in ("2", "b"))):
            if on:
                p = 2 * k + s
                w[p // 64] |= 1 << (p % 64)
    return w


def main(ref):
    out = {}
    # h8 / 6-31G example
    ex = os.path.join(ref, "examples", "h8_631g")
    gz(os.path.join(ex, "FCIDUMP"), os.path.join(HERE, "h8_631g.FCIDUMP.gz"))
    shutil.copy(os.path.join(ex, "dice.dat"), os.path.join(HERE, "h8_631g.dice.dat"))
    table = []
    result = None
    lines = open(os.path.join(ex, "dice.out")).read().splitlines()
    for i, ln in enumerate(lines):
        m = re.match(r"\s*(\d+)\s+(\d+)\s+([0-9.eE+-]+)\s+(\d+)\s+(-?[0-9.]+)\s+(\d+)\s+([0-9.]+)\s*$", ln)
        if m and result is None:
            table.append({"iter": int(m.group(1)), "eps1": float(m.group(3)), "ndets": int(m.group(4)),
                          "energy": float(m.group(5)), "davidson": int(m.group(6))})
        if ln.strip().startswith("Root") and "Energy" in ln:
            result = float(lines[i + 1].split()[1])
    dets, weights = [], []
    for ln in open(os.path.join(ex, "dets")):
        f = ln.split()
        if len(f) < 2:
            continue
        weights.append(float(f[0]))
        dets.append(det_from_string(f[1:]))
    np.savez_compressed(os.path.join(HERE, "h8_631g_dets.npz"),
                        dets=np.array(dets, dtype=np.uint64), weights=np.array(weights))
    out["h8_631g"] = {"table": table, "E_var": result, "ndets": len(dets),
                      "source": "examples/h8_631g/dice.out, examples/h8_631g/dets"}

    # restart fixture
    rs = os.path.join(ref, "tests", "SHCI", "restart")
    gz(os.path.join(rs, "FCIDUMP"), os.path.join(HERE, "restart.FCIDUMP.gz"))
    shutil.copy(os.path.join(rs, "input3.dat"), os.path.join(HERE, "restart.input3.dat"))
    shutil.copy(os.path.join(rs, "input2.dat"), os.path.join(HERE, "restart.input2.dat"))
    out["restart"] = {"E_var": read_e(os.path.join(rs, "trusted_hci.e")), "tol": 5e-5,
                      "source": "tests/SHCI/restart/trusted_hci.e (runTests.sh tolerance 5e-5)"}
    # time-reversal restart fixture (the same FCIDUMP as restart, Treversal 1)
    rt = os.path.join(ref, "tests", "SHCI", "restart_trev")
    shutil.copy(os.path.join(rt, "input2.dat"), os.path.join(HERE, "restart_trev.input2.dat"))
    shutil.copy(os.path.join(rt, "input3.dat"), os.path.join(HERE, "restart_trev.input3.dat"))
    out["restart_trev"] = {"E_var": read_e(os.path.join(rt, "trusted_hci.e")), "tol": 5e-5,
                           "fcidump": "restart.FCIDUMP.gz",
                           "source": "tests/SHCI/restart_trev/trusted_hci.e (runTests.sh tolerance 5e-5)"}

    # n2 with RAS restriction
    n2 = os.path.join(ref, "tests", "SHCI", "n2_RAS")
    gz(os.path.join(n2, "FCIDUMP"), os.path.join(HERE, "n2_RAS.FCIDUMP.gz"))
    shutil.copy(os.path.join(n2, "input.dat"), os.path.join(HERE, "n2_RAS.input.dat"))
    out["n2_RAS"] = {"E_var": read_e(os.path.join(n2, "trusted_hci.e")),
                     "source": "tests/SHCI/n2_RAS/trusted_hci.e"}

    # o2 with deterministic PT
    o2 = os.path.join(ref, "tests", "SHCI", "o2_det")
    gz(os.path.join(o2, "FCIDUMP"), os.path.join(HERE, "o2.FCIDUMP.gz"))
    shutil.copy(os.path.join(o2, "input.dat"), os.path.join(HERE, "o2.input.dat"))
    out["o2_det"] = {"E_total": read_e(os.path.join(o2, "trusted_hci.e")), "tol": 1e-6,
                     "source": "tests/SHCI/o2_det/trusted_hci.e (runSmallTests.sh tolerance 1e-6)"}

    # reduced density matrices: PySCF FCI references (H2He, h2co) and the
    # reference's own 2-RDM output (o2_stoc)
    shci = os.path.join(ref, "tests", "SHCI")
    gz(os.path.join(shci, "integrals", "H2H2_FCIDUMP_nosym"), os.path.join(HERE, "h2he_rdm.FCIDUMP.gz"))
    shutil.copy(os.path.join(shci, "H2He_rdm", "input.dat"), os.path.join(HERE, "h2he_rdm.input.dat"))
    gz(os.path.join(shci, "integrals", "h2co_FCIDUMP_nosymm"), os.path.join(HERE, "h2co_rdm.FCIDUMP.gz"))
    shutil.copy(os.path.join(shci, "h2co_rdm", "test_input.dat"), os.path.join(HERE, "h2co_rdm.input.dat"))
    rdm = {}
    for name, sub in (("h2he_rdm", "H2He_rdm"), ("h2co_rdm", "h2co_rdm")):
        arrays = {k: np.load(os.path.join(shci, sub, "pyscf_%s.npy" % k)) for k in ("1RDM", "2RDM")}
        np.savez_compressed(os.path.join(HERE, name + "_pyscf.npz"), **arrays)
        rdm[name] = {"source": "tests/SHCI/%s/pyscf_1RDM.npy, pyscf_2RDM.npy" % sub}
    rdm["h2he_rdm"]["tol"] = {"1RDM": 1e-9, "2RDM": 1e-9}
    rdm["h2co_rdm"]["tol"] = {"1RDM": 1e-8, "2RDM": 1e-9}
    gz(os.path.join(o2, "FCIDUMP"), os.path.join(HERE, "o2_stoc.FCIDUMP.gz"))
    shutil.copy(os.path.join(shci, "o2_stoc", "input.dat"), os.path.join(HERE, "o2_stoc.input.dat"))
    shutil.copy(os.path.join(shci, "o2_stoc", "trusted2RDM.txt"), os.path.join(HERE, "o2_stoc.trusted2RDM.txt"))
    rdm["o2_stoc"] = {"source": "tests/SHCI/o2_stoc/trusted2RDM.txt", "tol": {"2RDM": 1e-8}}
    out["rdm"] = rdm

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out)[:400])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the reference checkout (sanshar/Dice)>")
    main(sys.argv[1])
