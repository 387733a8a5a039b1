"""Seeded synthetic Hamiltonians written as FCIDUMP + Dice input files.

Two families:
  * hubbard_ring: 1-D periodic Hubbard model, U on (ii|ii), hopping -t on
    (i, i+1) including the wrap-around bond, the convention of the
    reference's tests/VMC/hubbard_1x10/makeFCIDUMP.py.
  * molecular: h_pp sorted uniform in [-2, 2]; h_pq (p != q) ~ N(0, 0.05),
    symmetric; (pq|rs) = sum_k L^k_pq L^k_rs with symmetric Cholesky vectors
    L^k_pq ~ N(0, 0.1) * exp(-|p-q|/6). 8-fold symmetric and positive
    semi-definite. Written as unique p>=q, r>=s, pq>=rs.

The numbers are random; no public benchmark data is involved.
"""
import os

import numpy as np

# Workloads: (norb, nalpha, nbeta, cholesky rank, eps1 schedule, nroots)
WORKLOADS = {
    "hubbard12": dict(kind="hubbard", norb=12, nalpha=6, nbeta=6, U=4.0, t=1.0,
                      schedule=[(0, 1e-3), (3, 1e-4)], maxiter=6, nroots=1),
    # final Davidson solve to 1e-6 (loose solves keep the reference's 5e-5), so
    # that E_var comparisons at the 1 uHa level are not dominated by where a
    # solve happened to stop below the reference's default tolerance
    # full CI space of 14,400 determinants: small enough for a brute-force
    # second-order check against the complete Hamiltonian
    "mol10": dict(kind="molecular", norb=10, nalpha=3, nbeta=3, rank=30, seed=20260005,
                  schedule=[(0, 2e-2)], maxiter=3, nroots=1, davidson_tol=1e-8),
    "mol24": dict(kind="molecular", norb=24, nalpha=12, nbeta=12, rank=72, seed=20260001,
                  schedule=[(0, 1e-3), (2, 3e-4), (4, 1e-4)], maxiter=7, nroots=1, davidson_tol=1e-6),
    "mol36": dict(kind="molecular", norb=36, nalpha=14, nbeta=14, rank=108, seed=20260002,
                  schedule=[(0, 1e-3), (2, 1e-4), (4, 3e-5)], maxiter=7, nroots=4),
    "mol50": dict(kind="molecular", norb=50, nalpha=16, nbeta=16, rank=150, seed=20260003,
                  schedule=[(0, 1e-3), (2, 1e-4), (4, 5e-5)], maxiter=7, nroots=1),
    "mol64": dict(kind="molecular", norb=64, nalpha=20, nbeta=20, rank=192, seed=20260004,
                  schedule=[(0, 1e-3), (2, 1e-4), (4, 2e-5)], maxiter=7, nroots=4),
}


def molecular_integrals(norb, rank, seed):
    rng = np.random.default_rng(seed)
    h = rng.normal(0.0, 0.05, size=(norb, norb))
    h = np.triu(h, 1)
    h = h + h.T
    h[np.diag_indices(norb)] = np.sort(rng.uniform(-2.0, 2.0, size=norb))
    p = np.arange(norb)
    decay = np.exp(-np.abs(p[:, None] - p[None, :]) / 6.0)
    L = rng.normal(0.0, 0.1, size=(rank, norb, norb))
    L = np.triu(L)
    L = L + np.transpose(np.triu(L, 1), (0, 2, 1))
    L *= decay[None]
    eri = np.einsum("kpq,krs->pqrs", L, L, optimize=True)
    return h, eri


def hubbard_integrals(norb, U, t):
    h = np.zeros((norb, norb))
    for i in range(norb):
        j = (i + 1) % norb
        h[i, j] = h[j, i] = -t
    eri = np.zeros((norb, norb, norb, norb))
    for i in range(norb):
        eri[i, i, i, i] = U
    return h, eri


def write_fcidump(path, h, eri, nelec, ms2=0, core=0.0, tol=0.0):
    n = h.shape[0]
    lines = [" &FCI NORB=%d,NELEC=%d,MS2=%d," % (n, nelec, ms2),
             "  ORBSYM=" + "1," * n, "  ISYM=1,", " &END"]
    out = []
    for pp in range(n):
        for qq in range(pp + 1):
            pq = pp * (pp + 1) // 2 + qq
            for rr in range(n):
                for ss in range(rr + 1):
                    rs = rr * (rr + 1) // 2 + ss
                    if rs > pq:
                        continue
                    v = eri[pp, qq, rr, ss]
                    if abs(v) > tol:
                        out.append("%.17g %d %d %d %d" % (v, pp + 1, qq + 1, rr + 1, ss + 1))
    for pp in range(n):
        for qq in range(pp + 1):
            v = h[pp, qq]
            if abs(v) > tol:
                out.append("%.17g %d %d 0 0" % (v, pp + 1, qq + 1))
    out.append("%.17g 0 0 0 0" % core)
    with open(path, "w") as f:
        f.write("\n".join(lines + out) + "\n")


def write_input(path, occupied, schedule, maxiter, nroots=1, davidson_tol=5e-5, dE=1e-8, extra=()):
    with open(path, "w") as f:
        f.write("nocc %d\n%s\nend\n" % (len(occupied), " ".join(str(o) for o in occupied)))
        f.write("orbitals FCIDUMP\nnroots %d\n" % nroots)
        f.write("schedule\n")
        for it, e in schedule:
            f.write("%d %g\n" % (it, e))
        f.write("end\n")
        f.write("davidsonTol %g\ndE %g\nmaxiter %d\nnoio\n" % (davidson_tol, dE, maxiter))
        for line in extra:
            f.write(line + "\n")


def reference_occupation(w):
    """Spin-orbital list of the starting determinant. Molecular: the lowest
    nalpha / nbeta orbitals. Hubbard: Neel order (alpha on even sites, beta on
    odd sites)."""
    if w["kind"] == "hubbard":
        return sorted([2 * s for s in range(0, w["norb"], 2)][: w["nalpha"]] +
                      [2 * s + 1 for s in range(1, w["norb"], 2)][: w["nbeta"]])
    return sorted([2 * i for i in range(w["nalpha"])] + [2 * i + 1 for i in range(w["nbeta"])])


def make_workload(name, directory, **overrides):
    """Write FCIDUMP and input.dat for a named workload into `directory`;
    returns the path of input.dat."""
    w = dict(WORKLOADS[name])
    w.update(overrides)
    os.makedirs(directory, exist_ok=True)
    fcidump = os.path.join(directory, "FCIDUMP")
    if w["kind"] == "hubbard":
        h, eri = hubbard_integrals(w["norb"], w["U"], w["t"])
    else:
        h, eri = molecular_integrals(w["norb"], w["rank"], w["seed"])
    write_fcidump(fcidump, h, eri, w["nalpha"] + w["nbeta"], ms2=w["nalpha"] - w["nbeta"])
    inp = os.path.join(directory, "input.dat")
    write_input(inp, reference_occupation(w), w["schedule"], w["maxiter"], nroots=w["nroots"],
                davidson_tol=w.get("davidson_tol", 5e-5), extra=w.get("extra", ()))
    return inp
