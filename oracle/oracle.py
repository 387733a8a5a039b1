"""ctypes binding of the CPU oracle (shci_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker the GPU library is compared against.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product (dice_gb300) never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")
CLI = os.path.join(HERE, "_build", "shci_oracle")

_c_double_p = ctypes.POINTER(ctypes.c_double)


def build(force=False):
    """Compile the oracle library and CLI with the Makefile beside this file."""
    if force or not (os.path.exists(LIB) and os.path.exists(CLI)) or \
            os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "shci_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "all"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.orc_load.restype = vp
        L.orc_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, i32]
        L.orc_free.argtypes = [vp]
        L.orc_info.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32), _c_double_p, _c_double_p]
        L.orc_i2_size.restype = i64
        L.orc_i2_size.argtypes = [vp]
        L.orc_i2_export.argtypes = [vp, vp]
        L.orc_i1_export.argtypes = [vp, vp]
        L.orc_hb_size.restype = i64
        L.orc_hb_size.argtypes = [vp, i32]
        L.orc_hb_export.argtypes = [vp, i32, vp, vp, vp, vp]
        L.orc_energy.restype = dbl
        L.orc_energy.argtypes = [vp, vp]
        L.orc_hij.restype = dbl
        L.orc_hij.argtypes = [vp, vp, vp]
        L.orc_select.restype = i64
        L.orc_select.argtypes = [vp, vp, i64, vp, dbl, vp, i64, i32, i32, vp, i32, vp, i64]
        L.orc_ham_build.restype = i64
        L.orc_ham_build.argtypes = [vp, vp, i64]
        L.orc_ham_export.argtypes = [vp, vp, vp, vp]
        L.orc_ham_build_strided.restype = i64
        L.orc_ham_build_strided.argtypes = [vp, vp, i64, i64]
        L.orc_sigma.argtypes = [vp, vp, vp]
        L.orc_sigma_mt.argtypes = [vp, vp, vp, ctypes.c_int]
        L.orc_davidson.restype = i32
        L.orc_davidson.argtypes = [vp, vp, i32, vp, i32, dbl, i32, vp, ctypes.POINTER(i32)]
        L.orc_set_threads.argtypes = [i32]
        L.orc_run_input.restype = i32
        L.orc_run_input.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p, ctypes.c_char_p, i32,
                                    ctypes.c_char_p, i32]
        L.orc_var_nroots.restype = i32
        L.orc_var_nroots.argtypes = [vp]
        L.orc_var_ndets.restype = i64
        L.orc_var_ndets.argtypes = [vp]
        L.orc_var_niters.restype = i32
        L.orc_var_niters.argtypes = [vp]
        L.orc_var_seconds.restype = dbl
        L.orc_var_seconds.argtypes = [vp]
        L.orc_var_nnz_lower.restype = i64
        L.orc_var_nnz_lower.argtypes = [vp]
        L.orc_var_energies.argtypes = [vp, vp]
        L.orc_var_log.argtypes = [vp, vp, vp, vp, vp, vp]
        L.orc_var_dets.argtypes = [vp, vp]
        L.orc_var_ci.argtypes = [vp, i32, vp]
        L.orc_pt_det.restype = dbl
        L.orc_pt_det.argtypes = [vp, vp, i64, vp, dbl, dbl, vp, i32]
        L.orc_pt_det_range.restype = dbl
        L.orc_pt_det_range.argtypes = [vp, vp, i64, vp, dbl, dbl, i64, i64]
        L.orc_rdm.argtypes = [vp, vp, i64, vp, vp, vp]
        L.orc_rdm_eval.argtypes = [vp, vp, vp, vp]
        L.orc_rdm_energy.restype = dbl
        L.orc_rdm_energy.argtypes = [vp, vp]
        L.orc_pt_stoch.restype = dbl
        L.orc_pt_stoch.argtypes = [vp, vp, i64, vp, dbl, dbl, dbl, i32, i32, dbl, ctypes.c_uint64, vp, vp, vp]
        L.orc_var_pt.restype = dbl
        L.orc_var_pt.argtypes = [vp, i32, dbl]
        L.orc_input_epsilon2.restype = dbl
        L.orc_input_epsilon2.argtypes = [vp]
        L.orc_input_deterministic.restype = i32
        L.orc_input_deterministic.argtypes = [vp]
        L.orc_pt_stats.argtypes = [vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _pack_restrictions(restrictions):
    """(min, max, spatial_orbital_list) triples -> int64[n, 4] rows
    (min, max, orbital mask, 0)."""
    r = np.zeros((max(1, len(restrictions)), 4), np.int64)
    for i, (lo, hi, orbs) in enumerate(restrictions):
        m = 0
        for o in orbs:
            m |= 1 << o
        r[i] = (lo, hi, np.uint64(m).view(np.int64) if m >= 2**63 else m, 0)
    return r


def _pt_stats(h):
    c, u, p, o = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
    lib().orc_pt_stats(h, ctypes.byref(c), ctypes.byref(u), ctypes.byref(p), ctypes.byref(o))
    return dict(candidates=c.value, unique=u.value, psi1_norm=p.value, outside=o.value)


class Oracle:
    """Integrals + heat-bath tables read from one FCIDUMP."""

    def __init__(self, fcidump=None, _handle=None):
        L = lib()
        if _handle is not None:
            self.h = _handle
        else:
            err = ctypes.create_string_buffer(512)
            self.h = L.orc_load(fcidump.encode(), err, 512)
            if not self.h:
                raise RuntimeError(err.value.decode())
        n, e = ctypes.c_int(), ctypes.c_int()
        c, m = ctypes.c_double(), ctypes.c_double()
        L.orc_info(self.h, ctypes.byref(n), ctypes.byref(e), ctypes.byref(c), ctypes.byref(m))
        self.norb, self.nelec, self.coreE, self.maxEntry = n.value, e.value, c.value, m.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_free(self.h)
            self.h = None

    def i2(self):
        out = np.zeros(lib().orc_i2_size(self.h), np.float64)
        lib().orc_i2_export(self.h, _p(out))
        return out

    def i1(self):
        out = np.zeros((2 * self.norb) ** 2, np.float64)
        lib().orc_i1_export(self.h, _p(out))
        return out

    def heatbath(self, same):
        L = lib()
        m = L.orc_hb_size(self.h, int(same))
        n = self.norb
        vals = np.zeros(m, np.float32)
        pairs = np.zeros(2 * m, np.int16)
        starts = np.zeros(n * (n + 1) // 2 + 1, np.uint64)
        singles = np.zeros((2 * n) ** 2, np.float64)
        L.orc_hb_export(self.h, int(same), _p(vals), _p(pairs), _p(starts), _p(singles))
        return vals, pairs, starts, singles

    def energy(self, det):
        d = np.ascontiguousarray(det, dtype=np.uint64)
        return lib().orc_energy(self.h, _p(d))

    def hij(self, bra, ket):
        b = np.ascontiguousarray(bra, dtype=np.uint64)
        k = np.ascontiguousarray(ket, dtype=np.uint64)
        return lib().orc_hij(self.h, _p(b), _p(k))

    def select(self, dets, cmax, eps1, existing_sorted, ncore=0, nact=1000000, restrictions=()):
        """restrictions: iterable of (min, max, spatial_orbital_list)."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        cmax = np.ascontiguousarray(cmax, dtype=np.float64)
        ex = np.ascontiguousarray(existing_sorted, dtype=np.uint64)
        r = _pack_restrictions(restrictions)
        cap = 1 << 16
        while True:
            out = np.zeros((cap, 2), np.uint64)
            n = lib().orc_select(self.h, _p(dets), len(dets), _p(cmax), eps1, _p(ex), len(ex), ncore, nact,
                                 _p(r), len(restrictions), _p(out), cap)
            if n <= cap:
                return out[:n]
            cap = n

    def pt_det(self, dets, ci, E0, eps2, restrictions=()):
        """Deterministic PT2 correction E2 for the space `dets` with
        coefficients `ci` (E0 including coreE). Returns (E2, stats) with
        stats = dict(candidates, unique, psi1_norm)."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        ci = np.ascontiguousarray(ci, dtype=np.float64)
        r = _pack_restrictions(restrictions)
        e2 = lib().orc_pt_det(self.h, _p(dets), len(dets), _p(ci), E0, eps2, _p(r), len(restrictions))
        return e2, _pt_stats(self.h)

    def pt_stoch(self, dets, ci, E0, eps2, eps2_large=1000.0, sample_n=200, max_iter=1000000,
                 target_error=1e-4, seed=1):
        """Semistochastic PT2 estimate E2 (E0 including coreE). Returns
        (E2, dict(stddev, iterations, e_large))."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        ci = np.ascontiguousarray(ci, dtype=np.float64)
        sd, el = ctypes.c_double(), ctypes.c_double()
        it = ctypes.c_int()
        e2 = lib().orc_pt_stoch(self.h, _p(dets), len(dets), _p(ci), E0, eps2, eps2_large, sample_n, max_iter,
                                target_error, seed, ctypes.byref(sd), ctypes.byref(it), ctypes.byref(el))
        return e2, dict(stddev=sd.value, iterations=it.value, e_large=el.value)

    def pt_det_range(self, dets, ci, E0, eps2, p0, p1):
        """pt_det with the candidates of parents [p0, p1) only (no
        restrictions), for timing a bounded sample."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        ci = np.ascontiguousarray(ci, dtype=np.float64)
        e2 = lib().orc_pt_det_range(self.h, _p(dets), len(dets), _p(ci), E0, eps2, p0, p1)
        return e2, _pt_stats(self.h)

    def rdm(self, dets, ci):
        """Spatial 2-RDM as an (n, n, n, n) array with [p, q, r, s] = the
        reference's s2RDM(p n + q, r n + s), and the spatial 1-RDM (n, n)."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        ci = np.ascontiguousarray(ci, dtype=np.float64)
        n = self.norb
        s2 = np.zeros((n, n, n, n))
        s1 = np.zeros((n, n))
        lib().orc_rdm(self.h, _p(dets), len(dets), _p(ci), _p(s2), _p(s1))
        return s2, s1

    def rdm_on_ham(self, ci):
        """rdm() on the space of the last ham() call, without rebuilding the
        connection lists."""
        ci = np.ascontiguousarray(ci, dtype=np.float64)
        n = self.norb
        s2 = np.zeros((n, n, n, n))
        s1 = np.zeros((n, n))
        lib().orc_rdm_eval(self.h, _p(ci), _p(s2), _p(s1))
        return s2, s1

    def rdm_energy(self, s2):
        """Energy (core energy included) from a spatial 2-RDM."""
        s2 = np.ascontiguousarray(s2, dtype=np.float64)
        return lib().orc_rdm_energy(self.h, _p(s2))

    def ham(self, dets):
        """Lower-triangle CSR as the reference's SparseHam holds it: row I is
        [I (diagonal), then every J < I connected to I], values in FP64."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        nnz = lib().orc_ham_build(self.h, _p(dets), len(dets))
        rowptr = np.zeros(len(dets) + 1, np.int64)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.float64)
        lib().orc_ham_export(self.h, _p(rowptr), _p(col), _p(val))
        self._n = len(dets)
        return rowptr, col, val

    def ham_rows(self, dets, stride):
        """The lower triangle of the space `dets` for every stride-th row only
        (the other rows empty): a bounded sample of the rows whose
        rank-parallel sigma (sigma_mt) can be timed. Returns the entries kept;
        the CSR stays inside the oracle."""
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        nnz = lib().orc_ham_build_strided(self.h, _p(dets), len(dets), int(stride))
        self._n = len(dets)
        return nnz

    def sigma(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        lib().orc_sigma(self.h, _p(x), _p(y))
        return y

    def sigma_mt(self, x, threads):
        """The reference's rank-parallel Hmult2 with `threads` workers."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        lib().orc_sigma_mt(self.h, _p(x), _p(y), int(threads))
        return y

    def davidson(self, x0, diag, max_copies, tol, direct=False):
        x0 = np.ascontiguousarray(x0, dtype=np.float64).copy()
        nroots = x0.shape[0]
        d = np.ascontiguousarray(diag, dtype=np.float64)
        e = np.zeros(nroots)
        it = ctypes.c_int()
        rc = lib().orc_davidson(self.h, _p(x0), nroots, _p(d), max_copies, tol, int(direct), _p(e),
                                ctypes.byref(it))
        if rc:
            raise RuntimeError("Davidson did not converge")
        return e, x0, it.value


class VarRun:
    """Result of a whole variational stage run by the oracle on an input file."""

    def __init__(self, h):
        self.h = h
        L = lib()
        nr = L.orc_var_nroots(h)
        self.E = np.zeros(nr)
        L.orc_var_energies(h, _p(self.E))
        nd = L.orc_var_ndets(h)
        self.dets = np.zeros((nd, 2), np.uint64)
        L.orc_var_dets(h, _p(self.dets))
        self.ci = np.zeros((nr, nd))
        for r in range(nr):
            row = np.zeros(nd)
            L.orc_var_ci(h, r, _p(row))
            self.ci[r] = row
        ni = L.orc_var_niters(h)
        self.ndets_log = np.zeros(ni, np.int64)
        self.energy_log = np.zeros(ni)
        self.davidson_log = np.zeros(ni, np.int32)
        self.eps1_log = np.zeros(ni)
        self.seconds_log = np.zeros(ni)
        L.orc_var_log(h, _p(self.ndets_log), _p(self.energy_log), _p(self.davidson_log), _p(self.eps1_log),
                      _p(self.seconds_log))
        self.seconds = L.orc_var_seconds(h)
        self.nnz_lower = L.orc_var_nnz_lower(h)
        self.oracle = Oracle(_handle=h)
        self.epsilon2 = L.orc_input_epsilon2(h)
        self.deterministic = bool(L.orc_input_deterministic(h))

    def pt(self, root=0, eps2=-1.0):
        """Deterministic PT2 on this run's space and coefficients (eps2 <= 0:
        the input's epsilon2). Returns (E2, stats)."""
        e2 = lib().orc_var_pt(self.h, root, eps2)
        return e2, _pt_stats(self.h)


def set_threads(threads):
    """Worker threads of the oracle's selection, Hamiltonian rows and sigma
    (1, the default, is the serial restatement the parity tests use)."""
    lib().orc_set_threads(int(threads))


def run_input(input_path, fcidump=None, verbose=False):
    """Run the whole variational stage of a Dice input file on the CPU."""
    h = ctypes.c_void_p()
    err = ctypes.create_string_buffer(512)
    cwd = os.getcwd()
    os.chdir(os.path.dirname(os.path.abspath(input_path)))
    try:
        rc = lib().orc_run_input(ctypes.byref(h), os.path.basename(input_path).encode(),
                                 fcidump.encode() if fcidump else None, int(verbose), err, 512)
    finally:
        os.chdir(cwd)
    if rc:
        raise RuntimeError(err.value.decode())
    return VarRun(h.value)
