"""ctypes binding of libshci_gpu (include/shci_gpu.h).

The Python layer only marshals arrays; every computation runs in the CUDA
library. If the library is missing this module raises instead of falling
back to anything else.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libshci_gpu.so")

MODE_FP64, MODE_MIXED, MODE_DIRECT, MODE_DIRECT_MIXED = 0, 1, 2, 3
MODES = {"fp64": MODE_FP64, "mixed": MODE_MIXED, "direct": MODE_DIRECT, "direct_mixed": MODE_DIRECT_MIXED}

_ERR = {1: "invalid argument", 2: "I/O error", 3: "CUDA error", 4: "out of device memory",
        5: "Davidson did not converge", 6: "device wait timed out", 7: "call out of order"}

# (name, restype, argtypes) of every exported entry point
_vp, _i32, _i64, _dbl, _u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_uint64
_P = ctypes.POINTER
SIGNATURES = [
    ("shci_ctx_create", _i32, [_i32, _P(_vp)]),
    ("shci_ctx_destroy", _i32, [_vp]),
    ("shci_last_error", ctypes.c_char_p, [_vp]),
    ("shci_ctx_stream", _vp, [_vp]),
    ("shci_set_alloc_cap", _i32, [_vp, _u64]),
    ("shci_read_fcidump", _i32, [_vp, ctypes.c_char_p, _P(_i32), _P(_i32), _P(_dbl)]),
    ("shci_heatbath_export", _i32, [_vp, _i32, _P(_i64), _vp, _vp, _vp, _vp]),
    ("shci_set_selection_params", _i32, [_vp, _i32, _i32, _i32, _vp, _vp, _vp]),
    ("shci_dets_set", _i32, [_vp, _vp, _i64]),
    ("shci_dets_count", _i32, [_vp, _P(_i64)]),
    ("shci_dets_get", _i32, [_vp, _vp, _i64]),
    ("shci_select", _i32, [_vp, _vp, _dbl, _P(_i64)]),
    ("shci_ham_build", _i32, [_vp, _i32, _P(_i64)]),
    ("shci_ham_build_rows", _i32, [_vp, _i32, _i64, _i64, _P(_i64)]),
    ("shci_select_candidates", _i32, [_vp, _vp, _dbl, _i32, _i32, _P(_i64)]),
    ("shci_candidates_get", _i32, [_vp, _vp, _i64]),
    ("shci_dets_append", _i32, [_vp, _vp, _i64]),
    ("shci_ham_export", _i32, [_vp, _vp, _vp, _vp]),
    ("shci_diag", _i32, [_vp, _vp]),
    ("shci_sigma", _i32, [_vp, _i32, _vp, _vp, _i32]),
    ("shci_sigma_device", _i32, [_vp, _i32, _vp, _vp, _i32, _i64]),
    ("shci_sigma_packed_device", _i32, [_vp, _i32, _vp, _i32, _i32, _vp, _i64]),
    ("shci_sigma_device_noalloc", _i32, [_vp, _i32, _vp, _vp, _i32, _i64]),
    ("shci_ham_bytes", _i32, [_vp, _P(_i64), _P(_i64)]),
    ("shci_sigma_bytes", _i32, [_vp, _i32, _i32, _P(_i64)]),
    ("shci_davidson", _i32, [_vp, _i32, _i32, _i32, _vp, _i32, _dbl, _vp, _P(_i32)]),
    ("shci_run_input", _i32, [_vp, ctypes.c_char_p, ctypes.c_char_p, _i32, _i32, _vp, _i32, _P(_i32)]),
    ("shci_run_log", _i32, [_vp, _i32, _P(_i32), _vp, _vp, _vp, _vp]),
    ("shci_run_ci", _i32, [_vp, _vp, _i64]),
    ("shci_run_timings", _i32, [_vp, _P(_dbl), _P(_dbl), _P(_dbl), _P(_dbl), _P(_i64), _P(_dbl)]),
    ("shci_set_preconditioner", _i32, [_vp, _i32]),
    ("shci_set_davidson_basis", _i32, [_vp, _i32, _i32]),
    ("shci_set_davidson_graphs", _i32, [_vp, _i32]),
    ("shci_fcidump_info", _i32, [ctypes.c_char_p, _P(_i32), _P(_i32), _P(_dbl), _P(_i64)]),
    ("shci_input_info", _i32, [ctypes.c_char_p, _vp, _i32, _P(_i32), _vp, _vp]),
    ("shci_pt2_shift", _i32, [_vp, _dbl, _vp]),
    ("shci_mlp_configure", _i32, [_vp, _i32, _i32, ctypes.c_float, _i64]),
    ("shci_mlp_train", _i32, [_vp, _dbl, _P(ctypes.c_float)]),
    ("shci_mlp_predict", _i32, [_vp, _dbl, _vp]),
    ("shci_mlp_params", _i32, [_vp, _vp, _i32, _P(_i32), _P(_dbl)]),
    ("shci_mlp_set_params", _i32, [_vp, _vp, _i32, _dbl]),
    ("shci_mlp_gradient", _i32, [_vp, _vp, _vp, _i32, _dbl, _vp, _P(ctypes.c_float)]),
    ("shci_run_stats", _i32, [_vp, _P(_i64), _P(_dbl), _P(ctypes.c_float)]),
    ("shci_pt_deterministic", _i32, [_vp, _vp, _dbl, _dbl, _P(_dbl)]),
    ("shci_run_pt", _i32, [_vp, _dbl, _vp, _i32, _P(_i32)]),
    ("shci_pt_stats", _i32, [_vp, _P(_i64), _P(_i64), _P(_i32), _P(_dbl), _P(_dbl)]),
    ("shci_set_pt_batch", _i32, [_vp, _i64]),
    ("shci_pt_semistochastic", _i32, [_vp, _vp, _dbl, _dbl, _dbl, _i32, _i32, _dbl, _u64, _P(_dbl), _P(_dbl),
                                      _P(_i32)]),
    ("shci_pt_error", _i32, [_vp, _P(_dbl), _P(_i32), _P(_dbl)]),
    ("shci_ints_info", _i32, [_vp, _P(_i32), _P(_i32), _P(_dbl)]),
    ("shci_rdm", _i32, [_vp, _vp, _vp, _vp]),
    ("shci_write_best_dets", _i32, [_vp, _i32, _i32, ctypes.c_char_p]),
    ("shci_run_rdm", _i32, [_vp, _i32, _vp, _vp]),
    ("shci_launch_count", _i32, [_vp, _P(_i64)]),
]

_lib = None


def write_spatial_rdm(path, s2):
    """The reference's spatialRDM text format (SHCI/SHCIrdm.cpp:478-510):
    n, then `p q r s value` for |value| > 1e-15."""
    n = s2.shape[0]
    with open(path, "w") as f:
        f.write("%d\n" % n)
        for idx in zip(*np.nonzero(np.abs(s2) > 1e-15)):
            f.write("%3d   %3d   %3d   %3d   %16.12g\n" % (tuple(int(i) for i in idx) + (s2[idx],)))


def write_spatial_1rdm(path, s1):
    """The reference's spatial1RDM text format (SHCI/SHCIrdm.cpp:356-385)."""
    n = s1.shape[0]
    with open(path, "w") as f:
        f.write("%d\n" % n)
        for idx in zip(*np.nonzero(np.abs(s1) > 1e-15)):
            f.write("%3d   %3d   %16.12g\n" % (tuple(int(i) for i in idx) + (s1[idx],)))


def load_library(path=LIB_PATH):
    """Load libshci_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("libshci_gpu.so not built: run `python -m dice_gb300.build` "
                               "(or __graft_entry__.build())")
        L = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class ShciError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d): %s" % (_ERR.get(code, "error"), code, msg))
        self.code = code


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _host_check(rc):
    if rc:
        raise ShciError(rc, load_library().shci_last_error(None).decode())


def fcidump_info(path):
    """Parse an FCIDUMP on the host only (no device): (norb, nelec, coreE,
    number of distinct nonzero two-electron integrals)."""
    norb, nelec, n2 = _i32(), _i32(), _i64()
    core = _dbl()
    _host_check(load_library().shci_fcidump_info(str(path).encode(), ctypes.byref(norb), ctypes.byref(nelec),
                                                 ctypes.byref(core), ctypes.byref(n2)))
    return norb.value, nelec.value, core.value, n2.value


def input_info(path):
    """Parse a Dice input file on the host only (no device): the expanded
    eps1 schedule and the variational settings, as a dict."""
    n = _i32()
    tols = np.zeros(3)
    ints = np.zeros(8, np.int32)
    _host_check(load_library().shci_input_info(str(path).encode(), None, 0, ctypes.byref(n), _p(tols), _p(ints)))
    eps = np.zeros(max(n.value, 1))
    _host_check(load_library().shci_input_info(str(path).encode(), _p(eps), n.value, ctypes.byref(n), None, None))
    keys = ("nroots", "ndet", "ncore", "nact", "precision", "blockdavidson", "precond", "davidson_basis")
    out = {k: int(v) for k, v in zip(keys, ints)}
    out.update(eps1=list(eps[:n.value]), davidsonTol=tols[0], davidsonTolLoose=tols[1], dE=tols[2])
    return out


class Engine:
    """One context of the GPU engine (one CUDA stream, device-resident state)."""

    def __init__(self, device=0):
        L = load_library()
        self.h = ctypes.c_void_p()
        rc = L.shci_ctx_create(device, ctypes.byref(self.h))
        if rc:
            raise ShciError(rc, L.shci_last_error(None).decode())
        self.norb = self.nelec = 0
        self.coreE = 0.0

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            load_library().shci_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise ShciError(rc, load_library().shci_last_error(self.h).decode())

    @property
    def stream(self):
        return load_library().shci_ctx_stream(self.h)

    def set_alloc_cap(self, nbytes):
        self._check(load_library().shci_set_alloc_cap(self.h, int(nbytes)))

    def read_fcidump(self, path):
        n, e, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._check(load_library().shci_read_fcidump(self.h, os.fspath(path).encode(), ctypes.byref(n),
                                                     ctypes.byref(e), ctypes.byref(c)))
        self.norb, self.nelec, self.coreE = n.value, e.value, c.value
        return self.norb, self.nelec, self.coreE

    def heatbath(self, same):
        L = load_library()
        cnt = ctypes.c_int64()
        self._check(L.shci_heatbath_export(self.h, int(same), ctypes.byref(cnt), None, None, None, None))
        n = self.norb
        vals = np.zeros(cnt.value, np.float32)
        pairs = np.zeros(2 * cnt.value, np.int16)
        starts = np.zeros(n * (n + 1) // 2 + 1, np.int64)
        singles = np.zeros((2 * n) ** 2, np.float64)
        self._check(L.shci_heatbath_export(self.h, int(same), ctypes.byref(cnt), _p(vals), _p(pairs), _p(starts),
                                           _p(singles)))
        return vals, pairs, starts, singles

    def set_selection_params(self, ncore=0, nact=1000000, restrictions=()):
        """restrictions: iterable of (min, max, spatial_orbital_list)."""
        nr = len(restrictions)
        rmin = np.array([r[0] for r in restrictions] or [0], np.int32)
        rmax = np.array([r[1] for r in restrictions] or [0], np.int32)
        masks = np.zeros(max(1, nr), np.uint64)
        for i, (_, _, orbs) in enumerate(restrictions):
            m = 0
            for o in orbs:
                m |= 1 << int(o)
            masks[i] = np.uint64(m)
        self._check(load_library().shci_set_selection_params(self.h, ncore, nact, nr, _p(rmin), _p(rmax),
                                                             _p(masks)))

    def set_dets(self, dets):
        d = np.ascontiguousarray(dets, dtype=np.uint64).reshape(-1, 2)
        self._check(load_library().shci_dets_set(self.h, _p(d), len(d)))

    def ndets(self):
        n = ctypes.c_int64()
        self._check(load_library().shci_dets_count(self.h, ctypes.byref(n)))
        return n.value

    def dets(self):
        n = self.ndets()
        out = np.zeros((n, 2), np.uint64)
        self._check(load_library().shci_dets_get(self.h, _p(out), n))
        return out

    def select(self, cmax, eps1):
        c = np.ascontiguousarray(cmax, dtype=np.float64)
        k = ctypes.c_int64()
        self._check(load_library().shci_select(self.h, _p(c), float(eps1), ctypes.byref(k)))
        return k.value

    def select_candidates(self, cmax, eps1, rank=0, world=1):
        """New determinants generated by this rank's parents (i % world ==
        rank), sorted and unique, not appended: (n, 2) uint64."""
        c = np.ascontiguousarray(cmax, dtype=np.float64)
        k = ctypes.c_int64()
        L = load_library()
        self._check(L.shci_select_candidates(self.h, _p(c), float(eps1), int(rank), int(world), ctypes.byref(k)))
        out = np.zeros((k.value, 2), np.uint64)
        self._check(L.shci_candidates_get(self.h, _p(out), k.value))
        return out

    def append_dets(self, dets):
        d = np.ascontiguousarray(dets, dtype=np.uint64).reshape(-1, 2)
        self._check(load_library().shci_dets_append(self.h, _p(d), len(d)))

    def ham_build_rows(self, r0, r1, mode="fp64"):
        """Full rows of the determinants [r0, r1) only (one rank's share)."""
        nnz = ctypes.c_int64()
        self._check(load_library().shci_ham_build_rows(self.h, MODES.get(mode, mode), int(r0), int(r1),
                                                       ctypes.byref(nnz)))
        return nnz.value

    def ham_build(self, mode="fp64"):
        nnz = ctypes.c_int64()
        self._check(load_library().shci_ham_build(self.h, MODES.get(mode, mode), ctypes.byref(nnz)))
        return nnz.value

    def ham_export(self, nnz):
        n = self.ndets()
        rowptr = np.zeros(n + 1, np.int64)
        col = np.zeros(max(1, nnz), np.int32)
        val = np.zeros(max(1, nnz), np.float64)
        self._check(load_library().shci_ham_export(self.h, _p(rowptr), _p(col), _p(val)))
        return rowptr, col[:nnz], val[:nnz]

    def diag(self):
        out = np.zeros(self.ndets(), np.float64)
        self._check(load_library().shci_diag(self.h, _p(out)))
        return out

    def sigma(self, x, mode="fp64"):
        """x: (N,) or (k, N) -> H x with the same shape."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        one = x.ndim == 1
        xx = x.reshape(1, -1) if one else x
        y = np.zeros_like(xx)
        self._check(load_library().shci_sigma(self.h, MODES.get(mode, mode), _p(xx), _p(y), xx.shape[0]))
        return y[0] if one else y

    def sigma_host(self, x_ptr, y_ptr, k, mode="fp64"):
        """shci_sigma on caller-owned host buffers (ints: addresses of k x N
        FP64 arrays, row-major by vector), e.g. pinned memory."""
        self._check(load_library().shci_sigma(self.h, MODES.get(mode, mode), ctypes.c_void_p(x_ptr),
                                              ctypes.c_void_p(y_ptr), k))

    def sigma_device(self, x_ptr, y_ptr, k, ld, mode="fp64"):
        """Device pointers (ints): column-major x, y with leading dimension ld."""
        self._check(load_library().shci_sigma_device(self.h, MODES.get(mode, mode), ctypes.c_void_p(x_ptr),
                                                     ctypes.c_void_p(y_ptr), k, ld))

    def sigma_device_noalloc(self, x_ptr, y_ptr, k, ld, mode="mixed"):
        """Allocation-free sigma on device pointers (see include/shci_gpu.h)."""
        self._check(load_library().shci_sigma_device_noalloc(self.h, MODES.get(mode, mode), ctypes.c_void_p(x_ptr),
                                                             ctypes.c_void_p(y_ptr), k, ld))

    def sigma_packed_device(self, xp_ptr, kp, k, y_ptr, ld, mode="mixed"):
        self._check(load_library().shci_sigma_packed_device(self.h, MODES.get(mode, mode), ctypes.c_void_p(xp_ptr),
                                                            kp, k, ctypes.c_void_p(y_ptr), ld))

    def ham_bytes(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(load_library().shci_ham_bytes(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def sigma_bytes(self, mode, k=1):
        """Algorithmic bytes of one stored-matrix sigma launch (roofline numerator)."""
        b = ctypes.c_int64()
        self._check(load_library().shci_sigma_bytes(self.h, MODES.get(mode, mode), int(k), ctypes.byref(b)))
        return b.value

    def davidson(self, x0, mode="fp64", block=False, max_copies=None, tol=5e-5, e_est=float("nan")):
        """e_est: energy estimate for the shifted preconditioners (NaN: none)."""
        x = np.ascontiguousarray(x0, dtype=np.float64).reshape(-1, self.ndets()).copy()
        nroots = x.shape[0]
        E = np.full(nroots, float(e_est))
        it = ctypes.c_int()
        mc = max_copies if max_copies is not None else nroots + 4
        self._check(load_library().shci_davidson(self.h, MODES.get(mode, mode), int(block), nroots, _p(x), mc,
                                                 float(tol), _p(E), ctypes.byref(it)))
        return E, x, it.value

    def run_input(self, path, mode=None, block=None, fcidump=None):
        """Whole variational stage of a Dice input file; returns E_var per root
        (core energy included). mode/block None: from the input file."""
        E = np.zeros(16)
        nr = ctypes.c_int()
        m = -1 if mode is None else MODES.get(mode, mode)
        b = -1 if block is None else int(block)
        self._check(load_library().shci_run_input(self.h, os.fspath(path).encode(),
                                                  fcidump.encode() if fcidump else None, m, b, _p(E), 16,
                                                  ctypes.byref(nr)))
        n, e, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._check(load_library().shci_ints_info(self.h, ctypes.byref(n), ctypes.byref(e), ctypes.byref(c)))
        self.norb, self.nelec, self.coreE = n.value, e.value, c.value
        return E[: nr.value].copy()

    def run_log(self):
        L = load_library()
        ni = ctypes.c_int()
        self._check(L.shci_run_log(self.h, 0, ctypes.byref(ni), None, None, None, None))
        n = ni.value
        nd = np.zeros(n, np.int64)
        en = np.zeros(n)
        di = np.zeros(n, np.int32)
        sec = np.zeros(n)
        self._check(L.shci_run_log(self.h, n, ctypes.byref(ni), _p(nd), _p(en), _p(di), _p(sec)))
        return {"ndets": nd, "energy": en, "davidson": di, "seconds": sec}

    def run_ci(self, nroots):
        n = self.ndets()
        out = np.zeros((nroots, n))
        self._check(load_library().shci_run_ci(self.h, _p(out), out.size))
        return out

    def timings(self):
        vals = [ctypes.c_double() for _ in range(4)]
        ns = ctypes.c_int64()
        ts = ctypes.c_double()
        self._check(load_library().shci_run_timings(self.h, *[ctypes.byref(v) for v in vals], ctypes.byref(ns),
                                                    ctypes.byref(ts)))
        keys = ["select", "ham", "davidson", "total"]
        out = {k: v.value for k, v in zip(keys, vals)}
        out["n_sigma"] = ns.value
        out["sigma"] = ts.value
        return out

    PRECOND = {"plain": 0, "pt2": 1, "mlp": 2}

    def set_preconditioner(self, mode):
        self._check(load_library().shci_set_preconditioner(self.h, self.PRECOND.get(mode, mode)))

    def set_davidson_basis(self, max_basis=0, keep=0):
        """Subspace of every Davidson solve of run_input: at most max_basis
        vectors, collapsed to keep; (0, 0) is the reference's rule."""
        self._check(load_library().shci_set_davidson_basis(self.h, int(max_basis), int(keep)))

    def set_davidson_graphs(self, on=True):
        """Davidson iterations as replayed CUDA graphs (default) or eager launches."""
        self._check(load_library().shci_set_davidson_graphs(self.h, int(bool(on))))

    def pt2_shift(self, E):
        out = np.zeros(self.ndets())
        self._check(load_library().shci_pt2_shift(self.h, float(E), _p(out)))
        return out

    def mlp_configure(self, steps=200, batch=4096, lr=1e-3, sample_rows=200000):
        self._check(load_library().shci_mlp_configure(self.h, steps, batch, lr, sample_rows))

    def mlp_train(self, E):
        loss = ctypes.c_float()
        self._check(load_library().shci_mlp_train(self.h, float(E), ctypes.byref(loss)))
        return loss.value

    def mlp_predict(self, E):
        out = np.zeros(self.ndets())
        self._check(load_library().shci_mlp_predict(self.h, float(E), _p(out)))
        return out

    def mlp_params(self):
        L = load_library()
        n, sig = ctypes.c_int(), ctypes.c_double()
        self._check(L.shci_mlp_params(self.h, None, 0, ctypes.byref(n), ctypes.byref(sig)))
        out = np.zeros(n.value, np.float32)
        self._check(L.shci_mlp_params(self.h, _p(out), n.value, ctypes.byref(n), ctypes.byref(sig)))
        return out, sig.value

    def mlp_set_params(self, params, sigma=1.0):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(load_library().shci_mlp_set_params(self.h, _p(p), len(p), float(sigma)))

    def mlp_gradient(self, rows, target, E):
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        n = len(self.mlp_params()[0])
        grad = np.zeros(n, np.float32)
        loss = ctypes.c_float()
        self._check(load_library().shci_mlp_gradient(self.h, _p(rows), _p(target), len(rows), float(E), _p(grad),
                                                     ctypes.byref(loss)))
        return loss.value, grad

    def run_stats(self):
        it, tm, loss = ctypes.c_int64(), ctypes.c_double(), ctypes.c_float()
        self._check(load_library().shci_run_stats(self.h, ctypes.byref(it), ctypes.byref(tm), ctypes.byref(loss)))
        return {"davidson_iters": it.value, "t_mlp": tm.value, "mlp_loss": loss.value}

    def pt_deterministic(self, ci, E0, eps2):
        """Deterministic PT2 correction E2 of the current space for host
        coefficients ci (one per determinant); E0 includes the core energy."""
        c = np.ascontiguousarray(ci, dtype=np.float64)
        if c.shape != (self.ndets(),):
            raise ValueError("ci must hold one coefficient per determinant")
        e2 = ctypes.c_double()
        self._check(load_library().shci_pt_deterministic(self.h, _p(c), float(E0), float(eps2), ctypes.byref(e2)))
        return e2.value

    def run_pt(self, eps2=-1.0):
        """After run_input: E_var + E2 per root (eps2 <= 0: the input's epsilon2)."""
        E = np.zeros(16)
        nr = ctypes.c_int()
        self._check(load_library().shci_run_pt(self.h, float(eps2), _p(E), 16, ctypes.byref(nr)))
        return E[:nr.value].copy()

    def pt_semistochastic(self, ci, E0, eps2, eps2_large=1000.0, sample_n=200, max_iter=1000000,
                          target_error=1e-4, seed=1):
        """Semistochastic PT2 estimate for host coefficients ci (E0 including
        the core energy). Returns (E2, standard error, iterations)."""
        c = np.ascontiguousarray(ci, dtype=np.float64)
        if c.shape != (self.ndets(),):
            raise ValueError("ci must hold one coefficient per determinant")
        e2, sd = ctypes.c_double(), ctypes.c_double()
        it = ctypes.c_int()
        self._check(load_library().shci_pt_semistochastic(self.h, _p(c), float(E0), float(eps2), float(eps2_large),
                                                          int(sample_n), int(max_iter), float(target_error),
                                                          int(seed), ctypes.byref(e2), ctypes.byref(sd),
                                                          ctypes.byref(it)))
        return e2.value, sd.value, it.value

    def pt_error(self):
        sd, el = ctypes.c_double(), ctypes.c_double()
        it = ctypes.c_int()
        self._check(load_library().shci_pt_error(self.h, ctypes.byref(sd), ctypes.byref(it), ctypes.byref(el)))
        return {"stddev": sd.value, "iterations": it.value, "e_large": el.value}

    def pt_stats(self):
        c, u, n = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        psi, t = ctypes.c_double(), ctypes.c_double()
        self._check(load_library().shci_pt_stats(self.h, ctypes.byref(c), ctypes.byref(u), ctypes.byref(n),
                                                 ctypes.byref(psi), ctypes.byref(t)))
        return {"candidates": c.value, "unique": u.value, "partitions": n.value, "psi1_norm": psi.value,
                "seconds": t.value}

    def set_pt_batch(self, max_candidates):
        self._check(load_library().shci_set_pt_batch(self.h, int(max_candidates)))

    def rdm(self, ci=None, root=0):
        """Spatial 2-RDM (norb, norb, norb, norb) with [p, q, r, s] =
        s2RDM(p n + q, r n + s) and spatial 1-RDM (norb, norb) of host
        coefficients ci on the current space, or of root `root` of the last
        run_input when ci is None."""
        n = self.norb
        s2 = np.zeros((n, n, n, n))
        s1 = np.zeros((n, n))
        if ci is None:
            self._check(load_library().shci_run_rdm(self.h, int(root), _p(s2), _p(s1)))
        else:
            c = np.ascontiguousarray(ci, dtype=np.float64)
            if c.shape != (self.ndets(),):
                raise ValueError("ci must hold one coefficient per determinant")
            self._check(load_library().shci_rdm(self.h, _p(c), _p(s2), _p(s1)))
        return s2, s1

    def write_best_dets(self, path, num, root=0):
        """The reference's dets.bin (writeBestDeterminants) for root `root`."""
        self._check(load_library().shci_write_best_dets(self.h, int(root), int(num), os.fspath(path).encode()))

    def launch_count(self):
        n = ctypes.c_int64()
        self._check(load_library().shci_launch_count(self.h, ctypes.byref(n)))
        return n.value
