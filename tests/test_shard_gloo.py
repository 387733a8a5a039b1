"""The sharded variational path (dice_gb300/shard.py) on two CPU ranks over
gloo: each rank selects from its own parents (i % 2 == rank), the candidates
are exchanged by hash owner, merged and appended; each rank holds the full
rows of its half of the space and the sigma rows are all-gathered. The
result must equal the single-process selection (same determinants, same
order) and the single-process sigma, bit for bit.

The per-rank work runs on the CPU oracle here (the engine needs a GPU); the
same orchestration drives dice_gb300.engine.Engine on GPUs."""
import os
import socket

import numpy as np
import pytest

from dice_gb300 import shard

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class OracleBackend:
    """The engine's per-rank calls, computed by the CPU oracle: selection from
    the rank's parents, full rows of a block of the space, sigma of those
    rows (summed in column order, as each row is summed wherever it lives)."""

    def __init__(self, fcidump, dets):
        from oracle import oracle as orc
        self.o = orc.Oracle(fcidump)
        self.dets = np.ascontiguousarray(dets, dtype=np.uint64)
        self.rows = None

    def select_candidates(self, cmax, eps1, rank, world):
        existing = self.dets[shard.ref_order(self.dets)]
        # the h8 example's own active space (nact 8) keeps the space small
        return self.o.select(self.dets[rank::world], np.asarray(cmax)[rank::world], eps1, existing, ncore=0, nact=8)

    def append_dets(self, new):
        self.dets = np.concatenate([self.dets, np.asarray(new, np.uint64).reshape(-1, 2)])

    def ham_build_rows(self, r0, r1, mode="fp64"):
        import scipy.sparse as sp
        rowptr, col, val = self.o.ham(self.dets)  # lower triangle with the diagonal first
        n = len(self.dets)
        rows = np.repeat(np.arange(n), np.diff(rowptr))
        low = sp.csr_matrix((val, (rows, col)), shape=(n, n))
        full = (low + sp.triu(low.T, 1)).tocsr()
        full.sort_indices()
        self.r0, self.r1 = r0, r1
        self.rows = full[r0:r1]
        self.full_diag = full.diagonal()
        return self.rows.nnz

    def diag(self):
        return self.full_diag.copy()

    def sigma(self, x, mode="fp64"):
        x = np.atleast_2d(x)
        y = np.full(x.shape, np.nan)
        for c in range(x.shape[0]):
            y[c, self.r0:self.r1] = self.rows @ x[c]
        return y


def _h8_start():
    import gzip
    d = np.load(os.path.join(GOLDEN, "h8_631g_dets.npz"))
    return d["dets"][:40].copy(), d["weights"][:40].copy()


def _fcidump(tmp):
    import gzip
    import shutil
    p = os.path.join(tmp, "FCIDUMP")
    with gzip.open(os.path.join(GOLDEN, "h8_631g.FCIDUMP.gz"), "rb") as f, open(p, "wb") as g:
        shutil.copyfileobj(f, g)
    return p


def _run(backend, comm, steps):
    """Two selection steps, then the Hamiltonian rows and a two-vector sigma."""
    rng = np.random.default_rng(3)
    for eps1 in steps:
        n = len(backend.dets)
        cmax = np.abs(rng.standard_normal(n)) * 0.05 + 1e-3
        shard.select(backend, comm, cmax, eps1)
    n = len(backend.dets)
    r0, r1 = shard.row_block(n, comm.rank, comm.world)
    backend.ham_build_rows(r0, r1)
    x = np.random.default_rng(7).standard_normal((2, n))
    return backend.dets.copy(), shard.sigma(backend, comm, x, n)


def _run_variational(backend, comm, steps):
    """The whole sharded loop: Davidson on the ranks' row blocks, sharded
    selection, and a final tight solve."""
    _, w = _h8_start()
    e, x, counts = shard.variational(backend, comm, steps, w.reshape(1, -1), tol_loose=1e-6, tol=1e-9)
    return backend.dets.copy(), e, x, np.array(counts)


def _worker_var(rank, world, port, tmp, steps):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dets, _ = _h8_start()
        backend = OracleBackend(_fcidump(os.path.join(tmp, "v%d" % rank)), dets)
        d, e, x, counts = _run_variational(backend, shard.Comm("cpu"), steps)
        np.savez(os.path.join(tmp, "var%d.npz" % rank), dets=d, e=e, x=x, counts=counts)
    finally:
        dist.destroy_process_group()


def _worker(rank, world, port, tmp, steps):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dets, _ = _h8_start()
        backend = OracleBackend(_fcidump(os.path.join(tmp, "r%d" % rank)), dets)
        d, y = _run(backend, shard.Comm("cpu"), steps)
        np.savez(os.path.join(tmp, "rank%d.npz" % rank), dets=d, y=y)
    finally:
        dist.destroy_process_group()


class _OneRank:
    rank, world = 0, 1

    def all_to_all_u64(self, parts):
        return np.concatenate([np.asarray(p, np.uint64) for p in parts])

    def all_gather_var(self, a, dtype):
        return np.ascontiguousarray(a, dtype=dtype).ravel()


def test_two_rank_selection_and_sigma_equal_one_process(tmp_path):
    import torch.multiprocessing as mp
    steps = (1e-4, 1e-6)
    for r in range(2):
        os.makedirs(tmp_path / ("r%d" % r))
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_worker, args=(2, port, str(tmp_path), steps), nprocs=2, join=True, start_method="spawn")
    os.makedirs(tmp_path / "one")
    dets, _ = _h8_start()
    ref_dets, ref_y = _run(OracleBackend(_fcidump(str(tmp_path / "one")), dets), _OneRank(), steps)
    assert len(ref_dets) > 1500
    for r in range(2):
        got = np.load(tmp_path / ("rank%d.npz" % r))
        assert np.array_equal(got["dets"], ref_dets), r  # same determinants, same order
        assert np.array_equal(got["y"], ref_y), r  # bit for bit


def test_owner_partition_and_reference_order():
    rng = np.random.default_rng(1)
    d = rng.integers(0, 2 ** 63, size=(1000, 2), dtype=np.uint64)
    d[::7, 1] |= np.uint64(1) << np.uint64(63)  # negative top words sort first
    own = shard.owner_of(d, 3)
    assert set(own.tolist()) == {0, 1, 2}
    assert np.array_equal(own, shard.owner_of(d[::-1], 3)[::-1])  # a function of the determinant only
    o = d[shard.ref_order(d)]
    hi, lo = o[:, 1].view(np.int64), o[:, 0].view(np.int64)
    assert np.all((hi[1:] > hi[:-1]) | ((hi[1:] == hi[:-1]) & (lo[1:] >= lo[:-1])))
    assert [shard.row_block(10, r, 3) for r in range(3)] == [(0, 3), (3, 6), (6, 10)]


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_variational_loop_equals_one_process(tmp_path, world):
    """shard.variational on gloo ranks (Davidson replicated, sigma and
    selection sharded; three ranks split rows and parents unevenly) selects
    the one-process run's determinants in the same order and converges to the
    same energy, which is the lowest eigenvalue of the final space's
    Hamiltonian."""
    import scipy.sparse.linalg as sla
    import torch.multiprocessing as mp
    steps = (1e-4, 1e-6)
    for r in range(world):
        os.makedirs(tmp_path / ("v%d" % r))
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_worker_var, args=(world, port, str(tmp_path), steps), nprocs=world, join=True,
                       start_method="spawn")
    os.makedirs(tmp_path / "one")
    dets, _ = _h8_start()
    one = OracleBackend(_fcidump(str(tmp_path / "one")), dets)
    ref_dets, ref_e, ref_x, ref_counts = _run_variational(one, _OneRank(), steps)
    assert len(ref_dets) > 1500
    one.ham_build_rows(0, len(ref_dets))
    lowest = sla.eigsh(one.rows, k=1, which="SA", tol=1e-12)[0][0]
    assert abs(ref_e[0] - lowest) < 1e-8
    for r in range(world):
        got = np.load(tmp_path / ("var%d.npz" % r))
        assert np.array_equal(got["dets"], ref_dets), r
        assert np.array_equal(got["counts"], ref_counts), r
        assert abs(got["e"][0] - ref_e[0]) < 1e-10, r
