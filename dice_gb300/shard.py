"""Sharded variational path: one process per GPU, torch.distributed between them
(NCCL across GPUs, gloo across host processes).

Selection (the parent loop and merge of SHCIbasics::DoVariational,
SHCI/SHCIbasics.cpp:954-1077): rank r generates the candidates of its parents,
the determinants i with i % world == r as in the reference (:969-970); they
come back from the rank's engine already sorted in the reference's order,
unique and absent from the space. Each candidate then goes to the rank
owner(d) = hash(d) % world -- one all-to-all, the partitioning the reference
uses to merge its perturbative candidates (Determinant::getHash,
:510-626) -- where the candidates arriving from all ranks are sorted and
uniqued. Every rank finally gathers the owners' disjoint lists, merges them
into the reference's order and appends them, so every rank holds the space the
single-process selection builds, in the same index order. The reference
itself merges its variational candidates up a binary tree of sends to rank 0
(:1002-1050); the result, the sorted union, is the same.

Sigma (Hmult2, SHCI/Hmult.h:52-150): rank r owns the full rows of the
determinants [r0, r1) of an equal split of the space (the reference deals
rows I % nprocs == rank and reduces private full-length vectors; with full
rows every element of y is owner-computed and no reduction is needed). Each
rank computes its rows of y from the whole x and the rows are all-gathered,
so every rank ends with the whole y -- bit for bit what one process computes,
because each row is summed over the same entries in the same order.

Davidson (SHCI/Davidson.cpp:111-348): the small Rayleigh matrices, the
basis rotations and the corrections are replicated on every rank (the same
numpy operations on the same data, so every rank holds the same basis); only
sigma is sharded. variational() runs the eps1 schedule of DoVariational with
these three steps.

The per-rank work goes through a backend with the engine's methods
(dice_gb300.engine.Engine on a GPU):
    select_candidates(cmax, eps1, rank, world) -> (n, 2) uint64
    append_dets(dets)
    ham_build_rows(r0, r1, mode) -> nnz
    sigma(x, mode) -> y   (only the rows [r0, r1) of y are meaningful)
    diag() -> (n,) diagonal energies
"""
import numpy as np

__all__ = ["row_block", "owner_of", "ref_order", "select", "sigma", "davidson", "variational", "Comm"]


def row_block(n, rank, world):
    """Rows [r0, r1) of rank `rank` in an equal split of n rows."""
    return n * rank // world, n * (rank + 1) // world


def owner_of(dets, world):
    """Owning rank of each determinant: a 64-bit mix of both words mod world
    (the same on every rank, independent of the index order)."""
    d = np.ascontiguousarray(dets, dtype=np.uint64).reshape(-1, 2)
    with np.errstate(over="ignore"):
        h = d[:, 0] * np.uint64(0x9E3779B97F4A7C15) ^ (d[:, 1] + np.uint64(0x632BE59BD9B4E019))
        h ^= h >> np.uint64(31)
        h *= np.uint64(0xBF58476D1CE4E5B9)
        h ^= h >> np.uint64(29)
    return (h % np.uint64(world)).astype(np.int64)


def ref_order(dets):
    """Indices that sort determinants as Determinant::operator< does: words
    compared as signed 64-bit integers from the top word down
    (SHCI/Determinants.h:490-498)."""
    d = np.ascontiguousarray(dets, dtype=np.uint64).reshape(-1, 2)
    return np.lexsort((d[:, 0].view(np.int64), d[:, 1].view(np.int64)))


def _sorted_unique(dets):
    d = np.ascontiguousarray(dets, dtype=np.uint64).reshape(-1, 2)
    if len(d) == 0:
        return d
    d = d[ref_order(d)]
    keep = np.ones(len(d), bool)
    keep[1:] = np.any(d[1:] != d[:-1], axis=1)
    return d[keep]


class Comm:
    """The collectives the sharded path needs, over torch.distributed. Tensors
    travel on `device` ("cuda" for NCCL, "cpu" for gloo)."""

    def __init__(self, device="cpu"):
        import torch.distributed as dist
        self.dist = dist
        self.rank = dist.get_rank()
        self.world = dist.get_world_size()
        self.device = device

    def _t(self, a):
        import torch
        return torch.from_numpy(np.ascontiguousarray(a)).to(self.device)

    def all_to_all_u64(self, parts):
        """parts[r]: uint64 array for rank r; returns the concatenation of
        what every rank sent here, in rank order."""
        import torch
        send_counts = np.array([len(p) for p in parts], np.int64)
        counts = self._t(send_counts)
        recv_counts = torch.empty_like(counts)
        self.dist.all_to_all_single(recv_counts, counts)
        rc = recv_counts.cpu().numpy()
        flat = np.concatenate([np.ascontiguousarray(p, dtype=np.uint64).view(np.int64) for p in parts]) \
            if len(parts) else np.zeros(0, np.int64)
        out = torch.empty(int(rc.sum()), dtype=torch.int64, device=self.device)
        self.dist.all_to_all_single(out, self._t(flat), [int(v) for v in rc], [int(v) for v in send_counts])
        return out.cpu().numpy().view(np.uint64)

    def all_gather_var(self, a, dtype):
        """Concatenation over ranks (in rank order) of arrays of any length."""
        import torch
        a = np.ascontiguousarray(a, dtype=dtype)
        n = self._t(np.array([a.size], np.int64))
        ns = [torch.empty_like(n) for _ in range(self.world)]
        self.dist.all_gather(ns, n)
        sizes = [int(v.item()) for v in ns]
        mx = max(sizes) if sizes else 0
        buf = np.zeros(mx, dtype=dtype)
        buf[: a.size] = a.ravel()
        t = self._t(buf)
        outs = [torch.empty_like(t) for _ in range(self.world)]
        self.dist.all_gather(outs, t)
        return np.concatenate([o.cpu().numpy()[:s] for o, s in zip(outs, sizes)])


def select(backend, comm, cmax, eps1):
    """One sharded selection step: appends to every rank's space the
    determinants the single-process selection appends, in the same order.
    Returns how many were appended."""
    rank, world = comm.rank, comm.world
    mine = np.ascontiguousarray(backend.select_candidates(cmax, eps1, rank, world), dtype=np.uint64)
    owner = owner_of(mine, world) if len(mine) else np.zeros(0, np.int64)
    parts = [mine[owner == r].ravel() for r in range(world)]
    got = comm.all_to_all_u64(parts).reshape(-1, 2)
    owned = _sorted_unique(got)  # the ranks' lists overlap where parents share children
    everything = comm.all_gather_var(owned.view(np.int64).ravel(), np.int64).view(np.uint64).reshape(-1, 2)
    new = everything[ref_order(everything)]  # the owners' lists are disjoint
    backend.append_dets(new)
    return len(new)


def sigma(backend, comm, x, n, mode="fp64"):
    """y = H x for the whole space of n determinants, every rank holding the
    Hamiltonian rows row_block(n, rank, world) (built by the caller with
    backend.ham_build_rows). x: (k, n) or (n,) float64 on every rank; returns
    the whole y, the same on every rank."""
    r0, r1 = row_block(n, comm.rank, comm.world)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.asarray(backend.sigma(x, mode))
    rows = y.reshape(-1, n)[:, r0:r1]  # (k, r1 - r0)
    # gather the row blocks column by column (each vector separately keeps the
    # rank-order concatenation equal to the row order)
    out = np.stack([comm.all_gather_var(rows[c], np.float64) for c in range(rows.shape[0])])
    return out.reshape(y.shape)


def davidson(backend, comm, n, diag, x0, tol, max_copies=None, mode="fp64", max_iter=None):
    """Lowest eigenpairs of the whole Hamiltonian, the rows of which are
    spread over the ranks (built with backend.ham_build_rows), by the
    reference's Davidson scheme (SHCI/Davidson.cpp:111-348): the basis is
    rotated to the Ritz vectors every iteration, the roots converge in order
    (residual norm below tol), the correction is the residual divided by
    (theta - H_ii) (1e-12 guard, :85-106), projected out of the basis and
    normalised, and a full basis of max_copies vectors collapses to nroots + 2
    Ritz vectors plus the new correction. x0: (nroots, n) start vectors, each
    with a nonzero norm. Returns (energies, vectors, iterations); raises
    RuntimeError past the reference's iteration cap (2000 per root)."""
    x0 = np.atleast_2d(np.asarray(x0, dtype=np.float64))
    nroots = x0.shape[0]
    max_copies = max_copies or nroots + 4
    max_iter = max_iter or 2000 * nroots
    diag = np.asarray(diag, dtype=np.float64)
    b = np.zeros((max_copies, n))
    sig = np.zeros((max_copies, n))
    for i in range(nroots):  # Gram-Schmidt of the start vectors
        v = x0[i] - b[:i].T @ (b[:i] @ x0[i]) if i else x0[i].copy()
        b[i] = v / np.linalg.norm(v)
    done, bsize, conv, it = 0, nroots, 0, 0
    while True:
        if done < bsize:
            sig[done:bsize] = sigma(backend, comm, b[done:bsize], n, mode)
            done = bsize
        hs = b[:bsize] @ sig[:bsize].T
        hs = 0.5 * (hs + hs.T)
        ev, vec = np.linalg.eigh(hs)
        b[:bsize] = vec.T @ b[:bsize]
        sig[:bsize] = vec.T @ sig[:bsize]
        for i in range(conv):  # an earlier root that drifted out of tolerance is taken up again
            if np.linalg.norm(sig[i] - ev[i] * b[i]) > tol:
                conv = i
                break
        r = sig[conv] - ev[conv] * b[conv]
        it += 1
        if bsize == n:
            return ev[:nroots].copy(), b[:nroots].copy(), it
        if np.linalg.norm(r) < tol:
            conv += 1
            if conv == nroots:
                return ev[:nroots].copy(), b[:nroots].copy(), it
            continue
        if it > max_iter:
            raise RuntimeError("Davidson did not converge in %d iterations" % max_iter)
        den = ev[conv] - diag
        den = np.where(np.abs(den) > 1e-12, den, den - 1e-12)
        r = r / den
        for i in range(bsize):
            r -= (b[i] @ r) / (b[i] @ b[i]) * b[i]
        r /= np.linalg.norm(r)
        if bsize < max_copies:
            b[bsize] = r
            bsize += 1
        else:  # keep nroots + 2 Ritz vectors (their sigmas too), add the correction
            bsize, done = nroots + 3, nroots + 2
            b[bsize - 1] = r


def variational(backend, comm, schedule, x0, tol_loose=5e-5, tol=1e-8, mode="fp64"):
    """The eps1 schedule of DoVariational (SHCI/SHCIbasics.cpp:783-1378) on
    the ranks: for each eps1, the Hamiltonian rows of the rank's block, a
    Davidson solve to tol_loose, and a sharded selection with cMax = max over
    roots |c_i|; after the last selection a solve to tol. x0: (nroots, n) start
    vectors on the backend's initial space. Returns (energies, vectors,
    determinant counts after each selection)."""
    x = np.atleast_2d(np.asarray(x0, dtype=np.float64))
    counts = []
    for eps1 in schedule:
        n = len(x[0])
        r0, r1 = row_block(n, comm.rank, comm.world)
        backend.ham_build_rows(r0, r1, mode)
        _, x, _ = davidson(backend, comm, n, backend.diag(), x, tol_loose, mode=mode)
        added = select(backend, comm, np.max(np.abs(x), axis=0), eps1)
        x = np.concatenate([x, np.zeros((x.shape[0], added))], axis=1)
        counts.append(n + added)
    n = len(x[0])
    r0, r1 = row_block(n, comm.rank, comm.world)
    backend.ham_build_rows(r0, r1, mode)
    e, x, _ = davidson(backend, comm, n, backend.diag(), x, tol, mode=mode)
    return e, x, counts
