"""The engine's sharded entry points on one GPU, two ranks emulated by two
contexts that run one after the other (no kernel waits on another):

* shci_select_candidates: each rank's parents (i % 2 == rank) generate their
  candidates; exchanged by hash owner, merged and appended with
  shci_dets_append, they equal what shci_select appends in one process --
  the same determinants in the same order;
* shci_ham_build_rows: each rank builds the full rows of its half of the
  space; the rows of y each computes, put together, equal the sigma of the
  whole matrix bit for bit (FP64 and FP32, one and two vectors), because a
  row is summed over the same entries in the same order wherever it lives;
* a context holding a row block refuses what needs the whole matrix."""
import numpy as np
import pytest

from dice_gb300 import engine as eng
from dice_gb300 import shard
from dice_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _space(tmp_path):
    inp = synthetic.make_workload("mol24", str(tmp_path / "m"), schedule=[(0, 3e-3)], maxiter=2)
    e = eng.Engine(0)
    e.run_input(inp, mode="fp64")
    dets, ci = e.dets(), e.run_ci(1)[0]
    e.close()
    return str(tmp_path / "m" / "FCIDUMP"), dets, ci


def test_sharded_selection_equals_one_process(tmp_path):
    fcidump, dets, ci = _space(tmp_path)
    cmax, eps1 = np.abs(ci), 3e-4
    one = eng.Engine(0)
    one.read_fcidump(fcidump)
    one.set_dets(dets)
    one.select(cmax, eps1)
    want = one.dets()
    one.close()
    ranks = []
    for r in range(2):
        e = eng.Engine(0)
        e.read_fcidump(fcidump)
        e.set_dets(dets)
        ranks.append(e)
    cands = [e.select_candidates(cmax, eps1, r, 2) for r, e in enumerate(ranks)]
    # the exchange: every candidate to its owner, where the two lists merge
    owned = []
    for dest in range(2):
        got = np.concatenate([c[shard.owner_of(c, 2) == dest] for c in cands])
        owned.append(shard._sorted_unique(got))
    new = np.concatenate(owned)
    new = new[shard.ref_order(new)]
    assert len(new) > 10000
    for e in ranks:
        e.append_dets(new)
        assert np.array_equal(e.dets(), want)
    # an append that breaks the order or repeats a determinant is refused
    with pytest.raises(eng.ShciError):
        ranks[0].append_dets(new[:2][::-1])
    with pytest.raises(eng.ShciError):
        ranks[0].append_dets(dets[:1])
    for e in ranks:
        e.close()


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_row_block_sigma_equals_whole_matrix(tmp_path, mode):
    fcidump, dets, _ = _space(tmp_path)
    n = len(dets)
    one = eng.Engine(0)
    one.read_fcidump(fcidump)
    one.set_dets(dets)
    one.ham_build(mode)
    x = np.random.default_rng(4).standard_normal((2, n))
    want1, want2 = one.sigma(x[0], mode), one.sigma(x, mode)
    one.close()
    got1, got2 = np.full(n, np.nan), np.full((2, n), np.nan)
    nnz = 0
    for r in range(2):
        r0, r1 = shard.row_block(n, r, 2)
        e = eng.Engine(0)
        e.read_fcidump(fcidump)
        e.set_dets(dets)
        nnz += e.ham_build_rows(r0, r1, mode)
        got1[r0:r1] = e.sigma(x[0], mode)[r0:r1]
        got2[:, r0:r1] = e.sigma(x, mode)[:, r0:r1]
        # what needs the whole matrix is refused on a row block
        with pytest.raises(eng.ShciError) as ei:
            e.davidson(np.ones((1, n)) / np.sqrt(n), mode=mode)
        assert ei.value.code == 7
        with pytest.raises(eng.ShciError):
            e.sigma_bytes(mode, 1)
        e.close()
    assert np.array_equal(got1, want1)
    assert np.array_equal(got2, want2)


def test_sharded_loop_on_the_engine_matches_the_oracle_backend(tmp_path):
    """shard.variational with an Engine as the rank's backend (one rank, the
    whole space as its row block) selects the determinants the same loop
    selects with the CPU oracle as the backend, in the same order, and
    reaches the same energy."""
    from test_shard_gloo import OracleBackend, _OneRank, _fcidump, _h8_start
    dets, w = _h8_start()
    steps = (1e-4, 1e-6)
    ob = OracleBackend(_fcidump(str(tmp_path)), dets)
    e_ref, _, counts_ref = shard.variational(ob, _OneRank(), steps, w.reshape(1, -1), tol_loose=1e-6, tol=1e-9)
    e = eng.Engine(0)
    e.read_fcidump(str(tmp_path / "FCIDUMP"))
    e.set_selection_params(ncore=0, nact=8)  # the h8 example's active space, as the oracle backend selects
    e.set_dets(dets)
    en, _, counts = shard.variational(e, _OneRank(), steps, w.reshape(1, -1), tol_loose=1e-6, tol=1e-9)
    assert counts == counts_ref
    assert np.array_equal(e.dets(), ob.dets)
    assert abs(en[0] - e_ref[0]) < 1e-10
    e.close()
