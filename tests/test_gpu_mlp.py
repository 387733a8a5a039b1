"""The learned preconditioner on the GPU: the project's own forward/backward
kernels against the FP64 CPU oracle (oracle/mlp_oracle.py), training, and
what the trained network gains over the reference's diagonal preconditioner."""
import os

import numpy as np
import pytest

from dice_gb300 import engine as eng
from dice_gb300 import synthetic
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _h8(gpu, golden):
    inp = golden("h8_631g", "dice.dat")
    dets = np.load(os.path.join(GOLDEN, "h8_631g_dets.npz"))["dets"]
    gpu.read_fcidump(os.path.join(os.path.dirname(inp), "FCIDUMP"))
    gpu.set_dets(dets)
    return dets


def test_gradient_matches_cpu_oracle(golden):
    gpu = eng.Engine(0)
    dets = _h8(gpu, golden)
    diag = gpu.diag()
    E = float(diag.min()) - 0.05
    params, _ = gpu.mlp_params()
    rng = np.random.default_rng(2)
    params = params + rng.normal(0, 0.02, params.shape).astype(np.float32)  # move biases off zero
    gpu.mlp_set_params(params, 1.0)
    rows = rng.choice(len(dets), 300, replace=False).astype(np.int32)
    target = rng.normal(0, 1, 300).astype(np.float32)
    loss, grad = gpu.mlp_gradient(rows, target, E)
    X = mo.features(dets[rows], diag[rows], E, 2 * gpu.norb)
    lref, gref, _ = mo.loss_and_grad(params.astype(np.float64), X, target.astype(np.float64))
    assert abs(loss - lref) < 1e-4 * (1 + abs(lref))
    scale = np.abs(gref).max()
    assert np.allclose(grad, gref, rtol=1e-3, atol=1e-4 * scale)
    gpu.close()


def test_training_fits_the_level_shifts(golden):
    gpu = eng.Engine(0)
    dets = _h8(gpu, golden)
    gpu.ham_build("fp64")
    diag = gpu.diag()
    E = -4.3933538948 - gpu.coreE
    s = gpu.pt2_shift(E)
    gpu.mlp_configure(steps=400, batch=1024, lr=2e-3, sample_rows=len(dets))
    gpu.mlp_train(E)
    pred = gpu.mlp_predict(E)
    # the fit explains most of the variance of the teacher shifts
    r2 = 1 - np.mean((pred - s) ** 2) / np.var(s)
    assert r2 > 0.6, r2
    gpu.close()


def test_learned_preconditioner_gains_over_diagonal(tmp_path):
    """What the trained network buys, against the reference's diagonal
    preconditioner and the exact second-order level shift. (1) Over a whole
    variational run: the network, trained on Davidson's (residual, correction)
    pairs and judged by the plain preconditioner on a held-out iteration,
    changes the Davidson iteration count by at most 10 % either way on this
    workload (it is used only where the judge lets it), while the level shift
    saves iterations; E_var moves only at the level at which any change of the
    loose solves moves the selected space (micro-hartrees). (2) On one fixed
    space all three converge to the same eigenvalue (convergence is judged on
    the unpreconditioned residual). The counts are printed."""
    inp = synthetic.make_workload("mol24", str(tmp_path / "m"), schedule=[(0, 1e-3), (2, 3e-4)], maxiter=4)
    out = {}
    for name in ("plain", "pt2", "mlp"):
        gpu = eng.Engine(0)
        gpu.set_preconditioner(name)
        E = gpu.run_input(inp, mode="fp64")
        st = gpu.run_stats()
        out[name] = (E[0], st["davidson_iters"], list(gpu.run_log()["davidson"]), st["t_mlp"])
        if name == "mlp":  # keep the trained network for the fixed-space comparison
            kept = gpu
        else:
            gpu.close()
    print("whole run (E_var, Davidson iterations, per iteration, training s):", out)
    assert out["pt2"][1] < out["plain"][1]
    assert out["mlp"][3] > 0.0  # the network was trained
    assert out["mlp"][1] <= 1.1 * out["plain"][1]
    assert abs(out["mlp"][0] - out["plain"][0]) < 1e-5
    # fixed space: the final space of the learned run, same start vector
    gpu = kept
    gpu.ham_build("fp64")
    n = gpu.ndets()
    E0 = out["mlp"][0] - gpu.coreE
    x0 = np.zeros((1, n))
    x0[0, np.argmin(gpu.diag())] = 1.0
    fixed = {}
    for name in ("plain", "pt2", "mlp"):
        gpu.set_preconditioner(name)
        e, _, it = gpu.davidson(x0, mode="fp64", tol=1e-6, e_est=E0)
        fixed[name] = (e[0], it)
    print("fixed space of %d determinants (E, iterations):" % n, fixed)
    assert abs(fixed["mlp"][0] - fixed["plain"][0]) < 1e-9
    assert abs(fixed["pt2"][0] - fixed["plain"][0]) < 1e-9
    assert fixed["pt2"][1] < fixed["plain"][1]
    gpu.close()


@pytest.mark.parametrize("direct", [False, True], ids=["stored", "matrix_free"])
def test_pair_trained_preconditioner_keeps_the_eigenvalue(tmp_path, direct):
    """Preconditioner 2 in a whole run: the network is trained on the
    (residual, correction) pairs each loose Davidson solve records, the plain
    preconditioner judges it on a held-out iteration, and the run -- stored or
    matrix-free, where no level shift is available -- converges to the same
    determinants and the same E_var as with the plain preconditioner."""
    # every solve converged tightly, so that both runs select the same
    # determinants; the matrix-free path (whose loose solves the reference
    # stops at 3e-2) selects once and then runs its final solve with the
    # network trained on the first
    if direct:
        inp = synthetic.make_workload("mol24", str(tmp_path / "m"), schedule=[(0, 2e-3)], maxiter=1,
                                      extra=("davidsonTol 1e-7", "DirectDavidson"))
    else:
        inp = synthetic.make_workload("mol24", str(tmp_path / "m"), schedule=[(0, 3e-3), (1, 1e-3)], maxiter=3,
                                      extra=("davidsonTol 1e-7", "davidsonTolLoose 1e-7"))
    out = {}
    for precond in ("plain", "mlp"):
        e = eng.Engine(0)
        e.set_preconditioner(precond)
        E = e.run_input(inp, mode="mixed")
        out[precond] = (E, e.dets(), e.run_stats())
        e.close()
    assert out["mlp"][2]["t_mlp"] > 0.0  # the network was trained during the run
    assert np.array_equal(out["mlp"][1], out["plain"][1])
    assert abs(out["mlp"][0][0] - out["plain"][0][0]) < 1e-6
