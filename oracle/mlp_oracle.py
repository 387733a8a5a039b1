"""FP64 restatement of the learned-preconditioner network (CPU).

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward/backward kernels
of dice_gb300/csrc/kernels_mlp.cu. The network has no counterpart in the
reference (its preconditioner is SHCI/Davidson.cpp:85-106); this file follows
the definition in kernels_mlp.cu:
  features x = [doubly occupied (n), singly occupied (n), (H_ii - E) / 10, 1]
  h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), out = w3 . h2 + b3  (128 units)
  loss = mean((out - target)^2)
W1 and W2 enter the forward pass rounded to BF16 (the GPU stores them so);
all arithmetic here is FP64.
"""
import numpy as np

H = 128


def bf16_round(a):
    """Round FP32 values to the nearest BF16 (ties to even), returned as FP64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> np.uint64(16)) & np.uint64(1)
    r = (u + np.uint64(0x7FFF) + lsb) & np.uint64(0xFFFF0000)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, F):
    o = 0
    W1 = params[o:o + H * F].reshape(H, F); o += H * F
    W2 = params[o:o + H * H].reshape(H, H); o += H * H
    b1 = params[o:o + H]; o += H
    b2 = params[o:o + H]; o += H
    w3 = params[o:o + H]; o += H
    b3 = params[o]
    return W1, W2, b1, b2, w3, b3


def features(dets, diag, E, nspin):
    """[doubly occupied of orbital k (k < n), singly occupied of orbital k,
    (H_ii - E) / 10, 1] -- spin-free, so invariant under the alpha<->beta flip."""
    dets = np.asarray(dets, dtype=np.uint64)
    n = len(dets)
    norb = nspin // 2
    X = np.zeros((n, nspin + 2))

    def occ(p):
        return ((dets[:, p // 64] >> np.uint64(p % 64)) & np.uint64(1)).astype(np.int64)

    for k in range(norb):
        a, b = occ(2 * k), occ(2 * k + 1)
        X[:, k] = a & b
        X[:, norb + k] = a ^ b
    X[:, nspin] = np.float32((np.asarray(diag) - E) * 0.1)
    X[:, nspin + 1] = 1.0
    return X


def loss_and_grad(params, X, target):
    """Mean squared error and its gradient with respect to every parameter."""
    F = X.shape[1]
    W1, W2, b1, b2, w3, b3 = unpack(np.asarray(params, dtype=np.float64), F)
    W1q = bf16_round(W1)
    W2q = bf16_round(W2)
    B = X.shape[0]
    a1 = X @ W1q.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2q.T + b2
    h2 = np.maximum(a2, 0.0)
    out = h2 @ w3 + b3
    err = out - target
    loss = np.mean(err ** 2)
    dout = 2.0 * err / B
    gb3 = dout.sum()
    gw3 = h2.T @ dout
    g2 = np.outer(dout, w3) * (h2 > 0)
    gb2 = g2.sum(0)
    gW2 = g2.T @ h1
    g1 = (g2 @ W2q) * (h1 > 0)
    gb1 = g1.sum(0)
    gW1 = g1.T @ X
    grad = np.concatenate([gW1.ravel(), gW2.ravel(), gb1, gb2, gw3, [gb3]])
    return loss, grad, out
