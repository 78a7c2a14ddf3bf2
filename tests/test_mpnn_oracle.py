"""The CPU FP64 message-passing network (oracle/mpnn.py): its analytic gradient
against central finite differences, and its symmetry properties."""
import numpy as np

import golden_cases as gc
from oracle import mpnn


def small_problem():
    fx = gc.load("b12_fastpoly")
    n = fx["K_local_rowptr"].shape[0] - 1
    adj = mpnn.normalized_adjacency(fx["K_local_rowptr"], fx["K_local_col"], fx["K_local_val"], n)
    a = gc.csr_to_dense(fx["K_inner_rowptr"], fx["K_inner_col"], fx["K_inner_val"], n, n)
    a = a + np.triu(a, 1).T
    return n, adj, a


def test_gradient_matches_finite_differences():
    n, adj, a = small_problem()
    rng = np.random.default_rng(1)
    e = rng.standard_normal(n)
    r = a @ e
    z = r / np.diag(a)
    W = mpnn.init_weights(seed=2, scale=1.0)
    loss, g = mpnn.loss_and_grad(adj, lambda v: a @ v, r, z, e, W)
    assert loss > 0
    h = 1e-6
    for name in ("w1", "w2", "w3", "w4"):
        idx = [tuple(rng.integers(0, s) for s in W[name].shape) for _ in range(4)]
        for ij in idx:
            wp = {k: v.copy() for k, v in W.items()}
            wm = {k: v.copy() for k, v in W.items()}
            wp[name][ij] += h
            wm[name][ij] -= h
            lp, _ = mpnn.loss_and_grad(adj, lambda v: a @ v, r, z, e, wp)
            lm, _ = mpnn.loss_and_grad(adj, lambda v: a @ v, r, z, e, wm)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[name][ij]) <= 1e-6 * max(1.0, abs(fd)), (name, ij, fd, g[name][ij])


def test_correction_is_odd_and_homogeneous():
    n, adj, a = small_problem()
    rng = np.random.default_rng(4)
    r = rng.standard_normal(n)
    z = r / np.diag(a)
    W = mpnn.init_weights(seed=5)
    p, _ = mpnn.forward(adj, r, z, W)
    pm, _ = mpnn.forward(adj, -r, -z, W)
    p3, _ = mpnn.forward(adj, 3.0 * r, 3.0 * z, W)
    np.testing.assert_allclose(pm, -p, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(p3, 3.0 * p, rtol=1e-12, atol=1e-12)


def test_adjacency_is_symmetric():
    n, adj, _ = small_problem()
    rp, c, w = adj
    dense = np.zeros((n, n))
    for i in range(n):
        dense[i, c[rp[i]:rp[i + 1]]] = w[rp[i]:rp[i + 1]]
    np.testing.assert_allclose(dense, dense.T, rtol=0, atol=1e-15)
    assert np.all(np.diag(dense) == 0)
