"""The network oracle (oracle/learned_oracle.py) checked on the CPU.

Its backward pass is pinned by central finite differences of its own FP64
loss (relative error <= 1e-5 per checked parameter, which is what step
1e-6 gives for a smooth loss away from ReLU kinks), and its bfloat16
rounding by torch's float32 -> bfloat16 conversion (bit-exact).
"""
import numpy as np

from oracle import learned_oracle as lo

NP = 2 * lo.H + 3 * 2 * lo.H * lo.H + lo.H


def _ring_graph(nc, rng):
    """Coarse graph of a symmetric, diagonally dominant operator."""
    A = np.zeros((nc, nc))
    for i in range(nc):
        for j in ((i + 1) % nc, (i + 3) % nc):
            A[i, j] = A[j, i] = -rng.uniform(0.5, 1.5)
    A[np.diag_indices(nc)] = -A.sum(1) + rng.uniform(0.1, 0.5, nc)
    cptr = np.zeros(nc + 1, np.int64)
    cols, wgt = [], []
    for i in range(nc):
        nb = np.nonzero(A[i])[0]
        cols += list(nb)
        wgt += [0.0 if j == i else -A[i, j] / A[i, i] for j in nb]
        cptr[i + 1] = len(cols)
    return dict(nc=nc, cptr=cptr, ccol=np.array(cols, np.int32), wgt=np.array(wgt),
                dinv=1.0 / np.diag(A)), A


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    cg, A = _ring_graph(12, rng)
    np.testing.assert_allclose(lo.coarse_operator(cg), A, rtol=1e-14, atol=1e-14)
    p = rng.normal(0, 0.2, NP)
    rc = rng.normal(size=12)
    L, g, _ = lo.loss_and_grad(p, cg, rc, 5.0, 7.0)
    assert np.isfinite(L)
    eps = 1e-6
    for i in rng.choice(NP, 40, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (lo.loss_and_grad(pp, cg, rc, 5.0, 7.0)[0] - lo.loss_and_grad(pm, cg, rc, 5.0, 7.0)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(g[i]), 1e-3), (i, fd, g[i])


def test_zero_network_loss_is_baseline():
    """With wout = 0 the correction vanishes and L = cA / eA."""
    rng = np.random.default_rng(1)
    cg, _ = _ring_graph(9, rng)
    p = rng.normal(0, 0.2, NP)
    p[-lo.H:] = 0.0
    L, _, ec = lo.loss_and_grad(p, cg, rng.normal(size=9), 2.0, 3.0)
    assert np.all(ec == 0.0) and L == 1.5


def test_exact_coarse_solve_minimises_loss():
    """The scaled loss depends only on the direction of ec and is smallest
    for the exact coarse solve Ac^-1 rc, where it is (cA - rc' Ac^-1 rc) / eA."""
    rng = np.random.default_rng(3)
    cg, A = _ring_graph(10, rng)
    rc = rng.normal(size=10)
    ex = np.linalg.solve(A, rc)

    def loss(ec):
        num, den = ec @ rc, ec @ A @ ec
        return (5.0 - num * num / den) / 2.0

    assert abs(loss(ex) - (5.0 - rc @ ex) / 2.0) <= 1e-12
    assert abs(loss(-3.0 * ex) - loss(ex)) <= 1e-12
    assert all(loss(ex) < loss(ex + 1e-2 * rng.normal(size=10)) for _ in range(20))


def test_bf16_rounding_matches_torch():
    import torch
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.normal(0, 1, 5000), rng.normal(0, 1e-30, 100), [0.0, -0.0, 1.0, 65504.0],
                        (1 + np.arange(64) / 128.0)])
    ref = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(lo.bf16(x).astype(np.float32), ref)
