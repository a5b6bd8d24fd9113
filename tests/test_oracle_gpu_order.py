"""The oracle's solvers restated in the GPU library's operation order
(oracle/gpu_order.cpp) are the same algorithms as its natural-order
restatement (oracle.cpp's or_solve): on the same systems they take the
same iterations and their residual histories agree up to the rounding
that a different summation order introduces (CPU only)."""
import numpy as np
import pytest


def _system(orc, shape=(14, 12, 9)):
    from oracle import cases
    c = cases.lowmach_case(*shape, seed=3)
    m, nd = c.mesh, c.node
    rp, ci, lid = orc.build_graph(m.nalu_id, m.edges, 1)
    lhs, rhs = orc.continuity_local(m.edges, m.coords, nd["velocity"], nd["dpdx"], nd["density"],
                                    nd["pressure"], nd["udiag"], m.area, c.opts["continuity"])
    vals, b = orc.sum_into(m.edges, 1, lhs, rhs, lid, rp, ci, nthreads=1, with_abs=False)[:2]
    return rp, ci, vals, b - b.mean()


def _greedy_classes(rp, ci):
    n = len(rp) - 1
    color = -np.ones(n, np.int64)
    for i in range(n):
        used = {color[j] for j in ci[rp[i]:rp[i + 1]] if j != i and color[j] >= 0}
        c = 0
        while c in used:
            c += 1
        color[i] = c
    order = np.argsort(color, kind="stable")
    cp = np.concatenate([[0], np.cumsum(np.bincount(color))])
    return order, cp


@pytest.mark.parametrize("method,pc,rtol", [(0, 0, 1e-7), (0, 1, 1e-7), (1, 1, 1e-9), (2, 1, 1e-7),
                                            (4, 1, 1e-7), (0, 4, 1e-8), (0, 2, 1e-7), (1, 2, 1e-8)])
def test_gpu_order_is_the_same_algorithm(orc, method, pc, rtol):
    rp, ci, vals, b = _system(orc)
    order = cp = None
    if pc == 2:
        order, cp = _greedy_classes(rp, ci)
    G = orc.gpu_reduction_blocks(len(b), 152)
    x1, h1, r1 = orc.solve(rp, ci, vals, b, method=method, precond=pc, order=order, kspace=30, max_iters=800,
                           tol=1e-8)
    x2, h2, r2 = orc.solve_gpu_order(rp, ci, vals, b, method=method, precond=pc, order=order, class_ptr=cp,
                                     kspace=30, max_iters=800, tol=1e-8, red_blocks=G, lanes=8)
    assert r1.converged and r2.converged
    assert abs(r1.iterations - r2.iterations) <= 1
    k = min(len(h1), len(h2))
    np.testing.assert_allclose(h2[:k], h1[:k], rtol=rtol)
    assert np.linalg.norm(x2 - x1) <= 1e3 * rtol * np.linalg.norm(x1)


def test_gpu_order_reduction_grid_changes_only_rounding(orc):
    """Two reduction grids: identical iteration counts, histories within the
    rounding a different grouping gives."""
    rp, ci, vals, b = _system(orc)
    out = [orc.solve_gpu_order(rp, ci, vals, b, method=1, precond=1, max_iters=500, tol=1e-10, red_blocks=G)
           for G in (3, 37)]
    assert out[0][2].iterations == out[1][2].iterations
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-9)


@pytest.mark.parametrize("sstep", [1, 3, 5])
def test_sstep_gmres_is_gmres_in_exact_arithmetic(orc, sstep):
    """s-step GMRES builds the same Krylov spaces as GMRES: with step size
    1 to 5 the histories agree with GMRES(30) to the basis' rounding."""
    rp, ci, vals, b = _system(orc)
    G = orc.gpu_reduction_blocks(len(b), 152)
    _, h1, r1 = orc.solve_gpu_order(rp, ci, vals, b, method=0, precond=1, kspace=30, max_iters=800, tol=1e-8,
                                    red_blocks=G)
    x2, h2, r2 = orc.solve_gpu_order(rp, ci, vals, b, method=5, precond=1, kspace=30, max_iters=800, tol=1e-8,
                                     red_blocks=G, sstep_size=sstep)
    assert r2.converged and abs(r1.iterations - r2.iterations) <= 2
    k = min(len(h1), len(h2), 60)
    np.testing.assert_allclose(h2[:k], h1[:k], rtol=1e-6)
    assert r2.final_abs_explicit <= 1.01e-8 * r2.rhs_norm
