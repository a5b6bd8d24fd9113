"""Colour classes of the multicolour Gauss-Seidel (nw_linsys_sgs_order /
nw_linsys_sgs_classes): a proper colouring of the CSR graph (no two rows of
a class coupled), every row in exactly one class, two node colours on a
hex box (one class per node colour and dof), and on a randomly numbered tet mesh no more classes than first fit in row
order (the library recolours class by class and keeps a recolouring only
when it needs fewer)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _classes(ls):
    order, nc = ls.sgs_order()
    cp = ls.sgs_classes()
    assert cp[0] == 0 and cp[-1] == order.size and np.all(np.diff(cp) > 0)
    cls = np.empty(order.size, np.int64)
    for c in range(nc):
        cls[order[cp[c]:cp[c + 1]]] = c
    assert np.array_equal(np.sort(order), np.arange(order.size))
    return cls, nc


def _check_proper(ls, cls):
    rp, ci = ls.graph()
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    off = ci != rows
    assert not np.any(cls[rows[off]] == cls[ci[off]])


def _first_fit_count(n, edges):
    nb = [[] for _ in range(n)]
    for a, b in edges.tolist():
        nb[a].append(b)
        nb[b].append(a)
    col = [-1] * n
    for r in range(n):
        used = {col[c] for c in nb[r] if col[c] >= 0}
        k = 0
        while k in used:
            k += 1
        col[r] = k
    return max(col) + 1


@pytest.mark.parametrize("ndof", [1, 3])
def test_hex_box_has_two_classes(nw, ndof):
    mesh = nw.Mesh(12, 10, 8, stretch_z=1.05, jitter=0.05, seed=3)
    ls = nw.LinearSystem(ndof)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges)
    ls.finalize()
    cls, nc = _classes(ls)
    assert nc == 2 * ndof
    _check_proper(ls, cls)


@pytest.mark.parametrize("ren", [1, 2])
def test_tet_classes_are_proper_and_no_more_than_first_fit(nw, ren):
    mesh = nw.Mesh(16, 15, 14, tets=True, jitter=0.05, seed=5, renumber=ren, renumber_seed=7)
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges)
    ls.finalize()
    cls, nc = _classes(ls)
    _check_proper(ls, cls)
    assert nc <= _first_fit_count(mesh.num_nodes, mesh.edges)
