"""Lumped-mass BDF node kernels on the GPU against the oracle (itself pinned
to the reference node-kernel golds in test_oracle_golds.py).

Each node row gets the sum of its nodes' terms (a periodic master and its
slaves); tolerance 1e-12 of the sum of the terms' magnitudes.
"""
import numpy as np
import pytest

from gpu_util import check_close, dev

import kat

pytestmark = pytest.mark.gpu


def _system(nw, mesh, nd):
    ls = nw.LinearSystem(nd)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    ls.finalize()
    ls.zero_system()
    return ls


def _diag_and_rhs(ls, nd):
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    nr = len(rhs)
    diag = np.array([vals[rp[r]:rp[r + 1]][ci[rp[r]:rp[r + 1]] == r][0] for r in range(nr)])
    return diag, rhs


def _rows(nw, ls, mesh, per_node, nd):
    """Sum per-node values (N x nd) into their rows (oracle side)."""
    lid = ls.node_lid(mesh.num_nodes)
    nr = ls.sizes()[0]
    out = np.zeros(nr)
    for d in range(nd):
        np.add.at(out, lid + d, per_node.reshape(-1, nd)[:, d])
    return out


@pytest.mark.parametrize("kind", ["scalar", "continuity", "momentum"])
def test_mass_bdf_matches_oracle(nw, orc, kind):
    mesh = nw.Mesh(10, 9, 8, periodic_x=True, jitter=0.05, seed=3)
    nd = 3 if kind == "momentum" else 1
    code = {"scalar": 0, "continuity": 1, "momentum": 2}[kind]
    rng = np.random.default_rng(7)
    N = mesh.num_nodes
    rho = tuple(rng.uniform(0.5, 1.5, N) for _ in range(3))
    dnv = tuple(mesh.dualvol * rng.uniform(0.9, 1.1, N) for _ in range(3))
    q = tuple(rng.normal(size=(N, nd)) if nd == 3 else rng.normal(size=N) for _ in range(3))
    dpdx = rng.normal(size=(N, 3))
    ls = _system(nw, mesh, nd)
    ls.assemble_mass_bdf(kind, [dev(a) for a in rho], [dev(a) for a in dnv],
                         q=[dev(a) for a in q] if kind != "continuity" else None,
                         dpdx=dev(dpdx) if kind == "momentum" else None, dt=0.05, gamma=(1.5, -2.0, 0.5))
    diag, rhs = _diag_and_rhs(ls, nd)
    lhs_o, rhs_o = orc.mass_bdf(code, rho, dnv, q=q if kind != "continuity" else None,
                                dpdx=dpdx if kind == "momentum" else None, dt=0.05, gamma=(1.5, -2.0, 0.5))
    # magnitudes: every term with |inputs|
    absq = [np.abs(a) for a in q]
    g = (1.5, 2.0, 0.5)
    m = sum(gk * np.abs(rho[k2]) * np.abs(dnv[k2]) * (absq[k2] if nd == 1 and kind == "scalar" else 1.0)
            for gk, k2 in zip(g, (2, 1, 0)))
    if kind == "momentum":
        m = sum(gk * (np.abs(rho[k2]) * np.abs(dnv[k2]))[:, None] * absq[k2] for gk, k2 in zip(g, (2, 1, 0)))
        m = m / 0.05 + np.abs(dpdx) * np.abs(dnv[2])[:, None]
    elif kind == "continuity":
        m = m / 0.05 * (1.5 / 0.05)
    else:
        m = m / 0.05
    check_close(rhs, _rows(nw, ls, mesh, rhs_o, nd), _rows(nw, ls, mesh, m, nd), f"{kind} rhs")
    lscale = _rows(nw, ls, mesh, np.repeat((1.5 * np.abs(rho[2]) * np.abs(dnv[2]) / 0.05)[:, None], nd, 1), nd)
    check_close(diag, _rows(nw, ls, mesh, lhs_o, nd), lscale + 1e-300, f"{kind} diag")


def test_mass_bdf_golds_through_gpu(nw, orc, golds):
    m = kat.hex1(orc)
    mesh_edges = m["edges"]
    ls = nw.LinearSystem(3)
    ls.build_edge_graph(8, mesh_edges)
    ls.finalize()
    ls.zero_system()
    z = np.zeros(8)
    V = m["dualvol"]
    cf = kat.continuity_fixture(orc)
    g = golds["momentum_mass_bdf_hex8"]
    ls.assemble_mass_bdf("momentum", [dev(z), dev(z), dev(np.ones(8))], [dev(V)] * 3,
                         q=[dev(np.zeros((8, 3))), dev(np.zeros((8, 3))), dev(kat.trig_velocity(m["coords"]))],
                         dpdx=dev(cf["dpdx"]), dt=g["dt"], gamma=g["gamma"])
    diag, rhs = _diag_and_rhs(ls, 3)
    np.testing.assert_allclose(rhs, g["rhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(diag, g["lhs_diag"], rtol=0, atol=1e-14)
