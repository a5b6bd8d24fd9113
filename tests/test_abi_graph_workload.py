"""CPU tests of the library's host side: C ABI exports, the Tpetra-identical
graph, and the synthetic-mesh geometry, each against the oracle."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(nw_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(nw):
    lib = nw.load()
    decl = declared_functions()
    assert len(decl) > 20
    missing = [n for n in decl if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding types every one of them
    assert set(decl) <= set(nw.SIGNATURES), set(decl) - set(nw.SIGNATURES)


def test_status_and_error_string(nw):
    lib = nw.load()
    import ctypes as C
    h = C.c_void_p()
    st = lib.nw_linsys_create(7, None, C.byref(h))
    assert st == 1  # NW_INVALID_ARG
    assert b"num_dof" in lib.nw_last_error_string()
    with pytest.raises(nw.NwError):
        nw.LinearSystem(num_dof=0)


def test_unfinalized_calls_are_rejected(nw):
    ls = nw.LinearSystem(1)
    with pytest.raises(nw.NwError) as e:
        ls.zero_system()
    assert e.value.status == 3  # NOT_FINALIZED


def _graph_pair(nw, orc, mesh, num_dof):
    ls = nw.LinearSystem(num_dof)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    rp, ci = ls.graph()
    lid = ls.node_lid(mesh.num_nodes)
    orp, oci, olid = orc.build_graph(mesh.nalu_id, mesh.edges, num_dof)
    return (rp, ci, lid), (orp, oci, olid)


@pytest.mark.parametrize("num_dof", [1, 3])
@pytest.mark.parametrize("kind", ["periodic", "stretched", "tets", "rcm"])
def test_graph_bit_exact_vs_oracle(nw, orc, num_dof, kind):
    if kind == "periodic":
        mesh = nw.Mesh(6, 5, 4, periodic_x=True, periodic_y=True)
    elif kind == "stretched":
        mesh = nw.Mesh(7, 5, 6, stretch_z=1.08, jitter=0.05, seed=3)
    elif kind == "tets":
        mesh = nw.Mesh(4, 3, 3, tets=True)
    else:
        mesh = nw.Mesh(5, 4, 4, tets=True, renumber=2, renumber_seed=9)
    (rp, ci, lid), (orp, oci, olid) = _graph_pair(nw, orc, mesh, num_dof)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    np.testing.assert_array_equal(lid, olid)


def test_periodic_rows_are_masters(nw):
    n = 8
    mesh = nw.Mesh(n, n, n, periodic_x=True, periodic_y=True)
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    nr, nnz = ls.sizes()
    assert mesh.num_nodes == (n + 1) ** 3
    assert nr == n * n * (n + 1)
    # 7-point stencil on a doubly periodic lattice
    assert nnz == nr + 2 * (3 * n * n * (n + 1) - n * n)


def _oracle_geometry_on(orc, mesh):
    oedges, ee = orc.hex8_edges(mesh.conn, mesh.num_nodes)
    area, vol = orc.hex8_geometry(mesh.coords, mesh.conn, ee, oedges)
    key = {tuple(e): i for i, e in enumerate(oedges.tolist())}
    perm = np.array([key[tuple(e)] for e in mesh.edges.tolist()])
    return area[perm], vol


@pytest.mark.parametrize("opts", [dict(), dict(stretch_z=1.08, jitter=0.05, seed=7, lz=0.5)])
def test_hex_geometry_vs_oracle(nw, orc, opts):
    mesh = nw.Mesh(6, 5, 4, **opts)
    area, vol = _oracle_geometry_on(orc, mesh)
    scale = np.abs(area).max()
    assert np.abs(mesh.area - area).max() <= 1e-14 * scale
    np.testing.assert_allclose(mesh.dualvol, vol, rtol=1e-13)
    # dual volumes tile the box
    assert abs(mesh.dualvol.sum() - mesh.coords.max(0).prod()) < 1e-12


def test_periodic_dual_volume_summed(nw, orc):
    mesh = nw.Mesh(4, 4, 3, periodic_x=True, periodic_y=True)
    _, vol = _oracle_geometry_on(orc, mesh)
    master = mesh.nalu_id - 1
    tot = np.bincount(master, vol, mesh.num_nodes)
    np.testing.assert_allclose(mesh.dualvol, tot[master], rtol=1e-13)


@pytest.mark.parametrize("renumber", [0, 1, 2])
def test_tet_geometry_closed_and_consistent(nw, renumber):
    mesh = nw.Mesh(4, 4, 3, tets=True, renumber=renumber, renumber_seed=5)
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    assert np.all(L < R)
    dx = mesh.coords[R] - mesh.coords[L]
    assert np.all(np.einsum("ed,ed->e", mesh.area, dx) > 0)
    assert abs(mesh.dualvol.sum() - 1.0) < 1e-12
    # interior dual cells are closed: sum of outward areas vanishes
    net = np.zeros((mesh.num_nodes, 3))
    np.add.at(net, L, mesh.area)
    np.add.at(net, R, -mesh.area)
    c = mesh.coords
    interior = np.all((c > 1e-12) & (c < 1 - 1e-12), axis=1)
    assert np.abs(net[interior]).max() < 1e-13
    # Kuhn split: mean degree approaches 14
    deg = np.bincount(L, minlength=mesh.num_nodes) + np.bincount(R, minlength=mesh.num_nodes)
    assert deg.max() == 14


def test_mesh_sizes_match_expected_counts(nw):
    mesh = nw.Mesh(32, 32, 32, periodic_x=True, periodic_y=True)
    assert mesh.num_nodes == 35937
    assert mesh.num_edges == 104544
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    nr, nnz = ls.sizes()
    assert (nr, nnz) == (33792, 234496)


def test_bad_inputs_rejected(nw):
    ls = nw.LinearSystem(1)
    with pytest.raises(nw.NwError):
        ls.build_edge_graph(4, np.array([[0, 5]]))  # node index out of range
    with pytest.raises(nw.NwError):
        ls.build_edge_graph(4, np.array([[0, 1]]), nalu_id=np.array([1, 9, 3, 4]))  # missing master
    with pytest.raises(nw.NwError):
        # both ends fold to one master
        ls.build_edge_graph(2, np.array([[0, 1]]), nalu_id=np.array([1, 1]))
    with pytest.raises(nw.NwError):
        nw.Mesh(0, 2, 2)


def test_face_ips_of_the_unit_cube_match_the_reference_side(nw):
    import kat
    ipn, area = nw.Mesh(1, 1, 1).face_ips(("x+",))
    assert np.array_equal(ipn, kat.XPLUS_IPN)
    np.testing.assert_allclose(area, kat.XPLUS_AREA, rtol=0, atol=1e-15)


@pytest.mark.parametrize("tets,renumber", [(False, 0), (True, 0), (False, 1), (True, 2)])
def test_face_ips_close_the_surface(nw, tets, renumber):
    """Sub-face area vectors of each side sum to the side's area vector; the
    whole surface is closed; each opposing node is a graph neighbour of its
    face node, off the face's plane."""
    m = nw.Mesh(5, 4, 3, lx=1.0, ly=2.0, lz=0.5, stretch_z=1.3, jitter=0.2, seed=3, tets=tets,
                renumber=renumber, renumber_seed=7)
    ipn, area = m.face_ips()
    np.testing.assert_allclose(area.sum(0), 0.0, atol=1e-13)
    want = {"x-": [-1.0, 0, 0], "x+": [1.0, 0, 0], "y-": [0, -0.5, 0], "y+": [0, 0.5, 0],
            "z-": [0, 0, -2.0], "z+": [0, 0, 2.0]}
    for side, w in want.items():
        i, a = m.face_ips((side,))
        np.testing.assert_allclose(a.sum(0), w, atol=1e-13)
        # each IP's sub-face points outward
        assert np.all(a @ np.array(w) > 0)
    pairs = set(map(tuple, np.sort(m.edges, 1).tolist()))
    assert all(tuple(sorted(p)) in pairs for p in ipn.tolist())
    d = m.coords[ipn[:, 0]] - m.coords[ipn[:, 1]]
    assert np.all(np.einsum("id,id->i", d, area) > 0)


def test_periodic_sides_have_no_face_ips(nw):
    m = nw.Mesh(4, 4, 2, periodic_x=True, periodic_y=True)
    for side in ("x-", "x+", "y-", "y+"):
        assert len(m.face_ips((side,))[0]) == 0
    assert len(m.face_ips(("z-", "z+"))[0]) == 2 * 4 * 16


@pytest.mark.parametrize("tets", [False, True])
def test_face_ip_areas_match_the_master_element_formulas(nw, orc, tets):
    """The generator's face-IP area vectors against the oracle's restatement
    of Quad3DSCS / Tri3DSCS on the same (outward-ordered) faces, on a
    jittered, stretched block."""
    m = nw.Mesh(4, 3, 3, stretch_z=1.2, jitter=0.2, seed=9, tets=tets)
    ipn, area = m.face_ips()
    nn = 3 if tets else 4
    faces = ipn[:, 0].reshape(-1, nn)
    ref = orc.face_scs_areas(faces, m.coords)
    np.testing.assert_allclose(area, ref, rtol=0, atol=1e-14 * np.abs(ref).max())


@pytest.mark.parametrize("tets,periodic", [(False, False), (True, False), (False, True)])
def test_lumped_boundary_area_is_the_shifted_closure(nw, orc, tets, periodic):
    """bnd_area equals the sum of each node's face-IP sub-face areas (the
    shifted NodalGradBndryElemAlg closure), periodic pairs summed."""
    m = nw.Mesh(4, 3, 3, stretch_z=1.1, jitter=0.1, seed=2, tets=tets, periodic_x=periodic, periodic_y=periodic)
    ipn, area = m.face_ips()
    ref = np.zeros((m.num_nodes, 3))
    np.add.at(ref, ipn[:, 0], area)
    ref = nw.workload.periodic_sum(m, ref)
    np.testing.assert_allclose(m.bnd_area, ref, rtol=0, atol=1e-15)


def test_solver_strings_map_like_the_reference(nw):
    """TpetraLinearSolverConfig::load's strings (src/LinearSolverConfig.C:
    37-140) through nw_solver_cfg_from_strings."""
    m = {"gmres": nw.GMRES, "cg": nw.CG, "tfqmr": nw.TFQMR, "bicgstab": nw.BICGSTAB, "sstep_gmres": nw.SSTEP_GMRES}
    p = {"jacobi": nw.PC_JACOBI, "default": nw.PC_JACOBI, "sgs": nw.PC_SGS_NATURAL, "mt_sgs": nw.PC_MT_SGS,
         "sgs2": nw.PC_SGS2, "riluk": nw.PC_RILUK}
    for ms, mv in m.items():
        for ps, pv in p.items():
            cfg = nw.solver_cfg_from_strings(ms, ps, kspace=30)
            assert (cfg.method, cfg.preconditioner, cfg.kspace) == (mv, pv, 30)
    for bad in ("ilut", "muelu", "foo"):
        with pytest.raises(nw.NwError) as e:
            nw.solver_cfg_from_strings("gmres", bad)
        assert e.value.status == 1
    with pytest.raises(nw.NwError):
        nw.solver_cfg_from_strings("lsqr", "jacobi")


def test_rcm_order_restores_locality(nw):
    """nw_mesh_rcm_order on a randomly numbered tet mesh: a permutation that
    cuts the bandwidth, and the same order the mesh generator applies for
    renumber = 2 (random, then RCM) from the same graph."""
    rnd = nw.Mesh(14, 12, 10, tets=True, renumber=1, renumber_seed=3)
    N = rnd.num_nodes
    order = nw.rcm_order(N, rnd.edges)
    np.testing.assert_array_equal(np.sort(order), np.arange(N))
    inv = np.empty(N, np.int64)
    inv[order] = np.arange(N)
    bw = lambda e: int(np.abs(e[:, 0] - e[:, 1]).max())
    assert bw(inv[rnd.edges]) * 8 < bw(rnd.edges)
    rcm = nw.Mesh(14, 12, 10, tets=True, renumber=2, renumber_seed=3)
    np.testing.assert_array_equal(rcm.coords, rnd.coords[order])
    with pytest.raises(nw.NwError):
        nw.rcm_order(3, np.array([[0, 3]]))


@pytest.mark.parametrize("renumber", [0, 2])
def test_tet_geometry_vs_oracle(nw, orc, renumber):
    """The generator's (and the GPU's) Tet4 geometry: sub-control-surface
    area vectors as small-integer combinations of the three edge-vector
    cross products (half the cross product of each quad's diagonals) and the
    sub-control volumes as quarters of the tet volume, against the oracle's
    restatement of TetSCS (triangle fans) and TetSCV (Grandy's formula)."""
    m = nw.Mesh(6, 5, 4, stretch_z=1.2, jitter=0.2, seed=4, tets=True, renumber=renumber, renumber_seed=3)
    area, vol = orc.tet4_geometry(m.coords, m.conn, m.edges)
    assert np.abs(m.area - area).max() <= 1e-14 * np.abs(area).max()
    assert np.abs(m.dualvol - vol).max() <= 1e-14 * vol.max()
