"""Pin the CPU oracle against the reference's own known-answer golds.

Golds: tests/golden/reference_golds.json (extracted from the nalu-wind unit
tests by tests/golden/make_golden.py). Tolerances are the reference tests'
own: 1e-14 for the Tpetra CSR values, 1e-12 for the dense edge systems.
"""
import numpy as np
import pytest

import kat


def scalar_system(orc, m):
    o = orc.ScalarOpts(**m["opts"])
    lhs, rhs = orc.scalar_local(m["edges"], m["coords"], m["velocity"], m["q"], m["dqdx"], m["density"],
                                m["diff"], m["area"], m["mdot"], o)
    rp, ci, lid = orc.build_graph(np.arange(1, 9), m["edges"], 1)
    vals, b, _, _ = orc.sum_into(m["edges"], 1, lhs, rhs, lid, rp, ci)
    return rp, ci, lid, vals, b


def test_geometry_unit_cube(orc, golds):
    m = kat.hex1(orc)
    g = golds["geometry_hex8_unit_cube"]
    assert m["edges"].shape[0] == g["num_edges"]
    np.testing.assert_allclose(m["dualvol"], g["dual_volume"], rtol=0, atol=1e-16)
    np.testing.assert_allclose((m["area"] ** 2).sum(1), g["area_mag_sq"], rtol=0, atol=1e-16)
    # node[0] is the lower id on every edge
    assert np.all(m["edges"][:, 0] < m["edges"][:, 1])


def test_mdot_unit_cube(orc, golds):
    m = kat.hex1(orc)
    g = golds["mdot_hex8_unit_cube"]
    v = np.full((8, 3), g["velocity"])
    md = orc.mdot_edge(m["edges"], m["coords"], v, np.zeros((8, 3)), np.full(8, g["density"]), np.zeros(8),
                       np.ones(8), m["area"])
    np.testing.assert_allclose(md, g["mdot"], rtol=0, atol=1e-14)


def test_peclet_functions(orc, golds):
    g = golds["peclet_classic"]
    for pe, f in zip(g["peclet"], g["factor"]):
        assert abs(orc.peclet_classic(pe, g["hybrid_factor"]) - f) < 1e-8
    g = golds["peclet_tanh"]
    for x, f in zip(g["x"], g["factor"]):
        assert abs(orc.peclet_tanh(x, g["c1"], g["c2"]) - f) < 1e-8


def test_scalar_tpetra_graph_and_values(orc, golds):
    m = kat.scalar_fixture(orc)
    g = golds["scalar_adv_diff_hex8"]
    rp, ci, lid, vals, b = scalar_system(orc, m)
    assert rp.tolist() == g["rowOffsets_serial"]
    assert ci.tolist() == g["cols_serial"]
    np.testing.assert_allclose(vals, g["vals_serial"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(b, g["rhs_serial"], rtol=0, atol=1e-14)


def test_scalar_fix_pressure_at_node(orc, golds):
    """FixPressureAtNodeAlgorithm resets node id 1's row to (1, rhs = ref - p)
    with p = density (UnitTestScalarAdvDiffEdge.C:229-293)."""
    m = kat.scalar_fixture(orc)
    g = golds["scalar_adv_diff_hex8"]
    rp, ci, lid, vals, b = scalar_system(orc, m)
    orc.reset_rows(np.array([0]), 0, 1, 1.0, 1.0 - m["density"][0], lid, rp, ci, vals, b)
    np.testing.assert_allclose(vals, g["fixed_vals_serial"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(b, g["fixed_rhs_serial"], rtol=0, atol=1e-14)


def test_scalar_dirichlet(orc, golds):
    """applyDirichletBCs on every node with q = 2, bc = 0 except node 1 = 1
    (UnitTestScalarAdvDiffEdge.C:295-381)."""
    m = kat.scalar_fixture(orc)
    g = golds["scalar_adv_diff_hex8"]
    rp, ci, lid, vals, b = scalar_system(orc, m)
    q = np.full(8, 2.0)
    bc = np.zeros(8)
    bc[0] = 1.0
    orc.apply_dirichlet(np.arange(8), 1, 0, 1, q, bc, lid, rp, ci, vals, b)
    np.testing.assert_allclose(vals, g["dirichlet_vals_serial"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(b, g["dirichlet_rhs_serial"], rtol=0, atol=1e-14)


def test_continuity_dense(orc, golds):
    m = kat.continuity_fixture(orc)
    o = orc.ContinuityOpts(**m["opts"])
    lhs, rhs = orc.continuity_local(m["edges"], m["coords"], m["velocity"], m["dpdx"], m["density"],
                                    m["pressure"], m["udiag"], m["area"], o)
    L, B = kat.dense_accumulate(m["edges"], lhs, rhs, 1, 8)
    g = golds["continuity_hex8"]
    np.testing.assert_allclose(L.ravel(), g["lhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(B, g["rhs"], rtol=0, atol=1e-12)


def test_momentum_dense_same_dof(orc, golds):
    m = kat.momentum_fixture(orc)
    o = orc.MomentumOpts(**m["opts"])
    lhs, rhs = orc.momentum_local(m["edges"], m["coords"], m["velocity"], m["velocity"], m["dudx"],
                                  m["viscosity"], m["density"], m["mask"], m["area"], m["mdot"],
                                  m["pecfac"], o)
    L, B = kat.dense_accumulate(m["edges"], lhs, rhs, 3, 8, same_dof_only=True)
    g = golds["momentum_hex8"]
    np.testing.assert_allclose(L.ravel(), g["lhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(B, g["rhs"], rtol=0, atol=1e-12)


def test_momentum_graph_block_structure(orc):
    """numDof = 3: every dof row of a node shares the node's column list,
    each column expanded to 3 consecutive columns
    (fill_in_extra_dof_rows_per_node, src/TpetraLinearSystemHelpers.C:361-381)."""
    m = kat.hex1(orc)
    rp1, ci1, _ = orc.build_graph(np.arange(1, 9), m["edges"], 1)
    rp3, ci3, lid3 = orc.build_graph(np.arange(1, 9), m["edges"], 3)
    assert rp3[-1] == 9 * rp1[-1]
    for r in range(8):
        cols1 = ci1[rp1[r]:rp1[r + 1]]
        expect = np.repeat(3 * cols1, 3) + np.tile(np.arange(3), len(cols1))
        for d in range(3):
            np.testing.assert_array_equal(ci3[rp3[3 * r + d]:rp3[3 * r + d + 1]], expect)
    np.testing.assert_array_equal(lid3, 3 * np.arange(8))


def test_threaded_sum_into_matches_serial(orc):
    """The OpenMP (atomic) sum_into agrees with the serial order to rounding."""
    m = kat.scalar_fixture(orc)
    o = orc.ScalarOpts(**m["opts"])
    lhs, rhs = orc.scalar_local(m["edges"], m["coords"], m["velocity"], m["q"], m["dqdx"], m["density"],
                                m["diff"], m["area"], m["mdot"], o)
    rp, ci, lid = orc.build_graph(np.arange(1, 9), m["edges"], 1)
    v1, b1, va, _ = orc.sum_into(m["edges"], 1, lhs, rhs, lid, rp, ci, nthreads=1)
    v4, b4, _, _ = orc.sum_into(m["edges"], 1, lhs, rhs, lid, rp, ci, nthreads=4)
    assert np.all(np.abs(v1 - v4) <= 1e-15 * va + 1e-300)


def test_oracle_gmres_solves_small_system(orc):
    """Restated GMRES / CG reach the requested relative residual."""
    m = kat.hex1(orc)
    rp, ci, lid = orc.build_graph(np.arange(1, 9), m["edges"], 1)
    # SPD Laplacian plus identity
    vals = np.zeros(ci.shape[0])
    for r in range(8):
        for p in range(rp[r], rp[r + 1]):
            vals[p] = 4.0 if ci[p] == r else -1.0
    b = np.arange(1.0, 9.0)
    for method in (0, 1):
        for pc in (0, 1, 2):
            x, hist, rep = orc.solve(rp, ci, vals, b, method=method, precond=pc, kspace=5, max_iters=60,
                                     tol=1e-12)
            assert rep.converged == 1
            r = b - orc.spmv(rp, ci, vals, x)
            assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(b)
            assert hist[0] == 1.0 and hist[-1] <= 1e-12


def test_oracle_sgs_is_forward_then_backward(orc):
    """Symmetric Gauss-Seidel with zero start equals the explicit
    (D + L)^-1 then (D + U)^-1 sweep pair."""
    rng = np.random.default_rng(0)
    n = 6
    A = rng.normal(size=(n, n)) + 8 * np.eye(n)
    rp = np.arange(0, n * n + 1, n, dtype=np.int64)
    ci = np.tile(np.arange(n, dtype=np.int32), n)
    x = rng.normal(size=n)
    y = orc.precond_apply(rp, ci, A.ravel(), 2, x)
    D = np.diag(np.diag(A))
    y1 = np.linalg.solve(np.tril(A), x)
    y2 = np.linalg.solve(np.triu(A), x - np.tril(A, -1) @ y1 - (np.triu(A, 1)) @ np.zeros(n))
    # backward sweep solves (D + U) y = x - L y1
    np.testing.assert_allclose(y, y2, rtol=1e-12, atol=1e-12)
    del D


def test_mass_bdf_node_kernels(orc, golds):
    """UnitTest{Momentum,Continuity,Scalar}MassBDFNodeKernel.C: only the
    current (Np1) states are filled by the fixtures; N and Nm1 stay zero."""
    m = kat.hex1(orc)
    V = m["dualvol"]
    z = np.zeros(8)
    dnv = (V, V, V)
    g = golds["momentum_mass_bdf_hex8"]
    cf = kat.continuity_fixture(orc)
    lhs, rhs = orc.mass_bdf(2, (z, z, np.ones(8)), dnv, q=(np.zeros((8, 3)), np.zeros((8, 3)),
                                                           kat.trig_velocity(m["coords"])),
                            dpdx=cf["dpdx"], dt=g["dt"], gamma=g["gamma"])
    np.testing.assert_allclose(rhs.ravel(), g["rhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(lhs, g["lhs_diag"], rtol=0, atol=1e-14)
    g = golds["continuity_mass_bdf_hex8"]
    lhs, rhs = orc.mass_bdf(1, (z, z, np.ones(8)), dnv, dt=g["dt"], gamma=g["gamma"])
    np.testing.assert_allclose(rhs, g["rhs"], rtol=0, atol=1e-12)
    assert np.all(lhs == 0.0)
    g = golds["scalar_mass_bdf_hex8"]
    sf = kat.scalar_fixture(orc)
    lhs, rhs = orc.mass_bdf(0, (z, z, sf["density"]), dnv, q=(z, z, sf["q"]), dt=g["dt"], gamma=g["gamma"])
    np.testing.assert_allclose(lhs, g["lhs_diag"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(rhs, g["rhs"], rtol=0, atol=1e-12)


def test_continuity_open_boundary(orc, golds):
    m = kat.continuity_open_fixture(orc)
    o = orc.ContinuityOpenOpts(**m["open_opts"])
    lhs, rhs = orc.continuity_open_local(m["ipn"], m["coords"], m["velocity"], m["dpdx"], m["density"],
                                         m["pressure"], m["pressure_bc"], m["udiag"], m["areav"], m["dynp"], o)
    L, B = kat.dense_accumulate(m["ipn"], lhs, rhs, 1, 8)
    g = golds["continuity_open_hex8_xplus"]
    np.testing.assert_allclose(L.ravel(), g["lhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(B, g["rhs"], rtol=0, atol=1e-12)


def test_momentum_open_boundary_computed_entrainment(orc, golds):
    m = kat.momentum_face_fixture(orc)
    o = orc.MomentumOpenOpts(include_div_u=0.0, nf_entrain=0.0, entrainment=0)
    lhs, rhs = orc.momentum_open_local(m["ipn"], m["coords"], m["velocity"], m["dudx"], m["viscosity"],
                                       m["velocity_bc"], m["areav"], m["open_mdot"], o)
    L, B = kat.dense_accumulate(m["ipn"], lhs, rhs, 3, 8)
    g = golds["momentum_open_hex8_xplus"]
    np.testing.assert_allclose(L.ravel(), g["lhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(B, g["rhs"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", [0, 1])
def test_momentum_symmetry_boundary(orc, golds, case):
    m = kat.momentum_face_fixture(orc)
    g = golds["momentum_symmetry_hex8_xplus"]
    o = orc.MomentumSymmetryOpts(include_div_u=0.0, penalty_factor=g["penalty_factor"][case])
    lhs, rhs = orc.momentum_symmetry_local(m["ipn"], m["coords"], m["velocity"], m["dudx"], m["viscosity"],
                                           m["areav"], o)
    L, B = kat.dense_accumulate(m["ipn"], lhs, rhs, 3, 8)
    # the gold is ordered by element node (check_against_gold_values)
    dof = (3 * m["conn"][0][:, None] + np.arange(3)).ravel()
    np.testing.assert_allclose(L[np.ix_(dof, dof)].ravel(), g["lhs"][case], rtol=0, atol=1e-12)
    np.testing.assert_allclose(B[dof], g["rhs"][case], rtol=0, atol=1e-12)


def test_scalar_open_boundary(orc, golds):
    g = golds["scalar_open_quad4"]
    tke, bc, mdot = orc.mt19937_uniform(g["draws"])
    n = g["nodes"]
    ipn = np.stack([np.arange(n), np.zeros(n, np.int64)], 1)
    for md in (mdot, -mdot):  # both branches of the upwind choice
        lhs, rhs = orc.scalar_open_local(ipn, np.full(n, tke), np.full(n, bc), np.full(n, md), relax=g["relax"])
        exp_rhs = -md * tke if md > 0 else -md * bc
        exp_lhs = md * 2.0 if md > 0 else 0.0
        np.testing.assert_allclose(rhs[:, 0], exp_rhs, rtol=0, atol=1e-12)
        np.testing.assert_allclose(lhs[:, 0], exp_lhs, rtol=0, atol=1e-12)
        assert np.all(lhs[:, 1:] == 0) and np.all(rhs[:, 1] == 0)


@pytest.mark.parametrize("method", [3, 4])
def test_oracle_bicgstab_tfqmr_solve_nonsymmetric_system(orc, method):
    """The restated Belos BiCGStab / TFQMR reach the tolerance on a
    nonsymmetric convection-diffusion matrix with every preconditioner; the
    reported history ends at or below the tolerance and the true residual
    agrees (BiCGStab) or lies below the TFQMR bound."""
    import scipy.sparse as sp
    n = 24
    T = sp.diags([-1.3, 4.0, -0.7], [-1, 0, 1], shape=(n, n))
    A = (sp.kron(sp.eye(n), T) + sp.kron(sp.diags([-1.1, 0.0, -0.9], [-1, 0, 1], shape=(n, n)), sp.eye(n))).tocsr()
    A.sort_indices()
    b = np.random.default_rng(0).normal(size=n * n)
    for pc in (0, 1, 2):
        x, h, rep = orc.solve(A.indptr, A.indices, A.data, b, method=method, precond=pc, max_iters=500, tol=1e-10)
        assert rep.converged == 1 and h[-1] <= 1e-10
        true = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
        assert true <= (1.01e-10 if method == 4 else 1e-9)


def test_open_mdot_unit_cube(orc, golds):
    """MdotOpenEdgeAlg on the z+ side ("surface_6") with rho = 1, u = 1,
    p = dpdx = 0 and the open correction active (pstabFac = 0)."""
    g = golds["mdot_open_hex8_zplus"]
    m = kat.hex1(orc)
    ipn = np.array([[4, 0], [5, 1], [7, 3], [6, 2]], np.int64)  # z+ side, opposed along z
    area = np.tile([0.0, 0.0, 0.25], (4, 1))
    N = 8
    md = orc.mdot_open(ipn, m["coords"], np.full((N, 3), g["velocity"]), np.zeros((N, 3)), np.full(N, g["density"]),
                       np.zeros(N), np.zeros(N), np.ones(N), area, None, noc_fac=1.0, pstab_fac=g["pstab_fac"])
    assert abs(md.sum() - g["mdot_open"]) <= 1e-15


def test_oracle_two_stage_sgs_limits(orc):
    """Two-stage SGS ("sgs2"): with many inner sweeps it is the exact
    natural-order symmetric Gauss-Seidel; with one it is a preconditioner
    between Jacobi and SGS in strength."""
    import scipy.sparse as sp
    n = 20
    T = sp.diags([-1.3, 4.0, -0.7], [-1, 0, 1], shape=(n, n))
    A = (sp.kron(sp.eye(n), T) + sp.kron(sp.diags([-1.1, 0.0, -0.9], [-1, 0, 1], shape=(n, n)), sp.eye(n))).tocsr()
    A.sort_indices()
    b = np.random.default_rng(1).normal(size=n * n)
    y_sgs = orc.precond_apply(A.indptr, A.indices, A.data, 2, b)
    y_ts = orc.precond_apply(A.indptr, A.indices, A.data, 4, b, inner_sweeps=300)
    assert np.abs(y_sgs - y_ts).max() <= 1e-13 * np.abs(y_sgs).max()
    its = {}
    for pc, inner in ((1, 1), (4, 1), (2, 1)):
        x, h, rep = orc.solve(A.indptr, A.indices, A.data, b, method=0, precond=pc, kspace=30, max_iters=500,
                              tol=1e-10, inner_sweeps=inner)
        assert rep.converged == 1 and np.linalg.norm(b - A @ x) <= 1.01e-10 * np.linalg.norm(b)
        its[pc] = rep.iterations
    assert its[2] <= its[4] <= its[1]


def test_abl_wall_function(orc, golds):
    """MomentumABLWallFuncEdgeKernel on the z- side of the unit cube, neutral
    (zero heat flux): lhs = u* kappa / ln(zh / z0) * 0.25 on the two
    tangential components, 0 on the normal one; rhs = (-u*^2 0.25, 0, 0)."""
    g = golds["abl_wall_function_quad4_zminus"]
    ustar = g["kappa"] * g["uh"] / np.log(g["zh"] / g["z0"])
    # z- side of the cube: ids (0, 2, 3, 1), opposed along z by (4, 6, 7, 5)
    ipn = np.array([[0, 4], [2, 6], [3, 7], [1, 5]], np.int64)
    area = np.tile([0.0, 0.0, -g["ip_area"]], (4, 1))
    N = 8
    vel = np.tile([g["uh"], 0.0, 0.0], (N, 1))
    o = orc.AblWallOpts(gravity=g["gravity"], z0=g["z0"], Tref=g["Tref"], kappa=g["kappa"], beta_m=5.0,
                        gamma_m=16.0)
    lhs, rhs = orc.abl_wall_local(ipn, vel, np.zeros((N, 3)), np.full(N, g["density"]), np.full(N, g["heat_flux"]),
                                  np.full(N, g["specific_heat"]), area, np.full(4, ustar), np.full(4, g["zh"]), o)
    L, B = kat.dense_accumulate(ipn, lhs, rhs, 3, N)
    lexact = ustar * g["kappa"] / np.log(g["zh"] / g["z0"]) * 0.25
    for node in range(4):  # the bottom nodes 0..3 carry one IP each
        for d, e in enumerate((lexact, lexact, 0.0)):
            assert abs(L[3 * node + d, 3 * node + d] - e) <= 1e-12
        np.testing.assert_allclose(B[3 * node:3 * node + 3], [-ustar * ustar * 0.25, 0.0, 0.0], rtol=0, atol=1e-12)
    off = L - np.diag(np.diag(L))
    assert np.abs(off).max() <= 1e-12
    assert np.all(B[12:] == 0.0)


@pytest.mark.parametrize("case", ["num_dof_1", "num_dof_3"])
def test_local_graph_arrays_insertion(orc, golds, case):
    """LocalGraphArrays (unit_tests/UnitTestLocalGraphArrays.C): unsorted
    inserts land sorted, numDof-expanded, and repeated inserts change
    nothing; every row is then full and colIndices[i] == i."""
    g = golds["local_graph_arrays"][case]
    nd = 3 if case == "num_dof_3" else 1
    out = orc.local_graph_replay(g["row_lengths"], [(r, c) for r, c in g["ops"]], num_dof=nd)
    assert out is not None
    rp, ci = out
    assert rp[-1] == sum(g["row_lengths"]) and np.array_equal(np.diff(rp), g["row_lengths"])
    assert np.array_equal(ci, np.arange(len(ci)))
    # one column too many overflows the pre-sized row
    assert orc.local_graph_replay([2], [(0, [0, 1, 2])], num_dof=1) is None


def test_nodal_grad_edge_linear_fields(orc, golds):
    """NodalGradEdgeAlg on the unit cube (interior edges only, divided by the
    dual volume) for phi = 2x + 2y + 2z and for u = (2x, 2y, 2z)."""
    g = golds["nodal_grad_edge_hex8"]
    m = kat.hex1(orc)
    x, y, z = m["coords"].T
    cx, cy, cz = g["coeff"]
    phi = (cx * x + cy * y + cz * z)[:, None]
    grad = orc.nodal_grad_edge(m["edges"], phi, m["area"], m["dualvol"], dim1=1)
    np.testing.assert_allclose(grad.ravel(), g["scalar"], rtol=0, atol=1e-15)
    u = np.stack([cx * x, cy * y, cz * z], 1)
    gu = orc.nodal_grad_edge(m["edges"], u, m["area"], m["dualvol"], dim1=3).reshape(8, 3, 3)
    diag = np.stack([gu[:, i, i] for i in range(3)], 1).ravel()
    np.testing.assert_allclose(diag, g["vector_diagonal"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("shifted", [False, True])
def test_nodal_grad_boundary_closure(orc, golds, shifted):
    """NodalGradBndryElemAlg on the unit cube's z- side for phi = 2x + 2y +
    2z: only the z component is non-zero, {-2, -4, -4, -6} interpolated and
    {0, -4, -4, -8} shifted at the side's nodes (ids 0..3)."""
    g = golds["nodal_grad_bndry_hex8_zminus"]
    m = kat.hex1(orc)
    x, y, z = m["coords"].T
    phi = (2 * x + 2 * y + 2 * z)[:, None]
    faces = np.array([[0, 2, 3, 1]], np.int64)  # z- side, outward (IP order)
    area = np.tile([0.0, 0.0, -0.25], (4, 1))
    grad = orc.nodal_grad_bndry(faces, area, phi, m["dualvol"], shifted=shifted)
    exp = g["shifted" if shifted else "unshifted"]
    np.testing.assert_allclose(grad[:4, 2], exp, rtol=0, atol=1e-15)
    assert np.all(grad[:4, :2] == 0.0) and np.all(grad[4:] == 0.0)
