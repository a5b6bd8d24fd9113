"""GPU edge assembly through the C ABI vs the CPU oracle and the reference
golds. Tolerances: see gpu_util.check_close (1e-12 relative to the summed
magnitudes); the CSR graph must be bit-exact."""
import numpy as np
import pytest

import kat
from gpu_util import (check_close, continuity_fields, dev, momentum_fields, oracle_continuity,
                      oracle_momentum, oracle_scalar, scalar_fields, to_dev_dict)

pytestmark = pytest.mark.gpu


def _linsys(nw, num_dof, N, edges, gid=None, nid=None):
    ls = nw.LinearSystem(num_dof)
    ls.build_edge_graph(N, edges, gid, nid)
    ls.finalize()
    return ls


# ---------------------------------------------------------------- golds
def test_gpu_scalar_matches_reference_golds(nw, orc, golds):
    m = kat.scalar_fixture(orc)
    g = golds["scalar_adv_diff_hex8"]
    ls = _linsys(nw, 1, 8, m["edges"])
    rp, ci = ls.graph()
    assert rp.tolist() == g["rowOffsets_serial"] and ci.tolist() == g["cols_serial"]
    d = to_dev_dict(dict(coords=m["coords"], velocity=m["velocity"], q=m["q"], dqdx=m["dqdx"],
                         density=m["density"], diff=m["diff"], area=m["area"], mdot=m["mdot"]))
    ls.zero_system()
    ls.assemble_scalar(scalar_fields(nw, d), nw.ScalarOpts(**m["opts"]))
    vals, rhs = ls.to_host()
    np.testing.assert_allclose(vals, g["vals_serial"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(rhs, g["rhs_serial"], rtol=0, atol=1e-14)
    # FixPressureAtNode (resetRows) and Dirichlet variants
    ls.reset_rows(1, dev(np.array([0], np.int64)), 0, 1, 1.0, 1.0 - m["density"][0])
    vals, rhs = ls.to_host()
    np.testing.assert_allclose(vals, g["fixed_vals_serial"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(rhs, g["fixed_rhs_serial"], rtol=0, atol=1e-14)
    q = np.full(8, 2.0)
    bc = np.zeros(8)
    bc[0] = 1.0
    ls.apply_dirichlet(8, dev(np.arange(8, dtype=np.int64)), 0, 1, dev(q), dev(bc))
    vals, rhs = ls.to_host()
    np.testing.assert_allclose(vals, g["dirichlet_vals_serial"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(rhs, g["dirichlet_rhs_serial"], rtol=0, atol=1e-14)


def _csr_to_dense(rp, ci, vals, n):
    A = np.zeros((n, n))
    for r in range(n):
        A[r, ci[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
    return A


def test_gpu_continuity_matches_reference_golds(nw, orc, golds):
    m = kat.continuity_fixture(orc)
    ls = _linsys(nw, 1, 8, m["edges"])
    d = to_dev_dict(dict(coords=m["coords"], velocity=m["velocity"], dpdx=m["dpdx"], density=m["density"],
                         pressure=m["pressure"], udiag=m["udiag"], area=m["area"]))
    ls.zero_system()
    ls.assemble_continuity(continuity_fields(nw, d), nw.ContinuityOpts(**m["opts"]))
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    g = golds["continuity_hex8"]
    np.testing.assert_allclose(_csr_to_dense(rp, ci, vals, 8).ravel(), g["lhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(rhs, g["rhs"], rtol=0, atol=1e-12)


def test_gpu_momentum_matches_reference_golds(nw, orc, golds):
    m = kat.momentum_fixture(orc)
    ls = _linsys(nw, 3, 8, m["edges"])
    d = to_dev_dict(dict(coords=m["coords"], velocity=m["velocity"], dudx=m["dudx"], viscosity=m["viscosity"],
                         density=m["density"], mask=m["mask"], area=m["area"], mdot=m["mdot"],
                         pecfac=m["pecfac"]))
    ls.zero_system()
    ls.assemble_momentum(momentum_fields(nw, d), nw.MomentumOpts(**m["opts"]))
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    A = _csr_to_dense(rp, ci, vals, 24)
    g = golds["momentum_hex8"]
    gl = np.array(g["lhs"]).reshape(24, 24)
    same = (np.arange(24)[:, None] % 3) == (np.arange(24)[None, :] % 3)
    # the reference's dense test backend keeps same-component couplings only
    np.testing.assert_allclose(A[same], gl[same], rtol=0, atol=1e-12)
    np.testing.assert_allclose(rhs, g["rhs"], rtol=0, atol=1e-12)
    # all couplings (cross-component lhsfacNS terms included) vs the oracle
    o = oracle_momentum(orc, m["edges"], np.arange(1, 9), dict(m, coords=m["coords"]), m["opts"])
    check_close(vals, o["vals"], o["vabs"], "momentum values")


# ---------------------------------------------------------------- workloads
def test_gpu_scalar_periodic_32cube_parity_and_determinism(nw, orc):
    wl = nw.workload
    case = wl.scalar_case(32, seed=1)
    mesh = case.mesh
    f = dict(coords=mesh.coords, velocity=case.node["velocity"], q=case.node["q"], dqdx=case.node["dqdx"],
             density=case.node["density"], diff=case.node["diff_coeff"], area=mesh.area, mdot=case.edge["mdot"])
    o = case.opts["scalar"]
    od = {k: getattr(o, k) for k, _ in o._fields_}
    ref = oracle_scalar(orc, mesh.edges, mesh.nalu_id, f, od)
    ls = _linsys(nw, 1, mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    rp, ci = ls.graph()
    np.testing.assert_array_equal(rp, ref["rp"])
    np.testing.assert_array_equal(ci, ref["ci"])
    d = to_dev_dict(f)
    runs = []
    for _ in range(2):
        ls.zero_system()
        ls.assemble_scalar(scalar_fields(nw, d), o)
        runs.append(ls.to_host())
    check_close(runs[0][0], ref["vals"], ref["vabs"], "scalar values")
    check_close(runs[0][1], ref["rhs"], ref["rabs"], "scalar rhs")
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    # Dirichlet rows on z faces
    nodes = case.extra["dirichlet_nodes"]
    ls.apply_dirichlet(len(nodes), dev(nodes), 0, 1, d["q"], dev(case.node["bc"]))
    vals, rhs = ls.to_host()
    ov, orr = ref["vals"].copy(), ref["rhs"].copy()
    orc.apply_dirichlet(nodes, 1, 0, 1, case.node["q"], case.node["bc"], ref["lid"], ref["rp"], ref["ci"], ov, orr)
    check_close(vals, ov, ref["vabs"], "dirichlet values")
    check_close(rhs, orr, np.maximum(ref["rabs"], np.abs(orr)), "dirichlet rhs")


@pytest.mark.parametrize("shape", [(24, 20, 12), (128, 128, 64)])
def test_gpu_lowmach_momentum_continuity_parity(nw, orc, shape):
    case = nw.workload.lowmach_case(*shape, seed=2)
    mesh = case.mesh
    nd = case.node
    fc = dict(coords=mesh.coords, velocity=nd["velocity"], dpdx=nd["dpdx"], density=nd["density"],
              pressure=nd["pressure"], udiag=nd["udiag"], area=mesh.area)
    fm = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
              density=nd["density"], mask=nd["mask"], area=mesh.area, mdot=case.edge["mdot"],
              pecfac=case.edge["pecfac"])
    co, mo = case.opts["continuity"], case.opts["momentum"]
    cod = {k: getattr(co, k) for k, _ in co._fields_}
    mod = {k: getattr(mo, k) for k, _ in mo._fields_}
    # continuity
    ref = oracle_continuity(orc, mesh.edges, mesh.nalu_id, fc, cod)
    ls = _linsys(nw, 1, mesh.num_nodes, mesh.edges)
    ls.zero_system()
    ls.assemble_continuity(continuity_fields(nw, to_dev_dict(fc)), co)
    vals, rhs = ls.to_host()
    np.testing.assert_array_equal(ls.graph()[1], ref["ci"])
    check_close(vals, ref["vals"], ref["vabs"], "continuity values")
    check_close(rhs, ref["rhs"], ref["rabs"], "continuity rhs")
    # momentum (3 dof)
    ref = oracle_momentum(orc, mesh.edges, mesh.nalu_id, fm, mod)
    ls3 = _linsys(nw, 3, mesh.num_nodes, mesh.edges)
    ls3.zero_system()
    ls3.assemble_momentum(momentum_fields(nw, to_dev_dict(fm)), mo)
    vals, rhs = ls3.to_host()
    rp, ci = ls3.graph()
    np.testing.assert_array_equal(rp, ref["rp"])
    np.testing.assert_array_equal(ci, ref["ci"])
    check_close(vals, ref["vals"], ref["vabs"], "momentum values")
    check_close(rhs, ref["rhs"], ref["rabs"], "momentum rhs")


@pytest.mark.parametrize("renumber", [1, 2])
def test_gpu_tet_momentum_continuity_parity_40cube(nw, orc, renumber):
    """The tet workload of the implicit step at 40^3 hexes x 6 tets (68,921
    nodes, 5 % jitter), node ids randomly permuted (1) or permuted then
    RCM-renumbered (2): interior momentum (3 dof) and continuity assembly
    against the oracle."""
    case = nw.workload.lowmach_case(40, 40, 40, seed=5, stretch=1.0, jitter=0.05, lz=1.0, tets=True,
                                    renumber=renumber, renumber_seed=7)
    mesh, nd = case.mesh, case.node
    fm = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
              density=nd["density"], mask=nd["mask"], area=mesh.area, mdot=case.edge["mdot"],
              pecfac=case.edge["pecfac"])
    fc = dict(coords=mesh.coords, velocity=nd["velocity"], dpdx=nd["dpdx"], density=nd["density"],
              pressure=nd["pressure"], udiag=nd["udiag"], area=mesh.area)
    mo, co = case.opts["momentum"], case.opts["continuity"]
    for opts in (mo, nw.MomentumOpts(alpha=0.2, alpha_upw=0.6, upw_factor=1.0, relax=0.7, include_div_u=1.0,
                                     use_limiter=1)):
        mod = {k: getattr(opts, k) for k, _ in opts._fields_}
        ref = oracle_momentum(orc, mesh.edges, mesh.nalu_id, fm, mod)
        ls3 = _linsys(nw, 3, mesh.num_nodes, mesh.edges)
        ls3.zero_system()
        ls3.assemble_momentum(momentum_fields(nw, to_dev_dict(fm)), opts)
        vals, rhs = ls3.to_host()
        np.testing.assert_array_equal(ls3.graph()[1], ref["ci"])
        check_close(vals, ref["vals"], ref["vabs"], f"tet momentum values (order {renumber})")
        check_close(rhs, ref["rhs"], ref["rabs"], f"tet momentum rhs (order {renumber})")
    cod = {k: getattr(co, k) for k, _ in co._fields_}
    ref = oracle_continuity(orc, mesh.edges, mesh.nalu_id, fc, cod)
    ls = _linsys(nw, 1, mesh.num_nodes, mesh.edges)
    ls.zero_system()
    ls.assemble_continuity(continuity_fields(nw, to_dev_dict(fc)), co)
    vals, rhs = ls.to_host()
    check_close(vals, ref["vals"], ref["vabs"], f"tet continuity values (order {renumber})")
    check_close(rhs, ref["rhs"], ref["rabs"], f"tet continuity rhs (order {renumber})")


def test_gpu_poisson_continuity_parity_256x256x128(nw, orc):
    """The full pressure-Poisson matrix of the solver benchmark (256 x 256 x
    128 stretched box: 8,520,321 rows, 59,377,537 nnz) against the oracle."""
    import torch
    case = nw.workload.poisson_case(256, 256, 128, seed=3, stretch=1.04)
    mesh, nd = case.mesh, case.node
    fc = dict(coords=mesh.coords, velocity=nd["velocity"], dpdx=nd["dpdx"], density=nd["density"],
              pressure=nd["pressure"], udiag=nd["udiag"], area=mesh.area)
    co = case.opts["continuity"]
    ref = oracle_continuity(orc, mesh.edges, mesh.nalu_id, fc, {k: getattr(co, k) for k, _ in co._fields_})
    ls = _linsys(nw, 1, mesh.num_nodes, mesh.edges)
    ls.zero_system()
    ls.assemble_continuity(continuity_fields(nw, to_dev_dict(fc)), co)
    vals, rhs = ls.to_host()
    assert vals.shape[0] == 59_377_537
    np.testing.assert_array_equal(ls.graph()[0], ref["rp"])
    check_close(vals, ref["vals"], ref["vabs"], "poisson 256x256x128 values")
    check_close(rhs, ref["rhs"], ref["rabs"], "poisson 256x256x128 rhs")
    del ls
    torch.cuda.empty_cache()


@pytest.mark.parametrize("renumber", [1, 2])
def test_gpu_tet_continuity_parity(nw, orc, renumber):
    mesh = nw.Mesh(10, 9, 8, tets=True, jitter=0.05, seed=4, renumber=renumber, renumber_seed=11)
    rng = np.random.default_rng(5)
    N = mesh.num_nodes
    f = dict(coords=mesh.coords, velocity=rng.normal(size=(N, 3)), dpdx=rng.normal(size=(N, 3)),
             density=rng.uniform(0.5, 2, N), pressure=rng.normal(size=N), udiag=rng.uniform(1, 3, N),
             area=mesh.area)
    od = dict(noc_fac=1.0, tau_scale=0.5, interp_together=0.5, solve_incompressible=1.0)
    ref = oracle_continuity(orc, mesh.edges, mesh.nalu_id, f, od)
    ls = _linsys(nw, 1, N, mesh.edges)
    ls.zero_system()
    ls.assemble_continuity(continuity_fields(nw, to_dev_dict(f)), nw.ContinuityOpts(**od))
    vals, rhs = ls.to_host()
    check_close(vals, ref["vals"], ref["vabs"], "tet continuity values")
    check_close(rhs, ref["rhs"], ref["rabs"], "tet continuity rhs")


def test_gpu_scalar_limiter_tanh_relax_options(nw, orc):
    """Limiter, tanh Peclet form, relaxation and upwinding options."""
    mesh = nw.Mesh(9, 8, 7, stretch_z=1.1, jitter=0.08, seed=6)
    rng = np.random.default_rng(8)
    N = mesh.num_nodes
    f = dict(coords=mesh.coords, velocity=rng.normal(size=(N, 3)), q=rng.uniform(size=N),
             dqdx=rng.normal(size=(N, 3)), density=rng.uniform(0.5, 2, N), diff=rng.uniform(1e-3, 1e-1, N),
             area=mesh.area, mdot=rng.normal(size=mesh.num_edges))
    for od in (dict(alpha=0.3, alpha_upw=0.7, upw_factor=1.0, relax=0.8, hybrid_factor=1.0, use_limiter=1,
                    tanh_form=0, tanh_trans=2.0, tanh_width=4.0),
               dict(alpha=0.0, alpha_upw=1.0, upw_factor=0.5, relax=1.0, hybrid_factor=0.0, use_limiter=0,
                    tanh_form=1, tanh_trans=2.0, tanh_width=4.0)):
        ref = oracle_scalar(orc, mesh.edges, mesh.nalu_id, f, od)
        ls = _linsys(nw, 1, N, mesh.edges)
        ls.zero_system()
        ls.assemble_scalar(scalar_fields(nw, to_dev_dict(f)), nw.ScalarOpts(**od))
        vals, rhs = ls.to_host()
        check_close(vals, ref["vals"], ref["vabs"], "scalar values")
        check_close(rhs, ref["rhs"], ref["rabs"], "scalar rhs")


def test_gpu_momentum_options(nw, orc):
    mesh = nw.Mesh(8, 7, 6, stretch_z=1.05, jitter=0.06, seed=12)
    rng = np.random.default_rng(13)
    N, E = mesh.num_nodes, mesh.num_edges
    f = dict(coords=mesh.coords, velocity=rng.normal(size=(N, 3)), dudx=rng.normal(size=(N, 9)),
             viscosity=rng.uniform(1e-3, 1e-1, N), density=np.ones(N), mask=rng.choice([0.0, 1.0], N),
             area=mesh.area, mdot=rng.normal(size=E), pecfac=rng.uniform(size=E))
    od = dict(alpha=0.2, alpha_upw=0.6, upw_factor=1.0, relax=0.7, include_div_u=1.0, use_limiter=1)
    ref = oracle_momentum(orc, mesh.edges, mesh.nalu_id, f, od)
    ls = _linsys(nw, 3, N, mesh.edges)
    ls.zero_system()
    ls.assemble_momentum(momentum_fields(nw, to_dev_dict(f)), nw.MomentumOpts(**od))
    vals, rhs = ls.to_host()
    check_close(vals, ref["vals"], ref["vabs"], "momentum values")
    check_close(rhs, ref["rhs"], ref["rabs"], "momentum rhs")


def test_gpu_accumulating_assembly_and_sum_into(nw, orc):
    """A second algorithm sums into an already assembled system, and the
    host sumInto adds one entity block (LinearSystem::sumInto)."""
    m = kat.continuity_fixture(orc)
    ls = _linsys(nw, 1, 8, m["edges"])
    d = to_dev_dict(dict(coords=m["coords"], velocity=m["velocity"], dpdx=m["dpdx"], density=m["density"],
                         pressure=m["pressure"], udiag=m["udiag"], area=m["area"]))
    ls.zero_system()
    ls.assemble_continuity(continuity_fields(nw, d), nw.ContinuityOpts(**m["opts"]))
    v1, r1 = ls.to_host()
    ls.assemble_continuity(continuity_fields(nw, d), nw.ContinuityOpts(**m["opts"]))
    v2, r2 = ls.to_host()
    np.testing.assert_allclose(v2, 2 * v1, rtol=1e-15, atol=0)
    np.testing.assert_allclose(r2, 2 * r1, rtol=1e-15, atol=0)
    rp, ci = ls.graph()
    lhs = np.array([[1.0, 2.0], [3.0, 4.0]])
    ls.sum_into([0, 1], [0.5, -0.5], lhs)
    v3, r3 = ls.to_host()
    dv = v3 - v2
    A = _csr_to_dense(rp, ci, dv, 8)
    np.testing.assert_allclose(A[:2, :2], lhs)
    assert np.count_nonzero(dv) == 4
    np.testing.assert_allclose(r3[:2] - r2[:2], [0.5, -0.5])


def test_gpu_rejects_bad_dirichlet_nodes(nw, orc):
    m = kat.continuity_fixture(orc)
    ls = _linsys(nw, 1, 8, m["edges"])
    ls.zero_system()
    with pytest.raises(nw.NwError):
        ls.apply_dirichlet(1, dev(np.array([99], np.int64)), 0, 1, dev(np.zeros(8)), dev(np.zeros(8)))
