"""Boundary face-IP kernels (continuity open, momentum open and symmetry,
scalar open) through the C ABI against the oracle, and the reference's
unit-cube golds on the GPU.

Tolerance: the running-magnitude bound of gpu_util (|gpu - oracle| <=
1e-12 S per entry, S from the oracle's *_local_mag kernels summed like the
values).
"""
import numpy as np
import pytest

import kat
from gpu_util import check_close, dev

pytestmark = pytest.mark.gpu

SIDES = ("x-", "x+", "y-", "y+", "z-", "z+")


def _mesh(nw, kind):
    if kind == "hex":
        return nw.Mesh(10, 8, 6, lx=1.0, ly=0.8, lz=0.5, stretch_z=1.15, jitter=0.15, seed=5)
    if kind == "tets":
        return nw.Mesh(6, 5, 4, jitter=0.1, seed=6, tets=True)
    if kind == "periodic":  # z sides only; their seam nodes are periodic slaves
        return nw.Mesh(8, 6, 5, periodic_x=True, periodic_y=True, jitter=0.1, seed=7)
    return nw.Mesh(7, 6, 5, jitter=0.1, seed=8, renumber=1, renumber_seed=3)


def _system(nw, mesh, nd):
    ls = nw.LinearSystem(nd)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    ls.finalize()
    ls.zero_system()
    return ls


def _oracle_sum(orc, mesh, nd, ipn, lhs, rhs, ml, mr):
    rp, ci, lid = orc.build_graph(mesh.nalu_id, mesh.edges, nd)
    vals, b, _, _ = orc.sum_into(ipn, nd, lhs, rhs, lid, rp, ci, with_abs=False)
    va, ba, _, _ = orc.sum_into(ipn, nd, ml, mr, lid, rp, ci, with_abs=False)
    return vals, b, va, ba


def _node_fields(mesh, rng):
    N = mesh.num_nodes
    master = mesh.nalu_id - 1
    f = dict(coords=mesh.coords, velocity=rng.normal(0, 1, (N, 3)), dpdx=rng.normal(0, 1, (N, 3)),
             density=rng.uniform(0.8, 1.2, N), pressure=rng.normal(0, 1, N), pressure_bc=rng.normal(0, 1, N),
             udiag=rng.uniform(0.5, 2.0, N), dudx=rng.normal(0, 1, (N, 9)), viscosity=rng.uniform(0.01, 0.2, N),
             velocity_bc=rng.normal(0, 1, (N, 3)), q=rng.normal(0, 1, N), q_bc=rng.normal(0, 1, N))
    for k, v in f.items():  # slaves carry their master's values
        if k != "coords":
            f[k] = np.ascontiguousarray(v[master])
    return f


@pytest.mark.parametrize("kind", ["hex", "tets", "periodic", "renumbered"])
def test_continuity_open_matches_oracle(nw, orc, kind):
    mesh = _mesh(nw, kind)
    rng = np.random.default_rng(11)
    f = _node_fields(mesh, rng)
    ipn, area = mesh.face_ips(("x+", "y-", "z+") if kind != "periodic" else ("z-", "z+"))
    dynp = rng.normal(0, 0.1, len(ipn))
    ls = _system(nw, mesh, 1)
    ss = ls.sideset(ipn)
    d = {k: dev(v) for k, v in dict(f, area=area, dynp=dynp).items()}
    fld = nw.ContinuityOpenFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dpdx", "density", "pressure",
                                                               "pressure_bc", "udiag", "area", "dynp")))
    oo = dict(tau_scale=0.7, noc_fac=1.0, pstab_fac=1.0, mdot_corr=0.01, solve_incompressible=0.0)
    ls.assemble_continuity_open(ss, fld, nw.ContinuityOpenOpts(**oo))
    vals, rhs = ls.to_host()
    o = orc.ContinuityOpenOpts(**oo)
    args = (ipn, f["coords"], f["velocity"], f["dpdx"], f["density"], f["pressure"], f["pressure_bc"],
            f["udiag"], area, dynp, o)
    ref = _oracle_sum(orc, mesh, 1, ipn, *orc.continuity_open_local(*args),
                      *orc.continuity_open_local(*args, mag=True))
    check_close(vals, ref[0], ref[2], "values")
    check_close(rhs, ref[1], ref[3], "rhs")
    n, rows = ss.sizes()
    assert n == len(ipn) and 0 < rows <= len(ipn)


@pytest.mark.parametrize("entrain", [0, 1])
@pytest.mark.parametrize("kind", ["hex", "tets", "periodic"])
def test_momentum_open_matches_oracle(nw, orc, kind, entrain):
    mesh = _mesh(nw, kind)
    rng = np.random.default_rng(12)
    f = _node_fields(mesh, rng)
    ipn, area = mesh.face_ips(SIDES)
    mdot = rng.normal(0, 0.05, len(ipn))  # both signs: outflow and entrainment
    ls = _system(nw, mesh, 3)
    ss = ls.sideset(ipn)
    d = {k: dev(v) for k, v in dict(f, area=area, mdot=mdot).items()}
    fld = nw.MomentumOpenFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dudx", "viscosity",
                                                             "velocity_bc", "area", "mdot")))
    oo = dict(include_div_u=1.0, nf_entrain=0.3, entrainment=entrain)
    ls.assemble_momentum_open(ss, fld, nw.MomentumOpenOpts(**oo))
    vals, rhs = ls.to_host()
    o = orc.MomentumOpenOpts(**oo)
    args = (ipn, f["coords"], f["velocity"], f["dudx"], f["viscosity"], f["velocity_bc"], area, mdot, o)
    ref = _oracle_sum(orc, mesh, 3, ipn, *orc.momentum_open_local(*args), *orc.momentum_open_local(*args, mag=True))
    check_close(vals, ref[0], ref[2], "values")
    check_close(rhs, ref[1], ref[3], "rhs")


@pytest.mark.parametrize("penalty", [0.0, 2.0])
@pytest.mark.parametrize("kind", ["hex", "tets", "renumbered"])
def test_momentum_symmetry_matches_oracle(nw, orc, kind, penalty):
    mesh = _mesh(nw, kind)
    rng = np.random.default_rng(13)
    f = _node_fields(mesh, rng)
    ipn, area = mesh.face_ips(("y-", "y+", "z-"))
    ls = _system(nw, mesh, 3)
    ss = ls.sideset(ipn)
    d = {k: dev(v) for k, v in dict(f, area=area).items()}
    fld = nw.MomentumSymmetryFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dudx", "viscosity", "area")))
    oo = dict(include_div_u=1.0, penalty_factor=penalty)
    ls.assemble_momentum_symmetry(ss, fld, nw.MomentumSymmetryOpts(**oo))
    vals, rhs = ls.to_host()
    o = orc.MomentumSymmetryOpts(**oo)
    args = (ipn, f["coords"], f["velocity"], f["dudx"], f["viscosity"], area, o)
    ref = _oracle_sum(orc, mesh, 3, ipn, *orc.momentum_symmetry_local(*args),
                      *orc.momentum_symmetry_local(*args, mag=True))
    check_close(vals, ref[0], ref[2], "values")
    check_close(rhs, ref[1], ref[3], "rhs")


@pytest.mark.parametrize("kind", ["hex", "tets"])
def test_scalar_open_matches_oracle(nw, orc, kind):
    mesh = _mesh(nw, kind)
    rng = np.random.default_rng(14)
    f = _node_fields(mesh, rng)
    ipn, area = mesh.face_ips(("x-", "x+"))
    mdot = rng.normal(0, 0.05, len(ipn))
    ls = _system(nw, mesh, 1)
    ss = ls.sideset(ipn)
    d = {k: dev(v) for k, v in dict(q=f["q"], q_bc=f["q_bc"], mdot=mdot).items()}
    ls.assemble_scalar_open(ss, nw.ScalarOpenFields(d["q"].data_ptr(), d["q_bc"].data_ptr(), d["mdot"].data_ptr()),
                            relax=0.7)
    vals, rhs = ls.to_host()
    args = (ipn, f["q"], f["q_bc"], mdot)
    ref = _oracle_sum(orc, mesh, 1, ipn, *orc.scalar_open_local(*args, relax=0.7),
                      *orc.scalar_open_local(*args, relax=0.7, mag=True))
    check_close(vals, ref[0], ref[2], "values")
    check_close(rhs, ref[1], ref[3], "rhs")


def _dense(nw, ls, nd, n_nodes):
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    A = np.zeros((n_nodes * nd, n_nodes * nd))
    for r in range(len(rp) - 1):
        A[r, ci[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
    return A, rhs


def test_unit_cube_golds_on_the_gpu(nw, orc, golds):
    """The reference's open / symmetry known answers through the C ABI."""
    mesh = nw.Mesh(1, 1, 1)
    ipn, area = mesh.face_ips(("x+",))
    c = kat.continuity_open_fixture(orc)
    ls = _system(nw, mesh, 1)
    ss = ls.sideset(ipn)
    d = {k: dev(v) for k, v in dict(coords=c["coords"], velocity=c["velocity"], dpdx=c["dpdx"], density=c["density"],
                                     pressure=c["pressure"], pbc=c["pressure_bc"], udiag=c["udiag"], area=area,
                                     dynp=c["dynp"]).items()}
    ls.assemble_continuity_open(ss, nw.ContinuityOpenFields(*(d[k].data_ptr() for k in (
        "coords", "velocity", "dpdx", "density", "pressure", "pbc", "udiag", "area", "dynp"))),
        nw.ContinuityOpenOpts(**c["open_opts"]))
    A, b = _dense(nw, ls, 1, 8)
    g = golds["continuity_open_hex8_xplus"]
    np.testing.assert_allclose(A.ravel(), g["lhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(b, g["rhs"], rtol=0, atol=1e-12)

    m = kat.momentum_face_fixture(orc)
    d = {k: dev(v) for k, v in dict(coords=m["coords"], velocity=m["velocity"], dudx=m["dudx"],
                                     viscosity=m["viscosity"], ubc=m["velocity_bc"], area=area,
                                     mdot=m["open_mdot"]).items()}
    ls = _system(nw, mesh, 3)
    ss = ls.sideset(ipn)
    ls.assemble_momentum_open(ss, nw.MomentumOpenFields(*(d[k].data_ptr() for k in (
        "coords", "velocity", "dudx", "viscosity", "ubc", "area", "mdot"))),
        nw.MomentumOpenOpts(0.0, 0.0, nw.ENTRAIN_COMPUTED))
    A, b = _dense(nw, ls, 3, 8)
    g = golds["momentum_open_hex8_xplus"]
    np.testing.assert_allclose(A.ravel(), g["lhs"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(b, g["rhs"], rtol=0, atol=1e-12)

    g = golds["momentum_symmetry_hex8_xplus"]
    dof = (3 * m["conn"][0][:, None] + np.arange(3)).ravel()
    for case, pen in enumerate(g["penalty_factor"]):
        ls = _system(nw, mesh, 3)
        ss = ls.sideset(ipn)
        ls.assemble_momentum_symmetry(ss, nw.MomentumSymmetryFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dudx", "viscosity", "area"))), nw.MomentumSymmetryOpts(0.0, pen))
        A, b = _dense(nw, ls, 3, 8)
        np.testing.assert_allclose(A[np.ix_(dof, dof)].ravel(), g["lhs"][case], rtol=0, atol=1e-12)
        np.testing.assert_allclose(b[dof], g["rhs"][case], rtol=0, atol=1e-12)


def test_boundary_adds_to_the_interior_assembly(nw, orc):
    """Interior continuity edges, then the open boundary: the sum matches the
    oracle's interior + boundary contributions."""
    from gpu_util import continuity_fields, oracle_continuity
    mesh = _mesh(nw, "hex")
    rng = np.random.default_rng(15)
    f = _node_fields(mesh, rng)
    ipn, area = mesh.face_ips(SIDES)
    ls = _system(nw, mesh, 1)
    ss = ls.sideset(ipn)
    d = {k: dev(v) for k, v in dict(f, area=mesh.area, farea=area).items()}
    co = nw.ContinuityOpts(1.0, 0.7, 1.0, 0.0)
    ls.assemble_continuity(continuity_fields(nw, d), co)
    oo = dict(tau_scale=0.7, noc_fac=1.0, pstab_fac=1.0, mdot_corr=0.0, solve_incompressible=0.0)
    ls.assemble_continuity_open(ss, nw.ContinuityOpenFields(*(d[k].data_ptr() for k in (
        "coords", "velocity", "dpdx", "density", "pressure", "pressure_bc", "udiag", "farea")), None),
        nw.ContinuityOpenOpts(**oo))
    vals, rhs = ls.to_host()
    hi = oracle_continuity(orc, mesh.edges, mesh.nalu_id, dict(f, area=mesh.area),
                           {k: getattr(co, k) for k, _ in co._fields_})
    args = (ipn, f["coords"], f["velocity"], f["dpdx"], f["density"], f["pressure"], f["pressure_bc"],
            f["udiag"], area, None, orc.ContinuityOpenOpts(**oo))
    bo = _oracle_sum(orc, mesh, 1, ipn, *orc.continuity_open_local(*args),
                     *orc.continuity_open_local(*args, mag=True))
    check_close(vals, hi["vals"] + bo[0], hi["vabs"] + bo[2], "values")
    check_close(rhs, hi["rhs"] + bo[1], hi["rabs"] + bo[3], "rhs")


def test_side_set_errors(nw):
    mesh = _mesh(nw, "hex")
    ls = _system(nw, mesh, 1)
    with pytest.raises(nw.NwError, match="not joined"):
        ls.sideset(np.array([[0, mesh.num_nodes - 1]]))
    with pytest.raises(nw.NwError, match="out of range"):
        ls.sideset(np.array([[0, mesh.num_nodes]]))
    ipn, area = mesh.face_ips(("x+",))
    ss = ls.sideset(ipn)
    z = dev(np.zeros(mesh.num_nodes * 9))
    with pytest.raises(nw.NwError, match="num_dof 3"):
        ls.assemble_momentum_symmetry(ss, nw.MomentumSymmetryFields(*(z.data_ptr(),) * 5),
                                      nw.MomentumSymmetryOpts(0.0, 0.0))
    ls3 = _system(nw, mesh, 3)
    with pytest.raises(nw.NwError, match="another linear system"):
        ls3.assemble_momentum_symmetry(ss, nw.MomentumSymmetryFields(*(z.data_ptr(),) * 5),
                                       nw.MomentumSymmetryOpts(0.0, 0.0))
    empty = ls.sideset(np.zeros((0, 2), np.int64))
    assert empty.sizes() == (0, 0)
    ls.assemble_scalar_open(empty, nw.ScalarOpenFields(z.data_ptr(), z.data_ptr(), z.data_ptr()), relax=1.0)


@pytest.mark.parametrize("kind", ["hex", "tets", "periodic"])
def test_open_mdot_matches_oracle(nw, orc, kind):
    import torch
    mesh = _mesh(nw, kind)
    rng = np.random.default_rng(16)
    f = _node_fields(mesh, rng)
    ipn, area = mesh.face_ips(("z-", "z+") if kind == "periodic" else SIDES)
    dynp = rng.normal(0, 0.1, len(ipn))
    ls = _system(nw, mesh, 1)
    ss = ls.sideset(ipn)
    d = {k: dev(v) for k, v in dict(f, area=area, dynp=dynp).items()}
    fld = nw.ContinuityOpenFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dpdx", "density", "pressure",
                                                               "pressure_bc", "udiag", "area", "dynp")))
    for pstab in (1.0, 0.0):
        md = torch.zeros(len(ipn), dtype=torch.float64, device="cuda")
        total = ls.open_mdot(ss, fld, md, noc_fac=1.0, pstab_fac=pstab)
        ref = orc.mdot_open(ipn, f["coords"], f["velocity"], f["dpdx"], f["density"], f["pressure"],
                            f["pressure_bc"], f["udiag"], area, dynp, noc_fac=1.0, pstab_fac=pstab)
        got = md.cpu().numpy()
        # running magnitude of each IP's formula
        R, L = ipn[:, 0], ipn[:, 1]
        A = np.abs(area)
        pts = pstab / np.abs(f["udiag"][R])
        dx = 0.5 * np.abs(f["coords"][R] - f["coords"][L])
        asq = (A * A).sum(1)
        axdx = np.abs(np.einsum("id,id->i", area, 0.5 * (f["coords"][R] - f["coords"][L])))
        G = np.abs(f["dpdx"][R])
        S = pts * (np.abs(f["pressure_bc"][R]) + np.abs(dynp) + np.abs(f["pressure"][R]) + np.abs(f["pressure"][L])) \
            * asq / axdx + ((np.abs(f["density"][R, None] * f["velocity"][R]) + pts[:, None] * G) * A).sum(1) \
            + (pts[:, None] * (A + asq[:, None] / axdx[:, None] * dx) * G).sum(1)
        check_close(got, ref, S, "open mdot")
        assert abs(total - got.sum()) <= 1e-12 * S.sum()
        # deterministic: a second call gives the same bits
        md2 = torch.zeros_like(md)
        assert ls.open_mdot(ss, fld, md2, noc_fac=1.0, pstab_fac=pstab) == total
        assert torch.equal(md, md2)


def test_open_mdot_golds_on_the_gpu(nw, golds):
    import torch
    mesh = nw.Mesh(1, 1, 1)
    g = golds["mdot_open_hex8_zplus"]
    ipn, area = mesh.face_ips(("z+",))
    ls = _system(nw, mesh, 1)
    ss = ls.sideset(ipn)
    N = 8
    d = {k: dev(v) for k, v in dict(coords=mesh.coords, velocity=np.full((N, 3), g["velocity"]),
                                     dpdx=np.zeros((N, 3)), density=np.full(N, g["density"]), p=np.zeros(N),
                                     pbc=np.zeros(N), udiag=np.ones(N), area=area).items()}
    fld = nw.ContinuityOpenFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dpdx", "density", "p", "pbc",
                                                               "udiag", "area")), None)
    md = torch.zeros(len(ipn), dtype=torch.float64, device="cuda")
    assert abs(ls.open_mdot(ss, fld, md, pstab_fac=g["pstab_fac"]) - g["mdot_open"]) <= 1e-15
    # MdotAlgDriver's open correction on the z- side ("surface_5", 4 IPs),
    # the open field zero: correction (inflow + open) / 24 IPs
    c = golds["mdot_open_correction_hex8"]
    corr = (c["inflow"] + c["open"]) / c["ip_count"]
    assert corr == c["correction"]
    ipn5, _ = mesh.face_ips(("z-",))
    ss5 = ls.sideset(ipn5)
    md5 = torch.zeros(len(ipn5), dtype=torch.float64, device="cuda")
    assert abs(ls.correct_open_mdot(ss5, corr, md5) - c["post"]) <= 1e-15


def test_extract_diagonal_and_udiag_postprocess(nw, orc):
    """momentum_diag from the assembled momentum system (interior edges plus
    a symmetry boundary) against the oracle's per-local-system extraction,
    then the LowMach post-processing against its formula."""
    import torch
    case = nw.workload.lowmach_case(14, 12, 10, seed=4)
    mesh = case.mesh
    nd = case.node
    host = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
                density=nd["density"], mask=nd["mask"], area=mesh.area, mdot=case.edge["mdot"],
                pecfac=case.edge["pecfac"])
    d = {k: dev(v) for k, v in host.items()}
    mo = nw.MomentumOpts(alpha=0.2, alpha_upw=0.9, upw_factor=1.0, relax=0.7, include_div_u=1.0, use_limiter=0)
    ls = _system(nw, mesh, 3)
    ls.assemble_momentum(nw.MomentumFields(*(d[k].data_ptr() for k in (
        "coords", "velocity", "dudx", "viscosity", "density", "mask", "area", "mdot", "pecfac"))), mo)
    ipn, area = mesh.face_ips(("y-", "z+"))
    ss = ls.sideset(ipn)
    fa = dev(area)
    so = dict(include_div_u=1.0, penalty_factor=1.5)
    ls.assemble_momentum_symmetry(ss, nw.MomentumSymmetryFields(d["coords"].data_ptr(), d["velocity"].data_ptr(),
                                                                d["dudx"].data_ptr(), d["viscosity"].data_ptr(),
                                                                fa.data_ptr()), nw.MomentumSymmetryOpts(**so))
    N = mesh.num_nodes
    ud = torch.zeros(N, dtype=torch.float64, device="cuda")
    ls.extract_diagonal(ud, dof=0)
    om = orc.MomentumOpts(**{k: getattr(mo, k) for k, _ in mo._fields_})
    eargs = (mesh.edges, mesh.coords, nd["velocity"], nd["velocity"], nd["dudx"], nd["viscosity"], nd["density"],
             nd["mask"], mesh.area, case.edge["mdot"], case.edge["pecfac"], om)
    sargs = (ipn, mesh.coords, nd["velocity"], nd["dudx"], nd["viscosity"], area, orc.MomentumSymmetryOpts(**so))
    ref = orc.extract_diagonal(mesh.edges, orc.momentum_local(*eargs)[0], 3, N) + \
        orc.extract_diagonal(ipn, orc.momentum_symmetry_local(*sargs)[0], 3, N)
    S = orc.extract_diagonal(mesh.edges, orc.momentum_local(*eargs, mag=True)[0], 3, N) + \
        orc.extract_diagonal(ipn, orc.momentum_symmetry_local(*sargs, mag=True)[0], 3, N)
    check_close(ud.cpu().numpy(), ref, S, "momentum_diag")
    rng = np.random.default_rng(7)
    rho, vol = rng.uniform(0.8, 1.2, N), mesh.dualvol
    dt, g1, relax = 0.05, 1.5, 0.7
    ls.udiag_postprocess(dev(rho), dev(vol), ud, dt=dt, gamma1=g1, relax=relax)
    exp = (ref / (rho * vol) - g1 / dt) * relax + g1 / dt
    scale = (S / (rho * vol) + g1 / dt) * relax + g1 / dt
    check_close(ud.cpu().numpy(), exp, scale, "post-processed momentum_diag")


@pytest.mark.parametrize("kind", ["hex", "tets"])
def test_abl_wall_function_matches_oracle(nw, orc, kind):
    """Stable, unstable and neutral nodes (heat flux of both signs and zero)
    on the z- side."""
    mesh = _mesh(nw, kind)
    rng = np.random.default_rng(17)
    N = mesh.num_nodes
    ipn, area = mesh.face_ips(("z-",))
    n = len(ipn)
    hf = rng.choice([-1.0, 0.0, 1.0], N) * rng.uniform(0.01, 0.2, N)
    host = dict(vel=rng.normal(0, 1, (N, 3)), bcvel=rng.normal(0, 0.1, (N, 3)), rho=rng.uniform(0.9, 1.3, N),
                hf=hf, cp=rng.uniform(900, 1100, N), area=area, ustar=rng.uniform(0.1, 0.6, n),
                zh=rng.uniform(0.5, 3.0, n))
    d = {k: dev(v) for k, v in host.items()}
    oo = dict(gravity=9.81, z0=0.05, Tref=300.0, kappa=0.41, beta_m=5.0, gamma_m=16.0)
    ls = _system(nw, mesh, 3)
    ss = ls.sideset(ipn)
    ls.assemble_momentum_abl_wall(ss, nw.AblWallFields(*(d[k].data_ptr() for k in (
        "vel", "bcvel", "rho", "hf", "cp", "area", "ustar", "zh"))), nw.AblWallOpts(**oo))
    vals, rhs = ls.to_host()
    args = (ipn, host["vel"], host["bcvel"], host["rho"], host["hf"], host["cp"], area, host["ustar"], host["zh"],
            orc.AblWallOpts(**oo))
    ref = _oracle_sum(orc, mesh, 3, ipn, *orc.abl_wall_local(*args), *orc.abl_wall_local(*args, mag=True))
    check_close(vals, ref[0], ref[2], "values")
    check_close(rhs, ref[1], ref[3], "rhs")


def test_abl_wall_function_gold_on_the_gpu(nw, golds):
    g = golds["abl_wall_function_quad4_zminus"]
    ustar = g["kappa"] * g["uh"] / np.log(g["zh"] / g["z0"])
    mesh = nw.Mesh(1, 1, 1)
    ipn, area = mesh.face_ips(("z-",))
    N = 8
    d = {k: dev(v) for k, v in dict(vel=np.tile([g["uh"], 0.0, 0.0], (N, 1)), bcvel=np.zeros((N, 3)),
                                     rho=np.full(N, g["density"]), hf=np.full(N, g["heat_flux"]),
                                     cp=np.full(N, g["specific_heat"]), area=area, ustar=np.full(4, ustar),
                                     zh=np.full(4, g["zh"])).items()}
    ls = _system(nw, mesh, 3)
    ls.assemble_momentum_abl_wall(ls.sideset(ipn), nw.AblWallFields(*(d[k].data_ptr() for k in (
        "vel", "bcvel", "rho", "hf", "cp", "area", "ustar", "zh"))),
        nw.AblWallOpts(g["gravity"], g["z0"], g["Tref"], g["kappa"], 5.0, 16.0))
    A, b = _dense(nw, ls, 3, N)
    lexact = ustar * g["kappa"] / np.log(g["zh"] / g["z0"]) * 0.25
    for node in range(4):
        np.testing.assert_allclose(np.diag(A)[3 * node:3 * node + 3], [lexact, lexact, 0.0], rtol=0, atol=1e-12)
        np.testing.assert_allclose(b[3 * node:3 * node + 3], [-ustar * ustar * 0.25, 0.0, 0.0], rtol=0, atol=1e-12)
    assert np.abs(A - np.diag(np.diag(A))).max() <= 1e-12 and np.all(b[12:] == 0.0)


@pytest.mark.parametrize("slip", [True, False])
@pytest.mark.parametrize("kind", ["hex", "tets", "periodic"])
def test_abl_wall_shear_stress_matches_oracle(nw, orc, kind, slip):
    """rhs-only wall stress on the face nodes (slip) or their opposing nodes
    (no slip; on tets three face IPs share one opposing node)."""
    mesh = _mesh(nw, kind)
    rng = np.random.default_rng(18)
    ipn, area = mesh.face_ips(("z-",))
    tau = rng.normal(0, 1, (len(ipn), 3))
    ls = _system(nw, mesh, 3)
    ss = ls.sideset(ipn)
    ls.assemble_momentum_abl_wall_shear_stress(ss, dev(area), dev(tau), slip=slip)
    vals, rhs = ls.to_host()
    ref = _oracle_sum(orc, mesh, 3, ipn, *orc.abl_shear_local(ipn, area, tau, slip),
                      *orc.abl_shear_local(ipn, area, tau, slip, mag=True))
    check_close(rhs, ref[1], ref[3], "rhs")
    assert np.all(vals == 0.0)
