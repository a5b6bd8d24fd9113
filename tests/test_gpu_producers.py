"""GPU input producers (mass flow rate, nodal gradient, Peclet factor)
against the oracle, through the C ABI.

Tolerance as for the assembly: |gpu - oracle| <= 1e-12 S per entry, S the
running magnitude of the entry (the formula evaluated on |inputs| with
|a - b| -> |a| + |b|, |a / b| -> |a| / |b|), computed here in numpy.
"""
import numpy as np
import pytest

from gpu_util import check_close, dev

pytestmark = pytest.mark.gpu


def _handle(nw, mesh, num_dof=1):
    ls = nw.LinearSystem(num_dof)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    ls.finalize()
    return ls


def _fields(case, rng):
    N = case.mesh.num_nodes
    nd = dict(case.node)
    nd["udiag"] = rng.uniform(0.5, 2.0, N)
    nd["density"] = rng.uniform(0.8, 1.2, N)
    nd["pressure"] = rng.normal(0.0, 1.0, N)
    nd["dpdx"] = rng.normal(0.0, 1.0, (N, 3))
    return nd


@pytest.mark.parametrize("interp", [1.0, 0.3])
def test_mdot_matches_oracle(nw, orc, interp):
    import torch
    case = nw.workload.lowmach_case(24, 20, 12, seed=2)
    mesh = case.mesh
    rng = np.random.default_rng(4)
    nd = _fields(case, rng)
    d = {k: dev(v) for k, v in dict(coords=mesh.coords, velocity=nd["velocity"], dpdx=nd["dpdx"],
                                     density=nd["density"], pressure=nd["pressure"], udiag=nd["udiag"],
                                     area=mesh.area).items()}
    ls = _handle(nw, mesh)
    out = torch.zeros(mesh.num_edges, dtype=torch.float64, device="cuda")
    f = nw.ContinuityFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dpdx", "density", "pressure",
                                                        "udiag", "area")))
    ls.compute_mdot(f, out, noc_fac=1.0, interp_together=interp)
    ref = orc.mdot_edge(mesh.edges, mesh.coords, nd["velocity"], nd["dpdx"], nd["density"], nd["pressure"],
                        nd["udiag"], mesh.area, noc=1.0, interp=interp)
    # running magnitude
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    A = np.abs(mesh.area)
    mdx = np.abs(mesh.coords[R]) + np.abs(mesh.coords[L])
    axdx = np.abs(np.einsum("ed,ed->e", mesh.area, mesh.coords[R] - mesh.coords[L]))
    masq = (A * A).sum(1)
    mw = masq / axdx * (1 + (A * mdx).sum(1) / axdx)
    iu = 1 / np.abs(nd["udiag"])
    mpts = 0.5 * (iu[L] + iu[R])
    rho, u, g = np.abs(nd["density"]), np.abs(nd["velocity"]), np.abs(nd["dpdx"])
    S = mpts * (np.abs(nd["pressure"][R]) + np.abs(nd["pressure"][L])) * mw
    mG = 0.5 * (g[R] * iu[R, None] + g[L] * iu[L, None])
    mrU = 0.5 * (rho[R, None] * u[R] + rho[L, None] * u[L])
    mU = 0.5 * 0.5 * (rho[R] + rho[L])[:, None] * (u[R] + u[L])
    S += ((abs(interp) * mrU + abs(1 - interp) * mU + mG) * A).sum(1) + ((A + mw[:, None] * mdx) * mG).sum(1)
    check_close(out.cpu().numpy(), ref, S, "mdot")


@pytest.mark.parametrize("periodic", [False, True])
def test_nodal_gradient_matches_oracle(nw, orc, periodic):
    import torch
    if periodic:
        mesh = nw.Mesh(14, 12, 10, periodic_x=True, periodic_y=True, jitter=0.05, seed=8)
    else:
        mesh = nw.Mesh(20, 16, 12, stretch_z=1.1, jitter=0.08, seed=6)
    rng = np.random.default_rng(5)
    N = mesh.num_nodes
    master = mesh.nalu_id - 1
    for dim1 in (1, 3):
        phi = rng.normal(0.0, 1.0, (N, dim1))
        phi = phi[master]  # slaves carry their master's value
        ls = _handle(nw, mesh)
        grad = torch.zeros((N, 3 * dim1), dtype=torch.float64, device="cuda")
        ls.nodal_gradient(dev(phi), dev(mesh.area), dev(mesh.dualvol), grad, bnd_area_dev=dev(mesh.bnd_area),
                          dim1=dim1)
        # oracle: per-node edge sums (each divided by the node's volume), the
        # boundary closure, then the periodic sum
        inner = orc.nodal_grad_edge(mesh.edges, phi, mesh.area, mesh.dualvol, dim1=dim1)
        bnd = (mesh.bnd_area[:, None, :] * phi[:, :, None]).reshape(N, 3 * dim1) / mesh.dualvol[:, None]
        ref = nw.workload.periodic_sum(mesh, inner + bnd)
        L, R = mesh.edges[:, 0], mesh.edges[:, 1]
        pip = 0.5 * (np.abs(phi[L]) + np.abs(phi[R]))
        contrib = (np.abs(mesh.area)[:, None, :] * pip[:, :, None]).reshape(-1, 3 * dim1)
        S = np.zeros((N, 3 * dim1))
        for k in range(3 * dim1):
            S[:, k] = np.bincount(L, contrib[:, k], N) + np.bincount(R, contrib[:, k], N)
        S += (np.abs(mesh.bnd_area)[:, None, :] * np.abs(phi)[:, :, None]).reshape(N, 3 * dim1)
        S = nw.workload.periodic_sum(mesh, S) / mesh.dualvol[:, None]
        check_close(grad.cpu().numpy().ravel(), ref.ravel(), S.ravel(), f"grad dim1={dim1}")


@pytest.mark.parametrize("tanh_form", [0, 1])
def test_peclet_factor_matches_oracle(nw, orc, tanh_form):
    import torch
    case = nw.workload.lowmach_case(20, 16, 12, seed=2)
    mesh = case.mesh
    nd = case.node
    rng = np.random.default_rng(6)
    rho = rng.uniform(0.8, 1.2, mesh.num_nodes)
    ls = _handle(nw, mesh)
    E = mesh.num_edges
    pecnum = torch.zeros(E, dtype=torch.float64, device="cuda")
    pecfac = torch.zeros(E, dtype=torch.float64, device="cuda")
    o = nw.PecletOpts(tanh_form, 1.0, 2.0, 4.0, 1e-16)
    ls.peclet_factor(dev(mesh.coords), dev(rho), dev(nd["viscosity"]), dev(nd["velocity"]), pecfac, opts=o,
                     pecnum_dev=pecnum)
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    mu, u, x = nd["viscosity"], nd["velocity"], mesh.coords
    diff = 0.5 * (mu[L] / rho[L] + mu[R] / rho[R])
    udotx = np.einsum("ed,ed->e", 0.5 * (x[R] - x[L]), u[R] + u[L])
    pe = np.abs(udotx) / (diff + 1e-16)
    if tanh_form:
        f = np.array([orc.peclet_tanh(v, 2.0, 4.0) for v in pe])
        fp = 0.5 / 4.0 * (1 - np.tanh((pe - 2.0) / 4.0) ** 2)
    else:
        f = np.array([orc.peclet_classic(v, 1.0) for v in pe])
        fp = 10 * pe / (5 + pe * pe) ** 2
    Spe = (0.5 * (np.abs(x[R]) + np.abs(x[L])) * (np.abs(u[R]) + np.abs(u[L]))).sum(1) / (diff + 1e-16) + pe
    check_close(pecnum.cpu().numpy(), pe, Spe, "peclet number")
    check_close(pecfac.cpu().numpy(), f, fp * Spe + np.abs(f) + 1e-3, "peclet factor")


def test_nodal_gradient_golds_on_the_gpu(nw, orc, golds):
    """The reference's interior edge-gradient golds (unit cube, linear
    fields) through the C ABI, without the boundary closure."""
    import torch
    g = golds["nodal_grad_edge_hex8"]
    mesh = nw.Mesh(1, 1, 1)  # node ids as in the reference fixture (x fastest)
    x, y, z = mesh.coords.T
    cx, cy, cz = g["coeff"]
    ls = _handle(nw, mesh)
    grad = torch.zeros((8, 3), dtype=torch.float64, device="cuda")
    ls.nodal_gradient(dev((cx * x + cy * y + cz * z)[:, None]), dev(mesh.area), dev(mesh.dualvol), grad, dim1=1)
    np.testing.assert_allclose(grad.cpu().numpy().ravel(), g["scalar"], rtol=0, atol=1e-14)
    gu = torch.zeros((8, 9), dtype=torch.float64, device="cuda")
    ls.nodal_gradient(dev(np.stack([cx * x, cy * y, cz * z], 1)), dev(mesh.area), dev(mesh.dualvol), gu, dim1=3)
    d = gu.cpu().numpy().reshape(8, 3, 3)
    np.testing.assert_allclose(np.stack([d[:, i, i] for i in range(3)], 1).ravel(), g["vector_diagonal"], rtol=0,
                               atol=1e-14)


def test_nodal_gradient_boundary_closure_gold_on_the_gpu(nw, golds):
    """Interior edges plus the shifted closure of the z- side (bnd_area from
    that side's face IPs): on the side's nodes the z component is the
    interior gold plus the reference's shifted boundary gold."""
    import torch
    gi = golds["nodal_grad_edge_hex8"]["scalar"]
    gb = golds["nodal_grad_bndry_hex8_zminus"]["shifted"]
    mesh = nw.Mesh(1, 1, 1)
    ipn, area = mesh.face_ips(("z-",))
    bnd = np.zeros((8, 3))
    np.add.at(bnd, ipn[:, 0], area)
    x, y, z = mesh.coords.T
    ls = _handle(nw, mesh)
    grad = torch.zeros((8, 3), dtype=torch.float64, device="cuda")
    ls.nodal_gradient(dev((2 * x + 2 * y + 2 * z)[:, None]), dev(mesh.area), dev(mesh.dualvol), grad,
                      bnd_area_dev=dev(bnd), dim1=1)
    gz = grad.cpu().numpy()[:4, 2]
    np.testing.assert_allclose(gz, np.array(gi).reshape(8, 3)[:4, 2] + np.array(gb), rtol=0, atol=1e-14)
