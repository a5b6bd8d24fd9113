"""Seeded synthetic inputs for the edge-assembly + Krylov benchmarks.

Meshes come from the library (nw_mesh_box); node and edge fields are built
here with numpy from fixed seeds, so every consumer (GPU path, CPU oracle,
benchmark) sees identical inputs. Field definitions:

scalar (32^3 unit cube, periodic in x and y, Dirichlet 0 / 1 on z = 0 / 1):
    u = sin(2 pi x + p1) cos(2 pi y + p2) cos(pi z)
    v = -cos(2 pi x + p1) sin(2 pi y + p2) cos(pi z),  w = 0
    (Taylor-Green, amplitude 1, phases p1, p2 ~ U[0, 2 pi) from the seed),
    rho = 1, diffFluxCoeff = 1e-3, q ~ U[0, 1] per master node.
lowmach (128 x 128 x 64 box [0,1] x [0,1] x [0,0.5], z stretched 1.08,
    interior jitter 5%): u = log-law ln(1 + z/z0)/ln(1 + Lz/z0) in x
    (z0 = 1e-3) plus N(0, 0.05^2) noise on every component; mu_eff
    log-uniform in [1e-5, 1e-2]; rho = 1; momentum_diag = 1;
    p ~ N(0, 0.01^2); abl mask = 1.
poisson (256 x 256 x 128 unit box, z stretched 1.04): continuity operator
    with u = 0, grad p = 0, rho = 1, momentum_diag = 1 (a Laplacian);
    rhs ~ N(0, 1) projected to zero mean.
Gradients are Green-Gauss: the NodalGradEdgeAlg edge terms
(src/ngp_algorithms/NodalGradEdgeAlg.C:85-109) plus lumped boundary-face
closure, summed over periodic pairs. mdot is the unit-test formula
0.5 (rhoL uL + rhoR uR) . A (unit_tests/kernels/UnitTestKernelUtils.C:
725-769); the momentum peclet_factor is MomentumEdgePecletAlg
(src/edge_kernels/MomentumEdgePecletAlg.C:74-101) with the classic Peclet
function and hybrid factor 1.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import Mesh, ScalarOpts, MomentumOpts, ContinuityOpts


def _edge_scatter(N: int, L: np.ndarray, R: np.ndarray, vals: np.ndarray) -> np.ndarray:
    """out[L] += vals, out[R] -= vals (vals: (E,) or (E, k))."""
    if vals.ndim == 1:
        return np.bincount(L, vals, N) - np.bincount(R, vals, N)
    out = np.empty((N, vals.shape[1]))
    for k in range(vals.shape[1]):
        out[:, k] = np.bincount(L, vals[:, k], N) - np.bincount(R, vals[:, k], N)
    return out


def periodic_sum(mesh: Mesh, a: np.ndarray) -> np.ndarray:
    """Masters and their slaves hold the summed value (parallel_sum over
    periodic pairs)."""
    master = mesh.nalu_id - 1
    slaves = np.nonzero(master != np.arange(mesh.num_nodes))[0]
    if slaves.size == 0:
        return a
    a = a.copy()
    np.add.at(a, master[slaves], a[slaves])
    a[slaves] = a[master[slaves]]
    return a


def sync_slaves(mesh: Mesh, a: np.ndarray) -> np.ndarray:
    master = mesh.nalu_id - 1
    return a[master]


def green_gauss(mesh: Mesh, phi: np.ndarray) -> np.ndarray:
    """Nodal gradient (N, k*3) of phi (N,) or (N, k), row-major per node as
    STK stores dudx (component i, direction j at i*3 + j)."""
    p = phi if phi.ndim == 2 else phi[:, None]
    k = p.shape[1]
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    pip = 0.5 * (p[L] + p[R])
    out = np.empty((mesh.num_nodes, k * 3))
    for i in range(k):
        for j in range(3):
            g = _edge_scatter(mesh.num_nodes, L, R, mesh.area[:, j] * pip[:, i])
            g = g + mesh.bnd_area[:, j] * p[:, i]
            out[:, 3 * i + j] = g
    out = periodic_sum(mesh, out)
    return out / mesh.dualvol[:, None]


def mdot_unit_test(mesh: Mesh, rho: np.ndarray, vel: np.ndarray) -> np.ndarray:
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    return np.einsum("ed,ed->e", 0.5 * (rho[L, None] * vel[L] + rho[R, None] * vel[R]), mesh.area)


def peclet_factor(mesh: Mesh, rho, visc, vel, hybrid=1.0, eps=1e-16) -> np.ndarray:
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    diff = 0.5 * (visc[L] / rho[L] + visc[R] / rho[R])
    dx = mesh.coords[R] - mesh.coords[L]
    udotx = np.einsum("ed,ed->e", 0.5 * dx, vel[R] + vel[L])
    pe = np.abs(udotx) / (diff + eps)
    m = hybrid * pe
    return m * m / (5.0 + m * m)


@dataclass
class Case:
    mesh: Mesh
    node: dict = field(default_factory=dict)
    edge: dict = field(default_factory=dict)
    opts: dict = field(default_factory=dict)
    extra: dict = field(default_factory=dict)


def scalar_case(n: int = 32, seed: int = 1) -> Case:
    """Scalar advection-diffusion on an n^3 periodic unit cube."""
    mesh = Mesh(n, n, n, periodic_x=True, periodic_y=True)
    rng = np.random.default_rng(seed)
    p1, p2 = rng.uniform(0, 2 * np.pi, 2)
    x, y, z = mesh.coords.T
    vel = np.zeros((mesh.num_nodes, 3))
    vel[:, 0] = np.sin(2 * np.pi * x + p1) * np.cos(2 * np.pi * y + p2) * np.cos(np.pi * z)
    vel[:, 1] = -np.cos(2 * np.pi * x + p1) * np.sin(2 * np.pi * y + p2) * np.cos(np.pi * z)
    vel = sync_slaves(mesh, vel)
    q = sync_slaves(mesh, rng.uniform(0.0, 1.0, mesh.num_nodes))
    rho = np.ones(mesh.num_nodes)
    gam = np.full(mesh.num_nodes, 1e-3)
    dqdx = green_gauss(mesh, q)
    mdot = mdot_unit_test(mesh, rho, vel)
    zmax = mesh.coords[:, 2].max()
    bottom = np.nonzero(np.abs(mesh.coords[:, 2]) < 1e-12)[0]
    top = np.nonzero(np.abs(mesh.coords[:, 2] - zmax) < 1e-12)[0]
    bc = np.zeros(mesh.num_nodes)
    bc[top] = 1.0
    opts = ScalarOpts(alpha=0.0, alpha_upw=0.5, upw_factor=1.0, relax=1.0, hybrid_factor=1.0,
                      use_limiter=0, tanh_form=0, tanh_trans=2.0, tanh_width=4.0)
    return Case(mesh, node=dict(coords=mesh.coords, velocity=vel, q=q, dqdx=dqdx, density=rho,
                                diff_coeff=gam, bc=bc),
                edge=dict(area=mesh.area, mdot=mdot), opts=dict(scalar=opts),
                extra=dict(dirichlet_nodes=np.concatenate([bottom, top]).astype(np.int64)))


def lowmach_case(nx=128, ny=128, nz=64, seed=2, stretch=1.08, jitter=0.05, lz=0.5, tets=False,
                 renumber=0, renumber_seed=0) -> Case:
    """Momentum + continuity inputs on a stretched, jittered box (hex, or
    each hex split into 6 tets; renumber 1 = random node order, 2 = random
    then reverse Cuthill-McKee)."""
    mesh = Mesh(nx, ny, nz, lx=1.0, ly=1.0, lz=lz, stretch_z=stretch, jitter=jitter, seed=seed, tets=tets,
                renumber=renumber, renumber_seed=renumber_seed)
    rng = np.random.default_rng(seed)
    N = mesh.num_nodes
    z = mesh.coords[:, 2]
    z0 = 1e-3
    vel = rng.normal(0.0, 0.05, (N, 3))
    vel[:, 0] += np.log1p(np.maximum(z, 0.0) / z0) / np.log1p(lz / z0)
    visc = np.exp(rng.uniform(np.log(1e-5), np.log(1e-2), N))
    rho = np.ones(N)
    udiag = np.ones(N)
    p = rng.normal(0.0, 0.01, N)
    mask = np.ones(N)
    dudx = green_gauss(mesh, vel)
    dpdx = green_gauss(mesh, p)
    mdot = mdot_unit_test(mesh, rho, vel)
    pec = peclet_factor(mesh, rho, visc, vel)
    mo = MomentumOpts(alpha=0.0, alpha_upw=1.0, upw_factor=1.0, relax=1.0, include_div_u=0.0,
                      use_limiter=0)
    co = ContinuityOpts(noc_fac=1.0, tau_scale=1.0, interp_together=1.0, solve_incompressible=0.0)
    return Case(mesh, node=dict(coords=mesh.coords, velocity=vel, dudx=dudx, viscosity=visc, density=rho,
                                mask=mask, pressure=p, dpdx=dpdx, udiag=udiag),
                edge=dict(area=mesh.area, mdot=mdot, pecfac=pec), opts=dict(momentum=mo, continuity=co))


def poisson_case(nx=256, ny=256, nz=128, seed=3, stretch=1.04, jitter=0.0, tets=False) -> Case:
    """Pressure-Poisson operator (continuity with zero velocity)."""
    mesh = Mesh(nx, ny, nz, stretch_z=stretch, jitter=jitter, seed=seed, tets=tets)
    rng = np.random.default_rng(seed)
    N = mesh.num_nodes
    zeros3 = np.zeros((N, 3))
    co = ContinuityOpts(noc_fac=1.0, tau_scale=1.0, interp_together=1.0, solve_incompressible=0.0)
    b = rng.normal(0.0, 1.0, N)
    b -= b.mean()
    return Case(mesh, node=dict(coords=mesh.coords, velocity=zeros3, dpdx=zeros3, density=np.ones(N),
                                pressure=np.zeros(N), udiag=np.ones(N)),
                edge=dict(area=mesh.area), opts=dict(continuity=co), extra=dict(rhs=b))


def poisson_system(shape, seed=3, stretch=1.04, jitter=0.0, rhs_seed=None, stream=None, tets=False):
    """Assembled pressure-Poisson LinearSystem of a box (device inputs via
    torch); the right-hand side is the case's seeded zero-mean Gaussian,
    or a fresh one from rhs_seed."""
    import torch

    from . import ContinuityFields, LinearSystem
    case = poisson_case(*shape, seed=seed, stretch=stretch, jitter=jitter, tets=tets)
    mesh = case.mesh
    nd = case.node
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in dict(
        coords=mesh.coords, velocity=nd["velocity"], dpdx=nd["dpdx"], density=nd["density"],
        pressure=nd["pressure"], udiag=nd["udiag"], area=mesh.area).items()}
    ls = LinearSystem(1, stream=stream)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges)
    ls.finalize()
    ls.zero_system()
    ls.assemble_continuity(ContinuityFields(*(d[k].data_ptr() for k in (
        "coords", "velocity", "dpdx", "density", "pressure", "udiag", "area"))), case.opts["continuity"])
    rhs = case.extra["rhs"]
    if rhs_seed is not None:
        rhs = np.random.default_rng(rhs_seed).normal(0.0, 1.0, rhs.shape)
        rhs -= rhs.mean()
    ls.from_host(rhs=rhs)
    ls.sync()
    return ls
