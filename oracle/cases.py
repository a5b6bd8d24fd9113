"""Seeded benchmark workloads rebuilt from the oracle alone.

TEST INFRASTRUCTURE ONLY: the CPU reference arm of the benchmark and the
tests build their inputs here, so that timing the restated reference path
never loads the product library. The definitions are those of the
benchmark workloads (stretched, jittered hex box; log-law velocity with
Gaussian noise; log-uniform effective viscosity; Green-Gauss gradients;
the unit-test mass flow rate 0.5 (rhoL uL + rhoR uR) . A of
unit_tests/kernels/UnitTestKernelUtils.C:725-769; the momentum Peclet factor
of src/edge_kernels/MomentumEdgePecletAlg.C:74-101 with the classic Peclet
function, hybrid factor 1). Mesh, edges and geometry come from the oracle's
STK / Hex8 restatements (oracle.h); node fields draw the same numpy
generator sequence as the product's workload module, so both see the same
inputs (edge order may differ; tests compare them edge by edge).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import oracle as orc

# local node ordinals of the six box sides x-, x+, y-, y+, z-, z+ (Exodus side
# ordering of HexSCS::sideNodeOrdinals_, include/master_element/Hex8CVFEM.h:
# 395-401)
HEX_BOX_SIDE = ((0, 4, 7, 3), (1, 2, 6, 5), (0, 1, 5, 4), (2, 3, 7, 6), (0, 3, 2, 1), (4, 5, 6, 7))


@dataclass
class OracleMesh:
    nx: int
    ny: int
    nz: int
    coords: np.ndarray
    conn: np.ndarray
    edges: np.ndarray
    area: np.ndarray
    dualvol: np.ndarray
    bnd_area: np.ndarray

    @property
    def num_nodes(self) -> int:
        return self.coords.shape[0]

    @property
    def num_edges(self) -> int:
        return self.edges.shape[0]

    @property
    def nalu_id(self) -> np.ndarray:
        return np.arange(1, self.num_nodes + 1, dtype=np.int64)


@dataclass
class OracleCase:
    mesh: OracleMesh
    node: dict = field(default_factory=dict)
    edge: dict = field(default_factory=dict)
    opts: dict = field(default_factory=dict)


def boundary_faces(nx: int, ny: int, nz: int, conn: np.ndarray, coords: np.ndarray) -> np.ndarray:
    """Exposed quad faces of the box (nf, 4), outward, in side order, then
    element order along the side."""
    out = []
    for sd in range(6):
        d, up = sd // 2, sd % 2
        n = (nx, ny, nz)
        layer = n[d] - 1 if up else 0
        o1, o2 = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))
        for b in range(n[o2]):
            for a in range(n[o1]):
                ijk = [0, 0, 0]
                ijk[d], ijk[o1], ijk[o2] = layer, a, b
                h = ijk[0] + nx * (ijk[1] + ny * ijk[2])
                fn = conn[h, list(HEX_BOX_SIDE[sd])]
                p = coords[fn]
                c = p.mean(0)
                nrm = np.cross(p - c, np.roll(p, -1, 0) - c).sum(0)
                if nrm @ (c - coords[conn[h]].mean(0)) < 0:
                    fn = np.concatenate([fn[:1], fn[1:][::-1]])
                out.append(fn)
    return np.array(out, np.int64)


def box_mesh(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, stretch=1.0, jitter=0.0, seed=0) -> OracleMesh:
    coords = orc.box_coords(nx, ny, nz, lx, ly, lz, stretch, jitter, seed)
    _, conn = orc.hex_box(nx, ny, nz)
    edges, ee = orc.hex8_edges(conn, coords.shape[0])
    area, vol = orc.hex8_geometry(coords, conn, ee, edges)
    faces = boundary_faces(nx, ny, nz, conn, coords)
    fa = orc.face_scs_areas(faces, coords)
    bnd = np.zeros_like(coords)
    for d in range(3):
        bnd[:, d] = np.bincount(faces.ravel(), fa[:, d], coords.shape[0])
    return OracleMesh(nx, ny, nz, coords, conn, edges, area, vol, bnd)


def green_gauss(mesh: OracleMesh, phi: np.ndarray) -> np.ndarray:
    """Nodal gradient (N, 3 k): the NodalGradEdgeAlg edge terms plus the
    lumped boundary closure (shifted face IPs), over the dual volume."""
    p = phi if phi.ndim == 2 else phi[:, None]
    k = p.shape[1]
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    pip = 0.5 * (p[L] + p[R])
    out = np.empty((mesh.num_nodes, 3 * k))
    for i in range(k):
        for j in range(3):
            v = mesh.area[:, j] * pip[:, i]
            g = np.bincount(L, v, mesh.num_nodes) - np.bincount(R, v, mesh.num_nodes)
            out[:, 3 * i + j] = g + mesh.bnd_area[:, j] * p[:, i]
    return out / mesh.dualvol[:, None]


def lowmach_case(nx=128, ny=128, nz=64, seed=2, stretch=1.08, jitter=0.05, lz=0.5) -> OracleCase:
    """Momentum + continuity inputs on the stretched, jittered box (the
    momentum / continuity assembly workload): u = log-law
    ln(1 + z/z0) / ln(1 + Lz/z0) in x (z0 = 1e-3) plus N(0, 0.05^2) noise on
    every component, mu_eff log-uniform in [1e-5, 1e-2], rho = 1,
    momentum_diag = 1, p ~ N(0, 0.01^2), abl mask = 1."""
    mesh = box_mesh(nx, ny, nz, 1.0, 1.0, lz, stretch, jitter, seed)
    rng = np.random.default_rng(seed)
    N = mesh.num_nodes
    z = mesh.coords[:, 2]
    vel = rng.normal(0.0, 0.05, (N, 3))
    vel[:, 0] += np.log1p(np.maximum(z, 0.0) / 1e-3) / np.log1p(lz / 1e-3)
    visc = np.exp(rng.uniform(np.log(1e-5), np.log(1e-2), N))
    rho = np.ones(N)
    p = rng.normal(0.0, 0.01, N)
    L, R = mesh.edges[:, 0], mesh.edges[:, 1]
    mdot = np.einsum("ed,ed->e", 0.5 * (rho[L, None] * vel[L] + rho[R, None] * vel[R]), mesh.area)
    diff = 0.5 * (visc[L] / rho[L] + visc[R] / rho[R])
    dx = mesh.coords[R] - mesh.coords[L]
    pe = np.abs(np.einsum("ed,ed->e", 0.5 * dx, vel[R] + vel[L])) / (diff + 1e-16)
    pec = pe * pe / (5.0 + pe * pe)
    mo = orc.MomentumOpts(alpha=0.0, alpha_upw=1.0, upw_factor=1.0, relax=1.0, include_div_u=0.0, use_limiter=0)
    co = orc.ContinuityOpts(noc_fac=1.0, tau_scale=1.0, interp_together=1.0, solve_incompressible=0.0)
    return OracleCase(mesh, node=dict(coords=mesh.coords, velocity=vel, dudx=green_gauss(mesh, vel),
                                      viscosity=visc, density=rho, mask=np.ones(N), pressure=p,
                                      dpdx=green_gauss(mesh, p), udiag=np.ones(N)),
                      edge=dict(area=mesh.area, mdot=mdot, pecfac=pec), opts=dict(momentum=mo, continuity=co))
