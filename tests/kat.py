"""Known-answer fixtures of the reference unit tests, rebuilt as arrays.

Each builder restates a nalu-wind test fixture on the single-hex
"generated:1x1x1" mesh (unit cube, node ids 1..8):
  scalar:     MixtureFractionKernelHex8Mesh (unit_tests/kernels/
              UnitTestKernelUtils.h:1357-1456) as used by
              unit_tests/edge_kernels/UnitTestScalarAdvDiffEdge.C:159-205
  continuity: ContinuityEdgeHex8Mesh (UnitTestKernelUtils.h:376-482) as used
              by unit_tests/edge_kernels/UnitTestContinuityAdvEdge.C:110-140
  momentum:   MomentumEdgeHex8Mesh (UnitTestKernelUtils.h:484-590) as used
              by unit_tests/edge_kernels/UnitTestMomentumAdvDiffEdge.C
The fixtures fill the edge "mass_flow_rate" field, declared with three
components per edge, through a scalar pointer (calc_mass_flow_rate,
unit_tests/kernels/UnitTestKernelUtils.C:725-769), so edge k reads the
value computed for edge 3k (zero for 3k >= 12). The golds depend on that,
and `mdot_fixture` reproduces it.
"""
from __future__ import annotations

import numpy as np

A_TRIG = 0.3  # TrigFieldFunction::a


def hex1(orc):
    coords, conn = orc.hex_box(1, 1, 1)
    edges, ee = orc.hex8_edges(conn, 8)
    area, vol = orc.hex8_geometry(coords, conn, ee, edges)
    return dict(coords=coords, conn=conn, edges=edges, elem_edges=ee, area=area, dualvol=vol)


def trig_velocity(coords):
    x, y = coords[:, 0], coords[:, 1]
    v = np.zeros((coords.shape[0], 3))
    v[:, 0] = -np.cos(A_TRIG * np.pi * x) * np.sin(A_TRIG * np.pi * y)
    v[:, 1] = np.sin(A_TRIG * np.pi * x) * np.cos(A_TRIG * np.pi * y)
    return v


def trig_dudx(coords):
    x, y = coords[:, 0], coords[:, 1]
    ap = A_TRIG * np.pi
    g = np.zeros((coords.shape[0], 9))
    g[:, 0] = ap * np.sin(ap * x) * np.sin(ap * y)
    g[:, 1] = -ap * np.cos(ap * x) * np.cos(ap * y)
    g[:, 3] = ap * np.cos(ap * x) * np.cos(ap * y)
    g[:, 4] = -ap * np.sin(ap * x) * np.sin(ap * y)
    return g


def mdot_fixture(orc, m, vel, rho):
    true = orc.mdot_unit_test(m["edges"], vel, rho, m["area"])
    E = true.shape[0]
    return np.array([true[3 * k] if 3 * k < E else 0.0 for k in range(E)])


def scalar_fixture(orc):
    m = hex1(orc)
    x, y, z = m["coords"].T
    zf = 2.0 * np.cos(np.pi * x) * np.cos(np.pi * y) * np.cos(np.pi * z)
    rho = 1.0 / (zf / 0.163 + (1.0 - zf) / 1.18)
    mu = 1.967e-5 * zf + 1.85e-5 * (1.0 - zf)
    vel = trig_velocity(m["coords"])
    m.update(q=zf, density=rho, diff=mu, velocity=vel, dqdx=np.zeros((8, 3)),
             mdot=mdot_fixture(orc, m, vel, rho),
             opts=dict(alpha=0.0, alpha_upw=0.0, upw_factor=0.0, relax=1.0, hybrid_factor=0.0,
                       use_limiter=0, tanh_form=0, tanh_trans=2.0, tanh_width=4.0))
    return m


def continuity_fixture(orc):
    m = hex1(orc)
    x, y = m["coords"][:, 0], m["coords"][:, 1]
    a = A_TRIG
    p = -0.25 * (np.cos(2 * a * np.pi * x) + np.cos(2 * a * np.pi * y))
    dpdx = np.zeros((8, 3))
    dpdx[:, 0] = 0.5 * a * np.pi * np.sin(2 * a * np.pi * x)
    dpdx[:, 1] = 0.5 * a * np.pi * np.sin(2 * a * np.pi * y)
    m.update(velocity=trig_velocity(m["coords"]), pressure=p, dpdx=dpdx, density=np.ones(8),
             udiag=np.ones(8), opts=dict(noc_fac=1.0, tau_scale=1.0, interp_together=1.0,
                                         solve_incompressible=0.0))
    return m


def momentum_fixture(orc):
    m = hex1(orc)
    vel = trig_velocity(m["coords"])
    rho = np.ones(8)
    m.update(velocity=vel, dudx=trig_dudx(m["coords"]), viscosity=np.full(8, 0.1), density=rho,
             mask=np.ones(8), mdot=mdot_fixture(orc, m, vel, rho), pecfac=np.zeros(12),
             opts=dict(alpha=0.0, alpha_upw=0.0, upw_factor=0.0, relax=1.0, include_div_u=0.0,
                       use_limiter=0))
    return m


def dense_accumulate(edges, lhs, rhs, num_dof, n_nodes, same_dof_only=False):
    """TestEdgeLinearSystem's dense fake backend (unit_tests/UnitTestLinearSystem.h:42-72);
    with same_dof_only it adds lhs(ioff+d, joff+d) couplings only."""
    nd = num_dof
    Ld = np.zeros((n_nodes * nd, n_nodes * nd))
    B = np.zeros(n_nodes * nd)
    nl = 2 * nd
    for e, (i, j) in enumerate(edges):
        ns = (i, j)
        for a in range(2):
            for d in range(nd):
                B[ns[a] * nd + d] += rhs[e, a * nd + d]
        for a in range(2):
            for b in range(2):
                for d in range(nd):
                    if same_dof_only:
                        Ld[ns[a] * nd + d, ns[b] * nd + d] += lhs[e, (a * nd + d) * nl + b * nd + d]
                    else:
                        for c in range(nd):
                            Ld[ns[a] * nd + d, ns[b] * nd + c] += lhs[e, (a * nd + d) * nl + b * nd + c]
    return Ld, B


# The x+ side ("surface_2") of the unit cube: Exodus side 1 of the hex,
# element nodes (1, 2, 6, 5) = node ids (1, 3, 7, 5) (0-based), opposed
# across the element by (0, 3, 7, 4) = ids (0, 2, 6, 4). Each face IP's
# sub-face is a quarter of the unit square, normal +x.
XPLUS_IPN = np.array([[1, 0], [3, 2], [7, 6], [5, 4]], np.int64)
XPLUS_AREA = np.tile([0.25, 0.0, 0.0], (4, 1))


def quad_scv_weights():
    """Bilinear shape functions of a quad at its four sub-control-volume
    centroids (AlgTraitsQuad4 SCV quadrature, unshifted): 9/16 for the IP's
    own node, 3/16 for its two face neighbours, 1/16 for the opposite node."""
    w = np.zeros((4, 4))
    for ip in range(4):
        w[ip, ip] = 9 / 16
        w[ip, (ip + 1) % 4] = 3 / 16
        w[ip, (ip + 3) % 4] = 3 / 16
        w[ip, (ip + 2) % 4] = 1 / 16
    return w


def open_mdot(ipn, area, vel, rho):
    """calc_open_mass_flow_rate (unit_tests/kernels/UnitTestKernelUtils.C:
    856-940) on one quad face: rho u interpolated to each IP, dotted with its
    exposed area vector."""
    fn = ipn[:, 0]
    rhoU = quad_scv_weights() @ (rho[fn, None] * vel[fn])
    return np.einsum("id,id->i", rhoU, area)


def continuity_open_fixture(orc):
    """ContinuityKernelHex8Mesh (UnitTestKernelUtils.h:442-468) as used by
    UnitTestContinuityOpenEdge.C:104-147: pressure_bc = dynamic_pressure = 0,
    tauScale = dt / gamma1 = 1, open mdot correction off (pstabFac = 1)."""
    m = continuity_fixture(orc)
    m.update(ipn=XPLUS_IPN, areav=XPLUS_AREA, pressure_bc=np.zeros(8), dynp=np.zeros(4),
             open_opts=dict(tau_scale=1.0, noc_fac=1.0, pstab_fac=1.0, mdot_corr=0.0,
                            solve_incompressible=0.0))
    return m


def momentum_face_fixture(orc):
    """MomentumKernelHex8Mesh (UnitTestKernelUtils.h:484-545) on the x+
    side: open_velocity_bc left zero, open mass flow from the face
    interpolation of rho u, includeDivU = nearestFaceEntrain = 0."""
    m = momentum_fixture(orc)
    m.update(ipn=XPLUS_IPN, areav=XPLUS_AREA, velocity_bc=np.zeros((8, 3)),
             open_mdot=open_mdot(XPLUS_IPN, XPLUS_AREA, m["velocity"], m["density"]))
    return m
