"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the
benchmark's CPU-baseline / reference arm. It is the checker, never the thing
measured as the product. See oracle.h for the reference file:line each
routine restates.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

I64 = C.POINTER(C.c_int64)
I32 = C.POINTER(C.c_int32)
DP = C.POINTER(C.c_double)


class ScalarOpts(C.Structure):
    _fields_ = [("alpha", C.c_double), ("alpha_upw", C.c_double), ("upw_factor", C.c_double),
                ("relax", C.c_double), ("hybrid_factor", C.c_double), ("use_limiter", C.c_int),
                ("tanh_form", C.c_int), ("tanh_trans", C.c_double), ("tanh_width", C.c_double)]


class MomentumOpts(C.Structure):
    _fields_ = [("alpha", C.c_double), ("alpha_upw", C.c_double), ("upw_factor", C.c_double),
                ("relax", C.c_double), ("include_div_u", C.c_double), ("use_limiter", C.c_int)]


class ContinuityOpts(C.Structure):
    _fields_ = [("noc_fac", C.c_double), ("tau_scale", C.c_double),
                ("interp_together", C.c_double), ("solve_incompressible", C.c_double)]


class ContinuityOpenOpts(C.Structure):
    _fields_ = [("tau_scale", C.c_double), ("noc_fac", C.c_double), ("pstab_fac", C.c_double),
                ("mdot_corr", C.c_double), ("solve_incompressible", C.c_double)]


class MomentumOpenOpts(C.Structure):
    _fields_ = [("include_div_u", C.c_double), ("nf_entrain", C.c_double), ("entrainment", C.c_int)]


class MomentumSymmetryOpts(C.Structure):
    _fields_ = [("include_div_u", C.c_double), ("penalty_factor", C.c_double)]


class AblWallOpts(C.Structure):
    _fields_ = [("gravity", C.c_double), ("z0", C.c_double), ("Tref", C.c_double), ("kappa", C.c_double),
                ("beta_m", C.c_double), ("gamma_m", C.c_double)]


class SolveReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("final_rel_implicit", C.c_double),
                ("final_abs_explicit", C.c_double), ("rhs_norm", C.c_double)]


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} is not built; run oracle/build.py")
        _lib = C.CDLL(str(LIB))
        _lib.or_hex_box_num_nodes.restype = C.c_int64
        _lib.or_hex_box_num_elems.restype = C.c_int64
        _lib.or_hex8_edges.restype = C.c_int64
        _lib.or_build_graph.restype = C.c_int64
        _lib.or_peclet_classic.restype = C.c_double
        _lib.or_peclet_classic.argtypes = [C.c_double, C.c_double]
        _lib.or_peclet_tanh.restype = C.c_double
        _lib.or_peclet_tanh.argtypes = [C.c_double, C.c_double, C.c_double]
        _lib.or_solve.restype = C.c_int
    return _lib


def hex_box(nx, ny, nz):
    L = lib()
    N = L.or_hex_box_num_nodes(nx, ny, nz)
    M = L.or_hex_box_num_elems(nx, ny, nz)
    coords = np.zeros((N, 3))
    conn = np.zeros((M, 8), np.int64)
    L.or_hex_box(nx, ny, nz, _p(coords, C.c_double), _p(conn, C.c_int64))
    return coords, conn


def box_coords(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, stretch=1.0, jitter=0.0, seed=0):
    """Seeded stretched / jittered box coordinates (or_box_coords)."""
    L = lib()
    N = L.or_hex_box_num_nodes(nx, ny, nz)
    coords = np.zeros((N, 3))
    L.or_box_coords(nx, ny, nz, C.c_double(lx), C.c_double(ly), C.c_double(lz), C.c_double(stretch),
                    C.c_double(jitter), C.c_uint64(seed), _p(coords, C.c_double))
    return coords


def hex8_edges(conn, nnodes):
    L = lib()
    conn = _i64(conn)
    M = conn.shape[0]
    cap = 12 * M
    edges = np.zeros((cap, 2), np.int64)
    ee = np.zeros((M, 12), np.int64)
    E = L.or_hex8_edges(C.c_int64(M), _p(conn, C.c_int64), C.c_int64(nnodes), C.c_int64(cap),
                        _p(edges, C.c_int64), _p(ee, C.c_int64))
    return edges[:E].copy(), ee


def hex8_geometry(coords, conn, elem_edges, edges):
    coords, conn, ee, edges = _f64(coords), _i64(conn), _i64(elem_edges), _i64(edges)
    area = np.zeros((edges.shape[0], 3))
    vol = np.zeros(coords.shape[0])
    lib().or_hex8_geometry(C.c_int64(coords.shape[0]), _p(coords, C.c_double), C.c_int64(conn.shape[0]),
                           _p(conn, C.c_int64), _p(ee, C.c_int64), C.c_int64(edges.shape[0]),
                           _p(edges, C.c_int64), _p(area, C.c_double), _p(vol, C.c_double))
    return area, vol


# TetSCS / TetSCV restated in numpy (src/master_element/Tet4CVFEM.C:243-360,
# 522-620): the element's points are its nodes, edge midpoints, face
# centroids and centroid; each sub-control surface is the quad (edge
# midpoint, face centroid, centroid, face centroid) whose area vector is
# the triangle fan about the quad centre (Quad3DSCS::determinant_scs), and
# each sub-control volume the hexahedron (node, midpoints, face centroids,
# centroid) by Grandy's 24-triangle formula (Hex8GeometryFunctions.h).
_TET_LR = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
_TET_FACET = [(4, 7, 14, 13), (7, 14, 10, 5), (6, 12, 14, 7), (11, 13, 14, 12), (13, 9, 10, 14),
              (10, 8, 12, 14)]
_TET_SUB = [(0, 4, 7, 6, 11, 13, 14, 12), (1, 5, 7, 4, 9, 10, 14, 13), (2, 6, 7, 5, 8, 12, 14, 10),
            (3, 9, 13, 11, 8, 10, 14, 12)]
_GRANDY_FACES = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 3, 7)]
_GRANDY_TRI = [(0, 8, 1), (8, 2, 1), (3, 2, 8), (3, 8, 0), (6, 9, 5), (7, 9, 6), (4, 9, 7), (4, 5, 9),
               (10, 0, 1), (5, 10, 1), (4, 10, 5), (4, 0, 10), (7, 6, 11), (6, 2, 11), (2, 3, 11),
               (3, 7, 11), (6, 12, 2), (5, 12, 6), (5, 1, 12), (1, 2, 12), (0, 4, 13), (4, 7, 13),
               (7, 3, 13), (3, 0, 13)]


def _fan_area(q):
    xm = q.mean(axis=1, keepdims=True)
    r = q - xm
    return 0.5 * sum(np.cross(r[:, t], r[:, (t + 1) % 4]) for t in range(4))


def _grandy(s):
    cv = np.concatenate([s, np.stack([s[:, list(f)].mean(axis=1) for f in _GRANDY_FACES], axis=1)], axis=1)
    vol = 0.0
    for a, b, c in _GRANDY_TRI:
        p, q, r = cv[:, a], cv[:, b], cv[:, c]
        vol = vol + np.einsum("md,md->m", p + q + r, np.cross(q - p, r - p))
    return vol / 18.0


def tet4_geometry(coords, conn, edges):
    """Edge area vectors and dual volumes of a Tet4 mesh (edges: E x 2 with
    edges[:, 0] < edges[:, 1]; an element edge adds its area vector with
    the sign of its orientation relative to the edge)."""
    coords, conn, edges = _f64(coords), _i64(conn), _i64(edges)
    c = coords[conn]  # M x 4 x 3
    mid = lambda a, b: 0.5 * (c[:, a] + c[:, b])
    fc = lambda a, b, d: (c[:, a] + c[:, b] + c[:, d]) / 3.0
    p = np.stack([c[:, 0], c[:, 1], c[:, 2], c[:, 3], mid(0, 1), mid(1, 2), mid(2, 0), fc(0, 1, 2),
                  mid(2, 3), mid(3, 1), fc(1, 2, 3), mid(0, 3), fc(0, 2, 3), fc(0, 1, 3),
                  c.mean(axis=1)], axis=1)
    N, E = coords.shape[0], edges.shape[0]
    key = edges[:, 0] * N + edges[:, 1]
    order = np.argsort(key)
    area = np.zeros((E, 3))
    for ip, (a, b) in enumerate(_TET_LR):
        s = _fan_area(p[:, list(_TET_FACET[ip])])
        na, nb = conn[:, a], conn[:, b]
        lo, hi = np.minimum(na, nb), np.maximum(na, nb)
        e = order[np.searchsorted(key[order], lo * N + hi)]
        np.add.at(area, e, np.where((na == lo)[:, None], s, -s))
    vol = np.zeros(N)
    for j in range(4):
        np.add.at(vol, conn[:, j], _grandy(p[:, list(_TET_SUB[j])]))
    return area, vol


def build_graph(nalu_id, edges, num_dof=1):
    nalu_id, edges = _i64(nalu_id), _i64(edges)
    N = nalu_id.shape[0]
    nnz = C.c_int64()
    L = lib()
    nrows = L.or_build_graph(C.c_int64(N), _p(nalu_id, C.c_int64), C.c_int64(edges.shape[0]),
                             _p(edges, C.c_int64), num_dof, C.byref(nnz), None, None, None)
    rp = np.zeros(nrows + 1, np.int64)
    ci = np.zeros(nnz.value, np.int32)
    lid = np.zeros(N, np.int64)
    L.or_build_graph(C.c_int64(N), _p(nalu_id, C.c_int64), C.c_int64(edges.shape[0]),
                     _p(edges, C.c_int64), num_dof, C.byref(nnz), _p(rp, C.c_int64),
                     _p(ci, C.c_int32), _p(lid, C.c_int64))
    return rp, ci, lid


def scalar_local(*args, mag=False, **kw):
    return _scalar_local(*args, mag=mag, **kw)


def _scalar_local(edges, coords, vrtm, q, dqdx, density, diff, area, mdot, opts: ScalarOpts, mag=False):
    edges = _i64(edges)
    E = edges.shape[0]
    lhs = np.zeros((E, 4))
    rhs = np.zeros((E, 2))
    args = [_f64(a) for a in (coords, vrtm, q, dqdx, density, diff, area, mdot)]
    fn = lib().or_scalar_edge_local_mag if mag else lib().or_scalar_edge_local
    fn(C.c_int64(E), _p(edges, C.c_int64), *[_p(a, C.c_double) for a in args],
                               C.byref(opts), _p(lhs, C.c_double), _p(rhs, C.c_double))
    return lhs, rhs


def continuity_local(*args, mag=False, **kw):
    return _continuity_local(*args, mag=mag, **kw)


def _continuity_local(edges, coords, vel, dpdx, density, pressure, udiag, area, opts: ContinuityOpts,
                      mag=False):
    edges = _i64(edges)
    E = edges.shape[0]
    lhs = np.zeros((E, 4))
    rhs = np.zeros((E, 2))
    args = [_f64(a) for a in (coords, vel, dpdx, density, pressure, udiag, area)]
    fn = lib().or_continuity_edge_local_mag if mag else lib().or_continuity_edge_local
    fn(C.c_int64(E), _p(edges, C.c_int64), *[_p(a, C.c_double) for a in args],
                                   C.byref(opts), _p(lhs, C.c_double), _p(rhs, C.c_double))
    return lhs, rhs


def momentum_local(*args, mag=False, **kw):
    return _momentum_local(*args, mag=mag, **kw)


def _momentum_local(edges, coords, vrtm, vel, dudx, visc, density, mask, area, mdot, pecfac,
                    opts: MomentumOpts, mag=False):
    edges = _i64(edges)
    E = edges.shape[0]
    lhs = np.zeros((E, 36))
    rhs = np.zeros((E, 6))
    args = [_f64(a) for a in (coords, vrtm, vel, dudx, visc, density, mask, area, mdot, pecfac)]
    fn = lib().or_momentum_edge_local_mag if mag else lib().or_momentum_edge_local
    fn(C.c_int64(E), _p(edges, C.c_int64), *[_p(a, C.c_double) for a in args],
                                 C.byref(opts), _p(lhs, C.c_double), _p(rhs, C.c_double))
    return lhs, rhs


def sum_into(edges, num_dof, lhs, rhs, node_lid, row_ptr, col_idx, nthreads=1, with_abs=True):
    edges, lhs, rhs = _i64(edges), _f64(lhs), _f64(rhs)
    node_lid, row_ptr = _i64(node_lid), _i64(row_ptr)
    col_idx = np.ascontiguousarray(col_idx, np.int32)
    nnz, nrows = col_idx.shape[0], row_ptr.shape[0] - 1
    vals = np.zeros(nnz)
    b = np.zeros(nrows)
    va = np.zeros(nnz) if with_abs else None
    ba = np.zeros(nrows) if with_abs else None
    lib().or_sum_into_edges(C.c_int64(edges.shape[0]), _p(edges, C.c_int64), num_dof, _p(lhs, C.c_double),
                            _p(rhs, C.c_double), _p(node_lid, C.c_int64), _p(row_ptr, C.c_int64),
                            _p(col_idx, C.c_int32), _p(vals, C.c_double), _p(b, C.c_double),
                            _p(va, C.c_double), _p(ba, C.c_double), nthreads)
    return vals, b, va, ba


def apply_dirichlet(nodes, num_dof, begin, end, q, bc, node_lid, row_ptr, col_idx, vals, rhs):
    nodes, q, bc = _i64(nodes), _f64(q), _f64(bc)
    lib().or_apply_dirichlet(C.c_int64(nodes.shape[0]), _p(nodes, C.c_int64), num_dof, begin, end,
                             _p(q, C.c_double), _p(bc, C.c_double), _p(_i64(node_lid), C.c_int64),
                             _p(_i64(row_ptr), C.c_int64),
                             _p(np.ascontiguousarray(col_idx, np.int32), C.c_int32),
                             _p(vals, C.c_double), _p(rhs, C.c_double))


def reset_rows(nodes, begin, end, diag, rhs_value, node_lid, row_ptr, col_idx, vals, rhs):
    nodes = _i64(nodes)
    lib().or_reset_rows(C.c_int64(nodes.shape[0]), _p(nodes, C.c_int64), begin, end, C.c_double(diag),
                        C.c_double(rhs_value), _p(_i64(node_lid), C.c_int64), _p(_i64(row_ptr), C.c_int64),
                        _p(np.ascontiguousarray(col_idx, np.int32), C.c_int32), _p(vals, C.c_double),
                        _p(rhs, C.c_double))


def spmv(row_ptr, col_idx, vals, x, nthreads=1):
    row_ptr, vals, x = _i64(row_ptr), _f64(vals), _f64(x)
    col_idx = np.ascontiguousarray(col_idx, np.int32)
    y = np.zeros(row_ptr.shape[0] - 1)
    lib().or_spmv(C.c_int64(y.shape[0]), _p(row_ptr, C.c_int64), _p(col_idx, C.c_int32),
                  _p(vals, C.c_double), _p(x, C.c_double), _p(y, C.c_double), nthreads)
    return y


def solve(row_ptr, col_idx, vals, b, method=0, precond=1, order=None, kspace=50, max_iters=50,
          tol=1e-8, nthreads=1, inner_sweeps=1):
    row_ptr, vals, b = _i64(row_ptr), _f64(vals), _f64(b)
    col_idx = np.ascontiguousarray(col_idx, np.int32)
    n = b.shape[0]
    x = np.zeros(n)
    hist = np.zeros(max_iters + 1)
    rep = SolveReport()
    od = None if order is None else _i64(order)
    lib().or_solve(C.c_int64(n), _p(row_ptr, C.c_int64), _p(col_idx, C.c_int32), _p(vals, C.c_double),
                   _p(b, C.c_double), _p(x, C.c_double), method, precond, _p(od, C.c_int64), kspace,
                   max_iters, C.c_double(tol), _p(hist, C.c_double), C.byref(rep), nthreads, inner_sweeps)
    return x, hist[:rep.iterations + 1].copy(), rep


def gpu_reduction_blocks(n: int, sms: int) -> int:
    """Blocks of the GPU library's FP64 reductions for n rows on a device
    with `sms` multiprocessors (KrylovSolver::setup)."""
    return max(1, min(8 * sms, (n + 511) // 512))


def solve_gpu_order(row_ptr, col_idx, vals, b, method=0, precond=1, order=None, class_ptr=None, kspace=50,
                    max_iters=50, tol=1e-8, inner_sweeps=1, red_blocks=1, lanes=8, sstep_size=5):
    """The FP64 solvers in the GPU library's operation order
    (or_solve_gpu_order): returns x, history (iterations + 1), report."""
    row_ptr, vals, b = _i64(row_ptr), _f64(vals), _f64(b)
    col_idx = np.ascontiguousarray(col_idx, np.int32)
    n = b.shape[0]
    x = np.zeros(n)
    hist = np.zeros(max_iters + 1)
    rep = SolveReport()
    od = None if order is None else _i64(order)
    cp = None if class_ptr is None else _i64(class_ptr)
    nc = 0 if cp is None else len(cp) - 1
    st = lib().or_solve_gpu_order(C.c_int64(n), _p(row_ptr, C.c_int64), _p(col_idx, C.c_int32),
                                  _p(vals, C.c_double), _p(b, C.c_double), _p(x, C.c_double), method, precond,
                                  _p(od, C.c_int64), _p(cp, C.c_int64), nc, kspace, max_iters, C.c_double(tol),
                                  _p(hist, C.c_double), C.byref(rep), inner_sweeps, red_blocks, lanes,
                                  sstep_size)
    if st == 1:
        raise ValueError("or_solve_gpu_order: Gauss-Seidel needs the colour classes")
    return x, hist[:rep.iterations + 1].copy(), rep


def precond_apply(row_ptr, col_idx, vals, kind, x, order=None, inner_sweeps=1):
    row_ptr, vals, x = _i64(row_ptr), _f64(vals), _f64(x)
    col_idx = np.ascontiguousarray(col_idx, np.int32)
    y = np.zeros_like(x)
    od = None if order is None else _i64(order)
    lib().or_precond_apply(C.c_int64(x.shape[0]), _p(row_ptr, C.c_int64), _p(col_idx, C.c_int32),
                           _p(vals, C.c_double), kind, _p(od, C.c_int64), _p(x, C.c_double),
                           _p(y, C.c_double), inner_sweeps)
    return y


def mdot_unit_test(edges, vel, rho, area):
    edges = _i64(edges)
    out = np.zeros(edges.shape[0])
    lib().or_mdot_unit_test(C.c_int64(edges.shape[0]), _p(edges, C.c_int64), _p(_f64(vel), C.c_double),
                            _p(_f64(rho), C.c_double), _p(_f64(area), C.c_double), _p(out, C.c_double))
    return out


def mdot_edge(edges, coords, vel, dpdx, rho, p, udiag, area, noc=1.0, interp=1.0):
    edges = _i64(edges)
    out = np.zeros(edges.shape[0])
    args = [_f64(a) for a in (coords, vel, dpdx, rho, p, udiag, area)]
    lib().or_mdot_edge(C.c_int64(edges.shape[0]), _p(edges, C.c_int64), *[_p(a, C.c_double) for a in args],
                       C.c_double(noc), C.c_double(interp), _p(out, C.c_double))
    return out


def nodal_grad_edge(edges, phi, area, dualvol, dim1=1):
    edges = _i64(edges)
    N = dualvol.shape[0]
    grad = np.zeros((N, dim1 * 3))
    lib().or_nodal_grad_edge(C.c_int64(edges.shape[0]), _p(edges, C.c_int64), dim1,
                             _p(_f64(phi), C.c_double), _p(_f64(area), C.c_double),
                             _p(_f64(dualvol), C.c_double), _p(grad, C.c_double))
    return grad


def peclet_classic(pe, hf):
    return lib().or_peclet_classic(pe, hf)


def peclet_tanh(x, c1, c2):
    return lib().or_peclet_tanh(x, c1, c2)


def mass_bdf(kind, rho, dnv, q=None, dpdx=None, dt=0.1, gamma=(1.0, -1.0, 0.0)):
    """Lumped-mass BDF node kernels (kind 0 scalar, 1 continuity, 2 momentum):
    rho, dnv, q are (Nm1, N, Np1) triples of node arrays; returns the per-node
    diagonal LHS and rhs (N, or N x 3 for momentum)."""
    n = rho[2].shape[0]
    nd = 3 if kind == 2 else 1
    zeros = np.zeros(n * nd)
    qq = [(_f64(a) if a is not None else zeros) for a in (q if q is not None else (None, None, None))]
    dp = _f64(dpdx) if dpdx is not None else np.zeros(3 * n)
    lhs, rhs = np.zeros(n * nd), np.zeros(n * nd)
    args = [_f64(a) for a in (*rho, *dnv)] + qq + [dp]
    lib().or_mass_bdf(C.c_int(kind), C.c_int64(n), *[_p(a, C.c_double) for a in args], C.c_double(dt),
                      *[C.c_double(g) for g in gamma], _p(lhs, C.c_double), _p(rhs, C.c_double))
    return (lhs.reshape(n, 3), rhs.reshape(n, 3)) if nd == 3 else (lhs, rhs)


def _face_local(fn, nl, ipn, arrays, tail):
    ipn = _i64(ipn)
    n = ipn.shape[0]
    lhs = np.zeros((n, nl * nl))
    rhs = np.zeros((n, nl))
    keep = [None if a is None else _f64(a) for a in arrays]
    ptrs = [None if a is None else _p(a, C.c_double) for a in keep]
    fn(C.c_int64(n), _p(ipn, C.c_int64), *ptrs, *tail, _p(lhs, C.c_double), _p(rhs, C.c_double))
    return lhs, rhs


def continuity_open_local(ipn, coords, vel, dpdx, density, pressure, pressure_bc, udiag, areav, dynp,
                          opts: ContinuityOpenOpts, mag=False):
    """Face-IP local systems (node order R, L) of ContinuityOpenEdgeKernel."""
    fn = lib().or_continuity_open_local_mag if mag else lib().or_continuity_open_local
    return _face_local(fn, 2, ipn, (coords, vel, dpdx, density, pressure, pressure_bc, udiag, areav, dynp),
                       [C.byref(opts)])


def momentum_open_local(ipn, coords, vel, dudx, visc, velocity_bc, areav, mdot, opts: MomentumOpenOpts,
                        mag=False):
    fn = lib().or_momentum_open_local_mag if mag else lib().or_momentum_open_local
    return _face_local(fn, 6, ipn, (coords, vel, dudx, visc, velocity_bc, areav, mdot), [C.byref(opts)])


def momentum_symmetry_local(ipn, coords, vel, dudx, visc, areav, opts: MomentumSymmetryOpts, mag=False):
    fn = lib().or_momentum_symmetry_local_mag if mag else lib().or_momentum_symmetry_local
    return _face_local(fn, 6, ipn, (coords, vel, dudx, visc, areav), [C.byref(opts)])


def scalar_open_local(ipn, q, q_bc, mdot, relax=1.0, mag=False):
    fn = lib().or_scalar_open_local_mag if mag else lib().or_scalar_open_local
    return _face_local(fn, 2, ipn, (q, q_bc, mdot), [C.c_double(relax)])


def mt19937_uniform(bounds):
    """Draws of a default-seeded std::mt19937 through
    std::uniform_real_distribution<double>(lo, hi), one per (lo, hi)."""
    lo = np.array([b[0] for b in bounds], np.float64)
    hi = np.array([b[1] for b in bounds], np.float64)
    out = np.zeros(len(bounds))
    lib().or_mt19937_uniform(C.c_int(len(bounds)), _p(lo, C.c_double), _p(hi, C.c_double),
                             _p(out, C.c_double))
    return out


def mdot_open(ipn, coords, vel, dpdx, density, pressure, pressure_bc, udiag, areav, dynp=None, noc_fac=1.0,
              pstab_fac=1.0):
    """Open mass flow rate per face IP (MdotOpenEdgeAlg)."""
    ipn = _i64(ipn)
    out = np.zeros(ipn.shape[0])
    keep = [None if a is None else _f64(a) for a in (coords, vel, dpdx, density, pressure, pressure_bc, udiag,
                                                     areav, dynp)]
    lib().or_mdot_open(C.c_int64(ipn.shape[0]), _p(ipn, C.c_int64), *[_p(a, C.c_double) for a in keep],
                       C.c_double(noc_fac), C.c_double(pstab_fac), _p(out, C.c_double))
    return out


def extract_diagonal(pairs, lhs, num_dof, num_nodes):
    """NGPApplyCoeff::extract_diagonal (src/SolverAlgorithm.C:89-104): every
    two-node local system (edge, or face IP as (R, L)) adds lhs(ix, ix),
    ix = node * num_dof, to its node's momentum_diag entry."""
    pairs = _i64(pairs)
    nl = 2 * num_dof
    out = np.zeros(num_nodes)
    for a in range(2):
        ix = a * num_dof
        np.add.at(out, pairs[:, a], lhs[:, ix * nl + ix])
    return out


def abl_wall_local(ipn, vel, bcvel, density, heatflux, cp, areav, ustar, zh, opts: AblWallOpts, mag=False):
    """Face-IP local systems (node order R, L) of MomentumABLWallFuncEdgeKernel."""
    fn = lib().or_abl_wall_local_mag if mag else lib().or_abl_wall_local
    return _face_local(fn, 6, ipn, (vel, bcvel, density, heatflux, cp, areav, ustar, zh), [C.byref(opts)])


def abl_shear_local(ipn, areav, tau, slip, mag=False):
    """Face-IP local systems (node order R, L) of MomentumABLWallShearStressEdgeKernel."""
    fn = lib().or_abl_shear_local_mag if mag else lib().or_abl_shear_local
    return _face_local(fn, 6, ipn, (areav, tau), [C.c_int(int(slip))])


def set_threads(n):
    """Threads of the oracle's OpenMP loops without an explicit count."""
    lib().or_set_threads(C.c_int(int(n)))


def local_graph_replay(row_lengths, ops, num_dof=1):
    """LocalGraphArrays: pre-sized rows, then insertIndices(row, cols, numDof)
    for each (row, cols) in ops. Returns (rowPointers, colIndices) or None on
    row overflow."""
    rl = np.asarray(row_lengths, np.int64)
    rows = np.array([r for r, _ in ops], np.int32)
    ns = np.array([len(c) for _, c in ops], np.int32)
    cols = np.array([x for _, c in ops for x in c], np.int32)
    rp = np.zeros(len(rl) + 1, np.int64)
    ci = np.zeros(int(rl.sum()), np.int32)
    rc = lib().or_local_graph_replay(C.c_int(len(rl)), _p(rl, C.c_int64), C.c_int(len(ops)), _p(rows, C.c_int32),
                                     _p(ns, C.c_int32), _p(cols, C.c_int32), C.c_int(num_dof), _p(rp, C.c_int64),
                                     _p(ci, C.c_int32))
    return None if rc else (rp, ci)


def face_scs_areas(faces, coords):
    """Sub-face area vectors of quad (Quad3DSCS) or triangle (Tri3DSCS)
    faces, one per face node: (nfaces * nn, 3)."""
    faces = _i64(faces)
    nf, nn = faces.shape
    out = np.zeros((nf * nn, 3))
    lib().or_face_scs_areas(C.c_int64(nf), C.c_int(nn), _p(faces, C.c_int64), _p(_f64(coords), C.c_double),
                            _p(out, C.c_double))
    return out


def nodal_grad_bndry(faces, area, phi, dualvol, shifted=True):
    """NodalGradBndryElemAlg (src/ngp_algorithms/NodalGradBndryElemAlg.C:
    130-152) on quad faces: each face IP adds q_ip A_ip / V to its node's
    gradient, q_ip = the IP node's value (shifted) or the quad's bilinear
    interpolation at the sub-control-volume centre (weights 9/16 own node,
    3/16 face neighbours, 1/16 opposite). faces: (nf, 4) node ids in IP
    order; area: (nf * 4, 3); phi: (N, dim1). Returns (N, 3 * dim1)."""
    faces = _i64(faces)
    phi = np.asarray(phi, np.float64).reshape(len(dualvol), -1)
    dim1 = phi.shape[1]
    out = np.zeros((len(dualvol), 3 * dim1))
    nf, nn = faces.shape
    for f in range(nf):
        for ip in range(nn):
            if shifted:
                q = phi[faces[f, ip]]
            else:
                w = np.zeros(nn)
                w[ip] = 9 / 16
                w[(ip + 1) % nn] = w[(ip + 3) % nn] = 3 / 16
                w[(ip + 2) % nn] = 1 / 16
                q = w @ phi[faces[f]]
            node = faces[f, ip]
            out[node] += (q[:, None] * area[nn * f + ip][None, :]).ravel() / dualvol[node]
    return out
