"""Edge cases through the C ABI: no edges (empty rows, zero rhs, trivial
solve), nodes in no edge, a system too small for aggregation to coarsen,
and the smallest 3-dof system (one edge)."""
import numpy as np
import pytest

from gpu_util import check_close, dev, oracle_continuity, oracle_momentum

pytestmark = pytest.mark.gpu


def _continuity_fields(nw, coords, area, N, rng):
    d = dict(coords=coords, velocity=rng.normal(size=(N, 3)), dpdx=rng.normal(size=(N, 3)),
             density=np.ones(N), pressure=rng.normal(size=N), udiag=np.ones(N), area=area)
    t = {k: dev(np.ascontiguousarray(v)) for k, v in d.items()}
    f = nw.ContinuityFields(*(t[k].data_ptr() for k in ("coords", "velocity", "dpdx", "density", "pressure",
                                                        "udiag", "area")))
    return f, t


def test_no_edges_gives_zero_rows_and_a_trivial_solve(nw, orc):
    import torch
    N = 17
    rng = np.random.default_rng(0)
    edges = np.zeros((0, 2), np.int64)
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(N, edges)
    ls.finalize()
    rp, ci = ls.graph()
    orp, oci, _ = orc.build_graph(np.arange(1, N + 1), edges, 1)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    # as in the reference's edge graph, a node in no edge has an empty row
    assert len(ci) == 0 and np.all(rp == 0)
    f, keep = _continuity_fields(nw, rng.normal(size=(N, 3)), np.zeros((1, 3)), N, rng)
    ls.from_host(rhs=np.full(N, 3.0))
    ls.zero_system()
    ls.assemble_continuity(f, nw.ContinuityOpts(1.0, 1.0, 1.0, 0.0))
    vals, rhs = ls.to_host()
    assert len(vals) == 0 and np.all(rhs == 0.0)
    # a node kernel needs the diagonal entry, which these rows do not have
    z = dev(np.zeros(N))
    with pytest.raises(nw.NwError, match="no diagonal"):
        ls.assemble_mass_bdf("scalar", [z, z, z], [z, z, z], q=[z, z, z])
    x = torch.zeros(N, dtype=torch.float64, device="cuda")
    rep = ls.solve(x)
    assert rep.converged == 1 and rep.iterations == 0 and rep.rhs_norm == 0.0
    assert torch.count_nonzero(x).item() == 0


def test_isolated_nodes_match_oracle(nw, orc):
    mesh = nw.Mesh(4, 3, 3, jitter=0.05, seed=2)
    N0 = mesh.num_nodes
    extra = 5  # nodes in no edge, appended after the mesh nodes
    N = N0 + extra
    rng = np.random.default_rng(1)
    coords = np.vstack([mesh.coords, rng.normal(size=(extra, 3))])
    f, keep = _continuity_fields(nw, coords, mesh.area, N, rng)
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(N, mesh.edges)
    ls.finalize()
    ls.zero_system()
    co = nw.ContinuityOpts(1.0, 1.0, 1.0, 0.0)
    ls.assemble_continuity(f, co)
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    h = {k: v.cpu().numpy() for k, v in keep.items()}
    o = oracle_continuity(orc, mesh.edges, np.arange(1, N + 1), h,
                          {k: getattr(co, k) for k, _ in co._fields_})
    assert np.array_equal(rp, o["rp"]) and np.array_equal(ci, o["ci"])
    check_close(vals, o["vals"], o["vabs"], "values")
    check_close(rhs, o["rhs"], o["rabs"], "rhs")
    # the isolated nodes' rows are empty and their rhs zero
    lid = ls.node_lid(N)
    for node in range(N0, N):
        r = lid[node]
        assert rp[r + 1] == rp[r] and rhs[r] == 0.0


def test_learned_preconditioner_on_a_tiny_graph(nw):
    import torch
    ls = nw.workload.poisson_system((3, 3, 2), seed=3)
    net = nw.Learned(seed=0)
    ls.attach_learned(net)
    cg = ls.coarse_graph()
    assert cg["nc"] >= 1
    ls.set_solver_cfg(nw.solver_cfg(method=nw.FGMRES, preconditioner=nw.PC_LEARNED, precision=nw.PREC_MIXED,
                                    kspace=30, inner_kspace=30, max_iterations=500, tolerance=1e-8))
    x = torch.zeros(ls.sizes()[0], dtype=torch.float64, device="cuda")
    rep = ls.solve(x)
    assert rep.converged == 1 and rep.final_abs_residual <= 1.01e-8 * rep.rhs_norm


def test_single_edge_momentum(nw, orc):
    """Two nodes, one edge: the smallest 3-dof system (6 x 6, fully dense)."""
    N = 2
    edges = np.array([[0, 1]], np.int64)
    coords = np.array([[0.0, 0.0, 0.0], [0.3, 0.1, -0.05]])
    area = np.array([[0.2, 0.05, 0.01]])
    rng = np.random.default_rng(4)
    host = dict(coords=coords, velocity=rng.normal(size=(N, 3)), dudx=rng.normal(size=(N, 9)),
                viscosity=np.array([1e-3, 2e-3]), density=np.ones(N), mask=np.ones(N), area=area,
                mdot=np.array([0.7]), pecfac=np.array([0.3]))
    t = {k: dev(np.ascontiguousarray(v)) for k, v in host.items()}
    fm = nw.MomentumFields(*(t[k].data_ptr() for k in ("coords", "velocity", "dudx", "viscosity", "density",
                                                        "mask", "area", "mdot", "pecfac")))
    ls = nw.LinearSystem(3)
    ls.build_edge_graph(N, edges)
    ls.finalize()
    ls.zero_system()
    mo = nw.MomentumOpts(alpha=0.3, alpha_upw=0.8, upw_factor=1.0, relax=0.7, include_div_u=1.0, use_limiter=1)
    ls.assemble_momentum(fm, mo)
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    assert vals.shape[0] == 36
    o = oracle_momentum(orc, edges, np.arange(1, N + 1), host, {k: getattr(mo, k) for k, _ in mo._fields_})
    assert np.array_equal(rp, o["rp"]) and np.array_equal(ci, o["ci"])
    check_close(vals, o["vals"], o["vabs"], "values")
    check_close(rhs, o["rhs"], o["rabs"], "rhs")


def test_momentum_in_edge_ranges_equals_one_call(nw):
    """Edge phase over uneven edge ranges, then the row phase: the same
    values and rhs, bit for bit, as one nw_assemble_momentum_edges call; the
    range bounds are checked."""
    import torch
    case = nw.workload.lowmach_case(20, 16, 12, seed=2)
    mesh = case.mesh
    nd = case.node
    host = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
                density=nd["density"], mask=nd["mask"], area=mesh.area, mdot=case.edge["mdot"],
                pecfac=case.edge["pecfac"])
    d = {k: dev(v) for k, v in host.items()}
    fm = nw.MomentumFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dudx", "viscosity", "density", "mask",
                                                        "area", "mdot", "pecfac")))
    mo = case.opts["momentum"]
    out = []
    for split in (None, [0, 1, 777, 5000, mesh.num_edges]):
        ls = nw.LinearSystem(3)
        ls.build_edge_graph(mesh.num_nodes, mesh.edges)
        ls.finalize()
        ls.zero_system()
        if split is None:
            ls.assemble_momentum(fm, mo)
        else:
            for a, b in zip(split[:-1], split[1:]):
                ls.assemble_momentum_range(fm, mo, a, b)
            ls.assemble_momentum_rows(mo)
            with pytest.raises(nw.NwError, match="edge range"):
                ls.assemble_momentum_range(fm, mo, 5, mesh.num_edges + 1)
        out.append(ls.to_host())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_momentum_row_ranges_pipeline_with_edge_ranges(nw):
    """Edge ranges each followed by the row range their edges complete
    (rows below the chunk's last first node), as the streamed end-to-end
    step runs them: bit for bit the one-call assembly. On a zeroed system
    the row ranges must come in order; stopping part-way and reading the
    system gives zeros in the rows not yet covered; on an assembled system
    a range adds into its rows."""
    case = nw.workload.lowmach_case(20, 16, 12, seed=2)
    mesh = case.mesh
    nd = case.node
    host = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
                density=nd["density"], mask=nd["mask"], area=mesh.area, mdot=case.edge["mdot"],
                pecfac=case.edge["pecfac"])
    d = {k: dev(v) for k, v in host.items()}
    fm = nw.MomentumFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dudx", "viscosity", "density", "mask",
                                                        "area", "mdot", "pecfac")))
    mo = case.opts["momentum"]
    N, E = mesh.num_nodes, mesh.num_edges

    def fresh():
        ls = nw.LinearSystem(3)
        ls.build_edge_graph(N, mesh.edges)
        ls.finalize()
        ls.zero_system()
        return ls

    ref = fresh()
    ref.assemble_momentum(fm, mo)
    v_ref, r_ref = ref.to_host()
    # rows complete after edge chunk [.., b): every incident edge index < b
    maxinc = np.full(N, -1)
    np.maximum.at(maxinc, mesh.edges[:, 0], np.arange(E))
    np.maximum.at(maxinc, mesh.edges[:, 1], np.arange(E))
    ready = lambda b: int(np.searchsorted(np.maximum.accumulate(maxinc), b))  # rows r with prefix max < b
    ls = fresh()
    bounds = [0, 1000, 2500, 4000, E]
    done = 0
    for a, b in zip(bounds[:-1], bounds[1:]):
        ls.assemble_momentum_range(fm, mo, a, b)
        r = ready(b) if b < E else N
        ls.assemble_momentum_rows_range(mo, done, r)
        done = r
    v, rh = ls.to_host()
    assert np.array_equal(v, v_ref) and np.array_equal(rh, r_ref)
    # out of order on a zeroed system
    ls = fresh()
    ls.assemble_momentum_range(fm, mo, 0, E)
    with pytest.raises(nw.NwError, match="row ranges"):
        ls.assemble_momentum_rows_range(mo, 10, 20)
    # part-way, then read: the rows not covered are zero
    half = N // 2
    ls.assemble_momentum_rows_range(mo, 0, half)
    v, rh = ls.to_host()
    rp, _ = ls.graph()
    cut = rp[3 * half]
    assert np.array_equal(v[:cut], v_ref[:cut]) and not np.any(v[cut:])
    assert np.array_equal(rh[:3 * half], r_ref[:3 * half]) and not np.any(rh[3 * half:])
    # on an assembled system a range adds
    ls.assemble_momentum_rows_range(mo, 0, N)
    v2, rh2 = ls.to_host()
    np.testing.assert_array_equal(v2[cut:], v_ref[cut:])
    np.testing.assert_allclose(v2[:cut], 2 * v_ref[:cut], rtol=1e-15, atol=0)


@pytest.mark.parametrize("general", [False, True])
def test_continuity_edge_ranges_equal_the_one_call_assembly(nw, general):
    """Continuity edge ranges in order from edge 0, then the row phase, as
    the streamed end-to-end step runs them: bit for bit the one-call
    assembly, on the node pre-pass route (the reference's default options)
    and on the general one (interpolated velocity blend, incompressible
    density scaling). Ranges out of order, and a row phase before the
    ranges cover every edge, are refused."""
    case = nw.workload.lowmach_case(20, 16, 12, seed=4)
    mesh = case.mesh
    nd = case.node
    host = dict(coords=mesh.coords, velocity=nd["velocity"], dpdx=nd["dpdx"], density=nd["density"],
                pressure=nd["pressure"], udiag=nd["udiag"], area=mesh.area)
    d = {k: dev(v) for k, v in host.items()}
    fc = nw.ContinuityFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dpdx", "density", "pressure",
                                                        "udiag", "area")))
    co = case.opts["continuity"]
    if general:
        co = nw.ContinuityOpts(**{k: getattr(co, k) for k, _ in co._fields_})
        co.interp_together = 0.5
        co.solve_incompressible = 1.0
    N, E = mesh.num_nodes, mesh.num_edges

    def fresh():
        ls = nw.LinearSystem(1)
        ls.build_edge_graph(N, mesh.edges)
        ls.finalize()
        ls.zero_system()
        return ls

    ref = fresh()
    ref.assemble_continuity(fc, co)
    v_ref, r_ref = ref.to_host()
    ls = fresh()
    bounds = [0, 0, 1000, 2500, 2500, 4000, E]
    for a, b in zip(bounds[:-1], bounds[1:]):
        ls.assemble_continuity_range(fc, co, a, b)
    ls.assemble_continuity_rows()
    v, rh = ls.to_host()
    assert np.array_equal(v, v_ref) and np.array_equal(rh, r_ref)
    # a second assembly on the same handle: ranges restart at edge 0
    ls.zero_system()
    for a, b in ((0, E // 2), (E // 2, E)):
        ls.assemble_continuity_range(fc, co, a, b)
    ls.assemble_continuity_rows()
    v, rh = ls.to_host()
    assert np.array_equal(v, v_ref) and np.array_equal(rh, r_ref)
    # refused: a gap, a range past the end, rows before every edge is done,
    # rows twice without new ranges
    ls = fresh()
    ls.assemble_continuity_range(fc, co, 0, 1000)
    with pytest.raises(nw.NwError, match="follow each other"):
        ls.assemble_continuity_range(fc, co, 1500, 2000)
    with pytest.raises(nw.NwError, match="out of bounds"):
        ls.assemble_continuity_range(fc, co, 1000, E + 1)
    with pytest.raises(nw.NwError, match="cover every edge"):
        ls.assemble_continuity_rows()
    ls.assemble_continuity_range(fc, co, 1000, E)
    ls.assemble_continuity_rows()
    with pytest.raises(nw.NwError, match="cover every edge"):
        ls.assemble_continuity_rows()


def test_streamed_step_reads_only_the_node_fields_it_has(nw):
    """The streamed end-to-end step: node fields arrive in index order, a
    slice ahead of each edge chunk (up to the largest node index of the
    edges so far); the rest of every node field is NaN until its slice
    lands. Momentum and continuity edge ranges, momentum row ranges and the
    continuity row phase then give the one-call assemblies bit for bit: no
    range reads a node field it was not given."""
    import torch
    case = nw.workload.lowmach_case(20, 16, 12, seed=6)
    mesh = case.mesh
    nd = case.node
    host = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
                density=nd["density"], mask=nd["mask"], pressure=nd["pressure"], dpdx=nd["dpdx"],
                udiag=nd["udiag"], area=mesh.area, mdot=case.edge["mdot"], pecfac=case.edge["pecfac"])
    N, E = mesh.num_nodes, mesh.num_edges
    edge_keys = ("area", "mdot", "pecfac")
    full = {k: dev(v) for k, v in host.items()}
    part = {k: (v.clone() if k in edge_keys else torch.full_like(v, float("nan"))) for k, v in full.items()}
    mo, co = case.opts["momentum"], case.opts["continuity"]

    def fields(d):
        fm = nw.MomentumFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dudx", "viscosity", "density", "mask", "area", "mdot", "pecfac")))
        fc = nw.ContinuityFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dpdx", "density", "pressure", "udiag", "area")))
        return fm, fc

    def fresh(ndof):
        ls = nw.LinearSystem(ndof)
        ls.build_edge_graph(N, mesh.edges)
        ls.finalize()
        ls.zero_system()
        return ls

    fm, fc = fields(full)
    rm, rc = fresh(3), fresh(1)
    rm.assemble_momentum(fm, mo)
    rc.assemble_continuity(fc, co)
    vm_ref, bm_ref = rm.to_host()
    vc_ref, bc_ref = rc.to_host()
    fm, fc = fields(part)
    lsm, lsc = fresh(3), fresh(1)
    reach = np.maximum.accumulate(mesh.edges.max(axis=1)) + 1  # nodes needed by edges 0..e
    maxinc = np.full(N, -1)
    np.maximum.at(maxinc, mesh.edges[:, 0], np.arange(E))
    np.maximum.at(maxinc, mesh.edges[:, 1], np.arange(E))
    bounds = [0, 700, 1900, 3100, 4400, E]
    have = done = 0
    for a, b in zip(bounds[:-1], bounds[1:]):
        need = int(reach[b - 1])
        for k in host:
            if k not in edge_keys:
                part[k][have:need] = full[k][have:need]
        have = need
        lsm.assemble_momentum_range(fm, mo, a, b)
        r = int(np.searchsorted(np.maximum.accumulate(maxinc), b)) if b < E else N
        lsm.assemble_momentum_rows_range(mo, done, r)
        done = r
        lsc.assemble_continuity_range(fc, co, a, b)
    lsc.assemble_continuity_rows()
    vm, bm = lsm.to_host()
    vc, bc = lsc.to_host()
    assert np.array_equal(vm, vm_ref) and np.array_equal(bm, bm_ref)
    assert np.array_equal(vc, vc_ref) and np.array_equal(bc, bc_ref)
