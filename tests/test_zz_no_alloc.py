"""The no-allocation continuity assembly (nw_assemble_continuity_edges_noalloc).

This entry point is for callers that cannot allocate device memory when they
assemble, such as a host code that hands out all device memory from its own
pool allocator, sized up front. It keeps its per-edge
scratch in a fixed array inside the library and writes into the caller's
arrays. The test calls it through the C ABI twice in a row, with different
inputs, and checks each result against the regular entry point
(nw_assemble_continuity_edges) within the assembly tests' tolerance
(1e-12 times the oracle's running magnitude of each entry). It also checks
that the calls leave the device's free memory unchanged, that meshes
above the stated edge limit are refused, and that the call captures into a
CUDA graph whose replays equal eager calls.

Named test_zz_* so pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import check_close, continuity_fields, oracle_continuity, to_dev_dict

pytestmark = pytest.mark.gpu


def _free_bytes():
    import torch
    free, _ = torch.cuda.mem_get_info()
    return free


def _inputs(nw, seed):
    case = nw.workload.lowmach_case(24, 20, 12, seed=seed)
    m, nd = case.mesh, case.node
    f = dict(coords=m.coords, velocity=nd["velocity"], dpdx=nd["dpdx"], density=nd["density"],
             pressure=nd["pressure"], udiag=nd["udiag"], area=m.area)
    return case, f


def test_noalloc_matches_regular_entry_point_twice(nw, orc):
    import torch
    case, f1 = _inputs(nw, seed=2)
    mesh = case.mesh
    co = case.opts["continuity"]
    od = {k: getattr(co, k) for k, _ in co._fields_}
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges)
    ls.finalize()
    nr, nnz = ls.sizes()
    # second input set: same mesh, different fields
    rng = np.random.default_rng(11)
    f2 = dict(f1, velocity=rng.normal(size=f1["velocity"].shape), pressure=rng.normal(size=mesh.num_nodes),
              udiag=rng.uniform(1.0, 3.0, mesh.num_nodes))
    d1, d2 = to_dev_dict(f1), to_dev_dict(f2)
    # caller-owned outputs, prefilled with garbage: every entry gets written
    vals = torch.full((nnz,), 7.0, dtype=torch.float64, device="cuda")
    rhs = torch.full((nr,), -3.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    results = []
    free_before = None
    for d, f in ((d1, f1), (d2, f2)):
        ls.assemble_continuity_noalloc(continuity_fields(nw, d), co, vals, rhs)
        torch.cuda.synchronize()
        if free_before is None:
            free_before = _free_bytes()  # after the first call's one-time set-up
        got_v, got_r = vals.cpu().numpy().copy(), rhs.cpu().numpy().copy()
        ls.zero_system()
        ls.assemble_continuity(continuity_fields(nw, d), co)
        ref_v, ref_r = ls.to_host()
        ref = oracle_continuity(orc, mesh.edges, mesh.nalu_id, f, od)
        check_close(got_v, ref_v, ref["vabs"], "noalloc values vs regular entry point")
        check_close(got_r, ref_r, ref["rabs"], "noalloc rhs vs regular entry point")
        check_close(got_v, ref["vals"], ref["vabs"], "noalloc values vs oracle")
        results.append(got_v)
    assert not np.array_equal(results[0], results[1])
    # a third call after the regular one allocates nothing either
    ls.assemble_continuity_noalloc(continuity_fields(nw, d1), co, vals, rhs)
    torch.cuda.synchronize()
    assert _free_bytes() == free_before


def test_noalloc_rejects_meshes_above_the_limit(nw):
    import torch
    mesh = nw.Mesh(64, 64, 44)
    assert mesh.num_edges > 524288
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges)
    ls.finalize()
    N = mesh.num_nodes
    z3 = torch.zeros((N, 3), dtype=torch.float64, device="cuda")
    one = torch.ones(N, dtype=torch.float64, device="cuda")
    area = torch.from_numpy(mesh.area).cuda()
    coords = torch.from_numpy(mesh.coords).cuda()
    f = nw.ContinuityFields(coords.data_ptr(), z3.data_ptr(), z3.data_ptr(), one.data_ptr(), one.data_ptr(),
                            one.data_ptr(), area.data_ptr())
    nr, nnz = ls.sizes()
    vals = torch.zeros(nnz, dtype=torch.float64, device="cuda")
    rhs = torch.zeros(nr, dtype=torch.float64, device="cuda")
    with pytest.raises(nw.NwError) as e:
        ls.assemble_continuity_noalloc(f, nw.ContinuityOpts(1.0, 1.0, 1.0, 0.0), vals, rhs)
    assert e.value.status == 1 and "524288" in str(e.value)


def test_noalloc_call_captures_into_a_cuda_graph(nw):
    """The call allocates nothing and makes no synchronous call, so it can be
    captured into a CUDA graph on the handle's stream: captured once after a
    warm-up call, the graph is replayed with new field values written into
    the same device buffers, and each replay equals an eager call bit for
    bit (the same kernels on the same inputs)."""
    import torch
    case, f = _inputs(nw, seed=4)
    mesh = case.mesh
    co = case.opts["continuity"]
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges)
    ls.finalize()
    nr, nnz = ls.sizes()
    s = torch.cuda.Stream()
    ls.set_stream(s.cuda_stream)
    d = to_dev_dict(f)
    fields = continuity_fields(nw, d)
    vals = torch.zeros(nnz, dtype=torch.float64, device="cuda")
    rhs = torch.zeros(nr, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        ls.assemble_continuity_noalloc(fields, co, vals, rhs)  # one-time set-up outside the capture
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ls.assemble_continuity_noalloc(fields, co, vals, rhs)
    torch.cuda.synchronize()
    rng = np.random.default_rng(21)
    prev = None
    for _ in range(2):
        d["velocity"].copy_(torch.from_numpy(rng.normal(size=f["velocity"].shape)))
        d["pressure"].copy_(torch.from_numpy(rng.normal(size=mesh.num_nodes)))
        d["udiag"].copy_(torch.from_numpy(rng.uniform(1.0, 3.0, mesh.num_nodes)))
        vals.fill_(7.0)
        rhs.fill_(-3.0)
        g.replay()
        torch.cuda.synchronize()
        got_v, got_r = vals.cpu().numpy().copy(), rhs.cpu().numpy().copy()
        ev = torch.full((nnz,), 5.0, dtype=torch.float64, device="cuda")
        er = torch.full((nr,), 5.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            ls.assemble_continuity_noalloc(fields, co, ev, er)
        s.synchronize()
        np.testing.assert_array_equal(got_v, ev.cpu().numpy())
        np.testing.assert_array_equal(got_r, er.cpu().numpy())
        if prev is not None:
            assert not np.array_equal(prev, got_v)
        prev = got_v
