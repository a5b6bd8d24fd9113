"""The single-kernel momentum assembly (momentum_fused_k: edge chunks and
row blocks of one persistent kernel, the coefficients passing through an
L2-sized ring) against the two-kernel form it replaces: the same CSR values
and rhs bit for bit, on a ring and on the whole-buffer fallback, for every
option specialisation, when accumulating, and over repeated launches. The
oracle parity of the default path is in test_gpu_assembly.py."""
import numpy as np
import pytest

from gpu_util import momentum_fields, to_dev_dict

pytestmark = pytest.mark.gpu

OPTS = [dict(alpha=0.0, alpha_upw=1.0, upw_factor=1.0, relax=1.0, include_div_u=0.0, use_limiter=0),
        dict(alpha=0.0, alpha_upw=1.0, upw_factor=1.0, relax=0.8, include_div_u=1.0, use_limiter=1),
        dict(alpha=0.2, alpha_upw=0.6, upw_factor=1.0, relax=0.7, include_div_u=1.0, use_limiter=1),
        dict(alpha=0.3, alpha_upw=0.9, upw_factor=0.5, relax=1.0, include_div_u=0.0, use_limiter=0),
        dict(alpha=0.0, alpha_upw=1.0, upw_factor=1.0, relax=1.0, include_div_u=0.0, use_limiter=1),
        dict(alpha=0.0, alpha_upw=1.0, upw_factor=1.0, relax=1.0, include_div_u=1.0, use_limiter=0),
        dict(alpha=0.1, alpha_upw=1.0, upw_factor=1.0, relax=1.0, include_div_u=1.0, use_limiter=0),
        dict(alpha=0.1, alpha_upw=1.0, upw_factor=1.0, relax=1.0, include_div_u=0.0, use_limiter=1)]


def _fields(mesh, seed):
    rng = np.random.default_rng(seed)
    N, E = mesh.num_nodes, mesh.num_edges
    return dict(coords=mesh.coords, velocity=rng.normal(size=(N, 3)), dudx=rng.normal(size=(N, 9)),
                viscosity=rng.uniform(1e-3, 1e-1, N), density=np.ones(N), mask=rng.choice([0.0, 1.0], N),
                area=mesh.area, mdot=rng.normal(size=E), pecfac=rng.uniform(size=E))


def _both(nw, mesh, f, od, gid=None, nid=None, repeats=1):
    out = []
    for path in (nw.ASSEMBLY_TWO_KERNELS, nw.ASSEMBLY_SINGLE_KERNEL):
        ls = nw.LinearSystem(3)
        ls.build_edge_graph(mesh.num_nodes, mesh.edges, gid, nid)
        ls.finalize()
        ls.set_assembly_path(path)
        mf = momentum_fields(nw, to_dev_dict(f))
        for _ in range(repeats):
            ls.zero_system()
            ls.assemble_momentum(mf, nw.MomentumOpts(**od))
        v1, r1 = ls.to_host()
        ls.assemble_momentum(mf, nw.MomentumOpts(**od))  # accumulates
        v2, r2 = ls.to_host()
        out.append((v1, r1, v2, r2, ls.assembly_schedule()))
    return out


def _same(a, b):
    for x, y in zip(a[:4], b[:4]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("k", range(len(OPTS)))
def test_every_option_specialisation_matches_two_kernels(nw, k):
    # 194k nodes, 2,237 edge chunks: large enough for a ring at the lag of
    # a full GPU of resident blocks
    mesh = nw.Mesh(64, 60, 48, stretch_z=1.05, jitter=0.06, seed=12)
    two, one = _both(nw, mesh, _fields(mesh, 13 + k), OPTS[k])
    _same(two, one)
    s = one[4]
    assert s["single_kernel"] == 1 and 0 < s["ring_chunks"] < s["edge_chunks"]


@pytest.mark.parametrize("kind", ["random_tets", "rcm_tets", "periodic", "tiny"])
def test_ring_fallback_periodic_and_small_meshes(nw, kind):
    if kind == "random_tets":
        mesh = nw.Mesh(24, 22, 20, tets=True, renumber=1, renumber_seed=5)
    elif kind == "rcm_tets":
        mesh = nw.Mesh(24, 22, 20, tets=True, renumber=2, renumber_seed=9)
    elif kind == "periodic":
        mesh = nw.Mesh(20, 18, 12, periodic_x=True, periodic_y=True)
    else:
        mesh = nw.Mesh(2, 1, 1)
    gid = mesh.global_id if kind == "periodic" else None
    nid = mesh.nalu_id if kind == "periodic" else None
    two, one = _both(nw, mesh, _fields(mesh, 3), OPTS[1], gid, nid, repeats=3)
    _same(two, one)
    if kind == "random_tets":
        assert one[4]["ring_bytes"] == 0  # one slot per chunk


def test_lowmach_128x128x64_matches_two_kernels(nw):
    """The benchmark workload: ring in L2, 12.5k edge chunks, 12.7k row
    blocks, repeated launches."""
    case = nw.workload.lowmach_case(128, 128, 64, seed=2)
    mesh, nd = case.mesh, case.node
    f = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
             density=nd["density"], mask=nd["mask"], area=mesh.area, mdot=case.edge["mdot"],
             pecfac=case.edge["pecfac"])
    mo = case.opts["momentum"]
    od = {k: getattr(mo, k) for k, _ in mo._fields_}
    two, one = _both(nw, mesh, f, od, repeats=4)
    _same(two, one)
    s = one[4]
    assert 0 < s["ring_bytes"] <= 64 << 20
