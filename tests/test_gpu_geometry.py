"""Edge area vectors and dual volumes on the GPU (nw_geometry_*, the
GeometryInteriorAlg path) against the host mesh generator, bit for bit, and
against the oracle's Hex8 restatement and the reference's geometry golds."""
import numpy as np
import pytest

from gpu_util import dev

pytestmark = pytest.mark.gpu


def _gpu_geometry(nw, mesh):
    import torch
    g = nw.Geometry(mesh.num_nodes, mesh.conn, mesh.edges, mesh.nalu_id)
    area = torch.zeros((mesh.num_edges, 3), dtype=torch.float64, device="cuda")
    vol = torch.zeros(mesh.num_nodes, dtype=torch.float64, device="cuda")
    g.compute(dev(mesh.coords), area, vol)
    torch.cuda.synchronize()
    return area.cpu().numpy(), vol.cpu().numpy()


@pytest.mark.parametrize("kind", ["stretched", "periodic", "tets_random", "tets_rcm"])
def test_gpu_geometry_equals_host_generator(nw, kind):
    if kind == "stretched":
        mesh = nw.Mesh(12, 10, 8, stretch_z=1.08, jitter=0.05, seed=3, lz=0.5)
    elif kind == "periodic":
        mesh = nw.Mesh(6, 5, 4, periodic_x=True, periodic_y=True, jitter=0.0)
    elif kind == "tets_random":
        mesh = nw.Mesh(7, 6, 5, tets=True, jitter=0.05, seed=4, renumber=1, renumber_seed=3)
    else:
        mesh = nw.Mesh(7, 6, 5, tets=True, jitter=0.05, seed=4, renumber=2, renumber_seed=3)
    area, vol = _gpu_geometry(nw, mesh)
    np.testing.assert_array_equal(area, mesh.area)
    np.testing.assert_array_equal(vol, mesh.dualvol)


def test_gpu_geometry_against_oracle_and_golds(nw, orc, golds):
    mesh = nw.Mesh(9, 8, 7, stretch_z=1.1, jitter=0.07, seed=5)
    area, vol = _gpu_geometry(nw, mesh)
    oedges, ee = orc.hex8_edges(mesh.conn, mesh.num_nodes)
    oarea, ovol = orc.hex8_geometry(mesh.coords, mesh.conn, ee, oedges)
    key = {tuple(e): i for i, e in enumerate(oedges.tolist())}
    perm = np.array([key[tuple(e)] for e in mesh.edges.tolist()])
    assert np.abs(area - oarea[perm]).max() <= 1e-14 * np.abs(oarea).max()
    np.testing.assert_allclose(vol, ovol, rtol=1e-13)
    # the reference's unit-cube golds (UnitTestGeometryAlg.C): dual volume
    # 0.125 at every node, |A|^2 = 0.0625 on every edge
    one = nw.Mesh(1, 1, 1)
    a1, v1 = _gpu_geometry(nw, one)
    g = golds["geometry_hex8_unit_cube"]
    np.testing.assert_allclose(v1, g["dual_volume"], rtol=0, atol=1e-15)
    assert a1.shape[0] == g["num_edges"]
    np.testing.assert_allclose((a1 ** 2).sum(1), g["area_mag_sq"], rtol=0, atol=1e-15)


def test_gpu_geometry_rejects_edges_missing_from_the_list(nw):
    mesh = nw.Mesh(3, 3, 3)
    with pytest.raises(nw.NwError) as e:
        nw.Geometry(mesh.num_nodes, mesh.conn, mesh.edges[:-5])
    assert e.value.status == 1
