"""MatrixMarket export (TpetraLinearSystem::writeToFile layout) and import."""
import numpy as np
import pytest

from gpu_util import dev, scalar_fields, to_dev_dict

pytestmark = pytest.mark.gpu


def _scalar_system(nw):
    case = nw.workload.scalar_case(10, seed=1)
    mesh = case.mesh
    f = dict(coords=mesh.coords, velocity=case.node["velocity"], q=case.node["q"], dqdx=case.node["dqdx"],
             density=case.node["density"], diff=case.node["diff_coeff"], area=mesh.area, mdot=case.edge["mdot"])
    ls = nw.LinearSystem(1)
    ls.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    ls.finalize()
    d = to_dev_dict(f)
    ls.zero_system()
    ls.assemble_scalar(scalar_fields(nw, d), case.opts["scalar"])
    return ls, mesh


@pytest.mark.filterwarnings("ignore::DeprecationWarning")
def test_write_read_roundtrip(nw, tmp_path):
    scipy_io = pytest.importorskip("scipy.io")
    ls, mesh = _scalar_system(nw)
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    x = np.arange(len(rhs), dtype=np.float64) * 0.5
    ls.write_matrix_market(tmp_path / "scalar", 3, x=x)
    A = scipy_io.mmread(str(tmp_path / "scalar-O-3.mm.1")).tocsr()
    # rows of this system are the periodic masters in nalu-id order
    masters = np.sort(mesh.global_id[mesh.nalu_id == mesh.global_id])
    gid = masters  # 1 dof: GID = nalu id
    assert A.shape == (int(masters.max()), int(masters.max()))
    assert A.nnz == len(vals)
    for r in range(len(rhs)):
        row = A.getrow(int(gid[r]) - 1)
        cols = np.sort(row.indices)
        np.testing.assert_array_equal(cols + 1, np.sort(gid[ci[rp[r]:rp[r + 1]]]))
        got = dict(zip(row.indices + 1, row.data))
        for p in range(rp[r], rp[r + 1]):
            assert got[int(gid[ci[p]])] == vals[p]
    b = scipy_io.mmread(str(tmp_path / "scalar-O-3.rhs.1")).ravel()
    np.testing.assert_array_equal(b[gid - 1], rhs)
    xs = scipy_io.mmread(str(tmp_path / "scalar-O-3.sln.1")).ravel()
    np.testing.assert_array_equal(xs[gid - 1], x)
    # import into a fresh handle on the same graph
    ls2 = nw.LinearSystem(1)
    ls2.build_edge_graph(mesh.num_nodes, mesh.edges, mesh.global_id, mesh.nalu_id)
    ls2.finalize()
    ls2.read_matrix_market(tmp_path / "scalar-O-3.mm.1", tmp_path / "scalar-O-3.rhs.1")
    v2, r2 = ls2.to_host()
    np.testing.assert_array_equal(v2, vals)
    np.testing.assert_array_equal(r2, rhs)


def test_read_rejects_entries_outside_the_graph(nw, tmp_path):
    ls, mesh = _scalar_system(nw)
    ls.write_matrix_market(tmp_path / "s", 0)
    text = (tmp_path / "s-O-0.mm.1").read_text().splitlines()
    n = int(text[2].split()[0])
    # an entry coupling the first and the last dof is not an edge of the mesh
    text[3] = f"1 {n} 1.0"
    (tmp_path / "bad.mm").write_text("\n".join(text) + "\n")
    with pytest.raises(nw.NwError, match="not in the graph"):
        ls.read_matrix_market(tmp_path / "bad.mm")
