"""The oracle's own rebuild of the benchmark workload (oracle/cases.py, used
by the CPU reference arm so that it never loads the product library) gives
the inputs the product's workload module gives."""
import numpy as np
import pytest


@pytest.mark.parametrize("shape,opts", [((9, 7, 6), dict(seed=2, stretch=1.08, jitter=0.05, lz=0.5)),
                                        ((5, 6, 4), dict(seed=11, stretch=1.0, jitter=0.0, lz=1.0))])
def test_oracle_lowmach_case_matches_library_case(nw, shape, opts):
    from oracle import cases
    ref = cases.lowmach_case(*shape, **opts)
    lib = nw.workload.lowmach_case(*shape, **opts)
    np.testing.assert_array_equal(ref.mesh.coords, lib.mesh.coords)
    np.testing.assert_array_equal(ref.mesh.nalu_id, lib.mesh.nalu_id)
    key = {tuple(e): i for i, e in enumerate(ref.mesh.edges.tolist())}
    perm = np.array([key[tuple(e)] for e in lib.mesh.edges.tolist()])
    assert sorted(perm.tolist()) == list(range(ref.mesh.num_edges))
    tol = dict(rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(ref.mesh.area[perm], lib.mesh.area, **tol)
    np.testing.assert_allclose(ref.mesh.dualvol, lib.mesh.dualvol, **tol)
    np.testing.assert_allclose(ref.mesh.bnd_area, lib.mesh.bnd_area, **tol)
    for k in ("velocity", "viscosity", "density", "mask", "pressure", "udiag"):
        np.testing.assert_array_equal(ref.node[k], lib.node[k])
    for k in ("dudx", "dpdx"):
        s = np.abs(lib.node[k]).max()
        assert np.abs(ref.node[k] - lib.node[k]).max() <= 1e-13 * s
    for k in ("mdot", "pecfac"):
        s = np.abs(lib.edge[k]).max()
        assert np.abs(ref.edge[k][perm] - lib.edge[k]).max() <= 1e-13 * s
