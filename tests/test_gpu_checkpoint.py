"""Checkpoint / resume of a linear system (nw_linsys_checkpoint_save /
_load): graph, values, rhs, solver configuration, last report, residual
history and the solution round-trip bit for bit, a resumed solve repeats the
original one exactly, and corrupted, truncated or mismatched files are
refused with NW_INVALID_ARG (faults injected in the file, on the host)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _poisson(nw, shape, seed=3):
    return nw.workload.poisson_system(shape, seed=seed, stretch=1.04)


def test_checkpoint_round_trip_and_resume(nw, tmp_path):
    import torch
    ls = _poisson(nw, (20, 18, 12))
    nr, _ = ls.sizes()
    ls.set_solver_cfg(nw.solver_cfg(kspace=30, max_iterations=2000, tolerance=1e-9,
                                    preconditioner=nw.PC_SGS_NATURAL))
    x = torch.zeros(nr, dtype=torch.float64, device="cuda")
    rep = ls.solve(x)
    assert rep.converged
    hist = ls.residual_history()
    vals, rhs = ls.to_host()
    path = tmp_path / "system.nwckpt"
    ls.checkpoint_save(path, x)

    other = _poisson(nw, (20, 18, 12), seed=8)  # same graph, other rhs
    x2 = torch.zeros(nr, dtype=torch.float64, device="cuda")
    rep2 = other.checkpoint_load(path, x2)
    v2, r2 = other.to_host()
    np.testing.assert_array_equal(v2, vals)
    np.testing.assert_array_equal(r2, rhs)
    np.testing.assert_array_equal(x2.cpu().numpy(), x.cpu().numpy())
    np.testing.assert_array_equal(other.residual_history(), hist)
    assert (rep2.iterations, rep2.converged, rep2.final_abs_residual) == (rep.iterations, rep.converged,
                                                                          rep.final_abs_residual)
    # the restored configuration and system repeat the solve exactly
    x3 = torch.zeros(nr, dtype=torch.float64, device="cuda")
    rep3 = other.solve(x3)
    assert rep3.iterations == rep.iterations
    np.testing.assert_array_equal(other.residual_history(), hist)
    np.testing.assert_array_equal(x3.cpu().numpy(), x.cpu().numpy())


def test_checkpoint_faults_are_refused(nw, tmp_path):
    ls = _poisson(nw, (10, 9, 8))
    path = tmp_path / "a.nwckpt"
    ls.checkpoint_save(path)
    raw = path.read_bytes()
    bad = bytearray(raw)
    bad[len(bad) // 2] ^= 0x40
    (tmp_path / "flipped.nwckpt").write_bytes(bytes(bad))
    (tmp_path / "short.nwckpt").write_bytes(raw[:-17])
    for name, what in (("flipped.nwckpt", "checksum"), ("short.nwckpt", "truncated")):
        with pytest.raises(nw.NwError) as e:
            ls.checkpoint_load(tmp_path / name)
        assert e.value.status == 1 and what in str(e.value)
    other = _poisson(nw, (10, 9, 7))
    with pytest.raises(nw.NwError) as e:
        other.checkpoint_load(path)
    assert e.value.status == 1
    import torch
    with pytest.raises(nw.NwError):
        ls.checkpoint_load(path, torch.zeros(ls.sizes()[0], dtype=torch.float64, device="cuda"))
