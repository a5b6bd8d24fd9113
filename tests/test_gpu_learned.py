"""Learned two-level preconditioner on the GPU, through the C ABI.

Tolerances, all written against the oracle (oracle/learned_oracle.py):
* BF16 tensor-core GEMMs vs torch FP32 matmul of the same BF16 operands:
  FP32 outputs within 1e-5 of the sum of |products| per entry; the BF16
  output of the forward GEMM within 2^-7 relative (one BF16 rounding step
  after a differently ordered FP32 sum) plus 1e-5 of the |product| sum.
* Forward output and every parameter-gradient block vs the oracle with the
  same BF16 rounding points: relative L2 error <= 5e-3 (what remains is
  FP32 accumulation, which can move a value across a BF16 rounding
  boundary). Vs the pure FP64 oracle: cosine >= 0.99 and relative L2
  error <= 0.1 per block (BF16 keeps 8 significant bits).
"""
import numpy as np
import pytest

from gpu_util import dev

from oracle import learned_oracle as lo

pytestmark = pytest.mark.gpu


def _bf16_tensor(a):
    import torch
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).cuda()


@pytest.mark.parametrize("m", [37, 5003])
def test_bf16_gemms_match_torch(nw, m):
    import torch
    rng = np.random.default_rng(m)
    a = _bf16_tensor(rng.normal(size=(m, 128)))
    wt = _bf16_tensor(rng.normal(size=(64, 128)) * 0.1)
    out = torch.empty((m, 64), dtype=torch.bfloat16, device="cuda")
    nw.gemm_bf16(0, m, a, wt, out)
    ref = (a.float() @ wt.float().T)
    scale = (a.float().abs() @ wt.float().abs().T)
    err = (out.float() - torch.relu(ref)).abs()
    assert bool((err <= 2.0 ** -7 * ref.abs() + 1e-5 * scale).all())

    dz = _bf16_tensor(rng.normal(size=(m, 64)))
    w = _bf16_tensor(rng.normal(size=(128, 64)) * 0.1)
    dx = torch.empty((m, 128), dtype=torch.float32, device="cuda")
    nw.gemm_bf16(1, m, dz, w, dx)
    ref = dz.float() @ w.float().T
    assert bool(((dx - ref).abs() <= 1e-5 * (dz.float().abs() @ w.float().abs().T) + 1e-30).all())

    dw = torch.empty((128, 64), dtype=torch.float32, device="cuda")
    nw.gemm_bf16(2, m, a, dz, dw)
    ref = a.float().T @ dz.float()
    assert bool(((dw - ref).abs() <= 1e-5 * (a.float().abs().T @ dz.float().abs()) + 1e-30).all())


@pytest.mark.parametrize("kind", [3, 4])
@pytest.mark.parametrize("m", [1, 127, 128, 129, 5003, 65553])
def test_tcgen05_forward_gemm_matches_torch_and_mma_sync(nw, m, kind):
    """The tensor-core (tcgen05, TMEM accumulator) forward layer GEMM, tiles
    staged by cp.async (kind 3) or by TMA with the 128-byte swizzle (kind 4):
    within BF16 rounding of torch's FP32 product, on full and ragged 128-row
    tiles; and against the mma.sync kernel, which differs at most by the
    BF16 rounding of FP32 sums taken in another order."""
    import torch
    rng = np.random.default_rng(100 + m)
    a = _bf16_tensor(rng.normal(size=(m, 128)))
    wt = _bf16_tensor(rng.normal(size=(64, 128)) * 0.1)
    out = torch.full((m, 64), 7.0, dtype=torch.bfloat16, device="cuda")
    nw.gemm_bf16(kind, m, a, wt, out)
    ref = a.float() @ wt.float().T
    scale = a.float().abs() @ wt.float().abs().T
    err = (out.float() - torch.relu(ref)).abs()
    assert bool((err <= 2.0 ** -7 * ref.abs() + 1e-5 * scale).all())
    out0 = torch.empty_like(out)
    nw.gemm_bf16(0, m, a, wt, out0)
    d = (out.float() - out0.float()).abs()
    assert bool((d <= 2.0 ** -7 * out0.float().abs() + 1e-5 * scale).all())


@pytest.mark.parametrize("m", [1, 37, 128, 129, 5003, 65553])
def test_tcgen05_backward_gemms_match_torch_and_mma_sync(nw, m):
    """The training step's backward GEMMs on the tcgen05 tensor cores: dX =
    dZ W^T with TMA tiles (kind 5) and dW = X^T dZ with the node chunks
    transposed while staged (kind 6), FP32 outputs within 1e-5 of the sum of
    |products| of torch's FP32 product of the same BF16 operands, and of the
    mma.sync kernels (kinds 1, 2) they replaced."""
    import torch
    rng = np.random.default_rng(300 + m)
    x = _bf16_tensor(rng.normal(size=(m, 128)))
    dz = _bf16_tensor(rng.normal(size=(m, 64)))
    w = _bf16_tensor(rng.normal(size=(128, 64)) * 0.1)
    dx = torch.full((m, 128), 7.0, dtype=torch.float32, device="cuda")
    nw.gemm_bf16(5, m, dz, w, dx)
    ref = dz.float() @ w.float().T
    scale = dz.float().abs() @ w.float().abs().T
    assert bool(((dx - ref).abs() <= 1e-5 * scale + 1e-30).all())
    dx1 = torch.empty_like(dx)
    nw.gemm_bf16(1, m, dz, w, dx1)
    assert bool(((dx - dx1).abs() <= 2e-5 * scale + 1e-30).all())
    dw = torch.full((128, 64), 7.0, dtype=torch.float32, device="cuda")
    nw.gemm_bf16(6, m, x, dz, dw)
    ref = x.float().T @ dz.float()
    scale = x.float().abs().T @ dz.float().abs()
    assert bool(((dw - ref).abs() <= 1e-5 * scale + 1e-30).all())
    dw1 = torch.empty_like(dw)
    nw.gemm_bf16(2, m, x, dz, dw1)
    assert bool(((dw - dw1).abs() <= 2e-5 * scale + 1e-30).all())


def _poisson(nw, shape, seed=3, stretch=1.04, jitter=0.0, rhs_seed=None):
    return nw.workload.poisson_system(shape, seed=seed, stretch=stretch, jitter=jitter, rhs_seed=rhs_seed)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _blocks(g):
    H = lo.H
    o = [0, 2 * H, 2 * H + 2 * H * H, 2 * H + 4 * H * H, 2 * H + 6 * H * H, len(g)]
    return [g[o[i]:o[i + 1]] for i in range(5)]


def test_forward_and_gradient_match_oracle(nw):
    import torch
    ls = _poisson(nw, (14, 12, 10))
    net = nw.Learned(seed=5)
    ls.attach_learned(net)
    cg = ls.coarse_graph()
    nc = cg["nc"]
    rng = np.random.default_rng(11)
    # a fresh network's output layer is zero (no gradient reaches the
    # hidden layers): check with every layer random
    H = lo.H
    net.set_params(np.concatenate([rng.uniform(-1.7, 1.7, 2 * H), rng.uniform(-0.2, 0.2, 6 * H * H),
                                   rng.uniform(-0.2, 0.2, H)]).astype(np.float32))
    rc = rng.normal(size=nc).astype(np.float32)
    ea, ca = 40.0, 25.0
    rc_d = dev(rc)
    ec_d = torch.zeros(nc, dtype=torch.float32, device="cuda")
    net.forward(ls, rc_d, ec_d)
    L, g = net.loss_grad(ls, rc_d, ea, ca)
    p = net.params().astype(np.float64)
    Lb, gb, ecb = lo.loss_and_grad(p, cg, rc, ea, ca, bf16_points=True)
    Lf, gf, ecf = lo.loss_and_grad(p, cg, rc, ea, ca)
    ec = ec_d.cpu().numpy().astype(np.float64)
    assert _rel(ec, ecb) <= 5e-3
    assert _rel(ec, ecf) <= 0.1
    Ac = lo.coarse_operator(cg)
    lscale = (np.abs(ecb) @ np.abs(Ac) @ np.abs(ecb) + 2 * np.abs(ecb) @ np.abs(rc) + ca) / ea
    assert abs(L - Lb) <= 5e-3 * lscale
    for blk, (a, b, f) in enumerate(zip(_blocks(g.astype(np.float64)), _blocks(gb), _blocks(gf))):
        assert _rel(a, b) <= 5e-3, (blk, _rel(a, b))
        cos = float(a @ f / (np.linalg.norm(a) * np.linalg.norm(f)))
        assert cos >= 0.99 and _rel(a, f) <= 0.1, (blk, cos, _rel(a, f))


def test_weight_file_roundtrip_and_corruption(nw, tmp_path):
    net = nw.Learned(seed=1)
    p = net.params()
    path = tmp_path / "w.bin"
    net.save(path)
    other = nw.Learned(seed=2)
    assert not np.array_equal(other.params(), p)
    other.load(path)
    np.testing.assert_array_equal(other.params(), p)
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.bin"
    raw[100] ^= 0x40
    bad.write_bytes(bytes(raw))
    with pytest.raises(nw.NwError, match="checksum"):
        other.load(bad)
    bad.write_bytes(path.read_bytes()[:1000])
    with pytest.raises(nw.NwError, match="truncated"):
        other.load(bad)
    bad.write_bytes(b"XXXXXXXX" + path.read_bytes()[8:])
    with pytest.raises(nw.NwError, match="not a network weight file"):
        other.load(bad)
    np.testing.assert_array_equal(other.params(), p)  # failed loads change nothing


def _solve(nw, ls, pc, method, tol=1e-8):
    import torch
    ls.set_solver_cfg(nw.solver_cfg(method=method, preconditioner=pc, precision=nw.PREC_MIXED, kspace=30,
                                    inner_kspace=30, max_iterations=20000, tolerance=tol))
    nr, _ = ls.sizes()
    x = torch.zeros(nr, dtype=torch.float64, device="cuda")
    rep = ls.solve(x)
    # FP64-verified residual
    vals, rhs = ls.to_host()
    rp, ci = ls.graph()
    xh = x.cpu().numpy()
    ax = np.add.reduceat(vals * xh[ci], rp[:-1]) if len(vals) else np.zeros(nr)
    true_rel = np.linalg.norm(rhs - ax) / np.linalg.norm(rhs)
    return rep, true_rel


def test_training_reduces_loss_and_speeds_up_the_solve(nw):
    """Train on pairs from two systems, then solve a held-out system and
    right-hand side with the trained network and with the same cycle
    without it: the same network untrained (random initialisation, seed 0),
    the non-learned coarse direction D_c^-1 r_c (same energy-optimal
    scaling), and no coarse correction (output layer zeroed: the two SGS
    sweeps alone). Training must cut the FGMRES iteration count against the
    untrained network and against no coarse correction."""
    net = nw.Learned(seed=0)
    train_a = _poisson(nw, (40, 40, 24), seed=3, stretch=1.04)
    train_b = _poisson(nw, (40, 40, 24), seed=4, stretch=1.10, jitter=0.05)
    npairs = 0
    for ls in (train_a, train_b):
        ls.attach_learned(net)
        npairs = net.harvest(ls, restarts=24, kspace=30)
    assert npairs >= 40
    before = net.evaluate(train_a)
    net.train(train_a, epochs=30, batch=4, lr=2e-3, seed=1)
    after = net.evaluate(train_a)
    assert after < before, (before, after)
    test = _poisson(nw, (40, 40, 24), seed=9, stretch=1.07, jitter=0.03, rhs_seed=99)
    without = nw.Learned(seed=0)
    p0 = without.params()
    p0[-lo.H:] = 0.0  # zero output layer: alpha = 0, no coarse correction
    without.set_params(p0)
    test.attach_learned(without)
    rep_0, rel_0 = _solve(nw, test, nw.PC_LEARNED, nw.FGMRES)
    untrained = nw.Learned(seed=0)
    test.attach_learned(untrained)
    rep_u, rel_u = _solve(nw, test, nw.PC_LEARNED, nw.FGMRES)
    jac = nw.Learned(seed=0)
    jac.set_coarse_direction(1)
    test.attach_learned(jac)
    rep_j, rel_j = _solve(nw, test, nw.PC_LEARNED, nw.FGMRES)
    test.attach_learned(net)
    rep_l, rel_l = _solve(nw, test, nw.PC_LEARNED, nw.FGMRES)
    its = dict(trained=rep_l.iterations, untrained=rep_u.iterations, jacobi_coarse=rep_j.iterations,
               no_coarse=rep_0.iterations)
    for r, rel in ((rep_0, rel_0), (rep_u, rel_u), (rep_j, rel_j), (rep_l, rel_l)):
        assert r.converged and r.fallback == 0 and rel <= 1.01e-8, its
    assert rep_l.iterations < rep_0.iterations, its
    assert rep_l.iterations < rep_u.iterations, its


def test_broken_network_falls_back_to_sgs(nw):
    ls = _poisson(nw, (20, 20, 12))
    net = nw.Learned(seed=0)
    ls.attach_learned(net)
    net.set_params(np.full(net.num_params, np.nan, np.float32))
    rep, rel = _solve(nw, ls, nw.PC_LEARNED, nw.FGMRES)
    assert rep.fallback == 1 and rep.converged == 1 and rel <= 1.01e-8


def test_committed_128cube_network_loads_and_solves(nw):
    """The network of the 128^3-node training set (nalu-wind_gb300/weights,
    made by train_poisson.py: 200 systems, ~20k pairs) loads with its
    checksum and recipe, differs from the untrained initialisation, and
    preconditions a held-out system's mixed FGMRES to 1e-8."""
    import torch
    from pathlib import Path
    path = Path(nw.__file__).parent / "weights" / "poisson_128cube.nwl"
    net, info = nw.training.load_poisson_network(path)
    assert info["systems"] == 200 and info["pairs"] >= 19000 and info["shape"] == [127, 127, 127]
    assert not np.allclose(net.params(), nw.Learned(seed=0).params())
    ls = _poisson(nw, (40, 36, 30), seed=77, stretch=1.06, jitter=0.05)
    ls.attach_learned(net)
    ls.set_solver_cfg(nw.solver_cfg(method=nw.FGMRES, kspace=30, inner_kspace=30, max_iterations=3000,
                                    tolerance=1e-8, precision=nw.PREC_MIXED_BF16,
                                    preconditioner=nw.PC_LEARNED))
    x = torch.zeros(ls.sizes()[0], dtype=torch.float64, device="cuda")
    rep = ls.solve(x)
    assert rep.converged == 1 and not rep.fallback


def test_strength_aggregation_option(nw):
    """nw_learned_set_aggregation: aggregation over strong connections
    covers every row with more, smaller aggregates than plain aggregation
    on a stretched box, and the two-level cycle (two Jacobi sweeps on A_c
    as the coarse direction) still converges to 1e-8 with it."""
    import torch
    ls = _poisson(nw, (40, 36, 30), seed=21, stretch=1.12, jitter=0.05)
    sizes = {}
    for theta in (0.0, 0.08):
        net = nw.Learned(seed=0)
        net.set_aggregation(theta)
        net.set_coarse_direction(2)
        ls.attach_learned(net)
        g = ls.coarse_graph()
        agg, nc = g["agg"], g["nc"]
        assert agg.min() == 0 and agg.max() == nc - 1 and len(np.unique(agg)) == nc
        sizes[theta] = nc
        ls.set_solver_cfg(nw.solver_cfg(method=nw.FGMRES, kspace=30, inner_kspace=30, max_iterations=6000,
                                        tolerance=1e-8, precision=nw.PREC_MIXED, preconditioner=nw.PC_LEARNED))
        x = torch.zeros(ls.sizes()[0], dtype=torch.float64, device="cuda")
        rep = ls.solve(x)
        assert rep.converged == 1
    assert sizes[0.08] > sizes[0.0]
    with pytest.raises(nw.NwError):
        nw.Learned(seed=0).set_aggregation(1.5)
