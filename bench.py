"""Benchmark: GB300 edge assembly (+ Poisson solve) of the nalu-wind hot path.

Contract (one JSON line from rank 0):
  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
A step assembles the 128 x 128 x 64 stretched, jittered box (1,081,665
nodes, 3,211,584 edges): the 3-dof momentum system (MomentumEdgeSolverAlg,
67,543,497 nnz) and the continuity / pressure-Poisson system
(ContinuityEdgeSolverAlg, 7,504,833 nnz), each zeroed then assembled through
the C ABI. value = nnz assembled per second (Gnnz/s). Inputs are resident
in HBM for `value`; `e2e` copies every input field from pinned host memory
and reads both rhs vectors back inside the timed region.

The run also solves the pressure-Poisson system of the 256 x 256 x 128 box
(8,520,321 rows; --no-poisson skips it): ms to 1e-8 FP64 relative residual
for plain FP64 GMRES(50) + Jacobi, mixed-precision GMRES(50) + SGS, and the
learned-preconditioned mixed-precision FGMRES(30) (network trained first,
untimed, on other seeded systems). It then times one implicit step on a
perturbed 127^3-hex block split into tets (2,097,152 nodes), in random and
in RCM node order (--no-step skips it).

Multi-GPU (torchrun, N > 1): every rank runs an independent replica of the
same workload (weak scaling); the timed region is bracketed by barriers and
the max over ranks is reported. --impl reference times the CPU oracle (the
restated reference path, OpenMP on all host cores) on rank 0 only.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "nalu-wind_gb300"
MOMENTUM_NNZ = 67_543_497
CONTINUITY_NNZ = 7_504_833


def _package():
    if "nalu_wind_gb300" in sys.modules:
        return sys.modules["nalu_wind_gb300"]
    spec = importlib.util.spec_from_file_location(
        "nalu_wind_gb300", PKG / "__init__.py", submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["nalu_wind_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def algorithmic_bytes(kind: str, N: int, E: int, nnz: int) -> int:
    """Compulsory bytes of one assembly: inputs read once, outputs written
    once, 32-bit edge node ids; nnz is the 1-dof nnz (N + 2E)."""
    if kind == "continuity":
        return 32 * E + 96 * N + 8 * nnz + 8 * N
    if kind == "momentum":
        return 48 * E + 144 * N + 8 * 9 * nnz + 24 * N
    if kind == "scalar":
        return 40 * E + 96 * N + 8 * nnz + 8 * N
    raise ValueError(kind)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def stop(self) -> dict:
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


def traffic_table() -> dict:
    """DRAM bytes per launch measured by ncu (profiles/traffic.txt: one
    `key bytes` pair per line; the ncu command is in the matching summary)."""
    p = ROOT / "profiles" / "traffic.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) == 2:
                out[parts[0]] = {"bytes_per_launch": int(parts[1])}
    return out


def dist_setup(n_gpus: int):
    rank, world = 0, 1
    if n_gpus > 1 or "RANK" in os.environ:
        import torch.distributed as dist
        rank = int(os.environ.get("RANK", 0))
        world = int(os.environ.get("WORLD_SIZE", 1))
        if world > 1:
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = "nccl"
            try:
                import torch
                if not torch.cuda.is_available():
                    backend = "gloo"
            except Exception:
                backend = "gloo"
            dist.init_process_group(backend=backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
def build_inputs(nw, shape):
    return nw.workload.lowmach_case(*shape, seed=2)


def run_ours(args, rank, world):
    import torch

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    nw = _package()
    nw.load()
    nw.check(nw.load().nw_set_device(local))
    case = build_inputs(nw, args.shape)
    mesh = case.mesh
    N, E = mesh.num_nodes, mesh.num_edges
    stream = torch.cuda.current_stream()
    nd = case.node
    host = dict(coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
                density=nd["density"], mask=nd["mask"], pressure=nd["pressure"], dpdx=nd["dpdx"],
                udiag=nd["udiag"], area=mesh.area, mdot=case.edge["mdot"], pecfac=case.edge["pecfac"])
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in host.items()}
    pinned = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in host.items()}
    lsm = nw.LinearSystem(3, stream=stream.cuda_stream)
    lsm.build_edge_graph(N, mesh.edges)
    lsm.finalize()
    lsc = nw.LinearSystem(1, stream=stream.cuda_stream)
    lsc.build_edge_graph(N, mesh.edges)
    lsc.finalize()
    nnz_m = lsm.sizes()[1]
    nnz_c = lsc.sizes()[1]
    nnz1 = nnz_c
    mo, co = case.opts["momentum"], case.opts["continuity"]

    def fields(d):
        fm = nw.MomentumFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dudx", "viscosity", "density", "mask", "area", "mdot", "pecfac")))
        fc = nw.ContinuityFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dpdx", "density", "pressure", "udiag", "area")))
        return fm, fc

    fm, fc = fields(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    mom_ms, con_ms = [], []

    def step(timed_kernels=False):
        if timed_kernels:
            ev[0].record(stream)
        lsm.zero_system()
        lsm.assemble_momentum(fm, mo)
        if timed_kernels:
            ev[1].record(stream)
        lsc.zero_system()
        lsc.assemble_continuity(fc, co)
        if timed_kernels:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    # The K-step loop is repeated until the timed region lasts about 1.5 s,
    # so that the clock sampler sees the GPU under load; every repeat is
    # exactly K steps bracketed by a barrier and a synchronize.
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    reps = args.repeats or max(1, min(1000, int(np.ceil(1.5 / max(time.perf_counter() - t, 1e-4)))))
    sampler = ClockSampler(local)
    sampler.start()
    ms_total = 0.0
    torch.cuda.nvtx.range_push("assembly_timed")
    for _ in range(reps):
        barrier(world)
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(args.steps):
            step()
        t1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        ms_total += t0.elapsed_time(t1)
    torch.cuda.nvtx.range_pop()
    clocks = sampler.stop()
    # per-assembly kernel durations (separate pass, same stream)
    for _ in range(args.steps):
        step(timed_kernels=True)
        torch.cuda.synchronize()
        mom_ms.append(ev[0].elapsed_time(ev[1]))
        con_ms.append(ev[1].elapsed_time(ev[2]))
    # the single-kernel form of the momentum assembly (same bits; its edge
    # coefficients pass through a ring in L2), timed the same way
    lsm.set_assembly_path(nw.ASSEMBLY_SINGLE_KERNEL)
    fused_ms = []
    for i in range(max(3, args.steps) + 1):
        ev[0].record(stream)
        lsm.zero_system()
        lsm.assemble_momentum(fm, mo)
        ev[1].record(stream)
        torch.cuda.synchronize()
        if i:
            fused_ms.append(ev[0].elapsed_time(ev[1]))
    lsm.sync()
    lsm.set_assembly_path(nw.ASSEMBLY_TWO_KERNELS)
    f_avg = float(np.mean(fused_ms))
    ft = traffic_table().get("momentum_single_kernel_128x128x64")
    B_m0 = algorithmic_bytes("momentum", N, E, nnz_c)
    single = {"avg_ms": round(f_avg, 4), "frac": round(B_m0 / (f_avg * 1e-3) / 1e9 / peaks()["hbm_gbs"], 4),
              "traffic": (ft["bytes_per_launch"] if ft else None), "schedule": lsm.assembly_schedule()}
    # e2e: host inputs -> device -> assemble -> rhs back to host
    rhs_m_host = torch.empty(3 * (lsm.sizes()[0] // 3), dtype=torch.float64).pin_memory()
    rhs_c_host = torch.empty(lsc.sizes()[0], dtype=torch.float64).pin_memory()
    _, rm_dev, _, _ = lsm.device_arrays()
    _, rc_dev, _, _ = lsc.device_arrays()
    h2d = sum(int(t.numel() * t.element_size()) for t in pinned.values())
    d2h = int(rhs_m_host.numel() * 8 + rhs_c_host.numel() * 8)
    import ctypes

    # Within one step the copies overlap the compute on three streams (copy,
    # compute, read-back). The node fields of both systems go first, then
    # the per-edge inputs (area, mdot, pecfac) in edge chunks; as each chunk
    # arrives, the momentum edge phase runs over its edges, then the row
    # phase over the node rows whose incident edges are all done
    # (nw_assemble_momentum_rows_range, their rhs read back at once), then
    # the continuity edge phase over the same edges
    # (nw_assemble_continuity_edge_range); after the last chunk the
    # continuity row phase runs and its rhs is read back. Steps do not
    # overlap one another (a solver's next inputs depend on this step's
    # solve). (Node fields copied in slices ahead of each chunk, so that
    # the compute starts earlier, measured slower: three times as many
    # copies.)
    copy_s = torch.cuda.Stream()
    d2h_s = torch.cuda.Stream()
    # the continuity system assembles on its own stream, beside the momentum
    # kernels of the same chunk
    con_s = torch.cuda.Stream()
    lsc.set_stream(con_s.cuda_stream)
    edge_keys = ("area", "mdot", "pecfac")
    node_keys = [k for k in pinned if k not in edge_keys]
    n_chunks = 8
    bounds = [E * c // n_chunks for c in range(n_chunks + 1)]
    ecols = {k: (pinned[k].numel() // E) for k in edge_keys}
    # node rows complete after each chunk: every incident edge index below
    # the chunk's end (node rows are the nodes in index order here)
    maxinc = np.full(N, -1, np.int64)
    np.maximum.at(maxinc, mesh.edges[:, 0], np.arange(E))
    np.maximum.at(maxinc, mesh.edges[:, 1], np.arange(E))
    row_ready = [int(np.searchsorted(np.maximum.accumulate(maxinc), b)) for b in bounds[1:-1]] + [N]

    def e2e_step():
        copy_s.wait_stream(stream)
        chunk_ev = []
        with torch.cuda.stream(copy_s):
            for k in node_keys:
                dev[k].copy_(pinned[k], non_blocking=True)
            for a, b in zip(bounds[:-1], bounds[1:]):
                for k in edge_keys:
                    w = ecols[k]
                    dev[k].view(-1)[a * w:b * w].copy_(pinned[k].view(-1)[a * w:b * w], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy_s)
                chunk_ev.append(ev)
        lsm.zero_system()
        con_s.wait_stream(stream)
        lsc.zero_system()
        done = 0
        for (a, b), ev, r in zip(zip(bounds[:-1], bounds[1:]), chunk_ev, row_ready):
            stream.wait_event(ev)
            con_s.wait_event(ev)
            lsm.assemble_momentum_range(fm, mo, a, b)
            lsc.assemble_continuity_range(fc, co, a, b)
            if r > done:
                lsm.assemble_momentum_rows_range(mo, done, r)
                ev_mr = torch.cuda.Event()
                ev_mr.record(stream)
                d2h_s.wait_event(ev_mr)
                cudart_copy(rhs_m_host.data_ptr() + 24 * done, rm_dev + 24 * done, 24 * (r - done),
                            d2h_s.cuda_stream)
                done = r
        lsc.assemble_continuity_rows()
        ev_cr = torch.cuda.Event()
        ev_cr.record(con_s)
        d2h_s.wait_event(ev_cr)
        cudart_copy(rhs_c_host.data_ptr(), rc_dev, rhs_c_host.numel() * 8, d2h_s.cuda_stream)
        stream.wait_stream(d2h_s)

    libcudart = _cudart()

    def cudart_copy(dst, src, nbytes, s):
        r = libcudart.cudaMemcpyAsync(ctypes.c_void_p(dst), ctypes.c_void_p(src), ctypes.c_size_t(nbytes),
                                      ctypes.c_int(2), ctypes.c_void_p(s))
        if r != 0:
            raise RuntimeError(f"cudaMemcpyAsync failed {r}")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    t0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    t1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms_e2e = t0.elapsed_time(t1)
    # the streamed step's rhs read-backs are the assembled systems' rhs
    if not (np.array_equal(rhs_m_host.numpy(), lsm.to_host()[1])
            and np.array_equal(rhs_c_host.numpy(), lsc.to_host()[1])):
        raise RuntimeError("end-to-end rhs differs from the assembled rhs")
    ms_total = max_over_ranks(ms_total, world)
    ms_e2e = max_over_ranks(ms_e2e, world)
    nnz_step = nnz_m + nnz_c
    value = world * nnz_step * args.steps * reps / (ms_total * 1e-3) / 1e9
    e2e = world * nnz_step * args.steps / (ms_e2e * 1e-3) / 1e9
    pk = peaks()
    B_m = algorithmic_bytes("momentum", N, E, nnz1)
    B_c = algorithmic_bytes("continuity", N, E, nnz1)
    mom_avg = float(np.mean(mom_ms))
    con_avg = float(np.mean(con_ms))
    achieved = B_m / (mom_avg * 1e-3) / 1e9
    tt = traffic_table().get("momentum_128x128x64")
    out = {
        "metric": "edge-assembly Gnnz/s", "value": round(value, 4), "unit": "Gnnz/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "repeats": reps,
        "timed_s": round(ms_total * 1e-3, 3), "ms_per_step": round(ms_total / (args.steps * reps), 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 128x128x64 stretched, jittered hex box; log-law velocity + noise)",
        "config": {"workload": "lowmach 128x128x64: momentum (3-dof) + continuity edge assembly",
                   "nodes": N, "edges": E, "nnz_momentum": nnz_m, "nnz_continuity": nnz_c,
                   "l2": "inputs and outputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e, 4), "unit": "Gnnz/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"kernel": "momentum assembly (edge + row kernels)", "bound": "hbm",
                     "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / pk["hbm_gbs"], 4), "peak_src": pk["src"],
                     "algorithmic_bytes": B_m, "avg_ms": round(mom_avg, 4),
                     "traffic": (tt["bytes_per_launch"] if tt else None)},
        "continuity": {"avg_ms": round(con_avg, 4), "algorithmic_bytes": B_c,
                       "achieved_gbs": round(B_c / (con_avg * 1e-3) / 1e9, 1),
                       "frac": round(B_c / (con_avg * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
                       "gnnz_s": round(nnz_c / (con_avg * 1e-3) / 1e9, 4)},
        "momentum": {"avg_ms": round(mom_avg, 4), "gnnz_s": round(nnz_m / (mom_avg * 1e-3) / 1e9, 4),
                     "single_kernel": single},
        # momentum: edge + row kernels; continuity: node + edge + row kernels
        "gpu_launches": 5 * args.steps * reps,
        "clocks": clocks,
    }
    poisson_csr = None
    if not args.no_poisson:
        out["poisson"] = poisson_solves(nw, stream, args)
        poisson_csr = out["poisson"].pop("_csr", None)
        net = out["poisson"].pop("_net")
        net_run = out["poisson"].pop("_net_run")
        if args.heldout > 0:
            out["poisson_heldout_128"] = heldout_poisson(nw, stream, args, net, net_run)
    if not args.no_step:
        out["implicit_step_tets"] = implicit_step(nw, stream, args)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(case, args, poisson_csr=poisson_csr)
    return out


def _cudart():
    import ctypes
    import torch
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    lib_dir = Path(torch.__file__).parent / "lib"
    for p in sorted(lib_dir.glob("libcudart*.so*")):
        return ctypes.CDLL(str(p))
    import glob
    for p in glob.glob(str(Path(sys.prefix) / "lib/python3*/site-packages/nvidia/cuda_runtime/lib/libcudart.so*")):
        return ctypes.CDLL(p)
    raise RuntimeError("libcudart not found")


def fp64_gmres_bytes(n, nnz, iterations, m) -> int:
    """Algorithmic bytes of right-preconditioned FP64 Jacobi-GMRES(m) with
    two-pass classical Gram-Schmidt: per iteration j of a restart cycle the
    SpMV (values, 32-bit columns and row offsets, x read, y written), the
    Jacobi scaling, 2 x (dots over j + 1 basis vectors and w, update of w by
    them) and the norm and scaling of the new vector."""
    total = 0
    for it in range(iterations):
        j = it % m
        total += 12 * nnz + 4 * (n + 1) + 16 * n + 24 * n + 2 * (8 * n * (j + 2) + 8 * n * (j + 3)) + 24 * n
    return total


def poisson_solves(nw, stream, args) -> dict:
    """Pressure Poisson to 1e-8 FP64 relative residual on the 256 x 256 x 128
    stretched box: plain FP64 GMRES(50) + Jacobi against the mixed-precision
    solvers, the headline being learned-preconditioned mixed FGMRES(30).
    The network is the one of the 128^3-node training set (weights file
    made by nalu-wind_gb300/train_poisson.py); a second network is trained
    in the run (untimed) on a family of 64 x 64 x 48 systems with other
    seeds, and both are reported. Every solve starts from x = 0. Errors are
    measured against an FP64 reference solution (FP64 GMRES(50) + SGS to
    1e-11; zero-mean parts: the system is singular, its null space the
    constants). The mixed SGS solver is also run to 1e-10, the refinement
    target of the mixed-precision configuration."""
    import torch
    ls = nw.workload.poisson_system(args.poisson_shape, seed=3, stretch=1.04, stream=stream.cuda_stream)
    nr, nnz = ls.sizes()
    res = {"workload": f"pressure Poisson {'x'.join(map(str, args.poisson_shape))} box, stretch 1.04",
           "rows": nr, "nnz": nnz, "tol": 1e-8,
           "mixed_precision": "FP64 outer residual / refinement; FP32 inner Krylov, SpMV and network "
                              "coarse step; BF16 Gauss-Seidel matrix values with FP32 accumulation"}
    # the networks are only needed when a learned variant runs
    need_net = (not args.poisson_variants or args.heldout > 0
                or any("learned" in v or "two_level" in v for v in args.poisson_variants.split(",")))
    if not need_net:
        net_run, info = None, None
    else:
        net_run, info = nw.training.train_poisson_network(epochs=args.train_epochs, lr=args.train_lr,
                                                          stream=stream.cuda_stream)
    res["training_in_run"] = info
    # the network of the 128^3-node training set (nalu-wind_gb300/
    # train_poisson.py), trained once and loaded here; without its weights
    # file the in-run network takes its place
    net = net_run
    wpath = Path(args.weights) if args.weights else None
    if need_net and wpath is not None and wpath.exists():
        net, recipe = nw.training.load_poisson_network(wpath)
        res["training"] = dict(recipe, weights=str(wpath.relative_to(ROOT) if wpath.is_relative_to(ROOT)
                                                   else wpath))
    elif need_net:
        res["training"] = dict(info, weights=None)
    res["_net"] = net
    res["_net_run"] = net_run if net is not net_run else None
    controls = learned_controls(nw)
    maxit = args.poisson_maxit
    variants = [
        ("plain_fp64_gmres50_jacobi", None,
         nw.solver_cfg(kspace=50, max_iterations=maxit, tolerance=1e-8)),
        ("mixed_gmres50_sgs", None,
         nw.solver_cfg(kspace=50, max_iterations=maxit, tolerance=1e-8, precision=nw.PREC_MIXED_BF16,
                       inner_kspace=50, inner_tolerance=1e-4, preconditioner=nw.PC_SGS)),
        *[(f"mixed_fgmres30_two_level_{cname}", cnet,
           nw.solver_cfg(method=nw.FGMRES, kspace=30, max_iterations=maxit, tolerance=1e-8,
                         precision=nw.PREC_MIXED_BF16, inner_kspace=30, preconditioner=nw.PC_LEARNED))
          for cname, cnet in controls.items()],
        ("learned_mixed_fgmres30", net,
         nw.solver_cfg(method=nw.FGMRES, kspace=30, max_iterations=maxit, tolerance=1e-8,
                       precision=nw.PREC_MIXED_BF16, inner_kspace=30, preconditioner=nw.PC_LEARNED)),
    ]
    if net is not net_run:
        variants.append(("learned_mixed_fgmres30_in_run_network", net_run,
                         nw.solver_cfg(method=nw.FGMRES, kspace=30, max_iterations=maxit, tolerance=1e-8,
                                       precision=nw.PREC_MIXED_BF16, inner_kspace=30,
                                       preconditioner=nw.PC_LEARNED)))
    variants.append(("mixed_gmres50_sgs_to_1e-10", None,
                     nw.solver_cfg(kspace=50, max_iterations=maxit, tolerance=1e-10,
                                   precision=nw.PREC_MIXED_BF16, inner_kspace=50, inner_tolerance=1e-4,
                                   preconditioner=nw.PC_SGS)))
    if args.poisson_variants:
        keep = set(args.poisson_variants.split(","))
        variants = [v for v in variants if v[0] in keep]
    x_ref = None
    if not args.poisson_variants:
        ls.set_solver_cfg(nw.solver_cfg(kspace=50, max_iterations=maxit, tolerance=1e-11,
                                        preconditioner=nw.PC_SGS))
        xr = torch.zeros(nr, dtype=torch.float64, device="cuda")
        rep = ls.solve(xr)
        res["fp64_reference_gmres50_sgs_to_1e-11"] = {
            "ms": round(rep.solve_ms, 2), "iterations": rep.iterations,
            "rel_residual_fp64": rep.final_abs_residual / rep.rhs_norm, "converged": bool(rep.converged)}
        x_ref = xr - xr.mean()
    for name, learned, cfg in variants:
        if learned is not None:
            ls.attach_learned(learned)
        ls.set_solver_cfg(cfg)
        x = torch.zeros(nr, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(name)  # NVTX range: profilers can select one solve
        t = time.perf_counter()
        rep = ls.solve(x)
        wall = (time.perf_counter() - t) * 1e3
        torch.cuda.nvtx.range_pop()
        r = {"ms": round(rep.solve_ms, 2), "wall_ms": round(wall, 2), "iterations": rep.iterations,
             "outer": rep.outer_iterations, "rel_residual_fp64": rep.final_abs_residual / rep.rhs_norm,
             "converged": bool(rep.converged), "fallback": bool(rep.fallback)}
        if x_ref is not None:
            xc = x - x.mean()
            r["rel_error_vs_fp64_reference"] = float(torch.linalg.norm(xc - x_ref) / torch.linalg.norm(x_ref))
        if name == "plain_fp64_gmres50_jacobi":
            if not args.no_cpu_baseline:
                rp_h, ci_h = ls.graph()
                vals_h, rhs_h = ls.to_host()
                res["_csr"] = (rp_h, ci_h, vals_h, rhs_h, rep.iterations)
            gb = fp64_gmres_bytes(nr, nnz, rep.iterations, 50) / 1e9
            pk = peaks()["hbm_gbs"]
            r["solver_phase"] = {"algorithmic_gb": round(gb, 2),
                                 "achieved_gbs": round(gb / (rep.solve_ms * 1e-3), 1),
                                 "frac_of_hbm": round(gb / (rep.solve_ms * 1e-3) / pk, 4),
                                 "formula": "per iteration j of a cycle: SpMV 12 nnz + 4 (N+1) + 16 N, "
                                            "Jacobi 24 N, two-pass CGS 2 (8 N (j+2) + 8 N (j+3)), "
                                            "norm/scale 24 N"}
        res[name] = r
    if "plain_fp64_gmres50_jacobi" in res:
        base = res["plain_fp64_gmres50_jacobi"]["ms"]
        for name, key in (("learned_mixed_fgmres30", "speedup_learned_mixed_vs_plain_fp64"),
                          ("mixed_gmres50_sgs", "speedup_mixed_sgs_vs_plain_fp64")):
            if name in res:
                res[key] = round(base / res[name]["ms"], 2)
    return res


def learned_controls(nw) -> dict:
    """The learned preconditioner's cycle without the trained network, to
    measure what training adds: the same network untrained (random
    initialisation, seed 0), the non-learned coarse directions D_c^-1 r_c and
    two Jacobi sweeps on the Galerkin operator (each with the same
    energy-optimal scaling), and no coarse correction (output layer zeroed:
    the two Gauss-Seidel sweeps alone)."""
    untrained = nw.Learned(seed=0)
    jac1 = nw.Learned(seed=0)
    jac1.set_coarse_direction(1)
    jac2 = nw.Learned(seed=0)
    jac2.set_coarse_direction(2)
    none = nw.Learned(seed=0)
    p0 = none.params()
    p0[-64:] = 0.0
    none.set_params(p0)
    return {"untrained_network": untrained, "jacobi_coarse_direction": jac1, "two_jacobi_coarse_sweeps": jac2,
            "no_coarse_correction": none}


def heldout_poisson(nw, stream, args, net, net_run=None) -> dict:
    """The learned preconditioner on held-out seeds of the training family's
    distribution at 128^3 nodes (127^3 hexes; stretch ratio from U[1.0, 1.15],
    interior jitter from U[0, 10 %], seeds 1000 + k): learned mixed FGMRES(30)
    against plain FP64 Jacobi-GMRES(30), both to 1e-8 FP64-verified (plain
    capped at --poisson-maxit iterations)."""
    import torch
    rng = np.random.default_rng(1000)
    out = {"workload": "held-out 128^3-node Poisson systems", "systems": []}
    controls = learned_controls(nw)
    for k in range(args.heldout):
        stretch, jitter = float(rng.uniform(1.0, 1.15)), float(rng.uniform(0.0, 0.1))
        ls = nw.workload.poisson_system((127, 127, 127), seed=1000 + k, stretch=stretch, jitter=jitter,
                                        stream=stream.cuda_stream)
        nr = ls.sizes()[0]
        r = {"seed": 1000 + k, "stretch": round(stretch, 4), "jitter": round(jitter, 4)}
        lcfg = nw.solver_cfg(method=nw.FGMRES, kspace=30, inner_kspace=30, max_iterations=args.poisson_maxit,
                             tolerance=1e-8, precision=nw.PREC_MIXED_BF16, preconditioner=nw.PC_LEARNED)
        runs = [("plain_fp64_gmres30_jacobi", None, nw.solver_cfg(kspace=30, max_iterations=args.poisson_maxit,
                                                                   tolerance=1e-8)),
                ("learned_mixed_fgmres30", net, lcfg)]
        if net_run is not None:
            runs.append(("learned_mixed_fgmres30_in_run_network", net_run, lcfg))
        runs += [(f"mixed_fgmres30_two_level_{c}", cn, lcfg) for c, cn in controls.items()
                 if c in ("untrained_network", "jacobi_coarse_direction")]
        # the same non-learned cycle on aggregates of strong connections
        strong = nw.Learned(seed=0)
        strong.set_aggregation(0.08)
        strong.set_coarse_direction(2)
        runs.append(("mixed_fgmres30_two_level_two_jacobi_coarse_sweeps_strength_aggregation_0.08", strong, lcfg))
        for name, lnet, cfg in runs:
            if lnet is not None:
                ls.attach_learned(lnet)
            ls.set_solver_cfg(cfg)
            x = torch.zeros(nr, dtype=torch.float64, device="cuda")
            rep = ls.solve(x)
            r[name] = {"ms": round(rep.solve_ms, 2), "iterations": rep.iterations,
                       "rel_residual_fp64": rep.final_abs_residual / rep.rhs_norm,
                       "converged": bool(rep.converged), "fallback": bool(rep.fallback)}
        out["systems"].append(r)
        del ls
    return out


def implicit_step(nw, stream, args) -> dict:
    """One implicit step on an unstructured mesh: a perturbed block of n^3
    hexes (n = 127: 2,097,152 nodes) split into 6 tets each, node ids
    randomly permuted, then that order RCM-renumbered; both orderings timed.
    The step is the input producers (mass flow rate, open-boundary mass
    flow rate, nodal gradients of u and p, Peclet factor), the momentum
    (3-dof) and continuity edge assembly, the boundary face kernels (an open
    boundary on the x+ side for both systems, symmetry on the y and z sides
    for momentum), then the continuity (pressure-Poisson) system solved to
    1e-8 FP64 relative residual by learned mixed FGMRES(30) and by plain FP64
    GMRES(50) + Jacobi. The network is trained first (untimed) on small tet
    systems."""
    import torch
    n = args.step_n
    res = {"workload": f"{n}^3-hex block, 6 tets per hex, 5 % jitter; random and RCM node orders",
           "step": "producers (edge area vectors and dual volumes, mdot, open mdot, grad u, grad p, Peclet "
                   "factor) + momentum and continuity assembly + open (x+) and symmetry (y, z sides) "
                   "boundary kernels + continuity solve to 1e-8"}

    def dev_t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()
    net, info = nw.training.train_poisson_network(shape=(40, 40, 40), tets=True, systems=8, restarts=40,
                                                  epochs=100, stream=stream.cuda_stream)
    res["training"] = info
    for name, ren in (("random", 1), ("rcm", 2)):
        case = nw.workload.lowmach_case(n, n, n, seed=5, stretch=1.0, jitter=0.05, lz=1.0, tets=True,
                                        renumber=ren, renumber_seed=7)
        mesh = case.mesh
        nd = case.node
        d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in dict(
            coords=mesh.coords, velocity=nd["velocity"], dudx=nd["dudx"], viscosity=nd["viscosity"],
            density=nd["density"], mask=nd["mask"], pressure=nd["pressure"], dpdx=nd["dpdx"],
            udiag=nd["udiag"], area=mesh.area, mdot=case.edge["mdot"], pecfac=case.edge["pecfac"]).items()}
        fm = nw.MomentumFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dudx", "viscosity", "density", "mask", "area", "mdot", "pecfac")))
        fc = nw.ContinuityFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dpdx", "density", "pressure", "udiag", "area")))
        lsm = nw.LinearSystem(3, stream=stream.cuda_stream)
        lsm.build_edge_graph(mesh.num_nodes, mesh.edges)
        lsm.finalize()
        lsc = nw.LinearSystem(1, stream=stream.cuda_stream)
        lsc.build_edge_graph(mesh.num_nodes, mesh.edges)
        lsc.finalize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        mo, co = case.opts["momentum"], case.opts["continuity"]
        # boundaries: open on x+, symmetry on the y and z sides
        ipn_o, area_o = mesh.face_ips(("x+",))
        ipn_s, area_s = mesh.face_ips(("y-", "y+", "z-", "z+"))
        ss_oc, ss_om, ss_s = lsc.sideset(ipn_o), lsm.sideset(ipn_o), lsm.sideset(ipn_s)
        bd = {"area_o": dev_t(area_o), "area_s": dev_t(area_s), "pbc": dev_t(np.zeros(mesh.num_nodes)),
              "omdot": torch.zeros(len(ipn_o), dtype=torch.float64, device="cuda")}
        fco = nw.ContinuityOpenFields(*(d[k].data_ptr() for k in (
            "coords", "velocity", "dpdx", "density", "pressure")), bd["pbc"].data_ptr(), d["udiag"].data_ptr(),
            bd["area_o"].data_ptr(), None)
        fmo = nw.MomentumOpenFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dudx", "viscosity")),
                                    d["velocity"].data_ptr(), bd["area_o"].data_ptr(), bd["omdot"].data_ptr())
        fms = nw.MomentumSymmetryFields(*(d[k].data_ptr() for k in ("coords", "velocity", "dudx", "viscosity")),
                                        bd["area_s"].data_ptr())
        oco = nw.ContinuityOpenOpts(tau_scale=co.tau_scale, noc_fac=co.noc_fac, pstab_fac=1.0, mdot_corr=0.0,
                                    solve_incompressible=co.solve_incompressible)
        omo = nw.MomentumOpenOpts(include_div_u=mo.include_div_u, nf_entrain=0.0, entrainment=nw.ENTRAIN_COMPUTED)
        osy = nw.MomentumSymmetryOpts(include_div_u=mo.include_div_u, penalty_factor=0.0)
        # input producers: edge area vectors and dual volumes (as after a
        # mesh motion), mdot, nodal gradients of u and p, Peclet factor
        dv, ba = dev_t(mesh.dualvol), dev_t(mesh.bnd_area)
        pec_o = nw.PecletOpts(0, 1.0, 2.0, 4.0, 1e-16)
        geo = nw.Geometry(mesh.num_nodes, mesh.conn, mesh.edges, mesh.nalu_id)

        def producers():
            geo.compute(d["coords"], d["area"], dv, stream.cuda_stream)
            ev[5].record(stream)
            lsc.compute_mdot(fc, d["mdot"], noc_fac=co.noc_fac, interp_together=co.interp_together)
            lsc.open_mdot(ss_oc, fco, bd["omdot"], noc_fac=co.noc_fac, pstab_fac=1.0)
            lsc.nodal_gradient(d["velocity"], d["area"], dv, d["dudx"], bnd_area_dev=ba, dim1=3)
            lsc.nodal_gradient(d["pressure"], d["area"], dv, d["dpdx"], bnd_area_dev=ba, dim1=1)
            lsc.peclet_factor(d["coords"], d["density"], d["viscosity"], d["velocity"], d["pecfac"], opts=pec_o)

        prod, mom, con, bnd, geom = [], [], [], [], []
        for it in range(5):
            ev[0].record(stream)
            producers()
            ev[1].record(stream)
            lsm.zero_system()
            lsm.assemble_momentum(fm, mo)
            ev[2].record(stream)
            lsc.zero_system()
            lsc.assemble_continuity(fc, co)
            ev[3].record(stream)
            lsm.assemble_momentum_open(ss_om, fmo, omo)
            lsm.assemble_momentum_symmetry(ss_s, fms, osy)
            lsc.assemble_continuity_open(ss_oc, fco, oco)
            ev[4].record(stream)
            torch.cuda.synchronize()
            if it >= 2:
                prod.append(ev[0].elapsed_time(ev[1]))
                geom.append(ev[0].elapsed_time(ev[5]))
                mom.append(ev[1].elapsed_time(ev[2]))
                con.append(ev[2].elapsed_time(ev[3]))
                bnd.append(ev[3].elapsed_time(ev[4]))
        nnz_m, nnz_c = lsm.sizes()[1], lsc.sizes()[1]
        r = {"nodes": mesh.num_nodes, "edges": mesh.num_edges, "nnz_momentum": nnz_m, "nnz_continuity": nnz_c,
             "face_ips_open": len(ipn_o), "face_ips_symmetry": len(ipn_s),
             "producers_ms": round(float(np.mean(prod)), 4),
             "geometry_ms": round(float(np.mean(geom)), 4),
             "momentum_ms": round(float(np.mean(mom)), 4), "continuity_ms": round(float(np.mean(con)), 4),
             "boundary_ms": round(float(np.mean(bnd)), 4)}
        r["assembly_gnnz_s"] = round((nnz_m + nnz_c) / ((r["momentum_ms"] + r["continuity_ms"]) * 1e-3) / 1e9, 3)
        nr = lsc.sizes()[0]
        for vname, learned, cfg in (
                ("plain_fp64_gmres50_jacobi", None,
                 nw.solver_cfg(kspace=50, max_iterations=args.poisson_maxit, tolerance=1e-8)),
                ("learned_mixed_fgmres30", net,
                 nw.solver_cfg(method=nw.FGMRES, kspace=30, max_iterations=args.poisson_maxit, tolerance=1e-8,
                               precision=nw.PREC_MIXED_BF16, inner_kspace=30, preconditioner=nw.PC_LEARNED))):
            if learned is not None:
                lsc.attach_learned(learned)
            lsc.set_solver_cfg(cfg)
            x = torch.zeros(nr, dtype=torch.float64, device="cuda")
            rep = lsc.solve(x)
            r[vname] = {"ms": round(rep.solve_ms, 2), "iterations": rep.iterations,
                        "rel_residual_fp64": rep.final_abs_residual / rep.rhs_norm,
                        "converged": bool(rep.converged), "fallback": bool(rep.fallback)}
        asm = r["producers_ms"] + r["momentum_ms"] + r["continuity_ms"] + r["boundary_ms"]
        r["step_ms_learned_mixed"] = round(asm + r["learned_mixed_fgmres30"]["ms"], 2)
        r["step_ms_plain_fp64"] = round(asm + r["plain_fp64_gmres50_jacobi"]["ms"], 2)
        res[name] = r
        del ss_oc, ss_om, ss_s, geo
        del lsm, lsc, d
        torch.cuda.empty_cache()
    return res


def one_assembly(orc, case, omo, oco, g1, g3, threads):
    """One full momentum + continuity assembly by the oracle: per-edge local
    systems, then TpetraLinearSystem::sum_into with OpenMP atomics."""
    mesh, nd = case.mesh, case.node
    rp1, ci1, lid1 = g1
    rp3, ci3, lid3 = g3
    lhs, rhs = orc.momentum_local(mesh.edges, mesh.coords, nd["velocity"], nd["velocity"], nd["dudx"],
                                  nd["viscosity"], nd["density"], nd["mask"], mesh.area, case.edge["mdot"],
                                  case.edge["pecfac"], omo)
    orc.sum_into(mesh.edges, 3, lhs, rhs, lid3, rp3, ci3, nthreads=threads, with_abs=False)
    lhs, rhs = orc.continuity_local(mesh.edges, mesh.coords, nd["velocity"], nd["dpdx"], nd["density"],
                                    nd["pressure"], nd["udiag"], mesh.area, oco)
    orc.sum_into(mesh.edges, 1, lhs, rhs, lid1, rp1, ci1, nthreads=threads, with_abs=False)


def cpu_baseline(case, args, steps=None, poisson_csr=None, warmup=0) -> dict:
    """Oracle (restated reference path) on the host cores: per-edge kernels
    plus the atomic sum_into, OpenMP on all cores, FP64. steps=None: as many
    full assemblies as fit in about 10 s (at least 3), plus one run on one
    thread; otherwise `warmup` untimed then exactly `steps` timed assemblies.
    With poisson_csr (row_ptr, col_idx, values, rhs, GPU iteration count), a
    bounded sample of the FP64 Poisson solve."""
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob
    ob.build()
    from oracle import oracle as orc
    mesh = case.mesh
    nd = case.node
    threads = os.cpu_count() or 1
    rp1, ci1, lid1 = orc.build_graph(mesh.nalu_id, mesh.edges, 1)
    rp3, ci3, lid3 = orc.build_graph(mesh.nalu_id, mesh.edges, 3)
    mo, co = case.opts["momentum"], case.opts["continuity"]
    omo = orc.MomentumOpts(*(getattr(mo, k) for k, _ in mo._fields_))
    oco = orc.ContinuityOpts(*(getattr(co, k) for k, _ in co._fields_))
    for _ in range(warmup):
        one_assembly(orc, case, omo, oco, (rp1, ci1, lid1), (rp3, ci3, lid3), threads)
    times = []
    target = steps
    k = 0
    while True:
        t = time.perf_counter()
        one_assembly(orc, case, omo, oco, (rp1, ci1, lid1), (rp3, ci3, lid3), threads)
        times.append(time.perf_counter() - t)
        k += 1
        if target is None:
            target = int(min(40, max(3, 10.0 / max(times[0], 1e-3))))
        if k >= target:
            break
    nnz = int(ci3.shape[0] + ci1.shape[0])
    sec = float(np.mean(times))
    out = {"value": round(nnz / sec / 1e9, 5), "unit": "Gnnz/s", "cores": threads, "kind": "port",
           "sample": f"full momentum + continuity assemblies of the same workload ({nnz} nnz): "
                     f"{k} runs, mean {sec:.3f} s"}
    if steps is None:
        # the same assembly on one thread (one run)
        orc.set_threads(1)
        t = time.perf_counter()
        one_assembly(orc, case, omo, oco, (rp1, ci1, lid1), (rp3, ci3, lid3), 1)
        s1 = time.perf_counter() - t
        orc.set_threads(threads)
        out["one_thread"] = {"value": round(nnz / s1 / 1e9, 5), "unit": "Gnnz/s", "sample": f"1 run, {s1:.3f} s"}
    if poisson_csr is not None:
        # FP64 GMRES(50) + Jacobi on the Poisson system, a bounded number of
        # iterations on all cores; the full solve's time is projected from
        # the iteration count the same algorithm needs on the GPU
        rp, ci, vals, rhs, its_full = poisson_csr
        n_it = 20
        t = time.perf_counter()
        _, _, rep = orc.solve(rp, ci, vals, rhs, method=0, precond=1, kspace=50, max_iters=n_it, tol=1e-30,
                              nthreads=threads)
        s_it = (time.perf_counter() - t) / max(rep.iterations, 1)
        out["poisson_fp64_gmres50_jacobi"] = {
            "ms_per_iteration": round(s_it * 1e3, 2), "cores": threads,
            "sample": f"{rep.iterations} iterations of the 8.5M-row solve",
            "projected_ms_to_1e-8": round(s_it * 1e3 * its_full, 1) if its_full else None}
    return out


def oracle_inputs(shape):
    """The assembly workload rebuilt by the oracle alone (oracle/cases.py),
    so that the reference arm never loads the product library."""
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob
    ob.build()
    from oracle import cases
    return cases.lowmach_case(*shape, seed=2)


def run_reference(args, rank, world):
    """The restated reference path (CPU oracle, OpenMP on all host cores) on
    the same workload, with the --steps and --warmup it is given: each step is
    one full momentum + continuity assembly."""
    if rank != 0:
        return None
    case = oracle_inputs(args.shape)
    steps = max(1, args.steps)
    cb = cpu_baseline(case, args, steps=steps, warmup=args.warmup)
    return {"metric": "edge-assembly Gnnz/s", "value": cb["value"], "unit": "Gnnz/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (same seeded workload, rebuilt by the oracle)",
            "config": {"workload": "lowmach 128x128x64: momentum (3-dof) + continuity edge assembly",
                       "note": "CPU oracle restating the reference path; the reference build needs "
                               "Trilinos/STK/Kokkos/MPI, absent here"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "Gnnz/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--repeats", type=int, default=0,
                    help="repeats of the timed K-step loop (0: enough for about 1.5 s)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shape", type=int, nargs=3, default=[128, 128, 64])
    ap.add_argument("--no-poisson", action="store_true", help="skip the Poisson solves")
    ap.add_argument("--poisson-shape", type=int, nargs=3, default=[256, 256, 128])
    ap.add_argument("--poisson-maxit", type=int, default=20000)
    ap.add_argument("--poisson-variants", default="", help="comma-separated subset of the solver variants")
    ap.add_argument("--no-step", action="store_true", help="skip the implicit step on the tet mesh")
    ap.add_argument("--heldout", type=int, default=2, help="held-out 128^3 Poisson systems to solve")
    ap.add_argument("--step-n", type=int, default=127, help="hexes per side of the tet-mesh block")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--train-epochs", type=int, default=100, help="training epochs of the Poisson network")
    ap.add_argument("--train-lr", type=float, default=1e-3, help="Adam learning rate of the Poisson network")
    ap.add_argument("--weights", default=str(PKG / "weights" / "poisson_128cube.nwl"),
                    help="weights of the 128^3-node recipe (train_poisson.py); '' trains in the run only")
    args = ap.parse_args()
    args.shape = tuple(args.shape)
    args.poisson_shape = tuple(args.poisson_shape)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank, world = dist_setup(args.gpus)
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        sys.path.insert(0, str(ROOT))
        import __graft_entry__ as ge
        ge.build()
        out = run_ours(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
