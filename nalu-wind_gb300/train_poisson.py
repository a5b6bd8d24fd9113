"""Train the learned Poisson preconditioner and save its weights.

Usage (repository root, on a GPU):
    python nalu-wind_gb300/train_poisson.py [--systems 200] [--restarts 100]
        [--shape 127 127 127] [--epochs 4] [--out nalu-wind_gb300/weights/poisson_128cube.nwl]

The default recipe is the 128^3-node training set: 200 seeded pressure-
Poisson boxes of 127^3 hexes (128^3 nodes), z-stretching ratio drawn from
U[1.0, 1.15] and coordinate jitter from U[0, 10 %] of the local spacing
(seeds 100, 101, ...), up to `restarts` (residual, error) pairs per system
from restarted FP64 Jacobi-GMRES(30) (nw_learned_harvest), then Adam on the
GPU by the library's own forward and backward kernels. The weights go to
--out (checksummed binary, nw_learned_save) and the recipe with the losses
and timings to the same path with the suffix .json.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import sys
import time
from pathlib import Path

PKG = Path(__file__).resolve().parent


def _package():
    if "nalu_wind_gb300" in sys.modules:
        return sys.modules["nalu_wind_gb300"]
    spec = importlib.util.spec_from_file_location(
        "nalu_wind_gb300", PKG / "__init__.py", submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["nalu_wind_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--systems", type=int, default=200)
    ap.add_argument("--restarts", type=int, default=100)
    ap.add_argument("--shape", type=int, nargs=3, default=(127, 127, 127))
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=str(PKG / "weights" / "poisson_128cube.nwl"))
    a = ap.parse_args(argv)
    nw = _package()
    nw.load()
    import torch
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    t = time.perf_counter()
    net, info = nw.training.train_poisson_network(
        shape=tuple(a.shape), systems=a.systems, restarts=a.restarts, epochs=a.epochs, batch=a.batch,
        lr=a.lr, seed=a.seed, stream=stream.cuda_stream)
    info.update(restarts=a.restarts, batch=a.batch, lr=a.lr, seed=a.seed,
                stretch="U[1.0, 1.15]", jitter="U[0, 0.1]", seeds=f"100..{99 + a.systems}",
                wall_s=round(time.perf_counter() - t, 1))
    out = Path(a.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    net.save(out)
    out.with_suffix(".json").write_text(json.dumps(info, indent=1) + "\n")
    print(json.dumps(info))
    return info


if __name__ == "__main__":
    main()
