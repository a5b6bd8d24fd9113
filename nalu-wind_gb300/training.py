"""Training recipe of the learned Poisson preconditioner.

A family of seeded pressure-Poisson systems on one box shape (stretching
ratio drawn from U[1.0, 1.15], interior coordinate jitter from U[0, 10%]
of the local spacing) supplies (residual, error) pairs harvested at the
restarts of plain FP64 Jacobi-GMRES(30); the network is then trained on
the GPU (Adam, mini-batches of pairs) by the library's own forward and
backward kernels. The systems use seeds 100, 101, ...; the solves it is
meant for use other seeds.
"""
from __future__ import annotations

import time

import numpy as np

from . import Learned, NwError
from .workload import poisson_system


def train_poisson_network(shape=(64, 64, 48), systems=16, restarts=40, kspace=30, epochs=100,
                          batch=8, lr=1e-3, seed=0, agg_passes=2, stream=None, tets=False, smoother=0):
    """Returns (network, info). info: pairs, harvest / train seconds and
    the mean energy-norm loss over the pairs before and after training."""
    net = Learned(seed=seed)
    net.configure(post_smooth=True, agg_passes=agg_passes, smoother=smoother)
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    first = None
    pairs = 0
    skipped = []
    for k in range(systems):
        stretch, jitter = float(rng.uniform(1.0, 1.15)), float(rng.uniform(0.0, 0.1))
        ls = poisson_system(shape, seed=100 + k, stretch=stretch, jitter=jitter, stream=stream, tets=tets)
        ls.attach_learned(net)
        try:
            pairs = net.harvest(ls, restarts=restarts, kspace=kspace)
        except NwError as err:
            # a system whose FP64 reference solve cannot get below 1e-6
            # (the most stretched draws at 128^3 nodes) gives no pairs
            if err.status != 5:  # NW_NOT_CONVERGED
                raise
            skipped.append({"seed": 100 + k, "stretch": round(stretch, 4)})
            continue
        if first is None:
            first = ls
    t1 = time.perf_counter()
    before = net.evaluate(first)
    net.train(first, epochs=epochs, batch=batch, lr=lr, seed=seed)
    after = net.evaluate(first)
    t2 = time.perf_counter()
    net.clear_data()
    info = {"systems": systems, "shape": list(shape), "tets": bool(tets), "pairs": pairs, "epochs": epochs,
            "updates": epochs * ((pairs + batch - 1) // batch), "agg_passes": agg_passes, "smoother": smoother,
            "systems_without_reference": skipped,
            "harvest_s": round(t1 - t0, 3), "train_s": round(t2 - t1, 3),
            "loss_before": round(before, 5), "loss_after": round(after, 5)}
    return net, info


def load_poisson_network(path, seed=0):
    """A network saved by train_poisson.py: the weights (checksummed) and
    the application settings of its recipe from the .json beside them.
    Returns (network, recipe)."""
    import json
    from pathlib import Path

    path = Path(path)
    info = json.loads(path.with_suffix(".json").read_text())
    net = Learned(seed=seed)
    net.configure(post_smooth=True, agg_passes=int(info.get("agg_passes", 2)),
                  smoother=int(info.get("smoother", 0)))
    net.load(path)
    return net, info
