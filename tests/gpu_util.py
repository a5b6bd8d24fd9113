"""Helpers for GPU tests: device copies (torch is only the allocator here)
and the CSR comparison tolerance used by every assembly parity test.

Tolerance: |gpu - oracle| <= 1e-12 * S + 1e-300 per CSR value and rhs
entry. S is the running magnitude of the entry: every edge's formula for
the entry evaluated on |inputs| (|a+b| -> |a|+|b|, |ab| -> |a||b|,
|a/b| -> |a|/|b|, computed by the oracle's *_local_mag kernels) and summed
over the contributing edges. Any evaluation order (FMA contraction on the
GPU, a different summation order of edges into the entry) changes the
result by a small multiple of eps * S, so the bound scales with the terms of
the computation rather than with their possibly cancelling total.
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-12


def dev(a, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


# Per-entry relative check: every entry whose oracle value is at least
# REL_FLOOR times its running magnitude S agrees to RTOL relative to its own
# value. The GPU evaluates the edge formulas in float-float arithmetic
# (about 47 bits: errors up to about 5e-14 S over a formula's dozen or so
# operations), the oracle in FP64 in the reference's order (about 1e-16 S),
# so entries that cancel to below 1e-1 S can differ by more than RTOL of
# their own size while staying far within the running-magnitude bound; their
# worst ratios are reported (NW_PARITY_REPORT).
REL_FLOOR = 1e-1
PARITY_STATS: list = []


def check_close(gpu, ref, scale, what, rtol=RTOL, rel_floor=REL_FLOOR):
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    scale = np.broadcast_to(np.asarray(scale, dtype=np.float64), ref.shape)
    err = np.abs(gpu - ref)
    bound = rtol * scale + 1e-300
    bad = np.nonzero(err > bound)[0]
    assert bad.size == 0, (f"{what}: {bad.size} entries out of tolerance; worst "
                           f"{np.max(err / np.maximum(scale, 1e-300)):.3e} at {bad[:5]}")
    aref = np.abs(ref)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(aref > 0, err / aref, np.where(err > 0, np.inf, 0.0))
        ratio_s = np.where(scale > 0, aref / scale, 1.0)
    stats = {"what": what, "entries": int(ref.size),
             "max_err_over_S": float(np.max(err / np.maximum(scale, 1e-300))) if ref.size else 0.0}
    for t in (1e-1, 1e-2, 1e-3, 1e-4, 1e-6):
        sel = ratio_s >= t
        stats[f"max_rel_where_ref_ge_{t:g}S"] = float(rel[sel].max()) if sel.any() else 0.0
        stats[f"entries_below_{t:g}S"] = int((~sel).sum())
    PARITY_STATS.append(stats)
    sel = ratio_s >= rel_floor
    if sel.any():
        worst = float(rel[sel].max())
        assert worst <= rtol, (f"{what}: an entry with |oracle| >= {rel_floor:g} S differs by "
                               f"{worst:.3e} of its value")


def scalar_fields(nw, d):
    return nw.ScalarFields(d["coords"].data_ptr(), d["velocity"].data_ptr(), d["q"].data_ptr(),
                           d["dqdx"].data_ptr(), d["density"].data_ptr(), d["diff"].data_ptr(),
                           d["area"].data_ptr(), d["mdot"].data_ptr())


def continuity_fields(nw, d):
    return nw.ContinuityFields(d["coords"].data_ptr(), d["velocity"].data_ptr(), d["dpdx"].data_ptr(),
                               d["density"].data_ptr(), d["pressure"].data_ptr(), d["udiag"].data_ptr(),
                               d["area"].data_ptr())


def momentum_fields(nw, d):
    return nw.MomentumFields(d["coords"].data_ptr(), d["velocity"].data_ptr(), d["dudx"].data_ptr(),
                             d["viscosity"].data_ptr(), d["density"].data_ptr(), d["mask"].data_ptr(),
                             d["area"].data_ptr(), d["mdot"].data_ptr(), d["pecfac"].data_ptr())


def to_dev_dict(arrs: dict) -> dict:
    return {k: dev(v) for k, v in arrs.items() if isinstance(v, np.ndarray)}


def oracle_scalar(orc, edges, nalu_id, f, opts_dict):
    o = orc.ScalarOpts(**opts_dict)
    lhs, rhs = orc.scalar_local(edges, f["coords"], f["velocity"], f["q"], f["dqdx"], f["density"], f["diff"],
                                f["area"], f["mdot"], o)
    ml, mr = orc.scalar_local(edges, f["coords"], f["velocity"], f["q"], f["dqdx"], f["density"], f["diff"],
                              f["area"], f["mdot"], o, mag=True)
    return _assemble(orc, edges, nalu_id, 1, lhs, rhs, ml, mr)


def _assemble(orc, edges, nalu_id, nd, lhs, rhs, ml, mr):
    rp, ci, lid = orc.build_graph(nalu_id, edges, nd)
    vals, b, _, _ = orc.sum_into(edges, nd, lhs, rhs, lid, rp, ci, with_abs=False)
    va, ba, _, _ = orc.sum_into(edges, nd, ml, mr, lid, rp, ci, with_abs=False)
    return dict(rp=rp, ci=ci, lid=lid, vals=vals, rhs=b, vabs=va, rabs=ba)


def oracle_continuity(orc, edges, nalu_id, f, opts_dict):
    o = orc.ContinuityOpts(**opts_dict)
    args = (edges, f["coords"], f["velocity"], f["dpdx"], f["density"], f["pressure"], f["udiag"], f["area"], o)
    lhs, rhs = orc.continuity_local(*args)
    ml, mr = orc.continuity_local(*args, mag=True)
    return _assemble(orc, edges, nalu_id, 1, lhs, rhs, ml, mr)


def oracle_momentum(orc, edges, nalu_id, f, opts_dict):
    o = orc.MomentumOpts(**opts_dict)
    args = (edges, f["coords"], f["velocity"], f["velocity"], f["dudx"], f["viscosity"], f["density"], f["mask"],
            f["area"], f["mdot"], f["pecfac"], o)
    lhs, rhs = orc.momentum_local(*args)
    ml, mr = orc.momentum_local(*args, mag=True)
    return _assemble(orc, edges, nalu_id, 3, lhs, rhs, ml, mr)
