"""CPU tests of the work list of the single-kernel momentum assembly
(nw_momentum_schedule; the kernel is momentum_fused_k in assemble.cu).

The kernel's blocks take items in list order; a row block waits for the
edge chunks it reads, and an edge chunk that reuses a ring slot waits for
the row blocks that read the slot's previous chunk. The list is correct
when (1) it holds every item once, (2) every wait points to earlier items
(so it cannot deadlock, whatever the number of resident blocks), and (3)
executing it in list order, a row block finds each of its input chunks
still in its ring slot."""
import numpy as np
import pytest


def _check(sched, edges, rows):
    E = edges.shape[0]
    ch, kb = sched["chunk_edges"], sched["block_rows"]
    nch, nrb, S = sched["edge_chunks"], sched["row_blocks"], sched["ring_chunks"]
    assert nch == -(-E // ch) and nrb == -(-rows // kb)
    items = sched["items"]
    assert sorted(items.tolist()) == sorted([2 * c for c in range(nch)] + [2 * k + 1 for k in range(nrb)])
    pos = np.full(2 * max(nch, nrb) + 2, -1, np.int64)
    pos[items] = np.arange(items.size)  # list position of item 2c / 2k+1
    # true input chunks per row block and reader blocks per chunk
    chunk = np.repeat(np.arange(E) // ch, 2)
    blk = edges.reshape(-1) // kb
    lo = np.full(nrb, np.iinfo(np.int32).max)
    hi = np.full(nrb, -1)
    np.minimum.at(lo, blk, chunk)
    np.maximum.at(hi, blk, chunk)
    np.testing.assert_array_equal(sched["chunk_lo"], lo)
    np.testing.assert_array_equal(sched["chunk_hi"], hi)
    blo = np.full(nch, np.iinfo(np.int32).max)
    bhi = np.full(nch, -1)
    np.minimum.at(blo, chunk, blk)
    np.maximum.at(bhi, chunk, blk)
    np.testing.assert_array_equal(sched["block_lo"], blo)
    np.testing.assert_array_equal(sched["block_hi"], bhi)
    # (2) waits point backwards: every chunk in a block's range, and every
    # reader of a slot's previous chunk
    for k in range(nrb):
        if hi[k] >= 0:
            assert pos[2 * hi[k]] < pos[2 * k + 1]  # chunks are placed in order
    if S < nch:
        nchunks_before = np.cumsum(items % 2 == 0) - (items % 2 == 0)
        for c in range(S, nch):
            assert pos[2 * bhi[c - S] + 1] < pos[2 * c]
            assert all(pos[2 * b + 1] < pos[2 * c] for b in range(blo[c - S], bhi[c - S] + 1))
            # ... and the last of them came at least lag chunks before it
            assert nchunks_before[pos[2 * bhi[c - S] + 1]] + sched["lag_chunks"] <= c
    # (3) list-order execution against the ring
    owner = np.full(min(S, nch), -1)
    inc = [[] for _ in range(nrb)]
    for b, c in zip(blk.tolist(), chunk.tolist()):
        inc[b].append(c)
    for it in items.tolist():
        if it % 2 == 0:
            owner[(it // 2) % S] = it // 2
        else:
            for c in inc[it // 2]:
                assert owner[c % S] == c
    return pos


@pytest.mark.parametrize("conc", [8, 64])
def test_lexicographic_hex_box_gets_a_small_ring(nw, conc):
    mesh = nw.Mesh(40, 36, 30, stretch_z=1.08, jitter=0.05, seed=2)
    s = nw.momentum_schedule(mesh.num_nodes, mesh.edges, conc)
    pos = _check(s, mesh.edges, mesh.num_nodes)
    assert s["ring_chunks"] < s["edge_chunks"]
    assert 0 < s["ring_bytes"] <= 64 << 20
    # the lag: a block comes at least lag chunks after its last input
    # (the ring was sized so that no block had to come early)
    items = s["items"]
    nchunks_before = np.cumsum(items % 2 == 0)
    for k in range(s["row_blocks"]):
        p = pos[2 * k + 1]
        if s["chunk_hi"][k] >= 0 and nchunks_before[p] < s["edge_chunks"]:
            assert nchunks_before[p] - 1 - s["chunk_hi"][k] >= s["lag_chunks"]


def test_random_order_falls_back_to_one_slot_per_chunk(nw):
    mesh = nw.Mesh(20, 18, 16, tets=True, renumber=1, renumber_seed=5)
    s = nw.momentum_schedule(mesh.num_nodes, mesh.edges, 608)
    _check(s, mesh.edges, mesh.num_nodes)
    assert s["ring_chunks"] == s["edge_chunks"] and s["ring_bytes"] == 0


@pytest.mark.parametrize("max_ring", [64 << 20, 3 << 20])
def test_rcm_tets_and_a_tight_ring_limit(nw, max_ring):
    mesh = nw.Mesh(24, 22, 20, tets=True, renumber=2, renumber_seed=9)
    s = nw.momentum_schedule(mesh.num_nodes, mesh.edges, 64, max_ring)
    _check(s, mesh.edges, mesh.num_nodes)
    assert s["ring_bytes"] <= max_ring


def test_small_and_degenerate_graphs(nw):
    # one edge; isolated rows; rows beyond the last edge
    e = np.array([[0, 1]], np.int64)
    _check(nw.momentum_schedule(2, e, 4), e, 2)
    e = np.array([[0, 300], [5, 6], [299, 1]], np.int64)
    _check(nw.momentum_schedule(400, e, 4), e, 400)
    with pytest.raises(nw.NwError):
        nw.momentum_schedule(2, np.array([[0, 2]], np.int64), 4)
