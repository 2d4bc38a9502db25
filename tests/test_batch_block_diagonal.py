"""A batch's multigrid couples no two graphs (host only, on the oracle).

The batch path (svxg_set_graphs) builds the reference's hierarchy over the union of its graphs
with one switch: aggregation pass 3 keeps uncoupled leftover rows single instead of grouping them
eight at a time (the oracle's svxo_set_group_isolated; the GPU setup equals the oracle's on the
same union, tests/test_gpu_batch.py). The device's batch iterations skip the rows of graphs whose
sequence has stopped, at every level, which is exact only if every level is block diagonal by
graph. Checked here on a union of ten graphs of 10-700 fragments: every level's operator and
prolongation join rows of one graph only, every coarse row takes exactly one graph from its fine
rows (the device's k_coarse_gmap rule), and the coarsest level's dense Cholesky factor is exactly
zero between graphs (so its inverse, applied in the cycle, is too).
"""
import numpy as np

import oracle
from oracle import Port
from opus_destruct_2_gb300 import synth
from opus_destruct_2_gb300.graph import BOND_DTYPE, StressOptions, default_materials

MATS = default_materials()


def union(gs):
    nodes = np.concatenate([g[0] for g in gs])
    bl, off = [], 0
    for n, b in gs:
        b = b.copy()
        b["a"] += off
        b["b"] = np.where(b["b"] >= 0, b["b"] + off, b["b"])
        bl.append(b)
        off += len(n)
    return nodes, np.concatenate(bl).astype(BOND_DTYPE)


def test_batch_hierarchy_is_block_diagonal():
    gs = []
    for k, (size, free) in enumerate([(12, True), (40, False), (150, True), (300, False), (700, True),
                                      (90, False), (500, True), (260, False), (30, True), (420, False)]):
        n, b, _, _ = synth.piece_graph(size, free=free, seed=700 + k)
        gs.append((n, b))
    nodes, bonds = union(gs)
    graph_of_node = np.concatenate([np.full(len(n), g, np.int32) for g, (n, _) in enumerate(gs)])
    oracle.set_group_isolated(False)  # (the batch's pass 3)
    try:
        O = Port(nodes, bonds, MATS)
        O.keep_levels(True)
        assert O.assemble(StressOptions(amg_min_nodes=32))
    finally:
        oracle.set_group_isolated(True)
    dof = O.matrix()["dof"]
    free = dof >= 0
    gmap = np.full(int(free.sum()), -1, np.int32)
    gmap[dof[free]] = graph_of_node[free]
    assert (gmap >= 0).all()
    levels = O.levels()
    assert len(levels) >= 3
    for l, L in enumerate(levels):
        assert L.n == len(gmap)
        rows = np.repeat(np.arange(L.n), np.diff(L.rowptr))
        assert np.array_equal(gmap[rows], gmap[L.col]), f"level {l}: an operator block joins two graphs"
        if l + 1 < len(levels):
            fine = np.repeat(np.arange(L.n), np.diff(L.prow))
            coarse = np.full(levels[l + 1].n, -1, np.int32)
            coarse[L.pcol] = gmap[fine]
            # every entry of the prolongation names a coarse row of its fine row's graph, and every
            # coarse row has one
            assert np.array_equal(coarse[L.pcol], gmap[fine]), f"level {l}: an aggregate spans two graphs"
            assert (coarse >= 0).all(), f"level {l + 1}: a coarse row no fine row names"
            gmap = coarse
    c = O.chol()
    assert c.shape[0] == 6 * len(gmap) and c.shape[0] > 0
    g6 = np.repeat(gmap, 6)
    cross = g6[:, None] != g6[None, :]
    assert np.all(c[cross] == 0.0), "the coarsest factor couples two graphs"
    assert len(np.unique(gmap)) > 1  # (several graphs reach the coarsest level)
