"""GPU queries and normals on random meshes (holes, flipped faces, permuted
ids, isolated vertices) with random, disconnected partitions and random
vertex owners, built through the C ABI's partitioned constructor: every
query against the oracle (rows as sets for CSR ops, in order for FV, EV, FE,
EVDiamond, EE), normals within FP32 rounding.  The CPU decode of the same
layouts is checked in tests/test_abi.py; this runs the kernels on them."""
import numpy as np
import pytest
import torch

from test_abi import random_mesh, random_partition

pytestmark = pytest.mark.gpu


def pairs(off, val, row_ids, val_ids):
    off = np.asarray(off, np.int64)
    rows = np.repeat(np.asarray(row_ids, np.int64), np.diff(off))
    vals = np.asarray(val_ids, np.int64)[np.asarray(val, np.int64)]
    o = np.lexsort((vals, rows))
    return rows[o], vals[o]


def ref_pairs(off, val):
    off = np.asarray(off, np.int64)
    rows = np.repeat(np.arange(off.size - 1), np.diff(off))
    vals = np.asarray(val, np.int64)
    o = np.lexsort((vals, rows))
    return rows[o], vals[o]


@pytest.mark.parametrize("seed", range(16))
def test_random_partition_queries(oracle, seed):
    from rxmesh_gb300 import Op, RXMeshStatic, device_check
    rng = np.random.default_rng(100 + seed)
    fv, nv = random_mesh(rng)
    fp, vp = random_partition(rng, fv, nv)
    rx = RXMeshStatic(fv, nv, face_patch=fp, vertex_patch=vp)
    vl, el, fl = rx.linear_to_input("v"), rx.linear_to_input("e"), rx.linear_to_input("f")
    ev, fe = oracle.edges(fv)
    for op, ref, rows, tgt in ((Op.VV, oracle.vv(nv, ev), vl, vl),
                               (Op.VE, oracle.vv(nv, ev, want_edges=True), vl, el),
                               (Op.VF, oracle.vf(nv, fv), vl, fl),
                               (Op.EF, oracle.ef(fv), el, fl),
                               (Op.FF, oracle.ff(fv), fl, fl)):
        off, val = rx.query(op)
        gr, gv = pairs(off.cpu().numpy(), val.cpu().numpy(), rows, tgt)
        wr, wv = ref_pairs(*ref)
        assert np.array_equal(gr, wr) and np.array_equal(gv, wv), (seed, op)
    _, fvq = rx.query(Op.FV)
    assert np.array_equal(vl[fvq.cpu().numpy().reshape(-1, 3)][np.argsort(fl)], fv), seed
    _, evq = rx.query(Op.EV)
    assert np.array_equal(vl[evq.cpu().numpy().reshape(-1, 2)][np.argsort(el)], ev), seed
    _, feq = rx.query(Op.FE)
    assert np.array_equal(el[feq.cpu().numpy().reshape(-1, 3)][np.argsort(fl)], fe), seed
    if rx.is_edge_manifold() and rx.is_oriented():
        _, dq = rx.query(Op.EVD)
        dq = dq.cpu().numpy().reshape(-1, 4)
        assert np.array_equal(np.where(dq >= 0, vl[np.maximum(dq, 0)], -1)[np.argsort(el)],
                              oracle.ev_diamond(fv)), seed
        _, eq = rx.query(Op.EE)
        eq = eq.cpu().numpy().reshape(-1, 4)
        assert np.array_equal(np.where(eq >= 0, el[np.maximum(eq, 0)], -1)[np.argsort(el)],
                              oracle.ee(fv)), seed
    # normals, area weights, on random positions: FP32 against the FP64 oracle
    x = rng.normal(size=(nv, 3)).astype(np.float32)
    n = rx.to_input(rx.vertex_normals(rx.to_linear(torch.tensor(x, device="cuda")), "area")).cpu().numpy()
    ref = oracle.vertex_normals(fv, x.astype(np.float64), 1).reshape(-1, 3)
    scale = np.abs(x).max() ** 2
    assert np.abs(n - ref).max() <= 1e-5 * scale * 8, seed
    device_check()
