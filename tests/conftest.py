import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through librxg.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


def golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


def sorted_rows(off, val):
    """CSR -> tuple of sorted tuples (set form of the reference verifier)."""
    off = np.asarray(off, np.int64)
    val = np.asarray(val)
    return [tuple(sorted(val[off[i]:off[i + 1]].tolist())) for i in range(off.size - 1)]


def kat_system(oracle, name):
    # setup() of tests/RXMesh_test/test_solver.cu:79-119: A(v,u)=1 on edges,
    # A(v,v)=2*valence+100, B = valence*(7.4,2.6,10.3), X0 = coords*valence
    g = golden(name)
    nv = len(g["xyz"])
    ev, _ = oracle.edges(g["fv"])
    voff, vval = oracle.vv(nv, ev)
    val_ = np.diff(voff).astype(np.float64)
    rp = np.zeros(nv + 1, np.int64)
    rp[1:] = np.cumsum(val_ + 1)
    col = np.empty(rp[-1], np.int32)
    val = np.empty(rp[-1], np.float64)
    for p in range(nv):
        col[rp[p]] = p
        val[rp[p]] = 2 * val_[p] + 100.0
        col[rp[p] + 1:rp[p + 1]] = vval[voff[p]:voff[p + 1]]
        val[rp[p] + 1:rp[p + 1]] = 1.0
    B = val_[:, None] * np.array([7.4, 2.6, 10.3])
    X0 = g["xyz"] * val_[:, None]
    return rp, col, val, B, X0


def edge_case_meshes():
    """Small meshes on the edge cases of the mesh build: vertices in no face
    (face-less patches), an edge with three faces (not edge-manifold), and two
    disconnected components.  name -> (xyz (nv,3), fv (nf,3))."""
    from rxmesh_gb300 import meshgen
    out = {}
    v, f = meshgen.icosphere(2)
    out["isolated"] = (np.concatenate([v, np.random.default_rng(0).normal(size=(5, 3))]), f)
    x, g = meshgen.plane(8, 8)
    a, b = int(g[20][0]), int(g[20][1])          # an interior edge of the grid
    x = np.concatenate([x, [[0.5, 0.5, 1.0]]])
    out["nonmanifold"] = (x, np.concatenate([g, [[a, b, len(x) - 1]]]).astype(np.int32))
    v1, f1 = meshgen.icosphere(1)
    v2, f2 = meshgen.icosphere(2)
    out["components"] = (np.concatenate([v1, v2 + 3.0]),
                         np.concatenate([f1, f2 + len(v1)]).astype(np.int32))
    return out
