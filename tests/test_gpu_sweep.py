"""rxg_query_sweep (VV, VE, VF, FV, EV and normals in one launch) against
the separate queries: the same offsets, the same rows as sets, FV / EV and
normals bit for bit; any subset of outputs; argument checks."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import edge_case_meshes, golden
from rxmesh_gb300 import meshgen
from test_abi import random_mesh, random_partition

pytestmark = pytest.mark.gpu


def row_pairs(off, val):
    off = np.asarray(off, np.int64)
    rows = np.repeat(np.arange(off.size - 1), np.diff(off))
    vals = np.asarray(val, np.int64)
    o = np.lexsort((vals, rows))
    return rows[o], vals[o]


def check_against_queries(rx, x, ops=("VV", "VE", "VF", "FV", "EV", "normals")):
    from rxmesh_gb300 import Op, device_check
    xl = rx.to_linear(torch.tensor(np.asarray(x, np.float32), device="cuda"))
    for w in ("area", "max"):
        got = rx.query_sweep(ops, xyz=xl, weighting=w)
        torch.cuda.synchronize()
        for name in ops:
            if name == "normals":
                assert torch.equal(got[name], rx.vertex_normals(xl, w)), w
                continue
            op = Op.NAMES[name]
            off, val = rx.query(op)
            if op in Op.CSR:
                go, gv = got[name]
                assert torch.equal(go, off), name
                a, b = row_pairs(go.cpu().numpy(), gv.cpu().numpy()), row_pairs(off.cpu().numpy(), val.cpu().numpy())
                assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), name
            else:
                assert torch.equal(got[name], val), name
    device_check()


MESHES = {
    "icosphere4": (lambda: meshgen.icosphere(4), 64),
    "icosphere4_512": (lambda: meshgen.icosphere(4), 512),
    "torus": (lambda: meshgen.torus(64, 48, jitter=1e-3, seed=1), 256),
    "bunnyhead": (lambda: (golden("bunnyhead")["xyz"], golden("bunnyhead")["fv"]), 256),
    "components": (lambda: edge_case_meshes()["components"], 64),
    "isolated": (lambda: edge_case_meshes()["isolated"], 64),
    "nonmanifold": (lambda: edge_case_meshes()["nonmanifold"], 64),
}


@pytest.mark.parametrize("name", list(MESHES))
def test_sweep_equals_separate_queries(name):
    from rxmesh_gb300 import RXMeshStatic
    make, patch = MESHES[name]
    x, f = make()
    rx = RXMeshStatic(f, len(x), patch_size=patch)
    check_against_queries(rx, x)


@pytest.mark.parametrize("seed", range(6))
def test_sweep_on_random_partitions(seed):
    from rxmesh_gb300 import RXMeshStatic
    rng = np.random.default_rng(200 + seed)
    fv, nv = random_mesh(rng)
    fp, vp = random_partition(rng, fv, nv)
    rx = RXMeshStatic(fv, nv, face_patch=fp, vertex_patch=vp)
    check_against_queries(rx, rng.normal(size=(nv, 3)))


@pytest.mark.parametrize("ops", [("VE",), ("VV",), ("VF", "normals"), ("FV", "EV"), ("VE", "VF"), ("normals",)])
def test_sweep_subsets(ops):
    from rxmesh_gb300 import RXMeshStatic
    x, f = meshgen.icosphere(4)
    rx = RXMeshStatic(f, len(x), patch_size=128)
    check_against_queries(rx, x, ops)


def test_sweep_rejects_bad_arguments():
    from rxmesh_gb300 import RXGError, RXMeshStatic, _lib
    L = _lib.load()
    x, f = meshgen.icosphere(2)
    rx = RXMeshStatic(f, len(x), patch_size=64)
    so = _lib.SweepOut()
    val = torch.empty(2 * rx.get_num_edges(), dtype=torch.int32, device="cuda")
    so.vv_values = val.data_ptr()  # values without offsets
    with pytest.raises(RXGError):
        _lib.check(L.rxg_query_sweep(rx._h, ctypes.byref(so), None))
    host = np.zeros(3 * rx.get_num_faces(), np.int32)
    so = _lib.SweepOut()
    so.fv_values = host.ctypes.data  # host array
    with pytest.raises(RXGError):
        _lib.check(L.rxg_query_sweep(rx._h, ctypes.byref(so), None))
    so = _lib.SweepOut()
    so.normals = torch.empty(len(x), 3, device="cuda").data_ptr()  # no positions
    with pytest.raises(RXGError):
        _lib.check(L.rxg_query_sweep(rx._h, ctypes.byref(so), None))
