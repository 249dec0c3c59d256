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


@pytest.mark.parametrize("ops", [("VE",), ("VV",), ("VF", "normals"), ("FV", "EV"), ("VE", "VF"), ("normals",),
                                 ("VF", "FV"), ("VV", "VE", "EV")])
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


def check_host_sweep(rx, x, ops=("VV", "VE", "VF", "FV", "EV", "normals"), xyz_host=True):
    """rxg_query_sweep_ex with page-locked host outputs: the separate
    queries' offsets, rows as the same sets (a row's order comes from
    shared-memory atomics), FV / EV and normals bit for bit."""
    from rxmesh_gb300 import Op, device_check
    xl = rx.to_linear(torch.tensor(np.asarray(x, np.float32), device="cuda"))
    xin = xl.cpu().pin_memory() if xyz_host else xl
    s = torch.cuda.Stream()
    got = rx.query_sweep(ops, xyz=xin, weighting="area", stream=s, host=True)
    s.synchronize()
    for name in ops:
        if name == "normals":
            assert not got[name].is_cuda
            assert torch.equal(got[name], rx.vertex_normals(xl, "area").cpu())
            continue
        op = Op.NAMES[name]
        off, val = rx.query(op)
        if op in Op.CSR:
            go, gv = got[name]
            assert torch.equal(go, off.cpu()), name
            a, b = row_pairs(go.numpy(), gv.numpy()), row_pairs(off.cpu().numpy(), val.cpu().numpy())
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), name
        else:
            assert torch.equal(got[name], val.cpu()), name
    device_check()


@pytest.mark.parametrize("name", ["icosphere4", "torus", "bunnyhead", "components", "nonmanifold"])
def test_host_sweep_equals_separate_queries(name):
    from rxmesh_gb300 import RXMeshStatic
    make, patch = MESHES[name]
    x, f = make()
    rx = RXMeshStatic(f, len(x), patch_size=patch)
    check_host_sweep(rx, x)
    check_host_sweep(rx, x, xyz_host=False)


@pytest.mark.parametrize("ops", [("EV",), ("VF", "normals"), ("VV", "FV"), ("normals",)])
def test_host_sweep_subsets(ops):
    from rxmesh_gb300 import RXMeshStatic
    x, f = meshgen.torus(40, 30, jitter=1e-3, seed=3)
    rx = RXMeshStatic(f, len(x), patch_size=128)
    check_host_sweep(rx, x, ops)


def test_host_sweep_mixed_outputs_and_repeats():
    """Some outputs on the device, some in page-locked host memory, three
    calls in a row on one stream into the same buffers."""
    from rxmesh_gb300 import Op, RXMeshStatic, _lib
    x, f = meshgen.torus(50, 40, jitter=1e-3, seed=4)
    rx = RXMeshStatic(f, len(x), patch_size=128)
    L = _lib.load()
    rows, nval = rx.query_size(Op.VV)
    vv_off = torch.empty(rows + 1, dtype=torch.int32, device="cuda")
    vv_val = torch.empty(nval, dtype=torch.int32).pin_memory()
    ev = torch.empty(2 * rx.get_num_edges(), dtype=torch.int32, device="cuda")
    fv = torch.empty(3 * rx.get_num_faces(), dtype=torch.int32).pin_memory()
    so = _lib.SweepOut()
    so.vv_offsets, so.vv_values = vv_off.data_ptr(), vv_val.data_ptr()
    so.ev_values, so.fv_values = ev.data_ptr(), fv.data_ptr()
    s = torch.cuda.Stream()
    for _ in range(3):
        _lib.check(L.rxg_query_sweep_ex(rx._h, ctypes.byref(so), 1, ctypes.c_void_p(s.cuda_stream)))
    s.synchronize()
    off, val = rx.query(Op.VV)
    assert torch.equal(vv_off, off)
    a, b = row_pairs(vv_off.cpu().numpy(), vv_val.numpy()), row_pairs(off.cpu().numpy(), val.cpu().numpy())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert torch.equal(ev, rx.query(Op.EV)[1]) and torch.equal(fv, rx.query(Op.FV)[1].cpu())


def test_host_sweep_rejects_bad_arguments():
    from rxmesh_gb300 import RXGError, RXMeshStatic, _lib
    L = _lib.load()
    x, f = meshgen.icosphere(2)
    rx = RXMeshStatic(f, len(x), patch_size=64)
    so = _lib.SweepOut()
    pageable = np.zeros(3 * rx.get_num_faces(), np.int32)
    so.fv_values = pageable.ctypes.data  # host memory that is not page-locked
    with pytest.raises(RXGError):
        _lib.check(L.rxg_query_sweep_ex(rx._h, ctypes.byref(so), 1, None))
    so = _lib.SweepOut()
    so.fv_values = torch.empty(3 * rx.get_num_faces(), dtype=torch.int32).pin_memory().data_ptr()
    with pytest.raises(RXGError):
        _lib.check(L.rxg_query_sweep_ex(rx._h, ctypes.byref(so), 4, None))  # unknown flag
