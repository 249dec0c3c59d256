"""GPU parity of the patch queries and vertex normals against the oracle.

Adjacency is compared bit-exactly as sorted sets in input ids (the form of
tests/RXMesh_test/rxmesh_test.h:347-440); normals within 1e-6 relative."""
import numpy as np
import pytest
import torch

from conftest import edge_case_meshes, golden, sorted_rows
from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu

MESHES = {
    "torus64": lambda: meshgen.torus(64, 48, jitter=1e-3, seed=1),
    "icosphere4": lambda: meshgen.icosphere(4),
    "plane": lambda: meshgen.plane(40, 23),
    "sphere3": lambda: (golden("sphere3")["xyz"], golden("sphere3")["fv"]),
    "cloth": lambda: (golden("cloth")["xyz"], golden("cloth")["fv"]),
    "bunnyhead": lambda: (golden("bunnyhead")["xyz"], golden("bunnyhead")["fv"]),
    "plane_5": lambda: (golden("plane_5")["xyz"], golden("plane_5")["fv"]),
    "isolated": lambda: edge_case_meshes()["isolated"],
    "nonmanifold": lambda: edge_case_meshes()["nonmanifold"],
    "components": lambda: edge_case_meshes()["components"],
}


# (mesh, patch size); "patcher": the partition RXMesh saved for the mesh
# (input/<name>_patches, kept in the golden fixture); "gpu": the GPU patcher
CASES = ([(n, p) for n in MESHES for p in (64, 512)] + [("sphere3", "patcher"), ("torus", "patcher")]
         + [(n, "gpu") for n in ("torus64", "icosphere4", "sphere3", "isolated", "nonmanifold",
                                 "components")])


def make_rx(name, patch, tmp_path):
    from rxmesh_gb300 import RXMeshStatic
    if patch == "patcher":
        g = golden(name)
        path = tmp_path / (name + "_patches")
        path.write_bytes(g["patcher_file"].tobytes())
        return g["xyz"], g["fv"], RXMeshStatic(g["fv"], len(g["xyz"]), patcher_file=str(path))
    x, f = MESHES[name]()
    if patch == "gpu":  # partitioned on the GPU (Lloyd), 64-face patches
        return x, f, RXMeshStatic(f, len(x), patch_size=64, gpu_patcher=True)
    return x, f, RXMeshStatic(f, len(x), patch_size=patch)


def gpu_rows(rx, op):
    from rxmesh_gb300 import Op
    vl = rx.linear_to_input("v")
    tgt = {Op.VV: vl, Op.VE: rx.linear_to_input("e"), Op.VF: rx.linear_to_input("f")}[op]
    off, val = rx.query(op)
    torch.cuda.synchronize()
    off, val = off.cpu().numpy(), val.cpu().numpy()
    rows = [None] * len(vl)
    for lin in range(len(vl)):
        rows[vl[lin]] = tuple(sorted(tgt[val[off[lin]:off[lin + 1]]].tolist()))
    return rows, off


@pytest.mark.parametrize("name,patch", CASES)
def test_queries_bit_exact(oracle, name, patch, tmp_path):
    from rxmesh_gb300 import Op, device_check
    x, f, rx = make_rx(name, patch, tmp_path)
    nv = len(x)
    ev, _ = oracle.edges(f)
    o, v = oracle.vv(nv, ev)
    got, off = gpu_rows(rx, Op.VV)
    assert got == sorted_rows(o, v)
    assert off[0] == 0 and off[-1] == 2 * len(ev)
    o, v = oracle.vv(nv, ev, want_edges=True)
    assert gpu_rows(rx, Op.VE)[0] == sorted_rows(o, v)
    o, v = oracle.vf(nv, f)
    assert gpu_rows(rx, Op.VF)[0] == sorted_rows(o, v)
    vl, el, fl = rx.linear_to_input("v"), rx.linear_to_input("e"), rx.linear_to_input("f")
    _, fvq = rx.query(Op.FV)
    _, evq = rx.query(Op.EV)
    fvq = fvq.cpu().numpy().reshape(-1, 3)
    evq = evq.cpu().numpy().reshape(-1, 2)
    assert np.array_equal(vl[fvq][np.argsort(fl)], np.asarray(f))
    assert np.array_equal(vl[evq][np.argsort(el)], ev)
    device_check()


@pytest.mark.parametrize("name,patch", CASES)
def test_edge_and_face_queries_bit_exact(oracle, name, patch, tmp_path):
    """EF, FF (rows as sets), FE and EVDiamond (rows in order) against the
    oracle, in input ids (Op::EF/FE/FF/EVDiamond, kernels/rxmesh_queries.cuh)."""
    from rxmesh_gb300 import Op, device_check
    x, f, rx = make_rx(name, patch, tmp_path)
    vl, el, fl = rx.linear_to_input("v"), rx.linear_to_input("e"), rx.linear_to_input("f")
    ev, fe = oracle.edges(f)

    def rows_in_input(op, row_ids, val_ids):
        off, val = rx.query(op)
        off, val = off.cpu().numpy(), val.cpu().numpy()
        rows = [None] * len(row_ids)
        for lin in range(len(row_ids)):
            rows[row_ids[lin]] = tuple(sorted(val_ids[val[off[lin]:off[lin + 1]]].tolist()))
        return rows, off

    o, v = oracle.ef(f)
    got, off = rows_in_input(Op.EF, el, fl)
    assert got == sorted_rows(o, v) and off[-1] == 3 * len(f)
    o, v = oracle.ff(f)
    got, off = rows_in_input(Op.FF, fl, fl)
    assert got == sorted_rows(o, v) and off[-1] == len(v)
    _, feq = rx.query(Op.FE)
    feq = feq.cpu().numpy().reshape(-1, 3)
    assert np.array_equal(el[feq][np.argsort(fl)], fe)
    if not rx.info["is_edge_manifold"]:  # EVDiamond is refused, not raced
        from rxmesh_gb300 import RXGError
        with pytest.raises(RXGError):
            rx.query(Op.EVD)
        device_check()
        return
    _, dq = rx.query(Op.EVD)
    dq = dq.cpu().numpy().reshape(-1, 4)
    din = np.where(dq >= 0, vl[np.maximum(dq, 0)], -1)[np.argsort(el)]
    assert np.array_equal(din, oracle.ev_diamond(f))
    _, eq = rx.query(Op.EE)
    eq = eq.cpu().numpy().reshape(-1, 4)
    assert np.array_equal(np.where(eq >= 0, el[np.maximum(eq, 0)], -1)[np.argsort(el)], oracle.ee(f))
    device_check()


@pytest.mark.parametrize("patch", [64, 512])
def test_ff_ef_on_inconsistently_oriented_mesh(oracle, patch):
    """One flipped face: FF takes the general per-patch EF counting sort (the
    two-slot kernel needs consistent orientation); EF and FE do not depend on
    orientation; EVDiamond is refused."""
    from rxmesh_gb300 import Op, RXMeshStatic, RXGError
    _, f = meshgen.icosphere(4)
    f = np.array(f, np.int32).copy()
    f[17] = f[17][::-1]
    rx = RXMeshStatic(f, int(f.max()) + 1, patch_size=patch)
    el, fl = rx.linear_to_input("e"), rx.linear_to_input("f")
    for op, rows_ids, val_ids, ref in ((Op.FF, fl, fl, oracle.ff(f)), (Op.EF, el, fl, oracle.ef(f))):
        off, val = rx.query(op)
        off, val = off.cpu().numpy(), val.cpu().numpy()
        got = [None] * len(rows_ids)
        for lin in range(len(rows_ids)):
            got[rows_ids[lin]] = tuple(sorted(val_ids[val[off[lin]:off[lin + 1]]].tolist()))
        assert got == sorted_rows(*ref), op
    with pytest.raises(RXGError):
        rx.query(Op.EVD)


@pytest.mark.parametrize("level,patch", [(3, 128), (5, 128)])
def test_query_into_host_buffers(oracle, level, patch):
    """Host outputs (sliced launches, copies overlapped) equal the device outputs."""
    import ctypes
    from rxmesh_gb300 import Op, RXMeshStatic, _lib
    x, f = meshgen.icosphere(level)
    rx = RXMeshStatic(f, len(x), patch_size=patch)
    for op in (Op.VV, Op.VE, Op.VF, Op.FV, Op.EV, Op.EF, Op.FE, Op.FF, Op.EVD, Op.EE):
        rows, nval = rx.query_size(op)
        csr = op in Op.CSR
        off = np.full(rows + 1, -7, np.int32) if csr else None
        val = np.full(nval, -7, np.int32)
        rx.query_host(op, off, val)
        d_off, d_val = rx.query(op)
        if csr:  # rows are sets (their order comes from shared-memory atomics)
            assert np.array_equal(off, d_off.cpu().numpy()), op
            assert sorted_rows(off, val) == sorted_rows(off, d_val.cpu().numpy()), op
        else:
            assert np.array_equal(val, d_val.cpu().numpy()), op
    # normals: host positions in, host normals out
    x32 = np.ascontiguousarray(rx.to_linear(torch.tensor(x, device="cuda")).cpu().numpy(), np.float32)
    out = np.full_like(x32, np.nan)
    L = _lib.load()
    _lib.check(L.rxg_vertex_normals(rx._h, 1, ctypes.c_void_p(x32.ctypes.data),
                                    ctypes.c_void_p(out.ctypes.data), None))
    dev = rx.vertex_normals(torch.tensor(x32, device="cuda"), "area").cpu().numpy()
    assert np.allclose(out, dev, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("level,patch", [(3, 128), (5, 512)])
def test_query_into_pinned_host_buffers(oracle, level, patch):
    """Page-locked (and mixed page-locked / pageable) host outputs and inputs
    through the C ABI give the device results bit for bit (normals) or as the
    same row sets (adjacency rows are ordered by shared-memory atomics)."""
    import ctypes
    from rxmesh_gb300 import Op, RXMeshStatic, _lib
    L = _lib.load()
    x, f = meshgen.icosphere(level)
    rx = RXMeshStatic(f, len(x), patch_size=patch)
    for op in (Op.VV, Op.VE, Op.VF, Op.FV, Op.EV, Op.EF, Op.FE, Op.FF, Op.EVD, Op.EE):
        rows, nval = rx.query_size(op)
        csr = op in Op.CSR
        d_off, d_val = rx.query(op)
        for pin_off, pin_val in ((True, True), (False, True), (True, False)):
            if not csr and not pin_val:
                continue
            off = None
            if csr:
                off = torch.full((rows + 1,), -7, dtype=torch.int32)
                off = off.pin_memory() if pin_off else off
            val = torch.full((nval,), -7, dtype=torch.int32)
            val = val.pin_memory() if pin_val else val
            _lib.check(L.rxg_query(rx._h, int(op),
                                   ctypes.c_void_p(off.data_ptr()) if csr else None,
                                   ctypes.c_void_p(val.data_ptr()), None))
            if csr:
                assert torch.equal(off, d_off.cpu()), (op, pin_off, pin_val)
                assert sorted_rows(off.numpy(), val.numpy()) == \
                    sorted_rows(off.numpy(), d_val.cpu().numpy()), (op, pin_off, pin_val)
            else:
                assert torch.equal(val, d_val.cpu()), op
    x32 = rx.to_linear(torch.tensor(x, device="cuda")).float()
    dev = rx.vertex_normals(x32, "max").cpu()
    for pin_in in (True, False):
        xin = x32.cpu().pin_memory() if pin_in else x32.cpu()
        out = torch.full_like(xin, float("nan")).pin_memory()
        _lib.check(L.rxg_vertex_normals(rx._h, 0, ctypes.c_void_p(xin.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), None))
        assert torch.equal(out, dev), pin_in


@pytest.mark.parametrize("flags", [1, 2, 3])
def test_query_ex_stream_ordered(flags):
    """rxg_query_ex / rxg_vertex_normals_ex with RXG_HOST_ASYNC (1),
    RXG_HOST_DIRECT (2) or both: every op issued on its own stream before
    any of them is waited for, page-locked (and device-offset / pageable)
    outputs; after the streams complete the host arrays equal the device
    results (row sets for CSR rows, bit for bit otherwise)."""
    import ctypes
    from rxmesh_gb300 import Op, RXGError, RXMeshStatic, _lib
    L = _lib.load()
    x, f = meshgen.icosphere(5)
    rx = RXMeshStatic(f, len(x), patch_size=128)
    ops = (Op.VV, Op.VE, Op.VF, Op.FV, Op.EV, Op.EF, Op.FE, Op.FF, Op.EVD, Op.EE)
    cases = []
    for op in ops:
        rows, nval = rx.query_size(op)
        csr = op in Op.CSR
        for kind in ("pinned", "device_offsets", "pageable"):
            if kind == "device_offsets" and not csr:
                continue
            off = None
            if csr:
                off = torch.full((rows + 1,), -7, dtype=torch.int32,
                                 device="cuda" if kind == "device_offsets" else "cpu")
                off = off.pin_memory() if kind == "pinned" else off
            val = torch.full((nval,), -7, dtype=torch.int32)
            val = val if kind == "pageable" else val.pin_memory()
            cases.append((op, kind, off, val, torch.cuda.Stream()))
    x32 = rx.to_linear(torch.tensor(x, device="cuda")).float()
    xin = x32.cpu().pin_memory()
    nrm = torch.full_like(xin, float("nan")).pin_memory()
    ns = torch.cuda.Stream()
    torch.cuda.synchronize()
    for op, kind, off, val, s in cases:
        _lib.check(L.rxg_query_ex(rx._h, int(op), ctypes.c_void_p(off.data_ptr()) if off is not None else None,
                                  ctypes.c_void_p(val.data_ptr()), flags, ctypes.c_void_p(s.cuda_stream)))
    _lib.check(L.rxg_vertex_normals_ex(rx._h, 1, ctypes.c_void_p(xin.data_ptr()),
                                       ctypes.c_void_p(nrm.data_ptr()), flags, ctypes.c_void_p(ns.cuda_stream)))
    torch.cuda.synchronize()
    for op, kind, off, val, s in cases:
        d_off, d_val = rx.query(op)
        if off is not None:
            assert torch.equal(off.cpu(), d_off.cpu()), (op, kind)
            o = off.cpu().numpy()
            assert sorted_rows(o, val.numpy()) == sorted_rows(o, d_val.cpu().numpy()), (op, kind)
        else:
            assert torch.equal(val, d_val.cpu()), (op, kind)
    assert torch.equal(nrm, rx.vertex_normals(x32, "area").cpu())
    val = torch.empty(rx.query_size(Op.VV)[1], dtype=torch.int32).pin_memory()
    off = torch.empty(rx.query_size(Op.VV)[0] + 1, dtype=torch.int32).pin_memory()
    with pytest.raises(RXGError):
        _lib.check(L.rxg_query_ex(rx._h, int(Op.VV), ctypes.c_void_p(off.data_ptr()),
                                  ctypes.c_void_p(val.data_ptr()), 4, None))


def test_query_host_asynchronous_python():
    """RXMeshStatic.query_host(..., asynchronous=True) on page-locked tensors
    and a side stream: after the stream completes, the rows equal query()."""
    from rxmesh_gb300 import Op, RXMeshStatic
    x, f = meshgen.icosphere(4)
    rx = RXMeshStatic(f, len(x), patch_size=128)
    s = torch.cuda.Stream()
    for op in (Op.VV, Op.FV, Op.EE):
        rows, nval = rx.query_size(op)
        off = torch.full((rows + 1,), -7, dtype=torch.int32).pin_memory() if op in Op.CSR else None
        val = torch.full((nval,), -7, dtype=torch.int32).pin_memory()
        rx.query_host(op, off, val, asynchronous=True, stream=s)
        s.synchronize()
        d_off, d_val = rx.query(op)
        if off is not None:
            assert torch.equal(off, d_off.cpu())
            o = off.numpy()
            assert sorted_rows(o, val.numpy()) == sorted_rows(o, d_val.cpu().numpy())
        else:
            assert torch.equal(val, d_val.cpu()), op


@pytest.mark.parametrize("name,patch", [(n, 256) for n in ("sphere3", "torus", "cloth", "bunnyhead")]
                         + [("sphere3", "patcher"), ("torus", "patcher")])
def test_normals_against_reference_fixture(oracle, name, patch, tmp_path):
    # fixtures: output of the reference's own vertex_normal_ref (FP64 and FP32)
    from rxmesh_gb300 import RXMeshStatic
    g = golden(name)
    if patch == "patcher":
        rx = make_rx(name, patch, tmp_path)[2]
    else:
        rx = RXMeshStatic(g["fv"], len(g["xyz"]), patch_size=patch)
    x32 = g["xyz"].astype(np.float32)
    x = torch.tensor(x32, device="cuda")
    n = rx.to_input(rx.vertex_normals(rx.to_linear(x), "max")).cpu().numpy()
    # 1e-6 relative against the FP64 oracle on the same (FP32) positions
    ref = oracle.vertex_normals(g["fv"], x32.astype(np.float64), 0)
    err = np.linalg.norm(n - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() < 1e-6
    # the reference's FP32 run, with its own absolute check (vertex_normal.cu:90-108)
    assert np.abs(np.abs(n) - np.abs(g["ref_normals_f32"])).max() <= 1e-4
    # and its FP64 run on the unrounded positions (input quantisation only)
    ref64 = g["ref_normals_f64"]
    assert (np.linalg.norm(n - ref64, axis=1) / np.linalg.norm(ref64, axis=1)).max() < 1e-5


@pytest.mark.parametrize("weighting", ["max", "area"])
def test_normals_torus(oracle, weighting):
    from rxmesh_gb300 import RXMeshStatic
    x, f = meshgen.torus(128, 96, jitter=1e-3, seed=3)
    rx = RXMeshStatic(f, len(x), patch_size=512)
    xt = torch.tensor(x, device="cuda")
    n = rx.to_input(rx.vertex_normals(rx.to_linear(xt), weighting)).cpu().numpy()
    ref = oracle.vertex_normals(f, x.astype(np.float64), 0 if weighting == "max" else 1)
    err = np.linalg.norm(n - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() < 1e-6


def test_oriented_vv_gpu(oracle):
    from rxmesh_gb300 import RXMeshStatic
    for x, f in [meshgen.icosphere(3), meshgen.plane(17, 11), meshgen.torus(20, 12)]:
        nv = len(x)
        rx = RXMeshStatic(f, nv, patch_size=64)
        off, val, bnd = (t.cpu().numpy() for t in rx.query_oriented_vv())
        vl = rx.linear_to_input("v")
        o_off, o_ring, o_bnd = oracle.oriented_vv(nv, f)
        for lin in range(nv):
            p = vl[lin]
            r = vl[val[off[lin]:off[lin + 1]]].tolist()
            w = o_ring[o_off[p]:o_off[p + 1]].tolist()
            assert bnd[lin] == o_bnd[p]
            if o_bnd[p]:
                assert r == w  # same boundary start, same direction
            else:
                k = w.index(r[0])
                assert r == w[k:] + w[:k]  # same cyclic order


def test_full_torus_properties():
    # 1024 x 1024 torus at full size: size-independent properties
    from rxmesh_gb300 import Op, RXMeshStatic
    x, f = meshgen.torus(1024, 1024, jitter=1e-3, seed=0)
    rx = RXMeshStatic(f, len(x), patch_size=512)
    off, val = rx.query(Op.VV)
    assert int(off[-1]) == 2 * rx.get_num_edges()
    deg = (off[1:] - off[:-1])
    assert int(deg.min()) == 6 and int(deg.max()) == 6
    # symmetry: sum over rows of (row id, neighbour) pairs equals its transpose
    rows = torch.repeat_interleave(torch.arange(len(deg), device="cuda"), deg.long())
    fwd = rows.long() * len(deg) + val.long()
    bwd = val.long() * len(deg) + rows.long()
    assert torch.equal(torch.sort(fwd).values, torch.sort(bwd).values)
    _, fvq = rx.query(Op.FV)
    assert int(torch.bincount(fvq.long(), minlength=len(deg)).min()) == 6


def test_boundary_vertices_device():
    """get_boundary_vertices into device memory equals the host copy;
    bunnyhead's 98 (tests/RXMesh_test/test_boundary.cu)."""
    from rxmesh_gb300 import RXMeshStatic
    g = golden("bunnyhead")
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), patch_size=256)
    host = RXMeshStatic(g["fv"], len(g["xyz"]), patch_size=256, host_only=True)
    b = rx.get_boundary_vertices()
    assert b.is_cuda and int(b.sum().item()) == 98
    assert np.array_equal(b.cpu().numpy(), host.get_boundary_vertices())


@pytest.mark.parametrize("name", ["torus64", "icosphere4", "plane", "sphere3", "plane_5"])
def test_edge_edge_query(oracle, name):
    """Op.EE (e_e_manifold, rxmesh_queries.cuh:269-340) on the GPU
    (k_query_elem<RXG_OP_EE>) against the oracle, also into host arrays;
    refused on a mesh whose faces are not consistently oriented."""
    from rxmesh_gb300 import Op, RXGError, RXMeshStatic
    x, f = MESHES[name]()
    rx = RXMeshStatic(f, len(x), patch_size=64)
    _, ee = rx.query(Op.EE)
    assert ee.is_cuda
    el = rx.linear_to_input("e")
    ee = ee.cpu().numpy().reshape(-1, 4)
    got = np.where(ee >= 0, el[np.maximum(ee, 0)], -1)[np.argsort(el)]
    assert np.array_equal(got, oracle.ee(f))
    host = np.full(4 * rx.get_num_edges(), -7, np.int32)
    rx.query_host(Op.EE, None, host)
    assert np.array_equal(host.reshape(-1, 4), ee)
    g = np.array(f, np.int32).copy()
    g[3] = g[3][::-1]
    with pytest.raises(RXGError):
        RXMeshStatic(g, len(x), patch_size=64).query(Op.EE)


def test_bounded_wait_reports_and_context_survives():
    """A device wait that can never complete gives up, sets the error word
    (rxg_device_check -> RXG_ERR_DEVICE_TIMEOUT, then cleared) and leaves the
    context usable: no fault, trap or hang is involved."""
    from rxmesh_gb300 import Op, RXGError, RXMeshStatic, _lib, device_check
    L = _lib.load()
    device_check()
    _lib.check(L.rxg_selftest_bounded_wait(None))
    with pytest.raises(RXGError) as e:
        device_check()
    assert e.value.status == 7 and "timed out" in str(e.value)
    device_check()  # cleared
    x, f = meshgen.icosphere(2)
    off, val = RXMeshStatic(f, len(x), patch_size=64).query(Op.VV)
    assert int(off[-1].item()) == val.numel()
