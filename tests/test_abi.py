"""CPU tests of librxg.so: exports, host-side mesh build and patch layout.

No compute kernel runs here; the patch arena is decoded on the CPU and the
queries it encodes are compared bit-exactly with the oracle."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, edge_case_meshes, golden, sorted_rows
from rxmesh_gb300 import meshgen


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "rxg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return set(re.findall(r"\b(rxg_[a-z0-9_]+)\s*\(", txt))


def test_library_exports_every_declared_symbol():
    from rxmesh_gb300 import _lib
    import ctypes
    L = ctypes.CDLL(_lib.load().__dict__["_name"])
    missing = [s for s in sorted(header_symbols()) if not hasattr(L, s)]
    assert not missing, missing
    assert header_symbols() <= set(_lib.SIGNATURES), "bindings lag the header"


def test_invalid_arguments_return_status():
    import ctypes
    from rxmesh_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    bad = np.array([[0, 1, 5]], np.int32)
    assert L.rxg_mesh_create_ex(bad.ctypes.data, 1, 3, 64, 1, ctypes.byref(h)) == 1
    assert b"outside" in L.rxg_last_error()
    rep = np.array([[0, 1, 1]], np.int32)
    assert L.rxg_mesh_create_ex(rep.ctypes.data, 1, 3, 64, 1, ctypes.byref(h)) == 1
    ok = np.array([[0, 1, 2]], np.int32)
    assert L.rxg_mesh_create_ex(ok.ctypes.data, 1, 3, 8, 1, ctypes.byref(h)) == 1  # patch too small
    assert L.rxg_status_string(6) == b"RXG_ERR_NOT_CONVERGED"


def test_newton_and_matfree_entry_points_reject_bad_arguments():
    """The Newton-step helpers and the matrix-free solver return
    RXG_ERR_INVALID with a message, without touching a GPU, on NULL or host
    arguments and on a requested preconditioner."""
    import ctypes
    from rxmesh_gb300 import RXMeshStatic, _lib
    L = _lib.load()
    assert L.rxg_bcsr_to_csr(None, None, None) == 1
    assert b"rxg_bcsr_to_csr" in L.rxg_last_error()
    assert L.rxg_bcsr_apply_bc(None, None, None, None) == 1
    _, f = meshgen.icosphere(1)
    rx = RXMeshStatic(f, int(np.max(f)) + 1, patch_size=64, host_only=True)
    x = np.zeros((rx.get_num_vertices(), 3))
    o = _lib.SolverOpts(10, 0.0, 1e-12, 1)
    st = L.rxg_arap_cg_matfree(rx._h, 1, x.ctypes.data, x.ctypes.data, 0, None,
                               x.ctypes.data, x.ctypes.data, ctypes.byref(o), None, None)
    assert st == 1 and b"device arrays" in L.rxg_last_error()
    assert L.rxg_arap_hvp(rx._h, 1, x.ctypes.data, x.ctypes.data, 0, None, None, None, None) == 1


def test_dense_and_partition_entry_points_reject_bad_arguments(tmp_path):
    """rxg_dense_*, the partition and patch-file calls: RXG_ERR_INVALID with a
    message on NULL, host or inconsistent arguments, without a GPU."""
    import ctypes
    from rxmesh_gb300 import RXMeshStatic, _lib
    L = _lib.load()
    x = np.zeros(12)
    out = ctypes.c_double()
    assert L.rxg_dense_axpby(12, 1, 1.0, x.ctypes.data, 1.0, x.ctypes.data, None) == 1
    assert b"device arrays" in L.rxg_last_error()
    assert L.rxg_dense_axpby(12, 1, 1.0, None, 1.0, x.ctypes.data, None) == 1  # x NULL, a != 0
    assert L.rxg_dense_axpby(12, 7, 0.0, None, 1.0, x.ctypes.data, None) == 1  # bad dtype
    assert L.rxg_dense_dot(12, 1, x.ctypes.data, x.ctypes.data, ctypes.byref(out), None) == 1
    assert L.rxg_dense_dot(12, 1, None, x.ctypes.data, ctypes.byref(out), None) == 1
    mask = np.zeros(4, np.int8)
    assert L.rxg_dense_zero_rows(4, 3, 1, mask.ctypes.data, x.ctypes.data, None) == 1
    assert b"device arrays" in L.rxg_last_error()
    assert L.rxg_dense_zero_rows(4, 0, 1, mask.ctypes.data, x.ctypes.data, None) == 1  # no columns
    assert L.rxg_query_sweep_ex(None, None, 1, None) == 1
    for fn in (L.rxg_edge_term_gather, L.rxg_vertex_term_gather, L.rxg_face_term_gather):
        assert fn(None, 1, 3, x.ctypes.data, 0, None, None, None, None, None) == 1      # no mesh
    assert L.rxg_edge_term_gather(None, 1, 4, x.ctypes.data, 0, None, None, None, None, None) == 1
    assert L.rxg_mesh_partition(None, None, None, None) == 1
    _, f = meshgen.icosphere(1)
    f = np.ascontiguousarray(f, np.int32)
    nv = int(f.max()) + 1
    h = ctypes.c_void_p()
    fp = np.zeros(len(f), np.int32)
    assert L.rxg_mesh_create_partitioned(f.ctypes.data, len(f), nv, None, None, None, -1, 1,
                                         ctypes.byref(h)) == 1          # no face_patch
    assert L.rxg_mesh_create_partitioned(f.ctypes.data, len(f), nv, fp.ctypes.data, None, None,
                                         -1, 3, ctypes.byref(h)) == 1   # split flag
    assert L.rxg_mesh_create_partitioned(f.ctypes.data, len(f), nv, fp.ctypes.data, None,
                                         fp.ctypes.data, -1, 1, ctypes.byref(h)) == 1  # ne < 0
    assert L.rxg_mesh_create_from_patch_file(f.ctypes.data, len(f), nv, None, 1,
                                             ctypes.byref(h)) == 1
    rx = RXMeshStatic(f, nv, patch_size=64, host_only=True)
    assert L.rxg_mesh_save_patch_file(rx._h, None) == 1
    assert L.rxg_mesh_save_patch_file(rx._h, str(tmp_path / "no" / "such" / "dir").encode()) == 1
    assert b"cannot create" in L.rxg_last_error()


def decode(rx):
    """Per-patch decoding of the arena into linear-id queries (CPU)."""
    hdr, arena = rx.patches()
    nv, ne, nf = rx.get_num_vertices(), rx.get_num_edges(), rx.get_num_faces()
    vv = [None] * nv
    ve = [None] * nv
    vf = [None] * nv
    fvq = np.full((nf, 3), -1, np.int64)
    evq = np.full((ne, 2), -1, np.int64)
    ef = [None] * ne
    ff = [None] * nf
    feq = np.full((nf, 3), -1, np.int64)
    evd = np.full((ne, 4), -2, np.int64)
    ee = np.full((ne, 4), -2, np.int64)
    for h in hdr:
        nVo, nVl, nEo, nEl, nFo, nFl, vb, eb, fb, vvb, vfb, evo, feo, rvo, reo, rfo = h.tolist()
        ev = arena[evo:evo + nEl]
        a, b = (ev & 0xFFFF).astype(np.int64), (ev >> 16).astype(np.int64)
        fe = arena[feo:feo + (3 * nFl + 1) // 2 + 4].view(np.uint16)[:3 * nFl].reshape(-1, 3).astype(np.int64)
        rv = arena[rvo:rvo + nVl - nVo].astype(np.int64)
        re_ = arena[reo:reo + nEl - nEo].astype(np.int64)
        rf = arena[rfo:rfo + nFl - nFo].astype(np.int64)
        linv = lambda l: np.where(l < nVo, vb + l, rv[np.maximum(l - nVo, 0)] if rv.size else 0)
        line = lambda l: np.where(l < nEo, eb + l, re_[np.maximum(l - nEo, 0)] if re_.size else 0)
        linf = lambda l: np.where(l < nFo, fb + l, rf[np.maximum(l - nFo, 0)] if rf.size else 0)
        fvl = np.where(fe & 1, b[fe >> 1], a[fe >> 1])
        for v in range(nVo):
            m1, m2 = a == v, b == v
            vv[vb + v] = sorted(linv(np.concatenate([b[m1], a[m2]])).tolist())
            ve[vb + v] = sorted(line(np.concatenate([np.nonzero(m1)[0], np.nonzero(m2)[0]])).tolist())
            vf[vb + v] = sorted(linf(np.nonzero((fvl == v).any(1))[0]).tolist())
        if nFo:
            fvq[fb:fb + nFo] = linv(fvl[:nFo])
        if nEo:
            evq[eb:eb + nEo] = np.stack([linv(a[:nEo]), linv(b[:nEo])], 1)
        # edge / face queries from the same slices: every face of an owned
        # edge and every edge neighbour of an owned face must be local
        fel = fe >> 1
        for e in range(nEo):
            ef[eb + e] = sorted(linf(np.nonzero((fel == e).any(1))[0]).tolist())
            d = [linv(np.array([a[e]]))[0], -1, linv(np.array([b[e]]))[0], -1]
            for f, k in zip(*np.nonzero(fel == e)):
                d[1 + 2 * int(fe[f, k] & 1)] = int(linv(np.array([fvl[f, (k + 2) % 3]]))[0])
            evd[eb + e] = d
            # EE: per direction bit of FE, that face's next and previous edge
            q = [-1, -1, -1, -1]
            for f, k in zip(*np.nonzero(fel == e)):
                dd = 2 * int(fe[f, k] & 1)
                q[dd] = int(line(np.array([fel[f, (k + 1) % 3]]))[0])
                q[dd + 1] = int(line(np.array([fel[f, (k + 2) % 3]]))[0])
            ee[eb + e] = q
        for f in range(nFo):
            nb = set()
            for k in range(3):
                nb |= set(np.nonzero((fel == fel[f, k]).any(1))[0].tolist())
            nb.discard(f)
            ff[fb + f] = sorted(linf(np.array(sorted(nb), np.int64)).tolist()) if nb else []
            feq[fb + f] = line(fel[f])
    return vv, ve, vf, fvq, evq, ef, ff, feq, evd, ee


MESHES = {
    "torus": lambda: meshgen.torus(24, 16)[::-1],
    "icosphere": lambda: meshgen.icosphere(3)[::-1],
    "plane": lambda: meshgen.plane(13, 9)[::-1],
    "bunnyhead": lambda: (golden("bunnyhead")["fv"], golden("bunnyhead")["xyz"]),
    "isolated": lambda: edge_case_meshes()["isolated"][::-1],
    "nonmanifold": lambda: edge_case_meshes()["nonmanifold"][::-1],
    "components": lambda: edge_case_meshes()["components"][::-1],
}


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("patch", [32, 512])
def test_patch_layout_encodes_exact_queries(oracle, name, patch):
    from rxmesh_gb300 import RXMeshStatic
    fv, x = MESHES[name]()
    nv = len(x)
    rx = RXMeshStatic(fv, nv, patch_size=patch, host_only=True)
    check_layout(oracle, rx, fv, nv, patch)


def random_mesh(rng):
    """A torus or grid with faces removed (holes, several components),
    some faces flipped, vertex ids permuted, faces shuffled, and a few
    vertices in no face."""
    if rng.random() < 0.5:
        x, f = meshgen.torus(int(rng.integers(6, 14)), int(rng.integers(5, 12)))
    else:
        x, f = meshgen.plane(int(rng.integers(5, 13)), int(rng.integers(4, 12)))
    f = np.asarray(f)
    f = f[rng.random(len(f)) > rng.uniform(0.0, 0.35)]
    flip = rng.random(len(f)) < rng.uniform(0.0, 0.15)
    f[flip] = f[flip][:, ::-1]
    f = f[rng.permutation(len(f))]
    used = np.unique(f)
    extra = int(rng.integers(0, 4))
    perm = rng.permutation(len(used) + extra)
    remap = np.full(int(f.max()) + 1, -1)
    remap[used] = perm[:len(used)]
    return np.ascontiguousarray(remap[f], np.int32), len(used) + extra


def random_partition(rng, fv, nv):
    """Face patches in random order (patches need not be connected), and
    vertex owners picked at random among each vertex's face patches."""
    nf = len(fv)
    k = int(rng.integers(1, max(2, nf // 8)))
    fp = rng.integers(0, k, nf)
    fp[rng.permutation(nf)[:k]] = np.arange(k)          # no empty patch id
    vp = np.full(nv, -1, np.int32)
    for f in rng.permutation(nf):
        for v in fv[f]:
            if vp[v] < 0 or rng.random() < 0.3:
                vp[v] = fp[f]
    return fp.astype(np.int32), vp


@pytest.mark.parametrize("seed", range(12))
def test_random_meshes_and_partitions_encode_exact_queries(oracle, seed):
    """Random holes, flips, vertex permutations and isolated vertices, built
    with the BFS partitioner at three patch sizes and on a random
    (disconnected) partition with random vertex owners: the arena decodes to
    exactly the oracle's queries every time."""
    from rxmesh_gb300 import RXMeshStatic
    rng = np.random.default_rng(seed)
    fv, nv = random_mesh(rng)
    for patch in (16, 64, 512):
        rx = RXMeshStatic(fv, nv, patch_size=patch, host_only=True)
        check_layout(oracle, rx, fv, nv, patch)
    fp, vp = random_partition(rng, fv, nv)
    rx = RXMeshStatic(fv, nv, host_only=True, face_patch=fp, vertex_patch=vp)
    got_fp, got_vp, _ = rx.partition()
    assert np.array_equal(got_fp, fp)
    infaces = np.zeros(nv, bool)
    infaces[fv.reshape(-1)] = True
    assert np.array_equal(got_vp[infaces], vp[infaces])
    check_layout(oracle, rx, fv, nv, 4096)


def check_layout(oracle, rx, fv, nv, patch):
    assert rx.get_num_faces() == len(fv) and rx.get_num_vertices() == nv
    # mesh properties (rxmesh.h:134-220) against the oracle's adjacency
    ef_off, _ = oracle.ef(fv)
    ff_off, _ = oracle.ff(fv)
    assert rx.get_input_max_edge_incident_faces() == np.diff(ef_off).max()
    assert rx.get_input_max_face_adjacent_faces() == np.diff(ff_off).max()
    from oracle.patcher import face_graph
    assert rx.get_num_components() == len(np.unique(face_graph(fv)[2]))
    directed = {(int(t[k]), int(t[(k + 1) % 3])) for t in np.asarray(fv) for k in range(3)}
    assert rx.is_oriented() == (len(directed) == 3 * len(fv))
    ev_ref, _ = oracle.edges(fv)
    assert np.array_equal(rx.input_edges(), ev_ref)  # reference edge numbering
    vl, el, fl = rx.linear_to_input("v"), rx.linear_to_input("e"), rx.linear_to_input("f")
    for m, n in ((vl, nv), (el, len(ev_ref)), (fl, len(fv))):
        assert np.array_equal(np.sort(m), np.arange(n))
    hdr, _ = rx.patches()
    assert (hdr[:, 4] <= patch).all()
    vv, ve, vf, fvq, evq, ef, ff, feq, evd, ee = decode(rx)
    off, val = oracle.vv(nv, ev_ref)
    want = sorted_rows(off, val)
    got = [None] * nv
    for lin in range(nv):
        got[vl[lin]] = tuple(sorted(vl[np.array(vv[lin], np.int64)].tolist()))
    assert got == want
    off, val = oracle.vv(nv, ev_ref, want_edges=True)
    want = sorted_rows(off, val)
    for lin in range(nv):
        got[vl[lin]] = tuple(sorted(el[np.array(ve[lin], np.int64)].tolist()))
    assert got == want
    off, val = oracle.vf(nv, fv)
    want = sorted_rows(off, val)
    for lin in range(nv):
        got[vl[lin]] = tuple(sorted(fl[np.array(vf[lin], np.int64)].tolist()))
    assert got == want
    assert np.array_equal(vl[fvq][np.argsort(fl)], np.asarray(fv))  # FV in input vertex order
    assert np.array_equal(vl[evq][np.argsort(el)], ev_ref)          # EV as first encountered
    ne, nf = len(ev_ref), len(fv)
    off, val = oracle.ef(fv)
    got_e = [None] * ne
    for lin in range(ne):
        got_e[el[lin]] = tuple(sorted(fl[np.array(ef[lin], np.int64)].tolist()))
    assert got_e == sorted_rows(off, val)
    off, val = oracle.ff(fv)
    got_f = [None] * nf
    for lin in range(nf):
        got_f[fl[lin]] = tuple(sorted(fl[np.array(ff[lin], np.int64)].tolist()))
    assert got_f == sorted_rows(off, val)
    _, fe_ref = oracle.edges(fv)
    assert np.array_equal(el[feq][np.argsort(fl)], fe_ref)          # FE in face-edge order
    directed = {(int(t[k]), int(t[(k + 1) % 3])) for t in np.asarray(fv) for k in range(3)}
    oriented = len(directed) == 3 * len(fv)
    # EVDiamond and EE are defined (and run on the GPU) on edge-manifold,
    # consistently oriented meshes
    if rx.info["is_edge_manifold"] and oriented:
        d = np.where(evd >= 0, vl[np.maximum(evd, 0)], -1)[np.argsort(el)]
        assert np.array_equal(d, oracle.ev_diamond(fv))
        # EE: the GPU kernel's slot rule over the same patch slices
        got = np.where(ee >= 0, el[np.maximum(ee, 0)], -1)[np.argsort(el)]
        assert np.array_equal(got, oracle.ee(fv))


def test_ev_diamond_needs_consistent_orientation():
    """One flipped face: the two faces of its edges traverse them the same
    way, so EVDiamond is refused (RXG_ERR_NONMANIFOLD) before any launch."""
    import ctypes
    from rxmesh_gb300 import Op, RXMeshStatic, _lib
    L = _lib.load()
    _, f = meshgen.icosphere(2)
    good = RXMeshStatic(f, f.max() + 1, patch_size=64, host_only=True)
    assert L.rxg_query(good._h, Op.EVD, None, None, None) == 1   # only the NULL buffer
    g = np.array(f, np.int32).copy()
    g[5] = g[5][::-1]
    bad = RXMeshStatic(g, g.max() + 1, patch_size=64, host_only=True)
    assert L.rxg_query(bad._h, Op.EVD, None, None, None) == 4
    assert b"oriented" in L.rxg_last_error()


def test_boundary_vertices_known_answer():
    """RXMesh's own test (tests/RXMesh_test/test_boundary.cu): bunnyhead has
    98 boundary vertices; closed meshes have none; an open grid's border."""
    from conftest import golden
    from rxmesh_gb300 import RXMeshStatic
    g = golden("bunnyhead")
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), patch_size=256, host_only=True)
    b = rx.get_boundary_vertices()
    assert b.dtype == np.int8 and int(b.sum()) == 98
    # the same set from the edge face counts, in input ids
    ev, fe = meshgen_edges(g["fv"])
    cnt = np.bincount(fe.reshape(-1), minlength=len(ev))
    want = np.zeros(len(g["xyz"]), np.int8)
    want[ev[cnt < 2].reshape(-1)] = 1
    assert np.array_equal(b[rx.input_to_linear("v")], want)
    _, f = meshgen.icosphere(2)
    assert RXMeshStatic(f, int(np.max(f)) + 1, patch_size=64,
                        host_only=True).get_boundary_vertices().sum() == 0
    x, f = meshgen.plane(7, 5)
    assert RXMeshStatic(f, len(x), patch_size=64, host_only=True).get_boundary_vertices().sum() == 2 * (7 + 5) - 4


def meshgen_edges(fv):
    """Edge list in first-appearance order and each face's three edge ids."""
    ids, ev, fe = {}, [], []
    for t in np.asarray(fv):
        row = []
        for k in range(3):
            a, b = int(t[k]), int(t[(k + 1) % 3])
            key = (min(a, b), max(a, b))
            if key not in ids:
                ids[key] = len(ev)
                ev.append((a, b))
            row.append(ids[key])
        fe.append(row)
    return np.array(ev), np.array(fe)


def diag_first_csr(M):
    """scipy CSR -> (row_ptr, col, val) with each row's diagonal first."""
    M = M.tocsr()
    M.sort_indices()
    rp, col, val = M.indptr.copy(), M.indices.copy(), M.data.copy()
    for i in range(M.shape[0]):
        seg = slice(rp[i], rp[i + 1])
        c, v = col[seg].copy(), val[seg].copy()
        o = np.argsort(c != i, kind="stable")
        col[seg], val[seg] = c[o], v[o]
    return rp, col, val


def test_sparse_matrix_user_managed_and_transpose():
    """SparseMatrix from user CSR arrays and A(i, j) (the reference's
    SparseMatrixUserManaged test, test_sparse_matrix.cu:244-323), and
    transpose (SparseMatrixTranspose, :325-367), on CPU tensors."""
    sp = pytest.importorskip("scipy.sparse")
    import torch
    from rxmesh_gb300 import SparseMatrix
    rng = np.random.default_rng(3)
    # 10 x 10 from 20 random triplets, duplicates summed (Eigen setFromTriplets)
    r, c, v = rng.integers(0, 10, 20), rng.integers(0, 10, 20), rng.random(20)
    E = sp.coo_matrix((v, (r, c)), shape=(10, 10)).tocsr()
    E.sum_duplicates()
    rp, col, val = diag_first_csr(E)
    A = SparseMatrix(row_ptr=torch.tensor(rp, dtype=torch.int32), col=torch.tensor(col, dtype=torch.int32),
                     val=torch.tensor(val))
    assert (A.rows(), A.cols(), A.non_zeros()) == (10, 10, E.nnz)
    D = E.toarray()
    for i in range(10):
        for j in range(10):
            assert abs(A(i, j) - D[i, j]) <= 1e-12
    # transpose of a symmetric-pattern, diagonal-first matrix (the VV pattern)
    _, f = meshgen.icosphere(2)
    nv = int(np.max(f)) + 1
    P = sp.coo_matrix((np.ones(3 * len(f)), (np.asarray(f)[:, [0, 1, 2]].reshape(-1),
                                              np.asarray(f)[:, [1, 2, 0]].reshape(-1))),
                      shape=(nv, nv))
    P = ((P + P.T) > 0).astype(float) + sp.eye(nv)
    P.data = rng.random(P.nnz)  # random values on the pattern, not symmetric
    rp, col, val = diag_first_csr(P)
    A = SparseMatrix(row_ptr=torch.tensor(rp, dtype=torch.int32), col=torch.tensor(col, dtype=torch.int32),
                     val=torch.tensor(val))
    T = A.transpose()
    assert abs(T.to_scipy() - P.T.tocsr()).max() == 0
    trp, tcol = T.row_ptr.numpy(), T.col.numpy()
    assert all(tcol[trp[i]] == i for i in range(nv))  # diagonal first
    assert abs(T.transpose().to_scipy() - P.tocsr()).max() == 0
