"""ctypes wrapper over oracle/_build/liboracle.so (the CPU restatement).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
legs are the only users.  Every function documents the reference routine it
restates in rxg_oracle.c.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
I64 = ctypes.c_int64


def build(ref_root=None):
    """Compile the oracle; with ref_root (an RXMesh source tree) also the
    reference's own routines into oracle/_ref."""
    cmd = ["make", "-s", "-C", _HERE]
    if ref_root:
        cmd.append("REF=" + ref_root)
    subprocess.check_call(cmd, stdout=subprocess.DEVNULL)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_build_edges.restype = I64
        L.orc_build_edges.argtypes = [I64, i32p, i32p, i32p]
        L.orc_vv_ve.argtypes = [I64, I64, i32p, ctypes.c_int, i64p, i32p]
        L.orc_vf.argtypes = [I64, I64, i32p, i64p, i32p]
        L.orc_ef.argtypes = [I64, I64, i32p, i64p, i32p]
        L.orc_ff.restype = I64
        L.orc_ff.argtypes = [I64, I64, i64p, i32p, i64p, ctypes.c_void_p]
        L.orc_ev_diamond.argtypes = [I64, I64, i32p, i32p, i32p, i32p]
        L.orc_vertex_normals.argtypes = [I64, I64, i32p, f64p, ctypes.c_int, f64p]
        L.orc_oriented_vv.restype = ctypes.c_int
        L.orc_oriented_vv.argtypes = [I64, i32p, i64p, i32p, i64p, i32p, i8p]
        L.orc_mcf_assemble.argtypes = [I64, i64p, i32p, i8p, f64p, ctypes.c_double,
                                       i64p, i32p, f64p, f64p]
        L.orc_cg.restype = ctypes.c_int
        L.orc_cg.argtypes = [I64, ctypes.c_int, i64p, i32p, f64p, f64p, f64p,
                             ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double)]
        L.orc_spmm.argtypes = [I64, ctypes.c_int, i64p, i32p, f64p, f64p, f64p]
        L.orc_rest_frame.argtypes = [I64, i32p, f64p, f64p, f64p]
        L.orc_arap_face.restype = ctypes.c_double
        L.orc_arap_face.argtypes = [f64p, f64p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_arap_assemble.restype = ctypes.c_double
        L.orc_arap_assemble.argtypes = [I64, I64, i32p, f64p, f64p, f64p, i64p, i32p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_arap_assemble_ex.restype = ctypes.c_double
        L.orc_arap_assemble_ex.argtypes = [I64, I64, i32p, f64p, f64p, f64p, i64p, i32p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_double]
        L.orc_project_pd.argtypes = [ctypes.c_int, f64p, ctypes.c_double]
        L.orc_partial_voronoi_area.restype = ctypes.c_double
        L.orc_partial_voronoi_area.argtypes = [f64p, f64p, f64p]
        L.orc_half_cot.restype = ctypes.c_double
        L.orc_half_cot.argtypes = [f64p, f64p, f64p]
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's own vertex_normal_ref compiled from its source, or None."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libref_normals.so")
        if not os.path.exists(path):
            return None
        try:
            R = ctypes.CDLL(path)
        except OSError:
            return None
        R.ref_vertex_normal_f32.argtypes = [I64, I64, i32p, f32p, f32p]
        R.ref_vertex_normal_f64.argtypes = [I64, I64, i32p, f64p, f64p]
        _REF = R
    return _REF


_GEO = None


def ref_geometry():
    """The reference's own geometry_util.cuh cotangent / Voronoi routines
    compiled from its source into oracle/_ref, or None."""
    global _GEO
    if _GEO is None:
        path = os.path.join(_HERE, "_ref", "libref_geometry.so")
        if not os.path.exists(path):
            return None
        try:
            R = ctypes.CDLL(path)
        except OSError:
            return None
        for t, p in (("f64", f64p), ("f32", f32p)):
            getattr(R, "ref_partial_voronoi_area_" + t).argtypes = [I64, p, p, p, p]
            getattr(R, "ref_edge_cotan_weight_" + t).argtypes = [I64, p, p, p, p, p]
        R.ref_tri_area_f64.argtypes = [I64, f64p, f64p, f64p, f64p]
        _GEO = R
    return _GEO


def partial_voronoi_area(P, Q, R):
    """Oracle restatement of partial_voronoi_area (geometry_util.cuh:117-167),
    row by row over (n, 3) arrays."""
    L = lib()
    P, Q, R = (np.ascontiguousarray(a, np.float64) for a in (P, Q, R))
    return np.array([L.orc_partial_voronoi_area(P[i], Q[i], R[i]) for i in range(len(P))])


def edge_cotan_weight(P, R, Q, S):
    """Oracle restatement of edge_cotan_weight (geometry_util.cuh:173-206):
    the two half-cotangents of edge p-r opposite q and s."""
    L = lib()
    P, R, Q, S = (np.ascontiguousarray(a, np.float64) for a in (P, R, Q, S))
    return np.array([L.orc_half_cot(P[i], R[i], Q[i]) + L.orc_half_cot(P[i], R[i], S[i])
                     for i in range(len(P))])


def _fv(fv):
    return np.ascontiguousarray(fv, dtype=np.int32).reshape(-1)


def edges(fv):
    """Reference edge numbering (rxmesh.cpp:518-620). Returns (ev[ne,2], fe[nf,3])."""
    f = _fv(fv)
    nf = f.size // 3
    ev = np.empty(6 * nf, np.int32)
    fe = np.empty(3 * nf, np.int32)
    ne = lib().orc_build_edges(nf, f, ev, fe)
    if ne < 0:
        raise MemoryError("oracle edge map")
    return ev[: 2 * ne].reshape(-1, 2).copy(), fe.reshape(-1, 3)


def vv(nv, ev, want_edges=False):
    """Sorted VV (or VE) rows as CSR (off int64[nv+1], val int32)."""
    e = np.ascontiguousarray(ev, np.int32).reshape(-1)
    off = np.empty(nv + 1, np.int64)
    val = np.empty(e.size, np.int32)
    lib().orc_vv_ve(nv, e.size // 2, e, int(want_edges), off, val)
    return off, val


def vf(nv, fv):
    """Sorted VF rows as CSR."""
    f = _fv(fv)
    off = np.empty(nv + 1, np.int64)
    val = np.empty(f.size, np.int32)
    lib().orc_vf(nv, f.size // 3, f, off, val)
    return off, val


def ef(fv):
    """Sorted EF rows as CSR over the reference edge numbering (edges(fv))."""
    f = _fv(fv)
    ev, fe = edges(fv)
    off = np.empty(len(ev) + 1, np.int64)
    val = np.empty(f.size, np.int32)
    lib().orc_ef(len(ev), f.size // 3, np.ascontiguousarray(fe, np.int32).reshape(-1), off, val)
    return off, val


def ff(fv):
    """Sorted FF rows (faces sharing an edge) as CSR."""
    f = _fv(fv)
    nf = f.size // 3
    eoff, eval_ = ef(fv)
    off = np.empty(nf + 1, np.int64)
    n = lib().orc_ff(nf, len(eoff) - 1, eoff, eval_, off, None)
    val = np.empty(max(n, 1), np.int32)
    lib().orc_ff(nf, len(eoff) - 1, eoff, eval_, off, val.ctypes.data)
    return off, val[:n]


def ev_diamond(fv):
    """EVDiamond rows (ne, 4): [v0, opposite in the v0->v1 face, v1, opposite in the v1->v0 face], -1 = none."""
    f = _fv(fv)
    ev, fe = edges(fv)
    out = np.empty(4 * len(ev), np.int32)
    lib().orc_ev_diamond(len(ev), f.size // 3, f, np.ascontiguousarray(ev, np.int32).reshape(-1),
                         np.ascontiguousarray(fe, np.int32).reshape(-1), out)
    return out.reshape(-1, 4)


def ee(fv):
    """EE rows (ne, 4) in input edge ids, restating e_e_manifold
    (include/rxmesh/kernels/rxmesh_queries.cuh:269-340) on an edge-manifold,
    consistently oriented mesh: for the face that traverses edge e in
    direction d (0: from its first vertex, as numbered by edges()), slot
    2d holds the face's next edge and slot 2d+1 its previous edge; -1 where
    e has no such face.  (The reference computes the previous edge's index
    as (cur - 1) % 3, which is -1 for the first edge in C++; the previous
    edge is (cur + 2) % 3.)  Every face corner k writes the slots of its
    edge k (vectorised; one writer per slot on such a mesh)."""
    f = np.asarray(fv, np.int64)
    ev, fe = edges(fv)
    ev, fe = np.asarray(ev, np.int64), np.asarray(fe, np.int64)
    out = np.full((len(ev), 4), -1, np.int32)
    d = (f != ev[fe][..., 0]).astype(np.int64)  # (nf, 3): direction of edge k in face
    slot = 4 * fe + 2 * d
    out.reshape(-1)[slot.reshape(-1)] = np.roll(fe, -1, axis=1).reshape(-1)
    out.reshape(-1)[(slot + 1).reshape(-1)] = np.roll(fe, 1, axis=1).reshape(-1)
    return out


def vertex_normals(fv, xyz, weighting=0):
    """weighting 0 = Max weights (vertex_normal_ref.h), 1 = area weights."""
    f = _fv(fv)
    x = np.ascontiguousarray(xyz, np.float64).reshape(-1)
    out = np.empty_like(x)
    lib().orc_vertex_normals(x.size // 3, f.size // 3, f, x, int(weighting), out)
    return out.reshape(-1, 3)


def ref_vertex_normals(fv, xyz, dtype=np.float32):
    """Run the reference's own vertex_normal_ref, if compiled here."""
    R = ref_lib()
    if R is None:
        return None
    f = _fv(fv)
    x = np.ascontiguousarray(xyz, dtype).reshape(-1)
    out = np.empty_like(x)
    fn = R.ref_vertex_normal_f32 if dtype == np.float32 else R.ref_vertex_normal_f64
    fn(x.size // 3, f.size // 3, f, x, out)
    return out.reshape(-1, 3)


def oriented_vv(nv, fv):
    """Oriented one-ring CSR + boundary flags (rxmesh_queries.cuh:376-499)."""
    f = _fv(fv)
    voff, vval = vf(nv, f)
    off = np.empty(nv + 1, np.int64)
    val = np.empty(2 * f.size, np.int32)  # 2E <= 6F (open meshes have 2E > 3F)
    bnd = np.empty(nv, np.int8)
    rc = lib().orc_oriented_vv(nv, f, voff, vval, off, val, bnd)
    if rc != 0:
        raise ValueError("non-manifold vertex fan")
    return off, val[: off[-1]].copy(), bnd


def mcf_system(fv, xyz, dt, ring=None):
    """(row_ptr, col, val, B) of the MCF system (mcf_kernels.cuh:302-426)."""
    x = np.ascontiguousarray(xyz, np.float64).reshape(-1)
    nv = x.size // 3
    if ring is None:
        ring = oriented_vv(nv, fv)
    off, rv, bnd = ring
    nnz = int(off[-1]) + nv
    rp = np.empty(nv + 1, np.int64)
    col = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float64)
    B = np.empty(3 * nv, np.float64)
    lib().orc_mcf_assemble(nv, off, np.ascontiguousarray(rv, np.int32), bnd, x,
                           float(dt), rp, col, val, B)
    return rp, col, val, B.reshape(-1, 3)


def cg(rp, col, val, B, X0, max_iter=1000, abs_tol=1e-6, rel_tol=0.0, precond=False):
    """CGSolver/PCGSolver recurrence (cg_solver.h:37-125, pcg_solver.h:34-144).

    Returns (X, iters, start_res, final_res, converged)."""
    Bm = np.ascontiguousarray(B, np.float64)
    nc = Bm.shape[1] if Bm.ndim == 2 else 1
    n = rp.size - 1
    X = np.ascontiguousarray(X0, np.float64).reshape(-1).copy()
    it = ctypes.c_int(0)
    r0 = ctypes.c_double(0)
    r1 = ctypes.c_double(0)
    conv = lib().orc_cg(n, nc, np.ascontiguousarray(rp, np.int64), np.ascontiguousarray(col, np.int32),
                        np.ascontiguousarray(val, np.float64), Bm.reshape(-1), X, int(max_iter),
                        float(abs_tol), float(rel_tol), int(bool(precond)),
                        ctypes.byref(it), ctypes.byref(r0), ctypes.byref(r1))
    return X.reshape(Bm.shape), it.value, r0.value, r1.value, bool(conv)


def spmm(rp, col, val, X):
    Xm = np.ascontiguousarray(X, np.float64)
    nc = Xm.shape[1] if Xm.ndim == 2 else 1
    Y = np.empty_like(Xm).reshape(-1)
    lib().orc_spmm(rp.size - 1, nc, np.ascontiguousarray(rp, np.int64),
                   np.ascontiguousarray(col, np.int32), np.ascontiguousarray(val, np.float64),
                   Xm.reshape(-1), Y)
    return Y.reshape(Xm.shape)


def rest_frame(fv, xyz_rest):
    """Per-face Mr^{-1} (nf,2,2) and rest area (param.cu:113-141)."""
    f = _fv(fv)
    x = np.ascontiguousarray(xyz_rest, np.float64).reshape(-1)
    nf = f.size // 3
    minv = np.empty(4 * nf, np.float64)
    area = np.empty(nf, np.float64)
    lib().orc_rest_frame(nf, f, x, minv, area)
    return minv.reshape(nf, 2, 2), area


def arap_face(x9, minv, area, want_hess=True):
    x = np.ascontiguousarray(x9, np.float64).reshape(9)
    m = np.ascontiguousarray(minv, np.float64).reshape(4)
    g = np.empty(9, np.float64)
    H = np.empty(81, np.float64)
    E = lib().orc_arap_face(x, m, float(area), g.ctypes.data, H.ctypes.data if want_hess else None)
    return E, g, H.reshape(9, 9)


def project_pd(H, eps=1e-9):
    """project_positive_definite of one symmetric k x k matrix (copy)."""
    h = np.ascontiguousarray(H, np.float64).copy()
    lib().orc_project_pd(h.shape[0], h.reshape(-1), float(eps))
    return h


def arap_assemble(fv, x, minv, area, rp, col, want_hess=True, project=False, eps=1e-9):
    """Total energy, per-face energy, gradient (nv,3), Hessian blocks (nnz,3,3);
    project: each face's 9x9 Hessian made positive definite first."""
    f = _fv(fv)
    xx = np.ascontiguousarray(x, np.float64).reshape(-1)
    nv = xx.size // 3
    nf = f.size // 3
    fe = np.empty(nf, np.float64)
    g = np.empty(3 * nv, np.float64)
    nnz = int(rp[-1])
    H = np.empty(9 * nnz, np.float64) if want_hess else None
    E = lib().orc_arap_assemble_ex(nv, nf, f, xx, np.ascontiguousarray(minv, np.float64).reshape(-1),
                                   np.ascontiguousarray(area, np.float64), np.ascontiguousarray(rp, np.int64),
                                   np.ascontiguousarray(col, np.int32), fe.ctypes.data, g.ctypes.data,
                                   H.ctypes.data if want_hess else None, int(project), float(eps))
    return E, fe, g.reshape(nv, 3), (H.reshape(nnz, 3, 3) if want_hess else None)


def symmetric_dirichlet(fv, uv, rest_minv):
    """Per-face symmetric Dirichlet energy of apps/Param/param.cu:146-183:
    M = [b - a, c - a] of the uv positions (nv, 2), J = M Mr^{-1} with the
    face's rest-frame inverse rest_minv (nf, 4, row-major, as rest_frame
    returns it), A = det(Mr) / 2, E = A (|J|_F^2 + |J^{-1}|_F^2); +inf-like
    (the largest double) where det(M) <= 0.  FP64, vectorised over faces."""
    f = np.asarray(fv, np.int64)
    a, b, c = uv[f[:, 0]], uv[f[:, 1]], uv[f[:, 2]]
    M = np.stack([b - a, c - a], axis=2)  # columns: edge vectors
    mi = np.asarray(rest_minv, np.float64).reshape(-1, 2, 2)
    A = 0.5 / np.linalg.det(mi)
    J = M @ mi
    dM = np.linalg.det(M)
    Ji = np.linalg.inv(np.where(dM[:, None, None] > 0, J, np.eye(2)))
    E = A * ((J ** 2).sum((1, 2)) + (Ji ** 2).sum((1, 2)))
    return np.where(dM > 0, E, np.finfo(np.float64).max)
