"""rxmesh_gb300: GB300-native RXMesh hot path (host-side mirror of the reference API).

Names follow the reference: RXMeshStatic (include/rxmesh/rxmesh_static.h),
Op (include/rxmesh/types.h), SparseMatrix (matrix/sparse_matrix.h), CGSolver /
PCGSolver (matrix/cg_solver.h, pcg_solver.h).  All compute goes through the C
ABI of librxg.so (include/rxg.h); device memory and streams come from torch.
"""
import ctypes
import os

import numpy as np
import torch

from . import _lib
from ._lib import RXGError, check

__all__ = ["Op", "RXMeshStatic", "SparseMatrix", "CGSolver", "PCGSolver", "RXGError",
           "DiffScalarProblem", "BlockSparseMatrix", "NewtonSolver", "mcf_step", "MeshBatch",
           "device_check"]


class Op:
    """Query operations (RXMesh's Op enum, include/rxmesh/types.h).  EVD is
    Op::EVDiamond.  CSR (offsets + values): VV, VE, VF, EF, FF; fixed rows:
    FV (3), EV (2), FE (3), EVD (4, -1 where the edge has no such face),
    EE (4, -1 likewise: per direction the next and previous edge of the face
    traversing the edge that way)."""
    VV, VE, VF, FV, EV, EF, FE, FF, EVD, EE = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9
    NAMES = {"VV": 0, "VE": 1, "VF": 2, "FV": 3, "EV": 4, "EF": 5, "FE": 6, "FF": 7, "EVD": 8,
             "EE": 9}
    CSR = (0, 1, 2, 5, 7)


_ELEM = {"v": 0, "vertex": 0, "e": 1, "edge": 1, "f": 2, "face": 2}
_DT = {torch.float32: 0, torch.float64: 1}


def _stream(stream=None):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def device_check(stream=None):
    """Sync and read the device error word (rxg_device_check)."""
    L = _lib.load()
    check(L.rxg_device_check(_stream(stream)))


class RXMeshStatic:
    """Static triangle mesh split into patches (RXMeshStatic, rxmesh_static.h:61-100).

    fv: (nf, 3) int array of input vertex ids.  patch_size: faces per patch.
    The patch topology lives on the current CUDA device unless host_only.
    patcher_file: a partition that RXMesh (or save()) wrote; face_patch
    (nf,), with optional vertex_patch (nv,) and edge_patch (ne,) owners: a
    partition given as arrays (rxg_mesh_create_partitioned).  Either replaces
    the library's own partition and patch_size.  gpu_patcher: partition on
    the GPU with Lloyd region growing (RXMesh's patcher) instead of the host
    BFS partitioner.
    """

    def __init__(self, fv, num_vertices=None, patch_size=512, host_only=False,
                 patcher_file=None, face_patch=None, vertex_patch=None, edge_patch=None,
                 gpu_patcher=False):
        L = _lib.load()
        f = np.ascontiguousarray(fv, dtype=np.int32).reshape(-1, 3)
        nv = int(f.max()) + 1 if num_vertices is None else int(num_vertices)
        self._fv = f
        h = ctypes.c_void_p()
        flags = 1 if host_only else 0
        if sum(x is not None and x is not False for x in (patcher_file, face_patch, gpu_patcher)) > 1:
            raise ValueError("give at most one of patcher_file, face_patch and gpu_patcher")
        if patcher_file is not None:
            check(L.rxg_mesh_create_from_patch_file(f.ctypes.data, f.shape[0], nv,
                                                    os.fsencode(patcher_file), flags,
                                                    ctypes.byref(h)))
        elif face_patch is not None:
            arr = [None if a is None else np.ascontiguousarray(a, dtype=np.int32).reshape(-1)
                   for a in (face_patch, vertex_patch, edge_patch)]
            if len(arr[0]) != f.shape[0] or (arr[1] is not None and len(arr[1]) != nv):
                raise ValueError("face_patch needs one entry per face, vertex_patch one per vertex")
            ptr = [None if a is None else a.ctypes.data for a in arr]
            ne = -1 if arr[2] is None else len(arr[2])
            check(L.rxg_mesh_create_partitioned(f.ctypes.data, f.shape[0], nv, ptr[0], ptr[1],
                                                ptr[2], ne, flags, ctypes.byref(h)))
        else:
            if gpu_patcher:
                flags |= 4  # RXG_MESH_GPU_PATCHER
            check(L.rxg_mesh_create_ex(f.ctypes.data, f.shape[0], nv, int(patch_size), flags,
                                       ctypes.byref(h)))
        self._h = h
        self._L = L
        self.host_only = host_only
        info = _lib.MeshInfo()
        check(L.rxg_mesh_get_info(h, ctypes.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in info._fields_}
        self._maps = {}
        self._dmaps = {}

    @classmethod
    def from_obj(cls, path, patcher_file=None, patch_size=512, **kw):
        """RXMeshStatic(file_path, patcher_file, patch_size)
        (rxmesh_static.h:61-66): the mesh of an OBJ file (polygons fanned
        into triangles).  The positions (float64, input order) are kept as
        input_vertex_coordinates."""
        from .meshgen import read_obj
        xyz, fv = read_obj(path)
        rx = cls(fv, len(xyz), patch_size=patch_size, patcher_file=patcher_file, **kw)
        rx.input_vertex_coordinates = xyz
        return rx

    @classmethod
    def from_objs(cls, paths, patch_size=512, **kw):
        """RXMeshStatic(files_path, patch_size) (rxmesh_static.cu:66-160):
        several OBJ files as one mesh of disjoint regions, file after file;
        get_region_label() gives each element's file index."""
        from .meshgen import read_obj
        xs, fs, fends, vends = [], [], [], []
        base = 0
        for p in paths:
            x, f = read_obj(p)
            xs.append(x)
            fs.append(f + base)
            base += len(x)
            fends.append(sum(len(g) for g in fs))
            vends.append(base)
        if not paths:
            raise ValueError("no files")
        rx = cls(np.concatenate(fs), base, patch_size=patch_size, **kw)
        rx.input_vertex_coordinates = np.concatenate(xs)
        rx._regions = (np.array(fends), np.array(vends))
        return rx

    def get_num_regions(self):
        r = getattr(self, "_regions", None)
        return 1 if r is None else len(r[0])

    def get_region_label(self, elem="f"):
        """Region (file) index of every face / vertex / edge, input ids
        (get_face_region_label and the like, rxmesh_static.h:826-849)."""
        r = getattr(self, "_regions", None)
        n = {"f": self.get_num_faces(), "v": self.get_num_vertices(), "e": self.get_num_edges()}[elem]
        if r is None:
            return np.zeros(n, np.int32)
        if elem == "e":
            return np.searchsorted(r[1], self.input_edges()[:, 0], side="right").astype(np.int32)
        return np.searchsorted(r[0] if elem == "f" else r[1], np.arange(n), side="right").astype(np.int32)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.rxg_mesh_destroy(h)
            self._h = None

    # ---- sizes (get_num_vertices & co., rxmesh.h) ---------------------
    def get_num_vertices(self):
        return self.info["num_vertices"]

    def get_num_edges(self):
        return self.info["num_edges"]

    def get_num_faces(self):
        return self.info["num_faces"]

    def export_obj(self, path, xyz):
        """RXMeshStatic::export_obj (rxmesh_static.inl:366-397): vertices in
        linear order from xyz (linear order, (nv, 3), tensor or array), faces
        in linear order over linear vertex ids."""
        x = xyz.detach().cpu().numpy() if hasattr(xyz, "detach") else np.asarray(xyz)
        x = x.reshape(-1, 3)
        if len(x) != self.get_num_vertices():
            raise ValueError("one position per vertex expected")
        vi2l = self.input_to_linear("v")
        faces = vi2l[self._fv[self.linear_to_input("f")]] + 1
        with open(path, "w") as fh:
            fh.writelines("v %.17g %.17g %.17g\n" % tuple(p) for p in x)
            fh.writelines("f %d %d %d\n" % tuple(t) for t in faces)

    def get_boundary_vertices(self, stream=None):
        """1 for every vertex on an edge with fewer than two faces
        (get_boundary_vertices, rxmesh_static.inl:281-323): int8 in linear
        order, a CUDA tensor (numpy for a host-only mesh)."""
        if self.host_only:
            out = np.empty(self.get_num_vertices(), np.int8)
            check(self._L.rxg_mesh_boundary_vertices(self._h, out.ctypes.data, None))
            return out
        out = torch.empty(self.get_num_vertices(), dtype=torch.int8, device="cuda")
        check(self._L.rxg_mesh_boundary_vertices(self._h, _ptr(out), _stream(stream)))
        return out

    def partition(self):
        """(face_patch, vertex_patch, edge_patch): the owner patch of every
        face, vertex and edge in input ids (rxg_mesh_partition)."""
        fp = np.empty(self.get_num_faces(), np.int32)
        vp = np.empty(self.get_num_vertices(), np.int32)
        ep = np.empty(self.get_num_edges(), np.int32)
        check(self._L.rxg_mesh_partition(self._h, fp.ctypes.data, vp.ctypes.data, ep.ctypes.data))
        return fp, vp, ep

    def save(self, filename):
        """RXMesh::save (rxmesh.h:326-329): write the partition as a patcher
        file that RXMesh and RXMeshStatic(..., patcher_file=) load."""
        check(self._L.rxg_mesh_save_patch_file(self._h, os.fsencode(filename)))

    def get_num_patches(self):
        return self.info["num_patches"]

    def is_closed(self):
        return bool(self.info["is_closed"])

    def is_edge_manifold(self):
        return bool(self.info["is_edge_manifold"])

    def is_oriented(self):
        return bool(self.info["is_oriented"])

    def get_num_components(self):
        return self.info["num_components"]

    def get_input_max_valence(self):
        return self.info["max_valence"]

    def get_input_max_edge_incident_faces(self):
        return self.info["max_edge_incident_faces"]

    def get_input_max_face_adjacent_faces(self):
        return self.info["max_face_adjacent_faces"]

    def _n(self, elem):
        return (self.get_num_vertices(), self.get_num_edges(), self.get_num_faces())[elem]

    # ---- numbering ------------------------------------------------------
    def linear_to_input(self, elem="v"):
        """Input id of every linear id (map_to_global, rxmesh_static.h:874-905)."""
        e = _ELEM[elem]
        if e not in self._maps:
            out = np.empty(self._n(e), np.int32)
            check(self._L.rxg_mesh_linear_to_input(self._h, e, out.ctypes.data))
            self._maps[e] = out
        return self._maps[e]

    def input_to_linear(self, elem="v"):
        m = self.linear_to_input(elem)
        inv = np.empty_like(m)
        inv[m] = np.arange(m.size, dtype=np.int32)
        return inv

    def input_edges(self):
        """(ne, 2) edge list in RXMesh's global edge order (rxmesh.cpp:518-620)."""
        out = np.empty(2 * self.get_num_edges(), np.int32)
        check(self._L.rxg_mesh_input_edges(self._h, out.ctypes.data))
        return out.reshape(-1, 2)

    def patches(self):
        """(headers (np, 16) int32, arena uint32) of the patch layout."""
        words = ctypes.c_int64()
        check(self._L.rxg_mesh_patches(self._h, None, None, ctypes.byref(words)))
        hdr = np.empty((self.get_num_patches(), 16), np.int32)
        arena = np.empty(words.value, np.uint32)
        check(self._L.rxg_mesh_patches(self._h, hdr.ctypes.data, arena.ctypes.data,
                                       ctypes.byref(words)))
        return hdr, arena

    def to_linear(self, t, elem="v", stream=None):
        """Device tensor in input order -> new device tensor in linear order."""
        return self._permute(t, elem, 1, stream)

    def to_input(self, t, elem="v", stream=None):
        """Device tensor in linear order -> new device tensor in input order."""
        return self._permute(t, elem, 0, stream)

    def _permute(self, t, elem, to_linear, stream):
        e = _ELEM[elem]
        t = t.contiguous()
        if t.shape[0] != self._n(e) or t.dtype not in _DT or not t.is_cuda:
            raise ValueError("expected a CUDA float32/float64 tensor with %d rows" % self._n(e))
        out = torch.empty_like(t)
        ncomp = t.numel() // max(1, t.shape[0])
        check(self._L.rxg_permute(self._h, e, to_linear, _DT[t.dtype], ncomp, _ptr(t), _ptr(out),
                                  _stream(stream)))
        return out

    # ---- queries (Query::dispatch / for_each<Op>) -------------------------
    def query_size(self, op):
        rows, vals = ctypes.c_int64(), ctypes.c_int64()
        check(self._L.rxg_query_size(self._h, int(op), ctypes.byref(rows), ctypes.byref(vals)))
        return rows.value, vals.value

    def query(self, op, stream=None, offsets=None, values=None):
        """Materialise query `op` for all owned elements, in linear ids.

        Returns (offsets, values) int32 CUDA tensors; offsets is None for the
        fixed-row ops FV, EV, FE, EVD, EE (3, 2, 3, 4, 4 values per row)."""
        op = Op.NAMES.get(op, op) if isinstance(op, str) else int(op)
        rows, nval = self.query_size(op)
        dev = torch.device("cuda", torch.cuda.current_device())
        csr = int(op) in Op.CSR
        if csr and offsets is None:
            offsets = torch.empty(rows + 1, dtype=torch.int32, device=dev)
        if values is None:
            values = torch.empty(nval, dtype=torch.int32, device=dev)
        check(self._L.rxg_query(self._h, op, _ptr(offsets) if csr else None, _ptr(values),
                                _stream(stream)))
        return (offsets if csr else None), values

    def query_host(self, op, offsets, values, asynchronous=False, stream=None):
        """Same as query() into host arrays: numpy arrays, or CPU torch
        tensors (copies inside the call; returns with the results in place).
        asynchronous=True with page-locked tensors (tensor.pin_memory()):
        the work and its copies are enqueued on `stream` (rxg_query_ex with
        RXG_HOST_ASYNC) and the results are there once the stream has run
        them; pageable arrays fall back to the synchronous call."""
        ptr = lambda a: None if a is None else (a.ctypes.data if isinstance(a, np.ndarray) else a.data_ptr())
        if asynchronous:
            check(self._L.rxg_query_ex(self._h, int(op), ptr(offsets), ptr(values), 1, _stream(stream)))
        else:
            check(self._L.rxg_query(self._h, int(op), ptr(offsets), ptr(values), None))
        return offsets, values

    def query_sweep(self, ops=("VV", "VE", "VF", "FV", "EV", "normals"), xyz=None, weighting="area",
                    stream=None, out=None, host=False):
        """Several queries (VV, VE, VF, FV, EV) and vertex normals in one
        launch (rxg_query_sweep): a dict op -> (offsets, values) for the CSR
        ops, values for FV / EV, the (nv, 3) normals for "normals" (which
        needs linear-order FP32 positions xyz).  out: the same dict of
        preallocated tensors, to write into.  host=True: the results go to
        page-locked host tensors (allocated here unless given in out; xyz may
        be a page-locked host tensor too) through rxg_query_sweep_ex, stream
        ordered: they hold the results once `stream` has run up to this call."""
        dev = torch.device("cuda", torch.cuda.current_device()) if not host else None

        def empty(n, dtype):
            return torch.empty(n, dtype=dtype, device=dev) if not host else \
                torch.empty(n, dtype=dtype).pin_memory()
        res = {} if out is None else dict(out)
        so = _lib.SweepOut()
        for name in ops:
            if name == "normals":
                if xyz is None or xyz.dtype != torch.float32 or (not xyz.is_cuda and not host):
                    raise ValueError("normals need float32 positions xyz (nv, 3), on the GPU (or "
                                     "page-locked with host=True)")
                xyz = xyz.contiguous()
                if name not in res:
                    res[name] = empty(xyz.numel(), torch.float32).view(-1, 3)
                so.xyz, so.normals = xyz.data_ptr(), res[name].data_ptr()
                so.weighting = {"max": 0, "area": 1}[weighting] if isinstance(weighting, str) else int(weighting)
                continue
            op = Op.NAMES[name]
            rows, nval = self.query_size(op)
            if name not in res:
                res[name] = (empty(rows + 1, torch.int32), empty(nval, torch.int32)) if op in Op.CSR else \
                    empty(nval, torch.int32)
            r = res[name]
            if op in Op.CSR:
                setattr(so, name.lower() + "_offsets", r[0].data_ptr())
                setattr(so, name.lower() + "_values", r[1].data_ptr())
            elif name in ("FV", "EV"):
                setattr(so, name.lower() + "_values", r.data_ptr())
            else:
                raise ValueError("query_sweep covers VV, VE, VF, FV, EV and normals, not %s" % name)
        if host:
            check(self._L.rxg_query_sweep_ex(self._h, ctypes.byref(so), 1, _stream(stream)))
        else:
            check(self._L.rxg_query_sweep(self._h, ctypes.byref(so), _stream(stream)))
        return res

    def query_oriented_vv(self, stream=None):
        """Oriented one-ring (rxmesh_queries.cuh:376-499): (offsets, values, boundary)."""
        nv = self.get_num_vertices()
        dev = torch.device("cuda", torch.cuda.current_device())
        off = torch.empty(nv + 1, dtype=torch.int32, device=dev)
        val = torch.empty(2 * self.get_num_edges(), dtype=torch.int32, device=dev)
        bnd = torch.empty(nv, dtype=torch.int8, device=dev)
        check(self._L.rxg_query_oriented_vv(self._h, _ptr(off), _ptr(val), _ptr(bnd),
                                            _stream(stream)))
        return off, val, bnd

    def vertex_normals(self, xyz, weighting="max", stream=None, out=None):
        """Vertex normals (linear order, FP32) of linear-order positions xyz (nv, 3)."""
        w = {"max": 0, "area": 1}[weighting] if isinstance(weighting, str) else int(weighting)
        xyz = xyz.contiguous()
        if xyz.dtype != torch.float32 or not xyz.is_cuda or xyz.numel() != 3 * self.get_num_vertices():
            raise ValueError("xyz must be a CUDA float32 tensor of shape (nv, 3)")
        if out is None:
            out = torch.empty_like(xyz)
        check(self._L.rxg_vertex_normals(self._h, w, _ptr(xyz), _ptr(out), _stream(stream)))
        return out


from ._solvers import (SparseMatrix, CGSolver, PCGSolver, mcf_step, MeshBatch, mcf_matvec,  # noqa: E402
                       mcf_init_b, mcf_solve_matfree, mcf_step_matfree)
from ._diff import (DiffScalarProblem, BlockSparseMatrix, NewtonSolver, ArapEnergy, MCFFlow,  # noqa: E402
                    arap_energy, mcf_flow, mcf_step_backward)
