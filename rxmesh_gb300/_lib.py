"""ctypes bindings of librxg.so (the C ABI declared in include/rxg.h).

The library is the only compute path: if it is missing or fails to load,
every call raises; there is no CPU fallback.
"""
import ctypes
import os

from . import build as _build

_L = None

RXG_OK = 0
STATUS = {0: "RXG_OK", 1: "RXG_ERR_INVALID", 2: "RXG_ERR_NOMEM", 3: "RXG_ERR_CUDA",
          4: "RXG_ERR_NONMANIFOLD", 5: "RXG_ERR_PATCH_LIMIT", 6: "RXG_ERR_NOT_CONVERGED",
          7: "RXG_ERR_DEVICE_TIMEOUT", 8: "RXG_ERR_UNSUPPORTED", 9: "RXG_ERR_NO_DEVICE"}


class RXGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class SweepOut(ctypes.Structure):
    """rxg_sweep_out (include/rxg.h)."""
    _fields_ = [("vv_offsets", ctypes.c_void_p), ("vv_values", ctypes.c_void_p),
                ("ve_offsets", ctypes.c_void_p), ("ve_values", ctypes.c_void_p),
                ("vf_offsets", ctypes.c_void_p), ("vf_values", ctypes.c_void_p),
                ("fv_values", ctypes.c_void_p), ("ev_values", ctypes.c_void_p),
                ("xyz", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("weighting", ctypes.c_int32)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_int64), ("num_edges", ctypes.c_int64),
                ("num_faces", ctypes.c_int64), ("num_patches", ctypes.c_int64),
                ("max_valence", ctypes.c_int64), ("is_closed", ctypes.c_int32),
                ("is_edge_manifold", ctypes.c_int32), ("patch_faces", ctypes.c_int32),
                ("max_local_vertices", ctypes.c_int32), ("max_local_edges", ctypes.c_int32),
                ("max_local_faces", ctypes.c_int32), ("ribbon_vertices", ctypes.c_int64),
                ("ribbon_faces", ctypes.c_int64), ("device_bytes", ctypes.c_int64),
                ("num_components", ctypes.c_int32), ("is_oriented", ctypes.c_int32),
                ("max_edge_incident_faces", ctypes.c_int32),
                ("max_face_adjacent_faces", ctypes.c_int32), ("num_face_patches", ctypes.c_int32),
                ("lloyd_runs", ctypes.c_int32)]


class CSR(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nnz", ctypes.c_int64), ("row_ptr", ctypes.c_void_p),
                ("col", ctypes.c_void_p), ("val", ctypes.c_void_p), ("dtype", ctypes.c_int32)]


class BCSR(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nnzb", ctypes.c_int64), ("row_ptr", ctypes.c_void_p),
                ("col", ctypes.c_void_p), ("val", ctypes.c_void_p), ("dtype", ctypes.c_int32),
                ("block_dim", ctypes.c_int32)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int32), ("abs_tol", ctypes.c_double),
                ("rel_tol", ctypes.c_double), ("precond", ctypes.c_int32)]


class SolverStats(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("start_res", ctypes.c_double), ("final_res", ctypes.c_double)]


P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
D = ctypes.c_double

# name -> argtypes (restype is rxg_status = int unless listed in _RESTYPE)
SIGNATURES = {
    "rxg_status_string": [I32],
    "rxg_last_error": [],
    "rxg_mesh_create": [P, I64, I64, I32, P],
    "rxg_mesh_create_ex": [P, I64, I64, I32, I32, P],
    "rxg_mesh_create_partitioned": [P, I64, I64, P, P, P, I64, I32, P],
    "rxg_mesh_partition": [P, P, P, P],
    "rxg_mesh_boundary_vertices": [P, P, P],
    "rxg_mesh_create_from_patch_file": [P, I64, I64, ctypes.c_char_p, I32, P],
    "rxg_mesh_save_patch_file": [P, ctypes.c_char_p],
    "rxg_mesh_destroy": [P],
    "rxg_mesh_get_info": [P, P],
    "rxg_mesh_linear_to_input": [P, I32, P],
    "rxg_mesh_input_edges": [P, P],
    "rxg_mesh_patches": [P, P, P, P],
    "rxg_permute": [P, I32, I32, I32, I32, P, P, P],
    "rxg_query_size": [P, I32, P, P],
    "rxg_query": [P, I32, P, P, P],
    "rxg_query_oriented_vv": [P, P, P, P, P],
    "rxg_vertex_normals": [P, I32, P, P, P],
    "rxg_device_check": [P],
    "rxg_selftest_bounded_wait": [P],
    "rxg_mcf_pattern_size": [P, P, P],
    "rxg_mcf_assemble": [P, D, P, P, P, P],
    "rxg_spmm": [P, I32, P, P, P],
    "rxg_cg_solve": [P, I32, P, P, P, P, P],
    "rxg_cg_solve_noalloc": [P, I32, P, P, P, P, P],
    "rxg_mcf_step": [P, D, I32, I32, D, I32, P, P, P],
    "rxg_mcf_step_backward": [P, D, P, P, P, P, D, I32, P, P],
    "rxg_arap_rest": [P, P, I32, P, P],
    "rxg_batch_create": [I32, P, P, P, I32, P],
    "rxg_batch_destroy": [P],
    "rxg_batch_mesh": [P, P],
    "rxg_batch_mcf": [P, D, I32, D, I32, P, P],
    "rxg_batch_stats": [P, P, P],
    "rxg_batch_autotune": [P, D, I32, D, I32, P, P, P, P, P],
    "rxg_arap_eval": [P, I32, P, P, P, P, P, P, P],
    "rxg_arap_eval_ex": [P, I32, P, P, I32, P, P, P, P, P],
    "rxg_bcsr_to_csr": [P, P, P],
    "rxg_dense_axpby": [I64, I32, ctypes.c_double, P, ctypes.c_double, P, P],
    "rxg_dense_dot": [I64, I32, P, P, P, P],
    "rxg_bcsr_apply_bc": [P, P, P, P],
    "rxg_arap_hvp": [P, I32, P, P, I32, P, P, P, P],
    "rxg_arap_cg_matfree": [P, I32, P, P, I32, P, P, P, P, P, P],
    "rxg_mesh_device_context": [P, P],
    "rxg_mcf_matvec": [P, D, I32, I32, P, P, P, P],
    "rxg_mcf_init_b": [P, I32, I32, P, P, P],
    "rxg_mcf_solve_matfree": [P, D, I32, I32, P, P, P, P, P, P],
    "rxg_mcf_step_matfree": [P, D, I32, I32, D, I32, P, P, P],
    "rxg_face_term_gather": [P, I32, I32, P, I32, P, P, P, P, P],
    "rxg_edge_term_gather": [P, I32, I32, P, I32, P, P, P, P, P],
    "rxg_vertex_term_gather": [P, I32, I32, P, I32, P, P, P, P, P],
    "rxg_symdir_eval": [P, I32, P, P, I32, P, P, P, P, P],
    "rxg_inertia_eval": [P, I32, I32, P, P, D, I32, P, P, P, P],
    "rxg_dense_zero_rows": [I64, I32, I32, P, P, P],
    "rxg_query_ex": [P, I32, P, P, I32, P],
    "rxg_query_sweep": [P, P, P],
    "rxg_query_sweep_ex": [P, P, I32, P],
    "rxg_vertex_normals_ex": [P, I32, P, P, I32, P],
}
_RESTYPE = {"rxg_status_string": ctypes.c_char_p, "rxg_last_error": ctypes.c_char_p,
            "rxg_mesh_destroy": None, "rxg_batch_destroy": None}


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load librxg.so (building it in-tree first when it is absent or stale)."""
    global _L
    if _L is not None:
        return _L
    path = lib_path()
    if build_if_missing:
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("librxg.so is not built (%s); run python -m rxmesh_gb300.build" % path)
    L = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue  # reported by exported_symbols()
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, ctypes.c_int)
    _L = L
    return L


def exported_symbols():
    """Names declared in include/rxg.h that the loaded library exports."""
    L = load()
    return {n for n in SIGNATURES if getattr(L, n, None) is not None}


def check(status):
    if status != RXG_OK:
        msg = _L.rxg_last_error().decode() if _L is not None else ""
        raise RXGError(status, msg)
    return status
