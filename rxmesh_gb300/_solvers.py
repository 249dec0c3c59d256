"""SparseMatrix / CGSolver / PCGSolver / mcf_step over the C ABI.

Mirrors include/rxmesh/matrix/sparse_matrix.h (SparseMatrix<T>(rx, Op::VV)),
matrix/cg_solver.h and matrix/pcg_solver.h; mcf_step mirrors the MCF app's
run_cg (apps/MCF/mcf_cg.h:12-129).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check, RXGError

_DT = {torch.float32: 0, torch.float64: 1}


def _stream(stream=None):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class SparseMatrix:
    """CSR matrix in linear vertex order, diagonal first (SparseMatrix<T>, sparse_matrix.h:77)."""

    def __init__(self, rx=None, dtype=torch.float64, row_ptr=None, col=None, val=None):
        self._L = _lib.load()
        if rx is not None:
            n, nnz = ctypes.c_int64(), ctypes.c_int64()
            check(self._L.rxg_mcf_pattern_size(rx._h, ctypes.byref(n), ctypes.byref(nnz)))
            dev = torch.device("cuda", torch.cuda.current_device())
            self.row_ptr = torch.zeros(n.value + 1, dtype=torch.int32, device=dev)
            self.col = torch.zeros(nnz.value, dtype=torch.int32, device=dev)
            self.val = torch.zeros(nnz.value, dtype=dtype, device=dev)
        else:
            self.row_ptr, self.col, self.val = row_ptr.contiguous(), col.contiguous(), val.contiguous()
        self.rx = rx

    @property
    def dtype(self):
        return self.val.dtype

    def rows(self):
        return self.row_ptr.numel() - 1

    def cols(self):
        return self.rows()

    def csr(self):
        c = _lib.CSR()
        c.n = self.rows()
        c.nnz = self.col.numel()
        c.row_ptr = self.row_ptr.data_ptr()
        c.col = self.col.data_ptr()
        c.val = self.val.data_ptr()
        c.dtype = _DT[self.val.dtype]
        return c

    def multiply(self, X, Y=None, stream=None):
        """Y = A X (sparse_matrix.h:1173-1263); X is (n, nc) of the matrix dtype."""
        X = X.contiguous()
        nc = 1 if X.dim() == 1 else X.shape[1]
        if Y is None:
            Y = torch.empty_like(X)
        c = self.csr()
        check(self._L.rxg_spmm(ctypes.byref(c), nc, _ptr(X), _ptr(Y), _stream(stream)))
        return Y

    def non_zeros(self):
        return self.col.numel()

    def __call__(self, row, col):
        """A(row, col), 0 where the pattern has no entry (operator(),
        sparse_matrix.h:412-471); a host lookup."""
        lo, hi = (int(v) for v in self.row_ptr[row:row + 2].tolist())
        cols = self.col[lo:hi].tolist()
        return float(self.val[lo + cols.index(col)]) if col in cols else 0.0

    def transpose(self):
        """A^T as a new SparseMatrix on the same device (transpose,
        sparse_matrix.h; tests/RXMesh_test/test_sparse_matrix.cu:325-367):
        each row keeps its diagonal entry first, then the rest by column."""
        n = self.rows()
        dev = self.row_ptr.device
        counts = (self.row_ptr[1:] - self.row_ptr[:-1]).to(torch.int64)
        rows = torch.repeat_interleave(torch.arange(n, device=dev), counts)
        cols = self.col.to(torch.int64)
        off_diag = (rows != cols).to(torch.int64)
        # sort by (new row = old col, diagonal first, new col = old row)
        key = (cols * 2 + off_diag) * n + rows
        order = torch.argsort(key)
        new_ptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        new_ptr[1:] = torch.cumsum(torch.bincount(cols, minlength=n), 0)
        return SparseMatrix(row_ptr=new_ptr.to(torch.int32), col=rows[order].to(torch.int32),
                            val=self.val[order])

    def to_scipy(self):
        import scipy.sparse as sp
        n = self.rows()
        return sp.csr_matrix((self.val.cpu().numpy(), self.col.cpu().numpy(),
                              self.row_ptr.cpu().numpy()), shape=(n, n))


def mcf_assemble(rx, xyz_lin, dt, dtype=torch.float64, stream=None):
    """(A, B) of the MCF system (mcf_A_setup / mcf_B_setup) at linear positions xyz_lin."""
    A = SparseMatrix(rx, dtype)
    B = torch.empty((rx.get_num_vertices(), 3), dtype=dtype, device=A.val.device)
    c = A.csr()
    x = xyz_lin.to(torch.float64).contiguous()
    check(A._L.rxg_mcf_assemble(rx._h, float(dt), _ptr(x), ctypes.byref(c), _ptr(B), _stream(stream)))
    return A, B


class CGSolver:
    """CGSolver(A, unknown_dim, max_iter, abs_tol, rel_tol) (cg_solver.h:17-35)."""
    PRECOND = 0

    def __init__(self, A, unknown_dim, max_iter, abs_tol=1e-6, rel_tol=0.0):
        self.A, self.nc = A, int(unknown_dim)
        self.max_iter, self.abs_tol, self.rel_tol = int(max_iter), float(abs_tol), float(rel_tol)
        self._stats = _lib.SolverStats()
        self._L = _lib.load()

    def pre_solve(self, B, X, stream=None):
        # the residual set-up runs inside solve() (same kernel launch)
        return None

    def solve(self, B, X, stream=None):
        o = _lib.SolverOpts(self.max_iter, self.abs_tol, self.rel_tol, self.PRECOND)
        c = self.A.csr()
        st = self._L.rxg_cg_solve(ctypes.byref(c), self.nc, _ptr(B.contiguous()), _ptr(X),
                                  ctypes.byref(o), ctypes.byref(self._stats), _stream(stream))
        if st not in (0, 6):
            check(st)
        return X

    def iter_taken(self):
        return self._stats.iters

    def start_residual(self):
        return self._stats.start_res

    def final_residual(self):
        return self._stats.final_res

    def converged(self):
        return bool(self._stats.converged)


class PCGSolver(CGSolver):
    """Jacobi-preconditioned CG (pcg_solver.h:14-213)."""
    PRECOND = 1


def mcf_step(rx, xyz_lin, dt, nsteps=1, precision="f64", tol=1e-6, max_iter=5000, stream=None):
    """Implicit MCF steps in place on xyz_lin ((nv,3) float64 CUDA tensor, linear order).

    Returns the solver stats dict of the last step."""
    L = _lib.load()
    if xyz_lin.dtype != torch.float64 or not xyz_lin.is_contiguous():
        raise ValueError("xyz_lin must be a contiguous float64 tensor")
    prec = {"f64": 1, "f32": 0, "mixed": 0}[precision]
    st = _lib.SolverStats()
    ptr = xyz_lin.data_ptr() if xyz_lin.is_cuda else xyz_lin.numpy().ctypes.data
    rc = L.rxg_mcf_step(rx._h, float(dt), int(nsteps), prec, float(tol), int(max_iter),
                        ctypes.c_void_p(ptr), ctypes.byref(st), _stream(stream))
    if rc not in (0, 6):
        check(rc)
    return {"iters": st.iters, "converged": bool(st.converged), "start_res": st.start_res,
            "final_res": st.final_res}


def _mf_flags(uniform, jacobi=False):
    return (1 if uniform else 0) | (2 if jacobi else 0)


def mcf_matvec(rx, xyz_lin, v, dt, uniform=False, jacobi=False, out=None, stream=None):
    """Matrix-free product of the implicit-MCF operator A = 2M + dt L at
    positions xyz_lin ((nv,3) float64, linear order) with v ((nv,3) float32
    or float64): A v, or D^-1 v with jacobi (matvec / precond_matvec,
    apps/MCF/mcf_kernels.cuh:101-299).  uniform: the uniform Laplacian."""
    L = _lib.load()
    out = torch.empty_like(v) if out is None else out
    dtype = 1 if v.dtype == torch.float64 else 0
    check(L.rxg_mcf_matvec(rx._h, float(dt), _mf_flags(uniform, jacobi), dtype, _ptr(xyz_lin), _ptr(v),
                           _ptr(out), _stream(stream)))
    return out


def mcf_init_b(rx, xyz_lin, uniform=False, dtype=torch.float64, stream=None):
    """Right-hand side B = (1 / v_weight) x of the implicit MCF step
    (init_B, apps/MCF/mcf_kernels.cuh:58-98)."""
    L = _lib.load()
    B = torch.empty(xyz_lin.shape, dtype=dtype, device=xyz_lin.device)
    check(L.rxg_mcf_init_b(rx._h, _mf_flags(uniform), 1 if dtype == torch.float64 else 0, _ptr(xyz_lin),
                           _ptr(B), _stream(stream)))
    return B


def mcf_solve_matfree(rx, xyz_lin, B, X, dt, max_iter=5000, abs_tol=0.0, rel_tol=1e-12, precond=True,
                      uniform=False, stream=None):
    """Solve A(xyz_lin) X = B with the matrix-free operator
    (CGMatFreeAttrSolver / PCGMatFreeAttrSolver); X is the initial guess and
    is overwritten.  Returns the solver stats dict."""
    L = _lib.load()
    st = _lib.SolverStats()
    o = _lib.SolverOpts(int(max_iter), float(abs_tol), float(rel_tol), 1 if precond else 0)
    rc = L.rxg_mcf_solve_matfree(rx._h, float(dt), _mf_flags(uniform), 1 if X.dtype == torch.float64 else 0,
                                 _ptr(xyz_lin), _ptr(B), _ptr(X), ctypes.byref(o), ctypes.byref(st),
                                 _stream(stream))
    if rc not in (0, 6):
        check(rc)
    return {"iters": st.iters, "converged": bool(st.converged), "start_res": st.start_res,
            "final_res": st.final_res}


def mcf_step_matfree(rx, xyz_lin, dt, nsteps=1, tol=1e-6, max_iter=5000, uniform=False, stream=None):
    """Implicit MCF steps in place on xyz_lin with the matrix-free operator
    (FP64, Jacobi PCG; run_cg_mat_free, apps/MCF/mcf_cg_mat_free.h)."""
    L = _lib.load()
    if xyz_lin.dtype != torch.float64 or not xyz_lin.is_cuda or not xyz_lin.is_contiguous():
        raise ValueError("xyz_lin must be a contiguous float64 CUDA tensor")
    st = _lib.SolverStats()
    rc = L.rxg_mcf_step_matfree(rx._h, float(dt), int(nsteps), _mf_flags(uniform), float(tol), int(max_iter),
                                _ptr(xyz_lin), ctypes.byref(st), _stream(stream))
    if rc not in (0, 6):
        check(rc)
    return {"iters": st.iters, "converged": bool(st.converged), "start_res": st.start_res,
            "final_res": st.final_res}


class MeshBatch:
    """Many meshes packed for one-launch batched MCF (rxg_batch_*).

    meshes: list of (fv, nv) with vertex ids local to each mesh.  Positions
    are passed as one (sum nv, 3) float64 CUDA tensor, meshes one after
    another in their input order."""

    def __init__(self, meshes, patch_size=256):
        import numpy as np
        self._L = _lib.load()
        fvs = [np.ascontiguousarray(f, np.int32).reshape(-1, 3) for f, _ in meshes]
        nf = np.array([len(f) for f in fvs], np.int64)
        nv = np.array([int(v) for _, v in meshes], np.int64)
        allf = np.ascontiguousarray(np.concatenate(fvs), np.int32)
        h = ctypes.c_void_p()
        check(self._L.rxg_batch_create(len(fvs), allf.ctypes.data, nf.ctypes.data, nv.ctypes.data,
                                       int(patch_size), ctypes.byref(h)))
        self._h = h
        self.nmesh = len(fvs)
        self.nv = nv
        self.nf = nf
        self.voff = np.concatenate([[0], np.cumsum(nv)])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.rxg_batch_destroy(h)
            self._h = None

    def mcf(self, xyz, dt, nsteps=1, tol=1e-6, max_iter=5000, stream=None):
        """Mixed-precision implicit MCF on every mesh, in place on xyz."""
        if xyz.dtype != torch.float64 or not xyz.is_cuda or not xyz.is_contiguous():
            raise ValueError("xyz must be a contiguous float64 CUDA tensor")
        check(self._L.rxg_batch_mcf(self._h, float(dt), int(nsteps), float(tol), int(max_iter),
                                    _ptr(xyz), _stream(stream)))
        return xyz

    def stats(self):
        import numpy as np
        it = np.empty(self.nmesh, np.int32)
        cv = np.empty(self.nmesh, np.int32)
        check(self._L.rxg_batch_stats(self._h, it.ctypes.data, cv.ctypes.data))
        return it, cv.astype(bool)

    def autotune(self, xyz, dt, nsteps=1, tol=1e-6, max_iter=5000, stream=None):
        """Pick the fastest CTA size / CTAs per SM for this batch (xyz untouched)."""
        t = ctypes.c_int32()
        b = ctypes.c_int32()
        ms = ctypes.c_float()
        check(self._L.rxg_batch_autotune(self._h, float(dt), int(nsteps), float(tol), int(max_iter),
                                         _ptr(xyz), ctypes.byref(t), ctypes.byref(b), ctypes.byref(ms),
                                         _stream(stream)))
        return t.value, b.value, ms.value
