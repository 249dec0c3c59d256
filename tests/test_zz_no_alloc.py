"""rxg_cg_solve_noalloc: the CG entry point that allocates no device memory.

It serves callers that may not allocate at solve time (an application that
owns all device memory through its own pool, a plugin that must not allocate
behind its host).  The test calls it through the C ABI and checks it against
rxg_cg_solve on two calls in a row (the shared static scratch must not carry
state from one call into the next), for CG and Jacobi-PCG, FP64 and FP32.
This file sorts last so that a run stopping at the first failure has run every
other test before it; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu

# tolerance of the other solver tests: solutions agree to 1e-12 of |X| in
# FP64 and 1e-6 in FP32 (the two entry points run the same kernel, so in
# practice the results are identical)
TOL = {torch.float64: 1e-12, torch.float32: 1e-6}
# relative residual |A X - B| / |B| the stopping rules above reach (delta
# relative 1e-20 in FP64 -> ~1e-10 in the 2-norm; 1e-10 in FP32 -> ~1e-5,
# limited by FP32 rounding of the recursive residual)
RES = {torch.float64: 1e-8, torch.float32: 1e-4}


def _system(dtype):
    from rxmesh_gb300 import RXMeshStatic
    from rxmesh_gb300._solvers import mcf_assemble
    v, f = meshgen.icosphere(4)
    x = meshgen.radial_noise(v, 0.02, 5)
    rx = RXMeshStatic(f, len(x), patch_size=256)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    A, B = mcf_assemble(rx, xl, 0.01, dtype)
    return rx, A, B, xl.to(dtype)


def _solve(fn, A, B, X0, precond):
    from rxmesh_gb300 import _lib
    X = X0.clone()
    o = _lib.SolverOpts(2000, 0.0, 1e-20 if A.dtype == torch.float64 else 1e-10, precond)
    st = _lib.SolverStats()
    c = A.csr()
    rc = fn(ctypes.byref(c), 3, ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(X.data_ptr()),
            ctypes.byref(o), ctypes.byref(st), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc, X, st


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("precond", [0, 1])
def test_noalloc_matches_allocating_solver_twice(dtype, precond):
    from rxmesh_gb300 import _lib
    L = _lib.load()
    rx, A, B, X0 = _system(dtype)
    import scipy.sparse as sp
    As = sp.csr_matrix((A.val.double().cpu().numpy(), A.col.cpu().numpy(), A.row_ptr.cpu().numpy()),
                       shape=(A.rows(), A.rows()))
    # two calls in a row with different right-hand sides and initial guesses
    for k, (b, x0) in enumerate([(B, X0), (0.5 * B + 0.01, torch.zeros_like(X0))]):
        rc_a, Xa, sa = _solve(L.rxg_cg_solve, A, b, x0, precond)
        rc_n, Xn, sn = _solve(L.rxg_cg_solve_noalloc, A, b, x0, precond)
        assert rc_a == 0 and rc_n == 0, (k, rc_a, rc_n, L.rxg_last_error())
        assert sn.converged and sn.iters == sa.iters
        assert abs(sn.final_res - sa.final_res) <= TOL[dtype] * abs(sa.start_res)
        err = (Xn - Xa).abs().max().item() / Xa.abs().max().item()
        assert err <= TOL[dtype], (k, err)
        # the solution itself, independent of the other entry point: the
        # residual |A X - B| computed in FP64 by scipy from the same matrix
        Xh = Xn.double().cpu().numpy()
        res = np.linalg.norm(As @ Xh - b.double().cpu().numpy()) / np.linalg.norm(b.double().cpu().numpy())
        assert res <= RES[dtype], (k, res)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from rxmesh_gb300 import _lib
    L = _lib.load()
    n = 131072 + 1
    rp = torch.arange(n + 1, dtype=torch.int32, device="cuda")
    col = torch.arange(n, dtype=torch.int32, device="cuda")
    val = torch.ones(n, dtype=torch.float64, device="cuda")
    c = _lib.CSR(n, n, rp.data_ptr(), col.data_ptr(), val.data_ptr(), 1)
    B = torch.ones(n, 3, dtype=torch.float64, device="cuda")
    X = torch.zeros_like(B)
    o = _lib.SolverOpts(10, 0.0, 1e-10, 1)
    st = _lib.SolverStats()
    rc = L.rxg_cg_solve_noalloc(ctypes.byref(c), 3, ctypes.c_void_p(B.data_ptr()),
                                ctypes.c_void_p(X.data_ptr()), ctypes.byref(o), ctypes.byref(st), None)
    assert rc == 1 and b"exceeds the fixed scratch" in L.rxg_last_error()
    assert X.abs().max().item() == 0.0


def test_noalloc_rejects_host_matrix_arrays():
    """A's row_ptr and col must be device arrays too: host copies are
    refused before any launch."""
    from rxmesh_gb300 import _lib
    L = _lib.load()
    rx, A, B, X0 = _system(torch.float64)
    X = X0.clone()
    o = _lib.SolverOpts(10, 0.0, 1e-10, 1)
    st = _lib.SolverStats()
    rp_h, col_h = A.row_ptr.cpu(), A.col.cpu()
    for rp, col in ((rp_h, A.col), (A.row_ptr, col_h)):
        c = _lib.CSR(A.rows(), A.col.numel(), rp.data_ptr(), col.data_ptr(), A.val.data_ptr(), 1)
        for fn in (L.rxg_cg_solve_noalloc, L.rxg_cg_solve):
            rc = fn(ctypes.byref(c), 3, ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                    ctypes.byref(o), ctypes.byref(st), None)
            assert rc == 1 and b"must be device arrays" in L.rxg_last_error()
    assert torch.equal(X, X0)
