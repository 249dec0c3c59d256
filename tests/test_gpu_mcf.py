"""GPU parity of the MCF system, SpMM, CG/PCG and the MCF step."""
import numpy as np
import pytest
import torch

from conftest import golden, kat_system
from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu


def mesh(level=4, seed=1):
    v, f = meshgen.icosphere(level)
    return meshgen.radial_noise(v, 0.02, seed), f


def to_input_csr(rx, A):
    """GPU CSR (linear ids) -> dict (input row, input col) -> value."""
    import scipy.sparse as sp
    vl = rx.linear_to_input("v")
    S = A.to_scipy().tocoo()
    n = S.shape[0]
    return sp.csr_matrix((S.data, (vl[S.row], vl[S.col])), shape=(n, n))


# FP64 assembly: 1e-12 of the row diagonal; FP32 weights (FP64 only for
# triangles with an angle below 1e-3 rad): 1e-5 of the row diagonal.
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("kind", ["sphere", "plane", "bunnyhead"])
def test_mcf_assembly_matches_oracle(oracle, dtype, tol, kind):
    import scipy.sparse as sp
    from rxmesh_gb300 import RXMeshStatic
    from rxmesh_gb300._solvers import mcf_assemble
    if kind == "sphere":
        x, f = mesh(4)
    elif kind == "plane":
        x, f = meshgen.plane(30, 20, 0.1)
        x = x + np.random.default_rng(2).normal(0, 0.01, x.shape)
    else:
        g = golden("bunnyhead")
        x, f = g["xyz"], g["fv"]
    rx = RXMeshStatic(f, len(x), patch_size=128)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    A, B = mcf_assemble(rx, xl, 0.01, dtype)
    Ag = to_input_csr(rx, A)
    rp, col, val, Bo = oracle.mcf_system(f, x, 0.01)
    Ao = sp.csr_matrix((val, col, rp), shape=Ag.shape)
    assert Ag.nnz == Ao.nnz
    diag = Ao.diagonal()
    D = abs(Ag - Ao).tocsr()
    row_err = np.array([D[i].max() if D[i].nnz else 0.0 for i in range(D.shape[0])])
    assert (row_err <= tol * diag).all(), (row_err / diag).max()
    Bg = rx.to_input(B.to(torch.float64)).cpu().numpy()
    assert (np.abs(Bg - Bo).max(1) <= tol * np.abs(Bo).max(1) + 1e-300).all()


def test_spmm_matches_oracle(oracle):
    from rxmesh_gb300 import RXMeshStatic
    from rxmesh_gb300._solvers import mcf_assemble
    x, f = mesh(4)
    rx = RXMeshStatic(f, len(x), patch_size=256)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    A, _ = mcf_assemble(rx, xl, 0.01, torch.float64)
    Y = A.multiply(xl)
    S = A.to_scipy()
    assert np.abs(Y.cpu().numpy() - S @ xl.cpu().numpy()).max() < 1e-13


def _kat(oracle, rx, g):
    """setup() of tests/RXMesh_test/test_solver.cu:79-119 in linear order."""
    from rxmesh_gb300 import SparseMatrix
    rp, col, val, B, X0 = kat_system(oracle, "sphere3")
    il = rx.input_to_linear("v")
    vl = rx.linear_to_input("v")
    n = len(vl)
    lrp = np.zeros(n + 1, np.int64)
    lrp[1:] = np.cumsum(np.diff(rp)[vl])
    lcol = np.concatenate([il[col[rp[p]:rp[p + 1]]] for p in vl]).astype(np.int32)
    lval = np.concatenate([val[rp[p]:rp[p + 1]] for p in vl])
    t = lambda a, d: torch.tensor(a, dtype=d, device="cuda")
    A = SparseMatrix(row_ptr=t(lrp, torch.int32), col=t(lcol, torch.int32), val=t(lval, torch.float64))
    return A, t(B[vl], torch.float64), t(X0[vl], torch.float64), (rp, col, val, B, X0)


@pytest.mark.parametrize("precond", [False, True])
def test_solver_kat_gpu(oracle, precond):
    # Solver.CG / Solver.PCG (test_solver.cu:339-401): abs_tol 1e-7, |Ax-b| <= 1e-3
    from rxmesh_gb300 import CGSolver, PCGSolver, RXMeshStatic
    g = golden("sphere3")
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), patch_size=512)
    A, B, X, (rp, col, val, Bo, X0) = _kat(oracle, rx, g)
    S = (PCGSolver if precond else CGSolver)(A, 3, 5000, 1e-7)
    S.pre_solve(B, X)
    S.solve(B, X)
    assert S.converged()
    Ax = A.multiply(X)
    assert (Ax - B).abs().max().item() <= 1e-3
    Xo, it, r0, r1, conv = oracle.cg(rp, col, val, Bo, X0, 5000, 1e-7, 0.0, precond)
    assert abs(S.iter_taken() - it) <= 2
    assert abs(S.start_residual() - r0) <= 1e-9 * abs(r0)
    assert np.abs(X.cpu().numpy() - Xo[rx.linear_to_input("v")]).max() < 1e-6


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_mcf_step_matches_oracle(oracle, precision):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    from rxmesh_gb300 import RXMeshStatic, mcf_step
    x, f = mesh(5)
    rx = RXMeshStatic(f, len(x), patch_size=256)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    st = mcf_step(rx, xl, 0.01, 1, precision, tol=1e-8)
    assert st["converged"]
    rp, col, val, B = oracle.mcf_system(f, x, 0.01)
    A = sp.csr_matrix((val, col, rp), shape=(len(x), len(x))).tocsc()
    X = spl.spsolve(A, B)
    got = rx.to_input(xl).cpu().numpy()
    rel = np.linalg.norm(got - X) / np.linalg.norm(X)
    upd = np.linalg.norm(got - X) / np.linalg.norm(X - x)
    assert rel < 1e-6, (rel, upd, st)


def test_mcf_step_host_buffer_and_multi_step(oracle):
    from rxmesh_gb300 import RXMeshStatic, mcf_step
    x, f = mesh(4, seed=3)
    rx = RXMeshStatic(f, len(x), patch_size=256)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    host = xl.cpu().clone()
    mcf_step(rx, xl, 1e-3, 3, "f64", tol=1e-10)
    mcf_step(rx, host, 1e-3, 3, "f64", tol=1e-10)
    assert np.abs(host.numpy() - xl.cpu().numpy()).max() < 1e-12


def test_sparse_matrix_edge_length_spmv_and_transpose(oracle):
    """The reference's SparseMatrixEdgeLen test (test_sparse_matrix.cu:175-242):
    every off-diagonal entry of the VV pattern set to its edge length, times
    a vector of ones, gives each vertex's summed edge lengths (FP32, sphere3);
    and transpose on the device (test_sparse_matrix.cu:325-367)."""
    from rxmesh_gb300 import RXMeshStatic
    from rxmesh_gb300._solvers import SparseMatrix, mcf_assemble
    g = golden("sphere3")
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), patch_size=256)
    xl = rx.to_linear(torch.tensor(g["xyz"], device="cuda"))
    A, _ = mcf_assemble(rx, xl, 0.01, torch.float32)
    n = A.rows()
    rows = torch.repeat_interleave(torch.arange(n, device="cuda"),
                                   (A.row_ptr[1:] - A.row_ptr[:-1]).long())
    cols = A.col.long()
    A.val.copy_(torch.linalg.norm(xl[rows] - xl[cols], dim=1).float())
    y = A.multiply(torch.ones(n, 1, dtype=torch.float32, device="cuda")).cpu().numpy()[:, 0]
    ev, _ = oracle.edges(g["fv"])
    want = np.zeros(len(g["xyz"]))
    lens = np.linalg.norm(g["xyz"][ev[:, 0]] - g["xyz"][ev[:, 1]], axis=1)
    np.add.at(want, ev[:, 0], lens)
    np.add.at(want, ev[:, 1], lens)
    got = y[rx.input_to_linear("v")]
    assert np.abs(got - want).max() <= 1e-5 * want.max()
    # transpose: the pattern is symmetric, so A^T = A here, diagonal kept first
    A.val.copy_(torch.rand(A.non_zeros(), device="cuda"))
    T = A.transpose()
    assert T.row_ptr.is_cuda
    assert abs(T.to_scipy() - A.to_scipy().T.tocsr()).max() == 0
    assert torch.equal(T.col[T.row_ptr[:-1].long()], torch.arange(n, device="cuda", dtype=torch.int32))
