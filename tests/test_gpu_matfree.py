"""The matrix-free implicit-MCF operator (init_B / matvec / precond_matvec,
apps/MCF/mcf_kernels.cuh:58-299) and its CG (CGMatFreeAttrSolver,
matrix/cg_mat_free_attr_solver.h:45-115) against the assembled system and
the oracle."""
import numpy as np
import pytest
import torch

from conftest import golden
from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu


def meshes():
    v, f = meshgen.icosphere(4)
    yield "sphere", meshgen.radial_noise(v, 0.02, 1), f
    x, f = meshgen.plane(30, 20, 0.1)
    yield "plane", x + np.random.default_rng(2).normal(0, 0.01, x.shape), f
    g = golden("bunnyhead")
    yield "bunnyhead", g["xyz"], g["fv"]


@pytest.mark.parametrize("name", ["sphere", "plane", "bunnyhead"])
def test_matvec_equals_assembled_spmm(name):
    """FP64: A(x) v through the matrix-free operator equals rxg_spmm on the
    assembled matrix to 1e-12; the Jacobi product equals v / diag(A); init_B
    equals the assembled right-hand side."""
    from rxmesh_gb300 import RXMeshStatic, mcf_init_b, mcf_matvec
    from rxmesh_gb300._solvers import mcf_assemble
    x, f = {n: (a, b) for n, a, b in meshes()}[name]
    rx = RXMeshStatic(f, len(x), patch_size=128)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    dt = 0.01
    A, B = mcf_assemble(rx, xl, dt, torch.float64)
    v = torch.randn_like(xl)
    want = A.multiply(v)
    got = mcf_matvec(rx, xl, v, dt)
    assert (got - want).abs().max().item() <= 1e-12 * want.abs().max().item()
    S = A.to_scipy()
    d = torch.tensor(S.diagonal(), device="cuda")
    gj = mcf_matvec(rx, xl, v, dt, jacobi=True)
    assert (gj - v / d[:, None]).abs().max().item() <= 1e-13 * (v / d[:, None]).abs().max().item()
    gb = mcf_init_b(rx, xl)
    assert (gb - B).abs().max().item() <= 1e-13 * B.abs().max().item()
    # FP32 operator against the FP64 one
    g32 = mcf_matvec(rx, xl, v.float(), dt)
    assert (g32.double() - want).abs().max().item() <= 1e-5 * want.abs().max().item()


def test_uniform_laplace_mode(oracle):
    """use_uniform_laplace: weight dt per neighbour, diagonal valence (1 + dt),
    B = valence x."""
    from rxmesh_gb300 import RXMeshStatic, mcf_init_b, mcf_matvec
    x, f = meshgen.icosphere(3)
    rx = RXMeshStatic(f, len(x), patch_size=64)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    dt = 0.05
    ev, _ = oracle.edges(f)
    off, nb = oracle.vv(len(x), ev)
    deg = np.diff(off).astype(np.float64)
    v = np.random.default_rng(3).normal(size=x.shape)
    want = deg[:, None] * (1 + dt) * v
    rows = np.repeat(np.arange(len(x)), np.diff(off))
    np.add.at(want, rows, -dt * v[nb])
    vl = rx.linear_to_input("v")
    got = mcf_matvec(rx, xl, torch.tensor(v[vl], device="cuda"), dt, uniform=True).cpu().numpy()
    assert np.abs(got - want[vl]).max() <= 1e-12 * np.abs(want).max()
    gb = mcf_init_b(rx, xl, uniform=True).cpu().numpy()
    assert np.abs(gb - (deg[:, None] * x)[vl]).max() <= 1e-12 * np.abs(x).max() * deg.max()


@pytest.mark.parametrize("precond", [False, True])
def test_solve_matfree_residual(precond):
    """The matrix-free CG / PCG solves the assembled system: |A X - B| small."""
    from rxmesh_gb300 import RXMeshStatic, mcf_init_b, mcf_solve_matfree
    from rxmesh_gb300._solvers import mcf_assemble
    v, f = meshgen.icosphere(5)
    x = meshgen.radial_noise(v, 0.02, 4)
    rx = RXMeshStatic(f, len(x), patch_size=256)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    B = mcf_init_b(rx, xl)
    X = xl.clone()
    st = mcf_solve_matfree(rx, xl, B, X, 0.01, max_iter=5000, rel_tol=1e-20, precond=precond)
    assert st["converged"]
    A, _ = mcf_assemble(rx, xl, 0.01, torch.float64)
    S = A.to_scipy()
    r = S @ X.cpu().numpy() - B.cpu().numpy()
    assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(B.cpu().numpy())


def test_solve_matfree_fp32():
    """The FP32 operator (positions rounded to FP32 once per call or solve):
    a product with FP64 positions equals the product with the same positions
    pre-rounded to FP32, bit for bit; the FP32 PCG converges and its solution
    satisfies the FP64 assembled system to FP32 accuracy."""
    from rxmesh_gb300 import RXMeshStatic, mcf_init_b, mcf_matvec, mcf_solve_matfree
    from rxmesh_gb300._solvers import mcf_assemble
    v, f = meshgen.icosphere(5)
    x = meshgen.radial_noise(v, 0.02, 4)
    rx = RXMeshStatic(f, len(x), patch_size=256)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    u = torch.randn_like(xl).float()
    assert torch.equal(mcf_matvec(rx, xl, u, 0.01), mcf_matvec(rx, xl.float().double(), u, 0.01))
    B = mcf_init_b(rx, xl)
    X = xl.float().clone()
    st = mcf_solve_matfree(rx, xl, B.float(), X, 0.01, max_iter=2000, rel_tol=1e-8, precond=True)
    assert st["converged"], st
    A, _ = mcf_assemble(rx, xl, 0.01, torch.float64)
    r = A.to_scipy() @ X.double().cpu().numpy() - B.cpu().numpy()
    assert np.linalg.norm(r) <= 1e-3 * np.linalg.norm(B.cpu().numpy())


def test_step_matfree_matches_assembled_step_and_oracle(oracle):
    """Three matrix-free MCF steps equal three assembled FP64 steps (the same
    Jacobi PCG and stopping rule) and the oracle's steps."""
    from rxmesh_gb300 import RXMeshStatic, mcf_step, mcf_step_matfree
    v, f = meshgen.icosphere(5)
    x = meshgen.radial_noise(v, 0.02, 6)
    rx = RXMeshStatic(f, len(x), patch_size=256)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    xa, xm = xl.clone(), xl.clone()
    sa = mcf_step(rx, xa, 1e-3, 3, "f64", tol=1e-10)
    sm = mcf_step_matfree(rx, xm, 1e-3, 3, tol=1e-10)
    assert sa["converged"] and sm["converged"]
    assert (xa - xm).abs().max().item() <= 1e-9 * xa.abs().max().item()
    xo = x
    for _ in range(3):
        rp, col, val, B = oracle.mcf_system(f, xo, 1e-3)
        xo = oracle.cg(rp, col, val, B, xo, 20000, 0.0, 1e-24, True)[0]
    got = rx.to_input(xm).cpu().numpy()
    assert np.linalg.norm(got - xo) / np.linalg.norm(xo) <= 1e-9
