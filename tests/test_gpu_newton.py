"""Newton step of the differentiable path (NewtonSolver, diff/newton_solver.h):
the scalar form of the block Hessian, the boundary conditions, the direction
H dir = -grad, and whole Newton iterations with the backtracking line search,
against a numpy / scipy restatement on the oracle's projected Hessian."""
import numpy as np
import pytest
import torch

from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu
sp = pytest.importorskip("scipy.sparse")
spla = pytest.importorskip("scipy.sparse.linalg")


def cloth(n=24, seed=4):
    x0, f = meshgen.plane(n, n, 1.0 / (n - 1))
    rng = np.random.default_rng(seed)
    x = x0.copy()
    corners = [0, n - 1, n * (n - 1), n * n - 1]
    x[corners] += rng.uniform(-0.2, 0.2, size=(4, 3))
    x += 0.01 * rng.normal(size=x.shape)
    return x0, x, f, corners


def setup(dtype=torch.float64):
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    x0, x, f, corners = cloth()
    rx = RXMeshStatic(f, len(x0), patch_size=128)
    x0l = rx.to_linear(torch.tensor(x0, device="cuda"))
    xl = rx.to_linear(torch.tensor(x, device="cuda")).to(dtype)
    prob = DiffScalarProblem(rx, dtype).add_arap_term(x0l, project_hessian=True)
    il = rx.input_to_linear("v")
    bc = torch.zeros(len(x0), dtype=torch.int8, device="cuda")
    bc[torch.tensor(il[corners], device="cuda", dtype=torch.long)] = 1
    return rx, prob, xl, bc, (x0, x, f, corners)


def oracle_system(oracle, rx, prob, f, x0, x, bc_in, eps=1e-9):
    """E, g (nv,3), H (scipy, input ids) with projection and boundary conditions."""
    minv, area = oracle.rest_frame(f, x0)
    vl = rx.linear_to_input("v")
    il = rx.input_to_linear("v")
    rp = prob.hess.row_ptr.cpu().numpy().astype(np.int64)
    col = prob.hess.col.cpu().numpy()
    nv = len(vl)
    rp_in = np.zeros(nv + 1, np.int64)
    order = []
    for p in range(nv):
        lin = il[p]
        order.append(np.arange(rp[lin], rp[lin + 1]))
        rp_in[p + 1] = rp_in[p] + rp[lin + 1] - rp[lin]
    order = np.concatenate(order)
    col_in = vl[col][order].astype(np.int32)
    E, _, g, H = oracle.arap_assemble(f, x, minv, area, rp_in, col_in, project=True, eps=eps)
    H = H.copy()
    g = g.copy()
    rows = np.repeat(np.arange(nv), np.diff(rp_in))
    for t in range(len(col_in)):
        i, j = rows[t], col_in[t]
        if i == j and bc_in[i]:
            H[t] = np.eye(3)
        elif i != j and (bc_in[i] or bc_in[j]):
            H[t] = 0
    g[bc_in.astype(bool)] = 0
    A = sp.bsr_matrix((H, col_in, rp_in), shape=(3 * nv, 3 * nv)).tocsr()
    return E, g, A


def test_bcsr_to_csr_and_apply_bc():
    rx, prob, xl, bc, _ = setup()
    prob.eval_terms(xl)
    B = prob.hess.to_scipy().tocsr()
    A = prob.hess.to_csr()
    S = sp.csr_matrix((A.val.cpu().numpy(), A.col.cpu().numpy(), A.row_ptr.cpu().numpy()),
                      shape=B.shape)
    assert abs(S - B).max() == 0
    # boundary conditions on the block form against a numpy restatement
    H = prob.hess.val.cpu().numpy().copy()
    rp = prob.hess.row_ptr.cpu().numpy()
    col = prob.hess.col.cpu().numpy()
    b = bc.cpu().numpy().astype(bool)
    g = prob.grad.cpu().numpy().copy()
    for i in range(len(rp) - 1):
        for t in range(rp[i], rp[i + 1]):
            j = col[t]
            if i == j and b[i]:
                H[t] = np.eye(3)
            elif i != j and (b[i] or b[j]):
                H[t] = 0
    g[b] = 0
    prob.hess.apply_bc(bc, prob.grad)
    assert np.array_equal(prob.hess.val.cpu().numpy(), H)
    assert np.array_equal(prob.grad.cpu().numpy(), g)


def test_direction_matches_direct_solve(oracle):
    from rxmesh_gb300 import NewtonSolver
    rx, prob, xl, bc, (x0, x, f, corners) = setup()
    prob.eval_terms(xl)
    prob.hess.apply_bc(bc, prob.grad)
    newton = NewtonSolver(prob, "pcg", max_iter=5000, abs_tol=0.0, rel_tol=1e-24)
    g_before = prob.grad.clone()
    newton.compute_direction()
    assert torch.equal(prob.grad, -g_before)  # left negated, as the reference does
    bc_in = np.zeros(len(x0), bool)
    bc_in[corners] = True
    E, g, A = oracle_system(oracle, rx, prob, f, x0, x, bc_in)
    want = spla.spsolve(A.tocsc(), -g.reshape(-1)).reshape(-1, 3)
    got = rx.to_input(newton.dir).cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-8 * np.linalg.norm(want)
    assert abs(prob.get_current_loss() - E) <= 1e-10 * abs(E)


def test_newton_iterations_match_oracle(oracle):
    """Five Newton iterations with the corners fixed: the same step lengths and
    energies as a numpy restatement of compute_direction + line_search."""
    from rxmesh_gb300 import NewtonSolver
    rx, prob, xl, bc, (x0, x, f, corners) = setup()
    newton = NewtonSolver(prob, "pcg", max_iter=5000, abs_tol=0.0, rel_tol=1e-24)
    bc_in = np.zeros(len(x0), bool)
    bc_in[corners] = True
    minv, area = oracle.rest_frame(f, x0)
    xo = x.copy()
    energies = []
    for it in range(5):
        prob.eval_terms(xl)
        prob.hess.apply_bc(bc, prob.grad)
        newton.compute_direction()
        assert newton.line_search()
        energies.append(prob.get_current_loss())
        # restatement
        E, g, A = oracle_system(oracle, rx, prob, f, x0, xo, bc_in)
        ng = -g.reshape(-1)
        d = spla.spsolve(A.tocsc(), ng)
        slope = float(d @ ng)
        s = 1.0
        for _ in range(64):
            t = xo + s * d.reshape(-1, 3)
            En = oracle.arap_assemble(f, t, minv, area, np.zeros(len(x0) + 1, np.int64),
                                      np.zeros(0, np.int32), want_hess=False)[0]
            if En <= E + 1e-4 * s * slope:
                break
            s *= 0.8
        xo = t
        assert abs(energies[-1] - En) <= 1e-8 * abs(En), (it, energies[-1], En)
    assert energies[-1] < energies[0]
    got = rx.to_input(xl).cpu().numpy()
    assert np.abs(got - xo).max() <= 1e-8


@pytest.mark.parametrize("project", [False, True])
@pytest.mark.parametrize("with_bc", [False, True])
def test_hessian_vector_product_matches_assembled(project, with_bc):
    """eval_matvec (diff_query_kernel.cuh:26-148) without assembly equals the
    assembled Hessian (after apply_bc when constrained) times v."""
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    x0, x, f, corners = cloth()
    rx = RXMeshStatic(f, len(x0), patch_size=128)
    x0l = rx.to_linear(torch.tensor(x0, device="cuda"))
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    prob = DiffScalarProblem(rx, torch.float64).add_arap_term(x0l, project_hessian=project)
    prob.eval_terms(xl)
    bc = None
    if with_bc:
        bc = torch.zeros(len(x0), dtype=torch.int8, device="cuda")
        bc[torch.tensor(rx.input_to_linear("v")[corners], device="cuda", dtype=torch.long)] = 1
        prob.hess.apply_bc(bc, prob.grad)
    H = prob.hess.to_scipy().tocsr()
    v = torch.randn(len(x0), 3, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(5))
    y = prob.eval_matvec(v, bc=bc).cpu().numpy().reshape(-1)
    want = H @ v.cpu().numpy().reshape(-1)
    assert np.abs(y - want).max() <= 1e-12 * np.abs(want).max()


def test_matfree_newton_matches_assembled():
    """CGMatFreeSolver path: the same directions and iterates as PCG on the
    assembled, projected, constrained Hessian (both solved tightly)."""
    from rxmesh_gb300 import NewtonSolver
    rx, prob, xl, bc, _ = setup()
    rx2, prob2, xl2, bc2, _ = setup()
    a = NewtonSolver(prob, "pcg", max_iter=5000, abs_tol=0.0, rel_tol=1e-26)
    b = NewtonSolver(prob2, "cg_matfree", max_iter=5000, abs_tol=0.0, rel_tol=1e-26)
    for it in range(3):
        prob.eval_terms(xl)
        a.apply_bc(bc)
        a.compute_direction()
        prob2.eval_terms(xl2)
        b.apply_bc(bc2)
        b.compute_direction()
        assert torch.norm(a.dir - b.dir) <= 1e-8 * torch.norm(a.dir), it
        assert b.iter_taken() > 0
        assert a.line_search() and b.line_search()
        assert abs(prob.get_current_loss() - prob2.get_current_loss()) <= 1e-9 * abs(prob.get_current_loss())
    assert torch.allclose(xl, xl2, rtol=0, atol=1e-8)


def test_inertia_hessian_is_mass_identity():
    """The reference's Diff.Hess (tests/RXMesh_test/test_hess.cu:117-153):
    the inertia term's Hessian on a 16 x 16 plane (dx = 1/15) is mass I on
    the diagonal and zero elsewhere (the reference checks 1e-3)."""
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    n = 16
    x, f = meshgen.plane(n, n, 1.0 / (n - 1))
    rx = RXMeshStatic(f, len(x), patch_size=64)
    xl = rx.to_linear(torch.tensor(x, device="cuda")).float()
    mass = 0.01
    prob = DiffScalarProblem(rx, torch.float32).add_inertia_term(xl, mass)
    prob.eval_terms(xl)
    H = prob.hess.to_scipy().toarray()
    assert np.abs(np.diag(H) - mass).max() <= 1e-6
    assert np.abs(H - np.diag(np.diag(H))).max() == 0.0
    assert abs(prob.get_current_loss()) == 0.0 and prob.grad.abs().max().item() == 0.0
    # away from the target: E = m/2 |d|^2, gradient m d
    d = torch.randn_like(xl)
    prob.eval_terms(xl + d)
    assert abs(prob.get_current_loss() - 0.5 * mass * float((d.double() ** 2).sum())) <= 1e-5 * prob.get_current_loss()
    assert (prob.grad - mass * d).abs().max().item() <= 1e-6


def test_newton_arap_with_inertia_converges_each_solve():
    """ARAP plus the inertia term (mass 0.01): the Newton system is positive
    definite, so every PCG solve converges (the ARAP term alone has the
    near-null space of isometric bending, where PCG runs to max_iter)."""
    from rxmesh_gb300 import DiffScalarProblem, NewtonSolver, RXMeshStatic
    n = 32
    x0, f = meshgen.plane(n, n, 1.0)
    rng = np.random.default_rng(5)
    x = x0.copy()
    corners = [0, n - 1, n * (n - 1), n * n - 1]
    x[corners] += rng.uniform(-0.2, 0.2, size=(4, 3))
    rx = RXMeshStatic(f, len(x), patch_size=128)
    rest = rx.to_linear(torch.tensor(x0, device="cuda"))
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    prob = (DiffScalarProblem(rx, torch.float64).add_arap_term(rest, project_hessian=True)
            .add_inertia_term(xl, 0.01))
    bc = torch.zeros(len(x), dtype=torch.int8, device="cuda")
    bc[torch.tensor(rx.input_to_linear("v")[corners], device="cuda", dtype=torch.long)] = 1
    newton = NewtonSolver(prob, "pcg", max_iter=2000, abs_tol=0.0, rel_tol=1e-12)
    xn = xl.clone()
    prob.eval_terms(xn)
    e = [prob.get_current_loss()]
    for _ in range(4):
        prob.eval_terms()
        newton.apply_bc(bc)
        newton.compute_direction()
        assert newton.solver.converged() and newton.iter_taken() < 2000
        newton.line_search()
        prob.eval_terms()
        e.append(prob.get_current_loss())
    assert all(b <= a for a, b in zip(e, e[1:])), e


def test_dense_zero_rows():
    """rxg_dense_zero_rows (the gradient half of apply_bc without an assembled
    Hessian) zeroes exactly the masked rows, FP32 and FP64."""
    import ctypes
    from rxmesh_gb300 import _lib
    L = _lib.load()
    for dt, code in ((torch.float32, 0), (torch.float64, 1)):
        x = torch.randn(1000, 3, dtype=dt, device="cuda")
        mask = (torch.rand(1000, device="cuda") < 0.3).to(torch.int8)
        want = x.clone()
        want[mask.bool()] = 0
        _lib.check(L.rxg_dense_zero_rows(1000, 3, code, ctypes.c_void_p(mask.data_ptr()),
                                         ctypes.c_void_p(x.data_ptr()), None))
        assert torch.equal(x, want)
