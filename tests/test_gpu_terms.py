"""Generic per-face energy terms: Param's symmetric Dirichlet energy
(apps/Param/param.cu:146-183) evaluated through the forward-mode Scalar of
include/rxg/diff.cuh and assembled by rxg_face_term_gather, against the
oracle's energy, torch float64 autograd (gradient and full Hessian) and
central differences; a Newton solve on it with 2x2-block Hessians."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import torch

from rxmesh_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bent_grid(n=12, seed=0):
    """n x n grid bent out of its plane (rest shape) and uv = the flat grid
    plus a small jitter (no flipped triangle)."""
    x, f = meshgen.plane(n, n, 1.0 / (n - 1))
    f = np.asarray(f)[:, [0, 2, 1]]  # counter-clockwise in the (x, y) plane: det(M) > 0
    rng = np.random.default_rng(seed)
    rest = x.copy()
    rest[:, 2] = 0.25 * np.sin(2.0 * rest[:, 0]) * np.cos(1.5 * rest[:, 1])
    uv = x[:, :2] + 0.01 / n * rng.normal(size=(len(x), 2))
    return rest, uv, np.asarray(f, np.int32)


def torch_energy(fv, minv, uv):
    """The same energy as a torch float64 function of uv (nv, 2)."""
    f = torch.tensor(np.asarray(fv, np.int64))
    mi = torch.tensor(np.asarray(minv, np.float64).reshape(-1, 2, 2))
    a, b, c = uv[f[:, 0]], uv[f[:, 1]], uv[f[:, 2]]
    M = torch.stack([b - a, c - a], dim=2)
    A = 0.5 / torch.linalg.det(mi)
    J = M @ mi
    return (A * ((J ** 2).sum((1, 2)) + (torch.linalg.inv(J) ** 2).sum((1, 2)))).sum()


def setup(dtype, n=12, proj=False):
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    rest, uv, f = bent_grid(n)
    rx = RXMeshStatic(f, len(rest), patch_size=64)
    prob = DiffScalarProblem(rx, dtype, dim=2)
    prob.add_symmetric_dirichlet_term(rx.to_linear(torch.tensor(rest, device="cuda")), project_hessian=proj)
    uvl = rx.to_linear(torch.tensor(uv, device="cuda")).to(dtype)
    return rx, prob, rest, uv, f, uvl


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-11), (torch.float32, 2e-4)])
def test_symmetric_dirichlet_matches_oracle_and_autograd(oracle, dtype, rtol):
    rx, prob, rest, uv, f, uvl = setup(dtype)
    prob.eval_terms(uvl)
    minv, _ = oracle.rest_frame(f, rest)
    fe = oracle.symmetric_dirichlet(f, uv.astype(np.float32).astype(np.float64)
                                    if dtype == torch.float32 else uv, minv)
    fl = rx.linear_to_input("f")
    assert np.abs(prob.face_energy.double().cpu().numpy() - fe[fl]).max() <= rtol * fe.max()
    assert abs(prob.get_current_loss() - fe.sum()) <= rtol * fe.sum()
    # gradient and Hessian against torch float64 autograd of the whole energy
    u = torch.tensor(uv if dtype == torch.float64 else uv.astype(np.float32).astype(np.float64),
                     requires_grad=True)
    g_ref = torch.autograd.grad(torch_energy(f, minv, u), u)[0].numpy()
    gg = rx.to_input(prob.grad).double().cpu().numpy()
    assert np.abs(gg - g_ref).max() <= rtol * np.abs(g_ref).max()
    H_ref = torch.autograd.functional.hessian(lambda z: torch_energy(f, minv, z.reshape(-1, 2)),
                                              u.detach().reshape(-1)).numpy()
    H = prob.hess.to_scipy().toarray()
    vl = rx.linear_to_input("v")
    perm = np.empty(2 * len(vl), np.int64)  # linear (v, c) -> input (vl[v], c)
    perm[0::2], perm[1::2] = 2 * vl, 2 * vl + 1
    Hin = np.zeros_like(H)
    Hin[np.ix_(perm, perm)] = H
    assert np.abs(Hin - H_ref).max() <= rtol * np.abs(H_ref).max()


@pytest.mark.gpu
def test_symmetric_dirichlet_central_differences():
    rx, prob, rest, uv, f, uvl = setup(torch.float64)
    prob.eval_terms(uvl)
    g = prob.grad.clone()
    rng = np.random.default_rng(1)
    h = 1e-6
    for _ in range(16):
        d = torch.tensor(rng.normal(size=uvl.shape), device="cuda")
        fd = (prob.eval_terms_passive(uvl + h * d).item() - prob.eval_terms_passive(uvl - h * d).item()) / (2 * h)
        an = (g * d).sum().item()
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1.0), (fd, an)


@pytest.mark.gpu
def test_flipped_face_gets_the_largest_value_and_no_derivative(oracle):
    rx, prob, rest, uv, f, uvl = setup(torch.float64)
    uv2 = uv.copy()
    t = f[7]
    uv2[t[0]], uv2[t[1]] = uv[t[1]].copy(), uv[t[0]].copy()  # swap two corners: flipped
    prob.eval_terms(rx.to_linear(torch.tensor(uv2, device="cuda")))
    fl = rx.linear_to_input("f")
    fe = prob.face_energy.cpu().numpy()[np.argsort(fl)]
    assert fe[7] == np.finfo(np.float64).max


@pytest.mark.gpu
def test_projected_hessian_is_positive_semidefinite():
    rx, prob, rest, uv, f, uvl = setup(torch.float64, proj=True)
    # a stretched state, where the unprojected Hessian is indefinite
    prob.eval_terms(uvl * torch.tensor([1.6, 0.5], dtype=torch.float64, device="cuda"))
    H = prob.hess.to_scipy().toarray()
    assert np.linalg.eigvalsh(0.5 * (H + H.T)).min() >= -1e-9 * np.abs(H).max()


@pytest.mark.gpu
def test_newton_on_symmetric_dirichlet_decreases_energy():
    """Param's Newton loop (diff/newton_solver.h) on the 2x2-block Hessian:
    projected Hessian, PCG on its scalar form, Armijo line search."""
    from rxmesh_gb300 import NewtonSolver
    rx, prob, rest, uv, f, uvl = setup(torch.float64, n=16, proj=True)
    x = uvl * torch.tensor([1.3, 0.8], dtype=torch.float64, device="cuda")
    prob.eval_terms(x)
    e = [prob.get_current_loss()]
    newton = NewtonSolver(prob, "pcg", max_iter=2000, abs_tol=0.0, rel_tol=1e-12)
    for _ in range(6):
        prob.eval_terms()
        newton.compute_direction()
        assert newton.line_search()
        prob.eval_terms()
        e.append(prob.get_current_loss())
    assert all(b <= a + 1e-12 for a, b in zip(e, e[1:])), e
    assert e[-1] < 0.9 * e[0], e


@pytest.fixture(scope="module")
def term_example(tmp_path_factory):
    """tests/cpp/term_example.cu: energies written by the application with
    include/rxg/diff.cuh, built with nvcc against librxg.so."""
    from rxmesh_gb300 import _lib
    _lib.load()
    libdir = os.path.dirname(_lib.lib_path())
    exe = str(tmp_path_factory.mktemp("terms") / "term_example")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-std=c++17", "--extended-lambda", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           os.path.join(ROOT, "tests", "cpp", "term_example.cu"), "-I", os.path.join(ROOT, "include"),
           "-L", libdir, "-lrxg", "-Xlinker", "-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_term_example_compiles(term_example):
    assert os.path.exists(term_example)


@pytest.mark.gpu
def test_application_written_terms(term_example, tmp_path):
    """The application's symmetric Dirichlet lambda equals the built-in term
    (checked inside the program), and its spring energy's gradient equals
    the analytic one: sum over the faces' edges of k (x_i - x_j)."""
    r = subprocess.run([term_example, str(tmp_path)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
    ld = lambda n, t: np.fromfile(str(tmp_path / (n + ".bin")), dtype=t)
    g = ld("spring_grad", np.float64).reshape(-1, 3)
    x = ld("rest", np.float64).reshape(-1, 3)  # linear order
    l2i = ld("l2i", np.int32)
    f = ld("fv", np.int32).reshape(-1, 3)      # input ids
    il = np.empty_like(l2i)
    il[l2i] = np.arange(len(l2i))
    fl = il[f]
    want = np.zeros_like(x)
    for i in range(3):
        a, b = fl[:, i], fl[:, (i + 1) % 3]
        d = 2.5 * (x[a] - x[b])
        np.add.at(want, a, d)
        np.add.at(want, b, -d)
    assert np.abs(g - want).max() <= 1e-12 * np.abs(want).max()


# ---- terms given by their records (add_term<Op::FV / EV / V>) -------------

def element_records(energy, xe):
    """Records [E, gradient, packed upper Hessian] of energy(xe_i) for each
    row xe_i of xe (n, K), by torch.func (the reference's forward-mode
    Scalar computes the same three quantities per element)."""
    from torch.func import grad, hessian, vmap
    K = xe.shape[1]
    E = vmap(energy)(xe)
    G = vmap(grad(energy))(xe)
    H = vmap(hessian(energy))(xe)
    iu = torch.triu_indices(K, K, device=xe.device)  # row-major upper triangle
    return torch.cat([E[:, None], G, H[:, iu[0], iu[1]]], dim=1)


def spring_mesh(n=10, seed=3):
    from rxmesh_gb300 import RXMeshStatic
    rest, uv, f = bent_grid(n, seed)
    rx = RXMeshStatic(f, len(rest), patch_size=32)
    x = rx.to_linear(torch.tensor(rest, device="cuda"))
    x = x + 0.05 * torch.randn(x.shape, generator=torch.Generator("cpu").manual_seed(seed),
                               dtype=torch.float64).to(x.device)
    return rx, x


def spring(L):
    """A nonlinear edge energy: (|x0 - x1|^2 - L^2)^2, plus a vertex-pair
    coupling so the Hessian blocks are not multiples of I."""
    def e(xe):
        d = xe[:3] - xe[3:]
        return (d @ d - L * L) ** 2 + 0.3 * torch.sin(xe[0] * xe[4])
    return e


def vertex_energy(xv):
    return torch.sin(xv[0]) * xv[1] + 0.5 * (xv ** 2).sum() * torch.cos(xv[2])


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-11), (torch.float32, 2e-4)])
def test_edge_and_vertex_terms_match_autograd(dtype, rtol):
    """An edge term and a vertex term (records from torch.func) assembled by
    rxg_edge_term_gather / rxg_vertex_term_gather: energy, gradient and the
    block Hessian equal torch autograd of the summed energy (FP64)."""
    from rxmesh_gb300 import DiffScalarProblem
    rx, x = spring_mesh()
    ev = rx.query("EV")[1].reshape(-1, 2).long()
    L = 0.08
    prob = DiffScalarProblem(rx, dtype, dim=3)
    prob.add_term("EV", lambda x: element_records(spring(L), torch.cat([x[ev[:, 0]], x[ev[:, 1]]], 1)))
    prob.add_term("V", lambda x: element_records(vertex_energy, x))
    xd = x.to(dtype)
    prob.eval_terms(xd)

    evc = ev.cpu()

    def total(y):
        d = y[evc[:, 0]] - y[evc[:, 1]]
        e = ((d * d).sum(1) - L * L) ** 2 + 0.3 * torch.sin(y[evc[:, 0], 0] * y[evc[:, 1], 1])
        v = torch.sin(y[:, 0]) * y[:, 1] + 0.5 * (y ** 2).sum(1) * torch.cos(y[:, 2])
        return e.sum() + v.sum()

    x64 = xd.double().cpu().requires_grad_(True)
    E = total(x64)
    g = torch.autograd.grad(E, x64)[0]
    H = torch.autograd.functional.hessian(total, x64.detach()).reshape(x64.numel(), x64.numel())
    assert abs(prob.get_current_loss() - E.item()) <= rtol * abs(E.item())
    assert torch.allclose(prob.grad.double().cpu(), g, rtol=0, atol=rtol * g.abs().max().item())
    Hg = torch.tensor(prob.hess.to_scipy().toarray())
    assert (Hg - H).abs().max().item() <= rtol * H.abs().max().item()


@pytest.mark.gpu
def test_face_edge_vertex_records_accumulate():
    """A face term given by records, an edge term and the inertia term in one
    problem: the gradient and Hessian are the sums of the separate ones."""
    from rxmesh_gb300 import DiffScalarProblem
    rx, x = spring_mesh(8)
    fv = rx.query("FV")[1].reshape(-1, 3).long()
    ev = rx.query("EV")[1].reshape(-1, 2).long()

    def face_e(xe):
        a, b, c = xe[:3], xe[3:6], xe[6:]
        n = torch.linalg.cross(b - a, c - a)
        return (n @ n) + (a @ c) * 0.1

    fterm = lambda y: element_records(face_e, torch.cat([y[fv[:, 0]], y[fv[:, 1]], y[fv[:, 2]]], 1))
    eterm = lambda y: element_records(spring(0.1), torch.cat([y[ev[:, 0]], y[ev[:, 1]]], 1))
    parts = []
    for terms in (["f"], ["e"], ["i"], ["f", "e", "i"]):
        p = DiffScalarProblem(rx, torch.float64, dim=3)
        for t in terms:
            if t == "f":
                p.add_term("FV", fterm)
            elif t == "e":
                p.add_term("EV", eterm)
            else:
                p.add_inertia_term(x * 0.9, 2.0)
        p.eval_terms(x)
        parts.append((p.get_current_loss(), p.grad.clone(), p.hess.val.clone(), p.face_energy.clone()))
    e_sum = sum(q[0] for q in parts[:3])
    assert abs(parts[3][0] - e_sum) <= 1e-12 * abs(e_sum)
    g_sum = parts[0][1] + parts[1][1] + parts[2][1]
    assert torch.allclose(parts[3][1], g_sum, rtol=0, atol=1e-12 * g_sum.abs().max().item())
    h_sum = parts[0][2] + parts[1][2] + parts[2][2]
    assert torch.allclose(parts[3][2], h_sum, rtol=0, atol=1e-12 * h_sum.abs().max().item())
    # per-face energies: those of the face term
    assert torch.equal(parts[3][3], parts[0][3])


@pytest.mark.gpu
def test_smoothing_newton_brings_vertices_together():
    """Diff.SmoothingNewton (tests/RXMesh_test/test_grad.h:14-105): the edge
    term |x_0 - x_1|^2 in FP32, Newton steps with PCG on its Hessian (the
    graph Laplacian, singular but consistent) until 0.5 grad . dir < 1e-2;
    every vertex ends at one position (within 1e-3)."""
    from rxmesh_gb300 import DiffScalarProblem, NewtonSolver
    rx, x = spring_mesh(12)
    ev = rx.query("EV")[1].reshape(-1, 2).long()
    prob = DiffScalarProblem(rx, torch.float32, dim=3)
    sq = lambda xe: ((xe[:3] - xe[3:]) ** 2).sum()
    prob.add_term("EV", lambda y: element_records(sq, torch.cat([y[ev[:, 0]], y[ev[:, 1]]], 1)))
    X = x.float().contiguous()
    prob.opt_var = X
    newton = NewtonSolver(prob, "pcg", max_iter=2000, abs_tol=0.0, rel_tol=1e-6)
    for it in range(100):
        prob.eval_terms()
        newton.compute_direction()
        if 0.5 * float((prob.grad * newton.dir).sum()) < 1e-2:
            break
        newton.line_search()
    assert it < 100
    assert (X - X[0]).abs().max().item() <= 1e-3


@pytest.mark.gpu
def test_while_loop_vertex_term_dim1():
    """Diff.WhileLoop (tests/RXMesh_test/test_grad.h:107-211) with one
    component per vertex: the vertex term sqrt(a) computed by a Newton loop;
    its gradient is 1 / (2 sqrt(a)).  (The loop itself runs in the C++
    example's device lambda; here the records of sqrt are given directly.)"""
    from rxmesh_gb300 import DiffScalarProblem
    rx, x = spring_mesh(9)
    a = (x[:, 0] - 0.37) ** 2
    prob = DiffScalarProblem(rx, torch.float32, assemble_hessian=False, dim=1)
    prob.add_term("V", lambda y: element_records(lambda v: torch.sqrt(v[0]), y))
    prob.eval_terms(a.float().reshape(-1, 1).contiguous())
    s = a.sqrt()
    keep = s > 1e-3
    g = prob.grad[:, 0].double()
    assert keep.sum().item() > 0
    assert (g[keep] - 1.0 / (2.0 * s[keep])).abs().max().item() <= 1e-3


def test_term_records_shape_is_checked():
    """A records function of the wrong width is refused before any call."""
    from rxmesh_gb300._diff import DiffScalarProblem
    p = DiffScalarProblem.__new__(DiffScalarProblem)
    with pytest.raises(ValueError):
        DiffScalarProblem.add_term(p, "FE", lambda x: x)


@pytest.fixture(scope="module")
def diff_arap_example(tmp_path_factory):
    """tests/cpp/diff_arap_example.cu: the reference's DiffARAP application
    (EVDiamond cotangent weights, per-vertex rotations over VE, a per-edge
    add_term<Op::EV, true>, Newton with constraints) on the facade."""
    from rxmesh_gb300 import _lib
    _lib.load()
    libdir = os.path.dirname(_lib.lib_path())
    exe = str(tmp_path_factory.mktemp("diffarap") / "diff_arap_example")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-std=c++17", "--extended-lambda", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           os.path.join(ROOT, "tests", "cpp", "diff_arap_example.cu"), "-I", os.path.join(ROOT, "include"),
           "-L", libdir, "-lrxg", "-Xlinker", "-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_diff_arap_example_compiles(diff_arap_example):
    assert os.path.exists(diff_arap_example)


@pytest.mark.gpu
def test_diff_arap_application(diff_arap_example):
    """The DiffARAP steps: weights equal the host formula on the EVD query,
    rotations are proper (R^T R = I, det 1; identity when undeformed), each
    Newton solve converges and lowers the energy, which equals the host sum
    at the final state, local/global iterations do not raise it, and the
    constrained vertices stay where the constraints put them."""
    r = subprocess.run([diff_arap_example], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


@pytest.mark.gpu
def test_newton_on_one_component_variable():
    """Newton with 1x1 blocks (dim=1): the vertex term (a - t)^2 per vertex
    plus the edge term (a0 - a1)^2 (a graph Laplacian) is quadratic, so one
    Newton step (PCG on the scalar form of the 1x1-block Hessian) reaches
    its minimiser: H a = t, checked against scipy; a constrained vertex
    keeps its value (apply_bc)."""
    import scipy.sparse.linalg as spl
    from rxmesh_gb300 import DiffScalarProblem, NewtonSolver
    rx, x = spring_mesh(10)
    ev = rx.query("EV")[1].reshape(-1, 2).long()
    t = torch.sin(3.0 * x[:, 0]) + x[:, 1]
    prob = DiffScalarProblem(rx, torch.float64, dim=1)
    tt = t.reshape(-1, 1)
    prob.add_term("V", lambda y: torch.cat([((y - tt) ** 2), 2 * (y - tt), torch.full_like(y, 2.0)], 1))
    prob.add_term("EV", lambda y: element_records(lambda e: (e[0] - e[1]) ** 2,
                                                  torch.cat([y[ev[:, 0]], y[ev[:, 1]]], 1)))
    a = torch.zeros(rx.get_num_vertices(), 1, dtype=torch.float64, device="cuda")
    prob.opt_var = a
    newton = NewtonSolver(prob, "pcg", max_iter=5000, abs_tol=0.0, rel_tol=1e-24)
    bc = torch.zeros(rx.get_num_vertices(), dtype=torch.int8, device="cuda")
    bc[0] = 1
    prob.eval_terms()
    newton.apply_bc(bc)
    newton.compute_direction()
    newton.line_search()
    prob.eval_terms()
    H = prob.hess.to_scipy().tocsr()
    free = np.arange(1, rx.get_num_vertices())
    want = np.zeros(rx.get_num_vertices())
    Hf = H[free][:, free]
    want[free] = spl.spsolve(Hf.tocsc(), 2.0 * t.cpu().numpy()[free])
    got = a[:, 0].cpu().numpy()
    assert got[0] == 0.0
    assert np.abs(got - want).max() <= 1e-8 * np.abs(want).max()
