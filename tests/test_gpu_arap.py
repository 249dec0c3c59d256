"""GPU parity of the per-face ARAP energy, gradient and block Hessian."""
import numpy as np
import pytest
import torch

from conftest import golden
from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu


def cloth(n=24, seed=4):
    """create_plane grid, flat rest shape, corners displaced (the cloth workload, small)."""
    x0, f = meshgen.plane(n, n, 1.0 / (n - 1))
    rng = np.random.default_rng(seed)
    x = x0.copy()
    corners = [0, n - 1, n * (n - 1), n * n - 1]
    x[corners] += rng.uniform(-0.2, 0.2, size=(4, 3))
    x += 0.01 * rng.normal(size=x.shape)  # generic interior state
    return x0, x, f


def oracle_ref(oracle, f, x0, x, rx, prob, project=False, eps=1e-9):
    minv, area = oracle.rest_frame(f, x0)
    rp = prob.hess.row_ptr.cpu().numpy().astype(np.int64)
    vl = rx.linear_to_input("v")
    col_in = vl[prob.hess.col.cpu().numpy()]
    # oracle assembles on the GPU's block pattern, expressed in input ids
    il = rx.input_to_linear("v")
    rows = np.repeat(np.arange(len(vl)), np.diff(rp))
    order = []
    rp_in = np.zeros(len(vl) + 1, np.int64)
    for p in range(len(vl)):
        lin = il[p]
        order.append(np.arange(rp[lin], rp[lin + 1]))
        rp_in[p + 1] = rp_in[p] + rp[lin + 1] - rp[lin]
    order = np.concatenate(order)
    E, fE, g, H = oracle.arap_assemble(f, x, minv, area, rp_in, col_in[order].astype(np.int32),
                                       project=project, eps=eps)
    Hlin = np.empty_like(H)
    Hlin[order] = H
    return E, fE, g, Hlin, minv


@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-11), (torch.float32, 2e-4)])
@pytest.mark.parametrize("kind", ["cloth", "bunnyhead", "sphere", "cloth_one_patch"])
@pytest.mark.parametrize("with_hessian", [True, False])
def test_arap_matches_oracle(oracle, dtype, rtol, kind, with_hessian):
    """cloth_one_patch: the whole 3,042-face cloth in one patch.  with_hessian
    False: the gradient-only evaluation agrees with the full one."""
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    patch = 128
    if kind == "cloth":
        x0, x, f = cloth()
    elif kind == "cloth_one_patch":
        x0, x, f = cloth(40, 6)
        patch = 4096
    elif kind == "bunnyhead":
        g = golden("bunnyhead")
        x0, f = g["xyz"], g["fv"]
        x = x0 + 0.002 * np.random.default_rng(1).normal(size=x0.shape)
    else:
        v, f = meshgen.icosphere(3)
        x0 = v
        x = meshgen.radial_noise(v, 0.05, 2)
    rx = RXMeshStatic(f, len(x0), patch_size=patch)
    dev = "cuda"
    x0l = rx.to_linear(torch.tensor(x0, device=dev))
    xl = rx.to_linear(torch.tensor(x, device=dev))
    prob = DiffScalarProblem(rx, dtype).add_arap_term(x0l)
    if not with_hessian:
        # gradient and energies alone first; the full evaluation below must agree
        prob.eval_terms(xl, with_hessian=False)
        g_only = prob.grad.clone()
        e_only = prob.get_current_loss()
    prob.eval_terms(xl)
    if not with_hessian:
        tol = 1e-12 if dtype == torch.float64 else 1e-6
        scale = prob.grad.abs().max().item()
        assert (g_only - prob.grad).abs().max().item() <= tol * scale
        assert abs(e_only - prob.get_current_loss()) <= tol * abs(e_only)
    E, fE, g, H, minv = oracle_ref(oracle, f, x0, x, rx, prob)
    # rest frames
    fl = rx.linear_to_input("f")
    assert np.abs(prob.rest.double().cpu().numpy() - minv[fl].reshape(-1, 4)).max() <= rtol * np.abs(minv).max()
    assert abs(prob.get_current_loss() - E) <= rtol * abs(E) + 1e-300
    fe = prob.face_energy.double().cpu().numpy()
    assert np.abs(fe - fE[fl]).max() <= rtol * np.abs(fE).max()
    gg = rx.to_input(prob.grad).double().cpu().numpy()
    assert np.abs(gg - g).max() <= rtol * np.abs(g).max()
    Hg = prob.hess.val.double().cpu().numpy()
    assert np.abs(Hg - H).max() <= rtol * np.abs(H).max()


def test_arap_gradient_central_differences():
    # FP64 central differences h = 1e-6 on random directions
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    x0, x, f = cloth(12, seed=9)
    rx = RXMeshStatic(f, len(x0), patch_size=64)
    x0l = rx.to_linear(torch.tensor(x0, device="cuda"))
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    prob = DiffScalarProblem(rx, torch.float64).add_arap_term(x0l)
    prob.eval_terms(xl)
    g = prob.grad.clone()
    Hs = prob.hess.to_scipy()
    rng = np.random.default_rng(0)
    h = 1e-6
    for _ in range(16):
        d = torch.tensor(rng.normal(size=x.shape), device="cuda")
        ep = prob.eval_terms(xl + h * d, with_hessian=False).item()
        em = prob.eval_terms(xl - h * d, with_hessian=False).item()
        fd = (ep - em) / (2 * h)
        an = (g * d).sum().item()
        assert abs(fd - an) <= 1e-5 * max(1.0, abs(an))
        prob.eval_terms(xl + h * d, with_hessian=False)
        gp = prob.grad.clone()
        prob.eval_terms(xl - h * d, with_hessian=False)
        gm = prob.grad.clone()
        fdg = ((gp - gm) / (2 * h)).cpu().numpy().ravel()
        hd = Hs @ d.cpu().numpy().ravel()
        assert np.abs(fdg - hd).max() <= 1e-5 * max(1.0, np.abs(hd).max())


@pytest.mark.parametrize("dtype,rtol,eps", [(torch.float64, 1e-10, 1e-9), (torch.float32, 5e-4, 1e-6)])
@pytest.mark.parametrize("kind", ["cloth", "bunnyhead", "sphere"])
def test_projected_hessian_matches_oracle(oracle, dtype, rtol, eps, kind):
    """add_term<Op::FV, ProjectHess = true>: every face's 9x9 Hessian made
    positive definite before assembly; the assembled Hessian is then positive
    semi-definite, and energy and gradient are those of the plain evaluation."""
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    if kind == "cloth":
        x0, x, f = cloth()
    elif kind == "bunnyhead":
        g = golden("bunnyhead")
        x0, f = g["xyz"], g["fv"]
        x = x0 + 0.002 * np.random.default_rng(1).normal(size=x0.shape)
    else:
        v, f = meshgen.icosphere(3)
        x0 = v
        x = meshgen.radial_noise(v, 0.05, 2)
    rx = RXMeshStatic(f, len(x0), patch_size=128)
    x0l = rx.to_linear(torch.tensor(x0, device="cuda"))
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    plain = DiffScalarProblem(rx, dtype).add_arap_term(x0l)
    plain.eval_terms(xl)
    prob = DiffScalarProblem(rx, dtype).add_arap_term(x0l, project_hessian=True)
    prob.eval_terms(xl)
    E, fE, g, H, _ = oracle_ref(oracle, f, x0, x, rx, prob, project=True, eps=eps)
    assert abs(prob.get_current_loss() - E) <= rtol * abs(E)
    gg = rx.to_input(prob.grad).double().cpu().numpy()
    assert np.abs(gg - g).max() <= rtol * np.abs(g).max()
    assert torch.allclose(prob.grad, plain.grad, rtol=0, atol=1e-6 * plain.grad.abs().max().item())
    Hg = prob.hess.val.double().cpu().numpy()
    assert np.abs(Hg - H).max() <= rtol * np.abs(H).max()
    if kind == "cloth":  # displaced corners: some faces are indefinite, so projection acts
        assert np.abs(Hg - plain.hess.val.double().cpu().numpy()).max() > 1e-3 * np.abs(H).max()
    A = prob.hess.to_scipy().astype(np.float64)
    rng = np.random.default_rng(3)
    for _ in range(8):
        z = rng.normal(size=A.shape[0])
        assert z @ (A @ z) >= -1e-6 * abs(z @ z) * np.abs(H).max()

