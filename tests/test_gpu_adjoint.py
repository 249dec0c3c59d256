"""Adjoint of the implicit MCF step and of the ARAP energy through
torch.autograd, checked against FP64 central differences (h = 1e-6)."""
import numpy as np
import pytest
import torch

from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu


def sphere(level=3, seed=2):
    v, f = meshgen.icosphere(level)
    return meshgen.radial_noise(v, 0.02, seed), f


def cloth(n=16, seed=3):
    """create_plane grid (dx = 1, its default), corners displaced by U(-0.2, 0.2).

    The grid is also jittered by N(0, 0.1): the reference's Voronoi area
    (geometry_util.cuh:117-167) jumps from A to A/4 when an angle crosses 90
    degrees, and an unjittered grid has every quad corner at exactly 90
    degrees, where the flow has no derivative for differences to converge to."""
    x0, f = meshgen.plane(n, n, 1.0)
    rng = np.random.default_rng(seed)
    x = x0.copy()
    for c in [0, n - 1, n * (n - 1), n * n - 1]:
        x[c] += rng.uniform(-0.2, 0.2, size=3)
    x += 0.1 * rng.normal(size=x.shape)
    return x0, x, f


@pytest.mark.parametrize("kind", ["sphere", "cloth"])
def test_single_step_adjoint_fd(kind):
    from rxmesh_gb300 import RXMeshStatic, mcf_step, mcf_step_backward
    if kind == "sphere":
        x, f = sphere()
    else:
        _, x, f = cloth()
    rx = RXMeshStatic(f, len(x), patch_size=64)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    dt = 1e-2
    rng = np.random.default_rng(0)
    w = torch.tensor(rng.normal(size=x.shape), device="cuda")  # l = <w, x1>

    def fwd(xin):
        y = xin.clone()
        mcf_step(rx, y, dt, 1, "f64", tol=1e-13, max_iter=20000)
        return y

    x1 = fwd(xl)
    g = mcf_step_backward(rx, xl, x1, w, dt, tol=1e-13)
    h = 1e-6
    for _ in range(16):
        d = torch.tensor(rng.normal(size=x.shape), device="cuda")
        fd = ((w * fwd(xl + h * d)).sum() - (w * fwd(xl - h * d)).sum()).item() / (2 * h)
        an = (g * d).sum().item()
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3 * g.abs().sum().item()), (fd, an)


def test_unrolled_flow_with_arap_loss_fd():
    # ARAP energy after 20 implicit MCF steps, d/dx0 through autograd with
    # checkpoints every 5 steps, against central differences
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic, arap_energy, mcf_flow
    x0r, x, f = cloth(10)
    rx = RXMeshStatic(f, len(x), patch_size=64)
    rest = rx.to_linear(torch.tensor(x0r, device="cuda"))
    prob = DiffScalarProblem(rx, torch.float64, assemble_hessian=False).add_arap_term(rest)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    dt, n = 1e-3, 20

    def loss(x0):
        return arap_energy(mcf_flow(x0, rx, dt, n, 5), prob)

    x0 = xl.clone().requires_grad_(True)
    L0 = loss(x0)
    (g,) = torch.autograd.grad(L0, x0)
    rng = np.random.default_rng(4)
    h = 1e-6
    for _ in range(16):
        d = torch.tensor(rng.normal(size=x.shape), device="cuda")
        with torch.no_grad():
            fd = (loss(xl + h * d) - loss(xl - h * d)).item() / (2 * h)
        an = (g * d).sum().item()
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-6), (fd, an)


def test_checkpoint_interval_does_not_change_gradient():
    from rxmesh_gb300 import RXMeshStatic, mcf_flow
    x, f = sphere(2)
    rx = RXMeshStatic(f, len(x), patch_size=64)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    w = torch.randn(xl.shape, dtype=torch.float64, device="cuda")
    grads = []
    for k in (1, 3, 7):
        x0 = xl.clone().requires_grad_(True)
        (g,) = torch.autograd.grad((w * mcf_flow(x0, rx, 1e-3, 7, k)).sum(), x0)
        grads.append(g)
    for g in grads[1:]:
        assert (g - grads[0]).abs().max().item() <= 1e-12 * grads[0].abs().max().item()
