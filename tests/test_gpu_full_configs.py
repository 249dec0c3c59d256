"""Parity at the full sizes of the benchmarked workloads.

The other GPU tests compare against the oracle on small meshes; these run
the same comparisons on the meshes the benchmark measures:
  - torus 1024 x 1024 (1,048,576 vertices, 2,097,152 faces, patches of at
    most 512 faces): VV, VE, VF bit-exact as sorted sets, FV and EV
    bit-exact in order, both normal weightings within 1e-6 of the
    magnitude of each vertex's summed face contributions;
  - icosphere level 8 (655,362 vertices), 10 implicit MCF steps at dt 1e-3
    in FP64 and in mixed precision, against the FP64 oracle's 10 steps;
  - cloth 512 x 512 (262,144 vertices, 522,242 faces): per-face ARAP energy,
    gradient and 3x3-block Hessian against the oracle, and the adjoint of 20
    implicit MCF steps against 16 central differences;
  - the 256-mesh batch (icospheres of levels 2-6, grids 16-256), 5 mixed
    steps, every mesh against the FP64 oracle.
Set comparisons are vectorised: each CSR is flattened to (row, value) pairs
in input ids and sorted with np.lexsort, which is the set form of
tests/RXMesh_test/rxmesh_test.h:347-440 without a per-row Python loop.
"""
import numpy as np
import pytest
import torch

from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu


def pairs(off, val, row_ids=None, val_ids=None):
    """CSR -> (rows, values) sorted lexicographically, optionally renumbered."""
    off = np.asarray(off, np.int64)
    val = np.asarray(val, np.int64)
    n = off.size - 1
    rows = np.repeat(np.arange(n) if row_ids is None else np.asarray(row_ids, np.int64), np.diff(off))
    vals = val if val_ids is None else np.asarray(val_ids, np.int64)[val]
    o = np.lexsort((vals, rows))
    return rows[o], vals[o]


@pytest.fixture(scope="module")
def torus1024():
    from rxmesh_gb300 import RXMeshStatic
    x, f = meshgen.torus(1024, 1024, jitter=1e-3, seed=0)
    rx = RXMeshStatic(f, len(x), patch_size=512)
    return x, f, rx


def test_torus1024_vertex_queries_bit_exact(oracle, torus1024):
    from rxmesh_gb300 import Op, device_check
    x, f, rx = torus1024
    nv = len(x)
    assert rx.get_num_patches() > 4000  # thousands of patches and their ribbons
    vl, el, fl = rx.linear_to_input("v"), rx.linear_to_input("e"), rx.linear_to_input("f")
    ev, _ = oracle.edges(f)
    for op, ref, tgt in ((Op.VV, oracle.vv(nv, ev), vl),
                         (Op.VE, oracle.vv(nv, ev, want_edges=True), el),
                         (Op.VF, oracle.vf(nv, f), fl)):
        off, val = rx.query(op)
        off, val = off.cpu().numpy(), val.cpu().numpy()
        gr, gv = pairs(off, val, vl, tgt)
        wr, wv = pairs(*ref)
        assert np.array_equal(gr, wr) and np.array_equal(gv, wv), op
    _, fvq = rx.query(Op.FV)
    _, evq = rx.query(Op.EV)
    fvq = fvq.cpu().numpy().reshape(-1, 3)
    evq = evq.cpu().numpy().reshape(-1, 2)
    assert np.array_equal(vl[fvq][np.argsort(fl)], np.asarray(f))
    assert np.array_equal(vl[evq][np.argsort(el)], ev)
    device_check()


def normal_contribution_norms(f, x, weighting):
    """Per vertex, the sum over its faces of |contribution| (the face's
    unnormalised normal, divided by the two adjacent squared edge lengths for
    the max weights): the scale of the rounding error of a floating-point sum
    of those contributions."""
    f = np.asarray(f)
    p = [x[f[:, k]] for k in range(3)]
    nn = np.linalg.norm(np.cross(p[1] - p[0], p[2] - p[0]), axis=1)
    l = [np.sum((p[i] - p[(i + 1) % 3]) ** 2, axis=1) for i in range(3)]
    S = np.zeros(len(x))
    for i in range(3):
        np.add.at(S, f[:, i], nn / (l[i] + l[(i + 2) % 3]) if weighting == "max" else nn)
    return S


@pytest.mark.parametrize("weighting", ["max", "area"])
def test_torus1024_normals(oracle, torus1024, weighting):
    """FP32 normals against the FP64 oracle on the same FP32 positions.  The
    N(0, 1e-3) jitter folds the surface at a few vertices, where the face
    contributions nearly cancel (the worst sum's condition number
    sum|c_f| / |sum c_f| is 275), so the error is bounded relative to the
    contributions' magnitude, the forward error bound of a floating-point
    sum: |n - n_ref| <= 1e-6 sum_f |c_f|.  Relative to each vertex's own
    normal, 99.99% of the vertices are within 1e-6 and the median is ~5e-8
    (an FP32 emulation of the same sums in numpy gives the same figures)."""
    x, f, rx = torus1024
    x32 = x.astype(np.float32)
    n = rx.to_input(rx.vertex_normals(rx.to_linear(torch.tensor(x32, device="cuda")), weighting))
    n = n.cpu().numpy()
    x64 = x32.astype(np.float64)
    ref = oracle.vertex_normals(f, x64, 0 if weighting == "max" else 1)
    S = normal_contribution_norms(f, x64, weighting)
    absr = np.linalg.norm(n - ref, axis=1)
    assert (absr <= 1e-6 * S).all(), (absr / S).max()
    rel = absr / np.linalg.norm(ref, axis=1)
    assert (rel <= 1e-6).mean() >= 0.9999, (rel <= 1e-6).mean()
    assert np.median(rel) <= 1e-7, np.median(rel)


def test_torus1024_fused_sweep_equals_queries(torus1024):
    """rxg_query_sweep on the full torus: VV, VE, VF offsets equal and rows
    the same sets as the separate queries; FV, EV and area normals equal."""
    from rxmesh_gb300 import Op
    x, f, rx = torus1024
    xl = rx.to_linear(torch.tensor(np.asarray(x, np.float32), device="cuda"))
    got = rx.query_sweep(xyz=xl, weighting="area")
    for name in ("VV", "VE", "VF"):
        off, val = rx.query(getattr(Op, name))
        go, gv = got[name]
        assert torch.equal(go, off), name
        a = pairs(go.cpu().numpy(), gv.cpu().numpy())
        b = pairs(off.cpu().numpy(), val.cpu().numpy())
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), name
    assert torch.equal(got["FV"], rx.query(Op.FV)[1])
    assert torch.equal(got["EV"], rx.query(Op.EV)[1])
    assert torch.equal(got["normals"], rx.vertex_normals(xl, "area"))


def test_torus1024_host_sweep_equals_queries(torus1024):
    """rxg_query_sweep_ex into page-locked host memory on the full torus:
    the separate queries' offsets and rows (as sets), FV, EV and normals
    bit for bit."""
    from rxmesh_gb300 import Op
    x, f, rx = torus1024
    xl = rx.to_linear(torch.tensor(np.asarray(x, np.float32), device="cuda"))
    s = torch.cuda.Stream()
    got = rx.query_sweep(xyz=xl.cpu().pin_memory(), weighting="area", stream=s, host=True)
    s.synchronize()
    for name in ("VV", "VE", "VF"):
        off, val = rx.query(getattr(Op, name))
        go, gv = got[name]
        assert torch.equal(go, off.cpu()), name
        a, b = pairs(go.numpy(), gv.numpy()), pairs(off.cpu().numpy(), val.cpu().numpy())
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), name
    assert torch.equal(got["FV"], rx.query(Op.FV)[1].cpu())
    assert torch.equal(got["EV"], rx.query(Op.EV)[1].cpu())
    assert torch.equal(got["normals"], rx.vertex_normals(xl, "area").cpu())


def test_torus1024_edge_face_queries_bit_exact(oracle, torus1024):
    """EF, FF as sets; FE, EVDiamond and EE in order, on the full torus."""
    from rxmesh_gb300 import Op
    x, f, rx = torus1024
    vl, el, fl = rx.linear_to_input("v"), rx.linear_to_input("e"), rx.linear_to_input("f")
    for op, ref, rows, tgt in ((Op.EF, oracle.ef(f), el, fl), (Op.FF, oracle.ff(f), fl, fl)):
        off, val = rx.query(op)
        gr, gv = pairs(off.cpu().numpy(), val.cpu().numpy(), rows, tgt)
        wr, wv = pairs(*ref)
        assert np.array_equal(gr, wr) and np.array_equal(gv, wv), op
    _, fe = oracle.edges(f)
    _, feq = rx.query(Op.FE)
    assert np.array_equal(el[feq.cpu().numpy().reshape(-1, 3)][np.argsort(fl)], fe)
    _, dq = rx.query(Op.EVD)
    dq = dq.cpu().numpy().reshape(-1, 4)
    din = np.where(dq >= 0, vl[np.maximum(dq, 0)], -1)[np.argsort(el)]
    assert np.array_equal(din, oracle.ev_diamond(f))
    _, eq = rx.query(Op.EE)
    eq = eq.cpu().numpy().reshape(-1, 4)
    assert np.array_equal(np.where(eq >= 0, el[np.maximum(eq, 0)], -1)[np.argsort(el)], oracle.ee(f))


# --------------------------------------------------------------------------
# icosphere level 8, 10 implicit MCF steps at dt = 1e-3
# --------------------------------------------------------------------------

# Per-step solver tolerance of the benchmarked runs (relative, Jacobi-weighted
# residual), and the bar on the positions after all 10 steps: relative
# 2-norm error against the FP64 oracle solved to 1e-12 every step.
MCF_TOL = 1e-6
MCF_BAR = 1e-6


@pytest.fixture(scope="module")
def level8_oracle(oracle):
    v, f = meshgen.icosphere(8)
    x0 = meshgen.radial_noise(v, 0.02, 0)
    xs = [x0]
    x = x0
    for _ in range(10):
        rp, col, val, B = oracle.mcf_system(f, x, 1e-3)
        x = oracle.cg(rp, col, val, B, x, 20000, 0.0, 1e-24, True)[0]
        xs.append(x)
    return f, xs


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_level8_ten_mcf_steps(level8_oracle, precision):
    from rxmesh_gb300 import RXMeshStatic, mcf_step
    f, xs = level8_oracle
    rx = RXMeshStatic(f, len(xs[0]), patch_size=256)
    x = rx.to_linear(torch.tensor(xs[0], device="cuda"))
    errs = []
    for k in range(1, 11):
        st = mcf_step(rx, x, 1e-3, 1, precision, tol=MCF_TOL)
        assert st["converged"], (k, st)
        got = rx.to_input(x).cpu().numpy()
        errs.append(float(np.linalg.norm(got - xs[k]) / np.linalg.norm(xs[k])))
    assert max(errs) <= MCF_BAR, errs


# --------------------------------------------------------------------------
# cloth 512 x 512: per-face ARAP and the adjoint of 20 MCF steps
# --------------------------------------------------------------------------

def cloth512(jitter=0.0, seed=0):
    """create_plane grid 512 x 512 (dx = 1), flat rest shape, the 4 corners
    displaced by U(-0.2, 0.2), fp32 positions (the benchmark's cloth)."""
    n = 512
    x0, f = meshgen.plane(n, n, 1.0)
    rng = np.random.default_rng(seed)
    x = x0.copy()
    for c in [0, n - 1, n * (n - 1), n * n - 1]:
        x[c] += rng.uniform(-0.2, 0.2, size=3)
    if jitter:
        x += jitter * rng.normal(size=x.shape)
    return x0, x.astype(np.float32).astype(np.float64), f


# FP32: 5e-4 of the largest entry.  The cloth's coordinates reach 511 with
# unit edges, and the displaced corners' faces are strongly deformed; FP32
# arithmetic there leaves ~3e-4 of the largest gradient entry (1e-4 or less
# on the small cloths of test_gpu_arap.py).
@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-11), (torch.float32, 5e-4)])
def test_cloth512_arap_matches_oracle(oracle, dtype, rtol):
    from test_gpu_arap import oracle_ref
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic
    x0, x, f = cloth512()
    # a generic interior state as well as the corner handles, so that every
    # face has a non-trivial rotation and Hessian; rounded to FP32 so that the
    # oracle and the FP32 evaluation see the same positions
    x = (x + 0.01 * np.random.default_rng(1).normal(size=x.shape)).astype(np.float32).astype(np.float64)
    rx = RXMeshStatic(f, len(x0), patch_size=512)
    x0l = rx.to_linear(torch.tensor(x0, device="cuda"))
    xl = rx.to_linear(torch.tensor(x, device="cuda")).to(dtype)
    prob = DiffScalarProblem(rx, dtype).add_arap_term(x0l)
    prob.eval_terms(xl)
    E, fE, g, H, _ = oracle_ref(oracle, f, x0, x, rx, prob)
    fl = rx.linear_to_input("f")
    assert abs(prob.get_current_loss() - E) <= rtol * abs(E)
    assert np.abs(prob.face_energy.double().cpu().numpy() - fE[fl]).max() <= rtol * np.abs(fE).max()
    gg = rx.to_input(prob.grad).double().cpu().numpy()
    assert np.abs(gg - g).max() <= rtol * np.abs(g).max()
    Hg = prob.hess.val.double().cpu().numpy()
    assert np.abs(Hg - H).max() <= rtol * np.abs(H).max()


def triangle_angles(x, f):
    """All corner angles (radians) of the faces f at positions x."""
    f = np.asarray(f)
    out = []
    for k in range(3):
        a, b, c = x[f[:, k]], x[f[:, (k + 1) % 3]], x[f[:, (k + 2) % 3]]
        u, v = b - a, c - a
        cos = np.sum(u * v, axis=1) / (np.linalg.norm(u, axis=1) * np.linalg.norm(v, axis=1))
        out.append(np.arccos(np.clip(cos, -1.0, 1.0)))
    return np.concatenate(out)


def test_cloth512_adjoint_20_steps_fd():
    """ARAP energy after 20 implicit MCF steps (checkpoints every 5) on the
    full 512 x 512 cloth, d/dx0 through autograd, against FP64 central
    differences (h = 1e-6) on 16 random directions over all vertices.

    The reference's Voronoi area (geometry_util.cuh:117-167) jumps when a
    triangle angle crosses 90 degrees, so the flow has no derivative there and
    a difference quotient across a jump is meaningless.  A create_plane grid
    has every quad corner at exactly 90 degrees, and a jittered one has
    ~1.5 M angles spread around 90: somewhere on the full mesh a perturbation
    of 1e-6 then crosses the jump.  The grid is therefore sheared by 0.3 of y
    (quad corners at 73 and 107 degrees) before the corner handles and a
    N(0, 0.01) jitter are applied, and the test first checks that every
    angle stays at least 0.05 rad from 90 degrees."""
    from rxmesh_gb300 import DiffScalarProblem, RXMeshStatic, arap_energy, mcf_flow
    x0r, x, f = cloth512()
    x = x.copy()
    x[:, 0] += 0.3 * x[:, 1]
    x += 0.01 * np.random.default_rng(3).normal(size=x.shape)
    assert np.abs(triangle_angles(x, f) - np.pi / 2).min() > 0.05
    rx = RXMeshStatic(f, len(x), patch_size=512)
    rest = rx.to_linear(torch.tensor(x0r, device="cuda"))
    prob = DiffScalarProblem(rx, torch.float64, assemble_hessian=False).add_arap_term(rest)
    xl = rx.to_linear(torch.tensor(x, device="cuda"))
    # Every solve runs a fixed 80 Jacobi-PCG iterations (far past convergence
    # at dt = 1e-3; a tolerance of 1e-30 is never met), so the flow is the same
    # smooth map for every perturbed start: with a tolerance, the two runs of
    # a central difference could stop at different iteration counts and
    # differ by the solver's residual.
    tol, iters = 1e-30, 80

    def flow(x0):
        return mcf_flow(x0, rx, 1e-3, 20, 5, tol=tol, max_iter=iters)

    x0 = xl.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(arap_energy(flow(x0), prob), x0)

    def face_energies(x0):
        with torch.no_grad():
            prob.eval_terms(flow(x0), with_hessian=False)
        return prob.face_energy.clone()

    # A random direction's derivative g.d can come out far smaller than its
    # typical size |g|_2 (the terms cancel), while a difference quotient's
    # error does not shrink with it, so the bar is relative to
    # max(|g.d|, |g|_2).  Measured on this mesh, the central differences
    # converge as h^2 (1.4e-3, 1.4e-5, 1.4e-7 of g.d at h = 1e-2, 1e-3, 1e-4)
    # down to ~1e-7 at h = 1e-6.
    rng = np.random.default_rng(4)
    h = 1e-6
    gnorm = g.norm().item()
    for _ in range(16):
        d = torch.tensor(rng.normal(size=x.shape), device="cuda")
        # per-face differences first: the total (~5e3) summed over 522k faces
        # would lose the directional derivative's digits
        fd = (face_energies(xl + h * d) - face_energies(xl - h * d)).sum().item() / (2 * h)
        an = (g * d).sum().item()
        assert abs(fd - an) <= 1e-5 * max(abs(an), gnorm), (fd, an, gnorm)


# --------------------------------------------------------------------------
# the 256-mesh batch
# --------------------------------------------------------------------------

def test_batch256_matches_oracle(oracle):
    """The benchmark's batch (seed 7): 128 icospheres of levels 2-6 and 128
    create_plane grids of 16-256 vertices a side, N(0, 0.02) noise, 5 mixed
    steps at dt 1e-3 in one persistent launch; every mesh against 5 FP64
    oracle steps solved to 1e-12."""
    from rxmesh_gb300 import MeshBatch
    rng = np.random.default_rng(7)
    meshes = []
    for i in range(256):
        if i % 2 == 0:
            v, f = meshgen.icosphere(int(rng.integers(2, 7)))
            x = meshgen.radial_noise(v, 0.02, 1000 + i)
        else:
            n = int(rng.integers(16, 257))
            x, f = meshgen.plane(n, n, 1.0)
            x = x + rng.normal(0.0, 0.02, size=x.shape)
        meshes.append((x, f))
    b = MeshBatch([(f, len(x)) for x, f in meshes], patch_size=256)
    X = torch.tensor(np.concatenate([x for x, _ in meshes]), device="cuda")
    b.mcf(X, 1e-3, 5, tol=MCF_TOL)
    it, cv = b.stats()
    assert cv.all() and (it > 0).all()
    got = X.cpu().numpy()
    errs = []
    for m, (x, f) in enumerate(meshes):
        for _ in range(5):
            rp, col, val, B = oracle.mcf_system(f, x, 1e-3)
            x = oracle.cg(rp, col, val, B, x, 20000, 0.0, 1e-24, True)[0]
        g = got[b.voff[m]:b.voff[m + 1]]
        errs.append(np.linalg.norm(g - x) / np.linalg.norm(x))
    assert max(errs) <= MCF_BAR, (int(np.argmax(errs)), max(errs))
