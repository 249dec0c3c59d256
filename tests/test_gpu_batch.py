"""Batched MCF: every mesh of a mixed batch matches its own FP64 oracle."""
import numpy as np
import pytest
import torch

from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu


def batch_meshes(seed=0, count=10):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        if i % 2 == 0:
            v, f = meshgen.icosphere(int(rng.integers(1, 4)))
            x = meshgen.radial_noise(v, 0.02, seed + i)
        else:
            n = int(rng.integers(6, 24))
            x, f = meshgen.plane(n, n, 1.0)
            x = x + rng.normal(0, 0.02, x.shape)
        out.append((x, f))
    return out


def oracle_step(oracle, x, f, dt, steps):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    for _ in range(steps):
        rp, col, val, B = oracle.mcf_system(f, x, dt)
        x = spl.spsolve(sp.csr_matrix((val, col, rp), shape=(len(x), len(x))).tocsc(), B)
    return x


@pytest.mark.parametrize("steps", [1, 3])
def test_batch_matches_oracle(oracle, steps):
    from rxmesh_gb300 import MeshBatch
    meshes = batch_meshes()
    b = MeshBatch([(f, len(x)) for x, f in meshes], patch_size=64)
    X = torch.tensor(np.concatenate([x for x, _ in meshes]), device="cuda")
    b.mcf(X, 1e-3, steps, tol=1e-9)
    it, cv = b.stats()
    assert cv.all() and (it > 0).all()
    got = X.cpu().numpy()
    for m, (x, f) in enumerate(meshes):
        want = oracle_step(oracle, x, f, 1e-3, steps)
        g = got[b.voff[m]:b.voff[m + 1]]
        assert np.linalg.norm(g - want) / np.linalg.norm(want) < 1e-6, m


def test_batch_autotune_and_repeat():
    from rxmesh_gb300 import MeshBatch
    meshes = batch_meshes(3, 6)
    b = MeshBatch([(f, len(x)) for x, f in meshes], patch_size=64)
    X0 = torch.tensor(np.concatenate([x for x, _ in meshes]), device="cuda")
    t, bps, ms = b.autotune(X0, 1e-3, 2)
    assert t in (256, 512, 1024) and bps >= 1 and ms > 0
    X1, X2 = X0.clone(), X0.clone()
    b.mcf(X1, 1e-3, 2)
    b.mcf(X2, 1e-3, 2)
    assert torch.equal(X1, X2)  # deterministic across launches


def test_batch_gangs_match_oracle(oracle):
    """Meshes larger than one CTA's tile run on gangs of CTAs (k > 1)."""
    from rxmesh_gb300 import MeshBatch
    rng = np.random.default_rng(11)
    meshes = []
    x, f = meshgen.plane(120, 120, 1.0)  # 14,400 vertices: a gang of 4 at the default tile
    meshes.append((x + rng.normal(0, 0.02, x.shape), f))
    v, f = meshgen.icosphere(5)  # 10,242 vertices: a gang of 3
    meshes.append((meshgen.radial_noise(v, 0.02, 5), f))
    v, f = meshgen.icosphere(2)
    meshes.append((meshgen.radial_noise(v, 0.02, 6), f))
    b = MeshBatch([(f, len(x)) for x, f in meshes], patch_size=256)
    X = torch.tensor(np.concatenate([x for x, _ in meshes]), device="cuda")
    X0 = X.clone()
    b.mcf(X, 1e-3, 2, tol=1e-9)
    it, cv = b.stats()
    assert cv.all() and (it > 0).all()
    got = X.cpu().numpy()
    for m, (x, f) in enumerate(meshes):
        want = oracle_step(oracle, x, f, 1e-3, 2)
        g = got[b.voff[m]:b.voff[m + 1]]
        assert np.linalg.norm(g - want) / np.linalg.norm(want) < 1e-6, m
    X2 = X0.clone()
    b.mcf(X2, 1e-3, 2, tol=1e-9)
    assert torch.equal(X, X2)  # gang sums are deterministic
