"""Vertex normals on the edge cases of the patch layout: small, default and
largest patches (64, 512, 4096 faces), both weightings, and positions that
start one float into a larger buffer (not 16-byte aligned).  Each owned
vertex sums its incident faces in a fixed order, so a rerun, and the run on
the unaligned copy, give bit-identical normals.  The reference's check for
normals is an absolute 1e-4 (apps/VertexNormal/vertex_normal.cu:90-108);
this one is 1e-6 relative per vertex against the oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def meshes():
    from rxmesh_gb300 import meshgen
    v, f = meshgen.icosphere(5)
    return {"torus": meshgen.torus(96, 64, jitter=1e-3, seed=4),
            "sphere": (meshgen.radial_noise(v, 0.02, 5), f)}


@pytest.mark.parametrize("name", ["torus", "sphere"])
@pytest.mark.parametrize("patch_size", [64, 512, 4096])
def test_normals_patch_sizes_and_alignment(oracle, name, patch_size):
    from rxmesh_gb300 import RXMeshStatic
    x, f = meshes()[name]
    x32 = np.asarray(x, np.float32)
    rx = RXMeshStatic(f, len(x32), patch_size=patch_size)
    xl = rx.to_linear(torch.tensor(x32, device="cuda"))
    buf = torch.zeros(xl.numel() + 1, dtype=torch.float32, device="cuda")
    buf[1:] = xl.reshape(-1)
    xu = buf[1:].view(-1, 3)
    for w, code in (("max", 0), ("area", 1)):
        n = rx.vertex_normals(xl, w)
        again = rx.vertex_normals(xl, w)
        nu = rx.vertex_normals(xu, w)
        assert torch.equal(n, again) and torch.equal(n, nu), w
        got = rx.to_input(n).cpu().numpy()
        ref = oracle.vertex_normals(np.asarray(f), x32.astype(np.float64), code).reshape(-1, 3)
        err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert err.max() < 1e-6, (w, err.max())
