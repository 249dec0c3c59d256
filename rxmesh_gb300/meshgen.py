"""Seeded synthetic meshes for the hot-path workloads, and a minimal OBJ reader.

- icosphere(level): recursive midpoint subdivision of the icosahedron,
  projected to the unit sphere (V = 10*4^l + 2, F = 20*4^l).
- torus(nu, nv): periodic (u, v) grid, two triangles per quad.
- plane(nx, ny): the triangulation of RXMesh's create_plane
  (include/rxmesh/geometry_factory.h:12-75): quad (a,b,c,d) -> (a,b,c),(c,b,d).
"""
import numpy as np


def icosphere(level):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.sort(e, axis=1)
        uniq, inv = np.unique(key[:, 0] * (len(v) + 1) + key[:, 1], return_inverse=True)
        a = uniq // (len(v) + 1)
        b = uniq % (len(v) + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + len(v)  # midpoints of (01, 12, 20)
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m[:, 0], m[:, 2]], 1),
            np.stack([f[:, 1], m[:, 1], m[:, 0]], 1),
            np.stack([f[:, 2], m[:, 2], m[:, 1]], 1),
            np.stack([m[:, 0], m[:, 1], m[:, 2]], 1)])
    return v, f.astype(np.int32)


def radial_noise(v, sigma, seed):
    """x <- x * (1 + N(0, sigma)) per vertex (radial displacement)."""
    rng = np.random.default_rng(seed)
    return v * (1.0 + rng.normal(0.0, sigma, size=(len(v), 1)))


def torus(nu, nv, R=1.0, r=0.3, jitter=0.0, seed=0, dtype=np.float32):
    """Closed torus on a periodic nu x nv grid; vertex (i, j) has id i*nv + j."""
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    u = 2 * np.pi * i.ravel() / nu
    w = 2 * np.pi * j.ravel() / nv
    x = np.stack([(R + r * np.cos(w)) * np.cos(u), (R + r * np.cos(w)) * np.sin(u), r * np.sin(w)], 1)
    if jitter > 0:
        x = x + np.random.default_rng(seed).normal(0.0, jitter, size=x.shape)
    a = (i * nv + j).ravel()
    b = (((i + 1) % nu) * nv + j).ravel()
    c = (i * nv + (j + 1) % nv).ravel()
    d = (((i + 1) % nu) * nv + (j + 1) % nv).ravel()
    f = np.empty((2 * nu * nv, 3), np.int32)
    f[0::2] = np.stack([a, b, d], 1)
    f[1::2] = np.stack([a, d, c], 1)
    return x.astype(dtype), f


def plane(nx, ny, dx=1.0, axis=2, dtype=np.float64):
    """create_plane (geometry_factory.h:12-75): row i, column j -> id i*nx + j."""
    ii, jj = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    x = np.zeros((nx * ny, 3), dtype)
    cols = {0: (1, 2), 1: (0, 2), 2: (0, 1)}[axis]
    x[:, cols[0]] = dx * jj.ravel()
    x[:, cols[1]] = dx * ii.ravel()
    i, j = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    idx = (i * nx + j).ravel()
    a, b, c, d = idx, idx + nx, idx + 1, idx + nx + 1
    f = np.empty((2 * len(idx), 3), np.int32)
    f[0::2] = np.stack([a, b, c], 1)
    f[1::2] = np.stack([c, b, d], 1)
    return x, f


def read_obj(path):
    """Vertices and triangles of an OBJ file (faces fan-triangulated; an
    index is 1-based, or negative: relative to the vertices read so far)."""
    vs, fs = [], []
    with open(path) as fh:
        for line in fh:
            if line.startswith(("v ", "v\t")):
                vs.append([float(t) for t in line.split()[1:4]])
            elif line.startswith(("f ", "f\t")):
                ids = []
                for t in line.split("#")[0].split()[1:]:
                    i = int(t.split("/")[0])
                    ids.append(i - 1 if i > 0 else len(vs) + i)
                for k in range(1, len(ids) - 1):
                    fs.append([ids[0], ids[k], ids[k + 1]])
    return np.array(vs, np.float64), np.array(fs, np.int32).reshape(-1, 3)
