"""Regenerate the golden fixtures in this folder.

Reads fixture meshes from the RXMesh tree (input/*.obj) and runs the
reference's own serial vertex-normal routine (apps/VertexNormal/
vertex_normal_ref.h, compiled into oracle/_ref by oracle/Makefile) on them.
Writes <name>.npz with fv (int32), xyz (float64), and the reference normals
in FP32 and FP64; where the tree holds a saved partition of the mesh
(input/<name>_patches, written by RXMesh's Patcher::save), its raw bytes as
patcher_file (uint8).  Also writes geometry_util.npz: seeded triangles of
every branch of the reference's cotangent and Voronoi-area routines
(include/rxmesh/geometry_util.cuh:107-206, compiled into oracle/_ref from
the tree) with the reference's FP64 and FP32 outputs.  Run where the
reference tree exists:

    python tests/golden/make_golden.py /path/to/RXMesh [name ...]

plane_5 is the fixture of the reference's EVDiamond test
(tests/RXMesh_test/test_ev_diamond.cu).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import oracle as O  # noqa: E402
from rxmesh_gb300.meshgen import read_obj  # noqa: E402

MESHES = ["sphere3", "torus", "cloth", "bunnyhead", "plane_5"]


def geometry_cases(seed=0, n=4000):
    """Triangles (p, q, r) and diamonds (p, r, q, s) covering every branch of
    partial_voronoi_area and edge_cotan_weight: generic, obtuse at p, obtuse
    at q or r, within 1e-9 .. 1e-3 rad of a right angle, cotangents beyond
    the +-19.1 clamp (angles under 3 degrees), near-degenerate slivers and
    exactly collinear (zero-area) triangles."""
    rng = np.random.default_rng(seed)
    P = rng.normal(size=(n, 3))
    Q = P + rng.normal(size=(n, 3))
    R = P + rng.normal(size=(n, 3))
    k = n // 8
    # right angle at p, q or r, perturbed by 1e-9 .. 1e-3 (in the plane)
    for j, (a, b, c) in enumerate(((P, Q, R), (Q, R, P), (R, P, Q))):
        sl = slice((1 + j) * k, (2 + j) * k)
        u = rng.normal(size=(k, 3))
        v = np.cross(u, rng.normal(size=(k, 3)))
        eps = 10.0 ** rng.uniform(-9, -3, size=(k, 1)) * rng.choice([-1, 1], size=(k, 1))
        b[sl] = a[sl] + u
        c[sl] = a[sl] + v + eps * np.linalg.norm(v, axis=1, keepdims=True) * u / np.linalg.norm(u, axis=1, keepdims=True)
    # slivers: r close to the line p-q (tiny angles, clamped cotangents)
    sl = slice(4 * k, 5 * k)
    t = rng.uniform(-0.5, 1.5, size=(k, 1))
    R[sl] = P[sl] + t * (Q[sl] - P[sl]) + 10.0 ** rng.uniform(-8, -1, size=(k, 1)) * rng.normal(size=(k, 3))
    # exactly collinear (zero area) and repeated points
    sl = slice(5 * k, 5 * k + k // 2)
    R[sl] = P[sl] + 2.0 * (Q[sl] - P[sl])
    sl = slice(5 * k + k // 2, 6 * k)
    R[sl] = Q[sl]
    S = P + rng.normal(size=(n, 3))
    return P, Q, R, S


def make_geometry(out_dir=HERE):
    G = O.ref_geometry()
    if G is None:
        raise SystemExit("oracle/_ref/libref_geometry.so was not built")
    P, Q, R, S = geometry_cases()
    n = len(P)
    res = {}
    for t, dt in (("f64", np.float64), ("f32", np.float32)):
        a = [np.ascontiguousarray(x, dt) for x in (P, Q, R, S)]
        vor = np.empty(n, dt)
        cot = np.empty(n, dt)
        getattr(G, "ref_partial_voronoi_area_" + t)(n, a[0], a[1], a[2], vor)
        # edge p-q with opposite vertices r and s
        getattr(G, "ref_edge_cotan_weight_" + t)(n, a[0], a[1], a[2], a[3], cot)
        res["voronoi_" + t] = vor
        res["cotan_" + t] = cot
    path = os.path.join(out_dir, "geometry_util.npz")
    np.savez_compressed(path, P=P, Q=Q, R=R, S=S, **res)
    print("geometry_util", n, os.path.getsize(path))


def main(ref_root, names=None):
    O.build(ref_root)
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref was not built (reference tree missing?)")
    make_geometry()
    if names == ["geometry"]:
        return
    for name in names or MESHES:
        xyz, fv = read_obj(os.path.join(ref_root, "input", name + ".obj"))
        n32 = O.ref_vertex_normals(fv, xyz.astype(np.float32), np.float32)
        n64 = O.ref_vertex_normals(fv, xyz, np.float64)
        out = os.path.join(HERE, name + ".npz")
        extra = {}
        patches = os.path.join(ref_root, "input", name + "_patches")
        if os.path.exists(patches):
            with open(patches, "rb") as fh:
                extra["patcher_file"] = np.frombuffer(fh.read(), np.uint8)
        np.savez_compressed(out, fv=fv, xyz=xyz, ref_normals_f32=n32, ref_normals_f64=n64, **extra)
        print(name, xyz.shape, fv.shape, os.path.getsize(out))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <RXMesh source tree> [mesh names...]")
    main(sys.argv[1], sys.argv[2:])
