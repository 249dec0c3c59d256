"""Regenerate the golden fixtures in this folder.

Reads fixture meshes from the RXMesh tree (input/*.obj) and runs the
reference's own serial vertex-normal routine (apps/VertexNormal/
vertex_normal_ref.h, compiled into oracle/_ref by oracle/Makefile) on them.
Writes <name>.npz with fv (int32), xyz (float64), and the reference normals
in FP32 and FP64; where the tree holds a saved partition of the mesh
(input/<name>_patches, written by RXMesh's Patcher::save), its raw bytes as
patcher_file (uint8).  Run here, where the reference tree exists:

    python tests/golden/make_golden.py [/path/to/RXMesh [name ...]]

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


def main(ref_root, names=None):
    O.build()
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref was not built (reference tree missing?)")
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
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference", sys.argv[2:])
