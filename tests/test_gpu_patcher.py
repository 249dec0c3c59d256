"""The GPU patcher (RXG_MESH_GPU_PATCHER; RXMesh's Lloyd patcher,
include/rxmesh/patcher/patcher.cu:828-960): the partition equals the numpy
restatement in oracle/patcher.py face for face, every patch holds at most
patch_size faces and is connected, and two runs agree.  Query parity on
GPU-partitioned meshes runs in test_gpu_queries.py."""
import numpy as np
import pytest

from conftest import edge_case_meshes, golden
from rxmesh_gb300 import meshgen

pytestmark = pytest.mark.gpu

MESHES = {
    "torus64": lambda: meshgen.torus(64, 48, jitter=1e-3, seed=1),
    "icosphere4": lambda: meshgen.icosphere(4),
    "plane": lambda: meshgen.plane(40, 23),
    "sphere3": lambda: (golden("sphere3")["xyz"], golden("sphere3")["fv"]),
    "isolated": lambda: edge_case_meshes()["isolated"],
    "nonmanifold": lambda: edge_case_meshes()["nonmanifold"],
    "components": lambda: edge_case_meshes()["components"],
}


def connected_regions(fv, fp):
    from oracle.patcher import face_graph
    off, val, _ = face_graph(fv)
    for p in np.unique(fp):
        faces = np.nonzero(fp == p)[0]
        seen = {int(faces[0])}
        stack = [int(faces[0])]
        while stack:
            f = stack.pop()
            for g in val[off[f]:off[f + 1]]:
                if fp[g] == p and int(g) not in seen:
                    seen.add(int(g))
                    stack.append(int(g))
        if len(seen) != len(faces):
            return False
    return True


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("P", [64, 512])
def test_gpu_patcher_matches_restatement(name, P):
    from oracle.patcher import lloyd_partition
    from rxmesh_gb300 import RXMeshStatic, device_check
    x, f = MESHES[name]()
    rx = RXMeshStatic(f, len(x), patch_size=P, gpu_patcher=True)
    fp, vp, ep = rx.partition()
    want, _ = lloyd_partition(f, P)
    assert np.array_equal(fp, want)
    assert np.bincount(fp).max() <= P
    assert connected_regions(f, fp)
    again = RXMeshStatic(f, len(x), patch_size=P, gpu_patcher=True)
    assert all(np.array_equal(a, b) for a, b in zip(rx.patches(), again.patches()))
    device_check()
