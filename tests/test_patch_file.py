"""Reproducible partitions: meshes built on a given partition, and RXMesh's
saved-patcher files (RXMeshStatic(fv, patcher_file), Patcher::serialize,
include/rxmesh/patcher/patcher.h:162-181).

Pinned to the two partitions RXMesh ships with its inputs
(input/sphere3_patches, input/torus_patches, kept byte for byte in the golden
fixtures): the file's face, vertex and edge owners come back unchanged; with
the face partition alone, the vertex and edge owners follow RXMesh's
Patcher::assign_patch rule (patcher/patcher.cu:719-757) and equal the file's;
a saved file carries the same owners, patches and external ribbons
(patcher.cu:640-716).  Host-only meshes: no GPU needed."""
import struct

import numpy as np
import pytest

from conftest import golden
from rxmesh_gb300 import meshgen


def decode(buf):
    """The patcher file as RXMesh writes it (cereal portable binary archive):
    endianness byte, nine uint32, seven uint32 vectors (uint64 count first),
    one float."""
    assert buf[0] == 1
    names = ["patch_size", "num_patches", "num_vertices", "num_edges", "num_faces",
             "num_seeds", "max_num_patches", "num_components", "num_lloyd_run"]
    out = dict(zip(names, struct.unpack_from("<9I", buf, 1)))
    pos = 37
    for name in ["face_patch", "vertex_patch", "edge_patch", "patches_val", "patches_offset",
                 "ribbon_ext_val", "ribbon_ext_offset"]:
        n = struct.unpack_from("<Q", buf, pos)[0]
        pos += 8
        out[name] = np.frombuffer(buf, "<u4", n, pos).astype(np.int64)
        pos += 4 * n
    out["patching_time_ms"] = struct.unpack_from("<f", buf, pos)[0]
    assert pos + 4 == len(buf)
    return out


def per_patch(vals, offsets, np_):
    ends = offsets[:np_]
    starts = np.r_[0, ends[:-1]]
    return [vals[s:e] for s, e in zip(starts, ends)]


def write_fixture(name, tmp_path):
    g = golden(name)
    path = tmp_path / (name + "_patches")
    path.write_bytes(g["patcher_file"].tobytes())
    return g, path


@pytest.mark.parametrize("name", ["sphere3", "torus"])
def test_reference_patch_file_loads(name, tmp_path):
    from rxmesh_gb300 import RXMeshStatic
    g, path = write_fixture(name, tmp_path)
    ref = decode(g["patcher_file"].tobytes())
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), host_only=True, patcher_file=str(path))
    assert rx.get_num_patches() == ref["num_patches"]
    assert rx.get_num_edges() == ref["num_edges"]
    fp, vp, ep = rx.partition()
    assert np.array_equal(fp, ref["face_patch"])
    assert np.array_equal(vp, ref["vertex_patch"])
    assert np.array_equal(ep, ref["edge_patch"])
    # the edge numbering the owners index is RXMesh's: (fv[f][k], fv[f][k+1])
    # by first appearance in face order
    ev = rx.input_edges()
    seen = {}
    for f in g["fv"]:
        for k in range(3):
            a, b = int(f[k]), int(f[(k + 1) % 3])
            seen.setdefault((min(a, b), max(a, b)), len(seen))
    assert [seen[(min(a, b), max(a, b))] for a, b in ev] == list(range(len(ev)))


@pytest.mark.parametrize("name", ["sphere3", "torus"])
def test_owner_rule_matches_reference(name):
    """Face partition alone: vertex and edge owners by assign_patch's rule."""
    from rxmesh_gb300 import RXMeshStatic
    g = golden(name)
    ref = decode(g["patcher_file"].tobytes())
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), host_only=True, face_patch=ref["face_patch"])
    fp, vp, ep = rx.partition()
    assert np.array_equal(fp, ref["face_patch"])
    assert np.array_equal(vp, ref["vertex_patch"])
    assert np.array_equal(ep, ref["edge_patch"])


def reference_ribbon(fv, face_patch, patches_val, patches_offset, np_):
    """Patcher's external ribbon (patcher.cu:640-716) on a given face order."""
    nv = int(fv.max()) + 1
    vf = [[] for _ in range(nv)]
    for f, tri in enumerate(fv):
        for v in tri:
            vf[v].append(f)
    out = []
    for p, faces in enumerate(per_patch(patches_val, patches_offset, np_)):
        r = []
        for f in faces:
            for v in fv[f]:
                for n in vf[v]:
                    if face_patch[n] != p and n not in r:
                        r.append(n)
        out.append(r)
    return out


@pytest.mark.parametrize("name", ["sphere3", "torus"])
def test_save_round_trip(name, tmp_path):
    from rxmesh_gb300 import RXMeshStatic
    g, path = write_fixture(name, tmp_path)
    ref = decode(g["patcher_file"].tobytes())
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), host_only=True, patcher_file=str(path))
    out = tmp_path / "saved_patches"
    rx.save(str(out))
    got = decode(out.read_bytes())
    for k in ("num_patches", "num_vertices", "num_edges", "num_faces", "num_components",
              "patch_size"):
        assert got[k] == ref[k], k
    for k in ("face_patch", "vertex_patch", "edge_patch"):
        assert np.array_equal(got[k], ref[k]), k
    np_ = ref["num_patches"]
    for a, b in zip(per_patch(got["patches_val"], got["patches_offset"], np_),
                    per_patch(ref["patches_val"], ref["patches_offset"], np_)):
        assert sorted(a) == sorted(b)
    for a, b in zip(per_patch(got["ribbon_ext_val"], got["ribbon_ext_offset"], np_),
                    per_patch(ref["ribbon_ext_val"], ref["ribbon_ext_offset"], np_)):
        assert sorted(a) == sorted(b)
    # in the order the reference's rule gives on the saved face order
    want = reference_ribbon(g["fv"], got["face_patch"], got["patches_val"],
                            got["patches_offset"], np_)
    assert [list(r) for r in per_patch(got["ribbon_ext_val"], got["ribbon_ext_offset"], np_)] == want
    # and the saved file loads back to the same layout
    rx2 = RXMeshStatic(g["fv"], len(g["xyz"]), host_only=True, patcher_file=str(out))
    assert all(np.array_equal(a, b) for a, b in zip(rx.partition(), rx2.partition()))
    assert all(np.array_equal(a, b) for a, b in zip(rx.patches(), rx2.patches()))


def test_own_partition_round_trip(tmp_path):
    """The library's own partition given back (arrays, or a saved file)
    rebuilds the identical patch layout, isolated vertices included."""
    from rxmesh_gb300 import RXMeshStatic
    from conftest import edge_case_meshes
    for x, f in (meshgen.torus(40, 24, jitter=1e-3, seed=2), edge_case_meshes()["isolated"],
                 edge_case_meshes()["components"]):
        rx = RXMeshStatic(f, len(x), patch_size=64, host_only=True)
        fp, vp, ep = rx.partition()
        assert fp.max() + 1 <= rx.get_num_patches()
        rx2 = RXMeshStatic(f, len(x), host_only=True, face_patch=fp, vertex_patch=vp,
                           edge_patch=ep)
        assert all(np.array_equal(a, b) for a, b in zip(rx.patches(), rx2.patches()))
        for e in ("v", "e", "f"):
            assert np.array_equal(rx.linear_to_input(e), rx2.linear_to_input(e))
        path = tmp_path / "own_patches"
        rx.save(str(path))
        rx3 = RXMeshStatic(f, len(x), host_only=True, patcher_file=str(path))
        assert all(np.array_equal(a, b) for a, b in zip(rx.patches(), rx3.patches()))


def test_bad_partitions_and_files(tmp_path):
    from rxmesh_gb300 import RXGError, RXMeshStatic
    g, path = write_fixture("sphere3", tmp_path)
    fv, nv = g["fv"], len(g["xyz"])
    ref = decode(g["patcher_file"].tobytes())
    fp = ref["face_patch"].astype(np.int32)
    with pytest.raises(RXGError):  # a patch id with no face
        RXMeshStatic(fv, nv, host_only=True, face_patch=np.where(fp == 1, 2, fp))
    with pytest.raises(RXGError):  # negative id
        RXMeshStatic(fv, nv, host_only=True, face_patch=np.where(fp == 1, -1, fp))
    with pytest.raises(RXGError):  # more than 4096 faces in a patch
        big, bigf = meshgen.plane(60, 60)
        RXMeshStatic(bigf, len(big), host_only=True, face_patch=np.zeros(len(bigf), np.int32))
    vp = ref["vertex_patch"].astype(np.int32).copy()
    inner = np.setdiff1d(np.unique(fv[fp == 0]), np.unique(fv[fp == 1]))[0]
    vp[inner] = 1  # owner patch holds none of the vertex's faces
    with pytest.raises(RXGError):
        RXMeshStatic(fv, nv, host_only=True, face_patch=fp, vertex_patch=vp)
    with pytest.raises(RXGError):  # edge_patch of the wrong length
        RXMeshStatic(fv, nv, host_only=True, face_patch=fp,
                     edge_patch=ref["edge_patch"][:-1])
    raw = g["patcher_file"].tobytes()
    for bad in (raw[:-3], raw[:200], b"", b"\x07" + raw[1:]):
        p = tmp_path / "bad_patches"
        p.write_bytes(bad)
        with pytest.raises(RXGError):
            RXMeshStatic(fv, nv, host_only=True, patcher_file=str(p))
    with pytest.raises(RXGError):  # written for another mesh
        t = golden("torus")
        RXMeshStatic(t["fv"], len(t["xyz"]), host_only=True, patcher_file=str(path))
    with pytest.raises(RXGError):
        RXMeshStatic(fv, nv, host_only=True, patcher_file=str(tmp_path / "missing"))
    with pytest.raises(ValueError):  # two partition sources
        RXMeshStatic(fv, nv, host_only=True, patcher_file=str(path), face_patch=fp)
    with pytest.raises(ValueError):
        RXMeshStatic(fv, nv, host_only=True, face_patch=fp, gpu_patcher=True)


@pytest.mark.parametrize("P", [64, 512])
def test_lloyd_restatement_gives_valid_partitions(P):
    """The oracle's restatement of the Lloyd patcher (which the GPU patcher
    must equal): every face in a region of at most P faces, at least one
    region per component, and the partition builds."""
    from conftest import edge_case_meshes
    from oracle.patcher import face_graph, lloyd_partition
    from rxmesh_gb300 import RXMeshStatic
    meshes = [meshgen.torus(40, 24, jitter=1e-3, seed=2), meshgen.icosphere(3)]
    meshes += list(edge_case_meshes().values())
    for x, f in meshes:
        fp, runs = lloyd_partition(f, P)
        again, _ = lloyd_partition(f, P)
        assert np.array_equal(fp, again) and runs >= 1
        assert fp.min() == 0 and np.bincount(fp).min() >= 1 and np.bincount(fp).max() <= P
        _, _, comp = face_graph(f)
        for c in np.unique(comp):
            assert len(np.unique(fp[comp == c])) >= 1
            assert not np.isin(np.unique(fp[comp == c]), fp[comp != c]).any()
        rx = RXMeshStatic(f, len(x), host_only=True, face_patch=fp)
        assert rx.get_num_patches() >= fp.max() + 1


def test_obj_constructor(tmp_path):
    """RXMeshStatic.from_obj: the OBJ forms RXMesh's import_obj reads (v/t/n
    indices, negative indices, polygons)."""
    from rxmesh_gb300 import RXMeshStatic
    p = tmp_path / "quad.obj"
    p.write_text("# two faces\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 2 0 0\nvt 0 0\nvn 0 0 1\n"
                 "f 1 2 3 4\nf 2/1/1 -1/1/1 3/1/1\n")
    rx = RXMeshStatic.from_obj(str(p), patch_size=64, host_only=True)
    assert (rx.get_num_vertices(), rx.get_num_edges(), rx.get_num_faces()) == (5, 7, 3)
    assert rx.input_vertex_coordinates.shape == (5, 3)
    same = RXMeshStatic(np.array([[0, 1, 2], [0, 2, 3], [1, 4, 2]]), 5, patch_size=64,
                        host_only=True)
    assert all(np.array_equal(a, b) for a, b in zip(rx.patches(), same.patches()))


def test_multi_file_regions(tmp_path):
    """RXMeshStatic.from_objs: files become disjoint regions with labels."""
    from rxmesh_gb300 import RXMeshStatic
    a = tmp_path / "a.obj"
    a.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3\nf 1 3 4\n")
    b = tmp_path / "b.obj"
    b.write_text("v 0 0 1\nv 1 0 1\nv 0 1 1\nf 1 2 3\n")
    rx = RXMeshStatic.from_objs([str(a), str(b)], patch_size=64, host_only=True)
    assert rx.get_num_regions() == 2
    assert (rx.get_num_vertices(), rx.get_num_faces(), rx.get_num_edges()) == (7, 3, 8)
    assert rx.get_region_label("f").tolist() == [0, 0, 1]
    assert rx.get_region_label("v").tolist() == [0, 0, 0, 0, 1, 1, 1]
    assert sorted(rx.get_region_label("e").tolist()) == [0] * 5 + [1] * 3
    assert rx.input_vertex_coordinates.shape == (7, 3)


def test_export_obj_round_trip(tmp_path):
    """export_obj (rxmesh_static.inl:366-397): linear numbering; reading the
    file back gives the same mesh under the linear-to-input map."""
    from rxmesh_gb300 import RXMeshStatic
    from rxmesh_gb300.meshgen import read_obj
    g = golden("sphere3")
    rx = RXMeshStatic(g["fv"], len(g["xyz"]), patch_size=64, host_only=True)
    vl = rx.linear_to_input("v")
    path = tmp_path / "out.obj"
    rx.export_obj(str(path), g["xyz"][vl])
    x, f = read_obj(str(path))
    assert np.array_equal(x, g["xyz"][vl])
    assert np.array_equal(vl[f], g["fv"][rx.linear_to_input("f")])


@pytest.mark.parametrize("name", ["sphere3", "torus"])
def test_reference_partitions_have_the_lloyd_properties(name):
    """RXMesh's saved Lloyd partitions satisfy what the restatement in
    oracle/patcher.py guarantees: every region at most patch_size faces and
    connected through shared edges."""
    from oracle.patcher import face_graph
    g = golden(name)
    ref = decode(g["patcher_file"].tobytes())
    fp = ref["face_patch"]
    assert np.bincount(fp).max() <= ref["patch_size"]
    off, val, _ = face_graph(g["fv"])
    for p in range(ref["num_patches"]):
        faces = np.nonzero(fp == p)[0]
        seen, stack = {int(faces[0])}, [int(faces[0])]
        while stack:
            f = stack.pop()
            for h in val[off[f]:off[f + 1]]:
                if fp[h] == p and int(h) not in seen:
                    seen.add(int(h))
                    stack.append(int(h))
        assert len(seen) == len(faces), p


def test_partition_argument_checks():
    from rxmesh_gb300 import RXGError, RXMeshStatic
    _, f = meshgen.icosphere(1)
    f = np.asarray(f)
    nv = int(f.max()) + 1
    with pytest.raises(ValueError):  # one id per face
        RXMeshStatic(f, nv, host_only=True, face_patch=np.zeros(len(f) - 1, np.int32))
    with pytest.raises(ValueError):  # one owner per vertex
        RXMeshStatic(f, nv, host_only=True, face_patch=np.zeros(len(f), np.int32),
                     vertex_patch=np.zeros(nv - 1, np.int32))
    with pytest.raises(RXGError):    # patch id beyond the face count
        RXMeshStatic(f, nv, host_only=True, face_patch=np.full(len(f), len(f), np.int32))
    rx = RXMeshStatic(f, nv, host_only=True, face_patch=np.zeros(len(f), np.int32))
    assert rx.get_num_patches() == 1 and rx.info["patch_faces"] == len(f)
