"""Device-side queries through the facade (include/rxg/query.cuh).

tests/cpp/for_each_example.cu is written like an RXMesh application:
RXMeshStatic::for_each<Op, 256>(device lambda) for every query op (and
oriented VV), attributes read and written through handles (an umbrella
operator on the input coordinates), for_each_vertex / for_each_face on the
device and the host, and run_kernel with kernels of its own that drive
Query<blockThreads> (dispatch with an active-set predicate and
compute_vertex_valence; prologue / run_compute / epilogue).  It writes its
results to binary files; this test compares them with the oracle in input
ids: rows as sorted sets (the form of tests/RXMesh_test/rxmesh_test.h:
347-440), FV / FE / EV / EVDiamond / EE rows and the oriented ring in order.
The program compiles here (nvcc cross-compiles without a GPU); it runs on
the GPU.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import edge_case_meshes, golden
from rxmesh_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


@pytest.fixture(scope="module")
def example(tmp_path_factory):
    from rxmesh_gb300 import _lib
    _lib.load()  # builds librxg.so when missing or stale
    libdir = os.path.dirname(_lib.lib_path())
    exe = str(tmp_path_factory.mktemp("for_each") / "for_each_example")
    cmd = [_nvcc(), "-std=c++17", "--extended-lambda", "-O2",
           "-gencode", "arch=compute_103a,code=sm_103a",
           os.path.join(ROOT, "tests", "cpp", "for_each_example.cu"),
           "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lrxg",
           "-Xlinker", "-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_for_each_example_compiles(example):
    assert os.path.exists(example)


def write_obj(path, x, f):
    with open(path, "w") as fh:
        for p in x:
            fh.write("v %.17g %.17g %.17g\n" % tuple(p))
        for t in np.asarray(f):
            fh.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))


MESHES = {
    "icosphere4": (lambda: meshgen.icosphere(4), 128),
    "plane": (lambda: meshgen.plane(31, 17, 0.1), 64),
    "torus": (lambda: meshgen.torus(64, 48, jitter=1e-3, seed=2), 64),
    "bunnyhead": (lambda: (golden("bunnyhead")["xyz"], golden("bunnyhead")["fv"]), 256),
    "components": (lambda: edge_case_meshes()["components"], 64),
}


def load(d, name, dtype=np.int32):
    return np.fromfile(os.path.join(d, name + ".bin"), dtype=dtype)


def pairs(rows, vals):
    o = np.lexsort((vals, rows))
    return rows[o], vals[o]


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(MESHES))
def test_for_each_matches_oracle(oracle, example, tmp_path, name):
    make, patch = MESHES[name]
    x, f = make()
    x = np.asarray(x, np.float64)
    f = np.asarray(f, np.int32)
    nv, nf = len(x), len(f)
    obj = str(tmp_path / "mesh.obj")
    write_obj(obj, x, f)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([example, obj, str(patch), str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
    d = str(out)
    l2i = [load(d, "l2i_%d" % e).astype(np.int64) for e in range(3)]
    ev, fe = oracle.edges(f)
    ne = len(ev)
    sizes = {0: nv, 1: ne, 2: nf}

    def rows_of(tag, src, dst, W):
        cnt = load(d, tag + "_cnt")
        val = load(d, tag + "_val").reshape(-1, W)
        assert cnt.shape[0] == sizes[src] and (cnt >= 0).all() and (cnt <= W).all(), tag
        mask = np.arange(W)[None, :] < cnt[:, None]
        assert (val[mask] >= 0).all(), tag  # every entry resolved to a linear id
        rows = np.repeat(l2i[src], cnt)
        vals = l2i[dst][val[mask]]
        return cnt, val, rows, vals

    # sets
    for tag, src, dst, W, ref in (("vv", 0, 0, 16, oracle.vv(nv, ev)),
                                  ("ve", 0, 1, 16, oracle.vv(nv, ev, want_edges=True)),
                                  ("vf", 0, 2, 16, oracle.vf(nv, f)),
                                  ("ef", 1, 2, 8, oracle.ef(f)),
                                  ("ff", 2, 2, 16, oracle.ff(f))):
        _, _, rows, vals = rows_of(tag, src, dst, W)
        off, v = ref
        wr, wv = pairs(np.repeat(np.arange(len(off) - 1), np.diff(off)), np.asarray(v, np.int64))
        gr, gv = pairs(rows, vals)
        assert np.array_equal(gr, wr) and np.array_equal(gv, wv), tag
    # fixed-size rows, in order
    for tag, src, dst, W, want in (("fv", 2, 0, 3, f), ("fe", 2, 1, 3, fe), ("ev", 1, 0, 2, ev)):
        cnt, val, _, _ = rows_of(tag, src, dst, W)
        assert (cnt == W).all(), tag
        got = np.empty((sizes[src], W), np.int64)
        got[l2i[src]] = l2i[dst][val]
        assert np.array_equal(got, want), tag
    if rx_manifold_oriented(f):
        cnt = load(d, "evd_cnt")
        val = load(d, "evd_val").reshape(-1, 4)
        assert (cnt == 4).all()
        got = np.empty((ne, 4), np.int64)
        got[l2i[1]] = np.where(val >= 0, l2i[0][np.maximum(val, 0)], -1)
        assert np.array_equal(got, oracle.ev_diamond(f))
        cnt = load(d, "ee_cnt")
        val = load(d, "ee_val").reshape(-1, 4)
        assert (cnt == 4).all()
        got = np.empty((ne, 4), np.int64)
        got[l2i[1]] = np.where(val >= 0, l2i[1][np.maximum(val, 0)], -1)
        assert np.array_equal(got, oracle.ee(f))
        # oriented VV: the oracle's rotational order (cyclic for interior vertices)
        o_off, o_ring, o_bnd = oracle.oriented_vv(nv, f)
        cnt = load(d, "vvo_cnt")
        val = load(d, "vvo_val").reshape(-1, 16)
        for lin in range(nv):
            p = l2i[0][lin]
            r_ = l2i[0][val[lin, :cnt[lin]]].tolist()
            w = o_ring[o_off[p]:o_off[p + 1]].tolist()
            if o_bnd[p]:
                assert r_ == w, (lin, r_, w)
            elif w:
                k = w.index(r_[0])
                assert r_ == w[k:] + w[:k], (lin, r_, w)
    # attributes through handles: umbrella operator on the input coordinates
    lap = load(d, "lap", np.float64).reshape(-1, 3)
    off, v = oracle.vv(nv, ev)
    rows = np.repeat(np.arange(nv), np.diff(off))
    want = np.zeros((nv, 3))
    np.add.at(want, rows, x[v] - x[rows])
    got = np.empty((nv, 3))
    got[l2i[0]] = lap
    assert np.abs(got - want).max() <= 1e-12 * max(1.0, np.abs(x).max())
    # run_kernel: active set (even linear ids) and vertex valence
    act = load(d, "active")
    deg = np.diff(off)[l2i[0]]
    even = (np.arange(nv) % 2) == 0
    assert np.array_equal(act[even], 1001 * deg[even])
    assert (act[~even] == -1).all()
    # prologue / run_compute / epilogue: per face, the sum of its vertices' linear ids
    il_v = np.empty(nv, np.int64)
    il_v[l2i[0]] = np.arange(nv)
    fsum = load(d, "fsum")
    assert np.array_equal(fsum, il_v[f[l2i[2]]].sum(1))


def rx_manifold_oriented(f):
    """Edge-manifold and consistently oriented (no directed edge twice)."""
    f = np.asarray(f, np.int64)
    d = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    key = d[:, 0] * (f.max() + 1) + d[:, 1]
    return len(np.unique(key)) == len(key)
