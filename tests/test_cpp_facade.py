"""The C++ facade (include/rxg/rxmesh.hpp) compiles against the C ABI and runs.

The example program tests/cpp/facade_example.cpp is built with g++ and linked
to librxg.so; `host` mode runs here (mesh build, numbering, error path,
a patcher-file round trip),
`gpu` mode runs the whole path (queries, MCF assembly + PCGSolver, mcf_step,
DiffScalarProblem ARAP, MeshBatch) on the GPU.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


@pytest.fixture(scope="module")
def example(tmp_path_factory):
    from rxmesh_gb300 import _lib
    _lib.load()  # builds librxg.so when missing or stale
    libdir = os.path.dirname(_lib.lib_path())
    cuda = _cuda_home()
    cudalib = os.path.join(cuda, "lib64")
    if not os.path.isdir(cudalib):
        cudalib = os.path.join(cuda, "lib")
    exe = str(tmp_path_factory.mktemp("cpp") / "facade_example")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           os.path.join(ROOT, "tests", "cpp", "facade_example.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           "-L", libdir, "-lrxg", "-L", cudalib, "-lcudart",
           "-Wl,-rpath," + libdir, "-Wl,-rpath," + cudalib, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_host(example, tmp_path):
    r = subprocess.run([example, "host", str(tmp_path)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


@pytest.mark.gpu
def test_facade_gpu(example, tmp_path):
    r = subprocess.run([example, "gpu", str(tmp_path)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
