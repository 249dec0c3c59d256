"""Compile librxg.so (every CUDA translation unit, sm_103a only) in-tree.

Usage: python -m rxmesh_gb300.build   (or rxmesh_gb300.build.build())
Objects go to rxmesh_gb300/_build/, the library to rxmesh_gb300/_build/librxg.so.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librxg.so")

SOURCES = ["rxg_mesh.cpp", "rxg_patchfile.cpp", "rxg_patcher.cu", "rxg_query.cu", "rxg_mcf.cu", "rxg_onchip.cu", "rxg_dense.cu", "rxg_arap.cu", "rxg_batch.cu", "rxg_term.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(HERE, "..", "include")]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OUT, src.rsplit(".", 1)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + ["-lineinfo", "-c", path, "-o", obj]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-warn-spills"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def _stale(objs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "rxg.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and not _stale(None):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        res = list(ex.map(_compile, SOURCES))
    if verbose:
        for _, err in res:
            if err.strip():
                sys.stderr.write(err)
    objs = [o for o, _ in res]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
