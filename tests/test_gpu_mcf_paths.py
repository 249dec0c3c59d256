"""The mixed MCF step's two solver paths agree: the one-launch on-chip solve
and the launch-per-sweep solve it falls back to for meshes too large for the
on-chip state (RXG_MCF_ONCHIP=0 forces the latter; the switch is read once
per process, so each path runs in its own child process)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np, torch
sys.path.insert(0, %r)
from rxmesh_gb300 import RXMeshStatic, meshgen, mcf_step
v, f = meshgen.icosphere(5)
x0 = meshgen.radial_noise(v, 0.02, 3)
rx = RXMeshStatic(f, len(x0), patch_size=256)
x = rx.to_linear(torch.tensor(x0, device="cuda"))
st = mcf_step(rx, x, 1e-3, 3, "mixed", tol=1e-9)
print(json.dumps({"x": rx.to_input(x).cpu().numpy().ravel().tolist(), "st": st}))
"""


def run_child(onchip):
    env = dict(os.environ)
    env["RXG_MCF_ONCHIP"] = "1" if onchip else "0"
    r = subprocess.run([sys.executable, "-c", CHILD % ROOT], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return np.array(d["x"]), d["st"]


def test_onchip_and_sweep_paths_agree(oracle):
    a, sa = run_child(True)
    b, sb = run_child(False)
    assert sa["converged"] and sb["converged"]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-8
