"""The bounds-checked build (-DOGS_BOUNDS_CHECK: every SELL slot and column,
element node, lattice neighbour, Dirichlet row and ILU column index is
checked before its access) on the small cases of tests/bounds_cases.py, in
a child process that loads libogs_gpu_debug.so: no kernel meets an index
out of range.  The substitute for a memory checker on this path."""
import json
import os
import subprocess
import sys

import pytest

from ogs5_gb300 import build as B

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_small_cases_stay_in_bounds():
    lib = B.build(debug=True)
    env = dict(os.environ, OGS_GPU_LIB=lib)
    r = subprocess.run([sys.executable, "-m", "tests.bounds_cases"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert lines and lines[-1] == {"all": "clean"}
    assert len(lines) >= 14  # every case ran
