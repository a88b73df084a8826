"""The C++ mirror of Linear_EQS (include/ogs_gpu.hpp): it compiles with g++
against the C ABI alone and links against libogs_gpu.so (CPU), and drives
the 100 x 100 quad deck to the exact bilinear solution (GPU)."""
import os
import subprocess

import pytest

from ogs5_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "linear_eqs_quad100.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build", "linear_eqs_quad100")


def _compile():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    lib = B.build()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", OUT,
           "-L", os.path.dirname(lib), "-logs_gpu", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_mirror_compiles_and_links():
    _compile()
    assert os.path.exists(OUT)


@pytest.mark.gpu
def test_cpp_mirror_quad100_deck():
    _compile()
    r = subprocess.run([OUT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "PASS" in r.stdout, r.stdout + r.stderr


def test_cpp_deck_reader(tmp_path):
    """ogs_gpu::Deck (C++ mirror, host code only) reads a generated hex deck:
    mesh size and the surface Dirichlet rows equal the Python reader's."""
    from ogs5_gb300 import capi
    from ogs5_gb300 import deck as D
    from ogs5_gb300 import mesh as M
    src = os.path.join(ROOT, "tests", "cpp", "deck_reader.cpp")
    out = os.path.join(ROOT, "tests", "cpp", "_build", "deck_reader")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    lib = B.build()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", out,
           "-L", os.path.dirname(lib), "-logs_gpu", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    m = M.structured_hex(5, 4, 3)
    D.write_msh(m, str(tmp_path / "h.msh"))
    D.write_gli(str(tmp_path / "h.gli"), [(0, 0, 0), (0, 4, 0), (0, 4, 3), (0, 0, 3)],
                {"left": ([0, 1, 2, 3, 0], None)}, {"LEFT": ["left"]})
    D.write_bc(str(tmp_path / "h.bc"), [("GROUNDWATER_FLOW", "HEAD", "SURFACE", "LEFT", 2.5)])
    r = subprocess.run([out, str(tmp_path / "h.msh"), str(tmp_path / "h.gli"), str(tmp_path / "h.bc")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0].startswith(f"nodes {m.n_nodes} elements {m.n_elements} type 1 h 1.000000 bc ")
    rows = [int(l.split()[0]) for l in lines[1:]]
    want, vals = capi.Deck(str(tmp_path / "h.msh"), str(tmp_path / "h.gli"), str(tmp_path / "h.bc")).dirichlet(
        "GROUNDWATER_FLOW")
    assert rows == want.tolist() == m.face_nodes(0, 0).tolist()
    assert all(float(l.split()[1]) == 2.5 for l in lines[1:])
