"""The C++ mirror of Linear_EQS (include/ogs_gpu.hpp): it compiles with g++
against the C ABI alone and links against libogs_gpu.so (CPU), and drives
the 100 x 100 quad deck to the exact bilinear solution (GPU)."""
import os
import subprocess

import pytest

from ogs5_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "linear_eqs_config1.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build", "linear_eqs_config1")


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
def test_cpp_mirror_config1_deck():
    _compile()
    r = subprocess.run([OUT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "PASS" in r.stdout, r.stdout + r.stderr
