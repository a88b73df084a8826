"""The C-ABI library builds, loads without a GPU and exports every entry
point include/ogs_gpu.h declares; ctypes structure layouts equal the C ones."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "ogs_gpu.h")).read()
    return sorted(set(re.findall(r"\b(ogs_(?:gpu|deck)_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def built():
    from ogs5_gb300 import build
    build.build()
    from ogs5_gb300 import capi
    return capi


def test_exports_every_declared_symbol(built):
    names = header_functions()
    assert len(names) >= 19
    L = built.lib()
    for n in names:
        getattr(L, n)
    assert set(names) == set(built.EXPORTS)
    assert b"sm_103a" in L.ogs_gpu_version()


def test_struct_layouts_match_c(built, tmp_path):
    import ctypes as C
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "ogs_gpu.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(ogs_mesh_desc),'
                   'sizeof(ogs_assembly_params), sizeof(ogs_solver_config), sizeof(ogs_solve_stats),'
                   'offsetof(ogs_assembly_params, alpha_l), offsetof(ogs_solve_stats, solve_ms));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [C.sizeof(built.MeshDesc), C.sizeof(built.AssemblyParams), C.sizeof(built.SolverConfig),
            C.sizeof(built.SolveStats), built.AssemblyParams.alpha_l.offset,
            built.SolveStats.solve_ms.offset]
    assert got == want


def test_calls_without_gpu_fail_loudly(built):
    """No CPU fallback: with no device the library reports an error."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("machine has a GPU")
    from ogs5_gb300 import mesh as M
    with pytest.raises(built.OgsError):
        built.GpuMesh(M.structured_hex(2, 2, 2))


def test_bad_arguments_rejected_before_device_work(built):
    import ctypes as C
    L = built.lib()
    h = C.c_void_p()
    assert L.ogs_gpu_mesh_create(None, C.byref(h)) == built.BAD_ARG
    assert L.ogs_gpu_configure(None, None) == built.BAD_ARG
    assert L.ogs_gpu_solve(None, None, None) == built.BAD_ARG
    assert b"NULL" in L.ogs_gpu_last_error()
