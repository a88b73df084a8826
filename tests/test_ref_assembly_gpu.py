"""The CUDA path, through the C ABI, against the reference OGS-5's own
element assembly, Cal_Velocity and Picard loop (tests/golden/ref_assembly.npz,
written by the reference compiled from its sources).

Bars (the benchmark spec): matrix entries and right-hand sides 1e-12 relative (floor
1e-14 x row maximum); Gauss-point velocities 1e-12 relative to the largest
flux; Picard heads 1e-10 relative, on linear solves to 1e-14, with the
reference's number of Picard iterations.
"""
import numpy as np
import pytest

from tests import ref_cases as RC
from tests.helpers import assert_matrix_close, assert_vector_close, rel_max_err

pytestmark = pytest.mark.gpu


def gpu_params(gpu, p: dict):
    return gpu.make_params(**p)


def system(gpu, c):
    gm = gpu.GpuMesh(c.mesh, gauss_points=c.ngauss)
    eqs = gpu.LinearEQS(gm)
    return gm, eqs


@pytest.mark.parametrize("name", RC.by_kind("assembly"))
def test_assembly_matches_reference(gpu, name):
    c = RC.case(name)
    gm, eqs = system(gpu, c)
    eqs.Initialize()
    gpv = c["gp_vel"] if "gp_vel" in c else None
    eqs.GlobalAssembly(gpu_params(gpu, c.params), c.arrays.get("elem_k"), c["u0"], gpv)
    rp, col, val = eqs.get_csr()
    assert np.array_equal(rp, c["row_ptr"]) and np.array_equal(col, c["col"])
    assert_matrix_close(rp, val, c["val"])
    assert_vector_close(eqs.get_rhs(), c["b"])
    if "val_2" in c:
        # $MEMORY_TYPE: the second step combines the operators stored by the
        # first with the new dt and u0; its velocities are not read
        eqs.Initialize()
        p2 = gpu_params(gpu, dict(c.params, dt=c.meta["dt_2"]))
        eqs.GlobalAssembly(p2, None, c["u0_2"], c["gp_vel_2"])
        _, _, val2 = eqs.get_csr()
        assert_matrix_close(rp, val2, c["val_2"])
        assert_vector_close(eqs.get_rhs(), c["b_2"])


@pytest.mark.parametrize("name", RC.by_kind("velocity"))
def test_gp_velocity_matches_reference(gpu, name):
    c = RC.case(name)
    gm, eqs = system(gpu, c)
    q = eqs.gp_velocity(gpu_params(gpu, c.params), c["elem_k"], c["u"])
    assert_vector_close(q.ravel(), c["gp_vel"].ravel())


@pytest.mark.parametrize("name", RC.by_kind("richards"))
def test_richards_assembly_matches_reference(gpu, name):
    c = RC.case(name)
    gm, eqs = system(gpu, c)
    eqs.Initialize()
    r = gpu.richards_params(**c.meta["richards"])
    eqs.AssembleRichards(gpu_params(gpu, c.params), r, c["elem_k"], c["p_old"], c["p_iter"])
    rp, col, val = eqs.get_csr()
    assert_matrix_close(rp, val, c["val"])
    assert_vector_close(eqs.get_rhs(), c["b"])


ERROR_METHODS = {"LMAX": 1, "ENORM": 2, "EVNORM": 3, "ERNORM": 4}


@pytest.mark.parametrize("name", RC.by_kind("picard"))
def test_richards_picard_matches_reference(gpu, name):
    c = RC.case(name)
    gm, eqs = system(gpu, c)
    pc = c.meta["picard"]
    eqs.ConfigNumerics(ls_method=gpu.LS_BICGSTAB, ls_precond=gpu.PRECOND_JACOBI,
                       ls_max_iterations=5000, ls_error_tolerance=pc["linear_tol"])
    r = gpu.richards_params(**c.meta["richards"])
    it = np.array(c["p_old"], dtype=np.float64)
    st = eqs.RichardsStep(gpu_params(gpu, c.params), r, c["elem_k"], c["p_old"], it, c["bc_rows"],
                          c["bc_vals"], mode=gpu.DIRICHLET_ROW_ONLY,
                          error_method=ERROR_METHODS[pc["error_method"]],
                          max_iterations=pc["max_iterations"], tolerance=pc["tolerance"], allow_fail=True)
    # the reference's iter_nlin is the loop index at exit: iterations run - 1
    assert st["iterations"] == int(c["iterations"]) + 1
    assert rel_max_err(it, c["p_new"]) < 1e-10


@pytest.mark.parametrize("name", RC.by_kind("solve"))
def test_solution_matches_reference(gpu, name):
    """GPU assembly, Dirichlet (row-only as the SP build, symmetric as
    MXRandbed) and the configured Krylov solve to 1e-14, against the heads
    the reference solved (SP Linear_EQS::BiCGStab; legacy SpCG and the
    M34Vorkond incomplete LDU): 1e-10 relative."""
    c = RC.case(name)
    s = c.meta["solve"]
    gm, eqs = system(gpu, c)
    eqs.ConfigNumerics(ls_method=s["ls_method"], ls_precond=s["precond"], ls_max_iterations=20000,
                       ls_error_tolerance=s["tol"])
    eqs.Initialize()
    eqs.GlobalAssembly(gpu_params(gpu, c.params), c["elem_k"], c["u0"])
    mode = gpu.DIRICHLET_SYMMETRIC if s["dirichlet"] == "symmetric" else gpu.DIRICHLET_ROW_ONLY
    eqs.SetKnownX(c["bc_rows"], c["bc_vals"], mode)
    x = np.array(c["u0"], dtype=np.float64)
    eqs.Solver(x)
    assert rel_max_err(x, c["x_ref"]) < 1e-10
