"""The C restatement (oracle/ogs_oracle.c) against the reference OGS-5's own
element assembly, Cal_Velocity and Picard loop (tests/golden/ref_assembly.npz,
written by the reference compiled from its sources).

Bars: matrix entries and right-hand sides 1e-12 relative (floor 1e-14 x row
maximum); Gauss-point velocities 1e-12 relative to the largest flux; Picard
heads 1e-10 relative with the same number of Picard iterations.
"""
import numpy as np
import pytest

from tests import ref_cases as RC
from tests.helpers import assert_matrix_close, assert_vector_close, rel_max_err


def oracle_params(O, p: dict):
    return O.make_params(**p)


@pytest.mark.parametrize("name", RC.by_kind("assembly"))
def test_assembly_matches_reference(oracle, name):
    c = RC.case(name)
    rp, col = oracle.build_pattern(c.mesh.n_nodes, c.mesh.conn)
    assert np.array_equal(rp, c["row_ptr"]) and np.array_equal(col, c["col"]), \
        "SparseTable CRS pattern differs from the reference's"
    p = oracle_params(oracle, c.params)
    gpv = c["gp_vel"] if "gp_vel" in c else None
    val, b = oracle.assemble(c.mesh, rp, col, p, elem_k=c.arrays.get("elem_k"), u0=c["u0"],
                             gp_vel=gpv, ngauss=c.ngauss)
    assert_matrix_close(rp, val, c["val"])
    assert_vector_close(b, c["b"])
    if "val_2" in c:
        # $MEMORY_TYPE: the reference's second step recombines the element
        # matrices of the first step (its velocities) with the new dt and u0
        p2 = oracle_params(oracle, dict(c.params, dt=c.meta["dt_2"], memory_type=0))
        val2, b2 = oracle.assemble(c.mesh, rp, col, p2, u0=c["u0_2"], gp_vel=gpv, ngauss=c.ngauss)
        assert_matrix_close(rp, val2, c["val_2"])
        assert_vector_close(b2, c["b_2"])


@pytest.mark.parametrize("name", RC.by_kind("velocity"))
def test_gp_velocity_matches_reference(oracle, name):
    c = RC.case(name)
    q = oracle.gp_velocity(c.mesh, oracle_params(oracle, c.params), c["elem_k"], c["u"], ngauss=c.ngauss)
    want = c["gp_vel"]
    assert_vector_close(q.ravel(), want.ravel())


@pytest.mark.parametrize("name", RC.by_kind("richards"))
def test_richards_assembly_matches_reference(oracle, name):
    c = RC.case(name)
    rp, col = oracle.build_pattern(c.mesh.n_nodes, c.mesh.conn)
    r = oracle.richards_params(**c.meta["richards"])
    val, b = oracle.assemble_richards(c.mesh, rp, col, oracle_params(oracle, c.params), r, c["elem_k"],
                                      c["p_old"], c["p_iter"], ngauss=c.ngauss)
    assert_matrix_close(rp, val, c["val"])
    assert_vector_close(b, c["b"])


ERROR_METHODS = {"LMAX": 1, "ENORM": 2, "EVNORM": 3, "ERNORM": 4}


@pytest.mark.parametrize("name", RC.by_kind("picard"))
def test_richards_picard_matches_reference(oracle, name):
    c = RC.case(name)
    rp, col = oracle.build_pattern(c.mesh.n_nodes, c.mesh.conn)
    r = oracle.richards_params(**c.meta["richards"])
    pc = c.meta["picard"]
    x, info = oracle.richards_picard(
        c.mesh, rp, col, oracle_params(oracle, c.params), r, c["elem_k"], c["p_old"], c["p_old"],
        c["bc_rows"], c["bc_vals"], symmetric=False, error_method=ERROR_METHODS[pc["error_method"]],
        tolerance=pc["tolerance"], max_iterations=pc["max_iterations"], method=2, precond=1,
        max_iter=5000, tol=pc["linear_tol"])
    # the reference's iter_nlin is the loop index at exit: iterations run - 1
    assert info["iterations"] == int(c["iterations"]) + 1
    assert rel_max_err(x, c["p_new"]) < 1e-10


@pytest.mark.parametrize("name", RC.by_kind("solve"))
def test_solution_matches_reference(oracle, name):
    """A GROUNDWATER_FLOW step with Dirichlet faces solved by the reference:
    the SP build's Diagonize + Linear_EQS::BiCGStab (same iterations, same
    heads), the legacy build's MXRandbed + SpCG, and its M34Vorkond
    incomplete LDU under SpCG / SpBICGSTAB (heads at the solution bar; the
    factorisation orders differ, so only converged heads compare)."""
    c = RC.case(name)
    s = c.meta["solve"]
    rp, col = oracle.build_pattern(c.mesh.n_nodes, c.mesh.conn)
    val, b = oracle.assemble(c.mesh, rp, col, oracle_params(oracle, c.params), elem_k=c["elem_k"], u0=c["u0"])
    oracle.dirichlet(rp, col, val, b, c["bc_rows"], c["bc_vals"], symmetric=s["dirichlet"] == "symmetric")
    x, info = oracle.solve(rp, col, val, b, c["u0"].copy(), method=s["ls_method"], precond=s["precond"],
                           max_iter=20000, tol=s["tol"])
    assert rel_max_err(x, c["x_ref"]) < 1e-10
    if s["build"] == "SP":
        assert info["iterations"] == int(c["iterations"])
        assert rel_max_err(x, c["x_ref"]) == 0.0
