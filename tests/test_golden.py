"""The oracle against golden fixtures written by the reference's own code
(tests/golden/make_golden.py): bit-identical Gauss/shape tables, Diagonize,
and Linear_EQS::Solver (BiCGStab and CG with Jacobi).  Runs everywhere,
including machines without the reference sources."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def tables():
    return np.load(os.path.join(GOLDEN, "ref_tables.npz"))


@pytest.fixture(scope="module")
def eqs():
    return np.load(os.path.join(GOLDEN, "ref_linear_eqs.npz"))


def test_gauss_constants(oracle, tables):
    for g in range(1, 5):
        for p in range(g):
            assert oracle.lib().orc_gauss_point(g, p) == tables["gauss_points"][g - 1, p]
            assert oracle.lib().orc_gauss_weight(g, p) == tables["gauss_weights"][g - 1, p]
    v = np.zeros(4)
    for n in range(5):
        oracle.lib().orc_tet5_point(n, v)
        assert np.array_equal(v, tables["tet5"][n])


@pytest.mark.parametrize("et,name", [(0, "quad"), (1, "hex"), (2, "tet")])
def test_shape_tables(oracle, tables, et, name):
    xi, w, N, dN = oracle.shape_table(et, 3)
    assert np.array_equal(xi, tables[f"{name}_xi"])
    assert np.array_equal(N, tables[f"{name}_N"])
    assert np.array_equal(dN.reshape(len(w), -1), tables[f"{name}_dN"])


def test_diagonize_and_solvers(oracle, eqs):
    rp, col = eqs["row_ptr"], eqs["col"]
    v, b = eqs["val"].copy(), eqs["b"].copy()
    oracle.dirichlet(rp, col, v, b, eqs["bc_rows"], eqs["bc_vals"])
    assert np.array_equal(v, eqs["val_row_only"]) and np.array_equal(b, eqs["b_row_only"])
    x, info = oracle.solve(rp, col, v, b, eqs["x0"], method=2, precond=1, max_iter=2000, tol=1e-12)
    assert info["iterations"] == int(eqs["iter_bicgstab"])
    assert info["rel_residual"] == float(eqs["err_bicgstab"])
    assert np.array_equal(x, eqs["x_bicgstab"])
    vs, bs = eqs["val"].copy(), eqs["b"].copy()
    oracle.dirichlet(rp, col, vs, bs, eqs["bc_rows"], eqs["bc_vals"], symmetric=True)
    assert np.array_equal(vs, eqs["val_sym"]) and np.array_equal(bs, eqs["b_sym"])
    x, info = oracle.solve(rp, col, vs, bs, eqs["x0"], method=5, precond=1, max_iter=2000, tol=1e-12)
    assert info["iterations"] == int(eqs["iter_cg"])
    assert np.array_equal(x, eqs["x_cg"])


def test_fixture_assembly_reproduces(oracle, eqs):
    """The fixture's matrix is the oracle's assembly of the seeded deck."""
    from ogs5_gb300 import mesh as M
    m = M.structured_hex(*[int(v) for v in eqs["shape"]])
    p = oracle.make_params(pcs_type=0, dt=3600.0, storage=1e-4)
    val, b = oracle.assemble(m, eqs["row_ptr"], eqs["col"], p, elem_k=eqs["elem_k"], u0=eqs["u0"])
    assert np.array_equal(val, eqs["val"]) and np.array_equal(b, eqs["b"])
