"""The oracle against the reference's own compiled code (oracle/_ref:
FEM/mathlib.cpp, FEM/matrix_class.cpp, FEM/equation_class.cpp), where the
reference sources are present; elsewhere the committed golden fixtures made
from the same library stand in (test_golden.py)."""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M


@pytest.fixture(scope="module")
def ref(oracle):
    import os
    if not os.path.isdir("/root/reference"):
        pytest.skip("reference sources not present on this machine")
    oracle.build("/root/reference")
    if not oracle.ref_available():
        pytest.skip("reference harness not built")
    return oracle.ref()


def test_gauss_tables_identical(oracle, ref):
    for g in (1, 2, 3, 4):
        for p in range(g):
            assert oracle.lib().orc_gauss_point(g, p) == ref.ref_gauss_point(g, p)
            assert oracle.lib().orc_gauss_weight(g, p) == ref.ref_gauss_weight(g, p)
    a, b = np.zeros(4), np.zeros(4)
    for n in range(5):
        oracle.lib().orc_tet5_point(n, a)
        ref.ref_tet5_point(n, b)
        assert np.array_equal(a, b)


@pytest.mark.parametrize("et", [0, 1, 2])
@pytest.mark.parametrize("ng", [1, 2, 3])
def test_shape_tables_identical(oracle, ref, et, ng):
    xi, w, N, dN = oracle.shape_table(et, ng)
    nn, dim = N.shape[1], dN.shape[1]
    for gp in range(len(w)):
        Nr, dNr = np.zeros(nn), np.zeros(nn * dim)
        ref.ref_shape(et, np.ascontiguousarray(xi[gp]), Nr, dNr)
        assert np.array_equal(Nr, N[gp]) and np.array_equal(dNr, dN[gp].ravel())


def _system(oracle, m, ek, u0, dt, ss):
    rp, col = oracle.build_pattern(m.n_nodes, m.conn)
    p = oracle.make_params(pcs_type=0, dt=dt, storage=ss)
    val, b = oracle.assemble(m, rp, col, p, elem_k=ek, u0=u0)
    return rp, col, val, b


def test_scatter_through_operator_parenthesis(oracle, ref):
    """The oracle's CSR position search equals CSparseMatrix::operator()."""
    m = M.structured_tet(3, 3, 2)
    rp, col = oracle.build_pattern(m.n_nodes, m.conn)
    rs = oracle.RefSystem(rp, col)
    rs.set(np.zeros(len(col)), np.zeros(m.n_nodes))
    rng = np.random.default_rng(0)
    want = np.zeros(len(col))
    for e in range(m.n_elements):
        for i in m.conn[e]:
            for j in m.conn[e]:
                v = rng.standard_normal()
                rs.add(i, j, v)
                k = rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], j)
                want[k] += v
    got, _ = rs.get()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("method,precond,symmetric", [(2, 1, False), (2, 0, False), (5, 1, True),
                                                     (5, 0, True)])
def test_solver_identical_to_linear_eqs(oracle, ref, method, precond, symmetric):
    """Same iterations, residual and solution bits as Linear_EQS::Solver."""
    m = M.structured_hex(8, 6, 5)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 3.0, seed=4)
    rp, col, val, b = _system(oracle, m, ek, np.zeros(m.n_nodes), 3600.0, 1e-4)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    rs = oracle.RefSystem(rp, col, method=method, precond=precond, max_iter=3000, tol=1e-12)
    v2, b2 = val.copy(), b.copy()
    if symmetric:
        oracle.dirichlet(rp, col, v2, b2, rows, vals, symmetric=True)
        rs.set(v2, b2)
    else:
        rs.set(val, b)
        rs.set_known(rows, vals)
        oracle.dirichlet(rp, col, v2, b2, rows, vals)
        vr, br = rs.get()
        assert np.array_equal(vr, v2) and np.array_equal(br, b2)  # Diagonize
    xr, ir = rs.solve(x0)
    xo, io = oracle.solve(rp, col, v2, b2, x0, method=method, precond=precond, max_iter=3000,
                          tol=1e-12)
    assert ir["iterations"] == io["iterations"]
    assert ir["rel_residual"] == io["rel_residual"]
    assert np.array_equal(xr, xo)


def test_spmv_identical_to_multivec(oracle, ref):
    m = M.structured_quad(17, 11)
    rp, col, val, b = _system(oracle, m, np.full(m.n_elements, 2e-4), np.zeros(m.n_nodes), 10.0, 1e-3)
    rs = oracle.RefSystem(rp, col)
    rs.set(val, b)
    x = np.random.default_rng(1).standard_normal(m.n_nodes)
    assert np.array_equal(rs.spmv(x), oracle.spmv(rp, col, val, x))


def test_bicgstab_breakdown_with_ic_zero(oracle, ref):
    """BiCGStab breaks down (|rho| < DBL_MIN) when x0 violates the row-only
    Dirichlet values, in the reference and the oracle alike."""
    m = M.structured_quad(10, 10)
    rp, col, val, b = _system(oracle, m, np.full(m.n_elements, 1e-4), np.zeros(m.n_nodes), 1.0, 0.0)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.ones(len(lf)), np.zeros(len(rf))])
    v2, b2 = val.copy(), b.copy()
    oracle.dirichlet(rp, col, v2, b2, rows, vals)
    rs = oracle.RefSystem(rp, col, method=2, precond=1, max_iter=1000, tol=1e-10)
    rs.set(v2, b2)
    xr, ir = rs.solve(np.zeros(m.n_nodes))
    xo, io = oracle.solve(rp, col, v2, b2, np.zeros(m.n_nodes), method=2, precond=1, tol=1e-10)
    # Solver() stores BiCGStab()'s return value, 0 at a breakdown; the oracle
    # reports the iteration at which |rho| fell below DBL_MIN
    assert io["breakdown"] and ir["iterations"] == 0 and io["iterations"] == 2
    assert io["rel_residual"] > 1e-3 and np.array_equal(xr, xo)


def test_write_bin_layout(oracle, ref):
    """Linear_EQS::Write_BIN emits the CRS arrays the C ABI's get_csr returns."""
    m = M.structured_quad(3, 2)
    rp, col, val, b = _system(oracle, m, np.full(m.n_elements, 1.0), np.zeros(m.n_nodes), 1.0, 0.0)
    rs = oracle.RefSystem(rp, col)
    rs.set(val, b)
    raw = rs.write_bin()
    assert len(raw) > 0
    # the value array appears verbatim in the dump
    assert val.tobytes() in raw
