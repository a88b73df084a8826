"""ILU(0) preconditioner (ls_precond 100) on the GPU against the oracle.

Factors: every entry of the GPU factorisation equals the oracle's IKJ
ILU(0) on the same matrix within 1e-12 relative (both round products and
differences separately, in the same order per row).  Solves: BiCGStab and CG
with ILU(0) converge to the oracle's heads/concentrations within 1e-10
relative, with iteration counts within 2 of the oracle's.
"""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import SOLUTION_RTOL, assert_matrix_close, rel_max_err, renumber
from tests.test_parity_gpu import _flow_system, k_field

pytestmark = pytest.mark.gpu


def _transport_system(gpu, m, seed=5):
    """MASS_TRANSPORT on m with a Darcy field, c = 1 on the x = 0 face."""
    gm = gpu.GpuMesh(m)
    ngp = gm.n_gauss
    rng = np.random.default_rng(seed)
    gpv = np.zeros((m.n_elements, ngp, 3))
    gpv[:, :, 0] = 1e-5 * (1.0 + 0.3 * rng.standard_normal((m.n_elements, ngp)))
    gpv[:, :, 1] = 2e-6 * rng.standard_normal((m.n_elements, ngp))
    p = gpu.make_params(gpu.MASS_TRANSPORT, dt=600.0, theta=1.0, porosity=0.3,
                        alpha_l=1.0, alpha_t=0.1, diffusion=1e-9)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    c0 = np.zeros(m.n_nodes)
    eqs.GlobalAssembly(p, None, c0, gpv)
    lf = m.face_nodes(0, 0)
    eqs.SetKnownX(lf, np.ones(len(lf)), gpu.DIRICHLET_ROW_ONLY)
    rp, col, val = eqs.get_csr()
    b = eqs.get_rhs()
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 1.0
    return eqs, (rp, col, val, b), x0


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
def test_ilu0_factors_match_oracle(gpu, oracle, kind):
    m = {"quad": M.structured_quad(20, 15), "hex": M.structured_hex(8, 7, 5),
         "tet": M.structured_tet(6, 5, 4)}[kind]
    eqs, (rp, col, val, b), x0 = _flow_system(gpu, oracle, m, k_field(m, 4), symmetric=True,
                                              dt=3600.0, storage=1e-4, left=2.0, right=1.0)
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_ILU0, 500, 1e-12)
    x = x0.copy()
    eqs.Solver(x)
    lu = eqs.get_ilu0()
    want = oracle.ilu0_factor(rp, col, val)
    assert_matrix_close(rp, lu, want)


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_bicgstab_ilu0_transport(gpu, oracle, kind):
    m = M.structured_hex(10, 6, 5) if kind == "hex" else M.structured_tet(8, 5, 4)
    eqs, (rp, col, val, b), x0 = _transport_system(gpu, m)
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_ILU0, 1000, 1e-13, check_norm_rhs=False)
    x = x0.copy()
    it = eqs.Solver(x)
    xo, info = oracle.solve(rp, col, val, b, x0, method=2, precond=100, max_iter=1000, tol=1e-13)
    assert abs(it - info["iterations"]) <= 2
    assert rel_max_err(x, xo) < SOLUTION_RTOL
    # fewer iterations than Jacobi on the same system
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 1000, 1e-13, check_norm_rhs=False)
    xj = x0.copy()
    itj = eqs.Solver(xj)
    assert it < itj
    assert rel_max_err(xj, xo) < SOLUTION_RTOL


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
def test_cg_ilu0_flow(gpu, oracle, kind):
    if kind == "quad":
        m = M.structured_quad(40, 30)
        ek = k_field(m, 3)
    elif kind == "hex":
        m = M.structured_hex(12, 10, 6)
        ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 3.0, seed=4)
    else:
        m = M.structured_tet(8, 6, 5)
        ek = np.repeat(fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 3.0, seed=4), 6)
    eqs, (rp, col, val, b), x0 = _flow_system(gpu, oracle, m, ek, symmetric=True, dt=3600.0,
                                              storage=1e-4, left=10.0, right=0.0)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_ILU0, 3000, 1e-13)
    x = x0.copy()
    it = eqs.Solver(x)
    xo, info = oracle.solve(rp, col, val, b, x0, method=5, precond=100, max_iter=3000, tol=1e-13)
    assert abs(it - info["iterations"]) <= 2
    assert rel_max_err(x, xo) < SOLUTION_RTOL


def test_ilu0_repeated_solves_refactor(gpu, oracle):
    """Each solve factors the current matrix: a re-assembled system gives the
    oracle's answer for the new values, not the old factors'."""
    m = M.structured_hex(6, 6, 4)
    eqs, (rp, col, val, b), x0 = _flow_system(gpu, oracle, m, k_field(m, 1), symmetric=True,
                                              dt=100.0, storage=1e-3, left=1.0, right=0.0)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_ILU0, 1000, 1e-13, check_norm_rhs=False)
    x = x0.copy()
    eqs.Solver(x)
    eqs2, (rp2, col2, val2, b2), x02 = _flow_system(gpu, oracle, m, k_field(m, 9), symmetric=True,
                                                    dt=100.0, storage=1e-3, left=1.0, right=0.0)
    # same LinearEQS object, new values
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=100.0, storage=1e-3)
    eqs.Initialize()
    eqs.GlobalAssembly(p, k_field(m, 9), np.zeros(m.n_nodes))
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    eqs.SetKnownX(np.concatenate([lf, rf]), np.concatenate([np.ones(len(lf)), np.zeros(len(rf))]),
                  gpu.DIRICHLET_SYMMETRIC)
    x = x02.copy()
    eqs.Solver(x)
    xo, _ = oracle.solve(rp2, col2, val2, b2, x02, method=5, precond=100, max_iter=1000, tol=1e-13)
    assert rel_max_err(x, xo) < SOLUTION_RTOL
    assert_matrix_close(rp2, eqs.get_ilu0(), oracle.ilu0_factor(rp2, col2, val2))


def test_ilu0_zero_pivot_is_breakdown(gpu):
    """An all-zero matrix (K = 0, no storage) has a zero pivot in row 0: the
    solve stops with OGS_BREAKDOWN before iterating."""
    m = M.structured_quad(4, 4)
    gm = gpu.GpuMesh(m)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=1.0, storage=0.0, steady=1)
    eqs.GlobalAssembly(p, np.zeros(m.n_elements), np.zeros(m.n_nodes))
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_ILU0, 100, 1e-10, check_norm_rhs=False)
    x = np.ones(m.n_nodes)
    with pytest.raises(gpu.OgsError) as e:
        eqs.Solver(x)
    assert e.value.status == gpu.BREAKDOWN
    assert "zero pivot" in str(e.value)


def test_ilu0_rejected_in_fp32_mode(gpu):
    m = M.structured_quad(4, 4)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_ILU0, 100, 1e-10, precision=gpu.PRECISION_FP32_REFINED)
    with pytest.raises(gpu.OgsError) as e:
        eqs.Solver(np.zeros(m.n_nodes))
    assert e.value.status == gpu.BAD_ARG


@pytest.mark.parametrize("cells", [(8, 5, 4), (7, 8, 9), (16, 16, 8), (17, 9, 10), (3, 3, 2)])
def test_tile_sweeps_match_level_sweeps(gpu, oracle, monkeypatch, cells):
    """On a Kuhn-tet lattice the factorisation and the sweeps walk tiles of
    8^3 nodes; with OGS_ILU_SWEEP=levels they walk dependency levels of rows.
    The same system solved both ways (one assembly: the element scatter's
    FP64 atomics make two assemblies differ in the last bits): the same
    arithmetic per row gives bit for bit the same factors, the same
    iterations and the same solution (full and partial tiles, BiCGStab and
    CG)."""
    m = M.structured_tet(*cells)
    eqs, _, x0 = _transport_system(gpu, m)
    assert eqs.gmesh.ilu_tiles > 0
    ek = np.repeat(fields.lognormal_k(cells, np.log(1e-5), 1.0, 3.0, seed=4), 6)
    feqs, _, f0 = _flow_system(gpu, oracle, m, ek, symmetric=True, dt=3600.0, storage=1e-4, left=10.0, right=0.0)
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_ILU0, 1000, 1e-13, check_norm_rhs=False)
    feqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_ILU0, 3000, 1e-13)
    out = {}
    for mode in ("tiles", "levels", "tiles again"):
        if mode == "levels":
            monkeypatch.setenv("OGS_ILU_SWEEP", "levels")
        else:
            monkeypatch.delenv("OGS_ILU_SWEEP", raising=False)
        x, h = x0.copy(), f0.copy()
        it, fit = eqs.Solver(x), feqs.Solver(h)
        out[mode] = (it, x, fit, h, eqs.get_ilu0(), feqs.get_ilu0())
    for mode in ("levels", "tiles again"):
        it, x, fit, h, lu, flu = out[mode]
        assert np.array_equal(lu, out["tiles"][4]) and np.array_equal(flu, out["tiles"][5])
        assert it == out["tiles"][0] and fit == out["tiles"][2]
        assert np.array_equal(x, out["tiles"][1]) and np.array_equal(h, out["tiles"][3])


def test_ilu_tiles_only_on_monotone_lattices(gpu):
    """Tiles for Kuhn tets in lattice order; none for 27-point hexes (a
    column left of the diagonal at x + 1) or a renumbered tet mesh."""
    assert gpu.GpuMesh(M.structured_tet(9, 8, 7)).ilu_tiles == 2 * 2 * 1
    assert gpu.GpuMesh(M.structured_hex(9, 8, 7)).ilu_tiles == 0
    assert gpu.GpuMesh(renumber(M.structured_tet(9, 8, 7), 3)[0]).ilu_tiles == 0
