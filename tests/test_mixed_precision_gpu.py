"""FP32-inner CG with FP64 residual replacement against the plain FP64 path:
heads within 1e-8 relative (the precision extension's accuracy bar), FP64
relative residual below the tolerance, on the diagonal-offset FP32 operator
(structured hex and tet patterns) and on the SELL-32 FP32 fallback."""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import rel_max_err, renumber

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-8


def _deck(gpu, m, ek, left=10.0, right=0.0, steady=False):
    # a steady flow system has no storage (the flow assembly keeps M/dt
    # whatever the time type)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=0.0 if steady else 1e-4,
                        steady=1 if steady else 0)
    gm = gpu.GpuMesh(m)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    eqs.GlobalAssembly(p, ek, np.zeros(m.n_nodes))
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), left), np.full(len(rf), right)])
    eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC)
    x0 = np.zeros(m.n_nodes)
    x0[lf] = left
    return eqs, x0


def _both(gpu, eqs, x0, tol=1e-10, precision=None):
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, tol, check_norm_rhs=False)
    x64 = x0.copy()
    it64 = eqs.Solver(x64)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, tol,
                       precision=gpu.PRECISION_FP32_REFINED if precision is None else precision,
                       check_norm_rhs=False)
    x32 = x0.copy()
    it32 = eqs.Solver(x32)
    return x64, it64, x32, it32, eqs.stats()


@pytest.mark.parametrize("kind", ["hex", "tet", "hex_renumbered"])
def test_fp32_refined_matches_fp64(gpu, kind):
    if kind == "tet":
        m = M.structured_tet(14, 10, 8)
        ek = np.repeat(fields.lognormal_k((14, 10, 8), np.log(1e-5), 1.0, 4.0, seed=3), 6)
    else:
        m = M.structured_hex(24, 20, 12)
        ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=3)
    if kind == "hex_renumbered":
        m, _ = renumber(m, 5)
    eqs, x0 = _deck(gpu, m, ek)
    x64, it64, x32, it32, st = _both(gpu, eqs, x0)
    assert st["status"] == gpu.OK and st["rel_residual"] < 1e-10
    assert st["refinements"] >= 2
    assert rel_max_err(x32, x64) < MIXED_RTOL
    # residual replacement keeps the Krylov space: iterations near the FP64
    # count (measured 1.10 x on hex and 1.12 x on tet)
    assert it32 <= 1.2 * it64 + 5


def test_fp32_refined_quad100(gpu):
    """The FP32-inner form on the 100 x 100 quad deck (K=1e-4) to 1e-10."""
    m = M.structured_quad(100, 100)
    ek = np.full(m.n_elements, 1e-4)
    eqs, x0 = _deck(gpu, m, ek, 1.0, 0.0, steady=True)
    x64, it64, x32, it32, st = _both(gpu, eqs, x0)
    assert rel_max_err(x32, x64) < MIXED_RTOL
    assert np.abs(x32 - (1 - m.x / 100)).max() < 1e-8


def test_fp32_refined_rejects_bicgstab(gpu):
    m = M.structured_hex(4, 4, 4)
    eqs, x0 = _deck(gpu, m, np.ones(m.n_elements))
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 100, 1e-10, precision=gpu.PRECISION_FP32_REFINED)
    with pytest.raises(gpu.OgsError) as ei:
        eqs.Solver(x0.copy())
    assert ei.value.status == gpu.BAD_ARG


# hex cells (x, y, z): node counts nx = x + 1 and nxy = nx (y + 1) cover
# every nx mod 4 and every nxy mod 4 the product's window alignments depend on
LATTICES = [(3, 4, 3), (4, 4, 3), (5, 3, 3), (6, 4, 3), (5, 4, 4), (6, 5, 2), (4, 5, 3), (3, 6, 2), (4, 2, 5),
            (24, 20, 12)]


@pytest.mark.parametrize("cells", LATTICES)
def test_lattice_product_bitwise(gpu, cells):
    """The four-rows-per-thread product of the 27-point lattice operator
    (aligned 16-byte windows, zero pads instead of bounds predicates) gives
    bit for bit the row kernel's values, boundary rows included."""
    m = M.structured_hex(*cells)
    nx, nxy = cells[0] + 1, (cells[0] + 1) * (cells[1] + 1)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=3)
    eqs, x0 = _deck(gpu, m, ek)
    _both(gpu, eqs, x0)
    rng = np.random.default_rng(nx * 7 + nxy)
    for x in (rng.standard_normal(m.n_nodes), np.ones(m.n_nodes), -np.arange(m.n_nodes, dtype=float)):
        y_rows, y_lines = eqs.debug_fp32_product(x)
        assert np.abs(y_rows).max() > 0
        # equal values; for non-zero floats that is equal bits
        assert np.array_equal(y_rows, y_lines)


@pytest.mark.parametrize("cells", [(3, 4), (4, 3), (5, 6), (6, 2), (120, 90)])
def test_quad_lattice_product_bitwise(gpu, cells):
    """The same four-rows-per-thread product on the 9-point operator of a
    quad lattice (one line pair): bit for bit the row kernel's values, for
    every nx mod 4."""
    m = M.structured_quad(*cells)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=3)
    eqs, x0 = _deck(gpu, m, ek)
    _both(gpu, eqs, x0)
    rng = np.random.default_rng(cells[0] * 31 + cells[1])
    for x in (rng.standard_normal(m.n_nodes), np.ones(m.n_nodes)):
        y_rows, y_lines = eqs.debug_fp32_product(x)
        assert np.abs(y_rows).max() > 0
        assert np.array_equal(y_rows, y_lines)


def test_lattice_product_needs_lattice_operator(gpu):
    m, _ = renumber(M.structured_hex(8, 6, 4), 5)  # SELL-32 FP32 operator
    eqs, x0 = _deck(gpu, m, np.ones(m.n_elements))
    _both(gpu, eqs, x0)
    with pytest.raises(gpu.OgsError) as ei:
        eqs.debug_fp32_product(np.ones(m.n_nodes))
    assert ei.value.status == gpu.BAD_ARG


def test_lattice_product_solve_matches_row_kernel(gpu, monkeypatch):
    """The solve with the four-rows-per-thread product and with the row
    kernel (OGS_FP32_PRODUCT=rows): the same products, partial sums grouped
    differently, so heads within the solve tolerance of each other and
    iteration counts within a few."""
    m = M.structured_hex(30, 22, 14)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=5)
    eqs, x0 = _deck(gpu, m, ek)
    x64, it64, xl, itl, st = _both(gpu, eqs, x0)
    assert st["status"] == gpu.OK
    monkeypatch.setenv("OGS_FP32_PRODUCT", "rows")
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-10, precision=gpu.PRECISION_FP32_REFINED,
                       check_norm_rhs=False)
    xr = x0.copy()
    itr = eqs.Solver(xr)
    assert eqs.stats()["status"] == gpu.OK
    assert rel_max_err(xl, xr) < MIXED_RTOL and rel_max_err(xl, x64) < MIXED_RTOL
    assert abs(itl - itr) <= max(5, itr // 50)


@pytest.mark.parametrize("mixed,schedule", [(False, 0), (True, 0), (True, 1)])
def test_profile_counts_spmv_launches(gpu, mixed, schedule):
    """ogs_gpu_profile times one SpMV in four iterations of the graph
    schedules, and every launch of the persistent FP32 kernel with the
    iterations it ran."""
    m = M.structured_hex(16, 12, 8)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=1)
    eqs, x0 = _deck(gpu, m, ek)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, 1e-10,
                       precision=gpu.PRECISION_FP32_REFINED if mixed else gpu.PRECISION_FP64,
                       schedule=schedule)
    eqs.profile(True)
    x = x0.copy()
    it = eqs.Solver(x)
    pr = eqs.profile(False)
    assert pr["solves"] == 1
    if mixed and schedule == gpu.SCHEDULE_PERSISTENT:
        # an iteration that asks for a replacement is redone after it
        rep = eqs.stats()["refinements"]
        assert pr["persist_ms"] > 0 and it <= pr["persist_iters"] <= it + rep + 1
        assert pr["spmv_launches"] == 0
    else:
        assert pr["spmv_ms"] > 0 and pr["persist_iters"] == 0
        assert abs(pr["spmv_launches"] - it / 4) <= it / 16 + 3


@pytest.mark.parametrize("kind", ["hex", "tet", "hex_renumbered", "quad"])
def test_fp32_schedules_agree(gpu, kind):
    """The persistent cooperative kernel (preconditioned form) and the graph
    schedule (CG on the Jacobi-scaled system) run the same recurrence in
    exact arithmetic: heads within the FP32 bar of each other and of FP64;
    iteration counts near FP64 CG's and within one replacement cycle of
    each other (the last FP64 check can fall on either side of the
    tolerance)."""
    if kind == "tet":
        m = M.structured_tet(14, 10, 8)
        ek = np.repeat(fields.lognormal_k((14, 10, 8), np.log(1e-5), 1.0, 4.0, seed=5), 6)
    elif kind == "quad":
        m = M.structured_quad(120, 90)
        ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 6.0, seed=5)
    else:
        m = M.structured_hex(30, 22, 14)
        ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=5)
    if kind == "hex_renumbered":
        m, _ = renumber(m, 7)  # SELL-32 FP32 operator
    eqs, x0 = _deck(gpu, m, ek)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-10, check_norm_rhs=False)
    x64 = x0.copy()
    it64 = eqs.Solver(x64)
    out = {}
    for sch in (gpu.SCHEDULE_GRAPH, gpu.SCHEDULE_PERSISTENT):
        eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-10, precision=gpu.PRECISION_FP32_REFINED,
                           check_norm_rhs=False, schedule=sch)
        x = x0.copy()
        it = eqs.Solver(x)
        st = eqs.stats()
        assert st["status"] == gpu.OK and st["rel_residual"] < 1e-10
        assert rel_max_err(x, x64) < MIXED_RTOL
        assert it <= 1.3 * it64 + 5
        out[sch] = (x, it)
    (xg, itg), (xp, itp) = out[gpu.SCHEDULE_GRAPH], out[gpu.SCHEDULE_PERSISTENT]
    assert rel_max_err(xp, xg) < MIXED_RTOL
    assert abs(itp - itg) <= max(10, itg // 5)


def test_schedule_rejects_unknown(gpu):
    m = M.structured_hex(4, 4, 4)
    eqs, _ = _deck(gpu, m, np.ones(m.n_elements))
    with pytest.raises(gpu.OgsError):
        eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 100, 1e-10, precision=gpu.PRECISION_FP32_REFINED,
                           schedule=7)


def test_fp32_stall_falls_back_to_fp64(gpu):
    """Steady heterogeneous 375 x 375 quads: the FP32 recurrence stalls
    (cond(A) near 1/eps_fp32 for the Jacobi-scaled operator); the solve
    detects the stalled cycle, finishes in FP64 CG from the accumulated x64
    and still meets the tolerance and the FP64 path's heads."""
    m = M.structured_quad(375, 375)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 8.0, seed=3)
    eqs, x0 = _deck(gpu, m, ek, steady=True)
    x64, it64, x32, it32, st = _both(gpu, eqs, x0)
    assert st["status"] == gpu.OK and st["rel_residual"] < 1e-10
    assert st["fp64_fallback"] == 1
    assert rel_max_err(x32, x64) < MIXED_RTOL


def test_fp32_no_fallback_when_cycles_gain(gpu):
    """Transient hex deck: every FP32 cycle gains about 1/delta, no fallback."""
    m = M.structured_hex(24, 20, 12)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=6)
    eqs, x0 = _deck(gpu, m, ek)
    x64, it64, x32, it32, st = _both(gpu, eqs, x0)
    assert st["status"] == gpu.OK and st["fp64_fallback"] == 0
    assert rel_max_err(x32, x64) < MIXED_RTOL


def _solve_pair(gpu, eqs, x0, tol=1e-10):
    x64, _, x32, _, st = _both(gpu, eqs, x0, tol, precision=gpu.PRECISION_FP32_CELLS)
    assert st["status"] == gpu.OK and st["rel_residual"] < tol
    assert rel_max_err(x32, x64) < MIXED_RTOL
    return st


def _hex_system(gpu, m, ek, params, mode, repeat=1, reassemble_after_bc=False, gauss=3):
    eqs = gpu.LinearEQS(gpu.GpuMesh(m, gauss_points=gauss))
    eqs.Initialize()
    for _ in range(repeat):
        eqs.GlobalAssembly(params, ek, np.zeros(m.n_nodes))
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.full(len(rf), 2.0)])
    eqs.SetKnownX(rows, vals, mode)
    if reassemble_after_bc:
        eqs.GlobalAssembly(params, ek, np.zeros(m.n_nodes))
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    return eqs, x0


@pytest.mark.parametrize("case", ["symmetric", "row_only", "twice", "liquid_gravity", "steady", "spacing"])
def test_cell_coefficient_operator(gpu, case):
    """PRECISION_FP32_CELLS on a regular hex lattice: the FP32 inner CG
    applies the operator from one coefficient per cell (fp32_operator 2);
    heads within 1e-8 of the FP64 path for symmetric and row-only Dirichlet
    sets, two assemblies summed, LIQUID_FLOW with gravity, steady flow and
    anisotropic spacing.  PRECISION_FP32_REFINED keeps the stored diagonal
    operator (fp32_operator 0) on the same system."""
    m = M.structured_hex(30, 22, 14, *((2.0, 0.5, 0.75) if case == "spacing" else (1.0, 1.0, 1.0)))
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=9)
    if case == "liquid_gravity":
        p = gpu.make_params(gpu.LIQUID_FLOW, dt=3600.0, storage=1e-4, porosity=0.2, drho_dp=1e-7,
                            viscosity=1e-3, density=1000.0, gravity=9.81, gravity_on=1)
        ek = ek * 1e-7
    else:
        p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=0.0 if case == "steady" else 1e-4,
                            steady=1 if case == "steady" else 0)
    mode = gpu.DIRICHLET_ROW_ONLY if case == "row_only" else gpu.DIRICHLET_SYMMETRIC
    eqs, x0 = _hex_system(gpu, m, ek, p, mode, repeat=2 if case == "twice" else 1)
    st = _solve_pair(gpu, eqs, x0)
    assert st["fp32_operator"] == 2
    # the stored FP32 operator: upper-half diagonal offsets for symmetric
    # matrices, SELL-32 once row-only Dirichlet rows break the symmetry
    x64, _, x32, _, st = _both(gpu, eqs, x0)
    assert st["fp32_operator"] == (1 if case == "row_only" else 0)
    assert rel_max_err(x32, x64) < MIXED_RTOL


@pytest.mark.parametrize("case", ["lumping", "one_gauss_point", "reassembled_after_bc", "stretched"])
def test_cell_coefficient_operator_falls_back(gpu, case):
    """Matrices without the cell-coefficient form keep the stored FP32
    operator: mass lumping, one Gauss point (under-integrated Laplace), an
    assembly added after the Dirichlet elimination (caught by the check of
    the FP32 operator against the FP64 matrix), a non-uniform lattice."""
    if case == "stretched":
        m = M.structured_hex(20, 12, 8)
        m.x = m.x ** 1.1  # graded in x
    else:
        m = M.structured_hex(20, 12, 8)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=2)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4, mass_lumping=1 if case == "lumping" else 0)
    eqs, x0 = _hex_system(gpu, m, ek, p, gpu.DIRICHLET_SYMMETRIC,
                          reassemble_after_bc=case == "reassembled_after_bc",
                          gauss=1 if case == "one_gauss_point" else 3)
    x64, _, x32, _, st = _both(gpu, eqs, x0, precision=gpu.PRECISION_FP32_CELLS)
    assert st["status"] == gpu.OK and st["fp32_operator"] == 0 and st["rel_residual"] < 1e-10
    if case != "one_gauss_point":  # hourglass modes: heads as ill-conditioned as the system
        assert rel_max_err(x32, x64) < MIXED_RTOL
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-10, check_norm_rhs=False)
    eqs.Solver(x0.copy())
    assert eqs.stats()["fp32_operator"] == -1
