"""RICHARDS_FLOW on the GPU (ogs_gpu_assemble_richards, ogs_gpu_richards_step)
against the oracle: the assembled system at a partly unsaturated iterate
within 1e-12 per entry, and a Picard time step with the same number of
iterations and the same heads (1e-10 relative, the linear solves stopping at
1e-13)."""
import numpy as np
import pytest

from ogs5_gb300 import mesh as M
from tests.helpers import SOLUTION_RTOL, assert_matrix_close, assert_vector_close, distort, rel_max_err

pytestmark = pytest.mark.gpu

RHO_G = 1000.0 * 9.81
LINEAR_TOL = 1e-13  # linear solves inside the Picard loops, GPU and oracle


def _mesh(kind):
    if kind == "quad":
        return M.structured_quad(10, 14, 0.2, 0.1)
    if kind == "hex":
        return distort(M.structured_hex(4, 3, 8, 0.5, 0.5, 0.25), 0.1, seed=3)
    if kind == "hex_box":  # axis-aligned boxes: the constant-geometry path
        return M.structured_hex(4, 3, 8, 0.5, 0.5, 0.25)
    return M.structured_tet(3, 3, 5, 0.5, 0.5, 0.3)


def _params(gpu, oracle, **kw):
    base = dict(dt=600.0, storage=1e-6, porosity=0.35, drho_dp=4.4e-10, viscosity=1e-3, density=1000.0,
                time_unit_factor=1.0)
    base.update(kw)
    return (gpu.make_params(gpu.RICHARDS_FLOW, **base), oracle.make_params(pcs_type=3, **base))


def _curves(gpu, oracle, model):
    kw = dict(capillary_model=model, permeability_model=model, pb=5.0e3, slr=0.08, slm=0.98,
              m=0.55 if model == 4 else 1.8, kr_slr=0.08, kr_slm=0.98, kr_m=0.55 if model == 4 else 1.8, kr_min=1e-9)
    return gpu.richards_params(**kw), oracle.richards_params(**kw)


def _pressure(m, seed):
    """hydrostatic-ish profile: saturated below a water table, suction above"""
    rng = np.random.default_rng(seed)
    top = m.z.max() if m.dim == 3 else m.y.max()
    h = (m.z if m.dim == 3 else m.y)
    return RHO_G * (0.4 * top - h) * 4.0 + rng.normal(0.0, 500.0, m.n_nodes)


@pytest.mark.parametrize("kind", ["quad", "hex", "hex_box", "tet"])
@pytest.mark.parametrize("opts", [(4, 0, 0), (4, 1, 1), (6, 1, 0), (6, 0, 1)])
def test_richards_assembly_matches_oracle(gpu, oracle, kind, opts):
    model, gravity, lumping = opts
    m = _mesh(kind)
    rng = np.random.default_rng(7)
    ek = np.exp(np.log(1e-12) + 0.5 * rng.standard_normal(m.n_elements))
    gp, op = _params(gpu, oracle, gravity=9.81 if gravity else 0.0, gravity_on=gravity, mass_lumping=lumping)
    gr, orr = _curves(gpu, oracle, model)
    p_old = _pressure(m, 1)
    p_it = _pressure(m, 2)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.Initialize()
    eqs.AssembleRichards(gp, gr, ek, p_old, p_it)
    rp, col, val = eqs.get_csr()
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    oval, ob = oracle.assemble_richards(m, orp, ocol, op, orr, ek, p_old, p_it)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(eqs.get_rhs(), ob)
    assert (p_it < 0).any() and (p_it > 0).any()  # both branches of CalCoefMass


@pytest.mark.parametrize("kind,method", [("quad", 2), ("hex", 4), ("tet", 1)])
def test_richards_picard_step_matches_oracle(gpu, oracle, kind, method):
    """Infiltration into a dry column: top pressure 0 (saturated), bottom
    held at its suction; one Picard step of dt = 60 s from the dry state."""
    m = _mesh(kind)
    rng = np.random.default_rng(11)
    ek = np.exp(np.log(5e-12) + 0.3 * rng.standard_normal(m.n_elements))
    gp, op = _params(gpu, oracle, dt=60.0, gravity=9.81, gravity_on=1)
    gr, orr = _curves(gpu, oracle, 4)
    vert = m.z if m.dim == 3 else m.y
    p_old = np.full(m.n_nodes, -1.0e4)
    top = np.flatnonzero(vert == vert.max())
    bottom = np.flatnonzero(vert == vert.min())
    rows = np.concatenate([top, bottom])
    vals = np.concatenate([np.zeros(len(top)), np.full(len(bottom), -1.0e4)])
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, LINEAR_TOL, check_norm_rhs=False)
    it = p_old.copy()
    st = eqs.RichardsStep(gp, gr, ek, p_old, it, rows, vals, gpu.DIRICHLET_SYMMETRIC, error_method=method,
                          max_iterations=30, tolerance=1e-3 if method == 4 else 1.0)
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    oit, info = oracle.richards_picard(m, orp, ocol, op, orr, ek, p_old, p_old, rows, vals, True,
                                       error_method=method, tolerance=1e-3 if method == 4 else 1.0,
                                       max_iterations=30, method=5, precond=1, tol=LINEAR_TOL)
    assert st["converged"] and info["converged"]
    assert st["iterations"] == info["iterations"] and st["iterations"] >= 3
    assert rel_max_err(it, oit) < SOLUTION_RTOL
    # the wetting front: pressures rose from the dry state, top held at 0
    assert np.all(it[top] == 0.0) and it.max() <= 1e-6 and np.mean(it) > -1.0e4


def test_richards_relaxation_and_stagnation(gpu, oracle):
    """nls_relaxation 0.5: relax0 / relax1 weigh the Laplace term and the
    iterate moves half way (theta 0.5), as in the oracle (converges in the
    same number of iterations); from a drier state with a longer step the
    error stops falling by 1 % twice in a row: stagnation, NOT_CONVERGED,
    after the same iterations as the oracle."""
    m = _mesh("quad")
    ek = np.full(m.n_elements, 5e-12)
    gr, orr = _curves(gpu, oracle, 4)
    top = np.flatnonzero(m.y == m.y.max())
    vals = np.zeros(len(top))
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, LINEAR_TOL, check_norm_rhs=False)
    for dt, dry, ok in ((10.0, -5.0e3, True), (60.0, -2.0e4, False)):
        gp, op = _params(gpu, oracle, dt=dt, gravity=9.81, gravity_on=1, nls_relaxation=0.5)
        p_old = np.full(m.n_nodes, dry)
        it = p_old.copy()
        st = eqs.RichardsStep(gp, gr, ek, p_old, it, top, vals, gpu.DIRICHLET_SYMMETRIC, error_method=2,
                              max_iterations=40, tolerance=1.0, allow_fail=True)
        oit, info = oracle.richards_picard(m, orp, ocol, op, orr, ek, p_old, p_old, top, vals, True, error_method=2,
                                           tolerance=1.0, max_iterations=40, tol=LINEAR_TOL)
        assert st["iterations"] == info["iterations"]
        assert st["converged"] == info["converged"] == ok and st["diverged"] == info["diverged"] == (not ok)
        assert st["status"] == (gpu.OK if ok else gpu.NOT_CONVERGED)
        if ok:
            assert rel_max_err(it, oit) < SOLUTION_RTOL


def test_richards_rejects_bad_input(gpu):
    m = _mesh("quad")
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    p = gpu.make_params(gpu.RICHARDS_FLOW, dt=1.0, viscosity=1e-3)
    z = np.zeros(m.n_nodes)
    with pytest.raises(gpu.OgsError):
        eqs.AssembleRichards(p, gpu.richards_params(capillary_model=5), np.ones(m.n_elements), z, z)
    with pytest.raises(gpu.OgsError):
        eqs.AssembleRichards(p, gpu.richards_params(m=1.5), np.ones(m.n_elements), z, z)
    with pytest.raises(gpu.OgsError):  # RICHARDS_FLOW is not an ogs_gpu_assemble process
        eqs.GlobalAssembly(p, np.ones(m.n_elements), z)
