"""Parity of the CUDA path (through the C ABI) against the CPU oracle.

Assembly: every entry of A and b within 1e-12 relative (floor 1e-14 x row
max), for quad/hex/tet x GROUNDWATER_FLOW/LIQUID_FLOW/MASS_TRANSPORT, on
affine meshes (affine kernels) and distorted meshes (per-Gauss-point
kernels).  Solves: converged heads within 1e-10 relative of the oracle's
Linear_EQS iteration on the same system and initial guess.
"""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import (SOLUTION_RTOL, assert_matrix_close, assert_vector_close, distort,
                           rel_max_err)

pytestmark = pytest.mark.gpu


def small_mesh(kind):
    if kind == "quad":
        return M.structured_quad(12, 9, 1.0, 0.5)
    if kind == "hex":
        return M.structured_hex(6, 5, 4, 1.0, 2.0, 0.5)
    return M.structured_tet(4, 3, 3, 1.0, 1.5, 0.75)


def k_field(m, seed=1):
    rng = np.random.default_rng(seed)
    return np.exp(np.log(1e-5) + rng.standard_normal(m.n_elements))


def oracle_params(O, gp, **over):
    """oracle AssemblyParams with the same values as a capi AssemblyParams"""
    names = [f[0] for f in gp._fields_]
    return O.make_params(**{n: getattr(gp, n) for n in names if n != "pad0"})


def run_assembly(gpu, oracle, m, params, ek=None, u0=None, gpv=None, ngauss=3):
    gm = gpu.GpuMesh(m, gauss_points=ngauss)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    eqs.GlobalAssembly(params, ek, u0, gpv)
    rp, col, val = eqs.get_csr()
    b = eqs.get_rhs()
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol), "CSR pattern differs"
    oval, ob = oracle.assemble(m, orp, ocol, oracle_params(oracle, params), elem_k=ek, u0=u0,
                               gp_vel=gpv, ngauss=ngauss)
    return eqs, gm, (rp, col, val, b), (oval, ob)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("distorted", [False, True])
@pytest.mark.parametrize("ngauss", [2, 3])
def test_assembly_groundwater_flow(gpu, oracle, kind, distorted, ngauss):
    if kind == "tet" and ngauss == 2:
        pytest.skip("tets always use the 5-point rule")
    m = small_mesh(kind)
    if distorted:
        m = distort(m, 0.2, seed=3)
    ek = k_field(m)
    rng = np.random.default_rng(7)
    u0 = rng.uniform(0, 10, m.n_nodes)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4)
    eqs, gm, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, ek, u0, ngauss=ngauss)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)


def sheared(m):
    """The mesh under one linear map of its coordinates: every element stays
    affine (a parallelepiped / parallelogram) but none is an axis-aligned box,
    so the affine kernels take their full-tensor branch."""
    import copy
    s = copy.copy(m)
    x, y = m.x.astype(float), m.y.astype(float)
    z = m.z.astype(float) if m.dim == 3 else np.zeros_like(x)
    s.x = x + 0.31 * y + 0.17 * z
    s.y = 0.93 * y + 0.22 * z - 0.12 * x
    if m.dim == 3:
        s.z = 1.07 * z + 0.05 * x
    return s


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("pcs", ["gwf", "liquid", "transport"])
def test_assembly_sheared_affine(gpu, oracle, kind, pcs):
    """Affine, non-box elements through the affine kernels: entries within
    1e-12 of the oracle for each process."""
    m = sheared(small_mesh(kind))
    rng = np.random.default_rng(21)
    u0 = rng.uniform(0, 10, m.n_nodes)
    if pcs == "transport":
        ngp = {"quad": 9, "hex": 27, "tet": 5}[kind]
        gpv = rng.normal(0, 1e-5, (m.n_elements, ngp, 3))
        if m.dim == 2:
            gpv[:, :, 2] = 0.0
        p = gpu.make_params(gpu.MASS_TRANSPORT, dt=3600.0, theta=0.6, porosity=0.3,
                            alpha_l=1.0, alpha_t=0.1, diffusion=1e-9, decay=1e-7, retardation=1.5)
        _, _, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, None, u0, gpv)
    elif pcs == "liquid":
        p = gpu.make_params(gpu.LIQUID_FLOW, dt=100.0, storage=1e-9, porosity=0.3, drho_dp=4.5e-10,
                            viscosity=1e-3, density=1000.0, gravity=9.81, gravity_on=1)
        _, _, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, k_field(m, 4) * 1e-7, u0)
    else:
        p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4, mass_lumping=1)
        _, _, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, k_field(m, 5), u0)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
def test_assembly_groundwater_relaxation_and_steady(gpu, oracle, kind):
    m = small_mesh(kind)
    ek = k_field(m, 2)
    u0 = np.random.default_rng(1).uniform(0, 1, m.n_nodes)
    for kw in ({"nls_relaxation": 0.6, "storage": 2e-4, "dt": 10.0},
               {"steady": 1, "storage": 1e-4, "dt": 1.0}):
        p = gpu.make_params(gpu.GROUNDWATER_FLOW, **kw)
        _, _, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, ek, u0)
        assert_matrix_close(rp, val, oval)
        assert_vector_close(b, ob)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("distorted", [False, True])
def test_assembly_liquid_flow_gravity(gpu, oracle, kind, distorted):
    m = small_mesh(kind)
    if distorted:
        m = distort(m, 0.15, seed=5)
    ek = k_field(m, 3) * 1e-7  # permeability
    u0 = np.random.default_rng(2).uniform(1e5, 2e5, m.n_nodes)
    p = gpu.make_params(gpu.LIQUID_FLOW, dt=100.0, storage=1e-9, porosity=0.3, drho_dp=4.5e-10,
                        viscosity=1e-3, density=1000.0, gravity=9.81, gravity_on=1)
    _, _, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, ek, u0)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("distorted", [False, True])
@pytest.mark.parametrize("flux", ["per_point", "per_element"])
def test_assembly_mass_transport(gpu, oracle, kind, distorted, flux):
    """per_element: every Gauss point of an element carries the same flux
    (what Cal_Velocity gives on affine tets), on every other element; the
    tet kernel then forms the dispersion tensor once per element."""
    m = small_mesh(kind)
    if distorted:
        m = distort(m, 0.15, seed=9)
    ngp = {"quad": 9, "hex": 27, "tet": 5}[kind]
    rng = np.random.default_rng(11)
    gpv = rng.normal(0, 1e-5, (m.n_elements, ngp, 3))
    if flux == "per_element":
        gpv[::2] = gpv[::2, :1, :]
    if m.dim == 2:
        gpv[:, :, 2] = 0.0
    gpv[0, :, :] = 0.0  # zero-velocity branch of the dispersion tensor
    c0 = rng.uniform(0, 1, m.n_nodes)
    p = gpu.make_params(gpu.MASS_TRANSPORT, dt=3600.0, theta=0.6, porosity=0.3,
                        alpha_l=1.0, alpha_t=0.1, diffusion=1e-9, decay=1e-7, retardation=1.5)
    _, _, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, None, c0, gpv)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("distorted", [False, True])
@pytest.mark.parametrize("pcs", ["flow", "transport"])
def test_assembly_mass_lumping(gpu, oracle, kind, distorted, pcs):
    """ele_mass_lumping on the affine and per-Gauss-point kernels, flow and
    transport: every entry within 1e-12 of the oracle's CalcLumpedMass."""
    m = small_mesh(kind)
    if distorted:
        m = distort(m, 0.2, seed=5)
    rng = np.random.default_rng(21)
    u0 = rng.uniform(0, 1, m.n_nodes)
    if pcs == "flow":
        p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=600.0, storage=1e-3, mass_lumping=1)
        out = run_assembly(gpu, oracle, m, p, k_field(m, 6), u0)
    else:
        ngp = {"quad": 9, "hex": 27, "tet": 5}[kind]
        gpv = rng.normal(0, 1e-5, (m.n_elements, ngp, 3))
        if m.dim == 2:
            gpv[:, :, 2] = 0.0
        p = gpu.make_params(gpu.MASS_TRANSPORT, dt=600.0, theta=0.7, porosity=0.3, alpha_l=1.0,
                            alpha_t=0.1, diffusion=1e-9, decay=1e-7, retardation=1.5, mass_lumping=1)
        out = run_assembly(gpu, oracle, m, p, None, u0, gpv)
    _, _, (rp, col, val, b), (oval, ob) = out
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("opts", [{}, {"mass_lumping": 1}, {"supg_method": 1}])
def test_transport_stored_operators(gpu, oracle, kind, opts):
    """$MEMORY_TYPE 1 (fem_ele_std.cpp:8534-8588): the first assembly stores
    the operators; a later one with another dt, theta, u0 and velocity field
    combines the stored ones -- the oracle's assembly with the first
    velocities and the later dt, theta, u0 -- also without gp_velocity; after
    ResetOperators the new velocities are taken."""
    m = distort(small_mesh(kind), 0.15, seed=4) if kind != "tet" else small_mesh(kind)
    ngp = {"quad": 9, "hex": 27, "tet": 5}[kind]
    rng = np.random.default_rng(31)
    gpv1, gpv2 = rng.normal(0, 1e-5, (2, m.n_elements, ngp, 3))
    if m.dim == 2:
        gpv1[:, :, 2] = gpv2[:, :, 2] = 0.0
    c1, c2 = rng.uniform(0, 1, (2, m.n_nodes))
    base = dict(porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=1e-9, decay=1e-7, retardation=1.5, **opts)
    p1 = gpu.make_params(gpu.MASS_TRANSPORT, dt=600.0, theta=0.7, memory_type=1, **base)
    p2 = gpu.make_params(gpu.MASS_TRANSPORT, dt=1800.0, theta=0.55, memory_type=1, **base)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)

    def check(p, c, gpv_gpu, gpv_oracle):
        eqs.Initialize()
        eqs.GlobalAssembly(p, None, c, gpv_gpu)
        rp, _, val = eqs.get_csr()
        oval, ob = oracle.assemble(m, orp, ocol, oracle_params(oracle, p), u0=c, gp_vel=gpv_oracle)
        assert_matrix_close(rp, val, oval)
        assert_vector_close(eqs.get_rhs(), ob)

    check(p1, c1, gpv1, gpv1)
    check(p2, c2, gpv2, gpv1)
    check(p2, c2, None, gpv1)
    eqs.ResetOperators()
    check(p2, c2, gpv2, gpv2)
    with pytest.raises(gpu.OgsError):
        eqs.ResetOperators()
        eqs.GlobalAssembly(p2, None, c2, None)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("opts", [(1, 0, 0), (2, 1, 1), (2, 2, 2), (1, 2, 0)])
def test_assembly_supg(gpu, oracle, kind, opts):
    """ele_supg_method / _length / _diffusivity on transport: the SUPG mass
    and advection terms on distorted meshes, every entry within 1e-12 of the
    oracle (also through the affine-tet dispatch, which SUPG bypasses)."""
    method, length, diffusivity = opts
    m = distort(small_mesh(kind), 0.15, seed=8) if kind != "tet" else small_mesh(kind)
    ngp = {"quad": 9, "hex": 27, "tet": 5}[kind]
    rng = np.random.default_rng(23)
    gpv = rng.normal(0, 1e-5, (m.n_elements, ngp, 3))
    if m.dim == 2:
        gpv[:, :, 2] = 0.0
    gpv[1, :, :] = 0.0  # tau = 0 branch
    c0 = rng.uniform(0, 1, m.n_nodes)
    p = gpu.make_params(gpu.MASS_TRANSPORT, dt=600.0, theta=0.8, porosity=0.3, alpha_l=1.0, alpha_t=0.1,
                        diffusion=1e-9, decay=1e-7, retardation=1.5, supg_method=method,
                        supg_length=length, supg_diffusivity=diffusivity)
    _, _, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, None, c0, gpv)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)


@pytest.mark.parametrize("kind", ["quad", "hex", "tet"])
@pytest.mark.parametrize("distorted", [False, True])
def test_gp_velocity(gpu, oracle, kind, distorted):
    m = small_mesh(kind)
    if distorted:
        m = distort(m, 0.2, seed=4)
    ek = k_field(m, 4)
    h = np.random.default_rng(3).uniform(0, 10, m.n_nodes)
    for pcs, kw in ((gpu.GROUNDWATER_FLOW, {}),
                    (gpu.LIQUID_FLOW, {"gravity": 9.81, "gravity_on": 1, "viscosity": 1e-3})):
        p = gpu.make_params(pcs, **kw)
        gm = gpu.GpuMesh(m)
        eqs = gpu.LinearEQS(gm)
        q = eqs.gp_velocity(p, ek, h)
        qo = oracle.gp_velocity(m, oracle_params(oracle, p), ek, h)
        assert_vector_close(q.ravel(), qo.ravel())


@pytest.mark.parametrize("symmetric", [False, True])
def test_dirichlet(gpu, oracle, symmetric):
    m = M.structured_hex(7, 5, 4)
    ek = k_field(m, 5)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4)
    u0 = np.zeros(m.n_nodes)
    eqs, gm, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, ek, u0)
    rows = np.concatenate([m.face_nodes(0, 0), m.face_nodes(0, 1), m.face_nodes(2, 0)[:7]])
    rows = np.concatenate([rows, rows[:3]])  # duplicates, as repeated SetKnownX_i calls
    vals = np.concatenate([np.full(len(m.face_nodes(0, 0)), 10.0),
                           np.zeros(len(m.face_nodes(0, 1))), np.linspace(1, 2, 7)])
    vals = np.concatenate([vals, vals[:3]])
    eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC if symmetric else gpu.DIRICHLET_ROW_ONLY)
    val2 = eqs.get_values()
    b2 = eqs.get_rhs()
    oracle.dirichlet(rp, col, oval, ob, rows, vals, symmetric=symmetric)
    assert_matrix_close(rp, val2, oval)
    assert_vector_close(b2, ob)


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_dirichlet_sets_in_sequence(gpu, oracle, kind):
    """One system re-assembled and given Dirichlet sets in turn: the same set
    again (kept on the device), a different set (rows and values), the first
    set again; every time the matrix and b of the oracle's elimination."""
    m = M.structured_hex(9, 6, 5) if kind == "hex" else M.structured_tet(6, 5, 4)
    ek = k_field(m, 5)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4)
    u0 = np.random.default_rng(2).uniform(0, 1, m.n_nodes)
    lf, rf, bf = m.face_nodes(0, 0), m.face_nodes(0, 1), m.face_nodes(2, 0)
    set_a = (np.concatenate([lf, rf]), np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))]))
    set_b = (np.concatenate([lf, bf]), np.concatenate([np.full(len(lf), 4.0), np.linspace(1, 2, len(bf))]))
    set_c = (set_a[0], np.concatenate([np.full(len(lf), 9.0), np.zeros(len(rf))]))
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    for rows, vals in (set_a, set_a, set_b, set_c, set_a):
        eqs.Initialize()
        eqs.GlobalAssembly(p, ek, u0)
        eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC)
        oval, ob = oracle.assemble(m, orp, ocol, oracle_params(oracle, p), elem_k=ek, u0=u0)
        oracle.dirichlet(orp, ocol, oval, ob, rows, vals, symmetric=True)
        assert_matrix_close(orp, eqs.get_values(), oval)
        assert_vector_close(eqs.get_rhs(), ob)


def test_lattice_assembly_adds_to_what_is_there(gpu, oracle):
    """On a hex lattice the flow assembly runs row by row and stores right
    after Initialize; a second GlobalAssembly adds to the first (A and b
    twice the oracle's), as the element kernels do."""
    m = M.structured_hex(9, 7, 5)
    ek = k_field(m, 3)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4)
    u0 = np.random.default_rng(5).uniform(0, 1, m.n_nodes)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.Initialize()
    eqs.GlobalAssembly(p, ek, u0)
    eqs.GlobalAssembly(p, ek, u0)
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    oval, ob = oracle.assemble(m, orp, ocol, oracle_params(oracle, p), elem_k=ek, u0=u0)
    assert_matrix_close(orp, eqs.get_values(), 2.0 * oval)
    assert_vector_close(eqs.get_rhs(), 2.0 * ob)


def test_spmv(gpu, oracle):
    m = M.structured_tet(5, 4, 3)
    ek = k_field(m, 6)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=1.0, storage=1e-3)
    eqs, gm, (rp, col, val, b), (oval, ob) = run_assembly(gpu, oracle, m, p, ek, np.zeros(m.n_nodes))
    x = np.random.default_rng(0).standard_normal(m.n_nodes)
    y = eqs.spmv(x)
    yo = oracle.spmv(rp, col, val, x)
    assert_vector_close(y, yo, rtol=1e-12, scale=np.abs(val).max() * np.abs(x).max())


def _flow_system(gpu, oracle, m, ek, symmetric, dt=None, storage=0.0, left=1.0, right=0.0):
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=dt or 1.0, storage=storage, steady=0 if dt else 1)
    gm = gpu.GpuMesh(m)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    u0 = np.zeros(m.n_nodes)
    eqs.GlobalAssembly(p, ek, u0)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), left), np.full(len(rf), right)])
    eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC if symmetric else gpu.DIRICHLET_ROW_ONLY)
    rp, col, val = eqs.get_csr()
    b = eqs.get_rhs()
    x0 = np.full(m.n_nodes, 0.5 * (left + right))
    x0[lf] = left
    x0[rf] = right
    return eqs, (rp, col, val, b), x0


def test_quad100_bicgstab_jacobi_linear_profile(gpu, oracle):
    """The 100 x 100 quad deck: K=1e-4, h=1|0 on the x faces, BiCGStab+Jacobi.

    At the deck's tolerance 1e-10 both codes stop on |r|/|b| < 1e-10 within
    two iterations of each other; their heads then differ by up to
    cond(A) x 1e-10 (about 3e-9 here), so head parity is checked on the same
    system solved to 1e-13, where both iterations have converged."""
    m = M.structured_quad(100, 100)
    ek = np.full(m.n_elements, 1e-4)
    eqs, (rp, col, val, b), x0 = _flow_system(gpu, oracle, m, ek, symmetric=False)
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 1000, 1e-10)
    x = x0.copy()
    it = eqs.Solver(x)
    xo, info = oracle.solve(rp, col, val, b, x0, method=2, precond=1, max_iter=1000, tol=1e-10)
    assert abs(it - info["iterations"]) <= 2
    assert eqs.stats()["rel_residual"] < 1e-10
    assert np.abs(x - (1.0 - m.x / 100.0)).max() < 1e-8  # exact bilinear solution
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 2000, 1e-13, check_norm_rhs=False)
    x = x0.copy()
    eqs.Solver(x)
    xo, info = oracle.solve(rp, col, val, b, x0, method=2, precond=1, max_iter=2000, tol=1e-13)
    assert rel_max_err(x, xo) < SOLUTION_RTOL


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_cg_jacobi_heterogeneous(gpu, oracle, kind):
    m = M.structured_hex(16, 12, 8) if kind == "hex" else M.structured_tet(10, 8, 6)
    nh = (m.shape[0] * m.shape[1] * m.shape[2])
    kh = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 3.0, seed=2)
    ek = kh if kind == "hex" else np.repeat(kh, 6)
    assert len(ek) == m.n_elements and nh > 0
    eqs, (rp, col, val, b), x0 = _flow_system(gpu, oracle, m, ek, symmetric=True, dt=3600.0,
                                              storage=1e-4, left=10.0, right=0.0)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, 1e-13)
    x = x0.copy()
    it = eqs.Solver(x)
    xo, info = oracle.solve(rp, col, val, b, x0, method=5, precond=1, max_iter=5000, tol=1e-13)
    assert abs(it - info["iterations"]) <= max(2, info["iterations"] // 50)
    assert rel_max_err(x, xo) < SOLUTION_RTOL


@pytest.mark.parametrize("precond", [0, 1])
def test_bicgstab_matches_oracle_iterates(gpu, oracle, precond):
    m = M.structured_hex(10, 8, 6)
    ek = k_field(m, 8)
    eqs, (rp, col, val, b), x0 = _flow_system(gpu, oracle, m, ek, symmetric=False, dt=100.0,
                                              storage=1e-3, left=3.0, right=1.0)
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, precond, 2000, 1e-12)
    x = x0.copy()
    it = eqs.Solver(x)
    xo, info = oracle.solve(rp, col, val, b, x0, method=2, precond=precond, max_iter=2000, tol=1e-12)
    # unpreconditioned BiCGStab near the attainable accuracy reacts to the
    # summation order of its dot products; the heads are the parity bar
    slack = 2 if precond else max(2, info["iterations"] // 10)
    assert abs(it - info["iterations"]) <= slack
    assert rel_max_err(x, xo) < SOLUTION_RTOL


def test_check_norm_rhs_and_max_iter_status(gpu, oracle):
    """CheckNormRHS: a second solve whose |b| dropped below tol*|b_prev| returns
    at once; max_iter=1 reports NOT_CONVERGED (host-side fault injection)."""
    m = M.structured_quad(20, 20)
    ek = np.full(m.n_elements, 1e-4)
    eqs, (rp, col, val, b), x0 = _flow_system(gpu, oracle, m, ek, symmetric=False)
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 1, 1e-10)
    x = x0.copy()
    eqs.Solver(x, allow_fail=True)
    assert eqs.stats()["status"] == gpu.NOT_CONVERGED
    # second solve, b scaled by 1e-12: |b|/|b_prev| < tol -> immediate return
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 1000, 1e-10)
    eqs.Initialize()
    eqs.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, steady=1), ek * 1e-12, np.zeros(m.n_nodes))
    lf = m.face_nodes(0, 0)
    eqs.SetKnownX(lf, np.full(len(lf), 1.0))
    x2 = np.zeros(m.n_nodes)
    it = eqs.Solver(x2)
    assert it == 0 and eqs.stats()["status"] == gpu.OK


def test_error_statuses(gpu):
    m = M.structured_hex(3, 3, 3)
    # degenerate element -> SINGULAR_JACOBIAN, not a trap
    bad = M.structured_hex(3, 3, 3)
    bad.x = bad.x.copy()
    e0 = bad.conn[0]
    bad.x[e0] = bad.x[e0[0]]
    bad.y = bad.y.copy()
    bad.y[e0] = bad.y[e0[0]]
    bad.z = bad.z.copy()
    bad.z[e0] = bad.z[e0[0]]
    gm = gpu.GpuMesh(bad)
    eqs = gpu.LinearEQS(gm)
    with pytest.raises(gpu.OgsError) as ei:
        eqs.GlobalAssembly(gpu.make_params(), np.ones(bad.n_elements), np.zeros(bad.n_nodes))
    assert ei.value.status == gpu.SINGULAR_JACOBIAN
    # NaN conductivity -> NONFINITE from the solver
    gm = gpu.GpuMesh(m)
    eqs = gpu.LinearEQS(gm)
    ek = np.ones(m.n_elements)
    ek[5] = np.nan
    eqs.GlobalAssembly(gpu.make_params(steady=1), ek, np.zeros(m.n_nodes))
    eqs.SetKnownX(m.face_nodes(0, 0), np.ones(len(m.face_nodes(0, 0))))
    x = np.zeros(m.n_nodes)
    eqs.Solver(x, allow_fail=True)
    assert eqs.stats()["status"] == gpu.NONFINITE
    # bad arguments
    with pytest.raises(gpu.OgsError) as ei:
        eqs.SetKnownX([m.n_nodes + 5], [1.0])
    assert ei.value.status == gpu.BAD_ARG
    with pytest.raises(gpu.OgsError):
        eqs.ConfigNumerics(ls_method=13)
    with pytest.raises(gpu.OgsError):
        eqs.GlobalAssembly(gpu.make_params(dt=0.0), np.ones(m.n_elements), np.zeros(m.n_nodes))


def test_device_pointers(gpu, oracle):
    """torch CUDA tensors are used in place (no host staging)."""
    import torch
    m = M.structured_hex(8, 6, 5)
    ek = k_field(m, 9)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4)
    gm = gpu.GpuMesh(m)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    ek_d = torch.tensor(ek, device="cuda")
    u_d = torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda")
    eqs.GlobalAssembly(p, ek_d, u_d)
    torch.cuda.synchronize()
    rp, col, val = eqs.get_csr()
    oval, ob = oracle.assemble(m, rp, col, oracle_params(oracle, p), elem_k=ek, u0=np.zeros(m.n_nodes))
    assert_matrix_close(rp, val, oval)
    # steady system with one Dirichlet face: the solution is that value everywhere
    eqs.Initialize()
    eqs.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, steady=1), ek_d, u_d)
    lf = torch.tensor(m.face_nodes(0, 0), device="cuda")
    eqs.SetKnownX(lf, torch.full((len(lf),), 2.0, dtype=torch.float64, device="cuda"),
                  gpu.DIRICHLET_SYMMETRIC)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 2000, 1e-12)
    x = torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda")
    eqs.Solver(x)
    assert torch.allclose(x, torch.full_like(x, 2.0), rtol=0, atol=1e-9)


def test_golden_system_on_gpu(gpu):
    """The GPU path on the golden deck: matrix within 1e-12 of the fixture,
    CG heads within 1e-10 of the reference's own Linear_EQS::CG solution."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_linear_eqs.npz"))
    m = M.structured_hex(*[int(v) for v in g["shape"]])
    gm = gpu.GpuMesh(m)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    eqs.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4), g["elem_k"], g["u0"])
    rp, col, val = eqs.get_csr()
    assert np.array_equal(rp, g["row_ptr"]) and np.array_equal(col, g["col"])
    assert_matrix_close(rp, val, g["val"])
    assert_vector_close(eqs.get_rhs(), g["b"])
    eqs.SetKnownX(g["bc_rows"], g["bc_vals"], gpu.DIRICHLET_SYMMETRIC)
    assert_matrix_close(rp, eqs.get_values(), g["val_sym"])
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 2000, 1e-12)
    x = g["x0"].copy()
    it = eqs.Solver(x)
    assert abs(it - int(g["iter_cg"])) <= 1
    assert rel_max_err(x, g["x_cg"]) < SOLUTION_RTOL
