"""Closed-form known answers for the oracle's element matrices."""
import numpy as np
import pytest

from ogs5_gb300 import mesh as M


def unit_elem(et):
    if et == 1:
        m = M.structured_hex(1, 1, 1)
    elif et == 0:
        m = M.structured_quad(1, 1)
    else:
        m = M.structured_tet(1, 1, 1)
        m.conn = m.conn[:1]
    return np.stack([m.x[m.conn[0]], m.y[m.conn[0]], m.z[m.conn[0]]], axis=1)


def test_unit_cube_hex_laplace(oracle):
    c = unit_elem(1)
    m = oracle.element_matrices(1, c, oracle.make_params(pcs_type=0, storage=1.0), k_e=1.0)
    L, Ms = m["laplace"], m["mass"]
    assert np.allclose(np.diag(L), 1 / 3, rtol=1e-13)
    assert np.allclose(L.sum(axis=1), 0.0, atol=1e-14)
    # nodes 0 and 6 are opposite corners: -1/12; face diagonal 0-2: -1/12; edge 0-1: 0
    assert abs(L[0, 6] + 1 / 12) < 1e-14 and abs(L[0, 2] + 1 / 12) < 1e-14 and abs(L[0, 1]) < 1e-14
    # consistent mass of the unit cube: diag 1/27, total 1
    assert abs(Ms[0, 0] - 1 / 27) < 1e-14 and abs(Ms.sum() - 1.0) < 1e-13


def test_unit_square_quad(oracle):
    c = unit_elem(0)
    m = oracle.element_matrices(0, c, oracle.make_params(pcs_type=0, storage=1.0), k_e=1.0)
    L, Ms = m["laplace"], m["mass"]
    assert np.allclose(np.diag(L), 2 / 3, rtol=1e-13)
    assert abs(L[0, 2] + 1 / 3) < 1e-14 and abs(L[0, 1] + 1 / 6) < 1e-14
    assert abs(Ms[0, 0] - 1 / 9) < 1e-14 and abs(Ms.sum() - 1.0) < 1e-13


def test_reference_tet(oracle):
    c = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    m = oracle.element_matrices(2, c, oracle.make_params(pcs_type=0, storage=1.0), k_e=1.0)
    L, Ms = m["laplace"], m["mass"]
    vol = 1 / 6
    g = np.array([[-1, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    assert np.allclose(L, vol * g @ g.T, rtol=1e-12, atol=1e-15)
    # the 5-point rule (negative centre weight) integrates N_i N_j exactly
    want = vol / 20 * (np.ones((4, 4)) + np.eye(4))
    assert np.allclose(Ms, want, rtol=1e-12)


def test_linear_profile_exact(oracle):
    """The 100 x 100 quad deck: h = 1 - x/100 is reproduced to rounding."""
    m = M.structured_quad(100, 100)
    rp, col = oracle.build_pattern(m.n_nodes, m.conn)
    assert len(col) == 301 * 301  # 90,601 stored entries
    p = oracle.make_params(pcs_type=0, steady=1)
    val, b = oracle.assemble(m, rp, col, p, elem_k=np.full(m.n_elements, 1e-4), u0=np.zeros(m.n_nodes))
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.ones(len(lf)), np.zeros(len(rf))])
    oracle.dirichlet(rp, col, val, b, rows, vals)
    x0 = np.full(m.n_nodes, 0.5)
    x0[lf], x0[rf] = 1.0, 0.0
    x, info = oracle.solve(rp, col, val, b, x0, method=2, precond=1, tol=1e-10)
    assert info["rel_residual"] < 1e-10
    assert np.abs(x - (1 - m.x / 100)).max() < 1e-8  # residual 1e-10 x conditioning


def test_advection_dispersion_known_answer(oracle):
    """Tet, uniform flux q along x: advection row sums vanish (sum_j dN_j = 0)
    and the dispersion tensor is alpha_L|q| along x, alpha_T|q| across."""
    c = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    q = 2e-5
    vel = np.zeros((5, 3))
    vel[:, 0] = q
    p = oracle.make_params(pcs_type=2, porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=0.0)
    m = oracle.element_matrices(2, c, p, vel=vel)
    assert np.allclose(m["advection"].sum(axis=1), 0.0, atol=1e-20)
    g = np.array([[-1, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    D = np.diag([1.0 * q, 0.1 * q, 0.1 * q])
    assert np.allclose(m["laplace"], (1 / 6) * g @ D @ g.T, rtol=1e-11, atol=1e-22)


def test_ilu0_reproduces_matrix_on_pattern(oracle):
    """ILU(0) property: (L U)_ij = a_ij for every (i, j) of the pattern, and
    for a tridiagonal matrix ILU(0) is the exact LU factorisation."""
    from ogs5_gb300 import mesh as M
    m = M.structured_quad(7, 5)
    rp, col = oracle.build_pattern(m.n_nodes, m.conn)
    p = oracle.make_params(pcs_type=0, dt=10.0, storage=1e-3, time_unit_factor=1.0, theta=1.0)
    val, _ = oracle.assemble(m, rp, col, p, elem_k=np.full(m.n_elements, 1e-4),
                             u0=np.zeros(m.n_nodes))
    lu = oracle.ilu0_factor(rp, col, val)
    n = m.n_nodes
    A = np.zeros((n, n))
    L = np.eye(n)
    U = np.zeros((n, n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            j = col[k]
            A[i, j] = val[k]
            if j < i:
                L[i, j] = lu[k]
            else:
                U[i, j] = lu[k]
    P = L @ U
    mask = A != 0
    assert np.allclose(P[mask], A[mask], rtol=1e-12, atol=1e-14 * np.abs(A).max())
    # tridiagonal: exact
    t = 9
    trp = np.concatenate([[0], np.cumsum([2] + [3] * (t - 2) + [2])]).astype(np.int64)
    tcol = []
    for i in range(t):
        tcol += [j for j in (i - 1, i, i + 1) if 0 <= j < t]
    tcol = np.array(tcol, dtype=np.int64)
    rng = np.random.default_rng(0)
    tval = rng.uniform(-1, 0, len(tcol))
    T = np.zeros((t, t))
    for i in range(t):
        for k in range(trp[i], trp[i + 1]):
            T[i, tcol[k]] = tval[k]
        T[i, i] = 4.0
    for i in range(t):
        for k in range(trp[i], trp[i + 1]):
            tval[k] = T[i, tcol[k]]
    tlu = oracle.ilu0_factor(trp, tcol, tval)
    L = np.eye(t)
    U = np.zeros((t, t))
    for i in range(t):
        for k in range(trp[i], trp[i + 1]):
            (L if tcol[k] < i else U)[i, tcol[k]] = tlu[k]
    assert np.allclose(L @ U, T, rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("et,vol", [(0, 1.0), (1, 1.0), (2, None)])
def test_lumped_mass_is_volume_over_nodes(oracle, et, vol):
    """ele_mass_lumping: the mass matrix is diag(c * V_e / n) (CalcLumpedMass),
    V_e from the mesh's volume decomposition; its sum equals the consistent
    mass's sum, c * V_e."""
    c = unit_elem(et)
    nn = c.shape[0]
    cons = oracle.element_matrices(et, c, oracle.make_params(pcs_type=0, storage=2.5), k_e=1.0)["mass"]
    lump = oracle.element_matrices(et, c, oracle.make_params(pcs_type=0, storage=2.5, mass_lumping=1),
                                   k_e=1.0)["mass"]
    assert np.count_nonzero(lump - np.diag(np.diag(lump))) == 0
    assert np.allclose(np.diag(lump), lump[0, 0], rtol=0, atol=0)
    assert abs(lump.sum() - cons.sum()) < 1e-13 * abs(cons.sum())
    if vol is not None:
        assert abs(lump[0, 0] - 2.5 * vol / nn) < 1e-14
    # distorted hexahedron: the six-tetrahedra volume, not the Gauss volume
    if et == 1:
        d = c.copy()
        d[6] += np.array([0.3, 0.2, 0.1])
        tets = [(4, 7, 5, 0), (5, 3, 1, 0), (5, 7, 3, 0), (5, 7, 6, 2), (1, 3, 5, 2), (3, 7, 5, 2)]
        v = sum(abs(np.linalg.det(np.array([d[a] - d[q], d[b] - d[q], d[cc] - d[q]]))) / 6
                for a, b, cc, q in tets)
        lm = oracle.element_matrices(1, d, oracle.make_params(pcs_type=0, storage=1.0, mass_lumping=1),
                                     k_e=1.0)["mass"]
        assert abs(lm[0, 0] - v / 8) < 1e-14


@pytest.mark.parametrize("method", [1, 2])
def test_supg_terms_on_a_tet(oracle, method):
    """SUPG (ele_supg_method) on the reference tet with a constant flux:
    w_i = v . grad N_i and tau are constant, so the added advection is
    V tau w_i w_j and the added mass c tau w_i V / 4 (the 5-point rule
    integrates N_j exactly); tau from the longest edge and the largest
    dispersion entry."""
    c = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    vol = 1 / 6
    g = np.array([[-1, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    v = np.array([2e-5, -1e-5, 5e-6])
    vel = np.tile(v, (5, 1))
    kw = dict(pcs_type=2, dt=600.0, porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=1e-9,
              retardation=1.2)
    off = oracle.element_matrices(2, c, oracle.make_params(**kw), vel=vel)
    on = oracle.element_matrices(2, c, oracle.make_params(supg_method=method, **kw), vel=vel)
    vm = np.linalg.norm(v)
    D = 0.1 * vm * np.eye(3) + (1.0 - 0.1) * np.outer(v, v) / vm + 1e-9 * 0.3 * np.eye(3)
    diff = D.max()
    L = np.sqrt(2.0)  # longest edge of the reference tet
    if method == 1:
        a = 0.5 * vm * L / diff
        tau = 0.5 * L / vm * (1 / np.tanh(a) - 1 / a if a < 20 else 1.0)
    else:
        tau = 1 / np.sqrt((2 / 600.0) ** 2 + (2 * vm / L) ** 2 + (4 * diff / L ** 2) ** 2)
    w = g @ v
    cm = 0.3 * 1.0 * 1.2
    assert np.allclose(on["advection"] - off["advection"], vol * tau * np.outer(w, w), rtol=1e-10, atol=0)
    assert np.allclose(on["mass"] - off["mass"], cm * tau * np.outer(w, np.full(4, vol / 4)), rtol=1e-10,
                       atol=0)
    assert np.allclose(on["laplace"], off["laplace"], rtol=0, atol=0)


@pytest.mark.parametrize("model", [4, 6])
def test_richards_curves(oracle, model):
    """Saturation, dSw/dpc and k_rel of the Richards medium (van Genuchten
    and Brooks-Corey, rf_mmp_new.cpp:5243-5520, 2576-2635): closed forms,
    the clamps to [slr + eps, slm - eps], and dSw/dpc(S(pc)) against a
    centred difference of S(pc)."""
    m = 0.6 if model == 4 else 2.0
    r = oracle.richards_params(capillary_model=model, permeability_model=model, pb=2.0e3, slr=0.15, slm=0.95,
                               m=m, kr_slr=0.15, kr_slm=0.95, kr_m=m, kr_min=1e-8)
    eps = np.finfo(float).eps
    for pc in (3.0e3, 1.0e4, 4.0e4):
        s = oracle.rich_curves(r, pc=pc)["saturation"]
        if model == 4:
            se = (1.0 + (pc / 2.0e3) ** (1.0 / (1.0 - m))) ** (-m)
        else:
            se = (pc / 2.0e3) ** (-m)
        assert abs(s - (0.15 + 0.8 * se)) < 1e-14
        h = pc * 1e-6
        fd = (oracle.rich_curves(r, pc=pc + h)["saturation"] - oracle.rich_curves(r, pc=pc - h)["saturation"]) / (2 * h)
        d = oracle.rich_curves(r, sw=s)["dsdpc"]
        assert d < 0 and abs(d - fd) < 1e-6 * abs(fd)
        se_k = (s - 0.15) / 0.8
        kr = (np.sqrt(se_k) * (1 - (1 - se_k ** (1 / m)) ** m) ** 2 if model == 4 else se_k ** (3 + 2 / m))
        assert abs(oracle.rich_curves(r, sw=s)["krel"] - max(kr, 1e-8)) < 1e-13
    # full saturation: pc <= 0 (van Genuchten) or pc <= pb (Brooks-Corey)
    assert oracle.rich_curves(r, pc=-5.0)["saturation"] == 0.95 - eps
    assert oracle.rich_curves(r, sw=0.1)["krel"] == 1e-8  # below residual: minimum k_rel


def test_richards_coefficients(oracle):
    """CalCoefMass / CalCoefLaplace of RICHARDS_FLOW: saturated (p >= 0)
    storage Ss + n drho/dp and K / mu; unsaturated adds n dSw/dp (> 0)
    and scales K by k_rel(S(-p))."""
    r = oracle.richards_params()
    p = oracle.make_params(pcs_type=3, storage=1e-6, porosity=0.35, drho_dp=4.4e-10, viscosity=1e-3,
                           density=1000.0, time_unit_factor=1.0)
    mc, lc = oracle.rich_coefficients(p, r, 1e-12, 2.0e3)
    assert abs(mc - (1e-6 + 0.35 * 4.4e-10)) < 1e-20
    kr_sat = oracle.rich_curves(r, sw=1.0 - np.finfo(float).eps)["krel"]
    assert abs(lc - 1e-12 * (kr_sat / 1e-3)) < 1e-22
    mc, lc = oracle.rich_coefficients(p, r, 1e-12, -1.5e4)
    s = oracle.rich_curves(r, pc=1.5e4)["saturation"]
    d = -oracle.rich_curves(r, sw=s)["dsdpc"]
    assert abs(mc - (1e-6 * s + 0.35 * s * 4.4e-10 + 0.35 * d)) < 1e-18
    assert abs(lc - 1e-12 * (oracle.rich_curves(r, sw=s)["krel"] / 1e-3)) < 1e-24
