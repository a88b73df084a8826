"""Run-to-run determinism of the CUDA path (the substitute for a race
detector on this path).

The element kernels scatter with FP64 atomics, so two assemblies of the
same system add each entry's element contributions in whatever order the
atomics land: entries agree within the matrix bar (1e-12 relative), not
bitwise.  Everything else is ordered: the Krylov kernels add their block
partials in a fixed order, the batch kernel assembles row-centrically
without atomics, so a solve repeated on the same system gives bitwise the
same heads.
"""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import assert_matrix_close, assert_vector_close, distort

pytestmark = pytest.mark.gpu


def _assemble(gpu, m, p, ek, u0, gpv=None):
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.Initialize()
    eqs.GlobalAssembly(p, ek, u0, gpv)
    rp, col, val = eqs.get_csr()
    return eqs, rp, val, eqs.get_rhs()


@pytest.mark.parametrize("kind", ["hex", "tet_transport", "quad_distorted"])
def test_two_assemblies_agree(gpu, kind):
    rng = np.random.default_rng(4)
    gpv = None
    if kind == "hex":
        m = M.structured_hex(20, 16, 12)
        p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4)
        ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=2)
    elif kind == "tet_transport":
        m = M.structured_tet(10, 8, 6)
        p = gpu.make_params(gpu.MASS_TRANSPORT, dt=3600.0, theta=0.6, porosity=0.3, alpha_l=1.0, alpha_t=0.1,
                            diffusion=1e-9)
        ek = None
        gpv = rng.normal(0, 1e-5, (m.n_elements, 5, 3))
    else:
        m = distort(M.structured_quad(60, 40), 0.2, seed=5)
        p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=100.0, storage=1e-3)
        ek = np.exp(np.log(1e-5) + rng.standard_normal(m.n_elements))
    u0 = rng.uniform(0, 1, m.n_nodes)
    _, rp, v1, b1 = _assemble(gpu, m, p, ek, u0, gpv)
    _, _, v2, b2 = _assemble(gpu, m, p, ek, u0, gpv)
    assert_matrix_close(rp, v1, v2)
    assert_vector_close(b1, b2)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_repeated_solve_is_bitwise(gpu, precision):
    m = M.structured_hex(24, 18, 12)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 4.0, seed=8)
    eqs, rp, val, b = _assemble(gpu, m, gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4), ek,
                                np.zeros(m.n_nodes))
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    eqs.SetKnownX(np.concatenate([lf, rf]), np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))]),
                  gpu.DIRICHLET_SYMMETRIC)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, 1e-10, check_norm_rhs=False,
                       precision=gpu.PRECISION_FP64 if precision == "fp64" else gpu.PRECISION_FP32_REFINED)
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    heads, iters = [], []
    for _ in range(2):
        x = x0.copy()
        iters.append(eqs.Solver(x))
        heads.append(x)
    assert iters[0] == iters[1]
    assert np.array_equal(heads[0], heads[1])


def test_batch_solve_is_bitwise(gpu):
    rng = np.random.default_rng(3)
    reals = []
    for q, (nx, ny, nz) in enumerate([(8, 7, 6), (12, 9, 7), (5, 5, 5), (16, 10, 8)]):
        ek = fields.lognormal_k((nx - 1, ny - 1, nz - 1), np.log(1e-5), 1.0, 3.0, seed=q)
        reals.append((nx, ny, nz, ek, float(rng.uniform(5, 15)), 0.0))
    out = []
    for _ in range(2):
        b = gpu.Batch(reals, tol=1e-10)
        b.solve()
        out.append(np.concatenate(b.heads()))
        b.close()
    assert np.array_equal(out[0], out[1])
