"""Parity of the CUDA path with the oracle at the benchmark decks' full
sizes (the oracle itself is pinned to the reference OGS-5 on small decks by
tests/test_ref_assembly.py).

* Hex 128 x 128 x 64 (1,081,665 nodes, 28,607,425 stored entries): one
  transient GROUNDWATER_FLOW assembly, every entry of A and b at 1e-12;
  the heads of one step (symmetric Dirichlet faces, CG + Jacobi to 1e-13)
  at 1e-10, and the FP32-inner path's heads (tolerance 1e-10) within 1e-8
  of them.
* The same lattice split into 6,291,456 Kuhn tets: Gauss-point Darcy flux
  of a head field at 1e-12, the MASS_TRANSPORT assembly with that flux
  (every entry at 1e-12), and the concentrations of one BiCGStab + Jacobi
  step to 1e-13 at 1e-10.

The oracle runs single-threaded on the host: a few tens of seconds.
"""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import SOLUTION_RTOL, assert_matrix_close, assert_vector_close, rel_max_err

pytestmark = pytest.mark.gpu

NX, NY, NZ = 128, 128, 64
SEED = 2
DT, SS = 3600.0, 1e-4


def _faces(m):
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    return lf, rf, rows, vals, x0


def test_hex_128x128x64_assembly_and_step(gpu, oracle):
    m = M.structured_hex(NX, NY, NZ)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 8.0, seed=SEED)
    lf, rf, rows, vals, x0 = _faces(m)
    u0 = x0.copy()
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=DT, storage=SS)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.Initialize()
    eqs.GlobalAssembly(p, ek, u0)
    rp, col, val = eqs.get_csr()
    b = eqs.get_rhs()
    assert len(col) == 385 * 385 * 193
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    oval, ob = oracle.assemble(m, orp, ocol, oracle.make_params(pcs_type=0, dt=DT, storage=SS), elem_k=ek, u0=u0)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)
    # one step: symmetric Dirichlet, CG + Jacobi to 1e-13
    eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-13)
    x = x0.copy()
    eqs.Solver(x)
    oracle.dirichlet(orp, ocol, oval, ob, rows, vals, symmetric=True)
    xo, info = oracle.solve(orp, ocol, oval, ob, x0.copy(), method=5, precond=1, max_iter=20000, tol=1e-13)
    assert rel_max_err(x, xo) < SOLUTION_RTOL
    # the FP32-inner path at the deck tolerance, against the FP64 heads
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-10, precision=gpu.PRECISION_FP32_REFINED)
    x32 = x0.copy()
    eqs.Solver(x32)
    assert rel_max_err(x32, xo) < 1e-8


def test_tet_128x128x64_flux_transport_assembly_and_step(gpu, oracle):
    m = M.structured_tet(NX, NY, NZ)
    ek = np.repeat(fields.lognormal_k((NX, NY, NZ), np.log(1e-5), 1.0, 8.0, seed=SEED), 6)
    lf, rf, rows, vals, x0 = _faces(m)
    gm = gpu.GpuMesh(m)
    flow = gpu.LinearEQS(gm)
    flow.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-10)
    flow.Initialize()
    flow.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, dt=DT, storage=SS), ek, x0)
    flow.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC)
    h = x0.copy()
    flow.Solver(h)
    pf = gpu.make_params(gpu.GROUNDWATER_FLOW)
    q = flow.gp_velocity(pf, ek, h)
    del flow
    qo = oracle.gp_velocity(m, oracle.make_params(pcs_type=0), ek, h)
    assert_vector_close(q.ravel(), qo.ravel())
    kw = dict(dt=DT, theta=1.0, porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=1e-9)
    mt = gpu.LinearEQS(gm)
    mt.Initialize()
    c0 = np.zeros(m.n_nodes)
    mt.GlobalAssembly(gpu.make_params(gpu.MASS_TRANSPORT, **kw), None, c0, q)
    rp, col, val = mt.get_csr()
    b = mt.get_rhs()
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    oval, ob = oracle.assemble(m, orp, ocol, oracle.make_params(pcs_type=2, **kw), u0=c0, gp_vel=q)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)
    # one transport step: concentration 1 on the inflow face (row only)
    crow, cval = lf, np.ones(len(lf))
    mt.SetKnownX(crow, cval, gpu.DIRICHLET_ROW_ONLY)
    mt.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 5000, 1e-13, check_norm_rhs=False)
    x0c = np.zeros(m.n_nodes)
    x0c[lf] = 1.0
    c = x0c.copy()
    mt.Solver(c)
    oracle.dirichlet(orp, ocol, oval, ob, crow, cval, symmetric=False)
    co, _ = oracle.solve(orp, ocol, oval, ob, x0c.copy(), method=2, precond=1, max_iter=5000, tol=1e-13)
    assert rel_max_err(c, co) < SOLUTION_RTOL
