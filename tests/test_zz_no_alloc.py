"""ogs_gpu_csr_cg_noalloc: the CG entry point for callers that cannot
allocate device memory (their HBM already belongs to a caching allocator or
memory pool, where each solver buffer would fail or fragment the pool).  It
must give the same heads as the regular solver (ogs_gpu_solve, same
tolerance as the other solver parity tests: 1e-10 relative) on two calls in
a row, since all calls share one static scratch array that keeps the
previous contents; a following call on a smaller, different system must not
see the larger system's leftovers; and a call must leave the device's free
memory unchanged.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import SOLUTION_RTOL, rel_max_err

pytestmark = pytest.mark.gpu


def test_noalloc_cg_matches_regular_solver_twice(gpu):
    import torch
    m = M.structured_hex(40, 30, 20)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 5.0, seed=7)
    gm = gpu.GpuMesh(m)
    eqs = gpu.LinearEQS(gm)
    eqs.Initialize()
    eqs.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4), ek,
                       np.zeros(m.n_nodes))
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    eqs.SetKnownX(np.concatenate([lf, rf]), np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))]),
                  gpu.DIRICHLET_SYMMETRIC)
    rp, col, val = eqs.get_csr()
    b = eqs.get_rhs()
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    # regular entry point, fresh-system stopping rule (no carried |b|)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, 1e-12, check_norm_rhs=False)
    x_ref = x0.copy()
    it_ref = eqs.Solver(x_ref)
    # the caller owns the matrix and vectors on the device
    rp_d = torch.tensor(rp.astype(np.int32), device="cuda")
    col_d = torch.tensor(col.astype(np.int32), device="cuda")
    val_d = torch.tensor(val, device="cuda")
    b_d = torch.tensor(b, device="cuda")
    for call in range(2):
        x_d = torch.tensor(x0, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = gpu.csr_cg_noalloc(rp_d, col_d, val_d, b_d, x_d, max_iter=5000, tol=1e-12)
        torch.cuda.synchronize()
        if call == 1:
            # nothing allocated (the first call may load this library's
            # kernels, which the driver does lazily)
            assert torch.cuda.mem_get_info()[0] == free_before
        assert st["status"] == gpu.OK, (call, st)
        assert st["rel_residual"] < 1e-12
        assert abs(st["iterations"] - it_ref) <= 2, (call, st["iterations"], it_ref)
        assert rel_max_err(x_d.cpu().numpy(), x_ref) < SOLUTION_RTOL, call
    # a smaller, different system after the larger one: the shared scratch
    # still holds the larger system's vectors past the new system's rows
    m2 = M.structured_quad(60, 45)
    ek2 = fields.lognormal_k(m2.shape, np.log(1e-4), 0.5, 4.0, seed=3)
    gm2 = gpu.GpuMesh(m2)
    eqs2 = gpu.LinearEQS(gm2)
    eqs2.Initialize()
    eqs2.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, dt=100.0, storage=1e-3), ek2,
                        np.zeros(m2.n_nodes))
    lf2, rf2 = m2.face_nodes(1, 0), m2.face_nodes(1, 1)
    eqs2.SetKnownX(np.concatenate([lf2, rf2]), np.concatenate([np.full(len(lf2), 3.0), np.full(len(rf2), 1.0)]),
                   gpu.DIRICHLET_SYMMETRIC)
    rp2, col2, val2 = eqs2.get_csr()
    b2 = eqs2.get_rhs()
    x02 = np.zeros(m2.n_nodes)
    x02[lf2], x02[rf2] = 3.0, 1.0
    eqs2.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, 1e-12, check_norm_rhs=False)
    x_ref2 = x02.copy()
    eqs2.Solver(x_ref2)
    x2_d = torch.tensor(x02, device="cuda")
    st2 = gpu.csr_cg_noalloc(torch.tensor(rp2.astype(np.int32), device="cuda"),
                             torch.tensor(col2.astype(np.int32), device="cuda"),
                             torch.tensor(val2, device="cuda"), torch.tensor(b2, device="cuda"), x2_d,
                             max_iter=5000, tol=1e-12)
    torch.cuda.synchronize()
    assert st2["status"] == gpu.OK, st2
    assert rel_max_err(x2_d.cpu().numpy(), x_ref2) < SOLUTION_RTOL


def test_noalloc_rejects_oversized_and_host_arrays(gpu):
    import torch
    L = gpu.lib()
    small_i = torch.zeros(8, dtype=torch.int32, device="cuda")
    small_d = torch.zeros(8, dtype=torch.float64, device="cuda")
    p_i, p_d = small_i.data_ptr(), small_d.data_ptr()
    st = gpu.SolveStats()
    rc = L.ogs_gpu_csr_cg_noalloc(gpu.NOALLOC_MAX_ROWS + 1, p_i, p_i, p_d, p_d, p_d, 10, 1e-10, None,
                                  C.byref(st))
    assert rc == gpu.BAD_ARG and b"exceed" in L.ogs_gpu_last_error()
    host = np.zeros(8)
    rc = L.ogs_gpu_csr_cg_noalloc(7, p_i, p_i, p_d, host.ctypes.data, p_d, 10, 1e-10, None, C.byref(st))
    assert rc == gpu.BAD_ARG and b"device memory" in L.ogs_gpu_last_error()
