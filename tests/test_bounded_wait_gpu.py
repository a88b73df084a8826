"""The bounded grid-barrier waits of the two cooperative persistent kernels
(the persistent FP32 CG kernel and the Monte-Carlo batch kernel) end in an
error status instead of hanging: one block withholds its arrival, so the
others wait on a barrier word that nothing sets until their poll limit runs
out.  The same for the row waits of the ILU(0) kernels: a row left out of
the sweep is never published, so the rows after it give up.  The failure is
made on purpose only through that withheld arrival or row; the context stays
usable afterwards (a regular solve follows)."""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M

pytestmark = pytest.mark.gpu

SHORT_LIMIT = 1 << 14  # polls of the barrier word, a few milliseconds


@pytest.mark.parametrize("which", [0, 1])
def test_barrier_passes_when_every_block_arrives(gpu, which):
    r = gpu.selftest_barrier(which, spin_limit=SHORT_LIMIT)
    assert r["status"] == gpu.OK, r
    assert r["passed"] > 0


@pytest.mark.parametrize("which", [0, 1])
def test_withheld_arrival_times_out_with_an_error(gpu, which):
    r = gpu.selftest_barrier(which, spin_limit=SHORT_LIMIT, withhold=True)
    assert r["status"] == gpu.CUDA_ERROR, r
    assert "barrier timeout" in r["error"]
    assert r["passed"] == 0  # no waiting block passed
    # the context is still usable: the barrier passes again, and a solve runs
    assert gpu.selftest_barrier(which, spin_limit=SHORT_LIMIT)["status"] == gpu.OK
    m = M.structured_hex(8, 6, 5)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 3.0, seed=1)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 2000, 1e-10)
    eqs.Initialize()
    eqs.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4), ek, np.zeros(m.n_nodes))
    lf = m.face_nodes(0, 0)
    eqs.SetKnownX(lf, np.ones(len(lf)), gpu.DIRICHLET_SYMMETRIC)
    x = np.zeros(m.n_nodes)
    x[lf] = 1.0
    eqs.Solver(x)
    assert eqs.stats()["status"] == gpu.OK


def test_selftest_rejects_bad_arguments(gpu):
    assert gpu.selftest_barrier(3)["status"] == gpu.BAD_ARG
    assert gpu.selftest_barrier(0, grid=100000)["status"] == gpu.BAD_ARG


def test_ilu_row_waits_pass_when_every_row_is_published(gpu):
    r = gpu.selftest_barrier(2, spin_limit=SHORT_LIMIT)
    assert r["status"] == gpu.OK, r
    assert r["passed"] == 64  # every row of the chain exact


def test_ilu_unpublished_row_times_out_with_an_error(gpu):
    r = gpu.selftest_barrier(2, spin_limit=SHORT_LIMIT, withhold=True)
    assert r["status"] == gpu.CUDA_ERROR, r
    assert "ILU row wait timeout" in r["error"]
    assert r["passed"] < 64
    # the context is still usable: the sweep passes again, and an ILU solve runs
    assert gpu.selftest_barrier(2, spin_limit=SHORT_LIMIT)["status"] == gpu.OK
    m = M.structured_tet(6, 5, 4)
    ek = np.repeat(fields.lognormal_k((6, 5, 4), np.log(1e-5), 1.0, 3.0, seed=2), 6)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, gpu.PRECOND_ILU0, 2000, 1e-10)
    eqs.Initialize()
    eqs.GlobalAssembly(gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4), ek, np.zeros(m.n_nodes))
    lf = m.face_nodes(0, 0)
    eqs.SetKnownX(lf, np.ones(len(lf)), gpu.DIRICHLET_ROW_ONLY)
    x = np.zeros(m.n_nodes)
    x[lf] = 1.0
    eqs.Solver(x)
    assert eqs.stats()["status"] == gpu.OK
