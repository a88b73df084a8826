"""Monte-Carlo batch (ogs_gpu_batch_*): one persistent launch assembles and
solves many steady flow realisations of different sizes.

Bar: every realisation's heads within 1e-8 relative of the plain FP64 GPU
path (GpuMesh + LinearEQS: element assembly, symmetric Dirichlet, FP64
Jacobi-CG) on the same field, and the batch's own FP64 residual below its
tolerance.
"""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import rel_max_err

pytestmark = pytest.mark.gpu

BATCH_RTOL = 1e-8


def _realisations(sizes, seed=0, var=1.0):
    rng = np.random.default_rng(seed)
    out = []
    for q, (nx, ny, nz) in enumerate(sizes):
        ek = fields.lognormal_k((nx - 1, ny - 1, nz - 1), np.log(1e-5), var,
                                float(rng.uniform(2, 4)), seed=seed * 1000 + q)
        out.append((nx, ny, nz, ek, float(rng.uniform(5, 15)), float(rng.uniform(-1, 1))))
    return out


def _plain_fp64(gpu, nx, ny, nz, ek, hl, hr, tol=1e-13, spacing=(1.0, 1.0, 1.0)):
    m = M.structured_hex(nx - 1, ny - 1, nz - 1, *spacing)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.Initialize()
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, steady=1)
    eqs.GlobalAssembly(p, ek, np.zeros(m.n_nodes))
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    eqs.SetKnownX(np.concatenate([lf, rf]), np.concatenate([np.full(len(lf), hl), np.full(len(rf), hr)]),
                  gpu.DIRICHLET_SYMMETRIC)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, tol)
    x = np.zeros(m.n_nodes)
    x[lf], x[rf] = hl, hr
    eqs.Solver(x)
    return x


def test_batch_matches_plain_fp64_path(gpu):
    sizes = [(6, 5, 4), (9, 7, 5), (12, 10, 8), (3, 3, 3), (20, 6, 9), (15, 15, 15)]
    reals = _realisations(sizes, seed=1)
    b = gpu.Batch(reals, tol=1e-11)
    stats = b.solve()
    heads = b.heads()
    for (nx, ny, nz, ek, hl, hr), st, h in zip(reals, stats, heads):
        assert st["status"] == gpu.OK
        assert st["rel_residual"] < 1e-11
        assert st["iterations"] > 0 and st["refinements"] >= 2
        ref = _plain_fp64(gpu, nx, ny, nz, ek, hl, hr)
        assert rel_max_err(h, ref) < BATCH_RTOL, (nx, ny, nz)


def test_batch_homogeneous_linear_profile(gpu):
    """Homogeneous K: h = hl + (hr - hl) x / L exactly in trilinear FE."""
    reals = [(n, 4, 3, np.full((n - 1) * 3 * 2, 2e-4), 3.0, 1.0) for n in (5, 11, 17)]
    b = gpu.Batch(reals, hx=0.5, hy=2.0, hz=1.5, tol=1e-12)
    b.solve()
    for (nx, ny, nz, _, hl, hr), h in zip(reals, b.heads()):
        ix = np.arange(nx * ny * nz) % nx
        exact = hl + (hr - hl) * ix / (nx - 1)
        assert np.abs(h - exact).max() < 1e-9


def test_batch_tunings_agree_and_autotune(gpu):
    sizes = [(10, 8, 6), (14, 9, 7), (7, 7, 7), (18, 12, 5)]
    reals = _realisations(sizes, seed=3, var=2.0)
    b = gpu.Batch(reals, tol=1e-10)
    results = []
    for tr, nt, bps in ((64, 256, 1), (256, 512, 1), (4096, 256, 2)):
        b.set_tuning(tr, nt, bps)
        st = b.solve()
        assert all(s["status"] == gpu.OK for s in st)
        results.append(b.heads_flat())
    for r in results[1:]:
        assert rel_max_err(r, results[0]) < BATCH_RTOL
    t = b.autotune()
    assert t["tile_rows"] in (2048, 4096, 8192) and t["block_threads"] in (256, 512)
    assert t["blocks_per_sm"] >= 1 and t["ms_per_step"] > 0
    st = b.solve()
    assert all(s["status"] == gpu.OK for s in st)
    assert rel_max_err(b.heads_flat(), results[0]) < BATCH_RTOL


def test_batch_zero_rhs_and_not_converged(gpu):
    """h = 0 on both faces: b = 0, CheckNormRHS ends the solve at once with
    x = 0; a max_iter of 3 leaves the other realisations NOT_CONVERGED."""
    reals = [(6, 6, 6, np.full(125, 1e-5), 0.0, 0.0), (8, 6, 5, np.full(7 * 5 * 4, 1e-5), 1.0, 0.0)]
    b = gpu.Batch(reals, tol=1e-10)
    st = b.solve()
    assert st[0]["status"] == gpu.OK and st[0]["iterations"] == 0
    h = b.heads()
    assert np.all(h[0] == 0.0)
    b2 = gpu.Batch(reals, tol=1e-10, max_iter=3)
    st2 = b2.solve(allow_fail=True)
    assert st2[0]["status"] == gpu.OK
    assert st2[1]["status"] == gpu.NOT_CONVERGED


def test_batch_set_k_resolves(gpu):
    sizes = [(8, 7, 6), (11, 5, 4)]
    reals = _realisations(sizes, seed=5)
    b = gpu.Batch(reals, tol=1e-11)
    b.solve()
    new = _realisations(sizes, seed=6)
    b.set_k(np.concatenate([r[3] for r in new]))
    b.solve()
    for (nx, ny, nz, _, hl, hr), (_, _, _, ek, _, _), h in zip(reals, new, b.heads()):
        ref = _plain_fp64(gpu, nx, ny, nz, ek, hl, hr)
        assert rel_max_err(h, ref) < BATCH_RTOL


def test_batch_rejects_bad_input(gpu):
    with pytest.raises(gpu.OgsError):
        gpu.Batch([(2, 5, 5, np.ones(16), 1.0, 0.0)])
    with pytest.raises(ValueError):
        gpu.Batch([(4, 4, 4, np.ones(5), 1.0, 0.0)])
