"""Request server (ogs_gpu_server_*): continuous batching of flow and
transport requests.

Bars: every request's result in a mix of concurrent requests equals its
result when served alone, and the blocking single-system API's on the same
system, within the solution parity bar (1e-10 relative max-norm; each
request runs the single-system kernels on a system of its own, and only the
assembly's FP64 atomics may round the matrix differently between runs).
FP32-inner requests are solved to a tenth of their tolerance, so the
blocking API is configured the same way.  With dynamic batching, requests
served by one batch launch are within 1e-8 of an FP64 solve to 1e-13 of
the same system (the precision extension's bar) at tolerance 1e-10.
"""
import numpy as np
import pytest

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import rel_max_err

pytestmark = pytest.mark.gpu


def _classes(gpu, srv):
    torch = pytest.importorskip("torch")
    out = []
    specs = [("quad", M.structured_quad(60, 40), gpu.REQUEST_FLOW),
             ("hex", M.structured_hex(14, 10, 8), gpu.REQUEST_FLOW),
             ("tet", M.structured_tet(8, 6, 5), gpu.REQUEST_TRANSPORT),
             ("hex", M.structured_hex(12, 8, 6), gpu.REQUEST_TRANSPORT)]
    for name, m, kind in specs:
        gm = gpu.GpuMesh(m)
        lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
        if kind == gpu.REQUEST_FLOW:
            rows = np.concatenate([lf, rf])
            vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
            p = gpu.make_params(gpu.GROUNDWATER_FLOW, steady=1)
            cfg = gpu.solver_config(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000,
                                    precision=gpu.PRECISION_FP32_REFINED)
            cid = srv.add_class(gm, kind, p, rows, vals, gpu.DIRICHLET_SYMMETRIC, cfg)
        else:
            rows, vals = lf, np.ones(len(lf))
            p = gpu.make_params(gpu.MASS_TRANSPORT, dt=3600.0, porosity=0.3, alpha_l=1.0, alpha_t=0.1,
                                diffusion=1e-9)
            fp = gpu.make_params(gpu.GROUNDWATER_FLOW)
            head = 10.0 * (1.0 - m.x / m.x.max())
            cfg = gpu.solver_config(gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI, 5000)
            cid = srv.add_class(gm, kind, p, rows, vals, gpu.DIRICHLET_ROW_ONLY, cfg, flow_params=fp,
                                flow_head=head)
        out.append((cid, m, gm, kind, p, rows, vals, cfg))
    return torch, out


def _k(torch, m, seed):
    """element conductivities on the device (tets: the field of the parent hex)"""
    k = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 3.0, seed=seed)
    if len(k) != m.n_elements:
        k = np.repeat(k, m.n_elements // len(k))
    return torch.tensor(k, device="cuda")


def test_server_mix_equals_alone_and_blocking_api(gpu):
    srv = gpu.Server(max_active=64, flags=gpu.SERVER_PRIORITY | gpu.SERVER_SJF)
    torch, classes = _classes(gpu, srv)
    reqs = []
    for q in range(16):
        cid, m, gm, kind, p, rows, vals, cfg = classes[q % len(classes)]
        tol = 1e-10 if q % 3 else 1e-6
        reqs.append((cid, m, _k(torch, m, 100 + q), tol, classes[q % len(classes)]))
    # alone: one request at a time
    alone = []
    for cid, m, k, tol, _ in reqs:
        out = torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda")
        rid = srv.submit(cid, k, tol, out)
        srv.drain()
        r = srv.result(rid)
        assert r["state"] == 2 and r["status"] == gpu.OK, r
        assert r["rel_residual"] < tol
        alone.append(out.cpu().numpy())
    # mix: half submitted up front, the rest while those run
    outs = [torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda") for _, m, _, _, _ in reqs]
    ids = [None] * len(reqs)
    for q in range(8):
        ids[q] = srv.submit(reqs[q][0], reqs[q][2], reqs[q][3], outs[q])
    srv.progress()
    overlapped = srv.info()["running"]
    for q in range(8, len(reqs)):
        ids[q] = srv.submit(reqs[q][0], reqs[q][2], reqs[q][3], outs[q])
        srv.progress()
    srv.drain()
    assert overlapped > 1  # requests were in flight together
    for q, (cid, m, k, tol, cl) in enumerate(reqs):
        r = srv.result(ids[q])
        assert r["status"] == gpu.OK and r["rel_residual"] < tol
        mix = outs[q].cpu().numpy()
        assert rel_max_err(mix, alone[q]) <= 1e-10, (q, rel_max_err(mix, alone[q]))
    # the blocking single-system API on the same systems
    for q in (0, 1, 2, 3):
        cid, m, k, tol, (cid_, m_, gm, kind, p, rows, vals, cfg) = reqs[q]
        eqs = gpu.LinearEQS(gm)
        stop = tol * 0.1 if cfg.precision != gpu.PRECISION_FP64 else tol
        eqs.ConfigNumerics(cfg.method, cfg.precond, cfg.max_iter, stop, precision=cfg.precision)
        eqs.Initialize()
        x0 = np.zeros(m.n_nodes)
        x0[rows] = vals
        if kind == gpu.REQUEST_FLOW:
            eqs.GlobalAssembly(p, k, x0)
            eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC)
        else:
            head = 10.0 * (1.0 - m.x / m.x.max())
            q_gp = eqs.gp_velocity(gpu.make_params(gpu.GROUNDWATER_FLOW), k, head)
            eqs.GlobalAssembly(p, None, x0, q_gp)
            eqs.SetKnownX(rows, vals, gpu.DIRICHLET_ROW_ONLY)
        x = x0.copy()
        eqs.Solver(x)
        assert rel_max_err(x, alone[q]) <= 1e-10
    srv.close()


def _fp64_converged(gpu, gm, m, p, k, rows, vals):
    eqs = gpu.LinearEQS(gm)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, 1e-13)
    eqs.Initialize()
    x0 = np.zeros(m.n_nodes)
    x0[rows] = vals
    eqs.GlobalAssembly(p, k, x0)
    eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC)
    x = x0.copy()
    eqs.Solver(x)
    return x


def test_server_batches_same_class_requests(gpu):
    """Dynamic batching: requests of one steady hex-lattice flow class with
    the same tolerance, queued together, are served by one batch launch;
    every result within 1e-8 of an FP64 solve to 1e-13; a request of
    another tolerance is served on a slot; a later group of the same size
    reuses the batch object with new fields."""
    torch = pytest.importorskip("torch")
    m = M.structured_hex(16, 12, 10, 1.0, 2.0, 0.5)
    gm = gpu.GpuMesh(m)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 7.0), np.full(len(rf), 2.0)])
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, steady=1)
    cfg = gpu.solver_config(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, precision=gpu.PRECISION_FP32_REFINED)
    srv = gpu.Server(max_active=8, flags=gpu.SERVER_SJF | gpu.SERVER_BATCH)
    cid = srv.add_class(gm, gpu.REQUEST_FLOW, p, rows, vals, gpu.DIRICHLET_SYMMETRIC, cfg)
    for group in range(2):
        ks = [_k(torch, m, 300 + 10 * group + q) for q in range(7)]
        tols = [1e-10] * 6 + [1e-6]
        outs = [torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda") for _ in ks]
        ids = [srv.submit(cid, k, t, o) for k, t, o in zip(ks, tols, outs)]
        srv.drain()
        res = [srv.result(i) for i in ids]
        assert all(r["status"] == gpu.OK for r in res), res
        assert [r["batch_size"] for r in res[:6]] == [6] * 6
        assert all(r["iterations"] > 0 for r in res)
        assert res[6]["batch_size"] == 0  # alone of its tolerance: a slot
        for q in range(6):
            x = _fp64_converged(gpu, gm, m, p, ks[q], rows, vals)
            assert rel_max_err(outs[q].cpu().numpy(), x) < 1e-8, (group, q)
    assert srv.info()["batched"] == 12
    srv.close()


def test_server_admission_respects_budget_and_max_active(gpu):
    torch = pytest.importorskip("torch")
    m = M.structured_hex(10, 8, 6)
    gm = gpu.GpuMesh(m)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.ones(len(lf)), np.zeros(len(rf))])
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, steady=1)
    cfg = gpu.solver_config(precision=gpu.PRECISION_FP32_REFINED)
    # max_active 2
    srv = gpu.Server(max_active=2)
    cid = srv.add_class(gm, gpu.REQUEST_FLOW, p, rows, vals, gpu.DIRICHLET_SYMMETRIC, cfg)
    outs = [torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda") for _ in range(6)]
    ks = [_k(torch, m, q) for q in range(6)]
    ids = [srv.submit(cid, ks[q], 1e-10, outs[q]) for q in range(6)]
    peak = 0
    while True:
        r, qd = srv.progress()
        peak = max(peak, r)
        if (r, qd) == (0, 0):
            break
    assert 1 <= peak <= 2
    assert all(srv.result(i)["status"] == gpu.OK for i in ids)
    assert srv.info()["slots"] <= 2
    srv.close()
    # idle slots reserved beyond max_active do not raise the cap
    srv = gpu.Server(max_active=2)
    cid = srv.add_class(gm, gpu.REQUEST_FLOW, p, rows, vals, gpu.DIRICHLET_SYMMETRIC, cfg)
    srv.reserve(cid, 5)
    assert srv.info()["slots"] == 5
    ids = [srv.submit(cid, ks[q], 1e-10, outs[q]) for q in range(6)]
    peak = 0
    while True:
        r, qd = srv.progress()
        peak = max(peak, r)
        if (r, qd) == (0, 0):
            break
    assert 1 <= peak <= 2
    assert all(srv.result(i)["status"] == gpu.OK for i in ids)
    srv.close()
    # a budget that holds one slot only: requests run one after another
    srv = gpu.Server(max_active=8)
    cid = srv.add_class(gm, gpu.REQUEST_FLOW, p, rows, vals, gpu.DIRICHLET_SYMMETRIC, cfg)
    one = srv.info()
    srv.close()
    srv2 = gpu.Server(budget_bytes=1, max_active=8)
    cid = srv2.add_class(gm, gpu.REQUEST_FLOW, p, rows, vals, gpu.DIRICHLET_SYMMETRIC, cfg)
    rid = srv2.submit(cid, ks[0], 1e-10, outs[0])
    for _ in range(100):
        srv2.progress()
    assert srv2.result(rid)["state"] == 0  # nothing fits a 1-byte budget: stays queued
    srv2.close()
    del one


@pytest.mark.parametrize("policy", [True, False])
def test_server_serves_a_stalling_class_in_fp64(gpu, policy):
    """Steady heterogeneous 375 x 375 quads, where the FP32 recurrence stalls
    and the solve finishes in FP64 CG: with OGS_SERVER_PRECISION_FALLBACK the
    class's next request is solved in FP64 from the start; without it, in
    the FP32-inner mode again.  Heads within 1e-8 of an FP64 solve to 1e-13
    either way."""
    torch = pytest.importorskip("torch")
    m = M.structured_quad(375, 375)
    gm = gpu.GpuMesh(m)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, steady=1)
    cfg = gpu.solver_config(gpu.LS_CG, gpu.PRECOND_JACOBI, 20000, precision=gpu.PRECISION_FP32_REFINED)
    srv = gpu.Server(max_active=4, flags=gpu.SERVER_PRECISION_FALLBACK if policy else 0)
    cid = srv.add_class(gm, gpu.REQUEST_FLOW, p, rows, vals, gpu.DIRICHLET_SYMMETRIC, cfg)
    ks = [torch.tensor(fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 8.0, seed=3 + q), device="cuda")
          for q in range(2)]
    outs = [torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda") for _ in range(2)]
    res = []
    for q in range(2):
        rid = srv.submit(cid, ks[q], 1e-10, outs[q])
        srv.drain()
        res.append(srv.result(rid))
    assert all(r["status"] == gpu.OK for r in res)
    assert res[0]["precision"] == gpu.PRECISION_FP32_REFINED and res[0]["fp64_fallback"] == 1
    if policy:
        assert res[1]["precision"] == gpu.PRECISION_FP64 and res[1]["fp64_fallback"] == 0
        assert srv.info()["fp64_classes"] == 1
    else:
        assert res[1]["precision"] == gpu.PRECISION_FP32_REFINED
        assert srv.info()["fp64_classes"] == 0
    for q in range(2):
        x = _fp64_converged(gpu, gm, m, p, ks[q], rows, vals)
        assert rel_max_err(outs[q].cpu().numpy(), x) < 1e-8
    srv.close()
