"""Benchmark: transient GROUNDWATER_FLOW on a 128x128x64 hex mesh.

Workload (the configuration the solves/s metric is quoted on): 1,081,665
nodes, 1,048,576 linear hexes, element-wise ln K a seeded Gaussian random
field (mean ln 1e-5, variance 1, exponential covariance, correlation length
8 cells), Ss = 1e-4 1/m, 20 implicit-Euler steps of dt = 3600 s, heads 10 m
/ 0 m on the x faces (symmetric Dirichlet elimination), CG + Jacobi to a
1e-10 relative residual.  One step = one global assembly (27 Gauss points
per hex, FP64) + Dirichlet + one CG solve: one "solve".

Two solver paths are timed on the same steps:
  * the plain FP64 path (the parity path), and
  * the FP32-inner CG with FP64 residual replacement, whose heads are
    checked against the FP64 path step by step (max relative error
    reported; the metric is quoted at <= 1e-8).
`value` is the FP32-inner path with every input resident on the device;
`e2e` times the same steps through the C ABI with host buffers
(conductivity, previous heads and the initial guess copied in, heads copied
out every step).  The FP64 matrix (343 MB values + indices) is rebuilt every
step and is larger than L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU implementation of the path (the oracle, a C
restatement of the reference's own code) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY, NZ = 128, 128, 64
STEPS_TOTAL = 20
DT = 3600.0
SS = 1e-4
TOL = 1e-10
SEED = 2
WORKLOAD = ("transient GROUNDWATER_FLOW hex 128x128x64, lnK GRF var 1 ell 8, 20 steps dt 3600, "
            "CG+Jacobi 1e-10")

def make_deck(nx=NX, ny=NY, nz=NZ):
    from ogs5_gb300 import fields
    from ogs5_gb300 import mesh as M
    m = M.structured_hex(nx, ny, nz)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 8.0, seed=SEED)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf]).astype(np.int64)
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    h0 = np.zeros(m.n_nodes)
    h0[lf] = 10.0
    return m, ek, rows, vals, h0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev=0):
        self.dev = dev
        self.proc = None
        # raw samples in a temporary file; the summary goes into the JSON line
        fd, self.path = tempfile.mkstemp(prefix="ogs_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].strip() == "Active":
                    reasons.add(nm)
        load = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(rows)}


def measured_traffic(name: str):
    """DRAM bytes per launch from the committed ncu summary profiles/<name>."""
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith("dram_bytes_per_launch:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run_steps(eqs, capi, p, ek, rows, vals, h0, k_steps, host: bool, torch, stream, keep=False):
    """k_steps implicit-Euler steps from the initial heads h0; returns
    (elapsed ms, per-step ms, Krylov iterations, final heads, heads per step
    when keep)."""
    n = len(h0)
    if host:
        ek_b = torch.empty(len(ek), dtype=torch.float64, pin_memory=True).numpy()
        ek_b[:] = ek
        u = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        x = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        u[:] = h0
        rws, vls = rows, vals
    else:
        ek_b = torch.tensor(ek, device="cuda")
        u = torch.tensor(h0, device="cuda")
        x = torch.empty_like(u)
        rws = torch.tensor(rows, device="cuda")
        vls = torch.tensor(vals, device="cuda")
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(k_steps + 1)]
    iters = 0
    kept = []
    evs[0].record(stream)
    for k in range(k_steps):
        eqs.Initialize()
        eqs.GlobalAssembly(p, ek_b, u)
        eqs.SetKnownX(rws, vls, capi.DIRICHLET_SYMMETRIC)
        if host:
            x[:] = u
        else:
            x.copy_(u)
        iters += eqs.Solver(x)
        if host:
            u[:] = x
        else:
            u.copy_(x)
        evs[k + 1].record(stream)
        if keep:
            kept.append(x.copy() if host else x.clone())
    torch.cuda.synchronize()
    per = [evs[k].elapsed_time(evs[k + 1]) for k in range(k_steps)]
    heads = x.copy() if host else x.cpu().numpy()
    return evs[0].elapsed_time(evs[-1]), per, iters, heads, kept


def configure(eqs, capi, mixed: bool):
    if mixed:
        eqs.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 20000, TOL,
                           precision=capi.PRECISION_FP32_REFINED)
    else:
        eqs.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 20000, TOL)


def time_path(eqs, capi, p, deck, k_steps, warm, torch, stream, mixed, keep=False):
    """Warm-up steps, then the timed K steps with in-graph SpMV timing on."""
    m, ek, rows, vals, h0 = deck
    configure(eqs, capi, mixed)
    run_steps(eqs, capi, p, ek, rows, vals, h0, warm, False, torch, stream)
    eqs.profile(True)
    capi.kernel_launches(reset=True)
    ms, per, iters, heads, kept = run_steps(eqs, capi, p, ek, rows, vals, h0, k_steps, False, torch,
                                            stream, keep)
    launches = capi.kernel_launches(reset=True)
    prof = eqs.profile(False)
    return {"ms": ms, "per": per, "iters": iters, "heads": heads, "kept": kept,
            "launches": launches, "prof": prof}


class PortDeck:
    """The deck on the oracle's C restatement (the reference's algorithm,
    one thread): full element assembly (CFiniteElementStd::Assembly through
    GlobalAssembly), symmetric Dirichlet elimination and Linear_EQS::CG with
    Jacobi to 1e-10 -- one implicit-Euler step exactly as the GPU path takes
    it.  Built once per process (mesh, conductivities, sparsity pattern)."""

    def __init__(self, dims=(NX, NY, NZ)):
        from oracle import oracle as O
        O.build("/nonexistent")  # the prebuilt restatement only
        self.O = O
        self.m, self.ek, self.rows, self.vals, self.h0 = make_deck(*dims)
        self.rp, self.col = O.build_pattern(self.m.n_nodes, self.m.conn)
        self.p = O.make_params(pcs_type=0, dt=DT, storage=SS)
        self.b_norm = None

    def step(self, u):
        """One step from heads u: (new heads, CG iterations, assembly s, CG s)."""
        O = self.O
        t0 = time.perf_counter()
        val, b = O.assemble(self.m, self.rp, self.col, self.p, elem_k=self.ek, u0=u)
        O.dirichlet(self.rp, self.col, val, b, self.rows, self.vals, symmetric=True)
        t1 = time.perf_counter()
        x, info = O.solve(self.rp, self.col, val, b, u.copy(), method=5, precond=1, max_iter=20000, tol=TOL,
                          b_norm=self.b_norm)
        self.b_norm = info["b_norm"]  # Linear_EQS keeps |b| of the previous step for CheckNormRHS
        return x, info["iterations"], t1 - t0, time.perf_counter() - t1


def cpu_baseline_step():
    """One full step of the deck on one core (the oracle port): no sample,
    no extrapolation.  Returns (seconds, CG iterations, assembly s, CG s)."""
    d = PortDeck()
    t0 = time.perf_counter()
    _, its, t_asm, t_cg = d.step(d.h0.copy())
    return time.perf_counter() - t0, its, t_asm, t_cg


# ------------------------------------------------------------------
# Transport on the Kuhn-tet split of the deck (flow -> Darcy flux ->
# MASS_TRANSPORT with BiCGStab + ILU(0))
# ------------------------------------------------------------------
TRANSPORT_WORKLOAD = ("hex 128x128x64 split into 6 Kuhn tets (6,291,456 tets, 1,081,665 nodes), conductivity "
                      "of the parent hex; one transient flow step (CG + Jacobi, FP32 inner) -> Gauss-point "
                      "Darcy flux -> one MASS_TRANSPORT step (dt 3600 s, porosity 0.3, alpha_L/alpha_T "
                      "1.0/0.1 m, D 1e-9 m2/s, c = 1 on x = 0), BiCGStab 1e-10")


def transport_leg(capi, torch, steps=3):
    """One MASS_TRANSPORT step per measured step, ILU(0) and Jacobi."""
    from ogs5_gb300 import fields
    from ogs5_gb300 import mesh as M
    m = M.structured_tet(NX, NY, NZ)
    ek = torch.tensor(np.repeat(fields.lognormal_k((NX, NY, NZ), np.log(1e-5), 1.0, 8.0, seed=SEED), 6),
                      device="cuda")
    gm = capi.GpuMesh(m)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    # flow step from h0 (heads 10 / 0 on the x faces)
    flow = capi.LinearEQS(gm)
    flow.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 20000, TOL, precision=capi.PRECISION_FP32_REFINED)
    h0 = np.zeros(m.n_nodes)
    h0[lf] = 10.0
    h = torch.tensor(h0, device="cuda")
    flow.Initialize()
    flow.GlobalAssembly(capi.make_params(capi.GROUNDWATER_FLOW, dt=DT, storage=SS), ek, h)
    flow.SetKnownX(np.concatenate([lf, rf]), np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))]),
                   capi.DIRICHLET_SYMMETRIC)
    flow_it = flow.Solver(h)
    q = torch.empty((m.n_elements, gm.n_gauss, 3), dtype=torch.float64, device="cuda")
    flow.gp_velocity(capi.make_params(capi.GROUNDWATER_FLOW), ek, h, q)
    del flow
    p = capi.make_params(capi.MASS_TRANSPORT, dt=DT, porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=1e-9)
    mt = capi.LinearEQS(gm)
    c0 = torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda")
    rows = torch.tensor(lf, device="cuda")
    vals = torch.ones(len(lf), dtype=torch.float64, device="cuda")
    out = {"workload": TRANSPORT_WORKLOAD, "nodes": m.n_nodes, "elements": m.n_elements,
           "flow_fp32_iterations": flow_it}
    # $MEMORY_TYPE 1: the first assembly stores the operators, later ones
    # combine them (the flux field is the same every step here)
    p_mem = capi.make_params(capi.MASS_TRANSPORT, dt=DT, porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=1e-9,
                             memory_type=1)
    res = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    asm = {}
    for name, pp in (("element_kernel", p), ("stored_operators", p_mem)):
        ts = []
        for k in range(6):
            torch.cuda.synchronize()
            e0.record()
            mt.Initialize()
            mt.GlobalAssembly(pp, None, c0, q)
            e1.record()
            e1.synchronize()
            if k:  # the first stored-operator call fills the store
                ts.append(e0.elapsed_time(e1))
        asm[name] = round(statistics.median(ts), 3)
    out["assembly_ms"] = asm
    for name, pre, pp in (("ilu0", capi.PRECOND_ILU0, p), ("jacobi", capi.PRECOND_JACOBI, p),
                          ("jacobi_stored_operators", capi.PRECOND_JACOBI, p_mem)):
        mt.ConfigNumerics(capi.LS_BICGSTAB, pre, 5000, TOL, check_norm_rhs=False)
        times, its = [], []
        for k in range(steps + 1):
            x = c0.clone()
            torch.cuda.synchronize()
            e0.record()
            mt.Initialize()
            mt.GlobalAssembly(pp, None, c0, q)
            mt.SetKnownX(rows, vals, capi.DIRICHLET_ROW_ONLY)
            its.append(mt.Solver(x))
            e1.record()
            e1.synchronize()
            if k:  # the first step builds the graphs and factor buffers
                times.append(e0.elapsed_time(e1))
        st = mt.stats()
        res[name] = x
        out[name] = {"value": round(1e3 / statistics.median(times), 3), "unit": "solves/s",
                     "ms_per_step": round(statistics.median(times), 3), "iterations": its[-1],
                     "solve_ms": round(st["solve_ms"], 3), "rel_residual": st["rel_residual"]}
    out["max_rel_diff_ilu0_vs_jacobi"] = float((res["ilu0"] - res["jacobi"]).abs().max()
                                               / res["jacobi"].abs().max())
    out["max_rel_diff_stored_vs_jacobi"] = float((res["jacobi_stored_operators"] - res["jacobi"]).abs().max()
                                                 / res["jacobi"].abs().max())
    return out


# ------------------------------------------------------------------
# RICHARDS_FLOW: one Picard time step on the deck's hex box
# ------------------------------------------------------------------
RICH_SPACING = (0.25, 0.25, 0.0625)  # 32 m x 32 m x 4 m
RICH_WORKLOAD = ("RICHARDS_FLOW on hex 128x128x64 (1,081,665 nodes), 0.25 x 0.25 x 0.0625 m cells, ln k GRF "
                 "(mean ln 1e-12 m2, var 0.5, ell 4 cells), van Genuchten pb 5 kPa, m 0.55, Sr 0.08, Smax 0.98, "
                 "gravity; water table at mid-depth, top raised to -5 kPa; dt 3600 s; Picard ENORM 1 Pa; "
                 "CG + Jacobi 1e-10")


def richards_deck():
    from ogs5_gb300 import fields
    from ogs5_gb300 import mesh as M
    m = M.structured_hex(NX, NY, NZ, *RICH_SPACING)
    ek = fields.lognormal_k((NX, NY, NZ), np.log(1e-12), 0.5, 4.0, seed=SEED)
    depth = NZ * RICH_SPACING[2]
    p_old = 9810.0 * (0.5 * depth - m.z)  # hydrostatic, water table at mid-depth
    top = np.flatnonzero(m.z == m.z.max())
    bot = np.flatnonzero(m.z == m.z.min())
    rows = np.concatenate([top, bot])
    vals = np.concatenate([np.full(len(top), -5.0e3), p_old[bot]])
    return m, ek, p_old, rows, vals


RICH_MEDIUM = dict(capillary_model=4, permeability_model=4, pb=5.0e3, slr=0.08, slm=0.98, m=0.55, kr_slr=0.08,
                   kr_slm=0.98, kr_m=0.55, kr_min=1e-9)
RICH_FLUID = dict(dt=3600.0, storage=1e-6, porosity=0.35, drho_dp=4.4e-10, viscosity=1e-3, density=1000.0,
                  time_unit_factor=1.0, gravity=9.81, gravity_on=1)


def richards_leg(capi, torch, steps=2):
    """One Picard time step per measured step (the same step repeated from
    the same state), device time of the whole loop."""
    m, ek, p_old, rows, vals = richards_deck()
    gm = capi.GpuMesh(m)
    eqs = capi.LinearEQS(gm)
    eqs.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 20000, TOL, check_norm_rhs=False)
    p = capi.make_params(capi.RICHARDS_FLOW, **RICH_FLUID)
    r = capi.richards_params(**RICH_MEDIUM)
    ekd = torch.tensor(ek, device="cuda")
    pod = torch.tensor(p_old, device="cuda")
    rowsd = torch.tensor(rows, device="cuda")
    valsd = torch.tensor(vals, device="cuda")
    times, res = [], None
    for k in range(steps + 1):
        it = pod.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = eqs.RichardsStep(p, r, ekd, pod, it, rowsd, valsd, capi.DIRICHLET_SYMMETRIC, error_method=capi.ENORM,
                               max_iterations=40, tolerance=1.0)
        torch.cuda.synchronize()
        if k:  # the first step allocates and captures the solver graphs
            times.append((time.perf_counter() - t0) * 1e3)
    ms = statistics.median(times)
    return {"workload": RICH_WORKLOAD, "value": round(1e3 / ms, 3), "unit": "Picard time steps/s",
            "ms_per_step": round(ms, 3), "device_ms": round(res["solve_ms"], 3),
            "picard_iterations": res["iterations"], "linear_iterations": res["linear_iterations"],
            "final_error_over_tol": res["error"], "converged": res["converged"],
            "nodes": m.n_nodes, "elements": m.n_elements}


def richards_cpu_sample(picard_its):
    """One full Picard iteration of the Richards deck on one core by the
    oracle port (assembly of every hex at the iterate, symmetric Dirichlet,
    CG + Jacobi to 1e-10: the loop body of CRFProcess::ExecuteNonLinear),
    times the GPU run's Picard iterations per time step."""
    from oracle import oracle as O
    O.build("/nonexistent")
    m, ek, p_old, rows, vals = richards_deck()
    op = O.make_params(pcs_type=3, **RICH_FLUID)
    r = O.richards_params(**RICH_MEDIUM)
    rp, col = O.build_pattern(m.n_nodes, m.conn)
    t0 = time.perf_counter()
    _, info = O.richards_picard(m, rp, col, op, r, ek, p_old, p_old, rows, vals, True, error_method=2,
                                tolerance=1.0, max_iterations=1, method=5, precond=1, max_iter=20000, tol=TOL)
    t_it = time.perf_counter() - t0
    return {"value": round(1.0 / (picard_its * t_it), 6), "unit": "Picard time steps/s", "cores": 1, "kind": "port",
            "sample": f"one full Picard iteration on one core by the oracle port: assembly of {m.n_elements} hexes "
                      f"at the iterate, Dirichlet, CG + Jacobi to {TOL:g} ({info['linear']} iterations), "
                      f"{t_it:.2f} s, times the {picard_its} Picard iterations of the GPU run's time step"}


# ------------------------------------------------------------------
# Monte-Carlo batch (512 steady realisations of uneven size)
# ------------------------------------------------------------------
BATCH_REALS = 512
BATCH_SEED = 4
# Both arms of the batch comparison stop at 1e-11: at 1e-10 the FP64 path's
# own heads on these steady boxes are up to 2.5e-8 from an FP64 solve to
# 1e-13, so no path can be held to 1e-8 of it; at 1e-11 both are within
# 3e-9 of that reference and of each other.
BATCH_TOL = 1e-11
BATCH_WORKLOAD = ("512 steady GROUNDWATER_FLOW realisations, hex boxes n^3 nodes with n ~ U{24..96}, "
                  "lnK GRF mean ln 1e-5, var ~ U(0.5, 2), ell ~ U(4, 16) cells, heads 10/0 m on the x faces, "
                  "Jacobi-CG (1e-11 in both arms)")


def batch_deck(torch, n_real=BATCH_REALS, n_lo=24, n_hi=96, seed=BATCH_SEED):
    """Realisation sizes and conductivity fields (generated on the GPU)."""
    from ogs5_gb300 import fields
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_lo, n_hi + 1, n_real)
    var = rng.uniform(0.5, 2.0, n_real)
    ell = rng.uniform(4.0, 16.0, n_real)
    ks = [fields.lognormal_k_device((n - 1, n - 1, n - 1), np.log(1e-5), float(v), float(e),
                                    seed=seed * 100000 + q)
          for q, (n, v, e) in enumerate(zip(ns, var, ell))]
    return [int(n) for n in ns], ks


def batch_plain_fp64(capi, torch, ns, ks, heads_batch, tol):
    """Each realisation through the plain FP64 single-system path (element
    assembly, symmetric Dirichlet, FP64 Jacobi-CG to tol): device time of
    assembly + Dirichlet + solve per realisation.  Errors: the batch heads
    against these, and both against an FP64 solve of the same system to
    1e-13 (untimed), the FP64 reference."""
    from ogs5_gb300 import mesh as M
    order = sorted(range(len(ns)), key=lambda q: ns[q])
    times = [0.0] * len(ns)
    iters = [0] * len(ns)
    err = err_b_ref = err_p_ref = 0.0
    p = capi.make_params(capi.GROUNDWATER_FLOW, steady=1)
    cur_n, eqs, mesh_obj = None, None, None
    stream = torch.cuda.current_stream()
    for q in order:
        n = ns[q]
        if n != cur_n:
            eqs = None
            m = M.structured_hex(n - 1, n - 1, n - 1)
            gm = capi.GpuMesh(m)
            eqs = capi.LinearEQS(gm, stream=stream.cuda_stream)
            eqs.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 20000, tol)
            lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
            rows = torch.tensor(np.concatenate([lf, rf]), device="cuda")
            vals = torch.tensor(np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))]), device="cuda")
            x0 = torch.zeros(m.n_nodes, dtype=torch.float64, device="cuda")
            x0[rows[: len(lf)]] = 10.0
            u0 = torch.zeros_like(x0)
            cur_n = n
        x = x0.clone()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eqs.Initialize()
        eqs.GlobalAssembly(p, ks[q], u0)
        eqs.SetKnownX(rows, vals, capi.DIRICHLET_SYMMETRIC)
        iters[q] = eqs.Solver(x)
        e1.record(stream)
        e1.synchronize()
        times[q] = e0.elapsed_time(e1)
        hb = torch.from_numpy(heads_batch[q]).cuda()
        err = max(err, float((hb - x).abs().max() / x.abs().max()))
        # FP64 reference: same system, CG to 1e-13 (CheckNormRHS off: same b)
        eqs.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 40000, 1e-13, check_norm_rhs=False)
        xr = x.clone()
        eqs.Solver(xr)
        eqs.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 20000, tol)
        nr = float(xr.abs().max())
        err_b_ref = max(err_b_ref, float((hb - xr).abs().max()) / nr)
        err_p_ref = max(err_p_ref, float((x - xr).abs().max()) / nr)
    return times, iters, err, err_b_ref, err_p_ref


def batch_leg(capi, torch, steps=2, n_real=BATCH_REALS, n_hi=96, plain=True, tol=BATCH_TOL):
    """Config: 512 realisations in one persistent launch per batch solve."""
    ns, ks = batch_deck(torch, n_real=n_real, n_hi=n_hi)
    reals = [(n, n, n, k, 10.0, 0.0) for n, k in zip(ns, ks)]
    b = capi.Batch(reals, tol=tol, max_iter=20000)
    k_all = torch.cat(ks)
    tune = b.autotune()
    b.solve()  # warm-up
    torch.cuda.synchronize()
    # device-resident: conductivities already on the device
    t_dev, stats = [], None
    for _ in range(steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        b.set_k(k_all)
        stats = b.solve()
        e1.record()
        e1.synchronize()
        t_dev.append(e0.elapsed_time(e1))
    # end to end: conductivities from pinned host memory, heads back to pinned host memory
    k_host = torch.empty(k_all.numel(), dtype=torch.float64, pin_memory=True)
    k_host.copy_(k_all)
    h_host = torch.empty(b.rows, dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.set_k(k_host)
    b.solve()
    b.heads_flat(h_host.numpy())
    t_e2e = (time.perf_counter() - t0) * 1e3
    heads = np.split(h_host.numpy().copy(), np.cumsum(b.sizes)[:-1])
    ms = statistics.median(t_dev)
    fin = [s["finish_ms"] for s in stats]
    it = [s["iterations"] for s in stats]
    rf = [s["refinements"] for s in stats]
    rows = np.array(b.sizes, dtype=np.float64)
    # algorithmic bytes: an FP32 CG step moves 116 B per row (14 FP32
    # operator values, u, w, r and the vector update: read u w p s x r d,
    # write p s x r u); a residual replacement 180 B per row (14 FP64
    # operator values, x64, x32, b, r64 and the restart sweep); the assembly
    # writes 14 x 12 B of operator per row plus 8 vectors and reads K
    bytes_alg = float((rows * (116.0 * np.array(it) + 180.0 * np.array(rf) + 14 * 12 + 44)).sum())
    bytes_alg += 8.0 * b.elements
    hbm, _ = peaks()
    gbs = bytes_alg / (ms * 1e-3) / 1e9
    out = {"workload": BATCH_WORKLOAD if n_real == BATCH_REALS else f"{n_real} realisations, n <= {n_hi}",
           "realisations": n_real, "rows": b.rows, "elements": b.elements,
           "value": round(n_real / (ms * 1e-3), 3), "unit": "solves/s", "ms_per_batch": round(ms, 3),
           "dof_per_s": round(b.rows / (ms * 1e-3), 1),
           "p50_latency_ms": round(float(np.percentile(fin, 50)), 3),
           "p99_latency_ms": round(float(np.percentile(fin, 99)), 3),
           "latency": "device time from the start of the batch launch to each realisation's convergence",
           "fp32_iterations_total": int(sum(it)), "replacements_total": int(sum(rf)),
           "launches_per_batch": 1, "tuning": tune,
           "hbm": {"achieved_gbs": round(gbs, 1), "peak": hbm, "frac": round(gbs / hbm, 4),
                   "bytes": "116 B per row per FP32 CG step, 180 B per row per FP64 replacement, "
                            "assembly 212 B per row + 8 B per element"},
           "e2e": {"value": round(n_real / (t_e2e * 1e-3), 3), "unit": "solves/s",
                   "h2d_bytes_per_step": 8 * b.elements, "d2h_bytes_per_step": 8 * b.rows}}
    out["tol"] = tol
    if plain:
        times, its64, err, err_b_ref, err_p_ref = batch_plain_fp64(capi, torch, ns, ks, heads, tol)
        t64 = sum(times)
        out["fp64_path"] = {"value": round(n_real / (t64 * 1e-3), 3), "unit": "solves/s",
                            "ms_total": round(t64, 3), "cg_iterations_total": int(sum(its64)),
                            "how": "each realisation through GpuMesh/LinearEQS: assembly + symmetric "
                                   f"Dirichlet + FP64 Jacobi-CG {tol:g}, device time summed"}
        out["speedup_vs_fp64_path"] = round(out["value"] / out["fp64_path"]["value"], 3)
        out["max_rel_err_vs_fp64"] = err
        out["max_rel_err_vs_fp64_reference"] = err_b_ref
        out["fp64_path"]["max_rel_err_vs_fp64_reference"] = err_p_ref
    b.close()
    return out


# ------------------------------------------------------------------
# Serving: Poisson arrivals of flow and transport requests
# ------------------------------------------------------------------
SERVE_RATE = 200.0        # requests per second
SERVE_REQUESTS = 400
SERVE_SEED = 5
SERVE_DOF = (1e4, 2e6)
SERVE_CLASSES = 5         # log-spaced size classes per mesh type (meshes are cached)
SERVE_WARM_SLOTS = 4      # slots per class created before the timed run
# requests in flight at most, and the scheduling policy: smallest class first
# at admission, higher stream priority for smaller classes (measured on 400
# requests: p50 267 ms against 508 ms for arrival order with 128 in flight,
# the same throughput)
SERVE_MAX_ACTIVE = 16
# capi.SERVER_PRIORITY | SERVER_SJF | SERVER_BATCH | SERVER_PRECISION_FALLBACK
SERVE_FLAGS = 15
SERVE_WORKLOAD = ("Poisson arrivals 200/s of flow (steady GWF, heads 10/0 m on the x faces) and transport "
                  "(one MASS_TRANSPORT step, flux from a linear head field) requests on quad, hex and "
                  "hex-split-tet meshes, 1e4-2e6 DOF log-uniform (5 size classes per type), log-normal K "
                  "per request, tol 1e-6 or 1e-10")


def serve_meshes(n_classes=SERVE_CLASSES):
    """Mesh of every (type, size class): quad n x n cells, hex and tet n^3 cells."""
    from ogs5_gb300 import mesh as M
    dofs = np.geomspace(SERVE_DOF[0], SERVE_DOF[1], n_classes)
    out = {}
    for t in ("quad", "hex", "tet"):
        for c, d in enumerate(dofs):
            if t == "quad":
                n = max(4, int(round(np.sqrt(d))) - 1)
                out[(t, c)] = M.structured_quad(n, n)
            else:
                n = max(3, int(round(np.cbrt(d))) - 1)
                out[(t, c)] = M.structured_hex(n, n, n) if t == "hex" else M.structured_tet(n, n, n)
    return dofs, out


def serve_requests(torch, dofs, meshes, n_req=SERVE_REQUESTS, rate=SERVE_RATE, seed=SERVE_SEED):
    from ogs5_gb300 import fields
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    reqs = []
    for q in range(n_req):
        t = ("quad", "hex", "tet")[rng.integers(3)]
        d = np.exp(rng.uniform(np.log(SERVE_DOF[0]), np.log(SERVE_DOF[1])))
        c = int(np.argmin(np.abs(np.log(dofs) - np.log(d))))
        kind = int(rng.integers(2))
        tol = 1e-6 if rng.integers(2) else 1e-10
        m = meshes[(t, c)]
        var = float(rng.uniform(0.5, 1.5))
        k = fields.lognormal_k_device(m.shape, np.log(1e-5), var, 8.0, seed=seed * 100000 + q)
        if k.numel() != m.n_elements:  # tets: the field of the parent hex
            k = k.repeat_interleave(m.n_elements // k.numel())
        reqs.append({"t": float(arrivals[q]), "key": (t, c), "kind": kind, "tol": tol, "k": k})
    return reqs


def serve_class_setup(capi, m, kind):
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    if kind == 0:
        rows = np.concatenate([lf, rf])
        vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
        p = capi.make_params(capi.GROUNDWATER_FLOW, steady=1)
        return rows, vals, capi.DIRICHLET_SYMMETRIC, p, None, None
    p = capi.make_params(capi.MASS_TRANSPORT, dt=3600.0, porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=1e-9)
    head = 10.0 * (1.0 - m.x / m.x.max())
    return lf, np.ones(len(lf)), capi.DIRICHLET_ROW_ONLY, p, capi.make_params(capi.GROUNDWATER_FLOW), head


def _serve_breakdown(reqs, res):
    """Per mesh type and request kind: requests, mean solver iterations and
    the summed per-request solve time (overlapping requests each count)."""
    out = {}
    for r, x in zip(reqs, res):
        g = out.setdefault(f"{r['key'][0]}-{'flow' if r['kind'] == 0 else 'mt'}", [0, 0, 0.0])
        g[0] += 1
        g[1] += x["iterations"]
        g[2] += x["solve_ms"]
    return {k: {"requests": n, "mean_iterations": round(it / n, 1), "sum_solve_ms": round(ms, 1)}
            for k, (n, it, ms) in sorted(out.items())}


def serve_leg(capi, torch, n_req=SERVE_REQUESTS, flags=None, max_active=None, plain=True):
    t_setup = time.perf_counter()
    dofs, meshes = serve_meshes()
    gms = {key: capi.GpuMesh(m) for key, m in meshes.items()}
    reqs = serve_requests(torch, dofs, meshes, n_req=n_req)
    print(f"serve: meshes and fields {time.perf_counter() - t_setup:.1f} s", file=sys.stderr)
    flags = SERVE_FLAGS if flags is None else flags
    max_active = SERVE_MAX_ACTIVE if max_active is None else max_active
    srv = capi.Server(max_active=max_active, flags=flags)
    cls = {}
    for key, m in meshes.items():
        for kind in (0, 1):
            rows, vals, mode, p, fp, head = serve_class_setup(capi, m, kind)
            cfg = (capi.solver_config(capi.LS_CG, capi.PRECOND_JACOBI, 20000,
                                      precision=capi.PRECISION_FP32_REFINED) if kind == 0 else
                   capi.solver_config(capi.LS_BICGSTAB, capi.PRECOND_JACOBI, 5000))
            cls[(key, kind)] = srv.add_class(gms[key], kind, p, rows, vals, mode, cfg, flow_params=fp,
                                             flow_head=head)
    outs = [torch.zeros(meshes[r["key"]].n_nodes, dtype=torch.float64, device="cuda") for r in reqs]
    # warm-up: SERVE_WARM_SLOTS slots reserved for every class and as many
    # requests of it served, so each class starts with slots whose buffers
    # and graphs exist
    warm_out = []
    for (key, kind), cid in cls.items():
        k = next((r["k"] for r in reqs if r["key"] == key), None)
        if k is None:
            continue
        srv.reserve(cid, SERVE_WARM_SLOTS)
        for _ in range(SERVE_WARM_SLOTS):
            warm_out.append(torch.zeros(meshes[key].n_nodes, dtype=torch.float64, device="cuda"))
            srv.submit(cid, k, 1e-6, warm_out[-1])
    srv.drain()
    del warm_out
    torch.cuda.synchronize()
    print(f"serve: warm-up done {time.perf_counter() - t_setup:.1f} s", file=sys.stderr)
    # served run in real time
    ids = []
    t0 = time.perf_counter()
    for q, r in enumerate(reqs):
        while time.perf_counter() - t0 < r["t"]:
            srv.progress()
        ids.append(srv.submit(cls[(r["key"], r["kind"])], r["k"], r["tol"], outs[q]))
        srv.progress()
    srv.drain()
    makespan = time.perf_counter() - t0
    res = [srv.result(i) for i in ids]
    lat = [x["latency_ms"] for x in res]
    ok = sum(1 for x in res if x["status"] == capi.OK)
    fails = {}
    for r, x in zip(reqs, res):
        if x["status"] != capi.OK:
            key = f"{r['key'][0]}{r['key'][1]}-{'flow' if r['kind'] == 0 else 'mt'}-{r['tol']:g}-s{x['status']}"
            fails[key] = fails.get(key, 0) + 1
    info = srv.info()
    served = {"value": round(n_req / makespan, 3), "unit": "solves/s",
              "p50_latency_ms": round(float(np.percentile(lat, 50)), 3),
              "p99_latency_ms": round(float(np.percentile(lat, 99)), 3),
              "ok": ok, "failed": fails, "slots": info["slots"], "hbm_bytes_used": info["bytes_used"]}
    policy = {"max_active": max_active, "priority_streams": bool(flags & capi.SERVER_PRIORITY),
              "admission": "smallest class first" if flags & capi.SERVER_SJF else "arrival order",
              "dynamic_batching": bool(flags & capi.SERVER_BATCH),
              "fp64_after_fp32_fallback": bool(flags & capi.SERVER_PRECISION_FALLBACK),
              "fp32_internal_tol": "a tenth of the request's tolerance"}
    served["batched"] = info["batched"]
    served["fp64_classes"] = info["fp64_classes"]
    served["by_kind"] = _serve_breakdown(reqs, res)
    srv.close()
    if not plain:
        return {"requests": n_req, "served": served, "policy": policy}
    # plain FP64 path: the same arrivals replayed in real time through a
    # server that admits one request at a time (FIFO, no batching) on the
    # FP64 single-system solvers (CG / BiCGStab + Jacobi)
    srv64 = capi.Server(max_active=1, flags=0)
    cls64 = {}
    for key, m in meshes.items():
        for kind in (0, 1):
            rows, vals, mode, p, fp, head = serve_class_setup(capi, m, kind)
            cfg = (capi.solver_config(capi.LS_CG, capi.PRECOND_JACOBI, 20000) if kind == 0 else
                   capi.solver_config(capi.LS_BICGSTAB, capi.PRECOND_JACOBI, 5000))
            cls64[(key, kind)] = srv64.add_class(gms[key], kind, p, rows, vals, mode, cfg, flow_params=fp,
                                                 flow_head=head)
    outs64 = [torch.zeros(meshes[r["key"]].n_nodes, dtype=torch.float64, device="cuda") for r in reqs]
    warm64 = []
    for (key, kind), cid in cls64.items():  # one warm slot per class
        k = next((r["k"] for r in reqs if r["key"] == key), None)
        if k is not None:
            warm64.append(torch.zeros(meshes[key].n_nodes, dtype=torch.float64, device="cuda"))
            srv64.submit(cid, k, 1e-6, warm64[-1])
            srv64.drain()
    torch.cuda.synchronize()
    ids64 = []
    t0 = time.perf_counter()
    for q, r in enumerate(reqs):
        while time.perf_counter() - t0 < r["t"]:
            srv64.progress()
        ids64.append(srv64.submit(cls64[(r["key"], r["kind"])], r["k"], r["tol"], outs64[q]))
        srv64.progress()
    srv64.drain()
    makespan64 = time.perf_counter() - t0
    res64 = [srv64.result(i) for i in ids64]
    lat64 = [x["latency_ms"] for x in res64]
    srv64.close()
    fp64 = {"value": round(n_req / makespan64, 3), "unit": "solves/s",
            "p50_latency_ms": round(float(np.percentile(lat64, 50)), 3),
            "p99_latency_ms": round(float(np.percentile(lat64, 99)), 3),
            "ok": sum(1 for x in res64 if x["status"] == capi.OK),
            "by_kind": _serve_breakdown(reqs, res64),
            "how": "same arrivals replayed in real time, one request at a time (FIFO), FP64 CG / BiCGStab + "
                   "Jacobi on the single-system solvers"}
    # accuracy: every served result against an FP64 solve of its system to
    # 1e-13 (converged), and against the FP64 path's result at its tolerance
    eqs_by = {}
    err_conv = {1e-6: 0.0, 1e-10: 0.0}
    err_path = {1e-6: 0.0, 1e-10: 0.0}
    worst = []
    for q, r in enumerate(reqs):
        key, kind = r["key"], r["kind"]
        m = meshes[key]
        if (key, kind) not in eqs_by:
            e = capi.LinearEQS(gms[key])
            rows, vals, mode, p, fp, head = serve_class_setup(capi, m, kind)
            x0 = np.zeros(m.n_nodes)
            x0[rows] = vals
            eqs_by[(key, kind)] = (e, mode, p, fp, None if head is None else torch.tensor(head, device="cuda"),
                                   torch.tensor(x0, device="cuda"), torch.tensor(rows, device="cuda"),
                                   torch.tensor(vals, device="cuda"))
        e, mode, p, fp, head, x0, rows_d, vals_d = eqs_by[(key, kind)]
        e.Initialize()
        if kind == 0:
            e.ConfigNumerics(capi.LS_CG, capi.PRECOND_JACOBI, 40000, 1e-13, check_norm_rhs=False)
            e.GlobalAssembly(p, r["k"], x0)
        else:
            e.ConfigNumerics(capi.LS_BICGSTAB, capi.PRECOND_JACOBI, 10000, 1e-13, check_norm_rhs=False)
            qbuf = torch.empty((m.n_elements, gms[key].n_gauss, 3), dtype=torch.float64, device="cuda")
            e.gp_velocity(fp, r["k"], head, qbuf)
            e.GlobalAssembly(p, None, x0, qbuf)
        e.SetKnownX(rows_d, vals_d, mode)
        x = x0.clone()
        e.Solver(x, allow_fail=True)
        scale = float(x.abs().max())
        ec = float((outs[q] - x).abs().max()) / scale
        ep = float((outs[q] - outs64[q]).abs().max()) / scale
        if res[q]["status"] == capi.OK:
            err_conv[r["tol"]] = max(err_conv[r["tol"]], ec)
            err_path[r["tol"]] = max(err_path[r["tol"]], ep)
        worst.append((ec, f"{r['key'][0]}{r['key'][1]}-{'flow' if r['kind'] == 0 else 'mt'}-{r['tol']:g}",
                      res[q]["status"], res[q]["iterations"], res[q]["batch_size"]))
    return {"workload": SERVE_WORKLOAD, "requests": n_req, "rate_per_s": SERVE_RATE,
            "classes": len(cls), "served": served, "policy": policy, "fp64_path": fp64,
            "speedup_vs_fp64_path": round(served["value"] / fp64["value"], 3),
            "max_rel_err_vs_fp64_converged": {"tol_1e-6": err_conv[1e-6], "tol_1e-10": err_conv[1e-10]},
            "max_rel_err_vs_fp64_path": {"tol_1e-6": err_path[1e-6], "tol_1e-10": err_path[1e-10]},
            "error_how": "served heads against an FP64 solve of the same system to |r|/|b| < 1e-13 "
                         "(converged), and against the FP64 path's heads at the request's tolerance",
            "worst": sorted(worst, reverse=True)[:8],
            "served_value": served["value"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=STEPS_TOTAL)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--path", default="both", choices=["both", "fp64", "mixed", "batch", "serve", "transport", "richards"],
                    help="fp64 / mixed / batch: time one path only (profiling driver)")
    ap.add_argument("--batch-reals", type=int, default=BATCH_REALS)
    ap.add_argument("--batch-max-n", type=int, default=96)
    ap.add_argument("--batch-tol", type=float, default=BATCH_TOL)
    ap.add_argument("--batch-plain", action="store_true", help="--path batch: also time the FP64 path")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-transport", action="store_true")
    ap.add_argument("--no-richards", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=SERVE_REQUESTS)
    ap.add_argument("--serve-flags", type=int, default=None)
    ap.add_argument("--serve-max-active", type=int, default=None)
    ap.add_argument("--serve-no-plain", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return reference_arm(args, rank)

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from ogs5_gb300 import build as B
    B.build()
    from ogs5_gb300 import capi

    if args.path == "richards":
        import torch
        from ogs5_gb300 import capi
        print(json.dumps(richards_leg(capi, torch, steps=max(1, args.steps))))
        return
    if args.path == "transport":
        from ogs5_gb300 import capi
        print(json.dumps(transport_leg(capi, torch, steps=max(1, args.steps))))
        return
    if args.path == "serve":
        from ogs5_gb300 import capi
        print(json.dumps(serve_leg(capi, torch, n_req=args.serve_requests, flags=args.serve_flags,
                                   max_active=args.serve_max_active, plain=not args.serve_no_plain)))
        return
    if args.path == "batch":
        from ogs5_gb300 import capi
        print(json.dumps(batch_leg(capi, torch, steps=max(1, args.steps), n_real=args.batch_reals,
                                   n_hi=args.batch_max_n, plain=args.batch_plain, tol=args.batch_tol)))
        return
    deck = make_deck()
    m, ek, rows, vals, h0 = deck
    stream = torch.cuda.Stream()
    gm = capi.GpuMesh(m)
    eqs = capi.LinearEQS(gm, stream=stream)
    p = capi.make_params(capi.GROUNDWATER_FLOW, dt=DT, storage=SS)
    k_steps = max(1, args.steps)
    warm = max(3, args.warmup)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        dist.barrier()

    if args.path != "both":
        # one path only: warm-up steps, then the timed steps (ncu driver)
        r = time_path(eqs, capi, p, deck, k_steps, warm, torch, stream, mixed=args.path == "mixed")
        pr = r["prof"]
        print(json.dumps({"path": args.path, "solves_per_s": round(k_steps / (r["ms"] * 1e-3), 4),
                          "ms_per_step": round(r["ms"] / k_steps, 3), "iterations": r["iters"],
                          "spmv_ms": round(pr["spmv_ms"] / max(1, pr["spmv_launches"]), 5)}))
        return

    # plain FP64 path (the parity path), then the FP32-inner / FP64 path
    f64 = time_path(eqs, capi, p, deck, k_steps, warm, torch, stream, mixed=False, keep=True)
    with ClockSampler(local) as clk:
        mix = time_path(eqs, capi, p, deck, k_steps, warm, torch, stream, mixed=True, keep=True)
    err = max(float((a - b).abs().max() / b.abs().max()) for a, b in zip(mix["kept"], f64["kept"]))
    f64["kept"] = mix["kept"] = None
    torch.cuda.empty_cache()
    # end to end through the C ABI with host buffers (FP32-inner path)
    configure(eqs, capi, True)
    ms_e2e, per_e2e, it_e2e, heads_e2e, _ = run_steps(eqs, capi, p, ek, rows, vals, h0, k_steps, True,
                                                      torch, stream)
    ms, ms_e2e, f64["ms"] = replica_times([mix["ms"], ms_e2e, f64["ms"]], world)

    N, nnz = gm.n_rows, gm.nnz
    cfg = deck_config(world)
    assert (cfg["nodes"], cfg["elements"], cfg["nnz"]) == (N, m.n_elements, nnz)
    hbm, peak_kind = peaks()
    pr = mix["prof"]
    t_spmv = pr["spmv_ms"] / max(1, pr["spmv_launches"])
    # per row: the 13 stored upper off-diagonal values of the 27-point hex
    # pattern (the Jacobi-scaled operator's unit diagonal is not stored),
    # the iterate r (4 B) and the product w (4 B)
    n_vals = 13
    spmv_bytes = (4 * n_vals + 8) * N
    achieved = spmv_bytes / (t_spmv * 1e-3) / 1e9
    pr64 = f64["prof"]
    t64 = pr64["spmv_ms"] / max(1, pr64["spmv_launches"])
    b64 = nnz * 12 + N * 20
    value = job_rate(world, k_steps, ms)
    value64 = job_rate(world, k_steps, f64["ms"])
    e2e = job_rate(world, k_steps, ms_e2e)
    h2d = 8 * m.n_elements + 8 * N * 2 + 12 * len(rows)
    d2h = 8 * N
    out = {
        "metric": "solves/s", "value": round(value, 4), "unit": "solves/s", "n_gpus": world,
        "steps": k_steps, "warmup": warm, "ms_per_step": round(ms / k_steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 inner CG, f64 residual/solution/convergence",
        "data": "synthetic (seeded GRF conductivity, generated mesh)",
        "config": cfg,
        "p50_step_ms": round(float(np.percentile(mix["per"], 50)), 3),
        "p99_step_ms": round(float(np.percentile(mix["per"], 99)), 3),
        "max_rel_err_vs_fp64": err,
        "krylov_iterations": mix["iters"], "dof_per_s": round(value * N, 1),
        "fp64_path": {"value": round(value64, 4), "unit": "solves/s",
                      "ms_per_step": round(f64["ms"] / k_steps, 3), "cg_iterations": f64["iters"],
                      "spmv": {"kernel": "k_cg_spmv (SELL-32 FP64 + fused p.s)",
                               "launch_ms": round(t64, 4), "bytes_per_launch": b64,
                               "achieved_gbs": round(b64 / (t64 * 1e-3) / 1e9, 1)}},
        "speedup_vs_fp64_path": round(value / value64, 3),
        "e2e": {"value": round(e2e, 4), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "e2e_heads_match": bool(np.abs(heads_e2e - mix["heads"]).max()
                                <= 1e-8 * np.abs(mix["heads"]).max()),
        "gpu_launches": int(mix["launches"]),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4),
                     "traffic": measured_traffic("k_mp_spmv_lines_hex128x128x64.md"),
                     "kernel": "k_mp_spmv_lines (FP32 Jacobi-scaled upper-diagonal-offset SpMV of the 27-point "
                               "lattice, four rows per thread from 16-byte windows, unit diagonal, + fused dots)",
                     "bytes_per_launch": spmv_bytes, "launch_ms": round(t_spmv, 5),
                     "launches": pr["spmv_launches"], "peak_kind": peak_kind},
        "clocks": clk.summary(),
    }
    if not args.no_transport:
        out["transport"] = transport_leg(capi, torch)
    if not args.no_richards:
        out["richards"] = richards_leg(capi, torch)
    if not args.no_serve:
        out["serve"] = serve_leg(capi, torch, n_req=args.serve_requests)
    if not args.no_batch:
        out["batch"] = batch_leg(capi, torch, n_real=args.batch_reals, n_hi=args.batch_max_n,
                                 tol=args.batch_tol)
    if rank == 0 and not args.no_cpu_baseline:
        t_step, its, t_asm, t_cg = cpu_baseline_step()
        out["cpu_baseline"] = {"value": round(1.0 / t_step, 6), "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": (f"one full step of the deck (the first, from the initial heads) on one "
                                          f"core by the oracle C port: assembly of {m.n_elements} hexes + "
                                          f"Dirichlet {t_asm:.2f} s, CG + Jacobi to {TOL:g} {its} iterations "
                                          f"{t_cg:.2f} s")}
        if "richards" in out:
            rr = out["richards"]
            rr["cpu_baseline"] = richards_cpu_sample(rr["picard_iterations"])
    if rank == 0:
        print(json.dumps(out))


def hex_pattern_nnz(nx, ny, nz):
    """Stored entries of the 27-point pattern of an nx x ny x nz hex lattice:
    per axis, (n + 1) nodes couple to 3 each except the 2 end nodes."""
    return (3 * nx + 1) * (3 * ny + 1) * (3 * nz + 1)


def replica_times(times, world):
    """Each timing (ms) as the maximum over the ranks, on every rank: with
    one replica per GPU and no exchange between them, the job takes as long
    as its slowest replica.  A barrier follows, so no rank prints before all
    have timed."""
    if world <= 1:
        return list(times)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(times), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return [float(v) for v in t]


def job_rate(world, steps, ms):
    """Whole-job solves/s: each of the world replicas did steps solves
    within ms milliseconds."""
    return world * steps / (ms * 1e-3)


def deck_config(world=1):
    """The workload's `config`, the same dict in both arms."""
    return {"workload": WORKLOAD, "nodes": (NX + 1) * (NY + 1) * (NZ + 1), "elements": NX * NY * NZ,
            "nnz": hex_pattern_nnz(NX, NY, NZ),
            "l2": "inputs larger than L2 (FP64 matrix 343 MB re-assembled every step), no flush",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def _split(total, workers):
    q, r = divmod(total, workers)
    return [q + (1 if i < r else 0) for i in range(workers)]


def _reference_binary():
    """The reference's own executable (oracle/_ref/ogs_sp, built from its
    sources) when it exists and was built for this host's architecture."""
    path = os.path.join(ROOT, "oracle", "_ref", "ogs_sp")
    if not os.access(path, os.X_OK):
        return None
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return None
    machine = {62: "x86_64", 183: "aarch64"}.get(int.from_bytes(head[18:20], "little"))
    return path if head[:4] == b"\x7fELF" and machine == platform.machine() else None


def _port_worker(widx, n_warm, n_timed, barrier, q, dims):
    """One process of the reference arm on the port: setup, its warm-up
    steps, then its share of the timed steps (from the initial heads)."""
    try:
        d = PortDeck(dims)
        barrier.wait(timeout=1800)
        u = d.h0.copy()
        for _ in range(n_warm):
            u = d.step(u)[0]
        barrier.wait(timeout=1800)
        d.b_norm = None
        u = d.h0.copy()
        its = []
        t0 = time.perf_counter()
        for _ in range(n_timed):
            u, it, _, _ = d.step(u)
            its.append(it)
        q.put((widx, t0, time.perf_counter(), its, None))
    except BaseException as e:  # report, and release the others from the barrier
        try:
            barrier.abort()
        except Exception:
            pass
        q.put((widx, 0.0, 0.0, [], repr(e)))


def _run_port(workers, warm, timed, dims=(NX, NY, NZ)):
    import multiprocessing as mp
    import queue as Q
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(workers)
    q = ctx.Queue()
    procs = [ctx.Process(target=_port_worker, args=(i, warm[i], timed[i], barrier, q, dims))
             for i in range(workers)]
    for pr in procs:
        pr.start()
    res = []
    try:
        for _ in procs:
            res.append(q.get(timeout=3600))
    except Q.Empty:
        res.append((-1, 0.0, 0.0, [], "a worker did not report"))
    for pr in procs:
        pr.join(timeout=60)
        if pr.is_alive():
            pr.kill()
    errs = [r[4] for r in res if r[4]]
    if errs:
        raise RuntimeError("reference arm worker failed: " + errs[0])
    wall = max(r[2] for r in res) - min(r[1] for r in res)
    its = [it for r in res for it in r[3]]
    return wall, its


def _run_binary(binary, workers, warm, timed):
    """The reference executable, one process per worker on its own copy of
    the deck running its warm-up + timed steps; the timed span of a worker
    runs from the assembly of its first timed step to the acceptance of its
    last (the reference's own stdout markers)."""
    import shutil
    from concurrent.futures import ThreadPoolExecutor

    from oracle import time_reference as TR
    tmp = tempfile.mkdtemp(prefix="ogs_ref_arm_")

    def one(i):
        path = TR.write_deck(os.path.join(tmp, f"w{i}"), "sp", warm[i] + timed[i])
        t_launch = time.perf_counter()
        r = TR.run_reference(binary, path)
        a = [t for k, t in r["marks"] if k == "assemble"]
        acc = [t for k, t in r["marks"] if k == "accepted"]
        if r["rc"] != 0 or len(a) < warm[i] + timed[i] or len(acc) < warm[i] + timed[i]:
            raise RuntimeError(f"reference run {i}: rc {r['rc']}, {len(a)} assemblies, {len(acc)} accepted steps")
        return t_launch + a[warm[i]], t_launch + acc[warm[i] + timed[i] - 1], len(r["iterations"])

    try:
        with ThreadPoolExecutor(workers) as ex:
            res = list(ex.map(one, range(workers)))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return max(r[1] for r in res) - min(r[0] for r in res), [r[2] for r in res]


def reference_arm(args, rank):
    """The path on the host's cores without the GPU: the K timed steps
    (after W warm-up steps) shared among one single-threaded process per
    core, each step a full step of the deck (assembly of every hex,
    Dirichlet, CG + Jacobi to 1e-10).  Runs the reference's own executable
    where its build for this host exists, else the oracle's C restatement
    of the same algorithm."""
    if rank != 0:
        return
    k_steps, warm_steps = max(1, args.steps), max(3, args.warmup)
    cores = os.cpu_count() or 1
    workers = min(cores, k_steps)
    warm, timed = _split(warm_steps, workers), _split(k_steps, workers)
    binary = _reference_binary()
    if binary:
        wall, its = _run_binary(binary, workers, warm, timed)
        kind = "reference"
        what = (f"the reference OGS-5 (SP build: Linear_EQS, its own main), built from its sources by "
                f"oracle/refbuild.mk, one process per core on its own copy of the deck")
    else:
        wall, its = _run_port(workers, warm, timed)
        kind = "port"
        what = ("the oracle's C restatement of the reference's assembly, Dirichlet elimination and "
                "Linear_EQS::CG + Jacobi, one process per core; the reference's own executable is not used "
                "here: its sources are not on this host and its build from them is for another "
                "architecture")
    value = k_steps / wall
    out = {"metric": "solves/s", "value": round(value, 6), "unit": "solves/s", "n_gpus": 0,
           "steps": k_steps, "warmup": warm_steps, "ms_per_step": round(1e3 * wall / k_steps, 1),
           "impl": "reference", "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (seeded GRF conductivity, generated mesh)",
           "config": deck_config(int(os.environ.get("WORLD_SIZE", "1"))),
           "cpu_baseline": {"value": round(value, 6), "unit": "solves/s", "cores": workers, "kind": kind,
                            "sample": (f"{what}: {k_steps} full steps of the deck from the initial heads "
                                       f"(shares {timed}) after {warm_steps} warm-up steps, wall {wall:.1f} s "
                                       f"between barriers on {platform.machine()}")},
           "e2e": {"value": round(value, 6), "unit": "solves/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    if kind == "port":
        out["cpu_baseline"]["cg_iterations_per_step"] = round(float(np.mean(its)), 1)
    cal = os.path.join(ROOT, "oracle", "reference_timing.json")
    if os.path.exists(cal):
        with open(cal) as f:
            out["calibration"] = json.load(f).get("summary")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
