"""The small cases run through the bounds-checked build of the library
(libogs_gpu_debug.so, compiled with -DOGS_BOUNDS_CHECK): every kernel
family on quad, hex (lattice and distorted) and tet meshes -- flow and
transport assembly, Dirichlet sets in both modes, CG / BiCGStab with Jacobi
and ILU(0), the FP32-inner path on the diagonal-offset and SELL-32
operators, a Monte-Carlo batch and a Richards Picard step.  After each case
the library is asked for the first out-of-range index its kernels met.

Run as a child process with OGS_GPU_LIB pointing at the debug library
(tests/test_bounds_gpu.py does); prints one line per case and exits 1 on
the first recorded out-of-range index.
"""
import json
import sys

import numpy as np

from ogs5_gb300 import capi as gpu
from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import distort


def _faces(m):
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    return lf, rows, vals, x0


def _k(m, seed):
    rng = np.random.default_rng(seed)
    return np.exp(np.log(1e-5) + rng.standard_normal(m.n_elements))


def flow_case(m, mode, method, precond, precision=gpu.PRECISION_FP64, steady=False):
    lf, rows, vals, x0 = _faces(m)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=0.0 if steady else 1e-4, steady=1 if steady else 0)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.ConfigNumerics(method, precond, 5000, 1e-10, precision=precision, check_norm_rhs=False)
    eqs.Initialize()
    eqs.GlobalAssembly(p, _k(m, 1), x0)
    eqs.SetKnownX(rows, vals, mode)
    x = x0.copy()
    eqs.Solver(x, allow_fail=True)
    eqs.spmv(x)


def transport_case(m, precond):
    lf, rows, vals, x0 = _faces(m)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    q = eqs.gp_velocity(gpu.make_params(gpu.GROUNDWATER_FLOW), _k(m, 2), 10.0 * (1.0 - m.x / m.x.max()))
    eqs.ConfigNumerics(gpu.LS_BICGSTAB, precond, 1000, 1e-10, check_norm_rhs=False)
    eqs.Initialize()
    p = gpu.make_params(gpu.MASS_TRANSPORT, dt=3600.0, porosity=0.3, alpha_l=1.0, alpha_t=0.1, diffusion=1e-9)
    eqs.GlobalAssembly(p, None, np.zeros(m.n_nodes), q)
    eqs.SetKnownX(lf, np.ones(len(lf)), gpu.DIRICHLET_ROW_ONLY)
    c = np.zeros(m.n_nodes)
    c[lf] = 1.0
    eqs.Solver(c, allow_fail=True)


def batch_case():
    reals = [(n, n - 1, n + 1, fields.lognormal_k((n - 1, n - 2, n), np.log(1e-5), 1.0, 3.0, seed=n), 10.0, 0.0)
             for n in (5, 7, 9)]
    b = gpu.Batch(reals, tol=1e-10)
    b.solve(allow_fail=True)
    b.heads()
    b.close()


def richards_case():
    m = M.structured_quad(8, 10, 0.2, 0.1)
    gp = gpu.make_params(gpu.RICHARDS_FLOW, dt=600.0, storage=1e-6, porosity=0.35, drho_dp=4.4e-10,
                         viscosity=1e-3, density=1000.0, time_unit_factor=1.0)
    r = gpu.richards_params(capillary_model=4, permeability_model=4, pb=5.0e3, slr=0.08, slm=0.98, m=0.55,
                            kr_slr=0.08, kr_slm=0.98, kr_m=0.55, kr_min=1e-9)
    top = np.flatnonzero(m.y == m.y.max())
    p_old = np.full(m.n_nodes, -1.0e4)
    it = p_old.copy()
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, 1e-12, check_norm_rhs=False)
    eqs.RichardsStep(gp, r, np.full(m.n_elements, 5e-12), p_old, it, top, np.zeros(len(top)),
                     gpu.DIRICHLET_SYMMETRIC, error_method=2, max_iterations=20, tolerance=1.0, allow_fail=True)


def cases():
    hex_lat = M.structured_hex(12, 9, 7)
    hex_dist = distort(M.structured_hex(8, 6, 5), 0.2, seed=1)
    tet = M.structured_tet(7, 6, 5)
    quad = M.structured_quad(20, 14)
    S, R = gpu.DIRICHLET_SYMMETRIC, gpu.DIRICHLET_ROW_ONLY
    yield "hex lattice CG Jacobi symmetric", lambda: flow_case(hex_lat, S, gpu.LS_CG, gpu.PRECOND_JACOBI)
    yield "hex lattice BiCGStab ILU row-only", lambda: flow_case(hex_lat, R, gpu.LS_BICGSTAB, gpu.PRECOND_ILU0)
    yield "hex lattice FP32-inner", lambda: flow_case(hex_lat, S, gpu.LS_CG, gpu.PRECOND_JACOBI,
                                                      gpu.PRECISION_FP32_REFINED)
    yield "hex lattice FP32 cells", lambda: flow_case(hex_lat, S, gpu.LS_CG, gpu.PRECOND_JACOBI,
                                                      gpu.PRECISION_FP32_CELLS, steady=True)
    yield "hex distorted CG ILU symmetric", lambda: flow_case(hex_dist, S, gpu.LS_CG, gpu.PRECOND_ILU0)
    yield "hex distorted FP32-inner row-only (SELL)", lambda: flow_case(hex_dist, R, gpu.LS_CG, gpu.PRECOND_JACOBI,
                                                                        gpu.PRECISION_FP32_REFINED)
    yield "tet CG Jacobi symmetric", lambda: flow_case(tet, S, gpu.LS_CG, gpu.PRECOND_JACOBI)
    yield "tet FP32-inner", lambda: flow_case(tet, S, gpu.LS_CG, gpu.PRECOND_JACOBI, gpu.PRECISION_FP32_REFINED)
    yield "quad BiCGStab Jacobi row-only", lambda: flow_case(quad, R, gpu.LS_BICGSTAB, gpu.PRECOND_JACOBI)
    yield "quad FP32-inner", lambda: flow_case(quad, S, gpu.LS_CG, gpu.PRECOND_JACOBI, gpu.PRECISION_FP32_REFINED)
    yield "tet transport BiCGStab ILU", lambda: transport_case(tet, gpu.PRECOND_ILU0)
    yield "hex transport BiCGStab Jacobi", lambda: transport_case(hex_dist, gpu.PRECOND_JACOBI)
    yield "batch", batch_case
    yield "richards", richards_case


def main():
    site, _ = gpu.debug_oob()
    if site == -1:
        print(json.dumps({"error": "not a bounds-checked build"}))
        return 2
    for name, run in cases():
        run()
        site, index = gpu.debug_oob()
        print(json.dumps({"case": name, "site": site, "index": index}), flush=True)
        if site != 0:
            return 1
    print(json.dumps({"all": "clean"}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
