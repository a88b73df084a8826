"""ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the ogs5_gb300 product path.

Three libraries are wrapped:
  * ``_build/libogs_oracle.so`` -- the C restatement of the OGS-5 path
    (ogs_oracle.c), always built;
  * ``_ref/libogs5ref.so`` -- the reference's own FEM/mathlib.cpp,
    FEM/matrix_class.cpp and FEM/equation_class.cpp behind ref_harness.cpp,
    built only where the reference sources are present;
  * ``_ref/libogs5geo.so`` -- the reference's own GEOLIB surface, polygon
    and polyline code behind ref_geo_harness.cpp (node searches of the deck
    reader), built only where the reference sources are present.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libogs_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libogs5ref.so")
GEO_SO = os.path.join(HERE, "_ref", "libogs5geo.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

QUAD4, HEX8, TET4 = 0, 1, 2
GWF, LIQUID, MT = 0, 1, 2


def build(ref: str | None = None) -> None:
    """Runs oracle/Makefile (C restatement; reference harness when present)."""
    args = ["make", "-s", "-j", str(min(16, os.cpu_count() or 1)), "-C", HERE]
    if ref:
        args.append(f"REF={ref}")
    subprocess.run(args, check=True)


class AssemblyParams(C.Structure):
    """Mirror of ogs_assembly_params (include/ogs_gpu.h)."""
    _fields_ = [
        ("pcs_type", C.c_int32), ("steady", C.c_int32), ("dt", C.c_double),
        ("theta", C.c_double), ("nls_relaxation", C.c_double),
        ("time_unit_factor", C.c_double), ("storage", C.c_double),
        ("porosity", C.c_double), ("drho_dp", C.c_double),
        ("viscosity", C.c_double), ("density", C.c_double),
        ("gravity", C.c_double), ("gravity_on", C.c_int32), ("mass_lumping", C.c_int32),
        ("alpha_l", C.c_double), ("alpha_t", C.c_double),
        ("diffusion", C.c_double), ("decay", C.c_double),
        ("retardation", C.c_double), ("saturation", C.c_double),
        ("supg_method", C.c_int32), ("supg_length", C.c_int32), ("supg_diffusivity", C.c_int32),
        ("memory_type", C.c_int32),
    ]


class RichardsParams(C.Structure):
    """Mirror of ogs_richards_params (include/ogs_gpu.h)."""
    _fields_ = [("capillary_model", C.c_int32), ("permeability_model", C.c_int32), ("pb", C.c_double),
                ("slr", C.c_double), ("slm", C.c_double), ("m", C.c_double), ("kr_slr", C.c_double),
                ("kr_slm", C.c_double), ("kr_m", C.c_double), ("kr_min", C.c_double)]


def richards_params(**kw) -> RichardsParams:
    r = RichardsParams(4, 4, 1.0e4, 0.1, 1.0, 0.5, 0.1, 1.0, 0.5, 1e-9)
    for k, v in kw.items():
        if not hasattr(r, k):
            raise AttributeError(k)
        setattr(r, k, v)
    return r


def make_params(**kw) -> AssemblyParams:
    p = AssemblyParams()
    p.dt = 1.0
    p.theta = 1.0
    p.time_unit_factor = 1.0
    p.viscosity = 1.0
    p.density = 1000.0
    p.retardation = 1.0
    p.saturation = 1.0
    for k, v in kw.items():
        setattr(p, k, v)
    return p


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        L.orc_gauss_point.restype = C.c_double
        L.orc_gauss_point.argtypes = [C.c_long, C.c_long]
        L.orc_gauss_weight.restype = C.c_double
        L.orc_gauss_weight.argtypes = [C.c_long, C.c_long]
        L.orc_tet5_point.argtypes = [C.c_int, _dp]
        L.orc_shape_table.restype = C.c_int
        L.orc_shape_table.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_void_p]
        L.orc_num_gauss_points.restype = C.c_int
        L.orc_num_gauss_points.argtypes = [C.c_int, C.c_int]
        L.orc_element_matrices.restype = C.c_int
        L.orc_element_matrices.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_void_p,
                                           C.POINTER(AssemblyParams), C.c_double, C.c_void_p,
                                           C.c_void_p]
        L.orc_build_pattern.restype = C.c_int64
        L.orc_build_pattern.argtypes = [C.c_int64, C.c_int64, C.c_int, _i32p, C.c_void_p, C.c_void_p]
        L.orc_assemble.restype = C.c_int64
        L.orc_assemble.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64, _dp, _dp,
                                   C.c_void_p, _i32p, _i64p, _i64p, C.POINTER(AssemblyParams),
                                   C.c_void_p, C.c_void_p, C.c_void_p, _dp, _dp]
        L.orc_gp_velocity.restype = C.c_int64
        L.orc_gp_velocity.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, _dp, _dp, C.c_void_p,
                                      _i32p, C.POINTER(AssemblyParams), _dp, _dp, _dp]
        L.orc_dirichlet_row_only.argtypes = [_i64p, _i64p, _dp, _dp, C.c_int64, _i64p, _dp]
        L.orc_dirichlet_symmetric.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, C.c_int64,
                                              _i64p, _dp]
        L.orc_spmv.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _dp]
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _dp, C.c_int, C.c_int,
                                C.c_int, C.c_double, C.c_void_p, _dp]
        L.orc_ilu0_factor.restype = C.c_int
        L.orc_ilu0_factor.argtypes = [C.c_int64, _i64p, _i64p, _dp, _dp, _i64p]
        rp = C.POINTER(RichardsParams)
        for name in ("orc_rich_saturation", "orc_rich_dsdpc", "orc_rich_krel"):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [rp, C.c_double]
        L.orc_rich_mass_coef.restype = C.c_double
        L.orc_rich_mass_coef.argtypes = [C.c_void_p, rp, C.c_double]
        L.orc_rich_lap_coef.restype = C.c_double
        L.orc_rich_lap_coef.argtypes = [C.c_void_p, rp, C.c_double, C.c_double]
        L.orc_element_matrices_richards.restype = C.c_int
        L.orc_element_matrices_richards.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_void_p,
                                                    C.c_void_p, rp, C.c_double, _dp, C.c_void_p]
        L.orc_assemble_richards.restype = C.c_int64
        L.orc_assemble_richards.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, _dp, _dp, C.c_void_p,
                                            _i32p, _i64p, _i64p, C.c_void_p, rp, _dp, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------
# oracle functions
# --------------------------------------------------------------------------

def shape_table(etype: int, ngauss: int = 3):
    """(xi[ngp,3], w[ngp], N[ngp,nn], dN[ngp,dim,nn]) of ShapeFunctionPool."""
    nn = 8 if etype == HEX8 else 4
    dim = 2 if etype == QUAD4 else 3
    ngp = lib().orc_num_gauss_points(etype, ngauss)
    xi = np.zeros(ngp * 3)
    w = np.zeros(ngp)
    N = np.zeros(ngp * nn)
    dN = np.zeros(ngp * nn * dim)
    lib().orc_shape_table(etype, ngauss, xi, w, N, dN, None)
    return xi.reshape(ngp, 3), w, N.reshape(ngp, nn), dN.reshape(ngp, dim, nn)


class ElemMats(C.Structure):
    _fields_ = [("mass", C.c_double * 64), ("laplace", C.c_double * 64),
                ("advection", C.c_double * 64), ("storage", C.c_double * 64),
                ("rhs_gravity", C.c_double * 8)]


def element_matrices(etype, coords, params, k_e=1.0, vel=None, ngauss=3):
    """Local mass, Laplace, advection, storage matrices of one element."""
    nn = 8 if etype == HEX8 else 4
    dim = 2 if etype == QUAD4 else 3
    X = np.ascontiguousarray(coords[:, 0], dtype=np.float64)
    Y = np.ascontiguousarray(coords[:, 1], dtype=np.float64)
    Z = np.ascontiguousarray(coords[:, 2], dtype=np.float64) if dim == 3 else None
    m = ElemMats()
    v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
    rc = lib().orc_element_matrices(etype, ngauss, dim, X, Y, _ptr(Z), C.byref(params), k_e,
                                    _ptr(v), C.byref(m))
    if rc:
        raise ValueError("singular Jacobian")
    out = {}
    for name in ("mass", "laplace", "advection", "storage"):
        out[name] = np.frombuffer(getattr(m, name), dtype=np.float64)[: nn * nn].reshape(nn, nn).copy()
    out["rhs_gravity"] = np.frombuffer(m.rhs_gravity, dtype=np.float64)[:nn].copy()
    return out


def rich_curves(r: RichardsParams, pc=None, sw=None):
    """Saturation S(pc), dS/dpc(S) and k_rel(S) of the medium (scalars)."""
    L = lib()
    out = {}
    if pc is not None:
        out["saturation"] = L.orc_rich_saturation(C.byref(r), pc)
    if sw is not None:
        out["dsdpc"] = L.orc_rich_dsdpc(C.byref(r), sw)
        out["krel"] = L.orc_rich_krel(C.byref(r), sw)
    return out


def rich_coefficients(params, r: RichardsParams, k, PG):
    """CalCoefMass and CalCoefLaplace of RICHARDS_FLOW at pressure PG."""
    L = lib()
    return (L.orc_rich_mass_coef(C.byref(params), C.byref(r), PG),
            L.orc_rich_lap_coef(C.byref(params), C.byref(r), k, PG))


def element_matrices_richards(etype, coords, params, r, k_e, u1, ngauss=3):
    nn = 8 if etype == HEX8 else 4
    dim = 2 if etype == QUAD4 else 3
    X = np.ascontiguousarray(coords[:, 0], dtype=np.float64)
    Y = np.ascontiguousarray(coords[:, 1], dtype=np.float64)
    Z = np.ascontiguousarray(coords[:, 2], dtype=np.float64) if dim == 3 else None
    m = ElemMats()
    rc = lib().orc_element_matrices_richards(etype, ngauss, dim, X, Y, _ptr(Z), C.byref(params), C.byref(r),
                                             k_e, np.ascontiguousarray(u1, dtype=np.float64), C.byref(m))
    if rc:
        raise ValueError("singular Jacobian")
    return {"mass": np.frombuffer(m.mass, dtype=np.float64)[: nn * nn].reshape(nn, nn).copy(),
            "laplace": np.frombuffer(m.laplace, dtype=np.float64)[: nn * nn].reshape(nn, nn).copy(),
            "rhs_gravity": np.frombuffer(m.rhs_gravity, dtype=np.float64)[:nn].copy()}


def assemble_richards(mesh, row_ptr, col, params, r, elem_k, p_old, p_iter, ngauss=3):
    """RICHARDS_FLOW global A values (on the pattern) and b at the iterate."""
    val = np.zeros(len(col))
    b = np.zeros(mesh.n_nodes)
    z = mesh.z if mesh.dim == 3 else None
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    rc = lib().orc_assemble_richards(mesh.elem_type, ngauss, mesh.dim, mesh.n_elements, mesh.x, mesh.y, _ptr(z),
                                     mesh.conn.ravel(), row_ptr, col, C.byref(params), C.byref(r), f(elem_k),
                                     f(p_old), f(p_iter), val, b)
    if rc:
        raise ValueError(f"singular Jacobian in element {-rc - 1}")
    return val, b


def richards_picard(mesh, row_ptr, col, params, r, elem_k, p_old, p_iter0, rows, vals, symmetric,
                    error_method=2, tolerance=1e-6, max_iterations=20, method=5, precond=1, max_iter=5000,
                    tol=1e-12, ngauss=3):
    """One RICHARDS_FLOW time step by Picard iteration, restating
    CRFProcess::ExecuteNonLinear (rf_pcs.cpp:9636-9960) with Execute
    (:4695-5080) and CalcIterationNODError (:9170-9600).  Returns (iterate,
    info)."""
    it = np.array(p_iter0, dtype=np.float64)
    theta0 = 1.0 - params.nls_relaxation
    if theta0 < np.finfo(float).eps:
        theta0 = 1.0
    last, fails, info = 1.0, 0, {"iterations": 0, "converged": False, "diverged": False, "linear": 0}
    for k in range(max_iterations):
        val, b = assemble_richards(mesh, row_ptr, col, params, r, elem_k, p_old, it, ngauss)
        dirichlet(row_ptr, col, val, b, rows, vals, symmetric=symmetric)
        x, li = solve(row_ptr, col, val, b, it, method=method, precond=precond, max_iter=max_iter, tol=tol)
        info["linear"] += li["iterations"]
        d = it - x
        if error_method == 1:
            abs_err = np.abs(d).max()
        elif error_method == 4:
            abs_err = np.sqrt(np.sum(d * d)) / (np.sqrt(np.sum(it * it)) + np.finfo(float).eps)
        else:
            abs_err = np.sqrt(np.sum(d * d))
        err = abs_err / tolerance
        theta = 1.0 if err < 1.0 else theta0
        it = x.copy() if theta == 1.0 else (1.0 - theta) * it + theta * x
        info["iterations"], info["error"] = k + 1, err
        if err <= 1.0:
            info["converged"] = True
            break
        percent = 100.0 * ((last - err) / last)
        fails = fails + 1 if (k > 0 and percent < 1.0) else 0
        last = err
        if fails > 1:
            info["diverged"] = True
            break
    return it, info


def build_pattern(n_nodes, conn):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    ne, nn = conn.shape
    nnz = lib().orc_build_pattern(n_nodes, ne, nn, conn.ravel(), None, None)
    row_ptr = np.zeros(n_nodes + 1, dtype=np.int64)
    col = np.zeros(nnz, dtype=np.int64)
    lib().orc_build_pattern(n_nodes, ne, nn, conn.ravel(), _ptr(row_ptr), _ptr(col))
    return row_ptr, col


def assemble(mesh, row_ptr, col, params, elem_k=None, u0=None, gp_vel=None, ngauss=3):
    """Global A values (on the pattern) and b."""
    n = mesh.n_nodes
    val = np.zeros(len(col))
    b = np.zeros(n)
    ek = None if elem_k is None else np.ascontiguousarray(elem_k, dtype=np.float64)
    u = None if u0 is None else np.ascontiguousarray(u0, dtype=np.float64)
    gv = None if gp_vel is None else np.ascontiguousarray(gp_vel, dtype=np.float64)
    z = mesh.z if mesh.dim == 3 else None
    rc = lib().orc_assemble(mesh.elem_type, ngauss, mesh.dim, n, mesh.n_elements, mesh.x, mesh.y,
                            _ptr(z), mesh.conn.ravel(), row_ptr, col, C.byref(params),
                            _ptr(ek), _ptr(u), _ptr(gv), val, b)
    if rc:
        raise ValueError(f"singular Jacobian in element {-rc - 1}")
    return val, b


def gp_velocity(mesh, params, elem_k, u, ngauss=3):
    ngp = lib().orc_num_gauss_points(mesh.elem_type, ngauss)
    q = np.zeros(mesh.n_elements * ngp * 3)
    z = mesh.z if mesh.dim == 3 else None
    rc = lib().orc_gp_velocity(mesh.elem_type, ngauss, mesh.dim, mesh.n_elements, mesh.x, mesh.y,
                               _ptr(z), mesh.conn.ravel(), C.byref(params),
                               np.ascontiguousarray(elem_k, dtype=np.float64),
                               np.ascontiguousarray(u, dtype=np.float64), q)
    if rc:
        raise ValueError("singular Jacobian")
    return q.reshape(mesh.n_elements, ngp, 3)


def dirichlet(row_ptr, col, val, b, rows, vals, symmetric=False):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    if symmetric:
        lib().orc_dirichlet_symmetric(len(b), row_ptr, col, val, b, len(rows), rows, vals)
    else:
        lib().orc_dirichlet_row_only(row_ptr, col, val, b, len(rows), rows, vals)


def ilu0_factor(row_ptr, col, val):
    """orc_ilu0_factor: ILU(0) (IKJ) on the CSR pattern; returns the in-place
    factors (unit lower L below the diagonal, U on and above it)."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int64)
    lu = np.zeros(len(cl))
    dpos = np.zeros(len(rp) - 1, dtype=np.int64)
    rc = lib().orc_ilu0_factor(len(rp) - 1, rp, cl, np.ascontiguousarray(val, dtype=np.float64), lu, dpos)
    if rc:
        raise ValueError("ILU(0): zero pivot")
    return lu


def spmv(row_ptr, col, val, x):
    y = np.zeros(len(row_ptr) - 1)
    lib().orc_spmv(len(y), row_ptr, col, val, np.ascontiguousarray(x, dtype=np.float64), y)
    return y


def solve(row_ptr, col, val, b, x0, method=2, precond=1, max_iter=1000, tol=1e-10,
          b_norm: float | None = None):
    """Linear_EQS::Solver semantics.  Returns (x, info dict)."""
    n = len(b)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    out = np.zeros(4)
    bn = None
    if b_norm is not None:
        bn = C.c_double(b_norm)
    rc = lib().orc_solve(n, row_ptr, col, val, np.ascontiguousarray(b, dtype=np.float64), x,
                         method, precond, max_iter, tol,
                         None if bn is None else C.cast(C.pointer(bn), C.c_void_p), out)
    if rc:
        raise ValueError("oracle solve failed (bad method or zero ILU pivot)")
    return x, {"iterations": int(out[0]), "rel_residual": out[1], "b_norm": out[2],
               "breakdown": bool(out[3])}


# --------------------------------------------------------------------------
# the reference's own code
# --------------------------------------------------------------------------

_ref = None
_ref_geo = None


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def has_ref_geo() -> bool:
    return os.path.exists(GEO_SO)


def ref_geo():
    """The reference's GEOLIB/MathLib geometry behind ref_geo_harness.cpp,
    with numpy front ends: surface_nodes, polyline_nodes, point_in_polygon."""
    global _ref_geo
    if _ref_geo is None:
        L = C.CDLL(GEO_SO)
        L.ref_geo_surface_nodes.argtypes = [C.c_int, _dp, C.c_int64, _dp, C.c_double, C.c_void_p]
        L.ref_geo_polyline_nodes.argtypes = [C.c_int, _dp, C.c_int64, _dp, C.c_double, _i64p, _dp]
        L.ref_geo_polyline_nodes.restype = C.c_int64
        L.ref_geo_point_in_polygon.argtypes = [C.c_int, _dp, C.c_int64, _dp, C.c_void_p]
        _ref_geo = L
    return _ref_geo


def _xyz(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, 3))


def ref_surface_nodes(polygon, nodes, eps):
    """Mesh nodes on the surface of a closed polygon (GetNODOnSFC loop)."""
    P, X = _xyz(polygon), _xyz(nodes)
    mask = np.zeros(len(X), dtype=np.uint8)
    if ref_geo().ref_geo_surface_nodes(len(P), P.ravel(), len(X), X.ravel(), eps, mask.ctypes.data) != 0:
        raise RuntimeError("Surface::createSurface failed")
    return np.flatnonzero(mask)


def ref_polyline_nodes(points, nodes, radius):
    """Mesh nodes along a polyline in MeshNodesAlongPolyline order."""
    P, X = _xyz(points), _xyz(nodes)
    ids = np.zeros(len(X), dtype=np.int64)
    dist = np.zeros(len(X))
    n = ref_geo().ref_geo_polyline_nodes(len(P), P.ravel(), len(X), X.ravel(), radius, ids, dist)
    return ids[:n], dist[:n]


def ref_point_in_polygon(polygon, points):
    P, X = _xyz(polygon), _xyz(points)
    mask = np.zeros(len(X), dtype=np.uint8)
    ref_geo().ref_geo_point_in_polygon(len(P), P.ravel(), len(X), X.ravel(), mask.ctypes.data)
    return mask.astype(bool)


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        L.ref_gauss_point.restype = C.c_double
        L.ref_gauss_point.argtypes = [C.c_long, C.c_long]
        L.ref_gauss_weight.restype = C.c_double
        L.ref_gauss_weight.argtypes = [C.c_long, C.c_long]
        L.ref_tet5_point.argtypes = [C.c_int, _dp]
        L.ref_shape.argtypes = [C.c_int, _dp, _dp, _dp]
        L.ref_system_create.restype = C.c_void_p
        L.ref_system_create.argtypes = [C.c_long, _i64p, _i64p, C.c_int, C.c_int, C.c_int,
                                        C.c_double]
        L.ref_system_destroy.argtypes = [C.c_void_p]
        L.ref_system_set.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_system_add.argtypes = [C.c_void_p, C.c_long, C.c_long, C.c_double]
        L.ref_system_set_known.argtypes = [C.c_void_p, C.c_long, C.c_double]
        L.ref_system_get.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_system_spmv.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_system_solve.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_system_write_bin.restype = C.c_long
        L.ref_system_write_bin.argtypes = [C.c_void_p, C.c_void_p, C.c_long]
        _ref = L
    return _ref


class RefSystem:
    """The reference's Linear_EQS on a CRS SparseTable."""

    def __init__(self, row_ptr, col, method=2, precond=1, max_iter=1000, tol=1e-10):
        self.n = len(row_ptr) - 1
        self.nnz = int(row_ptr[-1])
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int64)
        self.h = ref().ref_system_create(self.n, self.row_ptr, self.col, method, precond,
                                         max_iter, tol)

    def close(self):
        if self.h:
            ref().ref_system_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set(self, val, b):
        ref().ref_system_set(self.h, np.ascontiguousarray(val, dtype=np.float64),
                             np.ascontiguousarray(b, dtype=np.float64))

    def add(self, r, c, v):
        ref().ref_system_add(self.h, int(r), int(c), float(v))

    def set_known(self, rows, vals):
        for r, v in zip(rows, vals):
            ref().ref_system_set_known(self.h, int(r), float(v))

    def get(self):
        val = np.zeros(self.nnz)
        b = np.zeros(self.n)
        ref().ref_system_get(self.h, _ptr(val), _ptr(b))
        return val, b

    def spmv(self, x):
        y = np.zeros(self.n)
        ref().ref_system_spmv(self.h, np.ascontiguousarray(x, dtype=np.float64), y)
        return y

    def solve(self, x0):
        x = np.ascontiguousarray(x0, dtype=np.float64).copy()
        out = np.zeros(4)
        ref().ref_system_solve(self.h, x, out)
        return x, {"ret": int(out[0]), "iterations": int(out[1]), "rel_residual": out[2],
                   "b_norm": out[3]}

    def write_bin(self) -> bytes:
        n = ref().ref_system_write_bin(self.h, None, 0)
        buf = C.create_string_buffer(n)
        ref().ref_system_write_bin(self.h, C.cast(buf, C.c_void_p), n)
        return buf.raw
