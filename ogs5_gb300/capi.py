"""ctypes binding of include/ogs_gpu.h and a host-side mirror of the OGS-5
solver surface (Linear_EQS, CRFProcess::GlobalAssembly) over it.

The mirror keeps the reference's names and argument meanings so that test
code reads like the reference's own driver code:

    eqs = LinearEQS(mesh)                      # Linear_EQS(SparseTable, dof)
    eqs.ConfigNumerics(ls_method=5, ls_precond=1, ls_max_iterations=1000,
                       ls_error_tolerance=1e-10)
    eqs.Initialize()                           # A = 0, b = 0
    eqs.GlobalAssembly(params, elem_k, u0)     # element loop + scatter
    eqs.SetKnownX(rows, values)                # SetKnownX_i over a node set
    iters = eqs.Solver(x)                      # x: initial guess in, solution out

Arrays may be numpy (host) or torch CUDA tensors (device, used in place).
Errors raise OgsError carrying the ogs_status and the library's message.
There is no CPU fallback: without the compiled library or a GPU every call
fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

OK, NOT_CONVERGED, BREAKDOWN, NONFINITE, OOM, BAD_ARG, CUDA_ERROR, SINGULAR_JACOBIAN = range(8)
STATUS_NAMES = ["OK", "NOT_CONVERGED", "BREAKDOWN", "NONFINITE", "OOM", "BAD_ARG", "CUDA_ERROR",
                "SINGULAR_JACOBIAN"]
QUAD4, HEX8, TET4 = 0, 1, 2
GROUNDWATER_FLOW, LIQUID_FLOW, MASS_TRANSPORT = 0, 1, 2
DIRICHLET_ROW_ONLY, DIRICHLET_SYMMETRIC = 0, 1
LS_BICGSTAB, LS_CG = 2, 5
PRECOND_NONE, PRECOND_JACOBI, PRECOND_ILU0 = 0, 1, 100
PRECISION_FP64, PRECISION_FP32_REFINED, PRECISION_FP32_CELLS = 0, 1, 2
SCHEDULE_GRAPH, SCHEDULE_PERSISTENT = 0, 1

# every entry point include/ogs_gpu.h declares
EXPORTS = [
    "ogs_gpu_last_error", "ogs_gpu_version", "ogs_gpu_mesh_create", "ogs_gpu_mesh_destroy",
    "ogs_gpu_mesh_info", "ogs_gpu_system_create", "ogs_gpu_system_destroy", "ogs_gpu_configure",
    "ogs_gpu_initialize", "ogs_gpu_assemble", "ogs_gpu_set_dirichlet", "ogs_gpu_solve",
    "ogs_gpu_gp_velocity", "ogs_gpu_get_csr", "ogs_gpu_get_rhs", "ogs_gpu_get_x",
    "ogs_gpu_spmv", "ogs_gpu_mesh_gauss_points", "ogs_gpu_mesh_ilu_tiles", "ogs_gpu_kernel_launches",
    "ogs_gpu_profile",
    "ogs_gpu_csr_cg_noalloc", "ogs_gpu_get_ilu0",
    "ogs_gpu_batch_create", "ogs_gpu_batch_destroy", "ogs_gpu_batch_set_k", "ogs_gpu_batch_autotune",
    "ogs_gpu_batch_set_tuning", "ogs_gpu_batch_solve", "ogs_gpu_batch_get_heads", "ogs_gpu_batch_info",
    "ogs_gpu_solve_begin", "ogs_gpu_solve_poll", "ogs_gpu_solve_end",
    "ogs_gpu_server_create", "ogs_gpu_server_destroy", "ogs_gpu_server_add_class", "ogs_gpu_server_submit",
    "ogs_gpu_server_progress", "ogs_gpu_server_result", "ogs_gpu_server_info", "ogs_gpu_server_reserve",
    "ogs_gpu_cache_reset", "ogs_gpu_assemble_richards", "ogs_gpu_richards_step",
    "ogs_deck_read", "ogs_deck_destroy", "ogs_deck_mesh", "ogs_deck_geo_nodes", "ogs_deck_dirichlet",
    "ogs_gpu_selftest_barrier", "ogs_gpu_debug_oob", "ogs_gpu_debug_fp32_product",
]
REQUEST_FLOW, REQUEST_TRANSPORT = 0, 1
RICHARDS_FLOW = 3
LMAX, ENORM, EVNORM, ERNORM = 1, 2, 3, 4
SERVER_PRIORITY, SERVER_SJF, SERVER_BATCH, SERVER_PRECISION_FALLBACK = 1, 2, 4, 8
NOALLOC_MAX_ROWS = 524288


class OgsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {msg}")
        self.status = status


class MeshDesc(C.Structure):
    _fields_ = [("elem_type", C.c_int32), ("dim", C.c_int32), ("n_nodes", C.c_int64),
                ("n_elements", C.c_int64), ("x", C.c_void_p), ("y", C.c_void_p),
                ("z", C.c_void_p), ("connectivity", C.c_void_p), ("gauss_points", C.c_int32)]


class AssemblyParams(C.Structure):
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


class SolverConfig(C.Structure):
    _fields_ = [("method", C.c_int32), ("precond", C.c_int32), ("max_iter", C.c_int32),
                ("precision", C.c_int32), ("tol", C.c_double), ("inner_tol", C.c_double),
                ("check_norm_rhs", C.c_int32), ("schedule", C.c_int32)]


class Profile(C.Structure):
    _fields_ = [("spmv_ms", C.c_double), ("spmv_launches", C.c_int64), ("solve_ms", C.c_double),
                ("solves", C.c_int64), ("persist_ms", C.c_double), ("persist_iters", C.c_int64)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("status", C.c_int32), ("rel_residual", C.c_double),
                ("b_norm", C.c_double), ("refinements", C.c_int32), ("fp64_fallback", C.c_int32),
                ("solve_ms", C.c_double), ("fp32_operator", C.c_int32), ("pad0", C.c_int32)]


class BatchRealisation(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("pad0", C.c_int32),
                ("elem_k", C.c_void_p), ("h_left", C.c_double), ("h_right", C.c_double)]


class BatchConfig(C.Structure):
    _fields_ = [("hx", C.c_double), ("hy", C.c_double), ("hz", C.c_double),
                ("time_unit_factor", C.c_double), ("tol", C.c_double), ("inner_tol", C.c_double),
                ("max_iter", C.c_int32), ("pad0", C.c_int32)]


class BatchTuning(C.Structure):
    _fields_ = [("tile_rows", C.c_int32), ("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("graph", C.c_int32), ("ms_per_step", C.c_double)]


class BatchStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("status", C.c_int32), ("refinements", C.c_int32),
                ("pad0", C.c_int32), ("rel_residual", C.c_double), ("finish_ms", C.c_double)]


class ServerClass(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("kind", C.c_int32), ("bc_mode", C.c_int32),
                ("params", AssemblyParams), ("flow_params", AssemblyParams), ("n_elements", C.c_int64),
                ("flow_head", C.c_void_p), ("bc_rows", C.c_void_p), ("bc_values", C.c_void_p),
                ("n_bc", C.c_int64), ("solver", SolverConfig)]


class ServerResult(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("iterations", C.c_int32),
                ("refinements", C.c_int32), ("rel_residual", C.c_double), ("latency_ms", C.c_double),
                ("queue_ms", C.c_double), ("solve_ms", C.c_double), ("batch_size", C.c_int32),
                ("precision", C.c_int32), ("fp64_fallback", C.c_int32), ("pad0", C.c_int32)]


class ServerInfo(C.Structure):
    _fields_ = [("slots", C.c_int32), ("running", C.c_int32), ("queued", C.c_int32), ("fp64_classes", C.c_int32),
                ("completed", C.c_int64), ("bytes_used", C.c_int64), ("bytes_budget", C.c_int64),
                ("batched", C.c_int64)]


class RichardsParams(C.Structure):
    _fields_ = [("capillary_model", C.c_int32), ("permeability_model", C.c_int32), ("pb", C.c_double),
                ("slr", C.c_double), ("slm", C.c_double), ("m", C.c_double), ("kr_slr", C.c_double),
                ("kr_slm", C.c_double), ("kr_m", C.c_double), ("kr_min", C.c_double)]


class PicardConfig(C.Structure):
    _fields_ = [("error_method", C.c_int32), ("max_iterations", C.c_int32), ("tolerance", C.c_double)]


class PicardStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("diverged", C.c_int32),
                ("linear_iterations", C.c_int32), ("error", C.c_double), ("solve_ms", C.c_double)]


def richards_params(**kw) -> RichardsParams:
    """ogs_richards_params; defaults: van Genuchten curves, pb 1e4 Pa,
    residual 0.1, maximum 1, exponent 0.5, minimum k_rel 1e-9."""
    r = RichardsParams(4, 4, 1.0e4, 0.1, 1.0, 0.5, 0.1, 1.0, 0.5, 1e-9)
    for k, v in kw.items():
        if not hasattr(r, k):
            raise AttributeError(k)
        setattr(r, k, v)
    return r


def make_params(pcs_type=GROUNDWATER_FLOW, **kw) -> AssemblyParams:
    """ogs_assembly_params with the defaults of an OGS-5 deck."""
    p = AssemblyParams()
    p.pcs_type = pcs_type
    p.dt = 1.0
    p.theta = 1.0
    p.time_unit_factor = 1.0
    p.viscosity = 1.0e-3
    p.density = 1000.0
    p.retardation = 1.0
    p.saturation = 1.0
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


_LIB = None


def library_path() -> str:
    """The library to load: OGS_GPU_LIB when set (e.g. the bounds-checked
    build), else the in-tree build."""
    return os.environ.get("OGS_GPU_LIB") or _build.LIB


def lib():
    """Loads libogs_gpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise OSError(f"{path} is missing: run ogs5_gb300.build.build() (nvcc) first")
        L = C.CDLL(path)
        vp = C.c_void_p
        st = C.c_int
        L.ogs_gpu_last_error.restype = C.c_char_p
        L.ogs_gpu_version.restype = C.c_char_p
        L.ogs_gpu_mesh_create.argtypes = [C.POINTER(MeshDesc), C.POINTER(vp)]
        L.ogs_gpu_mesh_destroy.argtypes = [vp]
        L.ogs_gpu_mesh_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.ogs_gpu_system_create.argtypes = [vp, vp, C.POINTER(vp)]
        L.ogs_gpu_system_destroy.argtypes = [vp]
        L.ogs_gpu_configure.argtypes = [vp, C.POINTER(SolverConfig)]
        L.ogs_gpu_initialize.argtypes = [vp]
        L.ogs_gpu_assemble.argtypes = [vp, C.POINTER(AssemblyParams), vp, vp, vp]
        L.ogs_gpu_set_dirichlet.argtypes = [vp, vp, vp, C.c_int64, C.c_int32]
        L.ogs_gpu_solve.argtypes = [vp, vp, C.POINTER(SolveStats)]
        L.ogs_gpu_gp_velocity.argtypes = [vp, C.POINTER(AssemblyParams), vp, vp, vp]
        L.ogs_gpu_get_csr.argtypes = [vp, vp, vp, vp]
        L.ogs_gpu_get_rhs.argtypes = [vp, vp]
        L.ogs_gpu_get_x.argtypes = [vp, vp]
        L.ogs_gpu_get_ilu0.argtypes = [vp, vp]
        L.ogs_gpu_spmv.argtypes = [vp, vp, vp]
        L.ogs_gpu_mesh_gauss_points.argtypes = [vp]
        L.ogs_gpu_mesh_gauss_points.restype = C.c_int32
        L.ogs_gpu_mesh_ilu_tiles.argtypes = [vp]
        L.ogs_gpu_mesh_ilu_tiles.restype = C.c_int32
        L.ogs_gpu_profile.argtypes = [vp, C.c_int32, C.POINTER(Profile)]
        L.ogs_gpu_profile.restype = st
        L.ogs_gpu_csr_cg_noalloc.argtypes = [C.c_int64, vp, vp, vp, vp, vp, C.c_int32, C.c_double, vp,
                                             C.POINTER(SolveStats)]
        L.ogs_gpu_csr_cg_noalloc.restype = st
        L.ogs_gpu_batch_create.argtypes = [C.POINTER(BatchConfig), C.POINTER(BatchRealisation), C.c_int32,
                                           vp, C.POINTER(vp)]
        L.ogs_gpu_batch_destroy.argtypes = [vp]
        L.ogs_gpu_batch_set_k.argtypes = [vp, vp]
        L.ogs_gpu_batch_autotune.argtypes = [vp, C.POINTER(BatchTuning)]
        L.ogs_gpu_batch_set_tuning.argtypes = [vp, C.POINTER(BatchTuning)]
        L.ogs_gpu_batch_solve.argtypes = [vp, C.POINTER(BatchStats)]
        L.ogs_gpu_batch_get_heads.argtypes = [vp, vp]
        L.ogs_gpu_batch_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        for name in ("ogs_gpu_batch_create", "ogs_gpu_batch_destroy", "ogs_gpu_batch_set_k",
                     "ogs_gpu_batch_autotune", "ogs_gpu_batch_set_tuning", "ogs_gpu_batch_solve",
                     "ogs_gpu_batch_get_heads", "ogs_gpu_batch_info"):
            getattr(L, name).restype = st
        L.ogs_gpu_solve_begin.argtypes = [vp, vp]
        L.ogs_gpu_solve_poll.argtypes = [vp, C.POINTER(C.c_int32)]
        L.ogs_gpu_solve_end.argtypes = [vp, C.POINTER(SolveStats)]
        L.ogs_gpu_server_create.argtypes = [C.c_int64, C.c_int32, C.c_int32, C.POINTER(vp)]
        L.ogs_gpu_server_destroy.argtypes = [vp]
        L.ogs_gpu_server_add_class.argtypes = [vp, C.POINTER(ServerClass), C.POINTER(C.c_int32)]
        L.ogs_gpu_server_submit.argtypes = [vp, C.c_int32, vp, C.c_double, vp, C.POINTER(C.c_int64)]
        L.ogs_gpu_server_progress.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.ogs_gpu_server_result.argtypes = [vp, C.c_int64, C.POINTER(ServerResult)]
        L.ogs_gpu_server_info.argtypes = [vp, C.POINTER(ServerInfo)]
        L.ogs_gpu_server_reserve.argtypes = [vp, C.c_int32, C.c_int32]
        L.ogs_gpu_server_reserve.restype = st
        for name in ("ogs_gpu_solve_begin", "ogs_gpu_solve_poll", "ogs_gpu_solve_end", "ogs_gpu_server_create",
                     "ogs_gpu_server_destroy", "ogs_gpu_server_add_class", "ogs_gpu_server_submit",
                     "ogs_gpu_server_progress", "ogs_gpu_server_result", "ogs_gpu_server_info"):
            getattr(L, name).restype = st
        L.ogs_gpu_cache_reset.argtypes = [vp]
        L.ogs_gpu_cache_reset.restype = st
        L.ogs_gpu_assemble_richards.argtypes = [vp, C.POINTER(AssemblyParams), C.POINTER(RichardsParams), vp, vp,
                                                vp]
        L.ogs_gpu_assemble_richards.restype = st
        L.ogs_gpu_richards_step.argtypes = [vp, C.POINTER(AssemblyParams), C.POINTER(RichardsParams), vp, vp, vp,
                                            vp, vp, C.c_int64, C.c_int32, C.POINTER(PicardConfig),
                                            C.POINTER(PicardStats)]
        L.ogs_gpu_richards_step.restype = st
        cp = C.c_char_p
        i64p = C.POINTER(C.c_int64)
        L.ogs_deck_read.argtypes = [cp, cp, cp, C.POINTER(vp)]
        L.ogs_deck_destroy.argtypes = [vp]
        L.ogs_deck_mesh.argtypes = [vp, C.POINTER(MeshDesc), C.POINTER(C.c_double)]
        L.ogs_deck_geo_nodes.argtypes = [vp, cp, cp, vp, C.c_int64, i64p]
        L.ogs_deck_dirichlet.argtypes = [vp, cp, cp, vp, vp, C.c_int64, i64p]
        for name in ("ogs_deck_read", "ogs_deck_destroy", "ogs_deck_mesh", "ogs_deck_geo_nodes",
                     "ogs_deck_dirichlet"):
            getattr(L, name).restype = st
        L.ogs_gpu_kernel_launches.argtypes = [C.c_int32]
        L.ogs_gpu_kernel_launches.restype = C.c_int64
        L.ogs_gpu_selftest_barrier.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]
        L.ogs_gpu_selftest_barrier.restype = st
        for name in ("ogs_gpu_mesh_create", "ogs_gpu_mesh_destroy", "ogs_gpu_mesh_info",
                     "ogs_gpu_system_create", "ogs_gpu_system_destroy", "ogs_gpu_configure",
                     "ogs_gpu_initialize", "ogs_gpu_assemble", "ogs_gpu_set_dirichlet",
                     "ogs_gpu_solve", "ogs_gpu_gp_velocity", "ogs_gpu_get_csr", "ogs_gpu_get_rhs",
                     "ogs_gpu_get_x", "ogs_gpu_spmv", "ogs_gpu_get_ilu0"):
            getattr(L, name).restype = st
        L.ogs_gpu_debug_oob.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.ogs_gpu_debug_oob.restype = st
        L.ogs_gpu_debug_fp32_product.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ogs_gpu_debug_fp32_product.restype = st
        _LIB = L
    return _LIB


def debug_oob():
    """(site, index) of the first out-of-range index met since the last
    call (debug build); (0, 0) none, (-1, 0) a build without the checks."""
    site, index = C.c_int64(), C.c_int64()
    _check(lib().ogs_gpu_debug_oob(C.byref(site), C.byref(index)))
    return site.value, index.value


def _check(status: int, allow=()):
    if status != OK and status not in allow:
        raise OgsError(status, lib().ogs_gpu_last_error().decode())
    return status


def _ptr(a):
    """Raw pointer of a numpy array or torch tensor (None passes through)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)}")


def _f64(a):
    if a is None or hasattr(a, "data_ptr"):
        return a
    return np.ascontiguousarray(a, dtype=np.float64)


def selftest_barrier(which: int, grid: int = 0, spin_limit: int = 0, withhold: bool = False) -> dict:
    """ogs_gpu_selftest_barrier: one grid barrier of the persistent FP32 CG
    kernel (which 0) or of the batch kernel (1), optionally with block 0
    withholding its arrival, or the ILU(0) row waits (2) with row 0 left
    unpublished; returns status, blocks (rows) passed and the error text."""
    n = C.c_int32(0)
    status = lib().ogs_gpu_selftest_barrier(which, grid, spin_limit, 1 if withhold else 0, C.byref(n))
    return {"status": status, "passed": n.value, "error": lib().ogs_gpu_last_error().decode()}


def kernel_launches(reset: bool = False) -> int:
    return int(lib().ogs_gpu_kernel_launches(1 if reset else 0))


class GpuMesh:
    """CSR pattern + slot map of a mesh on the device (SparseTable)."""

    def __init__(self, mesh, gauss_points: int = 3):
        self.mesh = mesh
        self._keep = [np.ascontiguousarray(mesh.x, dtype=np.float64),
                      np.ascontiguousarray(mesh.y, dtype=np.float64),
                      np.ascontiguousarray(mesh.z, dtype=np.float64),
                      np.ascontiguousarray(mesh.conn, dtype=np.int32)]
        d = MeshDesc(mesh.elem_type, mesh.dim, mesh.n_nodes, mesh.n_elements,
                     _ptr(self._keep[0]), _ptr(self._keep[1]),
                     _ptr(self._keep[2]) if mesh.dim == 3 else None, _ptr(self._keep[3]),
                     gauss_points)
        h = C.c_void_p()
        _check(lib().ogs_gpu_mesh_create(C.byref(d), C.byref(h)))
        self.h = h
        n, nnz = C.c_int64(), C.c_int64()
        _check(lib().ogs_gpu_mesh_info(h, C.byref(n), C.byref(nnz)))
        self.n_rows, self.nnz = n.value, nnz.value
        self.n_gauss = int(lib().ogs_gpu_mesh_gauss_points(h))
        self.ilu_tiles = int(lib().ogs_gpu_mesh_ilu_tiles(h))

    def close(self):
        if getattr(self, "h", None):
            lib().ogs_gpu_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LinearEQS:
    """Mirror of Math_Group::Linear_EQS (FEM/equation_class.h:56) on the GPU."""

    def __init__(self, gmesh: GpuMesh, stream=None):
        self.gmesh = gmesh
        h = C.c_void_p()
        sptr = None if stream is None else getattr(stream, "cuda_stream", stream)
        _check(lib().ogs_gpu_system_create(gmesh.h, sptr, C.byref(h)))
        self.h = h
        self.n = gmesh.n_rows
        self.last_stats = SolveStats()

    def close(self):
        if getattr(self, "h", None):
            lib().ogs_gpu_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # Linear_EQS::ConfigNumerics
    def ConfigNumerics(self, ls_method=LS_BICGSTAB, ls_precond=PRECOND_JACOBI,
                       ls_max_iterations=1000, ls_error_tolerance=1e-12,
                       precision=PRECISION_FP64, inner_tol=0.0, check_norm_rhs=True,
                       schedule=SCHEDULE_GRAPH):
        c = SolverConfig(ls_method, ls_precond, ls_max_iterations, precision, ls_error_tolerance,
                         inner_tol, 1 if check_norm_rhs else 0, schedule)
        _check(lib().ogs_gpu_configure(self.h, C.byref(c)))

    # Linear_EQS::Initialize
    def Initialize(self):
        _check(lib().ogs_gpu_initialize(self.h))

    # CRFProcess::GlobalAssembly element loop
    def GlobalAssembly(self, params: AssemblyParams, elem_k=None, u0=None, gp_velocity=None):
        ek, u, gv = _f64(elem_k), _f64(u0), _f64(gp_velocity)
        _check(lib().ogs_gpu_assemble(self.h, C.byref(params), _ptr(ek), _ptr(u), _ptr(gv)))

    # RICHARDS_FLOW: AssembleParabolicEquation + Assemble_Gravity at the iterate
    def AssembleRichards(self, params: AssemblyParams, r: RichardsParams, elem_k, p_old, p_iter):
        ek, po, pi = _f64(elem_k), _f64(p_old), _f64(p_iter)
        _check(lib().ogs_gpu_assemble_richards(self.h, C.byref(params), C.byref(r), _ptr(ek), _ptr(po), _ptr(pi)))

    # one RICHARDS_FLOW time step by Picard iteration (ExecuteNonLinear);
    # p_iter (numpy float64 or device tensor) is updated in place
    def RichardsStep(self, params: AssemblyParams, r: RichardsParams, elem_k, p_old, p_iter, rows, values,
                     mode=DIRICHLET_SYMMETRIC, error_method=ENORM, max_iterations=20, tolerance=1e-6,
                     allow_fail=False) -> dict:
        ek, po = _f64(elem_k), _f64(p_old)
        rr = rows if hasattr(rows, "data_ptr") else np.ascontiguousarray(rows, dtype=np.int64)
        vv = _f64(values)
        cfg = PicardConfig(error_method, max_iterations, tolerance)
        stt = PicardStats()
        status = lib().ogs_gpu_richards_step(self.h, C.byref(params), C.byref(r), _ptr(ek), _ptr(po), _ptr(p_iter),
                                             _ptr(rr), _ptr(vv), len(rr), mode, C.byref(cfg), C.byref(stt))
        if not allow_fail:
            _check(status)
        return {"status": status, "iterations": stt.iterations, "converged": bool(stt.converged),
                "diverged": bool(stt.diverged), "linear_iterations": stt.linear_iterations, "error": stt.error,
                "solve_ms": stt.solve_ms}

    # forget the transport operators stored under memory_type > 0 (the
    # reference's first time step recomputes them)
    def ResetOperators(self):
        _check(lib().ogs_gpu_cache_reset(self.h))

    # SetKnownX_i over a node set (IncorporateBoundaryConditions)
    def SetKnownX(self, rows, values, mode=DIRICHLET_ROW_ONLY):
        r = rows if hasattr(rows, "data_ptr") else np.ascontiguousarray(rows, dtype=np.int64)
        v = _f64(values)
        _check(lib().ogs_gpu_set_dirichlet(self.h, _ptr(r), _ptr(v), len(r), mode))

    # Linear_EQS::Solver; x is updated in place; returns the iteration count
    def Solver(self, x, allow_fail=False):
        st = SolveStats()
        status = lib().ogs_gpu_solve(self.h, _ptr(x), C.byref(st))
        self.last_stats = st
        if not allow_fail:
            _check(status)
        return st.iterations

    def stats(self) -> dict:
        s = self.last_stats
        return {"iterations": s.iterations, "status": s.status, "rel_residual": s.rel_residual,
                "b_norm": s.b_norm, "refinements": s.refinements, "fp64_fallback": s.fp64_fallback,
                "solve_ms": s.solve_ms, "fp32_operator": s.fp32_operator}

    def gp_velocity(self, params: AssemblyParams, elem_k, u, out=None):
        ng = self.gmesh.n_gauss
        if out is None:
            out = np.zeros((self.gmesh.mesh.n_elements, ng, 3))
        _check(lib().ogs_gpu_gp_velocity(self.h, C.byref(params), _ptr(_f64(elem_k)),
                                         _ptr(_f64(u)), _ptr(out)))
        return out

    def profile(self, enable: bool) -> dict:
        """Turns SpMV timing on/off; returns (and resets) the totals so far."""
        p = Profile()
        _check(lib().ogs_gpu_profile(self.h, 1 if enable else 0, C.byref(p)))
        return {"spmv_ms": p.spmv_ms, "spmv_launches": p.spmv_launches, "solve_ms": p.solve_ms,
                "solves": p.solves, "persist_ms": p.persist_ms, "persist_iters": p.persist_iters}

    def get_csr(self):
        nnz = self.gmesh.nnz
        rp = np.zeros(self.n + 1, dtype=np.int64)
        col = np.zeros(nnz, dtype=np.int64)
        val = np.zeros(nnz)
        _check(lib().ogs_gpu_get_csr(self.h, _ptr(rp), _ptr(col), _ptr(val)))
        return rp, col, val

    def get_values(self, out=None):
        if out is None:
            out = np.zeros(self.gmesh.nnz)
        _check(lib().ogs_gpu_get_csr(self.h, None, None, _ptr(out)))
        return out

    def get_ilu0(self):
        """ILU(0) factors of the last ls_precond 100 solve on the CSR pattern."""
        out = np.zeros(self.gmesh.nnz)
        _check(lib().ogs_gpu_get_ilu0(self.h, _ptr(out)))
        return out

    def get_rhs(self, out=None):
        if out is None:
            out = np.zeros(self.n)
        _check(lib().ogs_gpu_get_rhs(self.h, _ptr(out)))
        return out

    def spmv(self, x, out=None):
        if out is None:
            out = np.zeros(self.n)
        _check(lib().ogs_gpu_spmv(self.h, _ptr(_f64(x)), _ptr(out)))
        return out

    def debug_fp32_product(self, x):
        """(y_rows, y_lines): the FP32 product of the Jacobi-scaled lattice
        operator on x by the row kernel and by the four-rows-per-thread
        kernel (after a FP32_REFINED solve on a hex lattice)."""
        xs = np.ascontiguousarray(x, dtype=np.float32)
        y_rows, y_lines = np.zeros(self.n, np.float32), np.zeros(self.n, np.float32)
        _check(lib().ogs_gpu_debug_fp32_product(self.h, _ptr(xs), _ptr(y_rows), _ptr(y_lines)))
        return y_rows, y_lines


def csr_cg_noalloc(row_ptr, col, val, b, x, max_iter=1000, tol=1e-10, stream=None):
    """ogs_gpu_csr_cg_noalloc on torch CUDA tensors (int32 row_ptr/col,
    float64 val/b/x; x updated in place).  Returns the solve statistics."""
    st = SolveStats()
    sptr = None if stream is None else getattr(stream, "cuda_stream", stream)
    status = lib().ogs_gpu_csr_cg_noalloc(len(b), _ptr(row_ptr), _ptr(col), _ptr(val), _ptr(b), _ptr(x),
                                         max_iter, tol, sptr, C.byref(st))
    _check(status, allow=(NOT_CONVERGED,))
    return {"iterations": st.iterations, "status": st.status, "rel_residual": st.rel_residual,
            "b_norm": st.b_norm}


class Batch:
    """Monte-Carlo batch of steady GROUNDWATER_FLOW realisations on
    structured hex boxes (ogs_gpu_batch_*): one persistent launch assembles
    and solves them all.

        b = Batch([(nx, ny, nz, elem_k, h_left, h_right), ...], tol=1e-10)
        b.autotune()
        stats = b.solve()          # list of dicts, one per realisation
        heads = b.heads()          # list of arrays (nx*ny*nz each)
    """

    def __init__(self, reals, hx=1.0, hy=1.0, hz=1.0, tol=1e-10, max_iter=5000, inner_tol=0.0,
                 time_unit_factor=1.0, stream=None):
        self.h = None
        cfg = BatchConfig(hx, hy, hz, time_unit_factor, tol, inner_tol, max_iter, 0)
        arr = (BatchRealisation * len(reals))()
        self._keep = []
        self.sizes = []
        for i, (nx, ny, nz, ek, hl, hr) in enumerate(reals):
            if not hasattr(ek, "data_ptr"):  # numpy / sequence (host); tensors are used in place
                ek = np.ascontiguousarray(ek, dtype=np.float64)
            size = ek.numel() if hasattr(ek, "numel") else ek.size
            if size != (nx - 1) * (ny - 1) * (nz - 1):
                raise ValueError(f"realisation {i}: {size} conductivities for {nx}x{ny}x{nz} nodes")
            self._keep.append(ek)
            arr[i] = BatchRealisation(nx, ny, nz, 0, _ptr(ek), hl, hr)
            self.sizes.append(nx * ny * nz)
        h = C.c_void_p()
        s = None if stream is None else C.c_void_p(stream)
        _check(lib().ogs_gpu_batch_create(C.byref(cfg), arr, len(reals), s, C.byref(h)))
        self.h = h
        self._keep = None
        rows, elems = C.c_int64(), C.c_int64()
        _check(lib().ogs_gpu_batch_info(self.h, C.byref(rows), C.byref(elems)))
        self.rows, self.elements = rows.value, elems.value
        self.n = len(reals)

    def close(self):
        if self.h is not None and _LIB is not None:
            lib().ogs_gpu_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _tuning_dict(t):
        return {"tile_rows": t.tile_rows, "block_threads": t.block_threads,
                "blocks_per_sm": t.blocks_per_sm, "graph": t.graph, "ms_per_step": t.ms_per_step}

    def autotune(self) -> dict:
        t = BatchTuning()
        _check(lib().ogs_gpu_batch_autotune(self.h, C.byref(t)))
        return self._tuning_dict(t)

    def set_tuning(self, tile_rows, block_threads, blocks_per_sm):
        t = BatchTuning(tile_rows, block_threads, blocks_per_sm, 0, 0.0)
        _check(lib().ogs_gpu_batch_set_tuning(self.h, C.byref(t)))

    def set_k(self, elem_k_all):
        k = elem_k_all if hasattr(elem_k_all, "data_ptr") else _f64(elem_k_all)
        _check(lib().ogs_gpu_batch_set_k(self.h, _ptr(k)))

    def solve(self, allow_fail=False) -> list:
        st = (BatchStats * self.n)()
        status = lib().ogs_gpu_batch_solve(self.h, st)
        if not allow_fail:
            _check(status)
        return [{"iterations": s.iterations, "status": s.status, "refinements": s.refinements,
                 "rel_residual": s.rel_residual, "finish_ms": s.finish_ms} for s in st]

    def heads_flat(self, out=None):
        if out is None:
            out = np.zeros(self.rows)
        _check(lib().ogs_gpu_batch_get_heads(self.h, _ptr(out)))
        return out

    def heads(self) -> list:
        flat = self.heads_flat()
        return np.split(flat, np.cumsum(self.sizes)[:-1])


def solver_config(method=LS_CG, precond=PRECOND_JACOBI, max_iter=20000, tol=1e-10,
                  precision=PRECISION_FP64, inner_tol=0.0, check_norm_rhs=True,
                  schedule=SCHEDULE_GRAPH) -> SolverConfig:
    return SolverConfig(method, precond, max_iter, precision, tol, inner_tol, 1 if check_norm_rhs else 0,
                        schedule)


class Server:
    """Request server with continuous batching (ogs_gpu_server_*).

        srv = Server(budget_bytes=0, max_active=64)
        c = srv.add_class(gmesh, REQUEST_FLOW, params, bc_rows, bc_values, DIRICHLET_SYMMETRIC,
                          solver_config(precision=PRECISION_FP32_REFINED))
        rid = srv.submit(c, k_device_tensor, 1e-10, out_tensor)
        while srv.progress() != (0, 0): ...
        srv.result(rid)
    """

    def __init__(self, budget_bytes=0, max_active=64, flags=0):
        self.h = None
        h = C.c_void_p()
        _check(lib().ogs_gpu_server_create(int(budget_bytes), int(max_active), int(flags), C.byref(h)))
        self.h = h
        self._refs = {}

    def close(self):
        if self.h is not None and _LIB is not None:
            lib().ogs_gpu_server_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_class(self, gmesh, kind, params, bc_rows, bc_values, bc_mode, solver, flow_params=None,
                  flow_head=None) -> int:
        rows = np.ascontiguousarray(bc_rows, dtype=np.int64)
        vals = np.ascontiguousarray(bc_values, dtype=np.float64)
        head = None if flow_head is None else _f64(flow_head)
        c = ServerClass()
        c.mesh = gmesh.h
        c.kind = kind
        c.bc_mode = bc_mode
        c.params = params
        if flow_params is not None:
            c.flow_params = flow_params
        c.n_elements = gmesh.mesh.n_elements
        c.flow_head = _ptr(head)
        c.bc_rows = rows.ctypes.data
        c.bc_values = vals.ctypes.data
        c.n_bc = len(rows)
        c.solver = solver
        cid = C.c_int32()
        _check(lib().ogs_gpu_server_add_class(self.h, C.byref(c), C.byref(cid)))
        return cid.value

    def reserve(self, class_id, n_slots):
        _check(lib().ogs_gpu_server_reserve(self.h, class_id, n_slots))

    def submit(self, class_id, elem_k, tol, out) -> int:
        rid = C.c_int64()
        _check(lib().ogs_gpu_server_submit(self.h, class_id, _ptr(elem_k), tol, _ptr(out), C.byref(rid)))
        self._refs[rid.value] = (elem_k, out)  # inputs stay alive until the request is done
        return rid.value

    def progress(self):
        r, q = C.c_int32(), C.c_int32()
        _check(lib().ogs_gpu_server_progress(self.h, C.byref(r), C.byref(q)))
        return r.value, q.value

    def drain(self):
        while self.progress() != (0, 0):
            pass

    def result(self, rid) -> dict:
        r = ServerResult()
        _check(lib().ogs_gpu_server_result(self.h, rid, C.byref(r)))
        if r.state == 2:
            self._refs.pop(rid, None)
        return {"state": r.state, "status": r.status, "iterations": r.iterations,
                "refinements": r.refinements, "rel_residual": r.rel_residual, "latency_ms": r.latency_ms,
                "queue_ms": r.queue_ms, "solve_ms": r.solve_ms, "batch_size": r.batch_size,
                "precision": r.precision, "fp64_fallback": r.fp64_fallback}

    def info(self) -> dict:
        i = ServerInfo()
        _check(lib().ogs_gpu_server_info(self.h, C.byref(i)))
        return {"slots": i.slots, "running": i.running, "queued": i.queued, "completed": i.completed,
                "bytes_used": i.bytes_used, "bytes_budget": i.bytes_budget, "batched": i.batched,
                "fp64_classes": i.fp64_classes}


class Deck:
    """An OGS-5 input deck read by the library's native reader (host only):
    mesh (.msh), geometry (.gli) and CONSTANT Dirichlet conditions (.bc).

    ``mesh`` is a :class:`ogs5_gb300.mesh.Mesh` ready for :class:`GpuMesh`;
    ``dirichlet(pcs_type)`` gives the rows and values for
    ``LinearEQS.SetKnownX`` in the order CRFProcess::bc_node_value holds them
    (FEM/rf_bc_new.cpp:1272-1560)."""

    def __init__(self, msh: str, gli: str | None = None, bc: str | None = None):
        h = C.c_void_p()
        enc = (lambda p: None if p is None else os.fsencode(p))
        _check(lib().ogs_deck_read(enc(msh), enc(gli), enc(bc), C.byref(h)))
        self.h = h

    @property
    def min_edge_length(self) -> float:
        d, h = MeshDesc(), C.c_double()
        lib().ogs_deck_mesh(self.h, C.byref(d), C.byref(h))  # h is set even off the GPU path
        return h.value

    @property
    def mesh(self):
        from . import mesh as M
        d = MeshDesc()
        _check(lib().ogs_deck_mesh(self.h, C.byref(d), None))
        nn, ne = d.n_nodes, d.n_elements
        npe = M.NODES_PER_ELEMENT[d.elem_type]
        f64 = C.POINTER(C.c_double)
        x = np.ctypeslib.as_array(C.cast(d.x, f64), (nn,)).copy()
        y = np.ctypeslib.as_array(C.cast(d.y, f64), (nn,)).copy()
        z = (np.ctypeslib.as_array(C.cast(d.z, f64), (nn,)).copy() if d.z else np.zeros(nn))
        conn = np.ctypeslib.as_array(C.cast(d.connectivity, C.POINTER(C.c_int32)), (ne * npe,))
        return M.Mesh(d.elem_type, d.dim, x, y, z, conn.reshape(ne, npe).copy())

    def geo_nodes(self, geo_type: str, name: str) -> np.ndarray:
        n = C.c_int64()
        _check(lib().ogs_deck_geo_nodes(self.h, geo_type.encode(), name.encode(), None, 0, C.byref(n)))
        rows = np.empty(n.value, dtype=np.int64)
        _check(lib().ogs_deck_geo_nodes(self.h, geo_type.encode(), name.encode(), _ptr(rows), len(rows),
                                        C.byref(n)))
        return rows

    def dirichlet(self, pcs_type: str, primary_variable: str | None = None):
        n = C.c_int64()
        pv = None if primary_variable is None else primary_variable.encode()
        _check(lib().ogs_deck_dirichlet(self.h, pcs_type.encode(), pv, None, None, 0, C.byref(n)))
        rows = np.empty(n.value, dtype=np.int64)
        vals = np.empty(n.value, dtype=np.float64)
        _check(lib().ogs_deck_dirichlet(self.h, pcs_type.encode(), pv, _ptr(rows), _ptr(vals), len(rows),
                                        C.byref(n)))
        return rows, vals

    def close(self):
        if getattr(self, "h", None):
            lib().ogs_deck_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
