/*
 * ogs_gpu.h -- C ABI of the GB300 flow/transport path for OpenGeoSys 5.
 *
 * The OGS-5 host code keeps its own process and solver surface
 * (CRFProcess::GlobalAssembly, Linear_EQS::Solver); at the call sites listed
 * beside each entry point it calls into this library instead of running its
 * serial element loop and CPU Krylov solver.  All arithmetic is FP64 unless a
 * solver configuration asks for the FP32-inner / FP64-refinement mode.
 *
 * Conventions
 *   - Every entry point returns an ogs_status; nothing aborts or traps.
 *     ogs_gpu_last_error() returns a text for the last failure on the
 *     calling thread.
 *   - Array arguments are plain pointers.  Host pointers are copied to the
 *     device inside the call; device pointers (cudaMalloc'd memory of the
 *     current device) are used in place.
 *   - Row, column and node indices are zero based; the equation index of a
 *     node equals its node index (linear elements, one DOF per node), as in
 *     CFEMesh::RenumberNodesForGlobalAssembly for meshes without quadratic
 *     nodes (MSH/msh_mesh.cpp:1308).
 *   - One ogs_system per host thread or stream; handles are not thread safe.
 */
#ifndef OGS_GPU_H
#define OGS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum
{
    OGS_OK = 0,
    OGS_NOT_CONVERGED = 1, /* max_iter reached (Linear_EQS::Message warning) */
    OGS_BREAKDOWN = 2,     /* |rho| or |omega| < DBL_MIN in BiCGStab       */
    OGS_NONFINITE = 3,     /* NaN/Inf in a residual norm                   */
    OGS_OOM = 4,
    OGS_BAD_ARG = 5,
    OGS_CUDA_ERROR = 6,
    OGS_SINGULAR_JACOBIAN = 7 /* |det J| < DBL_EPSILON (fem_ele.cpp:639,695) */
} ogs_status;

/* Element types on the path (MshElemType QUAD, HEXAHEDRON, TETRAHEDRON). */
typedef enum
{
    OGS_ELEM_QUAD4 = 0,
    OGS_ELEM_HEX8 = 1,
    OGS_ELEM_TET4 = 2
} ogs_elem_type;

/* Process types on the path (FiniteElement::ProcessType). */
typedef enum
{
    OGS_PCS_GROUNDWATER_FLOW = 0,
    OGS_PCS_LIQUID_FLOW = 1,
    OGS_PCS_MASS_TRANSPORT = 2,
    OGS_PCS_RICHARDS_FLOW = 3  /* through ogs_gpu_assemble_richards only */
} ogs_pcs_type;

/* Dirichlet treatment.  ROW_ONLY is CSparseMatrix::Diagonize of the SP
 * build (FEM/matrix_class.cpp:1663): the row is zeroed except the diagonal
 * and b_i = a_ii * value; the column stays.  SYMMETRIC is MXRandbed of the
 * legacy build (FEM/matrix_routines.cpp:2314): the column is lifted into the
 * right-hand side, row and column are zeroed, the diagonal is kept. */
typedef enum
{
    OGS_DIRICHLET_ROW_ONLY = 0,
    OGS_DIRICHLET_SYMMETRIC = 1
} ogs_dirichlet_mode;

/* Linear solver codes of $LINEAR_SOLVER (FEM/equation_class.cpp:197-244). */
enum
{
    OGS_LS_BICGSTAB = 2,
    OGS_LS_CG = 5
};
/* Preconditioner codes of $LINEAR_SOLVER (FEM/equation_class.cpp:294-308). */
enum
{
    OGS_PRECOND_NONE = 0,
    OGS_PRECOND_JACOBI = 1,
    OGS_PRECOND_ILU0 = 100
};
/* Arithmetic of the Krylov iteration. */
enum
{
    OGS_PRECISION_FP64 = 0,
    OGS_PRECISION_FP32_REFINED = 1, /* FP32 matrix + inner sweeps, FP64 IR */
    OGS_PRECISION_FP32_CELLS = 2    /* as FP32_REFINED, but on a regular hex
                                       lattice whose matrix is a sum of
                                       scaled box-element matrices (flow
                                       without mass lumping) the inner CG
                                       applies the operator from one FP32
                                       coefficient per cell (4 B per cell
                                       instead of 56 B per row); elsewhere
                                       the stored FP32 operator            */
};

/* Mesh description: the data CFEMesh hands to SparseTable and the element
 * loop (node coordinates, element connectivity).  Host arrays. */
typedef struct
{
    int32_t elem_type;          /* ogs_elem_type                               */
    int32_t dim;                /* 2 for quad meshes in the x-y plane, else 3  */
    int64_t n_nodes;
    int64_t n_elements;
    const double* x;            /* node coordinates, n_nodes each              */
    const double* y;
    const double* z;            /* may be NULL when dim == 2                   */
    const int32_t* connectivity;/* n_elements * nodes_per_element, element-major,
                                   OGS node order of CElem::nodes_index       */
    int32_t gauss_points;       /* $ELE_GAUSS_POINTS for quad/hex (1..3);
                                   tets always use the 5-point rule            */
} ogs_mesh_desc;

/* Material and time-stepping parameters of one assembly call.  Each field
 * names the OGS-5 source of the value. */
typedef struct
{
    int32_t pcs_type;          /* ogs_pcs_type                                 */
    int32_t steady;            /* TimType::STEADY.  MASS_TRANSPORT: no mass
                                  matrix (fem_ele_std.cpp:8549).  Flow
                                  processes ignore it: AssembleParabolicEquation
                                  (:7702) keeps M/dt, so a steady flow deck is
                                  one with storage 0                           */
    double dt;                 /* pcs->Tim->time_step_length                   */
    double theta;              /* m_num->ls_theta, MT time weighting           */
    double nls_relaxation;     /* m_num->nls_relaxation, flow LHS weight;
                                  < DBL_MIN means 1 (fem_ele_std.cpp:7715)     */
    double time_unit_factor;   /* CElement::time_unit_factor (1 for seconds)  */
    double storage;            /* StorageFunction, storage_model 1             */
    double porosity;           /* Porosity, constant model                     */
    double drho_dp;            /* LIQUID_FLOW: FluidProp->drho_dp, rho = rho_0 */
    double viscosity;          /* LIQUID_FLOW: FluidProp->Viscosity()          */
    double density;            /* LIQUID_FLOW: FluidProp->Density()            */
    double gravity;            /* gravity_constant; < DBL_EPSILON = HEAD form  */
    int32_t gravity_on;        /* coordinate_system % 10 == 2 and
                                  FluidProp->CheckGravityCalculation()         */
    int32_t mass_lumping;      /* m_num->ele_mass_lumping (rf_num_new.cpp:125,
                                  684): the mass matrix becomes diagonal,
                                  CalCoefMass * element volume / nodes
                                  (CalcLumpedMass, fem_ele_std.cpp:4598-4660) */
    double alpha_l;            /* MT: mass_dispersion_longitudinal             */
    double alpha_t;            /* MT: mass_dispersion_transverse               */
    double diffusion;          /* MT: Daq * TortuosityFunction                 */
    double decay;              /* MT: CalcElementDecayRateNew                  */
    double retardation;        /* MT: CalcElementRetardationFactorNew          */
    double saturation;         /* MT: SATURATION1 of the flow process (1)      */
    int32_t supg_method;       /* MT: m_num->ele_supg_method (rf_num_new.cpp:704):
                                  0 off, 1 tau from the Langevin function,
                                  2 tau with the time step
                                  (CalcSUPGCoefficient, fem_ele_std.cpp:3908) */
    int32_t supg_length;       /* ele_supg_method_length: 0 longest edge,
                                  1 shortest, 2 "average" (the reference sums
                                  edges 1..n-1 and divides by n)
                                  (CalcSUPGEffectiveElemenetLength, :4034)     */
    int32_t supg_diffusivity;  /* ele_supg_method_diffusivity: 0 largest entry
                                  of the dispersion tensor, 1 smallest, 2 the
                                  last diagonal entry (the reference assigns
                                  rather than sums the squares)                */
    int32_t memory_type;       /* MT: pcs->Memory_Type ($MEMORY_TYPE, rf_pcs.cpp
                                  :2142-2146, 972).  0: element matrices recomputed
                                  every assembly.  > 0: the first assembly
                                  after creation or ogs_gpu_cache_reset stores
                                  the mass and the Laplace + advection +
                                  storage operators, later assemblies combine
                                  the stored ones with this call's dt, theta
                                  and u0 and ignore gp_velocity, porosity and
                                  the other material values
                                  (fem_ele_std.cpp:8534-8588)                  */
} ogs_assembly_params;

/* Linear_EQS::ConfigNumerics inputs (CNumerics, FEM/rf_num_new.h:34-60). */
typedef struct
{
    int32_t method;            /* ls_method: OGS_LS_BICGSTAB or OGS_LS_CG      */
    int32_t precond;           /* ls_precond: 0, 1 (Jacobi), 100 (ILU(0))      */
    int32_t max_iter;          /* ls_max_iterations                            */
    int32_t precision;         /* OGS_PRECISION_*                              */
    double tol;                /* ls_error_tolerance (relative to |b|)         */
    double inner_tol;          /* FP32 mode: the FP64 residual is recomputed
                                  when the FP32 residual fell by this factor
                                  since the last replacement (0 selects 1e-2) */
    int32_t check_norm_rhs;    /* 1: keep Linear_EQS::CheckNormRHS, i.e.
                                  return at once when |b|/|b_prev| < tol
                                  (equation_class.cpp:1104-1121)               */
    int32_t schedule;          /* FP32 mode: OGS_SCHEDULE_GRAPH (0) two
                                  kernels per iteration in captured graphs;
                                  OGS_SCHEDULE_PERSISTENT (1) many iterations
                                  in one cooperative launch with two grid
                                  barriers per iteration (graph schedule where
                                  the device cannot launch it)               */
} ogs_solver_config;

enum
{
    OGS_SCHEDULE_GRAPH = 0,
    OGS_SCHEDULE_PERSISTENT = 1
};

typedef struct
{
    int32_t iterations;        /* Krylov iterations (FP32 iterations in FP32 mode) */
    int32_t status;            /* ogs_status of the solve                      */
    double rel_residual;       /* |r| / |b| at exit (Linear_EQS::error)        */
    double b_norm;             /* |b| at entry (Linear_EQS::bNorm)             */
    int32_t refinements;       /* FP32 mode: FP64 residual replacements        */
    int32_t fp64_fallback;     /* FP32 mode: 1 if the FP32 cycles stopped
                                  gaining (a plateau of the FP32 residual, or
                                  a replacement that lowered the FP64
                                  residual far less than the FP32 recurrence
                                  claimed) and the solve finished in FP64 CG
                                  from x (iterations count both phases)       */
    double solve_ms;           /* device time of the solve, CUDA events        */
    int32_t fp32_operator;     /* FP32 mode: the inner CG's operator, 0 FP32
                                  diagonal offsets, 1 FP32 SELL-32, 2 one
                                  coefficient per cell of a regular hex
                                  lattice; -1 in FP64 mode                    */
    int32_t pad0;
} ogs_solve_stats;

typedef struct ogs_mesh ogs_mesh;
typedef struct ogs_system ogs_system;

/* Text of the last error on the calling thread ("" if none). */
const char* ogs_gpu_last_error(void);

/* Library version string. */
const char* ogs_gpu_version(void);

/* Builds the CSR pattern of the node-node adjacency and the element -> CSR
 * slot map on the device.  Replaces CFEMesh::ConnectedNodes
 * (MSH/msh_mesh.cpp:2931), SparseTable::SparseTable in CRS storage
 * (FEM/matrix_class.cpp:691-776) and the per-entry search of
 * CSparseMatrix::operator() (FEM/matrix_class.cpp:1178-1237).  Called where
 * CRFProcess::CreateEQS_LinearSolver creates the SparseTable
 * (FEM/rf_pcs.cpp:13455-13481). */
ogs_status ogs_gpu_mesh_create(const ogs_mesh_desc* desc, ogs_mesh** out);
ogs_status ogs_gpu_mesh_destroy(ogs_mesh* mesh);
/* Number of rows and stored entries of the pattern. */
ogs_status ogs_gpu_mesh_info(const ogs_mesh* mesh, int64_t* n_rows,
                             int64_t* nnz);

/* Creates the equation system on a mesh: matrix values, b, x and Krylov
 * buffers.  Replaces `new Linear_EQS(*sp, dof)` (FEM/equation_class.cpp:85).
 * stream: a cudaStream_t, or NULL for the default stream. */
ogs_status ogs_gpu_system_create(ogs_mesh* mesh, void* stream,
                                 ogs_system** out);
ogs_status ogs_gpu_system_destroy(ogs_system* sys);

/* Linear_EQS::ConfigNumerics (FEM/equation_class.cpp:191-318). */
ogs_status ogs_gpu_configure(ogs_system* sys, const ogs_solver_config* cfg);

/* ---- RICHARDS_FLOW -------------------------------------------------------
 * Material curves of the unsaturated medium (CMediumProperties, the $MMP
 * keywords $CAPILLARY_PRESSURE and $PERMEABILITY_SATURATION). */
typedef struct
{
    int32_t capillary_model;   /* capillary_pressure_model: 4 van Genuchten,
                                  6 Brooks-Corey                               */
    int32_t permeability_model;/* permeability_saturation_model[0]: 4 van
                                  Genuchten-Mualem, 6 Brooks-Corey             */
    double pb;                 /* capillary_pressure_values[0]: entry pressure */
    double slr, slm;           /* capillary_pressure_values[1], [2]: residual and
                                  maximum saturation of the pressure curve    */
    double m;                  /* capillary_pressure_values[3]: exponent      */
    double kr_slr, kr_slm;     /* residual_saturation[0], maximum_saturation[0] */
    double kr_m;               /* saturation_exponent[0]                      */
    double kr_min;             /* minimum_relative_permeability               */
} ogs_richards_params;

/* One RICHARDS_FLOW assembly (fem_ele_std.cpp:9470-9481:
 * AssembleParabolicEquation + Assemble_Gravity) with the storage and
 * conductivity of the iterate p_iter at every Gauss point (CalCoefMass
 * :1721-1770, CalCoefLaplace :2614-2640, saturation curves
 * rf_mmp_new.cpp:5243-5520 and 2490-2640), added to A and b:
 *   A += M(p_iter) / dt + relax0 L(p_iter)
 *   b += (M(p_iter) / dt - relax1 L(p_iter)) p_old + gravity(p_iter).
 * p uses pcs_type OGS_PCS_RICHARDS_FLOW, dt, nls_relaxation,
 * time_unit_factor, storage, porosity, drho_dp, viscosity, density, gravity,
 * gravity_on, mass_lumping (the lumped storage taken at the element centre,
 * CalcLumpedMass).  elem_k: intrinsic permeability per element. */
ogs_status ogs_gpu_assemble_richards(ogs_system* sys, const ogs_assembly_params* p, const ogs_richards_params* r,
                                     const double* elem_k, const double* p_old, const double* p_iter);

/* $NON_LINEAR_ITERATIONS of a Picard process (CNumerics). */
typedef struct
{
    int32_t error_method;      /* FiniteElement::ErrorMethod: 1 LMAX, 2 ENORM,
                                  3 EVNORM, 4 ERNORM                           */
    int32_t max_iterations;    /* nls_max_iterations                          */
    double tolerance;          /* nls_error_tolerance[0]                      */
} ogs_picard_config;

typedef struct
{
    int32_t iterations;        /* Picard iterations run                       */
    int32_t converged;         /* error / tolerance <= 1 reached              */
    int32_t diverged;          /* two iterations in a row gained < 1 %        */
    int32_t linear_iterations; /* Krylov iterations, all Picard iterations    */
    double error;              /* last error / tolerance                       */
    double solve_ms;           /* device time of the whole step               */
} ogs_picard_stats;

/* One time step of RICHARDS_FLOW by Picard iteration: the loop of
 * CRFProcess::ExecuteNonLinear with nls_method PICARD (rf_pcs.cpp:9636-9960)
 * around CRFProcess::Execute (:4695-5080).  Each iteration: A = 0, b = 0,
 * ogs_gpu_assemble_richards at the iterate, the Dirichlet set (mode as
 * ogs_gpu_set_dirichlet), the configured linear solve from the iterate,
 * the error of CalcIterationNODError (:9170-9600) divided by the
 * tolerance, and the update iterate = (1 - theta) iterate + theta x with
 * theta = 1 - nls_relaxation (1 once converged).  Stops when the error is
 * <= 1, after two iterations that each lowered it by less than 1 %, or after
 * max_iterations.  p_iter: the first iterate in, the last one out (host or
 * device, n_nodes doubles).  Returns OGS_NOT_CONVERGED when the loop ended
 * unconverged. */
ogs_status ogs_gpu_richards_step(ogs_system* sys, const ogs_assembly_params* p, const ogs_richards_params* r,
                                 const double* elem_k, const double* p_old, double* p_iter,
                                 const int64_t* bc_rows, const double* bc_values, int64_t n_bc, int32_t bc_mode,
                                 const ogs_picard_config* nls, ogs_picard_stats* stats);

/* Forgets the transport operators stored under memory_type > 0, so that the
 * next such assembly computes and stores them again: the reference's first
 * time step (aktueller_zeitschritt == 1, fem_ele_std.cpp:8534). */
ogs_status ogs_gpu_cache_reset(ogs_system* sys);

/* Linear_EQS::Initialize (FEM/equation_class.cpp:325-332): A = 0, b = 0. */
ogs_status ogs_gpu_initialize(ogs_system* sys);

/* One global assembly: the element loop of CRFProcess::GlobalAssembly
 * (FEM/rf_pcs.cpp:5738-5757) calling CFiniteElementStd::Assembly
 * (FEM/fem_ele_std.cpp:9367) for GROUNDWATER_FLOW, LIQUID_FLOW or
 * MASS_TRANSPORT, with add2GlobalMatrixII (fem_ele_std.cpp:8272-8352) and the
 * RHS scatter.  Adds into the current A and b (call ogs_gpu_initialize
 * first, as CRFProcess::Execute does).
 *   elem_k       flow: conductivity (GWF) or permeability (LIQUID) per
 *                element, isotropic (PermeabilityTensor, rf_mmp_new.cpp:4517);
 *                ignored for MASS_TRANSPORT (may be NULL)
 *   u0           primary variable of the previous time level per node
 *                (NodalVal0 / NodalVal1 of Config, fem_ele_std.cpp:9184)
 *   gp_velocity  MASS_TRANSPORT only: Darcy flux at the Gauss points,
 *                n_elements * n_gauss * 3, from ogs_gpu_gp_velocity. */
ogs_status ogs_gpu_assemble(ogs_system* sys, const ogs_assembly_params* p,
                            const double* elem_k, const double* u0,
                            const double* gp_velocity);

/* Dirichlet values on a node set: the SetKnownX_i loop of
 * CRFProcess::IncorporateBoundaryConditions (FEM/rf_pcs.cpp:6930-6995).
 * Also records the values so that ogs_gpu_solve starts from an x0 that
 * carries them. */
ogs_status ogs_gpu_set_dirichlet(ogs_system* sys, const int64_t* rows,
                                 const double* values, int64_t n_rows,
                                 int32_t mode);

/* Linear_EQS::Solver (FEM/equation_class.cpp:857-895), CG
 * (equation_class.cpp:1129-1187) or BiCGStab (equation_class.cpp:1287-1420)
 * with Jacobi (CSparseMatrix::Precond_Jacobi, matrix_class.cpp:1786-1822) or
 * ILU(0).  x_inout: initial guess in, solution out (n_rows doubles).  Called
 * at `iter_lin = eqs_new->Solver()` (FEM/rf_pcs.cpp:4847). */
ogs_status ogs_gpu_solve(ogs_system* sys, double* x_inout,
                         ogs_solve_stats* stats);

/* The same solve split so that one host thread can keep the solves of many
 * systems in flight (no counterpart in the reference): _begin enqueues the
 * start of the solve on the system's stream and returns; _poll checks
 * without blocking whether the GPU has reached the next decision point and,
 * if so, enqueues the next chunk of iterations (finished = 1 once x_inout
 * holds the solution); _end waits for the rest and returns what
 * ogs_gpu_solve returns.  The kernels, launch shapes and order are those of
 * ogs_gpu_solve, so results are bitwise the same.  x_inout must stay valid
 * until _end; for a host array use pinned memory to keep _poll
 * non-blocking. */
ogs_status ogs_gpu_solve_begin(ogs_system* sys, double* x_inout);
ogs_status ogs_gpu_solve_poll(ogs_system* sys, int32_t* finished);
ogs_status ogs_gpu_solve_end(ogs_system* sys, ogs_solve_stats* stats);

/* Gauss-point Darcy flux q = -mat * grad(u) (CFiniteElementStd::Cal_Velocity,
 * FEM/fem_ele_std.cpp:6554-6870, driven by CRFProcess::
 * CalIntegrationPointValue, FEM/rf_pcs.cpp:5915).  q_gp: n_elements * n_gauss
 * * 3 doubles, Gauss point g of element e at [(e * n_gauss + g) * 3]. */
ogs_status ogs_gpu_gp_velocity(ogs_system* sys, const ogs_assembly_params* p,
                               const double* elem_k, const double* u,
                               double* q_gp);

/* Read-back for checks: the CRS arrays of Linear_EQS::Write_BIN
 * (FEM/equation_class.cpp:409, matrix_class.cpp:1403-1460) and b, x. */
ogs_status ogs_gpu_get_csr(const ogs_system* sys, int64_t* row_ptr,
                           int64_t* col, double* val);
ogs_status ogs_gpu_get_rhs(const ogs_system* sys, double* b);
ogs_status ogs_gpu_get_x(const ogs_system* sys, double* x);

/* ILU(0) factors of the last solve with ls_precond 100, on the CSR pattern
 * of ogs_gpu_get_csr (nnz doubles): unit lower L below the diagonal, U on
 * and above it.  The SP build substitutes Jacobi for precond 100
 * (FEM/equation_class.cpp:294-308); the legacy build factors an incomplete
 * LDU (M34Vorkond, FEM/matrix_routines.cpp:3271-3427).  Read-back for
 * checks. */
ogs_status ogs_gpu_get_ilu0(const ogs_system* sys, double* lu);

/* y = A x with the current matrix (CSparseMatrix::multiVec,
 * FEM/matrix_class.cpp:1467-1555). */
ogs_status ogs_gpu_spmv(ogs_system* sys, const double* x, double* y);

/* Number of Gauss points per element of the mesh (9/27 at the default
 * $ELE_GAUSS_POINTS 3 for quad/hex, 5 for tets). */
int32_t ogs_gpu_mesh_gauss_points(const ogs_mesh* mesh);

/* Tiles of 8^3 nodes the ILU(0) sweeps walk on this mesh: non-zero when the
 * pattern is a lattice numbered line by line whose columns left of the
 * diagonal lie at no larger x, y, z than their row (Kuhn tets, 7-point
 * stencils); 0 when the sweeps walk dependency levels of rows.
 * (Instrumentation, no counterpart in the reference.) */
int32_t ogs_gpu_mesh_ilu_tiles(const ogs_mesh* mesh);

/* Number of this library's kernels launched on the calling thread since the
 * last reset (instrumentation for benchmarks). */
int64_t ogs_gpu_kernel_launches(int32_t reset);

/* Self-test of the bounded waits of the two cooperative persistent kernels
 * (no counterpart in the reference).  Launches `grid` blocks (0: two per
 * SM, the most allowed) that each pass one grid barrier of the persistent
 * FP32 CG kernel (which = 0) or of the Monte-Carlo batch kernel (which = 1),
 * the wait limited to `spin_limit` polls of the barrier word (0: the
 * kernel's own limit, about a second).  withhold != 0: block 0 leaves
 * without arriving, so the other blocks wait on a word nothing sets until
 * the limit and give up.  *passed: the blocks that passed.  Returns OGS_OK
 * when every arriving block passed, OGS_CUDA_ERROR with "barrier timeout"
 * in ogs_gpu_last_error when a wait gave up (the context stays usable).
 * which = 2: the row waits of the ILU(0) kernels, on a forward sweep over a
 * 64-row lower bidiagonal factor (grid ignored); withhold != 0 leaves row 0
 * unpublished, so every later row's wait runs out; *passed: the rows with
 * their exact value; OGS_CUDA_ERROR with "ILU row wait timeout" when a wait
 * gave up. */
ogs_status ogs_gpu_selftest_barrier(int32_t which, int32_t grid, int32_t spin_limit, int32_t withhold,
                                    int32_t* passed);

/* Bounds checks of the debug build (compiled with -DOGS_BOUNDS_CHECK): the
 * first out-of-range index any kernel met since the previous call (the
 * access was skipped), as its site (1 element-assembly slot, 2 element
 * node, 3 lattice slot, 4 lattice node, 5 FP64 product column, 6 FP32
 * product column, 7 Dirichlet column/row, 8 Dirichlet slot, 9 ILU column,
 * 10 FP32 lattice product window) and index; site 0: none; site -1: a build without the checks.  Waits for
 * the device.  (Instrumentation, no counterpart in the reference.) */
ogs_status ogs_gpu_debug_oob(int64_t* site, int64_t* index);

/* The FP32 product of the Jacobi-scaled operator on x (n host values), by
 * the row kernel (y_rows) and by the four-rows-per-thread lattice kernel
 * (y_lines), n host values each; the two are bit for bit equal.  Needs the
 * FP32 operator of a 27-point (hex) or 9-point (quad) lattice, i.e. a
 * solve with OGS_PRECISION_FP32_REFINED on such a mesh before; OGS_BAD_ARG
 * otherwise.  (Instrumentation, no counterpart in the reference.) */
ogs_status ogs_gpu_debug_fp32_product(ogs_system* sys, const float* x, float* y_rows, float* y_lines);

/* Device time of the SpMV kernel of every Krylov iteration, measured with
 * CUDA events recorded around it inside the captured iteration graphs
 * (instrumentation, no counterpart in the reference). */
typedef struct
{
    double spmv_ms;            /* summed SpMV kernel time                     */
    int64_t spmv_launches;     /* SpMV launches that did work                 */
    double solve_ms;           /* summed device time of the solves            */
    int64_t solves;
    double persist_ms;         /* summed time of the persistent FP32 CG
                                  launches (OGS_SCHEDULE_PERSISTENT)          */
    int64_t persist_iters;     /* FP32 iterations those launches ran          */
} ogs_profile;

/* enable != 0 turns the timing on (graphs are re-captured with the events);
 * out (may be NULL) receives the totals since the previous call, which are
 * then reset. */
ogs_status ogs_gpu_profile(ogs_system* sys, int32_t enable, ogs_profile* out);

/* Jacobi-preconditioned CG that allocates no device memory.  It has no
 * counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc: a process whose HBM is already owned by a caching allocator or
 * memory pool (a solve server, a PyTorch process), where every buffer a
 * solver allocates fails or fragments the pool.  The caller owns every
 * array (device memory): the CSR matrix (row_ptr n+1, col and val
 * row_ptr[n] entries), b (n) and x (n, initial guess in, solution out).  The
 * Krylov vectors, scalars and reduction partials live in a static device
 * array of OGS_NOALLOC_MAX_ROWS rows (16 MiB, held by every GPU that loads
 * the library until exit); larger systems are rejected with OGS_BAD_ARG.
 * The first call on a device looks up the array's address (do it before any
 * stream capture); cudaDeviceReset after it is not supported.  The call
 * reads the solver state back and synchronises its stream every 16
 * iterations.  All calls share the array: calls whose work overlaps on the
 * GPU race and must be serialised by the caller.  Iteration and stopping
 * rule are those of Linear_EQS::CG for a fresh system (tol relative to |b|,
 * at most max_iter iterations).  stream: a cudaStream_t or NULL. */
#define OGS_NOALLOC_MAX_ROWS 524288
ogs_status ogs_gpu_csr_cg_noalloc(int64_t n, const int32_t* row_ptr,
                                  const int32_t* col, const double* val,
                                  const double* b, double* x,
                                  int32_t max_iter, double tol, void* stream,
                                  ogs_solve_stats* stats);

/* ------------------------------------------------------------------------
 * Monte-Carlo batch (extension; no single counterpart in the reference,
 * which runs one realisation per ogs process: CRFProcess::GlobalAssembly,
 * IncorporateBoundaryConditions and Linear_EQS::Solver once per deck).
 *
 * Many steady GROUNDWATER_FLOW realisations on structured hex boxes of
 * different sizes, each with its own element conductivity field, Dirichlet
 * heads on the two x faces (symmetric elimination, as
 * OGS_DIRICHLET_SYMMETRIC) and no-flow elsewhere, are assembled and solved
 * by ONE cooperative persistent kernel launch (captured in a CUDA graph):
 * row-centric assembly straight into the upper diagonal-offset form (no
 * slot map, no atomics), then Jacobi-preconditioned CG with FP32 matrix
 * and sweeps and FP64 residual replacement (as OGS_PRECISION_FP32_REFINED)
 * for all realisations at once; converged realisations drop out of the
 * work list.  Node (ix, iy, iz) of a box has index ix + nx (iy + ny iz);
 * element (ex, ey, ez) has index ex + (nx-1) (ey + (ny-1) ez).
 * ---------------------------------------------------------------------- */
typedef struct ogs_batch ogs_batch;

typedef struct
{
    int32_t nx, ny, nz;         /* nodes per axis (>= 2 each)                  */
    int32_t pad0;
    const double* elem_k;       /* (nx-1)(ny-1)(nz-1) conductivities, host    */
    double h_left, h_right;     /* heads on the x = 0 and x = max faces       */
} ogs_batch_realisation;

typedef struct
{
    double hx, hy, hz;          /* cell sizes, all realisations                */
    double time_unit_factor;    /* CalCoefLaplace factor (1 for seconds)       */
    double tol;                 /* |b - A x| / |b| < tol                       */
    double inner_tol;           /* FP32 residual drop per replacement (0: 1e-2) */
    int32_t max_iter;           /* FP32 iterations per realisation             */
    int32_t pad0;
} ogs_batch_config;

/* Launch shape of the persistent kernel (chosen by ogs_gpu_batch_autotune
 * or set by the caller): rows per work tile, threads per block, resident
 * blocks per SM (the grid is blocks_per_sm x SM count). */
typedef struct
{
    int32_t tile_rows;
    int32_t block_threads;      /* 256 or 512                                  */
    int32_t blocks_per_sm;
    int32_t graph;              /* out: 1 if the launch runs as a CUDA graph   */
    double ms_per_step;         /* out (autotune): measured time per CG step   */
} ogs_batch_tuning;

typedef struct
{
    int32_t iterations;         /* FP32 inner iterations                       */
    int32_t status;             /* ogs_status                                  */
    int32_t refinements;        /* FP64 residual replacements                  */
    int32_t pad0;
    double rel_residual;        /* final FP64 |b - A x| / |b|                  */
    double finish_ms;           /* device time from the start of the launch to
                                   this realisation's convergence              */
} ogs_batch_stats;

/* Copies the realisations' fields to the device and lays out the batch. */
ogs_status ogs_gpu_batch_create(const ogs_batch_config* cfg,
                                const ogs_batch_realisation* reals,
                                int32_t n_real, void* stream, ogs_batch** out);
ogs_status ogs_gpu_batch_destroy(ogs_batch* b);
/* Replaces the conductivity field of every realisation (host or device
 * array of all elements, realisations in order). */
ogs_status ogs_gpu_batch_set_k(ogs_batch* b, const double* elem_k_all);
/* Times every candidate launch shape on this batch (a bounded number of CG
 * steps each) and keeps the fastest; *chosen receives it (may be NULL). */
ogs_status ogs_gpu_batch_autotune(ogs_batch* b, ogs_batch_tuning* chosen);
ogs_status ogs_gpu_batch_set_tuning(ogs_batch* b, const ogs_batch_tuning* t);
/* Assembly and solve of every realisation in one launch.  stats: n_real
 * entries (may be NULL).  Returns OGS_OK when every realisation converged,
 * else the first failing status. */
ogs_status ogs_gpu_batch_solve(ogs_batch* b, ogs_batch_stats* stats);
/* Heads of all realisations, concatenated (host or device array). */
ogs_status ogs_gpu_batch_get_heads(const ogs_batch* b, double* heads);
/* Total rows (sum of nx ny nz) and elements of the batch. */
ogs_status ogs_gpu_batch_info(const ogs_batch* b, int64_t* rows, int64_t* elements);

/* ------------------------------------------------------------------------
 * Request server with continuous batching (serving extension; no
 * counterpart in the reference).  Requests of registered classes (mesh,
 * kind, Dirichlet set, solver configuration) arrive at any time with their
 * own conductivity field and tolerance; admitted requests run concurrently,
 * one CUDA stream and one device-resident equation system ("slot") each,
 * and join or leave between chunks of Krylov iterations.  Slots are reused
 * per class and created while their device bytes fit the HBM budget.  Each
 * request is a fresh Linear_EQS (CheckNormRHS against bNorm = 1.0).
 * ---------------------------------------------------------------------- */
typedef struct ogs_server ogs_server;

enum
{
    OGS_REQUEST_FLOW = 0,      /* steady or transient flow solve              */
    OGS_REQUEST_TRANSPORT = 1  /* MASS_TRANSPORT step; the Darcy flux comes from
                                  the class's head field and the request's K */
};

typedef struct
{
    ogs_mesh* mesh;             /* kept alive by the caller                    */
    int32_t kind;               /* OGS_REQUEST_*                               */
    int32_t bc_mode;            /* ogs_dirichlet_mode                          */
    ogs_assembly_params params; /* assembly of the solved equation             */
    ogs_assembly_params flow_params; /* transport: flux parameters (flow)     */
    int64_t n_elements;         /* transport: elements of the mesh             */
    const double* flow_head;    /* transport: head field (n_nodes), copied     */
    const int64_t* bc_rows;     /* Dirichlet rows and values (host), copied    */
    const double* bc_values;
    int64_t n_bc;
    ogs_solver_config solver;   /* tol is replaced by each request's tol (a
                                   tenth of it in FP32-inner mode: two solves
                                   stopped at |r|/|b| < tol differ by up to
                                   cond(A) tol, the tighter stop keeps served
                                   heads within the FP64 path's accuracy)    */
} ogs_server_class;

typedef struct
{
    int32_t state;              /* 0 queued, 1 running, 2 done                 */
    int32_t status;             /* ogs_status (state 2)                        */
    int32_t iterations;
    int32_t refinements;
    double rel_residual;
    double latency_ms;          /* submit -> completion seen by the server     */
    double queue_ms;            /* submit -> admission                         */
    double solve_ms;            /* device time of the solve                    */
    int32_t batch_size;         /* requests of the batch launch that served it
                                   (0: served alone on a slot)                 */
    int32_t precision;          /* OGS_PRECISION_* the request was solved in   */
    int32_t fp64_fallback;      /* FP32-inner solve finished in FP64 CG        */
    int32_t pad0;
} ogs_server_result;

typedef struct
{
    int32_t slots, running, queued;
    int32_t fp64_classes;       /* FP32 classes served in FP64 after a fallback
                                   (OGS_SERVER_PRECISION_FALLBACK)             */
    int64_t completed;
    int64_t bytes_used, bytes_budget;
    int64_t batched;            /* requests served by batch launches           */
} ogs_server_info;

/* Scheduling policy bits of ogs_gpu_server_create. */
enum
{
    OGS_SERVER_PRIORITY = 1,  /* smaller classes get higher CUDA stream priorities */
    OGS_SERVER_SJF = 2,       /* admit the queued request of the smallest class
                                 first (arrival order among equals); default:
                                 arrival order                                 */
    OGS_SERVER_PRECISION_FALLBACK = 8, /* a class whose FP32-inner solve finished
                                 in FP64 CG (the FP32 cycles stopped gaining,
                                 ogs_solve_stats.fp64_fallback) is served in
                                 FP64 from its next request on              */
    OGS_SERVER_BATCH = 4      /* dynamic batching: two or more queued requests
                                 of one steady hex-lattice flow class (heads on
                                 the two x faces, FP32-inner CG) with the same
                                 tolerance are solved together by one
                                 Monte-Carlo batch launch (ogs_gpu_batch_*),
                                 which progress runs to completion           */
};

/* hbm_budget_bytes <= 0: 80% of the free device memory at creation.
 * max_active: requests in flight at most.  flags: OGS_SERVER_* bits. */
ogs_status ogs_gpu_server_create(int64_t hbm_budget_bytes, int32_t max_active, int32_t flags,
                                 ogs_server** out);
ogs_status ogs_gpu_server_destroy(ogs_server* srv);
ogs_status ogs_gpu_server_add_class(ogs_server* srv, const ogs_server_class* cls, int32_t* class_id);
/* Creates idle slots of a class up to n_slots in total (within the budget),
 * so that the first requests do not pay for allocation and graph capture. */
ogs_status ogs_gpu_server_reserve(ogs_server* srv, int32_t class_id, int32_t n_slots);
/* Queues a request.  elem_k: device array (n_elements), complete when this
 * is called (the server's streams do not wait on the caller's), that stays
 * valid until the request is done; out: n_nodes doubles (device or pinned
 * host), written when the request is done. */
ogs_status ogs_gpu_server_submit(ogs_server* srv, int32_t class_id, const double* elem_k, double tol,
                                 double* out, int64_t* request_id);
/* One scheduling round: polls running requests, retires finished ones,
 * admits queued ones.  Blocks on the GPU only for a batch launch
 * (OGS_SERVER_BATCH). */
ogs_status ogs_gpu_server_progress(ogs_server* srv, int32_t* n_running, int32_t* n_queued);
ogs_status ogs_gpu_server_result(const ogs_server* srv, int64_t request_id, ogs_server_result* r);
ogs_status ogs_gpu_server_info(const ogs_server* srv, ogs_server_info* info);

/* ---- Input decks (host only, no GPU call) --------------------------------
 * Reads an OGS-5 deck's mesh (.msh), geometry (.gli) and boundary
 * conditions (.bc) and yields what the GPU path consumes: the mesh
 * description for ogs_gpu_mesh_create and the Dirichlet rows and values for
 * ogs_gpu_set_dirichlet.  Replaces, for quad/hex/tet meshes and CONSTANT
 * conditions on points, polylines and planar surfaces:
 *   CFEMesh::Read (MSH/msh_mesh.cpp:421-495), CElem::Read
 *   (MSH/msh_elem.cpp:578-736);
 *   GEOLIB's readGLIFileV4 points/polylines/surfaces
 *   (FileIO/OGSIOVer4.cpp:54-503);
 *   BCRead / CBoundaryCondition::Read (FEM/rf_bc_new.cpp:250-560) and the
 *   node search of CBoundaryConditionsGroup::Set
 *   (FEM/rf_bc_new.cpp:1272-1560): GetNODOnPNT, GetNODOnPLY, GetNODOnSFC
 *   (MSH/msh_mesh.cpp:1434, 1562, 1779). */
typedef struct ogs_deck ogs_deck;

/* gli_path and bc_path may be NULL.  Errors (unreadable file, element type
 * off the GPU path, mixed element types, unsupported $DIS_TYPE or geometry)
 * return OGS_BAD_ARG with the reason in ogs_gpu_last_error. */
ogs_status ogs_deck_read(const char* msh_path, const char* gli_path, const char* bc_path,
                         ogs_deck** out);
ogs_status ogs_deck_destroy(ogs_deck* deck);
/* The mesh; the arrays stay owned by the deck.  min_edge_length (may be
 * NULL): CFEMesh::getMinEdgeLength. */
ogs_status ogs_deck_mesh(const ogs_deck* deck, ogs_mesh_desc* desc, double* min_edge_length);
/* Mesh nodes of one geometry ("POINT" | "POLYLINE" | "SURFACE", name) as a
 * CONSTANT condition without $EPSILON selects them.  rows NULL: *n gets the
 * count only; otherwise capacity >= *n. */
ogs_status ogs_deck_geo_nodes(const ogs_deck* deck, const char* geo_type, const char* name,
                              int64_t* rows, int64_t capacity, int64_t* n);
/* Dirichlet rows and values of every condition whose $PCS_TYPE equals
 * pcs_type (and $PRIMARY_VARIABLE / $COMP_NAME primary_variable unless
 * NULL), in the order CRFProcess::bc_node_value holds them: file order, and
 * within a condition the node order of its search.  rows NULL: count only. */
ogs_status ogs_deck_dirichlet(const ogs_deck* deck, const char* pcs_type, const char* primary_variable,
                              int64_t* rows, double* values, int64_t capacity, int64_t* n);

#ifdef __cplusplus
}
#endif

#endif /* OGS_GPU_H */
