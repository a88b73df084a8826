// api.cu -- the extern "C" surface of include/ogs_gpu.h: equation systems,
// assembly dispatch, Dirichlet conditions, solve orchestration, read-back.
#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <cstring>
#include <vector>

#include "krylov.cuh"

namespace ogs {

bool launch_assembly(const ogs_mesh* m, const AsmArgs& a, bool affine, int kind, cudaStream_t s);
void launch_spmv(const CsrView<double>& A, const double* x, double* y, int G, cudaStream_t s);
void launch_dinv(const double* val, const int32_t* diag_pos, double* dinv, int n, cudaStream_t s);
void launch_krylov_init(const SolveArgs& a, int kind, int G, cudaStream_t s);
void launch_krylov_iteration(const SolveArgs& a, int kind, int G, cudaStream_t s);
void launch_bicgstab_finish(const SolveArgs& a, cudaStream_t s);
int kernels_per_iteration(int kind);
int row_group(double avg_nnz);
int vec_grid(int n);

// ------------------------------------------------------------------
// small kernels
// ------------------------------------------------------------------
__global__ void k_dirichlet_row_only(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                     const int32_t* __restrict__ diag_pos, double* val, double* b,
                                     const int32_t* __restrict__ rows, const double* __restrict__ vals,
                                     int nbc)
{
    // CSparseMatrix::Diagonize, CRS, column kept (matrix_class.cpp:1663-1700,1783)
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nbc; q += gridDim.x * blockDim.x)
    {
        const int id = rows[q];
        const int dp = diag_pos[id];
        const double vdiag = dp >= 0 ? val[dp] : 0.0;
        for (int k = rp[id]; k < rp[id + 1]; k++)
            if (col[k] != id) val[k] = 0.0;
        b[id] = vdiag * vals[q];
    }
}

__global__ void k_dirichlet_symmetric(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                      const int32_t* __restrict__ diag_pos, double* val, double* b,
                                      const unsigned char* __restrict__ flag,
                                      const double* __restrict__ valn, int n)
{
    // MXRandbed (matrix_routines.cpp:2314-2520): lift column into b, zero
    // row and column, keep the diagonal (a zero diagonal -> DBL_EPSILON)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        if (flag[i])
        {
            const int dp = diag_pos[i];
            double d = dp >= 0 ? val[dp] : 0.0;
            if (fabs(d) < DBL_MIN) d = DBL_EPSILON;
            for (int k = rp[i]; k < rp[i + 1]; k++) val[k] = 0.0;
            if (dp >= 0) val[dp] = d;
            b[i] = valn[i] * d;
        }
        else
        {
            double bi = b[i];
            for (int k = rp[i]; k < rp[i + 1]; k++)
            {
                const int c = col[k];
                if (flag[c])
                {
                    bi -= val[k] * valn[c];
                    val[k] = 0.0;
                }
            }
            b[i] = bi;
        }
    }
}

__global__ void k_scatter_rows(double* x, const int32_t* __restrict__ rows, const double* __restrict__ vals,
                               int nbc)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nbc; q += gridDim.x * blockDim.x)
        x[rows[q]] = vals[q];
}

__global__ void k_mark_rows(unsigned char* flag, double* valn, const int32_t* __restrict__ rows,
                            const double* __restrict__ vals, int nbc)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nbc; q += gridDim.x * blockDim.x)
    {
        flag[rows[q]] = 1;
        valn[rows[q]] = vals[q];
    }
}

__global__ void k_i32_to_i64(const int32_t* __restrict__ a, int64_t* __restrict__ b, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

static bool is_device_ptr(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace ogs

using namespace ogs;

struct ogs_system
{
    ogs_mesh* m = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int n = 0;
    double *val = nullptr, *b = nullptr, *x = nullptr;
    double *r = nullptr, *r0 = nullptr, *p = nullptr, *ph = nullptr, *s = nullptr, *sh = nullptr,
           *t = nullptr, *v = nullptr, *dinv = nullptr;
    double *ek = nullptr, *u0 = nullptr, *gpv = nullptr, *qbuf = nullptr, *vec_in = nullptr,
           *vec_out = nullptr;
    KState* st = nullptr;
    KState* h_st = nullptr;   // pinned header copy
    int* d_bad = nullptr;
    int* h_bad = nullptr;     // pinned
    ogs_solver_config cfg{};
    bool configured = false;
    double bnorm_prev = 1.0;  // Linear_EQS ctor: bNorm = 1.0
    // Dirichlet
    int nbc = 0;
    int32_t* bc_rows = nullptr;
    double* bc_vals = nullptr;
    int bc_cap = 0;
    unsigned char* bc_flag = nullptr;
    double* bc_valn = nullptr;
    // iteration chunks captured as graphs, per solver kind
    cudaGraphExec_t chunk[2] = {nullptr, nullptr};
    int chunk_iters[2] = {0, 0};
    int G = 1;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

constexpr size_t kStateHeader = offsetof(KState, ticket);

ogs_status stage_in(ogs_system* s, const double* src, size_t n, double** scratch, const double** out)
{
    if (!src) { *out = nullptr; return OGS_OK; }
    if (is_device_ptr(src)) { *out = src; return OGS_OK; }
    if (!*scratch) OGS_CUDA_TRY(cudaMalloc(scratch, std::max<size_t>(1, n) * sizeof(double)));
    OGS_CUDA_TRY(cudaMemcpyAsync(*scratch, src, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    *out = *scratch;
    return OGS_OK;
}

SolveArgs make_solve_args(ogs_system* s)
{
    SolveArgs a;
    a.A.row_ptr = s->m->row_ptr;
    a.A.col = s->m->col;
    a.A.val = s->val;
    a.A.n = s->n;
    std::memset(&a.v, 0, sizeof a.v);
    a.v.x = s->x; a.v.b = s->b; a.v.r = s->r; a.v.r0 = s->r0; a.v.p = s->p; a.v.ph = s->ph;
    a.v.s = s->s; a.v.sh = s->sh; a.v.t = s->t; a.v.v = s->v; a.v.dinv = s->dinv;
    a.st = s->st;
    a.precond = s->cfg.precond == OGS_PRECOND_JACOBI ? OGS_PRECOND_JACOBI : 0;
    return a;
}

void drop_graphs(ogs_system* s)
{
    for (int k = 0; k < 2; k++)
        if (s->chunk[k]) { cudaGraphExecDestroy(s->chunk[k]); s->chunk[k] = nullptr; }
}

ogs_status get_chunk(ogs_system* s, int kind, const SolveArgs& a, cudaGraphExec_t* out, int* iters)
{
    if (!s->chunk[kind])
    {
        const int C = kind == SK_CG ? 16 : 8;
        cudaGraph_t g;
        OGS_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < C; i++) launch_krylov_iteration(a, kind, s->G, s->stream);
        cudaError_t e = cudaStreamEndCapture(s->stream, &g);
        if (e != cudaSuccess) { set_error("graph capture: %s", cudaGetErrorString(e)); return OGS_CUDA_ERROR; }
        e = cudaGraphInstantiate(&s->chunk[kind], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { set_error("graph instantiate: %s", cudaGetErrorString(e)); return OGS_CUDA_ERROR; }
        s->chunk_iters[kind] = C;
    }
    *out = s->chunk[kind];
    *iters = s->chunk_iters[kind];
    return OGS_OK;
}

}  // namespace

extern "C" ogs_status ogs_gpu_system_destroy(ogs_system* s)
{
    if (!s) return OGS_OK;
    drop_graphs(s);
    double* bufs[] = {s->val, s->b, s->x, s->r, s->r0, s->p, s->ph, s->s, s->sh, s->t, s->v, s->dinv,
                      s->ek, s->u0, s->gpv, s->qbuf, s->vec_in, s->vec_out, s->bc_vals, s->bc_valn};
    for (double* p : bufs) cudaFree(p);
    cudaFree(s->st);
    cudaFree(s->d_bad);
    cudaFree(s->bc_rows);
    cudaFree(s->bc_flag);
    if (s->h_st) cudaFreeHost(s->h_st);
    if (s->h_bad) cudaFreeHost(s->h_bad);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_system_create(ogs_mesh* m, void* stream, ogs_system** out)
{
    if (!m || !out) { set_error("system_create: NULL argument"); return OGS_BAD_ARG; }
    *out = nullptr;
    ogs_system* s = new ogs_system;
    s->m = m;
    s->n = (int)m->n_nodes;
    if (stream)
        s->stream = (cudaStream_t)stream;
    else
    {
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        {
            delete s;
            set_error("system_create: stream creation failed");
            return OGS_CUDA_ERROR;
        }
        s->own_stream = true;
    }
    const size_t nb = (size_t)s->n * sizeof(double);
    double** vecs[] = {&s->b, &s->x, &s->r, &s->r0, &s->p, &s->ph, &s->s, &s->sh, &s->t, &s->v, &s->dinv};
    cudaError_t e = cudaMalloc(&s->val, std::max<int64_t>(1, m->nnz) * sizeof(double));
    for (double** p : vecs)
        if (e == cudaSuccess) e = cudaMalloc(p, nb);
    if (e == cudaSuccess) e = cudaMalloc(&s->st, sizeof(KState));
    if (e == cudaSuccess) e = cudaMemset(s->st, 0, sizeof(KState));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_bad, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_st, sizeof(KState));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_bad, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->bc_flag, std::max(1, s->n));
    if (e == cudaSuccess) e = cudaMalloc(&s->bc_valn, nb);
    if (e == cudaSuccess) e = cudaMemset(s->val, 0, m->nnz * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(s->b, 0, nb);
    if (e == cudaSuccess) e = cudaMemset(s->x, 0, nb);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e != cudaSuccess)
    {
        set_error("system_create: %s", cudaGetErrorString(e));
        ogs_gpu_system_destroy(s);
        return e == cudaErrorMemoryAllocation ? OGS_OOM : OGS_CUDA_ERROR;
    }
    s->G = row_group((double)m->nnz / std::max<int64_t>(1, m->n_nodes));
    // CNumerics defaults (rf_num_new.cpp:77-165): BiCGStab, Jacobi, 1000, 1e-12
    s->cfg.method = OGS_LS_BICGSTAB;
    s->cfg.precond = OGS_PRECOND_JACOBI;
    s->cfg.max_iter = 1000;
    s->cfg.tol = 1e-12;
    s->cfg.check_norm_rhs = 1;
    s->configured = true;
    *out = s;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_configure(ogs_system* s, const ogs_solver_config* c)
{
    if (!s || !c) { set_error("configure: NULL argument"); return OGS_BAD_ARG; }
    if (c->method != OGS_LS_CG && c->method != OGS_LS_BICGSTAB)
    {
        set_error("configure: ls_method %d not supported (2 BiCGStab, 5 CG)", c->method);
        return OGS_BAD_ARG;
    }
    if (c->precond != OGS_PRECOND_NONE && c->precond != OGS_PRECOND_JACOBI && c->precond != OGS_PRECOND_ILU0)
    {
        set_error("configure: ls_precond %d not supported (0, 1, 100)", c->precond);
        return OGS_BAD_ARG;
    }
    if (c->max_iter < 0 || !(c->tol >= 0.0)) { set_error("configure: bad max_iter/tol"); return OGS_BAD_ARG; }
    if (c->precision != OGS_PRECISION_FP64 && c->precision != OGS_PRECISION_FP32_REFINED)
    {
        set_error("configure: unknown precision %d", c->precision);
        return OGS_BAD_ARG;
    }
    s->cfg = *c;
    drop_graphs(s);
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_initialize(ogs_system* s)
{
    if (!s) { set_error("initialize: NULL system"); return OGS_BAD_ARG; }
    OGS_CUDA_TRY(cudaMemsetAsync(s->val, 0, s->m->nnz * sizeof(double), s->stream));
    OGS_CUDA_TRY(cudaMemsetAsync(s->b, 0, (size_t)s->n * sizeof(double), s->stream));
    return OGS_OK;
}

static ogs_status check_params(const ogs_assembly_params* p)
{
    if (!p) { set_error("assemble: NULL params"); return OGS_BAD_ARG; }
    if (p->pcs_type < 0 || p->pcs_type > 2) { set_error("assemble: bad pcs_type %d", p->pcs_type); return OGS_BAD_ARG; }
    if (!(p->dt > 0.0)) { set_error("assemble: dt must be > 0"); return OGS_BAD_ARG; }
    if (!(p->time_unit_factor != 0.0)) { set_error("assemble: time_unit_factor must be non-zero"); return OGS_BAD_ARG; }
    return OGS_OK;
}

static ogs_status run_element_kernel(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                     const double* u0, const double* gpv, int kind, double* q_out)
{
    ogs_mesh* m = s->m;
    AsmArgs a;
    std::memset(&a, 0, sizeof a);
    a.E = m->n_elem;
    a.x = m->x; a.y = m->y; a.z = m->z;
    a.conn_t = m->conn_t;
    a.slot_t = m->slot_t;
    a.tab = m->tab;
    a.aff = m->aff;
    a.val = s->val;
    a.b = s->b;
    a.q_out = q_out;
    a.bad_elem = s->d_bad;
    a.p = *p;
    ogs_status st;
    if ((st = stage_in(s, elem_k, m->n_elem, &s->ek, &a.elem_k))) return st;
    if ((st = stage_in(s, u0, m->n_nodes, &s->u0, &a.u0))) return st;
    if ((st = stage_in(s, gpv, (size_t)m->n_elem * m->ngp * 3, &s->gpv, &a.gpv))) return st;
    const int big = 0x7fffffff;
    OGS_CUDA_TRY(cudaMemcpyAsync(s->d_bad, &big, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    if (!launch_assembly(m, a, m->affine, kind, s->stream))
    {
        set_error("no kernel for element type %d with %d Gauss points", m->elem_type, m->ngp);
        return OGS_BAD_ARG;
    }
    OGS_LAUNCH_CHECK();
    OGS_CUDA_TRY(cudaMemcpyAsync(s->h_bad, s->d_bad, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (*s->h_bad != big)
    {
        set_error("singular Jacobian (|det J| < DBL_EPSILON) in element %d", *s->h_bad - 1);
        return OGS_SINGULAR_JACOBIAN;
    }
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_assemble(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                       const double* u0, const double* gp_velocity)
{
    if (!s) { set_error("assemble: NULL system"); return OGS_BAD_ARG; }
    ogs_status st = check_params(p);
    if (st) return st;
    if (p->pcs_type != OGS_PCS_MASS_TRANSPORT && !elem_k) { set_error("assemble: flow needs elem_k"); return OGS_BAD_ARG; }
    if (p->pcs_type == OGS_PCS_MASS_TRANSPORT && !gp_velocity) { set_error("assemble: transport needs gp_velocity"); return OGS_BAD_ARG; }
    return run_element_kernel(s, p, elem_k, u0, gp_velocity, p->pcs_type == OGS_PCS_MASS_TRANSPORT ? 1 : 0, nullptr);
}

extern "C" ogs_status ogs_gpu_gp_velocity(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                          const double* u, double* q_gp)
{
    if (!s || !elem_k || !u || !q_gp) { set_error("gp_velocity: NULL argument"); return OGS_BAD_ARG; }
    if (!p || p->pcs_type == OGS_PCS_MASS_TRANSPORT || !(p->time_unit_factor != 0.0))
    {
        set_error("gp_velocity: needs flow parameters");
        return OGS_BAD_ARG;
    }
    const size_t nq = (size_t)s->m->n_elem * s->m->ngp * 3;
    double* dst = q_gp;
    const bool dev = is_device_ptr(q_gp);
    if (!dev)
    {
        if (!s->qbuf) OGS_CUDA_TRY(cudaMalloc(&s->qbuf, nq * sizeof(double)));
        dst = s->qbuf;
    }
    ogs_status st = run_element_kernel(s, p, elem_k, u, nullptr, 2, dst);
    if (st) return st;
    if (!dev)
    {
        OGS_CUDA_TRY(cudaMemcpyAsync(q_gp, dst, nq * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    }
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_set_dirichlet(ogs_system* s, const int64_t* rows, const double* values,
                                            int64_t n_rows, int32_t mode)
{
    if (!s || (n_rows > 0 && (!rows || !values)) || n_rows < 0) { set_error("set_dirichlet: bad arguments"); return OGS_BAD_ARG; }
    if (mode != OGS_DIRICHLET_ROW_ONLY && mode != OGS_DIRICHLET_SYMMETRIC) { set_error("set_dirichlet: bad mode %d", mode); return OGS_BAD_ARG; }
    if (n_rows > s->n) { set_error("set_dirichlet: more rows than unknowns"); return OGS_BAD_ARG; }
    std::vector<int32_t> r32(n_rows);
    std::vector<double> vh(n_rows);
    const bool rdev = is_device_ptr(rows), vdev = is_device_ptr(values);
    std::vector<int64_t> rh;
    const int64_t* rsrc = rows;
    if (rdev && n_rows)
    {
        rh.resize(n_rows);
        OGS_CUDA_TRY(cudaMemcpy(rh.data(), rows, n_rows * sizeof(int64_t), cudaMemcpyDeviceToHost));
        rsrc = rh.data();
    }
    for (int64_t q = 0; q < n_rows; q++)
    {
        if (rsrc[q] < 0 || rsrc[q] >= s->n) { set_error("set_dirichlet: row %lld out of range", (long long)rsrc[q]); return OGS_BAD_ARG; }
        r32[q] = (int32_t)rsrc[q];
    }
    if (n_rows > s->bc_cap)
    {
        cudaFree(s->bc_rows);
        cudaFree(s->bc_vals);
        s->bc_rows = nullptr;
        s->bc_vals = nullptr;
        OGS_CUDA_TRY(cudaMalloc(&s->bc_rows, n_rows * sizeof(int32_t)));
        OGS_CUDA_TRY(cudaMalloc(&s->bc_vals, n_rows * sizeof(double)));
        s->bc_cap = (int)n_rows;
    }
    s->nbc = (int)n_rows;
    if (!n_rows) return OGS_OK;
    OGS_CUDA_TRY(cudaMemcpyAsync(s->bc_rows, r32.data(), n_rows * sizeof(int32_t), cudaMemcpyHostToDevice, s->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(s->bc_vals, values, n_rows * sizeof(double),
                                 vdev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s->stream));
    ogs_mesh* m = s->m;
    const int g = std::max(1, std::min(1024, (int)((n_rows + 255) / 256)));
    if (mode == OGS_DIRICHLET_ROW_ONLY)
    {
        k_dirichlet_row_only<<<g, 256, 0, s->stream>>>(m->row_ptr, m->col, m->diag_pos, s->val, s->b,
                                                       s->bc_rows, s->bc_vals, s->nbc);
        OGS_LAUNCH_CHECK();
    }
    else
    {
        OGS_CUDA_TRY(cudaMemsetAsync(s->bc_flag, 0, s->n, s->stream));
        k_mark_rows<<<g, 256, 0, s->stream>>>(s->bc_flag, s->bc_valn, s->bc_rows, s->bc_vals, s->nbc);
        OGS_LAUNCH_CHECK();
        k_dirichlet_symmetric<<<vec_grid(s->n), 256, 0, s->stream>>>(m->row_ptr, m->col, m->diag_pos, s->val,
                                                                      s->b, s->bc_flag, s->bc_valn, s->n);
        OGS_LAUNCH_CHECK();
    }
    // values must stay valid until the copies above ran
    if (!vdev) OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_solve(ogs_system* s, double* x_inout, ogs_solve_stats* stats)
{
    if (!s || !x_inout) { set_error("solve: NULL argument"); return OGS_BAD_ARG; }
    const ogs_solver_config& c = s->cfg;
    if (c.precond == OGS_PRECOND_ILU0 || c.precision != OGS_PRECISION_FP64)
    {
        set_error("solve: ILU(0) / FP32 refinement not available in this build");
        return OGS_BAD_ARG;
    }
    const int kind = c.method == OGS_LS_CG ? SK_CG : SK_BICGSTAB;
    const size_t nb = (size_t)s->n * sizeof(double);
    const bool xdev = is_device_ptr(x_inout);
    OGS_CUDA_TRY(cudaEventRecord(s->ev0, s->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(s->x, x_inout, nb, xdev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 s->stream));
    if (s->nbc)
    {
        k_scatter_rows<<<std::max(1, std::min(1024, (s->nbc + 255) / 256)), 256, 0, s->stream>>>(s->x, s->bc_rows,
                                                                                               s->bc_vals, s->nbc);
        OGS_LAUNCH_CHECK();
    }
    SolveArgs a = make_solve_args(s);
    if (a.precond == OGS_PRECOND_JACOBI)
    {
        launch_dinv(s->val, s->m->diag_pos, s->dinv, s->n, s->stream);
        OGS_LAUNCH_CHECK();
    }
    KState* h = s->h_st;
    std::memset(h, 0, kStateHeader);
    h->bnorm = c.check_norm_rhs ? s->bnorm_prev : -1.0;
    h->tol = c.tol;
    h->error = 1.0e10;
    h->max_iter = c.max_iter;
    h->alpha = h->omega = h->rho0 = 1.0;
    OGS_CUDA_TRY(cudaMemcpyAsync(s->st, h, kStateHeader, cudaMemcpyHostToDevice, s->stream));
    launch_krylov_init(a, kind, s->G, s->stream);
    OGS_LAUNCH_CHECK();
    cudaGraphExec_t ge;
    int per = 0;
    ogs_status st = get_chunk(s, kind, a, &ge, &per);
    if (st) return st;
    int launched = 0;
    for (;;)
    {
        OGS_CUDA_TRY(cudaMemcpyAsync(h, s->st, kStateHeader, cudaMemcpyDeviceToHost, s->stream));
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        if (h->done || launched > c.max_iter + per) break;
        OGS_CUDA_TRY(cudaGraphLaunch(ge, s->stream));
        count_launches((int64_t)per * kernels_per_iteration(kind));
        launched += per;
    }
    if (!h->done)
    {
        set_error("solve: solver state did not finish");
        return OGS_CUDA_ERROR;
    }
    if (h->finish_s)
    {
        launch_bicgstab_finish(a, s->stream);
        OGS_LAUNCH_CHECK();
    }
    OGS_CUDA_TRY(cudaMemcpyAsync(x_inout, s->x, nb, xdev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                 s->stream));
    OGS_CUDA_TRY(cudaEventRecord(s->ev1, s->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->bnorm_prev = h->bnorm;
    if (stats)
    {
        std::memset(stats, 0, sizeof *stats);
        stats->iterations = h->iter;
        stats->status = h->status;
        stats->rel_residual = h->error;
        stats->b_norm = h->bnorm;
        stats->solve_ms = ms;
    }
    return h->status == OGS_OK ? OGS_OK : (ogs_status)h->status;
}

extern "C" ogs_status ogs_gpu_spmv(ogs_system* s, const double* x, double* y)
{
    if (!s || !x || !y) { set_error("spmv: NULL argument"); return OGS_BAD_ARG; }
    const size_t nb = (size_t)s->n * sizeof(double);
    const double* xd = x;
    if (!is_device_ptr(x))
    {
        if (!s->vec_in) OGS_CUDA_TRY(cudaMalloc(&s->vec_in, nb));
        OGS_CUDA_TRY(cudaMemcpyAsync(s->vec_in, x, nb, cudaMemcpyHostToDevice, s->stream));
        xd = s->vec_in;
    }
    const bool ydev = is_device_ptr(y);
    double* yd = y;
    if (!ydev)
    {
        if (!s->vec_out) OGS_CUDA_TRY(cudaMalloc(&s->vec_out, nb));
        yd = s->vec_out;
    }
    CsrView<double> A{s->m->row_ptr, s->m->col, s->val, s->n};
    launch_spmv(A, xd, yd, s->G, s->stream);
    OGS_LAUNCH_CHECK();
    if (!ydev) OGS_CUDA_TRY(cudaMemcpyAsync(y, yd, nb, cudaMemcpyDeviceToHost, s->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_get_csr(const ogs_system* s, int64_t* row_ptr, int64_t* col, double* val)
{
    if (!s) { set_error("get_csr: NULL system"); return OGS_BAD_ARG; }
    const ogs_mesh* m = s->m;
    if (row_ptr || col)
    {
        std::vector<int32_t> rp(m->n_nodes + 1), cl(m->nnz);
        OGS_CUDA_TRY(cudaMemcpy(rp.data(), m->row_ptr, rp.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
        OGS_CUDA_TRY(cudaMemcpy(cl.data(), m->col, cl.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
        if (row_ptr) for (size_t i = 0; i < rp.size(); i++) row_ptr[i] = rp[i];
        if (col) for (size_t i = 0; i < cl.size(); i++) col[i] = cl[i];
    }
    if (val)
    {
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        OGS_CUDA_TRY(cudaMemcpy(val, s->val, m->nnz * sizeof(double),
                                is_device_ptr(val) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
    }
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_get_rhs(const ogs_system* s, double* b)
{
    if (!s || !b) { set_error("get_rhs: NULL argument"); return OGS_BAD_ARG; }
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    OGS_CUDA_TRY(cudaMemcpy(b, s->b, (size_t)s->n * sizeof(double),
                            is_device_ptr(b) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_get_x(const ogs_system* s, double* x)
{
    if (!s || !x) { set_error("get_x: NULL argument"); return OGS_BAD_ARG; }
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    OGS_CUDA_TRY(cudaMemcpy(x, s->x, (size_t)s->n * sizeof(double),
                            is_device_ptr(x) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
    return OGS_OK;
}
