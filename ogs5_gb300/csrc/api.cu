// api.cu -- the extern "C" surface of include/ogs_gpu.h: equation systems,
// assembly dispatch, Dirichlet conditions, solve orchestration, read-back.
#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "krylov.cuh"

namespace ogs {

bool launch_assembly(const ogs_mesh* m, const AsmArgs& a, bool affine, int kind, cudaStream_t s);
void launch_spmv(const SellView<double>& A, const double* x, double* y, cudaStream_t s);
void launch_dinv(const double* val, const int32_t* diag_pos, double* dinv, int n, cudaStream_t s);
void launch_krylov_init(const SolveArgs& a, int kind, cudaStream_t s);
void launch_krylov_iteration(const SolveArgs& a, int kind, cudaStream_t s, cudaEvent_t eb, cudaEvent_t ee);
void launch_bicgstab_finish(const SolveArgs& a, cudaStream_t s);
void launch_norm_b(const SolveArgs& a, cudaStream_t s);
void launch_mp_convert(const MixedArgs& a, const int32_t* row_len, const int8_t* slot_up, float* U,
                       float* val32, const double* dinv64, float* d32, cudaStream_t s);
void launch_mp_replace(const MixedArgs& a, cudaStream_t s);
void launch_mp_iteration(const MixedArgs& a, cudaStream_t s, cudaEvent_t eb, cudaEvent_t ee);
int mp_persist_grid(const MixedArgs& a);
void launch_mp_convert_cells(const MixedArgs& a, const double* coef, int64_t cells, float* alpha32, float* beta32,
                             unsigned char* mask, float* dbc, const int32_t* diag_pos, const double* dinv64,
                             float* d32, int bc_mode, const unsigned char* bc_flag, const int32_t* bc_rows, int nbc,
                             cudaStream_t s);
void launch_mp_check(const MixedArgs& a, unsigned* out, cudaStream_t s);
int cell_spmv_grid(int nx, int ny, int nz);
void launch_flow_cell_coef(const AsmArgs& a, double* coef, cudaStream_t s);
cudaError_t launch_mp_persist(const MixedArgs& a, int grid, int iters, cudaStream_t s);
int kernels_per_iteration(int kind, int precond);
int krylov_init_launches(int kind, int precond);
void launch_ilu_factor(const IluView& f, const double* val, const int32_t* csr2sell, int64_t nnz,
                       const KState* st, cudaStream_t s);
int vec_grid(int n);
int red_grid(int n);
int mp_spmv_grid(const MixedArgs& a);
void launch_mp_product_pair(const MixedArgs& a, float* y_rows, float* y_lines, cudaStream_t s);
void launch_ilu_tile_pattern(const IluView& f, cudaStream_t s);
cudaError_t launch_mp_barrier_selftest(KState* st, int grid, int withhold, unsigned limit, int* go, cudaStream_t s);
cudaError_t ilu_wait_selftest(int withhold, unsigned limit, int* gave_up, int* rows_ok, cudaStream_t s);
size_t batch_ctl_bytes();
cudaError_t launch_batch_barrier_selftest(void* ctl, unsigned limit, int grid, int withhold, int* go, cudaStream_t s);

// ------------------------------------------------------------------
// small kernels
// ------------------------------------------------------------------
// stored entries of row r in SELL-32 order: slot(j) = slice_ptr[r/32] + 32 j + r%32
struct SellRow
{
    int beg, len;
    __device__ __forceinline__ SellRow(const int32_t* slice_ptr, const int32_t* row_len, int r)
        : beg(slice_ptr[r >> 5] + (r & 31)), len(row_len[r]) {}
    __device__ __forceinline__ int slot(int j) const { return beg + (j << 5); }
};

// Transport assembly from the stored operators (memory_type > 0, after the
// first assembly): the element loop of AssembleMixedHyperbolicParabolicEquation
// with EleMat's matrices (fem_ele_std.cpp:8575-8640) summed over elements --
// A += M / dt + theta K,  b += (M / dt - (1 - theta) K) u0, one thread a row.
__global__ void k_mt_from_operators(const int32_t* __restrict__ slice_ptr, const int32_t* __restrict__ row_len,
                                    const int32_t* __restrict__ col, const double* __restrict__ M,
                                    const double* __restrict__ K, const double* __restrict__ u, double dt_inverse,
                                    double th, double* val, double* b, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const SellRow R(slice_ptr, row_len, i);
        double bi = 0.0;
        for (int j = 0; j < R.len; j++)
        {
            const int k = R.slot(j);
            const double m = M[k] * dt_inverse, kk = K[k];
            val[k] += m + kk * th;
            if (u) bi += (m + kk * (-(1.0 - th))) * u[col[k]];
        }
        b[i] += bi;
    }
}

__global__ void k_dirichlet_row_only(const int32_t* __restrict__ slice_ptr, const int32_t* __restrict__ row_len,
                                     const int32_t* __restrict__ col, const int32_t* __restrict__ diag_pos,
                                     double* val, double* b, const int32_t* __restrict__ rows,
                                     const double* __restrict__ vals, int nbc)
{
    // CSparseMatrix::Diagonize, CRS, column kept (matrix_class.cpp:1663-1700,1783)
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nbc; q += gridDim.x * blockDim.x)
    {
        const int id = rows[q];
        const int dp = diag_pos[id];
        const double vdiag = dp >= 0 ? val[dp] : 0.0;
        const SellRow R(slice_ptr, row_len, id);
        for (int j = 0; j < R.len; j++)
            if (col[R.slot(j)] != id) val[R.slot(j)] = 0.0;
        b[id] = vdiag * vals[q];
    }
}

__global__ void k_dirichlet_symmetric(const int32_t* __restrict__ slice_ptr,
                                      const int32_t* __restrict__ row_len, const int32_t* __restrict__ col,
                                      const int32_t* __restrict__ diag_pos, double* val, double* b,
                                      const unsigned char* __restrict__ flag,
                                      const double* __restrict__ valn, const double* __restrict__ valf,
                                      const int32_t* __restrict__ rows, int n, int nrows)
{
    // MXRandbed (matrix_routines.cpp:2314-2520): lift column into b, zero
    // row and column, keep the diagonal (a zero diagonal -> DBL_EPSILON).
    // A row given twice is lifted with its first value (the column is zero
    // afterwards) and keeps its last value on the diagonal, as the
    // sequential SetKnownX loop leaves it.  rows: the Dirichlet rows and the
    // rows with a Dirichlet column, in row order (every other row is left as
    // it is); one thread per row, the column loads of a group of entries
    // issued together before the flags.
    constexpr int G = 16;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    {
        const int i = rows[q];
        if (!OGS_IN(i, nrows, kOobDirCol)) continue;
        const SellRow R(slice_ptr, row_len, i);
        if (flag[i])
        {
            const int dp = diag_pos[i];
            double d = dp >= 0 ? val[dp] : 0.0;
            if (fabs(d) < DBL_MIN) d = DBL_EPSILON;
            for (int j = 0; j < R.len; j++) val[R.slot(j)] = 0.0;
            if (dp >= 0) val[dp] = d;
            b[i] = valn[i] * d;
        }
        else
        {
            double bi = b[i];
            for (int j0 = 0; j0 < R.len; j0 += G)
            {
                int c[G];
#pragma unroll
                for (int t = 0; t < G; t++) c[t] = j0 + t < R.len ? col[R.slot(j0 + t)] : -1;
                bool f[G];
#pragma unroll
                for (int t = 0; t < G; t++) f[t] = c[t] >= 0 && OGS_IN(c[t], nrows, kOobDirCol) && flag[c[t]];
#pragma unroll
                for (int t = 0; t < G; t++)
                    if (f[t])
                    {
                        const int k = R.slot(j0 + t);
                        bi -= val[k] * valf[c[t]];
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

__global__ void k_mark_rows(unsigned char* flag, double* valn, double* valf, const int32_t* __restrict__ rows,
                            const double* __restrict__ vals, const double* __restrict__ vfirst, int nbc)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nbc; q += gridDim.x * blockDim.x)
    {
        flag[rows[q]] = 1;
        valn[rows[q]] = vals[q];
        valf[rows[q]] = vfirst[q];
    }
}

// the rows a symmetric Dirichlet set touches: its own rows and, the
// pattern being structurally symmetric, the columns of their rows
__global__ void k_mark_touched(const int32_t* __restrict__ slice_ptr, const int32_t* __restrict__ row_len,
                               const int32_t* __restrict__ col, const int32_t* __restrict__ rows, int nbc,
                               unsigned char* touch)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nbc; q += gridDim.x * blockDim.x)
    {
        const SellRow R(slice_ptr, row_len, rows[q]);
        for (int j = 0; j < R.len; j++) touch[col[R.slot(j)]] = 1;
    }
}

__global__ void k_sell_to_csr(const double* __restrict__ sell, const int32_t* __restrict__ csr2sell,
                              double* __restrict__ out, int64_t nnz)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = sell[csr2sell[k]];
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

// state of a solve in flight (see solve_begin / solve_advance)
struct SolveTask
{
    cudaEvent_t ev = nullptr;   // marks the pending header (or x) copy
    int phase = 0;              // 0 idle, 1 iterating, 2 copying x out, 3 finished
    bool mixed = false, xdev = false;
    int kind = 0;
    cudaGraphExec_t ge = nullptr;
    int per = 0, launched = 0, rounds = 0, chunk_before = -1;
    int fp32_iters = 0, fp32_repl = 0;  // FP32 phase of a solve that fell back to FP64
    int fp32_fmt = -1;                  // operator format of the FP32 phase
    double* x_out = nullptr;
    ogs_status status = OGS_OK;
    float ms = 0.f;
};

struct ogs_system
{
    ogs_mesh* m = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int n = 0;
    double *val = nullptr, *b = nullptr, *x = nullptr;
    double *r = nullptr, *r0 = nullptr, *p = nullptr, *ph = nullptr, *s = nullptr, *sh = nullptr,
           *t = nullptr, *v = nullptr, *dinv = nullptr;
    double* lu = nullptr;     // ILU(0) factors on the CSR pattern (allocated on first use)
    // transport operators stored under memory_type > 0 (SELL order, allocated
    // on first use): mass, and Laplace + advection + storage
    double *op_mass = nullptr, *op_k = nullptr;
    bool op_valid = false;
    int* d_ilu_bad = nullptr;
    int* ilu_flags = nullptr;                // [3][n] rows published per launch (ILU kernels)
    unsigned long long* ilu_ticket = nullptr;  // [3] block tickets of the ILU kernels
    int32_t *ilu_pl_row = nullptr, *ilu_pl_col = nullptr, *ilu_pu_row = nullptr, *ilu_pu_col = nullptr;
    double *ilu_pl_val = nullptr, *ilu_pu_val = nullptr, *ilu_pu_diag = nullptr;  // packed sweep rows
    double* ilu_rdiag = nullptr;  // [n] 1 / u_ii of the factored rows
    // the tile sweeps' rows (lattice patterns), flags and tickets
    bool ilu_use_tiles = false;
    int* ilu_tile_flags = nullptr;
    unsigned long long* ilu_tile_ticket = nullptr;
    double *ilu_tl_val = nullptr, *ilu_tu_val = nullptr, *ilu_tu_dg = nullptr, *ilu_tu_piv = nullptr;
    int32_t* ilu_t_rb = nullptr;
    unsigned char *ilu_tl_mask = nullptr, *ilu_tu_mask = nullptr;
    double *ek = nullptr, *u0 = nullptr, *gpv = nullptr, *qbuf = nullptr, *vec_in = nullptr,
           *vec_out = nullptr, *u1 = nullptr;
    // RICHARDS_FLOW Picard step: iterate, solution, old level, reductions
    double *rich_it = nullptr, *rich_x = nullptr, *rich_old = nullptr, *rich_red = nullptr;
    double* h_rich = nullptr;  // pinned: sum d^2, sum it^2, max |d|
    KState* st = nullptr;
    KState* h_st = nullptr;   // pinned header copy
    int* d_bad = nullptr;
    int* h_bad = nullptr;     // pinned
    ogs_solver_config cfg{};
    bool configured = false;
    double bnorm_prev = 1.0;  // Linear_EQS ctor: bNorm = 1.0
    bool val_zero = true;     // val holds zeros only (Initialize, nothing added since)
    // Dirichlet
    int nbc = 0;
    int bc_mode = OGS_DIRICHLET_ROW_ONLY;
    // the set on the device, as uploaded (rows, values, first values): an
    // identical upload leaves the device arrays as they are
    std::vector<int32_t> bc_host_rows;
    std::vector<double> bc_host_vals, bc_host_vfirst;
    bool bc_host_valid = false;
    int32_t* bc_rows = nullptr;
    double* bc_vals = nullptr;
    int bc_cap = 0;
    unsigned char* bc_flag = nullptr;
    int32_t* bc_touch = nullptr;   // symmetric sets: the rows the elimination changes
    unsigned char* bc_mask = nullptr;
    int ntouch = 0;
    double* bc_valn = nullptr;
    double* bc_valf = nullptr;
    double* bc_vfirst = nullptr;
    // iteration chunks captured as graphs, per solver kind
    cudaGraphExec_t chunk[2] = {nullptr, nullptr};
    int chunk_iters[2] = {0, 0};
    void* vec_block = nullptr;
    size_t vec_stride = 0;
    // FP32-inner / FP64-refinement buffers (allocated on first use)
    void* f32_block = nullptr;
    size_t f32_bytes = 0;
    float *x32 = nullptr, *r32 = nullptr, *p32 = nullptr, *s32 = nullptr, *d32 = nullptr, *U = nullptr,
          *val32 = nullptr, *u32 = nullptr, *w32 = nullptr;
    int fmt = -1;
    int f32_pad = 0;       // zero pad in front of every FP32 vector and operator row (values)
    int f32_ustride = 0;   // values per operator row of the diagonal-offset form
    int mp_lines = 0;      // product kernel the captured iterations use (MixedArgs::lines)
    cudaGraphExec_t mp_chunk = nullptr, mp_replace = nullptr;
    int mp_replace_scaled = 0;  // form (MixedArgs::scaled) mp_replace was captured with
    // persistent FP32 CG (OGS_SCHEDULE_PERSISTENT): the arguments of the
    // direct cooperative launches and their grid (0: graph schedule)
    MixedArgs mp_args{};
    int mp_grid = 0;
    // cell coefficients of the flow operator on a hex lattice (mesh grid):
    // alpha per cell, beta at [cells], summed over the assemblies since
    // Initialize; mf_state 1 while the assembled matrix has that form
    double* mf_coef = nullptr;
    int mf_state = 0;
    // the assembled matrix is symmetric (flow assembly, symmetric Dirichlet
    // elimination); the FP32 upper-half diagonal operator needs it
    bool symmetric = true;
    float *mf_alpha32 = nullptr, *mf_beta32 = nullptr, *mf_dbc = nullptr;
    unsigned char* mf_mask = nullptr;
    unsigned* d_check = nullptr;
    unsigned* h_check = nullptr;  // pinned
    double prof_persist_ms = 0.0;
    int64_t prof_persist_iters = 0;
    // SpMV timing inside the chunk graphs (ogs_gpu_profile)
    static constexpr int kChunk = 16;
    bool prof_on = false;
    cudaEvent_t prof_b[kChunk] = {}, prof_e[kChunk] = {};
    double prof_spmv_ms = 0.0, prof_solve_ms = 0.0;
    int64_t prof_spmv_n = 0, prof_solves = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    SolveTask task;
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
    std::memset(&a, 0, sizeof a);  // every field not set below is 0 (no tiles, the default spin limit)
    a.A.slice_ptr = s->m->slice_ptr;
    a.A.col = s->m->sell_col;
    a.A.val = s->val;
    a.A.n = s->n;
    a.v.x = s->x; a.v.b = s->b; a.v.r = s->r; a.v.r0 = s->r0; a.v.p = s->p; a.v.ph = s->ph;
    a.v.s = s->s; a.v.sh = s->sh; a.v.t = s->t; a.v.v = s->v; a.v.dinv = s->dinv;
    a.st = s->st;
    a.precond = s->cfg.precond;
    ogs_mesh* m = s->m;
    a.ilu.row_ptr = m->row_ptr;
    a.ilu.col = m->col;
    a.ilu.diag = m->csr_diag;
    a.ilu.lu = s->lu;
    a.ilu.lrows = m->lvl_rows;
    a.ilu.urows = m->ulvl_rows;
    a.ilu.n = s->n;
    a.ilu.n_lpos = m->n_lpos;
    a.ilu.n_upos = m->n_upos;
    a.ilu.flags = s->ilu_flags;
    a.ilu.ticket = s->ilu_ticket;
    a.ilu.lptr = m->lvl_ptr;
    a.ilu.uptr = m->ulvl_ptr;
    a.ilu.n_lev = m->n_lvl;
    a.ilu.n_ulev = m->n_ulvl;
    a.ilu.kl = m->ilu_kl;
    a.ilu.ku = m->ilu_ku;
    a.ilu.pl_row = s->ilu_pl_row; a.ilu.pl_col = s->ilu_pl_col; a.ilu.pl_val = s->ilu_pl_val;
    a.ilu.pu_row = s->ilu_pu_row; a.ilu.pu_col = s->ilu_pu_col; a.ilu.pu_val = s->ilu_pu_val;
    a.ilu.pu_diag = s->ilu_pu_diag;
    a.ilu.bad = s->d_ilu_bad;
    a.ilu.rdiag = s->ilu_rdiag;
    if (s->ilu_use_tiles && s->ilu_tile_flags)
    {
        a.ilu.tiles = m->tiles;
        a.ilu.lnx = m->lnx; a.ilu.lny = m->lny; a.ilu.lnz = m->lnz;
        a.ilu.tnx = m->tnx; a.ilu.tny = m->tny; a.ilu.tnz = m->tnz;
        a.ilu.tile_order = m->tile_order;
        a.ilu.tile_flags = s->ilu_tile_flags;
        a.ilu.tile_ticket = s->ilu_tile_ticket;
        a.ilu.tl_val = s->ilu_tl_val; a.ilu.tu_val = s->ilu_tu_val; a.ilu.tu_dg = s->ilu_tu_dg;
        a.ilu.tu_piv = s->ilu_tu_piv; a.ilu.t_rb = s->ilu_t_rb;
        a.ilu.tl_mask = s->ilu_tl_mask; a.ilu.tu_mask = s->ilu_tu_mask;
    }
    return a;
}

void drop_graphs(ogs_system* s)
{
    for (int k = 0; k < 2; k++)
        if (s->chunk[k]) { cudaGraphExecDestroy(s->chunk[k]); s->chunk[k] = nullptr; }
    if (s->mp_chunk) { cudaGraphExecDestroy(s->mp_chunk); s->mp_chunk = nullptr; }
    if (s->mp_replace) { cudaGraphExecDestroy(s->mp_replace); s->mp_replace = nullptr; }
}

// Event pairs bracket the SpMV of every kProfEvery-th iteration of a chunk
// (one pair per iteration slowed the chunk by ~10%); the sampled launches
// give the average SpMV duration.
constexpr int kProfEvery = 4;
// FP32 iterations per persistent launch (a due replacement ends it sooner)
constexpr int kPersistIters = 64;

void accumulate_prof(ogs_system* s, int executed)
{
    for (int i = 0; i < executed; i += kProfEvery)
    {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s->prof_b[i], s->prof_e[i]) == cudaSuccess)
        {
            s->prof_spmv_ms += ms;
            s->prof_spmv_n += 1;
        }
        else
            cudaGetLastError();
    }
}

template <class F>
ogs_status capture(ogs_system* s, cudaGraphExec_t* out, F body)
{
    cudaGraph_t g;
    OGS_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    body();
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (e != cudaSuccess) { set_error("graph capture: %s", cudaGetErrorString(e)); return OGS_CUDA_ERROR; }
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { set_error("graph instantiate: %s", cudaGetErrorString(e)); return OGS_CUDA_ERROR; }
    return OGS_OK;
}

ogs_status get_chunk(ogs_system* s, int kind, const SolveArgs& a, cudaGraphExec_t* out, int* iters)
{
    if (!s->chunk[kind])
    {
        const int C = ogs_system::kChunk;
        cudaGraph_t g;
        OGS_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < C; i++)
        {
            const bool ev = s->prof_on && i % kProfEvery == 0;  // timing sample
            launch_krylov_iteration(a, kind, s->stream, ev ? s->prof_b[i] : nullptr, ev ? s->prof_e[i] : nullptr);
        }
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
    if (s->vec_block) cudaStreamSynchronize(s->stream);
    double* bufs[] = {s->val,     s->ek,      s->u0,      s->gpv,     s->qbuf,     s->vec_in,
                      s->vec_out, s->bc_vals, s->bc_valn, s->bc_valf, s->bc_vfirst};
    for (double* p : bufs) cudaFree(p);
    cudaFree(s->vec_block);
    cudaFree(s->f32_block);
    cudaFree(s->lu);
    cudaFree(s->op_mass);
    cudaFree(s->op_k);
    cudaFree(s->mf_coef);
    cudaFree(s->u1);
    cudaFree(s->rich_it);
    cudaFree(s->rich_x);
    cudaFree(s->rich_old);
    cudaFree(s->rich_red);
    if (s->h_rich) cudaFreeHost(s->h_rich);
    cudaFree(s->d_check);
    if (s->h_check) cudaFreeHost(s->h_check);
    cudaFree(s->d_ilu_bad);
    cudaFree(s->ilu_flags);
    cudaFree(s->ilu_ticket);
    cudaFree(s->ilu_pl_row);
    cudaFree(s->ilu_pl_col);
    cudaFree(s->ilu_pl_val);
    cudaFree(s->ilu_pu_row);
    cudaFree(s->ilu_pu_col);
    cudaFree(s->ilu_pu_val);
    cudaFree(s->ilu_pu_diag);
    cudaFree(s->ilu_rdiag);
    cudaFree(s->ilu_tile_flags);
    cudaFree(s->ilu_tile_ticket);
    cudaFree(s->ilu_tl_val);
    cudaFree(s->ilu_tu_val);
    cudaFree(s->ilu_tu_dg);
    cudaFree(s->ilu_tu_piv);
    cudaFree(s->ilu_t_rb);
    cudaFree(s->ilu_tl_mask);
    cudaFree(s->ilu_tu_mask);
    cudaFree(s->st);
    cudaFree(s->d_bad);
    cudaFree(s->bc_rows);
    cudaFree(s->bc_flag);
    cudaFree(s->bc_touch);
    cudaFree(s->bc_mask);
    if (s->h_st) cudaFreeHost(s->h_st);
    if (s->h_bad) cudaFreeHost(s->h_bad);
    for (int i = 0; i < ogs_system::kChunk; i++)
    {
        if (s->prof_b[i]) cudaEventDestroy(s->prof_b[i]);
        if (s->prof_e[i]) cudaEventDestroy(s->prof_e[i]);
    }
    if (s->task.ev) cudaEventDestroy(s->task.ev);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return OGS_OK;
}

// cell-coefficient record of a new assembly cycle (Initialize)
static ogs_status mf_reset(ogs_system* s)
{
    const ogs_mesh* m = s->m;
    s->symmetric = true;
    s->mf_state = 0;
    if (!m->grid || m->ngauss < 2) return OGS_OK;  // one Gauss point under-integrates L_box
    const size_t cells = (size_t)(m->gx - 1) * (m->gy - 1) * (m->gz - 1);
    if (!s->mf_coef) OGS_CUDA_TRY(cudaMalloc(&s->mf_coef, (cells + 1) * sizeof(double)));
    OGS_CUDA_TRY(cudaMemsetAsync(s->mf_coef, 0, (cells + 1) * sizeof(double), s->stream));
    s->mf_state = 1;
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
    double** vecs[] = {&s->p, &s->r, &s->s, &s->x, &s->dinv, &s->ph, &s->sh, &s->r0, &s->v, &s->t, &s->b};
    cudaError_t e = cudaMalloc(&s->val, std::max<int64_t>(1, m->sell_nnz) * sizeof(double));
    // Krylov vectors in one allocation (one cudaMalloc per system)
    const size_t nvec = sizeof(vecs) / sizeof(vecs[0]);
    const size_t stride = (nb + 255) & ~size_t(255);
    if (e == cudaSuccess) e = cudaMalloc(&s->vec_block, stride * nvec);
    for (size_t k = 0; k < nvec && e == cudaSuccess; k++)
        *vecs[k] = (double*)((char*)s->vec_block + k * stride);
    s->vec_stride = stride;
    if (e == cudaSuccess) e = cudaMalloc(&s->st, sizeof(KState));
    if (e == cudaSuccess) e = cudaMemsetAsync(s->st, 0, sizeof(KState), s->stream);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_bad, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_st, sizeof(KState));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_bad, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->bc_flag, std::max(1, s->n));
    if (e == cudaSuccess) e = cudaMalloc(&s->bc_valn, nb);
    if (e == cudaSuccess) e = cudaMalloc(&s->bc_valf, nb);
    // stream-ordered: work on the system's (possibly non-blocking) stream
    // must not overtake these
    if (e == cudaSuccess) e = cudaMemsetAsync(s->val, 0, m->sell_nnz * sizeof(double), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->b, 0, nb, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->x, 0, nb, s->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e != cudaSuccess)
    {
        set_error("system_create: %s", cudaGetErrorString(e));
        ogs_gpu_system_destroy(s);
        return e == cudaErrorMemoryAllocation ? OGS_OOM : OGS_CUDA_ERROR;
    }
    // CNumerics defaults (rf_num_new.cpp:77-165): BiCGStab, Jacobi, 1000, 1e-12
    s->cfg.method = OGS_LS_BICGSTAB;
    s->cfg.precond = OGS_PRECOND_JACOBI;
    s->cfg.max_iter = 1000;
    s->cfg.tol = 1e-12;
    s->cfg.check_norm_rhs = 1;
    s->configured = true;
    if (mf_reset(s) != OGS_OK)
    {
        ogs_gpu_system_destroy(s);
        return OGS_CUDA_ERROR;
    }
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
    if (c->precision != OGS_PRECISION_FP64 && c->precision != OGS_PRECISION_FP32_REFINED &&
        c->precision != OGS_PRECISION_FP32_CELLS)
    {
        set_error("configure: unknown precision %d", c->precision);
        return OGS_BAD_ARG;
    }
    if (c->schedule != OGS_SCHEDULE_PERSISTENT && c->schedule != OGS_SCHEDULE_GRAPH)
    {
        set_error("configure: unknown schedule %d", c->schedule);
        return OGS_BAD_ARG;
    }
    s->cfg = *c;
    drop_graphs(s);
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_initialize(ogs_system* s)
{
    if (!s) { set_error("initialize: NULL system"); return OGS_BAD_ARG; }
    OGS_CUDA_TRY(cudaMemsetAsync(s->val, 0, s->m->sell_nnz * sizeof(double), s->stream));
    OGS_CUDA_TRY(cudaMemsetAsync(s->b, 0, (size_t)s->n * sizeof(double), s->stream));
    s->val_zero = true;
    return mf_reset(s);
}

static ogs_status check_params(const ogs_assembly_params* p)
{
    if (!p) { set_error("assemble: NULL params"); return OGS_BAD_ARG; }
    if (p->pcs_type < 0 || p->pcs_type > 2)
    {
        set_error(p->pcs_type == OGS_PCS_RICHARDS_FLOW ? "assemble: RICHARDS_FLOW goes through ogs_gpu_assemble_richards"
                                                       : "assemble: bad pcs_type %d",
                  p->pcs_type);
        return OGS_BAD_ARG;
    }
    if (!(p->dt > 0.0)) { set_error("assemble: dt must be > 0"); return OGS_BAD_ARG; }
    if (!(p->time_unit_factor != 0.0)) { set_error("assemble: time_unit_factor must be non-zero"); return OGS_BAD_ARG; }
    return OGS_OK;
}

__global__ void k_set_int(int* p, int v) { *p = v; }

constexpr int kNoBadElement = 0x7fffffff;

// Enqueues an element kernel (kind 0 flow, 1 transport assembly, 2 Gauss-
// point flux); the singular-Jacobian flag lands in s->h_bad (pinned) once
// the stream has passed this point.
static ogs_status enqueue_element_kernel(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                         const double* u0, const double* gpv, int kind, double* q_out,
                                         double* val = nullptr, double* val2 = nullptr,
                                         const double* u1 = nullptr, const ogs_richards_params* rp = nullptr)
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
    a.val = val ? val : s->val;
    a.b = s->b;
    a.val2 = val2;
    a.q_out = q_out;
    a.bad_elem = s->d_bad;
    a.p = *p;
    ogs_status st;
    if ((st = stage_in(s, elem_k, m->n_elem, &s->ek, &a.elem_k))) return st;
    if ((st = stage_in(s, u0, m->n_nodes, &s->u0, &a.u0))) return st;
    if ((st = stage_in(s, gpv, (size_t)m->n_elem * m->ngp * 3, &s->gpv, &a.gpv))) return st;
    if ((st = stage_in(s, u1, m->n_nodes, &s->u1, &a.u1))) return st;
    if (rp) a.r = *rp;
    a.val_store = kind == 0 && a.val == s->val && s->val_zero ? 1 : 0;
    a.nslots = m->sell_nnz;
    a.nrows = m->n_nodes;
    k_set_int<<<1, 1, 0, s->stream>>>(s->d_bad, kNoBadElement);
    OGS_LAUNCH_CHECK();
    if (!launch_assembly(m, a, m->affine, kind, s->stream))
    {
        set_error("no kernel for element type %d with %d Gauss points", m->elem_type, m->ngp);
        return OGS_BAD_ARG;
    }
    OGS_LAUNCH_CHECK();
    if (kind != 2 && a.val == s->val) s->val_zero = false;  // the velocity kernel writes q only
    // the cell-coefficient form holds for flow without mass lumping
    if (kind == 0 && s->mf_state == 1)
    {
        if (p->mass_lumping)
            s->mf_state = 0;
        else
        {
            launch_flow_cell_coef(a, s->mf_coef, s->stream);
            OGS_LAUNCH_CHECK();
        }
    }
    if (kind == 1)
    {
        s->mf_state = 0;
        s->symmetric = false;  // advection
    }
    if (kind == 3) s->mf_state = 0;  // coefficients vary inside the cells
    OGS_CUDA_TRY(cudaMemcpyAsync(s->h_bad, s->d_bad, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    return OGS_OK;
}

static ogs_status element_flag_status(const ogs_system* s)
{
    if (*s->h_bad != kNoBadElement)
    {
        set_error("singular Jacobian (|det J| < DBL_EPSILON) in element %d", *s->h_bad - 1);
        return OGS_SINGULAR_JACOBIAN;
    }
    return OGS_OK;
}

static ogs_status run_element_kernel(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                     const double* u0, const double* gpv, int kind, double* q_out)
{
    ogs_status st = enqueue_element_kernel(s, p, elem_k, u0, gpv, kind, q_out);
    if (st) return st;
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return element_flag_status(s);
}

extern "C" ogs_status ogs_gpu_assemble(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                       const double* u0, const double* gp_velocity)
{
    if (!s) { set_error("assemble: NULL system"); return OGS_BAD_ARG; }
    ogs_status st = check_params(p);
    if (st) return st;
    if (p->pcs_type != OGS_PCS_MASS_TRANSPORT && !elem_k) { set_error("assemble: flow needs elem_k"); return OGS_BAD_ARG; }
    const bool stored = p->pcs_type == OGS_PCS_MASS_TRANSPORT && p->memory_type > 0;
    if (p->pcs_type == OGS_PCS_MASS_TRANSPORT && !gp_velocity && !(stored && s->op_valid))
    {
        set_error("assemble: transport needs gp_velocity");
        return OGS_BAD_ARG;
    }
    if (!stored) return run_element_kernel(s, p, elem_k, u0, gp_velocity, p->pcs_type == OGS_PCS_MASS_TRANSPORT ? 1 : 0, nullptr);
    // Memory_Type > 0: the reference computes and stores the element
    // matrices on the first time step and reuses them afterwards
    // (fem_ele_std.cpp:8534-8588); here the first assembly scatters the
    // mass and the theta-weighted operator into two stored matrices
    const ogs_mesh* m = s->m;
    const size_t bytes = (size_t)std::max<int64_t>(1, m->sell_nnz) * sizeof(double);
    if (!s->op_valid)
    {
        if (!s->op_mass) OGS_CUDA_TRY(cudaMalloc(&s->op_mass, bytes));
        if (!s->op_k) OGS_CUDA_TRY(cudaMalloc(&s->op_k, bytes));
        OGS_CUDA_TRY(cudaMemsetAsync(s->op_mass, 0, bytes, s->stream));
        OGS_CUDA_TRY(cudaMemsetAsync(s->op_k, 0, bytes, s->stream));
        st = enqueue_element_kernel(s, p, elem_k, u0, gp_velocity, 1, nullptr, s->op_mass, s->op_k);
        if (st) return st;
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        if ((st = element_flag_status(s))) return st;
        s->op_valid = true;
    }
    s->mf_state = 0;
    s->symmetric = false;
    const double* du;
    if ((st = stage_in(s, u0, m->n_nodes, &s->u0, &du))) return st;
    k_mt_from_operators<<<vec_grid(s->n), 256, 0, s->stream>>>(m->slice_ptr, m->row_len, m->sell_col, s->op_mass,
                                                             s->op_k, du, 1.0 / p->dt, p->theta, s->val, s->b, s->n);
    s->val_zero = false;
    OGS_LAUNCH_CHECK();
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_cache_reset(ogs_system* s)
{
    if (!s) { set_error("cache_reset: NULL system"); return OGS_BAD_ARG; }
    s->op_valid = false;
    return OGS_OK;
}

// ------------------------------------------------------------------
// RICHARDS_FLOW
// ------------------------------------------------------------------
static ogs_status dirichlet_upload(ogs_system* s, const int64_t* rows, const double* values, int64_t n_rows,
                                   int32_t mode);
static ogs_status dirichlet_apply(ogs_system* s);

static ogs_status check_richards(const ogs_assembly_params* p, const ogs_richards_params* r)
{
    if (!p || !r) { set_error("richards: NULL params"); return OGS_BAD_ARG; }
    if (p->pcs_type != OGS_PCS_RICHARDS_FLOW) { set_error("richards: pcs_type must be OGS_PCS_RICHARDS_FLOW"); return OGS_BAD_ARG; }
    if (!(p->dt > 0.0) || !(p->time_unit_factor != 0.0) || !(p->viscosity > 0.0))
    {
        set_error("richards: dt, time_unit_factor and viscosity must be set (> 0)");
        return OGS_BAD_ARG;
    }
    if ((r->capillary_model != 4 && r->capillary_model != 6) || (r->permeability_model != 4 && r->permeability_model != 6))
    {
        set_error("richards: capillary model %d / permeability model %d not supported (4 van Genuchten, 6 Brooks-Corey)",
                  r->capillary_model, r->permeability_model);
        return OGS_BAD_ARG;
    }
    const bool vg_ok = r->capillary_model != 4 || (r->m > 0.0 && r->m < 1.0);
    const bool kr_ok = r->permeability_model != 4 || (r->kr_m > 0.0 && r->kr_m <= 1.0);
    if (!(r->pb > 0.0) || !(r->slm > r->slr) || !(r->m > 0.0) || !vg_ok || !(r->kr_slm > r->kr_slr) ||
        !(r->kr_m > 0.0) || !kr_ok)
    {
        set_error("richards: bad curve parameters (pb > 0, slm > slr, van Genuchten 0 < m < 1)");
        return OGS_BAD_ARG;
    }
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_assemble_richards(ogs_system* s, const ogs_assembly_params* p, const ogs_richards_params* r,
                                                const double* elem_k, const double* p_old, const double* p_iter)
{
    if (!s || !elem_k || !p_iter) { set_error("assemble_richards: NULL argument"); return OGS_BAD_ARG; }
    ogs_status st = check_richards(p, r);
    if (st) return st;
    if ((st = enqueue_element_kernel(s, p, elem_k, p_old, nullptr, 3, nullptr, nullptr, nullptr, p_iter, r))) return st;
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return element_flag_status(s);
}

// sum (it - x)^2, sum it^2 (grid_sum, fixed order) and max |it - x| of a
// Picard iteration; out[0..2]
__global__ void k_picard_error(const double* __restrict__ it, const double* __restrict__ x, int n, double* part,
                               unsigned* ticket, double* out)
{
    double v[2] = {0.0, 0.0}, mx = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const double d = it[i] - x[i];
        v[0] += d * d;
        v[1] += it[i] * it[i];
        mx = fmax(mx, fabs(d));
    }
    atomicMax((unsigned long long*)(out + 2), (unsigned long long)__double_as_longlong(mx));
    double o[2];
    if (grid_sum<2, double>(v, o, part, ticket) && threadIdx.x == 0)
    {
        out[0] = o[0];
        out[1] = o[1];
    }
}

// iterate = (1 - theta) iterate + theta x  (the new value itself for theta 1)
__global__ void k_picard_update(double* it, const double* __restrict__ x, int n, double theta)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        it[i] = theta == 1.0 ? x[i] : (1.0 - theta) * it[i] + theta * x[i];
}

extern "C" ogs_status ogs_gpu_richards_step(ogs_system* s, const ogs_assembly_params* p, const ogs_richards_params* r,
                                            const double* elem_k, const double* p_old, double* p_iter,
                                            const int64_t* bc_rows, const double* bc_values, int64_t n_bc,
                                            int32_t bc_mode, const ogs_picard_config* nls, ogs_picard_stats* stats)
{
    if (!s || !elem_k || !p_old || !p_iter || !nls) { set_error("richards_step: NULL argument"); return OGS_BAD_ARG; }
    ogs_status st = check_richards(p, r);
    if (st) return st;
    if (nls->error_method < 1 || nls->error_method > 4 || nls->max_iterations < 1 || !(nls->tolerance > 0.0))
    {
        set_error("richards_step: error_method 1..4 (LMAX, ENORM, EVNORM, ERNORM), max_iterations >= 1, tolerance > 0");
        return OGS_BAD_ARG;
    }
    const int n = s->n;
    const size_t nb = (size_t)n * sizeof(double);
    if (!s->rich_it)
    {
        OGS_CUDA_TRY(cudaMalloc(&s->rich_it, nb));
        OGS_CUDA_TRY(cudaMalloc(&s->rich_x, nb));
        OGS_CUDA_TRY(cudaMalloc(&s->rich_old, nb));
        OGS_CUDA_TRY(cudaMalloc(&s->rich_red, (2 * kMaxBlocks + 4) * sizeof(double)));
        OGS_CUDA_TRY(cudaMemset(s->rich_red, 0, (2 * kMaxBlocks + 4) * sizeof(double)));
        OGS_CUDA_TRY(cudaMallocHost(&s->h_rich, 3 * sizeof(double)));
    }
    OGS_CUDA_TRY(cudaMemcpyAsync(s->rich_it, p_iter, nb, cudaMemcpyDefault, s->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(s->rich_old, p_old, nb, cudaMemcpyDefault, s->stream));
    if ((st = dirichlet_upload(s, bc_rows, bc_values, n_bc, bc_mode))) return st;
    double* red = s->rich_red;
    unsigned* ticket = (unsigned*)(red + 2 * kMaxBlocks + 3);
    // own events: the linear solves time themselves with ev0 / ev1
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    OGS_CUDA_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess)
    {
        cudaEventDestroy(e0);
        set_error("richards_step: cudaEventCreate failed");
        return OGS_CUDA_ERROR;
    }
    struct EvGuard
    {
        cudaEvent_t a, b;
        ~EvGuard()
        {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } guard{e0, e1};
    OGS_CUDA_TRY(cudaEventRecord(e0, s->stream));
    double theta0 = 1.0 - p->nls_relaxation;  // nl_theta (rf_pcs.cpp:9652)
    if (theta0 < DBL_EPSILON) theta0 = 1.0;
    ogs_picard_stats out{};
    double last = 1.0;
    int fails = 0;
    for (int it = 0; it < nls->max_iterations; it++)
    {
        // CRFProcess::Execute: assembly at the iterate, conditions, solve
        if ((st = ogs_gpu_initialize(s))) return st;
        if ((st = enqueue_element_kernel(s, p, elem_k, s->rich_old, nullptr, 3, nullptr, nullptr, nullptr,
                                         s->rich_it, r)))
            return st;
        if ((st = dirichlet_apply(s))) return st;
        OGS_CUDA_TRY(cudaMemcpyAsync(s->rich_x, s->rich_it, nb, cudaMemcpyDeviceToDevice, s->stream));
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        if ((st = element_flag_status(s))) return st;
        ogs_solve_stats ls{};
        st = ogs_gpu_solve(s, s->rich_x, &ls);
        out.linear_iterations += ls.iterations;
        if (st != OGS_OK && st != OGS_NOT_CONVERGED) return st;
        // CalcIterationNODError (PICARD branch): iterate against the solution
        OGS_CUDA_TRY(cudaMemsetAsync(red + 2 * kMaxBlocks, 0, 3 * sizeof(double), s->stream));
        k_picard_error<<<red_grid(n), 256, 0, s->stream>>>(s->rich_it, s->rich_x, n, red, ticket, red + 2 * kMaxBlocks);
        OGS_LAUNCH_CHECK();
        OGS_CUDA_TRY(cudaMemcpyAsync(s->h_rich, red + 2 * kMaxBlocks, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                     s->stream));
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        const double* h = s->h_rich;
        double abs_err;
        if (nls->error_method == 1) abs_err = h[2];                                     // LMAX
        else if (nls->error_method == 4) abs_err = sqrt(h[0]) / (sqrt(h[1]) + DBL_EPSILON);  // ERNORM
        else abs_err = sqrt(h[0]);                                                      // ENORM, EVNORM
        const double err = abs_err / nls->tolerance;
        const double theta = err < 1.0 ? 1.0 : theta0;
        k_picard_update<<<vec_grid(n), 256, 0, s->stream>>>(s->rich_it, s->rich_x, n, theta);
        OGS_LAUNCH_CHECK();
        out.iterations = it + 1;
        out.error = err;
        // ExecuteNonLinear, default error branch (rf_pcs.cpp:9735-9760)
        if (err <= 1.0)
        {
            out.converged = 1;
            break;
        }
        const double percent = 100.0 * ((last - err) / last);
        fails = (it > 0 && percent < 1.0) ? fails + 1 : 0;
        last = err;
        if (fails > 1)
        {
            out.diverged = 1;
            break;
        }
    }
    OGS_CUDA_TRY(cudaEventRecord(e1, s->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(p_iter, s->rich_it, nb, cudaMemcpyDefault, s->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    out.solve_ms = ms;
    if (stats) *stats = out;
    if (!out.converged)
    {
        set_error("richards_step: Picard iteration %s after %d iterations (error/tolerance %.3e)",
                  out.diverged ? "stagnated" : "did not converge", out.iterations, out.error);
        return OGS_NOT_CONVERGED;
    }
    return OGS_OK;
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

// Dirichlet set of the system: host checks and de-duplication, device
// arrays (rows, values; for SYMMETRIC the row flags and the diagonal / lift
// values per row).  Waits for its copies.
static ogs_status dirichlet_upload(ogs_system* s, const int64_t* rows, const double* values, int64_t n_rows,
                                   int32_t mode)
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
    // SetKnownX_i is applied row by row in list order, so a row listed twice
    // keeps its last value: keep the last occurrence of every row
    std::vector<double> vsrc(n_rows), vfirst;
    if (n_rows) OGS_CUDA_TRY(cudaMemcpy(vsrc.data(), values, n_rows * sizeof(double),
                                        vdev ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    {
        std::vector<int64_t> order(n_rows);
        for (int64_t q = 0; q < n_rows; q++) order[q] = q;
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return r32[a] < r32[b]; });
        std::vector<int32_t> ru;
        std::vector<double> vu;
        ru.reserve(n_rows);
        vu.reserve(n_rows);
        vfirst.reserve(n_rows);
        double first = 0.0;
        for (int64_t k = 0; k < n_rows; k++)
        {
            const int64_t q = order[k];
            if (k == 0 || r32[order[k - 1]] != r32[q]) first = vsrc[q];
            if (k + 1 < n_rows && r32[order[k + 1]] == r32[q]) continue;  // a later duplicate follows
            ru.push_back(r32[q]);
            vu.push_back(vsrc[q]);
            vfirst.push_back(first);
        }
        r32.swap(ru);
        vh.swap(vu);
        n_rows = (int64_t)r32.size();
    }
    auto same_bits = [](const std::vector<double>& x, const std::vector<double>& y) {
        return x.size() == y.size() && (x.empty() || std::memcmp(x.data(), y.data(), x.size() * sizeof(double)) == 0);
    };
    if (s->bc_host_valid && s->bc_mode == mode && s->bc_host_rows == r32 && same_bits(s->bc_host_vals, vh) &&
        same_bits(s->bc_host_vfirst, vfirst))
        return OGS_OK;
    s->bc_host_valid = false;
    if (n_rows > s->bc_cap)
    {
        cudaFree(s->bc_rows);
        cudaFree(s->bc_vals);
        cudaFree(s->bc_vfirst);
        s->bc_rows = nullptr;
        s->bc_vals = nullptr;
        s->bc_vfirst = nullptr;
        OGS_CUDA_TRY(cudaMalloc(&s->bc_rows, n_rows * sizeof(int32_t)));
        OGS_CUDA_TRY(cudaMalloc(&s->bc_vals, n_rows * sizeof(double)));
        OGS_CUDA_TRY(cudaMalloc(&s->bc_vfirst, n_rows * sizeof(double)));
        s->bc_cap = (int)n_rows;
    }
    s->nbc = (int)n_rows;
    s->bc_mode = mode;
    if (!n_rows) return OGS_OK;
    OGS_CUDA_TRY(cudaMemcpyAsync(s->bc_rows, r32.data(), n_rows * sizeof(int32_t), cudaMemcpyHostToDevice, s->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(s->bc_vals, vh.data(), n_rows * sizeof(double), cudaMemcpyHostToDevice,
                                 s->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(s->bc_vfirst, vfirst.data(), n_rows * sizeof(double),
                                 cudaMemcpyHostToDevice, s->stream));
    if (mode == OGS_DIRICHLET_SYMMETRIC)
    {
        const int g = std::max(1, std::min(1024, (int)((n_rows + 255) / 256)));
        OGS_CUDA_TRY(cudaMemsetAsync(s->bc_flag, 0, s->n, s->stream));
        k_mark_rows<<<g, 256, 0, s->stream>>>(s->bc_flag, s->bc_valn, s->bc_valf, s->bc_rows, s->bc_vals,
                                              s->bc_vfirst, s->nbc);
        OGS_LAUNCH_CHECK();
        // the touched rows, through a byte mask, listed in row order (warps
        // on neighbouring rows share the SELL segments of their entries)
        ogs_mesh* m = s->m;
        if (!s->bc_touch) OGS_CUDA_TRY(cudaMalloc(&s->bc_touch, std::max(1, s->n) * sizeof(int32_t)));
        if (!s->bc_mask) OGS_CUDA_TRY(cudaMalloc(&s->bc_mask, std::max(1, s->n)));
        OGS_CUDA_TRY(cudaMemsetAsync(s->bc_mask, 0, s->n, s->stream));
        k_mark_touched<<<g, 256, 0, s->stream>>>(m->slice_ptr, m->row_len, m->sell_col, s->bc_rows, s->nbc,
                                                 s->bc_mask);
        OGS_LAUNCH_CHECK();
        std::vector<unsigned char> hm((size_t)s->n);
        OGS_CUDA_TRY(cudaMemcpyAsync(hm.data(), s->bc_mask, s->n, cudaMemcpyDeviceToHost, s->stream));
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        std::vector<int32_t> list;
        for (int i = 0; i < s->n; i++)
            if (hm[i]) list.push_back(i);
        s->ntouch = (int)list.size();
        if (!list.empty())
            OGS_CUDA_TRY(cudaMemcpyAsync(s->bc_touch, list.data(), list.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, s->stream));
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));  // list is a host array
    }
    // the host staging vectors must outlive the copies above
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->bc_host_rows = r32;
    s->bc_host_vals = vh;
    s->bc_host_vfirst = vfirst;
    s->bc_host_valid = true;
    return OGS_OK;
}

// applies the uploaded Dirichlet set to the assembled matrix and b
// (kernels only)
static ogs_status dirichlet_apply(ogs_system* s)
{
    if (!s->nbc) return OGS_OK;
    s->val_zero = false;
    ogs_mesh* m = s->m;
    if (s->bc_mode == OGS_DIRICHLET_ROW_ONLY)
    {
        const int g = std::max(1, std::min(1024, (s->nbc + 255) / 256));
        k_dirichlet_row_only<<<g, 256, 0, s->stream>>>(m->slice_ptr, m->row_len, m->sell_col, m->diag_pos,
                                                       s->val, s->b, s->bc_rows, s->bc_vals, s->nbc);
        OGS_LAUNCH_CHECK();
    }
    else
    {
        k_dirichlet_symmetric<<<std::max(1, (s->ntouch + 127) / 128), 128, 0, s->stream>>>(
                                                                           m->slice_ptr, m->row_len, m->sell_col,
                                                                           m->diag_pos, s->val, s->b, s->bc_flag,
                                                                           s->bc_valn, s->bc_valf, s->bc_touch,
                                                                           s->ntouch, s->n);
        OGS_LAUNCH_CHECK();
    }
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_set_dirichlet(ogs_system* s, const int64_t* rows, const double* values,
                                            int64_t n_rows, int32_t mode)
{
    ogs_status st = dirichlet_upload(s, rows, values, n_rows, mode);
    if (st) return st;
    if (mode == OGS_DIRICHLET_ROW_ONLY && n_rows > 0) s->symmetric = false;  // the columns stay
    if ((st = dirichlet_apply(s))) return st;
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return OGS_OK;
}

// FP32 inner CG with FP64 residual replacement (mixed.cu): buffers, FP32
// operator, first replacement; x64 already holds the initial guess with the
// Dirichlet values, dinv the FP64 Jacobi inverse.  Leaves the replacement
// graph launched; the task loop reads the header next.
// The 14 upper offsets of a 27-point lattice numbered line by line, with
// nx = off[3] nodes per line and nxy = off[9] per plane: 0, 1, then
// B - 1, B, B + 1 for the line bases B = nx, nxy - nx, nxy, nxy + nx
static bool lattice27_offsets(const std::vector<int32_t>& off)
{
    if (off.size() != 14) return false;
    const int64_t nx = off[3], nxy = off[9];
    if (nx < 3 || nxy - nx - 1 <= nx + 1) return false;
    const int64_t base[4] = {nx, nxy - nx, nxy, nxy + nx};
    if (off[0] != 0 || off[1] != 1) return false;
    for (int l = 0; l < 4; l++)
        for (int dx = -1; dx <= 1; dx++)
            if (off[2 + 3 * l + dx + 1] != base[l] + dx) return false;
    return true;
}

// The 5 upper offsets of a 9-point plane lattice numbered line by line
// (quads), nx = off[3] nodes per line: 0, 1, nx - 1, nx, nx + 1
static bool lattice9_offsets(const std::vector<int32_t>& off)
{
    if (off.size() != 5) return false;
    const int64_t nx = off[3];
    return nx >= 3 && off[0] == 0 && off[1] == 1 && off[2] == nx - 1 && off[4] == nx + 1;
}

// which four-rows-per-thread product the offsets allow (MixedArgs::lines)
static int lattice_lines(const std::vector<int32_t>& off)
{
    return lattice27_offsets(off) ? 1 : lattice9_offsets(off) ? 2 : 0;
}

static ogs_status begin_fp32_refined(ogs_system* s, KState* h)
{
    ogs_mesh* m = s->m;
    const ogs_solver_config& c = s->cfg;
    const int n = s->n;
    // FP32 operator: cell coefficients on a hex lattice whose matrix has
    // that form (fmt 2, on request), else for symmetric matrices the upper
    // half of the diagonal-offset form for the hex (14), Kuhn-tet (8) and
    // quad (5) patterns (fmt 0), else SELL-32 with FP32 values (fmt 1)
    const bool cells_ok = c.precision == OGS_PRECISION_FP32_CELLS && s->mf_state == 1 &&
                          cell_spmv_grid(m->gx, m->gy, m->gz) <= kMaxBlocks;
    const int want = cells_ok ? 2 : s->symmetric && (m->n_up == 14 || m->n_up == 8 || m->n_up == 5) ? 0 : 1;
    const size_t cells = m->grid ? (size_t)(m->gx - 1) * (m->gy - 1) * (m->gz - 1) : 0;
    if (s->fmt != want && s->fmt >= 0)
    {
        cudaFree(s->f32_block);
        s->f32_block = nullptr;
        s->fmt = -1;
        drop_graphs(s);  // the captured iterations hold the operator format
    }
    if (s->fmt < 0)
    {
        s->fmt = want;
        auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
        // diagonal-offset form: zero pads of pad values in front of every
        // operator row and FP32 vector and of pad + 64 behind, so the
        // lattice product's windows (at most the largest offset + 4 values
        // outside [0, n)) read zeros
        const int pad = s->fmt == 0 ? (m->host_up_off.back() + 16 + 31) & ~31 : 0;
        s->f32_pad = pad;
        s->f32_ustride = s->fmt == 0 ? (pad + n + 64 + 31) & ~31 : (n + 31) & ~31;
        const size_t v4 = al(((size_t)n + 2 * (size_t)pad + 64) * sizeof(float));
        const size_t op = s->fmt == 0 ? (size_t)m->n_up * s->f32_ustride * sizeof(float)
                        : s->fmt == 1 ? (size_t)m->sell_nnz * sizeof(float)
                                      : al(cells * sizeof(float)) + 256 + v4 + al((size_t)n);
        s->f32_bytes = 7 * v4 + op;
        OGS_CUDA_TRY(cudaMalloc(&s->f32_block, s->f32_bytes));
        OGS_CUDA_TRY(cudaMemsetAsync(s->f32_block, 0, s->f32_bytes, s->stream));
        char* p = (char*)s->f32_block;
        auto vec = [&](int k) { return (float*)(p + k * v4) + pad; };
        s->p32 = vec(0); s->r32 = vec(1); s->x32 = vec(2); s->s32 = vec(3); s->d32 = vec(4);
        s->u32 = vec(5); s->w32 = vec(6);
        char* opb = p + 7 * v4;
        s->U = nullptr; s->val32 = nullptr;
        if (s->fmt == 0) s->U = (float*)opb + pad;
        else if (s->fmt == 1) s->val32 = (float*)opb;
        else
        {
            s->mf_alpha32 = (float*)opb;
            s->mf_beta32 = (float*)(opb + al(cells * sizeof(float)));
            s->mf_dbc = (float*)(opb + al(cells * sizeof(float)) + 256);
            s->mf_mask = (unsigned char*)(opb + al(cells * sizeof(float)) + 256 + v4);
        }
    }
    MixedArgs a;
    std::memset(&a, 0, sizeof a);
    a.A.slice_ptr = m->slice_ptr; a.A.col = m->sell_col; a.A.val = s->val; a.A.n = n;
    a.fmt = s->fmt; a.U = s->U; a.ustride = s->f32_ustride; a.pad = s->f32_pad; a.up_off = m->up_off;
    a.n_up = m->n_up;
    a.val32 = s->val32;
    for (int d = 0; d < 16 && d < (int)m->host_up_off.size(); d++) a.off[d] = m->host_up_off[d];
    a.d32 = s->d32; a.x = s->x; a.b = s->b; a.r64 = s->r;
    // stored FP32 operators iterate on the Jacobi-scaled system; the cell
    // operator and the persistent kernel use the preconditioned form
    a.scaled = s->fmt != 2 && c.schedule == OGS_SCHEDULE_GRAPH;
    // the four-rows-per-thread product when the offsets are a line-by-line
    // 27-point lattice's (OGS_FP32_PRODUCT=rows keeps the row kernel, for
    // comparisons)
    {
        const char* e = std::getenv("OGS_FP32_PRODUCT");
        a.lines = s->fmt == 0 && a.scaled && !(e && !std::strcmp(e, "rows")) ? lattice_lines(m->host_up_off) : 0;
        if (a.lines != s->mp_lines)
        {
            drop_graphs(s);  // the captured iterations hold the product kernel
            s->mp_lines = a.lines;
        }
    }
    a.x32 = s->x32; a.r32 = s->r32; a.p32 = s->p32; a.s32 = s->s32; a.u32 = s->u32; a.w32 = s->w32;
    a.st = s->st; a.n = n;
    if (s->fmt == 2)
    {
        a.gx = m->gx; a.gy = m->gy; a.gz = m->gz;
        a.mf_alpha = s->mf_alpha32; a.mf_beta = s->mf_beta32; a.mf_mask = s->mf_mask; a.mf_dbc = s->mf_dbc;
        // unit-coefficient box matrices by corner-equality pattern (bit 0 x,
        // 1 y, 2 z): 1-D stiffness +-1/h and mass h/3 | h/6, tensor products
        const double hs[3] = {m->ghx, m->ghy, m->ghz};
        for (int pat = 0; pat < 8; pat++)
        {
            double K1[3], M1[3];
            for (int d = 0; d < 3; d++)
            {
                const bool eq = (pat >> d) & 1;
                K1[d] = (eq ? 1.0 : -1.0) / hs[d];
                M1[d] = hs[d] * (eq ? 1.0 / 3.0 : 1.0 / 6.0);
            }
            a.mf_L[pat] = (float)(K1[0] * M1[1] * M1[2] + M1[0] * K1[1] * M1[2] + M1[0] * M1[1] * K1[2]);
            a.mf_M[pat] = (float)(M1[0] * M1[1] * M1[2]);
        }
        for (int d = 0; d < 3; d++)
        {
            a.mf_m1[2 * d] = (float)(hs[d] / 3.0);
            a.mf_m1[2 * d + 1] = (float)(hs[d] / 6.0);
        }
        launch_mp_convert_cells(a, s->mf_coef, (int64_t)cells, s->mf_alpha32, s->mf_beta32, s->mf_mask, s->mf_dbc,
                                m->diag_pos, s->dinv, s->d32, s->bc_mode, s->bc_flag, s->bc_rows, s->nbc,
                                s->stream);
        OGS_LAUNCH_CHECK();
        // the FP32 operator must reproduce the assembled FP64 matrix (up to
        // FP32 rounding); a matrix changed by other means falls back
        if (!s->d_check) OGS_CUDA_TRY(cudaMalloc(&s->d_check, 2 * sizeof(unsigned)));
        if (!s->h_check) OGS_CUDA_TRY(cudaMallocHost(&s->h_check, 2 * sizeof(unsigned)));
        launch_mp_check(a, s->d_check, s->stream);
        OGS_LAUNCH_CHECK();
        OGS_CUDA_TRY(cudaMemcpyAsync(s->h_check, s->d_check, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost,
                                     s->stream));
        OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        float dmax, smax;
        std::memcpy(&dmax, &s->h_check[0], sizeof(float));
        std::memcpy(&smax, &s->h_check[1], sizeof(float));
        if (!(dmax <= 1e-5f * smax))
        {
            s->mf_state = 0;
            return begin_fp32_refined(s, h);
        }
    }
    else
    {
        launch_mp_convert(a, m->row_len, m->slot_up, s->U, s->val32, s->dinv, s->d32, s->stream);
        OGS_LAUNCH_CHECK();
    }
    OGS_CUDA_TRY(cudaMemsetAsync(s->x32, 0, (size_t)n * sizeof(float), s->stream));
    h->scale = 1.0;
    h->ratio = 1.0;
    h->first = 1;
    h->nb_spmv = s->fmt == 2 ? cell_spmv_grid(m->gx, m->gy, m->gz) : mp_spmv_grid(a);
    a.nb_spmv = h->nb_spmv;
    h->nb_upd = red_grid(n);
    h->delta = c.inner_tol > 0.0 ? c.inner_tol : 1e-2;
    OGS_CUDA_TRY(cudaMemcpyAsync(s->st, h, kStateHeader, cudaMemcpyHostToDevice, s->stream));
    SolveArgs sa = make_solve_args(s);
    launch_norm_b(sa, s->stream);
    OGS_LAUNCH_CHECK();
    if (s->mp_replace && s->mp_replace_scaled != a.scaled)
    {
        cudaGraphExecDestroy(s->mp_replace);  // captured for the other form
        s->mp_replace = nullptr;
    }
    if (!s->mp_replace)
    {
        s->mp_replace_scaled = a.scaled;
        ogs_status st = capture(s, &s->mp_replace, [&]() { launch_mp_replace(a, s->stream); });
        if (st) return st;
    }
    s->mp_args = a;
    s->mp_grid = c.schedule == OGS_SCHEDULE_PERSISTENT ? mp_persist_grid(a) : 0;
    if (!s->mp_chunk && s->mp_grid == 0)
    {
        ogs_status st = capture(s, &s->mp_chunk, [&]() {
            for (int i = 0; i < ogs_system::kChunk; i++)
            {
                const bool ev = s->prof_on && i % kProfEvery == 0;  // timing sample
                launch_mp_iteration(a, s->stream, ev ? s->prof_b[i] : nullptr, ev ? s->prof_e[i] : nullptr);
            }
        });
        if (st) return st;
    }
    OGS_CUDA_TRY(cudaGraphLaunch(s->mp_replace, s->stream));
    count_launches(4);
    s->task.fp32_fmt = s->fmt;
    return OGS_OK;
}

// ILU(0) of the current matrix (every solve: assembly and Dirichlet
// conditions change the values); a zero pivot ends the solve with
// OGS_BREAKDOWN before any iteration.
static ogs_status ilu_factor(ogs_system* s)
{
    ogs_mesh* m = s->m;
    if (!s->lu)
    {
        OGS_CUDA_TRY(cudaMalloc(&s->lu, std::max<int64_t>(1, m->nnz) * sizeof(double)));
        OGS_CUDA_TRY(cudaMalloc(&s->d_ilu_bad, sizeof(int)));
        OGS_CUDA_TRY(cudaMalloc(&s->ilu_rdiag, std::max(1, s->n) * sizeof(double)));
        // publication flags start below every launch number, tickets at 0
        OGS_CUDA_TRY(cudaMalloc(&s->ilu_flags, 3 * (size_t)std::max(1, s->n) * sizeof(int)));
        OGS_CUDA_TRY(cudaMalloc(&s->ilu_ticket, 3 * sizeof(unsigned long long)));
        OGS_CUDA_TRY(cudaMemsetAsync(s->ilu_flags, 0, 3 * (size_t)std::max(1, s->n) * sizeof(int), s->stream));
        OGS_CUDA_TRY(cudaMemsetAsync(s->ilu_ticket, 0, 3 * sizeof(unsigned long long), s->stream));
        // the sweeps' packed rows (rows of at most 16 L / U entries)
        if (std::max(m->ilu_kl, m->ilu_ku) <= 16)
        {
            const size_t nl = std::max(1, m->n_lpos), nu = std::max(1, m->n_upos);
            const size_t kl = std::max(1, m->ilu_kl), ku = std::max(1, m->ilu_ku);
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_pl_row, nl * sizeof(int32_t)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_pl_col, kl * nl * sizeof(int32_t)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_pl_val, kl * nl * sizeof(double)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_pu_row, nu * sizeof(int32_t)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_pu_col, ku * nu * sizeof(int32_t)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_pu_val, ku * nu * sizeof(double)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_pu_diag, nu * sizeof(double)));
        }
        drop_graphs(s);  // captured sweeps hold the factor pointer
    }
    // the tile sweeps on lattice patterns (OGS_ILU_SWEEP=levels: the level
    // kernels, for comparisons; read at every factorisation)
    {
        const char* e = std::getenv("OGS_ILU_SWEEP");
        const bool tiles = m->tiles && !(e && !std::strcmp(e, "levels"));
        if (tiles != s->ilu_use_tiles)
        {
            drop_graphs(s);  // the captured iterations hold the sweep kernels
            s->ilu_use_tiles = tiles;
        }
        if (tiles && !s->ilu_tile_flags)
        {
            const size_t rows = (size_t)m->tiles * kIluTile * kIluTile * kIluTile;
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tile_flags, 3 * (size_t)m->tiles * sizeof(int)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tile_ticket, 3 * sizeof(unsigned long long)));
            OGS_CUDA_TRY(cudaMemsetAsync(s->ilu_tile_flags, 0, 3 * (size_t)m->tiles * sizeof(int), s->stream));
            OGS_CUDA_TRY(cudaMemsetAsync(s->ilu_tile_ticket, 0, 3 * sizeof(unsigned long long), s->stream));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tl_val, 7 * rows * sizeof(double)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tu_val, 7 * rows * sizeof(double)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tu_dg, rows * sizeof(double)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tu_piv, rows * sizeof(double)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_t_rb, rows * sizeof(int32_t)));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tl_mask, rows));
            OGS_CUDA_TRY(cudaMalloc(&s->ilu_tu_mask, rows));
            SolveArgs pa = make_solve_args(s);
            launch_ilu_tile_pattern(pa.ilu, s->stream);
            OGS_LAUNCH_CHECK();
        }
    }
    const int big = 0x7fffffff;
    OGS_CUDA_TRY(cudaMemcpyAsync(s->d_ilu_bad, &big, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    SolveArgs a = make_solve_args(s);
    launch_ilu_factor(a.ilu, s->val, m->csr2sell, m->nnz, s->st, s->stream);
    OGS_LAUNCH_CHECK();
    count_launches(1);
    OGS_CUDA_TRY(cudaMemcpyAsync(s->h_bad, s->d_ilu_bad, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (*s->h_bad == -1)
    {
        set_error("solve: ILU(0) factorisation: a wait for a row gave up");
        return OGS_CUDA_ERROR;
    }
    if (*s->h_bad != big)
    {
        set_error("solve: ILU(0) zero pivot in row %d", *s->h_bad);
        return OGS_BREAKDOWN;
    }
    return OGS_OK;
}

// x = v everywhere (no-preconditioner Jacobi inverse of the FP32 mode)
__global__ void k_fill(double* x, double v, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = v;
}

// ------------------------------------------------------------------
// A solve as a resumable task.  solve_begin enqueues the start of the
// solve (initial guess, Dirichlet values, preconditioner, first residual,
// first chunk of iterations or the first FP64 replacement) and the copy of
// the solver header behind it; solve_advance waits for (or, non-blocking,
// checks) that copy, reads the header and enqueues what comes next -- a
// chunk of iterations, a residual replacement, or the copy of x out.  No
// host synchronisation between the launches of one solve, so one host
// thread can keep many systems' solves in flight (the request server);
// ogs_gpu_solve is begin + blocking advances, the same launches in the same
// order.
// ------------------------------------------------------------------
static ogs_status task_fail(ogs_system* s, ogs_status st)
{
    s->task.phase = 3;
    s->task.status = st;
    return st;
}

static ogs_status enqueue_header(ogs_system* s)
{
    OGS_CUDA_TRY(cudaMemcpyAsync(s->h_st, s->st, kStateHeader, cudaMemcpyDeviceToHost, s->stream));
    OGS_CUDA_TRY(cudaEventRecord(s->task.ev, s->stream));
    return OGS_OK;
}

static ogs_status solve_begin(ogs_system* s, double* x_inout)
{
    if (!s || !x_inout) { set_error("solve: NULL argument"); return OGS_BAD_ARG; }
    const ogs_solver_config& c = s->cfg;
    if (c.precision != OGS_PRECISION_FP64 && c.method != OGS_LS_CG)
    {
        set_error("solve: the FP32-inner / FP64-refinement mode runs CG (ls_method 5)");
        return OGS_BAD_ARG;
    }
    if (c.precision != OGS_PRECISION_FP64 && c.precond == OGS_PRECOND_ILU0)
    {
        set_error("solve: the FP32-inner / FP64-refinement mode takes Jacobi or no preconditioner");
        return OGS_BAD_ARG;
    }
    if (s->task.phase == 1 || s->task.phase == 2)
    {
        set_error("solve: a solve of this system is still in flight");
        return OGS_BAD_ARG;
    }
    SolveTask& T = s->task;
    T = SolveTask{T.ev};
    if (!T.ev) OGS_CUDA_TRY(cudaEventCreateWithFlags(&T.ev, cudaEventDisableTiming));
    T.x_out = x_inout;
    T.xdev = is_device_ptr(x_inout);
    T.mixed = c.precision != OGS_PRECISION_FP64;
    T.kind = c.method == OGS_LS_CG ? SK_CG : SK_BICGSTAB;
    if (c.precond == OGS_PRECOND_ILU0)
    {
        ogs_status st = ilu_factor(s);
        if (st) return st;
    }
    const size_t nb = (size_t)s->n * sizeof(double);
    OGS_CUDA_TRY(cudaEventRecord(s->ev0, s->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(s->x, x_inout, nb, T.xdev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
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
    else if (T.mixed)
    {
        // no preconditioner: M^-1 = I
        k_fill<<<vec_grid(s->n), kThreads, 0, s->stream>>>(s->dinv, 1.0, s->n);
        OGS_LAUNCH_CHECK();
    }
    KState* h = s->h_st;
    std::memset(h, 0, kStateHeader);
    h->bnorm = c.check_norm_rhs ? s->bnorm_prev : -1.0;
    h->tol = c.tol;
    h->error = 1.0e10;
    h->max_iter = c.max_iter;
    h->alpha = h->omega = h->rho0 = 1.0;
    if (T.mixed)
    {
        ogs_status st = begin_fp32_refined(s, h);
        if (st) return st;
    }
    else
    {
        h->nb_spmv = vec_grid(s->n);
        h->nb_upd = red_grid(s->n);
        OGS_CUDA_TRY(cudaMemcpyAsync(s->st, h, kStateHeader, cudaMemcpyHostToDevice, s->stream));
        launch_krylov_init(a, T.kind, s->stream);
        OGS_LAUNCH_CHECK();
        count_launches(krylov_init_launches(T.kind, a.precond) - 1);
        ogs_status st = get_chunk(s, T.kind, a, &T.ge, &T.per);
        if (st) return st;
    }
    {
        ogs_status st = enqueue_header(s);
        if (st) return st;
    }
    T.phase = 1;
    return OGS_OK;
}

// One step of the task.  block: wait for the pending header copy; else
// return at once (finished = false) while it is in flight.
static ogs_status solve_advance(ogs_system* s, bool block, bool* finished)
{
    SolveTask& T = s->task;
    *finished = false;
    if (T.phase == 0 || T.phase == 3)
    {
        *finished = T.phase == 3;
        return OGS_OK;
    }
    if (block)
    {
        cudaError_t e = cudaEventSynchronize(T.ev);
        if (e != cudaSuccess) { set_error("solve: %s", cudaGetErrorString(e)); return task_fail(s, OGS_CUDA_ERROR); }
    }
    else
    {
        cudaError_t e = cudaEventQuery(T.ev);
        if (e == cudaErrorNotReady) return OGS_OK;
        if (e != cudaSuccess) { set_error("solve: %s", cudaGetErrorString(e)); return task_fail(s, OGS_CUDA_ERROR); }
    }
    const ogs_solver_config& c = s->cfg;
    KState* h = s->h_st;
    if (T.phase == 2)
    {
        // x has landed: close the solve
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s->ev0, s->ev1);
        s->bnorm_prev = h->bnorm;
        if (s->prof_on)
        {
            s->prof_solve_ms += ms;
            s->prof_solves += 1;
        }
        T.ms = ms;
        T.status = (ogs_status)h->status;
        T.phase = 3;
        *finished = true;
        return OGS_OK;
    }
    // phase 1: a header copy has landed
    if (T.mixed && h->done && h->fallback)
    {
        // FP32 cycles stopped gaining: continue with FP64 CG from x64
        T.fp32_iters = h->iter;
        T.fp32_repl = h->replacements;
        T.mixed = false;
        T.kind = SK_CG;
        T.chunk_before = -1;
        const double bn = h->bnorm;
        std::memset(h, 0, kStateHeader);
        h->bnorm = bn;  // |b| / bn = 1: CheckNormRHS does not return early
        h->tol = c.tol;
        h->error = 1.0e10;
        h->max_iter = std::max(1, c.max_iter - T.fp32_iters);
        h->alpha = h->omega = h->rho0 = 1.0;
        h->nb_spmv = vec_grid(s->n);
        h->nb_upd = red_grid(s->n);
        SolveArgs a = make_solve_args(s);
        if (cudaMemcpyAsync(s->st, h, kStateHeader, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
            return task_fail(s, OGS_CUDA_ERROR);
        launch_krylov_init(a, SK_CG, s->stream);
        if (cudaGetLastError() != cudaSuccess) return task_fail(s, OGS_CUDA_ERROR);
        count_launches(krylov_init_launches(SK_CG, a.precond));
        ogs_status st = get_chunk(s, SK_CG, a, &T.ge, &T.per);
        if (st) return task_fail(s, st);
        if (enqueue_header(s)) return task_fail(s, OGS_CUDA_ERROR);
        return OGS_OK;
    }
    if (T.mixed)
    {
        if (T.chunk_before >= 0)
        {
            if (s->prof_on && s->mp_grid > 0)
            {
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, s->prof_b[0], s->prof_e[0]) == cudaSuccess)
                {
                    s->prof_persist_ms += ms;
                    s->prof_persist_iters += h->iter - T.chunk_before;
                }
                else
                    cudaGetLastError();
            }
            else if (s->prof_on)
                accumulate_prof(s, std::min(ogs_system::kChunk, h->iter - T.chunk_before));
            T.chunk_before = -1;
        }
        if (!h->done)
        {
            if (++T.rounds > 4 * c.max_iter + 64)
            {
                set_error("solve: mixed-precision state did not finish");
                return task_fail(s, OGS_CUDA_ERROR);
            }
            if (h->replace)
            {
                if (cudaGraphLaunch(s->mp_replace, s->stream) != cudaSuccess) return task_fail(s, OGS_CUDA_ERROR);
                count_launches(4);
            }
            else if (s->mp_grid > 0)
            {
                // one cooperative launch runs up to kPersistIters iterations;
                // it returns early when a replacement is due or the solve ended
                T.chunk_before = h->iter;
                if (s->prof_on) cudaEventRecord(s->prof_b[0], s->stream);
                if (launch_mp_persist(s->mp_args, s->mp_grid, kPersistIters, s->stream) != cudaSuccess)
                {
                    set_error("solve: cooperative launch of the FP32 CG kernel failed: %s",
                              cudaGetErrorString(cudaGetLastError()));
                    return task_fail(s, OGS_CUDA_ERROR);
                }
                if (s->prof_on) cudaEventRecord(s->prof_e[0], s->stream);
                count_launches(1);
            }
            else
            {
                T.chunk_before = h->iter;
                if (cudaGraphLaunch(s->mp_chunk, s->stream) != cudaSuccess) return task_fail(s, OGS_CUDA_ERROR);
                count_launches(3 * ogs_system::kChunk);
            }
            if (enqueue_header(s)) return task_fail(s, OGS_CUDA_ERROR);
            return OGS_OK;
        }
    }
    else
    {
        if (T.chunk_before >= 0 && s->prof_on)
            accumulate_prof(s, std::min(T.per, h->iter - T.chunk_before + (T.kind == SK_BICGSTAB && h->done ? 1 : 0)));
        T.chunk_before = -1;
        if (!h->done)
        {
            if (T.launched > c.max_iter + T.per)
            {
                set_error("solve: solver state did not finish");
                return task_fail(s, OGS_CUDA_ERROR);
            }
            T.chunk_before = h->iter;
            if (cudaGraphLaunch(T.ge, s->stream) != cudaSuccess) return task_fail(s, OGS_CUDA_ERROR);
            count_launches((int64_t)T.per * kernels_per_iteration(T.kind, s->cfg.precond));
            T.launched += T.per;
            if (enqueue_header(s)) return task_fail(s, OGS_CUDA_ERROR);
            return OGS_OK;
        }
        if (h->finish_s)
        {
            SolveArgs a = make_solve_args(s);
            launch_bicgstab_finish(a, s->stream);
            if (cudaGetLastError() != cudaSuccess) return task_fail(s, OGS_CUDA_ERROR);
            count_launches(1);
        }
    }
    // done: x out, then close at the next advance
    const size_t nb = (size_t)s->n * sizeof(double);
    if (cudaMemcpyAsync(T.x_out, s->x, nb, T.xdev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                        s->stream) != cudaSuccess ||
        cudaEventRecord(s->ev1, s->stream) != cudaSuccess || cudaEventRecord(T.ev, s->stream) != cudaSuccess)
    {
        set_error("solve: copying x out failed");
        return task_fail(s, OGS_CUDA_ERROR);
    }
    T.phase = 2;
    return OGS_OK;
}

static ogs_status solve_end(ogs_system* s, ogs_solve_stats* stats)
{
    SolveTask& T = s->task;
    const KState* h = s->h_st;
    if (s->cfg.precond == OGS_PRECOND_ILU0 && s->d_ilu_bad && T.status == OGS_OK)
    {
        // an ILU sweep that gave up waiting for a row marked -1
        int bad = 0;
        if (cudaMemcpy(&bad, s->d_ilu_bad, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            T.status = OGS_CUDA_ERROR;
        else if (bad == -1)
        {
            set_error("solve: an ILU(0) sweep gave up waiting for a row");
            T.status = OGS_CUDA_ERROR;
        }
    }
    if (stats)
    {
        std::memset(stats, 0, sizeof *stats);
        stats->iterations = h->iter + T.fp32_iters;
        stats->status = T.status;
        stats->rel_residual = h->error;
        stats->b_norm = h->bnorm;
        stats->refinements = h->replacements + T.fp32_repl;
        stats->fp64_fallback = T.fp32_iters > 0 || T.fp32_repl > 0 ? 1 : 0;
        stats->solve_ms = T.ms;
        stats->fp32_operator = T.fp32_fmt;
    }
    const ogs_status st = T.status;
    T.phase = 0;
    return st;
}

extern "C" ogs_status ogs_gpu_solve(ogs_system* s, double* x_inout, ogs_solve_stats* stats)
{
    ogs_status st = solve_begin(s, x_inout);
    if (st) return st;
    bool fin = false;
    while (!fin)
    {
        st = solve_advance(s, true, &fin);
        if (st) { s->task.phase = 0; return st; }
    }
    return solve_end(s, stats);
}

extern "C" ogs_status ogs_gpu_solve_begin(ogs_system* s, double* x_inout) { return solve_begin(s, x_inout); }

extern "C" ogs_status ogs_gpu_solve_poll(ogs_system* s, int32_t* finished)
{
    if (!s || !finished) { set_error("solve_poll: NULL argument"); return OGS_BAD_ARG; }
    bool fin = false;
    ogs_status st = solve_advance(s, false, &fin);
    *finished = fin ? 1 : 0;
    return st;
}

extern "C" ogs_status ogs_gpu_solve_end(ogs_system* s, ogs_solve_stats* stats)
{
    if (!s) { set_error("solve_end: NULL system"); return OGS_BAD_ARG; }
    bool fin = s->task.phase == 3;
    while (!fin && s->task.phase != 0)
    {
        ogs_status st = solve_advance(s, true, &fin);
        if (st) { s->task.phase = 0; return st; }
    }
    return solve_end(s, stats);
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
    SellView<double> A{s->m->slice_ptr, s->m->sell_col, s->val, s->n};
    launch_spmv(A, xd, yd, s->stream);
    OGS_LAUNCH_CHECK();
    if (!ydev) OGS_CUDA_TRY(cudaMemcpyAsync(y, yd, nb, cudaMemcpyDeviceToHost, s->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return OGS_OK;
}

// device array of the system -> caller's array (host or device), ordered on
// the system's stream, complete on return
static ogs_status copy_out(const ogs_system* s, void* dst, const void* src, size_t bytes)
{
    OGS_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s->stream));
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
        // gather the SELL-32 slots back into CSR order
        double* tmp = nullptr;
        OGS_CUDA_TRY(cudaMalloc(&tmp, std::max<int64_t>(1, m->nnz) * sizeof(double)));
        k_sell_to_csr<<<vec_grid((int)std::min<int64_t>(m->nnz, 1 << 30)), 256, 0, s->stream>>>(
            s->val, m->csr2sell, tmp, m->nnz);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(val, tmp, m->nnz * sizeof(double), cudaMemcpyDefault, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        cudaFree(tmp);
        if (e != cudaSuccess) { set_error("get_csr: %s", cudaGetErrorString(e)); return OGS_CUDA_ERROR; }
    }
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_get_rhs(const ogs_system* s, double* b)
{
    if (!s || !b) { set_error("get_rhs: NULL argument"); return OGS_BAD_ARG; }
    return copy_out(s, b, s->b, (size_t)s->n * sizeof(double));
}

extern "C" ogs_status ogs_gpu_get_x(const ogs_system* s, double* x)
{
    if (!s || !x) { set_error("get_x: NULL argument"); return OGS_BAD_ARG; }
    return copy_out(s, x, s->x, (size_t)s->n * sizeof(double));
}

extern "C" ogs_status ogs_gpu_get_ilu0(const ogs_system* s, double* lu)
{
    if (!s || !lu) { set_error("get_ilu0: NULL argument"); return OGS_BAD_ARG; }
    if (!s->lu) { set_error("get_ilu0: no ILU(0) factorisation yet (solve with ls_precond 100 first)"); return OGS_BAD_ARG; }
    return copy_out(s, lu, s->lu, (size_t)s->m->nnz * sizeof(double));
}

extern "C" ogs_status ogs_gpu_profile(ogs_system* s, int32_t enable, ogs_profile* out)
{
    if (!s) { set_error("profile: NULL system"); return OGS_BAD_ARG; }
    if (out)
    {
        out->spmv_ms = s->prof_spmv_ms;
        out->spmv_launches = s->prof_spmv_n;
        out->solve_ms = s->prof_solve_ms;
        out->solves = s->prof_solves;
        out->persist_ms = s->prof_persist_ms;
        out->persist_iters = s->prof_persist_iters;
    }
    s->prof_spmv_ms = s->prof_solve_ms = s->prof_persist_ms = 0.0;
    s->prof_spmv_n = s->prof_solves = s->prof_persist_iters = 0;
    const bool on = enable != 0;
    if (on && !s->prof_b[0])
        for (int i = 0; i < ogs_system::kChunk; i++)
        {
            OGS_CUDA_TRY(cudaEventCreate(&s->prof_b[i]));
            OGS_CUDA_TRY(cudaEventCreate(&s->prof_e[i]));
        }
    if (on != s->prof_on)
    {
        s->prof_on = on;
        drop_graphs(s);  // re-capture with / without the events
    }
    return OGS_OK;
}

// ------------------------------------------------------------------
// Internal entry points of the request server (server.cu): the pieces of
// one solve request, enqueued on the system's stream without host waits.
// ------------------------------------------------------------------
namespace ogs {

cudaStream_t system_stream(ogs_system* s) { return s->stream; }

int64_t system_rows(const ogs_system* s) { return s->n; }

// device bytes of a system on mesh m (matrix values, Krylov vectors,
// solver state, Dirichlet arrays, FP32-mode block when fp32)
size_t system_bytes(const ogs_mesh* m, bool fp32)
{
    const size_t n = (size_t)m->n_nodes;
    const size_t vec = ((n * 8 + 255) & ~size_t(255)) * 11;
    size_t b = (size_t)m->sell_nnz * 8 + vec + sizeof(KState) + 3 * n * 8 + n;
    if (fp32)
    {
        const size_t v4 = (n * 4 + 255) & ~size_t(255);
        const bool dia = m->n_up == 14 || m->n_up == 8 || m->n_up == 5;
        b += 7 * v4 + (dia ? (size_t)m->n_up * n * 4 : (size_t)m->sell_nnz * 4);
    }
    return b;
}

// a fresh Linear_EQS for every request: bNorm = 1.0 (equation_class.cpp:
// 85-143), tolerance of the request
void system_reset_request(ogs_system* s, double tol)
{
    s->bnorm_prev = 1.0;
    s->cfg.tol = tol;
}

ogs_status system_upload_dirichlet(ogs_system* s, const int64_t* rows, const double* vals, int64_t n, int32_t mode)
{
    return dirichlet_upload(s, rows, vals, n, mode);
}

// Initialize + element assembly + the uploaded Dirichlet set, enqueued
ogs_status system_enqueue_assembly(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                   const double* u0, const double* gpv)
{
    ogs_status st = ogs_gpu_initialize(s);
    if (st) return st;
    if ((st = enqueue_element_kernel(s, p, elem_k, u0, gpv, p->pcs_type == OGS_PCS_MASS_TRANSPORT ? 1 : 0,
                                     nullptr)))
        return st;
    return dirichlet_apply(s);
}

// Gauss-point Darcy flux into the device array q (enqueued)
ogs_status system_enqueue_velocity(ogs_system* s, const ogs_assembly_params* p, const double* elem_k,
                                   const double* u, double* q)
{
    return enqueue_element_kernel(s, p, elem_k, u, nullptr, 2, q);
}

// singular-Jacobian flag of the last element kernel (valid once the stream
// has passed it)
ogs_status system_element_status(const ogs_system* s) { return element_flag_status(s); }

}  // namespace ogs

// ------------------------------------------------------------------
// self-test of the bounded waits of the cooperative persistent kernels
// ------------------------------------------------------------------
extern "C" ogs_status ogs_gpu_selftest_barrier(int32_t which, int32_t grid, int32_t spin_limit, int32_t withhold,
                                               int32_t* passed)
{
    if (which < 0 || which > 2 || grid < 0 || spin_limit < 0 || !passed)
    {
        set_error("selftest_barrier: bad arguments");
        return OGS_BAD_ARG;
    }
    if (which == 2)
    {
        int gave_up = 0, ok = 0;
        const cudaError_t e = ilu_wait_selftest(withhold ? 1 : 0, spin_limit ? (unsigned)spin_limit : 0u, &gave_up, &ok,
                                                nullptr);
        if (e != cudaSuccess)
        {
            set_error("selftest_barrier: %s", cudaGetErrorString(e));
            return OGS_CUDA_ERROR;
        }
        *passed = ok;
        count_launches(1);
        if (gave_up)
        {
            set_error("selftest_barrier: ILU row wait timeout (%d of 64 rows exact)", ok);
            return OGS_CUDA_ERROR;
        }
        return OGS_OK;
    }
    int dev = 0, sms = 0, coop = 0;
    OGS_CUDA_TRY(cudaGetDevice(&dev));
    OGS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    OGS_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop)
    {
        set_error("selftest_barrier: the device cannot launch cooperative kernels");
        return OGS_CUDA_ERROR;
    }
    // two blocks per SM stay co-resident for both kernels (256 threads, few
    // registers); the cooperative launch checks it
    const int g = grid > 0 ? grid : 2 * sms;
    if (g > 2 * sms)
    {
        set_error("selftest_barrier: grid %d exceeds two blocks per SM", g);
        return OGS_BAD_ARG;
    }
    const size_t ctl_bytes = which == 0 ? sizeof(KState) : batch_ctl_bytes();
    void* ctl = nullptr;
    int* go = nullptr;
    OGS_CUDA_TRY(cudaMalloc(&ctl, ctl_bytes));
    cudaError_t e = cudaMalloc(&go, sizeof(int) * g);
    if (e == cudaSuccess) e = cudaMemset(ctl, 0, ctl_bytes);
    if (e == cudaSuccess) e = cudaMemset(go, 0, sizeof(int) * g);
    if (e == cudaSuccess)
        e = which == 0 ? launch_mp_barrier_selftest((KState*)ctl, g, withhold ? 1 : 0,
                                                    spin_limit ? (unsigned)spin_limit : (1u << 24), go, 0)
                       : launch_batch_barrier_selftest(ctl, (unsigned)spin_limit, g, withhold ? 1 : 0, go, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    std::vector<int> h(g, 0);
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), go, sizeof(int) * g, cudaMemcpyDeviceToHost);
    cudaFree(go);
    cudaFree(ctl);
    if (e != cudaSuccess)
    {
        set_error("selftest_barrier: %s", cudaGetErrorString(e));
        return OGS_CUDA_ERROR;
    }
    int n = 0;
    for (int v : h) n += v;
    *passed = n;
    count_launches(1);
    if (n < g - (withhold ? 1 : 0))
    {
        set_error("selftest_barrier: barrier timeout (%d of %d arriving blocks passed)", n, g - (withhold ? 1 : 0));
        return OGS_CUDA_ERROR;
    }
    return OGS_OK;
}

// ------------------------------------------------------------------
// bounds checks of the debug build
// ------------------------------------------------------------------
unsigned long long ogs_oob_assembly();
unsigned long long ogs_oob_krylov();
unsigned long long ogs_oob_mixed();
unsigned long long ogs_oob_ilu();

extern "C" ogs_status ogs_gpu_debug_oob(int64_t* site, int64_t* index)
{
    if (!site || !index) { set_error("debug_oob: NULL argument"); return OGS_BAD_ARG; }
#ifdef OGS_BOUNDS_CHECK
    OGS_CUDA_TRY(cudaDeviceSynchronize());
    unsigned long long w = ogs::oob_take();
    for (unsigned long long v : {ogs_oob_assembly(), ogs_oob_krylov(), ogs_oob_mixed(), ogs_oob_ilu()})
        w = std::min(w, v);
    if (w == ~0ull)
    {
        *site = 0;
        *index = 0;
    }
    else
    {
        *site = (int64_t)(w >> 40);
        *index = (int64_t)(w & 0xffffffffffull);
    }
#else
    *site = -1;  // not a bounds-checked build
    *index = 0;
#endif
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_debug_fp32_product(ogs_system* s, const float* x, float* y_rows, float* y_lines)
{
    if (!s || !x || !y_rows || !y_lines) { set_error("debug_fp32_product: NULL argument"); return OGS_BAD_ARG; }
    if (s->fmt != 0 || !s->U || !lattice_lines(s->m->host_up_off))
    {
        set_error("debug_fp32_product: no FP32 operator of a 27-point or 9-point lattice (solve with "
                  "OGS_PRECISION_FP32_REFINED on a hex or quad lattice first)");
        return OGS_BAD_ARG;
    }
    MixedArgs a = s->mp_args;
    a.lines = lattice_lines(s->m->host_up_off);
    const size_t bytes = (size_t)s->n * sizeof(float);
    float* d = nullptr;
    OGS_CUDA_TRY(cudaMalloc(&d, 2 * bytes));
    // r32 is the product's padded input; the next solve rebuilds it
    cudaError_t e = cudaMemcpyAsync(s->r32, x, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
    {
        launch_mp_product_pair(a, d, d + s->n, s->stream);
        count_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(y_rows, d, bytes, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(y_lines, d + s->n, bytes, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess)
    {
        set_error("debug_fp32_product: %s", cudaGetErrorString(e));
        return OGS_CUDA_ERROR;
    }
    return OGS_OK;
}
