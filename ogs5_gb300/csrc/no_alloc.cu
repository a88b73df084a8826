// no_alloc.cu -- Jacobi-preconditioned CG that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a process whose device memory is
// owned by a caching allocator or memory pool that has already reserved
// the HBM (a solve server, a PyTorch process) gets an out-of-memory error,
// or an allocation that fragments the pool, for every buffer a solver asks
// for.  For them ogs_gpu_csr_cg_noalloc solves A x = b on a CSR matrix they
// own, with the Krylov vectors (r, p, s and the Jacobi inverse), the solver
// scalars and the reduction partials in the file-scope array below.
//
//  * The array holds OGS_NOALLOC_MAX_ROWS rows worth of vectors (4 x 8 B per
//    row, 16 MiB, plus 256 KiB of reduction partials); every GPU that loads
//    this library holds it until the process exits.
//  * Host code cannot use the array's name as a device address, so the
//    first call on each device (with that device current) looks the address
//    up with cudaGetSymbolAddress and caches it.  Make that first call
//    before any stream capture.  The cached address is not looked up again:
//    cudaDeviceReset after the first call on a device is not supported (the
//    module may be loaded again at another address).
//  * All calls share the array and it keeps the last call's contents: each
//    call clears the counters and flags that must start at zero.  Calls
//    whose work overlaps on the GPU (different streams, or threads) race on
//    the array and must be serialised by the caller.
//
// The iteration is Linear_EQS::CG (FEM/equation_class.cpp:1129-1187) with
// CSparseMatrix::Precond_Jacobi; one thread per CSR row sums its entries in
// ascending column order.
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <mutex>

#include "krylov.cuh"

namespace ogs {

namespace {

constexpr int kNaBlocks = 1024;  // grid cap of these kernels (reduction partial slots)

struct NaState
{
    double bnorm, tol, error, rr, alpha, beta;
    int iter, max_iter, done, status;
    unsigned int ticket[4];
};

// layout of the scratch array, in doubles
constexpr size_t kNaHeader = 64;                       // NaState, rounded up
constexpr size_t kNaPart = 8 * (size_t)kMaxBlocks;    // 4 kernels x 2 sums, grid_sum stride
constexpr size_t kNaVectors = 4 * (size_t)OGS_NOALLOC_MAX_ROWS;
static_assert(sizeof(NaState) <= kNaHeader * sizeof(double), "header too small");

}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[kNaHeader + kNaPart + kNaVectors];

namespace {

struct NaArgs
{
    int n;
    const int32_t* rp;
    const int32_t* col;
    const double* val;
    const double* b;
    double* x;
    NaState* st;
    double* part;  // [4 kernels][2 sums][kMaxBlocks] (grid_sum layout)
    double *r, *p, *s, *dinv;
};

__device__ __forceinline__ double csr_row(const NaArgs& a, const double* __restrict__ v, int i)
{
    double acc = 0.0;
    for (int k = a.rp[i]; k < a.rp[i + 1]; k++) acc += a.val[k] * v[a.col[k]];
    return acc;
}

// Jacobi inverse and |b| with Linear_EQS::CheckNormRHS for a fresh system
__global__ void __launch_bounds__(kThreads) k_na_init(NaArgs a)
{
    NaState* st = a.st;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        double d = 0.0;
        for (int k = a.rp[i]; k < a.rp[i + 1]; k++)
            if (a.col[k] == i) d = a.val[k];
        if (fabs(d) < DBL_MIN) d = 1.0;
        a.dinv[i] = 1.0 / d;
        v[0] += a.b[i] * a.b[i];
    }
    double out[1];
    if (grid_sum<1, double>(v, out, a.part, &st->ticket[0]) && threadIdx.x == 0)
    {
        const double nb = sqrt(out[0]);
        if (!isfinite(nb)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        // a fresh Linear_EQS has bNorm = 1
        if (nb / 1.0 < st->tol) { st->error = nb; st->bnorm = nb; st->done = 1; return; }
        st->bnorm = nb;
        if (nb < DBL_MIN) { st->error = 0.0; st->done = 1; }
    }
}

// r = b - A x ; p = M^-1 r ; |r| test ; rr = r . M^-1 r
__global__ void __launch_bounds__(kThreads) k_na_residual(NaArgs a)
{
    NaState* st = a.st;
    if (st->done) return;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        const double r = a.b[i] - csr_row(a, a.x, i);
        const double z = r * a.dinv[i];
        a.r[i] = r;
        a.p[i] = z;
        v[0] += r * r;
        v[1] += r * z;
    }
    double out[2];
    if (grid_sum<2, double>(v, out, a.part + 2 * kMaxBlocks, &st->ticket[1]) && threadIdx.x == 0)
    {
        st->error = sqrt(out[0]) / st->bnorm;
        st->iter = 0;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->done = 1; return; }
        if (st->max_iter < 1) { st->status = OGS_NOT_CONVERGED; st->done = 1; return; }
        st->iter = 1;
        st->rr = out[1];
    }
}

// s = A p ; alpha = rr / (p . s)
__global__ void __launch_bounds__(kThreads) k_na_spmv(NaArgs a)
{
    NaState* st = a.st;
    if (st->done) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        const double s = csr_row(a, a.p, i);
        a.s[i] = s;
        v[0] += a.p[i] * s;
    }
    double out[1];
    if (grid_sum<1, double>(v, out, a.part + 4 * kMaxBlocks, &st->ticket[2]) && threadIdx.x == 0)
        st->alpha = st->rr / out[0];
}

// x += alpha p ; r -= alpha s ; |r| test ; beta
__global__ void __launch_bounds__(kThreads) k_na_update(NaArgs a)
{
    NaState* st = a.st;
    if (st->done) return;
    const double alpha = st->alpha;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        a.x[i] += alpha * a.p[i];
        const double r = a.r[i] - alpha * a.s[i];
        a.r[i] = r;
        v[0] += r * r;
        v[1] += (r * a.dinv[i]) * r;
    }
    double out[2];
    if (grid_sum<2, double>(v, out, a.part + 6 * kMaxBlocks, &st->ticket[3]) && threadIdx.x == 0)
    {
        st->error = sqrt(out[0]) / st->bnorm;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->done = 1; return; }
        if (st->iter >= st->max_iter) { st->status = OGS_NOT_CONVERGED; st->done = 1; return; }
        const double rrM1 = st->rr;
        st->rr = out[1];
        st->beta = st->rr / rrM1;
        st->iter += 1;
    }
}

// p = M^-1 r + beta p
__global__ void __launch_bounds__(kThreads) k_na_p(NaArgs a)
{
    NaState* st = a.st;
    if (st->done) return;
    const double beta = st->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
        a.p[i] = a.r[i] * a.dinv[i] + beta * a.p[i];
}

// per-device address of g_noalloc_scratch, looked up on first use
std::mutex g_na_mutex;
constexpr int kNaMaxDevices = 64;
double* g_na_addr[kNaMaxDevices] = {};

ogs_status scratch_address(double** out)
{
    int dev = 0;
    OGS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices) { set_error("csr_cg_noalloc: device %d out of range", dev); return OGS_BAD_ARG; }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev])
    {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
        {
            set_error("csr_cg_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return OGS_CUDA_ERROR;
        }
        g_na_addr[dev] = (double*)p;
    }
    *out = g_na_addr[dev];
    return OGS_OK;
}

}  // namespace
}  // namespace ogs

using namespace ogs;

extern "C" ogs_status ogs_gpu_csr_cg_noalloc(int64_t n, const int32_t* row_ptr, const int32_t* col,
                                             const double* val, const double* b, double* x,
                                             int32_t max_iter, double tol, void* stream,
                                             ogs_solve_stats* stats)
{
    if (n <= 0 || !row_ptr || !col || !val || !b || !x || max_iter < 0 || !(tol >= 0.0))
    {
        set_error("csr_cg_noalloc: bad arguments");
        return OGS_BAD_ARG;
    }
    if (n > OGS_NOALLOC_MAX_ROWS)
    {
        set_error("csr_cg_noalloc: %lld rows exceed the static scratch of %d rows", (long long)n,
                  (int)OGS_NOALLOC_MAX_ROWS);
        return OGS_BAD_ARG;
    }
    const void* arrays[] = {row_ptr, col, val, b, x};
    for (const void* p : arrays)
    {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
            (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged))
        {
            cudaGetLastError();
            set_error("csr_cg_noalloc: every array must be device memory");
            return OGS_BAD_ARG;
        }
    }
    double* base = nullptr;
    ogs_status st = scratch_address(&base);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    NaArgs a;
    a.n = (int)n;
    a.rp = row_ptr;
    a.col = col;
    a.val = val;
    a.b = b;
    a.x = x;
    a.st = (NaState*)base;
    a.part = base + kNaHeader;
    double* vec = base + kNaHeader + kNaPart;
    a.r = vec;
    a.p = vec + OGS_NOALLOC_MAX_ROWS;
    a.s = vec + 2 * (size_t)OGS_NOALLOC_MAX_ROWS;
    a.dinv = vec + 3 * (size_t)OGS_NOALLOC_MAX_ROWS;
    // the scratch keeps the previous call's contents: reset the state
    NaState h;
    std::memset(&h, 0, sizeof h);
    h.tol = tol;
    h.max_iter = max_iter;
    h.error = 1.0e10;
    OGS_CUDA_TRY(cudaMemcpyAsync(a.st, &h, sizeof h, cudaMemcpyHostToDevice, s));
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int g = std::max(1, std::min<int>((int)((n + kThreads - 1) / kThreads), std::min(sms * 4, kNaBlocks)));
    k_na_init<<<g, kThreads, 0, s>>>(a);
    k_na_residual<<<g, kThreads, 0, s>>>(a);
    OGS_LAUNCH_CHECK();
    count_launches(1);
    constexpr int kChunk = 16;
    for (int done_iters = 0;;)
    {
        OGS_CUDA_TRY(cudaMemcpyAsync(&h, a.st, sizeof h, cudaMemcpyDeviceToHost, s));
        OGS_CUDA_TRY(cudaStreamSynchronize(s));
        if (h.done || (int64_t)done_iters > (int64_t)max_iter + kChunk) break;
        for (int k = 0; k < kChunk; k++)
        {
            k_na_spmv<<<g, kThreads, 0, s>>>(a);
            k_na_update<<<g, kThreads, 0, s>>>(a);
            k_na_p<<<g, kThreads, 0, s>>>(a);
        }
        OGS_LAUNCH_CHECK();
        count_launches(3 * kChunk - 1);
        done_iters += kChunk;
    }
    if (!h.done) { set_error("csr_cg_noalloc: solver state did not finish"); return OGS_CUDA_ERROR; }
    if (stats)
    {
        std::memset(stats, 0, sizeof *stats);
        stats->iterations = h.iter;
        stats->status = h.status;
        stats->rel_residual = h.error;
        stats->b_norm = h.bnorm;
    }
    return (ogs_status)h.status;
}
