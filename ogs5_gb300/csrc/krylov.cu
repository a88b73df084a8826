// krylov.cu -- CSR SpMV, fused vector updates and the device-resident
// CG / BiCGStab iterations of Linear_EQS (FEM/equation_class.cpp).
//
// Each iteration is a short fixed sequence of kernels.  Every kernel that
// needs a global dot product writes per-block partial sums; the last block
// to finish (atomic ticket) adds them in block order -- deterministic for a
// fixed launch shape -- and updates the solver scalars in KState: step
// lengths, the convergence test |r|/|b| < tol, breakdown tests and the
// iteration counter.  After `done` is set every later kernel returns at
// once, so the host can replay a captured chunk of iterations (CUDA graph)
// and poll a single flag between chunks: no host round trip per iteration.
#include <algorithm>
#include <cfloat>

#include "krylov.cuh"

namespace ogs {

// ------------------------------------------------------------------
// reductions
// ------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void warp_sum(double* v)
{
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// Block-reduces v[NV]; thread 0 stores the block partials; returns true in
// every thread of the last block to arrive, with the grid totals in v.
template <int NV>
__device__ __forceinline__ bool grid_reduce(double* v, double* part, unsigned int* ticket)
{
    __shared__ double sm[NV][kThreads / 32];
    __shared__ bool last;
    warp_sum<NV>(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sm[k][wid] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
    {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; k++)
        {
            double s = 0.0;
            for (int w = 0; w < nw; w++) s += sm[k][w];
            part[k * kMaxBlocks + blockIdx.x] = s;
        }
        __threadfence();
        const unsigned int t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; k++)
    {
        double s = 0.0;
        for (int bidx = threadIdx.x; bidx < (int)gridDim.x; bidx += blockDim.x)
            s += *((volatile double*)&part[k * kMaxBlocks + bidx]);
        v[k] = s;
    }
    warp_sum<NV>(v);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sm[k][wid] = v[k];
    __syncthreads();
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
    {
        double s = 0.0;
        for (int w = 0; w < nw; w++) s += sm[k][w];
        v[k] = s;
    }
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// ------------------------------------------------------------------
// SpMV: G lanes per row, lane-strided partial sums, shuffle within the group
// ------------------------------------------------------------------
template <int G>
__device__ __forceinline__ double row_dot(const int32_t* __restrict__ rp,
                                          const int32_t* __restrict__ col,
                                          const double* __restrict__ val,
                                          const double* __restrict__ x, int row, int lane,
                                          bool valid)
{
    const int beg = valid ? __ldg(rp + row) : 0, end = valid ? __ldg(rp + row + 1) : 0;
    double s = 0.0;
    for (int k = beg + lane; k < end; k += G) s += __ldcs(val + k) * __ldg(x + __ldcs(col + k));
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
    return s;
}

__device__ __forceinline__ double apply_jacobi(const SolveArgs& a, int i, double r)
{
    return a.precond == OGS_PRECOND_JACOBI ? r * a.v.dinv[i] : r;
}

// Jacobi reciprocal diagonal: CSparseMatrix::Precond_Jacobi uses
// s_i / a_ii with a_ii -> 1 when |a_ii| < DBL_MIN (matrix_class.cpp:1813)
__global__ void k_dinv(const double* __restrict__ val, const int32_t* __restrict__ diag_pos,
                       double* __restrict__ dinv, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        double d = diag_pos[i] >= 0 ? val[diag_pos[i]] : 0.0;
        if (fabs(d) < DBL_MIN) d = 1.0;
        dinv[i] = 1.0 / d;
    }
}

// y = A x (ogs_gpu_spmv, CSparseMatrix::multiVec)
template <int G>
__global__ void __launch_bounds__(kThreads) k_spmv(CsrView<double> A, const double* __restrict__ x,
                                                   double* __restrict__ y)
{
    const int lane = threadIdx.x & (G - 1);
    const int rows_per_block = blockDim.x / G;
    const int sub = (threadIdx.x & 31) / G;              // row slot within the warp
    const int wrow = (threadIdx.x >> 5) * (32 / G);      // warp's first row in the block
    for (int base = blockIdx.x * rows_per_block + wrow; base < A.n;
         base += gridDim.x * rows_per_block)
    {
        const int row = base + sub;
        const bool valid = row < A.n;
        const double s = row_dot<G>(A.row_ptr, A.col, A.val, x, row, lane, valid);
        if (valid && lane == 0) y[row] = s;
    }
}

// |b| and Linear_EQS::CheckNormRHS (equation_class.cpp:1104-1121)
__global__ void __launch_bounds__(kThreads) k_norm_b(SolveArgs a)
{
    KState* st = a.st;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
        v[0] += a.v.b[i] * a.v.b[i];
    if (grid_reduce<1>(v, st->part[0], &st->ticket[0]) && threadIdx.x == 0)
    {
        const double nb = sqrt(v[0]);
        if (!isfinite(nb)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->bnorm > 0.0 && (nb / st->bnorm) < st->tol)
        {
            st->error = nb / st->bnorm;
            st->bnorm = nb;
            st->done = 1;
            st->status = OGS_OK;
            return;
        }
        st->bnorm = nb;
        if (st->bnorm < DBL_MIN) { st->error = 0.0; st->done = 1; st->status = OGS_OK; }
    }
}

// r = b - A x; CG: z = M^-1 r, p = z, dots r.r, r.z;  BiCGStab: r0 = r,
// v = p = 0, dots r.r
template <int G>
__global__ void __launch_bounds__(kThreads) k_init_residual(SolveArgs a, int kind)
{
    KState* st = a.st;
    if (st->done) return;
    const int lane = threadIdx.x & (G - 1);
    const int rows_per_block = blockDim.x / G;
    const int sub = (threadIdx.x & 31) / G;              // row slot within the warp
    const int wrow = (threadIdx.x >> 5) * (32 / G);      // warp's first row in the block
    double v[2] = {0.0, 0.0};
    for (int base = blockIdx.x * rows_per_block + wrow; base < a.A.n;
         base += gridDim.x * rows_per_block)
    {
        const int row = base + sub;
        const bool valid = row < a.A.n;
        const double ax = row_dot<G>(a.A.row_ptr, a.A.col, a.A.val, a.v.x, row, lane, valid);
        if (valid && lane == 0)
        {
            const double r = a.v.b[row] - ax;
            a.v.r[row] = r;
            if (kind == SK_CG)
            {
                const double z = apply_jacobi(a, row, r);
                a.v.p[row] = z;
                v[1] += r * z;
            }
            else
            {
                a.v.r0[row] = r;
                a.v.v[row] = 0.0;
                a.v.p[row] = 0.0;
            }
            v[0] += r * r;
        }
    }
    if (grid_reduce<2>(v, st->part[1], &st->ticket[1]) && threadIdx.x == 0)
    {
        st->error = sqrt(v[0]) / st->bnorm;
        st->iter = 0;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->status = OGS_OK; st->done = 1; return; }
        if (st->max_iter < 1) { st->status = OGS_NOT_CONVERGED; st->done = 1; return; }
        st->iter = 1;
        if (kind == SK_CG)
            st->rr = v[1];
        else
        {
            st->rho1 = v[0];  // r0 . r with r0 = r
            if (fabs(st->rho1) < DBL_MIN) { st->status = OGS_BREAKDOWN; st->done = 1; }
        }
    }
}

// ------------------------------------------------------------------
// CG (Linear_EQS::CG, equation_class.cpp:1129-1187)
// ------------------------------------------------------------------
// s = A p ; alpha = rr / (p . s)
template <int G>
__global__ void __launch_bounds__(kThreads) k_cg_spmv(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const int lane = threadIdx.x & (G - 1);
    const int rows_per_block = blockDim.x / G;
    const int sub = (threadIdx.x & 31) / G;              // row slot within the warp
    const int wrow = (threadIdx.x >> 5) * (32 / G);      // warp's first row in the block
    double v[1] = {0.0};
    for (int base = blockIdx.x * rows_per_block + wrow; base < a.A.n;
         base += gridDim.x * rows_per_block)
    {
        const int row = base + sub;
        const bool valid = row < a.A.n;
        const double s = row_dot<G>(a.A.row_ptr, a.A.col, a.A.val, a.v.p, row, lane, valid);
        if (valid && lane == 0)
        {
            a.v.s[row] = s;
            v[0] += a.v.p[row] * s;
        }
    }
    if (grid_reduce<1>(v, st->part[2], &st->ticket[2]) && threadIdx.x == 0)
        st->alpha = st->rr / v[0];
}

// x += alpha p ; r -= alpha s ; convergence test ; z = M^-1 r ; beta
__global__ void __launch_bounds__(kThreads) k_cg_update(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const double alpha = st->alpha;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
    {
        a.v.x[i] += alpha * a.v.p[i];
        const double r = a.v.r[i] - alpha * a.v.s[i];
        a.v.r[i] = r;
        const double z = apply_jacobi(a, i, r);
        v[0] += r * r;
        v[1] += z * r;
    }
    if (grid_reduce<2>(v, st->part[3], &st->ticket[3]) && threadIdx.x == 0)
    {
        st->error = sqrt(v[0]) / st->bnorm;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->status = OGS_OK; st->done = 1; return; }
        if (st->iter >= st->max_iter) { st->status = OGS_NOT_CONVERGED; st->done = 1; return; }
        const double rrM1 = st->rr;
        st->rr = v[1];
        st->beta = st->rr / rrM1;
        st->iter += 1;
    }
}

// p = z + beta p
__global__ void __launch_bounds__(kThreads) k_cg_p(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const double beta = st->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
        a.v.p[i] = apply_jacobi(a, i, a.v.r[i]) + beta * a.v.p[i];
}

// ------------------------------------------------------------------
// BiCGStab (Linear_EQS::BiCGStab, equation_class.cpp:1287-1420)
// ------------------------------------------------------------------
// p = r (first) or r + beta (p - omega v) ; p_h = M^-1 p
__global__ void __launch_bounds__(kThreads) k_bi_p(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const bool first = st->iter == 1;
    const double beta = st->beta, omega = st->omega;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
    {
        const double p = first ? a.v.r[i] : a.v.r[i] + beta * (a.v.p[i] - omega * a.v.v[i]);
        a.v.p[i] = p;
        a.v.ph[i] = apply_jacobi(a, i, p);
    }
}

// v = A p_h ; alpha = rho1 / (r0 . v)
template <int G>
__global__ void __launch_bounds__(kThreads) k_bi_v(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const int lane = threadIdx.x & (G - 1);
    const int rows_per_block = blockDim.x / G;
    const int sub = (threadIdx.x & 31) / G;              // row slot within the warp
    const int wrow = (threadIdx.x >> 5) * (32 / G);      // warp's first row in the block
    double v[1] = {0.0};
    for (int base = blockIdx.x * rows_per_block + wrow; base < a.A.n;
         base += gridDim.x * rows_per_block)
    {
        const int row = base + sub;
        const bool valid = row < a.A.n;
        const double s = row_dot<G>(a.A.row_ptr, a.A.col, a.A.val, a.v.ph, row, lane, valid);
        if (valid && lane == 0)
        {
            a.v.v[row] = s;
            v[0] += a.v.r0[row] * s;
        }
    }
    if (grid_reduce<1>(v, st->part[4], &st->ticket[4]) && threadIdx.x == 0)
        st->alpha = st->rho1 / v[0];
}

// s = r - alpha v ; |s| test ; s_h = M^-1 s
__global__ void __launch_bounds__(kThreads) k_bi_s(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const double alpha = st->alpha;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
    {
        const double s = a.v.r[i] - alpha * a.v.v[i];
        a.v.s[i] = s;
        a.v.sh[i] = apply_jacobi(a, i, s);
        v[0] += s * s;
    }
    if (grid_reduce<1>(v, st->part[5], &st->ticket[5]) && threadIdx.x == 0)
    {
        st->error = sqrt(v[0]) / st->bnorm;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->finish_s = 1; st->status = OGS_OK; st->done = 1; }
    }
}

// t = A s_h ; omega = (t . s) / (t . t), or 1 when t . t <= DBL_MIN
template <int G>
__global__ void __launch_bounds__(kThreads) k_bi_t(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const int lane = threadIdx.x & (G - 1);
    const int rows_per_block = blockDim.x / G;
    const int sub = (threadIdx.x & 31) / G;              // row slot within the warp
    const int wrow = (threadIdx.x >> 5) * (32 / G);      // warp's first row in the block
    double v[2] = {0.0, 0.0};
    for (int base = blockIdx.x * rows_per_block + wrow; base < a.A.n;
         base += gridDim.x * rows_per_block)
    {
        const int row = base + sub;
        const bool valid = row < a.A.n;
        const double t = row_dot<G>(a.A.row_ptr, a.A.col, a.A.val, a.v.sh, row, lane, valid);
        if (valid && lane == 0)
        {
            a.v.t[row] = t;
            v[0] += t * t;
            v[1] += t * a.v.s[row];
        }
    }
    if (grid_reduce<2>(v, st->part[6], &st->ticket[6]) && threadIdx.x == 0)
        st->omega = v[0] > DBL_MIN ? v[1] / v[0] : 1.0;
}

// x += alpha p_h + omega s_h ; r = s - omega t ; tests ; next rho, beta
__global__ void __launch_bounds__(kThreads) k_bi_x(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const double alpha = st->alpha, omega = st->omega;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
    {
        a.v.x[i] += alpha * a.v.ph[i] + omega * a.v.sh[i];
        const double r = a.v.s[i] - omega * a.v.t[i];
        a.v.r[i] = r;
        v[0] += r * r;
        v[1] += a.v.r0[i] * r;
    }
    if (grid_reduce<2>(v, st->part[7], &st->ticket[7]) && threadIdx.x == 0)
    {
        st->rho0 = st->rho1;
        st->error = sqrt(v[0]) / st->bnorm;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->status = OGS_OK; st->done = 1; return; }
        if (fabs(omega) < DBL_MIN) { st->status = OGS_BREAKDOWN; st->done = 1; return; }
        if (st->iter >= st->max_iter) { st->status = OGS_NOT_CONVERGED; st->done = 1; return; }
        st->rho1 = v[1];
        if (fabs(st->rho1) < DBL_MIN) { st->status = OGS_BREAKDOWN; st->done = 1; return; }
        st->beta = (st->rho1 / st->rho0) * (alpha / omega);
        st->iter += 1;
    }
}

// early exit at the s-test: x += alpha p_h
__global__ void k_bi_finish(SolveArgs a)
{
    const double alpha = a.st->alpha;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
        a.v.x[i] += alpha * a.v.ph[i];
}

// ------------------------------------------------------------------
// host side launchers
// ------------------------------------------------------------------
int vec_grid(int n)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int need = (n + kThreads - 1) / kThreads;
    return std::max(1, std::min(need, std::min(sms * 8, kMaxBlocks)));
}

int row_group(double avg_nnz)
{
    if (avg_nnz >= 20.0) return 4;
    if (avg_nnz >= 6.0) return 2;
    return 1;
}

static int spmv_grid(int n, int G)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int rows_per_block = kThreads / G;
    const int need = (n + rows_per_block - 1) / rows_per_block;
    return std::max(1, std::min(need, std::min(sms * 8, kMaxBlocks)));
}

#define OGS_G_DISPATCH(G, KERNEL, GRID, ...)                                               \
    do                                                                                     \
    {                                                                                      \
        if (G == 4) KERNEL<4><<<GRID, kThreads, 0, s>>>(__VA_ARGS__);                      \
        else if (G == 2) KERNEL<2><<<GRID, kThreads, 0, s>>>(__VA_ARGS__);                 \
        else if (G == 8) KERNEL<8><<<GRID, kThreads, 0, s>>>(__VA_ARGS__);                 \
        else KERNEL<1><<<GRID, kThreads, 0, s>>>(__VA_ARGS__);                             \
    } while (0)

void launch_spmv(const CsrView<double>& A, const double* x, double* y, int G, cudaStream_t s)
{
    OGS_G_DISPATCH(G, k_spmv, spmv_grid(A.n, G), A, x, y);
}

void launch_dinv(const double* val, const int32_t* diag_pos, double* dinv, int n, cudaStream_t s)
{
    k_dinv<<<vec_grid(n), kThreads, 0, s>>>(val, diag_pos, dinv, n);
}

// start of a solve: |b| check and initial residual
void launch_krylov_init(const SolveArgs& a, int kind, int G, cudaStream_t s)
{
    const int vg = vec_grid(a.A.n), sg = spmv_grid(a.A.n, G);
    k_norm_b<<<vg, kThreads, 0, s>>>(a);
    OGS_G_DISPATCH(G, k_init_residual, sg, a, kind);
}

// one iteration's kernels (captured into the chunk graph)
void launch_krylov_iteration(const SolveArgs& a, int kind, int G, cudaStream_t s)
{
    const int vg = vec_grid(a.A.n), sg = spmv_grid(a.A.n, G);
    if (kind == SK_CG)
    {
        OGS_G_DISPATCH(G, k_cg_spmv, sg, a);
        k_cg_update<<<vg, kThreads, 0, s>>>(a);
        k_cg_p<<<vg, kThreads, 0, s>>>(a);
    }
    else
    {
        k_bi_p<<<vg, kThreads, 0, s>>>(a);
        OGS_G_DISPATCH(G, k_bi_v, sg, a);
        k_bi_s<<<vg, kThreads, 0, s>>>(a);
        OGS_G_DISPATCH(G, k_bi_t, sg, a);
        k_bi_x<<<vg, kThreads, 0, s>>>(a);
    }
}

int kernels_per_iteration(int kind) { return kind == SK_CG ? 3 : 5; }

void launch_bicgstab_finish(const SolveArgs& a, cudaStream_t s)
{
    k_bi_finish<<<vec_grid(a.A.n), kThreads, 0, s>>>(a);
}

}  // namespace ogs
