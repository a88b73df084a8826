// krylov.cu -- SELL-32 SpMV, fused vector updates and the device-resident
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
//
// GB300 issues about two FP64 FMAs per clock per SM, so the SpMV is written
// to spend exactly one DFMA per stored entry: one thread per row, SELL-32
// slices read warp-coalesced with streaming (evict-first) loads, the row
// sum accumulated in ascending column order like CSparseMatrix::multiVec,
// no shuffle reductions.  Vector kernels load four elements per thread
// before computing to keep enough bytes in flight.
#include <algorithm>
#include <cfloat>

#include "krylov.cuh"

namespace ogs {

// ------------------------------------------------------------------
// reductions
// ------------------------------------------------------------------
// grid_reduce: FP64 grid sum (krylov.cuh grid_sum) with the totals
// broadcast back into v for the calling thread 0
template <int NV>
__device__ __forceinline__ bool grid_reduce(double* v, double* part, unsigned int* ticket)
{
    double out[NV];
    if (!grid_sum<NV, double>(v, out, part, ticket)) return false;
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = out[k];
    return true;
}

// ------------------------------------------------------------------
// SELL-32 row product: entries of row r sit at slice_ptr[r/32] + 32 j + r%32
// ------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ double sell_row(const SellView<T>& A, const double* __restrict__ x,
                                           int row)
{
    const int s = row >> 5;
    const int b0 = __ldg(A.slice_ptr + s), b1 = __ldg(A.slice_ptr + s + 1);
    const int w = (b1 - b0) >> 5;
    const int beg = b0 + (row & 31);
    double acc = 0.0;
#pragma unroll 3
    for (int j = 0; j < w; j++)
    {
        const int k = beg + (j << 5);
        const int c = __ldcs(A.col + k);
        if (OGS_IN(c, A.n, kOobSpmvCol)) acc += (double)__ldcs(A.val + k) * __ldg(x + c);
    }
    return acc;
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
__global__ void __launch_bounds__(kThreads) k_spmv(SellView<double> A, const double* __restrict__ x,
                                                   double* __restrict__ y)
{
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x)
        y[row] = sell_row(A, x, row);
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
__global__ void __launch_bounds__(kThreads) k_init_residual(SolveArgs a, int kind)
{
    KState* st = a.st;
    if (st->done) return;
    double v[2] = {0.0, 0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < a.A.n; row += gridDim.x * blockDim.x)
    {
        const double r = a.v.b[row] - sell_row(a.A, a.v.x, row);
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
    if (grid_reduce<2>(v, st->part[1], &st->ticket[1]) && threadIdx.x == 0)
    {
        st->error = sqrt(v[0]) / st->bnorm;
        st->iter = 0;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->status = OGS_OK; st->done = 1; return; }
        if (st->max_iter < 1) { st->status = OGS_NOT_CONVERGED; st->done = 1; return; }
        if (kind == SK_CG)
        {
            // CG: the SpMV kernel advances iter; r.z of iteration 0
            st->rz_base = v[1];
            st->base_iter = 0;
        }
        else
        {
            st->iter = 1;
            st->rho1 = v[0];  // r0 . r with r0 = r
            if (fabs(st->rho1) < DBL_MIN) { st->status = OGS_BREAKDOWN; st->done = 1; }
        }
    }
}

// ------------------------------------------------------------------
// CG (Linear_EQS::CG, equation_class.cpp:1129-1187), ticket-free:
//   k_cg_spmv   iter += 1 (block 0) ; s = A p ; partials of p . s
//   k_cg_update alpha = rz_prev / (p . s) ; x += alpha p ; r -= alpha s ;
//               partials of r . r and r . M^-1 r (parity buffer iter & 1)
//   k_cg_p      |r| / |b| test, max_iter ; beta = rz / rz_prev ; p = z + beta p
// ------------------------------------------------------------------
// r . z of the previous iteration: the base value right after a (re)start,
// else the other parity buffer
__device__ __forceinline__ double cg_rz_prev(const KState* st, int it)
{
    return it == st->base_iter + 1 ? st->rz_base : st->rz_hist[(it - 1) & 1];
}

// s = A p ; partials of p . s
__global__ void __launch_bounds__(kThreads) k_cg_spmv(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->iter += 1;  // no block of this kernel reads iter
    double v[1] = {0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < a.A.n; row += gridDim.x * blockDim.x)
    {
        const double s = sell_row(a.A, a.v.p, row);
        a.v.s[row] = s;
        v[0] += a.v.p[row] * s;
    }
    write_partials<1, double>(v, st->cg_ps);
}

constexpr int kU = 4;  // elements per thread per step in the vector kernels

// x += alpha p ; r -= alpha s ; partials of r . r and z . r (PC: 0 none,
// 1 Jacobi, 2 ILU(0) -- z comes from the sweeps, k_cg_dots_z writes the partials)
template <int PC>
__global__ void __launch_bounds__(kThreads) k_cg_update(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const int it = st->iter;
    double ps[1];
    reduce_partials_bcast<1>(st->cg_ps, st->nb_spmv, ps);
    const double alpha = cg_rz_prev(st, it) / ps[0];
    const int n = a.A.n;
    double v[2] = {0.0, 0.0};
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x; base < n; base += kU * stride)
    {
        double xv[kU], pv[kU], rv[kU], sv[kU], dv[kU];
#pragma unroll
        for (int u = 0; u < kU; u++)
        {
            const int i = base + u * stride;
            if (i < n)
            {
                xv[u] = a.v.x[i];
                pv[u] = a.v.p[i];
                rv[u] = a.v.r[i];
                sv[u] = a.v.s[i];
                dv[u] = PC == 1 ? a.v.dinv[i] : 1.0;
            }
        }
#pragma unroll
        for (int u = 0; u < kU; u++)
        {
            const int i = base + u * stride;
            if (i < n)
            {
                a.v.x[i] = xv[u] + alpha * pv[u];
                const double r = rv[u] - alpha * sv[u];
                a.v.r[i] = r;
                v[0] += r * r;
                v[1] += PC == 1 ? (r * dv[u]) * r : r * r;
            }
        }
    }
    if (PC != 2) write_partials<2, double>(v, st->cg_upd[it & 1]);
}

// convergence test ; beta ; p = z + beta p (z = dinv r, r, or the ILU(0)
// sweep result in ph)
template <int PC>
__global__ void __launch_bounds__(kThreads) k_cg_p(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const int it = st->iter;
    double rr_rz[2];
    reduce_partials_bcast<2>(st->cg_upd[it & 1], st->nb_upd, rr_rz);
    const double rz_prev = cg_rz_prev(st, it);
    const double error = sqrt(rr_rz[0]) / st->bnorm;
    int stop = -1;
    if (!isfinite(error)) stop = OGS_NONFINITE;
    else if (error < st->tol) stop = OGS_OK;
    else if (it >= st->max_iter) stop = OGS_NOT_CONVERGED;
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        st->error = error;              // read by the host only
        st->rz_hist[it & 1] = rr_rz[1];  // read from iteration it + 1 on
        if (stop >= 0) { st->status = stop; st->done = 1; }
    }
    if (stop >= 0) return;
    const double beta = rr_rz[1] / rz_prev;
    const int n = a.A.n;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x; base < n; base += kU * stride)
    {
        double rv[kU], dv[kU], pv[kU];
#pragma unroll
        for (int u = 0; u < kU; u++)
        {
            const int i = base + u * stride;
            if (i < n)
            {
                rv[u] = PC == 2 ? a.v.ph[i] : a.v.r[i];
                dv[u] = PC == 1 ? a.v.dinv[i] : 1.0;
                pv[u] = a.v.p[i];
            }
        }
#pragma unroll
        for (int u = 0; u < kU; u++)
        {
            const int i = base + u * stride;
            if (i < n) a.v.p[i] = (PC == 1 ? rv[u] * dv[u] : rv[u]) + beta * pv[u];
        }
    }
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
__global__ void __launch_bounds__(kThreads) k_bi_v(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    double v[1] = {0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < a.A.n; row += gridDim.x * blockDim.x)
    {
        const double s = sell_row(a.A, a.v.ph, row);
        a.v.v[row] = s;
        v[0] += a.v.r0[row] * s;
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
__global__ void __launch_bounds__(kThreads) k_bi_t(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    double v[2] = {0.0, 0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < a.A.n; row += gridDim.x * blockDim.x)
    {
        const double t = sell_row(a.A, a.v.sh, row);
        a.v.t[row] = t;
        v[0] += t * t;
        v[1] += t * a.v.s[row];
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
static int sm_count()
{
    static int sms = 0;
    if (!sms)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    return sms;
}

int vec_grid(int n)
{
    const int need = (n + kThreads - 1) / kThreads;
    return std::max(1, std::min(need, std::min(sm_count() * 8, kMaxBlocks)));
}

// Grid of the reducing vector kernels: two blocks per SM, so each thread
// handles a dozen or more elements and the FP64 adds of the block
// reduction stay a small fraction of the FP64 work.
int red_grid(int n)
{
    const int need = (n + kThreads - 1) / kThreads;
    return std::max(1, std::min(need, std::min(sm_count() * 2, kMaxBlocks)));
}

void launch_spmv(const SellView<double>& A, const double* x, double* y, cudaStream_t s)
{
    k_spmv<<<vec_grid(A.n), kThreads, 0, s>>>(A, x, y);
}

void launch_dinv(const double* val, const int32_t* diag_pos, double* dinv, int n, cudaStream_t s)
{
    k_dinv<<<vec_grid(n), kThreads, 0, s>>>(val, diag_pos, dinv, n);
}

void launch_norm_b(const SolveArgs& a, cudaStream_t s)
{
    k_norm_b<<<vec_grid(a.A.n), kThreads, 0, s>>>(a);
}

void launch_ilu_apply(const IluView& f, const double* in, double* out, const KState* st, cudaStream_t s);
void launch_cg_dots_z(const SolveArgs& a, int grid, cudaStream_t s);
void launch_cg_init_z(const SolveArgs& a, int grid, cudaStream_t s);

// start of a solve: |b| check and initial residual (ILU(0) CG: then
// z = M^-1 r, p = z, r . z)
void launch_krylov_init(const SolveArgs& a, int kind, cudaStream_t s)
{
    const int vg = vec_grid(a.A.n);
    k_norm_b<<<vg, kThreads, 0, s>>>(a);
    k_init_residual<<<vg, kThreads, 0, s>>>(a, kind);
    if (kind == SK_CG && a.precond == OGS_PRECOND_ILU0)
    {
        launch_ilu_apply(a.ilu, a.v.r, a.v.ph, a.st, s);
        launch_cg_init_z(a, vg, s);
    }
}

int krylov_init_launches(int kind, int precond)
{
    return kind == SK_CG && precond == OGS_PRECOND_ILU0 ? 5 : 2;
}

// one iteration's kernels (captured into the chunk graph); eb/ee, when
// given, are recorded around the iteration's first SpMV
void launch_krylov_iteration(const SolveArgs& a, int kind, cudaStream_t s, cudaEvent_t eb, cudaEvent_t ee)
{
    const int vg = vec_grid(a.A.n), rg = red_grid(a.A.n);
    const bool ilu = a.precond == OGS_PRECOND_ILU0;
    if (kind == SK_CG)
    {
        if (eb) cudaEventRecordWithFlags(eb, s, cudaEventRecordExternal);
        k_cg_spmv<<<vg, kThreads, 0, s>>>(a);
        if (ee) cudaEventRecordWithFlags(ee, s, cudaEventRecordExternal);
        if (a.precond == OGS_PRECOND_JACOBI)
        {
            k_cg_update<1><<<rg, kThreads, 0, s>>>(a);
            k_cg_p<1><<<rg, kThreads, 0, s>>>(a);
        }
        else if (ilu)
        {
            k_cg_update<2><<<rg, kThreads, 0, s>>>(a);
            launch_ilu_apply(a.ilu, a.v.r, a.v.ph, a.st, s);
            launch_cg_dots_z(a, rg, s);  // same grid as the update: k_cg_p adds nb_upd partials
            k_cg_p<2><<<rg, kThreads, 0, s>>>(a);
        }
        else
        {
            k_cg_update<0><<<rg, kThreads, 0, s>>>(a);
            k_cg_p<0><<<rg, kThreads, 0, s>>>(a);
        }
    }
    else
    {
        k_bi_p<<<vg, kThreads, 0, s>>>(a);
        if (ilu) launch_ilu_apply(a.ilu, a.v.p, a.v.ph, a.st, s);
        if (eb) cudaEventRecordWithFlags(eb, s, cudaEventRecordExternal);
        k_bi_v<<<vg, kThreads, 0, s>>>(a);
        if (ee) cudaEventRecordWithFlags(ee, s, cudaEventRecordExternal);
        k_bi_s<<<rg, kThreads, 0, s>>>(a);
        if (ilu) launch_ilu_apply(a.ilu, a.v.s, a.v.sh, a.st, s);
        k_bi_t<<<vg, kThreads, 0, s>>>(a);
        k_bi_x<<<rg, kThreads, 0, s>>>(a);
    }
}

int kernels_per_iteration(int kind, int precond)
{
    const bool ilu = precond == OGS_PRECOND_ILU0;
    return kind == SK_CG ? (ilu ? 6 : 3) : (ilu ? 9 : 5);
}

void launch_bicgstab_finish(const SolveArgs& a, cudaStream_t s)
{
    k_bi_finish<<<vec_grid(a.A.n), kThreads, 0, s>>>(a);
}

}  // namespace ogs

unsigned long long ogs_oob_krylov() { return ogs::oob_take(); }
