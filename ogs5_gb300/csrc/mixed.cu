// mixed.cu -- FP32 inner CG inside FP64 iterative refinement.
//
// The precision extension of Linear_EQS::CG: the matrix and every inner
// sweep (SpMV, vector updates) run in FP32, which halves the bytes moved and
// uses FP32 FMAs (GB300: ~60x the FP64 rate).  The solution x, the true
// residual r = b - A x and the convergence test |r|/|b| < tol stay FP64:
//
//   r64 = b - A64 x64 ; r32 = r64 / |r64| ; u = M^-1 r32
//   repeat  (FP32 CG on A32 d = r32, Jacobi preconditioned, in the
//            Chronopoulos-Gear form: one SpMV and one grid reduction per
//            iteration)
//     S: w = A32 u ; gamma = r.u, delta = w.u, rho = r.r
//     V: beta = gamma / gamma_prev ; eta = delta - beta^2 eta_prev ;
//        alpha = gamma / eta ; p = u + beta p ; s = w + beta s ;
//        x32 += alpha p ; r32 -= alpha s ; u = M^-1 r32
//     when |r32| fell by `delta` since the last replacement, or the FP32
//     recurrence claims convergence:  x64 += |r64| x32 ; x32 = 0 ;
//     r64 = b - A64 x64 (FP64) ; replace r32 by r64 / |r64|, rescale p, s
//   until |r64| / |b| < tol
//
// The FP64 residual replacement (a reliable-update form of iterative
// refinement) keeps the FP32 Krylov space instead of restarting it, so the
// iteration count stays close to FP64 CG.  Convergence is only ever
// declared on the FP64 residual.  Dot products accumulate FP32 per thread
// and FP64 across threads and blocks.
//
// FP32 operator storage: for patterns with at most 64 distinct column
// offsets (structured grids) the symmetric matrix is stored as the upper
// half of its diagonal-offset form, U[d][i] = A[i][i + off_d] for off_d >= 0
// (14 rows of 4 bytes per node for hexes: the config-2 matrix is 61 MB and
// stays in L2 with the FP32 vectors); y_i = sum_d U[d][i] x_{i+off_d} +
// sum_{d>0} U[d][i-off_d] x_{i-off_d}.  Other patterns use SELL-32 with
// FP32 values.
#include <algorithm>
#include <cfloat>

#include "krylov.cuh"

namespace ogs {


// ------------------------------------------------------------------
// FP32 operator
// ------------------------------------------------------------------
// Diagonal-offset row with the number of stored offsets known at compile
// time.  All 2*NU-1 (value, x) pairs of the row are loaded into registers
// before any FMA, so a warp keeps ~50 independent loads in flight (the
// kernel is latency-bound otherwise); out-of-range neighbours are
// predicated off.  Summation order: diagonal, then per offset the upper and
// the mirrored lower entry.
//
// X_NC: x is read through the non-coherent read-only path (__ldg), valid
// only when x does not change during the launch; the persistent kernel,
// which rewrites x between its grid barriers, reads it with plain loads.
template <bool X_NC>
__device__ __forceinline__ float ldx(const float* x, int i)
{
    if constexpr (X_NC)
        return __ldg(x + i);
    else
        return x[i];
}

template <int NU, bool X_NC = true>
__device__ __forceinline__ float dia_row(const MixedArgs& a, const float* x, int i)
{
    constexpr int K = 2 * NU - 1;
    const int n = a.n;
    float uv[K], xv[K];
    uv[0] = __ldg(a.U + i);
    xv[0] = ldx<X_NC>(x, i);
#pragma unroll
    for (int d = 1; d < NU; d++)
    {
        const int o = a.off[d];
        const float* Ud = a.U + (size_t)d * n;
        const bool up = i + o < n, lo = i - o >= 0;
        uv[2 * d - 1] = up ? __ldg(Ud + i) : 0.f;
        xv[2 * d - 1] = up ? ldx<X_NC>(x, i + o) : 0.f;
        uv[2 * d] = lo ? __ldg(Ud + i - o) : 0.f;
        xv[2 * d] = lo ? ldx<X_NC>(x, i - o) : 0.f;
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) acc += uv[k] * xv[k];
    return acc;
}

template <bool X_NC = true>
__device__ __forceinline__ float sell32_row(const MixedArgs& a, const float* x, int row)
{
    const int s = row >> 5;
    const int b0 = __ldg(a.A.slice_ptr + s), b1 = __ldg(a.A.slice_ptr + s + 1);
    const int w = (b1 - b0) >> 5;
    const int beg = b0 + (row & 31);
    float acc = 0.f;
#pragma unroll 3
    for (int j = 0; j < w; j++)
    {
        const int k = beg + (j << 5);
        acc += __ldg(a.val32 + k) * ldx<X_NC>(x, __ldg(a.A.col + k));
    }
    return acc;
}

// NU > 0: diagonal-offset operator with NU stored offsets; NU == 0: SELL-32
template <int NU, bool X_NC = true>
__device__ __forceinline__ float op_row(const MixedArgs& a, const float* x, int i)
{
    if constexpr (NU > 0)
        return dia_row<NU, X_NC>(a, x, i);
    else
        return sell32_row<X_NC>(a, x, i);
}


// U[d][i] = (float) A[i][i + off_d]; d32 = (float) (1 / a_ii)
__global__ void k_mp_convert(MixedArgs a, const int32_t* __restrict__ row_len,
                             const int8_t* __restrict__ slot_up, float* U, float* val32,
                             const double* __restrict__ dinv64, float* d32)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        d32[i] = (float)dinv64[i];
        const int beg = a.A.slice_ptr[i >> 5] + (i & 31);
        const int len = row_len[i];
        for (int j = 0; j < len; j++)
        {
            const int k = beg + (j << 5);
            if (a.fmt == 0)
            {
                const int d = slot_up[k];
                if (d >= 0) U[(size_t)d * a.n + i] = (float)a.A.val[k];
            }
            else
                val32[k] = (float)a.A.val[k];
        }
    }
}

// ------------------------------------------------------------------
// FP64 residual replacement
// ------------------------------------------------------------------
// x64 += x32 / scale ; x32 = 0
__global__ void __launch_bounds__(kThreads) k_mp_accumulate(MixedArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const double inv = 1.0 / st->scale;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        a.x[i] += (double)a.x32[i] * inv;
        a.x32[i] = 0.f;
    }
}

// a full replacement cycle that lowers |r64| by less than 4x, or a short
// one that gains less than a quarter of what the FP32 recurrence claimed,
// hands over to FP64
constexpr double kMinCycleGain = 4.0;
constexpr double kCycleSlack = 0.25;
// iterations without a new smallest FP32 residual that count as a plateau
constexpr int kPlateau = 64;

// r64 = b - A64 x64 ; |r64| ; convergence on the FP64 residual ; new scale
__global__ void __launch_bounds__(kThreads) k_mp_residual(MixedArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    double v[1] = {0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < a.n; row += gridDim.x * blockDim.x)
    {
        const int s = row >> 5;
        const int b0 = __ldg(a.A.slice_ptr + s), b1 = __ldg(a.A.slice_ptr + s + 1);
        const int w = (b1 - b0) >> 5;
        const int beg = b0 + (row & 31);
        double acc = 0.0;
        for (int j = 0; j < w; j++)
        {
            const int k = beg + (j << 5);
            acc += __ldcs(a.A.val + k) * __ldg(a.x + __ldcs(a.A.col + k));
        }
        const double r = a.b[row] - acc;
        a.r64[row] = r;
        v[0] += r * r;
    }
    double out[1];
    if (grid_sum<1, double>(v, out, st->part[0], &st->ticket[0]) && threadIdx.x == 0)
    {
        const double rn = sqrt(out[0]);
        st->error = rn / st->bnorm;
        st->replacements += 1;
        if (!isfinite(st->error)) { st->status = OGS_NONFINITE; st->done = 1; return; }
        if (st->error < st->tol) { st->status = OGS_OK; st->done = 1; return; }
        if (st->iter >= st->max_iter) { st->status = OGS_NOT_CONVERGED; st->done = 1; return; }
        // A cycle of FP32 iterations lowers the true residual about as much
        // as the FP32 recurrence claims (rmax / rn_req: 1/delta for a full
        // cycle).  When the FP32 operator is too coarse for the system's
        // conditioning (cond(A) near 1/eps_fp32) the true gain falls far
        // behind the claimed one; the solve then finishes in FP64 CG from x64.
        const double claimed = st->rn_req > 0.0 ? st->rmax / st->rn_req : 1.0;
        const double gain = st->err_prev / st->error;
        if (st->stalled || (!st->first && gain < fmin(kMinCycleGain, kCycleSlack * claimed)))
        {
            st->fallback = 1;
            st->done = 1;
            return;
        }
        st->err_prev = st->error;
        const double ns = rn > DBL_MIN ? 1.0 / rn : 1.0;
        st->ratio = st->first ? 1.0 : ns / st->scale;
        st->scale = ns;
    }
}

// r32 = scale r64 ; u = M^-1 r32 ; p32, s32 rescaled (zero at the first
// restart) ; the last iteration's gamma and eta rescaled to the new units
__global__ void __launch_bounds__(kThreads) k_mp_restart(MixedArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const double sc = st->scale;
    const float ratio = (float)st->ratio;
    const bool first = st->first != 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        const float r = (float)(a.r64[i] * sc);
        a.r32[i] = r;
        a.u32[i] = r * a.d32[i];
        a.p32[i] = first ? 0.f : a.p32[i] * ratio;
        a.s32[i] = first ? 0.f : a.s32[i] * ratio;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        // The iteration that asked for the replacement stopped before forming
        // its search direction: it is redone with the replaced residual, so
        // the counter steps back and the scalars of the iteration before it
        // are carried into the new units.
        int it = st->iter;
        if (!first) it -= 1;
        st->iter = it;
        const double r2 = st->ratio * st->ratio;
        st->gam_hist[it & 1] *= r2;
        st->eta_hist[it & 1] *= r2;
        st->base_iter = it;
        st->rmax = -1.0;  // set from the first rho after the restart
        st->replace = 0;
        st->stalled = 0;
    }
}

// ------------------------------------------------------------------
// FP32 CG iteration (Chronopoulos-Gear, ticket-free, see krylov.cuh)
// ------------------------------------------------------------------
// S: iter += 1 ; w32 = A32 u32 ; partials of r.u, w.u, r.r
template <int NU>
__global__ void __launch_bounds__(kThreads, 3) k_mp_spmv(MixedArgs a)
{
    KState* st = a.st;
    if (st->done || st->replace) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->iter += 1;  // no block of this kernel reads iter
    float v[3] = {0.f, 0.f, 0.f};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        const float w = op_row<NU>(a, a.u32, i);
        a.w32[i] = w;
        const float u = a.u32[i], r = a.r32[i];
        v[0] += r * u;
        v[1] += w * u;
        v[2] += r * r;
    }
    write_partials<3, float>(v, st->cg_ps);
}

constexpr int kU32 = 8;  // elements per thread per step, loaded before use

// V: scalars from the S partials ; replacement test ; p, s, x32, r32, u32
__global__ void __launch_bounds__(kThreads) k_mp_update(MixedArgs a)
{
    KState* st = a.st;
    if (st->done || st->replace) return;
    const int it = st->iter;
    double g[3];
    reduce_partials<3>(st->cg_ps, st->nb_spmv, g);
    const double gamma = g[0], delta = g[1], rn = sqrt(g[2]);
    const bool first = it == 1;                  // no search direction yet: beta = 0
    const bool fresh = it == st->base_iter + 1;  // first iteration after a (re)start
    const double rmax = fresh ? rn : st->rmax;
    const double beta = first ? 0.0 : gamma / st->gam_hist[(it - 1) & 1];
    const double eta = first ? delta : delta - beta * beta * st->eta_hist[(it - 1) & 1];
    const double alpha = gamma / eta;
    const double est = rn / st->scale / st->bnorm;  // estimate of |r64| / |b|
    const bool nonfinite = !isfinite(rn) || !isfinite(alpha);
    // plateau: no new smallest |r32| in the cycle for max(64, half the
    // cycle) iterations (parity slots of the previous iteration: written by
    // block 0 of the previous launch)
    const double rb_prev = fresh ? rn : ((it - 1) & 1 ? st->rbest[1] : st->rbest[0]);
    const int ib_prev = fresh ? it : ((it - 1) & 1 ? st->itbest[1] : st->itbest[0]);
    const bool better = rn < rb_prev;
    const double rb = better ? rn : rb_prev;
    const int ib = better ? it : ib_prev;
    const bool stalled = it - ib > max(kPlateau, (it - st->base_iter) / 2);
    // right after a replacement r32 is the true residual (checked in FP64 by
    // k_mp_residual), so a fresh iteration never asks for another one
    const bool repl = !nonfinite && !fresh &&
                      (est < st->tol || rn < st->delta * rmax || it > st->max_iter || stalled);
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        if (it & 1) { st->rbest[1] = rb; st->itbest[1] = ib; }
        else { st->rbest[0] = rb; st->itbest[0] = ib; }
        if (fresh) st->rmax = rn;
        st->gam_hist[it & 1] = gamma;
        st->eta_hist[it & 1] = eta;
        st->first = 0;  // read by the replacement kernels only
        if (nonfinite) { st->status = OGS_NONFINITE; st->done = 1; }
        else if (repl)
        {
            st->replace = 1;
            st->rn_req = rn;
            st->stalled = stalled && !(est < st->tol || rn < st->delta * rmax || it > st->max_iter);
        }
    }
    if (nonfinite || repl) return;
    const float fb = (float)beta, fa = (float)alpha;
    const int n = a.n, stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x; base < n; base += kU32 * stride)
    {
        float uv[kU32], wv[kU32], pv[kU32], sv[kU32], xv[kU32], rv[kU32], dv[kU32];
#pragma unroll
        for (int k = 0; k < kU32; k++)
        {
            const int i = base + k * stride;
            const bool in = i < n;
            uv[k] = in ? a.u32[i] : 0.f;
            wv[k] = in ? a.w32[i] : 0.f;
            pv[k] = in ? a.p32[i] : 0.f;
            sv[k] = in ? a.s32[i] : 0.f;
            xv[k] = in ? a.x32[i] : 0.f;
            rv[k] = in ? a.r32[i] : 0.f;
            dv[k] = in ? a.d32[i] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < kU32; k++)
        {
            const int i = base + k * stride;
            if (i < n)
            {
                const float p = uv[k] + fb * pv[k];
                const float s = wv[k] + fb * sv[k];
                const float r = rv[k] - fa * s;
                a.p32[i] = p;
                a.s32[i] = s;
                a.x32[i] = xv[k] + fa * p;
                a.r32[i] = r;
                a.u32[i] = r * dv[k];
            }
        }
    }
}

// ------------------------------------------------------------------
// Persistent FP32 CG: the S and V steps of many iterations in one
// cooperative launch (all blocks resident), two grid barriers per
// iteration -- after the partial sums and after the vector update, whose u
// the next product reads at neighbouring rows.  Every block adds the
// partials itself in the same order, so all hold the same scalars and take
// the same branch; block 0 publishes the state the replacement kernels and
// the host read.  A thread owns the rows gtid + k * stride in both steps,
// so w is read back by the thread that wrote it.
// ------------------------------------------------------------------
constexpr unsigned kBarSpinLimit = 1u << 24;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// false in every thread of the block once any block gave up waiting
__device__ bool mp_grid_barrier(KState* st)
{
    __shared__ int s_go;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int go = 1;
        const unsigned gen = ld_acquire(&st->bar_gen);
        __threadfence();
        if (atomicAdd(&st->bar_count, 1u) + 1u == gridDim.x)
        {
            st->bar_count = 0u;
            __threadfence();
            st_release(&st->bar_gen, gen + 1u);
        }
        else
        {
            unsigned spins = 0;
            while (ld_acquire(&st->bar_gen) == gen)
            {
                if (++spins > kBarSpinLimit || *(volatile int*)&st->bar_err)
                {
                    atomicExch(&st->bar_err, 1);
                    go = 0;
                    break;
                }
                if (spins > 64) __nanosleep(32);
            }
        }
        __threadfence();
        s_go = go;
    }
    __syncthreads();
    return s_go != 0;
}

template <int NU>
__global__ void __launch_bounds__(kThreads) k_mp_persist(MixedArgs a, int iters)
{
    KState* st = a.st;
    // launch-time state: nothing writes it before every block has passed the
    // first barrier, which comes after these reads
    if (st->done || st->replace) return;
    const int it0 = st->iter, base_iter = st->base_iter, max_iter = st->max_iter;
    const double scale = st->scale, bnorm = st->bnorm, tol = st->tol, dlt = st->delta;
    double rmax = st->rmax;
    double gam_prev = st->gam_hist[it0 & 1], eta_prev = st->eta_hist[it0 & 1];
    double rb_prev = (it0 & 1) ? st->rbest[1] : st->rbest[0];
    int ib_prev = (it0 & 1) ? st->itbest[1] : st->itbest[0];
    const int n = a.n, stride = gridDim.x * blockDim.x, gtid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int t = 0; t < iters; t++)
    {
        const int it = it0 + t + 1;
        // S: w32 = A32 u32 ; partials of r.u, w.u, r.r
        float v[3] = {0.f, 0.f, 0.f};
        for (int i = gtid; i < n; i += stride)
        {
            const float w = op_row<NU, false>(a, a.u32, i);
            a.w32[i] = w;
            const float u = a.u32[i], r = a.r32[i];
            v[0] += r * u;
            v[1] += w * u;
            v[2] += r * r;
        }
        write_partials<3, float>(v, st->cg_ps);
        if (!mp_grid_barrier(st)) break;
        double g[3];
        reduce_partials<3>(st->cg_ps, gridDim.x, g);
        // V: the scalars of k_mp_update from this block's copies
        const double gamma = g[0], delta = g[1], rn = sqrt(g[2]);
        const bool first = it == 1;
        const bool fresh = it == base_iter + 1;
        if (fresh) rmax = rn;
        const double beta = first ? 0.0 : gamma / gam_prev;
        const double eta = first ? delta : delta - beta * beta * eta_prev;
        const double alpha = gamma / eta;
        const double est = rn / scale / bnorm;
        const bool nonfinite = !isfinite(rn) || !isfinite(alpha);
        const double rbp = fresh ? rn : rb_prev;
        const int ibp = fresh ? it : ib_prev;
        const bool better = rn < rbp;
        const double rb = better ? rn : rbp;
        const int ib = better ? it : ibp;
        const bool stalled = it - ib > max(kPlateau, (it - base_iter) / 2);
        const bool repl = !nonfinite && !fresh && (est < tol || rn < dlt * rmax || it > max_iter || stalled);
        if (blockIdx.x == 0 && threadIdx.x == 0)
        {
            st->iter = it;
            if (it & 1) { st->rbest[1] = rb; st->itbest[1] = ib; }
            else { st->rbest[0] = rb; st->itbest[0] = ib; }
            if (fresh) st->rmax = rn;
            st->gam_hist[it & 1] = gamma;
            st->eta_hist[it & 1] = eta;
            st->first = 0;
            if (nonfinite) { st->status = OGS_NONFINITE; st->done = 1; }
            else if (repl)
            {
                st->replace = 1;
                st->rn_req = rn;
                st->stalled = stalled && !(est < tol || rn < dlt * rmax || it > max_iter);
            }
        }
        if (nonfinite || repl) break;
        gam_prev = gamma;
        eta_prev = eta;
        rb_prev = rb;
        ib_prev = ib;
        const float fb = (float)beta, fa = (float)alpha;
        for (int base = gtid; base < n; base += kU32 * stride)
        {
            float uv[kU32], wv[kU32], pv[kU32], sv[kU32], xv[kU32], rv[kU32], dv[kU32];
#pragma unroll
            for (int k = 0; k < kU32; k++)
            {
                const int i = base + k * stride;
                const bool in = i < n;
                uv[k] = in ? a.u32[i] : 0.f;
                wv[k] = in ? a.w32[i] : 0.f;
                pv[k] = in ? a.p32[i] : 0.f;
                sv[k] = in ? a.s32[i] : 0.f;
                xv[k] = in ? a.x32[i] : 0.f;
                rv[k] = in ? a.r32[i] : 0.f;
                dv[k] = in ? a.d32[i] : 0.f;
            }
#pragma unroll
            for (int k = 0; k < kU32; k++)
            {
                const int i = base + k * stride;
                if (i < n)
                {
                    const float p = uv[k] + fb * pv[k];
                    const float s = wv[k] + fb * sv[k];
                    const float r = rv[k] - fa * s;
                    a.p32[i] = p;
                    a.s32[i] = s;
                    a.x32[i] = xv[k] + fa * p;
                    a.r32[i] = r;
                    a.u32[i] = r * dv[k];
                }
            }
        }
        if (!mp_grid_barrier(st)) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && *(volatile int*)&st->bar_err)
    {
        st->status = OGS_CUDA_ERROR;
        st->done = 1;
    }
}

// ------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------
int vec_grid(int n);

void launch_mp_convert(const MixedArgs& a, const int32_t* row_len, const int8_t* slot_up, float* U,
                       float* val32, const double* dinv64, float* d32, cudaStream_t s)
{
    k_mp_convert<<<vec_grid(a.n), kThreads, 0, s>>>(a, row_len, slot_up, U, val32, dinv64, d32);
}

int red_grid(int n);

// grids of the FP32 CG kernels (the update/p kernels add this many SpMV
// partials, the p kernel this many update partials)
int mp_spmv_grid(int n)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // three blocks of the register-heavy diagonal kernel are resident per SM
    return std::max(1, std::min((n + kThreads - 1) / kThreads, std::min(sms * 3, kMaxBlocks)));
}

// FP64 residual replacement: accumulate, residual, restart
void launch_mp_replace(const MixedArgs& a, cudaStream_t s)
{
    const int g = vec_grid(a.n);
    k_mp_accumulate<<<g, kThreads, 0, s>>>(a);
    k_mp_residual<<<g, kThreads, 0, s>>>(a);
    k_mp_restart<<<g, kThreads, 0, s>>>(a);
}

// resident blocks of the persistent kernel for the operator format (0 when
// the device cannot launch it cooperatively)
template <int NU>
static int persist_grid_for(int n)
{
    int dev = 0, sms = 152, coop = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mp_persist<NU>, kThreads, 0) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    const int need = (n + kThreads - 1) / kThreads;
    return std::max(1, std::min(need, std::min(per_sm * sms, kMaxBlocks)));
}

int mp_persist_grid(const MixedArgs& a)
{
    switch (a.fmt == 0 ? a.n_up : 0)
    {
        case 14: return persist_grid_for<14>(a.n);
        case 8: return persist_grid_for<8>(a.n);
        case 5: return persist_grid_for<5>(a.n);
        default: return persist_grid_for<0>(a.n);
    }
}

// up to `iters` FP32 iterations in one cooperative launch of `grid` blocks
cudaError_t launch_mp_persist(const MixedArgs& a, int grid, int iters, cudaStream_t s)
{
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(kThreads);
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    switch (a.fmt == 0 ? a.n_up : 0)
    {
        case 14: return cudaLaunchKernelEx(&lc, k_mp_persist<14>, a, iters);
        case 8: return cudaLaunchKernelEx(&lc, k_mp_persist<8>, a, iters);
        case 5: return cudaLaunchKernelEx(&lc, k_mp_persist<5>, a, iters);
        default: return cudaLaunchKernelEx(&lc, k_mp_persist<0>, a, iters);
    }
}

void launch_mp_iteration(const MixedArgs& a, cudaStream_t s, cudaEvent_t eb, cudaEvent_t ee)
{
    const int gs = mp_spmv_grid(a.n), gr = red_grid(a.n);
    if (eb) cudaEventRecordWithFlags(eb, s, cudaEventRecordExternal);
    switch (a.fmt == 0 ? a.n_up : 0)
    {
        case 14: k_mp_spmv<14><<<gs, kThreads, 0, s>>>(a); break;  // hex, 27-point
        case 8: k_mp_spmv<8><<<gs, kThreads, 0, s>>>(a); break;    // Kuhn tets, 15-point
        case 5: k_mp_spmv<5><<<gs, kThreads, 0, s>>>(a); break;    // quads, 9-point
        default: k_mp_spmv<0><<<gs, kThreads, 0, s>>>(a); break;   // SELL-32 FP32
    }
    if (ee) cudaEventRecordWithFlags(ee, s, cudaEventRecordExternal);
    k_mp_update<<<gr, kThreads, 0, s>>>(a);
}

}  // namespace ogs
