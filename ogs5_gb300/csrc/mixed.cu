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
// Jacobi scaling: with the diagonal S = D^-1/2 stored operators hold
// S A S (unit diagonal) and the inner CG runs unpreconditioned on it with
// r32 = S r64 scaled to unit norm; u = M^-1 r of the form above becomes r
// itself, so an iteration reads neither u nor d (the same iterates in
// exact arithmetic: S^-1 p, S^-1 x are the preconditioned directions).
// S is kept in FP32 (d32) and used as rounded everywhere.
// The cell-coefficient operator and the persistent kernel keep the
// preconditioned form.
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
// (14 rows of 4 bytes per node for hexes: the 129 x 129 x 65 lattice's matrix is 61 MB and
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

template <int NU, bool X_NC = true, bool UNIT = false>
__device__ __forceinline__ float dia_row(const MixedArgs& a, const float* x, int i)
{
    constexpr int K = 2 * NU - 1;
    const int n = a.n;
    float uv[K], xv[K];
    uv[0] = UNIT ? 1.f : __ldg(a.U + i);
    xv[0] = ldx<X_NC>(x, i);
#pragma unroll
    for (int d = 1; d < NU; d++)
    {
        const int o = a.off[d];
        const float* Ud = a.U + (size_t)d * a.ustride;
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
        const int c = __ldg(a.A.col + k);
        if (OGS_IN(c, a.n, kOobMixedCol)) acc += __ldg(a.val32 + k) * ldx<X_NC>(x, c);
    }
    return acc;
}

// NU > 0: diagonal-offset operator with NU stored offsets; NU == 0: SELL-32
// Operator from cell coefficients on a regular hex lattice (fmt 2): row i
// of sum_c (alpha_c L_box + beta M_box) over the up to eight cells around
// node i, with the eliminated columns of the Dirichlet set dropped and the
// Dirichlet rows reduced to their kept diagonal.  L_box and M_box entries
// depend only on which corner coordinates of the two nodes agree (three
// bits), so the 64 corner pairs read two 8-entry tables.  Per row: 27
// values of x, 27 mask bytes and up to 8 coefficients instead of 27
// stored matrix values.
template <bool X_NC>
__device__ __forceinline__ float mf_row(const MixedArgs& a, const float* x, int i)
{
    const unsigned char mk = __ldg(a.mf_mask + i);
    if (mk & 1) return __ldg(a.mf_dbc + i) * ldx<X_NC>(x, i);
    const int nx = a.gx, ny = a.gy;
    const int ix = i % nx, t = i / nx, iy = t % ny, iz = t / ny;
    const bool vx0 = ix > 0, vx1 = ix < nx - 1, vy0 = iy > 0, vy1 = iy < ny - 1, vz0 = iz > 0,
               vz1 = iz < a.gz - 1;
    float xv[27];
#pragma unroll
    for (int dz = -1; dz <= 1; dz++)
#pragma unroll
        for (int dy = -1; dy <= 1; dy++)
#pragma unroll
            for (int dx = -1; dx <= 1; dx++)
            {
                const bool in = (dx < 0 ? vx0 : dx > 0 ? vx1 : true) && (dy < 0 ? vy0 : dy > 0 ? vy1 : true) &&
                                (dz < 0 ? vz0 : dz > 0 ? vz1 : true);
                const int j = i + dx + nx * (dy + ny * dz);
                const float v = in ? ldx<X_NC>(x, j) : 0.f;
                const int mk = in ? (int)__ldg(a.mf_mask + j) : 2;
                xv[(dx + 1) + 3 * ((dy + 1) + 3 * (dz + 1))] = (mk & 2) ? 0.f : v;
            }
    const int ncx = nx - 1, ncy = ny - 1;
    float accL = 0.f, accM = 0.f;
#pragma unroll
    for (int ez = 0; ez < 2; ez++)
#pragma unroll
        for (int ey = 0; ey < 2; ey++)
#pragma unroll
            for (int ex = 0; ex < 2; ex++)
            {
                // the cell with corner (ix - 1 + ex, iy - 1 + ey, iz - 1 + ez);
                // node i is its corner (1 - ex, 1 - ey, 1 - ez)
                if (!((ex ? vx1 : vx0) && (ey ? vy1 : vy0) && (ez ? vz1 : vz0))) continue;
                const int c = (ix - 1 + ex) + ncx * ((iy - 1 + ey) + ncy * (iz - 1 + ez));
                float sL = 0.f, sM = 0.f;
#pragma unroll
                for (int bz = 0; bz < 2; bz++)
#pragma unroll
                    for (int by = 0; by < 2; by++)
#pragma unroll
                        for (int bx = 0; bx < 2; bx++)
                        {
                            const int pat = ((1 - ex) == bx ? 1 : 0) | ((1 - ey) == by ? 2 : 0) | ((1 - ez) == bz ? 4 : 0);
                            const float xb = xv[(ex + bx) + 3 * ((ey + by) + 3 * (ez + bz))];
                            sL += a.mf_L[pat] * xb;
                            sM += a.mf_M[pat] * xb;
                        }
                accL += __ldg(a.mf_alpha + c) * sL;
                accM += sM;
            }
    return accL + __ldg(a.mf_beta) * accM;
}

// NU > 0: diagonal-offset operator with NU stored offsets; NU == 0: SELL-32;
// NU == -1: cell coefficients of a regular hex lattice.  UNIT: the
// diagonal-offset operator of the Jacobi-scaled system, whose diagonal is
// 1 and is not read (a row whose a_ii was not positive is then off by its
// diagonal: the inner solve stops gaining and the solve ends in FP64 CG)
template <int NU, bool X_NC = true, bool UNIT = false>
__device__ __forceinline__ float op_row(const MixedArgs& a, const float* x, int i)
{
    if constexpr (NU > 0)
        return dia_row<NU, X_NC, UNIT>(a, x, i);
    else if constexpr (NU == 0)
        return sell32_row<X_NC>(a, x, i);
    else
        return mf_row<X_NC>(a, x, i);
}


// S = D^-1/2 of the Jacobi scaling: 1 / sqrt(a_ii), 1 where the Jacobi
// inverse is not positive (CG needs a positive diagonal anyway)
__device__ __forceinline__ double jacobi_scale(double dinv)
{
    return dinv > 0.0 ? sqrt(dinv) : 1.0;
}

// d32: the FP32 Jacobi inverse (preconditioned form) or the FP32 scale
// s_i (scaled form; the operator, the restart and the accumulation all use
// these rounded values, so the transformation is exactly S A S for them)
__global__ void k_mp_scale(MixedArgs a, const double* __restrict__ dinv64, float* d32)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
        d32[i] = (float)(a.scaled ? jacobi_scale(dinv64[i]) : dinv64[i]);
}

// U[d][i] = (float) A[i][i + off_d] (times s_i s_j when scaled)
__global__ void k_mp_convert(MixedArgs a, const int32_t* __restrict__ row_len,
                             const int8_t* __restrict__ slot_up, float* U, float* val32, const float* __restrict__ d32)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        const double si = a.scaled ? (double)d32[i] : 1.0;
        const int beg = a.A.slice_ptr[i >> 5] + (i & 31);
        const int len = row_len[i];
        for (int j = 0; j < len; j++)
        {
            const int k = beg + (j << 5);
            // the diagonal-offset form stores the upper half only: the lower
            // entries' FP64 products (GB300's scarce FP64) and scale loads
            // are skipped
            const int d = a.fmt == 0 ? (int)slot_up[k] : 0;
            if (d < 0) continue;
            const double v = a.scaled ? a.A.val[k] * si * (double)d32[a.A.col[k]] : a.A.val[k];
            if (a.fmt == 0)
                U[(size_t)d * a.ustride + i] = (float)v;
            else
                val32[k] = (float)v;
        }
    }
}

// fmt 2: FP32 cell coefficients, the Dirichlet mask and kept diagonals,
// and the Jacobi inverse
__global__ void k_mp_convert_cells(const double* __restrict__ coef, int64_t cells, float* alpha32, float* beta32)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x)
        alpha32[c] = (float)coef[c];
    if (blockIdx.x == 0 && threadIdx.x == 0) *beta32 = (float)coef[cells];
}

// mask from the Dirichlet set: SYMMETRIC (row flags) eliminates rows and
// columns, ROW_ONLY (row list) only rows
__global__ void k_mp_mask_symmetric(const unsigned char* __restrict__ flag, unsigned char* mask, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mask[i] = flag[i] ? 3 : 0;
}

__global__ void k_mp_mask_rows(const int32_t* __restrict__ rows, int nbc, unsigned char* mask)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nbc; q += gridDim.x * blockDim.x) mask[rows[q]] = 1;
}

__global__ void k_mp_dbc(MixedArgs a, const int32_t* __restrict__ diag_pos, const double* __restrict__ dinv64,
                         float* d32, float* dbc)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        d32[i] = (float)dinv64[i];
        const int dp = diag_pos[i];
        dbc[i] = (a.mf_mask[i] & 1) && dp >= 0 ? (float)a.A.val[dp] : 0.f;
    }
}

// Check of an FP32 operator against the FP64 matrix on a fixed test vector
// v (in w32): out[0] = max |y32 - y64|, out[1] = max sum_j |a_ij v_j|, as
// float bits (non-negative floats order like their bits)
__device__ __forceinline__ float test_vector(int i)
{
    unsigned h = (unsigned)i * 2654435761u;
    h ^= h >> 15;
    return 0.5f + (float)(h & 0xffffu) * (1.0f / 65536.0f);
}

__global__ void k_mp_check_fill(float* v, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = test_vector(i);
}

template <int NU>
__global__ void k_mp_check(MixedArgs a, unsigned* out)
{
    float dmax = 0.f, smax = 0.f;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < a.n; row += gridDim.x * blockDim.x)
    {
        const float y32 = op_row<NU>(a, a.w32, row);
        const int s = row >> 5;
        const int b0 = a.A.slice_ptr[s], b1 = a.A.slice_ptr[s + 1];
        const int beg = b0 + (row & 31);
        double y = 0.0, sa = 0.0;
        for (int j = 0; j < (b1 - b0) >> 5; j++)
        {
            const int k = beg + (j << 5);
            const double t = a.A.val[k] * (double)a.w32[a.A.col[k]];
            y += t;
            sa += fabs(t);
        }
        dmax = fmaxf(dmax, (float)fabs((double)y32 - y));
        smax = fmaxf(smax, (float)sa);
    }
    atomicMax(out, __float_as_uint(dmax));
    atomicMax(out + 1, __float_as_uint(smax));
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
        const double si = a.scaled ? (double)a.d32[i] : 1.0;  // x = S x_scaled
        a.x[i] += (double)a.x32[i] * inv * si;
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
    double v[2] = {0.0, 0.0};  // |r64|^2 ; |S r64|^2 (scaled form)
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
        if (a.scaled)
        {
            const double q = r * (double)a.d32[row];
            v[1] += q * q;
        }
    }
    double out[2];
    if (grid_sum<2, double>(v, out, st->part[0], &st->ticket[0]) && threadIdx.x == 0)
    {
        const double rn = sqrt(out[0]);
        const double rc = a.scaled ? sqrt(out[1]) : rn;  // |r64| in the units of the inner CG
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
        const double ec = rc / st->bnorm;
        const double gain = st->err_prev / ec;
        if (st->stalled || (!st->first && gain < fmin(kMinCycleGain, kCycleSlack * claimed)))
        {
            st->fallback = 1;
            st->done = 1;
            return;
        }
        st->err_prev = ec;
        st->est_unit = st->error;  // scaled form: r32 starts at unit norm
        const double ns = rc > DBL_MIN ? 1.0 / rc : 1.0;
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
        if (a.scaled)
            a.r32[i] = (float)(a.r64[i] * (double)a.d32[i] * sc);
        else
        {
            const float r = (float)(a.r64[i] * sc);
            a.r32[i] = r;
            a.u32[i] = r * a.d32[i];
        }
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
// FP32 CG iteration (Chronopoulos-Gear)
// ------------------------------------------------------------------
// r.u, w.u, r.r of the product: block partials, added by the update
// kernel's blocks
__device__ __forceinline__ void mp_sum_products(const float (&v)[3], KState* st)
{
    write_partials<3, float>(v, st->cg_ps);
}

// V scalars: beta = gamma / gamma_prev ; eta = delta - beta^2 eta_prev ;
// alpha = gamma / eta ; the replacement test.  Called by warp 0 of every
// update block: one warp adds the product partials in FP64 (the same fixed
// order in every block, so all blocks hold bitwise the same scalars), lane
// 0 does the scalar work and, when `record`, writes the iteration's state.
// Lane 0 returns stop (non-finite or a replacement is due), alpha, beta.
__device__ __forceinline__ void mp_iteration_scalars(const MixedArgs& a, bool record, int& stop, double& alpha_out,
                                                     double& beta_out)

{
    KState* st = a.st;
    // lane 0 loads the state it needs (both parity slots, and the flags that
    // end the iteration) before the partial sums, so the loads overlap
    // instead of following each other
    int it = 0, base = 0, max_iter = 0, ibs[2] = {0, 0}, ended = 0;
    double gh[2] = {0.0, 0.0}, eh[2] = {0.0, 0.0}, rbs[2] = {0.0, 0.0};
    double rmax_prev = 0.0, scale = 1.0, bnorm = 1.0, tol = 0.0, dl = 0.0, eu = 0.0;
    if (threadIdx.x == 0)
    {
        it = st->iter; base = st->base_iter; max_iter = st->max_iter;
        gh[0] = st->gam_hist[0]; gh[1] = st->gam_hist[1];
        eh[0] = st->eta_hist[0]; eh[1] = st->eta_hist[1];
        rbs[0] = st->rbest[0]; rbs[1] = st->rbest[1];
        ibs[0] = st->itbest[0]; ibs[1] = st->itbest[1];
        rmax_prev = st->rmax; scale = st->scale; bnorm = st->bnorm; tol = st->tol; dl = st->delta;
        eu = st->est_unit;
        ended = st->done | st->replace;
    }
    double g[3];
    if (!reduce_partials_warp<3>(st->cg_ps, a.nb_spmv, g) || threadIdx.x != 0) return;
    if (ended)
    {
        stop = 1;  // solve over or replacement pending: the product did not run
        return;
    }
    const int pp = (it - 1) & 1;                 // parity slot of the previous iteration
    const double gamma = g[0], delta = g[1], rn = sqrt(g[2]);
    const bool first = it == 1;                  // no search direction yet: beta = 0
    const bool fresh = it == base + 1;           // first iteration after a (re)start
    const double rmax = fresh ? rn : rmax_prev;
    const double beta = first ? 0.0 : gamma / (pp ? gh[1] : gh[0]);
    const double eta = first ? delta : delta - beta * beta * (pp ? eh[1] : eh[0]);
    const double alpha = gamma / eta;
    const double est = a.scaled ? rn * eu : rn / scale / bnorm;  // estimate of |r64| / |b|
    const bool nonfinite = !isfinite(rn) || !isfinite(alpha);
    // plateau: no new smallest |r32| in the cycle for max(64, half the
    // cycle) iterations
    const double rb_prev = fresh ? rn : (pp ? rbs[1] : rbs[0]);
    const int ib_prev = fresh ? it : (pp ? ibs[1] : ibs[0]);
    const bool better = rn < rb_prev;
    const double rb = better ? rn : rb_prev;
    const int ib = better ? it : ib_prev;
    const bool stalled = it - ib > max(kPlateau, (it - base) / 2);
    // right after a replacement r32 is the true residual (checked in FP64 by
    // k_mp_residual), so a fresh iteration never asks for another one
    const bool repl = !nonfinite && !fresh && (est < tol || rn < dl * rmax || it > max_iter || stalled);
    stop = nonfinite || repl;
    alpha_out = alpha;
    beta_out = beta;
    if (!record) return;
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
        st->stalled = stalled && !(est < tol || rn < dl * rmax || it > max_iter);
    }
}

// S: iter += 1 ; w32 = A32 u32 ; partials of r.u, w.u, r.r
template <int NU, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, 3) k_mp_spmv(MixedArgs a)
{
    KState* st = a.st;
    if (st->done || st->replace) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->iter += 1;  // no block of this kernel reads iter
    float v[3] = {0.f, 0.f, 0.f};
    const float* xin = a.scaled ? a.r32 : a.u32;  // scaled form: u = r
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
    {
        const float w = op_row<NU, true, UNIT>(a, xin, i);
        a.w32[i] = w;
        const float u = xin[i], r = a.r32[i];
        v[0] += r * u;
        v[1] += w * u;
        v[2] += r * r;
    }
    mp_sum_products(v, st);
}

// ------------------------------------------------------------------
// The Jacobi-scaled 27-point lattice product, four rows per thread
// ------------------------------------------------------------------
// When the 13 upper offsets are those of a lattice numbered line by line
// (1 ; nx - 1, nx, nx + 1 ; nxy - nx - 1 .. nxy - nx + 1 ; nxy - 1 ..
// nxy + 1 ; nxy + nx - 1 .. nxy + nx + 1, nx nodes per line and nxy per
// plane), the 27 columns of a row form nine lines of three consecutive
// nodes, and rows 4g .. 4g + 3 need six consecutive x of each line.  A
// thread then reads every operand as aligned 16-byte words: its own
// operator values U[d][4g .. 4g + 3] (13 words), each line's six x (two or
// three words) and each mirrored window U[d][4g - off_d ..] (one or two
// words) -- 55 to 62 wide loads for four rows by the windows' alignments
// (57 for nx = nxy = 1 mod 4), instead of 53 four-byte loads with bounds
// predicates per row.  The word alignment of every window depends
// only on nx mod 4 and nxy mod 4 (template arguments RX, RXY).  There are
// no bounds predicates: the operator rows and the FP32 vectors carry zero
// pads of at least nxy + nx + 16 values on both sides, so a window that
// leaves [0, n) reads zeros where the predicated form adds 0 * 0.  The
// terms are added in the order of dia_row<14, true, true> (unit diagonal,
// then per offset the upper and the mirrored lower entry), so the product
// is bit for bit that of k_mp_spmv<14, true>.
__host__ __device__ constexpr int mod4(int v) { return ((v % 4) + 4) % 4; }

// Aligned 16-byte words q[0 .. W - 1] of p from index f = 0 (mod 4).  The
// debug build checks that they lie in [-pad, hi) of their padded row or
// vector (and reads zeros otherwise).
template <int W>
__device__ __forceinline__ void words(const float* p, int f, int pad, int hi, float (&w)[4 * W])
{
    if (!OGS_IN(f + pad, hi + pad - 4 * W + 1, kOobMixedWindow))
    {
#pragma unroll
        for (int k = 0; k < 4 * W; k++) w[k] = 0.f;
        return;
    }
    const float4* q = reinterpret_cast<const float4*>(p + f);
#pragma unroll
    for (int k = 0; k < W; k++)
    {
        const float4 v = __ldg(q + k);
        w[4 * k] = v.x; w[4 * k + 1] = v.y; w[4 * k + 2] = v.z; w[4 * k + 3] = v.w;
    }
}

// p[start .. start + 3], start = T (mod 4), from aligned 16-byte words
template <int T>
__device__ __forceinline__ void window4(const float* p, int start, int pad, int hi, float (&o)[4])
{
    constexpr int W = T == 0 ? 1 : 2;
    float w[4 * W];
    words<W>(p, start - T, pad, hi, w);
#pragma unroll
    for (int k = 0; k < 4; k++) o[k] = w[T + k];
}

// p[start .. start + 5], start = S (mod 4)
template <int S>
__device__ __forceinline__ void window6(const float* p, int start, int pad, int hi, float (&o)[6])
{
    constexpr int W = S > 2 ? 3 : 2;
    float w[4 * W];
    words<W>(p, start - S, pad, hi, w);
#pragma unroll
    for (int k = 0; k < 6; k++) o[k] = w[S + k];
}

// offset off_d = B + DX of a line with base B: the upper entries
// U_d[i + m] x[i + m + B + DX] (xu = x[i + B - 1 ..]) and the mirrored lower
// entries U_d[i + m - off_d] x[i + m - off_d] (xl = x[i - B - 1 ..]); the
// lower window starts at i - off_d = T (mod 4)
template <int T, int DX>
__device__ __forceinline__ void lines_entry(const MixedArgs& a, const float* Ud, int i, int lo_start,
                                            const float (&xu)[6], const float (&xl)[6], float (&acc)[4])
{
    const int uhi = a.ustride - a.pad;  // a U row holds indices [-pad, ustride - pad)
    float uo[4], ul[4];
    words<1>(Ud, i, a.pad, uhi, uo);
    window4<T>(Ud, lo_start, a.pad, uhi, ul);
#pragma unroll
    for (int m = 0; m < 4; m++)
    {
        acc[m] = fmaf(uo[m], xu[m + 1 + DX], acc[m]);
        acc[m] = fmaf(ul[m], xl[m + 1 - DX], acc[m]);
    }
}

// the line (DY, DZ) with base B = DY nx + DZ nxy, stored offsets D0 .. D0 + 2
// (B - 1 .. B + 1), and its mirror (-DY, -DZ)
template <int RX, int RXY, int DY, int DZ, int D0>
__device__ __forceinline__ void lines_pair(const MixedArgs& a, const float* x, int i, int nx, int nxy,
                                           float (&acc)[4])
{
    constexpr int SB = mod4(DY * RX + DZ * RXY);
    const int B = DY * nx + DZ * nxy, xhi = a.n + a.pad + 64;
    float xu[6], xl[6];
    window6<mod4(SB - 1)>(x, i + B - 1, a.pad, xhi, xu);
    window6<mod4(-SB - 1)>(x, i - B - 1, a.pad, xhi, xl);
    const float* U0 = a.U + (size_t)D0 * a.ustride;
    lines_entry<mod4(1 - SB), -1>(a, U0, i, i - B + 1, xu, xl, acc);
    lines_entry<mod4(-SB), 0>(a, U0 + a.ustride, i, i - B, xu, xl, acc);
    lines_entry<mod4(-1 - SB), 1>(a, U0 + 2 * (size_t)a.ustride, i, i - B - 1, xu, xl, acc);
}

// rows i .. i + 3 (i = 0 mod 4) of S A S x; x0 receives x[i - 1 .. i + 4].
// NP line pairs: 4 for the 27-point lattice, 1 for the 9-point plane
// lattice of quads (upper offsets 1 ; nx - 1, nx, nx + 1: the same terms in
// the same order as dia_row<5, true, true>)
template <int RX, int RXY, int NP>
__device__ __forceinline__ void lines_group(const MixedArgs& a, const float* x, int i, float (&acc)[4],
                                            float (&x0)[6])
{
    const int nx = a.off[3], nxy = a.off[9];
    window6<3>(x, i - 1, a.pad, a.n + a.pad + 64, x0);
#pragma unroll
    for (int m = 0; m < 4; m++) acc[m] = 0.f + x0[m + 1];
    lines_entry<3, 1>(a, a.U + a.ustride, i, i - 1, x0, x0, acc);  // offset 1
    lines_pair<RX, RXY, 1, 0, 2>(a, x, i, nx, nxy, acc);
    if constexpr (NP == 4)
    {
        lines_pair<RX, RXY, -1, 1, 5>(a, x, i, nx, nxy, acc);
        lines_pair<RX, RXY, 0, 1, 8>(a, x, i, nx, nxy, acc);
        lines_pair<RX, RXY, 1, 1, 11>(a, x, i, nx, nxy, acc);
    }
}

// S: iter += 1 ; w32 = S A S r32 ; partials of r.r, w.r, r.r
// One block per SM (up to 255 registers: the loads of several line pairs
// in flight at once); the grid is one block per SM, so the product's
// partial sums are one per SM for the update kernel to add.
template <int RX, int RXY, int NP>
__global__ void __launch_bounds__(kThreads, 1) k_mp_spmv_lines(MixedArgs a)
{
    KState* st = a.st;
    if (st->done || st->replace) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->iter += 1;  // no block of this kernel reads iter
    const float* x = a.r32;
    const int ng = (a.n + 3) >> 2;
    float v[3] = {0.f, 0.f, 0.f};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
    {
        float acc[4], x0[6];
        lines_group<RX, RXY, NP>(a, x, 4 * g, acc, x0);
        // rows n .. 4 ng - 1 come out 0 (zero operator rows, zero r pad)
        reinterpret_cast<float4*>(a.w32)[g] = make_float4(acc[0], acc[1], acc[2], acc[3]);
#pragma unroll
        for (int m = 0; m < 4; m++)
        {
            const float r = x0[m + 1], w = acc[m];
            v[0] += r * r;
            v[1] += w * r;
            v[2] += r * r;
        }
    }
    mp_sum_products(v, st);
}

// Both forms of the product on a.r32 (instrumentation): y_rows by the row
// kernel's dia_row, y_lines by lines_group, n values each
template <int RX, int RXY, int NP>
__global__ void k_mp_product_pair(MixedArgs a, float* y_rows, float* y_lines)
{
    const int ng = (a.n + 3) >> 2;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
    {
        float acc[4], x0[6];
        lines_group<RX, RXY, NP>(a, a.r32, 4 * g, acc, x0);
#pragma unroll
        for (int m = 0; m < 4; m++)
        {
            const int i = 4 * g + m;
            if (i < a.n)
            {
                y_lines[i] = acc[m];
                y_rows[i] = dia_row<NP == 4 ? 14 : 5, true, true>(a, a.r32, i);
            }
        }
    }
}

// fmt 2 product on the lattice: blocks of 4 warps, a warp holds 32
// consecutive x-columns of one y-line and marches up kCellZ planes in z.
// x at ix +- 1 comes from the neighbouring lanes (loads at the warp edges
// only); three planes of the 3 x 3 neighbourhood and two layers of 2 x 2
// cells stay in registers, so a node costs one x, one mask byte per line
// and plane step, two cell coefficients and its r instead of the 27 + 27
// + 8 loads of mf_row.
constexpr int kCellZ = 16;
constexpr int kCellWarps = 4;

struct CellGrid
{
    int bx, by, bz;  // blocks along x (32 columns), y (kCellWarps lines), z (kCellZ planes)
};

__host__ __device__ inline CellGrid cell_grid(int nx, int ny, int nz)
{
    return {(nx + 31) / 32, (ny + kCellWarps - 1) / kCellWarps, (nz + kCellZ - 1) / kCellZ};
}

// Raw loads of one line (iy, z) of a plane: x and mask at ix, and at ix - 1
// (lane 0) / ix + 1 (lane 31) -- issued one plane step ahead of their use,
// without depending on each other.  cell_line_finish masks them and takes
// the neighbours of the inner lanes from the shuffles.
struct LineRaw
{
    float xc, xe;   // x at ix, and at the warp-edge neighbour
    int mc, me;     // mask bytes (2 = eliminated or outside)
};

__device__ __forceinline__ void cell_line_fetch(const MixedArgs& a, const float* x, int ix, int iy, int z, bool lv,
                                                LineRaw& R)
{
    const int nx = a.gx, lane = threadIdx.x & 31;
    const int j = ix + nx * (iy + a.gy * z);
    const bool in = lv && ix < nx;
    R.xc = in ? x[j] : 0.f;
    R.mc = in ? (int)__ldg(a.mf_mask + j) : 2;
    const int je = lane == 0 ? j - 1 : j + 1;
    const bool ein = lv && (lane == 0 ? (ix >= 1 && ix - 1 < nx) : (lane == 31 && ix + 1 < nx));
    R.xe = ein ? x[je] : 0.f;
    R.me = ein ? (int)__ldg(a.mf_mask + je) : 2;
}

__device__ __forceinline__ void cell_line_finish(const LineRaw& R, float& l, float& c, float& r)
{
    const int lane = threadIdx.x & 31;
    const float v = (R.mc & 2) ? 0.f : R.xc;
    const float e = (R.me & 2) ? 0.f : R.xe;
    float lf = __shfl_up_sync(0xffffffffu, v, 1), rt = __shfl_down_sync(0xffffffffu, v, 1);
    if (lane == 0) lf = e;
    if (lane == 31) rt = e;
    l = lf;
    c = v;
    r = rt;
}

// cell coefficients (cx, cy, cz), cx in {ix - 1, ix}, cy in {iy - 1, iy}:
// raw loads (own column, and ix - 1 on lane 0), then the shuffle
struct LayerRaw
{
    float v[2], e[2];
};

__device__ __forceinline__ void cell_layer_fetch(const MixedArgs& a, int ix, int iy, int cz, LayerRaw& R)
{
    const int ncx = a.gx - 1, ncy = a.gy - 1, lane = threadIdx.x & 31;
    const bool zin = cz >= 0 && cz < a.gz - 1;
#pragma unroll
    for (int ey = 0; ey < 2; ey++)
    {
        const int cy = iy - 1 + ey;
        const bool yin = zin && cy >= 0 && cy < ncy;
        const int base = ncx * (cy + ncy * cz);
        R.v[ey] = yin && ix < ncx ? __ldg(a.mf_alpha + base + ix) : 0.f;
        R.e[ey] = lane == 0 && yin && ix >= 1 && ix - 1 < ncx ? __ldg(a.mf_alpha + base + ix - 1) : 0.f;
    }
}

__device__ __forceinline__ void cell_layer_finish(const LayerRaw& R, float (&A)[2][2])
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int ey = 0; ey < 2; ey++)
    {
        float lf = __shfl_up_sync(0xffffffffu, R.v[ey], 1);
        if (lane == 0) lf = R.e[ey];
        A[ey][1] = R.v[ey];
        A[ey][0] = lf;
    }
}

// per-thread constants of the fmt 2 product
struct CellCtx
{
    const float* x;
    int ix, iy, nx, ny, nz, z1;
    bool act, px0, px1, py0, py1;
    bool lv[3];
    float beta;
};

// One node of the column: planes z-1, z, z+1 in P[A], P[B], P[C] (P[C] is
// filled here from the prefetched raw loads), cell layers z-1 and z in
// Ac[J0], Ac[J1] (Ac[J1] filled here); then the loads of plane z+2 and
// layer z+1 are issued for the next step.  The slots rotate with the step,
// so the window is never copied.
// The node's own u, mask byte and r come one step ahead too (NU: u and mask
// of node z + 1 from the raw line loads, rn: its r).
struct NodeNext
{
    float u, r;
    int m;
};

template <int A, int B, int C, int J0, int J1>
__device__ __forceinline__ void cell_step(const MixedArgs& a, const CellCtx& t, int z, float (&P)[3][3][3],
                                          float (&Ac)[2][2][2], LineRaw (&NR)[3], LayerRaw& NA, NodeNext& nn,
                                          float (&v)[3])
{
    const float u = nn.u, r = nn.r;
    const int mk = nn.m;
    const int i = t.ix + t.nx * (t.iy + t.ny * z);
    nn.u = NR[1].xc;  // node z + 1 (raw, unmasked)
    nn.m = NR[1].mc;
#pragma unroll
    for (int l = 0; l < 3; l++) cell_line_finish(NR[l], P[C][l][0], P[C][l][1], P[C][l][2]);
    cell_layer_finish(NA, Ac[J1]);
    if (z + 1 < t.z1)
    {
#pragma unroll
        for (int l = 0; l < 3; l++)
            cell_line_fetch(a, t.x, t.ix, t.iy + l - 1, z + 2, t.lv[l] && z + 2 < t.nz, NR[l]);
        cell_layer_fetch(a, t.ix, t.iy, z + 1, NA);
        nn.r = t.act ? a.r32[i + t.nx * t.ny] : 0.f;
    }
    if (!t.act) return;  // lanes past the lattice: only the shuffles above
    float w;
    if (mk & 1)
        w = __ldg(a.mf_dbc + i) * u;
    else
    {
        const int pl[3] = {A, B, C};
        const int jl[2] = {J0, J1};
        // Laplace: per cell around the node (absent cells have alpha 0)
        float accL = 0.f;
#pragma unroll
        for (int ez = 0; ez < 2; ez++)
#pragma unroll
            for (int ey = 0; ey < 2; ey++)
#pragma unroll
                for (int ex = 0; ex < 2; ex++)
                {
                    float sL = 0.f;
#pragma unroll
                    for (int bz = 0; bz < 2; bz++)
#pragma unroll
                        for (int by = 0; by < 2; by++)
#pragma unroll
                            for (int bx = 0; bx < 2; bx++)
                            {
                                const int pat = ((1 - ex) == bx ? 1 : 0) | ((1 - ey) == by ? 2 : 0) |
                                                ((1 - ez) == bz ? 4 : 0);
                                sL += a.mf_L[pat] * P[pl[ez + bz]][ey + by][ex + bx];
                            }
                    accL += Ac[jl[ez]][ey][ex] * sL;
                }
        // mass: M_box and the presence of the cells are tensor products, so
        // the sum over the present cells is the 3 x 3 x 3 stencil
        // mx (x) my (x) mz with per-axis weights -- summed axis by axis
        const bool pz0 = z > 0, pz1 = z < t.nz - 1;
        const float mx0 = t.px0 ? a.mf_m1[1] : 0.f, mx2 = t.px1 ? a.mf_m1[1] : 0.f;
        const float mx1 = (t.px0 ? a.mf_m1[0] : 0.f) + (t.px1 ? a.mf_m1[0] : 0.f);
        const float my0 = t.py0 ? a.mf_m1[3] : 0.f, my2 = t.py1 ? a.mf_m1[3] : 0.f;
        const float my1 = (t.py0 ? a.mf_m1[2] : 0.f) + (t.py1 ? a.mf_m1[2] : 0.f);
        const float mz0 = pz0 ? a.mf_m1[5] : 0.f, mz2 = pz1 ? a.mf_m1[5] : 0.f;
        const float mz1 = (pz0 ? a.mf_m1[4] : 0.f) + (pz1 ? a.mf_m1[4] : 0.f);
        float accM = 0.f;
#pragma unroll
        for (int q = 0; q < 3; q++)
        {
            float sy = 0.f;
#pragma unroll
            for (int l = 0; l < 3; l++)
            {
                const float* row = P[pl[q]][l];
                const float sx = mx0 * row[0] + mx1 * row[1] + mx2 * row[2];
                sy += (l == 0 ? my0 : l == 1 ? my1 : my2) * sx;
            }
            accM += (q == 0 ? mz0 : q == 1 ? mz1 : mz2) * sy;
        }
        w = accL + t.beta * accM;
    }
    a.w32[i] = w;
    v[0] += r * u;
    v[1] += w * u;
    v[2] += r * r;
}

// S for fmt 2: iter += 1 ; w32 = A32 u32 ; partials of r.u, w.u, r.r
__global__ void __launch_bounds__(32 * kCellWarps) k_mp_spmv_cells(MixedArgs a)
{
    KState* st = a.st;
    if (st->done || st->replace) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->iter += 1;  // no block of this kernel reads iter
    CellCtx t;
    t.nx = a.gx; t.ny = a.gy; t.nz = a.gz;
    const CellGrid G = cell_grid(t.nx, t.ny, t.nz);
    const int b = blockIdx.x, bxi = b % G.bx, byi = (b / G.bx) % G.by, bzi = b / (G.bx * G.by);
    t.ix = bxi * 32 + (threadIdx.x & 31);
    t.iy = byi * kCellWarps + (threadIdx.x >> 5);
    const int z0 = bzi * kCellZ;
    t.z1 = min(t.nz, z0 + kCellZ);
    const bool yv = t.iy < t.ny;
    t.act = yv && t.ix < t.nx;
    t.x = a.u32;
    t.beta = __ldg(a.mf_beta);
    t.px0 = t.ix > 0; t.px1 = t.ix < t.nx - 1; t.py0 = t.iy > 0; t.py1 = t.iy < t.ny - 1;
#pragma unroll
    for (int dy = -1; dy <= 1; dy++) t.lv[dy + 1] = yv && t.iy + dy >= 0 && t.iy + dy < t.ny;
    // P[slot][line dy+1][dx+1]: three rotating plane slots; Ac[slot][ey][ex]
    float P[3][3][3];
    float Ac[2][2][2];
    LineRaw NR[3];
    LayerRaw NA;
    // planes z0 - 1 -> slot 0, z0 -> slot 1; layer z0 - 1 -> slot 0
#pragma unroll
    for (int q = 0; q < 2; q++)
    {
        const int z = z0 - 1 + q;
        const bool zv = z >= 0 && z < t.nz;
#pragma unroll
        for (int l = 0; l < 3; l++) cell_line_fetch(a, t.x, t.ix, t.iy + l - 1, z, t.lv[l] && zv, NR[l]);
#pragma unroll
        for (int l = 0; l < 3; l++) cell_line_finish(NR[l], P[q][l][0], P[q][l][1], P[q][l][2]);
    }
    cell_layer_fetch(a, t.ix, t.iy, z0 - 1, NA);
    cell_layer_finish(NA, Ac[0]);
    // node z0: u and mask from the raw center line of plane z0 (still in NR)
    NodeNext nn;
    nn.u = NR[1].xc;
    nn.m = NR[1].mc;
    nn.r = t.act ? a.r32[t.ix + t.nx * (t.iy + t.ny * z0)] : 0.f;
#pragma unroll
    for (int l = 0; l < 3; l++) cell_line_fetch(a, t.x, t.ix, t.iy + l - 1, z0 + 1, t.lv[l] && z0 + 1 < t.nz, NR[l]);
    cell_layer_fetch(a, t.ix, t.iy, z0, NA);
    float v[3] = {0.f, 0.f, 0.f};
    for (int z = z0; z < t.z1; z += 6)
    {
        cell_step<0, 1, 2, 0, 1>(a, t, z, P, Ac, NR, NA, nn, v);
        if (z + 1 >= t.z1) break;
        cell_step<1, 2, 0, 1, 0>(a, t, z + 1, P, Ac, NR, NA, nn, v);
        if (z + 2 >= t.z1) break;
        cell_step<2, 0, 1, 0, 1>(a, t, z + 2, P, Ac, NR, NA, nn, v);
        if (z + 3 >= t.z1) break;
        cell_step<0, 1, 2, 1, 0>(a, t, z + 3, P, Ac, NR, NA, nn, v);
        if (z + 4 >= t.z1) break;
        cell_step<1, 2, 0, 0, 1>(a, t, z + 4, P, Ac, NR, NA, nn, v);
        if (z + 5 >= t.z1) break;
        cell_step<2, 0, 1, 1, 0>(a, t, z + 5, P, Ac, NR, NA, nn, v);
    }
    mp_sum_products(v, st);
}

int cell_spmv_grid(int nx, int ny, int nz)
{
    const CellGrid G = cell_grid(nx, ny, nz);
    return G.bx * G.by * G.bz;
}

constexpr int kU32 = 8;  // elements per thread per step, loaded before use
constexpr int kU4 = 2;   // 16-byte groups per array, thread and step in k_mp_update

// one row of the Chronopoulos-Gear update
__device__ __forceinline__ void mp_update_one(float u, float w, float pp, float sp, float xp, float rp, float d, float fa,
                                              float fb, float& p, float& s, float& x, float& r, float& un)
{
    p = u + fb * pp;
    s = w + fb * sp;
    r = rp - fa * s;
    x = xp + fa * p;
    un = r * d;
}

// V: p, s, x32, r32 (and u32 = M^-1 r32 in the preconditioned form).  The
// block's first vector loads are issued before warp 0 forms alpha and beta
// from the product partials, so they overlap the reduction.
template <bool SCALED>
__device__ __forceinline__ void mp_load4(const MixedArgs& a, int i, bool in, float4& u, float4& w, float4& p, float4& s,
                                         float4& x, float4& r, float4& d)
{
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    w = in ? ((const float4*)a.w32)[i] : z4;
    p = in ? ((const float4*)a.p32)[i] : z4;
    s = in ? ((const float4*)a.s32)[i] : z4;
    x = in ? ((const float4*)a.x32)[i] : z4;
    r = in ? ((const float4*)a.r32)[i] : z4;
    if constexpr (SCALED)
    {
        u = r;
        d = z4;
    }
    else
    {
        u = in ? ((const float4*)a.u32)[i] : z4;
        d = in ? ((const float4*)a.d32)[i] : z4;
    }
}

template <bool SCALED>
__global__ void __launch_bounds__(kThreads) k_mp_update(MixedArgs a)
{
    // 16-byte accesses over the first 4 * (n / 4) rows (the FP32 vectors
    // are 256-byte aligned), kU4 of them per array and thread in flight;
    // the last n % 4 rows one by one.  Scaled form: u is r itself.  The
    // first loads go out before the state is read (they are in bounds and
    // unused when the iteration has ended).
    const int n = a.n, n4 = n >> 2, stride = gridDim.x * blockDim.x;
    float4 uv[kU4], wv[kU4], pv[kU4], sv[kU4], xv[kU4], rv[kU4], dv[kU4];
    int base = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int k = 0; k < kU4; k++)
        mp_load4<SCALED>(a, base + k * stride, base + k * stride < n4, uv[k], wv[k], pv[k], sv[k], xv[k], rv[k], dv[k]);
    __shared__ double s_ab[2];
    __shared__ int s_stop;
    if (threadIdx.x < 32)
    {
        int stop = 0;
        double al = 0.0, be = 0.0;
        mp_iteration_scalars(a, blockIdx.x == 0, stop, al, be);
        if (threadIdx.x == 0)
        {
            s_ab[0] = al;
            s_ab[1] = be;
            s_stop = stop;
        }
    }
    __syncthreads();
    if (s_stop) return;
    const float fa = (float)s_ab[0], fb = (float)s_ab[1];
    float4* p4 = (float4*)a.p32;
    float4* s4 = (float4*)a.s32;
    float4* x4 = (float4*)a.x32;
    float4* r4 = (float4*)a.r32;
    float4* uo4 = (float4*)a.u32;
    while (base < n4)
    {
#pragma unroll
        for (int k = 0; k < kU4; k++)
        {
            const int i = base + k * stride;
            if (i < n4)
            {
                float4 p, s, x, r, u;
                mp_update_one(uv[k].x, wv[k].x, pv[k].x, sv[k].x, xv[k].x, rv[k].x, dv[k].x, fa, fb, p.x, s.x, x.x, r.x, u.x);
                mp_update_one(uv[k].y, wv[k].y, pv[k].y, sv[k].y, xv[k].y, rv[k].y, dv[k].y, fa, fb, p.y, s.y, x.y, r.y, u.y);
                mp_update_one(uv[k].z, wv[k].z, pv[k].z, sv[k].z, xv[k].z, rv[k].z, dv[k].z, fa, fb, p.z, s.z, x.z, r.z, u.z);
                mp_update_one(uv[k].w, wv[k].w, pv[k].w, sv[k].w, xv[k].w, rv[k].w, dv[k].w, fa, fb, p.w, s.w, x.w, r.w, u.w);
                p4[i] = p;
                s4[i] = s;
                x4[i] = x;
                r4[i] = r;
                if constexpr (!SCALED) uo4[i] = u;
            }
        }
        base += kU4 * stride;
        if (base >= n4) break;
#pragma unroll
        for (int k = 0; k < kU4; k++)
            mp_load4<SCALED>(a, base + k * stride, base + k * stride < n4, uv[k], wv[k], pv[k], sv[k], xv[k], rv[k],
                             dv[k]);
    }
    for (int i = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        float p, s, x, r, u;
        const float ri = a.r32[i];
        mp_update_one(SCALED ? ri : a.u32[i], a.w32[i], a.p32[i], a.s32[i], a.x32[i], ri, SCALED ? 0.f : a.d32[i], fa,
                      fb, p, s, x, r, u);
        a.p32[i] = p;
        a.s32[i] = s;
        a.x32[i] = x;
        a.r32[i] = r;
        if (!SCALED) a.u32[i] = u;
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

// false in every thread of the block once any block gave up waiting (after
// `limit` polls of the generation word)
__device__ bool mp_grid_barrier(KState* st, unsigned limit = kBarSpinLimit)
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
                if (++spins > limit || *(volatile int*)&st->bar_err)
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
        reduce_partials_bcast<3>(st->cg_ps, gridDim.x, g);
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
    k_mp_scale<<<vec_grid(a.n), kThreads, 0, s>>>(a, dinv64, d32);
    k_mp_convert<<<vec_grid(a.n), kThreads, 0, s>>>(a, row_len, slot_up, U, val32, d32);
}

int red_grid(int n);

// fmt 2 operator: FP32 coefficients, mask, kept diagonals, Jacobi inverse.
// bc_mode / bc_flag / bc_rows describe the Dirichlet set (nbc rows).
void launch_mp_convert_cells(const MixedArgs& a, const double* coef, int64_t cells, float* alpha32, float* beta32,
                             unsigned char* mask, float* dbc, const int32_t* diag_pos, const double* dinv64,
                             float* d32, int bc_mode, const unsigned char* bc_flag, const int32_t* bc_rows, int nbc,
                             cudaStream_t s)
{
    const int g = vec_grid(a.n);
    k_mp_convert_cells<<<vec_grid((int)std::min<int64_t>(cells, 1 << 30)), kThreads, 0, s>>>(coef, cells, alpha32,
                                                                                             beta32);
    cudaMemsetAsync(mask, 0, (size_t)a.n, s);
    if (nbc > 0)
    {
        if (bc_mode == OGS_DIRICHLET_SYMMETRIC)
            k_mp_mask_symmetric<<<g, kThreads, 0, s>>>(bc_flag, mask, a.n);
        else
            k_mp_mask_rows<<<std::max(1, std::min(1024, (nbc + kThreads - 1) / kThreads)), kThreads, 0, s>>>(
                bc_rows, nbc, mask);
    }
    k_mp_dbc<<<g, kThreads, 0, s>>>(a, diag_pos, dinv64, d32, dbc);
}

// enqueues the operator check; out (2 unsigned, device) is zeroed first
void launch_mp_check(const MixedArgs& a, unsigned* out, cudaStream_t s)
{
    const int g = vec_grid(a.n);
    cudaMemsetAsync(out, 0, 2 * sizeof(unsigned), s);
    k_mp_check_fill<<<g, kThreads, 0, s>>>(a.w32, a.n);
    switch (a.fmt == 0 ? a.n_up : a.fmt == 2 ? -1 : 0)
    {
        case 14: k_mp_check<14><<<g, kThreads, 0, s>>>(a, out); break;
        case 8: k_mp_check<8><<<g, kThreads, 0, s>>>(a, out); break;
        case 5: k_mp_check<5><<<g, kThreads, 0, s>>>(a, out); break;
        case -1: k_mp_check<-1><<<g, kThreads, 0, s>>>(a, out); break;
        default: k_mp_check<0><<<g, kThreads, 0, s>>>(a, out); break;
    }
}

// grids of the FP32 CG kernels (the update/p kernels add this many SpMV
// partials, the p kernel this many update partials)
using LinesKernel = void (*)(MixedArgs);
using PairKernel = void (*)(MixedArgs, float*, float*);

template <int RX>
static LinesKernel lines_kernel_rx(int rxy, int plane, PairKernel* pair)
{
    if (plane)
    {
        *pair = k_mp_product_pair<RX, 0, 1>;
        return k_mp_spmv_lines<RX, 0, 1>;
    }
    switch (rxy)
    {
        case 0: *pair = k_mp_product_pair<RX, 0, 4>; return k_mp_spmv_lines<RX, 0, 4>;
        case 1: *pair = k_mp_product_pair<RX, 1, 4>; return k_mp_spmv_lines<RX, 1, 4>;
        case 2: *pair = k_mp_product_pair<RX, 2, 4>; return k_mp_spmv_lines<RX, 2, 4>;
        default: *pair = k_mp_product_pair<RX, 3, 4>; return k_mp_spmv_lines<RX, 3, 4>;
    }
}

// the instantiations for nx mod 4 and nxy mod 4 (a.lines 1: the 27-point
// lattice) or nx mod 4 (a.lines 2: the 9-point plane lattice); pair: the
// comparison kernel, may be NULL
static LinesKernel lines_kernel(const MixedArgs& a, PairKernel* pair = nullptr)
{
    PairKernel p = nullptr;
    LinesKernel k;
    const int rxy = a.off[9] & 3, plane = a.lines == 2;
    switch (a.off[3] & 3)
    {
        case 0: k = lines_kernel_rx<0>(rxy, plane, &p); break;
        case 1: k = lines_kernel_rx<1>(rxy, plane, &p); break;
        case 2: k = lines_kernel_rx<2>(rxy, plane, &p); break;
        default: k = lines_kernel_rx<3>(rxy, plane, &p); break;
    }
    if (pair) *pair = p;
    return k;
}

// both products of the lattice operator on a.r32 (a.lines set)
void launch_mp_product_pair(const MixedArgs& a, float* y_rows, float* y_lines, cudaStream_t s)
{
    PairKernel pair = nullptr;
    lines_kernel(a, &pair);
    pair<<<vec_grid((a.n + 3) / 4), kThreads, 0, s>>>(a, y_rows, y_lines);
}

int mp_spmv_grid(const MixedArgs& a)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (a.lines)
    {
        // as many blocks as are resident at once, each thread a group of
        // four rows per pass
        int occ = 2;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lines_kernel(a), kThreads, 0);
        const int need = ((a.n + 3) / 4 + kThreads - 1) / kThreads;
        return std::max(1, std::min(need, std::min(sms * std::max(1, occ), kMaxBlocks)));
    }
    // three blocks of the register-heavy diagonal kernel are resident per SM
    return std::max(1, std::min((a.n + kThreads - 1) / kThreads, std::min(sms * 3, kMaxBlocks)));
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
    switch (a.fmt == 0 ? a.n_up : a.fmt == 2 ? -1 : 0)
    {
        case 14: return persist_grid_for<14>(a.n);
        case 8: return persist_grid_for<8>(a.n);
        case 5: return persist_grid_for<5>(a.n);
        case -1: return persist_grid_for<-1>(a.n);
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
    switch (a.fmt == 0 ? a.n_up : a.fmt == 2 ? -1 : 0)
    {
        case 14: return cudaLaunchKernelEx(&lc, k_mp_persist<14>, a, iters);
        case 8: return cudaLaunchKernelEx(&lc, k_mp_persist<8>, a, iters);
        case 5: return cudaLaunchKernelEx(&lc, k_mp_persist<5>, a, iters);
        case -1: return cudaLaunchKernelEx(&lc, k_mp_persist<-1>, a, iters);
        default: return cudaLaunchKernelEx(&lc, k_mp_persist<0>, a, iters);
    }
}

// Self-test of the bounded wait: every block passes one barrier of the
// persistent FP32 kernel; with `withhold`, block 0 leaves without arriving,
// so the others wait on a generation word nothing bumps and give up after
// `limit` polls.  go[b]: whether block b passed.
__global__ void k_mp_barrier_selftest(KState* st, int withhold, unsigned limit, int* go)
{
    if (withhold && blockIdx.x == 0)
    {
        if (threadIdx.x == 0) go[0] = 0;
        return;
    }
    const bool ok = mp_grid_barrier(st, limit);
    if (threadIdx.x == 0) go[blockIdx.x] = ok ? 1 : 0;
}

cudaError_t launch_mp_barrier_selftest(KState* st, int grid, int withhold, unsigned limit, int* go, cudaStream_t s)
{
    void* args[] = {&st, &withhold, &limit, &go};
    return cudaLaunchCooperativeKernel((const void*)k_mp_barrier_selftest, dim3(grid), dim3(kThreads), args, 0, s);
}

void launch_mp_iteration(const MixedArgs& a, cudaStream_t s, cudaEvent_t eb, cudaEvent_t ee)
{
    const int gs = mp_spmv_grid(a);
    if (eb) cudaEventRecordWithFlags(eb, s, cudaEventRecordExternal);
    switch (a.fmt == 0 ? a.n_up : a.fmt == 2 ? -1 : 0)
    {
        case 14:  // hex, 27-point
            if (a.lines) lines_kernel(a)<<<gs, kThreads, 0, s>>>(a);
            else if (a.scaled) k_mp_spmv<14, true><<<gs, kThreads, 0, s>>>(a);
            else k_mp_spmv<14><<<gs, kThreads, 0, s>>>(a);
            break;
        case 8:  // Kuhn tets, 15-point
            if (a.scaled) k_mp_spmv<8, true><<<gs, kThreads, 0, s>>>(a);
            else k_mp_spmv<8><<<gs, kThreads, 0, s>>>(a);
            break;
        case 5:  // quads, 9-point
            if (a.lines) lines_kernel(a)<<<gs, kThreads, 0, s>>>(a);
            else if (a.scaled) k_mp_spmv<5, true><<<gs, kThreads, 0, s>>>(a);
            else k_mp_spmv<5><<<gs, kThreads, 0, s>>>(a);
            break;
        case -1:  // hex lattice, cell coefficients
            k_mp_spmv_cells<<<cell_spmv_grid(a.gx, a.gy, a.gz), 32 * kCellWarps, 0, s>>>(a);
            break;
        default: k_mp_spmv<0><<<gs, kThreads, 0, s>>>(a); break;   // SELL-32 FP32
    }
    if (ee) cudaEventRecordWithFlags(ee, s, cudaEventRecordExternal);
    if (a.scaled)
        k_mp_update<true><<<red_grid(a.n), kThreads, 0, s>>>(a);
    else
        k_mp_update<false><<<red_grid(a.n), kThreads, 0, s>>>(a);
}

}  // namespace ogs

unsigned long long ogs_oob_mixed() { return ogs::oob_take(); }
