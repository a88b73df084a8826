// batch.cu -- Monte-Carlo batches: many steady GROUNDWATER_FLOW
// realisations on structured hex boxes of different sizes, assembled and
// solved by ONE cooperative persistent kernel.
//
// Per realisation the work is that of the single-system path (element
// Laplace matrices of CFiniteElementStd::CalcLaplace with mat = K *
// time_unit_factor, fem_ele_std.cpp:4948-5070 / 2308-2384; the symmetric
// Dirichlet elimination of MXRandbed, matrix_routines.cpp:2314-2520; CG of
// Linear_EQS with Jacobi, equation_class.cpp:1129-1187, run as FP32 inner
// CG with FP64 residual replacement like mixed.cu).  What changes for a
// batch:
//
//  * Layout.  A structured box needs no pattern and no slot map: every row
//    has the 27-point stencil, stored as the upper half of its
//    diagonal-offset form U[d][i] = A[i][i + off_d], 14 offsets, FP64 (for
//    the residual) and FP32 (for the sweeps).  Realisations are
//    concatenated; rows are cut into equal work tiles.
//  * Assembly is row-centric: row i sums, for each stored offset, the
//    contributions of the (at most 8) elements that hold both nodes -- a
//    gather, so no atomics and a fixed summation order.  The element matrix
//    of a box cell is K_e times one 8x8 local matrix.
//  * One launch.  The kernel is launched cooperatively (all blocks
//    resident) and walks: assembly | barrier | { phase A | barrier |
//    phase B | barrier } until every realisation has converged.  Phase A
//    is the matrix product of each active tile (FP32 operator for CG
//    steps, FP64 for residual replacements) with its partial dot products;
//    phase B reduces the partials of the tile's realisation (every tile of
//    a realisation adds them in the same order, so all hold bitwise the
//    same scalars), decides and updates its rows.  Each tile keeps its own
//    copy of the realisation's solver scalars, so no scalar is written by
//    one block and read by another within a phase.
//  * Converged realisations leave the work list: the last block to reach
//    the end-of-step barrier rebuilds the list of active realisations and
//    their tile prefix, so the remaining tiles are spread over all blocks
//    again (round robin, equal tile sizes).
//  * Grid barrier: an arrival counter and a generation word; waits are
//    bounded (a timeout sets an error flag, after which every block leaves
//    the kernel at its next barrier).
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

#include "krylov.cuh"

namespace ogs {

// upper stencil offsets (dx, dy, dz): linear offset dx + nx dy + nx ny dz
// >= 0, ascending for nx, ny >= 3 (compile-time table: unrolled loops fold
// each offset into one integer multiply-add)
__host__ __device__ constexpr int kUpX(int d) { return d == 0 ? 0 : d == 1 ? 1 : (d - 2) % 3 - 1; }
__host__ __device__ constexpr int kUpY(int d) { return d < 2 ? 0 : d < 5 ? 1 : (d - 5) / 3 - 1; }
__host__ __device__ constexpr int kUpZ(int d) { return d < 5 ? 0 : 1; }

__device__ __forceinline__ int up_offset(int d, int nx, int nxy) { return kUpX(d) + nx * kUpY(d) + nxy * kUpZ(d); }

struct BReal
{
    int nx, ny, nz, n;
    int64_t row0;   // first row in the batch vectors
    int64_t elem0;  // first element in the conductivity array
    int tile0, ntiles;
    double h_left, h_right;
};

struct BTile
{
    int r, i0, i1, pad;
};

// solver scalars of one realisation, one copy per tile
struct TState
{
    double bnorm, scale, ratio, rmax, gam[2], eta[2], error;
    int iter, base_iter, mode, status, first, replacements, done, pad;
};

enum { kModeReplace = 0, kModeIter = 1 };

struct BCtl
{
    unsigned bar_count, bar_gen;
    int err, exit;
    int done_count, seen_done;
    int step, max_steps;
    int n_act, n_act_tiles;
    unsigned long long t0;  // %globaltimer at the start of the launch (ns)
    unsigned spin_limit;    // polls before a wait gives up (0: kSpinLimit)
};

struct BatchArgs
{
    const BReal* real;
    const BTile* tiles;
    int n_real, n_tiles;
    const double* ek;
    double *U64, *b, *x64, *r64;
    float *U32, *x32, *r32, *p32, *s32, *u32, *w32, *d32;
    TState* ts;
    double* part;      // [n_tiles][4]
    BCtl* ctl;
    int* act_real;     // [n_real]
    int* act_pref;     // [n_real + 1]
    int* real_done;    // [n_real]
    ogs_batch_stats* out;
    double tol, delta;
    int max_iter;
    const double* kloc;  // [64] local Laplace of a cell, corner-bit order, times time_unit_factor
};

// ------------------------------------------------------------------
// bounded grid barrier
// ------------------------------------------------------------------
constexpr unsigned kSpinLimit = 1u << 25;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Returns false in every thread of the block when the batch must stop
// (timeout anywhere, or ctl->exit set by the last arriver).  on_last runs
// in the one thread that completes the barrier, before the release.
template <class F>
__device__ bool grid_barrier(BCtl* c, F on_last)
{
    __shared__ int s_go;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int go = 1;
        if (ld_volatile(&c->err))
            go = 0;
        else
        {
            const unsigned gen = ld_acquire_u32(&c->bar_gen);
            __threadfence();
            const unsigned arrived = atomicAdd(&c->bar_count, 1u) + 1u;
            if (arrived == gridDim.x)
            {
                c->bar_count = 0u;
                on_last();
                __threadfence();
                st_release_u32(&c->bar_gen, gen + 1u);
            }
            else
            {
                unsigned spins = 0;
                const unsigned limit = c->spin_limit ? c->spin_limit : kSpinLimit;
                while (ld_acquire_u32(&c->bar_gen) == gen)
                {
                    if (++spins > limit)
                    {
                        atomicExch(&c->err, 1);
                        go = 0;
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __threadfence();
            if (go && (ld_volatile(&c->err) || ld_volatile(&c->exit))) go = 0;
        }
        s_go = go;
    }
    __syncthreads();
    return s_go != 0;
}

// ------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------
template <int NV, int NT, typename T>
__device__ __forceinline__ void tile_partials(const T* vin, double* dst)
{
    __shared__ double sm[NV][NT / 32];
    T w[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) w[k] = vin[k];
    warp_allsum<NV, T>(w);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sm[k][wid] = (double)w[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++)
        {
            double s = 0.0;
            for (int q = 0; q < NT / 32; q++) s += sm[k][q];
            __stcg(dst + k, s);
        }
    __syncthreads();
}

// sum of the partials of tiles tile0 .. tile0+nt-1, identical in every thread
// of every block
template <int NV, int NT>
__device__ __forceinline__ void realisation_sum(const double* part, int tile0, int nt, double* out)
{
    __shared__ double sm[NV][NT / 32];
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = 0.0;
    for (int q = threadIdx.x; q < nt; q += NT)
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] += __ldcg(part + (size_t)(tile0 + q) * 4 + k);
    warp_allsum<NV, double>(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sm[k][wid] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++)
    {
        double s = 0.0;
        for (int q = 0; q < NT / 32; q++) s += sm[k][q];
        out[k] = s;
    }
    __syncthreads();
}

// tile state written by another block in an earlier step: L2 loads, field
// by field (keeps the copy in registers)
__device__ __forceinline__ TState load_state(const TState* p)
{
    TState s;
    s.bnorm = __ldcg(&p->bnorm);
    s.scale = __ldcg(&p->scale);
    s.ratio = __ldcg(&p->ratio);
    s.rmax = __ldcg(&p->rmax);
    s.gam[0] = __ldcg(&p->gam[0]);
    s.gam[1] = __ldcg(&p->gam[1]);
    s.eta[0] = __ldcg(&p->eta[0]);
    s.eta[1] = __ldcg(&p->eta[1]);
    s.error = __ldcg(&p->error);
    s.iter = __ldcg(&p->iter);
    s.base_iter = __ldcg(&p->base_iter);
    s.mode = __ldcg(&p->mode);
    s.status = __ldcg(&p->status);
    s.first = __ldcg(&p->first);
    s.replacements = __ldcg(&p->replacements);
    s.done = __ldcg(&p->done);
    s.pad = 0;
    return s;
}

// A[i][j] before the Dirichlet elimination, j = i + (dx, dy, dz)
__device__ __forceinline__ double stencil_entry(const BatchArgs& a, const BReal& R, const double* __restrict__ ek,
                                                int ix, int iy, int iz, int dx, int dy, int dz)
{
    const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
    if (jx < 0 || jy < 0 || jz < 0 || jx >= R.nx || jy >= R.ny || jz >= R.nz) return 0.0;
    const int ex0 = max(ix, jx) - 1, ex1 = min(ix, jx);
    const int ey0 = max(iy, jy) - 1, ey1 = min(iy, jy);
    const int ez0 = max(iz, jz) - 1, ez1 = min(iz, jz);
    double acc = 0.0;
    for (int ez = max(ez0, 0); ez <= min(ez1, R.nz - 2); ez++)
        for (int ey = max(ey0, 0); ey <= min(ey1, R.ny - 2); ey++)
            for (int ex = max(ex0, 0); ex <= min(ex1, R.nx - 2); ex++)
            {
                const int ca = (ix - ex) + 2 * (iy - ey) + 4 * (iz - ez);
                const int cb = (jx - ex) + 2 * (jy - ey) + 4 * (jz - ez);
                const double k = __ldg(ek + ex + (R.nx - 1) * (ey + (R.ny - 1) * ez));
                acc += k * __ldg(a.kloc + ca * 8 + cb);
            }
    return acc;
}


// ------------------------------------------------------------------
// phases
// ------------------------------------------------------------------
// assembly of one tile: U64, U32, b, d32 and the initial x64 (heads on the
// Dirichlet faces, 0 elsewhere)
template <int NT>
__device__ void assemble_tile(const BatchArgs& a, const BTile& T)
{
    const BReal R = a.real[T.r];
    const double* ek = a.ek + R.elem0;
    double* U64 = a.U64 + 14 * R.row0;
    float* U32 = a.U32 + 14 * R.row0;
    const int nxy = R.nx * R.ny;
    for (int i = T.i0 + threadIdx.x; i < T.i1; i += NT)
    {
        const int iz = i / nxy, rem = i - iz * nxy, iy = rem / R.nx, ix = rem - iy * R.nx;
        const bool bc = ix == 0 || ix == R.nx - 1;
        const double hb = ix == 0 ? R.h_left : R.h_right;
        double diag = stencil_entry(a, R, ek, ix, iy, iz, 0, 0, 0);
        double bi = 0.0;
        if (bc)
        {
            if (fabs(diag) < DBL_MIN) diag = DBL_EPSILON;
            bi = diag * hb;
        }
        else if (ix == 1 || ix == R.nx - 2)
        {
            // lift the Dirichlet columns into b
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++)
                    {
                        const int jx = ix + dx;
                        if (jx != 0 && jx != R.nx - 1) continue;
                        const double aij = stencil_entry(a, R, ek, ix, iy, iz, dx, dy, dz);
                        bi -= aij * (jx == 0 ? R.h_left : R.h_right);
                    }
        }
        U64[i] = diag;
        U32[i] = (float)diag;
#pragma unroll
        for (int d = 1; d < 14; d++)
        {
            const int jx = ix + kUpX(d);
            double v = 0.0;
            if (!bc && jx != 0 && jx != R.nx - 1)
                v = stencil_entry(a, R, ek, ix, iy, iz, kUpX(d), kUpY(d), kUpZ(d));
            U64[(size_t)d * R.n + i] = v;
            U32[(size_t)d * R.n + i] = (float)v;
        }
        const int64_t g = R.row0 + i;
        a.b[g] = bi;
        a.x64[g] = bc ? hb : 0.0;
        a.x32[g] = 0.f;
        a.p32[g] = 0.f;
        a.s32[g] = 0.f;
        const double dinv = fabs(diag) < DBL_MIN ? 1.0 : 1.0 / diag;
        a.d32[g] = (float)dinv;
    }
}

// FP64 row of the half diagonal-offset operator applied to x64 + x32 / scale
__device__ __forceinline__ double row64(const double* __restrict__ U, int nx, int nxy, int n, int i,
                                        const double* x64, const float* x32, double inv)
{
    double acc = U[i] * (x64[i] + (double)x32[i] * inv);
#pragma unroll
    for (int d = 1; d < 14; d++)
    {
        const int o = up_offset(d, nx, nxy);
        const double* Ud = U + (size_t)d * n;
        if (i + o < n) acc += Ud[i] * (x64[i + o] + (double)x32[i + o] * inv);
        if (i - o >= 0) acc += Ud[i - o] * (x64[i - o] + (double)x32[i - o] * inv);
    }
    return acc;
}

// FP32 row, all pairs loaded before the FMAs (27 independent loads per thread)
__device__ __forceinline__ float row32(const float* __restrict__ U, int nx, int nxy, int n, int i,
                                       const float* x)
{
    float uv[27], xv[27];
    uv[0] = U[i];
    xv[0] = x[i];
#pragma unroll
    for (int d = 1; d < 14; d++)
    {
        const int o = up_offset(d, nx, nxy);
        const float* Ud = U + (size_t)d * n;
        const bool up = i + o < n, lo = i - o >= 0;
        uv[2 * d - 1] = up ? Ud[i] : 0.f;
        xv[2 * d - 1] = up ? x[i + o] : 0.f;
        uv[2 * d] = lo ? Ud[i - o] : 0.f;
        xv[2 * d] = lo ? x[i - o] : 0.f;
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 27; k++) acc += uv[k] * xv[k];
    return acc;
}

template <int NT>
__device__ void phase_a(const BatchArgs& a, int g)
{
    const BTile T = a.tiles[g];
    const BReal R = a.real[T.r];
    const TState S = load_state(a.ts + g);
    const int nxy = R.nx * R.ny;
    const int64_t r0 = R.row0;
    if (S.mode == kModeReplace)
    {
        const double inv = 1.0 / S.scale;
        const double* U = a.U64 + 14 * r0;
        double v[2] = {0.0, 0.0};
        for (int i = T.i0 + threadIdx.x; i < T.i1; i += NT)
        {
            const double bi = a.b[r0 + i];
            const double r = bi - row64(U, R.nx, nxy, R.n, i, a.x64 + r0, a.x32 + r0, inv);
            a.r64[r0 + i] = r;
            v[0] += r * r;
            v[1] += bi * bi;
        }
        tile_partials<2, NT, double>(v, a.part + (size_t)g * 4);
    }
    else
    {
        const float* U = a.U32 + 14 * r0;
        const float* u = a.u32 + r0;
        float v[3] = {0.f, 0.f, 0.f};
        for (int c = T.i0; c < T.i1; c += NT)
        {
            // bulk L2 prefetch of the next chunk of every other operator
            // stream (as the single-system FP32 SpMV)
            const int d = 2 * threadIdx.x, nb = c + NT;
            if (d < 14 && nb < T.i1)
            {
                const float* seg = U + (size_t)d * R.n;
                bulk_prefetch_l2(seg + nb, (size_t)min(NT, T.i1 - nb) * sizeof(float), seg, seg + R.n);
            }
            const int i = c + threadIdx.x;
            if (i >= T.i1) continue;
            const float w = row32(U, R.nx, nxy, R.n, i, u);
            a.w32[r0 + i] = w;
            const float ui = u[i], ri = a.r32[r0 + i];
            v[0] += ri * ui;
            v[1] += w * ui;
            v[2] += ri * ri;
        }
        tile_partials<3, NT, float>(v, a.part + (size_t)g * 4);
    }
}

template <int NT>
__device__ void finish_realisation(const BatchArgs& a, const BTile& T, int g, const BReal& R, const TState& S)
{
    if (threadIdx.x == 0 && g == R.tile0)
    {
        ogs_batch_stats o;
        o.iterations = S.iter;
        o.status = S.status;
        o.refinements = S.replacements;
        o.pad0 = 0;
        o.rel_residual = S.error;
        o.finish_ms = (double)(global_ns() - *(volatile unsigned long long*)&a.ctl->t0) * 1e-6;
        a.out[T.r] = o;
        a.real_done[T.r] = 1;
        atomicAdd(&a.ctl->done_count, 1);
    }
}

// p = u + beta p ; s = w + beta s ; x += alpha p ; r -= alpha s ; u = d r
// over rows [q0, q0 + len): four rows per thread per pass, all loads first,
// so each thread keeps 28 loads in flight
constexpr int kVU = 4;

template <int NT>
__device__ __forceinline__ void cg_update(const BatchArgs& a, int64_t q0, int len, float fb, float fa)
{
    float* __restrict__ u32 = a.u32 + q0;
    const float* __restrict__ w32 = a.w32 + q0;
    const float* __restrict__ d32 = a.d32 + q0;
    float* __restrict__ p32 = a.p32 + q0;
    float* __restrict__ s32 = a.s32 + q0;
    float* __restrict__ x32 = a.x32 + q0;
    float* __restrict__ r32 = a.r32 + q0;
    for (int base = threadIdx.x; base < len; base += kVU * NT)
    {
        float uv[kVU], wv[kVU], pv[kVU], sv[kVU], xv[kVU], rv[kVU], dv[kVU];
#pragma unroll
        for (int k = 0; k < kVU; k++)
        {
            const int i = base + k * NT;
            const bool in = i < len;
            uv[k] = in ? u32[i] : 0.f;
            wv[k] = in ? w32[i] : 0.f;
            pv[k] = in ? p32[i] : 0.f;
            sv[k] = in ? s32[i] : 0.f;
            xv[k] = in ? x32[i] : 0.f;
            rv[k] = in ? r32[i] : 0.f;
            dv[k] = in ? d32[i] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < kVU; k++)
        {
            const int i = base + k * NT;
            if (i < len)
            {
                const float p = uv[k] + fb * pv[k];
                const float s = wv[k] + fb * sv[k];
                const float r = rv[k] - fa * s;
                p32[i] = p;
                s32[i] = s;
                x32[i] = xv[k] + fa * p;
                r32[i] = r;
                u32[i] = r * dv[k];
            }
        }
    }
}

template <int NT>
__device__ void phase_b(const BatchArgs& a, int g)
{
    const BTile T = a.tiles[g];
    const BReal R = a.real[T.r];
    TState S = load_state(a.ts + g);
    const int64_t r0 = R.row0;
    if (S.mode == kModeReplace)
    {
        double rb[2];
        realisation_sum<2, NT>(a.part, R.tile0, R.ntiles, rb);
        const double inv_old = 1.0 / S.scale;
        bool done = false;
        if (S.first)
        {
            // Linear_EQS::CheckNormRHS of a fresh system (bNorm = 1.0)
            const double bn = sqrt(rb[1]);
            if (!isfinite(bn)) { S.status = OGS_NONFINITE; S.error = bn; done = true; }
            else if (bn / 1.0 < a.tol) { S.status = OGS_OK; S.error = bn; done = true; }
            else if (bn < DBL_MIN) { S.status = OGS_OK; S.error = 0.0; done = true; }
            S.bnorm = bn;
        }
        if (!done)
        {
            const double rn = sqrt(rb[0]);
            S.error = rn / S.bnorm;
            S.replacements += 1;
            if (!isfinite(S.error)) { S.status = OGS_NONFINITE; done = true; }
            else if (S.error < a.tol) { S.status = OGS_OK; done = true; }
            else if (S.iter >= a.max_iter) { S.status = OGS_NOT_CONVERGED; done = true; }
            if (!done)
            {
                const double ns = rn > DBL_MIN ? 1.0 / rn : 1.0;
                const double ratio = S.first ? 1.0 : ns / S.scale;
                const float fr = (float)ratio;
                const bool first = S.first != 0;
                for (int i = T.i0 + threadIdx.x; i < T.i1; i += NT)
                {
                    const int64_t q = r0 + i;
                    a.x64[q] += (double)a.x32[q] * inv_old;
                    a.x32[q] = 0.f;
                    const float r = (float)(a.r64[q] * ns);
                    a.r32[q] = r;
                    a.u32[q] = r * a.d32[q];
                    a.p32[q] = first ? 0.f : a.p32[q] * fr;
                    a.s32[q] = first ? 0.f : a.s32[q] * fr;
                }
                // the iteration that asked for the replacement is redone
                int it = S.iter;
                if (!first) it -= 1;
                S.iter = it;
                const double r2 = ratio * ratio;
                if (it & 1) { S.gam[1] *= r2; S.eta[1] *= r2; }
                else { S.gam[0] *= r2; S.eta[0] *= r2; }
                S.base_iter = it;
                S.rmax = -1.0;
                S.mode = kModeIter;
                S.scale = ns;
                S.ratio = ratio;
                S.first = 0;
            }
        }
        if (done)
        {
            for (int i = T.i0 + threadIdx.x; i < T.i1; i += NT)
            {
                const int64_t q = r0 + i;
                a.x64[q] += (double)a.x32[q] * inv_old;
                a.x32[q] = 0.f;
            }
            S.done = 1;
            finish_realisation<NT>(a, T, g, R, S);
        }
    }
    else
    {
        double gdr[3];
        realisation_sum<3, NT>(a.part, R.tile0, R.ntiles, gdr);
        const int it = S.iter + 1;
        const double gamma = gdr[0], delta = gdr[1], rn = sqrt(gdr[2]);
        const bool first = it == 1;
        const bool fresh = it == S.base_iter + 1;
        const double rmax = fresh ? rn : S.rmax;
        // scalars of the previous iteration (parity slots, selected without
        // dynamic indexing so the state stays in registers)
        const double gam_prev = (it - 1) & 1 ? S.gam[1] : S.gam[0];
        const double eta_prev = (it - 1) & 1 ? S.eta[1] : S.eta[0];
        const double beta = first ? 0.0 : gamma / gam_prev;
        const double eta = first ? delta : delta - beta * beta * eta_prev;
        const double alpha = gamma / eta;
        const double est = rn / S.scale / S.bnorm;
        const bool nonfinite = !isfinite(rn) || !isfinite(alpha);
        const bool repl = !nonfinite && !fresh && (est < a.tol || rn < a.delta * rmax || it > a.max_iter);
        if (fresh) S.rmax = rn;
        if (it & 1) { S.gam[1] = gamma; S.eta[1] = eta; }
        else { S.gam[0] = gamma; S.eta[0] = eta; }
        S.iter = it;
        if (nonfinite)
        {
            S.status = OGS_NONFINITE;
            S.error = rn;
            S.done = 1;
            finish_realisation<NT>(a, T, g, R, S);
        }
        else if (repl)
            S.mode = kModeReplace;
        else
            cg_update<NT>(a, r0 + T.i0, T.i1 - T.i0, (float)beta, (float)alpha);
    }
    __syncthreads();
    if (threadIdx.x == 0) a.ts[g] = S;
}

// active tile t -> tile index (binary search over the active prefix)
__device__ __forceinline__ int active_tile(const BatchArgs& a, int n_act, int t)
{
    int lo = 0, hi = n_act - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (a.act_pref[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int r = a.act_real[lo];
    return a.real[r].tile0 + (t - a.act_pref[lo]);
}

// run by the one thread that completes the end-of-step barrier
__device__ void end_of_step(const BatchArgs& a)
{
    BCtl* c = a.ctl;
    const int dc = ld_volatile(&c->done_count);
    if (dc != c->seen_done)
    {
        int k = 0, acc = 0;
        for (int r = 0; r < a.n_real; r++)
            if (!ld_volatile(a.real_done + r))
            {
                a.act_real[k] = r;
                a.act_pref[k] = acc;
                acc += a.real[r].ntiles;
                k++;
            }
        a.act_pref[k] = acc;
        c->n_act = k;
        c->n_act_tiles = acc;
        c->seen_done = dc;
    }
    c->step += 1;
    if (c->n_act == 0 || c->step >= c->max_steps) c->exit = 1;
}

// 256 threads: three blocks per SM (<= 85 registers); 512: one (<= 128)
template <int NT>
__global__ void __launch_bounds__(NT, NT == 256 ? 3 : 1) k_batch(BatchArgs a)
{
    BCtl* c = a.ctl;
    if (blockIdx.x == 0 && threadIdx.x == 0) c->t0 = global_ns();
    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) assemble_tile<NT>(a, a.tiles[t]);
    if (!grid_barrier(c, [] {})) return;
    for (;;)
    {
        const int n_act = ld_volatile(&c->n_act), nat = ld_volatile(&c->n_act_tiles);
        for (int t = blockIdx.x; t < nat; t += gridDim.x) phase_a<NT>(a, active_tile(a, n_act, t));
        if (!grid_barrier(c, [] {})) return;
        for (int t = blockIdx.x; t < nat; t += gridDim.x) phase_b<NT>(a, active_tile(a, n_act, t));
        if (!grid_barrier(c, [&] { end_of_step(a); })) return;
    }
}

// Self-test of the bounded wait: every block passes one barrier of the
// batch kernel; with `withhold`, block 0 leaves without arriving, so the
// others wait on a generation word nothing bumps and give up after
// c->spin_limit polls.  go[b]: whether block b passed.
__global__ void k_batch_barrier_selftest(BCtl* c, int withhold, int* go)
{
    if (withhold && blockIdx.x == 0)
    {
        if (threadIdx.x == 0) go[0] = 0;
        return;
    }
    const bool ok = grid_barrier(c, [] {});
    if (threadIdx.x == 0) go[blockIdx.x] = ok ? 1 : 0;
}

// the control block of the self-test (zeroed, then the spin limit set) and
// its launch
size_t batch_ctl_bytes() { return sizeof(BCtl); }

cudaError_t launch_batch_barrier_selftest(void* ctl, unsigned limit, int grid, int withhold, int* go, cudaStream_t s)
{
    BCtl h;
    std::memset(&h, 0, sizeof h);
    h.spin_limit = limit;
    cudaError_t e = cudaMemcpyAsync(ctl, &h, sizeof h, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    BCtl* c = (BCtl*)ctl;
    void* args[] = {&c, &withhold, &go};
    return cudaLaunchCooperativeKernel((const void*)k_batch_barrier_selftest, dim3(grid), dim3(256), args, 0, s);
}

}  // namespace ogs

using namespace ogs;

// ------------------------------------------------------------------
// host side
// ------------------------------------------------------------------
struct ogs_batch
{
    ogs_batch_config cfg{};
    int n_real = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<BReal> real;
    int64_t rows = 0, elems = 0;
    // device
    BReal* d_real = nullptr;
    BTile* d_tiles = nullptr;
    double* ek = nullptr;
    double *U64 = nullptr, *b = nullptr, *x64 = nullptr, *r64 = nullptr;
    float* f32 = nullptr;      // U32 and the FP32 vectors
    float *U32 = nullptr, *x32 = nullptr, *r32 = nullptr, *p32 = nullptr, *s32 = nullptr, *u32 = nullptr,
          *w32 = nullptr, *d32 = nullptr;
    TState* ts = nullptr;
    double* part = nullptr;
    BCtl* ctl = nullptr;
    int *act_real = nullptr, *act_pref = nullptr, *real_done = nullptr;
    ogs_batch_stats* out = nullptr;
    int tile_cap = 0;          // tiles allocated
    // pinned staging of the per-launch control state
    char* h_init = nullptr;    // BCtl | act_real | act_pref | real_done | TState[n_tiles]
    size_t init_bytes = 0;
    size_t off_ar = 0, off_ap = 0, off_rd = 0, off_ts = 0;  // offsets in h_init (16-byte aligned)
    BCtl* h_ctl = nullptr;     // the control block inside h_init
    BCtl* h_res = nullptr;     // pinned copy of the control block after a launch
    // launch shape
    ogs_batch_tuning tune{};
    int n_tiles = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = -1;      // max_steps captured in the graph
    double kloc[64];
    double* d_kloc = nullptr;
};

namespace {

int sm_count_dev()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 152;
}

// local Laplace matrix of a box cell in corner-bit order (corner c at
// (c & 1, c >> 1 & 1, c >> 2)): the trilinear element integrates exactly
// to sum over axes of K1 (x) M1 (x) M1 with K1 = [[1,-1],[-1,1]] / h and
// M1 = [[2,1],[1,2]] h / 6
void local_laplace(double hx, double hy, double hz, double tuf, double* k)
{
    const double h[3] = {hx, hy, hz};
    for (int a = 0; a < 8; a++)
        for (int b = 0; b < 8; b++)
        {
            double s = 0.0;
            for (int ax = 0; ax < 3; ax++)
            {
                double t = 1.0;
                for (int c = 0; c < 3; c++)
                {
                    const bool same = ((a >> c) & 1) == ((b >> c) & 1);
                    t *= c == ax ? (same ? 1.0 : -1.0) / h[c] : h[c] / 6.0 * (same ? 2.0 : 1.0);
                }
                s += t;
            }
            k[a * 8 + b] = s * tuf;
        }
}

ogs_status layout_tiles(ogs_batch* B, int tile_rows)
{
    std::vector<BTile> tiles;
    for (int r = 0; r < B->n_real; r++)
    {
        BReal& R = B->real[r];
        R.tile0 = (int)tiles.size();
        for (int i0 = 0; i0 < R.n; i0 += tile_rows)
            tiles.push_back({r, i0, std::min(R.n, i0 + tile_rows), 0});
        R.ntiles = (int)tiles.size() - R.tile0;
    }
    const int nt = (int)tiles.size();
    if (nt > B->tile_cap)
    {
        cudaFree(B->d_tiles);
        cudaFree(B->ts);
        cudaFree(B->part);
        B->d_tiles = nullptr;
        B->ts = nullptr;
        B->part = nullptr;
        OGS_CUDA_TRY(cudaMalloc(&B->d_tiles, nt * sizeof(BTile)));
        OGS_CUDA_TRY(cudaMalloc(&B->ts, nt * sizeof(TState)));
        OGS_CUDA_TRY(cudaMalloc(&B->part, (size_t)nt * 4 * sizeof(double)));
        B->tile_cap = nt;
    }
    B->n_tiles = nt;
    OGS_CUDA_TRY(cudaMemcpy(B->d_tiles, tiles.data(), nt * sizeof(BTile), cudaMemcpyHostToDevice));
    OGS_CUDA_TRY(cudaMemcpy(B->d_real, B->real.data(), B->n_real * sizeof(BReal), cudaMemcpyHostToDevice));
    // launch-time initial state: control block, full active list, no
    // realisation done, every tile at its first residual replacement
    if (B->h_init) cudaFreeHost(B->h_init);
    B->h_init = nullptr;
    const size_t nr = B->n_real;
    auto al = [](size_t v) { return (v + 15) & ~size_t(15); };
    B->off_ar = al(sizeof(BCtl));
    B->off_ap = B->off_ar + al(sizeof(int) * nr);
    B->off_rd = B->off_ap + al(sizeof(int) * (nr + 1));
    B->off_ts = B->off_rd + al(sizeof(int) * nr);
    B->init_bytes = B->off_ts + sizeof(TState) * nt;
    OGS_CUDA_TRY(cudaMallocHost(&B->h_init, B->init_bytes));
    std::memset(B->h_init, 0, B->init_bytes);
    BCtl* c = (BCtl*)B->h_init;
    int* ar = (int*)(B->h_init + B->off_ar);
    int* ap = (int*)(B->h_init + B->off_ap);
    int acc = 0;
    for (size_t r = 0; r < nr; r++)
    {
        ar[r] = (int)r;
        ap[r] = acc;
        acc += B->real[r].ntiles;
    }
    ap[nr] = acc;
    c->n_act = (int)nr;
    c->n_act_tiles = acc;
    c->seen_done = 0;
    TState* ts = (TState*)(B->h_init + B->off_ts);
    for (int t = 0; t < nt; t++)
    {
        ts[t].scale = 1.0;
        ts[t].ratio = 1.0;
        ts[t].rmax = -1.0;
        ts[t].bnorm = 1.0;
        ts[t].mode = kModeReplace;
        ts[t].first = 1;
        ts[t].status = OGS_NOT_CONVERGED;
    }
    B->h_ctl = c;
    return OGS_OK;
}

BatchArgs make_args(ogs_batch* B)
{
    BatchArgs a;
    std::memset(&a, 0, sizeof a);
    a.real = B->d_real;
    a.tiles = B->d_tiles;
    a.n_real = B->n_real;
    a.n_tiles = B->n_tiles;
    a.ek = B->ek;
    a.U64 = B->U64; a.b = B->b; a.x64 = B->x64; a.r64 = B->r64;
    a.U32 = B->U32; a.x32 = B->x32; a.r32 = B->r32; a.p32 = B->p32; a.s32 = B->s32; a.u32 = B->u32;
    a.w32 = B->w32; a.d32 = B->d32;
    a.ts = B->ts;
    a.part = B->part;
    a.ctl = B->ctl;
    a.act_real = B->act_real;
    a.act_pref = B->act_pref;
    a.real_done = B->real_done;
    a.out = B->out;
    a.tol = B->cfg.tol;
    a.delta = B->cfg.inner_tol > 0.0 ? B->cfg.inner_tol : 1e-2;
    a.max_iter = B->cfg.max_iter;
    a.kloc = B->d_kloc;
    return a;
}

int max_blocks_per_sm(int threads)
{
    int n = 0;
    cudaError_t e = threads == 512 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<512>, 512, 0)
                                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<256>, 256, 0);
    if (e != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}

// initial state copies and the cooperative launch, on B->stream
cudaError_t enqueue(ogs_batch* B, int max_steps)
{
    B->h_ctl->max_steps = max_steps;
    const size_t nr = B->n_real;
    const char* h = B->h_init;
    const cudaMemcpyKind k = cudaMemcpyHostToDevice;
    cudaError_t e = cudaMemcpyAsync(B->ctl, h, sizeof(BCtl), k, B->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B->act_real, h + B->off_ar, sizeof(int) * nr, k, B->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B->act_pref, h + B->off_ap, sizeof(int) * (nr + 1), k, B->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B->real_done, h + B->off_rd, sizeof(int) * nr, k, B->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B->ts, h + B->off_ts, sizeof(TState) * B->n_tiles, k, B->stream);
    if (e != cudaSuccess) return e;
    BatchArgs a = make_args(B);
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(B->tune.blocks_per_sm * sm_count_dev());
    lc.blockDim = dim3(B->tune.block_threads);
    lc.stream = B->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    if (B->tune.block_threads == 512) return cudaLaunchKernelEx(&lc, k_batch<512>, a);
    return cudaLaunchKernelEx(&lc, k_batch<256>, a);
}

void drop_graph(ogs_batch* B)
{
    if (B->graph) cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
    B->graph_steps = -1;
}

// one launch (graph when it can be captured); waits for it
ogs_status run(ogs_batch* B, int max_steps, float* ms)
{
    cudaEvent_t e0, e1;
    OGS_CUDA_TRY(cudaEventCreate(&e0));
    OGS_CUDA_TRY(cudaEventCreate(&e1));
    if (B->graph_steps != max_steps)
    {
        drop_graph(B);
        cudaGraph_t g = nullptr;
        bool ok = cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok)
        {
            const cudaError_t le = enqueue(B, max_steps);
            const cudaError_t ce = cudaStreamEndCapture(B->stream, &g);
            ok = le == cudaSuccess && ce == cudaSuccess && g &&
                 cudaGraphInstantiate(&B->graph, g, 0) == cudaSuccess;
            if (g) cudaGraphDestroy(g);
        }
        if (!ok)
        {
            cudaGetLastError();
            B->graph = nullptr;
        }
        B->graph_steps = ok ? max_steps : -1;
        B->tune.graph = ok ? 1 : 0;
    }
    OGS_CUDA_TRY(cudaEventRecord(e0, B->stream));
    if (B->graph)
    {
        OGS_CUDA_TRY(cudaGraphLaunch(B->graph, B->stream));
    }
    else
    {
        const cudaError_t le = enqueue(B, max_steps);
        if (le != cudaSuccess)
        {
            set_error("batch: launch failed: %s", cudaGetErrorString(le));
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return OGS_CUDA_ERROR;
        }
    }
    count_launches(1);
    OGS_CUDA_TRY(cudaEventRecord(e1, B->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(B->h_res, B->ctl, sizeof(BCtl), cudaMemcpyDeviceToHost, B->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(B->stream));
    if (ms) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return OGS_OK;
}

}  // namespace

extern "C" ogs_status ogs_gpu_batch_destroy(ogs_batch* B)
{
    if (!B) return OGS_OK;
    if (B->stream) cudaStreamSynchronize(B->stream);
    drop_graph(B);
    cudaFree(B->d_real);
    cudaFree(B->d_tiles);
    cudaFree(B->ek);
    cudaFree(B->U64);
    cudaFree(B->b);
    cudaFree(B->x64);
    cudaFree(B->r64);
    cudaFree(B->f32);
    cudaFree(B->ts);
    cudaFree(B->part);
    cudaFree(B->ctl);
    cudaFree(B->act_real);
    cudaFree(B->act_pref);
    cudaFree(B->real_done);
    cudaFree(B->out);
    cudaFree(B->d_kloc);
    if (B->h_init) cudaFreeHost(B->h_init);
    if (B->h_res) cudaFreeHost(B->h_res);
    if (B->own_stream && B->stream) cudaStreamDestroy(B->stream);
    delete B;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_batch_create(const ogs_batch_config* cfg, const ogs_batch_realisation* reals,
                                           int32_t n_real, void* stream, ogs_batch** out)
{
    if (!cfg || !reals || !out || n_real <= 0) { set_error("batch_create: bad arguments"); return OGS_BAD_ARG; }
    *out = nullptr;
    if (!(cfg->hx > 0 && cfg->hy > 0 && cfg->hz > 0) || !(cfg->tol >= 0.0) || cfg->max_iter < 0 ||
        !(cfg->time_unit_factor != 0.0))
    {
        set_error("batch_create: bad configuration");
        return OGS_BAD_ARG;
    }
    int dev = 0, coop = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) { set_error("batch_create: device has no cooperative launch"); return OGS_CUDA_ERROR; }
    ogs_batch* B = new ogs_batch;
    B->cfg = *cfg;
    B->n_real = n_real;
    local_laplace(cfg->hx, cfg->hy, cfg->hz, cfg->time_unit_factor, B->kloc);
    B->real.resize(n_real);
    int64_t rows = 0, elems = 0;
    for (int r = 0; r < n_real; r++)
    {
        const ogs_batch_realisation& q = reals[r];
        if (q.nx < 3 || q.ny < 3 || q.nz < 3 || !q.elem_k ||
            (int64_t)q.nx * q.ny * q.nz >= (int64_t(1) << 31) / 14)
        {
            delete B;
            set_error("batch_create: realisation %d: need 3 <= nodes per axis and elem_k", r);
            return OGS_BAD_ARG;
        }
        BReal& R = B->real[r];
        R.nx = q.nx; R.ny = q.ny; R.nz = q.nz;
        R.n = q.nx * q.ny * q.nz;
        R.row0 = rows;
        R.elem0 = elems;
        R.h_left = q.h_left;
        R.h_right = q.h_right;
        rows += R.n;
        elems += (int64_t)(q.nx - 1) * (q.ny - 1) * (q.nz - 1);
    }
    B->rows = rows;
    B->elems = elems;
    if (stream)
        B->stream = (cudaStream_t)stream;
    else
    {
        if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess)
        {
            delete B;
            set_error("batch_create: stream creation failed");
            return OGS_CUDA_ERROR;
        }
        B->own_stream = true;
    }
    const size_t v4 = ((size_t)rows * sizeof(float) + 255) & ~size_t(255);
    cudaError_t e = cudaMalloc(&B->d_real, n_real * sizeof(BReal));
    if (e == cudaSuccess) e = cudaMalloc(&B->ek, elems * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&B->U64, (size_t)rows * 14 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&B->b, rows * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&B->x64, rows * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&B->r64, rows * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&B->f32, 14 * v4 + 7 * v4);
    if (e == cudaSuccess) e = cudaMalloc(&B->ctl, sizeof(BCtl));
    if (e == cudaSuccess) e = cudaMalloc(&B->act_real, n_real * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&B->act_pref, (n_real + 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&B->real_done, n_real * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&B->out, n_real * sizeof(ogs_batch_stats));
    if (e == cudaSuccess) e = cudaMallocHost(&B->h_res, sizeof(BCtl));
    if (e == cudaSuccess) e = cudaMalloc(&B->d_kloc, sizeof B->kloc);
    if (e == cudaSuccess) e = cudaMemcpy(B->d_kloc, B->kloc, sizeof B->kloc, cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        set_error("batch_create: %s (%lld rows)", cudaGetErrorString(e), (long long)rows);
        ogs_gpu_batch_destroy(B);
        return e == cudaErrorMemoryAllocation ? OGS_OOM : OGS_CUDA_ERROR;
    }
    char* f = (char*)B->f32;
    B->U32 = (float*)f;
    f += 14 * v4;
    float** vs[] = {&B->x32, &B->r32, &B->p32, &B->s32, &B->u32, &B->w32, &B->d32};
    for (float** v : vs) { *v = (float*)f; f += v4; }
    for (int r = 0; r < n_real; r++)
    {
        const BReal& R = B->real[r];
        const size_t ne = (size_t)(R.nx - 1) * (R.ny - 1) * (R.nz - 1);
        e = cudaMemcpyAsync(B->ek + R.elem0, reals[r].elem_k, ne * sizeof(double), cudaMemcpyDefault, B->stream);
        if (e != cudaSuccess)
        {
            set_error("batch_create: copying elem_k of realisation %d: %s", r, cudaGetErrorString(e));
            ogs_gpu_batch_destroy(B);
            return OGS_CUDA_ERROR;
        }
    }
    // the caller may release its arrays when this returns
    if ((e = cudaStreamSynchronize(B->stream)) != cudaSuccess)
    {
        set_error("batch_create: %s", cudaGetErrorString(e));
        ogs_gpu_batch_destroy(B);
        return OGS_CUDA_ERROR;
    }
    // default launch shape; ogs_gpu_batch_autotune refines it
    B->tune.tile_rows = 4096;
    B->tune.block_threads = 256;
    B->tune.blocks_per_sm = std::max(1, std::min(4, max_blocks_per_sm(256)));
    ogs_status st = layout_tiles(B, B->tune.tile_rows);
    if (st) { ogs_gpu_batch_destroy(B); return st; }
    *out = B;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_batch_set_k(ogs_batch* B, const double* k)
{
    if (!B || !k) { set_error("batch_set_k: NULL argument"); return OGS_BAD_ARG; }
    OGS_CUDA_TRY(cudaMemcpyAsync(B->ek, k, B->elems * sizeof(double), cudaMemcpyDefault, B->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(B->stream));
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_batch_set_tuning(ogs_batch* B, const ogs_batch_tuning* t)
{
    if (!B || !t) { set_error("batch_set_tuning: NULL argument"); return OGS_BAD_ARG; }
    if ((t->block_threads != 256 && t->block_threads != 512) || t->tile_rows < 32 || t->blocks_per_sm < 1)
    {
        set_error("batch_set_tuning: block_threads 256|512, tile_rows >= 32, blocks_per_sm >= 1");
        return OGS_BAD_ARG;
    }
    const int occ = max_blocks_per_sm(t->block_threads);
    if (t->blocks_per_sm > occ)
    {
        set_error("batch_set_tuning: %d blocks of %d threads per SM do not fit (at most %d)", t->blocks_per_sm,
                  t->block_threads, occ);
        return OGS_BAD_ARG;
    }
    drop_graph(B);
    B->tune.tile_rows = t->tile_rows;
    B->tune.block_threads = t->block_threads;
    B->tune.blocks_per_sm = t->blocks_per_sm;
    B->tune.ms_per_step = t->ms_per_step;
    return layout_tiles(B, t->tile_rows);
}

extern "C" ogs_status ogs_gpu_batch_autotune(ogs_batch* B, ogs_batch_tuning* chosen)
{
    if (!B) { set_error("batch_autotune: NULL batch"); return OGS_BAD_ARG; }
    // per-step time from two launches of different length (the assembly
    // and the first replacement cancel); every realisation stays active
    // for this many steps unless it converges sooner
    const int s_short = 4, s_long = 16;
    ogs_batch_tuning best{};
    double best_ms = 1e300;
    const int tiles[] = {2048, 4096, 8192};
    const int threads[] = {256, 512};
    for (int nt : threads)
    {
        const int occ = max_blocks_per_sm(nt);
        for (int bps = 1; bps <= std::min(occ, 4); bps++)
            for (int tr : tiles)
            {
                ogs_batch_tuning t{};
                t.tile_rows = tr;
                t.block_threads = nt;
                t.blocks_per_sm = bps;
                ogs_status st = ogs_gpu_batch_set_tuning(B, &t);
                if (st) return st;
                float m1 = 0.f, m2 = 0.f;
                if ((st = run(B, s_short, &m1))) return st;  // also warms the graph
                if ((st = run(B, s_short, &m1))) return st;
                if (B->h_res->err) { set_error("batch_autotune: grid barrier timed out"); return OGS_CUDA_ERROR; }
                if ((st = run(B, s_long, &m2))) return st;
                if ((st = run(B, s_long, &m2))) return st;
                if (B->h_res->err) { set_error("batch_autotune: grid barrier timed out"); return OGS_CUDA_ERROR; }
                drop_graph(B);
                const int steps = B->h_res->step - s_short;
                const double per = steps > 0 ? (m2 - m1) / steps : 1e300;
                if (per < best_ms)
                {
                    best_ms = per;
                    best = t;
                    best.ms_per_step = per;
                }
            }
    }
    if (best.tile_rows == 0) { set_error("batch_autotune: no launch shape fits"); return OGS_CUDA_ERROR; }
    ogs_status st = ogs_gpu_batch_set_tuning(B, &best);
    if (st) return st;
    if (chosen) *chosen = B->tune;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_batch_solve(ogs_batch* B, ogs_batch_stats* stats)
{
    if (!B) { set_error("batch_solve: NULL batch"); return OGS_BAD_ARG; }
    // bound on the persistent loop: every realisation converges or hits
    // max_iter within this many steps (each replacement redoes one step)
    const int max_steps = 4 * B->cfg.max_iter + 64;
    ogs_status st = run(B, max_steps, nullptr);
    if (st) return st;
    const BCtl& c = *B->h_res;
    if (c.err)
    {
        set_error("batch_solve: grid barrier timed out");
        return OGS_CUDA_ERROR;
    }
    std::vector<ogs_batch_stats> o(B->n_real);
    std::vector<int> done(B->n_real);
    OGS_CUDA_TRY(cudaMemcpy(o.data(), B->out, B->n_real * sizeof(ogs_batch_stats), cudaMemcpyDeviceToHost));
    OGS_CUDA_TRY(cudaMemcpy(done.data(), B->real_done, B->n_real * sizeof(int), cudaMemcpyDeviceToHost));
    ogs_status ret = OGS_OK;
    for (int r = 0; r < B->n_real; r++)
    {
        if (!done[r])
        {
            std::memset(&o[r], 0, sizeof o[r]);
            o[r].status = OGS_NOT_CONVERGED;
        }
        if (o[r].status != OGS_OK && ret == OGS_OK) ret = (ogs_status)o[r].status;
    }
    if (stats) std::memcpy(stats, o.data(), B->n_real * sizeof(ogs_batch_stats));
    if (ret != OGS_OK) set_error("batch_solve: some realisations did not converge");
    return ret;
}

extern "C" ogs_status ogs_gpu_batch_get_heads(const ogs_batch* B, double* h)
{
    if (!B || !h) { set_error("batch_get_heads: NULL argument"); return OGS_BAD_ARG; }
    OGS_CUDA_TRY(cudaStreamSynchronize(B->stream));
    OGS_CUDA_TRY(cudaMemcpyAsync(h, B->x64, B->rows * sizeof(double), cudaMemcpyDefault, B->stream));
    OGS_CUDA_TRY(cudaStreamSynchronize(B->stream));
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_batch_info(const ogs_batch* B, int64_t* rows, int64_t* elements)
{
    if (!B) { set_error("batch_info: NULL batch"); return OGS_BAD_ARG; }
    if (rows) *rows = B->rows;
    if (elements) *elements = B->elems;
    return OGS_OK;
}
