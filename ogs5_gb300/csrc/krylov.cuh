// krylov.cuh -- device-resident Krylov solver state shared by the kernels.
#pragma once

#include "common.cuh"

namespace ogs {

// Scalars of one solve, kept on the device; every kernel reads them, the
// last block of each reduction kernel writes them (Linear_EQS members
// bNorm, error, iter and the CG/BiCGStab locals).
struct KState
{
    double bnorm, tol, error;
    double rr;                   // CG: r . M^-1 r
    double alpha, beta, omega, rho0, rho1;
    double pdot;                 // spare
    int iter, max_iter, done, status;
    int finish_s;                // BiCGStab left at the s-test (x += alpha p_h pending)
    int pad;
    // FP32 inner CG with FP64 residual replacement
    double scale;                // r32 = scale * r64 (scale = 1 / |r64| at the last replacement)
    double ratio;                // scale_new / scale_old at a replacement
    double rmax;                 // |r32| right after the last replacement
    double delta;                // replace when |r32| < delta * rmax
    int replace;                 // 1: the FP64 residual replacement is due
    int replacements;
    int first;                   // first restart of a solve (p = z)
    int fallback;                // FP32 cycles stopped gaining: finish in FP64 CG
    double err_prev;             // |r64| / |b| at the previous replacement
    double rn_req;               // |r32| when the pending replacement was asked for
    double rbest[2];             // smallest |r32| of the cycle up to iteration k, at [k & 1]
    int itbest[2];               // the iteration where it was reached, at [k & 1]
    int stalled;                 // the pending replacement was forced by a plateau
    int pad4;
    // ticket-free CG: r.z of the iteration after `base_iter` comes from
    // rz_base (initial residual or the last replacement), later ones from
    // the parity-buffered partials of the update kernel
    double rz_base;
    double rz_hist[2];           // r.z of iteration k at [k & 1], written by block 0 of the p kernel
    double gam_hist[2], eta_hist[2];  // FP32 CG (Chronopoulos-Gear): gamma, eta of iteration k at [k & 1]
    int base_iter;
    int nb_spmv, nb_upd;         // producer grid sizes (partials to add)
    int pad3;
    // grid barrier of the persistent FP32 CG kernel (reset with the header)
    unsigned int bar_count, bar_gen;
    int bar_err, pad5;
    double est_unit;             // |r64| / |b| estimate = est_unit * |r32| (set at each replacement)
    unsigned int ticket[8];
    double part[8][2 * kMaxBlocks];
    double cg_ps[3 * kMaxBlocks];        // per SpMV block: p . s (FP64 CG); r.u, w.u, r.r (FP32 CG)
    double cg_upd[2][2 * kMaxBlocks];    // r . r and r . z per update block, by parity
};

enum SolveKind
{
    SK_CG = 0,
    SK_BICGSTAB = 1
};

// SELL-32 view of the matrix in the precision of the sweep.
template <typename T>
struct SellView
{
    const int32_t* slice_ptr;
    const int32_t* col;
    const T* val;
    int32_t n;
};

struct KrylovVecs
{
    double *x, *b, *r, *r0, *p, *ph, *s, *sh, *t, *v, *dinv;
};

// ILU(0) factors on the CSR pattern (unit lower L below the diagonal, U on
// and above it, in place) and the dependency levels of the two sweeps: the
// rows of a level depend only on rows of earlier levels.
struct IluView
{
    const int32_t* row_ptr;
    const int32_t* col;
    const int32_t* diag;      // CSR position of the diagonal
    double* lu;
    const int32_t* lrows;     // rows by forward level, levels padded to 32 with -1
    const int32_t* urows;     // rows by backward level, the same
    int n, n_lpos, n_upos;
    int* flags;               // [3][n]: launch number with which a row was published
                              // (factorisation, forward, backward sweep)
    unsigned long long* ticket;  // [3] block tickets handed out so far, per kernel
    int* bad;                 // smallest row with a zero pivot (factorisation);
                              // -1: a sweep gave up waiting
    unsigned spin;            // polls of one wait before it gives up (0: the default)
    double* rdiag;            // [n] 1 / u_ii of each factored row (published with the row)
    // the sweeps' rows packed by position (level order, padded levels):
    // level starts, the row (-1: padding or no diagonal), and the row's L
    // (forward) or U (backward) entries as columns / values [k][pos]
    // (column -1 past the row's entries), the reciprocal of the diagonal for
    // the backward sweep
    const int32_t* lptr;      // [n_lev + 1]
    const int32_t* uptr;      // [n_ulev + 1]
    int n_lev, n_ulev;
    int kl, ku;               // entries per row in the packed arrays
    int32_t *pl_row, *pl_col, *pu_row, *pu_col;
    double *pl_val, *pu_val, *pu_diag;
    // lattice tiles (ogs_mesh::tiles; 0: the level kernels sweep): per tile
    // and its 8 z layers the 64 rows (x, y) of a layer, their entries by
    // neighbour slot (forward: the 7 neighbours at offsets in {-1, 0}^3,
    // backward: in {0, 1}^3, each in ascending column order) and a mask
    // (bit s: slot s is an entry of the row; bit 7: the row exists and has
    // a diagonal)
    int tiles, lnx, lny, lnz, tnx, tny, tnz;
    const int32_t* tile_order;       // [tiles] by the sum of the tile coordinates
    int* tile_flags;                 // [3][tiles] launch number of the forward / backward sweep's and the
                                     // factorisation's publication
    unsigned long long* tile_ticket; // [3]
    double *tl_val, *tu_val;         // [tiles][8][7][64]
    double* tu_dg;                   // [tiles][8][64] 1 / U_ii
    double* tu_piv;                  // [tiles][8][64] U_ii
    int32_t* t_rb;                   // [tiles][8][64] CSR start of the row (-1: none)
    unsigned char *tl_mask, *tu_mask;  // [tiles][8][64]
};

struct SolveArgs
{
    SellView<double> A;
    KrylovVecs v;
    KState* st;
    int precond;  // OGS_PRECOND_NONE / JACOBI / ILU0
    IluView ilu;
};

// ------------------------------------------------------------------
// Grid-wide sums.  Each block reduces its threads' values and stores one
// partial per value; the last block to take a ticket adds the partials of
// all blocks with all of its threads (block order fixed by the strided
// loop and the tree, so the result is deterministic for a launch shape)
// and resets the ticket.  FP32 inputs are reduced in FP32 inside a warp
// (cheap FADDs) and in FP64 from the warp sums on.
// ------------------------------------------------------------------
template <int NV, typename T>
__device__ __forceinline__ void warp_allsum(T* v)
{
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// returns true in every thread of the last block; out[] valid in thread 0
template <int NV, typename T>
__device__ __forceinline__ bool grid_sum(const T* vin, double* out, double* part, unsigned int* ticket)
{
    __shared__ double sm[NV][kThreads / 32];
    __shared__ bool last;
    T w[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) w[k] = vin[k];
    warp_allsum<NV, T>(w);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sm[k][wid] = (double)w[k];
    __syncthreads();
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < NV; k++)
        {
            double s = 0.0;
            for (int q = 0; q < nw; q++) s += sm[k][q];
            part[k * kMaxBlocks + blockIdx.x] = s;
        }
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; k++)
    {
        double s = 0.0;
        for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x)
            s += *((volatile double*)&part[k * kMaxBlocks + q]);
        v[k] = s;
    }
    warp_allsum<NV, double>(v);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sm[k][wid] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < NV; k++)
        {
            double s = 0.0;
            for (int q = 0; q < nw; q++) s += sm[k][q];
            out[k] = s;
        }
        *ticket = 0u;
    }
    return true;
}

// ------------------------------------------------------------------
// Ticket-free grid sums for the CG kernels.  A producer kernel only writes
// one partial per block and value (write_partials); every block of the
// consumer kernel adds the partials itself, in the same fixed order
// (reduce_partials_warp / _bcast), so all blocks hold bitwise the same total without a
// last-block step or atomics.  Partial buffers are double-buffered by
// iteration parity where a kernel reads last iteration's sums.
// ------------------------------------------------------------------
// One warp adds nb partials per value in FP64 (each lane a strided share,
// then the lanes): GB300's FP64 rate makes FP64 work of the whole block
// cost ~8x the cycles of one warp's.  out[] valid in every lane of warp 0;
// the other warps leave at once.
template <int NV>
__device__ __forceinline__ bool reduce_partials_warp(const double* part, int nb, double* out)
{
    if (threadIdx.x >= 32) return false;
#pragma unroll
    for (int k = 0; k < NV; k++)
    {
        double s = 0.0;
        for (int q = threadIdx.x; q < nb; q += 32) s += __ldcg(part + k * kMaxBlocks + q);
        out[k] = s;
    }
    warp_allsum<NV, double>(out);
    return true;
}

// reduce_partials_warp for a whole block: warp 0 adds, the totals reach
// every thread through shared memory
template <int NV>
__device__ __forceinline__ void reduce_partials_bcast(const double* part, int nb, double* out)
{
    __shared__ double sm[NV];
    double v[NV];
    if (reduce_partials_warp<NV>(part, nb, v) && threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sm[k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = sm[k];
}

template <int NV, typename T>
__device__ __forceinline__ void write_partials(const T* vin, double* part)
{
    __shared__ double sm[NV][kThreads / 32];
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
            for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sm[k][q];
            part[k * kMaxBlocks + blockIdx.x] = s;
        }
}

// out[k] = sum of part[k * kMaxBlocks + 0 .. nb-1], identical in every thread

// cp.async.bulk.prefetch.L2 of [p, p + bytes), widened to 16-byte
// boundaries (the instruction's alignment rule) and clipped to [lo, hi)
__device__ __forceinline__ void bulk_prefetch_l2(const void* p, size_t bytes, const void* lo, const void* hi)
{
    size_t b = (size_t)p & ~(size_t)15;
    size_t e = ((size_t)p + bytes + 15) & ~(size_t)15;
    const size_t l = ((size_t)lo + 15) & ~(size_t)15, h = (size_t)hi & ~(size_t)15;
    if (b < l) b = l;
    if (e > h) e = h;
    if (e > b) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b), "r"((unsigned)(e - b)) : "memory");
}

// Arguments of the FP32-inner / FP64-refinement kernels (mixed.cu).
struct MixedArgs
{
    SellView<double> A;       // FP64 matrix
    int fmt;                  // 0: diagonal-offset upper half, 1: SELL-32 FP32
    const float* U;           // [n_up][ustride]
    int ustride;              // values per U row (a multiple of 32: every row starts on a 128-byte line);
                              // U[d] = U + d * ustride, zero pads before [0, n) and after it
    int lines;                // four rows per thread (k_mp_spmv_lines): 1 the 27-point lattice, 2 the 9-point
                              // plane lattice; 0 the row kernel
    int pad;                  // zero values in front of each U row and FP32 vector (n + pad + 64 behind)
    const int32_t* up_off;    // [n_up]
    int n_up;
    int off[16];              // up_off by value (diagonal-offset kernels)
    const float* val32;       // SELL-32 FP32 values
    const float* d32;         // Jacobi inverse (preconditioned form) or the scale 1 / sqrt(a_ii), FP32
    int scaled;               // 1: CG on D^-1/2 A D^-1/2 (the iterate u is r itself)
    double* x;                // FP64 solution
    const double* b;
    double* r64;
    float *x32, *r32, *p32, *s32, *u32, *w32;
    KState* st;
    int n;
    int nb_spmv;              // blocks of the product (partials to add)
    // fmt 2: operator from one coefficient per cell of a regular hex lattice
    int gx, gy, gz;
    const float* mf_alpha;          // [cells] Laplace coefficient
    const float* mf_beta;           // mass coefficient (one value)
    const unsigned char* mf_mask;   // [n] bit 0: Dirichlet row, bit 1: column eliminated
    const float* mf_dbc;            // [n] kept diagonal of Dirichlet rows
    float mf_L[8], mf_M[8];         // box Laplace / mass entries by corner-equality pattern
    float mf_m1[6];                 // 1-D mass entries per axis: (x: same, other), (y: ...), (z: ...)
};

}  // namespace ogs
