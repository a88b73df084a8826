// ilu.cu -- ILU(0) preconditioner (ls_precond 100): factorisation on the
// CSR pattern and the forward/backward sweeps of (LU) z = r.
//
// The SP build's Linear_EQS::ConfigNumerics maps precond 100 to Jacobi
// ("ILU not available", FEM/equation_class.cpp:294-308); the legacy
// RF-solver build factors an incomplete LDU on its own storage
// (M34Vorkond, FEM/matrix_routines.cpp:3271-3427).  This file gives the
// textbook ILU(0) in natural row order: IKJ elimination restricted to the
// CSR pattern, unit lower L and U stored in place.
//
// GPU form.  Row i of either sweep, and of the factorisation, only reads
// rows that come earlier in the sweep's dependency order, so rows are
// grouped into levels (rows of a level are independent; computed once per
// mesh on the host).  A structured grid in natural order has
// nx + ny + nz levels (Kuhn tets) or about nx + 2 ny + 4 nz (27-point
// hexes): hundreds of levels of a few thousand rows each.  The whole GPU
// walks them in one launch per sweep without grid-wide barriers: the rows
// lie in level order (each level padded to whole warps); a persistent grid
// of blocks takes consecutive ranges of them from a ticket counter; one
// thread per row polls the flags of the rows its row reads (relaxed loads,
// backing off), takes one acquire fence, computes, and publishes its value
// with a release store of its flag (the launch number).  A block waits only
// on ranges taken earlier, by blocks that are resident and do not wait on
// later ranges, so the sweep cannot deadlock; a warp holds one level, so no
// lane waits on a lane of its warp.  Every wait polls at most kIluSpin
// times and then records -1 in f.bad and goes on (the host reports the
// solve as failed).  That is the factorisation's kernel (the most FP64
// work per row, which needs the whole GPU's FP64 units).
//
// The sweeps do little work per row, so a level costs what its dependent
// loads cost.  After each factorisation the rows' L and U entries are
// packed by sweep position (k_ilu_pack); one thread-block cluster (16 CTAs
// where the device allows, else 8) walks the levels, the threads of a level
// holding their rows' packed entries in registers: a level is one
// dependent L2 round trip (the neighbours' results) between two halves of
// the cluster barrier, and the next level's entries are loaded while the
// barrier completes.
//
// Lattice patterns whose lower columns lie at no larger x, y, z than their
// row (Kuhn tets in lattice order: ogs_mesh::tiles) take a third form for
// the factorisation and both sweeps: tiles of 8^3 rows in the order of the
// sum of their tile coordinates, the rows of a tile in 22 steps of
// lx + ly + lz from shared memory (k_ilu_factor_tiles, k_ilu_tiles below).
// Every form does the same arithmetic per row, so all give bit for bit the
// same factors and sweep results.
#include <algorithm>
#include <cstring>
#include <vector>

#include "krylov.cuh"

namespace ogs {

constexpr int kIluBlock = 128;          // rows (positions) per ticket and block
constexpr int kIluBlocksPerSm = 4;      // persistent grid
constexpr unsigned kIluSpin = 1u << 18;  // polls of one wait before it gives up
constexpr int kIluRowMax = 32;          // factorisation: rows held in a local array
constexpr int kIluUMax = 16;            // U entries of a pivot row loaded per batch

// lu = A on the CSR pattern (values live in SELL-32 order)
__global__ void k_ilu_copy(const double* __restrict__ val, const int32_t* __restrict__ csr2sell,
                           double* __restrict__ lu, int64_t nnz)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
        lu[k] = val[csr2sell[k]];
}

__device__ __forceinline__ int ld_relaxed_s32(const int* p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_s32(int* p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// until row j is published by this launch (relaxed polls with a growing
// pause, bounded; once any wait of the launch has given up, f.bad is -1
// and the others stop waiting too).  The caller takes the acquire fence
// after all its waits.
__device__ __forceinline__ void ilu_wait(const int* flags, int j, int launch, int* bad, unsigned limit,
                                         unsigned max_pause = 512u)
{
    if (ld_relaxed_s32(flags + j) >= launch) return;
    unsigned spins = 0, pause = 32;
    while (ld_relaxed_s32(flags + j) < launch)
    {
        if (++spins > limit || ((spins & 255) == 0 && *(volatile int*)bad == -1))
        {
            atomicMin(bad, -1);
            return;
        }
        __nanosleep(pause);
        pause = min(pause * 2, max_pause);
    }
}

// the tile kernels' waits: few waiting blocks (one per SM), each on the
// critical path of the sweep, so they poll at most 128 ns apart
constexpr unsigned kTilePause = 128u;

__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// l_ik = a_ik / u_kk in the elimination, from r = 1 / u_kk (one IEEE
// division per pivot row, done when that row is finished) by Markstein's
// division step: q = a r, the remainder e = a - u q exact by one FMA, then
// q + e r.  Two dependent FMAs after the product instead of a division on
// the row's dependent chain: GB300's FP64 units make each dependent FP64
// operation slow, and a row of the factorisation divides by up to 7 pivots
// in sequence.  The quotient is within rounding of a / u (every form of
// the factorisation uses this, so they agree bit for bit; the factors stay
// within 1e-12 of the oracle's IEEE divisions).
__device__ __forceinline__ double ilu_div(double a, double u, double r)
{
    const double q = __dmul_rn(a, r);
    const double e = __fma_rn(-q, u, a);
    return __fma_rn(e, r, q);
}

// one row of MODE 0 / 1 / 2 (below)
template <int MODE>
__device__ __forceinline__ void ilu_row(const IluView& f, const double* __restrict__ in, double* out, int* flags,
                                        int i, int launch, double (*s_a)[kIluBlock], int (*s_cj)[kIluBlock])
{
    const int rb = __ldg(f.row_ptr + i), re = __ldg(f.row_ptr + i + 1);
    const int d = __ldg(f.diag + i);
    if (d < 0)
    {
        // a node in no element has no diagonal: a zero pivot
        if (MODE == 0) atomicMin(f.bad, i);
        st_release_s32(flags + i, launch);
        return;
    }
    // the rows this row reads: its columns before (MODE 0, 1) or after
    // (MODE 2) the diagonal
    const int w0 = MODE == 2 ? d + 1 : rb, w1 = MODE == 2 ? re : d;
    for (int k = w0; k < w1; k++)
    {
        const int c = __ldg(f.col + k);
        if (OGS_IN(c, f.n, kOobIluCol)) ilu_wait(flags, c, launch, f.bad, f.spin ? f.spin : kIluSpin);
    }
    fence_acquire();
    if (MODE == 0 && re - rb <= kIluRowMax && f.ku <= kIluUMax)
    {
        // row i -= l_ik row k for every k < i of the pattern, in column
        // order; l_ik by ilu_div from row k's published reciprocal pivot,
        // products and differences rounded separately (no FMA), like the
        // sequential elimination.  Row i stays in shared memory for the
        // whole elimination (a column per thread); row k's U part is loaded
        // into registers in one batch, the next k's batch issued before this
        // one is used.
        const int len = re - rb, nlow = d - rb, t = threadIdx.x;
        for (int q = 0; q < len; q++)
        {
            s_cj[q][t] = __ldg(f.col + rb + q);
            s_a[q][t] = __ldcg(f.lu + rb + q);
        }
        int uc[kIluUMax], nc[kIluUMax];
        double uv[kIluUMax], nv[kIluUMax], piv = 0.0, npiv = 0.0, rpiv = 0.0, nrpiv = 0.0;
        auto fetch = [&](int kk, int* c, double* v, double& pv, double& rv) {
            const int k = s_cj[kk][t];
            const int dk = __ldg(f.diag + k), ke = __ldg(f.row_ptr + k + 1);
            pv = __ldcg(f.lu + dk);
            rv = __ldcg(f.rdiag + k);
#pragma unroll
            for (int q = 0; q < kIluUMax; q++)
            {
                const bool in = dk + 1 + q < ke;
                c[q] = in ? __ldg(f.col + dk + 1 + q) : 0x7fffffff;
                v[q] = in ? __ldcg(f.lu + dk + 1 + q) : 0.0;
            }
        };
        if (nlow > 0) fetch(0, uc, uv, piv, rpiv);
        for (int kk = 0; kk < nlow; kk++)
        {
            if (kk + 1 < nlow) fetch(kk + 1, nc, nv, npiv, nrpiv);
            if (piv == 0.0) atomicMin(f.bad, s_cj[kk][t]);
            const double lik = ilu_div(s_a[kk][t], piv, rpiv);
            s_a[kk][t] = lik;
            int p = kk + 1;
#pragma unroll
            for (int q = 0; q < kIluUMax; q++)
            {
                const int j = uc[q];
                while (p < len && s_cj[p][t] < j) p++;
                if (p < len && s_cj[p][t] == j) s_a[p][t] = __dsub_rn(s_a[p][t], __dmul_rn(lik, uv[q]));
            }
#pragma unroll
            for (int q = 0; q < kIluUMax; q++)
            {
                uc[q] = nc[q];
                uv[q] = nv[q];
            }
            piv = npiv;
            rpiv = nrpiv;
        }
        for (int q = 0; q < len; q++) __stcg(f.lu + rb + q, s_a[q][t]);
        if (s_a[nlow][t] == 0.0) atomicMin(f.bad, i);
        __stcg(f.rdiag + i, 1.0 / s_a[nlow][t]);
    }
    else if (MODE == 0)
    {
        // rows longer than the local array: the same elimination in place
        for (int kk = rb; kk < d; kk++)
        {
            const int k = __ldg(f.col + kk);
            const int dk = __ldg(f.diag + k), ke = __ldg(f.row_ptr + k + 1);
            const double piv = __ldcg(f.lu + dk);
            if (piv == 0.0) atomicMin(f.bad, k);
            const double lik = ilu_div(__ldcg(f.lu + kk), piv, __ldcg(f.rdiag + k));
            __stcg(f.lu + kk, lik);
            int p = kk + 1;
            for (int q = dk + 1; q < ke; q++)
            {
                const int j = __ldg(f.col + q);
                while (p < re && __ldg(f.col + p) < j) p++;
                if (p < re && __ldg(f.col + p) == j)
                    __stcg(f.lu + p, __dsub_rn(__ldcg(f.lu + p), __dmul_rn(lik, __ldcg(f.lu + q))));
            }
        }
        if (__ldcg(f.lu + d) == 0.0) atomicMin(f.bad, i);
        __stcg(f.rdiag + i, 1.0 / __ldcg(f.lu + d));
    }
    else if (MODE == 1)
    {
        double s = in[i];
        for (int k = rb; k < d; k++)
            s = __dsub_rn(s, __dmul_rn(__ldg(f.lu + k), __ldcg(out + __ldg(f.col + k))));
        __stcg(out + i, s);
    }
    else
    {
        double s = __ldcg(out + i);
        for (int k = d + 1; k < re; k++)
            s = __dsub_rn(s, __dmul_rn(__ldg(f.lu + k), __ldcg(out + __ldg(f.col + k))));
        __stcg(out + i, s / __ldg(f.lu + d));
    }
    st_release_s32(flags + i, launch);
}

// MODE 0: factorisation (IKJ, rows in forward levels)
// MODE 1: forward sweep  out_i = in_i - sum_{k<i} L_ik out_k
// MODE 2: backward sweep out_i = (out_i - sum_{j>i} U_ij out_j) / U_ii
// Persistent blocks take tickets until this launch's are used up: a launch
// hands out nblk + gridDim.x tickets (nblk ranges of kIluBlock positions,
// then one closing ticket per block), so the launch number follows from
// any ticket.  The sweeps return at once when the solve has finished
// (uniform over the grid: st->done is not written while this kernel runs,
// so either every block takes its tickets or none does).
template <int MODE>
__global__ void __launch_bounds__(kIluBlock) k_ilu_flow(IluView f, const double* __restrict__ in, double* out,
                                                       const KState* st)
{
    if (MODE != 0 && st->done) return;
    const int npos = MODE == 2 ? f.n_upos : f.n_lpos;
    const unsigned long long nblk = (unsigned long long)((npos + kIluBlock - 1) / kIluBlock);
    const unsigned long long per = nblk + gridDim.x;
    const int32_t* rows = MODE == 2 ? f.urows : f.lrows;
    int* flags = f.flags + (size_t)MODE * f.n;
    __shared__ unsigned long long s_ticket;
    // the factorisation's rows, a column per thread
    __shared__ double s_a[MODE == 0 ? kIluRowMax : 1][kIluBlock];
    __shared__ int s_cj[MODE == 0 ? kIluRowMax : 1][kIluBlock];
    for (;;)
    {
        __syncthreads();
        if (threadIdx.x == 0) s_ticket = atomicAdd(f.ticket + MODE, 1ull);
        __syncthreads();
        const unsigned long long t = s_ticket;
        const unsigned long long blk = t % per;
        if (blk >= nblk) return;  // this block's closing ticket
        const int launch = (int)(t / per) + 1;
        const int pos = (int)blk * kIluBlock + threadIdx.x;
        if (pos < npos)
        {
            const int i = __ldg(rows + pos);
            if (i >= 0) ilu_row<MODE>(f, in, out, flags, i, launch, s_a, s_cj);  // i < 0: padding of a level
        }
    }
}

// after a factorisation: the sweeps' rows packed by position (rows without
// a diagonal as -1: the factorisation has reported them)
__global__ void k_ilu_pack(IluView f)
{
    const int stride = gridDim.x * blockDim.x;
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < f.n_lpos; pos += stride)
    {
        int i = __ldg(f.lrows + pos);
        const int d = i >= 0 ? __ldg(f.diag + i) : -1;
        if (d < 0) i = -1;
        const int rb = i >= 0 ? __ldg(f.row_ptr + i) : 0;
        f.pl_row[pos] = i;
        for (int k = 0; k < f.kl; k++)
        {
            const bool in = i >= 0 && rb + k < d;
            f.pl_col[(size_t)k * f.n_lpos + pos] = in ? __ldg(f.col + rb + k) : -1;
            f.pl_val[(size_t)k * f.n_lpos + pos] = in ? f.lu[rb + k] : 0.0;
        }
    }
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < f.n_upos; pos += stride)
    {
        int i = __ldg(f.urows + pos);
        const int d = i >= 0 ? __ldg(f.diag + i) : -1;
        if (d < 0) i = -1;
        const int re = i >= 0 ? __ldg(f.row_ptr + i + 1) : 0;
        f.pu_row[pos] = i;
        f.pu_diag[pos] = i >= 0 ? 1.0 / f.lu[d] : 1.0;  // the sweep multiplies by it
        for (int k = 0; k < f.ku; k++)
        {
            const bool in = i >= 0 && d + 1 + k < re;
            f.pu_col[(size_t)k * f.n_upos + pos] = in ? __ldg(f.col + d + 1 + k) : -1;
            f.pu_val[(size_t)k * f.n_upos + pos] = in ? f.lu[d + 1 + k] : 0.0;
        }
    }
}

// One packed row: index, entries, start value (forward: in_i, backward:
// the forward result out_i), reciprocal of the diagonal (backward)
template <int K>
struct PackedRow
{
    int i;
    int c[K];
    double v[K];
    double s0, dg;
};

template <int MODE, int K>
__device__ __forceinline__ void ilu_fetch(const IluView& f, const double* __restrict__ in, const double* out,
                                          int pos, int npos, PackedRow<K>& R)
{
    const int32_t* prow = MODE == 2 ? f.pu_row : f.pl_row;
    const int32_t* pcol = MODE == 2 ? f.pu_col : f.pl_col;
    const double* pval = MODE == 2 ? f.pu_val : f.pl_val;
    const int kmax = MODE == 2 ? f.ku : f.kl;
    R.i = pos >= 0 ? __ldg(prow + pos) : -1;
#pragma unroll
    for (int k = 0; k < K; k++)
    {
        const bool in_k = R.i >= 0 && k < kmax;
        R.c[k] = in_k ? __ldg(pcol + (size_t)k * npos + pos) : -1;
        R.v[k] = in_k ? __ldg(pval + (size_t)k * npos + pos) : 0.0;
    }
    R.s0 = R.i >= 0 ? (MODE == 1 ? in[R.i] : __ldcg(out + R.i)) : 0.0;
    R.dg = R.i >= 0 && MODE == 2 ? __ldg(f.pu_diag + pos) : 1.0;
}

// the row's result: s0 - sum_k v_k out_{c_k} in column order (one FMA per
// entry: the cluster's 16 SMs retire FP64 at 1/64 of the FP32 rate, and a
// level's FP64 work is on its critical path), then times the reciprocal of
// the diagonal (MODE 2; formed once per factorisation, no division in the
// level)
template <int MODE, int K>
__device__ __forceinline__ void ilu_solve_row(const IluView& f, const PackedRow<K>& R, double* out)
{
    if (R.i < 0) return;
    double x[K];
#pragma unroll
    for (int k = 0; k < K; k++) x[k] = R.c[k] >= 0 && OGS_IN(R.c[k], f.n, kOobIluCol) ? __ldcg(out + R.c[k]) : 0.0;
    double s = R.s0;
#pragma unroll
    for (int k = 0; k < K; k++)
        if (R.c[k] >= 0) s = __fma_rn(-R.v[k], x[k], s);
    if (MODE == 2) s = s * R.dg;  // the packed reciprocal of U_ii
    __stcg(out + R.i, s);
}

// L2 prefetch of level l's packed rows (row, the K column and value arrays,
// the diagonal): levels start on multiples of 32 positions, so every
// segment starts and ends on a 128-byte boundary.  The cluster's CTAs share
// the segments.
template <int MODE>
__device__ __forceinline__ void ilu_prefetch_level(const IluView& f, int b, int e)
{
    if (threadIdx.x != 0 || e <= b) return;
    const int npos = MODE == 2 ? f.n_upos : f.n_lpos;
    const int kmax = MODE == 2 ? f.ku : f.kl;
    const int32_t* prow = MODE == 2 ? f.pu_row : f.pl_row;
    const int32_t* pcol = MODE == 2 ? f.pu_col : f.pl_col;
    const double* pval = MODE == 2 ? f.pu_val : f.pl_val;
    const int nseg = 2 * kmax + (MODE == 2 ? 2 : 1);
    const unsigned n4 = (unsigned)(e - b) * 4u, n8 = (unsigned)(e - b) * 8u;
    for (int q = blockIdx.x; q < nseg; q += gridDim.x)
    {
        const void* p;
        unsigned bytes;
        if (q == 0) { p = prow + b; bytes = n4; }
        else if (q <= kmax) { p = pcol + (size_t)(q - 1) * npos + b; bytes = n4; }
        else if (q <= 2 * kmax) { p = pval + (size_t)(q - 1 - kmax) * npos + b; bytes = n8; }
        else { p = f.pu_diag + b; bytes = n8; }
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
    }
}

// the two halves of the cluster barrier (.aligned: the warp reconverges
// first, after the divergent row work)
__device__ __forceinline__ void cluster_arrive_release()
{
    __syncwarp();
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire()
{
    __syncwarp();
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// MODE 1: forward sweep, MODE 2: backward sweep over the packed rows; the
// grid is one cluster.  A thread's first row of the next level is fetched
// between the arrive and the wait of the barrier that ends this level.
template <int MODE, int K, int NT>
__global__ void __launch_bounds__(NT, 1) k_ilu_sweep(IluView f, const double* __restrict__ in, double* out,
                                                    const KState* st)
{
    if (st->done) return;
    const int tid = blockIdx.x * NT + threadIdx.x, nt = gridDim.x * NT;
    const int32_t* ptr = MODE == 2 ? f.uptr : f.lptr;
    const int nl = MODE == 2 ? f.n_ulev : f.n_lev;
    const int npos = MODE == 2 ? f.n_upos : f.n_lpos;
    PackedRow<K> R;
    {
        const int b = __ldg(ptr), e = __ldg(ptr + 1);
        if (nl > 1) ilu_prefetch_level<MODE>(f, e, __ldg(ptr + 2));
        ilu_fetch<MODE, K>(f, in, out, b + tid < e ? b + tid : -1, npos, R);
    }
    for (int l = 0; l < nl; l++)
    {
        const int b = __ldg(ptr + l), e = __ldg(ptr + l + 1);
        if (l + 2 < nl) ilu_prefetch_level<MODE>(f, __ldg(ptr + l + 2), __ldg(ptr + l + 3));
        ilu_solve_row<MODE, K>(f, R, out);
        // a level wider than the cluster: its further rows fetched here
        for (int pos = b + tid + nt; pos < e; pos += nt)
        {
            PackedRow<K> T;
            ilu_fetch<MODE, K>(f, in, out, pos, npos, T);
            ilu_solve_row<MODE, K>(f, T, out);
        }
        cluster_arrive_release();
        if (l + 1 < nl)
        {
            const int b1 = e, e1 = __ldg(ptr + l + 2);
            ilu_fetch<MODE, K>(f, in, out, b1 + tid < e1 ? b1 + tid : -1, npos, R);
        }
        cluster_wait_acquire();
    }
}

// ------------------------------------------------------------------
// Tiled sweeps of lattice patterns (ogs_mesh::tiles).  Row (x, y, z) of the
// forward sweep reads only rows of [x-1, x] x [y-1, y] x [z-1, z], so the
// lattice is cut into tiles of 8^3 rows: a tile reads only itself and the
// up to 7 tiles before it on each axis, and the tiles go in the order of
// the sum of their tile coordinates.  A block of 64 threads takes a tile
// (tickets, as the level kernels take rows), loads the entries of its 512
// rows into shared memory before it waits, waits for the neighbouring
// tiles' flags, loads their results at its faces into a 9^3 cube in shared
// memory, and walks its rows in 22 steps of lx + ly + lz with a block
// barrier between steps: a thread owns the column (lx, ly) and does row lz
// at step lx + ly + lz.  Every value a row reads is then in shared memory,
// and a tile costs two dependent global round trips (its flags, its faces)
// instead of one per level of rows.  The backward sweep is the mirror
// image (tiles from the end of the list, steps reversed, faces at +1).
// Each row's arithmetic is the level kernels' (ilu_solve_row): the start
// value, one FMA per entry in column order, then times 1 / U_ii
// (backward), so the results are bit for bit the same.
//
// Slots: forward slot s is the neighbour -(q & 1, q >> 1 & 1, q >> 2 & 1)
// with q = 7 - s, backward slot u the neighbour (q & 1, q >> 1 & 1, q >> 2
// & 1) with q = u + 1: both in ascending column order on a lattice with
// nxy > nx + 1 > 2.
constexpr int kTileT = kIluTile * kIluTile;       // threads of a tile block
constexpr int kTileSteps = 3 * kIluTile - 2;       // steps of lx + ly + lz
constexpr int kTileCube = (kIluTile + 1) * (kIluTile + 1) * (kIluTile + 1);

__device__ __forceinline__ int tile_slot_offset(int mode, int slot)
{
    const int q = mode == 1 ? 7 - slot : slot + 1;
    const int sg = mode == 1 ? -1 : 1;
    return sg * ((q & 1) + (kIluTile + 1) * (((q >> 1) & 1) + (kIluTile + 1) * ((q >> 2) & 1)));
}

// The tile rows' pattern, once per system: the slots of each row's entries
// (bit 7: the row lies in the lattice and has a diagonal) and its CSR start
__global__ void k_ilu_tile_pattern(IluView f)
{
    const int64_t total = (int64_t)f.tiles * kIluTile * kTileT;
    const int nxy = f.lnx * f.lny;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
    {
        const int t = (int)(idx % kTileT), lz = (int)((idx / kTileT) % kIluTile);
        const int tile = (int)(idx / ((int64_t)kTileT * kIluTile));
        const int a = tile % f.tnx, b = (tile / f.tnx) % f.tny, c = tile / (f.tnx * f.tny);
        const int x = a * kIluTile + t % kIluTile, y = b * kIluTile + t / kIluTile, z = c * kIluTile + lz;
        unsigned lm = 0, um = 0;
        int rb = -1;
        if (x < f.lnx && y < f.lny && z < f.lnz)
        {
            const int i = x + f.lnx * (y + f.lny * z);
            const int d = __ldg(f.diag + i);
            if (d >= 0)
            {
                lm = um = 0x80;
                rb = __ldg(f.row_ptr + i);
                const int re = __ldg(f.row_ptr + i + 1);
                for (int k = rb; k < re; k++)
                {
                    if (k == d) continue;
                    const int j = __ldg(f.col + k);
                    const int dx = j % f.lnx - x, dy = (j / f.lnx) % f.lny - y, dz = j / nxy - z;
                    // 1 .. 7 on a checked pattern
                    const int q = k < d ? (-dx) | ((-dy) << 1) | ((-dz) << 2) : dx | (dy << 1) | (dz << 2);
                    if (OGS_IN(q - 1, 7, kOobIluCol))
                    {
                        if (k < d) lm |= 1u << (7 - q);
                        else um |= 1u << (q - 1);
                    }
                }
            }
        }
        const size_t row = ((size_t)tile * kIluTile + lz) * kTileT + t;
        f.tl_mask[row] = (unsigned char)lm;
        f.tu_mask[row] = (unsigned char)um;
        f.t_rb[row] = rb;
    }
}

// The entry of row i that a_ij -= l_ik u_kj updates, for row k = i + (lower
// slot s) and j = k + (upper slot u of row k): 0 .. 6 a lower slot, 7 the
// diagonal, 8 .. 14 an upper slot; -1 when j - i has components of both
// signs (no entry of a monotone pattern)
__host__ __device__ constexpr int tile_target(int s, int u)
{
    const int ql = 7 - s, qu = u + 1;
    const int sx = (qu & 1) - (ql & 1), sy = ((qu >> 1) & 1) - ((ql >> 1) & 1),
              sz = ((qu >> 2) & 1) - ((ql >> 2) & 1);
    if (sx == 0 && sy == 0 && sz == 0) return 7;
    if (sx <= 0 && sy <= 0 && sz <= 0) return 7 - ((-sx) | ((-sy) << 1) | ((-sz) << 2));
    if (sx >= 0 && sy >= 0 && sz >= 0) return 8 + ((sx | (sy << 1) | (sz << 2)) - 1);
    return -1;
}

// ILU(0) tile by tile (lattice patterns): rows of a tile eliminated in the
// order of lx + ly + lz, each in the IKJ order of the level kernel (its
// lower entries in column order, l_ik = a_ik / u_kk by ilu_div, then a_ij
// -= l_ik u_kj over row k's upper entries, products and differences
// rounded separately), with the pivot rows' U parts (u_kk, 1 / u_kk and 7
// upper values) in a 9^3 cube in shared memory: this tile's rows as they
// are done, the faces from the tiles before it.  Writes the factors in CSR order (lu) and the
// sweeps' tile arrays.  Dynamic shared memory: kTileFactorSmem bytes.
constexpr size_t kTileFactorSmem = sizeof(double) * (kIluTile * 15 * kTileT + kTileCube * 9) +
                                   sizeof(int) * kIluTile * kTileT + kTileCube + 2 * kIluTile * kTileT;

__global__ void __launch_bounds__(kTileT) k_ilu_factor_tiles(IluView f)
{
    extern __shared__ double dsm[];
    double(*s_a)[15][kTileT] = reinterpret_cast<double(*)[15][kTileT]>(dsm);  // the rows' entries
    double(*s_u)[8] = reinterpret_cast<double(*)[8]>(dsm + kIluTile * 15 * kTileT);  // U parts of the cube
    double* s_r = dsm + kIluTile * 15 * kTileT + kTileCube * 8;                          // 1 / u_kk of the cube
    int* s_rb = reinterpret_cast<int*>(dsm + kIluTile * 15 * kTileT + kTileCube * 9);
    unsigned char* s_um = reinterpret_cast<unsigned char*>(s_rb + kIluTile * kTileT);  // cube: upper mask
    unsigned char* s_lm = s_um + kTileCube;                                           // rows: lower mask
    unsigned char* s_ur = s_lm + kIluTile * kTileT;                                   // rows: upper mask
    __shared__ unsigned long long s_ticket;
    const int ntiles = f.tiles;
    const unsigned long long per = (unsigned long long)ntiles + gridDim.x;
    int* tflags = f.tile_flags + 2 * ntiles;
    const int t = threadIdx.x, lx = t % kIluTile, ly = t / kIluTile;
    constexpr int E = kIluTile + 1;
    const int64_t nrows = (int64_t)ntiles * kIluTile * kTileT;
    for (;;)
    {
        __syncthreads();
        if (t == 0) s_ticket = atomicAdd(f.tile_ticket + 2, 1ull);
        __syncthreads();
        const unsigned long long tk = s_ticket;
        const unsigned long long idx = tk % per;
        if (idx >= (unsigned long long)ntiles) return;  // this block's closing ticket
        const int launch = (int)(tk / per) + 1;
        const int tile = __ldg(f.tile_order + (int)idx);
        const int a = tile % f.tnx, b = (tile / f.tnx) % f.tny, c = tile / (f.tnx * f.tny);
        const int x = a * kIluTile + lx, y = b * kIluTile + ly;
        // the rows' entries (the matrix values in lu), before the wait
#pragma unroll
        for (int lz = 0; lz < kIluTile; lz++)
        {
            const size_t row = ((size_t)tile * kIluTile + lz) * kTileT + t;
            const bool rin = OGS_IN(row, nrows, kOobIluCol);
            const unsigned lm = rin ? __ldg(f.tl_mask + row) : 0u, um = rin ? __ldg(f.tu_mask + row) : 0u;
            const int rb = rin ? __ldg(f.t_rb + row) : -1;
            s_lm[lz * kTileT + t] = (unsigned char)lm;
            s_ur[lz * kTileT + t] = (unsigned char)um;
            s_rb[lz * kTileT + t] = rb;
            const int z = c * kIluTile + lz;
            if (lm & 0x80)
            {
                int p = rb;
#pragma unroll
                for (int q = 0; q < 7; q++)
                    if (lm & (1u << q)) s_a[lz][q][t] = __ldcg(f.lu + p++);
                s_a[lz][7][t] = __ldcg(f.lu + p++);
#pragma unroll
                for (int q = 0; q < 7; q++)
                    if (um & (1u << q)) s_a[lz][8 + q][t] = __ldcg(f.lu + p++);
            }
            else if (x < f.lnx && y < f.lny && z < f.lnz)
                atomicMin(f.bad, x + f.lnx * (y + f.lny * z));  // no diagonal: a zero pivot
        }
        // the tiles before this one
        if (t < 7)
        {
            const int q = t + 1;
            const int na = a - (q & 1), nb = b - ((q >> 1) & 1), nc = c - ((q >> 2) & 1);
            const int nt = na + f.tnx * (nb + f.tny * nc);
            if (na >= 0 && nb >= 0 && nc >= 0 && OGS_IN(nt, ntiles, kOobIluCol))
                ilu_wait(tflags, nt, launch, f.bad, f.spin ? f.spin : kIluSpin, kTilePause);
            fence_acquire();  // the block barrier below passes it on to the other threads
        }
        __syncthreads();
        // their rows' U parts at this tile's faces (cube index 0 on some axis)
        for (int h = t; h < kTileCube; h += kTileT)
        {
            const int cx = h % E, cy = (h / E) % E, cz = h / (E * E);
            if (cx != 0 && cy != 0 && cz != 0) continue;
            const int gx = a * kIluTile + cx - 1, gy = b * kIluTile + cy - 1, gz = c * kIluTile + cz - 1;
            unsigned um = 0;
            if (gx >= 0 && gy >= 0 && gz >= 0)
            {
                const int tt = gx / kIluTile + f.tnx * (gy / kIluTile + f.tny * (gz / kIluTile));
                const size_t r8 = ((size_t)tt * kIluTile + gz % kIluTile) * kTileT + gx % kIluTile +
                                  kIluTile * (gy % kIluTile);
                if (OGS_IN(r8, nrows, kOobIluCol))
                {
                    um = __ldg(f.tu_mask + r8);
                    if (um & 0x80)
                    {
                        s_u[h][0] = __ldcg(f.tu_piv + r8);
                        s_r[h] = __ldcg(f.tu_dg + r8);
                        const size_t v0 = ((size_t)tt * kIluTile + gz % kIluTile) * 7 * kTileT + gx % kIluTile +
                                          kIluTile * (gy % kIluTile);
#pragma unroll
                        for (int q = 0; q < 7; q++) s_u[h][1 + q] = __ldcg(f.tu_val + v0 + (size_t)q * kTileT);
                    }
                }
            }
            s_um[h] = (unsigned char)um;
        }
        __syncthreads();
        for (int step = 0; step < kTileSteps; step++)
        {
            const int lz = step - lx - ly;
            if (lz >= 0 && lz < kIluTile)
            {
                const unsigned lm = s_lm[lz * kTileT + t], um = s_ur[lz * kTileT + t];
                if (lm & 0x80)
                {
                    const int z = c * kIluTile + lz;
                    const int i = x + f.lnx * (y + f.lny * z);
                    const int ci = (lx + 1) + E * ((ly + 1) + E * (lz + 1));
                    double av[15];
#pragma unroll
                    for (int q = 0; q < 15; q++) av[q] = s_a[lz][q][t];
#pragma unroll
                    for (int sl = 0; sl < 7; sl++)
                    {
                        if (!(lm & (1u << sl))) continue;
                        const int nb = ci + tile_slot_offset(1, sl);
                        const double piv = s_u[nb][0];
                        const unsigned kum = s_um[nb];
                        if (piv == 0.0)
                        {
                            const int qq = 7 - sl;
                            atomicMin(f.bad, i - ((qq & 1) + f.lnx * (((qq >> 1) & 1) + f.lny * ((qq >> 2) & 1))));
                        }
                        const double lik = ilu_div(av[sl], piv, s_r[nb]);
                        av[sl] = lik;
#pragma unroll
                        for (int u = 0; u < 7; u++)
                        {
                            const int T = tile_target(sl, u);
                            if (T < 0 || !(kum & (1u << u))) continue;
                            const bool present = T < 7 ? (lm >> T) & 1u : T == 7 ? 1u : (um >> (T - 8)) & 1u;
                            if (present) av[T] = __dsub_rn(av[T], __dmul_rn(lik, s_u[nb][1 + u]));
                        }
                    }
                    if (av[7] == 0.0) atomicMin(f.bad, i);
                    // this row's U part for the rows after it
                    const double rd = 1.0 / av[7];
                    s_u[ci][0] = av[7];
                    s_r[ci] = rd;
#pragma unroll
                    for (int q = 0; q < 7; q++) s_u[ci][1 + q] = av[8 + q];
                    s_um[ci] = (unsigned char)um;
                    // the factors: CSR order, and the sweeps' tile arrays
                    int p = s_rb[lz * kTileT + t];
#pragma unroll
                    for (int q = 0; q < 7; q++)
                        if (lm & (1u << q)) __stcg(f.lu + p++, av[q]);
                    __stcg(f.lu + p++, av[7]);
#pragma unroll
                    for (int q = 0; q < 7; q++)
                        if (um & (1u << q)) __stcg(f.lu + p++, av[8 + q]);
                    const size_t row = ((size_t)tile * kIluTile + lz) * kTileT + t;
                    const size_t v0 = ((size_t)tile * kIluTile + lz) * 7 * kTileT + t;
#pragma unroll
                    for (int q = 0; q < 7; q++)
                    {
                        __stcg(f.tl_val + v0 + (size_t)q * kTileT, (lm & (1u << q)) ? av[q] : 0.0);
                        __stcg(f.tu_val + v0 + (size_t)q * kTileT, (um & (1u << q)) ? av[8 + q] : 0.0);
                    }
                    __stcg(f.tu_piv + row, av[7]);
                    __stcg(f.tu_dg + row, rd);
                }
            }
            __syncthreads();
        }
        // the block's stores are ordered before thread 0's fence by the last
        // step's barrier (the grid-barrier pattern: one fence per block)
        if (t == 0)
        {
            __threadfence();
            st_release_s32(tflags + tile, launch);
        }
    }
}

// MODE 1: forward sweep, MODE 2: backward sweep, tile by tile
template <int MODE>
__global__ void __launch_bounds__(kTileT) k_ilu_tiles(IluView f, const double* __restrict__ in, double* out,
                                                     const KState* st)
{
    if (st->done) return;
    const int ntiles = f.tiles;
    const unsigned long long per = (unsigned long long)ntiles + gridDim.x;
    int* tflags = f.tile_flags + (MODE - 1) * ntiles;
    const double* vals = MODE == 1 ? f.tl_val : f.tu_val;
    const unsigned char* masks = MODE == 1 ? f.tl_mask : f.tu_mask;
    __shared__ double s_x[kTileCube];                 // results: the tile and its faces
    __shared__ double s_v[kIluTile][7][kTileT];       // entries of the block's rows
    __shared__ double s_s0[kIluTile][kTileT];         // start values
    __shared__ double s_dg[MODE == 2 ? kIluTile : 1][kTileT];
    __shared__ unsigned char s_mk[kIluTile][kTileT];
    __shared__ unsigned long long s_ticket;
    const int t = threadIdx.x, lx = t % kIluTile, ly = t / kIluTile;
    constexpr int E = kIluTile + 1;
    for (;;)
    {
        __syncthreads();
        if (t == 0) s_ticket = atomicAdd(f.tile_ticket + (MODE - 1), 1ull);
        __syncthreads();
        const unsigned long long tk = s_ticket;
        const unsigned long long idx = tk % per;
        if (idx >= (unsigned long long)ntiles) return;  // this block's closing ticket
        const int launch = (int)(tk / per) + 1;
        const int tile = __ldg(f.tile_order + (MODE == 1 ? (int)idx : ntiles - 1 - (int)idx));
        const int a = tile % f.tnx, b = (tile / f.tnx) % f.tny, c = tile / (f.tnx * f.tny);
        const int x = a * kIluTile + lx, y = b * kIluTile + ly;
        // the rows' entries, masks and start values (final before this
        // launch: the forward input, or the forward results for MODE 2)
#pragma unroll
        for (int lz = 0; lz < kIluTile; lz++)
        {
            const size_t row = ((size_t)tile * kIluTile + lz) * kTileT + t;
            const size_t v0 = ((size_t)tile * kIluTile + lz) * 7 * kTileT + t;
            const unsigned mk = OGS_IN(row, (int64_t)ntiles * kIluTile * kTileT, kOobIluCol) ? __ldg(masks + row) : 0u;
            const int z = c * kIluTile + lz;
            const int i = x + f.lnx * (y + f.lny * z);
            s_mk[lz][t] = (unsigned char)mk;
            s_s0[lz][t] = (mk & 0x80) && OGS_IN(i, f.n, kOobIluCol) ? (MODE == 1 ? in[i] : __ldcg(out + i)) : 0.0;
            if constexpr (MODE == 2) s_dg[lz][t] = __ldg(f.tu_dg + row);
#pragma unroll
            for (int q = 0; q < 7; q++) s_v[lz][q][t] = __ldg(vals + v0 + (size_t)q * kTileT);
        }
        // the neighbouring tiles before this one in the sweep
        if (t < 7)
        {
            const int q = t + 1, sg = MODE == 1 ? -1 : 1;
            const int na = a + sg * (q & 1), nb = b + sg * ((q >> 1) & 1), nc = c + sg * ((q >> 2) & 1);
            const int nt = na + f.tnx * (nb + f.tny * nc);
            if (na >= 0 && na < f.tnx && nb >= 0 && nb < f.tny && nc >= 0 && nc < f.tnz &&
                OGS_IN(nt, ntiles, kOobIluCol))
                ilu_wait(tflags, nt, launch, f.bad, f.spin ? f.spin : kIluSpin, kTilePause);
            fence_acquire();  // the block barrier below passes it on to the other threads
        }
        __syncthreads();
        // their results at this tile's faces (forward: cube index 0 on some
        // axis, the lattice coordinate one below the tile; backward: index 8)
        for (int h = t; h < kTileCube; h += kTileT)
        {
            const int cx = h % E, cy = (h / E) % E, cz = h / (E * E);
            const int face = MODE == 1 ? 0 : kIluTile;
            if (cx != face && cy != face && cz != face) continue;
            const int o = MODE == 1 ? -1 : 0;
            const int gx = a * kIluTile + cx + o, gy = b * kIluTile + cy + o, gz = c * kIluTile + cz + o;
            const bool in_l = gx >= 0 && gx < f.lnx && gy >= 0 && gy < f.lny && gz >= 0 && gz < f.lnz;
            const int gi = gx + f.lnx * (gy + f.lny * gz);
            s_x[h] = in_l && OGS_IN(gi, f.n, kOobIluCol) ? __ldcg(out + gi) : 0.0;
        }
        __syncthreads();
        // the tile's rows, step by step
        const int co = MODE == 1 ? 1 : 0;  // cube index of local coordinate 0
        for (int step = 0; step < kTileSteps; step++)
        {
            const int sl = MODE == 1 ? step : kTileSteps - 1 - step;
            const int lz = sl - lx - ly;
            if (lz >= 0 && lz < kIluTile)
            {
                const unsigned mk = s_mk[lz][t];
                if (mk & 0x80)
                {
                    const int ci = (lx + co) + E * ((ly + co) + E * (lz + co));
                    double s = s_s0[lz][t];
#pragma unroll
                    for (int q = 0; q < 7; q++)
                        if (mk & (1u << q)) s = __fma_rn(-s_v[lz][q][t], s_x[ci + tile_slot_offset(MODE, q)], s);
                    if (MODE == 2) s = s * s_dg[lz][t];
                    s_x[ci] = s;
                    const int i = x + f.lnx * (y + f.lny * (c * kIluTile + lz));
                    if (OGS_IN(i, f.n, kOobIluCol)) __stcg(out + i, s);
                }
            }
            __syncthreads();
        }
        // publish the tile: the block's stores are ordered before thread 0's
        // fence by the last step's barrier (the grid-barrier pattern)
        if (t == 0)
        {
            __threadfence();
            st_release_s32(tflags + tile, launch);
        }
    }
}

// ------------------------------------------------------------------
// CG with ILU(0): the update kernel leaves r, z = M^-1 r comes from the
// sweeps, this kernel writes the partials of r . r and r . z for k_cg_p
// ------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_cg_dots_z(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    const int it = st->iter;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
    {
        const double r = a.v.r[i];
        v[0] += r * r;
        v[1] += r * a.v.ph[i];
    }
    write_partials<2, double>(v, st->cg_upd[it & 1]);
}

// start of CG with ILU(0): p = z = M^-1 r0 and rz_base = r0 . z
__global__ void __launch_bounds__(kThreads) k_cg_init_z(SolveArgs a)
{
    KState* st = a.st;
    if (st->done) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.A.n; i += gridDim.x * blockDim.x)
    {
        const double z = a.v.ph[i];
        a.v.p[i] = z;
        v[0] += a.v.r[i] * z;
    }
    double out[1];
    if (grid_sum<1, double>(v, out, st->part[2], &st->ticket[2]) && threadIdx.x == 0) st->rz_base = out[0];
}

// ------------------------------------------------------------------
// host side
// ------------------------------------------------------------------
// the persistent grid (the same for every launch of a system: tickets per
// launch depend on it)
static int ilu_grid(int npos)
{
    static int sms = 0;
    if (!sms)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    return std::max(1, std::min((npos + kIluBlock - 1) / kIluBlock, sms * kIluBlocksPerSm));
}

// the tile factorisation's persistent grid (dynamic shared memory opted in)
static int tile_factor_grid()
{
    static int g = 0;
    if (!g)
    {
        int dev = 0, sms = 152, o = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaFuncSetAttribute(k_ilu_factor_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTileFactorSmem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_ilu_factor_tiles, kTileT, kTileFactorSmem) !=
                cudaSuccess)
        {
            cudaGetLastError();
            o = 1;
        }
        g = std::max(1, sms * std::max(1, o));
    }
    return g;
}

void launch_ilu_factor(const IluView& f, const double* val, const int32_t* csr2sell, int64_t nnz,
                       const KState* st, cudaStream_t s)
{
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((nnz + 255) / 256, 4096));
    k_ilu_copy<<<g, 256, 0, s>>>(val, csr2sell, f.lu, nnz);
    if (f.tiles)
    {
        k_ilu_factor_tiles<<<tile_factor_grid(), kTileT, kTileFactorSmem, s>>>(f);
        return;
    }
    k_ilu_flow<0><<<ilu_grid(f.n_lpos), kIluBlock, 0, s>>>(f, nullptr, nullptr, st);
    if (f.pl_row) k_ilu_pack<<<ilu_grid(std::max(f.n_lpos, f.n_upos)), kIluBlock, 0, s>>>(f);
}

// once per system: the tile rows' slots and CSR starts
void launch_ilu_tile_pattern(const IluView& f, cudaStream_t s)
{
    const int64_t rows = (int64_t)f.tiles * kIluTile * kTileT;
    k_ilu_tile_pattern<<<(int)std::min<int64_t>((rows + 255) / 256, 8192), 256, 0, s>>>(f);
}

// the tile sweeps' persistent grid: one block per SM (a tile level of the
// 129 x 129 x 65 lattice holds at most ~130 tiles; more blocks only add
// blocks that wait and poll; the same for every launch: tickets per launch
// depend on it)
static int tile_grid()
{
    static int g = 0;
    if (!g)
    {
        int dev = 0, sms = 152, o1 = 0, o2 = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k_ilu_tiles<1>, kTileT, 0) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_ilu_tiles<2>, kTileT, 0) != cudaSuccess)
        {
            cudaGetLastError();
            o1 = o2 = 1;
        }
        g = std::max(1, sms * std::max(1, std::min(std::min(o1, o2), 1)));
    }
    return g;
}

// the cluster sweeps: rows of at most 8 (tets, quads) or 16 (hexes) L / U
// entries, a 16-CTA cluster where the device takes one, else 8
template <int MODE, int K, int NT>
static cudaError_t launch_sweep(const IluView& f, const double* in, double* out, const KState* st, int ctas,
                                cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(NT);
    cfg.stream = s;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = ctas;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_ilu_sweep<MODE, K, NT>, f, in, out, st);
}

template <int K, int NT>
static int sweep_ctas()
{
    static int ctas = -1;
    if (ctas < 0)
    {
        ctas = 0;
        const int want[2] = {16, 8};
        for (int c : want)
        {
            if (c > 8)
            {
                if (cudaFuncSetAttribute(k_ilu_sweep<1, K, NT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                        cudaSuccess ||
                    cudaFuncSetAttribute(k_ilu_sweep<2, K, NT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                        cudaSuccess)
                {
                    cudaGetLastError();
                    continue;
                }
            }
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(NT);
            cudaLaunchAttribute attr;
            attr.id = cudaLaunchAttributeClusterDimension;
            attr.val.clusterDim.x = c;
            attr.val.clusterDim.y = 1;
            attr.val.clusterDim.z = 1;
            cfg.attrs = &attr;
            cfg.numAttrs = 1;
            int n1 = 0, n2 = 0;
            if (cudaOccupancyMaxActiveClusters(&n1, k_ilu_sweep<1, K, NT>, &cfg) == cudaSuccess &&
                cudaOccupancyMaxActiveClusters(&n2, k_ilu_sweep<2, K, NT>, &cfg) == cudaSuccess && n1 > 0 && n2 > 0)
            {
                ctas = c;
                break;
            }
            cudaGetLastError();
        }
    }
    return ctas;
}

// out = (LU)^-1 in
void launch_ilu_apply(const IluView& f, const double* in, double* out, const KState* st, cudaStream_t s)
{
    if (f.tiles)
    {
        const int g = tile_grid();
        k_ilu_tiles<1><<<g, kTileT, 0, s>>>(f, in, out, st);
        k_ilu_tiles<2><<<g, kTileT, 0, s>>>(f, nullptr, out, st);
        return;
    }
    const int k = std::max(f.kl, f.ku);
    if (f.pl_row && k <= 8 && sweep_ctas<8, 1024>() > 0)
    {
        const int c = sweep_ctas<8, 1024>();
        launch_sweep<1, 8, 1024>(f, in, out, st, c, s);
        launch_sweep<2, 8, 1024>(f, nullptr, out, st, c, s);
        return;
    }
    if (f.pl_row && k <= 16 && sweep_ctas<16, 512>() > 0)
    {
        const int c = sweep_ctas<16, 512>();
        launch_sweep<1, 16, 512>(f, in, out, st, c, s);
        launch_sweep<2, 16, 512>(f, nullptr, out, st, c, s);
        return;
    }
    k_ilu_flow<1><<<ilu_grid(f.n_lpos), kIluBlock, 0, s>>>(f, in, out, st);
    k_ilu_flow<2><<<ilu_grid(f.n_upos), kIluBlock, 0, s>>>(f, nullptr, out, st);
}

// Self-test of the bounded row waits: a forward sweep over a 64-row lower
// bidiagonal L (row i reads row i - 1; one row per level, each level padded
// to a warp).  withhold: row 0 is left out of the level list, so nothing
// publishes it and every later row's wait runs out (f.bad = -1).  Returns
// through *gave_up whether a wait gave up and through *rows_ok how many
// rows hold the chain's exact value.
cudaError_t ilu_wait_selftest(int withhold, unsigned limit, int* gave_up, int* rows_ok, cudaStream_t s)
{
    constexpr int n = 64, npos = n * 32;
    std::vector<int32_t> rp(n + 1), col, dg(n), rows(npos, -1);
    std::vector<double> lu;
    for (int i = 0; i < n; i++)
    {
        rp[i] = (int32_t)col.size();
        if (i > 0)
        {
            col.push_back(i - 1);
            lu.push_back(0.5);
        }
        dg[i] = (int32_t)col.size();
        col.push_back(i);
        lu.push_back(1.0);
        rows[32 * i] = withhold && i == 0 ? -1 : i;
    }
    rp[n] = (int32_t)col.size();
    const int nnz = (int)col.size();
    char* buf = nullptr;
    const size_t bytes = 4096 + sizeof(int32_t) * (n + 1 + nnz + n + npos + 3 * n + 1) + sizeof(double) * (nnz + 2 * n) +
                         sizeof(unsigned long long) * 3 + sizeof(KState);
    cudaError_t e = cudaMalloc(&buf, bytes);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(buf, 0, bytes, s);
    size_t off = 0;
    auto take = [&](size_t b) { char* p = buf + off; off = (off + b + 255) & ~size_t(255); return p; };
    int32_t* d_rp = (int32_t*)take(sizeof(int32_t) * (n + 1));
    int32_t* d_col = (int32_t*)take(sizeof(int32_t) * nnz);
    int32_t* d_dg = (int32_t*)take(sizeof(int32_t) * n);
    int32_t* d_rows = (int32_t*)take(sizeof(int32_t) * npos);
    int* d_flags = (int*)take(sizeof(int) * 3 * n);
    int* d_bad = (int*)take(sizeof(int));
    double* d_lu = (double*)take(sizeof(double) * nnz);
    double* d_in = (double*)take(sizeof(double) * n);
    double* d_out = (double*)take(sizeof(double) * n);
    unsigned long long* d_ticket = (unsigned long long*)take(sizeof(unsigned long long) * 3);
    KState* d_st = (KState*)take(sizeof(KState));
    std::vector<double> ones(n, 1.0);
    const int big = 0x7fffffff;
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rp, rp.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_col, col.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_dg, dg.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rows, rows.data(), sizeof(int32_t) * npos, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_lu, lu.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_bad, &big, sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
    {
        IluView f;
        std::memset(&f, 0, sizeof f);
        f.row_ptr = d_rp; f.col = d_col; f.diag = d_dg; f.lu = d_lu;
        f.lrows = d_rows; f.urows = d_rows;
        f.n = n; f.n_lpos = npos; f.n_upos = npos;
        f.flags = d_flags; f.ticket = d_ticket; f.bad = d_bad; f.spin = limit;
        k_ilu_flow<1><<<ilu_grid(npos), kIluBlock, 0, s>>>(f, d_in, d_out, d_st);
        e = cudaGetLastError();
    }
    int bad = 0;
    std::vector<double> out(n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.data(), d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    if (e != cudaSuccess) return e;
    // exact chain: x_0 = 1, x_i = 1 - x_{i-1} / 2 (products and differences rounded as the kernel does)
    int ok = 0;
    double x = 0.0;
    for (int i = 0; i < n; i++)
    {
        x = i == 0 ? 1.0 : 1.0 - 0.5 * x;
        ok += out[i] == x ? 1 : 0;
    }
    *gave_up = bad == -1 ? 1 : 0;
    *rows_ok = ok;
    return cudaSuccess;
}

void launch_cg_dots_z(const SolveArgs& a, int grid, cudaStream_t s)
{
    k_cg_dots_z<<<grid, kThreads, 0, s>>>(a);
}

void launch_cg_init_z(const SolveArgs& a, int grid, cudaStream_t s)
{
    k_cg_init_z<<<grid, kThreads, 0, s>>>(a);
}

}  // namespace ogs

unsigned long long ogs_oob_ilu() { return ogs::oob_take(); }
