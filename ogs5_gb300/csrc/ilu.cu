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
// hexes): hundreds of levels of a few thousand rows each -- far too
// little work per level for the whole GPU, and far too many levels for
// one launch each.  One thread-block cluster (8 CTAs x 1024 threads) walks
// all levels in a single launch and separates levels with the hardware
// cluster barrier (barrier.cluster arrive.release / wait.acquire): no
// spin-waits, no grid-wide synchronisation, no launch per level.  Values
// written by other CTAs of the cluster are read with L2 (.cg) loads.
#include <cooperative_groups.h>

#include <algorithm>

#include "krylov.cuh"

namespace cg = cooperative_groups;

namespace ogs {

constexpr int kIluCtas = 8;       // portable cluster size
constexpr int kIluThreads = 1024;

// lu = A on the CSR pattern (values live in SELL-32 order)
__global__ void k_ilu_copy(const double* __restrict__ val, const int32_t* __restrict__ csr2sell,
                           double* __restrict__ lu, int64_t nnz)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
        lu[k] = val[csr2sell[k]];
}

// MODE 0: factorisation (IKJ, rows in forward levels)
// MODE 1: forward sweep  out_i = in_i - sum_{k<i} L_ik out_k
// MODE 2: backward sweep out_i = (out_i - sum_{j>i} U_ij out_j) / U_ii
// The sweeps return at once when the solve has finished (uniform over the
// cluster: st->done is not written while this kernel runs).
template <int MODE>
__global__ void __cluster_dims__(kIluCtas, 1, 1) __launch_bounds__(kIluThreads)
    k_ilu_levels(IluView f, const double* __restrict__ in, double* out, const KState* st)
{
    if (MODE != 0 && st->done) return;
    cg::cluster_group cluster = cg::this_cluster();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = gridDim.x * blockDim.x;
    const int32_t* rows = MODE == 2 ? f.urows : f.lrows;
    const int32_t* ptr = MODE == 2 ? f.uptr : f.lptr;
    const int nl = MODE == 2 ? f.n_ulev : f.n_lev;
    for (int l = 0; l < nl; l++)
    {
        const int b = __ldg(ptr + l), e = __ldg(ptr + l + 1);
        for (int t = b + tid; t < e; t += nt)
        {
            const int i = __ldg(rows + t);
            const int rb = __ldg(f.row_ptr + i), re = __ldg(f.row_ptr + i + 1);
            const int d = __ldg(f.diag + i);
            if (d < 0)
            {
                // a node in no element has no diagonal: a zero pivot
                if (MODE == 0) atomicMin(f.bad, i);
                continue;
            }
            if (MODE == 0)
            {
                // row i -= l_ik row k for every k < i of the pattern, in
                // column order; products and differences rounded
                // separately (no FMA), like the sequential elimination
                for (int kk = rb; kk < d; kk++)
                {
                    const int k = __ldg(f.col + kk);
                    const int dk = __ldg(f.diag + k), ke = __ldg(f.row_ptr + k + 1);
                    const double piv = __ldcg(f.lu + dk);
                    if (piv == 0.0) atomicMin(f.bad, k);
                    const double lik = __ldcg(f.lu + kk) / piv;
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
        }
        cluster.sync();
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
bool ilu_cluster_ok()
{
    static int ok = -1;
    if (ok < 0)
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kIluCtas);
        cfg.blockDim = dim3(kIluThreads);
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = kIluCtas;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        int n0 = 0, n1 = 0, n2 = 0;
        const bool q = cudaOccupancyMaxActiveClusters(&n0, k_ilu_levels<0>, &cfg) == cudaSuccess &&
                       cudaOccupancyMaxActiveClusters(&n1, k_ilu_levels<1>, &cfg) == cudaSuccess &&
                       cudaOccupancyMaxActiveClusters(&n2, k_ilu_levels<2>, &cfg) == cudaSuccess;
        if (!q) cudaGetLastError();
        ok = q && n0 > 0 && n1 > 0 && n2 > 0;
    }
    return ok == 1;
}

void launch_ilu_factor(const IluView& f, const double* val, const int32_t* csr2sell, int64_t nnz,
                       const KState* st, cudaStream_t s)
{
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((nnz + 255) / 256, 4096));
    k_ilu_copy<<<g, 256, 0, s>>>(val, csr2sell, f.lu, nnz);
    k_ilu_levels<0><<<kIluCtas, kIluThreads, 0, s>>>(f, nullptr, nullptr, st);
}

// out = (LU)^-1 in
void launch_ilu_apply(const IluView& f, const double* in, double* out, const KState* st, cudaStream_t s)
{
    k_ilu_levels<1><<<kIluCtas, kIluThreads, 0, s>>>(f, in, out, st);
    k_ilu_levels<2><<<kIluCtas, kIluThreads, 0, s>>>(f, nullptr, out, st);
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
