// common.cuh -- shared types of the GB300 flow/transport library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ogs_gpu.h"

namespace ogs {

// Thread-local error text behind ogs_gpu_last_error().
void set_error(const char* fmt, ...);
const char* last_error();

// Count of this library's kernel launches (ogs_gpu_kernel_launches).
void count_launches(int64_t n);

// Bounds checks of the debug build (-DOGS_BOUNDS_CHECK): OGS_IN(i, n, site)
// is true when 0 <= i < n; otherwise it records (site, i) in this file's
// device word (the smallest site first) and is false, and the caller skips
// the access.  Without the macro it is true and costs nothing.  The sites:
enum OobSite
{
    kOobAsmSlot = 1,     // element assembly: SELL slot of an (i, j) pair
    kOobAsmNode = 2,     // element assembly: node of an element
    kOobLatSlot = 3,     // lattice assembly: SELL slot of a row entry
    kOobLatNode = 4,     // lattice assembly: neighbour node / cell
    kOobSpmvCol = 5,     // FP64 SELL product: column
    kOobMixedCol = 6,    // FP32 SELL product: column
    kOobDirCol = 7,      // Dirichlet elimination: column / row
    kOobDirSlot = 8,     // Dirichlet elimination: slot
    kOobIluCol = 9,      // ILU(0) sweeps and factorisation: column
    kOobMixedWindow = 10,  // FP32 lattice product: a 16-byte window outside its padded row / vector
};
#ifdef OGS_BOUNDS_CHECK
static __device__ unsigned long long g_oob = ~0ull;
__device__ __forceinline__ bool oob_ok(long long i, long long n, int site)
{
    if (i >= 0 && i < n) return true;
    atomicMin(&g_oob, ((unsigned long long)site << 40) | ((unsigned long long)i & 0xffffffffffull));
    return false;
}
#define OGS_IN(i, n, site) ::ogs::oob_ok((long long)(i), (long long)(n), (site))
// this file's word, then reset
static inline unsigned long long oob_take()
{
    unsigned long long v = ~0ull, r = ~0ull;
    if (cudaMemcpyFromSymbol(&v, g_oob, sizeof v) != cudaSuccess || cudaMemcpyToSymbol(g_oob, &r, sizeof r) != cudaSuccess)
    {
        cudaGetLastError();
        return ~0ull;
    }
    return v;
}
#else
#define OGS_IN(i, n, site) true
static inline unsigned long long oob_take() { return ~0ull; }
#endif

#define OGS_CUDA_TRY(expr)                                                  \
    do                                                                      \
    {                                                                       \
        cudaError_t e_ = (expr);                                            \
        if (e_ != cudaSuccess)                                              \
        {                                                                   \
            ::ogs::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,     \
                             cudaGetErrorString(e_));                       \
            return e_ == cudaErrorMemoryAllocation ? OGS_OOM                \
                                                   : OGS_CUDA_ERROR;        \
        }                                                                   \
    } while (0)

#define OGS_LAUNCH_CHECK()                                                  \
    do                                                                      \
    {                                                                       \
        cudaError_t e_ = cudaGetLastError();                                \
        if (e_ != cudaSuccess)                                              \
        {                                                                   \
            ::ogs::set_error("%s:%d launch: %s", __FILE__, __LINE__,        \
                             cudaGetErrorString(e_));                       \
            return OGS_CUDA_ERROR;                                          \
        }                                                                   \
        ::ogs::count_launches(1);                                           \
    } while (0)

constexpr int kThreads = 256;
constexpr int kIluTile = 8;  // ILU(0) tile edge (nodes per axis)
constexpr int kMaxBlocks = 4096;  // reduction partial slots per kernel

inline int nodes_per_element(int et) { return et == OGS_ELEM_HEX8 ? 8 : 4; }
inline int elem_dim(int et) { return et == OGS_ELEM_QUAD4 ? 2 : 3; }
inline int num_gauss_points(int et, int ngauss)
{
    if (et == OGS_ELEM_QUAD4) return ngauss * ngauss;
    if (et == OGS_ELEM_HEX8) return ngauss * ngauss * ngauss;
    return 5;
}

// Shape-function tables of one (element type, Gauss order): per Gauss point
// N[nn], dN/dxi[dim][nn] row-major and the per-direction weights w3[3]
// (GetGaussData multiplies det * w_r * w_s * w_t left to right).
struct ShapeTable
{
    int ngp = 0, nn = 0, dim = 0;
    std::vector<double> N, dN, w3, wprod;
};
ShapeTable make_shape_table(int et, int ngauss);

// Device-side view of a shape table (lives in global memory; kernels stage
// it into shared memory).
struct DevTable
{
    const double* N;
    const double* dN;
    const double* w3;
    int ngp;
};

// Affine-element reference tensors: for elements whose Jacobian is constant
// (parallelogram quads, parallelepiped hexes, all tets)
//   Q[a][b][i][j] = sum_gp w_gp dN_a,i(gp) dN_b,j(gp)
//   M0[i][j]      = sum_gp w_gp N_i(gp) N_j(gp)
// so that Laplace_ij = |J| sum_ab C_ab Q_abij and Mass_ij = c |J| M0_ij with
// C = invJ^T mat invJ.
struct AffineTable
{
    std::vector<double> Q;   // [dim][dim][nn][nn]
    std::vector<double> M0;  // [nn][nn]
    std::vector<double> dNc; // dN/dxi at the element centre [dim][nn]
};
AffineTable make_affine_table(int et, int ngauss);

// Arguments of the element kernels (assembly and Gauss-point flux).
struct AsmArgs
{
    int64_t E;
    const double* x;
    const double* y;
    const double* z;
    const int32_t* conn_t;
    const int32_t* slot_t;
    const double* tab;
    const double* aff;
    const double* elem_k;
    const double* u0;
    const double* gpv;  // [e][gp][3]
    double* val;
    double* b;
    double* val2;       // transport with memory_type > 0, first assembly:
                        // val gets the mass, val2 the Laplace + advection +
                        // storage operator, b nothing
    double* q_out;      // velocity kernel output [e][gp][3]
    int* bad_elem;      // first element with a singular Jacobian + 1
    ogs_assembly_params p;
    const double* u1;   // RICHARDS_FLOW: the Picard iterate (coefficients)
    ogs_richards_params r;
    int val_store;      // val is all zeros (Initialize, nothing added since):
                        // a row kernel may store instead of add
    int64_t nslots, nrows;  // SELL slots and rows (the debug build's bounds)
};

}  // namespace ogs

// Matrix values live in SELL-32 order on the device: rows are grouped in
// slices of 32 consecutive rows; inside a slice, entry j of every row is
// stored contiguously (j-major), so one warp -- one thread per row -- reads
// 32 consecutive values per step.  Rows shorter than the slice width are
// padded with (own column, 0.0).  The CSR pattern of SparseTable is kept for
// read-back; csr2sell maps a CSR position to its SELL slot.
constexpr int kSlice = 32;

struct ogs_mesh
{
    int elem_type = 0, dim = 3, nn = 8, ngauss = 3, ngp = 27;
    int64_t n_nodes = 0, n_elem = 0;
    int64_t nnz = 0;          // CSR entries (SparseTable size_entry_column)
    int64_t sell_nnz = 0;     // SELL-32 slots including padding
    int n_slices = 0;
    bool affine = false;      // every element has a constant Jacobian
    // regular lattice of hexahedra: node i = ix + gx (iy + gy iz) at
    // (x0 + ix hx, ...), cell c = cx + (gx-1) (cy + (gy-1) cz) in the OGS
    // corner order; the FP32 inner CG can then apply the operator from one
    // coefficient per cell instead of stored matrix values
    bool grid = false;
    int gx = 0, gy = 0, gz = 0;
    double ghx = 0.0, ghy = 0.0, ghz = 0.0;
    int device = 0;
    // device arrays
    double *x = nullptr, *y = nullptr, *z = nullptr;
    int32_t* conn_t = nullptr;     // [nn][n_elem]
    int32_t* row_ptr = nullptr;    // CSR [n_nodes+1]
    int32_t* col = nullptr;        // CSR [nnz]
    int32_t* csr2sell = nullptr;   // [nnz] SELL slot of each CSR entry
    int32_t* slice_ptr = nullptr;  // [n_slices+1] first SELL slot of a slice
    int32_t* sell_col = nullptr;   // [sell_nnz]
    int32_t* row_len = nullptr;    // [n_nodes] stored entries per row
    int32_t* diag_pos = nullptr;   // [n_nodes] SELL slot of the diagonal
    int32_t* slot_t = nullptr;     // [nn*nn][n_elem] SELL slot of (i, j)
    // ILU(0): CSR diagonal positions and the dependency levels of the
    // forward (lower) and backward (upper) sweeps in natural row order;
    // the rows by level, each level padded with -1 to a multiple of 32
    int32_t* csr_diag = nullptr;   // [n_nodes]
    int32_t* lvl_rows = nullptr;   // [n_lpos] rows by forward level
    int32_t* lvl_ptr = nullptr;    // [n_lvl + 1] first position of a level
    int32_t* ulvl_rows = nullptr;  // [n_upos] rows by backward level
    int32_t* ulvl_ptr = nullptr;   // [n_ulvl + 1]
    int n_lvl = 0, n_ulvl = 0;
    int n_lpos = 0, n_upos = 0;
    int ilu_kl = 0, ilu_ku = 0;    // most entries left / right of the diagonal in a row
    // ILU(0) tiles: a lattice pattern numbered line by line whose columns
    // left of the diagonal lie at no larger x, y, z than their row (and
    // those right of it at no smaller), every entry at most one step away
    // on each axis (Kuhn tets, 7-point stencils): lnx x lny x lnz nodes,
    // tiles of kIluTile^3 nodes, tnx x tny x tnz of them, listed in
    // tile_order by the sum of their tile coordinates.  tiles == 0: the
    // pattern is not of that form.
    int tiles = 0;
    int lnx = 0, lny = 0, lnz = 0, tnx = 0, tny = 0, tnz = 0;
    int32_t* tile_order = nullptr;  // [tiles]
    // diagonal-offset form of the pattern (structured grids): the distinct
    // column offsets (col - row), sorted, and per SELL slot the index of
    // its offset (-1 for padding); n_off == 0 when there are too many
    int n_off = 0;
    int n_up = 0;                  // offsets >= 0 (the first is the diagonal)
    int32_t* up_off = nullptr;     // [n_up] offsets >= 0, ascending
    int8_t* slot_up = nullptr;     // [sell_nnz] index into up_off, -1 if col < row or padding
    std::vector<int32_t> host_up_off;
    double* tab = nullptr;         // shape table block (N, dN, w3)
    double* aff = nullptr;         // affine table block (Q, M0, dNc)
    ogs::ShapeTable host_tab;
};
