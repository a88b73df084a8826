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
    double* q_out;      // velocity kernel output [e][gp][3]
    int* bad_elem;      // first element with a singular Jacobian + 1
    ogs_assembly_params p;
};

}  // namespace ogs

struct ogs_mesh
{
    int elem_type = 0, dim = 3, nn = 8, ngauss = 3, ngp = 27;
    int64_t n_nodes = 0, n_elem = 0;
    int64_t nnz = 0;
    bool affine = false;      // every element has a constant Jacobian
    int device = 0;
    // device arrays
    double *x = nullptr, *y = nullptr, *z = nullptr;
    int32_t* conn_t = nullptr;   // [nn][n_elem]
    int32_t* row_ptr = nullptr;  // [n_nodes+1]
    int32_t* col = nullptr;      // [nnz]
    int32_t* diag_pos = nullptr; // [n_nodes]
    int32_t* slot_t = nullptr;   // [nn*nn][n_elem]
    double* tab = nullptr;       // shape table block (N, dN, w3)
    double* aff = nullptr;       // affine table block (Q, M0, dNc)
    ogs::ShapeTable host_tab;
    // structured 27/9-point form (hex/quad box meshes): diagonal offsets
    int n_diag = 0;
    int32_t* dia_off = nullptr;  // [n_diag] column offset of each diagonal
    int32_t* dia_slot = nullptr; // [n_diag][n_nodes] CSR slot or -1
};
