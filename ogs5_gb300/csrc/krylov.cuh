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
    unsigned int ticket[8];
    double part[8][2 * kMaxBlocks];
};

enum SolveKind
{
    SK_CG = 0,
    SK_BICGSTAB = 1
};

// Views of the matrix in the precision of the sweep.
template <typename T>
struct CsrView
{
    const int32_t* row_ptr;
    const int32_t* col;
    const T* val;
    int32_t n;
};

struct KrylovVecs
{
    double *x, *b, *r, *r0, *p, *ph, *s, *sh, *t, *v, *dinv;
    // ILU(0)
    const double* lu;           // factors on the CSR pattern
    const int32_t* diag_pos;
    const int32_t* lvl_rows;    // rows ordered by level (lower solve)
    const int32_t* lvl_ptr;     // level boundaries
    int n_levels;
    const int32_t* ulvl_rows;   // rows ordered by level (upper solve)
    const int32_t* ulvl_ptr;
    int n_ulevels;
};


struct SolveArgs
{
    CsrView<double> A;
    KrylovVecs v;
    KState* st;
    int precond;  // 0 none, 1 Jacobi
};

}  // namespace ogs
