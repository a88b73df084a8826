/*
 * ref_harness.cpp -- C entry points into the reference's own compiled code.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together
 * with three unmodified OGS-5 sources -- FEM/mathlib.cpp (Gauss points,
 * shape functions), FEM/matrix_class.cpp (SparseTable, CSparseMatrix) and
 * FEM/equation_class.cpp (Linear_EQS and its Krylov solvers) -- into
 * oracle/_ref/libogs5ref.so.  Tests use it to pin oracle/ogs_oracle.c and,
 * through it, the GPU library.
 *
 * SparseTable is normally built from a CFEMesh (matrix_class.cpp:691); the
 * mesh library is not part of this build, so the harness fills the CRS
 * members of a SparseTable directly, exactly as the CRS branch of that
 * constructor leaves them (num_column_entries = row pointer, entry_column =
 * column indices, diag_entry = diagonal position; matrix_class.cpp:741-776).
 * Linear_EQS is then constructed, configured and solved through its own
 * public methods.  CNumerics is only read for POD fields by
 * Linear_EQS::ConfigNumerics (equation_class.cpp:191-318), so a zeroed
 * object with those fields set stands in for one read from a .num file.
 */
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#define private public
#define protected public
#include "matrix_class.h"
#include "equation_class.h"
#include "rf_num_new.h"
#undef private
#undef protected

/* FEM/mathlib.cpp, declared in FEM/mathlib.h */
extern double MXPGaussPkt(long grd, long pkt);
extern double MXPGaussFkt(long grd, long pkt);
extern void SamplePointTet5(const int nsample, double* SPoint);
extern void ShapeFunctionQuad(double* N4, const double* u);
extern void GradShapeFunctionQuad(double* dN4, const double* u);
extern void ShapeFunctionHex(double* N8, const double* x);
extern void GradShapeFunctionHex(double* dN8, const double* x);
extern void ShapeFunctionTet(double* Nt4, const double* x);
extern void GradShapeFunctionTet(double* dNt4, const double* dummy);

/* Symbols that mathlib.cpp references from libraries outside this build;
 * none of the functions called here reaches them. */
double MSkalarprodukt(double*, double*, long) { std::abort(); }
void M3KreuzProdukt(double*, double*, double*) { std::abort(); }
double MCalcDistancePointToPoint(double*, double*) { std::abort(); }
namespace Display
{
void DisplayErrorMsg(const char*) { std::abort(); }
}

using Math_Group::CSparseMatrix;
using Math_Group::Linear_EQS;
using Math_Group::SparseTable;

extern "C" {

double ref_gauss_point(long grd, long pkt) { return MXPGaussPkt(grd, pkt); }
double ref_gauss_weight(long grd, long pkt) { return MXPGaussFkt(grd, pkt); }
void ref_tet5_point(int n, double* sp) { SamplePointTet5(n, sp); }

/* etype 0 quad, 1 hex, 2 tet: N and dN/dxi at local point u */
void ref_shape(int etype, const double* u, double* N, double* dN)
{
    if (etype == 0)
    {
        ShapeFunctionQuad(N, u);
        GradShapeFunctionQuad(dN, u);
    }
    else if (etype == 1)
    {
        ShapeFunctionHex(N, u);
        GradShapeFunctionHex(dN, u);
    }
    else
    {
        ShapeFunctionTet(N, u);
        GradShapeFunctionTet(dN, u);
    }
}

struct ref_system
{
    SparseTable* table;
    Linear_EQS* eqs;
    CNumerics* num;
};

/* A CRS SparseTable over the given pattern, a Linear_EQS on it, configured
 * with ls_method / ls_precond / max_iter / tol.  Returns an opaque handle. */
void* ref_system_create(long n, const long* row_ptr, const long* col,
                        int ls_method, int ls_precond, int max_iter, double tol)
{
    ref_system* s = new ref_system;
    s->table = static_cast<SparseTable*>(std::calloc(1, sizeof(SparseTable)));
    SparseTable* t = s->table;
    t->symmetry = false;
    t->storage_type = Math_Group::CRS;
    t->rows = n;
    t->size_entry_column = row_ptr[n];
    t->max_columns = 0;
    t->num_column_entries = new long[n + 1];
    t->entry_column = new long[row_ptr[n]];
    t->diag_entry = new long[n];
    t->row_index_mapping_n2o = NULL;
    t->row_index_mapping_o2n = NULL;
    for (long i = 0; i <= n; i++) t->num_column_entries[i] = row_ptr[i];
    for (long k = 0; k < row_ptr[n]; k++) t->entry_column[k] = col[k];
    for (long i = 0; i < n; i++)
        for (long k = row_ptr[i]; k < row_ptr[i + 1]; k++)
            if (col[k] == i) t->diag_entry[i] = k;
    s->eqs = new Linear_EQS(*t, 1, false);
    s->num = static_cast<CNumerics*>(std::calloc(1, sizeof(CNumerics)));
    s->num->ls_method = ls_method;
    s->num->ls_precond = ls_precond;
    s->num->ls_max_iterations = max_iter;
    s->num->ls_error_tolerance = tol;
    s->num->nls_method = 0;
    s->eqs->ConfigNumerics(s->num);
    return s;
}

void ref_system_destroy(void* h)
{
    ref_system* s = static_cast<ref_system*>(h);
    delete s->eqs;
    delete[] s->table->num_column_entries;
    delete[] s->table->entry_column;
    delete[] s->table->diag_entry;
    std::free(s->table);
    std::free(s->num);
    delete s;
}

/* Linear_EQS::Initialize, then A and b set to the given values */
void ref_system_set(void* h, const double* val, const double* b)
{
    ref_system* s = static_cast<ref_system*>(h);
    s->eqs->Initialize();
    const long nnz = s->table->size_entry_column;
    for (long k = 0; k < nnz; k++) s->eqs->A->entry[k] = val[k];
    for (long i = 0; i < s->eqs->size_A; i++) s->eqs->b[i] = b[i];
}

/* element-matrix scatter through CSparseMatrix::operator() + b */
void ref_system_add(void* h, long r, long c, double v)
{
    ref_system* s = static_cast<ref_system*>(h);
    (*s->eqs->A)(r, c) += v;
}

/* Linear_EQS::SetKnownX_i -> CSparseMatrix::Diagonize */
void ref_system_set_known(void* h, long i, double v)
{
    static_cast<ref_system*>(h)->eqs->SetKnownX_i(i, v);
}

void ref_system_get(void* h, double* val, double* b)
{
    ref_system* s = static_cast<ref_system*>(h);
    const long nnz = s->table->size_entry_column;
    if (val)
        for (long k = 0; k < nnz; k++) val[k] = s->eqs->A->entry[k];
    if (b)
        for (long i = 0; i < s->eqs->size_A; i++) b[i] = s->eqs->b[i];
}

/* CSparseMatrix::multiVec */
void ref_system_spmv(void* h, const double* x, double* y)
{
    ref_system* s = static_cast<ref_system*>(h);
    std::vector<double> xs(x, x + s->eqs->size_A);
    s->eqs->A->multiVec(xs.data(), y);
}

/* Linear_EQS::Solver with x as initial guess.  out: [return value of
 * Solver(), iter, error, bNorm]. */
void ref_system_solve(void* h, double* x, double* out)
{
    ref_system* s = static_cast<ref_system*>(h);
    for (long i = 0; i < s->eqs->size_A; i++) s->eqs->x[i] = x[i];
    const int ret = s->eqs->Solver();
    for (long i = 0; i < s->eqs->size_A; i++) x[i] = s->eqs->x[i];
    out[0] = ret;
    out[1] = s->eqs->iter;
    out[2] = s->eqs->error;
    out[3] = s->eqs->bNorm;
}

/* Linear_EQS::Write_BIN into a buffer (capacity bytes); returns bytes */
long ref_system_write_bin(void* h, char* buf, long capacity)
{
    ref_system* s = static_cast<ref_system*>(h);
    std::ostringstream os(std::ios::binary);
    s->eqs->Write_BIN(os);
    const std::string d = os.str();
    const long n = static_cast<long>(d.size());
    if (buf && capacity >= n) std::memcpy(buf, d.data(), n);
    return n;
}

}  // extern "C"
