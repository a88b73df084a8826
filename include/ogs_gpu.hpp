// ogs_gpu.hpp -- C++ mirror of the OGS-5 solver surface over the C ABI of
// ogs_gpu.h (header only, no CUDA headers needed by the including code).
//
// The names and argument meanings follow the reference so that a GPU build
// of CRFProcess changes call sites, not logic:
//
//   Linear_EQS (FEM/equation_class.h:56-197)      -> ogs_gpu::LinearEQS
//     ConfigNumerics(CNumerics*)  equation_class.cpp:191-318
//     Initialize()                equation_class.cpp:325-332   (A = 0, b = 0)
//     SetKnownX_i(i, x)           equation_class.cpp:926-929   (Dirichlet row)
//     Solver()                    equation_class.cpp:857-895   (returns iterations)
//     X(i), RHS(i)                equation_class.h:122-123
//     Write_BIN CRS arrays        equation_class.cpp:409
//   CRFProcess::GlobalAssembly element loop (FEM/rf_pcs.cpp:5738-5757)
//                                                 -> LinearEQS::GlobalAssembly
//   CRFProcess::CalIntegrationPointValue (FEM/rf_pcs.cpp:5915)
//                                                 -> LinearEQS::GaussPointVelocity
//
// SetKnownX_i rows are collected and applied as one set (the same result as
// the reference's row-by-row Diagonize, a row given twice keeping its last
// value) before the next Solver() or matrix read-back.  Errors throw
// ogs_gpu::Error carrying the ogs_status and the library's message; the
// reference exits or prints a warning instead.
#ifndef OGS_GPU_HPP
#define OGS_GPU_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ogs_gpu.h"

namespace ogs_gpu
{

class Error : public std::runtime_error
{
public:
    Error(ogs_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    ogs_status status;
};

inline void check(ogs_status s, const char* where)
{
    if (s != OGS_OK)
    {
        const char* m = ogs_gpu_last_error();
        throw Error(s, std::string(where) + ": " + (m ? m : "error"));
    }
}

// CNumerics fields read by Linear_EQS::ConfigNumerics (FEM/rf_num_new.h:34-60),
// with the CNumerics defaults (FEM/rf_num_new.cpp:77-165)
struct Numerics
{
    int ls_method = OGS_LS_BICGSTAB;
    int ls_precond = OGS_PRECOND_JACOBI;
    int ls_max_iterations = 1000;
    double ls_error_tolerance = 1e-12;
    int precision = OGS_PRECISION_FP64;  // extension: OGS_PRECISION_FP32_REFINED
    double inner_tol = 0.0;
    bool check_norm_rhs = true;
};

// Node coordinates and element connectivity as CFEMesh hands them to
// SparseTable and the element loop; owns the device pattern and slot map.
class Mesh
{
public:
    Mesh(ogs_elem_type type, int dim, const std::vector<double>& x, const std::vector<double>& y,
         const std::vector<double>& z, const std::vector<int32_t>& connectivity, int gauss_points = 3)
    {
        const int nn = type == OGS_ELEM_HEX8 ? 8 : 4;
        ogs_mesh_desc d{};
        d.elem_type = type;
        d.dim = dim;
        d.n_nodes = (int64_t)x.size();
        d.n_elements = (int64_t)(connectivity.size() / nn);
        d.x = x.data();
        d.y = y.data();
        d.z = z.empty() ? nullptr : z.data();
        d.connectivity = connectivity.data();
        d.gauss_points = gauss_points;
        check(ogs_gpu_mesh_create(&d, &h_), "ogs_gpu_mesh_create");
        n_elements_ = d.n_elements;
        check(ogs_gpu_mesh_info(h_, &n_nodes_, &nnz_), "ogs_gpu_mesh_info");
    }
    ~Mesh() { if (h_) ogs_gpu_mesh_destroy(h_); }
    Mesh(const Mesh&) = delete;
    Mesh& operator=(const Mesh&) = delete;

    ogs_mesh* handle() const { return h_; }
    int64_t nodes() const { return n_nodes_; }
    int64_t elements() const { return n_elements_; }
    int64_t nnz() const { return nnz_; }
    int gauss_points() const { return ogs_gpu_mesh_gauss_points(h_); }

private:
    ogs_mesh* h_ = nullptr;
    int64_t n_nodes_ = 0, n_elements_ = 0, nnz_ = 0;
};

// Linear_EQS over one mesh: A, b and x live on the device; x() holds the
// host copy of the last solution (eqs_new->x of the reference).
class LinearEQS
{
public:
    explicit LinearEQS(const Mesh& mesh, void* stream = nullptr) : mesh_(mesh)
    {
        check(ogs_gpu_system_create(mesh.handle(), stream, &h_), "ogs_gpu_system_create");
        x_.assign((size_t)mesh.nodes(), 0.0);
    }
    ~LinearEQS() { if (h_) ogs_gpu_system_destroy(h_); }
    LinearEQS(const LinearEQS&) = delete;
    LinearEQS& operator=(const LinearEQS&) = delete;

    void ConfigNumerics(const Numerics& num)
    {
        ogs_solver_config c{};
        c.method = num.ls_method;
        c.precond = num.ls_precond;
        c.max_iter = num.ls_max_iterations;
        c.precision = num.precision;
        c.tol = num.ls_error_tolerance;
        c.inner_tol = num.inner_tol;
        c.check_norm_rhs = num.check_norm_rhs ? 1 : 0;
        check(ogs_gpu_configure(h_, &c), "ogs_gpu_configure");
    }

    void Initialize()
    {
        check(ogs_gpu_initialize(h_), "ogs_gpu_initialize");
        known_rows_.clear();
        known_vals_.clear();
    }

    // element loop + scatter of CRFProcess::GlobalAssembly; elem_k per
    // element (flow), u0 the previous time level, gp_velocity the Darcy flux
    // at the Gauss points (transport)
    void GlobalAssembly(const ogs_assembly_params& p, const double* elem_k, const double* u0,
                        const double* gp_velocity = nullptr)
    {
        check(ogs_gpu_assemble(h_, &p, elem_k, u0, gp_velocity), "ogs_gpu_assemble");
    }

    // forget the transport operators stored under memory_type > 0
    void ResetOperators() { check(ogs_gpu_cache_reset(h_), "ogs_gpu_cache_reset"); }

    void SetKnownX_i(long i, double x)
    {
        known_rows_.push_back((int64_t)i);
        known_vals_.push_back(x);
    }

    // Dirichlet mode of the collected rows: OGS_DIRICHLET_ROW_ONLY is the SP
    // build's Diagonize, OGS_DIRICHLET_SYMMETRIC the legacy MXRandbed
    void SetDirichletMode(ogs_dirichlet_mode m) { mode_ = m; }

    // Linear_EQS::Solver: x() is the initial guess in, the solution out;
    // returns the iteration count
    int Solver()
    {
        flush_known();
        ogs_solve_stats st{};
        const ogs_status s = ogs_gpu_solve(h_, x_.data(), &st);
        stats_ = st;
        if (s != OGS_OK && s != OGS_NOT_CONVERGED) check(s, "ogs_gpu_solve");
        return st.iterations;
    }

    std::vector<double>& x() { return x_; }
    double X(long i) const { return x_[(size_t)i]; }
    const ogs_solve_stats& stats() const { return stats_; }

    std::vector<double> RHS()
    {
        flush_known();
        std::vector<double> b((size_t)mesh_.nodes());
        check(ogs_gpu_get_rhs(h_, b.data()), "ogs_gpu_get_rhs");
        return b;
    }

    // CRS arrays of Linear_EQS::Write_BIN
    void CRS(std::vector<int64_t>& row_ptr, std::vector<int64_t>& col, std::vector<double>& val)
    {
        flush_known();
        row_ptr.resize((size_t)mesh_.nodes() + 1);
        col.resize((size_t)mesh_.nnz());
        val.resize((size_t)mesh_.nnz());
        check(ogs_gpu_get_csr(h_, row_ptr.data(), col.data(), val.data()), "ogs_gpu_get_csr");
    }

    // q = -mat grad(u) at every Gauss point: elements x gauss points x 3
    std::vector<double> GaussPointVelocity(const ogs_assembly_params& p, const double* elem_k,
                                           const double* u)
    {
        std::vector<double> q((size_t)mesh_.elements() * mesh_.gauss_points() * 3);
        check(ogs_gpu_gp_velocity(h_, &p, elem_k, u, q.data()), "ogs_gpu_gp_velocity");
        return q;
    }

    ogs_system* handle() const { return h_; }

private:
    void flush_known()
    {
        if (known_rows_.empty()) return;
        check(ogs_gpu_set_dirichlet(h_, known_rows_.data(), known_vals_.data(), (int64_t)known_rows_.size(),
                                    mode_),
              "ogs_gpu_set_dirichlet");
        known_rows_.clear();
        known_vals_.clear();
    }

    const Mesh& mesh_;
    ogs_system* h_ = nullptr;
    std::vector<double> x_;
    std::vector<int64_t> known_rows_;
    std::vector<double> known_vals_;
    ogs_dirichlet_mode mode_ = OGS_DIRICHLET_ROW_ONLY;
    ogs_solve_stats stats_{};
};

// assembly parameters with the defaults of an OGS-5 deck
inline ogs_assembly_params make_params(ogs_pcs_type pcs)
{
    ogs_assembly_params p{};
    p.pcs_type = pcs;
    p.dt = 1.0;
    p.theta = 1.0;
    p.time_unit_factor = 1.0;
    p.viscosity = 1.0e-3;
    p.density = 1000.0;
    p.retardation = 1.0;
    p.saturation = 1.0;
    return p;
}

}  // namespace ogs_gpu

#endif  // OGS_GPU_HPP
