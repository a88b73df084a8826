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
//   CRFProcess::ExecuteNonLinear, RICHARDS_FLOW Picard (FEM/rf_pcs.cpp:9636)
//                                                 -> LinearEQS::RichardsStep
//   FEMRead / GEOLIB_Read_GeoLib / BCRead (MSH/msh_mesh.cpp:421,
//   FileIO/OGSIOVer4.cpp, FEM/rf_bc_new.cpp)      -> ogs_gpu::Deck
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

    // RICHARDS_FLOW: one time step by Picard iteration (CRFProcess::
    // ExecuteNonLinear); the collected SetKnownX_i rows are the Dirichlet
    // set, x() the first iterate in and the last one out.  Returns the stats;
    // throws unless the loop converged (or allow_fail).
    ogs_picard_stats RichardsStep(const ogs_assembly_params& p, const ogs_richards_params& r, const double* elem_k,
                                  const double* p_old, const ogs_picard_config& nls, bool allow_fail = false)
    {
        ogs_picard_stats st{};
        const ogs_status s = ogs_gpu_richards_step(h_, &p, &r, elem_k, p_old, x_.data(), known_rows_.data(),
                                                   known_vals_.data(), (int64_t)known_rows_.size(), mode_, &nls, &st);
        known_rows_.clear();
        known_vals_.clear();
        if (s != OGS_OK && !(allow_fail && s == OGS_NOT_CONVERGED)) check(s, "ogs_gpu_richards_step");
        return st;
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

// An OGS-5 deck read from disk (FEMRead / GEOLIB / BCRead): the mesh for
// Mesh, and the CONSTANT Dirichlet rows of a process for SetKnownX_i.
class Deck
{
public:
    Deck(const std::string& msh, const std::string& gli = "", const std::string& bc = "")
    {
        check(ogs_deck_read(msh.c_str(), gli.empty() ? nullptr : gli.c_str(), bc.empty() ? nullptr : bc.c_str(), &h_),
              "ogs_deck_read");
    }
    ~Deck() { ogs_deck_destroy(h_); }
    Deck(const Deck&) = delete;
    Deck& operator=(const Deck&) = delete;

    ogs_mesh_desc mesh_desc() const
    {
        ogs_mesh_desc d{};
        check(ogs_deck_mesh(h_, &d, nullptr), "ogs_deck_mesh");
        return d;
    }

    double min_edge_length() const
    {
        ogs_mesh_desc d{};
        double h = 0.0;
        ogs_deck_mesh(h_, &d, &h);
        return h;
    }

    // (row, value) pairs of every CONSTANT condition of the process, in the
    // order CRFProcess::bc_node_value holds them
    std::vector<std::pair<int64_t, double>> dirichlet(const std::string& pcs_type,
                                                      const std::string& primary_variable = "") const
    {
        const char* pv = primary_variable.empty() ? nullptr : primary_variable.c_str();
        int64_t n = 0;
        check(ogs_deck_dirichlet(h_, pcs_type.c_str(), pv, nullptr, nullptr, 0, &n), "ogs_deck_dirichlet");
        std::vector<int64_t> rows((size_t)n);
        std::vector<double> vals((size_t)n);
        check(ogs_deck_dirichlet(h_, pcs_type.c_str(), pv, rows.data(), vals.data(), n, &n), "ogs_deck_dirichlet");
        std::vector<std::pair<int64_t, double>> out;
        for (size_t k = 0; k < (size_t)n; k++) out.emplace_back(rows[k], vals[k]);
        return out;
    }

    const ogs_deck* handle() const { return h_; }

private:
    ogs_deck* h_ = nullptr;
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
