// Drives the reference OGS-5, compiled from its own sources by refbuild.mk,
// through its public process and solver API and writes what it computes in
// binary, so that the tests can compare the GPU path and the C restatement
// with the reference itself.  TEST INFRASTRUCTURE ONLY.
//
// Usage:  ref_assemble_{sp,fem} <deck base path> <command file>
//
// The deck is read by the reference's own Problem constructor
// (FEM/problem.cpp:120; it reads .pcs .num .tim .mmp .mfp .mcp .msh .gli .bc
// .ic .st .out and creates the processes).  Then one command per line:
//
//   step <n> <dt>          time step n of length dt, as Euler_TimeDiscretize
//                          sets them (FEM/problem.cpp:1166-1200):
//                          aktueller_zeitschritt = n, the global dt (read by
//                          CalcSUPGCoefficient) and every process's
//                          Tim->time_step_length = dt, the time advanced
//   nodal <pcs> <level> <file>  primary variable of process <pcs> (index in
//                          pcs_vector) from a file of n_nodes doubles
//                          (CRFProcess::SetNodeValue); level 0 the old time
//                          level, 1 the new one (the Picard iterate), 2 both
//   velocity_in <file>     Gauss-point Darcy flux of every element,
//                          n_elements * n_gp * 3 doubles, written into
//                          ele_gp_value[e]->Velocity(d, gp), gp < n_gp (the
//                          matrix has room for more points than a linear
//                          element's rule uses)
//   assemble <pcs> <out>   the preamble of CRFProcess::Execute
//                          (rf_pcs.cpp:4730-4800: SetDOF, ConfigNumerics,
//                          Initialize, x from the node values), then
//                          CRFProcess::GlobalAssembly (:5626, with source
//                          terms and Dirichlet conditions), then
//                          Linear_EQS::Write_BIN (equation_class.cpp:409)
//   solve <out>            after `assemble`: Linear_EQS::Solver()
//                          (equation_class.cpp:857), writes int64 iterations
//                          and x (n doubles)
//   execute <pcs> <out>    CRFProcess::Execute (rf_pcs.cpp:4695: assembly,
//                          solve, node values updated), then the assembled
//                          system (Write_BIN), int64 linear iterations
//                          (iter_lin) and the new primary variable (n
//                          doubles; Execute reuses Linear_EQS::x afterwards)
//   nonlinear <pcs> <out>  CRFProcess::ExecuteNonLinear (rf_pcs.cpp:9636),
//                          writes int64 Picard iterations, int64 linear
//                          iterations of the last one, and the new primary
//                          variable (n doubles)
//   velocity_out <pcs> <n_gp> <out>  CRFProcess::CalIntegrationPointValue
//                          (rf_pcs.cpp:5915) with the current node values,
//                          then ele_gp_value velocities as velocity_in
//   legacy_execute <pcs> <out>  (FEM configuration) CRFProcess::Execute with
//                          the legacy RF solver; writes int64 iterations and
//                          the new primary variable
//
// In the SP configuration (NEW_EQS) Write_BIN writes long rows, long
// row_ptr[rows+1], long col[nnz], double val[nnz], then double b[rows].
#include <cfloat>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

// The harness reads members the reference keeps protected or private
// (CRFProcess::eqs_new, Tim; Linear_EQS::x).  Access specifiers do not change
// the layout GCC gives these classes, so the reference's own objects, compiled
// without this, are read as they are.
#define protected public
#define private public
#include "FileTools.h"
#include "fem_ele_std.h"
#include "msh_mesh.h"
#include "problem.h"
#include "rf_pcs.h"
#include "rf_tim_new.h"
#ifdef NEW_EQS
#include "equation_class.h"
#endif

extern std::string FileName;
extern std::string FilePath;
extern std::string defaultOutputPath;

namespace
{
std::vector<double> read_doubles(const std::string& path)
{
    std::ifstream f(path.c_str(), std::ios::binary);
    if (!f.good())
    {
        std::fprintf(stderr, "harness: cannot read %s\n", path.c_str());
        std::exit(2);
    }
    f.seekg(0, std::ios::end);
    const std::streamoff bytes = f.tellg();
    f.seekg(0, std::ios::beg);
    std::vector<double> v(static_cast<size_t>(bytes) / sizeof(double));
    f.read(reinterpret_cast<char*>(v.data()), v.size() * sizeof(double));
    return v;
}

CRFProcess* pcs_at(int i)
{
    if (i < 0 || i >= static_cast<int>(pcs_vector.size()))
    {
        std::fprintf(stderr, "harness: no process %d\n", i);
        std::exit(2);
    }
    return pcs_vector[i];
}

void set_nodal(CRFProcess* pcs, const std::vector<double>& v, int level)
{
    const long n = pcs->m_msh->GetNodesNumber(false);
    if (static_cast<long>(v.size()) != n)
    {
        std::fprintf(stderr, "harness: %zu nodal values for %ld nodes\n", v.size(), n);
        std::exit(2);
    }
    const int idx0 = pcs->GetNodeValueIndex(pcs->pcs_primary_function_name[0]);
    for (long k = 0; k < n; ++k)
    {
        if (level != 1)
            pcs->SetNodeValue(k, idx0, v[k]);
        if (level != 0)
            pcs->SetNodeValue(k, idx0 + 1, v[k]);
    }
}

void write_primary(CRFProcess* pcs, std::ofstream& out)
{
    const long n = pcs->m_msh->GetNodesNumber(false);
    const int idx1 = pcs->GetNodeValueIndex(pcs->pcs_primary_function_name[0]) + 1;
    for (long k = 0; k < n; ++k)
    {
        const double v = pcs->GetNodeValue(k, idx1);
        out.write(reinterpret_cast<const char*>(&v), sizeof(double));
    }
}

#ifdef NEW_EQS
// The part of CRFProcess::Execute before GlobalAssembly (rf_pcs.cpp:4730-4800)
// for a linear process outside a non-linear loop.
void execute_preamble(CRFProcess* pcs)
{
    Linear_EQS* eqs = pcs->eqs_new;
    eqs->SetDOF(pcs->pcs_number_of_primary_nvals);
    eqs->ConfigNumerics(pcs->m_num);
    eqs->Initialize();
    const long n = pcs->m_msh->GetNodesNumber(false);
    const int idx1 = pcs->GetNodeValueIndex(pcs->pcs_primary_function_name[0]) + 1;
    for (long j = 0; j < n; ++j)
        eqs->x[j] = pcs->GetNodeValue(pcs->m_msh->Eqs2Global_NodeIndex[j], idx1);
}
#endif

void write_velocities(std::ofstream& out, int ngp)
{
    for (size_t e = 0; e < ele_gp_value.size(); ++e)
    {
        FiniteElement::ElementValue* ev = ele_gp_value[e];
        const int dim = static_cast<int>(ev->Velocity.Rows());
        for (int g = 0; g < ngp; ++g)
            for (int d = 0; d < 3; ++d)
            {
                const double v = d < dim ? ev->Velocity(d, g) : 0.0;
                out.write(reinterpret_cast<const char*>(&v), sizeof(double));
            }
    }
}
}  // namespace

int main(int argc, char* argv[])
{
    if (argc != 3)
    {
        std::fprintf(stderr, "usage: %s <deck base path> <command file>\n", argv[0]);
        return 2;
    }
    FileName = argv[1];
    FilePath = pathDirname(FileName);
    defaultOutputPath = FilePath;
    FilePath = FilePath + getDirSep();

    Problem* problem = new Problem(FileName.data());
    std::ifstream cmds(argv[2]);
    std::string line;
    while (std::getline(cmds, line))
    {
        std::istringstream in(line);
        std::string cmd;
        if (!(in >> cmd) || cmd[0] == '#')
            continue;
        std::fprintf(stderr, "harness: %s\n", line.c_str());
        if (cmd == "step")
        {
            long n = 1;
            double dt = 0.0;
            in >> n >> dt;
            aktueller_zeitschritt = static_cast<size_t>(n);
            ::dt = dt;
            for (size_t i = 0; i < pcs_vector.size(); ++i)
                if (pcs_vector[i]->Tim)
                    pcs_vector[i]->Tim->time_step_length = dt;
            aktuelle_zeit += dt;
        }
        else if (cmd == "nodal")
        {
            int i = 0, level = 2;
            std::string path;
            in >> i >> level >> path;
            set_nodal(pcs_at(i), read_doubles(path), level);
        }
        else if (cmd == "velocity_in")
        {
            std::string path;
            in >> path;
            const std::vector<double> v = read_doubles(path);
            const size_t ne = ele_gp_value.size();
            const int ngp = ne ? static_cast<int>(v.size() / (3 * ne)) : 0;
            size_t k = 0;
            for (size_t e = 0; e < ne; ++e)
            {
                FiniteElement::ElementValue* ev = ele_gp_value[e];
                if (ngp > static_cast<int>(ev->Velocity.Cols()))
                {
                    std::fprintf(stderr, "harness: %d Gauss points, room for %d\n", ngp,
                                 static_cast<int>(ev->Velocity.Cols()));
                    return 2;
                }
                const int dim = static_cast<int>(ev->Velocity.Rows());
                for (int g = 0; g < ngp; ++g)
                    for (int d = 0; d < 3; ++d, ++k)
                        if (d < dim && k < v.size())
                            ev->Velocity(d, g) = v[k];
            }
            if (k != v.size())
            {
                std::fprintf(stderr, "harness: %zu velocity values, %zu expected\n", v.size(), k);
                return 2;
            }
        }
#ifdef NEW_EQS
        else if (cmd == "assemble")
        {
            int i = 0;
            std::string path;
            in >> i >> path;
            CRFProcess* pcs = pcs_at(i);
            execute_preamble(pcs);
            pcs->GlobalAssembly();
            std::ofstream out(path.c_str(), std::ios::binary | std::ios::trunc);
            pcs->eqs_new->Write_BIN(out);
        }
        else if (cmd == "solve")
        {
            int i = 0;
            std::string path;
            in >> i >> path;
            CRFProcess* pcs = pcs_at(i);
            const int64_t iters = pcs->eqs_new->Solver();
            std::ofstream out(path.c_str(), std::ios::binary | std::ios::trunc);
            out.write(reinterpret_cast<const char*>(&iters), sizeof(iters));
            const long n = pcs->m_msh->GetNodesNumber(false);
            out.write(reinterpret_cast<const char*>(pcs->eqs_new->x), n * sizeof(double));
        }
        else if (cmd == "execute")
        {
            int i = 0;
            std::string path;
            in >> i >> path;
            CRFProcess* pcs = pcs_at(i);
            pcs->Execute();
            std::ofstream out(path.c_str(), std::ios::binary | std::ios::trunc);
            pcs->eqs_new->Write_BIN(out);
            const int64_t iters = pcs->iter_lin;
            out.write(reinterpret_cast<const char*>(&iters), sizeof(iters));
            write_primary(pcs, out);
        }
#endif
        else if (cmd == "legacy_execute")
        {
            int i = 0;
            std::string path;
            in >> i >> path;
            CRFProcess* pcs = pcs_at(i);
            pcs->Execute();
            std::ofstream out(path.c_str(), std::ios::binary | std::ios::trunc);
            const int64_t iters = pcs->iter_lin;
            out.write(reinterpret_cast<const char*>(&iters), sizeof(iters));
            write_primary(pcs, out);
        }
        else if (cmd == "nonlinear")
        {
            int i = 0;
            std::string path;
            in >> i >> path;
            CRFProcess* pcs = pcs_at(i);
            pcs->ExecuteNonLinear(0, true);
            std::ofstream out(path.c_str(), std::ios::binary | std::ios::trunc);
            const int64_t it = pcs->iter_nlin;
            const int64_t lin = pcs->iter_lin;
            out.write(reinterpret_cast<const char*>(&it), sizeof(it));
            out.write(reinterpret_cast<const char*>(&lin), sizeof(lin));
            write_primary(pcs, out);
        }
        else if (cmd == "velocity_out")
        {
            int i = 0, ngp = 0;
            std::string path;
            in >> i >> ngp >> path;
            pcs_at(i)->CalIntegrationPointValue();
            std::ofstream out(path.c_str(), std::ios::binary | std::ios::trunc);
            write_velocities(out, ngp);
        }
        else
        {
            std::fprintf(stderr, "harness: unknown command '%s'\n", cmd.c_str());
            return 2;
        }
    }
    delete problem;
    return 0;
}
