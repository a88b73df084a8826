// The 100 x 100 quad deck (steady GROUNDWATER_FLOW, K = 1e-4, h = 1 at x = 0
// and 0 at x = 100, BiCGStab + Jacobi to 1e-10) driven through the C++
// mirror of Linear_EQS, the way CRFProcess::Execute drives the reference:
// Initialize, GlobalAssembly, SetKnownX_i per boundary node, Solver, X(i).
// The bilinear solution is exact: h = 1 - x / 100.
#include <cmath>
#include <cstdio>
#include <vector>

#include "ogs_gpu.hpp"

int main()
{
    const int n = 100;
    std::vector<double> x, y, z;
    for (int j = 0; j <= n; j++)
        for (int i = 0; i <= n; i++)
        {
            x.push_back(i);
            y.push_back(j);
        }
    std::vector<int32_t> conn;
    auto id = [&](int i, int j) { return (int32_t)(i + (n + 1) * j); };
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
        {
            const int32_t e[4] = {id(i, j), id(i + 1, j), id(i + 1, j + 1), id(i, j + 1)};
            conn.insert(conn.end(), e, e + 4);
        }
    try
    {
        ogs_gpu::Mesh mesh(OGS_ELEM_QUAD4, 2, x, y, z, conn);
        ogs_gpu::LinearEQS eqs(mesh);
        ogs_gpu::Numerics num;
        num.ls_method = OGS_LS_BICGSTAB;
        num.ls_precond = OGS_PRECOND_JACOBI;
        num.ls_max_iterations = 1000;
        num.ls_error_tolerance = 1e-10;
        eqs.ConfigNumerics(num);
        eqs.Initialize();
        ogs_assembly_params p = ogs_gpu::make_params(OGS_PCS_GROUNDWATER_FLOW);
        p.steady = 1;
        std::vector<double> k(mesh.elements(), 1e-4), u0(mesh.nodes(), 0.0);
        eqs.GlobalAssembly(p, k.data(), u0.data());
        for (long q = 0; q < mesh.nodes(); q++)
        {
            if (x[q] == 0.0) eqs.SetKnownX_i(q, 1.0);
            if (x[q] == n) eqs.SetKnownX_i(q, 0.0);
        }
        std::vector<int64_t> rp, col;
        std::vector<double> val;
        eqs.CRS(rp, col, val);
        for (auto& v : eqs.x()) v = 0.5;
        const int iters = eqs.Solver();
        double err = 0.0;
        for (long q = 0; q < mesh.nodes(); q++) err = std::fmax(err, std::fabs(eqs.X(q) - (1.0 - x[q] / n)));
        std::printf("nnz %lld iterations %d rel_residual %.3e max_err %.3e\n", (long long)rp.back(), iters,
                    eqs.stats().rel_residual, err);
        const bool ok = rp.back() == 301LL * 301LL && eqs.stats().status == OGS_OK && err < 1e-8 && iters > 0;
        std::printf("%s\n", ok ? "PASS" : "FAIL");
        return ok ? 0 : 1;
    }
    catch (const ogs_gpu::Error& e)
    {
        std::printf("FAIL: %s\n", e.what());
        return 2;
    }
}
