// mesh.cu -- shape tables, CSR pattern and element -> CSR slot map.
//
// Replaces, once per mesh, what OGS-5 does per run and per entry:
//   CFEMesh::ConnectedNodes           MSH/msh_mesh.cpp:2931-2980
//   SparseTable::SparseTable (CRS)    FEM/matrix_class.cpp:691-776
//   CSparseMatrix::operator() search  FEM/matrix_class.cpp:1178-1237
// The slot map stores, for every element and local pair (i, j), the CSR
// position of (node_i, node_j); the assembly kernels scatter through it
// without searching.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <thread>

#include "common.cuh"

namespace ogs {

static thread_local std::string g_error;
static thread_local int64_t g_launches = 0;

void set_error(const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
}
const char* last_error() { return g_error.c_str(); }
void count_launches(int64_t n) { g_launches += n; }
int64_t launches(int reset)
{
    int64_t v = g_launches;
    if (reset) g_launches = 0;
    return v;
}

// ---------------------------------------------------------------------
// Shape functions: MXPGaussPkt/MXPGaussFkt (FEM/mathlib.cpp:1112,1174),
// SamplePointTet5 (:1285), ShapeFunctionQuad/Hex/Tet and their gradients
// (:1880,1908,2079,2103,2224,2264).  Same constants, same node order.
// ---------------------------------------------------------------------
static double gauss_point(int grd, int pkt)
{
    switch (grd)
    {
        case 1: return 0.0;
        case 2: return pkt == 0 ? 0.577350269189626 : -0.577350269189626;
        case 3: return pkt == 0 ? 0.774596669241483 : (pkt == 1 ? 0.0 : -0.774596669241483);
    }
    return 0.0;
}
static double gauss_weight(int grd, int pkt)
{
    switch (grd)
    {
        case 1: return 2.0;
        case 2: return 1.0;
        case 3: return pkt == 1 ? 0.888888888888889 : 0.555555555555556;
    }
    return 0.0;
}
static void tet5_point(int n, double* sp)
{
    const double a = 0.166666666666667;
    const double pts[5][4] = {{0.25, 0.25, 0.25, -0.133333333333333},
                              {a, a, a, 0.075},
                              {0.5, a, a, 0.075},
                              {a, 0.5, a, 0.075},
                              {a, a, 0.5, 0.075}};
    for (int i = 0; i < 4; i++) sp[i] = pts[n][i];
}
// local node coordinates implied by the shape functions
static const double kQuadNode[4][2] = {{1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
static const double kHexNode[8][3] = {{1, 1, 1},   {-1, 1, 1},  {-1, -1, 1},
                                      {1, -1, 1},  {1, 1, -1},  {-1, 1, -1},
                                      {-1, -1, -1}, {1, -1, -1}};

static void shape_eval(int et, const double* u, double* N, double* dN)
{
    if (et == OGS_ELEM_QUAD4)
    {
        for (int i = 0; i < 4; i++)
        {
            const double a = kQuadNode[i][0], b = kQuadNode[i][1];
            N[i] = 0.25 * ((1.0 + a * u[0]) * (1.0 + b * u[1]));
            dN[i] = 0.25 * (a * (1.0 + b * u[1]));
            dN[4 + i] = 0.25 * (b * (1.0 + a * u[0]));
        }
    }
    else if (et == OGS_ELEM_HEX8)
    {
        for (int i = 0; i < 8; i++)
        {
            const double a = kHexNode[i][0], b = kHexNode[i][1], c = kHexNode[i][2];
            N[i] = 0.125 * ((1.0 + a * u[0]) * (1.0 + b * u[1]) * (1.0 + c * u[2]));
            dN[i] = 0.125 * (a * (1.0 + b * u[1]) * (1.0 + c * u[2]));
            dN[8 + i] = 0.125 * (b * (1.0 + a * u[0]) * (1.0 + c * u[2]));
            dN[16 + i] = 0.125 * (c * (1.0 + a * u[0]) * (1.0 + b * u[1]));
        }
    }
    else
    {
        N[0] = 1. - u[0] - u[1] - u[2];
        N[1] = u[0];
        N[2] = u[1];
        N[3] = u[2];
        const double g[12] = {-1, 1, 0, 0, -1, 0, 1, 0, -1, 0, 0, 1};
        for (int i = 0; i < 12; i++) dN[i] = g[i];
    }
}

ShapeTable make_shape_table(int et, int ngauss)
{
    ShapeTable t;
    t.nn = nodes_per_element(et);
    t.dim = elem_dim(et);
    t.ngp = num_gauss_points(et, ngauss);
    t.N.assign(t.ngp * t.nn, 0.0);
    t.dN.assign(t.ngp * t.nn * t.dim, 0.0);
    t.w3.assign(t.ngp * 3, 1.0);
    t.wprod.assign(t.ngp, 0.0);
    for (int gp = 0; gp < t.ngp; gp++)
    {
        double u[4] = {0, 0, 0, 0};
        double* w = &t.w3[gp * 3];
        if (et == OGS_ELEM_QUAD4)
        {
            const int gr = gp / ngauss, gs = gp % ngauss;
            u[0] = gauss_point(ngauss, gr);
            u[1] = gauss_point(ngauss, gs);
            w[0] = gauss_weight(ngauss, gr);
            w[1] = gauss_weight(ngauss, gs);
        }
        else if (et == OGS_ELEM_HEX8)
        {
            const int gr = gp / (ngauss * ngauss);
            int gs = gp % (ngauss * ngauss);
            const int gt = gs % ngauss;
            gs /= ngauss;
            u[0] = gauss_point(ngauss, gr);
            u[1] = gauss_point(ngauss, gs);
            u[2] = gauss_point(ngauss, gt);
            w[0] = gauss_weight(ngauss, gr);
            w[1] = gauss_weight(ngauss, gs);
            w[2] = gauss_weight(ngauss, gt);
        }
        else
        {
            tet5_point(gp, u);
            w[0] = u[3];
        }
        t.wprod[gp] = w[0] * w[1] * w[2];
        shape_eval(et, u, &t.N[gp * t.nn], &t.dN[gp * t.nn * t.dim]);
    }
    return t;
}

AffineTable make_affine_table(int et, int ngauss)
{
    const ShapeTable t = make_shape_table(et, ngauss);
    AffineTable a;
    const int nn = t.nn, dim = t.dim;
    a.Q.assign(dim * dim * nn * nn, 0.0);
    a.M0.assign(nn * nn, 0.0);
    for (int gp = 0; gp < t.ngp; gp++)
    {
        const double w = t.wprod[gp];
        const double* dN = &t.dN[gp * nn * dim];
        const double* N = &t.N[gp * nn];
        for (int ia = 0; ia < dim; ia++)
            for (int ib = 0; ib < dim; ib++)
                for (int i = 0; i < nn; i++)
                    for (int j = 0; j < nn; j++)
                        a.Q[((ia * dim + ib) * nn + i) * nn + j] +=
                            w * dN[ia * nn + i] * dN[ib * nn + j];
        for (int i = 0; i < nn; i++)
            for (int j = 0; j < nn; j++) a.M0[i * nn + j] += w * N[i] * N[j];
    }
    a.dNc.assign(dim * nn, 0.0);
    double uc[3] = {0, 0, 0}, Nc[8];
    if (et == OGS_ELEM_TET4) uc[0] = uc[1] = uc[2] = 0.25;
    shape_eval(et, uc, Nc, a.dNc.data());
    return a;
}

// ---------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------
template <class F>
static void parallel_for(int64_t n, F f)
{
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 65536) nt = 1;
    std::vector<std::thread> th;
    const int64_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++)
    {
        const int64_t lo = t * chunk, hi = std::min<int64_t>(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([=]() { f(lo, hi); });
    }
    for (auto& x : th) x.join();
}

// Coefficients of the non-affine terms of the isoparametric map; an element
// is affine when they vanish (relative to the linear terms).
static bool element_affine(int et, const double* X, const double* Y,
                           const double* Z)
{
    if (et == OGS_ELEM_TET4) return true;
    const double* cs[3] = {X, Y, Z};
    if (et == OGS_ELEM_QUAD4)
    {
        for (int c = 0; c < 2; c++)
        {
            double lin = 0.0, bil = 0.0;
            for (int i = 0; i < 4; i++)
            {
                lin += std::fabs(cs[c][i]);
                bil += cs[c][i] * kQuadNode[i][0] * kQuadNode[i][1];
            }
            if (std::fabs(bil) > 1e-14 * lin) return false;
        }
        return true;
    }
    for (int c = 0; c < 3; c++)
    {
        double lin = 0.0, t4 = 0, t5 = 0, t6 = 0, t7 = 0;
        for (int i = 0; i < 8; i++)
        {
            const double a = kHexNode[i][0], b = kHexNode[i][1], d = kHexNode[i][2];
            const double v = cs[c][i];
            lin += std::fabs(v);
            t4 += v * a * b;
            t5 += v * b * d;
            t6 += v * a * d;
            t7 += v * a * b * d;
        }
        const double tol = 1e-14 * lin;
        if (std::fabs(t4) > tol || std::fabs(t5) > tol || std::fabs(t6) > tol ||
            std::fabs(t7) > tol)
            return false;
    }
    return true;
}

template <class T>
static ogs_status upload(T** dst, const T* src, size_t n)
{
    OGS_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(1, n) * sizeof(T)));
    if (n) OGS_CUDA_TRY(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return OGS_OK;
}

}  // namespace ogs

using namespace ogs;

extern "C" const char* ogs_gpu_last_error(void) { return ogs::last_error(); }
extern "C" const char* ogs_gpu_version(void) { return "ogs5_gb300 0.1 (sm_103a)"; }
extern "C" int64_t ogs_gpu_kernel_launches(int32_t reset) { return ogs::launches(reset); }

// Dependency levels of a triangular sweep over the CSR pattern (natural row
// order): a row's level is one more than the deepest row it reads -- the
// columns below the diagonal for the forward sweep, above it for the
// backward sweep.  Rows are returned grouped by level, ascending inside a
// level; ptr holds the level boundaries.
// Is the pattern that of a lattice numbered line by line (nx nodes per
// line, nxy = nx ny per plane), every entry joining nodes at most one step
// apart on each axis, with the columns left of the diagonal at no larger
// x, y and z than the row?  Row 0's columns give the candidate: 0, 1, nx
// (nx + 1), then nxy; every entry is then checked.
static bool lattice_monotone(int64_t N, const std::vector<int32_t>& row_ptr, const std::vector<int32_t>& col,
                             int& nx, int& ny, int& nz)
{
    if (N < 8) return false;
    const int32_t* c0 = col.data() + row_ptr[0];
    const int64_t n0 = row_ptr[1] - row_ptr[0];
    if (n0 < 4 || c0[0] != 0 || c0[1] != 1) return false;
    const int64_t cx = c0[2];
    int64_t cxy = -1;
    for (int64_t k = 0; k < n0; k++)
        if (c0[k] != 0 && c0[k] != 1 && c0[k] != cx && c0[k] != cx + 1)
        {
            cxy = c0[k];
            break;
        }
    if (cx < 3 || cxy < 3 * cx || cxy % cx != 0 || N % cxy != 0 || N / cxy < 2) return false;
    const int64_t x_n = cx, y_n = cxy / cx, z_n = N / cxy;
    std::atomic<bool> ok(true);
    parallel_for(N, [&](int64_t lo, int64_t hi) {
        for (int64_t r = lo; r < hi && ok.load(std::memory_order_relaxed); r++)
        {
            const int64_t rx = r % x_n, ry = (r / x_n) % y_n, rz = r / cxy;
            for (int64_t k = row_ptr[r]; k < row_ptr[r + 1]; k++)
            {
                const int64_t j = col[k];
                const int64_t dx = j % x_n - rx, dy = (j / x_n) % y_n - ry, dz = j / cxy - rz;
                const bool near = dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1;
                const bool mono = j < r ? dx <= 0 && dy <= 0 && dz <= 0 : dx >= 0 && dy >= 0 && dz >= 0;
                if (!near || !mono)
                {
                    ok = false;
                    break;
                }
            }
        }
    });
    if (!ok) return false;
    nx = (int)x_n;
    ny = (int)y_n;
    nz = (int)z_n;
    return true;
}

static void sweep_levels(int64_t N, const std::vector<int32_t>& row_ptr, const std::vector<int32_t>& col,
                         bool forward, std::vector<int32_t>& rows, std::vector<int32_t>& ptr)
{
    std::vector<int32_t> lev(N, 0);
    int32_t nl = N ? 1 : 0;
    for (int64_t q = 0; q < N; q++)
    {
        const int64_t r = forward ? q : N - 1 - q;
        int32_t l = 0;
        for (int32_t k = row_ptr[r]; k < row_ptr[r + 1]; k++)
        {
            const int32_t c = col[k];
            if (forward ? c < r : c > r) l = std::max(l, lev[c] + 1);
        }
        lev[r] = l;
        nl = std::max(nl, l + 1);
    }
    // rows by level, every level padded with -1 to a whole number of warps
    // (32 positions): a warp of the sweep kernels then holds rows of one
    // level only, which never wait on each other
    ptr.assign((size_t)nl + 1, 0);
    for (int64_t r = 0; r < N; r++) ptr[lev[r] + 1]++;
    for (int32_t l = 0; l < nl; l++) ptr[l + 1] = ptr[l] + ((ptr[l + 1] + 31) & ~31);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    rows.assign((size_t)ptr[nl], -1);
    for (int64_t r = 0; r < N; r++) rows[fill[lev[r]]++] = (int32_t)r;
}

extern "C" ogs_status ogs_gpu_mesh_destroy(ogs_mesh* m)
{
    if (!m) return OGS_OK;
    cudaFree(m->x);
    cudaFree(m->y);
    cudaFree(m->z);
    cudaFree(m->conn_t);
    cudaFree(m->row_ptr);
    cudaFree(m->col);
    cudaFree(m->diag_pos);
    cudaFree(m->slot_t);
    cudaFree(m->tab);
    cudaFree(m->aff);
    cudaFree(m->csr2sell);
    cudaFree(m->slice_ptr);
    cudaFree(m->sell_col);
    cudaFree(m->row_len);
    cudaFree(m->up_off);
    cudaFree(m->slot_up);
    cudaFree(m->csr_diag);
    cudaFree(m->lvl_rows);
    cudaFree(m->lvl_ptr);
    cudaFree(m->ulvl_rows);
    cudaFree(m->ulvl_ptr);
    cudaFree(m->tile_order);
    delete m;
    return OGS_OK;
}

// Is the hex mesh a regular lattice in lexicographic node order (x fastest)
// with uniform spacing and cells in lexicographic order with the OGS corner
// order (bottom face counter-clockwise, then the top face)?
static void detect_grid(const ogs_mesh_desc* d, ogs_mesh* m)
{
    m->grid = false;
    if (d->elem_type != OGS_ELEM_HEX8) return;
    const int64_t N = d->n_nodes, E = d->n_elements;
    const double *x = d->x, *y = d->y, *z = d->z;
    int64_t nx = 1;
    while (nx < N && x[nx] != x[0]) nx++;
    if (nx < 2 || N % nx) return;
    int64_t ny = 1;
    while (ny * nx < N && y[ny * nx] != y[0]) ny++;
    if (ny < 2 || N % (nx * ny)) return;
    const int64_t nz = N / (nx * ny);
    if (nz < 2 || E != (nx - 1) * (ny - 1) * (nz - 1)) return;
    const double hx = x[1] - x[0], hy = y[nx] - y[0], hz = z[nx * ny] - z[0];
    if (!(hx > 0.0 && hy > 0.0 && hz > 0.0)) return;
    std::atomic<bool> ok{true};
    parallel_for(N, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi && ok.load(std::memory_order_relaxed); i++)
        {
            const int64_t ix = i % nx, t = i / nx, iy = t % ny, iz = t / ny;
            if (std::fabs(x[i] - (x[0] + ix * hx)) > 1e-9 * hx || std::fabs(y[i] - (y[0] + iy * hy)) > 1e-9 * hy ||
                std::fabs(z[i] - (z[0] + iz * hz)) > 1e-9 * hz)
                ok = false;
        }
    });
    if (!ok) return;
    const int32_t* conn = d->connectivity;
    parallel_for(E, [&](int64_t lo, int64_t hi) {
        for (int64_t e = lo; e < hi && ok.load(std::memory_order_relaxed); e++)
        {
            const int64_t cx = e % (nx - 1), t = e / (nx - 1), cy = t % (ny - 1), cz = t / (ny - 1);
            const int64_t n0 = cx + nx * (cy + ny * cz);
            const int64_t want[8] = {n0, n0 + 1, n0 + 1 + nx, n0 + nx, n0 + nx * ny, n0 + 1 + nx * ny,
                                     n0 + 1 + nx + nx * ny, n0 + nx + nx * ny};
            for (int k = 0; k < 8; k++)
                if (conn[e * 8 + k] != want[k]) ok = false;
        }
    });
    if (!ok) return;
    m->grid = true;
    m->gx = (int)nx; m->gy = (int)ny; m->gz = (int)nz;
    m->ghx = hx; m->ghy = hy; m->ghz = hz;
}

extern "C" ogs_status ogs_gpu_mesh_create(const ogs_mesh_desc* d, ogs_mesh** out)
{
    if (!d || !out) { set_error("mesh_create: NULL argument"); return OGS_BAD_ARG; }
    *out = nullptr;
    if (d->elem_type < 0 || d->elem_type > 2) { set_error("mesh_create: bad elem_type %d", d->elem_type); return OGS_BAD_ARG; }
    const int et = d->elem_type;
    const int nn = nodes_per_element(et);
    const int dim = elem_dim(et);
    if (d->dim != dim) { set_error("mesh_create: dim %d does not match element type", d->dim); return OGS_BAD_ARG; }
    if (d->n_nodes <= 0 || d->n_elements <= 0 || !d->x || !d->y || !d->connectivity || (dim == 3 && !d->z))
    {
        set_error("mesh_create: empty mesh or missing arrays");
        return OGS_BAD_ARG;
    }
    if (d->n_nodes >= (int64_t(1) << 31) || d->n_elements >= (int64_t(1) << 31))
    {
        set_error("mesh_create: more than 2^31 nodes or elements");
        return OGS_BAD_ARG;
    }
    int ng = d->gauss_points;
    if (et != OGS_ELEM_TET4 && (ng < 1 || ng > 3)) { set_error("mesh_create: gauss_points must be 1..3"); return OGS_BAD_ARG; }
    if (et == OGS_ELEM_TET4) ng = 3;
    const int64_t N = d->n_nodes, E = d->n_elements;
    const int32_t* conn = d->connectivity;
    for (int64_t k = 0; k < E * nn; k++)
        if (conn[k] < 0 || conn[k] >= N) { set_error("mesh_create: connectivity entry %lld out of range", (long long)k); return OGS_BAD_ARG; }

    ogs_mesh* m = new ogs_mesh;
    m->elem_type = et; m->dim = dim; m->nn = nn; m->ngauss = ng;
    m->ngp = num_gauss_points(et, ng);
    m->n_nodes = N; m->n_elem = E;
    cudaGetDevice(&m->device);
    detect_grid(d, m);

    // node -> element incidence
    std::vector<int64_t> ne_ptr(N + 1, 0);
    for (int64_t k = 0; k < E * nn; k++) ne_ptr[conn[k] + 1]++;
    for (int64_t i = 0; i < N; i++) ne_ptr[i + 1] += ne_ptr[i];
    std::vector<int32_t> ne_idx(E * nn);
    {
        std::vector<int64_t> fill(ne_ptr.begin(), ne_ptr.end() - 1);
        for (int64_t e = 0; e < E; e++)
            for (int i = 0; i < nn; i++) ne_idx[fill[conn[e * nn + i]]++] = (int32_t)e;
    }
    // rows: sorted unique neighbours (ConnectedNodes + SparseTable CRS)
    std::vector<int32_t> deg(N, 0);
    parallel_for(N, [&](int64_t lo, int64_t hi) {
        std::vector<int32_t> buf;
        for (int64_t r = lo; r < hi; r++)
        {
            buf.clear();
            for (int64_t q = ne_ptr[r]; q < ne_ptr[r + 1]; q++)
                for (int j = 0; j < nn; j++) buf.push_back(conn[(int64_t)ne_idx[q] * nn + j]);
            std::sort(buf.begin(), buf.end());
            deg[r] = (int32_t)(std::unique(buf.begin(), buf.end()) - buf.begin());
        }
    });
    std::vector<int32_t> row_ptr(N + 1, 0);
    int64_t nnz = 0;
    for (int64_t r = 0; r < N; r++) { row_ptr[r] = (int32_t)nnz; nnz += deg[r]; if (nnz >= (int64_t(1) << 31)) break; }
    if (nnz >= (int64_t(1) << 31)) { delete m; set_error("mesh_create: nnz exceeds 2^31"); return OGS_BAD_ARG; }
    row_ptr[N] = (int32_t)nnz;
    m->nnz = nnz;
    std::vector<int32_t> col(nnz), diag(N, -1);
    parallel_for(N, [&](int64_t lo, int64_t hi) {
        std::vector<int32_t> buf;
        for (int64_t r = lo; r < hi; r++)
        {
            buf.clear();
            for (int64_t q = ne_ptr[r]; q < ne_ptr[r + 1]; q++)
                for (int j = 0; j < nn; j++) buf.push_back(conn[(int64_t)ne_idx[q] * nn + j]);
            std::sort(buf.begin(), buf.end());
            const int64_t u = std::unique(buf.begin(), buf.end()) - buf.begin();
            for (int64_t k = 0; k < u; k++)
            {
                col[row_ptr[r] + k] = buf[k];
                if (buf[k] == r) diag[r] = (int32_t)(row_ptr[r] + k);
            }
        }
    });
    // ILU(0) sweep orders (CSR diagonal positions before they become SELL slots)
    std::vector<int32_t> csr_diag(diag), lvl_rows, lvl_ptr, ulvl_rows, ulvl_ptr;
    sweep_levels(N, row_ptr, col, true, lvl_rows, lvl_ptr);
    sweep_levels(N, row_ptr, col, false, ulvl_rows, ulvl_ptr);
    m->n_lvl = (int)lvl_ptr.size() - 1;
    m->n_ulvl = (int)ulvl_ptr.size() - 1;
    m->n_lpos = lvl_ptr.back();
    m->n_upos = ulvl_ptr.back();
    for (int64_t r = 0; r < N; r++)
        if (diag[r] >= 0)
        {
            m->ilu_kl = std::max(m->ilu_kl, diag[r] - row_ptr[r]);
            m->ilu_ku = std::max(m->ilu_ku, row_ptr[r + 1] - diag[r] - 1);
        }
    // ILU(0) tiles, ordered by the sum of their coordinates (the forward
    // sweep's dependency order between tiles; the backward sweep walks the
    // list from its end)
    std::vector<int32_t> tile_order;
    if (N < (int64_t(1) << 30) &&
        lattice_monotone(N, row_ptr, col, m->lnx, m->lny, m->lnz))
    {
        m->tnx = (m->lnx + kIluTile - 1) / kIluTile;
        m->tny = (m->lny + kIluTile - 1) / kIluTile;
        m->tnz = (m->lnz + kIluTile - 1) / kIluTile;
        const int64_t nt = (int64_t)m->tnx * m->tny * m->tnz;
        if (nt * kIluTile * kIluTile * kIluTile < (int64_t(1) << 31))
        {
            m->tiles = (int)nt;
            for (int l = 0; l <= m->tnx + m->tny + m->tnz - 3; l++)
                for (int c = 0; c < m->tnz; c++)
                    for (int b = 0; b < m->tny; b++)
                    {
                        const int a = l - b - c;
                        if (a >= 0 && a < m->tnx) tile_order.push_back(a + m->tnx * (b + m->tny * c));
                    }
        }
    }
    // SELL-32 layout of the pattern
    const int n_slices = (int)((N + kSlice - 1) / kSlice);
    std::vector<int32_t> slice_ptr(n_slices + 1, 0);
    int64_t sell_nnz = 0;
    for (int s = 0; s < n_slices; s++)
    {
        int w = 0;
        for (int64_t r = (int64_t)s * kSlice; r < std::min<int64_t>(N, (int64_t)(s + 1) * kSlice); r++)
            w = std::max(w, deg[r]);
        slice_ptr[s] = (int32_t)sell_nnz;
        sell_nnz += (int64_t)w * kSlice;
        if (sell_nnz >= (int64_t(1) << 31)) { delete m; set_error("mesh_create: padded nnz exceeds 2^31"); return OGS_BAD_ARG; }
    }
    slice_ptr[n_slices] = (int32_t)sell_nnz;
    m->sell_nnz = sell_nnz;
    m->n_slices = n_slices;
    std::vector<int32_t> csr2sell(nnz), sell_col(sell_nnz);
    parallel_for(N, [&](int64_t lo, int64_t hi) {
        for (int64_t r = lo; r < hi; r++)
        {
            const int64_t s = r / kSlice, l = r % kSlice;
            const int w = (slice_ptr[s + 1] - slice_ptr[s]) / kSlice;
            for (int j = 0; j < w; j++)
            {
                const int64_t slot = slice_ptr[s] + (int64_t)j * kSlice + l;
                if (j < deg[r])
                {
                    csr2sell[row_ptr[r] + j] = (int32_t)slot;
                    sell_col[slot] = col[row_ptr[r] + j];
                }
                else
                    sell_col[slot] = (int32_t)r;  // padding: own column, value 0
            }
            if (diag[r] >= 0) diag[r] = csr2sell[diag[r]];
        }
    });
    // pad rows of the last, partial slice
    for (int64_t r = N; r < (int64_t)n_slices * kSlice; r++)
    {
        const int64_t s = r / kSlice, l = r % kSlice;
        const int w = (slice_ptr[s + 1] - slice_ptr[s]) / kSlice;
        for (int j = 0; j < w; j++) sell_col[slice_ptr[s] + (int64_t)j * kSlice + l] = 0;
    }
    // distinct column offsets: a structured grid has a handful (27 for
    // hexes, 15 for Kuhn tets, 9 for quads)
    std::vector<int32_t> up_off;
    std::vector<int8_t> slot_up;
    {
        std::vector<int32_t> offs;
        bool few = true;
        for (int64_t r = 0; r < N && few; r++)
            for (int64_t k = row_ptr[r]; k < row_ptr[r + 1]; k++)
            {
                const int32_t o = col[k] - (int32_t)r;
                auto it = std::lower_bound(offs.begin(), offs.end(), o);
                if (it == offs.end() || *it != o)
                {
                    offs.insert(it, o);
                    if (offs.size() > 64) { few = false; break; }
                }
            }
        if (few)
        {
            for (int32_t o : offs)
                if (o >= 0) up_off.push_back(o);
            std::sort(up_off.begin(), up_off.end());
            m->n_off = (int)offs.size();
            m->n_up = (int)up_off.size();
            m->host_up_off = up_off;
            slot_up.assign(sell_nnz, (int8_t)-1);
            parallel_for(N, [&](int64_t lo, int64_t hi) {
                for (int64_t r = lo; r < hi; r++)
                    for (int64_t k = row_ptr[r]; k < row_ptr[r + 1]; k++)
                    {
                        const int32_t o = col[k] - (int32_t)r;
                        if (o < 0) continue;
                        const int d = (int)(std::lower_bound(up_off.begin(), up_off.end(), o) - up_off.begin());
                        slot_up[csr2sell[k]] = (int8_t)d;
                    }
            });
        }
    }
    // slot map (SELL slots), transposed [i*nn+j][e] for coalesced loads
    std::vector<int32_t> slot_t((size_t)nn * nn * E);
    std::vector<int32_t> conn_t((size_t)nn * E);
    std::vector<char> aff(E, 1);
    const double* X = d->x;
    const double* Y = d->y;
    const double* Z = d->z;
    parallel_for(E, [&](int64_t lo, int64_t hi) {
        for (int64_t e = lo; e < hi; e++)
        {
            const int32_t* en = conn + e * nn;
            for (int i = 0; i < nn; i++)
            {
                conn_t[(size_t)i * E + e] = en[i];
                const int32_t r = en[i];
                const int32_t* cb = col.data() + row_ptr[r];
                const int32_t* ce = col.data() + row_ptr[r + 1];
                for (int j = 0; j < nn; j++)
                {
                    const int32_t* p = std::lower_bound(cb, ce, en[j]);
                    slot_t[(size_t)(i * nn + j) * E + e] = csr2sell[p - col.data()];
                }
            }
            double ex[8], ey[8], ez[8];
            for (int i = 0; i < nn; i++)
            {
                ex[i] = X[en[i]];
                ey[i] = Y[en[i]];
                ez[i] = Z ? Z[en[i]] : 0.0;
            }
            aff[e] = element_affine(et, ex, ey, ez) ? 1 : 0;
        }
    });
    m->affine = std::all_of(aff.begin(), aff.end(), [](char c) { return c != 0; });

    // tables
    m->host_tab = make_shape_table(et, ng);
    std::vector<double> tab;
    tab.insert(tab.end(), m->host_tab.N.begin(), m->host_tab.N.end());
    tab.insert(tab.end(), m->host_tab.dN.begin(), m->host_tab.dN.end());
    tab.insert(tab.end(), m->host_tab.w3.begin(), m->host_tab.w3.end());
    const AffineTable at = make_affine_table(et, ng);
    std::vector<double> affb;
    affb.insert(affb.end(), at.Q.begin(), at.Q.end());
    affb.insert(affb.end(), at.M0.begin(), at.M0.end());
    affb.insert(affb.end(), at.dNc.begin(), at.dNc.end());

    std::vector<double> zz;
    if (!Z) zz.assign(N, 0.0);
    ogs_status st;
    if ((st = upload(&m->x, X, N)) || (st = upload(&m->y, Y, N)) ||
        (st = upload(&m->z, Z ? Z : zz.data(), N)) ||
        (st = upload(&m->conn_t, conn_t.data(), conn_t.size())) ||
        (st = upload(&m->row_ptr, row_ptr.data(), row_ptr.size())) ||
        (st = upload(&m->col, col.data(), col.size())) ||
        (st = upload(&m->diag_pos, diag.data(), diag.size())) ||
        (st = upload(&m->csr2sell, csr2sell.data(), csr2sell.size())) ||
        (st = upload(&m->slice_ptr, slice_ptr.data(), slice_ptr.size())) ||
        (st = upload(&m->sell_col, sell_col.data(), sell_col.size())) ||
        (st = upload(&m->row_len, deg.data(), deg.size())) ||
        (m->n_up && (st = upload(&m->up_off, up_off.data(), up_off.size()))) ||
        (m->n_up && (st = upload(&m->slot_up, slot_up.data(), slot_up.size()))) ||
        (st = upload(&m->slot_t, slot_t.data(), slot_t.size())) ||
        (st = upload(&m->csr_diag, csr_diag.data(), csr_diag.size())) ||
        (st = upload(&m->lvl_rows, lvl_rows.data(), lvl_rows.size())) ||
        (st = upload(&m->lvl_ptr, lvl_ptr.data(), lvl_ptr.size())) ||
        (st = upload(&m->ulvl_rows, ulvl_rows.data(), ulvl_rows.size())) ||
        (st = upload(&m->ulvl_ptr, ulvl_ptr.data(), ulvl_ptr.size())) ||
        (m->tiles && (st = upload(&m->tile_order, tile_order.data(), tile_order.size()))) ||
        (st = upload(&m->tab, tab.data(), tab.size())) ||
        (st = upload(&m->aff, affb.data(), affb.size())))
    {
        ogs_gpu_mesh_destroy(m);
        return st;
    }
    *out = m;
    return OGS_OK;
}

extern "C" ogs_status ogs_gpu_mesh_info(const ogs_mesh* m, int64_t* n_rows, int64_t* nnz)
{
    if (!m) { set_error("mesh_info: NULL mesh"); return OGS_BAD_ARG; }
    if (n_rows) *n_rows = m->n_nodes;
    if (nnz) *nnz = m->nnz;
    return OGS_OK;
}

extern "C" int32_t ogs_gpu_mesh_gauss_points(const ogs_mesh* m) { return m ? m->ngp : 0; }

extern "C" int32_t ogs_gpu_mesh_ilu_tiles(const ogs_mesh* m) { return m ? m->tiles : 0; }
