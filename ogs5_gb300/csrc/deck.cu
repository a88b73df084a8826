// deck.cu -- reader of OGS-5 input decks (host code): the mesh file (.msh),
// the geometry file (.gli) and constant Dirichlet conditions (.bc), turned
// into an ogs_mesh_desc and the (row, value) list of ogs_gpu_set_dirichlet.
//
//   .msh  CFEMesh::Read (MSH/msh_mesh.cpp:421-495) with CElem::Read for the
//         msh file type (MSH/msh_elem.cpp:578-736): "$NODES n" then
//         "index x y z [$AREA a]" lines, "$ELEMENTS n" then
//         "index patch [-1] type node..." lines; element nodes are positions
//         in the node list.  The first mesh of the file, one element type:
//         line, tri, quad, tet or hex (quad, hex and tet are assembled on
//         the GPU; line and tri decks still give node sets).
//   .gli  readPoints / readPolyline / readSurface (FileIO/OGSIOVer4.cpp:54-
//         503): "#POINTS" lines "id x y z [$MD d] [$NAME name]", a point's
//         position in the file being its index; polylines list indices,
//         one-based when the first written id is not 0; a $NAME maps to the
//         written id used as an index, as the reference's name map does;
//         "#POLYLINE" with $NAME,
//         $EPSILON (CGLPolyline::epsilon, default 0.01, GEO/geo_ply.cpp:33,
//         604-611) and $POINTS (repeated consecutive points dropped);
//         "#SURFACE" with $NAME and $POLYLINES, of which the last one listed
//         is the surface's boundary, closed if it is open.
//   .bc   #BOUNDARY_CONDITION blocks (CBoundaryCondition::Read,
//         FEM/rf_bc_new.cpp:250-560): $PCS_TYPE, $PRIMARY_VARIABLE (or
//         $COMP_NAME), $GEO_TYPE (POINT | POLYLINE | SURFACE name),
//         $DIS_TYPE CONSTANT v, $EPSILON e; each value on the next non-blank
//         line.
//
// Node sets, as CBoundaryConditionsGroup::Set builds them for CONSTANT
// conditions (FEM/rf_bc_new.cpp:1272-1560), without PETSc:
//   point     the nearest mesh node (CFEMesh::GetNODOnPNT through the mesh
//             grid, MSH/msh_mesh.cpp:1473-1476);
//   polyline  MeshNodesAlongPolyline with the polyline's epsilon as search
//             radius (the BC sets the mesh's minimum edge length to it before
//             CFEMesh::GetNODOnPLY, msh_mesh.cpp:1562-1605): per segment, a
//             node whose distance to the segment's line is at most the radius
//             and whose projection parameter lies within radius/length of
//             [0, 1] (MSH/MeshNodesAlongPolyline.cpp:30-75,
//             MathLib/MathTools.cpp:24-42); the BC sorts the nodes by index;
//   surface   the polygon is ear-clipped into triangles (Surface::
//             createSurface, GEO/Surface.cpp:64-94) and a node belongs to the
//             surface when it is within the search length of the bounding
//             box (AABB::containsPoint, GEO/AxisAlignedBoundingBox.cpp:73-90)
//             and in one triangle by MathLib::isPointInTriangle
//             (MathLib/AnalyticalGeometry.cpp:180-221) among the triangles
//             of the surface grid's cell that holds the node -- a node
//             outside the grid (the bounding box grown by 1e-6 relative at
//             its upper corner) belongs to no triangle (GEOLIB::SurfaceGrid,
//             GEO/SurfaceGrid.cpp:29-240, 367-395); the search length is
//             the BC's $EPSILON or 0.375 * h_min / 2 (msh_mesh.cpp:944-946,
//             1917-1928), h_min the mesh's minimum edge length.
// Deliberate difference: the merging of coordinate-equal geometry points is
// not restated; decks with repeated point coordinates can differ.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"

namespace {

struct Polyline
{
    std::vector<size_t> pts;  // positions in the point list
    double eps = 0.01;
};

struct Surface
{
    std::string ply;  // the boundary polyline
};

struct Bc
{
    std::string pcs, var, geo_type, geo_name;
    double value = 0.0;
    double eps = -1.0;
};

std::string trim(const std::string& s)
{
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

// element types CElem reads (MSH/MSHEnums.cpp:33-50): node count, edges
// (MSH/msh_elem.cpp:984-1052) and the GPU path's element type, -1 if the
// type is read (for its nodes and edges) but not assembled on the GPU
struct ElemKind
{
    const char* name;
    int nodes, n_edges, gpu_type;
    int edges[12][2];
};
const ElemKind kElemKinds[] = {
    {"line", 2, 1, -1, {{0, 1}}},
    {"tri", 3, 3, -1, {{0, 1}, {1, 2}, {2, 0}}},
    {"quad", 4, 4, OGS_ELEM_QUAD4, {{0, 1}, {1, 2}, {2, 3}, {3, 0}}},
    {"tet", 4, 6, OGS_ELEM_TET4, {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}}},
    {"hex", 8, 12, OGS_ELEM_HEX8,
     {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}}},
};

const ElemKind* elem_kind(const std::string& t)
{
    for (const ElemKind& k : kElemKinds)
        if (t == k.name) return &k;
    return nullptr;
}

double dist3(const double* a, const double* b)
{
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

}  // namespace

struct ogs_deck
{
    const ElemKind* kind = nullptr;
    int elem_type = -1, dim = 3;
    std::vector<double> x, y, z;
    std::vector<int32_t> conn;
    std::vector<double> px, py, pz;  // geometry points, in file order
    std::map<std::string, long> point_names;  // $NAME -> written id
    std::map<std::string, Polyline> polylines;
    std::map<std::string, Surface> surfaces;
    std::vector<Bc> bcs;
    double min_edge = 0.0;
};

namespace {

using ogs::set_error;

ogs_status read_msh(ogs_deck* d, const char* path)
{
    std::ifstream in(path);
    if (!in) { set_error("deck: cannot open %s", path); return OGS_BAD_ARG; }
    std::string line;
    int meshes = 0;
    while (std::getline(in, line))
    {
        if (line.find("#STOP") != std::string::npos) break;
        if (line.find("#FEM_MSH") != std::string::npos && ++meshes > 1) break;
        if (line.find("$NODES") != std::string::npos)
        {
            size_t n = 0;
            if (!(in >> n)) { set_error("deck: %s: bad $NODES count", path); return OGS_BAD_ARG; }
            std::getline(in, line);
            d->x.resize(n);
            d->y.resize(n);
            d->z.resize(n);
            for (size_t i = 0; i < n; i++)
            {
                long idx;
                if (!std::getline(in, line)) { set_error("deck: %s: %zu of %zu nodes", path, i, n); return OGS_BAD_ARG; }
                std::istringstream ls(line);
                if (!(ls >> idx >> d->x[i] >> d->y[i] >> d->z[i]))
                {
                    set_error("deck: %s: bad node line '%s'", path, trim(line).c_str());
                    return OGS_BAD_ARG;
                }
            }
        }
        else if (line.find("$ELEMENTS") != std::string::npos)
        {
            size_t n = 0;
            if (!(in >> n)) { set_error("deck: %s: bad $ELEMENTS count", path); return OGS_BAD_ARG; }
            std::getline(in, line);
            for (size_t e = 0; e < n; e++)
            {
                if (!std::getline(in, line)) { set_error("deck: %s: %zu of %zu elements", path, e, n); return OGS_BAD_ARG; }
                std::istringstream ls(line);
                long idx, patch;
                std::string buf, name;
                ls >> idx >> patch >> buf;
                if (buf.find("-1") != std::string::npos) ls >> name;  // grid adaptation flag
                else name = buf;
                const ElemKind* kind = elem_kind(name);
                if (!kind || !ls)
                {
                    set_error("deck: %s: element line '%s': type not read (line, tri, quad, tet, hex)", path,
                              trim(line).c_str());
                    return OGS_BAD_ARG;
                }
                if (!d->kind) d->kind = kind;
                else if (d->kind != kind)
                {
                    set_error("deck: %s: mixed element types (%s, %s)", path, d->kind->name, name.c_str());
                    return OGS_BAD_ARG;
                }
                const int nn = kind->nodes;
                for (int k = 0; k < nn; k++)
                {
                    long v;
                    if (!(ls >> v) || v < 0 || v >= (long)d->x.size())
                    {
                        set_error("deck: %s: element %ld: bad node index", path, idx);
                        return OGS_BAD_ARG;
                    }
                    d->conn.push_back((int32_t)v);
                }
            }
        }
    }
    if (d->x.empty() || d->conn.empty()) { set_error("deck: %s: no $NODES or $ELEMENTS", path); return OGS_BAD_ARG; }
    d->elem_type = d->kind->gpu_type;
    d->dim = 3;
    if (d->elem_type == OGS_ELEM_QUAD4)
    {
        for (double zz : d->z)
            if (zz != d->z[0])
            {
                set_error("deck: %s: quad meshes must lie in a z = const plane", path);
                return OGS_BAD_ARG;
            }
        d->dim = 2;
    }
    // minimum edge length over the element edges (CFEMesh::computeMinEdgeLength,
    // msh_mesh.cpp:331-344)
    const int nn = d->kind->nodes;
    double h = INFINITY;
    for (size_t el = 0; el < d->conn.size() / nn; el++)
        for (int k = 0; k < d->kind->n_edges; k++)
        {
            const int a = d->conn[el * nn + d->kind->edges[k][0]], b = d->conn[el * nn + d->kind->edges[k][1]];
            const double pa[3] = {d->x[a], d->y[a], d->z[a]}, pb[3] = {d->x[b], d->y[b], d->z[b]};
            h = std::min(h, dist3(pa, pb));
        }
    d->min_edge = h;
    return OGS_OK;
}

// next token of the stream ("" at the end)
std::string token(std::istream& in)
{
    std::string t;
    if (!(in >> t)) t.clear();
    return t;
}

ogs_status read_gli(ogs_deck* d, const char* path)
{
    std::ifstream in(path);
    if (!in) { set_error("deck: cannot open %s", path); return OGS_BAD_ARG; }
    std::string line, kw;
    bool zero_based = true;
    // #POINTS: line based, up to the next '#' keyword
    while (std::getline(in, line))
    {
        if (line.find("#POINTS") != std::string::npos)
        {
            while (std::getline(in, line))
            {
                if (line.find('#') != std::string::npos) break;
                std::istringstream ls(line);
                long id;
                double x, y, z;
                if (!(ls >> id >> x >> y >> z)) continue;
                if (d->px.empty()) zero_based = id == 0;
                d->px.push_back(x);
                d->py.push_back(y);
                d->pz.push_back(z);
                const size_t pos = line.find("$NAME");
                if (pos != std::string::npos)
                {
                    std::istringstream ns(line.substr(pos + 5));
                    std::string name;
                    if (ns >> name) d->point_names[name] = id;
                }
            }
        }
        if (line.find('#') != std::string::npos)
        {
            kw = trim(line);
            break;
        }
    }
    // #POLYLINE / #SURFACE blocks: token based, each up to the next '#'
    while (!kw.empty() && kw.find("#STOP") == std::string::npos)
    {
        const bool ply = kw.find("#POLYLINE") != std::string::npos;
        const bool sfc = kw.find("#SURFACE") != std::string::npos;
        std::string name, t = token(in);
        Polyline P;
        Surface S;
        while (!t.empty() && t.find('#') == std::string::npos)
        {
            if (t == "$NAME") name = token(in), t = token(in);
            else if (t == "$EPSILON") P.eps = std::strtod(token(in).c_str(), nullptr), t = token(in);
            else if (t == "$ID" || t == "$TYPE" || t == "$MAT_GROUP") token(in), t = token(in);
            else if (t == "$TIN" || t == "$POINT_VECTOR")
            {
                set_error("deck: %s: %s geometries are not supported", path, t.c_str());
                return OGS_BAD_ARG;
            }
            else if (t == "$POINTS" || t == "$POLYLINES")
            {
                const bool pts = t == "$POINTS";
                for (t = token(in); !t.empty() && t.find('#') == std::string::npos && t.find('$') == std::string::npos;
                     t = token(in))
                {
                    if (pts)
                    {
                        const long id = std::strtol(t.c_str(), nullptr, 10) - (zero_based ? 0 : 1);
                        if (id < 0 || id >= (long)d->px.size())
                        {
                            set_error("deck: %s: polyline %s: unknown point %s", path, name.c_str(), t.c_str());
                            return OGS_BAD_ARG;
                        }
                        if (P.pts.empty() || P.pts.back() != (size_t)id) P.pts.push_back((size_t)id);
                    }
                    else
                        S.ply = t;  // the last one listed wins
                }
            }
            else
                t = token(in);
        }
        if (ply) d->polylines[name] = P;
        if (sfc) d->surfaces[name] = S;
        kw = t;
    }
    return OGS_OK;
}

ogs_status read_bc(ogs_deck* d, const char* path)
{
    std::ifstream in(path);
    if (!in) { set_error("deck: cannot open %s", path); return OGS_BAD_ARG; }
    std::string line;
    Bc* cur = nullptr;
    // readNonBlankLineFromInputStream: the next line with content
    auto next_line = [&in](std::string& out) {
        while (std::getline(in, out))
            if (!trim(out).empty()) return true;
        return false;
    };
    while (next_line(line))
    {
        if (line.find("#BOUNDARY_CONDITION") != std::string::npos)
        {
            d->bcs.emplace_back();
            cur = &d->bcs.back();
            continue;
        }
        if (line.find("#STOP") != std::string::npos) break;
        if (!cur || line.find('$') == std::string::npos) continue;
        const bool pcs = line.find("$PCS_TYPE") != std::string::npos;
        const bool var = line.find("$PRIMARY_VARIABLE") != std::string::npos ||
                         line.find("$COMP_NAME") != std::string::npos;
        const bool geo = line.find("$GEO_TYPE") != std::string::npos;
        const bool dis = line.find("$DIS_TYPE") != std::string::npos;
        const bool eps = line.find("$EPSILON") != std::string::npos;
        if (!(pcs || var || geo || dis || eps)) continue;
        std::string v;
        if (!next_line(v)) break;
        std::istringstream ls(v);
        if (pcs) ls >> cur->pcs;
        else if (var) ls >> cur->var;
        else if (geo) ls >> cur->geo_type >> cur->geo_name;
        else if (eps) ls >> cur->eps;
        else
        {
            std::string kind;
            ls >> kind;
            if (kind != "CONSTANT" || !(ls >> cur->value))
            {
                set_error("deck: %s: only $DIS_TYPE CONSTANT is supported ('%s')", path, trim(v).c_str());
                return OGS_BAD_ARG;
            }
        }
    }
    return OGS_OK;
}

int64_t nearest(const ogs_deck* d, const double* p)
{
    int64_t best = -1;
    double bd = INFINITY;
    for (size_t j = 0; j < d->x.size(); j++)
    {
        const double dx = d->x[j] - p[0], dy = d->y[j] - p[1], dz = d->z[j] - p[2];
        const double s = dx * dx + dy * dy + dz * dz;
        if (s < bd) { bd = s; best = (int64_t)j; }
    }
    return best;
}

// MeshNodesAlongPolyline: nodes in order of their distance along the polyline
void nodes_on_polyline(const ogs_deck* d, const Polyline& P, double radius, std::vector<int64_t>& out)
{
    std::vector<std::pair<double, int64_t>> found;
    std::vector<char> taken(d->x.size(), 0);
    double run = 0.0;  // polyline length up to the segment start
    for (size_t k = 0; k + 1 < P.pts.size(); k++)
    {
        const double a[3] = {d->px[P.pts[k]], d->py[P.pts[k]], d->pz[P.pts[k]]};
        const double b[3] = {d->px[P.pts[k + 1]], d->py[P.pts[k + 1]], d->pz[P.pts[k + 1]]};
        const double v[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        const double seg = dist3(a, b);
        const double lo = -radius / seg, hi = 1 + radius / seg;
        for (size_t j = 0; j < d->x.size(); j++)
        {
            const double p[3] = {d->x[j], d->y[j], d->z[j]};
            const double lambda = ((p[0] - a[0]) * v[0] + (p[1] - a[1]) * v[1] + (p[2] - a[2]) * v[2]) / vv;
            const double q[3] = {a[0] + lambda * v[0], a[1] + lambda * v[1], a[2] + lambda * v[2]};
            if (dist3(p, q) <= radius && lo <= lambda && lambda <= hi && !taken[j])
            {
                taken[j] = 1;
                found.push_back({run + dist3(q, a), (int64_t)j});
            }
        }
        run += seg;
    }
    std::stable_sort(found.begin(), found.end(),
                     [](const std::pair<double, int64_t>& p, const std::pair<double, int64_t>& q) { return p.first < q.first; });
    for (auto& f : found) out.push_back(f.second);
}

// MathLib::isPointInTriangle restated: near a vertex, or the projection's
// parameters within eps of the triangle and the projection within eps
bool in_triangle(const double* q, const double* a, const double* b, const double* c, double eps)
{
    if (dist3(q, a) < eps || dist3(q, b) < eps || dist3(q, c) < eps) return true;
    const double v[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    const double m00 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double m01 = v[0] * w[0] + v[1] * w[1] + v[2] * w[2];
    const double m11 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const double r0 = v[0] * (q[0] - a[0]) + v[1] * (q[1] - a[1]) + v[2] * (q[2] - a[2]);
    const double r1 = w[0] * (q[0] - a[0]) + w[1] * (q[1] - a[1]) + w[2] * (q[2] - a[2]);
    const double det = m00 * m11 - m01 * m01;
    if (det == 0.0) return false;
    const double y0 = (r0 * m11 - r1 * m01) / det, y1 = (m00 * r1 - m01 * r0) / det;
    if (!(-eps <= y0 && y0 <= 1 + eps && -eps <= y1 && y1 <= 1 + eps && y0 + y1 <= 1 + eps)) return false;
    const double p[3] = {a[0] + y0 * v[0] + y1 * w[0], a[1] + y0 * v[1] + y1 * w[1], a[2] + y0 * v[2] + y1 * w[2]};
    return dist3(q, p) < eps;
}

// ear clipping of a simple polygon given in 2-D plane coordinates
void ear_clip(const std::vector<double>& u, const std::vector<double>& v, std::vector<int>& tris)
{
    std::vector<int> idx(u.size());
    for (size_t k = 0; k < u.size(); k++) idx[k] = (int)k;
    double area = 0;
    for (size_t k = 0, m = u.size() - 1; k < u.size(); m = k++) area += u[m] * v[k] - u[k] * v[m];
    if (area < 0) std::reverse(idx.begin(), idx.end());  // counter-clockwise
    auto cross = [&](int a, int b, int c) { return (u[b] - u[a]) * (v[c] - v[a]) - (v[b] - v[a]) * (u[c] - u[a]); };
    while (idx.size() > 3)
    {
        const size_t n = idx.size();
        size_t ear = n;
        for (size_t k = 0; k < n && ear == n; k++)
        {
            const int a = idx[(k + n - 1) % n], b = idx[k], c = idx[(k + 1) % n];
            if (cross(a, b, c) <= 0) continue;  // reflex or flat corner
            bool empty = true;
            for (size_t m = 0; m < n && empty; m++)
            {
                const int p = idx[m];
                if (p == a || p == b || p == c) continue;
                empty = !(cross(a, b, p) >= 0 && cross(b, c, p) >= 0 && cross(c, a, p) >= 0);
            }
            if (empty) ear = k;
        }
        if (ear == n) ear = 0;  // only flat corners left: clip one
        tris.push_back(idx[(ear + n - 1) % n]);
        tris.push_back(idx[ear]);
        tris.push_back(idx[(ear + 1) % n]);
        idx.erase(idx.begin() + (long)ear);
    }
    tris.insert(tris.end(), idx.begin(), idx.end());
}

// The grid of a surface's triangles that bounds its node search: the
// bounding box with its upper corner moved out by 1e-6 relative (a flat
// axis widened by 1e-3 of the largest extent), cut into cells so that
// about five triangles fall into one; a triangle is listed in every cell of
// the index box of its corners.  Cell indices are the truncated offsets;
// a negative offset truncates toward zero on the reference's x86 build
// (offsets in (-1, 0) give cell 0, lower ones no cell), which cell_of
// reproduces on every host.
struct SurfaceCells
{
    double lo[3], hi[3], inv[3];
    size_t n[3] = {1, 1, 1};
    std::vector<std::vector<int>> tri;  // per cell: first corners' offsets in the triangle list

    bool axis(int k, double p, size_t& i) const
    {
        const double t = std::trunc((p - lo[k]) * inv[k]);
        if (!(t > -1.0) || t >= (double)n[k]) return false;
        i = (size_t)(t < 0.0 ? 0.0 : t);
        return true;
    }
    bool cell_of(const double* p, size_t& c) const
    {
        size_t i, j, k;
        if (!axis(0, p[0], i) || !axis(1, p[1], j) || !axis(2, p[2], k)) return false;
        c = i + n[0] * (j + n[1] * k);
        return true;
    }
};

SurfaceCells surface_cells(const double* lo, const double* hi, const std::vector<double>& P,
                           const std::vector<int>& tris)
{
    SurfaceCells g;
    double dl[3];
    const double eps = std::numeric_limits<double>::epsilon();
    for (int k = 0; k < 3; k++)
    {
        g.lo[k] = lo[k];
        g.hi[k] = hi[k] + std::fabs(hi[k]) * 1e-6;
        if (std::fabs(g.hi[k]) < eps) g.hi[k] = (g.hi[k] - g.lo[k]) * (1.0 + 1e-6);
        dl[k] = g.hi[k] - g.lo[k];
    }
    for (int k = 0; k < 3; k++)
        if (dl[k] < eps)
        {
            const double m = std::max(dl[(k + 1) % 3], dl[(k + 2) % 3]);
            g.lo[k] -= m * 0.5e-3;
            g.hi[k] += m * 0.5e-3;
            dl[k] = g.hi[k] - g.lo[k];
        }
    const double nt = (double)(tris.size() / 3), per = 5.0;
    const bool f0 = std::fabs(dl[0]) < eps, f1 = std::fabs(dl[1]) < eps, f2 = std::fabs(dl[2]) < eps;
    auto up = [](double v) { return (size_t)std::ceil(v); };
    if (f0 || f1 || f2)
    {
        if (f1 && f2) g.n[0] = up(nt / per);
        else if (f0 && f2) g.n[1] = up(nt / per);
        else if (f0 && f1) g.n[2] = up(nt / per);
        else if (f1)
        {
            g.n[0] = up(std::sqrt(nt * dl[0] / (per * dl[2])));
            g.n[2] = up(g.n[0] * dl[2] / dl[0]);
        }
        else if (f2)
        {
            g.n[0] = up(std::sqrt(nt * dl[0] / (per * dl[1])));
            g.n[1] = up(g.n[0] * dl[1] / dl[0]);
        }
        else
        {
            g.n[1] = up(std::sqrt(nt / per * dl[1] / dl[2]));
            g.n[2] = up(nt * dl[2] / (per * dl[1]));
        }
    }
    else
    {
        g.n[0] = up(std::pow(nt * dl[0] * dl[0] / (per * dl[1] * dl[2]), 1.0 / 3.0));
        g.n[1] = up(g.n[0] * std::min(dl[1] / dl[0], 100.0));
        g.n[2] = up(g.n[0] * std::min(dl[2] / dl[0], 100.0));
    }
    for (int k = 0; k < 3; k++) g.inv[k] = 1.0 / (dl[k] / (double)g.n[k]);
    g.tri.assign(g.n[0] * g.n[1] * g.n[2], {});
    for (size_t t = 0; t < tris.size(); t += 3)
    {
        // the corners' cells (a corner is inside the grid by construction)
        size_t mn[3] = {SIZE_MAX, SIZE_MAX, SIZE_MAX}, mx[3] = {0, 0, 0};
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++)
            {
                size_t i = 0;
                if (!g.axis(k, P[3 * tris[t + v] + k], i)) i = 0;
                mn[k] = std::min(mn[k], i);
                mx[k] = std::max(mx[k], i);
            }
        for (size_t i = mn[0]; i <= mx[0]; i++)
            for (size_t j = mn[1]; j <= mx[1]; j++)
                for (size_t k = mn[2]; k <= mx[2]; k++)
                    g.tri[i + g.n[0] * (j + g.n[1] * k)].push_back((int)t);
    }
    return g;
}

ogs_status nodes_on_surface(const ogs_deck* d, const Surface& S, double eps, std::vector<int64_t>& out)
{
    auto it = d->polylines.find(S.ply);
    if (it == d->polylines.end()) { set_error("deck: surface uses unknown polyline '%s'", S.ply.c_str()); return OGS_BAD_ARG; }
    std::vector<size_t> poly = it->second.pts;
    if (poly.size() > 1 && poly.front() == poly.back()) poly.pop_back();  // closed
    if (poly.size() < 3) { set_error("deck: surface needs a polygon of at least 3 points"); return OGS_BAD_ARG; }
    const size_t np = poly.size();
    std::vector<double> P(3 * np);
    double nrm[3] = {0, 0, 0}, c[3] = {0, 0, 0};
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t k = 0; k < np; k++)
    {
        P[3 * k] = d->px[poly[k]];
        P[3 * k + 1] = d->py[poly[k]];
        P[3 * k + 2] = d->pz[poly[k]];
    }
    // Newell normal and an in-plane frame for the triangulation
    for (size_t k = 0; k < np; k++)
    {
        const double* a = &P[3 * k];
        const double* b = &P[3 * ((k + 1) % np)];
        nrm[0] += (a[1] - b[1]) * (a[2] + b[2]);
        nrm[1] += (a[2] - b[2]) * (a[0] + b[0]);
        nrm[2] += (a[0] - b[0]) * (a[1] + b[1]);
        for (int q = 0; q < 3; q++)
        {
            c[q] += a[q] / (double)np;
            lo[q] = std::min(lo[q], a[q]);
            hi[q] = std::max(hi[q], a[q]);
        }
    }
    const double nl = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    if (!(nl > 0)) { set_error("deck: degenerate surface polygon"); return OGS_BAD_ARG; }
    for (double& q : nrm) q /= nl;
    double e1[3] = {P[3] - P[0], P[4] - P[1], P[5] - P[2]};
    const double l1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (double& q : e1) q /= l1;
    const double e2[3] = {nrm[1] * e1[2] - nrm[2] * e1[1], nrm[2] * e1[0] - nrm[0] * e1[2], nrm[0] * e1[1] - nrm[1] * e1[0]};
    std::vector<double> pu(np), pv(np);
    for (size_t k = 0; k < np; k++)
    {
        const double w[3] = {P[3 * k] - c[0], P[3 * k + 1] - c[1], P[3 * k + 2] - c[2]};
        pu[k] = w[0] * e1[0] + w[1] * e1[1] + w[2] * e1[2];
        pv[k] = w[0] * e2[0] + w[1] * e2[1] + w[2] * e2[2];
    }
    std::vector<int> tris;
    ear_clip(pu, pv, tris);
    const SurfaceCells grid = surface_cells(lo, hi, P, tris);
    for (size_t j = 0; j < d->x.size(); j++)
    {
        const double p[3] = {d->x[j], d->y[j], d->z[j]};
        bool in_bv = true;
        for (int q = 0; q < 3; q++)
            in_bv = in_bv && ((lo[q] <= p[q] && p[q] <= hi[q]) || std::fabs(lo[q] - p[q]) < eps ||
                              std::fabs(p[q] - hi[q]) < eps);
        size_t cell = 0;
        if (!in_bv || !grid.cell_of(p, cell)) continue;
        for (int t : grid.tri[cell])
            if (in_triangle(p, &P[3 * tris[t]], &P[3 * tris[t + 1]], &P[3 * tris[t + 2]], eps))
            {
                out.push_back((int64_t)j);
                break;
            }
    }
    return OGS_OK;
}

// the node set of one CONSTANT boundary condition, in the order the
// reference appends its nodes to bc_node_value
ogs_status bc_nodes(const ogs_deck* d, const std::string& type, const std::string& name, double bc_eps,
                    std::vector<int64_t>& out)
{
    if (type == "POINT")
    {
        auto it = d->point_names.find(name);
        if (it == d->point_names.end() || it->second < 0 || it->second >= (long)d->px.size())
        {
            set_error("deck: unknown point '%s'", name.c_str());
            return OGS_BAD_ARG;
        }
        const double p[3] = {d->px[it->second], d->py[it->second], d->pz[it->second]};
        out.push_back(nearest(d, p));
        return OGS_OK;
    }
    if (type == "POLYLINE")
    {
        auto it = d->polylines.find(name);
        if (it == d->polylines.end()) { set_error("deck: unknown polyline '%s'", name.c_str()); return OGS_BAD_ARG; }
        const size_t first = out.size();
        nodes_on_polyline(d, it->second, it->second.eps, out);
        std::sort(out.begin() + (long)first, out.end());
        return OGS_OK;
    }
    if (type == "SURFACE")
    {
        auto it = d->surfaces.find(name);
        if (it == d->surfaces.end()) { set_error("deck: unknown surface '%s'", name.c_str()); return OGS_BAD_ARG; }
        return nodes_on_surface(d, it->second, bc_eps != -1 ? bc_eps : 0.375 * d->min_edge / 2, out);
    }
    set_error("deck: geometry type '%s' is not supported (POINT, POLYLINE, SURFACE)", type.c_str());
    return OGS_BAD_ARG;
}

ogs_status copy_out(const std::vector<int64_t>& rows, const std::vector<double>* vals, int64_t* r, double* v,
                    int64_t cap, int64_t* n)
{
    if (n) *n = (int64_t)rows.size();
    if (!r) return OGS_OK;  // size query
    if ((int64_t)rows.size() > cap)
    {
        set_error("deck: %zu rows do not fit a capacity of %lld", rows.size(), (long long)cap);
        return OGS_BAD_ARG;
    }
    std::copy(rows.begin(), rows.end(), r);
    if (vals && v) std::copy(vals->begin(), vals->end(), v);
    return OGS_OK;
}

}  // namespace

extern "C" ogs_status ogs_deck_read(const char* msh_path, const char* gli_path, const char* bc_path, ogs_deck** out)
{
    if (!msh_path || !out) { set_error("deck_read: NULL argument"); return OGS_BAD_ARG; }
    *out = nullptr;
    ogs_deck* d = new ogs_deck;
    ogs_status st = read_msh(d, msh_path);
    if (!st && gli_path) st = read_gli(d, gli_path);
    if (!st && bc_path) st = read_bc(d, bc_path);
    if (st) { delete d; return st; }
    *out = d;
    return OGS_OK;
}

extern "C" ogs_status ogs_deck_destroy(ogs_deck* d)
{
    delete d;
    return OGS_OK;
}

extern "C" ogs_status ogs_deck_mesh(const ogs_deck* d, ogs_mesh_desc* desc, double* min_edge_length)
{
    if (!d || !desc) { set_error("deck_mesh: NULL argument"); return OGS_BAD_ARG; }
    if (min_edge_length) *min_edge_length = d->min_edge;
    std::memset(desc, 0, sizeof *desc);
    if (d->elem_type < 0)
    {
        set_error("deck_mesh: %s elements are not on the GPU path (quad, hex, tet)", d->kind->name);
        return OGS_BAD_ARG;
    }
    desc->elem_type = d->elem_type;
    desc->dim = d->dim;
    desc->n_nodes = (int64_t)d->x.size();
    desc->n_elements = (int64_t)(d->conn.size() / d->kind->nodes);
    desc->x = d->x.data();
    desc->y = d->y.data();
    desc->z = d->dim == 3 ? d->z.data() : nullptr;
    desc->connectivity = d->conn.data();
    desc->gauss_points = 3;
    return OGS_OK;
}

extern "C" ogs_status ogs_deck_geo_nodes(const ogs_deck* d, const char* geo_type, const char* name, int64_t* rows,
                                         int64_t capacity, int64_t* n)
{
    if (!d || !geo_type || !name) { set_error("deck_geo_nodes: NULL argument"); return OGS_BAD_ARG; }
    std::vector<int64_t> r;
    const ogs_status st = bc_nodes(d, geo_type, name, -1.0, r);
    if (st) return st;
    return copy_out(r, nullptr, rows, nullptr, capacity, n);
}

extern "C" ogs_status ogs_deck_dirichlet(const ogs_deck* d, const char* pcs_type, const char* primary_variable,
                                         int64_t* rows, double* values, int64_t capacity, int64_t* n)
{
    if (!d || !pcs_type) { set_error("deck_dirichlet: NULL argument"); return OGS_BAD_ARG; }
    std::vector<int64_t> r;
    std::vector<double> v;
    for (const Bc& b : d->bcs)
    {
        if (b.pcs != pcs_type) continue;
        if (primary_variable && b.var != primary_variable) continue;
        const ogs_status st = bc_nodes(d, b.geo_type, b.geo_name, b.eps, r);
        if (st) return st;
        v.resize(r.size(), b.value);
    }
    return copy_out(r, &v, rows, values, capacity, n);
}
