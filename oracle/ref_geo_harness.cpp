// TEST INFRASTRUCTURE ONLY: a C front end of the reference's own geometry
// code (GEO/Surface.cpp, GEO/SurfaceGrid.cpp, GEO/Polygon.cpp,
// GEO/Polyline.cpp, MathLib/AnalyticalGeometry.cpp,
// MathLib/EarClippingTriangulation.cpp, MathLib/MathTools.cpp,
// FEM/mathlib.cpp, compiled unmodified where they lie) for checking the deck
// reader's node searches.  Built into _ref/libogs5geo.so by oracle/Makefile
// only where the reference sources are present.
//
// The loops over mesh nodes are the few lines of the reference's callers,
// which live in CFEMesh and cannot be compiled without the whole mesh
// library; each names what it follows.
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "MathTools.h"
#include "Point.h"
#include "Polygon.h"
#include "Polyline.h"
#include "Surface.h"
#include "display.h"
#include "quicksort.h"

/* Symbols that the geometry sources and FEM/mathlib.cpp (linked for
 * NormalizeVector, which Triangle::calculateNormal calls) reference from
 * libraries outside this build; none of the functions called here reaches
 * the aborting ones. */
double MSkalarprodukt(double*, double*, long) { std::abort(); }
void M3KreuzProdukt(double*, double*, double*) { std::abort(); }
double MCalcDistancePointToPoint(double*, double*) { std::abort(); }
namespace Display
{
void ScreenMessage(const char*, ...) {}
void DisplayErrorMsg(const char*) { std::abort(); }
}

namespace {

std::vector<GEOLIB::Point*>* points(int n, const double* xyz)
{
    auto* v = new std::vector<GEOLIB::Point*>;
    for (int i = 0; i < n; i++) v->push_back(new GEOLIB::Point(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
    return v;
}

void free_points(std::vector<GEOLIB::Point*>* v)
{
    for (GEOLIB::Point* p : *v) delete p;
    delete v;
}

}  // namespace

extern "C" {

/* CFEMesh::GetNODOnSFC without PETSc (MSH/msh_mesh.cpp:1917-1928) on the
 * surface of a closed polygon (Surface::createSurface). */
int ref_geo_surface_nodes(int np, const double* poly_xyz, int64_t nn, const double* nodes, double eps,
                          uint8_t* mask)
{
    std::vector<GEOLIB::Point*>* pts = points(np, poly_xyz);
    GEOLIB::Polyline ply(*pts);
    for (int i = 0; i < np; i++) ply.addPoint(i);
    ply.addPoint(0);
    GEOLIB::Surface* sfc = GEOLIB::Surface::createSurface(ply);
    if (!sfc) { free_points(pts); return -1; }
    sfc->initSurfaceGrid();
    for (int64_t j = 0; j < nn; j++)
        mask[j] = sfc->isPntInBV(nodes + 3 * j, eps) && sfc->isPntInSfc(nodes + 3 * j, eps);
    delete sfc;
    free_points(pts);
    return 0;
}

/* MeshNodesAlongPolyline::MeshNodesAlongPolyline for a linear mesh
 * (MSH/MeshNodesAlongPolyline.cpp:30-80): node ids in order of their
 * distance along the polyline; returns the count. */
int64_t ref_geo_polyline_nodes(int np, const double* xyz, int64_t nn, const double* nodes, double radius,
                               int64_t* ids, double* dist)
{
    std::vector<GEOLIB::Point*>* pts = points(np, xyz);
    GEOLIB::Polyline ply(*pts);
    for (int i = 0; i < np; i++) ply.addPoint(i);
    std::vector<size_t> found;
    std::vector<double> d;
    for (size_t k = 0; k + 1 < ply.getNumberOfPoints(); k++)
    {
        const double act = ply.getLength(k);
        const double seg = sqrt(MathLib::sqrDist(ply.getPoint(k), ply.getPoint(k + 1)));
        const double lo = -radius / seg, hi = 1 + radius / seg;
        for (int64_t j = 0; j < nn; j++)
        {
            double lambda, d0;
            if (MathLib::calcProjPntToLineAndDists(nodes + 3 * j, ply.getPoint(k)->getData(),
                                                   ply.getPoint(k + 1)->getData(), lambda, d0) <= radius &&
                lo <= lambda && lambda <= hi)
            {
                bool have = false;
                for (size_t f : found) have |= f == (size_t)j;
                if (!have)
                {
                    found.push_back((size_t)j);
                    d.push_back(act + d0);
                }
            }
        }
    }
    Quicksort<double>(d, 0, d.size(), found);
    for (size_t k = 0; k < found.size(); k++)
    {
        ids[k] = (int64_t)found[k];
        dist[k] = d[k];
    }
    free_points(pts);
    return (int64_t)found.size();
}

/* GEOLIB::Polygon::isPntInPolygon of a closed polygon. */
int ref_geo_point_in_polygon(int np, const double* poly_xyz, int64_t nq, const double* q, uint8_t* mask)
{
    std::vector<GEOLIB::Point*>* pts = points(np, poly_xyz);
    GEOLIB::Polyline ply(*pts);
    for (int i = 0; i < np; i++) ply.addPoint(i);
    ply.addPoint(0);
    GEOLIB::Polygon polygon(ply);
    for (int64_t j = 0; j < nq; j++) mask[j] = polygon.isPntInPolygon(q[3 * j], q[3 * j + 1], q[3 * j + 2]);
    free_points(pts);
    return 0;
}

}  // extern "C"
