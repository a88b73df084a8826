/*
 * ogs_oracle.c -- CPU restatement of the OGS-5 flow/transport hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  The product path (ogs5_gb300, libogs_gpu.so) never calls it.
 *
 * Every function follows the reference function cited beside it, in the
 * reference's operation order where that is cheap to keep, so that results
 * agree with OGS-5 to rounding.  Plain C99, single thread, FP64, compiled
 * with -ffp-contract=off so x86 and Arm give the same bits.
 *
 * Pinning: the Gauss/shape tables are checked against the reference's own
 * FEM/mathlib.cpp, and the CSR solve path against the reference's own
 * Linear_EQS / CSparseMatrix (FEM/equation_class.cpp, FEM/matrix_class.cpp),
 * both compiled from the reference sources into oracle/_ref by
 * oracle/Makefile; element matrices are pinned by closed-form known answers.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/ogs_gpu.h"

#define ORC_MAX_GP 27

/* ------------------------------------------------------------------ */
/* Quadrature and shape functions                                      */
/* ------------------------------------------------------------------ */

/* MXPGaussPkt (FEM/mathlib.cpp:1112): Gauss-Legendre abscissae, the
 * reference's 15-digit constants. */
double orc_gauss_point(long grd, long pkt)
{
    switch (grd)
    {
        case 1:
            return 0.0;
        case 2:
            return pkt == 0 ? 0.577350269189626 : -0.577350269189626;
        case 3:
            if (pkt == 0) return 0.774596669241483;
            if (pkt == 1) return 0.0;
            return -0.774596669241483;
        case 4:
            if (pkt == 0) return 0.861136311594053;
            if (pkt == 1) return 0.339981043584856;
            if (pkt == 2) return -0.339981043584856;
            return -0.861136311594053;
    }
    return 0.0;
}

/* MXPGaussFkt (FEM/mathlib.cpp:1174): Gauss-Legendre weights. */
double orc_gauss_weight(long grd, long pkt)
{
    switch (grd)
    {
        case 1:
            return 2.0;
        case 2:
            return 1.0;
        case 3:
            return pkt == 1 ? 0.888888888888889 : 0.555555555555556;
        case 4:
            return (pkt == 0 || pkt == 3) ? 0.347854845137454
                                          : 0.652145154862546;
    }
    return 0.0;
}

/* SamplePointTet5 (FEM/mathlib.cpp:1285): 5-point tet rule, one negative
 * weight. sp[0..2] local coordinates, sp[3] weight. */
void orc_tet5_point(int n, double* sp)
{
    const double a = 0.166666666666667;
    switch (n)
    {
        case 0: sp[0] = 0.25; sp[1] = 0.25; sp[2] = 0.25; sp[3] = -0.133333333333333; break;
        case 1: sp[0] = a; sp[1] = a; sp[2] = a; sp[3] = 0.07500000000000; break;
        case 2: sp[0] = 0.5; sp[1] = a; sp[2] = a; sp[3] = 0.07500000000000; break;
        case 3: sp[0] = a; sp[1] = 0.5; sp[2] = a; sp[3] = 0.07500000000000; break;
        case 4: sp[0] = a; sp[1] = a; sp[2] = 0.5; sp[3] = 0.07500000000000; break;
        default: break;
    }
}

/* ShapeFunctionQuad / GradShapeFunctionQuad (FEM/mathlib.cpp:1880,1908). */
static void shape_quad(double* N, double* dN, const double* u)
{
    N[0] = (1.0 + u[0]) * (1.0 + u[1]);
    N[1] = (1.0 - u[0]) * (1.0 + u[1]);
    N[2] = (1.0 - u[0]) * (1.0 - u[1]);
    N[3] = (1.0 + u[0]) * (1.0 - u[1]);
    for (int i = 0; i < 4; i++) N[i] *= 0.25;
    dN[0] = +(1.0 + u[1]);
    dN[1] = -(1.0 + u[1]);
    dN[2] = -(1.0 - u[1]);
    dN[3] = +(1.0 - u[1]);
    dN[4] = +(1.0 + u[0]);
    dN[5] = +(1.0 - u[0]);
    dN[6] = -(1.0 - u[0]);
    dN[7] = -(1.0 + u[0]);
    for (int i = 0; i < 8; i++) dN[i] *= 0.25;
}

/* ShapeFunctionHex / GradShapeFunctionHex (FEM/mathlib.cpp:2224,2264). */
static void shape_hex(double* N, double* dN, const double* x)
{
    const double r = x[0], s = x[1], t = x[2];
    N[0] = (1.0 + r) * (1.0 + s) * (1.0 + t);
    N[1] = (1.0 - r) * (1.0 + s) * (1.0 + t);
    N[2] = (1.0 - r) * (1.0 - s) * (1.0 + t);
    N[3] = (1.0 + r) * (1.0 - s) * (1.0 + t);
    N[4] = (1.0 + r) * (1.0 + s) * (1.0 - t);
    N[5] = (1.0 - r) * (1.0 + s) * (1.0 - t);
    N[6] = (1.0 - r) * (1.0 - s) * (1.0 - t);
    N[7] = (1.0 + r) * (1.0 - s) * (1.0 - t);
    for (int i = 0; i < 8; i++) N[i] *= 0.125;
    dN[0] = +(1.0 + s) * (1.0 + t);
    dN[1] = -(1.0 + s) * (1.0 + t);
    dN[2] = -(1.0 - s) * (1.0 + t);
    dN[3] = +(1.0 - s) * (1.0 + t);
    dN[4] = +(1.0 + s) * (1.0 - t);
    dN[5] = -(1.0 + s) * (1.0 - t);
    dN[6] = -(1.0 - s) * (1.0 - t);
    dN[7] = +(1.0 - s) * (1.0 - t);
    dN[8] = +(1.0 + r) * (1.0 + t);
    dN[9] = +(1.0 - r) * (1.0 + t);
    dN[10] = -(1.0 - r) * (1.0 + t);
    dN[11] = -(1.0 + r) * (1.0 + t);
    dN[12] = +(1.0 + r) * (1.0 - t);
    dN[13] = +(1.0 - r) * (1.0 - t);
    dN[14] = -(1.0 - r) * (1.0 - t);
    dN[15] = -(1.0 + r) * (1.0 - t);
    dN[16] = +(1.0 + r) * (1.0 + s);
    dN[17] = +(1.0 - r) * (1.0 + s);
    dN[18] = +(1.0 - r) * (1.0 - s);
    dN[19] = +(1.0 + r) * (1.0 - s);
    dN[20] = -(1.0 + r) * (1.0 + s);
    dN[21] = -(1.0 - r) * (1.0 + s);
    dN[22] = -(1.0 - r) * (1.0 - s);
    dN[23] = -(1.0 + r) * (1.0 - s);
    for (int i = 0; i < 24; i++) dN[i] *= 0.125;
}

/* ShapeFunctionTet / GradShapeFunctionTet (FEM/mathlib.cpp:2079,2103). */
static void shape_tet(double* N, double* dN, const double* x)
{
    N[0] = 1. - x[0] - x[1] - x[2];
    N[1] = x[0];
    N[2] = x[1];
    N[3] = x[2];
    static const double g[12] = {-1.0, 1.0, 0.0, 0.0, -1.0, 0.0,
                                 1.0,  0.0, -1.0, 0.0, 0.0, 1.0};
    memcpy(dN, g, sizeof g);
}

int orc_nodes_per_element(int etype)
{
    return etype == OGS_ELEM_HEX8 ? 8 : 4;
}

int orc_elem_dim(int etype)
{
    return etype == OGS_ELEM_QUAD4 ? 2 : 3;
}

/* CElement::SetIntegrationPointNumber (FEM/fem_ele.cpp:362-393). */
int orc_num_gauss_points(int etype, int ngauss)
{
    if (etype == OGS_ELEM_QUAD4) return ngauss * ngauss;
    if (etype == OGS_ELEM_HEX8) return ngauss * ngauss * ngauss;
    return 5;
}

/* ShapeFunctionPool::computeQuadratures (FEM/ShapeFunctionPool.cpp:110-160)
 * with CElement::SetGaussPoint and GetGaussData (FEM/fem_ele.cpp:885-1000):
 * per Gauss point the local coordinates, the weight product, N and dN/dxi
 * (row-major [dim][nn]).  Returns the number of Gauss points. */
int orc_shape_table(int etype, int ngauss, double* xi, double* w, double* N,
                    double* dN, double* w3)
{
    const int nn = orc_nodes_per_element(etype);
    const int dim = orc_elem_dim(etype);
    const int ngp = orc_num_gauss_points(etype, ngauss);
    for (int gp = 0; gp < ngp; gp++)
    {
        double u[4] = {0, 0, 0, 0};
        double wt;
        if (etype == OGS_ELEM_QUAD4)
        {
            int gr = gp / ngauss, gs = gp % ngauss;
            u[0] = orc_gauss_point(ngauss, gr);
            u[1] = orc_gauss_point(ngauss, gs);
            wt = orc_gauss_weight(ngauss, gr) * orc_gauss_weight(ngauss, gs);
            if (w3)
            {
                w3[gp * 3 + 0] = orc_gauss_weight(ngauss, gr);
                w3[gp * 3 + 1] = orc_gauss_weight(ngauss, gs);
                w3[gp * 3 + 2] = 1.0;
            }
            shape_quad(N + gp * nn, dN + gp * nn * dim, u);
        }
        else if (etype == OGS_ELEM_HEX8)
        {
            int gr = gp / (ngauss * ngauss);
            int gs = gp % (ngauss * ngauss);
            int gt = gs % ngauss;
            gs /= ngauss;
            u[0] = orc_gauss_point(ngauss, gr);
            u[1] = orc_gauss_point(ngauss, gs);
            u[2] = orc_gauss_point(ngauss, gt);
            /* GetGaussData multiplies det * w_r * w_s * w_t left to right */
            wt = orc_gauss_weight(ngauss, gr) * orc_gauss_weight(ngauss, gs) *
                 orc_gauss_weight(ngauss, gt);
            if (w3)
            {
                w3[gp * 3 + 0] = orc_gauss_weight(ngauss, gr);
                w3[gp * 3 + 1] = orc_gauss_weight(ngauss, gs);
                w3[gp * 3 + 2] = orc_gauss_weight(ngauss, gt);
            }
            shape_hex(N + gp * nn, dN + gp * nn * dim, u);
        }
        else
        {
            orc_tet5_point(gp, u);
            wt = u[3];
            if (w3)
            {
                w3[gp * 3 + 0] = u[3];
                w3[gp * 3 + 1] = 1.0;
                w3[gp * 3 + 2] = 1.0;
            }
            shape_tet(N + gp * nn, dN + gp * nn * dim, u);
        }
        if (xi)
        {
            xi[gp * 3 + 0] = u[0];
            xi[gp * 3 + 1] = u[1];
            xi[gp * 3 + 2] = etype == OGS_ELEM_QUAD4 ? 0.0 : u[2];
        }
        w[gp] = wt;
    }
    return ngp;
}

/* ------------------------------------------------------------------ */
/* Element geometry                                                    */
/* ------------------------------------------------------------------ */

/* CElement::computeJacobian (FEM/fem_ele.cpp:585-743) followed by
 * CElement::ComputeGradShapefct (fem_ele.cpp:1128-1200): global gradients
 * dNg[j*nn+i] = sum_k invJ[j*dim+k] dN[k*nn+i] and |det J|.
 * Returns 0 on success, -1 when |det J| < DBL_EPSILON (the reference aborts). */
static int grad_global(int dim, int nn, const double* X, const double* Y,
                       const double* Z, const double* dN, double* dNg,
                       double* detabs)
{
    double J[9] = {0}, iJ[9];
    double det;
    if (dim == 2)
    {
        for (int i = 0, j = nn; i < nn; i++, j++)
        {
            J[0] += X[i] * dN[i];
            J[1] += Y[i] * dN[i];
            J[2] += X[i] * dN[j];
            J[3] += Y[i] * dN[j];
        }
        det = J[0] * J[3] - J[1] * J[2];
        if (fabs(det) < DBL_EPSILON) return -1;
        iJ[0] = J[3];
        iJ[1] = -J[1];
        iJ[2] = -J[2];
        iJ[3] = J[0];
        for (int i = 0; i < 4; i++) iJ[i] /= det;
    }
    else
    {
        for (int i = 0; i < nn; i++)
        {
            const int j = i + nn, k = i + 2 * nn;
            J[0] += X[i] * dN[i];
            J[1] += Y[i] * dN[i];
            J[2] += Z[i] * dN[i];
            J[3] += X[i] * dN[j];
            J[4] += Y[i] * dN[j];
            J[5] += Z[i] * dN[j];
            J[6] += X[i] * dN[k];
            J[7] += Y[i] * dN[k];
            J[8] += Z[i] * dN[k];
        }
        det = J[0] * (J[4] * J[8] - J[7] * J[5]) +
              J[6] * (J[1] * J[5] - J[4] * J[2]) +
              J[3] * (J[2] * J[7] - J[8] * J[1]);
        if (fabs(det) < DBL_EPSILON) return -1;
        iJ[0] = J[4] * J[8] - J[7] * J[5];
        iJ[1] = J[2] * J[7] - J[1] * J[8];
        iJ[2] = J[1] * J[5] - J[2] * J[4];
        iJ[3] = J[5] * J[6] - J[8] * J[3];
        iJ[4] = J[0] * J[8] - J[6] * J[2];
        iJ[5] = J[2] * J[3] - J[5] * J[0];
        iJ[6] = J[3] * J[7] - J[6] * J[4];
        iJ[7] = J[1] * J[6] - J[7] * J[0];
        iJ[8] = J[0] * J[4] - J[3] * J[1];
        for (int i = 0; i < 9; i++) iJ[i] /= det;
    }
    for (int i = 0; i < nn; i++)
        for (int j = 0; j < dim; j++)
        {
            double s = 0.0;
            for (int k = 0; k < dim; k++) s += iJ[j * dim + k] * dN[k * nn + i];
            dNg[j * nn + i] = s;
        }
    *detabs = fabs(det);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Element matrices                                                    */
/* ------------------------------------------------------------------ */

typedef struct
{
    double mass[64], laplace[64], advection[64], storage[64];
    double rhs_gravity[8];
} orc_elem_mats;

/* MassDispersionTensorNew (FEM/rf_mmp_new.cpp:3090-3328), isotropic
 * tortuosity, no bubble velocity, no Chiogna alpha_t model, no hard
 * stabilisation.  Returns the dim x dim tensor in D. */
static void dispersion_tensor(int dim, const ogs_assembly_params* p,
                              const double* v, double* D)
{
    const double dm = p->diffusion * p->porosity * p->saturation;
    const double vg = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double md[9] = {0};
    for (int i = 0; i < dim; i++) md[i * dim + i] = dm;
    if (fabs(vg) > DBL_EPSILON)
    {
        const double al = p->alpha_l, at = p->alpha_t;
        if (dim == 2)
        {
            D[0] = (at * vg) + (al - at) * (v[0] * v[0]) / vg;
            D[1] = ((al - at) * (v[0] * v[1])) / vg;
            D[2] = ((al - at) * (v[1] * v[0])) / vg;
            D[3] = (at * vg) + (al - at) * (v[1] * v[1]) / vg;
            D[0] += md[0];
            D[3] += md[3];
        }
        else
        {
            D[0] = (at * vg) + (al - at) * (v[0] * v[0]) / vg;
            D[1] = ((al - at) * (v[0] * v[1])) / vg;
            D[2] = ((al - at) * (v[0] * v[2])) / vg;
            D[3] = ((al - at) * (v[1] * v[0])) / vg;
            D[4] = (at * vg) + (al - at) * (v[1] * v[1]) / vg;
            D[5] = ((al - at) * (v[1] * v[2])) / vg;
            D[6] = ((al - at) * (v[2] * v[0])) / vg;
            D[7] = ((al - at) * (v[2] * v[1])) / vg;
            D[8] = (at * vg) + (al - at) * (v[2] * v[2]) / vg;
            D[0] += md[0];
            D[4] += md[4];
            D[8] += md[8];
        }
    }
    else
        for (int i = 0; i < dim * dim; i++) D[i] = md[i];
}

/* ComputeDetTri (FEM/mathlib.cpp:2911-2928): area of the triangle */
static double det_tri(const double* x1, const double* x2, const double* x3)
{
    double u[3], v[3], z[3];
    for (int k = 0; k < 3; k++)
    {
        u[k] = x3[k] - x1[k];
        v[k] = x2[k] - x1[k];
    }
    z[0] = u[1] * v[2] - u[2] * v[1];
    z[1] = u[2] * v[0] - u[0] * v[2];
    z[2] = u[0] * v[1] - u[1] * v[0];
    return 0.5 * sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
}

/* ComputeDetTex (FEM/mathlib.cpp:2945-2955): volume of the tetrahedron */
static double det_tex(const double* x1, const double* x2, const double* x3, const double* x4)
{
    return fabs((x1[0] - x4[0]) * ((x2[1] - x4[1]) * (x3[2] - x4[2]) - (x2[2] - x4[2]) * (x3[1] - x4[1])) -
                (x1[1] - x4[1]) * ((x2[0] - x4[0]) * (x3[2] - x4[2]) - (x2[2] - x4[2]) * (x3[0] - x4[0])) +
                (x1[2] - x4[2]) * ((x2[0] - x4[0]) * (x3[1] - x4[1]) - (x2[1] - x4[1]) * (x3[0] - x4[0]))) /
           6.0;
}

/* CElem::calcVolume (MSH/msh_elem.cpp:1511-1576): quads as two triangles,
 * hexahedra as six tetrahedra, in the node order of the mesh */
double orc_element_volume(int etype, const double* X, const double* Y, const double* Z)
{
    double P[8][3];
    const int nn = orc_nodes_per_element(etype);
    for (int i = 0; i < nn; i++)
    {
        P[i][0] = X[i];
        P[i][1] = Y[i];
        P[i][2] = Z ? Z[i] : 0.0;
    }
    if (etype == OGS_ELEM_QUAD4) return det_tri(P[0], P[1], P[2]) + det_tri(P[2], P[3], P[0]);
    if (etype == OGS_ELEM_TET4) return det_tex(P[0], P[1], P[2], P[3]);
    double v = det_tex(P[4], P[7], P[5], P[0]);
    v += det_tex(P[5], P[3], P[1], P[0]);
    v += det_tex(P[5], P[7], P[3], P[0]);
    v += det_tex(P[5], P[7], P[6], P[2]);
    v += det_tex(P[1], P[3], P[5], P[2]);
    v += det_tex(P[3], P[7], P[5], P[2]);
    return v;
}

/* MLangevin (FEM/mathlib.cpp:3009-3021): coth(v) - 1/v, its series
 * v/3 - v^3/45 + 2 v^5/945 below 0.01, 1 from 20 on */
static double langevin(double v)
{
    double s = 0.0;
    if (v < 0.01)
        s = v * (1.0 / 3.0 + v * v * (-1.0 / 45.0 + 18.0 / 8505.0 * v * v));
    else if (0.01 <= v && v < 20)
        s = (exp(v) + exp(-v)) / (exp(v) - exp(-v)) - 1 / v;
    else if (20 <= v)
        s = 1.0;
    return s;
}

/* CalcSUPGEffectiveElemenetLength (fem_ele_std.cpp:4034-4095) over the
 * edges of CElem::GetLocalIndicesOfEdgeNodes (MSH/msh_elem.cpp:984-1052) */
double orc_supg_length(int etype, const double* X, const double* Y, const double* Z, int method)
{
    int ne, a[12], b[12];
    if (etype == OGS_ELEM_QUAD4)
    {
        ne = 4;
        for (int e = 0; e < 4; e++) { a[e] = e; b[e] = (e + 1) % 4; }
    }
    else if (etype == OGS_ELEM_HEX8)
    {
        ne = 12;
        for (int e = 0; e < 12; e++)
        {
            if (e < 8) { a[e] = e; b[e] = (e + 1) % 4 + 4 * (e / 4); }
            else { a[e] = e % 4; b[e] = e % 4 + 4; }
        }
    }
    else
    {
        ne = 6;
        for (int e = 0; e < 6; e++)
        {
            if (e < 3) { a[e] = e; b[e] = (e + 1) % 3; }
            else { a[e] = 3; b[e] = (e + 1) % 3; }
        }
    }
    double len[12];
    for (int e = 0; e < ne; e++)
    {
        const double dx = X[b[e]] - X[a[e]], dy = Y[b[e]] - Y[a[e]], dz = (Z ? Z[b[e]] - Z[a[e]] : 0.0);
        len[e] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    double L = 0.0;
    if (method == 1)
    {
        double mn = len[0];
        for (int e = 1; e < ne; e++) { L = len[e]; if (L < mn) mn = L; }
        L = mn;
    }
    else if (method == 2)
    {
        double t = 0.0;
        for (int e = 1; e < ne; e++) t += len[e];  /* the reference starts at edge 1 */
        L = t / ne;
    }
    else
    {
        double mx = len[0];
        for (int e = 1; e < ne; e++) { L = len[e]; if (L > mx) mx = L; }
        L = mx;
    }
    return L;
}

/* CalcSUPGCoefficient (fem_ele_std.cpp:3908-3995) for MASS_TRANSPORT:
 * D is the raw MassDispersionTensorNew of the Gauss point */
static double supg_tau(const ogs_assembly_params* p, int dim, const double* vel, const double* D, double L)
{
    const double v_mag = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    if (v_mag == 0.0) return 0.0;
    double diff;
    if (p->supg_diffusivity == 1)
    {
        diff = D[0];
        for (int i = 1; i < dim * dim; i++)
            if (D[i] < diff) diff = D[i];
    }
    else if (p->supg_diffusivity == 2)
    {
        double t = 0.0;
        for (int i = 0; i < dim; i++) t = D[i + i * dim] * D[i + i * dim];
        diff = sqrt(t);
    }
    else
    {
        diff = D[0];
        for (int i = 1; i < dim * dim; i++)
            if (D[i] > diff) diff = D[i];
    }
    double tau = 0.0;
    if (p->supg_method == 1)
    {
        const double alpha = 0.5 * v_mag * L / diff;
        tau = 0.5 * L / v_mag * langevin(alpha);
    }
    else if (p->supg_method == 2)
        tau = 1.0 / sqrt((2.0 / p->dt) * (2.0 / p->dt) + (2.0 * v_mag / L) * (2.0 * v_mag / L) +
                         (4.0 * diff / (L * L)) * (4.0 * diff / (L * L)));
    return tau;
}

/* Local matrices of one element:
 *   CalcMass (fem_ele_std.cpp:3753-3900) with CalCoefMass (:1569-1717),
 *   CalcLaplace (:4948-5070) with CalCoefLaplace (:2202-2384, :2545-2562),
 *   CalcAdvection (:5280-5470) with CalCoefAdvection (:3641-3646),
 *   CalcStorage (:4840-4890) with CalCoefStorage (:2071-2090),
 *   Assemble_Gravity (:5859-6000) for LIQUID_FLOW.
 * k_e: element conductivity / permeability (flow); vel: GP flux
 * [ngp][3] (transport).  Returns 0, or -1 on a singular Jacobian. */
int orc_element_matrices(int etype, int ngauss, int dim, const double* X,
                         const double* Y, const double* Z,
                         const ogs_assembly_params* p, double k_e,
                         const double* vel, orc_elem_mats* m)
{
    const int nn = orc_nodes_per_element(etype);
    double w[ORC_MAX_GP], N[ORC_MAX_GP * 8], dN[ORC_MAX_GP * 24];
    double w3[ORC_MAX_GP * 3];
    const int ngp = orc_shape_table(etype, ngauss, NULL, w, N, dN, w3);
    const int pcs = p->pcs_type;
    memset(m, 0, sizeof *m);

    /* material coefficients, constant over the element */
    double c_mass = 0.0, c_stor = 0.0;
    double mat[9] = {0};
    if (pcs == OGS_PCS_GROUNDWATER_FLOW)
    {
        c_mass = p->storage;
        for (int i = 0; i < dim; i++)
            mat[i * dim + i] = k_e * p->time_unit_factor * 1.0;
    }
    else if (pcs == OGS_PCS_LIQUID_FLOW)
    {
        c_mass = p->storage + p->porosity * p->drho_dp;
        double mat_fac = p->viscosity;
        if (p->gravity < DBL_EPSILON) mat_fac = 1.0;
        for (int i = 0; i < dim; i++)
            mat[i * dim + i] = p->time_unit_factor * k_e / mat_fac * 1.0 * 1.0;
    }
    else
    {
        c_mass = p->porosity * p->saturation * p->retardation;
        c_stor = p->porosity * p->saturation * p->decay * p->retardation;
    }
    /* only the transport assembly drops the mass matrix of a STEADY process
     * (fem_ele_std.cpp:8549); AssembleParabolicEquation has no such branch */
    if (p->steady && p->pcs_type == OGS_PCS_MASS_TRANSPORT) c_mass = 0.0;

    double X3[8], Y3[8], Z3[8];
    for (int i = 0; i < nn; i++)
    {
        X3[i] = X[i];
        Y3[i] = Y[i];
        Z3[i] = Z ? Z[i] : 0.0;
    }
    /* SUPG (transport): non-symmetric mass term kept apart from the
     * mirrored consistent mass */
    const int supg = pcs == OGS_PCS_MASS_TRANSPORT && p->supg_method > 0;
    double msupg[64] = {0};
    const double L_supg = supg ? orc_supg_length(etype, X3, Y3, Z3, p->supg_length) : 0.0;

    for (int gp = 0; gp < ngp; gp++)
    {
        double dNg[24], det;
        if (grad_global(dim, nn, X3, Y3, Z3, dN + gp * nn * dim, dNg, &det))
            return -1;
        /* GetGaussData: det * w_r (* w_s (* w_t)), left to right */
        const double fkt = etype == OGS_ELEM_HEX8
                               ? det * w3[gp * 3] * w3[gp * 3 + 1] * w3[gp * 3 + 2]
                           : etype == OGS_ELEM_QUAD4 ? det * w3[gp * 3] * w3[gp * 3 + 1]
                                                     : det * w3[gp * 3];
        const double* sf = N + gp * nn;
        /* mass, lower triangle (mirrored below) */
        if (c_mass != 0.0 || pcs == OGS_PCS_MASS_TRANSPORT)
        {
            const double mf = c_mass * fkt * 1.0;
            for (int i = 0; i < nn; i++)
                for (int j = 0; j <= i; j++)
                    m->mass[i * nn + j] += mf * sf[i] * sf[j];
        }
        /* Laplace / dispersion */
        double matg[9];
        if (pcs == OGS_PCS_MASS_TRANSPORT)
        {
            double v[3] = {vel[gp * 3 + 0], vel[gp * 3 + 1], vel[gp * 3 + 2]};
            double D[9];
            dispersion_tensor(dim, p, v, D);
            for (int i = 0; i < dim * dim; i++)
                matg[i] = D[i] * 1.0 * p->time_unit_factor;
        }
        else
            for (int i = 0; i < dim * dim; i++) matg[i] = mat[i];
        for (int i = 0; i < nn; i++)
            for (int j = 0; j < nn; j++)
                for (int k = 0; k < dim; k++)
                    for (int l = 0; l < dim; l++)
                        m->laplace[i * nn + j] += fkt * dNg[k * nn + i] *
                                                  matg[dim * k + l] *
                                                  dNg[l * nn + j];
        if (pcs == OGS_PCS_MASS_TRANSPORT)
        {
            const double mf = 1.0 * p->time_unit_factor;
            const double v[3] = {mf * vel[gp * 3 + 0], mf * vel[gp * 3 + 1],
                                 mf * vel[gp * 3 + 2]};
            for (int i = 0; i < nn; i++)
                for (int j = 0; j < nn; j++)
                    for (int k = 0; k < dim; k++)
                        m->advection[i * nn + j] +=
                            fkt * sf[i] * v[k] * dNg[k * nn + j];
            const double fs = fkt * c_stor;
            for (int i = 0; i < nn; i++)
                for (int j = 0; j < nn; j++)
                    m->storage[i * nn + j] += fs * sf[i] * sf[j];
        }
        if (supg)
        {
            /* CalcSUPGWeightingFunction (:4004-4025): w_i = v . grad N_i with the
             * raw Gauss-point flux; CalcMass SUPG term (:3856-3879) and
             * CalcAdvection SUPG term (:5467-5490) */
            double v[3] = {vel[gp * 3 + 0], vel[gp * 3 + 1], vel[gp * 3 + 2]};
            double D[9], wf[8];
            dispersion_tensor(dim, p, v, D);
            const double tau = supg_tau(p, dim, v, D, L_supg);
            for (int i = 0; i < nn; i++)
            {
                wf[i] = 0.0;
                for (int k = 0; k < dim; k++) wf[i] += dNg[k * nn + i] * v[k];
            }
            const double mat_fac = c_mass * fkt * 1.0;
            for (int i = 0; i < nn; i++)
                for (int j = 0; j < nn; j++)
                {
                    msupg[i * nn + j] += mat_fac * tau * wf[i] * sf[j];
                    m->advection[i * nn + j] += fkt * (1.0 * p->time_unit_factor) * tau * wf[i] * wf[j];
                }
        }
        if (pcs == OGS_PCS_LIQUID_FLOW && p->gravity_on)
        {
            double rho = p->density;
            if (p->gravity < DBL_EPSILON)
                rho = 1.0;
            else
                rho *= p->gravity;
            const double fg = fkt * rho;
            for (int i = 0; i < nn; i++)
                for (int k = 0; k < dim; k++)
                    m->rhs_gravity[i] -=
                        fg * dNg[k * nn + i] * matg[dim * k + dim - 1];
        }
    }
    for (int i = 0; i < nn; i++)
        for (int j = 0; j < nn; j++)
            if (i > j) m->mass[j * nn + i] = m->mass[i * nn + j];
    if (supg)
        for (int i = 0; i < nn * nn; i++) m->mass[i] += msupg[i];
    if (p->mass_lumping)
    {
        /* CalcLumpedMass (fem_ele_std.cpp:4598-4660): factor = CalCoefMass()
         * * ElementVolumeMultiplyer (1) * volume / nnodes on the diagonal */
        double factor = c_mass;
        factor *= 1.0;
        factor *= orc_element_volume(etype, X3, Y3, Z3) / (double)nn;
        for (int i = 0; i < nn * nn; i++) m->mass[i] = 0.0;
        for (int i = 0; i < nn; i++) m->mass[i * nn + i] = factor;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Sparse pattern                                                      */
/* ------------------------------------------------------------------ */

static int cmp_i64(const void* a, const void* b)
{
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

/* CFEMesh::ConnectedNodes (MSH/msh_mesh.cpp:2931-2980) + SparseTable CRS
 * (FEM/matrix_class.cpp:741-776): row i holds the sorted set of nodes that
 * share an element with node i (itself included).  row_ptr has n+1 entries;
 * col must hold the returned nnz (call once with col == NULL to count).
 * Returns nnz, or -1 on allocation failure. */
int64_t orc_build_pattern(int64_t n_nodes, int64_t n_elem, int nn,
                          const int32_t* conn, int64_t* row_ptr, int64_t* col)
{
    int64_t* deg = (int64_t*)calloc((size_t)n_nodes + 1, sizeof(int64_t));
    if (!deg) return -1;
    for (int64_t e = 0; e < n_elem; e++)
        for (int i = 0; i < nn; i++) deg[conn[e * nn + i]] += nn;
    int64_t* start = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n_nodes + 1));
    int64_t total = 0;
    for (int64_t i = 0; i < n_nodes; i++)
    {
        start[i] = total;
        total += deg[i];
    }
    start[n_nodes] = total;
    int64_t* buf = (int64_t*)malloc(sizeof(int64_t) * (size_t)(total + 1));
    int64_t* fill = (int64_t*)calloc((size_t)n_nodes, sizeof(int64_t));
    for (int64_t e = 0; e < n_elem; e++)
        for (int i = 0; i < nn; i++)
        {
            int64_t r = conn[e * nn + i];
            for (int j = 0; j < nn; j++)
                buf[start[r] + fill[r]++] = conn[e * nn + j];
        }
    int64_t nnz = 0;
    for (int64_t r = 0; r < n_nodes; r++)
    {
        int64_t* seg = buf + start[r];
        qsort(seg, (size_t)fill[r], sizeof(int64_t), cmp_i64);
        if (row_ptr) row_ptr[r] = nnz;
        for (int64_t k = 0; k < fill[r]; k++)
        {
            if (k > 0 && seg[k] == seg[k - 1]) continue;
            if (col) col[nnz] = seg[k];
            nnz++;
        }
    }
    if (row_ptr) row_ptr[n_nodes] = nnz;
    free(deg);
    free(start);
    free(buf);
    free(fill);
    return nnz;
}

/* binarySearch over a CRS row (Base/binarySearch.cpp via
 * CSparseMatrix::operator(), FEM/matrix_class.cpp:1222-1235). */
static int64_t csr_find(const int64_t* row_ptr, const int64_t* col, int64_t r,
                        int64_t c)
{
    int64_t lo = row_ptr[r], hi = row_ptr[r + 1] - 1;
    while (lo <= hi)
    {
        int64_t mid = (lo + hi) / 2;
        if (col[mid] == c) return mid;
        if (col[mid] < c)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

/* ------------------------------------------------------------------ */
/* Global assembly                                                     */
/* ------------------------------------------------------------------ */

/* CRFProcess::GlobalAssembly element loop (FEM/rf_pcs.cpp:5738-5757) with
 * CFiniteElementStd::Assembly (fem_ele_std.cpp:9367): per element the local
 * matrices, the LHS and RHS combination of AssembleParabolicEquation
 * (:7855-8121) or AssembleMixedHyperbolicParabolicEquation (:8592-8692),
 * and the scatter of add2GlobalMatrixII (:8328-8343).  Adds into val and b.
 * Returns 0, or -(1+e) when element e has a singular Jacobian. */
int64_t orc_assemble(int etype, int ngauss, int dim, int64_t n_nodes,
                     int64_t n_elem, const double* x, const double* y,
                     const double* z, const int32_t* conn,
                     const int64_t* row_ptr, const int64_t* col,
                     const ogs_assembly_params* p, const double* elem_k,
                     const double* u0, const double* gp_vel, double* val,
                     double* b)
{
    (void)n_nodes;
    const int nn = orc_nodes_per_element(etype);
    const int ngp = orc_num_gauss_points(etype, ngauss);
    const double dt_inverse = 1.0 / p->dt;
    orc_elem_mats m;
    for (int64_t e = 0; e < n_elem; e++)
    {
        double X[8], Y[8], Z[8], Sm[64], Rm[64], u[8], r[8];
        const int32_t* en = conn + e * nn;
        for (int i = 0; i < nn; i++)
        {
            X[i] = x[en[i]];
            Y[i] = y[en[i]];
            Z[i] = z ? z[en[i]] : 0.0;
            u[i] = u0 ? u0[en[i]] : 0.0;
        }
        const double ke = elem_k ? elem_k[e] : 0.0;
        const double* ve = gp_vel ? gp_vel + e * ngp * 3 : NULL;
        if (orc_element_matrices(etype, ngauss, dim, X, Y, z ? Z : NULL, p, ke,
                                 ve, &m))
            return -(1 + e);
        if (p->pcs_type == OGS_PCS_MASS_TRANSPORT)
        {
            const double th = p->theta;
            for (int k = 0; k < nn * nn; k++)
            {
                /* StiffMatrix = M/dt + th*L + th*A + th*S (:8603-8619) */
                double s = m.mass[k] * dt_inverse;
                s += m.laplace[k] * th;
                s += m.advection[k] * th;
                s += m.storage[k] * th;
                Sm[k] = s;
                /* AuxMatrix1 = M/dt - (1-th)(L + A + S) (:8651-8676) */
                double q = m.mass[k] * dt_inverse;
                q += m.laplace[k] * (-(1.0 - th));
                q += m.advection[k] * (-(1.0 - th));
                q += m.storage[k] * (-(1.0 - th));
                Rm[k] = q;
            }
        }
        else
        {
            double relax0 = p->nls_relaxation;
            if (relax0 < DBL_MIN) relax0 = 1.0;
            const double relax1 = 1.0 - relax0;
            for (int k = 0; k < nn * nn; k++)
            {
                /* StiffMatrix = M*fac1 + L*fac2 (:7855-7880) */
                Sm[k] = m.mass[k] * dt_inverse + m.laplace[k] * relax0;
                /* AuxMatrix1 = M*fac1 - L*relax1 (:7975-7998) */
                Rm[k] = m.mass[k] * dt_inverse - m.laplace[k] * relax1;
            }
        }
        /* Matrix::multi(NodalVal0, NodalVal) (matrix_class.cpp) */
        for (int i = 0; i < nn; i++)
        {
            double s = 0.0;
            for (int j = 0; j < nn; j++) s += Rm[i * nn + j] * u[j];
            r[i] = s;
        }
        for (int i = 0; i < nn; i++)
        {
            b[en[i]] += r[i];
            if (p->pcs_type == OGS_PCS_LIQUID_FLOW && p->gravity_on)
                b[en[i]] += m.rhs_gravity[i];
        }
        for (int i = 0; i < nn; i++)
            for (int j = 0; j < nn; j++)
            {
                int64_t k = csr_find(row_ptr, col, en[i], en[j]);
                val[k] += Sm[i * nn + j];
            }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* RICHARDS_FLOW                                                       */
/* ------------------------------------------------------------------ */

static double orc_mrange(double a, double b, double c)
{
    /* MRange (FEM/mathlib.cpp:447-455) */
    if (b < a) return a;
    if (b > c) return c;
    return b;
}

/* SaturationCapillaryPressureFunction, models 4 and 6
 * (FEM/rf_mmp_new.cpp:5243-5328) */
double orc_rich_saturation(const ogs_richards_params* r, double pc)
{
    double se, sl;
    if (r->capillary_model == 4)
    {
        if (pc < 0.0) pc = 0.0;
        se = pow(pc / r->pb, 1.0 / (1.0 - r->m)) + 1.0;
        se = pow(se, -r->m);
    }
    else
    {
        if (pc < r->pb) pc = r->pb;
        se = pow(pc / r->pb, -r->m);
    }
    sl = se * (r->slm - r->slr) + r->slr;
    return orc_mrange(r->slr + DBL_EPSILON, sl, r->slm - DBL_EPSILON);
}

/* PressureSaturationDependency(Sw, invert = true) = dSw/dPc
 * (FEM/rf_mmp_new.cpp:5425-5520) */
double orc_rich_dsdpc(const ogs_richards_params* r, double sl)
{
    double dpds, v1, v2, dsdp;
    if (r->capillary_model == 4)
    {
        sl = orc_mrange(r->slr + DBL_EPSILON, sl, r->slm - DBL_EPSILON);
        v1 = pow((sl - r->slr) / (r->slm - r->slr), -1.0 / r->m);
        v2 = pow(v1 - 1.0, -r->m);
        dpds = (r->pb * (r->m - 1.0) * v1 * v2) / (r->m * (sl - r->slr));
    }
    else
    {
        sl = orc_mrange(r->slr + DBL_EPSILON, sl, r->slm);
        v1 = pow((sl - r->slr) / (r->slm - r->slr), -1.0 / r->m);
        dpds = (r->pb * v1) / (r->m * (r->slr - sl));
    }
    dsdp = 1.0 / dpds;
    if (dsdp < (-1.0) / DBL_EPSILON) dsdp = (-1.0) / DBL_EPSILON;
    return dsdp;
}

/* PermeabilitySaturationFunction(Sw, 0), models 4 and 6
 * (FEM/rf_mmp_new.cpp:2576-2635) */
double orc_rich_krel(const ogs_richards_params* r, double sl)
{
    double se, kr;
    sl = orc_mrange(r->kr_slr, sl, r->kr_slm);
    se = (sl - r->kr_slr) / (r->kr_slm - r->kr_slr);
    if (r->permeability_model == 4)
        kr = sqrt(se) * pow(1.0 - pow(1.0 - pow(se, 1.0 / r->kr_m), r->kr_m), 2);
    else
        kr = pow(se, 3.0 + 2.0 / r->kr_m);
    if (kr < r->kr_min) kr = r->kr_min;
    return kr;
}

/* CalCoefMass, EPT_RICHARDS_FLOW (fem_ele_std.cpp:1721-1770) */
double orc_rich_mass_coef(const ogs_assembly_params* p, const ogs_richards_params* r, double PG)
{
    double Sw = 1.0, dSdp = 0.0, val;
    if (PG < 0.0)
    {
        Sw = orc_rich_saturation(r, -PG);
        dSdp = -orc_rich_dsdpc(r, Sw);
    }
    val = p->storage * Sw;
    if (p->density > 0.0) val += p->porosity * Sw * p->drho_dp;
    if (PG < 0.0) val += p->porosity * dSdp;
    return val;
}

/* CalCoefLaplace, EPT_RICHARDS_FLOW (fem_ele_std.cpp:2614-2640) */
double orc_rich_lap_coef(const ogs_assembly_params* p, const ogs_richards_params* r, double k, double PG)
{
    const double Sw = orc_rich_saturation(r, -PG);
    const double mat_fac = p->time_unit_factor * orc_rich_krel(r, Sw) / p->viscosity;
    return k * mat_fac * 1.0;
}

/* Element matrices of RICHARDS_FLOW at the nodal iterate u1: CalcMass /
 * CalcLumpedMass, CalcLaplace and Assemble_Gravity with the coefficients at
 * each Gauss point (the lumped storage at the element centre). */
int orc_element_matrices_richards(int etype, int ngauss, int dim, const double* X, const double* Y,
                                  const double* Z, const ogs_assembly_params* p,
                                  const ogs_richards_params* r, double k_e, const double* u1,
                                  orc_elem_mats* m)
{
    const int nn = orc_nodes_per_element(etype);
    double w[ORC_MAX_GP], N[ORC_MAX_GP * 8], dN[ORC_MAX_GP * 24];
    double w3[ORC_MAX_GP * 3];
    const int ngp = orc_shape_table(etype, ngauss, NULL, w, N, dN, w3);
    double X3[8], Y3[8], Z3[8];
    memset(m, 0, sizeof *m);
    for (int i = 0; i < nn; i++)
    {
        X3[i] = X[i];
        Y3[i] = Y[i];
        Z3[i] = Z ? Z[i] : 0.0;
    }
    for (int gp = 0; gp < ngp; gp++)
    {
        double dNg[24], det, PG = 0.0;
        if (grad_global(dim, nn, X3, Y3, Z3, dN + gp * nn * dim, dNg, &det)) return -1;
        const double fkt = etype == OGS_ELEM_HEX8
                               ? det * w3[gp * 3] * w3[gp * 3 + 1] * w3[gp * 3 + 2]
                           : etype == OGS_ELEM_QUAD4 ? det * w3[gp * 3] * w3[gp * 3 + 1]
                                                     : det * w3[gp * 3];
        const double* sf = N + gp * nn;
        for (int i = 0; i < nn; i++) PG += u1[i] * sf[i]; /* interpolate(NodalVal1) */
        const double mat = orc_rich_lap_coef(p, r, k_e, PG);
        const double mf = orc_rich_mass_coef(p, r, PG) * fkt * 1.0;
        for (int i = 0; i < nn; i++)
            for (int j = 0; j <= i; j++) m->mass[i * nn + j] += mf * sf[i] * sf[j];
        for (int i = 0; i < nn; i++)
            for (int j = 0; j < nn; j++)
                for (int k = 0; k < dim; k++)
                    m->laplace[i * nn + j] += fkt * dNg[k * nn + i] * mat * dNg[k * nn + j];
        if (p->gravity_on)
        {
            /* Assemble_Gravity (fem_ele_std.cpp:5859-6000) */
            double rho = p->density;
            if (p->gravity < DBL_EPSILON)
                rho = 1.0;
            else
                rho *= p->gravity;
            const double fg = fkt * rho;
            for (int i = 0; i < nn; i++) m->rhs_gravity[i] -= fg * dNg[(dim - 1) * nn + i] * mat;
        }
    }
    for (int i = 0; i < nn; i++)
        for (int j = 0; j < nn; j++)
            if (i > j) m->mass[j * nn + i] = m->mass[i * nn + j];
    if (p->mass_lumping)
    {
        double PG = 0.0, factor;
        for (int i = 0; i < nn; i++) PG += u1[i] * (1.0 / nn);
        factor = orc_rich_mass_coef(p, r, PG);
        factor *= 1.0;
        factor *= orc_element_volume(etype, X3, Y3, Z3) / (double)nn;
        for (int i = 0; i < nn * nn; i++) m->mass[i] = 0.0;
        for (int i = 0; i < nn; i++) m->mass[i * nn + i] = factor;
    }
    return 0;
}

/* RICHARDS_FLOW global assembly (AssembleParabolicEquation + Assemble_Gravity,
 * fem_ele_std.cpp:7702-8120, 5859-6000): A += M/dt + relax0 L,
 * b += (M/dt - relax1 L) u0 + gravity, coefficients at u1. */
int64_t orc_assemble_richards(int etype, int ngauss, int dim, int64_t n_elem, const double* x, const double* y,
                              const double* z, const int32_t* conn, const int64_t* row_ptr, const int64_t* col,
                              const ogs_assembly_params* p, const ogs_richards_params* r, const double* elem_k,
                              const double* u0, const double* u1, double* val, double* b)
{
    const int nn = orc_nodes_per_element(etype);
    const double dt_inverse = 1.0 / p->dt;
    double relax0 = p->nls_relaxation;
    if (relax0 < DBL_MIN) relax0 = 1.0;
    const double relax1 = 1.0 - relax0;
    orc_elem_mats m;
    for (int64_t e = 0; e < n_elem; e++)
    {
        double X[8], Y[8], Z[8], Sm[64], Rm[64], u[8], v1[8];
        const int32_t* en = conn + e * nn;
        for (int i = 0; i < nn; i++)
        {
            X[i] = x[en[i]];
            Y[i] = y[en[i]];
            Z[i] = z ? z[en[i]] : 0.0;
            u[i] = u0 ? u0[en[i]] : 0.0;
            v1[i] = u1[en[i]];
        }
        if (orc_element_matrices_richards(etype, ngauss, dim, X, Y, z ? Z : NULL, p, r, elem_k[e], v1, &m))
            return -(1 + e);
        for (int k = 0; k < nn * nn; k++)
        {
            Sm[k] = m.mass[k] * dt_inverse + m.laplace[k] * relax0;
            Rm[k] = m.mass[k] * dt_inverse - m.laplace[k] * relax1;
        }
        for (int i = 0; i < nn; i++)
        {
            double s = 0.0;
            for (int j = 0; j < nn; j++) s += Rm[i * nn + j] * u[j];
            b[en[i]] += s;
            if (p->gravity_on) b[en[i]] += m.rhs_gravity[i];
        }
        for (int i = 0; i < nn; i++)
            for (int j = 0; j < nn; j++) val[csr_find(row_ptr, col, en[i], en[j])] += Sm[i * nn + j];
    }
    return 0;
}

/* Cal_Velocity scalar branch (fem_ele_std.cpp:6627-6870): per GP
 * q_i = -sum_j mat[i][j] * vel[j] / time_unit_factor with vel = grad u
 * (plus rho*g on the last axis for LIQUID_FLOW with gravity).  Output
 * [e][gp][3], unused components zero.  Returns 0 or -(1+e). */
int64_t orc_gp_velocity(int etype, int ngauss, int dim, int64_t n_elem,
                        const double* x, const double* y, const double* z,
                        const int32_t* conn, const ogs_assembly_params* p,
                        const double* elem_k, const double* u, double* q)
{
    const int nn = orc_nodes_per_element(etype);
    double w[ORC_MAX_GP], N[ORC_MAX_GP * 8], dN[ORC_MAX_GP * 24];
    const int ngp = orc_shape_table(etype, ngauss, NULL, w, N, dN, NULL);
    for (int64_t e = 0; e < n_elem; e++)
    {
        double X[8], Y[8], Z[8], h[8];
        const int32_t* en = conn + e * nn;
        for (int i = 0; i < nn; i++)
        {
            X[i] = x[en[i]];
            Y[i] = y[en[i]];
            Z[i] = z ? z[en[i]] : 0.0;
            h[i] = u[en[i]];
        }
        double mat[9] = {0};
        const double ke = elem_k[e];
        if (p->pcs_type == OGS_PCS_LIQUID_FLOW)
        {
            double mat_fac = p->viscosity;
            if (p->gravity < DBL_EPSILON) mat_fac = 1.0;
            for (int i = 0; i < dim; i++)
                mat[i * dim + i] = p->time_unit_factor * ke / mat_fac * 1.0 * 1.0;
        }
        else
            for (int i = 0; i < dim; i++)
                mat[i * dim + i] = ke * p->time_unit_factor * 1.0;
        for (int gp = 0; gp < ngp; gp++)
        {
            double dNg[24], det;
            if (grad_global(dim, nn, X, Y, Z, dN + gp * nn * dim, dNg, &det))
                return -(1 + e);
            double vel[3] = {0, 0, 0};
            for (int i = 0; i < dim; i++)
            {
                vel[i] = 0.0;
                for (int j = 0; j < nn; j++) vel[i] += h[j] * dNg[i * nn + j];
            }
            if (p->pcs_type == OGS_PCS_LIQUID_FLOW && p->gravity_on &&
                p->gravity >= DBL_EPSILON)
                vel[dim - 1] += p->gravity * p->density;
            double* qo = q + (e * ngp + gp) * 3;
            qo[0] = qo[1] = qo[2] = 0.0;
            for (int i = 0; i < dim; i++)
                for (int j = 0; j < dim; j++)
                    qo[i] -= mat[dim * i + j] * vel[j] / p->time_unit_factor;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Dirichlet conditions                                                */
/* ------------------------------------------------------------------ */

/* CSparseMatrix::Diagonize, CRS branch without colDEBUG
 * (FEM/matrix_class.cpp:1663-1700,1783): zero row, keep diagonal,
 * b_i = a_ii * value. */
void orc_dirichlet_row_only(const int64_t* row_ptr, const int64_t* col,
                            double* val, double* b, int64_t n_bc,
                            const int64_t* rows, const double* vals)
{
    for (int64_t q = 0; q < n_bc; q++)
    {
        const int64_t id = rows[q];
        double vdiag = 0.0;
        for (int64_t k = row_ptr[id]; k < row_ptr[id + 1]; k++)
        {
            if (col[k] == id)
            {
                vdiag = val[k];
                continue;
            }
            val[k] = 0.0;
        }
        b[id] = vdiag * vals[q];
    }
}

/* MXRandbed (FEM/matrix_routines.cpp:2314-2520): column lifted into the
 * RHS, row and column zeroed, diagonal kept (a zero diagonal becomes
 * DBL_EPSILON), b_i = value * diag. */
void orc_dirichlet_symmetric(int64_t n, const int64_t* row_ptr,
                             const int64_t* col, double* val, double* b,
                             int64_t n_bc, const int64_t* rows,
                             const double* vals)
{
    for (int64_t q = 0; q < n_bc; q++)
    {
        const int64_t ir = rows[q];
        const double Ri = vals[q];
        int64_t kd = csr_find(row_ptr, col, ir, ir);
        double diag = kd >= 0 ? val[kd] : 0.0;
        if (fabs(diag) < DBL_MIN) diag = DBL_EPSILON;
        /* column ir of every other row: the pattern is structurally
         * symmetric, so the rows holding column ir are the columns of row ir */
        for (int64_t k = row_ptr[ir]; k < row_ptr[ir + 1]; k++)
        {
            const int64_t i = col[k];
            if (i == ir) continue;
            int64_t ki = csr_find(row_ptr, col, i, ir);
            if (ki >= 0)
            {
                b[i] -= val[ki] * Ri;
                val[ki] = 0.0;
            }
            val[k] = 0.0;
        }
        b[ir] = Ri * diag;
        if (kd >= 0) val[kd] = diag;
    }
    (void)n;
}

/* ------------------------------------------------------------------ */
/* Linear algebra (Linear_EQS semantics)                               */
/* ------------------------------------------------------------------ */

/* CSparseMatrix::multiVec, CRS, DOF = 1 (matrix_class.cpp:1520-1540). */
void orc_spmv(int64_t n, const int64_t* row_ptr, const int64_t* col,
              const double* val, const double* xv, double* yv)
{
    for (int64_t i = 0; i < n; i++) yv[i] = 0.0;
    for (int64_t ii = 0; ii < n; ii++)
        for (int64_t j = row_ptr[ii]; j < row_ptr[ii + 1]; j++)
            yv[ii] += val[j] * xv[col[j]];
}

/* Linear_EQS::dot (equation_class.cpp:981-995). */
static double dot(int64_t n, const double* a, const double* b)
{
    double v = 0.;
    for (int64_t i = 0; i < n; i++) v += a[i] * b[i];
    return v;
}

static double norm2(int64_t n, const double* a) { return sqrt(dot(n, a, a)); }

typedef struct
{
    int64_t n;
    const int64_t *row_ptr, *col;
    const double* val;
    int precond;
    const double* diag; /* Jacobi */
    const double* lu;   /* ILU(0) factors on the pattern */
    const int64_t* dpos;
} orc_op;

/* ILU(0) forward/backward solve on the CSR pattern: (LU) z = r with unit
 * lower L and upper U stored in place. */
static void ilu0_apply(const orc_op* op, const double* r, double* z)
{
    const int64_t n = op->n;
    for (int64_t i = 0; i < n; i++)
    {
        double s = r[i];
        for (int64_t k = op->row_ptr[i]; k < op->dpos[i]; k++)
            s -= op->lu[k] * z[op->col[k]];
        z[i] = s;
    }
    for (int64_t i = n - 1; i >= 0; i--)
    {
        double s = z[i];
        for (int64_t k = op->dpos[i] + 1; k < op->row_ptr[i + 1]; k++)
            s -= op->lu[k] * z[op->col[k]];
        z[i] = s / op->lu[op->dpos[i]];
    }
}

/* Linear_EQS::Precond (equation_class.cpp:935-963) with
 * CSparseMatrix::Precond_Jacobi (matrix_class.cpp:1805-1821). */
static void precond(const orc_op* op, const double* s, double* r)
{
    if (op->precond == OGS_PRECOND_JACOBI)
    {
        for (int64_t i = 0; i < op->n; i++)
        {
            double d = op->diag[i];
            if (fabs(d) < DBL_MIN) d = 1.0;
            r[i] = s[i] / d;
        }
    }
    else if (op->precond == OGS_PRECOND_ILU0)
        ilu0_apply(op, s, r);
    else
        for (int64_t i = 0; i < op->n; i++) r[i] = s[i];
}

/* ILU(0) factorisation (IKJ variant) on the CSR pattern; diagonal
 * positions in dpos.  Returns 0 or -1 on a zero pivot. */
int orc_ilu0_factor(int64_t n, const int64_t* row_ptr, const int64_t* col,
                    const double* val, double* lu, int64_t* dpos)
{
    memcpy(lu, val, sizeof(double) * (size_t)row_ptr[n]);
    for (int64_t i = 0; i < n; i++)
    {
        dpos[i] = csr_find(row_ptr, col, i, i);
        if (dpos[i] < 0) return -1;
    }
    for (int64_t i = 0; i < n; i++)
    {
        for (int64_t kk = row_ptr[i]; kk < dpos[i]; kk++)
        {
            const int64_t k = col[kk];
            const double piv = lu[dpos[k]];
            if (piv == 0.0) return -1;
            const double lik = lu[kk] / piv;
            lu[kk] = lik;
            /* row i -= lik * row k (upper part), on the pattern of row i */
            int64_t p = kk + 1;
            for (int64_t q = dpos[k] + 1; q < row_ptr[k + 1]; q++)
            {
                const int64_t j = col[q];
                while (p < row_ptr[i + 1] && col[p] < j) p++;
                if (p < row_ptr[i + 1] && col[p] == j) lu[p] -= lik * lu[q];
            }
        }
        if (lu[dpos[i]] == 0.0) return -1;
    }
    return 0;
}

typedef struct
{
    double b_norm;   /* carried across calls: Linear_EQS::bNorm */
    double error;
    int iter;
} orc_solver_state;

/* Linear_EQS::CheckNormRHS (equation_class.cpp:1104-1121). */
static int check_norm_rhs(orc_solver_state* st, double normb_new, double tol)
{
    if (st->b_norm > 0.0)
        if ((normb_new / st->b_norm) < tol)
        {
            st->error = normb_new / st->b_norm;
            st->b_norm = normb_new;
            return 1;
        }
    st->b_norm = normb_new;
    if (st->b_norm < DBL_MIN)
    {
        st->error = 0.;
        return 1;
    }
    return 0;
}

/* Linear_EQS::CG (equation_class.cpp:1129-1187).  Returns the iteration
 * count at exit (the reference returns iter <= max_iter). */
static int cg(const orc_op* op, const double* b, double* x, int max_iter,
              double tol, orc_solver_state* st)
{
    const int64_t n = op->n;
    double* p = (double*)malloc(sizeof(double) * (size_t)n);
    double* r = (double*)malloc(sizeof(double) * (size_t)n);
    double* s = (double*)malloc(sizeof(double) * (size_t)n);
    int iter = 0;
    if (check_norm_rhs(st, norm2(n, b), tol)) goto done;
    orc_spmv(n, op->row_ptr, op->col, op->val, x, s);
    for (int64_t i = 0; i < n; i++) r[i] = b[i] - s[i];
    precond(op, r, s);
    for (int64_t i = 0; i < n; i++) p[i] = s[i];
    if ((st->error = norm2(n, r) / st->b_norm) < tol) goto done;
    double rr = dot(n, r, s);
    for (iter = 1; iter <= max_iter; ++iter)
    {
        orc_spmv(n, op->row_ptr, op->col, op->val, p, s);
        const double alpha = rr / dot(n, p, s);
        for (int64_t i = 0; i < n; i++)
        {
            x[i] += alpha * p[i];
            r[i] -= alpha * s[i];
        }
        if ((st->error = norm2(n, r) / st->b_norm) < tol) goto done;
        precond(op, r, s);
        const double rrM1 = rr;
        rr = dot(n, s, r);
        const double beta = rr / rrM1;
        for (int64_t i = 0; i < n; i++) p[i] = s[i] + beta * p[i];
    }
    iter = max_iter;
done:
    free(p);
    free(r);
    free(s);
    return iter;
}

/* Linear_EQS::BiCGStab (equation_class.cpp:1287-1420).  Returns the
 * iteration count; *breakdown set when |rho| or |omega| < DBL_MIN ended it. */
static int bicgstab(const orc_op* op, const double* b, double* x, int max_iter,
                    double tol, orc_solver_state* st, int* breakdown)
{
    const int64_t n = op->n;
    double* buf = (double*)malloc(sizeof(double) * (size_t)n * 8);
    double *r0 = buf, *r = buf + n, *s = buf + 2 * n, *s_h = buf + 3 * n,
           *t = buf + 4 * n, *v = buf + 5 * n, *p = buf + 6 * n,
           *p_h = buf + 7 * n;
    double rho_0 = 1.0, rho_1, alpha = 1.0, beta, omega = 1.0, tt, norm_r;
    int iter = 0;
    *breakdown = 0;
    if (check_norm_rhs(st, norm2(n, b), tol)) goto done;
    orc_spmv(n, op->row_ptr, op->col, op->val, x, s);
    for (int64_t i = 0; i < n; i++) r0[i] = b[i] - s[i];
    for (int64_t i = 0; i < n; i++)
    {
        r[i] = r0[i];
        v[i] = 0.;
        p[i] = 0.;
    }
    if ((st->error = norm2(n, r) / st->b_norm) < tol) goto done;
    for (iter = 1; iter <= max_iter; iter++)
    {
        rho_1 = dot(n, r0, r);
        if (fabs(rho_1) < DBL_MIN)
        {
            *breakdown = 1;
            goto done;
        }
        if (iter == 1)
            for (int64_t i = 0; i < n; i++) p[i] = r[i];
        else
        {
            beta = (rho_1 / rho_0) * (alpha / omega);
            for (int64_t i = 0; i < n; i++)
                p[i] = r[i] + beta * (p[i] - omega * v[i]);
        }
        precond(op, p, p_h);
        orc_spmv(n, op->row_ptr, op->col, op->val, p_h, v);
        alpha = rho_1 / dot(n, r0, v);
        for (int64_t i = 0; i < n; i++) s[i] = r[i] - alpha * v[i];
        if ((st->error = norm2(n, s) / st->b_norm) < tol)
        {
            for (int64_t i = 0; i < n; i++) x[i] += alpha * p_h[i];
            goto done;
        }
        precond(op, s, s_h);
        orc_spmv(n, op->row_ptr, op->col, op->val, s_h, t);
        tt = dot(n, t, t);
        if (tt > DBL_MIN)
            omega = dot(n, t, s) / tt;
        else
            omega = 1.0;
        for (int64_t i = 0; i < n; i++)
        {
            x[i] += alpha * p_h[i] + omega * s_h[i];
            r[i] = s[i] - omega * t[i];
        }
        rho_0 = rho_1;
        norm_r = norm2(n, r);
        if ((st->error = norm_r / st->b_norm) < tol) goto done;
        if (fabs(omega) < DBL_MIN)
        {
            st->error = norm_r / st->b_norm;
            *breakdown = 1;
            goto done;
        }
    }
    iter = max_iter;
done:
    free(buf);
    return iter;
}

/* Linear_EQS::Solver (equation_class.cpp:857-895) for CG / BiCGStab with
 * no, Jacobi or ILU(0) preconditioning.  b_norm_io carries
 * Linear_EQS::bNorm between calls (1.0 for a fresh system, as the
 * Linear_EQS constructor sets it; NULL means a fresh system).
 * out[0] = iterations, out[1] = relative residual, out[2] = |b|,
 * out[3] = 1 on breakdown.  Returns 0, or -1 on bad input / zero pivot. */
int orc_solve(int64_t n, const int64_t* row_ptr, const int64_t* col,
              const double* val, const double* b, double* x, int method,
              int precond_type, int max_iter, double tol, double* b_norm_io,
              double* out)
{
    orc_op op;
    memset(&op, 0, sizeof op);
    op.n = n;
    op.row_ptr = row_ptr;
    op.col = col;
    op.val = val;
    op.precond = precond_type;
    double* diag = NULL;
    double* lu = NULL;
    int64_t* dpos = NULL;
    if (precond_type == OGS_PRECOND_JACOBI)
    {
        diag = (double*)malloc(sizeof(double) * (size_t)n);
        for (int64_t i = 0; i < n; i++)
        {
            int64_t k = csr_find(row_ptr, col, i, i);
            diag[i] = k >= 0 ? val[k] : 0.0;
        }
        op.diag = diag;
    }
    else if (precond_type == OGS_PRECOND_ILU0)
    {
        lu = (double*)malloc(sizeof(double) * (size_t)row_ptr[n]);
        dpos = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
        if (orc_ilu0_factor(n, row_ptr, col, val, lu, dpos))
        {
            free(lu);
            free(dpos);
            return -1;
        }
        op.lu = lu;
        op.dpos = dpos;
    }
    orc_solver_state st;
    /* Linear_EQS ctor sets bNorm = 1.0 (equation_class.cpp:131) */
    st.b_norm = b_norm_io ? *b_norm_io : 1.0;
    st.error = 1.0e10;
    int breakdown = 0, iters;
    if (method == OGS_LS_CG)
        iters = cg(&op, b, x, max_iter, tol, &st);
    else if (method == OGS_LS_BICGSTAB)
        iters = bicgstab(&op, b, x, max_iter, tol, &st, &breakdown);
    else
    {
        free(diag);
        free(lu);
        free(dpos);
        return -1;
    }
    if (b_norm_io) *b_norm_io = st.b_norm;
    out[0] = iters;
    out[1] = st.error;
    out[2] = st.b_norm;
    out[3] = breakdown;
    free(diag);
    free(lu);
    free(dpos);
    return 0;
}
