// assembly.cu -- element-per-thread global assembly and Gauss-point flux.
//
// One thread per element.  The element loop of CRFProcess::GlobalAssembly
// (FEM/rf_pcs.cpp:5738-5757) with CFiniteElementStd::Assembly
// (FEM/fem_ele_std.cpp:9367) becomes one launch: each thread gathers its
// node coordinates and primary variable, forms the local matrices in
// registers, combines them into the LHS and RHS exactly as
// AssembleParabolicEquation (fem_ele_std.cpp:7702-8126) or
// AssembleMixedHyperbolicParabolicEquation (:8504-8735) does, and scatters
// with FP64 atomics through the precomputed CSR slot map (no colouring).
//
// Two element paths:
//  * general -- per Gauss point Jacobian, inverse and global gradients,
//    CElement::computeJacobian / ComputeGradShapefct (FEM/fem_ele.cpp:585,
//    1128), then CalcMass / CalcLaplace / CalcAdvection / CalcStorage in
//    the reference's summation order;
//  * affine  -- elements with a constant Jacobian (every tet, parallelogram
//    quads, parallelepiped hexes): Laplace_ij = |J| sum_ab C_ab Q_abij and
//    Mass_ij = c |J| M0_ij with reference tensors Q, M0 summed once over
//    the Gauss points.  Mathematically identical, ~25x fewer FP64 FMAs on
//    hexes, which matters on a part with 1.2 TFLOP/s of FP64.
// Tables (N, dN/dxi, weights; Q, M0) are staged in shared memory per block.
#include <cfloat>
#include <cstdio>

#include "common.cuh"

namespace ogs {

template <int ET> struct ElemTraits;
template <> struct ElemTraits<OGS_ELEM_QUAD4> { static constexpr int NN = 4, DIM = 2; };
template <> struct ElemTraits<OGS_ELEM_HEX8> { static constexpr int NN = 8, DIM = 3; };
template <> struct ElemTraits<OGS_ELEM_TET4> { static constexpr int NN = 4, DIM = 3; };

// Jacobian (row = local direction), |det| and the inverse, as
// CElement::computeJacobian.  Returns false on |det| < DBL_EPSILON.
template <int NN, int DIM>
__device__ __forceinline__ bool jacobian(const double* X, const double* Y,
                                         const double* Z, const double* dN,
                                         double* iJ, double& det)
{
    double J[DIM * DIM];
#pragma unroll
    for (int k = 0; k < DIM * DIM; k++) J[k] = 0.0;
    if (DIM == 2)
    {
#pragma unroll
        for (int i = 0; i < NN; i++)
        {
            J[0] += X[i] * dN[i];
            J[1] += Y[i] * dN[i];
            J[2] += X[i] * dN[NN + i];
            J[3] += Y[i] * dN[NN + i];
        }
        det = J[0] * J[3] - J[1] * J[2];
        if (fabs(det) < DBL_EPSILON) return false;
        // one FP64 division (the cofactors times 1/det; the reference divides
        // each, the results differ by rounding only)
        const double id = 1.0 / det;
        iJ[0] = J[3] * id;
        iJ[1] = -J[1] * id;
        iJ[2] = -J[2] * id;
        iJ[3] = J[0] * id;
    }
    else
    {
#pragma unroll
        for (int i = 0; i < NN; i++)
        {
            J[0] += X[i] * dN[i];
            J[1] += Y[i] * dN[i];
            J[2] += Z[i] * dN[i];
            J[3] += X[i] * dN[NN + i];
            J[4] += Y[i] * dN[NN + i];
            J[5] += Z[i] * dN[NN + i];
            J[6] += X[i] * dN[2 * NN + i];
            J[7] += Y[i] * dN[2 * NN + i];
            J[8] += Z[i] * dN[2 * NN + i];
        }
        det = J[0] * (J[4] * J[8] - J[7] * J[5]) + J[6] * (J[1] * J[5] - J[4] * J[2]) +
              J[3] * (J[2] * J[7] - J[8] * J[1]);
        if (fabs(det) < DBL_EPSILON) return false;
        const double id = 1.0 / det;
        iJ[0] = (J[4] * J[8] - J[7] * J[5]) * id;
        iJ[1] = (J[2] * J[7] - J[1] * J[8]) * id;
        iJ[2] = (J[1] * J[5] - J[2] * J[4]) * id;
        iJ[3] = (J[5] * J[6] - J[8] * J[3]) * id;
        iJ[4] = (J[0] * J[8] - J[6] * J[2]) * id;
        iJ[5] = (J[2] * J[3] - J[5] * J[0]) * id;
        iJ[6] = (J[3] * J[7] - J[6] * J[4]) * id;
        iJ[7] = (J[1] * J[6] - J[7] * J[0]) * id;
        iJ[8] = (J[0] * J[4] - J[3] * J[1]) * id;
    }
    det = fabs(det);
    return true;
}

// global gradients dNg[j*NN+i] = sum_k iJ[j*DIM+k] dN[k*NN+i]
template <int NN, int DIM>
__device__ __forceinline__ void grad_global(const double* iJ, const double* dN, double* dNg)
{
#pragma unroll
    for (int i = 0; i < NN; i++)
#pragma unroll
        for (int j = 0; j < DIM; j++)
        {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < DIM; k++) s += iJ[j * DIM + k] * dN[k * NN + i];
            dNg[j * NN + i] = s;
        }
}

// MassDispersionTensorNew (FEM/rf_mmp_new.cpp:3090-3328), isotropic
// tortuosity: D = n S Daq tau I + alpha_T |q| I + (alpha_L - alpha_T) q q^T / |q|
template <int DIM>
__device__ __forceinline__ void dispersion_raw(const ogs_assembly_params& p, const double* v,
                                               double* D)
{
    const double dm = p.diffusion * p.porosity * p.saturation;
    const double vg = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
#pragma unroll
    for (int i = 0; i < DIM * DIM; i++) D[i] = 0.0;
    if (fabs(vg) > DBL_EPSILON)
    {
        // one division per point: (alpha_L - alpha_T) / |q| times q_i q_j
        // (the reference divides each entry; the results differ by rounding
        // only), the symmetric entries formed once
        const double al = p.alpha_l, at = p.alpha_t;
        const double c = (al - at) / vg;
#pragma unroll
        for (int i = 0; i < DIM; i++)
#pragma unroll
            for (int j = 0; j < i; j++) D[i * DIM + j] = D[j * DIM + i] = c * (v[i] * v[j]);
#pragma unroll
        for (int i = 0; i < DIM; i++) D[i * DIM + i] = (at * vg) + c * (v[i] * v[i]) + dm;
    }
    else
    {
#pragma unroll
        for (int i = 0; i < DIM; i++) D[i * DIM + i] = dm;
    }
}

template <int DIM>
__device__ __forceinline__ void dispersion(const ogs_assembly_params& p, const double* v, double* D)
{
    dispersion_raw<DIM>(p, v, D);
#pragma unroll
    for (int i = 0; i < DIM * DIM; i++) D[i] = D[i] * 1.0 * p.time_unit_factor;
}

// MLangevin (FEM/mathlib.cpp:3009-3021): coth(v) - 1/v, its series below 0.01
__device__ __forceinline__ double langevin(double v)
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

// CalcSUPGEffectiveElemenetLength (fem_ele_std.cpp:4034-4095) over the edges
// of CElem::GetLocalIndicesOfEdgeNodes (MSH/msh_elem.cpp:984-1052)
template <int ET>
__device__ __forceinline__ double supg_length(const double* X, const double* Y, const double* Z, int method)
{
    constexpr int NE = ET == OGS_ELEM_HEX8 ? 12 : ET == OGS_ELEM_QUAD4 ? 4 : 6;
    double len[NE];
#pragma unroll
    for (int e = 0; e < NE; e++)
    {
        int a, b;
        if (ET == OGS_ELEM_QUAD4) { a = e; b = (e + 1) % 4; }
        else if (ET == OGS_ELEM_HEX8)
        {
            if (e < 8) { a = e; b = (e + 1) % 4 + 4 * (e / 4); }
            else { a = e % 4; b = e % 4 + 4; }
        }
        else if (e < 3) { a = e; b = (e + 1) % 3; }
        else { a = 3; b = (e + 1) % 3; }
        const double dx = X[b] - X[a], dy = Y[b] - Y[a], dz = Z[b] - Z[a];
        len[e] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    double L = 0.0;
    if (method == 1)
    {
        double mn = len[0];
#pragma unroll
        for (int e = 1; e < NE; e++) { L = len[e]; if (L < mn) mn = L; }
        L = mn;
    }
    else if (method == 2)
    {
        double t = 0.0;
#pragma unroll
        for (int e = 1; e < NE; e++) t += len[e];  // the reference starts at edge 1
        L = t / NE;
    }
    else
    {
        double mx = len[0];
#pragma unroll
        for (int e = 1; e < NE; e++) { L = len[e]; if (L > mx) mx = L; }
        L = mx;
    }
    return L;
}

// CalcSUPGCoefficient (fem_ele_std.cpp:3908-3995), MASS_TRANSPORT; D is the
// raw MassDispersionTensorNew of the Gauss point
template <int DIM>
__device__ __forceinline__ double supg_tau(const ogs_assembly_params& p, const double* vel, const double* D, double L)
{
    const double v_mag = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    if (v_mag == 0.0) return 0.0;
    double diff;
    if (p.supg_diffusivity == 1)
    {
        diff = D[0];
#pragma unroll
        for (int i = 1; i < DIM * DIM; i++)
            if (D[i] < diff) diff = D[i];
    }
    else if (p.supg_diffusivity == 2)
    {
        double t = 0.0;
#pragma unroll
        for (int i = 0; i < DIM; i++) t = D[i + i * DIM] * D[i + i * DIM];  // the reference assigns
        diff = sqrt(t);
    }
    else
    {
        diff = D[0];
#pragma unroll
        for (int i = 1; i < DIM * DIM; i++)
            if (D[i] > diff) diff = D[i];
    }
    double tau = 0.0;
    if (p.supg_method == 1)
    {
        const double alpha = 0.5 * v_mag * L / diff;
        tau = 0.5 * L / v_mag * langevin(alpha);
    }
    else if (p.supg_method == 2)
        tau = 1.0 / sqrt((2.0 / p.dt) * (2.0 / p.dt) + (2.0 * v_mag / L) * (2.0 * v_mag / L) +
                         (4.0 * diff / (L * L)) * (4.0 * diff / (L * L)));
    return tau;
}

// flow coefficient of the Laplace term: CalCoefLaplace GWF (:2308-2384,
// mat = K * time_unit_factor * k_rel) or LIQUID_FLOW (:2232-2306,
// mat = time_unit_factor * k / mu, mu -> 1 in the HEAD form)
__device__ __forceinline__ double flow_mat(const ogs_assembly_params& p, double k)
{
    if (p.pcs_type == OGS_PCS_LIQUID_FLOW)
    {
        double mat_fac = p.viscosity;
        if (p.gravity < DBL_EPSILON) mat_fac = 1.0;
        return p.time_unit_factor * k / mat_fac * 1.0 * 1.0;
    }
    return k * p.time_unit_factor * 1.0;
}

// CElem::calcVolume (MSH/msh_elem.cpp:1511-1576) with ComputeDetTri /
// ComputeDetTex (FEM/mathlib.cpp:2911-2955): quads as two triangles,
// hexahedra as six tetrahedra in the mesh's node order
__device__ __forceinline__ double vol_tri(const double* X, const double* Y, const double* Z, int a, int b, int c)
{
    const double u0 = X[c] - X[a], u1 = Y[c] - Y[a], u2 = Z[c] - Z[a];
    const double v0 = X[b] - X[a], v1 = Y[b] - Y[a], v2 = Z[b] - Z[a];
    const double z0 = u1 * v2 - u2 * v1, z1 = u2 * v0 - u0 * v2, z2 = u0 * v1 - u1 * v0;
    return 0.5 * sqrt(z0 * z0 + z1 * z1 + z2 * z2);
}

__device__ __forceinline__ double vol_tet(const double* X, const double* Y, const double* Z, int a, int b, int c,
                                          int d)
{
    const double ax = X[a] - X[d], ay = Y[a] - Y[d], az = Z[a] - Z[d];
    const double bx = X[b] - X[d], by = Y[b] - Y[d], bz = Z[b] - Z[d];
    const double cx = X[c] - X[d], cy = Y[c] - Y[d], cz = Z[c] - Z[d];
    return fabs(ax * (by * cz - bz * cy) - ay * (bx * cz - bz * cx) + az * (bx * cy - by * cx)) / 6.0;
}

template <int ET>
__device__ __forceinline__ double element_volume(const double* X, const double* Y, const double* Z)
{
    if (ET == OGS_ELEM_QUAD4) return vol_tri(X, Y, Z, 0, 1, 2) + vol_tri(X, Y, Z, 2, 3, 0);
    if (ET == OGS_ELEM_TET4) return vol_tet(X, Y, Z, 0, 1, 2, 3);
    double v = vol_tet(X, Y, Z, 4, 7, 5, 0);
    v += vol_tet(X, Y, Z, 5, 3, 1, 0);
    v += vol_tet(X, Y, Z, 5, 7, 3, 0);
    v += vol_tet(X, Y, Z, 5, 7, 6, 2);
    v += vol_tet(X, Y, Z, 1, 3, 5, 2);
    v += vol_tet(X, Y, Z, 3, 7, 5, 2);
    return v;
}

// CalcLumpedMass (fem_ele_std.cpp:4598-4660), selected by
// m_num->ele_mass_lumping: the packed lower-triangle mass becomes
// diag(CalCoefMass * ElementVolumeMultiplyer (1) * volume / nnodes)
template <int ET, int NN>
__device__ __forceinline__ void lump_mass(const double* X, const double* Y, const double* Z, double cm, double* Ml)
{
    double f = cm;
    f *= 1.0;
    f *= element_volume<ET>(X, Y, Z) / (double)NN;
#pragma unroll
    for (int i = 0; i < NN; i++)
#pragma unroll
        for (int j = 0; j <= i; j++) Ml[i * (i + 1) / 2 + j] = i == j ? f : 0.0;
}

// CalCoefMass for GWF (StorageFunction) and LIQUID_FLOW (Ss + n drho/dp).
// AssembleParabolicEquation (fem_ele_std.cpp:7702-8126) has no steady branch:
// a STEADY flow process keeps M/dt, so p.steady is not read here.
__device__ __forceinline__ double flow_mass_coef(const ogs_assembly_params& p)
{
    if (p.pcs_type == OGS_PCS_LIQUID_FLOW) return p.storage + p.porosity * p.drho_dp;
    return p.storage;
}

__device__ __forceinline__ void flag_bad(int* bad, int64_t e)
{
    atomicMin(bad, (int)(e + 1));
}

// stage a table block into shared memory
__device__ __forceinline__ void stage(double* dst, const double* src, int n)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

template <int NN>
__device__ __forceinline__ void gather(const AsmArgs& a, int64_t e, int* nd, double* X,
                                       double* Y, double* Z, double* U)
{
    const int64_t E = a.E;
#pragma unroll
    for (int i = 0; i < NN; i++)
    {
        nd[i] = __ldg(a.conn_t + (int64_t)i * E + e);
        if (!OGS_IN(nd[i], a.nrows, kOobAsmNode)) nd[i] = 0;
    }
#pragma unroll
    for (int i = 0; i < NN; i++)
    {
        X[i] = __ldg(a.x + nd[i]);
        Y[i] = __ldg(a.y + nd[i]);
        Z[i] = __ldg(a.z + nd[i]);
        U[i] = a.u0 ? __ldg(a.u0 + nd[i]) : 0.0;
    }
}

template <int NN>
__device__ __forceinline__ void scatter(const AsmArgs& a, int64_t e, const int* nd,
                                        const double* S, const double* r)
{
    const int64_t E = a.E;
#pragma unroll
    for (int i = 0; i < NN; i++)
    {
#pragma unroll
        for (int j = 0; j < NN; j++)
        {
            const int32_t k = __ldg(a.slot_t + (int64_t)(i * NN + j) * E + e);
            if (OGS_IN(k, a.nslots, kOobAsmSlot)) atomicAdd(a.val + k, S[i * NN + j]);
        }
        atomicAdd(a.b + nd[i], r[i]);
    }
}

// ------------------------------------------------------------------
// flow: GROUNDWATER_FLOW / LIQUID_FLOW
// ------------------------------------------------------------------
template <int NN>
__device__ __forceinline__ void flow_combine(const AsmArgs& a, int64_t e, const int* nd,
                                             const double* U, const double* Ml,
                                             const double* Ll, const double* grav)
{
    // AssembleParabolicEquation: fac1 = 1/dt, fac2 = relax0; RHS with relax1
    const double dt_inverse = 1.0 / a.p.dt;
    double relax0 = a.p.nls_relaxation;
    if (relax0 < DBL_MIN) relax0 = 1.0;
    const double relax1 = 1.0 - relax0;
    // the element matrices are symmetric: each distinct entry of the LHS
    // and of the RHS operator is formed once (the same expressions as per
    // (i, j), so the values are the same bit for bit)
    constexpr int NL = NN * (NN + 1) / 2;
    double Sl[NL], Tl[NL];
#pragma unroll
    for (int l = 0; l < NL; l++)
    {
        const double m = Ml[l], lp = Ll[l];
        Sl[l] = m * dt_inverse + lp * relax0;
        Tl[l] = m * dt_inverse - lp * relax1;
    }
    double S[NN * NN], r[NN];
#pragma unroll
    for (int i = 0; i < NN; i++) r[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NN; i++)
#pragma unroll
        for (int j = 0; j < NN; j++)
        {
            const int l = i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
            S[i * NN + j] = Sl[l];
            r[i] += Tl[l] * U[j];
        }
    if ((a.p.pcs_type == OGS_PCS_LIQUID_FLOW || a.p.pcs_type == OGS_PCS_RICHARDS_FLOW) && a.p.gravity_on)
#pragma unroll
        for (int i = 0; i < NN; i++) r[i] += grav[i];
    scatter<NN>(a, e, nd, S, r);
}

template <int ET, int NGP>
__global__ void __launch_bounds__(128) k_flow_general(AsmArgs a)
{
    constexpr int NN = ElemTraits<ET>::NN, DIM = ElemTraits<ET>::DIM;
    __shared__ double sN[NGP * NN], sdN[NGP * NN * DIM], sw[NGP * 3];
    stage(sN, a.tab, NGP * NN);
    stage(sdN, a.tab + NGP * NN, NGP * NN * DIM);
    stage(sw, a.tab + NGP * NN + NGP * NN * DIM, NGP * 3);
    __syncthreads();
    const double cm = flow_mass_coef(a.p);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.E;
         e += (int64_t)gridDim.x * blockDim.x)
    {
        int nd[NN];
        double X[NN], Y[NN], Z[NN], U[NN];
        gather<NN>(a, e, nd, X, Y, Z, U);
        const double mat = flow_mat(a.p, __ldg(a.elem_k + e));
        double Ml[NN * (NN + 1) / 2], Ll[NN * (NN + 1) / 2], grav[NN];
#pragma unroll
        for (int l = 0; l < NN * (NN + 1) / 2; l++) Ml[l] = Ll[l] = 0.0;
#pragma unroll
        for (int i = 0; i < NN; i++) grav[i] = 0.0;
        bool ok = true;
#pragma unroll 1
        for (int gp = 0; gp < NGP; gp++)
        {
            double iJ[DIM * DIM], det, dNg[DIM * NN];
            if (!jacobian<NN, DIM>(X, Y, Z, sdN + gp * NN * DIM, iJ, det)) { ok = false; break; }
            grad_global<NN, DIM>(iJ, sdN + gp * NN * DIM, dNg);
            const double* w = sw + gp * 3;
            const double fkt = ET == OGS_ELEM_HEX8 ? det * w[0] * w[1] * w[2]
                             : ET == OGS_ELEM_QUAD4 ? det * w[0] * w[1] : det * w[0];
            const double* sf = sN + gp * NN;
            const double mf = cm * fkt * 1.0;
            const double cl = fkt * mat;  // the Gauss-point factors hoisted
#pragma unroll
            for (int i = 0; i < NN; i++)
            {
                const double mi = mf * sf[i];
#pragma unroll
                for (int j = 0; j <= i; j++)
                {
                    const int l = i * (i + 1) / 2 + j;
                    Ml[l] += mi * sf[j];
                    double g = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; k++) g += dNg[k * NN + i] * dNg[k * NN + j];
                    Ll[l] += cl * g;
                }
            }
            if (a.p.pcs_type == OGS_PCS_LIQUID_FLOW && a.p.gravity_on)
            {
                const double rho = a.p.gravity < DBL_EPSILON ? 1.0 : a.p.density * a.p.gravity;
                const double fg = fkt * rho;
#pragma unroll
                for (int i = 0; i < NN; i++) grav[i] -= fg * dNg[(DIM - 1) * NN + i] * mat;
            }
        }
        if (!ok) { flag_bad(a.bad_elem, e); continue; }
        if (a.p.mass_lumping) lump_mass<ET, NN>(X, Y, Z, cm, Ml);
        flow_combine<NN>(a, e, nd, U, Ml, Ll, grav);
    }
}

// affine flow: C = mat * iJ^T iJ (isotropic), Laplace = |J| sum_ab C_ab Q_ab
template <int ET>
__global__ void __launch_bounds__(128) k_flow_affine(AsmArgs a)
{
    constexpr int NN = ElemTraits<ET>::NN, DIM = ElemTraits<ET>::DIM;
    constexpr int NQ = DIM * DIM * NN * NN;
    __shared__ double sQ[NQ], sM0[NN * NN], sdNc[DIM * NN];
    stage(sQ, a.aff, NQ);
    stage(sM0, a.aff + NQ, NN * NN);
    stage(sdNc, a.aff + NQ + NN * NN, DIM * NN);
    __syncthreads();
    const double cm = flow_mass_coef(a.p);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.E;
         e += (int64_t)gridDim.x * blockDim.x)
    {
        int nd[NN];
        double X[NN], Y[NN], Z[NN], U[NN];
        gather<NN>(a, e, nd, X, Y, Z, U);
        const double mat = flow_mat(a.p, __ldg(a.elem_k + e));
        double iJ[DIM * DIM], det;
        if (!jacobian<NN, DIM>(X, Y, Z, sdNc, iJ, det)) { flag_bad(a.bad_elem, e); continue; }
        // axis-aligned boxes: the off-diagonal entries of J^-1, hence of C,
        // are exactly 0, and the sums over the DIM diagonal terms equal the
        // full sums bit for bit (the other terms add +-0)
        bool box = true;
#pragma unroll
        for (int p = 0; p < DIM; p++)
#pragma unroll
            for (int q = 0; q < DIM; q++)
                if (p != q && iJ[p * DIM + q] != 0.0) box = false;
        double C[DIM * DIM];
#pragma unroll
        for (int p = 0; p < DIM; p++)
#pragma unroll
            for (int q = 0; q < DIM; q++)
            {
                if (box && p != q)
                {
                    C[p * DIM + q] = 0.0;
                    continue;
                }
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; k++) s += iJ[k * DIM + p] * iJ[k * DIM + q];
                C[p * DIM + q] = det * mat * s;
            }
        double Ml[NN * (NN + 1) / 2], Ll[NN * (NN + 1) / 2], grav[NN];
        const double md = cm * det;
        if (box)
        {
#pragma unroll
            for (int i = 0; i < NN; i++)
#pragma unroll
                for (int j = 0; j <= i; j++)
                {
                    const int l = i * (i + 1) / 2 + j;
                    double s = 0.0;
#pragma unroll
                    for (int p = 0; p < DIM; p++) s += C[p * DIM + p] * sQ[((p * DIM + p) * NN + i) * NN + j];
                    Ll[l] = s;
                    Ml[l] = md * sM0[i * NN + j];
                }
        }
        else
        {
#pragma unroll
            for (int i = 0; i < NN; i++)
#pragma unroll
                for (int j = 0; j <= i; j++)
                {
                    const int l = i * (i + 1) / 2 + j;
                    double s = 0.0;
#pragma unroll
                    for (int pq = 0; pq < DIM * DIM; pq++) s += C[pq] * sQ[(pq * NN + i) * NN + j];
                    Ll[l] = s;
                    Ml[l] = md * sM0[i * NN + j];
                }
        }
        if (a.p.mass_lumping) lump_mass<ET, NN>(X, Y, Z, cm, Ml);
#pragma unroll
        for (int i = 0; i < NN; i++) grav[i] = 0.0;
        if (a.p.pcs_type == OGS_PCS_LIQUID_FLOW && a.p.gravity_on)
        {
            // -rho g |J| sum_gp w dNg_last,i = -rho g |J| sum_k iJ[last][k] sum_gp w dN_k,i;
            // sum_gp w dN_k,i is Q-independent: recompute from the centre
            // gradient (constant for affine tets) via the weight sum
            const double rho = a.p.gravity < DBL_EPSILON ? 1.0 : a.p.density * a.p.gravity;
            // sum_gp w_gp dN(gp) for affine maps equals vol_ref * dN(centre)
            const double vol_ref = ET == OGS_ELEM_HEX8 ? 8.0 : ET == OGS_ELEM_QUAD4 ? 4.0 : 1.0 / 6.0;
#pragma unroll
            for (int i = 0; i < NN; i++)
            {
                double g = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; k++) g += iJ[(DIM - 1) * DIM + k] * sdNc[k * NN + i];
                grav[i] = -(det * rho * vol_ref) * g * mat;
            }
        }
        flow_combine<NN>(a, e, nd, U, Ml, Ll, grav);
    }
}

// ------------------------------------------------------------------
// flow on a regular lattice of axis-aligned boxes, one thread per row
// ------------------------------------------------------------------
// Every cell of the lattice has the same Jacobian, so its element matrices
// are mat_c L_box + M_box with L_box, M_box common to all cells, and on a
// box an entry L_box[a][b] depends only on which coordinates of corners a
// and b agree (the pattern: bit 0 x, 1 y, 2 z).  Row i of the assembled
// system, at the column j = i + (dx, dy, dz), is therefore
//   A_ij = cnt_ij M_pat / dt + relax0 L_pat S_ij,  S_ij = sum of mat_c
// over the cells holding both nodes, and b_i = sum_j (cnt_ij M_pat / dt -
// relax1 L_pat S_ij) u0_j (+ the gravity term of LIQUID_FLOW): the same
// element matrices as k_flow_affine (whose per-element Gauss sums, FP64
// atomics and scatter this replaces), added in another order.  The tables
// come from element 0 through the element kernel's own formulas.
struct LatticeArgs
{
    const int32_t* slice_ptr;
    int nx, ny, nz;
    int64_t n;
};

__host__ __device__ constexpr int kCornerX(int k) { return (k == 1 || k == 2 || k == 5 || k == 6) ? 1 : 0; }
__host__ __device__ constexpr int kCornerY(int k) { return (k == 2 || k == 3 || k == 6 || k == 7) ? 1 : 0; }
__host__ __device__ constexpr int kCornerZ(int k) { return k >= 4 ? 1 : 0; }

// PLAIN: relax0 = 1 (no NLS relaxation), so b takes the mass term only
template <bool PLAIN>
__global__ void __launch_bounds__(256, 2) k_flow_lattice(AsmArgs a, LatticeArgs g)
{
    // sL: L_pat; sMC[pat][c] = c M_pat / dt for c shared cells (the product
    // formed once here, looked up per entry); sG: gravity per corner
    __shared__ double sL[8], sMC[8][9], sG[8];
    __shared__ int s_ok;
    if (threadIdx.x == 0)
    {
        int nd[8];
        double X[8], Y[8], Z[8], U[8];
        gather<8>(a, 0, nd, X, Y, Z, U);
        const double* Q = a.aff;
        const double* M0 = a.aff + 9 * 64;
        const double* dNc = a.aff + 9 * 64 + 64;
        double iJ[9], det;
        const bool ok = jacobian<8, 3>(X, Y, Z, dNc, iJ, det);
        s_ok = ok ? 1 : 0;
        if (!ok)
            flag_bad(a.bad_elem, 0);  // every cell has this Jacobian: element 0 is the first singular one
        else
        {
            double c[3];
            for (int q = 0; q < 3; q++)
            {
                double t = 0.0;
                for (int k = 0; k < 3; k++) t += iJ[k * 3 + q] * iJ[k * 3 + q];
                c[q] = det * t;
            }
            const double cm = flow_mass_coef(a.p), dt_inverse = 1.0 / a.p.dt;
            const double lumped = element_volume<OGS_ELEM_HEX8>(X, Y, Z) / 8.0;
            for (int pat = 0; pat < 8; pat++)
            {
                // corner b with this pattern against corner 0 = (0, 0, 0)
                int b = 0;
                for (int k = 0; k < 8; k++)
                    if ((kCornerX(k) == 0) == ((pat & 1) != 0) && (kCornerY(k) == 0) == ((pat & 2) != 0) &&
                        (kCornerZ(k) == 0) == ((pat & 4) != 0))
                        b = k;
                double l = 0.0;
                for (int q = 0; q < 3; q++) l += c[q] * Q[((q * 3 + q) * 8 + 0) * 8 + b];
                sL[pat] = l;
                const double m = a.p.mass_lumping ? (pat == 7 ? cm * 1.0 * lumped : 0.0) : cm * det * M0[b];
                const double mdt = m * dt_inverse;
                for (int n = 0; n <= 8; n++) sMC[pat][n] = (double)n * mdt;
            }
            const bool grav = a.p.pcs_type == OGS_PCS_LIQUID_FLOW && a.p.gravity_on;
            const double rho = a.p.gravity < DBL_EPSILON ? 1.0 : a.p.density * a.p.gravity;
            for (int k = 0; k < 8; k++)
            {
                double t = 0.0;
                for (int q = 0; q < 3; q++) t += iJ[2 * 3 + q] * dNc[q * 8 + k];
                sG[k] = grav ? -(det * rho * 8.0) * t : 0.0;
            }
        }
    }
    __syncthreads();
    if (!s_ok) return;
    double relax0 = a.p.nls_relaxation;
    if (relax0 < DBL_MIN) relax0 = 1.0;
    const double relax1 = 1.0 - relax0;
    const bool grav = a.p.pcs_type == OGS_PCS_LIQUID_FLOW && a.p.gravity_on;
    // GROUNDWATER_FLOW with time_unit_factor 1: mat = k * 1.0 * 1.0 = k
    const bool unit_mat = a.p.pcs_type == OGS_PCS_GROUNDWATER_FLOW && a.p.time_unit_factor == 1.0;
    const int nx = g.nx, ny = g.ny, nz = g.nz, ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    const int64_t nxy = (int64_t)nx * ny;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int iz = (int)(i / nxy), rem = (int)(i - iz * nxy), iy = rem / nx, ix = rem - iy * nx;
        // the eight cells around the node, (ix - 1 + ex, iy - 1 + ey, iz - 1 + ez)
        double mc[2][2][2];
        int pc[2][2][2];
        double gb = 0.0;
#pragma unroll
        for (int ez = 0; ez < 2; ez++)
#pragma unroll
            for (int ey = 0; ey < 2; ey++)
#pragma unroll
                for (int ex = 0; ex < 2; ex++)
                {
                    const int cx = ix - 1 + ex, cy = iy - 1 + ey, cz = iz - 1 + ez;
                    const bool in = cx >= 0 && cx < ncx && cy >= 0 && cy < ncy && cz >= 0 && cz < ncz;
                    const double k = in ? __ldg(a.elem_k + cx + (int64_t)ncx * (cy + (int64_t)ncy * cz)) : 0.0;
                    const double m = unit_mat ? k : flow_mat(a.p, k);
                    mc[ez][ey][ex] = m;
                    pc[ez][ey][ex] = in ? 1 : 0;
                    // the node is the cell's corner (1 - ex, 1 - ey, 1 - ez)
                    if (grav) gb += m * sG[(1 - ez) * 4 + ((1 - ey) ? ((1 - ex) ? 2 : 3) : ((1 - ex) ? 1 : 0))];
                }
        // sums over the cells shared with the neighbour at offset d: per axis
        // index 0 (d = -1: the lower cell), 1 (d = 0: both), 2 (d = +1)
        double sx[2][2][3], sy[2][3][3], S[3][3][3];
        int cx_[2][2][3], cy_[2][3][3], C[3][3][3];
#pragma unroll
        for (int ez = 0; ez < 2; ez++)
#pragma unroll
            for (int ey = 0; ey < 2; ey++)
            {
                sx[ez][ey][0] = mc[ez][ey][0];
                sx[ez][ey][2] = mc[ez][ey][1];
                sx[ez][ey][1] = mc[ez][ey][0] + mc[ez][ey][1];
                cx_[ez][ey][0] = pc[ez][ey][0];
                cx_[ez][ey][2] = pc[ez][ey][1];
                cx_[ez][ey][1] = pc[ez][ey][0] + pc[ez][ey][1];
            }
#pragma unroll
        for (int ez = 0; ez < 2; ez++)
#pragma unroll
            for (int kx = 0; kx < 3; kx++)
            {
                sy[ez][0][kx] = sx[ez][0][kx];
                sy[ez][2][kx] = sx[ez][1][kx];
                sy[ez][1][kx] = sx[ez][0][kx] + sx[ez][1][kx];
                cy_[ez][0][kx] = cx_[ez][0][kx];
                cy_[ez][2][kx] = cx_[ez][1][kx];
                cy_[ez][1][kx] = cx_[ez][0][kx] + cx_[ez][1][kx];
            }
#pragma unroll
        for (int ky = 0; ky < 3; ky++)
#pragma unroll
            for (int kx = 0; kx < 3; kx++)
            {
                S[0][ky][kx] = sy[0][ky][kx];
                S[2][ky][kx] = sy[1][ky][kx];
                S[1][ky][kx] = sy[0][ky][kx] + sy[1][ky][kx];
                C[0][ky][kx] = cy_[0][ky][kx];
                C[2][ky][kx] = cy_[1][ky][kx];
                C[1][ky][kx] = cy_[0][ky][kx] + cy_[1][ky][kx];
            }
        // the row's stored entries in column order: (dz, dy, dx) lexicographic
        const int64_t s0 = __ldg(g.slice_ptr + (i >> 5)) + (i & 31);
        double* __restrict__ v = a.val + s0;
        double bi = gb;
        int rank = 0;
#pragma unroll
        for (int dz = -1; dz <= 1; dz++)
#pragma unroll
            for (int dy = -1; dy <= 1; dy++)
#pragma unroll
                for (int dx = -1; dx <= 1; dx++)
                {
                    const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
                    if (jx < 0 || jx >= nx || jy < 0 || jy >= ny || jz < 0 || jz >= nz) continue;
                    const int pat = (dx == 0 ? 1 : 0) | (dy == 0 ? 2 : 0) | (dz == 0 ? 4 : 0);
                    const double mt = sMC[pat][C[dz + 1][dy + 1][dx + 1]];
                    const double lt = sL[pat] * S[dz + 1][dy + 1][dx + 1];
                    const int64_t j = i + dx + nx * (dy + (int64_t)ny * dz);
                    const double u = a.u0 && OGS_IN(j, g.n, kOobLatNode) ? __ldg(a.u0 + j) : 0.0;
                    const double e = PLAIN ? mt + lt : mt + lt * relax0;
                    if (OGS_IN(s0 + (int64_t)rank * kSlice, a.nslots, kOobLatSlot))
                    {
                        if (a.val_store)
                            v[(int64_t)rank * kSlice] = e;
                        else
                            v[(int64_t)rank * kSlice] += e;
                    }
                    if constexpr (PLAIN)
                        bi += mt * u;
                    else
                        bi += (mt - lt * relax1) * u;
                    rank++;
                }
        a.b[i] += bi;
    }
}

// ------------------------------------------------------------------
// MASS_TRANSPORT
// ------------------------------------------------------------------
// STORE: the kernel may be the one that fills the stored operators (the SUPG
// instantiation, whose extra terms vanish with supg_method 0)
template <int NN, bool STORE = false>
__device__ __forceinline__ void mt_combine(const AsmArgs& a, int64_t e, const int* nd,
                                           const double* U, const double* Ml,
                                           const double* L, const double* A,
                                           const double* St, const double* Mx = nullptr)
{
    // Mx: the non-symmetric SUPG mass term (full NN x NN), added to the mass
    // AssembleMixedHyperbolicParabolicEquation (fem_ele_std.cpp:8592-8692)
    if (STORE && a.val2)
    {
        // the operators stored for memory_type > 0 (EleMat->SetMass_notsym,
        // SetLaplace, SetAdvection, SetStorage; fem_ele_std.cpp:8565-8573),
        // scattered: their time weights are applied per assembly
#pragma unroll
        for (int i = 0; i < NN; i++)
#pragma unroll
            for (int j = 0; j < NN; j++)
            {
                const int l = i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
                const int k = i * NN + j;
                const int32_t slot = __ldg(a.slot_t + (int64_t)k * a.E + e);
                atomicAdd(a.val + slot, Mx ? Ml[l] + Mx[k] : Ml[l]);
                atomicAdd(a.val2 + slot, L[k] + A[k] + St[l]);
            }
        return;
    }
    const double dt_inverse = 1.0 / a.p.dt;
    const double th = a.p.theta;
    double S[NN * NN], r[NN];
#pragma unroll
    for (int i = 0; i < NN; i++) r[i] = 0.0;
#pragma unroll
    for (int i = 0; i < NN; i++)
#pragma unroll
        for (int j = 0; j < NN; j++)
        {
            const int l = i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
            const int k = i * NN + j;
            const double mij = Mx ? Ml[l] + Mx[k] : Ml[l];
            double s = mij * dt_inverse;
            s += L[k] * th;
            s += A[k] * th;
            s += St[l] * th;
            S[k] = s;
            double q = mij * dt_inverse;
            q += L[k] * (-(1.0 - th));
            q += A[k] * (-(1.0 - th));
            q += St[l] * (-(1.0 - th));
            r[i] += q * U[j];
        }
    scatter<NN>(a, e, nd, S, r);
}

// SUPG: with the streamline-upwind terms of ele_supg_method > 0
template <int ET, int NGP, bool SUPG>
__global__ void __launch_bounds__(128) k_mt_general(AsmArgs a)
{
    constexpr int NN = ElemTraits<ET>::NN, DIM = ElemTraits<ET>::DIM;
    __shared__ double sN[NGP * NN], sdN[NGP * NN * DIM], sw[NGP * 3];
    stage(sN, a.tab, NGP * NN);
    stage(sdN, a.tab + NGP * NN, NGP * NN * DIM);
    stage(sw, a.tab + NGP * NN + NGP * NN * DIM, NGP * 3);
    __syncthreads();
    const ogs_assembly_params& p = a.p;
    const double cm = p.steady ? 0.0 : p.porosity * p.saturation * p.retardation;
    const double cs = p.porosity * p.saturation * p.decay * p.retardation;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.E;
         e += (int64_t)gridDim.x * blockDim.x)
    {
        int nd[NN];
        double X[NN], Y[NN], Z[NN], U[NN];
        gather<NN>(a, e, nd, X, Y, Z, U);
        // Ls: the symmetric dispersion term, lower triangle (expanded for
        // the combine)
        double Ml[NN * (NN + 1) / 2], St[NN * (NN + 1) / 2], Ls[NN * (NN + 1) / 2], A[NN * NN];
        double Mx[SUPG ? NN * NN : 1];
#pragma unroll
        for (int l = 0; l < NN * (NN + 1) / 2; l++) Ml[l] = St[l] = Ls[l] = 0.0;
#pragma unroll
        for (int k = 0; k < NN * NN; k++) A[k] = 0.0;
#pragma unroll
        for (int k = 0; k < (SUPG ? NN * NN : 1); k++) Mx[k] = 0.0;
        const double Lsupg = SUPG ? supg_length<ET>(X, Y, Z, p.supg_length) : 0.0;
        bool ok = true;
        const double* ve = a.gpv + e * NGP * 3;
#pragma unroll 1
        for (int gp = 0; gp < NGP; gp++)
        {
            double iJ[DIM * DIM], det, dNg[DIM * NN];
            if (!jacobian<NN, DIM>(X, Y, Z, sdN + gp * NN * DIM, iJ, det)) { ok = false; break; }
            grad_global<NN, DIM>(iJ, sdN + gp * NN * DIM, dNg);
            const double* w = sw + gp * 3;
            const double fkt = ET == OGS_ELEM_HEX8 ? det * w[0] * w[1] * w[2]
                             : ET == OGS_ELEM_QUAD4 ? det * w[0] * w[1] : det * w[0];
            const double* sf = sN + gp * NN;
            const double v[3] = {__ldg(ve + gp * 3), __ldg(ve + gp * 3 + 1), __ldg(ve + gp * 3 + 2)};
            double D[DIM * DIM];
            dispersion<DIM>(p, v, D);
            const double mf = cm * fkt * 1.0;
            const double fs = fkt * cs;
            const double vt[3] = {1.0 * p.time_unit_factor * v[0], 1.0 * p.time_unit_factor * v[1],
                                  1.0 * p.time_unit_factor * v[2]};
            // the Gauss-point sums with their factors hoisted: T = D grad N
            // once, the symmetric dispersion term over distinct pairs,
            // vd_j = v . grad N_j once (rounding-level differences from the
            // per-entry products)
            double T[DIM * NN], vd[NN];
#pragma unroll
            for (int j = 0; j < NN; j++)
            {
                double q = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; k++)
                {
                    double t = 0.0;
#pragma unroll
                    for (int l2 = 0; l2 < DIM; l2++) t += D[DIM * k + l2] * dNg[l2 * NN + j];
                    T[k * NN + j] = t;
                    q += vt[k] * dNg[k * NN + j];
                }
                vd[j] = q;
            }
#pragma unroll
            for (int i = 0; i < NN; i++)
            {
                const double mi = mf * sf[i], si = fs * sf[i], ai = fkt * sf[i];
#pragma unroll
                for (int j = 0; j <= i; j++)
                {
                    const int l = i * (i + 1) / 2 + j;
                    Ml[l] += mi * sf[j];
                    St[l] += si * sf[j];
                    double g = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; k++) g += dNg[k * NN + i] * T[k * NN + j];
                    Ls[l] += fkt * g;
                }
#pragma unroll
                for (int j = 0; j < NN; j++) A[i * NN + j] += ai * vd[j];
            }
            if constexpr (SUPG)
            {
                // CalcSUPGWeightingFunction (fem_ele_std.cpp:4004-4025): w_i =
                // v . grad N_i with the raw flux; SUPG mass (CalcMass :3856-3879)
                // and advection (CalcAdvection :5467-5490) terms
                double Dr[DIM * DIM], wf[NN];
                dispersion_raw<DIM>(p, v, Dr);
                const double tau = supg_tau<DIM>(p, v, Dr, Lsupg);
#pragma unroll
                for (int i = 0; i < NN; i++)
                {
                    wf[i] = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; k++) wf[i] += dNg[k * NN + i] * v[k];
                }
#pragma unroll
                for (int i = 0; i < NN; i++)
#pragma unroll
                    for (int j = 0; j < NN; j++)
                    {
                        Mx[i * NN + j] += mf * tau * wf[i] * sf[j];
                        A[i * NN + j] += fkt * (1.0 * p.time_unit_factor) * tau * wf[i] * wf[j];
                    }
            }
        }
        if (!ok) { flag_bad(a.bad_elem, e); continue; }
        double L[NN * NN];
#pragma unroll
        for (int i = 0; i < NN; i++)
#pragma unroll
            for (int j = 0; j < NN; j++) L[i * NN + j] = Ls[i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i];
        if (p.mass_lumping)
        {
            // CalcLumpedMass has no SUPG term
            lump_mass<ET, NN>(X, Y, Z, cm, Ml);
            mt_combine<NN, SUPG>(a, e, nd, U, Ml, L, A, St);
        }
        else
            mt_combine<NN, SUPG>(a, e, nd, U, Ml, L, A, St, SUPG ? Mx : nullptr);
    }
}

// affine MASS_TRANSPORT on tets: gradients are constant, so
// Laplace = |J| dNg^T (sum_gp w D(gp)) dNg and
// Advection_ij = |J| sum_gp w N_i(gp) (v(gp) . dNg_j)
__global__ void __launch_bounds__(128) k_mt_tet_affine(AsmArgs a)
{
    constexpr int NN = 4, DIM = 3, NGP = 5;
    __shared__ double sN[NGP * NN], sw[NGP * 3], sM0[NN * NN], sdNc[DIM * NN];
    stage(sN, a.tab, NGP * NN);
    stage(sw, a.tab + NGP * NN + NGP * NN * DIM, NGP * 3);
    stage(sM0, a.aff + DIM * DIM * NN * NN, NN * NN);
    stage(sdNc, a.aff + DIM * DIM * NN * NN + NN * NN, DIM * NN);
    __syncthreads();
    const ogs_assembly_params& p = a.p;
    const double cm = p.steady ? 0.0 : p.porosity * p.saturation * p.retardation;
    const double cs = p.porosity * p.saturation * p.decay * p.retardation;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.E;
         e += (int64_t)gridDim.x * blockDim.x)
    {
        int nd[NN];
        double X[NN], Y[NN], Z[NN], U[NN];
        gather<NN>(a, e, nd, X, Y, Z, U);
        double iJ[DIM * DIM], det, dNg[DIM * NN];
        if (!jacobian<NN, DIM>(X, Y, Z, sdNc, iJ, det)) { flag_bad(a.bad_elem, e); continue; }
        grad_global<NN, DIM>(iJ, sdNc, dNg);
        const double* ve = a.gpv + e * NGP * 3;
        double Ds[DIM * DIM], A[NN * NN];
#pragma unroll
        for (int k = 0; k < DIM * DIM; k++) Ds[k] = 0.0;
#pragma unroll
        for (int k = 0; k < NN * NN; k++) A[k] = 0.0;
        // the Gauss-point fluxes; when all five are bit for bit the same (a
        // linear head field on an affine tet: Cal_Velocity gives one flux)
        // the dispersion tensor and v . grad N are formed once and reused,
        // which gives the same values as forming them per point
        double vg[NGP][3];
        bool same = true;
#pragma unroll
        for (int gp = 0; gp < NGP; gp++)
#pragma unroll
            for (int k = 0; k < 3; k++)
            {
                vg[gp][k] = __ldg(ve + gp * 3 + k);
                same = same && __double_as_longlong(vg[gp][k]) == __double_as_longlong(vg[0][k]);
            }
        const double tf = 1.0 * p.time_unit_factor;
        double D0[DIM * DIM], vd0[NN];
        dispersion<DIM>(p, vg[0], D0);
#pragma unroll
        for (int j = 0; j < NN; j++)
            vd0[j] = tf * vg[0][0] * dNg[j] + tf * vg[0][1] * dNg[NN + j] + tf * vg[0][2] * dNg[2 * NN + j];
#pragma unroll
        for (int gp = 0; gp < NGP; gp++)
        {
            const double w = sw[gp * 3];
            const double* v = vg[gp];
            double D[DIM * DIM], vd[NN];
            if (gp == 0 || same)
            {
#pragma unroll
                for (int k = 0; k < DIM * DIM; k++) D[k] = D0[k];
#pragma unroll
                for (int j = 0; j < NN; j++) vd[j] = vd0[j];
            }
            else
            {
                dispersion<DIM>(p, v, D);
#pragma unroll
                for (int j = 0; j < NN; j++)
                    vd[j] = tf * v[0] * dNg[j] + tf * v[1] * dNg[NN + j] + tf * v[2] * dNg[2 * NN + j];
            }
#pragma unroll
            for (int k = 0; k < DIM * DIM; k++) Ds[k] += w * D[k];
            const double wd = det * w;
#pragma unroll
            for (int i = 0; i < NN; i++)
            {
                const double wn = wd * sN[gp * NN + i];
#pragma unroll
                for (int j = 0; j < NN; j++) A[i * NN + j] += wn * vd[j];
            }
        }
        // L = |J| G^T Ds G (G the constant gradients): T = Ds G once, then
        // the symmetric product, one entry per pair
        double T[DIM * NN];
#pragma unroll
        for (int k = 0; k < DIM; k++)
#pragma unroll
            for (int j = 0; j < NN; j++)
            {
                double t = 0.0;
#pragma unroll
                for (int l = 0; l < DIM; l++) t += Ds[k * DIM + l] * dNg[l * NN + j];
                T[k * NN + j] = t;
            }
        double L[NN * NN], Ml[NN * (NN + 1) / 2], St[NN * (NN + 1) / 2];
#pragma unroll
        for (int i = 0; i < NN; i++)
#pragma unroll
            for (int j = 0; j <= i; j++)
            {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < DIM; k++) s += dNg[k * NN + i] * T[k * NN + j];
                L[i * NN + j] = L[j * NN + i] = det * s;
            }
#pragma unroll
        for (int i = 0; i < NN; i++)
#pragma unroll
            for (int j = 0; j <= i; j++)
            {
                const int l = i * (i + 1) / 2 + j;
                Ml[l] = cm * det * sM0[i * NN + j];
                St[l] = cs * det * sM0[i * NN + j];
            }
        if (p.mass_lumping) lump_mass<OGS_ELEM_TET4, NN>(X, Y, Z, cm, Ml);
        mt_combine<NN>(a, e, nd, U, Ml, L, A, St);
    }
}

// ------------------------------------------------------------------
// Gauss-point Darcy flux (Cal_Velocity scalar branch, fem_ele_std.cpp:6627-6870)
// ------------------------------------------------------------------
template <int ET, int NGP>
__global__ void __launch_bounds__(128) k_gp_velocity(AsmArgs a)
{
    constexpr int NN = ElemTraits<ET>::NN, DIM = ElemTraits<ET>::DIM;
    __shared__ double sdN[NGP * NN * DIM];
    stage(sdN, a.tab + NGP * NN, NGP * NN * DIM);
    __syncthreads();
    const ogs_assembly_params& p = a.p;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.E;
         e += (int64_t)gridDim.x * blockDim.x)
    {
        int nd[NN];
        double X[NN], Y[NN], Z[NN], U[NN];
        gather<NN>(a, e, nd, X, Y, Z, U);
        const double mat = flow_mat(p, __ldg(a.elem_k + e));
        double* qo = a.q_out + e * NGP * 3;
#pragma unroll 1
        for (int gp = 0; gp < NGP; gp++)
        {
            double iJ[DIM * DIM], det, dNg[DIM * NN];
            if (!jacobian<NN, DIM>(X, Y, Z, sdN + gp * NN * DIM, iJ, det)) { flag_bad(a.bad_elem, e); break; }
            grad_global<NN, DIM>(iJ, sdN + gp * NN * DIM, dNg);
            double vel[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int i = 0; i < DIM; i++)
            {
                double s = 0.0;
#pragma unroll
                for (int j = 0; j < NN; j++) s += U[j] * dNg[i * NN + j];
                vel[i] = s;
            }
            if (p.pcs_type == OGS_PCS_LIQUID_FLOW && p.gravity_on && p.gravity >= DBL_EPSILON)
                vel[DIM - 1] += p.gravity * p.density;
            double q[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int i = 0; i < DIM; i++) q[i] -= mat * vel[i] / p.time_unit_factor;
            qo[gp * 3 + 0] = q[0];
            qo[gp * 3 + 1] = q[1];
            qo[gp * 3 + 2] = q[2];
        }
    }
}

// ------------------------------------------------------------------
// RICHARDS_FLOW (fem_ele_std.cpp:9470-9481): AssembleParabolicEquation and
// Assemble_Gravity with the storage and conductivity of the Picard iterate
// at each Gauss point
// ------------------------------------------------------------------
__device__ __forceinline__ double mrange(double a, double b, double c)
{
    return b < a ? a : b > c ? c : b;  // MRange (FEM/mathlib.cpp:447)
}

// CMediumProperties::SaturationCapillaryPressureFunction, models 4 (van
// Genuchten) and 6 (Brooks-Corey) (rf_mmp_new.cpp:5243-5328)
// x^y for x >= 0 as exp(y log x): the curves' bases are never negative, and
// 0^y (0 for y > 0, inf for y < 0) comes out of log(0) = -inf.  Cheaper than
// pow on GB300's FP64 unit; the result is within |y log x| ulps of pow's
// (<= ~1e-14 relative on the curves' range)
__device__ __forceinline__ double powp(double x, double y) { return exp(y * log(x)); }

__device__ __forceinline__ double rich_saturation(const ogs_richards_params& r, double pc)
{
    // divisions by parameters as products with their reciprocals (loop
    // invariants of the Gauss-point loop; rounding-level differences)
    const double ipb = 1.0 / r.pb;
    double se;
    if (r.capillary_model == 4)
    {
        if (pc < 0.0) pc = 0.0;
        se = powp(pc * ipb, 1.0 / (1.0 - r.m)) + 1.0;
        se = powp(se, -r.m);
    }
    else
    {
        if (pc < r.pb) pc = r.pb;
        se = powp(pc * ipb, -r.m);
    }
    const double sl = se * (r.slm - r.slr) + r.slr;
    return mrange(r.slr + DBL_EPSILON, sl, r.slm - DBL_EPSILON);
}

// PressureSaturationDependency(Sw, invert = true): dSw/dpc (<= 0), bounded
// below by -1/DBL_EPSILON (rf_mmp_new.cpp:5425-5520)
__device__ __forceinline__ double rich_dsdpc(const ogs_richards_params& r, double sl)
{
    // dS/dpc = 1 / (dpc/dS) formed as one quotient; divisions by
    // parameters as products with their reciprocals
    const double isr = 1.0 / (r.slm - r.slr);
    double dsdp;
    if (r.capillary_model == 4)
    {
        sl = mrange(r.slr + DBL_EPSILON, sl, r.slm - DBL_EPSILON);
        const double v1 = powp((sl - r.slr) * isr, -1.0 / r.m);
        const double v2 = powp(v1 - 1.0, -r.m);
        dsdp = (r.m * (sl - r.slr)) / (r.pb * (r.m - 1.0) * v1 * v2);
    }
    else
    {
        sl = mrange(r.slr + DBL_EPSILON, sl, r.slm);
        const double v1 = powp((sl - r.slr) * isr, -1.0 / r.m);
        dsdp = (r.m * (r.slr - sl)) / (r.pb * v1);
    }
    const double lim = (-1.0) / DBL_EPSILON;
    if (dsdp < lim) dsdp = lim;
    return dsdp;
}

// PermeabilitySaturationFunction(Sw, 0), models 4 (van Genuchten-Mualem)
// and 6 (Brooks-Corey) (rf_mmp_new.cpp:2576-2635)
__device__ __forceinline__ double rich_krel(const ogs_richards_params& r, double sl)
{
    sl = mrange(r.kr_slr, sl, r.kr_slm);
    const double se = (sl - r.kr_slr) * (1.0 / (r.kr_slm - r.kr_slr));
    double kr;
    if (r.permeability_model == 4)
    {
        const double b = 1.0 - powp(1.0 - powp(se, 1.0 / r.kr_m), r.kr_m);
        kr = sqrt(se) * (b * b);
    }
    else
        kr = powp(se, 3.0 + 2.0 / r.kr_m);
    if (kr < r.kr_min) kr = r.kr_min;
    return kr;
}

// CalCoefMass, EPT_RICHARDS_FLOW (fem_ele_std.cpp:1721-1770), isothermal,
// constant drho_dp
__device__ __forceinline__ double rich_mass_coef(const ogs_assembly_params& p, const ogs_richards_params& r,
                                                 double PG)
{
    double Sw = 1.0, dSdp = 0.0;
    if (PG < 0.0)
    {
        Sw = rich_saturation(r, -PG);
        dSdp = -rich_dsdpc(r, Sw);
    }
    double val = p.storage * Sw;
    if (p.density > 0.0) val += p.porosity * Sw * p.drho_dp;
    if (PG < 0.0) val += p.porosity * dSdp;
    return val;
}

// element geometry constant over the Gauss points (see k_richards)
template <int ET>
__device__ __forceinline__ bool const_geometry(const double* X, const double* Y, const double* Z)
{
    if (ET == OGS_ELEM_TET4) return true;
    const bool rect = (X[0] == X[3] && X[1] == X[2] && Y[0] == Y[1] && Y[2] == Y[3]) ||
                      (X[0] == X[1] && X[2] == X[3] && Y[0] == Y[3] && Y[1] == Y[2]);
    if (ET == OGS_ELEM_QUAD4) return rect;
    bool box = rect && Z[0] == Z[1] && Z[0] == Z[2] && Z[0] == Z[3] && Z[4] == Z[5] && Z[4] == Z[6] && Z[4] == Z[7];
#pragma unroll
    for (int k = 0; k < 4; k++) box = box && X[k + 4] == X[k] && Y[k + 4] == Y[k];
    return box;
}

template <int ET, int NGP>
__global__ void __launch_bounds__(128) k_richards(AsmArgs a)
{
    constexpr int NN = ElemTraits<ET>::NN, DIM = ElemTraits<ET>::DIM;
    __shared__ double sN[NGP * NN], sdN[NGP * NN * DIM], sw[NGP * 3];
    stage(sN, a.tab, NGP * NN);
    stage(sdN, a.tab + NGP * NN, NGP * NN * DIM);
    stage(sw, a.tab + NGP * NN + NGP * NN * DIM, NGP * 3);
    __syncthreads();
    const ogs_assembly_params& p = a.p;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.E;
         e += (int64_t)gridDim.x * blockDim.x)
    {
        int nd[NN];
        double X[NN], Y[NN], Z[NN], U[NN], U1[NN];
        gather<NN>(a, e, nd, X, Y, Z, U);
#pragma unroll
        for (int i = 0; i < NN; i++) U1[i] = __ldg(a.u1 + nd[i]);
        const double ke = __ldg(a.elem_k + e);
        double Ml[NN * (NN + 1) / 2], Ll[NN * (NN + 1) / 2], grav[NN];
#pragma unroll
        for (int l = 0; l < NN * (NN + 1) / 2; l++) Ml[l] = Ll[l] = 0.0;
#pragma unroll
        for (int i = 0; i < NN; i++) grav[i] = 0.0;
        // geometry constant over the Gauss points: linear tets (constant shape
        // gradients), and hexes / quads that are axis-aligned boxes (exact
        // coordinate equalities; J is then diagonal, its off-diagonal sums
        // cancel exactly): J^-1 and |J| from the first Gauss point
        const bool cgeo = const_geometry<ET>(X, Y, Z);
        double iJ[DIM * DIM], det = 0.0, dNg[DIM * NN];
        bool ok = !cgeo || jacobian<NN, DIM>(X, Y, Z, sdN, iJ, det);
        if (ok && cgeo && ET == OGS_ELEM_TET4) grad_global<NN, DIM>(iJ, sdN, dNg);
#pragma unroll 1
        for (int gp = 0; gp < NGP && ok; gp++)
        {
            const double* dNr = sdN + gp * NN * DIM;
            if (!cgeo)
            {
                if (!jacobian<NN, DIM>(X, Y, Z, dNr, iJ, det)) { ok = false; break; }
                grad_global<NN, DIM>(iJ, dNr, dNg);
            }
            else if (ET != OGS_ELEM_TET4)
            {
#pragma unroll
                for (int k = 0; k < DIM; k++)
#pragma unroll
                    for (int i = 0; i < NN; i++) dNg[k * NN + i] = iJ[k * DIM + k] * dNr[k * NN + i];
            }
            const double* w = sw + gp * 3;
            const double fkt = ET == OGS_ELEM_HEX8 ? det * w[0] * w[1] * w[2]
                             : ET == OGS_ELEM_QUAD4 ? det * w[0] * w[1] : det * w[0];
            const double* sf = sN + gp * NN;
            double PG = 0.0;  // interpolate(NodalVal1)
#pragma unroll
            for (int i = 0; i < NN; i++) PG += U1[i] * sf[i];
            // CalCoefLaplace (fem_ele_std.cpp:2614-2640): K * (time_unit_factor
            // * kr(Sw) / mu) * fac_perm (1); CalCoefMass (:1721-1770) reuses
            // S(-PG), the same call, when unsaturated
            const double Sw = rich_saturation(a.r, -PG);
            const double mat = ke * (p.time_unit_factor * rich_krel(a.r, Sw) * (1.0 / p.viscosity)) * 1.0;
            double mc;
            {
                const double Sm = PG < 0.0 ? Sw : 1.0;
                mc = p.storage * Sm;
                if (p.density > 0.0) mc += p.porosity * Sm * p.drho_dp;
                if (PG < 0.0) mc += p.porosity * -rich_dsdpc(a.r, Sw);
            }
            const double mf = mc * fkt * 1.0;
            const double cl = fkt * mat;
#pragma unroll
            for (int i = 0; i < NN; i++)
            {
                const double mi = mf * sf[i];
#pragma unroll
                for (int j = 0; j <= i; j++)
                {
                    const int l = i * (i + 1) / 2 + j;
                    Ml[l] += mi * sf[j];
                    double g = 0.0;
#pragma unroll
                    for (int k = 0; k < DIM; k++) g += dNg[k * NN + i] * dNg[k * NN + j];
                    Ll[l] += cl * g;
                }
            }
            if (p.gravity_on)
            {
                // Assemble_Gravity (:5859-6000): rho g, or 1 in the head form
                const double rho = p.gravity < DBL_EPSILON ? 1.0 : p.density * p.gravity;
                const double fg = fkt * rho;
#pragma unroll
                for (int i = 0; i < NN; i++) grav[i] -= fg * dNg[(DIM - 1) * NN + i] * mat;
            }
        }
        if (!ok) { flag_bad(a.bad_elem, e); continue; }
        if (p.mass_lumping)
        {
            // CalcLumpedMass: CalCoefMass at the element centre (equal shape
            // function values 1/NN there)
            double PG = 0.0;
#pragma unroll
            for (int i = 0; i < NN; i++) PG += U1[i] * (1.0 / NN);
            lump_mass<ET, NN>(X, Y, Z, rich_mass_coef(p, a.r, PG), Ml);
        }
        flow_combine<NN>(a, e, nd, U, Ml, Ll, grav);
    }
}

static int grid_for(int64_t E, int threads)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t need = (E + threads - 1) / threads;
    const int64_t cap = (int64_t)sms * 16;
    return (int)std::max<int64_t>(1, std::min(need, cap));
}

template <int ET, int NGP>
static void launch_flow(const AsmArgs& a, bool affine, cudaStream_t s)
{
    const int g = grid_for(a.E, 128);
    if (affine)
        k_flow_affine<ET><<<g, 128, 0, s>>>(a);
    else
        k_flow_general<ET, NGP><<<g, 128, 0, s>>>(a);
}

template <int ET, int NGP>
static void launch_mt(const AsmArgs& a, bool affine, cudaStream_t s)
{
    const int g = grid_for(a.E, 128);
    // the affine tet kernel folds the Gauss points away; SUPG needs them.
    // Filling the stored operators (a.val2) goes through the SUPG kernel,
    // exact for supg_method 0 too (tau = 0 adds zeros).
    if (a.val2)
        k_mt_general<ET, NGP, true><<<g, 128, 0, s>>>(a);
    else if (ET == OGS_ELEM_TET4 && affine && a.p.supg_method == 0)
        k_mt_tet_affine<<<g, 128, 0, s>>>(a);
    else if (a.p.supg_method > 0)
        k_mt_general<ET, NGP, true><<<g, 128, 0, s>>>(a);
    else
        k_mt_general<ET, NGP, false><<<g, 128, 0, s>>>(a);
}

template <int ET, int NGP>
static void launch_richards(const AsmArgs& a, cudaStream_t s)
{
    k_richards<ET, NGP><<<grid_for(a.E, 128), 128, 0, s>>>(a);
}

template <int ET, int NGP>
static void launch_vel(const AsmArgs& a, cudaStream_t s)
{
    k_gp_velocity<ET, NGP><<<grid_for(a.E, 128), 128, 0, s>>>(a);
}

// Cell coefficients of the flow operator on a regular hex lattice.  Without
// mass lumping the left-hand side flow_combine scatters is
// sum_c (alpha_c L_box + beta M_box) with alpha_c = relax0 * mat(K_c) and
// beta = CalCoefMass / dt, L_box and M_box the Laplace and mass matrices of
// the unit-coefficient box; the FP32 inner CG applies the operator from
// these (summed over the assemblies since Initialize).  beta sits at
// coef[E].
__global__ void k_flow_cell_coef(ogs_assembly_params p, const double* __restrict__ elem_k, int64_t E,
                                 double* coef)
{
    double relax0 = p.nls_relaxation;
    if (relax0 < DBL_MIN) relax0 = 1.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x)
        coef[e] += relax0 * flow_mat(p, __ldg(elem_k + e));
    if (blockIdx.x == 0 && threadIdx.x == 0) coef[E] += flow_mass_coef(p) * (1.0 / p.dt);
}

void launch_flow_cell_coef(const AsmArgs& a, double* coef, cudaStream_t s)
{
    k_flow_cell_coef<<<grid_for(a.E, 256), 256, 0, s>>>(a.p, a.elem_k, a.E, coef);
}

// dispatch on (element type, Gauss points); returns false for an
// unsupported combination.  Flow on a regular hex lattice takes the row
// kernel (not for the split assembly of memory_type, which needs the terms
// apart)
bool launch_assembly(const ogs_mesh* m, const AsmArgs& a, bool affine, int kind,
                     cudaStream_t s)
{
    const int et = m->elem_type, ngp = m->ngp;
    if (kind == 0 && et == OGS_ELEM_HEX8 && m->grid && affine && !a.val2 &&
        (a.p.pcs_type == OGS_PCS_GROUNDWATER_FLOW || a.p.pcs_type == OGS_PCS_LIQUID_FLOW))
    {
        LatticeArgs g;
        g.slice_ptr = m->slice_ptr;
        g.nx = m->gx; g.ny = m->gy; g.nz = m->gz;
        g.n = m->n_nodes;
        double relax0 = a.p.nls_relaxation;
        if (relax0 < DBL_MIN) relax0 = 1.0;
        if (relax0 == 1.0)
            k_flow_lattice<true><<<grid_for(g.n, 256), 256, 0, s>>>(a, g);
        else
            k_flow_lattice<false><<<grid_for(g.n, 256), 256, 0, s>>>(a, g);
        return true;
    }
#define OGS_DISPATCH(ET_, NGP_)                                      \
    if (et == ET_ && ngp == NGP_)                                    \
    {                                                                \
        if (kind == 0) launch_flow<ET_, NGP_>(a, affine, s);         \
        else if (kind == 1) launch_mt<ET_, NGP_>(a, affine, s);      \
        else if (kind == 3) launch_richards<ET_, NGP_>(a, s);        \
        else launch_vel<ET_, NGP_>(a, s);                            \
        return true;                                                 \
    }
    OGS_DISPATCH(OGS_ELEM_QUAD4, 1)
    OGS_DISPATCH(OGS_ELEM_QUAD4, 4)
    OGS_DISPATCH(OGS_ELEM_QUAD4, 9)
    OGS_DISPATCH(OGS_ELEM_HEX8, 1)
    OGS_DISPATCH(OGS_ELEM_HEX8, 8)
    OGS_DISPATCH(OGS_ELEM_HEX8, 27)
    OGS_DISPATCH(OGS_ELEM_TET4, 5)
#undef OGS_DISPATCH
    return false;
}

}  // namespace ogs

unsigned long long ogs_oob_assembly() { return ogs::oob_take(); }
