"""Writes the golden fixtures of tests/golden/ from the reference's own code.

Run where the reference sources exist (they are compiled by oracle/Makefile
into oracle/_ref/libogs5ref.so: FEM/mathlib.cpp, FEM/matrix_class.cpp and
FEM/equation_class.cpp, unmodified):

    python tests/golden/make_golden.py [/path/to/reference]

Fixtures:
  ref_tables.npz   MXPGaussPkt / MXPGaussFkt (orders 1-4), SamplePointTet5,
                   and ShapeFunction{Quad,Hex,Tet} + gradients at every
                   Gauss point of the default rules
  ref_linear_eqs.npz
                   a 7x6x5-node hex system (GROUNDWATER_FLOW, seeded ln K,
                   Ss 1e-4, dt 3600): the assembled CRS values and b (the
                   assembly is the oracle's; the reference's element loop
                   cannot be built without its cmake-generated sources), then
                   the reference's Diagonize (row-only Dirichlet) result,
                   Linear_EQS::Solver with BiCGStab + Jacobi on it, and
                   Linear_EQS::Solver with CG + Jacobi on the symmetrically
                   eliminated system: solutions, iteration counts, errors.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main(ref_dir):
    from oracle import oracle as O
    from ogs5_gb300 import fields
    from ogs5_gb300 import mesh as M
    O.build(ref_dir)
    R = O.ref()
    out = {}
    gp = np.array([[R.ref_gauss_point(g, p) if p < g else np.nan for p in range(4)] for g in range(1, 5)])
    gw = np.array([[R.ref_gauss_weight(g, p) if p < g else np.nan for p in range(4)] for g in range(1, 5)])
    t5 = np.zeros((5, 4))
    for n in range(5):
        v = np.zeros(4)
        R.ref_tet5_point(n, v)
        t5[n] = v
    out.update(gauss_points=gp, gauss_weights=gw, tet5=t5)
    for et, name, ng in ((0, "quad", 3), (1, "hex", 3), (2, "tet", 3)):
        xi, w, N, dN = O.shape_table(et, ng)
        nn, dim = N.shape[1], dN.shape[1]
        Nr = np.zeros((len(w), nn))
        dNr = np.zeros((len(w), dim * nn))
        for g in range(len(w)):
            a, b = np.zeros(nn), np.zeros(nn * dim)
            R.ref_shape(et, np.ascontiguousarray(xi[g]), a, b)
            Nr[g], dNr[g] = a, b
        out[f"{name}_xi"] = xi
        out[f"{name}_N"] = Nr
        out[f"{name}_dN"] = dNr
    np.savez_compressed(os.path.join(HERE, "ref_tables.npz"), **out)

    m = M.structured_hex(6, 5, 4)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 3.0, seed=11)
    rp, col = O.build_pattern(m.n_nodes, m.conn)
    p = O.make_params(pcs_type=0, dt=3600.0, storage=1e-4)
    u0 = np.linspace(0.0, 1.0, m.n_nodes)
    val, b = O.assemble(m, rp, col, p, elem_k=ek, u0=u0)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    rs = O.RefSystem(rp, col, method=2, precond=1, max_iter=2000, tol=1e-12)
    rs.set(val, b)
    rs.set_known(rows, vals)
    val_ro, b_ro = rs.get()
    x_bi, info_bi = rs.solve(x0)
    rs.close()
    vs, bs = val.copy(), b.copy()
    O.dirichlet(rp, col, vs, bs, rows, vals, symmetric=True)
    rc = O.RefSystem(rp, col, method=5, precond=1, max_iter=2000, tol=1e-12)
    rc.set(vs, bs)
    x_cg, info_cg = rc.solve(x0)
    rc.close()
    np.savez_compressed(
        os.path.join(HERE, "ref_linear_eqs.npz"), shape=np.array(m.shape), elem_k=ek, u0=u0,
        row_ptr=rp, col=col, val=val, b=b, bc_rows=rows, bc_vals=vals, x0=x0,
        val_row_only=val_ro, b_row_only=b_ro, val_sym=vs, b_sym=bs,
        x_bicgstab=x_bi, iter_bicgstab=info_bi["iterations"], err_bicgstab=info_bi["rel_residual"],
        x_cg=x_cg, iter_cg=info_cg["iterations"], err_cg=info_cg["rel_residual"])
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
