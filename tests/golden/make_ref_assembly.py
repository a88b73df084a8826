"""Writes tests/golden/ref_assembly.npz: systems assembled by the reference
OGS-5 itself (its own CFiniteElementStd::Assembly, GlobalAssembly,
Cal_Velocity and Picard loop), compiled from its sources by
oracle/refbuild.mk and driven by oracle/ref_assemble_harness.cpp.

    make -C oracle -f refbuild.mk -j8
    python tests/golden/make_ref_assembly.py

Every case is a small deck (quad, hex or tet mesh; affine, sheared or
distorted) read by the reference's Problem constructor, with element-wise
conductivity (#MEDIUM_PROPERTIES_DISTRIBUTED), random nodal values of the
primary variable and, for MASS_TRANSPORT, random Gauss-point fluxes written
into ele_gp_value.  The fixture keeps, per case, the mesh, the inputs, the
ogs_assembly_params values equivalent to the deck, and what the reference
produced: the CRS values and right-hand side of Linear_EQS (Write_BIN), the
Gauss-point velocities, or the Picard result.  tests/test_ref_assembly.py
checks the C restatement against it, tests/test_ref_assembly_gpu.py the CUDA
path.
"""
from __future__ import annotations

import copy
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import ref_decks as R  # noqa: E402
from ogs5_gb300 import mesh as M  # noqa: E402

NGP = {M.QUAD4: 9, M.HEX8: 27, M.TET4: 5}
GRAVITY = 9.81  # gravity_constant of the reference (FEM/makros.cpp)


def base_mesh(kind):
    if kind == "quad":
        return M.structured_quad(6, 4, 1.0, 0.5)
    if kind == "hex":
        return M.structured_hex(4, 3, 2, 1.0, 2.0, 0.5)
    return M.structured_tet(3, 2, 2, 1.0, 1.5, 0.75)


def sheared(m):
    s = copy.copy(m)
    x, y, z = m.x.astype(float), m.y.astype(float), m.z.astype(float)
    s.x = x + 0.31 * y + 0.17 * z
    s.y = 0.93 * y + 0.22 * z - 0.12 * x
    if m.dim == 3:
        s.z = 1.07 * z + 0.05 * x
    return s


def distorted(m, amount=0.15, seed=3):
    rng = np.random.default_rng(seed)
    out = copy.copy(m)
    coords = [m.x.copy(), m.y.copy(), m.z.copy()]
    for a in range(m.dim):
        c = coords[a]
        inner = (c > c.min()) & (c < c.max())
        c[inner] += amount * rng.uniform(-1, 1, inner.sum())
    out.x, out.y, out.z = coords
    return out


def mesh_of(kind, geom):
    m = base_mesh(kind)
    if geom == "sheared":
        return sheared(m)
    if geom == "distorted":
        return distorted(m)
    return m


def params(**kw):
    """ogs_assembly_params values (names of include/ogs_gpu.h)."""
    p = dict(pcs_type=0, steady=0, dt=1.0, theta=1.0, nls_relaxation=0.0, time_unit_factor=1.0,
             storage=0.0, porosity=0.0, drho_dp=0.0, viscosity=1.0, density=1000.0, gravity=0.0,
             gravity_on=0, mass_lumping=0, alpha_l=0.0, alpha_t=0.0, diffusion=0.0, decay=0.0,
             retardation=1.0, saturation=1.0, supg_method=0, supg_length=0, supg_diffusivity=0,
             memory_type=0)
    p.update(kw)
    return p


class Writer:
    def __init__(self):
        self.out = {}
        self.names = []
        self.tmp = tempfile.mkdtemp(prefix="ogs_ref_")

    def add(self, name, m, ngauss, p, arrays, meta=None):
        self.names.append(name)
        self.out[f"{name}/mesh"] = np.array([m.elem_type, m.dim, ngauss], dtype=np.int64)
        self.out[f"{name}/xyz"] = np.stack([m.x, m.y, m.z]).astype(np.float64)
        self.out[f"{name}/conn"] = np.asarray(m.conn, dtype=np.int32)
        self.out[f"{name}/params"] = np.array(json.dumps(p))
        if meta is not None:
            self.out[f"{name}/meta"] = np.array(json.dumps(meta))
        for k, v in arrays.items():
            self.out[f"{name}/{k}"] = np.asarray(v)

    def deck_dir(self, name):
        d = os.path.join(self.tmp, name)
        os.makedirs(d, exist_ok=True)
        return d


def k_field(m, seed, scale=1e-5):
    rng = np.random.default_rng(seed)
    return np.exp(np.log(scale) + rng.standard_normal(m.n_elements))


def flow_case(W, name, kind, geom, pcs, seed, ngauss=3, steady=False, lumping=False, relax=0.0,
              liquid_drho=False):
    m = mesh_of(kind, geom)
    rng = np.random.default_rng(seed)
    dt = 3600.0 if pcs == "GROUNDWATER_FLOW" else 100.0
    nonlinear = ("PICARD", "LMAX", 1, relax, 1e-6) if relax else None
    proc = R.Process(pcs, steady=steady, dt=dt, gauss_points=ngauss, mass_lumping=int(lumping),
                     nonlinear=nonlinear)
    if pcs == "GROUNDWATER_FLOW":
        ek = k_field(m, seed)
        u0 = rng.uniform(0, 10, m.n_nodes)
        med = R.Medium(dim=m.dim, storage=1e-4)
        fl = R.Fluid()
        p = params(pcs_type=0, steady=int(steady), dt=dt, storage=1e-4, mass_lumping=int(lumping),
                   nls_relaxation=relax)
    else:
        ek = k_field(m, seed, 1e-12)
        gravity = m.dim == 3
        if liquid_drho:
            # density model 2, rho = rho_0 (1 + drho_dp (max(p, 0) - p_0)) with
            # p_0 = 0 and pressures below zero: rho = rho_0 at every Gauss point
            u0 = rng.uniform(-2e5, -1e5, m.n_nodes)
            fl = R.Fluid(density=1000.0, drho_dp=4.5e-10, viscosity=1e-3, gravity=gravity)
        else:
            u0 = rng.uniform(1e5, 2e5, m.n_nodes)
            fl = R.Fluid(density=998.0, viscosity=1.2e-3, gravity=gravity)
        med = R.Medium(dim=m.dim, storage=1e-9, porosity=0.3)
        p = params(pcs_type=1, steady=int(steady), dt=dt, storage=1e-9, porosity=0.3,
                   drho_dp=fl.drho_dp, viscosity=fl.viscosity, density=fl.density,
                   gravity=GRAVITY, gravity_on=int(gravity),
                   mass_lumping=int(lumping), nls_relaxation=relax)
    deck = R.Deck(mesh=m, processes=[proc], medium=med, fluid=fl, elem_k=ek)
    path = R.write(deck, W.deck_dir(name))
    R.write_doubles(path + ".u0", u0)
    R.run(R.REF_SP, path, ["step 1 %r" % dt, "nodal 0 2 %s.u0" % path, "assemble 0 %s.sys" % path])
    s = R.read_system(path + ".sys")
    W.add(name, m, ngauss, p, dict(elem_k=ek, u0=u0, row_ptr=s["row_ptr"], col=s["col"],
                                   val=s["val"], b=s["b"]))


def transport_case(W, name, kind, geom, seed, lumping=False, supg=None, memory=False, decay=None,
                   kd=None):
    m = mesh_of(kind, geom)
    rng = np.random.default_rng(seed)
    ngp = NGP[m.elem_type]
    dt, theta = 3600.0, 0.6
    flow = R.Process("GROUNDWATER_FLOW", dt=dt)
    mt = R.Process("MASS_TRANSPORT", dt=dt, theta=theta, mass_lumping=int(lumping), supg=supg,
                   memory_type=int(memory))
    med = R.Medium(dim=m.dim, storage=1e-4, porosity=0.3, tortuosity=0.7, alpha_l=1.0, alpha_t=0.1)
    comp = R.Component(diffusion=1e-9, decay=decay, kd=kd)
    deck = R.Deck(mesh=m, processes=[flow, mt], medium=med, component=comp, elem_k=k_field(m, seed))
    path = R.write(deck, W.deck_dir(name))
    vel = rng.normal(0, 1e-5, (m.n_elements, ngp, 3))
    if m.dim == 2:
        vel[:, :, 2] = 0.0
    c0 = rng.uniform(0, 1, m.n_nodes)
    R.write_doubles(path + ".c0", c0)
    R.write_doubles(path + ".vel", vel)
    cmds = ["step 1 %r" % dt, "nodal 1 2 %s.c0" % path, "velocity_in %s.vel" % path,
            "assemble 1 %s.sys" % path]
    arrays = dict(u0=c0, gp_vel=vel)
    dt2 = 1800.0
    if memory:
        vel2 = rng.normal(0, 1e-5, vel.shape)
        c1 = rng.uniform(0, 1, m.n_nodes)
        R.write_doubles(path + ".c1", c1)
        R.write_doubles(path + ".vel2", vel2)
        cmds += ["step 2 %r" % dt2, "nodal 1 2 %s.c1" % path, "velocity_in %s.vel2" % path,
                 "assemble 1 %s.sys2" % path]
        arrays.update(u0_2=c1, gp_vel_2=vel2)
    R.run(R.REF_SP, path, cmds)
    s = R.read_system(path + ".sys")
    arrays.update(row_ptr=s["row_ptr"], col=s["col"], val=s["val"], b=s["b"])
    if memory:
        s2 = R.read_system(path + ".sys2")
        arrays.update(val_2=s2["val"], b_2=s2["b"])
    sm, sl, sd = supg if supg else (0, 0, 0)
    p = params(pcs_type=2, dt=dt, theta=theta, porosity=0.3, alpha_l=1.0, alpha_t=0.1,
               diffusion=1e-9 * 0.7, decay=decay or 0.0, retardation=comp.retardation(0.3),
               mass_lumping=int(lumping), supg_method=sm,
               supg_length=sl, supg_diffusivity=sd, memory_type=int(memory))
    W.add(name, m, 3, p, arrays, meta={"dt_2": dt2} if memory else None)


def velocity_case(W, name, kind, geom, pcs, seed):
    m = mesh_of(kind, geom)
    rng = np.random.default_rng(seed)
    liquid = pcs == "LIQUID_FLOW"
    ek = k_field(m, seed, 1e-12 if liquid else 1e-5)
    gravity = liquid and m.dim == 3
    fl = R.Fluid(density=998.0, viscosity=1.2e-3, gravity=gravity) if liquid else R.Fluid()
    proc = R.Process(pcs, dt=1.0)
    deck = R.Deck(mesh=m, processes=[proc], medium=R.Medium(dim=m.dim, storage=1e-4, porosity=0.3),
                  fluid=fl, elem_k=ek)
    path = R.write(deck, W.deck_dir(name))
    h = rng.uniform(1e5, 2e5, m.n_nodes) if liquid else rng.uniform(0, 10, m.n_nodes)
    R.write_doubles(path + ".h", h)
    R.run(R.REF_SP, path, ["step 1 1.0", "nodal 0 2 %s.h" % path, "velocity_out 0 %d %s.vel" % (NGP[m.elem_type], path)])
    q = np.fromfile(path + ".vel", dtype=np.float64).reshape(m.n_elements, NGP[m.elem_type], 3)
    p = params(pcs_type=1 if liquid else 0, dt=1.0, storage=1e-4, porosity=0.3,
               viscosity=fl.viscosity, density=fl.density, gravity=GRAVITY,
               gravity_on=int(gravity))
    W.add(name, m, 3, p, dict(elem_k=ek, u=h, gp_vel=q))


RICHARDS = {
    # capillary (model, pb, slr, slm, m, pc_max) and relative permeability
    # (model, slr, slm, m, kr_min); the values of ogs_richards_params
    "vg": ((4, 1.0e4, 0.1, 1.0, 0.5, 1.0e10), (4, 0.1, 1.0, 0.5, 1e-9)),
    "bc": ((6, 5.0e3, 0.05, 0.95, 2.0, 1.0e10), (6, 0.05, 0.95, 2.0, 1e-9)),
}


def richards_deck(W, name, m, curve, seed, lumping, bc=None, nonlinear=None):
    cap, kr = RICHARDS[curve]
    dt = 3600.0
    proc = R.Process("RICHARDS_FLOW", dt=dt, mass_lumping=int(lumping), ls_tol=1e-14,
                     ls_max_iter=5000, nonlinear=nonlinear)
    med = R.Medium(dim=m.dim, storage=1e-6, porosity=0.35, capillary=cap[:5] + (cap[5], 0),
                   rel_perm=kr)
    fl = R.Fluid(density=1000.0, viscosity=1e-3, gravity=m.dim == 3)
    deck = R.Deck(mesh=m, processes=[proc], medium=med, fluid=fl, elem_k=k_field(m, seed, 1e-12),
                  bc=bc or [])
    return deck, R.write(deck, W.deck_dir(name)), dt


def richards_params_of(curve):
    cap, kr = RICHARDS[curve]
    return dict(capillary_model=cap[0], permeability_model=kr[0], pb=cap[1], slr=cap[2], slm=cap[3],
                m=cap[4], kr_slr=kr[1], kr_slm=kr[2], kr_m=kr[3], kr_min=kr[4])


def richards_assembly_case(W, name, kind, geom, curve, seed, lumping=False):
    m = mesh_of(kind, geom)
    rng = np.random.default_rng(seed)
    deck, path, dt = richards_deck(W, name, m, curve, seed, lumping)
    # partly unsaturated: pressures on both sides of zero
    p_old = rng.uniform(-3e4, 1e4, m.n_nodes)
    p_it = p_old + rng.uniform(-5e3, 5e3, m.n_nodes)
    R.write_doubles(path + ".p0", p_old)
    R.write_doubles(path + ".p1", p_it)
    R.run(R.REF_SP, path, ["step 1 %r" % dt, "nodal 0 0 %s.p0" % path, "nodal 0 1 %s.p1" % path,
                           "assemble 0 %s.sys" % path])
    s = R.read_system(path + ".sys")
    gravity = m.dim == 3
    p = params(pcs_type=3, dt=dt, storage=1e-6, porosity=0.35, viscosity=1e-3, density=1000.0,
               gravity=GRAVITY, gravity_on=int(gravity), mass_lumping=int(lumping))
    W.add(name, m, 3, p, dict(elem_k=deck.elem_k, p_old=p_old, p_iter=p_it, row_ptr=s["row_ptr"],
                              col=s["col"], val=s["val"], b=s["b"]),
          meta={"richards": richards_params_of(curve)})


def richards_picard_case(W, name, kind, curve, seed, error_method, relax):
    m = base_mesh(kind)
    rng = np.random.default_rng(seed)
    axis = 1 if m.dim == 2 else 2
    c = (m.x, m.y, m.z)[axis]
    top = np.nonzero(c == c.max())[0]
    bottom = np.nonzero(c == c.min())[0]
    bc = [("RICHARDS_FLOW", "PRESSURE1", top, -2.0e4), ("RICHARDS_FLOW", "PRESSURE1", bottom, 5.0e3)]
    nl = ("PICARD", error_method, 40, relax, 1e-3 if error_method != "LMAX" else 1e-2)
    deck, path, dt = richards_deck(W, name, m, curve, seed, False, bc=bc, nonlinear=nl)
    p_old = rng.uniform(-1.5e4, -5e3, m.n_nodes)
    p_old[top] = -2.0e4
    p_old[bottom] = 5.0e3
    R.write_doubles(path + ".p0", p_old)
    R.run(R.REF_SP, path, ["step 1 %r" % dt, "nodal 0 2 %s.p0" % path, "nonlinear 0 %s.res" % path])
    raw = np.fromfile(path + ".res", dtype=np.int64, count=2)
    x = np.fromfile(path + ".res", dtype=np.float64, offset=16)
    gravity = m.dim == 3
    p = params(pcs_type=3, dt=dt, storage=1e-6, porosity=0.35, viscosity=1e-3, density=1000.0,
               gravity=GRAVITY, gravity_on=int(gravity),
               nls_relaxation=relax)
    rows = np.concatenate([top, bottom])
    vals = np.concatenate([np.full(len(top), -2.0e4), np.full(len(bottom), 5.0e3)])
    W.add(name, m, 3, p, dict(elem_k=deck.elem_k, p_old=p_old, bc_rows=rows, bc_vals=vals,
                              iterations=raw[0], p_new=x),
          meta={"richards": richards_params_of(curve),
                "picard": {"error_method": error_method, "max_iterations": nl[2],
                           "tolerance": nl[4], "linear_tol": 1e-14}})


def solve_case(W, name, kind, binary, ls_method, precond, storage, transient=True):
    """A GROUNDWATER_FLOW step with Dirichlet heads on the two x faces, solved
    by the reference: the SP build (Linear_EQS: row-only Diagonize, its CG or
    BiCGStab) through CRFProcess::Execute, or the legacy FEM build (MXRandbed
    symmetric elimination, SpCG / SpBICGSTAB with diagonal scaling or the
    M34Vorkond incomplete LDU) through the same call."""
    m = base_mesh(kind) if kind != "hex" else M.structured_hex(6, 4, 3, 1.0, 2.0, 0.5)
    rng = np.random.default_rng(len(name))
    dt = 3600.0
    ek = k_field(m, len(name) + 5)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    bc = [("GROUNDWATER_FLOW", "HEAD", lf, 10.0), ("GROUNDWATER_FLOW", "HEAD", rf, 0.0)]
    proc = R.Process("GROUNDWATER_FLOW", dt=dt, ls_method=ls_method, precond=precond, storage=storage,
                     ls_tol=1e-14, ls_max_iter=20000)
    Ss = 1e-4 if transient else 0.0
    deck = R.Deck(mesh=m, processes=[proc], medium=R.Medium(dim=m.dim, storage=Ss), elem_k=ek, bc=bc)
    path = R.write(deck, W.deck_dir(name))
    u0 = rng.uniform(0, 10, m.n_nodes)
    u0[lf], u0[rf] = 10.0, 0.0
    R.write_doubles(path + ".u0", u0)
    legacy = binary == R.REF_FEM
    R.run(binary, path, ["step 1 %r" % dt, "nodal 0 2 %s.u0" % path,
                         ("legacy_execute 0 %s.res" if legacy else "execute 0 %s.res") % path])
    if legacy:
        iters = int(np.fromfile(path + ".res", dtype=np.int64, count=1)[0])
        x = np.fromfile(path + ".res", dtype=np.float64, offset=8)
    else:
        s = R.read_system(path + ".res", with_x=True)
        iters, x = s["iterations"], s["x"]
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    p = params(pcs_type=0, dt=dt, storage=Ss)
    W.add(name, m, 3, p, dict(elem_k=ek, u0=u0, bc_rows=rows, bc_vals=vals, x_ref=x, iterations=iters),
          meta={"solve": {"build": "FEM" if legacy else "SP", "ls_method": ls_method, "precond": precond,
                          "dirichlet": "symmetric" if legacy else "row_only", "tol": 1e-14}})


def main():
    if not os.path.exists(R.REF_SP):
        sys.exit("build the reference first: make -C oracle -f refbuild.mk -j8")
    W = Writer()
    seed = 100
    for kind in ("quad", "hex", "tet"):
        for geom in ("box", "sheared", "distorted"):
            seed += 1
            flow_case(W, f"gwf_{kind}_{geom}", kind, geom, "GROUNDWATER_FLOW", seed)
            flow_case(W, f"liquid_{kind}_{geom}", kind, geom, "LIQUID_FLOW", seed + 50)
            transport_case(W, f"mt_{kind}_{geom}", kind, geom, seed + 70, decay=1e-7, kd=2e-4)
            velocity_case(W, f"vel_gwf_{kind}_{geom}", kind, geom, "GROUNDWATER_FLOW", seed + 80)
        seed += 1
        flow_case(W, f"gwf_steady_{kind}", kind, "distorted", "GROUNDWATER_FLOW", seed, steady=True)
        flow_case(W, f"gwf_lumped_{kind}_box", kind, "box", "GROUNDWATER_FLOW", seed, lumping=True)
        flow_case(W, f"gwf_lumped_{kind}_distorted", kind, "distorted", "GROUNDWATER_FLOW", seed,
                  lumping=True)
        flow_case(W, f"gwf_relax_{kind}", kind, "sheared", "GROUNDWATER_FLOW", seed, relax=0.6)
        if kind != "tet":
            flow_case(W, f"gwf_gauss2_{kind}", kind, "distorted", "GROUNDWATER_FLOW", seed, ngauss=2)
        flow_case(W, f"liquid_drho_{kind}", kind, "distorted", "LIQUID_FLOW", seed, liquid_drho=True)
        flow_case(W, f"liquid_lumped_{kind}", kind, "box", "LIQUID_FLOW", seed, lumping=True)
        velocity_case(W, f"vel_liquid_{kind}", kind, "distorted", "LIQUID_FLOW", seed + 90)
        transport_case(W, f"mt_lumped_{kind}", kind, "distorted", seed + 3, lumping=True)
        for i, sp in enumerate(((1, 0, 0), (2, 1, 1), (1, 2, 2))):
            transport_case(W, f"mt_supg{i}_{kind}", kind, "distorted" if i else "box", seed + 4 + i,
                           supg=sp)
        transport_case(W, f"mt_memory_{kind}", kind, "sheared", seed + 9, memory=True)
        transport_case(W, f"mt_memory_lumped_{kind}", kind, "box", seed + 10, memory=True, lumping=True)
        for curve in ("vg", "bc"):
            richards_assembly_case(W, f"rich_{curve}_{kind}", kind, "distorted", curve, seed + 11)
            richards_assembly_case(W, f"rich_{curve}_lumped_{kind}", kind, "box", curve, seed + 12,
                                   lumping=True)
        richards_picard_case(W, f"picard_vg_{kind}", kind, "vg", seed + 13, "ERNORM", 0.0)
        richards_picard_case(W, f"picard_bc_{kind}", kind, "bc", seed + 14, "LMAX", 0.0)
    for kind in ("quad", "hex", "tet"):
        # legacy RF build: MXRandbed + SpCG unpreconditioned (vorkond 0; its
        # diagonal scaling, vorkond 1, scales rows to D^-1 A, which is not
        # symmetric, and SpCG then stalls on these heterogeneous decks), and
        # the M34Vorkond incomplete LDU (storage 4, vorkond 100) under SpCG
        # and SpBICGSTAB
        solve_case(W, f"legacy_cg_plain_{kind}", kind, R.REF_FEM, 5, 0, 2)
        solve_case(W, f"legacy_cg_ilu_{kind}", kind, R.REF_FEM, 5, 100, 4)
        solve_case(W, f"legacy_bicgstab_ilu_{kind}", kind, R.REF_FEM, 2, 100, 4)
        # SP build: Diagonize (row only) + Linear_EQS::BiCGStab with Jacobi
        solve_case(W, f"sp_bicgstab_jacobi_{kind}", kind, R.REF_SP, 2, 1, 100)
    W.out["cases"] = np.array(json.dumps(W.names))
    np.savez_compressed(os.path.join(HERE, "ref_assembly.npz"), **W.out)
    print(len(W.names), "cases")


if __name__ == "__main__":
    main()
