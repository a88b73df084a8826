"""Complete OGS-5 input decks for the reference build, and a runner for its
harness (``oracle/_ref/ref_assemble_{sp,fem}``, built by
``oracle/refbuild.mk``).  TEST INFRASTRUCTURE ONLY: used by the scripts that
write the golden fixtures of this folder, never by the product or by the
tests at run time (the reference is not present where the GPU tests run).

A deck is the set of files the reference's Problem constructor reads
(FEM/problem.cpp:120 -> ReadData): .pcs (PCSRead, FEM/rf_pcs.cpp:1963-2320),
.num (NUMRead, FEM/rf_num_new.cpp:382-712), .tim (TIMRead), .mmp (MMPRead,
FEM/rf_mmp_new.cpp:317-2110), .mfp (MFPRead, FEM/rf_mfp_new.cpp), .mcp
(CPRead, FEM/rfmat_cp.cpp:322-680), .msh, .ic, .bc and, for element-wise
conductivity, a #MEDIUM_PROPERTIES_DISTRIBUTED file with $DIS_TYPE ELEMENT
(CMediumProperties::SetDistributedELEProperties, rf_mmp_new.cpp:5740-5930).
Numbers are written with 17 significant digits, so every double reaches the
reference unchanged.
"""
from __future__ import annotations

import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

from ogs5_gb300 import deck as D
from ogs5_gb300 import mesh as M

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_SP = os.path.join(ROOT, "oracle", "_ref", "ref_assemble_sp")
REF_FEM = os.path.join(ROOT, "oracle", "_ref", "ref_assemble_fem")

PRIMARY = {"GROUNDWATER_FLOW": "HEAD", "LIQUID_FLOW": "PRESSURE1", "RICHARDS_FLOW": "PRESSURE1",
           "MASS_TRANSPORT": "Conc"}


def g(v: float) -> str:
    return "%.17g" % v


@dataclass
class Process:
    """One #PROCESS block with its numerics and time stepping."""
    pcs: str
    steady: bool = False
    dt: float = 1.0
    # $LINEAR_SOLVER: method error_method tol max_iter theta precond storage
    ls_method: int = 2
    ls_tol: float = 1e-12
    ls_max_iter: int = 1000
    theta: float = 1.0
    precond: int = 1
    storage: int = 100          # CRS: the SparseTable storage Write_BIN needs
    gauss_points: int = 3
    mass_lumping: int = 0
    supg: tuple | None = None   # (method, length, diffusivity)
    memory_type: int = 0
    # $NON_LINEAR_ITERATIONS: method error_method max_iter relaxation tol
    nonlinear: tuple | None = None
    initial: float = 0.0


@dataclass
class Medium:
    dim: int
    porosity: float = 0.3
    tortuosity: float = 1.0
    storage: float = 0.0
    permeability: float = 1.0   # overridden by the element field when given
    alpha_l: float | None = None
    alpha_t: float | None = None
    capillary: tuple | None = None      # (model, pb, slr, slm, m)
    rel_perm: tuple | None = None       # (model, slr, slm, m, kr_min)


@dataclass
class Fluid:
    density: float = 1000.0
    drho_dp: float = 0.0        # density model 2 when non-zero
    p0: float = 0.0
    viscosity: float = 1.0
    gravity: bool = False


@dataclass
class Component:
    diffusion: float = 0.0      # $DIFFUSION 1 Daq (multiplied by tortuosity)
    decay: float | None = None  # $DECAY 1 lambda 1 (first order)
    kd: float | None = None     # $ISOTHERM 1 Kd (linear sorption)
    solid_density: float = 2000.0  # .msp $DENSITY 1 rho_s

    def retardation(self, porosity: float) -> float:
        """CompProperties::CalcElementRetardationFactorNew for a linear
        isotherm (FEM/rfmat_cp.cpp:1575-1580)."""
        if self.kd is None:
            return 1.0
        return 1.0 + (1.0 - porosity) * self.solid_density * self.kd / porosity


@dataclass
class Deck:
    mesh: M.Mesh
    processes: list
    medium: Medium
    fluid: Fluid = field(default_factory=Fluid)
    component: Component | None = None
    elem_k: np.ndarray | None = None
    bc: list = field(default_factory=list)   # [(pcs, pv, rows, value)] as node POINTs


def write(deck: Deck, dirpath: str, base: str = "deck") -> str:
    """Writes the deck files; returns the base path the reference opens."""
    os.makedirs(dirpath, exist_ok=True)
    path = os.path.join(dirpath, base)
    m = deck.mesh
    D.write_msh(m, path + ".msh")
    with open(path + ".pcs", "w") as f:
        for p in deck.processes:
            f.write("#PROCESS\n $PCS_TYPE\n  %s\n $NUM_TYPE\n  NEW\n" % p.pcs)
            if p.pcs == "MASS_TRANSPORT":
                f.write(" $PRIMARY_VARIABLE\n  %s\n" % PRIMARY[p.pcs])
            if p.steady:
                f.write(" $TIM_TYPE\n  STEADY\n")
            if p.memory_type:
                f.write(" $MEMORY_TYPE\n  %d\n" % p.memory_type)
        f.write("#STOP\n")
    with open(path + ".num", "w") as f:
        for p in deck.processes:
            f.write("#NUMERICS\n $PCS_TYPE\n  %s\n" % p.pcs)
            f.write(" $LINEAR_SOLVER\n  %d 1 %s %d %s %d %d\n"
                    % (p.ls_method, g(p.ls_tol), p.ls_max_iter, g(p.theta), p.precond, p.storage))
            f.write(" $ELE_GAUSS_POINTS\n  %d\n" % p.gauss_points)
            if p.mass_lumping:
                f.write(" $ELE_MASS_LUMPING\n  1\n")
            if p.supg:
                f.write(" $ELE_SUPG\n  %d %d %d\n" % p.supg)
            if p.nonlinear:
                meth, err, it, relax, tol = p.nonlinear
                f.write(" $NON_LINEAR_ITERATIONS\n  %s %s %d %s %s\n" % (meth, err, it, g(relax), g(tol)))
        f.write("#STOP\n")
    with open(path + ".tim", "w") as f:
        for p in deck.processes:
            f.write("#TIME_STEPPING\n $PCS_TYPE\n  %s\n $TIME_START\n  0\n $TIME_END\n  %s\n"
                    " $TIME_STEPS\n  1 %s\n" % (p.pcs, g(p.dt), g(p.dt)))
        f.write("#STOP\n")
    md = deck.medium
    with open(path + ".mmp", "w") as f:
        f.write("#MEDIUM_PROPERTIES\n $GEOMETRY_DIMENSION\n  %d\n $GEOMETRY_AREA\n  1.0\n" % md.dim)
        f.write(" $POROSITY\n  1 %s\n $TORTUOSITY\n  1 %s\n" % (g(md.porosity), g(md.tortuosity)))
        f.write(" $STORAGE\n  1 %s\n" % g(md.storage))
        f.write(" $PERMEABILITY_TENSOR\n  ISOTROPIC %s\n" % g(md.permeability))
        if deck.elem_k is not None:
            f.write(" $PERMEABILITY_DISTRIBUTION\n  %s.kdist\n" % base)
        if md.alpha_l is not None:
            f.write(" $MASS_DISPERSION\n  1 %s %s\n" % (g(md.alpha_l), g(md.alpha_t)))
        if md.capillary is not None:
            f.write(" $CAPILLARY_PRESSURE\n  %d %s\n" % (md.capillary[0],
                                                         " ".join(g(v) for v in md.capillary[1:])))
        if md.rel_perm is not None:
            f.write(" $PERMEABILITY_SATURATION\n  %d %s\n" % (md.rel_perm[0],
                                                              " ".join(g(v) for v in md.rel_perm[1:])))
        f.write("#STOP\n")
    if deck.elem_k is not None:
        with open(path + ".kdist", "w") as f:
            f.write("#MEDIUM_PROPERTIES_DISTRIBUTED\n $MSH_TYPE\n  %s\n $MMP_TYPE\n  PERMEABILITY\n"
                    " $DIS_TYPE\n  ELEMENT\n $DATA\n" % deck.processes[0].pcs)
            for e, k in enumerate(np.asarray(deck.elem_k, dtype=np.float64)):
                f.write("%d %s\n" % (e, g(k)))
            f.write("#STOP\n")
    fl = deck.fluid
    with open(path + ".mfp", "w") as f:
        f.write("#FLUID_PROPERTIES\n $FLUID_TYPE\n  LIQUID\n $PCS_TYPE\n  PRESSURE1\n")
        if fl.drho_dp != 0.0:
            f.write(" $DENSITY\n  2 %s %s %s\n" % (g(fl.density), g(fl.p0), g(fl.drho_dp)))
        else:
            f.write(" $DENSITY\n  1 %s\n" % g(fl.density))
        f.write(" $VISCOSITY\n  1 %s\n" % g(fl.viscosity))
        if not fl.gravity:
            f.write(" $NON_GRAVITY\n")
        f.write("#STOP\n")
    if deck.component is not None:
        c = deck.component
        with open(path + ".mcp", "w") as f:
            f.write("#COMPONENT_PROPERTIES\n $NAME\n  %s\n $MOBILE\n  1\n $DIFFUSION\n  1 %s\n"
                    % (PRIMARY["MASS_TRANSPORT"], g(c.diffusion)))
            if c.decay is not None:
                f.write(" $DECAY\n  1 %s 1\n" % g(c.decay))
            if c.kd is not None:
                f.write(" $ISOTHERM\n  1 %s\n" % g(c.kd))
            f.write("#STOP\n")
        with open(path + ".msp", "w") as f:
            f.write("#SOLID_PROPERTIES\n $DENSITY\n  1 %s\n#STOP\n" % g(c.solid_density))
    with open(path + ".ic", "w") as f:
        for p in deck.processes:
            f.write("#INITIAL_CONDITION\n $PCS_TYPE\n  %s\n $PRIMARY_VARIABLE\n  %s\n"
                    " $GEO_TYPE\n  DOMAIN\n $DIS_TYPE\n  CONSTANT %s\n"
                    % (p.pcs, PRIMARY[p.pcs], g(p.initial)))
        f.write("#STOP\n")
    points = []
    conds = []
    for pcs, pv, rows, value in deck.bc:
        for r in np.asarray(rows, dtype=np.int64):
            name = "P%d" % len(points)
            points.append((m.x[r], m.y[r], m.z[r], name))
            conds.append((pcs, pv, "POINT", name, value))
    D.write_gli(path + ".gli", points if points else [(m.x[0], m.y[0], m.z[0], "P0")])
    D.write_bc(path + ".bc", conds)
    return path


# Address-space cap of one reference run: the decks here need well under
# 1 GB, and a deck the reference misreads can otherwise allocate without
# bound.
MEMORY_LIMIT_BYTES = 4 << 30


def _limit_memory():
    import resource
    resource.setrlimit(resource.RLIMIT_AS, (MEMORY_LIMIT_BYTES, MEMORY_LIMIT_BYTES))


def run(binary: str, deck_path: str, commands: list, timeout: float = 600.0) -> str:
    """Runs the harness on a deck; commands are the harness's lines.  Returns
    the combined output (the reference prints its progress).  Results must
    not use an extension the reference reads as input (.out is its output
    definition file): the scripts here write .res, .sys and raw arrays."""
    cmd_file = deck_path + ".cmd"
    with open(cmd_file, "w") as f:
        f.write("\n".join(commands) + "\n")
    r = subprocess.run([binary, deck_path, cmd_file], capture_output=True, text=True,
                       timeout=timeout, cwd=os.path.dirname(deck_path), preexec_fn=_limit_memory)
    if r.returncode != 0:
        raise RuntimeError("reference harness failed (%d):\n%s\n%s" % (r.returncode, r.stdout[-4000:],
                                                                       r.stderr[-4000:]))
    return r.stdout


def read_system(path: str, with_x: bool = False):
    """Reads Linear_EQS::Write_BIN output (DOF 1): rows, row_ptr, col, val, b
    [, then the harness's int64 iterations and x of an `execute`]."""
    raw = open(path, "rb").read()
    rows = int(np.frombuffer(raw, dtype=np.int64, count=1)[0])
    off = 8
    rp = np.frombuffer(raw, dtype=np.int64, count=rows + 1, offset=off)
    off += 8 * (rows + 1)
    nnz = int(rp[-1])
    col = np.frombuffer(raw, dtype=np.int64, count=nnz, offset=off)
    off += 8 * nnz
    val = np.frombuffer(raw, dtype=np.float64, count=nnz, offset=off)
    off += 8 * nnz
    b = np.frombuffer(raw, dtype=np.float64, count=rows, offset=off)
    off += 8 * rows
    out = {"row_ptr": rp.copy(), "col": col.copy(), "val": val.copy(), "b": b.copy()}
    if with_x:
        out["iterations"] = int(np.frombuffer(raw, dtype=np.int64, count=1, offset=off)[0])
        out["x"] = np.frombuffer(raw, dtype=np.float64, count=rows, offset=off + 8).copy()
    return out


def write_doubles(path: str, v) -> str:
    np.ascontiguousarray(v, dtype=np.float64).tofile(path)
    return path
