"""Writers of OGS-5 input decks: mesh (.msh), geometry (.gli) and constant
Dirichlet conditions (.bc), in the text layout the OGS-5 readers take
(CFEMesh::Read, MSH/msh_mesh.cpp:421-495; readGLIFileV4,
FileIO/OGSIOVer4.cpp:54-503; CBoundaryCondition::Read,
FEM/rf_bc_new.cpp:250-560).  The reader is native: :class:`ogs5_gb300.capi.Deck`.
"""
from __future__ import annotations

import numpy as np

from . import mesh as M

ELEM_NAMES = {M.QUAD4: "quad", M.HEX8: "hex", M.TET4: "tet"}


def write_msh(mesh: M.Mesh, path: str) -> None:
    """One #FEM_MSH block: $NODES "i x y z", $ELEMENTS "i 0 type nodes"."""
    name = ELEM_NAMES[mesh.elem_type]
    with open(path, "w") as f:
        f.write("#FEM_MSH\n $PCS_TYPE\n  NO_PCS\n $NODES\n  %d\n" % mesh.n_nodes)
        for i in range(mesh.n_nodes):
            f.write("%d %.17g %.17g %.17g\n" % (i, mesh.x[i], mesh.y[i], mesh.z[i]))
        f.write(" $ELEMENTS\n  %d\n" % mesh.n_elements)
        for e, nodes in enumerate(np.asarray(mesh.conn)):
            f.write("%d 0 %s %s\n" % (e, name, " ".join(str(int(v)) for v in nodes)))
        f.write("#STOP\n")


def write_gli(path: str, points, polylines=None, surfaces=None) -> None:
    """points: [(x, y, z) or (x, y, z, name)]; polylines: {name: ([point
    indices], epsilon or None)}; surfaces: {name: [polyline names]}.  Point
    ids are zero-based.  A point name is followed by a space: the reference's
    readPoints registers a name only up to the next blank
    (FileIO/OGSIOVer4.cpp:92-97)."""
    with open(path, "w") as f:
        f.write("#POINTS\n")
        for i, p in enumerate(points):
            f.write("%d %.17g %.17g %.17g" % (i, p[0], p[1], p[2]))
            f.write(" $NAME %s \n" % p[3] if len(p) > 3 else "\n")
        for name, (ids, eps) in (polylines or {}).items():
            f.write("#POLYLINE\n $NAME\n  %s\n" % name)
            if eps is not None:
                f.write(" $EPSILON\n  %.17g\n" % eps)
            f.write(" $POINTS\n")
            for i in ids:
                f.write("  %d\n" % i)
        for name, plys in (surfaces or {}).items():
            f.write("#SURFACE\n $NAME\n  %s\n $TYPE\n  0\n $POLYLINES\n" % name)
            for p in plys:
                f.write("  %s\n" % p)
        f.write("#STOP\n")


def write_bc(path: str, conditions) -> None:
    """conditions: [(pcs_type, primary_variable, geo_type, geo_name, value)
    or the same with a sixth entry, the $EPSILON of the condition]."""
    with open(path, "w") as f:
        for c in conditions:
            pcs, pv, gt, gn, val = c[:5]
            f.write("#BOUNDARY_CONDITION\n $PCS_TYPE\n  %s\n $PRIMARY_VARIABLE\n  %s\n"
                    " $GEO_TYPE\n  %s %s\n $DIS_TYPE\n  CONSTANT %.17g\n" % (pcs, pv, gt, gn, val))
            if len(c) > 5:
                f.write(" $EPSILON\n  %.17g\n" % c[5])
        f.write("#STOP\n")
