"""Structured synthetic meshes in OGS-5 element node order.

OGS-5 reads meshes from ``.msh`` files (CFEMesh::Read, MSH/msh_mesh.cpp:421);
the synthetic decks here are generated in memory instead.  Node numbering is
lexicographic (x fastest), which is also the equation numbering of
CFEMesh::RenumberNodesForGlobalAssembly for linear meshes.  Element node
order follows CElem: quads counter-clockwise, hexes bottom face then top
face, tets from the Kuhn split of each hex along its (0,0,0)-(1,1,1)
diagonal (six tets per hex, element 6*h + t belongs to hex h).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from itertools import permutations

import numpy as np

QUAD4, HEX8, TET4 = 0, 1, 2
NODES_PER_ELEMENT = {QUAD4: 4, HEX8: 8, TET4: 4}


@dataclass
class Mesh:
    elem_type: int
    dim: int
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    conn: np.ndarray          # int32 [n_elements, nodes_per_element]
    shape: tuple = ()         # structured cells per axis
    spacing: tuple = ()
    extra: dict = field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return int(self.x.shape[0])

    @property
    def n_elements(self) -> int:
        return int(self.conn.shape[0])

    @property
    def nodes_per_element(self) -> int:
        return int(self.conn.shape[1])

    def face_nodes(self, axis: int, side: int) -> np.ndarray:
        """Node ids on the structured boundary plane axis = 0 (side 0) or max (side 1)."""
        coords = (self.x, self.y, self.z)[axis]
        target = coords.min() if side == 0 else coords.max()
        return np.nonzero(coords == target)[0].astype(np.int64)


def structured_quad(nx: int, ny: int, dx: float = 1.0, dy: float = 1.0) -> Mesh:
    i = np.arange(nx + 1)
    j = np.arange(ny + 1)
    X, Y = np.meshgrid(i * dx, j * dy, indexing="xy")
    nid = lambda a, b: a + (nx + 1) * b  # noqa: E731
    ei, ej = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    ei, ej = ei.ravel(), ej.ravel()
    conn = np.stack([nid(ei, ej), nid(ei + 1, ej), nid(ei + 1, ej + 1), nid(ei, ej + 1)], axis=1)
    n = (nx + 1) * (ny + 1)
    return Mesh(QUAD4, 2, X.ravel().astype(np.float64), Y.ravel().astype(np.float64),
                np.zeros(n), conn.astype(np.int32), (nx, ny), (dx, dy))


def _hex_node_grid(nx, ny, nz, dx, dy, dz):
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    return (i.ravel() * dx).astype(np.float64), (j.ravel() * dy).astype(np.float64), \
        (k.ravel() * dz).astype(np.float64)


def structured_hex(nx: int, ny: int, nz: int, dx: float = 1.0, dy: float = 1.0,
                   dz: float = 1.0) -> Mesh:
    x, y, z = _hex_node_grid(nx, ny, nz, dx, dy, dz)
    nid = lambda a, b, c: a + (nx + 1) * (b + (ny + 1) * c)  # noqa: E731
    ek, ej, ei = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ei, ej, ek = ei.ravel(), ej.ravel(), ek.ravel()
    conn = np.stack([nid(ei, ej, ek), nid(ei + 1, ej, ek), nid(ei + 1, ej + 1, ek),
                     nid(ei, ej + 1, ek), nid(ei, ej, ek + 1), nid(ei + 1, ej, ek + 1),
                     nid(ei + 1, ej + 1, ek + 1), nid(ei, ej + 1, ek + 1)], axis=1)
    return Mesh(HEX8, 3, x, y, z, conn.astype(np.int32), (nx, ny, nz), (dx, dy, dz))


# hex corner (a,b,c) -> position in the OGS hex node order used above
_HEX_CORNER = {(0, 0, 0): 0, (1, 0, 0): 1, (1, 1, 0): 2, (0, 1, 0): 3,
               (0, 0, 1): 4, (1, 0, 1): 5, (1, 1, 1): 6, (0, 1, 1): 7}


def _kuhn_tets():
    tets = []
    for perm in permutations(range(3)):
        v = [0, 0, 0]
        path = [_HEX_CORNER[tuple(v)]]
        for ax in perm:
            v[ax] = 1
            path.append(_HEX_CORNER[tuple(v)])
        tets.append(path)
    return np.array(tets, dtype=np.int64)  # [6, 4] local hex corners


KUHN_TETS = _kuhn_tets()


def hex_to_tet(h: Mesh) -> Mesh:
    """Six Kuhn tets per hex; element 6*e + t comes from hex e."""
    conn = h.conn[:, KUHN_TETS].reshape(-1, 4)
    return Mesh(TET4, 3, h.x, h.y, h.z, conn.astype(np.int32), h.shape, h.spacing,
                {"parent_hex": True})


def structured_tet(nx: int, ny: int, nz: int, dx=1.0, dy=1.0, dz=1.0) -> Mesh:
    return hex_to_tet(structured_hex(nx, ny, nz, dx, dy, dz))
