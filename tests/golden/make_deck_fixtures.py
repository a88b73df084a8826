"""Writes the deck fixtures of tests/golden/deck/ from the reference.

Run where the reference sources exist:

    python tests/golden/make_deck_fixtures.py [/path/to/reference]

Fixtures:
  deck/bmskel.msh, .gli, .bc
        the reference's benchmark skeleton deck (tests/data/bmskel/a.msh,
        a.gli, a.bc), copied unchanged: a two-node line mesh with a
        CONSTANT 274 condition on POINT0.
  deck/point_in_polygon.gli
        the reference's polygon of GEO::PointInPolygon
        (tests/data/GEO/TestDataPointInPolygon.gli), copied unchanged.
  deck_node_sets.npz
        node sets the reference's own GEOLIB code (oracle/_ref/libogs5geo.so)
        selects on the meshes that :func:`jittered_tet_deck` and
        :func:`polygon_grid_nodes` build: polylines at three search radii
        (MeshNodesAlongPolyline order), surfaces at two search lengths
        (GetNODOnSFC), and the point-in-polygon mask of the GEO test grid.
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DECK = os.path.join(HERE, "deck")
NODE_SETS = os.path.join(HERE, "deck_node_sets.npz")

POLYLINE_RADII = (0.01, 0.2, 0.6)
SURFACE_EPS = (None, 0.05, 0.2, 0.6)  # None: 0.375 * h_min / 2; 0.2 and 0.6 reach past the mesh spacing


def jittered_tet_deck():
    """A 12x10x8 Kuhn-tet mesh of spacing 0.5 whose interior nodes are moved
    by up to 0.1 (seeded), with polylines (straight, bent, along edges) and
    planar surfaces (tilted quad, triangle, bottom face, L-shaped top)."""
    from ogs5_gb300 import mesh as M
    rng = np.random.default_rng(0)
    m = M.structured_tet(12, 10, 8, 0.5, 0.5, 0.5)
    inner = (m.x > 0) & (m.x < 6) & (m.y > 0) & (m.y < 5) & (m.z > 0) & (m.z < 4)
    m.x = m.x + inner * rng.uniform(-0.1, 0.1, m.n_nodes)
    m.y = m.y + inner * rng.uniform(-0.1, 0.1, m.n_nodes)
    m.z = m.z + inner * rng.uniform(-0.1, 0.1, m.n_nodes)
    polylines = {
        "diag": [[0, 0, 0], [6, 5, 4.0]],
        "bent": [[0.3, 0.2, 0.1], [3.1, 2.2, 1.7], [5.9, 0.4, 3.3], [2.0, 4.9, 3.9]],
        "edge": [[0, 0, 0], [6, 0, 0], [6, 5, 0]],
    }
    surfaces = {
        "tilt": [[0, 0, 0], [6, 0, 2.0], [6, 5, 2.0], [0, 5, 0]],
        "tri": [[0.5, 0.5, 1.0], [5.5, 1.0, 3.0], [2.0, 4.5, 2.0]],
        "face": [[0, 0, 0], [6, 0, 0], [6, 5, 0], [0, 5, 0]],
        "lshape": [[0, 0, 4], [6, 0, 4], [6, 2, 4], [2, 2, 4], [2, 5, 4], [0, 5, 4]],
    }
    return m, polylines, surfaces


def read_gli_polygon(path):
    """Points of the first polyline of a .gli file, in polyline order."""
    pts, ids, mode = [], [], None
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0].startswith("#"):
                mode = t[0]
                continue
            if mode == "#POINTS":
                pts.append([float(v) for v in t[1:4]])
            elif mode == "#POLYLINE" and t[0].lstrip("-").isdigit():
                ids.append(int(t[0]))
    P = np.array(pts)[ids]
    return P[:-1] if np.array_equal(P[0], P[-1]) else P


def polygon_grid_nodes():
    """The 920 x 320 test points of GEO::PointInPolygon
    (tests/GEO/TestPointInPolygon.cpp:39-46), j-major."""
    k = np.tile(np.arange(920), 320)
    j = np.repeat(np.arange(320), 920)
    return 0.9 + k / 100.0, -1.1 + j / 100.0


def min_edge(m):
    from ogs5_gb300 import mesh as M
    edges = {M.TET4: [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]}[m.elem_type]
    X = np.stack([m.x, m.y, m.z], 1)
    return min(np.linalg.norm(X[m.conn[:, a]] - X[m.conn[:, b]], axis=1).min() for a, b in edges)


def main(ref_dir):
    from oracle import oracle as O
    O.build(ref_dir)
    os.makedirs(DECK, exist_ok=True)
    for ext in ("msh", "gli", "bc"):
        shutil.copyfile(os.path.join(ref_dir, "tests", "data", "bmskel", "a." + ext),
                        os.path.join(DECK, "bmskel." + ext))
    shutil.copyfile(os.path.join(ref_dir, "tests", "data", "GEO", "TestDataPointInPolygon.gli"),
                    os.path.join(DECK, "point_in_polygon.gli"))
    out = {}
    m, polylines, surfaces = jittered_tet_deck()
    X = np.stack([m.x, m.y, m.z], 1)
    h = min_edge(m)
    for r in POLYLINE_RADII:
        for name, P in polylines.items():
            ids, dist = O.ref_polyline_nodes(P, X, r)
            out[f"ply_{name}_{r}"] = ids
            out[f"plydist_{name}_{r}"] = dist
    for eps in SURFACE_EPS:
        e = 0.375 * h / 2 if eps is None else eps
        for name, P in surfaces.items():
            out[f"sfc_{name}_{eps}"] = O.ref_surface_nodes(P, X, e)
    poly = read_gli_polygon(os.path.join(DECK, "point_in_polygon.gli"))
    gx, gy = polygon_grid_nodes()
    G = np.stack([gx, gy, np.zeros_like(gx)], 1)
    out["pip_mask"] = np.packbits(O.ref_point_in_polygon(poly, G))
    sfc = np.zeros(len(G), dtype=bool)
    sfc[O.ref_surface_nodes(poly, G, 0.375 * 0.01 / 2)] = True
    out["pip_surface_mask"] = np.packbits(sfc)
    np.savez_compressed(NODE_SETS, **out)
    print("wrote", NODE_SETS, "and", DECK)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
