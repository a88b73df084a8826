"""OGS-5 deck reader (ogs_deck_*, host code of libogs_gpu.so): .msh, .gli and
.bc files to the mesh description and Dirichlet rows of the GPU path.

Node searches are checked against node sets the reference's own GEOLIB code
selected (tests/golden/deck_node_sets.npz, made by make_deck_fixtures.py;
re-checked live against oracle/_ref/libogs5geo.so where it is built), and on
structured decks against the faces and edges they must select.
"""
import os

import numpy as np
import pytest

from ogs5_gb300 import capi
from ogs5_gb300 import deck as D
from ogs5_gb300 import mesh as M
from tests.golden import make_deck_fixtures as F

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def node_sets():
    return np.load(os.path.join(GOLDEN, "deck_node_sets.npz"))


@pytest.fixture(scope="module")
def tet_deck(tmp_path_factory):
    """The jittered tet deck written to disk: mesh, geometry with one
    polyline per search radius and one closed boundary per surface."""
    d = tmp_path_factory.mktemp("tetdeck")
    m, polylines, surfaces = F.jittered_tet_deck()
    D.write_msh(m, str(d / "t.msh"))
    pts, plys, sfcs = [], {}, {}
    for name, P in polylines.items():
        ids = list(range(len(pts), len(pts) + len(P)))
        pts += [tuple(p) for p in P]
        for r in F.POLYLINE_RADII:
            plys[f"{name}_{r}"] = (ids, r)
    for name, P in surfaces.items():
        ids = list(range(len(pts), len(pts) + len(P)))
        pts += [tuple(p) for p in P]
        plys[name + "_boundary"] = (ids + [ids[0]], None)
        sfcs[name] = [name + "_boundary"]
    D.write_gli(str(d / "t.gli"), pts, plys, sfcs)
    return d, m, polylines, surfaces


def test_bmskel_point_condition():
    """The reference's skeleton benchmark: a line mesh (read for its nodes,
    not assembled on the GPU) and CONSTANT 274 on POINT0 = node 0."""
    dk = capi.Deck(*(os.path.join(GOLDEN, "deck", "bmskel." + e) for e in ("msh", "gli", "bc")))
    rows, vals = dk.dirichlet("HEAT_TRANSPORT")
    assert rows.tolist() == [0] and vals.tolist() == [274.0]
    assert dk.dirichlet("HEAT_TRANSPORT", "TEMPERATURE1")[0].tolist() == [0]
    assert len(dk.dirichlet("HEAT_TRANSPORT", "PRESSURE1")[0]) == 0
    assert len(dk.dirichlet("GROUNDWATER_FLOW")[0]) == 0
    assert dk.min_edge_length == pytest.approx(1.0)
    with pytest.raises(capi.OgsError, match="not on the GPU path"):
        dk.mesh


def test_polylines_match_reference(tet_deck, node_sets):
    d, m, polylines, _ = tet_deck
    dk = capi.Deck(str(d / "t.msh"), str(d / "t.gli"))
    for r in F.POLYLINE_RADII:
        for name in polylines:
            # a CONSTANT condition takes the nodes sorted by index
            ref = node_sets[f"ply_{name}_{r}"]
            got = dk.geo_nodes("POLYLINE", f"{name}_{r}")
            assert got.tolist() == sorted(ref.tolist()), (name, r)


@pytest.mark.parametrize("eps", F.SURFACE_EPS)
def test_surfaces_match_reference(tet_deck, node_sets, eps):
    d, m, _, surfaces = tet_deck
    conds = [("GROUNDWATER_FLOW", "HEAD", "SURFACE", name, float(i)) + (() if eps is None else (eps,))
             for i, name in enumerate(surfaces)]
    D.write_bc(str(d / "t.bc"), conds)
    dk = capi.Deck(str(d / "t.msh"), str(d / "t.gli"), str(d / "t.bc"))
    rows, vals = dk.dirichlet("GROUNDWATER_FLOW")
    start = 0
    for i, name in enumerate(surfaces):
        ref = node_sets[f"sfc_{name}_{eps}"]
        assert rows[start:start + len(ref)].tolist() == ref.tolist(), name
        assert np.all(vals[start:start + len(ref)] == float(i))
        start += len(ref)
    assert start == len(rows)


def test_polygon_surface_matches_reference(tmp_path, node_sets):
    """The non-convex 17-gon of the reference's GEO::PointInPolygon test as a
    surface over a quad mesh whose nodes are that test's 294,400 points:
    the default search length selects exactly the reference's nodes."""
    poly = F.read_gli_polygon(os.path.join(GOLDEN, "deck", "point_in_polygon.gli"))
    gx, gy = F.polygon_grid_nodes()
    m = M.structured_quad(919, 319)
    m.x, m.y = gx, gy
    D.write_msh(m, str(tmp_path / "g.msh"))
    D.write_gli(str(tmp_path / "g.gli"), [tuple(p) for p in poly],
                {"ply": (list(range(len(poly))) + [0], None)}, {"S": ["ply"]})
    D.write_bc(str(tmp_path / "g.bc"), [("GROUNDWATER_FLOW", "HEAD", "SURFACE", "S", 1.0)])
    dk = capi.Deck(str(tmp_path / "g.msh"), str(tmp_path / "g.gli"), str(tmp_path / "g.bc"))
    assert dk.min_edge_length == pytest.approx(0.01, rel=1e-10)
    rows, _ = dk.dirichlet("GROUNDWATER_FLOW")
    want = np.flatnonzero(np.unpackbits(node_sets["pip_surface_mask"])[:len(gx)])
    assert len(want) == 95751
    assert np.array_equal(rows, want)
    # the polygon test's own known answer (tests/GEO/TestPointInPolygon.cpp:73):
    # 95,511 points in the polygon; the surface also takes points on its edges
    inside = np.unpackbits(node_sets["pip_mask"])[:len(gx)].astype(bool)
    assert inside.sum() == 95511
    assert np.all(np.isin(np.flatnonzero(inside), rows))


def test_reference_harness_reproduces_fixtures(node_sets):
    """Where the reference is built here, its geometry code still selects
    the committed node sets, and its polygon test answer is 95,511."""
    from oracle import oracle as O
    if not O.has_ref_geo():
        pytest.skip("reference geometry harness not built")
    m, polylines, surfaces = F.jittered_tet_deck()
    X = np.stack([m.x, m.y, m.z], 1)
    for name, P in polylines.items():
        ids, _ = O.ref_polyline_nodes(P, X, 0.2)
        assert ids.tolist() == node_sets[f"ply_{name}_0.2"].tolist()
    for name, P in surfaces.items():
        assert O.ref_surface_nodes(P, X, 0.05).tolist() == node_sets[f"sfc_{name}_0.05"].tolist()
    poly = F.read_gli_polygon(os.path.join(GOLDEN, "deck", "point_in_polygon.gli"))
    gx, gy = F.polygon_grid_nodes()
    assert O.ref_point_in_polygon(poly, np.stack([gx, gy, 0 * gx], 1)).sum() == 95511


@pytest.mark.parametrize("et", [M.QUAD4, M.HEX8, M.TET4])
def test_structured_deck_faces_edges_points(tmp_path, et):
    """Left/right faces as surfaces (3-D) or polylines (2-D), an edge
    polyline, a named point; rows in condition order, sorted within a
    polyline; the mesh survives the write/read round trip bit for bit."""
    if et == M.QUAD4:
        m = M.structured_quad(9, 5, 0.5, 2.0)
    elif et == M.HEX8:
        m = M.structured_hex(6, 4, 3, 1.0, 0.5, 2.0)
    else:
        m = M.structured_tet(4, 3, 2, 1.0, 1.0, 0.5)
    Lx, Ly, Lz = m.x.max(), m.y.max(), m.z.max()
    pts = [(0, 0, 0), (0, Ly, 0), (Lx, 0, 0), (Lx, Ly, 0), (0, 0, Lz), (0, Ly, Lz), (Lx, 0, Lz), (Lx, Ly, Lz),
           (Lx / 2 + 0.01, Ly, Lz, "TOP")]
    plys = {"left": ([0, 1], None), "right": ([2, 3], None), "bottom": ([0, 2], None)}
    sfcs = {}
    if et != M.QUAD4:
        plys["left_b"] = ([0, 1, 5, 4, 0], None)
        plys["right_b"] = ([2, 3, 7, 6, 2], None)
        sfcs = {"LEFT": ["left_b"], "RIGHT": ["right_b"]}
    D.write_msh(m, str(tmp_path / "s.msh"))
    D.write_gli(str(tmp_path / "s.gli"), pts, plys, sfcs)
    geo = ("SURFACE", "LEFT", "RIGHT") if et != M.QUAD4 else ("POLYLINE", "left", "right")
    D.write_bc(str(tmp_path / "s.bc"), [
        ("GROUNDWATER_FLOW", "HEAD", geo[0], geo[1], 10.0),
        ("GROUNDWATER_FLOW", "HEAD", geo[0], geo[2], 5.0),
        ("MASS_TRANSPORT", "Tracer", "POLYLINE", "bottom", 1.0),
        ("GROUNDWATER_FLOW", "HEAD", "POINT", "TOP", 7.5),
    ])
    dk = capi.Deck(str(tmp_path / "s.msh"), str(tmp_path / "s.gli"), str(tmp_path / "s.bc"))
    r = dk.mesh
    assert r.elem_type == et and r.dim == m.dim
    assert np.array_equal(r.x, m.x) and np.array_equal(r.y, m.y) and np.array_equal(r.conn, m.conn)
    if m.dim == 3:
        assert np.array_equal(r.z, m.z)
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    top = int(np.argmin((m.x - (Lx / 2 + 0.01)) ** 2 + (m.y - Ly) ** 2 + (m.z - Lz) ** 2))
    rows, vals = dk.dirichlet("GROUNDWATER_FLOW", "HEAD")
    assert rows.tolist() == sorted(lf.tolist()) + sorted(rf.tolist()) + [top]
    assert vals.tolist() == [10.0] * len(lf) + [5.0] * len(rf) + [7.5]
    bottom = np.flatnonzero((m.y == 0) & (m.z == 0))
    rows, vals = dk.dirichlet("MASS_TRANSPORT")
    assert rows.tolist() == bottom.tolist() and np.all(vals == 1.0)
    assert dk.geo_nodes("POLYLINE", "bottom").tolist() == bottom.tolist()


def test_gli_one_based_ids_and_epsilon(tmp_path):
    """One-based point ids (first id 1) index points from 1; a polyline's
    $EPSILON is its search radius (default 0.01)."""
    m = M.structured_quad(4, 4, 1.0, 1.0)
    D.write_msh(m, str(tmp_path / "q.msh"))
    (tmp_path / "q.gli").write_text(
        "#POINTS\n1 0 0.3 0\n2 4 0.3 0\n#POLYLINE\n $NAME\n  narrow\n $POINTS\n  1\n  2\n"
        "#POLYLINE\n $NAME\n  wide\n $EPSILON\n  0.5\n $POINTS\n  1\n  2\n#STOP\n")
    dk = capi.Deck(str(tmp_path / "q.msh"), str(tmp_path / "q.gli"))
    assert len(dk.geo_nodes("POLYLINE", "narrow")) == 0
    assert dk.geo_nodes("POLYLINE", "wide").tolist() == [0, 1, 2, 3, 4]


def test_deck_errors(tmp_path):
    m = M.structured_hex(2, 2, 2)
    D.write_msh(m, str(tmp_path / "h.msh"))
    D.write_gli(str(tmp_path / "h.gli"), [(0, 0, 0), (2, 0, 0)], {"p": ([0, 1], None)})
    with pytest.raises(capi.OgsError, match="cannot open"):
        capi.Deck(str(tmp_path / "missing.msh"))
    (tmp_path / "bad.bc").write_text(
        "#BOUNDARY_CONDITION\n $PCS_TYPE\n  GROUNDWATER_FLOW\n $DIS_TYPE\n  LINEAR 2\n#STOP\n")
    with pytest.raises(capi.OgsError, match="CONSTANT"):
        capi.Deck(str(tmp_path / "h.msh"), None, str(tmp_path / "bad.bc"))
    D.write_bc(str(tmp_path / "u.bc"), [("GROUNDWATER_FLOW", "HEAD", "POLYLINE", "nope", 1.0)])
    dk = capi.Deck(str(tmp_path / "h.msh"), str(tmp_path / "h.gli"), str(tmp_path / "u.bc"))
    with pytest.raises(capi.OgsError, match="unknown polyline"):
        dk.dirichlet("GROUNDWATER_FLOW")
    with pytest.raises(capi.OgsError, match="not supported"):
        dk.geo_nodes("VOLUME", "v")
    (tmp_path / "mixed.msh").write_text(
        "#FEM_MSH\n $NODES\n  4\n0 0 0 0\n1 1 0 0\n2 0 1 0\n3 0 0 1\n $ELEMENTS\n  2\n"
        "0 0 tet 0 1 2 3\n1 0 tri 0 1 2\n#STOP\n")
    with pytest.raises(capi.OgsError, match="mixed element types"):
        capi.Deck(str(tmp_path / "mixed.msh"))
    (tmp_path / "pris.msh").write_text(
        "#FEM_MSH\n $NODES\n  1\n0 0 0 0\n $ELEMENTS\n  1\n0 0 pris 0 0 0 0 0 0\n#STOP\n")
    with pytest.raises(capi.OgsError, match="type not read"):
        capi.Deck(str(tmp_path / "pris.msh"))
    (tmp_path / "range.msh").write_text(
        "#FEM_MSH\n $NODES\n  2\n0 0 0 0\n1 1 0 0\n $ELEMENTS\n  1\n0 0 line 0 5\n#STOP\n")
    with pytest.raises(capi.OgsError, match="bad node index"):
        capi.Deck(str(tmp_path / "range.msh"))
