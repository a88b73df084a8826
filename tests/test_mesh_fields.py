"""Synthetic decks: mesh sizes, pattern sizes (SparseTable CRS), GRF stats."""
import numpy as np

from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M


def test_config_sizes():
    q = M.structured_quad(100, 100)
    assert q.n_nodes == 10201 and q.n_elements == 10000
    h = M.structured_hex(8, 6, 4)
    assert h.n_nodes == 9 * 7 * 5 and h.n_elements == 8 * 6 * 4
    t = M.hex_to_tet(h)
    assert t.n_elements == 6 * h.n_elements


def test_pattern_nnz_formulas(oracle):
    # hex: 27-point couplings -> (3n-2) per axis product; quad 9-point
    h = M.structured_hex(6, 5, 4)
    rp, col = oracle.build_pattern(h.n_nodes, h.conn)
    assert len(col) == (3 * 7 - 2) * (3 * 6 - 2) * (3 * 5 - 2)
    # Kuhn tets: 7 edge directions -> 15 couplings per interior node
    t = M.structured_tet(5, 5, 5)
    rp, col = oracle.build_pattern(t.n_nodes, t.conn)
    deg = np.diff(rp)
    assert deg.max() == 15
    # symmetric pattern, sorted rows, diagonal present
    for r in range(0, t.n_nodes, 17):
        row = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0) and r in row


def test_tet_volumes_positive_and_cover_hex():
    t = M.structured_tet(2, 2, 2, 1.0, 2.0, 3.0)
    P = np.stack([t.x, t.y, t.z], 1)[t.conn]
    v = np.abs(np.einsum("eij,ej->ei", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])[:, None, :],
                         P[:, 3] - P[:, 0]).ravel()) / 6
    assert np.all(v > 0)
    assert abs(v.sum() - 2 * 2 * 2 * 6.0) < 1e-12


def test_grf_statistics():
    g = fields.gaussian_random_field((64, 64, 32), 1.0, 8.0, seed=3)
    assert abs(g.mean()) < 0.5 and 0.5 < g.var() < 1.5
    k = fields.lognormal_k((32, 32, 16), np.log(1e-5), 1.0, 8.0, seed=5)
    assert k.shape == (32 * 32 * 16,) and np.all(k > 0)
    assert np.array_equal(k, fields.lognormal_k((32, 32, 16), np.log(1e-5), 1.0, 8.0, seed=5))
