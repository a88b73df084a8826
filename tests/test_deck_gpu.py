"""A deck on disk through the GPU path: the native reader's mesh and
Dirichlet rows feed GpuMesh / LinearEQS; the assembled system and heads
match the oracle's on the same deck."""
import numpy as np
import pytest

from ogs5_gb300 import deck as D
from ogs5_gb300 import fields
from ogs5_gb300 import mesh as M
from tests.helpers import SOLUTION_RTOL, assert_matrix_close, assert_vector_close, rel_max_err

pytestmark = pytest.mark.gpu


def _write_deck(tmp_path, m):
    Lx, Ly, Lz = m.x.max(), m.y.max(), m.z.max()
    pts = [(0, 0, 0), (0, Ly, 0), (0, Ly, Lz), (0, 0, Lz), (Lx, 0, 0), (Lx, Ly, 0), (Lx, Ly, Lz), (Lx, 0, Lz),
           (Lx / 2, Ly / 2, Lz, "WELL")]
    D.write_msh(m, str(tmp_path / "d.msh"))
    D.write_gli(str(tmp_path / "d.gli"), pts,
                {"left_b": ([0, 1, 2, 3, 0], None), "right_b": ([4, 5, 6, 7, 4], None)},
                {"LEFT": ["left_b"], "RIGHT": ["right_b"]})
    D.write_bc(str(tmp_path / "d.bc"), [("GROUNDWATER_FLOW", "HEAD", "SURFACE", "LEFT", 12.0),
                                        ("GROUNDWATER_FLOW", "HEAD", "SURFACE", "RIGHT", 3.0),
                                        ("GROUNDWATER_FLOW", "HEAD", "POINT", "WELL", 4.5)])


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_deck_flow_solve_matches_oracle(gpu, oracle, tmp_path, kind):
    src = M.structured_hex(14, 9, 6, 1.0, 1.0, 0.5) if kind == "hex" else M.structured_tet(8, 6, 4)
    _write_deck(tmp_path, src)
    dk = gpu.Deck(str(tmp_path / "d.msh"), str(tmp_path / "d.gli"), str(tmp_path / "d.bc"))
    m = dk.mesh
    rows, vals = dk.dirichlet("GROUNDWATER_FLOW", "HEAD")
    assert len(rows) == len(src.face_nodes(0, 0)) + len(src.face_nodes(0, 1)) + 1
    kh = fields.lognormal_k(src.shape, np.log(1e-5), 1.0, 3.0, seed=4)
    ek = kh if kind == "hex" else np.repeat(kh, 6)
    p = gpu.make_params(gpu.GROUNDWATER_FLOW, dt=3600.0, storage=1e-4)
    eqs = gpu.LinearEQS(gpu.GpuMesh(m))
    eqs.Initialize()
    eqs.GlobalAssembly(p, ek, np.zeros(m.n_nodes))
    eqs.SetKnownX(rows, vals, gpu.DIRICHLET_SYMMETRIC)
    rp, col, val = eqs.get_csr()
    b = eqs.get_rhs()
    orp, ocol = oracle.build_pattern(m.n_nodes, m.conn)
    op = oracle.make_params(pcs_type=0, dt=3600.0, storage=1e-4)
    oval, ob = oracle.assemble(m, orp, ocol, op, elem_k=ek, u0=np.zeros(m.n_nodes))
    oracle.dirichlet(orp, ocol, oval, ob, rows, vals, symmetric=True)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert_matrix_close(rp, val, oval)
    assert_vector_close(b, ob)
    eqs.ConfigNumerics(gpu.LS_CG, gpu.PRECOND_JACOBI, 5000, 1e-13)
    x0 = np.full(m.n_nodes, 7.0)
    x0[rows] = vals
    x = x0.copy()
    eqs.Solver(x)
    xo, _ = oracle.solve(orp, ocol, oval, ob, x0, method=5, precond=1, max_iter=5000, tol=1e-13)
    assert rel_max_err(x, xo) < SOLUTION_RTOL
    assert np.all(x[rows] == vals)
