"""Shared helpers for the parity tests (tolerances are stated here)."""
import numpy as np

# matrix entries: 1e-12 relative, with an absolute floor of 1e-14 x the
# largest entry of the row (entries that are zero in exact arithmetic come
# out as rounding noise of the row scale in both codes)
MATRIX_RTOL = 1e-12
MATRIX_FLOOR = 1e-14
# heads / concentrations: 1e-10 relative to the largest value
SOLUTION_RTOL = 1e-10


def rowmax(rp, val):
    n = len(rp) - 1
    out = np.zeros(n)
    counts = np.diff(rp)
    rows = np.repeat(np.arange(n), counts)
    np.maximum.at(out, rows, np.abs(val))
    return out, rows


def assert_matrix_close(rp, got, want, rtol=MATRIX_RTOL, floor=MATRIX_FLOOR):
    rm, rows = rowmax(rp, want)
    tol = rtol * np.maximum(np.abs(got), np.abs(want)) + floor * rm[rows]
    err = np.abs(got - want)
    bad = np.nonzero(err > tol)[0]
    assert bad.size == 0, (f"{bad.size} entries differ; worst rel "
                           f"{(err / np.maximum(np.abs(want), 1e-300)).max():.3e} at {bad[:5]}")


def assert_vector_close(got, want, rtol=MATRIX_RTOL, scale=None):
    s = np.abs(want).max() if scale is None else scale
    err = np.abs(got - want)
    tol = rtol * np.maximum(np.abs(got), np.abs(want)) + MATRIX_FLOOR * s
    bad = np.nonzero(err > tol)[0]
    assert bad.size == 0, f"{bad.size} entries differ; max abs err {err.max():.3e} (scale {s:.3e})"


def rel_max_err(got, want):
    return float(np.abs(got - want).max() / max(np.abs(want).max(), 1e-300))


def distort(mesh, amount, seed):
    """Moves interior nodes by up to amount*spacing (non-affine elements)."""
    rng = np.random.default_rng(seed)
    m = mesh
    coords = [m.x.copy(), m.y.copy(), m.z.copy()]
    for a in range(m.dim):
        c = coords[a]
        interior = (c > c.min()) & (c < c.max())
        c[interior] += amount * rng.uniform(-1, 1, interior.sum())
    import copy
    out = copy.copy(m)
    out.x, out.y, out.z = coords
    return out


def renumber(mesh, seed):
    """Random node renumbering (scatters the CSR pattern: no diagonal form)."""
    import copy
    rng = np.random.default_rng(seed)
    perm = rng.permutation(mesh.n_nodes)          # new id of old node i
    inv = np.empty_like(perm)
    inv[perm] = np.arange(mesh.n_nodes)
    out = copy.copy(mesh)
    out.x, out.y, out.z = mesh.x[inv], mesh.y[inv], mesh.z[inv]
    out.conn = perm[mesh.conn].astype(np.int32)
    return out, perm
