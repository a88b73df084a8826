"""Host logic of bench.py's CPU arms (no GPU): the step shares, the pattern
size in the shared config, the reference arm's port processes on a small
lattice, and the calibration summary of oracle/time_reference.py."""
import numpy as np
import pytest

import bench
from oracle import time_reference as TR


def test_split_shares_every_step():
    for total in range(0, 40):
        for workers in range(1, 17):
            sh = bench._split(total, workers)
            assert sum(sh) == total and len(sh) == workers and max(sh) - min(sh) <= 1


@pytest.mark.parametrize("dims", [(2, 3, 4), (5, 1, 3), (4, 4, 2)])
def test_pattern_nnz_matches_the_sparsity_pattern(oracle, dims):
    from ogs5_gb300 import mesh as M
    m = M.structured_hex(*dims)
    rp, col = oracle.build_pattern(m.n_nodes, m.conn)
    assert len(col) == bench.hex_pattern_nnz(*dims)


def test_config_is_the_same_dict_in_both_arms():
    c = bench.deck_config()
    assert c == bench.deck_config(1)
    assert (c["nodes"], c["elements"], c["nnz"]) == (1081665, 1048576, 385 * 385 * 193)


def test_port_step_is_one_full_step(oracle):
    d = bench.PortDeck((6, 5, 4))
    x, its, t_asm, t_cg = d.step(d.h0.copy())
    rp, col = oracle.build_pattern(d.m.n_nodes, d.m.conn)
    val, b = oracle.assemble(d.m, rp, col, oracle.make_params(pcs_type=0, dt=bench.DT, storage=bench.SS),
                             elem_k=d.ek, u0=d.h0)
    oracle.dirichlet(rp, col, val, b, d.rows, d.vals, symmetric=True)
    xo, info = oracle.solve(rp, col, val, b, d.h0.copy(), method=5, precond=1, max_iter=20000, tol=bench.TOL)
    assert its == info["iterations"] > 0
    assert np.array_equal(x, xo)


def test_reference_arm_port_processes(oracle):
    """Two spawned processes, warm-up and timed shares, barriers: every timed
    step reports its CG iterations and the wall is positive."""
    wall, its = bench._run_port(2, [1, 0], [2, 1], dims=(6, 5, 4))
    assert wall > 0 and len(its) == 3 and all(i > 0 for i in its)


def test_calibration_summary_from_markers():
    marks = [["assemble", 10.0], ["solve", 30.0], ["velocity", 50.0], ["accepted", 52.0],
             ["assemble", 53.0], ["solve", 70.0], ["velocity", 85.0], ["accepted", 86.0]]
    res = {"host": "x", "reference_sp": {"marks": marks, "iterations": [200, 150], "setup_s": 10.0},
           "port": {"assembly_s": 5.0, "cg_s": 10.0, "cg_iterations": 250}}
    s = TR.summarise(res)
    assert s["reference_sp"]["steps"] == [{"assembly_s": 20.0, "solve_s": 20.0, "rest_s": 2.0},
                                          {"assembly_s": 17.0, "solve_s": 15.0, "rest_s": 1.0}]
    r = s["reference_sp_over_port"]
    assert r["assembly"] == 4.0 and r["first_step_assembly_plus_solve"] == round(40 / 15, 2)
    assert r["time_per_cg_iteration"] == round((20 / 200) / (10 / 250), 2)


def test_roofline_traffic_comes_from_the_committed_profile():
    """The bench line's roofline traffic is read from the ncu summary of the
    roofline kernel; every profile that names a per-launch figure keeps it
    readable."""
    import glob
    import os
    t = bench.measured_traffic("k_mp_spmv_lines_hex128x128x64.md")
    assert isinstance(t, int) and 0.9 * 64.9e6 < t < 1.1 * 64.9e6
    for p in glob.glob(os.path.join(bench.ROOT, "profiles", "*.md")):
        for line in open(p):
            if line.startswith("dram_bytes_per_launch:"):
                assert int(line.split(":")[1]) > 0
