"""Times the reference OGS-5 itself (oracle/_ref/ogs_sp, ogs_fem: its own
main, built from its sources by refbuild.mk) on the benchmark deck, and the
oracle's C restatement on the same host, phase by phase.  TEST
INFRASTRUCTURE ONLY: a calibration run where the reference's sources exist
(the GPU host has neither the sources nor an x86 build of them).

    python oracle/time_reference.py [--steps 1] [--out file.json]

Deck: hex 128 x 128 x 64 cells (1,081,665 nodes), ln K Gaussian random
field (mean ln 1e-5, variance 1, correlation length 8 cells, the bench's
seed) as a #MEDIUM_PROPERTIES_DISTRIBUTED element file, Ss 1e-4, dt 3600 s,
heads 10 / 0 m on the x faces (two GLI surfaces), initial heads 0 except
10 m on the x = 0 face.
Phases come from the reference's own stdout markers, read line by line as
they are printed ("Assembling equation system...", "Calling linear
solver...", FEM/rf_pcs.cpp:4818,4826) and the solver's iteration report.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if sys.path and os.path.abspath(sys.path[0]) == HERE:
    sys.path.pop(0)  # run as a script: oracle/oracle.py must not shadow the oracle package
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def write_deck(dirpath, build, steps):
    import ref_decks as R
    from ogs5_gb300 import fields
    from ogs5_gb300 import deck as D
    from ogs5_gb300 import mesh as M
    m = M.structured_hex(128, 128, 64)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 8.0, seed=2)
    if build == "sp":   # Linear_EQS: BiCGStab + Jacobi (its CG does not converge with row-only Dirichlet)
        proc = R.Process("GROUNDWATER_FLOW", dt=3600.0, ls_method=2, precond=1, storage=100, ls_tol=1e-10,
                         ls_max_iter=20000)
    else:               # legacy: SpCG on the MXRandbed (symmetric) system
        proc = R.Process("GROUNDWATER_FLOW", dt=3600.0, ls_method=5, precond=0, storage=2, ls_tol=1e-10,
                         ls_max_iter=20000)
    deck = R.Deck(mesh=m, processes=[proc], medium=R.Medium(dim=3, storage=1e-4), elem_k=ek)
    path = R.write(deck, dirpath)
    with open(path + ".tim", "w") as f:
        f.write("#TIME_STEPPING\n $PCS_TYPE\n  GROUNDWATER_FLOW\n $TIME_START\n  0\n $TIME_END\n  %r\n"
                " $TIME_STEPS\n  %d 3600\n#STOP\n" % (3600.0 * steps, steps))
    # the x faces as two surfaces (rectangles in the y-z plane)
    pts = [(0, 0, 0), (0, 128, 0), (0, 128, 64), (0, 0, 64),
           (128, 0, 0), (128, 128, 0), (128, 128, 64), (128, 0, 64)]
    D.write_gli(path + ".gli", pts, polylines={"LEFT": ([0, 1, 2, 3, 0], None), "RIGHT": ([4, 5, 6, 7, 4], None)},
                surfaces={"LEFT_FACE": ["LEFT"], "RIGHT_FACE": ["RIGHT"]})
    D.write_bc(path + ".bc", [("GROUNDWATER_FLOW", "HEAD", "SURFACE", "LEFT_FACE", 10.0),
                              ("GROUNDWATER_FLOW", "HEAD", "SURFACE", "RIGHT_FACE", 0.0)])
    # initial heads carry the Dirichlet values (with heads 0 on the x = 0
    # face the SP build's BiCGStab breaks down at its second iteration,
    # equation_class.cpp:1343-1348)
    with open(path + ".ic", "w") as f:
        f.write("#INITIAL_CONDITION\n $PCS_TYPE\n  GROUNDWATER_FLOW\n $PRIMARY_VARIABLE\n  HEAD\n"
                " $GEO_TYPE\n  DOMAIN\n $DIS_TYPE\n  CONSTANT 0\n"
                "#INITIAL_CONDITION\n $PCS_TYPE\n  GROUNDWATER_FLOW\n $PRIMARY_VARIABLE\n  HEAD\n"
                " $GEO_TYPE\n  SURFACE LEFT_FACE\n $DIS_TYPE\n  CONSTANT 10\n#STOP\n")
    with open(path + ".out", "w") as f:
        f.write("#STOP\n")
    return path


def run_reference(binary, path):
    """Runs the reference's own executable; returns phase times (s) from
    its stdout lines."""
    t0 = time.perf_counter()
    def cap():  # the run needs a few GB; a misread deck must not take the host's memory
        import resource
        resource.setrlimit(resource.RLIMIT_AS, (24 << 30, 24 << 30))
    proc = subprocess.Popen(["stdbuf", "-oL", binary, path], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                            text=True, cwd=os.path.dirname(path), preexec_fn=cap)
    marks, iters = [], []
    for line in proc.stdout:
        t = time.perf_counter() - t0
        if "Assembling equation system" in line:
            marks.append(("assemble", t))
        elif "Calling linear solver" in line:
            marks.append(("solve", t))
        elif "Calculate velocity" in line or "->Calculate" in line:
            marks.append(("velocity", t))
        elif "This step is accepted" in line:
            marks.append(("accepted", t))
        mm = re.search(r"^\s*(\d+)\|\s*\d+\|", line) or re.search(r"SpCG iteration: (\d+)/", line)
        if mm:
            iters.append(int(mm.group(1)))
    proc.wait()
    total = time.perf_counter() - t0
    out = {"total_s": total, "iterations": iters, "marks": marks, "rc": proc.returncode}
    a = [t for k, t in marks if k == "assemble"]
    s = [t for k, t in marks if k == "solve"]
    if a:
        out["setup_s"] = a[0]
        out["assembly_s"] = [si - ai for ai, si in zip(a, s)]
    return out


def time_port():
    """The oracle's C restatement on the same deck: full assembly and CG
    iterations (one thread)."""
    from oracle import oracle as O
    from ogs5_gb300 import fields
    from ogs5_gb300 import mesh as M
    O.build()
    m = M.structured_hex(128, 128, 64)
    ek = fields.lognormal_k(m.shape, np.log(1e-5), 1.0, 8.0, seed=2)
    rp, col = O.build_pattern(m.n_nodes, m.conn)
    u0 = np.zeros(m.n_nodes)
    t = time.perf_counter()
    val, b = O.assemble(m, rp, col, O.make_params(pcs_type=0, dt=3600.0, storage=1e-4), elem_k=ek, u0=u0)
    t_asm = time.perf_counter() - t
    lf, rf = m.face_nodes(0, 0), m.face_nodes(0, 1)
    rows = np.concatenate([lf, rf])
    vals = np.concatenate([np.full(len(lf), 10.0), np.zeros(len(rf))])
    O.dirichlet(rp, col, val, b, rows, vals, symmetric=True)
    x0 = np.zeros(m.n_nodes)
    x0[lf] = 10.0
    t = time.perf_counter()
    x, info = O.solve(rp, col, val, b, x0, method=5, precond=1, max_iter=20000, tol=1e-10)
    t_cg = time.perf_counter() - t
    return {"assembly_s": t_asm, "cg_s": t_cg, "cg_iterations": info["iterations"],
            "cg_iteration_ms": 1e3 * t_cg / max(1, info["iterations"])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--out", default=None)
    ap.add_argument("--no-port", action="store_true")
    ap.add_argument("--builds", default="sp,fem")
    args = ap.parse_args()
    res = {"host": os.uname().machine, "cores_used": 1}
    tmp = tempfile.mkdtemp(prefix="ogs_time_")
    for build in [b for b in args.builds.split(",") if b]:
        binary = os.path.join(HERE, "_ref", "ogs_" + build)
        path = write_deck(os.path.join(tmp, build), build, args.steps)
        res["reference_" + build] = run_reference(binary, path)
        print(build, json.dumps(res["reference_" + build])[:600], flush=True)
    if not args.no_port:
        res["port"] = time_port()
        print("port", res["port"], flush=True)
    res["summary"] = summarise(res)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)


def _steps(r):
    """Per step of a reference run: assembly, linear solve and the rest of
    the step (Cal_Velocity, output), seconds, from the stdout markers."""
    out, mk = [], r.get("marks", [])
    starts = [i for i, (k, _) in enumerate(mk) if k == "assemble"]
    for q, i in enumerate(starts):
        end = starts[q + 1] if q + 1 < len(starts) else len(mk)
        t = {k: v for k, v in mk[i:end]}
        if "solve" in t and "accepted" in t:
            after = t.get("velocity", t["accepted"])
            out.append({"assembly_s": round(t["solve"] - t["assemble"], 2),
                        "solve_s": round(after - t["solve"], 2),
                        "rest_s": round(t["accepted"] - after, 2)})
    return out


def summarise(res):
    """Assembly + linear solve of a step, reference builds against the
    oracle's C restatement on the same host."""
    s = {"host": res["host"], "deck": "hex 128 x 128 x 64, 1,081,665 nodes, 1,048,576 hexes, CG + Jacobi 1e-10"}
    for key in ("reference_sp", "reference_fem"):
        if key in res:
            st = _steps(res[key])
            its = res[key].get("iterations", [])
            s[key] = {"setup_s": round(res[key].get("setup_s", 0.0), 1), "steps": st,
                      "linear_iterations": its[:len(st)]}
    if "port" in res:
        p = res["port"]
        s["port"] = {"assembly_s": round(p["assembly_s"], 2), "solve_s": round(p["cg_s"], 2),
                     "linear_iterations": p["cg_iterations"]}
        if "reference_sp" in s and s["reference_sp"]["steps"]:
            f = s["reference_sp"]["steps"][0]
            ip = max(1, p["cg_iterations"])
            ir = max(1, (s["reference_sp"]["linear_iterations"] or [ip])[0])
            s["reference_sp_over_port"] = {
                "assembly": round(f["assembly_s"] / p["assembly_s"], 2),
                "time_per_cg_iteration": round((f["solve_s"] / ir) / (p["cg_s"] / ip), 2),
                "first_step_assembly_plus_solve": round((f["assembly_s"] + f["solve_s"]) /
                                                        (p["assembly_s"] + p["cg_s"]), 2)}
    return s


if __name__ == "__main__":
    main()
