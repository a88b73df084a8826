"""Loader of tests/golden/ref_assembly.npz, the systems the reference OGS-5
itself assembled (tests/golden/make_ref_assembly.py), shared by the oracle
and GPU parity tests."""
from __future__ import annotations

import json
import os
from dataclasses import dataclass

import numpy as np

from ogs5_gb300 import mesh as M

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_assembly.npz")

_data = None


def data():
    global _data
    if _data is None:
        _data = dict(np.load(FIXTURE))
    return _data


def names():
    return json.loads(str(data()["cases"]))


@dataclass
class Case:
    name: str
    mesh: M.Mesh
    ngauss: int
    params: dict
    meta: dict
    arrays: dict

    def __getitem__(self, k):
        return self.arrays[k]

    def __contains__(self, k):
        return k in self.arrays

    @property
    def kind(self):
        if "x_ref" in self.arrays:
            return "solve"
        if "p_new" in self.arrays:
            return "picard"
        if "p_iter" in self.arrays:
            return "richards"
        if "val" not in self.arrays:
            return "velocity"
        return "assembly"


def case(name: str) -> Case:
    d = data()
    et, dim, ng = (int(v) for v in d[f"{name}/mesh"])
    xyz = d[f"{name}/xyz"]
    conn = d[f"{name}/conn"]
    m = M.Mesh(et, dim, xyz[0].copy(), xyz[1].copy(), xyz[2].copy(), conn.copy())
    params = json.loads(str(d[f"{name}/params"]))
    meta = json.loads(str(d[f"{name}/meta"])) if f"{name}/meta" in d else {}
    skip = {"mesh", "xyz", "conn", "params", "meta"}
    arrays = {k.split("/", 1)[1]: v for k, v in d.items()
              if k.startswith(name + "/") and k.split("/", 1)[1] not in skip}
    return Case(name, m, ng, params, meta, arrays)


def by_kind(kind: str):
    return [n for n in names() if case(n).kind == kind]
