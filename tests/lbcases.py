"""Golden cases: reference tables and reference outputs from tests/golden/*.npz,
with the initial state built the way the reference mains build it."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["channel_256x64", "disc_40x32", "pack_20", "box_12x10x8"]


class Case:
    def __init__(self, name, bclbm):
        self.name = name
        self.z = np.load(GOLDEN / f"{name}.npz")
        self.meta = json.loads(bytes(self.z["meta"]).decode())
        self.nq, self.nd, self.nf, self.n_nodes = (self.meta[k] for k in ("nq", "nd", "nf", "n_nodes"))
        L = bclbm.lbsolver
        self.lat = L.Lattice(self.nq, self.z["neigh"], self.z["types"], self.z["pos"], self.z["bulk"],
                             shape=self.z["mask"].shape, periodic=self.meta["periodic"])
        self.L = L
        self.runs = {r["tag"]: r for r in self.meta["runs"]}

    def attr(self, name):
        return self.lat.attribute(self.z["attr_" + name])

    def force(self, run):
        return [run.get("fx", 0.0), run.get("fy", 0.0), run.get("fz", 0.0)][:self.nd]

    def init(self, run):
        """(f_init, rho_init or None) in reference layout."""
        if run["mode"] == "single":
            return self.L.initiate_single(self.lat, self.attr("init_rho")), None
        return self.L.initiate_twophase(self.lat, self.attr("rho0"), self.attr("rho1"), self.attr("wettability"))

    def expected(self, tag):
        z = self.z
        out = {"f": z[tag + "_f"], "rho": z[tag + "_rho"], "vel": z[tag + "_vel"]}
        if tag + "_cg" in z:
            out["cg"] = z[tag + "_cg"]
            out["force"] = z[tag + "_force"]
        return out

    def bulk_rows(self, f, nfields):
        return f.reshape(self.n_nodes, nfields, self.nq)[self.lat.bulk]


def all_runs():
    out = []
    for name in CASES:
        meta = json.loads(bytes(np.load(GOLDEN / f"{name}.npz")["meta"]).decode())
        for r in meta["runs"]:
            out.append((name, r["tag"]))
    return out
