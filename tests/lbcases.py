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


ONEPHASE_CASES = ["onephase_ghost", "onephase_open"]


class OnephaseCase:
    """A std_one_phase fixture: tables, node attributes (reference numbering),
    the reference's f / rho / vel / mass flux after meta['steps'] steps."""

    def __init__(self, name, bclbm):
        self.name = name
        self.z = np.load(GOLDEN / f"{name}.npz")
        self.meta = json.loads(bytes(self.z["meta"]).decode())
        self.n_nodes, self.nf = self.meta["n_nodes"], self.meta["nf"]
        L = bclbm.lbsolver
        self.L = L
        self.lat = L.Lattice(19, self.z["neigh"], self.z["types"], self.z["pos"], self.z["bulk"],
                             shape=self.z["mask"].shape, periodic="xy")
        self.tags = self.node_attr("nodetags")
        self.labels = self.node_attr("interior_domains")
        self.force_on = self.node_attr("force")
        self.force = [self.meta["fx"], self.meta["fy"], self.meta["fz"]]

    def node_attr(self, name):
        """A voxel attribute at the nodes (0 at node 0), as Nodes/LBvtk read it."""
        v = self.z["attr_" + name]
        out = np.zeros(self.n_nodes, dtype=np.int32 if v.dtype.kind == "i" else np.float64)
        p = self.lat.pos.reshape(-1, 3)[1:]
        sh = v.shape
        out[1:] = v[p[:, 0] % sh[0], p[:, 1] % sh[1], p[:, 2] % sh[2]]
        return out

    def f_init(self):
        """calcfeq at rho = 1, u = 0: w_q at the bulk nodes (main.cpp:457-464)."""
        return self.L.initiate_single(self.lat, np.ones(self.n_nodes))

    def solver(self, **kw):
        return self.L.Solver(self.lat, self.f_init(), collision=self.L.LINKS, tau=(self.meta["tau"],) * 2,
                             force=self.force, tags=self.tags, labels=self.labels, force_on=self.force_on, **kw)
