"""ctypes wrapper of the plain-C oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by the tests (as the checker), by
``__graft_entry__.smoke`` and by the CPU-baseline leg of ``bench.py``.  The
product package never imports this module.

All arrays are in the reference's layout and numbering (see bclbm_oracle.h).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
_lib = None


def build(force: bool = False) -> Path:
    """Compiles liboracle.so with the Makefile in this folder."""
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < (HERE / "bclbm_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return LIB_PATH


class _Grid(ctypes.Structure):
    _fields_ = [("nq", ctypes.c_int), ("n_nodes", ctypes.c_int), ("neigh", ctypes.c_void_p),
                ("types", ctypes.c_void_p), ("n_bulk", ctypes.c_int), ("bulk", ctypes.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.oracle_single_run.argtypes = [ctypes.POINTER(_Grid), ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, dp, dp, dp, dp, dp, ctypes.c_int]
        _lib.oracle_twophase_run.argtypes = [ctypes.POINTER(_Grid), ctypes.c_int, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_double, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int]
        vp = ctypes.c_void_p
        _lib.oracle_links_run.argtypes = [ctypes.POINTER(_Grid), ctypes.c_int, ctypes.c_double, dp, vp, vp, vp,
                                          ctypes.c_double, dp, dp, dp, dp, dp, ctypes.c_int]
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleGrid:
    """Reference Grid/Nodes arrays held for the oracle calls."""

    def __init__(self, nq, neigh, types, bulk=None):
        self.nq = int(nq)
        self.neigh = np.ascontiguousarray(neigh, dtype=np.int32).reshape(-1)
        self.types = np.ascontiguousarray(types, dtype=np.int16)
        self.n_nodes = self.types.size
        if bulk is None:
            bulk = np.nonzero(self.types > 1)[0]
        self.bulk = np.ascontiguousarray(bulk, dtype=np.int32)
        self._s = _Grid(self.nq, self.n_nodes, self.neigh.ctypes.data, self.types.ctypes.data,
                        self.bulk.size, self.bulk.ctypes.data)

    @property
    def nd(self):
        return 2 if self.nq == 9 else 3


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


class SingleRunner:
    """std_case loop on the oracle with reusable buffers (two LbField(1,N), rho, vel)."""

    def __init__(self, g: OracleGrid, f, tau, force, trt=False, tau_anti=1.0, nthreads=1):
        self.g = g
        self.bufs = [np.ascontiguousarray(f, dtype=np.float64).reshape(-1).copy(), None]
        self.bufs[1] = np.zeros_like(self.bufs[0])
        self.rho = np.zeros(g.n_nodes)
        self.vel = np.zeros(g.n_nodes * g.nd)
        self.F = np.zeros(3)
        self.F[:len(force)] = force
        self.tau, self.tau_anti, self.trt, self.nthreads = float(tau), float(tau_anti), int(bool(trt)), int(nthreads)

    @property
    def f(self):
        return self.bufs[0]

    def run(self, nsteps):
        rc = lib().oracle_single_run(ctypes.byref(self.g._s), int(nsteps), self.trt, self.tau, self.tau_anti,
                                     _dp(self.F), _dp(self.bufs[0]), _dp(self.bufs[1]), _dp(self.rho),
                                     _dp(self.vel), self.nthreads)
        if rc < 0:
            raise RuntimeError(f"oracle_single_run failed with {rc}")
        if rc == 1:
            self.bufs.reverse()
        return self.bufs[0]


def single_run(g: OracleGrid, f, nsteps, tau, force, trt=False, tau_anti=1.0, nthreads=1):
    """std_case loop from the LbField(1,N) data f [N*Q].
    Returns (f, rho [N], vel [N*nD]) with the last step's moments."""
    r = SingleRunner(g, f, tau, force, trt, tau_anti, nthreads)
    r.run(nsteps)
    return r.f, r.rho, r.vel


def twophase_run(g: OracleGrid, f, rho, nsteps, tau0, tau1, sigma, beta, force, mom_x=None, nthreads=1):
    """twophase loop; f is LbField(2,N) data [N*2*Q], rho ScalarField(2,N) data
    with the solid boundary densities set.  Returns (f, rho, vel, cg, force_log)."""
    bufs = [np.ascontiguousarray(f, dtype=np.float64).reshape(-1).copy(), None]
    bufs[1] = np.zeros_like(bufs[0])
    rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1).copy()
    vel = np.zeros(g.n_nodes * g.nd)
    cg = np.zeros(g.n_nodes)
    F = np.zeros(3)
    F[:len(force)] = force
    log = np.zeros(max(1, int(nsteps)))
    rc = lib().oracle_twophase_run(ctypes.byref(g._s), int(nsteps), float(tau0), float(tau1), float(sigma),
                                   float(beta), int(mom_x is not None), float(mom_x or 0.0), _dp(F), _dp(bufs[0]),
                                   _dp(bufs[1]), _dp(rho), _dp(vel), _dp(cg), _dp(log), int(nthreads))
    if rc < 0:
        raise RuntimeError(f"oracle_twophase_run failed with {rc}")
    return bufs[rc], rho, vel, cg, log[:int(nsteps)]


def links_run(g: OracleGrid, f, nsteps, tau, force, tags, labels, force_on, rho_w=1.0, nthreads=1):
    """std_one_phase loop (D3Q19) from the LbField(1,N) data f [N*19]; tags,
    labels, force_on are the node attributes [N].  Returns (f, rho [N],
    vel [N*3], flux [2]) with the last step's moments (rho starts at 1, vel at 0
    at every node, as the reference initialises them)."""
    bufs = [np.ascontiguousarray(f, dtype=np.float64).reshape(-1).copy(), None]
    bufs[1] = np.zeros_like(bufs[0])
    rho = np.ones(g.n_nodes)
    vel = np.zeros(g.n_nodes * 3)
    flux = np.zeros(2)
    F = np.zeros(3)
    F[:len(force)] = force
    t = np.ascontiguousarray(tags, dtype=np.int32)
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    fo = np.ascontiguousarray(force_on, dtype=np.int32)
    rc = lib().oracle_links_run(ctypes.byref(g._s), int(nsteps), float(tau), _dp(F), t.ctypes.data, lab.ctypes.data,
                                fo.ctypes.data, float(rho_w), _dp(bufs[0]), _dp(bufs[1]), _dp(rho), _dp(vel),
                                _dp(flux), int(nthreads))
    if rc < 0:
        raise RuntimeError(f"oracle_links_run failed with {rc}")
    return bufs[rc], rho, vel, flux
