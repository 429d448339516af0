"""Host-side mirror of the reference lbsolver set-up, above the C ABI.

The names and argument meanings follow the reference's lbsolver API so that a
user of ``src/std_case`` / ``src/twophase`` finds the same steps:

* ``Lattice``            Grid + Nodes + findBulkNodes of one rank
                         (src/lbsolver/LBgrid.h:127-148, LBnodes.h:112-209,
                         LBgeometry.h:11-56);
* ``weights``            DXQY::w (src/lbsolver/LBd2q9.h:32, LBd3q19.h:32);
* ``initiate_single``    f = w_q rho at the bulk nodes (src/std_case/main.cpp:92-96);
* ``initiate_twophase``  rho0/rho1/wettability read as float, the wettability
                         densities on boundary solids, and initiateLbField for
                         both phases (src/twophase/main_TWOPHASE.cpp:156-207,
                         src/lbsolver/LBinitiatefield.h:33-57);
* ``Solver``             the device time step through the C ABI in
                         ``include/bclbm.h`` (see ``native``).

Arrays are numpy, in the reference's layout and numbering.
"""

from __future__ import annotations

import numpy as np

from . import geometry as _geometry
from . import native as _native

BGK, TRT, RK, LINKS = 0, 1, 2, 3
F64, F32, F16, BF16 = 0, 1, 2, 3
PRECISION = {"f64": F64, "f32": F32, "f16": F16, "bf16": BF16}
FLAG_EXACT = 1
FLAG_SFC_ORDER = 2
FLAG_FP64_FMA = 4
FLAG_NO_MASS_FIX = 8
FLAG_LAGGED_COLOUR = 16


def weights(nq: int) -> np.ndarray:
    """Lattice weights in the reference's direction order, computed as the
    reference's constexpr divisions."""
    if nq == 9:
        w0, w1, w2 = 16.0 / 36.0, 4.0 / 36.0, 1.0 / 36.0
        return np.array([w1, w2, w1, w2, w1, w2, w1, w2, w0])
    if nq == 19:
        w0, w1, w2 = 12.0 / 36.0, 2.0 / 36.0, 1.0 / 36.0
        return np.array([w1] * 3 + [w2] * 6 + [w1] * 3 + [w2] * 6 + [w0])
    raise ValueError(f"unsupported lattice with {nq} directions")


class Lattice:
    """One rank's Grid/Nodes arrays: neighbour table, node types, positions, bulk list."""

    def __init__(self, nq, neigh, types, pos=None, bulk=None, shape=None, periodic=""):
        self.nq = int(nq)
        self.nd = 2 if self.nq == 9 else 3
        self.neigh = np.ascontiguousarray(neigh, dtype=np.int32).reshape(-1)
        self.types = np.ascontiguousarray(types, dtype=np.int16)
        self.n_nodes = int(self.types.size)
        if self.neigh.size != self.n_nodes * self.nq:
            raise ValueError("neighbour table size does not match the node count")
        self.pos = None if pos is None else np.ascontiguousarray(pos, dtype=np.int32).reshape(-1)
        if bulk is None:  # findBulkNodes: every fluid node of this rank, in node order
            bulk = np.nonzero(self.types > 1)[0]
        self.bulk = np.ascontiguousarray(bulk, dtype=np.int32)
        self.shape = None if shape is None else tuple(int(n) for n in shape)
        self.periodic = periodic

    @classmethod
    def from_geometry(cls, geo, lattice: str, periodic: str = ""):
        lat = _geometry.build_lattice(geo, lattice, periodic)
        return cls(lat["nq"], lat["neigh"], lat["types"], lat["pos"], shape=np.asarray(geo).shape,
                   periodic=periodic)

    @classmethod
    def from_vtklb(cls, path, lattice: str):
        """Grid + Nodes of one rank from a .vtklb file (bclbm_lattice_read_vtklb)."""
        lat = _geometry.read_vtklb(path, lattice)
        return cls(lat["nq"], lat["neigh"], lat["types"], lat["pos"])

    @property
    def n_bulk(self) -> int:
        return int(self.bulk.size)

    def attribute(self, values: np.ndarray) -> np.ndarray:
        """A per-voxel attribute at every node's position, the way vtklb.py
        writes it (periodic rim positions take the opposite interior value);
        node 0 gets 0."""
        values = np.asarray(values)
        p = self.pos.reshape(-1, self.nd)
        idx = tuple(np.mod(p[:, d], values.shape[d]) for d in range(self.nd))
        out = values[idx].astype(values.dtype, copy=True)
        out[0] = 0
        return out

    def solid_boundary(self) -> np.ndarray:
        """findSolidBndNodes (src/lbsolver/LBgeometry.h:37-45)."""
        return np.nonzero(self.types == 1)[0].astype(np.int32)


def initiate_single(lat: Lattice, rho_node: np.ndarray) -> np.ndarray:
    """std_case start: f(0,q,n) = w_q rho(0,n) at bulk nodes, 0 elsewhere."""
    w = weights(lat.nq)
    f = np.zeros((lat.n_nodes, lat.nq))
    b = lat.bulk
    f[b] = w[None, :] * np.asarray(rho_node, dtype=np.float64)[b][:, None]
    return f.reshape(-1)


def initiate_twophase(lat: Lattice, rho0_node, rho1_node, wett_node):
    """twophase start.  Inputs are per-node attribute values (Lattice.attribute).

    The reference reads rho0, rho1 and wettability as float
    (main_TWOPHASE.cpp:158, 166, 173) and sets rho1 = 1 - wettability in float
    arithmetic on boundary solids.  Returns (f [N*2*Q], rho [N*2]).
    """
    r0 = np.asarray(rho0_node).astype(np.float32).astype(np.float64)
    r1 = np.asarray(rho1_node).astype(np.float32).astype(np.float64)
    wt = np.asarray(wett_node).astype(np.float32)
    sb = lat.types == 1
    r0[sb] = wt[sb].astype(np.float64)
    r1[sb] = (np.float32(1.0) - wt[sb]).astype(np.float64)
    r0[0] = 0.0
    r1[0] = 0.0
    w = weights(lat.nq)
    f = np.zeros((lat.n_nodes, 2, lat.nq))
    b = lat.bulk
    # initiateLbField with zero velocity: w_q * rho * (1 + 0) (LBinitiatefield.h:50-55)
    f[b, 0, :] = (w[None, :] * r0[b][:, None]) * 1.0
    f[b, 1, :] = (w[None, :] * r1[b][:, None]) * 1.0
    rho = np.stack([r0, r1], axis=1).reshape(-1)
    return f.reshape(-1), rho


def write_lblbf(path, f, nfields: int, nq: int):
    """LbField::writeToFile's binary format (src/lbsolver/LBfield.h:378-393): int32
    nFields, nQ, nNodes, then the FP64 data [node][field][q], little endian."""
    f = np.ascontiguousarray(f, dtype="<f8").reshape(-1)
    n_nodes = f.size // (nfields * nq)
    if n_nodes * nfields * nq != f.size:
        raise ValueError("f does not hold nNodes x nFields x nQ values")
    with open(path, "wb") as fh:
        fh.write(np.array([nfields, nq, n_nodes], dtype="<i4").tobytes())
        fh.write(f.tobytes())


def read_lblbf(path):
    """LbField::readFromFile's format: returns (f [N*nF*Q], nfields, nq, n_nodes)."""
    raw = np.fromfile(path, dtype=np.uint8)
    nfields, nq, n_nodes = (int(x) for x in raw[:12].view("<i4"))
    f = raw[12:].view("<f8")
    if f.size != nfields * nq * n_nodes:
        raise ValueError(f"{path}: {f.size} values for {nfields} x {nq} x {n_nodes}")
    return f.astype(np.float64), nfields, nq, n_nodes


class Solver:
    """One device lattice instance behind the C ABI (bclbm_create ... bclbm_destroy)."""

    def __init__(self, lat: Lattice, f_init, collision=BGK, precision=F64, tau=(1.0, 1.0), force=(0.0, 0.0, 0.0),
                 sigma=0.0, beta=0.0, flux_control=False, mom_x=0.0, rho_init=None, exact=False, sfc=False,
                 rho_ref=1.0, store_scale=0.0, fma64=False, mass_fix=True, tags=None, labels=None, force_on=None,
                 rho_w=1.0, lagged_colour=False):
        """collision LINKS is the std_one_phase step (src/std_one_phase/main.cpp):
        tags, labels (interior domains) and force_on are its node attributes [N]
        (Nodes tags, interior_domains, force), rho_w the pressure-boundary density.
        lagged_colour: two-phase shifted storage in one pass per step, the colour
        gradient from the previous step's colours (BCLBM_FLAG_LAGGED_COLOUR)."""
        if isinstance(precision, str):
            precision = PRECISION[precision]
        links = None
        if collision == LINKS:
            if tags is None or labels is None:
                raise ValueError("the std_one_phase step needs tags and labels")
            self._links = tuple(None if a is None else np.ascontiguousarray(a, dtype=np.int32)
                                for a in (tags, labels, force_on))
            for a in self._links:
                if a is not None and a.size != lat.n_nodes:
                    raise ValueError("tags, labels and force_on have one value per node")
            links = self._links + (float(rho_w),)
        self.lat = lat
        self.nfields = 2 if collision == RK else 1
        flags = (FLAG_EXACT if exact else 0) | (FLAG_SFC_ORDER if sfc else 0) | (FLAG_FP64_FMA if fma64 else 0) | \
            (0 if mass_fix else FLAG_NO_MASS_FIX) | (FLAG_LAGGED_COLOUR if lagged_colour else 0)
        F = np.zeros(3)
        F[:len(force)] = force
        self._h = _native.create(lat, np.ascontiguousarray(f_init, dtype=np.float64), collision, precision, flags,
                                 tuple(float(t) for t in tau) + ((1.0,) if len(tau) == 1 else ()), F, sigma, beta,
                                 int(bool(flux_control)), mom_x, rho_ref, store_scale,
                                 None if rho_init is None else np.ascontiguousarray(rho_init, dtype=np.float64),
                                 links)

    def step(self, nsteps: int = 1):
        _native.check(_native.lib().bclbm_step(self._h, int(nsteps)), self._h)

    def step_timed(self, nsteps: int) -> dict:
        """Steps with CUDA events on the handle's own stream (bclbm_step_timed)."""
        return _native.step_timed(self._h, nsteps)

    def download_f(self, out=None):
        if out is None:
            out = np.zeros(self.lat.n_nodes * self.nfields * self.lat.nq)
        _native.check(_native.lib().bclbm_download_f(self._h, _native.dp(out)), self._h)
        return out

    def checkpoint(self, path):
        """The populations after the last step, as the reference's LbField::writeToFile
        writes them; a Solver created from read_lblbf(path) continues the run exactly."""
        write_lblbf(path, self.download_f(), self.nfields, self.lat.nq)

    def _macro_arrays(self, rho, vel, cg):
        n = self.lat.n_nodes
        want = ((rho, n * self.nfields), (vel, n * self.lat.nd), (cg, n if self.nfields == 2 else 0))
        out = []
        for a, size in want:
            if a is None:
                a = np.zeros(size) if size else None
            elif a.dtype != np.float64 or not a.flags.c_contiguous or a.size != size:
                raise ValueError(f"macro arrays are contiguous float64 of {size} values (reference layout)")
            out.append(a)
        return out

    def download_macros(self, rho=None, vel=None, cg=None):
        """rho / vel (/ cg) of the last step in the reference layout, written into
        the given arrays (e.g. the fields an ``output.Output`` reads) or new ones."""
        rho, vel, cg = self._macro_arrays(rho, vel, cg)
        _native.check(_native.lib().bclbm_download_macros(self._h, _native.dp(rho), _native.dp(vel),
                                                          _native.dp(cg)), self._h)
        return rho, vel, cg

    def macros_begin(self):
        """Starts the download of the last step's rho / vel / cg (bclbm_macros_begin)."""
        _native.check(_native.lib().bclbm_macros_begin(self._h), self._h)

    def macros_collect(self, rho=None, vel=None, cg=None):
        """Waits for the download started by macros_begin and returns (rho, vel, cg)."""
        rho, vel, cg = self._macro_arrays(rho, vel, cg)
        _native.check(_native.lib().bclbm_macros_collect(self._h, _native.dp(rho), _native.dp(vel),
                                                         _native.dp(cg)), self._h)
        return rho, vel, cg

    def reduce(self) -> dict:
        return _native.reduce(self._h)

    def pressure_flux(self) -> np.ndarray:
        """std_one_phase: the write step's (q1, q2), 0.5 * sum of rho u_z over the
        pressure-boundary nodes of each phase after the last step."""
        q = np.zeros(2)
        _native.check(_native.lib().bclbm_pressure_flux(self._h, _native.dp(q)), self._h)
        return q

    def set_force(self, force):
        F = np.zeros(3)
        F[:len(force)] = force
        _native.check(_native.lib().bclbm_set_force(self._h, _native.dp(F)), self._h)

    def node_perm(self) -> np.ndarray:
        out = np.zeros(self.lat.n_bulk, dtype=np.int32)
        _native.check(_native.lib().bclbm_node_perm(self._h, _native.ip(out)), self._h)
        return out

    def sync(self):
        _native.check(_native.lib().bclbm_sync(self._h), self._h)

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().bclbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
