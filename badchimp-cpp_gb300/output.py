"""The reference's VTU output step, written by libbclbm's native writer.

``Output`` mirrors ``Output<LT, T, FMT>`` of src/io/Output.h:26-177 (over
VTK::Output, src/io/VTK.h:1421-1550): the same constructors, ``add_file``,
``add_scalar_variables``, ``add_vector_variables``, ``add_variable_with_names``,
``add_variables`` and ``write``, and the same files, byte for byte
(``<dir>/<name>_<n:07>.pvtu`` and ``<dir>/vtu/<rank:04>_<name>_<n:07>.vtu``).

Fields are numpy arrays in the reference's layout: a ScalarField is
``[n_nodes]`` or ``[n_nodes, n_fields]`` (LBfield.h:69), a VectorField
``[n_nodes, n_dims]`` or ``[n_nodes, n_fields, n_dims]`` (LBfield.h:219).  As in
the reference the object keeps references to them and reads their values at
each ``write``; write the moments into the same arrays between writes (e.g.
with ``Solver.download_macros(rho, vel)``).

``write_async`` reads the values at the call and writes the files on a
background thread; the next call (or ``wait``) waits for it, so the host's
file write overlaps the GPU steps that follow.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import native as _native

FLOAT64, FLOAT32, INT32 = 0, 1, 2
BINARY, ASCII, BINARY64 = 0, 1, 2
_TYPES = {np.dtype(np.float64): FLOAT64, np.dtype(np.float32): FLOAT32, np.dtype(np.int32): INT32}


def _value_type(dtype) -> int:
    dt = np.dtype(dtype)
    if dt not in _TYPES:
        raise ValueError(f"output type {dt}: the writer writes float64, float32 or int32")
    return _TYPES[dt]


class Output:
    """Output(lattice, nodes, dir, rank=0, nproc=1, dtype=float64, fmt=BINARY):
    the Output(grid, nodes, dir, rank, nproc) form (Output.h:51-54): one cell per
    node of ``nodes`` at ``lattice.pos``.

    ``Output.from_positions(pos, nd, dir, ...)`` is the Output(pos, dir, rank,
    nproc[, varname, var]) form (Output.h:33-47), for plain vectors only."""

    def __init__(self, lattice, nodes, dir, rank: int = 0, nproc: int = 1, dtype=np.float64, fmt: int = BINARY,
                 _pos=None, _nd=None):
        L = _native.lib()
        if lattice is not None:
            if lattice.pos is None:
                raise ValueError("the lattice has no node positions")
            nd = lattice.nd
            nodes = np.ascontiguousarray(nodes, dtype=np.int32).reshape(-1)
            pos = np.ascontiguousarray(lattice.pos.reshape(-1, nd)[nodes], dtype=np.int32)
        else:
            nd = int(_nd)
            pos = np.ascontiguousarray(_pos, dtype=np.int32).reshape(-1, nd)
            nodes = None
        self.nd = nd
        self.n_cells = int(pos.shape[0])
        self._nodes = nodes
        self._pos = pos
        self._keep = []  # the arrays the writer reads
        self._dtype = np.dtype(dtype)
        h = ctypes.c_void_p()
        _native.check(L.bclbm_output_create(nd, self.n_cells, _native.dp(pos), _native.dp(nodes),
                                            os.fsencode(str(dir)), int(rank), int(nproc), _value_type(dtype),
                                            int(fmt), ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_positions(cls, pos, nd: int, dir, rank: int = 0, nproc: int = 1, varname=None, var=None,
                       dtype=np.float64, fmt: int = BINARY):
        o = cls(None, None, dir, rank, nproc, dtype, fmt, _pos=pos, _nd=nd)
        if varname is not None:
            o.add_file(varname)
            o.add_variables([varname], [var])
        return o

    # --- the reference's Output methods -------------------------------------------------
    def add_file(self, name: str):
        self._check(_native.lib().bclbm_output_add_file(self._handle(), name.encode()))

    def add_scalar_variables(self, names, fields):
        for name, f in zip(names, fields):
            self._add_field(name, f, 1)

    def add_vector_variables(self, names, fields):
        for name, f in zip(names, fields):
            self._add_field(name, f, self.nd)

    def add_variable_with_names(self, names, field, vector: bool = False):
        """One variable per field of a multi-field ScalarField / VectorField, named
        explicitly (Output.h:111-126)."""
        dim = self.nd if vector else 1
        a = self._field_array(field, dim)
        nf = a.size // (a.shape[0] * dim)
        if len(names) != nf:
            raise ValueError(f"size of names-vector does not match number of fields, {len(names)} != {nf}")
        for i, name in enumerate(names):
            self._add_field(name, a, dim, field_no=i)

    def add_variables(self, names, vectors):
        """Plain vectors (std::vector<T> in the reference), contiguous, one or nD
        values per cell."""
        for name, v in zip(names, vectors):
            a = np.asarray(v)
            if not a.flags.c_contiguous or a.dtype not in _TYPES:
                raise ValueError("vectors must be contiguous float64, float32 or int32 arrays")
            self._keep.append(a)
            self._check(_native.lib().bclbm_output_add_array(self._handle(), name.encode(), _native.dp(a),
                                                             _TYPES[a.dtype], a.size))

    def write(self, time: float = 0.0):
        self._check(_native.lib().bclbm_output_write(self._handle(), float(time)))

    def write_async(self, time: float = 0.0):
        self._check(_native.lib().bclbm_output_write_async(self._handle(), float(time)))

    def wait(self):
        self._check(_native.lib().bclbm_output_wait(self._handle()))

    @property
    def n_points(self) -> int:
        n = ctypes.c_int64()
        self._check(_native.lib().bclbm_output_info(self._handle(), ctypes.byref(n), None, None))
        return int(n.value)

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().bclbm_output_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- helpers ------------------------------------------------------------------------
    def _handle(self):
        if not getattr(self, "_h", None):
            raise _native.BclbmError("the output is closed")
        return self._h

    def _check(self, rc):
        _native.check(rc, output=self._h)

    def _field_array(self, f, dim):
        a = np.asarray(f)
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError("fields are contiguous float64 arrays in the reference layout (they are read at write)")
        if a.ndim == 1 and dim > 1:
            raise ValueError("a VectorField is [n_nodes, n_dims] or [n_nodes, n_fields, n_dims]")
        return a

    def _add_field(self, name, f, dim, field_no=-1):
        if self._nodes is None:
            raise ValueError("fields need the Output(lattice, nodes, ...) form")
        a = self._field_array(f, dim)
        n_nodes = a.shape[0]
        if a.size % (n_nodes * dim) != 0 or (dim > 1 and a.shape[-1] != dim):
            raise ValueError(f"field {name}: shape {a.shape} is not a field of {dim} components per node")
        nf = a.size // (n_nodes * dim)
        if self._nodes.size and int(self._nodes.max()) >= n_nodes:
            raise ValueError(f"field {name} has {n_nodes} nodes, the output writes node {int(self._nodes.max())}")
        self._keep.append(a)
        self._check(_native.lib().bclbm_output_add_field(self._handle(), name.encode(), _native.dp(a), nf, dim,
                                                         int(field_no)))
