"""ctypes binding of the C ABI in include/bclbm.h (libbclbm.so, built in-tree).

There is no fallback: if the shared library is missing or fails to load, every
entry point raises.  The library is loaded from this package's folder only.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_NAME = "libbclbm.so"
_lib = None


class BclbmError(RuntimeError):
    pass


class Desc(ctypes.Structure):
    _fields_ = [
        ("lattice_q", ctypes.c_int32),
        ("n_nodes", ctypes.c_int32),
        ("neigh", ctypes.c_void_p),
        ("types", ctypes.c_void_p),
        ("n_bulk", ctypes.c_int32),
        ("bulk", ctypes.c_void_p),
        ("pos", ctypes.c_void_p),
        ("collision", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("flags", ctypes.c_uint32),
        ("tau", ctypes.c_double * 2),
        ("force", ctypes.c_double * 3),
        ("sigma", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("flux_control", ctypes.c_int32),
        ("mom_x", ctypes.c_double),
        ("rho_ref", ctypes.c_double),
        ("store_scale", ctypes.c_double),
        ("f_init", ctypes.c_void_p),
        ("rho_init", ctypes.c_void_p),
        ("tags", ctypes.c_void_p),
        ("labels", ctypes.c_void_p),
        ("force_on", ctypes.c_void_p),
        ("rho_w", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("mass", ctypes.c_double * 2),
        ("momentum", ctypes.c_double * 3),
        ("flux_fc", ctypes.c_double * 3),
        ("saturation", ctypes.c_double),
        ("max_abs_f", ctypes.c_double),
        ("n_bulk", ctypes.c_int64),
        ("steps_done", ctypes.c_int64),
        ("nonfinite", ctypes.c_int32),
    ]


class Timing(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_double), ("step_kernel_ms", ctypes.c_double),
                ("density_ms", ctypes.c_double), ("launches", ctypes.c_int64), ("nsteps", ctypes.c_int32)]


EXPORTS = ["bclbm_create", "bclbm_step", "bclbm_step_timed", "bclbm_download_f", "bclbm_download_macros",
           "bclbm_macros_begin", "bclbm_macros_collect", "bclbm_reduce", "bclbm_set_force", "bclbm_pressure_flux", "bclbm_node_perm",
           "bclbm_footprint", "bclbm_sync", "bclbm_destroy", "bclbm_trim", "bclbm_error", "bclbm_last_error", "bclbm_launch_count",
           "bclbm_moments_static", "bclbm_batch_create", "bclbm_batch_admit", "bclbm_batch_admit_steps",
           "bclbm_batch_attach", "bclbm_batch_retire", "bclbm_batch_step", "bclbm_batch_stats",
           "bclbm_batch_download_f", "bclbm_batch_info", "bclbm_batch_sync", "bclbm_batch_last_error",
           "bclbm_batch_destroy", "bclbm_lattice_build", "bclbm_lattice_info", "bclbm_lattice_export",
           "bclbm_lattice_free", "bclbm_lattice_read_vtklb", "bclbm_lattice_attribute", "bclbm_output_create",
           "bclbm_output_add_file", "bclbm_output_add_field", "bclbm_output_add_array", "bclbm_output_write",
           "bclbm_output_write_async", "bclbm_output_wait", "bclbm_output_info", "bclbm_output_last_error",
           "bclbm_output_destroy"]


def lib_path() -> Path:
    return HERE / LIB_NAME


def lib():
    """Loads libbclbm.so (raising if it is absent) and declares the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not path.exists():
        raise BclbmError(f"{path} is missing: build it with build() (nvcc, sm_103a); there is no CPU fallback")
    L = ctypes.CDLL(str(path))
    vp = ctypes.c_void_p
    L.bclbm_create.argtypes = [ctypes.POINTER(Desc), ctypes.POINTER(vp)]
    L.bclbm_create.restype = ctypes.c_int
    L.bclbm_step.argtypes = [vp, ctypes.c_int]
    L.bclbm_step.restype = ctypes.c_int
    L.bclbm_step_timed.argtypes = [vp, ctypes.c_int, ctypes.POINTER(Timing)]
    L.bclbm_step_timed.restype = ctypes.c_int
    L.bclbm_download_f.argtypes = [vp, vp]
    L.bclbm_download_f.restype = ctypes.c_int
    L.bclbm_download_macros.argtypes = [vp, vp, vp, vp]
    L.bclbm_download_macros.restype = ctypes.c_int
    L.bclbm_macros_begin.argtypes = [vp]
    L.bclbm_macros_begin.restype = ctypes.c_int
    L.bclbm_macros_collect.argtypes = [vp, vp, vp, vp]
    L.bclbm_macros_collect.restype = ctypes.c_int
    L.bclbm_reduce.argtypes = [vp, ctypes.POINTER(Stats)]
    L.bclbm_reduce.restype = ctypes.c_int
    L.bclbm_set_force.argtypes = [vp, vp]
    L.bclbm_pressure_flux.argtypes = [vp, vp]
    L.bclbm_pressure_flux.restype = ctypes.c_int
    L.bclbm_set_force.restype = ctypes.c_int
    L.bclbm_node_perm.argtypes = [vp, vp]
    L.bclbm_node_perm.restype = ctypes.c_int
    L.bclbm_footprint.argtypes = [ctypes.POINTER(Desc), ctypes.POINTER(ctypes.c_size_t)]
    L.bclbm_footprint.restype = ctypes.c_int
    L.bclbm_sync.argtypes = [vp]
    L.bclbm_sync.restype = ctypes.c_int
    L.bclbm_destroy.argtypes = [vp]
    L.bclbm_destroy.restype = None
    L.bclbm_trim.argtypes = []
    L.bclbm_trim.restype = ctypes.c_int
    L.bclbm_error.argtypes = [ctypes.c_int]
    L.bclbm_error.restype = ctypes.c_char_p
    L.bclbm_last_error.argtypes = [vp]
    L.bclbm_last_error.restype = ctypes.c_char_p
    L.bclbm_launch_count.argtypes = []
    L.bclbm_launch_count.restype = ctypes.c_int64
    L.bclbm_moments_static.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_int32, vp, ctypes.c_double, ctypes.c_double, vp, vp]
    L.bclbm_moments_static.restype = ctypes.c_int
    i32 = ctypes.c_int32
    L.bclbm_batch_create.argtypes = [i32, i32, i32, ctypes.c_uint32, i32, ctypes.c_size_t, i32, ctypes.POINTER(vp)]
    L.bclbm_batch_admit.argtypes = [vp, ctypes.POINTER(Desc), ctypes.POINTER(i32)]
    L.bclbm_batch_admit_steps.argtypes = [vp, ctypes.POINTER(Desc), i32, ctypes.POINTER(i32)]
    L.bclbm_batch_attach.argtypes = [vp, vp, ctypes.POINTER(i32)]
    L.bclbm_batch_retire.argtypes = [vp, i32]
    L.bclbm_batch_step.argtypes = [vp, i32]
    L.bclbm_batch_stats.argtypes = [vp, i32, vp, ctypes.POINTER(Stats)]
    L.bclbm_batch_download_f.argtypes = [vp, i32, vp]
    L.bclbm_batch_info.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(i32),
                                   ctypes.POINTER(ctypes.c_int64)]
    L.bclbm_batch_sync.argtypes = [vp]
    for name in ("bclbm_batch_create", "bclbm_batch_admit", "bclbm_batch_admit_steps", "bclbm_batch_attach",
                 "bclbm_batch_retire", "bclbm_batch_step", "bclbm_batch_stats", "bclbm_batch_download_f",
                 "bclbm_batch_info", "bclbm_batch_sync"):
        getattr(L, name).restype = ctypes.c_int
    L.bclbm_batch_last_error.argtypes = [vp]
    L.bclbm_batch_last_error.restype = ctypes.c_char_p
    L.bclbm_batch_destroy.argtypes = [vp]
    L.bclbm_batch_destroy.restype = None
    i64p = ctypes.POINTER(ctypes.c_int64)
    L.bclbm_lattice_build.argtypes = [i32, i32, vp, vp, ctypes.c_uint32, ctypes.POINTER(vp)]
    L.bclbm_lattice_build.restype = ctypes.c_int
    L.bclbm_lattice_info.argtypes = [vp, i64p, i64p, i64p]
    L.bclbm_lattice_info.restype = ctypes.c_int
    L.bclbm_lattice_export.argtypes = [vp, vp, vp, vp]
    L.bclbm_lattice_export.restype = ctypes.c_int
    L.bclbm_lattice_free.argtypes = [vp]
    L.bclbm_lattice_free.restype = None
    L.bclbm_lattice_read_vtklb.argtypes = [ctypes.c_char_p, i32, ctypes.POINTER(vp)]
    L.bclbm_lattice_read_vtklb.restype = ctypes.c_int
    L.bclbm_lattice_attribute.argtypes = [vp, ctypes.c_char_p, vp]
    L.bclbm_lattice_attribute.restype = ctypes.c_int
    L.bclbm_output_create.argtypes = [i32, ctypes.c_int64, vp, vp, ctypes.c_char_p, i32, i32, i32, i32,
                                      ctypes.POINTER(vp)]
    L.bclbm_output_add_file.argtypes = [vp, ctypes.c_char_p]
    L.bclbm_output_add_field.argtypes = [vp, ctypes.c_char_p, vp, i32, i32, i32]
    L.bclbm_output_add_array.argtypes = [vp, ctypes.c_char_p, vp, i32, ctypes.c_int64]
    L.bclbm_output_write.argtypes = [vp, ctypes.c_double]
    L.bclbm_output_write_async.argtypes = [vp, ctypes.c_double]
    L.bclbm_output_wait.argtypes = [vp]
    L.bclbm_output_info.argtypes = [vp, i64p, i64p, ctypes.POINTER(i32)]
    for name in ("bclbm_output_create", "bclbm_output_add_file", "bclbm_output_add_field", "bclbm_output_add_array",
                 "bclbm_output_write", "bclbm_output_write_async", "bclbm_output_wait", "bclbm_output_info"):
        getattr(L, name).restype = ctypes.c_int
    L.bclbm_output_last_error.argtypes = [vp]
    L.bclbm_output_last_error.restype = ctypes.c_char_p
    L.bclbm_output_destroy.argtypes = [vp]
    L.bclbm_output_destroy.restype = None
    _lib = L
    return L


def dp(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


ip = dp


def check(rc: int, handle=None, batch=None, output=None):
    if rc != 0:
        msg = lib().bclbm_error(rc).decode()
        if handle or batch or output:
            if handle:
                detail = lib().bclbm_last_error(handle)
            elif batch:
                detail = lib().bclbm_batch_last_error(batch)
            else:
                detail = lib().bclbm_output_last_error(output)
            if detail:
                msg += ": " + detail.decode()
        err = BclbmError(f"bclbm status {rc}: {msg}")
        err.status = rc
        raise err


def make_desc(lat, f_init, collision, precision, flags, tau, force, sigma, beta, flux_control, mom_x, rho_ref,
              store_scale, rho_init, links=None):
    d = Desc()
    d.lattice_q = lat.nq
    d.n_nodes = lat.n_nodes
    d.neigh = lat.neigh.ctypes.data
    d.types = lat.types.ctypes.data
    d.n_bulk = lat.n_bulk
    d.bulk = lat.bulk.ctypes.data
    d.pos = lat.pos.ctypes.data if lat.pos is not None else None
    d.collision = int(collision)
    d.precision = int(precision)
    d.flags = int(flags)
    d.tau[0], d.tau[1] = float(tau[0]), float(tau[1])
    for k in range(3):
        d.force[k] = float(force[k])
    d.sigma = float(sigma)
    d.beta = float(beta)
    d.flux_control = int(flux_control)
    d.mom_x = float(mom_x)
    d.rho_ref = float(rho_ref)
    d.store_scale = float(store_scale)
    d.f_init = f_init.ctypes.data if f_init is not None else None
    d.rho_init = rho_init.ctypes.data if rho_init is not None else None
    if links is not None:  # (tags, labels, force_on or None, rho_w): int32 [N] arrays the caller keeps alive
        tags, labels, force_on, rho_w = links
        d.tags = tags.ctypes.data
        d.labels = labels.ctypes.data
        d.force_on = force_on.ctypes.data if force_on is not None else None
        d.rho_w = float(rho_w)
    return d


def create(lat, f_init, collision, precision, flags, tau, force, sigma, beta, flux_control, mom_x, rho_ref,
           store_scale, rho_init, links=None):
    d = make_desc(lat, f_init, collision, precision, flags, tau, force, sigma, beta, flux_control, mom_x, rho_ref,
                  store_scale, rho_init, links)
    h = ctypes.c_void_p()
    rc = lib().bclbm_create(ctypes.byref(d), ctypes.byref(h))
    check(rc)
    return h


def footprint(lat, collision, precision, flags=0):
    d = make_desc(lat, None, collision, precision, flags, (1.0, 1.0), (0.0, 0.0, 0.0), 0.0, 0.0, 0, 0.0, 1.0, 0.0,
                  None)
    n = ctypes.c_size_t()
    check(lib().bclbm_footprint(ctypes.byref(d), ctypes.byref(n)))
    return int(n.value)


def stats_dict(s: Stats) -> dict:
    return {"mass": list(s.mass), "momentum": list(s.momentum), "flux_fc": list(s.flux_fc),
            "saturation": s.saturation, "max_abs_f": s.max_abs_f, "n_bulk": s.n_bulk,
            "steps_done": s.steps_done, "nonfinite": bool(s.nonfinite)}


def reduce(h) -> dict:
    s = Stats()
    check(lib().bclbm_reduce(h, ctypes.byref(s)), h)
    return stats_dict(s)


def step_timed(h, nsteps: int) -> dict:
    t = Timing()
    check(lib().bclbm_step_timed(h, int(nsteps), ctypes.byref(t)), h)
    return {"total_ms": t.total_ms, "step_kernel_ms": t.step_kernel_ms, "density_ms": t.density_ms,
            "launches": int(t.launches), "nsteps": int(t.nsteps)}


def launch_count() -> int:
    return int(lib().bclbm_launch_count())


def read_vtklb(path, nq: int, attributes=()):
    """bclbm_lattice_read_vtklb: (neigh, types, pos, nf, ns, {name: [N] doubles})."""
    h = ctypes.c_void_p()
    check(lib().bclbm_lattice_read_vtklb(str(path).encode(), nq, ctypes.byref(h)))
    try:
        n, nf, ns = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().bclbm_lattice_info(h, ctypes.byref(n), ctypes.byref(nf), ctypes.byref(ns)))
        nd = 2 if nq == 9 else 3
        neigh = np.empty(n.value * nq, dtype=np.int32)
        types = np.empty(n.value, dtype=np.int16)
        pos = np.empty(n.value * nd, dtype=np.int32)
        check(lib().bclbm_lattice_export(h, dp(neigh), dp(types), dp(pos)))
        attrs = {}
        for name in attributes:
            a = np.empty(n.value)
            check(lib().bclbm_lattice_attribute(h, name.encode(), dp(a)))
            attrs[name] = a
    finally:
        lib().bclbm_lattice_free(h)
    return neigh, types, pos, int(nf.value), int(ns.value), attrs


def lattice_tables(mask, nq: int, periodic_bits: int):
    """bclbm_lattice_build: (neigh int32 [N*Q], types int16 [N], pos int32 [N*nD], nf, ns)."""
    m = np.ascontiguousarray(mask, dtype=np.int8)
    shape = np.asarray(m.shape, dtype=np.int32)
    h = ctypes.c_void_p()
    check(lib().bclbm_lattice_build(nq, m.ndim, dp(shape), dp(m), periodic_bits, ctypes.byref(h)))
    try:
        n, nf, ns = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().bclbm_lattice_info(h, ctypes.byref(n), ctypes.byref(nf), ctypes.byref(ns)))
        neigh = np.empty(n.value * nq, dtype=np.int32)
        types = np.empty(n.value, dtype=np.int16)
        pos = np.empty(n.value * m.ndim, dtype=np.int32)
        check(lib().bclbm_lattice_export(h, dp(neigh), dp(types), dp(pos)))
    finally:
        lib().bclbm_lattice_free(h)
    return neigh, types, pos, int(nf.value), int(ns.value)
