"""The C ABI library: loads, exports every declared entry point, validates
descriptors on the host (no GPU needed for these calls)."""

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import lbcases

HEADER = Path(__file__).resolve().parent.parent / "include" / "bclbm.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bclbm_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native_lib):
    names = declared_functions()
    assert "bclbm_create" in names and "bclbm_step" in names
    for n in names:
        assert hasattr(native_lib, n), n


def test_python_binding_lists_every_export(bclbm):
    assert sorted(bclbm.native.EXPORTS) == declared_functions()


def test_trim_without_device_memory_is_a_no_op(native_lib):
    assert native_lib.bclbm_trim() == 0


def test_error_strings(native_lib):
    assert native_lib.bclbm_error(0) == b"ok"
    assert native_lib.bclbm_error(-2).startswith(b"inconsistent")
    assert native_lib.bclbm_error(-999) == b"unknown status"


def test_footprint_on_host(bclbm, native_lib):
    case = lbcases.Case("pack_20", bclbm)
    n64 = bclbm.native.footprint(case.lat, bclbm.lbsolver.BGK, bclbm.lbsolver.F64)
    n16 = bclbm.native.footprint(case.lat, bclbm.lbsolver.BGK, bclbm.lbsolver.F16)
    nrk = bclbm.native.footprint(case.lat, bclbm.lbsolver.RK, bclbm.lbsolver.F64)
    pad = (case.nf + 63) // 64 * 64
    assert n64 >= 2 * 19 * pad * 8 + 18 * pad * 4
    assert n16 < n64 and nrk > n64


def _create_rc(bclbm, lat, f_init, **kw):
    N = bclbm.native
    d = N.make_desc(lat, f_init, kw.get("collision", 0), kw.get("precision", 0), kw.get("flags", 0),
                    kw.get("tau", (0.8, 0.8)), (0.0, 0.0, 0.0), kw.get("sigma", 0.0), 0.0, kw.get("flux", 0), 0.0,
                    1.0, 0.0, kw.get("rho_init"))
    h = ctypes.c_void_p()
    return N.lib().bclbm_create(ctypes.byref(d), ctypes.byref(h))


def test_create_rejects_asymmetric_table(bclbm, native_lib):
    case = lbcases.Case("pack_20", bclbm)
    lat = case.lat
    neigh = lat.neigh.copy().reshape(-1, 19)
    x = int(lat.bulk[5])
    y = neigh[x, 9]  # upstream along c_0
    # point some other fluid node's +x link at x as well: two pushers into one slot
    z = int(lat.bulk[40])
    if lat.types[y] > 1 and z != y:
        neigh[z, 0] = x
    bad = bclbm.lbsolver.Lattice(19, neigh.reshape(-1), lat.types, lat.pos, lat.bulk)
    f0 = bclbm.lbsolver.initiate_single(bad, np.ones(bad.n_nodes))
    assert _create_rc(bclbm, bad, f0) == -2


def test_create_rejects_out_of_range_neighbour(bclbm, native_lib):
    case = lbcases.Case("box_12x10x8", bclbm)
    neigh = case.lat.neigh.copy()
    neigh[19 * 3 + 2] = case.n_nodes + 5
    bad = bclbm.lbsolver.Lattice(19, neigh, case.lat.types, case.lat.pos, case.lat.bulk)
    f0 = bclbm.lbsolver.initiate_single(bad, np.ones(bad.n_nodes))
    assert _create_rc(bclbm, bad, f0) == -2


def test_create_rejects_bad_descriptor(bclbm, native_lib):
    case = lbcases.Case("box_12x10x8", bclbm)
    f0 = bclbm.lbsolver.initiate_single(case.lat, np.ones(case.n_nodes))
    assert _create_rc(bclbm, case.lat, f0, precision=7) == -1
    assert _create_rc(bclbm, case.lat, f0, precision=2, flags=1) == -1  # exact needs F64
    assert _create_rc(bclbm, case.lat, None) == -1


def test_create_rejects_modes_outside_their_range(bclbm, native_lib, capfd):
    """Descriptor checks made before any device work: the fixed-point FP64 step's
    parameter ranges and the one-pass two-phase step's requirements."""
    L = bclbm.lbsolver
    case = lbcases.Case("box_12x10x8", bclbm)
    f0 = L.initiate_single(case.lat, np.ones(case.n_nodes))
    assert _create_rc(bclbm, case.lat, f0, tau=(0.5, 0.5)) == -1
    assert "tau > 0.5" in capfd.readouterr().err
    assert _create_rc(bclbm, case.lat, f0, flags=L.FLAG_LAGGED_COLOUR) == -1  # single phase
    assert "BCLBM_FLAG_LAGGED_COLOUR" in capfd.readouterr().err
    ones = np.ones(case.n_nodes)
    f2, rho = L.initiate_twophase(case.lat, ones, 0 * ones, ones)
    rk = dict(collision=L.RK, rho_init=rho)
    assert _create_rc(bclbm, case.lat, f2, precision=L.F64, flags=L.FLAG_LAGGED_COLOUR, **rk) == -1
    assert "BCLBM_FLAG_LAGGED_COLOUR" in capfd.readouterr().err
    assert _create_rc(bclbm, case.lat, f2, precision=L.F16, flags=L.FLAG_LAGGED_COLOUR, flux=1, **rk) == -1
    assert "constant body force" in capfd.readouterr().err
    assert _create_rc(bclbm, case.lat, f2, precision=L.F64, sigma=4.0, **rk) == -1
    assert "sigma" in capfd.readouterr().err


def test_create_rejects_element_numbers_past_int32(bclbm, native_lib, capfd):
    """Q x n_bulk rounded up to 64 must stay at most 2^31 - 1 (the 32-bit element
    numbers of the pull): checked on the descriptor before any array is read, so
    the sizes alone are enough (two-phase, whose create reads no array before it)."""
    N = bclbm.native
    L = bclbm.lbsolver
    case = lbcases.Case("box_12x10x8", bclbm)
    ones = np.ones(case.n_nodes)
    f2, rho = L.initiate_twophase(case.lat, ones, 0 * ones, ones)
    d = N.make_desc(case.lat, f2, L.RK, L.F16, 0, (0.8, 0.8), (0.0, 0.0, 0.0), 0.0, 0.0, 0, 0.0, 1.0, 0.0, rho)
    d.n_bulk = 113_025_409  # rounded up: 113,025,472 x 19 = 2,147,483,968
    d.n_nodes = d.n_bulk + 1
    h = ctypes.c_void_p()
    assert N.lib().bclbm_create(ctypes.byref(d), ctypes.byref(h)) == -5
    assert "int32 element numbers" in capfd.readouterr().err
    assert not h.value


def test_missing_library_fails_loudly(bclbm, tmp_path, monkeypatch):
    N = bclbm.native
    monkeypatch.setattr(N, "_lib", None)
    monkeypatch.setattr(N, "HERE", tmp_path)
    with pytest.raises(N.BclbmError):
        N.lib()


def test_batch_create_validates_on_host(bclbm, native_lib):
    b = ctypes.c_void_p()
    L = bclbm.native.lib()
    assert L.bclbm_batch_create(19, 0, 0, 0, 4, 1 << 30, 50, None) == -1
    assert L.bclbm_batch_create(7, 0, 0, 0, 4, 1 << 30, 50, ctypes.byref(b)) == -1
    assert L.bclbm_batch_create(19, 2, 0, 0, 4, 1 << 30, 50, ctypes.byref(b)) == -1  # RK is not batched
    assert L.bclbm_batch_create(19, 0, 5, 0, 4, 1 << 30, 50, ctypes.byref(b)) == -1
    assert L.bclbm_batch_create(19, 0, 0, 0, 0, 1 << 30, 50, ctypes.byref(b)) == -1
    assert L.bclbm_batch_create(19, 0, 0, 1, 4, 1 << 30, 50, ctypes.byref(b)) == -5  # reference order not batched
    assert not b.value
    assert L.bclbm_batch_admit(None, None, None) == -1
    assert L.bclbm_batch_step(None, 1) == -1
    L.bclbm_batch_destroy(None)


def test_batch_create_without_gpu_says_so(bclbm, native_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    b = ctypes.c_void_p()
    assert bclbm.native.lib().bclbm_batch_create(19, 0, 2, 0, 4, 1 << 30, 50, ctypes.byref(b)) == -8
