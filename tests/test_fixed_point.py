"""The 64-bit fixed-point collision (csrc/bclbm_fixed.cuh) checked on the CPU.

The device kernel runs the same __host__ __device__ code; here its host
branch (128-bit multiplies) is compiled into a test-only library
(tests/fx_selfcheck.cu) and stepped through the reference fixtures with a
plain pull loop.  Tolerances are those of the FMA FP64 path.
"""

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import lbcases

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "badchimp-cpp_gb300" / "csrc"


@pytest.fixture(scope="module")
def fxlib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("fx") / "libfxcheck.so"
    subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-shared", "-Xcompiler", "-fPIC",
                    f"-I{CSRC}", str(HERE / "fx_selfcheck.cu"), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    vp = ctypes.c_void_p
    lib.fx_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp, ctypes.c_int,
                           ctypes.c_double, ctypes.c_double, vp, vp, vp, vp]
    lib.fx_primitives.argtypes = [vp, vp, ctypes.c_int]
    lib.fx_collide_ovf.argtypes = [ctypes.c_double]
    lib.fx_unit_normal_check.argtypes = [ctypes.c_int, ctypes.c_uint, vp]
    lib.fx_unit_normal_check.restype = None
    return lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def test_primitives_against_128bit_reference(fxlib):
    rng = np.random.default_rng(5)
    a = np.concatenate([rng.uniform(-7.9, 7.9, 20000), rng.uniform(-1e-3, 1e-3, 20000),
                        rng.uniform(0.01, 0.4, 20000), 10.0 ** rng.uniform(-17, 0, 20000)])
    b = np.concatenate([rng.uniform(-1.0, 1.0, 20000), rng.uniform(-2.0, 2.0, 20000),
                        rng.uniform(0.5, 1.5, 20000), rng.uniform(-1.0, 1.0, 20000)])
    # multipliers of the k-form products: [0, 1), with both ends
    a = np.concatenate([a, rng.uniform(-7.9, 7.9, 20000), [-7.999, 7.999, 0.0, -1e-18, 1e-18]])
    b = np.concatenate([b, rng.uniform(0.0, 1.0, 20000), [0.999999999, 0.0, 0.5, 1e-18, 0.999999999]])
    assert fxlib.fx_primitives(_p(a), _p(b), a.size) == 0


def test_colour_gradient_normal(fxlib):
    """The two-phase collision's |G| and G / |G| from the integer colour gradient
    (fx::unit_normal, the device code compiled for the host): the direction within
    2^-56 and |G| within 2^-51 of long-double norms, over 60 binary orders of
    magnitude of the gradient; below |G| = 2^-52 the reference's G / (|G| + 1) = G."""
    worst = np.zeros(3)
    fxlib.fx_unit_normal_check(400000, 7, _p(worst))
    assert worst[0] <= 2.0 ** -56, worst
    assert worst[1] <= 2.0 ** -51, worst
    assert worst[2] <= 2.0 ** -58, worst


def test_range_guard(fxlib):
    for rho, flagged in ((1.0, 0), (0.2, 0), (6.5, 0), (0.1, 1), (9.0, 1), (20.0, 1)):
        assert fxlib.fx_collide_ovf(rho) == flagged, rho


SINGLE = [(n, t) for n, t in lbcases.all_runs() if not t.startswith("rk")]


@pytest.mark.parametrize("name,tag", SINGLE, ids=[f"{n}-{t}" for n, t in SINGLE])
def test_fixed_point_step_matches_reference(bclbm, fxlib, name, tag):
    case = lbcases.Case(name, bclbm)
    run = case.runs[tag]
    if run["steps"] > 2000:
        pytest.skip("long run covered on the GPU")
    f0, _ = case.init(run)
    f = f0.copy()
    rho = np.zeros(case.n_nodes)
    vel = np.zeros(case.n_nodes * case.nd)
    F = np.zeros(3)
    F[:case.nd] = case.force(run)
    lat = case.lat
    ovf = fxlib.fx_run(case.nq, int(bool(run.get("trt"))), case.n_nodes, _p(lat.neigh), _p(lat.types), lat.n_bulk,
                       _p(lat.bulk), run["steps"], run["tau"], run.get("tau_anti", run["tau"]), _p(F), _p(f), _p(rho),
                       _p(vel))
    assert ovf == 0
    exp = case.expected(tag)
    got_f = case.bulk_rows(f, 1)
    assert np.linalg.norm(got_f - exp["f"]) / np.linalg.norm(exp["f"]) <= 1e-12
    assert np.linalg.norm(rho[lat.bulk] - exp["rho"][:, 0]) / np.linalg.norm(exp["rho"]) <= 1e-12
    eu = exp["vel"][:, 0, :]
    floor = 8 * np.finfo(np.float64).eps * np.abs(exp["f"]).max() * np.sqrt(run["steps"])
    assert np.abs(vel.reshape(-1, case.nd)[lat.bulk] - eu).max() <= max(1e-12 * np.abs(eu).max(), floor)
