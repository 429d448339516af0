"""A compiled C++ program calls the C ABI on the GPU, with no Python in its path.

tests/abi_caller.cpp includes include/bclbm.h only and links libbclbm.so; it
runs the shape of the reference's std_case loop (src/std_case/main.cpp:109-157:
one bclbm_step per iteration, bclbm_download_macros on output steps) on the
256x64 channel of the golden fixtures for its 20,000 steps and writes f, rho
and u in the reference's layout.  The exact FP64 step must equal the
reference's own output bit for bit, the default (fixed-point) FP64 step within
1e-12.
"""

import subprocess
from pathlib import Path

import numpy as np
import pytest

import lbcases

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def caller(tmp_path_factory, gpu):
    exe = tmp_path_factory.mktemp("abi_caller") / "abi_caller"
    lib = REPO / "badchimp-cpp_gb300"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", f"-I{REPO / 'include'}", str(REPO / "tests" / "abi_caller.cpp"),
           "-o", str(exe), f"-L{lib}", "-lbclbm", f"-Wl,-rpath,{lib}"]
    subprocess.run(cmd, check=True)
    return exe


def relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("flags", [1, 0], ids=["exact", "fixed_point"])
def test_cpp_caller_channel_20000_steps(bclbm, caller, tmp_path, flags):
    case = lbcases.Case("channel_256x64", bclbm)
    run = case.runs["bgk_20000"]
    exp = case.expected("bgk_20000")
    f0, _ = case.init(run)
    (tmp_path / "meta.txt").write_text(f"{case.nq} {case.n_nodes} {case.lat.bulk.size} {run['steps']} 5000 "
                                       f"{run['tau']!r} {run['fx']!r} 0 0\n")
    case.lat.neigh.astype(np.int32).tofile(tmp_path / "neigh.i32")
    case.lat.types.astype(np.int16).tofile(tmp_path / "types.i16")
    case.lat.bulk.astype(np.int32).tofile(tmp_path / "bulk.i32")
    np.asarray(f0, dtype=np.float64).tofile(tmp_path / "f.f64")
    res = subprocess.run([str(caller), str(tmp_path), str(flags)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and res.stdout.startswith("ok 20000 "), res.stdout + res.stderr
    b = case.lat.bulk
    f = np.fromfile(tmp_path / f"out_{flags}_f.f64").reshape(case.n_nodes, case.nq)[b]
    rho = np.fromfile(tmp_path / f"out_{flags}_rho.f64")[b]
    vel = np.fromfile(tmp_path / f"out_{flags}_vel.f64").reshape(case.n_nodes, case.nd)[b]
    ef = exp["f"].reshape(-1, case.nq)  # the fixtures hold the bulk rows
    erho = exp["rho"].reshape(-1)
    evel = exp["vel"].reshape(-1, case.nd)
    if flags == 1:
        assert np.array_equal(f, ef)
        assert np.array_equal(rho, erho)
        assert np.array_equal(vel, evel)
    else:
        assert relerr(f, ef) <= 1e-12
        assert relerr(rho, erho) <= 1e-12
        floor = 8 * np.finfo(np.float64).eps * np.abs(ef).max() * np.sqrt(run["steps"])
        assert np.abs(vel - evel).max() <= max(1e-12 * np.abs(evel).max(), floor)
