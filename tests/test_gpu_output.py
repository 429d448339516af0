"""The output step end to end on the GPU: the device moments downloaded into the
fields an Output reads and written as VTU, against the reference's own rho/vel
of the same run (bit-identical with the exact FP64 step), and the asynchronous
write overlapping the next steps giving the same file as a synchronous one."""

import re

import numpy as np
import pytest

import lbcases
from test_vtu import read_appended

pytestmark = pytest.mark.gpu


def test_vtu_of_device_moments_equals_reference(bclbm, gpu, tmp_path):
    case = lbcases.Case("channel_256x64", bclbm)
    run = case.runs["bgk_100"]
    exp = case.expected("bgk_100")
    L = case.L
    f0, _ = case.init(run)
    lat = case.lat
    rho = np.zeros((lat.n_nodes, 1))
    vel = np.zeros((lat.n_nodes, 1, 2))
    with L.Solver(lat, f0, collision=L.BGK, tau=(run["tau"], run["tau"]), force=case.force(run), exact=True) as s, \
            bclbm.output.Output(lat, lat.bulk, tmp_path / "out") as o:
        o.add_file("lb_run")
        o.add_scalar_variables(["rho"], [rho])
        o.add_vector_variables(["vel"], [vel])
        s.step(run["steps"])
        s.download_macros(rho.reshape(-1), vel.reshape(-1))
        o.write(run["steps"])
        # the same values, written on the writer thread while the GPU takes more steps
        o.write_async(run["steps"])
        s.step(200)
        o.wait()
    arr = read_appended(tmp_path / "out" / "vtu" / "0000_lb_run_0000000.vtu")
    assert np.array_equal(arr["rho"], exp["rho"][:, 0])
    v3 = arr["vel"].reshape(-1, 3)
    assert np.array_equal(v3[:, :2], exp["vel"][:, 0, :]) and np.all(v3[:, 2] == 0.0)
    a = (tmp_path / "out" / "vtu" / "0000_lb_run_0000000.vtu").read_bytes()
    b = (tmp_path / "out" / "vtu" / "0000_lb_run_0000001.vtu").read_bytes()
    assert a == b
    p = (tmp_path / "out" / "lb_run_0000001.pvtu").read_bytes()
    assert re.search(rb"<!-- time = 100 s -->", p)
