"""The oracle (plain-C restatement) pinned against the reference's own outputs.

The golden fixtures were produced by running the reference lbsolver itself
(tests/golden/make_golden.py); the oracle must reproduce every population,
density, velocity, colour value and flux-controller force bit for bit.
"""

import numpy as np
import pytest

import lbcases

RUNS = lbcases.all_runs()


@pytest.mark.parametrize("name,tag", RUNS, ids=[f"{n}-{t}" for n, t in RUNS])
def test_oracle_bit_exact_vs_reference(bclbm, oracle, name, tag):
    case = lbcases.Case(name, bclbm)
    run = case.runs[tag]
    f0, rho0 = case.init(run)
    g = oracle.OracleGrid(case.nq, case.lat.neigh, case.lat.types, case.lat.bulk)
    exp = case.expected(tag)
    nthreads = oracle.default_threads()
    if run["mode"] == "single":
        f, rho, vel = oracle.single_run(g, f0, run["steps"], run["tau"], case.force(run), trt=run.get("trt", 0),
                                        tau_anti=run.get("tau_anti", 1.0), nthreads=nthreads)
        assert np.array_equal(case.bulk_rows(f, 1), exp["f"])
        assert np.array_equal(rho[case.lat.bulk], exp["rho"][:, 0])
        assert np.array_equal(vel.reshape(-1, case.nd)[case.lat.bulk], exp["vel"][:, 0, :])
    else:
        f, rho, vel, cg, log = oracle.twophase_run(g, f0, rho0, run["steps"], run["tau0"], run["tau1"],
                                                   run["sigma"], run["beta"], case.force(run),
                                                   mom_x=run.get("momx"), nthreads=nthreads)
        assert np.array_equal(case.bulk_rows(f, 2), exp["f"])
        assert np.array_equal(rho.reshape(-1, 2)[case.lat.bulk], exp["rho"])
        assert np.array_equal(vel.reshape(-1, case.nd)[case.lat.bulk], exp["vel"][:, 0, :])
        assert np.array_equal(cg, exp["cg"])
        assert np.array_equal(log, exp["force"])


def test_oracle_thread_count_does_not_change_results(bclbm, oracle):
    case = lbcases.Case("pack_20", bclbm)
    run = case.runs["bgk_500"]
    f0, _ = case.init(run)
    g = oracle.OracleGrid(case.nq, case.lat.neigh, case.lat.types, case.lat.bulk)
    a = oracle.single_run(g, f0.copy(), 30, 0.8, case.force(run), nthreads=1)[0]
    b = oracle.single_run(g, f0.copy(), 30, 0.8, case.force(run), nthreads=4)[0]
    assert np.array_equal(a, b)


def test_poiseuille_known_answer(bclbm):
    """The 256x64 channel after 20,000 reference steps against the analytic channel profile
    u(y) = g/(2 nu) (y - y0)(y1 - y), walls half-way between nodes: the profile's
    relative L2 error stays near 1e-4 (the slowest diffusive mode has not decayed)."""
    case = lbcases.Case("channel_256x64", bclbm)
    vel = case.expected("bgk_20000")["vel"][:, 0, :]
    y = case.lat.pos.reshape(-1, 2)[case.lat.bulk, 1].astype(np.float64)
    nu = (1.0 - 0.5) / 3.0
    g = 1e-6
    y0, y1 = 0.5, 62.5
    u_an = g / (2 * nu) * (y - y0) * (y1 - y)
    err = np.linalg.norm(vel[:, 0] - u_an) / np.linalg.norm(u_an)
    assert err < 2e-4
    assert abs(vel[:, 0].max() - u_an.max()) / u_an.max() < 2e-4
    assert np.abs(vel[:, 1]).max() < 1e-14


def test_oracle_mass_conservation(bclbm, oracle):
    case = lbcases.Case("pack_20", bclbm)
    run = case.runs["rk_100"]
    f0, rho0 = case.init(run)
    g = oracle.OracleGrid(case.nq, case.lat.neigh, case.lat.types, case.lat.bulk)
    f, *_ = oracle.twophase_run(g, f0, rho0, 50, 1.0, 1.0, 0.01, 0.99, case.force(run))
    m0 = case.bulk_rows(f0, 2).sum(axis=(0, 2))
    m1 = case.bulk_rows(f, 2).sum(axis=(0, 2))
    assert np.allclose(m0, m1, rtol=1e-12, atol=0)
