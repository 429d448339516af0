"""Host logic of the serving loop (no GPU): the request generator and the
convergence rule."""

import math

import numpy as np


def test_request_distribution(bclbm):
    S = bclbm.serving
    reqs = S.sample_requests(4000, rate=50.0, seed=3)
    sizes = np.array([r.size for r in reqs])
    assert sizes.min() >= 32 and sizes.max() <= 256
    # log-uniform: about a third of the sides below 64, a third above 128
    assert abs(np.mean(sizes < 64) - 1 / 3) < 0.03 and abs(np.mean(sizes > 128) - 1 / 3) < 0.03
    rad = np.array([r.radius for r in reqs])
    por = np.array([r.porosity for r in reqs])
    tau = np.array([r.tau for r in reqs])
    assert 4.0 <= rad.min() and rad.max() <= 12.0 and abs(rad.mean() - 8.0) < 0.2
    assert 0.30 <= por.min() and por.max() <= 0.50
    assert 0.6 <= tau.min() and tau.max() <= 1.2
    arr = np.array([r.arrival for r in reqs])
    gaps = np.diff(arr)
    assert np.all(gaps >= 0)
    assert abs(gaps.mean() - 1 / 50.0) / (1 / 50.0) < 0.06  # Poisson: exponential gaps at the rate
    assert S.sample_requests(5, rate=0.0, seed=3)[4].arrival == 0.0
    a = S.sample_requests(10, rate=1.0, seed=9)
    b = S.sample_requests(10, rate=1.0, seed=9)
    assert [(r.seed, r.size, r.tau) for r in a] == [(r.seed, r.size, r.tau) for r in b]


def test_convergence_rule(bclbm):
    srv = bclbm.serving.Server(check_every=500, tol=1e-6, max_steps=50000)
    assert srv._done(None, 1.0, 501) == (False, False)
    assert srv._done(1.0, 1.0 + 5e-7, 1001) == (True, True)
    assert srv._done(1.0, 1.0 + 5e-6, 1001) == (False, False)
    assert srv._done(1.0, 1.1, 50001) == (True, False)


def test_permeability_formula(bclbm):
    S = bclbm.serving
    r = S.Request(rid=0, seed=1, size=10, radius=4.0, porosity=0.4, tau=0.8, gx=1e-5)
    assert math.isclose(S.permeability(2.0, r), (0.3 / 3.0) * 2.0 / (1000 * 1e-5))


def test_summary_percentiles(bclbm):
    S = bclbm.serving
    res = [S.Result(i, 1.0, 10, True, 0.0, 0.0, float(i + 1), 5) for i in range(100)]
    rep = S.summarize(res, 0.0, 100.0)
    assert rep["solves_per_s"] == 1.0 and rep["lattice_updates"] == 100 * 50
    assert abs(rep["p50_s"] - 50.5) < 1e-9 and abs(rep["p99_s"] - 99.01) < 1e-9


def test_lblbf_round_trip_and_header(bclbm, tmp_path):
    L = bclbm.lbsolver
    f = np.random.default_rng(1).random(7 * 2 * 19)
    p = tmp_path / "x.lblbf"
    L.write_lblbf(p, f, 2, 19)
    raw = p.read_bytes()
    assert np.frombuffer(raw[:12], dtype="<i4").tolist() == [2, 19, 7]
    assert len(raw) == 12 + f.size * 8
    g, nf, nq, n = L.read_lblbf(p)
    assert (nf, nq, n) == (2, 19, 7) and np.array_equal(f, g)
    (tmp_path / "bad.lblbf").write_bytes(raw[:-8])
    import pytest
    with pytest.raises(ValueError):
        L.read_lblbf(tmp_path / "bad.lblbf")
