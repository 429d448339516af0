"""Parity at the benchmark's own sizes, against the oracle on the host cores.

* D3Q19 single phase, the benchmark workload: periodic 256^3 sphere pack
  (radius 10, seeded centres, porosity 0.40), tau 0.8, gx 1e-5, 30 steps of
  the std_case loop (src/std_case/main.cpp:109-146).  The exact FP64 kernel is
  bit-identical to the oracle; the default fixed-point FP64 kernel, BGK and TRT
  (Lambda = 3/16, calcOmegaBGKTRT), is within 1e-12 in f and rho and within
  1e-12 of max |u| (or the rounding floor of sum_q f c_q) in u.
* D3Q19 Rothman-Keller two-phase on a periodic 96^3 pack (radius 8, porosity
  0.40, red/blue i.i.d. p = 0.5, tau 1/1, A = 0.01, beta = 0.99, neutral
  wetting, constant gx 1e-5), 100 steps of src/twophase/main_TWOPHASE.cpp:236-392:
  exact FP64 bit-identical in f, rho, u and the colour field, the default
  fixed-point FP64 and FP64 with FMA within 1e-12, FP16 shifted storage within
  its stated bounds.
* The two-phase mass-drift correction: FP16 storage over 2,000 steps with the
  correction keeps the saturation within 1e-7 of its start and much closer
  than without it (BCLBM_FLAG_NO_MASS_FIX).

The oracle (oracle/bclbm_oracle.c) is the plain-C restatement of those loops,
bit-identical to the reference's own build on every golden fixture.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZE, RADIUS, POROSITY, SEED, TAU, GX, STEPS = 256, 10.0, 0.40, 2024, 0.8, 1e-5, 30
TAU_ANTI = 0.5 + (3.0 / 16.0) / (TAU - 0.5)  # Lambda = (tau+ - 1/2)(tau- - 1/2) = 3/16


def relerr(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def u_bound(exp_vel, exp_f, steps):
    """|u - u_ref| bound: 1e-12 of max |u|, or the rounding floor of sum_q f c_q
    (8 eps max f sqrt(steps)) where that is larger."""
    floor = 8 * np.finfo(np.float64).eps * np.abs(exp_f).max() * np.sqrt(steps)
    return max(1e-12 * np.abs(exp_vel).max(), floor)


@pytest.fixture(scope="module")
def pack(bclbm, gpu):
    geo, _, phi = bclbm.geometry.sphere_pack((SIZE,) * 3, radius=RADIUS, porosity=POROSITY, seed=SEED)
    assert abs(phi - POROSITY) <= 0.01
    lat = bclbm.lbsolver.Lattice.from_geometry(geo, "D3Q19", "xyz")
    f0 = bclbm.lbsolver.initiate_single(lat, np.ones(lat.n_nodes))
    return lat, f0


@pytest.fixture(scope="module")
def oracle_runs(pack, oracle):
    """The oracle's f / rho / u after STEPS steps, BGK and TRT (bulk rows)."""
    lat, f0 = pack
    g = oracle.OracleGrid(lat.nq, lat.neigh, lat.types, lat.bulk)
    out = {}
    for trt in (False, True):
        f, rho, vel = oracle.single_run(g, f0.copy(), STEPS, TAU, (GX, 0.0, 0.0), trt=trt, tau_anti=TAU_ANTI,
                                        nthreads=oracle.default_threads())
        b = lat.bulk
        out[trt] = (f.reshape(-1, 19)[b].copy(), rho[b].copy(), vel.reshape(-1, 3)[b].copy())
    return out


def gpu_run(bclbm, lat, f0, trt, **kw):
    L = bclbm.lbsolver
    coll = L.TRT if trt else L.BGK
    with L.Solver(lat, f0, collision=coll, tau=(TAU, TAU_ANTI if trt else TAU), force=(GX, 0.0, 0.0), **kw) as s:
        s.step(STEPS)
        f = s.download_f(np.zeros_like(f0))
        rho, vel, _ = s.download_macros()
    b = lat.bulk
    return f.reshape(-1, 19)[b], rho[b], vel.reshape(-1, 3)[b]


def test_exact_f64_256_bit_identical(bclbm, pack, oracle_runs):
    lat, f0 = pack
    f, rho, vel = gpu_run(bclbm, lat, f0, False, exact=True)
    ef, erho, evel = oracle_runs[False]
    assert np.array_equal(f, ef)
    assert np.array_equal(rho, erho)
    assert np.array_equal(vel, evel)


@pytest.mark.parametrize("trt", [False, True], ids=["bgk", "trt"])
def test_fixed_point_f64_256_within_1e12(bclbm, pack, oracle_runs, trt):
    lat, f0 = pack
    f, rho, vel = gpu_run(bclbm, lat, f0, trt)
    ef, erho, evel = oracle_runs[trt]
    assert relerr(f, ef) <= 1e-12
    assert relerr(rho, erho) <= 1e-12
    assert np.abs(vel - evel).max() <= u_bound(evel, ef, STEPS)


# ---------------------------------------------------------------------------
# two-phase
# ---------------------------------------------------------------------------
TP_SIZE, TP_RADIUS, TP_STEPS = 96, 8.0, 100
SIGMA, BETA = 0.01, 0.99


@pytest.fixture(scope="module")
def tp_pack(bclbm, gpu):
    L = bclbm.lbsolver
    geo, _, phi = bclbm.geometry.sphere_pack((TP_SIZE,) * 3, radius=TP_RADIUS, porosity=POROSITY, seed=SEED)
    lat = L.Lattice.from_geometry(geo, "D3Q19", "xyz")
    red = np.random.default_rng(SEED + 1).random(geo.shape) < 0.5
    rho0 = np.where(geo == 1, red, 0.0)
    rho1 = np.where(geo == 1, ~red, 0.0).astype(np.float64)
    f0, rho = L.initiate_twophase(lat, lat.attribute(rho0), lat.attribute(rho1),
                                  lat.attribute(np.full(geo.shape, 0.5)))
    return lat, f0, rho


@pytest.fixture(scope="module")
def tp_oracle(tp_pack, oracle):
    lat, f0, rho = tp_pack
    g = oracle.OracleGrid(lat.nq, lat.neigh, lat.types, lat.bulk)
    f, r, vel, cg, _ = oracle.twophase_run(g, f0.copy(), rho.copy(), TP_STEPS, 1.0, 1.0, SIGMA, BETA, (GX, 0.0, 0.0),
                                           nthreads=oracle.default_threads())
    b = lat.bulk
    return f.reshape(-1, 2, 19)[b].copy(), r.reshape(-1, 2)[b].copy(), vel.reshape(-1, 3)[b].copy(), cg[b].copy()


def tp_solver(bclbm, lat, f0, rho, **kw):
    L = bclbm.lbsolver
    return L.Solver(lat, f0, collision=L.RK, tau=(1.0, 1.0), force=(GX, 0.0, 0.0), sigma=SIGMA, beta=BETA,
                    rho_init=rho, **kw)


def tp_outputs(lat, s):
    f = s.download_f()
    r, vel, cg = s.download_macros()
    b = lat.bulk
    return f.reshape(-1, 2, 19)[b], r.reshape(-1, 2)[b], vel.reshape(-1, 3)[b], cg[b]


@pytest.mark.parametrize("mode", ["exact", "fixed", "fma"])
def test_two_phase_96_against_oracle(bclbm, tp_pack, tp_oracle, mode):
    lat, f0, rho = tp_pack
    kw = {"exact": dict(exact=True), "fixed": {}, "fma": dict(fma64=True)}[mode]
    with tp_solver(bclbm, lat, f0, rho, **kw) as s:
        s.step(TP_STEPS)
        f, r, vel, cg = tp_outputs(lat, s)
    ef, er, evel, ecg = tp_oracle
    if mode == "exact":
        assert np.array_equal(f, ef)
        assert np.array_equal(r, er)
        assert np.array_equal(vel, evel)
        assert np.array_equal(cg, ecg)
    else:
        assert relerr(f, ef) <= 1e-12
        assert relerr(r, er) <= 1e-12
        assert relerr(cg, ecg) <= 1e-12
        assert np.abs(vel - evel).max() <= u_bound(evel, ef, TP_STEPS)


def test_two_phase_96_f16_saturation(bclbm, tp_pack, tp_oracle):
    """FP16 storage of both colour sets, FP32 arithmetic, FP64 reductions: the
    saturation within 1e-6 of the oracle's and the densities within 5e-3."""
    lat, f0, rho = tp_pack
    with tp_solver(bclbm, lat, f0, rho, precision="f16") as s:
        s.step(TP_STEPS)
        st = s.reduce()
        f, r, vel, cg = tp_outputs(lat, s)
    ef, er, evel, ecg = tp_oracle
    sat_ref = er[:, 0].sum() / er.sum()
    assert abs(st["saturation"] - sat_ref) <= 1e-6
    assert relerr(r, er) <= 5e-3


DRIFT_STEPS = 2000


def test_two_phase_mass_drift_correction(bclbm, gpu):
    """FP16 two-phase storage over 2,000 steps on a 64^3 pack: the saturation
    stays within 1e-7 of its initial value with the correction, and the
    uncorrected run drifts at least 10x further."""
    L = bclbm.lbsolver
    geo, _, _ = bclbm.geometry.sphere_pack((64,) * 3, radius=TP_RADIUS, porosity=POROSITY, seed=SEED)
    lat = L.Lattice.from_geometry(geo, "D3Q19", "xyz")
    red = np.random.default_rng(SEED + 1).random(geo.shape) < 0.5
    rho0 = np.where(geo == 1, red, 0.0)
    rho1 = np.where(geo == 1, ~red, 0.0).astype(np.float64)
    f0, rho = L.initiate_twophase(lat, lat.attribute(rho0), lat.attribute(rho1),
                                  lat.attribute(np.full(geo.shape, 0.5)))
    drift = {}
    for fix in (True, False):
        with tp_solver(bclbm, lat, f0, rho, precision="f16", mass_fix=fix) as s:
            s0 = s.reduce()["saturation"]
            s.step(DRIFT_STEPS)
            drift[fix] = abs(s.reduce()["saturation"] - s0)
    assert drift[True] <= 1e-7, drift
    assert drift[False] >= 10 * drift[True], drift


UV_TAUS, UV_WETT, UV_SIGMA, UV_STEPS = (0.7, 1.3), 0.8, 0.02, 100


@pytest.mark.parametrize("lattice,shape,radius", [("D3Q19", (40, 40, 40), 6.0), ("D2Q9", (160, 128), 9.0)])
def test_two_phase_unequal_viscosities(bclbm, gpu, oracle, lattice, shape, radius):
    """tau_r != tau_b (the relaxation rate varies with the phase mix at every node)
    and non-neutral wetting (boundary solids of colour 0.6): exact FP64 equal to
    the oracle, the fixed-point and FMA forms within 1e-12 after 100 steps."""
    L = bclbm.lbsolver
    geo, _, _ = bclbm.geometry.sphere_pack(shape, radius=radius, porosity=POROSITY, seed=SEED + 7)
    lat = L.Lattice.from_geometry(geo, lattice, "xyz"[:len(shape)])
    nq = lat.nq
    red = np.random.default_rng(SEED + 8).random(geo.shape) < 0.5
    rho0 = np.where(geo == 1, red, 0.0)
    rho1 = np.where(geo == 1, ~red, 0.0).astype(np.float64)
    f0, rho = L.initiate_twophase(lat, lat.attribute(rho0), lat.attribute(rho1),
                                  lat.attribute(np.full(geo.shape, UV_WETT)))
    force = (GX, 0.0, 0.0)
    g = oracle.OracleGrid(lat.nq, lat.neigh, lat.types, lat.bulk)
    ef, er, evel, ecg, _ = oracle.twophase_run(g, f0.copy(), rho.copy(), UV_STEPS, *UV_TAUS, UV_SIGMA, BETA, force,
                                               nthreads=oracle.default_threads())
    b = lat.bulk
    nd = 2 if nq == 9 else 3
    ef = ef.reshape(-1, 2, nq)[b]
    er = er.reshape(-1, 2)[b]
    evel = evel.reshape(-1, nd)[b]
    ecg = ecg[b]
    sb = lat.types == 1
    assert sb.any()
    for mode, kw in (("exact", dict(exact=True)), ("fixed", {}), ("fma", dict(fma64=True))):
        with L.Solver(lat, f0, collision=L.RK, tau=UV_TAUS, force=force, sigma=UV_SIGMA, beta=BETA,
                      rho_init=rho, **kw) as s:
            s.step(UV_STEPS)
            f = s.download_f().reshape(-1, 2, nq)[b]
            r, vel, cg = s.download_macros()
        r, vel, cgb = r.reshape(-1, 2)[b], vel.reshape(-1, nd)[b], cg[b]
        # the boundary solids report the wetting colour (rho0 - rho1) / (rho0 + rho1)
        assert np.allclose(cg[sb], (UV_WETT - (1 - UV_WETT)) / 1.0, atol=1e-7), mode
        if mode == "exact":
            assert np.array_equal(f, ef), mode
            assert np.array_equal(r, er), mode
            assert np.array_equal(cgb, ecg), mode
        else:
            assert relerr(f, ef) <= 1e-12, mode
            assert relerr(r, er) <= 1e-12, mode
            assert relerr(cgb, ecg) <= 1e-12, mode
            assert np.abs(vel - evel).max() <= u_bound(evel, ef, UV_STEPS), mode


def _developed(bclbm, size=64, steps=1000):
    """A 64^3 two-phase pack after `steps` exact FP64 steps (interfaces formed)."""
    L = bclbm.lbsolver
    geo, _, _ = bclbm.geometry.sphere_pack((size,) * 3, radius=TP_RADIUS, porosity=POROSITY, seed=SEED)
    lat = L.Lattice.from_geometry(geo, "D3Q19", "xyz")
    red = np.random.default_rng(SEED + 1).random(geo.shape) < 0.5
    rho0 = np.where(geo == 1, red, 0.0)
    rho1 = np.where(geo == 1, ~red, 0.0).astype(np.float64)
    f0, rho = L.initiate_twophase(lat, lat.attribute(rho0), lat.attribute(rho1),
                                  lat.attribute(np.full(geo.shape, 0.5)))
    with tp_solver(bclbm, lat, f0, rho, exact=True) as s:
        s.step(steps)
        f = s.download_f()
        r, _, _ = s.download_macros()
    rho_dev = rho.reshape(-1, 2).copy()
    rho_dev[lat.bulk] = r.reshape(-1, 2)[lat.bulk]
    return lat, f, rho_dev.reshape(-1)


LAG_STEPS = 200


def test_two_phase_lagged_colour(bclbm, gpu):
    """BCLBM_FLAG_LAGGED_COLOUR (one pass per step, the gradient from the previous
    step's colours) on FP32 storage, from a developed 64^3 state: its first step is
    the two-pass step bit for bit; after 200 steps the saturation stays within 1e-7
    of exact FP64, the colour field within a mean of 5e-3 and the phase fluxes within
    5% (the deviations FP16 storage itself makes over such runs)."""
    lat, f, rho = _developed(bclbm)
    b = lat.bulk
    cx = np.array([1, 0, 0, 1, 1, 1, 1, 0, 0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 0], dtype=np.float64)

    def run(n, **kw):
        with tp_solver(bclbm, lat, f, rho, **kw) as s:
            s.step(n)
            st = s.reduce()
            g = s.download_f().reshape(-1, 2, 19)[b]
            _, _, cg = s.download_macros()
        return st["saturation"], g, cg[b], [(g[:, k, :] * cx[None, :]).sum() for k in range(2)]

    _, g2, _, _ = run(1, precision="f32")
    _, gl, _, _ = run(1, precision="f32", lagged_colour=True)
    assert np.array_equal(g2, gl)
    s_ref, _, cg_ref, fl_ref = run(LAG_STEPS, exact=True)
    s_lag, g_lag, cg_lag, fl_lag = run(LAG_STEPS, precision="f32", lagged_colour=True)
    _, g_two, _, _ = run(LAG_STEPS, precision="f32")
    assert not np.array_equal(g_lag, g_two)  # the one-pass step ran
    assert abs(s_lag - s_ref) <= 1e-7
    assert np.abs(cg_lag - cg_ref).mean() <= 5e-3
    for a, c in zip(fl_lag, fl_ref):
        assert abs(a - c) <= 0.05 * abs(c)


def test_two_phase_lagged_colour_mass(bclbm, gpu):
    """FP16 storage in one pass per step over 2,000 steps on the 64^3 pack: the
    lag-aware mass correction keeps the saturation within 1e-6 of its start, 10x
    closer than the uncorrected run."""
    lat, f, rho = _developed(bclbm, steps=10)
    drift = {}
    for fix in (True, False):
        with tp_solver(bclbm, lat, f, rho, precision="f16", lagged_colour=True, mass_fix=fix) as s:
            s0 = s.reduce()["saturation"]
            s.step(DRIFT_STEPS)
            drift[fix] = abs(s.reduce()["saturation"] - s0)
    assert drift[True] <= 1e-6, drift
    assert drift[False] >= 10 * drift[True], drift
