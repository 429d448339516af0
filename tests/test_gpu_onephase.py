"""The std_one_phase step (BCLBM_LINKS) on the GPU against the reference's own
run of src/std_one_phase/main.cpp (tests/golden/onephase_*.npz):

* exact FP64 (BCLBM_FLAG_EXACT): populations, rho, u and the write step's mass
  flux bit-identical, in reference and in Morton node order;
* FP64 storage with 64-bit fixed-point arithmetic (the default) and with FP64
  FMA arithmetic (BCLBM_FLAG_FP64_FMA): relative L2 error <= 1e-12 in f and
  rho, u within 1e-12 of max |u|, mass flux within 1e-10;
* shifted F32 / F16 / BF16 storage with FP32 arithmetic within the tolerances
  of test_shifted_storage;
* the set-up errors: a link without a boundary rule, an interior domain
  without source nodes, combinations that are not built."""

import numpy as np
import pytest

import lbcases

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def run(c, steps, pieces=1, **kw):
    with c.solver(**kw) as s:
        left = steps
        for k in range(pieces):
            n = left // (pieces - k)
            s.step(n)
            left -= n
        f = s.download_f()
        rho, vel, _ = s.download_macros()
        flux = s.pressure_flux()
        st = s.reduce()
        perm = s.node_perm()
    b = c.lat.bulk
    return {"f": f.reshape(-1, 19)[b], "rho": rho[b], "vel": vel.reshape(-1, 3)[b], "flux": flux, "stats": st,
            "perm": perm}


@pytest.mark.parametrize("sfc", [False, True], ids=["refOrder", "morton"])
@pytest.mark.parametrize("name", lbcases.ONEPHASE_CASES)
def test_exact_matches_reference(bclbm, gpu, name, sfc):
    c = lbcases.OnephaseCase(name, bclbm)
    got = run(c, c.meta["steps"], exact=True, sfc=sfc)
    assert np.array_equal(got["f"], c.z["f"][:, 0, :])
    assert np.array_equal(got["rho"], c.z["rho"][:, 0])
    assert np.array_equal(got["vel"], c.z["vel"][:, 0, :])
    assert np.array_equal(got["flux"], c.z["flux"])
    assert np.array_equal(np.sort(got["perm"]), c.lat.bulk)


@pytest.mark.parametrize("name", lbcases.ONEPHASE_CASES)
def test_exact_in_pieces_and_stats(bclbm, gpu, name):
    """Steps taken in several calls (the velocity store and the moments carry
    over) give the same state; the sums of bclbm_reduce are those of f."""
    c = lbcases.OnephaseCase(name, bclbm)
    got = run(c, c.meta["steps"], pieces=3, exact=True)
    assert np.array_equal(got["f"], c.z["f"][:, 0, :])
    assert np.array_equal(got["flux"], c.z["flux"])
    st = got["stats"]
    fe = c.z["f"][:, 0, :]
    assert abs(st["mass"][0] - fe.sum()) <= 1e-13 * fe.sum()
    cx = np.array([1, 0, 0, 1, 1, 1, 1, 0, 0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 0])
    jx = (fe * cx).sum()
    assert abs(st["flux_fc"][0] - jx) <= 1e-12 * np.abs(fe * cx).sum()


@pytest.mark.parametrize("arith", ["fixed", "fma"])
@pytest.mark.parametrize("name", lbcases.ONEPHASE_CASES)
def test_fast_f64_within_1e12(bclbm, gpu, name, arith):
    c = lbcases.OnephaseCase(name, bclbm)
    got = run(c, c.meta["steps"], fma64=(arith == "fma"))
    fe = c.z["f"][:, 0, :]
    assert relerr(got["f"], fe) <= 1e-12
    assert relerr(got["rho"], c.z["rho"][:, 0]) <= 1e-12
    # u = (sum_q f c_q + F/2) / rho: the fixed-point sums are exact, the reference's
    # FP64 sums carry their own rounding (~eps max f per step, random-walking over
    # the steps), so the bound is 1e-12 of max |u| or that floor, as for std_case
    ve = c.z["vel"][:, 0, :]
    floor = 8 * np.finfo(np.float64).eps * np.abs(fe).max() * np.sqrt(c.meta["steps"])
    assert np.abs(got["vel"] - ve).max() <= max(1e-12 * np.abs(ve).max(), floor)
    assert np.abs(got["flux"] - c.z["flux"]).max() <= 1e-10 * np.abs(c.z["flux"]).max()


@pytest.mark.parametrize("prec,tol_f,tol_u,tol_q", [("f32", 1e-6, 1e-5, 1e-5), ("f16", 1e-4, 1e-3, 1e-3),
                                                   ("bf16", 1e-3, 1e-2, 1e-2)])
@pytest.mark.parametrize("name", lbcases.ONEPHASE_CASES)
def test_shifted_storage(bclbm, gpu, name, prec, tol_f, tol_u, tol_q):
    """Shifted storage with FP32 arithmetic on the deviations f - w rho_ref:
    errors against the reference after the fixture's steps within the stated
    tolerances (f: relative L2; u: of max |u|; mass flux: relative)."""
    c = lbcases.OnephaseCase(name, bclbm)
    got = run(c, c.meta["steps"], precision=prec)
    assert relerr(got["f"], c.z["f"][:, 0, :]) <= tol_f
    ve = c.z["vel"][:, 0, :]
    assert np.abs(got["vel"] - ve).max() <= tol_u * np.abs(ve).max()
    assert np.abs(got["flux"] - c.z["flux"]).max() <= tol_q * np.abs(c.z["flux"]).max()


def test_setup_errors(bclbm, gpu):
    N = bclbm.native
    c = lbcases.OnephaseCase("onephase_ghost", bclbm)
    # a fluid node next to a solid without the fluid-solid bit: no rule for that link
    nb = c.z["neigh"].reshape(-1, 19)
    t = c.tags.copy()
    n = next(int(n) for n in c.lat.bulk if (t[n] >> 3) & 1)
    t[n] &= ~8
    with pytest.raises(N.BclbmError) as e:
        c.L.Solver(c.lat, c.f_init(), collision=c.L.LINKS, tags=t, labels=c.labels, force_on=c.force_on)
    assert e.value.status == -2
    # an interior domain whose nodes all carry interface bits: no source node
    lab = c.labels.copy()
    iface = [int(n) for n in c.lat.bulk if t[n] >= 3 and lab[n] == 0]
    lab[iface[0]] = 3
    with pytest.raises(N.BclbmError) as e:
        c.L.Solver(c.lat, c.f_init(), collision=c.L.LINKS, tags=c.tags, labels=lab, force_on=c.force_on)
    assert e.value.status == -1
    # the exact kernel is FP64 only
    with pytest.raises(N.BclbmError) as e:
        c.solver(precision="f32", exact=True)
    assert e.value.status == -1
    assert nb.shape[1] == 19


@pytest.mark.parametrize("labels_on", [True, False], ids=["domains", "no-domains"])
def test_generated_pack_matches_oracle(bclbm, gpu, labels_on):
    """A tagged pack from geometry.tagged_pack (many interior domains, pressure
    ghosts on both z faces) and the same pack without interior domains: the
    exact kernel equals the oracle's restatement bit for bit after 120 steps."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
    import oracle
    L = bclbm.lbsolver
    mask, attrs = bclbm.geometry.tagged_pack((40, 36, 48), 5.0, 0.45, 7, blob_radius=3.5, blob_spacing=12)
    lat = L.Lattice.from_geometry(mask, "D3Q19", "xy")
    tags, labels, fon = (lat.attribute(attrs[k]).astype(np.int32) for k in ("nodetags", "interior_domains", "force"))
    if not labels_on:
        labels[:] = 0
    else:
        assert labels.max() >= 4
    f0 = L.initiate_single(lat, np.ones(lat.n_nodes))
    force = (2e-6, 1e-6, 1e-5)
    g = oracle.OracleGrid(19, lat.neigh, lat.types, lat.bulk)
    fe, rhoe, vele, fluxe = oracle.links_run(g, f0, 120, 0.9, force, tags, labels, fon, nthreads=4)
    with L.Solver(lat, f0, collision=L.LINKS, tau=(0.9, 0.9), force=force, tags=tags, labels=labels,
                  force_on=fon, exact=True) as s:
        s.step(120)
        f = s.download_f()
        rho, vel, _ = s.download_macros()
        flux = s.pressure_flux()
    b = lat.bulk
    assert np.array_equal(f.reshape(-1, 19)[b], fe.reshape(-1, 19)[b])
    assert np.array_equal(rho[b], rhoe[b]) and np.array_equal(vel.reshape(-1, 3)[b], vele.reshape(-1, 3)[b])
    assert np.array_equal(flux, fluxe)


@pytest.mark.parametrize("prec,tol_f,tol_u,tol_q", [("f32", 1e-6, 1e-5, 1e-5), ("f16", 1e-4, 1e-3, 1e-3)])
@pytest.mark.parametrize("seed,n_bulk", [(7, 29767), (8, 29406)], ids=["odd", "even"])
def test_generated_pack_shifted(bclbm, gpu, seed, n_bulk, prec, tol_f, tol_u, tol_q):
    """Shifted storage on generated tagged packs (interior domains, pressure ghosts
    on both z faces) with an odd and an even number of fluid slots: within the
    tolerances of test_shifted_storage of the oracle's FP64 run after 120 steps."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
    import oracle
    L = bclbm.lbsolver
    mask, attrs = bclbm.geometry.tagged_pack((40, 36, 48), 5.0, 0.45, seed, blob_radius=3.5, blob_spacing=12)
    lat = L.Lattice.from_geometry(mask, "D3Q19", "xy")
    assert lat.n_bulk == n_bulk
    tags, labels, fon = (lat.attribute(attrs[k]).astype(np.int32) for k in ("nodetags", "interior_domains", "force"))
    f0 = L.initiate_single(lat, np.ones(lat.n_nodes))
    force = (2e-6, 1e-6, 1e-5)
    g = oracle.OracleGrid(19, lat.neigh, lat.types, lat.bulk)
    fe, _, vele, fluxe = oracle.links_run(g, f0, 120, 0.9, force, tags, labels, fon, nthreads=4)
    with L.Solver(lat, f0, collision=L.LINKS, tau=(0.9, 0.9), force=force, tags=tags, labels=labels,
                  force_on=fon, precision=prec) as s:
        s.step(120)
        f = s.download_f()
        _, vel, _ = s.download_macros()
        flux = s.pressure_flux()
    b = lat.bulk
    ef = relerr(f.reshape(-1, 19)[b], fe.reshape(-1, 19)[b])
    ve = vele.reshape(-1, 3)[b]
    eu = np.abs(vel.reshape(-1, 3)[b] - ve).max() / np.abs(ve).max()
    eq = np.abs(np.asarray(flux) - np.asarray(fluxe)).max() / np.abs(np.asarray(fluxe)).max()
    assert ef <= tol_f and eu <= tol_u and eq <= tol_q, (ef, eu, eq)
