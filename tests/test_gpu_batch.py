"""The multi-instance batch (bclbm_batch_*) and the serving loop on the GPU.

Per-request isolation: every instance's populations and FP64 sums must be
bit-identical to a single handle created from the same descriptor and stepped
the same number of times, whether the instance runs alone or among others
admitted and retired at other times, with or without the captured graph, and
after the work list has grown.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BUDGET = 8 << 30


def pack(bclbm, size, seed, radius=3.0, porosity=0.45):
    geo, _, _ = bclbm.geometry.sphere_pack((size,) * 3, radius=radius, porosity=porosity, seed=seed)
    lat = bclbm.lbsolver.Lattice.from_geometry(geo, "D3Q19", "xyz")
    return lat, bclbm.lbsolver.initiate_single(lat, np.ones(lat.n_nodes))


@pytest.fixture(scope="module")
def lattices(bclbm, gpu):
    return [pack(bclbm, 20, 1), pack(bclbm, 27, 2, radius=4.0), pack(bclbm, 16, 3, porosity=0.35),
            pack(bclbm, 33, 4, radius=5.0)]


TAUS = [0.8, 0.62, 1.1, 0.95]
FORCE = (1e-5, 0.0, 0.0)


def single(bclbm, lat, f0, tau, steps, precision, collision=0, fma64=False):
    taus = (tau, 3.0 / 16.0 / (tau - 0.5) + 0.5) if collision else (tau, tau)
    with bclbm.lbsolver.Solver(lat, f0, collision=collision, tau=taus, force=FORCE, precision=precision,
                               fma64=fma64) as s:
        s.step(steps)
        return s.download_f(), s.reduce()


def admit(batch, lat, f0, tau, collision=0):
    return batch.admit(lat, f0, (tau, 3.0 / 16.0 / (tau - 0.5) + 0.5) if collision else (tau, tau), FORCE)


def same_stats(a, b):
    for k in ("mass", "momentum", "flux_fc"):
        assert a[k] == b[k], (k, a[k], b[k])
    assert a["max_abs_f"] == b["max_abs_f"]
    assert a["steps_done"] == b["steps_done"]


@pytest.mark.parametrize("precision,fma64", [("f64", False), ("f64", True), ("f32", False), ("f16", False),
                                             ("bf16", False)])
@pytest.mark.parametrize("collision", [0, 1])
def test_batch_equals_single_handle(bclbm, lattices, precision, fma64, collision):
    S = bclbm.serving
    with S.Batch(precision=precision, fma64=fma64, collision=collision, hbm_budget=BUDGET,
                 steps_per_graph=25) as b:
        ids = [admit(b, lat, f0, t, collision) for (lat, f0), t in zip(lattices, TAUS)]
        b.step(120)
        stats = b.stats(ids)
        for (lat, f0), t, i, st in zip(lattices, TAUS, ids, stats):
            f_ref, st_ref = single(bclbm, lat, f0, t, 121, precision, collision, fma64)
            assert np.array_equal(b.download_f(i), f_ref)
            same_stats(st, st_ref)


def test_alone_and_in_the_mix(bclbm, lattices):
    """Instance A alone, and A among instances admitted and retired around it."""
    S = bclbm.serving
    (la, fa), (lb, fb), (lc, fc), (ld, fd) = lattices
    with S.Batch(precision="f16", hbm_budget=BUDGET, steps_per_graph=20) as alone:
        a = admit(alone, la, fa, TAUS[0])
        alone.step(300)
        f_alone, st_alone = alone.download_f(a), alone.stats([a])[0]
    with S.Batch(precision="f16", hbm_budget=BUDGET, steps_per_graph=20) as mix:
        c = admit(mix, lc, fc, TAUS[2])
        mix.step(37)
        a = admit(mix, la, fa, TAUS[0])
        bb = admit(mix, lb, fb, TAUS[1])
        mix.step(100)
        mix.retire(c)
        d = admit(mix, ld, fd, TAUS[3])
        mix.step(150)
        mix.retire(bb)
        mix.step(50)
        f_mix, st_mix = mix.download_f(a), mix.stats([a, d])[0]
    assert np.array_equal(f_alone, f_mix)
    same_stats(st_alone, st_mix)


def test_graph_and_direct_launches_agree(bclbm, lattices):
    S = bclbm.serving
    out = []
    for spg in (0, 7, 64):
        with S.Batch(precision="f64", hbm_budget=BUDGET, steps_per_graph=spg) as b:
            ids = [admit(b, lat, f0, t) for (lat, f0), t in zip(lattices[:2], TAUS)]
            b.step(130)
            out.append([b.download_f(i) for i in ids])
    for run in out[1:]:
        for x, y in zip(out[0], run):
            assert np.array_equal(x, y)


def test_work_list_growth_keeps_results(bclbm, lattices):
    """Admissions beyond the initial work-list capacity reallocate it (and drop the graph)."""
    S = bclbm.serving
    big = pack(bclbm, 72, 9, radius=6.0)  # > 1024 blocks of 256 nodes with the others
    with S.Batch(precision="f32", hbm_budget=BUDGET, steps_per_graph=10) as b:
        a = admit(b, *lattices[0], TAUS[0])
        b.step(30)
        g1 = admit(b, *big, 0.7)
        g2 = admit(b, *big, 0.9)
        b.step(40)
        f_a = b.download_f(a)
        f_g2 = b.download_f(g2)
        assert b.info()["active"] == 3
    f_ref, _ = single(bclbm, *lattices[0], TAUS[0], 71, "f32")
    assert np.array_equal(f_a, f_ref)
    f_ref2, _ = single(bclbm, *big, 0.9, 41, "f32")
    assert np.array_equal(f_g2, f_ref2)
    assert g1 is not None


def test_admission_by_hbm_footprint(bclbm, lattices):
    S = bclbm.serving
    lat, f0 = lattices[3]
    fp = bclbm.native.footprint(lat, 0, 2)
    with S.Batch(precision="f16", hbm_budget=int(fp * 2.5), max_instances=8) as b:
        x = admit(b, lat, f0, 0.8)
        y = admit(b, lat, f0, 0.8)
        assert x is not None and y is not None
        assert admit(b, lat, f0, 0.8) is None  # over budget: refused, nothing allocated
        assert b.info()["active"] == 2 and b.info()["used_bytes"] == 2 * fp
        b.step(10)
        b.retire(x)
        z = admit(b, lat, f0, 0.8)
        assert z == x  # the freed slot is reused
        b.step(10)
        st = b.stats([y, z])
        assert st[0]["steps_done"] == 21 and st[1]["steps_done"] == 11
    with S.Batch(precision="f16", hbm_budget=BUDGET, max_instances=1) as b:
        assert admit(b, lat, f0, 0.8) is not None
        assert admit(b, lat, f0, 0.8) is None  # no free slot


def test_batch_rejects_mismatched_descriptor(bclbm, lattices):
    S = bclbm.serving
    lat, f0 = lattices[0]
    with S.Batch(precision="f16", hbm_budget=BUDGET) as b:
        d = bclbm.native.make_desc(lat, f0, 0, 0, 0, (0.8, 0.8), np.array([1e-5, 0, 0]), 0.0, 0.0, 0, 0.0, 1.0,
                                   0.0, None)
        import ctypes
        i = ctypes.c_int32()
        assert bclbm.native.lib().bclbm_batch_admit(b._b, ctypes.byref(d), ctypes.byref(i)) == -1
        with pytest.raises(bclbm.native.BclbmError):
            b.retire(5)


def test_server_matches_sequential_and_fp64(bclbm):
    """A small request stream: the batched FP16 server returns exactly the
    sequential FP16 solves, and FP16 permeabilities are within 1e-3 of FP64."""
    S = bclbm.serving
    reqs = S.sample_requests(6, rate=0.0, seed=11, size_range=(16, 40), radius_range=(3.0, 4.0),
                             porosity_range=(0.45, 0.50))
    srv = S.Server(precision="f16", hbm_budget=BUDGET, check_every=100, tol=1e-5, max_steps=3000,
                   steps_per_graph=25, prep_workers=2)
    rep = srv.run(reqs)
    seq16 = srv.run_sequential(reqs, precision="f16")
    seq64 = srv.run_sequential(reqs, precision="f64")
    assert rep["solves"] == 6 and rep["counters"]["retired"] == 6
    for a, b, c in zip(rep["results"], seq16["results"], seq64["results"]):
        assert a.rid == b.rid == c.rid
        assert a.steps == b.steps and a.permeability == b.permeability
        assert abs(a.permeability - c.permeability) / abs(c.permeability) <= 1e-3
    assert rep["p99_s"] >= rep["p50_s"] > 0.0


def test_server_precision_ladder(bclbm):
    """f16>f32: every request converges, and k is FP32-accurate against FP64."""
    S = bclbm.serving
    reqs = S.sample_requests(5, rate=0.0, seed=12, size_range=(16, 36), radius_range=(3.0, 4.0),
                             porosity_range=(0.45, 0.50))
    # the stopping rule of the permeability requests: |dk/k| < 1e-6 over 500 steps (a shorter
    # block makes the rule looser: a slow mode can still hold 1e-3 of k)
    srv = S.Server(precision="f16>f32", hbm_budget=BUDGET, check_every=500, tol=1e-6, max_steps=10000,
                   steps_per_graph=25, prep_workers=2, promote_tol=2e-5)
    rep = srv.run(reqs)
    seq64 = srv.run_sequential(reqs, precision="f64")
    assert rep["counters"]["promoted"] == 5 and rep["counters"]["retired"] == 5
    for a, c in zip(rep["results"], seq64["results"]):
        assert a.converged and c.converged
        assert abs(a.permeability - c.permeability) / abs(c.permeability) <= 2e-5


def test_attach_a_created_handle(bclbm, lattices):
    """bclbm_batch_attach: a handle created and stepped outside joins the batch and
    continues exactly; unsuitable handles are refused and stay the caller's."""
    S = bclbm.serving
    lat, f0 = lattices[1]
    with S.Batch(precision="f32", hbm_budget=BUDGET) as b:
        s = bclbm.lbsolver.Solver(lat, f0, tau=(TAUS[1], TAUS[1]), force=FORCE, precision="f32")
        fresh = bclbm.lbsolver.Solver(lat, f0, tau=(TAUS[1], TAUS[1]), force=FORCE, precision="f32")
        wrong = bclbm.lbsolver.Solver(lat, f0, tau=(TAUS[1], TAUS[1]), force=FORCE, precision="f16")
        wrong.step(1)
        with pytest.raises(bclbm.native.BclbmError):
            b.attach(fresh)  # no step taken yet
        with pytest.raises(bclbm.native.BclbmError):
            b.attach(wrong)
        s.step(3)
        i = b.attach(s)
        assert s._h is None
        b.step(60)
        f = b.download_f(i)
        fresh.step(63)
        assert np.array_equal(f, fresh.download_f())
        wrong.close()
        fresh.close()


def _small_requests(bclbm, n, seed):
    S = bclbm.serving
    return S.sample_requests(n, rate=0.0, seed=seed, size_range=(16, 30), radius_range=(3.0, 4.0),
                             porosity_range=(0.45, 0.50))


def test_server_retires_a_poisoned_request_and_keeps_the_others(bclbm):
    """A NaN in one request's host copy of the populations: the FP64 statistics flag
    that request, which retires with status nonfinite; the others finish exactly as
    in a run without it."""
    S = bclbm.serving
    reqs = _small_requests(bclbm, 4, 21)
    prepared = {r.rid: S.prepare(r) for r in reqs}
    srv = S.Server(precision="f32", hbm_budget=BUDGET, check_every=100, tol=1e-5, max_steps=2000,
                   steps_per_graph=25, prep_workers=2)
    clean = srv.run(reqs, prepared=prepared)
    lat, f0 = prepared[2]
    bad = f0.copy()
    bad[int(lat.bulk[len(lat.bulk) // 3]) * 19 + 4] = np.nan
    poisoned = dict(prepared)
    poisoned[2] = (lat, bad)
    rep = srv.run(reqs, prepared=poisoned)
    st = {r.rid: r for r in rep["results"]}
    assert st[2].status == "nonfinite" and rep["counters"]["nonfinite"] == 1
    for a in clean["results"]:
        if a.rid != 2:
            assert st[a.rid].status == a.status and st[a.rid].permeability == a.permeability
    seq = srv.run_sequential(reqs, precision="f32", prepared=poisoned)
    assert {r.rid: r.status for r in seq["results"]}[2] == "nonfinite"


def test_server_cancellation(bclbm):
    S = bclbm.serving
    reqs = _small_requests(bclbm, 3, 22)
    reqs[1].cancel_at = 0.0  # withdrawn before it is admitted
    srv = S.Server(precision="f32", hbm_budget=BUDGET, check_every=100, tol=1e-5, max_steps=1500,
                   steps_per_graph=25, prep_workers=2)
    rep = srv.run(reqs)
    st = {r.rid: r.status for r in rep["results"]}
    assert st[1] == "cancelled" and st[0] in ("converged", "capped") and st[2] in ("converged", "capped")
    assert rep["counters"]["cancelled"] == 1


@pytest.mark.parametrize("precision,exact", [("f64", True), ("f16", False), ("f32", False), ("f64", False)])
def test_checkpoint_and_resume(bclbm, lattices, tmp_path, precision, exact):
    """Solver.checkpoint writes LbField's .lblbf format; a solver created from it
    continues exactly as the uninterrupted run when the device state is FP64 or a
    shifted format (the file holds it exactly).  The default FP64 step keeps its
    state in 64-bit fixed point, finer than FP64 for populations above 2^-8: its
    checkpoint is that state rounded to FP64, and the resumed run stays within
    FP64 rounding of the uninterrupted one."""
    L = bclbm.lbsolver
    lat, f0 = lattices[1]
    kw = dict(tau=(0.9, 0.9), force=FORCE, precision=precision, exact=exact)
    with L.Solver(lat, f0, **kw) as s:
        s.step(150)
        s.checkpoint(tmp_path / "c.lblbf")
        s.step(90)
        f_cont = s.download_f()
    f_chk, nf, nq, n = L.read_lblbf(tmp_path / "c.lblbf")
    assert (nf, nq, n) == (1, 19, lat.n_nodes)
    with L.Solver(lat, f_chk, **kw) as s:
        s.step(90)
        f_res = s.download_f()
    if precision == "f64" and not exact:
        assert np.abs(f_res - f_cont).max() <= 4 * np.finfo(np.float64).eps * np.abs(f_cont).max()
    else:
        assert np.array_equal(f_res, f_cont)
