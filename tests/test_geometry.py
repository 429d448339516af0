"""The in-process geometry builder against the tables the reference builds from
vtklb.py files (bit-exact), plus generator properties."""

import numpy as np
import pytest

import lbcases


@pytest.mark.parametrize("name", lbcases.CASES)
def test_build_lattice_matches_reference_tables(bclbm, name):
    case = lbcases.Case(name, bclbm)
    z = case.z
    lat = bclbm.geometry.build_lattice(z["mask"].astype(np.int8), case.meta["lattice"], case.meta["periodic"])
    assert lat["nf"] == case.nf
    assert 1 + lat["nf"] + lat["ns"] == case.n_nodes
    assert np.array_equal(lat["neigh"], z["neigh"])
    assert np.array_equal(lat["types"], z["types"])
    assert np.array_equal(lat["pos"], z["pos"])
    bulk = np.nonzero(lat["types"] > 1)[0]
    assert np.array_equal(bulk, z["bulk"])
    assert np.array_equal(np.nonzero(lat["types"] == 2)[0], z["fluidbnd"])
    assert np.array_equal(np.nonzero(lat["types"] == 1)[0], z["solidbnd"])


@pytest.mark.parametrize("name", lbcases.CASES)
@pytest.mark.parametrize("which", ["fluidbnd", "bulk"])
def test_bounce_back_link_classes_match_reference(bclbm, name, which):
    case = lbcases.Case(name, bclbm)
    z = case.z
    links = bclbm.geometry.bounce_back_links(z["neigh"], z["types"], z[which], case.nq)
    rec = []
    for node, beta, gamma, delta in links:
        rec += [node, len(beta), len(gamma), len(delta)] + beta + gamma + delta
    assert np.array_equal(np.array(rec, dtype=np.int32), z["links_" + which])


def test_sphere_pack_is_seeded_and_hits_porosity(bclbm):
    a, ca, pa = bclbm.geometry.sphere_pack((48, 40, 32), radius=5.0, porosity=0.4, seed=123)
    b, cb, pb = bclbm.geometry.sphere_pack((48, 40, 32), radius=5.0, porosity=0.4, seed=123)
    c, _, _ = bclbm.geometry.sphere_pack((48, 40, 32), radius=5.0, porosity=0.4, seed=124)
    assert np.array_equal(a, b) and np.array_equal(ca, cb)
    assert not np.array_equal(a, c)
    assert pa <= 0.4 and pa > 0.37
    assert abs(pa - a.mean()) < 1e-12


def test_periodic_tables_are_symmetric(bclbm):
    geo, _, _ = bclbm.geometry.sphere_pack((18, 14, 10), radius=3.0, porosity=0.5, seed=9)
    lat = bclbm.geometry.build_lattice(geo, "D3Q19", "xyz")
    nq, nf = lat["nq"], lat["nf"]
    nb = lat["neigh"].reshape(-1, nq)
    rev = [(q + 9) % 18 if q < 18 else 18 for q in range(19)]
    types = lat["types"]
    for x in range(1, nf + 1):
        for q in range(18):
            y = nb[x, rev[q]]
            if types[y] > 1:
                assert nb[y, q] == x
        assert nb[x, 18] == x


@pytest.mark.parametrize("lattice,shape", [("D2Q9", (23, 17)), ("D3Q19", (13, 11, 9)), ("D3Q19", (1, 6, 5)),
                                           ("D2Q9", (2, 40))])
@pytest.mark.parametrize("periodic", ["", "x", "y", "xz", "xyz"])
def test_native_lattice_builder_matches_numpy(bclbm, lattice, shape, periodic):
    rng = np.random.default_rng(len(shape) * 100 + sum(shape) + len(periodic))
    geo = (rng.random(shape) < 0.6).astype(np.int8)
    a = bclbm.geometry.build_lattice(geo, lattice, periodic)
    b = bclbm.geometry.build_lattice_numpy(geo, lattice, periodic)
    for k in ("neigh", "types", "pos"):
        assert np.array_equal(a[k], b[k]), k
    assert (a["nf"], a["ns"]) == (b["nf"], b["ns"])


def test_native_lattice_builder_rejects_bad_masks(bclbm):
    with pytest.raises(ValueError):
        bclbm.geometry.build_lattice(np.full((4, 4, 4), 2, dtype=np.int8), "D3Q19", "")
    with pytest.raises(bclbm.native.BclbmError):
        bclbm.native.lattice_tables(np.full((4, 4, 4), 2, dtype=np.int8), 19, 0)
    with pytest.raises(bclbm.native.BclbmError):
        bclbm.native.lattice_tables(np.ones((4, 4), dtype=np.int8), 19, 0)


def test_native_builder_from_concurrent_threads(bclbm):
    """The library's host loops share one pool of worker threads: calls from several
    host threads at once (one loop on the pool, the others on their callers' threads)
    give the same tables as one call at a time."""
    from concurrent.futures import ThreadPoolExecutor
    geo, _, _ = bclbm.geometry.sphere_pack((48, 40, 44), radius=5.0, porosity=0.45, seed=11)
    ref = bclbm.geometry.build_lattice(geo, "D3Q19", "xyz")
    with ThreadPoolExecutor(6) as ex:
        outs = list(ex.map(lambda _: bclbm.geometry.build_lattice(geo, "D3Q19", "xyz"), range(12)))
    for out in outs:
        for k in ("neigh", "types", "pos"):
            assert np.array_equal(out[k], ref[k]), k
