"""The std_one_phase oracle (oracle_links_run) against the reference's own run
(tests/golden/onephase_*.npz, written by oracle/ref_onephase.cpp around the
unmodified src/std_one_phase/main.cpp): populations, moments and the write
step's mass flux bit for bit.  Host only."""

import sys
from pathlib import Path

import numpy as np
import pytest

import lbcases

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import oracle  # noqa: E402


@pytest.mark.parametrize("name", lbcases.ONEPHASE_CASES)
def test_oracle_matches_reference(bclbm, name):
    c = lbcases.OnephaseCase(name, bclbm)
    g = oracle.OracleGrid(19, c.z["neigh"], c.z["types"], c.z["bulk"])
    f, rho, vel, flux = oracle.links_run(g, c.f_init(), c.meta["steps"], c.meta["tau"], c.force, c.tags, c.labels,
                                         c.force_on)
    b = c.lat.bulk
    assert np.array_equal(f.reshape(-1, 19)[b], c.z["f"][:, 0, :])
    assert np.array_equal(rho[b], c.z["rho"][:, 0])
    assert np.array_equal(vel.reshape(-1, 3)[b], c.z["vel"][:, 0, :])
    assert np.array_equal(flux, c.z["flux"])


def test_fixture_exercises_every_rule(bclbm):
    """Both fixtures hold solid-fluid, pressure and fluid-fluid links, interior
    domains with sources and a zero force layer; the open one streams into node 0
    through pressure links (node 0's tag is -1, which counts as a ghost)."""
    for name in lbcases.ONEPHASE_CASES:
        c = lbcases.OnephaseCase(name, bclbm)
        t, nb = c.tags, c.z["neigh"].reshape(-1, 19)
        b = c.lat.bulk
        tb = t[b]
        assert np.any((tb >> 3) & 1) and np.any((tb >> 4) & 1) and np.any((tb >> 2) & 1)
        assert c.labels.max() == 2 and np.any(c.force_on[b] == 0)
        touches0 = np.any(nb[b] == 0, axis=1) & ((tb >> 4) & 1).astype(bool)
        assert touches0.any() == (not c.meta["ghost_layers"])


def test_tagged_pack_links_all_have_a_rule(bclbm):
    """geometry.tagged_pack's tags give every link of every fluid node one of the
    std_one_phase rules (solid-fluid, pressure-fluid, fluid-fluid) or a fluid
    upstream node, which bclbm_create requires (main.cpp:24-129); its interior
    domains all have source nodes (tag < 3)."""
    mask, attrs = bclbm.geometry.tagged_pack((30, 28, 40), 4.0, 0.45, 11, blob_radius=3.5, blob_spacing=12)
    lat = bclbm.lbsolver.Lattice.from_geometry(mask, "D3Q19", "xy")
    tags = lat.attribute(attrs["nodetags"]).astype(np.int64)
    tags[0] = -1  # Nodes initialises node 0's tag to -1
    labels = lat.attribute(attrs["interior_domains"]).astype(np.int64)
    nb = lat.neigh.reshape(-1, 19)
    fluid = lat.types > 1
    rev = np.array([(q + 9) % 18 for q in range(18)])
    b = lat.bulk
    tn = tags[b][:, None]
    y = nb[b][:, rev]          # upstream node of each incoming direction q
    ty = tags[y]
    sf = ((tn >> 3) & 1).astype(bool) & ((ty & 3) == 0)
    pf = ((tn >> 4) & 1).astype(bool) & ((ty & 3) == 3)
    ff = (((tn & 3) == 1) & ((tn >> 2) & 1).astype(bool) & ((ty & 3) == 2)) | \
         (((tn & 3) == 2) & ((ty & 3) == 1) & ((ty >> 2) & 1).astype(bool))
    plain = (y != 0) & fluid[y]
    assert np.all(sf | pf | ff | plain)
    assert pf.any() and sf.any() and ff.any()
    for lab in range(1, labels.max() + 1):
        assert np.any((labels[1:] == lab) & (tags[1:] < 3)), lab


def test_solver_checks_links_arguments(bclbm):
    """The Python mirror refuses a std_one_phase solver without its node
    attributes, or with attributes of the wrong length, before calling the
    library."""
    c = lbcases.OnephaseCase("onephase_ghost", bclbm)
    L = c.L
    with pytest.raises(ValueError):
        L.Solver(c.lat, c.f_init(), collision=L.LINKS, tau=(0.9, 0.9))
    with pytest.raises(ValueError):
        L.Solver(c.lat, c.f_init(), collision=L.LINKS, tau=(0.9, 0.9), tags=c.tags[:-1], labels=c.labels)
