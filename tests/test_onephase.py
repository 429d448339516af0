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
