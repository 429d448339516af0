"""bclbm_lattice_read_vtklb: .vtklb files written by the reference's own
PythonScripts/vtklb.py read into the tables the reference's Grid/Nodes build
(compared bit for bit with the fixtures' reference tables and with the
in-process builder), the scalar attributes, and the errors on files it does not
read.  Needs the reference's vtklb.py to write the files (skipped without it)."""

import os
import sys
from pathlib import Path

import numpy as np
import pytest

import lbcases

REPO = Path(__file__).resolve().parent.parent
REF = Path(os.environ.get("BCLBM_REFERENCE", Path(__file__).resolve().parents[2] / "reference"))
sys.path.insert(0, str(REPO / "tests" / "golden"))

pytestmark = pytest.mark.skipif(not (REF / "PythonScripts" / "vtklb.py").exists(),
                                reason="the reference's vtklb.py is absent")


@pytest.mark.parametrize("name", lbcases.CASES)
def test_reader_equals_reference_tables(bclbm, tmp_path, name):
    import make_golden
    case = lbcases.Case(name, bclbm)
    z = case.z
    mask = z["mask"].astype(np.int8)
    rng = np.random.default_rng(7)
    rho = rng.uniform(0.9, 1.1, mask.shape)
    vtk = make_golden.write_vtklb(REF, tmp_path, mask, case.meta["lattice"], case.meta["periodic"],
                                  {"init_rho": rho})
    neigh, types, pos, nf, ns, attrs = bclbm.native.read_vtklb(vtk, case.nq, ("init_rho", "nodetype"))
    assert np.array_equal(neigh, z["neigh"])
    assert np.array_equal(types, z["types"])
    assert np.array_equal(pos, z["pos"])
    assert nf == case.nf and 1 + nf + ns == case.n_nodes
    lat = bclbm.lbsolver.Lattice(case.nq, neigh, types, pos)
    got = attrs["init_rho"]
    want = lat.attribute(rho)
    # vtklb.py writes floats with numpy's default text format
    assert np.allclose(got[1:], want[1:], rtol=1e-6, atol=0) and got[0] == 0.0


def test_reader_errors(bclbm, tmp_path):
    import make_golden
    N = bclbm.native
    geo = np.ones((6, 5), dtype=np.int8)
    geo[:, 0] = 0
    vtk = make_golden.write_vtklb(REF, tmp_path, geo, "D2Q9", "x", {"init_rho": np.ones(geo.shape)})
    text = Path(vtk).read_text()
    with pytest.raises(N.BclbmError):
        N.read_vtklb(vtk, 19)  # wrong lattice
    cut = tmp_path / "cut.vtklb"
    cut.write_text(text[: len(text) // 2])
    with pytest.raises(N.BclbmError):
        N.read_vtklb(cut, 9)
    binary = tmp_path / "bin.vtklb"
    binary.write_text(text.replace("ASCII", "BINARY", 1))
    # LBvtk reads a BINARY header's file as text too (its flag is unused)
    got = N.read_vtklb(binary, 9)
    want = N.read_vtklb(vtk, 9)
    assert all(np.array_equal(a, b) for a, b in zip(got[:3], want[:3]))
    other = tmp_path / "other.vtklb"
    other.write_text(text.replace("ASCII", "XML", 1))
    with pytest.raises(N.BclbmError) as e:
        N.read_vtklb(other, 9)
    assert e.value.status == -1
    with pytest.raises(N.BclbmError):
        N.read_vtklb(tmp_path / "missing.vtklb", 9)
    # the intact file reads
    neigh, types, pos, nf, ns, _ = N.read_vtklb(vtk, 9)
    assert nf == 6 * 4
