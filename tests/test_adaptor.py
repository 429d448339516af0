"""The C++ adaptor header (include/bclbm_lbsolver.hpp) compiled against the
reference's own lbsolver headers and run on the reference's Grid/Nodes objects.

Needs the reference sources (skipped where they are absent, e.g. on the GPU
machine); runs on the CPU: the tables it extracts must equal the reference's
tables bit for bit, and without a GPU the LbStep constructor must report the
C ABI's BCLBM_ERR_NOCUDA through the adaptor's error path.
"""

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
REF = Path(os.environ.get("BCLBM_REFERENCE", Path(__file__).resolve().parents[2] / "reference"))

pytestmark = pytest.mark.skipif(not (REF / "src" / "LBSOLVER.h").exists(), reason="reference sources absent")


@pytest.fixture(scope="module")
def checker(tmp_path_factory, native_lib):
    exe = tmp_path_factory.mktemp("adaptor") / "adaptor_check"
    lib = REPO / "badchimp-cpp_gb300"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-w", f"-I{REF / 'src'}", f"-I{REPO / 'oracle' / 'mpi_stub'}",
           f"-I{REPO / 'include'}", str(REPO / "tests" / "adaptor_check.cpp"), "-o", str(exe), f"-L{lib}", "-lbclbm",
           f"-Wl,-rpath,{lib}"]
    subprocess.run(cmd, check=True)
    return exe


def test_adaptor_tables_equal_the_reference(bclbm, checker, tmp_path):
    import sys
    sys.path.insert(0, str(REPO / "tests" / "golden"))
    import make_golden
    geo, _, _ = bclbm.geometry.sphere_pack((14, 12, 10), radius=3.0, porosity=0.45, seed=4)
    vtk = make_golden.write_vtklb(REF, tmp_path, geo, "D3Q19", "xyz", {"init_rho": np.ones(geo.shape)})
    res = subprocess.run([str(checker), str(vtk), str(tmp_path)], capture_output=True, text=True, check=True)
    neigh = np.fromfile(tmp_path / "neigh.i32", dtype=np.int32)
    types = np.fromfile(tmp_path / "types.i16", dtype=np.int16)
    pos = np.fromfile(tmp_path / "pos.i32", dtype=np.int32)
    bulk = np.fromfile(tmp_path / "bulk.i32", dtype=np.int32)
    lat = bclbm.geometry.build_lattice(geo, "D3Q19", "xyz")
    assert np.array_equal(neigh, lat["neigh"])
    assert np.array_equal(types, lat["types"])
    assert np.array_equal(pos, lat["pos"])
    assert np.array_equal(bulk, np.nonzero(lat["types"] > 1)[0])
    # bclbm::Output writes the reference Output's files byte for byte
    import re
    created = re.compile(rb"<!-- Created [^>]* -->")
    ref_files = sorted(p.relative_to(tmp_path / "ref_out") for p in (tmp_path / "ref_out").rglob("*") if p.is_file())
    our_files = sorted(p.relative_to(tmp_path / "our_out") for p in (tmp_path / "our_out").rglob("*") if p.is_file())
    assert ref_files == our_files and len(ref_files) == 10
    for rel in ref_files:
        a = created.sub(b"", (tmp_path / "ref_out" / rel).read_bytes())
        b = created.sub(b"", (tmp_path / "our_out" / rel).read_bytes())
        assert a == b, rel
    import torch
    lines = res.stdout.splitlines()
    if not torch.cuda.is_available():
        assert lines[0].startswith("status bclbm: bclbm_create failed: "), res.stdout
        assert bclbm.native.lib().bclbm_error(-8).decode() in lines[0]
        assert lines[1].startswith("links status bclbm: bclbm_create failed: "), res.stdout
    else:
        assert lines[0].startswith("ran ") and lines[1].startswith("links ran "), res.stdout
