"""The VTU writer (bclbm_output_*) against the reference's own output step
(src/io/Output.h, src/io/VTK.h): the same write sequence on the same fields
gives the same files byte for byte (the PVTU "Created" time aside).

The fixtures tests/golden/vtu_<case>.npz hold the reference's files (written by
oracle/ref_driver.cpp's vtu mode, see tests/golden/make_golden.py); where the
reference and its compiled driver are present, a larger case is also run live.
Host code only: no GPU."""

import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import lbcases

REPO = Path(__file__).resolve().parent.parent
GOLDEN = REPO / "tests" / "golden"
REF = Path(os.environ.get("BCLBM_REFERENCE", Path(__file__).resolve().parents[2] / "reference"))
CREATED = re.compile(rb"<!-- Created [^>]* -->")


def write_ours(bclbm, lat, rho, vel, root: Path):
    """The sequence of the reference driver's vtu mode, with bclbm.output.Output."""
    O = bclbm.output
    bulk = lat.bulk
    o64 = O.Output(lat, bulk, root / "f64")
    o64.add_file("lb_run")
    o64.add_scalar_variables(["rho"], [rho])
    o64.add_vector_variables(["vel"], [vel])
    o64.add_file("second")
    o64.add_scalar_variables(["rho"], [rho])
    o64.write(0)
    rho *= 2.0  # in place: the writer reads the arrays at each write
    o64.write(1000)
    o64.close()
    o32 = O.Output(lat, bulk, root / "f32", dtype=np.float32)
    o32.add_file("lb_f32")
    o32.add_vector_variables(["vel"], [vel])
    o32.add_scalar_variables(["rho"], [rho])
    o32.write(0.5)
    o32.close()
    oa = O.Output(lat, bulk, root / "ascii", fmt=O.ASCII)
    oa.add_file("lb_ascii")
    oa.add_scalar_variables(["rho"], [rho])
    oa.add_vector_variables(["vel"], [vel])
    oa.write(2)
    oa.close()
    # Nodes::geo (src/lbsolver/LBnodes.h:93-99): 1 solid, 0 fluid, -1 at the ghost node
    geo = np.where(lat.types <= 1, 1, 0).astype(np.int32)
    geo[0] = -1
    go = O.Output.from_positions(lat.pos, lat.nd, root / "geo", varname="geo", var=geo, dtype=np.int32)
    go.write()
    go.close()


def read_tree(root: Path):
    out = {}
    for sub in ("f64", "f32", "ascii", "geo"):
        for p in sorted((root / sub).rglob("*")):
            if p.is_file():
                out[str(p.relative_to(root))] = p.read_bytes()
    return out


def same_files(got: dict, want: dict):
    assert sorted(got) == sorted(want)
    for k in want:
        a, b = CREATED.sub(b"", got[k]), CREATED.sub(b"", want[k])
        assert a == b, (k, len(a), len(b), next((i for i in range(min(len(a), len(b))) if a[i] != b[i]), None))


@pytest.mark.parametrize("name", ["disc_40x32", "box_12x10x8"])
def test_files_equal_the_reference_fixture(bclbm, tmp_path, name):
    case = lbcases.Case(name, bclbm)
    z = np.load(GOLDEN / f"vtu_{name}.npz")
    names = bytes(z["names"]).decode().split("\n")
    want = {n: bytes(z[f"file{i}"]) for i, n in enumerate(names)}
    rho, vel = z["rho"].copy(), z["vel"].copy()
    write_ours(bclbm, case.lat, rho, vel, tmp_path)
    same_files(read_tree(tmp_path), want)
    # the created line is there and well formed
    pvtu = (tmp_path / "f64" / "lb_run_0000000.pvtu").read_bytes()
    assert re.search(rb"<!-- Created \d\d\.\d\d\.\d{4} \d\d:\d\d:\d\d -->", pvtu)


@pytest.mark.skipif(not (REF / "PythonScripts" / "vtklb.py").exists()
                    or not (REPO / "oracle" / "_ref" / "ref_driver_d3q19").exists(),
                    reason="needs the reference's vtklb.py and oracle/_ref (make -C oracle ref)")
def test_files_equal_the_reference_live(bclbm, tmp_path):
    sys.path.insert(0, str(GOLDEN))
    import make_golden
    case = lbcases.Case("pack_20", bclbm)
    mask = case.z["mask"]
    vtk = make_golden.write_vtklb(REF, tmp_path, mask, "D3Q19", case.meta["periodic"],
                                  {"init_rho": np.ones(mask.shape)})
    rho, vel = make_golden.vtu_fields(case.n_nodes, 2, 3, 99)
    want = make_golden.reference_vtu(REF, tmp_path, vtk, "D3Q19", 2, rho.copy(), vel.copy())
    ours = tmp_path / "ours"
    ours.mkdir()  # the writer makes the last two levels only, as the reference does
    write_ours(bclbm, case.lat, rho.copy(), vel.copy(), ours)
    same_files(read_tree(ours), want)


def read_appended(path: Path):
    """The arrays of a binary VTU (raw appended data, UInt32 or UInt64 counts)."""
    data = path.read_bytes()
    head, _, rest = data.partition(b'<AppendedData encoding="raw">\n_')
    wide = b'header_type="UInt64"' in head
    arrays = {}
    for m in re.finditer(rb'<DataArray Name="([^"]+)" type="([^"]+)" NumberOfComponents="(\d+)" '
                         rb'format="appended" offset="(\d+)"', head):
        name, typ, off = m.group(1).decode(), m.group(2).decode(), int(m.group(4))
        hdr = 8 if wide else 4
        n = int(np.frombuffer(rest[off:off + hdr], dtype=np.uint64 if wide else np.uint32)[0])
        dt = {"Float64": np.float64, "Float32": np.float32, "Int32": np.int32}[typ]
        arrays[name] = np.frombuffer(rest[off + hdr:off + hdr + n], dtype=dt)
    return arrays


def test_values_and_mesh(bclbm, tmp_path):
    """Size-independent checks on a larger lattice: cell values are the fields at
    the written nodes, connectivity points at the cells' corners, async writes
    give the same files as synchronous ones."""
    mask = bclbm.geometry.sphere_pack((48, 40, 36), radius=5, porosity=0.4, seed=3)[0]
    lat = bclbm.lbsolver.Lattice.from_geometry(mask, "D3Q19", "xyz")
    rng = np.random.default_rng(5)
    rho = rng.uniform(0.9, 1.1, (lat.n_nodes, 1))
    vel = rng.normal(0, 1e-3, (lat.n_nodes, 1, 3))
    O = bclbm.output
    with O.Output(lat, lat.bulk, tmp_path / "a") as o:
        o.add_file("run")
        o.add_scalar_variables(["rho"], [rho])
        o.add_vector_variables(["vel"], [vel])
        o.write(0)
        o.write_async(1)
        o.wait()
        npts = o.n_points
    arr = read_appended(tmp_path / "a" / "vtu" / "0000_run_0000000.vtu")
    assert np.array_equal(arr["rho"], rho[lat.bulk, 0])
    assert np.array_equal(arr["vel"].reshape(-1, 3), vel[lat.bulk, 0])
    pts = arr["points"].reshape(-1, 3)
    assert pts.shape[0] == npts
    conn = arr["connectivity"].reshape(-1, 8)
    pos = lat.pos.reshape(-1, 3)[lat.bulk]
    corner = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1]])
    assert np.array_equal(pts[conn], (pos[:, None, :] + corner[None]).astype(np.float32) - 0.5)
    assert np.array_equal(arr["offsets"], 8 * np.arange(1, lat.n_bulk + 1))
    assert np.all(arr["types"] == 11)
    a = (tmp_path / "a" / "vtu" / "0000_run_0000000.vtu").read_bytes()
    b = (tmp_path / "a" / "vtu" / "0000_run_0000001.vtu").read_bytes()
    assert a == b  # async write of the same values


def test_errors(bclbm, tmp_path):
    O = bclbm.output
    N = bclbm.native
    case = lbcases.Case("disc_40x32", bclbm)
    lat = case.lat
    rho = np.ones((lat.n_nodes, 1))
    o = O.Output(lat, lat.bulk, tmp_path / "e")
    with pytest.raises(N.BclbmError, match="add an output file"):
        o.add_scalar_variables(["rho"], [rho])
    o.add_file("x")
    with pytest.raises(ValueError):
        o.add_vector_variables(["vel"], [np.ones((lat.n_nodes, 1, 3))])  # 3 components on a 2-D lattice
    with pytest.raises(N.BclbmError, match="wrong dimension"):
        o.add_variables(["bad"], [np.ones(lat.n_bulk * 5)])
    with pytest.raises(ValueError):
        o.add_variable_with_names(["a"], np.ones((lat.n_nodes, 2)))
    o.close()
    with pytest.raises(N.BclbmError):
        o.write(0)
    with pytest.raises(N.BclbmError):
        O.Output(lat, lat.bulk, tmp_path / "m", nproc=2, rank=0)  # several ranks share the PVTU
    # a directory that cannot be made: the write reports it
    blocker = tmp_path / "file"
    blocker.write_text("x")
    o = O.Output(lat, lat.bulk, blocker / "sub")
    o.add_file("x")
    o.add_scalar_variables(["rho"], [rho])
    with pytest.raises(N.BclbmError, match="cannot open"):
        o.write(0)
    o.write_async(0)
    with pytest.raises(N.BclbmError, match="cannot open"):
        o.wait()
    o.close()


def test_add_variable_with_names(bclbm, tmp_path):
    O = bclbm.output
    case = lbcases.Case("disc_40x32", bclbm)
    lat = case.lat
    rng = np.random.default_rng(1)
    rho = rng.uniform(0, 1, (lat.n_nodes, 2))
    with O.Output(lat, lat.bulk, tmp_path / "n") as o:
        o.add_file("x")
        o.add_variable_with_names(["red", "blue"], rho)
        o.write(0)
    arr = read_appended(tmp_path / "n" / "vtu" / "0000_x_0000000.vtu")
    # the reference appends the field number to these names too (Output.h:166-169)
    assert np.array_equal(arr["red0"], rho[lat.bulk, 0]) and np.array_equal(arr["blue1"], rho[lat.bulk, 1])


def test_uint64_header_form(bclbm, tmp_path):
    """BCLBM_VTU_BINARY64: the same arrays with header_type="UInt64", 64-bit
    counts and offsets (the form the writer switches to past 2^31 bytes)."""
    O = bclbm.output
    case = lbcases.Case("box_12x10x8", bclbm)
    lat = case.lat
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.9, 1.1, (lat.n_nodes, 1))
    vel = rng.normal(0, 1e-3, (lat.n_nodes, 1, 3))
    arrs = {}
    for fmt, sub in ((O.BINARY, "n"), (O.BINARY64, "w")):
        with O.Output(lat, lat.bulk, tmp_path / sub, fmt=fmt) as o:
            o.add_file("x")
            o.add_scalar_variables(["rho"], [rho])
            o.add_vector_variables(["vel"], [vel])
            o.write(0)
        path = tmp_path / sub / "vtu" / "0000_x_0000000.vtu"
        head = path.read_bytes().split(b"<AppendedData")[0]
        assert (b'header_type="UInt64"' in head) == (fmt == O.BINARY64)
        arrs[sub] = read_appended(path)
    assert sorted(arrs["n"]) == sorted(arrs["w"])
    for k in arrs["n"]:
        assert np.array_equal(arrs["n"][k], arrs["w"][k]), k
    assert np.array_equal(arrs["w"]["rho"], rho[lat.bulk, 0])
