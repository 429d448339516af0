"""Generates the golden fixtures in this folder from the reference itself.

Run from the repository root where the reference sources are present:

    make -C oracle ref                       # builds oracle/_ref from the reference sources
    python tests/golden/make_golden.py [--reference PATH]

For every case it writes the geometry with the reference's own
``PythonScripts/vtklb.py`` (imported from the reference tree), runs the
reference lbsolver through ``oracle/_ref/ref_driver_<lattice>`` and stores

* the tables the reference builds from that file (neighbour table, node types,
  positions, bulk / fluid-boundary / solid-boundary lists, half-way
  bounce-back link classes), and
* the reference's populations, densities, velocities (and colour field) after
  the stated number of steps, restricted to the fluid nodes,

in ``<case>.npz``.  The 256x64 channel is additionally run through
the UNMODIFIED ``src/std_case/main.cpp`` and its VTU output is compared with
the ref_driver dump, which pins ref_driver itself.

``vtu_<case>.npz`` holds the reference's own output step (``src/io/Output.h``
through ``ref_driver vtu``) on seeded fields: the fields and the bytes of every
VTU/PVTU file it wrote.

The fixtures are inputs to the tests; nothing at test time reads the
reference tree.
"""

from __future__ import annotations

import argparse
import importlib.util
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def load_geometry():
    spec = importlib.util.spec_from_file_location("bclbm_geometry", REPO / "badchimp-cpp_gb300" / "geometry.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


geometry = load_geometry()


def read_lbfield(path):
    with open(path, "rb") as fh:
        nf, nq, nn = np.frombuffer(fh.read(12), dtype=np.int32)
        data = np.frombuffer(fh.read(), dtype=np.float64)
    return data.reshape(nn, nf, nq)


def read_scalar(path):
    with open(path, "rb") as fh:
        nf, nn = np.frombuffer(fh.read(8), dtype=np.int32)
        data = np.frombuffer(fh.read(), dtype=np.float64)
    return data.reshape(nn, nf)


def read_vector(path):
    with open(path, "rb") as fh:
        nf, nd, nn = np.frombuffer(fh.read(12), dtype=np.int32)
        data = np.frombuffer(fh.read(), dtype=np.float64)
    return data.reshape(nn, nf, nd)


def read_vtu_array(path, name):
    """One float64 DataArray of a raw-appended VTU (src/io/VTK.h:1165-1178, 730-765)."""
    raw = Path(path).read_bytes()
    head_end = raw.index(b'<AppendedData encoding="raw">')
    head = raw[:head_end].decode("ascii", "replace")
    m = re.search(r'<DataArray[^>]*Name="%s"[^>]*>' % re.escape(name), head)
    if m is None:
        raise KeyError(name)
    off = int(re.search(r'offset="(\d+)"', m.group(0)).group(1))
    start = raw.index(b"_", head_end) + 1 + off
    nbytes = int(np.frombuffer(raw[start:start + 4], dtype=np.uint32)[0])
    return np.frombuffer(raw[start + 4:start + 4 + nbytes], dtype=np.float64).copy()


def write_vtklb(ref: Path, workdir: Path, mask, lattice, periodic, attrs):
    sys.path.insert(0, str(ref / "PythonScripts"))
    try:
        import vtklb as vtklb_mod  # the reference's own writer
    finally:
        sys.path.pop(0)
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        vt = vtklb_mod.vtklb(np.asarray(mask, dtype=int), lattice, periodic, "tmp", str(workdir) + "/")
        for name, arr in attrs.items():
            vt.append_data_set(name, np.asarray(arr))
    return workdir / "tmp0.vtklb"


def run(cmd, cwd=None):
    res = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {res.stdout}\n{res.stderr}")
    return res.stdout


def two_phase_fields(mask, seed, p=0.5, wett=0.5):
    rng = np.random.default_rng(seed)
    red = (rng.random(mask.shape) < p).astype(np.float64)
    rho0 = np.where(mask == 1, red, 0.0)
    rho1 = np.where(mask == 1, 1.0 - red, 0.0)
    return {"rho0": rho0, "rho1": rho1, "wettability": np.full(mask.shape, wett)}


def cases():
    """Geometries and runs.  Sizes are chosen so the oracle finishes in seconds,
    except the 256x64 channel at its full 20,000 steps."""
    out = []
    # D2Q9 channel 256x64, walls at y=0 and y=63, periodic x, tau=1, gx=1e-6.
    ch = geometry.channel_2d(256, 64)
    out.append(dict(name="channel_256x64", lattice="D2Q9", periodic="x", mask=ch,
                    attrs={"init_rho": np.ones(ch.shape)},
                    runs=[dict(tag="bgk_100", mode="single", steps=100, tau=1.0, fx=1e-6),
                          dict(tag="bgk_20000", mode="single", steps=20000, tau=1.0, fx=1e-6)]))
    # Small D2Q9 porous box, periodic in x and y, for the 2D two-phase path and TRT.
    m2, _, _ = geometry.sphere_pack((40, 32), radius=4.0, porosity=0.6, seed=7)
    out.append(dict(name="disc_40x32", lattice="D2Q9", periodic="xy", mask=m2,
                    attrs={"init_rho": np.ones(m2.shape), **two_phase_fields(m2, 11)},
                    runs=[dict(tag="trt_300", mode="single", steps=300, tau=0.8, tau_anti=1.125, trt=1, fx=1e-5),
                          dict(tag="rk_200", mode="twophase", steps=200, tau0=1.0, tau1=1.0, sigma=0.01,
                               beta=0.99, fx=1e-5)]))
    # D3Q19 periodic sphere packs (the 256^3 / 192^3 configurations, scaled down).
    m3, _, _ = geometry.sphere_pack((20, 20, 20), radius=4.0, porosity=0.45, seed=3)
    out.append(dict(name="pack_20", lattice="D3Q19", periodic="xyz", mask=m3,
                    attrs={"init_rho": np.ones(m3.shape), **two_phase_fields(m3, 5)},
                    runs=[dict(tag="bgk_500", mode="single", steps=500, tau=0.8, fx=1e-5),
                          dict(tag="trt_500", mode="single", steps=500, tau=0.8, tau_anti=1.125, trt=1, fx=1e-5),
                          dict(tag="rk_100", mode="twophase", steps=100, tau0=1.0, tau1=1.0, sigma=0.01,
                               beta=0.99, fx=1e-5),
                          dict(tag="rkflux_60", mode="twophase", steps=60, tau0=1.0, tau1=0.7, sigma=0.01,
                               beta=0.99, fx=0.0, momx=1e-4)]))
    # Non-periodic D3Q19 box (x periodic only): faces without periodicity bounce back off node 0.
    mb = np.ones((12, 10, 8), dtype=np.int8)
    xx, yy, zz = np.indices(mb.shape)
    mb[(xx - 6) ** 2 + (yy - 5) ** 2 + (zz - 4) ** 2 <= 6.5] = 0
    out.append(dict(name="box_12x10x8", lattice="D3Q19", periodic="x", mask=mb,
                    attrs={"init_rho": np.ones(mb.shape)},
                    runs=[dict(tag="bgk_400", mode="single", steps=400, tau=0.9, fx=1e-5, fy=2e-6)]))
    return out


def make_case(ref: Path, case: dict, keep_dir=None):
    lt = case["lattice"].lower()
    drv = REPO / "oracle" / "_ref" / f"ref_driver_{lt}"
    if not drv.exists():
        raise SystemExit(f"{drv} missing: run 'make -C oracle ref' first")
    work = Path(tempfile.mkdtemp(prefix="bclbm_golden_"))
    try:
        vtk = write_vtklb(ref, work, case["mask"], case["lattice"], case["periodic"], case["attrs"])
        tdir = work / "tables"
        tdir.mkdir()
        run([str(drv), "tables", str(vtk), str(tdir)])
        nq = geometry.LATTICE_Q[case["lattice"]]
        nd = 2 if nq == 9 else 3
        arrays = {
            "mask": np.asarray(case["mask"], dtype=np.uint8),
            "neigh": np.fromfile(tdir / "neigh.i32", dtype=np.int32),
            "types": np.fromfile(tdir / "types.i16", dtype=np.int16),
            "pos": np.fromfile(tdir / "pos.i32", dtype=np.int32),
            "bulk": np.fromfile(tdir / "bulk.i32", dtype=np.int32),
            "fluidbnd": np.fromfile(tdir / "fluidbnd.i32", dtype=np.int32),
            "solidbnd": np.fromfile(tdir / "solidbnd.i32", dtype=np.int32),
            "links_fluidbnd": np.fromfile(tdir / "links_fluidbnd.i32", dtype=np.int32),
            "links_bulk": np.fromfile(tdir / "links_bulk.i32", dtype=np.int32),
        }
        nf = arrays["bulk"].size
        for name, arr in case["attrs"].items():
            arrays["attr_" + name] = np.asarray(arr, dtype=np.float64)
        meta = {"name": case["name"], "lattice": case["lattice"], "periodic": case["periodic"],
                "nq": nq, "nd": nd, "nf": int(nf), "n_nodes": int(arrays["types"].size), "runs": []}
        for r in case["runs"]:
            rdir = work / r["tag"]
            rdir.mkdir()
            kv = [f"{k}={v!r}" for k, v in r.items() if k not in ("tag", "mode")]
            run([str(drv), r["mode"], str(vtk), str(rdir)] + kv)
            f = read_lbfield(rdir / "f.lblbf")
            rho = read_scalar(rdir / "rho.lbsca")
            vel = read_vector(rdir / "vel.lbvec")
            arrays[f"{r['tag']}_f"] = f[1:nf + 1].copy()
            arrays[f"{r['tag']}_rho"] = rho[1:nf + 1].copy()
            arrays[f"{r['tag']}_vel"] = vel[1:nf + 1].copy()
            if r["mode"] == "twophase":
                arrays[f"{r['tag']}_cg"] = read_scalar(rdir / "cg.lbsca")[:, 0].copy()
                arrays[f"{r['tag']}_force"] = np.fromfile(rdir / "force.f64", dtype=np.float64)
            meta["runs"].append({k: v for k, v in r.items()})
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(HERE / f"{case['name']}.npz", **arrays)
        print(f"{case['name']}: N={meta['n_nodes']} Nf={nf} runs={[r['tag'] for r in case['runs']]}")
        if case["name"] == "channel_256x64":
            pin_std_case(ref, vtk, work)
    finally:
        if keep_dir is None:
            shutil.rmtree(work, ignore_errors=True)


def pin_std_case(ref: Path, vtk: Path, work: Path):
    """Runs the unmodified std_case main on the 256x64 channel and compares its VTU output
    with the ref_driver dump after the same number of steps."""
    exe = REPO / "oracle" / "_ref" / "std_case_d2q9"
    root = work / "std_case"
    (root / "input" / "mpi").mkdir(parents=True)
    (root / "output").mkdir()
    (root / "run").mkdir()
    shutil.copy(vtk, root / "input" / "mpi" / "tmp0.vtklb")
    n_it = 300
    (root / "input" / "input.dat").write_text(
        f"<iterations>\n  max {n_it}\n  write {n_it}\n<end>\n"
        "<fluid>\n  tau 1.0\n  bodyforce 1e-6 0.0\n<end>\n")
    run([str(exe)], cwd=root / "run")
    vtus = sorted((root / "output").rglob("*lb_run*.vtu"))
    last = vtus[-1]
    rho_vtu = read_vtu_array(last, "rho")
    vel_vtu = read_vtu_array(last, "vel").reshape(-1, 3)[:, :2]  # VTK vectors carry 3 components
    drv = REPO / "oracle" / "_ref" / "ref_driver_d2q9"
    ddir = work / "pin"
    ddir.mkdir()
    # std_case runs iterations 0..max inclusive; the moments written at the last
    # iteration are those of ref_driver's last step when it runs max+1 steps.
    run([str(drv), "single", str(root / "input" / "mpi" / "tmp0.vtklb"), str(ddir),
         f"steps={n_it + 1}", "tau=1.0", "fx=1e-6"])
    nf = rho_vtu.size
    rho_d = read_scalar(ddir / "rho.lbsca")[1:nf + 1, 0]
    vel_d = read_vector(ddir / "vel.lbvec")[1:nf + 1, 0, :]
    if not (np.array_equal(rho_vtu, rho_d) and np.array_equal(vel_vtu, vel_d)):
        raise SystemExit("driver does not reproduce the unmodified std_case output")
    (HERE / "std_case_pin.json").write_text(json.dumps({
        "what": "unmodified src/std_case/main.cpp (D2Q9) vs oracle/ref_driver.cpp, 256x64 channel geometry",
        "iterations": n_it, "fluid_nodes": int(nf), "rho_bit_exact": True, "vel_bit_exact": True,
        "vtu": last.name}, indent=1) + "\n")
    print(f"std_case pin: {last.name} rho/vel bit-exact against ref_driver ({nf} nodes)")


# The VTU fixtures: (case, fields per node, seed)
VTU_CASES = [("disc_40x32", 2, 11), ("box_12x10x8", 1, 12)]


def vtu_fields(n_nodes, nfields, nd, seed):
    """Seeded rho [N, nF] and vel [N, nF, nD], with zeros, a negative zero and
    values below the ASCII writer's 1e-20 cut."""
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.5, 1.5, (n_nodes, nfields))
    vel = rng.normal(0.0, 0.01, (n_nodes, nfields, nd))
    rho[3, 0] = 0.0
    rho[5, 0] = 1e-25
    vel[4, 0, 0] = -0.0
    vel[6, 0, nd - 1] = -3e-22
    vel[7, 0, 0] = 123456.789
    return rho, vel


def reference_vtu(ref: Path, work: Path, vtk: Path, lattice: str, nfields: int, rho, vel):
    """Runs the reference's output step on the fields; returns {relative path: bytes}."""
    out = work / "vtu_ref"
    out.mkdir(parents=True, exist_ok=True)
    with open(out / "fields.bin", "wb") as fh:
        fh.write(np.ascontiguousarray(rho, dtype=np.float64).tobytes())
        fh.write(np.ascontiguousarray(vel, dtype=np.float64).tobytes())
    exe = REPO / "oracle" / "_ref" / f"ref_driver_{lattice.lower()}"
    run([str(exe), "vtu", str(vtk), str(out), f"nfields={nfields}"])
    files = {}
    for sub in ("f64", "f32", "ascii", "geo"):
        for p in sorted((out / sub).rglob("*")):
            if p.is_file():
                files[str(p.relative_to(out))] = p.read_bytes()
    return files


def make_vtu(ref: Path, name: str, nfields: int, seed: int):
    z = np.load(HERE / f"{name}.npz")
    meta = json.loads(bytes(z["meta"]).decode())
    work = Path(tempfile.mkdtemp(prefix="bclbm_vtu_"))
    try:
        mask = z["mask"]
        vtk = write_vtklb(ref, work, mask, meta["lattice"], meta["periodic"], {"init_rho": np.ones(mask.shape)})
        rho, vel = vtu_fields(meta["n_nodes"], nfields, meta["nd"], seed)
        files = reference_vtu(ref, work, vtk, meta["lattice"], nfields, rho, vel)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    arrays = {"rho": rho, "vel": vel, "nfields": np.array(nfields),
              "names": np.frombuffer("\n".join(files).encode(), dtype=np.uint8)}
    for i, (k, v) in enumerate(files.items()):
        arrays[f"file{i}"] = np.frombuffer(v, dtype=np.uint8)
    np.savez_compressed(HERE / f"vtu_{name}.npz", **arrays)
    print(f"vtu_{name}.npz: {len(files)} files, {sum(len(v) for v in files.values())} bytes")


# ---------------------------------------------------------------------------
# std_one_phase: relative-permeability geometry with node tags (0 solid, 1 / 2
# fluid phase, 3 pressure ghost, +4 fluid-fluid, +8 fluid-solid, +16 pressure
# boundary), interior domains with mass sources, a force indicator and normals.
# ---------------------------------------------------------------------------
ONEPHASE_DIRS = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1], [0, 1, 1],
                          [0, 1, -1], [-1, 0, 0], [0, -1, 0], [0, 0, -1], [-1, -1, 0], [-1, 1, 0], [-1, 0, -1],
                          [-1, 0, 1], [0, -1, -1], [0, -1, 1]])


def onephase_geometry(shape, seed, ghost_layers=True):
    """Mask (1 fluid) and voxel attributes of a periodic-in-x,y box whose z faces
    are pressure boundaries: with ghost_layers the faces z = 0 and z = nz-1 are
    ghost nodes (tag 3, solid); without, the fluid reaches the faces and their
    neighbour beyond is node 0 (tag -1 in Nodes, which counts as a ghost)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    x, y, z = np.indices(shape)
    mask = np.ones(shape, dtype=np.int8)
    z0, z1 = (1, nz - 2) if ghost_layers else (0, nz - 1)
    # phase 2: two blobs away from the pressure faces (interior domains 1 and 2),
    # kept free of solid so that each has interior (untagged) nodes
    blobs = [((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= 3.0 ** 2)
             for c in ((3.0, 3.0, nz / 2 - 1), (nx - 3.5, ny - 4.0, nz / 2 + 1))]
    for _ in range(3):
        c = rng.uniform([0, 0, z0 + 3], [nx, ny, z1 - 2])
        d2 = sum(np.minimum(np.abs(a - ci), n - np.abs(a - ci)) ** 2 for a, ci, n in ((x, c[0], nx), (y, c[1], ny))) \
            + (z - c[2]) ** 2
        mask[(d2 <= 2.2 ** 2) & ~blobs[0] & ~blobs[1]] = 0
    if ghost_layers:
        mask[:, :, 0] = 0
        mask[:, :, -1] = 0
    ghost = np.zeros(shape, dtype=bool)
    if ghost_layers:
        ghost[:, :, 0] = ghost[:, :, -1] = True
    phase = np.where(mask == 1, 1, 0)
    labels = np.zeros(shape, dtype=np.int64)
    for lab, b in enumerate(blobs, start=1):
        blob = b & (mask == 1)
        phase[blob] = 2
        labels[blob] = lab
    tags = np.where(ghost, 3, np.where(mask == 1, phase, 0)).astype(np.int64)
    base = tags.copy()
    for c in ONEPHASE_DIRS:
        nb = np.roll(base, shift=(-c[0], -c[1]), axis=(0, 1))
        # z neighbours: shifted, outside the box is node 0 (tag -1, & 3 == 3)
        if c[2] != 0:
            nb = np.roll(nb, shift=-c[2], axis=2)
            if c[2] > 0:
                nb[:, :, -1] = -1
            else:
                nb[:, :, 0] = -1
        fl = mask == 1
        other = np.where(phase == 1, 2, 1)
        tags[fl & ((nb & 3) == other) & ((nb & 3) != 0)] |= 4
        tags[fl & ((nb & 3) == 0) & (nb >= 0)] |= 8
        tags[fl & ((nb & 3) == 3)] |= 16
    force = np.where(mask == 1, 1, 0).astype(np.int64)
    force[:, :, z0] = 0  # no body force on the first fluid layer
    nrm = rng.normal(size=(3,) + shape)
    nrm /= np.linalg.norm(nrm, axis=0)
    attrs = {"nodetags": tags, "force": force, "interior_domains": labels,
             "normal_x": nrm[0], "normal_y": nrm[1], "normal_z": nrm[2]}
    return mask, attrs


ONEPHASE_CASES = [
    dict(name="onephase_ghost", shape=(10, 9, 14), seed=21, ghost_layers=True, steps=300, tau=0.9,
         fx=2e-6, fy=0.0, fz=1e-5),
    dict(name="onephase_open", shape=(9, 10, 12), seed=22, ghost_layers=False, steps=200, tau=0.8,
         fx=0.0, fy=1e-6, fz=2e-5),
]


def make_onephase(ref: Path, case: dict):
    drv = REPO / "oracle" / "_ref" / "ref_onephase"
    tdrv = REPO / "oracle" / "_ref" / "ref_driver_d3q19"
    if not drv.exists():
        raise SystemExit(f"{drv} missing: run 'make -C oracle ref' first")
    mask, attrs = onephase_geometry(case["shape"], case["seed"], case["ghost_layers"])
    work = Path(tempfile.mkdtemp(prefix="bclbm_onephase_"))
    try:
        vtk = write_vtklb(ref, work, mask, "D3Q19", "xy", attrs)
        tdir = work / "tables"
        tdir.mkdir()
        run([str(tdrv), "tables", str(vtk), str(tdir)])
        rdir = work / "run"
        rdir.mkdir()
        kv = [f"{k}={case[k]!r}" for k in ("steps", "tau", "fx", "fy", "fz")]
        msg = run([str(drv), str(vtk), str(rdir)] + kv)
        arrays = {"mask": mask.astype(np.uint8),
                  "neigh": np.fromfile(tdir / "neigh.i32", dtype=np.int32),
                  "types": np.fromfile(tdir / "types.i16", dtype=np.int16),
                  "pos": np.fromfile(tdir / "pos.i32", dtype=np.int32),
                  "bulk": np.fromfile(tdir / "bulk.i32", dtype=np.int32)}
        nf = arrays["bulk"].size
        for k, v in attrs.items():
            arrays["attr_" + k] = np.asarray(v)
        arrays["f"] = read_lbfield(rdir / "f.lblbf")[1:nf + 1].copy()
        arrays["rho"] = read_scalar(rdir / "rho.lbsca")[1:nf + 1].copy()
        arrays["vel"] = read_vector(rdir / "vel.lbvec")[1:nf + 1].copy()
        arrays["flux"] = np.array([float(v) for v in (rdir / "flux.txt").read_text().split()])
        meta = {k: case[k] for k in ("name", "shape", "seed", "ghost_layers", "steps", "tau", "fx", "fy", "fz")}
        meta.update(nq=19, nd=3, nf=int(nf), n_nodes=int(arrays["types"].size), periodic="xy", driver=msg.strip())
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(HERE / f"{case['name']}.npz", **arrays)
        print(f"{case['name']}: N={meta['n_nodes']} Nf={nf}; {msg.strip()}")
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("BCLBM_REFERENCE", str(Path(__file__).resolve().parents[3] / "reference")))
    ap.add_argument("--only", default=None)
    ap.add_argument("--pin-only", action="store_true", help="only rerun the std_case pin of the 256x64 channel")
    ap.add_argument("--vtu-only", action="store_true", help="only rewrite the VTU fixtures")
    ap.add_argument("--onephase-only", action="store_true", help="only rewrite the std_one_phase fixtures")
    args = ap.parse_args()
    ref = Path(args.reference)
    if args.pin_only:
        work = Path(tempfile.mkdtemp(prefix="bclbm_pin_"))
        try:
            ch = geometry.channel_2d(256, 64)
            vtk = write_vtklb(ref, work, ch, "D2Q9", "x", {"init_rho": np.ones(ch.shape)})
            pin_std_case(ref, vtk, work)
        finally:
            shutil.rmtree(work, ignore_errors=True)
        return
    if args.onephase_only:
        for case in ONEPHASE_CASES:
            make_onephase(ref, case)
        return
    if args.vtu_only:
        for name, nf, seed in VTU_CASES:
            make_vtu(ref, name, nf, seed)
        return
    for case in cases():
        if args.only and case["name"] != args.only:
            continue
        make_case(ref, case)
    for name, nf, seed in VTU_CASES:
        if not args.only or args.only == name:
            make_vtu(ref, name, nf, seed)
    for case in ONEPHASE_CASES:
        if not args.only or args.only == case["name"]:
            make_onephase(ref, case)


if __name__ == "__main__":
    main()
