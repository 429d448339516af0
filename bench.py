"""Benchmark of the lattice-Boltzmann time step on GB300.

Workload (one bench step = one time step over every fluid node):
  D3Q19 single phase, periodic 256^3 box of solid spheres (radius 10, seeded
  uniform centres, overlap allowed) filled to porosity 0.40, tau = 0.8,
  body force gx = 1e-5; BGK in plain FP64 is the headline, TRT (Lambda = 3/16)
  and FP32 / FP16 / BF16 shifted storage are reported as variants.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
  (N > 1 under torchrun: independent replicas, one per GPU, weak scaling)

value         MLUPS over all ranks, populations resident in HBM, CUDA events on
              the library's stream, max over ranks
e2e           the same metric through the C ABI with host buffers: create from
              the reference-layout host arrays, K steps with a statistics
              read-back every 50 steps, download of f / rho / u, destroy
roofline      algorithmic bytes per launch (fluid nodes x bytes per update) over
              the average step-kernel duration, against MEASURED_PEAKS.json
cpu_baseline  the oracle (plain-C restatement of the reference step) on the
              host cores, a bounded sample of steps of the same workload
serving       (rank 0) a sample of the serving workload: --requests permeability
              requests from the serving distribution, served by the batched
              server and by sequential single-instance FP64 solves: solves/s,
              p50/p99 latency, permeability error against FP64

  python bench.py --workload serving [--requests R --rates 0,2,5]
  prints the serving measurement as the bench line (solves/s).

  python bench.py --workload output [--size 256 --write-every 1000 --writes 4]
  the std_case loop with VTU output steps, synchronous against asynchronous writes.

  python bench.py --workload links [--size 192]
  the std_one_phase step (link boundaries from node tags, interior-domain mass
  sources) on a tagged sphere pack: FP64 fixed-point, FMA and exact kernels, the
  shifted formats, oracle on the host.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

if int(os.environ.get("WORLD_SIZE", "1")) > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
    # one GPU per rank, seen as device 0 by torch and by libbclbm alike
    os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "D3Q19 MLUPS, HBM GB/s; solves/s, p99 latency vs plain FP64 at ≤1e-3 perm err"
L2_BYTES = 129 * 1024 * 1024
# algorithmic bytes per fluid-node update, pull scheme, int32 neighbours:
# 2 Q s_f (read + write populations) + (Q - 1) * 4 (neighbour table)
BYTES_PER_UPDATE = {"f64": 2 * 19 * 8 + 18 * 4, "f32": 2 * 19 * 4 + 18 * 4, "f16": 2 * 19 * 2 + 18 * 4,
                    "bf16": 2 * 19 * 2 + 18 * 4}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "of measured"
    return 6800.0, "of fallback"


def committed_traffic(kernel_tag: str):
    """dram bytes per launch from the committed ncu summary (profiles/), or None."""
    f = REPO / "profiles" / "traffic.json"
    if not f.exists():
        return None
    try:
        d = json.loads(f.read_text())
        return d.get(kernel_tag, {}).get("traffic_bytes_per_launch")
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu_index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(size: int, radius: float, porosity: float, seed: int):
    import __graft_entry__ as ge
    bclbm = ge.load()
    t = time.time()
    geo, centres, phi = bclbm.geometry.sphere_pack((size, size, size), radius=radius, porosity=porosity, seed=seed)
    lat = bclbm.lbsolver.Lattice.from_geometry(geo, "D3Q19", "xyz")
    log(f"geometry {size}^3: porosity {phi:.4f}, {len(centres)} spheres, fluid {lat.n_bulk}, "
        f"nodes {lat.n_nodes} ({time.time() - t:.1f}s)")
    return bclbm, lat, phi


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
        if backend == "nccl":
            torch.cuda.set_device(0)
    return world, rank


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mlups(world: int, units_per_rank: int, steps: int, max_seconds: float) -> float:
    """Replicas: every rank updates units_per_rank nodes per step; the job took the
    slowest rank's time (max over ranks)."""
    return world * units_per_rank * steps / max_seconds / 1e6


def cpu_port_rate(lat, steps_target_s: float, nthreads: int, tau: float, force, max_steps: int = 1000):
    """Oracle MLUPS on the host cores for a bounded number of steps."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    g = oracle.OracleGrid(lat.nq, lat.neigh, lat.types, lat.bulk)
    from importlib import import_module
    L = import_module("bclbm").lbsolver
    runner = oracle.SingleRunner(g, L.initiate_single(lat, np.ones(lat.n_nodes)), tau, force, nthreads=nthreads)
    t = time.time()
    runner.run(1)
    one = max(time.time() - t, 1e-3)
    steps = int(max(1, min(max_steps, steps_target_s / one)))
    t = time.time()
    runner.run(steps)
    dt = time.time() - t
    return lat.n_bulk * steps / dt / 1e6, steps, dt


class _ReferenceLattice:
    """The tables the reference arm needs: Grid / Nodes / bulk list of one rank."""

    def __init__(self, tables):
        self.nq = tables["nq"]
        self.neigh = tables["neigh"]
        self.types = tables["types"]
        self.n_nodes = int(self.types.size)
        self.bulk = np.arange(1, tables["nf"] + 1, dtype=np.int32)  # findBulkNodes: fluid nodes 1..Nf
        self.n_bulk = int(self.bulk.size)


def reference_workload(size: int, radius: float, porosity: float, seed: int):
    """The benchmark lattice for the reference arm, built without the bclbm
    package: geometry.py is loaded as a file of its own (it needs numpy only) and
    its numpy numbering is used, so that this process loads no libbclbm.so.
    Returns (tables, porosity, f0) with f0 = w_q at the bulk nodes
    (src/std_case/main.cpp:92-96)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bclbm_geometry_numpy", REPO / "badchimp-cpp_gb300" / "geometry.py")
    geometry = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(geometry)
    t = time.time()
    geo, centres, phi = geometry.sphere_pack((size, size, size), radius=radius, porosity=porosity, seed=seed)
    lat = _ReferenceLattice(geometry.build_lattice_numpy(geo, "D3Q19", "xyz"))
    w = np.array([2.0 / 36.0] * 3 + [1.0 / 36.0] * 6 + [2.0 / 36.0] * 3 + [1.0 / 36.0] * 6 + [12.0 / 36.0])
    f0 = np.zeros((lat.n_nodes, lat.nq))
    f0[lat.bulk] = w[None, :]
    log(f"geometry {size}^3 (numpy numbering): porosity {phi:.4f}, {len(centres)} spheres, fluid {lat.n_bulk}, "
        f"nodes {lat.n_nodes} ({time.time() - t:.1f}s)")
    return lat, phi, f0.reshape(-1)


def loaded_shared_objects():
    """Shared objects of this repository mapped into the process (from /proc/self/maps)."""
    try:
        lines = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return None
    out = set()
    for ln in lines:
        p = ln.split()[-1] if ln.split() else ""
        if p.endswith(".so") and p.startswith(str(REPO)):
            out.add(str(Path(p).relative_to(REPO)))
    return sorted(out)


def run_reference(args, world, rank):
    """--impl reference: the CPU implementation of the step on all host cores.

    Timed: oracle/liboracle.so, the plain-C restatement of the reference's
    std_case step (push + half-way bounce-back, src/std_case/main.cpp:109-146),
    bit-identical to the reference's own build on every fixture.  The reference's
    own build (oracle/_ref) is compiled from its sources, which do not exist on
    the GPU machine, so the restatement stands in for it there.  Nothing of the
    bclbm package is imported: the lattice comes from geometry.py's numpy path."""
    if rank != 0:
        return
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    lat, phi, f0 = reference_workload(args.size, args.radius, args.porosity, args.seed)
    nthreads = oracle.default_threads()
    g = oracle.OracleGrid(lat.nq, lat.neigh, lat.types, lat.bulk)
    F = (args.gx, 0.0, 0.0)
    runner = oracle.SingleRunner(g, f0, args.tau, F, nthreads=nthreads)
    # one call per block of steps: the oracle's threads start once per call
    runner.run(args.warmup)
    t = time.time()
    runner.run(args.steps)
    dt = time.time() - t
    mlups = lat.n_bulk * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, lat, phi, "bgk"),
        "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": nthreads, "kind": "port",
                         "sample": f"{args.steps} timed steps of the full workload, oracle (plain-C restatement "
                                   f"of the reference std_case step, push + bounce-back) on {nthreads} host threads"},
        "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "timed_library": "oracle/liboracle.so (oracle_single_run)",
        "shared_objects_loaded": loaded_shared_objects(),
    }
    print(json.dumps(line), flush=True)


def workload_config(args, lat, phi, collision):
    return {"workload": f"D3Q19 {collision.upper()} periodic {args.size}^3 sphere pack, radius {args.radius:g}, "
                        f"porosity {phi:.4f} (target {args.porosity:g}), tau {args.tau:g}, gx {args.gx:g}",
            "fluid_nodes": lat.n_bulk, "lattice_nodes": lat.n_nodes, "seed": args.seed,
            "l2": "inputs larger than L2 (population buffers of several GB against 129 MB L2)",
            "parallelism": f"replicas x{args.gpus}"}


def time_solver(solver, steps, warmup):
    if warmup:
        solver.step(warmup)
        solver.sync()
    return solver.step_timed(steps)


def run_mine(args, world, rank):
    import torch
    bclbm, lat, phi = build_workload(args.size, args.radius, args.porosity, args.seed)
    L = bclbm.lbsolver
    F = (args.gx, 0.0, 0.0)
    f0 = L.initiate_single(lat, np.ones(lat.n_nodes))
    tau_anti = 0.5 + (3.0 / 16.0) / (args.tau - 0.5)
    peak, peak_kind = peaks()
    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0) \
        if os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else 0

    # ---- headline: plain FP64 BGK (by default), resident in HBM -------------------
    launches0 = bclbm.native.launch_count()
    hp = args.precision
    hcoll = L.TRT if args.collision == "trt" else L.BGK
    htau = (args.tau, tau_anti if hcoll == L.TRT else args.tau)
    with L.Solver(lat, f0, collision=hcoll, precision=hp, tau=htau, force=F, exact=args.exact,
                  fma64=args.fma64) as s:
        s.step(args.warmup)
        s.sync()
        torch.cuda.synchronize()
        barrier(world)
        l0 = bclbm.native.launch_count()
        with ClockSampler(gpu_index) as clk:
            tm = s.step_timed(args.steps)
        launches = bclbm.native.launch_count() - l0
        torch.cuda.synchronize()
        barrier(world)
        st = s.reduce()
    total_ms = allreduce_max(world, tm["total_ms"])
    kernel_ms = tm["step_kernel_ms"] / args.steps
    mlups = whole_job_mlups(world, lat.n_bulk, args.steps, total_ms * 1e-3)
    bpu = BYTES_PER_UPDATE[hp]
    achieved = lat.n_bulk * bpu / (kernel_ms * 1e-3) / 1e9
    arith = "exact" if args.exact else ("fma" if args.fma64 else ("fixed" if hp == "f64" else "fp32"))
    kernel_tag = f"k_single_d3q19_{hp}_{arith}_{args.collision}"
    traffic = committed_traffic(kernel_tag)

    # ---- end to end through the C ABI with host buffers (right after the headline, so
    # that the host's memory is in the same state for it as for the headline) -------
    torch.cuda.synchronize()
    barrier(world)
    # the caller's host arrays exist before the solve (the reference's LbField / ScalarField /
    # VectorField are allocated and written at set-up): touch them outside the timed region
    host_f = np.ones_like(f0)
    host_rho = np.ones(lat.n_nodes)
    host_vel = np.ones(lat.n_nodes * 3)
    t = time.perf_counter()
    with L.Solver(lat, f0, collision=L.BGK, precision="f64", tau=(args.tau, args.tau), force=F) as s:
        t_created = time.perf_counter()
        done = 0
        nred = 0
        while done < args.steps:
            n = min(50, args.steps - done)
            s.step(n)
            s.reduce()
            nred += 1
            done += n
        t_stepped = time.perf_counter()
        s.download_f(host_f)
        s.download_macros(host_rho, host_vel)
        t_downloaded = time.perf_counter()
    e2e_s = time.perf_counter() - t
    e2e_parts = {"create_s": t_created - t, "steps_and_reductions_s": t_stepped - t_created,
                 "downloads_s": t_downloaded - t_stepped, "destroy_s": t + e2e_s - t_downloaded}
    e2e_s = allreduce_max(world, e2e_s)
    e2e_mlups = whole_job_mlups(world, lat.n_bulk, args.steps, e2e_s)
    h2d = lat.neigh.nbytes + lat.types.nbytes + lat.bulk.nbytes + f0.nbytes
    d2h = nred * 96 + lat.n_bulk * 19 * 8 + lat.n_bulk * (1 + 3) * 8

    # ---- variants ----------------------------------------------------------------
    variants = {}
    if not args.no_variants:
        for tag, coll, prec in (("trt_f64", L.TRT, "f64"), ("bgk_f32", L.BGK, "f32"), ("bgk_f16", L.BGK, "f16"),
                                ("bgk_bf16", L.BGK, "bf16"), ("bgk_f64_exact", L.BGK, "f64x"),
                                ("bgk_f64_fma", L.BGK, "f64fma")):
            kw = dict(exact=True) if prec == "f64x" else (dict(fma64=True) if prec == "f64fma" else {})
            p = "f64" if prec.startswith("f64") else prec
            with L.Solver(lat, f0, collision=coll, precision=p, tau=(args.tau, tau_anti if coll == L.TRT else args.tau),
                          force=F, **kw) as s:
                vsteps = max(5, args.steps // 2)
                tv = time_solver(s, vsteps, args.warmup)
                stv = s.reduce()
            km = tv["step_kernel_ms"] / vsteps
            v_mlups = lat.n_bulk * vsteps / (tv["total_ms"] * 1e-3) / 1e6
            v_gbs = lat.n_bulk * BYTES_PER_UPDATE[p] / (km * 1e-3) / 1e9
            variants[tag] = {"mlups": v_mlups, "kernel_ms": km, "achieved_gbs": v_gbs,
                             "frac": v_gbs / peak, "bytes_per_update": BYTES_PER_UPDATE[p],
                             "flux_x_after": stv["momentum"][0]}
        if "bgk_f16" in variants:
            variants["f16_speedup_vs_f64"] = variants["bgk_f16"]["mlups"] / mlups * world

    # ---- accuracy: permeability of the shifted formats against FP64 -------------
    accuracy = None
    if rank == 0 and args.accuracy_steps > 0:
        nu = (args.tau - 0.5) / 3.0
        vol = float(args.size) ** 3
        ks = {}
        for prec in ("f64", "f32", "f16", "bf16"):
            with L.Solver(lat, f0, collision=L.BGK, precision=prec, tau=(args.tau, args.tau), force=F) as s:
                s.step(args.accuracy_steps)
                ks[prec] = nu * s.reduce()["momentum"][0] / (vol * args.gx)
        accuracy = {"steps": args.accuracy_steps, "permeability_f64": ks["f64"],
                    "definition": "k = nu * sum_fluid(rho u_x) / (V F_x), FP64 reductions on the GPU",
                    "rel_err_vs_f64": {p: abs(ks[p] - ks["f64"]) / abs(ks["f64"]) for p in ("f32", "f16", "bf16")}}

    # ---- serving: continuous batching against sequential FP64 solves -------------
    serving = None
    if rank == 0 and not args.no_serving:
        serving = serving_measure(args, bclbm)
        for k in ("_head", "_prepared", "_reqs"):
            serving.pop(k)

    # ---- CPU baseline: the oracle on the host cores (rank 0, N = 1) ---------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, str(REPO / "oracle"))
        import oracle
        nth = oracle.default_threads()
        rate, csteps, cdt = cpu_port_rate(lat, args.cpu_seconds, nth, args.tau, F)
        cpu = {"value": rate, "unit": "MLUPS", "cores": nth, "kind": "port",
               "sample": f"{csteps} steps of the same {args.size}^3 workload in {cdt:.1f}s, oracle (plain-C "
                         f"restatement of the reference std_case step) on {nth} host threads"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": hp,
            "data": "synthetic: seeded periodic sphere pack (numpy default_rng), no dataset",
            "config": workload_config(args, lat, phi, args.collision),
            "hbm_gbs": achieved,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": kernel_tag + " (pull stream + fused bounce-back)",
                         "bytes_per_update": bpu, "units_per_launch": lat.n_bulk,
                         "kernel_ms": kernel_ms},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "e2e": {"value": e2e_mlups, "unit": "MLUPS", "seconds": e2e_parts, "h2d_bytes_per_step": h2d / args.steps,
                    "d2h_bytes_per_step": d2h / args.steps,
                    "path": "bclbm_create from host arrays, bclbm_step x K with bclbm_reduce every 50 steps, "
                            "bclbm_download_f + bclbm_download_macros, bclbm_destroy"},
            "gpu_launches": launches,
            "launches_total": bclbm.native.launch_count() - launches0,
            "variants": variants,
            "accuracy": accuracy,
            "serving": serving,
            "check": {"mass": st["mass"][0], "flux_x": st["momentum"][0], "nonfinite": st["nonfinite"]},
        }
        print(json.dumps(line), flush=True)


def serving_measure(args, bclbm):
    """Continuous batching of permeability requests against sequential
    single-instance FP64 solves of the same requests (rank 0, one GPU)."""
    import torch
    import concurrent.futures as cf
    S = bclbm.serving
    reqs = S.sample_requests(args.requests, rate=0.0, seed=args.seed, size_range=(args.size_min, args.size_max),
                             gx=args.gx)
    t = time.time()
    prepared = {}
    with cf.ThreadPoolExecutor(max_workers=8) as pool:
        for r, res in zip(reqs, pool.map(S.prepare, reqs)):
            prepared[r.rid] = res
    log(f"prepared {len(reqs)} requests in {time.time() - t:.1f}s; sides {sorted(r.size for r in reqs)}")
    srv = S.Server(precision=args.serving_precision, check_every=args.check_every, tol=args.tol,
                   max_steps=args.max_steps, steps_per_graph=args.steps_per_graph, promote_tol=args.promote_tol)
    # warm-up: one small request through both paths (graph capture, module load)
    warm = S.sample_requests(1, rate=0.0, seed=1, size_range=(24, 24))
    S.Server(precision=args.serving_precision, check_every=50, max_steps=101).run(warm)
    srv.run_sequential(warm, precision=args.baseline_precision)
    torch.cuda.synchronize()
    out = {}
    rates = [float(x) for x in args.rates.split(",")]
    l0 = bclbm.native.launch_count()
    with ClockSampler(0) as clk:
        base = srv.run_sequential(reqs, precision=args.baseline_precision, prepared=prepared)
        for rate in rates:
            sched = S.sample_requests(args.requests, rate=rate, seed=args.seed,
                                      size_range=(args.size_min, args.size_max), gx=args.gx)
            out[rate] = srv.run(sched, prepared=prepared)
    launches = bclbm.native.launch_count() - l0
    head = out[rates[0]]
    kb = {r.rid: r.permeability for r in base["results"]}
    errs = [abs(r.permeability - kb[r.rid]) / abs(kb[r.rid]) for r in head["results"] if kb[r.rid] != 0]

    def brief(rep):
        return {k: rep[k] for k in ("solves", "seconds", "solves_per_s", "p50_s", "p99_s", "converged",
                                    "lattice_updates")} | {"mlups": rep["lattice_updates"] / rep["seconds"] / 1e6}

    workload = (f"serving: {args.requests} D3Q19 BGK permeability requests, side log-uniform "
                f"[{args.size_min},{args.size_max}], radius U[4,12], porosity U[0.30,0.50], tau U[0.6,1.2], "
                f"gx {args.gx:g}; until |dk/k| < {args.tol:g} over {args.check_every} steps or {args.max_steps} steps")
    return {
        "workload": workload, "precision": args.serving_precision, "rates": rates,
        "arrivals": f"Poisson, rates {rates} /s (0 = all at t=0)",
        "host_preparation": "geometry and node tables built before the timed region for both arms",
        "solves_per_s": head["solves_per_s"], "p50_s": head["p50_s"], "p99_s": head["p99_s"],
        "serving": {str(r): brief(out[r]) | {"counters": out[r]["counters"]} for r in rates},
        "sequential_baseline": brief(base) | {"precision": args.baseline_precision},
        "speedup_solves_per_s": head["solves_per_s"] / base["solves_per_s"],
        "accuracy": {"max_rel_perm_err_vs_baseline": max(errs) if errs else None,
                     "median_rel_perm_err_vs_baseline": float(np.median(errs)) if errs else None},
        "requests": [{"rid": q.rid, "side": q.size, "tau": round(q.tau, 4), "radius": round(q.radius, 3),
                      "porosity": round(q.porosity, 4), "fluid": a.n_fluid, "steps": a.steps,
                      "steps_baseline": c.steps, "latency_s": round(a.latency, 4),
                      "latency_baseline_s": round(c.latency, 4), "k": a.permeability, "k_baseline": c.permeability}
                     for q, a, c in zip(reqs, head["results"], base["results"])],
        "clocks": clk.summary(), "gpu_launches": launches, "_head": head, "_prepared": prepared, "_reqs": reqs,
    }


def run_serving(args, world, rank):
    """--workload serving: the serving measurement as the bench line."""
    import __graft_entry__ as ge
    bclbm = ge.load()
    if rank != 0:
        return
    m = serving_measure(args, bclbm)
    head, prepared, reqs = m.pop("_head"), m.pop("_prepared"), m.pop("_reqs")
    peak, peak_kind = peaks()
    achieved = head["lattice_updates"] / head["seconds"] * BYTES_PER_UPDATE[args.serving_precision.split(">")[-1]] / 1e9
    line = {
        "metric": METRIC, "value": m["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
        "steps": args.requests, "warmup": 1, "ms_per_step": head["seconds"] / max(1, head["solves"]) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.serving_precision,
        "data": "synthetic: seeded periodic sphere packs (numpy default_rng), no dataset",
        "config": {"workload": m["workload"], "arrivals": m["arrivals"], "host_preparation": m["host_preparation"],
                   "l2": "instances of up to several GB against 129 MB L2"},
        "clocks": m.pop("clocks"), "gpu_launches": m.pop("gpu_launches"),
        "e2e": {"value": m["solves_per_s"], "unit": "solves/s",
                "h2d_bytes_per_step": float(np.mean([prepared[r.rid][1].nbytes + prepared[r.rid][0].neigh.nbytes
                                                     + prepared[r.rid][0].types.nbytes for r in reqs])),
                "d2h_bytes_per_step": 96.0 * args.max_steps / args.check_every,
                "path": "per request: bclbm_create + first step on a host thread, bclbm_batch_attach, batched "
                        "steps, bclbm_batch_stats every check block, bclbm_batch_retire"},
        "roofline": {"bound": "hbm", "peak": peak, "unit": "GB/s", "peak_kind": peak_kind, "achieved": achieved,
                     "frac": achieved / peak, "traffic": None,
                     "note": "algorithmic bytes of all lattice updates over the whole serving run (wall clock)"},
    } | m
    print(json.dumps(line), flush=True)


# two-phase algorithmic bytes per fluid-node update: two population sets read and
# written, the neighbour table, the colour scalar read and written
BYTES_PER_UPDATE_RK = {"f64": 4 * 19 * 8 + 18 * 4 + 2 * 8, "f16": 4 * 19 * 2 + 18 * 4 + 2 * 4,
                       "bf16": 4 * 19 * 2 + 18 * 4 + 2 * 4, "f32": 4 * 19 * 4 + 18 * 4 + 2 * 4}


def run_twophase(args, world, rank):
    """--workload twophase: the Rothman-Keller step on a seeded sphere pack, FP64
    against shifted FP16 storage (time per step, saturation and phase-flux error)."""
    import torch
    import __graft_entry__ as ge
    bclbm = ge.load()
    L = bclbm.lbsolver
    if rank != 0:
        return
    t = time.time()
    geo, centres, phi = bclbm.geometry.sphere_pack((args.size,) * 3, radius=args.radius, porosity=args.porosity,
                                                   seed=args.seed)
    lat = L.Lattice.from_geometry(geo, "D3Q19", "xyz")
    rng = np.random.default_rng(args.seed + 1)
    red = rng.random(geo.shape) < args.saturation
    rho0 = np.where(geo == 1, red, 0.0)
    rho1 = np.where(geo == 1, ~red, 0.0).astype(np.float64)
    f0, rho = L.initiate_twophase(lat, lat.attribute(rho0), lat.attribute(rho1),
                                  lat.attribute(np.full(geo.shape, 0.5)))
    log(f"two-phase geometry {args.size}^3: porosity {phi:.4f}, fluid {lat.n_bulk}, nodes {lat.n_nodes} "
        f"({time.time() - t:.1f}s)")
    peak, peak_kind = peaks()
    cx = np.array([1, 0, 0, 1, 1, 1, 1, 0, 0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 0], dtype=np.float64)
    res = {}
    l0 = bclbm.native.launch_count()
    with ClockSampler(0) as clk:
        for prec in args.tp_precisions.split(","):
            # "f64": fixed point; "f64-fma": FMA contraction; "f64-exact": reference order;
            # "f16-lag" (any shifted format): one pass per step, BCLBM_FLAG_LAGGED_COLOUR
            base = prec.split("-")[0]
            with L.Solver(lat, f0, collision=L.RK, precision=base, tau=(1.0, 1.0), force=(args.gx, 0.0, 0.0),
                          sigma=args.sigma, beta=args.beta, rho_init=rho, fma64=prec.endswith("-fma"),
                          exact=prec.endswith("-exact"), lagged_colour=prec.endswith("-lag")) as s:
                s.step(args.warmup)
                s.sync()
                tm = s.step_timed(args.steps)
                done = args.warmup + args.steps
                t0 = time.time()
                if args.tp_steps > done:
                    s.step(args.tp_steps - done)
                st = s.reduce()
                t_acc = time.time() - t0
                f = s.download_f()
            F = f.reshape(-1, 2, 19)[lat.bulk]
            flux = [(F[:, k, :] * cx[None, :]).sum() for k in range(2)]
            mlups = lat.n_bulk * args.steps / (tm["total_ms"] * 1e-3) / 1e6
            kernel_ms = (tm["step_kernel_ms"] + tm["density_ms"]) / args.steps
            ach = lat.n_bulk * BYTES_PER_UPDATE_RK[base] / (kernel_ms * 1e-3) / 1e9
            fp = bclbm.native.footprint(lat, L.RK, L.PRECISION[base])
            res[prec] = {"footprint_bytes": fp, "mlups": mlups, "ms_per_step": tm["total_ms"] / args.steps,
                         "collide_ms": tm["step_kernel_ms"] /
                         args.steps, "density_ms": tm["density_ms"] / args.steps, "achieved_gbs": ach,
                         "frac": ach / peak, "bytes_per_update": BYTES_PER_UPDATE_RK[base],
                         "saturation": st["saturation"], "mass": st["mass"], "phase_flux_x": flux,
                         "steps_total": max(done, args.tp_steps), "seconds_after_timing": t_acc}
            log(f"{prec}: {mlups:.0f} MLUPS, S = {st['saturation']:.9f}, flux {flux}")
    launches = bclbm.native.launch_count() - l0
    ref_key = next((k for k in ("f64-exact", "f64", "f64-fma") if k in res), None)
    ref = res.get(ref_key) if ref_key else None
    errs = {}
    if ref:
        for prec, r in res.items():
            if prec == ref_key:
                continue
            errs[prec] = {"saturation_abs": abs(r["saturation"] - ref["saturation"]),
                          "phase_flux_rel": [abs(a - b) / abs(b) if b else None for a, b in
                                             zip(r["phase_flux_x"], ref["phase_flux_x"])]}
    head = res[args.tp_precisions.split(",")[0]]
    line = {
        "metric": METRIC, "value": head["mlups"], "unit": "MLUPS", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.tp_precisions.split(",")[0],
        "data": "synthetic: seeded periodic sphere pack and i.i.d. phase field (numpy default_rng), no dataset",
        "config": {"workload": f"D3Q19 Rothman-Keller two-phase, periodic {args.size}^3 sphere pack, radius "
                               f"{args.radius:g}, porosity {phi:.4f} (target {args.porosity:g}), fluid nodes red with "
                               f"p={args.saturation:g}, tau_r = tau_b = 1, A = {args.sigma:g}, beta = {args.beta:g}, "
                               f"neutral wetting, gx {args.gx:g}; {args.tp_steps} steps for the errors",
                   "fluid_nodes": lat.n_bulk, "lattice_nodes": lat.n_nodes,
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": head["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": head["frac"], "traffic": None, "peak_kind": peak_kind,
                     "kernel": "k_rk_density + k_rk_collide (both passes of a step)",
                     "bytes_per_update": head["bytes_per_update"], "units_per_launch": lat.n_bulk},
        "precisions": res, "errors_vs_f64": errs, "clocks": clk.summary(), "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def links_traffic(n_fluid):
    """DRAM bytes of one k_links_collide_fixed launch (the default FP64 step) from the
    committed ncu capture, scaled by the fluid nodes, or None."""
    f = REPO / "profiles" / "traffic.json"
    try:
        bpn = json.loads(f.read_text())["k_links_collide_d3q19_f64_fixed"]["bytes_per_node"]
        return int(bpn * n_fluid)
    except Exception:
        return None


def links_bytes(lat, tags, labels, sf=8):
    """Algorithmic bytes of one std_one_phase step: every fluid node reads its 19
    pulled populations, 18 table entries, its info word and force attribute and
    writes 19 populations; the labelled nodes are read once more by the mass pass
    (plus their list entry and the 1 - rho written); the pressure-boundary nodes
    read and write their velocity (and read its index)."""
    b = lat.bulk
    nlab = int(np.count_nonzero(labels[b] > 0))
    npress = int(np.count_nonzero((tags[b] >> 4) & 1))
    per = 2 * 19 * sf + 18 * 4 + 4 + 4
    return lat.n_bulk * per + nlab * (19 * sf + 18 * 4 + 4 + 4 + 8) + npress * (4 + 48), nlab, npress


def run_links(args, world, rank):
    """--workload links: the std_one_phase step (interior-domain mass sources and
    the solid / pressure / fluid-fluid link boundaries of the node tags) on a
    tagged sphere pack: FP64 storage with the fixed-point collision (the line's
    value), FP64 with FMA, the reference-order exact FP64 kernel and the shifted
    formats, against the oracle on the host cores."""
    import __graft_entry__ as ge
    bclbm = ge.load()
    L = bclbm.lbsolver
    if rank != 0:
        return
    t = time.time()
    mask, attrs = bclbm.geometry.tagged_pack((args.size,) * 3, args.radius, args.porosity, args.seed)
    lat = L.Lattice.from_geometry(mask, "D3Q19", "xy")
    tags, labels, fon = (lat.attribute(attrs[k]).astype(np.int32) for k in ("nodetags", "interior_domains", "force"))
    phi = float(mask[:, :, 1:-1].mean())
    log(f"tagged pack {args.size}^3: porosity {phi:.4f}, fluid {lat.n_bulk}, nodes {lat.n_nodes}, "
        f"{labels.max()} interior domains ({time.time() - t:.1f}s)")
    f0 = L.initiate_single(lat, np.ones(lat.n_nodes))
    force = (args.gx, 0.0, args.gx)
    peak, peak_kind = peaks()
    nbytes, nlab, npress = links_bytes(lat, tags, labels)
    res, fs = {}, {}
    l0 = bclbm.native.launch_count()
    with ClockSampler(0) as clk:
        for name, exact, prec in (("f64", False, "f64"), ("f64-fma", False, "f64"), ("f64-exact", True, "f64"),
                                  ("f32", False, "f32"), ("f16", False, "f16")):
            with L.Solver(lat, f0, collision=L.LINKS, precision=prec, tau=(args.tau, args.tau), force=force,
                          tags=tags, labels=labels, force_on=fon, exact=exact, fma64=(name == "f64-fma")) as s:
                tm = time_solver(s, args.steps, args.warmup)
                fs[name] = s.download_f()
                q = s.pressure_flux()
            mlups = lat.n_bulk * args.steps / (tm["total_ms"] * 1e-3) / 1e6
            nb_prec = links_bytes(lat, tags, labels, {"f64": 8, "f32": 4, "f16": 2}[prec])[0]
            ach = nb_prec / (tm["step_kernel_ms"] / args.steps * 1e-3) / 1e9
            res[name] = {"mlups": mlups, "ms_per_step": tm["total_ms"] / args.steps, "achieved_gbs": ach,
                         "frac": ach / peak, "bytes_per_step": nb_prec, "mass_flux": [float(v) for v in q]}
            log(f"{name}: {mlups:.0f} MLUPS, {ach:.0f} GB/s ({ach / peak:.3f}), flux {q}")
    launches = bclbm.native.launch_count() - l0
    ex = fs["f64-exact"].reshape(-1, 19)[lat.bulk]
    rel = {k: float(np.linalg.norm(v.reshape(-1, 19)[lat.bulk] - ex) / np.linalg.norm(ex)) for k, v in fs.items()
           if k != "f64-exact"}
    qex = res["f64-exact"]["mass_flux"][0]
    for k in res:
        res[k]["mass_flux_rel_err"] = abs(res[k]["mass_flux"][0] - qex) / abs(qex) if qex else None
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, str(REPO / "oracle"))
        import oracle
        n = max(24, args.size // 4)
        m2, a2 = bclbm.geometry.tagged_pack((n,) * 3, args.radius / 4 + 1, args.porosity, args.seed)
        l2 = L.Lattice.from_geometry(m2, "D3Q19", "xy")
        t2, lb2, fo2 = (l2.attribute(a2[k]).astype(np.int32) for k in ("nodetags", "interior_domains", "force"))
        g = oracle.OracleGrid(19, l2.neigh, l2.types, l2.bulk)
        nth = oracle.default_threads()
        steps2 = 2
        t0 = time.time()
        oracle.links_run(g, L.initiate_single(l2, np.ones(l2.n_nodes)), steps2, args.tau, force, t2, lb2, fo2,
                         nthreads=nth)
        dt = time.time() - t0
        steps2 = max(2, int(steps2 * min(args.cpu_seconds / max(dt, 1e-3), 5000)))
        t0 = time.time()
        oracle.links_run(g, L.initiate_single(l2, np.ones(l2.n_nodes)), steps2, args.tau, force, t2, lb2, fo2,
                         nthreads=nth)
        dt = time.time() - t0
        cpu = {"value": l2.n_bulk * steps2 / dt / 1e6, "unit": "MLUPS", "cores": nth, "kind": "port",
               "sample": f"oracle (C restatement of src/std_one_phase/main.cpp:470-575) on a {n}^3 tagged pack, "
                         f"{l2.n_bulk} fluid nodes, {steps2} steps, {dt:.1f} s"}
    head = res["f64"]
    line = {
        "metric": METRIC, "value": head["mlups"], "unit": "MLUPS", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded sphere pack with phase-2 blobs and node tags (numpy default_rng), no dataset",
        "config": {"workload": f"D3Q19 std_one_phase step, {args.size}^3 sphere pack radius {args.radius:g} periodic "
                               f"in x, y with pressure-ghost z faces, porosity {phi:.4f}, tau {args.tau:g}, "
                               f"force ({args.gx:g}, 0, {args.gx:g})",
                   "fluid_nodes": lat.n_bulk, "labelled_nodes": nlab, "pressure_nodes": npress,
                   "interior_domains": int(labels.max()), "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": head["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": head["frac"], "traffic": links_traffic(lat.n_bulk), "peak_kind": peak_kind,
                     "kernel": "k_links_mass + k_links_label_sum + k_links_collide (one step)",
                     "bytes_per_step": nbytes, "units_per_launch": lat.n_bulk},
        "variants": res, "rel_l2_f_vs_exact": rel, "cpu_baseline": cpu, "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def run_output(args, world, rank):
    """--workload output: the std_case loop with an output step every --write-every
    steps (download of the device moments into the fields the VTU writer reads,
    then the write), synchronous against asynchronous writes; the line's value
    is the MLUPS of the asynchronous loop including the writes."""
    import shutil
    import tempfile
    bclbm, lat, phi = build_workload(args.size, args.radius, args.porosity, args.seed)
    if rank != 0:
        return
    L = bclbm.lbsolver
    f0 = L.initiate_single(lat, np.ones(lat.n_nodes))
    rho = np.zeros((lat.n_nodes, 1))
    vel = np.zeros((lat.n_nodes, 1, 3))
    W, nw = args.write_every, args.writes
    root = Path(tempfile.mkdtemp(prefix="bclbm_vtu_"))
    res = {}
    l0 = bclbm.native.launch_count()
    try:
        with ClockSampler(0) as clk, L.Solver(lat, f0, tau=(args.tau, args.tau), force=(args.gx, 0, 0)) as s:
            s.step(args.warmup)
            s.sync()
            for mode in ("steps_only", "sync", "async", "writes_only"):
                d = root / mode
                d.mkdir()
                with bclbm.output.Output(lat, lat.bulk, d) as o:
                    o.add_file("lb_run")
                    o.add_scalar_variables(["rho"], [rho])
                    o.add_vector_variables(["vel"], [vel])
                    t0 = time.perf_counter()
                    for k in range(nw):
                        if mode != "writes_only":
                            s.step(W)
                        if mode == "steps_only":
                            s.sync()
                            continue
                        s.download_macros(rho.reshape(-1), vel.reshape(-1))
                        if mode == "async":
                            o.write_async(k)
                        else:
                            o.write(k)
                    if mode == "async":
                        o.wait()
                    s.sync()
                    res[mode] = time.perf_counter() - t0
                nbytes = sum(p.stat().st_size for p in d.rglob("*") if p.is_file())
                res[mode + "_bytes"] = nbytes
                shutil.rmtree(d, ignore_errors=True)
                log(f"{mode}: {res[mode]:.3f} s ({nbytes / 1e6:.0f} MB written)")
    finally:
        shutil.rmtree(root, ignore_errors=True)
    launches = bclbm.native.launch_count() - l0
    steps = W * nw
    mlups = {m: lat.n_bulk * steps / res[m] / 1e6 for m in ("steps_only", "sync", "async")}
    hidden = (res["sync"] - res["async"]) / max(res["writes_only"], 1e-9)
    line = {
        "metric": METRIC, "value": mlups["async"], "unit": "MLUPS", "n_gpus": 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": res["async"] / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded periodic sphere pack (numpy default_rng), no dataset",
        "config": {"workload": f"D3Q19 BGK periodic {args.size}^3 sphere pack, FP64 step, an output step (rho, vel "
                               f"VTU, Float64, binary) every {W} steps, {nw} writes",
                   "fluid_nodes": lat.n_bulk, "l2": "inputs larger than L2"},
        "seconds": {k: v for k, v in res.items() if not k.endswith("_bytes")},
        "vtu_bytes_per_write": res["sync_bytes"] // max(nw, 1), "mlups_by_mode": mlups,
        "write_time_hidden": hidden, "clocks": clk.summary(), "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--radius", type=float, default=10.0)
    ap.add_argument("--porosity", type=float, default=0.40)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--tau", type=float, default=0.8)
    ap.add_argument("--gx", type=float, default=1e-5)
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "f16", "bf16"],
                    help="storage of the headline run (f64 = plain FP64, the reference's precision)")
    ap.add_argument("--collision", default="bgk", choices=["bgk", "trt"])
    ap.add_argument("--exact", action="store_true", help="headline with the reference-order FP64 kernel")
    ap.add_argument("--fma64", action="store_true", help="headline with the native-FP64 FMA kernel")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--accuracy-steps", type=int, default=10000,
                    help="steps of the FP64 / FP32 / FP16 / BF16 permeability comparison (0: skip)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving sample of the pack workload line")
    ap.add_argument("--workload", default="pack", choices=["pack", "serving", "twophase", "links", "output"],
                    help="pack: the 256^3 sphere-pack time step; serving: the request loop; twophase: the "
                         "Rothman-Keller step (use --size 192 --radius 8 for the 192^3 case)")
    ap.add_argument("--tp-steps", type=int, default=20000, help="twophase: total steps of the accuracy run")
    ap.add_argument("--write-every", type=int, default=1000, help="output: steps between output steps")
    ap.add_argument("--writes", type=int, default=4, help="output: output steps")
    ap.add_argument("--tp-precisions", default="f64-exact,f16")
    ap.add_argument("--saturation", type=float, default=0.5)
    ap.add_argument("--sigma", type=float, default=0.01)
    ap.add_argument("--beta", type=float, default=0.99)
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--rates", default="0", help="comma-separated Poisson arrival rates (/s) of the serving runs")
    ap.add_argument("--size-min", type=int, default=32)
    ap.add_argument("--size-max", type=int, default=256)
    ap.add_argument("--check-every", type=int, default=500)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--max-steps", type=int, default=50000)
    ap.add_argument("--steps-per-graph", type=int, default=50)
    ap.add_argument("--serving-precision", default="f32",
                    help="storage format of the batched server, or a ladder such as f16>f32")
    ap.add_argument("--promote-tol", type=float, default=2e-5,
                    help="ladder: |dk/k| per check block at which a request moves to the next format")
    ap.add_argument("--baseline-precision", default="f64", choices=["f64", "f32", "f16", "bf16"])
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error(f"--warmup {args.warmup}: at least 3 untimed warm-up steps are required before the timed steps")
    world, rank = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        import __graft_entry__ as ge
        ge._load_build_module().build()
        if args.workload == "serving":
            run_serving(args, world, rank)
        elif args.workload == "twophase":
            run_twophase(args, world, rank)
        elif args.workload == "links":
            run_links(args, world, rank)
        elif args.workload == "output":
            run_output(args, world, rank)
        else:
            run_mine(args, world, rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
