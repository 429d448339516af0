"""Serving loop: continuous batching of porous-media permeability solves on one GPU.

A request is one single-phase D3Q19 permeability solve: a periodic sphere pack
(seed, cube side, sphere radius, porosity), a relaxation time and a body force.
Its time loop is the reference's std_case loop (src/std_case/main.cpp:110-145)
over its own lattice, with permeability k = nu * sum(rho u_x) / (V * g_x)
from the FP64 flux reduction, run until k changes by less than ``tol``
(relative) over ``check_every`` steps or until ``max_steps``.

``Server.run`` serves a list of requests that arrive over time:

* host preparation (geometry and node tables) of each request starts when it
  arrives, on a pool of host threads;
* prepared requests are admitted in arrival order into a ``Batch`` (the
  C ABI's bclbm_batch_*) while the HBM budget and slot count allow;
* all admitted instances advance together, ``check_every`` steps at a time,
  through one persistent kernel over their concatenated node lists, replayed
  from a captured CUDA graph;
* after each block the FP64 sums of every instance give its permeability;
  converged instances are retired and their HBM is free for the next request;
* the storage format is FP32-shifted by default.  FP16 rounding leaves k a
  noise floor of 1e-6..1e-5 per 500-step block, above the 1e-6 stopping
  tolerance, so an FP16 solve stops late or not at all; a precision ladder
  ("f16>f32") runs a request in FP16 while its flow develops and moves it to
  FP32 once k has settled to within ``promote_tol`` per block.

``Server.run_sequential`` serves the same requests one at a time through the
single-instance ``Solver`` (the baseline).  Both report per-request latency
(arrival to result), p50/p99 and solves/s.
"""

from __future__ import annotations

import concurrent.futures as cf
import ctypes
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import geometry as _geometry
from . import lbsolver as _lb
from . import native as _native

BUDGET = -7
NONFINITE = -6


@dataclass
class Request:
    rid: int
    seed: int
    size: int
    radius: float
    porosity: float
    tau: float
    gx: float = 1e-5
    arrival: float = 0.0  # seconds after the start of the run
    cancel_at: float | None = None  # seconds after the start: withdrawn by then


@dataclass
class Result:
    rid: int
    permeability: float
    steps: int
    converged: bool
    arrival: float
    admitted: float
    finished: float
    n_fluid: int
    history: list = field(default_factory=list)
    status: str = "converged"  # converged | capped | nonfinite | cancelled | rejected

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def sample_requests(n: int, rate: float, seed: int = 7, size_range=(32, 256), radius_range=(4.0, 12.0),
                    porosity_range=(0.30, 0.50), tau_range=(0.6, 1.2), gx: float = 1e-5):
    """n requests with Poisson arrivals at ``rate`` per second (rate <= 0: all at t=0),
    cube side log-uniform in size_range, radius, porosity and tau uniform."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        if rate > 0:
            t += rng.exponential(1.0 / rate)
        size = int(round(math.exp(rng.uniform(math.log(size_range[0]), math.log(size_range[1])))))
        out.append(Request(rid=i, seed=int(rng.integers(1, 2**31 - 1)), size=size,
                           radius=float(rng.uniform(*radius_range)), porosity=float(rng.uniform(*porosity_range)),
                           tau=float(rng.uniform(*tau_range)), gx=gx, arrival=t if rate > 0 else 0.0))
    return out


def prepare(req: Request):
    """Host set-up of one request: geometry, node tables and the initial populations."""
    geo, _, _ = _geometry.sphere_pack((req.size,) * 3, radius=req.radius, porosity=req.porosity, seed=req.seed)
    lat = _lb.Lattice.from_geometry(geo, "D3Q19", "xyz")
    f0 = _lb.initiate_single(lat, np.ones(lat.n_nodes))
    return lat, f0


def permeability(momentum_x: float, req: Request) -> float:
    nu = (req.tau - 0.5) / 3.0
    return nu * momentum_x / (req.size ** 3 * req.gx)


class Batch:
    """Many single-phase instances stepped together (bclbm_batch_* of include/bclbm.h)."""

    def __init__(self, lattice_q: int = 19, collision: int = _lb.BGK, precision=_lb.F16, fma64: bool = False,
                 max_instances: int = 256, hbm_budget: int | None = None, steps_per_graph: int = 50):
        if isinstance(precision, str):
            precision = _lb.PRECISION[precision]
        if hbm_budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(free * 0.8)
        self.precision = precision
        self.collision = collision
        self.flags = _lb.FLAG_FP64_FMA if fma64 else 0
        self.budget = int(hbm_budget)
        self.max_instances = int(max_instances)
        L = _native.lib()
        self._b = ctypes.c_void_p()
        _native.check(L.bclbm_batch_create(lattice_q, collision, precision, self.flags, self.max_instances,
                                           self.budget, steps_per_graph, ctypes.byref(self._b)))
        self._lat = {}

    def _check(self, rc):
        _native.check(rc, batch=self._b)

    def footprint(self, lat) -> int:
        return _native.footprint(lat, self.collision, self.precision, self.flags)

    def admit(self, lat, f_init, tau, force, first_steps: int = 1):
        """Admits one instance (taking its first ``first_steps`` steps); returns its id,
        or None when the budget or slots are full."""
        F = np.zeros(3)
        F[:len(force)] = force
        f_init = np.ascontiguousarray(f_init, dtype=np.float64)
        d = _native.make_desc(lat, f_init, self.collision, self.precision, self.flags,
                              (float(tau[0]), float(tau[-1])), F, 0.0, 0.0, 0, 0.0, 1.0, 0.0, None)
        i = ctypes.c_int32(-1)
        rc = _native.lib().bclbm_batch_admit_steps(self._b, ctypes.byref(d), int(first_steps), ctypes.byref(i))
        if rc == BUDGET:
            return None
        self._check(rc)
        self._lat[i.value] = lat
        return i.value

    def attach(self, solver):
        """Admits a Solver created elsewhere (it must have taken >= 1 step); the batch
        takes its handle over.  Returns the id, or None when the budget or slots are full."""
        i = ctypes.c_int32(-1)
        rc = _native.lib().bclbm_batch_attach(self._b, solver._h, ctypes.byref(i))
        if rc == BUDGET:
            return None
        self._check(rc)
        solver._h = None  # owned by the batch from here on
        self._lat[i.value] = solver.lat
        return i.value

    def retire(self, iid: int):
        self._check(_native.lib().bclbm_batch_retire(self._b, int(iid)))
        self._lat.pop(iid, None)

    def step(self, nsteps: int):
        self._check(_native.lib().bclbm_batch_step(self._b, int(nsteps)))

    def stats(self, ids) -> list:
        """Sums of each instance; an instance with NaN/Inf populations (or outside the
        fixed-point range) has nonfinite set, the others are unaffected."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        out = (_native.Stats * max(1, len(ids)))()
        rc = _native.lib().bclbm_batch_stats(self._b, len(ids), _native.dp(ids), out)
        if rc != NONFINITE:
            self._check(rc)
        return [_native.stats_dict(out[j]) for j in range(len(ids))]

    def download_f(self, iid: int):
        lat = self._lat[iid]
        f = np.zeros(lat.n_nodes * lat.nq)
        self._check(_native.lib().bclbm_batch_download_f(self._b, int(iid), _native.dp(f)))
        return f

    def info(self) -> dict:
        used, n, steps = ctypes.c_size_t(), ctypes.c_int32(), ctypes.c_int64()
        self._check(_native.lib().bclbm_batch_info(self._b, ctypes.byref(used), ctypes.byref(n), ctypes.byref(steps)))
        return {"used_bytes": int(used.value), "active": int(n.value), "steps": int(steps.value)}

    def sync(self):
        self._check(_native.lib().bclbm_batch_sync(self._b))

    def close(self):
        if getattr(self, "_b", None):
            _native.lib().bclbm_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _percentile(x, p):
    return float(np.percentile(np.asarray(x, dtype=np.float64), p)) if len(x) else float("nan")


def summarize(results, t_start: float, t_end: float) -> dict:
    lat = [r.latency for r in results]
    span = t_end - t_start
    return {"solves": len(results), "seconds": span, "solves_per_s": len(results) / span if span > 0 else 0.0,
            "p50_s": _percentile(lat, 50), "p99_s": _percentile(lat, 99),
            "converged": int(sum(r.converged for r in results)),
            "lattice_updates": int(sum(r.n_fluid * r.steps for r in results))}


class Server:
    """Continuous-batching server for permeability requests on one GPU."""

    def __init__(self, precision="f32", max_instances: int = 256, hbm_budget: int | None = None,
                 check_every: int = 500, tol: float = 1e-6, max_steps: int = 50000, steps_per_graph: int = 50,
                 prep_workers: int = 4, fma64: bool = False, promote_tol: float = 1e-4):
        self.precision = precision
        self.stages = [p.strip() for p in precision.split(">")]
        self.promote_tol = float(promote_tol)
        self.max_instances = max_instances
        self.hbm_budget = hbm_budget
        self.check_every = int(check_every)
        self.tol = float(tol)
        self.max_steps = int(max_steps)
        self.steps_per_graph = int(steps_per_graph)
        self.prep_workers = int(prep_workers)
        self.fma64 = fma64
        self.counters = {}

    def _done(self, k_prev, k, steps) -> tuple:
        if k_prev is not None and k != 0.0 and abs(k - k_prev) / abs(k) < self.tol:
            return True, True
        return steps >= self.max_steps, False

    def _create(self, stage: int, lat, f_init, r: Request, first_steps: int):
        """Host thread: a single-instance handle in the stage's format, stepped
        first_steps times on its own stream (overlaps the running batch)."""
        s = _lb.Solver(lat, f_init, tau=(r.tau, r.tau), force=(r.gx, 0.0, 0.0), precision=self.stages[stage],
                       fma64=self.fma64)
        s.step(first_steps)
        s.sync()
        return s

    def run(self, requests, prepared=None) -> dict:
        """Serves ``requests`` with continuous batching; returns the report.
        ``prepared`` optionally maps rid -> (lattice, f0) built beforehand.

        Instances are created (upload and first step) on host threads while the
        batch runs, and attached between blocks.  With a precision ladder such
        as "f16>f32", an instance starts in the first storage format; once its
        permeability changes by less than ``promote_tol`` over a block, its
        populations (the reference f after the last step) move into the next
        format, where the convergence test runs afresh."""
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        by_id = {r.rid: r for r in reqs}
        results = []
        cnt = {"admitted": 0, "retired": 0, "promoted": 0, "refused_budget": 0, "rejected_too_large": 0,
               "cancelled": 0, "nonfinite": 0, "blocks": 0, "peak_active": 0, "peak_bytes": 0}
        # seconds of the loop in: launching steps + waiting for the statistics (the GPU's
        # share), attaching, retiring, and waiting with nothing admitted
        tm = {"step_and_stats_s": 0.0, "attach_s": 0.0, "retire_s": 0.0, "idle_s": 0.0}
        prep_pool = cf.ThreadPoolExecutor(max_workers=self.prep_workers)
        make_pool = cf.ThreadPoolExecutor(max_workers=2)
        budget = self.hbm_budget
        if budget is None:
            import torch
            budget = int(torch.cuda.mem_get_info()[0] * 0.8)
        batches = [Batch(precision=p, max_instances=self.max_instances, hbm_budget=budget,
                         steps_per_graph=self.steps_per_graph, fma64=self.fma64) for p in self.stages]
        creating = []  # [stage, future, need, record]
        try:
            pending = deque(reqs)
            preps = deque()  # (rid, future) in arrival order
            ready = deque()  # (rid, lattice, f0)
            active = {}  # (stage, iid) -> record
            t0 = time.perf_counter()
            clock = lambda: time.perf_counter() - t0  # noqa: E731

            def used():
                return sum(b.info()["used_bytes"] for b in batches)

            def committed():
                return used() + sum(c[2] for c in creating)

            fp_cache = {}

            def footprint(st, rid, lat):
                # bclbm_footprint plans the whole lattice: once per request and format
                if (st, rid) not in fp_cache:
                    fp_cache[(st, rid)] = batches[st].footprint(lat)
                return fp_cache[(st, rid)]

            def in_stage(st):
                return sum(1 for k in active if k[0] == st) + sum(1 for c in creating if c[0] == st)

            while len(results) < len(reqs):
                now = clock()
                while pending and pending[0].arrival <= now:
                    r = pending.popleft()
                    if prepared is not None and r.rid in prepared:
                        preps.append((r.rid, None))
                    else:
                        preps.append((r.rid, prep_pool.submit(prepare, r)))
                while preps and (preps[0][1] is None or preps[0][1].done()):
                    rid, fut = preps.popleft()
                    lat, f0 = prepared[rid] if fut is None else fut.result()
                    ready.append((rid, lat, f0))
                # admission by HBM footprint, in arrival order
                while ready:
                    rid, lat, f0 = ready[0]
                    r = by_id[rid]
                    if max(footprint(j, rid, lat) for j in range(len(batches))) > budget:
                        ready.popleft()
                        cnt["rejected_too_large"] += 1
                        results.append(Result(rid, float("nan"), 0, False, r.arrival, clock(), clock(), lat.n_bulk,
                                              status="rejected"))
                        continue
                    if r.cancel_at is not None and clock() >= r.cancel_at:
                        ready.popleft()
                        cnt["cancelled"] += 1
                        results.append(Result(rid, float("nan"), 0, False, r.arrival, clock(), clock(), lat.n_bulk,
                                              status="cancelled"))
                        continue
                    need = footprint(0, rid, lat)
                    if committed() + need > budget or in_stage(0) >= self.max_instances:
                        cnt["refused_budget"] += 1
                        break
                    ready.popleft()
                    rec = {"rid": rid, "k": None, "admitted": clock(), "n": lat.n_bulk, "hist": [], "lat": lat,
                           "offset": 0}
                    creating.append([0, make_pool.submit(self._create, 0, lat, f0, r, 1), need, rec])
                # attach the instances whose set-up has finished
                t_a = time.perf_counter()
                for c in [c for c in creating if c[1].done()]:
                    st, fut, need, rec = c
                    iid = batches[st].attach(fut.result())
                    if iid is None:
                        raise RuntimeError("attach refused an instance whose footprint was reserved")
                    creating.remove(c)
                    active[(st, iid)] = rec
                    if st == 0:
                        cnt["admitted"] += 1
                tm["attach_s"] += time.perf_counter() - t_a
                if not active:
                    t_i = time.perf_counter()
                    if creating:
                        cf.wait([c[1] for c in creating], timeout=0.05, return_when=cf.FIRST_COMPLETED)
                    else:
                        time.sleep(0.0005)
                    tm["idle_s"] += time.perf_counter() - t_i
                    continue
                cnt["peak_active"] = max(cnt["peak_active"], len(active))
                cnt["peak_bytes"] = max(cnt["peak_bytes"], used())
                live = sorted({st for st, _ in active})
                t_s = time.perf_counter()
                for st in live:
                    batches[st].step(self.check_every)
                cnt["blocks"] += 1
                all_stats = {}
                for st in live:
                    keys = sorted(k for k in active if k[0] == st)
                    all_stats[st] = (keys, batches[st].stats([k[1] for k in keys]))
                tm["step_and_stats_s"] += time.perf_counter() - t_s
                for st in live:
                    keys, stats = all_stats[st]
                    now = clock()
                    for key, sd in zip(keys, stats):
                        a = active[key]
                        r = by_id[a["rid"]]
                        steps = a["offset"] + int(sd["steps_done"])
                        stop = None
                        if sd["nonfinite"]:
                            stop, k = "nonfinite", float("nan")
                            cnt["nonfinite"] += 1
                        elif r.cancel_at is not None and now >= r.cancel_at:
                            stop, k = "cancelled", float("nan")
                            cnt["cancelled"] += 1
                        if stop:
                            batches[st].retire(key[1])
                            results.append(Result(a["rid"], k, steps, False, r.arrival, a["admitted"], now, a["n"],
                                                  a["hist"], status=stop))
                            del active[key]
                            continue
                        k = permeability(sd["momentum"][0], r)
                        a["hist"].append(k)
                        if st < len(batches) - 1:
                            # an earlier format never finishes by convergence: it
                            # hands over once k settles to within promote_tol
                            done, conv = steps >= self.max_steps, False
                            if not done and a["k"] is not None and k != 0.0 \
                                    and abs(k - a["k"]) / abs(k) < self.promote_tol:
                                lat = a["lat"]
                                need = footprint(st + 1, a["rid"], lat)
                                if committed() - footprint(st, a["rid"], lat) + need <= budget:
                                    f = batches[st].download_f(key[1])
                                    batches[st].retire(key[1])
                                    del active[key]
                                    # two first steps keep the parity of the step count at the
                                    # checks: the flux of a pack can differ between odd and even
                                    # steps (a period-2 mode of the step), by 1e-3 of k in small packs
                                    a.update(k=None, offset=steps)
                                    creating.append([st + 1, make_pool.submit(self._create, st + 1, lat, f, r, 2),
                                                     need, a])
                                    cnt["promoted"] += 1
                                    continue
                        else:
                            done, conv = self._done(a["k"], k, steps)
                        a["k"] = k
                        if done:
                            t_r = time.perf_counter()
                            batches[st].retire(key[1])
                            tm["retire_s"] += time.perf_counter() - t_r
                            cnt["retired"] += 1
                            results.append(Result(a["rid"], k, steps, conv, r.arrival, a["admitted"], now, a["n"],
                                                  a["hist"], status="converged" if conv else "capped"))
                            del active[key]
            t_end = clock()
        finally:
            for c in creating:
                try:
                    c[1].result().close()
                except Exception:
                    pass
            for b in batches:
                b.close()
            prep_pool.shutdown(wait=True)
            make_pool.shutdown(wait=True)
        results.sort(key=lambda x: x.rid)
        rep = summarize(results, 0.0, t_end)
        rep["counters"] = cnt | {k: round(v, 4) for k, v in tm.items()}
        rep["results"] = results
        return rep

    def run_sequential(self, requests, precision="f64", prepared=None) -> dict:
        """The same requests one at a time through the single-instance Solver
        (host preparation still overlaps on the thread pool)."""
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        results = []
        pool = cf.ThreadPoolExecutor(max_workers=self.prep_workers)
        futs = {}
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731
        pending = deque(reqs)

        def submit_arrived():
            now = clock()
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                futs[r.rid] = None if (prepared is not None and r.rid in prepared) else pool.submit(prepare, r)

        for r in reqs:
            while r.rid not in futs:
                submit_arrived()
                if r.rid not in futs:
                    time.sleep(0.0005)
            fut = futs.pop(r.rid)
            lat, f0 = prepared[r.rid] if fut is None else fut.result()
            t_adm = clock()
            hist = []
            status = None
            with _lb.Solver(lat, f0, tau=(r.tau, r.tau), force=(r.gx, 0.0, 0.0), precision=precision,
                            fma64=self.fma64) as s:
                s.step(1)
                steps, k_prev = 1, None
                while True:
                    if r.cancel_at is not None and clock() >= r.cancel_at:
                        status, k, conv = "cancelled", float("nan"), False
                        break
                    s.step(self.check_every)
                    submit_arrived()
                    steps += self.check_every
                    try:
                        st = s.reduce()
                    except _native.BclbmError as e:
                        if getattr(e, "status", 0) != NONFINITE:
                            raise
                        status, k, conv = "nonfinite", float("nan"), False
                        break
                    k = permeability(st["momentum"][0], r)
                    hist.append(k)
                    done, conv = self._done(k_prev, k, steps)
                    k_prev = k
                    if done:
                        break
            results.append(Result(r.rid, k, steps, conv, r.arrival, t_adm, clock(), lat.n_bulk, hist,
                                  status=status or ("converged" if conv else "capped")))
        t_end = clock()
        pool.shutdown(wait=True)
        results.sort(key=lambda x: x.rid)
        rep = summarize(results, 0.0, t_end)
        rep["results"] = results
        return rep
