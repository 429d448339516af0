"""bclbm_moments_static: the entry point for callers that cannot allocate.

A caller whose device memory belongs to its own allocator, or whose loop
cannot afford a cudaMalloc, holds the populations itself and asks for the FP64
moment sums without the library allocating anything.  This test allocates the
caller's device buffers itself (through torch), calls the entry point through
the C ABI, and checks its sums against bclbm_reduce on a handle holding the
same populations, within the tolerance the reduction tests use (rtol 1e-13),
on calls made back to back: D3Q19 and D2Q9, FP64 and every shifted storage
format (F16 with its default scale), one and two fields.  It also checks the
non-finite flag (max |f| is +Inf when a value is NaN or Inf) and that a size
above the stated maximum is refused before anything runs on the GPU.
"""

import ctypes

import numpy as np
import pytest

import lbcases

pytestmark = pytest.mark.gpu

# default store_scale of bclbm_create per shifted format (0 passed = this value)
DEFAULT_SCALE = {"f32": 1.0, "f16": 4096.0, "bf16": 1.0}


def stored_values(precision, shape, rng):
    """Random stored deviations that the storage format holds exactly and that
    bclbm_create's encoding of f = w (rho_ref + v / scale) gives back exactly."""
    if precision == "f16":
        return rng.integers(-2000, 2000, size=shape) / 16.0  # 11 significant bits at most
    if precision == "bf16":
        return rng.integers(-255, 256, size=shape) / 4096.0  # 8 significant bits at most
    return rng.integers(-3000, 3000, size=shape) / 65536.0   # f32


def shifted_init(case, precision, seed=7):
    """(f_init in reference layout, stored values [n_bulk, Q]) for one field."""
    w = case.L.weights(case.nq)
    nb = case.lat.bulk.size
    v = stored_values(precision, (nb, case.nq), np.random.default_rng(seed))
    f = np.zeros((case.n_nodes, case.nq))
    f[case.lat.bulk] = w[None, :] * (1.0 + v / DEFAULT_SCALE[precision])
    return f.reshape(-1), v


def device_soa(torch, case, rows, nfields, precision):
    """The caller's copy of the populations in the library's device layout
    [Q][stride][nfields], on the GPU: plain FP64 values of f (F64), or the
    stored values of a shifted format."""
    nb = rows.shape[0]
    stride = nb + 37  # any stride >= n_slots is allowed
    soa = np.zeros((case.nq, stride, nfields))
    soa[:, :nb, :] = rows.reshape(nb, nfields, case.nq).transpose(2, 0, 1)
    dtype = {"f64": torch.float64, "f32": torch.float32, "f16": torch.float16, "bf16": torch.bfloat16}[precision]
    dev = torch.from_numpy(soa).to(dtype).cuda()
    # the conversion to the storage type must be exact (the values were chosen so)
    assert np.array_equal(dev.double().cpu().numpy(), soa)
    return dev, nb, stride


def static_sums(bclbm, torch, case, dev, nb, stride, nfields, precision):
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    prec = bclbm.lbsolver.PRECISION[precision]
    rc = bclbm.native.lib().bclbm_moments_static(case.nq, prec, nfields, nb, stride, ctypes.c_void_p(dev.data_ptr()),
                                                 1.0, 0.0, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def make_solver(case, run, precision, f0=None):
    L = case.L
    finit, rho0 = case.init(run)
    if f0 is not None:
        finit = f0
    if run["mode"] == "single":
        return L.Solver(case.lat, finit, collision=L.BGK, tau=(run["tau"], run["tau"]), force=case.force(run),
                        precision=precision)
    return L.Solver(case.lat, finit, collision=L.RK, tau=(run["tau0"], run["tau1"]), force=case.force(run),
                    sigma=run["sigma"], beta=run["beta"], rho_init=rho0, precision=precision)


def handle_sums(st):
    return np.array(st["mass"] + st["flux_fc"] + [st["max_abs_f"]])


def close(a, b):
    return np.allclose(a, b, rtol=1e-13, atol=1e-15)


F64_CASES = [("pack_20", "bgk_500"), ("pack_20", "rk_100"), ("disc_40x32", "trt_300")]


@pytest.mark.parametrize("name,tag", F64_CASES, ids=[f"{n}-{t}" for n, t in F64_CASES])
def test_static_moments_match_handle_reduce_f64(bclbm, gpu, name, tag):
    """FP64 populations: the initial state and the state after 17 steps."""
    torch = pytest.importorskip("torch")
    case = lbcases.Case(name, bclbm)
    run = case.runs[tag]
    nfields = 2 if run["mode"] == "twophase" else 1
    f0, _ = case.init(run)
    with make_solver(case, run, "f64") as s:
        ref0 = handle_sums(s.reduce())  # initial state
        s.step(17)
        f17 = s.download_f(np.zeros(case.n_nodes * nfields * case.nq))
        ref17 = handle_sums(s.reduce())
    dev0, nb, stride = device_soa(torch, case, case.bulk_rows(f0, nfields), nfields, "f64")
    first = static_sums(bclbm, torch, case, dev0, nb, stride, nfields, "f64")
    assert close(first, ref0), (first, ref0)
    dev17, nb, stride = device_soa(torch, case, case.bulk_rows(f17, nfields), nfields, "f64")
    second = static_sums(bclbm, torch, case, dev17, nb, stride, nfields, "f64")
    assert close(second, ref17), (second, ref17)
    again = static_sums(bclbm, torch, case, dev0, nb, stride, nfields, "f64")
    assert close(again, ref0) and np.array_equal(again, first)


SHIFTED_CASES = [("pack_20", "bgk_500", p) for p in ("f32", "f16", "bf16")] + [("disc_40x32", "trt_300", "f16")]


@pytest.mark.parametrize("name,tag,precision", SHIFTED_CASES, ids=[f"{n}-{t}-{p}" for n, t, p in SHIFTED_CASES])
def test_static_moments_match_handle_reduce_shifted(bclbm, gpu, name, tag, precision):
    """Shifted storage with the default scale (store_scale 0): a handle created
    from f = w (1 + v / scale) stores v; the entry point reads the same v from
    the caller's array.  Two calls in a row, on two different arrays."""
    torch = pytest.importorskip("torch")
    case = lbcases.Case(name, bclbm)
    run = case.runs[tag]
    sums = []
    for seed in (7, 8):
        f0, v = shifted_init(case, precision, seed)
        with make_solver(case, run, precision, f0=f0) as s:
            ref = handle_sums(s.reduce())
        dev, nb, stride = device_soa(torch, case, v, 1, precision)
        got = static_sums(bclbm, torch, case, dev, nb, stride, 1, precision)
        assert close(got, ref), (seed, got, ref)
        sums.append(got)
    assert not np.array_equal(sums[0], sums[1])


def test_static_moments_flag_nonfinite(bclbm, gpu):
    """max |f| comes back +Inf when any population is NaN or Inf."""
    torch = pytest.importorskip("torch")
    case = lbcases.Case("pack_20", bclbm)
    f0, _ = case.init(case.runs["bgk_500"])
    rows = case.bulk_rows(f0, 1)
    for bad in (np.nan, np.inf, -np.inf):
        dev, nb, stride = device_soa(torch, case, rows, 1, "f64")
        dev[5, nb // 2, 0] = float(bad)
        got = static_sums(bclbm, torch, case, dev, nb, stride, 1, "f64")
        assert got[5] == np.inf, (bad, got)
    dev, nb, stride = device_soa(torch, case, rows, 1, "f64")
    got = static_sums(bclbm, torch, case, dev, nb, stride, 1, "f64")
    assert np.isfinite(got).all()


def test_static_moments_refuse_oversize(bclbm, gpu):
    torch = pytest.importorskip("torch")
    lib = bclbm.native.lib()
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    n = 8388608 + 1  # BCLBM_STATIC_MAX_SLOTS + 1
    rc = lib.bclbm_moments_static(19, 0, 1, n, n, ctypes.c_void_p(dummy.data_ptr()), 1.0, 0.0,
                                  ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -1
    assert float(out.abs().sum().cpu()) == 0.0
