"""bclbm_moments_static: the entry point for callers that cannot allocate.

A caller whose device memory belongs to its own allocator, or whose loop
cannot afford a cudaMalloc, holds the populations itself and asks for the FP64
moment sums without the library allocating anything.  This test allocates the
caller's device buffers itself (through torch), calls the entry point through
the C ABI, and checks its sums against bclbm_reduce on a handle holding the
same populations, within the tolerance the reduction tests use (rtol 1e-13),
on calls made back to back.  It also checks that a size above the stated
maximum is refused before anything runs on the GPU.
"""

import ctypes

import numpy as np
import pytest

import lbcases

pytestmark = pytest.mark.gpu


def device_soa(torch, case, f_ref, nfields, precision, rho_ref=1.0, scale=1.0):
    """The caller's copy of the populations in the library's device layout
    [nfields][Q][stride] and storage format, on the GPU."""
    rows = case.bulk_rows(f_ref, nfields)  # [n_bulk, nfields, Q]
    nb = rows.shape[0]
    stride = nb + 37  # any stride >= n_slots is allowed
    soa = np.zeros((nfields, case.nq, stride))
    if precision == "f64":
        soa[:, :, :nb] = rows.transpose(1, 2, 0)
        dev = torch.from_numpy(soa).cuda()
    else:  # f32: shifted, weight-normalised deviation (f - w rho_ref) / w * scale
        w = case.L.weights(case.nq)
        dev_rows = (rows[:, 0, :] - w[None, :] * rho_ref) / w[None, :] * scale
        soa[0, :, :nb] = dev_rows.T
        dev = torch.from_numpy(soa.astype(np.float32)).cuda()
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


def make_solver(case, run, precision):
    L = case.L
    f0, rho0 = case.init(run)
    if run["mode"] == "single":
        return L.Solver(case.lat, f0, collision=L.BGK, tau=(run["tau"], run["tau"]), force=case.force(run),
                        precision=precision)
    return L.Solver(case.lat, f0, collision=L.RK, tau=(run["tau0"], run["tau1"]), force=case.force(run),
                    sigma=run["sigma"], beta=run["beta"], rho_init=rho0, precision=precision)


def handle_sums(st):
    return np.array(st["mass"] + st["flux_fc"] + [st["max_abs_f"]])


def close(a, b):
    return np.allclose(a, b, rtol=1e-13, atol=1e-15)


CASES = [("pack_20", "bgk_500", "f64"), ("pack_20", "bgk_500", "f32"), ("pack_20", "rk_100", "f64")]


@pytest.mark.parametrize("name,tag,precision", CASES, ids=[f"{n}-{t}-{p}" for n, t, p in CASES])
def test_static_moments_match_handle_reduce(bclbm, gpu, name, tag, precision):
    torch = pytest.importorskip("torch")
    case = lbcases.Case(name, bclbm)
    run = case.runs[tag]
    nfields = 2 if run["mode"] == "twophase" else 1
    f0, _ = case.init(run)
    with make_solver(case, run, precision) as s:
        ref0 = handle_sums(s.reduce())  # initial state
        if precision == "f64":
            s.step(17)
            f17 = s.download_f(np.zeros(case.n_nodes * nfields * case.nq))
            ref17 = handle_sums(s.reduce())
    dev0, nb, stride = device_soa(torch, case, f0, nfields, precision)
    first = static_sums(bclbm, torch, case, dev0, nb, stride, nfields, precision)
    assert close(first, ref0), (first, ref0)
    if precision == "f64":
        dev17, nb, stride = device_soa(torch, case, f17, nfields, precision)
        second = static_sums(bclbm, torch, case, dev17, nb, stride, nfields, precision)
        assert close(second, ref17), (second, ref17)
    again = static_sums(bclbm, torch, case, dev0, nb, stride, nfields, precision)
    assert close(again, ref0) and np.array_equal(again, first)


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
