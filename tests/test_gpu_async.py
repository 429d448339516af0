"""bclbm_macros_begin / bclbm_macros_collect: the split download returns the
macros of the step at which it began, while later steps run behind it."""

import numpy as np
import pytest

import lbcases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,tag", [("pack_20", "bgk_500"), ("pack_20", "rk_100")])
@pytest.mark.parametrize("precision", ["f64", "f16"])
def test_split_download_equals_download_at_that_step(bclbm, gpu, name, tag, precision):
    case = lbcases.Case(name, bclbm)
    run = case.runs[tag]
    from test_gpu_parity import make_solver
    with make_solver(case, run, precision=precision) as a, make_solver(case, run, precision=precision) as b:
        a.step(37)
        a.macros_begin()
        a.step(50)  # queued behind the copies
        ra, va, ca = a.macros_collect()
        b.step(37)
        rb, vb, cb = b.download_macros()
        assert np.array_equal(ra, rb) and np.array_equal(va, vb)
        if ca is not None:
            assert np.array_equal(ca, cb)
        # the later steps ran: the macros now differ from those at step 37
        rc, vc, _ = a.download_macros()
        assert not np.array_equal(vc, vb)


def test_split_download_misuse_is_an_error(bclbm, gpu):
    case = lbcases.Case("pack_20", bclbm)
    from test_gpu_parity import make_solver
    with make_solver(case, case.runs["bgk_500"]) as s:
        with pytest.raises(bclbm.native.BclbmError):
            s.macros_collect()  # nothing pending
        with pytest.raises(bclbm.native.BclbmError):
            s.macros_begin()  # no step yet
        s.step(2)
        s.macros_begin()
        with pytest.raises(bclbm.native.BclbmError):
            s.macros_begin()  # one pending at a time
        s.macros_collect()
