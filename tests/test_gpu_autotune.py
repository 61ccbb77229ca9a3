"""The tile-shape autotuner of the FP64 grouped GEMM (imps_plan_autotune): it times every launch
shape of a stage once per process, caches the fastest under the stage's output-block histogram,
and leaves results exact (every shape computes the same products, only the summation order
differs: 1e-12 against the oracle) and the caller's buffers untouched."""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops
from oracle import imps_oracle as O
from tests import imps_testlib as T
from tests.test_gpu_parity import RTOL, _hac_setup, dev, host, relerr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["xxz_d512", "hubbard_d1024"])
def test_autotune_hac(cuda_ctx, name):
    model, dims0, params = T.workload_dims(name)
    p = T.hac_problem(model, dims0, seed=71, **params)
    B.autotune_clear()
    plan, lac = _hac_setup(cuda_ctx, p)
    x = p["rng"].standard_normal(lac.nelem)
    xin, out = dev(x), dev(np.full(lac.nelem, 7.0))
    ops.ApplyHAvec(plan, xin, out)
    before_in, before_out = host(xin).copy(), host(out).copy()
    assert plan.autotune(reps=3) >= 1
    # no caller buffer was read for timing or written
    assert np.array_equal(host(xin), before_in) and np.array_equal(host(out), before_out)
    tile, splits, key = plan.stage_shape(0)
    assert tile in (16, 32) and 1 <= splits <= 8
    ref = O.ApplyHAvec(x, O.mps_sizes(p["AC"]), p["EHL"], p["EHR"], p["HL"], p["HR"])
    out2 = dev(np.full(lac.nelem, np.nan))
    ops.ApplyHAvec(plan, xin, out2)
    assert relerr(host(out2), ref) < RTOL
    # a second plan with the same sector structure takes the cached shape without timing
    plan2, _ = _hac_setup(cuda_ctx, p)
    assert plan2.stage_shape(0) == (tile, splits, key)
    assert plan2.autotune(reps=3) == 0
    B.autotune_clear()
