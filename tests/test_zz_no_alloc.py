"""The transfer-matrix apply that allocates no device memory (imps_tm_apply_noalloc).

It exists for callers that cannot call cudaMalloc when they apply the transfer matrix (GPU
memory reserved up front by another allocator, or a latency-critical loop that must not pay
cudaMalloc's implicit synchronisation).  Its result must equal the regular plan-based entry
point (imps_plan_tm + imps_tm_apply) and the oracle's ApplyTMLeft / ApplyTMRight to the FP64
tolerance of the other parity tests, on two calls in a row (the second call reuses the static
scratch and the task tables left behind by the first).
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from imps_cpp_tools_gb300 import _native as N
from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops
from oracle import imps_oracle as O
from tests import imps_testlib as T

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def _dev(x):
    import torch
    return torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def _bd_dims(lay):
    return {qi: np.zeros((r, c)) for (_, qi, _, r, c) in lay.blocks}


def _relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("model,dims0", [
    ("xxz", {(-4,): 1, (-2,): 3, (0,): 5, (2,): 3, (4,): 1}),
    ("fhub", {(0, 0): 4, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2, (2, 0): 1, (0, 2): 1}),
    ("xxz", "xxz_d512"),
])
@pytest.mark.parametrize("direction", [0, 1])
def test_noalloc_matches_plan_path(cuda_ctx, model, dims0, direction):
    import torch
    params = {}
    if isinstance(dims0, str):
        model, dims0, params = T.workload_dims(dims0)
    st = T.random_state(model, dims0, seed=53, **params)
    A, dv, rng = st["AL"][0], st["dimvec"], st["rng"]
    ns = len(st["I2K"][0])
    la = B.Layout(T.mps_blocks(A), ns)
    lin = B.Layout.blockdiag(dv[0] if direction == 0 else dv[1])
    lout = B.Layout.blockdiag(dv[1] if direction == 0 else dv[0])
    ref_plan = B.plan_tm(cuda_ctx, [la], direction, lin, lout)
    dA = _dev(O.mps_vec(A))
    ref_plan.bind(2, dA)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # two calls in a row share the static scratch
        X = _dev(rng.standard_normal(lin.nelem))
        ref = _dev(np.zeros(lout.nelem))
        ops.ApplyTM(ref_plan, X, ref)
        Y = _dev(np.full(lout.nelem, np.nan))  # every element must be written
        st_ = N.load().imps_tm_apply_noalloc(la.handle, lin.handle, lout.handle, direction, C.c_void_p(dA.data_ptr()),
                                             C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), stream)
        assert st_ == 0, N.STATUS.get(st_)
        torch.cuda.synchronize()
        y, r = Y.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(y).all()
        assert _relerr(y, r) < RTOL, (call, _relerr(y, r))
        # and the oracle's ApplyTMLeft / ApplyTMRight (TMBlockFunctions.hpp:33-84, 155-205)
        xin = O.bd_from_vec(X.cpu().numpy(), O.bd_sizes(_bd_dims(lin)))
        want = O.bd_vec((O.ApplyTMLeft if direction == 0 else O.ApplyTMRight)(A, xin))
        assert _relerr(y, want) < RTOL, (call, _relerr(y, want))


def test_noalloc_rejects_oversized(cuda_ctx):
    """A tensor larger than the fixed scratch is refused with IMPS_ERR_TOO_LARGE."""
    import torch
    big = {(q,): 400 for q in range(-3, 4)}  # 2 * 7 * 400^2 > 1,048,576 elements
    I2K = [(1,), (-1,)]
    b1 = {(q + 1,): m for (q,), m in big.items()}
    la = B.Layout.mps(I2K, big, b1)
    assert la.nelem > (1 << 20)
    lin, lout = B.Layout.blockdiag(big), B.Layout.blockdiag(b1)
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(d.data_ptr())
    st_ = N.load().imps_tm_apply_noalloc(la.handle, lin.handle, lout.handle, 0, p, p, p,
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st_ == -9
