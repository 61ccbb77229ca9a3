"""Tensor-core (tcgen05) split-BF16 engine: the same planner stages executed with three-way
BF16 splitting and FP32 accumulation must agree with the FP64 engine to 1e-5 relative
(max-norm of the difference over max-norm of the result; the split keeps ~24 significant
bits per operand, FP32 accumulation over K <= ~400 terms dominates: measured ~2e-6)."""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import _native as N
from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops
from oracle import imps_oracle as O
from tests import imps_testlib as T
from tests.test_gpu_parity import SMALL, _hac_setup, dev, host, relerr

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-5


@pytest.mark.parametrize("model,dims0", SMALL + [("xxz", "xxz_d512"), ("fhub", "hubbard_d1024")])
def test_hac_bf16x6_vs_fp64(cuda_ctx, model, dims0):
    params = {}
    if isinstance(dims0, str):
        model, dims0, params = T.workload_dims(dims0)
    p = T.hac_problem(model, dims0, seed=41, **params)
    plan, lac = _hac_setup(cuda_ctx, p)
    x = dev(p["rng"].standard_normal(lac.nelem))
    ref = dev(np.zeros(lac.nelem))
    ops.ApplyHAvec(plan, x, ref)
    plan.set_precision(N.PREC_BF16X6)
    out = dev(np.full(lac.nelem, np.nan))
    ops.ApplyHAvec(plan, x, out)
    r, o = host(ref), host(out)
    assert np.isfinite(o).all()
    assert relerr(o, r) < TOL_MIXED
    # second apply reuses the cached operator packs
    out2 = dev(np.zeros(lac.nelem))
    ops.ApplyHAvec(plan, x, out2)
    assert np.array_equal(host(out2), o)
    plan.set_precision(N.PREC_FP64)


@pytest.mark.parametrize("direction", [0, 1])
def test_tm_bf16x6_vs_fp64(cuda_ctx, direction):
    model, dims0, params = T.workload_dims("xxz_d256")
    st = T.random_state(model, dims0, seed=43, **params)
    AL, dv, rng = st["AL"], st["dimvec"], st["rng"]
    l0, l1 = B.Layout(T.mps_blocks(AL[0]), 1), B.Layout(T.mps_blocks(AL[1]), 1)
    bond = B.Layout.blockdiag(dv[0])
    plan = B.plan_tm(cuda_ctx, [l0, l1], direction, bond, bond)
    plan.bind(2, dev(O.mps_vec(AL[0])))
    plan.bind(3, dev(O.mps_vec(AL[1])))
    x = dev(O.bd_vec(T.rand_bd(dv[0], rng, sym=False)))
    ref, out = dev(np.zeros(bond.nelem)), dev(np.zeros(bond.nelem))
    ops.ApplyTM(plan, x, ref)
    plan.set_precision(N.PREC_BF16X6)
    ops.ApplyTM(plan, x, out)
    assert relerr(host(out), host(ref)) < TOL_MIXED


def test_hc_bf16x6_vs_fp64(cuda_ctx):
    st = T.random_state("fhub", SMALL[1][1], seed=47)
    d, AL, AR, C, rng = st["d"], st["AL"], st["AR"], st["C"], st["rng"]
    Cd = {q: m.shape[0] for q, m in C[1].items()}
    lc = B.Layout(T.bd_blocks(C[1]), 2)
    plan = B.plan_hc(cuda_ctx, lc, lc, lc, B.Layout(T.mps_blocks(AL[1]), 2), B.Layout(T.mps_blocks(AR[0]), 2),
                     d, st["hnnz"])
    for s, v in ((2, O.bd_vec(T.rand_bd(Cd, rng))), (3, O.bd_vec(T.rand_bd(Cd, rng))), (4, O.mps_vec(AL[1])),
                 (5, O.mps_vec(AR[0]))):
        plan.bind(s, dev(v))
    plan.prepare()
    x = dev(rng.standard_normal(lc.nelem))
    ref, out = dev(np.zeros(lc.nelem)), dev(np.zeros(lc.nelem))
    ops.ApplyHCvec(plan, x, ref)
    plan.set_precision(N.PREC_BF16X6)
    plan.prepare()
    ops.ApplyHCvec(plan, x, out)
    assert relerr(host(out), host(ref)) < TOL_MIXED
