"""GPU parity of the hot-path kernels against the CPU oracle, through the C ABI.

Tolerance: FP64 kernels agree with the oracle to 1e-12 relative (max-norm of the difference
over max-norm of the reference vector) -- the only differences are summation order."""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops
from oracle import imps_oracle as O
from tests import imps_testlib as T

pytestmark = pytest.mark.gpu
RTOL = 1e-12

SMALL = [("xxz", {(-4,): 1, (-2,): 3, (0,): 5, (2,): 3, (4,): 1}),
         ("fhub", {(0, 0): 4, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2, (2, 0): 1, (0, 2): 1})]


def dev(x):
    import torch
    return torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def relerr(got, ref):
    return float(np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300))


def _hac_setup(ctx, p):
    d = p["d"]
    ns = len(p["I2K"][0])
    lac = B.Layout(T.mps_blocks(p["AC"]), ns)
    lel, ler = B.Layout(T.bd_blocks(p["EHL"]), ns), B.Layout(T.bd_blocks(p["EHR"]), ns)
    lhl, lhr = B.Layout(T.redop_blocks(p["HL"], d), ns), B.Layout(T.redop_blocks(p["HR"], d), ns)
    plan = B.plan_hac(ctx, lac, lel, ler, lhl, lhr, d)
    plan.bind(2, dev(O.bd_vec(p["EHL"])))
    plan.bind(3, dev(O.bd_vec(p["EHR"])))
    plan.bind(4, dev(T.redop_vec(p["HL"], d)))
    plan.bind(5, dev(T.redop_vec(p["HR"], d)))
    return plan, lac


@pytest.mark.parametrize("model,dims0", SMALL + [("xxz", "xxz_d64")])
def test_hac_apply(cuda_ctx, model, dims0):
    if isinstance(dims0, str):
        model, dims0, _ = T.workload_dims(dims0)
    p = T.hac_problem(model, dims0, seed=21)
    plan, lac = _hac_setup(cuda_ctx, p)
    x = p["rng"].standard_normal(lac.nelem)
    ref = O.ApplyHAvec(x, O.mps_sizes(p["AC"]), p["EHL"], p["EHR"], p["HL"], p["HR"])
    out = dev(np.full(lac.nelem, np.nan))  # out must be fully overwritten (reference memset)
    ops.ApplyHAvec(plan, dev(x), out)
    assert relerr(host(out), ref) < RTOL


@pytest.mark.parametrize("name", ["xxz_d512", "hubbard_d1024"])
def test_hac_apply_full_size(cuda_ctx, name):
    model, dims0, params = T.workload_dims(name)
    p = T.hac_problem(model, dims0, seed=3, **params)
    plan, lac = _hac_setup(cuda_ctx, p)
    x = p["rng"].standard_normal(lac.nelem)
    ref = O.ApplyHAvec(x, O.mps_sizes(p["AC"]), p["EHL"], p["EHR"], p["HL"], p["HR"])
    out = dev(np.zeros(lac.nelem))
    ops.ApplyHAvec(plan, dev(x), out)
    assert relerr(host(out), ref) < RTOL
    # linearity at full size: H(a x + b y) = a H x + b H y
    y = p["rng"].standard_normal(lac.nelem)
    o2, o3 = dev(np.zeros(lac.nelem)), dev(np.zeros(lac.nelem))
    ops.ApplyHAvec(plan, dev(y), o2)
    ops.ApplyHAvec(plan, dev(0.5 * x - 2.0 * y), o3)
    assert relerr(host(o3), 0.5 * host(out) - 2.0 * host(o2)) < 1e-12


@pytest.mark.parametrize("model,dims0", SMALL)
def test_hc_apply(cuda_ctx, model, dims0):
    st = T.random_state(model, dims0, seed=8)
    d, AL, AR, C, rng = st["d"], st["AL"], st["AR"], st["C"], st["rng"]
    ns = len(st["I2K"][0])
    Cd = {q: m.shape[0] for q, m in C[1].items()}
    EHL, EHR = T.rand_bd(Cd, rng), T.rand_bd(Cd, rng)
    lc = B.Layout(T.bd_blocks(C[1]), ns)
    plan = B.plan_hc(cuda_ctx, lc, lc, lc, B.Layout(T.mps_blocks(AL[1]), ns), B.Layout(T.mps_blocks(AR[0]), ns),
                     d, st["hnnz"])
    plan.bind(2, dev(O.bd_vec(EHL)))
    plan.bind(3, dev(O.bd_vec(EHR)))
    plan.bind(4, dev(O.mps_vec(AL[1])))
    plan.bind(5, dev(O.mps_vec(AR[0])))
    plan.prepare()
    x = rng.standard_normal(lc.nelem)
    ref = O.ApplyHCvec(x, O.bd_sizes(C[1]), EHL, EHR, st["hnnz"], d, AL[1], AR[0])
    out = dev(np.zeros(lc.nelem))
    ops.ApplyHCvec(plan, dev(x), out)
    assert relerr(host(out), ref) < RTOL


@pytest.mark.parametrize("model,dims0", SMALL)
@pytest.mark.parametrize("direction", [0, 1])
def test_tm_apply_and_proj(cuda_ctx, model, dims0, direction):
    st = T.random_state(model, dims0, seed=13)
    AL, dv, rng = st["AL"], st["dimvec"], st["rng"]
    ns = len(st["I2K"][0])
    l0, l1 = B.Layout(T.mps_blocks(AL[0]), ns), B.Layout(T.mps_blocks(AL[1]), ns)
    bond = B.Layout.blockdiag(dv[0])
    plan = B.plan_tm(cuda_ctx, [l0, l1], direction, bond, bond)
    plan.bind(2, dev(O.mps_vec(AL[0])))
    plan.bind(3, dev(O.mps_vec(AL[1])))
    X = T.rand_bd(dv[0], rng, sym=False)
    ref = O.bd_vec(O.ApplyTMLeftUC(AL, X) if direction == 0 else O.ApplyTMRightUC(AL, X))
    out = dev(np.zeros(bond.nelem))
    ops.ApplyTM(plan, dev(O.bd_vec(X)), out)
    assert relerr(host(out), ref) < RTOL
    rin, rout = T.rand_bd(dv[0], rng), T.rand_bd(dv[0], rng)
    sizes = O.bd_sizes(X)
    fun = (lambda Y: O.ApplyTMLeftUC(AL, Y)) if direction == 0 else (lambda Y: O.ApplyTMRightUC(AL, Y))
    ref = O.InvEfun_proj(O.bd_vec(X), fun, rin, rout, sizes)
    out2 = dev(np.zeros(bond.nelem))
    ops.InvEfun_proj(plan, dev(O.bd_vec(X)), dev(O.bd_vec(rin)), dev(O.bd_vec(rout)), out2)
    assert relerr(host(out2), ref) < RTOL


@pytest.mark.parametrize("model,dims0", SMALL)
@pytest.mark.parametrize("direction", ["l", "r"])
def test_redop_and_optm(cuda_ctx, model, dims0, direction):
    st = T.random_state(model, dims0, seed=17)
    d, hnnz = st["d"], st["hnnz"]
    ns = len(st["I2K"][0])
    A0, A1 = st["AL"] if direction == "l" else st["AR"]
    la0, la1 = B.Layout(T.mps_blocks(A0), ns), B.Layout(T.mps_blocks(A1), ns)
    plan = B.plan_redop(cuda_ctx, la1, d, hnnz, 0 if direction == "l" else 1)
    lo = plan.derived(0)
    out = dev(np.zeros(lo.nelem))
    plan.bind(0, dev(O.mps_vec(A1)))
    plan.bind(1, out)
    plan.run()
    ref = T.redop_vec(O.ReducedOp(hnnz, A1, d, direction), d)
    assert relerr(host(out), ref) < RTOL
    # operator transfer matrix on the 2-site product
    AA = O.mps_mul_mps(A0, A1)
    refd = O.ApplyOpTMLeftDiag(hnnz, AA) if direction == "l" else O.ApplyOpTMRightDiag(hnnz, AA)
    lout = B.Layout.blockdiag({q: M.shape[0] for q, M in refd.items()})
    p2 = B.plan_optm(cuda_ctx, la0, la1, d, hnnz, 0 if direction == "l" else 1, lout)
    o2 = dev(np.zeros(lout.nelem))
    p2.bind(0, dev(O.mps_vec(A0)))
    p2.bind(1, dev(O.mps_vec(A1)))
    p2.bind(2, o2)
    p2.run()
    assert relerr(host(o2), O.bd_vec(refd)) < RTOL


def test_mps_bd_products(cuda_ctx):
    st = T.random_state("fhub", SMALL[1][1], seed=19)
    AR, C = st["AR"], st["C"]
    ns = 2
    la = B.Layout(T.mps_blocks(AR[0]), ns)
    lc = B.Layout(T.bd_blocks(C[1]), ns)
    p = B.plan_mps_bd(cuda_ctx, la, lc, 0)  # C * AR
    out = dev(np.zeros(la.nelem))
    p.bind(0, dev(O.mps_vec(AR[0])))
    p.bind(1, dev(O.bd_vec(C[1])))
    p.bind(2, out)
    p.run()
    assert relerr(host(out), O.mps_vec(O.bd_mul_mps(C[1], AR[0]))) < RTOL
    lc0 = B.Layout(T.bd_blocks(C[0]), ns)
    p2 = B.plan_mps_bd(cuda_ctx, la, lc0, 1, alpha=-2.0, transpose_x=True)  # -2 * AR * C^T
    o2 = dev(np.zeros(la.nelem))
    p2.bind(0, dev(O.mps_vec(AR[0])))
    p2.bind(1, dev(O.bd_vec(C[0])))
    p2.bind(2, o2)
    p2.run()
    ref = O.mps_vec(O.mps_mul_bd(AR[0], O.bd_t(C[0])))
    assert relerr(host(o2), -2.0 * ref) < RTOL


FULL = ["xxz_d512", "hubbard_d1024"]


def _full_state(name, seed):
    model, dims0, params = T.workload_dims(name)
    return T.random_state(model, dims0, seed=seed, **params)


@pytest.mark.parametrize("name", FULL)
def test_hc_apply_full_size(cuda_ctx, name):
    """ApplyHCvec (VUMPS_helpers.hpp:114-133) at the benchmark sizes against the oracle's
    literal chained form, 1e-12."""
    st = _full_state(name, 31)
    d, AL, AR, C, rng = st["d"], st["AL"], st["AR"], st["C"], st["rng"]
    ns = len(st["I2K"][0])
    Cd = {q: m.shape[0] for q, m in C[1].items()}
    EHL, EHR = T.rand_bd(Cd, rng), T.rand_bd(Cd, rng)
    lc = B.Layout(T.bd_blocks(C[1]), ns)
    plan = B.plan_hc(cuda_ctx, lc, lc, lc, B.Layout(T.mps_blocks(AL[1]), ns), B.Layout(T.mps_blocks(AR[0]), ns),
                     d, st["hnnz"])
    for slot, v in ((2, O.bd_vec(EHL)), (3, O.bd_vec(EHR)), (4, O.mps_vec(AL[1])), (5, O.mps_vec(AR[0]))):
        plan.bind(slot, dev(v))
    plan.prepare()
    x = rng.standard_normal(lc.nelem)
    ref = O.ApplyHCvec(x, O.bd_sizes(C[1]), EHL, EHR, st["hnnz"], d, AL[1], AR[0])
    out = dev(np.full(lc.nelem, np.nan))
    ops.ApplyHCvec(plan, dev(x), out)
    assert relerr(host(out), ref) < RTOL


@pytest.mark.parametrize("name", FULL)
@pytest.mark.parametrize("direction", [0, 1])
def test_tm_chain_and_proj_full_size(cuda_ctx, name, direction):
    """The unit-cell TM chain (TMBlockFunctions.hpp:542-625) and InvEfun_proj
    (InvEBlockFunctions.hpp:12-47) at the benchmark sizes against the oracle, 1e-12."""
    st = _full_state(name, 37)
    AL, dv, rng = st["AL"], st["dimvec"], st["rng"]
    ns = len(st["I2K"][0])
    l0, l1 = B.Layout(T.mps_blocks(AL[0]), ns), B.Layout(T.mps_blocks(AL[1]), ns)
    bond = B.Layout.blockdiag(dv[0])
    plan = B.plan_tm(cuda_ctx, [l0, l1], direction, bond, bond)
    plan.bind(2, dev(O.mps_vec(AL[0])))
    plan.bind(3, dev(O.mps_vec(AL[1])))
    X = T.rand_bd(dv[0], rng, sym=False)
    fun = (lambda Y: O.ApplyTMLeftUC(AL, Y)) if direction == 0 else (lambda Y: O.ApplyTMRightUC(AL, Y))
    out = dev(np.full(bond.nelem, np.nan))
    ops.ApplyTM(plan, dev(O.bd_vec(X)), out)
    assert relerr(host(out), O.bd_vec(fun(X))) < RTOL
    rin, rout = T.rand_bd(dv[0], rng), T.rand_bd(dv[0], rng)
    ref = O.InvEfun_proj(O.bd_vec(X), fun, rin, rout, O.bd_sizes(X))
    out2 = dev(np.zeros(bond.nelem))
    ops.InvEfun_proj(plan, dev(O.bd_vec(X)), dev(O.bd_vec(rin)), dev(O.bd_vec(rout)), out2)
    assert relerr(host(out2), ref) < RTOL


@pytest.mark.parametrize("name", FULL)
def test_inverte_proj_full_size(cuda_ctx, name):
    """InvertE_proj (InvEBlockFunctions.hpp:201-266) for the left environment of a canonical
    unit cell at the benchmark sizes: the device's restarted GMRES against the reference's
    GMRES restated in the oracle, both to 1e-12; solutions agree to 1e-8 relative."""
    st = _full_state(name, 41)
    AL, C, dv, hnnz = st["AL"], st["C"], st["dimvec"], st["hnnz"]
    ns = len(st["I2K"][0])
    l0, l1 = B.Layout(T.mps_blocks(AL[0]), ns), B.Layout(T.mps_blocks(AL[1]), ns)
    bond = B.Layout.blockdiag(dv[0])
    R = O.bd_mul(C[1], O.bd_t(C[1]))
    _, R = O.TMDominantEig(AL, dv[0], "r", 1e-14, R)
    x = O.GetHL(AL, hnnz)
    eye = O.bd_eye(dv[0])
    yref, flag = O.InvertE_proj(AL, x, eye, R, "l", 1e-12)
    assert flag > 0
    plan = B.plan_tm(cuda_ctx, [l0, l1], 0, bond, bond)
    plan.bind(2, dev(O.mps_vec(AL[0])))
    plan.bind(3, dev(O.mps_vec(AL[1])))
    y = dev(np.zeros(bond.nelem))
    it, rr, conv = ops.InvertE_proj(plan, dev(O.bd_vec(x)), dev(O.bd_vec(eye)), dev(O.bd_vec(R)), "l", y, 1e-12)
    assert conv, (it, rr)
    assert relerr(host(y), O.bd_vec(yref)) < 1e-8
