"""GPU parity of the Krylov solvers (device Lanczos for eigs_rs, device GMRES for InvertE_proj,
TMDominantEig) and of GradNormRight against the oracle's ARPACK / reference-GMRES path.

Eigenvalues: 1e-10 relative; solutions of the environment solve: 1e-8 relative at
tol = 1e-12 (GMRES stopping is on the residual, so the solutions differ by up to
cond * tol); fixed points and gradient norms: 1e-9 relative."""
import math

import numpy as np
import pytest

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops
from oracle import imps_oracle as O
from tests import imps_testlib as T
from tests.test_gpu_parity import SMALL, _hac_setup, dev, host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model,dims0", SMALL + [("xxz", "xxz_d64")])
def test_eigs_rs_hac(cuda_ctx, model, dims0):
    if isinstance(dims0, str):
        model, dims0, _ = T.workload_dims(dims0)
    p = T.hac_problem(model, dims0, seed=23)
    plan, lac = _hac_setup(cuda_ctx, p)
    sizes = O.mps_sizes(p["AC"])
    x0 = O.mps_vec(p["AC"])
    vals, vecs = O.eigs_rs(lambda v: O.ApplyHAvec(v, sizes, p["EHL"], p["EHR"], p["HL"], p["HR"]),
                           lac.nelem, 1e-13, x0)
    x = dev(x0)
    ev, napp, conv = ops.eigs_rs(plan, x, 1e-13)
    assert conv
    assert abs(ev - vals[0]) <= 1e-10 * abs(vals[0])
    xv = host(x)
    assert abs(np.linalg.norm(xv) - 1) < 1e-12
    assert abs(abs(xv @ vecs[:, 0]) - 1.0) < 1e-8
    # residual with an FP64 apply
    hx = dev(np.zeros(lac.nelem))
    ops.ApplyHAvec(plan, x, hx)
    assert np.linalg.norm(host(hx) - ev * xv) < 1e-9 * abs(ev)


def test_eigs_rs_hc(cuda_ctx):
    st = T.random_state("xxz", {(-4,): 2, (-2,): 4, (0,): 6, (2,): 4, (4,): 2}, seed=5)
    d, AL, AR, C, rng = st["d"], st["AL"], st["AR"], st["C"], st["rng"]
    Cd = {q: m.shape[0] for q, m in C[1].items()}
    EHL, EHR = T.rand_bd(Cd, rng), T.rand_bd(Cd, rng)
    lc = B.Layout(T.bd_blocks(C[1]), 1)
    plan = B.plan_hc(cuda_ctx, lc, lc, lc, B.Layout(T.mps_blocks(AL[1]), 1), B.Layout(T.mps_blocks(AR[0]), 1),
                     d, st["hnnz"])
    for s, v in ((2, O.bd_vec(EHL)), (3, O.bd_vec(EHR)), (4, O.mps_vec(AL[1])), (5, O.mps_vec(AR[0]))):
        plan.bind(s, dev(v))
    plan.prepare()
    sizes = O.bd_sizes(C[1])
    x0 = O.bd_vec(C[1])
    vals, vecs = O.eigs_rs(lambda v: O.ApplyHCvec(v, sizes, EHL, EHR, st["hnnz"], d, AL[1], AR[0]),
                           lc.nelem, 1e-13, x0)
    x = dev(x0)
    ev, _, conv = ops.eigs_rs(plan, x, 1e-13)
    assert conv and abs(ev - vals[0]) <= 1e-10 * abs(vals[0])
    assert abs(abs(host(x) @ vecs[:, 0]) - 1.0) < 1e-8


@pytest.mark.parametrize("model,dims0", SMALL)
@pytest.mark.parametrize("direction", ["l", "r"])
def test_inverte_proj(cuda_ctx, model, dims0, direction):
    st = T.random_state(model, dims0, seed=29)
    ns = len(st["I2K"][0])
    Avec = st["AL"] if direction == "l" else st["AR"]
    dv, rng = st["dimvec"], st["rng"]
    bond = B.Layout.blockdiag(dv[0])
    la = [B.Layout(T.mps_blocks(A), ns) for A in Avec]
    plan = B.plan_tm(cuda_ctx, la, 0 if direction == "l" else 1, bond, bond)
    for k, A in enumerate(Avec):
        plan.bind(2 + k, dev(O.mps_vec(A)))
    _, rho = O.TMDominantEig(Avec, dv[0], "r" if direction == "l" else "l", 1e-14)
    eye = O.bd_eye(dv[0])
    L, R = (eye, rho) if direction == "l" else (rho, eye)
    x = T.rand_bd(dv[0], rng)
    y0 = T.rand_bd(dv[0], rng)
    yref, flag = O.InvertE_proj(Avec, x, L, R, direction, 1e-12, 0, y0)
    assert flag > 0
    y = dev(O.bd_vec(y0))
    it, rr, conv = ops.InvertE_proj(plan, dev(O.bd_vec(x)), dev(O.bd_vec(L)), dev(O.bd_vec(R)), direction, y,
                                    1e-12)
    assert conv and rr < 1e-12
    yr = O.bd_vec(yref)
    assert np.abs(host(y) - yr).max() < 1e-8 * np.abs(yr).max()


@pytest.mark.parametrize("model,dims0", SMALL)
@pytest.mark.parametrize("direction", ["l", "r"])
def test_tm_dominant(cuda_ctx, model, dims0, direction):
    st = T.random_state(model, dims0, seed=31)
    ns = len(st["I2K"][0])
    # right fixed point of the AL unit cell / left fixed point of the AR unit cell (isometric)
    Avec = st["AL"] if direction == "r" else st["AR"]
    dv = st["dimvec"]
    bond = B.Layout.blockdiag(dv[0])
    la = [B.Layout(T.mps_blocks(A), ns) for A in Avec]
    plan = B.plan_tm(cuda_ctx, la, 1 if direction == "r" else 0, bond, bond)
    for k, A in enumerate(Avec):
        plan.bind(2 + k, dev(O.mps_vec(A)))
    lam_ref, Vref = O.TMDominantEig(Avec, dv[0], direction, 1e-14)
    V = dev(np.zeros(bond.nelem))
    lam, it, conv = ops.TMDominantEig(plan, V, None, 1e-14)
    assert conv
    assert abs(lam - 1.0) < 1e-12 and abs(lam_ref - 1.0) < 1e-10
    vr = O.bd_vec(Vref)
    assert np.abs(host(V) - vr).max() < 1e-9 * np.abs(vr).max()


@pytest.mark.parametrize("model,dims0", SMALL)
def test_grad_norm_right(cuda_ctx, model, dims0):
    p = T.hac_problem(model, dims0, seed=37)
    ns = len(p["I2K"][0])
    plan, lac = _hac_setup(cuda_ctx, p)
    AR, C = p["AR"], p["C"]
    HA = lambda X: O.ApplyHA(X, p["EHL"], p["EHR"], p["HL"], p["HR"])
    Fref = O.GradNormRight(AR[0], C[1], HA)
    y = dev(np.zeros(lac.nelem))
    ops.ApplyHAvec(plan, dev(O.mps_vec(p["AC"])), y)
    lar = B.Layout(T.mps_blocks(AR[0]), ns)
    g = B.plan_grad_right(cuda_ctx, lac, lar)
    g.bind(0, y)
    g.bind(1, dev(O.mps_vec(AR[0])))
    g.bind(2, dev(np.zeros(lar.nelem)))
    F = ops.GradNormRight(g)
    assert math.isfinite(F) and abs(F - Fref) <= 1e-9 * Fref
