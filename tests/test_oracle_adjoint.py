"""CPU checks of the energy-density gradient (the adjoint check of the unit cell): the oracle's
adjoint-method gradient against central finite differences of the energy of a general uniform
MPS, against the reference's tangent-space gradient on tangent directions, and the device
programs' tables executed with numpy against the oracle."""
import numpy as np
import pytest

from oracle import imps_oracle as O
from tests import imps_testlib as T

XXZ_DIMS = {(-2,): 2, (0,): 4, (2,): 2}
HUB_DIMS = {(0, 0): 2, (1, 1): 1, (-1, -1): 1, (1, -1): 1, (-1, 1): 1}

# The XXZ anisotropies 0.5, 1.0, 1.5 in the reference's sign convention (J > 0, Delta > 0 is
# ferromagnetic there, so the antiferromagnetic points are Delta = -0.5, -1, -1.5) and the
# Hubbard U = 2, 4 at t = 1.
CASES = [("xxz", XXZ_DIMS, dict(J=1.0, Delta=-0.5)), ("xxz", XXZ_DIMS, dict(J=1.0, Delta=-1.0)),
         ("xxz", XXZ_DIMS, dict(J=1.0, Delta=-1.5)), ("fhub", HUB_DIMS, dict(t=1.0, U=2.0)),
         ("fhub", HUB_DIMS, dict(t=1.0, U=4.0))]


def _state(model, dims0, params, seed=4):
    st = T.random_state(model, dims0, seed=seed, **params)
    st["R"] = O.bd_mul(st["C"][-1], O.bd_t(st["C"][-1]))  # right fixed point on bond 0
    return st


def _perturbed(AL, D, eps):
    return [[{q: (qo, M + eps * D[n][s][q][1]) for q, (qo, M) in bm.items()} for s, bm in enumerate(A)]
            for n, A in enumerate(AL)]


def _rand_like(AL, rng):
    return [[{q: (qo, rng.standard_normal(M.shape)) for q, (qo, M) in bm.items()} for bm in A] for A in AL]


@pytest.mark.parametrize("model,dims0,params", CASES)
def test_gradient_matches_central_differences(model, dims0, params):
    """dE/dA_L by the adjoint method (TM and H_AC-type adjoints, fixed points by transposed
    GMRES) against central differences with step 1e-6 of the energy of the perturbed, no longer
    isometric, unit cell (fixed points from a dense eigendecomposition): 1e-6 relative."""
    st = _state(model, dims0, params)
    AL, hnnz = st["AL"], st["hnnz"]
    G, e = O.energy_gradient(AL, st["R"], hnnz, tol=1e-14)
    assert abs(e - O.energy_uniform(AL, hnnz)) < 1e-12 * max(1.0, abs(e))
    rng = np.random.default_rng(1)
    for _ in range(2):
        D = _rand_like(AL, rng)
        eps = 1e-6
        fd = (O.energy_uniform(_perturbed(AL, D, eps), hnnz) - O.energy_uniform(_perturbed(AL, D, -eps), hnnz)) / (2 * eps)
        an = sum(O.mps_dot(G[n], D[n]) for n in range(2))
        assert abs(fd - an) <= 1e-6 * abs(fd), (fd, an)


@pytest.mark.parametrize("model,dims0,params", [CASES[1], CASES[4]])
def test_coupling_gradient_matches_central_differences(model, dims0, params):
    """dE/dg at fixed A for every coupling g of h (h is linear in them): the energy with h
    replaced by dh/dg, against central differences of the energy in g."""
    from imps_cpp_tools_gb300 import adjoint, models
    st = _state(model, dims0, params)
    AL, R = st["AL"], st["R"]
    for name, hk in adjoint.coupling_terms(model, **params):
        _, e = O.energy_gradient(AL, R, hk, tol=1e-14) if hk else (None, 0.0)
        eps = 1e-6
        hp = models.h_nonzeros(models.build_model(model, **{**params, name: params.get(name, 0.0) + eps})[2])
        hm = models.h_nonzeros(models.build_model(model, **{**params, name: params.get(name, 0.0) - eps})[2])
        fd = (O.energy_uniform(AL, hp) - O.energy_uniform(AL, hm)) / (2 * eps)
        assert abs(fd - e) <= 1e-6 * max(abs(fd), 1e-3), (name, fd, e)


def test_tangent_projection_equals_vumps_gradient():
    """On tangent directions N_L X the gradient equals the reference's tangent-space gradient:
    <G_0, N_L X> = <H_AC AC_0 - AL_0 H_C C_0, N_L X C_0> (VUMPS_helpers.hpp:135-177; the AL H_C C
    part vanishes on N_L), H_AC with the environments of the E0-shifted h."""
    from imps_cpp_tools_gb300 import models
    st = _state("xxz", {(-2,): 3, (0,): 5, (2,): 3}, dict(J=1.0, Delta=-1.0))
    AL, AR, C, hnnz, d = st["AL"], st["AR"], st["C"], st["hnnz"], st["d"]
    R = st["R"]
    L = O.bd_mul(O.bd_t(C[1]), C[1])
    G, e = O.energy_gradient(AL, R, hnnz)
    h = models.build_model("xxz", J=1.0, Delta=-1.0)[2]
    hs = O.sparse_nnz(h - e * np.eye(h.shape[0]))
    HLtot, HRtot = O.HeffConstants(AL, AR, L, R, hs, tol=1e-14)
    AC0 = O.mps_mul_bd(AL[0], C[0])
    Y = O.ApplyHA(AC0, HLtot[1], HRtot[1], O.ReducedOp(hs, AL[1], d, "l"), O.ReducedOp(hs, AR[1], d, "r"))
    NL = O.Nullspace(AL[0], "l")
    rng = np.random.default_rng(3)
    for _ in range(3):
        X = {}
        for bm in NL:
            for qi, (qo, M) in bm.items():
                X.setdefault(qo, (qo, rng.standard_normal((M.shape[1], C[0][qo].shape[0]))))
        B = O.mps_mul_bm(NL, X)
        lhs, rhs = O.mps_dot(G[0], B), O.mps_dot(Y, O.mps_mul_bd(B, C[0]))
        assert abs(lhs - rhs) <= 1e-9 * abs(rhs), (lhs, rhs)


@pytest.mark.parametrize("model,dims0,params", [CASES[1], CASES[3]])
def test_gradient_program_tables_match_oracle(model, dims0, params):
    """The device programs of the gradient (imps_cpp_tools_gb300.adjoint), executed table by table
    with numpy and the oracle's InvertE_proj for the two transposed solves, reproduce the
    oracle's gradient: the sector matching and term expansion checked without a GPU."""
    from imps_cpp_tools_gb300 import adjoint as AD
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300.excitations import ES, OPS, OUT, RHS, SCR
    from tests.test_oracle_excitations import run_tables
    st = _state(model, dims0, params)
    AL, R, hnnz, d = st["AL"], st["R"], st["hnnz"], st["d"]
    ns = len(st["I2K"][0])
    LA = [B.Layout(T.mps_blocks(a), ns) for a in AL]
    C = st["C"]
    LB = [B.Layout(T.bd_blocks(C[1]), ns), B.Layout(T.bd_blocks(C[0]), ns)]  # bond 0, bond 1
    pr = AD.EnergyGradientProgram(LA, LB, hnnz, d)
    bufs = {k: np.zeros(max(int(pr.sizes.get(k, 0)), 1)) for k in range(6)}
    r = O.bd_scale(R, 1.0 / O.bd_trace(R))
    bufs[OPS][pr.a0_off:pr.a0_off + LA[0].nelem] = O.mps_vec(AL[0])
    bufs[OPS][pr.a1_off:pr.a1_off + LA[1].nelem] = O.mps_vec(AL[1])
    nb = LB[0].nelem
    bufs[OPS][pr.r_off:pr.r_off + nb] = O.bd_vec(r)
    run_tables(pr.prog_a.stages, bufs)
    N0 = float(bufs[SCR][pr.g0a_off:pr.g0a_off + LA[0].nelem] @ O.mps_vec(AL[0]))
    N1 = float(bufs[SCR][pr.g1b_off:pr.g1b_off + LA[1].nelem] @ O.mps_vec(AL[1]))
    E2, E2l = N0 + N1, N0 + 2 * N1
    sizes = O.bd_sizes(r)
    I0 = O.bd_eye(dict(sizes))
    gl = bufs[RHS][pr.gl_off:pr.gl_off + nb] - 0.5 * E2 * O.bd_vec(r)
    gr = bufs[RHS][pr.gr_off:pr.gr_off + nb] - 0.5 * E2 * O.bd_vec(I0)
    yl, _ = O.InvertE_proj(AL, O.bd_from_vec(gl, sizes), I0, r, "r", tol=1e-14)
    yr, _ = O.InvertE_proj(AL, O.bd_from_vec(gr, sizes), I0, r, "l", tol=1e-14)
    bufs[ES][pr.yl_off:pr.yl_off + nb] = O.bd_vec(yl)
    bufs[ES][pr.yr_off:pr.yr_off + nb] = O.bd_vec(yr)
    run_tables(pr.prog_b.stages, bufs)
    G0 = bufs[OUT][pr.g0_off:pr.g0_off + LA[0].nelem] - E2l * bufs[SCR][pr.a0r1_off:pr.a0r1_off + LA[0].nelem]
    G1 = bufs[OUT][pr.g1_off:pr.g1_off + LA[1].nelem] - E2l * bufs[SCR][pr.a1r_off:pr.a1r_off + LA[1].nelem]
    Gref, e = O.energy_gradient(AL, R, hnnz, tol=1e-14)
    assert abs(0.5 * E2 - e) < 1e-12
    for got, ref in ((G0, O.mps_vec(Gref[0])), (G1, O.mps_vec(Gref[1]))):
        assert np.linalg.norm(got - ref) <= 1e-9 * np.linalg.norm(ref)
