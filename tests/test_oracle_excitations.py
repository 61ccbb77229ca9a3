"""CPU checks that pin the oracle's restatement of the mixed transfer matrices and the factored
environment solves used by the excitation ansatz (TMBlockFunctions.hpp, InvEBlockFunctions.hpp)."""
import numpy as np
import pytest

from oracle import imps_oracle as O
from tests import imps_testlib as T

B0 = {(-4,): 3, (-2,): 8, (0,): 10, (2,): 8, (4,): 3}


def offset_bm(dims, K, rng, cplx=False):
    """Random BlockMat on one bond with charge offset K: blocks q -> q + K where both exist."""
    X = {}
    for q in sorted(dims):
        qo = O.kadd(q, K)
        if qo in dims:
            M = rng.standard_normal((dims[q], dims[qo]))
            if cplx:
                M = M + 1j * rng.standard_normal(M.shape)
            X[q] = (qo, M)
    return X


def inner(X, Y):
    return sum(np.vdot(X[q][1], Y[q][1]) for q in X if q in Y)


@pytest.fixture(scope="module")
def state():
    return T.random_state("xxz", B0, seed=3, J=1.0, Delta=-1.0)


def test_mixed_tm_reduces_to_plain_tm(state):
    AL, dv, rng = state["AL"], state["dimvec"], np.random.default_rng(1)
    X = T.rand_bd(dv[0], rng, sym=False)
    Xb = {q: (q, M) for q, M in X.items()}
    left = O.ApplyTMmixedLeftUC(AL, AL, Xb)
    right = O.ApplyTMmixedRightUC(AL, AL, Xb)
    ref_l, ref_r = O.ApplyTMLeftUC(AL, X), O.ApplyTMRightUC(AL, X)
    for q in ref_l:
        assert np.allclose(left[q][1], ref_l[q], atol=1e-13)
    for q in ref_r:
        assert np.allclose(right[q][1], ref_r[q], atol=1e-13)


@pytest.mark.parametrize("K", [(2,), (0,), (-2,)])
def test_mixed_tm_left_right_adjoint(state, K):
    """<Y, sum_s B_s^T X A_s> = <sum_s B_s Y A_s^T, X> (the two mixed maps are adjoint)."""
    AL, AR, dv = state["AL"], state["AR"], state["dimvec"]
    rng = np.random.default_rng(2)
    X = offset_bm(dv[0], K, rng)
    Y = offset_bm(dv[1], K, rng)
    lhs = inner(Y, O.ApplyTMmixedLeftX(AR[0], AL[0], X))
    rhs = inner(O.ApplyTMmixedRightX(AL[0], AR[0], Y), X)
    assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(lhs))


def test_invert_e_fac_solves_its_equation(state):
    AL, AR, dv = state["AL"], state["AR"], state["dimvec"]
    rng = np.random.default_rng(4)
    x = offset_bm(dv[0], (2,), rng, cplx=True)
    fac = np.exp(0.7j)
    y, flag = O.InvertE_fac(AL, AR, x, "r", fac, tol=1e-13)
    assert flag >= 0
    res = O.bm_vec(y) - fac * O.bm_vec(O.ApplyTMmixedRightUC(AL, AR, y)) - O.bm_vec(x)
    assert np.linalg.norm(res) < 1e-11 * np.linalg.norm(O.bm_vec(x))
