"""Shared helpers for the tests: random block-sparse problems built with the oracle and
conversion between oracle structures and native layouts / flat vectors."""
from __future__ import annotations

import numpy as np

from imps_cpp_tools_gb300 import configs, models
from oracle import imps_oracle as O


def mps_blocks(A):
    return [(s, qi, A[s][qi][0], A[s][qi][1].shape[0], A[s][qi][1].shape[1])
            for s in range(len(A)) for qi in sorted(A[s])]


def bd_blocks(X):
    return [(0, q, q, X[q].shape[0], X[q].shape[1]) for q in sorted(X)]


def bm_blocks(X):
    """General BlockMat (one block per incoming charge)."""
    return [(0, q, X[q][0], X[q][1].shape[0], X[q][1].shape[1]) for q in sorted(X)]


def redop_blocks(R, d):
    return [(i * d + j, qi, R[i][j][qi][0], R[i][j][qi][1].shape[0], R[i][j][qi][1].shape[1])
            for i in range(d) for j in range(d) for qi in sorted(R[i][j])]


def redop_vec(R, d):
    parts = [O.bm_vec(R[i][j]) for i in range(d) for j in range(d) if R[i][j]]
    return np.concatenate(parts) if parts else np.zeros(0)


def rand_bd(dims, rng, sym=True):
    X = {}
    for q in sorted(dims):
        m = dims[q]
        M = rng.standard_normal((m, m))
        X[q] = 0.5 * (M + M.T) if sym else M
    return X


def random_state(model, dims0, seed=0, **params):
    """Left/right-canonical 2-site unit cell from the oracle's randMPS_LR, plus model data."""
    d, I2K, h = models.build_model(model, **params)
    hnnz = models.h_nonzeros(h)
    rng = np.random.default_rng(seed)
    dimvec = O.make_dims(dims0, 2, I2K)
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, rng)
    return dict(d=d, I2K=I2K, h=h, hnnz=hnnz, dimvec=dimvec, AL=AL, AR=AR, C=C, rng=rng)


def hac_problem(model, dims0, seed=0, **params):
    """A random H_AC apply problem: AC = C*AR, EHL/EHR random symmetric, HL/HR = ReducedOp."""
    st = random_state(model, dims0, seed, **params)
    d, hnnz, rng = st["d"], st["hnnz"], st["rng"]
    AL, AR, C = st["AL"], st["AR"], st["C"]
    # layout during the sweep: AC(n) = C(n-1)*AR(n) with AL(n-1) on its left and AR(n+1) on its right
    AC = O.bd_mul_mps(C[1], AR[0])
    HL = O.ReducedOp(hnnz, AL[1], d, "l")
    HR = O.ReducedOp(hnnz, AR[1], d, "r")
    EHL = rand_bd({q: m.shape[0] for q, m in C[1].items()}, rng)
    EHR = rand_bd({q: m.shape[1] for q, m in C[0].items()}, rng)
    st.update(AC=AC, HL=HL, HR=HR, EHL=EHL, EHR=EHR)
    return st


def workload_dims(name):
    model, dims_fn, params = configs.WORKLOADS[name]
    return model, dims_fn(), params
