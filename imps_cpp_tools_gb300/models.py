"""Models and charge bookkeeping of the hot path (host side, integer-exact).

Restates, for the GB300 driver, the pieces of MPShelpers/src/Models.cpp and
include/Block/ItoKey.hpp that define the inputs of the hot path: the two-site Hamiltonian h
(as its nonzeros in armadillo SpMat iteration order), the physical-index -> charge map I2K,
validpath and MakeDims, for U(1) (XXZ, Fermi-Hubbard, Bose-Hubbard) and Z(N) charges (quantum
Ising, quantum Potts; charges.py holds the group arithmetic).
"""
from __future__ import annotations

import math

import numpy as np


from . import charges


def _kadd(a, b, periods=None):
    return charges.add(a, b, periods) if periods else tuple(x + y for x, y in zip(a, b))


def xxz_i2k(N=2, QN=(0,), d=2):
    """XXZModel::GetdQ + GetI2K (Models.cpp:216-295), spin-1/2."""
    m = QN[0]
    if abs(m) >= N:
        raise ValueError("|m| must be < N")
    div = math.gcd(N - m, N + m)
    first, second = 2 * N // div, -((N + m) // div)
    return [(second + s * first,) for s in range(d - 1, -1, -1)]


def fhub_i2k(N=2, QN=(2, 0)):
    """FermiHubbardModel::GetdQ + GetI2K, (N,M) representation (Models.cpp:642-718)."""
    n, m = QN
    if n + m <= 0 or n + m >= 2 * N or n - m <= 0 or n - m >= 2 * N:
        raise ValueError("QN out of range")
    divn = math.gcd(math.gcd(N - n, 2 * N - n), n)
    divm = math.gcd(math.gcd(N - m, N + m), m)
    a1, a0 = N // divn, -(n // divn)
    b1, b0 = N // divm, -((N + m) // divm)
    return [(a0, b0 + b1), (a0 + a1, b0), (a0 + a1, b0 + 2 * b1), (a0 + 2 * a1, b0 + b1)]


def bhub_i2k(N=2, QN=(2,), d=4):
    """BoseHubbardModel::GetdQ + GetI2K (Models.cpp:825-862): n = QN[0] bosons per N-site cell,
    charge of level i = (i N - n) / gcd(N, n)."""
    n = QN[0]
    if n < 1 or n >= N * d:
        raise ValueError(f"0 < n < {N * d}")
    div = math.gcd(N, n)
    first, second = N // div, -(n // div)
    return [(second + i * first,) for i in range(d)]


def qim_i2k():
    """QuantumIsingModel::GetI2K (Models.cpp:371-375): the Z(2) parity of sz, [0, 1]."""
    return charges.I2K([(0,), (1,)], (2,))


def potts_i2k(q):
    """QuantumPottsModel::GetI2K (Models.cpp:498-504): level i -> i in Z(q)."""
    return charges.I2K([(i,) for i in range(q)], (q,))


def validpath(N, I2K):
    """ItoKey.hpp:126-165: indices j_1..j_N with sum I2K[j] = 0, first-found depth-first order."""
    per = charges.periods_of(I2K)

    def it(n, key):
        if n == 1:
            for j, k in enumerate(I2K):
                if _kadd(key, k, per) == I2K[0]:
                    return [j]
            return None
        for j, k in enumerate(I2K):
            p = it(n - 1, _kadd(key, k, per))
            if p is not None:
                return p + [j]
        return None
    p = it(N, I2K[0])
    if p is None:
        raise ValueError("no valid path for this I2K")
    return p


def make_dims(dmap0, N, I2K):
    """ModelBase::MakeDims (Models.cpp:13-32): bond dims k = 0..N-1 from bond 0."""
    path = validpath(N, I2K)
    out, cur = [], dict(dmap0)
    for k in range(N):
        out.append(dict(cur))
        sh = I2K[path[N - k - 1]]
        cur = {_kadd(q, sh, charges.periods_of(I2K)): m for q, m in cur.items()}
    return out


def xxz_h(J=1.0, Delta=1.0, hz=0.0):
    """XYZAbstractModel::MakeOps (Models.cpp:57-93) with Jx=Jy=J, Jz=Delta (d=2)."""
    sx = np.array([[0.0, 0.5], [0.5, 0.0]])
    syi = np.array([[0.0, -0.5], [0.5, 0.0]])
    sz = np.diag([0.5, -0.5])
    one = np.eye(2)
    return (-J * np.kron(sx, sx) + J * np.kron(syi, syi) - Delta * np.kron(sz, sz)
            - 0.5 * hz * (np.kron(sz, one) + np.kron(one, sz)))


def fhub_h(t=1.0, U=4.0, V=0.0, mu=0.0, hz=0.0):
    """FermiHubbardModel::MakeOps (Models.cpp:543-572)."""
    cup = np.zeros((4, 4)); cup[0, 2] = 1.0; cup[1, 3] = 1.0
    cdo = np.zeros((4, 4)); cdo[0, 1] = 1.0; cdo[2, 3] = -1.0
    nup = np.diag([0.0, 0.0, 1.0, 1.0]); ndo = np.diag([0.0, 1.0, 0.0, 1.0])
    one = np.eye(4); F = np.diag([1.0, -1.0, -1.0, 1.0])
    nup2, ndo2 = nup - 0.5 * one, ndo - 0.5 * one
    nund, nupnd, nupnd2, sz = nup2 @ ndo2, nup + ndo, nup2 + ndo2, 0.5 * (nup - ndo)
    hop = (np.kron(cup.T @ F, cup) - np.kron(cup @ F, cup.T) + np.kron(cdo.T @ F, cdo)
           - np.kron(cdo @ F, cdo.T))
    return (-t * hop + 0.5 * U * (np.kron(nund, one) + np.kron(one, nund)) + V * np.kron(nupnd2, nupnd2)
            - 0.5 * mu * (np.kron(nupnd, one) + np.kron(one, nupnd))
            - 0.5 * hz * (np.kron(sz, one) + np.kron(one, sz)))


def observables(model, names, d=4):
    """GetObservables (Models.cpp:95-147 for the XYZ models incl. quantum Ising, 436-468 for
    Potts with q = d, 575-632 for Fermi-Hubbard, 782-823 for Bose-Hubbard with d levels): the
    one-site operators named in ``names`` as (name, d x d matrix) pairs, in the order given.
    An unknown name is skipped with the reference's message ("operator X not defined")."""
    import sys
    if model in ("xxz", "qim"):
        sx = np.array([[0.0, 0.5], [0.5, 0.0]])
        syi = np.array([[0.0, -0.5], [0.5, 0.0]])
        sz = np.diag([0.5, -0.5])
        table = {"sx": sx, "syi": syi, "sz": sz, "sp": sx - syi, "sm": sx + syi, "rx": 2 * sx, "rz": 2 * sz}
    elif model == "fhub":
        cup = np.zeros((4, 4)); cup[0, 2] = 1.0; cup[1, 3] = 1.0
        cdo = np.zeros((4, 4)); cdo[0, 1] = 1.0; cdo[2, 3] = -1.0
        nup, ndo = np.diag([0.0, 0.0, 1.0, 1.0]), np.diag([0.0, 1.0, 0.0, 1.0])
        rx = np.zeros((4, 4))
        for r, c, v in ((0, 0, 1.0), (1, 2, 1.0), (2, 1, 1.0), (3, 3, -1.0)):
            rx[r, c] = v
        table = {"cup": cup, "cdo": cdo, "cupd": cup.T.copy(), "cdod": cdo.T.copy(), "nup": nup, "ndo": ndo,
                 "sz": 0.5 * (nup - ndo), "n": nup + ndo, "rx": rx, "rz": np.diag([1.0, -1.0, 1.0, -1.0])}
    elif model == "potts":
        X, Z = potts_ops(d)
        table = {"X": X, "Z": Z}
    elif model == "bhub":
        b, n = bhub_ops(d)
        nmax = np.zeros((d, d))
        nmax[d - 1, d - 1] = 1.0
        table = {"b": b, "b2": b @ b, "n": n, "nmax": nmax}
    else:
        raise ValueError(f"unknown model {model}")
    out = []
    for name in names:
        if name not in table:
            print(f"operator {name} not defined", file=sys.stderr)
            continue
        out.append((name, table[name]))
    return out


def qim_h(J=1.0, h=1.0):
    """QuantumIsingModel = XYZAbstractModel(QIM, J, 0, 0, h, 2) (Models.cpp:323-330, 91):
    -J sx sx - h/2 (sz 1 + 1 sz) with spin-1/2 operators."""
    sx = np.array([[0.0, 0.5], [0.5, 0.0]])
    sz = np.diag([0.5, -0.5])
    one = np.eye(2)
    return -J * np.kron(sx, sx) - 0.5 * h * (np.kron(sz, one) + np.kron(one, sz))


def potts_ops(q):
    """X (cyclic shift, X(i-1, i) = 1, X(q-1, 0) = 1) and Z = diag(q - 1, -1, ..., -1) of
    QuantumPottsModel::MakeOps (Models.cpp:405-418)."""
    X = np.zeros((q, q))
    X[q - 1, 0] = 1.0
    for i in range(1, q):
        X[i - 1, i] = 1.0
    Z = -np.eye(q)
    Z[0, 0] = q - 1
    return X, Z


def potts_h(q=3, h=1.0):
    """QuantumPottsModel::MakeOps (Models.cpp:405-425): -h/2 (Z 1 + 1 Z) - sum_k X^k X^(q-k)."""
    X, Z = potts_ops(q)
    one = np.eye(q)
    H = -0.5 * h * (np.kron(Z, one) + np.kron(one, Z))
    P = [np.linalg.matrix_power(X, k) for k in range(1, q)]
    for i in range(q - 1):
        H -= np.kron(P[i], P[q - 2 - i])
    return H


def bhub_ops(d=4):
    """Annihilator b and number operator n of BoseHubbardModel::MakeOps (Models.cpp:768-779)."""
    b = np.zeros((d, d))
    n = np.zeros((d, d))
    for i in range(1, d):
        b[i - 1, i] = math.sqrt(i)
        n[i, i] = i
    return b, n


def bhub_h(d=4, t=1.0, U=4.0, mu=0.0):
    """BoseHubbardModel::MakeOps (Models.cpp:768-779): -t (b b^+ + b^+ b) plus the on-site
    0.5 U n (n - 1) - mu n shared equally by the two sites."""
    b, n = bhub_ops(d)
    one = np.eye(d)
    onsite = 0.5 * U * n @ (n - one) - mu * n
    return -t * (np.kron(b, b.T) + np.kron(b.T, b)) + 0.5 * (np.kron(onsite, one) + np.kron(one, onsite))


def h_nonzeros(h):
    """Nonzeros (row, col, value) in armadillo SpMat iteration order (column-major)."""
    out = []
    for c in range(h.shape[1]):
        for r in range(h.shape[0]):
            if h[r, c] != 0.0:
                out.append((r, c, float(h[r, c])))
    return out


def build_model(name, **params):
    """Return (d, I2K, h) for 'xxz' (U(1), QN=[0]), 'fhub' (U(1)xU(1), QN=[2,0]), 'bhub' (U(1), n
    bosons per cell, d levels per site), 'qim' (Z(2)) or 'potts' (Z(q)), all with N = 2 sites per
    unit cell."""
    if name == "xxz":
        return 2, xxz_i2k(2, (0,)), xxz_h(params.get("J", 1.0), params.get("Delta", -1.0), params.get("hz", 0.0))
    if name == "fhub":
        return 4, fhub_i2k(2, (2, 0)), fhub_h(params.get("t", 1.0), params.get("U", 4.0), params.get("V", 0.0),
                                              params.get("mu", 0.0), params.get("hz", 0.0))
    if name == "qim":
        return 2, qim_i2k(), qim_h(params.get("J", 1.0), params.get("h", 1.0))
    if name == "potts":
        q = int(params.get("q", 3))
        return q, potts_i2k(q), potts_h(q, params.get("h", 1.0))
    if name == "bhub":
        d = int(params.get("d", 4))
        return d, bhub_i2k(2, (int(params.get("n", 2)),), d), bhub_h(d, params.get("t", 1.0), params.get("U", 4.0),
                                                                      params.get("mu", 0.0))
    raise ValueError(f"unknown model {name}")
