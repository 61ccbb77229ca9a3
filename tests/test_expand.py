"""ExpandFromH (MPSBlockUtilities.hpp:409-601) on the CPU.

* The oracle's restatement keeps what the reference's construction guarantees: AL stays
  left-isometric and AR right-isometric, AL C AR is unchanged (C is padded with zeros), at
  most dmmax states are added and they carry the largest singular values, and new charges
  enter the bond.
* The host side of the device version (imps_cpp_tools_gb300/expand.py: sector bookkeeping and
  the grouped-GEMM program tables) executed by a numpy interpreter of the program tables, with
  numpy stand-ins for the device plans, null spaces and SVD, against the oracle: same states
  added per charge and the same new directions (the two-site tensor AL' W AR' with W the new
  singular values on the new states is independent of the null-space basis and of the signs of
  singular vectors).
"""
import numpy as np
import pytest
import torch

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import expand as E
from imps_cpp_tools_gb300 import models
from oracle import imps_oracle as O

FHUB0 = {(0, 0): 3, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2, (2, 0): 1, (0, 2): 1, (-2, 0): 1, (0, -2): 1}


def _state(model, seed):
    params = {"J": 1.0, "Delta": -1.0} if model == "xxz" else {"t": 1.0, "U": 4.0}
    d, I2K, h = models.build_model(model, **params)
    dims0 = {(-2,): 2, (0,): 3, (2,): 2} if model == "xxz" else FHUB0
    dimvec = models.make_dims(dims0, 2, I2K)
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, np.random.default_rng(seed))
    # the bond right of site 0: AL(0) (bond 0 -> 1), C right of site 0, AR(1) (bond 1 -> 0)
    return d, I2K, models.h_nonzeros(h), dimvec, AL[0], C[0], AR[1]


def _two_site(AL, C, AR):
    return O.mps_mul_mps(O.mps_mul_bd(AL, C), AR)


def _max_diff(t0, t1):
    err = 0.0
    for a, b in zip(t0, t1):
        for q in set(a) | set(b):
            A = a[q][1] if q in a else 0.0
            Bm = b[q][1] if q in b else 0.0
            err = max(err, float(np.abs(A - Bm).max()))
    return err


@pytest.mark.parametrize("model", ["xxz", "fhub"])
@pytest.mark.parametrize("dmmax", [3, 20, 500])
def test_oracle_expansion_invariants(model, dmmax):
    d, I2K, hnnz, dimvec, AL, C, AR = _state(model, 3)
    ALn, ARn, Cn, dm = O.ExpandFromH(hnnz, I2K, AL, AR, C, dmmax)
    added = sum(dm.values())
    assert 0 < added <= dmmax
    for q, G in O.GetDenseMat(ALn, "l").items():
        assert np.allclose(G[0].T @ G[0], np.eye(G[0].shape[1]), atol=1e-12)
    for q, G in O.GetDenseMat(ARn, "r").items():
        assert np.allclose(G[0] @ G[0].T, np.eye(G[0].shape[0]), atol=1e-12)
    # unchanged up to the summation order of the padded products
    assert _max_diff(_two_site(AL, C, AR), _two_site(ALn, Cn, ARn)) < 1e-13
    for q, m in Cn.items():
        m0 = C[q].shape[0] if q in C else 0
        assert m.shape[0] == m0 + dm.get(q, 0) and not np.any(m[m0:, :]) and not np.any(m[:, m0:])
    assert any(q not in C for q in Cn)  # H reaches charges the bond did not carry


def _getm(v, off, ld, r, c):
    return v[off + np.arange(r)[:, None] + ld * np.arange(c)[None, :]]


def _setm(v, off, ld, M):
    r, c = M.shape
    v[off + np.arange(r)[:, None] + ld * np.arange(c)[None, :]] = M


def _program_run(self, ctx, bufs):
    """The semantics of imps_plan_program: per stage, every output block (slot, off, ld, M, N)
    = sum alpha op(A) op(B) over its terms, outputs of a stage written after all are read."""
    arrs = [b.numpy() for b in bufs]
    for st in self.stages:
        res = []
        for (cs, coff, cld, M, Nn, tl) in st:
            acc = np.zeros((M, Nn))
            for (sa, oa, la, ta, sb, ob, lb, tb, k, al) in tl:
                A = _getm(arrs[sa], oa, la, k, M).T if ta else _getm(arrs[sa], oa, la, M, k)
                Bm = _getm(arrs[sb], ob, lb, Nn, k).T if tb else _getm(arrs[sb], ob, lb, k, Nn)
                acc += al * (A @ Bm)
            res.append((cs, coff, cld, acc))
        for (cs, coff, cld, acc) in res:
            _setm(arrs[cs], coff, max(cld, 1), acc)


class _MulPlan:
    """A * X for an MPS layout and a block-diagonal layout (side 1)."""

    def __init__(self, LA, LC):
        self.LA, self.LC, self.slots = LA, LC, {}

    def bind(self, k, t):
        self.slots[k] = t

    def run(self):
        A, X, out = (self.slots[k].numpy() for k in range(3))
        cb = {b[1]: (o, b[3]) for b, o in zip(self.LC.blocks, self.LC.offsets)}
        for (s, qi, qo, r, c), o in zip(self.LA.blocks, self.LA.offsets):
            co, m = cb[qo]
            _setm(out, o, r, _getm(A, o, r, r, c) @ _getm(X, co, m, m, m))


class _Dec:
    """The tables of a dir-l decomposition plan: sector matrices per outgoing charge (blocks
    stacked in layout order), the null-space layout (block rows x nullity of its sector) and
    the square right-factor layout."""

    def __init__(self, L):
        self.L, self.secs = L, {}
        for i, b in enumerate(L.blocks):
            self.secs.setdefault(b[2], []).append(i)
        ns, rl = [], []
        for q in sorted(self.secs):
            n = L.blocks[self.secs[q][0]][4]
            rl.append((0, q, q, n, n))
        for (g, qi, qo, r, c) in L.blocks:
            nul = sum(L.blocks[i][3] for i in self.secs[qo]) - c
            if nul > 0:
                ns.append((g, qi, qo, r, nul))
        self.nslayout = B.Layout(ns, L.nsym)
        self.rlayout = B.Layout(rl, L.nsym)
        self.nsv = sum(b[3] for b in rl)

    def stacked(self, v, q):
        L = self.L
        return np.vstack([_getm(v, L.offsets[i], L.blocks[i][3], L.blocks[i][3], L.blocks[i][4])
                          for i in self.secs[q]])


def _nullspace(dec, A, NL):
    from scipy.linalg import null_space
    a, out = A.numpy(), NL.numpy()
    for q, ids in dec.secs.items():
        M = dec.stacked(a, q)
        if M.shape[0] <= M.shape[1]:
            continue
        Nn, r0 = null_space(M.T), 0
        for i in ids:
            g, qi, qo, r, c = dec.L.blocks[i]
            _setm(out, dec.nslayout.offsets[dec.nslayout.find(g, qi)], r, Nn[r0:r0 + r])
            r0 += r
    return NL


def _svd(dec, A, U, S, V):
    """imps_sector_svd for a dir-l plan: U in A's layout, S descending, V^T (the reference's
    DiagIso) in the square layout."""
    a, u_, s_, v_ = A.numpy(), U.numpy(), S.numpy(), V.numpy()
    so = 0
    for (g, qi, qo, r, c), o, vo in zip(dec.L.blocks, dec.L.offsets, dec.rlayout.offsets):
        u, s, vt = np.linalg.svd(_getm(a, o, r, r, c), full_matrices=False)
        _setm(u_, o, r, u)
        _setm(v_, vo, c, vt)
        s_[so:so + c] = s
        so += c
    return True


@pytest.fixture
def host_only(monkeypatch):
    monkeypatch.setattr(E, "_zeros", lambda n: torch.zeros(max(int(n), 1), dtype=torch.float64))
    monkeypatch.setattr(E, "_eye", lambda n: torch.eye(max(int(n), 1), dtype=torch.float64).reshape(-1))
    monkeypatch.setattr(E._Program, "run", _program_run)
    monkeypatch.setattr(E.B, "plan_mps_bd", lambda ctx, LA, LC, side: _MulPlan(LA, LC))
    monkeypatch.setattr(E.B, "plan_decomp", lambda ctx, L, direction: _Dec(L))
    monkeypatch.setattr(E.ops, "Nullspace", _nullspace)
    monkeypatch.setattr(E.ops, "svd", _svd)


def _weighted(AL, AR, C, dm, lam):
    """AL W AR with W = diag(0 on the old states, the new singular values on the new ones)."""
    W = {}
    for q, Cq in C.items():
        m, k = Cq.shape[0], dm.get(q, 0)
        w = np.zeros(m)
        if k:
            w[m - k:] = lam[q][:k]
        W[q] = np.diag(w)
    return _two_site(AL, W, AR)


@pytest.mark.parametrize("model", ["xxz", "fhub"])
@pytest.mark.parametrize("dmmax", [3, 30, 500])
def test_device_tables_against_the_oracle(host_only, model, dmmax):
    d, I2K, hnnz, dimvec, AL, C, AR = _state(model, 5)
    LA = B.Layout.mps(I2K, dimvec[0], dimvec[1])
    LR = B.Layout.mps(I2K, dimvec[1], dimvec[0])
    LC = B.Layout.blockdiag(dimvec[1])
    t = lambda v: torch.tensor(v, dtype=torch.float64)
    res = E.expand_from_h(None, I2K, hnnz, LA, t(O.mps_vec(AL)), LR, t(O.mps_vec(AR)), LC, t(O.bd_vec(C)), dmmax)
    ALo, ARo, Co, dmo = O.ExpandFromH(hnnz, I2K, AL, AR, C, dmmax)
    assert {q: k for q, k in res["dm"].items() if k} == {q: k for q, k in dmo.items() if k}
    sizes = lambda L: [[(qi, qo, r, c) for (g, qi, qo, r, c) in L.blocks if g == s] for s in range(d)]
    ALd = O.mps_from_vec(res["AL"].numpy(), sizes(res["LA"]))
    ARd = O.mps_from_vec(res["AR"].numpy(), sizes(res["LR"]))
    Cd = O.bd_from_vec(res["C"].numpy(), [(b[1], b[3]) for b in res["LC"].blocks])
    assert set(Cd) == set(Co) and all(np.array_equal(Cd[q], Co[q]) for q in Co)
    assert _max_diff(_two_site(AL, C, AR), _two_site(ALd, Cd, ARd)) < 1e-13
    err = _max_diff(_weighted(ALd, ARd, Cd, res["dm"], res["lam"]), _weighted(ALo, ARo, Co, dmo, res["lam"]))
    assert err < 1e-12, err
    for q, G in O.GetDenseMat(ALd, "l").items():
        assert np.allclose(G[0].T @ G[0], np.eye(G[0].shape[1]), atol=1e-12)
    for q, G in O.GetDenseMat(ARd, "r").items():
        assert np.allclose(G[0] @ G[0].T, np.eye(G[0].shape[0]), atol=1e-12)


def test_relayout_pads_with_zeros(host_only):
    d, I2K, hnnz, dimvec, AL, C, AR = _state("xxz", 2)
    grown = dict(dimvec[1])
    grown[(-1,)] += 2
    grown[(-3,)] = 1
    old = B.Layout.mps(I2K, dimvec[0], dimvec[1])
    new = B.Layout.mps(I2K, dimvec[0], grown)
    out = E.relayout(None, old, new, torch.tensor(O.mps_vec(AL))).numpy()
    for (g, qi, qo, r, c), o in zip(new.blocks, new.offsets):
        M = _getm(out, o, r, r, c)
        if qi in AL[g]:
            c0 = AL[g][qi][1].shape[1]
            assert np.array_equal(M[:, :c0], AL[g][qi][1]) and not np.any(M[:, c0:])
        else:
            assert not np.any(M)


def test_oracle_vumps_with_bond_expansion():
    """The oracle's VUMPS loop with the reference's expansion branch (VUMPS_main.cpp:270-308):
    from D = 7 per bond, mmax 24, dmmax 8, expansion after every second site update once the
    previous sweep's error is below 1e-5.  The bonds grow to mmax, the state stays a consistent
    mixed-canonical cell, and the energy approaches the Bethe-ansatz value far closer than at
    the starting dimension."""
    import math
    d, I2K, h = models.build_model("xxz", J=1.0, Delta=-1.0)
    dimvec = models.make_dims({(-2,): 2, (0,): 3, (2,): 2}, 2, I2K)
    v = O.VUMPS(O.xxz_h(1.0, -1.0), 2, O.xxz_i2k(2, [0]), dimvec[0], dimvec=dimvec, seed=4, mmax=24, dmmax=8,
                expand_pause=2)
    e7 = None
    for k in range(80):
        E, F, prec = v.sweep()
        if k == 24:
            e7 = float(E.mean())  # converged at D = 7, before the first expansion
            assert v.expansions == 0 and F.max() < 1e-4
        if not v.keep_running(1e-9):
            break
    dims = [sum(M.shape[1] for M in C.values()) for C in v.C]
    e0 = 0.25 - math.log(2)
    assert v.expansions >= 3 and dims == [24, 24]
    assert float(E.mean()) < e7 - 5e-4 and abs(float(E.mean()) - e0) < 5e-5
    # AL(n) C(n) = C(n-1) AR(n) in the reference's arrangement (AR shifted back by one)
    AR = O.shift(v.AR, 1)
    for n in range(2):
        Cr, Cl = v.C[n], v.C[(n - 1) % 2]
        for s in range(d):
            for q, (qo, al) in v.AL[n][s].items():
                assert np.abs(al @ Cr[qo] - Cl[q] @ AR[n][s][q][1]).max() < 1e-5
