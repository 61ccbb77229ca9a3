"""Pinning the CPU oracle (no reference golden vectors exist, see oracle/__init__.py):
dense re-evaluation of every block-sparse contraction, the reference's own inline identities,
and the Bethe-ansatz energy of the Heisenberg chain."""
import math

import numpy as np
import pytest

from imps_cpp_tools_gb300 import models
from oracle import imps_oracle as O
from tests import imps_testlib as T


def _bond_index(dims):
    """global index offsets of a bond: sectors in key order."""
    off, o = {}, 0
    for q in sorted(dims):
        off[q] = o
        o += dims[q]
    return off, o


def _dense_mps(A, dl, dr):
    ol, Dl = _bond_index(dl)
    orr, Dr = _bond_index(dr)
    out = np.zeros((len(A), Dl, Dr))
    for s, bm in enumerate(A):
        for qi, (qo, M) in bm.items():
            out[s, ol[qi]:ol[qi] + M.shape[0], orr[qo]:orr[qo] + M.shape[1]] = M
    return out


def _dense_bd(X, dims):
    o, D = _bond_index(dims)
    out = np.zeros((D, D))
    for q, M in X.items():
        out[o[q]:o[q] + M.shape[0], o[q]:o[q] + M.shape[1]] = M
    return out


@pytest.mark.parametrize("model,dims0", [("xxz", {(-2,): 2, (0,): 3, (2,): 2}),
                                         ("fhub", {(0, 0): 3, (1, 1): 2, (-1, -1): 2, (1, -1): 1, (-1, 1): 1})])
def test_hac_dense(model, dims0):
    """ApplyHA block-sparse == dense einsum with HL/HR built densely from AL/AR and h."""
    p = T.hac_problem(model, dims0, seed=3)
    d, h, AL, AR, C = p["d"], p["h"], p["AL"], p["AR"], p["C"]
    dv = p["dimvec"]
    out = O.ApplyHA(p["AC"], p["EHL"], p["EHR"], p["HL"], p["HR"])
    # dense: AC lives on bond1 -> bond0 (site 1 of the cell, AR[0] in shifted layout is site n)
    # here AC = C[1] * AR[0]: C[1] on bond0 (right of AL[1]); AR[0] maps bond0 -> bond1
    b0, b1 = dv[0], dv[1]
    ACd = _dense_mps(p["AC"], b0, b1)
    ALd = _dense_mps(AL[1], b1, b0)  # AL[1]: bond1 -> bond0
    ARd = _dense_mps(AR[1], b1, b0)  # AR[1]: bond1 -> bond0
    EHLd, EHRd = _dense_bd(p["EHL"], b0), _dense_bd(p["EHR"], b1)
    H4 = h.reshape(d, d, d, d)  # [i0,i1,j0,j1]
    HLd = np.einsum("abcd,aij,cik->bdjk", H4, ALd, ALd)   # HL[i1][j1] = sum h AL[i0]^T AL[j0]
    HRd = np.einsum("abcd,dij,bkj->acik", H4, ARd, ARd)   # HR[i0][j0] = sum h AR[j1] AR[i1]^T
    ref = (np.einsum("ij,sjk->sik", EHLd, ACd) + np.einsum("sij,jk->sik", ACd, EHRd)
           + np.einsum("stij,tjk->sik", HLd, ACd) + np.einsum("tij,stjk->sik", ACd, HRd))
    got = _dense_mps(out, b0, b1)
    # only sectors present in AC are produced by the reference's buffer-backed out
    mask = _dense_mps([{q: (qo, np.ones_like(M)) for q, (qo, M) in bm.items()} for bm in p["AC"]], b0, b1)
    np.testing.assert_allclose(got, ref * mask, rtol=0, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("model,dims0", [("xxz", {(-2,): 2, (0,): 3, (2,): 2}),
                                         ("fhub", {(0, 0): 3, (1, 1): 2, (-1, -1): 2})])
def test_tm_dense(model, dims0):
    st = T.random_state(model, dims0, seed=5)
    AL, dv = st["AL"], st["dimvec"]
    X = T.rand_bd(dv[0], st["rng"], sym=False)
    got = O.ApplyTMLeftUC(AL, X)
    A0, A1 = _dense_mps(AL[0], dv[0], dv[1]), _dense_mps(AL[1], dv[1], dv[0])
    Xd = _dense_bd(X, dv[0])
    Y = np.einsum("sji,jk,skl->il", A0, Xd, A0)
    Y = np.einsum("sji,jk,skl->il", A1, Y, A1)
    np.testing.assert_allclose(_dense_bd(got, dv[0]), Y, atol=1e-12 * np.abs(Y).max())
    got = O.ApplyTMRightUC(AL, X)
    Y = np.einsum("sij,jk,slk->il", A1, Xd, A1)
    Y = np.einsum("sij,jk,slk->il", A0, Y, A0)
    np.testing.assert_allclose(_dense_bd(got, dv[0]), Y, atol=1e-12 * np.abs(Y).max())


def test_hc_literal_equals_grouped():
    """The literal per-nonzero chain of ApplyHC equals the (i1,j1)-grouped form used on the GPU."""
    st = T.random_state("fhub", {(0, 0): 3, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2}, seed=2)
    d, hnnz, AL, AR, C, rng = st["d"], st["hnnz"], st["AL"], st["AR"], st["C"], st["rng"]
    Cin = T.rand_bd({q: m.shape[0] for q, m in C[1].items()}, rng, sym=False)
    EHL = T.rand_bd({q: m.shape[0] for q, m in C[1].items()}, rng)
    EHR = T.rand_bd({q: m.shape[0] for q, m in C[1].items()}, rng)
    lit = O.ApplyHC(Cin, EHL, EHR, hnnz, d, AL[1], AR[0])
    HLp = O.ReducedOp(hnnz, AL[1], d, "l")
    grp = O.bd_add(O.bd_mul(EHL, Cin), O.bd_mul(Cin, EHR))
    for i1 in range(d):
        for j1 in range(d):
            if not HLp[i1][j1]:
                continue
            Rr = O.bm_mul(AR[0][j1], O.bm_t(AR[0][i1]))
            X = O.bm_mul(O.bm_mul(HLp[i1][j1], {q: (q, M) for q, M in Cin.items()}), Rr)
            for q, (qo, M) in X.items():
                assert q == qo
                grp[q] = grp[q] + M
    for q in lit:
        np.testing.assert_allclose(lit[q], grp[q], atol=1e-12)


def test_inverte_identity():
    """Excitations_helpers.hpp:828-913 (teststuff): y - T(y) + tr(y R) L = x - tr(x R) L."""
    st = T.random_state("xxz", {(-2,): 2, (0,): 4, (2,): 2}, seed=7)
    AL, C, rng = st["AL"], st["C"], st["rng"]
    _, R = O.TMDominantEig(AL, st["dimvec"][0], "r", 1e-14)
    L = O.bd_eye(st["dimvec"][0])
    x = T.rand_bd(st["dimvec"][0], rng)
    y, flag = O.InvertE_proj(AL, x, L, R, "l", 1e-13)
    assert flag > 0
    lhs = O.bd_add(O.bd_add(y, {q: -M for q, M in O.ApplyTMLeftUC(AL, y).items()}),
                   {q: O.bd_trace(O.bd_mul(y, R)) * M for q, M in L.items()})
    rhs = O.bd_add(x, {q: -O.bd_trace(O.bd_mul(x, R)) * M for q, M in L.items()})
    for q in lhs:
        np.testing.assert_allclose(lhs[q], rhs[q], atol=1e-11)


def test_canonical_forms():
    """randMPS_LR invariants: AL^T AL = 1 per sector, AR AR^T = 1, AL[n] C[n] = C[n-1] AR[n]."""
    st = T.random_state("fhub", {(0, 0): 4, (1, 1): 2, (-1, -1): 2, (2, 0): 1, (0, 2): 1}, seed=1)
    AL, AR, C = st["AL"], st["AR"], st["C"]
    for A in AL:
        X = O.ApplyTMLeft(A, O.bd_eye({q: M.shape[0] for bm in A for q, (_, M) in bm.items()}))
        for q, M in X.items():
            np.testing.assert_allclose(M, np.eye(M.shape[0]), atol=1e-12)
    for A in AR:
        X = O.ApplyTMRight(A, O.bd_eye({qo: M.shape[1] for bm in A for _, (qo, M) in bm.items()}))
        for q, M in X.items():
            np.testing.assert_allclose(M, np.eye(M.shape[0]), atol=1e-12)
    for n in range(2):
        lhs = O.mps_mul_bd(AL[n], C[n])
        rhs = O.bd_mul_mps(C[n - 1], AR[n])
        assert O.mps_norm_inf(O.mps_sub(lhs, rhs)) < 1e-10


def test_i2k_and_dims_match_reference_rules():
    assert models.xxz_i2k(2, (0,)) == O.xxz_i2k(2, [0]) == [(1,), (-1,)]
    assert models.fhub_i2k(2, (2, 0)) == O.fhub_i2k(2, [2, 0]) == [(-1, 0), (0, -1), (0, 1), (1, 0)]
    assert models.validpath(2, [(1,), (-1,)]) == [1, 0]
    assert models.validpath(2, [(-1, 0), (0, -1), (0, 1), (1, 0)]) == [3, 0]
    d0 = {(0,): 3, (2,): 1}
    assert models.make_dims(d0, 2, [(1,), (-1,)]) == O.make_dims(d0, 2, [(1,), (-1,)])
    assert models.h_nonzeros(models.xxz_h(1, -1)) == O.sparse_nnz(O.xxz_h(1, -1))
    assert len(models.h_nonzeros(models.xxz_h(1, -1))) == 6
    assert models.h_nonzeros(models.fhub_h(1, 4)) == O.sparse_nnz(O.fhub_h(1, 4))


@pytest.mark.slow
def test_heisenberg_bethe_ansatz():
    """VUMPS (oracle) on the isotropic AFM Heisenberg chain, reference sign convention
    (J=1, Delta=-1, Models.cpp:91), approaches e0 = 1/4 - ln 2 (Bethe ansatz)."""
    b0 = {(-4,): 3, (-2,): 8, (0,): 10, (2,): 8, (4,): 3}
    b1 = {(-5,): 1, (-3,): 5, (-1,): 10, (1,): 10, (3,): 5, (5,): 1}
    h = O.xxz_h(1.0, -1.0)
    I2K = O.xxz_i2k(2, [0])
    orig = O.make_dims
    O.make_dims = lambda dmap0, N, I2K: [b0, b1]
    try:
        v = O.VUMPS(h, 2, I2K, b0, seed=3)
    finally:
        O.make_dims = orig
    for _ in range(14):
        E, F, prec = v.sweep()
    e0 = 0.25 - math.log(2)
    assert abs(E.mean() - e0) < 2e-4
    assert F.max() < 1e-3


def test_bose_hubbard_model():
    """BoseHubbardModel (Models.cpp:739-862): the package's h, I2K and GetObservables against
    the oracle's element-wise restatement; h conserves the boson number; and the oracle's VUMPS
    at unit filling (n = 2 per two-site cell) in the Mott regime follows strong-coupling
    perturbation theory, e0 = -4 t^2 / U + O(t^4 / U^3): the remainder scales as t^4."""
    for d in (3, 4, 5):
        assert np.array_equal(models.bhub_h(d, 0.7, 3.0, 0.4), O.bhub_h(d, 0.7, 3.0, 0.4))
        assert models.bhub_i2k(2, (2,), d) == O.bhub_i2k(2, [2], d)
    d, I2K, h = models.build_model("bhub", d=4, t=0.3, U=2.0, n=2)
    q = [tuple(a + b for a, b in zip(I2K[s1], I2K[s2])) for s1 in range(d) for s2 in range(d)]
    assert all(q[r] == q[c] for r in range(d * d) for c in range(d * d) if h[r, c] != 0.0)
    names = [n for n, _ in models.observables("bhub", ["b", "b2", "n", "nmax"], d=4)]
    assert names == ["b", "b2", "n", "nmax"]
    rem = []
    for t in (0.05, 0.1):
        bd = {(-2,): 1, (-1,): 3, (0,): 4, (1,): 3, (2,): 1}
        v = O.VUMPS(O.bhub_h(4, t, 1.0, 0.0), 4, O.bhub_i2k(2, [2], 4), bd, dimvec=[bd, bd], seed=2)
        for _ in range(40):
            E, F, _ = v.sweep()
            if F.max() < 1e-10:
                break
        assert F.max() < 1e-9 and abs(E[0] - E[1]) < 1e-9
        rem.append(E.mean() + 4 * t * t)
    assert 0 < rem[0] < 5e-5
    assert 14.0 < rem[1] / rem[0] < 18.0


def test_zn_models():
    """Quantum Ising (Z(2)) and quantum Potts (Z(q)) (Models.cpp:323-504): the package's h and
    I2K against the oracle's element-wise restatement, charge conservation modulo N, and the
    oracle's VUMPS with the Z(N) charge arithmetic (symobj.hpp:120-158):
    * quantum Ising -J sx sx - h/2 (sz 1 + 1 sz) at the exact transverse-field Ising energy
      e0 = -(1/2pi) int sqrt(J'^2 + h'^2 - 2 J' h' cos k) dk, J' = J/4, h' = h/2;
    * Potts q = 3 deep in the field-polarised phase on strong-field perturbation theory,
      e0 = -h(q-1) - (q-1)/(2hq) - 1/(18 h^2) + O(h^-3) (the h^-2 term: three shifts by the
      same bond term return to |0 0>, X^3 = 1)."""
    from scipy.integrate import quad
    from imps_cpp_tools_gb300 import charges
    assert np.array_equal(models.qim_h(0.7, 1.3), O.qim_h(0.7, 1.3))
    assert list(models.qim_i2k()) == O.qim_i2k() and models.qim_i2k().periods == (2,)
    for q in (2, 3, 4, 5):
        assert np.array_equal(models.potts_h(q, 0.6), O.potts_h(q, 0.6))
        assert list(models.potts_i2k(q)) == O.potts_i2k(q)
    for name, kw in (("qim", {}), ("potts", {"q": 3}), ("potts", {"q": 4})):
        d, I2K, h = models.build_model(name, **kw)
        per = charges.periods_of(I2K)
        qq = [charges.add(I2K[a], I2K[b], per) for a in range(d) for b in range(d)]
        assert all(qq[r] == qq[c] for r in range(d * d) for c in range(d * d) if h[r, c] != 0.0)
    J, hf = 1.0, 0.7
    Jp, hp = J / 4, hf / 2
    e0 = -quad(lambda k: math.sqrt(Jp ** 2 + hp ** 2 - 2 * Jp * hp * math.cos(k)), -math.pi, math.pi,
               epsabs=1e-14)[0] / (2 * math.pi)
    with O.charge_group((2,)):
        v = O.VUMPS(O.qim_h(J, hf), 2, O.qim_i2k(), {(0,): 8, (1,): 8}, seed=2)
        for _ in range(60):
            E, F, _ = v.sweep()
            if F.max() < 1e-11:
                break
    assert F.max() < 1e-10 and np.abs(E - e0).max() < 1e-11
    for hq, tol in ((10.0, 5e-5), (20.0, 1e-5)):
        with O.charge_group((3,)):
            v = O.VUMPS(O.potts_h(3, hq), 3, O.potts_i2k(3), {(0,): 4, (1,): 2, (2,): 2}, seed=2)
            for _ in range(60):
                E, F, _ = v.sweep()
                if F.max() < 1e-11:
                    break
        pt = -2 * hq - 2 / (6 * hq) - 1 / (18 * hq * hq)
        assert F.max() < 1e-10 and abs(E.mean() - pt) < tol, (hq, E, pt)


def _zn_run(model, params, dims, periods, warm, pert, sweeps):
    """The oracle's VUMPS from randMPS_LR(7) after `warm` sweeps, C of bond 1 scaled by
    (1 + pert), then `sweeps` sweeps; returns the energies."""
    import copy
    d, I2K, h = models.build_model(model, **params)
    with O.charge_group(periods):
        dimvec = models.make_dims(dims, 2, I2K)
        AL, AR, C = O.randMPS_LR(2, I2K, dimvec, np.random.default_rng(7))
        if warm:
            o = O.VUMPS(h, d, I2K, dimvec[0], dimvec=dimvec, init=(AL, AR, C), fixed_tol=1e-12, seed=7)
            for _ in range(warm):
                o.sweep()
            AL, AR, C = copy.deepcopy(o.AL), O.shift(copy.deepcopy(o.AR), 1), copy.deepcopy(o.C)
        C[0] = {q: M * (1.0 + pert) for q, M in C[0].items()}
        o = O.VUMPS(h, d, I2K, dimvec[0], dimvec=dimvec, init=(AL, AR, C), fixed_tol=1e-12, seed=7)
        return np.array([o.sweep()[0] for _ in range(sweeps)])


def test_vumps_transient_is_chaotic():
    """Why the sweep-parity tests start from a few sweeps on: in the oracle alone, a relative
    change of 1e-13 of the random start state (transverse-field Ising, Z(2) sectors 6 + 6,
    J = 1, h = 0.7) moves the energies of sweep 1 by more than 1e-5 (measured 3e-4); from the
    state after 5 sweeps the same change stays below 1e-11 (measured 4e-13).  So two correct
    eigensolvers at tol 1e-12 (ARPACK, the device Lanczos) cannot agree on the first sweeps
    from a random state, and agree to the rounding level once the iteration contracts."""
    args = ("qim", {"J": 1.0, "h": 0.7}, {(0,): 6, (1,): 6}, (2,))
    a, b = _zn_run(*args, 0, 0.0, 2), _zn_run(*args, 0, 1e-13, 2)
    assert np.abs(a[1] - b[1]).max() > 1e-5
    a, b = _zn_run(*args, 5, 0.0, 3), _zn_run(*args, 5, 1e-13, 3)
    assert np.abs(a - b).max() < 1e-11


@pytest.mark.parametrize("N", [3, 4])
def test_oracle_vumps_longer_unit_cells(N):
    """The reference's VUMPS takes any unit-cell length N >= 2 (VUMPS_main.cpp:31,55-56; its site
    loop rotates the unit-cell arrays, :256-259); the oracle follows it for any N.  At N = 3 and 4
    the quantum Ising chain (Z(2) charges, J = 1, h = 0.7) reaches the exact transverse-field
    Ising energy on every bond."""
    from scipy.integrate import quad
    J, hf = 1.0, 0.7
    Jp, hp = J / 4, hf / 2
    e0 = -quad(lambda k: math.sqrt(Jp ** 2 + hp ** 2 - 2 * Jp * hp * math.cos(k)), -math.pi, math.pi,
               epsabs=1e-14)[0] / (2 * math.pi)
    with O.charge_group((2,)):
        v = O.VUMPS(O.qim_h(J, hf), 2, O.qim_i2k(), {(0,): 8, (1,): 8}, N=N, seed=2)
        for _ in range(60):
            E, F, _ = v.sweep()
            if F.max() < 1e-11:
                break
    assert len(E) == N and F.max() < 1e-10 and np.abs(E - e0).max() < 1e-11
