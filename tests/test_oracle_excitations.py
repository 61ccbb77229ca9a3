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


def excitation_setup(K, seed=3, dims0=None):
    """A random left/right-canonical two-site XXZ state (the oracle's randMPS_LR), h shifted by
    its energy density E0, its environments (HeffConstants) and null spaces, and the X sector
    structure for charge K."""
    from imps_cpp_tools_gb300 import models
    st = T.random_state("xxz", dims0 or B0, seed=seed, J=1.0, Delta=-1.0)
    AL, AR, C, d = st["AL"], st["AR"], st["C"], st["d"]
    C0 = C[-1]  # bond 0
    R = O.bd_mul(C0, O.bd_t(C0))
    L = O.bd_mul(O.bd_t(C0), C0)
    _, _, h = models.build_model("xxz", J=1.0, Delta=-1.0)
    hn = O.sparse_nnz(h)
    HL0 = O.ApplyOpTMLeftDiag(hn, O.mps_mul_mps(AL[1], AL[0]))
    HL1 = O.bd_add(O.ApplyOpTMLeftDiag(hn, O.mps_mul_mps(AL[0], AL[1])), O.ApplyTMLeft(AL[1], HL0))
    E0 = O.bd_trace(O.bd_mul(HL1, R)) / 2
    hs = O.sparse_nnz(h - E0 * np.eye(h.shape[0]))
    HLtot, HRtot = O.HeffConstants(AL, AR, L, R, hs, tol=1e-13)
    NL = [O.Nullspace(AL[n], "l") for n in range(2)]
    xd = O.XDims(NL, AR, K)
    return dict(AL=AL, AR=AR, NL=NL, d=d, h=hs, HLtot=HLtot, HRtot=HRtot, xdims=xd, E0=E0)


def rand_x(xdims, rng):
    return [{qi: (qo, rng.standard_normal((ml, mr)) + 1j * rng.standard_normal((ml, mr)))
             for (qi, qo, ml, mr) in dims} for dims in xdims]


def x_inner(X, Y, xdims):
    return sum(np.vdot(X[n][qi][1], Y[n][qi][1]) for n, dims in enumerate(xdims) for (qi, _, _, _) in dims)


@pytest.mark.parametrize("K,p", [((2,), 0.6), ((-2,), 2.4)])
def test_heff_is_hermitian(K, p):
    """The excitation effective Hamiltonian (with E0 subtracted and exact environments) is
    Hermitian in the X inner product: <Y, H X> = <H Y, X>."""
    e = excitation_setup(K)
    rng = np.random.default_rng(11)
    X, Y = rand_x(e["xdims"], rng), rand_x(e["xdims"], rng)
    kfac = np.exp(1j * p)
    args = (kfac, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"])
    HX = O.ApplyHeff(X, *args, tol=1e-13)
    HY = O.ApplyHeff(Y, *args, tol=1e-13)
    a, b = x_inner(Y, HX, e["xdims"]), x_inner(HY, X, e["xdims"])
    assert abs(a - b) < 1e-10 * abs(a), (a, b)


def run_tables(stages, bufs):
    """Execute grouped-GEMM program stages with numpy (the device engine's semantics)."""
    def mat(slot, off, ld, rows, cols):
        idx = off + np.arange(rows)[:, None] + np.arange(cols)[None, :] * ld
        return bufs[slot][idx]
    for stage in stages:
        res = []
        for (cs, coff, cld, M, Nn, acc, tl) in stage:
            Cm = np.zeros((M, Nn))
            for (sa, oa, la, ta, sb, ob, lb, tb, k, alpha) in tl:
                A = mat(sa, oa, la, k, M).T if ta else mat(sa, oa, la, M, k)
                Bm = mat(sb, ob, lb, Nn, k).T if tb else mat(sb, ob, lb, k, Nn)
                Cm += alpha * (A @ Bm)
            res.append((cs, coff, cld, M, Nn, acc, Cm))
        for (cs, coff, cld, M, Nn, acc, Cm) in res:
            if M and Nn:
                idx = coff + np.arange(M)[:, None] + np.arange(Nn)[None, :] * cld
                bufs[cs][idx] = bufs[cs][idx] + Cm if acc else Cm


@pytest.mark.parametrize("K,p", [((2,), 0.6), ((-2,), 2.4)])
@pytest.mark.parametrize("which", ["h", "sz"])
def test_heff_program_tables_match_oracle(K, p, which):
    """The host compilation of ApplyHeff (imps_cpp_tools_gb300.excitations.HeffProgram), executed
    table by table with numpy and the oracle's InvertE_fac for the two solves, reproduces the
    oracle's ApplyHeff: a check of the sector matching and term expansion without a GPU.  With
    which = "sz" the two-site operator is the bond form of the one-site sz (mean subtracted),
    as measure_excitations compiles it; its result is also -K/2 times X exactly."""
    from imps_cpp_tools_gb300 import excitations as EX
    e = excitation_setup(K)
    if which == "sz":
        _, _, _, _, hn, HLs, HRs = _opeff_setup(K)
        e = dict(e, h=hn, HLtot=HLs, HRtot=HRs)
    kfac = np.exp(1j * p)
    pr = EX.HeffProgram(e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"], kfac)
    bufs = {k: np.zeros(max(int(pr.sizes.get(k, 0)), 1)) for k in range(6)}
    bufs[EX.OPS][:pr.ops_vec.size] = pr.ops_vec
    X = rand_x(e["xdims"], np.random.default_rng(12))
    for (xo, n), x in zip(pr.xoff, X):
        v = O.bm_vec(x)
        bufs[EX.XS][xo:xo + n], bufs[EX.XS][xo + n:xo + 2 * n] = v.real, v.imag
    run_tables(pr.prog_a.stages, bufs)

    def to_bm(t_re, t_im, slot):
        return {k[1]: (qo, (bufs[slot][o1:o1 + r * c] + 1j * bufs[slot][t_im.blocks[k][3]:t_im.blocks[k][3] + r * c])
                       .reshape(c, r).T) for k, (qo, r, c, o1) in t_re.blocks.items()}

    xr, xl = to_bm(*pr.rhs_r, EX.RHS), to_bm(*pr.rhs_l, EX.RHS)
    yr, _ = O.InvertE_fac(e["AL"], e["AR"], xr, "r", kfac, tol=1e-13)
    yl, _ = O.InvertE_fac(e["AR"], e["AL"], xl, "l", np.conj(kfac), tol=1e-13)
    vr, vl = O.bm_vec(yr), O.bm_vec(yl)
    nr, nl = pr.nr, pr.nl
    bufs[EX.ES][:nr], bufs[EX.ES][nr:2 * nr] = vr.real, vr.imag
    bufs[EX.ES][2 * nr:2 * nr + nl], bufs[EX.ES][2 * nr + nl:2 * nr + 2 * nl] = vl.real, vl.imag
    run_tables(pr.prog_b.stages, bufs)
    ref = O.ApplyHeff(X, kfac, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"], tol=1e-13)
    for n, ((xo, nn), dims) in enumerate(zip(pr.xoff, e["xdims"])):
        got = bufs[EX.OUT][xo:xo + nn] + 1j * bufs[EX.OUT][xo + nn:xo + 2 * nn]
        refv = np.concatenate([ref[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims])
        assert np.linalg.norm(got - refv) / np.linalg.norm(refv) < 1e-9, n
        if which == "sz":
            xv = np.concatenate([X[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims])
            assert np.linalg.norm(got - (-K[0] / 2) * xv) < 1e-9 * np.linalg.norm(xv), n


def test_lroverlaps_dominant_eigenmatrices(state):
    """LRoverlaps at K = 0 (Excitations_helpers.hpp:915-946): for AL C = C AR the dominant left
    and right eigenmatrices of the mixed TM of AL and AR are C^T and C (bond 0), overlap 1; the
    eigen-relations hold for the oracle's ARPACK eigenpairs."""
    AL, AR, C0 = state["AL"], state["AR"], state["C"][-1]
    LM, RM, OL, OLLv, OLRv = O.LRoverlaps(AL, AR, (0,), 3)
    assert abs(abs(OL) - 1.0) < 1e-12 and abs(OLLv[0].imag) < 1e-12 and abs(OLRv[0].imag) < 1e-12
    assert np.all(np.abs(OLLv[1:]) <= np.abs(OLLv[0]) + 1e-12)
    res_l = O.bm_add(O.ApplyTMmixedLeftUC(AL, AR, LM), O.bm_scale(LM, -OLLv[0].real))
    res_r = O.bm_add(O.ApplyTMmixedRightUC(AL, AR, RM), O.bm_scale(RM, -OLRv[0].real))
    assert np.linalg.norm(O.bm_vec(res_l)) < 1e-12 and np.linalg.norm(O.bm_vec(res_r)) < 1e-12
    Cm = {q: (q, M) for q, M in C0.items()}
    for X, ref in [(LM, O.bm_t(Cm)), (RM, Cm)]:
        a, b = O.bm_vec(X), O.bm_vec(ref)
        assert abs(abs(a @ b) - np.linalg.norm(a) * np.linalg.norm(b)) < 1e-11


def test_lroverlaps_charge_offset_sectors(state):
    """K != 0: the left problem runs in sector -K, the right one in K; sizes follow XDims-style
    pairing (q, q + K) and the leading overlaps are below 1 in modulus."""
    AL, AR = state["AL"], state["AR"]
    vl, VL, sl = O.TMmixedEigs(AL, AR, "l", (-2,), 2, "LM", 1e-13)
    vr, VR, sr = O.TMmixedEigs(AL, AR, "r", (2,), 2, "LM", 1e-13)
    assert all(qo == (q[0] - 2,) for (q, qo, _, _) in sl) and all(qo == (q[0] + 2,) for (q, qo, _, _) in sr)
    assert abs(vl[0]) < 1 - 1e-6 and abs(abs(vl[0]) - abs(vr[0])) < 1e-10


def test_projected_heff_is_hermitian():
    """p = 0, K = 0: ApplyHeff with the projected environment solves (LM, RM from LRoverlaps) is
    Hermitian in the X inner product."""
    e = excitation_setup((0,))
    LM, RM, OL, _, _ = O.LRoverlaps(e["AL"], e["AR"], (0,), 2)
    assert OL > 0
    rng = np.random.default_rng(5)
    X, Y = rand_x(e["xdims"], rng), rand_x(e["xdims"], rng)
    args = (1.0 + 0j, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"])
    HX = O.ApplyHeff(X, *args, LM=LM, RM=RM, tol=1e-13)
    HY = O.ApplyHeff(Y, *args, LM=LM, RM=RM, tol=1e-13)
    a, b = x_inner(Y, HX, e["xdims"]), x_inner(HY, X, e["xdims"])
    assert abs(a - b) < 1e-10 * abs(a), (a, b)


def _opeff_setup(K):
    """The excitation setup with the one-site sz, its mean subtracted, in both forms: the
    reference's OPeffConstants (Excitations_helpers.hpp:548-606) and the bond operator
    (sz x 1 + 1 x sz) / 2 with HeffConstants."""
    e = excitation_setup(K)
    st = T.random_state("xxz", B0, seed=3, J=1.0, Delta=-1.0)
    C = st["C"]
    R, L = O.bd_mul(C[-1], O.bd_t(C[-1])), O.bd_mul(O.bd_t(C[-1]), C[-1])
    Lb = [O.bd_mul(O.bd_t(C[0]), C[0]), L]  # left of site 1, left of site 0
    sz = np.diag([0.5, -0.5])
    eobs = float(np.mean(O.MeasureObservables([("sz", sz)], e["AR"], Lb)["sz"]))
    onnz = O.sparse_nnz(sz - eobs * np.eye(2))
    OPL, OPR = O.OPeffConstants(e["AL"], e["AR"], L, R, onnz, tol=1e-13)
    hn = O.sparse_nnz(0.5 * (np.kron(sz, np.eye(2)) + np.kron(np.eye(2), sz)) - eobs * np.eye(4))
    HL, HR = O.HeffConstants(e["AL"], e["AR"], L, R, hn, tol=1e-13)
    return e, onnz, OPL, OPR, hn, HL, HR


@pytest.mark.parametrize("K,p,proj", [((2,), 0.6, False), ((-2,), 2.4, False), ((0,), 0.0, True)])
def test_opeff_is_the_bond_form_of_heff(K, p, proj):
    """ApplyOPeff (Excitations_helpers.hpp:350-545) with a one-site O equals ApplyHeff with the
    two-site (O x 1 + 1 x O) / 2 (the same operator on the infinite chain), which is how the
    device evaluates MeasureExcitations; and for O = sz the excitation-space operator is the
    sector's Sz shift times the identity (K = +-2 in label units: -+1), exactly."""
    e, onnz, OPL, OPR, hn, HL, HR = _opeff_setup(K)
    LM = RM = None
    if proj:
        LM, RM, _, _, _ = O.LRoverlaps(e["AL"], e["AR"], K, 2)
    X = rand_x(e["xdims"], np.random.default_rng(7))
    kfac = np.exp(1j * p)
    XO = O.ApplyOPeff(X, kfac, e["AL"], e["AR"], e["NL"], onnz, OPL, OPR, LM=LM, RM=RM, tol=1e-13)
    XH = O.ApplyHeff(X, kfac, e["AL"], e["AR"], e["NL"], hn, 2, HL, HR, LM=LM, RM=RM, tol=1e-13)
    c = -K[0] / 2
    for n, dims in enumerate(e["xdims"]):
        for (q, _, _, _) in dims:
            assert np.abs(XO[n][q][1] - XH[n][q][1]).max() < 1e-11
            assert np.abs(XO[n][q][1] - c * X[n][q][1]).max() < 1e-11


def _ising_setup(J=1.0, h=1.0):
    """A converged transverse-field Ising ground state (Z(2) charges, D = 8 + 8) and its
    excitation inputs for the odd sector K = 1; call inside O.charge_group((2,))."""
    H = O.qim_h(J, h)
    v = O.VUMPS(H, 2, O.qim_i2k(), {(0,): 8, (1,): 8}, seed=2)
    for _ in range(80):
        E, F, _ = v.sweep()
        if F.max() < 1e-12:
            break
    AL, AR, C0 = v.AL, O.shift(v.AR, 1), v.C[-1]
    R, L = O.bd_mul(C0, O.bd_t(C0)), O.bd_mul(O.bd_t(C0), C0)
    hs = O.sparse_nnz(H - float(E.mean()) * np.eye(4))
    K = (1,)
    _, _, OL, _, _ = O.LRoverlaps(AL, AR, K, 2)
    if OL < 0:  # Excitations_main.cpp:177-178
        AR = [[{q: (qo, -M) for q, (qo, M) in bm.items()} for bm in AR[0]], AR[1]]
    HL, HR = O.HeffConstants(AL, AR, L, R, hs, tol=1e-13)
    NL = [O.Nullspace(AL[n], "l") for n in range(2)]
    return dict(AL=AL, AR=AR, NL=NL, h=hs, HLtot=HL, HRtot=HR, xdims=O.XDims(NL, AR, K), d=2, K=K)


def test_ising_tables_and_xdims():
    """The device path's host side with Z(2) charges: XDims from the layouts with the group's
    modular arithmetic (excitations.xdims_from_layouts) equals the oracle's, and the H_eff
    program tables, run with numpy, reproduce the oracle's ApplyHeff."""
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300 import excitations as EX
    with O.charge_group((2,)):
        e = _ising_setup()
        lay = lambda A: B.Layout([(s, qi, bm[qi][0], bm[qi][1].shape[0], bm[qi][1].shape[1])
                                  for s, bm in enumerate(A) for qi in sorted(bm)], 1)
        for n in range(2):
            got = EX.xdims_from_layouts(lay(e["NL"][n]), lay(e["AR"][(n + 1) % 2]), e["K"], (2,))
            assert got == e["xdims"][n]
        kfac = np.exp(0.9j)
        pr = EX.HeffProgram(e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], 2, e["xdims"], kfac)
        bufs = {k: np.zeros(max(int(pr.sizes.get(k, 0)), 1)) for k in range(6)}
        bufs[EX.OPS][:pr.ops_vec.size] = pr.ops_vec
        X = rand_x(e["xdims"], np.random.default_rng(4))
        for (xo, nn), x in zip(pr.xoff, X):
            vv = O.bm_vec(x)
            bufs[EX.XS][xo:xo + nn], bufs[EX.XS][xo + nn:xo + 2 * nn] = vv.real, vv.imag
        run_tables(pr.prog_a.stages, bufs)

        def to_bm(t_re, t_im, slot):
            return {k[1]: (qo, (bufs[slot][o1:o1 + r * c] + 1j * bufs[slot][t_im.blocks[k][3]:t_im.blocks[k][3] + r * c])
                           .reshape(c, r).T) for k, (qo, r, c, o1) in t_re.blocks.items()}

        yr, _ = O.InvertE_fac(e["AL"], e["AR"], to_bm(*pr.rhs_r, EX.RHS), "r", kfac, tol=1e-13)
        yl, _ = O.InvertE_fac(e["AR"], e["AL"], to_bm(*pr.rhs_l, EX.RHS), "l", np.conj(kfac), tol=1e-13)
        vr, vl = O.bm_vec(yr), O.bm_vec(yl)
        nr, nl = pr.nr, pr.nl
        bufs[EX.ES][:nr], bufs[EX.ES][nr:2 * nr] = vr.real, vr.imag
        bufs[EX.ES][2 * nr:2 * nr + nl], bufs[EX.ES][2 * nr + nl:2 * nr + 2 * nl] = vl.real, vl.imag
        run_tables(pr.prog_b.stages, bufs)
        ref = O.ApplyHeff(X, kfac, e["AL"], e["AR"], e["NL"], e["h"], 2, e["HLtot"], e["HRtot"], tol=1e-13)
    for n, ((xo, nn), dims) in enumerate(zip(pr.xoff, e["xdims"])):
        got = bufs[EX.OUT][xo:xo + nn] + 1j * bufs[EX.OUT][xo + nn:xo + 2 * nn]
        refv = np.concatenate([ref[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims])
        assert np.linalg.norm(got - refv) / np.linalg.norm(refv) < 1e-9, n


def test_ising_dispersion_is_exact():
    """The excitation ansatz on the transverse-field Ising chain with Z(2) charges (the odd
    sector K = 1) against its exact quasiparticle dispersion eps(k) = 2 sqrt(J'^2 + h'^2 -
    2 J' h' cos k), J' = J/4, h' = h/2: a two-site cell at momentum P holds k = P/2 and P/2 + pi,
    and the two lowest H_eff eigenvalues are those two energies (to rounding at D = 16)."""
    import math
    from scipy.sparse.linalg import LinearOperator, eigsh
    J, h = 1.0, 1.0
    Jp, hp = J / 4, h / 2
    eps = lambda k: 2 * math.sqrt(Jp ** 2 + hp ** 2 - 2 * Jp * hp * math.cos(k))
    with O.charge_group((2,)):
        e = _ising_setup(J, h)
        AL, AR, NL, hs, HL, HR, xd = e["AL"], e["AR"], e["NL"], e["h"], e["HLtot"], e["HRtot"], e["xdims"]
        n = sum(ml * mr for dd in xd for (_, _, ml, mr) in dd)

        def tox(vec):
            out, pos = [], 0
            for dd in xd:
                bm = {}
                for (qi, qo, ml, mr) in dd:
                    bm[qi] = (qo, vec[pos:pos + ml * mr].reshape(mr, ml).T.copy())
                    pos += ml * mr
                out.append(bm)
            return out

        def fromx(X):
            return np.concatenate([X[m][qi][1].T.reshape(-1) for m, dd in enumerate(xd) for (qi, _, _, _) in dd])

        for P in (0.3, 2.0):
            kfac = np.exp(1j * P)
            op = LinearOperator((n, n), dtype=complex, matvec=lambda x: fromx(O.ApplyHeff(
                tox(np.asarray(x, complex).ravel()), kfac, AL, AR, NL, hs, 2, HL, HR, tol=1e-13)))
            w = np.sort(eigsh(op, k=2, which="SA", tol=1e-10)[0])
            exact = sorted([eps(P / 2), eps(P / 2 + math.pi)])
            assert np.abs(w - exact).max() < 1e-10, (P, w, exact)


def run_flat_tables(nouts, outs, terms, alphas, bufs):
    """Execute flat imps_plan_program tables (stage_nouts, outs, terms, alphas) with numpy."""
    stages, o, t = [], 0, 0
    for n in nouts:
        st = []
        for _ in range(int(n)):
            cs, coff, cld, M, Nn, acc, nt = (int(x) for x in outs[o])
            tl = [tuple(int(x) for x in terms[t + q]) + (float(alphas[t + q]),) for q in range(nt)]
            st.append((cs, coff, cld, M, Nn, acc, tl))
            o += 1
            t += nt
        stages.append(st)
    run_tables(stages, bufs)


def test_batched_heff_tables_equal_per_momentum():
    """The batched H_eff program tables (excitations.batched_program_tables: P momenta, copy j in
    slot region j) executed with numpy give, in every copy, exactly what the single momentum's
    program gives: a CPU check of the offsets and per-copy alphas of ExcitationsBatchGPU."""
    from imps_cpp_tools_gb300 import excitations as EX
    e = excitation_setup((2,))
    kfs = [np.exp(1j * p) for p in (0.4, 1.3, 2.7)]
    prs = [EX.HeffProgram(e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"], k)
           for k in kfs]
    S = {k: max(int(prs[0].sizes.get(k, 0)), 1) for k in range(6)}
    for which in ("prog_a", "prog_b"):
        nouts, outs, terms, alphas, sizes = EX.batched_program_tables([getattr(p, which) for p in prs], prs[0].sizes)
        assert list(sizes) == [S[k] if k == EX.OPS else 3 * S[k] for k in range(6)]
        rng = np.random.default_rng(5)
        big = {k: rng.standard_normal(int(sizes[k])) for k in range(6)}
        big[EX.OPS][:prs[0].ops_vec.size] = prs[0].ops_vec
        ref = []
        for j, pr in enumerate(prs):
            small = {k: (big[k].copy() if k == EX.OPS else big[k][j * S[k]:(j + 1) * S[k]].copy()) for k in range(6)}
            run_tables(getattr(pr, which).stages, small)
            ref.append(small)
        run_flat_tables(nouts, outs, terms, alphas, big)
        for j in range(3):
            for k in range(6):
                if k == EX.OPS:
                    continue
                assert np.array_equal(big[k][j * S[k]:(j + 1) * S[k]], ref[j][k]), (which, j, k)


def _cell_excitation_setup(model, N, dims, K, params):
    """A random N-site state of the oracle (randMPS_LR), h shifted by its energy density, its
    environments (HeffConstants), null spaces and the X structure for charge K."""
    from imps_cpp_tools_gb300 import models
    d, I2K, h = models.build_model(model, **params)
    dimvec = models.make_dims(dims, N, I2K)
    AL, AR, C = O.randMPS_LR(N, I2K, dimvec, np.random.default_rng(3))
    C0 = C[-1]  # bond 0
    R, L = O.bd_mul(C0, O.bd_t(C0)), O.bd_mul(O.bd_t(C0), C0)
    hn = O.sparse_nnz(h)
    E0 = O.bd_trace(O.bd_mul(O.GetHL(AL, hn), R)) / N
    hs = O.sparse_nnz(h - E0 * np.eye(h.shape[0]))
    HLtot, HRtot = O.HeffConstants(AL, AR, L, R, hs, tol=1e-13)
    NL = [O.Nullspace(AL[n], "l") for n in range(N)]
    return dict(AL=AL, AR=AR, NL=NL, d=d, h=hs, HLtot=HLtot, HRtot=HRtot, xdims=O.XDims(NL, AR, K))


@pytest.mark.parametrize("model,N,dims,K,params,periods", [
    ("qim", 3, {(0,): 4, (1,): 3}, (1,), dict(J=1.0, h=0.7), (2,)),
    ("xxz", 4, {(-2,): 1, (0,): 3, (2,): 2}, (2,), dict(J=1.0, Delta=-1.0), None),
])
def test_heff_program_longer_unit_cells(model, N, dims, K, params, periods):
    """Excitations_main.cpp runs any unit-cell length; the host compilation of ApplyHeff
    (HeffProgram) takes the cell length from its inputs.  For a three-site quantum Ising cell
    (Z(2), odd sector) and a four-site XXZ cell, its tables executed with numpy and the oracle's
    two factored solves reproduce the oracle's ApplyHeff on every site."""
    import contextlib
    from imps_cpp_tools_gb300 import excitations as EX
    with (O.charge_group(periods) if periods else contextlib.nullcontext()):
        e = _cell_excitation_setup(model, N, dims, K, params)
        kfac = np.exp(0.6j)
        pr = EX.HeffProgram(e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"], kfac)
        bufs = {k: np.zeros(max(int(pr.sizes.get(k, 0)), 1)) for k in range(6)}
        bufs[EX.OPS][:pr.ops_vec.size] = pr.ops_vec
        X = rand_x(e["xdims"], np.random.default_rng(12))
        for (xo, n), x in zip(pr.xoff, X):
            v = O.bm_vec(x)
            bufs[EX.XS][xo:xo + n], bufs[EX.XS][xo + n:xo + 2 * n] = v.real, v.imag
        run_tables(pr.prog_a.stages, bufs)

        def to_bm(t_re, t_im, slot):
            return {k[1]: (qo, (bufs[slot][o1:o1 + r * c] + 1j * bufs[slot][t_im.blocks[k][3]:t_im.blocks[k][3] + r * c])
                           .reshape(c, r).T) for k, (qo, r, c, o1) in t_re.blocks.items()}

        yr, _ = O.InvertE_fac(e["AL"], e["AR"], to_bm(*pr.rhs_r, EX.RHS), "r", kfac, tol=1e-13)
        yl, _ = O.InvertE_fac(e["AR"], e["AL"], to_bm(*pr.rhs_l, EX.RHS), "l", np.conj(kfac), tol=1e-13)
        vr, vl = O.bm_vec(yr), O.bm_vec(yl)
        nr, nl = pr.nr, pr.nl
        bufs[EX.ES][:nr], bufs[EX.ES][nr:2 * nr] = vr.real, vr.imag
        bufs[EX.ES][2 * nr:2 * nr + nl], bufs[EX.ES][2 * nr + nl:2 * nr + 2 * nl] = vl.real, vl.imag
        run_tables(pr.prog_b.stages, bufs)
        ref = O.ApplyHeff(X, kfac, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"], tol=1e-13)
    assert len(pr.xoff) == N
    for n, ((xo, nn), dims_n) in enumerate(zip(pr.xoff, e["xdims"])):
        got = bufs[EX.OUT][xo:xo + nn] + 1j * bufs[EX.OUT][xo + nn:xo + 2 * nn]
        refv = np.concatenate([ref[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims_n])
        assert np.linalg.norm(got - refv) / np.linalg.norm(refv) < 1e-9, n


@pytest.mark.parametrize("N", [3, 4])
def test_ising_dispersion_longer_unit_cells(N):
    """The excitation ansatz of Excitations_main.cpp on an N-site cell of the transverse-field
    Ising chain (Z(2), odd sector K = 1, D = 8 + 8 per bond): at cell momentum P the N lowest
    H_eff eigenvalues are the exact quasiparticle energies eps((P + 2 pi m) / N), m = 0..N-1."""
    import math
    from scipy.sparse.linalg import LinearOperator, eigsh
    J, h = 1.0, 1.0
    Jp, hp = J / 4, h / 2
    eps = lambda k: 2 * math.sqrt(Jp ** 2 + hp ** 2 - 2 * Jp * hp * math.cos(k))  # noqa: E731
    with O.charge_group((2,)):
        H = O.qim_h(J, h)
        v = O.VUMPS(H, 2, O.qim_i2k(), {(0,): 8, (1,): 8}, N=N, seed=2)
        for _ in range(80):
            E, F, _ = v.sweep()
            if F.max() < 1e-12:
                break
        AL, AR, C0 = v.AL, O.shift(v.AR, 1), v.C[-1]
        R, L = O.bd_mul(C0, O.bd_t(C0)), O.bd_mul(O.bd_t(C0), C0)
        hs = O.sparse_nnz(H - float(E.mean()) * np.eye(4))
        K = (1,)
        _, _, OL, _, _ = O.LRoverlaps(AL, AR, K, 2)
        if OL < 0:  # Excitations_main.cpp:177-178
            AR = [[{q: (qo, -M) for q, (qo, M) in bm.items()} for bm in AR[0]]] + list(AR[1:])
        HL, HR = O.HeffConstants(AL, AR, L, R, hs, tol=1e-13)
        NL = [O.Nullspace(AL[n], "l") for n in range(N)]
        xd = O.XDims(NL, AR, K)
        n = sum(ml * mr for dd in xd for (_, _, ml, mr) in dd)

        def tox(vec):
            out, pos = [], 0
            for dd in xd:
                bm = {}
                for (qi, qo, ml, mr) in dd:
                    bm[qi] = (qo, vec[pos:pos + ml * mr].reshape(mr, ml).T.copy())
                    pos += ml * mr
                out.append(bm)
            return out

        def fromx(X):
            return np.concatenate([X[m][qi][1].T.reshape(-1) for m, dd in enumerate(xd) for (qi, _, _, _) in dd])

        for P in (0.3, 2.0):
            kfac = np.exp(1j * P)
            op = LinearOperator((n, n), dtype=complex, matvec=lambda x: fromx(O.ApplyHeff(
                tox(np.asarray(x, complex).ravel()), kfac, AL, AR, NL, hs, 2, HL, HR, tol=1e-13)))
            w = np.sort(eigsh(op, k=N, which="SA", tol=1e-10)[0])
            exact = sorted(eps((P + 2 * math.pi * m) / N) for m in range(N))
            assert np.abs(w - exact).max() < 1e-10, (P, w, exact)
