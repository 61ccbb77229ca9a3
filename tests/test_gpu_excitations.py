"""Mixed transfer matrices on general BlockMats and the factored environment solves of the
excitation ansatz (TMBlockFunctions.hpp:336-344, 474-482, 669-744; InvEBlockFunctions.hpp:
90-197, 277-451): device plans and solvers against the oracle."""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops
from oracle import imps_oracle as O
from tests import imps_testlib as T
from tests.test_gpu_parity import dev, host, relerr
from tests.test_oracle_excitations import B0, offset_bm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def state():
    return T.random_state("xxz", B0, seed=3, J=1.0, Delta=-1.0)


def _layouts(st):
    ns = len(st["I2K"][0])
    lay = lambda A: [B.Layout(T.mps_blocks(a), ns) for a in A]
    return ns, lay(st["AL"]), lay(st["AR"])


@pytest.mark.parametrize("direction", ["l", "r"])
@pytest.mark.parametrize("K", [(2,), (0,), (-2,)])
def test_mixed_tm_apply_matches_oracle(cuda_ctx, state, direction, K):
    ns, LAL, LAR = _layouts(state)
    AL, AR = state["AL"], state["AR"]
    rng = np.random.default_rng(5)
    X = offset_bm(state["dimvec"][0], K, rng)
    lx = B.Layout(T.bm_blocks(X), ns)
    if direction == "l":  # lower AR, upper AL: out = sum_s AL_s^T X AR_s (the EHBL chain)
        plan = B.plan_tm_mixed(cuda_ctx, LAR, LAL, 0, lx, lx)
        A, Bm, ref = AR, AL, O.ApplyTMmixedLeftUC(AR, AL, X)
    else:  # lower AL, upper AR: out = sum_s AL_s X AR_s^T (the EBR chain)
        plan = B.plan_tm_mixed(cuda_ctx, LAL, LAR, 1, lx, lx)
        A, Bm, ref = AL, AR, O.ApplyTMmixedRightUC(AL, AR, X)
    for k in range(2):
        plan.bind(2 + k, dev(O.mps_vec(A[k])))
        plan.bind(4 + k, dev(O.mps_vec(Bm[k])))
    out = dev(np.zeros(lx.nelem))
    ops.ApplyTM(plan, dev(O.bm_vec(X)), out)
    refv = np.concatenate([ref[q][1].reshape(-1, order="F") for q in sorted(X)])
    assert relerr(host(out), refv) < 1e-12


def _solve_pair(cuda_ctx, state, direction, K, fac, proj):
    ns, LAL, LAR = _layouts(state)
    AL, AR = state["AL"], state["AR"]
    rng = np.random.default_rng(6)
    x = offset_bm(state["dimvec"][0], K, rng, cplx=True)
    lx = B.Layout(T.bm_blocks(x), ns)
    if direction == "r":
        Avec, Bvec, code = AL, AR, 1
    else:
        Avec, Bvec, code = AR, AL, 0
    plan = B.plan_tm_mixed(cuda_ctx, [B.Layout(T.mps_blocks(a), ns) for a in Avec],
                           [B.Layout(T.mps_blocks(b), ns) for b in Bvec], code, lx, lx)
    for k in range(2):
        plan.bind(2 + k, dev(O.mps_vec(Avec[k])))
        plan.bind(4 + k, dev(O.mps_vec(Bvec[k])))
    xv = O.bm_vec(x)
    y0 = np.random.default_rng(7).standard_normal(xv.size) + 0j
    yre, yim = dev(y0.real.copy()), dev(y0.imag.copy())
    if proj:
        # any L, R of the transposed structure define a regular projected system for |fac| < 1
        L = {qo: (qi, 0.1 * rng.standard_normal(M.shape[::-1])) for qi, (qo, M) in x.items()}
        R = {qo: (qi, 0.1 * rng.standard_normal(M.shape[::-1])) for qi, (qo, M) in x.items()}
        it, rr, conv = ops.InvertE_proj_fac(plan, dev(xv.real.copy()), dev(xv.imag.copy()), dev(O.bm_vec(L)),
                                            dev(O.bm_vec(R)), direction, fac, yre, yim, 1e-12)
        yo, flag = O.InvertE_proj_fac(Avec, Bvec, x, L, R, direction, fac, tol=1e-12,
                                      y0=O.bm_from_vec(y0, O.bm_sizes(x)))
    else:
        it, rr, conv = ops.InvertE_fac(plan, dev(xv.real.copy()), dev(xv.imag.copy()), fac, yre, yim, 1e-12)
        yo, flag = O.InvertE_fac(Avec, Bvec, x, direction, fac, tol=1e-12, y0=O.bm_from_vec(y0, O.bm_sizes(x)))
    assert conv and flag >= 0
    yg = host(yre) + 1j * host(yim)
    return yg, O.bm_vec(yo)


@pytest.mark.parametrize("direction", ["l", "r"])
@pytest.mark.parametrize("K,p", [((2,), 0.7), ((-2,), 2.1), ((0,), 1.3)])
def test_invert_e_fac_matches_oracle(cuda_ctx, state, direction, K, p):
    """Charge offset K != 0, or momentum p != 0: (1 - e^{ip} T) is regular, no projection."""
    yg, yo = _solve_pair(cuda_ctx, state, direction, K, np.exp(1j * p), proj=False)
    assert np.linalg.norm(yg - yo) / np.linalg.norm(yo) < 1e-9


@pytest.mark.parametrize("direction", ["l", "r"])
def test_invert_e_proj_fac_matches_oracle(cuda_ctx, state, direction):
    yg, yo = _solve_pair(cuda_ctx, state, direction, (0,), 0.9 * np.exp(0.4j), proj=True)
    assert np.linalg.norm(yg - yo) / np.linalg.norm(yo) < 1e-9


@pytest.mark.parametrize("K,p", [((2,), 0.6), ((-2,), 2.4)])
def test_heff_apply_matches_oracle(cuda_ctx, K, p):
    """ApplyHeff (Excitations_helpers.hpp:20-228) compiled into grouped-GEMM programs around the
    two factored solves, against the oracle's restatement on the same state and X."""
    from imps_cpp_tools_gb300.excitations import HeffGPU
    from tests.test_oracle_excitations import excitation_setup, rand_x
    e = excitation_setup(K)
    kfac = np.exp(1j * p)
    H = HeffGPU(cuda_ctx, e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"], kfac,
                tol=1e-13)
    X = rand_x(e["xdims"], np.random.default_rng(12))
    H.x_to_planes([O.bm_vec(x) for x in X])
    assert H.apply()
    got = H.y_from_planes()
    ref = O.ApplyHeff(X, kfac, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"], tol=1e-13)
    for n, dims in enumerate(e["xdims"]):
        refv = np.concatenate([ref[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims])
        assert np.linalg.norm(got[n] - refv) / np.linalg.norm(refv) < 1e-9, n


def test_excitation_energies_match_oracle(cuda_ctx):
    """The 4 lowest eigenvalues of H_eff at one momentum (Excitations_main.cpp:270-279, eigs_n
    "SR"): the device Lanczos on the real form of H_eff against ARPACK (scipy) on the oracle's
    ApplyHeff."""
    from scipy.sparse.linalg import LinearOperator, eigsh
    from imps_cpp_tools_gb300.excitations import ExcitationsGPU
    from tests.test_oracle_excitations import excitation_setup
    dims0 = {(-2,): 3, (0,): 5, (2,): 3}
    e = excitation_setup((2,), dims0=dims0)
    kfac = np.exp(0.9j)
    ex = ExcitationsGPU(cuda_ctx, e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"],
                        tol=1e-13)
    ev, conv = ex.energies(kfac, nev=4, eig_tol=1e-10)
    assert conv
    sizes = [[(qi, qo, ml, mr) for (qi, qo, ml, mr) in dims] for dims in e["xdims"]]
    lens = [sum(ml * mr for (_, _, ml, mr) in dims) for dims in sizes]
    mtot = sum(lens)

    def hop(v):
        parts, pos = [], 0
        for dims, ln in zip(sizes, lens):
            parts.append(O.bm_from_vec(v[pos:pos + ln], dims))
            pos += ln
        out = O.ApplyHeff(parts, kfac, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"], tol=1e-13)
        return np.concatenate([np.concatenate([out[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims])
                               for n, dims in enumerate(sizes)])

    op = LinearOperator((mtot, mtot), matvec=hop, dtype=np.complex128)
    ref = np.sort(eigsh(op, k=4, which="SA", tol=1e-11, return_eigenvectors=False))
    assert np.abs(np.sort(ev) - ref).max() < 1e-8 * max(1.0, np.abs(ref).max()), (ev, ref)


def _mps_from_vec(v, layout):
    """Device-layout vector -> map-of-blocks MPS (list over s of {qin: (qout, M)})."""
    ng = max(b[0] for b in layout.blocks) + 1 if layout.blocks else 1
    out = [dict() for _ in range(ng)]
    pos = 0
    for (g, qi, qo, r, c) in layout.blocks:
        out[g][tuple(qi)] = (tuple(qo), np.array(v[pos:pos + r * c]).reshape(c, r).T.copy())
        pos += r * c
    return out


def test_nullspace_on_device(cuda_ctx, state):
    """Nullspace(A, l) on the device: orthonormal columns per right sector, orthogonal to A."""
    ns = len(state["I2K"][0])
    for A in state["AL"]:
        plan = B.plan_decomp(cuda_ctx, B.Layout(T.mps_blocks(A), ns), "l")
        NLd = dev(np.zeros(plan.nslayout.nelem))
        ops.Nullspace(plan, dev(O.mps_vec(A)), NLd)
        NL = _mps_from_vec(host(NLd), plan.nslayout)
        NL += [dict() for _ in range(len(A) - len(NL))]
        G = O.ApplyTMmixedLeft(NL, NL)  # sum_s NL_s^T NL_s per sector
        for q, (qo, M) in G.items():
            assert np.abs(M - np.eye(M.shape[0])).max() < 1e-12
        X = O.ApplyTMmixedLeft(NL, A)  # sum_s A_s^T NL_s
        assert max((np.abs(M).max() for (_, M) in X.values()), default=0.0) < 1e-12


def test_excitation_energies_with_device_nullspace(cuda_ctx):
    """Excitation energies do not depend on the null-space basis: the device N_L gives the same
    4 lowest energies as the oracle's (SVD-based) N_L."""
    from imps_cpp_tools_gb300.excitations import ExcitationsGPU
    from tests.test_oracle_excitations import excitation_setup
    dims0 = {(-2,): 3, (0,): 5, (2,): 3}
    e = excitation_setup((2,), dims0=dims0)
    ns = 1
    NLd = []
    for A in e["AL"]:
        plan = B.plan_decomp(cuda_ctx, B.Layout(T.mps_blocks(A), ns), "l")
        v = dev(np.zeros(plan.nslayout.nelem))
        ops.Nullspace(plan, dev(O.mps_vec(A)), v)
        m = _mps_from_vec(host(v), plan.nslayout)
        NLd.append(m + [dict() for _ in range(len(A) - len(m))])
    xd = O.XDims(NLd, e["AR"], (2,))
    assert [[(q, qo, a, b) for (q, qo, a, b) in dd] for dd in xd] == e["xdims"]
    kfac = np.exp(0.9j)
    args = (e["AL"], e["AR"])
    ev_dev, c1 = ExcitationsGPU(cuda_ctx, *args, NLd, e["HLtot"], e["HRtot"], e["h"], e["d"], xd,
                                tol=1e-13).energies(kfac, nev=4, eig_tol=1e-10)
    ev_ora, c2 = ExcitationsGPU(cuda_ctx, *args, e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"],
                                tol=1e-13).energies(kfac, nev=4, eig_tol=1e-10)
    assert c1 and c2
    assert np.abs(np.array(ev_dev) - np.array(ev_ora)).max() < 1e-8


def test_excitations_from_converged_vumps_state(cuda_ctx):
    """The whole excitation pipeline from a converged GPU VUMPS state (HeffConstants, N_L and
    XDims on the device / from layouts), against the oracle's HeffConstants and ARPACK on the
    oracle's H_eff for the same state."""
    from scipy.sparse.linalg import LinearOperator, eigsh
    from imps_cpp_tools_gb300.excitations import ExcitationsGPU, excitation_inputs
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    b0 = {(-2,): 3, (0,): 5, (2,): 3}
    from imps_cpp_tools_gb300 import models
    dimvec = models.make_dims(b0, 2, models.build_model("xxz", J=1.0, Delta=-1.0)[1])
    v = VumpsGPU(cuda_ctx, "xxz", dimvec=dimvec, seed=5, InvETol=1e-13, J=1.0, Delta=-1.0)
    for _ in range(200):
        E, F, _ = v.sweep()
        if F.max() < 1e-11:
            break
    assert F.max() < 1e-10
    inp = excitation_inputs(v, (2,), tol=1e-13)
    # the overlap of the K = +-2 sectors only sets the sign of AR[0] (Excitations_main.cpp:177-178)
    assert 0.0 < abs(inp["OL"]) < 1.0
    # HeffConstants against the oracle on the same (downloaded) state
    C0 = O.bd_from_vec(v.C[0].cpu().numpy(), [(tuple(b[1]), b[3]) for b in v.LB[0].blocks])
    R = O.bd_mul(C0, O.bd_t(C0))
    L = O.bd_mul(O.bd_t(C0), C0)
    HLo, HRo = O.HeffConstants(inp["AL"], inp["AR"], L, R, inp["h"], tol=1e-13)
    for got, ref in ((inp["HLtot"], HLo), (inp["HRtot"], HRo)):
        for n in range(2):
            for q in ref[n]:
                assert np.abs(got[n][q] - ref[n][q]).max() < 1e-8 * max(1.0, np.abs(ref[n][q]).max())
    kfac = np.exp(1.1j)
    ex = ExcitationsGPU(cuda_ctx, inp["AL"], inp["AR"], inp["NL"], inp["HLtot"], inp["HRtot"], inp["h"], inp["d"],
                        inp["xdims"], tol=1e-13)
    ev, conv = ex.energies(kfac, nev=3, eig_tol=1e-10)
    assert conv
    sizes = inp["xdims"]
    lens = [sum(ml * mr for (_, _, ml, mr) in dd) for dd in sizes]

    def hop(x):
        parts, pos = [], 0
        for dd, ln in zip(sizes, lens):
            parts.append(O.bm_from_vec(x[pos:pos + ln], dd))
            pos += ln
        out = O.ApplyHeff(parts, kfac, inp["AL"], inp["AR"], inp["NL"], inp["h"], inp["d"], inp["HLtot"],
                          inp["HRtot"], tol=1e-13)
        return np.concatenate([np.concatenate([out[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dd])
                               for n, dd in enumerate(sizes)])

    mtot = sum(lens)
    ref = np.sort(eigsh(LinearOperator((mtot, mtot), matvec=hop, dtype=np.complex128), k=3, which="SA",
                        tol=1e-11, return_eigenvectors=False))
    assert np.abs(np.sort(ev) - ref).max() < 1e-8 * max(1.0, np.abs(ref).max()), (ev, ref)
    # K = 0, p = 0: the projected case from the same state; the overlap of AL and AR is +-1 and,
    # the state being a variational minimum, H_eff - E0 is positive on the ansatz space
    inp0 = excitation_inputs(v, (0,), tol=1e-13)
    assert abs(abs(inp0["OL"]) - 1.0) < 1e-8
    ex0 = ExcitationsGPU(cuda_ctx, inp0["AL"], inp0["AR"], inp0["NL"], inp0["HLtot"], inp0["HRtot"], inp0["h"],
                         inp0["d"], inp0["xdims"], tol=1e-13, LM=inp0["LM"], RM=inp0["RM"])
    ev0, conv0 = ex0.energies(1.0 + 0j, nev=2, eig_tol=1e-10)
    assert conv0 and ev0[0] > -1e-6, ev0


def _dense_op(ctx, M):
    """Device callback applying the dense matrix M (the context shares torch's stream)."""
    import ctypes as C
    import torch
    from imps_cpp_tools_gb300 import _native as N
    Md = torch.tensor(M, dtype=torch.float64, device="cuda")
    n = M.shape[0]
    xin = torch.zeros(n, dtype=torch.float64, device="cuda")
    keep = {}

    def apply(pin, pout):
        N.call("imps_axpby", ctx.handle, 1.0, C.c_void_p(pin), 0.0, C.c_void_p(xin.data_ptr()), n)
        keep["y"] = Md @ xin
        N.call("imps_axpby", ctx.handle, 1.0, C.c_void_p(keep["y"].data_ptr()), 0.0, C.c_void_p(pout), n)
    return apply


@pytest.mark.parametrize("which,want", [("LM", [3.0, 2.5 + 1j, 2.5 - 1j, -2.6]),
                                        ("LR", [3.0, 2.5 + 1j, 2.5 - 1j, 1.5]),
                                        ("SR", [-2.6, -1.9, -1.2 + 0.5j, -1.2 - 0.5j])])
def test_eigs_n_dense_spectrum(cuda_ctx, which, want):
    """eigs_n (eigs.cpp:193-342) by the device Arnoldi on a real nonsymmetric matrix with a known
    spectrum (real eigenvalues and conjugate pairs): values in the requested order, unit-norm
    eigenvectors with small residuals."""
    import torch
    rng = np.random.default_rng(3)
    n = 300
    D = np.zeros((n, n))
    specials = [3.0, -2.6, 1.5, -1.9]
    for i, l in enumerate(specials):
        D[i, i] = l
    for i, (a, b) in enumerate([(2.5, 1.0), (-1.2, 0.5)]):
        j = 4 + 2 * i
        D[j:j + 2, j:j + 2] = [[a, b], [-b, a]]
    D[8:, 8:] = np.diag(rng.uniform(-1.0, 1.0, n - 8))
    X = np.eye(n) + 0.1 * rng.standard_normal((n, n))
    M = X @ D @ np.linalg.inv(X)
    nev = 4
    ere = torch.zeros((nev, n), dtype=torch.float64, device="cuda")
    eim = torch.zeros((nev, n), dtype=torch.float64, device="cuda")
    vals, na, conv = ops.eigs_n_op(cuda_ctx, n, _dense_op(cuda_ctx, M), nev=nev, which=which, tol=1e-13,
                                   ncv=30, evecs_re=ere, evecs_im=eim)
    assert conv and na > 0
    assert np.abs(vals - np.array(want)).max() < 1e-10, vals
    V = host(ere) + 1j * host(eim)
    for i in range(nev):
        assert abs(np.linalg.norm(V[i]) - 1.0) < 1e-12
        assert np.linalg.norm(M @ V[i] - vals[i] * V[i]) < 1e-9 * np.linalg.norm(M, 2)


@pytest.mark.parametrize("direction", ["l", "r"])
@pytest.mark.parametrize("K", [(0,), (2,)])
def test_tm_mixed_eigs_matches_arpack(cuda_ctx, state, direction, K):
    """TMmixedEigs (EigsBlockFunctions.hpp:282-391): the device Arnoldi on the mixed-TM plan
    against ARPACK (scipy, the library eigs.cpp drives) on the oracle's mixed TM."""
    from imps_cpp_tools_gb300.excitations import tm_mixed_eigs
    AL, AR = state["AL"], state["AR"]
    vg, Vg, sg, na, conv = tm_mixed_eigs(cuda_ctx, AL, AR, direction, K, 3, "LM", 1e-13)
    vo, Vo, so = O.TMmixedEigs(AL, AR, direction, K, 3, "LM", 1e-13)
    assert conv and sg == so
    for a in vg:  # each device eigenvalue has an ARPACK partner (conjugate pairs may swap)
        assert np.abs(vo - a).min() < 1e-10 * max(1.0, abs(a)), (vg, vo)
    j = int(np.argmin(np.abs(vo - vg[0])))  # the partner (conjugates may be listed either way)
    a, b = O.bm_vec(Vg[0]), O.bm_vec(Vo[j])
    assert abs(abs(np.vdot(a, b)) / (np.linalg.norm(a) * np.linalg.norm(b)) - 1.0) < 1e-9
    res = O.bm_vec(O.ApplyTMmixedLeftUC(AL, AR, Vg[0]) if direction == "l" else
                   O.ApplyTMmixedRightUC(AL, AR, Vg[0])) - vg[0] * a
    assert np.linalg.norm(res) < 1e-11


def test_lroverlaps_on_device(cuda_ctx, state):
    """LRoverlaps (Excitations_helpers.hpp:915-946): overlap and dominant eigenmatrices against
    the oracle's (real parts; the eigenvectors' sign is free)."""
    from imps_cpp_tools_gb300.excitations import LRoverlaps
    AL, AR = state["AL"], state["AR"]
    LM, RM, OL, vl, vr, conv = LRoverlaps(cuda_ctx, AL, AR, (0,), 2)
    LMo, RMo, OLo, _, _ = O.LRoverlaps(AL, AR, (0,), 2)
    assert conv and abs(OL - OLo) < 1e-12
    for X, Y in ((LM, LMo), (RM, RMo)):
        a, b = O.bm_vec(X), O.bm_vec(Y)
        assert min(np.abs(a - b).max(), np.abs(a + b).max()) < 1e-10


def _proj_setup():
    from tests.test_oracle_excitations import excitation_setup
    e = excitation_setup((0,), dims0={(-2,): 3, (0,): 5, (2,): 3})
    LM, RM, OL, _, _ = O.LRoverlaps(e["AL"], e["AR"], (0,), 2)
    return e, LM, RM


def test_projected_heff_apply_matches_oracle(cuda_ctx):
    """p = 0, K = 0: ApplyHeff with the projected environment solves (InvertE_proj_fac with LM,
    RM) on the device against the oracle."""
    from imps_cpp_tools_gb300.excitations import HeffGPU
    from tests.test_oracle_excitations import rand_x
    e, LM, RM = _proj_setup()
    H = HeffGPU(cuda_ctx, e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"], 1.0 + 0j,
                tol=1e-13, LM=LM, RM=RM)
    X = rand_x(e["xdims"], np.random.default_rng(13))
    H.x_to_planes([O.bm_vec(x) for x in X])
    assert H.apply()
    got = H.y_from_planes()
    ref = O.ApplyHeff(X, 1.0 + 0j, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"], LM=LM, RM=RM,
                      tol=1e-13)
    for n, dims in enumerate(e["xdims"]):
        refv = np.concatenate([ref[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims])
        assert np.linalg.norm(got[n] - refv) / np.linalg.norm(refv) < 1e-9, n


def test_projected_energies_match_oracle(cuda_ctx):
    """The excitation energies at p = 0, K = 0 (the projected case of Excitations_main.cpp:
    263-279) against ARPACK on the oracle's projected H_eff."""
    from scipy.sparse.linalg import LinearOperator, eigsh
    from imps_cpp_tools_gb300.excitations import ExcitationsGPU
    e, LM, RM = _proj_setup()
    ex = ExcitationsGPU(cuda_ctx, e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"],
                        tol=1e-13, LM=LM, RM=RM)
    assert ex.projected(0.0) and not ex.projected(0.3)
    ev, conv = ex.energies(1.0 + 0j, nev=3, eig_tol=1e-10)
    assert conv
    sizes = e["xdims"]
    lens = [sum(ml * mr for (_, _, ml, mr) in dd) for dd in sizes]

    def hop(x):
        parts, pos = [], 0
        for dd, ln in zip(sizes, lens):
            parts.append(O.bm_from_vec(x[pos:pos + ln], dd))
            pos += ln
        out = O.ApplyHeff(parts, 1.0 + 0j, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"], LM=LM,
                          RM=RM, tol=1e-13)
        return np.concatenate([np.concatenate([out[n][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dd])
                               for n, dd in enumerate(sizes)])

    mtot = sum(lens)
    ref = np.sort(eigsh(LinearOperator((mtot, mtot), matvec=hop, dtype=np.complex128), k=3, which="SA",
                        tol=1e-11, return_eigenvectors=False))
    assert np.abs(np.sort(ev) - ref).max() < 1e-8 * max(1.0, np.abs(ref).max()), (ev, ref)

