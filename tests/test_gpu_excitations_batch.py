"""Excitation energies at several momenta in one batched run (ExcitationsBatchGPU: P copies of the
H_eff programs per launch, the environment solves of all momenta as one stacked GMRES on the
replicated mixed transfer matrix, P Lanczos runs in lockstep) against the per-momentum path and
the oracle's ApplyHeff."""
import numpy as np
import pytest

from oracle import imps_oracle as O

pytestmark = pytest.mark.gpu

PS = [0.4, 1.3, 2.7]


def _setup():
    from tests.test_oracle_excitations import excitation_setup
    return excitation_setup((2,), dims0={(-2,): 3, (0,): 5, (2,): 3})


def test_batched_heff_apply_matches_oracle(cuda_ctx):
    """One batched apply equals the oracle's ApplyHeff at every momentum (1e-9)."""
    import torch
    from imps_cpp_tools_gb300.excitations import XS, OUT, ExcitationsBatchGPU
    from tests.test_oracle_excitations import rand_x
    e = _setup()
    kf = [np.exp(1j * p) for p in PS]
    ex = ExcitationsBatchGPU(cuda_ctx, e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"],
                             kf, tol=1e-13)
    S = ex.sizes
    Xs = [rand_x(e["xdims"], np.random.default_rng(20 + j)) for j in range(len(PS))]
    for j, X in enumerate(Xs):
        for (xo, n), x in zip(ex.pr.xoff, [O.bm_vec(x) for x in X]):
            base = j * S[XS] + xo
            ex.buf[XS][base:base + n].copy_(torch.from_numpy(np.ascontiguousarray(x.real)))
            ex.buf[XS][base + n:base + 2 * n].copy_(torch.from_numpy(np.ascontiguousarray(x.imag)))
    assert ex.apply()
    out = ex.buf[OUT].cpu().numpy()
    for j, (X, k) in enumerate(zip(Xs, kf)):
        ref = O.ApplyHeff(X, k, e["AL"], e["AR"], e["NL"], e["h"], e["d"], e["HLtot"], e["HRtot"], tol=1e-13)
        for nsite, ((xo, n), dims) in enumerate(zip(ex.pr.xoff, e["xdims"])):
            got = out[j * S[OUT] + xo: j * S[OUT] + xo + n] + 1j * out[j * S[OUT] + xo + n: j * S[OUT] + xo + 2 * n]
            refv = np.concatenate([ref[nsite][qi][1].reshape(-1, order="F") for (qi, _, _, _) in dims])
            assert np.linalg.norm(got - refv) / np.linalg.norm(refv) < 1e-9, (j, nsite)


def test_batched_energies_match_per_momentum(cuda_ctx):
    """The 4 lowest energies at 3 momenta from one batched run equal those of the per-momentum
    device path (each checked against ARPACK on the oracle's H_eff in test_gpu_excitations.py)
    to 1e-8."""
    from imps_cpp_tools_gb300.excitations import ExcitationsBatchGPU, ExcitationsGPU
    e = _setup()
    args = (e["AL"], e["AR"], e["NL"], e["HLtot"], e["HRtot"], e["h"], e["d"], e["xdims"])
    kf = [np.exp(1j * p) for p in PS]
    eb, convb, na = ExcitationsBatchGPU(cuda_ctx, *args, kf, tol=1e-13).energies(nev=4, eig_tol=1e-10)
    assert all(convb), convb
    single = ExcitationsGPU(cuda_ctx, *args, tol=1e-13)
    for j, k in enumerate(kf):
        ev, conv = single.energies(k, nev=4, eig_tol=1e-10)
        assert conv
        assert np.abs(np.array(eb[j]) - np.array(ev)).max() < 1e-8, (j, eb[j], ev)
