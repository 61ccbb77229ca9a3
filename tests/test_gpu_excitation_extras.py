"""GPU tests of the excitation-side additions: MeasureExcitations (Excitations_helpers.hpp:754-808),
the excitation ansatz with Z(2) charges (the exact transverse-field Ising dispersion) and the
excitation driver's saveALRN file (Excitations_main.cpp:232-237)."""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import imps_io as F
from tests.test_gpu_imps_io import saved  # noqa: F401  (module fixture)

pytestmark = pytest.mark.gpu


def test_measure_excitations_total_sz(cuda_ctx):
    """MeasureExcitations (Excitations_helpers.hpp:754-808) on the device, end to end.  The
    excitation-space operator of the total Sz minus its mean is the sector's Sz shift times the
    identity (the oracle's ApplyOPeff shows it exactly), so on the normalised random X the
    per-site values sum to -K/2 in label units.  A charge-changing observable gives zero."""
    from imps_cpp_tools_gb300 import models
    from imps_cpp_tools_gb300.excitations import measure_excitations
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    b0 = {(-2,): 3, (0,): 5, (2,): 3}
    dimvec = models.make_dims(b0, 2, models.build_model("xxz", J=1.0, Delta=-1.0)[1])
    v = VumpsGPU(cuda_ctx, "xxz", dimvec=dimvec, seed=5, InvETol=1e-13, J=1.0, Delta=-1.0)
    for _ in range(200):
        E, F, _ = v.sweep()
        if F.max() < 1e-11:
            break
    assert F.max() < 1e-10
    for K, p in (((2,), 0.7), ((-2,), 2.1)):
        vals = measure_excitations(v, K, ["sz", "sx"], np.exp(1j * p))
        assert abs(vals["sz"].sum() - (-K[0] / 2)) < 1e-8, (K, vals["sz"])
        assert np.all(vals["sx"] == 0)


def test_ising_dispersion_on_gpu(cuda_ctx):
    """The device excitation pipeline with Z(2) charges (quantum Ising, odd sector K = 1): the
    two lowest energies at cell momentum P are the exact quasiparticle energies at k = P/2 and
    P/2 + pi, eps(k) = 2 sqrt(J'^2 + h'^2 - 2 J' h' cos k), J' = J/4, h' = h/2."""
    import math
    from imps_cpp_tools_gb300.excitations import ExcitationsGPU, excitation_inputs
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    J, h = 1.0, 1.0
    Jp, hp = J / 4, h / 2
    eps = lambda k: 2 * math.sqrt(Jp ** 2 + hp ** 2 - 2 * Jp * hp * math.cos(k))
    b = {(0,): 8, (1,): 8}
    v = VumpsGPU(cuda_ctx, "qim", dimvec=[b, b], seed=2, InvETol=1e-13, J=J, h=h)
    for _ in range(80):
        E, F, _ = v.sweep()
        if F.max() < 1e-12:
            break
    assert F.max() < 1e-10
    inp = excitation_inputs(v, (1,), tol=1e-13)
    ex = ExcitationsGPU(cuda_ctx, inp["AL"], inp["AR"], inp["NL"], inp["HLtot"], inp["HRtot"], inp["h"], inp["d"],
                        inp["xdims"], tol=1e-13, LM=inp["LM"], RM=inp["RM"])
    for P in (0.3, 2.0):
        ev, conv = ex.energies(np.exp(1j * P), nev=2, eig_tol=1e-11)
        assert conv
        exact = sorted([eps(P / 2), eps(P / 2 + math.pi)])
        assert np.abs(np.array(ev) - exact).max() < 1e-8, (P, ev, exact)


def test_alrn_file_of_the_excitation_inputs(cuda_ctx, saved, tmp_path):
    """saveALRN as the excitation driver writes it (Excitations_main.cpp:232-237): C right of
    each site, L = C^T C and R = C C^T formed on the device, AL as the state file has it."""
    from imps_cpp_tools_gb300.excitations import excitation_inputs, save_alrn
    v, path = saved
    inp = excitation_inputs(v, (2,), tol=1e-13)
    st = F.loadALRN(save_alrn(v, inp, "x_ALRN", folder=str(tmp_path)))
    ref = F.loadIMPS(path)
    for n in range(2):
        assert st.C[n].keys() == ref.C[n].keys()
        for q, C in st.C[n].items():
            assert np.array_equal(C, ref.C[n][q])
            assert np.allclose(st.L[n][q], C.T @ C, atol=1e-13) and np.allclose(st.R[n][q], C @ C.T, atol=1e-13)
        for s in range(v.d):
            for q, (qo, M) in st.AL[n].blocks[s].items():
                assert np.array_equal(M, ref.AL[n].blocks[s][q][1])
        assert sum(len(b) for b in st.NL[n].blocks) > 0
