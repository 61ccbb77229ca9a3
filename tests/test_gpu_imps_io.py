"""State files from and into the GPU VUMPS driver (saveIMPS at VUMPS_main.cpp:403, loadIMPS at
Excitations_main.cpp:89).

A converged XXZ state is saved by the driver and checked on the host: Lamvec[n] are the
singular values of Cvec[n], C is normalised, and the arrangement satisfies the reference's
gauge check AL(n) Cvec[n] = Cvec[n-1] AR(n) (VUMPS_main.cpp:381-382).  A driver started from
the file holds the same buffers and energy, keeps sweeping to the same energy, and gives the
same excitation inputs and energies as the live state.
"""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import imps_io as F
from imps_cpp_tools_gb300 import models
from imps_cpp_tools_gb300.vumps import VumpsGPU

pytestmark = pytest.mark.gpu

XXZ = {"J": 1.0, "Delta": -1.0}


@pytest.fixture(scope="module")
def saved(cuda_ctx, tmp_path_factory):
    b0 = {(-2,): 3, (0,): 5, (2,): 3}
    dimvec = models.make_dims(b0, 2, models.build_model("xxz", **XXZ)[1])
    v = VumpsGPU(cuda_ctx, "xxz", dimvec=dimvec, seed=5, InvETol=1e-13, **XXZ)
    for _ in range(200):
        E, F_, _ = v.sweep()
        if F_.max() < 1e-11:
            break
    assert F_.max() < 1e-10
    path = v.save_imps("UMPS_xxz_N2", folder=str(tmp_path_factory.mktemp("state")))
    return v, path


def test_saved_file_is_the_state(saved):
    v, path = saved
    st = F.loadIMPS(path)
    assert len(st.AL) == len(st.AR) == len(st.C) == len(st.Lam) == 2
    for n in range(2):
        for q, m in st.C[n].items():
            assert np.allclose(st.Lam[n][q], np.linalg.svd(m, compute_uv=False), atol=1e-12, rtol=0)
        assert abs(sum(float(np.sum(l * l)) for l in st.Lam[n].values()) - 1.0) < 1e-12
        # gauge check of the reference: AL(n) Cvec[n] = Cvec[n-1] AR(n)
        Cr, Cl = st.C[n], st.C[(n + 1) % 2]
        err = 0.0
        for s in range(v.d):
            for q, (qo, al) in st.AL[n].blocks[s].items():
                qo2, ar = st.AR[n].blocks[s][q]
                assert qo2 == qo
                err = max(err, np.abs(al @ Cr[qo] - Cl[q] @ ar).max())
        assert err < 1e-8, (n, err)


def test_driver_restarts_from_the_file(cuda_ctx, saved):
    v, path = saved
    w = VumpsGPU.from_imps(cuda_ctx, "xxz", path, InvETol=1e-13, **XXZ)
    for a, b in ((v.AL, w.AL), (v.AR, w.AR), (v.C, w.C)):
        for n in range(2):
            assert bool((a[n] == b[n]).all())
    assert np.abs(w.energy() - v.energy()).max() < 1e-14
    Ev, Ew = v.energy(), None
    for _ in range(2):
        Ew, Fw, _ = w.sweep()
    # the restarted driver begins at the loose end of the tolerance schedule (its first sweep
    # solves at tolmax, VUMPS_main.cpp:177, as the reference after a fresh start)
    assert np.abs(Ew - Ev).max() < 1e-9 and Fw.max() < 1e-7
    with pytest.raises(F.IMPSFormatError):
        VumpsGPU.from_imps(cuda_ctx, "fhub", path)  # d = 4 model on a d = 2 state


def test_excitations_from_the_file(cuda_ctx, saved):
    """Excitations_main.cpp:84-101 loads the state and builds everything from it."""
    from imps_cpp_tools_gb300.excitations import ExcitationsGPU, excitation_inputs
    v, path = saved
    w = VumpsGPU.from_imps(cuda_ctx, "xxz", path, InvETol=1e-13, **XXZ)
    res = []
    for drv in (v, w):
        inp = excitation_inputs(drv, (2,), tol=1e-13)
        ex = ExcitationsGPU(cuda_ctx, inp["AL"], inp["AR"], inp["NL"], inp["HLtot"], inp["HRtot"], inp["h"],
                            inp["d"], inp["xdims"], tol=1e-13)
        ev, conv = ex.energies(np.exp(0.7j), nev=2, eig_tol=1e-10)
        assert conv
        res.append((inp, np.sort(ev)))
    (a, ea), (b, eb) = res
    for n in range(2):
        for q in a["HLtot"][n]:
            assert np.abs(a["HLtot"][n][q] - b["HLtot"][n][q]).max() < 1e-9
    assert np.abs(ea - eb).max() < 1e-8, (ea, eb)
