"""Unit cells of any length N (vumps_cell.VumpsCellGPU; the reference takes N >= 2 from its command
line, VUMPS_main.cpp:31,55-56): for N = 2 the sweeps of the two-site driver, for N = 3 and 4 the
oracle's VUMPS with the same N sweep by sweep, and the exact transverse-field Ising energy."""
import copy
import math

import numpy as np
import pytest

from imps_cpp_tools_gb300 import models
from imps_cpp_tools_gb300.vumps import VumpsGPU
from imps_cpp_tools_gb300.vumps_cell import VumpsCellGPU
from oracle import imps_oracle as O
from tests.test_gpu_parity import dev
from tests.test_gpu_vumps import B0, B1

pytestmark = pytest.mark.gpu


def _init(AL, AR, C):
    """randMPS_LR's arrangement (AR(n) at n, C[k] on bond k+1) as the drivers' init_state (C[b]
    on bond b)."""
    N = len(AL)
    return {"AL": [dev(O.mps_vec(a)) for a in AL], "AR": [dev(O.mps_vec(a)) for a in AR],
            "C": [dev(O.bd_vec(C[(b - 1) % N])) for b in range(N)]}


def test_cell_n2_equals_two_site_driver(cuda_ctx):
    d, I2K, h = models.build_model("xxz", J=1.0, Delta=-1.0)
    dimvec = [B0, B1]
    st = O.randMPS_LR(2, I2K, dimvec, np.random.default_rng(7))
    a = VumpsGPU(cuda_ctx, "xxz", dimvec=dimvec, init_state=_init(*st), fixed_tol=1e-12, J=1.0, Delta=-1.0)
    b = VumpsCellGPU(cuda_ctx, "xxz", 2, dimvec=dimvec, init_state=_init(*st), fixed_tol=1e-12, J=1.0, Delta=-1.0)
    for sweep in range(3):
        Ea, Fa, pa = a.sweep()
        Eb, Fb, pb = b.sweep()
        assert np.abs(Ea - Eb).max() < 1e-12, (sweep, Ea, Eb)
        assert np.allclose(Fa, Fb, rtol=1e-9, atol=1e-14) and np.allclose(pa, pb, rtol=1e-9, atol=1e-14)


@pytest.mark.parametrize("N", [3, 4])
def test_cell_sweeps_match_oracle(cuda_ctx, N):
    """Quantum Ising (Z(2)), J = 1, h = 0.7, sector dims differing from bond to bond: from the
    oracle's state 5 sweeps past its seeded random start (the first sweeps are chaotic), every
    sweep of the device driver agrees with the oracle's to 1e-9 in the energies."""
    J, hf = 1.0, 0.7
    d, I2K, h = models.build_model("qim", J=J, h=hf)
    dimvec = [{(0,): 6, (1,): 5}, {(0,): 4, (1,): 7}, {(0,): 5, (1,): 5}, {(0,): 7, (1,): 3}][:N]
    with O.charge_group((2,)):
        AL, AR, C = O.randMPS_LR(N, I2K, dimvec, np.random.default_rng(7))
        ora = O.VUMPS(h, d, I2K, dimvec[0], N=N, dimvec=dimvec, init=(AL, AR, C), fixed_tol=1e-12, seed=7)
        for _ in range(5):
            ora.sweep()
        st = (copy.deepcopy(ora.AL), O.shift(copy.deepcopy(ora.AR), 1), copy.deepcopy(ora.C))
        ora = O.VUMPS(h, d, I2K, dimvec[0], N=N, dimvec=dimvec, init=st, fixed_tol=1e-12, seed=7)
        gpu = VumpsCellGPU(cuda_ctx, "qim", N, dimvec=dimvec, init_state=_init(*st), fixed_tol=1e-12, J=J, h=hf)
        for sweep in range(3):
            Eo, Fo, _ = ora.sweep()
            Eg, Fg, _ = gpu.sweep()
            assert len(Eg) == N and np.abs(Eg - Eo).max() < 1e-9, (sweep, Eg, Eo)
            assert np.allclose(Fg, Fo, rtol=1e-3, atol=1e-10), (sweep, Fg, Fo)


def test_cell_quantum_ising_exact_energy(cuda_ctx):
    """A three-site cell of the transverse-field Ising chain reaches the exact energy on every
    bond on the device."""
    from scipy.integrate import quad
    J, hf = 1.0, 0.7
    Jp, hp = J / 4, hf / 2
    e0 = -quad(lambda k: math.sqrt(Jp ** 2 + hp ** 2 - 2 * Jp * hp * math.cos(k)), -math.pi, math.pi,
               epsabs=1e-14)[0] / (2 * math.pi)
    b = {(0,): 8, (1,): 8}
    gpu = VumpsCellGPU(cuda_ctx, "qim", 3, dimvec=[b, b, b], seed=2, J=J, h=hf)
    for _ in range(60):
        E, F, _ = gpu.sweep()
        if F.max() < 1e-11:
            break
    assert F.max() < 1e-10 and np.abs(E - e0).max() < 1e-10, (E, e0)
