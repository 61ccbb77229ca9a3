"""End-to-end parity of the GPU VUMPS driver with the oracle's restatement of VUMPS_main.cpp,
from the same initial state, at fixed eigensolver/GMRES tolerance 1e-12; and the Heisenberg
Bethe-ansatz energy reached by the GPU path alone."""
import math

import numpy as np
import pytest

from imps_cpp_tools_gb300 import models
from imps_cpp_tools_gb300.vumps import VumpsGPU
from oracle import imps_oracle as O
from tests.test_gpu_parity import dev

pytestmark = pytest.mark.gpu

B0 = {(-4,): 3, (-2,): 8, (0,): 10, (2,): 8, (4,): 3}
B1 = {(-5,): 1, (-3,): 5, (-1,): 10, (1,): 10, (3,): 5, (5,): 1}


def _pair(cuda_ctx, model, dimvec, seed, fixed_tol=1e-12, **params):
    d, I2K, h = models.build_model(model, **params)
    rng = np.random.default_rng(seed)
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, rng)
    ora = O.VUMPS(h, d, I2K, dimvec[0], dimvec=dimvec, init=(AL, AR, C), fixed_tol=fixed_tol, seed=seed)
    init = {"AL": [dev(O.mps_vec(a)) for a in AL], "AR": [dev(O.mps_vec(a)) for a in AR],
            "C": [dev(O.bd_vec(C[1])), dev(O.bd_vec(C[0]))]}  # C[b] = C on bond b
    gpu = VumpsGPU(cuda_ctx, model, dimvec=dimvec, init_state=init, fixed_tol=fixed_tol, **params)
    return ora, gpu


BH = {(-2,): 1, (-1,): 3, (0,): 4, (1,): 3, (2,): 1}


@pytest.mark.parametrize("model,dimvec,params", [
    ("xxz", [B0, B1], {"J": 1.0, "Delta": -1.0}),
    ("fhub", None, {"t": 1.0, "U": 4.0}),
    ("bhub", [BH, BH], {"d": 4, "t": 0.3, "U": 2.0, "n": 2}),
])
def test_vumps_sweeps_match_oracle(cuda_ctx, model, dimvec, params):
    if dimvec is None:
        dims0 = {(0, 0): 4, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2, (2, 0): 1, (0, 2): 1, (-2, 0): 1,
                 (0, -2): 1}
        dimvec = models.make_dims(dims0, 2, models.fhub_i2k())
    ora, gpu = _pair(cuda_ctx, model, dimvec, seed=7, **params)
    # Sweep 0 must agree to 1e-9.  Later sweeps of this far-from-converged start run the SVD
    # polar step (prec > 5e-7, VUMPS_main.cpp:211-220), whose polar factor amplifies the
    # 1e-12-level differences between ARPACK and the device Lanczos (different Krylov
    # sequences, same tolerance); there the trajectories agree to ~1e-7.
    for sweep in range(3):
        Eo, Fo, po = ora.sweep()
        Eg, Fg, pg = gpu.sweep()
        tol = 1e-9 if sweep == 0 else 1e-5
        assert np.abs(Eg - Eo).max() < tol, (sweep, Eg, Eo)
        assert np.allclose(Fg, Fo, rtol=1e-3 if sweep else 1e-5, atol=1e-12), (sweep, Fg, Fo)
        assert np.allclose(pg, po, rtol=1e-3 if sweep else 1e-4, atol=1e-12), (sweep, pg, po)


def test_vumps_gpu_bethe_ansatz(cuda_ctx):
    gpu = VumpsGPU(cuda_ctx, "xxz", dimvec=[B0, B1], seed=3, J=1.0, Delta=-1.0)
    for _ in range(14):
        E, F, prec = gpu.sweep()
    assert abs(E.mean() - (0.25 - math.log(2))) < 2e-4
    assert F.max() < 1e-3
    assert np.isfinite(E).all()


@pytest.fixture(scope="module")
def oracle_ground_state():
    """The oracle's VUMPS (VUMPS_main.cpp restated) run to |grad| < 1e-11 from a seeded state,
    reference tolerance schedule (tol = min(max(prec/100, 5e-16), 1e-6))."""
    d, I2K, h = models.build_model("xxz", J=1.0, Delta=-1.0)
    rng = np.random.default_rng(11)
    AL, AR, C = O.randMPS_LR(2, I2K, [B0, B1], rng)
    ora = O.VUMPS(h, d, I2K, B0, dimvec=[B0, B1], init=(AL, AR, C), InvETol=1e-13, seed=11)
    for _ in range(250):
        E, F, _ = ora.sweep()
        if F.max() < 1e-11:
            break
    assert F.max() < 1e-11
    return (AL, AR, C), E


@pytest.mark.parametrize("precision,tol_abs", [("fp64", None), ("bf16x6", 1e-9)])
def test_vumps_ground_state_energy_matches_oracle(cuda_ctx, oracle_ground_state, precision, tol_abs):
    """Independent runs to convergence from the same state: the FP64 ground-state energy density
    agrees with the oracle's to 1e-10 relative, the mixed (split-BF16) one to 1e-9."""
    (AL, AR, C), Eo = oracle_ground_state
    init = {"AL": [dev(O.mps_vec(a)) for a in AL], "AR": [dev(O.mps_vec(a)) for a in AR],
            "C": [dev(O.bd_vec(C[1])), dev(O.bd_vec(C[0]))]}
    gpu = VumpsGPU(cuda_ctx, "xxz", dimvec=[B0, B1], init_state=init, InvETol=1e-13, precision=precision,
                   J=1.0, Delta=-1.0)
    fmin, Eg = np.inf, None
    for _ in range(250):
        E, F, _ = gpu.sweep()
        if F.max() < fmin:
            fmin, Eg = F.max(), E
        if F.max() < 1e-11:
            break
    bound = 1e-10 * abs(Eo.mean()) if tol_abs is None else tol_abs
    assert abs(Eg.mean() - Eo.mean()) <= bound, (precision, Eg, Eo, fmin)
    if precision == "fp64":
        assert fmin < 1e-11


@pytest.mark.parametrize("model,params,dims,periods", [
    ("qim", {"J": 1.0, "h": 0.7}, {(0,): 6, (1,): 6}, (2,)),
    ("potts", {"q": 3, "h": 0.8}, {(0,): 4, (1,): 3, (2,): 3}, (3,)),
])
def test_zn_vumps_sweeps_match_oracle(cuda_ctx, model, params, dims, periods):
    """Z(N) charges (quantum Ising Z(2), Potts Z(3)): the GPU driver against the oracle run with
    the same modular charge arithmetic, from the same initial state."""
    dimvec = models.make_dims(dims, 2, models.build_model(model, **params)[1])
    with O.charge_group(periods):
        ora, gpu = _pair(cuda_ctx, model, dimvec, seed=7, **params)
        for sweep in range(3):
            Eo, Fo, po = ora.sweep()
            Eg, Fg, pg = gpu.sweep()
            # The shared initial state comes from the oracle's randMPS_LR, whose fixed-point solve
            # starts ARPACK from scipy's process-wide random state, so it moves at the 1e-14
            # level with test order.  From it, the nearly degenerate Z(2) effective Hamiltonians
            # of the first sweeps (ARPACK against the device Lanczos, both at tol 1e-12) agree to
            # 3e-9 .. 8e-7; a wrong sector shows at 1e-2.  The converged energy is pinned to the
            # exact solution by test_quantum_ising_exact_energy (GPU) and tests/test_oracle.py.
            assert np.abs(Eg - Eo).max() < 1e-5, (sweep, Eg, Eo)


def test_quantum_ising_exact_energy(cuda_ctx):
    """The transverse-field Ising energy (exact) through the GPU path with Z(2) sectors."""
    from scipy.integrate import quad
    J, h = 1.0, 0.7
    Jp, hp = J / 4, h / 2
    e0 = -quad(lambda k: math.sqrt(Jp ** 2 + hp ** 2 - 2 * Jp * hp * math.cos(k)), -math.pi, math.pi,
               epsabs=1e-14)[0] / (2 * math.pi)
    b = {(0,): 8, (1,): 8}
    gpu = VumpsGPU(cuda_ctx, "qim", dimvec=[b, b], seed=2, J=J, h=h)
    for _ in range(60):
        E, F, _ = gpu.sweep()
        if F.max() < 1e-11:
            break
    assert F.max() < 1e-10 and np.abs(E - e0).max() < 1e-10, (E, e0)
