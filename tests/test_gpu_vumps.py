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


def warm_state(model, dimvec, seed, sweeps, fixed_tol=1e-12, **params):
    """The oracle's state after `sweeps` sweeps from randMPS_LR(seed), in randMPS_LR's
    arrangement (ALvec, ARvec, Cvec).  The first sweeps from a random state are chaotic: a
    1e-13 change of the start moves the energies of sweep 1 by up to 1e-3 in the oracle alone
    (tests/test_oracle.py::test_vumps_transient_is_chaotic); from a state a few sweeps on, the
    same change stays at the rounding level, so parity is checked from there."""
    import copy
    d, I2K, h = models.build_model(model, **params)
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, np.random.default_rng(seed))
    if sweeps == 0:
        return AL, AR, C
    ora = O.VUMPS(h, d, I2K, dimvec[0], dimvec=dimvec, init=(AL, AR, C), fixed_tol=fixed_tol, seed=seed)
    for _ in range(sweeps):
        ora.sweep()
    return copy.deepcopy(ora.AL), O.shift(copy.deepcopy(ora.AR), 1), copy.deepcopy(ora.C)


def _pair(cuda_ctx, model, dimvec, seed, fixed_tol=1e-12, warm=0, **params):
    d, I2K, h = models.build_model(model, **params)
    AL, AR, C = warm_state(model, dimvec, seed, warm, fixed_tol, **params)
    ora = O.VUMPS(h, d, I2K, dimvec[0], dimvec=dimvec, init=(AL, AR, C), fixed_tol=fixed_tol, seed=seed)
    init = {"AL": [dev(O.mps_vec(a)) for a in AL], "AR": [dev(O.mps_vec(a)) for a in AR],
            "C": [dev(O.bd_vec(C[1])), dev(O.bd_vec(C[0]))]}  # C[b] = C on bond b
    gpu = VumpsGPU(cuda_ctx, model, dimvec=dimvec, init_state=init, fixed_tol=fixed_tol, **params)
    return ora, gpu


BH = {(-2,): 1, (-1,): 3, (0,): 4, (1,): 3, (2,): 1}


@pytest.mark.parametrize("warm", [0, 5])
@pytest.mark.parametrize("model,dimvec,params", [
    ("xxz", [B0, B1], {"J": 1.0, "Delta": -1.0}),
    ("fhub", None, {"t": 1.0, "U": 4.0}),
    ("bhub", [BH, BH], {"d": 4, "t": 0.3, "U": 2.0, "n": 2}),
])
def test_vumps_sweeps_match_oracle(cuda_ctx, model, dimvec, params, warm):
    """The GPU driver against the oracle from the same state.  From the seeded random start
    (warm = 0) sweep 0 agrees to 1e-9; the sweeps after it run the SVD polar step on a state far
    from convergence, where the iteration itself amplifies rounding-level differences (in the
    oracle alone a 1e-13 change of the start moves sweep 2 by up to 5e-6, see warm_state), so
    they are held to 1e-5.  From the oracle's state after 5 sweeps (warm = 5) every sweep
    agrees to 1e-9."""
    if dimvec is None:
        dims0 = {(0, 0): 4, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2, (2, 0): 1, (0, 2): 1, (-2, 0): 1,
                 (0, -2): 1}
        dimvec = models.make_dims(dims0, 2, models.fhub_i2k())
    ora, gpu = _pair(cuda_ctx, model, dimvec, seed=7, warm=warm, **params)
    for sweep in range(3):
        Eo, Fo, po = ora.sweep()
        Eg, Fg, pg = gpu.sweep()
        tol = 1e-9 if (sweep == 0 or warm) else 1e-5
        assert np.abs(Eg - Eo).max() < tol, (sweep, Eg, Eo)
        assert np.allclose(Fg, Fo, rtol=1e-3 if (sweep or warm) else 1e-5, atol=1e-12), (sweep, Fg, Fo)
        assert np.allclose(pg, po, rtol=1e-3 if (sweep or warm) else 1e-4, atol=1e-12), (sweep, pg, po)


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
    the same modular charge arithmetic, from the same state: the oracle's after 5 sweeps from
    the seeded random start (the sweeps before are chaotic, see warm_state).  Every sweep
    agrees to 1e-9 in the energies."""
    dimvec = models.make_dims(dims, 2, models.build_model(model, **params)[1])
    with O.charge_group(periods):
        ora, gpu = _pair(cuda_ctx, model, dimvec, seed=7, warm=5, **params)
        for sweep in range(3):
            Eo, Fo, po = ora.sweep()
            Eg, Fg, pg = gpu.sweep()
            assert np.abs(Eg - Eo).max() < 1e-9, (sweep, Eg, Eo)
            assert np.allclose(Fg, Fo, rtol=1e-3, atol=1e-10), (sweep, Fg, Fo)


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


def test_sweep_from_warm_state_matches_oracle_full_size(cuda_ctx):
    """The benchmark's configuration at full size: XXZ D=512 (21 sectors), one sweep from the
    committed warmed state at eigensolver tol 1e-12 and GMRES tol 1e-8, on the GPU and in the
    oracle (ARPACK, the reference's GMRES): the energies agree to 1e-9 (measured 1.8e-10)."""
    import torch
    import bench
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300 import workload as W
    name = "xxz_d512"
    state = W.load_warm_state(name)
    assert state is not None
    model, fn, params = configs.WORKLOADS[name]
    init = {k: [torch.from_numpy(a).to("cuda") for a in state[k]] for k in ("AL", "AR", "C")}
    gpu = VumpsGPU(cuda_ctx, model, dims0=fn(), init_state=init, fixed_tol=bench.TIMED_TOLS["eig"],
                   InvETol=bench.TIMED_TOLS["gmres"], eig_margin=1.0, **params)
    Eg, Fg, _ = gpu.sweep()
    times, Eo, _, cut = bench.cpu_site_updates(name, state, 0, 2, 600.0)
    assert not cut
    assert np.abs(Eg - np.asarray(Eo)).max() < 1e-9, (Eg, Eo)


def test_concurrent_hc_solves_equal_serial(cuda_ctx):
    """The H_C eigensolves run on their own contexts and host threads beside the H_AC eigensolve,
    and the right-environment chain beside the left one (concurrent=True, the default), or all of
    them one after another on one stream: the sweeps are bit-identical (no state is shared
    between the solves), from the committed warmed XXZ D=512 state at the benchmark's
    tolerances."""
    import torch
    import bench
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300 import workload as W
    name = "xxz_d512"
    state = W.load_warm_state(name)
    model, fn, params = configs.WORKLOADS[name]
    runs = []
    for concurrent in (False, True):
        init = {k: [torch.from_numpy(a).to("cuda") for a in state[k]] for k in ("AL", "AR", "C")}
        gpu = VumpsGPU(cuda_ctx, model, dims0=fn(), init_state=init, fixed_tol=bench.TIMED_TOLS["eig"],
                       InvETol=bench.TIMED_TOLS["gmres"], eig_margin=1.0, concurrent=concurrent, **params)
        runs.append([gpu.sweep() for _ in range(2)] + [dict(gpu.stats)] + [gpu.host_state()])
    for a, b in zip(runs[0][:2], runs[1][:2]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y), (x, y)
    assert runs[0][2] == runs[1][2]
    for k in ("AL", "AR", "C"):
        for x, y in zip(runs[0][3][k], runs[1][3][k]):
            assert np.array_equal(x, y)
