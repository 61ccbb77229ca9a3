"""The energy-density gradient on the device (imps_cpp_tools_gb300.adjoint: two grouped-GEMM
programs around two InvertE_proj solves on the transposed transfer matrices) against the
oracle's adjoint-method gradient, which the CPU tests pin to central finite differences."""
import numpy as np
import pytest

from oracle import imps_oracle as O
from tests import imps_testlib as T
from tests.test_gpu_parity import dev, host
from tests.test_oracle_adjoint import CASES, _state

pytestmark = pytest.mark.gpu


def _layouts(st):
    from imps_cpp_tools_gb300 import blocks as B
    ns = len(st["I2K"][0])
    C = st["C"]
    return ([B.Layout(T.mps_blocks(a), ns) for a in st["AL"]],
            [B.Layout(T.bd_blocks(C[1]), ns), B.Layout(T.bd_blocks(C[0]), ns)])


@pytest.mark.parametrize("model,dims0,params", CASES)
def test_energy_gradient_matches_oracle(cuda_ctx, model, dims0, params):
    from imps_cpp_tools_gb300.adjoint import EnergyGradientGPU
    st = _state(model, dims0, params)
    AL, R, hnnz, d = st["AL"], st["R"], st["hnnz"], st["d"]
    LA, LB = _layouts(st)
    g = EnergyGradientGPU(cuda_ctx, LA, LB, hnnz, d, tol=1e-13)
    G0, G1, e, _, conv = g(dev(O.mps_vec(AL[0])), dev(O.mps_vec(AL[1])), dev(O.bd_vec(R)))
    Gref, eref = O.energy_gradient(AL, R, hnnz, tol=1e-14)
    assert conv and abs(e - eref) < 1e-12 * max(1.0, abs(eref))
    for got, ref in ((host(G0), O.mps_vec(Gref[0])), (host(G1), O.mps_vec(Gref[1]))):
        assert np.linalg.norm(got - ref) <= 1e-9 * np.linalg.norm(ref)


def test_coupling_gradient_matches_oracle(cuda_ctx):
    from imps_cpp_tools_gb300.adjoint import CouplingGradientGPU, coupling_terms
    model, dims0, params = CASES[4]
    st = _state(model, dims0, params)
    LA, LB = _layouts(st)
    cg = CouplingGradientGPU(cuda_ctx, LA, LB, model, st["d"], **params)
    got = cg(dev(O.mps_vec(st["AL"][0])), dev(O.mps_vec(st["AL"][1])), dev(O.bd_vec(st["R"])))
    for name, hk in coupling_terms(model, **params):
        ref = O.energy_gradient(st["AL"], st["R"], hk, tol=1e-14)[1] if hk else 0.0
        assert abs(got[name] - ref) <= 1e-11 * max(1.0, abs(ref)), name


def test_energy_gradient_from_vumps_state_xxz_d256(cuda_ctx):
    """The adjoint check's XXZ D=256 shape: the gradient at the left-isometric unit cell of a GPU
    VUMPS state (a few sweeps from a random start, so far from stationary) against the oracle."""
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300.adjoint import EnergyGradientGPU
    from imps_cpp_tools_gb300.excitations import mps_to_host, bd_to_host
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    model, fn, params = configs.WORKLOADS["xxz_d256"]
    v = VumpsGPU(cuda_ctx, model, dims0=fn(), seed=2, **params)
    for _ in range(3):
        v.sweep()
    AL = [mps_to_host(v.AL[n], v.LA[n], v.d) for n in range(2)]
    C0 = bd_to_host(v.C[0], v.LB[0])
    R = O.bd_mul(C0, O.bd_t(C0))
    g = EnergyGradientGPU(cuda_ctx, v.LA, v.LB, v.hnnz, v.d, tol=1e-13)
    G0, G1, e, _, conv = g(v.AL[0], v.AL[1], dev(O.bd_vec(R)))
    Gref, eref = O.energy_gradient(AL, R, v.hnnz, tol=1e-13, solver=O.invert_e_proj_scipy)
    assert conv and abs(e - eref) < 1e-11 * abs(eref)
    for got, ref in ((host(G0), O.mps_vec(Gref[0])), (host(G1), O.mps_vec(Gref[1]))):
        assert np.linalg.norm(got - ref) <= 1e-8 * np.linalg.norm(ref)
