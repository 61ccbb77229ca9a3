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


def test_energy_gradient_at_config_size_xxz_d256(cuda_ctx):
    """The adjoint check's XXZ D=256 shape: the gradient at the left-isometric unit cell of the GPU
    driver's seeded random start (a fixed input far from stationary) against the oracle, both
    environment solves converged to 1e-13.  States a few sweeps on are not used: the first sweeps
    from a random start are chaotic (a rounding-level change of any kernel moves the state they
    reach), and for some of those states the transfer-matrix systems do not resolve 1e-13 in
    either solver, which then leaves the two gradients ~1e-8 apart."""
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300.adjoint import EnergyGradientGPU
    from imps_cpp_tools_gb300.excitations import mps_to_host, bd_to_host
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    model, fn, params = configs.WORKLOADS["xxz_d256"]
    v = VumpsGPU(cuda_ctx, model, dims0=fn(), seed=2, **params)
    AL = [mps_to_host(v.AL[n], v.LA[n], v.d) for n in range(2)]
    C0 = bd_to_host(v.C[0], v.LB[0])
    R = O.bd_mul(C0, O.bd_t(C0))
    g = EnergyGradientGPU(cuda_ctx, v.LA, v.LB, v.hnnz, v.d, tol=1e-13)
    G0, G1, e, _, conv = g(v.AL[0], v.AL[1], dev(O.bd_vec(R)))
    Gref, eref = O.energy_gradient(AL, R, v.hnnz, tol=1e-13, solver=O.invert_e_proj_scipy)
    assert conv and abs(e - eref) < 1e-11 * abs(eref)
    for got, ref in ((host(G0), O.mps_vec(Gref[0])), (host(G1), O.mps_vec(Gref[1]))):
        assert np.linalg.norm(got - ref) <= 1e-8 * np.linalg.norm(ref)


def test_autograd_wrapper(cuda_ctx):
    """The gradient as the backward of a torch.autograd.Function (test harness only): autograd's
    gradient of e with respect to both site tensors equals the device gradient, and its
    directional derivative matches central differences of the oracle's energy."""
    import torch
    from imps_cpp_tools_gb300.adjoint import EnergyGradientGPU
    model, dims0, params = CASES[1]
    st = _state(model, dims0, params)
    AL, R, hnnz, d = st["AL"], st["R"], st["hnnz"], st["d"]
    LA, LB = _layouts(st)
    g = EnergyGradientGPU(cuda_ctx, LA, LB, hnnz, d, tol=1e-13)

    class Energy(torch.autograd.Function):
        @staticmethod
        def forward(fctx, A0, A1):
            G0, G1, e, _, _ = g(A0.detach(), A1.detach(), dev(O.bd_vec(R)))
            fctx.save_for_backward(G0.clone(), G1.clone())
            return torch.tensor(e, dtype=torch.float64, device=A0.device)

        @staticmethod
        def backward(fctx, ge):
            G0, G1 = fctx.saved_tensors
            return ge * G0, ge * G1

    A0 = dev(O.mps_vec(AL[0])).requires_grad_(True)
    A1 = dev(O.mps_vec(AL[1])).requires_grad_(True)
    e = Energy.apply(A0, A1)
    e.backward()
    Gref, eref = O.energy_gradient(AL, R, hnnz, tol=1e-14)
    assert abs(float(e) - eref) < 1e-12
    assert np.linalg.norm(host(A0.grad) - O.mps_vec(Gref[0])) <= 1e-9 * np.linalg.norm(O.mps_vec(Gref[0]))
    rng = np.random.default_rng(2)
    D = [[{q: (qo, rng.standard_normal(M.shape)) for q, (qo, M) in bm.items()} for bm in A] for A in AL]
    pert = lambda s: [[{q: (qo, M + s * D[n][k][q][1]) for q, (qo, M) in bm.items()} for k, bm in enumerate(A)]
                      for n, A in enumerate(AL)]
    eps = 1e-6
    fd = (O.energy_uniform(pert(eps), hnnz) - O.energy_uniform(pert(-eps), hnnz)) / (2 * eps)
    an = float(host(A0.grad) @ O.mps_vec(D[0]) + host(A1.grad) @ O.mps_vec(D[1]))
    assert abs(fd - an) <= 1e-6 * abs(fd)
