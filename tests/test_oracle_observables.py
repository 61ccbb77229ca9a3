"""MeasureObservables (MPSBlockUtilities.hpp:1017-1073, dir r) in the oracle, and the operator
tables of GetObservables (Models.cpp:95-147, 575-632).

* With O = h it is the energy per bond of the VUMPS driver (energy_right).
* A one-site O equals O x 1 on the two-site product AR(n) AR(n+1) (AR(n+1) right-isometric):
  the form the device evaluates.
* Charge-changing operators give exactly zero (the BlockMat trace sums only blocks with equal
  charges, BlockObj.hpp:1340-1350).
* The unit-cell sums of conserved densities are the sector's charges: N = 2 and Sz = 0 per
  two-site cell for Fermi-Hubbard at half filling (QN = [2, 0]), Sz = 0 for XXZ (QN = [0]).
"""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import models
from oracle import imps_oracle as O
from tests.test_expand import FHUB0


def _state(model, seed=6):
    params = {"J": 1.0, "Delta": -1.0} if model == "xxz" else {"t": 1.0, "U": 4.0}
    d, I2K, h = models.build_model(model, **params)
    dims0 = {(-2,): 2, (0,): 3, (2,): 2} if model == "xxz" else FHUB0
    dimvec = models.make_dims(dims0, 2, I2K)
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, np.random.default_rng(seed))
    # C[m] is right of site m; L left of site n = C[n-1]^T C[n-1]
    L = [O.bd_mul(O.bd_t(Cm), Cm) for Cm in C]
    return d, h, AR, L


@pytest.mark.parametrize("model", ["xxz", "fhub"])
def test_energy_is_the_two_site_observable(model):
    d, h, AR, L = _state(model)
    got = O.MeasureObservables([("h", h)], AR, L)["h"]
    ref = O.energy_right(models.h_nonzeros(h), AR, L)
    assert np.allclose(got, ref, atol=1e-14, rtol=0)


@pytest.mark.parametrize("model", ["xxz", "fhub"])
def test_one_site_operators(model):
    d, h, AR, L = _state(model)
    names = ["sx", "syi", "sz", "sp", "sm", "rx", "rz"] if model == "xxz" else \
        ["cup", "cdo", "cupd", "cdod", "nup", "ndo", "sz", "n", "rx", "rz"]
    ops = models.observables(model, names + ["nonsense"])
    assert [n for n, _ in ops] == names
    one = O.MeasureObservables(ops, AR, L)
    two = O.MeasureObservables([(n, np.kron(m, np.eye(d))) for n, m in ops], AR, L)
    for n in names:
        assert np.allclose(one[n], two[n], atol=1e-14, rtol=0), n
    zero = ["sx", "syi", "sp", "sm", "rx"] if model == "xxz" else ["cup", "cdo", "cupd", "cdod"]
    for n in zero:
        assert np.all(one[n] == 0.0), n
    assert abs(one["sz"].sum()) < 1e-13
    if model == "fhub":
        assert abs(one["n"].sum() - 2.0) < 1e-13
        assert np.allclose(one["n"], one["nup"] + one["ndo"], atol=1e-14)
    else:
        assert np.allclose(one["rz"], 2 * one["sz"], atol=1e-14)


def test_mixed_operator_follows_the_reference_map_insertion():
    """Fermi-Hubbard "rx" mixes charge-conserving (0,0), (3,3) and Sz-changing (1,2), (2,1)
    entries.  The reference keeps, per incoming charge, the first block ApplyTMmixedRight
    creates (std::map::emplace_hint), so its value is the conserving part traced over the
    sectors whose first block is diagonal: VumpsGPU.first_block_sectors, checked here against
    the oracle's literal evaluation on the layouts the device uses."""
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    d, I2K, _ = models.build_model("fhub", t=1.0, U=4.0)
    dimvec = models.make_dims(FHUB0, 2, I2K)
    _, h, AR, L = _state("fhub")
    rx = dict(models.observables("fhub", ["rx"]))["rx"]
    cons = np.where(np.array([[I2K[r] == I2K[c] for c in range(d)] for r in range(d)]), rx, 0.0)
    literal = O.MeasureObservables([("rx", rx)], AR, L)["rx"]
    for n in range(2):
        LA = B.Layout.mps(I2K, dimvec[n], dimvec[1 - n])
        sel = VumpsGPU.first_block_sectors(LA, I2K, rx, sorted(dimvec[n]))
        X = O.ApplyTMmixedRight(O.ApplyOperator(AR[n], models.h_nonzeros(cons)), AR[n])
        Lm = L[(n - 1) % 2]
        val = sum(np.trace(Lm[q] @ M) for q, (qo, M) in X.items() if q == qo and q in sel)
        assert abs(val - literal[n]) < 1e-14, (n, val, literal[n])
    full = O.MeasureObservables([("c", cons)], AR, L)["c"]
    assert np.abs(full - literal).max() > 1e-3  # the dropped blocks matter on this state
