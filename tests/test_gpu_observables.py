"""MeasureObservables on the GB300 (VumpsGPU.measure) against the oracle's restatement of
MPSBlockUtilities.hpp:1017-1073 on the downloaded state, for every operator of GetObservables
(Models.cpp:95-147, 575-632), and the energy as the two-site observable h."""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import models
from imps_cpp_tools_gb300.excitations import bd_to_host, mps_to_host
from imps_cpp_tools_gb300.vumps import VumpsGPU
from oracle import imps_oracle as O
from tests.test_expand import FHUB0

pytestmark = pytest.mark.gpu


BH = {(-2,): 1, (-1,): 3, (0,): 4, (1,): 3, (2,): 1}
NAMES = {"xxz": ["sx", "syi", "sz", "sp", "sm", "rx", "rz"],
         "fhub": ["cup", "cdo", "cupd", "cdod", "nup", "ndo", "sz", "n", "rx", "rz"],
         "bhub": ["b", "b2", "n", "nmax"]}
PARAMS = {"xxz": {"J": 1.0, "Delta": -1.0}, "fhub": {"t": 1.0, "U": 4.0}, "bhub": {"d": 4, "t": 0.3, "U": 2.0, "n": 2}}


@pytest.mark.parametrize("model", ["xxz", "fhub", "bhub"])
def test_observables_match_oracle(cuda_ctx, model):
    params = PARAMS[model]
    d, I2K, h = models.build_model(model, **params)
    if model == "bhub":
        dimvec = [BH, BH]
    else:
        dims0 = {(-4,): 2, (-2,): 4, (0,): 6, (2,): 4, (4,): 2} if model == "xxz" else FHUB0
        dimvec = models.make_dims(dims0, 2, I2K)
    v = VumpsGPU(cuda_ctx, model, dimvec=dimvec, seed=3, **params)
    for _ in range(4):
        v.sweep()
    names = NAMES[model]
    got = v.measure(names)
    AR = [mps_to_host(v.AR[n], v.LA[n], d) for n in range(2)]
    Cb = [bd_to_host(v.C[b], v.LB[b]) for b in range(2)]
    L = [O.bd_mul(O.bd_t(Cb[(m + 1) % 2]), Cb[(m + 1) % 2]) for m in range(2)]  # left of site m + 1
    ref = O.MeasureObservables(models.observables(model, names, d=d), AR, L)
    for n in names:
        # device order: entry 0 is site 1, entry 1 site 0
        assert np.allclose(got[n], ref[n][::-1], atol=1e-12, rtol=0), (n, got[n], ref[n])
    e = v.measure([("h", h)])["h"]
    assert np.allclose(e, v.energy(), atol=1e-13, rtol=0)
    if model == "fhub":
        # N = 2 per cell up to the gauge error of a state four sweeps from its random start (L =
        # C^T C and AR agree to O(prec)); the exact identity is a CPU test on an exact state
        assert abs(got["n"].sum() - 2.0) < 1e-3
