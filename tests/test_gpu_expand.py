"""ExpandFromH on the GB300 (MPSBlockUtilities.hpp:409-601) and VUMPS with bond expansion
(VUMPS_main.cpp:270-308).

* The device expansion against the oracle's restatement on the same state: the same number of
  states per charge, the same new directions (AL' W AR' with W the new singular values on the
  new states, independent of the null-space basis and of singular-vector signs), AL C AR
  unchanged, isometries kept.
* A VUMPS run from a small bond dimension grows the bond through the driver up to mmax and
  ends closer to the Heisenberg ground-state energy than the fixed small bond dimension.
"""
import math

import numpy as np
import pytest

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import expand as E
from imps_cpp_tools_gb300 import models
from imps_cpp_tools_gb300.vumps import VumpsGPU
from oracle import imps_oracle as O
from tests.test_expand import FHUB0, _max_diff, _two_site, _weighted
from tests.test_gpu_parity import dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model", ["xxz", "fhub"])
@pytest.mark.parametrize("dmmax", [3, 30])
def test_device_expansion_matches_oracle(cuda_ctx, model, dmmax):
    params = {"J": 1.0, "Delta": -1.0} if model == "xxz" else {"t": 1.0, "U": 4.0}
    d, I2K, h = models.build_model(model, **params)
    hnnz = models.h_nonzeros(h)
    dims0 = {(-4,): 2, (-2,): 4, (0,): 6, (2,): 4, (4,): 2} if model == "xxz" else FHUB0
    dimvec = models.make_dims(dims0, 2, I2K)
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, np.random.default_rng(8))
    AL, AR, C = AL[0], AR[1], C[0]
    LA = B.Layout.mps(I2K, dimvec[0], dimvec[1])
    LR = B.Layout.mps(I2K, dimvec[1], dimvec[0])
    LC = B.Layout.blockdiag(dimvec[1])
    res = E.expand_from_h(cuda_ctx, I2K, hnnz, LA, dev(O.mps_vec(AL)), LR, dev(O.mps_vec(AR)), LC,
                          dev(O.bd_vec(C)), dmmax)
    assert res["converged"]
    ALo, ARo, Co, dmo = O.ExpandFromH(hnnz, I2K, AL, AR, C, dmmax)
    assert {q: k for q, k in res["dm"].items() if k} == {q: k for q, k in dmo.items() if k}
    sizes = lambda L: [[(qi, qo, r, c) for (g, qi, qo, r, c) in L.blocks if g == s] for s in range(d)]
    ALd = O.mps_from_vec(res["AL"].cpu().numpy()[:res["LA"].nelem], sizes(res["LA"]))
    ARd = O.mps_from_vec(res["AR"].cpu().numpy()[:res["LR"].nelem], sizes(res["LR"]))
    Cd = O.bd_from_vec(res["C"].cpu().numpy()[:res["LC"].nelem], [(b[1], b[3]) for b in res["LC"].blocks])
    assert set(Cd) == set(Co) and all(np.array_equal(Cd[q], Co[q]) for q in Co)
    assert _max_diff(_two_site(AL, C, AR), _two_site(ALd, Cd, ARd)) < 1e-13
    lam = res["lam"]
    err = _max_diff(_weighted(ALd, ARd, Cd, res["dm"], lam), _weighted(ALo, ARo, Co, dmo, lam))
    assert err < 1e-10, err
    for q, G in O.GetDenseMat(ALd, "l").items():
        assert np.allclose(G[0].T @ G[0], np.eye(G[0].shape[1]), atol=1e-11)
    for q, G in O.GetDenseMat(ARd, "r").items():
        assert np.allclose(G[0] @ G[0].T, np.eye(G[0].shape[0]), atol=1e-11)


def test_vumps_grows_the_bond(cuda_ctx):
    """Heisenberg chain from D ~ 7 per bond, mmax 40, dmmax 8, expansion after every second
    site update once the previous sweep's error is below 1e-5 (VUMPS_main.cpp:277)."""
    XXZ = {"J": 1.0, "Delta": -1.0}
    dimvec = models.make_dims({(-2,): 2, (0,): 3, (2,): 2}, 2, models.build_model("xxz", **XXZ)[1])
    fixed = VumpsGPU(cuda_ctx, "xxz", dimvec=dimvec, seed=4, **XXZ)
    grow = VumpsGPU(cuda_ctx, "xxz", dimvec=dimvec, seed=4, mmax=40, dmmax=8, expand_pause=2, **XXZ)
    for _ in range(30):
        Ef, Ff, _ = fixed.sweep()
    for _ in range(120):
        Eg, Fg, pg = grow.sweep()
        if not grow.keep_running(1e-9):
            break
    dims = [sum(grow.LB[b].dims().values()) for b in range(2)]
    e0 = 0.25 - math.log(2)
    assert grow.stats["expansions"] >= 4
    assert all(sum(dimvec[b].values()) < dims[b] <= 40 for b in range(2)), dims
    assert np.isfinite(Eg).all() and Fg.max() < 1e-6 and pg.max() < 1e-6
    assert Eg.mean() < Ef.mean() - 1e-4, (Eg, Ef)  # the grown bond is variationally better
    assert abs(Eg.mean() - e0) < 1e-3, Eg
    # the final state is a consistent mixed-canonical cell: AL(n) C[n+1] = C[n] AR(n)
    st = grow.imps_state()
    for n in range(2):
        Cr, Cl = st.C[n], st.C[(n + 1) % 2]
        err = max(float(np.abs(al @ Cr[qo] - Cl[q] @ st.AR[n].blocks[s][q][1]).max())
                  for s in range(grow.d) for q, (qo, al) in st.AL[n].blocks[s].items())
        # |AL C - C AR| <= |AL CR - AC| + |AC - CL AR|, the per-site errors behind prec
        assert err < 1e-5, (err, pg)
