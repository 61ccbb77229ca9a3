"""GPU parity of the per-sector decompositions (qr_pos QR, SVD / polar) against the oracle.
QR with diag(R) >= 0 and the polar factor U V^T are unique for full-rank sectors, so they are
compared element-wise (1e-11 relative); singular values to 1e-12 relative."""
import numpy as np
import pytest

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops
from oracle import imps_oracle as O
from tests import imps_testlib as T
from tests.test_gpu_parity import SMALL, dev, host, relerr

pytestmark = pytest.mark.gpu


def _rand_mps(model, dims0, seed):
    st = T.random_state(model, dims0, seed=seed)
    A = O.mps_rand(st["I2K"], st["dimvec"][0], st["dimvec"][1], st["rng"])
    return st, A


@pytest.mark.parametrize("model,dims0", SMALL + [("xxz", "xxz_d512")])
@pytest.mark.parametrize("direction", ["l", "r"])
def test_qr_mps(cuda_ctx, model, dims0, direction):
    if isinstance(dims0, str):
        model, dims0, _ = T.workload_dims(dims0)
    st, A = _rand_mps(model, dims0, 3)
    ns = len(st["I2K"][0])
    la = B.Layout(T.mps_blocks(A), ns)
    dec = B.plan_decomp(cuda_ctx, la, direction)
    Q, R = dev(np.zeros(la.nelem)), dev(np.zeros(dec.rlayout.nelem))
    ops.qr(dec, dev(O.mps_vec(A)), Q, R)
    Qr, Rr = O.qr_mps(A, direction)
    assert relerr(host(Q), O.mps_vec(Qr)) < 1e-11
    assert relerr(host(R), O.bd_vec(Rr)) < 1e-11


@pytest.mark.parametrize("direction", ["l", "r"])
def test_qr_blockdiag(cuda_ctx, direction):
    rng = np.random.default_rng(2)
    X = {(q,): rng.standard_normal((m, m)) for q, m in zip(range(-3, 4), [1, 2, 5, 9, 5, 2, 1])}
    lx = B.Layout(T.bd_blocks(X), 1)
    dec = B.plan_decomp(cuda_ctx, lx, direction)
    Q, R = dev(np.zeros(lx.nelem)), dev(np.zeros(lx.nelem))
    ops.qr(dec, dev(O.bd_vec(X)), Q, R)
    Qr, Rr = O.qr_bd(X, direction)
    assert relerr(host(Q), O.bd_vec(Qr)) < 1e-11
    assert relerr(host(R), O.bd_vec(Rr)) < 1e-11


@pytest.mark.parametrize("model,dims0", SMALL)
@pytest.mark.parametrize("direction", ["l", "r"])
def test_svd_polar(cuda_ctx, model, dims0, direction):
    st, A = _rand_mps(model, dims0, 5)
    ns = len(st["I2K"][0])
    la = B.Layout(T.mps_blocks(A), ns)
    dec = B.plan_decomp(cuda_ctx, la, direction)
    U, S, V = dev(np.zeros(la.nelem)), dev(np.zeros(dec.nsv)), dev(np.zeros(dec.rlayout.nelem))
    assert ops.svd(dec, dev(O.mps_vec(A)), U, S, V)
    Iso, Sr, DI = O.svd_mps(A, direction)
    sref = np.concatenate([Sr[q] for q in sorted(Sr)])
    assert relerr(host(S), sref) < 1e-12
    # polar factor: l -> Iso * DiagIso, r -> DiagIso * Iso (unique for full rank)
    lr = dec.rlayout
    pol = B.plan_mps_bd(cuda_ctx, la, lr, 1 if direction == "l" else 0)
    out = dev(np.zeros(la.nelem))
    pol.bind(0, U); pol.bind(1, V); pol.bind(2, out); pol.run()
    ref = O.mps_mul_bd(Iso, DI) if direction == "l" else O.bd_mul_mps(DI, Iso)
    assert relerr(host(out), O.mps_vec(ref)) < 1e-10


def test_svd_batch_equals_single_launches(cuda_ctx):
    """imps_sector_svd_batch (the two polar SVDs of a site update in one launch) gives exactly the
    outputs of separate imps_sector_svd calls on each plan."""
    st, A = _rand_mps("xxz", {(-2,): 3, (0,): 6, (2,): 3}, 5)
    ns = len(st["I2K"][0])
    la = B.Layout(T.mps_blocks(A), ns)
    decs = [B.plan_decomp(cuda_ctx, la, "l"), B.plan_decomp(cuda_ctx, la, "r")]
    a = dev(O.mps_vec(A))
    rng = np.random.default_rng(9)
    a2 = dev(O.mps_vec(A) + 0.1 * rng.standard_normal(la.nelem))
    single, batch = [], []
    for dec, x in zip(decs, (a, a2)):
        U, S, V = dev(np.zeros(la.nelem)), dev(np.zeros(dec.nsv)), dev(np.zeros(dec.rlayout.nelem))
        assert ops.svd(dec, x, U, S, V)
        single.append((host(U), host(S), host(V)))
    outs = [(dev(np.zeros(la.nelem)), dev(np.zeros(d.nsv)), dev(np.zeros(d.rlayout.nelem))) for d in decs]
    assert ops.svd_batch(decs, [a, a2], [o[0] for o in outs], [o[1] for o in outs], [o[2] for o in outs])
    for (U, S, V), ref in zip(outs, single):
        for got, r in zip((host(U), host(S), host(V)), ref):
            assert np.array_equal(got, r)


def test_colscale(cuda_ctx):
    rng = np.random.default_rng(4)
    X = {(q,): rng.standard_normal((m, m)) for q, m in zip(range(3), [2, 4, 3])}
    lx = B.Layout(T.bd_blocks(X), 1)
    dec = B.plan_decomp(cuda_ctx, lx, "l")
    s = rng.uniform(0.5, 2.0, dec.nsv)
    x = dev(O.bd_vec(X))
    ops.colscale(dec, x, dev(s), 0.5)
    ref, o = {}, 0
    for q in sorted(X):
        m = X[q].shape[0]
        ref[q] = X[q] * np.sqrt(s[o:o + m])[None, :]
        o += m
    assert relerr(host(x), O.bd_vec(ref)) < 1e-14
