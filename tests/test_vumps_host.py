"""Host logic of the VUMPS drivers without a GPU: the site loops of vumps.VumpsGPU (two sites) and
vumps_cell.VumpsCellGPU (any N) run on a host-only context (plans are sector tables only) with
every device operation replaced by a recorder.  Checked: every tensor bound to a plan slot has
the slot's size (a mismatch would be an out-of-bounds access on the device), every external slot
of a plan is bound when it runs, and the environments live on the bonds of the drivers'
convention (EHL on bond n, EHR on bond n+1, EHL1 on bond n+1, EHR1 on bond n at site n).  The
sector dimensions differ from bond to bond so that a tensor of the wrong bond is caught."""
import ctypes as C

import numpy as np
import pytest
import torch

from imps_cpp_tools_gb300 import _native as N
from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import ops

Q = lambda *p: {(q,): m for q, m in p}  # noqa: E731
CASES = [
    ("qim", [Q((0, 6), (1, 5)), Q((0, 4), (1, 7)), Q((0, 3), (1, 2))], dict(J=1.0, h=0.7)),
    ("qim", [Q((0, 6), (1, 5)), Q((0, 4), (1, 7)), Q((0, 3), (1, 2)), Q((0, 8), (1, 1))], dict(J=1.0, h=0.7)),
    ("xxz", [Q((-2, 2), (0, 3), (2, 2)), Q((-1, 4), (1, 1), (3, 2))], dict(J=1.0, Delta=-1.0)),
    ("xxz", [Q((-2, 2), (0, 3), (2, 2)), Q((-1, 4), (1, 1), (3, 2)), Q((0, 5), (2, 2), (-2, 1)),
             Q((-1, 3), (1, 3), (-3, 1))], dict(J=1.0, Delta=-1.0)),
]


def _slot(plan, s):
    k, n = C.c_int(), C.c_int64()
    N.call("imps_plan_slot_info", plan.handle, s, C.byref(k), C.byref(n))
    return k.value, n.value


@pytest.fixture
def fake_device(monkeypatch):
    """Host-only execution: CPU tensors, plan runs and solver calls recorded instead of launched.
    Returns the list of violations found."""
    errors = []

    def check_bound(plan, what, skip=()):
        for s in range(plan.info()["nslots"]):
            kind, _ = _slot(plan, s)
            if kind == 0 and s not in plan._bound and s not in skip:
                errors.append(("unbound", plan.kind, what, s))

    def bind(self, slot, t):
        _, n = _slot(self, slot)
        if t.numel() != n:
            errors.append(("size", self.kind, slot, t.numel(), n))
        self._bound[slot] = t

    def same(*ts):
        if len({t.numel() for t in ts}) != 1:
            errors.append(("vector sizes", [t.numel() for t in ts]))

    def tm_solve(plan, *vecs):  # in / out of a TM plan are the solver's own vectors
        check_bound(plan, "tm solve", skip=(0, 1))
        n0 = _slot(plan, 0)[1]
        for v in vecs:
            if v is not None and v.numel() != n0:
                errors.append(("tm vector", v.numel(), n0))

    def trace(ctx, lay, X, Y):
        if not X.numel() == Y.numel() == lay.nelem:
            errors.append(("trace", lay.nelem, X.numel(), Y.numel()))
        return 0.0

    fakes = {
        "eigs_rs": lambda plan, x, tol, **k: (check_bound(plan, "eigs", skip=(0, 1)), (0.0, 1, True))[1],
        "ApplyHAvec": lambda plan, i, o: check_bound(plan, "apply", skip=(0, 1)),
        "InvertE_proj": lambda plan, x, L, R, d, y, tol, **k: (tm_solve(plan, x, L, R, y), (1, 0.0, True))[1],
        "TMDominantEig": lambda plan, V, x0=None, tol=0, **k: (tm_solve(plan, V, x0), (1.0, 1, True))[1],
        "GradNormRight": lambda plan: (check_bound(plan, "grad"), 0.0)[1],
        "axpby": lambda ctx, a, x, b, y: (same(x, y), y)[1],
        "norm_inf": lambda ctx, x: 0.0,
        "sign_normalize": lambda ctx, x: x,
        "bd_trace_prod": trace,
        "qr": lambda dec, A, Q_, R: None,
        "svd": lambda *a, **k: None,
        "svd_batch": lambda *a, **k: None,
        "colscale": lambda *a, **k: None,
    }
    for name, f in fakes.items():
        monkeypatch.setattr(ops, name, f)
    monkeypatch.setattr(B.Plan, "bind", bind)
    monkeypatch.setattr(B.Plan, "run", lambda self: check_bound(self, "run"))
    monkeypatch.setattr(B.Plan, "prepare", lambda self: None)
    zeros, tensor = torch.zeros, torch.tensor
    monkeypatch.setattr(torch, "zeros", lambda *a, device=None, **k: zeros(*a, **k))
    monkeypatch.setattr(torch, "tensor", lambda *a, device=None, **k: tensor(*a, **k))
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: None)
    return errors


def _init(dimvec, I2K, LA, LB):
    return {"AL": [torch.zeros(l.nelem, dtype=torch.float64) for l in LA],
            "AR": [torch.zeros(l.nelem, dtype=torch.float64) for l in LA],
            "C": [torch.zeros(l.nelem, dtype=torch.float64) for l in LB]}


def _sweeps(v, n_sites, errors, sweeps=2):
    for _ in range(sweeps):
        for n in range(n_sites):
            for name, t, b in (("EHL", v.EHL, n), ("EHR", v.EHR, (n + 1) % n_sites),
                               ("EHL1", v.EHL1, (n + 1) % n_sites), ("EHR1", v.EHR1, n)):
                if t.numel() != v.LB[b].nelem:
                    errors.append(("environment bond", name, n, b))
            v.site_update(n)
        v.energy()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_cell_driver_host_logic(fake_device, case):
    from imps_cpp_tools_gb300 import models
    from imps_cpp_tools_gb300.vumps_cell import VumpsCellGPU
    model, dimvec, params = CASES[case]
    n_sites = len(dimvec)
    _, I2K, _ = models.build_model(model, **params)
    LA = [B.Layout.mps(I2K, dimvec[n], dimvec[(n + 1) % n_sites]) for n in range(n_sites)]
    LB = [B.Layout.blockdiag(dimvec[b]) for b in range(n_sites)]
    assert len({l.nelem for l in LB}) >= min(n_sites, 3)
    v = VumpsCellGPU(B.Context(-1), model, n_sites, dimvec=dimvec, init_state=_init(dimvec, I2K, LA, LB),
                     fixed_tol=1e-12, **params)
    _sweeps(v, n_sites, fake_device)
    assert fake_device == []


def test_two_site_driver_host_logic(fake_device):
    from imps_cpp_tools_gb300 import models
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    model, dimvec, params = CASES[2]
    _, I2K, _ = models.build_model(model, **params)
    LA = [B.Layout.mps(I2K, dimvec[n], dimvec[1 - n]) for n in range(2)]
    LB = [B.Layout.blockdiag(dimvec[b]) for b in range(2)]
    v = VumpsGPU(B.Context(-1), model, dimvec=dimvec, init_state=_init(dimvec, I2K, LA, LB), fixed_tol=1e-12,
                 concurrent=False, **params)
    _sweeps(v, 2, fake_device)
    assert fake_device == []


def test_two_site_driver_host_logic_concurrent(fake_device, monkeypatch):
    """The concurrent path (H_C eigensolves and the right-environment chain on side contexts from
    worker threads, with their own transfer-matrix plans) binds every slot with the right size
    too; the streams are stand-ins."""
    import contextlib
    from imps_cpp_tools_gb300 import models
    from imps_cpp_tools_gb300.vumps import VumpsGPU

    class _Stream:
        cuda_stream = 0

        def wait_stream(self, other):
            pass

    monkeypatch.setattr(torch.cuda, "Stream", _Stream)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: _Stream())
    monkeypatch.setattr(torch.cuda, "stream", lambda s: contextlib.nullcontext())
    monkeypatch.setattr(torch.Tensor, "record_stream", lambda self, s: None)
    model, dimvec, params = CASES[2]
    _, I2K, _ = models.build_model(model, **params)
    LA = [B.Layout.mps(I2K, dimvec[n], dimvec[1 - n]) for n in range(2)]
    LB = [B.Layout.blockdiag(dimvec[b]) for b in range(2)]
    v = VumpsGPU(B.Context(-1), model, dimvec=dimvec, init_state=_init(dimvec, I2K, LA, LB), fixed_tol=1e-12,
                 concurrent=True, **params)
    assert v._env is not None and all(p.ctx is v._side_ctx[1] for p in v._env.tm.values())
    assert all(p.ctx is v._side_ctx[0] for p in v.p_hcl) and all(p.ctx is v._side_ctx[1] for p in v.p_hcr)
    _sweeps(v, 2, fake_device)
    assert fake_device == []


def test_host_logic_check_catches_a_wrong_bond(fake_device, monkeypatch):
    """The recorder is not blind: a GetHR that returns the source on the wrong bond is caught."""
    from imps_cpp_tools_gb300 import models
    from imps_cpp_tools_gb300.vumps_cell import VumpsCellGPU
    model, dimvec, params = CASES[0]
    _, I2K, _ = models.build_model(model, **params)
    LA = [B.Layout.mps(I2K, dimvec[n], dimvec[(n + 1) % 3]) for n in range(3)]
    LB = [B.Layout.blockdiag(dimvec[b]) for b in range(3)]
    good = VumpsCellGPU._get_hr
    monkeypatch.setattr(VumpsCellGPU, "_get_hr", lambda self, n: good(self, (n + 1) % self.N))
    v = VumpsCellGPU(B.Context(-1), model, 3, dimvec=dimvec, init_state=_init(dimvec, I2K, LA, LB),
                     fixed_tol=1e-12, **params)
    _sweeps(v, 3, fake_device, sweeps=1)
    assert any(e[0] == "tm vector" for e in fake_device)
    assert np.isfinite(v.prec).all()
