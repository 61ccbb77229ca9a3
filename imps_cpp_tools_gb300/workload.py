"""Synthetic H_AC / H_C / TM workloads built with the product path only (numpy RNG for the
seeded inputs, native plans for every derived operator)."""
from __future__ import annotations

import numpy as np

from . import blocks as B
from . import configs, models


def bond_layouts(name):
    model, dims_fn, params = configs.WORKLOADS[name]
    d, I2K, h = models.build_model(model, **params)
    dimvec = models.make_dims(dims_fn(), 2, I2K)
    return model, d, I2K, h, dimvec


class HacWorkload:
    """H_AC apply on the two-site unit cell: AC(n) = C(n-1) AR(n) with AL(n-1) to its left and
    AR(n+1) to its right (VUMPS_main.cpp:179-186).  Operator values are seeded random (the
    apply cost does not depend on them); HL/HR come from the native ReducedOp plan."""

    def __init__(self, ctx, name="xxz_d512", seed=20261203):
        import torch
        self.name = name
        model, d, I2K, h, dimvec = bond_layouts(name)
        self.d, self.I2K, self.h, self.dimvec = d, I2K, h, dimvec
        self.hnnz = models.h_nonzeros(h)
        ns = len(I2K[0])
        b0, b1 = dimvec
        rng = np.random.default_rng(seed)
        self.rng = rng
        dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
        self.dev = dev
        # site n maps bond0 -> bond1, site n-1 / n+1 map bond1 -> bond0
        self.lac = B.Layout.mps(I2K, b0, b1)
        lal = B.Layout.mps(I2K, b1, b0)
        self.lehl = B.Layout.blockdiag(b0)
        self.lehr = B.Layout.blockdiag(b1)
        scale = 1.0 / np.sqrt(max(sum(b0.values()), 1))
        AL = dev(rng.standard_normal(lal.nelem) * scale)
        AR = dev(rng.standard_normal(lal.nelem) * scale)
        phl = B.plan_redop(ctx, lal, d, self.hnnz, 0)
        phr = B.plan_redop(ctx, lal, d, self.hnnz, 1)
        self.lhl, self.lhr = phl.derived(0), phr.derived(0)
        HL, HR = dev(np.zeros(self.lhl.nelem)), dev(np.zeros(self.lhr.nelem))
        phl.bind(0, AL); phl.bind(1, HL); phl.run()
        phr.bind(0, AR); phr.bind(1, HR); phr.run()

        def sym_bd(lay):
            v = np.zeros(lay.nelem)
            for (g, qi, qo, r, c), o in zip(lay.blocks, lay.offsets):
                M = rng.standard_normal((r, c))
                v[o:o + r * c] = (0.5 * (M + M.T)).reshape(-1, order="F")
            return dev(v)

        self.EHL, self.EHR, self.HL, self.HR = sym_bd(self.lehl), sym_bd(self.lehr), HL, HR
        self.plan = B.plan_hac(ctx, self.lac, self.lehl, self.lehr, self.lhl, self.lhr, d)
        for s, t in ((2, self.EHL), (3, self.EHR), (4, self.HL), (5, self.HR)):
            self.plan.bind(s, t)
        self.flops = self.plan.info()["flops_apply"]
        self.n = self.lac.nelem

    def bytes_per_apply(self):
        """Algorithmic bytes of one apply: read in + write out + read every operator once."""
        return 8 * (2 * self.n + self.lehl.nelem + self.lehr.nelem + self.lhl.nelem + self.lhr.nelem)

    def host_copies(self):
        """numpy copies of every operand (for the CPU baseline restatement)."""
        return {k: getattr(self, k).cpu().numpy() for k in ("EHL", "EHR", "HL", "HR")}


# ------------------------------------------------------------------------------------------------
# VUMPS start states of the sweep benchmark
# ------------------------------------------------------------------------------------------------

# sweeps of the reference's tolerance schedule (VUMPS_main.cpp:177) from randMPS_LR(seed 1)
# before a state counts as warmed: past the chaotic first sweeps of a random start
WARM_SWEEPS = {"xxz_d512": 20, "hubbard_d1024": 30}
WARM_SEED = 1


def warm_state_path(name):
    import os
    return os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden",
                        f"warm_{name}.npz")


def warm_on_device(ctx, name, verbose=False):
    """The warmed state of workload `name` computed on the device: VumpsGPU (FP64) from
    randMPS_LR(seed 1) for WARM_SWEEPS[name] sweeps of the tolerance schedule with tolmin =
    GMRES tolerance = 1e-12.  Returns (host state {"AL", "AR", "C"}, energy, gradient norm)."""
    from .vumps import VumpsGPU
    model, fn, params = configs.WORKLOADS[name]
    v = VumpsGPU(ctx, model, dims0=fn(), seed=WARM_SEED, tolmin=1e-12, InvETol=1e-12, verbose=verbose, **params)
    for _ in range(WARM_SWEEPS[name]):
        E, F, _ = v.sweep()
    return v.host_state(), E, F


def load_warm_state(name):
    """The committed warmed state of workload `name` (tests/golden/warm_<name>.npz, written by
    warm_on_device), or None: {"AL": [AL(0), AL(1)], "AR": [...], "C": [C on bond 0, bond 1]} as
    flat float64 arrays in the reference's Vectorize order."""
    import os
    path = warm_state_path(name)
    if not os.path.exists(path):
        return None
    f = np.load(path)
    return {k: [np.array(f[f"{k}{n}"]) for n in range(2)] for k in ("AL", "AR", "C")}

