"""VUMPS driver on the GPU: the loop of VUMPS/VUMPS_main.cpp:97-354 (two-site unit cell;
bond expansion by ExpandFromH when mmax is given) with every contraction, eigensolve, linear
solve and decomposition on the device through the C ABI.

Indices.  Site n (n = 0, 1) maps bond n -> bond n+1 (mod 2).  C[b] is the centre matrix on
bond b (the reference's Cvec[n] is the C right of site n, i.e. C[n+1]).  The reference
rotates its unit-cell arrays after every site update (shift(..,-1), VUMPS_main.cpp:256-259);
here the rotation is replaced by explicit indices: updating site n uses
  AC(n) = C[n] AR(n), HL from AL(n-1), HR from AR(n+1), CL = C[n], CR = C[n+1].
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from . import blocks as B
from . import models, ops


class _PlanSet:
    """Transfer-matrix plans of the right-environment chain of a site update on a context of its
    own, so that the chain runs beside the left-environment chain (VumpsGPU(concurrent=True))."""

    def __init__(self, ctx, stream):
        self.ctx, self.stream = ctx, stream
        self.tm, self.optm_r = {}, []
        self.iters = 0  # GMRES / fixed-point iterations, added to the driver's count after the join


class VumpsGPU:
    """The VUMPS sweep of VUMPS_main.cpp:97-354 on the device for a two-site unit cell.  `ctx`
    runs on torch's current stream (ctx.set_stream(torch.cuda.current_stream())): the driver's
    torch operations and its C-ABI calls share that stream, and with concurrent=True the side
    contexts are ordered against it."""

    def __init__(self, ctx, model, dims0=None, dimvec=None, seed=1, InvETol=5e-15, InvEfac=2.0,
                 fixed_tol=None, tolmin=5e-16, tolmax=1e-6, trueLR=True, svdthresh=5e-7, precision="fp64",
                 init_state=None, lanczos_maxit=300, gmres_maxit=4000, lanczos_ncv=126, eig_margin=0.1,
                 mixed_tm=False, verbose=False, mmax=None, dmmax=20, expand_pause=5, expand_thresh=1e-5,
                 lamthresh=1e-12, autotune=False, concurrent=True, **params):
        import torch
        self.torch = torch
        self.verbose = verbose
        self.ctx = ctx
        self._model = model
        self.d, self.I2K, h = models.build_model(model, **params)
        self.hnnz = models.h_nonzeros(h)
        if dimvec is None:
            dimvec = models.make_dims(dims0, 2, self.I2K)
        self.dimvec = dimvec
        self.InvETol, self.InvEfac, self.fixed_tol, self.trueLR = InvETol, InvEfac, fixed_tol, trueLR
        self.tolmin, self.tolmax = tolmin, tolmax  # VUMPS_main.cpp:37-38
        self.svdthresh = svdthresh
        self.lanczos_maxit, self.gmres_maxit = lanczos_maxit, gmres_maxit
        # Krylov dimension of the H_AC / H_C eigensolves.  eigs.cpp:4 uses 20; the effective
        # Hamiltonians of a poorly converged state have spectra spanning ~1e6 |E0|, where a
        # larger thick-restart basis needs far fewer applies.  Measured on XXZ D=512 over 50
        # sweeps (same final energy and gradient from 64 up): ncv 32: 0.36 sweeps/s (not
        # converged), 48: 2.3, 64: 5.1, 80: 6.1, 96: 6.2, 112: 5.8, 126: 6.5.  At the fixed
        # tolerance 1e-12 from a warmed XXZ D=512 state (4 sweeps): 32: 0.28, 48: 1.8, 64: 4.2,
        # 96: 4.4, 126: 4.65 (the largest basis one projection kernel takes).
        self.lanczos_ncv = lanczos_ncv
        self.eig_margin = eig_margin
        self.mixed_tm = mixed_tm
        self.precision = precision
        # time the FP64 launch shapes of every plan's stages once per process (imps_plan_autotune)
        self.autotune = autotune
        # The two H_C eigensolves of a site update (VUMPS_main.cpp:199-200) do not depend on its
        # H_AC eigensolve (:186), nor the right environment (:241-247) on the left one
        # (:236-240).  With concurrent=True each H_C eigensolve, and then the right-environment
        # chain, runs on a context of its own (own stream, Krylov workspace and pinned staging)
        # from a host thread of its own, beside the H_AC eigensolve / the left-environment chain
        # on this context: their small launches and host convergence checks fill each other's
        # gaps.  The results are those of the serial order (no shared state).
        self.concurrent = bool(concurrent)
        if self.concurrent:
            from concurrent.futures import ThreadPoolExecutor
            self._side_streams = [torch.cuda.Stream() for _ in range(2)]
            self._side_ctx = [B.Context(ctx.device, s) for s in self._side_streams]
            self._pool = ThreadPoolExecutor(max_workers=2, thread_name_prefix="imps-hc")
        self.rng = np.random.default_rng(seed)
        self.stats = {"lanczos_applies": 0, "gmres_iters": 0, "hac_applies": 0, "hc_applies": 0, "expansions": 0}
        # bond expansion (ExpandFromH at VUMPS_main.cpp:270-308), off unless mmax (the largest total
        # bond dimension, per site or one for both) is given; defaults of VUMPS_main.cpp:31-35
        self.mmax = None if mmax is None else ([int(mmax)] * 2 if np.isscalar(mmax) else [int(x) for x in mmax])
        self.dmmax, self.expand_pause = int(dmmax), int(expand_pause)
        self.expand_thresh, self.lamthresh = expand_thresh, lamthresh
        self.expand_ct = [0, 0]
        self.exp_prec = 1.0
        d, hnnz = self.d, self.hnnz
        self.LA = [B.Layout.mps(self.I2K, dimvec[n], dimvec[1 - n]) for n in range(2)]
        self.LB = [B.Layout.blockdiag(dimvec[b]) for b in range(2)]
        z = lambda lay: torch.zeros(lay.nelem, dtype=torch.float64, device="cuda")
        self._z = z
        self.AL = [z(self.LA[n]) for n in range(2)]
        self.AR = [z(self.LA[n]) for n in range(2)]
        self.C = [z(self.LB[b]) for b in range(2)]
        self._build_plans()
        if init_state is None:
            self._rand_mps_lr()
        else:
            for n in range(2):
                self.AL[n].copy_(init_state["AL"][n])
                self.AR[n].copy_(init_state["AR"][n])
                self.C[n].copy_(init_state["C"][n])
        self._init_environments()

    # ------------------------------------------------------------------ plans
    def _build_plans(self):
        ctx, d, hnnz, LA, LB = self.ctx, self.d, self.hnnz, self.LA, self.LB
        self.redop_l = [B.plan_redop(ctx, LA[m], d, hnnz, 0) for m in range(2)]  # HL from AL(m): bond m+1
        self.redop_r = [B.plan_redop(ctx, LA[m], d, hnnz, 1) for m in range(2)]  # HR from AR(m): bond m
        self.lHL = [p.derived(0) for p in self.redop_l]
        self.lHR = [p.derived(0) for p in self.redop_r]
        self.HLbuf = [self._z(l) for l in self.lHL]  # HL built from AL(m) (lives on bond m+1)
        self.HRbuf = [self._z(l) for l in self.lHR]  # HR built from AR(m) (lives on bond m)
        self.p_ac, self.p_hac, self.p_grad, self.p_hcl, self.p_hcr = [], [], [], [], []
        self.p_mul_r_t, self.p_mul_l_t, self.p_mul_r, self.p_mul_l = [], [], [], []
        self.dec_ac_l, self.dec_ac_r = [], []
        hc_ctx = self._side_ctx if self.concurrent else [ctx, ctx]
        self.tm = {}
        for n in range(2):
            l, r, m = n, 1 - n, 1 - n
            self.p_ac.append(B.plan_mps_bd(ctx, LA[n], LB[l], 0))                       # C[n] * AR(n)
            self.p_hac.append(B.plan_hac(ctx, LA[n], LB[l], LB[r], self.lHL[m], self.lHR[m], d))
            self.p_grad.append(B.plan_grad_right(ctx, LA[n], LA[n]))
            self.p_hcl.append(B.plan_hc(hc_ctx[0], LB[l], LB[l], LB[l], LA[m], LA[n], d, hnnz))  # CL = C[n]
            self.p_hcr.append(B.plan_hc(hc_ctx[1], LB[r], LB[r], LB[r], LA[n], LA[m], d, hnnz))  # CR = C[n+1]
            self.p_mul_r_t.append(B.plan_mps_bd(ctx, LA[n], LB[r], 1, transpose_x=True))  # A * X^T
            self.p_mul_l_t.append(B.plan_mps_bd(ctx, LA[n], LB[l], 0, transpose_x=True))  # X^T * A
            self.p_mul_r.append(B.plan_mps_bd(ctx, LA[n], LB[r], 1))                      # A * X
            self.p_mul_l.append(B.plan_mps_bd(ctx, LA[n], LB[l], 0))                      # X * A
            self.dec_ac_l.append(B.plan_decomp(ctx, LA[n], "l"))
            self.dec_ac_r.append(B.plan_decomp(ctx, LA[n], "r"))
            # unit-cell transfer matrices starting at site n, on bond n
            for kind, dirc in (("L", 0), ("R", 1)):
                self.tm[(kind, n)] = B.plan_tm(ctx, [LA[n], LA[m]], dirc, LB[l], LB[l])
            # single-site transfer matrices of site n: left bond n -> n+1, right bond n+1 -> n
            self.tm[("L1", n)] = B.plan_tm(ctx, [LA[n]], 0, LB[l], LB[r])
            self.tm[("R1", n)] = B.plan_tm(ctx, [LA[n]], 1, LB[r], LB[l])
        self.dec_b_l = [B.plan_decomp(ctx, LB[b], "l") for b in range(2)]
        self.dec_b_r = [B.plan_decomp(ctx, LB[b], "r") for b in range(2)]
        # operator transfer matrices on 2-site products A(a) A(1-a): left -> right bond of A(1-a)
        # (= bond a), right -> left bond of A(a) (= bond a)
        self.optm_l = [B.plan_optm(ctx, LA[a], LA[1 - a], d, hnnz, 0, LB[a]) for a in range(2)]
        self.optm_r = [B.plan_optm(ctx, LA[a], LA[1 - a], d, hnnz, 1, LB[a]) for a in range(2)]
        self.flops_hac = [p.info()["flops_apply"] for p in self.p_hac]
        # identity BlockDiagMats of the two bonds (made here, on this stream, for both chains)
        self.eyes = [self._make_eye(b) for b in range(2)]
        self._env = None
        if self.concurrent:
            # the right-environment chain's own plans (the left chain binds the same unit-cell
            # transfer matrices to AL at the same time), on the second H_C context
            ps = _PlanSet(self._side_ctx[1], self._side_streams[1])
            for n in range(2):
                l, r, m = n, 1 - n, 1 - n
                for kind, dirc in (("L", 0), ("R", 1)):
                    ps.tm[(kind, n)] = B.plan_tm(ps.ctx, [LA[n], LA[m]], dirc, LB[l], LB[l])
                ps.tm[("R1", n)] = B.plan_tm(ps.ctx, [LA[n]], 1, LB[r], LB[l])
                ps.tm[("cct", n, False)] = B.plan_mps_bd(ps.ctx, LB[n], LB[n], 0, transpose_x=True)
            ps.optm_r = [B.plan_optm(ps.ctx, LA[a], LA[1 - a], d, hnnz, 1, LB[a]) for a in range(2)]
            self._env = ps
        if self.autotune:
            plans = (self.redop_l + self.redop_r + self.p_ac + self.p_hac + self.p_grad + self.p_hcl + self.p_hcr
                     + self.p_mul_r_t + self.p_mul_l_t + self.p_mul_r + self.p_mul_l + self.optm_l + self.optm_r
                     + list(self.tm.values()))
            if self._env is not None:
                plans += list(self._env.tm.values()) + self._env.optm_r
            self.tuned_stages = sum(p.autotune() for p in plans)
        if self.precision == "bf16x6":
            # tensor-core applies inside the Krylov solvers; Krylov vectors, residuals,
            # decompositions and the energy stay FP64
            mixed = self.p_hac + self.p_hcl + self.p_hcr
            # transfer matrices of the GMRES environment / fixed-point solves: FP64 by default —
            # split-BF16 TM applies are cheaper, but the iterative refinement that brings their
            # GMRES back to FP64 accuracy restarts the Krylov space and doubles the iterations
            if self.mixed_tm:
                mixed += [self.tm[(k, n)] for k in ("L", "R") for n in range(2)]
                if self._env is not None:
                    mixed += [self._env.tm[(k, n)] for k in ("L", "R") for n in range(2)]
            for p in mixed:
                p.set_precision(N.PREC_BF16X6)
        if self.concurrent:
            # plan tables are uploaded by synchronous copies on the legacy default stream, whose
            # last DMA the non-blocking streams of the H_C contexts do not wait for
            self.torch.cuda.synchronize()

    # ------------------------------------------------------------------ small helpers
    def _tm(self, key, A, vin, vout, ps=None):
        p = (self.tm if ps is None else ps.tm)[key]
        n = key[1]
        if key[0] in ("L", "R"):
            p.bind(2, A[n]); p.bind(3, A[1 - n])
        else:
            p.bind(2, A[n])
        p.bind(0, vin); p.bind(1, vout)
        p.run()
        return vout

    def _optm(self, left, a, A, out, ps=None):
        p = (self.optm_l if left else (self.optm_r if ps is None else ps.optm_r))[a]
        p.bind(0, A[a]); p.bind(1, A[1 - a]); p.bind(2, out)
        p.run()
        return out

    def _mul(self, plan, A, X, out):
        plan.bind(0, A); plan.bind(1, X); plan.bind(2, out)
        plan.run()
        return out

    def _make_eye(self, b):
        v = np.zeros(self.LB[b].nelem)
        for (g, qi, qo, r, c), o in zip(self.LB[b].blocks, self.LB[b].offsets):
            v[o:o + r * c] = np.eye(r).reshape(-1)
        return self.torch.tensor(v, dtype=self.torch.float64, device="cuda")

    def _eye(self, b):
        """The identity BlockDiagMat of bond b (read only)."""
        return self.eyes[b]

    def _redops(self, sites=(0, 1)):
        """ReducedOp (MPSBlockUtilities.hpp:37-74): HL from AL(m), HR from AR(m)."""
        for m in sites:
            p = self.redop_l[m]; p.bind(0, self.AL[m]); p.bind(1, self.HLbuf[m]); p.run()
            p = self.redop_r[m]; p.bind(0, self.AR[m]); p.bind(1, self.HRbuf[m]); p.run()

    def _get_hl(self, n):
        """GetHL (VUMPS_helpers.hpp:3-18) of the unit cell [AL(n), AL(n+1)] -> bond n."""
        m = 1 - n
        t = self._optm(True, m, self.AL, self._z(self.LB[m]))       # OpTM(AL(n+1) AL(n)) on bond n+1
        out = self._tm(("L1", m), self.AL, t, self._z(self.LB[n]))   # through AL(n+1) -> bond n
        t2 = self._optm(True, n, self.AL, self._z(self.LB[n]))       # OpTM(AL(n) AL(n+1)) on bond n
        return ops.axpby(self.ctx, 1.0, t2, 1.0, out)

    def _get_hr(self, n, ps=None):
        """GetHR (VUMPS_helpers.hpp:20-36) of the unit cell [AR(n), AR(n+1)] -> bond n."""
        m = 1 - n
        t = self._optm(False, m, self.AR, self._z(self.LB[m]), ps)      # OpTM(AR(n+1) AR(n)) on bond n+1
        out = self._tm(("R1", n), self.AR, t, self._z(self.LB[n]), ps)   # through AR(n) -> bond n
        t2 = self._optm(False, n, self.AR, self._z(self.LB[n]), ps)      # OpTM(AR(n) AR(n+1)) on bond n
        return ops.axpby(self.ctx if ps is None else ps.ctx, 1.0, t2, 1.0, out)

    def _bind_uc(self, key, A, ps=None):
        p = (self.tm if ps is None else ps.tm)[key]
        n = key[1]
        p.bind(2, A[n]); p.bind(3, A[1 - n])
        return p

    def _count_iters(self, it, ps):
        if ps is None:
            self.stats["gmres_iters"] += it
        else:
            ps.iters += it

    def _invert_e(self, key, A, x, L, R, direction, y0, tol, ps=None):
        """InvertE_proj on the unit cell [A(n), A(n+1)], n = key[1]."""
        y = y0.clone() if y0 is not None else self._z_like(x)
        it, rr, conv = ops.InvertE_proj(self._bind_uc(key, A, ps), x, L, R, direction, y, tol,
                                        maxit=self.gmres_maxit)
        self._count_iters(it, ps)
        return y

    def _z_like(self, x):
        return self.torch.zeros_like(x)

    def _tm_dominant(self, key, A, x0, tol, ps=None):
        """TMDominantEig on the unit cell [A(n), A(n+1)], n = key[1]."""
        V = self._z_like(x0)
        _, it, _ = ops.TMDominantEig(self._bind_uc(key, A, ps), V, x0, tol, maxit=self.gmres_maxit)
        self._count_iters(it, ps)
        return V

    # ------------------------------------------------------------------ initial state
    def _rand_mps_lr(self):
        """randMPS_LR (MPSBlockUtilities.hpp:1093-1135) on the device."""
        torch = self.torch
        for n in range(2):
            X = torch.tensor(self.rng.standard_normal(self.LA[n].nelem), dtype=torch.float64, device="cuda")
            Rb = self._z(self.dec_ac_l[n].rlayout)
            ops.qr(self.dec_ac_l[n], X, self.AL[n], Rb)
        # right fixed point of [AL(0), AL(1)] on bond 0, C = qr(U sqrt(S), r).R
        R = self._tm_dominant(("R", 0), self.AL, self._eye(0), 1e-14)
        U = self._z(self.LB[0])
        S = torch.zeros(self.dec_b_l[0].nsv, dtype=torch.float64, device="cuda")
        ops.svd(self.dec_b_l[0], R, U, S, None)
        ops.colscale(self.dec_b_l[0], U, S, 0.5)
        Qb = self._z(self.LB[0])
        ops.qr(self.dec_b_r[0], U, Qb, self.C[0])
        Ctmp = self.C[0]  # C on bond 0 (right of AL(1))
        for n in (1, 0):
            self.C[(n + 1) % 2].copy_(Ctmp)
            X = self._mul(self.p_mul_r[n], self.AL[n], Ctmp, self._z(self.LA[n]))
            Cn = self._z(self.LB[n])
            ops.qr(self.dec_ac_r[n], X, self.AR[n], Cn)
            Ctmp = Cn

    def _init_environments(self):
        """VUMPS_main.cpp:103-136: reduced operators, EHL/EHR, EHL1/EHR1."""
        torch = self.torch
        self._redops()
        # R at bond 0 (right end of [AL(0), AL(1)]): C[0] C[0]^T (the reference's initial shift
        # puts it at the unit-cell boundary); the right environment's L is C[1]^T C[1]
        R = self._cct(0, right=True)
        self.EHL = self._invert_e(("L", 0), self.AL, self._get_hl(0), self._eye(0), R, "l", None, self.InvETol)
        self.EHR = self._invert_e(("R", 1), self.AR, self._get_hr(1), self._cct(1, right=False),
                                  self._eye(1), "r", None, self.InvETol)
        self.EHL1 = ops.axpby(self.ctx, 1.0, self._optm(True, 1, self.AL, self._z(self.LB[1])), 1.0,
                              self._tm(("L1", 0), self.AL, self.EHL, self._z(self.LB[1])))
        self.EHR1 = ops.axpby(self.ctx, 1.0, self._optm(False, 0, self.AR, self._z(self.LB[0])), 1.0,
                              self._tm(("R1", 0), self.AR, self.EHR, self._z(self.LB[0])))
        self.EHR0 = [None, None]
        self.prec = np.ones(2)
        self.F = np.ones(2)
        self.dosvd = True
        self.E = None
        torch.cuda.synchronize()

    def _cct(self, b, right=True, ps=None):
        """C C^T (right=True) or C^T C on bond b."""
        out = self._z(self.LB[b])
        ctx, tm = (self.ctx, self.tm) if ps is None else (ps.ctx, ps.tm)
        # BlockDiag products through the MPS x BlockDiag plans with d = 1 (layout of a BD)
        key = ("cct", b, right)
        if key not in tm:
            tm[key] = B.plan_mps_bd(ctx, self.LB[b], self.LB[b], 1 if right else 0, transpose_x=True)
        p = tm[key]
        # right: C * C^T ; left: C^T * C
        return self._mul(p, self.C[b], self.C[b], out)

    # ------------------------------------------------------------------ one site update
    def site_update(self, n):
        """One iteration of the site loop, VUMPS_main.cpp:171-313, for site n."""
        torch, ctx = self.torch, self.ctx
        l, r, m = n, 1 - n, 1 - n
        self.EHR0[n] = self.EHR
        hac = self.p_hac[n]
        hac.bind(2, self.EHL); hac.bind(3, self.EHR)
        hac.bind(4, self.HLbuf[m]); hac.bind(5, self.HRbuf[m])
        hac.prepare()  # operators changed (re-packs tensor-core operands in mixed mode)
        # gradient norm (GradNormRight, VUMPS_helpers.hpp:145-153) at AC = C[n] AR(n)
        AC = self._mul(self.p_ac[n], self.AR[n], self.C[l], self._z(self.LA[n]))
        Y = self._z(self.LA[n])
        # the gradient H_AC.AC - AL.H_C.C is a convergence measure: always FP64
        if self.precision == "bf16x6":
            hac.set_precision(N.PREC_FP64)
        ops.ApplyHAvec(hac, AC, Y)
        if self.precision == "bf16x6":
            hac.set_precision(N.PREC_BF16X6)
        g = self.p_grad[n]
        g.bind(0, Y); g.bind(1, self.AR[n]); g.bind(2, self._z(self.LA[n]))
        self.F[n] = ops.GradNormRight(g)
        tol = self.fixed_tol if self.fixed_tol else min(max(self.prec[n] / 100.0, self.tolmin), self.tolmax)
        # ARPACK (eigs.cpp) tests convergence once per restart cycle (every ncv - nev = 19 Lanczos
        # steps) and so returns Ritz residuals typically an order below its tol; the device
        # Lanczos tests every 4 steps and would stop right at the bound, where tol = prec/100
        # no longer contracts prec (eigenvector error ~ tol |theta| / gap ~ prec).  The margin
        # restores the reference's effective accuracy.
        tol_eig = tol * self.eig_margin
        # H_C eigensolves for CL = C[n] (EHL, EHR1) and CR = C[n+1] (EHL1, EHR)
        CL, CR = self.C[l].clone(), self.C[r].clone()
        main = torch.cuda.current_stream()
        if self.concurrent:
            for s in self._side_streams:
                s.wait_stream(main)  # the operands and start vectors are written on this stream
        pl = self.p_hcl[n]
        pl.bind(2, self.EHL); pl.bind(3, self.EHR1); pl.bind(4, self.AL[m]); pl.bind(5, self.AR[n]); pl.prepare()
        pr = self.p_hcr[n]
        pr.bind(2, self.EHL1); pr.bind(3, self.EHR); pr.bind(4, self.AL[n]); pr.bind(5, self.AR[m]); pr.prepare()
        kw = dict(ncv=self.lanczos_ncv, maxit=self.lanczos_maxit)
        if self.concurrent:
            jobs = [self._pool.submit(ops.eigs_rs, p, x, tol_eig, **kw) for p, x in ((pl, CL), (pr, CR))]
        # H_AC eigensolve (eigs_rs "SA", x0 = AC)
        ev, na, _ = ops.eigs_rs(hac, AC, tol_eig, **kw)
        self.stats["lanczos_applies"] += na
        self.stats["hac_applies"] += na + 1
        if self.concurrent:
            (_, na1, _), (_, na2, _) = (j.result() for j in jobs)
            for s in self._side_streams:
                main.wait_stream(s)
        else:
            _, na1, _ = ops.eigs_rs(pl, CL, tol_eig, **kw)
            _, na2, _ = ops.eigs_rs(pr, CR, tol_eig, **kw)
        self.stats["lanczos_applies"] += na1 + na2
        self.stats["hc_applies"] += na1 + na2
        ops.sign_normalize(ctx, CL)
        ops.sign_normalize(ctx, CR)
        if self.dosvd and self.prec[n] < self.svdthresh:
            self.dosvd = False
        ALnew, ARnew = self._z(self.LA[n]), self._z(self.LA[n])
        if self.dosvd:
            # polar: AL = U V^T of AC CR^T ; AR = U V^T of CL^T AC  (VUMPS_main.cpp:213-220); the
            # two independent SVDs share one launch
            X = self._mul(self.p_mul_r_t[n], AC, CR, self._z(self.LA[n]))
            X2 = self._mul(self.p_mul_l_t[n], AC, CL, self._z(self.LA[n]))
            U, V = self._z(self.LA[n]), self._z(self.dec_ac_l[n].rlayout)
            U2, V2 = self._z(self.LA[n]), self._z(self.dec_ac_r[n].rlayout)
            ops.svd_batch([self.dec_ac_l[n], self.dec_ac_r[n]], [X, X2], [U, U2], None, [V, V2])
            self._mul(self.p_mul_r[n], U, V, ALnew)
            self._mul(self.p_mul_l[n], U2, V2, ARnew)
        else:
            # QR scheme (VUMPS_main.cpp:221-234)
            QL, Rt = self._z(self.LA[n]), self._z(self.dec_ac_l[n].rlayout)
            ops.qr(self.dec_ac_l[n], AC, QL, Rt)
            PL = self._z(self.LB[r])
            ops.qr(self.dec_b_l[r], CR, PL, self._z(self.LB[r]))
            self._mul(self.p_mul_r_t[n], QL, PL, ALnew)
            QR, Rt2 = self._z(self.LA[n]), self._z(self.dec_ac_r[n].rlayout)
            ops.qr(self.dec_ac_r[n], AC, QR, Rt2)
            PR = self._z(self.LB[l])
            ops.qr(self.dec_b_r[l], CL, PR, self._z(self.LB[l]))
            self._mul(self.p_mul_l_t[n], QR, PR, ARnew)
        # errors err_l = |AC - AL CR|_inf, err_r = |AC - CL AR|_inf
        t = self._mul(self.p_mul_r[n], ALnew, CR, self._z(self.LA[n]))
        err_l = ops.norm_inf(ctx, ops.axpby(ctx, 1.0, AC, -1.0, t))
        t = self._mul(self.p_mul_l[n], ARnew, CL, self._z(self.LA[n]))
        err_r = ops.norm_inf(ctx, ops.axpby(ctx, 1.0, AC, -1.0, t))
        self.prec[n] = max(err_l, err_r)
        self.AL[n], self.AR[n], self.C[r], self.C[l] = ALnew, ARnew, CR, CL
        # left environment: R = CL CL^T, fixed point of [AL(n), AL(n+1)], EHL on bond n
        gtol = max(tol / self.InvEfac, self.InvETol)
        if self.concurrent:
            # the right-environment chain on its own context and thread (see __init__)
            ps = self._env
            ps.stream.wait_stream(main)  # AL, AR, C of this site update are written on this stream
            job = self._pool.submit(self._right_env_job, n, gtol, ps)
        R = self._cct(l, right=True)
        if self.trueLR:
            R = self._tm_dominant(("R", n), self.AL, R, 1e-15)
        HAL = self._get_hl(n)
        self.EHL = self._invert_e(("L", n), self.AL, HAL, self._eye(l), R, "l", self.EHL, gtol)
        # shift to site n+1: EHLtmp = OpTM(AL(n-1) AL(n)) + T_L(AL(n), EHL) on bond n+1
        EHLtmp = ops.axpby(ctx, 1.0, self._optm(True, m, self.AL, self._z(self.LB[r])), 1.0,
                           self._tm(("L1", n), self.AL, self.EHL, self._z(self.LB[r])))
        self.EHL1 = ops.axpby(ctx, 1.0, self._optm(True, n, self.AL, self._z(self.LB[l])), 1.0,
                              self._tm(("L1", m), self.AL, EHLtmp, self._z(self.LB[l])))
        if self.concurrent:
            self.EHR = job.result()
            main.wait_stream(ps.stream)
            self.EHR.record_stream(main)  # allocated on the chain's stream, used on this one
            self.stats["gmres_iters"] += ps.iters
            ps.iters = 0
        else:
            self.EHR = self._right_env(n, gtol)
        if self.mmax is not None and self._expand_now(n) and self._expand(n):
            # EHL on the grown bond (VUMPS_main.cpp:301); EHL1, EHR and the bond-n objects keep
            # their values (AL(n+1) only gained zero rows)
            EHLtmp = ops.axpby(ctx, 1.0, self._optm(True, m, self.AL, self._z(self.LB[r])), 1.0,
                               self._tm(("L1", n), self.AL, self.EHL, self._z(self.LB[r])))
        self.EHL = EHLtmp
        self.EHR1 = ops.axpby(ctx, 1.0, self._tm(("R1", m), self.AR, self.EHR, self._z(self.LB[r])), 1.0,
                              self._optm(False, m, self.AR, self._z(self.LB[r])))
        # HL = ReducedOp(H, AL(n), l), HR = ReducedOp(H, AR(n), r) (VUMPS_main.cpp:311-312)
        self._redops((n,))

    def _right_env(self, n, gtol, ps=None):
        """Right environment for site n+1 (VUMPS_main.cpp:241-247): L = C^T C on bond n (= bond
        n+2), its fixed point of [AR(n), AR(n+1)], then EHR by InvertE_proj from the previous
        EHR of this site; with the plans of `ps` (default: this context's)."""
        l, m = n, 1 - n
        Lm = self._cct(l, right=False, ps=ps)
        if self.trueLR:
            Lm = self._tm_dominant(("L", n), self.AR, Lm, 1e-15, ps)
        HAR = self._get_hr(n, ps)
        return self._invert_e(("R", n), self.AR, HAR, Lm, self._eye(l), "r", self.EHR0[m], gtol, ps)

    def _right_env_job(self, n, gtol, ps):
        with self.torch.cuda.stream(ps.stream):  # temporaries of the chain on its own stream
            return self._right_env(n, gtol, ps)

    def sweep(self):
        """One iteration of the outer loop (VUMPS_main.cpp:165-354); returns (E, F, prec)."""
        import sys
        import time
        t0 = time.perf_counter()
        s0 = dict(self.stats)
        self.exp_prec = float(np.max(self.prec))  # VUMPS_main.cpp:168
        for n in range(2):
            self.site_update(n)
        self.E = self.energy()
        if self.verbose:
            d = {k: self.stats[k] - s0.get(k, 0) for k in self.stats}
            print(f"[vumps {self.precision}] sweep {time.perf_counter() - t0:.3f}s E={self.E.mean():.12f} "
                  f"F={self.F.max():.3e} prec={self.prec.max():.3e} {d}", file=sys.stderr, flush=True)
        return self.E, self.F.copy(), self.prec.copy()

    def energy(self):
        """MeasureObservables(H, AR, L) (MPSBlockUtilities.hpp:1017-1073): the bond energy
        tr(L_k OpTM_R(AR(k) AR(k+1))) with L_k = C[k]^T C[k], listed in the reference's
        output order (its AR array is rotated by one, VUMPS_main.cpp:112, so E(0) is the
        bond that starts at site 1)."""
        E = []
        for k in (1, 0):
            X = self._optm(False, k, self.AR, self._z(self.LB[k]))
            Lk = self._cct(k, right=False)
            E.append(ops.bd_trace_prod(self.ctx, self.LB[k], Lk, X))
        return np.array(E)

    @staticmethod
    def first_block_sectors(LA, I2K, O, keys):
        """The left-bond sectors q (of ``keys``) at which the first block that
        ApplyTMmixedRight(ApplyOperator(A, O), A) creates (physical index order, TMBlockFunctions.hpp:
        445-473) is charge-diagonal, for a one-site O that mixes entries of different charge shifts.
        The reference's BlockMat holds one block per incoming charge and std::map::emplace_hint
        drops a later block with another outgoing charge, so at the other sectors every diagonal
        contribution is lost and the trace (BlockObj.hpp:1340-1350) sees none of them."""
        from . import charges
        d = len(I2K)
        per = charges.periods_of(I2K)
        out = set()
        for q in keys:
            first = None
            for r in range(d):
                for c in range(d):
                    if O[r, c] == 0.0 or LA.find(c, q) < 0:
                        continue
                    qb = charges.sub(charges.add(q, I2K[c], per), I2K[r], per)
                    if LA.find(r, qb) < 0:
                        continue
                    first = tuple(I2K[c]) == tuple(I2K[r])
                    break
                if first is not None:
                    break
            if first:
                out.add(tuple(q))
        return out

    def measure(self, obs):
        """MeasureObservables(obs, AR, L) (MPSBlockUtilities.hpp:1017-1073, dir r) as the driver
        calls it (VUMPS_main.cpp:344): for every operator, tr(L[n-1] OpTM_R(O, AR(n)...)) at both
        sites, in the reference's output order (its AR array is rotated by one, so entry 0
        belongs to site 1).  obs: names of GetObservables or (name, matrix) pairs, one-site
        (d x d) or two-site (d^2 x d^2).  The trace of a BlockMat sums only blocks with equal
        charges (BlockObj.hpp:1340-1350), so the charge-changing entries of O contribute exactly
        zero; the charge-conserving rest runs through the operator transfer matrix plans, a
        one-site O as O x 1 on AR(n) AR(n+1) (AR(n+1) right-isometric).  A one-site O with entries
        of both kinds (Fermi-Hubbard "rx") is traced over ``first_block_sectors`` only, as the
        reference's map insertion leaves it.  Returns {name: values}."""
        d = self.d
        if obs and isinstance(obs[0], str):
            obs = models.observables(self._model, obs, d=self.d)
        from . import charges
        charge = lambda s: tuple(self.I2K[s])
        per = charges.periods_of(self.I2K)
        out = {}
        for name, O in obs:
            O = np.asarray(O, dtype=np.float64)
            O1 = None
            if O.shape == (d, d):
                cons1 = np.array([[charge(r) == charge(c) for c in range(d)] for r in range(d)])
                if np.any(O[cons1] != 0.0) and np.any(O[~cons1] != 0.0):
                    O1 = O
                O = np.kron(O, np.eye(d))
            elif O.shape != (d * d, d * d):
                raise ValueError(f"operator {name}: shape {O.shape}, expected ({d}, {d}) or ({d * d}, {d * d})")
            q2 = [charges.add(charge(s1), charge(s2), per) for s1 in range(d) for s2 in range(d)]
            keep = np.array([[q2[r] == q2[c] for c in range(d * d)] for r in range(d * d)])
            if O1 is None and np.any(O[keep] != 0.0) and np.any(O[~keep] != 0.0):
                raise NotImplementedError(f"two-site operator {name} mixes charge-conserving and charge-changing "
                                          "entries")
            hnnz = models.h_nonzeros(np.where(keep, O, 0.0))
            vals = []
            for k in (1, 0):
                if not hnnz:
                    vals.append(0.0)
                    continue
                p = B.plan_optm(self.ctx, self.LA[k], self.LA[1 - k], d, hnnz, 1, self.LB[k])
                X = self._z(self.LB[k])
                p.bind(0, self.AR[k]); p.bind(1, self.AR[1 - k]); p.bind(2, X); p.run()
                L = self._cct(k, right=False)
                if O1 is not None:
                    sel = self.first_block_sectors(self.LA[k], self.I2K, O1, [b[1] for b in self.LB[k].blocks])
                    for (_, q, _, m, _), o in zip(self.LB[k].blocks, self.LB[k].offsets):
                        if tuple(q) not in sel:
                            L[o:o + m * m].zero_()
                vals.append(ops.bd_trace_prod(self.ctx, self.LB[k], L, X))
            out[name] = np.array(vals)
        return out

    def host_state(self):
        t = lambda x: x.cpu().numpy()
        return {"AL": [t(a) for a in self.AL], "AR": [t(a) for a in self.AR], "C": [t(c) for c in self.C]}

    # ------------------------------------------------------------------ bond expansion
    def _lam(self, b):
        """Singular values of C[b] per sector (svd(C), VUMPS_main.cpp:207-208), device SVD."""
        from . import imps_io
        S = self.torch.zeros(self.dec_b_l[b].nsv, dtype=self.torch.float64, device="cuda")
        ops.svd(self.dec_b_l[b], self.C[b], self._z(self.LB[b]), S, None)
        return imps_io.lam_from_flat(S.cpu().numpy(), self.LB[b])

    def _expand_now(self, n):
        """The expansion test of VUMPS_main.cpp:272-277 for the bond right of site n: enough site
        updates since the last one, the previous sweep converged below expand_thresh, room below
        mmax, and some sector whose smallest singular value is above lamthresh."""
        r = 1 - n
        mr_tot = sum(self.LB[r].dims().values())
        now = self.expand_ct[n] >= self.expand_pause and self.exp_prec < self.expand_thresh and mr_tot < self.mmax[n]
        if now:
            lam = self._lam(r)
            now = max(float(v.min()) for v in lam.values() if len(v)) > self.lamthresh
        if not now:
            self.expand_ct[n] += 1
        return now

    def _expand(self, n):
        """ExpandFromH(H, I2K, AL(n), AR(n+1), C[n+1], min(dmmax, mmax - m_tot)) and the zero
        padding of AR(n) (VUMPS_main.cpp:282-299), then every plan rebuilt for the grown bond.
        Returns False if nothing was added."""
        from . import expand
        r = m = 1 - n
        self.expand_ct[n] = 0
        mr_tot = sum(self.LB[r].dims().values())
        res = expand.expand_from_h(self.ctx, self.I2K, self.hnnz, self.LA[n], self.AL[n], self.LA[m], self.AR[m],
                                   self.LB[r], self.C[r], min(self.dmmax, self.mmax[n] - mr_tot))
        if res is None or sum(res["dm"].values()) == 0:
            return False
        oldLA, oldLB = list(self.LA), list(self.LB)
        dimvec = list(self.dimvec)
        dimvec[r] = res["dims"]
        self.dimvec = dimvec
        self.LA = [B.Layout.mps(self.I2K, dimvec[k], dimvec[1 - k]) for k in range(2)]
        self.LB = [B.Layout.blockdiag(dimvec[b]) for b in range(2)]
        if self.LA[n].blocks != res["LA"].blocks or self.LA[m].blocks != res["LR"].blocks:
            raise RuntimeError("expanded layouts differ from the driver's")
        # AR(n) (right index on the grown bond) is padded with zeros as in the reference; AL(n+1)
        # (left index there) gains zero rows and is replaced at its own site update
        na, nm, nb = self.LA[n].nelem, self.LA[m].nelem, self.LB[r].nelem
        self.AR[n] = expand.relayout(self.ctx, oldLA[n], self.LA[n], self.AR[n])[:na]
        self.AL[m] = expand.relayout(self.ctx, oldLA[m], self.LA[m], self.AL[m])[:nm]
        self.AL[n], self.AR[m], self.C[r] = res["AL"][:na], res["AR"][:nm], res["C"][:nb]
        if self.EHR0[n] is not None:  # initial guess of the next right-environment solve on that bond
            self.EHR0[n] = expand.relayout(self.ctx, oldLB[r], self.LB[r], self.EHR0[n])[:nb]
        self._build_plans()
        self.stats["expansions"] += 1
        if self.verbose:
            import sys
            print(f"[vumps] expanded bond {r}: +{sum(res['dm'].values())} -> {sum(res['dims'].values())}",
                  file=sys.stderr, flush=True)
        return True

    def keep_running(self, thresh=1e-14):
        """run_IDMRG (VUMPS_main.cpp:331-340): the gradient is above thresh, or (with expansion
        on) some bond below its mmax has a sector whose smallest singular value exceeds
        lamthresh."""
        if float(np.max(self.F)) > thresh:
            return True
        if self.mmax is None:
            return False
        too_large, too_small = [], []
        for n in range(2):
            b = (n + 1) % 2  # Lamvec[n] belongs to the C right of site n
            too_large.append(any(float(v.min()) > self.lamthresh for v in self._lam(b).values() if len(v)))
            too_small.append(sum(self.LB[b].dims().values()) < self.mmax[n])
        return any(too_large) and any(too_small)

    # ------------------------------------------------------------------ state files
    def imps_state(self):
        """The state in the arrangement saveIMPS writes at the end of VUMPS_main.cpp (:368-403,
        AR shifted back at :368): ALvec[n] = AL(n), ARvec[n] = AR(n), Cvec[n] = the C right of
        site n (C[n+1] here) and Lamvec[n] its singular values (svd(C), VUMPS_main.cpp:207-208),
        computed by the device sector SVD."""
        from . import imps_io
        torch = self.torch
        h = self.host_state()
        AL = [imps_io.flat_to_mps(h["AL"][n], self.LA[n], self.d) for n in range(2)]
        AR = [imps_io.flat_to_mps(h["AR"][n], self.LA[n], self.d) for n in range(2)]
        Cv, Lam = [], []
        for n in range(2):
            b = (n + 1) % 2
            Cv.append(imps_io.flat_to_bd(h["C"][b], self.LB[b]))
            S = torch.zeros(self.dec_b_l[b].nsv, dtype=torch.float64, device="cuda")
            ops.svd(self.dec_b_l[b], self.C[b], self._z(self.LB[b]), S, None)
            Lam.append(imps_io.lam_from_flat(S.cpu().numpy(), self.LB[b]))
        return imps_io.IMPSState(Lam, Cv, AL, AR)

    def save_imps(self, name, ending="bin", folder="."):
        """saveIMPS(Lamvec, Cvec, ALvec, ARvec, folder/name) (VUMPS_main.cpp:403); returns the path."""
        from . import imps_io
        s = self.imps_state()
        return imps_io.saveIMPS(s.Lam, s.C, s.AL, s.AR, name, ending, folder)

    @classmethod
    def from_imps(cls, ctx, model, state, **kw):
        """A driver started from a state file (a path, or an ``imps_io.IMPSState``), as
        Excitations_main.cpp:84-101 loads one: the bond dimensions come from the file's centre
        matrices, and the isometries must carry exactly the sectors the model's I2K gives for
        them ("AL not compatible with I2K from model" otherwise).  Unit cells of two sites."""
        import torch
        from . import imps_io
        st = imps_io.loadIMPS(state) if isinstance(state, (str, bytes)) or hasattr(state, "__fspath__") else state
        if not (len(st.AL) == len(st.AR) == len(st.C) == 2):
            raise imps_io.IMPSFormatError(f"unit cell of {len(st.AL)} sites; this driver runs two-site cells")
        d, I2K, _ = models.build_model(model, **kw)  # reads only the model's own parameters
        # Cvec[n] is the C right of site n, i.e. on bond n + 1
        dimvec = [imps_io.bond_dims(st.C[(b + 1) % 2]) for b in range(2)]
        nsym = len(I2K[0])
        for key, arr in (("AL", st.AL), ("AR", st.AR)):
            for n, A in enumerate(arr):
                if A.d != d or A.nsites != 1:
                    raise imps_io.IMPSFormatError(f"{key}({n}): d = {A.d}, {A.nsites} site(s); the model has d = {d}")
        if any(len(q) != nsym for b in range(2) for q in dimvec[b]):
            raise imps_io.IMPSFormatError(f"keys of the state do not have the model's {nsym} quantum number(s)")
        init = {"AL": [], "AR": [], "C": []}
        for n in range(2):
            lay = B.Layout.mps(I2K, dimvec[n], dimvec[1 - n])
            for key, A in (("AL", st.AL[n]), ("AR", st.AR[n])):
                try:
                    init[key].append(torch.from_numpy(imps_io.mps_to_flat(A, lay)))
                except imps_io.IMPSFormatError as e:
                    raise imps_io.IMPSFormatError(f"{key}({n}) not compatible with I2K from model: {e}") from None
        for b in range(2):
            init["C"].append(torch.from_numpy(imps_io.bd_to_flat(st.C[(b + 1) % 2], B.Layout.blockdiag(dimvec[b]))))
        return cls(ctx, model, dimvec=dimvec, init_state=init, **kw)
