"""VUMPS on the GPU for a unit cell of any length N >= 2 (VUMPS_main.cpp:31,55-56: the reference
takes N from its command line), FP64, bond expansion off: the loop of VUMPS_main.cpp:97-354 with
every contraction, eigensolve, linear solve and decomposition on the device through the C ABI.

Indices (the convention of vumps.VumpsGPU, for N sites).  Site n maps bond n -> bond n+1 (mod
N); C[b] is the centre matrix on bond b.  The reference rotates its unit-cell arrays after every
site update (shift(.., -1), VUMPS_main.cpp:256-259); here the rotation is replaced by explicit
indices.  Updating site n uses
  AC(n) = C[n] AR(n), H_AC with EHL on bond n, EHR on bond n+1, HL from AL(n-1), HR from AR(n+1);
  H_C of CL = C[n] with (EHL, EHR1 on bond n, AL(n-1), AR(n)) and of CR = C[n+1] with
  (EHL1 on bond n+1, EHR, AL(n), AR(n+1)).
Afterwards the left environment is solved on bond n for the cell starting at site n and shifted
to bond n+1 (the next site's EHL), the right environment on bond n+2 for the cell starting at
site n+2 (the next site's EHR), warm-started from the EHR that site n+1 began with in the
previous sweep (VUMPS_main.cpp:119,269).  For N = 2 these are the operations of VumpsGPU.
"""
from __future__ import annotations

import numpy as np

from . import blocks as B
from . import models, ops


class VumpsCellGPU:
    """VUMPS sweeps of an N-site unit cell on `ctx` (which runs on torch's current stream)."""

    def __init__(self, ctx, model, N, dims0=None, dimvec=None, seed=1, InvETol=5e-15, InvEfac=2.0,
                 fixed_tol=None, tolmin=5e-16, tolmax=1e-6, trueLR=True, svdthresh=5e-7, init_state=None,
                 lanczos_maxit=300, gmres_maxit=4000, lanczos_ncv=126, eig_margin=0.1, **params):
        import torch
        if N < 2:
            raise ValueError("unit cell size must be at least 2")  # VUMPS_main.cpp:56
        self.torch, self.ctx, self.N = torch, ctx, int(N)
        self.d, self.I2K, h = models.build_model(model, **params)
        self.hnnz = models.h_nonzeros(h)
        if dimvec is None:
            dimvec = models.make_dims(dims0, self.N, self.I2K)
        if len(dimvec) != self.N:
            raise ValueError("dimvec is not of length N")  # VUMPS_main.cpp:92
        self.dimvec = dimvec
        self.InvETol, self.InvEfac, self.fixed_tol, self.trueLR = InvETol, InvEfac, fixed_tol, trueLR
        self.tolmin, self.tolmax, self.svdthresh = tolmin, tolmax, svdthresh
        self.lanczos_maxit, self.gmres_maxit, self.lanczos_ncv = lanczos_maxit, gmres_maxit, lanczos_ncv
        self.eig_margin = eig_margin
        self.rng = np.random.default_rng(seed)
        self.stats = {"lanczos_applies": 0, "gmres_iters": 0}
        Nc = self.N
        self.LA = [B.Layout.mps(self.I2K, dimvec[n], dimvec[(n + 1) % Nc]) for n in range(Nc)]
        self.LB = [B.Layout.blockdiag(dimvec[b]) for b in range(Nc)]
        self._z = lambda lay: torch.zeros(lay.nelem, dtype=torch.float64, device="cuda")
        self.AL = [self._z(self.LA[n]) for n in range(Nc)]
        self.AR = [self._z(self.LA[n]) for n in range(Nc)]
        self.C = [self._z(self.LB[b]) for b in range(Nc)]
        self._build_plans()
        if init_state is None:
            self._rand_mps_lr()
        else:
            for n in range(Nc):
                self.AL[n].copy_(init_state["AL"][n])
                self.AR[n].copy_(init_state["AR"][n])
                self.C[n].copy_(init_state["C"][n])
        self._init_environments()

    def _s(self, n):
        return n % self.N

    # ------------------------------------------------------------------ plans
    def _build_plans(self):
        ctx, d, hnnz, LA, LB, Nc, s = self.ctx, self.d, self.hnnz, self.LA, self.LB, self.N, self._s
        self.redop_l = [B.plan_redop(ctx, LA[m], d, hnnz, 0) for m in range(Nc)]  # HL from AL(m): bond m+1
        self.redop_r = [B.plan_redop(ctx, LA[m], d, hnnz, 1) for m in range(Nc)]  # HR from AR(m): bond m
        lHL = [p.derived(0) for p in self.redop_l]
        lHR = [p.derived(0) for p in self.redop_r]
        self.HLbuf = [self._z(l) for l in lHL]
        self.HRbuf = [self._z(l) for l in lHR]
        self.p_ac, self.p_hac, self.p_grad, self.p_hcl, self.p_hcr = [], [], [], [], []
        self.p_mul_r_t, self.p_mul_l_t, self.p_mul_r, self.p_mul_l = [], [], [], []
        self.dec_ac_l, self.dec_ac_r = [], []
        self.tm = {}
        for n in range(Nc):
            l, r, mp, mn = n, s(n + 1), s(n - 1), s(n + 1)
            self.p_ac.append(B.plan_mps_bd(ctx, LA[n], LB[l], 0))                          # C[n] * AR(n)
            self.p_hac.append(B.plan_hac(ctx, LA[n], LB[l], LB[r], lHL[mp], lHR[mn], d))
            self.p_grad.append(B.plan_grad_right(ctx, LA[n], LA[n]))
            self.p_hcl.append(B.plan_hc(ctx, LB[l], LB[l], LB[l], LA[mp], LA[n], d, hnnz))   # CL = C[n]
            self.p_hcr.append(B.plan_hc(ctx, LB[r], LB[r], LB[r], LA[n], LA[mn], d, hnnz))   # CR = C[n+1]
            self.p_mul_r_t.append(B.plan_mps_bd(ctx, LA[n], LB[r], 1, transpose_x=True))    # A * X^T
            self.p_mul_l_t.append(B.plan_mps_bd(ctx, LA[n], LB[l], 0, transpose_x=True))    # X^T * A
            self.p_mul_r.append(B.plan_mps_bd(ctx, LA[n], LB[r], 1))                        # A * X
            self.p_mul_l.append(B.plan_mps_bd(ctx, LA[n], LB[l], 0))                        # X * A
            self.dec_ac_l.append(B.plan_decomp(ctx, LA[n], "l"))
            self.dec_ac_r.append(B.plan_decomp(ctx, LA[n], "r"))
            # unit-cell transfer matrices starting at site n, on bond n (sites n .. n+N-1)
            cell = [LA[s(n + k)] for k in range(Nc)]
            for kind, dirc in (("L", 0), ("R", 1)):
                self.tm[(kind, n)] = B.plan_tm(ctx, cell, dirc, LB[l], LB[l])
            # single-site transfer matrices of site n: left bond n -> n+1, right bond n+1 -> n
            self.tm[("L1", n)] = B.plan_tm(ctx, [LA[n]], 0, LB[l], LB[r])
            self.tm[("R1", n)] = B.plan_tm(ctx, [LA[n]], 1, LB[r], LB[l])
        self.dec_b_l = [B.plan_decomp(ctx, LB[b], "l") for b in range(Nc)]
        self.dec_b_r = [B.plan_decomp(ctx, LB[b], "r") for b in range(Nc)]
        # operator transfer matrices on A(a) A(a+1): left -> right bond of A(a+1) (bond a+2),
        # right -> left bond of A(a) (bond a)
        self.optm_l = [B.plan_optm(ctx, LA[a], LA[s(a + 1)], d, hnnz, 0, LB[s(a + 2)]) for a in range(Nc)]
        self.optm_r = [B.plan_optm(ctx, LA[a], LA[s(a + 1)], d, hnnz, 1, LB[a]) for a in range(Nc)]
        self.cct = {(b, right): B.plan_mps_bd(ctx, LB[b], LB[b], 1 if right else 0, transpose_x=True)
                    for b in range(Nc) for right in (False, True)}
        self.eyes = []
        for b in range(Nc):
            v = np.zeros(LB[b].nelem)
            for (g, qi, qo, rr, cc), o in zip(LB[b].blocks, LB[b].offsets):
                v[o:o + rr * cc] = np.eye(rr).reshape(-1)
            self.eyes.append(self.torch.tensor(v, dtype=self.torch.float64, device="cuda"))

    # ------------------------------------------------------------------ helpers
    def _mul(self, plan, A, X, out):
        plan.bind(0, A); plan.bind(1, X); plan.bind(2, out)
        plan.run()
        return out

    def _tm1(self, kind, n, A, vin, vout):
        """Single-site transfer matrix of site n (kind "L1" or "R1")."""
        p = self.tm[(kind, n)]
        p.bind(2, A[n]); p.bind(0, vin); p.bind(1, vout)
        p.run()
        return vout

    def _optm(self, left, a, A):
        """OpTM of the two-site product A(a) A(a+1): left -> bond a+2, right -> bond a."""
        out = self._z(self.LB[self._s(a + 2)] if left else self.LB[a])
        p = (self.optm_l if left else self.optm_r)[a]
        p.bind(0, A[a]); p.bind(1, A[self._s(a + 1)]); p.bind(2, out)
        p.run()
        return out

    def _cell(self, kind, n, A):
        """The unit-cell transfer matrix starting at site n with the tensors A(n), .., A(n+N-1)."""
        p = self.tm[(kind, n)]
        for k in range(self.N):
            p.bind(2 + k, A[self._s(n + k)])
        return p

    def _cct(self, b, right):
        """C C^T (right) or C^T C on bond b."""
        return self._mul(self.cct[(b, right)], self.C[b], self.C[b], self._z(self.LB[b]))

    def _get_hl(self, n):
        """GetHL (VUMPS_helpers.hpp:3-18) of the cell starting at site n -> bond n."""
        s = self._s
        HL = self._optm(True, s(n - 1), self.AL)  # OpTM(AL(n-1) AL(n)) on bond n+1
        for k in range(1, self.N):
            a = s(n + k)
            t = self._tm1("L1", a, self.AL, HL, self._z(self.LB[s(a + 1)]))
            HL = ops.axpby(self.ctx, 1.0, self._optm(True, s(a - 1), self.AL), 1.0, t)  # on bond a+1
        return HL

    def _get_hr(self, n):
        """GetHR (VUMPS_helpers.hpp:20-36) of the cell starting at site n -> bond n."""
        s = self._s
        HR = self._optm(False, s(n + self.N - 1), self.AR)  # OpTM(AR(n+N-1) AR(n+N)) on bond n+N-1
        for k in range(self.N - 2, -1, -1):
            a = s(n + k)
            t = self._tm1("R1", a, self.AR, HR, self._z(self.LB[a]))
            HR = ops.axpby(self.ctx, 1.0, self._optm(False, a, self.AR), 1.0, t)  # on bond a
        return HR

    def _invert_e(self, kind, n, A, x, L, R, direction, y0, tol):
        """InvertE_proj (InvEBlockFunctions.hpp:201-266) on the cell starting at site n."""
        y = y0.clone() if y0 is not None else self.torch.zeros_like(x)
        it, _, _ = ops.InvertE_proj(self._cell(kind, n, A), x, L, R, direction, y, tol, maxit=self.gmres_maxit)
        self.stats["gmres_iters"] += it
        return y

    def _tm_dominant(self, kind, n, A, x0, tol):
        """TMDominantEig (EigsBlockFunctions.hpp:91-172) on the cell starting at site n."""
        V = self.torch.zeros_like(x0)
        _, it, _ = ops.TMDominantEig(self._cell(kind, n, A), V, x0, tol, maxit=self.gmres_maxit)
        self.stats["gmres_iters"] += it
        return V

    def _redops(self, m):
        """ReducedOp (MPSBlockUtilities.hpp:37-74): HL from AL(m), HR from AR(m)."""
        p = self.redop_l[m]; p.bind(0, self.AL[m]); p.bind(1, self.HLbuf[m]); p.run()
        p = self.redop_r[m]; p.bind(0, self.AR[m]); p.bind(1, self.HRbuf[m]); p.run()

    # ------------------------------------------------------------------ initial state
    def _rand_mps_lr(self):
        """randMPS_LR (MPSBlockUtilities.hpp:1093-1135) on the device."""
        torch, Nc = self.torch, self.N
        for n in range(Nc):
            X = torch.tensor(self.rng.standard_normal(self.LA[n].nelem), dtype=torch.float64, device="cuda")
            ops.qr(self.dec_ac_l[n], X, self.AL[n], self._z(self.dec_ac_l[n].rlayout))
        # right fixed point of the cell on bond 0, C = qr(U sqrt(S), r).R
        R = self._tm_dominant("R", 0, self.AL, self.eyes[0], 1e-14)
        U = self._z(self.LB[0])
        S = torch.zeros(self.dec_b_l[0].nsv, dtype=torch.float64, device="cuda")
        ops.svd(self.dec_b_l[0], R, U, S, None)
        ops.colscale(self.dec_b_l[0], U, S, 0.5)
        ops.qr(self.dec_b_r[0], U, self._z(self.LB[0]), self.C[0])
        Ctmp = self.C[0]
        for n in range(Nc - 1, -1, -1):
            self.C[self._s(n + 1)].copy_(Ctmp)
            X = self._mul(self.p_mul_r[n], self.AL[n], Ctmp, self._z(self.LA[n]))
            Cn = self._z(self.LB[n])
            ops.qr(self.dec_ac_r[n], X, self.AR[n], Cn)
            Ctmp = Cn

    def _init_environments(self):
        """VUMPS_main.cpp:103-136: reduced operators, EHL (bond 0) / EHR (bond 1), EHL1 / EHR1."""
        s = self._s
        for m in range(self.N):
            self._redops(m)
        self.EHL = self._invert_e("L", 0, self.AL, self._get_hl(0), self.eyes[0], self._cct(0, True), "l", None,
                                  self.InvETol)
        self.EHR = self._invert_e("R", 1, self.AR, self._get_hr(1), self._cct(1, False), self.eyes[1], "r", None,
                                  self.InvETol)
        self.EHL1 = ops.axpby(self.ctx, 1.0, self._optm(True, s(-1), self.AL), 1.0,
                              self._tm1("L1", 0, self.AL, self.EHL, self._z(self.LB[1])))        # bond 1
        self.EHR1 = ops.axpby(self.ctx, 1.0, self._optm(False, 0, self.AR), 1.0,
                              self._tm1("R1", 0, self.AR, self.EHR, self._z(self.LB[0])))        # bond 0
        self.EHR0 = [None] * self.N
        self.prec = np.ones(self.N)
        self.F = np.ones(self.N)
        self.dosvd = True
        self.E = None
        self.torch.cuda.synchronize()

    # ------------------------------------------------------------------ one site update
    def site_update(self, n):
        """One iteration of the site loop, VUMPS_main.cpp:171-313, for site n."""
        ctx, s = self.ctx, self._s
        l, r, mp, mn = n, s(n + 1), s(n - 1), s(n + 1)
        self.EHR0[n] = self.EHR
        hac = self.p_hac[n]
        hac.bind(2, self.EHL); hac.bind(3, self.EHR)
        hac.bind(4, self.HLbuf[mp]); hac.bind(5, self.HRbuf[mn])
        hac.prepare()
        # gradient norm (GradNormRight, VUMPS_helpers.hpp:145-153) at AC = C[n] AR(n)
        AC = self._mul(self.p_ac[n], self.AR[n], self.C[l], self._z(self.LA[n]))
        Y = self._z(self.LA[n])
        ops.ApplyHAvec(hac, AC, Y)
        g = self.p_grad[n]
        g.bind(0, Y); g.bind(1, self.AR[n]); g.bind(2, self._z(self.LA[n]))
        self.F[n] = ops.GradNormRight(g)
        tol = self.fixed_tol if self.fixed_tol else min(max(self.prec[n] / 100.0, self.tolmin), self.tolmax)
        tol_eig = tol * self.eig_margin
        kw = dict(ncv=self.lanczos_ncv, maxit=self.lanczos_maxit)
        _, na, _ = ops.eigs_rs(hac, AC, tol_eig, **kw)
        pl = self.p_hcl[n]
        pl.bind(2, self.EHL); pl.bind(3, self.EHR1); pl.bind(4, self.AL[mp]); pl.bind(5, self.AR[n]); pl.prepare()
        pr = self.p_hcr[n]
        pr.bind(2, self.EHL1); pr.bind(3, self.EHR); pr.bind(4, self.AL[n]); pr.bind(5, self.AR[mn]); pr.prepare()
        CL, CR = self.C[l].clone(), self.C[r].clone()
        _, na1, _ = ops.eigs_rs(pl, CL, tol_eig, **kw)
        _, na2, _ = ops.eigs_rs(pr, CR, tol_eig, **kw)
        self.stats["lanczos_applies"] += na + na1 + na2
        ops.sign_normalize(ctx, CL)
        ops.sign_normalize(ctx, CR)
        if self.dosvd and self.prec[n] < self.svdthresh:
            self.dosvd = False
        ALnew, ARnew = self._z(self.LA[n]), self._z(self.LA[n])
        if self.dosvd:
            # polar: AL = U V^T of AC CR^T ; AR = U V^T of CL^T AC  (VUMPS_main.cpp:213-220)
            X = self._mul(self.p_mul_r_t[n], AC, CR, self._z(self.LA[n]))
            X2 = self._mul(self.p_mul_l_t[n], AC, CL, self._z(self.LA[n]))
            U, V = self._z(self.LA[n]), self._z(self.dec_ac_l[n].rlayout)
            U2, V2 = self._z(self.LA[n]), self._z(self.dec_ac_r[n].rlayout)
            ops.svd_batch([self.dec_ac_l[n], self.dec_ac_r[n]], [X, X2], [U, U2], None, [V, V2])
            self._mul(self.p_mul_r[n], U, V, ALnew)
            self._mul(self.p_mul_l[n], U2, V2, ARnew)
        else:
            # QR scheme (VUMPS_main.cpp:221-234)
            QL = self._z(self.LA[n])
            ops.qr(self.dec_ac_l[n], AC, QL, self._z(self.dec_ac_l[n].rlayout))
            PL = self._z(self.LB[r])
            ops.qr(self.dec_b_l[r], CR, PL, self._z(self.LB[r]))
            self._mul(self.p_mul_r_t[n], QL, PL, ALnew)
            QR = self._z(self.LA[n])
            ops.qr(self.dec_ac_r[n], AC, QR, self._z(self.dec_ac_r[n].rlayout))
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
        gtol = max(tol / self.InvEfac, self.InvETol)
        # left environment on bond n: R = CL CL^T, fixed point of the cell starting at site n
        R = self._cct(l, True)
        if self.trueLR:
            R = self._tm_dominant("R", n, self.AL, R, 1e-15)
        EHL = self._invert_e("L", n, self.AL, self._get_hl(n), self.eyes[l], R, "l", self.EHL, gtol)
        # the next site's EHL (bond n+1) and EHL1 (bond n+2)
        EHLtmp = ops.axpby(ctx, 1.0, self._optm(True, mp, self.AL), 1.0,
                           self._tm1("L1", n, self.AL, EHL, self._z(self.LB[r])))
        self.EHL1 = ops.axpby(ctx, 1.0, self._optm(True, n, self.AL), 1.0,
                              self._tm1("L1", mn, self.AL, EHLtmp, self._z(self.LB[s(n + 2)])))
        # right environment on bond n+2: L = C^T C there, fixed point of the cell starting at
        # site n+2, warm start from the EHR site n+1 began with in the previous sweep
        b2 = s(n + 2)
        Lm = self._cct(b2, False)
        if self.trueLR:
            Lm = self._tm_dominant("L", b2, self.AR, Lm, 1e-15)
        self.EHR = self._invert_e("R", b2, self.AR, self._get_hr(b2), Lm, self.eyes[b2], "r", self.EHR0[mn], gtol)
        self.EHL = EHLtmp
        # the next site's EHR1 (bond n+1) = T_R(AR(n+1), EHR) + OpTM(AR(n+1) AR(n+2))
        self.EHR1 = ops.axpby(ctx, 1.0, self._tm1("R1", mn, self.AR, self.EHR, self._z(self.LB[mn])), 1.0,
                              self._optm(False, mn, self.AR))
        self._redops(n)

    def sweep(self):
        """One iteration of the outer loop (VUMPS_main.cpp:165-354); returns (E, F, prec)."""
        for n in range(self.N):
            self.site_update(n)
        self.E = self.energy()
        return self.E, self.F.copy(), self.prec.copy()

    def energy(self):
        """MeasureObservables(H, AR, L) (MPSBlockUtilities.hpp:1017-1073): E[j] is the energy of
        the bond term starting at site b = j+1, tr(C[b]^T C[b] OpTM_R(AR(b) AR(b+1))), in the
        reference's output order (its AR array is rotated by one, VUMPS_main.cpp:112)."""
        E = []
        for j in range(self.N):
            b = self._s(j + 1)
            E.append(ops.bd_trace_prod(self.ctx, self.LB[b], self._cct(b, False), self._optm(False, b, self.AR)))
        return np.array(E)

    def host_state(self):
        t = lambda x: x.cpu().numpy()
        return {"AL": [t(a) for a in self.AL], "AR": [t(a) for a in self.AR], "C": [t(c) for c in self.C]}
