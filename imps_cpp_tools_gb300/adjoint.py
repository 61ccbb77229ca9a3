"""Gradient of the energy density of a uniform two-site MPS on the GPU (adjoint method).

At a left-isometric unit cell AL = [A0, A1] (transfer-matrix eigenvalue 1, left fixed point the
identity, right fixed point r = C C^T on bond 0) the energy density is
    e = (N0 / lam + N1 / lam^2) / (2 (l|r)),
with N0 the bond (0,1) term between l and r and N1 the bond (1,2) term between l1 = T_0(l) and
r1 = T~_1(r) (T_n(X) = sum_s A_s^T X A_s, T~_n(X) = sum_s A_s X A_s^T).  Its gradient with
respect to every entry of A0 and A1 collects
  * the direct two-site terms, H_AC-type contractions with the ReducedOp environments
    (MPSBlockUtilities.hpp:37-74 with r, r1 inserted): W[s][s'] = sum h A1[t'] r A1[t]^T,
    V[t][t'] = sum h A0[s]^T A0[s'] and their bond (1,2) counterparts W', V';
  * the adjoints of the transfer-matrix applies through l1, r1 and the eigenvalue
    (left TM: (Y|dT(X)) -> X A Y^T + X^T A Y; right TM: (Y|dT~(X)) -> Y A X^T + Y^T A X);
  * the fixed points by the implicit function theorem: g_l = de/dl and g_r = de/dr are
    orthogonal to the null directions (scale invariance), and the two adjoint solves are
    InvertE_proj (InvEBlockFunctions.hpp:201-266) on the *transposed* unit-cell TMs,
    (1 - T~ + |r)(l|) y_l = g_l and (1 - T + |l)(r|) y_r = g_r, on the device GMRES.
Every block product is compiled once, on the host, into two grouped-GEMM programs
(imps_plan_program, sector matching as for the excitation ansatz) around the two solves; the
scalars that depend on the state (N0, N1) enter at run time.  Restricted to tangent directions
N_L X the gradient equals the reference's tangent-space gradient:
<G0, N_L X> = <H_AC AC - AL H_C C, N_L X C> (VUMPS_helpers.hpp:135-177).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from . import blocks as B
from . import ops
from .excitations import ES, OPS, OUT, RHS, SCR, Program, Tensor, _left_group, _right_group, _same_group, expr


def _layout_tensor(prog, slot, lay, ngroups):
    """A tensor laid out exactly as the device layout `lay` (contiguous, in its block order)."""
    base = prog.alloc(slot, lay.nelem)
    blocks = {}
    for (g, qi, qo, r, c), off in zip(lay.blocks, lay.offsets):
        blocks[(g if ngroups > 1 else 0, tuple(qi))] = (tuple(qo), r, c, base + off)
    return (Tensor(slot, blocks, ngroups), None), base


def _hsplit(hnnz, d):
    return [(divmod(int(r), d), divmod(int(c), d), float(v)) for (r, c, v) in hnnz]


class EnergyGradientProgram:
    """Host compilation of the gradient for the layouts LA = [A0, A1] (MPS) and LB = [bond 0,
    bond 1] (block-diagonal), and the two-site nonzeros hnnz = [(row, col, value)] with
    row = s*d + t (bra) and col = s'*d + t' (ket)."""

    def __init__(self, LA, LB, hnnz, d):
        self.d = d
        pa = Program({})
        self.A0, self.a0_off = _layout_tensor(pa, OPS, LA[0], d)
        self.A1, self.a1_off = _layout_tensor(pa, OPS, LA[1], d)
        self.r, self.r_off = _layout_tensor(pa, OPS, LB[0], 1)
        mat = pa.materialize
        hs = _hsplit(hnnz, d)
        A0, A1, r = self.A0, self.A1, self.r

        def target(slot, lay, ng):
            t, off = _layout_tensor(pa, slot, lay, ng)
            return t, off

        # r1 = T~_1(r) on bond 1; A1 r, A0 r1 in the MPS layouts
        self.A1r, self.a1r_off = target(SCR, LA[1], d)
        mat([(expr(A1), expr(r), _left_group)], d, target=self.A1r)
        self.r1, _ = target(SCR, LB[1], 1)
        mat([(expr(self.A1r), expr(A1, t=True), _same_group)], 1, target=self.r1)
        self.A0r1, self.a0r1_off = target(SCR, LA[0], d)
        mat([(expr(A0), expr(self.r1), _left_group)], d, target=self.A0r1)
        # ReducedOp environments (d*d groups)
        const = lambda g: (lambda ga, gb: g)
        self.W = mat([(expr(self.A1r, coef=v, group=tp), expr(A1, group=t, t=True), const(s * d + sp))
                      for ((s, t), (sp, tp), v) in hs], d * d)[0]
        self.Wp = mat([(expr(self.A0r1, coef=v, group=sp), expr(A0, group=s, t=True), const(t * d + tp))
                       for ((t, s), (tp, sp), v) in hs], d * d)[0]
        self.V = mat([(expr(A0, coef=v, group=s, t=True), expr(A0, group=sp), const(t * d + tp))
                      for ((s, t), (sp, tp), v) in hs], d * d)[0]
        self.Vp = mat([(expr(A1, coef=v, group=t, t=True), expr(A1, group=tp), const(s * d + sp))
                       for ((t, s), (tp, sp), v) in hs], d * d)[0]
        # direct terms in the MPS layouts: G0a = sum A0[s'] W[s][s'], G0b = sum V'[s][s'] A0[s'],
        # G1a = sum V[t][t'] A1[t'], G1b = sum A1[t'] W'[t][t']
        rng = range(d)
        self.G0a, self.g0a_off = target(SCR, LA[0], d)
        mat(self._w_right(A0, self.W), d, target=self.G0a)
        self.G1b, self.g1b_off = target(SCR, LA[1], d)
        mat(self._w_right(A1, self.Wp), d, target=self.G1b)
        self.G1a, _ = target(SCR, LA[1], d)
        mat([(expr(self.V, group=t * d + tp), expr(A1, group=tp), const(t)) for t in rng for tp in rng], d,
            target=self.G1a)
        self.G0b, _ = target(SCR, LA[0], d)
        mat([(expr(self.Vp, group=s * d + sp), expr(A0, group=sp), const(s)) for s in rng for sp in rng], d,
            target=self.G0b)
        # E~1(r1) and E1(l1) on bond 1
        self.Et1, _ = target(SCR, LB[1], 1)
        mat([(expr(self.G1b), expr(A1, t=True), _same_group)], 1, target=self.Et1)
        self.E1l, _ = target(SCR, LB[1], 1)
        mat([(expr(A0, t=True), expr(self.G0b), _same_group)], 1, target=self.E1l)
        # right-hand sides (before the -E2/2 r and -E2/2 1 corrections):
        # g_l = (E~0(r) + T~_0(E~1(r1))) / 2, g_r = (E0(1) + T_1(E1(1))) / 2 on bond 0
        self.A0Et1 = mat([(expr(A0), expr(self.Et1), _left_group)], d)[0]
        self.E1lA1 = mat([(expr(self.E1l), expr(A1), _right_group)], d)[0]
        self.gl, self.gl_off = target(RHS, LB[0], 1)
        mat([(expr(self.G0a, coef=0.5), expr(A0, t=True), _same_group),
             (expr(self.A0Et1, coef=0.5), expr(A0, t=True), _same_group)], 1, target=self.gl)
        self.gr, self.gr_off = target(RHS, LB[0], 1)
        mat([(expr(A1, coef=0.5, t=True), expr(self.G1a), _same_group),
             (expr(A1, coef=0.5, t=True), expr(self.E1lA1), _same_group)], 1, target=self.gr)
        pa.closed = True
        self.prog_a = pa
        # ---- program B: from the adjoint solutions y_l, y_r (ES slot) to the gradient (OUT) ----
        pb = Program(dict(pa.sizes))
        self.yl, self.yl_off = _layout_tensor(pb, ES, LB[0], 1)
        self.yr, self.yr_off = _layout_tensor(pb, ES, LB[0], 1)
        matb = pb.materialize
        A1yl = matb([(expr(A1), expr(self.yl), _left_group)], d)[0]
        self.T1yl, _ = _layout_tensor(pb, SCR, LB[1], 1)
        matb([(expr(A1yl), expr(A1, t=True), _same_group)], 1, target=self.T1yl)
        yrA0 = matb([(expr(self.yr), expr(A0), _right_group)], d)[0]
        self.T0yr, _ = _layout_tensor(pb, SCR, LB[1], 1)
        matb([(expr(A0, t=True), expr(yrA0), _same_group)], 1, target=self.T0yr)
        T0yrA1 = matb([(expr(self.T0yr), expr(A1), _right_group)], d)[0]
        # z_l = -y_l, z_r = -y_r: the -2 (z ...) terms enter with +2
        self.G0, self.g0_off = _layout_tensor(pb, OUT, LA[0], d)
        matb(self._w_right(A0, self.W) + [
            (expr(self.G0b), expr(self.r1), _left_group),
            (expr(A0), expr(self.Et1), _left_group),
            (expr(A0, coef=2.0), expr(self.T1yl), _left_group),
            (expr(yrA0, coef=2.0), expr(self.r1), _left_group)], d, target=self.G0)
        self.G1, self.g1_off = _layout_tensor(pb, OUT, LA[1], d)
        matb(self._w_right(A1, self.Wp) + [
            (expr(self.G1a), expr(r), _left_group),
            (expr(self.E1lA1), expr(r), _left_group),
            (expr(T0yrA1, coef=2.0), expr(r), _left_group),
            (expr(A1, coef=2.0), expr(self.yl), _left_group)], d, target=self.G1)
        self.prog_b = pb
        self.sizes = dict(pb.sizes)

    def _w_right(self, A, W):
        """Products of sum_s' A[s'] W[s][s'] into group s."""
        d = self.d
        return [(expr(A, group=sp), expr(W, group=s * d + sp), (lambda ga, gb, g=s: g))
                for s in range(d) for sp in range(d)]


class EnergyGradientGPU:
    """dE/dA of the energy density at a left-isometric two-site unit cell on the device: program
    A, the two adjoint InvertE_proj solves on the transposed unit-cell TMs, program B."""

    def __init__(self, ctx, LA, LB, hnnz, d, tol=1e-13, maxit=0):
        import torch
        self.torch, self.ctx, self.d, self.tol, self.maxit = torch, ctx, d, tol, maxit
        self.LA, self.LB = LA, LB
        self.pr = pr = EnergyGradientProgram(LA, LB, hnnz, d)
        dev = lambda n: torch.zeros(max(int(n), 1), dtype=torch.float64, device="cuda")
        self.buf = {k: dev(pr.sizes.get(k, 0)) for k in range(6)}
        self.plan_a = self._plan(pr.prog_a)
        self.plan_b = self._plan(pr.prog_b)
        # transposed unit-cell TMs for the adjoint solves: right-acting for y_l, left-acting for y_r
        self.tm_r = B.plan_tm(ctx, [LA[0], LA[1]], 1, LB[0], LB[0])
        self.tm_l = B.plan_tm(ctx, [LA[0], LA[1]], 0, LB[0], LB[0])
        ops_buf = self.buf[OPS]
        a0 = ops_buf[pr.a0_off:pr.a0_off + LA[0].nelem]
        a1 = ops_buf[pr.a1_off:pr.a1_off + LA[1].nelem]
        for p in (self.tm_r, self.tm_l):
            p.bind(2, a0)
            p.bind(3, a1)
        eye = np.concatenate([np.eye(b[3]).reshape(-1) for b in LB[0].blocks]) if LB[0].blocks else np.zeros(1)
        self.eye0 = torch.from_numpy(eye).to("cuda")
        self.stats = {"gmres_iters": 0}

    def _plan(self, prog):
        nouts, outs, terms, alphas = prog.tables()
        sizes = np.array([max(int(self.buf[k].numel()), 1) for k in range(6)], np.int64)
        h = C.c_void_p()
        N.call("imps_plan_program", self.ctx.handle, 6, sizes.ctypes.data_as(N.P_i64), len(nouts),
               nouts.ctypes.data_as(N.P_i32), outs.ctypes.data_as(N.P_i64), terms.ctypes.data_as(N.P_i64),
               alphas.ctypes.data_as(N.P_dbl), C.byref(h))
        plan = B.Plan(self.ctx, h, "program")
        for k in range(6):
            plan.bind(k, self.buf[k])
        return plan

    def _seg(self, slot, off, n):
        return self.buf[slot][off:off + n]

    def __call__(self, AL0, AL1, R):
        """Gradient at the device tensors AL0, AL1 (layouts LA) with the right fixed point R
        (bond 0, any positive trace).  Returns (G0, G1, e, (N0, N1), converged)."""
        pr, ctx, LA, LB = self.pr, self.ctx, self.LA, self.LB
        n0, n1, nb = LA[0].nelem, LA[1].nelem, LB[0].nelem
        self._seg(OPS, pr.a0_off, n0).copy_(AL0)
        self._seg(OPS, pr.a1_off, n1).copy_(AL1)
        r = self._seg(OPS, pr.r_off, nb)
        r.copy_(R)
        tr = ops.bd_trace_prod(ctx, LB[0], r, self.eye0)
        r.mul_(1.0 / tr)
        self.plan_a.run()
        N0 = ops.dot(ctx, self._seg(SCR, pr.g0a_off, n0), self._seg(OPS, pr.a0_off, n0))
        N1 = ops.dot(ctx, self._seg(SCR, pr.g1b_off, n1), self._seg(OPS, pr.a1_off, n1))
        E2, E2l = N0 + N1, N0 + 2.0 * N1
        gl, gr = self._seg(RHS, pr.gl_off, nb), self._seg(RHS, pr.gr_off, nb)
        ops.axpby(ctx, -0.5 * E2, r, 1.0, gl)
        ops.axpby(ctx, -0.5 * E2, self.eye0, 1.0, gr)
        yl, yr = self._seg(ES, pr.yl_off, nb), self._seg(ES, pr.yr_off, nb)
        yl.zero_()
        yr.zero_()
        it1, _, c1 = ops.InvertE_proj(self.tm_r, gl, self.eye0, r, "r", yl, self.tol, self.maxit)
        it2, _, c2 = ops.InvertE_proj(self.tm_l, gr, self.eye0, r, "l", yr, self.tol, self.maxit)
        self.stats["gmres_iters"] += it1 + it2
        self.plan_b.run()
        G0 = self._seg(OUT, pr.g0_off, n0)
        G1 = self._seg(OUT, pr.g1_off, n1)
        ops.axpby(ctx, -E2l, self._seg(SCR, pr.a0r1_off, n0), 1.0, G0)
        ops.axpby(ctx, -E2l, self._seg(SCR, pr.a1r_off, n1), 1.0, G1)
        return G0, G1, 0.5 * E2, (N0, N1), c1 and c2


def coupling_terms(model, **params):
    """The two-site h as sum_k g_k h_k: the coupling names and the nonzeros of each h_k (h is
    linear in its couplings for both models)."""
    from . import models
    names = {"xxz": ("J", "Delta", "hz"), "fhub": ("t", "U", "V", "mu", "hz")}[model]
    out = []
    for k in names:
        unit = {n: (1.0 if n == k else 0.0) for n in names}
        _, _, hk = models.build_model(model, **unit)
        out.append((k, models.h_nonzeros(hk)))
    return out


class CouplingGradientGPU:
    """dE/dg_k at fixed A: the energy density with h replaced by h_k = dh/dg_k (Hellmann-Feynman
    at fixed state), from program A's N0 and N1 for each h_k."""

    def __init__(self, ctx, LA, LB, model, d, **params):
        self.terms = coupling_terms(model, **params)
        self.grads = [(k, EnergyGradientGPU(ctx, LA, LB, hk, d)) for k, hk in self.terms]

    def __call__(self, AL0, AL1, R):
        out = {}
        for k, g in self.grads:
            pr, ctx = g.pr, g.ctx
            n0, n1, nb = g.LA[0].nelem, g.LA[1].nelem, g.LB[0].nelem
            g._seg(OPS, pr.a0_off, n0).copy_(AL0)
            g._seg(OPS, pr.a1_off, n1).copy_(AL1)
            r = g._seg(OPS, pr.r_off, nb)
            r.copy_(R)
            r.mul_(1.0 / ops.bd_trace_prod(ctx, g.LB[0], r, g.eye0))
            g.plan_a.run()
            N0 = ops.dot(ctx, g._seg(SCR, pr.g0a_off, n0), g._seg(OPS, pr.a0_off, n0))
            N1 = ops.dot(ctx, g._seg(SCR, pr.g1b_off, n1), g._seg(OPS, pr.a1_off, n1))
            out[k] = 0.5 * (N0 + N1)
        return out
