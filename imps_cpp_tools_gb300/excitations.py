"""Effective Hamiltonian of the excitation ansatz on the GPU (Excitations_helpers.hpp:20-228).

ApplyHeff is compiled once per structure into two grouped-GEMM programs (imps_plan_program)
around the two factored environment solves (imps_invert_e_fac):

* the sector matching of every block product is done here, on the host, exactly once;
* complex tensors (X, B = N_L X, the environments of B) are pairs of real planes; every
  product has one real operand (AL, AR, N_L, the environments of the ground state), so
  a complex scalar (e^{ip}) or a sum of tensors becomes several GEMM terms with real alphas
  accumulated into the same output block, and ApplyOperator becomes terms weighted by the
  nonzeros of h;
* a product whose operand is itself a product is materialised first (one stage per
  materialisation, in order).

Block structures are passed as the reference's map-of-blocks: an MPS tensor is a list over the
physical index s of {qin: (qout, matrix)}, a BlockMat is {qin: (qout, matrix)}, a BlockDiagMat
is {q: matrix}.  Vectors use the reference's Vectorize order (s-major, std::map key order,
blocks column-major).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from . import blocks as B
from . import charges, models, ops

OPS, XS, OUT, SCR, ES, RHS = range(6)


def _kadd(a, b):
    return tuple(x + y for x, y in zip(a, b))


class Tensor:
    """A materialised real block tensor in one slot: blocks[(g, qin)] = (qout, rows, cols, off)."""

    def __init__(self, slot, blocks, ngroups):
        self.slot, self.blocks, self.ngroups = slot, blocks, ngroups

    def nelem(self):
        return sum(r * c for (_, r, c, _) in self.blocks.values())

    def view(self, group=None, t=False):
        return View(self, group, t)


class View:
    """Blocks of a tensor, optionally one physical group only (relabelled to group 0) and/or
    transposed: items (g, key_in, key_out, rows, cols, slot, off, ld, trans)."""

    def __init__(self, tensor, group=None, t=False):
        self.tensor, self.group, self.t = tensor, group, t

    def items(self):
        for (g, qi), (qo, r, c, off) in self.tensor.blocks.items():
            if self.group is not None and g != self.group:
                continue
            gg = 0 if self.group is not None else g
            if self.t:
                yield gg, qo, qi, c, r, self.tensor.slot, off, r, 1
            else:
                yield gg, qi, qo, r, c, self.tensor.slot, off, r, 0


def expr(ct, coef=1.0, group=None, t=False):
    """Linear expression of a complex (re, im) or real (re, None) tensor pair."""
    re, im = ct
    out = [(complex(coef), re.view(group, t))]
    if im is not None:
        out.append((complex(coef) * 1j, im.view(group, t)))
    return out


def scale(e, c):
    return [(coef * c, v) for coef, v in e]


class Program:
    """Stages of a grouped-GEMM program being compiled."""

    def __init__(self, sizes):
        self.sizes = dict(sizes)  # slot -> elements used
        self.stages = []
        self.closed = False  # set once a later program depends on this one's results

    def alloc(self, slot, n):
        off = self.sizes.get(slot, 0)
        self.sizes[slot] = off + n
        return off

    def materialize(self, products, ngroups, slot=SCR, target=None, force_complex=False):
        """Sum of products sum_p c_p op(A_p) op(B_p) into a new tensor pair (re, im).  products:
        list of (exprA, exprB, rule) with rule(gA, gB) -> output group or None.  target: a
        (re, im) pair of tensors with a fixed structure (sectors outside it are dropped)."""
        if self.closed:
            raise RuntimeError("materialisation into a closed program")
        terms = {}  # (plane, gkey) -> list of term tuples
        shape = {}  # gkey -> (qout, rows, cols)
        dropped = 0
        for ea, eb, rule in products:
            for ca, va in ea:
                for ca2, vb in eb:
                    idx = {}
                    for bi in vb.items():
                        idx.setdefault(bi[1], []).append(bi)
                    c = ca * ca2
                    for (ga, ki, ko, ra, kk, sa, oa, la, ta) in va.items():
                        for (gb, kbi, kbo, rb, cb, sb, ob, lb, tb) in idx.get(ko, ()):
                            g = rule(ga, gb)
                            if g is None:
                                continue
                            if kk != rb:
                                raise ValueError("inner dimensions do not match")
                            key = (g, ki)
                            if target is not None and key not in target[0].blocks:
                                dropped += 1
                                continue
                            sh = (kbo, ra, cb)
                            if shape.setdefault(key, sh) != sh:
                                raise ValueError("inconsistent output sector")
                            term = (sa, oa, la, ta, sb, ob, lb, tb, kk)
                            if c.real != 0.0:
                                terms.setdefault((0, key), []).append(term + (c.real,))
                            if c.imag != 0.0:
                                terms.setdefault((1, key), []).append(term + (c.imag,))
        cplx = force_complex or any(p == 1 for (p, _) in terms) or target is not None
        if target is None:
            off = 0
            keys = sorted(shape)
            nel = sum(shape[k][1] * shape[k][2] for k in keys)
            base_re = self.alloc(slot, nel)
            base_im = self.alloc(slot, nel) if cplx else None
            re_blocks, im_blocks = {}, {}
            for k in keys:
                qo, r, c = shape[k]
                re_blocks[k] = (qo, r, c, base_re + off)
                if cplx:
                    im_blocks[k] = (qo, r, c, base_im + off)
                off += r * c
            re = Tensor(slot, re_blocks, ngroups)
            im = Tensor(slot, im_blocks, ngroups) if cplx else None
        else:
            re, im = target
        outs = []
        for plane, t in ((0, re), (1, im)):
            if t is None:
                continue
            for key, (qo, r, c, off) in sorted(t.blocks.items()):
                outs.append((t.slot, off, r, r, c, 0, terms.get((plane, key), [])))
        self.stages.append(outs)
        return (re, im), dropped

    def tables(self):
        nouts = np.array([len(st) for st in self.stages], np.int32)
        outs, terms, alphas = [], [], []
        for st in self.stages:
            for (cs, coff, cld, M, Nn, acc, tl) in st:
                outs.append((cs, coff, max(cld, 1), M, Nn, acc, len(tl)))
                for tm in tl:
                    terms.append(tm[:9])
                    alphas.append(tm[9])
        return (nouts, np.array(outs, np.int64).reshape(-1, 7), np.array(terms, np.int64).reshape(-1, 9),
                np.array(alphas, np.float64))


def _same_group(ga, gb):
    return 0 if ga == gb else None


def _left_group(ga, gb):
    return ga


def _right_group(ga, gb):
    return gb


def _bm(ga, gb):
    return 0


class HeffProgram:
    """Host compilation of ApplyHeff for a unit cell of N sites at momentum factor kfac and a
    charge offset of X (unprojected solves: K != 0 or p != 0).  AL, AR, NL: lists (sites) of
    MPS tensors; HLtot, HRtot: lists of BlockDiagMats; hnnz: (row, col, value) nonzeros of the
    two-site h with E0 subtracted; xdims: per site [(qin, qout, rows, cols)] of X (XDims order).
    Produces program A (up to the right-hand sides of the two solves), the solves' structures,
    and program B (from their solutions to X_out), over six slots: operands, X, X_out, scratch,
    solutions, right-hand sides."""

    def __init__(self, AL, AR, NL, HLtot, HRtot, hnnz, d, xdims, kfac):
        self.d = d
        self.kfac = complex(kfac)
        self.NS = len(AL)
        ns = len(next(iter(xdims[0]))[0]) if xdims[0] else len(next(iter(AL[0][0])))
        self.nsym = ns
        Ns = self.NS
        P = lambda x: (x + Ns) % Ns
        prog_a = Program({})
        # ---- operands in the OPS slot (real) ----
        vals = []

        def add_mps(A):
            blocks = {}
            for s, bm in enumerate(A):
                for qi in sorted(bm):
                    qo, M = bm[qi]
                    off = prog_a.alloc(OPS, M.size)
                    blocks[(s, tuple(qi))] = (tuple(qo), M.shape[0], M.shape[1], off)
                    vals.append(np.asarray(M, np.float64).reshape(-1, order="F"))
            return (Tensor(OPS, blocks, len(A)), None)

        def add_bd(X):
            blocks = {}
            for q in sorted(X):
                M = X[q]
                off = prog_a.alloc(OPS, M.size)
                blocks[(0, tuple(q))] = (tuple(q), M.shape[0], M.shape[1], off)
                vals.append(np.asarray(M, np.float64).reshape(-1, order="F"))
            return (Tensor(OPS, blocks, 1), None)

        self.AL = [add_mps(a) for a in AL]
        self.AR = [add_mps(a) for a in AR]
        self.NL = [add_mps(a) for a in NL]
        self.HL = [add_bd(x) for x in HLtot]
        self.HR = [add_bd(x) for x in HRtot]
        self.ops_vec = np.concatenate(vals) if vals else np.zeros(1)
        # ---- X and the output (XS, OUT slots): per site [re | im] ----
        self.xdims = xdims
        self.X, self.Y, self.xoff = [], [], []
        xo = 0
        for dims in xdims:
            n = sum(r * c for (_, _, r, c) in dims)
            re, im, off = {}, {}, 0
            for (qi, qo, r, c) in dims:
                re[(0, tuple(qi))] = (tuple(qo), r, c, xo + off)
                im[(0, tuple(qi))] = (tuple(qo), r, c, xo + n + off)
                off += r * c
            self.X.append((Tensor(XS, re, 1), Tensor(XS, im, 1)))
            self.Y.append((Tensor(OUT, dict(re), 1), Tensor(OUT, dict(im), 1)))
            self.xoff.append((xo, n))
            xo += 2 * n
        self.mtot = sum(n for (_, n) in self.xoff)
        prog_a.sizes[XS] = prog_a.sizes[OUT] = xo
        kf, ck = self.kfac, self.kfac.conjugate()
        mat = prog_a.materialize
        ALe = lambda n, **kw: expr(self.AL[n], **kw)
        ARe = lambda n, **kw: expr(self.AR[n], **kw)
        # ---- program A: B = NL X, ABR chain, HBL chain ----
        Bin = [mat([(expr(self.NL[n]), expr(self.X[n]), _left_group)], d)[0] for n in range(Ns)]
        ABR = [None] * Ns

        def mixed_right(e_a, n):  # sum_s A_s AR[n]_s^T  (unity right, A an expression)
            return [(e_a, ARe(n, t=True), _same_group)]

        ABR[Ns - 1] = mat(mixed_right(expr(Bin[Ns - 1]), Ns - 1), 1, force_complex=True,
                          slot=RHS if Ns == 1 else SCR)[0]
        for n in range(Ns - 1, 0, -1):
            alabr = mat([(ALe(n - 1), expr(ABR[n]), _left_group)], d)[0]
            ABR[n - 1] = mat(mixed_right(expr(Bin[n - 1]) + expr(alabr), n - 1), 1, force_complex=True,
                             slot=RHS if n - 1 == 0 else SCR)[0]
        self.ABR = ABR

        def op_group(t2, ii):  # ApplyOperator(t2, h)[ii] as an expression (group relabelled to 0)
            e = []
            for (r, c, v) in hnnz:
                if r == ii:
                    e += expr(t2, coef=v, group=c)
            return e

        def optm_left(a2, aa, prods):  # ApplyOpTMLeftGen(h, a2, aa) = sum_g aa_g^T (h a2)_g
            for g in range(d * d):
                oe = []
                for t2, coef in a2:
                    oe += scale(op_group(t2, g), coef)
                if oe:
                    prods.append((expr(aa, group=g, t=True), oe, _bm))

        def mps2(ea, eb, materialize=mat):  # two-site product A_i B_j -> group i*d + j
            return materialize([(ea, eb, lambda ga, gb: ga * d + gb)], d * d)[0]

        HBL = []
        for n in range(Ns):
            prods = []
            if n == 0:
                hlb = mat([(expr(self.HL[Ns - 1]), expr(Bin[0]), _right_group)], d)[0]
                prods.append((expr(self.AL[0], t=True), expr(hlb), _same_group))
                a2 = [(mps2(ALe(Ns - 1), expr(Bin[0])), 1.0), (mps2(expr(Bin[Ns - 1]), ARe(0)), ck)]
                aa = mps2(ALe(Ns - 1), ALe(0))
            else:
                w1 = mat([(expr(HBL[-1]), ARe(n), _right_group)], d)[0]
                w2 = mat([(expr(self.HL[n - 1]), expr(Bin[n]), _right_group)], d)[0]
                prods.append((expr(self.AL[n], t=True), expr(w1) + expr(w2), _same_group))
                a2 = [(mps2(ALe(n - 1), expr(Bin[n])), 1.0), (mps2(expr(Bin[n - 1]), ARe(n)), 1.0)]
                aa = mps2(ALe(n - 1), ALe(n))
            optm_left(a2, aa, prods)
            HBL.append(mat(prods, 1, force_complex=True, slot=RHS if n == Ns - 1 else SCR)[0])
        self.HBL = HBL
        # right-hand sides of the two solves: ABR[0] and HBL[N-1], both in RHS
        self.rhs_r, self.rhs_l = ABR[0], HBL[Ns - 1]
        # the solutions of (1 - kfac T_R^{AL,AR}) EBR = ABR[0] and (1 - ck T_L^{AR,AL}) EHBL =
        # HBL[N-1] live in ES: EBR [re | im], EHBL [re | im], same structure as the rhs
        nr, nl = self.rhs_r[0].nelem(), self.rhs_l[0].nelem()

        def in_es(t, base):
            n = t.nelem()
            shift = lambda blocks, b0: {k: (v[0], v[1], v[2], b0 + (v[3] - min(x[3] for x in blocks.values())))
                                        for k, v in blocks.items()}
            return (Tensor(ES, shift(t.blocks, base), 1), Tensor(ES, shift(t.blocks, base + n), 1))

        EBR, EHBL = in_es(self.rhs_r[0], 0), in_es(self.rhs_l[0], 2 * nr)
        self.Bin, self.EBR, self.EHBL = Bin, EBR, EHBL
        self.es_size = 2 * (nr + nl)
        self.nr, self.nl = nr, nl
        # ---- program B: per-bond sums of the solutions, the output terms, X_out = NL^T B_out ----
        prog_a.closed = True
        prog_b = Program(prog_a.sizes)
        prog_b.sizes[ES] = self.es_size
        matb = prog_b.materialize
        ABRtot = [None] * Ns
        ABRtot[0] = expr(EBR, coef=kf)
        E = EBR
        for n in range(Ns - 1, 0, -1):
            w = matb([(ALe(n), expr(E), _left_group)], d)[0]
            E = matb([(expr(w), ARe(n, t=True), _same_group)], 1, force_complex=True)[0]
            ABRtot[n] = expr(ABR[n]) + expr(E, coef=kf)
        self.bouts = []  # B_out[n] (scratch), kept for inspection
        HBLtot = [None] * Ns
        HBLtot[Ns - 1] = expr(EHBL, coef=ck)
        E = EHBL
        for n in range(Ns - 1):
            w = matb([(expr(E), ARe(n), _right_group)], d)[0]
            E = matb([(expr(self.AL[n], t=True), expr(w), _same_group)], 1, force_complex=True)[0]
            HBLtot[n] = expr(HBL[n]) + expr(E, coef=ck)

        def contract(prods, n, left2=None, right2=None, coef=1.0):
            """+= coef sum_k AL[n-1][k]^T (h left2)[k d + s] + sum_k (h right2)[s d + k] AR[n+1][k]^T."""
            for s in range(d):
                for k in range(d):
                    if left2 is not None:
                        oe = op_group(left2, k * d + s)
                        if oe:
                            prods.append((expr(self.AL[P(n - 1)], group=k, t=True), scale(oe, coef),
                                          lambda ga, gb, s=s: s))
                    if right2 is not None:
                        oe = op_group(right2, s * d + k)
                        if oe:
                            prods.append((oe, expr(self.AR[P(n + 1)], group=k, t=True), lambda ga, gb, s=s: s))

        for n in range(Ns):
            prods = [(expr(self.HL[P(n - 1)]), expr(Bin[n]), _right_group),
                     (expr(Bin[n]), expr(self.HR[P(n + 1)]), _left_group)]
            # h on B and the output site
            contract(prods, n, mps2(ALe(P(n - 1)), expr(Bin[n]), matb), mps2(expr(Bin[n]), ARe(P(n + 1)), matb))
            # B left of the output site
            prods.append((HBLtot[P(n - 1)], ARe(n), _right_group))
            contract(prods, n, mps2(expr(Bin[P(n - 1)]), ARe(n), matb), None, ck if n == 0 else 1.0)
            # B right of the output site
            alabr2 = matb([(ALe(P(n + 1)), ABRtot[P(n + 2)], _left_group)], d, force_complex=True)[0]
            atmp = expr(Bin[P(n + 1)]) + expr(alabr2)
            if n == Ns - 1:
                atmp = scale(atmp, kf)
            alabr = matb([(ALe(n), ABRtot[P(n + 1)], _left_group)], d, force_complex=True)[0]
            prods.append((expr(self.HL[P(n - 1)]), expr(alabr), _right_group))
            a2d = mps2(ALe(P(n - 1)), expr(alabr), matb)
            a2e = matb([(ALe(n), atmp, lambda ga, gb: ga * d + gb)], d * d, force_complex=True)[0]
            contract(prods, n, a2d, a2e)
            bout = matb(prods, d, force_complex=True)[0]
            self.bouts.append(bout)
            # X_out[n] = sum_s NL[n]_s^T B_out[n]_s, into the output's X structure
            matb([(expr(self.NL[n], t=True), expr(bout), _same_group)], 1, target=self.Y[n])

        self.prog_a, self.prog_b = prog_a, prog_b
        self.sizes = {k: max(prog_a.sizes.get(k, 0), prog_b.sizes.get(k, 0)) for k in range(6)}
        self.sizes[ES] = self.es_size
        self.structs = (AL, AR)

    def rhs_planes(self):
        """(offset of re, offset of im, length) of the two right-hand sides in RHS."""
        lo = lambda t: min(v[3] for v in t.blocks.values())
        return ((lo(self.rhs_r[0]), lo(self.rhs_r[1]), self.nr), (lo(self.rhs_l[0]), lo(self.rhs_l[1]), self.nl))


class HeffGPU:
    """ApplyHeff on the device: the two programs of HeffProgram around two imps_invert_e_fac
    solves on mixed transfer-matrix plans; with LM and RM (the dominant eigenmatrices of the
    mixed TM, LRoverlaps) the solves are the projected imps_invert_e_proj_fac ones
    (Excitations_helpers.hpp:83, 124: EBR with (LM, RM), EHBL with (LM^T, RM^T))."""

    def __init__(self, ctx, AL, AR, NL, HLtot, HRtot, hnnz, d, xdims, kfac, tol=1e-14, maxit=0, LM=None, RM=None):
        import torch
        self.torch, self.ctx, self.d = torch, ctx, d
        self.tol, self.maxit = tol, maxit
        pr = HeffProgram(AL, AR, NL, HLtot, HRtot, hnnz, d, xdims, kfac)
        self.pr = pr
        self.kfac, self.NS, self.xoff, self.mtot = pr.kfac, pr.NS, pr.xoff, pr.mtot
        self.sizes, self.nr, self.nl = pr.sizes, pr.nr, pr.nl
        Ns, ns_ = pr.NS, pr.nsym
        lay_mps = lambda A: B.Layout([(s, tuple(qi), tuple(bm[qi][0]), bm[qi][1].shape[0], bm[qi][1].shape[1])
                                      for s, bm in enumerate(A) for qi in sorted(bm)], ns_)
        lay_t = lambda t: B.Layout([(0, k[1], v[0], v[1], v[2]) for k, v in sorted(t.blocks.items())], ns_)
        self.lay_AL = [lay_mps(a) for a in AL]
        self.lay_AR = [lay_mps(a) for a in AR]
        self.lay_r, self.lay_l = lay_t(pr.rhs_r[0]), lay_t(pr.rhs_l[0])
        self.plan_r = B.plan_tm_mixed(ctx, self.lay_AL, self.lay_AR, 1, self.lay_r, self.lay_r)
        self.plan_l = B.plan_tm_mixed(ctx, self.lay_AR, self.lay_AL, 0, self.lay_l, self.lay_l)
        self.AL, self.AR = pr.AL, pr.AR
        dev = lambda n: torch.zeros(max(int(n), 1), dtype=torch.float64, device="cuda")
        self.buf = {k: dev(self.sizes.get(k, 0)) for k in range(6)}
        self.buf[OPS].copy_(torch.from_numpy(pr.ops_vec))
        self.plan_a = self._plan(pr.prog_a)
        self.plan_b = self._plan(pr.prog_b)
        A_ = lambda lst, k: self._op_view(lst[k])
        for k in range(Ns):
            self.plan_r.bind(2 + k, A_(self.AL, k))
            self.plan_r.bind(2 + Ns + k, A_(self.AR, k))
            self.plan_l.bind(2 + k, A_(self.AR, k))
            self.plan_l.bind(2 + Ns + k, A_(self.AL, k))
        self.stats = {"gmres_iters": 0}
        self.proj = LM is not None and RM is not None
        if self.proj:
            # (rho_in, rho_out) of InvEfun_proj_fac: the EBR solve (dir r) takes (L, R) = (LM, RM),
            # the EHBL solve (dir l) (R, L) = (RM^T, LM^T); rho_out pairs with x's blocks, rho_in
            # with the transposed structure (InvEBlockFunctions.hpp:104-108)
            tdev = lambda v: torch.from_numpy(np.ascontiguousarray(v, np.float64)).to("cuda")
            bt = lambda X: {qo: (qi, M.T.copy()) for qi, (qo, M) in X.items()}
            self.proj_r = (tdev(_rho_vec(self.lay_r, LM, inside=True)), tdev(_rho_vec(self.lay_r, RM, inside=False)))
            self.proj_l = (tdev(_rho_vec(self.lay_l, bt(LM), inside=False)),
                           tdev(_rho_vec(self.lay_l, bt(RM), inside=True)))

    def _op_view(self, ct):
        t = ct[0]
        offs = [v[3] for v in t.blocks.values()]
        lo, n = min(offs), t.nelem()
        return self.buf[OPS][lo:lo + n]

    def _plan(self, prog):
        nouts, outs, terms, alphas = prog.tables()
        sizes = np.array([max(int(self.sizes.get(k, 0)), 1) for k in range(6)], np.int64)
        h = C.c_void_p()
        N.call("imps_plan_program", self.ctx.handle, 6, sizes.ctypes.data_as(N.P_i64), len(nouts),
               nouts.ctypes.data_as(N.P_i32), outs.ctypes.data_as(N.P_i64), terms.ctypes.data_as(N.P_i64),
               alphas.ctypes.data_as(N.P_dbl), C.byref(h))
        plan = B.Plan(self.ctx, h, "program")
        for k in range(6):
            plan.bind(k, self.buf[k])
        return plan

    def x_to_planes(self, xs):
        """Per-site complex vectors (XDims order) -> the XS slot."""
        torch = self.torch
        for (xo, n), x in zip(self.xoff, xs):
            x = np.asarray(x, np.complex128)
            self.buf[XS][xo:xo + n].copy_(torch.from_numpy(x.real.copy()))
            self.buf[XS][xo + n:xo + 2 * n].copy_(torch.from_numpy(x.imag.copy()))

    def y_from_planes(self):
        out = []
        for (xo, n) in self.xoff:
            re = self.buf[OUT][xo:xo + n].cpu().numpy()
            im = self.buf[OUT][xo + n:xo + 2 * n].cpu().numpy()
            out.append(re + 1j * im)
        return out

    def apply(self):
        """Y = H_eff X on the device buffers (XS -> OUT)."""
        self.plan_a.run()
        nr, nl = self.nr, self.nl
        rhs, es = self.buf[RHS], self.buf[ES]
        (off_r, off_ri, _), (off_l, off_li, _) = self.pr.rhs_planes()
        xr, xl = (rhs[off_r:off_r + nr], rhs[off_ri:off_ri + nr]), (rhs[off_l:off_l + nl], rhs[off_li:off_li + nl])
        yr, yl = (es[0:nr], es[nr:2 * nr]), (es[2 * nr:2 * nr + nl], es[2 * nr + nl:2 * nr + 2 * nl])
        ck = self.kfac.conjugate()
        if self.proj:
            it, _, conv_r = ops.InvertE_proj_fac(self.plan_r, *xr, *self.proj_r, "r", self.kfac, *yr, self.tol,
                                                 self.maxit)
            self.stats["gmres_iters"] += it
            it, _, conv_l = ops.InvertE_proj_fac(self.plan_l, *xl, *self.proj_l, "l", ck, *yl, self.tol, self.maxit)
        else:
            it, _, conv_r = ops.InvertE_fac(self.plan_r, *xr, self.kfac, *yr, self.tol, self.maxit)
            self.stats["gmres_iters"] += it
            it, _, conv_l = ops.InvertE_fac(self.plan_l, *xl, ck, *yl, self.tol, self.maxit)
        self.stats["gmres_iters"] += it
        self.plan_b.run()
        return conv_r and conv_l


class ExcitationsGPU:
    """Excitation energies of the ansatz (Excitations_main.cpp:255-297): for each momentum, the
    nev lowest eigenvalues of H_eff (eigs_n "SR" in the reference; H_eff is Hermitian, so here
    the device Lanczos on its real form over the [re | im] planes of X)."""

    def __init__(self, ctx, AL, AR, NL, HLtot, HRtot, hnnz, d, xdims, tol=1e-14, LM=None, RM=None):
        self.ctx, self.args, self.tol = ctx, (AL, AR, NL, HLtot, HRtot, hnnz, d, xdims), tol
        self.LM, self.RM = LM, RM
        qi, qo = next((b[0], b[1]) for dd in xdims for b in dd)
        self.K = tuple(b - a for a, b in zip(qi, qo))
        self.applies = 0

    def projected(self, p):
        """Excitations_main.cpp:263-268: the dominant subspace of the mixed TM is projected out of
        the environment solves only at K = 0 and momentum p = 0 (|p| < 10 InvETol)."""
        return self.LM is not None and all(k == 0 for k in self.K) and abs(p) < 10 * self.tol

    def energies(self, kfac, nev=4, eig_tol=1e-10, ncv=64, seed=1, p=None):
        """The nev lowest energies at kfac = e^{ip} (p: the momentum, default arg(kfac)).  ncv: the
        Lanczos basis (eigs.cpp's default is 20; with each H_eff apply costing two GMRES
        solves, 64 needs ~half the applies at XXZ D=256, with the same energies)."""
        import torch
        p = float(np.angle(kfac)) if p is None else float(p)
        LM, RM = (self.LM, self.RM) if self.projected(p) else (None, None)
        H = HeffGPU(self.ctx, *self.args, kfac, tol=self.tol, LM=LM, RM=RM)
        n = 2 * H.mtot
        xs, out = H.buf[XS], H.buf[OUT]

        def apply(pin, pout):
            N.call("imps_axpby", self.ctx.handle, 1.0, C.c_void_p(pin), 0.0, C.c_void_p(xs.data_ptr()), n)
            if not H.apply():
                raise RuntimeError("environment solve did not converge")
            N.call("imps_axpby", self.ctx.handle, 1.0, C.c_void_p(out.data_ptr()), 0.0, C.c_void_p(pout), n)

        g = torch.Generator(device="cpu").manual_seed(seed)
        x = torch.randn(n, generator=g, dtype=torch.float64).to("cuda")
        # the real form doubles every eigenvalue (x and i x); a Lanczos run finds each once in
        # exact arithmetic, but rounding can seed the partner: ask for 2 nev Ritz pairs and keep
        # the nev lowest distinct values
        want = min(2 * nev, n - 1)
        ev, na, conv = ops.eigs_rs_op(self.ctx, n, apply, x, nev=want, tol=eig_tol, ncv=ncv)
        self.applies += na
        out = []
        for v in sorted(ev):
            if not out or abs(v - out[-1]) > 10 * eig_tol * max(abs(v), 1.0):
                out.append(v)
        return out[:nev], conv and len(out) >= nev


def batched_program_tables(progs, sizes):
    """The tables of P copies of one H_eff program (the programs of P momenta, which must share
    their structure and differ only in their alphas) as one program: every stage holds the P
    copies' output blocks in turn, copy j's regions in every slot but the shared operands (OPS)
    offset by j times the slot's length, its terms carrying momentum j's alphas.  sizes: the
    single program's slot lengths.  Returns (stage_nouts, outs, terms, alphas, slot lengths) for
    imps_plan_program."""
    P = len(progs)
    S = {k: max(int(sizes.get(k, 0)), 1) for k in range(6)}
    tabs = [pg.tables() for pg in progs]
    nouts0, outs0, terms0, _ = tabs[0]
    for (no, ou, te, _) in tabs[1:]:
        if not (np.array_equal(no, nouts0) and np.array_equal(ou, outs0) and np.array_equal(te, terms0)):
            raise ValueError("the momenta's H_eff programs differ in structure (a special momentum?)")
    shift = np.array([0 if k == OPS else S[k] for k in range(6)], np.int64)
    nouts, outs, terms, alphas = [], [], [], []
    o0 = t0 = 0
    for st_n in nouts0:
        so = outs0[o0:o0 + st_n]
        nt = int(so[:, 6].sum())
        stt = terms0[t0:t0 + nt]
        for j in range(P):
            oj = so.copy()
            oj[:, 1] += j * shift[oj[:, 0]]
            tj = stt.copy()
            tj[:, 1] += j * shift[tj[:, 0]]
            tj[:, 5] += j * shift[tj[:, 4]]
            outs.append(oj)
            terms.append(tj)
            alphas.append(tabs[j][3][t0:t0 + nt])
        nouts.append(P * int(st_n))
        o0 += int(st_n)
        t0 += nt
    nouts = np.array(nouts, np.int32)
    outs = np.ascontiguousarray(np.concatenate(outs) if outs else np.zeros((0, 7), np.int64))
    terms = np.ascontiguousarray(np.concatenate(terms) if terms else np.zeros((0, 9), np.int64))
    alphas = np.ascontiguousarray(np.concatenate(alphas) if alphas else np.zeros(0))
    sizes_b = np.array([S[k] if k == OPS else P * S[k] for k in range(6)], np.int64)
    return nouts, outs, terms, alphas, sizes_b


class ExcitationsBatchGPU:
    """Excitation energies at P momenta together (the momentum loop of Excitations_main.cpp:255-297,
    unprojected solves: K != 0 or p != 0).  The H_eff programs of the momenta have the same tables
    and differ only in their alphas, so P copies of each (every slot but the shared operands offset
    per copy) run as one grouped-GEMM launch per stage; the two environment solves of all momenta
    are P GMRES runs in lockstep with the mixed transfer matrix replicated 2P times (one launch per
    stage for every plane of every momentum, imps_invert_e_fac_batch); the eigensolves are P
    Lanczos runs in lockstep (imps_eigs_rs_batch_op), one batched H_eff apply per step."""

    def __init__(self, ctx, AL, AR, NL, HLtot, HRtot, hnnz, d, xdims, kfacs, tol=1e-14, maxit=0, verbose=False):
        import torch
        self.verbose = verbose
        self.torch, self.ctx = torch, ctx
        self.kfacs = [complex(k) for k in kfacs]
        P = self.P = len(self.kfacs)
        self.tol, self.maxit = tol, maxit
        # momentum 0's HeffGPU holds the operands (OPS), the single-plane mixed TM plans and their
        # operand bindings; every momentum's program is compiled for its alphas
        self.H0 = HeffGPU(ctx, AL, AR, NL, HLtot, HRtot, hnnz, d, xdims, self.kfacs[0], tol=tol, maxit=maxit)
        prs = [self.H0.pr] + [HeffProgram(AL, AR, NL, HLtot, HRtot, hnnz, d, xdims, k) for k in self.kfacs[1:]]
        self.pr = pr0 = prs[0]
        self.sizes = S = {k: max(int(pr0.sizes.get(k, 0)), 1) for k in range(6)}
        for pr in prs[1:]:
            if {k: max(int(pr.sizes.get(k, 0)), 1) for k in range(6)} != S:
                raise ValueError("the momenta's H_eff programs differ in their slot sizes")
        self.mtot, self.nr, self.nl = pr0.mtot, pr0.nr, pr0.nl
        if S[XS] != 2 * self.mtot or S[OUT] != 2 * self.mtot:
            raise ValueError("unexpected X layout")
        dev = lambda n: torch.zeros(max(int(n), 1), dtype=torch.float64, device="cuda")
        self.buf = {k: (self.H0.buf[OPS] if k == OPS else dev(P * S[k])) for k in range(6)}
        self.plan_a = self._batched_plan([pr.prog_a for pr in prs])
        self.plan_b = self._batched_plan([pr.prog_b for pr in prs])
        self.rep_r = ops.plan_replicate(self.H0.plan_r, 2 * P)
        self.rep_l = ops.plan_replicate(self.H0.plan_l, 2 * P)
        self.stats = {"gmres_iters": 0, "applies": 0}

    def _batched_plan(self, progs):
        """One imps_plan_program holding P copies of a program (batched_program_tables)."""
        nouts, outs, terms, alphas, sizes = batched_program_tables(progs, self.sizes)
        h = C.c_void_p()
        N.call("imps_plan_program", self.ctx.handle, 6, sizes.ctypes.data_as(N.P_i64), len(nouts),
               nouts.ctypes.data_as(N.P_i32), outs.ctypes.data_as(N.P_i64), terms.ctypes.data_as(N.P_i64),
               alphas.ctypes.data_as(N.P_dbl), C.byref(h))
        plan = B.Plan(self.ctx, h, "program")
        for k in range(6):
            plan.bind(k, self.buf[k])
        return plan

    def apply(self):
        """Y_j = H_eff(p_j) X_j for every momentum (XS -> OUT, copy j at j times the slot length)."""
        P, S = self.P, self.sizes
        self.plan_a.run()
        (off_r, off_ri, nr), (off_l, off_li, nl) = self.pr.rhs_planes()
        rhs, es = self.buf[RHS], self.buf[ES]
        xr_re = [rhs[j * S[RHS] + off_r: j * S[RHS] + off_r + nr] for j in range(P)]
        xr_im = [rhs[j * S[RHS] + off_ri: j * S[RHS] + off_ri + nr] for j in range(P)]
        xl_re = [rhs[j * S[RHS] + off_l: j * S[RHS] + off_l + nl] for j in range(P)]
        xl_im = [rhs[j * S[RHS] + off_li: j * S[RHS] + off_li + nl] for j in range(P)]
        b = lambda j: j * S[ES]
        yr_re = [es[b(j):b(j) + nr] for j in range(P)]
        yr_im = [es[b(j) + nr:b(j) + 2 * nr] for j in range(P)]
        yl_re = [es[b(j) + 2 * nr:b(j) + 2 * nr + nl] for j in range(P)]
        yl_im = [es[b(j) + 2 * nr + nl:b(j) + 2 * nr + 2 * nl] for j in range(P)]
        tol = self.tol
        it, _, cr = ops.InvertE_fac_batch(self.rep_r, xr_re, xr_im, self.kfacs, yr_re, yr_im, tol, self.maxit)
        self.stats["gmres_iters"] += it
        it, _, cl = ops.InvertE_fac_batch(self.rep_l, xl_re, xl_im, [k.conjugate() for k in self.kfacs], yl_re,
                                          yl_im, tol, self.maxit)
        self.stats["gmres_iters"] += it
        self.plan_b.run()
        self.stats["applies"] += 1
        if self.verbose and self.stats["applies"] % 20 == 0:
            import sys
            print(f"[excitations batch] {self.stats['applies']} applies, {self.stats['gmres_iters']} GMRES iterations",
                  file=sys.stderr, flush=True)
        return cr and cl

    def energies(self, nev=4, eig_tol=1e-10, ncv=64, seed=1):
        """The nev lowest energies at every momentum (list of lists) and per-momentum convergence,
        from the real form of each Hermitian H_eff (eigenvalues doubled; 2 nev Ritz pairs kept, the
        nev lowest distinct values returned), every momentum started from the same seeded vector
        as ExcitationsGPU.energies."""
        import torch
        P, n = self.P, 2 * self.mtot
        xs, out = self.buf[XS], self.buf[OUT]

        def apply(pin, pout):
            N.call("imps_axpby", self.ctx.handle, 1.0, C.c_void_p(pin), 0.0, C.c_void_p(xs.data_ptr()), P * n)
            if not self.apply():
                raise RuntimeError("environment solve did not converge")
            N.call("imps_axpby", self.ctx.handle, 1.0, C.c_void_p(out.data_ptr()), 0.0, C.c_void_p(pout), P * n)

        g = torch.Generator(device="cpu").manual_seed(seed)
        x0 = torch.randn(n, generator=g, dtype=torch.float64)
        X = x0.repeat(P).to("cuda")
        want = min(2 * nev, n - 1)
        ev, na, conv = ops.eigs_rs_batch_op(self.ctx, P, n, apply, X, nev=want, tol=eig_tol, ncv=ncv)
        res = []
        for j in range(P):
            vals = []
            for v in sorted(ev[j]):
                if not vals or abs(v - vals[-1]) > 10 * eig_tol * max(abs(v), 1.0):
                    vals.append(v)
            res.append(vals[:nev])
        return res, [c and len(r) >= nev for c, r in zip(conv, res)], na


def save_alrn(v, inp, name, ending="bin", folder="."):
    """saveALRN as the excitation driver writes it (Excitations_main.cpp:232-237): the ground
    state the excitations of ``inp`` (excitation_inputs) are built from, with C[n] the centre
    matrix right of site n, L[n] = C[n]^T C[n] and R[n] = C[n] C[n]^T (formed on the device),
    AL, AR (after the sign fix of AR[0]) and the null spaces NL.  Returns the path written."""
    from . import imps_io
    Cv, Lv, Rv = [], [], []
    for n in range(2):
        b = (n + 1) % 2  # the C right of site n lives on bond n + 1
        Cv.append(bd_to_host(v.C[b], v.LB[b]))
        Lv.append(bd_to_host(v._cct(b, right=False), v.LB[b]))
        Rv.append(bd_to_host(v._cct(b, right=True), v.LB[b]))
    mps = lambda A: imps_io.MPSTensor(v.d, 1, A)
    return imps_io.saveALRN(Cv, Lv, Rv, [mps(a) for a in inp["AL"]], [mps(a) for a in inp["AR"]],
                            [mps(a) for a in inp["NL"]], name, ending, folder)


def measure_excitations(v, K, obs, kfac, seed=1, tol=1e-13):
    """MeasureExcitations (Excitations_helpers.hpp:754-808) on the device.  For each one-site
    observable O: its ground-state mean <O> is subtracted, and the excitation-space operator
    of sum_n (O_n - <O>) is applied to a random normalised X (complex, XDims order, seeded)
    at kfac = e^{ip}; the values tr(X[n]^+ Xout[n]) per site are returned ({name: array}).

    The reference builds OPeffConstants / ApplyOPeff for O; on an infinite chain sum_n O_n is the
    same operator as sum_bonds (O x 1 + 1 x O) / 2, so here H_eff's device programs run with
    that bond operator (minus <O>), whose environments come from excitation_inputs(op=...).
    The two agree in the oracle to rounding (ApplyOPeff against ApplyHeff).  The mean is taken
    from the right-canonical form; the reference averages it with the left-canonical one,
    which agrees to the state's gauge error.  The environment solves are projected at K = 0,
    p = 0 as in Excitations_main.cpp:205-215.  Charge-changing observables give zero (their
    Xout has no block in X's sectors)."""
    d = v.d
    if obs and isinstance(obs[0], str):
        obs = models.observables(v._model, obs, d=d)
    rng = np.random.default_rng(seed)
    p = float(np.angle(kfac))
    out = {}
    xs = None
    for name, O in obs:
        O = np.asarray(O, dtype=np.float64)
        cons = np.array([[tuple(v.I2K[r]) == tuple(v.I2K[c]) for c in range(d)] for r in range(d)])
        if not np.any(O[cons] != 0.0):
            out[name] = np.zeros(2, dtype=complex)
            continue
        if np.any(O[~cons] != 0.0):
            raise NotImplementedError(f"observable {name} mixes charge-conserving and charge-changing entries")
        eobs = float(np.mean(v.measure([(name, O)])[name]))
        hO = 0.5 * (np.kron(O, np.eye(d)) + np.kron(np.eye(d), O)) - eobs * np.eye(d * d)
        inp = excitation_inputs(v, K, tol=tol, op=hO)
        if xs is None:
            sizes = [sum(ml * mr for (_, _, ml, mr) in dd) for dd in inp["xdims"]]
            x = rng.standard_normal(sum(sizes)) + 1j * rng.standard_normal(sum(sizes))
            x /= np.linalg.norm(x)
            xs = np.split(x, np.cumsum(sizes)[:-1])
        proj = all(k == 0 for k in K) and abs(p) < 10 * tol
        H = HeffGPU(v.ctx, inp["AL"], inp["AR"], inp["NL"], inp["HLtot"], inp["HRtot"], inp["h"], d, inp["xdims"],
                    kfac, tol=tol, LM=inp["LM"] if proj else None, RM=inp["RM"] if proj else None)
        H.x_to_planes(xs)
        if not H.apply():
            raise RuntimeError("environment solve did not converge")
        ys = H.y_from_planes()
        out[name] = np.array([np.vdot(xs[n], ys[n]) for n in range(2)])
    return out


# ------------------------------------------------------------------------------------------------
# dominant eigenmatrices of the mixed transfer matrix (EigsBlockFunctions.hpp:282-391,
# Excitations_helpers.hpp:915-946)
# ------------------------------------------------------------------------------------------------

def _rho_vec(lay, M, inside):
    """Vector of the BlockMat M paired block by block with the X layout ``lay``: rho_out blocks have
    X's structure (key qin), rho_in blocks the transposed one (key qout)."""
    parts = []
    for (_, qi, qo, r, c) in _blocks(lay):
        key, other, shape = (qo, qi, (c, r)) if inside else (qi, qo, (r, c))
        if key not in M or tuple(M[key][0]) != other or M[key][1].shape != shape:
            raise ValueError("LM/RM sectors do not match the environment structure")
        parts.append(np.asarray(M[key][1], np.float64).reshape(-1, order="F"))
    return np.concatenate(parts) if parts else np.zeros(0)


def _mps_layout(A, nsym):
    return B.Layout([(s, tuple(qi), tuple(bm[qi][0]), bm[qi][1].shape[0], bm[qi][1].shape[1])
                     for s, bm in enumerate(A) for qi in sorted(bm)], nsym)


def _mps_vec(A):
    return np.concatenate([np.asarray(bm[qi][1], np.float64).reshape(-1, order="F") for bm in A for qi in sorted(bm)])


def _mps_ml(A):
    out = {}
    for bm in A:
        for qi, (qo, M) in bm.items():
            out.setdefault(tuple(qi), M.shape[0])
    return out


def tm_mixed_eigs(ctx, A, Bm, direction, K, nev, mode="LM", tol=1e-14, ncv=0, periods=None):
    """TMmixedEigs(A, B, V, dir, K, nev, mode, tol) (EigsBlockFunctions.hpp:282-391) on the device:
    the nev leading eigenpairs of the mixed unit-cell TM (ApplyTMmixedLeft/Right(A, B, X) over
    the sites) in the charge sector K, by the device Arnoldi (imps_eigs_n) on a mixed-TM plan.
    Sectors (q, q + K) for q in GetMl of A (dir r) or of B (dir l).  A, B: lists over sites of
    host MPS tensors.  Returns (complex eigenvalues sorted by |lambda| (LM) or Re lambda (LR)
    descending, the eigenvectors as complex BlockMats, the sector sizes, applies, converged)."""
    import torch
    if mode not in ("LM", "LR"):
        raise ValueError("TMmixedEigs: wrong mode " + mode)
    K = tuple(int(k) for k in K)
    nsym = len(K)
    diml, dimr = _mps_ml(A[0]), _mps_ml(Bm[0])
    if direction == "l":
        diml, dimr = dimr, diml
    kk = (lambda q: charges.add(q, K, periods)) if periods else (lambda q: _kadd(q, K))
    sizes = [(q, kk(q), diml[q], dimr[kk(q)]) for q in sorted(diml) if kk(q) in dimr]
    if not sizes:
        raise ValueError("TMmixedEigs: no TM eigenvalues for this quantum number")
    lay = B.Layout([(0, qi, qo, ml, mr) for (qi, qo, ml, mr) in sizes], nsym)
    lay_a, lay_b = [_mps_layout(a, nsym) for a in A], [_mps_layout(b, nsym) for b in Bm]
    plan = B.plan_tm_mixed(ctx, lay_a, lay_b, 0 if direction == "l" else 1, lay, lay)
    tdev = lambda v: torch.from_numpy(v).to("cuda")
    ops_a, ops_b = [tdev(_mps_vec(a)) for a in A], [tdev(_mps_vec(b)) for b in Bm]
    ns = len(A)
    for k in range(ns):
        plan.bind(2 + k, ops_a[k])
        plan.bind(2 + ns + k, ops_b[k])
    n = lay.nelem
    ere = torch.zeros((nev, n), dtype=torch.float64, device="cuda")
    eim = torch.zeros((nev, n), dtype=torch.float64, device="cuda")
    vals, na, conv = ops.eigs_n(plan, nev, mode, tol, ncv=ncv, evecs_re=ere, evecs_im=eim)
    vr, vi = ere.cpu().numpy(), eim.cpu().numpy()
    V = []
    for i in range(nev):
        v = vr[i] + 1j * vi[i]
        X, pos = {}, 0
        for (qi, qo, ml, mr) in sizes:
            X[qi] = (qo, v[pos:pos + ml * mr].reshape(mr, ml).T.copy())
            pos += ml * mr
        V.append(X)
    return vals, V, sizes, na, conv


def LRoverlaps(ctx, AL, AR, K, nev, OLtol=1e-14, periods=None):
    """LRoverlaps(LM, RM, AL, AR, K, nev, OLtol) (Excitations_helpers.hpp:915-946) on the device:
    the dominant left (sector -K) and right (sector K) eigenmatrices of the mixed TM of AL and
    AR, as real BlockMats, and the overlap OL = (Re OL_L + Re OL_R) / 2.  Returns
    (LM, RM, OL, OL_L eigenvalues, OL_R eigenvalues, converged)."""
    K = tuple(int(k) for k in K)
    mK = charges.neg(K, periods) if periods else tuple(-k for k in K)
    vl, VL, _, _, cl = tm_mixed_eigs(ctx, AL, AR, "l", mK, nev, "LM", OLtol, periods=periods)
    vr, VR, _, _, cr = tm_mixed_eigs(ctx, AL, AR, "r", K, nev, "LM", OLtol, periods=periods)
    real = lambda X: {qi: (qo, np.real(M).copy()) for qi, (qo, M) in X.items()}
    return real(VL[0]), real(VR[0]), 0.5 * (vl[0].real + vr[0].real), vl, vr, cl and cr


# ------------------------------------------------------------------------------------------------
# inputs of the excitation ansatz from a converged two-site VUMPS state on the device
# ------------------------------------------------------------------------------------------------

def _blocks(layout):
    return [(g, tuple(qi), tuple(qo), r, c) for (g, qi, qo, r, c) in layout.blocks]


def mps_to_host(vec, layout, d):
    """Device vector in an MPS layout -> list over s of {qin: (qout, matrix)}."""
    v = vec.detach().cpu().numpy()
    out, pos = [dict() for _ in range(d)], 0
    for (g, qi, qo, r, c) in _blocks(layout):
        out[g][qi] = (qo, v[pos:pos + r * c].reshape(c, r).T.copy())
        pos += r * c
    return out


def bd_to_host(vec, layout):
    v = vec.detach().cpu().numpy()
    out, pos = {}, 0
    for (g, qi, qo, r, c) in _blocks(layout):
        out[qi] = v[pos:pos + r * c].reshape(c, r).T.copy()
        pos += r * c
    return out


def xdims_from_layouts(ns_layout, ar_layout, K, periods=None):
    """XDims (Excitations_helpers.hpp:641-678): X_n maps the right sectors q of N_L[n] to the
    left sectors q + K of AR[n+1]."""
    ml, mr = {}, {}
    for (g, qi, qo, r, c) in _blocks(ns_layout):
        ml.setdefault(qo, c)
    for (g, qi, qo, r, c) in _blocks(ar_layout):
        mr.setdefault(qi, r)
    dims = []
    for q in sorted(ml):
        qk = charges.add(q, K, periods) if periods else _kadd(q, K)
        if qk in mr and ml[q] > 0 and mr[qk] > 0:
            dims.append((q, qk, ml[q], mr[qk]))
    return dims


def excitation_inputs(v, K, tol=1e-13, op=None):
    """AL, AR, N_L, HLtot, HRtot (HeffConstants, Excitations_helpers.hpp:258-331), h - E0 and
    XDims for charge K, from a converged VumpsGPU state (sites n: bond n -> n + 1; C[b] on bond
    b), every contraction and solve on the device; host copies as map-of-blocks structures.
    op: another two-site operator (d^2 x d^2, its mean already subtracted) in place of h - E0."""
    from . import ops as _ops
    from . import models as _models
    ctx, d, torch = v.ctx, v.d, v.torch
    AL, AR = v.AL, v.AR
    eye0 = v._eye(0)
    if op is None:
        E0 = float(np.mean(v.energy()))
        optl, optr, onnz = v.optm_l, v.optm_r, v.hnnz
    else:
        E0 = 0.0
        onnz = _models.h_nonzeros(np.asarray(op, dtype=np.float64))
        optl = [B.plan_optm(ctx, v.LA[a], v.LA[1 - a], d, onnz, 0, v.LB[a]) for a in range(2)]
        optr = [B.plan_optm(ctx, v.LA[a], v.LA[1 - a], d, onnz, 1, v.LB[a]) for a in range(2)]

    def optm(plans, a, A, b):
        p = plans[a]
        out = v._z(v.LB[b])
        p.bind(0, A[a]); p.bind(1, A[1 - a]); p.bind(2, out); p.run()
        return out

    # left: HL[0] = OpTM(AL1 AL0) on bond 1, HL[1] = OpTM(AL0 AL1) + T_L(AL1, HL[0]) on bond 0
    HL0 = optm(optl, 1, AL, 1)
    HL1 = _ops.axpby(ctx, 1.0, optm(optl, 0, AL, 0), 1.0, v._tm(("L1", 1), AL, HL0, v._z(v.LB[0])))
    R0 = v._tm_dominant(("R", 0), AL, v._cct(0, right=True), 1e-15)
    EHL1 = v._invert_e(("L", 0), AL, HL1, eye0, R0, "l", None, tol)
    EHL0 = v._tm(("L1", 0), AL, EHL1, v._z(v.LB[1]))
    # right: HR[1] = OpTM(AR1 AR0) on bond 1, HR[0] = OpTM(AR0 AR1) + T_R(AR0, HR[1]) on bond 0
    HR1 = optm(optr, 1, AR, 1)
    HR0 = _ops.axpby(ctx, 1.0, optm(optr, 0, AR, 0), 1.0, v._tm(("R1", 0), AR, HR1, v._z(v.LB[0])))
    L0 = v._tm_dominant(("L", 0), AR, v._cct(0, right=False), 1e-15)
    EHR0 = v._invert_e(("R", 0), AR, HR0, L0, eye0, "r", None, tol)
    EHR1 = v._tm(("R1", 1), AR, EHR0, v._z(v.LB[1]))
    # h - E0: for isometric tensors OpTM(h - E0) = OpTM(h) - E0 1 along each chain
    eye1 = v._eye(1)
    HLtot = [_ops.axpby(ctx, 1.0, EHL0, 1.0, _ops.axpby(ctx, -E0, eye1, 1.0, HL0.clone())), EHL1]
    HRtot = [EHR0, _ops.axpby(ctx, 1.0, EHR1, 1.0, _ops.axpby(ctx, -E0, eye1, 1.0, HR1.clone()))]
    # N_L on the device
    NL, nsl = [], []
    for n in range(2):
        plan = v.dec_ac_l[n]
        out = torch.zeros(max(plan.nslayout.nelem, 1), dtype=torch.float64, device="cuda")
        _ops.Nullspace(plan, AL[n], out)
        NL.append(mps_to_host(out, plan.nslayout, d))
        nsl.append(plan.nslayout)
    if op is None:
        hs = [(r, c, val - (E0 if r == c else 0.0)) for (r, c, val) in v.hnnz]
        diag = {r for (r, c, _) in v.hnnz if r == c}
        hs += [(i, i, -E0) for i in range(d * d) if i not in diag]
        hs.sort(key=lambda t: (t[1], t[0]))
    else:
        hs = list(onnz)
    per = charges.periods_of(v.I2K)
    xd = [xdims_from_layouts(nsl[n], v.LA[(n + 1) % 2], tuple(K), per) for n in range(2)]
    ALh = [mps_to_host(AL[n], v.LA[n], d) for n in range(2)]
    ARh = [mps_to_host(AR[n], v.LA[n], d) for n in range(2)]
    # overlap of AL and AR and the dominant mixed-TM eigenmatrices (Excitations_main.cpp:174-178);
    # AR[0] *= sign(OL) makes the overlap positive (it leaves HRtot unchanged)
    LM, RM, OL, _, _, _ = LRoverlaps(ctx, ALh, ARh, K, 2, 1e-14, periods=per)
    if OL < 0:
        ARh[0] = [{qi: (qo, -M) for qi, (qo, M) in bm.items()} for bm in ARh[0]]
    host = dict(AL=ALh, AR=ARh, NL=NL,
                HLtot=[bd_to_host(HLtot[0], v.LB[1]), bd_to_host(HLtot[1], v.LB[0])],
                HRtot=[bd_to_host(HRtot[0], v.LB[0]), bd_to_host(HRtot[1], v.LB[1])],
                h=hs, d=d, xdims=xd, E0=E0, LM=LM, RM=RM, OL=OL)
    return host

