"""ExpandFromH on the device: bond-dimension growth of VUMPS (MPSBlockUtilities.hpp:409-601,
called at VUMPS_main.cpp:277-308).

The bond between AL (left bond -> centre bond) and AR (centre bond -> right bond) grows by
the dominant directions of H acting on the two-site tensor AL C AR outside the current
tangent space.  In per-charge dense form, for every centre charge c:

    Phi[c]  rows (sl, ql = c - I2K[sl]) in increasing sl, columns (sr, qr = c + I2K[sr]) in
            increasing sr (GetDenseSplitMat, MPSBlockMat.hpp:533-565), block
            Phi[(sl,ql),(sr,qr)] = sum_{s1,s2} h[(sl sr),(s1 s2)] (AL C)_{s1}[ql] AR_{s2}[q1]
    M[c]    = NL[c]^T Phi[c] NR[c]^T for a charge already on the bond (NL, NR the orthonormal
            complements of the stacked AL / AR sector matrices; skipped if either is empty),
            Phi[c] itself for a new charge.

Device work, all through the C ABI: AL C by an MPS x BlockDiag plan, the null spaces by the
per-sector Householder complement (imps_sector_nullspace; NR as the complement of the
transposed AR), Phi and M by one grouped-GEMM program (imps_plan_program, three stages), the
SVD of every M[c] by the per-sector Jacobi SVD (each M[c] stored in its tall orientation), and
the new tensors by a second program: new columns NL U of AL, new rows V^T NR of AR, U and V^T
themselves for a new charge, written into the grown layouts next to the old blocks, which
identity products copy over; C is padded with zeros, so AL C AR is unchanged.  The host keeps
the integer bookkeeping and the global choice of the dmmax largest singular values
(std::sort in the reference, whose order for equal values is unspecified; here equal values
keep charge order).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from . import blocks as B
from . import charges, ops


class _Program:
    """Tables of a grouped-GEMM program: stages of output blocks (slot, off, ld, M, N) with
    their terms (a_slot, a_off, a_ld, a_trans, b_slot, b_off, b_ld, b_trans, k, alpha)."""

    def __init__(self):
        self.stages = []

    def stage(self):
        self.stages.append([])
        return self.stages[-1]

    def run(self, ctx, bufs):
        torch = __import__("torch")
        stages = [st for st in self.stages if st]
        if not stages:
            return
        nouts = np.array([len(st) for st in stages], np.int32)
        outs, terms, alphas = [], [], []
        for st in stages:
            for (cs, coff, cld, M, Nn, tl) in st:
                outs.append((cs, coff, max(cld, 1), M, Nn, 0, len(tl)))
                for t in tl:
                    terms.append(t[:9])
                    alphas.append(t[9])
        outs = np.array(outs, np.int64).reshape(-1, 7)
        terms = np.array(terms, np.int64).reshape(-1, 9)
        alphas = np.array(alphas, np.float64)
        sizes = np.array([max(int(b.numel()), 1) for b in bufs], np.int64)
        h = C.c_void_p()
        N.call("imps_plan_program", ctx.handle, len(bufs), sizes.ctypes.data_as(N.P_i64), len(nouts),
               nouts.ctypes.data_as(N.P_i32), outs.ctypes.data_as(N.P_i64), terms.ctypes.data_as(N.P_i64),
               alphas.ctypes.data_as(N.P_dbl), C.byref(h))
        plan = B.Plan(ctx, h, "program")
        for k, b in enumerate(bufs):
            plan.bind(k, b if b.numel() else torch.zeros(1, dtype=torch.float64, device="cuda"))
        plan.run()


def _zeros(n):
    torch = __import__("torch")
    return torch.zeros(max(int(n), 1), dtype=torch.float64, device="cuda")


def _eye(n):
    torch = __import__("torch")
    return torch.eye(max(int(n), 1), dtype=torch.float64, device="cuda").reshape(-1)


def relayout(ctx, old, new, x):
    """x (layout ``old``) copied into a zero tensor of layout ``new``: every block of ``old``
    into the top-left corner of the block of ``new`` with the same physical index and
    incoming charge (which must be at least as large); blocks only in ``new`` stay zero."""
    out = _zeros(new.nelem)
    if old.nelem == 0:
        return out
    maxr = max(r for (_, _, _, r, _) in old.blocks)
    eye = _eye(maxr)
    prog = _Program()
    st = prog.stage()
    for (g, qi, qo, r, c), off in zip(old.blocks, old.offsets):
        if r == 0 or c == 0:
            continue
        i = new.find(g, qi)
        if i < 0:
            raise ValueError(f"block ({g}, {qi}) missing in the new layout")
        _, _, qo2, r2, c2 = new.blocks[i]
        if tuple(qo2) != tuple(qo) or r2 < r or c2 < c:
            raise ValueError(f"block ({g}, {qi}) shrinks or changes its outgoing charge")
        st.append((2, new.offsets[i], r2, r, c, [(0, 0, maxr, 0, 1, off, r, 0, r, 1.0)]))
    prog.run(ctx, [eye, x, out])
    return out


def expand_from_h(ctx, I2K, hnnz, LA, AL, LR, AR, LC, Cc, dmmax):
    """ExpandFromH(H, I2K, AL, AR, C, dmmax) on device tensors in the layouts LA (AL: left bond
    -> centre bond), LR (AR: centre bond -> right bond) and LC (C on the centre bond).

    Returns a dict with ``dm`` ({charge: states added} for every charge considered), ``dims``
    (the grown centre bond), the new layouts ``LA``, ``LR``, ``LC`` and the new tensors ``AL``,
    ``AR``, ``C`` (device, in those layouts), and ``converged`` (the sector SVD's flag)."""
    d = len(I2K)
    dl, dc, dR = LA.dims(0), LC.dims(0), LR.dims(1)
    # AL C, and the null spaces of AL (dir l) and of AR (as the dir-l complement of AR^T)
    p_x = B.plan_mps_bd(ctx, LA, LC, 1)
    X = _zeros(LA.nelem)
    p_x.bind(0, AL); p_x.bind(1, Cc); p_x.bind(2, X); p_x.run()
    dec_l = B.plan_decomp(ctx, LA, "l")
    NL = _zeros(dec_l.nslayout.nelem)
    ops.Nullspace(dec_l, AL, NL)
    per = charges.periods_of(I2K)
    _kadd = lambda a, b: charges.add(a, b, per)
    _ksub = lambda a, b: charges.sub(a, b, per)
    LT = B.Layout.mps(charges.negated(I2K), dR, dc)
    ART = _zeros(LT.nelem)
    for (s, qc, qr, mc, mqr), off in zip(LR.blocks, LR.offsets):
        i = LT.find(s, qr)
        if i < 0:
            raise ValueError(f"AR block ({s}, {qc}) has no transposed counterpart")
        o2 = LT.offsets[i]
        ART[o2:o2 + mc * mqr].view(mc, mqr).copy_(AR[off:off + mc * mqr].view(mqr, mc).t())
    dec_t = B.plan_decomp(ctx, LT, "l")
    NRt = _zeros(dec_t.nslayout.nelem)
    ops.Nullspace(dec_t, ART, NRt)
    nl_off = {(b[0], b[1]): (o, b[4]) for b, o in zip(dec_l.nslayout.blocks, dec_l.nslayout.offsets)}
    nr_off = {(b[0], b[1]): (o, b[4]) for b, o in zip(dec_t.nslayout.blocks, dec_t.nslayout.offsets)}
    la_off = {(b[0], b[1]): o for b, o in zip(LA.blocks, LA.offsets)}
    lr_off = {(b[0], b[1]): o for b, o in zip(LR.blocks, LR.offsets)}

    # sector bookkeeping: rows (sl, ql) and columns (sr, qr) of Phi[c], and its terms
    cands = sorted({_kadd(ql, I2K[s]) for s in range(d) for ql in dl})
    secs = {}
    for c in cands:
        rows, r0 = [], 0
        for sl in range(d):
            ql = _ksub(c, I2K[sl])
            if ql in dl:
                rows.append((sl, ql, r0, dl[ql]))
                r0 += dl[ql]
        cols, c0 = [], 0
        for sr in range(d):
            qr = _kadd(c, I2K[sr])
            if qr in dR:
                cols.append((sr, qr, c0, dR[qr]))
                c0 += dR[qr]
        blocks = []
        for (sl, ql, ra, mr) in rows:
            for (sr, qr, ca, mc) in cols:
                tl = []
                for (hr, hc, hv) in hnnz:
                    if hr != sl * d + sr:
                        continue
                    s1, s2 = divmod(hc, d)
                    q1 = _kadd(ql, I2K[s1])
                    if q1 not in dc or _kadd(q1, I2K[s2]) != qr:
                        continue
                    tl.append((la_off[(s1, ql)], lr_off[(s2, q1)], dc[q1], hv))
                if tl:
                    blocks.append((ra, mr, ca, mc, tl))
        if not blocks:
            continue  # H creates nothing at this charge
        e = {"rows": rows, "cols": cols, "m": r0, "n": c0, "blocks": blocks, "new": c not in dc}
        if e["new"]:
            e["tr"] = r0 < c0
            e["shape"] = (max(r0, c0), min(r0, c0))
        else:
            nul_l, nul_r = r0 - dc[c], c0 - dc[c]
            if nul_l <= 0 or nul_r <= 0:
                continue  # already full rank on one side
            e["nul"] = (nul_l, nul_r)
            e["tr"] = nul_l < nul_r
            e["shape"] = (max(nul_l, nul_r), min(nul_l, nul_r))
        secs[c] = e
    if not secs:
        return None
    keys = sorted(secs)
    LM = B.Layout([(0, c, c, secs[c]["shape"][0], secs[c]["shape"][1]) for c in keys], LA.nsym)
    mt_off = dict(zip(keys, LM.offsets))
    phi_off, t_off, nphi, nt = {}, {}, 0, 0
    for c in keys:
        e = secs[c]
        if not e["new"]:
            phi_off[c] = nphi
            nphi += e["m"] * e["n"]
            t_off[c] = nt
            nt += e["nul"][0] * e["n"]
    PHI, T, MT = _zeros(nphi), _zeros(nt), _zeros(LM.nelem)
    # program 1, slots: 0 X, 1 AR, 2 NL, 3 NRt, 4 PHI, 5 T, 6 MT
    SX, SAR, SNL, SNR, SPHI, ST, SMT = range(7)
    prog = _Program()
    s_phi, s_t, s_m = prog.stage(), prog.stage(), prog.stage()
    for c in keys:
        e = secs[c]
        for (ra, mr, ca, mc, tl) in e["blocks"]:
            if not e["new"]:
                ld = e["m"]
                s_phi.append((SPHI, phi_off[c] + ca * ld + ra, ld, mr, mc,
                              [(SX, xo, mr, 0, SAR, ao, k, 0, k, hv) for (xo, ao, k, hv) in tl]))
            elif not e["tr"]:
                ld = e["m"]
                s_phi.append((SMT, mt_off[c] + ca * ld + ra, ld, mr, mc,
                              [(SX, xo, mr, 0, SAR, ao, k, 0, k, hv) for (xo, ao, k, hv) in tl]))
            else:  # Phi^T block (mc x mr) = sum h AR^T X^T
                ld = e["n"]
                s_phi.append((SMT, mt_off[c] + ra * ld + ca, ld, mc, mr,
                              [(SAR, ao, k, 1, SX, xo, mr, 1, k, hv) for (xo, ao, k, hv) in tl]))
        if e["new"]:
            continue
        nul_l, nul_r = e["nul"]
        # T = NL^T Phi  (nul_l x n)
        tl = []
        for (sl, ql, ra, mr) in e["rows"]:
            o, _ = nl_off[(sl, ql)]
            tl.append((SNL, o, mr, 1, SPHI, phi_off[c] + ra, e["m"], 0, mr, 1.0))
        s_t.append((ST, t_off[c], nul_l, nul_l, e["n"], tl))
        # M = T NR^T (nul_l x nul_r), or M^T = NR T^T when nul_l < nul_r
        tl = []
        for (sr, qr, ca, mc) in e["cols"]:
            o, _ = nr_off[(sr, qr)]
            if not e["tr"]:
                tl.append((ST, t_off[c] + ca * nul_l, nul_l, 0, SNR, o, mc, 0, mc, 1.0))
            else:
                tl.append((SNR, o, mc, 1, ST, t_off[c] + ca * nul_l, nul_l, 1, mc, 1.0))
        if not e["tr"]:
            s_m.append((SMT, mt_off[c], nul_l, nul_l, nul_r, tl))
        else:
            s_m.append((SMT, mt_off[c], nul_r, nul_r, nul_l, tl))
    prog.run(ctx, [X, AR, NL, NRt, PHI, T, MT])

    # SVD of every M[c] (tall orientation), and the global choice of the largest values
    dec_m = B.plan_decomp(ctx, LM, "l")
    U, S, V = _zeros(LM.nelem), _zeros(dec_m.nsv), _zeros(dec_m.rlayout.nelem)
    conv = ops.svd(dec_m, MT, U, S, V)
    Sh = S.cpu().numpy()[:dec_m.nsv]
    v_off = dict(zip(keys, dec_m.rlayout.offsets))
    lam, o = {}, 0
    for c in keys:
        k = secs[c]["shape"][1]
        lam[c] = Sh[o:o + k]
        o += k
    dmtot = sum(len(v) for v in lam.values())
    dm = {c: 0 for c in keys}
    if dmtot > dmmax:
        allv = [(-float(x), i, c) for i, c in enumerate(keys) for x in lam[c]]
        for (_, _, c) in sorted(allv, key=lambda t: (t[0], t[1]))[:max(dmmax, 0)]:
            dm[c] += 1
    else:
        dm = {c: len(lam[c]) for c in keys}

    # grown layouts; old blocks copied over, then the new columns / rows
    dcn = dict(dc)
    for c, k in dm.items():
        if k:
            dcn[c] = dcn.get(c, 0) + k
    LAn = B.Layout.mps(I2K, dl, dcn)
    LRn = B.Layout.mps(I2K, dcn, dR)
    LCn = B.Layout.blockdiag(dcn)
    ALn = relayout(ctx, LA, LAn, AL)
    ARn = relayout(ctx, LR, LRn, AR)
    Cn = relayout(ctx, LC, LCn, Cc)
    maxe = max([m for m in dl.values()] + [m for m in dR.values()] + [1])
    eye = _eye(maxe)
    # program 2, slots: 0 NL, 1 NRt, 2 U, 3 V, 4 EYE, 5 AL', 6 AR'
    SNL, SNR, SU, SV, SE, SAL, SARn = range(7)
    prog = _Program()
    st = prog.stage()
    ial = {(b[0], b[1]): (o, b[3], b[4]) for b, o in zip(LAn.blocks, LAn.offsets)}
    iar = {(b[0], b[1]): (o, b[3], b[4]) for b, o in zip(LRn.blocks, LRn.offsets)}
    def opnd(Y, i0, want_t):
        """Rows i0.. of the singular-vector matrix Y (first k columns used) as a GEMM operand:
        op = Y[i0:, :k] (want_t False) or its transpose.  Y = (slot, off, ld, stored_t); the
        SVD writes U as is and V transposed (imps_sector_svd, dir l: the reference's DiagIso)."""
        slot, off, ld, stored_t = Y
        if not stored_t:
            return (slot, off + i0, ld, 1 if want_t else 0)
        return (slot, off + i0 * ld, ld, 0 if want_t else 1)

    for c in keys:
        k = dm[c]
        if k == 0:
            continue
        e = secs[c]
        rt, ct = e["shape"]
        # U_M, V_M: left and right singular vectors of M (of the stored M^T swapped)
        u_st, v_st = (SU, mt_off[c], rt, False), (SV, v_off[c], ct, True)
        um, vm = (u_st, v_st) if not e["tr"] else (v_st, u_st)
        m0 = dc.get(c, 0)
        if not e["new"]:
            nul_l, nul_r = e["nul"]
            for (sl, ql, ra, mr) in e["rows"]:
                o, _ = nl_off[(sl, ql)]
                ob, rr, cc = ial[(sl, ql)]
                st.append((SAL, ob + m0 * rr, rr, rr, k, [(SNL, o, mr, 0) + opnd(um, 0, False) + (nul_l, 1.0)]))
            for (sr, qr, ca, mc) in e["cols"]:
                o, _ = nr_off[(sr, qr)]
                ob, rr, cc = iar[(sr, c)]
                st.append((SARn, ob + m0, rr, k, cc, [opnd(vm, 0, True) + (SNR, o, mc, 1, nul_r, 1.0)]))
        else:
            for (sl, ql, ra, mr) in e["rows"]:
                ob, rr, cc = ial[(sl, ql)]
                st.append((SAL, ob, rr, rr, k, [(SE, 0, maxe, 0) + opnd(um, ra, False) + (mr, 1.0)]))
            for (sr, qr, ca, mc) in e["cols"]:
                ob, rr, cc = iar[(sr, c)]
                st.append((SARn, ob, rr, k, cc, [opnd(vm, ca, True) + (SE, 0, maxe, 0, mc, 1.0)]))
    prog.run(ctx, [NL, NRt, U, V, eye, ALn, ARn])
    return {"dm": dm, "dims": dcn, "LA": LAn, "LR": LRn, "LC": LCn, "AL": ALn, "AR": ARn, "C": Cn,
            "converged": conv, "lam": lam}
