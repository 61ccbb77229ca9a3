"""Host-side mirror of the reference's block-sparse types for the GB300 path.

The reference keeps every block-sparse object as a ``std::map`` of dense armadillo blocks
(BlockObj.hpp:506-600 BlockMat, 1360-1467 BlockDiagMat; MPSBlockMat.hpp:41-175).  Here an
object is a *layout* (its sector table, held natively as an ``imps_layout``) plus one flat
device buffer in the reference's Vectorize order, so that the same vector can be handed to
ARPACK-style callers unchanged.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _keys_array(keys, nsym):
    a = np.asarray(keys, dtype=np.int32).reshape(-1, nsym) if len(keys) else np.zeros((0, nsym), np.int32)
    return np.ascontiguousarray(a)


def _ptr32(a):
    return a.ctypes.data_as(N.P_i32)


class Layout:
    """Sector table of one block-sparse object (GetSizesVector order).

    blocks: list of (group, qin, qout, rows, cols); group = physical index for MPS tensors,
    i*d+j for a RedOp grid, 0 otherwise.
    """

    def __init__(self, blocks, nsym, _handle=None):
        self.nsym = nsym
        self.blocks = [(int(g), tuple(qi), tuple(qo), int(r), int(c)) for (g, qi, qo, r, c) in blocks]
        offs, o = [], 0
        for (_, _, _, r, c) in self.blocks:
            offs.append(o)
            o += r * c
        self.offsets = offs
        self.nelem = o
        if _handle is not None:
            self._h = _handle
        else:
            n = len(self.blocks)
            qin = _keys_array([b[1] for b in self.blocks], nsym)
            qout = _keys_array([b[2] for b in self.blocks], nsym)
            rows = np.array([b[3] for b in self.blocks], np.int32)
            cols = np.array([b[4] for b in self.blocks], np.int32)
            grp = np.array([b[0] for b in self.blocks], np.int32)
            h = C.c_void_p()
            N.call("imps_layout_create", nsym, n, _ptr32(qin), _ptr32(qout), _ptr32(rows), _ptr32(cols),
                   _ptr32(grp), C.byref(h))
            self._h = h
        self._index = {(b[0], b[1]): i for i, b in enumerate(self.blocks)}

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and N._lib is not None:
            N._lib.imps_layout_destroy(h)
            self._h = None

    # --- constructors mirroring the reference ---
    @classmethod
    def blockdiag(cls, dims):
        """BlockDiagMat with sectors dims = {key: m} (std::map order)."""
        keys = sorted(dims)
        nsym = len(keys[0]) if keys else 1
        return cls([(0, k, k, dims[k], dims[k]) for k in keys], nsym)

    @classmethod
    def mps(cls, I2K, dl, dr):
        """MPSBlockMat(I2K, ml, mr) sector structure (MPSBlockMat.hpp:221-236)."""
        from . import charges
        per = charges.periods_of(I2K)
        blocks = []
        for s, sh in enumerate(I2K):
            for ql in sorted(dl):
                qr = charges.add(ql, sh, per)
                if qr in dr:
                    blocks.append((s, ql, qr, dl[ql], dr[qr]))
        return cls(blocks, len(I2K[0]))

    @classmethod
    def from_native(cls, h):
        n = N.load().imps_layout_nblocks(h)
        nsym = N.load().imps_layout_nsym(h)
        qin = np.zeros((max(n, 1), nsym), np.int32)
        qout = np.zeros((max(n, 1), nsym), np.int32)
        rows = np.zeros(max(n, 1), np.int32)
        cols = np.zeros(max(n, 1), np.int32)
        grp = np.zeros(max(n, 1), np.int32)
        N.call("imps_layout_get", h, _ptr32(qin), _ptr32(qout), _ptr32(rows), _ptr32(cols), _ptr32(grp), None)
        blocks = [(int(grp[i]), tuple(int(x) for x in qin[i]), tuple(int(x) for x in qout[i]), int(rows[i]),
                   int(cols[i])) for i in range(n)]
        return cls(blocks, nsym, _handle=h)

    def bond(self, side):
        """GetMl (side 0) / GetMr (side 1) as a BlockDiagMat layout."""
        h = C.c_void_p()
        N.call("imps_layout_bond", self._h, side, C.byref(h))
        return Layout.from_native(h)

    def dims(self, side=0):
        out = {}
        for (_, qi, qo, r, c) in self.blocks:
            if side == 0:
                out.setdefault(qi, r)
            else:
                out.setdefault(qo, c)
        return out

    def find(self, group, qin):
        return self._index.get((group, tuple(qin)), -1)

    def sizes(self):
        return [(b[1], b[2], b[3], b[4]) for b in self.blocks]

    def __len__(self):
        return len(self.blocks)


class Context:
    """One device + one CUDA stream (imps_ctx).  device=-1 builds tables only (no GPU)."""

    def __init__(self, device=0, stream=None):
        h = C.c_void_p()
        N.call("imps_ctx_create", int(device), C.byref(h))
        self._h = h
        self.device = device
        if stream is not None:
            self.set_stream(stream)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream):
        """Use a torch.cuda.Stream / raw cudaStream_t for every launch of this context."""
        raw = getattr(stream, "cuda_stream", stream)
        N.call("imps_ctx_set_stream", self._h, C.c_void_p(raw))

    def synchronize(self):
        N.call("imps_ctx_synchronize", self._h)

    def close(self):
        if getattr(self, "_h", None) is not None and N._lib is not None:
            N._lib.imps_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def _dptr(t):
    """Device pointer of a contiguous float64 CUDA tensor."""
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise TypeError("expected a contiguous float64 CUDA tensor")
    return C.c_void_p(t.data_ptr())


class Plan:
    """A compiled contraction (imps_plan)."""

    def __init__(self, ctx, h, kind=""):
        self.ctx = ctx
        self._h = h
        self.kind = kind
        self._bound = {}

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and N._lib is not None:
            N._lib.imps_plan_destroy(h)
            self._h = None

    def info(self):
        fa, fp, dr = C.c_int64(), C.c_int64(), C.c_int64()
        ns, nst = C.c_int(), C.c_int()
        N.call("imps_plan_info", self._h, C.byref(fa), C.byref(fp), C.byref(dr), C.byref(ns), C.byref(nst))
        return {"flops_apply": fa.value, "flops_prep": fp.value, "dropped": dr.value, "nslots": ns.value,
                "nstages": nst.value}

    def slot_nelem(self, slot):
        k, n = C.c_int(), C.c_int64()
        N.call("imps_plan_slot_info", self._h, slot, C.byref(k), C.byref(n))
        return n.value

    def derived(self, which):
        h = C.c_void_p()
        N.call("imps_plan_derived_layout", self._h, which, C.byref(h))
        return Layout.from_native(h)

    def bind(self, slot, tensor):
        N.call("imps_plan_bind", self._h, slot, _dptr(tensor))
        self._bound[slot] = tensor  # keep alive

    def prepare(self):
        N.call("imps_plan_prepare", self._h)

    def run(self):
        N.call("imps_plan_run", self._h)

    def set_precision(self, prec):
        N.call("imps_plan_set_precision", self._h, int(prec))

    def autotune(self, reps=5):
        """Time the FP64 launch shapes of every apply stage not yet tuned in this process and
        install the fastest (imps_plan_autotune; on stand-in buffers, nothing needs to be
        bound).  Returns the number of stages timed."""
        n = C.c_int()
        N.call("imps_plan_autotune", self._h, int(reps), C.byref(n))
        return n.value

    def stage_shape(self, stage=0):
        """(tile, splits, histogram key) of an apply stage."""
        t, sp, k = C.c_int(), C.c_int(), C.c_uint64()
        N.call("imps_plan_stage_shape", self._h, int(stage), C.byref(t), C.byref(sp), C.byref(k))
        return t.value, sp.value, k.value

    def table(self, stage=0, prep=False):
        """Sector-matching table of one stage: list over output blocks of
        (tag, [(a_slot, a_off, b_slot, b_off, k, alpha), ...])."""
        no, nt = C.c_int64(), C.c_int64()
        nul = None
        N.call("imps_plan_table", self._h, int(prep), stage, C.byref(no), C.byref(nt), nul, nul, nul, nul, nul,
               nul, nul, nul, nul)
        no, nt = no.value, nt.value
        tag = np.zeros(max(no, 1), np.int32); t0 = np.zeros_like(tag); t1 = np.zeros_like(tag)
        asl = np.zeros(max(nt, 1), np.int32); bsl = np.zeros_like(asl); kk = np.zeros_like(asl)
        aof = np.zeros(max(nt, 1), np.int64); bof = np.zeros_like(aof); al = np.zeros(max(nt, 1))
        N.call("imps_plan_table", self._h, int(prep), stage, None, None, _ptr32(tag), _ptr32(t0), _ptr32(t1),
               _ptr32(asl), aof.ctypes.data_as(N.P_i64), _ptr32(bsl), bof.ctypes.data_as(N.P_i64), _ptr32(kk),
               al.ctypes.data_as(N.P_dbl))
        out = []
        for i in range(no):
            terms = [(int(asl[t]), int(aof[t]), int(bsl[t]), int(bof[t]), int(kk[t]), float(al[t]))
                     for t in range(t0[i], t1[i])]
            out.append((int(tag[i]), terms))
        return out


def _hnnz_arrays(hnnz):
    r = np.array([z[0] for z in hnnz], np.int32)
    c = np.array([z[1] for z in hnnz], np.int32)
    v = np.array([z[2] for z in hnnz], np.float64)
    return r, c, v


def plan_hac(ctx, AC, EHL, EHR, HL, HR, d):
    h = C.c_void_p()
    N.call("imps_plan_hac", ctx.handle, AC.handle, EHL.handle, EHR.handle, HL.handle, HR.handle, d, C.byref(h))
    return Plan(ctx, h, "hac")


def plan_hc(ctx, Cl, EHL, EHR, AL, AR, d, hnnz):
    r, c, v = _hnnz_arrays(hnnz)
    h = C.c_void_p()
    N.call("imps_plan_hc", ctx.handle, Cl.handle, EHL.handle, EHR.handle, AL.handle, AR.handle, d, len(hnnz),
           _ptr32(r), _ptr32(c), v.ctypes.data_as(N.P_dbl), C.byref(h))
    p = Plan(ctx, h, "hc")
    p._keep = (r, c, v)
    return p


def plan_tm(ctx, A_layouts, direction, lin, lout):
    arr = (C.c_void_p * len(A_layouts))(*[a.handle.value for a in A_layouts])
    h = C.c_void_p()
    N.call("imps_plan_tm", ctx.handle, len(A_layouts), arr, int(direction), lin.handle, lout.handle, C.byref(h))
    return Plan(ctx, h, "tm")


def plan_tm_mixed(ctx, A_layouts, B_layouts, direction, lin, lout):
    """ApplyTMmixedLeft/Right(A, B, X) on a unit cell (A lower, B upper layer)."""
    arr_a = (C.c_void_p * len(A_layouts))(*[a.handle.value for a in A_layouts])
    arr_b = (C.c_void_p * len(B_layouts))(*[b.handle.value for b in B_layouts])
    h = C.c_void_p()
    N.call("imps_plan_tm_mixed", ctx.handle, len(A_layouts), arr_a, arr_b, int(direction), lin.handle,
           lout.handle, C.byref(h))
    return Plan(ctx, h, "tmx")


def plan_redop(ctx, A, d, hnnz, direction):
    r, c, v = _hnnz_arrays(hnnz)
    h = C.c_void_p()
    N.call("imps_plan_redop", ctx.handle, A.handle, d, len(hnnz), _ptr32(r), _ptr32(c),
           v.ctypes.data_as(N.P_dbl), int(direction), C.byref(h))
    return Plan(ctx, h, "redop")


def plan_optm(ctx, A0, A1, d, hnnz, direction, lout):
    r, c, v = _hnnz_arrays(hnnz)
    h = C.c_void_p()
    N.call("imps_plan_optm", ctx.handle, A0.handle, A1.handle, d, len(hnnz), _ptr32(r), _ptr32(c),
           v.ctypes.data_as(N.P_dbl), int(direction), lout.handle, C.byref(h))
    return Plan(ctx, h, "optm")


def plan_mps_bd(ctx, A, X, side, alpha=1.0, transpose_x=False):
    h = C.c_void_p()
    N.call("imps_plan_mps_bd", ctx.handle, A.handle, X.handle, int(side) | (2 if transpose_x else 0),
           float(alpha), C.byref(h))
    return Plan(ctx, h, "mps_bd")


def plan_grad_right(ctx, Y, AR):
    h = C.c_void_p()
    N.call("imps_plan_grad_right", ctx.handle, Y.handle, AR.handle, C.byref(h))
    return Plan(ctx, h, "grad")


def plan_decomp(ctx, A, direction):
    """Per-sector dense decomposition tables of A (GetDenseMat order); direction 'l'/'r'."""
    h = C.c_void_p()
    N.call("imps_plan_decomp", ctx.handle, A.handle, 0 if direction in ("l", 0) else 1, C.byref(h))
    p = Plan(ctx, h, "decomp")
    p.rlayout = p.derived(1)
    p.nsv = sum(b[3] for b in p.rlayout.blocks)
    if direction in ("l", 0):
        p.nslayout = p.derived(2)  # left null space (Nullspace(A, l))
    return p


def autotune_clear():
    """Forget every launch shape the autotuner cached in this process."""
    N.call("imps_autotune_clear")
