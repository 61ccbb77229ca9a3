"""Reference-named entry points of the hot path on device buffers.

Each function mirrors one reference function (named in its docstring) and runs entirely on
the GPU through the C ABI; vectors are float64 CUDA tensors in the reference's Vectorize
layout.  There is no CPU path: the native library is required.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .blocks import _dptr


def ApplyHAvec(plan, vin, vout):
    """ApplyHAvec (VUMPS_helpers.hpp:55-88): vout = H_AC vin; operators bound to slots 2..5."""
    N.call("imps_hac_apply", plan.handle, _dptr(vin), _dptr(vout), N.MEM_DEVICE)
    return vout


def ApplyHCvec(plan, vin, vout):
    """ApplyHCvec (VUMPS_helpers.hpp:114-133): vout = H_C vin (call plan.prepare() after AL/AR change)."""
    N.call("imps_hc_apply", plan.handle, _dptr(vin), _dptr(vout), N.MEM_DEVICE)
    return vout


def ApplyTM(plan, vin, vout):
    """ApplyTMLeft/ApplyTMRight on a unit cell (TMBlockFunctions.hpp:557-625) via TMMultDiag."""
    N.call("imps_tm_apply", plan.handle, _dptr(vin), _dptr(vout), N.MEM_DEVICE)
    return vout


def InvEfun_proj(plan, vin, rho_in, rho_out, vout):
    """InvEfun_proj (InvEBlockFunctions.hpp:12-47): vout = vin - T(vin) + tr(vin*rho_in)*rho_out."""
    N.call("imps_tm_proj_apply", plan.handle, _dptr(vin), _dptr(rho_in), _dptr(rho_out), _dptr(vout),
           N.MEM_DEVICE)
    return vout


def eigs_rs(plan, x, tol, ncv=0, maxit=0):
    """eigs_rs(fun, N, vals, vecs, nev=1, "SA", tol, x0) (eigs.cpp:369-494) on the device.

    ``x`` holds x0 on entry and the normalised eigenvector on exit.
    Returns (eigenvalue, number of operator applications, converged)."""
    ev, na = C.c_double(), C.c_int()
    st = N.call("imps_eigs_rs", plan.handle, _dptr(x), N.MEM_DEVICE, float(tol), int(ncv), int(maxit),
                C.byref(ev), C.byref(na))
    return ev.value, na.value, st == 0


def eigs_rs_op(ctx, n, apply, x, nev=1, tol=1e-12, ncv=0, maxit=0, evecs=None):
    """eigs_rs(fun, N, vals, vecs, nev, "SA", tol, x0) (eigs.cpp:369-494) for an operator given as a
    Python callable apply(in_ptr, out_ptr) on device pointers (enqueues work on the context's
    stream).  x: device start vector, on return the lowest Ritz vector; evecs: optional device
    (nev, n) tensor receiving the Ritz vectors.  Returns (eigenvalues, applies, converged)."""
    ev = (C.c_double * nev)()
    na = C.c_int()

    def cb(user, pin, pout):
        try:
            apply(pin, pout)
            return 0
        except Exception:  # a failing apply aborts the solve with an error status
            return -3

    fn = N.APPLY_FN(cb)
    st = N.call("imps_eigs_rs_op", ctx.handle, int(n), fn, None, _dptr(x), N.MEM_DEVICE, int(nev), float(tol), int(ncv),
                int(maxit), ev, None if evecs is None else _dptr(evecs), C.byref(na))
    return [ev[i] for i in range(nev)], na.value, st == 0


def _eigs_n_result(ev, nev, na, st):
    vals = np.array([complex(ev[2 * i], ev[2 * i + 1]) for i in range(nev)])
    return vals, na.value, st == 0


def eigs_n(plan, nev=1, which="LM", tol=1e-14, x0=None, ncv=0, maxit=0, evecs_re=None, evecs_im=None):
    """eigs_n(fun, N, vals, vecs, nev, whch, tol, x0) (eigs.cpp:193-342) for the square operator of
    ``plan`` (TM, mixed TM, H_AC, H_C) by the device Arnoldi.  x0: optional device start vector;
    evecs_re / evecs_im: optional device (nev, n) tensors receiving the Ritz vectors.  Returns
    (complex eigenvalues sorted by ``which``, applies, converged)."""
    ev = (C.c_double * (2 * nev))()
    na = C.c_int()
    st = N.call("imps_eigs_n", plan.handle, None if x0 is None else _dptr(x0), N.MEM_DEVICE, int(nev),
                N.WHICH[which], float(tol), int(ncv), int(maxit), ev,
                None if evecs_re is None else _dptr(evecs_re), None if evecs_im is None else _dptr(evecs_im),
                C.byref(na))
    return _eigs_n_result(ev, nev, na, st)


def eigs_n_op(ctx, n, apply, nev=1, which="LM", tol=1e-14, x0=None, ncv=0, maxit=0, evecs_re=None,
              evecs_im=None):
    """eigs_n for an operator given as a Python callable apply(in_ptr, out_ptr) on device
    pointers, as eigs_rs_op."""
    ev = (C.c_double * (2 * nev))()
    na = C.c_int()

    def cb(user, pin, pout):
        try:
            apply(pin, pout)
            return 0
        except Exception:  # a failing apply aborts the solve with an error status
            return -3

    fn = N.APPLY_FN(cb)
    st = N.call("imps_eigs_n_op", ctx.handle, int(n), fn, None, None if x0 is None else _dptr(x0), N.MEM_DEVICE,
                int(nev), N.WHICH[which], float(tol), int(ncv), int(maxit), ev,
                None if evecs_re is None else _dptr(evecs_re), None if evecs_im is None else _dptr(evecs_im),
                C.byref(na))
    return _eigs_n_result(ev, nev, na, st)


def InvertE_fac(plan, x_re, x_im, fac, y_re, y_im, tol, maxit=0, krylov=0):
    """InvertE_fac(A, B, x, dir, fac) (InvEBlockFunctions.hpp:413-451) for the mixed TM ``plan``:
    (1 - fac T) y = x with complex x, y as real / imaginary device planes (y holds y0 on entry).
    Returns (iterations, relative residual, converged)."""
    it, rr = C.c_int(), C.c_double()
    fac = complex(fac)
    st = N.call("imps_invert_e_fac", plan.handle, _dptr(x_re), _dptr(x_im), fac.real, fac.imag, _dptr(y_re),
                _dptr(y_im), N.MEM_DEVICE, float(tol), int(maxit), int(krylov), C.byref(it), C.byref(rr))
    return it.value, rr.value, st == 0


def InvertE_proj_fac(plan, x_re, x_im, L, R, direction, fac, y_re, y_im, tol, maxit=0, krylov=0):
    """InvertE_proj_fac(A, B, x, L, R, dir, fac) (InvEBlockFunctions.hpp:277-330) for the mixed TM
    ``plan``; L, R real BlockMats paired block by block with x."""
    it, rr = C.c_int(), C.c_double()
    fac = complex(fac)
    d = N.DIR_LEFT if direction in ("l", 0) else N.DIR_RIGHT
    st = N.call("imps_invert_e_proj_fac", plan.handle, _dptr(x_re), _dptr(x_im), _dptr(L), _dptr(R), d,
                fac.real, fac.imag, _dptr(y_re), _dptr(y_im), N.MEM_DEVICE, float(tol), int(maxit), int(krylov),
                C.byref(it), C.byref(rr))
    return it.value, rr.value, st == 0


def InvertE_proj(plan, x, L, R, direction, y, tol, maxit=0, krylov=0):
    """InvertE_proj (InvEBlockFunctions.hpp:201-266) for BlockDiagMat x on the unit cell of ``plan``.

    ``y`` holds y0 on entry and the solution on exit.  direction: 'l' or 'r'.
    Returns (iterations, relative residual, converged)."""
    it, rr = C.c_int(), C.c_double()
    d = N.DIR_LEFT if direction in ("l", 0) else N.DIR_RIGHT
    st = N.call("imps_invert_e_proj", plan.handle, _dptr(x), _dptr(L), _dptr(R), d, _dptr(y), N.MEM_DEVICE,
                float(tol), int(maxit), int(krylov), C.byref(it), C.byref(rr))
    return it.value, rr.value, st == 0


def TMDominantEig(plan, V, x0=None, tol=1e-14, maxit=0):
    """TMDominantEig (EigsBlockFunctions.hpp:91-172) for an isometric unit cell: V <- fixed point
    with unit trace.  Returns (eigenvalue estimate, iterations, converged)."""
    ev, it = C.c_double(), C.c_int()
    st = N.call("imps_tm_dominant", plan.handle, None if x0 is None else _dptr(x0), _dptr(V), N.MEM_DEVICE,
                float(tol), int(maxit), C.byref(ev), C.byref(it))
    return ev.value, it.value, st == 0


def qr(dec, A, Q, R):
    """qr(R, MPS|BlockDiagMat, dir) with diag(R) >= 0 (MPSBlockUtilities.hpp:181-244,
    BlockObj.hpp:2422-2459): Q in A's layout, R BlockDiagMat over the sectors."""
    N.call("imps_sector_qr", dec.handle, _dptr(A), _dptr(Q), _dptr(R), N.MEM_DEVICE)
    return Q, R


def svd(dec, A, U=None, S=None, V=None):
    """svd(S, DiagIso, MPS, dir) (MPSBlockUtilities.hpp:78-153): U = isometry in A's layout,
    S = singular values (sector order, descending), V = DiagIso.  Returns True if converged."""
    p = lambda t: None if t is None else _dptr(t)
    st = N.call("imps_sector_svd", dec.handle, _dptr(A), p(U), p(S), p(V), N.MEM_DEVICE)
    return st == 0


def svd_batch(decs, As, Us=None, Ss=None, Vs=None):
    """Several independent svd(S, DiagIso, MPS, dir) in one launch (imps_sector_svd_batch), e.g.
    the two polar steps of a site update.  Returns True if every one converged."""
    n = len(decs)
    arr = lambda ts: (C.c_void_p * n)(*[None if t is None else _dptr(t) for t in (ts or [None] * n)])
    hs = (C.c_void_p * n)(*[d.handle.value for d in decs])
    st = N.call("imps_sector_svd_batch", n, hs, arr(As), arr(Us), arr(Ss), arr(Vs), N.MEM_DEVICE)
    return st == 0


def Nullspace(plan, A, NL):
    """Nullspace(A, l) (MPSBlockUtilities.hpp:247-300) with a dir-l decomposition plan: NL in the
    plan's derived layout 2."""
    N.call("imps_sector_nullspace", plan.handle, _dptr(A), _dptr(NL), N.MEM_DEVICE)
    return NL


def colscale(dec, X, S, power):
    """X_q[:, j] *= S_q[j]**power on square sector blocks (BlockDiagMat << BlockLam)."""
    N.call("imps_sector_colscale", dec.handle, _dptr(X), _dptr(S), float(power), N.MEM_DEVICE)
    return X


def bd_trace_prod(ctx, layout, X, Y):
    """sum_q trace(X_q Y_q) over a BlockDiagMat layout."""
    r = C.c_double()
    N.call("imps_bd_trace_prod", ctx.handle, layout.handle, _dptr(X), _dptr(Y), C.byref(r))
    return r.value


def norm_inf(ctx, x):
    """norm_inf (helpers.hpp:148-151) of a device vector."""
    r = C.c_double()
    N.call("imps_absmax", ctx.handle, _dptr(x), x.numel(), C.byref(r))
    return r.value


def dot(ctx, x, y):
    """x^T y of two device vectors (fixed-order reduction)."""
    r = C.c_double()
    N.call("imps_dot", ctx.handle, _dptr(x), _dptr(y), int(x.numel()), C.byref(r))
    return r.value


def axpby(ctx, a, x, b, y):
    """y = a*x + b*y on the device."""
    N.call("imps_axpby", ctx.handle, float(a), _dptr(x), float(b), _dptr(y), y.numel())
    return y


def sign_normalize(ctx, x):
    """x /= sign(x[0]) (VUMPS_main.cpp:201-202)."""
    N.call("imps_sign_normalize", ctx.handle, _dptr(x), x.numel())
    return x


def GradNormRight(plan):
    """GradNormRight (VUMPS_helpers.hpp:145-153) from Y = H_AC(C*AR) bound to slot 0 and AR to slot 1."""
    F = C.c_double()
    N.call("imps_grad_norm_right", plan.handle, C.byref(F))
    return F.value


def plan_replicate(plan, copies):
    """imps_plan_replicate: a plan that applies `plan` to `copies` inputs in one launch per stage
    (inputs, outputs and scratch `copies` times as long, operators shared)."""
    from . import blocks as B
    h = C.c_void_p()
    N.call("imps_plan_replicate", plan.handle, int(copies), C.byref(h))
    return B.Plan(plan.ctx, h, "replicated")


def InvertE_fac_batch(rep, xs_re, xs_im, facs, ys_re, ys_im, tol, maxit=0, krylov=0):
    """InvertE_fac (InvEBlockFunctions.hpp:346-476) for P momenta at once on a replicated mixed-TM
    plan (plan_replicate(tm, 2P)): (1 - f_j T) y_j = x_j.  xs_*, ys_*: lists of P device tensors
    (ys_*: initial guesses, overwritten with the solutions).  P GMRES runs in lockstep.  Returns
    (lockstep iterations, the largest relative residual, every system converged)."""
    P = len(facs)
    ptrs = lambda lst: (C.c_void_p * P)(*[t.data_ptr() for t in lst])
    fre = (C.c_double * P)(*[complex(f).real for f in facs])
    fim = (C.c_double * P)(*[complex(f).imag for f in facs])
    it, rr = C.c_int(), C.c_double()
    st = N.call("imps_invert_e_fac_batch", rep.handle, P, ptrs(xs_re), ptrs(xs_im), fre, fim, ptrs(ys_re),
                ptrs(ys_im), float(tol), int(maxit), int(krylov), C.byref(it), C.byref(rr))
    return it.value, rr.value, st == 0


def eigs_rs_batch_op(ctx, P, n, apply, X, nev=1, tol=1e-12, ncv=0, maxit=0):
    """The nev lowest eigenpairs of P symmetric operators at once (imps_eigs_rs_batch_op): apply(in_ptr,
    out_ptr) applies all P operators to P consecutive device vectors of length n.  X: device (P, n)
    start vectors, on return each system's lowest Ritz vector.  Returns (eigenvalues as a (P, nev)
    array, batched applies, per-system convergence flags)."""
    ev = (C.c_double * (P * nev))()
    na = C.c_int()
    conv = (C.c_int * P)()

    def cb(user, pin, pout):
        try:
            apply(pin, pout)
            return 0
        except Exception:  # a failing apply aborts the solve with an error status
            return -3

    fn = N.APPLY_FN(cb)
    N.call("imps_eigs_rs_batch_op", ctx.handle, int(P), int(n), fn, None, _dptr(X), int(nev), float(tol), int(ncv),
           int(maxit), ev, C.byref(na), conv)
    return np.array(list(ev)).reshape(P, nev), na.value, [bool(conv[i]) for i in range(P)]
