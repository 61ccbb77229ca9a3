"""The host tridiagonal routines behind the device Lanczos (Sturm bisection, inverse iteration
with in-cluster orthogonalisation, thick-restart re-tridiagonalisation), compiled with g++
from the library's header and checked against LAPACK on the CPU."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("tridiag") / "libtridiag_shim.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", str(HERE / "native" / "tridiag_shim.cpp"),
                    "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    P = C.POINTER(C.c_double)
    lib.shim_tri_eigval.restype = C.c_double
    lib.shim_tri_eigval.argtypes = [C.c_int, P, P, C.c_int]
    lib.shim_tri_lowest.argtypes = [C.c_int, P, P, C.c_int, P, P]
    lib.shim_arrow_tridiag.argtypes = [C.c_int, P, P, P, P, P]
    return lib


def _p(x):
    return x.ctypes.data_as(C.POINTER(C.c_double))


def _dense(a, b):
    return np.diag(a) + np.diag(b, 1) + np.diag(b, -1)


def _lowest(lib, a, b, nlow):
    k = len(a)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(np.append(b, 0.0), dtype=np.float64)
    w = np.zeros(nlow)
    Z = np.zeros((nlow, k))  # rows = column-major columns
    lib.shim_tri_lowest(k, _p(a), _p(b), nlow, _p(w), _p(Z))
    return w, Z.T


@pytest.mark.parametrize("k,seed,scale", [(1, 0, 1.0), (2, 1, 1.0), (20, 2, 1.0), (80, 3, 3.6e6), (126, 4, 1e-3)])
def test_lowest_eigenpairs_match_lapack(shim, k, seed, scale):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(k) * scale
    b = rng.standard_normal(k - 1) * scale
    nlow = max(1, k // 2)
    w, Z = _lowest(shim, a, b, nlow)
    T = _dense(a, b)
    wr = np.linalg.eigvalsh(T)[:nlow]
    tn = np.abs(T).sum(1).max()
    assert np.abs(w - wr).max() <= 1e-13 * tn
    assert np.linalg.norm(T @ Z - Z * w, axis=0).max() <= 1e-12 * tn
    assert np.abs(Z.T @ Z - np.eye(nlow)).max() < 1e-10


def test_split_and_degenerate_spectrum(shim):
    # two identical decoupled blocks (b = 0 in the middle): every eigenvalue is doubled
    a0 = np.array([1.0, -2.0, 0.5, 3.0])
    b0 = np.array([0.7, -0.2, 1.1])
    a = np.concatenate([a0, a0])
    b = np.concatenate([b0, [0.0], b0])
    w, Z = _lowest(shim, a, b, 6)
    T = _dense(a, b)
    assert np.allclose(w, np.linalg.eigvalsh(T)[:6], atol=1e-13)
    assert np.linalg.norm(T @ Z - Z * w, axis=0).max() < 1e-12
    assert np.abs(Z.T @ Z - np.eye(6)).max() < 1e-10
    # diagonal (all b = 0) with repeated entries
    a = np.array([2.0, -1.0, -1.0, 0.0, -1.0])
    w, Z = _lowest(shim, a, np.zeros(4), 4)
    assert np.allclose(w, [-1, -1, -1, 0])
    assert np.abs(Z.T @ Z - np.eye(4)).max() < 1e-12


def _arrow(lib, th, s):
    kk = len(th)
    th = np.ascontiguousarray(th, dtype=np.float64)
    s = np.ascontiguousarray(s, dtype=np.float64)
    Q = np.zeros((kk, kk))
    qa = np.zeros(kk)
    qb = np.zeros(kk)
    lib.shim_arrow_tridiag(kk, _p(th), _p(s), _p(Q), _p(qa), _p(qb))
    return Q.T, qa, qb[:kk - 1]


@pytest.mark.parametrize("case", ["generic", "degenerate", "sparse_coupling", "zero_coupling"])
def test_arrow_tridiagonalisation(shim, case):
    rng = np.random.default_rng(5)
    kk = 12
    th = np.sort(rng.standard_normal(kk))
    s = rng.standard_normal(kk) * 1e-3
    if case == "degenerate":
        th[3:6] = th[3]
    if case == "sparse_coupling":
        s[::2] = 0.0
    if case == "zero_coupling":
        s[:] = 0.0
    Q, qa, qb = _arrow(shim, th, s)
    assert np.abs(Q.T @ Q - np.eye(kk)).max() < 1e-12
    M = Q.T @ np.diag(th) @ Q
    assert np.abs(M - _dense(qa, qb)).max() < 1e-11 * np.abs(th).max()
    # only the first new direction couples to the residual vector, with coupling |s|
    c = Q.T @ s
    assert abs(abs(c[0]) - np.linalg.norm(s)) < 1e-14 and np.abs(c[1:]).max() < 1e-14
    # the full restarted projected matrix has the same spectrum as the arrowhead it replaces
    alpha = rng.standard_normal()
    A = np.zeros((kk + 1, kk + 1))
    A[:kk, :kk] = np.diag(th)
    A[kk, :kk] = A[:kk, kk] = s
    A[kk, kk] = alpha
    Tq = np.zeros((kk + 1, kk + 1))
    Tq[:kk, :kk] = _dense(qa[::-1], qb[::-1])
    Tq[kk - 1, kk] = Tq[kk, kk - 1] = np.linalg.norm(s)
    Tq[kk, kk] = alpha
    assert np.allclose(np.linalg.eigvalsh(A), np.linalg.eigvalsh(Tq), atol=1e-12)


def test_nearly_degenerate_lowest_pair_large_norm(shim):
    """A lowest pair split by 6e-10 under |T| ~ 1e3 (the H_C spectra of a converged VUMPS
    state): eigenvalues in order and eigenvectors separated, not mixed."""
    rng = np.random.default_rng(9)
    k = 64
    Q, _ = np.linalg.qr(rng.standard_normal((k, k)))
    lam = np.concatenate([[-1.2980078565, -1.2980078559], np.sort(rng.uniform(-1.0, 1e3, k - 2))])
    A = (Q * lam) @ Q.T
    # Householder tridiagonalisation of A (numpy only): T = P^T A P
    T = A.copy()
    for j in range(k - 2):
        x = T[j + 1:, j].copy()
        v = x.copy()
        v[0] += np.copysign(np.linalg.norm(x), x[0])
        v /= np.linalg.norm(v)
        H = np.eye(k - j - 1) - 2.0 * np.outer(v, v)
        T[j + 1:, :] = H @ T[j + 1:, :]
        T[:, j + 1:] = T[:, j + 1:] @ H
    a, b = np.diag(T).copy(), np.diag(T, 1).copy()
    w, Z = _lowest(shim, a, b, 2)
    Td = _dense(a, b)
    wr = np.linalg.eigvalsh(Td)[:2]
    assert np.abs(w - wr).max() < 1e-12 * 1e3
    assert w[0] < w[1]
    assert np.linalg.norm(Td @ Z - Z * w, axis=0).max() < 1e-9
