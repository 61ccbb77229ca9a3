"""Host routines of the device Arnoldi solver (imps_nonsym.h: Hessenberg reduction, Francis
double-shift QR, inverse-iteration eigenvectors, Ritz ordering), compiled with g++ and checked
against LAPACK through numpy."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
P = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("nonsym") / "libnonsym_shim.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", str(HERE / "native" / "nonsym_shim.cpp"),
                    "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    lib.shim_dense_eigvals.restype = C.c_int
    lib.shim_dense_eigvals.argtypes = [C.c_int, P, P, P]
    lib.shim_dense_eigvec.argtypes = [C.c_int, P, C.c_double, C.c_double, C.c_double, P]
    lib.shim_order_ritz.argtypes = [C.c_int, P, P, C.c_int, C.POINTER(C.c_int)]
    return lib


def _p(a):
    return a.ctypes.data_as(P)


def eigvals(lib, G):
    k = G.shape[0]
    Gf = np.asfortranarray(G, dtype=np.float64)
    wr, wi = np.zeros(k), np.zeros(k)
    assert lib.shim_dense_eigvals(k, _p(Gf), _p(wr), _p(wi)) == 0
    return wr + 1j * wi, wr, wi


def eigvec(lib, G, lam):
    k = G.shape[0]
    Gf = np.asfortranarray(G, dtype=np.float64)
    y = np.zeros(2 * k)
    lib.shim_dense_eigvec(k, _p(Gf), float(np.linalg.norm(G)), lam.real, lam.imag, _p(y))
    return y[0::2] + 1j * y[1::2]


def _match(a, b, tol):
    """Every eigenvalue of a has a distinct partner in b within tol (greedy on sorted lists)."""
    b = list(b)
    for x in a:
        j = int(np.argmin([abs(x - y) for y in b]))
        assert abs(x - b[j]) <= tol, (x, b[j])
        b.pop(j)


@pytest.mark.parametrize("k,seed", [(3, 0), (8, 1), (20, 2), (41, 3), (64, 4)])
def test_eigenvalues_match_lapack(shim, k, seed):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((k, k))
    lam, wr, wi = eigvals(shim, G)
    ref = np.linalg.eigvals(G)
    _match(lam, ref, 1e-11 * np.linalg.norm(G))
    # conjugate pairs adjacent, +im first
    i = 0
    while i < k:
        if wi[i] != 0:
            assert wi[i] > 0 and wr[i + 1] == wr[i] and wi[i + 1] == -wi[i]
            i += 2
        else:
            i += 1


def test_structured_spectra(shim):
    # already upper Hessenberg, triangular, symmetric, a rotation block and a defective Jordan block
    rng = np.random.default_rng(7)
    H = np.triu(rng.standard_normal((12, 12)), -1)
    _match(eigvals(shim, H)[0], np.linalg.eigvals(H), 1e-11 * np.linalg.norm(H))
    T = np.triu(rng.standard_normal((9, 9)))
    _match(eigvals(shim, T)[0], np.diag(T), 1e-12 * np.linalg.norm(T))
    S = rng.standard_normal((15, 15))
    S = S + S.T
    lam = eigvals(shim, S)[0]
    assert np.max(np.abs(lam.imag)) < 1e-10
    _match(lam, np.linalg.eigvalsh(S), 1e-11 * np.linalg.norm(S))
    R = np.array([[0.0, -1.0], [1.0, 0.0]])
    _match(eigvals(shim, R)[0], [1j, -1j], 1e-15)
    J = np.diag(np.full(5, 2.0)) + np.diag(np.ones(4), 1)
    _match(eigvals(shim, J)[0], [2.0] * 5, 1e-2)  # defective: only eps^(1/5) accuracy exists
    assert np.all(eigvals(shim, np.zeros((4, 4)))[0] == 0)


def test_transfer_matrix_like_spectrum(shim):
    """A dominant real eigenvalue 1 well separated from a complex bulk (the mixed-TM case)."""
    rng = np.random.default_rng(11)
    k = 40
    X = rng.standard_normal((k, k))
    D = np.diag(np.concatenate([[1.0], 0.5 * rng.random(k - 1)]))
    G = X @ D @ np.linalg.inv(X)
    lam = eigvals(shim, G)[0]
    _match(lam, np.linalg.eigvals(G), 1e-9 * np.linalg.norm(G))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_eigenvectors(shim, seed):
    rng = np.random.default_rng(seed)
    k = 30
    G = rng.standard_normal((k, k))
    lam = eigvals(shim, G)[0]
    for li in lam[:12]:
        y = eigvec(shim, G, li)
        assert abs(np.linalg.norm(y) - 1) < 1e-12
        assert np.linalg.norm(G @ y - li * y) < 1e-11 * np.linalg.norm(G)
        imax = int(np.argmax(np.abs(y)))
        assert abs(y[imax].imag) < 1e-14 and y[imax].real > 0


def test_ritz_order(shim):
    wr = np.array([0.5, 0.5, -1.2, 0.9, 0.1])
    wi = np.array([1.0, -1.0, 0.0, 0.0, 0.0])
    idx = np.zeros(5, np.int32)
    for which, want in [(0, [2, 0, 1, 3, 4]), (1, [3, 0, 1, 4, 2]), (2, [2, 4, 0, 1, 3])]:
        shim.shim_order_ritz(5, _p(wr), _p(wi), which, idx.ctypes.data_as(C.POINTER(C.c_int)))
        assert list(idx) == want, (which, list(idx))
