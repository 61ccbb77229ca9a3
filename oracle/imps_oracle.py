"""CPU oracle (test infrastructure only): numpy restatement of IMPS_CPP_tools' hot path.

Parity status: UNPINNED by the reference (no reference tests/golden vectors; the
reference is not buildable here).  Pinned instead by dense re-evaluation, the
reference's inline identities and the Heisenberg Bethe-ansatz energy (see tests).

Data model, mirroring MPShelpers/include/Block/BlockObj.hpp and MPSBlockMat.hpp:
  * charge keys are tuples of ints; ``sorted()`` on tuples is the lexicographic
    ``std::vector<int>`` ``operator<`` that orders every ``std::map`` in the
    reference (KeyTypes.hpp:19-59, ordering inherited from std::vector).
  * BlockDiag  : dict  key -> 2-D ndarray            (BlockDiagMat, BlockObj.hpp:1360-1467)
  * BlockMat   : dict  qin -> (qout, 2-D ndarray)    (BlockMat, BlockObj.hpp:506-600)
  * MPS        : list over physical index s of BlockMat (MPSBlockMat.hpp:41-175)
  * vectors    : concatenation of column-major blocks in key order, s-major for
                 MPS (MPSBlockMat.hpp:448-465, BlockObj.hpp:767-780, 1712).
Only U(1)^k charges are restated (all configurations use U(1) or U(1)xU(1)).
"""
from __future__ import annotations

import math

import numpy as np

# ----------------------------------------------------------------------------------------------
# charges, I2K, dims  (KeyTypes.hpp:123-136, ItoKey.hpp:126-165, Models.cpp:13-32,216-295,642-733)
# ----------------------------------------------------------------------------------------------


# The charge group of the model being checked (symobj.hpp:120-158): None for U(1)^k, else one
# period per component (0 for U(1), N for Z(N), representatives in [0, N)).
_PERIODS = None


class charge_group:
    """Context in which kadd / ksub reduce the components with a nonzero period modulo it."""

    def __init__(self, periods):
        self.periods = tuple(periods) if periods else None

    def __enter__(self):
        global _PERIODS
        self.prev, _PERIODS = _PERIODS, self.periods
        return self

    def __exit__(self, *exc):
        global _PERIODS
        _PERIODS = self.prev
        return False


def _reduce(t):
    if not _PERIODS:
        return t
    return tuple(x % p if p else x for x, p in zip(t, _PERIODS))


def kadd(a, b):
    return _reduce(tuple(x + y for x, y in zip(a, b)))


def ksub(a, b):
    return _reduce(tuple(x - y for x, y in zip(a, b)))


def xxz_dQ(N, QN):
    """XXZModel::GetdQ (Models.cpp:216-240), spin-1/2 case."""
    m = QN[0]
    if abs(m) >= N:
        raise ValueError("|m| < N!")
    div = math.gcd(N - m, N + m)
    return [(2 * N // div, -((N + m) // div))]


def xxz_i2k(N, QN, d=2):
    """XXZModel::GetI2K (Models.cpp:262-295): I2K[k] = dQ.second + s*dQ.first, s = d-1 .. 0."""
    dQ = xxz_dQ(N, QN)
    return [(dQ[0][1] + s * dQ[0][0],) for s in range(d - 1, -1, -1)]


def fhub_dQ(N, QN):
    """FermiHubbardModel::GetdQ, (N,M) representation (Models.cpp:642-660)."""
    n, m = QN
    if n + m <= 0 or n + m >= 2 * N or n - m <= 0 or n - m >= 2 * N:
        raise ValueError("QN out of range")
    divn = math.gcd(math.gcd(N - n, 2 * N - n), n)
    divm = math.gcd(math.gcd(N - m, N + m), m)
    return [(N // divn, -(n // divn)), (N // divm, -((N + m) // divm))]


def fhub_i2k(N, QN):
    """FermiHubbardModel::GetI2K, (N,M) representation (Models.cpp:701-718)."""
    (a1, a0), (b1, b0) = fhub_dQ(N, QN)
    return [(a0, b0 + b1), (a0 + a1, b0), (a0 + a1, b0 + 2 * b1), (a0 + 2 * a1, b0 + b1)]


def qim_i2k():
    """QuantumIsingModel::GetI2K (Models.cpp:371-375), charges in Z(2)."""
    return [(0,), (1,)]


def qim_h(J=1.0, h=1.0):
    """XYZAbstractModel(QIM, J, 0, 0, h, 2) (Models.cpp:91): element by element, spin-1/2
    basis |up>, |down>: -J/4 flips both spins, -h/4 (+-1 +-1) on the diagonal."""
    H = np.zeros((4, 4))
    for s0 in range(2):
        for s1 in range(2):
            r = 2 * s0 + s1
            H[r, r] = -0.5 * h * ((0.5 if s0 == 0 else -0.5) + (0.5 if s1 == 0 else -0.5))
            H[2 * (1 - s0) + (1 - s1), r] += -0.25 * J
    return H


def potts_i2k(q):
    """QuantumPottsModel::GetI2K (Models.cpp:498-504), charges in Z(q)."""
    return [(i,) for i in range(q)]


def potts_h(q, h=1.0):
    """QuantumPottsModel::MakeOps (Models.cpp:405-425) element by element: X^k lowers a level by
    k (mod q), so X^k (x) X^(q-k) maps |i, j> to |i - k, j + k>; Z = q delta_{i0} - 1."""
    H = np.zeros((q * q, q * q))
    for i in range(q):
        for j in range(q):
            r = i * q + j
            H[r, r] = -0.5 * h * ((q if i == 0 else 0) - 1 + (q if j == 0 else 0) - 1)
            for k in range(1, q):
                H[((i - k) % q) * q + (j + k) % q, r] -= 1.0
    return H


def bhub_dQ(N, QN):
    """BoseHubbardModel::GetdQ (Models.cpp:825-838): (N / g, -n / g) with g = gcd(N, n)."""
    n = QN[0]
    if n < 1:
        raise ValueError("n must be positive")
    g = math.gcd(N, n)
    return N // g, -(n // g)


def bhub_i2k(N, QN, d):
    """BoseHubbardModel::GetI2K (Models.cpp:855-862): level i -> dQ.second + i dQ.first."""
    first, second = bhub_dQ(N, QN)
    return [(second + i * first,) for i in range(d)]


def bhub_h(d, t=1.0, U=4.0, mu=0.0):
    """BoseHubbardModel::MakeOps (Models.cpp:768-779), element by element."""
    D = d * d
    h = np.zeros((D, D))
    for i0 in range(d):
        for i1 in range(d):
            r = i0 * d + i1
            # on-site part shared by the two sites: 0.5 (U/2 n(n-1) - mu n) on each
            h[r, r] += 0.5 * (0.5 * U * i0 * (i0 - 1) - mu * i0) + 0.5 * (0.5 * U * i1 * (i1 - 1) - mu * i1)
            # b (x) b^+ moves a boson from site 0 to site 1, b^+ (x) b from 1 to 0
            if i0 >= 1 and i1 + 1 < d:
                h[(i0 - 1) * d + i1 + 1, r] += -t * math.sqrt(i0) * math.sqrt(i1 + 1)
            if i1 >= 1 and i0 + 1 < d:
                h[(i0 + 1) * d + i1 - 1, r] += -t * math.sqrt(i1) * math.sqrt(i0 + 1)
    return h


def _path_iter(N, key, I2K, zero):
    if N == 1:
        for j, k in enumerate(I2K):
            if kadd(key, k) == zero:
                return True, [j]
        return False, []
    for j, k in enumerate(I2K):
        ok, p = _path_iter(N - 1, kadd(key, k), I2K, zero)
        if ok:
            return True, p + [j]
    return False, []


def validpath(N, I2K):
    """ItoKey.hpp:126-165 (starts at I2K.front(), zero key = I2K.front())."""
    ok, p = _path_iter(N, I2K[0], I2K, I2K[0])
    if not ok:
        raise ValueError("validpath: no valid path found for current ItoKey")
    return p


def make_dims(dmap0, N, I2K):
    """ModelBase::MakeDims (Models.cpp:13-32): dims of bond k, k=0..N-1."""
    path = validpath(N, I2K)
    out, cur = [], dict(dmap0)
    for k in range(N):
        out.append(dict(cur))
        sh = I2K[path[N - k - 1]]
        cur = {kadd(q, sh): m for q, m in cur.items()}
    return out


# ----------------------------------------------------------------------------------------------
# two-site Hamiltonians (Models.cpp:57-93 XYZ/XXZ, :543-572 FHUB)
# ----------------------------------------------------------------------------------------------


def xxz_h(J=1.0, Delta=1.0, hz=0.0):
    """ham = -Jx sx.sx + Jy syi.syi - Jz sz.sz - hz/2 (sz.1 + 1.sz), with Jx=Jy=J, Jz=Delta."""
    sx = np.array([[0, 0.5], [0.5, 0]])
    syi = np.array([[0, -0.5], [0.5, 0]])
    sz = np.diag([0.5, -0.5])
    I = np.eye(2)
    return (-J * np.kron(sx, sx) + J * np.kron(syi, syi) - Delta * np.kron(sz, sz)
            - 0.5 * hz * (np.kron(sz, I) + np.kron(I, sz)))


def fhub_h(t=1.0, U=4.0, V=0.0, mu=0.0, hz=0.0):
    cup = np.zeros((4, 4)); cup[0, 2] = 1; cup[1, 3] = 1
    cdo = np.zeros((4, 4)); cdo[0, 1] = 1; cdo[2, 3] = -1
    nup = np.diag([0, 0, 1.0, 1.0]); ndo = np.diag([0, 1.0, 0, 1.0])
    I = np.eye(4); F = np.diag([1.0, -1, -1, 1])
    nup2 = nup - 0.5 * I; ndo2 = ndo - 0.5 * I
    nund = nup2 @ ndo2; nupnd = nup + ndo; nupnd2 = nup2 + ndo2; sz = 0.5 * (nup - ndo)
    return (-t * (np.kron(cup.T @ F, cup) - np.kron(cup @ F, cup.T) + np.kron(cdo.T @ F, cdo)
                  - np.kron(cdo @ F, cdo.T))
            + 0.5 * U * (np.kron(nund, I) + np.kron(I, nund)) + V * np.kron(nupnd2, nupnd2)
            - 0.5 * mu * (np.kron(nupnd, I) + np.kron(I, nupnd))
            - 0.5 * hz * (np.kron(sz, I) + np.kron(I, sz)))


def sparse_nnz(h):
    """Nonzeros of an armadillo SpMat in its iteration order (column-major, rows ascending)."""
    out = []
    for c in range(h.shape[1]):
        for r in range(h.shape[0]):
            if h[r, c] != 0.0:
                out.append((r, c, float(h[r, c])))
    return out


def num2ditvec(x, d):
    """helpers.cpp:3-17 for N=2: (left site index, right site index)."""
    return x // d, x % d


# ----------------------------------------------------------------------------------------------
# containers and layout (BlockObj.hpp, MPSBlockMat.hpp)
# ----------------------------------------------------------------------------------------------


def mps_rand(I2K, dl, dr, rng, dtype=np.float64):
    """MPSBlockMat(I2K, ml, mr, fill::randn) (MPSBlockMat.hpp:221-236), blocks filled column-major."""
    A = []
    for sh in I2K:
        bm = {}
        for ql in sorted(dl):
            qr = kadd(ql, sh)
            if qr in dr:
                ml, mr = dl[ql], dr[qr]
                bm[ql] = (qr, rng.standard_normal(ml * mr).reshape(mr, ml).T.astype(dtype).copy())
        A.append(bm)
    return A


def mps_sizes(A):
    """MPSBlockMat::GetSizesVector (MPSBlockMat.hpp:336-347)."""
    return [[(q, A[s][q][0], A[s][q][1].shape[0], A[s][q][1].shape[1]) for q in sorted(A[s])]
            for s in range(len(A))]


def mps_vec(A):
    parts = [A[s][q][1].reshape(-1, order="F") for s in range(len(A)) for q in sorted(A[s])]
    return np.concatenate(parts) if parts else np.zeros(0)


def mps_from_vec(v, sizes):
    A, pos = [], 0
    for blocks in sizes:
        bm = {}
        for (qi, qo, ml, mr) in blocks:
            bm[qi] = (qo, np.array(v[pos:pos + ml * mr]).reshape(mr, ml).T.copy())
            pos += ml * mr
        A.append(bm)
    return A


def mps_nelem(A):
    return sum(b[1].size for bm in A for b in bm.values())


def bd_sizes(X):
    return [(q, X[q].shape[0]) for q in sorted(X)]


def bd_vec(X):
    parts = [X[q].reshape(-1, order="F") for q in sorted(X)]
    return np.concatenate(parts) if parts else np.zeros(0)


def bd_from_vec(v, sizes):
    X, pos = {}, 0
    for (q, m) in sizes:
        X[q] = np.array(v[pos:pos + m * m]).reshape(m, m).T.copy()
        pos += m * m
    return X


def bm_vec(X):
    parts = [X[q][1].reshape(-1, order="F") for q in sorted(X)]
    return np.concatenate(parts) if parts else np.zeros(0)


def bm_from_vec(v, sizes):
    X, pos = {}, 0
    for (qi, qo, ml, mr) in sizes:
        X[qi] = (qo, np.array(v[pos:pos + ml * mr]).reshape(mr, ml).T.copy())
        pos += ml * mr
    return X


def bm_sizes(X):
    return [(q, X[q][0], X[q][1].shape[0], X[q][1].shape[1]) for q in sorted(X)]


def bd_eye(dims):
    return {q: np.eye(m) for q, m in dims.items()}


def bd_trace(X):
    return sum(np.trace(X[q]) for q in sorted(X))


def bm_t(X):
    """BlockMat::t(): key Qout -> (Qin, M^T)."""
    return {qo: (qi, M.T.copy()) for qi, (qo, M) in X.items()}


def bm_mul(L, R):
    """operator*(BlockMat, BlockMat) (BlockObj.hpp:2557-2568)."""
    out = {}
    for qi in sorted(L):
        qo, M = L[qi]
        if qo in R:
            out[qi] = (R[qo][0], M @ R[qo][1])
    return out


def bm_mul_bd(L, D):
    """operator*(BlockMat, BlockDiagMat) (BlockObj.hpp:2570-2589)."""
    return {qi: (qo, M @ D[qo]) for qi, (qo, M) in L.items() if qo in D}


def bd_mul_bm(D, R):
    """operator*(BlockDiagMat, BlockMat) (BlockObj.hpp:2591-2610)."""
    return {qi: (qo, D[qi] @ M) for qi, (qo, M) in R.items() if qi in D}


def bd_mul(A, B):
    return {q: A[q] @ B[q] for q in A if q in B}


def bm_scale(X, a):
    return {q: (qo, a * M) for q, (qo, M) in X.items()}


def bm_iadd(X, Y):
    """BlockMat::operator+= (BlockObj.hpp:1044-1063): adds, inserting missing sectors."""
    for qi in sorted(Y):
        qo, M = Y[qi]
        if qi in X:
            assert X[qi][0] == qo
            X[qi] = (qo, X[qi][1] + M)
        else:
            X[qi] = (qo, M.copy())
    return X


def bd_iadd(X, Y):
    for q, M in Y.items():
        X[q] = X[q] + M if q in X else M.copy()
    return X


def bd_add(X, Y):
    return bd_iadd({q: M.copy() for q, M in X.items()}, Y)


def bd_t(X):
    return {q: M.T.copy() for q, M in X.items()}


def mps_mul_bd(A, D):
    return [bm_mul_bd(a, D) for a in A]


def bd_mul_mps(D, A):
    return [bd_mul_bm(D, a) for a in A]


def mps_mul_mps(A, B):
    """2-site product (MPSBlockMat.hpp:934-947): out[i*d+j] = A[i]*B[j]."""
    return [bm_mul(a, b) for a in A for b in B]


def mps_sub(A, B):
    out = []
    for a, b in zip(A, B):
        c = {q: (qo, M.copy()) for q, (qo, M) in a.items()}
        bm_iadd(c, bm_scale(b, -1.0))
        out.append(c)
    return out


def mps_norm_inf(A):
    return max((np.abs(M).max() for bm in A for (_, M) in bm.values() if M.size), default=0.0)


# ----------------------------------------------------------------------------------------------
# H_AC / H_C (VUMPS/VUMPS_helpers.hpp:38-133)
# ----------------------------------------------------------------------------------------------


def _mps_add_into_existing(out, contrib):
    """out[s] += contrib[s] where out is a view on a fixed buffer: sectors absent from out are
    lost (the reference inserts them into the map of non-owning views, outside the buffer)."""
    for s, bm in enumerate(contrib):
        for qi, (qo, M) in bm.items():
            if qi in out[s]:
                assert out[s][qi][0] == qo
                out[s][qi][1][...] += M


def ApplyHA(inp, EHL, EHR, HL, HR):
    """ApplyHA (VUMPS_helpers.hpp:38-53): out = EHL*in + in*EHR + sum_ij HL[i][j]*in[j] + in[j]*HR[i][j]."""
    d = len(inp)
    out = [{q: (qo, np.zeros_like(M)) for q, (qo, M) in bm.items()} for bm in inp]
    t1 = bd_mul_mps(EHL, inp)
    t2 = mps_mul_bd(inp, EHR)
    _mps_add_into_existing(out, [bm_iadd(a, b) for a, b in zip(t1, t2)])
    for i in range(d):
        for j in range(d):
            c = bm_iadd(bm_mul(HL[i][j], inp[j]), bm_mul(inp[j], HR[i][j]))
            contrib = [dict() for _ in range(d)]
            contrib[i] = c
            _mps_add_into_existing(out, contrib)
    return out


def ApplyHAvec(vin, Adims, EHL, EHR, HL, HR):
    """ApplyHAvec (VUMPS_helpers.hpp:55-88)."""
    return mps_vec(ApplyHA(mps_from_vec(vin, Adims), EHL, EHR, HL, HR))


def ApplyHC(inp, EHL, EHR, hnnz, d, AL, AR):
    """ApplyHC (VUMPS_helpers.hpp:91-111), literal chained form per nonzero of h."""
    out = {q: np.zeros_like(M) for q, M in inp.items()}
    base = bd_add(bd_mul(EHL, inp), bd_mul(inp, EHR))
    for q in out:
        if q in base:
            out[q] += base[q]
    inp_bm = {q: (q, M) for q, M in inp.items()}
    for (r, c, h) in hnnz:
        i0, i1 = num2ditvec(r, d)
        j0, j1 = num2ditvec(c, d)
        X = bm_mul(bm_scale(bm_t(AL[i0]), h), AL[j0])
        X = bm_mul(X, inp_bm)
        X = bm_mul(X, AR[j1])
        X = bm_mul(X, bm_t(AR[i1]))
        for qi, (qo, M) in X.items():
            assert qi == qo
            if qi in out:
                out[qi] += M
    return out


def ApplyHCvec(vin, Cdims, EHL, EHR, hnnz, d, AL, AR):
    return bd_vec(ApplyHC(bd_from_vec(vin, Cdims), EHL, EHR, hnnz, d, AL, AR))


# ----------------------------------------------------------------------------------------------
# transfer matrices (MPShelpers/include/Block/TMBlockFunctions.hpp)
# ----------------------------------------------------------------------------------------------


def ApplyTMLeft(A, X):
    """TMBlockFunctions.hpp:33-56: out(Qout) += A_s^T (X(Qin) A_s)."""
    out = {}
    for bm in A:
        for qi in sorted(bm):
            qo, M = bm[qi]
            if qi in X:
                c = M.T @ (X[qi] @ M)
                out[qo] = out[qo] + c if qo in out else c
    return out


def ApplyTMRight(A, X):
    """TMBlockFunctions.hpp:155-177: out(Qin) += (A_s X(Qout)) A_s^T."""
    out = {}
    for bm in A:
        for qi in sorted(bm):
            qo, M = bm[qi]
            if qo in X:
                c = (M @ X[qo]) @ M.T
                out[qi] = out[qi] + c if qi in out else c
    return out


def ApplyTMLeftUC(Avec, X):
    """TMBlockFunctions.hpp:557-563 (sites in order)."""
    for A in Avec:
        X = ApplyTMLeft(A, X)
    return X


def ApplyTMRightUC(Avec, X):
    """TMBlockFunctions.hpp:600-606 (sites in reverse order)."""
    for A in reversed(Avec):
        X = ApplyTMRight(A, X)
    return X


def ApplyTMmixedLeftDiag(A, B):
    """TMBlockFunctions.hpp:259-289: out(Qout(B_s)) += B_s^T A_s, B found by Qin(A)."""
    out = {}
    for s in range(len(A)):
        if not A[s] or not B[s]:
            continue
        for qi in sorted(A[s]):
            qa, MA = A[s][qi]
            if qi in B[s]:
                qb, MB = B[s][qi]
                assert qb == qa
                c = MB.T @ MA
                out[qb] = out[qb] + c if qb in out else c
    return out


def ApplyTMmixedRightDiag(A, B):
    """TMBlockFunctions.hpp:401-434: out(Qin(A_s)) += A_s B_s^T, B found by Qin(A)."""
    out = {}
    for s in range(len(A)):
        if not A[s] or not B[s]:
            continue
        for qi in sorted(A[s]):
            qa, MA = A[s][qi]
            if qi in B[s]:
                qb, MB = B[s][qi]
                assert qb == qa
                c = MA @ MB.T
                out[qi] = out[qi] + c if qi in out else c
    return out


def bm_dK(X):
    qi = next(iter(sorted(X)))
    return ksub(X[qi][0], qi)


def ApplyTMmixedRight(A, B):
    """TMBlockFunctions.hpp:445-473 (general BlockMat result): out(Qin(A_s) -> Qin(B_s)) += A_s B_s^T,
    B found by Qout(A_s) - dK(B_s)."""
    out = {}
    for s in range(len(A)):
        if not A[s] or not B[s]:
            continue
        dKB = bm_dK(B[s])
        for qi in sorted(A[s]):
            qa, MA = A[s][qi]
            qbi = ksub(qa, dKB)
            if qbi in B[s]:
                _, MB = B[s][qbi]
                c = MA @ MB.T
                if qi in out and out[qi][0] == qbi:
                    out[qi] = (qbi, out[qi][1] + c)
                elif qi not in out:
                    out[qi] = (qbi, c)
                # else: std::map::emplace_hint keeps the block already there (same incoming,
                # other outgoing charge) and drops this one (TMBlockFunctions.hpp:466-468)
    return out


def ApplyTMmixedLeft(A, B):
    """TMBlockFunctions.hpp:306-330 (general BlockMat result): out(Qout(B_s) -> Qout(A_s)) += B_s^T A_s."""
    out = {}
    for s in range(len(A)):
        if not A[s] or not B[s]:
            continue
        for qi in sorted(A[s]):
            qa, MA = A[s][qi]
            if qi in B[s]:
                qb, MB = B[s][qi]
                c = MB.T @ MA
                if qb in out and out[qb][0] == qa:
                    out[qb] = (qa, out[qb][1] + c)
                elif qb not in out:
                    out[qb] = (qa, c)
                # else: dropped, as emplace_hint does (TMBlockFunctions.hpp:324-327)
    return out


def ApplyTMmixedLeftX(A, B, X):
    """ApplyTMmixedLeft(A, B, in) on a general BlockMat (TMBlockFunctions.hpp:336-344):
    ApplyTMmixedLeft(in*A, B), i.e. out(Qout(B_s) -> Qout(A_s)) += B_s^T X A_s."""
    return ApplyTMmixedLeft([bm_mul(X, a) for a in A], B)


def ApplyTMmixedRightX(A, B, X):
    """ApplyTMmixedRight(A, B, in) on a general BlockMat (TMBlockFunctions.hpp:474-482):
    ApplyTMmixedRight(A*in, B), i.e. out(Qin(A_s) -> Qin(B_s)) += A_s X B_s^T."""
    return ApplyTMmixedRight([bm_mul(a, X) for a in A], B)


def ApplyTMmixedLeftUC(Avec, Bvec, X):
    """Unit-cell chain in site order (TMBlockFunctions.hpp:669-676)."""
    for A, B in zip(Avec, Bvec):
        X = ApplyTMmixedLeftX(A, B, X)
    return X


def ApplyTMmixedRightUC(Avec, Bvec, X):
    """Unit-cell chain in reverse site order (TMBlockFunctions.hpp:737-744)."""
    for A, B in zip(reversed(Avec), reversed(Bvec)):
        X = ApplyTMmixedRightX(A, B, X)
    return X


def bm_trace_pairs(X, Rho):
    """sum_b tr(X_b Rho_b) with the blocks paired in iteration order, as
    InvEfun_proj_fac does (InvEBlockFunctions.hpp:104-108)."""
    return sum(np.trace(X[qx][1] @ Rho[qr][1]) for qx, qr in zip(sorted(X), sorted(Rho)))


def InvEfun_fac(invec, TMfun, sizes, fac):
    """InvEfun_fac for BlockMat (InvEBlockFunctions.hpp:166-197): y = x - fac * TM(x)."""
    x = bm_from_vec(invec, sizes)
    Tx = TMfun(x)
    y = np.array(invec, dtype=np.result_type(invec, fac)).copy()
    pos = 0
    for (qi, qo, ml, mr) in sizes:
        y[pos:pos + ml * mr] -= fac * Tx[qi][1].reshape(-1, order="F")
        pos += ml * mr
    return y


def InvEfun_proj_fac(invec, TMfun, rho_inside, rho_outside, sizes, fac):
    """InvEfun_proj_fac for BlockMat (InvEBlockFunctions.hpp:90-125):
    y = x - fac * TM(x) + tr(x * rho_in) * rho_out."""
    x = bm_from_vec(invec, sizes)
    tr = bm_trace_pairs(x, rho_inside)
    return InvEfun_fac(invec, TMfun, sizes, fac) + tr * bm_vec(rho_outside)


def InvertE_fac(Avec, Bvec, x, direction, fac, tol=1e-14, maxit=0, y0=None, rng=None):
    """InvertE_fac(A, B, x, dir, fac) (InvEBlockFunctions.hpp:413-451) with the reference's GMRES.
    Returns (y as BlockMat, flag)."""
    sizes = bm_sizes(x)
    mtot = sum(ml * mr for (_, _, ml, mr) in sizes)
    if maxit == 0:
        maxit = mtot
    if y0 is None:
        rng = rng if rng is not None else np.random.default_rng(0)
        y0v = rng.standard_normal(mtot) + 0j
    else:
        y0v = bm_vec(y0) + 0j
    TMfun = (lambda X: ApplyTMmixedLeftUC(Avec, Bvec, X)) if direction == "l" else \
        (lambda X: ApplyTMmixedRightUC(Avec, Bvec, X))
    y, flag = gmres(lambda v: InvEfun_fac(v, TMfun, sizes, fac), bm_vec(x) + 0j, y0v, tol, maxit)
    return bm_from_vec(y, sizes), flag


def InvertE_proj_fac(Avec, Bvec, x, L, R, direction, fac, tol=1e-14, maxit=0, y0=None, rng=None):
    """InvertE_proj_fac(A, B, x, L, R, dir, fac) (InvEBlockFunctions.hpp:277-330):
    dir l: b = x - tr(x R) L, operator with (rho_in, rho_out) = (R, L); dir r: b = x - tr(L x) R,
    (rho_in, rho_out) = (L, R)."""
    sizes = bm_sizes(x)
    mtot = sum(ml * mr for (_, _, ml, mr) in sizes)
    if maxit == 0:
        maxit = mtot
    if y0 is None:
        rng = rng if rng is not None else np.random.default_rng(0)
        y0v = rng.standard_normal(mtot) + 0j
    else:
        y0v = bm_vec(y0) + 0j
    xv = bm_vec(x) + 0j
    if direction == "l":
        xv = xv - bm_trace_pairs(x, R) * bm_vec(L)
        TMfun = lambda X: ApplyTMmixedLeftUC(Avec, Bvec, X)
        Afun = lambda v: InvEfun_proj_fac(v, TMfun, R, L, sizes, fac)
    else:
        xv = xv - bm_trace_pairs(x, L) * bm_vec(R)
        TMfun = lambda X: ApplyTMmixedRightUC(Avec, Bvec, X)
        Afun = lambda v: InvEfun_proj_fac(v, TMfun, L, R, sizes, fac)
    y, flag = gmres(Afun, xv, y0v, tol, maxit)
    return bm_from_vec(y, sizes), flag


# ----------------------------------------------------------------------------------------------
# excitation ansatz: effective Hamiltonian on X (Excitations/Excitations_helpers.hpp:20-228)
# ----------------------------------------------------------------------------------------------


def mps_mul_bm(A, X):
    """MPSBlockMat * BlockMat: [A_s X]."""
    return [bm_mul(a, X) for a in A]


def bm_mul_mps(X, A):
    """BlockMat * MPSBlockMat: [X A_s]."""
    return [bm_mul(X, a) for a in A]


def mps_add(A, B):
    """MPSBlockMat + MPSBlockMat (sector-wise, inserting missing sectors)."""
    out = [{q: (qo, M.copy()) for q, (qo, M) in a.items()} for a in A]
    for o, b in zip(out, B):
        bm_iadd(o, b)
    return out


def mps_scale(A, a):
    return [bm_scale(x, a) for x in A]


def bm_add(X, Y):
    return bm_iadd({q: (qo, M.copy()) for q, (qo, M) in X.items()}, Y)


def ApplyOpTMLeftGen(hnnz, A, B):
    """TMBlockFunctions.hpp:825-830: ApplyTMmixedLeft(ApplyOperator(A, O), B)."""
    return ApplyTMmixedLeft(ApplyOperator(A, hnnz), B)


def HeffConstants(AL, AR, L, R, hnnz, tol=1e-14, rng=None):
    """Excitations_helpers.hpp:258-331 (h with E0 already subtracted): the environments HLtot[n]
    (left of the bond right of site n) and HRtot[n] (right of the bond left of site n)."""
    N = len(AL)
    P = lambda x: (x + N) % N
    HL = [ApplyOpTMLeftDiag(hnnz, mps_mul_mps(AL[N - 1], AL[0]))]
    for n in range(1, N):
        HL.append(bd_add(ApplyOpTMLeftDiag(hnnz, mps_mul_mps(AL[n - 1], AL[n])), ApplyTMLeft(AL[n], HL[-1])))
    HR = [None] * N
    HR[N - 1] = ApplyOpTMRightDiag(hnnz, mps_mul_mps(AR[N - 1], AR[0]))
    for n in range(N - 2, -1, -1):
        HR[n] = bd_add(ApplyOpTMRightDiag(hnnz, mps_mul_mps(AR[n], AR[n + 1])), ApplyTMRight(AR[n], HR[n + 1]))
    HLtot, HRtot = [None] * N, [None] * N
    eyeR = bd_eye({q: M.shape[1] for q, M in R.items()})
    EHL = [None] * N
    EHL[N - 1], _ = InvertE_proj(AL, HL[N - 1], eyeR, R, "l", tol, rng=rng)
    HLtot[N - 1] = EHL[N - 1]
    for n in range(N - 1):
        EHL[n] = ApplyTMLeft(AL[n], EHL[P(n - 1)])
        HLtot[n] = bd_add(HL[n], EHL[n])
    eyeL = bd_eye({q: M.shape[1] for q, M in L.items()})
    EHR = [None] * N
    EHR[0], _ = InvertE_proj(AR, HR[0], L, eyeL, "r", tol, rng=rng)
    HRtot[0] = EHR[0]
    for n in range(N - 1, 0, -1):
        EHR[n] = ApplyTMRight(AR[n], EHR[P(n + 1)])
        HRtot[n] = bd_add(EHR[n], HR[n])
    return HLtot, HRtot


def XDims(NL, AR, K):
    """Excitations_helpers.hpp:641-678: sectors of X_n: NL[n] right keys q with AR[n+1] left keys
    q + K (both non-empty)."""
    N = len(NL)
    out = []
    for n in range(N):
        ml = {}
        for bm in NL[n]:
            for qi, (qo, M) in bm.items():
                ml.setdefault(qo, M.shape[1])
        mr = {}
        for bm in AR[(n + 1) % N]:
            for qi, (qo, M) in bm.items():
                mr.setdefault(qi, M.shape[0])
        dims = []
        for q in sorted(ml):
            qk = kadd(q, K)
            if qk in mr and ml[q] > 0 and mr[qk] > 0:
                dims.append((q, qk, ml[q], mr[qk]))
        out.append(dims)
    return out


def ApplyHeff(Xin, kfac, AL, AR, NL, hnnz, d, HLtot, HRtot, LM=None, RM=None, tol=1e-14, rng=None):
    """Effective Hamiltonian of the excitation ansatz applied to X (Excitations_helpers.hpp:20-211):
    B_n = NL_n X_n; the terms with B right of, on top of and left of the output site; the
    infinite sums closed by the factored environment solves EBR (right, fac = kfac) and EHBL
    (left, fac = conj(kfac)), projected when LM and RM are given.  Returns Xout (list of
    BlockMats; the caller keeps the sectors of its X structure)."""
    N = len(Xin)
    ck = np.conj(kfac)
    P = lambda x: (x + N) % N
    proj = LM is not None and RM is not None
    Bin = [mps_mul_bm(NL[n], Xin[n]) for n in range(N)]
    # B overlapping AR to the right within the unit cell (:64-72)
    ABR = [None] * N
    ABR[N - 1] = ApplyTMmixedRight(Bin[N - 1], AR[N - 1])
    for n in range(N - 1, 0, -1):
        ABR[n - 1] = ApplyTMmixedRight(mps_add(Bin[n - 1], mps_mul_bm(AL[n - 1], ABR[n])), AR[n - 1])
    # all unit cells to the right (:75-89), then per bond (:91-99): ABRtot[0] = kfac E,
    # ABRtot[n] = ABR[n] + kfac T_n...T_{N-1} E
    if proj:
        E, _ = InvertE_proj_fac(AL, AR, ABR[0], LM, RM, "r", kfac, tol, rng=rng)
    else:
        E, _ = InvertE_fac(AL, AR, ABR[0], "r", kfac, tol, rng=rng)
    ABRtot = [None] * N
    ABRtot[0] = bm_scale(E, kfac)
    for n in range(N - 1, 0, -1):
        E = ApplyTMmixedRightX(AL[n], AR[n], E)
        ABRtot[n] = bm_add(ABR[n], bm_scale(E, kfac))
    # H left of or on B within the unit cell, one step into the cell to the left (:104-115)
    HBL = [bm_add(ApplyTMmixedLeft(bd_mul_mps(HLtot[N - 1], Bin[0]), AL[0]),
                  ApplyOpTMLeftGen(hnnz, mps_add(mps_mul_mps(AL[N - 1], Bin[0]),
                                                 mps_scale(mps_mul_mps(Bin[N - 1], AR[0]), ck)),
                                   mps_mul_mps(AL[N - 1], AL[0])))]
    for n in range(1, N):
        HBL.append(bm_add(ApplyTMmixedLeft(mps_add(bm_mul_mps(HBL[-1], AR[n]), bd_mul_mps(HLtot[n - 1], Bin[n])),
                                           AL[n]),
                          ApplyOpTMLeftGen(hnnz, mps_add(mps_mul_mps(AL[n - 1], Bin[n]),
                                                         mps_mul_mps(Bin[n - 1], AR[n])),
                                           mps_mul_mps(AL[n - 1], AL[n]))))
    # all unit cells to the left (:118-132), then per bond (:134-140): HBLtot[n] = HBL[n] +
    # conj(kfac) T_n...T_0 E for n < N-1, HBLtot[N-1] = conj(kfac) E
    if proj:
        E, _ = InvertE_proj_fac(AR, AL, HBL[-1], bm_t(LM), bm_t(RM), "l", ck, tol, rng=rng)
    else:
        E, _ = InvertE_fac(AR, AL, HBL[-1], "l", ck, tol, rng=rng)
    HBLtot = [None] * N
    HBLtot[N - 1] = bm_scale(E, ck)
    for n in range(N - 1):
        E = ApplyTMmixedLeftX(AR[n], AL[n], E)
        HBLtot[n] = bm_add(HBL[n], bm_scale(E, ck))

    Bout = [mps_add(bd_mul_mps(HLtot[P(n - 1)], Bin[n]), mps_mul_bd(Bin[n], HRtot[P(n + 1)])) for n in range(N)]

    def contract(n, left2=None, right2=None, scale=1.0):
        """Bout[n][s] += scale * sum_k AL[n-1][k]^T left2[k*d+s] + sum_k right2[s*d+k] AR[n+1][k]^T."""
        for s_ in range(d):
            for k in range(d):
                if left2 is not None:
                    bm_iadd(Bout[n][s_], bm_scale(bm_mul(bm_t(AL[P(n - 1)][k]), left2[k * d + s_]), scale))
                if right2 is not None:
                    bm_iadd(Bout[n][s_], bm_mul(right2[s_ * d + k], bm_t(AR[P(n + 1)][k])))

    # h acting on B and the output site (:146-167)
    for n in range(N):
        contract(n, ApplyOperator(mps_mul_mps(AL[P(n - 1)], Bin[n]), hnnz),
                 ApplyOperator(mps_mul_mps(Bin[n], AR[P(n + 1)]), hnnz))
    # B left of the output site (:170-198)
    for n in range(N):
        for s_ in range(d):
            bm_iadd(Bout[n][s_], bm_mul(HBLtot[P(n - 1)], AR[n][s_]))
        contract(n, ApplyOperator(mps_mul_mps(Bin[P(n - 1)], AR[n]), hnnz), None, ck if n == 0 else 1.0)
    # B right of the output site (:203-224)
    for n in range(N):
        Atmp = mps_add(Bin[P(n + 1)], mps_mul_bm(AL[P(n + 1)], ABRtot[P(n + 2)]))
        if n == N - 1:
            Atmp = mps_scale(Atmp, kfac)
        ALABR = mps_mul_bm(AL[n], ABRtot[P(n + 1)])
        Bout[n] = mps_add(Bout[n], bd_mul_mps(HLtot[P(n - 1)], ALABR))
        contract(n, ApplyOperator(mps_mul_mps(AL[P(n - 1)], ALABR), hnnz),
                 ApplyOperator(mps_mul_mps(AL[n], Atmp), hnnz))
    # back to X (:227)
    return [ApplyTMmixedLeft(Bout[n], NL[n]) for n in range(N)]


def OPeffConstants(AL, AR, L, R, onnz, tol=1e-14, rng=None):
    """Excitations_helpers.hpp:548-606 for a one-site operator (its mean already subtracted):
    OPLtot[n] (left environment up to and including site n) and OPRtot[n] (right environment
    from site n on), the infinite parts closed by InvertE_proj."""
    N = len(AL)
    P = lambda x: (x + N) % N
    OPL = [ApplyOpTMLeftDiag(onnz, AL[0])]
    for n in range(1, N):
        OPL.append(bd_add(ApplyOpTMLeftDiag(onnz, AL[n]), ApplyTMLeft(AL[n], OPL[-1])))
    OPR = [None] * N
    OPR[N - 1] = ApplyOpTMRightDiag(onnz, AR[N - 1])
    for n in range(N - 2, -1, -1):
        OPR[n] = bd_add(ApplyOpTMRightDiag(onnz, AR[n]), ApplyTMRight(AR[n], OPR[n + 1]))
    OPLtot, OPRtot = [None] * N, [None] * N
    EOPL = [None] * N
    EOPL[N - 1], _ = InvertE_proj(AL, OPL[N - 1], bd_eye({q: M.shape[1] for q, M in R.items()}), R, "l", tol,
                                  rng=rng)
    OPLtot[N - 1] = EOPL[N - 1]
    for n in range(N - 1):
        EOPL[n] = ApplyTMLeft(AL[n], EOPL[P(n - 1)])
        OPLtot[n] = bd_add(OPL[n], EOPL[n])
    EOPR = [None] * N
    EOPR[0], _ = InvertE_proj(AR, OPR[0], L, bd_eye({q: M.shape[1] for q, M in L.items()}), "r", tol, rng=rng)
    OPRtot[0] = EOPR[0]
    for n in range(N - 1, 0, -1):
        EOPR[n] = ApplyTMRight(AR[n], EOPR[P(n + 1)])
        OPRtot[n] = bd_add(EOPR[n], OPR[n])
    return OPLtot, OPRtot


def ApplyOPeff(Xin, kfac, AL, AR, NL, onnz, OPLtot, OPRtot, LM=None, RM=None, tol=1e-14, rng=None):
    """Excitations_helpers.hpp:350-545: the one-site operator sum_n O_n of the excitation ansatz
    applied to X, as the reference writes it (B on, left of and right of the output site, the
    infinite sums closed by InvertE_fac / InvertE_proj_fac; the left solve skipped when its
    source is below 10 tol, :478)."""
    N = len(Xin)
    ck = np.conj(kfac)
    P = lambda x: (x + N) % N
    proj = LM is not None and RM is not None
    Bin = [mps_mul_bm(NL[n], Xin[n]) for n in range(N)]
    ABR = [None] * N
    ABR[N - 1] = ApplyTMmixedRight(Bin[N - 1], AR[N - 1])
    for n in range(N - 1, 0, -1):
        ABR[n - 1] = ApplyTMmixedRight(mps_add(Bin[n - 1], mps_mul_bm(AL[n - 1], ABR[n])), AR[n - 1])
    if proj:
        E, _ = InvertE_proj_fac(AL, AR, ABR[0], LM, RM, "r", kfac, tol, rng=rng)
    else:
        E, _ = InvertE_fac(AL, AR, ABR[0], "r", kfac, tol, rng=rng)
    ABRtot = [None] * N
    ABRtot[0] = bm_scale(E, kfac)
    for n in range(N - 1, 0, -1):
        E = ApplyTMmixedRightX(AL[n], AR[n], E)
        ABRtot[n] = bm_add(ABR[n], bm_scale(E, kfac))
    OPBL = [bm_add(ApplyTMmixedLeft(bd_mul_mps(OPLtot[N - 1], Bin[0]), AL[0]), ApplyOpTMLeftGen(onnz, Bin[0], AL[0]))]
    for n in range(1, N):
        OPBL.append(bm_add(ApplyTMmixedLeft(mps_add(bm_mul_mps(OPBL[-1], AR[n]), bd_mul_mps(OPLtot[n - 1], Bin[n])),
                                            AL[n]),
                           ApplyOpTMLeftGen(onnz, Bin[n], AL[n])))
    norm_inf = max((float(np.abs(M).max()) for (_, M) in OPBL[-1].values() if M.size), default=0.0)
    have = norm_inf > 10 * tol
    if have:
        if proj:
            EOP, _ = InvertE_proj_fac(AR, AL, OPBL[-1], bm_t(LM), bm_t(RM), "l", ck, tol, rng=rng)
        else:
            EOP, _ = InvertE_fac(AR, AL, OPBL[-1], "l", ck, tol, rng=rng)
    Bout = [mps_add(mps_add(bd_mul_mps(OPLtot[P(n - 1)], Bin[n]), mps_mul_bd(Bin[n], OPRtot[P(n + 1)])),
                    ApplyOperator(Bin[n], onnz)) for n in range(N)]
    if have:
        Bout[0] = mps_add(Bout[0], bm_mul_mps(bm_scale(EOP, ck), AR[0]))
    for n in range(1, N):
        tmp = OPBL[n - 1]
        if have:
            EOP = ApplyTMmixedLeftX(AR[n - 1], AL[n - 1], EOP)
            tmp = bm_add(tmp, bm_scale(EOP, ck))
        Bout[n] = mps_add(Bout[n], bm_mul_mps(tmp, AR[n]))
    for n in range(N):
        Bout[n] = mps_add(Bout[n], mps_add(mps_mul_bm(bd_mul_mps(OPLtot[P(n - 1)], AL[n]), ABRtot[P(n + 1)]),
                                          mps_mul_bm(ApplyOperator(AL[n], onnz), ABRtot[P(n + 1)])))
    return [ApplyTMmixedLeft(Bout[n], NL[n]) for n in range(N)]


def ApplyOperator(A, hnnz):
    """MPSBlockUtilities.hpp:17-34: out[ii] += h * in[jj]."""
    out = [dict() for _ in A]
    for (r, c, h) in hnnz:
        bm_iadd(out[r], bm_scale(A[c], h))
    return out


def ApplyOpTMLeftDiag(hnnz, A):
    """TMBlockFunctions.hpp:797-802."""
    return ApplyTMmixedLeftDiag(ApplyOperator(A, hnnz), A)


def ApplyOpTMRightDiag(hnnz, A):
    """TMBlockFunctions.hpp:831-836."""
    return ApplyTMmixedRightDiag(ApplyOperator(A, hnnz), A)


def ReducedOp(hnnz, A, d, direction):
    """MPSBlockUtilities.hpp:37-74."""
    Ored = [[dict() for _ in range(d)] for _ in range(d)]
    for (r, c, h) in hnnz:
        i0, i1 = num2ditvec(r, d)
        j0, j1 = num2ditvec(c, d)
        if direction == "r":
            term = bm_scale(bm_mul(A[j1], bm_t(A[i1])), h)
            bm_iadd(Ored[i0][j0], term)
        else:
            term = bm_scale(bm_mul(bm_t(A[i0]), A[j0]), h)
            bm_iadd(Ored[i1][j1], term)
    return Ored


def GetHL(ALvec, hnnz):
    """VUMPS_helpers.hpp:3-18."""
    HL = ApplyOpTMLeftDiag(hnnz, mps_mul_mps(ALvec[-1], ALvec[0]))
    for k in range(1, len(ALvec)):
        HL = bd_add(ApplyTMLeft(ALvec[k], HL), ApplyOpTMLeftDiag(hnnz, mps_mul_mps(ALvec[k - 1], ALvec[k])))
    return HL


def GetHR(ARvec, hnnz):
    """VUMPS_helpers.hpp:20-36."""
    N = len(ARvec)
    HR = ApplyOpTMRightDiag(hnnz, mps_mul_mps(ARvec[-1], ARvec[0]))
    for k in range(N - 2, -1, -1):
        HR = bd_add(ApplyTMRight(ARvec[k], HR), ApplyOpTMRightDiag(hnnz, mps_mul_mps(ARvec[k], ARvec[k + 1])))
    return HR


# ----------------------------------------------------------------------------------------------
# GMRES (IterativeSolvers.hpp:21-150) and environment solves (InvEBlockFunctions.hpp)
# ----------------------------------------------------------------------------------------------


def gmres(Afun, b, x0, tol, maxit, krylovdim=0):
    """Unrestarted GMRES exactly as IterativeSolvers.hpp:21-150 (MGS, Givens, |r| < tol*|b|).
    Returns (x, flag)."""
    dim = b.size
    cplx = np.iscomplexobj(b) or np.iscomplexobj(x0)
    T = np.complex128 if cplx else np.float64
    if maxit > dim:
        maxit = dim
    if krylovdim == 0:
        krylovdim = min(dim, maxit)
    krylovdim = min(krylovdim, dim)
    flag = -1
    r0 = b - Afun(x0)
    x = x0.astype(T).copy()
    bnorm = np.linalg.norm(b)
    rnorm = np.linalg.norm(r0)
    thresh = 2e-16
    # storage grows with the iteration count (the reference allocates dim x (krylovdim+1)
    # uninitialised, which only touches the columns it uses)
    V = [r0.astype(T) / rnorm]
    Hcols = []
    c, s = [], []
    gamma = [T(rnorm)]
    kdim = 0
    for j in range(krylovdim):
        w = Afun(V[j]).astype(T)
        h = np.zeros(j + 2, T)
        for i in range(j + 1):
            h[i] = np.vdot(V[i], w)
            w = w - h[i] * V[i]
        h[j + 1] = np.linalg.norm(w)
        for i in range(j):
            h1, h2 = h[i], h[i + 1]
            h[i] = c[i] * h1 + s[i] * h2
            h[i + 1] = -np.conj(s[i]) * h1 + c[i] * h2
        beta = np.linalg.norm(h[j:j + 2])
        if abs(beta) < thresh:
            flag = -2
            break
        V.append(w / h[j + 1])
        habs = abs(h[j])
        phase = h[j] / habs
        s.append(phase * np.conj(h[j + 1]) / beta)
        c.append(habs / beta)
        h[j] = phase * beta
        h[j + 1] = 0
        gamma.append(-np.conj(s[j]) * gamma[j])
        gamma[j] *= c[j]
        Hcols.append(h)
        kdim += 1
        rnorm = abs(gamma[j + 1])
        if rnorm < tol * bnorm:
            flag = kdim
            break
    if kdim:
        from scipy.linalg import solve_triangular
        Hk = np.zeros((kdim, kdim), T)
        for jj in range(kdim):
            Hk[:jj + 1, jj] = Hcols[jj][:jj + 1]
        alpha = solve_triangular(Hk, np.asarray(gamma[:kdim], T), lower=False)
        x = x + np.stack(V[:kdim], axis=1) @ alpha
    return x, flag


def InvEfun_proj(invec, TMfun, rho_inside, rho_outside, dims):
    """InvEBlockFunctions.hpp:12-47: y = x - TM(x) + trace(x*rho_in) * rho_out."""
    X = bd_from_vec(invec, dims)
    tr = sum(np.trace(X[q] @ rho_inside[q]) for q, _ in dims)
    Tx = TMfun(X)
    Y = {q: X[q] + tr * rho_outside[q] - Tx[q] for q, _ in dims}
    return bd_vec(Y)


def InvertE_proj(MPSarr, x, L, R, direction, tol=1e-14, maxit=0, y0=None, rng=None):
    """InvEBlockFunctions.hpp:201-266 for BlockDiagMat x on a unit cell."""
    dims = bd_sizes(x)
    m_tot = sum(m * m for _, m in dims)
    if maxit == 0:
        maxit = m_tot
    if y0 is None or bd_sizes(y0) != dims:
        rng = rng or np.random.default_rng(0)
        y0 = {q: rng.standard_normal((m, m)) for q, m in dims}
    xpv = bd_vec(x)
    if direction == "l":
        xpv = xpv - bd_trace(bd_mul(x, R)) * bd_vec(L)
        Afun = lambda v: InvEfun_proj(v, lambda X: ApplyTMLeftUC(MPSarr, X), R, L, dims)
    else:
        xpv = xpv - bd_trace(bd_mul(L, x)) * bd_vec(R)
        Afun = lambda v: InvEfun_proj(v, lambda X: ApplyTMRightUC(MPSarr, X), L, R, dims)
    y, flag = gmres(Afun, xpv, bd_vec(y0), tol, maxit)
    return bd_from_vec(y, dims), flag


# ----------------------------------------------------------------------------------------------
# eigensolvers: ARPACK as shipped in scipy stands in for eigs.cpp (eigs_rs / eigs_n)
# ----------------------------------------------------------------------------------------------


def eigs_rs(fun, N, tol, x0, nev=1, which="SA"):
    """eigs.cpp:369-494: dsaupd/dseupd with ncv = min(max(20, 2 nev), N), maxit = N."""
    from scipy.sparse.linalg import LinearOperator, eigsh
    ncv = min(max(20, 2 * nev), N)
    op = LinearOperator((N, N), matvec=lambda v: fun(np.asarray(v).ravel()), dtype=np.float64)
    vals, vecs = eigsh(op, k=nev, which=which, tol=tol, v0=x0, ncv=ncv, maxiter=N)
    order = np.argsort(vals)
    return vals[order], vecs[:, order]


def TMDominantEig(MPSarr, dims, direction, tol=1e-14, x0=None):
    """EigsBlockFunctions.hpp:91-172 (eigs_n "LR", nev=1), normalised by its trace."""
    from scipy.sparse.linalg import LinearOperator, eigs
    sizes = sorted(dims.items())
    D_tot = sum(m * m for _, m in sizes)
    if direction == "l":
        f = lambda v: bd_vec(ApplyTMLeftUC(MPSarr, bd_from_vec(v, sizes)))
    else:
        f = lambda v: bd_vec(ApplyTMRightUC(MPSarr, bd_from_vec(v, sizes)))
    op = LinearOperator((D_tot, D_tot), matvec=lambda v: f(np.real(np.asarray(v).ravel())), dtype=np.float64)
    v0 = bd_vec(x0) if x0 is not None else None
    vals, vecs = eigs(op, k=1, which="LR", tol=tol, v0=v0, ncv=min(20, D_tot), maxiter=D_tot)
    V = bd_from_vec(np.real(vecs[:, 0]), sizes)
    tr = bd_trace(V)
    V = {q: M / tr for q, M in V.items()}
    return float(np.real(vals[0])), V


def mps_ml(A):
    """MPSBlockMat::GetMl (MPSBlockMat.hpp:281-304): left charge -> left dimension over all s."""
    out = {}
    for bm in A:
        for qi, (qo, M) in bm.items():
            out.setdefault(qi, M.shape[0])
    return out


def mps_mr(A):
    """MPSBlockMat::GetMr (MPSBlockMat.hpp:306-323)."""
    out = {}
    for bm in A:
        for qi, (qo, M) in bm.items():
            out.setdefault(qo, M.shape[1])
    return out


def eigs_n(fun, N, nev, which="LM", tol=1e-14, x0=None, ncv=0, maxit=0):
    """eigs.cpp:193-342: dnaupd/dneupd (real nonsymmetric) with ncv = min(max(20, 2 nev + 1), N)
    and maxit = N; returns (complex eigenvalues, complex eigenvectors as columns)."""
    from scipy.sparse.linalg import LinearOperator, eigs
    if ncv <= 0:
        ncv = min(max(20, 2 * nev + 1), N)
    maxit = N if maxit <= 0 else min(maxit, N)
    op = LinearOperator((N, N), matvec=lambda v: fun(np.real(np.asarray(v).ravel())), dtype=np.float64)
    if x0 is None:
        x0 = np.random.default_rng(0).standard_normal(N)  # eigs.cpp: RESID = randn
    return eigs(op, k=nev, which=which, tol=tol, v0=x0, ncv=ncv, maxiter=maxit)


def TMmixedEigs(A, B, direction, K, nev, mode="LM", tol=1e-14, x0=None):
    """EigsBlockFunctions.hpp:282-391: the nev leading eigenpairs of the mixed unit-cell TM in the
    charge sector K.  Sectors (q, q + K) for q in diml with q + K in dimr, where diml, dimr =
    GetMl of A, B (swapped for dir l); TMMult over the vectorisation; eigs_n, then sorted by
    |lambda| (LM) or Re lambda (LR) descending.  Returns (vals, [complex BlockMats])."""
    if mode not in ("LM", "LR"):
        raise ValueError("TMmixedEigs: wrong mode " + mode)
    diml, dimr = mps_ml(A[0]), mps_ml(B[0])
    if mps_mr(A[-1]) != diml or mps_mr(B[-1]) != dimr:
        raise ValueError("left and right end of A, B need to have same dimensions")
    if direction == "l":
        diml, dimr = dimr, diml
    sizes = [(q, kadd(q, K), diml[q], dimr[kadd(q, K)]) for q in sorted(diml) if kadd(q, K) in dimr]
    if not sizes:
        raise ValueError("TMmixedEigs: no TM eigenvalues for this quantum number")
    D_tot = sum(ml * mr for (_, _, ml, mr) in sizes)
    if direction == "l":
        f = lambda v: bm_vec(ApplyTMmixedLeftUC(A, B, bm_from_vec(v, sizes)))
    else:
        f = lambda v: bm_vec(ApplyTMmixedRightUC(A, B, bm_from_vec(v, sizes)))
    v0 = bm_vec(x0) if x0 is not None and bm_sizes(x0) == sizes else None
    vals, vecs = eigs_n(f, D_tot, nev, mode, tol, v0)
    order = np.argsort(-np.abs(vals), kind="stable") if mode == "LM" else np.argsort(-vals.real, kind="stable")
    vals, vecs = vals[order], vecs[:, order]
    V = [bm_from_vec(vecs[:, i], sizes) for i in range(len(vals))]
    return vals, V, sizes


def bm_real(X):
    """BlockMat<KT,Real>(BlockMat<KT,Complex>) (BlockObj.hpp:612-629): the real part."""
    return {qi: (qo, np.real(M).copy()) for qi, (qo, M) in X.items()}


def LRoverlaps(AL, AR, K, nev, OLtol=1e-14):
    """Excitations_helpers.hpp:915-946: the dominant left (charge -K) and right (charge K)
    eigenmatrices LM, RM of the mixed TMs of AL and AR (real parts) and the overlap
    OL = (Re OL_L + Re OL_R) / 2.  Returns (LM, RM, OL, OLLv, OLRv)."""
    OLLv, VL, _ = TMmixedEigs(AL, AR, "l", tuple(-k for k in K), nev, "LM", OLtol)
    OLRv, VR, _ = TMmixedEigs(AL, AR, "r", tuple(K), nev, "LM", OLtol)
    LM, RM = bm_real(VL[0]), bm_real(VR[0])
    return LM, RM, 0.5 * (OLLv[0].real + OLRv[0].real), OLLv, OLRv


# ----------------------------------------------------------------------------------------------
# energy density of a uniform two-site MPS and its gradient (adjoint check).  The reference has
# no gradient of its own beyond the tangent-space residual H_AC AC - AL H_C C
# (VUMPS_helpers.hpp:135-177); these restate the energy of MeasureObservables
# (MPSBlockUtilities.hpp:1017-1091) for a general, non-isometric unit cell and differentiate it.
# ----------------------------------------------------------------------------------------------


def bd_dot(X, Y):
    """(X|Y) = sum_q tr(X_q^T Y_q)."""
    return float(sum(np.sum(X[q] * Y[q]) for q in X if q in Y))


def bd_scale(X, a):
    return {q: a * M for q, M in X.items()}


def mps_dot(A, B):
    return float(sum(np.sum(M * B[s][qi][1]) for s, bm in enumerate(A) for qi, (qo, M) in bm.items()
                     if qi in B[s]))


def opTM_left(A0, A1, l, hnnz):
    """sum_st (A0 A1)_st^T l (h A0 A1)_st: the two-site term E(l) carried from bond 0 to bond 2."""
    AA = mps_mul_mps(A0, A1)
    HA = ApplyOperator(AA, hnnz)
    out = {}
    for a, b in zip(AA, HA):
        for qi, (qo, M) in a.items():
            if qi in b and qi in l:
                c = M.T @ l[qi] @ b[qi][1]
                out[qo] = out[qo] + c if qo in out else c
    return out


def opTM_right(A0, A1, r, hnnz):
    """sum_st (h A0 A1)_st r (A0 A1)_st^T: the two-site term carried from bond 2 to bond 0."""
    AA = mps_mul_mps(A0, A1)
    HA = ApplyOperator(AA, hnnz)
    out = {}
    for a, b in zip(AA, HA):
        for qi, (qo, M) in a.items():
            if qi in b and qo in r:
                c = b[qi][1] @ r[qo] @ M.T
                out[qi] = out[qi] + c if qi in out else c
    return out


def _dense_map(f, sizes):
    n = sum(m * m for _, m in sizes)
    M = np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        M[:, i] = bd_vec(f(bd_from_vec(e, sizes)))
    return M


def energy_uniform(A, hnnz):
    """Energy density of the uniform MPS of the unit cell A = [A0, A1] (any, not necessarily
    isometric): e = (N0 / lam + N1 / lam^2) / (2 (l|r)) with lam, l, r the dominant eigenvalue and
    fixed points of the unit-cell TM (dense eigendecomposition: small bonds only), N0 the bond
    (0,1) term between l and r, N1 the bond (1,2) term between l1 = T_0(l) and r1 = T~_1(r)."""
    A0, A1 = A
    sizes = sorted(mps_ml(A0).items())
    w, V = np.linalg.eig(_dense_map(lambda X: ApplyTMLeftUC(A, X), sizes))
    i = int(np.argmax(w.real))
    lam = float(w[i].real)
    l = bd_from_vec(np.real(V[:, i]), sizes)
    w2, V2 = np.linalg.eig(_dense_map(lambda X: ApplyTMRightUC(A, X), sizes))
    r = bd_from_vec(np.real(V2[:, int(np.argmax(w2.real))]), sizes)
    l1, r1 = ApplyTMLeft(A0, l), ApplyTMRight(A1, r)
    N0 = bd_dot(l, opTM_right(A0, A1, r, hnnz))
    N1 = bd_dot(l1, opTM_right(A1, A0, r1, hnnz))
    return (N0 / lam + N1 / lam ** 2) / (2.0 * bd_dot(l, r))


def _redop_env(A, env, hnnz, d, direction):
    """ReducedOp (MPSBlockUtilities.hpp:37-74) with an environment inserted, as BlockMats (a pair
    i0 != j0 carries a charge offset): direction "r" gives W[i0][j0] = sum h_(i0 i1),(j0 j1)
    A[j1] env A[i1]^T, "l" gives V[i1][j1] = sum h A[i0]^T env A[j0]."""
    W = [[None] * d for _ in range(d)]
    for (rr, cc, h) in hnnz:
        i0, i1 = num2ditvec(rr, d)
        j0, j1 = num2ditvec(cc, d)
        if direction == "r":
            c, a, b = bm_mul(bm_mul_bd(A[j1], env), bm_t(A[i1])), i0, j0
        else:
            c, a, b = bm_mul(bm_mul_bd(bm_t(A[i0]), env), A[j0]), i1, j1
        W[a][b] = bm_iadd(W[a][b] if W[a][b] is not None else {}, bm_scale(c, h))
    return W


def invert_e_proj_scipy(MPSarr, x, L, R, direction, tol=1e-14):
    """The projected system of InvertE_proj (InvEBlockFunctions.hpp:201-266) solved with scipy's
    restarted GMRES: test infrastructure for bonds where the restated unrestarted GMRES is slow."""
    from scipy.sparse.linalg import LinearOperator, gmres as sp_gmres
    dims = bd_sizes(x)
    n = sum(m * m for _, m in dims)
    if direction == "l":
        b = bd_vec(x) - bd_trace(bd_mul(x, R)) * bd_vec(L)
        f = lambda v: InvEfun_proj(v, lambda X: ApplyTMLeftUC(MPSarr, X), R, L, dims)
    else:
        b = bd_vec(x) - bd_trace(bd_mul(L, x)) * bd_vec(R)
        f = lambda v: InvEfun_proj(v, lambda X: ApplyTMRightUC(MPSarr, X), L, R, dims)
    op = LinearOperator((n, n), matvec=lambda v: f(np.asarray(v).ravel()), dtype=np.float64)
    y, info = sp_gmres(op, b, rtol=tol, atol=0.0, restart=120, maxiter=200)
    return bd_from_vec(y, dims), info


def energy_gradient(AL, R, hnnz, tol=1e-14, solver=None):
    """Gradient of energy_uniform with respect to every entry of a left-isometric unit cell AL
    (lam = 1, l = l1 = 1, r = R with tr R = 1), by the adjoint method:
      * direct two-site terms: H_AC-type contractions with the ReducedOp environments W, V, W', V';
      * the dependence of r1 = T~_1(r) and l1 = T_0(l) on A (TM adjoints: left TM
        (Y|dT(X)) -> X A Y^T + X^T A Y, right TM (Y|dT~(X)) -> Y A X^T + Y^T A X);
      * the eigenvalue, dlam = (r1|dT_0(l)) + (r|dT_1(l1)), weighted by -(N0 + 2 N1) / 2;
      * the fixed points through the implicit function theorem: g_l = de/dl, g_r = de/dr (both
        orthogonal to the null directions by scale invariance), z_l = (1 - T~ + |r)(l|)^-1 (-g_l)
        and z_r = (1 - T + |l)(r|)^-1 (-g_r): GMRES on the transposed transfer matrices
        (InvertE_proj with the roles of the two directions exchanged), then
        -(z_l|dT(l)) - (z_r|dT~(r)) through the TM adjoints.
    solver: optional replacement of InvertE_proj with the same signature (a faster library
    GMRES for large bonds; the solution of the projected system does not depend on it).
    Returns ([G0, G1] as MPS structures, e)."""
    A0, A1 = AL
    d = len(A0)
    I0, I1 = bd_eye(mps_ml(A0)), bd_eye(mps_ml(A1))
    r = bd_scale(R, 1.0 / bd_trace(R))
    r1 = ApplyTMRight(A1, r)
    N0 = bd_dot(I0, opTM_right(A0, A1, r, hnnz))
    N1 = bd_dot(I1, opTM_right(A1, A0, r1, hnnz))
    E2, E2l = N0 + N1, N0 + 2.0 * N1
    Et1 = opTM_right(A1, A0, r1, hnnz)          # bond 1
    E1l = opTM_left(A1, A0, I1, hnnz)           # bond 1
    gl = bd_scale(bd_add(bd_add(opTM_right(A0, A1, r, hnnz), ApplyTMRight(A0, Et1)), bd_scale(r, -E2)), 0.5)
    gr = bd_scale(bd_add(bd_add(opTM_left(A0, A1, I0, hnnz), ApplyTMLeft(A1, E1l)), bd_scale(I0, -E2)), 0.5)
    solve = solver or InvertE_proj
    zl, _ = solve(AL, bd_scale(gl, -1.0), I0, r, "r", tol)
    zr, _ = solve(AL, bd_scale(gr, -1.0), I0, r, "l", tol)
    W = _redop_env(A1, r, hnnz, d, "r")    # bond 1
    V = _redop_env(A0, I0, hnnz, d, "l")   # bond 1
    Wp = _redop_env(A0, r1, hnnz, d, "r")  # bond 0 (= 2)
    Vp = _redop_env(A1, I1, hnnz, d, "l")  # bond 0 (= 2)
    T1zl = ApplyTMRight(A1, zl)            # bond 1
    T0zr = ApplyTMLeft(A0, zr)             # bond 1
    G0, G1 = [], []
    for s in range(d):
        g = {}
        for sp in range(d):
            if W[s][sp] is not None:
                bm_iadd(g, bm_mul(A0[sp], W[s][sp]))
            if Vp[s][sp] is not None:
                bm_iadd(g, bm_mul_bd(bm_mul(Vp[s][sp], A0[sp]), r1))
        Y1 = bd_add(bd_add(Et1, bd_scale(r1, -E2l)), bd_scale(T1zl, -2.0))
        bm_iadd(g, bm_mul_bd(A0[s], Y1))
        bm_iadd(g, bm_scale(bm_mul_bd(bd_mul_bm(zr, A0[s]), r1), -2.0))
        G0.append(g)
    for t in range(d):
        g = {}
        for tp in range(d):
            if V[t][tp] is not None:
                bm_iadd(g, bm_mul_bd(bm_mul(V[t][tp], A1[tp]), r))
            if Wp[t][tp] is not None:
                bm_iadd(g, bm_mul(A1[tp], Wp[t][tp]))
        bm_iadd(g, bm_mul_bd(bd_mul_bm(bd_add(E1l, bd_scale(T0zr, -2.0)), A1[t]), r))
        bm_iadd(g, bm_mul_bd(A1[t], bd_add(bd_scale(r, -E2l), bd_scale(zl, -2.0))))
        G1.append(g)
    return [G0, G1], 0.5 * E2


# ----------------------------------------------------------------------------------------------
# per-sector decompositions (helpers.hpp:181-195, MPSBlockUtilities.hpp:78-340, BlockObj.hpp:2422-2541)
# ----------------------------------------------------------------------------------------------


def qr_pos(X):
    """qr_econ + sign fix so that diag(R) >= 0 (helpers.hpp:181-195)."""
    Q, R = np.linalg.qr(X, mode="reduced")
    sg = np.where(np.diag(R) < 0, -1.0, 1.0)
    return Q * sg[None, :], R * sg[:, None]


def GetDenseMat(A, direction):
    """MPSBlockMat::GetDenseMat (MPSBlockMat.hpp:468-526) + GetSingleSecData (:636-719).
    Returns {sector: (dense, [(s, other_key, start, size)], ml_tot, mr_tot)}."""
    d = len(A)
    secs = {}
    if direction == "l":
        for s in range(d):
            for qi in sorted(A[s]):
                qo, M = A[s][qi]
                secs.setdefault(qo, {"mr": M.shape[1], "parts": {}})["parts"][s] = (qi, M)
        out = {}
        for qo in sorted(secs):
            parts = secs[qo]["parts"]
            rows, spans, pos = [], [], 0
            for s in sorted(parts):
                qi, M = parts[s]
                rows.append(M)
                spans.append((s, qi, pos, M.shape[0]))
                pos += M.shape[0]
            out[qo] = (np.vstack(rows), spans, pos, secs[qo]["mr"])
        return out
    for s in range(d):
        for qi in sorted(A[s]):
            qo, M = A[s][qi]
            secs.setdefault(qi, {"ml": M.shape[0], "parts": {}})["parts"][s] = (qo, M)
    out = {}
    for qi in sorted(secs):
        parts = secs[qi]["parts"]
        cols, spans, pos = [], [], 0
        for s in sorted(parts):
            qo, M = parts[s]
            cols.append(M)
            spans.append((s, qo, pos, M.shape[1]))
            pos += M.shape[1]
        out[qi] = (np.hstack(cols), spans, secs[qi]["ml"], pos)
    return out


def qr_mps(A, direction):
    """qr(R, MPS, dir) (MPSBlockUtilities.hpp:181-244): returns (Q MPS, R BlockDiag)."""
    d = len(A)
    Q = [dict() for _ in range(d)]
    R = {}
    for q, (M, spans, _, _) in GetDenseMat(A, direction).items():
        if direction == "l":
            Qm, Rm = qr_pos(M)
            R[q] = Rm
            for (s, qo, st, sz) in spans:
                Q[s][qo] = (q, Qm[st:st + sz, :].copy())
        else:
            Qm, Rm = qr_pos(M.T)
            R[q] = Rm.T.copy()
            for (s, qo, st, sz) in spans:
                Q[s][q] = (qo, Qm[st:st + sz, :].T.copy())
    return Q, R


def qr_bd(X, direction):
    """qr(R, BlockDiagMat, dir) (BlockObj.hpp:2422-2459): returns (Q, R)."""
    Q, R = {}, {}
    for q in sorted(X):
        if direction == "l":
            Q[q], R[q] = qr_pos(X[q])
        else:
            Qt, Rt = qr_pos(X[q].T)
            Q[q], R[q] = Qt.T.copy(), Rt.T.copy()
    return Q, R


def svd_mps(A, direction):
    """svd(S, DiagIso, MPS, dir) (MPSBlockUtilities.hpp:78-153): returns (MPSIso, S, DiagIso)."""
    d = len(A)
    Iso = [dict() for _ in range(d)]
    S, DI = {}, {}
    for q, (M, spans, _, _) in GetDenseMat(A, direction).items():
        U, sv, Vt = np.linalg.svd(M, full_matrices=False)
        S[q] = sv
        if direction == "l":
            DI[q] = Vt.copy()
            for (s, qo, st, sz) in spans:
                Iso[s][qo] = (q, U[st:st + sz, :].copy())
        else:
            DI[q] = U.copy()
            for (s, qo, st, sz) in spans:
                Iso[s][q] = (qo, Vt[:, st:st + sz].copy())
    return Iso, S, DI


def svd_bd(X):
    return {q: np.linalg.svd(X[q], compute_uv=False) for q in sorted(X)}


def Nullspace(A, direction):
    """MPSBlockUtilities.hpp:247-340 (sectors without a null space are omitted)."""
    from scipy.linalg import null_space
    d = len(A)
    NS = [dict() for _ in range(d)]
    for q, (M, spans, ml_tot, mr_tot) in GetDenseMat(A, direction).items():
        if direction == "l":
            if ml_tot > mr_tot:
                B = null_space(M.T)
                for (s, qo, st, sz) in spans:
                    NS[s][qo] = (q, B[st:st + sz, :].copy())
        else:
            if mr_tot > ml_tot:
                B = null_space(M)
                for (s, qo, st, sz) in spans:
                    NS[s][q] = (qo, B[st:st + sz, :].T.copy())
    return NS


def GetDenseSplitMat(phi, I2K):
    """MPSBlockMat::GetDenseSplitMat / GetDoubleSecData (MPSBlockMat.hpp:533-620) for a two-site
    tensor phi[sl*d + sr]: per centre charge c = ql + I2K[sl], the dense matrix with row spans
    per left physical index sl (its block ql = c - I2K[sl]) and column spans per right index sr,
    both in increasing index order.  Returns {c: (dense, [(sl, ql, start, rows)],
    [(sr, qr, start, cols)])}."""
    d = len(I2K)
    secs = {}
    for s, bm in enumerate(phi):
        sl, sr = divmod(s, d)
        for ql, (qr, M) in bm.items():
            c = kadd(ql, I2K[sl])
            e = secs.setdefault(c, {"left": {}, "right": {}, "blocks": []})
            e["left"][sl] = (ql, M.shape[0])
            e["right"][sr] = (qr, M.shape[1])
            e["blocks"].append((sl, sr, M))
    out = {}
    for c in sorted(secs):
        e = secs[c]
        lsp, rsp, pos = {}, {}, 0
        for sl in sorted(e["left"]):
            ql, m = e["left"][sl]
            lsp[sl] = (ql, pos, m)
            pos += m
        ml = pos
        pos = 0
        for sr in sorted(e["right"]):
            qr, m = e["right"][sr]
            rsp[sr] = (qr, pos, m)
            pos += m
        D = np.zeros((ml, pos))
        for sl, sr, M in e["blocks"]:
            _, r0, rm = lsp[sl]
            _, c0, cm = rsp[sr]
            D[r0:r0 + rm, c0:c0 + cm] = M
        out[c] = (D, [(sl, q, a, m) for sl, (q, a, m) in sorted(lsp.items())],
                  [(sr, q, a, m) for sr, (q, a, m) in sorted(rsp.items())])
    return out


def ExpandFromH(hnnz, I2K, AL, AR, C, dmmax):
    """ExpandFromH (MPSBlockUtilities.hpp:409-601): grow the bond between AL and AR by the
    dominant directions of H acting on AL C AR outside the current tangent space.

    phi = ApplyOperator(AL C AR, H); for every centre charge c already on the bond, the
    projection M[c] = sum_{sl,sr} NL[sl]^T phi[sl,sr] NR[sr]^T onto the null spaces (skipped
    if either null space is empty); for a charge not yet on the bond, the whole dense block of
    phi.  The singular values of all M[c] compete for dmmax new states (largest first; ties
    keep charge order, the reference's std::sort leaves their order unspecified).  New
    columns NL U (or U for a new charge) are appended to AL, new rows V^T NR (or V^T) to AR,
    and C is padded with zeros, so AL C AR is unchanged.  Returns (AL, AR, C, dm) with dm =
    {c: states added} for every charge considered."""
    d = len(I2K)
    phi = ApplyOperator(mps_mul_mps(mps_mul_bd(AL, C), AR), hnnz)
    dense = GetDenseSplitMat(phi, I2K)
    NL = Nullspace(AL, "l")
    NR = Nullspace(AR, "r")
    M = {}
    for sl in range(d):
        for sr in range(d):
            for ql, (qr, P) in phi[sl * d + sr].items():
                if ql not in NL[sl]:
                    continue
                c, nl = NL[sl][ql]
                if c not in NR[sr]:
                    continue
                qr2, nr = NR[sr][c]
                assert qr2 == qr
                M[c] = M.get(c, 0.0) + nl.T @ P @ nr.T
    svds = []
    for c, (D, lsp, rsp) in dense.items():
        isnew = c not in C
        if isnew:
            X = D
        elif c in M:
            X = M[c]
        else:
            continue  # no null space on one side: the sector is already full rank
        U, lam, Vt = np.linalg.svd(X, full_matrices=False)
        svds.append({"c": c, "new": isnew, "U": U, "lam": lam, "V": Vt.T, "lsp": lsp, "rsp": rsp, "dm": 0})
    dmtot = sum(len(e["lam"]) for e in svds)
    if dmtot > dmmax:
        allv = [(-float(x), i) for i, e in enumerate(svds) for x in e["lam"]]
        for _, i in sorted(allv, key=lambda t: t[0])[:dmmax]:
            svds[i]["dm"] += 1
    else:
        for e in svds:
            e["dm"] = len(e["lam"])
    AL = [dict(bm) for bm in AL]
    AR = [dict(bm) for bm in AR]
    C = dict(C)
    dm = {}
    for e in svds:
        c, k = e["c"], e["dm"]
        dm[c] = k
        if k == 0:
            continue
        m0 = C[c].shape[0] if c in C else 0
        Cn = np.zeros((m0 + k, m0 + k))
        if m0:
            Cn[:m0, :m0] = C[c]
        C[c] = Cn
        U, V = e["U"][:, :k], e["V"][:, :k]
        if e["new"]:
            for (sl, ql, r0, m) in e["lsp"]:
                AL[sl][ql] = (c, U[r0:r0 + m, :].copy())
            for (sr, qr, c0, m) in e["rsp"]:
                AR[sr][c] = (qr, V[c0:c0 + m, :].T.copy())
        else:
            for sl in range(d):
                for ql, (c2, nl) in NL[sl].items():
                    if c2 == c:
                        q2, A0 = AL[sl][ql]
                        AL[sl][ql] = (c, np.hstack([A0, nl @ U]))
            for sr in range(d):
                if c in NR[sr]:
                    qr, nr = NR[sr][c]
                    q2, A0 = AR[sr][c]
                    AR[sr][c] = (qr, np.vstack([A0, V.T @ nr]))
    return AL, AR, C, dm


def norm_scaled_bm(X):
    """helpers.hpp:146 norm(x)/sqrt(x.size()) on a BlockMat (Frobenius over all blocks)."""
    n = sum(M.size for (_, M) in X.values())
    if n == 0:
        return 0.0
    return math.sqrt(sum(float(np.sum(np.abs(M) ** 2)) for (_, M) in X.values())) / math.sqrt(n)


def GradNormRight(AR, C, HAfun):
    """VUMPS_helpers.hpp:145-153."""
    return norm_scaled_bm(ApplyTMmixedRight(HAfun(bd_mul_mps(C, AR)), Nullspace(AR, "r")))


def GradNormLeft(AL, C, HAfun):
    """VUMPS_helpers.hpp:135-143."""
    return norm_scaled_bm(ApplyTMmixedLeft(HAfun(mps_mul_bd(AL, C)), Nullspace(AL, "l")))


# ----------------------------------------------------------------------------------------------
# state preparation and observables (MPSBlockUtilities.hpp:1017-1169)
# ----------------------------------------------------------------------------------------------


def randMPS_LR(N, I2K, dimvec, rng):
    """MPSBlockUtilities.hpp:1093-1135: returns (ALvec, ARvec, Cvec)."""
    ALvec = []
    for n in range(1, N):
        Q, _ = qr_mps(mps_rand(I2K, dimvec[n - 1], dimvec[n], rng), "l")
        ALvec.append(Q)
    Q, _ = qr_mps(mps_rand(I2K, dimvec[-1], dimvec[0], rng), "l")
    ALvec.append(Q)
    # ARPACK's default start vector comes from a generator whose state persists across calls
    # in the process (its result then depends on what ran before); the identity is a fixed
    # start, the same one the device path takes
    _, R = TMDominantEig(ALvec, dimvec[0], "r", tol=1e-14, x0=bd_eye(dimvec[0]))
    C = {}
    for q in sorted(R):
        U, sv, _ = np.linalg.svd(R[q])
        X = U * np.sqrt(sv)[None, :]
        Qt, Rt = qr_pos(X.T)
        C[q] = Rt.T.copy()
    Cvec, ARvec = [], []
    Ctmp = C
    for A in reversed(ALvec):
        Cvec.insert(0, Ctmp)
        Qr, Rr = qr_mps(mps_mul_bd(A, Ctmp), "r")
        ARvec.insert(0, Qr)
        Ctmp = Rr
    return ALvec, ARvec, Cvec


def shift(arr, k):
    """MPSBlockUtilities.hpp:1154-1169 (shift(arr,-1) rotates left by one)."""
    k %= len(arr)
    return arr[-k:] + arr[:-k] if k else list(arr)


def MeasureObservables(obs, A, L):
    """MeasureObservables (MPSBlockUtilities.hpp:1017-1073) with dir = r (A = AR, L given): for
    every (name, O) with O acting on NS sites (d^NS x d^NS),
    val[n] = trace(L[n-1] ApplyOpTMRightGen(O, A[n] ... A[n+NS-1])) with ApplyOpTMRightGen =
    ApplyTMmixedRight(ApplyOperator(A, O), A) (TMBlockFunctions.hpp:851-856) and the BlockMat
    trace over blocks with equal charges only (BlockObj.hpp:1340-1350)."""
    N = len(A)
    d = len(A[0])
    out = {}
    for name, O in obs:
        O = np.asarray(O, dtype=np.float64)
        NS = int(round(math.log(O.shape[0]) / math.log(d)))
        hnnz = [(r, c, float(O[r, c])) for c in range(O.shape[1]) for r in range(O.shape[0]) if O[r, c] != 0.0]
        vals = []
        for n in range(N):
            At = A[n]
            for k in range(1, NS):
                At = mps_mul_mps(At, A[(n + k) % N])
            X = ApplyTMmixedRight(ApplyOperator(At, hnnz), At)
            Lm = L[(n - 1) % N]
            vals.append(float(sum(np.trace(Lm[qi] @ M) for qi, (qo, M) in X.items() if qi == qo and qi in Lm)))
        out[name] = np.array(vals)
    return out


def energy_right(hnnz, ARvec, Lvec):
    """MeasureObservables(H, AR, L) (MPSBlockUtilities.hpp:1017-1073, dir = r):
    E(n) = tr(L[n-1] * ApplyOpTMRight(H, AR[n] AR[n+1]))."""
    N = len(ARvec)
    E = []
    for n in range(N):
        AA = mps_mul_mps(ARvec[n], ARvec[(n + 1) % N])
        X = ApplyOpTMRightDiag(hnnz, AA)
        Lm = Lvec[(n - 1) % N]
        E.append(sum(np.trace(Lm[q] @ X[q]) for q in X if q in Lm))
    return np.array(E)


# ----------------------------------------------------------------------------------------------
# VUMPS driver (VUMPS/VUMPS_main.cpp:97-354), bond expansion disabled
# ----------------------------------------------------------------------------------------------


class VUMPS:
    """Restatement of one VUMPS_main run with ExpandFromH disabled (mmax = D)."""

    def __init__(self, h, d, I2K, dmap0, N=2, seed=1, InvETol=5e-15, InvEfac=2.0, fixed_tol=None,
                 tolmin=5e-16, tolmax=1e-6, trueLR=True, svdthresh=5e-7, dimvec=None, init=None, gmres_maxit=0,
                 mmax=None, dmmax=20, expand_pause=5, expand_thresh=1e-5, lamthresh=1e-12):
        self.hnnz = sparse_nnz(h)
        self.gmres_maxit = gmres_maxit  # 0: the reference's maxit = problem size
        # bond expansion (VUMPS_main.cpp:31-35, 149, 168, 270-308), off unless mmax is given
        self.mmax = None if mmax is None else ([int(mmax)] * N if np.isscalar(mmax) else [int(x) for x in mmax])
        self.dmmax, self.expand_pause, self.expand_thresh, self.lamthresh = dmmax, expand_pause, expand_thresh, lamthresh
        self.expand_ct = [0] * N
        self.exp_prec = 1.0
        self.expansions = 0
        self.d, self.N, self.I2K = d, N, I2K
        self.InvETol, self.InvEfac, self.fixed_tol, self.trueLR = InvETol, InvEfac, fixed_tol, trueLR
        self.tolmin, self.tolmax = tolmin, tolmax  # VUMPS_main.cpp:37-38
        self.svdthresh = svdthresh
        self.rng = np.random.default_rng(seed)
        if dimvec is None:
            dimvec = make_dims(dmap0, N, I2K)
        if init is None:
            AL, AR, C = randMPS_LR(N, I2K, dimvec, self.rng)
        else:
            AL, AR, C = [list(x) for x in init]
        L = [bd_mul(bd_t(c), c) for c in C]
        R = [bd_mul(c, bd_t(c)) for c in C]
        AR = shift(AR, -1)
        L = shift(L, -1)
        self.AL, self.AR, self.C, self.L = AL, AR, C, L
        hn = self.hnnz
        self.HL = ReducedOp(hn, AL[-1], d, "l")
        self.HR = ReducedOp(hn, AR[0], d, "r")
        Rb = R[-1]
        self.EHL, _ = InvertE_proj(AL, GetHL(AL, hn), bd_eye({q: m.shape[1] for q, m in C[-1].items()}), Rb, "l",
                                   InvETol, gmres_maxit, rng=self.rng)
        Lb = L[-1]
        self.EHR, _ = InvertE_proj(AR, GetHR(AR, hn), Lb, bd_eye({q: m.shape[0] for q, m in C[0].items()}), "r",
                                   InvETol, gmres_maxit, rng=self.rng)
        self.EHL1 = bd_add(ApplyTMLeft(AL[0], self.EHL), ApplyOpTMLeftDiag(hn, mps_mul_mps(AL[-1], AL[0])))
        self.EHR1 = bd_add(ApplyTMRight(AR[-1], self.EHR), ApplyOpTMRightDiag(hn, mps_mul_mps(AR[-1], AR[0])))
        self.prec = np.ones(N)
        self.F = np.ones(N)
        self.dosvd = True
        self.E = None
        self.EHR0 = [None] * N   # persists across sweeps (VUMPS_main.cpp:119)

    def site_update(self, nn):
        d, N, hn = self.d, self.N, self.hnnz
        self.EHR0[nn] = self.EHR
        AL, AR, C = self.AL, self.AR, self.C
        EHL, EHR, HL, HR = self.EHL, self.EHR, self.HL, self.HR
        HA = lambda X: ApplyHA(X, EHL, EHR, HL, HR)
        self.F[nn] = GradNormRight(AR[-1], C[-1], HA)
        tol = self.fixed_tol if self.fixed_tol else min(max(self.prec[nn] / 100.0, self.tolmin), self.tolmax)
        AC = bd_mul_mps(C[-1], AR[-1])
        Adims = mps_sizes(AC)
        Am = mps_nelem(AC)
        _, v = eigs_rs(lambda x: ApplyHAvec(x, Adims, EHL, EHR, HL, HR), Am, tol, mps_vec(AC))
        AC = mps_from_vec(v[:, 0], Adims)
        CLd, CRd = bd_sizes(C[-1]), bd_sizes(C[0])
        CLm, CRm = sum(m * m for _, m in CLd), sum(m * m for _, m in CRd)
        _, cl = eigs_rs(lambda x: ApplyHCvec(x, CLd, EHL, self.EHR1, hn, d, AL[-1], AR[-1]), CLm, tol, bd_vec(C[-1]))
        _, cr = eigs_rs(lambda x: ApplyHCvec(x, CRd, self.EHL1, EHR, hn, d, AL[0], AR[0]), CRm, tol, bd_vec(C[0]))
        cl = cl[:, 0] / np.sign(cl[0, 0])
        cr = cr[:, 0] / np.sign(cr[0, 0])
        CL, CR = bd_from_vec(cl, CLd), bd_from_vec(cr, CRd)
        if self.dosvd and self.prec[nn] < self.svdthresh:
            self.dosvd = False
        if self.dosvd:
            QL, _, PL = svd_mps([bm_mul_bd(a, bd_t(CR)) for a in AC], "l")
            ALnew = mps_mul_bd(QL, PL)
            QR, _, PR = svd_mps(bd_mul_mps(bd_t(CL), AC), "r")
            ARnew = bd_mul_mps(PR, QR)
        else:
            QL, _ = qr_mps(AC, "l")
            PL, _ = qr_bd(CR, "l")
            ALnew = mps_mul_bd(QL, bd_t(PL))
            QR, _ = qr_mps(AC, "r")
            PR, _ = qr_bd(CL, "r")
            ARnew = bd_mul_mps(bd_t(PR), QR)
        err_l = mps_norm_inf(mps_sub(AC, mps_mul_bd(ALnew, CR)))
        err_r = mps_norm_inf(mps_sub(AC, bd_mul_mps(CL, ARnew)))
        self.prec[nn] = max(err_l, err_r)
        AL[0] = ALnew
        AR[-1] = ARnew
        C[0] = CR
        C[-1] = CL
        Rm = bd_mul(CL, bd_t(CL))
        if self.trueLR:
            _, Rm = TMDominantEig(AL, {q: m.shape[0] for q, m in Rm.items()}, "r", 1e-15, Rm)
        HAL = GetHL(AL, hn)
        AAL = mps_mul_mps(AL[-1], AL[0])
        gtol = max(tol / self.InvEfac, self.InvETol)
        EHL, _ = InvertE_proj(AL, HAL, bd_eye({q: m.shape[1] for q, m in C[-1].items()}), Rm, "l", gtol, self.gmres_maxit, EHL)
        AL[:] = shift(AL, -1)
        AR[:] = shift(AR, -1)
        C[:] = shift(C, -1)
        EHLtmp = bd_add(ApplyOpTMLeftDiag(hn, AAL), ApplyTMLeft(AL[-1], EHL))
        AAL = mps_mul_mps(AL[-1], AL[0])
        self.EHL1 = bd_add(ApplyOpTMLeftDiag(hn, AAL), ApplyTMLeft(AL[0], EHLtmp))
        Lm = bd_mul(bd_t(C[0]), C[0])
        if self.trueLR:
            _, Lm = TMDominantEig(AR, {q: m.shape[0] for q, m in Lm.items()}, "l", 1e-15, Lm)
        HAR = GetHR(AR, hn)
        EHR0_next = self.EHR0[(nn + 1) % N]
        EHR, _ = InvertE_proj(AR, HAR, Lm, bd_eye({q: m.shape[0] for q, m in C[0].items()}), "r", gtol, self.gmres_maxit, EHR0_next)
        if self.mmax is not None and self._expand_now(nn, C[-1]):
            # VUMPS_main.cpp:280-301: grow the bond between AL.back() and AR.back(), pad AR[N-2]
            # with zeros to AL.back()'s sectors, and EHL on the grown bond
            self.expand_ct[nn] = 0
            mr_tot = sum(m.shape[1] for m in C[-1].values())
            AL[-1], AR[-1], C[-1], _ = ExpandFromH(hn, self.I2K, AL[-1], AR[-1], C[-1],
                                                   min(self.dmmax, self.mmax[nn] - mr_tot))
            for s_ in range(d):
                for ql, (c, Mal) in AL[-1][s_].items():
                    if ql in AR[N - 2][s_]:
                        qo, Mar = AR[N - 2][s_][ql]
                        AR[N - 2][s_][ql] = (qo, np.hstack([Mar, np.zeros((Mar.shape[0], Mal.shape[1] - Mar.shape[1]))]))
                    else:
                        AR[N - 2][s_][ql] = (c, np.zeros(Mal.shape))
            EHL = bd_add(ApplyOpTMLeftDiag(hn, mps_mul_mps(AL[N - 2], AL[-1])), ApplyTMLeft(AL[-1], EHL))
            self.expansions += 1
        else:
            EHL = EHLtmp
        self.EHR1 = bd_add(ApplyTMRight(AR[-1], EHR), ApplyOpTMRightDiag(hn, mps_mul_mps(AR[-1], AR[0])))
        self.HL = ReducedOp(hn, AL[-1], d, "l")
        self.HR = ReducedOp(hn, AR[0], d, "r")
        self.EHL, self.EHR = EHL, EHR

    def _expand_now(self, nn, Cr):
        """VUMPS_main.cpp:272-277 and the else branch at :303-306."""
        mr_tot = sum(m.shape[1] for m in Cr.values())
        now = self.expand_ct[nn] >= self.expand_pause and self.exp_prec < self.expand_thresh and mr_tot < self.mmax[nn]
        if now:
            minlam = max(float(np.linalg.svd(M, compute_uv=False).min()) for M in Cr.values() if M.size)
            now = minlam > self.lamthresh
        if not now:
            self.expand_ct[nn] += 1
        return now

    def keep_running(self, thresh=1e-14):
        """run_IDMRG (VUMPS_main.cpp:331-340)."""
        if float(np.max(self.F)) > thresh:
            return True
        if self.mmax is None:
            return False
        too_large = [any(float(np.linalg.svd(M, compute_uv=False).min()) > self.lamthresh for M in Cn.values() if M.size)
                     for Cn in self.C]
        too_small = [sum(M.shape[1] for M in self.C[n].values()) < self.mmax[n] for n in range(self.N)]
        return any(too_large) and any(too_small)

    def sweep(self):
        self.exp_prec = float(np.max(self.prec))  # VUMPS_main.cpp:168
        for nn in range(self.N):
            self.site_update(nn)
        for n in range(self.N):
            self.L[(n - 1) % self.N] = bd_mul(bd_t(self.C[n]), self.C[n])
        self.E = energy_right(self.hnnz, self.AR, self.L)
        return self.E, self.F.copy(), self.prec.copy()
