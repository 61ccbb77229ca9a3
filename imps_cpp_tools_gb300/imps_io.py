"""saveIMPS / loadIMPS: the reference's binary state file, read and written on the host.

A state file holds a unit cell's singular values, centre matrices and left/right isometries in
that order (saveIMPS, MPSBlockUtilities.hpp:1215-1244; loadIMPS :1271-1300):

    BLOCKLAMARRAY       Lamvec[n]  singular values of Cvec[n], one vector per sector
    RBLOCKDIAGMATARRAY  Cvec[n]    centre matrix right of site n (AL(n) C[n] = C[n-1] AR(n))
    RBLOCKMPSARRAY      ALvec[n]   left isometry of site n
    RBLOCKMPSARRAY      ARvec[n]   right isometry of site n

Every object starts with its type name and a newline (GetHeader, BlockObj.hpp:3156-3192,
MPSBlockMat.hpp:1418-1430), followed by a 4-byte unsigned count and its parts:

* array types: count = number of sites, then that many objects (BlockObj.hpp:2692-2708,
  2877-2893; MPSBlockMat.hpp:1326-1342);
* BLOCKLAM / RBLOCKDIAGMAT: count = number of sectors, then per sector its key and one
  armadillo matrix (BlockObj.hpp:150-183, 1968-2000);
* RBLOCKMAT: count = number of sectors, then per sector the in key, the out key and one
  armadillo matrix (BlockObj.hpp:905-945);
* RBLOCKMPS: two 4-byte unsigned integers d and NSites (1 for a one-site tensor), then d^NSites
  RBLOCKMAT objects, one per physical index (MPSBlockMat.hpp:1085-1104).

A key (KeyType::save, KeyTypes.hpp:94-117) is a 4-byte unsigned Nsym followed by Nsym 4-byte
signed labels; the symmetry group itself is not stored.  Sectors appear in std::map order:
keys compared lexicographically as integer vectors.

The dense blocks use armadillo's ``arma_binary`` format (armadillo, a third-party dependency
of the reference whose version the reference does not pin): the text line ``ARMA_MAT_BIN_FN008``
for double precision (``ARMA_MAT_BIN_FC016`` for complex double), the text line
``<n_rows> <n_cols>``, then n_rows * n_cols raw values in column-major order.  A singular value
vector is a column (n_cols = 1).  Integers and doubles are stored in the byte order of the
machine that wrote the file; both hosts this package runs on are little-endian, and this
module reads and writes little-endian explicitly.

Reading follows the reference's stream semantics: a type name or an armadillo size is a
whitespace-delimited token (``operator>>``), after which exactly one character (the newline)
is skipped (``file.get()``).  A type name that does not match raises ``IMPSFormatError`` with
the reference's message ("wrong header X, should be Y").

Host structures (plain numpy, independent of the device layouts):

* BlockLam: dict key -> 1-D array;
* BlockDiagMat: dict key -> 2-D array;
* MPS tensor: ``MPSTensor(d, nsites, blocks)``, blocks[s] a dict qin -> (qout, 2-D array).

Keys are tuples of ints.  ``mps_to_flat`` / ``flat_to_mps`` and ``bd_to_flat`` /
``flat_to_bd`` convert to and from the flat Vectorize buffers of ``blocks.Layout``.
"""
from __future__ import annotations

import io
import os
import struct
from dataclasses import dataclass, field

import numpy as np

HDR_LAM, HDR_LAMARRAY = "BLOCKLAM", "BLOCKLAMARRAY"
HDR_BDMAT, HDR_BDMATARRAY = "RBLOCKDIAGMAT", "RBLOCKDIAGMATARRAY"
HDR_BMAT = "RBLOCKMAT"
HDR_MPS, HDR_MPSARRAY = "RBLOCKMPS", "RBLOCKMPSARRAY"
ARMA_F64, ARMA_C128 = "ARMA_MAT_BIN_FN008", "ARMA_MAT_BIN_FC016"
_WS = b" \t\n\v\f\r"


class IMPSFormatError(ValueError):
    """A state file that does not follow the format (the reference's load returns false)."""


@dataclass
class MPSTensor:
    """One MPSBlockMat: blocks[s] maps the in key to (out key, dense block) for physical index s."""
    d: int
    nsites: int = 1
    blocks: list = field(default_factory=list)


@dataclass
class IMPSState:
    """The four arrays of a state file, indexed by site n of the unit cell."""
    Lam: list
    C: list
    AL: list
    AR: list


# ------------------------------------------------------------------------------------------------
# writing
# ------------------------------------------------------------------------------------------------

def _u32(f, x):
    f.write(struct.pack("<I", int(x)))


def _header(f, name):
    f.write(name.encode("ascii") + b"\n")


def write_key(f, key):
    """KeyType::save (KeyTypes.hpp:94-117): uint Nsym, then Nsym int labels."""
    key = tuple(int(k) for k in key)
    _u32(f, len(key))
    f.write(struct.pack(f"<{len(key)}i", *key))


def write_arma(f, mat):
    """Mat::save(file, arma_binary): header line, size line, column-major doubles."""
    a = np.asarray(mat, dtype=np.float64)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    if a.ndim != 2:
        raise ValueError("an armadillo matrix is two-dimensional")
    f.write(f"{ARMA_F64}\n{a.shape[0]} {a.shape[1]}\n".encode("ascii"))
    f.write(np.asarray(a, dtype="<f8").tobytes(order="F"))


def _sorted_items(dct):
    return sorted(((tuple(int(x) for x in k), v) for k, v in dct.items()), key=lambda kv: kv[0])


def write_blocklam(f, lam):
    """BlockLam::save (BlockObj.hpp:150-183)."""
    _header(f, HDR_LAM)
    items = _sorted_items(lam)
    _u32(f, len(items))
    for k, v in items:
        write_key(f, k)
        write_arma(f, np.asarray(v, dtype=np.float64).reshape(-1, 1))


def write_blockdiag(f, bd):
    """BlockDiagMat::save (BlockObj.hpp:1968-2000)."""
    _header(f, HDR_BDMAT)
    items = _sorted_items(bd)
    _u32(f, len(items))
    for k, m in items:
        write_key(f, k)
        write_arma(f, m)


def write_blockmat(f, bm):
    """BlockMat::save (BlockObj.hpp:905-945): dict qin -> (qout, block)."""
    _header(f, HDR_BMAT)
    items = _sorted_items(bm)
    _u32(f, len(items))
    for qin, (qout, m) in items:
        write_key(f, qin)
        write_key(f, qout)
        write_arma(f, m)


def write_mps(f, A):
    """MPSBlockMat::save (MPSBlockMat.hpp:1085-1104)."""
    if len(A.blocks) != A.d ** A.nsites:
        raise ValueError(f"an MPS tensor with d = {A.d} and {A.nsites} site(s) has {A.d ** A.nsites} "
                         f"physical indices, not {len(A.blocks)}")
    _header(f, HDR_MPS)
    _u32(f, A.d)
    _u32(f, A.nsites)
    for bm in A.blocks:
        write_blockmat(f, bm)


def _write_array(f, header, items, writer):
    _header(f, header)
    _u32(f, len(items))
    for it in items:
        writer(f, it)


def save_imps_stream(f, Lamvec, Cvec, ALvec, ARvec):
    """saveIMPS(Lamvec, Cvec, ALvec, ARvec, file) (MPSBlockUtilities.hpp:1215-1244)."""
    _write_array(f, HDR_LAMARRAY, Lamvec, write_blocklam)
    _write_array(f, HDR_BDMATARRAY, Cvec, write_blockdiag)
    _write_array(f, HDR_MPSARRAY, ALvec, write_mps)
    _write_array(f, HDR_MPSARRAY, ARvec, write_mps)


def unique_file_name(filename, ending="bin", folder="."):
    """GetUniqueFileName (MPShelpers/src/helpers.cpp:154-161, defaults helpers.h:36):
    folder/filename.ending, or folder/filename_v<k>.ending with the first k = 1, 2, ... that
    does not exist."""
    name = f"{folder}/{filename}.{ending}"
    k = 1
    while os.path.isfile(name):
        name = f"{folder}/{filename}_v{k}.{ending}"
        k += 1
    return name


def saveIMPS(Lamvec, Cvec, ALvec, ARvec, name, ending="bin", folder="."):
    """saveIMPS(Lamvec, Cvec, ALvec, ARvec, name, ending) (MPSBlockUtilities.hpp:1249-1267):
    writes to a new file named by ``unique_file_name`` and returns its path."""
    path = unique_file_name(name, ending, folder)
    buf = io.BytesIO()
    save_imps_stream(buf, Lamvec, Cvec, ALvec, ARvec)
    with open(path, "wb") as f:
        f.write(buf.getvalue())
    return path


# ------------------------------------------------------------------------------------------------
# reading
# ------------------------------------------------------------------------------------------------

class _Reader:
    """Byte stream with the two std::istream operations the reference's loaders use."""

    def __init__(self, data):
        self.b = memoryview(data)
        self.p = 0

    def token(self):
        """operator>>(istream, string): skip whitespace, read up to the next whitespace."""
        b, p, n = self.b, self.p, len(self.b)
        while p < n and b[p] in _WS:
            p += 1
        s = p
        while p < n and b[p] not in _WS:
            p += 1
        if s == p:
            raise IMPSFormatError("unexpected end of file")
        self.p = p
        return bytes(b[s:p]).decode("latin-1")

    def get(self):
        """istream::get(): one character."""
        if self.p >= len(self.b):
            raise IMPSFormatError("unexpected end of file")
        self.p += 1

    def read(self, n):
        if self.p + n > len(self.b):
            raise IMPSFormatError("unexpected end of file")
        out = self.b[self.p:self.p + n]
        self.p += n
        return out

    def u32(self):
        return struct.unpack("<I", self.read(4))[0]

    def header(self, expected):
        h = self.token()
        self.get()
        if h != expected:
            raise IMPSFormatError(f"wrong header {h}, should be {expected}")

    def key(self):
        """KeyType(file, GroupObj) (KeyTypes.hpp:75-90)."""
        n = self.u32()
        return tuple(struct.unpack(f"<{n}i", self.read(4 * n)))

    def arma(self):
        """Mat::load(file, arma_binary): header, rows and cols tokens, one character, data."""
        h = self.token()
        try:
            rows, cols = int(self.token()), int(self.token())
        except ValueError:
            raise IMPSFormatError("bad armadillo matrix size") from None
        if h != ARMA_F64:
            raise IMPSFormatError(f"armadillo matrix header {h}, should be {ARMA_F64}")
        self.get()
        a = np.frombuffer(self.read(8 * rows * cols), dtype="<f8").astype(np.float64)
        return a.reshape((rows, cols), order="F")


def read_blocklam(r):
    """BlockLam::load (BlockObj.hpp:210-248)."""
    r.header(HDR_LAM)
    out = {}
    for _ in range(r.u32()):
        k = r.key()
        out[k] = r.arma().reshape(-1)
    return out


def read_blockdiag(r):
    """BlockDiagMat::load (BlockObj.hpp:2026-2063)."""
    r.header(HDR_BDMAT)
    out = {}
    for _ in range(r.u32()):
        k = r.key()
        out[k] = r.arma()
    return out


def read_blockmat(r):
    """BlockMat::load (BlockObj.hpp:972-1012)."""
    r.header(HDR_BMAT)
    out = {}
    for _ in range(r.u32()):
        qin = r.key()
        qout = r.key()
        out[qin] = (qout, r.arma())
    return out


def read_mps(r):
    """MPSBlockMat::load (MPSBlockMat.hpp:1131-1165)."""
    r.header(HDR_MPS)
    d, nsites = r.u32(), r.u32()
    return MPSTensor(d, nsites, [read_blockmat(r) for _ in range(d ** nsites)])


def _read_array(r, header, reader):
    r.header(header)
    return [reader(r) for _ in range(r.u32())]


def load_imps_bytes(data):
    """loadIMPS(Lamvec, Cvec, ALvec, ARvec, GroupObj, file) (MPSBlockUtilities.hpp:1271-1300);
    the arrays of RBLOCKMPS tensors are read as in MPSBlockMatArray::load (MPSBlockMat.hpp:1373-1403)."""
    r = _Reader(data)
    Lam = _read_array(r, HDR_LAMARRAY, read_blocklam)
    Cv = _read_array(r, HDR_BDMATARRAY, read_blockdiag)
    AL = _read_array(r, HDR_MPSARRAY, read_mps)
    AR = _read_array(r, HDR_MPSARRAY, read_mps)
    return IMPSState(Lam, Cv, AL, AR)


def loadIMPS(filename):
    """loadIMPS(..., filename) (MPSBlockUtilities.hpp:1305-1327); raises FileNotFoundError for a
    missing file and IMPSFormatError for a malformed one."""
    if not os.path.isfile(filename):
        raise FileNotFoundError(f"file {filename} not found")
    with open(filename, "rb") as f:
        return load_imps_bytes(f.read())


# ------------------------------------------------------------------------------------------------
# the excitation driver's file: ground state with environments and null spaces
# ------------------------------------------------------------------------------------------------

@dataclass
class ALRNState:
    """The six arrays of saveALRN, indexed by site n: C[n] (right of site n), L[n] = C[n]^T C[n],
    R[n] = C[n] C[n]^T (Excitations_main.cpp:134-138), AL, AR (AR as the excitation driver
    uses it, after its shifts and the sign fix of AR[0]) and the left null spaces NL."""
    C: list
    L: list
    R: list
    AL: list
    AR: list
    NL: list


def save_alrn_stream(f, Cvec, Lvec, Rvec, ALvec, ARvec, NLvec):
    """saveALRN(Cvec, Lvec, Rvec, ALvec, ARvec, NLvec, file) (Excitations_helpers.hpp:949-989)."""
    for arr in (Cvec, Lvec, Rvec):
        _write_array(f, HDR_BDMATARRAY, arr, write_blockdiag)
    for arr in (ALvec, ARvec, NLvec):
        _write_array(f, HDR_MPSARRAY, arr, write_mps)


def saveALRN(Cvec, Lvec, Rvec, ALvec, ARvec, NLvec, name, ending="bin", folder="."):
    """saveALRN(..., name, ending) (Excitations_helpers.hpp:992-1013, called at
    Excitations_main.cpp:234-236): a new file named by ``unique_file_name``; returns its path."""
    path = unique_file_name(name, ending, folder)
    buf = io.BytesIO()
    save_alrn_stream(buf, Cvec, Lvec, Rvec, ALvec, ARvec, NLvec)
    with open(path, "wb") as f:
        f.write(buf.getvalue())
    return path


def load_alrn_bytes(data):
    """loadALRN(..., GroupObj, file) (Excitations_helpers.hpp:1017-1058)."""
    r = _Reader(data)
    C, L, R = (_read_array(r, HDR_BDMATARRAY, read_blockdiag) for _ in range(3))
    AL, AR, NL = (_read_array(r, HDR_MPSARRAY, read_mps) for _ in range(3))
    return ALRNState(C, L, R, AL, AR, NL)


def loadALRN(filename):
    """loadALRN(..., filename) (Excitations_helpers.hpp:1062-1085)."""
    if not os.path.isfile(filename):
        raise FileNotFoundError(f"file {filename} not found")
    with open(filename, "rb") as f:
        return load_alrn_bytes(f.read())


# ------------------------------------------------------------------------------------------------
# conversion to and from the flat Vectorize buffers of blocks.Layout
# ------------------------------------------------------------------------------------------------

def mps_to_flat(A, layout):
    """An MPSTensor into the flat buffer of ``layout`` (a Layout.mps): every layout block must be
    present with the same out key and shape, and the tensor must hold no other block."""
    out = np.zeros(layout.nelem, dtype=np.float64)
    seen = 0
    for (s, qin, qout, rows, cols), off in zip(layout.blocks, layout.offsets):
        if s >= len(A.blocks) or qin not in A.blocks[s]:
            raise IMPSFormatError(f"sector {qin} of physical index {s} missing")
        qo, m = A.blocks[s][qin]
        if tuple(qo) != tuple(qout) or m.shape != (rows, cols):
            raise IMPSFormatError(f"sector {qin} of physical index {s}: out key {qo} shape {m.shape}, "
                                  f"expected {qout} {(rows, cols)}")
        out[off:off + rows * cols] = m.ravel(order="F")
        seen += 1
    if seen != sum(len(b) for b in A.blocks):
        raise IMPSFormatError("the tensor holds sectors the layout does not")
    return out


def flat_to_mps(vec, layout, d):
    vec = np.asarray(vec, dtype=np.float64)
    blocks = [dict() for _ in range(d)]
    for (s, qin, qout, rows, cols), off in zip(layout.blocks, layout.offsets):
        blocks[s][qin] = (qout, vec[off:off + rows * cols].reshape((rows, cols), order="F").copy())
    return MPSTensor(d, 1, blocks)


def bd_to_flat(bd, layout):
    out = np.zeros(layout.nelem, dtype=np.float64)
    if len(bd) != len(layout.blocks):
        raise IMPSFormatError(f"{len(bd)} sectors, expected {len(layout.blocks)}")
    for (_, qin, _, rows, cols), off in zip(layout.blocks, layout.offsets):
        if qin not in bd or bd[qin].shape != (rows, cols):
            raise IMPSFormatError(f"sector {qin} missing or of the wrong shape")
        out[off:off + rows * cols] = bd[qin].ravel(order="F")
    return out


def flat_to_bd(vec, layout):
    vec = np.asarray(vec, dtype=np.float64)
    return {qin: vec[off:off + r * c].reshape((r, c), order="F").copy()
            for (_, qin, _, r, c), off in zip(layout.blocks, layout.offsets)}


def lam_from_flat(S, layout):
    """Singular values in sector order (one run of min(rows, cols) per sector) as a BlockLam."""
    S = np.asarray(S, dtype=np.float64)
    out, o = {}, 0
    for (_, qin, _, r, c) in layout.blocks:
        k = min(r, c)
        out[qin] = S[o:o + k].copy()
        o += k
    return out


def bond_dims(bd):
    """Sector dimensions {key: m} of a square block-diagonal matrix."""
    return {k: int(m.shape[0]) for k, m in bd.items()}
