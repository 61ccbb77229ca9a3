"""State files (saveIMPS / loadIMPS, MPSBlockUtilities.hpp:1215-1327) on the CPU.

* The byte layout of each object type against a byte string assembled here step by step from
  the reference's save sequence (GetHeader + '\\n', uint count, keys, arma_binary blocks).
* Round trips of an oracle state (randMPS_LR, MPSBlockUtilities.hpp:1093-1135); the flat
  buffers the device path takes equal the oracle's Vectorize of the same tensors.
* The reference's load errors (wrong header, truncated file, missing file) and its stream
  semantics (whitespace before a type name is skipped by operator>>).
* GetUniqueFileName's naming.
* The header-only C++ reader/writer (include/imps_io.hpp) and the Python one read each other's
  files and write them back byte for byte.
"""
import io
import json
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import imps_io as F
from imps_cpp_tools_gb300 import models
from oracle import imps_oracle as O

ROOT = Path(__file__).resolve().parent.parent
B0 = {(-4,): 3, (-2,): 8, (0,): 10, (2,): 8, (4,): 3}
B1 = {(-5,): 1, (-3,): 5, (-1,): 10, (1,): 10, (3,): 5, (5,): 1}


def _u32(x):
    return struct.pack("<I", x)


def _key(k):
    return _u32(len(k)) + struct.pack(f"<{len(k)}i", *k)


def _arma(m):
    m = np.asarray(m, dtype=np.float64)
    return (b"ARMA_MAT_BIN_FN008\n" + f"{m.shape[0]} {m.shape[1]}\n".encode() +
            m.astype("<f8").tobytes(order="F"))


def test_byte_layout_of_each_object():
    m1 = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])
    m2 = np.array([[-0.5]])
    # BlockDiagMat::save (BlockObj.hpp:1968-2000): sectors in key order, whatever the dict order
    f = io.BytesIO()
    F.write_blockdiag(f, {(2,): m2, (-1,): m1})
    assert f.getvalue() == b"RBLOCKDIAGMAT\n" + _u32(2) + _key((-1,)) + _arma(m1) + _key((2,)) + _arma(m2)
    # BlockLam::save (BlockObj.hpp:150-183): a column per sector
    f = io.BytesIO()
    F.write_blocklam(f, {(0, 1): np.array([0.75, 0.25])})
    assert f.getvalue() == b"BLOCKLAM\n" + _u32(1) + _key((0, 1)) + _arma(np.array([[0.75], [0.25]]))
    # MPSBlockMat::save (MPSBlockMat.hpp:1085-1104) over BlockMat::save (BlockObj.hpp:905-945)
    A = F.MPSTensor(2, 1, [{(1,): ((0,), m1)}, {}])
    f = io.BytesIO()
    F.write_mps(f, A)
    assert f.getvalue() == (b"RBLOCKMPS\n" + _u32(2) + _u32(1) + b"RBLOCKMAT\n" + _u32(1) + _key((1,)) + _key((0,)) +
                            _arma(m1) + b"RBLOCKMAT\n" + _u32(0))
    # the file: four arrays, saveIMPS order (MPSBlockUtilities.hpp:1215-1244)
    f = io.BytesIO()
    F.save_imps_stream(f, [{}], [{}], [A], [A])
    mps = f.getvalue().split(b"RBLOCKMPSARRAY\n")
    assert mps[0] == b"BLOCKLAMARRAY\n" + _u32(1) + b"BLOCKLAM\n" + _u32(0) + b"RBLOCKDIAGMATARRAY\n" + _u32(1) + \
        b"RBLOCKDIAGMAT\n" + _u32(0)
    assert len(mps) == 3 and mps[1] == mps[2] and mps[1].startswith(_u32(1) + b"RBLOCKMPS\n")


@pytest.fixture(scope="module")
def oracle_state():
    """An XXZ two-site state from the oracle's randMPS_LR, in the reference's saveIMPS
    arrangement: Cvec[n] right of site n, Lamvec[n] its singular values."""
    d, I2K, _ = models.build_model("xxz", J=1.0, Delta=-1.0)
    AL, AR, C = O.randMPS_LR(2, I2K, [B0, B1], np.random.default_rng(4))
    Lam = [{q: np.linalg.svd(m, compute_uv=False) for q, m in Cn.items()} for Cn in C]
    return d, I2K, F.IMPSState(Lam, C, [F.MPSTensor(d, 1, a) for a in AL], [F.MPSTensor(d, 1, a) for a in AR])


def _equal_state(a, b):
    for n in range(len(a.AL)):
        assert a.Lam[n].keys() == b.Lam[n].keys() and a.C[n].keys() == b.C[n].keys()
        for q in a.C[n]:
            assert np.array_equal(a.C[n][q], b.C[n][q]) and np.array_equal(a.Lam[n][q], b.Lam[n][q])
        for X, Y in ((a.AL[n], b.AL[n]), (a.AR[n], b.AR[n])):
            assert X.d == Y.d and len(X.blocks) == len(Y.blocks)
            for s in range(X.d):
                assert X.blocks[s].keys() == Y.blocks[s].keys()
                for q, (qo, m) in X.blocks[s].items():
                    assert Y.blocks[s][q][0] == qo and np.array_equal(Y.blocks[s][q][1], m)


def test_round_trip_and_flat_buffers(oracle_state, tmp_path):
    d, I2K, st = oracle_state
    path = F.saveIMPS(st.Lam, st.C, st.AL, st.AR, "UMPS_xxz", folder=str(tmp_path))
    assert path == f"{tmp_path}/UMPS_xxz.bin"
    back = F.loadIMPS(path)
    _equal_state(st, back)
    # the flat buffers of the device layouts are the oracle's Vectorize of the same tensors
    dimvec = [B0, B1]
    for n in range(2):
        lay = B.Layout.mps(I2K, dimvec[n], dimvec[1 - n])
        for A in (back.AL[n], back.AR[n]):
            v = F.mps_to_flat(A, lay)
            assert np.array_equal(v, O.mps_vec(A.blocks))
            again = F.flat_to_mps(v, lay, d)
            assert all(np.array_equal(again.blocks[s][q][1], A.blocks[s][q][1]) for s in range(d) for q in A.blocks[s])
        # Cvec[n] is on bond n + 1
        lb = B.Layout.blockdiag(dimvec[(n + 1) % 2])
        assert np.array_equal(F.bd_to_flat(back.C[n], lb), O.bd_vec(st.C[n]))
        assert F.bond_dims(back.C[n]) == dimvec[(n + 1) % 2]
    # writing what was read gives the same bytes
    f = io.BytesIO()
    F.save_imps_stream(f, back.Lam, back.C, back.AL, back.AR)
    assert f.getvalue() == Path(path).read_bytes()


def test_sector_mismatch_is_reported(oracle_state):
    d, I2K, st = oracle_state
    wrong = B.Layout.mps(I2K, B1, B0)  # bonds swapped: not the tensor's sectors
    with pytest.raises(F.IMPSFormatError):
        F.mps_to_flat(st.AL[0], wrong)


def test_load_errors(oracle_state, tmp_path):
    d, I2K, st = oracle_state
    f = io.BytesIO()
    F.save_imps_stream(f, st.Lam, st.C, st.AL, st.AR)
    data = f.getvalue()
    with pytest.raises(F.IMPSFormatError, match="wrong header RBLOCKDIAGMATARRAY, should be BLOCKLAMARRAY"):
        # a file without the singular values: the centre matrices come first
        F.load_imps_bytes(data[data.index(b"RBLOCKDIAGMATARRAY"):])
    with pytest.raises(F.IMPSFormatError, match="should be RBLOCKMPSARRAY"):
        F.load_imps_bytes(data.replace(b"RBLOCKMPSARRAY", b"CBLOCKMPSARRAY", 1))  # a complex state
    with pytest.raises(F.IMPSFormatError, match="unexpected end of file"):
        F.load_imps_bytes(data[:-3])
    with pytest.raises(FileNotFoundError):
        F.loadIMPS(str(tmp_path / "missing.bin"))
    # operator>> skips whitespace in front of a type name
    spaced = data.replace(b"RBLOCKDIAGMATARRAY\n", b" \n\tRBLOCKDIAGMATARRAY\n", 1)
    _equal_state(st, F.load_imps_bytes(spaced))


def test_unique_file_name(tmp_path):
    """GetUniqueFileName (helpers.cpp:154-161): name.bin, then name_v1.bin, name_v2.bin."""
    names = []
    for _ in range(3):
        p = F.saveIMPS([], [], [], [], "UMPS_x", folder=str(tmp_path))
        names.append(Path(p).name)
    assert names == ["UMPS_x.bin", "UMPS_x_v1.bin", "UMPS_x_v2.bin"]


@pytest.fixture(scope="module")
def io_check(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("imps_io") / "imps_io_check"
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "native" / "imps_io_check.cpp"), "-o", str(exe)], check=True)
    return exe


def _checksum(v):
    v = np.asarray(v, dtype=np.float64).reshape(-1)
    return float(np.sum(v * (np.arange(v.size) % 7 + 1)))


def test_cpp_reads_and_rewrites_python_files(io_check, oracle_state, tmp_path):
    d, I2K, st = oracle_state
    src = F.saveIMPS(st.Lam, st.C, st.AL, st.AR, "py", folder=str(tmp_path))
    dst = tmp_path / "cpp.bin"
    out = subprocess.run([str(io_check), "copy", src, str(dst)], check=True, capture_output=True, text=True)
    assert dst.read_bytes() == Path(src).read_bytes()
    summ = json.loads(out.stdout)
    dimvec = [B0, B1]
    assert summ["sites"] == 2
    for n in range(2):
        lay = B.Layout.mps(I2K, dimvec[n], dimvec[1 - n])
        for name, A in (("al", st.AL[n]), ("ar", st.AR[n])):
            v = F.mps_to_flat(A, lay)
            got = summ[name][n]
            assert (got["d"], got["nblocks"], got["nelem"]) == (d, len(lay.blocks), lay.nelem)
            assert got["checksum"] == pytest.approx(_checksum(v), rel=1e-14)
        lb = B.Layout.blockdiag(dimvec[(n + 1) % 2])
        assert summ["c"][n]["nelem"] == lb.nelem
        assert summ["c"][n]["checksum"] == pytest.approx(_checksum(F.bd_to_flat(st.C[n], lb)), rel=1e-14)
        lam = np.concatenate([st.Lam[n][q] for q in sorted(st.Lam[n])])
        assert summ["lam"][n]["checksum"] == pytest.approx(_checksum(lam), rel=1e-14)


def test_python_reads_and_rewrites_cpp_files(io_check, tmp_path):
    src = tmp_path / "made.bin"
    subprocess.run([str(io_check), "make", str(src)], check=True)
    st = F.loadIMPS(str(src))
    # the C++ program fills AL(0), AR(0), C/Lam right of site 0, AL(1), ... with 1/64, 2/64, ...
    # (AL and AR of a site are the same tensor there); check the sequence in file order
    seq = []
    for n in range(2):
        seq += [m for s in range(2) for q in sorted(st.AL[n].blocks[s]) for m in [st.AL[n].blocks[s][q][1]]]
        for q in sorted(st.C[n]):
            seq += [st.C[n][q], st.Lam[n][q].reshape(-1, 1)]
    flat = np.concatenate([m.reshape(-1, order="F") for m in seq])
    assert np.array_equal(flat, np.arange(1, flat.size + 1) / 64.0)
    assert st.AL[0].blocks[1][(1,)][0] == (2,)
    f = io.BytesIO()
    F.save_imps_stream(f, st.Lam, st.C, st.AL, st.AR)
    assert f.getvalue() == src.read_bytes()


def test_cpp_reports_a_wrong_header(io_check, tmp_path):
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"RBLOCKMPSARRAY\n" + _u32(0))
    r = subprocess.run([str(io_check), "copy", str(bad), str(tmp_path / "o.bin")], capture_output=True, text=True)
    assert r.returncode == 1 and "wrong header RBLOCKMPSARRAY, should be BLOCKLAMARRAY" in r.stderr


def test_driver_rejects_an_incompatible_state(oracle_state, tmp_path):
    """The checks of VumpsGPU.from_imps run before any device work (Excitations_main.cpp:101:
    "AL not compatible with I2K from model")."""
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    d, I2K, st = oracle_state
    path = F.saveIMPS(st.Lam, st.C, st.AL, st.AR, "xxz", folder=str(tmp_path))
    with pytest.raises(F.IMPSFormatError, match="the model has d = 4"):
        VumpsGPU.from_imps(None, "fhub", path)
    pad = lambda q: tuple(q) + (0,)
    two = F.IMPSState([{pad(q): v for q, v in L.items()} for L in st.Lam], [{pad(q): v for q, v in C.items()}
                                                                           for C in st.C], st.AL, st.AR)
    with pytest.raises(F.IMPSFormatError, match="1 quantum number"):
        VumpsGPU.from_imps(None, "xxz", two, J=1.0, Delta=-1.0)
    three = F.IMPSState(st.Lam * 2, st.C * 2, st.AL * 2, st.AR * 2)
    with pytest.raises(F.IMPSFormatError, match="two-site cells"):
        VumpsGPU.from_imps(None, "xxz", three)


def _alrn_state(oracle_state):
    d, I2K, st = oracle_state
    L = [{q: m.T @ m for q, m in C.items()} for C in st.C]
    R = [{q: m @ m.T for q, m in C.items()} for C in st.C]
    NL = [F.MPSTensor(d, 1, O.Nullspace(A.blocks, "l")) for A in st.AL]
    return st.C, L, R, st.AL, st.AR, NL


def test_alrn_round_trip(oracle_state, tmp_path):
    """saveALRN / loadALRN (Excitations_helpers.hpp:949-1085): C, L, R as RBLOCKDIAGMATARRAY,
    then AL, AR, NL as RBLOCKMPSARRAY, in that order."""
    arrs = _alrn_state(oracle_state)
    path = F.saveALRN(*arrs, "x_ALRN", folder=str(tmp_path))
    data = Path(path).read_bytes()
    assert data.startswith(b"RBLOCKDIAGMATARRAY\n" + _u32(2) + b"RBLOCKDIAGMAT\n")
    assert data.count(b"RBLOCKDIAGMATARRAY\n") == 3 and data.count(b"RBLOCKMPSARRAY\n") == 3
    back = F.loadALRN(path)
    for got, ref in zip((back.C, back.L, back.R), arrs[:3]):
        for n in range(2):
            assert got[n].keys() == ref[n].keys() and all(np.array_equal(got[n][q], ref[n][q]) for q in ref[n])
    for got, ref in zip((back.AL, back.AR, back.NL), arrs[3:]):
        for n in range(2):
            assert all(got[n].blocks[s].keys() == ref[n].blocks[s].keys() for s in range(ref[n].d))
    f = io.BytesIO()
    F.save_alrn_stream(f, back.C, back.L, back.R, back.AL, back.AR, back.NL)
    assert f.getvalue() == data
    with pytest.raises(F.IMPSFormatError, match="should be RBLOCKDIAGMATARRAY"):
        F.load_alrn_bytes(data[data.index(b"RBLOCKMPSARRAY"):])


def test_cpp_alrn_round_trip(io_check, oracle_state, tmp_path):
    src = F.saveALRN(*_alrn_state(oracle_state), "py_ALRN", folder=str(tmp_path))
    dst = tmp_path / "cpp_ALRN.bin"
    out = subprocess.run([str(io_check), "alrn", src, str(dst)], check=True, capture_output=True, text=True)
    assert dst.read_bytes() == Path(src).read_bytes()
    assert json.loads(out.stdout)["sites"] == 2
