"""CPU tests of the native library: it loads, exports every declared symbol, and its sector
planner (run in a host-only context, no GPU) produces exactly the block pairings the
reference's std::map lookups produce."""
import ctypes as C

import numpy as np
import pytest

from imps_cpp_tools_gb300 import _native as N
from imps_cpp_tools_gb300 import blocks as B
from oracle import imps_oracle as O
from tests import imps_testlib as T


@pytest.fixture(scope="module")
def host_ctx():
    N.load()
    return B.Context(-1)


def test_exports_every_header_symbol():
    lib = N.load()
    syms = N.header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.imps_version() >= 100
    assert N.load().imps_status_string(-2) == b"inconsistent sector table"


def test_layout_rejects_unsorted_keys():
    with pytest.raises(N.ImpsError) as e:
        B.Layout([(0, (2,), (3,), 1, 1), (0, (0,), (1,), 1, 1)], 1)
    assert e.value.status == -2
    with pytest.raises(N.ImpsError):
        B.Layout([(0, (0,), (1,), -1, 1)], 1)
    L = B.Layout([(0, (0,), (1,), 2, 3), (0, (2,), (3,), 1, 4), (1, (0,), (-1,), 2, 2)], 1)
    assert L.nelem == 6 + 4 + 4
    bd = L.bond(0)
    assert [b[1] for b in bd.blocks] == [(0,), (2,)] and [b[3] for b in bd.blocks] == [2, 1]


def _offsets(blocks):
    off, o = {}, 0
    for (g, qi, qo, r, c) in blocks:
        off[(g, qi)] = o
        o += r * c
    return off


def _expected_hac(p):
    """The products ApplyHA (VUMPS_helpers.hpp:48-52) forms, found with the reference's map
    lookups on the oracle's dicts, as (slot, offset) pairs per output block."""
    d, AC, EHL, EHR, HL, HR = p["d"], p["AC"], p["EHL"], p["EHR"], p["HL"], p["HR"]
    oac = _offsets(T.mps_blocks(AC))
    oel, oer = _offsets(T.bd_blocks(EHL)), _offsets(T.bd_blocks(EHR))
    ohl, ohr = _offsets(T.redop_blocks(HL, d)), _offsets(T.redop_blocks(HR, d))
    exp = []
    for s in range(d):
        for ql in sorted(AC[s]):
            qr = AC[s][ql][0]
            terms = []
            if ql in EHL:
                terms.append((2, oel[(0, ql)], 0, oac[(s, ql)]))
            if qr in EHR:
                terms.append((0, oac[(s, ql)], 3, oer[(0, qr)]))
            for j in range(d):
                if ql in HL[s][j]:
                    ql2 = HL[s][j][ql][0]
                    if ql2 in AC[j] and AC[j][ql2][0] == qr:
                        terms.append((4, ohl[(s * d + j, ql)], 0, oac[(j, ql2)]))
                if ql in AC[j]:
                    qr2 = AC[j][ql][0]
                    if qr2 in HR[s][j] and HR[s][j][qr2][0] == qr:
                        terms.append((0, oac[(j, ql)], 5, ohr[(s * d + j, qr2)]))
            exp.append(terms)
    return exp


@pytest.mark.parametrize("model,dims0", [
    ("xxz", {(-4,): 1, (-2,): 3, (0,): 5, (2,): 3, (4,): 1}),
    ("fhub", {(0, 0): 4, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2, (2, 0): 1, (0, 2): 1}),
])
def test_hac_sector_matching_bit_exact(host_ctx, model, dims0):
    p = T.hac_problem(model, dims0, seed=11)
    d = p["d"]
    lac = B.Layout(T.mps_blocks(p["AC"]), len(p["I2K"][0]))
    lel, ler = B.Layout(T.bd_blocks(p["EHL"]), lac.nsym), B.Layout(T.bd_blocks(p["EHR"]), lac.nsym)
    lhl, lhr = B.Layout(T.redop_blocks(p["HL"], d), lac.nsym), B.Layout(T.redop_blocks(p["HR"], d), lac.nsym)
    plan = B.plan_hac(host_ctx, lac, lel, ler, lhl, lhr, d)
    tab = plan.table(0)
    got = [[(a, ao, b, bo) for (a, ao, b, bo, k, al) in terms] for (_, terms) in sorted(tab)]
    assert got == _expected_hac(p)
    assert plan.info()["dropped"] == 0
    # useful flops of one apply = sum 2*M*N*K over the products
    fl = sum(2 * r * c * k for (g, qi, qo, r, c), (_, terms) in zip(lac.blocks, sorted(tab))
             for (_, _, _, _, k, _) in terms)
    assert plan.info()["flops_apply"] == fl


@pytest.mark.parametrize("direction", ["l", "r"])
def test_redop_layout_matches_reference_structure(host_ctx, direction):
    st = T.random_state("fhub", {(0, 0): 3, (1, 1): 2, (-1, -1): 2, (1, -1): 1, (-1, 1): 1}, seed=4)
    d, A = st["d"], st["AL"][1] if direction == "l" else st["AR"][1]
    R = O.ReducedOp(st["hnnz"], A, d, direction)
    la = B.Layout(T.mps_blocks(A), 2)
    plan = B.plan_redop(host_ctx, la, d, st["hnnz"], 0 if direction == "l" else 1)
    got = plan.derived(0).blocks
    assert got == [(g, qi, qo, r, c) for (g, qi, qo, r, c) in T.redop_blocks(R, d)]


@pytest.mark.parametrize("direction", [0, 1])
def test_tm_sector_matching(host_ctx, direction):
    st = T.random_state("xxz", {(-2,): 2, (0,): 4, (2,): 2, (4,): 1}, seed=9)
    AL, dv = st["AL"], st["dimvec"]
    l0, l1 = B.Layout(T.mps_blocks(AL[0]), 1), B.Layout(T.mps_blocks(AL[1]), 1)
    bond = B.Layout.blockdiag(dv[0])
    plan = B.plan_tm(host_ctx, [l0, l1], direction, bond, bond)
    info = plan.info()
    assert info["nstages"] == 4
    # stage 1 (first site reduction): every output sector gathers the A blocks whose
    # Qout (left TM) / Qin (right TM) equals it, in physical-index order
    A = AL[0] if direction == 0 else AL[1]
    la = l0 if direction == 0 else l1
    mid = la.bond(1 if direction == 0 else 0)
    tab = plan.table(1)
    oa = _offsets(la.blocks)
    for (tag, terms), blk in zip(tab, mid.blocks):
        q = blk[1]
        exp = []
        for s in range(len(A)):
            for qi in sorted(A[s]):
                qo = A[s][qi][0]
                if (direction == 0 and qo == q) or (direction == 1 and qi == q):
                    exp.append(oa[(s, qi)])
        assert [t[1] for t in terms] == exp


def test_dropped_sector_counted(host_ctx):
    """A HL block pointing at an in[j] block whose Qout differs from the output block is not
    added (the reference would insert it into a std::map of views outside the buffer)."""
    ac = B.Layout([(0, (0,), (1,), 1, 1), (1, (0,), (-1,), 1, 1)], 1)
    e = B.Layout([(0, (0,), (0,), 1, 1)], 1)
    er = B.Layout([(0, (-1,), (-1,), 1, 1), (0, (1,), (1,), 1, 1)], 1)
    hl = B.Layout([(1, (0,), (0,), 1, 1)], 1)  # HL[0][1]: maps 0 -> 0, but in[1](0) -> -1 != 1
    hr = B.Layout([], 1)
    plan = B.plan_hac(host_ctx, ac, e, er, hl, hr, 2)
    assert plan.info()["dropped"] == 1


def test_bad_dims_rejected(host_ctx):
    ac = B.Layout([(0, (0,), (1,), 2, 1)], 1)
    e = B.Layout([(0, (0,), (0,), 3, 3)], 1)  # EHL sector with wrong size
    er = B.Layout([(0, (1,), (1,), 1, 1)], 1)
    empty = B.Layout([], 1)
    with pytest.raises(N.ImpsError) as ex:
        B.plan_hac(host_ctx, ac, e, er, empty, empty, 1)
    assert ex.value.status == -2


def test_nullspace_layout_matches_oracle_structure():
    """The null-space layout of a dir-l decomposition plan has the sectors and dimensions of
    the reference's Nullspace(A, l) (MPSBlockUtilities.hpp:247-300), in std::map order."""
    from imps_cpp_tools_gb300 import blocks as B
    from oracle import imps_oracle as O
    from tests import imps_testlib as T
    st = T.random_state("xxz", {(-4,): 3, (-2,): 8, (0,): 10, (2,): 8, (4,): 3}, seed=3, J=1.0, Delta=-1.0)
    ns = len(st["I2K"][0])
    ctx = B.Context(-1)
    for A in st["AL"]:
        plan = B.plan_decomp(ctx, B.Layout(T.mps_blocks(A), ns), "l")
        NL = O.Nullspace(A, "l")
        ref = [(s, tuple(qi), tuple(NL[s][qi][0]), NL[s][qi][1].shape[0], NL[s][qi][1].shape[1])
               for s in range(len(NL)) for qi in sorted(NL[s]) if NL[s][qi][1].shape[1] > 0]
        got = [(b[0], tuple(b[1]), tuple(b[2]), b[3], b[4]) for b in plan.nslayout.blocks]
        assert got == ref


def _build_cpp_host(tmp_path, name="cpp_host_check"):
    """Compile and link a C++ host program of tests/native over the C ABI (include/imps_gb300.hpp)."""
    import shutil
    import subprocess
    from pathlib import Path
    gxx, nvcc = shutil.which("g++"), shutil.which("nvcc")
    if gxx is None or nvcc is None:
        pytest.skip("g++ or the CUDA toolkit not available")
    cuda = Path(nvcc).resolve().parent.parent
    N.load()
    lib = Path(N.lib_path()).parent
    root = Path(__file__).resolve().parent.parent
    exe = tmp_path / name
    cmd = [gxx, "-std=c++17", "-O2", "-I", str(root / "include"), "-I", str(cuda / "include"),
           str(root / "tests" / "native" / f"{name}.cpp"), "-L", str(lib), "-limps_gb300",
           "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{lib}", f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_host_program_builds(tmp_path):
    """The C++ host interface (RAII handles and the reference-named functors) compiles and
    links against the in-tree library; tests/test_gpu_cpp_host.py runs it."""
    assert _build_cpp_host(tmp_path).exists()



def test_cpp_program_check_builds(tmp_path):
    """The C++ grouped-GEMM program builder (imps_cpp::program) compiles and links;
    tests/test_gpu_cpp_program.py runs it."""
    assert _build_cpp_host(tmp_path, "cpp_program_check").exists()


def test_noalloc_rejects_bad_layouts_before_device_access():
    """imps_tm_apply_noalloc validates its layouts before it touches a device: an `out` (or
    `in`) layout with a non-square block is IMPS_ERR_BAD_TABLE, an MPS tensor beyond the static
    scratch is IMPS_ERR_TOO_LARGE.  The data pointers are dummies that are never read (no GPU
    here)."""
    import ctypes as C
    from imps_cpp_tools_gb300 import _native as N
    I2K = [(1,), (-1,)]
    b0 = {(-1,): 2, (1,): 2}
    b1 = {(0,): 3, (2,): 1, (-2,): 1}
    la = B.Layout.mps(I2K, b0, b1)
    lin = B.Layout.blockdiag(b0)
    bad_out = B.Layout([(0, (-2,), (-2,), 1, 1), (0, (0,), (0,), 3, 2), (0, (2,), (2,), 1, 1)], 1)
    dummy = C.c_void_p(16)
    lib = N.load()
    assert lib.imps_tm_apply_noalloc(la.handle, lin.handle, bad_out.handle, 0, dummy, dummy, dummy, None) == -2
    assert lib.imps_tm_apply_noalloc(la.handle, bad_out.handle, lin.handle, 1, dummy, dummy, dummy, None) == -2
    big = {(q,): 400 for q in range(-3, 4)}  # 2 * 7 * 400^2 > 1,048,576 elements
    lbig = B.Layout.mps(I2K, big, {(q + 1,): m for (q,), m in big.items()})
    lb_in, lb_out = B.Layout.blockdiag(big), B.Layout.blockdiag({(q + 1,): m for (q,), m in big.items()})
    assert lib.imps_tm_apply_noalloc(lbig.handle, lb_in.handle, lb_out.handle, 0, dummy, dummy, dummy, None) == -9


def test_autotune_needs_a_device():
    """The autotuner times launches: a host-only context refuses it (IMPS_ERR_NO_DEVICE) and
    still reports the stage's histogram key and the estimated shape."""
    import ctypes as C
    from imps_cpp_tools_gb300 import _native as N
    ctx = B.Context(-1)
    I2K = [(1,), (-1,)]
    b0 = {(-1,): 2, (1,): 2}
    b1 = {(0,): 3, (2,): 1, (-2,): 1}
    la = B.Layout.mps(I2K, b0, b1)
    plan = B.plan_tm(ctx, [la], 0, B.Layout.blockdiag(b0), B.Layout.blockdiag(b1))
    n = C.c_int(-1)
    assert N.load().imps_plan_autotune(plan.handle, 3, C.byref(n)) == -6
    tile, splits, key = plan.stage_shape(0)
    assert tile in (16, 32) and splits >= 1 and key != 0


def test_plan_replicate_tables():
    """imps_plan_replicate (host-only context: tables only): every stage repeated per copy, the
    input / output / scratch offsets shifted by the copy index times the slot's length, the
    operator slots shared."""
    from imps_cpp_tools_gb300 import ops
    ctx = B.Context(-1)
    I2K = [(1,), (-1,)]
    b0 = {(-1,): 2, (1,): 3}
    b1 = {(0,): 4, (2,): 1, (-2,): 2}
    la = B.Layout.mps(I2K, b0, b1)
    lb = B.Layout.mps(I2K, b1, b0)
    src = B.plan_tm(ctx, [la, lb], 0, B.Layout.blockdiag(b0), B.Layout.blockdiag(b0))
    rep = ops.plan_replicate(src, 3)
    nst = src.info()["nstages"]
    assert rep.info()["nstages"] == nst
    per = {0, 1} | {s for s in range(src.info()["nslots"]) if s > 3}  # in, out, and the plan's scratch
    for st in range(nst):
        a, b = src.table(st), rep.table(st)
        assert len(b) == 3 * len(a)
        for c in range(3):
            for (tag, terms), (tag2, terms2) in zip(a, b[c * len(a):(c + 1) * len(a)]):
                assert tag == tag2 and len(terms) == len(terms2)
                for (sa, oa, sb, ob, k, al), (sa2, oa2, sb2, ob2, k2, al2) in zip(terms, terms2):
                    assert (sa, sb, k, al) == (sa2, sb2, k2, al2)
                    assert oa2 == oa + (c * src.slot_nelem(sa) if sa in per else 0)
                    assert ob2 == ob + (c * src.slot_nelem(sb) if sb in per else 0)
    assert rep.info()["flops_apply"] == 3 * src.info()["flops_apply"]


def test_cpp_vumps_check_builds(tmp_path):
    """The C++ VUMPS driver (include/imps_vumps.hpp) compiles and links;
    tests/test_gpu_cpp_vumps.py runs it against the Python driver."""
    assert _build_cpp_host(tmp_path, "cpp_vumps_check").exists()
