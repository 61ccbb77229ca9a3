"""Generate the golden fixtures of tests/golden/ with the CPU oracle.

    python tests/golden/make_golden.py

Every fixture is seeded and small.  Contents:
  hac_<model>.npz   : an H_AC apply problem (sector tables, operators, input) and the oracle's
                      ApplyHAvec output (VUMPS_helpers.hpp:55-88)
  tm_xxz.npz        : unit-cell transfer-matrix applies, left and right (TMBlockFunctions.hpp)
  tables_<cfg>.npz  : the H_AC sector-matching table at full benchmark size (block pairs the
                      reference's std::map lookups multiply), integer-exact
  vumps_xxz.npz     : three oracle VUMPS sweeps from a fixed initial state (energies, gradient
                      norms, errors) on the Heisenberg D=48 configuration
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from imps_cpp_tools_gb300 import models  # noqa: E402
from oracle import imps_oracle as O  # noqa: E402
from tests import imps_testlib as T  # noqa: E402

SMALL = {"xxz": {(-4,): 1, (-2,): 3, (0,): 5, (2,): 3, (4,): 1},
         "fhub": {(0, 0): 4, (1, 1): 2, (-1, -1): 2, (1, -1): 2, (-1, 1): 2, (2, 0): 1, (0, 2): 1}}
BETHE_B0 = {(-4,): 3, (-2,): 8, (0,): 10, (2,): 8, (4,): 3}
BETHE_B1 = {(-5,): 1, (-3,): 5, (-1,): 10, (1,): 10, (3,): 5, (5,): 1}


def blocks_arrays(blocks, nsym):
    g = np.array([b[0] for b in blocks], np.int32)
    qi = np.array([b[1] for b in blocks], np.int32).reshape(-1, nsym)
    qo = np.array([b[2] for b in blocks], np.int32).reshape(-1, nsym)
    r = np.array([b[3] for b in blocks], np.int32)
    c = np.array([b[4] for b in blocks], np.int32)
    return g, qi, qo, r, c


def save_layout(d, prefix, blocks, nsym):
    g, qi, qo, r, c = blocks_arrays(blocks, nsym)
    d[prefix + "_g"], d[prefix + "_qin"], d[prefix + "_qout"], d[prefix + "_r"], d[prefix + "_c"] = g, qi, qo, r, c


def expected_hac_pairs(p):
    """The block pairs ApplyHA multiplies (map lookups on the oracle's dicts), flattened."""
    d, AC, EHL, EHR, HL, HR = p["d"], p["AC"], p["EHL"], p["EHR"], p["HL"], p["HR"]

    def offs(blocks):
        o, out = 0, {}
        for (g, qi, qo, r, c) in blocks:
            out[(g, qi)] = o
            o += r * c
        return out
    oac, oel, oer = offs(T.mps_blocks(AC)), offs(T.bd_blocks(EHL)), offs(T.bd_blocks(EHR))
    ohl, ohr = offs(T.redop_blocks(HL, d)), offs(T.redop_blocks(HR, d))
    rows = []
    blk = 0
    for s in range(d):
        for ql in sorted(AC[s]):
            qr = AC[s][ql][0]
            if ql in EHL:
                rows.append((blk, 2, oel[(0, ql)], 0, oac[(s, ql)]))
            if qr in EHR:
                rows.append((blk, 0, oac[(s, ql)], 3, oer[(0, qr)]))
            for j in range(d):
                if ql in HL[s][j]:
                    ql2 = HL[s][j][ql][0]
                    if ql2 in AC[j] and AC[j][ql2][0] == qr:
                        rows.append((blk, 4, ohl[(s * d + j, ql)], 0, oac[(j, ql2)]))
                if ql in AC[j]:
                    qr2 = AC[j][ql][0]
                    if qr2 in HR[s][j] and HR[s][j][qr2][0] == qr:
                        rows.append((blk, 0, oac[(j, ql)], 5, ohr[(s * d + j, qr2)]))
            blk += 1
    return np.array(rows, np.int64)


def make_hac(model, dims0, seed, **params):
    p = T.hac_problem(model, dims0, seed=seed, **params)
    d, ns = p["d"], len(p["I2K"][0])
    out = {"d": np.int32(d), "nsym": np.int32(ns)}
    save_layout(out, "ac", T.mps_blocks(p["AC"]), ns)
    save_layout(out, "ehl", T.bd_blocks(p["EHL"]), ns)
    save_layout(out, "ehr", T.bd_blocks(p["EHR"]), ns)
    save_layout(out, "hl", T.redop_blocks(p["HL"], d), ns)
    save_layout(out, "hr", T.redop_blocks(p["HR"], d), ns)
    out["EHL"], out["EHR"] = O.bd_vec(p["EHL"]), O.bd_vec(p["EHR"])
    out["HL"], out["HR"] = T.redop_vec(p["HL"], d), T.redop_vec(p["HR"], d)
    x = p["rng"].standard_normal(sum(b[3] * b[4] for b in T.mps_blocks(p["AC"])))
    out["x"] = x
    out["y"] = O.ApplyHAvec(x, O.mps_sizes(p["AC"]), p["EHL"], p["EHR"], p["HL"], p["HR"])
    return out, p


def main():
    os.makedirs(HERE, exist_ok=True)
    for model in ("xxz", "fhub"):
        out, _ = make_hac(model, SMALL[model], seed=101)
        np.savez_compressed(os.path.join(HERE, f"hac_{model}.npz"), **out)
    # transfer matrices on the XXZ small unit cell
    st = T.random_state("xxz", SMALL["xxz"], seed=102)
    AL, dv, rng = st["AL"], st["dimvec"], st["rng"]
    X = T.rand_bd(dv[0], rng, sym=False)
    tm = {"nsym": np.int32(1)}
    save_layout(tm, "a0", T.mps_blocks(AL[0]), 1)
    save_layout(tm, "a1", T.mps_blocks(AL[1]), 1)
    save_layout(tm, "bond", T.bd_blocks(X), 1)
    tm["A0"], tm["A1"], tm["X"] = O.mps_vec(AL[0]), O.mps_vec(AL[1]), O.bd_vec(X)
    tm["YL"], tm["YR"] = O.bd_vec(O.ApplyTMLeftUC(AL, X)), O.bd_vec(O.ApplyTMRightUC(AL, X))
    np.savez_compressed(os.path.join(HERE, "tm_xxz.npz"), **tm)
    # full-size sector-matching tables
    for cfg in ("xxz_d512", "hubbard_d1024"):
        model, dims0, params = T.workload_dims(cfg)
        p = T.hac_problem(model, dims0, seed=3, **params)
        ns = len(p["I2K"][0])
        tab = {"pairs": expected_hac_pairs(p), "nsym": np.int32(ns), "d": np.int32(p["d"])}
        save_layout(tab, "ac", T.mps_blocks(p["AC"]), ns)
        save_layout(tab, "ehl", T.bd_blocks(p["EHL"]), ns)
        save_layout(tab, "ehr", T.bd_blocks(p["EHR"]), ns)
        save_layout(tab, "hl", T.redop_blocks(p["HL"], p["d"]), ns)
        save_layout(tab, "hr", T.redop_blocks(p["HR"], p["d"]), ns)
        np.savez_compressed(os.path.join(HERE, f"tables_{cfg}.npz"), **tab)
    # three oracle VUMPS sweeps on the Heisenberg D=48 configuration
    d, I2K, h = models.build_model("xxz", J=1.0, Delta=-1.0)
    rng = np.random.default_rng(7)
    dimvec = [BETHE_B0, BETHE_B1]
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, rng)
    v = O.VUMPS(h, d, I2K, BETHE_B0, dimvec=dimvec, init=(AL, AR, C), fixed_tol=1e-12, seed=7)
    E, F, P = [], [], []
    for _ in range(3):
        e, f, pr = v.sweep()
        E.append(e); F.append(f); P.append(pr)
    vm = {"AL0": O.mps_vec(AL[0]), "AL1": O.mps_vec(AL[1]), "AR0": O.mps_vec(AR[0]), "AR1": O.mps_vec(AR[1]),
          "C_bond0": O.bd_vec(C[1]), "C_bond1": O.bd_vec(C[0]), "E": np.array(E), "F": np.array(F),
          "prec": np.array(P)}
    np.savez_compressed(os.path.join(HERE, "vumps_xxz.npz"), **vm)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
