"""Seeded synthetic workloads (no dataset is involved anywhere).

Sector dimensions follow the workload definitions of the benchmark: dims proportional to a
Gaussian weight over the charge sectors, rounded to the total bond dimension by the largest
remainder rule with a minimum of one state per sector.
"""
from __future__ import annotations

import math

import numpy as np


def apportion(weights, total):
    """Largest-remainder rounding of total*w/sum(w) with every entry >= 1."""
    w = np.asarray(weights, dtype=float)
    raw = w / w.sum() * total
    out = np.maximum(np.floor(raw).astype(int), 1)
    frac = raw - np.floor(raw)
    order = np.argsort(-frac, kind="stable")
    rem, i = total - int(out.sum()), 0
    while rem != 0:
        j = order[i % len(order)]
        if rem > 0:
            out[j] += 1
            rem -= 1
        elif out[j] > 1:
            out[j] -= 1
            rem += 1
        i += 1
    return [int(x) for x in out]


def xxz_bond_dims(D, qmax, den):
    """XXZ bond-0 sectors: label 2q (2*Sz), q = -qmax..qmax, dims ~ exp(-q^2/den)."""
    qs = list(range(-qmax, qmax + 1))
    dims = apportion([math.exp(-q * q / den) for q in qs], D)
    return {(2 * q,): m for q, m in zip(qs, dims)}


def hubbard_bond_dims(D, nsec=60):
    """Fermi-Hubbard bond-0 sectors (dN, 2Sz) with dN = 2Sz mod 2, the nsec largest weights
    exp(-(dN^2 + (2Sz)^2)/8) (ties broken lexicographically), dims ~ weight."""
    cand = [(a, b) for a in range(-14, 15) for b in range(-14, 15) if (a - b) % 2 == 0]
    cand.sort(key=lambda t: (-math.exp(-(t[0] ** 2 + t[1] ** 2) / 8.0), t))
    sel = cand[:nsec]
    dims = apportion([math.exp(-(a * a + b * b) / 8.0) for a, b in sel], D)
    return dict(zip(sel, dims))


# name -> (model, bond-0 dims builder, model params)
WORKLOADS = {
    "xxz_d64": ("xxz", lambda: xxz_bond_dims(64, 4, 4.0), {"J": 1.0, "Delta": -1.0}),
    "xxz_d256": ("xxz", lambda: xxz_bond_dims(256, 8, 10.0), {"J": 1.0, "Delta": -1.0}),
    "xxz_d512": ("xxz", lambda: xxz_bond_dims(512, 10, 18.0), {"J": 1.0, "Delta": -1.0}),
    "hubbard_d256": ("fhub", lambda: hubbard_bond_dims(256, 40), {"t": 1.0, "U": 4.0}),
    "hubbard_d1024": ("fhub", lambda: hubbard_bond_dims(1024, 60), {"t": 1.0, "U": 4.0}),
}
