"""Charge arithmetic of the symmetry group (symobj.hpp:120-158): U(1) components add as
integers, Z_N components modulo N with representatives in [0, N) (symobj's
(x + N) % N).  The device planner only compares charges; every sum is formed here, on the host.

An I2K list carries its group as ``periods`` (0 for a U(1) component, N for Z_N); a plain list
of tuples is all U(1).
"""
from __future__ import annotations


class I2K(list):
    """Physical index -> charge, with the periods of the charge components."""

    def __init__(self, keys, periods):
        super().__init__(tuple(int(x) for x in k) for k in keys)
        self.periods = tuple(int(p) for p in periods)
        if any(len(k) != len(self.periods) for k in self):
            raise ValueError("every charge needs one entry per symmetry component")


def periods_of(i2k):
    p = getattr(i2k, "periods", None)
    return p if p is not None else (0,) * (len(i2k[0]) if len(i2k) else 1)


def _red(x, p):
    return x % p if p else x


def add(a, b, periods):
    return tuple(_red(x + y, p) for x, y, p in zip(a, b, periods))


def sub(a, b, periods):
    return tuple(_red(x - y, p) for x, y, p in zip(a, b, periods))


def neg(a, periods):
    return tuple(_red(-x, p) for x, p in zip(a, periods))


def negated(i2k):
    """The I2K of the transposed tensors: every charge negated, same group."""
    per = periods_of(i2k)
    return I2K([neg(k, per) for k in i2k], per)
