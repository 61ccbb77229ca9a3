"""Charge arithmetic of the symmetry groups (symobj.hpp:120-158): U(1) components add as
integers, Z(N) components modulo N with representatives in [0, N); the oracle's kadd / ksub
follow the same rule inside charge_group."""
from imps_cpp_tools_gb300 import blocks as B
from imps_cpp_tools_gb300 import charges, models
from oracle import imps_oracle as O


def test_group_arithmetic():
    per = (0, 3)  # U(1) x Z(3)
    assert charges.add((2, 2), (-5, 2), per) == (-3, 1)
    assert charges.sub((0, 0), (1, 1), per) == (-1, 2)
    assert charges.neg((4, 1), per) == (-4, 2)
    i2k = charges.I2K([(1, 2), (-1, 0)], per)
    assert charges.periods_of(i2k) == per and charges.periods_of([(1,), (2,)]) == (0,)
    assert list(charges.negated(i2k)) == [(-1, 1), (1, 0)] and charges.negated(i2k).periods == per
    with O.charge_group(per):
        assert O.kadd((2, 2), (-5, 2)) == (-3, 1) and O.ksub((0, 0), (1, 1)) == (-1, 2)
    assert O.kadd((2, 2), (-5, 2)) == (-3, 4)  # outside the context: U(1)^2


def test_zn_layouts_wrap_around():
    """Layout.mps of a Z(3) model: level 2 on charge 2 lands on charge 1 (2 + 2 = 4 = 1 mod 3)."""
    d, I2K, _ = models.build_model("potts", q=3)
    dims = {(0,): 2, (1,): 1, (2,): 1}
    L = B.Layout.mps(I2K, dims, dims)
    assert L.find(2, (2,)) >= 0 and L.blocks[L.find(2, (2,))][2] == (1,)
    assert len(L.blocks) == 9  # every level from every sector stays inside Z(3)
