"""6j symbols: the product's double-double table and the oracle's long-double
values against exact rational evaluations (tests/golden/sixj_exact.npz), plus
closed forms and orthogonality at emax 10."""
import math
import os

import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import GOLDEN
from oracle import Oracle


@pytest.fixture(scope="module")
def exact():
    g = np.load(os.path.join(GOLDEN, "sixj_exact.npz"))
    return g["keys"], g["values"]


def test_product_sixj_exact(exact):
    keys, vals = exact
    ms = ig.ModelSpace(4)
    got = np.array([ms.GetSixJ(a / 2, b / 2, c, d / 2, e / 2, f) for (a, b, c, d, e, f) in keys])
    assert np.max(np.abs(got - vals)) <= 1e-16


def test_oracle_sixj_exact(exact):
    keys, vals = exact
    o = Oracle(4)
    got = np.array([o.sixj(a, b, c, d, e, f) for (a, b, c, d, e, f) in keys])
    assert np.max(np.abs(got - vals)) <= 1e-14


def test_closed_form_emax10():
    """{a b c; 0 c b} = (-1)^(a+b+c) / sqrt((2b+1)(2c+1)) written as
    {j c' J; ...} with half-integers: use {j1 j2 J; j2 j1 0} = (-1)^(j1+j2+J)/sqrt((2j1+1)(2j2+1))."""
    ms = ig.ModelSpace(10)
    for jj1 in range(1, 22, 2):
        for jj2 in range(1, 22, 2):
            for J in range(abs(jj1 - jj2) // 2, (jj1 + jj2) // 2 + 1):
                v = ms.GetSixJ(jj1 / 2, jj2 / 2, J, jj2 / 2, jj1 / 2, 0)
                ref = (-1) ** ((jj1 + jj2) // 2 + J) / math.sqrt((jj1 + 1) * (jj2 + 1))
                assert abs(v - ref) < 1e-15


def test_orthogonality_emax10():
    """sum_x (2x+1)(2J+1) {a b x; c d J} {a b x; c d J'} = delta_JJ'."""
    ms = ig.ModelSpace(10)
    for (a, b, c, d) in [(21, 19, 17, 15), (21, 21, 21, 21), (13, 3, 9, 7), (1, 21, 21, 1)]:
        xs = range(abs(a - b) // 2, (a + b) // 2 + 1)
        Js = [J for J in range(0, 22) if abs(a - d) <= 2 * J <= a + d and abs(c - b) <= 2 * J <= c + b]
        for J in Js:
            for Jp in Js:
                s = sum((2 * x + 1) * (2 * J + 1) * ms.GetSixJ(a / 2, b / 2, x, c / 2, d / 2, J)
                        * ms.GetSixJ(a / 2, b / 2, x, c / 2, d / 2, Jp) for x in xs)
                assert abs(s - (1.0 if J == Jp else 0.0)) < 1e-13
