"""Single-operator Pandya transform (Commutator::DoPandyaTransformation,
src/Commutator.cc:1319-1390,1487-1497) on the GPU through the C ABI, against
the reference's own output (golden fixtures) and the C oracle.  Tolerance
1e-14 absolute (unit-norm operators; each element is a short 6j-weighted sum)."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import load_golden
from oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("name,herm", [("X", True), ("Y", False)])
@pytest.mark.parametrize("orient", ["normal", "transpose"])
def test_pandya_vs_reference(emax, name, herm, orient):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    mats = ig.Commutator.DoPandyaTransformation(ig.Operator(ms, arena=g[name], hermitian=herm), orient)
    ref = g["pandya_%s_%s" % (name, orient)]
    pos = 0
    for ch, rows, cols in g["pandya_dims"]:
        shape = (rows, cols) if orient == "normal" else (cols, rows)
        R = ref[pos:pos + rows * cols].reshape(shape, order="F")
        pos += rows * cols
        assert mats[ch].shape == R.shape, ch
        assert np.abs(mats[ch] - R).max(initial=0.0) <= 1e-14, ch


@pytest.mark.parametrize("orient", ["normal", "transpose"])
def test_pandya_vs_oracle(orient):
    emax = 6
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    Z = o.ms.random_operator(909, hermitian=False)
    mats = ig.Commutator.DoPandyaTransformation(ig.Operator(ms, arena=Z, hermitian=False), orient)
    ref = o.pandya(Z, -1, transpose=orient == "transpose")
    assert sum(m.size for m in mats) > 100000
    for a, b in zip(mats, ref):
        assert a.shape == b.shape
        assert np.abs(a - b).max(initial=0.0) <= 1e-14
