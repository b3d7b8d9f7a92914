"""The C oracle (CPU restatement of the reference) against the reference's own
outputs: golden fixtures made by tests/golden/make_golden.py from the
reference compiled from its sources."""
import numpy as np
import pytest

from helpers import CASES, TERMS, load_golden, ref_space, rel_errors
from oracle import Oracle


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("use_blas", [True, False])
def test_oracle_terms_match_reference(emax, use_blas):
    g = load_golden(emax)
    o = Oracle(emax, use_blas=use_blas)
    ops = {"X": g["X"], "Y": g["Y"], "W": g["W"]}
    for cs, (a, b, ha, hb) in CASES.items():
        if cs + "_full" not in g:
            continue
        for t in TERMS:
            Z = o.zeros()
            o.term(t, ops[a], ops[b], Z, ha, hb)
            ref = g[cs + "_" + t]
            assert np.abs(Z - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), (cs, t)
        Z = o.commutator(ops[a], ops[b], ha, hb)
        assert max(rel_errors(o.ms, Z, g[cs + "_full"])) < 1e-13, cs


@pytest.mark.parametrize("emax", [2, 3])
def test_oracle_bch_matches_reference(emax):
    g = load_golden(emax)
    o = Oracle(emax)
    X, Y = g["X"], g["Y"]
    out, it = o.bch_transform(X, 1, Y * (0.25 / o.norm(Y)), -1)
    assert 1 <= it <= 40
    assert np.abs(out - g["bch"]).max() < 1e-13


@pytest.mark.parametrize("emax", [2, 3])
def test_oracle_norm_matches_reference(emax):
    g = load_golden(emax)
    o = Oracle(emax)
    for k, name in enumerate("XYW"):
        assert abs(o.norm(g[name]) - g["norms"][k]) < 1e-12 * g["norms"][k]


def test_term_switches():
    g = load_golden(2)
    o = Oracle(2)
    X, Y = g["X"], g["Y"]
    o.set_term("comm222_phss", False)
    Z = o.commutator(X, Y, 1, -1)
    o.set_term("comm222_phss", True)
    ref = g["xy_full"] - g["xy_comm222_phss"]
    assert np.abs(Z - ref).max() < 1e-13


def test_planted_mistake_is_caught():
    """A wrong phase planted in the oracle's input must be visible at the
    tolerance the parity tests use (the test is only as strong as this)."""
    g = load_golden(2)
    o = Oracle(2)
    X = g["X"].copy()
    ms = o.ms
    ch = next(c for c in range(ms.nch) if len(ms.channels[c][3]) > 3)
    blk = ms.block(X, ch)
    blk[1, 2] *= -1
    blk[2, 1] *= -1
    Z = o.commutator(X, g["Y"], 1, -1)
    assert max(rel_errors(ms, Z, g["xy_full"])) > 1e-6


@pytest.mark.parametrize("emax", [2, 3])
def test_oracle_pandya_matches_reference(emax):
    # Commutator::DoPandyaTransformation, both orientations, X hermitian and Y
    # anti-hermitian; the fixture holds every channel's matrix in channel order
    g = load_golden(emax)
    o = Oracle(emax)
    dims = g["pandya_dims"]
    for name, h in (("X", 1), ("Y", -1)):
        for orient in ("normal", "transpose"):
            mats = o.pandya(g[name], h, transpose=orient == "transpose")
            ref = g["pandya_%s_%s" % (name, orient)]
            pos = 0
            for ch, rows, cols in dims:
                shape = (rows, cols) if orient == "normal" else (cols, rows)
                R = ref[pos:pos + rows * cols].reshape(shape, order="F")
                pos += rows * cols
                assert mats[ch].shape == R.shape, (name, orient, ch)
                assert np.abs(mats[ch] - R).max(initial=0.0) <= 1e-14, (name, orient, ch)
            assert pos == ref.size


def parse_reference_binary(ms, raw):
    """Operator::WriteBinary layout (src/Operator.cc:341-363,
    src/TwoBodyME.cc:812-823) of a scalar two-body operator -> (arena,
    hermitian flags, header fields)."""
    import struct
    b = bytes(raw)
    rank_J, rank_T, parity, prank, legs, e2max, e3max = struct.unpack_from("<7i", b, 0)
    herm, anti = struct.unpack_from("<??", b, 28)
    nch, = struct.unpack_from("<i", b, 30)
    pos = 34
    a = np.zeros(ms.arena_size)
    a[0], = struct.unpack_from("<d", b, pos)
    pos += 8
    N = ms.norb
    a[32:32 + N * N] = np.frombuffer(b, dtype="<f8", count=N * N, offset=pos)
    pos += 8 * N * N
    nch2, h2, a2, rj, rt, par = struct.unpack_from("<Q??3i", b, pos)
    pos += 22
    for ch in range(ms.nch):
        n = len(ms.channels[ch][3])
        a[ms.off2[ch]:ms.off2[ch] + n * n] = np.frombuffer(b, dtype="<f8", count=n * n, offset=pos)
        pos += 8 * n * n
    assert pos == len(b)
    return a, (herm, anti, h2, a2), (rank_J, rank_T, parity, prank, legs, e3max, nch, nch2, rj, rt, par)


@pytest.mark.parametrize("emax", [2, 3])
def test_reference_binary_layout(emax):
    # the byte layout the GPU reader and writer follow, pinned on the
    # reference's own files
    g = load_golden(emax)
    ms = ref_space(emax)
    for name, h in (("X", 1), ("Y", -1)):
        a, flags, hdr = parse_reference_binary(ms, g[name + "_binary"])
        assert np.array_equal(a, g[name])
        assert flags == ((h == 1), (h == -1), (h == 1), (h == -1))
        assert hdr == (0, 0, 0, 2, 4, min(14, 3 * emax), ms.nch, ms.nch, 0, 0, 0)


def test_tensor_golden_o18_differs_from_o16():
    # the same X and T on O16's and O18's spaces: the fractional 0d5/2
    # occupations change the reference's scalar-tensor commutator
    from helpers import load_tensor_golden
    g16, g18 = load_tensor_golden(3), load_tensor_golden(3, "O18")
    assert np.array_equal(g16["X"], g18["X"]) and np.array_equal(g16["e2_T"], g18["e2_T"])
    assert np.abs(g16["e2_full"] - g18["e2_full"]).max() > 1e-3
