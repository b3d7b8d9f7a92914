"""GPU parity through the C ABI: every IMSRG(2) term, the full commutator and
the BCH transform against the reference's own outputs (golden fixtures,
emax 2 and 3) and against the C oracle (emax 4 to 6).

Tolerance (plain FP64 form): relative Frobenius error per body rank <= 1e-12
(summation order differs from the reference's BLAS, so results are not
bitwise equal)."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import CASES, TERMS, load_golden, rel_errors, ref_space
from oracle import Oracle

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def run_term(ms, name, A, B, hA, hB, hZ, precision="fp64"):
    with ig.DeviceOperator(ms, hA) as dA, ig.DeviceOperator(ms, hB) as dB, ig.DeviceOperator(ms, hZ) as dZ:
        dA.upload(A)
        dB.upload(B)
        if name == "comm222_pp_hh_221ss":
            ig.Commutator.device_term(name, dA, dB, dZ, precision)
        else:
            ig.Commutator.device_term(name, dA, dB, dZ, precision)
        return dZ.download()


def run_full(ms, A, B, hA, hB, precision="fp64"):
    with ig.DeviceOperator(ms, hA) as dA, ig.DeviceOperator(ms, hB) as dB, ig.DeviceOperator(ms, 1) as dZ:
        dA.upload(A)
        dB.upload(B)
        ig.Commutator.device_commutator(dA, dB, dZ, precision)
        return dZ.download(), dZ.hermiticity


@pytest.mark.parametrize("emax", [2, 3])
def test_terms_vs_reference(emax):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    ops = {"X": g["X"], "Y": g["Y"], "W": g["W"]}
    for cs, (a, b, ha, hb) in CASES.items():
        if cs + "_full" not in g:
            continue
        hz = -1 if ha == hb else 1
        scale = np.linalg.norm(g[cs + "_full"])
        for t in TERMS:
            Z = run_term(ms, t, ops[a], ops[b], ha, hb, hz)
            errs = rel_errors(r, Z, g[cs + "_" + t], floor=scale)
            assert max(errs) < TOL_FP64, (cs, t, errs)


@pytest.mark.parametrize("emax", [2, 3])
def test_full_commutator_vs_reference(emax):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    ops = {"X": g["X"], "Y": g["Y"], "W": g["W"]}
    for cs, (a, b, ha, hb) in CASES.items():
        if cs + "_full" not in g:
            continue
        Z, hz = run_full(ms, ops[a], ops[b], ha, hb)
        assert hz == (-1 if ha == hb else 1)
        errs = rel_errors(r, Z, g[cs + "_full"])
        assert max(errs) < TOL_FP64, (cs, errs)


@pytest.mark.parametrize("emax", [2, 3])
def test_bch_vs_reference(emax):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    X = ig.Operator(ms, arena=g["X"], hermitian=True)
    Y = ig.Operator(ms, arena=g["Y"], hermitian=False)
    Om = Y * (0.25 / Y.Norm())
    Hs = ig.BCH.BCH_Transform(X, Om, precision="fp64")
    errs = rel_errors(r, Hs.arena, g["bch"])
    assert max(errs) < TOL_FP64, errs
    assert abs(Hs.ZeroBody - g["bch"][0]) < 1e-12 * abs(g["bch"][0])


@pytest.mark.parametrize("emax", [4, 5])
def test_terms_vs_oracle(emax):
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    X = o.ms.random_operator(11 + emax, True)
    Y = o.ms.random_operator(21 + emax, False)
    for t in TERMS:
        R = o.zeros()
        o.term(t, X, Y, R, 1, -1)
        Z = run_term(ms, t, X, Y, 1, -1, 1)
        errs = rel_errors(o.ms, Z, R, floor=1.0)
        assert max(errs) < TOL_FP64, (t, errs)


def test_full_vs_oracle_emax6():
    o = Oracle(6)
    ms = ig.ModelSpace(6, "O16", "O16")
    X = o.ms.random_operator(101, True)
    Y = o.ms.random_operator(202, False)
    R = o.commutator(X, Y, 1, -1)
    Z, hz = run_full(ms, X, Y, 1, -1)
    errs = rel_errors(o.ms, Z, R)
    assert max(errs) < TOL_FP64, errs


def test_accumulates_into_z():
    """Terms add to what Z holds, as the reference's comm*ss(X, Y, Z) do."""
    g = load_golden(2)
    ms = ig.ModelSpace(2, "O16", "O16")
    r = ref_space(2)
    Z0 = r.random_operator(7, True)
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.upload(g["X"])
        dY.upload(g["Y"])
        dZ.upload(Z0)
        ig.Commutator.device_term("comm222_phss", dX, dY, dZ, "fp64")
        Z = dZ.download()
    errs = rel_errors(r, Z - Z0, g["xy_comm222_phss"], floor=1.0)
    assert max(errs) < TOL_FP64


def test_norm_and_axpy():
    g = load_golden(3)
    ms = ig.ModelSpace(3, "O16", "O16")
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY:
        dX.upload(g["X"])
        dY.upload(g["Y"])
        assert abs(dX.norm() - g["norms"][0]) < 1e-12 * g["norms"][0]
        dX.axpy(0.5, dY)
        ref = g["X"] + 0.5 * g["Y"]
        assert np.abs(dX.download() - ref).max() < 1e-15


def test_random_fill_symmetry():
    ms = ig.ModelSpace(4, "O16", "O16")
    r = ref_space(4)
    for h in (1, -1):
        with ig.DeviceOperator(ms, h) as d:
            d.fill_random(5)
            a = d.download()
        one = r.onebody(a)
        assert np.allclose(one, h * one.T, atol=0)
        assert abs(np.linalg.norm(one) - 1) < 1e-12
        for c in range(r.nch):
            b = r.block(a, c)
            if b.size:
                assert np.allclose(b, h * b.T, atol=0)
                if b.shape[0] > 1 or h == 1:  # a 1x1 anti-hermitian block is zero
                    assert abs(np.linalg.norm(b) - 1) < 1e-12
