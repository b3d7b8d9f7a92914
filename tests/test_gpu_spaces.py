"""The commutator on other reference nuclei and edge-case spaces, against the
C oracle (the reference's formulas carry general occupations: the pp/hh/ph
weights and the occupation factors of every term):

  emax 1, O16: every orbit occupied (no particle states, no pp kets, empty
               ladder and particle-hole products)
  emax 2, He4: a different hole set
  emax 3, O18: fractional occupations (0d5/2 neutrons at 1/3)
  emax 4, Ca40: holes up to the 1s0d shell

FP64 to 1e-12 and split to 1e-10 relative Frobenius per body rank."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import rel_errors
from oracle import Oracle

pytestmark = pytest.mark.gpu

SPACES = [(1, 16, 8, "O16"), (2, 4, 2, "He4"), (3, 18, 8, "O18"), (4, 40, 20, "Ca40")]


@pytest.mark.parametrize("emax,A,Z,name", SPACES)
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("split", 1e-10)])
@pytest.mark.parametrize("hy", [-1, 1])
def test_commutator_other_spaces(emax, A, Z, name, prec, tol, hy):
    o = Oracle(emax, A, Z)
    ms = ig.ModelSpace(emax, name, name)
    assert ms.norb == o.ms.norb and ms.arena_size == o.ms.arena_size
    occ = np.array([x[4] for x in ms.orbits])
    assert np.allclose(occ, o.ms.occ)
    X = o.ms.random_operator(100 + A, True)
    Y = o.ms.random_operator(200 + A, hy > 0)
    R = o.commutator(X, Y, 1, hy)
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, hy) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.upload(X)
        dY.upload(Y)
        ig.Commutator.device_commutator(dX, dY, dZ, prec)
        Z = dZ.download()
    errs = rel_errors(o.ms, Z, R)
    assert max(errs) < tol, (name, prec, errs)


def test_fractional_occupations_reach_the_result():
    # O18's partly filled 0d5/2 changes the commutator: the occupations are used
    o16, o18 = Oracle(3, 16, 8), Oracle(3, 18, 8)
    X = o16.ms.random_operator(5, True)
    Y = o16.ms.random_operator(6, False)
    assert np.abs(o16.commutator(X, Y, 1, -1) - o18.commutator(X, Y, 1, -1)).max() > 1e-3
