"""Scalar-tensor commutator [X, T] (X scalar, T a reduced tensor) on the GPU
through the C ABI, against the reference's own outputs
(golden_tensor_emax*.npz, from Commutator::CommutatorScalarTensor and its
terms, src/TensorCommutators.cc).  Tensor ranks (J, |dTz|, parity): (2, 0, 0)
hermitian, (1, 0, 1) hermitian, (1, 1, 0) anti-hermitian.  FP64 throughout;
tolerance 1e-12 relative Frobenius per body rank."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import load_flow_golden, load_tensor_golden, ref_space, tensor_rel_errors

pytestmark = pytest.mark.gpu

TOL = 1e-12
TERMS = ["comm111st", "comm121st", "comm122st", "comm222_pp_hh_221st", "comm222_phst"]
CASES = [(2, "e2"), (2, "e1"), (2, "gt"), (3, "e2")]


def setup(emax, case):
    g = load_tensor_golden(emax)
    lam, trank, par, herm = (int(x) for x in g[case + "_rank"])
    ms = ig.ModelSpace(emax, "O16", "O16")
    dX = ig.DeviceOperator(ms, 1)
    dX.upload(g["X"])
    dT = ig.DeviceOperator(ms, herm, (lam, trank, par))
    dT.upload(g[case + "_T"])
    return g, ms, dX, dT, (lam, trank, par), herm


@pytest.mark.parametrize("emax,case", CASES)
@pytest.mark.parametrize("term", TERMS)
def test_tensor_term_vs_reference(emax, case, term):
    g, ms, dX, dT, rank, herm = setup(emax, case)
    hz = -1 if herm == 1 else 1
    with ig.DeviceOperator(ms, hz, rank) as dZ:
        ig.Commutator.device_tensor_term(term, dX, dT, dZ)
        Z = dZ.download()
    R = g["%s_%s" % (case, term)]
    errs = tensor_rel_errors(ref_space(emax), rank, Z, R)
    assert max(errs) < TOL, (term, errs)


@pytest.mark.parametrize("emax,case", CASES)
def test_commutator_scalar_tensor_vs_reference(emax, case):
    g, ms, dX, dT, rank, herm = setup(emax, case)
    with ig.DeviceOperator(ms, 1, rank) as dZ:
        dZ.upload(np.full(dZ.size, 3.0))  # overwritten
        ig.Commutator.device_scalar_tensor(dX, dT, dZ)
        assert dZ.hermiticity == (-1 if herm == 1 else 1)
        Z = dZ.download()
    errs = tensor_rel_errors(ref_space(emax), rank, Z, g[case + "_full"])
    assert max(errs) < TOL, errs


def test_host_api_dispatch():
    # Commutator.Commutator dispatches on rank; [T, S] = -[S, T]
    g = load_tensor_golden(2)
    ms = ig.ModelSpace(2, "O16", "O16")
    X = ig.Operator(ms, arena=g["X"], hermitian=True)
    T = ig.Operator(ms, 2, 0, 0, 2, arena=g["e2_T"], hermitian=True)
    Z = ig.Commutator.Commutator(X, T)
    assert Z.rank == (2, 0, 0) and Z.IsAntiHermitian()
    assert max(tensor_rel_errors(ref_space(2), (2, 0, 0), Z.arena, g["e2_full"])) < TOL
    W = ig.Commutator.Commutator(T, X)
    assert np.allclose(W.arena, -Z.arena, rtol=0, atol=1e-15)


def test_tensor_rejected_by_scalar_paths():
    ms = ig.ModelSpace(2, "O16", "O16")
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, 1, (2, 0, 0)) as dT, \
            ig.DeviceOperator(ms, -1) as dZ:
        with pytest.raises(ig.IMSRGError):
            ig.Commutator.device_commutator(dX, dT, dZ)
        with pytest.raises(ig.IMSRGError):  # Omega must be scalar
            ig.BCH.device_transform(dX, dT, dZ)


# ------------------------------------------------------------- split form
# The ladder and Z bar products on the tensor cores (plain split products);
# every other sum stays FP64.  Tolerance 1e-10 relative Frobenius per body
# rank, as for the scalar commutator's split form.
SPLIT_TOL = 1e-10


@pytest.mark.parametrize("emax,case", CASES)
def test_commutator_scalar_tensor_split_vs_reference(emax, case):
    g, ms, dX, dT, rank, herm = setup(emax, case)
    with ig.DeviceOperator(ms, 1, rank) as dZ:
        dZ.upload(np.full(dZ.size, 3.0))  # overwritten
        ig.Commutator.device_scalar_tensor(dX, dT, dZ, precision="split")
        Z = dZ.download()
    errs = tensor_rel_errors(ref_space(emax), rank, Z, g[case + "_full"])
    assert max(errs) < SPLIT_TOL, errs


@pytest.mark.parametrize("emax,case", [(2, "e2"), (2, "gt"), (3, "e2")])
@pytest.mark.parametrize("term", ["comm222_pp_hh_221st", "comm222_phst"])
def test_tensor_term_split_vs_reference(emax, case, term):
    g, ms, dX, dT, rank, herm = setup(emax, case)
    hz = -1 if herm == 1 else 1
    with ig.DeviceOperator(ms, hz, rank) as dZ:
        ig.Commutator.device_tensor_term(term, dX, dT, dZ, precision="split")
        Z = dZ.download()
    errs = tensor_rel_errors(ref_space(emax), rank, Z, g["%s_%s" % (case, term)])
    assert max(errs) < SPLIT_TOL, (term, errs)


@pytest.mark.parametrize("rank,herm", [((2, 0, 0), 1), ((1, 1, 0), -1), ((3, 0, 1), 1), ((0, 1, 0), 1),
                                       ((4, 0, 0), -1), ((2, 1, 1), 1)])
def test_tensor_split_vs_fp64_emax5(rank, herm):
    # larger channels than the golden spaces (several 128-row tiles, ragged
    # edges, K past one pipeline stage): the split form against the FP64 one,
    # for ranks from lambda = 0 (isovector, |dTz| = 1) to lambda = 4
    ms = ig.ModelSpace(5, "O16", "O16")
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, herm, rank) as dT, \
            ig.DeviceOperator(ms, 1, rank) as dF, ig.DeviceOperator(ms, 1, rank) as dS:
        dX.fill_random(5)
        dT.upload(ref_space(5).random_tensor(9, *rank, hermitian=herm == 1))
        ig.Commutator.device_scalar_tensor(dX, dT, dF, precision="fp64")
        ig.Commutator.device_scalar_tensor(dX, dT, dS, precision="split")
        F, S = dF.download(), dS.download()
    errs = tensor_rel_errors(ref_space(5), rank, S, F)
    assert max(errs) < SPLIT_TOL, errs


# ------------------------------------------------- O18 (fractional occupations)
# The reference's terms on O18's space (0d5/2 neutrons at 1/3): the hole /
# particle branches of the one-body terms and the ladder weights see
# fractional occupations (golden_tensor_emax3_O18.npz).
@pytest.mark.parametrize("case", ["e2", "gt"])
@pytest.mark.parametrize("prec,tol", [("fp64", TOL), ("split", SPLIT_TOL)])
def test_tensor_o18_vs_reference(case, prec, tol):
    g = load_tensor_golden(3, "O18")
    lam, trank, par, herm = (int(x) for x in g[case + "_rank"])
    rank = (lam, trank, par)
    ms = ig.ModelSpace(3, "O18", "O18")
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, herm, rank) as dT, \
            ig.DeviceOperator(ms, 1, rank) as dZ:
        dX.upload(g["X"])
        dT.upload(g[case + "_T"])
        ig.Commutator.device_scalar_tensor(dX, dT, dZ, precision=prec)
        Z = dZ.download()
    errs = tensor_rel_errors(ref_space(3), rank, Z, g[case + "_full"])
    assert max(errs) < tol, (case, prec, errs)
    if prec == "fp64":
        hz = -1 if herm == 1 else 1
        for term in TERMS:
            with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, herm, rank) as dT, \
                    ig.DeviceOperator(ms, hz, rank) as dZ:
                dX.upload(g["X"])
                dT.upload(g[case + "_T"])
                ig.Commutator.device_tensor_term(term, dX, dT, dZ)
                R = g["%s_%s" % (case, term)]
                errs = tensor_rel_errors(ref_space(3), rank, dZ.download(), R)
            assert max(errs) < TOL, (case, term, errs)


# ------------------------------------------ norms, BCH_Transform, Transform
# Operator::Norm of a tensor, BCH::BCH_Transform of a tensor by a scalar
# Omega (the reference's own: Omega = 0.2 X / |X| and its transform of T are
# in the golden files), and IMSRGSolver::Transform of an observable.
@pytest.mark.parametrize("emax,case", CASES)
def test_tensor_norm_vs_reference(emax, case):
    g, ms, dX, dT, rank, herm = setup(emax, case)
    nT, nZ, nB, n1, n2 = g[case + "_norms"]
    assert abs(dT.norm() - nT) <= 1e-13 * nT
    with ig.DeviceOperator(ms, 1, rank) as dZ:
        ig.Commutator.device_scalar_tensor(dX, dT, dZ, precision="fp64")
        assert abs(dZ.norm() - nZ) <= 1e-12 * nZ


@pytest.mark.parametrize("emax,case", CASES)
@pytest.mark.parametrize("prec,tol", [("fp64", TOL), ("split", SPLIT_TOL)])
def test_tensor_bch_transform_vs_reference(emax, case, prec, tol):
    g, ms, dX, dT, rank, herm = setup(emax, case)
    with ig.DeviceOperator(ms, 1) as dOm, ig.DeviceOperator(ms, herm, rank) as dB:
        dOm.upload(g[case + "_omega"])
        n = ig.BCH.device_transform(dT, dOm, dB, prec)
        assert n >= 3
        B = dB.download()
        assert abs(dB.norm() - g[case + "_norms"][2]) <= 10 * tol * g[case + "_norms"][2]
    errs = tensor_rel_errors(ref_space(emax), rank, B, g[case + "_bch"])
    assert max(errs) < tol, (case, prec, errs)
    # host API: BCH.BCH_Transform keeps the tensor's rank
    T = ig.Operator(ms, *rank, arena=g[case + "_T"], hermitian=herm == 1)
    Om = ig.Operator(ms, arena=g[case + "_omega"])
    Bh = ig.BCH.BCH_Transform(T, Om, prec)
    assert Bh.rank == rank
    assert max(tensor_rel_errors(ref_space(emax), rank, Bh.arena, g[case + "_bch"])) < tol


def test_solver_transform_of_a_tensor_observable():
    # Transform(T) after a flow with several Omegas is the chain of
    # BCH_Transforms through them, and InverseTransform undoes it
    gf = load_flow_golden(3)
    g = load_tensor_golden(3)
    ms = ig.ModelSpace(3, "O16", "O16")
    rank = (2, 0, 0)
    H = ig.Operator(ms, arena=gf["H"])
    solver = ig.IMSRGSolver(H, precision="fp64")
    solver.SetOmegaNormMax(0.3)
    solver.SetSmax(2.0)
    solver.Solve()
    assert solver.GetOmegaSize() > 1
    T = ig.Operator(ms, *rank, arena=g["e2_T"], hermitian=True)
    Tt = solver.Transform(T)
    ref = T
    for i in range(solver.GetOmegaSize()):
        ref = ig.BCH.BCH_Transform(ref, solver.GetOmega(i), "fp64")
    assert max(tensor_rel_errors(ref_space(3), rank, Tt.arena, ref.arena)) < 1e-12
    back = solver.InverseTransform(Tt)
    assert max(tensor_rel_errors(ref_space(3), rank, back.arena, T.arena)) < 1e-8


@pytest.mark.parametrize("off,dropped", [("comm222_phst", ["comm222_phst"]),
                                         ("comm221st", ["comm222_pp_hh_221st"]),
                                         ("comm122st", ["comm122st"])])
def test_tensor_term_switches(off, dropped):
    # Commutator::TurnOffTerm, as CommutatorScalarTensor consults it
    # (comm222_pp_hh_221st needs both comm222_pp_hhst and comm221st)
    g, ms, dX, dT, rank, herm = setup(2, "e2")
    R = g["e2_full"].copy()
    for t in dropped:
        R -= g["e2_" + t]
    ig.Commutator.TurnOffTerm(off)
    try:
        for prec in ("fp64", "split"):
            with ig.DeviceOperator(ms, 1, rank) as dZ:
                ig.Commutator.device_scalar_tensor(dX, dT, dZ, precision=prec)
                Z = dZ.download()
            errs = tensor_rel_errors(ref_space(2), rank, Z, R)
            assert max(errs) < (TOL if prec == "fp64" else SPLIT_TOL), (off, prec, errs)
    finally:
        ig.Commutator.TurnOnTerm(off)
    assert ig.Commutator.IsTermOn(off)
