"""BCH_Product, the White-type generators and the Magnus-Euler solver on the
GPU through the C ABI, against the reference's own outputs
(golden_flow_emax*.npz) and the C oracle.

Tolerances: relative Frobenius error per body rank <= 1e-12 for one
BCH_Product in FP64 and <= 1e-10 in the split form (those of one commutator);
1e-13 elementwise for the generator (no products, only denominators); for a
flow of ten steps (about sixty commutators) the zero-body energy at every
step and the final H(s) and Omega per body rank to 1e-12 (FP64) and 1e-10
(split).  Measured on a GB300: at most 8e-16 (FP64) and 2.2e-13 (split)."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import load_flow_golden, rel_errors, ref_space
from oracle import FlowParams, Oracle

pytestmark = pytest.mark.gpu

TOL_PROD = {"fp64": 1e-12, "split": 1e-10}
TOL_E0 = {"fp64": 1e-12, "split": 1e-10}
TOL_OPS = {"fp64": 1e-12, "split": 1e-10}


def dev(ms, a, h):
    d = ig.DeviceOperator(ms, h)
    d.upload(a)
    return d


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_bch_product_vs_reference(emax, prec):
    g = load_flow_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    for scale, key in ((1.0, "bchp"), (None, "bchp_big")):
        A = g["A"] if scale else 6.0 * g["A"]
        B = g["B"] if scale else 2.0 * g["B"]
        with dev(ms, A, -1) as dA, dev(ms, B, -1) as dB, ig.DeviceOperator(ms, -1) as dZ:
            n = ig.BCH.device_product(dA, dB, dZ, prec)
            assert n >= 2
            assert dZ.hermiticity == -1
            errs = rel_errors(r, dZ.download(), g[key])
        assert max(errs) < TOL_PROD[prec], (key, errs)


def test_bch_product_aliasing():
    # Z may be X or Y (the Magnus step updates Omega in place)
    g = load_flow_golden(3)
    ms = ig.ModelSpace(3, "O16", "O16")
    A, B = 6.0 * g["A"], 2.0 * g["B"]
    with dev(ms, A, -1) as dA, dev(ms, B, -1) as dB, ig.DeviceOperator(ms, -1) as dZ:
        ig.BCH.device_product(dA, dB, dZ, "fp64")
        ref = dZ.download()
        ig.BCH.device_product(dA, dB, dB, "fp64")
        assert np.array_equal(dB.download(), ref)
        dB.upload(B)
        ig.BCH.device_product(dA, dB, dA, "fp64")
        assert np.array_equal(dA.download(), ref)


def test_bch_product_host_api():
    g = load_flow_golden(2)
    ms = ig.ModelSpace(2, "O16", "O16")
    X = ig.Operator(ms, arena=g["A"], hermitian=False)
    Y = ig.Operator(ms, arena=g["B"], hermitian=False)
    Z = ig.BCH.BCH_Product(X, Y, precision="fp64")
    assert Z.IsAntiHermitian()
    assert max(rel_errors(ref_space(2), Z.arena, g["bchp"])) < 1e-12


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("case", [("eta_white", "white", "Epstein_Nesbet"), ("eta_atan", "atan", "Epstein_Nesbet"),
                                  ("eta_white_mp", "white", "Moller_Plesset"),
                                  ("eta_qt", "qtransfer-atan", "Epstein_Nesbet"),
                                  ("eta_qt2", "qtransfer-atan_2", "Epstein_Nesbet")])
def test_generator_vs_reference(emax, case):
    key, kind, part = case
    g = load_flow_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    gen = ig.Generator()
    gen.SetType(kind)
    gen.SetDenominatorPartitioning(part)
    H = ig.Operator(ms, arena=g["H"])
    Eta = ig.Operator(ms, hermitian=False)
    Eta.arena[:] = 1.0  # Update overwrites
    gen.Update(H, Eta)
    assert Eta.IsAntiHermitian()
    assert np.abs(Eta.arena - g[key]).max() <= 1e-13 * np.abs(g[key]).max()


@pytest.mark.parametrize("kind", ["white", "wegner", "imaginary-time"])
def test_generator_vs_oracle(kind):
    emax = 6
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    H = o.ms.flow_hamiltonian(77, 0.5)
    # a delta on every denominator and a cutoff that catches some of them
    R = o.generator(H, kind, "Epstein_Nesbet", cutoff=0.5, delta=0.25, delta_index=-12345)
    gen = ig.Generator()
    gen.SetType(kind)
    gen.SetDenominatorCutoff(0.5)
    gen.SetDenominatorDelta(0.25)
    gen.SetDenominatorDeltaIndex(-12345)
    with dev(ms, H, 1) as dH, ig.DeviceOperator(ms, -1) as dE:
        gen.device_update(dH, dE)
        E = dE.download()
    assert np.abs(R).max() > 0
    assert np.abs(E - R).max() <= 1e-13 * np.abs(R).max()


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_fixed_step_flow_vs_reference(emax, prec):
    g = load_flow_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    steps = g["flow_steps"]
    solver = ig.IMSRGSolver(ig.Operator(ms, arena=g["H"]), precision=prec)
    solver.SetGenerator("white")
    solver.SetDs(0.5)
    solver.SetDsmax(0.5)
    solver.SetMagnusAdaptive(False)
    solver.SetOmegaNormMax(1e9)
    solver.SetEtaCriterion(1e-20)
    solver.SetSmax(0.5 * len(steps))
    solver.Solve()
    it, s, e0, _, _ = solver.history()
    assert list(it) == list(range(1, len(steps) + 1))
    np.testing.assert_array_equal(s, steps[:, 0])
    np.testing.assert_allclose(e0, steps[:, 1], rtol=TOL_E0[prec])
    assert solver.GetS() == steps[-1, 0]
    assert max(rel_errors(r, solver.GetH_s().arena, g["flow_Hs"])) < TOL_OPS[prec]
    assert max(rel_errors(r, solver.GetOmega(0).arena, g["flow_Omega"])) < TOL_OPS[prec]


@pytest.mark.parametrize("emax", [2, 3])
def test_adaptive_split_flow_vs_reference(emax):
    g = load_flow_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    s_ref, n_omega_ref, e0_ref = g["flow2"]
    solver = ig.IMSRGSolver(ig.Operator(ms, arena=g["H"]), precision="fp64")
    solver.SetGenerator("white")
    solver.SetOmegaNormMax(0.3)
    solver.SetEtaCriterion(1e-20)
    solver.SetSmax(2.0)
    solver.Solve()
    assert solver.GetS() == s_ref
    assert solver.GetOmegaSize() == int(n_omega_ref) > 1
    Hs = solver.GetH_s()
    assert abs(Hs.ZeroBody - e0_ref) <= TOL_E0["fp64"] * abs(e0_ref)
    assert max(rel_errors(r, Hs.arena, g["flow2_Hs"])) < TOL_OPS["fp64"]
    last = solver.GetOmega(solver.GetOmegaSize() - 1)
    assert max(rel_errors(r, last.arena, g["flow2_Omega"])) < TOL_OPS["fp64"]


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_fixed_step_flow_vs_oracle(prec):
    emax = 5
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    H = o.ms.flow_hamiltonian(5005, 0.5)
    p = FlowParams(ds=0.5, ds_max=0.5, smax=2.0, magnus_adaptive=0, omega_norm_max=1e9, eta_criterion=1e-20)
    R = o.magnus_euler(H, p)
    solver = ig.IMSRGSolver(ig.Operator(ms, arena=H), precision=prec)
    for name, v in (("SetDs", 0.5), ("SetDsmax", 0.5), ("SetSmax", 2.0), ("SetOmegaNormMax", 1e9),
                    ("SetEtaCriterion", 1e-20)):
        getattr(solver, name)(v)
    solver.SetMagnusAdaptive(False)
    solver.Solve()
    _, s, e0, _, _ = solver.history()
    assert len(e0) == R["steps"] == 4
    np.testing.assert_allclose(e0, R["e0_hist"], rtol=TOL_E0[prec])
    assert max(rel_errors(o.ms, solver.GetH_s().arena, R["Hs"])) < TOL_OPS[prec]


@pytest.mark.parametrize("hunter_gatherer", [False, True])
def test_transform_reproduces_flowing_hamiltonian(hunter_gatherer):
    # Omega split (or gathered) along the way: Transform(H0) through every
    # Omega is H(s), and InverseTransform undoes Transform
    g = load_flow_golden(3)
    ms = ig.ModelSpace(3, "O16", "O16")
    r = ref_space(3)
    H = ig.Operator(ms, arena=g["H"])
    solver = ig.IMSRGSolver(H, precision="fp64")
    solver.SetHunterGatherer(hunter_gatherer)
    solver.SetOmegaNormMax(0.3)
    solver.SetSmax(2.0)
    solver.Solve()
    assert solver.GetOmegaSize() > 1
    Hs = solver.GetH_s()
    T = solver.Transform(H)
    assert max(rel_errors(r, T.arena, Hs.arena)) < 1e-12
    B = solver.InverseTransform(T)
    assert max(rel_errors(r, B.arena, H.arena)) < 1e-8


def test_solver_settings_and_errors():
    ms = ig.ModelSpace(2, "O16", "O16")
    H = ig.Operator(ms, arena=load_flow_golden(2)["H"])
    solver = ig.IMSRGSolver(H)
    solver.SetEtaCriterion(1e-20)
    # stored as float, as IMSRGSolver::SetEtaCriterion(float) does
    assert solver._get("eta_criterion") == float(np.float32(1e-20))
    with pytest.raises(ig.IMSRGError):
        solver.SetGenerator("shell-model")
    with pytest.raises(ig.IMSRGError):
        solver._set("no_such_setting", 1.0)
    with pytest.raises(ig.IMSRGError):
        solver.SetDenominatorPartitioning("MP_isospin")
    assert solver.GetS() == 0.0 and solver.GetOmegaSize() == 1


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("method,key", [("magnus_modified_euler", "flow_me"), ("magnus_backoff", "flow_bo"),
                                        ("flow_RK4", "flow_rk4")])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_other_solver_methods_vs_reference(emax, method, key, prec):
    # IMSRGSolver::Solve_magnus_modified_euler, Solve_magnus_backoff (with
    # Omega splits) and Solve_flow_RK4 (src/IMSRGSolver.cc:324-636) to s = 2,
    # against the reference's own runs
    g = load_flow_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    s_ref, n_omega_ref, e0_ref = g[key]
    solver = ig.IMSRGSolver(ig.Operator(ms, arena=g["H"]), precision=prec)
    solver.SetGenerator("white")
    solver.SetMethod(method)
    solver.SetOmegaNormMax(0.3)
    solver.SetEtaCriterion(1e-20)
    solver.SetSmax(2.0)
    solver.Solve()
    assert abs(solver.GetS() - s_ref) <= 1e-12
    assert solver.GetOmegaSize() == int(n_omega_ref)
    Hs = solver.GetH_s()
    assert abs(Hs.ZeroBody - e0_ref) <= TOL_E0[prec] * abs(e0_ref)
    assert max(rel_errors(r, Hs.arena, g[key + "_Hs"])) < TOL_OPS[prec]


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_rk4_flows_added_operator_vs_reference(emax, prec):
    # IMSRGSolver::AddOperator + Solve_flow_RK4 (src/IMSRGSolver.hh:94,
    # src/IMSRGSolver.cc:505-636): the observable [A, H] flows with H(s)'s
    # stage generators; GetOperator(0) is H(s)
    g = load_flow_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    solver = ig.IMSRGSolver(ig.Operator(ms, arena=g["H"]), precision=prec)
    solver.SetGenerator("white")
    solver.SetMethod("flow_RK4")
    solver.SetSmax(2.0)
    solver.SetEtaCriterion(1e-20)
    assert solver.AddOperator(ig.Operator(ms, arena=g["flow_rk4_obs_in"])) == 1
    solver.Solve()
    O = solver.GetOperator(1)
    assert O.hermitian
    assert max(rel_errors(r, O.arena, g["flow_rk4_obs"])) < TOL_OPS[prec]
    np.testing.assert_array_equal(solver.GetOperator(0).arena, solver.GetH_s().arena)
    assert max(rel_errors(r, solver.GetH_s().arena, g["flow_rk4_Hs"])) < TOL_OPS[prec]
    with pytest.raises(ig.IMSRGError):
        solver.GetOperator(2)


def test_rk4_flows_added_tensor():
    # a reduced tensor added to the RK4 flow goes through the scalar-tensor
    # commutator at every stage; one step, against the stage sums formed here
    # from the same public calls
    emax = 2
    g = load_flow_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    rank = (2, 0, 0)
    T = ig.Operator(ms, *rank)
    rng = np.random.default_rng(11)
    T.arena[:] = rng.standard_normal(T.arena.size) * 1e-2
    T.hermitian = True
    H = ig.Operator(ms, arena=g["H"])
    solver = ig.IMSRGSolver(H, precision="fp64")
    solver.SetGenerator("white")
    solver.SetMethod("flow_RK4")
    solver.SetDsmax(0.1)
    solver.SetSmax(0.1)
    solver.SetEtaCriterion(1e-20)
    assert solver.AddOperator(T) == 1
    solver.Solve()
    out = solver.GetOperator(1)
    assert out.rank == rank and out.arena.shape == T.arena.shape and np.isfinite(out.arena).all()
    # the same RK4 step by hand: eta from each stage's H, K_i = [eta, O_i]
    gen = ig.Generator()
    gen.SetType("white")
    ds = 0.1
    Hk, Tk = H, T
    Ksum_H = Ksum_T = None
    for k, (wk, sk) in enumerate(zip((1.0, 2.0, 2.0, 1.0), (0.5, 0.5, 1.0, None))):
        eta = ig.Operator(ms, hermitian=False)
        gen.Update(Hk, eta)
        KH = ig.Commutator.Commutator(eta, Hk, precision="fp64")
        KT = ig.Commutator.CommutatorScalarTensor(eta, Tk, precision="fp64")
        Ksum_H = KH.arena * wk if Ksum_H is None else Ksum_H + wk * KH.arena
        Ksum_T = KT.arena * wk if Ksum_T is None else Ksum_T + wk * KT.arena
        if sk is not None:
            Hk = ig.Operator(ms, arena=H.arena + sk * ds * KH.arena)
            Tk = ig.Operator(ms, *rank, arena=T.arena + sk * ds * KT.arena, hermitian=True)
    want = T.arena + ds / 6.0 * Ksum_T
    assert np.max(np.abs(out.arena - want)) <= 1e-12 * np.max(np.abs(want))


def test_unknown_method_refused():
    ms = ig.ModelSpace(2, "O16", "O16")
    solver = ig.IMSRGSolver(ig.Operator(ms, arena=load_flow_golden(2)["H"]))
    for m in ("flow_adaptive", "flow_euler", "magnus_adaptive", "restore_4th_order"):
        with pytest.raises(ig.IMSRGError):
            solver.SetMethod(m)
    with pytest.raises(ig.IMSRGError):
        solver._set("method", 4.0)
