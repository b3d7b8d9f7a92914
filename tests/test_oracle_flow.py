"""The C oracle's BCH product, generators and Magnus-Euler solver against the
reference's own outputs (golden_flow_emax*.npz, made by
tests/golden/make_golden.py from the reference compiled from its sources)."""
import numpy as np
import pytest

from helpers import load_flow_golden, rel_errors
from oracle import FlowParams, Oracle

TOL = 1e-13


@pytest.mark.parametrize("emax", [2, 3])
def test_oracle_bch_product_matches_reference(emax):
    g = load_flow_golden(emax)
    o = Oracle(emax)
    Z, n = o.bch_product(g["A"], -1, g["B"], -1)
    assert n >= 2
    assert max(rel_errors(o.ms, Z, g["bchp"])) < TOL
    # larger operators: the 1/12 [X,[X,Y]] term and more of the series
    Z, n = o.bch_product(6.0 * g["A"], -1, 2.0 * g["B"], -1)
    assert n >= 3
    assert max(rel_errors(o.ms, Z, g["bchp_big"])) < TOL


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("case", [("eta_white", "white", "Epstein_Nesbet"), ("eta_atan", "atan", "Epstein_Nesbet"),
                                  ("eta_white_mp", "white", "Moller_Plesset")])
def test_oracle_generator_matches_reference(emax, case):
    key, kind, part = case
    g = load_flow_golden(emax)
    o = Oracle(emax)
    Eta = o.generator(g["H"], kind, part)
    assert np.abs(Eta - g[key]).max() <= TOL * np.abs(g[key]).max()


@pytest.mark.parametrize("emax", [2, 3])
def test_oracle_fixed_step_flow_matches_reference(emax):
    g = load_flow_golden(emax)
    o = Oracle(emax)
    steps = g["flow_steps"]
    p = FlowParams(ds=0.5, ds_max=0.5, smax=0.5 * len(steps), magnus_adaptive=0, omega_norm_max=1e9,
                   eta_criterion=1e-20)
    st = o.magnus_euler(g["H"], p)
    assert st["steps"] == len(steps)
    np.testing.assert_allclose(st["s_hist"], steps[:, 0], rtol=0, atol=0)
    np.testing.assert_allclose(st["e0_hist"], steps[:, 1], rtol=1e-12)
    assert max(rel_errors(o.ms, st["Hs"], g["flow_Hs"])) < 1e-12
    assert max(rel_errors(o.ms, st["Omega"], g["flow_Omega"])) < 1e-12


@pytest.mark.parametrize("emax", [2, 3])
def test_oracle_adaptive_split_flow_matches_reference(emax):
    g = load_flow_golden(emax)
    o = Oracle(emax)
    s_ref, n_omega_ref, e0_ref = g["flow2"]
    st = o.magnus_euler(g["H"], FlowParams(smax=2.0, omega_norm_max=0.3, eta_criterion=1e-20))
    assert st["s"] == s_ref
    assert st["n_omega"] == int(n_omega_ref) and st["n_omega"] > 1
    assert abs(st["Hs"][0] - e0_ref) <= 1e-12 * abs(e0_ref)
    assert max(rel_errors(o.ms, st["Hs"], g["flow2_Hs"])) < 1e-12
    assert max(rel_errors(o.ms, st["Omega"], g["flow2_Omega"])) < 1e-12


def test_oracle_flow_resumes():
    # two Solve() calls to s = 1 then s = 2.5 give the single call's flow
    g = load_flow_golden(2)
    o = Oracle(2)
    p = FlowParams(ds=0.5, ds_max=0.5, smax=2.5, magnus_adaptive=0, omega_norm_max=1e9, eta_criterion=1e-20)
    one = o.magnus_euler(g["H"], p)
    p.smax = 1.0
    a = o.magnus_euler(g["H"], p)
    p.smax = 2.5
    b = o.magnus_euler(g["H"], p, state=a)
    assert a["steps"] + b["steps"] == one["steps"] == 5
    assert np.array_equal(b["Hs"], one["Hs"])


@pytest.mark.parametrize("emax", [2, 3])
def test_oracle_rk4_flow_matches_reference(emax):
    # IMSRGSolver::Solve_flow_RK4 (src/IMSRGSolver.cc:505-636) restated over
    # the oracle's commutator and White generator: four RK4 steps of ds_max
    # = 0.5 to s = 2, flowing H and the added observable [A, H] with the
    # stage generators of H
    g = load_flow_golden(emax)
    o = Oracle(emax)
    s_ref, n_omega_ref, e0_ref = g["flow_rk4"]
    H, O = g["H"].copy(), g["flow_rk4_obs_in"].copy()
    s, ds = 0.0, 0.5
    eta = o.generator(H)
    while s < 2.0:
        assert o.norm(eta) >= 1e-20
        ds = min(0.5, 2.0 - s)
        s += ds
        sums = [np.zeros_like(H), np.zeros_like(O)]
        stage = [H, O]
        for wk, sk in zip((1.0, 2.0, 2.0, 1.0), (0.5, 0.5, 1.0, None)):
            K = [o.commutator(eta, X, -1, 1) for X in stage]
            sums = [acc + wk * k for acc, k in zip(sums, K)]
            if sk is not None:
                stage = [X0 + sk * ds * k for X0, k in zip((H, O), K)]
                eta = o.generator(stage[0])
        H = H + ds / 6.0 * sums[0]
        O = O + ds / 6.0 * sums[1]
        eta = o.generator(H)
    assert s == s_ref and int(n_omega_ref) == 1
    assert abs(H[0] - e0_ref) <= 1e-12 * abs(e0_ref)
    assert max(rel_errors(o.ms, H, g["flow_rk4_Hs"])) < 1e-12
    assert max(rel_errors(o.ms, O, g["flow_rk4_obs"])) < 1e-12
