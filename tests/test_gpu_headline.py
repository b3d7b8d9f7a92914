"""Parity at the benchmark's own sizes, through the C ABI.

- emax=10 (the headline commutator): both GPU forms against the C oracle (the
  reference's FP64 path restated, pinned to the reference's outputs) on the
  same seeded X and Y, per body rank: plain FP64 <= 1e-12, split <= 1e-10.
- emax=6, channel by channel: comm222_pp_hh_221ss, comm222_phss and comm221ss
  against the oracle, every two-body block and the one-body matrix.
- A 50-step Magnus-Euler flow (White generator, ds = 0.5): the zero-body value
  after the last step against the oracle's flow, <= 1e-8 relative, both forms.
- The double-float kernels of the split form against their FP64 twins on the
  same input: the inverse Pandya transform (same Z bar) and comm122ss (same X,
  Y), relative Frobenius <= 1e-13 at emax=8."""
import ctypes

import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import rel_errors, ref_space
from oracle import FlowParams, Oracle

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "split": 1e-10}
TOL_FLOW_E0 = 1e-8
TOL_DF = 1e-13


def gpu_commutator(ms, X, Y, prec):
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.upload(X)
        dY.upload(Y)
        ig.Commutator.device_commutator(dX, dY, dZ, prec)
        return dZ.download()


def test_emax10_both_forms_vs_oracle():
    emax = 10
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    X = o.ms.random_operator(1010, True)
    Y = o.ms.random_operator(2020, False)
    R = o.commutator(X, Y, 1, -1)
    for prec in ("fp64", "split"):
        Z = gpu_commutator(ms, X, Y, prec)
        errs = rel_errors(o.ms, Z, R)
        assert max(errs) < TOL[prec], (prec, errs)


@pytest.mark.parametrize("term", ["comm222_pp_hh_221ss", "comm222_phss", "comm221ss"])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_emax6_terms_channel_by_channel(term, prec):
    emax = 6
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    X = o.ms.random_operator(606, True)
    Y = o.ms.random_operator(707, False)
    R = o.zeros()
    o.term(term, X, Y, R, 1, -1)
    if term == "comm221ss" and prec == "split":
        pytest.skip("comm221ss has no dense product: one form only")
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.upload(X)
        dY.upload(Y)
        ig.Commutator.device_term(term, dX, dY, dZ, prec)
        Z = dZ.download()
    scale = np.linalg.norm(R)
    worst = 0.0
    for c in range(o.ms.nch):
        b, r = o.ms.block(Z, c), o.ms.block(R, c)
        nr = np.linalg.norm(r)
        if nr == 0:
            assert np.linalg.norm(b) < TOL[prec] * scale, c
            continue
        worst = max(worst, np.linalg.norm(b - r) / nr)
    z1, r1 = o.ms.onebody(Z), o.ms.onebody(R)
    if np.linalg.norm(r1) > 0:
        worst = max(worst, np.linalg.norm(z1 - r1) / np.linalg.norm(r1))
    assert worst < TOL[prec], (term, prec, worst)


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_flow_50_steps_final_e0_vs_oracle(prec):
    emax, steps = 5, 50
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    H = o.ms.flow_hamiltonian(5000 + emax, 0.5)
    p = FlowParams(ds=0.5, ds_max=0.5, smax=0.5 * steps, magnus_adaptive=0, omega_norm_max=1e9,
                   eta_criterion=1e-20)
    R = o.magnus_euler(H, p)
    assert R["steps"] == steps
    solver = ig.IMSRGSolver(ig.Operator(ms, arena=H), precision=prec)
    for name, v in (("SetDs", 0.5), ("SetDsmax", 0.5), ("SetSmax", 0.5 * steps), ("SetOmegaNormMax", 1e9),
                    ("SetEtaCriterion", 1e-20)):
        getattr(solver, name)(v)
    solver.SetMagnusAdaptive(False)
    solver.Solve()
    _, _, e0, _, _ = solver.history()
    assert len(e0) == steps
    e_final = solver.GetH_s().ZeroBody
    assert e_final == e0[-1]
    ref = R["Hs"][0]
    assert abs(e_final - ref) <= TOL_FLOW_E0 * abs(ref), (prec, e_final, ref)


def test_inverse_pandya_double_float_vs_fp64():
    emax = 8
    ms = ig.ModelSpace(emax, "O16", "O16")
    L = ig.lib()
    total = ctypes.c_longlong()
    assert L.imsrg_space_zbar_layout(ms._h, -1, None, None, None, ctypes.byref(total)) == 0
    import torch
    g = torch.Generator().manual_seed(88)
    zbar = (torch.rand(total.value, generator=g, dtype=torch.float64) * 2 - 1).cuda()
    out = {}
    for hz in (1, -1):
        for prec, code in (("fp64", 0), ("split", 1)):
            with ig.DeviceOperator(ms, hz) as dZ:
                rc = L.imsrg_add_inverse_pandya(ctypes.c_void_p(zbar.data_ptr()), dZ._h, code, None)
                assert rc == 0, L.imsrg_last_error()
                out[(hz, prec)] = dZ.download()
        r = ref_space(emax)
        errs = rel_errors(r, out[(hz, "split")], out[(hz, "fp64")])
        assert max(errs[1:]) < TOL_DF, (hz, errs)
        assert np.linalg.norm(out[(hz, "fp64")]) > 0


def test_comm122_double_float_vs_fp64():
    emax = 8
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    names = ["comm110ss", "comm220ss", "comm111ss", "comm121ss", "comm122ss", "comm221ss", "comm222_pp_hhss",
             "comm222_phss"]
    saved = {n: ig.Commutator.IsTermOn(n) for n in names}
    try:
        for n in names:
            if n != "comm122ss":
                ig.Commutator.TurnOffTerm(n)
        with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
            dX.fill_random(812)
            dY.fill_random(813)
            out = {}
            for prec in ("fp64", "split"):
                ig.Commutator.device_commutator(dX, dY, dZ, prec)
                out[prec] = dZ.download()
        errs = rel_errors(r, out["split"], out["fp64"])
        assert max(errs[1:]) < TOL_DF, errs
        assert np.linalg.norm(out["fp64"]) > 0
    finally:
        for n, on in saved.items():
            (ig.Commutator.TurnOnTerm if on else ig.Commutator.TurnOffTerm)(n)
