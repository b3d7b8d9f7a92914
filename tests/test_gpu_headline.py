"""Parity at the benchmark's own sizes, through the C ABI.

- emax=10 (the headline commutator): both GPU forms against the C oracle (the
  reference's FP64 path restated, pinned to the reference's outputs) on the
  same seeded X and Y, per body rank: plain FP64 <= 1e-12, split <= 1e-10.
- emax=6, channel by channel: comm222_pp_hh_221ss, comm222_phss and comm221ss
  against the oracle, every two-body block and the one-body matrix.
- A 50-step Magnus-Euler flow (White generator, ds = 0.5): the zero-body value
  after the last step against the oracle's flow, <= 1e-8 relative, both forms.
- The double-float kernels of the split form against their FP64 twins on the
  same input: the inverse Pandya transform (same Z bar; every kernel variant)
  and comm122ss (same X, Y), relative Frobenius <= 1e-13 at emax=8.
- The full commutator under every tuning choice against the oracle."""
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


def symmetric_zbar(ms, hz, seed):
    """A random Z bar with the symmetry of comm222_phss's (which the inverse
    transforms rely on): per cross-coupled channel, head H = R + hZ R^T and
    tail T = S + Phi S^T Phi, Phi = diag((-1)^((j_p + j_q) / 2)) of its kets."""
    import torch
    L = ig.lib()
    total = ctypes.c_longlong()
    assert L.imsrg_space_zbar_layout(ms._h, -1, None, None, None, ctypes.byref(total)) == 0
    z = np.zeros(total.value)
    rng = np.random.default_rng(seed)
    for ch in range(ms.nch):
        rows, cols, off = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        assert L.imsrg_space_zbar_layout(ms._h, ch, ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(off),
                                         None) == 0
        n = rows.value
        if n == 0:
            continue
        kets = ms.cc_channel(ch)["kets"]
        phi = np.array([(-1) ** ((ms.orbits[p][2] + ms.orbits[q][2]) // 2) for (p, q) in kets], dtype=float)
        R = rng.uniform(-1, 1, (n, n))
        S = rng.uniform(-1, 1, (n, n))
        H = R + hz * R.T
        T = S + phi[:, None] * S.T * phi[None, :]
        z[off.value:off.value + 2 * n * n] = np.concatenate([H.ravel(order="F"), T.ravel(order="F")])
    return torch.from_numpy(z).cuda()


def set_tuning(ms, name, value):
    L = ig.lib()
    assert L.imsrg_space_set_tuning(ms._h, name.encode(), value) == 0, L.imsrg_last_error()


@pytest.mark.parametrize("emax", [4, 8])
def test_inverse_pandya_kernels_vs_fp64(emax):
    """Every inverse Pandya kernel against the FP64 channel-tiled one on the
    same Z bar: the FP64 descriptor kernel to rounding (1e-15), the
    double-float ones to 1e-13."""
    ms = ig.ModelSpace(emax, "O16", "O16")
    L = ig.lib()
    r = ref_space(emax)
    # (form, tuning parameter, value, tolerance)
    variants = [("split", "inverse.split", 0, TOL_DF), ("split", "inverse.split", 1, TOL_DF),
                ("split", "inverse.split", 2, 1e-15), ("fp64", "inverse.fp64", 1, 1e-15),
                ("split", "inverse.desc_weights", 1, 1e-15), ("split", "inverse.split", 1, TOL_DF),
                ("split", "inverse.desc_ilp", 4, TOL_DF), ("split", "inverse.split", 2, 1e-15)]
    for hz in (1, -1):
        zbar = symmetric_zbar(ms, hz, 88 + emax)
        with ig.DeviceOperator(ms, hz) as dZ:
            set_tuning(ms, "inverse.fp64", 0)
            assert L.imsrg_add_inverse_pandya(ctypes.c_void_p(zbar.data_ptr()), dZ._h, 0, None) == 0
            ref = dZ.download()
            assert np.linalg.norm(ref) > 0
            for form, name, value, tol in variants:
                set_tuning(ms, name, value)
                dZ.zero()
                code = 1 if form == "split" else 0
                rc = L.imsrg_add_inverse_pandya(ctypes.c_void_p(zbar.data_ptr()), dZ._h, code, None)
                assert rc == 0, L.imsrg_last_error()
                errs = rel_errors(r, dZ.download(), ref)
                assert max(errs[1:]) < tol, (hz, name, value, errs)
        set_tuning(ms, "inverse.split", 0)
        set_tuning(ms, "inverse.fp64", 0)
        set_tuning(ms, "inverse.desc_weights", 0)
        set_tuning(ms, "inverse.desc_ilp", 1)


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_commutator_with_every_tuning(prec):
    """The full commutator with each tile shape, stage count, schedule and
    inverse Pandya kernel against the oracle."""
    emax = 5
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    X = o.ms.random_operator(505, True)
    Y = o.ms.random_operator(606, False)
    R = o.commutator(X, Y, 1, -1)
    settings = [{}, {"ladder.tile": 32, "zbar.tile": 64}, {"ladder.stages": 2, "zbar.stages": 2},
                {"ladder.schedule": 1, "zbar.schedule": 1}, {"inverse.split": 1, "inverse.fp64": 1},
                {"inverse.split": 2, "inverse.desc_stage": 256, "inverse.desc_results": 128},
                {"inverse.split": 1, "inverse.desc_weights": 1}, {"inverse.split": 2, "inverse.desc_weights": 1},
                {"inverse.split": 1, "inverse.desc_ilp": 4}, {"inverse.split": 2, "inverse.desc_ilp": 2},
                {"inverse.quad_budget": 16384}, {"comm122.fused": 1}, {"zbar.digits": 5},
                {"ladder.digits": 5}]
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.upload(X)
        dY.upload(Y)
        for st in settings:
            for k, v in st.items():
                set_tuning(ms, k, v)
            ig.Commutator.device_commutator(dX, dY, dZ, prec)
            errs = rel_errors(o.ms, dZ.download(), R)
            assert max(errs) < TOL[prec], (st, errs)
            for k in st:
                set_tuning(ms, k, 0 if k not in ("inverse.quad_budget", "inverse.desc_stage",
                                                 "inverse.desc_results", "inverse.desc_ilp") else
                           {"inverse.quad_budget": 36864, "inverse.desc_stage": 2048,
                            "inverse.desc_results": 2048, "inverse.desc_ilp": 1}[k])


def test_seven_digit_ladder_product_vs_fp64():
    """The split commutator with 7-digit ladder operands (42 bits: the ladder's
    digit width is 6 bits at emax 8) against the FP64 form on the same
    operators; exercises the 7-digit product kernel."""
    emax = 8
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.fill_random(871)
        dY.fill_random(872)
        ig.Commutator.device_commutator(dX, dY, dZ, "fp64")
        ref = dZ.download()
        try:
            ms.set_tuning("ladder.digits", 7)
            ig.Commutator.device_commutator(dX, dY, dZ, "split")
            out = dZ.download()
        finally:
            ms.set_tuning("ladder.digits", 0)
    errs = rel_errors(r, out, ref)
    assert max(errs) < TOL["split"], errs


@pytest.mark.parametrize("fused", [0, 1])
def test_comm122_double_float_vs_fp64(fused):
    emax = 8
    ms = ig.ModelSpace(emax, "O16", "O16")
    ms.set_tuning("comm122.fused", fused)
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


def test_tuning_file_applied():
    """A space whose size has a line in imsrg_gb300/tuning/gb300.txt gets that
    line's parameters when it builds its device tables; IMSRG_GB300_TUNING=off
    leaves the built-in defaults."""
    import os
    path = os.path.join(os.path.dirname(ig.__file__), "tuning", "gb300.txt")
    lines = {}
    for ln in open(path):
        if ln.startswith("#") or not ln.strip():
            continue
        kv = dict(tok.split("=") for tok in ln.split())
        lines[int(kv["emax"])] = {k: int(v) for k, v in kv.items() if k not in ("arena", "norb", "emax")}
    emax = 6
    ms = ig.ModelSpace(emax, "O16", "O16")
    with ig.DeviceOperator(ms, 1):
        t = ms.tuning()
    assert t["source"].endswith(".txt:%d" % ([i + 1 for i, ln in enumerate(open(path))
                                             if ln.startswith("arena=%d " % ms.arena_size)][0])), t
    for k, v in lines[emax].items():
        assert t[k] == v, (k, t[k], v)
    old = os.environ.get("IMSRG_GB300_TUNING")
    os.environ["IMSRG_GB300_TUNING"] = "off"
    try:
        ms2 = ig.ModelSpace(emax, "O16", "O16")
        with ig.DeviceOperator(ms2, 1):
            t2 = ms2.tuning()
        assert t2["source"] == "default" and t2["inverse.split"] == 0, t2
    finally:
        if old is None:
            del os.environ["IMSRG_GB300_TUNING"]
        else:
            os.environ["IMSRG_GB300_TUNING"] = old
