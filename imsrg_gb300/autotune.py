"""Autotuner of the GB300 commutator's kernels, per model space.

    python -m imsrg_gb300.autotune [--emax 6 8 10 12] [--reps 5]
        [--out imsrg_gb300/tuning/gb300.txt] [--log imsrg_gb300/tuning/gb300_search.json]

For each model space (O16 reference, the given emax) it measures, on the GPU,
the choices that imsrg_space_set_tuning exposes and keeps the fastest:

- the split products' tile shape (64 x 1 or 32 x 2 accumulator sets),
  pipeline depth and tile-to-CTA schedule (round-robin in size order, or
  longest-first greedy lists), ladder and Z bar product each, timed as whole
  split-form commutators (the products share the GPU with the second stream);
- the split form's comm122ss with W2 through memory or fused tile pairs,
  timed as whole split-form commutators;
- the digits per operand of each product family (the precision), kept only
  when the split commutator stays within a third of the 1e-10 error bound
  against the FP64 one on the same operators, in every two-body channel block;
- the inverse Pandya kernel of each form and its block sizes, timed alone
  (imsrg_add_inverse_pandya on a Z bar of the space's layout).  Among the
  split form's kernels, the FP64 descriptor kernel (the reference's FP64
  recoupling sums) is kept unless a double-float kernel is faster by more than
  --fp64-margin (default 10%).

The result is one line per space in the tuning file, which the library applies
when a space of that size builds its device tables, and the whole search in a
JSON log.  The reference's counterpart is OpenMP's dynamic schedule over
size-sorted channels (src/ModelSpace.cc:1183-1198, src/Commutator.cc:1113-1115).
"""
import argparse
import ctypes
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))

DEFAULTS = {"ladder.tile": 64, "ladder.stages": 0, "ladder.schedule": 0, "zbar.tile": 32, "zbar.stages": 0,
            "zbar.schedule": 0, "inverse.split": 0, "inverse.fp64": 0, "inverse.quad_budget": 36864,
            "inverse.desc_stage": 2048, "inverse.desc_results": 2048, "inverse.desc_weights": 0,
            "inverse.desc_ilp": 1, "comm122.fused": 0, "ladder.digits": 0, "zbar.digits": 0}


ERR_GATE = 1e-10 / 3


def _rank_error(a, b, ms):
    """Largest relative Frobenius difference of arena a against b over the
    zero- and one-body parts and every two-body channel block (blocks whose
    reference norm is below 1e-12 of the whole are compared against the
    whole)."""
    import numpy as np
    N = ms.norb
    tot = max(float(np.linalg.norm(b)), 1e-300)
    parts = [(a[:1], b[:1]), (a[32:32 + N * N], b[32:32 + N * N])]
    for c in ms.channels:
        n, o = c["nkets"], c["offset"]
        if n:
            parts.append((a[o:o + n * n], b[o:o + n * n]))
    worst = 0.0
    for x, y in parts:
        ny = float(np.linalg.norm(y))
        d = float(np.linalg.norm(x - y))
        worst = max(worst, d / ny if ny > 1e-12 * tot else d / tot)
    return worst


def _set(L, ms, name, value):
    rc = L.imsrg_space_set_tuning(ms._h, name.encode(), int(value))
    if rc != 0:
        raise RuntimeError("%s=%s: %s" % (name, value, L.imsrg_last_error().decode()))


def _timed(fn, reps, rounds=3):
    """Best over `rounds` of the mean CUDA-event time (ms) of `reps` calls."""
    import torch
    fn()
    torch.cuda.synchronize()
    best = None
    for _ in range(rounds):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / reps
        best = t if best is None else min(best, t)
    return best


def tune_space(ig, emax, reps, fp64_margin, log):
    import torch
    L = ig.lib()
    ms = ig.ModelSpace(emax, "O16", "O16")
    dX, dY, dZ = ig.DeviceOperator(ms, 1), ig.DeviceOperator(ms, -1), ig.DeviceOperator(ms, 1)
    dX.fill_random(11)
    dY.fill_random(12)
    ms.defer_status(True)
    for k, v in DEFAULTS.items():
        _set(L, ms, k, v)
    chosen = dict(DEFAULTS)
    rec = {"emax": emax, "arena": ms.arena_size, "norb": ms.norb, "trials": []}

    def commutator_ms():
        t = _timed(lambda: ig.Commutator.device_commutator(dX, dY, dZ, "split"), reps)
        ms.check_status()
        return t

    # 1. the inverse Pandya kernels, alone, on a Z bar of this space
    total = ctypes.c_longlong()
    L.imsrg_space_zbar_layout(ms._h, -1, None, None, None, ctypes.byref(total))
    zbar = (torch.rand(total.value, dtype=torch.float64, device="cuda") * 2 - 1)
    zp = ctypes.c_void_p(zbar.data_ptr())

    def inverse_ms(precision):
        def f():
            rc = L.imsrg_add_inverse_pandya(zp, dZ._h, precision, None)
            if rc != 0:
                raise RuntimeError(L.imsrg_last_error().decode())
        return _timed(f, reps)

    cands = {}
    for budget in (24576, 28672, 32768, 36864, 40960, 49152):
        _set(L, ms, "inverse.split", 0)
        _set(L, ms, "inverse.quad_budget", budget)
        t = inverse_ms(1)
        rec["trials"].append({"what": "inverse split", "inverse.split": 0, "inverse.quad_budget": budget, "ms": t})
        if 0 not in cands or t < cands[0][0]:
            cands[0] = (t, {"inverse.split": 0, "inverse.quad_budget": budget})
    _set(L, ms, "inverse.quad_budget", cands[0][1]["inverse.quad_budget"])
    # descriptor blocks of up to `stage` staged values and as many results,
    # 6j weights read from the table or staged per block (one descriptor build
    # per choice, both arithmetic variants timed on it)
    for weights in (0, 1):
        for stage in (512, 1024, 2048, 4096):
            _set(L, ms, "inverse.desc_weights", weights)
            _set(L, ms, "inverse.desc_stage", stage)
            _set(L, ms, "inverse.desc_results", stage)
            for variant in (1, 2):
                for ilp in (1, 2):
                    _set(L, ms, "inverse.split", variant)
                    _set(L, ms, "inverse.desc_ilp", ilp)
                    t = inverse_ms(1)
                    cfg = {"inverse.split": variant, "inverse.desc_stage": stage, "inverse.desc_results": stage,
                           "inverse.desc_weights": weights, "inverse.desc_ilp": ilp}
                    rec["trials"].append({"what": "inverse split", **cfg, "ms": t})
                    if variant not in cands or t < cands[variant][0]:
                        cands[variant] = (t, cfg)
    # FP64 sums unless a double-float kernel wins by more than the margin
    fastest = min(cands.values(), key=lambda c: c[0])
    pick = cands[2] if cands[2][0] <= fastest[0] * (1.0 + fp64_margin) else fastest
    for k, v in pick[1].items():
        chosen[k] = v
    for k in ("inverse.split", "inverse.desc_stage", "inverse.desc_results", "inverse.desc_weights",
              "inverse.desc_ilp", "inverse.quad_budget"):
        _set(L, ms, k, chosen[k])
    # the FP64 form's kernel: channel tiles or descriptors (same block sizes)
    f64 = {}
    for variant in (0, 1):
        _set(L, ms, "inverse.fp64", variant)
        f64[variant] = inverse_ms(0)
        rec["trials"].append({"what": "inverse fp64", "inverse.fp64": variant, "ms": f64[variant]})
    chosen["inverse.fp64"] = min(f64, key=f64.get)
    _set(L, ms, "inverse.fp64", chosen["inverse.fp64"])
    # 2. the split form's comm122ss: W2 through memory, or fused tile pairs
    best = None
    for fused in (0, 1):
        _set(L, ms, "comm122.fused", fused)
        t = commutator_ms()
        rec["trials"].append({"what": "split commutator", "comm122.fused": fused, "ms": t})
        if best is None or t < best[0]:
            best = (t, fused)
    chosen["comm122.fused"] = best[1]
    _set(L, ms, "comm122.fused", best[1])
    # 3. the split products: each family's (tile, stages, schedule), with the
    # inverse kernel chosen above (the descriptor kernels let the Z bar
    # product skip its mirror stores)
    for fam, tiles in (("ladder", (64, 32)), ("zbar", (32, 64))):
        best = None
        for tile in tiles:
            for stages in (0, 2):
                for sched in (0, 1):
                    cfg = {fam + ".tile": tile, fam + ".stages": stages, fam + ".schedule": sched}
                    for k, v in cfg.items():
                        _set(L, ms, k, v)
                    t = commutator_ms()
                    rec["trials"].append({"what": "split commutator", **cfg, "ms": t})
                    if best is None or t < best[0]:
                        best = (t, cfg)
        for k, v in best[1].items():
            _set(L, ms, k, v)
            chosen[k] = v
    # 4. digits per operand of each product family, under the accuracy gate:
    # the split commutator's error against the FP64 one on the same X, Y
    # (zero- and one-body parts and every two-body channel block, for a
    # hermitian and an anti-hermitian Z) stays within a third of the 1e-10 bound
    # both symmetry cases of Z: [X, Y] (X hermitian, Y anti-hermitian) and
    # [X, W] (both hermitian)
    dW = ig.DeviceOperator(ms, 1)
    dW.fill_random(13)
    refs = []
    for dB in (dY, dW):
        ig.Commutator.device_commutator(dX, dB, dZ, "fp64")
        refs.append((dB, dZ.download()))

    def split_error():
        worst = 0.0
        for dB, zf in refs:
            ig.Commutator.device_commutator(dX, dB, dZ, "split")
            ms.check_status()
            worst = max(worst, _rank_error(dZ.download(), zf, ms))
        return worst

    for fam in ("zbar", "ladder"):
        best = None
        for digits in (0, 5):
            _set(L, ms, fam + ".digits", digits)
            err = split_error()
            t = commutator_ms()
            rec["trials"].append({"what": "split commutator", fam + ".digits": digits, "ms": t, "max_rel_err": err})
            if err <= ERR_GATE and (best is None or t < best[0]):
                best = (t, digits)
        chosen[fam + ".digits"] = best[1] if best else 0
        _set(L, ms, fam + ".digits", chosen[fam + ".digits"])
    rec["split_max_rel_err_tuned"] = split_error()
    rec["inverse_split_candidates_ms"] = {str(k): v[0] for k, v in cands.items()}
    rec["commutator_ms_tuned"] = commutator_ms()
    for k, v in DEFAULTS.items():
        _set(L, ms, k, v)
    rec["commutator_ms_default"] = commutator_ms()
    rec["chosen"] = chosen
    log.append(rec)
    del zbar
    for d in (dX, dY, dZ, dW):
        d.close()
    return ms.arena_size, ms.norb, chosen


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--emax", type=int, nargs="+", default=[2, 3, 4, 5, 6, 8, 10, 12])
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--fp64-margin", type=float, default=0.10)
    ap.add_argument("--out", default=os.path.join(HERE, "tuning", "gb300.txt"))
    ap.add_argument("--log", default=os.path.join(HERE, "tuning", "gb300_search.json"))
    a = ap.parse_args()
    os.environ["IMSRG_GB300_TUNING"] = "off"  # search from the built-in defaults
    sys.path.insert(0, os.path.dirname(HERE))
    import torch
    import imsrg_gb300 as ig
    log, lines = [], []
    gpu = torch.cuda.get_device_name(0)
    for emax in a.emax:
        t0 = time.time()
        arena, norb, chosen = tune_space(ig, emax, a.reps, a.fp64_margin, log)
        log[-1]["search_s"] = time.time() - t0
        lines.append("arena=%d norb=%d emax=%d " % (arena, norb, emax) +
                     " ".join("%s=%d" % (k, v) for k, v in chosen.items()))
        print(json.dumps({k: log[-1][k] for k in ("emax", "chosen", "commutator_ms_default", "commutator_ms_tuned",
                                                   "inverse_split_candidates_ms", "search_s")}), flush=True)
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    with open(a.out, "w") as f:
        f.write("# imsrg_gb300 kernel tuning, written by python -m imsrg_gb300.autotune on %s (%s)\n"
                % (gpu, time.strftime("%Y-%m-%d")))
        f.write("# one line per model space: arena length, orbits, then imsrg_space_set_tuning parameters\n")
        for ln in lines:
            f.write(ln + "\n")
    with open(a.log, "w") as f:
        json.dump({"gpu": gpu, "when": time.strftime("%Y-%m-%dT%H:%M:%S"), "reps": a.reps,
                   "fp64_margin": a.fp64_margin, "spaces": log}, f, indent=1)


if __name__ == "__main__":
    main()
