#!/usr/bin/env python3
"""Benchmark: [X,Y] commutators/sec of the IMSRG(2) scalar commutator at emax=10.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step is one full CommutatorScalarScalar [X,Y] (all IMSRG(2) terms) on the
emax=10 O16 model space (132 orbits, largest two-body channel 1341 kets):
X hermitian and Y anti-hermitian, seeded uniform[-1,1] entries on
symmetry-allowed elements, each two-body channel block and the one-body matrix
scaled to unit Frobenius norm (synthetic; the reference publishes no dataset).

gb300 arm (default): value = whole-job commutators/s of the split-precision form
with operands resident in HBM, timed with CUDA events over K steps between
barriers + synchronisations (max over ranks), the library's phase timers off and
the kernels' status word read once after the K steps.  Every step reads X2, Y2
(280 MiB each) and writes Zbar (upper triangle, 380 MiB), so the working set
exceeds the 129 MB L2 between steps.  Also reported: per-step event times; the
plain FP64 form ("plain_fp64"); the per-body-rank error of both forms against
the C oracle on the same X, Y ("rel_err_vs_oracle"); ms per BCH step
(BCH_Transform(X, Omega) with |Omega| set so that 10-20 nested commutators run;
split, FP64 and CPU); e2e (host buffers in pinned memory, H2D of X and Y +
commutator + D2H of Z per step, through the C ABI; independent steps streamed
over two operator sets, with the serial figure beside it); the 64-pair batch
(emax 2..6, one CUDA graph, both forms); the roofline of the dominant kernel
(from the library's CUDA-event phase timers, in a separate pass over the same
steps); the applied kernel tuning; SM clocks sampled during the timed region;
the number of kernel launches; and a CPU baseline (the C oracle, a restatement
of the reference's OpenMP + BLAS path, on all host cores, on the benchmark's
own X and Y).

reference arm: the reference's CPU implementation of the path, here the C
oracle port (the reference's own build needs the reference sources, absent on
the GPU host), on all host threads; rank 0 only.
Multi-GPU: replicas only (each rank runs its own commutators; no collective
on the data path).

--workload batch: 64 independent (X, Y) pairs, emax drawn uniformly from
{2,...,6} by seed, each pair in its own model space; value = commutators/s of
the pairs replayed as one CUDA graph (imsrg_batch_*, split form), beside the
same pairs as 64 sequential single-pair calls, and both in FP64.

--workload tensor: the scalar-tensor commutator [X, T] (X hermitian scalar, T a
random hermitian reduced tensor of rank J=2, |dTz|=0, parity + (an E2-like
operator)) at emax=8 by default, FP64; value = ms per commutator.

--workload flow: the synthetic Magnus flow instead (IMSRGSolver,
magnus_euler, White generator, fixed ds = 0.5, no Omega split) at emax=12 by
default: H has one-body diagonal 2n+l+3/2, off-diagonal uniform[-0.1,0.1]
within (l, j2, tz2) blocks and a random hermitian two-body part scaled to
Frobenius norm 0.5 per channel.  value = ms per flow step of the split form
(after W warm-up steps of a separate flow), with the plain FP64 form's ms per
step and both forms' zero-body energies beside it.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "[X,Y] commutators/sec at emax={emax}: split-prec vs FP64 on 1 GB300, <=1e-10 rel err"
UNIT = "commutators/s"
WORKLOAD = ("IMSRG(2) CommutatorScalarScalar [X,Y], emax={emax} O16, X hermitian / Y anti-hermitian, "
            "uniform[-1,1], unit Frobenius per channel")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--emax", type=int, default=None, help="default 10 (commutator), 12 (flow)")
    p.add_argument("--workload", default="commutator", choices=["commutator", "flow", "batch", "tensor"])
    p.add_argument("--pairs", type=int, default=64, help="batch workload: independent (X, Y) pairs")
    p.add_argument("--batch-emax", type=int, default=None, help="batch workload: every pair at this emax")
    p.add_argument("--fp64-steps", type=int, default=None, help="flow steps timed in the FP64 form")
    p.add_argument("--cpu-flow-steps", type=int, default=1,
                   help="flow workload: steps of the C oracle's flow compared with the GPU flows' zero-body value")
    p.add_argument("--precision", default="split", choices=["split", "fp64"])
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batch", action="store_true", help="commutator workload: skip the 64-pair batch key")
    return p.parse_args()


# --------------------------------------------------------------- helpers
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# Multi-GPU is replicas only: every rank runs its own commutators on its own
# operators; the only communication is the barrier and the max of the timings.
def replica_seeds(rank):
    """Seeds of the X and Y operators of one replica."""
    return 1000 + rank, 2000 + rank


def whole_job_value(world, steps, elapsed_ms_max):
    """Whole-job commutators/s: every rank ran `steps`, the slowest took elapsed_ms_max."""
    return world * steps / (elapsed_ms_max / 1000.0)


def max_over_ranks(x, device=None):
    """Max of a float over the ranks of the default process group (identity
    without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.lines = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.idx)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def profiled_traffic(phase, emax):
    """DRAM bytes per launch of a phase's kernel from a committed ncu summary
    (lines `traffic: <phase> emax=<e> <bytes>` under profiles/), or None."""
    import glob
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 4 and parts[0] == "traffic:" and parts[1] == phase and parts[2] == "emax=%d" % emax:
                    return int(parts[3]), os.path.relpath(path, ROOT)
    return None


def algorithmic_work(ms):
    """Per-commutator algorithmic work of the dense phases and the gathers
    (FP64-equivalent flops; bytes of one read of each input and one write of
    each output)."""
    occ = [o[4] for o in ms.orbits]
    ladder = 0
    n2 = 0
    for c in ms.channels:
        n = c["nkets"]
        if n == 0:
            continue
        n2 += n * n
        K = 0
        for (p, q) in c["kets"]:
            hp, hq = occ[p] > 1e-6, occ[q] > 1e-6
            if (not hp and not hq) or (hp and hq):
                K += 1
        ladder += 2 * n * n * K
    zbar = 0
    zbar_elems = 0
    for ch in range(ms.nch):
        cc = ms.cc_channel(ch)
        ncc = cc["nkets"]
        nph = sum(1 for (p, q) in cc["kets"] if occ[p] > 1e-6 or occ[q] > 1e-6)
        zbar += 2 * ncc * (2 * nph) * (2 * ncc)
        zbar_elems += 2 * ncc * ncc
    return {"ladder_flops": ladder, "zbar_flops": zbar, "z2_elems": n2, "zbar_elems": zbar_elems}


def kernel_work(name, w):
    """(bound, algorithmic amount per launch, unit) of a profiled phase."""
    if name == "split_gemm_ladder":
        return "tensor", w["ladder_flops"], "flops"
    if name == "split_gemm_zbar":
        return "tensor", w["zbar_flops"], "flops"
    if name == "InversePandyaTransformation":
        return "hbm", 8 * (w["zbar_elems"] + 2 * w["z2_elems"]), "bytes"
    if name == "comm122ss":
        return "hbm", 8 * 4 * w["z2_elems"], "bytes"
    if name in ("split_slice_ladder",):
        return "hbm", 8 * 2 * w["z2_elems"], "bytes"
    return None


def rank_errors(a, b, norb):
    """Relative Frobenius difference per body rank (zero-, one-, two-body) of
    arena a against arena b."""
    import numpy as np
    N = norb
    o2 = (32 + N * N + 31) // 32 * 32
    out = {}
    for name, x, y in (("zero_body", a[:1], b[:1]), ("one_body", a[32:32 + N * N], b[32:32 + N * N]),
                       ("two_body", a[o2:], b[o2:])):
        ny = float(np.linalg.norm(y))
        out[name] = float(np.linalg.norm(x - y) / ny) if ny > 0 else float(np.linalg.norm(x - y))
    return out


# The CPU leg (rank 0, N=1): the C oracle, a restatement of the reference's
# OpenMP + BLAS path, run in a child process on all host cores.  It evaluates
# [X, Y] and BCH_Transform(X, c Y) on the benchmark's own operators (read from
# .npy files), which serves twice: as the reference result the GPU results are
# checked against per body rank, and as the timed CPU baseline (a bounded
# sample of commutators, one BCH step).
CPU_LEG = r"""
import sys, time, json
import numpy as np
sys.path.insert(0, %(oracle)r)
sys.path.insert(0, %(root)r)
from oracle import Oracle
from bench import rank_errors
d = %(dir)r
o = Oracle(%(emax)d)
N = o.ms.norb
X = np.load(d + "/X.npy"); Y = np.load(d + "/Y.npy")
t0 = time.perf_counter()
R = o.commutator(X, Y, 1, -1)
t_first = time.perf_counter() - t0
out = {"threads": o.num_threads(), "rel_err_vs_oracle": {}}
for form in ("split", "fp64"):
    out["rel_err_vs_oracle"][form] = rank_errors(np.load(d + "/Z_%%s.npy" %% form), R, N)
del R
n = 1; t = t_first
t0 = time.perf_counter()
while t < %(seconds)f and n < 50:
    o.commutator(X, Y, 1, -1); n += 1
    t = t_first + time.perf_counter() - t0
out["n"] = n; out["t"] = t
c = float(np.load(d + "/c.npy"))
if c > 0:
    t0 = time.perf_counter()
    B, it = o.bch_transform(X, 1, c * Y, -1)
    out["bch_ms"] = 1000.0 * (time.perf_counter() - t0)
    out["bch_nested"] = int(it)
    out["bch_rel_err_vs_oracle"] = {}
    for form in ("split", "fp64"):
        out["bch_rel_err_vs_oracle"][form] = rank_errors(np.load(d + "/B_%%s.npy" %% form), B, N)
print(json.dumps(out))
"""


def cpu_leg(emax, seconds, threads, arrays):
    """Run CPU_LEG on the arrays (dict name -> numpy array, written as .npy to
    a temporary directory); returns its JSON result."""
    import tempfile

    import numpy as np
    with tempfile.TemporaryDirectory() as td:
        for name, a in arrays.items():
            np.save(os.path.join(td, name + ".npy"), a)
        code = CPU_LEG % {"oracle": os.path.join(ROOT, "oracle"), "root": ROOT, "dir": td, "emax": emax,
                          "seconds": seconds}
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1", OMP_PROC_BIND="false")
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError("CPU oracle failed: " + r.stderr[-500:])
    return json.loads(r.stdout.strip().splitlines()[-1])


# --------------------------------------------------------------- arms
def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.build()
    threads = os.cpu_count() or 1
    env_code = r"""
import sys, time, json
sys.path.insert(0, %r)
from oracle import Oracle
o = Oracle(%d)
X = o.ms.random_operator(1, True); Y = o.ms.random_operator(2, False)
for _ in range(%d): o.commutator(X, Y, 1, -1)
t0 = time.perf_counter()
for _ in range(%d): o.commutator(X, Y, 1, -1)
t = time.perf_counter() - t0
print(json.dumps({"t": t, "threads": o.num_threads()}))
""" % (os.path.join(ROOT, "oracle"), args.emax, args.warmup, args.steps)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1")
    r = subprocess.run([sys.executable, "-c", env_code], capture_output=True, text=True, env=env, timeout=3600)
    if r.returncode != 0:
        print(json.dumps({"impl": "reference", "unavailable": "C oracle failed: " + r.stderr[-200:]}))
        return
    d = json.loads(r.stdout.strip().splitlines()[-1])
    value = args.steps / d["t"]
    out = {
        "metric": METRIC.format(emax=args.emax), "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * d["t"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": WORKLOAD.format(emax=args.emax), "emax": args.emax,
                   "precision": "fp64 (CPU, OpenMP + BLAS dgemm)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": d["threads"], "kind": "port",
                         "sample": "%d commutators at emax=%d after %d warm-up" % (args.steps, args.emax,
                                                                                   args.warmup)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def e2e_streamed(ig, ms, prec, hX, hY, hZ, steps, barrier, max_ms, nsets=3):
    """Wall time (ms) of `steps` independent host-to-host commutators through
    the C ABI with copies overlapped: uploads on one stream, commutators on a
    second, downloads on a third (issued from a worker thread, since a
    download returns only when its copy is done).  Events keep each operator
    set's upload, commutator and download in order; with `nsets` sets a step's
    upload may run up to nsets - 1 commutators ahead."""
    import concurrent.futures
    import torch
    sets = [(ig.DeviceOperator(ms, 1), ig.DeviceOperator(ms, -1), ig.DeviceOperator(ms, 1)) for _ in range(nsets)]
    sH, sC, sD = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ptr = {s: ctypes.c_void_p(s.cuda_stream) for s in (sH, sC, sD)}
    up = [torch.cuda.Event() for _ in range(nsets)]
    comp = [torch.cuda.Event() for _ in range(nsets)]
    down = [torch.cuda.Event() for _ in range(nsets)]
    for b in range(nsets):
        for e in (comp[b], down[b]):
            e.record(sC)
    pool = concurrent.futures.ThreadPoolExecutor(max_workers=1)

    def upload(k):
        b = k % nsets
        sH.wait_event(comp[b])  # the commutator that last read this set
        sets[b][0].upload_ptr(hX.data_ptr(), ptr[sH])
        sets[b][1].upload_ptr(hY.data_ptr(), ptr[sH])
        up[b].record(sH)

    def download(b):
        sets[b][2].download_ptr(hZ.data_ptr(), ptr[sD])
        down[b].record(sD)

    barrier()
    t0 = time.perf_counter()
    for k in range(min(nsets - 1, steps)):
        upload(k)
    pending = []
    for k in range(steps):
        b = k % nsets
        if k + nsets - 1 < steps:
            upload(k + nsets - 1)
        sC.wait_event(up[b])
        sC.wait_event(down[b])  # the download that last read this set's Z
        ig.Commutator.device_commutator(sets[b][0], sets[b][1], sets[b][2], prec, ptr[sC])
        comp[b].record(sC)
        sD.wait_event(comp[b])
        pending.append(pool.submit(download, b))
        if len(pending) > nsets - 1:
            pending.pop(0).result()
    for f in pending:
        f.result()
    torch.cuda.synchronize()
    barrier()
    ms_total = (time.perf_counter() - t0) * 1000.0
    pool.shutdown()
    return max_ms(ms_total)


def timed_steps(step, steps, barrier, max_ms):
    """CUDA-event time (ms, max over ranks) of `steps` calls of step(), with an
    event after every step; returns (total, per-step list)."""
    import torch
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    barrier()
    ev[0].record()
    for k in range(steps):
        step()
        ev[k + 1].record()
    torch.cuda.synchronize()
    barrier()
    per = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
    return max_ms(ev[0].elapsed_time(ev[-1])), per


def profiled_phases(L, step, nsteps):
    """The library's per-phase CUDA-event timers over nsteps calls of step()
    (a separate pass: the headline timing runs with the timers off)."""
    import torch
    torch.cuda.synchronize()
    L.imsrg_profiler_reset()
    L.imsrg_profiler_enable(1)
    for _ in range(nsteps):
        step()
    torch.cuda.synchronize()
    L.imsrg_profiler_enable(0)
    n = L.imsrg_profiler_names(None, 0)
    buf = ctypes.create_string_buffer(n)
    L.imsrg_profiler_names(buf, n)
    phases = {}
    for name in [x for x in buf.value.decode().split("\n") if x]:
        t = ctypes.c_double()
        c = ctypes.c_longlong()
        L.imsrg_profiler_get(name.encode(), ctypes.byref(t), ctypes.byref(c))
        phases[name] = (t.value, c.value)
    return phases


def roofline(phases, work, emax):
    """Roofline entry of the dominant profiled phase."""
    hbm_peak, bf16_peak, peak_src = measured_peaks()
    best = None
    for name, (tot, cnt) in phases.items():
        kw = kernel_work(name, work)
        if kw and cnt and (best is None or tot > phases[best][0]):
            best = name
    if not best:
        return None
    bound, amount, unit = kernel_work(best, work)
    avg_s = phases[best][0] / phases[best][1] / 1000.0
    if bound == "tensor":
        ach = amount / avg_s / 1e12
        roof = {"kernel": best, "bound": "tensor", "achieved": ach, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": ach / bf16_peak, "traffic": None,
                "issued_bf16_tflops": 21 * ach, "issued_frac": 21 * ach / bf16_peak,
                "note": "achieved counts FP64-equivalent algorithmic flops (the digit products issue 21x "
                        "as many BF16 flops); peak = bf16 dense burst, %s" % peak_src}
    else:
        ach = amount / avg_s / 1e9
        roof = {"kernel": best, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                "frac": ach / hbm_peak, "traffic": None, "note": "peak = HBM copy, %s" % peak_src}
    roof["launch_ms"] = avg_s * 1000.0
    if "CommutatorScalarScalar" in phases:
        roof["share"] = phases[best][0] / max(1e-9, phases["CommutatorScalarScalar"][0])
    tr = profiled_traffic(best, emax)
    if tr:
        roof["traffic"] = tr[0]
        roof["traffic_source"] = "dram__bytes_read.sum + dram__bytes_write.sum per launch, ncu capture of " \
                                 "the same kernel at this emax, summarised in " + tr[1]
    return roof


def calibrate_omega(ig, dX, dY, dOut, prec, lo=10, hi=20):
    """Scale c of Omega = c Y / |Y| for which BCH_Transform(X, Omega) runs a
    number of nested commutators in [lo, hi] (geometric search on |Omega|);
    returns (|Omega|, nested)."""
    ny = dY.norm()
    best = None
    t = 2.0
    for _ in range(16):
        with ig.DeviceOperator(dY.modelspace, -1) as dOm:
            dOm.copy_from(dY)
            dOm.scale(t / ny)
            n = ig.BCH.device_transform(dX, dOm, dOut, prec)
        if best is None or abs(n - (lo + hi) / 2) < abs(best[1] - (lo + hi) / 2):
            best = (t, n)
        if lo <= n <= hi:
            break
        t = t * 1.6 if n < lo else t / 1.3
    return best


def run_gb300(args):
    import numpy as np
    import torch

    import imsrg_gb300 as ig
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = ig.lib()
    ms = ig.ModelSpace(args.emax, "O16", "O16")
    dX = ig.DeviceOperator(ms, 1)
    dY = ig.DeviceOperator(ms, -1)
    dZ = ig.DeviceOperator(ms, 1)
    sx, sy = replica_seeds(rank)
    dX.fill_random(sx)
    dY.fill_random(sy)
    prec = args.precision
    # commutators queue on the stream without a host round trip each; the
    # kernels' status word is read once per timed region
    ms.defer_status(True)

    def step(p=prec):
        ig.Commutator.device_commutator(dX, dY, dZ, p)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def max_ms(x):
        return max_over_ranks(x, device="cuda")

    warm = max(args.warmup, 3)
    for _ in range(warm):
        step()
    ms.check_status()
    barrier()
    # ---- timed region: device-resident operands, phase timers off
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = L.imsrg_kernel_launches()
    elapsed_ms, per_step = timed_steps(step, args.steps, barrier, max_ms)
    launches = L.imsrg_kernel_launches() - launches0
    clocks.stop()
    ms.check_status()
    value = whole_job_value(world, args.steps, elapsed_ms)
    # ---- per-phase CUDA-event timers: a separate pass over the same steps
    nprof = max(1, min(args.steps, 10))
    phases = profiled_phases(L, step, nprof)
    ms.check_status()
    work = algorithmic_work(ms)
    roof = roofline(phases, work, args.emax)
    Zs = dZ.download()  # the split result of the timed region's inputs
    # ---- plain FP64 form (the metric compares split vs FP64)
    fp64 = None
    Zf = None
    if prec == "split":
        step("fp64")
        Zf = dZ.download()
        fp64_err = rank_errors(Zs, Zf, ms.norb)
        nf = 3
        fms, _ = timed_steps(lambda: step("fp64"), nf, barrier, max_ms)
        fms /= nf
        fp64 = {"value": world * 1000.0 / fms, "unit": UNIT, "ms_per_step": fms, "steps": nf,
                "split_vs_fp64_rel_err": fp64_err}
    # ---- ms per BCH step: BCH_Transform(X, Omega), Omega = c Y with |Omega|
    # chosen so that 10-20 nested commutators run
    bch = None
    Bs = Bf = None
    c_omega = 0.0
    if prec == "split":
        with ig.DeviceOperator(ms, 1) as dB, ig.DeviceOperator(ms, -1) as dOm:
            om_norm, _ = calibrate_omega(ig, dX, dY, dB, "split")
            c_omega = om_norm / dY.norm()
            dOm.copy_from(dY)
            dOm.scale(c_omega)
            bch = {"omega_norm": om_norm, "h_norm": dX.norm()}
            for form, reps in (("split", 3), ("fp64", 1)):
                ig.BCH.device_transform(dX, dOm, dB, form)  # warm-up
                nested = []

                def bstep(f=form):
                    nested.append(ig.BCH.device_transform(dX, dOm, dB, f))
                bms, _ = timed_steps(bstep, reps, barrier, max_ms)
                bch[form] = {"ms_per_bch_step": bms / reps, "nested_commutators": nested[-1], "steps": reps}
                if form == "split":
                    Bs = dB.download()
                else:
                    Bf = dB.download()
        bch["split_vs_fp64_rel_err"] = rank_errors(Bs, Bf, ms.norb)
        bch["fp64_over_split"] = bch["fp64"]["ms_per_bch_step"] / bch["split"]["ms_per_bch_step"]
    # ---- end to end: host buffers, H2D + commutator + D2H per step, through the C ABI
    A = ms.arena_size
    hX = torch.empty(A, dtype=torch.float64, pin_memory=True)
    hY = torch.empty(A, dtype=torch.float64, pin_memory=True)
    hZ = torch.empty(A, dtype=torch.float64, pin_memory=True)
    dX.download_ptr(hX.data_ptr())
    dY.download_ptr(hY.data_ptr())
    # as many steps as the device-resident timing: the streamed pipeline's
    # fill (the first upload) and drain (the last download) are inside the
    # timed region, spread over the same step count
    ne = max(1, args.steps)

    def serial_step():
        dX.upload_ptr(hX.data_ptr())
        dY.upload_ptr(hY.data_ptr())
        step()
        dZ.download_ptr(hZ.data_ptr())
    serial_ms, _ = timed_steps(serial_step, ne, barrier, max_ms)
    # streamed: independent commutators with three operator sets; the next
    # steps' uploads and the previous steps' downloads overlap step k's
    # commutator
    pipe_ms = e2e_streamed(ig, ms, prec, hX, hY, hZ, ne, barrier, max_ms)
    ms.check_status()
    ems = min(serial_ms, pipe_ms)
    e2e = {"value": world * ne / (ems / 1000.0), "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * A,
           "d2h_bytes_per_step": 8 * A,
           "mode": "streamed" if pipe_ms <= serial_ms else "serial",
           "serial": {"value": world * ne / (serial_ms / 1000.0), "ms_per_step": serial_ms / ne},
           "streamed": {"value": world * ne / (pipe_ms / 1000.0), "ms_per_step": pipe_ms / ne},
           "note": "per step: H2D of X and Y from pinned host memory, the commutator, D2H of Z, through the C ABI; "
                   "streamed = uploads / downloads on their own streams, three device operator sets"}
    # ---- the 64-pair batch (emax 2..6, one CUDA graph, both forms)
    batch = None
    if not args.no_batch:
        bres, bes, _ = batch_measure(ig, L, 64, 5, 3, 4 + rank)
        batch = {"pairs": 64, "emax_counts": {str(e): bes.count(e) for e in sorted(set(bes))},
                 "unit": "commutators/s",
                 "split": {k: bres["split"][k] for k in ("batched", "sequential", "speedup",
                                                         "grouped_product_launches", "kernel_nodes")},
                 "fp64": {k: bres["fp64"][k] for k in ("batched", "sequential", "speedup",
                                                       "grouped_product_launches", "kernel_nodes")}}
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    # ---- CPU leg (rank 0, N=1 only): baseline and the oracle check
    cpu = None
    oracle_err = None
    if world == 1 and not args.no_cpu_baseline:
        try:
            threads = os.cpu_count() or 1
            arrays = {"X": hX.numpy(), "Y": hY.numpy(), "Z_split": Zs,
                      "Z_fp64": Zf if Zf is not None else Zs, "c": np.array(c_omega)}
            if Bs is not None:
                arrays.update(B_split=Bs, B_fp64=Bf)
            d = cpu_leg(args.emax, args.cpu_seconds, threads, arrays)
            cpu = {"value": d["n"] / d["t"], "unit": UNIT, "cores": d["threads"], "kind": "port",
                   "sample": "%d commutator(s) at emax=%d on the benchmark's X, Y, C oracle (OpenMP over channels + "
                             "SciPy BLAS dgemm)" % (d["n"], args.emax)}
            if "bch_ms" in d:
                cpu["ms_per_bch_step"] = d["bch_ms"]
                cpu["bch_nested_commutators"] = d["bch_nested"]
                bch["cpu"] = {"ms_per_bch_step": d["bch_ms"], "nested_commutators": d["bch_nested"],
                              "cores": d["threads"], "kind": "port"}
                bch["rel_err_vs_oracle"] = d["bch_rel_err_vs_oracle"]
            oracle_err = d["rel_err_vs_oracle"]
        except Exception as ex:  # reported, not fatal
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": "failed: %s" % ex}
    out = {
        "metric": METRIC.format(emax=args.emax), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warm, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD.format(emax=args.emax), "emax": args.emax, "orbits": ms.norb,
                   "largest_2b_channel": max(c["nkets"] for c in ms.channels), "precision": prec,
                   "gemm": "Ozaki BF16 digits on tcgen05, FP32 accumulate, int64/FP64 recombination"
                   if prec == "split" else "FP64 CUDA cores",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "working set > L2 every step (X2, Y2 280 MiB each; Zbar 761 MiB)",
                   "timing": "phase timers off; kernels' status word read once after the K steps",
                   "tuning": ms.tuning()},
        "step_ms": {"min": min(per_step), "median": statistics.median(per_step), "max": max(per_step)},
        "plain_fp64": fp64,
        "split_vs_fp64_rel_err": fp64["split_vs_fp64_rel_err"] if fp64 else None,
        "rel_err_vs_oracle": oracle_err,
        "bch": bch,
        "bch_ms_per_step": {k: bch[k]["ms_per_bch_step"] for k in ("split", "fp64", "cpu") if k in bch}
        if bch else None,
        "e2e": e2e,
        "batch_64_pairs": batch,
        "roofline": roof,
        "phases_ms_per_step": {k: v[0] / nprof for k, v in sorted(phases.items())},
        "phases_steps": nprof,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "gpu_launches": int(launches),
    }
    print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


FLOW_METRIC = "ms per Magnus-Euler flow step (White generator, ds=0.5) at emax={emax}: split vs FP64 on 1 GB300"


def flow_hamiltonian(ig, ms, seed, v2=0.5):
    """The flow workload's H through the product API: a seeded random
    hermitian operator (imsrg_op_fill_random), one-body part replaced by the
    oscillator diagonal 2n+l+3/2 plus symmetric uniform[-0.1,0.1] couplings
    within each (l, j2, tz2) block, two-body part scaled by v2, ZeroBody 0."""
    import numpy as np
    with ig.DeviceOperator(ms, 1) as d:
        d.fill_random(seed)
        a = d.download()
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    N = ms.norb
    one = a[32:32 + N * N].reshape(N, N, order="F")
    one[:, :] = 0.0
    groups = {}
    for i, (n, l, j2, tz2, _) in enumerate(ms.orbits):
        groups.setdefault((l, j2, tz2), []).append(i)
    for grp in groups.values():
        m = len(grp)
        R = np.triu(rng.uniform(-0.1, 0.1, size=(m, m)), 1)
        S = R + R.T
        S[np.diag_indices(m)] = [2 * ms.orbits[i][0] + ms.orbits[i][1] + 1.5 for i in grp]
        one[np.ix_(grp, grp)] = S
    a[0] = 0.0
    a[ms.channels[0]["offset"]:] *= v2
    return a


def run_flow(args):
    import torch

    import imsrg_gb300 as ig
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    L = ig.lib()
    emax = args.emax
    ms = ig.ModelSpace(emax, "O16", "O16")
    H = ig.DeviceOperator(ms, 1)
    H.upload(flow_hamiltonian(ig, ms, 5000 + emax + rank))

    def solver(prec, nsteps):
        sv = ig.IMSRGSolver(H, precision=prec)
        sv.SetGenerator("white")
        sv.SetDs(0.5)
        sv.SetDsmax(0.5)
        sv.SetMagnusAdaptive(False)
        sv.SetOmegaNormMax(1e9)
        sv.SetEtaCriterion(1e-20)
        sv.SetSmax(0.5 * nsteps)
        return sv

    def timed_flow(prec, nsteps):
        sv = solver(prec, max(3, args.warmup))
        sv.Solve()  # warm-up flow: scratch, plans, tables
        del sv
        sv = solver(prec, nsteps)
        torch.cuda.synchronize()
        L.imsrg_profiler_reset()
        L.imsrg_profiler_enable(1)
        l0 = L.imsrg_kernel_launches()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        sv.Solve()
        e1.record()
        torch.cuda.synchronize()
        launches = L.imsrg_kernel_launches() - l0
        L.imsrg_profiler_enable(0)
        ncomm = ctypes.c_longlong()
        t = ctypes.c_double()
        L.imsrg_profiler_get(b"CommutatorScalarScalar", ctypes.byref(t), ctypes.byref(ncomm))
        it, s, e0s, ne, no = sv.history()
        ms_step = e0.elapsed_time(e1) / nsteps
        return {"ms_per_step": ms_step, "steps": int(len(it)), "e0": float(e0s[-1]), "s": float(s[-1]),
                "commutators_per_step": ncomm.value / nsteps, "commutator_ms_per_step": t.value / nsteps,
                "norm_eta_last": float(ne[-1]), "launches": int(launches)}, e0s

    clocks = ClockSampler(local)
    clocks.start()
    split, e_split = timed_flow("split", args.steps)
    clocks.stop()
    nf = args.fp64_steps if args.fp64_steps is not None else min(args.steps, 5)
    fp64, e_fp64 = timed_flow("fp64", nf)
    m = min(len(e_split), len(e_fp64))
    dev = float(max(abs(a - b) / abs(b) for a, b in zip(e_split[:m], e_fp64[:m]))) if m else None
    if rank != 0:
        return
    # CPU baseline: the C oracle's Magnus-Euler flow on the same H for the
    # first step(s), all host cores (bounded sample)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        import tempfile
        ncpu = max(1, args.cpu_flow_steps)
        ha = H.download()
        with tempfile.TemporaryDirectory() as td:
            fn = os.path.join(td, "H.npy")
            import numpy as np
            np.save(fn, ha)
            code = r"""
import sys, time, json
import numpy as np
sys.path.insert(0, %r)
from oracle import Oracle, FlowParams
o = Oracle(%d)
H = np.load(%r)
p = FlowParams(ds=0.5, ds_max=0.5, smax=0.5 * %d, magnus_adaptive=0, omega_norm_max=1e9, eta_criterion=1e-20)
t0 = time.perf_counter()
st = o.magnus_euler(H, p)
t = time.perf_counter() - t0
print(json.dumps({"t": t, "steps": st["steps"], "e0": list(st["e0_hist"]), "e0_final": float(st["Hs"][0]),
                  "threads": o.num_threads()}))
""" % (os.path.join(ROOT, "oracle"), emax, fn, ncpu)
            threads = os.cpu_count() or 1
            env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1")
            try:
                r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                                   timeout=1800)
                d = json.loads(r.stdout.strip().splitlines()[-1])
                e_cpu = d["e0"][0]
                cpu = {"value": 1000.0 * d["t"] / d["steps"], "unit": "ms/step", "cores": d["threads"],
                       "kind": "port", "sample": "%d flow step(s) at emax=%d, C oracle (OpenMP + SciPy BLAS); "
                                                 "table setup excluded" % (d["steps"], emax),
                       "e0_step1": e_cpu,
                       "e0_step1_rel_split": abs(e_split[0] - e_cpu) / abs(e_cpu),
                       "e0_step1_rel_fp64": abs(e_fp64[0] - e_cpu) / abs(e_cpu),
                       "steps": d["steps"], "e0_final": d["e0_final"]}
                # the zero-body value after the CPU flow's last step against
                # each GPU flow after the same step (history entry k holds
                # H(s).ZeroBody after step k + 1, in both flows)
                n = d["steps"]
                for form, e_hist in (("split", e_split), ("fp64", e_fp64)):
                    if 0 < n <= len(e_hist):
                        cpu["e0_final_rel_" + form] = abs(e_hist[n - 1] - d["e0_final"]) / abs(d["e0_final"])
            except Exception as ex:  # reported, not fatal
                cpu = {"value": None, "unit": "ms/step", "kind": "port", "sample": "failed: %s" % ex}
    out = {
        "metric": FLOW_METRIC.format(emax=emax), "value": split["ms_per_step"], "unit": "ms/step",
        "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": split["ms_per_step"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "Magnus-Euler flow, White generator, Epstein-Nesbet, ds=0.5 fixed, emax=%d O16, "
                               "H: oscillator 1b diagonal + uniform[-0.1,0.1] couplings, random hermitian 2b at "
                               "Frobenius 0.5 per channel" % emax,
                   "emax": emax, "orbits": ms.norb, "precision": "split",
                   "l2": "working set > L2 every step"},
        "split": split, "plain_fp64": fp64,
        "e0_max_rel_split_vs_fp64": dev, "e0_steps_compared": m, "cpu_baseline": cpu,
        "clocks": clocks.summary(), "gpu_launches": split["launches"],
    }
    print(json.dumps(out))


BATCH_METRIC = "[X,Y] commutators/sec, {n} independent pairs with emax drawn from {{2..6}}, one CUDA graph"


def batch_measure(ig, L, npairs, K, W, seed, batch_emax=None):
    """The 64-pair configuration: npairs independent (X, Y) pairs, emax drawn
    from {2..6} by seed, one model space per pair; both forms timed as one
    CUDA-graph batch and as one-by-one calls.  Returns (per form results,
    emax list, operator bytes)."""
    import numpy as np
    import torch
    rng = np.random.Generator(np.random.PCG64(seed))
    es = [int(e) for e in rng.choice([2, 3, 4, 5, 6], size=npairs)]
    if batch_emax is not None:
        es = [batch_emax] * npairs
    pairs = []
    arena_bytes = 0
    for i, e in enumerate(es):
        ms = ig.ModelSpace(e, "O16", "O16")
        dX, dY, dZ = ig.DeviceOperator(ms, 1), ig.DeviceOperator(ms, -1), ig.DeviceOperator(ms, 1)
        dX.fill_random(1000 + 2 * i)
        dY.fill_random(1001 + 2 * i)
        pairs.append((dX, dY, dZ))
        arena_bytes += 3 * 8 * ms.arena_size

    def timed(fn):
        for _ in range(W):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(K):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / K

    res = {}
    for prec in ("split", "fp64"):
        def sequential(p=prec):
            for dX, dY, dZ in pairs:
                ig.Commutator.device_commutator(dX, dY, dZ, p)
        seq_ms = timed(sequential)
        b = ig.CommutatorBatch(pairs, prec)
        n, groups, grouped, nodes = b.info()
        l0 = L.imsrg_kernel_launches()
        bat_ms = timed(b.launch)
        b.sync()
        launches = (L.imsrg_kernel_launches() - l0) // (K + W)
        res[prec] = {"batched_ms": bat_ms, "sequential_ms": seq_ms,
                     "batched": npairs * 1000.0 / bat_ms, "sequential": npairs * 1000.0 / seq_ms,
                     "speedup": seq_ms / bat_ms, "graph_branches": groups, "grouped_product_launches": grouped,
                     "kernel_nodes": nodes,
                     "launches_per_step": int(launches)}
        b.close()
    return res, es, arena_bytes


def run_batch(args):
    import torch

    import imsrg_gb300 as ig
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    L = ig.lib()
    K, W = args.steps, max(3, args.warmup)
    res, es, arena_bytes = batch_measure(ig, L, args.pairs, K, W, 4 + rank, args.batch_emax)
    if rank != 0:
        return
    sp = res["split"]
    out = {
        "metric": BATCH_METRIC.format(n=args.pairs), "value": sp["batched"], "unit": "commutators/s",
        "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": sp["batched_ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "%d pairs, X hermitian / Y anti-hermitian, emax per pair %s (seeded), one model "
                               "space per pair" % (args.pairs, "".join(str(e) for e in es)),
                   "emax_counts": {str(e): es.count(e) for e in sorted(set(es))},
                   "operator_bytes": arena_bytes, "precision": "split"},
        "split": sp, "plain_fp64": res["fp64"], "gpu_launches": sp["launches_per_step"] * K,
    }
    print(json.dumps(out))


TENSOR_METRIC = ("ms per scalar-tensor commutator [X,T], rank (J,dTz,parity)=(2,0,+), emax={emax}: {form} form "
                 "(split-prec vs FP64 products), 1 GB300")


def random_tensor(ms, seed, rank, hermitian=True):
    """Seeded random reduced tensor in the C ABI's tensor arena (uniform[-1,1]
    on allowed elements, unit Frobenius norm per block and for the one-body
    matrix, <j||T||i> = h (-1)^(ji-jj) <i||T||j>, diagonal blocks (anti)symmetric)."""
    import numpy as np
    lam, trank, par = rank
    rng = np.random.Generator(np.random.PCG64(seed))
    a = np.zeros(ms.tensor_size(*rank))
    h = 1.0 if hermitian else -1.0
    N = ms.norb
    orb = ms.orbits
    one = a[32:32 + N * N].reshape(N, N, order="F")
    for i in range(N):
        for j in range(i, N):
            li, ji, ti = orb[i][1], orb[i][2], orb[i][3]
            lj, jj, tj = orb[j][1], orb[j][2], orb[j][3]
            if (li + lj + par) % 2 or abs(ji - jj) > 2 * lam or ji + jj < 2 * lam or abs(ti - tj) != 2 * trank:
                continue
            ph = -1.0 if ((ji - jj) // 2) % 2 else 1.0
            if i == j and h * ph < 0:
                continue
            v = rng.uniform(-1, 1)
            one[i, j] = v
            one[j, i] = h * ph * v
    one /= max(np.linalg.norm(one), 1e-300)
    for (cb, ck), o in ms.tensor_layout(*rank).items():
        nb, nk = ms.channels[cb]["nkets"], ms.channels[ck]["nkets"]
        if nb == 0 or nk == 0:
            continue
        R = rng.uniform(-1, 1, size=(nb, nk))
        if cb == ck:
            R = 0.5 * (R + h * R.T)
        a[o:o + nb * nk] = (R / max(np.linalg.norm(R), 1e-300)).ravel(order="F")
    return a


def run_tensor(args):
    """Scalar-tensor commutator [X, T] at emax (default 8), both forms of its
    ladder and Z bar products: split (tensor cores) and FP64.  `value` is the
    form --precision names; the other is reported beside it, with the
    relative difference of the two results per body rank."""
    import numpy as np
    import torch

    import imsrg_gb300 as ig
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    L = ig.lib()
    emax = args.emax
    ms = ig.ModelSpace(emax, "O16", "O16")
    rk = (2, 0, 0)
    dX = ig.DeviceOperator(ms, 1)
    dX.fill_random(31 + rank)
    dT = ig.DeviceOperator(ms, 1, rk)
    dT.upload(random_tensor(ms, 41 + rank, rk))
    dZ = ig.DeviceOperator(ms, 1, rk)

    def timed(prec):
        for _ in range(max(3, args.warmup)):
            ig.Commutator.device_scalar_tensor(dX, dT, dZ, prec)
        torch.cuda.synchronize()
        L.imsrg_profiler_reset()
        L.imsrg_profiler_enable(1)
        l0 = L.imsrg_kernel_launches()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            ig.Commutator.device_scalar_tensor(dX, dT, dZ, prec)
        e1.record()
        torch.cuda.synchronize()
        launches = L.imsrg_kernel_launches() - l0
        L.imsrg_profiler_enable(0)
        n = L.imsrg_profiler_names(None, 0)
        buf = ctypes.create_string_buffer(n)
        L.imsrg_profiler_names(buf, n)
        phases = {}
        for name in [x for x in buf.value.decode().split("\n") if x]:
            t = ctypes.c_double()
            c = ctypes.c_longlong()
            L.imsrg_profiler_get(name.encode(), ctypes.byref(t), ctypes.byref(c))
            phases[name] = t.value / args.steps
        return e0.elapsed_time(e1) / args.steps, phases, int(launches), dZ.download()

    forms = [args.precision] + [p for p in ("split", "fp64") if p != args.precision]
    res = {p: timed(p) for p in forms}
    ms_step, phases, launches, Zv = res[args.precision]
    Zo = res[forms[1]][3]
    N = ms.norb
    diff = []
    for a, b in ((Zv[32:32 + N * N], Zo[32:32 + N * N]), (Zv[32 + N * N:], Zo[32 + N * N:])):
        nb = np.linalg.norm(b)
        diff.append(float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b)))
    if rank != 0:
        return
    out = {
        "metric": TENSOR_METRIC.format(emax=emax, form=args.precision), "value": ms_step, "unit": "ms/commutator",
        "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_step,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "CommutatorScalarTensor [X, T], X random hermitian scalar, T random hermitian "
                               "reduced tensor of rank (2, 0, 0), emax=%d O16" % emax, "emax": emax,
                   "tensor_arena_doubles": dT.size, "precision": args.precision},
        "phases_ms_per_step": phases, "gpu_launches": launches,
        forms[1]: {"ms_per_step": res[forms[1]][0], "phases_ms_per_step": res[forms[1]][1]},
        "rel_diff_%s_vs_%s" % (forms[0], forms[1]): {"one_body": diff[0], "two_body": diff[1]},
        "cpu_baseline": {"value": None, "unit": "ms/commutator", "kind": "port",
                         "sample": "not measured: the C oracle restates the scalar-scalar path only"},
    }
    print(json.dumps(out))


def main():
    args = parse_args()
    if args.emax is None:
        args.emax = {"flow": 12, "tensor": 8}.get(args.workload, 10)
    if args.workload == "tensor":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference's scalar-tensor commutator is not "
                              "built for the GPU host; the headline reference arm is the emax=10 commutator"}))
            return
        run_tensor(args)
        return
    if args.workload == "batch":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batch workload compares the GPU's batched "
                              "and one-by-one launches; the CPU reference arm is the emax=10 commutator"}))
            return
        run_batch(args)
        return
    if args.workload == "flow":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the CPU flow at emax=12 takes hours; the flow "
                              "parity tests compare against the reference's own flow at emax 2-3"}))
            return
        run_flow(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
