"""Test infrastructure: NOT part of the product.

Times the reference's own CommutatorScalarScalar (IMSRG++ compiled from its
sources by oracle/ref_build.mk: ref_harness with Armadillo's built-in product,
ref_harness_blas with SciPy's OpenBLAS) against the C oracle port
(oracle/imsrg_oracle.c with SciPy's dgemm) on the same seeded X, Y and the same
OpenMP thread count, one BLAS thread each.  Runs where the reference build
exists (the build container):

    make -f oracle/ref_build.mk REF=<checkout> SCIPY_OPENBLAS=<so> all blas -j8
    python oracle/time_reference.py [--emax 6 8] [--reps 3] [--threads N]

Prints one JSON line per emax with seconds per commutator of each.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def harness_time(exe, emax, xf, yf, reps, env):
    r = subprocess.run([exe, "time", str(emax), xf, yf, str(reps)], capture_output=True, text=True, env=env,
                       timeout=7200)
    if r.returncode != 0:
        raise RuntimeError("%s failed: %s" % (exe, r.stderr[-300:]))
    f = r.stdout.split()
    return float(f[f.index("seconds_per_commutator") + 1]), int(f[f.index("threads") + 1])


def oracle_time(emax, xf, yf, reps, env):
    code = r"""
import sys, time, json
import numpy as np
sys.path.insert(0, %r)
from oracle import Oracle
o = Oracle(%d)
X = np.fromfile(%r); Y = np.fromfile(%r)
o.commutator(X, Y, 1, -1)
t0 = time.perf_counter()
for _ in range(%d): o.commutator(X, Y, 1, -1)
print(json.dumps({"t": (time.perf_counter() - t0) / %d, "threads": o.num_threads()}))
""" % (HERE, emax, xf, yf, reps, reps)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=7200)
    if r.returncode != 0:
        raise RuntimeError("oracle failed: " + r.stderr[-300:])
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return d["t"], d["threads"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--emax", type=int, nargs="+", default=[6, 8])
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    from oracle import Oracle
    env = dict(os.environ, OMP_NUM_THREADS=str(a.threads), OPENBLAS_NUM_THREADS="1", OMP_PROC_BIND="false")
    out_dir = os.path.join(HERE, "_ref")
    for emax in a.emax:
        o = Oracle(emax)
        X = o.ms.random_operator(1, True)
        Y = o.ms.random_operator(2, False)
        del o
        with tempfile.TemporaryDirectory() as td:
            xf, yf = os.path.join(td, "X.bin"), os.path.join(td, "Y.bin")
            X.tofile(xf)
            Y.tofile(yf)
            row = {"emax": emax, "threads": a.threads, "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
            for name, exe in (("reference_builtin_product", "ref_harness"), ("reference_openblas", "ref_harness_blas")):
                path = os.path.join(out_dir, exe)
                if os.path.exists(path):
                    row[name] = harness_time(path, emax, xf, yf, a.reps, env)[0]
            row["c_oracle_port"] = oracle_time(emax, xf, yf, a.reps, env)[0]
        if "reference_openblas" in row:
            row["port_over_reference_openblas"] = row["c_oracle_port"] / row["reference_openblas"]
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
