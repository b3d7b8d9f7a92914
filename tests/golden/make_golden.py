"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference IMSRG++ commutator code, compiled from its own sources by
oracle/ref_build.mk into oracle/_ref/ref_harness, on seeded random operators
and stores inputs and outputs as compressed .npz files.  Needs the reference
sources (build container only):

    make -f oracle/ref_build.mk -j8
    python tests/golden/make_golden.py

Fixtures (arena layout: see oracle/modelspace_ref.py):
  golden_emax2.npz   X (hermitian), Y (anti-hermitian), W (hermitian); for the
                     cases xy=[X,Y], yx=[Y,X], xw=[X,W]: every IMSRG(2) term on a
                     zeroed Z and the full CommutatorScalarScalar; the
                     BCH_Transform of X with Omega = 0.25 Y/|Y|; the reference's
                     channel tables; Operator::Norm of the inputs; the
                     single-operator Pandya transform of X and Y in both
                     orientations (every cross-coupled channel, concatenated,
                     with the normal orientation's dimensions); the bytes
                     Operator::WriteBinary writes for X and Y.
  golden_emax3.npz   the same for the case xy only, plus bch.
  golden_flow_emax2.npz, golden_flow_emax3.npz
                     H (flow Hamiltonian, RefModelSpace.flow_hamiltonian with
                     two-body scale 0.5), A = 0.05 V/|V| and B = 0.5 U/|U|
                     (anti-hermitian); BCH::BCH_Product(A, B) and of (6A, 2B); the White,
                     atan, qtransfer-atan and qtransfer-atan_2 generators of H
                     (Epstein-Nesbet) and White with Moller-Plesset denominators; ten fixed Magnus-Euler steps
                     (ds 0.5, White generator) with s and E0 after each step and
                     the final H(s), Omega; an adaptive flow to s = 2 with Omega
                     split at |Omega| > 0.3 (final s, number of Omegas, E0,
                     H(s), last Omega); the same flow with the
                     magnus_modified_euler and magnus_backoff methods, and
                     the fixed-step flow_RK4 flow of H (final s, number of
                     Omegas, E0 and H(s)); flow_RK4 also flows an added
                     observable [A, H] (AddOperator; the input and GetOperator(1)).
  golden_tensor_emax2.npz, golden_tensor_emax3.npz
                     Commutator::CommutatorScalarTensor [X, T] and its five
                     IMSRG(2) terms (comm111st, comm121st, comm122st,
                     comm222_pp_hh_221st, comm222_phst) for X a random hermitian
                     scalar and T random reduced tensors (RefModelSpace.
                     random_tensor) of rank (J, T, parity) = (2, 0, 0)
                     hermitian, (1, 0, 1) hermitian and (1, 1, 0)
                     anti-hermitian at emax 2; the first case only at emax 3.
                     Per case also BCH::BCH_Transform(T, Omega) for the
                     scalar Omega = 0.2 X / |X| (with Omega itself), and the
                     Operator::Norm of T, of [X, T] and of the transform, with
                     T's one- and two-body norms, and Operator::WriteBinary of T.
  golden_tensor_emax3_O18.npz
                     the same on O18's space (fractional 0d5/2 neutron
                     occupations) for the ranks (2, 0, 0) hermitian and
                     (1, 1, 0) anti-hermitian.
  sixj_exact.npz     6j symbols {j1 j2 J3; j4 j5 J6} for half-integer
                     j <= 9/2 and integer J <= 9, evaluated in exact rational
                     arithmetic (Racah formula with Python integers), the pin for
                     every 6j implementation in this repository.
"""

import os
import subprocess
import sys
import tempfile
from fractions import Fraction
from math import factorial, isqrt
from decimal import Decimal, getcontext

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from modelspace_ref import RefModelSpace  # noqa: E402

TERMS = ["comm110ss", "comm220ss", "comm111ss", "comm121ss", "comm122ss",
         "comm222_pp_hh_221ss", "comm222_pp_hhss", "comm221ss", "comm222_phss", "full"]


def run_reference(emax, cases):
    ms = RefModelSpace(emax)
    X = ms.random_operator(1000 + emax, hermitian=True)
    Y = ms.random_operator(2000 + emax, hermitian=False)
    W = ms.random_operator(3000 + emax, hermitian=True)
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    with tempfile.TemporaryDirectory() as td:
        for name, a in (("X", X), ("Y", Y), ("W", W)):
            a.tofile(os.path.join(td, name + ".bin"))
        subprocess.run([harness, str(emax), os.path.join(td, "X.bin"), os.path.join(td, "Y.bin"),
                        os.path.join(td, "W.bin"), td], check=True, stdout=subprocess.DEVNULL,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
        out = {"X": X, "Y": Y, "W": W, "emax": np.array(emax)}
        for cs in cases:
            for t in TERMS:
                out["%s_%s" % (cs, t)] = np.fromfile(os.path.join(td, "%s_%s.bin" % (cs, t)))
        out["bch"] = np.fromfile(os.path.join(td, "bch.bin"))
        for k in ("X", "Y"):
            out[k + "_binary"] = np.fromfile(os.path.join(td, k + "_op.bin"), dtype=np.uint8)
        for k in ("X_normal", "X_transpose", "Y_normal", "Y_transpose"):
            out["pandya_" + k] = np.fromfile(os.path.join(td, "pandya_%s.bin" % k))
        out["pandya_dims"] = np.loadtxt(os.path.join(td, "pandya_dims.txt"), dtype=np.int64).reshape(-1, 3)
        with open(os.path.join(td, "tables.txt")) as f:
            out["tables"] = np.array(f.read())
        with open(os.path.join(td, "norms.txt")) as f:
            out["norms"] = np.array([float(x) for x in f.read().split()])
    return out


FLOW_STEPS = 10
FLOW_V2 = 0.5


def flow_inputs(emax):
    ms = RefModelSpace(emax)
    H = ms.flow_hamiltonian(5000 + emax, FLOW_V2)
    A = ms.random_operator(6000 + emax, hermitian=False)
    A *= 0.05 / ms.norm(A)
    B = ms.random_operator(7000 + emax, hermitian=False)
    B *= 0.5 / ms.norm(B)
    return H, A, B


def run_reference_flow(emax):
    H, A, B = flow_inputs(emax)
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    with tempfile.TemporaryDirectory() as td:
        for name, a in (("H", H), ("A", A), ("B", B)):
            a.tofile(os.path.join(td, name + ".bin"))
        subprocess.run([harness, "flow", str(emax), os.path.join(td, "H.bin"), os.path.join(td, "A.bin"),
                        os.path.join(td, "B.bin"), str(FLOW_STEPS), td], check=True, stdout=subprocess.DEVNULL,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
        out = {"H": H, "A": A, "B": B, "emax": np.array(emax), "v2": np.array(FLOW_V2)}
        for k in ("bchp", "bchp_big", "eta_white", "eta_atan", "eta_white_mp", "flow_Hs", "flow_Omega", "flow2_Hs",
                  "flow2_Omega", "flow_me_Hs", "flow_bo_Hs", "flow_rk4_Hs", "flow_rk4_obs_in", "flow_rk4_obs",
                  "eta_qt", "eta_qt2"):
            out[k] = np.fromfile(os.path.join(td, k + ".bin"))
        out["flow_steps"] = np.loadtxt(os.path.join(td, "flow_steps.txt"))
        out["flow2"] = np.loadtxt(os.path.join(td, "flow2.txt"))
        out["flow_me"] = np.loadtxt(os.path.join(td, "flow_me.txt"))
        out["flow_bo"] = np.loadtxt(os.path.join(td, "flow_bo.txt"))
        out["flow_rk4"] = np.loadtxt(os.path.join(td, "flow_rk4.txt"))
    return out


TENSOR_CASES = {"e2": (2, 0, 0, 1), "e1": (1, 0, 1, 1), "gt": (1, 1, 0, -1)}
TENSOR_TERMS = ["comm111st", "comm121st", "comm122st", "comm222_pp_hh_221st", "comm222_phst", "full"]


def run_reference_tensor(emax, cases, nucleus=None):
    """nucleus: None for O16, else (name, A, Z) of the reference the space
    is built on (its occupations enter the terms; the arenas' layout does
    not change)."""
    ms = RefModelSpace(emax) if nucleus is None else RefModelSpace(emax, nucleus[1], nucleus[2])
    X = ms.random_operator(1000 + emax, hermitian=True)
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    out = {"X": X, "emax": np.array(emax)}
    with tempfile.TemporaryDirectory() as td:
        X.tofile(os.path.join(td, "X.bin"))
        for i, name in enumerate(cases):
            lam, trank, par, herm = TENSOR_CASES[name]
            T = ms.random_tensor(8000 + 10 * emax + i, lam, trank, par, hermitian=herm > 0)
            T.tofile(os.path.join(td, "T.bin"))
            cmd = [harness, "tensor", str(emax), str(lam), str(trank), str(par), str(herm),
                   os.path.join(td, "X.bin"), os.path.join(td, "T.bin"), td]
            if nucleus is not None:
                cmd.append(nucleus[0])
            subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, env=dict(os.environ, OMP_NUM_THREADS="1"))
            out[name + "_T"] = T
            out[name + "_rank"] = np.array([lam, trank, par, herm])
            for t in TENSOR_TERMS:
                out["%s_%s" % (name, t)] = np.fromfile(os.path.join(td, "st_%s.bin" % t))
            out[name + "_omega"] = np.fromfile(os.path.join(td, "st_omega.bin"))
            out[name + "_bch"] = np.fromfile(os.path.join(td, "st_bch.bin"))
            out[name + "_norms"] = np.loadtxt(os.path.join(td, "st_norms.txt"))
            out[name + "_binary"] = np.fromfile(os.path.join(td, "st_T_op.bin"), dtype=np.uint8)
            out[name + "_blocks"] = np.loadtxt(os.path.join(td, "tensor_blocks.txt"), dtype=np.int64).reshape(-1, 4)
    return out


def _delta2(a, b, c):
    # a, b, c doubled
    return Fraction(factorial((a + b - c) // 2) * factorial((a - b + c) // 2) * factorial((-a + b + c) // 2),
                    factorial((a + b + c) // 2 + 1))


def _triad(a, b, c):
    return (a + b + c) % 2 == 0 and abs(a - b) <= c <= a + b


def sixj_exact(ja, jb, jc, jd, je, jf):
    """6j with doubled arguments, exact: Racah single sum in rationals, then
    sign * sqrt(prefactor^2) * |sum| rounded to double via 40-digit Decimal."""
    if not (_triad(ja, jb, jc) and _triad(ja, je, jf) and _triad(jd, jb, jf) and _triad(jd, je, jc)):
        return 0.0
    a1, a2, a3, a4 = (ja + jb + jc) // 2, (ja + je + jf) // 2, (jd + jb + jf) // 2, (jd + je + jc) // 2
    b1, b2, b3 = (ja + jb + jd + je) // 2, (ja + jc + jd + jf) // 2, (jb + jc + je + jf) // 2
    s = Fraction(0)
    for t in range(max(a1, a2, a3, a4), min(b1, b2, b3) + 1):
        den = (factorial(t - a1) * factorial(t - a2) * factorial(t - a3) * factorial(t - a4)
               * factorial(b1 - t) * factorial(b2 - t) * factorial(b3 - t))
        s += Fraction((-1) ** t * factorial(t + 1), den)
    if s == 0:
        return 0.0
    pre2 = _delta2(ja, jb, jc) * _delta2(ja, je, jf) * _delta2(jd, jb, jf) * _delta2(jd, je, jc)
    val2 = pre2 * s * s
    getcontext().prec = 40
    v = (Decimal(val2.numerator) / Decimal(val2.denominator)).sqrt()
    return float(v) if s > 0 else -float(v)


def make_sixj_table(jj1max=9, jmax=9):
    rows = []
    for ja in range(1, jj1max + 1, 2):
        for jb in range(1, jj1max + 1, 2):
            for J3 in range(0, jmax + 1):
                for jd in range(1, jj1max + 1, 2):
                    for je in range(1, jj1max + 1, 2):
                        for J6 in range(0, jmax + 1):
                            v = sixj_exact(ja, jb, 2 * J3, jd, je, 2 * J6)
                            if v != 0.0:
                                rows.append((ja, jb, J3, jd, je, J6, v))
    arr = np.array(rows)
    return arr[:, :6].astype(np.int16), arr[:, 6].copy()


def main():
    g2 = run_reference(2, ["xy", "yx", "xw"])
    np.savez_compressed(os.path.join(HERE, "golden_emax2.npz"), **g2)
    g3 = run_reference(3, ["xy"])
    np.savez_compressed(os.path.join(HERE, "golden_emax3.npz"), **g3)
    for e in (2, 3):
        np.savez_compressed(os.path.join(HERE, "golden_flow_emax%d.npz" % e), **run_reference_flow(e))
    np.savez_compressed(os.path.join(HERE, "golden_tensor_emax2.npz"), **run_reference_tensor(2, ["e2", "e1", "gt"]))
    np.savez_compressed(os.path.join(HERE, "golden_tensor_emax3.npz"), **run_reference_tensor(3, ["e2"]))
    np.savez_compressed(os.path.join(HERE, "golden_tensor_emax3_O18.npz"),
                        **run_reference_tensor(3, ["e2", "gt"], ("O18", 18, 8)))
    keys, vals = make_sixj_table()
    np.savez_compressed(os.path.join(HERE, "sixj_exact.npz"), keys=keys, values=vals)
    for f in ("golden_emax2.npz", "golden_emax3.npz", "golden_flow_emax2.npz", "golden_flow_emax3.npz",
              "golden_tensor_emax2.npz", "golden_tensor_emax3.npz", "golden_tensor_emax3_O18.npz", "sixj_exact.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    if sys.argv[1:] == ["--commutator"]:
        np.savez_compressed(os.path.join(HERE, "golden_emax2.npz"), **run_reference(2, ["xy", "yx", "xw"]))
        np.savez_compressed(os.path.join(HERE, "golden_emax3.npz"), **run_reference(3, ["xy"]))
    elif sys.argv[1:] == ["--tensor"]:
        np.savez_compressed(os.path.join(HERE, "golden_tensor_emax2.npz"),
                            **run_reference_tensor(2, ["e2", "e1", "gt"]))
        np.savez_compressed(os.path.join(HERE, "golden_tensor_emax3.npz"), **run_reference_tensor(3, ["e2"]))
        np.savez_compressed(os.path.join(HERE, "golden_tensor_emax3_O18.npz"),
                            **run_reference_tensor(3, ["e2", "gt"], ("O18", 18, 8)))
    elif sys.argv[1:] == ["--flow"]:
        for e in (2, 3):
            np.savez_compressed(os.path.join(HERE, "golden_flow_emax%d.npz" % e), **run_reference_flow(e))
    else:
        main()
