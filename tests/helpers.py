"""Shared helpers of the tests: golden fixtures and per-body-rank errors."""
import os

import numpy as np

from modelspace_ref import RefModelSpace

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TERMS = ["comm110ss", "comm220ss", "comm111ss", "comm121ss", "comm122ss", "comm222_pp_hh_221ss",
         "comm222_pp_hhss", "comm221ss", "comm222_phss"]
CASES = {"xy": ("X", "Y", 1, -1), "yx": ("Y", "X", -1, 1), "xw": ("X", "W", 1, 1)}


def load_golden(emax):
    return dict(np.load(os.path.join(GOLDEN, "golden_emax%d.npz" % emax)))


def body_parts(ms, a):
    """(0b scalar, 1b matrix, concatenated 2b blocks) of an arena."""
    z0 = a[0]
    z1 = ms.onebody(a)
    z2 = np.concatenate([ms.block(a, c).ravel() for c in range(ms.nch)])
    return z0, z1, z2


def rel_errors(ms, Z, R, floor=None):
    """Relative Frobenius error per body rank of Z against R.  When a rank of R
    vanishes the error is taken relative to `floor` (default: norm of R)."""
    z = body_parts(ms, Z)
    r = body_parts(ms, R)
    tot = max(np.linalg.norm(R), 1e-300) if floor is None else floor
    out = []
    for a, b in zip(z, r):
        d = np.linalg.norm(np.asarray(a) - np.asarray(b))
        nb = np.linalg.norm(b)
        out.append(d / nb if nb > 1e-12 * tot else d / tot)
    return out


def ref_space(emax):
    return RefModelSpace(emax)


def load_flow_golden(emax):
    return dict(np.load(os.path.join(GOLDEN, "golden_flow_emax%d.npz" % emax)))


def load_tensor_golden(emax, nucleus=None):
    suffix = "" if nucleus is None else "_" + nucleus
    return dict(np.load(os.path.join(GOLDEN, "golden_tensor_emax%d%s.npz" % (emax, suffix))))


def tensor_rel_errors(ms, rank, Z, R):
    """rel_errors for tensor arenas of rank (J, T, parity): one-body matrix and
    the concatenated two-body blocks."""
    blocks, offs, _ = ms.tensor_layout(*rank)

    def parts(a):
        N = ms.norb
        two = [a[o:o + len(ms.channels[cb][3]) * len(ms.channels[ck][3])] for (cb, ck), o in zip(blocks, offs)]
        return a[32:32 + N * N], np.concatenate(two) if two else np.zeros(0)

    tot = max(np.linalg.norm(R), 1e-300)
    out = []
    for x, y in zip(parts(Z), parts(R)):
        d = np.linalg.norm(x - y)
        ny = np.linalg.norm(y)
        out.append(d / ny if ny > 1e-12 * tot else d / tot)
    return out
