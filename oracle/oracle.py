"""Test infrastructure: NOT part of the product.

ctypes wrapper around the C oracle (oracle/imsrg_oracle.c), the CPU
restatement of the reference's IMSRG(2) commutator, BCH transform and
product, White-type generators and Magnus-Euler solver, used as the checker in
tests/ and as the CPU baseline in bench.py.  Compiled on first use with gcc
into oracle/_build/ (a plain C + OpenMP shared library).  Matrix products go
through SciPy's BLAS dgemm (the reference multiplies through BLAS too); pass
use_blas=False for the plain loop.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

from modelspace_ref import RefModelSpace

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libimsrg_oracle.so")
_lock = threading.Lock()
_lib = None

TERM_INDEX = {"comm110ss": 0, "comm220ss": 1, "comm111ss": 2, "comm121ss": 3, "comm122ss": 4,
              "comm222_pp_hhss": 5, "comm221ss": 6, "comm222_phss": 7}


def build(force=False):
    """Compile libimsrg_oracle.so (seconds)."""
    src = os.path.join(HERE, "imsrg_oracle.c")
    stub = os.path.join(HERE, "ref_stubs", "coupling_stub.c")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(stub))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=gnu11", "-I", HERE, src, "-o", tmp, "-lm"],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB)
            P = ctypes.c_void_p
            D = ctypes.POINTER(ctypes.c_double)
            I = ctypes.POINTER(ctypes.c_int)
            L.oracle_space_create.restype = P
            L.oracle_space_create.argtypes = [ctypes.c_int, ctypes.c_int, I, I, I, D, ctypes.c_int, I, I, I, I, I, I]
            L.oracle_space_destroy.argtypes = [P]
            L.oracle_arena_size.restype = ctypes.c_int64
            L.oracle_arena_size.argtypes = [P]
            L.oracle_set_dgemm.argtypes = [P, P]
            L.oracle_set_term.argtypes = [P, ctypes.c_int, ctypes.c_int]
            L.oracle_sixj.restype = ctypes.c_double
            L.oracle_sixj.argtypes = [P] + [ctypes.c_int] * 6
            for nm in ("oracle_comm110ss", "oracle_comm220ss"):
                getattr(L, nm).argtypes = [P, D, D, D, ctypes.c_int, ctypes.c_int]
            L.oracle_comm111ss.argtypes = [P, D, D, D]
            L.oracle_comm121ss.argtypes = [P, D, D, D, ctypes.c_int]
            L.oracle_comm122ss.argtypes = [P, D, D, D, ctypes.c_int]
            L.oracle_comm222_pp_hh_221ss.argtypes = [P, D, D, D, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            L.oracle_comm222_phss.argtypes = [P, D, D, D, ctypes.c_int, ctypes.c_int]
            L.oracle_commutator.argtypes = [P, D, D, D, ctypes.c_int, ctypes.c_int]
            L.oracle_norm.restype = ctypes.c_double
            L.oracle_norm.argtypes = [P, D]
            L.oracle_bch_transform.restype = ctypes.c_int
            L.oracle_bch_transform.argtypes = [P, D, ctypes.c_int, D, ctypes.c_int, D, ctypes.c_double]
            L.oracle_pandya_channel.restype = ctypes.c_int
            L.oracle_pandya_channel.argtypes = [P, D, ctypes.c_int, ctypes.c_int, ctypes.c_int, D]
            L.oracle_bch_product.restype = ctypes.c_int
            L.oracle_bch_product.argtypes = [P, D, ctypes.c_int, D, ctypes.c_int, D, ctypes.c_double]
            L.oracle_generator.argtypes = [P, D, D, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int]
            L.oracle_magnus_euler.restype = ctypes.c_int
            L.oracle_magnus_euler.argtypes = [P, D, D, D, D, D, ctypes.POINTER(FlowParams), D,
                                              ctypes.POINTER(ctypes.c_int), D, D, ctypes.c_int]
            L.oracle_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


GENERATORS = {"white": 0, "atan": 1, "wegner": 2, "imaginary-time": 3}
PARTITIONINGS = {"Epstein_Nesbet": 0, "Moller_Plesset": 1}


class FlowParams(ctypes.Structure):
    """oflow_params of imsrg_oracle.c; defaults of IMSRGSolver(H)
    (src/IMSRGSolver.cc:31-37), Generator() (src/Generator.cc:18-20) and BCH
    (src/BCH.cc:16-17)."""
    _fields_ = [("ds", ctypes.c_double), ("ds_max", ctypes.c_double), ("smax", ctypes.c_double),
                ("norm_domega", ctypes.c_double), ("omega_norm_max", ctypes.c_double),
                ("eta_criterion", ctypes.c_double), ("magnus_adaptive", ctypes.c_int), ("generator", ctypes.c_int),
                ("partitioning", ctypes.c_int), ("denominator_cutoff", ctypes.c_double),
                ("denominator_delta", ctypes.c_double), ("denominator_delta_index", ctypes.c_int),
                ("bch_transform_threshold", ctypes.c_double), ("bch_product_threshold", ctypes.c_double)]

    def __init__(self, **kw):
        d = dict(ds=0.1, ds_max=0.5, smax=2.0, norm_domega=0.1, omega_norm_max=2.0, eta_criterion=1e-6,
                 magnus_adaptive=1, generator=0, partitioning=0, denominator_cutoff=1e-6, denominator_delta=0.0,
                 denominator_delta_index=-1, bch_transform_threshold=1e-9, bch_product_threshold=1e-4)
        d.update(kw)
        super().__init__(**d)


def scipy_dgemm_pointer():
    """Address of SciPy's BLAS dgemm (Fortran calling convention), or None."""
    try:
        from scipy.linalg import cython_blas
    except Exception:
        return None
    cap = cython_blas.__pyx_capi__["dgemm"]
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(cap, get_name(cap))


def _dptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iarr(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.int32))


def z_hermiticity(hX, hY):
    if hX * hY == 1:
        return -1
    if hX * hY == -1:
        return 1
    return 0


class Oracle:
    """The reference's scalar IMSRG(2) commutator on the CPU, arena in / out."""

    def __init__(self, emax, A=16, Z=8, use_blas=True):
        self.lib = _load()
        self.ms = ms = RefModelSpace(emax, A, Z)
        kp = [p for c in ms.channels for (p, q) in c[3]]
        kq = [q for c in ms.channels for (p, q) in c[3]]
        cp = [p for c in ms.cc_channels for (p, q) in c[3]]
        cq = [q for c in ms.cc_channels for (p, q) in c[3]]
        self._keep = [_iarr(ms.l), _iarr(ms.j2), _iarr(ms.tz2), np.ascontiguousarray(ms.occ, dtype=np.float64),
                      _iarr([len(c[3]) for c in ms.channels]), _iarr(kp), _iarr(kq),
                      _iarr([len(c[3]) for c in ms.cc_channels]), _iarr(cp), _iarr(cq)]
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        k = self._keep
        self.s = self.lib.oracle_space_create(emax, ms.norb, ip(k[0]), ip(k[1]), ip(k[2]), _dptr(k[3]), ms.nch,
                                              ip(k[4]), ip(k[5]), ip(k[6]), ip(k[7]), ip(k[8]), ip(k[9]))
        assert self.lib.oracle_arena_size(self.s) == ms.arena_size
        if use_blas:
            p = scipy_dgemm_pointer()
            if p:
                self.lib.oracle_set_dgemm(self.s, p)

    def __del__(self):
        try:
            self.lib.oracle_space_destroy(self.s)
        except Exception:
            pass

    @property
    def arena_size(self):
        return self.ms.arena_size

    def zeros(self):
        return np.zeros(self.ms.arena_size)

    def set_term(self, name, on):
        self.lib.oracle_set_term(self.s, TERM_INDEX[name], 1 if on else 0)

    def sixj(self, jj1, jj2, j3, jj4, jj5, j6):
        return self.lib.oracle_sixj(self.s, jj1, jj2, j3, jj4, jj5, j6)

    def term(self, name, X, Y, Z, hX, hY):
        """Accumulate one reference term into Z (the reference's
        comm*ss(X, Y, Z) semantics)."""
        L, s = self.lib, self.s
        hZ = z_hermiticity(hX, hY)
        x, y, z = _dptr(X), _dptr(Y), _dptr(Z)
        if name == "comm110ss":
            L.oracle_comm110ss(s, x, y, z, hX, hY)
        elif name == "comm220ss":
            L.oracle_comm220ss(s, x, y, z, hX, hY)
        elif name == "comm111ss":
            L.oracle_comm111ss(s, x, y, z)
        elif name == "comm121ss":
            L.oracle_comm121ss(s, x, y, z, hZ)
        elif name == "comm122ss":
            L.oracle_comm122ss(s, x, y, z, hZ)
        elif name == "comm222_pp_hh_221ss":
            L.oracle_comm222_pp_hh_221ss(s, x, y, z, hZ, 1, 1)
        elif name == "comm222_pp_hhss":
            L.oracle_comm222_pp_hh_221ss(s, x, y, z, hZ, 1, 0)
        elif name == "comm221ss":
            L.oracle_comm222_pp_hh_221ss(s, x, y, z, hZ, 0, 1)
        elif name == "comm222_phss":
            L.oracle_comm222_phss(s, x, y, z, hY, hZ)
        else:
            raise KeyError(name)

    def commutator(self, X, Y, hX, hY):
        Z = self.zeros()
        self.lib.oracle_commutator(self.s, _dptr(X), _dptr(Y), _dptr(Z), hX, hY)
        return Z

    def norm(self, A):
        return self.lib.oracle_norm(self.s, _dptr(A))

    def bch_transform(self, H, hH, Omega, hOm, threshold=1e-9):
        out = self.zeros()
        it = self.lib.oracle_bch_transform(self.s, _dptr(H), hH, _dptr(Omega), hOm, _dptr(out), threshold)
        return out, it

    def pandya(self, Z, herm, transpose=False):
        """Commutator::DoPandyaTransformation(Z, mats, "normal" / "transpose"):
        one matrix per cross-coupled channel (2nph x ncc, or ncc x 2nph)."""
        out = []
        for ch, cc in enumerate(self.ms.cc_channels):
            ncc = len(cc[3])
            nph = sum(1 for (p, q) in cc[3] if self.ms.ket_class(p, q) in ("hh", "ph"))
            buf = np.zeros(max(1, 2 * nph * ncc))
            self.lib.oracle_pandya_channel(self.s, _dptr(Z), herm, ch, 1 if transpose else 0, _dptr(buf))
            shape = (ncc, 2 * nph) if transpose else (2 * nph, ncc)
            out.append(buf[:2 * nph * ncc].reshape(shape, order="F"))
        return out

    def bch_product(self, X, hX, Y, hY, threshold=1e-4):
        """BCH::BCH_Product(X, Y); returns (Z, commutators evaluated)."""
        Z = self.zeros()
        n = self.lib.oracle_bch_product(self.s, _dptr(X), hX, _dptr(Y), hY, _dptr(Z), threshold)
        return Z, n

    def generator(self, H, kind="white", partitioning="Epstein_Nesbet", cutoff=1e-6, delta=0.0, delta_index=-1):
        """Generator::Update(H, Eta) for a single-reference space."""
        Eta = self.zeros()
        self.lib.oracle_generator(self.s, _dptr(H), _dptr(Eta), GENERATORS[kind], PARTITIONINGS[partitioning],
                                  cutoff, delta, delta_index)
        return Eta

    def magnus_euler(self, H0, params, state=None, maxhist=10000):
        """IMSRGSolver::Solve_magnus_euler from `state` (a dict with s, Hs,
        Hsaved, Omega, n_omega; a fresh IMSRGSolver(H0) if None).  Returns
        the new state plus "steps", "s_hist" and "e0_hist"."""
        if state is None:
            state = dict(s=0.0, Hs=H0.copy(), Hsaved=H0.copy(), Omega=self.zeros(), n_omega=1)
        st = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in state.items()}
        Eta = self.zeros()
        s_io = np.array([st["s"]])
        n_om = ctypes.c_int(st["n_omega"])
        sh = np.zeros(maxhist)
        eh = np.zeros(maxhist)
        steps = self.lib.oracle_magnus_euler(self.s, _dptr(H0), _dptr(st["Hs"]), _dptr(st["Hsaved"]),
                                             _dptr(st["Omega"]), _dptr(Eta), ctypes.byref(params), _dptr(s_io),
                                             ctypes.byref(n_om), _dptr(sh), _dptr(eh), maxhist)
        st.update(s=float(s_io[0]), n_omega=n_om.value, Eta=Eta, steps=steps, s_hist=sh[:max(steps, 0)],
                  e0_hist=eh[:max(steps, 0)])
        return st

    def num_threads(self):
        return self.lib.oracle_num_threads()
