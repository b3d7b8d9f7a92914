"""Python mirror of the reference's operator / commutator interface on the
GB300 kernels.

Names, argument meaning and error behaviour follow the reference's pybind11
module (src/pyIMSRG.cc:649-706 Commutator, :738-747 BCH) so code written
against pyIMSRG reads the same:

    ms = ModelSpace(6, "O16", "O16")
    X = Operator(ms, 0, 0, 0, 2); X.SetHermitian()
    Y = Operator(ms, 0, 0, 0, 2); Y.SetAntiHermitian()
    Z = Commutator.Commutator(X, Y)            # CommutatorScalarScalar
    Commutator.comm222_phss(X, Y, Z)           # accumulate one term into Z
    Hs = BCH.BCH_Transform(H, Omega)
    solver = IMSRGSolver(H); solver.Solve(); Hs = solver.GetH_s()

Operator keeps its data on the host in the arena layout (numpy); every call
uploads the operands, runs the CUDA kernels and downloads the result.
DeviceOperator keeps an operator resident in HBM for chained device work
(the BCH series, benchmarks).
"""

import ctypes
import os
import re

import numpy as np

from . import _lib
from ._lib import check

_ELEMENTS = ("n H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se "
             "Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho "
             "Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn").split()


def parse_reference(ref):
    """'O16' -> (A=16, Z=8), as ModelSpace::GetAZfromString."""
    m = re.fullmatch(r"([A-Za-z]+)(\d+)", ref.strip())
    if not m:
        raise ValueError("cannot parse reference %r" % ref)
    sym, A = m.group(1), int(m.group(2))
    sym = sym[0].upper() + sym[1:].lower()
    if sym not in _ELEMENTS:
        raise ValueError("unknown element %r" % sym)
    return A, _ELEMENTS.index(sym)


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class ModelSpace:
    """ModelSpace(emax, reference, valence) for a single reference (the
    valence argument must name the same nucleus: no valence space)."""

    def __init__(self, emax, reference="O16", valence=None, orbits=None):
        L = _lib.lib()
        h = ctypes.c_void_p()
        if orbits is not None:
            n, l, j2, tz2, occ = (np.ascontiguousarray(x) for x in orbits)
            n, l, j2, tz2 = (np.asarray(x, dtype=np.int32) for x in (n, l, j2, tz2))
            occ = np.asarray(occ, dtype=np.float64)
            check(L.imsrg_space_create(emax, len(n), _ip(n), _ip(l), _ip(j2), _ip(tz2), _dp(occ), ctypes.byref(h)))
        else:
            if valence is not None and valence != reference:
                raise NotImplementedError("valence spaces are outside the IMSRG(2) commutator scope")
            A, Z = parse_reference(reference)
            check(L.imsrg_space_create_reference(emax, A, Z, ctypes.byref(h)))
        self._h = h
        self._L = L
        self.emax = emax
        norb, nch, arena = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        check(L.imsrg_space_sizes(h, ctypes.byref(norb), ctypes.byref(nch), ctypes.byref(arena)))
        self.norb, self.nch, self.arena_size = norb.value, nch.value, arena.value
        self.orbits = []
        for i in range(self.norb):
            v = [ctypes.c_int() for _ in range(4)]
            o = ctypes.c_double()
            check(L.imsrg_space_orbit(h, i, *[ctypes.byref(x) for x in v], ctypes.byref(o)))
            self.orbits.append((v[0].value, v[1].value, v[2].value, v[3].value, o.value))
        self.channels = []
        for ch in range(self.nch):
            J, par, Tz, nk = (ctypes.c_int() for _ in range(4))
            off = ctypes.c_longlong()
            check(L.imsrg_space_channel(h, ch, ctypes.byref(J), ctypes.byref(par), ctypes.byref(Tz), ctypes.byref(nk),
                                        ctypes.byref(off)))
            p = np.zeros(max(nk.value, 1), dtype=np.int32)
            q = np.zeros(max(nk.value, 1), dtype=np.int32)
            if nk.value:
                check(L.imsrg_space_channel_kets(h, ch, _ip(p), _ip(q)))
            self.channels.append(dict(J=J.value, parity=par.value, Tz=Tz.value, nkets=nk.value, offset=off.value,
                                      kets=list(zip(p[:nk.value].tolist(), q[:nk.value].tolist()))))

    def __del__(self):
        try:
            self._L.imsrg_space_destroy(self._h)
        except Exception:
            pass

    def defer_status(self, on=True):
        """Split-precision commutators and terms on this space return without
        reading the kernels' status word (no stream synchronisation);
        check_status() reads it once for all of them."""
        check(self._L.imsrg_space_defer_status(self._h, 1 if on else 0))

    def check_status(self, stream=None):
        """Synchronise the stream and raise if a kernel reported an error since
        the last read."""
        check(self._L.imsrg_space_check_status(self._h, stream))

    def tuning(self):
        """The space's kernel tuning, {"source": ..., name: value}
        (imsrg_space_describe_tuning)."""
        n = self._L.imsrg_space_describe_tuning(self._h, None, 0)
        buf = ctypes.create_string_buffer(n)
        check(self._L.imsrg_space_describe_tuning(self._h, buf, n))
        out = {}
        for tok in buf.value.decode().split():
            k, v = tok.split("=", 1)
            out[k] = os.path.basename(v) if k == "source" else int(v)
        return out

    def set_tuning(self, name, value):
        check(self._L.imsrg_space_set_tuning(self._h, name.encode(), int(value)))

    def GetNumberOrbits(self):
        return self.norb

    def GetNumberTwoBodyChannels(self):
        return self.nch

    def cc_channel(self, ch):
        J, par, Tz, nk = (ctypes.c_int() for _ in range(4))
        check(self._L.imsrg_space_cc_channel(self._h, ch, ctypes.byref(J), ctypes.byref(par), ctypes.byref(Tz),
                                             ctypes.byref(nk), None, None))
        p = np.zeros(max(nk.value, 1), dtype=np.int32)
        q = np.zeros(max(nk.value, 1), dtype=np.int32)
        check(self._L.imsrg_space_cc_channel(self._h, ch, None, None, None, None, _ip(p), _ip(q)))
        return dict(J=J.value, parity=par.value, Tz=Tz.value, nkets=nk.value,
                    kets=list(zip(p[:nk.value].tolist(), q[:nk.value].tolist())))

    def tensor_layout(self, jrank, trank, parity):
        """{(ch_bra, ch_ket): arena offset} of the two-body blocks of a tensor
        operator of that rank (TwoBodyME::Allocate order)."""
        key = (int(jrank), int(trank), int(parity))
        cache = self.__dict__.setdefault("_tensor_layouts", {})
        if key not in cache:
            nb, tot = ctypes.c_int(), ctypes.c_longlong()
            check(self._L.imsrg_space_tensor_layout(self._h, *key, -1, None, None, None, ctypes.byref(nb),
                                                    ctypes.byref(tot)))
            blocks = {}
            for b in range(nb.value):
                cb, ck, off = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
                check(self._L.imsrg_space_tensor_layout(self._h, *key, b, ctypes.byref(cb), ctypes.byref(ck),
                                                        ctypes.byref(off), None, None))
                blocks[(cb.value, ck.value)] = off.value
            cache[key] = (blocks, tot.value)
        return cache[key][0]

    def tensor_size(self, jrank, trank, parity):
        self.tensor_layout(jrank, trank, parity)
        return self._tensor_layouts[(int(jrank), int(trank), int(parity))][1]

    def GetNineJ(self, ja, jd, J1, jb, jc, J2, Jbra, Jket, lam):
        """{ja jd J1; jb jc J2; Jbra Jket lam} with ja..jd half-integers, the
        other six integers (ModelSpace::GetNineJ argument order)."""
        out = ctypes.c_double()
        check(self._L.imsrg_space_ninej(self._h, int(lam), int(round(2 * ja)), int(round(2 * jd)), int(J1),
                                        int(round(2 * jb)), int(round(2 * jc)), int(J2), int(Jbra), int(Jket),
                                        ctypes.byref(out)))
        return out.value

    def GetSixJ(self, j1, j2, j3, j4, j5, j6):
        """{j1 j2 j3; j4 j5 j6} with j1, j2, j4, j5 half-integer and j3, j6
        integer (ModelSpace::GetCachedSixJ argument convention doubled)."""
        out = ctypes.c_double()
        check(self._L.imsrg_space_sixj(self._h, int(round(2 * j1)), int(round(2 * j2)), int(j3), int(round(2 * j4)),
                                       int(round(2 * j5)), int(j6), ctypes.byref(out)))
        return out.value


class _TwoBody:
    def __init__(self, op):
        self._op = op

    def GetMatrix(self, ch_bra, ch_ket=None):
        ms = self._op.modelspace
        if self._op.rank != (0, 0, 0):
            ch_ket = ch_bra if ch_ket is None else ch_ket
            blocks = ms.tensor_layout(*self._op.rank)
            if (ch_bra, ch_ket) not in blocks:
                raise KeyError("no block (%d, %d) for this tensor rank" % (ch_bra, ch_ket))
            o = blocks[(ch_bra, ch_ket)]
            nb, nk = ms.channels[ch_bra]["nkets"], ms.channels[ch_ket]["nkets"]
            return self._op.arena[o:o + nb * nk].reshape(nb, nk, order="F")
        if ch_ket is not None and ch_ket != ch_bra:
            raise KeyError("scalar operators only store diagonal channel blocks")
        c = ms.channels[ch_bra]
        n, o = c["nkets"], c["offset"]
        return self._op.arena[o:o + n * n].reshape(n, n, order="F")


class Operator:
    """Two-body operator in the arena layout, host resident:
    Operator(ms, 0, 0, 0, 2) a scalar (J=0, parity +, Tz=0), Operator(ms,
    jrank, trank, parity, 2) a reduced tensor (tensor arena of that rank)."""

    def __init__(self, ms, jrank=0, trank=0, parity=0, particle_rank=2, arena=None, hermitian=True):
        if particle_rank != 2:
            raise NotImplementedError("only particle-rank-2 operators are on the GPU path")
        self.modelspace = ms
        self.rank = (int(jrank), int(trank), int(parity))
        size = ms.arena_size if self.rank == (0, 0, 0) else ms.tensor_size(*self.rank)
        self.arena = np.zeros(size) if arena is None else np.ascontiguousarray(arena, dtype=np.float64)
        if self.arena.shape != (size,):
            raise ValueError("arena has the wrong length")
        self.hermitian = 1 if hermitian else -1
        self.TwoBody = _TwoBody(self)

    def GetJRank(self):
        return self.rank[0]

    def GetTRank(self):
        return self.rank[1]

    def GetParity(self):
        return self.rank[2]

    # hermiticity
    def SetHermitian(self):
        self.hermitian = 1

    def SetAntiHermitian(self):
        self.hermitian = -1

    def IsHermitian(self):
        return self.hermitian == 1

    def IsAntiHermitian(self):
        return self.hermitian == -1

    @property
    def ZeroBody(self):
        return float(self.arena[0])

    @ZeroBody.setter
    def ZeroBody(self, v):
        self.arena[0] = v

    @property
    def OneBody(self):
        N = self.modelspace.norb
        return self.arena[32:32 + N * N].reshape(N, N, order="F")

    def copy(self):
        return Operator(self.modelspace, *self.rank, arena=self.arena.copy(), hermitian=self.hermitian == 1)

    def Erase(self):
        self.arena[:] = 0

    def Norm(self):
        with DeviceOperator.from_host(self) as d:
            return d.norm()

    def WriteBinary(self, path):
        """Operator::WriteBinary to a file path."""
        with DeviceOperator.from_host(self) as d:
            d.write_binary(path)

    def ReadBinary(self, path):
        """Operator::ReadBinary from a file path (hermiticity from the file)."""
        with DeviceOperator(self.modelspace, self.hermitian, getattr(self, "rank", (0, 0, 0))) as d:
            d.read_binary(path)
            d.download(self.arena)
            self.hermitian = d.hermiticity

    def __iadd__(self, other):
        self.arena += other.arena
        return self

    def __isub__(self, other):
        self.arena -= other.arena
        return self

    def __imul__(self, a):
        self.arena *= a
        return self

    def __mul__(self, a):
        out = self.copy()
        out.arena *= a
        return out

    __rmul__ = __mul__


class DeviceOperator:
    """Operator resident in device memory (imsrg_op)."""

    def __init__(self, ms, hermiticity=1, rank=(0, 0, 0)):
        self.modelspace = ms
        self._L = _lib.lib()
        self._owned = True
        self._h = ctypes.c_void_p()
        self.rank = tuple(int(x) for x in rank)
        if self.rank == (0, 0, 0):
            check(self._L.imsrg_op_create(ms._h, int(hermiticity), ctypes.byref(self._h)))
            self.size = ms.arena_size
        else:
            check(self._L.imsrg_op_create_tensor(ms._h, *self.rank, int(hermiticity), ctypes.byref(self._h)))
            self.size = ms.tensor_size(*self.rank)

    @classmethod
    def _view(cls, ms, handle, owner, rank=(0, 0, 0)):
        """An operator owned by another object (a solver's H(s), Eta, Omega,
        added operators)."""
        d = cls.__new__(cls)
        d.modelspace = ms
        d._L = _lib.lib()
        d._owned = False
        d._owner = owner
        d._h = handle
        d.rank = tuple(int(x) for x in rank)
        d.size = ms.arena_size if d.rank == (0, 0, 0) else ms.tensor_size(*d.rank)
        return d

    @classmethod
    def from_host(cls, op, stream=None):
        d = cls(op.modelspace, op.hermitian, getattr(op, "rank", (0, 0, 0)))
        d.upload(op.arena, stream)
        return d

    def close(self):
        if self._h and self._owned:
            self._L.imsrg_op_destroy(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def hermiticity(self):
        h = ctypes.c_int()
        check(self._L.imsrg_op_hermiticity(self._h, ctypes.byref(h)))
        return h.value

    @hermiticity.setter
    def hermiticity(self, h):
        check(self._L.imsrg_op_set_hermiticity(self._h, int(h)))

    def upload(self, arena, stream=None):
        a = np.ascontiguousarray(arena, dtype=np.float64)
        assert a.shape == (self.size,)
        check(self._L.imsrg_op_upload(self._h, _dp(a), stream))
        if stream is not None:
            self._keep = a

    def upload_ptr(self, host_ptr, stream=None):
        """Copy the arena from a host address (e.g. pinned memory)."""
        check(self._L.imsrg_op_upload(self._h, ctypes.cast(host_ptr, ctypes.POINTER(ctypes.c_double)), stream))

    def download_ptr(self, host_ptr, stream=None):
        """Copy the arena to a host address; synchronises the stream."""
        check(self._L.imsrg_op_download(self._h, ctypes.cast(host_ptr, ctypes.POINTER(ctypes.c_double)), stream))

    def download(self, out=None, stream=None):
        if out is None:
            out = np.empty(self.size)
        check(self._L.imsrg_op_download(self._h, _dp(out), stream))
        return out

    def to_host(self):
        return Operator(self.modelspace, *self.rank, arena=self.download(), hermitian=self.hermiticity == 1)

    def device_ptr(self):
        p = ctypes.c_void_p()
        check(self._L.imsrg_op_device_arena(self._h, ctypes.byref(p)))
        return p.value

    def zero(self, stream=None):
        check(self._L.imsrg_op_zero(self._h, stream))

    def copy_from(self, other, stream=None):
        check(self._L.imsrg_op_copy(self._h, other._h, stream))

    def scale(self, a, stream=None):
        check(self._L.imsrg_op_scale(self._h, float(a), stream))

    def axpy(self, a, x, stream=None):
        check(self._L.imsrg_op_axpy(self._h, float(a), x._h, stream))

    def norm(self, stream=None):
        out = ctypes.c_double()
        check(self._L.imsrg_op_norm(self._h, ctypes.byref(out), stream))
        return out.value

    def fill_random(self, seed, stream=None):
        check(self._L.imsrg_op_fill_random(self._h, int(seed), stream))

    def write_binary(self, path, stream=None):
        """Operator::WriteBinary layout (files interchange with IMSRG++)."""
        check(self._L.imsrg_op_write_binary(self._h, os.fsencode(path), stream))

    def read_binary(self, path, stream=None):
        """Operator::ReadBinary; hermiticity taken from the file."""
        check(self._L.imsrg_op_read_binary(self._h, os.fsencode(path), stream))


def _precision(p):
    if p is None:
        v = ctypes.c_int()
        check(_lib.lib().imsrg_get_default_precision(ctypes.byref(v)))
        return v.value
    if isinstance(p, str):
        return {"fp64": _lib.PREC_FP64, "split": _lib.PREC_SPLIT}[p.lower()]
    return int(p)


class _CommutatorNamespace:
    """Commutator:: free functions (src/Commutator.hh:57-87)."""

    _TERMS_3 = ("comm110ss", "comm220ss", "comm111ss", "comm121ss", "comm122ss", "comm221ss")
    _TERMS_P = ("comm222_pp_hhss", "comm222_pp_hh_221ss", "comm222_phss")
    _TERMS_ST = ("comm111st", "comm121st", "comm122st", "comm222_pp_hh_221st", "comm222_phst")

    def TurnOnTerm(self, name):
        check(_lib.lib().imsrg_set_term(name.encode(), 1))

    def TurnOffTerm(self, name):
        check(_lib.lib().imsrg_set_term(name.encode(), 0))

    def IsTermOn(self, name):
        v = ctypes.c_int()
        check(_lib.lib().imsrg_get_term(name.encode(), ctypes.byref(v)))
        return bool(v.value)

    def SetPrecision(self, p):
        check(_lib.lib().imsrg_set_default_precision(_precision(p)))

    def GetPrecision(self):
        return _precision(None)

    def _run_term(self, name, X, Y, Z, precision=None):
        L = _lib.lib()
        with DeviceOperator.from_host(X) as dx, DeviceOperator.from_host(Y) as dy, \
                DeviceOperator.from_host(Z) as dz:
            fn = getattr(L, "imsrg_" + name)
            if name in self._TERMS_P:
                check(fn(dx._h, dy._h, dz._h, _precision(precision), None))
            else:
                check(fn(dx._h, dy._h, dz._h, None))
            dz.download(Z.arena)

    def CommutatorScalarScalar(self, X, Y, precision=None):
        ms = X.modelspace
        Z = Operator(ms)
        with DeviceOperator.from_host(X) as dx, DeviceOperator.from_host(Y) as dy, DeviceOperator(ms) as dz:
            check(_lib.lib().imsrg_commutator_scalar_scalar(dx._h, dy._h, dz._h, _precision(precision), None))
            dz.download(Z.arena)
            Z.hermitian = dz.hermiticity
        return Z

    def CommutatorScalarTensor(self, X, Y, precision=None):
        """Commutator::CommutatorScalarTensor(X, Y): X scalar, Y a reduced tensor."""
        ms = X.modelspace
        Z = Operator(ms, *Y.rank)
        with DeviceOperator.from_host(X) as dx, DeviceOperator.from_host(Y) as dy, \
                DeviceOperator(ms, 1, Y.rank) as dz:
            self.device_scalar_tensor(dx, dy, dz, precision)
            dz.download(Z.arena)
            Z.hermitian = dz.hermiticity
        return Z

    def device_scalar_tensor(self, dX, dY, dZ, precision=None, stream=None):
        check(_lib.lib().imsrg_commutator_scalar_tensor(dX._h, dY._h, dZ._h, _precision(precision), stream))

    _TERMS_STP = ("comm222_pp_hh_221st", "comm222_phst")

    def device_tensor_term(self, name, dX, dY, dZ, precision=None, stream=None):
        """One scalar-tensor term (comm111st, comm121st, comm122st,
        comm222_pp_hh_221st, comm222_phst) accumulated into dZ; precision
        applies to the two with products."""
        if name not in self._TERMS_ST:
            raise KeyError(name)
        fn = getattr(_lib.lib(), "imsrg_" + name)
        if name in self._TERMS_STP:
            check(fn(dX._h, dY._h, dZ._h, _precision(precision), stream))
        else:
            check(fn(dX._h, dY._h, dZ._h, stream))

    def Commutator(self, X, Y, precision=None):
        """Commutator::Commutator: dispatch on the tensor ranks
        (src/Commutator.cc:182-276)."""
        rx, ry = getattr(X, "rank", (0, 0, 0)), getattr(Y, "rank", (0, 0, 0))
        if rx == (0, 0, 0) and ry == (0, 0, 0):
            return self.CommutatorScalarScalar(X, Y, precision)
        if rx == (0, 0, 0):
            return self.CommutatorScalarTensor(X, Y, precision)
        if ry == (0, 0, 0):
            Z = self.CommutatorScalarTensor(Y, X, precision)  # [T, S] = -[S, T]
            Z.arena *= -1
            return Z
        raise NotImplementedError("tensor-tensor commutators are not implemented in the reference either")

    def pandya_layout(self, ms):
        """[(rows, cols, offset)] per cross-coupled channel and the buffer length."""
        L = _lib.lib()
        total = ctypes.c_longlong()
        check(L.imsrg_space_pandya_layout(ms._h, -1, None, None, None, ctypes.byref(total)))
        out = []
        for ch in range(ms.nch):
            r, c, o = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
            check(L.imsrg_space_pandya_layout(ms._h, ch, ctypes.byref(r), ctypes.byref(c), ctypes.byref(o), None))
            out.append((r.value, c.value, o.value))
        return out, total.value

    def device_pandya(self, dZ, out_ptr, orientation="normal", stream=None):
        """Pandya transform of a device operator into a device buffer (layout:
        pandya_layout)."""
        if orientation not in ("normal", "transpose"):
            raise ValueError("unknown orientation %r" % orientation)
        check(_lib.lib().imsrg_pandya_transform(dZ._h, 1 if orientation == "transpose" else 0,
                                                ctypes.c_void_p(out_ptr), stream))

    def DoPandyaTransformation(self, Z, orientation="normal"):
        """Commutator::DoPandyaTransformation(Z, TwoBody_CC_ph, orientation):
        one matrix per cross-coupled channel, 2nph x ncc ("normal") or
        ncc x 2nph times herm (n_a - n_b) ("transpose")."""
        import torch
        ms = Z.modelspace
        layout, total = self.pandya_layout(ms)
        buf = torch.empty(total, dtype=torch.float64, device="cuda")
        with DeviceOperator.from_host(Z) as dz:
            self.device_pandya(dz, buf.data_ptr(), orientation)
            host = buf.cpu().numpy()
        mats = []
        for rows, cols, off in layout:
            shape = (rows, cols) if orientation == "normal" else (cols, rows)
            mats.append(host[off:off + rows * cols].reshape(shape, order="F").copy())
        return mats

    def device_commutator(self, dX, dY, dZ, precision=None, stream=None):
        """[X,Y] on device-resident operators (Z overwritten)."""
        check(_lib.lib().imsrg_commutator_scalar_scalar(dX._h, dY._h, dZ._h, _precision(precision), stream))

    def device_term(self, name, dX, dY, dZ, precision=None, stream=None):
        fn = getattr(_lib.lib(), "imsrg_" + name)
        if name in self._TERMS_P:
            check(fn(dX._h, dY._h, dZ._h, _precision(precision), stream))
        else:
            check(fn(dX._h, dY._h, dZ._h, stream))


class CommutatorBatch:
    """Many independent commutators Z_i = [X_i, Y_i] (device operators of any
    mix of model spaces) captured once into a CUDA graph and replayed by
    launch(); pairs of different spaces run concurrently.  The operators must
    stay alive and in place while the batch exists (the batch keeps references)."""

    def __init__(self, pairs, precision=None):
        self._L = _lib.lib()
        self.pairs = list(pairs)
        n = len(self.pairs)
        arr = [(ctypes.c_void_p * n)(*[p[k]._h.value for p in self.pairs]) for k in range(3)]
        self._h = ctypes.c_void_p()
        check(self._L.imsrg_batch_create(n, arr[0], arr[1], arr[2], _precision(precision), ctypes.byref(self._h)))

    def launch(self, stream=None):
        check(self._L.imsrg_batch_launch(self._h, stream))

    def sync(self, stream=None):
        check(self._L.imsrg_batch_sync(self._h, stream))

    def info(self):
        """(pairs, graph branches, grouped product launches per product
        family (0: products per pair), kernel nodes per replay)"""
        a, b, g, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        check(self._L.imsrg_batch_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(g), ctypes.byref(c)))
        return a.value, b.value, g.value, c.value

    def close(self):
        if getattr(self, "_h", None):
            self._L.imsrg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _make_term(name):
    def f(self, X, Y, Z, precision=None):
        self._run_term(name, X, Y, Z, precision)
    f.__name__ = name
    f.__doc__ = "Commutator::%s(X, Y, Z): accumulate the term into Z." % name
    return f


for _n in _CommutatorNamespace._TERMS_3 + _CommutatorNamespace._TERMS_P:
    setattr(_CommutatorNamespace, _n, _make_term(_n))

Commutator = _CommutatorNamespace()


class _BCHNamespace:
    """BCH:: free functions (src/BCH.hh:22-25)."""

    def __init__(self):
        self.bch_transform_threshold = 1e-9
        self.bch_product_threshold = 1e-4

    def Set_BCH_Transform_Threshold(self, x):
        self.bch_transform_threshold = float(x)

    def Set_BCH_Product_Threshold(self, x):
        self.bch_product_threshold = float(x)

    def BCH_Product(self, X, Y, precision=None):
        """Z with e^Z = e^X e^Y (src/BCH.cc:267-350)."""
        ms = X.modelspace
        out = Operator(ms)
        with DeviceOperator.from_host(X) as dx, DeviceOperator.from_host(Y) as dy, DeviceOperator(ms) as dz:
            self.last_n_commutators = self.device_product(dx, dy, dz, precision)
            dz.download(out.arena)
            out.hermitian = dz.hermiticity
        return out

    def device_product(self, dX, dY, dZ, precision=None, stream=None):
        """BCH_Product on device operators; dZ may be dX or dY.  Returns the
        number of commutators evaluated."""
        n = ctypes.c_int()
        check(_lib.lib().imsrg_bch_product(dX._h, dY._h, dZ._h, self.bch_product_threshold, _precision(precision),
                                           ctypes.byref(n), stream))
        return n.value

    def BCH_Transform(self, OpIn, Omega, precision=None):
        """BCH::BCH_Transform(OpIn, Omega): OpIn scalar or a reduced tensor,
        Omega scalar."""
        ms = OpIn.modelspace
        rank = getattr(OpIn, "rank", (0, 0, 0))
        out = Operator(ms, *rank) if rank != (0, 0, 0) else Operator(ms)
        with DeviceOperator.from_host(OpIn) as di, DeviceOperator.from_host(Omega) as dom, \
                DeviceOperator(ms, 1, rank) as do:
            self.last_n_nested = self.device_transform(di, dom, do, precision)
            do.download(out.arena)
            out.hermitian = do.hermiticity
        return out

    def device_transform(self, dIn, dOmega, dOut, precision=None, stream=None):
        n = ctypes.c_int()
        check(_lib.lib().imsrg_bch_transform(dIn._h, dOmega._h, dOut._h, self.bch_transform_threshold,
                                             _precision(precision), ctypes.byref(n), stream))
        return n.value


BCH = _BCHNamespace()


_GENERATOR_TYPES = {"white": 0, "atan": 1, "wegner": 2, "imaginary-time": 3, "qtransfer-atan": 101}
_GENERATOR_TYPES.update({"qtransfer-atan_%d" % n: 100 + n for n in range(1, 17)})
DELTA_ALL = -12345


class Generator:
    """Generator (src/Generator.hh:21-90) for the single-reference types
    white, atan, wegner and imaginary-time; Epstein-Nesbet (default) or
    Moller-Plesset denominators."""

    def __init__(self):
        self.generator_type = "white"
        self.denominator_partitioning = "Epstein_Nesbet"
        self.denominator_cutoff = 1e-6
        self.denominator_delta = 0.0
        self.denominator_delta_index = -1

    def SetType(self, g):
        if g not in _GENERATOR_TYPES:
            raise NotImplementedError("generator type %r is not on the GPU path" % g)
        self.generator_type = g

    def GetType(self):
        return self.generator_type

    def SetDenominatorPartitioning(self, dp):
        if dp == "MP_isospin":
            raise NotImplementedError("MP_isospin partitioning is not on the GPU path")
        self.denominator_partitioning = "Moller_Plesset" if dp == "Moller_Plesset" else "Epstein_Nesbet"

    def SetDenominatorCutoff(self, c):
        self.denominator_cutoff = float(c)

    def SetDenominatorDelta(self, d):
        self.denominator_delta = float(d)

    def SetDenominatorDeltaIndex(self, i):
        self.denominator_delta_index = int(i)

    def device_update(self, dH, dEta, stream=None):
        part = 1 if self.denominator_partitioning == "Moller_Plesset" else 0
        check(_lib.lib().imsrg_generator_update(dH._h, dEta._h, _GENERATOR_TYPES[self.generator_type], part,
                                                self.denominator_cutoff, self.denominator_delta,
                                                self.denominator_delta_index, stream))

    def Update(self, H, Eta):
        """Generator::Update(H_s, Eta_s): Eta overwritten (anti-hermitian)."""
        with DeviceOperator.from_host(H) as dh, DeviceOperator(H.modelspace, -1) as de:
            self.device_update(dh, de)
            de.download(Eta.arena)
        Eta.hermitian = -1


class IMSRGSolver:
    """IMSRGSolver (src/IMSRGSolver.hh:35-210) with the Magnus-Euler method,
    every operator resident on the device.  H may be a host Operator (copied to
    the device) or a DeviceOperator (used in place; it must not change while
    the solver lives)."""

    def __init__(self, H, precision=None):
        ms = H.modelspace
        self.modelspace = ms
        self._L = _lib.lib()
        self._H0 = H if isinstance(H, DeviceOperator) else DeviceOperator.from_host(H)
        self._h = ctypes.c_void_p()
        check(self._L.imsrg_solver_create(self._H0._h, ctypes.byref(self._h)))
        self.precision = precision
        self.method = "magnus_euler"

    def close(self):
        if getattr(self, "_h", None):
            self._L.imsrg_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _set(self, name, v):
        check(self._L.imsrg_solver_set(self._h, name.encode(), float(v)))

    def _get(self, name):
        v = ctypes.c_double()
        check(self._L.imsrg_solver_get(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    # settings (pyIMSRG names, src/pyIMSRG.cc:539-595)
    def SetDs(self, d):
        self._set("ds", d)

    def SetDsmax(self, d):
        self._set("ds_max", d)

    def SetSmax(self, d):
        self._set("smax", d)

    def SetdOmega(self, d):
        self._set("domega", d)

    def SetOmegaNormMax(self, x):
        self._set("omega_norm_max", x)

    def SetEtaCriterion(self, x):
        self._set("eta_criterion", x)

    def SetMagnusAdaptive(self, b=True):
        self._set("magnus_adaptive", 1 if b else 0)

    def SetHunterGatherer(self, b=True):
        self._set("hunter_gatherer", 1 if b else 0)

    _METHODS = {"magnus_euler": 0, "magnus": 0, "magnus_modified_euler": 1, "magnus_backoff": 2, "flow_RK4": 3}

    def SetMethod(self, m):
        """IMSRGSolver::SetMethod: magnus_euler (magnus), magnus_modified_euler,
        magnus_backoff or flow_RK4 (fixed RK4 steps of ds_max on H(s), no
        Omega); the boost::odeint methods (flow, flow_adaptive, flow_euler,
        magnus_adaptive, restore_4th_order) are not on the GPU path."""
        if m not in self._METHODS:
            raise _lib.IMSRGError(_lib.ERR_UNSUPPORTED, "method %s is not on the GPU path" % m)
        self._set("method", self._METHODS[m])
        self.method = m

    def SetDenominatorCutoff(self, c):
        self._set("denominator_cutoff", c)

    def SetDenominatorDelta(self, d):
        self._set("denominator_delta", d)

    def SetDenominatorDeltaIndex(self, i):
        self._set("denominator_delta_index", i)

    def SetScratchDir(self, d):
        check(self._L.imsrg_solver_set_scratch_dir(self._h, os.fsencode(d)))

    def GetNOmegaWritten(self):
        return int(self._get("n_omega_written"))

    def SetGenerator(self, g, stream=None):
        check(self._L.imsrg_solver_set_generator(self._h, g.encode(), stream))

    def SetDenominatorPartitioning(self, dp):
        check(self._L.imsrg_solver_set_denominator_partitioning(self._h, dp.encode()))

    def SetBCHTransformThreshold(self, x):
        self._set("bch_transform_threshold", x)

    def SetBCHProductThreshold(self, x):
        self._set("bch_product_threshold", x)

    # flow
    def Solve(self, stream=None):
        check(self._L.imsrg_solver_solve(self._h, _precision(self.precision), stream))

    def GetS(self):
        return self._get("s")

    def GetOmegaSize(self):
        return int(self._get("n_omega"))

    def device_hs(self):
        h = ctypes.c_void_p()
        check(self._L.imsrg_solver_hs(self._h, ctypes.byref(h)))
        return DeviceOperator._view(self.modelspace, h, self)

    def device_eta(self):
        h = ctypes.c_void_p()
        check(self._L.imsrg_solver_eta(self._h, ctypes.byref(h)))
        return DeviceOperator._view(self.modelspace, h, self)

    def device_omega(self, i):
        h = ctypes.c_void_p()
        check(self._L.imsrg_solver_omega(self._h, int(i), ctypes.byref(h)))
        return DeviceOperator._view(self.modelspace, h, self)

    def AddOperator(self, op):
        """IMSRGSolver::AddOperator: a copy of op (scalar or reduced tensor)
        joins the flowing operators (flow_RK4 flows it with H(s)); returns
        its index for GetOperator."""
        rank = getattr(op, "rank", (0, 0, 0))
        idx = ctypes.c_int()
        with DeviceOperator.from_host(op) as d:
            check(self._L.imsrg_solver_add_operator(self._h, d._h, ctypes.byref(idx), None))
        self._ranks = getattr(self, "_ranks", [(0, 0, 0)]) + [tuple(rank)]
        return idx.value

    def device_operator(self, i):
        h = ctypes.c_void_p()
        check(self._L.imsrg_solver_get_operator(self._h, int(i), ctypes.byref(h)))
        ranks = getattr(self, "_ranks", [(0, 0, 0)])
        return DeviceOperator._view(self.modelspace, h, self, ranks[i] if 0 <= i < len(ranks) else (0, 0, 0))

    def GetOperator(self, i):
        """IMSRGSolver::GetOperator: flowing operator i (0 is H(s))."""
        return self.device_operator(i).to_host()

    def GetH_s(self):
        return self.device_hs().to_host()

    def GetEta(self):
        return self.device_eta().to_host()

    def GetOmega(self, i):
        return self.device_omega(i).to_host()

    def history(self):
        """Per step: (istep, s, E0, |eta|, |Omega|) arrays."""
        n = ctypes.c_int()
        check(self._L.imsrg_solver_history(self._h, 0, None, None, None, None, None, ctypes.byref(n)))
        m = n.value
        it = np.zeros(max(m, 1), dtype=np.int32)
        cols = [np.zeros(max(m, 1)) for _ in range(4)]
        check(self._L.imsrg_solver_history(self._h, m, _ip(it), *[_dp(c) for c in cols], ctypes.byref(n)))
        return it[:m], cols[0][:m], cols[1][:m], cols[2][:m], cols[3][:m]

    def _transform(self, fn, op):
        # scalar operators or reduced tensors (observables) alike
        rank = getattr(op, "rank", (0, 0, 0))
        out = Operator(op.modelspace, *rank) if rank != (0, 0, 0) else Operator(op.modelspace)
        with DeviceOperator.from_host(op) as di, DeviceOperator(op.modelspace, op.hermitian, rank) as do:
            check(fn(self._h, di._h, do._h, _precision(self.precision), None))
            do.download(out.arena)
            out.hermitian = do.hermiticity
        return out

    def Transform(self, op):
        """IMSRGSolver::Transform: e^Omega op e^-Omega through every Omega."""
        return self._transform(self._L.imsrg_solver_transform, op)

    def InverseTransform(self, op):
        return self._transform(self._L.imsrg_solver_inverse_transform, op)
