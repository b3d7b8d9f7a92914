"""imsrg_comm122ss_noalloc: the comm122ss variant for callers that cannot
allocate device memory (its W2 intermediate lives in a static device array).

Through the C ABI, with caller-owned device buffers (torch tensors), it must
give the same result as the regular imsrg_comm122ss, call after call, and
refuse spaces whose arena exceeds its static array.  This file is collected
last so a failure here comes after every other test has run."""
import ctypes

import numpy as np
import pytest

import imsrg_gb300 as ig
from imsrg_gb300 import _lib
from helpers import rel_errors, ref_space

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    emax = 5
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    X = r.random_operator(71, True)
    Y = r.random_operator(72, False)
    L = _lib.lib()
    # regular entry point (library-allocated scratch)
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.upload(X)
        dY.upload(Y)
        ig.Commutator.device_term("comm122ss", dX, dY, dZ)
        ref = dZ.download()
    # caller-owned device buffers
    tX = torch.from_numpy(X).cuda()
    tY = torch.from_numpy(Y).cuda()
    for call in range(2):
        tZ = torch.zeros(ms.arena_size, dtype=torch.float64, device="cuda")
        rc = L.imsrg_comm122ss_noalloc(ms._h, ctypes.c_void_p(tX.data_ptr()), ctypes.c_void_p(tY.data_ptr()),
                                       ctypes.c_void_p(tZ.data_ptr()), 1, None)
        assert rc == _lib.OK, L.imsrg_last_error()
        torch.cuda.synchronize()
        Z = tZ.cpu().numpy()
        errs = rel_errors(r, Z, ref)
        assert max(errs) < TOL_FP64, (call, errs)


def test_noalloc_rejects_spaces_beyond_its_array():
    ms = ig.ModelSpace(7, "O16", "O16")  # arena of 2.7M doubles > 2^21
    with ig.DeviceOperator(ms, 1) as dX:
        p = dX.device_ptr()
        L = _lib.lib()
        rc = L.imsrg_comm122ss_noalloc(ms._h, ctypes.c_void_p(p), ctypes.c_void_p(p), ctypes.c_void_p(p), 1, None)
        assert rc == _lib.ERR_ARG
        assert b"too large" in L.imsrg_last_error()
