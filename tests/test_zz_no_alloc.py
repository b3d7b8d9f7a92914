"""imsrg_comm122ss_noalloc: the comm122ss variant for callers that cannot
allocate device memory where they evaluate the term (its W2 intermediate lives
in a static device array, set up when the space's device tables are built).

Through the C ABI, with caller-owned device buffers (torch tensors), on a
fresh model space: two calls in a row must leave the device's free memory
unchanged and give the same result as the regular imsrg_comm122ss (which
allocates its own scratch, so it runs last).  Spaces whose arena exceeds the
static array are refused.  This file is collected last so a failure here
comes after every other test has run."""
import ctypes

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
    # set-up: the space's device tables (with them the no-alloc entry's
    # scratch address), and every caller-owned buffer
    with ig.DeviceOperator(ms, 1):
        pass
    tX = torch.from_numpy(X).cuda()
    tY = torch.from_numpy(Y).cuda()
    tZ = [torch.zeros(ms.arena_size, dtype=torch.float64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for call in range(2):
        rc = L.imsrg_comm122ss_noalloc(ms._h, ctypes.c_void_p(tX.data_ptr()), ctypes.c_void_p(tY.data_ptr()),
                                       ctypes.c_void_p(tZ[call].data_ptr()), 1, None)
        assert rc == _lib.OK, L.imsrg_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    # the regular entry point (library-allocated scratch) on the same inputs
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, ig.DeviceOperator(ms, 1) as dZ:
        dX.upload(X)
        dY.upload(Y)
        ig.Commutator.device_term("comm122ss", dX, dY, dZ)
        ref = dZ.download()
    for call in range(2):
        errs = rel_errors(r, tZ[call].cpu().numpy(), ref)
        assert max(errs) < TOL_FP64, (call, errs)


def test_noalloc_rejects_spaces_beyond_its_array():
    ms = ig.ModelSpace(7, "O16", "O16")  # arena of 2.7M doubles > 2^21
    with ig.DeviceOperator(ms, 1) as dX:
        p = dX.device_ptr()
        L = _lib.lib()
        rc = L.imsrg_comm122ss_noalloc(ms._h, ctypes.c_void_p(p), ctypes.c_void_p(p), ctypes.c_void_p(p), 1, None)
        assert rc == _lib.ERR_ARG
        assert b"too large" in L.imsrg_last_error()
