"""Failure path of the bounded waits in the split products, on the GPU
without a fault: a kernel waits on an mbarrier that nothing arrives on,
through the products' own wait loop with a short bound, gives up, sets the
space's status word and returns; the host reports IMSRG_ERR_KERNEL and clears
the word, and the same context then evaluates a split commutator that matches
the FP64 one.  The wait's measured length also bounds the production wait."""
import ctypes
import time

import numpy as np
import pytest

import imsrg_gb300 as ig
from imsrg_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_and_context_survives():
    ms = ig.ModelSpace(4, "O16", "O16")
    L = ig.lib()
    cyc = ctypes.c_longlong()
    prod = ctypes.c_uint()
    limit = 1 << 14
    with ig.DeviceOperator(ms, 1) as dX, ig.DeviceOperator(ms, -1) as dY, \
            ig.DeviceOperator(ms, 1) as dZ, ig.DeviceOperator(ms, 1) as dF:
        dX.fill_random(3)
        dY.fill_random(4)
        t0 = time.time()
        rc = L.imsrg_space_wait_selftest(ms._h, limit, ctypes.byref(cyc), ctypes.byref(prod), None)
        dt = time.time() - t0
        assert rc == _lib.ERR_KERNEL
        assert b"105" in L.imsrg_last_error()
        assert cyc.value > limit  # it waited through every iteration
        assert dt < 10.0
        # the production bound, extrapolated from this wait's cycles at the
        # maximum SM clock (2.07 GHz), ends within a few seconds
        est_s = cyc.value / limit * prod.value / 2.07e9
        print("wait: %d cycles for %d iterations; production bound %d iterations ~ %.2f s"
              % (cyc.value, limit, prod.value, est_s))
        assert 0.1 < est_s < 5.0
        # the status word was cleared: a second run reports once more, and the
        # split commutator runs clean afterwards
        assert L.imsrg_space_wait_selftest(ms._h, 64, None, None, None) == _lib.ERR_KERNEL
        ig.Commutator.device_commutator(dX, dY, dZ, "split")
        ig.Commutator.device_commutator(dX, dY, dF, "fp64")
        z, f = dZ.download(), dF.download()
        assert np.linalg.norm(z - f) <= 1e-10 * np.linalg.norm(f)
