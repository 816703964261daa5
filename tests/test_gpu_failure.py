"""Failure detection without a GPU fault.

Every device-side wait of the step kernels is bounded: on expiry the kernel
raises the solver's error flag and returns, and the host reports
LBM_ERR_TIMEOUT.  lbm_selftest_bounded_wait makes such a wait run out (an
mbarrier that nothing arrives at, with a 20 ms limit) and the test checks the
status, that the wait really waited, and that the solver stays usable and
exact afterwards.
"""
import time

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

LBM_ERR_TIMEOUT = 11
LBM_ERR_INVALID_ARGUMENT = 1


def test_bounded_wait_times_out_and_solver_stays_usable(gpu, oracle):
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    n = (20, 14, 11)
    _, itau = orc.tau_of(0.0192, np.float32)
    lid = np.float32(0.05)
    want, _ = oracle.run_cavity(*n, np.float32, itau, lid, 24)
    with CLbmSolverGB300(n, itau, lid, storage="f32") as s:
        lib, h = s._lib, s._h
        s.run(10)
        assert lib.lbm_selftest_bounded_wait(h, 0) == LBM_ERR_INVALID_ARGUMENT
        t0 = time.perf_counter()
        assert lib.lbm_selftest_bounded_wait(h, 20000) == LBM_ERR_TIMEOUT
        waited = time.perf_counter() - t0
        assert 0.015 <= waited < 10.0, waited
        assert b"gave up waiting" in lib.lbm_last_error()
        assert lib.lbm_synchronize(h) == 0  # the flag was reported once and cleared
        s.run(14)
        got = s.get_all()
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
