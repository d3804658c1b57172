"""Failure detection without a GPU fault: the streaming kernels' bounded
mbarrier wait, run on a barrier that nothing completes, must give up, report
WAVE_ERR_TIMEOUT through the device error word and leave the context usable
(a simulation afterwards still matches the FP64 oracle)."""
import ctypes

import numpy as np
import pytest

from test_gpu_parity import TOL, make_case, rel, run_both

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives(wave, refcpu):
    status = ctypes.c_int(0)
    assert wave.lib().wave_selftest_bounded_wait(ctypes.byref(status)) == wave.WAVE_OK
    assert status.value == wave.WAVE_ERR_TIMEOUT
    gpu, ref = run_both(wave, refcpu, make_case(refcpu, "acoustic", 2, 4, 0, 2))
    assert rel(gpu, ref) < TOL
