"""Failure detection on the GPU without a GPU fault: every device-side wait
of the library is bounded, and a wait that runs out makes the call return
PA_ERR_TIMEOUT while the device stays usable.  The self-test entry point
runs a onesweep pass whose look-back polls a status word that no tile ever
publishes, with the poll budget lowered so that the wait runs out in about
a millisecond."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PA_OK, PA_ERR_TIMEOUT = 0, 4


@pytest.mark.parametrize("spin_limit", [1, 1000])
def test_lookback_wait_runs_out_and_is_reported(pa, port, spin_limit):
    from parallelalgorithms_gb300 import workloads
    lib = pa.lib()
    assert lib.pa_selftest_wait_expiry(spin_limit) == PA_ERR_TIMEOUT
    assert b"bounded wait" in lib.pa_last_error_message()
    # the error word was cleared and the GPU still answers: a sort afterwards is exact
    a = workloads.uniform_u32(1 << 20)
    got = a.copy()
    pa.SortRadixPar(got, np.empty_like(got), a.size)
    np.testing.assert_array_equal(got, port.sort(a)[0])


def test_selftest_rejects_a_zero_budget(pa):
    assert pa.lib().pa_selftest_wait_expiry(0) == 1
