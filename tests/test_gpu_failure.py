"""The failure path of the device waits, made to run without a GPU fault.

* A bounded bulk-copy wait that can never complete (a barrier armed with
  expect_tx and no copy issued) gives up after its poll limit, records the
  timeout in the status word and returns; the context stays usable.
* A timeout recorded in an analysis's status word surfaces from the next
  host evaluation as GWL_ERR_TIMEOUT (TimeoutError in Python), the word is
  cleared, and the evaluation after it succeeds with the same results.
"""
import ctypes

import numpy as np
import pytest

from tests.gpu_helpers import device_analysis, draw_points, params_block, small_workload

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_stays_usable(gpu):
    import torch
    from bilby_gb300 import _capi
    lib = _capi.load()
    status, arrived = ctypes.c_int(-1), ctypes.c_int(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.gwl_selftest_bounded_wait(2000, ctypes.c_void_p(stream), ctypes.byref(status), ctypes.byref(arrived))
    assert rc == _capi.GWL_ERR_TIMEOUT
    assert status.value == 1 and arrived.value == 0
    assert b"bounded device wait" in lib.gwl_last_error()
    with pytest.raises(TimeoutError):
        _capi.check(rc, "selftest")
    x = torch.arange(1000, device="cuda", dtype=torch.float64)
    assert float(x.sum()) == 499500.0


def test_timeout_status_surfaces_once_then_clears(gpu):
    from bilby_gb300 import _capi
    from oracle import data as OD
    w = small_workload("tf2_128s", duration=8.0, sampling_frequency=2048.0,
                       injection=dict(small_workload("tf2_128s").injection, geocent_time=1126259640.0 + 6.0))
    dets = OD.build_workload(w)
    an = device_analysis(dets, "taylorf2", w)
    block = params_block(draw_points(w, 64, np.random.default_rng(3)))
    for precision in ("fp64", "mixed"):
        good = an.log_likelihood_ratio_host(block, precision)
        _capi.check(_capi.load().gwl_inject_device_status(an._h, 1), "inject")
        with pytest.raises(TimeoutError):
            an.log_likelihood_ratio_host(block, precision)
        again = an.log_likelihood_ratio_host(block, precision)
        assert np.array_equal(again, good)
    an.close()
