"""The allocation-free entry point ``gwl_eval_device_noalloc``.

It exists for callers that cannot let a library call cudaMalloc -- a host
application that has reserved the GPU's memory for its own pool allocator,
or a sampler loop where cudaMalloc's device-wide synchronisation is not
acceptable.  Its work space is a static device buffer inside the library.
These tests call it through the C ABI and check it against the ordinary
entry point ``gwl_eval_device`` (same mixed-precision tolerance as the other
tests, |dlnL| <= 1e-3) on two calls in a row, and check that a batch too large
for the static buffer is refused with a clear error.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_ATOL = 1e-3


@pytest.fixture(scope="module")
def analysis(gpu):
    from dataclasses import replace
    from bilby_gb300.analysis import Analysis, DetectorData
    from bilby_gb300.workloads import WORKLOADS
    from oracle import data as OD
    base = WORKLOADS["tf2_128s"]
    w = replace(base, sampling_frequency=2048.0, duration=8.0,
                injection=dict(base.injection, geocent_time=base.start_time + 6.0))
    dets = OD.build_workload(w)
    an = Analysis("taylorf2", dets[0].frequency,
                  [DetectorData(d.name, d.vertex, d.tensor, d.start_time, d.masked_strain, d.psd, d.mask)
                   for d in dets], w.duration, w.sampling_frequency, w.minimum_frequency)
    return w, an


def noalloc(an, block, out, stream):
    from bilby_gb300 import _capi
    return _capi.load().gwl_eval_device_noalloc(an._h, ctypes.c_void_p(block.data_ptr()), block.shape[1],
                                                ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))


def test_matches_the_allocating_entry_point_twice(analysis):
    import torch
    from bilby_gb300 import _capi
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    w, an = analysis
    stream = torch.cuda.current_stream().cuda_stream
    for call, (n, seed) in enumerate(((777, 1), (300, 2))):
        block = torch.from_numpy(params_block(draw_points(w, n, np.random.default_rng(seed)))).cuda()
        got = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
        ref = torch.empty(n, dtype=torch.float64, device="cuda")
        _capi.check(noalloc(an, block, got, stream), "gwl_eval_device_noalloc")
        an.log_likelihood_ratio_device(block.data_ptr(), n, ref.data_ptr(), "mixed", stream)
        torch.cuda.synchronize()
        g, r = got.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(g)), call
        assert np.max(np.abs(g - r)) <= MIXED_ATOL, (call, np.max(np.abs(g - r)))


def test_refuses_a_batch_beyond_the_static_buffer(analysis):
    import torch
    from bilby_gb300 import _capi
    w, an = analysis
    n = 100_000
    block = torch.zeros((_capi.NPARAM, n), dtype=torch.float64, device="cuda")
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    status = noalloc(an, block, out, torch.cuda.current_stream().cuda_stream)
    assert status == _capi.GWL_ERR_ARGUMENT
    assert b"static buffer" in _capi.load().gwl_last_error()
    torch.cuda.synchronize()
    assert float(out.abs().sum()) == 0.0  # nothing ran
