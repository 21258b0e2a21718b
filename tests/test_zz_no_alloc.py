"""The allocation-free entry point ``gwl_eval_device_noalloc``.

It exists for callers that cannot let a library call cudaMalloc -- a host
application that has reserved the GPU's memory for its own pool allocator,
or a sampler loop where cudaMalloc's device-wide synchronisation is not
acceptable.  Its work space is a static device buffer inside the library.
These tests call it through the C ABI and check it against the ordinary
entry point ``gwl_eval_device`` on two calls in a row.  Both run the same
kernels with the same split-K layout and summation order, so the results are
bit-identical (which is stricter than the mixed-precision tolerance of the
other tests, |dlnL| <= 1e-3).  They also check that a call on a fresh analysis
changes the device's free memory by nothing, that points marked for the
accurate kernel take it on this path too, that the status word reads back
clear, and that a batch too large for the static buffer is refused with a
clear error.
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


def make_analysis(w):
    from bilby_gb300.analysis import Analysis, DetectorData
    from oracle import data as OD
    dets = OD.build_workload(w)
    return Analysis("taylorf2", dets[0].frequency,
                    [DetectorData(d.name, d.vertex, d.tensor, d.start_time, d.masked_strain, d.psd, d.mask)
                     for d in dets], w.duration, w.sampling_frequency, w.minimum_frequency)


def status_word(stream):
    from bilby_gb300 import _capi
    word = ctypes.c_int(-1)
    rc = _capi.load().gwl_noalloc_status(ctypes.c_void_p(stream), ctypes.byref(word))
    return rc, word.value


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
        assert torch.equal(got, ref), (call, np.max(np.abs(g - r)))
        assert status_word(stream) == (_capi.GWL_OK, 0)


def test_allocates_nothing_and_takes_the_accurate_kernel(analysis):
    """A fresh analysis with a refinement tolerance low enough that points are
    marked for the accurate kernel: the device's free memory is the same
    before and after the call, and the results equal the allocating entry
    point's bit for bit (so the marked points took the accurate kernel here
    as well)."""
    import torch
    from bilby_gb300 import _capi
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    w, warm = analysis
    n = 500
    stream = torch.cuda.current_stream().cuda_stream
    block = torch.from_numpy(params_block(draw_points(w, n, np.random.default_rng(9)))).cuda()
    got = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    ref = torch.empty(n, dtype=torch.float64, device="cuda")
    # the CUDA runtime loads each kernel on its first launch in the process;
    # launch them all once (accurate kernel included) before measuring
    tol = warm.refinement_tolerance
    warm.refinement_tolerance = 1e-9
    _capi.check(noalloc(warm, block, got, stream), "gwl_eval_device_noalloc")
    warm.refinement_tolerance = tol
    an = make_analysis(w)
    an.refinement_tolerance = 1e-9
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    _capi.check(noalloc(an, block, got, stream), "gwl_eval_device_noalloc")
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    an.log_likelihood_ratio_device(block.data_ptr(), n, ref.data_ptr(), "mixed", stream)
    assert an.last_refined(stream) > 0
    torch.cuda.synchronize()
    assert torch.equal(got, ref)
    assert status_word(stream) == (_capi.GWL_OK, 0)
    an.close()


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
