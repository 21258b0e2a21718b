"""The launch-shape autotuner of the mixed TaylorF2 kernel: it picks one of
its candidate split-K depths, the choice is kept by the analysis, results stay
bit-reproducible at a fixed depth and move only by float64 rounding between
depths, and the batcher follows a re-tuned analysis."""
import numpy as np
import pytest

from tests.gpu_helpers import WORKLOADS, device_analysis, draw_points, params_block, small_workload
from oracle import data as OD

pytestmark = pytest.mark.gpu

CANDIDATES = {2, 3, 4, 6, 8, 12, 16}


@pytest.fixture(scope="module")
def tf2_16s(gpu):
    w = small_workload("tf2_128s", duration=16.0,
                       injection=dict(WORKLOADS["tf2_128s"].injection,
                                      geocent_time=WORKLOADS["tf2_128s"].start_time + 14.0))
    dets = OD.build_workload(w)
    an = device_analysis(dets, "taylorf2", w)
    block = params_block(draw_points(w, 1000, np.random.default_rng(41)))
    return w, an, block


def test_autotune_picks_a_candidate_and_keeps_it(tf2_16s):
    import torch
    w, an, block = tf2_16s
    before = an.log_likelihood_ratio_host(block, "mixed")
    dev = torch.from_numpy(block).cuda()
    cpg, ms = an.autotune(dev.data_ptr(), block.shape[1], torch.cuda.current_stream().cuda_stream)
    assert cpg in CANDIDATES
    assert ms > 0
    assert an.chunks_per_group == cpg
    after = an.log_likelihood_ratio_host(block, "mixed")
    again = an.log_likelihood_ratio_host(block, "mixed")
    assert np.array_equal(after, again)
    # a different depth reorders float64 additions of chunk sums only
    assert np.allclose(after, before, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("cpg", [2, 4, 16])
def test_every_depth_agrees(tf2_16s, cpg):
    w, an, block = tf2_16s
    keep = an.chunks_per_group
    try:
        an.chunks_per_group = 4
        ref = an.log_likelihood_ratio_host(block, "mixed")
        an.chunks_per_group = cpg
        got = an.log_likelihood_ratio_host(block, "mixed")
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-9)
    finally:
        an.chunks_per_group = keep


def test_batcher_follows_the_tuned_depth(tf2_16s):
    from bilby_gb300.batching import Batcher
    w, an, block = tf2_16s
    keep = an.chunks_per_group
    bat = Batcher(use_graphs=True)
    try:
        for cpg in (3, 8):
            an.chunks_per_group = cpg
            single = an.log_likelihood_ratio_host(block, "mixed")
            for _ in range(2):  # capture, then replay
                got = bat.eval_host([(an, block)], "mixed")[0]
                assert np.array_equal(got, single), cpg
    finally:
        an.chunks_per_group = keep
        bat.close()


def test_bad_depth_is_rejected(tf2_16s):
    w, an, block = tf2_16s
    with pytest.raises(ValueError):
        an.chunks_per_group = 0
