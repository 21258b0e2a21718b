"""Several analyses of uneven duration, sampling rate and detector count in
one batched launch: each result equals the single-analysis result
bit for bit (alone and in the mix), with and without CUDA-graph replay."""
import numpy as np
import pytest

from bilby_gb300.analysis import params_block
from bilby_gb300.workloads import draw_points, uneven_analyses

pytestmark = pytest.mark.gpu


def build(w):
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    return GravitationalWaveTransient(ifos, wfg, precision="mixed")


@pytest.fixture(scope="module")
def mix(gpu):
    ws = [w for w in uneven_analyses(24, seed=7) if w.duration <= 32][:6]
    likes = [build(w) for w in ws]
    blocks = [params_block(draw_points(w, min(w.batch, 700), np.random.default_rng(q))) for q, w in enumerate(ws)]
    return ws, likes, blocks


@pytest.mark.parametrize("graphs", [False, True])
def test_batched_equals_single(mix, graphs):
    from bilby_gb300.batching import Batcher
    ws, likes, blocks = mix
    single = [lk.analysis.log_likelihood_ratio_host(b, "mixed") for lk, b in zip(likes, blocks)]
    bat = Batcher(use_graphs=graphs)
    # the same analysis twice and the items in another order
    items = [(lk.analysis, b) for lk, b in zip(likes, blocks)] + [(likes[0].analysis, blocks[0][:, :37])]
    for _ in range(3):  # capture + replays
        got = bat.eval_host(items)
        for q in range(len(likes)):
            assert np.array_equal(got[q], single[q]), q
        assert np.array_equal(got[-1], single[0][:37])
    rev = bat.eval_host(items[::-1])
    for q in range(len(likes)):
        assert np.array_equal(rev[len(items) - 1 - q], single[q])
    bat.close()


def test_batched_fp64_and_mixed_agree(mix):
    """Mixed vs float64 through the batcher: |dlnL| <= 1e-3 for every point,
    including templates far louder than the data (<h|h> ~ 1e5-1e6, which these
    10-40 Msun draws at 20-200 Mpc reach), whose sums the refinement step
    recomputes."""
    from bilby_gb300.batching import Batcher
    ws, likes, blocks = mix
    bat = Batcher()
    items = [(lk.analysis, b[:, :64]) for lk, b in zip(likes, blocks)]
    mixed = bat.eval_host(items, "mixed")
    fp64 = bat.eval_host(items, "fp64")
    for q in range(len(items)):
        err = np.abs(mixed[q] - fp64[q])
        assert np.all(err <= 1e-3), (err.max(), fp64[q][np.argmax(err)])
    bat.close()
