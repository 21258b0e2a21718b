"""Error control of the mixed-precision TaylorF2 likelihood: points whose
|dlnL| bound exceeds the refinement tolerance are evaluated by the accurate
variant of the kernel (float-float cosine, TwoSum accumulation), so every
point meets |dlnL| <= 1e-3 against the float64 kernel, including templates
far louder than the data in short segments with a loud injection (where the
hardware cosine's error adds up coherently)."""
import numpy as np
import pytest

from bilby_gb300.analysis import params_block
from bilby_gb300.workloads import draw_points, uneven_analyses

pytestmark = pytest.mark.gpu

TOL = 1e-3


def build(w, **kwargs):
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
    return GravitationalWaveTransient(ifos, wfg, precision="mixed", **kwargs)


@pytest.fixture(scope="module")
def short(gpu):
    """The 4 s and 8 s analyses (10-40 Msun, injections at 100-400 Mpc) of the
    64-analysis uneven workload, 256 points each (20-200 Mpc)."""
    ws = [w for w in uneven_analyses(64) if w.duration <= 8][:6]
    likes = [build(w) for w in ws]
    blocks = [params_block(draw_points(w, 256, np.random.default_rng(100 + q))) for q, w in enumerate(ws)]
    return ws, likes, blocks


def test_default_tolerance(short):
    ws, likes, blocks = short
    assert likes[0].analysis.refinement_tolerance == pytest.approx(5e-4)


def test_refined_within_tolerance(short):
    ws, likes, blocks = short
    n_refined = 0
    for lk, b in zip(likes, blocks):
        an = lk.analysis
        mixed = an.log_likelihood_ratio_host(b, "mixed")
        n_refined += an.last_refined()
        fp64 = an.log_likelihood_ratio_host(b, "fp64")
        err = np.abs(mixed - fp64)
        assert np.all(err <= TOL), (err.max(), fp64[np.argmax(err)])
    assert n_refined > 0


def test_refinement_changes_only_marked_points(short):
    """Off (tolerance 0) vs on: the unmarked points are bit-identical, the
    marked ones move, and the largest error does not grow."""
    ws, likes, blocks = short
    an, b = likes[0].analysis, blocks[0]
    fp64 = an.log_likelihood_ratio_host(b, "fp64")
    on = an.log_likelihood_ratio_host(b, "mixed")
    n_on = an.last_refined()
    tol = an.refinement_tolerance
    try:
        an.refinement_tolerance = 0.0
        off = an.log_likelihood_ratio_host(b, "mixed")
        assert an.last_refined() == 0
    finally:
        an.refinement_tolerance = tol
    changed = int(np.sum(on != off))
    assert 0 < changed <= n_on
    assert np.abs(on - fp64).max() <= np.abs(off - fp64).max()


def test_refined_point_independent_of_batch(short):
    ws, likes, blocks = short
    an, b = likes[1].analysis, blocks[1]
    full = an.log_likelihood_ratio_host(b, "mixed")
    for lo, hi in [(0, 1), (5, 6), (0, 37), (100, 256)]:
        part = an.log_likelihood_ratio_host(np.ascontiguousarray(b[:, lo:hi]), "mixed")
        assert np.array_equal(part, full[lo:hi])


@pytest.mark.parametrize("graphs", [False, True])
def test_batcher_refines_the_same_points(short, graphs):
    from bilby_gb300.batching import Batcher
    ws, likes, blocks = short
    single, count = [], 0
    for lk, b in zip(likes, blocks):
        single.append(lk.analysis.log_likelihood_ratio_host(b, "mixed"))
        count += lk.analysis.last_refined()
    bat = Batcher(use_graphs=graphs)
    items = [(lk.analysis, b) for lk, b in zip(likes, blocks)]
    for _ in range(2):
        got = bat.eval_host(items)
        assert bat.last_refined() == count
        for q in range(len(items)):
            assert np.array_equal(got[q], single[q]), q
    bat.close()


def test_phase_marginalized_refined(gpu):
    """The complex partial sums (phase marginalisation) have the same accurate variant."""
    w = [w for w in uneven_analyses(64) if w.duration <= 8][0]
    from bilby_gb300.prior import Uniform
    lk = build(w, phase_marginalization=True, priors={"phase": Uniform(0, 2 * np.pi)})
    b = params_block(draw_points(w, 256, np.random.default_rng(7)))
    an = lk.analysis
    mixed = an.log_likelihood_ratio_host(b, "mixed")
    assert an.last_refined() > 0
    fp64 = an.log_likelihood_ratio_host(b, "fp64")
    err = np.abs(mixed - fp64)
    assert np.all(err <= TOL), err.max()
