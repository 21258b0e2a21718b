"""The drop-in likelihood evaluated in a detector-pair frame with a detector
time reference gives the same lnL as the sky frame at the converted
parameters; a pickled likelihood rebuilds its device handle and gives the
same values (the state a multiprocessing sampler pool relies on)."""
import pickle

import numpy as np
import pytest

from bilby_gb300.workloads import WORKLOADS, draw_points

pytestmark = pytest.mark.gpu


def build(reference_frame="sky", time_reference="geocenter"):
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator
    w = WORKLOADS["tf2_marg_8s_2k"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    return w, GravitationalWaveTransient(ifos, wfg, reference_frame=reference_frame, time_reference=time_reference)


def test_detector_frame_equals_sky_frame(gpu):
    w, sky = build()
    _, det = build("H1L1", "H1")
    rng = np.random.default_rng(8)
    p = draw_points(w, 64, rng)
    q = {k: v for k, v in p.items() if k not in ("ra", "dec", "geocent_time")}
    q["zenith"] = np.arccos(rng.uniform(-1, 1, 64))
    q["azimuth"] = rng.uniform(0, 2 * np.pi, 64)
    q["H1_time"] = p["geocent_time"] + rng.uniform(-0.02, 0.02, 64)
    conv = det.get_sky_frame_parameters(q)
    r = dict(q)
    r.update(conv)
    a = det.log_likelihood_ratio_batch(q)
    b = sky.log_likelihood_ratio_batch({k: v for k, v in r.items() if k not in ("zenith", "azimuth", "H1_time")})
    assert np.array_equal(a, b)


def test_pickled_likelihood_rebuilds_and_agrees(gpu):
    w, like = build()
    p = draw_points(w, 32, np.random.default_rng(9))
    before = like.log_likelihood_ratio_batch(p)
    clone = pickle.loads(pickle.dumps(like))
    assert clone._analysis is None
    assert np.array_equal(clone.log_likelihood_ratio_batch(p), before)
    assert clone.noise_log_likelihood() == like.noise_log_likelihood()
