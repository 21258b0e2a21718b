"""Host set-up of the GPU relative-binning likelihood (bin edges and summary
data, bilby/gw/likelihood/relative.py:178-230 and 319-363) against the
oracle's restatement, on seeded data with a synthetic fiducial response.  No
GPU: the device part is in tests/test_gpu_relbin.py."""
import numpy as np
import pytest

from oracle import relbin as RB
from oracle import restate as R


class _Gen:
    def __init__(self, f):
        self.frequency_array = f
        self.waveform_arguments = {}


@pytest.fixture(scope="module")
def setup():
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.relative import RelativeBinningGravitationalWaveTransient
    grandom.seed(11)
    ifos = InterferometerList(["H1", "L1"])
    ifos.set_strain_data_from_power_spectral_densities(2048.0, 16.0, 1126259642.0)
    f = ifos[0].strain_data.frequency_array
    rng = np.random.default_rng(5)
    like = object.__new__(RelativeBinningGravitationalWaveTransient)
    like.interferometers = list(ifos)
    like.waveform_generator = _Gen(f)
    like.chi, like.epsilon, like.gamma = 1.0, 0.5, RB.GAMMA
    like.maximum_frequency = 700.0
    phase = 2 * np.pi * np.cumsum(rng.uniform(0, 1, len(f)))
    like.per_detector_fiducial_waveforms = {
        ifo.name: np.where(f <= 700.0, (f + 1.0) ** (-7 / 6) * np.exp(1j * phase) * (1 + 0.1 * q), 0)
        for q, ifo in enumerate(ifos)}
    like.per_detector_fiducial_waveform_points = {}
    return like, ifos, f


def oracle_dets(ifos):
    out = []
    for ifo in ifos:
        out.append(R.Detector(ifo.name, ifo.strain_data.frequency_array, ifo.strain_data.frequency_domain_strain,
                              ifo.power_spectral_density_array, ifo.strain_data.frequency_mask,
                              np.zeros(3), np.zeros((3, 3)), ifo.strain_data.duration, ifo.strain_data.start_time))
    return out


@pytest.mark.parametrize("epsilon", [0.5, 0.1, 0.02])
def test_bins_match_the_restatement(setup, epsilon):
    like, ifos, f = setup
    like.epsilon = epsilon
    like.setup_bins()
    inds, freqs = RB.setup_bins(oracle_dets(ifos), f, like.maximum_frequency, 1.0, epsilon,
                                [ifo.maximum_frequency for ifo in ifos], [ifo.minimum_frequency for ifo in ifos])
    assert np.array_equal(like.bin_inds, inds)
    assert np.array_equal(like.bin_freqs, freqs)
    assert like.waveform_generator.waveform_arguments["frequency_bin_edges"] is like.bin_freqs


def test_summary_data_match_the_restatement(setup):
    like, ifos, f = setup
    like.epsilon = 0.1
    like.setup_bins()
    like.compute_summary_data()
    ref = RB.summary_data(oracle_dets(ifos), [like.per_detector_fiducial_waveforms[i.name] for i in ifos],
                          like.bin_freqs)
    for ifo, r in zip(ifos, ref):
        ours = np.stack(like.summary_data[ifo.name])
        assert np.max(np.abs(ours - np.stack(r))) <= 1e-12 * np.max(np.abs(np.stack(r)))
